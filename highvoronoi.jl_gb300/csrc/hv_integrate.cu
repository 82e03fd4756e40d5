// hv_integrate.cu -- per-cell integrators on the GPU.
//
// VI_POLYGON (src/polyintegrator.jl:174-468): the cone over facet k of cell i
// is cut into simplices (x_i, c_F, c(L_1), ..., c(L_{d-3}), v1, v2), one per
// flag facet > ... > edge, where c(.) are vertex centroids of the faces of the
// flag and (v1, v2) the edge's end points; V_ik = sum |det| / d!, the
// interface area is A_ik = V_ik d / h_ik (src/polyintegrator.jl:308-316) and
// V_i = sum_k A_ik h_ik / d.  Interfaces are computed by the lower cell and
// copied to the higher one (src/cleanup_cell.jl:174-204).  One block per cell:
// the cell's vertices are staged in shared memory once and every facet of the
// cell is processed from there.  All sums run in a fixed order, so results
// are bitwise reproducible.
//
// VI_HEURISTIC_MC (src/mcintegrator.jl:98-226, src/heuristic_mc.jl:1-56): per
// cell, ndir Philox4x32-10 directions (FP32 Box-Muller), t = min over the
// neighbours of the ray parameter (FP32), V = pi^(d/2)/Gamma(1+d/2) mean(t^d)
// and A_j = d * const * mean over hits of t^(d-1)/|n_j.u|, accumulated in FP64;
// then two-sided averaging of the areas with the volume correction of
// src/mcintegrator.jl:172-201.
#include "hv_internal.cuh"
#include "hv_integrate.h"

namespace hv {

struct PolyArgs {
    int d, n;
    double lo[HV_MAXD], hi[HV_MAXD];
    const double* pts;       // original order, n x d
    const int* osig;         // V x (d+1), original 0-based items
    const double* oc;        // V x d
    const long long* inc_off;
    const int* inc;
    const long long* nbr_off;
    const int* nbr;
    double* area;            // aligned with nbr
    unsigned* status;        // bit 1: cell too large, bit 2: facet structure overflow
    int capC, capV, capF, capE, capI;
};

__device__ __forceinline__ double plane_height(const PolyArgs& A, const double* xi, int k) {
    const int p = k - A.n, q = p >> 1;
    return (p & 1) == 0 ? A.hi[q] - xi[q] : xi[q] - A.lo[q];
}

template <int D>
__device__ __forceinline__ double facet_height(const PolyArgs& A, const double* xi, int k) {
    if (k >= A.n) return plane_height(A, xi, k);
    double s = 0;
#pragma unroll
    for (int c = 0; c < D; ++c) { const double e = A.pts[(size_t)k * D + c] - xi[c]; s = fma(e, e, s); }
    return 0.5 * sqrt(s);
}

// Block-wide bitonic sort of `n2` (power of two) keys in shared memory.
template <class T>
__device__ void block_bitonic(T* a, int n2) {
    for (int k = 2; k <= n2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int x = threadIdx.x; x < n2; x += blockDim.x) {
                const int y = x ^ j;
                if (y > x) {
                    const bool up = (x & k) == 0;
                    const T p = a[x], q = a[y];
                    if ((p > q) == up) { a[x] = q; a[y] = p; }
                }
            }
            __syncthreads();
        }
    }
}

__device__ __forceinline__ int pow2_at_least(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

// Fixed-order block reduction of one double per thread.
__device__ double block_sum(double v, double* red) {
    red[threadIdx.x] = v;
    __syncthreads();
    for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
}

template <int D>
__device__ __forceinline__ double det_abs(double (&M)[D][D]) {
    int piv[D];
    if (!lu_factor<D, double>(M, piv)) return 0.0;
    double det = 1.0;
#pragma unroll
    for (int r = 0; r < D; ++r) det *= M[r][r];
    return fabs(det);
}

// Decode permutation number `w` (0 <= w < m!) of the m items into an order.
__device__ __forceinline__ void lehmer(int w, int m, int* ord) {
    int avail[HV_MAXD];
    for (int a = 0; a < m; ++a) avail[a] = a;
    int f = 1;
    for (int a = 2; a < m; ++a) f *= a;
    for (int pos = 0; pos < m; ++pos) {
        const int rem = m - pos;
        const int q = (rem > 1) ? w / f : 0;
        if (rem > 1) { w %= f; }
        ord[pos] = avail[q];
        for (int a = q; a < rem - 1; ++a) avail[a] = avail[a + 1];
        if (rem - 1 > 1) f /= (rem - 1);
    }
}

// Local item lists: every facet vertex has D-1 generators besides i and k,
// mapped to local indices < capI (10 bits) and kept sorted.  A face of the
// facet is a sorted subset of those indices, packed 10 bits per item with the
// length in bits 56..59, so faces sort and search as 64-bit keys.
__device__ __forceinline__ unsigned long long pack_face(const int* it, int len) {
    unsigned long long k = (unsigned long long)len << 56;
    for (int q = 0; q < len; ++q) k |= (unsigned long long)it[q] << (10 * q);
    return k;
}

// Is the sorted list `sub` (len items) contained in the sorted list `set` (m items)?
__device__ __forceinline__ bool contains_sorted(const int* set, int m, const int* sub, int len) {
    int p = 0;
    for (int q = 0; q < len; ++q) {
        while (p < m && set[p] < sub[q]) ++p;
        if (p == m || set[p] != sub[q]) return false;
        ++p;
    }
    return true;
}

// GLOBAL = false: work area in shared memory, all cells; cells with more than
// capC vertices are appended to `big` for the GLOBAL = true pass, whose work
// area is a per-block slab of global memory sized for the largest cell.
template <int D, bool GLOBAL>
__global__ void __launch_bounds__(128) k_poly_cells(PolyArgs A, const int* cells, int ncells, unsigned char* gbase,
                                                    size_t area_bytes, int* big, unsigned* nbig) {
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned char* base = GLOBAL ? gbase + (size_t)blockIdx.x * area_bytes : smem;
    const int capC = A.capC, capV = A.capV, capF = A.capF, capE = A.capE, capI = A.capI;
    constexpr int DM = (D > 1) ? D - 1 : 1;        // local items per facet vertex
    double* cx = (double*)base;                       // capC x D   cell vertex coords - x_i
    double* fcen = cx + (size_t)capC * D;             // capF x D   face centroids
    double* cF = fcen + (size_t)capF * D;             // D          facet centroid
    double* red = cF + D;                             // blockDim
    unsigned long long* flist = (unsigned long long*)(red + blockDim.x);  // capF (sorted face keys)
    unsigned long long* ftab = flist + capF;          // 2*capF hash table
    int* csig = (int*)(ftab + 2 * capF);              // capC x (D+1)
    int* fv = csig + (size_t)capC * (D + 1);          // capV (local cell-vertex index)
    int* vit = fv + capV;                             // capV x DM local item lists (sorted)
    int* ekey = vit + (size_t)capV * DM;              // capE (a << 16 | b)
    int* items = ekey + capE;                         // capI
    int* itab = items + capI;                         // 2*capI hash of items
    int* cnt = itab + 2 * capI;                       // 8 counters

    constexpr int NPERM = (D <= 3) ? 1 : (D == 4 ? 2 : (D == 5 ? 6 : 24));  // (D-2)!
    double fact = 1.0;
    for (int q = 2; q <= D; ++q) fact *= q;

    const int nwork = GLOBAL ? ncells : A.n;
    for (int wi = blockIdx.x; wi < nwork; wi += gridDim.x) {
        const int i = GLOBAL ? cells[wi] : wi;
        double xi[D];
#pragma unroll
        for (int c = 0; c < D; ++c) xi[c] = A.pts[(size_t)i * D + c];
        const long long vb = A.inc_off[i], ve = A.inc_off[i + 1];
        const int nc = (int)(ve - vb);
        if (nc > capC) {
            if (threadIdx.x == 0) {
                if (GLOBAL) atomicOr(A.status, 1u);
                else big[atomicAdd(nbig, 1u)] = i;
            }
            continue;
        }
        // ---- stage the cell's vertices
        for (int a = threadIdx.x; a < nc; a += blockDim.x) {
            const int v = A.inc[vb + a];
#pragma unroll
            for (int s = 0; s <= D; ++s) csig[a * (D + 1) + s] = A.osig[(size_t)v * (D + 1) + s];
#pragma unroll
            for (int c = 0; c < D; ++c) cx[a * D + c] = A.oc[(size_t)v * D + c] - xi[c];
        }
        __syncthreads();
        // ---- facets with k > i (planes included)
        for (long long t = A.nbr_off[i]; t < A.nbr_off[i + 1]; ++t) {
            const int k = A.nbr[t];
            if (k < i) continue;
            if (threadIdx.x < 8) cnt[threadIdx.x] = 0;
            for (int x = threadIdx.x; x < 2 * capI; x += blockDim.x) itab[x] = -1;
            __syncthreads();
            // facet vertices (cell-local indices)
            for (int a = threadIdx.x; a < nc; a += blockDim.x) {
                bool has = false;
#pragma unroll
                for (int s = 0; s <= D; ++s) has |= (csig[a * (D + 1) + s] == k);
                if (has) {
                    const int p = atomicAdd(&cnt[0], 1);
                    if (p < capV) fv[p] = a;
                }
            }
            __syncthreads();
            const int nv = cnt[0];
            if (nv > capV || nv < 2) {
                if (threadIdx.x == 0 && nv > capV) atomicOr(A.status, 2u);
                __syncthreads();
                continue;
            }
            const int nv2 = pow2_at_least(nv);
            for (int a = nv + threadIdx.x; a < nv2; a += blockDim.x) fv[a] = 0x7FFFFFFF;
            __syncthreads();
            block_bitonic<int>(fv, nv2);
            // local items (generators of the facet's vertices other than i and k)
            for (int a = threadIdx.x; a < nv; a += blockDim.x) {
                const int* sg = csig + fv[a] * (D + 1);
                for (int q = 0; q <= D; ++q) {
                    const int it = sg[q];
                    if (it == i || it == k) continue;
                    unsigned h = ((unsigned)it * 2654435761u) & (unsigned)(2 * capI - 1);
                    for (int pr = 0; pr < 2 * capI; ++pr) {
                        const int prev = atomicCAS(&itab[h], -1, it);
                        if (prev == -1) { atomicAdd(&cnt[1], 1); break; }
                        if (prev == it) break;
                        h = (h + 1) & (unsigned)(2 * capI - 1);
                    }
                }
            }
            __syncthreads();
            const int ni = cnt[1];
            if (ni > capI) {
                if (threadIdx.x == 0) atomicOr(A.status, 2u);
                __syncthreads();
                continue;
            }
            if (threadIdx.x == 0) {
                int w = 0;
                for (int x = 0; x < 2 * capI; ++x) if (itab[x] >= 0) items[w++] = itab[x];
                for (int x = w; x < capI; ++x) items[x] = 0x7FFFFFFF;
            }
            __syncthreads();
            block_bitonic<int>(items, capI);
            // per-vertex sorted local item lists
            for (int a = threadIdx.x; a < nv; a += blockDim.x) {
                const int* sg = csig + fv[a] * (D + 1);
                int loc[DM];
                int w = 0;
                for (int q = 0; q <= D; ++q) {
                    const int it = sg[q];
                    if (it == i || it == k) continue;
                    int lo = 0, hi = ni - 1;
                    while (lo < hi) { const int md = (lo + hi) >> 1; if (items[md] < it) lo = md + 1; else hi = md; }
                    if (w < DM) loc[w++] = lo;
                }
                for (int x = 1; x < w; ++x)
                    for (int y = x; y > 0 && loc[y] < loc[y - 1]; --y) { const int z = loc[y]; loc[y] = loc[y - 1]; loc[y - 1] = z; }
                for (int x = 0; x < DM; ++x) vit[a * DM + x] = x < w ? loc[x] : 0x7FFFFFFF;
            }
            __syncthreads();
            // facet centroid (fixed-order sums)
            if (D >= 3) {
                for (int c = 0; c < D; ++c) {
                    double sum = 0;
                    for (int a = threadIdx.x; a < nv; a += blockDim.x) sum += cx[fv[a] * D + c];
                    const double tot = block_sum(sum, red);
                    if (threadIdx.x == 0) cF[c] = tot / nv;
                }
            }
            // faces: sorted subsets of size 1..D-3 of the vertices' item lists (d >= 4)
            int nf = 0;
            if (D >= 4) {
                for (int x = threadIdx.x; x < 2 * capF; x += blockDim.x) ftab[x] = 0ull;
                __syncthreads();
                for (int a = threadIdx.x; a < nv; a += blockDim.x) {
                    const int* li = vit + a * DM;
                    for (unsigned sub = 1; sub < (1u << DM); ++sub) {
                        const int pc = __popc(sub);
                        if (pc > D - 3) continue;
                        int tup[DM];
                        int w = 0;
                        for (int x = 0; x < DM; ++x) if ((sub >> x) & 1u) tup[w++] = li[x];
                        const unsigned long long key = pack_face(tup, w);
                        const unsigned long long h = (key * 0x9E3779B97F4A7C15ull) >> 20;
                        for (int pr = 0; pr < 2 * capF; ++pr) {
                            const unsigned slot = (unsigned)((h + pr) & (unsigned long long)(2 * capF - 1));
                            const unsigned long long prev = atomicCAS(&ftab[slot], 0ull, key);
                            if (prev == 0ull) { atomicAdd(&cnt[2], 1); break; }
                            if (prev == key) break;
                        }
                    }
                }
                __syncthreads();
                nf = cnt[2];
                if (nf > capF) {
                    if (threadIdx.x == 0) atomicOr(A.status, 2u);
                    __syncthreads();
                    continue;
                }
                if (threadIdx.x == 0) {
                    int w = 0;
                    for (int x = 0; x < 2 * capF; ++x) if (ftab[x]) flist[w++] = ftab[x];
                }
                __syncthreads();
                const int nf2 = pow2_at_least(nf);
                for (int x = nf + threadIdx.x; x < nf2; x += blockDim.x) flist[x] = ~0ull;
                __syncthreads();
                block_bitonic<unsigned long long>(flist, nf2);
                for (int f = threadIdx.x; f < nf; f += blockDim.x) {
                    const unsigned long long key = flist[f];
                    const int len = (int)(key >> 56);
                    int tup[DM];
                    for (int q = 0; q < len; ++q) tup[q] = (int)((key >> (10 * q)) & 1023ull);
                    double sum[D];
#pragma unroll
                    for (int c = 0; c < D; ++c) sum[c] = 0;
                    int cntv = 0;
                    for (int a = 0; a < nv; ++a) {
                        if (contains_sorted(vit + a * DM, DM, tup, len)) {
                            ++cntv;
#pragma unroll
                            for (int c = 0; c < D; ++c) sum[c] += cx[fv[a] * D + c];
                        }
                    }
#pragma unroll
                    for (int c = 0; c < D; ++c) fcen[f * D + c] = sum[c] / cntv;
                }
            }
            // edges: vertex pairs sharing D-2 local items
            for (int a = threadIdx.x; a < nv; a += blockDim.x) {
                const int* la = vit + a * DM;
                for (int drop = 0; drop < DM; ++drop) {
                    int L[DM];
                    int w = 0;
                    for (int x = 0; x < DM; ++x) if (x != drop) L[w++] = la[x];
                    for (int b = a + 1; b < nv; ++b) {
                        if (contains_sorted(vit + b * DM, DM, L, w)) {
                            const int p = atomicAdd(&cnt[3], 1);
                            if (p < capE) ekey[p] = (a << 16) | b;
                            break;
                        }
                    }
                }
            }
            __syncthreads();
            const int ne = cnt[3];
            if (ne > capE) {
                if (threadIdx.x == 0) atomicOr(A.status, 2u);
                __syncthreads();
                continue;
            }
            const int ne2 = pow2_at_least(ne);
            for (int x = ne + threadIdx.x; x < ne2; x += blockDim.x) ekey[x] = 0x7FFFFFFF;
            __syncthreads();
            block_bitonic<int>(ekey, ne2);
            // flags: every edge with every order of its D-2 items
            double part = 0.0;
            const int nw = ne * NPERM;
            for (int w = threadIdx.x; w < nw; w += blockDim.x) {
                const int e = w / NPERM, perm = w % NPERM;
                const int a = ekey[e] >> 16, b = ekey[e] & 0xFFFF;
                double Mx[D][D];
                int col = 0;
                if (D >= 3) {
#pragma unroll
                    for (int c = 0; c < D; ++c) Mx[c][0] = cF[c];
                    col = 1;
                }
                if (D >= 4) {
                    // common items of a and b (the edge), in sorted order
                    int it[DM];
                    int m = 0;
                    const int* la = vit + a * DM;
                    const int* lb = vit + b * DM;
                    for (int x = 0; x < DM; ++x)
                        if (contains_sorted(lb, DM, la + x, 1)) it[m++] = la[x];
                    int ord[HV_MAXD];
                    lehmer(perm, D - 2, ord);
                    int pre[DM];
                    for (int j = 0; j < D - 3; ++j) {
                        // prefix {it[ord[0]], ..., it[ord[j]]}, sorted
                        int x = j;
                        pre[x] = it[ord[j]];
                        while (x > 0 && pre[x] < pre[x - 1]) { const int z = pre[x]; pre[x] = pre[x - 1]; pre[x - 1] = z; --x; }
                        const unsigned long long key = pack_face(pre, j + 1);
                        int lo = 0, hi = nf - 1;
                        while (lo < hi) { const int md = (lo + hi) >> 1; if (flist[md] < key) lo = md + 1; else hi = md; }
#pragma unroll
                        for (int c = 0; c < D; ++c) {
#pragma unroll
                            for (int cc = 0; cc < D; ++cc) if (cc == col) Mx[c][cc] = fcen[lo * D + c];
                        }
                        ++col;
                    }
                }
#pragma unroll
                for (int c = 0; c < D; ++c) {
#pragma unroll
                    for (int cc = 0; cc < D; ++cc) {
                        if (cc == D - 2) Mx[c][cc] = cx[fv[a] * D + c];
                        if (cc == D - 1) Mx[c][cc] = cx[fv[b] * D + c];
                    }
                }
                part += det_abs<D>(Mx);
            }
            const double S = block_sum(part, red);
            if (threadIdx.x == 0) {
                const double Vik = S / fact;
                const double h = facet_height<D>(A, xi, k);
                const double ar = Vik * D / h;
                A.area[t] = ar;
                if (k < A.n) {  // copy to the higher cell's interface
                    long long lo = A.nbr_off[k], hi = A.nbr_off[k + 1] - 1;
                    while (lo < hi) { const long long md = (lo + hi) >> 1; if (A.nbr[md] < i) lo = md + 1; else hi = md; }
                    if (A.nbr[lo] == i) A.area[lo] = ar;
                }
            }
            __syncthreads();
        }
        __syncthreads();
    }
}

template <int D>
__global__ void k_poly_volumes(PolyArgs A, double* vol) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
        double xi[D];
#pragma unroll
        for (int c = 0; c < D; ++c) xi[c] = A.pts[(size_t)i * D + c];
        double v = 0;
        for (long long t = A.nbr_off[i]; t < A.nbr_off[i + 1]; ++t) v += A.area[t] * facet_height<D>(A, xi, A.nbr[t]) / D;
        vol[i] = v;
    }
}

// ---------------------------------------------------------------------------
// heuristic Monte-Carlo
// ---------------------------------------------------------------------------
__device__ __forceinline__ void philox4x32_i(unsigned (&c)[4], unsigned k0, unsigned k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const unsigned hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
        const unsigned hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
        const unsigned o0 = hi1 ^ c[1] ^ k0, o2 = hi0 ^ c[3] ^ k1;
        c[0] = o0; c[1] = lo1; c[2] = o2; c[3] = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
}

// Unit direction s of cell i: Philox counter (s, i_lo, i_hi, block), key = seed,
// Box-Muller pairs in FP32 (same bits as the oracle's FP64 directions).
template <int D>
__device__ __forceinline__ void mc_direction(unsigned long long seed, unsigned s, unsigned long long cell, float (&u)[D]) {
    int got = 0;
#pragma unroll
    for (unsigned blk = 0; blk < (unsigned)((D + 3) / 4); ++blk) {
        unsigned c[4] = {s, (unsigned)cell, (unsigned)(cell >> 32), blk};
        philox4x32_i(c, (unsigned)seed, (unsigned)(seed >> 32));
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            const float u1 = ((float)c[2 * p] + 0.5f) * 2.3283064365386963e-10f;
            const float u2 = ((float)c[2 * p + 1] + 0.5f) * 2.3283064365386963e-10f;
            const float rr = sqrtf(-2.f * logf(fmaxf(u1, 1e-38f)));
            float sn, cs;
            sincospif(2.f * u2, &sn, &cs);
#pragma unroll
            for (int k = 0; k < D; ++k) {
                if (k == got) u[k] = rr * cs;
                if (k == got + 1) u[k] = rr * sn;
            }
            got += 2;
        }
    }
    float nn = 0.f;
#pragma unroll
    for (int k = 0; k < D; ++k) nn = fmaf(u[k], u[k], nn);
    nn = rsqrtf(nn);
#pragma unroll
    for (int k = 0; k < D; ++k) u[k] *= nn;
}

constexpr int MC_WPB = 2;

template <int D>
__global__ void __launch_bounds__(MC_WPB * 32) k_mc_cells(PolyArgs A, int ndir, unsigned long long seed, int capN,
                                                         double cvol, double* rawV, double* rawA, double* varV) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // per warp: capN x (D+1) floats (delta, |delta|^2 or plane code) + 32 x capN doubles
    float* nb = (float*)(smem) + (size_t)wib * capN * (D + 2);
    double* slab = (double*)((float*)smem + (size_t)MC_WPB * capN * (D + 2)) + (size_t)wib * 32 * capN;
    for (int i = blockIdx.x * MC_WPB + wib; i < A.n; i += gridDim.x * MC_WPB) {
        const long long b = A.nbr_off[i];
        const int deg = (int)(A.nbr_off[i + 1] - b);
        if (deg > capN) {
            if (lane == 0) atomicOr(A.status, 4u);
            continue;
        }
        float xi[D];
#pragma unroll
        for (int c = 0; c < D; ++c) xi[c] = (float)A.pts[(size_t)i * D + c];
        for (int t = lane; t < deg; t += 32) {
            const int k = A.nbr[b + t];
            float* e = nb + t * (D + 2);
            if (k < A.n) {
                float s = 0.f;
#pragma unroll
                for (int c = 0; c < D; ++c) {
                    const float dl = (float)(A.pts[(size_t)k * D + c] - A.pts[(size_t)i * D + c]);
                    e[c] = dl;
                    s = fmaf(dl, dl, s);
                }
                e[D] = s;
                e[D + 1] = rsqrtf(s);  // 1/|delta| for the normal
            } else {
                const int p = k - A.n, q = p >> 1;
#pragma unroll
                for (int c = 0; c < D; ++c) e[c] = 0.f;
                e[D] = (float)(-1 - p);  // plane marker
                e[D + 1] = (float)((p & 1) == 0 ? A.hi[q] - A.pts[(size_t)i * D + q]
                                                 : A.pts[(size_t)i * D + q] - A.lo[q]);
            }
            for (int l = 0; l < 32; ++l) slab[l * capN + t] = 0.0;
        }
        __syncwarp();
        double vs = 0.0, vs2 = 0.0;
        for (int s = lane; s < ndir; s += 32) {
            float u[D];
            mc_direction<D>(seed, (unsigned)s, (unsigned long long)i, u);
            float tb = INFINITY, cosb = 1.f;
            int jb = -1;
            for (int t = 0; t < deg; ++t) {
                const float* e = nb + t * (D + 2);
                float tt, cs;
                if (e[D] >= 0.f) {
                    float du = 0.f;
#pragma unroll
                    for (int c = 0; c < D; ++c) du = fmaf(e[c], u[c], du);
                    if (!(du > 0.f)) continue;
                    tt = e[D] / (2.f * du);
                    cs = du * e[D + 1];
                } else {
                    const int p = -1 - (int)e[D], q = p >> 1;
                    float uk = 0.f;
#pragma unroll
                    for (int c = 0; c < D; ++c) if (c == q) uk = u[c];
                    if ((p & 1) != 0) uk = -uk;
                    if (!(uk > 0.f)) continue;
                    tt = e[D + 1] / uk;
                    cs = uk;
                }
                if (tt > 0.f && tt < tb) { tb = tt; jb = t; cosb = cs; }
            }
            if (jb < 0) continue;
            const double td = (double)tb;
            double tpow = 1.0;
#pragma unroll
            for (int c = 0; c < D - 1; ++c) tpow *= td;
            const double tdd = tpow * td;
            vs += tdd;
            vs2 += tdd * tdd;
            slab[lane * capN + jb] += tpow / fabs((double)cosb);
        }
        // fixed-order reductions
        for (int off = 16; off > 0; off >>= 1) {
            vs += __shfl_down_sync(0xFFFFFFFFu, vs, off);
            vs2 += __shfl_down_sync(0xFFFFFFFFu, vs2, off);
        }
        __syncwarp();
        const double carea = D * cvol;
        for (int t = lane; t < deg; t += 32) {
            double s = 0.0;
            for (int l = 0; l < 32; ++l) s += slab[l * capN + t];
            rawA[b + t] = s * carea / ndir;
        }
        if (lane == 0) {
            rawV[i] = vs * cvol / ndir;
            const double m = vs / ndir;
            varV[i] = cvol * cvol * fmax(vs2 / ndir - m * m, 0.0) / ndir;
        }
        __syncwarp();
    }
}

// Two-sided area averaging (src/mcintegrator.jl:172-201): for the pair (i < k)
// the lower cell's estimate `neigh` and the higher cell's `old` become one
// value; each cell's volume moves by (new - own) h / d.
template <int D>
__global__ void k_mc_pairs(PolyArgs A, const double* rawA, double* outA) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
        for (long long t = A.nbr_off[i]; t < A.nbr_off[i + 1]; ++t) {
            const int k = A.nbr[t];
            if (k >= A.n || k < i) {
                if (k >= A.n) outA[t] = rawA[t];
                continue;
            }
            long long lo = A.nbr_off[k], hi = A.nbr_off[k + 1] - 1;
            while (lo < hi) { const long long md = (lo + hi) >> 1; if (A.nbr[md] < i) lo = md + 1; else hi = md; }
            const double neigh = rawA[t], old = rawA[lo];
            const double na = fabs(neigh) < old * 1.0e-10 ? old : 0.5 * (old + neigh);
            outA[t] = na;
            outA[lo] = na;
        }
    }
}

template <int D>
__global__ void k_mc_volumes(PolyArgs A, const double* rawV, const double* rawA, const double* outA, double* vol) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
        double xi[D];
#pragma unroll
        for (int c = 0; c < D; ++c) xi[c] = A.pts[(size_t)i * D + c];
        double v = rawV[i];
        for (long long t = A.nbr_off[i]; t < A.nbr_off[i + 1]; ++t) {
            const int k = A.nbr[t];
            if (k >= A.n) continue;
            v += (outA[t] - rawA[t]) * facet_height<D>(A, xi, k) / D;
        }
        vol[i] = v;
    }
}

// ---------------------------------------------------------------------------
#define HV_DISPATCH(d, CALL)                           \
    switch (d) {                                       \
        case 2: { constexpr int DD = 2; CALL; } break; \
        case 3: { constexpr int DD = 3; CALL; } break; \
        case 4: { constexpr int DD = 4; CALL; } break; \
        case 5: { constexpr int DD = 5; CALL; } break; \
        case 6: { constexpr int DD = 6; CALL; } break; \
        default: break;                                \
    }

static PolyArgs make_args(const IntegrateInput& in) {
    PolyArgs A;
    A.d = in.d; A.n = in.n;
    for (int k = 0; k < in.d; ++k) { A.lo[k] = in.lo[k]; A.hi[k] = in.hi[k]; }
    A.pts = in.pts; A.osig = in.osig; A.oc = in.oc;
    A.inc_off = in.inc_off; A.inc = in.inc; A.nbr_off = in.nbr_off; A.nbr = in.nbr;
    A.status = in.status;
    A.area = nullptr;
    A.capC = A.capV = A.capF = A.capE = A.capI = 0;
    return A;
}

size_t poly_smem_bytes(int d, int capC, int capV, int capF, int capE, int capI) {
    return sizeof(double) * ((size_t)capC * d + (size_t)capF * d + d + 128) +
           sizeof(unsigned long long) * (3 * (size_t)capF) +
           sizeof(int) * ((size_t)capC * (d + 1) + (size_t)capV * d + capE + 3 * (size_t)capI + 8);
}

template <int D>
static int poly_t(const IntegrateInput& in, const PolyCaps& cs, const PolyCaps& cg, int* big, unsigned* nbig,
                  unsigned nbig_host, unsigned char* gbase, int gblocks, double* area, double* vol, int pass,
                  int nsm, cudaStream_t st) {
    PolyArgs A = make_args(in);
    A.area = area;
    if (pass == 0) {
        A.capC = cs.capC; A.capV = cs.capV; A.capF = cs.capF; A.capE = cs.capE; A.capI = cs.capI;
        const size_t sm = poly_smem_bytes(D, cs.capC, cs.capV, cs.capF, cs.capE, cs.capI);
        if (cudaFuncSetAttribute(k_poly_cells<D, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
            cudaSuccess)
            return -1;
        int blocks = nsm * 4;
        if (blocks > in.n) blocks = in.n;
        if (blocks < 1) blocks = 1;
        k_poly_cells<D, false><<<blocks, 128, sm, st>>>(A, nullptr, 0, nullptr, 0, big, nbig);
    } else if (pass == 1) {
        A.capC = cg.capC; A.capV = cg.capV; A.capF = cg.capF; A.capE = cg.capE; A.capI = cg.capI;
        const size_t bytes = poly_smem_bytes(D, cg.capC, cg.capV, cg.capF, cg.capE, cg.capI);
        k_poly_cells<D, true><<<gblocks, 128, 0, st>>>(A, big, (int)nbig_host, gbase, (bytes + 255) / 256 * 256,
                                                        nullptr, nullptr);
    } else {
        k_poly_volumes<D><<<(in.n + 255) / 256, 256, 0, st>>>(A, vol);
    }
    return 0;
}

int launch_polygon(const IntegrateInput& in, const PolyCaps& cs, const PolyCaps& cg, int* big, unsigned* nbig,
                   unsigned nbig_host, unsigned char* gbase, int gblocks, double* area, double* vol, int pass,
                   int nsm, cudaStream_t st) {
    int rc = -1;
    HV_DISPATCH(in.d, (rc = poly_t<DD>(in, cs, cg, big, nbig, nbig_host, gbase, gblocks, area, vol, pass, nsm, st)));
    return rc;
}

template <int D>
static int mc_t(const IntegrateInput& in, int ndir, unsigned long long seed, int capN, double cvol, double* rawV,
                double* rawA, double* varV, double* outA, double* vol, int nsm, cudaStream_t st) {
    PolyArgs A = make_args(in);
    const size_t sm = (size_t)MC_WPB * capN * (D + 2) * sizeof(float) + (size_t)MC_WPB * 32 * capN * sizeof(double) + 16;
    if (cudaFuncSetAttribute(k_mc_cells<D>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) != cudaSuccess)
        return -1;
    int blocks = (in.n + MC_WPB - 1) / MC_WPB;
    if (blocks > nsm * 32) blocks = nsm * 32;
    if (blocks < 1) blocks = 1;
    k_mc_cells<D><<<blocks, MC_WPB * 32, sm, st>>>(A, ndir, seed, capN, cvol, rawV, rawA, varV);
    k_mc_pairs<D><<<(in.n + 255) / 256, 256, 0, st>>>(A, rawA, outA);
    k_mc_volumes<D><<<(in.n + 255) / 256, 256, 0, st>>>(A, rawV, rawA, outA, vol);
    return 0;
}

int launch_heuristic_mc(const IntegrateInput& in, int ndir, unsigned long long seed, int capN, double cvol,
                        double* rawV, double* rawA, double* varV, double* outA, double* vol, int nsm,
                        cudaStream_t st) {
    int rc = -1;
    HV_DISPATCH(in.d, (rc = mc_t<DD>(in, ndir, seed, capN, cvol, rawV, rawA, varV, outA, vol, nsm, st)));
    return rc;
}

}  // namespace hv
