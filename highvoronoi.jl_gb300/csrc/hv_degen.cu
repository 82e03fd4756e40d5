// hv_degen.cu -- vertices with more than d+1 generators.
//
// Lattice points and other co-spherical inputs put more than d+1 generators
// on one empty sphere.  The reference stores such a vertex with all of them:
// the tie set of the ray's inrange search joins the edge's generators
// (src/raycast.jl:794-970 with NearestNeighborModified/kd_tree.jl:683-791),
// and the vertex is left along the edges FastEdgeIterator finds
// (src/edgeiterate.jl:82-110).  The fast search breaks such ties and would
// return a wrong mesh, so a build that meets one walks the vertex graph again
// here, with vertices of any number of generators (up to GMAX):
//   vertex (G, c): G every generator with c on its sphere (points) or on its
//     hyperplane (planes); h(x) = (x, 1) for a point, h(p) = (n_p, 0) for a
//     plane;
//   edges of (G, c): directions (u, b) with (u, b).h(g) = 0 for the generators
//     F that stay equidistant / on their plane, < 0 for the rest of G, and F of
//     rank d (one free direction).  Every d-subset of G is tried (one warp per
//     vertex, FP64 Gauss-Jordan); the subset that is F's first basis in slot
//     order emits the edge, so every edge is found once per end point;
//   walk: the next vertex along (c, u) is at the smallest crossing parameter
//     over the generators outside G (planes, then the kd-tree with a shrinking
//     ball); every generator within 1e-9 relative of it joins F;
//   records: each walk of a level writes (G', c'); an insert kernel keeps the
//     first record of each generator set (open addressing on its FNV hash) and
//     a commit kernel appends the kept records to the vertex store.
// Output: the vertices in lexicographic order of their generator lists (CSR),
// the neighbour pairs that share a full interface (neighbors_of_cell,
// src/neighbors.jl:219-258: a vertex with exactly d+1 generators, else the
// shared vertices of affine rank d-1), and VI_POLYGON areas by the pulling
// decomposition of each facet over its faces.
#include <cub/device/device_merge_sort.cuh>

#include "hv_degen.h"

namespace hv {

namespace {

constexpr double GEN_REL = 1e-9;   // ties of the crossing parameter and of F
constexpr double GEN_RANK = 1e-10; // independence of rows / vertex differences

__device__ __forceinline__ unsigned long long gbinom(int a, int b) {
    if (b < 0 || a < b) return 0;
    unsigned long long r = 1;
    for (int q = 1; q <= b; ++q) r = r * (unsigned long long)(a - b + q) / q;
    return r;
}

template <int D>
__device__ __forceinline__ void gen_hom(const GenRun& R, int it, double* h) {
    if (it < R.M.n) {
#pragma unroll
        for (int k = 0; k < D; ++k) h[k] = R.x[(size_t)it * D + k];
        h[D] = 1.0;
    } else {
        const DevPlane& P = R.M.planes[it - R.M.n];
#pragma unroll
        for (int k = 0; k < D; ++k) h[k] = P.n[k];
        h[D] = 0.0;
    }
}

__device__ __forceinline__ bool in_sorted(const int* G, int m, int it) {
    int lo = 0, hi = m;
    while (lo < hi) {
        const int md = (lo + hi) >> 1;
        if (G[md] < it) lo = md + 1; else hi = md;
    }
    return lo < m && G[lo] == it;
}

template <int D>
__device__ __forceinline__ double gen_box_dist2(const DevMesh& M, int node, const double* c) {
    const float* lo = M.blo + (size_t)node * M.dp;
    const float* hi = M.bhi + (size_t)node * M.dp;
    double s = 0;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const double l = (double)lo[k], h = (double)hi[k];
        const double e = c[k] < l ? l - c[k] : (c[k] > h ? c[k] - h : 0.0);
        s = fma(e, e, s);
    }
    return s;
}

// Centre of the vertex with sorted generators G: d independent rows of
// (x_g - x_a).y = |x_g - x_a|^2 / 2 (points) and n_p.y = off_p - n_p.x_a
// (planes), c = x_a + y, x_a the first point of G.
template <int D>
__device__ bool gen_centre(const GenRun& R, const int* G, int m, double* c) {
    int a = -1;
    for (int s = 0; s < m; ++s)
        if (G[s] < R.M.n) { a = G[s]; break; }
    if (a < 0) return false;
    double xa[D];
#pragma unroll
    for (int k = 0; k < D; ++k) xa[k] = R.x[(size_t)a * D + k];
    double A[D][D], b[D], B[D][D];
    int bc[D];
    int nr = 0;
    for (int s = 0; s < m && nr < D; ++s) {
        const int it = G[s];
        if (it == a) continue;
        double row[D], rhs = 0.0, rn = 0.0;
        if (it < R.M.n) {
#pragma unroll
            for (int k = 0; k < D; ++k) {
                row[k] = R.x[(size_t)it * D + k] - xa[k];
                rhs = fma(row[k], row[k], rhs);
            }
            rhs *= 0.5;
        } else {
            const DevPlane& P = R.M.planes[it - R.M.n];
#pragma unroll
            for (int k = 0; k < D; ++k) row[k] = P.n[k];
            rhs = plane_height<D>(P, xa);
        }
        double r[D];
#pragma unroll
        for (int k = 0; k < D; ++k) { r[k] = row[k]; rn = fmax(rn, fabs(row[k])); }
        for (int q = 0; q < nr; ++q) {
            const double f = r[bc[q]] / B[q][bc[q]];
#pragma unroll
            for (int k = 0; k < D; ++k) r[k] -= f * B[q][k];
        }
        int pc = 0;
        double best = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k)
            if (fabs(r[k]) > best) { best = fabs(r[k]); pc = k; }
        if (!(best > GEN_RANK * rn)) continue;
#pragma unroll
        for (int k = 0; k < D; ++k) { B[nr][k] = r[k]; A[nr][k] = row[k]; }
        bc[nr] = pc;
        b[nr] = rhs;
        ++nr;
    }
    if (nr < D) return false;
    int piv[D];
    if (!lu_factor<D, double>(A, piv)) return false;
    lu_solve<D, double>(A, piv, b);
#pragma unroll
    for (int k = 0; k < D; ++k) c[k] = xa[k] + b[k];
    return true;
}

// Null vector of the d x (d+1) matrix H (Gauss-Jordan, partial pivoting);
// false if its rank is below d.
template <int D>
__device__ bool gen_null(double (&H)[D][D + 1], double (&z)[D + 1]) {
    double scale = 0.0;
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
        for (int k = 0; k <= D; ++k) scale = fmax(scale, fabs(H[r][k]));
    int pc[D];
    bool used[D + 1];
#pragma unroll
    for (int k = 0; k <= D; ++k) used[k] = false;
    int rank = 0;
    for (int c = 0; c <= D && rank < D; ++c) {
        int p = rank;
        double best = fabs(H[rank][c]);
        for (int r = rank + 1; r < D; ++r)
            if (fabs(H[r][c]) > best) { best = fabs(H[r][c]); p = r; }
        if (!(best > 1e-12 * scale)) continue;
        if (p != rank)
#pragma unroll
            for (int k = 0; k <= D; ++k) { const double t = H[p][k]; H[p][k] = H[rank][k]; H[rank][k] = t; }
        for (int r = 0; r < D; ++r) {
            if (r == rank) continue;
            const double f = H[r][c] / H[rank][c];
#pragma unroll
            for (int k = 0; k <= D; ++k) H[r][k] -= f * H[rank][k];
        }
        pc[rank] = c;
        used[c] = true;
        ++rank;
    }
    if (rank < D) return false;
    int fc = 0;
    while (used[fc]) ++fc;
#pragma unroll
    for (int k = 0; k <= D; ++k) z[k] = 0.0;
    z[fc] = 1.0;
    for (int r = 0; r < D; ++r) z[pc[r]] = -H[r][fc] / H[r][pc[r]];
    return true;
}

// Is idx the first basis of the slots in Fm (greedy in slot order)?
template <int D>
__device__ bool gen_first_basis(const double (*h)[D + 1], unsigned long long Fm, const int (&idx)[D]) {
    double B[D][D + 1];
    int bc[D];
    int nb = 0;
    for (unsigned long long f = Fm; f && nb < D; f &= f - 1) {
        const int a = __ffsll((long long)f) - 1;
        double r[D + 1], rn = 0.0;
#pragma unroll
        for (int k = 0; k <= D; ++k) { r[k] = h[a][k]; rn = fmax(rn, fabs(r[k])); }
        for (int q = 0; q < nb; ++q) {
            const double fct = r[bc[q]] / B[q][bc[q]];
#pragma unroll
            for (int k = 0; k <= D; ++k) r[k] -= fct * B[q][k];
        }
        int c = 0;
        double best = 0.0;
#pragma unroll
        for (int k = 0; k <= D; ++k)
            if (fabs(r[k]) > best) { best = fabs(r[k]); c = k; }
        if (!(best > GEN_RANK * rn)) continue;
        if (a != idx[nb]) return false;
#pragma unroll
        for (int k = 0; k <= D; ++k) B[nb][k] = r[k];
        bc[nb] = c;
        ++nb;
    }
    return nb == D;
}

template <int D>
__device__ __forceinline__ void gen_unrank(unsigned long long q, int m, int (&idx)[D]) {
    int x = 0;
#pragma unroll
    for (int p = 0; p < D; ++p) {
        for (;;) {
            const unsigned long long c = gbinom(m - x - 1, D - p - 1);
            if (q < c) break;
            q -= c;
            ++x;
        }
        idx[p] = x++;
    }
}

constexpr int GEN_WPB = 4;

template <int D>
__global__ void __launch_bounds__(GEN_WPB * 32) k_gen_edges(GenRun R, unsigned f0, unsigned f1) {
    __shared__ int sG[GEN_WPB][GMAX];
    __shared__ double sH[GEN_WPB][GMAX][D + 1];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (unsigned v = f0 + blockIdx.x * GEN_WPB + w; v < f1; v += gridDim.x * GEN_WPB) {
        const int m = R.vlen[v];
        for (int a = lane; a < m; a += 32) {
            const int it = R.vsig[(size_t)v * R.W + a];
            sG[w][a] = it;
            gen_hom<D>(R, it, sH[w][a]);
        }
        __syncwarp();
        const unsigned long long tot = gbinom(m, D);
        if (tot > (1ull << 22)) {
            if (lane == 0) atomicOr(R.status, GS_SUBSETS);
            __syncwarp();
            continue;
        }
        for (unsigned long long q = lane; q < tot; q += 32) {
            int idx[D];
            gen_unrank<D>(q, m, idx);
            double H[D][D + 1], z[D + 1];
#pragma unroll
            for (int r = 0; r < D; ++r)
#pragma unroll
                for (int k = 0; k <= D; ++k) H[r][k] = sH[w][idx[r]][k];
            if (!gen_null<D>(H, z)) continue;
            int pos = 0, neg = 0;
            bool real = false;
            unsigned long long Fm = 0;
            for (int a = 0; a < m; ++a) {
                double s = 0.0, sa = 0.0;
#pragma unroll
                for (int k = 0; k <= D; ++k) {
                    const double p = z[k] * sH[w][a][k];
                    s += p;
                    sa += fabs(p);
                }
                if (fabs(s) <= GEN_REL * sa) {
                    Fm |= 1ull << a;
                    real |= sG[w][a] < R.M.n;
                } else if (s > 0) {
                    ++pos;
                } else {
                    ++neg;
                }
            }
            if ((pos > 0 && neg > 0) || pos + neg == 0 || !real) continue;
            if (!gen_first_basis<D>(sH[w], Fm, idx)) continue;
            const unsigned e = atomicAdd(R.e_cnt, 1u);
            if (e >= R.e_cap) continue;  // counted: the host grows the buffer and redoes the level
            double un = 0.0;
#pragma unroll
            for (int k = 0; k < D; ++k) un = fma(z[k], z[k], un);
            const double sc = (pos > 0 ? -1.0 : 1.0) / sqrt(un);
            R.e_vert[e] = v;
            R.e_F[e] = Fm;
#pragma unroll
            for (int k = 0; k < D; ++k) R.e_u[(size_t)e * D + k] = sc * z[k];
        }
        __syncwarp();
    }
}

template <int D>
__global__ void __launch_bounds__(128) k_gen_walk(GenRun R, unsigned ne) {
    for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
        const unsigned v = R.e_vert[e];
        const int* G = R.vsig + (size_t)v * R.W;
        const int m = R.vlen[v];
        const unsigned long long Fm = R.e_F[e];
        double c[D], u[D], xa[D];
#pragma unroll
        for (int k = 0; k < D; ++k) { c[k] = R.vc[(size_t)v * D + k]; u[k] = R.e_u[(size_t)e * D + k]; }
        int a = -1;
        for (unsigned long long f = Fm; f; f &= f - 1) {
            const int it = G[__ffsll((long long)f) - 1];
            if (it < R.M.n) { a = it; break; }
        }
        if (a < 0) { atomicOr(R.status, GS_NUMERIC); continue; }
        double ca = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            xa[k] = R.x[(size_t)a * D + k];
            const double w = c[k] - xa[k];
            ca = fma(w, w, ca);
        }
        const double rad = sqrt(ca);
        auto tolf = [&](double t) { return GEN_REL * (fabs(t) + rad); };
        double tb = INFINITY;
        double tt[GMAX];
        int ti[GMAX];
        int nt = 0;
        bool over = false;
        auto consider = [&](double t, int it) {
            if (!(t <= tb + tolf(tb))) return;
            if (t < tb) {
                tb = t;
                int w = 0;
                for (int q = 0; q < nt; ++q)
                    if (tt[q] <= tb + tolf(tb)) { tt[w] = tt[q]; ti[w] = ti[q]; ++w; }
                nt = w;
            }
            if (nt < GMAX) { tt[nt] = t; ti[nt] = it; ++nt; }
            else over = true;
        };
        for (int p = 0; p < R.M.np; ++p) {
            const int it = R.M.n + p;
            if (in_sorted(G, m, it)) continue;
            const DevPlane& P = R.M.planes[p];
            double un = 0.0;
#pragma unroll
            for (int k = 0; k < D; ++k) un = fma(P.n[k], u[k], un);
            if (!(un > 1e-12)) continue;
            consider(plane_height<D>(P, c) / un, it);
        }
        int stack[64];
        int sp = 0;
        stack[sp++] = 1;
        while (sp > 0) {
            const int node = stack[--sp];
            const double tl = tb + tolf(tb);
            double ct[D], r2 = 0.0;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                ct[k] = isfinite(tl) ? fma(tl, u[k], c[k]) : c[k];
                const double w = ct[k] - xa[k];
                r2 = fma(w, w, r2);
            }
            if (isfinite(tl) && gen_box_dist2<D>(R.M, node, ct) > r2 * (1.0 + 1e-9) + 1e-300) continue;
            if (node >= R.M.P) {
                const int l = node - R.M.P;
                if (l >= R.M.nleaves) continue;
                const int s0 = l * R.M.leaf, s1 = min(s0 + R.M.leaf, R.M.n);
                for (int j = s0; j < s1; ++j) {
                    const int jo = R.M.perm[j];
                    if (in_sorted(G, m, jo)) continue;
                    const double* xj = R.M.pts + (size_t)j * D;
                    double den = 0.0, cj = 0.0, dn = 0.0;
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        const double dl = xj[k] - xa[k];
                        den = fma(u[k], dl, den);
                        dn = fmax(dn, fabs(dl));
                        const double w = c[k] - xj[k];
                        cj = fma(w, w, cj);
                    }
                    den *= 2.0;
                    if (!(den > 1e-12 * dn)) continue;
                    consider((cj - ca) / den, jo);
                }
            } else {
                // the child nearer the vertex first: the generators met first along
                // the edge lie near it, and the ball shrinks before the farther
                // child is tested
                if (sp + 2 > 64) { over = true; break; }
                const double dl = gen_box_dist2<D>(R.M, 2 * node, c), dr = gen_box_dist2<D>(R.M, 2 * node + 1, c);
                if (dl <= dr) { stack[sp++] = 2 * node + 1; stack[sp++] = 2 * node; }
                else { stack[sp++] = 2 * node; stack[sp++] = 2 * node + 1; }
            }
        }
        if (!isfinite(tb) || over) { atomicOr(R.status, over ? GS_WIDE : GS_NUMERIC); continue; }
        // G' = F + the ties, sorted
        int T[GMAX];
        int nT = 0;
        for (int q = 0; q < nt; ++q)
            if (tt[q] <= tb + tolf(tb)) {
                int x = nT++;
                while (x > 0 && T[x - 1] > ti[q]) { T[x] = T[x - 1]; --x; }
                T[x] = ti[q];
            }
        const int nF = __popcll((long long)Fm);
        if (nF + nT > R.W) { atomicOr(R.status, GS_WIDE); continue; }
        const unsigned r = atomicAdd(R.rcnt, 1u);  // rcap >= edges: always room
        int* out = R.rsig + (size_t)r * R.W;
        int nout = 0, qT = 0;
        for (unsigned long long f = Fm; f; f &= f - 1) {
            const int it = G[__ffsll((long long)f) - 1];
            while (qT < nT && T[qT] < it) out[nout++] = T[qT++];
            out[nout++] = it;
        }
        while (qT < nT) out[nout++] = T[qT++];
        R.rlen[r] = nout;
        R.rwin[r] = 0;
        if (!gen_centre<D>(R, out, nout, R.rc + (size_t)r * D)) atomicOr(R.status, GS_NUMERIC);
    }
}

__device__ __forceinline__ bool gen_same(const int* A, int ma, const int* B, int mb) {
    if (ma != mb) return false;
    for (int s = 0; s < ma; ++s)
        if (A[s] != B[s]) return false;
    return true;
}

__device__ __forceinline__ unsigned long long gen_hash(const int* G, int m) {
    unsigned long long h = 1469598103934665603ull;
    for (int s = 0; s < m; ++s) { h ^= (unsigned)G[s]; h *= 1099511628211ull; }
    return h;
}

// First record of each generator set: the slot's CAS winner (rwin = slot + 1).
// A slot holds a vertex of an earlier level or a record of this one, both
// complete when this kernel runs.
__global__ void k_gen_insert(GenRun R, unsigned nrec) {
    for (unsigned r = blockIdx.x * blockDim.x + threadIdx.x; r < nrec; r += gridDim.x * blockDim.x) {
        const int m = R.rlen[r];
        const int* G = R.rsig + (size_t)r * R.W;
        unsigned long long slot = gen_hash(G, m) & R.hmask;
        bool done = false;
        for (unsigned long long probe = 0; probe <= R.hmask && !done; ++probe) {
            const unsigned long long old = atomicCAS(R.htab + slot, SLOT_EMPTY, REC_TAG | r);
            if (old == SLOT_EMPTY) {
                R.rwin[r] = (unsigned)slot + 1u;
                done = true;
            } else if (old & REC_TAG) {
                const unsigned q = (unsigned)(old & 0xFFFFFFFFull);
                done = gen_same(R.rsig + (size_t)q * R.W, R.rlen[q], G, m);
            } else {
                done = gen_same(R.vsig + old * R.W, R.vlen[old], G, m);
            }
            if (!done) slot = (slot + 1) & R.hmask;
        }
        if (!done) atomicOr(R.status, GS_HASH);
    }
}

template <int D>
__global__ void k_gen_commit(GenRun R, unsigned nrec) {
    for (unsigned r = blockIdx.x * blockDim.x + threadIdx.x; r < nrec; r += gridDim.x * blockDim.x) {
        const unsigned w = R.rwin[r];
        if (!w) continue;
        const unsigned v = atomicAdd(R.vcnt, 1u);
        if (v >= R.vcap) { atomicOr(R.status, GS_CAP); continue; }
        const int m = R.rlen[r];
        for (int s = 0; s < m; ++s) R.vsig[(size_t)v * R.W + s] = R.rsig[(size_t)r * R.W + s];
        R.vlen[v] = m;
#pragma unroll
        for (int k = 0; k < D; ++k) R.vc[(size_t)v * D + k] = R.rc[(size_t)r * D + k];
        R.htab[w - 1] = v;
    }
}

// Vertex 0: the domain corner v with the planes through it and its nearest
// generators (all within 2e-9 relative of the smallest squared distance).
constexpr int SEED_T = 256;
template <int D>
__global__ void __launch_bounds__(SEED_T) k_gen_seed(GenRun R, const double* v) {
    __shared__ double smin[SEED_T];
    __shared__ int sG[GMAX];
    __shared__ int sm;
    __shared__ int sover;
    double c[D];
#pragma unroll
    for (int k = 0; k < D; ++k) c[k] = v[k];
    auto dist2 = [&](int j) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) { const double w = R.x[(size_t)j * D + k] - c[k]; s = fma(w, w, s); }
        return s;
    };
    double mn = INFINITY;
    for (int j = threadIdx.x; j < R.M.n; j += SEED_T) mn = fmin(mn, dist2(j));
    smin[threadIdx.x] = mn;
    if (threadIdx.x == 0) { sm = 0; sover = 0; }
    __syncthreads();
    for (int w = SEED_T / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + w]);
        __syncthreads();
    }
    const double dmin = smin[0];
    for (int j = threadIdx.x; j < R.M.n; j += SEED_T)
        if (dist2(j) <= dmin * (1.0 + 2.0 * GEN_REL)) {
            const int q = atomicAdd(&sm, 1);
            if (q < GMAX) sG[q] = j;
            else sover = 1;
        }
    __syncthreads();
    if (threadIdx.x != 0) return;
    const double rad = sqrt(dmin);
    int m = min(sm, GMAX);
    for (int p = 0; p < R.M.np; ++p)
        if (fabs(plane_height<D>(R.M.planes[p], c)) <= GEN_REL * (rad + 1e-300)) {
            if (m < GMAX) sG[m++] = R.M.n + p;
            else sover = 1;
        }
    if (sover || m > R.W) { atomicOr(R.status, GS_WIDE); return; }
    for (int a = 1; a < m; ++a) {
        const int x = sG[a];
        int b = a - 1;
        while (b >= 0 && sG[b] > x) { sG[b + 1] = sG[b]; --b; }
        sG[b + 1] = x;
    }
    for (int q = 0; q < m; ++q) R.vsig[q] = sG[q];
    R.vlen[0] = m;
    if (!gen_centre<D>(R, sG, m, R.vc)) atomicOr(R.status, GS_NUMERIC);
    R.htab[gen_hash(sG, m) & R.hmask] = 0;
    *R.vcnt = 1;
}

// Records of the search's vertices (d+1 internal ids each; the search broke
// the ties by index, but every sphere it found is empty): each completed with
// every generator on its sphere, so that the walk starts from all of them.
template <int D>
__global__ void __launch_bounds__(128) k_gen_seeds(GenRun R, const int* vsig, unsigned nseed) {
    for (unsigned v = blockIdx.x * blockDim.x + threadIdx.x; v < nseed; v += gridDim.x * blockDim.x) {
        int sig[D + 1];
#pragma unroll
        for (int k = 0; k <= D; ++k) {
            const int it = vsig[(size_t)v * (D + 1) + k];
            sig[k] = it < R.M.n ? R.M.perm[it] : it;
        }
        for (int a = 1; a <= D; ++a) {
            const int x = sig[a];
            int b = a - 1;
            while (b >= 0 && sig[b] > x) { sig[b + 1] = sig[b]; --b; }
            sig[b + 1] = x;
        }
        double c[D];
        if (!gen_centre<D>(R, sig, D + 1, c)) continue;  // a singular system: other seeds remain
        double ca = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) { const double w = c[k] - R.x[(size_t)sig[0] * D + k]; ca = fma(w, w, ca); }
        const double rad = sqrt(ca);
        int G[GMAX];
        int m = 0;
        bool over = false;
        auto add = [&](int it) {
            if (m == GMAX) { over = true; return; }
            int x = m++;
            while (x > 0 && G[x - 1] > it) { G[x] = G[x - 1]; --x; }
            G[x] = it;
        };
        int stack[64];
        int sp = 0;
        stack[sp++] = 1;
        while (sp > 0 && !over) {
            const int node = stack[--sp];
            if (gen_box_dist2<D>(R.M, node, c) > ca * (1.0 + 4.0 * GEN_REL) + 1e-300) continue;
            if (node >= R.M.P) {
                const int l = node - R.M.P;
                if (l >= R.M.nleaves) continue;
                const int s0 = l * R.M.leaf, s1 = min(s0 + R.M.leaf, R.M.n);
                for (int j = s0; j < s1; ++j) {
                    double dj = 0.0;
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        const double w = c[k] - R.M.pts[(size_t)j * D + k];
                        dj = fma(w, w, dj);
                    }
                    if (fabs(dj - ca) <= 2.0 * GEN_REL * ca) add(R.M.perm[j]);
                }
            } else {
                if (sp + 2 > 64) { over = true; break; }
                stack[sp++] = 2 * node + 1;
                stack[sp++] = 2 * node;
            }
        }
        for (int p = 0; p < R.M.np; ++p)
            if (fabs(plane_height<D>(R.M.planes[p], c)) <= GEN_REL * (rad + 1e-300)) add(R.M.n + p);
        if (over || m > R.W) { atomicOr(R.status, GS_WIDE); continue; }
        double cg[D];
        if (!gen_centre<D>(R, G, m, cg)) continue;  // other seeds remain
        const unsigned r = atomicAdd(R.rcnt, 1u);  // rcap >= nseed
        for (int q = 0; q < m; ++q) R.rsig[(size_t)r * R.W + q] = G[q];
        R.rlen[r] = m;
        R.rwin[r] = 0;
#pragma unroll
        for (int k = 0; k < D; ++k) R.rc[(size_t)r * D + k] = cg[k];
    }
}

// ---- output
struct GenLess {
    const int* vsig;
    const int* vlen;
    int W;
    __device__ bool operator()(const int& a, const int& b) const {
        const int ma = vlen[a], mb = vlen[b];
        const int* A = vsig + (size_t)a * W;
        const int* B = vsig + (size_t)b * W;
        const int m = ma < mb ? ma : mb;
        for (int s = 0; s < m; ++s)
            if (A[s] != B[s]) return A[s] < B[s];
        return ma < mb;
    }
};

__global__ void k_iota_i(int* o, unsigned V) {
    for (unsigned v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) o[v] = (int)v;
}

__global__ void k_gen_lens(GenRun R, unsigned V, const int* order, long long* lens, unsigned* maxlen) {
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < V; o += gridDim.x * blockDim.x) {
        const int m = R.vlen[order[o]];
        lens[o] = m;
        atomicMax(maxlen, (unsigned)m);
    }
}

template <int D>
__global__ void k_gen_fill(GenRun R, unsigned V, const int* order, const long long* off, int* sig, double* oc) {
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < V; o += gridDim.x * blockDim.x) {
        const int v = order[o];
        const int m = R.vlen[v];
        for (int s = 0; s < m; ++s) sig[off[o] + s] = R.vsig[(size_t)v * R.W + s];
#pragma unroll
        for (int k = 0; k < D; ++k) oc[(size_t)o * D + k] = R.vc[(size_t)v * D + k];
    }
}

__global__ void k_gen_pair_count(int n, unsigned V, const long long* off, const int* sig, long long* cnt) {
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < V; o += gridDim.x * blockDim.x) {
        const long long m = off[o + 1] - off[o];
        long long reals = 0;
        for (long long s = off[o]; s < off[o + 1]; ++s) reals += sig[s] < n;
        cnt[o] = reals * (m - 1);
    }
}

__global__ void k_gen_pair_emit(int n, unsigned V, const long long* off, const int* sig, const long long* poff,
                                unsigned long long* keys, int* vals) {
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < V; o += gridDim.x * blockDim.x) {
        long long p = poff[o];
        for (long long s = off[o]; s < off[o + 1]; ++s) {
            const int i = sig[s];
            if (i >= n) continue;
            for (long long t = off[o]; t < off[o + 1]; ++t) {
                if (t == s) continue;
                keys[p] = ((unsigned long long)(unsigned)i << 32) | (unsigned)sig[t];
                vals[p] = (int)o;
                ++p;
            }
        }
    }
}

// Affine rank of the points and the orthonormal basis of their differences.
template <int D>
__device__ int gen_mgs(const double* oc, const int* rows, int nr, double (&Q)[D][D]) {
    int r = 0;
    const double* p0 = oc + (size_t)rows[0] * D;
    for (int a = 1; a < nr && r < D; ++a) {
        const double* pa = oc + (size_t)rows[a] * D;
        double v[D], n0 = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) { v[k] = pa[k] - p0[k]; n0 = fmax(n0, fabs(v[k])); }
        for (int b = 0; b < r; ++b) {
            double s = 0.0;
#pragma unroll
            for (int k = 0; k < D; ++k) s = fma(v[k], Q[b][k], s);
#pragma unroll
            for (int k = 0; k < D; ++k) v[k] -= s * Q[b][k];
        }
        double nn = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) nn = fma(v[k], v[k], nn);
        const double len = sqrt(nn);
        if (!(len > GEN_RANK * n0)) continue;
#pragma unroll
        for (int k = 0; k < D; ++k) Q[r][k] = v[k] / len;
        ++r;
    }
    return r;
}

template <int D>
__global__ void k_gen_heads(long long npairs, const unsigned long long* keys, const int* vals, const long long* off,
                            const double* oc, long long* keep, long long* qend) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < npairs;
         q += (long long)gridDim.x * blockDim.x) {
        if (q > 0 && keys[q] == keys[q - 1]) { keep[q] = 0; continue; }
        long long e = q + 1;
        while (e < npairs && keys[e] == keys[q]) ++e;
        qend[q] = e;
        bool full = false;
        for (long long t = q; t < e && !full; ++t) full = off[vals[t] + 1] - off[vals[t]] == D + 1;
        if (!full) {
            // the shared vertices span d-1 dimensions (a full interface)
            int rows[GMAX];
            int nr = 0;
            for (long long t = q; t < e && nr < GMAX; ++t) rows[nr++] = vals[t];
            double Q[D][D];
            full = gen_mgs<D>(oc, rows, nr, Q) >= D - 1;
        }
        keep[q] = full ? 1 : 0;
    }
}

__global__ void k_gen_slots(long long npairs, const unsigned long long* keys, const long long* keep,
                            const long long* kpos, const long long* qend, int* nbr, int* fcell, long long* fbeg,
                            long long* fend, long long* ncnt) {
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < npairs;
         q += (long long)gridDim.x * blockDim.x) {
        if (!keep[q]) continue;
        const long long pos = kpos[q];
        const int i = (int)(keys[q] >> 32);
        nbr[pos] = (int)(keys[q] & 0xFFFFFFFFull);
        fcell[pos] = i;
        fbeg[pos] = q;
        fend[pos] = qend[q];
        atomicAdd((unsigned long long*)(ncnt + i), 1ull);
    }
}

__global__ void k_gen_inc_emit(int n, unsigned V, const long long* off, const int* sig, unsigned long long* keys,
                               long long* cnt) {
    for (unsigned o = blockIdx.x * blockDim.x + threadIdx.x; o < V; o += gridDim.x * blockDim.x)
        for (long long s = off[o]; s < off[o + 1]; ++s) {
            const int i = sig[s];
            if (i < n) {
                keys[s] = ((unsigned long long)(unsigned)i << 32) | o;
                atomicAdd((unsigned long long*)(cnt + i), 1ull);
            } else {
                keys[s] = ~0ull;
            }
        }
}

// ---- VI_POLYGON of such a mesh
__device__ __forceinline__ bool gen_has(const GenPoly& P, int v, int it) {
    long long lo = P.off[v], hi = P.off[v + 1];
    while (lo < hi) {
        const long long md = (lo + hi) >> 1;
        if (P.sig[md] < it) lo = md + 1; else hi = md;
    }
    return lo < P.off[v + 1] && P.sig[lo] == it;
}

constexpr int GEN_SEEN = 32;  // facets of one face

// (DIM)-volume of the face whose vertices are the bits of mask over fv:
// sum over its facets (the vertices that also carry one more generator l,
// affine rank DIM-1) that miss the face's first vertex v0 of
// dist(v0, facet) * vol(facet) / DIM.
template <int D, int DIM>
__device__ double gen_face(const GenPoly& P, const int* fv, unsigned long long mask) {
    if constexpr (DIM == 1) {
        double best = 0.0;
        for (unsigned long long ma = mask; ma; ma &= ma - 1) {
            const double* pa = P.oc + (size_t)fv[__ffsll((long long)ma) - 1] * D;
            for (unsigned long long mb = ma & (ma - 1); mb; mb &= mb - 1) {
                const double* pb = P.oc + (size_t)fv[__ffsll((long long)mb) - 1] * D;
                double s = 0.0;
#pragma unroll
                for (int k = 0; k < D; ++k) { const double w = pa[k] - pb[k]; s = fma(w, w, s); }
                best = fmax(best, s);
            }
        }
        return sqrt(best);
    } else {
        const int a0 = __ffsll((long long)mask) - 1;
        const int v0 = fv[a0];
        unsigned long long seen[GEN_SEEN];
        int ns = 0;
        double total = 0.0;
        for (unsigned long long ma = mask; ma; ma &= ma - 1) {
            const int a = __ffsll((long long)ma) - 1;
            const int va = fv[a];
            for (long long s = P.off[va]; s < P.off[va + 1]; ++s) {
                const int l = P.sig[s];
                bool earlier = false;  // count l once: at its first vertex in the face
                for (unsigned long long mb = mask & ((1ull << a) - 1); mb && !earlier; mb &= mb - 1)
                    earlier = gen_has(P, fv[__ffsll((long long)mb) - 1], l);
                if (earlier) continue;
                unsigned long long sub = 0;
                for (unsigned long long mb = mask; mb; mb &= mb - 1) {
                    const int b = __ffsll((long long)mb) - 1;
                    if (b == a || gen_has(P, fv[b], l)) sub |= 1ull << b;
                }
                if (sub == mask || ((sub >> a0) & 1ull) || __popcll((long long)sub) < DIM) continue;
                bool dup = false;
                for (int q = 0; q < ns; ++q) dup |= seen[q] == sub;
                if (dup) continue;
                if (ns == GEN_SEEN) { atomicOr(P.status, GS_FACET); return 0.0; }
                seen[ns++] = sub;
                int rows[GMAX];
                int nr = 0;
                for (unsigned long long mb = sub; mb; mb &= mb - 1) rows[nr++] = fv[__ffsll((long long)mb) - 1];
                double Q[D][D];
                if (gen_mgs<D>(P.oc, rows, nr, Q) != DIM - 1) continue;
                double w[D];
#pragma unroll
                for (int k = 0; k < D; ++k) w[k] = P.oc[(size_t)v0 * D + k] - P.oc[(size_t)rows[0] * D + k];
                for (int b = 0; b < DIM - 1; ++b) {
                    double sdot = 0.0;
#pragma unroll
                    for (int k = 0; k < D; ++k) sdot = fma(w[k], Q[b][k], sdot);
#pragma unroll
                    for (int k = 0; k < D; ++k) w[k] -= sdot * Q[b][k];
                }
                double hh = 0.0;
#pragma unroll
                for (int k = 0; k < D; ++k) hh = fma(w[k], w[k], hh);
                total += sqrt(hh) * gen_face<D, DIM - 1>(P, fv, sub) / DIM;
            }
        }
        return total;
    }
}

template <int D>
__device__ __forceinline__ double gen_h(const GenPoly& P, int i, int k) {
    const double* xi = P.pts + (size_t)i * D;
    if (k >= P.n) return plane_height<D>(P.planes[k - P.n], xi);
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < D; ++q) { const double e = P.pts[(size_t)k * D + q] - xi[q]; s = fma(e, e, s); }
    return 0.5 * sqrt(s);
}

template <int D>
__global__ void __launch_bounds__(64) k_gen_facets(GenPoly P, double* area) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < P.nslots;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = P.fcell[t], k = P.nbr[t];
        if (k < P.n && k < i) continue;  // the lower cell computes the facet
        const long long nf = P.fend[t] - P.fbeg[t];
        if (nf > GMAX) { atomicOr(P.status, GS_FACET); area[t] = 0.0; continue; }
        const int* fv = P.fvert + P.fbeg[t];
        const unsigned long long mask = nf == 64 ? ~0ull : ((1ull << nf) - 1ull);
        area[t] = gen_face<D, D - 1>(P, fv, mask);
    }
}

__global__ void k_gen_copy(GenPoly P, double* area) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < P.nslots;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = P.fcell[t], k = P.nbr[t];
        if (!(k < P.n && k < i)) continue;
        long long lo = P.nbr_off[k], hi = P.nbr_off[k + 1] - 1;
        if (hi < lo) { area[t] = 0.0; continue; }
        while (lo < hi) {
            const long long md = (lo + hi) >> 1;
            if (P.nbr[md] < i) lo = md + 1; else hi = md;
        }
        area[t] = P.nbr[lo] == i ? area[lo] : 0.0;
    }
}

template <int D>
__global__ void k_gen_volumes(GenPoly P, const double* area, double* vol) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x) {
        double v = 0.0;
        for (long long t = P.nbr_off[i]; t < P.nbr_off[i + 1]; ++t) v += area[t] * gen_h<D>(P, i, P.nbr[t]) / D;
        vol[i] = v;
    }
}

// The reference's vertex verification (verify_vertex / fraud_vertex,
// src/raycast.jl:477-502, src/sysvoronoi.jl:527-552): no generator strictly
// inside a vertex's sphere.  One thread per vertex: the deviation of its
// generators from the sphere (points) or of the centre from their planes, a
// ball query of the kd-tree, and the planes it does not carry.
template <int D>
__global__ void k_verify(DevMesh M, const double* x, unsigned V, const long long* off, const int* sig,
                         const double* oc, unsigned long long* cnt, unsigned long long* maxdev) {
    for (unsigned v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        const long long s0 = off ? off[v] : (long long)v * (D + 1);
        const long long s1 = off ? off[v + 1] : s0 + D + 1;
        const int* G = sig + s0;
        const int m = (int)(s1 - s0);
        double c[D];
#pragma unroll
        for (int k = 0; k < D; ++k) c[k] = oc[(size_t)v * D + k];
        int a = -1;
        for (int q = 0; q < m; ++q)
            if (G[q] < M.n) { a = G[q]; break; }
        if (a < 0) { atomicAdd(cnt, 1ull); continue; }
        double r2 = 0.0;
#pragma unroll
        for (int k = 0; k < D; ++k) { const double w = c[k] - x[(size_t)a * D + k]; r2 = fma(w, w, r2); }
        const double rad = sqrt(r2);
        double dev = 0.0;
        for (int q = 0; q < m; ++q) {
            const int it = G[q];
            if (it < M.n) {
                double s = 0.0;
#pragma unroll
                for (int k = 0; k < D; ++k) { const double w = c[k] - x[(size_t)it * D + k]; s = fma(w, w, s); }
                dev = fmax(dev, fabs(s - r2) / r2);
            } else {
                dev = fmax(dev, fabs(plane_height<D>(M.planes[it - M.n], c)) / rad);
            }
        }
        bool inside = false, tie = false;
        for (int p = 0; p < M.np; ++p) {
            if (in_sorted(G, m, M.n + p)) continue;
            const double h = plane_height<D>(M.planes[p], c);
            if (h < -1e-10 * rad) inside = true;
            else if (h <= 1e-10 * rad) tie = true;
        }
        int stack[64];
        int sp = 0;
        stack[sp++] = 1;
        while (sp > 0 && !inside) {
            const int node = stack[--sp];
            if (gen_box_dist2<D>(M, node, c) > r2 * (1.0 + 1e-9)) continue;
            if (node >= M.P) {
                const int l = node - M.P;
                if (l >= M.nleaves) continue;
                const int j0 = l * M.leaf, j1 = min(j0 + M.leaf, M.n);
                for (int j = j0; j < j1; ++j) {
                    if (in_sorted(G, m, M.perm[j])) continue;
                    double s = 0.0;
#pragma unroll
                    for (int k = 0; k < D; ++k) { const double w = c[k] - M.pts[(size_t)j * D + k]; s = fma(w, w, s); }
                    if (s < r2 * (1.0 - 1e-10)) inside = true;
                    else if (s <= r2 * (1.0 + 1e-10)) tie = true;
                }
            } else {
                if (sp + 2 > 64) { inside = true; break; }
                stack[sp++] = 2 * node + 1;
                stack[sp++] = 2 * node;
            }
        }
        if (inside) atomicAdd(cnt, 1ull);
        if (tie) atomicAdd(cnt + 1, 1ull);
        atomicMax(maxdev, (unsigned long long)__double_as_longlong(dev));
    }
}

unsigned gen_grid(unsigned long long n, int bs, unsigned cap = 1u << 20) {
    unsigned long long g = (n + bs - 1) / bs;
    if (g < 1) g = 1;
    return (unsigned)std::min<unsigned long long>(g, cap);
}

}  // namespace

#define HV_DISPATCH(d, CALL)                           \
    switch (d) {                                       \
        case 2: { constexpr int DD = 2; CALL; } break; \
        case 3: { constexpr int DD = 3; CALL; } break; \
        case 4: { constexpr int DD = 4; CALL; } break; \
        case 5: { constexpr int DD = 5; CALL; } break; \
        case 6: { constexpr int DD = 6; CALL; } break; \
        default: break;                                \
    }

void launch_gen_seed(const GenRun& R, const double* corner, cudaStream_t st) {
    HV_DISPATCH(R.M.d, (k_gen_seed<DD><<<1, SEED_T, 0, st>>>(R, corner)));
}

void launch_gen_seeds(const GenRun& R, const int* vsig, unsigned nseed, int nsm, cudaStream_t st) {
    if (!nseed) return;
    HV_DISPATCH(R.M.d, (k_gen_seeds<DD><<<gen_grid(nseed, 128, (unsigned)nsm * 16), 128, 0, st>>>(R, vsig, nseed)));
}

void launch_gen_edges(const GenRun& R, unsigned f0, unsigned f1, int nsm, cudaStream_t st) {
    if (f1 <= f0) return;
    const unsigned g = gen_grid(f1 - f0, GEN_WPB, (unsigned)nsm * 16);
    HV_DISPATCH(R.M.d, (k_gen_edges<DD><<<g, GEN_WPB * 32, 0, st>>>(R, f0, f1)));
}

void launch_gen_walk(const GenRun& R, unsigned ne, int nsm, cudaStream_t st) {
    if (!ne) return;
    HV_DISPATCH(R.M.d, (k_gen_walk<DD><<<gen_grid(ne, 128, (unsigned)nsm * 16), 128, 0, st>>>(R, ne)));
}

void launch_gen_insert(const GenRun& R, unsigned nrec, cudaStream_t st) {
    if (!nrec) return;
    k_gen_insert<<<gen_grid(nrec, 256), 256, 0, st>>>(R, nrec);
}

void launch_gen_commit(const GenRun& R, unsigned nrec, cudaStream_t st) {
    if (!nrec) return;
    HV_DISPATCH(R.M.d, (k_gen_commit<DD><<<gen_grid(nrec, 256), 256, 0, st>>>(R, nrec)));
}

size_t gen_sort_temp(unsigned V) {
    size_t b = 0;
    GenLess cmp{nullptr, nullptr, 0};
    cub::DeviceMergeSort::SortKeys(nullptr, b, (int*)nullptr, (long long)std::max(V, 1u), cmp);
    return b;
}

void gen_sort(const GenRun& R, unsigned V, int* order, void* temp, size_t temp_bytes, cudaStream_t st) {
    if (!V) return;
    k_iota_i<<<gen_grid(V, 256), 256, 0, st>>>(order, V);
    GenLess cmp{R.vsig, R.vlen, R.W};
    cub::DeviceMergeSort::SortKeys(temp, temp_bytes, order, (long long)V, cmp, st);
}

void launch_gen_lens(const GenRun& R, unsigned V, const int* order, long long* lens, unsigned* maxlen,
                     cudaStream_t st) {
    if (!V) return;
    k_gen_lens<<<gen_grid(V, 256), 256, 0, st>>>(R, V, order, lens, maxlen);
}

void launch_gen_fill(const GenRun& R, unsigned V, const int* order, const long long* off, int* sig, double* oc,
                     cudaStream_t st) {
    if (!V) return;
    HV_DISPATCH(R.M.d, (k_gen_fill<DD><<<gen_grid(V, 256), 256, 0, st>>>(R, V, order, off, sig, oc)));
}

void launch_gen_pair_count(int n, unsigned V, const long long* off, const int* sig, long long* cnt,
                           cudaStream_t st) {
    if (!V) return;
    k_gen_pair_count<<<gen_grid(V, 256), 256, 0, st>>>(n, V, off, sig, cnt);
}

void launch_gen_pair_emit(int n, unsigned V, const long long* off, const int* sig, const long long* poff,
                          unsigned long long* keys, int* vals, cudaStream_t st) {
    if (!V) return;
    k_gen_pair_emit<<<gen_grid(V, 256), 256, 0, st>>>(n, V, off, sig, poff, keys, vals);
}

void launch_gen_heads(int d, long long npairs, const unsigned long long* keys, const int* vals, const long long* off,
                      const double* oc, long long* keep, long long* qend, cudaStream_t st) {
    if (npairs <= 0) return;
    HV_DISPATCH(d, (k_gen_heads<DD><<<gen_grid(npairs, 128), 128, 0, st>>>(npairs, keys, vals, off, oc, keep, qend)));
}

void launch_gen_slots(long long npairs, const unsigned long long* keys, const long long* keep,
                      const long long* kpos, const long long* qend, int* nbr, int* fcell, long long* fbeg,
                      long long* fend, long long* ncnt, cudaStream_t st) {
    if (npairs <= 0) return;
    k_gen_slots<<<gen_grid(npairs, 256), 256, 0, st>>>(npairs, keys, keep, kpos, qend, nbr, fcell, fbeg, fend, ncnt);
}

void launch_gen_inc_emit(int n, unsigned V, const long long* off, const int* sig, unsigned long long* keys,
                         long long* cnt, cudaStream_t st) {
    if (!V) return;
    k_gen_inc_emit<<<gen_grid(V, 256), 256, 0, st>>>(n, V, off, sig, keys, cnt);
}

void launch_verify(const DevMesh& M, const double* x, unsigned V, const long long* off, const int* sig,
                   const double* oc, unsigned long long* cnt, unsigned long long* maxdev, cudaStream_t st) {
    if (!V) return;
    HV_DISPATCH(M.d, (k_verify<DD><<<gen_grid(V, 128), 128, 0, st>>>(M, x, V, off, sig, oc, cnt, maxdev)));
}

void launch_gen_polygon(const GenPoly& P, double* area, double* vol, int nsm, cudaStream_t st) {
    if (P.nslots > 0) {
        HV_DISPATCH(P.d, (k_gen_facets<DD><<<gen_grid(P.nslots, 64, (unsigned)nsm * 32), 64, 0, st>>>(P, area)));
        k_gen_copy<<<gen_grid(P.nslots, 256), 256, 0, st>>>(P, area);
    }
    if (P.n > 0) HV_DISPATCH(P.d, (k_gen_volumes<DD><<<gen_grid(P.n, 256), 256, 0, st>>>(P, area, vol)));
}

}  // namespace hv
