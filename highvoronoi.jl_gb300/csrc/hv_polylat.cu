// hv_polylat.cu -- VI_POLYGON over the face lattice of the whole mesh.
//
// A face of the tessellation is a set S of generators (|S| = c + 1 at
// codimension c, S[0] a point generator); its vertices are the mesh vertices
// whose signatures contain S.  The per-facet kernels (hv_poly.cu) build the face
// lattice of every facet on its own, so a face of codimension c is built and
// integrated once for each facet through it (a 2-face of a 6D mesh lies in 10
// facets).  Here every face is built and integrated once:
//   level 1 (facets): the pair (s_a, s_b) of a vertex's signature is the
//     neighbour slot of s_b in the row of s_a (the lower cell's slot; the
//     reference's interfaces are its neighbour pairs, src/polyintegrator.jl:174-316);
//   level c >= 2: every (c+1)-subset S of a vertex's signature gets the key
//     (face of S minus its largest generator, at level c-1) << gbits | max(S);
//     a stable radix sort groups the entries of a face, so a face's index is the
//     rank of its key; its reference vertex p_G is its first entry's vertex
//     (entries are numbered subset rank * V + vertex, so that the key pass
//     writes and reads whole lines);
//   pairs: each face H of level c+1 lists itself under every parent G = H - {l}
//     whose first vertex does not lie on H (sub-faces through the reference
//     point have zero height and are skipped, as in the pulling decomposition);
//   volumes, bottom-up: a 2-face from its edges (twice the triangle areas), a
//     face of dimension m > 2 as vol(G) = 1/m * sum over H of dist(p_G, aff H) *
//     vol(H), each parent's terms in the order of its children's indices (the
//     sums are bitwise reproducible); a facet's value is the interface area A_ik.
// Any vertex of G serves as p_G (every term is then a non-negative height
// times a volume); the per-facet kernels take each face's smallest vertex id,
// so the two paths sum the same decomposition with other reference points.
#include <algorithm>

#include "hv_integrate.h"
#include "hv_internal.cuh"
#include "hv_polygeo.cuh"

namespace hv {

__host__ __device__ constexpr int lat_binom(int n, int k) {
    if (k < 0 || k > n) return 0;
    int r = 1;
    for (int q = 0; q < k; ++q) r = r * (n - q) / (q + 1);
    return r;
}

int lat_subsets(int d, int c) { return lat_binom(d + 1, c + 1); }

// Ranks of the bit masks over a signature (at most 7 generators) among the
// masks of the same popcount in increasing numeric order (the combinatorial
// number system, the same rank for every signature length), and the inverse.
struct LatTabs {
    unsigned char rank[128];
    unsigned char mask[8][64];
};
__host__ __device__ constexpr LatTabs lat_tabs() {
    LatTabs t{};
    int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (unsigned m = 0; m < 128; ++m) {
        int k = 0;
        for (unsigned x = m; x; x &= x - 1) ++k;
        t.rank[m] = (unsigned char)cnt[k];
        t.mask[k][cnt[k]] = (unsigned char)m;
        ++cnt[k];
    }
    return t;
}
__device__ const LatTabs g_lat = lat_tabs();

__device__ __forceinline__ int lat_rank(unsigned m) { return __ldg(&g_lat.rank[m]); }
__device__ __forceinline__ unsigned lat_unrank(int r, int k) { return __ldg(&g_lat.mask[k][r]); }

__device__ __forceinline__ long long lat_find(const long long* off, const int* nbr, int row, int key) {
    long long lo = off[row], hi = off[row + 1];
    const long long end = hi;
    while (lo < hi) {
        const long long md = (lo + hi) >> 1;
        if (nbr[md] < key) lo = md + 1; else hi = md;
    }
    return lo < end && nbr[lo] == key ? lo : -1;
}

static int lat_grid(long long n, int bs) {
    const long long g = (n + bs - 1) / bs;
    return (int)std::max(1ll, std::min(g, 1ll << 20));
}

// ---- level 1: facet slots of every vertex pair, and each facet's smallest
// vertex (its reference vertex)
template <int D>
__global__ void k_lat_facets(LatIn L, int* F1, unsigned* fref1) {
    constexpr int G = D + 1;
    for (unsigned v = blockIdx.x * blockDim.x + threadIdx.x; v < L.V; v += gridDim.x * blockDim.x) {
        int s[G];
#pragma unroll
        for (int q = 0; q < G; ++q) s[q] = L.osig[(size_t)v * G + q];
        int r = 0;  // masks (1 << a) | (1 << b), a < b, in increasing order
#pragma unroll
        for (int b = 1; b < G; ++b)
#pragma unroll
            for (int a = 0; a < b; ++a, ++r) {
                long long t = -1;
                if (s[a] < L.n) {
                    t = lat_find(L.nbr_off, L.nbr, s[a], s[b]);
                    if (t < 0) atomicOr(L.status, 8u);
                    else atomicMin(fref1 + t, v);
                }
                F1[(size_t)r * L.V + v] = (int)t;
            }
    }
}

__global__ void k_lat_slot_cell(int n, const long long* nbr_off, int* slot_cell) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (long long t = nbr_off[i]; t < nbr_off[i + 1]; ++t) slot_cell[t] = i;
}

// ---- level c >= 2: one key per (vertex, (c+1)-subset); subsets whose smallest
// generator is a plane get the sentinel (they bound no cell's facet)
template <int D>
__global__ void k_lat_entries(LatIn L, int c, int gbits, const int* Fp, unsigned long long* keys, int* vals, int* Fc,
                              unsigned long long* nvalid) {
    constexpr int G = D + 1;
    unsigned long long cnt = 0;
    for (unsigned v = blockIdx.x * blockDim.x + threadIdx.x; v < L.V; v += gridDim.x * blockDim.x) {
        int s[G];
#pragma unroll
        for (int q = 0; q < G; ++q) s[q] = L.osig[(size_t)v * G + q];
        int r = 0;
        for (unsigned m = 1; m < (1u << G); ++m) {
            if (__popc(m) != c + 1) continue;
            const size_t e = (size_t)(r++) * L.V + v;
            const int lo = __ffs(m) - 1, hi = 31 - __clz(m);
            unsigned long long key = ~0ull;
            if (s[lo] < L.n) {
                const int pf = Fp[(size_t)lat_rank(m ^ (1u << hi)) * L.V + v];
                if (pf >= 0) {
                    key = ((unsigned long long)pf << gbits) | (unsigned long long)(unsigned)s[hi];
                    ++cnt;
                } else {
                    atomicOr(L.status, 8u);
                }
            }
            keys[e] = key;
            vals[e] = (int)e;
            if (key == ~0ull && Fc) Fc[e] = -1;
        }
    }
    cnt = __reduce_add_sync(0xFFFFFFFFu, (unsigned)cnt);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(nvalid, cnt);
}

__global__ void k_lat_heads(long long nval, const unsigned long long* sk, long long* flags) {
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x <= nval;
         x += (long long)gridDim.x * blockDim.x)
        flags[x] = x < nval && (x == 0 || sk[x] != sk[x - 1]) ? 1 : 0;
}

// face index of every entry, and each face's reference vertex (its first
// entry's) with the face's generators as a mask over that vertex's signature
// and, if asked, the face's first position; an edge must have exactly two
// vertices
template <int D>
__global__ void k_lat_scatter(LatIn L, int c, long long nval, const long long* fidx, const int* sv, int* Fc,
                              unsigned* fref, unsigned char* fmask, unsigned* fref2, long long* hstart) {
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < nval;
         x += (long long)gridDim.x * blockDim.x) {
        const long long f = fidx[x + 1] - 1;
        const int e = sv[x];
        if (Fc) Fc[e] = (int)f;  // (null for a table that no later pass reads)
        if (fidx[x] == fidx[x + 1]) continue;
        const unsigned v = (unsigned)e % L.V;
        fref[f] = v;
        if (hstart) hstart[f] = x;
        fmask[f] = (unsigned char)lat_unrank((int)((unsigned)e / L.V), c + 1);
        if (fref2) {
            const bool two = x + 1 < nval && fidx[x + 2] == fidx[x + 1] && (x + 2 >= nval || fidx[x + 3] != fidx[x + 2]);
            if (two) {
                fref2[f] = (unsigned)sv[x + 1] % L.V;
            } else {
                fref2[f] = v;
                atomicOr(L.status, 8u);
            }
        }
    }
}

// ---- parent -> child lists between levels c and c+1 (count, then fill at
// off[G] + a per-parent cursor; k_lat_prep orders each list)
template <int D, bool FILL>
__global__ void k_lat_pairs(LatIn L, int c, long long nH, const unsigned* frefH, const unsigned char* fmaskH,
                            const int* Fc, const unsigned* frefG, unsigned long long* cnt, const long long* off,
                            int* child, int* lgen, int* par) {
    constexpr int G = D + 1;
    for (long long h = blockIdx.x * (long long)blockDim.x + threadIdx.x; h < nH;
         h += (long long)gridDim.x * blockDim.x) {
        const unsigned p = frefH[h];
        const unsigned m = fmaskH[h];
        int s[G];
#pragma unroll
        for (int q = 0; q < G; ++q) s[q] = L.osig[(size_t)p * G + q];
#pragma unroll
        for (int q = 0; q < G; ++q) {
            if (!((m >> q) & 1u)) continue;
            const unsigned pm = m ^ (1u << q);
            if (s[__ffs(pm) - 1] >= L.n) continue;
            const int g = Fc[(size_t)lat_rank(pm) * L.V + p];
            if (g < 0) {
                atomicOr(L.status, 8u);
                continue;
            }
            const int l = s[q];
            const unsigned pg = frefG[g];
            bool through = false;
#pragma unroll
            for (int x = 0; x < G; ++x) through |= (L.osig[(size_t)pg * G + x] == l);
            if (through) continue;
            if (!FILL) {
                atomicAdd(cnt + g, 1ull);
            } else {
                const long long pos = off[g] + (long long)atomicAdd(cnt + g, 1ull);
                child[pos] = (int)h;
                lgen[pos] = l;
                par[pos] = g;
            }
        }
    }
}

// ---- volumes of the faces of level c from those of level c+1; level 1 writes
// the interface areas of both slots

// a parent's children in index order (its list is filled in arrival order)
__device__ __forceinline__ void lat_order(long long a, long long b, int* child, int* lgen) {
    for (long long x = a + 1; x < b; ++x) {
        const int h = child[x], l = lgen[x];
        long long y = x;
        for (; y > a && child[y - 1] > h; --y) {
            child[y] = child[y - 1];
            lgen[y] = lgen[y - 1];
        }
        child[y] = h;
        lgen[y] = l;
    }
}

__device__ __forceinline__ void lat_store(const LatIn& L, long long g, bool facets, const int* slot_cell, double vol,
                                          double* volG) {
    volG[g] = vol;
    if (facets) {  // the higher cell's slot of the same interface
        const int k = L.nbr[g];
        if (k < L.n) {
            const long long t = lat_find(L.nbr_off, L.nbr, k, slot_cell[g]);
            if (t >= 0) volG[t] = vol;
        }
    }
}

// Per parent: its children in index order and, above the 2-faces, its frame:
// the point generator x0 = S_G[0] and an orthonormal basis of the normals of
// S_G's other generators (c rows), frame[g * (c + 1) * D ...] = x0, Q.
template <int D>
__global__ void k_lat_prep(LatIn L, int c, long long nG, const long long* off, int* child, int* lgen,
                           const unsigned* frefG, const unsigned char* fmaskG, const int* slot_cell, double* frame) {
    constexpr int G = D + 1;
    constexpr int QR = D > 3 ? D - 3 : 1;
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nG;
         g += (long long)gridDim.x * blockDim.x) {
        const unsigned pg = frefG[g];
        if (pg == 0xFFFFFFFFu) continue;  // a slot of the higher cell
        if (off) lat_order(off[g], off[g + 1], child, lgen);
        if (c >= D - 2) continue;
        int sg[G];
        int ns = 0;
        if (c == 1) {
            sg[0] = slot_cell[g];
            sg[1] = L.nbr[g];
            ns = 2;
        } else {
            const unsigned m = fmaskG[g];
#pragma unroll
            for (int q = 0; q < G; ++q)
                if ((m >> q) & 1u) sg[ns++] = L.osig[(size_t)pg * G + q];
        }
        double x0[D];
#pragma unroll
        for (int q = 0; q < D; ++q) x0[q] = L.pts[(size_t)sg[0] * D + q];
        double Q[QR][D];
        int qm = 0;
        for (int u = 1; u < ns && qm < QR; ++u) {
            double nv[D];
            gen_normal<D>(L.n, L.pts, L.planes, sg[u], x0, nv);
            qm = mgs_add<D>(Q, qm, nv);
        }
        double* fr = frame + (size_t)g * (c + 1) * D;
#pragma unroll
        for (int q = 0; q < D; ++q) fr[q] = x0[q];
        for (int r = 0; r < qm; ++r)
#pragma unroll
            for (int q = 0; q < D; ++q) fr[(size_t)(r + 1) * D + q] = Q[r][q];
    }
}

// One term per (parent, child) pair: 2-faces |(p - a) ^ (b - a)| over their
// edges, higher faces dist(p_G, aff H) * vol(H) in the parent's frame (the
// arithmetic of lat_height below, inlined: 48 instead of 56 registers in 6D).
template <int D>
__global__ void __launch_bounds__(256) k_lat_terms(LatIn L, int c, long long npairs, const int* par, const int* child,
                                                   const int* lgen, const unsigned* frefG, const double* frame,
                                                   const unsigned* frefH, const unsigned* fref2H, const double* volH,
                                                   double* term) {
    for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < npairs;
         x += (long long)gridDim.x * blockDim.x) {
        const int g = par[x], h = child[x];
        const unsigned pg = frefG[g];
        double p[D];
#pragma unroll
        for (int q = 0; q < D; ++q) p[q] = L.oc[(size_t)pg * D + q];
        if (c == D - 2) {
            double va[D], vb[D];
            const unsigned ua = frefH[h], ub = fref2H[h];
#pragma unroll
            for (int q = 0; q < D; ++q) { va[q] = L.oc[(size_t)ua * D + q]; vb[q] = L.oc[(size_t)ub * D + q]; }
            term[x] = tri_area2<D>(p, va, vb);
        } else {
            const double* fr = frame + (size_t)g * (c + 1) * D;
            const int l = lgen[x];
            const unsigned uh = frefH[h];
            double r[D], num = 0.0;
            if (l < L.n) {
#pragma unroll
                for (int q = 0; q < D; ++q) r[q] = L.pts[(size_t)l * D + q] - fr[q];
            } else {
                const DevPlane& B = L.planes[l - L.n];
#pragma unroll
                for (int q = 0; q < D; ++q) r[q] = B.n[q];
            }
#pragma unroll
            for (int q = 0; q < D; ++q) num = fma(r[q], L.oc[(size_t)uh * D + q] - p[q], num);
            for (int s = 1; s <= c; ++s) {  // the component of n_l orthogonal to the frame
                const double* qs = fr + (size_t)s * D;
                double dt = 0;
#pragma unroll
                for (int q = 0; q < D; ++q) dt = fma(qs[q], r[q], dt);
#pragma unroll
                for (int q = 0; q < D; ++q) r[q] = fma(-dt, qs[q], r[q]);
            }
            double nn = 0;
#pragma unroll
            for (int q = 0; q < D; ++q) nn = fma(r[q], r[q], nn);
            term[x] = fabs(num) * rsqrt(nn) * volH[h];
        }
    }
}

// vol(G) = sum of its terms in child order / dim(G); level 1: both slots
template <int D>
__global__ void k_lat_sum(LatIn L, int c, long long nG, const long long* off, const double* term,
                          const unsigned* frefG, const int* slot_cell, double* volG) {
    for (long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x; g < nG;
         g += (long long)gridDim.x * blockDim.x) {
        if (frefG[g] == 0xFFFFFFFFu) continue;
        double sum = 0.0;
        for (long long x = off[g]; x < off[g + 1]; ++x) sum += term[x];
        lat_store(L, g, c == 1, slot_cell, sum / (double)(D - c), volG);
    }
}

// ---------------------------------------------------------------------------
// integrand quadrature (the reference's flag decomposition with face centroids)
// ---------------------------------------------------------------------------
// A flag F = L_1 > L_2 > ... > L_{D-2} > edge (r1, r2) of facet F of cell i has
// |det(c_F - x_i, c(L_2) - x_i, ..., r1 - x_i, r2 - x_i)| = h_F * prod_{j < D-2}
// dist(c(L_j), aff L_{j+1}) * |(c(L_{D-2}) - r1) ^ (r2 - r1)|, c(L) the mean of
// L's vertices, h_F the distance of x_i to F: the product of the heights of the
// successive centroids.  So for every face Q and every facet F containing it
// (a generator pair of S_Q) phi_Q[F] = the sum over the chains from F down to Q
// of the products of their heights, top-down over the face lattice; then each
// edge's sums per facet, and each (facet, vertex) weight.

// mean of each face's vertices: its entries from hstart[f] to the next face's
// start, in the sorted order
template <int D>
__global__ void k_lat_centroid(LatIn L, long long nf, long long nval, const long long* hstart, const int* sv,
                               double* cen) {
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nf;
         f += (long long)gridDim.x * blockDim.x) {
        const long long x0 = hstart[f], x1 = f + 1 < nf ? hstart[f + 1] : nval;
        double sum[D];
#pragma unroll
        for (int q = 0; q < D; ++q) sum[q] = 0.0;
        for (long long x = x0; x < x1; ++x) {
            const unsigned v = (unsigned)sv[x] % L.V;
#pragma unroll
            for (int q = 0; q < D; ++q) sum[q] += L.oc[(size_t)v * D + q];
        }
        const double inv = 1.0 / (double)(x1 - x0);
#pragma unroll
        for (int q = 0; q < D; ++q) cen[(size_t)f * D + q] = sum[q] * inv;
    }
}

// rank of the pair of positions (a, b) among the pairs of a set once position
// j (j != a, b) is removed
__device__ __forceinline__ int lat_pair_rank(int a, int b, int j) {
    const int a2 = a - (j < a ? 1 : 0), b2 = b - (j < b ? 1 : 0);
    return lat_rank((1u << a2) | (1u << b2));
}

// dist(p, aff Q) inside aff P for Q = P + {l}: the frame of P (x0, rows), a
// vertex vq of Q
template <int D>
__device__ __forceinline__ double lat_height(const LatIn& L, const double* fr, int rows, int l, const double* vq,
                                             const double* p) {
    double r[D], num = 0.0;
    if (l < L.n) {
#pragma unroll
        for (int q = 0; q < D; ++q) r[q] = L.pts[(size_t)l * D + q] - fr[q];
    } else {
        const DevPlane& B = L.planes[l - L.n];
#pragma unroll
        for (int q = 0; q < D; ++q) r[q] = B.n[q];
    }
#pragma unroll
    for (int q = 0; q < D; ++q) num = fma(r[q], vq[q] - p[q], num);
    for (int s = 1; s <= rows; ++s) {
        const double* qs = fr + (size_t)s * D;
        double dt = 0;
#pragma unroll
        for (int q = 0; q < D; ++q) dt = fma(qs[q], r[q], dt);
#pragma unroll
        for (int q = 0; q < D; ++q) r[q] = fma(-dt, qs[q], r[q]);
    }
    double nn = 0;
#pragma unroll
    for (int q = 0; q < D; ++q) nn = fma(r[q], r[q], nn);
    return fabs(num) * rsqrt(nn);
}

// phi of the faces Q of level c (2 <= c <= D-2), C(c+1, 2) values per face (the
// pairs of S_Q's positions in mask-rank order; 0 for a pair of two planes), from
// the parents of level c-1: their frames, centroids and phi (1 for a facet)
template <int D>
__global__ void k_lat_phi(LatIn L, int c, long long nQ, const unsigned* frefQ, const unsigned char* fmaskQ,
                          const int* Fp, const double* frameP, const double* cenP, const double* phiP, double* phiQ) {
    constexpr int G = D + 1;
    const int nq = lat_binom(c + 1, 2), npp = lat_binom(c, 2);
    for (long long h = blockIdx.x * (long long)blockDim.x + threadIdx.x; h < nQ;
         h += (long long)gridDim.x * blockDim.x) {
        const unsigned p = frefQ[h];
        const unsigned m = fmaskQ[h];
        int pos[G], gen[G];
        int k = 0;
#pragma unroll
        for (int q = 0; q < G; ++q)
            if ((m >> q) & 1u) { pos[k] = q; gen[k] = L.osig[(size_t)p * G + q]; ++k; }
        double vq[D];
#pragma unroll
        for (int q = 0; q < D; ++q) vq[q] = L.oc[(size_t)p * D + q];
        for (int r = 0; r < nq; ++r) phiQ[(size_t)h * nq + r] = 0.0;
        for (int j = 0; j <= c; ++j) {  // the parent P = Q - gen[j]
            const unsigned pm = m ^ (1u << pos[j]);
            if (L.osig[(size_t)p * G + __ffs(pm) - 1] >= L.n) continue;
            const int g = Fp[(size_t)lat_rank(pm) * L.V + p];
            if (g < 0) {
                atomicOr(L.status, 8u);
                continue;
            }
            const double* fr = frameP + (size_t)g * c * D;  // x0 and c - 1 rows
            const double ht = lat_height<D>(L, fr, c - 1, gen[j], vq, cenP + (size_t)g * D);
            for (int b = 1; b <= c; ++b)
                for (int a = 0; a < b; ++a) {
                    if (a == j || b == j || gen[a] >= L.n) continue;
                    const double ph = c == 2 ? 1.0 : phiP[(size_t)g * npp + lat_pair_rank(a, b, j)];
                    phiQ[(size_t)h * nq + lat_rank((1u << a) | (1u << b))] += ph * ht;
                }
        }
    }
}

// per edge (level D-1) and pair of its D generators: the sum over its 2-faces L
// of phi_L[pair] * |(c(L) - r1) ^ (r2 - r1)| (D = 3: the 2-faces are the facets,
// phi = 1)
template <int D>
__global__ void k_lat_edgew(LatIn L, long long nE, const unsigned* frefE, const unsigned* fref2E,
                            const unsigned char* fmaskE, const int* Fp, const double* cenP, const double* phiP,
                            double* pe) {
    constexpr int G = D + 1;
    constexpr int NE = lat_binom(D, 2), NP = lat_binom(D - 1, 2);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nE;
         e += (long long)gridDim.x * blockDim.x) {
        const unsigned p = frefE[e], p2 = fref2E[e];
        const unsigned m = fmaskE[e];
        int pos[D], gen[D];
        int k = 0;
#pragma unroll
        for (int q = 0; q < G; ++q)
            if (((m >> q) & 1u) && k < D) { pos[k] = q; gen[k] = L.osig[(size_t)p * G + q]; ++k; }
        double va[D], vb[D], acc[NE];
#pragma unroll
        for (int q = 0; q < D; ++q) { va[q] = L.oc[(size_t)p * D + q]; vb[q] = L.oc[(size_t)p2 * D + q]; }
#pragma unroll
        for (int r = 0; r < NE; ++r) acc[r] = 0.0;
#pragma unroll
        for (int j = 0; j < D; ++j) {  // the 2-face L = e - gen[j]
            const unsigned pm = m ^ (1u << pos[j]);
            if (L.osig[(size_t)p * G + __ffs(pm) - 1] >= L.n) continue;
            const int g = Fp[(size_t)lat_rank(pm) * L.V + p];
            if (g < 0) {
                atomicOr(L.status, 8u);
                continue;
            }
            const double t = tri_area2<D>(cenP + (size_t)g * D, va, vb);
#pragma unroll
            for (int b = 1; b < D; ++b)
#pragma unroll
                for (int a = 0; a < b; ++a) {
                    if (a == j || b == j || gen[a] >= L.n) continue;
                    const double ph = D == 3 ? 1.0 : phiP[(size_t)g * NP + lat_pair_rank(a, b, j)];
                    acc[lat_binom(b, 2) + a] += ph * t;
                }
        }
#pragma unroll
        for (int r = 0; r < NE; ++r) pe[(size_t)e * NE + r] = acc[r];
    }
}

// the weight of the a-th vertex v of facet t (i, k): h_F / 2 * the sum over the
// edges of v inside F (v's generators without one other than i and k) of the
// edge's sum for (i, k); the facet's flag sum = the sum of its weights
template <int D>
__global__ void k_lat_qweights(LatIn L, long long ns, const long long* foff, const unsigned* qv, const int* slot_cell,
                               const int* Fe, const double* pe, double* qw, double* qa) {
    constexpr int G = D + 1;
    constexpr int NE = lat_binom(D, 2);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < ns;
         t += (long long)gridDim.x * blockDim.x) {
        const long long f0 = foff[t], f1 = foff[t + 1];
        if (f0 == f1) continue;  // a slot of the higher cell
        const int i = slot_cell[t], k = L.nbr[t];
        double h;
        if (k >= L.n) {
            double xi[D];
#pragma unroll
            for (int q = 0; q < D; ++q) xi[q] = L.pts[(size_t)i * D + q];
            h = plane_height<D>(L.planes[k - L.n], xi);
        } else {
            double s2 = 0;
#pragma unroll
            for (int q = 0; q < D; ++q) {
                const double e = L.pts[(size_t)k * D + q] - L.pts[(size_t)i * D + q];
                s2 = fma(e, e, s2);
            }
            h = 0.5 * sqrt(s2);
        }
        double total = 0.0;
        for (long long x = f0; x < f1; ++x) {
            const unsigned v = qv[x];
            int s[G], pi = -1, pk = -1;
#pragma unroll
            for (int q = 0; q < G; ++q) {
                s[q] = L.osig[(size_t)v * G + q];
                if (s[q] == i) pi = q;
                if (s[q] == k) pk = q;
            }
            double w = 0.0;
            if (pi < 0 || pk < 0) {
                atomicOr(L.status, 8u);
            } else {
#pragma unroll
                for (int j = 0; j < G; ++j) {
                    if (j == pi || j == pk) continue;
                    const unsigned em = ((1u << G) - 1u) ^ (1u << j);
                    const int e = Fe[(size_t)lat_rank(em) * L.V + v];
                    if (e < 0) {
                        atomicOr(L.status, 8u);
                        continue;
                    }
                    w += pe[(size_t)e * NE + lat_pair_rank(pi, pk, j)];
                }
            }
            w *= 0.5 * h;
            qw[x] = w;
            total += w;
        }
        qa[t] = total;
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
#define LAT_DISPATCH(d, CALL)                          \
    switch (d) {                                       \
        case 3: { constexpr int DD = 3; CALL; } break; \
        case 4: { constexpr int DD = 4; CALL; } break; \
        case 5: { constexpr int DD = 5; CALL; } break; \
        case 6: { constexpr int DD = 6; CALL; } break; \
        default: break;                                \
    }

void launch_lat_facets(const LatIn& L, int* F1, unsigned* fref1, int* slot_cell, cudaStream_t st) {
    LAT_DISPATCH(L.d, (k_lat_facets<DD><<<lat_grid(L.V, 256), 256, 0, st>>>(L, F1, fref1)));
    k_lat_slot_cell<<<lat_grid(L.n, 256), 256, 0, st>>>(L.n, L.nbr_off, slot_cell);
}

void launch_lat_entries(const LatIn& L, int c, int gbits, const int* Fp, unsigned long long* keys, int* vals, int* Fc,
                        unsigned long long* nvalid, cudaStream_t st) {
    LAT_DISPATCH(L.d, (k_lat_entries<DD><<<lat_grid(L.V, 256), 256, 0, st>>>(L, c, gbits, Fp, keys, vals, Fc, nvalid)));
}

void launch_lat_heads(long long nval, const unsigned long long* sk, long long* flags, cudaStream_t st) {
    k_lat_heads<<<lat_grid(nval + 1, 256), 256, 0, st>>>(nval, sk, flags);
}

void launch_lat_scatter(const LatIn& L, int c, long long nval, const long long* fidx, const int* sv, int* Fc,
                        unsigned* fref, unsigned char* fmask, unsigned* fref2, long long* hstart, cudaStream_t st) {
    LAT_DISPATCH(L.d, (k_lat_scatter<DD><<<lat_grid(nval, 256), 256, 0, st>>>(L, c, nval, fidx, sv, Fc, fref, fmask,
                                                                           fref2, hstart)));
}

void launch_lat_pairs(const LatIn& L, int c, long long nH, const unsigned* frefH, const unsigned char* fmaskH,
                      const int* Fc, const unsigned* frefG, unsigned long long* cnt, const long long* off, int* child,
                      int* lgen, int* par, bool fill, cudaStream_t st) {
    if (fill) {
        LAT_DISPATCH(L.d, (k_lat_pairs<DD, true><<<lat_grid(nH, 256), 256, 0, st>>>(L, c, nH, frefH, fmaskH, Fc, frefG,
                                                                                cnt, off, child, lgen, par)));
    } else {
        LAT_DISPATCH(L.d, (k_lat_pairs<DD, false><<<lat_grid(nH, 256), 256, 0, st>>>(L, c, nH, frefH, fmaskH, Fc,
                                                                                 frefG, cnt, off, child, lgen, par)));
    }
}

void launch_lat_prep(const LatIn& L, int c, long long nG, const long long* off, int* child, int* lgen,
                     const unsigned* frefG, const unsigned char* fmaskG, const int* slot_cell, double* frame,
                     cudaStream_t st) {
    LAT_DISPATCH(L.d, (k_lat_prep<DD><<<lat_grid(nG, 256), 256, 0, st>>>(L, c, nG, off, child, lgen, frefG, fmaskG,
                                                                        slot_cell, frame)));
}

void launch_lat_terms(const LatIn& L, int c, long long npairs, const int* par, const int* child, const int* lgen,
                      const unsigned* frefG, const double* frame, const unsigned* frefH, const unsigned* fref2H,
                      const double* volH, double* term, cudaStream_t st) {
    LAT_DISPATCH(L.d, (k_lat_terms<DD><<<lat_grid(npairs, 256), 256, 0, st>>>(L, c, npairs, par, child, lgen, frefG,
                                                                             frame, frefH, fref2H, volH, term)));
}

void launch_lat_sum(const LatIn& L, int c, long long nG, const long long* off, const double* term,
                    const unsigned* frefG, const int* slot_cell, double* volG, cudaStream_t st) {
    LAT_DISPATCH(L.d, (k_lat_sum<DD><<<lat_grid(nG, 256), 256, 0, st>>>(L, c, nG, off, term, frefG, slot_cell, volG)));
}

void launch_lat_centroid(const LatIn& L, long long nf, long long nval, const long long* hstart, const int* sv,
                         double* cen, cudaStream_t st) {
    LAT_DISPATCH(L.d, (k_lat_centroid<DD><<<lat_grid(nf, 256), 256, 0, st>>>(L, nf, nval, hstart, sv, cen)));
}

void launch_lat_phi(const LatIn& L, int c, long long nQ, const unsigned* frefQ, const unsigned char* fmaskQ,
                    const int* Fp, const double* frameP, const double* cenP, const double* phiP, double* phiQ,
                    cudaStream_t st) {
    LAT_DISPATCH(L.d, (k_lat_phi<DD><<<lat_grid(nQ, 128), 128, 0, st>>>(L, c, nQ, frefQ, fmaskQ, Fp, frameP, cenP,
                                                                       phiP, phiQ)));
}

void launch_lat_edgew(const LatIn& L, long long nE, const unsigned* frefE, const unsigned* fref2E,
                      const unsigned char* fmaskE, const int* Fp, const double* cenP, const double* phiP, double* pe,
                      cudaStream_t st) {
    LAT_DISPATCH(L.d, (k_lat_edgew<DD><<<lat_grid(nE, 128), 128, 0, st>>>(L, nE, frefE, fref2E, fmaskE, Fp, cenP,
                                                                         phiP, pe)));
}

void launch_lat_qweights(const LatIn& L, long long ns, const long long* foff, const unsigned* qv,
                         const int* slot_cell, const int* Fe, const double* pe, double* qw, double* qa,
                         cudaStream_t st) {
    LAT_DISPATCH(L.d, (k_lat_qweights<DD><<<lat_grid(ns, 128), 128, 0, st>>>(L, ns, foff, qv, slot_cell, Fe, pe, qw,
                                                                            qa)));
}

long long lat_term_flops(int d, int c) {
    if (c == d - 2) return 2ll * d + 5ll * d * (d - 1) / 2 + 1;  // |(p - a) ^ (b - a)|
    return 6ll * d + 4ll * c * d + 3;                           // dist(p, aff H) * vol(H)
}

}  // namespace hv
