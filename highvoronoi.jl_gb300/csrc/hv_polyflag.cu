// hv_polyflag.cu -- VI_POLYGON areas from the vertices alone.
//
// The reference's flag decomposition (src/polyintegrator.jl:174-468) sums over
// the flags F = G_{d-1} > G_{d-2} > ... > G_0 (a vertex) of every facet F of
// cell i.  Its recursion
//     vol_m(G) = (1/m) sum over the facets G' of G of h(p_G, G') vol_{m-1}(G')
// holds for ANY reference point p_G of the affine hull of G when h is the
// signed distance (positive towards G's inside).  Take for the face G_S shared
// by the generators S the point of aff(G_S) nearest to S's points: the
// circumcentre p_S of S in its own affine hull (with boundary planes: the
// projection of a point of S onto {equidistant to S's points, on S's planes}).
// Then p_S depends on S only, and a flag of facet (i, j) that ends at vertex v
// is an ordering of the other d-1 generators of v:
//     A_ij = 1/(d-1)! sum_{v on F_ij} sum_{orderings} prod_m h(p_{S_m}, S_{m+1}),
//     h(p_S, S + l) = sign * |p_S - p_{S+l}|   (p_{S+l} is p_S projected onto
//                                               the face of S + l within aff(G_S)),
// with the sign of l's bisector (or plane) at p_S.  Summed over orderings this
// is a dynamic program over the subsets of v's generators: every vertex gives
// its share of every facet through it from its own d+1 generators -- no face
// lattice, no sorting, FP64 work proportional to the vertices.
//
// Two kernels:
//   k_vertex_flags  one warp per vertex: p_S of every generator subset, the
//                   heights of every (S, S + l) step (shared memory), then one
//                   lane per generator pair runs the subset DP; writes the
//                   share of each facet and the sum of the shares' absolute
//                   flag terms;
//   k_cell_flags    one warp per cell: walks the cell's vertices in ascending
//                   order (a fixed summation order, bitwise reproducible) and
//                   adds the shares of the facets it computes (those whose
//                   other generator is higher or a plane).
// A facet whose signed terms cancel (sum of |terms| > FLAG_COND x area, or an
// area that is not positive) is left to the exact face-lattice kernels
// (hv_poly.cu tier B), as is every facet of a cell with more neighbours than
// the warp's slots.
#include "hv_integrate.h"
#include "hv_internal.cuh"

namespace hv {

namespace {

constexpr int VF_WPB = 2;          // warps per block of k_vertex_flags (shared memory per warp up to 13.5 KB)
constexpr int CF_WPB = 4;          // warps per block of k_cell_flags
constexpr int CF_SLOTS = 512;      // neighbour slots per cell held in shared memory
constexpr double FLAG_COND = 1e3;  // tolerated cancellation of the signed flag terms

template <int D>
struct VF {
    static constexpr int NG = D + 1;                // generators of a vertex
    static constexpr int NS = 1 << NG;              // subsets
    static constexpr int NP = NG * (NG - 1) / 2;    // generator pairs
    static constexpr int NR = 1 << (NG - 2);        // subsets of the rest of a pair
};

// Position of pair (a, b), a < b < NG, in the row-major enumeration of pairs.
template <int NG>
__host__ __device__ __forceinline__ int pair_index(int a, int b) {
    return a * (2 * NG - a - 1) / 2 + (b - a - 1);
}

template <int D>
__global__ void __launch_bounds__(VF_WPB * 32) k_vertex_flags(FlagRun F) {
    constexpr int NG = VF<D>::NG, NS = VF<D>::NS, NP = VF<D>::NP, NR = VF<D>::NR;
    __shared__ double sp[VF_WPB][NS][D];   // p_S - c (c = the vertex)
    __shared__ double sh[VF_WPB][NS][NG];  // h(p_S, S + l)
    __shared__ double sy[VF_WPB][NG][D];   // points: x_g - c; planes: unit normal
    __shared__ double so[VF_WPB][NG];      // planes: off - n.c (about 0); points: |x_g - c|^2
    __shared__ int spl[VF_WPB][NG];        // 1: plane
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double fact = 1.0;
    for (int q = 2; q < D; ++q) fact *= q;
    for (unsigned v = blockIdx.x * VF_WPB + w; v < F.V; v += gridDim.x * VF_WPB) {
        if (lane < NG) {
            const int g = F.osig[(size_t)v * NG + lane];
            double c[D];
#pragma unroll
            for (int k = 0; k < D; ++k) c[k] = F.oc[(size_t)v * D + k];
            if (g < F.n) {
                double s = 0.0;
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    const double y = F.pts[(size_t)g * D + k] - c[k];
                    sy[w][lane][k] = y;
                    s = fma(y, y, s);
                }
                so[w][lane] = s;
                spl[w][lane] = 0;
            } else {
                const DevPlane& P = F.planes[g - F.n];
#pragma unroll
                for (int k = 0; k < D; ++k) sy[w][lane][k] = P.n[k];
                so[w][lane] = plane_height<D>(P, c);
                spl[w][lane] = 1;
            }
        }
        __syncwarp();
        // p_S for every subset with a point: the projection of its first point
        // y_a onto {p : (y_b - y_a).p = (|y_b|^2 - |y_a|^2)/2, n_q.p = off_q - n_q.c}
        for (int S = lane; S < NS; S += 32) {
            int a = -1;
            for (int g = 0; g < NG; ++g)
                if (((S >> g) & 1) && !spl[w][g]) { a = g; break; }
            if (a < 0 || __popc(S) < 2) continue;
            double A[D][D], r[D];
            int k = 0;
            for (int g = 0; g < NG; ++g) {
                if (!((S >> g) & 1) || g == a) continue;
                if (spl[w][g]) {
                    double ny = 0.0;
#pragma unroll
                    for (int q = 0; q < D; ++q) { A[k][q] = sy[w][g][q]; ny = fma(sy[w][g][q], sy[w][a][q], ny); }
                    r[k] = so[w][g] - ny;
                } else {
                    double dy = 0.0;
#pragma unroll
                    for (int q = 0; q < D; ++q) { A[k][q] = sy[w][g][q] - sy[w][a][q]; dy = fma(A[k][q], sy[w][a][q], dy); }
                    r[k] = 0.5 * (so[w][g] - so[w][a]) - dy;
                }
                ++k;
            }
            double p[D];
            if (k == D) {
#pragma unroll
                for (int q = 0; q < D; ++q) p[q] = 0.0;  // all generators: the vertex itself
            } else {
                // Gram system (A A^T) z = r, Cholesky; p = y_a + A^T z
                double L[D][D];
                bool ok = true;
                for (int x = 0; x < k && ok; ++x)
                    for (int y = 0; y <= x; ++y) {
                        double s = 0.0;
#pragma unroll
                        for (int q = 0; q < D; ++q) s = fma(A[x][q], A[y][q], s);
                        for (int t = 0; t < y; ++t) s -= L[x][t] * L[y][t];
                        if (x == y) {
                            if (!(s > 0)) { ok = false; break; }
                            L[x][x] = sqrt(s);
                        } else {
                            L[x][y] = s / L[y][y];
                        }
                    }
                double z[D];
                for (int x = 0; x < k; ++x) {
                    double s = r[x];
                    for (int t = 0; t < x; ++t) s -= L[x][t] * z[t];
                    z[x] = ok ? s / L[x][x] : 0.0;
                }
                for (int x = k - 1; x >= 0; --x) {
                    double s = z[x];
                    for (int t = x + 1; t < k; ++t) s -= L[t][x] * z[t];
                    z[x] = ok ? s / L[x][x] : 0.0;
                }
#pragma unroll
                for (int q = 0; q < D; ++q) {
                    double s = sy[w][a][q];
                    for (int x = 0; x < k; ++x) s = fma(A[x][q], z[x], s);
                    p[q] = s;
                }
                if (!ok) atomicOr(F.status, 2u);
            }
#pragma unroll
            for (int q = 0; q < D; ++q) sp[w][S][q] = p[q];
        }
        __syncwarp();
        // heights h(p_S, S + l): signed by l's side at p_S (inside: nearer to S's
        // points than to l, or below plane l)
        for (int e = lane; e < NS * NG; e += 32) {
            const int S = e / NG, l = e % NG;
            if (((S >> l) & 1) || __popc(S) < 2) continue;
            int a = -1;
            for (int g = 0; g < NG; ++g)
                if (((S >> g) & 1) && !spl[w][g]) { a = g; break; }
            if (a < 0) continue;
            const int T = S | (1 << l);
            double dist = 0.0, side = 0.0;
#pragma unroll
            for (int q = 0; q < D; ++q) {
                const double dq = sp[w][S][q] - sp[w][T][q];
                dist = fma(dq, dq, dist);
            }
            if (spl[w][l]) {
                double np = 0.0;
#pragma unroll
                for (int q = 0; q < D; ++q) np = fma(sy[w][l][q], sp[w][S][q], np);
                side = so[w][l] - np;
            } else {
                double dl = 0.0, da = 0.0;
#pragma unroll
                for (int q = 0; q < D; ++q) {
                    const double el = sp[w][S][q] - sy[w][l][q], ea = sp[w][S][q] - sy[w][a][q];
                    dl = fma(el, el, dl);
                    da = fma(ea, ea, da);
                }
                side = dl - da;
            }
            const double h = sqrt(dist);
            sh[w][S][l] = side >= 0.0 ? h : -h;
        }
        __syncwarp();
        // one lane per pair (i, j) with a point: the subset DP over the other d-1
        for (int pidx = lane; pidx < NP; pidx += 32) {
            int a = 0, b = 1;
            {
                int t = pidx;
                while (t >= NG - 1 - a) { t -= NG - 1 - a; ++a; }
                b = a + 1 + t;
            }
            double share = 0.0, sabs = 0.0;
            if (!(spl[w][a] && spl[w][b])) {
                int rest[NG - 2];
                int nr = 0;
                for (int g = 0; g < NG; ++g)
                    if (g != a && g != b) rest[nr++] = g;
                double W[NR], Wa[NR];
                W[0] = 1.0;
                Wa[0] = 1.0;
                const int base = (1 << a) | (1 << b);
                for (int M = 1; M < NR; ++M) {
                    int S = base;
                    for (int x = 0; x < NG - 2; ++x)
                        if ((M >> x) & 1) S |= 1 << rest[x];
                    double s = 0.0, sa = 0.0;
                    for (int x = 0; x < NG - 2; ++x) {
                        if (!((M >> x) & 1)) continue;
                        const int Mp = M & ~(1 << x);
                        const double h = sh[w][S & ~(1 << rest[x])][rest[x]];
                        s = fma(W[Mp], h, s);
                        sa = fma(Wa[Mp], fabs(h), sa);
                    }
                    W[M] = s;
                    Wa[M] = sa;
                }
                share = W[NR - 1] / fact;
                sabs = Wa[NR - 1] / fact;
            }
            F.share[(size_t)v * NP + pidx] = share;
            F.sabs[(size_t)v * NP + pidx] = (float)sabs;
        }
        __syncwarp();
    }
}

template <int D>
__global__ void __launch_bounds__(CF_WPB * 32) k_cell_flags(FlagRun F) {
    constexpr int NG = VF<D>::NG, NP = VF<D>::NP;
    __shared__ double acc[CF_WPB][CF_SLOTS];
    __shared__ float aab[CF_WPB][CF_SLOTS];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = blockIdx.x * CF_WPB + w; i < F.n; i += gridDim.x * CF_WPB) {
        const long long r0 = F.nbr_off[i], r1 = F.nbr_off[i + 1];
        const int deg = (int)(r1 - r0);
        if (deg > CF_SLOTS) {  // too many slots: the exact kernels take the cell's facets
            for (int t = lane; t < deg; t += 32) {
                const int k = F.nbr[r0 + t];
                if (k < F.n && k < i) continue;
                const unsigned q = atomicAdd(F.nbig, 1u);
                F.big[q] = r0 + t;
                atomicMax(F.maxnv, (unsigned)(F.foff[r0 + t + 1] - F.foff[r0 + t]));
            }
            continue;
        }
        for (int t = lane; t < deg; t += 32) { acc[w][t] = 0.0; aab[w][t] = 0.0f; }
        __syncwarp();
        const long long v0 = F.inc_off[i], v1 = F.inc_off[i + 1];
        for (long long base = v0; base < v1; base += 32) {
            const long long e = base + lane;
            int sl[NG];
            double val[NG];
            float vab[NG];
#pragma unroll
            for (int q = 0; q < NG; ++q) { sl[q] = -1; val[q] = 0.0; vab[q] = 0.0f; }
            if (e < v1) {
                const int v = F.inc[e];
                int sig[NG];
                int pi = 0;
#pragma unroll
                for (int q = 0; q < NG; ++q) {
                    sig[q] = F.osig[(size_t)v * NG + q];
                    if (sig[q] == i) pi = q;
                }
#pragma unroll
                for (int q = 0; q < NG; ++q) {
                    const int k = sig[q];
                    if (q == pi || (k < F.n && k < i)) continue;
                    long long lo = r0, hi = r1 - 1;
                    while (lo < hi) {
                        const long long md = (lo + hi) >> 1;
                        if (F.nbr[md] < k) lo = md + 1; else hi = md;
                    }
                    if (F.nbr[lo] != k) continue;
                    const int pidx = q < pi ? pair_index<NG>(q, pi) : pair_index<NG>(pi, q);
                    sl[q] = (int)(lo - r0);
                    val[q] = F.share[(size_t)v * NP + pidx];
                    vab[q] = F.sabs[(size_t)v * NP + pidx];
                }
            }
            // in vertex order, then generator order: lane (slot mod 32) adds
            const int nt = (int)min(32ll, v1 - base);
            for (int t = 0; t < nt; ++t)
#pragma unroll
                for (int q = 0; q < NG; ++q) {
                    const int s = __shfl_sync(0xFFFFFFFFu, sl[q], t);
                    const double x = __shfl_sync(0xFFFFFFFFu, val[q], t);
                    const float xa = __shfl_sync(0xFFFFFFFFu, vab[q], t);
                    if (s >= 0 && (s & 31) == lane) { acc[w][s] += x; aab[w][s] += xa; }
                }
        }
        __syncwarp();
        for (int t = lane; t < deg; t += 32) {
            const int k = F.nbr[r0 + t];
            if (k < F.n && k < i) continue;
            const double ar = acc[w][t];
            if (!(ar > 0.0) || (double)aab[w][t] > FLAG_COND * ar) {
                const unsigned q = atomicAdd(F.nbig, 1u);
                F.big[q] = r0 + t;
                atomicMax(F.maxnv, (unsigned)(F.foff[r0 + t + 1] - F.foff[r0 + t]));
                continue;
            }
            F.area[r0 + t] = ar;
            if (k < F.n) {
                long long lo = F.nbr_off[k], hi = F.nbr_off[k + 1] - 1;
                while (lo < hi) {
                    const long long md = (lo + hi) >> 1;
                    if (F.nbr[md] < i) lo = md + 1; else hi = md;
                }
                if (F.nbr[lo] == i) F.area[lo] = ar;
            }
        }
        __syncwarp();
    }
}

unsigned flag_grid(unsigned long long n, int per, int cap) {
    unsigned long long g = (n + per - 1) / per;
    if (g < 1) g = 1;
    return (unsigned)std::min<unsigned long long>(g, (unsigned long long)cap);
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

int flag_pairs(int d) { return (d + 1) * d / 2; }

void launch_vertex_flags(const FlagRun& F, int nsm, cudaStream_t st) {
    if (!F.V) return;
    HV_DISPATCH(F.d, (k_vertex_flags<DD><<<flag_grid(F.V, VF_WPB, nsm * 64), VF_WPB * 32, 0, st>>>(F)));
}

void launch_cell_flags(const FlagRun& F, int nsm, cudaStream_t st) {
    if (F.n <= 0) return;
    HV_DISPATCH(F.d, (k_cell_flags<DD><<<flag_grid(F.n, CF_WPB, nsm * 32), CF_WPB * 32, 0, st>>>(F)));
}

}  // namespace hv
