// hv_quad.cu -- integrals of a user function with VI_POLYGON's quadrature.
//
// The reference integrates an integrand f over every interface and cell along
// the flag decomposition of the polygon integrator (Polygon_Integrator with
// _function, src/polyintegrator.jl:80-123,174-330): the cone over facet F of
// cell i is cut into the simplices (x_i, c_F, c(G_2), ..., c(G_{d-2}), r1, r2)
// of the chains F > G_2 > ... > edge (r1, r2), c(G) the mean of G's vertices;
// each simplex weighs the edge value (f(r1) + f(r2)) / 2 with |det|, and
//   I_F    = (d-1)/d * sum |det| (f(r1)+f(r2))/2 / ((d-1)! h) + A_F f(c_F) / d
//   bulk_i = sum over the facets of cell i: V_iF f(x_i)/(d+1) + I_F h/(d+1)
// (src/polyintegrator.jl:139-160, 170-180), h the distance of x_i to the facet,
// A_F = sum |det| / ((d-1)! h), V_iF = A_F h / d.
//
// No callback: the library cannot call a Julia or Python function, so the
// work splits in two.  hv_mesh_facet_centers computes, once per mesh, the flag
// sums of every facet as weights on its vertices (W_v = sum over the flags
// whose edge ends at v of |det| / 2) and the facet centres; the caller
// evaluates f at the nodes (vertices, facet centres, generators); then
// hv_integrate_polygon_functions forms I_F and bulk_i from those values on
// the GPU.
//
// Weights: one thread per facet of its lower cell walks the chains with the
// facet's vertex lists as bit masks (one mask per depth) and solves one d x d
// determinant in FP64 per flag; facets of up to QUAD_MAXV vertices.  From 4D on
// the weights come from the mesh-wide face lattice instead (hv_polylat.cu: the
// same |det| as products of centroid heights, summed once per face); this file
// then gives the facets' sorted vertex lists and centres.
#include <algorithm>

#include "hv_integrate.h"
#include "hv_internal.cuh"

namespace hv {

constexpr int QUAD_MAXV = 1024;
constexpr int QUAD_WORDS = QUAD_MAXV / 32;

template <int D>
__device__ __forceinline__ bool has_item(const int* osig, unsigned v, int it) {
    bool h = false;
#pragma unroll
    for (int q = 0; q <= D; ++q) h |= osig[(size_t)v * (D + 1) + q] == it;
    return h;
}

template <int D, bool WEIGHTS>
__global__ void __launch_bounds__(64) k_poly_quad(QuadRun Q) {
    constexpr int DEP = D > 2 ? D - 1 : 2;  // depths 1 .. D-1
    unsigned mask[DEP][QUAD_WORDS];
    double cen[DEP][D];
    int last[DEP], chosen[DEP];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < Q.nslots;
         t += (long long)gridDim.x * blockDim.x) {
        const long long f0 = Q.foff[t];
        const int nv = (int)(Q.foff[t + 1] - f0);
        if (nv == 0) continue;  // a slot of the higher cell: its lower cell computes the facet
        if (WEIGHTS && nv > QUAD_MAXV) { atomicOr(Q.status, 1u); continue; }
        unsigned* qv = Q.qv + f0;
        double* qw = Q.qw + f0;
        // the facet's vertices in id order (the incidence fill left them unordered)
        for (int a = 0; a < nv; ++a) qv[a] = Q.fvert[f0 + a];
        for (int a = 1; a < nv; ++a) {
            const unsigned x = qv[a];
            int b = a - 1;
            while (b >= 0 && qv[b] > x) { qv[b + 1] = qv[b]; --b; }
            qv[b + 1] = x;
        }
        if (!WEIGHTS) {  // the vertex lists and the facet centres only
            double c[D];
#pragma unroll
            for (int q = 0; q < D; ++q) c[q] = 0.0;
            for (int a = 0; a < nv; ++a)
#pragma unroll
                for (int q = 0; q < D; ++q) c[q] += Q.oc[(size_t)qv[a] * D + q];
#pragma unroll
            for (int q = 0; q < D; ++q) Q.qc[(size_t)t * D + q] = c[q] / (double)nv;
            continue;
        }
        for (int a = 0; a < nv; ++a) qw[a] = 0.0;
        const int i = Q.slot_cell[t], k = Q.nbr[t];
        double xi[D];
#pragma unroll
        for (int q = 0; q < D; ++q) xi[q] = Q.pts[(size_t)i * D + q];
        const int nw = (nv + 31) >> 5;
        for (int w = 0; w < QUAD_WORDS; ++w)
            mask[0][w] = w < nw ? (w == nw - 1 && (nv & 31) ? (1u << (nv & 31)) - 1u : 0xFFFFFFFFu) : 0u;
        double area = 0.0;
        int depth = 0;  // depth j holds the face cut by k and chosen[0 .. j-1]
        last[0] = -1;
        bool fresh = true;
        int bad = 0;
        for (;;) {
            if (depth == D - 2) {  // an edge: one flag simplex
                int e[2], ne = 0;
                for (int w = 0; w < nw; ++w)
                    for (unsigned b = mask[depth][w]; b; b &= b - 1) {
                        if (ne < 2) e[ne] = (w << 5) + __ffs(b) - 1;
                        ++ne;
                    }
                if (ne != 2) {
                    bad = 1;
                } else {
                    double A[D][D];
                    for (int c = 0; c < D - 2; ++c)
#pragma unroll
                        for (int q = 0; q < D; ++q) A[q][c] = cen[c][q] - xi[q];
#pragma unroll
                    for (int q = 0; q < D; ++q) {
                        A[q][D - 2] = Q.oc[(size_t)qv[e[0]] * D + q] - xi[q];
                        A[q][D - 1] = Q.oc[(size_t)qv[e[1]] * D + q] - xi[q];
                    }
                    int piv[D];
                    double det = 0.0;
                    if (lu_factor<D, double>(A, piv)) {
                        det = 1.0;
#pragma unroll
                        for (int r = 0; r < D; ++r) det *= A[r][r];
                    }
                    const double w = fabs(det);
                    qw[e[0]] += 0.5 * w;
                    qw[e[1]] += 0.5 * w;
                    area += w;
                }
                if (depth == 0) break;
                --depth;
                continue;
            }
            if (fresh) {  // centre of the face at this depth
                int cnt = 0;
                double s[D];
#pragma unroll
                for (int q = 0; q < D; ++q) s[q] = 0.0;
                for (int w = 0; w < nw; ++w)
                    for (unsigned b = mask[depth][w]; b; b &= b - 1) {
                        const unsigned v = qv[(w << 5) + __ffs(b) - 1];
#pragma unroll
                        for (int q = 0; q < D; ++q) s[q] += Q.oc[(size_t)v * D + q];
                        ++cnt;
                    }
#pragma unroll
                for (int q = 0; q < D; ++q) cen[depth][q] = s[q] / (double)cnt;
                if (depth == 0)
#pragma unroll
                    for (int q = 0; q < D; ++q) Q.qc[(size_t)t * D + q] = cen[0][q];
                fresh = false;
            }
            // the next item (ascending) of this face's vertices beyond i, k and the
            // items chosen above
            int nxt = 0x7FFFFFFF;
            for (int w = 0; w < nw; ++w)
                for (unsigned b = mask[depth][w]; b; b &= b - 1) {
                    const unsigned v = qv[(w << 5) + __ffs(b) - 1];
#pragma unroll
                    for (int q = 0; q <= D; ++q) {
                        const int it = Q.osig[(size_t)v * (D + 1) + q];
                        if (it <= last[depth] || it >= nxt || it == i || it == k) continue;
                        bool used = false;
                        for (int u = 0; u < depth; ++u) used |= chosen[u] == it;
                        if (!used) nxt = it;
                    }
                }
            if (nxt == 0x7FFFFFFF) {
                if (depth == 0) break;
                --depth;
                continue;
            }
            last[depth] = nxt;
            int cnt = 0;
            for (int w = 0; w < nw; ++w) {
                unsigned m = 0;
                for (unsigned b = mask[depth][w]; b; b &= b - 1) {
                    const int a = (w << 5) + __ffs(b) - 1;
                    if (has_item<D>(Q.osig, qv[a], nxt)) m |= 1u << (a & 31);
                }
                mask[depth + 1][w] = m;
                cnt += __popc(m);
            }
            if (cnt < 2) continue;
            chosen[depth] = nxt;
            ++depth;
            last[depth] = -1;
            fresh = true;
        }
        if (bad) atomicOr(Q.status, 8u);
        Q.qa[t] = area;
    }
}

// Interface integrals of the facets computed by their lower cells, then the
// copies for the higher cells, then the cell integrals.
template <int D>
__device__ __forceinline__ double facet_h(const QuadRun& Q, const double* xi, int k) {
    if (k >= Q.n) return plane_height<D>(Q.planes[k - Q.n], xi);
    double s = 0;
#pragma unroll
    for (int q = 0; q < D; ++q) { const double e = Q.pts[(size_t)k * D + q] - xi[q]; s = fma(e, e, s); }
    return 0.5 * sqrt(s);
}

template <int D>
__global__ void k_quad_iface(QuadRun Q, int p, const double* fv, const double* fc, double* iface) {
    double f1 = 1.0;  // (d-1)!
    for (int q = 2; q < D; ++q) f1 *= q;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < Q.nslots;
         t += (long long)gridDim.x * blockDim.x) {
        const long long f0 = Q.foff[t], f1e = Q.foff[t + 1];
        if (f1e == f0) continue;
        const int i = Q.slot_cell[t], k = Q.nbr[t];
        double xi[D];
#pragma unroll
        for (int q = 0; q < D; ++q) xi[q] = Q.pts[(size_t)i * D + q];
        const double h = facet_h<D>(Q, xi, k);
        const double scale = 1.0 / (f1 * h);
        Q.af[t] = Q.qa[t] * scale;
        for (int c = 0; c < p; ++c) {
            double s = 0.0;
            for (long long x = f0; x < f1e; ++x) s += Q.qw[x] * fv[(size_t)Q.qv[x] * p + c];
            iface[t * p + c] = (D - 1.0) / D * s * scale + Q.qa[t] * scale * fc[t * p + c] / D;
        }
    }
}

template <int D>
__global__ void k_quad_copy(QuadRun Q, int p, double* iface) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Q.n; i += gridDim.x * blockDim.x)
        for (long long t = Q.nbr_off[i]; t < Q.nbr_off[i + 1]; ++t) {
            const int k = Q.nbr[t];
            if (k >= Q.n || k > i) continue;
            long long lo = Q.nbr_off[k], hi = Q.nbr_off[k + 1] - 1;
            while (lo < hi) { const long long md = (lo + hi) >> 1; if (Q.nbr[md] < i) lo = md + 1; else hi = md; }
            for (int c = 0; c < p; ++c) iface[t * p + c] = iface[lo * p + c];
        }
}

template <int D>
__global__ void k_quad_bulk(QuadRun Q, int p, const double* fx, const double* iface, double* bulk) {
    double f1 = 1.0;
    for (int q = 2; q < D; ++q) f1 *= q;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Q.n; i += gridDim.x * blockDim.x) {
        double xi[D];
#pragma unroll
        for (int q = 0; q < D; ++q) xi[q] = Q.pts[(size_t)i * D + q];
        for (int c = 0; c < p; ++c) {
            double s = 0.0;
            for (long long t = Q.nbr_off[i]; t < Q.nbr_off[i + 1]; ++t) {
                const double h = facet_h<D>(Q, xi, Q.nbr[t]);
                const double vik = Q.af[t] * h / D;
                s += fx[(size_t)i * p + c] * vik / (D + 1.0) + iface[t * p + c] * h / (D + 1.0);
            }
            bulk[(size_t)i * p + c] = s;
        }
    }
}

#define HV_DISPATCH(d, CALL)                           \
    switch (d) {                                       \
        case 2: { constexpr int DD = 2; CALL; } break; \
        case 3: { constexpr int DD = 3; CALL; } break; \
        case 4: { constexpr int DD = 4; CALL; } break; \
        case 5: { constexpr int DD = 5; CALL; } break; \
        case 6: { constexpr int DD = 6; CALL; } break; \
        default: break;                                \
    }

static unsigned grid_of(long long n, int bs, int cap) {
    long long g = (n + bs - 1) / bs;
    return (unsigned)std::max(1ll, std::min(g, (long long)cap));
}

void launch_poly_quad(const QuadRun& Q, bool weights, int nsm, cudaStream_t st) {
    if (weights) {
        HV_DISPATCH(Q.d, (k_poly_quad<DD, true><<<grid_of(Q.nslots, 64, nsm * 16), 64, 0, st>>>(Q)));
    } else {
        HV_DISPATCH(Q.d, (k_poly_quad<DD, false><<<grid_of(Q.nslots, 64, nsm * 16), 64, 0, st>>>(Q)));
    }
}

// The reference's heuristic integrand rule (src/heuristic.jl:105-166) on the
// areas the caller passes (from the Monte-Carlo integrator): per facet, the
// mean of f over its vertices with weight (d-1)/d and f at its centre with
// weight 1/d, times the area; the cell integral adds h/d (A f(x_i)/(d+1) +
// d/(d+1) I) over the facets.
template <int D>
__global__ void k_heur_iface(QuadRun Q, int p, const double* area, const double* fv, const double* fc, double* iface) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < Q.nslots;
         t += (long long)gridDim.x * blockDim.x) {
        const long long f0 = Q.foff[t], f1e = Q.foff[t + 1];
        if (f1e == f0) continue;
        for (int c = 0; c < p; ++c) {
            double s = 0.0;
            for (long long x = f0; x < f1e; ++x) s += fv[(size_t)Q.qv[x] * p + c];
            iface[t * p + c] = area[t] * ((D - 1.0) / D * s / (double)(f1e - f0) + fc[t * p + c] / D);
        }
    }
}

template <int D>
__global__ void k_heur_bulk(QuadRun Q, int p, const double* area, const double* fx, const double* iface, double* bulk) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Q.n; i += gridDim.x * blockDim.x) {
        double xi[D];
#pragma unroll
        for (int q = 0; q < D; ++q) xi[q] = Q.pts[(size_t)i * D + q];
        for (int c = 0; c < p; ++c) {
            double s = 0.0;
            for (long long t = Q.nbr_off[i]; t < Q.nbr_off[i + 1]; ++t) {
                const double h = facet_h<D>(Q, xi, Q.nbr[t]);
                s += h / D * (area[t] * fx[(size_t)i * p + c] / (D + 1.0) + D / (D + 1.0) * iface[t * p + c]);
            }
            bulk[(size_t)i * p + c] = s;
        }
    }
}

void launch_heur_integrals(const QuadRun& Q, int p, const double* area, const double* fv, const double* fc,
                           const double* fx, double* iface, double* bulk, cudaStream_t st) {
    HV_DISPATCH(Q.d, (k_heur_iface<DD><<<grid_of(Q.nslots, 256, 1 << 20), 256, 0, st>>>(Q, p, area, fv, fc, iface)));
    HV_DISPATCH(Q.d, (k_quad_copy<DD><<<grid_of(Q.n, 256, 1 << 20), 256, 0, st>>>(Q, p, iface)));
    if (bulk)
        HV_DISPATCH(Q.d, (k_heur_bulk<DD><<<grid_of(Q.n, 256, 1 << 20), 256, 0, st>>>(Q, p, area, fx, iface, bulk)));
}

void launch_quad_copy(const QuadRun& Q, int p, double* a, cudaStream_t st) {
    HV_DISPATCH(Q.d, (k_quad_copy<DD><<<grid_of(Q.n, 256, 1 << 20), 256, 0, st>>>(Q, p, a)));
}

void launch_quad_integrals(const QuadRun& Q, int p, const double* fv, const double* fc, const double* fx,
                           double* iface, double* bulk, cudaStream_t st) {
    HV_DISPATCH(Q.d, (k_quad_iface<DD><<<grid_of(Q.nslots, 256, 1 << 20), 256, 0, st>>>(Q, p, fv, fc, iface)));
    HV_DISPATCH(Q.d, (k_quad_copy<DD><<<grid_of(Q.n, 256, 1 << 20), 256, 0, st>>>(Q, p, iface)));
    HV_DISPATCH(Q.d, (k_quad_copy<DD><<<grid_of(Q.n, 256, 1 << 20), 256, 0, st>>>(Q, 1, Q.af)));
    if (bulk)
        HV_DISPATCH(Q.d, (k_quad_bulk<DD><<<grid_of(Q.n, 256, 1 << 20), 256, 0, st>>>(Q, p, fx, iface, bulk)));
}

}  // namespace hv
