// hv_integrate.cu -- per-cell integrators on the GPU.
//
// (VI_POLYGON lives in hv_poly.cu.)
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
    int np;                  // boundary planes: valid items are 0 .. n+np-1
    const DevPlane* planes;  // boundary planes, generator ids n + p
    const double* pts;       // original order, n x d
    const int* osig;         // V x (d+1), original 0-based items
    const double* oc;        // V x d
    const long long* inc_off;
    const int* inc;
    const long long* nbr_off;
    const int* nbr;
    double* area;            // aligned with nbr
    unsigned* status;        // 1: cell too large, 2: facet overflow, 4: degree over capacity,
                             // 8: neighbour item out of range, 16: neighbour CSR not sorted/symmetric
    int capC, capV, capF, capE, capI;
};

template <int D>
__device__ __forceinline__ double facet_height(const PolyArgs& A, const double* xi, int k) {
    if (k >= A.n) return plane_height<D>(A.planes[k - A.n], xi);
    double s = 0;
#pragma unroll
    for (int c = 0; c < D; ++c) { const double e = A.pts[(size_t)k * D + c] - xi[c]; s = fma(e, e, s); }
    return 0.5 * sqrt(s);
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

constexpr int MC_WPB = 4;
// neighbour records: D offsets, |delta|^2 (or -1 for a plane), 1/|delta| (or the
// plane's distance), padded to whole float4s
template <int D>
__host__ __device__ constexpr int mc_ep() { return D <= 2 ? 4 : 8; }

// One warp per cell, lane s % 32 casts direction s: the nearest bounding
// hyperplane along u over the cell's neighbours (FP32; a candidate that cannot
// beat the current minimum costs no division), t^d for the volume and
// t^(d-1)/|cos| for the facet hit, accumulated in FP64.  The facet sums are
// per warp: after every 32 directions the lanes that hit one facet add their
// contributions in direction order, so the result does not depend on the
// launch shape.
template <int D>
__global__ void __launch_bounds__(MC_WPB * 32) k_mc_cells(PolyArgs A, int ndir, unsigned long long seed, int capN,
                                                         double cvol, double* rawV, double* rawA, double* varV) {
    constexpr int EP = mc_ep<D>();
    extern __shared__ __align__(16) unsigned char smem[];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // per warp: capN x EP floats (records) + capN doubles (facet sums)
    float* nb = (float*)(smem) + (size_t)wib * capN * EP;
    double* acc = (double*)((float*)smem + (size_t)MC_WPB * capN * EP) + (size_t)wib * capN;
    for (int i = blockIdx.x * MC_WPB + wib; i < A.n; i += gridDim.x * MC_WPB) {
        const long long b = A.nbr_off[i];
        const int deg = (int)(A.nbr_off[i + 1] - b);
        if (deg > capN) {
            if (lane == 0) atomicOr(A.status, 4u);
            continue;
        }
        // every item must be another generator or one of the np planes
        bool bad = false;
        for (int t = lane; t < deg; t += 32) {
            const int k = A.nbr[b + t];
            bad |= k < 0 || k >= A.n + A.np || k == i;
        }
        if (__any_sync(0xFFFFFFFFu, bad)) {
            if (lane == 0) atomicOr(A.status, 8u);
            continue;
        }
        for (int t = lane; t < deg; t += 32) {
            const int k = A.nbr[b + t];
            float* e = nb + t * EP;
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
                const DevPlane& B = A.planes[k - A.n];
                double xd[D];
#pragma unroll
                for (int c = 0; c < D; ++c) { e[c] = B.n32[c]; xd[c] = A.pts[(size_t)i * D + c]; }
                e[D] = -1.f;  // plane marker
                e[D + 1] = (float)plane_height<D>(B, xd);
            }
#pragma unroll
            for (int c = D + 2; c < EP; ++c) e[c] = 0.f;
            acc[t] = 0.0;
        }
        __syncwarp();
        double vs = 0.0, vs2 = 0.0;
        for (int base = 0; base < ndir; base += 32) {
            const int s = base + lane;
            int jb = -1;
            double val = 0.0;
            if (s < ndir) {
                float u[D];
                mc_direction<D>(seed, (unsigned)s, (unsigned long long)i, u);
                float tb = INFINITY, cosb = 1.f;
                for (int t = 0; t < deg; ++t) {
                    float e[EP];
                    const float4* e4 = reinterpret_cast<const float4*>(nb + t * EP);
#pragma unroll
                    for (int h = 0; h < EP / 4; ++h) {
                        const float4 f = e4[h];
                        e[4 * h] = f.x; e[4 * h + 1] = f.y; e[4 * h + 2] = f.z; e[4 * h + 3] = f.w;
                    }
                    float du = 0.f;  // delta.u, or n.u (exactly +-u[axis] for axis planes)
#pragma unroll
                    for (int c = 0; c < D; ++c) du = fmaf(e[c], u[c], du);
                    if (!(du > 0.f)) continue;
                    float tt, cs;
                    if (e[D] >= 0.f) {
                        if (!(e[D] < tb * (2.f * du))) continue;
                        tt = e[D] / (2.f * du);
                        cs = du * e[D + 1];
                    } else {
                        if (!(e[D + 1] < tb * du)) continue;
                        tt = e[D + 1] / du;
                        cs = du;
                    }
                    if (tt > 0.f && tt < tb) { tb = tt; jb = t; cosb = cs; }
                }
                if (jb >= 0) {
                    const double td = (double)tb;
                    double tpow = 1.0;
#pragma unroll
                    for (int c = 0; c < D - 1; ++c) tpow *= td;
                    const double tdd = tpow * td;
                    vs += tdd;
                    vs2 += tdd * tdd;
                    val = tpow / fabs((double)cosb);
                }
            }
            // this round's hits: the lanes that hit the same facet sum their values in
            // lane (direction) order, the first of them adds the sum
            const unsigned grp = __match_any_sync(0xFFFFFFFFu, jb);
            double sum = 0.0;
            for (unsigned g = grp; g; g &= g - 1) sum += __shfl_sync(grp, val, __ffs(g) - 1);
            if (jb >= 0 && lane == __ffs(grp) - 1) acc[jb] += sum;
            __syncwarp();
        }
        // fixed-order reductions
        for (int off = 16; off > 0; off >>= 1) {
            vs += __shfl_down_sync(0xFFFFFFFFu, vs, off);
            vs2 += __shfl_down_sync(0xFFFFFFFFu, vs2, off);
        }
        __syncwarp();
        const double carea = D * cvol;
        for (int t = lane; t < deg; t += 32) rawA[b + t] = acc[t] * carea / ndir;
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
            if (lo > hi || A.nbr[lo] != i) {  // row k does not list i: not a sorted symmetric CSR
                atomicOr(A.status, 16u);
                continue;
            }
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
            if (k >= A.n || k < 0) continue;
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
    A.d = in.d; A.n = in.n; A.np = in.np;
    A.planes = in.planes;
    A.pts = in.pts; A.osig = in.osig; A.oc = in.oc;
    A.inc_off = in.inc_off; A.inc = in.inc; A.nbr_off = in.nbr_off; A.nbr = in.nbr;
    A.status = in.status;
    A.area = nullptr;
    A.capC = A.capV = A.capF = A.capE = A.capI = 0;
    return A;
}

template <int D>
static int mc_t(const IntegrateInput& in, int ndir, unsigned long long seed, int capN, double cvol, double* rawV,
                double* rawA, double* varV, double* outA, double* vol, int nsm, cudaStream_t st) {
    PolyArgs A = make_args(in);
    const size_t sm = mc_smem_bytes(D, capN);
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

size_t mc_smem_bytes(int d, int capN) {
    const int ep = d <= 2 ? 4 : 8;
    return (size_t)MC_WPB * capN * ep * sizeof(float) + (size_t)MC_WPB * capN * sizeof(double) + 16;
}

int launch_heuristic_mc(const IntegrateInput& in, int ndir, unsigned long long seed, int capN, double cvol,
                        double* rawV, double* rawA, double* varV, double* outA, double* vol, int nsm,
                        cudaStream_t st) {
    int rc = -1;
    HV_DISPATCH(in.d, (rc = mc_t<DD>(in, ndir, seed, capN, cvol, rawV, rawA, varV, outA, vol, nsm, st)));
    return rc;
}

}  // namespace hv
