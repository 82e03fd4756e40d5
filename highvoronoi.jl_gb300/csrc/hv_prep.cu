// hv_prep.cu -- point ordering, search tree and candidate lists.
//
// The reference builds a kd-tree with leaf size 10 split at the balanced index
// of the widest dimension (src/NearestNeighborModified/kd_tree.jl:27-158).  On
// the GPU the same role is played by an implicit complete binary tree over a
// Morton-ordered point array: leaves hold `leaf` consecutive points, node boxes
// are unions of their children and are built bottom-up in one pass.  Morton
// order adapts to clustered inputs the way the balanced kd split does (every
// leaf holds the same number of points) and keeps every later access to a
// generator's neighbourhood local in memory.
//
// Candidate lists: for every generator the K nearest other generators (FP32
// distances) and a radius `sec` such that every generator closer than `sec`
// is in the list.  The fast ray kernel accepts a decision only if the new
// empty sphere lies inside that radius (the security test).
#include <algorithm>

#include <cub/cub.cuh>

#include "hv_internal.cuh"
#include "hv_host.h"

namespace hv {

template <int D>
__global__ void k_morton(const double* __restrict__ in, int n, DevBox box, const DevPlane* __restrict__ planes, int np,
                         int B, unsigned long long* codes, int* idx, unsigned* status) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        unsigned q[D];
        bool ok = true;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const double x = in[(size_t)i * D + k];
            if (!(x > box.lo[k] && x < box.hi[k])) ok = false;
            double f = (x - box.lo[k]) / (box.hi[k] - box.lo[k]) * (double)(1u << B);
            f = fmin(fmax(f, 0.0), (double)((1u << B) - 1));
            q[k] = ok ? (unsigned)f : 0u;
        }
        // strictly inside every boundary plane
        for (int p = 0; p < np && ok; ++p) {
            double nx = 0;
#pragma unroll
            for (int k = 0; k < D; ++k) nx = fma(planes[p].n[k], in[(size_t)i * D + k], nx);
            if (!(nx < planes[p].off)) ok = false;
        }
        if (!ok) atomicOr(status, ST_BADINPUT);
        unsigned long long code = 0;
        for (int b = B - 1; b >= 0; --b) {
#pragma unroll
            for (int k = 0; k < D; ++k) code = (code << 1) | ((q[k] >> b) & 1u);
        }
        codes[i] = code;
        idx[i] = i;
    }
}

template <int D>
__global__ void k_gather(const double* __restrict__ in, const int* __restrict__ perm, int n, double* pts,
                         float* pts32, float* pts32lo) {
    constexpr int DP = (D <= 4) ? 4 : 8;
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const int o = perm[s];
        float f[DP], g[DP];
#pragma unroll
        for (int k = 0; k < DP; ++k) { f[k] = 0.f; g[k] = 0.f; }
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const double x = in[(size_t)o * D + k];
            pts[(size_t)s * D + k] = x;
            f[k] = (float)x;
            g[k] = (float)(x - (double)f[k]);
        }
        float4* dst = reinterpret_cast<float4*>(pts32 + (size_t)s * DP);
        float4* dlo = reinterpret_cast<float4*>(pts32lo + (size_t)s * DP);
#pragma unroll
        for (int h = 0; h < DP / 4; ++h) {
            dst[h] = make_float4(f[4 * h], f[4 * h + 1], f[4 * h + 2], f[4 * h + 3]);
            dlo[h] = make_float4(g[4 * h], g[4 * h + 1], g[4 * h + 2], g[4 * h + 3]);
        }
    }
}

// Bottom-up box construction: every leaf thread climbs while it is the second
// child to arrive at a node (the first arrival stops).
template <int D>
__global__ void k_bvh(DevMesh M, float* blo, float* bhi, unsigned* flags) {
    const int dp = M.dp;
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= M.P) return;
    float lo[D], hi[D];
#pragma unroll
    for (int k = 0; k < D; ++k) { lo[k] = INFINITY; hi[k] = -INFINITY; }
    if (l < M.nleaves) {
        const int s0 = l * M.leaf, s1 = min(s0 + M.leaf, M.n);
        for (int s = s0; s < s1; ++s) {
#pragma unroll
            for (int k = 0; k < D; ++k) {
                const double x = M.pts[(size_t)s * D + k];
                lo[k] = fminf(lo[k], __double2float_rd(x));
                hi[k] = fmaxf(hi[k], __double2float_ru(x));
            }
        }
    }
    int node = M.P + l;
#pragma unroll
    for (int k = 0; k < D; ++k) { blo[(size_t)node * dp + k] = lo[k]; bhi[(size_t)node * dp + k] = hi[k]; }
    __threadfence();
    while (node > 1) {
        const int parent = node >> 1;
        if (atomicAdd(&flags[parent], 1u) == 0u) return;
        __threadfence();
        const int c0 = 2 * parent, c1 = 2 * parent + 1;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            lo[k] = fminf(__ldcg(blo + (size_t)c0 * dp + k), __ldcg(blo + (size_t)c1 * dp + k));
            hi[k] = fmaxf(__ldcg(bhi + (size_t)c0 * dp + k), __ldcg(bhi + (size_t)c1 * dp + k));
            blo[(size_t)parent * dp + k] = lo[k];
            bhi[(size_t)parent * dp + k] = hi[k];
        }
        __threadfence();
        node = parent;
    }
}

// ---------------------------------------------------------------------------
// candidate lists: one warp per generator, shared-memory top-(K+1) buffer
// ---------------------------------------------------------------------------
constexpr int KNN_WPB = 4;

__device__ __forceinline__ bool pair_less(float da, int ia, float db, int ib) {
    return da < db || (da == db && ia < ib);
}

// Bitonic sort of n2 (power of two) (distance, index) pairs by a warp.
__device__ __forceinline__ void warp_bitonic_n(float* sd, int* si, int n2, int lane) {
#pragma unroll 1
    for (int k = 2; k <= n2; k <<= 1) {
#pragma unroll 1
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int q = lane; q < (n2 >> 1); q += 32) {
                const int i = ((q & ~(j - 1)) << 1) | (q & (j - 1));
                const int ixj = i | j;
                const bool up = (i & k) == 0;
                const float da = sd[i], db = sd[ixj];
                const int ia = si[i], ib = si[ixj];
                if (pair_less(db, ib, da, ia) == up) { sd[i] = db; sd[ixj] = da; si[i] = ib; si[ixj] = ia; }
            }
            __syncwarp();
        }
    }
}

// Keeps exactly the `need` smallest of the n buffered distances (n >= need):
// bisection over the bit patterns of the non-negative distances for the
// need-th smallest value t, then one ordered compaction keeping every entry
// below t and the first entries equal to t.  Returns t.
__device__ float warp_keep_smallest(float* sd, int* si, int n, int need, int lane) {
    const unsigned FULL = 0xFFFFFFFFu;
    unsigned lo = 0, hi = 0x7F800000u;
    while (lo < hi) {
        const unsigned mid = lo + ((hi - lo) >> 1);
        int c = 0;
        for (int x = lane; x < n; x += 32) c += (__float_as_uint(sd[x]) <= mid);
        c = __reduce_add_sync(FULL, c);
        if (c >= need) hi = mid; else lo = mid + 1;
    }
    const unsigned tb = lo;
    int clt = 0;
    for (int x = lane; x < n; x += 32) clt += (__float_as_uint(sd[x]) < tb);
    clt = __reduce_add_sync(FULL, clt);
    const int eq_budget = need - clt;
    int w = 0, eqseen = 0;
    for (int base = 0; base < n; base += 32) {
        const int x = base + lane;
        float dv = 0.f;
        int iv = 0;
        unsigned b = 0xFFFFFFFFu;
        if (x < n) { dv = sd[x]; iv = si[x]; b = __float_as_uint(dv); }
        const unsigned beq = __ballot_sync(FULL, x < n && b == tb);
        const unsigned lm = (1u << lane) - 1u;
        const bool keep = (x < n) && (b < tb || (b == tb && eqseen + __popc(beq & lm) < eq_budget));
        const unsigned bk = __ballot_sync(FULL, keep);
        if (keep) { sd[w + __popc(bk & lm)] = dv; si[w + __popc(bk & lm)] = iv; }
        w += __popc(bk);
        eqseen += __popc(beq);
    }
    __syncwarp();
    return __uint_as_float(tb);
}

// Keeps every buffered entry with distance <= t for a t whose count lies in
// [lo_need, hi_need] (lo_need <= n): interpolation on the volume law
// count ~ t^(D/2) from the largest distance, guarded by bisection, then one
// ordered compaction.  Typically one to three passes over the buffer instead of
// the 31 of the exact selection, which remains the fallback when ties leave no
// such t.  Returns t and sets `kept`.
template <int D>
__device__ float warp_keep_relaxed(float* sd, int* si, int n, int lo_need, int hi_need, int lane, int& kept) {
    const unsigned FULL = 0xFFFFFFFFu;
    unsigned bmin = 0xFFFFFFFFu, bmax = 0u;  // non-negative floats order as their bit patterns
    for (int x = lane; x < n; x += 32) {
        const unsigned b = __float_as_uint(sd[x]);
        bmin = min(bmin, b);
        bmax = max(bmax, b);
    }
    bmin = __reduce_min_sync(FULL, bmin);
    bmax = __reduce_max_sync(FULL, bmax);
    if (n <= hi_need) { kept = n; return __uint_as_float(bmax); }
    float lo = __uint_as_float(bmin), hi = __uint_as_float(bmax);
    const float target = 0.5f * (float)(lo_need + hi_need);
    float t = hi * exp2f(log2f(target / (float)n) * (2.f / D));
    int c = -1;
#pragma unroll 1
    for (int it = 0; it < 16; ++it) {
        if (!(t > lo && t < hi)) t = 0.5f * (lo + hi);
        if (!(t > lo && t < hi)) { c = -1; break; }  // adjacent values: ties
        int cc = 0;
        for (int x = lane; x < n; x += 32) cc += (sd[x] <= t);
        cc = __reduce_add_sync(FULL, cc);
        if (cc >= lo_need && cc <= hi_need) { c = cc; break; }
        if (cc < lo_need) lo = t; else hi = t;
        t *= exp2f(log2f(target / (float)max(cc, 1)) * (2.f / D));
        c = -1;
    }
    if (c < 0) {
        const float tb = warp_keep_smallest(sd, si, n, lo_need, lane);
        kept = lo_need;
        return tb;
    }
    int w = 0;
    for (int base = 0; base < n; base += 32) {
        const int x = base + lane;
        float dv = 0.f;
        int iv = 0;
        if (x < n) { dv = sd[x]; iv = si[x]; }
        const bool keep = x < n && dv <= t;
        const unsigned bk = __ballot_sync(FULL, keep);
        if (keep) { const int pos = w + __popc(bk & ((1u << lane) - 1u)); sd[pos] = dv; si[pos] = iv; }
        w += __popc(bk);
    }
    __syncwarp();
    kept = c;
    return t;
}

constexpr int KNN_STK = 768;  // traversal stack entries per warp (bounded by 32 x tree depth + 64)
constexpr int KNN_LQ = 64;     // queued leaves per warp

// One warp per generator.  Phase 1 inserts the generator's smallest ancestor
// subtree holding at least K+1+leaf points (a contiguous Morton range, read
// coalesced) and keeps about the K+1 nearest, which bounds the K+1-th
// distance.  Phase 2 walks the rest of the tree 32 nodes per step (one box test
// per lane; the walk starts at the 32 nodes of depth 5), queues the surviving
// leaves and scans them 64 points at a time.  The buffer is thinned to between
// K+1 and 1.25 K entries whenever it fills (every entry beyond its threshold is
// farther than the K+1 it keeps), and the final at most pow2(K+1) entries are
// sorted by (distance, index): the list is the first K, its complete radius the
// K+1-th distance.
// part 0 takes the generators q = 0, qs, 2 qs, ... (the descent seeds), part 1
// the others; qs <= 1: every generator.
template <int D, int CAP>
__global__ void __launch_bounds__(KNN_WPB * 32) k_knn(DevMesh M, int* knn, float* sec, int qs, int part) {
    constexpr int DP = (D <= 4) ? 4 : 8;
    __shared__ float sd[KNN_WPB][CAP];
    __shared__ int si[KNN_WPB][CAP];
    __shared__ int sstack[KNN_WPB][KNN_STK];
    __shared__ int sleaf[KNN_WPB][KNN_LQ];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int K = M.K;
    const int W = max(K / 4, 8);                        // slack of a thinned buffer
    int P1 = 32;                                         // final buffer bound (sorted)
    while (P1 < K + 1) P1 <<= 1;
    const unsigned FULL = 0xFFFFFFFFu;
    const unsigned lt = (1u << lane) - 1u;
    const float ex = M.ulp32;
    const int L = M.leaf;
    const int lsh = (L & (L - 1)) == 0 ? __ffs(L) - 1 : -1;  // leaf size as a shift when a power of two
    float* d = sd[wib];
    int* ix = si[wib];
    int* stk = sstack[wib];
    int* lq = sleaf[wib];
    const int nseed = qs <= 1 ? M.n : (M.n + qs - 1) / qs;
    const int nq = qs <= 1 ? M.n : (part == 0 ? nseed : M.n - nseed);
    for (int w = blockIdx.x * KNN_WPB + wib; w < nq; w += gridDim.x * KNN_WPB) {
        const int q = qs <= 1 ? w : (part == 0 ? w * qs : w + w / (qs - 1) + 1);
        float xq[DP];
        {
            const float4* p = reinterpret_cast<const float4*>(M.pts32 + (size_t)q * DP);
#pragma unroll
            for (int h = 0; h < DP / 4; ++h) {
                float4 f = __ldg(p + h);
                xq[4 * h] = f.x; xq[4 * h + 1] = f.y; xq[4 * h + 2] = f.z; xq[4 * h + 3] = f.w;
            }
        }
        int cnt = 0;
        float thr = INFINITY;
        auto dist2 = [&](int s) -> float {
            if (s < 0 || s >= M.n || s == q) return INFINITY;
            float xs[DP];
            const float4* p = reinterpret_cast<const float4*>(M.pts32 + (size_t)s * DP);
#pragma unroll
            for (int h = 0; h < DP / 4; ++h) {
                float4 f = __ldg(p + h);
                xs[4 * h] = f.x; xs[4 * h + 1] = f.y; xs[4 * h + 2] = f.z; xs[4 * h + 3] = f.w;
            }
            float d2 = 0.f;
#pragma unroll
            for (int k = 0; k < D; ++k) { const float e = xs[k] - xq[k]; d2 = fmaf(e, e, d2); }
            return d2;
        };
        // the points pt(0..np-1) (except q) with d2 < thr into the buffer, two
        // rounds of 32 per step (both loads in flight together)
        auto scan = [&](int np, auto pt) {
            for (int base = 0; base < np; base += 64) {
                const int s0 = base + lane < np ? pt(base + lane) : -1;
                const int s1 = base + 32 + lane < np ? pt(base + 32 + lane) : -1;
                const float d0 = dist2(s0), d1 = dist2(s1);
                const bool t0 = d0 < thr, t1 = d1 < thr;
                const unsigned b0 = __ballot_sync(FULL, t0), b1 = __ballot_sync(FULL, t1);
                if (t0) { const int pos = cnt + __popc(b0 & lt); d[pos] = d0; ix[pos] = s0; }
                cnt += __popc(b0);
                if (t1) { const int pos = cnt + __popc(b1 & lt); d[pos] = d1; ix[pos] = s1; }
                cnt += __popc(b1);
                __syncwarp();
                if (cnt > CAP - 64) thr = warp_keep_relaxed<D>(d, ix, cnt, K + 1, K + 1 + W, lane, cnt);
            }
        };
        // ---- phase 1: the smallest ancestor subtree with at least K+1+leaf points
        const int lq0 = q / L;
        int A = M.P + lq0, depthA = 0;  // node id and levels above the leaf
        int la0 = lq0, la1 = lq0 + 1;
        while (A > 1 && (min(la1 * L, M.n) - la0 * L) < K + 1 + L) {
            A >>= 1;
            ++depthA;
            la0 = (A << depthA) - M.P;
            la1 = ((A + 1) << depthA) - M.P;
            la0 = max(la0, 0);
            la1 = min(la1, M.nleaves);
        }
        {
            const int s0 = la0 * L;
            scan(min(la1 * L, M.n) - s0, [&](int x) { return s0 + x; });
        }
        if (cnt >= K + 1) thr = warp_keep_relaxed<D>(d, ix, cnt, K + 1, K + 1 + W, lane, cnt);
        // ---- phase 2: the rest of the tree, from the nodes of depth min(5, log2 P)
        if (A > 1) {
            const int lvA = 31 - __clz(A);
            const int lv0 = min(5, 31 - __clz(M.P));
            int sp = 1 << lv0, nl = 0;
            if (lane < sp) stk[lane] = (1 << lv0) + lane;
            __syncwarp();
            while (sp > 0 || nl > 0) {
                if (nl >= 2 || (sp == 0 && nl > 0)) {
                    if (lsh >= 0) scan(nl << lsh, [&](int x) { return (lq[x >> lsh] << lsh) + (x & (L - 1)); });
                    else scan(nl * L, [&](int x) { return lq[x / L] * L + x % L; });
                    nl = 0;
                    continue;
                }
                const int nt = min(sp, 32);
                const int node = lane < nt ? stk[sp - nt + lane] : 1;
                sp -= nt;
                __syncwarp();
                bool keep = lane < nt;
                if (keep) {
                    // already scanned: the phase-1 subtree
                    const int lv = 31 - __clz(node);
                    if (lv >= lvA && (node >> (lv - lvA)) == A) keep = false;
                }
                if (keep && isfinite(thr)) {
                    float bd = 0.f;
                    float bl[DP], bh[DP];
                    load_f4<DP>(M.blo + (size_t)node * DP, bl);
                    load_f4<DP>(M.bhi + (size_t)node * DP, bh);
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        const float l = bl[k], h = bh[k];
                        const float e = xq[k] < l ? l - xq[k] : (xq[k] > h ? xq[k] - h : 0.f);
                        bd = fmaf(e, e, bd);
                    }
                    keep = !(bd > thr * 1.00001f);
                }
                const bool isleaf = node >= M.P;
                const bool lvf = keep && isleaf && (node - M.P) < M.nleaves;
                const bool in = keep && !isleaf;
                const unsigned bl = __ballot_sync(FULL, lvf), bi = __ballot_sync(FULL, in);
                if (sp + 2 * __popc(bi) > KNN_STK) {
                    if (lane == 0) atomicOr(M.status, ST_STACK);
                    break;
                }
                if (lvf) lq[nl + __popc(bl & lt)] = node - M.P;
                if (in) {
                    const int p = sp + 2 * __popc(bi & lt);
                    stk[p] = 2 * node + 1;
                    stk[p + 1] = 2 * node;
                }
                nl += __popc(bl);
                sp += 2 * __popc(bi);
                __syncwarp();
            }
        }
        if (cnt > P1) warp_keep_relaxed<D>(d, ix, cnt, K + 1, P1, lane, cnt);
        int n2 = 32;
        while (n2 < cnt) n2 <<= 1;
        for (int i = cnt + lane; i < n2; i += 32) { d[i] = INFINITY; ix[i] = 0x7FFFFFFF; }
        __syncwarp();
        warp_bitonic_n(d, ix, n2, lane);
        for (int c = lane; c < K; c += 32) knn[(size_t)q * K + c] = (c < cnt) ? ix[c] : -1;
        if (lane == 0) {
            float r = INFINITY;
            if (cnt >= K + 1) {
                r = sqrtf(d[K]) * (1.f - 4e-6f) - 3.f * sqrtf((float)D) * ex;
                r = fmaxf(r, 0.f);
            }
            sec[q] = r;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// host launchers
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

int morton_bits(int d, int n) {
    // at least 2^8 grid cells per point: ties are rare even in clusters, and the
    // sort reads only these d * bits bits
    int lg = 0;
    while ((1ll << lg) < (long long)std::max(n, 1)) ++lg;
    const int bmax = std::min(21, 63 / d);
    return std::max(1, std::min(bmax, (lg + 8 + d - 1) / d));
}

void launch_morton(int d, const double* in, int n, const double* lo, const double* hi, const DevPlane* planes, int np,
                   unsigned long long* codes, int* idx, unsigned* status, cudaStream_t st) {
    if (n <= 0) return;
    const int bits = morton_bits(d, n);
    DevBox box;
    for (int k = 0; k < d; ++k) { box.lo[k] = lo[k]; box.hi[k] = hi[k]; }
    const int blocks = (n + 255) / 256;
    HV_DISPATCH(d, (k_morton<DD><<<blocks, 256, 0, st>>>(in, n, box, planes, np, bits, codes, idx, status)));
}

void launch_gather(int d, const double* in, const int* perm, int n, double* pts, float* pts32, float* pts32lo,
                   cudaStream_t st) {
    if (n <= 0) return;
    const int blocks = (n + 255) / 256;
    HV_DISPATCH(d, (k_gather<DD><<<blocks, 256, 0, st>>>(in, perm, n, pts, pts32, pts32lo)));
}

void launch_bvh(const DevMesh& M, float* blo, float* bhi, unsigned* flags, cudaStream_t st) {
    if (M.n <= 0) return;
    const int blocks = (M.P + 127) / 128;
    HV_DISPATCH(M.d, (k_bvh<DD><<<blocks, 128, 0, st>>>(M, blo, bhi, flags)));
}

template <int D>
static void launch_knn_t(const DevMesh& M, int* knn, float* sec, int qs, int part, cudaStream_t st) {
    const int nseed = qs <= 1 ? M.n : (M.n + qs - 1) / qs;
    const int nq = qs <= 1 ? M.n : (part == 0 ? nseed : M.n - nseed);
    if (nq <= 0) return;
    const int blocks = (nq + KNN_WPB - 1) / KNN_WPB;
    const int need = 2 * M.K + 64;
    if (need <= 128) k_knn<D, 128><<<blocks, KNN_WPB * 32, 0, st>>>(M, knn, sec, qs, part);
    else if (need <= 256) k_knn<D, 256><<<blocks, KNN_WPB * 32, 0, st>>>(M, knn, sec, qs, part);
    else if (need <= 512) k_knn<D, 512><<<blocks, KNN_WPB * 32, 0, st>>>(M, knn, sec, qs, part);
    else k_knn<D, 1024><<<blocks, KNN_WPB * 32, 0, st>>>(M, knn, sec, qs, part);
}

void launch_knn(const DevMesh& M, int* knn, float* sec, int qs, int part, cudaStream_t st) {
    if (M.n <= 0) return;
    HV_DISPATCH(M.d, (launch_knn_t<DD>(M, knn, sec, qs, part, st)));
}

size_t sort_pairs_u64_i32_temp(int n) {
    size_t b = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, b, (const unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                    (const int*)nullptr, (int*)nullptr, n);
    return b;
}
void sort_pairs_u64_i32(void* temp, size_t temp_bytes, const unsigned long long* kin, unsigned long long* kout,
                        const int* vin, int* vout, int n, int end_bit, cudaStream_t st) {
    cub::DeviceRadixSort::SortPairs(temp, temp_bytes, kin, kout, vin, vout, n, 0, end_bit, st);
}
size_t sort_pairs_u32_i32_temp(int n) {
    size_t b = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, b, (const unsigned*)nullptr, (unsigned*)nullptr, (const int*)nullptr,
                                    (int*)nullptr, n);
    return b;
}
void sort_pairs_u32_i32(void* temp, size_t temp_bytes, const unsigned* kin, unsigned* kout, const int* vin,
                        int* vout, int n, int end_bit, cudaStream_t st) {
    cub::DeviceRadixSort::SortPairs(temp, temp_bytes, kin, kout, vin, vout, n, 0, end_bit, st);
}
size_t sort_keys_u64_temp(long long n) {
    size_t b = 0;
    cub::DeviceRadixSort::SortKeys(nullptr, b, (const unsigned long long*)nullptr, (unsigned long long*)nullptr, n);
    return b;
}
void sort_keys_u64(void* temp, size_t temp_bytes, const unsigned long long* kin, unsigned long long* kout,
                   long long n, cudaStream_t st) {
    cub::DeviceRadixSort::SortKeys(temp, temp_bytes, kin, kout, n, 0, 64, st);
}
size_t scan_temp(int n) {
    size_t b = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, b, (const long long*)nullptr, (long long*)nullptr, n);
    return b;
}
void exclusive_scan_i64(void* temp, size_t temp_bytes, const long long* in, long long* out, int n, cudaStream_t st) {
    cub::DeviceScan::ExclusiveSum(temp, temp_bytes, in, out, n, st);
}

}  // namespace hv
