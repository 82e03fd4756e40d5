// hv_post.cu -- canonical vertex order, cell incidence and neighbour lists.
//
// After the search every vertex is renumbered in the lexicographic order of
// its signature written with original generator ids (planes as n+p).  The
// order is a pure function of the vertex set, so every later result (lists,
// integrals, sums) is bitwise reproducible regardless of the scheduling of
// the wavefront.
//
// Neighbours of cell i are the sorted union of the generators of its
// vertices, planes included (neighbors_of_cell_new, src/neighbors.jl:219-258).
#include "hv_internal.cuh"
#include "hv_host.h"

namespace hv {

template <int D>
__global__ void k_canon_keys(DevMesh M, unsigned V, unsigned* keys) {
    const bool shard = M.own0 > 0 || M.own1 < M.n;
    for (unsigned v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        if (shard) {
            // a shard keeps the vertices whose smallest generator (internal order) it
            // owns; the others get the largest key and sort behind them
            const int s0 = M.vsig[(size_t)v * (D + 1)];
            if (s0 < M.own0 || s0 >= M.own1) {
#pragma unroll
                for (int k = 0; k <= D; ++k) keys[(size_t)k * V + v] = 0xFFFFFFFFu;
                continue;
            }
            count_add(M.cnt + C_OWNED);
        }
        unsigned s[D + 1];
#pragma unroll
        for (int k = 0; k <= D; ++k) {
            const int it = M.vsig[(size_t)v * (D + 1) + k];
            s[k] = it < M.n ? (unsigned)__ldg(M.perm + it) : (unsigned)it;
        }
#pragma unroll
        for (int a = 1; a <= D; ++a) {
#pragma unroll
            for (int b = a; b > 0; --b) {
                if (s[b] < s[b - 1]) { unsigned x = s[b]; s[b] = s[b - 1]; s[b - 1] = x; }
            }
        }
#pragma unroll
        for (int k = 0; k <= D; ++k) keys[(size_t)k * V + v] = s[k];
    }
}

__global__ void k_gather_keys(const unsigned* __restrict__ keys_pos, const int* __restrict__ order, unsigned V,
                              unsigned* out) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < V; i += gridDim.x * blockDim.x)
        out[i] = keys_pos[order[i]];
}

template <int D>
__global__ void k_canon_gather(DevMesh M, unsigned V, const unsigned* __restrict__ keys,
                               const int* __restrict__ order, int* osig, double* oc) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < V; i += gridDim.x * blockDim.x) {
        const int v = order[i];
#pragma unroll
        for (int k = 0; k <= D; ++k) osig[(size_t)i * (D + 1) + k] = (int)keys[(size_t)k * V + v];
#pragma unroll
        for (int k = 0; k < D; ++k) oc[(size_t)i * D + k] = M.vc[(size_t)v * D + k];
    }
}

template <int D>
__global__ void k_inc_pairs(int n, unsigned V, const int* __restrict__ osig, unsigned long long* pairs,
                            long long* cnt) {
    for (unsigned v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
#pragma unroll
        for (int k = 0; k <= D; ++k) {
            const int it = osig[(size_t)v * (D + 1) + k];
            if (it < n) {
                pairs[(size_t)v * (D + 1) + k] = ((unsigned long long)(unsigned)it << 32) | v;
                atomicAdd((unsigned long long*)(cnt + it), 1ull);
            } else {
                pairs[(size_t)v * (D + 1) + k] = ~0ull;
            }
        }
    }
}

__global__ void k_inc_split(unsigned long long npairs, const unsigned long long* __restrict__ pairs, int* inc) {
    for (unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; t < npairs;
         t += (unsigned long long)gridDim.x * blockDim.x)
        inc[t] = (int)(unsigned)(pairs[t] & 0xFFFFFFFFull);
}

// One warp per cell: shared-memory hash set of the generators met.
constexpr int NB_WPB = 4;
constexpr int NB_HS = 1024;

template <int D>
__device__ int nbr_collect(int i, const long long* inc_off, const int* inc, const int* osig, int* hs, int lane) {
    for (int k = lane; k < NB_HS; k += 32) hs[k] = 0x7FFFFFFF;
    __syncwarp();
    int fresh = 0;
    for (long long t = inc_off[i] + lane; t < inc_off[i + 1]; t += 32) {
        const int v = inc[t];
#pragma unroll
        for (int k = 0; k <= D; ++k) {
            const int it = osig[(size_t)v * (D + 1) + k];
            if (it == i) continue;
            unsigned h = ((unsigned)it * 2654435761u) & (NB_HS - 1);
            for (int probe = 0; probe < NB_HS; ++probe) {
                const int prev = atomicCAS(&hs[h], 0x7FFFFFFF, it);
                if (prev == 0x7FFFFFFF) { ++fresh; break; }
                if (prev == it) break;
                h = (h + 1) & (NB_HS - 1);
            }
        }
    }
    __syncwarp();
    return __reduce_add_sync(0xFFFFFFFFu, fresh);
}

template <int D>
__global__ void __launch_bounds__(NB_WPB * 32) k_nbr_count(int n, const long long* inc_off, const int* inc,
                                                           const int* osig, long long* nnbr, unsigned* status) {
    __shared__ int shs[NB_WPB][NB_HS];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = blockIdx.x * NB_WPB + wib; i < n; i += gridDim.x * NB_WPB) {
        const int c = nbr_collect<D>(i, inc_off, inc, osig, shs[wib], lane);
        if (lane == 0) {
            nnbr[i] = c;
            if (c > NB_HS / 2) atomicOr(status, ST_HASH);
        }
        __syncwarp();
    }
}

template <int D>
__global__ void __launch_bounds__(NB_WPB * 32) k_nbr_fill(int n, const long long* inc_off, const int* inc,
                                                          const int* osig, const long long* nbr_off, int* nbr) {
    __shared__ int shs[NB_WPB][NB_HS];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int i = blockIdx.x * NB_WPB + wib; i < n; i += gridDim.x * NB_WPB) {
        int* hs = shs[wib];
        const int c = nbr_collect<D>(i, inc_off, inc, osig, hs, lane);
        // bitonic sort of the whole table (empty slots hold INT_MAX)
#pragma unroll 1
        for (int k = 2; k <= NB_HS; k <<= 1) {
#pragma unroll 1
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int a = lane; a < NB_HS; a += 32) {
                    const int b = a ^ j;
                    if (b > a) {
                        const bool up = (a & k) == 0;
                        const int x = hs[a], y = hs[b];
                        if ((x > y) == up) { hs[a] = y; hs[b] = x; }
                    }
                }
                __syncwarp();
            }
        }
        const long long o = nbr_off[i];
        for (int k = lane; k < c; k += 32) nbr[o + k] = hs[k];
        __syncwarp();
    }
}

template <int D>
__global__ void k_out_vertices(unsigned V, const int* __restrict__ osig, int64_t* out) {
    const unsigned long long total = (unsigned long long)V * (D + 1);
    for (unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; t < total;
         t += (unsigned long long)gridDim.x * blockDim.x)
        out[t] = (int64_t)osig[t] + 1;
}

__global__ void k_out_nbr(long long total, const int* __restrict__ nbr, int64_t* out) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total; t += (long long)gridDim.x * blockDim.x)
        out[t] = (int64_t)nbr[t] + 1;
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

static unsigned grid_for(unsigned long long n, int bs) {
    unsigned long long b = (n + bs - 1) / bs;
    if (b > 65535ull * 16) b = 65535ull * 16;
    return (unsigned)(b ? b : 1);
}

// ---------------------------------------------------------------------------
// incremental refinement (hv_mesh_refine): old vertices whose circumsphere a
// new generator invades disappear; the rest merge with the new vertices
// ---------------------------------------------------------------------------
constexpr int RK_TILE = 256;
template <int D>
__global__ void __launch_bounds__(RK_TILE) k_refine_keep(int n_old, int k, unsigned V, const int* __restrict__ osig,
                                                         const double* __restrict__ oc, const double* __restrict__ pts,
                                                         const double* __restrict__ newp, long long* keep,
                                                         unsigned* uncertain) {
    __shared__ double sq[RK_TILE][D];
    const unsigned v = blockIdx.x * blockDim.x + threadIdx.x;
    double c[D], r2 = 0.0;
    bool live = v < V, gone = false, unsure = false;
    if (live) {
        const int s0 = osig[(size_t)v * (D + 1)];  // the smallest item: a generator
#pragma unroll
        for (int q = 0; q < D; ++q) {
            c[q] = oc[(size_t)v * D + q];
            const double e = pts[(size_t)s0 * D + q] - c[q];
            r2 = fma(e, e, r2);
        }
    }
    for (int base = 0; base < k; base += RK_TILE) {
        __syncthreads();
        for (int x = threadIdx.x; x < RK_TILE && base + x < k; x += blockDim.x)
#pragma unroll
            for (int q = 0; q < D; ++q) sq[x][q] = newp[(size_t)(base + x) * D + q];
        __syncthreads();
        const int m = min(RK_TILE, k - base);
        if (live && !gone)
            for (int x = 0; x < m; ++x) {
                double dd = 0.0;
#pragma unroll
                for (int q = 0; q < D; ++q) { const double e = sq[x][q] - c[q]; dd = fma(e, e, dd); }
                // a margin far above the rounding of the stored centre and radius
                if (dd < r2 * (1.0 - 1e-9)) { gone = true; break; }
                if (dd <= r2 * (1.0 + 1e-9)) unsure = true;
            }
    }
    if (live) {
        keep[v] = gone ? 0 : 1;
        if (unsure && !gone) atomicAdd(uncertain, 1u);
    }
}

// Lexicographic comparison of a (d+1)-item row of the old mesh, with its
// boundary items n_old+p renumbered to n_old+k+p, against a row of the new one.
template <int D>
__device__ __forceinline__ int cmp_rows(const int* a, int n_old, int k, const int* b) {
#pragma unroll
    for (int q = 0; q <= D; ++q) {
        const int x = a[q] >= n_old ? a[q] + k : a[q];
        if (x != b[q]) return x < b[q] ? -1 : 1;
    }
    return 0;
}

template <int D>
__global__ void k_refine_merge_old(int n_old, int k, unsigned V_old, const int* __restrict__ osig,
                                   const double* __restrict__ oc, const long long* __restrict__ keep,
                                   const long long* __restrict__ rank, unsigned V_new, const int* __restrict__ nsig,
                                   int* out_sig, double* out_c) {
    for (unsigned v = blockIdx.x * blockDim.x + threadIdx.x; v < V_old; v += gridDim.x * blockDim.x) {
        if (!keep[v]) continue;
        const int* a = osig + (size_t)v * (D + 1);
        unsigned lo = 0, hi = V_new;  // new rows below this one
        while (lo < hi) {
            const unsigned md = (lo + hi) >> 1;
            if (cmp_rows<D>(a, n_old, k, nsig + (size_t)md * (D + 1)) > 0) lo = md + 1; else hi = md;
        }
        const size_t pos = (size_t)rank[v] + lo;
#pragma unroll
        for (int q = 0; q <= D; ++q) out_sig[pos * (D + 1) + q] = a[q] >= n_old ? a[q] + k : a[q];
#pragma unroll
        for (int q = 0; q < D; ++q) out_c[pos * D + q] = oc[(size_t)v * D + q];
    }
}

template <int D>
__global__ void k_refine_merge_new(int n_old, int k, unsigned V_old, const int* __restrict__ osig,
                                   const long long* __restrict__ rank, unsigned V_new, const int* __restrict__ nsig,
                                   const double* __restrict__ nc, int* out_sig, double* out_c) {
    for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < V_new; w += gridDim.x * blockDim.x) {
        const int* b = nsig + (size_t)w * (D + 1);
        unsigned lo = 0, hi = V_old;  // old rows below this one (kept or not)
        while (lo < hi) {
            const unsigned md = (lo + hi) >> 1;
            if (cmp_rows<D>(osig + (size_t)md * (D + 1), n_old, k, b) < 0) lo = md + 1; else hi = md;
        }
        const size_t pos = (size_t)rank[lo] + w;  // rank: exclusive count of kept rows (V_old + 1 entries)
#pragma unroll
        for (int q = 0; q <= D; ++q) out_sig[pos * (D + 1) + q] = b[q];
#pragma unroll
        for (int q = 0; q < D; ++q) out_c[pos * D + q] = nc[(size_t)w * D + q];
    }
}

void launch_refine_keep(int d, int n_old, int k, unsigned V, const int* osig, const double* oc, const double* pts,
                        const double* newp, long long* keep, unsigned* uncertain, cudaStream_t st) {
    if (!V) return;
    HV_DISPATCH(d, (k_refine_keep<DD><<<(V + RK_TILE - 1) / RK_TILE, RK_TILE, 0, st>>>(n_old, k, V, osig, oc, pts,
                                                                                       newp, keep, uncertain)));
}

void launch_refine_merge(int d, int n_old, int k, unsigned V_old, const int* osig, const double* oc,
                         const long long* keep, const long long* rank, unsigned V_new, const int* nsig,
                         const double* nc, int* out_sig, double* out_c, cudaStream_t st) {
    HV_DISPATCH(d, (k_refine_merge_old<DD><<<grid_for(std::max(V_old, 1u), 256), 256, 0, st>>>(
                        n_old, k, V_old, osig, oc, keep, rank, V_new, nsig, out_sig, out_c)));
    HV_DISPATCH(d, (k_refine_merge_new<DD><<<grid_for(std::max(V_new, 1u), 256), 256, 0, st>>>(
                        n_old, k, V_old, osig, rank, V_new, nsig, nc, out_sig, out_c)));
}

void launch_canon_keys(const DevMesh& M, unsigned V, unsigned* keys, cudaStream_t st) {
    if (!V) return;
    HV_DISPATCH(M.d, (k_canon_keys<DD><<<grid_for(V, 256), 256, 0, st>>>(M, V, keys)));
}
void launch_gather_keys(const unsigned* keys_pos, const int* order, unsigned V, unsigned* out, cudaStream_t st) {
    if (!V) return;
    k_gather_keys<<<grid_for(V, 256), 256, 0, st>>>(keys_pos, order, V, out);
}
// The first d items of every canonical signature packed into one 64-bit key
// (`bits` bits each, the first item most significant).
__global__ void k_pack_keys(const unsigned* __restrict__ keys, unsigned V, int d, int bits, unsigned long long* out) {
    for (unsigned v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        unsigned long long k = 0;
        for (int q = 0; q < d; ++q) k = (k << bits) | keys[(size_t)q * V + v];
        out[v] = k;
    }
}

// After the stable sort by the packed first d items, a run of equal keys holds
// the vertices sharing d generators -- the two end points of an edge -- and is
// put in the order of the last item.
__global__ void k_fix_runs(const unsigned long long* __restrict__ sk, const unsigned* __restrict__ last, unsigned V,
                           int* order) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i + 1 < V; i += gridDim.x * blockDim.x) {
        if (sk[i + 1] != sk[i] || (i > 0 && sk[i - 1] == sk[i])) continue;
        unsigned j = i + 2;
        while (j < V && sk[j] == sk[i]) ++j;
        for (unsigned x = i + 1; x < j; ++x)
            for (unsigned y = x; y > i && last[order[y]] < last[order[y - 1]]; --y) {
                const int z = order[y]; order[y] = order[y - 1]; order[y - 1] = z;
            }
    }
}

void launch_pack_keys(const unsigned* keys, unsigned V, int d, int bits, unsigned long long* out, cudaStream_t st) {
    if (!V) return;
    k_pack_keys<<<grid_for(V, 256), 256, 0, st>>>(keys, V, d, bits, out);
}
void launch_fix_runs(const unsigned long long* sk, const unsigned* last, unsigned V, int* order, cudaStream_t st) {
    if (V < 2) return;
    k_fix_runs<<<grid_for(V, 256), 256, 0, st>>>(sk, last, V, order);
}
void launch_canon_gather(const DevMesh& M, unsigned V, const unsigned* keys, const int* order, int* osig,
                         double* oc, cudaStream_t st) {
    if (!V) return;
    HV_DISPATCH(M.d, (k_canon_gather<DD><<<grid_for(V, 256), 256, 0, st>>>(M, V, keys, order, osig, oc)));
}
void launch_inc_pairs(int d, int n, unsigned V, const int* osig, unsigned long long* pairs, long long* cnt,
                      cudaStream_t st) {
    if (!V) return;
    HV_DISPATCH(d, (k_inc_pairs<DD><<<grid_for(V, 256), 256, 0, st>>>(n, V, osig, pairs, cnt)));
}
void launch_inc_split(unsigned long long npairs, const unsigned long long* pairs, int* inc, cudaStream_t st) {
    if (!npairs) return;
    k_inc_split<<<grid_for(npairs, 256), 256, 0, st>>>(npairs, pairs, inc);
}
void launch_nbr_count(int d, int n, const long long* inc_off, const int* inc, const int* osig, long long* nnbr,
                      unsigned* status, cudaStream_t st) {
    if (n <= 0) return;
    HV_DISPATCH(d, (k_nbr_count<DD><<<grid_for(n, NB_WPB), NB_WPB * 32, 0, st>>>(n, inc_off, inc, osig, nnbr, status)));
}
void launch_nbr_fill(int d, int n, const long long* inc_off, const int* inc, const int* osig,
                     const long long* nbr_off, int* nbr, cudaStream_t st) {
    if (n <= 0) return;
    HV_DISPATCH(d, (k_nbr_fill<DD><<<grid_for(n, NB_WPB), NB_WPB * 32, 0, st>>>(n, inc_off, inc, osig, nbr_off, nbr)));
}
void launch_out_vertices(int d, unsigned V, const int* osig, int64_t* out, cudaStream_t st) {
    if (!V) return;
    HV_DISPATCH(d, (k_out_vertices<DD><<<grid_for((unsigned long long)V * (DD + 1), 256), 256, 0, st>>>(V, osig, out)));
}
void launch_out_nbr(long long total, const int* nbr, int64_t* out, cudaStream_t st) {
    if (total <= 0) return;
    k_out_nbr<<<grid_for(total, 256), 256, 0, st>>>(total, nbr, out);
}

}  // namespace hv
