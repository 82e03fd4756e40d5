// hv_search.cu -- dimension dispatch of the vertex-search launchers
// (kernels in hv_search_impl.cuh, one translation unit per dimension).
#include "hv_internal.cuh"
#include "hv_host.h"

namespace hv {

void launch_register_d2(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st);
void launch_register_d3(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st);
void launch_register_d4(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st);
void launch_register_d5(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st);
void launch_register_d6(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st);
void launch_refine_d2(const DevMesh& M, unsigned V, int nsm, cudaStream_t st);
void launch_refine_d3(const DevMesh& M, unsigned V, int nsm, cudaStream_t st);
void launch_refine_d4(const DevMesh& M, unsigned V, int nsm, cudaStream_t st);
void launch_refine_d5(const DevMesh& M, unsigned V, int nsm, cudaStream_t st);
void launch_refine_d6(const DevMesh& M, unsigned V, int nsm, cudaStream_t st);
void launch_centers_d2(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st);
void launch_centers_d3(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st);
void launch_centers_d4(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st);
void launch_centers_d5(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st);
void launch_centers_d6(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st);
void launch_descent_d2(const DevMesh& M, int stride, int nseeds, unsigned long long seed, int* failed, unsigned* nfailed, int nsm, cudaStream_t st);
void launch_descent_d3(const DevMesh& M, int stride, int nseeds, unsigned long long seed, int* failed, unsigned* nfailed, int nsm, cudaStream_t st);
void launch_descent_d4(const DevMesh& M, int stride, int nseeds, unsigned long long seed, int* failed, unsigned* nfailed, int nsm, cudaStream_t st);
void launch_descent_d5(const DevMesh& M, int stride, int nseeds, unsigned long long seed, int* failed, unsigned* nfailed, int nsm, cudaStream_t st);
void launch_descent_d6(const DevMesh& M, int stride, int nseeds, unsigned long long seed, int* failed, unsigned* nfailed, int nsm, cudaStream_t st);
void launch_plain_d2(const DevMesh& M, unsigned f0, unsigned f1, int nsm, cudaStream_t st);
void launch_plain_d3(const DevMesh& M, unsigned f0, unsigned f1, int nsm, cudaStream_t st);
void launch_plain_d4(const DevMesh& M, unsigned f0, unsigned f1, int nsm, cudaStream_t st);
void launch_plain_d5(const DevMesh& M, unsigned f0, unsigned f1, int nsm, cudaStream_t st);
void launch_plain_d6(const DevMesh& M, unsigned f0, unsigned f1, int nsm, cudaStream_t st);
void launch_fast_d2(const DevMesh& M, unsigned f0, unsigned f1, unsigned long long* fq, unsigned* nfq, unsigned fqcap, unsigned long long* fx, unsigned* nfx, unsigned fxcap, int nsm, cudaStream_t st);
void launch_fast_d3(const DevMesh& M, unsigned f0, unsigned f1, unsigned long long* fq, unsigned* nfq, unsigned fqcap, unsigned long long* fx, unsigned* nfx, unsigned fxcap, int nsm, cudaStream_t st);
void launch_fast_d4(const DevMesh& M, unsigned f0, unsigned f1, unsigned long long* fq, unsigned* nfq, unsigned fqcap, unsigned long long* fx, unsigned* nfx, unsigned fxcap, int nsm, cudaStream_t st);
void launch_fast_d5(const DevMesh& M, unsigned f0, unsigned f1, unsigned long long* fq, unsigned* nfq, unsigned fqcap, unsigned long long* fx, unsigned* nfx, unsigned fxcap, int nsm, cudaStream_t st);
void launch_fast_d6(const DevMesh& M, unsigned f0, unsigned f1, unsigned long long* fq, unsigned* nfq, unsigned fqcap, unsigned long long* fx, unsigned* nfx, unsigned fxcap, int nsm, cudaStream_t st);
void launch_fallback_warp_d2(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned fqcap, unsigned maxq, unsigned long long* fx, unsigned* nfx, unsigned fxcap, const AmbQueue& aq, int nsm, cudaStream_t st);
void launch_fallback_warp_d3(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned fqcap, unsigned maxq, unsigned long long* fx, unsigned* nfx, unsigned fxcap, const AmbQueue& aq, int nsm, cudaStream_t st);
void launch_fallback_warp_d4(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned fqcap, unsigned maxq, unsigned long long* fx, unsigned* nfx, unsigned fxcap, const AmbQueue& aq, int nsm, cudaStream_t st);
void launch_fallback_warp_d5(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned fqcap, unsigned maxq, unsigned long long* fx, unsigned* nfx, unsigned fxcap, const AmbQueue& aq, int nsm, cudaStream_t st);
void launch_fallback_warp_d6(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned fqcap, unsigned maxq, unsigned long long* fx, unsigned* nfx, unsigned fxcap, const AmbQueue& aq, int nsm, cudaStream_t st);
void launch_fallback_d2(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned maxq, int nsm, cudaStream_t st);
void launch_fallback_d3(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned maxq, int nsm, cudaStream_t st);
void launch_fallback_d4(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned maxq, int nsm, cudaStream_t st);
void launch_fallback_d5(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned maxq, int nsm, cudaStream_t st);
void launch_fallback_d6(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned maxq, int nsm, cudaStream_t st);

void launch_descent_exact_d2(const DevMesh& M, int maxn, unsigned long long seed, int* failed, unsigned* nfailed, int nsm, cudaStream_t st);
void launch_descent_exact_d3(const DevMesh& M, int maxn, unsigned long long seed, int* failed, unsigned* nfailed, int nsm, cudaStream_t st);
void launch_descent_exact_d4(const DevMesh& M, int maxn, unsigned long long seed, int* failed, unsigned* nfailed, int nsm, cudaStream_t st);
void launch_descent_exact_d5(const DevMesh& M, int maxn, unsigned long long seed, int* failed, unsigned* nfailed, int nsm, cudaStream_t st);
void launch_descent_exact_d6(const DevMesh& M, int maxn, unsigned long long seed, int* failed, unsigned* nfailed, int nsm, cudaStream_t st);

// Graph-driven levels: the start of a level clears the ray counters of its
// parity; the advance moves the frontier to the vertices found since, counts
// the level and keeps the loop running while a frontier or queued rays remain
// and no stop bit (capacity or a fatal error) is set.
__global__ void k_level_begin(DevMesh M) {
    if (threadIdx.x == 0) {
        const unsigned p = M.G.lvl[2] & 1u;
        M.G.qc[2 * p] = 0;
        M.G.qc[2 * p + 1] = 0;
    }
}

__global__ void k_level_advance(DevMesh M, cudaGraphConditionalHandle h, unsigned stop_bits) {
    if (threadIdx.x != 0) return;
    const unsigned L = M.G.lvl[2], p = L & 1u;
    const unsigned f1 = M.G.lvl[1];
    const unsigned e = min(*M.vcount, M.vcap);
    const bool queued = M.G.qc[2 * p] + M.G.qc[2 * p + 1] > 0;
    M.G.lvl[0] = f1;
    M.G.lvl[1] = e;
    M.G.lvl[2] = L + 1;
    const bool stop = (*M.status & stop_bits) != 0;
    cudaGraphSetConditional(h, (!stop && (e > f1 || queued)) ? 1u : 0u);
}

void launch_level_begin(const DevMesh& M, cudaStream_t st) { k_level_begin<<<1, 32, 0, st>>>(M); }
void launch_level_advance(const DevMesh& M, cudaGraphConditionalHandle h, unsigned stop_bits, cudaStream_t st) {
    k_level_advance<<<1, 32, 0, st>>>(M, h, stop_bits);
}

void launch_register_edges(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st) {
    switch (M.d) {
        case 2: launch_register_d2(M, v0, v1, nsm, st); break;
        case 3: launch_register_d3(M, v0, v1, nsm, st); break;
        case 4: launch_register_d4(M, v0, v1, nsm, st); break;
        case 5: launch_register_d5(M, v0, v1, nsm, st); break;
        case 6: launch_register_d6(M, v0, v1, nsm, st); break;
        default: break;
    }
}
void launch_refine_centers(const DevMesh& M, unsigned V, int nsm, cudaStream_t st) {
    switch (M.d) {
        case 2: launch_refine_d2(M, V, nsm, st); break;
        case 3: launch_refine_d3(M, V, nsm, st); break;
        case 4: launch_refine_d4(M, V, nsm, st); break;
        case 5: launch_refine_d5(M, V, nsm, st); break;
        case 6: launch_refine_d6(M, V, nsm, st); break;
        default: break;
    }
}
void launch_centers(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st) {
    switch (M.d) {
        case 2: launch_centers_d2(M, v0, v1, nsm, st); break;
        case 3: launch_centers_d3(M, v0, v1, nsm, st); break;
        case 4: launch_centers_d4(M, v0, v1, nsm, st); break;
        case 5: launch_centers_d5(M, v0, v1, nsm, st); break;
        case 6: launch_centers_d6(M, v0, v1, nsm, st); break;
        default: break;
    }
}
void launch_descent(const DevMesh& M, int stride, int nseeds, unsigned long long seed, int* failed, unsigned* nfailed, int nsm, cudaStream_t st) {
    switch (M.d) {
        case 2: launch_descent_d2(M, stride, nseeds, seed, failed, nfailed, nsm, st); break;
        case 3: launch_descent_d3(M, stride, nseeds, seed, failed, nfailed, nsm, st); break;
        case 4: launch_descent_d4(M, stride, nseeds, seed, failed, nfailed, nsm, st); break;
        case 5: launch_descent_d5(M, stride, nseeds, seed, failed, nfailed, nsm, st); break;
        case 6: launch_descent_d6(M, stride, nseeds, seed, failed, nfailed, nsm, st); break;
        default: break;
    }
}
void launch_expand_plain(const DevMesh& M, unsigned f0, unsigned f1, int nsm, cudaStream_t st) {
    switch (M.d) {
        case 2: launch_plain_d2(M, f0, f1, nsm, st); break;
        case 3: launch_plain_d3(M, f0, f1, nsm, st); break;
        case 4: launch_plain_d4(M, f0, f1, nsm, st); break;
        case 5: launch_plain_d5(M, f0, f1, nsm, st); break;
        case 6: launch_plain_d6(M, f0, f1, nsm, st); break;
        default: break;
    }
}
void launch_expand_fast(const DevMesh& M, unsigned f0, unsigned f1, unsigned long long* fq, unsigned* nfq, unsigned fqcap, unsigned long long* fx, unsigned* nfx, unsigned fxcap, int nsm, cudaStream_t st) {
    switch (M.d) {
        case 2: launch_fast_d2(M, f0, f1, fq, nfq, fqcap, fx, nfx, fxcap, nsm, st); break;
        case 3: launch_fast_d3(M, f0, f1, fq, nfq, fqcap, fx, nfx, fxcap, nsm, st); break;
        case 4: launch_fast_d4(M, f0, f1, fq, nfq, fqcap, fx, nfx, fxcap, nsm, st); break;
        case 5: launch_fast_d5(M, f0, f1, fq, nfq, fqcap, fx, nfx, fxcap, nsm, st); break;
        case 6: launch_fast_d6(M, f0, f1, fq, nfq, fqcap, fx, nfx, fxcap, nsm, st); break;
        default: break;
    }
}
void launch_fallback_warp(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned fqcap, unsigned maxq, unsigned long long* fx, unsigned* nfx, unsigned fxcap, const AmbQueue& aq, int nsm, cudaStream_t st) {
    switch (M.d) {
        case 2: launch_fallback_warp_d2(M, fq, nfq, fqcap, maxq, fx, nfx, fxcap, aq, nsm, st); break;
        case 3: launch_fallback_warp_d3(M, fq, nfq, fqcap, maxq, fx, nfx, fxcap, aq, nsm, st); break;
        case 4: launch_fallback_warp_d4(M, fq, nfq, fqcap, maxq, fx, nfx, fxcap, aq, nsm, st); break;
        case 5: launch_fallback_warp_d5(M, fq, nfq, fqcap, maxq, fx, nfx, fxcap, aq, nsm, st); break;
        case 6: launch_fallback_warp_d6(M, fq, nfq, fqcap, maxq, fx, nfx, fxcap, aq, nsm, st); break;
        default: break;
    }
}
void launch_fallback(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned maxq, int nsm, cudaStream_t st) {
    switch (M.d) {
        case 2: launch_fallback_d2(M, fq, nfq, maxq, nsm, st); break;
        case 3: launch_fallback_d3(M, fq, nfq, maxq, nsm, st); break;
        case 4: launch_fallback_d4(M, fq, nfq, maxq, nsm, st); break;
        case 5: launch_fallback_d5(M, fq, nfq, maxq, nsm, st); break;
        case 6: launch_fallback_d6(M, fq, nfq, maxq, nsm, st); break;
        default: break;
    }
}

void launch_descent_exact(const DevMesh& M, int maxn, unsigned long long seed, int* failed, unsigned* nfailed, int nsm, cudaStream_t st) {
    switch (M.d) {
        case 2: launch_descent_exact_d2(M, maxn, seed, failed, nfailed, nsm, st); break;
        case 3: launch_descent_exact_d3(M, maxn, seed, failed, nfailed, nsm, st); break;
        case 4: launch_descent_exact_d4(M, maxn, seed, failed, nfailed, nsm, st); break;
        case 5: launch_descent_exact_d5(M, maxn, seed, failed, nfailed, nsm, st); break;
        case 6: launch_descent_exact_d6(M, maxn, seed, failed, nfailed, nsm, st); break;
        default: break;
    }
}

}  // namespace hv
