// hv_search_d6.cu -- vertex search kernels instantiated for d = 6.
#include "hv_search_impl.cuh"

namespace hv {

void launch_register_d6(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st) { launch_register_t<6>(M, v0, v1, nsm, st); }
void launch_centers_d6(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st) { launch_centers_t<6>(M, v0, v1, nsm, st); }
void launch_refine_d6(const DevMesh& M, unsigned V, int nsm, cudaStream_t st) { launch_refine_t<6>(M, V, nsm, st); }
void launch_descent_d6(const DevMesh& M, int stride, int nseeds, unsigned long long seed, int* failed,                              unsigned* nfailed, int nsm, cudaStream_t st) { launch_descent_t<6>(M, stride, nseeds, seed, failed, nfailed, nsm, st); }
void launch_plain_d6(const DevMesh& M, unsigned f0, unsigned f1, int nsm, cudaStream_t st) { launch_plain_t<6>(M, f0, f1, nsm, st); }
void launch_fast_d6(const DevMesh& M, unsigned f0, unsigned f1, unsigned long long* fq, unsigned* nfq,                           unsigned fqcap, unsigned long long* fx, unsigned* nfx, unsigned fxcap, int nsm,                           cudaStream_t st) { launch_fast_t<6>(M, f0, f1, fq, nfq, fqcap, fx, nfx, fxcap, nsm, st); }
void launch_fallback_warp_d6(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq,                                    unsigned fqcap, unsigned maxq, unsigned long long* fx, unsigned* nfx,                                    unsigned fxcap, const AmbQueue& aq, int nsm, cudaStream_t st) { launch_fallback_warp_t<6>(M, fq, nfq, fqcap, maxq, fx, nfx, fxcap, aq, nsm, st); }
void launch_fallback_d6(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned maxq,                               int nsm, cudaStream_t st) { launch_fallback_t<6>(M, fq, nfq, maxq, nsm, st); }
void launch_descent_exact_d6(const DevMesh& M, int maxn, unsigned long long seed, int* failed, unsigned* nfailed, int nsm, cudaStream_t st) { launch_descent_exact_t<6>(M, maxn, seed, failed, nfailed, nsm, st); }

}  // namespace hv
