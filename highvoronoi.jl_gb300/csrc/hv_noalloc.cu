// hv_noalloc.cu -- heuristic Monte-Carlo integration that allocates nothing.
//
// For callers that cannot allocate device memory (an embedding application
// that owns the whole device memory budget, a real-time loop that forbids
// allocator calls, or code handed fixed buffers by a framework).  The caller
// passes every input and output in device memory; the integrator's scratch
// (raw per-cell volumes and variances, raw interface areas, the cuboid's
// box planes, a status word) lives in one file-scope static device array of HV_NOALLOC_SCRATCH_BYTES
// (16 MiB), which every GPU that loads this library holds until exit.  The
// domain is the cuboid [lo, hi]: its 2d faces are the planes n .. n+2d-1 in
// the order of hv_mesh_build (n+2k: x_k = hi_k, n+2k+1: x_k = lo_k).
//
// The array's name is only a host-side stand-in for the symbol, so its device
// address is fetched once per device with cudaGetSymbolAddress (at the first
// call on that device, with that device current) and passed to the kernels.
// All calls share the array: calls that overlap on the GPU race on it, and each
// call clears the status word it reads back.  No cudaMalloc, cudaFree or
// allocating library routine is called here.
#include <cmath>
#include <mutex>

#include <cuda_runtime.h>

#include "hv_host.h"
#include "hv_integrate.h"
#include "hv_internal.cuh"
#include "hvgpu.h"

namespace {

constexpr size_t kScratchBytes = HV_NOALLOC_SCRATCH_BYTES;
constexpr size_t kStatusBytes = 256;
constexpr size_t kPlaneBytes = 2 * HV_MAXD * sizeof(hv::DevPlane) + 256 - (2 * HV_MAXD * sizeof(hv::DevPlane)) % 256;
constexpr int kMaxDevices = 64;
static_assert(kStatusBytes + kPlaneBytes == HV_NOALLOC_FIXED_BYTES, "fixed part of the scratch layout");

static __device__ __align__(256) unsigned char g_mc_scratch[kScratchBytes];

std::mutex g_mu;
void* g_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set up once).
int scratch_address(int dev, unsigned char** out) {
    if (dev < 0 || dev >= kMaxDevices) return HV_E_CUDA;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_mc_scratch) != cudaSuccess || !p) return HV_E_CUDA;
        g_addr[dev] = p;
    }
    *out = (unsigned char*)g_addr[dev];
    return HV_OK;
}

}  // namespace

extern "C" int hv_integrate_heuristic_mc_noalloc(int d, int64_t n, const double* d_pts, const double* lo,
                                                 const double* hi, const int64_t* d_nbr_off, const int32_t* d_nbr,
                                                 int64_t nnbr, int max_degree, int ndir, uint64_t seed,
                                                 double* d_vol, double* d_area, void* stream) {
    if (d < 2 || d > 6 || n <= 0 || nnbr < 0 || ndir <= 0 || max_degree <= 0 || !d_pts || !lo || !hi ||
        !d_nbr_off || (nnbr > 0 && (!d_nbr || !d_area)) || !d_vol)
        return HV_E_INVALID_ARG;
    for (int k = 0; k < d; ++k)
        if (!(lo[k] < hi[k])) return HV_E_INVALID_ARG;
    // scratch: status | planes | raw volume (n) | variance (n) | raw area (nnbr), in doubles
    const double need = (double)(kStatusBytes + kPlaneBytes) + 8.0 * (2.0 * (double)n + (double)nnbr);
    if (need > (double)kScratchBytes) return HV_E_CAPACITY;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return HV_E_CUDA;
    unsigned char* base = nullptr;
    int rc = scratch_address(dev, &base);
    if (rc != HV_OK) return rc;
    int nsm = 1, smax = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const int capN = (max_degree + 7) / 8 * 8;
    const size_t sm = hv::mc_smem_bytes(d, capN);
    if ((long long)sm > smax) return HV_E_CAPACITY;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned* status = (unsigned*)base;
    hv::DevPlane* planes = (hv::DevPlane*)(base + kStatusBytes);
    double* rawV = (double*)(base + kStatusBytes + kPlaneBytes);
    double* varV = rawV + n;
    double* rawA = varV + n;
    if (cudaMemsetAsync(status, 0, sizeof(unsigned), st) != cudaSuccess) return HV_E_CUDA;
    hv::DevPlane hp[2 * HV_MAXD];
    hv::box_planes(d, lo, hi, hp);
    // pageable source: the copy has read hp when the call returns
    if (cudaMemcpyAsync(planes, hp, sizeof(hv::DevPlane) * 2 * d, cudaMemcpyHostToDevice, st) != cudaSuccess)
        return HV_E_CUDA;
    hv::IntegrateInput in{d, (int)n, lo, hi, 2 * d, planes, d_pts, nullptr, nullptr, nullptr, nullptr,
                          (const long long*)d_nbr_off, d_nbr, status};
    const double cvol = std::pow(M_PI, d / 2.0) / std::tgamma(1.0 + d / 2.0);  // unit-ball volume
    if (hv::launch_heuristic_mc(in, ndir, seed, capN, cvol, rawV, rawA, varV, d_area, d_vol, nsm, st) != 0)
        return HV_E_CUDA;
    if (cudaGetLastError() != cudaSuccess) return HV_E_CUDA;
    unsigned hs = 0;
    if (cudaMemcpyAsync(&hs, status, sizeof(unsigned), cudaMemcpyDeviceToHost, st) != cudaSuccess) return HV_E_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return HV_E_CUDA;
    // 4: a row longer than max_degree; 8: an item outside 0 .. n+2d-1 (or a cell
    // listing itself); 16: a row k that does not list i although row i lists k
    return hs ? HV_E_INVALID_ARG : HV_OK;
}
