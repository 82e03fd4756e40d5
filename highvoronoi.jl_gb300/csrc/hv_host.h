// hv_host.h -- launchers shared between the libhvgpu translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace hv {
struct DevMesh;
struct DevPlane;

// Rays whose FP32 decision left a small ambiguous candidate set: the queue
// entry (vertex << 4 | flags | slot), the set size and up to AMB_SET ids each.
constexpr int AMB_SET = 32;
struct AmbQueue {
    unsigned long long* e;
    int* n;
    int* ids;
    unsigned* count;
    unsigned cap;
};


// hv_prep.cu
// hv_domain.cu: boundary planes (cuboid faces 2k upper, 2k+1 lower; or from
// base points and normals, normals scaled to unit length) and the domain's
// bounding box; the strings are empty on success, else the error text.
void box_planes(int d, const double* lo, const double* hi, DevPlane* out);
std::string make_planes(int d, int np, const double* base, const double* normal, DevPlane* out);
std::string planes_bbox(int d, int np, const DevPlane* P, double* lo, double* hi);

int morton_bits(int d, int n);  // bits per axis of the Morton codes (the sort reads d times as many)
void launch_morton(int d, const double* in, int n, const double* lo, const double* hi, const DevPlane* planes,
                   int np, unsigned long long* codes, int* idx, unsigned* status, cudaStream_t st);
void launch_gather(int d, const double* in, const int* perm, int n, double* pts, float* pts32, float* pts32lo,
                   cudaStream_t st);
void launch_bvh(const DevMesh& M, float* blo, float* bhi, unsigned* flags, cudaStream_t st);
// candidate lists: part 0 the generators 0, qs, 2 qs, ... (descent seeds), part 1 the rest (qs <= 1: all)
void launch_knn(const DevMesh& M, int* knn, float* sec, int qs, int part, cudaStream_t st);
size_t sort_pairs_u64_i32_temp(int n);
void sort_pairs_u64_i32(void* temp, size_t temp_bytes, const unsigned long long* kin, unsigned long long* kout,
                        const int* vin, int* vout, int n, int end_bit, cudaStream_t st);
size_t sort_pairs_u32_i32_temp(int n);
void sort_pairs_u32_i32(void* temp, size_t temp_bytes, const unsigned* kin, unsigned* kout, const int* vin,
                        int* vout, int n, int end_bit, cudaStream_t st);
size_t sort_keys_u64_temp(long long n);
void sort_keys_u64(void* temp, size_t temp_bytes, const unsigned long long* kin, unsigned long long* kout,
                   long long n, cudaStream_t st);
size_t scan_temp(int n);
void exclusive_scan_i64(void* temp, size_t temp_bytes, const long long* in, long long* out, int n, cudaStream_t st);

// hv_search.cu
void launch_descent(const DevMesh& M, int stride, int nseeds, unsigned long long seed, int* failed,
                    unsigned* nfailed, int nsm, cudaStream_t st);
void launch_descent_exact(const DevMesh& M, int maxn, unsigned long long seed, int* failed, unsigned* nfailed,
                          int nsm, cudaStream_t st);
void launch_centers(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st);
// residual correction of the ill-conditioned centres after the search (fast method)
void launch_refine_centers(const DevMesh& M, unsigned V, int nsm, cudaStream_t st);
void launch_register_edges(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st);
void launch_level_begin(const DevMesh& M, cudaStream_t st);
void launch_level_advance(const DevMesh& M, cudaGraphConditionalHandle h, unsigned stop_bits, cudaStream_t st);
void launch_expand_plain(const DevMesh& M, unsigned f0, unsigned f1, int nsm, cudaStream_t st);
void launch_expand_fast(const DevMesh& M, unsigned f0, unsigned f1, unsigned long long* fq, unsigned* nfq,
                        unsigned fqcap, unsigned long long* fx, unsigned* nfx, unsigned fxcap, int nsm,
                        cudaStream_t st);
// FP32 warp tree search of the queued rays, then the FP64 decision of their
// ambiguous candidate sets (queued in aq); the rest goes to fx.
void launch_fallback_warp(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned fqcap,
                          unsigned maxq, unsigned long long* fx, unsigned* nfx, unsigned fxcap, const AmbQueue& aq,
                          int nsm, cudaStream_t st);
void launch_fallback(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned maxq, int nsm,
                     cudaStream_t st);

// hv_post.cu
// canonical keys: original 0-based items of each vertex, sorted, SoA by position
// incremental refinement: keep[v] = 1 unless a new point lies strictly inside
// old vertex v's circumsphere (uncertain: within the rounding margin), then
// the merge of the kept old rows (plane items renumbered) with the new rows
void launch_refine_keep(int d, int n_old, int k, unsigned V, const int* osig, const double* oc, const double* pts,
                        const double* newp, long long* keep, unsigned* uncertain, cudaStream_t st);
void launch_refine_merge(int d, int n_old, int k, unsigned V_old, const int* osig, const double* oc,
                         const long long* keep, const long long* rank, unsigned V_new, const int* nsig,
                         const double* nc, int* out_sig, double* out_c, cudaStream_t st);
void launch_canon_keys(const DevMesh& M, unsigned V, unsigned* keys, cudaStream_t st);
void launch_gather_keys(const unsigned* keys_pos, const int* order, unsigned V, unsigned* out, cudaStream_t st);
void launch_pack_keys(const unsigned* keys, unsigned V, int d, int bits, unsigned long long* out, cudaStream_t st);
void launch_fix_runs(const unsigned long long* sk, const unsigned* last, unsigned V, int* order, cudaStream_t st);
void launch_canon_gather(const DevMesh& M, unsigned V, const unsigned* keys, const int* order, int* osig,
                         double* oc, cudaStream_t st);
void launch_inc_pairs(int d, int n, unsigned V, const int* osig, unsigned long long* pairs, long long* cnt,
                      cudaStream_t st);
void launch_inc_split(unsigned long long npairs, const unsigned long long* pairs, int* inc, cudaStream_t st);
void launch_nbr_count(int d, int n, const long long* inc_off, const int* inc, const int* osig, long long* nnbr,
                      unsigned* status, cudaStream_t st);
void launch_nbr_fill(int d, int n, const long long* inc_off, const int* inc, const int* osig,
                     const long long* nbr_off, int* nbr, cudaStream_t st);
void launch_out_vertices(int d, unsigned V, const int* osig, int64_t* sig_out, cudaStream_t st);
void launch_out_nbr(long long total, const int* nbr, int64_t* out, cudaStream_t st);
}  // namespace hv
