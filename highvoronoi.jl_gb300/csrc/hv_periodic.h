// hv_periodic.h -- launchers of the periodic-cuboid kernels (hv_periodic.cu).
#pragma once
#include <cuda_runtime.h>

#include "hv_internal.cuh"

namespace hv {

// The cuboid [lo, hi] with side lengths L, periodic axes pmask (bit k), and
// the image margin delta per axis (0 on the other axes).
struct PerBox {
    int d;
    int pmask;
    double lo[HV_MAXD], hi[HV_MAXD], L[HV_MAXD], delta[HV_MAXD];
    double scale;  // max |coordinate| of the widened box
};

void launch_in_box(const PerBox& B, const double* pts, int n, unsigned* bad, cudaStream_t st);
void launch_img_count(const PerBox& B, const double* pts, int n, long long* cnt, cudaStream_t st);
// images after the n originals in ext ((n + nimg) x d), with their original and shift code
void launch_img_fill(const PerBox& B, const double* pts, int n, const long long* off, double* ext, int* ref,
                     short* icode, cudaStream_t st);
void launch_per_validate(const PerBox& B, const int* osig, const double* oc, unsigned V, int n, int n_ext,
                         const double* ext, unsigned* bad, cudaStream_t st);
void launch_pub_flag(int d, const int* osig, unsigned V, int n, long long* flag, cudaStream_t st);
void launch_pub_fill(int d, const int* osig, const double* oc, unsigned V, int n, int n_ext, const int* ref,
                     const short* icode, const long long* pos, int* psig, double* pc, int* ext2pub, cudaStream_t st);
void launch_pub_nbr(int d, int n, int n_ext, const long long* off, const int* nbr, const int* ref, const short* icode,
                    int* pnbr, signed char* pshift, int* perm, cudaStream_t st);
void launch_pub_inc(long long total, const int* inc, const int* ext2pub, int* pinc, cudaStream_t st);
void launch_pub_area(int n, const long long* off, const int* perm, const double* ext_area, double* area,
                     cudaStream_t st);

}  // namespace hv
