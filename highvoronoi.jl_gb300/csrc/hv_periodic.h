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
// Rows of osig: off (a CSR, vertices of any number of generators) or d+1 wide
// when off is null.
void launch_per_validate(const PerBox& B, const long long* off, const int* osig, const double* oc, unsigned V,
                         int n, int n_ext, const double* ext, unsigned* bad, cudaStream_t st);
// flag (V+1): vertices of original cells; len (V+1, may be null): their lengths
void launch_pub_flag(int d, const long long* off, const int* osig, unsigned V, int n, long long* flag,
                     long long* len, cudaStream_t st);
// public rows: vertex pos[v], items at rowpos[v] (scan of len; null: d+1 wide),
// poff[pos[v]] = rowpos[v] when poff is not null
void launch_pub_fill(int d, const long long* off, const int* osig, const double* oc, unsigned V, int n, int n_ext,
                     const int* ref, const short* icode, const long long* pos, const long long* rowpos,
                     long long* poff, int* psig, double* pc, int* ext2pub, cudaStream_t st);
void launch_pub_nbr(int d, int n, int n_ext, const long long* off, const int* nbr, const int* ref, const short* icode,
                    int* pnbr, signed char* pshift, int* perm, cudaStream_t st);
void launch_pub_inc(long long total, const int* inc, const int* ext2pub, int* pinc, cudaStream_t st);
void launch_pub_area(int n, const long long* off, const int* perm, const double* ext_area, double* area,
                     cudaStream_t st);

}  // namespace hv
