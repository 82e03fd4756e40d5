// hv_polygeo.cuh -- FP64 geometry shared by the VI_POLYGON kernels (the
// per-facet face lattices of hv_poly.cu and the mesh-wide face lattice of
// hv_polylat.cu): the terms of the pulling decomposition
//     vol_m(G) = (1/m) * sum over the facets G' of G of dist(p_G, aff G') * vol_{m-1}(G').
#pragma once
#include "hv_internal.cuh"

namespace hv {

// Normal of generator g's bounding hyperplane relative to the point generator
// x0: x_g - x0 for a point (the bisector's normal), the plane's unit normal for
// a boundary plane (generator ids n + p).
template <int D>
__device__ __forceinline__ void gen_normal(int n, const double* pts, const DevPlane* planes, int g, const double* x0,
                                           double* nv) {
    if (g < n) {
#pragma unroll
        for (int q = 0; q < D; ++q) nv[q] = pts[(size_t)g * D + q] - x0[q];
    } else {
        const DevPlane& B = planes[g - n];
#pragma unroll
        for (int q = 0; q < D; ++q) nv[q] = B.n[q];
    }
}

// |(p - a) ^ (b - a)| = dist(p, line ab) * |b - a| (twice the triangle's area),
// by Lagrange's identity as the root of the sum of the squared 2x2 minors; each
// minor is formed with one rounding (FMA), so there is no cancellation beyond it.
template <int D>
__device__ __forceinline__ double tri_area2(const double* p, const double* a, const double* b) {
    double w[D], u[D];
#pragma unroll
    for (int q = 0; q < D; ++q) { w[q] = p[q] - a[q]; u[q] = b[q] - a[q]; }
    double s2 = 0;
#pragma unroll
    for (int x = 0; x < D; ++x)
#pragma unroll
        for (int y = x + 1; y < D; ++y) {
            const double m = fma(w[x], u[y], -(w[y] * u[x]));
            s2 = fma(m, m, s2);
        }
    return sqrt(s2);
}

// Orthonormal basis (modified Gram-Schmidt) of the normals of a face's
// defining generators; returns the count.
template <int D, int R>
__device__ __forceinline__ int mgs_add(double (&Q)[R][D], int m, const double* nv) {
    double r[D];
#pragma unroll
    for (int q = 0; q < D; ++q) r[q] = nv[q];
    for (int s = 0; s < m; ++s) {
        double dt = 0;
#pragma unroll
        for (int q = 0; q < D; ++q) dt = fma(Q[s][q], r[q], dt);
#pragma unroll
        for (int q = 0; q < D; ++q) r[q] = fma(-dt, Q[s][q], r[q]);
    }
    double nn = 0;
#pragma unroll
    for (int q = 0; q < D; ++q) nn = fma(r[q], r[q], nn);
    const double inv = rsqrt(nn);
#pragma unroll
    for (int q = 0; q < D; ++q) Q[m][q] = r[q] * inv;
    return m + 1;
}

// |n_x . (v - p)| / |component of n_x orthogonal to span(Q[0..m))|: the
// distance from p to the hyperplane of aff(parent) cut out by generator x
// (v: a point of that hyperplane inside the parent's affine hull).
template <int D, int R>
__device__ __forceinline__ double plane_dist(const double (&Q)[R][D], int m, const double* nx, const double* v,
                                             const double* p) {
    double r[D], num = 0;
#pragma unroll
    for (int q = 0; q < D; ++q) { r[q] = nx[q]; num = fma(nx[q], v[q] - p[q], num); }
    for (int s = 0; s < m; ++s) {
        double dt = 0;
#pragma unroll
        for (int q = 0; q < D; ++q) dt = fma(Q[s][q], r[q], dt);
#pragma unroll
        for (int q = 0; q < D; ++q) r[q] = fma(-dt, Q[s][q], r[q]);
    }
    double nn = 0;
#pragma unroll
    for (int q = 0; q < D; ++q) nn = fma(r[q], r[q], nn);
    return fabs(num) * rsqrt(nn);
}

}  // namespace hv
