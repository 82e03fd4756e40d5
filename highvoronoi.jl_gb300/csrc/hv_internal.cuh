// hv_internal.cuh -- device data layout and small numerical kernels shared by
// the libhvgpu translation units.
//
// Data layout in HBM (one mesh):
//   pts      n x d doubles, points in Morton order ("internal" ids)
//   pts32    n x DP floats (DP = 4 for d <= 4, 8 otherwise), same order
//   pts32lo  n x DP floats: x - (float)x (double-float coordinates)
//   perm     internal id -> original 0-based id
//   blo/bhi  (2P) x DP floats: boxes of an implicit complete binary tree over
//            leaves of `leaf` consecutive points (node 1 = root, leaves P..2P-1),
//            rounded outwards so that every box contains its FP64 points
//   knn/sec  n x K candidate lists (internal ids, nearest first) and the
//            radius below which a list is complete (FP32, rounded down)
//   vsig     vcap x (d+1) ints: sorted signature of each vertex; items >= n
//            are boundary planes n+p (p = 2k upper face, 2k+1 lower face)
//   vc       vcap x d doubles: FP64 circumcentre
//   vrho32   vcap x DP floats: rounded FP64 (centre - x_anchor), anchor = sig[0]
//   vinv32   vcap x d x d floats: rounded FP64 inverse of the vertex's constraint
//            matrix (columns give every ray direction of the vertex)
//   vnew     vcap ints: generator added by the ray that found the vertex
//   vhash    open-addressing table of 64-bit entries (fingerprint << 32 | id)
#pragma once
#include <type_traits>
#include <cuda_runtime.h>
#include <stdint.h>

#define HV_MAXD 6
#define HV_NAMB 8

namespace hv {

enum : unsigned {
    ST_VCAP = 1u,      // vertex capacity exceeded
    ST_HASH = 2u,      // hash table full
    ST_TIMEOUT = 4u,   // a bounded spin gave up
    ST_DEGEN = 8u,     // tie surviving double-double
    ST_BADINPUT = 16u, // point outside the open box / not finite
    ST_STACK = 32u,    // traversal stack overflow
    ST_QUEUE = 64u,    // fallback queue overflow
    ST_DESCENT = 128u, // no seed vertex found for a generator
    ST_NUMERIC = 256u, // singular vertex system / no candidate
    ST_AMB = 512u,     // more ambiguous candidates than HV_NAMB
    ST_ECAP = 1024u,   // edge table full
};

enum {
    C_RAYS = 0, C_FALLBACK, C_UNCERT, C_INSECURE, C_DD, C_DEGEN, C_DESCENT, C_DRETRY, C_EDGECLOSED,
    C_FBTREE, C_FBNODES, C_FBLEAVES, C_FBPOINTS, C_AMBSET, C_OWNED,
    C_NCOUNT
};

constexpr unsigned long long HASH_EMPTY = 0ull;
constexpr unsigned long long HASH_BUSY = ~0ull;
constexpr unsigned INVALID_ID = 0xFFFFFFFFu;
constexpr int SPIN_LIMIT = 1 << 22;

// A boundary plane {x : n.x = off} with outer unit normal n (the domain is n.x <= off).
// axis >= 0 marks n = sgn e_axis exactly (cuboid faces): those keep the exact
// single-coordinate arithmetic.
constexpr int HV_MAXP = 64;
struct DevPlane {
    double n[HV_MAXD];
    double off;
    float n32[HV_MAXD];
    float off32;
    int axis, sgn;
};

// Distance off - n.x of x below plane B (exact single subtraction for axis planes).
template <int D>
__device__ __forceinline__ double plane_height(const DevPlane& B, const double* x) {
    if (B.axis >= 0) return B.sgn > 0 ? B.off - x[B.axis] : B.off + x[B.axis];
    double h = B.off;
#pragma unroll
    for (int q = 0; q < D; ++q) h = fma(-B.n[q], x[q], h);
    return h;
}

struct DevBox {
    double lo[HV_MAXD], hi[HV_MAXD];
};

// The wavefront as one CUDA graph launch (a conditional WHILE node runs the
// levels): the frontier [lvl[0], lvl[1]) and the level index lvl[2] live in
// device memory, and the kernels pick the ray queues of a level by its parity
// (qc[2p], qc[2p+1]: queued and exact rays of parity p).  lvl == nullptr: the
// host drives the levels and passes ranges and queues as arguments.
struct LevelQueues {
    unsigned* lvl;
    unsigned long long* fq[2];
    unsigned long long* fx[2];
    float* fqh[2];
    unsigned* qc;
};

struct DevMesh {
    int d, n;
    LevelQueues G;
    // generators own0 .. own1-1 (internal order) belong to this mesh; a shard
    // of a mesh split over ranks walks only edges that keep one of them and
    // keeps the vertices whose smallest generator is one of them (0, n: all)
    int own0, own1;
    // refinement: only the generators with original id >= own_from are new;
    // the search walks only edges that keep one of them (-1: all generators)
    int own_from;
    int leaf, nleaves, P;
    int K, dp;
    unsigned vcap;
    unsigned long long vhmask;
    unsigned long long ehmask;
    double lo[HV_MAXD], hi[HV_MAXD];  // bounding box of the domain
    double xscale;  // bound on |coordinate|
    int np;                   // boundary planes, generator ids n .. n+np-1
    const DevPlane* planes;   // np entries
    int box;                  // planes are the cuboid faces 2k (x_k <= hi_k), 2k+1 (x_k >= lo_k)
    // FP32 copies for the FP32 kernels (rounded once on the host)
    float lo32[HV_MAXD], hi32[HV_MAXD];  // the cuboid's bounds when box
    float xs32;      // (float)xscale
    float tiny32;    // (float)(4e-14 xscale)
    float e13_32;    // (float)(1e-13 xscale)
    float e12_32;    // (float)(1e-12 xscale)
    float ulp32;     // (float)(xscale 2^-24)
    const double* pts;
    const float* pts32;
    const float* pts32lo;  // residual x - (float)x, so that x = hi + lo to ~2^-48
    const int* perm;
    const float* blo;
    const float* bhi;
    const int* knn;
    const float* sec;
    int* vsig;
    double* vc;
    float* vrho32;  // vcap x DP: FP32 (centre - anchor)
    float* vinv32;  // vcap x D x D: rounded FP64 inverse of the constraint matrix (row-major)
    float* vcond;   // vcap: condition estimate |M| |M^-1|
    int* vnew;
    unsigned* vcount;
    unsigned long long* vhash;
    unsigned long long* ehash;  // edge table: fingerprint << 32 | (vertex*8 + slot)
    unsigned* ecnt;             // per-vertex bit mask of edges found twice
    unsigned* status;
    unsigned long long* cnt;
    // rays the expansion decided, inserted by a separate kernel: (vertex << 3 | ray, winner)
    uint2* dq;
    unsigned* ndq;
    unsigned dqcap;
    // per queued insecure ray: the upper bound of the expansion's best candidate
    // (+inf if none), the fallback's starting bound instead of a second list pass
    float* fqh;
};

__device__ __forceinline__ void set_status(const DevMesh& M, unsigned bits) { atomicOr(M.status, bits); }

// Warp-aggregated counter increment.
__device__ __forceinline__ void count_add(unsigned long long* p, unsigned v = 1) {
    unsigned m = __activemask();
    unsigned tot = __reduce_add_sync(m, v);
    if ((threadIdx.x & 31) == (unsigned)(__ffs(m) - 1)) atomicAdd(p, (unsigned long long)tot);
}

// FNV-1a over the 32-bit items followed by the SplitMix64 finaliser.
__device__ __forceinline__ unsigned long long hash_items(const int* s, int len) {
    unsigned long long h = 1469598103934665603ull;
    for (int i = 0; i < len; ++i) { h ^= (unsigned)s[i]; h *= 1099511628211ull; }
    h ^= h >> 30; h *= 0xbf58476d1ce4e5b9ull;
    h ^= h >> 27; h *= 0x94d049bb133111ebull;
    h ^= h >> 31;
    return h;
}

// ---------------------------------------------------------------------------
// double-double arithmetic (Dekker 1971, Knuth TAOCP 4.2.2; two-product via FMA)
// ---------------------------------------------------------------------------
struct dd { double hi, lo; };

__device__ __forceinline__ dd dd_quick(double a, double b) { double s = a + b; return {s, b - (s - a)}; }
__device__ __forceinline__ dd dd_two_sum(double a, double b) {
    double s = a + b, bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ dd operator+(dd a, dd b) {
    dd s = dd_two_sum(a.hi, b.hi), t = dd_two_sum(a.lo, b.lo);
    s.lo += t.hi; s = dd_quick(s.hi, s.lo); s.lo += t.lo;
    return dd_quick(s.hi, s.lo);
}
__device__ __forceinline__ dd operator-(dd a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dd operator-(dd a, dd b) { return a + (-b); }
__device__ __forceinline__ dd operator*(dd a, dd b) {
    double p = a.hi * b.hi;
    double e = fma(a.hi, b.hi, -p);
    e = fma(a.hi, b.lo, e);
    e = fma(a.lo, b.hi, e);
    return dd_quick(p, e);
}
__device__ __forceinline__ dd operator/(dd a, dd b) {
    double q1 = a.hi / b.hi;
    dd r = a - b * dd{q1, 0.0};
    double q2 = r.hi / b.hi;
    r = r - b * dd{q2, 0.0};
    double q3 = r.hi / b.hi;
    return dd_quick(q1, q2) + dd{q3, 0.0};
}
__device__ __forceinline__ dd& operator+=(dd& a, dd b) { a = a + b; return a; }
__device__ __forceinline__ dd& operator-=(dd& a, dd b) { a = a - b; return a; }
__device__ __forceinline__ dd& operator/=(dd& a, dd b) { a = a / b; return a; }
__device__ __forceinline__ bool operator<(dd a, dd b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(dd a, dd b) { return b < a; }
__device__ __forceinline__ dd mk(double x) { return {x, 0.0}; }
__device__ __forceinline__ double tabs(double x) { return fabs(x); }
__device__ __forceinline__ float tabs(float x) { return fabsf(x); }
__device__ __forceinline__ bool is_zero(float x) { return x == 0.f; }
__device__ __forceinline__ dd tabs(dd x) { return x.hi < 0 ? -x : x; }
__device__ __forceinline__ bool is_zero(double x) { return x == 0.0; }
__device__ __forceinline__ bool is_zero(dd x) { return x.hi == 0.0; }
template <class T> __device__ __forceinline__ T from_d(double x);
template <> __device__ __forceinline__ double from_d<double>(double x) { return x; }
template <> __device__ __forceinline__ dd from_d<dd>(double x) { return mk(x); }
// exact difference of two doubles
template <class T> __device__ __forceinline__ T diff_d(double a, double b);
template <> __device__ __forceinline__ double diff_d<double>(double a, double b) { return a - b; }
template <> __device__ __forceinline__ dd diff_d<dd>(double a, double b) { return dd_two_sum(a, -b); }

// ---------------------------------------------------------------------------
// dense LU with partial pivoting, fully unrolled for compile-time D
// ---------------------------------------------------------------------------
template <int D, class T>
__device__ __forceinline__ bool lu_factor(T (&A)[D][D], int (&piv)[D]) {
#pragma unroll
    for (int c = 0; c < D; ++c) {
        int p = c;
        T best = tabs(A[c][c]);
#pragma unroll
        for (int r = c + 1; r < D; ++r) { T v = tabs(A[r][c]); if (v > best) { best = v; p = r; } }
        piv[c] = p;
        if (is_zero(best)) return false;
        if (p != c) {
#pragma unroll
            for (int k = 0; k < D; ++k) {
                // select-based swap keeps the arrays in registers
#pragma unroll
                for (int r = c + 1; r < D; ++r) {
                    if (r == p) { T t = A[c][k]; A[c][k] = A[r][k]; A[r][k] = t; }
                }
            }
        }
#pragma unroll
        for (int r = c + 1; r < D; ++r) {
            T f = A[r][c] / A[c][c];
            A[r][c] = f;
#pragma unroll
            for (int k = c + 1; k < D; ++k) A[r][k] -= f * A[c][k];
        }
    }
    return true;
}

template <int D, class T>
__device__ __forceinline__ void lu_solve(const T (&A)[D][D], const int (&piv)[D], T (&b)[D]) {
#pragma unroll
    for (int c = 0; c < D; ++c) {
#pragma unroll
        for (int r = c + 1; r < D; ++r) {
            if (piv[c] == r) { T t = b[c]; b[c] = b[r]; b[r] = t; }
        }
    }
#pragma unroll
    for (int r = 0; r < D; ++r) {
#pragma unroll
        for (int k = 0; k < r; ++k) b[r] -= A[r][k] * b[k];
    }
#pragma unroll
    for (int r = D - 1; r >= 0; --r) {
#pragma unroll
        for (int k = r + 1; k < D; ++k) b[r] -= A[r][k] * b[k];
        b[r] /= A[r][r];
    }
}

// off - n . xa in double-double (one rounding for the double result).
template <int D>
__device__ __forceinline__ dd plane_rhs_dd(const DevPlane& P, const double* xa) {
    dd s = mk(P.off);
#pragma unroll
    for (int q = 0; q < D; ++q) s = s - mk(P.n[q]) * mk(xa[q]);
    return s;
}
// For axis planes (n = +-e_k) the FMA chain adds exact zeros and rounds
// off -+ xa_k once, so it equals the double-double result rounded.
template <int D, class T>
__device__ __forceinline__ T plane_rhs(const DevPlane& P, const double* xa) {
    if constexpr (std::is_same<T, dd>::value) {
        return plane_rhs_dd<D>(P, xa);
    } else {
        if (P.axis >= 0) {
            double h = P.off;
#pragma unroll
            for (int q = 0; q < D; ++q) h = fma(-P.n[q], xa[q], h);
            return h;
        }
        const dd s = plane_rhs_dd<D>(P, xa);
        return s.hi + s.lo;
    }
}

// Constraint row of item `it` relative to the real anchor xa:
//   generator g : (x_g - x_a) . rho = |x_g - x_a|^2 / 2
//   plane p     : n_p . rho = off_p - n_p . x_a
template <int D, class T>
__device__ __forceinline__ void con_row(const DevMesh& M, const double* xa, int it, T (&row)[D], T& rhs) {
    if (it < M.n) {
        const double* xg = M.pts + (size_t)it * D;
        T s = from_d<T>(0.0);
#pragma unroll
        for (int k = 0; k < D; ++k) { row[k] = diff_d<T>(__ldg(xg + k), xa[k]); s += row[k] * row[k]; }
        rhs = s * from_d<T>(0.5);
    } else {
        // n . rho = off - n . xa: one rounding (exact for T = dd)
        const DevPlane& P = M.planes[it - M.n];
#pragma unroll
        for (int q = 0; q < D; ++q) row[q] = from_d<T>(P.n[q]);
        rhs = plane_rhs<D, T>(P, xa);
    }
}

// DP (4 or 8) floats from a 16-byte aligned address as float4 loads.
template <int DP>
__device__ __forceinline__ void load_f4(const float* p, float (&x)[DP]) {
    const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
    for (int h = 0; h < DP / 4; ++h) {
        const float4 f = __ldg(q + h);
        x[4 * h] = f.x; x[4 * h + 1] = f.y; x[4 * h + 2] = f.z; x[4 * h + 3] = f.w;
    }
}

// Insertion of `item` into a sorted signature with one slot removed.
template <int D>
__device__ __forceinline__ void make_sig(const int (&sig)[D + 1], int drop, int item, int (&out)[D + 1]) {
    int o = 0;
    bool placed = false;
#pragma unroll
    for (int s = 0; s <= D; ++s) {
        if (s == drop) continue;
        if (!placed && item < sig[s]) { out[o++] = item; placed = true; }
        out[o++] = sig[s];
    }
    if (!placed) out[D] = item;
}

}  // namespace hv
