// hv_periodic.cu -- periodic cuboids.
//
// The reference makes a cuboid periodic by mirroring the generators of the
// cells that touch a periodic face into the other side of the domain and
// searching the cells again (periodize!, Create_Discrete_Domain,
// src/domain.jl:139-213); the public view then names every mirrored
// generator by the original it copies (references / reference_shifts,
// src/voronoidata.jl:9-15,540-543).
//
// Here the extended generator set is built in one pass: every periodic image
// x + s*L (s in {-1,0,1} on the periodic axes, s != 0) that falls strictly
// inside the box widened by a margin delta on the periodic axes.  The mesh of
// the extended set in the widened box is computed by the ordinary search, and
// a vertex of an original cell is a vertex of the periodic tessellation when
// its circumsphere stays inside the widened box (every generator there is
// present) and none of its items is a widened face; otherwise the host widens
// the margin and searches again.  The public view then maps image ids to
// (original id, lattice shift): neighbour lists sorted by (id, shift), vertex
// signatures sorted by id, cell -> vertex lists, integrals gathered from the
// original cells.
#include "hv_internal.cuh"
#include "hv_periodic.h"

namespace hv {

namespace {

__host__ __device__ inline int pow3(int d) {
    int p = 1;
    for (int k = 0; k < d; ++k) p *= 3;
    return p;
}

// shift of axis k in the code c = sum (s_k + 1) 3^k
__device__ __forceinline__ int shift_of(int code, int k) {
    for (int q = 0; q < k; ++q) code /= 3;
    return code % 3 - 1;
}

// periodic image of x under shift code c, if it is a new point inside the widened box
template <int D>
__device__ __forceinline__ bool image_of(const PerBox& B, const double* x, int c, double* y) {
    int cc = c;
    bool moved = false;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const int s = cc % 3 - 1;
        cc /= 3;
        if (s != 0 && !((B.pmask >> k) & 1)) return false;
        moved |= s != 0;
        y[k] = x[k] + (double)s * B.L[k];
        if (s != 0 && !(y[k] > B.lo[k] - B.delta[k] && y[k] < B.hi[k] + B.delta[k])) return false;
    }
    return moved;
}

template <int D>
__global__ void k_img_count(const double* __restrict__ pts, int n, PerBox B, long long* cnt) {
    const int nc = pow3(D);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double x[D], y[D];
#pragma unroll
        for (int k = 0; k < D; ++k) x[k] = pts[(size_t)i * D + k];
        long long c = 0;
        for (int code = 0; code < nc; ++code) c += image_of<D>(B, x, code, y) ? 1 : 0;
        cnt[i] = c;
    }
}

template <int D>
__global__ void k_img_fill(const double* __restrict__ pts, int n, PerBox B, const long long* __restrict__ off,
                           double* ext, int* ref, short* icode) {
    const int nc = pow3(D);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double x[D], y[D];
#pragma unroll
        for (int k = 0; k < D; ++k) x[k] = pts[(size_t)i * D + k];
        long long o = off[i];
        for (int code = 0; code < nc; ++code) {
            if (!image_of<D>(B, x, code, y)) continue;
#pragma unroll
            for (int k = 0; k < D; ++k) ext[(size_t)(n + o) * D + k] = y[k];
            ref[o] = i;
            icode[o] = (short)code;
            ++o;
        }
    }
}

// original generators strictly inside the box
template <int D>
__global__ void k_in_box(const double* __restrict__ pts, int n, PerBox B, unsigned* bad) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        bool ok = true;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const double x = pts[(size_t)i * D + k];
            ok &= x > B.lo[k] && x < B.hi[k];
        }
        if (!ok) atomicOr(bad, 1u);
    }
}

// A vertex of an original cell is exact when its circumsphere lies inside the
// widened box on every periodic axis and it holds no widened face.  Rows of
// osig: off (a CSR, vertices of any number of generators) or d+1 wide.
template <int D>
__global__ void k_per_validate(const long long* __restrict__ off, const int* __restrict__ osig,
                               const double* __restrict__ oc, unsigned V, int n, int n_ext,
                               const double* __restrict__ ext, PerBox B, unsigned* bad) {
    for (unsigned v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        const long long s0 = off ? off[v] : (long long)v * (D + 1);
        const int m = off ? (int)(off[v + 1] - s0) : D + 1;
        const int* s = osig + s0;
        if (s[0] >= n) continue;  // sorted: s[0] is the smallest item
        bool ok = true;
        for (int k = 0; k < m; ++k) {
            const int it = s[k];
            if (it >= n_ext && ((B.pmask >> ((it - n_ext) >> 1)) & 1)) ok = false;
        }
        double r2 = 0, c[D];
#pragma unroll
        for (int k = 0; k < D; ++k) {
            c[k] = oc[(size_t)v * D + k];
            const double e = c[k] - ext[(size_t)s[0] * D + k];
            r2 = fma(e, e, r2);
        }
        const double R = sqrt(r2) * (1.0 + 1e-12) + 1e-12 * B.scale;
#pragma unroll
        for (int k = 0; k < D; ++k)
            if ((B.pmask >> k) & 1)
                if (!(c[k] - R > B.lo[k] - B.delta[k] && c[k] + R < B.hi[k] + B.delta[k])) ok = false;
        if (!ok) atomicAdd(bad, 1u);
    }
}

// public id and shift code of an extended item
__device__ __forceinline__ void map_item(int e, int n, int n_ext, const int* ref, const short* icode, int center,
                                         int& id, int& code) {
    if (e < n) { id = e; code = center; }
    else if (e < n_ext) { id = ref[e - n]; code = icode[e - n]; }
    else { id = n + (e - n_ext); code = center; }
}

// flag[v] = 1 for the vertices of original cells; len[v] their signature
// length (0 for the others), so that a scan of len places the public rows
template <int D>
__global__ void k_pub_flag(const long long* __restrict__ off, const int* __restrict__ osig, unsigned V, int n,
                           long long* flag, long long* len) {
    for (unsigned v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        const long long s0 = off ? off[v] : (long long)v * (D + 1);
        const bool pub = osig[s0] < n;
        flag[v] = pub ? 1 : 0;
        if (len) len[v] = pub ? (off ? off[v + 1] - s0 : D + 1) : 0;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        flag[V] = 0;
        if (len) len[V] = 0;
    }
}

constexpr int PUB_MAXSIG = 64;  // generators of one vertex

template <int D>
__global__ void k_pub_fill(const long long* __restrict__ off, const int* __restrict__ osig,
                           const double* __restrict__ oc, unsigned V, int n, int n_ext, const int* __restrict__ ref,
                           const short* __restrict__ icode, const long long* __restrict__ pos,
                           const long long* __restrict__ rowpos, long long* poff, int* psig, double* pc,
                           int* ext2pub) {
    const int center = (pow3(D) - 1) / 2;
    for (unsigned v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        const long long s0 = off ? off[v] : (long long)v * (D + 1);
        const int m = off ? (int)(off[v + 1] - s0) : D + 1;
        const int* s = osig + s0;
        if (s[0] >= n) { ext2pub[v] = -1; continue; }
        const long long p = pos[v];
        ext2pub[v] = (int)p;
        const long long dst = rowpos ? rowpos[v] : p * (D + 1);
        if (poff) poff[p] = dst;
        int mm[PUB_MAXSIG];
        const int mc = m < PUB_MAXSIG ? m : PUB_MAXSIG;
        for (int k = 0; k < mc; ++k) {
            int code, id;
            map_item(s[k], n, n_ext, ref, icode, center, id, code);
            int b = k;
            while (b > 0 && mm[b - 1] > id) { mm[b] = mm[b - 1]; --b; }
            mm[b] = id;
        }
        for (int k = 0; k < mc; ++k) psig[dst + k] = mm[k];
#pragma unroll
        for (int k = 0; k < D; ++k) pc[(size_t)p * D + k] = oc[(size_t)v * D + k];
    }
}

// Row i of the public neighbour list: the extended row i mapped to (id, shift)
// and sorted by (id, shift code); perm records the extended position.
template <int D>
__global__ void k_pub_nbr(int n, int n_ext, const long long* __restrict__ off, const int* __restrict__ nbr,
                          const int* __restrict__ ref, const short* __restrict__ icode, int* pnbr, signed char* pshift,
                          int* perm) {
    const int center = (pow3(D) - 1) / 2;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const long long b = off[i], e = off[i + 1];
        for (long long t = b; t < e; ++t) {  // insertion of entry t into the sorted prefix [b, t)
            int id, code;
            map_item(nbr[t], n, n_ext, ref, icode, center, id, code);
            const unsigned long long key = ((unsigned long long)(unsigned)id << 16) | (unsigned)code;
            // keys of the sorted prefix are rebuilt from the stored (id, shift) pairs
            long long u = t;
            while (u > b) {
                int pc = 0;
#pragma unroll
                for (int k = D - 1; k >= 0; --k) pc = pc * 3 + (pshift[(size_t)(u - 1) * D + k] + 1);
                const unsigned long long kp = ((unsigned long long)(unsigned)pnbr[u - 1] << 16) | (unsigned)pc;
                if (kp <= key) break;
                pnbr[u] = pnbr[u - 1];
                perm[u] = perm[u - 1];
#pragma unroll
                for (int k = 0; k < D; ++k) pshift[(size_t)u * D + k] = pshift[(size_t)(u - 1) * D + k];
                --u;
            }
            pnbr[u] = id;
            perm[u] = (int)(t - b);
#pragma unroll
            for (int k = 0; k < D; ++k) pshift[(size_t)u * D + k] = (signed char)shift_of(code, k);
        }
    }
}

__global__ void k_pub_inc(long long total, const int* __restrict__ inc, const int* __restrict__ ext2pub, int* pinc) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x)
        pinc[t] = ext2pub[inc[t]];
}

__global__ void k_pub_area(int n, const long long* __restrict__ off, const int* __restrict__ perm,
                           const double* __restrict__ ext_area, double* area) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (long long t = off[i]; t < off[i + 1]; ++t) area[t] = ext_area[off[i] + perm[t]];
}

unsigned grid_of(long long n, int bs) {
    long long g = (n + bs - 1) / bs;
    if (g < 1) g = 1;
    if (g > 65535) g = 65535;
    return (unsigned)g;
}

}  // namespace

#define HV_DISPATCH(d, CALL)                           \
    switch (d) {                                       \
        case 2: { constexpr int DD = 2; CALL; } break; \
        case 3: { constexpr int DD = 3; CALL; } break; \
        case 4: { constexpr int DD = 4; CALL; } break; \
        case 5: { constexpr int DD = 5; CALL; } break; \
        case 6: { constexpr int DD = 6; CALL; } break; \
        default: break;                                \
    }

void launch_in_box(const PerBox& B, const double* pts, int n, unsigned* bad, cudaStream_t st) {
    if (n <= 0) return;
    HV_DISPATCH(B.d, (k_in_box<DD><<<grid_of(n, 256), 256, 0, st>>>(pts, n, B, bad)));
}
void launch_img_count(const PerBox& B, const double* pts, int n, long long* cnt, cudaStream_t st) {
    if (n <= 0) return;
    HV_DISPATCH(B.d, (k_img_count<DD><<<grid_of(n, 128), 128, 0, st>>>(pts, n, B, cnt)));
}
void launch_img_fill(const PerBox& B, const double* pts, int n, const long long* off, double* ext, int* ref,
                     short* icode, cudaStream_t st) {
    if (n <= 0) return;
    HV_DISPATCH(B.d, (k_img_fill<DD><<<grid_of(n, 128), 128, 0, st>>>(pts, n, B, off, ext, ref, icode)));
}
void launch_per_validate(const PerBox& B, const long long* off, const int* osig, const double* oc, unsigned V,
                         int n, int n_ext, const double* ext, unsigned* bad, cudaStream_t st) {
    if (!V) return;
    HV_DISPATCH(B.d, (k_per_validate<DD><<<grid_of(V, 256), 256, 0, st>>>(off, osig, oc, V, n, n_ext, ext, B, bad)));
}
void launch_pub_flag(int d, const long long* off, const int* osig, unsigned V, int n, long long* flag,
                     long long* len, cudaStream_t st) {
    HV_DISPATCH(d, (k_pub_flag<DD><<<grid_of(V, 256), 256, 0, st>>>(off, osig, V, n, flag, len)));
}
void launch_pub_fill(int d, const long long* off, const int* osig, const double* oc, unsigned V, int n, int n_ext,
                     const int* ref, const short* icode, const long long* pos, const long long* rowpos,
                     long long* poff, int* psig, double* pc, int* ext2pub, cudaStream_t st) {
    if (!V) return;
    HV_DISPATCH(d, (k_pub_fill<DD><<<grid_of(V, 256), 256, 0, st>>>(off, osig, oc, V, n, n_ext, ref, icode, pos,
                                                                      rowpos, poff, psig, pc, ext2pub)));
}
void launch_pub_nbr(int d, int n, int n_ext, const long long* off, const int* nbr, const int* ref, const short* icode,
                    int* pnbr, signed char* pshift, int* perm, cudaStream_t st) {
    if (n <= 0) return;
    HV_DISPATCH(d, (k_pub_nbr<DD><<<grid_of(n, 128), 128, 0, st>>>(n, n_ext, off, nbr, ref, icode, pnbr, pshift,
                                                                     perm)));
}
void launch_pub_inc(long long total, const int* inc, const int* ext2pub, int* pinc, cudaStream_t st) {
    if (total <= 0) return;
    k_pub_inc<<<grid_of(total, 256), 256, 0, st>>>(total, inc, ext2pub, pinc);
}
void launch_pub_area(int n, const long long* off, const int* perm, const double* ext_area, double* area,
                     cudaStream_t st) {
    if (n <= 0) return;
    k_pub_area<<<grid_of(n, 128), 128, 0, st>>>(n, off, perm, ext_area, area);
}

}  // namespace hv
