// hv_poly.cu -- VI_POLYGON on the GPU: interface areas A_ik and cell volumes.
//
// The reference (src/polyintegrator.jl:174-468) cuts the cone over facet k of
// cell i into flag simplices (x_i, c_F, c(L_1), ..., v1, v2) and sums
// |det| / d!.  The volume of such a simplex is the product of its successive
// heights / d!, so the flag sum is the recursion
//     vol_m(G) = (1/m) * sum over the facets G' of G of dist(p_G, aff G') * vol_{m-1}(G')
// evaluated over the face lattice of the facet, with the same value for any
// reference point p_G in G.  This file takes p_G = the first vertex of G
// (a pulling decomposition): every term is non-negative, terms of sub-faces
// through p_G vanish and are skipped, and each (face, sub-face) pair costs a
// few FP64 dot products instead of the (d-2)! determinants per edge of the
// flag form -- FP64 is the scarce unit on this GPU.  A_ik = vol_{d-1}(F),
// V_i = sum_k A_ik h_ik / d (src/polyintegrator.jl:308-316); every facet is
// computed by its lower cell and copied to the higher one
// (src/cleanup_cell.jl:174-204).
//
// Data flow:
//   1. facet -> vertex CSR over the neighbour slots t of the lower cells
//      (count, scan, fill; each facet's list is sorted in the facet kernel);
//   2. one group (a warp, or NW warps) per facet builds the face lattice from
//      sorts of packed keys -- no hash tables, no atomics on values, fixed
//      summation order, so results are bitwise reproducible;
//   3. facets beyond the shared-memory capacity are redone by block groups
//      with 64-bit keys in global-memory work areas;
//   4. volumes.
//
// Face encoding (B bits per field): a facet vertex has d-1 "items" (its
// generators other than i and k), numbered 0..ni-1 in generator order.  A
// face of level j is a set T of j items (its vertices are those whose items
// contain T); its code is T[0] at level 1 and (index of T minus its largest
// item at level j-1) << B | max(T) above, so codes of a level sort and search
// as plain integers.  Level d-2 faces are the facet's edges.
#include <algorithm>
#include <vector>

#include "hv_integrate.h"
#include "hv_internal.cuh"
#include "hv_polygeo.cuh"

namespace hv {

template <class K> struct KeyBits;
template <> struct KeyBits<unsigned> { static constexpr int B = 10; };
template <> struct KeyBits<unsigned long long> { static constexpr int B = 20; };

struct PolyIn {
    int n;
    const DevPlane* planes;   // boundary planes, generator ids n + p
    const double* pts;        // n x d, original order
    const int* osig;          // V x (d+1), sorted 0-based items, planes n+p
    const double* oc;         // V x d
    const long long* nbr_off;
    const int* nbr;
    const long long* foff;    // facet slot -> range of fvert
    const unsigned* fvert;    // facet vertex ids (unsorted within a facet)
    const int* slot_cell;     // slot -> cell
    double* area;             // aligned with nbr
    unsigned* status;         // 1: capacity (tier B), 8: facet not simple
};

struct FCaps {
    int capV, capI, capB, capF;  // vertices (pow2), items, sort buffer (pow2), faces of all levels
    int capT;                    // edge-term slots (groups of more than one warp; 0 for one warp)
};

template <int D>
__host__ __device__ constexpr int binom(int n, int k) {
    int r = 1;
    for (int q = 0; q < k; ++q) r = r * (n - q) / (q + 1);
    return r;
}

template <int D, class K>
__host__ __device__ inline size_t farea_bytes(const FCaps& c) {
    constexpr int DM = D > 1 ? D - 1 : 1;
    size_t b = 0;
    b += 8 * (size_t)c.capF;          // fvol
    b += 8 * (size_t)c.capT;          // dterm
    b += 8 * 16;                      // dred + ll
    b += sizeof(K) * (size_t)c.capB;  // buf
    b += sizeof(K) * 2 * (size_t)c.capF;  // fcode, faux
    b += 4 * (size_t)c.capV;          // fv
    b += 4 * (size_t)c.capV * DM;     // vit
    b += 4 * (size_t)c.capI;          // its
    b += 4 * ((size_t)c.capF + 1);    // seg
    b += 4 * 16;                      // wsum
    b += (size_t)c.capF;              // fneed
    return (b + 255) / 256 * 256;
}

template <int D, class K>
struct FArea {
    double* fvol; double* dterm; double* dred; long long* ll; K* buf; K* fcode; K* faux;
    unsigned* fv; unsigned* vit; unsigned* its; unsigned* seg; int* wsum; unsigned char* fneed;
    __device__ FArea(unsigned char* base, const FCaps& c) {
        constexpr int DM = D > 1 ? D - 1 : 1;
        fvol = (double*)base;
        dterm = fvol + c.capF;
        dred = dterm + c.capT;
        ll = (long long*)(dred + 8);
        buf = (K*)(ll + 8);
        fcode = buf + c.capB;
        faux = fcode + c.capF;
        fv = (unsigned*)(faux + c.capF);
        vit = fv + c.capV;
        its = vit + (size_t)c.capV * DM;
        seg = its + c.capI;
        wsum = (int*)(seg + c.capF + 1);
        fneed = (unsigned char*)(wsum + 16);
    }
};

// A group of NW warps working on one facet.  NW > 1 uses named barrier
// 1 + gid (several groups may share a block).
template <int NW>
struct Grp {
    int rank, gid;
    static constexpr int size = NW * 32;
    __device__ Grp(int r, int g) : rank(r), gid(g) {}
    __device__ __forceinline__ void sync() const {
        if (NW == 1) __syncwarp();
        else asm volatile("bar.sync %0, %1;" ::"r"(1 + gid), "r"(NW * 32) : "memory");
    }
};

template <int NW, class K>
__device__ void g_sort(K* a, int n2, const Grp<NW>& g) {
    g.sync();
    for (int k = 2; k <= n2; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int q = g.rank; q < (n2 >> 1); q += g.size) {
                const int x = ((q & ~(j - 1)) << 1) | (q & (j - 1));
                const int y = x | j;
                const K p = a[x], r = a[y];
                const bool up = (x & k) == 0;
                if ((p > r) == up) { a[x] = r; a[y] = p; }
            }
            g.sync();
        }
}

// Stream compaction over x < n: write(x, rank of x among the kept) for
// every x with pred(x); returns the count (same value in every thread).
template <int NW, class P, class Wr>
__device__ int g_compact(const Grp<NW>& g, int n, P pred, Wr write, int* wsum) {
    int total = 0;
    const int lane = g.rank & 31, w = g.rank >> 5;
    for (int base = 0; base < n; base += g.size) {
        const int x = base + g.rank;
        const bool p = x < n && pred(x);
        const unsigned bal = __ballot_sync(0xFFFFFFFFu, p);
        const int lt = __popc(bal & ((1u << lane) - 1u));
        if (NW == 1) {
            if (p) write(x, total + lt);
            total += __popc(bal);
        } else {
            if (lane == 0) wsum[w] = __popc(bal);
            g.sync();
            int off = 0, tot = 0;
            for (int q = 0; q < NW; ++q) {
                const int c = wsum[q];
                if (q < w) off += c;
                tot += c;
            }
            if (p) write(x, total + off + lt);
            total += tot;
            g.sync();
        }
    }
    g.sync();
    return total;
}

// Fixed-order group sum (bitwise reproducible).
template <int NW>
__device__ double g_sum(const Grp<NW>& g, double v, double* dred) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, off);
    if (NW == 1) return v;
    if ((g.rank & 31) == 0) dred[g.rank >> 5] = v;
    g.sync();
    double s = 0;
    for (int q = 0; q < NW; ++q) s += dred[q];
    g.sync();
    return s;
}

template <int NW>
__device__ int g_or(const Grp<NW>& g, int v, int* wsum) {
    g.sync();  // also orders the group's preceding writes
    v = __any_sync(0xFFFFFFFFu, v != 0);
    if (NW == 1) return v;
    if ((g.rank & 31) == 0) wsum[g.rank >> 5] = v;
    g.sync();
    int r = 0;
    for (int q = 0; q < NW; ++q) r |= wsum[q];
    g.sync();
    return r;
}

__device__ __forceinline__ int pow2_ge(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

template <class K>
__device__ __forceinline__ int lower_bound_k(const K* a, int n, K key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int md = (lo + hi) >> 1;
        if (a[md] < key) lo = md + 1; else hi = md;
    }
    return lo;
}

template <int D>
__device__ __forceinline__ void normal_of(const PolyIn& P, int g, const double* xi, double* nv) {
    if (g < P.n) {
#pragma unroll
        for (int q = 0; q < D; ++q) nv[q] = P.pts[(size_t)g * D + q] - xi[q];
    } else {
        const DevPlane& B = P.planes[g - P.n];
#pragma unroll
        for (int q = 0; q < D; ++q) nv[q] = B.n[q];
    }
}

template <int D>
__device__ __forceinline__ void vload(const PolyIn& P, unsigned v, double* x) {
#pragma unroll
    for (int q = 0; q < D; ++q) x[q] = P.oc[(size_t)v * D + q];
}

enum { F_OK = 0, F_CAP = 1, F_BAD = 2 };

// The face lattice and area of facet (i, k) at slot t.  All control flow
// depends on group-uniform values only.
template <int D, int NW, class K>
__device__ int poly_facet(const PolyIn& P, int i, int k, long long t, const FArea<D, K>& W, const FCaps& c,
                          const Grp<NW>& g, double& area) {
    constexpr int B = KeyBits<K>::B;
    constexpr int DM = D > 1 ? D - 1 : 1;
    constexpr unsigned MASK = (1u << B) - 1u;
    const K SENT = ~(K)0;
    const long long f0 = P.foff[t];
    const int nv = (int)(P.foff[t + 1] - f0);
    area = 0.0;
    if (nv < 2) return F_OK;
    if (D == 2) {
        if (nv != 2) return F_BAD;
        double a[D], b[D];
        vload<D>(P, P.fvert[f0], a);
        vload<D>(P, P.fvert[f0 + 1], b);
        double s = 0;
#pragma unroll
        for (int q = 0; q < D; ++q) s = fma(a[q] - b[q], a[q] - b[q], s);
        area = sqrt(s);
        return F_OK;
    }
    if (nv > c.capV || nv > (int)MASK) return F_CAP;
    double xi[D];
#pragma unroll
    for (int q = 0; q < D; ++q) xi[q] = P.pts[(size_t)i * D + q];
    // ---- facet vertices in id order
    {
        const int n2 = pow2_ge(nv);
        for (int a = g.rank; a < n2; a += g.size) W.fv[a] = a < nv ? P.fvert[f0 + a] : 0xFFFFFFFFu;
        g.sync();
        g_sort<NW, unsigned>(W.fv, n2, g);
    }
    // ---- items
    int ni;
    {
        const int n1 = nv * DM, n2 = pow2_ge(n1);
        if (n2 > c.capB) return F_CAP;
        int bad = 0;
        for (int a = g.rank; a < nv; a += g.size) {
            const unsigned v = W.fv[a];
            int w = 0;
#pragma unroll
            for (int q = 0; q <= D; ++q) {
                const int it = P.osig[(size_t)v * (D + 1) + q];
                if (it != i && it != k) {
                    if (w < DM) W.buf[a * DM + w] = (K)(unsigned)it;
                    ++w;
                }
            }
            bad |= (w != DM);
        }
        for (int x = n1 + g.rank; x < n2; x += g.size) W.buf[x] = SENT;
        if (g_or(g, bad, W.wsum)) return F_BAD;
        g_sort<NW, K>(W.buf, n2, g);
        const K* bb = W.buf;
        unsigned* its = W.its;
        const int capI = c.capI;
        ni = g_compact(g, n1, [&](int x) { return x == 0 || bb[x] != bb[x - 1]; },
                       [&](int x, int pos) { if (pos < capI) its[pos] = (unsigned)bb[x]; }, W.wsum);
        if (ni > c.capI || ni > (int)MASK) return F_CAP;
        for (int a = g.rank; a < nv; a += g.size) {
            const unsigned v = W.fv[a];
            unsigned loc[DM];
            int w = 0;
#pragma unroll
            for (int q = 0; q <= D; ++q) {
                const int it = P.osig[(size_t)v * (D + 1) + q];
                if (it == i || it == k || w >= DM) continue;
                loc[w++] = (unsigned)lower_bound_k<unsigned>(W.its, ni, (unsigned)it);
            }
            for (int x = 1; x < DM; ++x)
                for (int y = x; y > 0 && loc[y] < loc[y - 1]; --y) { const unsigned z = loc[y]; loc[y] = loc[y - 1]; loc[y - 1] = z; }
#pragma unroll
            for (int x = 0; x < DM; ++x) W.vit[a * DM + x] = loc[x];
        }
        g.sync();
    }
    // ---- levels 1..D-2 of the face lattice
    int off[D], nf[D];
    off[1] = 0;
    // code of the sorted item tuple T at level l (lookups in the levels below)
    auto code_of = [&](const unsigned* T, int l, K& code) -> bool {
        K cc = T[0];
        for (int q = 1; q < l; ++q) {
            int idx = (int)cc;
            if (q > 1) {
                idx = lower_bound_k<K>(W.fcode + off[q], nf[q], cc);
                if (idx >= nf[q] || W.fcode[off[q] + idx] != cc) return false;
            }
            cc = ((K)idx << B) | (K)T[q];
        }
        code = cc;
        return true;
    };
    auto items_of = [&](int l, int f, unsigned* T) {
        K cc = W.fcode[off[l] + f];
        for (int q = l; q >= 2; --q) {
            T[q - 1] = (unsigned)(cc & (K)MASK);
            cc = W.fcode[off[q - 1] + (int)(cc >> B)];
        }
        T[0] = (unsigned)cc;
    };
    for (int j = 1; j <= D - 2; ++j) {
        const int cnt = binom<D>(DM, j);
        const int np = nv * cnt, n2 = pow2_ge(np);
        if (n2 > c.capB) return F_CAP;
        int bad = 0;
        for (int a = g.rank; a < nv; a += g.size) {
            const unsigned* li = W.vit + a * DM;
            int r = 0;
            for (unsigned sub = 1; sub < (1u << DM); ++sub) {
                if (__popc(sub) != j) continue;
                unsigned T[DM];
                int m = 0;
                for (int x = 0; x < DM; ++x) if ((sub >> x) & 1u) T[m++] = li[x];
                K code = 0;
                if (!code_of(T, j, code)) bad = 1;
                W.buf[a * cnt + r++] = (code << B) | (K)a;
            }
        }
        for (int x = np + g.rank; x < n2; x += g.size) W.buf[x] = SENT;
        if (g_or(g, bad, W.wsum)) return F_BAD;
        g_sort<NW, K>(W.buf, n2, g);
        const K* bb = W.buf;
        unsigned* seg = W.seg;
        const int room = c.capF - off[j];
        const int m = g_compact(g, np, [&](int x) { return x == 0 || (bb[x] >> B) != (bb[x - 1] >> B); },
                                [&](int x, int pos) { if (pos < room) seg[pos] = (unsigned)x; }, W.wsum);
        if (m > room || m > (int)MASK) return F_CAP;
        nf[j] = m;
        if (g.rank == 0) W.seg[m] = (unsigned)np;
        g.sync();
        bad = 0;
        for (int s = g.rank; s < m; s += g.size) {
            const int x0 = (int)W.seg[s], x1 = (int)W.seg[s + 1];
            const K a = W.buf[x0] & (K)MASK;
            W.fcode[off[j] + s] = W.buf[x0] >> B;
            if (j == D - 2) {  // an edge: exactly two vertices in a simple facet
                if (x1 - x0 != 2) { bad = 1; continue; }
                const K b = W.buf[x0 + 1] & (K)MASK;
                W.faux[off[j] + s] = a | (b << B);
                W.fvol[off[j] + s] = 0.0;  // edge terms use |(p - a) ^ (b - a)| directly
            } else {
                W.faux[off[j] + s] = a;
                W.fvol[off[j] + s] = 0.0;
            }
        }
        if (g_or(g, bad, W.wsum)) return F_BAD;
        if (j + 1 < D) off[j + 1] = off[j] + m;
    }
    // ---- faces whose volume is used: the level-1 faces off facet vertex 0, then
    // every sub-face of a used face that misses that face's reference vertex
    if (D >= 4) {
        for (int f = g.rank; f < nf[1]; f += g.size) {
            bool through = false;
#pragma unroll
            for (int x = 0; x < DM; ++x) through |= (W.vit[x] == (unsigned)f);
            W.fneed[off[1] + f] = through ? 0 : 1;
        }
        g.sync();
        int bad = 0;
        for (int j = 1; j <= D - 3; ++j) {
            for (int ch = g.rank; ch < nf[j + 1]; ch += g.size) {
                unsigned T[DM];
                items_of(j + 1, ch, T);
                const K cc = W.fcode[off[j + 1] + ch];
                unsigned char nd = 0;
                for (int q = 0; q <= j && !nd; ++q) {
                    int pidx;
                    if (q == j) {
                        pidx = (int)(cc >> B);
                    } else {
                        unsigned Pt[DM];
                        int w = 0;
                        for (int x = 0; x <= j; ++x) if (x != q) Pt[w++] = T[x];
                        K pc = 0;
                        if (!code_of(Pt, j, pc)) { bad = 1; break; }
                        if (j == 1) pidx = (int)pc;
                        else {
                            pidx = lower_bound_k<K>(W.fcode + off[j], nf[j], pc);
                            if (pidx >= nf[j] || W.fcode[off[j] + pidx] != pc) { bad = 1; break; }
                        }
                    }
                    if (!W.fneed[off[j] + pidx]) continue;
                    const unsigned rep = (unsigned)W.faux[off[j] + pidx];
                    bool through = false;
#pragma unroll
                    for (int x = 0; x < DM; ++x) through |= (W.vit[rep * DM + x] == T[q]);
                    if (!through) nd = 1;
                }
                W.fneed[off[j + 1] + ch] = nd;
            }
            g.sync();
        }
        if (g_or(g, bad, W.wsum)) return F_BAD;
    }
    // ---- volumes of the used faces, bottom-up (levels D-3 .. 1)
    for (int j = D - 3; j >= 1; --j) {
        const int nc = nf[j + 1], mm = j + 1;
        const int np = nc * mm, n2 = pow2_ge(np);
        if (n2 > c.capB) return F_CAP;
        int bad = 0;
        for (int ch = g.rank; ch < nc; ch += g.size) {
            unsigned T[DM];
            items_of(j + 1, ch, T);
            const K cc = W.fcode[off[j + 1] + ch];
            for (int q = 0; q <= j; ++q) {
                int pidx;
                if (q == j) {
                    pidx = (int)(cc >> B);
                } else {
                    unsigned Pt[DM];
                    int w = 0;
                    for (int x = 0; x <= j; ++x) if (x != q) Pt[w++] = T[x];
                    K pc = 0;
                    if (!code_of(Pt, j, pc)) { bad = 1; pidx = 0; }
                    else if (j == 1) pidx = (int)pc;
                    else {
                        pidx = lower_bound_k<K>(W.fcode + off[j], nf[j], pc);
                        if (pidx >= nf[j] || W.fcode[off[j] + pidx] != pc) { bad = 1; pidx = 0; }
                    }
                }
                // skip unused parents and sub-faces through the parent's reference vertex
                const unsigned rep = (unsigned)W.faux[off[j] + pidx];
                bool through = !W.fneed[off[j] + pidx];
#pragma unroll
                for (int x = 0; x < DM; ++x) through |= (W.vit[rep * DM + x] == T[q]);
                W.buf[ch * mm + q] = through ? SENT : (((K)pidx << B) | (K)ch);
            }
        }
        for (int x = np + g.rank; x < n2; x += g.size) W.buf[x] = SENT;
        if (g_or(g, bad, W.wsum)) return F_BAD;
        g_sort<NW, K>(W.buf, n2, g);
        const K* bb = W.buf;
        unsigned* seg = W.seg;
        const int room = c.capF + 1;
        const int m = g_compact(g, np, [&](int x) { return bb[x] != SENT && (x == 0 || (bb[x] >> B) != (bb[x - 1] >> B)); },
                                [&](int x, int pos) { if (pos < room) seg[pos] = (unsigned)x; }, W.wsum);
        if (m > room) return F_CAP;
        if (j + 1 == D - 2) {
            // edge children: one term per lane over the whole sorted pair list (the
            // terms of a parent vary 1..6 in number), then each parent's sum in order
            const int nvalid = g_compact(g, np, [&](int x) { return bb[x] != SENT; }, [&](int, int) {}, W.wsum);
            auto edge_term = [&](int x, int& pidx) -> double {
                pidx = (int)(W.buf[x] >> B);
                const int ch = (int)(W.buf[x] & (K)MASK);
                double p[D], va[D], vb[D];
                vload<D>(P, W.fv[(int)W.faux[off[j] + pidx]], p);
                const K ab = W.faux[off[j + 1] + ch];
                vload<D>(P, W.fv[(int)(ab & (K)MASK)], va);
                vload<D>(P, W.fv[(int)(ab >> B)], vb);
                return tri_area2<D>(p, va, vb);
            };
            if (NW == 1) {
                // one warp: segmented scan of each 32-pair chunk, the last lane of a
                // parent's run adds the chunk's partial (chunks in order)
                const int lane = g.rank;
                for (int f = lane; f < nf[j]; f += 32) W.fvol[off[j] + f] = 0.0;
                __syncwarp();
                for (int base = 0; base < nvalid; base += 32) {
                    const int x = base + lane;
                    int key = -1 - lane;
                    double v = 0.0;
                    if (x < nvalid) v = edge_term(x, key);
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const double vu = __shfl_up_sync(0xFFFFFFFFu, v, o);
                        const int ku = __shfl_up_sync(0xFFFFFFFFu, key, o);
                        if (lane >= o && ku == key) v += vu;
                    }
                    const int kn = __shfl_down_sync(0xFFFFFFFFu, key, 1);
                    if (x < nvalid && (lane == 31 || kn != key)) W.fvol[off[j] + key] += v;
                    __syncwarp();
                }
                for (int f = lane; f < nf[j]; f += 32) W.fvol[off[j] + f] /= (double)(D - 1 - j);
                __syncwarp();
            } else {
                if (nvalid > c.capT) return F_CAP;
                for (int x = g.rank; x < nvalid; x += g.size) {
                    int pidx;
                    W.dterm[x] = edge_term(x, pidx);
                }
                g.sync();
                for (int s = g.rank; s < m; s += g.size) {
                    int x = (int)W.seg[s];
                    const int pidx = (int)(W.buf[x] >> B);
                    double sum = 0.0;
                    for (; x < nvalid && (int)(W.buf[x] >> B) == pidx; ++x) sum += W.dterm[x];
                    W.fvol[off[j] + pidx] = sum / (double)(D - 1 - j);
                }
                g.sync();
            }
            continue;
        }
        for (int s = g.rank; s < m; s += g.size) {
            int x = (int)W.seg[s];
            const int pidx = (int)(W.buf[x] >> B);
            unsigned Pt[DM];
            items_of(j, pidx, Pt);
            double p[D];
            vload<D>(P, W.fv[(int)W.faux[off[j] + pidx]], p);
            double Q[D][D];
            int qm = 0;
            if (j + 1 < D - 2) {
                double nv_[D];
                normal_of<D>(P, k, xi, nv_);
                qm = mgs_add<D>(Q, qm, nv_);
                for (int q = 0; q < j; ++q) {
                    normal_of<D>(P, (int)W.its[Pt[q]], xi, nv_);
                    qm = mgs_add<D>(Q, qm, nv_);
                }
            }
            double sum = 0.0;
            for (; x < n2 && W.buf[x] != SENT && (int)(W.buf[x] >> B) == pidx; ++x) {
                const int ch = (int)(W.buf[x] & (K)MASK);
                double h, cv;
                if (j + 1 == D - 2) {  // an edge: height times length in one
                    const K ab = W.faux[off[j + 1] + ch];
                    double va[D], vb[D];
                    vload<D>(P, W.fv[(int)(ab & (K)MASK)], va);
                    vload<D>(P, W.fv[(int)(ab >> B)], vb);
                    h = tri_area2<D>(p, va, vb);
                    cv = 1.0;
                } else {
                    unsigned T[DM];
                    items_of(j + 1, ch, T);
                    unsigned xit = T[j];
                    for (int q = 0; q <= j; ++q) {
                        bool inP = false;
                        for (int r = 0; r < j; ++r) inP |= (Pt[r] == T[q]);
                        if (!inP) { xit = T[q]; break; }
                    }
                    double nx[D], vc[D];
                    normal_of<D>(P, (int)W.its[xit], xi, nx);
                    vload<D>(P, W.fv[(int)W.faux[off[j + 1] + ch]], vc);
                    h = plane_dist<D>(Q, qm, nx, vc, p);
                    cv = W.fvol[off[j + 1] + ch];
                }
                sum += h * cv;
            }
            W.fvol[off[j] + pidx] = sum / (double)(D - 1 - j);
        }
        g.sync();
    }
    // ---- the facet: reference vertex = facet vertex 0, children = level-1 faces
    double p[D];
    vload<D>(P, W.fv[0], p);
    double Q[D][D];
    int qm = 0;
    if (D > 3) {
        double nv_[D];
        normal_of<D>(P, k, xi, nv_);
        qm = mgs_add<D>(Q, qm, nv_);
    }
    double part = 0.0;
    for (int f = g.rank; f < nf[1]; f += g.size) {
        bool through = false;
#pragma unroll
        for (int x = 0; x < DM; ++x) through |= (W.vit[x] == (unsigned)f);
        if (through) continue;
        if (D == 3) {  // edges: height times length in one
            const K ab = W.faux[off[1] + f];
            double va[D], vb[D];
            vload<D>(P, W.fv[(int)(ab & (K)MASK)], va);
            vload<D>(P, W.fv[(int)(ab >> B)], vb);
            part += tri_area2<D>(p, va, vb);
        } else {
            double nx[D], vc[D];
            normal_of<D>(P, (int)W.its[f], xi, nx);
            vload<D>(P, W.fv[(int)W.faux[off[1] + f]], vc);
            part += plane_dist<D>(Q, qm, nx, vc, p) * W.fvol[off[1] + f];
        }
    }
    area = g_sum(g, part, W.dred) / (double)(D - 1);
    return F_OK;
}

template <int D>
__device__ __forceinline__ void write_area(const PolyIn& P, int i, int k, long long t, double ar) {
    P.area[t] = ar;
    if (k < P.n) {
        long long lo = P.nbr_off[k], hi = P.nbr_off[k + 1] - 1;
        while (lo < hi) { const long long md = (lo + hi) >> 1; if (P.nbr[md] < i) lo = md + 1; else hi = md; }
        if (P.nbr[lo] == i) P.area[lo] = ar;
    }
}

template <int NW>
__device__ __forceinline__ long long g_claim(const Grp<NW>& g, unsigned long long* next, long long* ll) {
    long long t = 0;
    if (g.rank == 0) t = (long long)atomicAdd(next, 1ull);
    if (NW == 1) return __shfl_sync(0xFFFFFFFFu, t, 0);
    if (g.rank == 0) ll[0] = t;
    g.sync();
    t = ll[0];
    g.sync();
    return t;
}

// Tier A: GPB groups of NW warps per block, 32-bit keys, shared-memory work
// areas.  Facets over the caps are listed in `big`.
template <int D, int NW, int GPB>
__global__ void __launch_bounds__(NW * 32 * GPB) k_poly_facets(PolyIn P, FCaps c, long long nslots,
                                                               unsigned long long* next, long long* big,
                                                               unsigned* nbig, unsigned* maxnv) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int gib = threadIdx.x / (NW * 32);
    const Grp<NW> g(threadIdx.x % (NW * 32), gib);
    const FArea<D, unsigned> W(smem + (size_t)gib * farea_bytes<D, unsigned>(c), c);
    for (;;) {
        const long long t = g_claim(g, next, W.ll + 1);
        if (t >= nslots) break;
        const long long nvl = P.foff[t + 1] - P.foff[t];
        if (nvl == 0) continue;  // slots of the higher cell
        const int i = P.slot_cell[t], k = P.nbr[t];
        double ar = 0.0;
        const int r = poly_facet<D, NW, unsigned>(P, i, k, t, W, c, g, ar);
        if (g.rank == 0) {
            if (r == F_OK) write_area<D>(P, i, k, t, ar);
            else if (r == F_CAP) {
                big[atomicAdd(nbig, 1u)] = t;
                atomicMax(maxnv, (unsigned)nvl);
            } else {
                atomicOr(P.status, 8u);
            }
        }
        g.sync();
    }
}

// Tier B: one group of NW warps per block, 64-bit keys, over a list of facets.
// SMEM: work area in shared memory; facets over its caps go to `out`.
// Otherwise: one global-memory work area per block; over the caps is fatal.
template <int D, int NW, bool SMEM>
__global__ void __launch_bounds__(NW * 32) k_poly_big(PolyIn P, FCaps c, const long long* in, long long nin,
                                                      unsigned long long* next, unsigned char* slab, long long* out,
                                                      unsigned* nout, unsigned* maxnv) {
    extern __shared__ __align__(16) unsigned char smem[];
    const Grp<NW> g(threadIdx.x, 0);
    unsigned char* base = SMEM ? smem : slab + (size_t)blockIdx.x * farea_bytes<D, unsigned long long>(c);
    const FArea<D, unsigned long long> W(base, c);
    for (;;) {
        const long long f = g_claim(g, next, W.ll + 1);
        if (f >= nin) break;
        const long long t = in[f];
        const int i = P.slot_cell[t], k = P.nbr[t];
        double ar = 0.0;
        const int r = poly_facet<D, NW, unsigned long long>(P, i, k, t, W, c, g, ar);
        if (g.rank == 0) {
            if (r == F_OK) write_area<D>(P, i, k, t, ar);
            else if (r == F_CAP && SMEM) {
                out[atomicAdd(nout, 1u)] = t;
                atomicMax(maxnv, (unsigned)(P.foff[t + 1] - P.foff[t]));
            } else {
                atomicOr(P.status, r == F_CAP ? 1u : 8u);
            }
        }
        g.sync();
    }
}

// facet -> vertex incidences: vertex v with sorted generators s_0 < ... < s_d
// lies on facet (s_a, s_b) for every a < b with s_a a cell; the facet is the
// neighbour slot of s_b in the list of s_a.
template <int D, bool FILL>
__global__ void k_facet_incidence(int n, unsigned V, const int* __restrict__ osig, const long long* __restrict__ nbr_off,
                                  const int* __restrict__ nbr, unsigned long long* cnt, const long long* foff,
                                  unsigned* fvert) {
    for (unsigned v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        int s[D + 1];
#pragma unroll
        for (int q = 0; q <= D; ++q) s[q] = osig[(size_t)v * (D + 1) + q];
#pragma unroll
        for (int a = 0; a < D; ++a) {
            if (s[a] >= n) break;
            long long lo = nbr_off[s[a]];
            const long long end = nbr_off[s[a] + 1];
#pragma unroll
            for (int b = a + 1; b <= D; ++b) {
                long long l = lo, h = end;
                while (l < h) { const long long md = (l + h) >> 1; if (nbr[md] < s[b]) l = md + 1; else h = md; }
                if (l < end && nbr[l] == s[b]) {
                    const unsigned long long p = atomicAdd(cnt + l, 1ull);
                    if (FILL) fvert[foff[l] + (long long)p] = v;
                    lo = l + 1;
                }
            }
        }
    }
}

__global__ void k_slot_cell(int n, const long long* nbr_off, int* slot_cell) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (long long t = nbr_off[i]; t < nbr_off[i + 1]; ++t) slot_cell[t] = i;
}

template <int D>
__global__ void k_cell_volumes(PolyIn P, double* vol) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x) {
        double xi[D];
#pragma unroll
        for (int q = 0; q < D; ++q) xi[q] = P.pts[(size_t)i * D + q];
        double v = 0;
        for (long long t = P.nbr_off[i]; t < P.nbr_off[i + 1]; ++t) {
            const int k = P.nbr[t];
            double h;
            if (k >= P.n) {
                h = plane_height<D>(P.planes[k - P.n], xi);
            } else {
                double s2 = 0;
#pragma unroll
                for (int q = 0; q < D; ++q) { const double e = P.pts[(size_t)k * D + q] - xi[q]; s2 = fma(e, e, s2); }
                h = 0.5 * sqrt(s2);
            }
            v += P.area[t] * h / D;
        }
        vol[i] = v;
    }
}

// ---------------------------------------------------------------------------
// host side
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

static int grid_of(unsigned long long n, int bs) {
    unsigned long long g = (n + bs - 1) / bs;
    return (int)std::max(1ull, std::min(g, 1ull << 20));
}

// faces of all levels per facet vertex (upper bound used for the caps) and
// sort-buffer entries per vertex
static void face_mults(int d, int& fmul, int& bmul) {
    static const int fm[7] = {0, 0, 1, 2, 3, 4, 7};
    static const int bm[7] = {0, 0, 1, 2, 3, 6, 10};
    fmul = fm[d];
    bmul = bm[d];
}

static FCaps caps_for(int d, int capV, int widen) {
    int fmul, bmul;
    face_mults(d, fmul, bmul);
    FCaps c;
    c.capV = capV;
    c.capI = std::max(32, capV * widen);
    long long b = 1;
    while (b < (long long)capV * bmul * widen) b <<= 1;
    c.capB = (int)std::max(64ll, b);
    c.capF = std::max(32, capV * fmul * widen);
    c.capT = c.capB;
    return c;
}

template <int D>
struct TierA {
    static constexpr int NW = D == 6 ? 4 : 1;
    static constexpr int GPB = D == 6 ? 2 : 4;
};

template <int D>
static size_t bytes_a(FCaps c) {
    if (TierA<D>::NW == 1) c.capT = 0;
    return farea_bytes<D, unsigned>(c);
}
template <int D>
static size_t bytes_b(const FCaps& c) { return farea_bytes<D, unsigned long long>(c); }

template <int D>
static int poly_run(const PolyRun& R) {
    PolyIn P;
    P.n = R.n;
    P.planes = R.planes;
    P.pts = R.pts; P.osig = R.osig; P.oc = R.oc; P.nbr_off = R.nbr_off; P.nbr = R.nbr;
    P.foff = R.foff; P.fvert = R.fvert; P.slot_cell = R.slot_cell; P.area = R.area; P.status = R.status;
    cudaStream_t st = R.stream;
    if (R.pass == 0) {  // incidence count
        k_facet_incidence<D, false><<<grid_of(R.V, 256), 256, 0, st>>>(R.n, R.V, R.osig, R.nbr_off, R.nbr, R.cnt,
                                                                         nullptr, nullptr);
        k_slot_cell<<<grid_of(R.n, 256), 256, 0, st>>>(R.n, R.nbr_off, R.slot_cell);
    } else if (R.pass == 1) {  // incidence fill
        k_facet_incidence<D, true><<<grid_of(R.V, 256), 256, 0, st>>>(R.n, R.V, R.osig, R.nbr_off, R.nbr, R.cnt,
                                                                        R.foff, R.fvert);
    } else if (R.pass == 2) {  // tier A
        constexpr int NW = TierA<D>::NW, GPB = TierA<D>::GPB;
        FCaps c = caps_for(D, R.capV, 1);
        if (NW == 1) c.capT = 0;
        const size_t sm = GPB * bytes_a<D>(c);
        if (cudaFuncSetAttribute(k_poly_facets<D, NW, GPB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
            cudaSuccess)
            return -1;
        int per = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_poly_facets<D, NW, GPB>, NW * 32 * GPB, sm) !=
                cudaSuccess || per < 1)
            return -1;
        k_poly_facets<D, NW, GPB><<<R.nsm * per, NW * 32 * GPB, sm, st>>>(P, c, R.nslots, R.next, R.big, R.nbig,
                                                                         R.maxnv);
    } else if (R.pass == 3) {  // tier B, shared memory
        const FCaps c = caps_for(D, R.capV, 1);
        const size_t sm = bytes_b<D>(c);
        if (cudaFuncSetAttribute(k_poly_big<D, 8, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) !=
            cudaSuccess)
            return -1;
        int per = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_poly_big<D, 8, true>, 256, sm) != cudaSuccess ||
            per < 1)
            return -1;
        const long long blocks = std::min<long long>(R.nbig_host, (long long)R.nsm * per);
        k_poly_big<D, 8, true><<<(int)blocks, 256, sm, st>>>(P, c, R.big, R.nbig_host, R.next, nullptr, R.big2,
                                                             R.nbig2, R.maxnv2);
    } else if (R.pass == 5) {  // tier B, global memory
        const FCaps c = caps_for(D, R.capV, R.widen);
        k_poly_big<D, 8, false><<<R.blocks, 256, 0, st>>>(P, c, R.big2, R.nbig_host, R.next, R.slab, nullptr,
                                                          nullptr, nullptr);
    } else {
        k_cell_volumes<D><<<grid_of(R.n, 256), 256, 0, st>>>(P, R.vol);
    }
    return 0;
}

int launch_poly(const PolyRun& R) {
    int rc = -1;
    HV_DISPATCH(R.d, (rc = poly_run<DD>(R)));
    return rc;
}

size_t poly_area_bytes(int d, int capV, int widen, bool tier_b) {
    size_t b = 0;
    HV_DISPATCH(d, (b = tier_b ? bytes_b<DD>(caps_for(DD, capV, widen))
                               : TierA<DD>::GPB * bytes_a<DD>(caps_for(DD, capV, widen))));
    return b;
}

}  // namespace hv
