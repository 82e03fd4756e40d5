// hv_search_impl.cuh -- Voronoi vertex search on the GPU (kernels and
// per-dimension launch templates; instantiated by hv_search_d{2..6}.cu).
//
// The vertex set is explored as a wavefront over the graph of Voronoi
// vertices: level 0 holds one seed vertex per generator (descent), level k+1
// the vertices first reached by walking the edges of level k.  A walk from
// vertex S along the edge S \ {q} is the incircle raycast of the reference
// (raycast_des2, src/raycast.jl:794-970): the next generator is the argmin over
// u.(x_j - x_b) > 0 of t_j = (|x_j - r|^2 - |x_b - r|^2) / (2 u.(x_j - x_b)),
// with boundary planes entering through their crossing parameter (the t of the
// mirror node N+p, src/raycast.jl:354-375).  New vertices are deduplicated in
// an open-addressing hash keyed on the sorted generator tuple (the role of
// the reference's vertex database / QueueHashTable, src/hvdatabase.jl:111,
// src/queuehashing.jl:8-104).
//
// Two ray kernels:
//  * exact (one ray per thread, FP64): shrinking-ball search over the tree
//    (the fused kd traversal of RCCombined, src/raycast.jl:504-528); used for
//    the PLAIN method and as the fallback of the fast kernel;
//  * fast (one warp per vertex): all open edges of a vertex scan the FP32
//    candidate list of the vertex's anchor generator in one pass, with a
//    forward error bound per candidate; a decision is kept only if it is
//    certified and the new empty sphere lies inside the list's complete
//    radius, otherwise the ray is redone by the exact kernel.
#pragma once
#include "hv_internal.cuh"
#include "hv_host.h"

namespace hv {

constexpr double EPS64 = 1.1102230246251565e-16;

// ---------------------------------------------------------------------------
// vertex hash
// ---------------------------------------------------------------------------
// A slot read with acquire semantics: a published id orders the reads of its
// record after it (the writer fences before publishing).
__device__ __forceinline__ unsigned long long load_acquire(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
// Publication of a slot this thread owns (BUSY): its record's writes before it.
__device__ __forceinline__ void store_release(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
// Compare-and-swap whose read has acquire semantics: one round trip claims an
// empty slot or reads an occupied one as load_acquire would.
__device__ __forceinline__ unsigned long long cas_acquire(unsigned long long* p, unsigned long long cmp,
                                                          unsigned long long v) {
    unsigned long long old;
    asm volatile("atom.acquire.gpu.global.cas.b64 %0, [%1], %2, %3;" : "=l"(old) : "l"(p), "l"(cmp), "l"(v) : "memory");
    return old;
}

template <int D>
__device__ unsigned vertex_insert(const DevMesh& M, const int (&s)[D + 1], int newitem, bool& is_new) {
    is_new = false;
    const unsigned long long h = hash_items(s, D + 1);
    const unsigned fp = ((unsigned)(h >> 32) & 0x7FFFFFFFu) | 1u;
    unsigned long long slot = h & M.vhmask;
    for (unsigned long long probe = 0; probe <= M.vhmask; ++probe) {
        unsigned long long e = cas_acquire(&M.vhash[slot], HASH_EMPTY, HASH_BUSY);
        if (e == HASH_EMPTY) {
            unsigned vid = atomicAdd(M.vcount, 1u);
            if (vid >= M.vcap) {
                set_status(M, ST_VCAP);
                atomicExch(&M.vhash[slot], ((unsigned long long)fp << 32) | INVALID_ID);
                return INVALID_ID;
            }
#pragma unroll
            for (int k = 0; k <= D; ++k) M.vsig[(size_t)vid * (D + 1) + k] = s[k];
            M.vnew[vid] = newitem;
            store_release(&M.vhash[slot], ((unsigned long long)fp << 32) | vid);
            is_new = true;
            return vid;
        }
        int spins = 0;
        while (e == HASH_BUSY) {
            if (++spins > SPIN_LIMIT) { set_status(M, ST_TIMEOUT); return INVALID_ID; }
            __nanosleep(32);
            e = load_acquire(&M.vhash[slot]);
        }
        if ((unsigned)(e >> 32) == fp) {
            unsigned id = (unsigned)e;
            if (id != INVALID_ID) {
                bool eq = true;
#pragma unroll
                for (int k = 0; k <= D; ++k) eq &= (__ldcg(&M.vsig[(size_t)id * (D + 1) + k]) == s[k]);
                if (eq) return id;
            }
        }
        slot = (slot + 1) & M.vhmask;
    }
    set_status(M, ST_HASH);
    return INVALID_ID;
}

// FP64 circumcentre of a signature.
template <int D>
__device__ bool vertex_center(const DevMesh& M, const int (&s)[D + 1], double (&c)[D]) {
    double xa[D], A[D][D], rhs[D];
    const double* pa = M.pts + (size_t)s[0] * D;
#pragma unroll
    for (int k = 0; k < D; ++k) xa[k] = __ldg(pa + k);
#pragma unroll
    for (int r = 0; r < D; ++r) con_row<D, double>(M, xa, s[r + 1], A[r], rhs[r]);
    int piv[D];
    if (!lu_factor<D, double>(A, piv)) return false;
    lu_solve<D, double>(A, piv, rhs);
#pragma unroll
    for (int k = 0; k < D; ++k) c[k] = xa[k] + rhs[k];
    return true;
}

// ---------------------------------------------------------------------------
// exact FP64 search
// ---------------------------------------------------------------------------
struct Cand { int item; double t, lo, hi; };

struct SearchOut {
    Cand best;
    double second_lo;
    Cand amb[HV_NAMB];
    int namb;
    bool overflow;
};

template <int D>
struct Query {
    int a;
    double xa[D], rho[D], u[D], db[D];
    double lam;
    int excl[D + 1];
    int nexcl;
    double erho, eu;
};

__device__ __forceinline__ void consider(SearchOut& R, const Cand& c) {
    // a candidate may be met twice (seed set and tree): keep one copy
    if (c.item == R.best.item) return;
    for (int k = 0; k < R.namb; ++k) if (R.amb[k].item == c.item) return;
    if (c.lo < R.best.lo) {
        if (R.best.item >= 0) {
            R.second_lo = R.best.lo;
            if (R.best.lo <= c.hi) {
                if (R.namb < HV_NAMB) R.amb[R.namb++] = R.best; else R.overflow = true;
            }
        }
        R.best = c;
    } else {
        if (c.lo < R.second_lo) R.second_lo = c.lo;
        if (c.lo <= R.best.hi) {
            if (R.namb == HV_NAMB) {  // compact: drop what the current best excludes
                int w = 0;
                for (int k = 0; k < HV_NAMB; ++k) if (R.amb[k].lo <= R.best.hi) R.amb[w++] = R.amb[k];
                R.namb = w;
            }
            if (R.namb < HV_NAMB) R.amb[R.namb++] = c; else R.overflow = true;
        }
    }
}

template <int D>
__device__ __forceinline__ bool q_excluded(const Query<D>& q, int it) {
    bool ex = false;
#pragma unroll
    for (int s = 0; s <= D; ++s) ex |= (s < q.nexcl && q.excl[s] == it);
    return ex;
}

// FP64 interval of generator j's crossing parameter; false if the ray moves away from it.
template <int D>
__device__ __forceinline__ bool cand_point(const DevMesh& M, const Query<D>& q, int j, Cand& c) {
    const double* xj = M.pts + (size_t)j * D;
    double nd = 0, dr = 0, du = 0, sdr = 0, sdu = 0, l1 = 0;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        double dl = __ldg(xj + k) - q.xa[k];
        nd = fma(dl, dl, nd); dr = fma(dl, q.rho[k], dr); du = fma(dl, q.u[k], du);
        sdr += fabs(dl * q.rho[k]); sdu += fabs(dl * q.u[k]); l1 += fabs(dl);
    }
    double num = nd - 2.0 * dr;
    double den = 2.0 * (du - q.lam);
    double e_num = (4.0 * D + 8.0) * EPS64 * (nd + 2.0 * sdr) + 2.0 * l1 * q.erho;
    double e_den = (2.0 * D + 8.0) * EPS64 * 2.0 * (sdu + fabs(q.lam)) + 4.0 * l1 * q.eu;
    c.item = j;
    if (den > e_den) {
        c.t = num / den;
        double et = (e_num + fabs(c.t) * e_den) / (den - e_den) + 4.0 * EPS64 * fabs(c.t);
        c.lo = c.t - et; c.hi = c.t + et;
    } else if (den < -e_den) {
        return false;
    } else {
        if (num - e_num > 0) {
            if (!(den + e_den > 0)) return false;
            c.lo = (num - e_num) / (den + e_den); c.hi = INFINITY; c.t = c.lo;
        } else {
            c.lo = -INFINITY; c.hi = INFINITY; c.t = 0;
        }
    }
    return true;
}

template <int D>
__device__ __forceinline__ void eval_point(const DevMesh& M, const Query<D>& q, int j, SearchOut& R) {
    Cand c;
    if (!cand_point<D>(M, q, j, c)) return;
    if (c.lo < R.best.hi || c.lo < R.second_lo) consider(R, c);
}

// FP64 intervals of the boundary planes' crossings: sink(Cand) for each plane the ray approaches.
template <int D, class Sink>
__device__ __forceinline__ void cand_planes(const DevMesh& M, const Query<D>& q, Sink&& sink) {
#pragma unroll
    for (int p = 0; p < M.np; ++p) {
        const int it = M.n + p;
        if (q_excluded<D>(q, it)) continue;
        const DevPlane& P = M.planes[p];
        double uk, num, e_num, e_den;
        if (P.axis >= 0) {  // cuboid face: n = +-e_k, every product below is exact
            double nc = 0, ac = 0;
            uk = 0;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                nc = fma(P.n[k], q.xa[k] + q.rho[k], nc);
                uk = fma(P.n[k], q.u[k], uk);
                ac += fabs(P.n[k]) * (fabs(q.xa[k]) + fabs(q.rho[k]));
            }
            num = P.off - nc;
            e_num = 4.0 * EPS64 * (fabs(P.off) + ac) + q.erho;
            e_den = q.eu + 2.0 * EPS64 * fabs(uk);
        } else {  // off - n.(xa + rho): the xa part in double-double
            const dd sx = plane_rhs_dd<D>(P, q.xa);
            double nr = 0, nu = 0, an = 0, anr = 0, anu = 0;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                nr = fma(P.n[k], q.rho[k], nr);
                nu = fma(P.n[k], q.u[k], nu);
                an += fabs(P.n[k]);
                anr += fabs(P.n[k] * q.rho[k]);
                anu += fabs(P.n[k] * q.u[k]);
            }
            num = (sx.hi + sx.lo) - nr;
            uk = nu;
            e_num = 4.0 * EPS64 * fabs(num) + (D + 4.0) * EPS64 * anr + q.erho * an;
            e_den = q.eu * an + (D + 2.0) * EPS64 * anu;
        }
        Cand c; c.item = it;
        if (uk > e_den) {
            c.t = num / uk;
            double et = (e_num + fabs(c.t) * e_den) / (uk - e_den) + 4.0 * EPS64 * fabs(c.t);
            c.lo = c.t - et; c.hi = c.t + et;
        } else if (uk < -e_den) {
            continue;
        } else {
            if (num - e_num > 0) { c.lo = (num - e_num) / (fabs(uk) + e_den); c.hi = INFINITY; c.t = c.lo; }
            else { c.lo = -INFINITY; c.hi = INFINITY; c.t = 0; }
        }
        sink(c);
    }
}

template <int D>
__device__ __forceinline__ void eval_planes(const DevMesh& M, const Query<D>& q, SearchOut& R) {
    cand_planes<D>(M, q, [&](const Cand& c) { consider(R, c); });
}

template <int D>
__device__ __forceinline__ double box_dist2(const DevMesh& M, int node, const double (&c)[D]) {
    const float* lo = M.blo + (size_t)node * M.dp;
    const float* hi = M.bhi + (size_t)node * M.dp;
    double s = 0;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        double l = (double)__ldg(lo + k), h = (double)__ldg(hi + k);
        double e = c[k] < l ? l - c[k] : (c[k] > h ? c[k] - h : 0.0);
        s = fma(e, e, s);
    }
    return s;
}

// Shrinking-ball tree search for argmin t (certified with forward error bounds).
template <int D>
__device__ void exact_search(const DevMesh& M, const Query<D>& q, SearchOut& R) {
    R.best = Cand{-1, INFINITY, INFINITY, INFINITY};
    R.second_lo = INFINITY;
    R.namb = 0;
    R.overflow = false;
    eval_planes<D>(M, q, R);
    // start from the anchor's neighbourhood so that the ball is small before
    // the tree is entered: its leaf, then the head of its candidate list
    {
        const int la = q.a / M.leaf;
        const int s0 = la * M.leaf, s1 = min(s0 + M.leaf, M.n);
        for (int j = s0; j < s1; ++j) if (!q_excluded<D>(q, j)) eval_point<D>(M, q, j, R);
        const int kh = min(M.K, 32);
        for (int c = 0; c < kh; ++c) {
            const int j = __ldg(M.knn + (size_t)q.a * M.K + c);
            if (j >= 0 && !q_excluded<D>(q, j)) eval_point<D>(M, q, j, R);
        }
    }
    int stack[64];
    int sp = 0;
    stack[sp++] = 1;
    while (sp > 0) {
        const int node = stack[--sp];
        const double tp = R.best.hi;
        if (isfinite(tp)) {
            const double tpp = tp * (1.0 + 1e-9) + 1e-300;
            double c[D];
            double r2 = 0;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                double off = q.rho[k] + tpp * q.u[k];
                c[k] = q.xa[k] + off;
                double w = q.db[k] - off;
                r2 = fma(w, w, r2);
            }
            if (box_dist2<D>(M, node, c) > r2 * (1.0 + 1e-9) + 1e-280) continue;
        }
        if (node >= M.P) {
            const int l = node - M.P;
            if (l >= M.nleaves) continue;
            const int s0 = l * M.leaf;
            const int s1 = min(s0 + M.leaf, M.n);
            for (int j = s0; j < s1; ++j) {
                if (q_excluded<D>(q, j)) continue;
                eval_point<D>(M, q, j, R);
            }
        } else {
            const double tp2 = isfinite(R.best.hi) ? R.best.hi : 0.0;
            double c[D];
#pragma unroll
            for (int k = 0; k < D; ++k) c[k] = q.xa[k] + q.rho[k] + tp2 * q.u[k];
            const double dl = box_dist2<D>(M, 2 * node, c);
            const double dr = box_dist2<D>(M, 2 * node + 1, c);
            if (sp + 2 > 64) { set_status(M, ST_STACK); break; }
            if (dl <= dr) { stack[sp++] = 2 * node + 1; stack[sp++] = 2 * node; }
            else { stack[sp++] = 2 * node; stack[sp++] = 2 * node + 1; }
        }
    }
    int w = 0;
    for (int k = 0; k < R.namb; ++k)
        if (R.amb[k].item != R.best.item && R.amb[k].lo <= R.best.hi) R.amb[w++] = R.amb[k];
    R.namb = w;
}

// Every item whose FP64 interval starts at or below H (planes, then the tree
// with the ball of parameter H): visit(item).  Used when more candidates than
// HV_NAMB tie with the winner within FP64 (near-degenerate generators).
template <int D, class Visit>
__device__ void exact_visit(const DevMesh& M, const Query<D>& q, double H, Visit&& visit) {
    cand_planes<D>(M, q, [&](const Cand& c) { if (c.lo <= H) visit(c.item); });
    const double tpp = H * (1.0 + 1e-9) + 1e-300;
    double c[D];
    double r2 = 0;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const double off = q.rho[k] + tpp * q.u[k];
        c[k] = q.xa[k] + off;
        const double w = q.db[k] - off;
        r2 = fma(w, w, r2);
    }
    r2 = r2 * (1.0 + 1e-9) + 1e-280;
    int stack[64];
    int sp = 0;
    stack[sp++] = 1;
    while (sp > 0) {
        const int node = stack[--sp];
        if (box_dist2<D>(M, node, c) > r2) continue;
        if (node >= M.P) {
            const int l = node - M.P;
            if (l >= M.nleaves) continue;
            const int s0 = l * M.leaf, s1 = min(s0 + M.leaf, M.n);
            for (int j = s0; j < s1; ++j) {
                if (q_excluded<D>(q, j)) continue;
                Cand cj;
                if (cand_point<D>(M, q, j, cj) && cj.lo <= H) visit(j);
            }
        } else {
            if (sp + 2 > 64) { set_status(M, ST_STACK); return; }
            stack[sp++] = 2 * node + 1;
            stack[sp++] = 2 * node;
        }
    }
}

// Is any real generator outside S strictly inside the sphere (c, r2)?
template <int D>
__device__ bool ball_occupied(const DevMesh& M, const double (&c)[D], double r2, const int (&S)[D + 1], double tol) {
    int stack[64];
    int sp = 0;
    stack[sp++] = 1;
    while (sp > 0) {
        const int node = stack[--sp];
        if (box_dist2<D>(M, node, c) >= r2) continue;
        if (node >= M.P) {
            const int l = node - M.P;
            if (l >= M.nleaves) continue;
            const int s0 = l * M.leaf, s1 = min(s0 + M.leaf, M.n);
            for (int j = s0; j < s1; ++j) {
                bool ex = false;
#pragma unroll
                for (int s = 0; s <= D; ++s) ex |= (S[s] == j);
                if (ex) continue;
                const double* xj = M.pts + (size_t)j * D;
                double dd2 = 0;
#pragma unroll
                for (int k = 0; k < D; ++k) { double e = __ldg(xj + k) - c[k]; dd2 = fma(e, e, dd2); }
                if (dd2 < r2 * (1.0 - tol)) return true;
            }
        } else {
            if (sp + 2 > 64) { set_status(M, ST_STACK); return true; }
            stack[sp++] = 2 * node; stack[sp++] = 2 * node + 1;
        }
    }
    return false;
}

// ---------------------------------------------------------------------------
// double-double re-scoring of ambiguous decisions
// ---------------------------------------------------------------------------
template <int D>
__device__ int dd_rescore_walk(const DevMesh& M, const int (&sig)[D + 1], int m, const int* items, int nitems,
                               bool& degen) {
    degen = false;
    double xa[D];
    const double* pa = M.pts + (size_t)sig[0] * D;
#pragma unroll
    for (int k = 0; k < D; ++k) xa[k] = __ldg(pa + k);
    dd A[D][D], rho[D], u[D], db[D];
#pragma unroll
    for (int r = 0; r < D; ++r) con_row<D, dd>(M, xa, sig[r + 1], A[r], rho[r]);
    int piv[D];
    if (!lu_factor<D, dd>(A, piv)) { degen = true; return nitems > 0 ? items[0] : -1; }
    lu_solve<D, dd>(A, piv, rho);
#pragma unroll
    for (int k = 0; k < D; ++k) { u[k] = mk(0.0); db[k] = mk(0.0); }
    if (m >= 1) {
#pragma unroll
        for (int k = 0; k < D; ++k) u[k] = mk(k == m - 1 ? 1.0 : 0.0);
        lu_solve<D, dd>(A, piv, u);
#pragma unroll
        for (int k = 0; k < D; ++k) u[k] = -u[k];
    } else {
        int b = -1;
#pragma unroll
        for (int r = 0; r < D; ++r) {
            bool real = sig[r + 1] < M.n;
            u[r] = mk(real ? 1.0 : 0.0);
            if (real && b < 0) b = sig[r + 1];
        }
        lu_solve<D, dd>(A, piv, u);
        if (b >= 0) {
            const double* pb = M.pts + (size_t)b * D;
#pragma unroll
            for (int k = 0; k < D; ++k) db[k] = diff_d<dd>(__ldg(pb + k), xa[k]);
        }
    }
    dd lam = mk(0.0);
#pragma unroll
    for (int k = 0; k < D; ++k) lam += u[k] * db[k];
    int best = -1, second = -1;
    dd bt = mk(0.0), st = mk(0.0);
    for (int c = 0; c < nitems; ++c) {
        const int it = items[c];
        dd t;
        if (it < M.n) {
            const double* xj = M.pts + (size_t)it * D;
            dd nd = mk(0.0), dr = mk(0.0), du = mk(0.0);
#pragma unroll
            for (int k = 0; k < D; ++k) {
                dd dl = diff_d<dd>(__ldg(xj + k), xa[k]);
                nd += dl * dl; dr += dl * rho[k]; du += dl * u[k];
            }
            dd den = (du - lam) * mk(2.0);
            if (!(den.hi > 0)) continue;
            t = (nd - dr * mk(2.0)) / den;
        } else {
            // off - n.(xa + rho) over n.u; for axis planes the zero terms and
            // the +-1 products are exact
            const DevPlane& P = M.planes[it - M.n];
            dd uk = mk(0.0), num = mk(P.off);
#pragma unroll
            for (int k = 0; k < D; ++k) {
                uk += mk(P.n[k]) * u[k];
                num -= mk(P.n[k]) * (mk(xa[k]) + rho[k]);
            }
            if (!(uk.hi > 0)) continue;
            t = num / uk;
        }
        if (best < 0 || t < bt || (!(bt < t) && it < best)) { second = best; st = bt; best = it; bt = t; }
        else if (second < 0 || t < st) { second = it; st = t; }
    }
    if (best >= 0 && second >= 0) {
        dd gap = st - bt;
        if (gap.hi <= 1e-27 * (fabs(bt.hi) + 1e-3)) degen = true;
    }
    return best;
}

// Re-evaluate a descent step in double-double from the FP64 state.
template <int D>
__device__ int dd_rescore_point(const DevMesh& M, const Query<D>& q, const int* items, int nitems, double& tout) {
    int best = -1;
    dd bt = mk(0.0);
    for (int c = 0; c < nitems; ++c) {
        const int it = items[c];
        dd t;
        if (it < M.n) {
            const double* xj = M.pts + (size_t)it * D;
            dd nd = mk(0.0), dr = mk(0.0), du = mk(0.0);
#pragma unroll
            for (int k = 0; k < D; ++k) {
                dd dl = diff_d<dd>(__ldg(xj + k), q.xa[k]);
                nd += dl * dl; dr += dl * mk(q.rho[k]); du += dl * mk(q.u[k]);
            }
            dd den = (du - mk(q.lam)) * mk(2.0);
            if (!(den.hi > 0)) continue;
            t = (nd - dr * mk(2.0)) / den;
        } else {
            const DevPlane& P = M.planes[it - M.n];
            if (P.axis >= 0) {  // n = +-e_k: the three dot products are exact
                double uk = 0, xk = 0, rk = 0;
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    uk = fma(P.n[k], q.u[k], uk);
                    xk = fma(P.n[k], q.xa[k], xk);
                    rk = fma(P.n[k], q.rho[k], rk);
                }
                if (!(uk > 0)) continue;
                t = (mk(P.off) - (mk(xk) + mk(rk))) / mk(uk);
            } else {
                dd uk = mk(0.0);
                dd num = plane_rhs_dd<D>(P, q.xa);
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    uk += mk(P.n[k]) * mk(q.u[k]);
                    num -= mk(P.n[k]) * mk(q.rho[k]);
                }
                if (!(uk.hi > 0)) continue;
                t = num / uk;
            }
        }
        if (best < 0 || t < bt || (!(bt < t) && it < best)) { best = it; bt = t; }
    }
    tout = bt.hi;
    return best;
}

// ---------------------------------------------------------------------------
// exact walk of one edge (PLAIN method and fallback)
// ---------------------------------------------------------------------------
// Sets up the ray leaving vertex `sig` along the edge sig \ {sig[m]}.
template <int D>
__device__ bool setup_walk(const DevMesh& M, const int (&sig)[D + 1], int m, Query<D>& q) {
    q.a = sig[0];
    const double* pa = M.pts + (size_t)q.a * D;
#pragma unroll
    for (int k = 0; k < D; ++k) q.xa[k] = __ldg(pa + k);
    double A[D][D], rhs[D];
#pragma unroll
    for (int r = 0; r < D; ++r) con_row<D, double>(M, q.xa, sig[r + 1], A[r], rhs[r]);
    double nrm = 0;
#pragma unroll
    for (int r = 0; r < D; ++r) {
        double s = 0;
#pragma unroll
        for (int k = 0; k < D; ++k) s += fabs(A[r][k]);
        nrm = fmax(nrm, s);
    }
    int piv[D];
    if (!lu_factor<D, double>(A, piv)) { set_status(M, ST_NUMERIC); return false; }
#pragma unroll
    for (int k = 0; k < D; ++k) q.rho[k] = rhs[k];
    lu_solve<D, double>(A, piv, q.rho);
    double rows[D];
    int b = -1;
#pragma unroll
    for (int k = 0; k < D; ++k) { rows[k] = 0; q.u[k] = 0; q.db[k] = 0; }
#pragma unroll
    for (int c = 0; c < D; ++c) {
        double col[D];
#pragma unroll
        for (int k = 0; k < D; ++k) col[k] = (k == c) ? 1.0 : 0.0;
        lu_solve<D, double>(A, piv, col);
#pragma unroll
        for (int k = 0; k < D; ++k) rows[k] += fabs(col[k]);
        const bool real = sig[c + 1] < M.n;
        if (m >= 1 && c == m - 1) {
#pragma unroll
            for (int k = 0; k < D; ++k) q.u[k] = -col[k];
        }
        if (m == 0 && real) {
#pragma unroll
            for (int k = 0; k < D; ++k) q.u[k] += col[k];
            if (b < 0) b = sig[c + 1];
        }
    }
    if (m == 0) {
        if (b < 0) return false;  // the edge holds only planes: no walk
        const double* pb = M.pts + (size_t)b * D;
#pragma unroll
        for (int k = 0; k < D; ++k) q.db[k] = __ldg(pb + k) - q.xa[k];
    }
    double ninv = 0;
#pragma unroll
    for (int k = 0; k < D; ++k) ninv = fmax(ninv, rows[k]);
    const double cond = nrm * ninv;
    double nu = 0;
#pragma unroll
    for (int k = 0; k < D; ++k) nu = fma(q.u[k], q.u[k], nu);
    nu = sqrt(nu);
    if (!(nu > 0)) { set_status(M, ST_NUMERIC); return false; }
    q.lam = 0;
    double nr = 0, nuu = 0;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        q.u[k] /= nu;
        q.lam = fma(q.u[k], q.db[k], q.lam);
        nr = fmax(nr, fabs(q.rho[k]));
        nuu = fmax(nuu, fabs(q.u[k]));
    }
    const double kap = 8.0 * D * fmax(cond, 1.0) * EPS64;
    q.erho = kap * (nr + 1e-3);
    q.eu = kap * (nuu + 1e-3);
#pragma unroll
    for (int s = 0; s <= D; ++s) q.excl[s] = sig[s];
    q.nexcl = D + 1;
    return true;
}

template <int D>
__device__ void exact_walk(const DevMesh& M, unsigned v, int m) {
    int sig[D + 1];
#pragma unroll
    for (int k = 0; k <= D; ++k) sig[k] = M.vsig[(size_t)v * (D + 1) + k];
    Query<D> q;
    if (!setup_walk<D>(M, sig, m, q)) return;
    SearchOut R;
    exact_search<D>(M, q, R);
    if (R.best.item < 0) { set_status(M, ST_NUMERIC); return; }
    int win = R.best.item;
    if (!(R.best.hi < R.second_lo)) {
        count_add(M.cnt + C_DD);
        int items[HV_NAMB + 1];
        bool degen = false;
        if (!R.overflow) {
            items[0] = R.best.item;
            for (int k = 0; k < R.namb; ++k) items[k + 1] = R.amb[k].item;
            win = dd_rescore_walk<D>(M, sig, m, items, R.namb + 1, degen);
        } else {
            // more near-ties than the set holds: every item whose interval reaches
            // below the winner's upper bound is re-scored in double-double, HV_NAMB
            // at a time against the running winner
            int nb = 0;
            auto flush = [&]() {
                items[0] = win;
                bool d2 = false;
                const int w2 = dd_rescore_walk<D>(M, sig, m, items, nb + 1, d2);
                if (w2 >= 0) {  // a tie counts while its winner stands
                    degen = (w2 == win) ? (degen || d2) : d2;
                    win = w2;
                }
                nb = 0;
            };
            exact_visit<D>(M, q, R.best.hi, [&](int it) {
                if (it == win) return;
                items[1 + nb++] = it;
                if (nb == HV_NAMB) flush();
            });
            if (nb > 0) flush();
        }
        if (degen) { count_add(M.cnt + C_DEGEN); set_status(M, ST_DEGEN); }
        if (win < 0) { set_status(M, ST_NUMERIC); return; }
    }
    int ns[D + 1];
    make_sig<D>(sig, m, win, ns);
    bool is_new;
    vertex_insert<D>(M, ns, win, is_new);
}

// Edge sig \ {sig[m]} is walkable if it is not the edge the vertex was found
// through and if it still contains a real generator (in a shard: one of the
// shard's own generators, so that only the shard's cells are explored).
template <int D>
__device__ __forceinline__ bool walkable(const DevMesh& M, const int (&sig)[D + 1], int vnew, int m) {
    if (sig[m] == vnew) return false;
    if (M.own_from >= 0) {
        bool own = false;
#pragma unroll
        for (int s = 0; s <= D; ++s) own |= (s != m && sig[s] < M.n && __ldg(M.perm + sig[s]) >= M.own_from);
        return own;
    }
    if (M.own0 > 0 || M.own1 < M.n) {
        bool own = false;
#pragma unroll
        for (int s = 0; s <= D; ++s) own |= (s != m && sig[s] >= M.own0 && sig[s] < M.own1);
        return own;
    }
    if (m == 0) return sig[1] < M.n;
    return true;
}

template <int D>
__global__ void __launch_bounds__(128) k_expand_plain(DevMesh M, unsigned f0, unsigned f1) {
    const unsigned long long total = (unsigned long long)(f1 - f0) * (D + 1);
    for (unsigned long long r = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; r < total;
         r += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned v = f0 + (unsigned)(r / (D + 1));
        const int m = (int)(r % (D + 1));
        int sig[D + 1];
#pragma unroll
        for (int k = 0; k <= D; ++k) sig[k] = M.vsig[(size_t)v * (D + 1) + k];
        if (!walkable<D>(M, sig, M.vnew[v], m)) continue;
        if (M.ecnt && ((__ldg(M.ecnt + v) >> m) & 1u)) continue;  // both end points known
        count_add(M.cnt + C_RAYS);
        exact_walk<D>(M, v, m);
    }
}

template <int D>
__global__ void __launch_bounds__(128) k_fallback(DevMesh M, const unsigned long long* fq, const unsigned* nfq,
                                                  unsigned fqcap) {
    if (M.G.lvl) {  // graph-driven levels: the exact queue of the previous level
        const int p = (M.G.lvl[2] + 1) & 1;
        fq = M.G.fx[p]; nfq = M.G.qc + 2 * p + 1;
    }
    const unsigned n = min(*nfq, fqcap);  // entries past the capacity were never written
    for (unsigned r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const unsigned long long e = fq[r];
        count_add(M.cnt + C_FALLBACK);
        exact_walk<D>(M, (unsigned)(e >> 4), (int)(e & 7));
    }
}

// ---------------------------------------------------------------------------
// descent: one seed vertex per selected generator (src/raycast.jl:45-109)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void philox4x32(unsigned (&c)[4], unsigned k0, unsigned k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        unsigned hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
        unsigned hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
        unsigned o0 = hi1 ^ c[1] ^ k0, o2 = hi0 ^ c[3] ^ k1;
        c[0] = o0; c[1] = lo1; c[2] = o2; c[3] = lo0;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
}

template <int D>
__device__ void gauss_dir(unsigned long long seed, unsigned a, unsigned long long b, double (&g)[D]) {
    int got = 0;
#pragma unroll
    for (unsigned blk = 0; blk < (unsigned)((D + 3) / 4); ++blk) {
        unsigned c[4] = {a, (unsigned)b, (unsigned)(b >> 32), blk};
        philox4x32(c, (unsigned)seed, (unsigned)(seed >> 32));
#pragma unroll
        for (int p = 0; p < 2; ++p) {
            // Box-Muller in FP32: the descent needs random directions, not accurate
            // ones, and FP64 transcendentals cost a lane-0 latency chain per step
            const float u1 = ((float)(c[2 * p] >> 8) + 0.5f) * 5.9604645e-08f;  // (0, 1), 24 bits
            const float u2 = ((float)(c[2 * p + 1] >> 8) + 0.5f) * 5.9604645e-08f;
            const double rr = (double)sqrtf(-2.f * logf(u1));
            float snf, csf;
            sincospif(2.f * u2, &snf, &csf);
            const double sn = snf, cs = csf;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                if (k == got) g[k] = rr * cs;
                if (k == got + 1) g[k] = rr * sn;
            }
            got += 2;
        }
    }
}

template <int D>
__global__ void __launch_bounds__(128) k_descent(DevMesh M, int stride, int nseeds, unsigned long long seed,
                                                 const int* list, const unsigned* nlist) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (list && idx >= (int)*nlist) return;
    if (!list && idx >= nseeds) return;
    const int i = list ? list[idx] : M.own0 + idx * stride;
    if (i >= M.own1) return;
    if (!list && M.own_from >= 0 && __ldg(M.perm + i) < M.own_from) return;  // refinement: new cells only
    count_add(M.cnt + C_DESCENT);
    for (int attempt = 0; attempt < 16; ++attempt) {
        Query<D> q;
        q.a = i;
        const double* pa = M.pts + (size_t)i * D;
#pragma unroll
        for (int k = 0; k < D; ++k) { q.xa[k] = __ldg(pa + k); q.rho[k] = 0; q.db[k] = 0; }
        q.lam = 0; q.erho = 1e-12; q.eu = 1e-13;
        q.excl[0] = i; q.nexcl = 1;
#pragma unroll
        for (int s = 1; s <= D; ++s) q.excl[s] = -1;
        bool ok = true;
        for (int step = 1; step <= D && ok; ++step) {
            double g[D];
            gauss_dir<D>(seed, (unsigned)(attempt * 16 + step), (unsigned long long)i, g);
            // Gram-Schmidt basis of the constraint rows of the current set
            double B[D][D];
#pragma unroll
            for (int s = 1; s < D; ++s) {
                if (s >= q.nexcl) break;
                double row[D], rh;
                con_row<D, double>(M, q.xa, q.excl[s], row, rh);
#pragma unroll
                for (int t = 0; t < D - 1; ++t) {
                    if (t >= s - 1) break;
                    double pr = 0;
#pragma unroll
                    for (int k = 0; k < D; ++k) pr = fma(row[k], B[t][k], pr);
#pragma unroll
                    for (int k = 0; k < D; ++k) row[k] -= pr * B[t][k];
                }
                double nn = 0;
#pragma unroll
                for (int k = 0; k < D; ++k) nn = fma(row[k], row[k], nn);
                nn = sqrt(nn);
                if (!(nn > 1e-300)) { ok = false; break; }
#pragma unroll
                for (int k = 0; k < D; ++k) B[s - 1][k] = row[k] / nn;
            }
            if (!ok) break;
            for (int rep = 0; rep < 2; ++rep) {
#pragma unroll
                for (int t = 0; t < D - 1; ++t) {
                    if (t >= q.nexcl - 1) break;
                    double pr = 0;
#pragma unroll
                    for (int k = 0; k < D; ++k) pr = fma(g[k], B[t][k], pr);
#pragma unroll
                    for (int k = 0; k < D; ++k) g[k] -= pr * B[t][k];
                }
            }
            double nn = 0;
#pragma unroll
            for (int k = 0; k < D; ++k) nn = fma(g[k], g[k], nn);
            nn = sqrt(nn);
            if (!(nn > 1e-12)) { ok = false; break; }
#pragma unroll
            for (int k = 0; k < D; ++k) q.u[k] = g[k] / nn;
            SearchOut R;
            exact_search<D>(M, q, R);
            if (R.best.item < 0) { ok = false; break; }
            int win = R.best.item;
            double t = R.best.t;
            if (!(R.best.hi < R.second_lo) && R.overflow) { ok = false; break; }  // near-degenerate step: retry
            if (!(R.best.hi < R.second_lo)) {
                int items[HV_NAMB + 1];
                items[0] = R.best.item;
                for (int k = 0; k < R.namb; ++k) items[k + 1] = R.amb[k].item;
                win = dd_rescore_point<D>(M, q, items, R.namb + 1, t);
                if (win < 0) { ok = false; break; }
            }
            if (!(t > 0) || !isfinite(t)) { ok = false; break; }
#pragma unroll
            for (int k = 0; k < D; ++k) q.rho[k] = fma(t, q.u[k], q.rho[k]);
#pragma unroll
            for (int s = 0; s <= D; ++s) if (s == q.nexcl) q.excl[s] = win;
            q.nexcl++;
        }
        if (ok) {
            int S[D + 1];
#pragma unroll
            for (int s = 0; s <= D; ++s) S[s] = q.excl[s];
            // sort (insertion, D+1 <= 7)
#pragma unroll
            for (int s = 1; s <= D; ++s) {
#pragma unroll
                for (int t = s; t > 0; --t) {
                    if (S[t] < S[t - 1]) { int x = S[t]; S[t] = S[t - 1]; S[t - 1] = x; }
                }
            }
            double c[D];
            bool good = vertex_center<D>(M, S, c);
            if (good) {
                double r2 = 0;
                const double* p0 = M.pts + (size_t)S[0] * D;
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    double e = __ldg(p0 + k) - c[k];
                    r2 = fma(e, e, r2);
                }
                // inside the domain (every plane, with a small tolerance)
                for (int p = 0; p < M.np && good; ++p) {
                    const DevPlane& P = M.planes[p];
                    double nc = 0, anc = 0;
#pragma unroll
                    for (int k = 0; k < D; ++k) { nc = fma(P.n[k], c[k], nc); anc += fabs(P.n[k] * c[k]); }
                    if (nc > P.off + 1e-12 * (1.0 + fabs(P.off) + anc)) good = false;
                }
                if (good) good = !ball_occupied<D>(M, c, r2, S, 1e-10);
            }
            if (good) {
                bool is_new;
                vertex_insert<D>(M, S, -1, is_new);
                return;
            }
        }
        count_add(M.cnt + C_DRETRY);
    }
    set_status(M, ST_DESCENT);
}

// ---------------------------------------------------------------------------
// edge registry (src/edgehashing.jl:49-111): an edge is the sorted d-tuple
// sig \ {sig[m]}; the table entry references (vertex, slot) so the key is read
// back from the vertex record.  The second end point to register an edge
// closes it for both: neither walks it (both end points are known).
// ---------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(256) k_register_edges(DevMesh M, unsigned v0, unsigned v1) {
    if (M.G.lvl) { v0 = M.G.lvl[0]; v1 = M.G.lvl[1]; }
    const unsigned long long total = (unsigned long long)(v1 - v0) * (D + 1);
    for (unsigned long long r = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; r < total;
         r += (unsigned long long)gridDim.x * blockDim.x) {
        const unsigned v = v0 + (unsigned)(r / (D + 1));
        const int m = (int)(r % (D + 1));
        int sig[D + 1];
#pragma unroll
        for (int k = 0; k <= D; ++k) sig[k] = M.vsig[(size_t)v * (D + 1) + k];
        if (m == 0 && sig[1] >= M.n) continue;  // the edge holds only planes
        int e[D];
        int o = 0;
#pragma unroll
        for (int k = 0; k <= D; ++k) if (k != m) e[o++] = sig[k];
        const unsigned long long h = hash_items(e, D);
        const unsigned fp = ((unsigned)(h >> 32) & 0x7FFFFFFFu) | 1u;
        const unsigned long long mine = ((unsigned long long)fp << 32) | ((unsigned long long)v * 8u + (unsigned)m);
        unsigned long long slot = h & M.ehmask;
        bool done = false;
        for (unsigned long long probe = 0; probe <= M.ehmask && !done; ++probe) {
            const unsigned long long prev = atomicCAS(&M.ehash[slot], HASH_EMPTY, mine);
            if (prev == HASH_EMPTY) { done = true; break; }
            if ((unsigned)(prev >> 32) == fp) {
                const unsigned ref = (unsigned)prev;
                const unsigned ov = ref >> 3, om = ref & 7u;
                int q = 0;
                bool eq = true;
#pragma unroll
                for (int k = 0; k <= D; ++k) {
                    if (k == (int)om) continue;
                    const int x = M.vsig[(size_t)ov * (D + 1) + k];
#pragma unroll
                    for (int z = 0; z < D; ++z) if (z == q) eq &= (x == e[z]);
                    ++q;
                }
                if (eq) {
                    atomicOr(M.ecnt + ov, 1u << om);
                    atomicOr(M.ecnt + v, 1u << m);
                    count_add(M.cnt + C_EDGECLOSED);
                    done = true;
                    break;
                }
            }
            slot = (slot + 1) & M.ehmask;
        }
        if (!done) set_status(M, ST_ECAP);
    }
}

// ---------------------------------------------------------------------------
// FP64 circumcentres of new vertices, one thread per vertex (full-warp FP64)
// ---------------------------------------------------------------------------
// LU with partial pivoting keeping the reciprocals of the pivots: one FP64
// division per pivot instead of one per eliminated entry and per solve step
// (the centres and the inverse below need d + 1 solves per vertex).
template <int D>
__device__ __forceinline__ bool lu_factor_rcp(double (&A)[D][D], int (&piv)[D], double (&rd)[D]) {
#pragma unroll
    for (int c = 0; c < D; ++c) {
        int p = c;
        double best = fabs(A[c][c]);
#pragma unroll
        for (int r = c + 1; r < D; ++r) { const double v = fabs(A[r][c]); if (v > best) { best = v; p = r; } }
        piv[c] = p;
        if (best == 0.0) return false;
        if (p != c) {
#pragma unroll
            for (int k = 0; k < D; ++k) {
#pragma unroll
                for (int r = c + 1; r < D; ++r) {
                    if (r == p) { const double t = A[c][k]; A[c][k] = A[r][k]; A[r][k] = t; }
                }
            }
        }
        rd[c] = 1.0 / A[c][c];
#pragma unroll
        for (int r = c + 1; r < D; ++r) {
            const double f = A[r][c] * rd[c];
            A[r][c] = f;
#pragma unroll
            for (int k = c + 1; k < D; ++k) A[r][k] = fma(-f, A[c][k], A[r][k]);
        }
    }
    return true;
}

template <int D>
__device__ __forceinline__ void lu_solve_rcp(const double (&A)[D][D], const int (&piv)[D], const double (&rd)[D],
                                             double (&b)[D]) {
#pragma unroll
    for (int c = 0; c < D; ++c) {
#pragma unroll
        for (int r = c + 1; r < D; ++r) {
            if (piv[c] == r) { const double t = b[c]; b[c] = b[r]; b[r] = t; }
        }
    }
#pragma unroll
    for (int r = 0; r < D; ++r) {
#pragma unroll
        for (int k = 0; k < r; ++k) b[r] = fma(-A[r][k], b[k], b[r]);
    }
#pragma unroll
    for (int r = D - 1; r >= 0; --r) {
#pragma unroll
        for (int k = r + 1; k < D; ++k) b[r] = fma(-A[r][k], b[k], b[r]);
        b[r] *= rd[r];
    }
}

// Residual correction of the ill-conditioned centres (near-degenerate
// generators; condition estimate above 1e6), after the search: r = b - A rho
// with the exact rows and right-hand sides in double-double, then A delta = r
// with the FP64 factors, twice -- the double-double residual step of the
// reference's high-precision vertex correction (src/raycast.jl:633-707).  Only
// the output coordinates need it: the search itself decides from the signature.
template <int D>
__global__ void __launch_bounds__(128) k_refine_centers(DevMesh M, unsigned V) {
    for (unsigned v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        if (!(M.vcond[v] > 1e6f)) continue;
        int s[D + 1];
#pragma unroll
        for (int k = 0; k <= D; ++k) s[k] = M.vsig[(size_t)v * (D + 1) + k];
        double xa[D], A[D][D], rho[D];
#pragma unroll
        for (int k = 0; k < D; ++k) xa[k] = M.pts[(size_t)s[0] * D + k];
#pragma unroll
        for (int r = 0; r < D; ++r) con_row<D, double>(M, xa, s[r + 1], A[r], rho[r]);
        int piv[D];
        double rd[D];
        if (!lu_factor_rcp<D>(A, piv, rd)) continue;
        lu_solve_rcp<D>(A, piv, rd, rho);
#pragma unroll 1
        for (int it = 0; it < 2; ++it) {
            double r[D];
#pragma unroll
            for (int row = 0; row < D; ++row) {
                dd rw[D], rh;
                con_row<D, dd>(M, xa, s[row + 1], rw, rh);
#pragma unroll
                for (int k = 0; k < D; ++k) rh = rh - rw[k] * mk(rho[k]);
                r[row] = rh.hi + rh.lo;
            }
            lu_solve_rcp<D>(A, piv, rd, r);
#pragma unroll
            for (int k = 0; k < D; ++k) rho[k] += r[k];
        }
#pragma unroll
        for (int k = 0; k < D; ++k) M.vc[(size_t)v * D + k] = xa[k] + rho[k];
    }
}

template <int D>
__global__ void __launch_bounds__(128) k_centers(DevMesh M, unsigned v0, unsigned v1) {
    constexpr int DP = (D <= 4) ? 4 : 8;
    if (M.G.lvl) { v0 = M.G.lvl[0]; v1 = M.G.lvl[1]; }
    for (unsigned v = v0 + blockIdx.x * blockDim.x + threadIdx.x; v < v1; v += gridDim.x * blockDim.x) {
        int s[D + 1];
#pragma unroll
        for (int k = 0; k <= D; ++k) s[k] = M.vsig[(size_t)v * (D + 1) + k];
        double xa[D], A[D][D], rho[D];
        const double* pa = M.pts + (size_t)s[0] * D;
#pragma unroll
        for (int k = 0; k < D; ++k) xa[k] = __ldg(pa + k);
#pragma unroll
        for (int r = 0; r < D; ++r) con_row<D, double>(M, xa, s[r + 1], A[r], rho[r]);
        int piv[D];
        double rd[D];
        const bool ok = lu_factor_rcp<D>(A, piv, rd);
        if (!ok) {
            set_status(M, ST_NUMERIC);
#pragma unroll
            for (int k = 0; k < D; ++k) rho[k] = 0.0;
        } else {
            lu_solve_rcp<D>(A, piv, rd, rho);
        }
        float r32[DP];
#pragma unroll
        for (int k = 0; k < DP; ++k) r32[k] = 0.f;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            M.vc[(size_t)v * D + k] = xa[k] + rho[k];
            r32[k] = (float)rho[k];
        }
        float4* dst = reinterpret_cast<float4*>(M.vrho32 + (size_t)v * DP);
#pragma unroll
        for (int h = 0; h < DP / 4; ++h) dst[h] = make_float4(r32[4 * h], r32[4 * h + 1], r32[4 * h + 2], r32[4 * h + 3]);
        if (M.vinv32) {
            // FP64 inverse, rounded once to FP32: every ray direction of the vertex.
            // A^-1 = U^-1 L^-1 P: column j of U^-1 L^-1 (L^-1 unit lower triangular,
            // its column j zero above j) is column idx[j] of A^-1, idx = the row
            // order after the pivoting swaps -- fewer FP64 operations than D full
            // solves with unit vectors.
            int idx[D];
#pragma unroll
            for (int k = 0; k < D; ++k) idx[k] = k;
#pragma unroll
            for (int c = 0; c < D; ++c) {
#pragma unroll
                for (int r = c + 1; r < D; ++r)
                    if (piv[c] == r) { const int t = idx[c]; idx[c] = idx[r]; idx[r] = t; }
            }
            float rows[D];  // row sums of |A^-1| (condition estimate; FP32 suffices)
#pragma unroll
            for (int k = 0; k < D; ++k) rows[k] = 0.f;
            float* out = M.vinv32 + (size_t)v * D * D;
#pragma unroll
            for (int j = 0; j < D; ++j) {
                double x[D];
#pragma unroll
                for (int r = 0; r < D; ++r) {
                    if (r < j) x[r] = 0.0;
                    else if (r == j) x[r] = 1.0;
                    else {
                        double y = -A[r][j];
#pragma unroll
                        for (int k = j + 1; k < r; ++k) y = fma(-A[r][k], x[k], y);
                        x[r] = y;
                    }
                }
#pragma unroll
                for (int r = D - 1; r >= 0; --r) {
                    double y = x[r];
#pragma unroll
                    for (int k = r + 1; k < D; ++k) y = fma(-A[r][k], x[k], y);
                    x[r] = y * rd[r];
                }
                const int c = idx[j];
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    const float f = ok ? (float)x[k] : (k == c ? 1.f : 0.f);
                    out[k * D + c] = f;
                    rows[k] += fabsf(f);
                }
            }
            float ninv = 0.f;
#pragma unroll
            for (int k = 0; k < D; ++k) ninv = fmaxf(ninv, rows[k]);
            // infinity norm of A from the FP32 split coordinates (the estimate only)
            float nrm = 0.f;
            {
                float xa32[DP], xal32[DP];
                const float4* p = reinterpret_cast<const float4*>(M.pts32 + (size_t)s[0] * DP);
                const float4* pl = reinterpret_cast<const float4*>(M.pts32lo + (size_t)s[0] * DP);
#pragma unroll
                for (int h = 0; h < DP / 4; ++h) {
                    const float4 f = __ldg(p + h), g = __ldg(pl + h);
                    xa32[4 * h] = f.x; xa32[4 * h + 1] = f.y; xa32[4 * h + 2] = f.z; xa32[4 * h + 3] = f.w;
                    xal32[4 * h] = g.x; xal32[4 * h + 1] = g.y; xal32[4 * h + 2] = g.z; xal32[4 * h + 3] = g.w;
                }
#pragma unroll
                for (int r = 0; r < D; ++r) {
                    const int it = s[r + 1];
                    float sr = 0.f;
                    if (it < M.n) {
                        const float4* q = reinterpret_cast<const float4*>(M.pts32 + (size_t)it * DP);
                        const float4* ql = reinterpret_cast<const float4*>(M.pts32lo + (size_t)it * DP);
                        float xg[DP], xgl[DP];
#pragma unroll
                        for (int h = 0; h < DP / 4; ++h) {
                            const float4 f = __ldg(q + h), g = __ldg(ql + h);
                            xg[4 * h] = f.x; xg[4 * h + 1] = f.y; xg[4 * h + 2] = f.z; xg[4 * h + 3] = f.w;
                            xgl[4 * h] = g.x; xgl[4 * h + 1] = g.y; xgl[4 * h + 2] = g.z; xgl[4 * h + 3] = g.w;
                        }
#pragma unroll
                        for (int k = 0; k < D; ++k) sr += fabsf((xg[k] - xa32[k]) + (xgl[k] - xal32[k]));
                    } else {
                        const DevPlane& P = M.planes[it - M.n];
#pragma unroll
                        for (int k = 0; k < D; ++k) sr += fabsf(P.n32[k]);
                    }
                    nrm = fmaxf(nrm, sr);
                }
            }
            M.vcond[v] = ok ? nrm * ninv * 1.0001f : INFINITY;
        }
    }
}

// ---------------------------------------------------------------------------
// fast kernel: one warp expands one vertex entirely in FP32
// ---------------------------------------------------------------------------
// FP32 crossing of boundary plane P by the ray from c0 = xa + (xal + rho) along
// u, as the interval [lo, hi] of its parameter; false if the ray moves away
// from the plane.  Cuboid faces use the single coordinate; other planes bound
// the rounding of the split coordinates, of the FP32 copies of n and off and of
// the dot products.
// Parameter interval [lo, hi] of the crossing num / uk given the absolute
// error bounds of both; false if the ray moves away from the plane.
__device__ __forceinline__ bool crossing32(float num, float e_num, float uk, float e_den, float& lo, float& hi) {
    const float S32 = 5.9604645e-08f;
    if (uk > e_den) {
        const float t = __fdividef(num, uk);
        const float et = __fdividef(e_num + fabsf(t) * e_den, uk - e_den) * 1.00001f + 8.f * S32 * fabsf(t);
        lo = t - et; hi = t + et;
    } else if (uk < -e_den) {
        return false;
    } else {
        if (num - e_num > 0.f) { lo = __fdividef(num - e_num, fabsf(uk) + e_den) * 0.99999f; hi = INFINITY; }
        else { lo = -INFINITY; hi = INFINITY; }
    }
    return true;
}

template <int D>
__device__ __forceinline__ bool plane32(const DevPlane& P, const float* xa, const float* xal, const float* rho,
                                        const float* u, float erho, float relu, float TINY, float& lo, float& hi) {
    const float S32 = 5.9604645e-08f;
    float num, e_num, uk, e_den;
    if (P.axis >= 0) {  // n = +-e_k: the dot products are exact
        float nc = 0.f, ac = 0.f;
        uk = 0.f;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            nc = fmaf(P.n32[k], xa[k] + (xal[k] + rho[k]), nc);
            uk = fmaf(P.n32[k], u[k], uk);
            ac += fabsf(P.n32[k]) * (fabsf(xa[k]) + fabsf(rho[k]));
        }
        num = P.off32 - nc;
        e_num = 4.f * S32 * (fabsf(P.off32) + ac) + erho + TINY;
        e_den = relu + 2.f * S32 * fabsf(uk);
    } else {
        float nc = 0.f, nu = 0.f, an = 0.f, anc = 0.f, anu = 0.f;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            const float ck = xa[k] + (xal[k] + rho[k]);
            nc = fmaf(P.n32[k], ck, nc);
            nu = fmaf(P.n32[k], u[k], nu);
            an += fabsf(P.n32[k]);
            anc += fabsf(P.n32[k]) * (fabsf(xa[k]) + fabsf(rho[k]));
            anu += fabsf(P.n32[k] * u[k]);
        }
        num = P.off32 - nc;
        uk = nu;
        e_num = (2.f * D + 8.f) * S32 * (fabsf(P.off32) + anc) + erho * an + TINY;
        e_den = relu * an + (D + 4.f) * S32 * anu;
    }
    return crossing32(num, e_num, uk, e_den, lo, hi);
}

// Cuboid face p (2k upper, 2k+1 lower) with p known at compile time after
// unrolling: one coordinate, bounds from the kernel parameters.
template <int D>
__device__ __forceinline__ bool box32(const DevMesh& M, int p, const float* xa, const float* xal, const float* rho,
                                      const float* u, float erho, float relu, float TINY, float& lo, float& hi) {
    const float S32 = 5.9604645e-08f;
    const int k = p >> 1;
    const bool upper = (p & 1) == 0;
    const float uk = upper ? u[k] : -u[k];
    const float hk = M.hi32[k], lk = M.lo32[k];
    const float ck = xa[k] + (xal[k] + rho[k]);
    const float num = upper ? (hk - ck) : (ck - lk);
    const float e_num = 4.f * S32 * (fabsf(hk) + fabsf(lk) + fabsf(xa[k]) + fabsf(rho[k])) + erho + TINY;
    const float e_den = relu + 2.f * S32 * fabsf(uk);
    return crossing32(num, e_num, uk, e_den, lo, hi);
}

// Visits every boundary plane not excluded by excl(item) whose FP32 crossing
// interval exists: f(item, lo, hi).  Cuboid domains unroll over their 2D faces.
template <int D, class Excl, class F>
__device__ __forceinline__ void planes32(const DevMesh& M, const float* xa, const float* xal, const float* rho,
                                         const float* u, float erho, float relu, float TINY, Excl&& excl, F&& f) {
    if (M.box) {
#pragma unroll
        for (int p = 0; p < 2 * D; ++p) {
            const int it = M.n + p;
            if (excl(it)) continue;
            float lo, hi;
            if (!box32<D>(M, p, xa, xal, rho, u, erho, relu, TINY, lo, hi)) continue;
            f(it, lo, hi);
        }
    } else {
#pragma unroll 1
        for (int p = 0; p < M.np; ++p) {
            const int it = M.n + p;
            if (excl(it)) continue;
            float lo, hi;
            if (!plane32<D>(M.planes[p], xa, xal, rho, u, erho, relu, TINY, lo, hi)) continue;
            f(it, lo, hi);
        }
    }
}

// Parameter interval [lo, hi] of a candidate's crossing t = num / den from the
// error bounds of both; false if the ray moves away from the candidate.
__device__ __forceinline__ bool cand_t32(float num, float e_num, float den, float e_den, float& lo, float& hi) {
    const float S32 = 5.9604645e-08f;
    if (den > e_den) {
        const float r = __fdividef(1.f, den);
        const float t = num * r;
        float et;
        if (e_den < 1e-3f * den) et = (e_num + fabsf(t) * e_den) * r * 1.0021f;
        else et = __fdividef(e_num + fabsf(t) * e_den, den - e_den) * 1.00001f;
        et += 8.f * S32 * fabsf(t);
        lo = t - et; hi = t + et;
        return true;
    }
    if (den < -e_den) return false;
    if (num - e_num > 0.f) {
        if (!(den + e_den > 0.f)) return false;
        lo = __fdividef(num - e_num, den + e_den) * 0.99999f; hi = INFINITY;
    } else {
        lo = -INFINITY; hi = INFINITY;
    }
    return true;
}

constexpr int FAST_WPB = 4;  // warps per block
// Candidate records in shared memory (D + 4 words per candidate and warp) for
// d <= 5; in 6D (lists of 384) they would cost more resident warps than the
// shared pass saves: there each pass over the list meets two open rays (the
// list read once per pass, not once per ray: 6D/10k expansion 59 -> 48 ms).
__host__ __device__ constexpr bool fast_staged(int d) { return d <= 5; }
inline size_t fast_smem_bytes(int d, int K) {
    return fast_staged(d) ? (size_t)FAST_WPB * (d + 4) * (K > 0 ? K : 1) * sizeof(float) : 0;
}

template <int D>
__device__ __forceinline__ void load_pt32(const DevMesh& M, int j, float (&x)[(D <= 4) ? 4 : 8]) {
    constexpr int DP = (D <= 4) ? 4 : 8;
    const float4* p = reinterpret_cast<const float4*>(M.pts32 + (size_t)j * DP);
#pragma unroll
    for (int h = 0; h < DP / 4; ++h) {
        float4 f = __ldg(p + h);
        x[4 * h] = f.x; x[4 * h + 1] = f.y; x[4 * h + 2] = f.z; x[4 * h + 3] = f.w;
    }
}

template <int D>
__device__ __forceinline__ void load_pt32lo(const DevMesh& M, int j, float (&x)[(D <= 4) ? 4 : 8]) {
    constexpr int DP = (D <= 4) ? 4 : 8;
    const float4* p = reinterpret_cast<const float4*>(M.pts32lo + (size_t)j * DP);
#pragma unroll
    for (int h = 0; h < DP / 4; ++h) {
        float4 f = __ldg(p + h);
        x[4 * h] = f.x; x[4 * h + 1] = f.y; x[4 * h + 2] = f.z; x[4 * h + 3] = f.w;
    }
}

// 8 resident blocks (64 registers, 32 warps per SM) for d <= 4, whose records
// leave room for them in shared memory; 6 for d >= 5 (5D records allow 5
// blocks; the 6D kernel would spill at 64 registers).
template <int D>
__global__ void __launch_bounds__(FAST_WPB * 32, D <= 4 ? 8 : 6) k_expand_fast(DevMesh M, unsigned f0, unsigned f1,
                                                               unsigned long long* fq, unsigned* nfq,
                                                               unsigned fqcap, unsigned long long* fx,
                                                               unsigned* nfx, unsigned fxcap) {
    constexpr int R = D + 1;
    constexpr int DP = (D <= 4) ? 4 : 8;
    __shared__ float sInv[FAST_WPB][D][D];
    __shared__ float sU[FAST_WPB][R][D];
    __shared__ float sLam[FAST_WPB][R];
    __shared__ float sLb[FAST_WPB][R];
    __shared__ float sU1[FAST_WPB][R];
    __shared__ float sRlo1[FAST_WPB][R], sRhi1[FAST_WPB][R], sRlo2[FAST_WPB][R];
    __shared__ int sRj1[FAST_WPB][R];
    __shared__ float sCond[FAST_WPB];
    __shared__ float sDb[FAST_WPB][D];  // x_b - x_a of the edge that drops the anchor (ray 0)
    extern __shared__ float sCand[];  // FAST_WPB x CW x K candidate records
    constexpr int CW = D + 4;
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned FULL = 0xFFFFFFFFu;
    float* fqh = M.fqh;
    if (M.G.lvl) {  // graph-driven levels: this level's range and queues
        f0 = M.G.lvl[0];
        f1 = M.G.lvl[1];
        const int p = M.G.lvl[2] & 1;
        fq = M.G.fq[p]; nfq = M.G.qc + 2 * p;
        fx = M.G.fx[p]; nfx = M.G.qc + 2 * p + 1;
        fqh = M.G.fqh[p];
    }
    const unsigned nf = f1 - f0;
    const float S32 = 5.9604645e-08f;                          // 2^-24
    for (unsigned w = blockIdx.x * FAST_WPB + wib; w < nf; w += gridDim.x * FAST_WPB) {
        const unsigned v = f0 + w;
        int sig[R];
#pragma unroll
        for (int k = 0; k < R; ++k) sig[k] = M.vsig[(size_t)v * R + k];
        const int vnew = M.vnew[v];
        // ---- open rays first: a vertex whose edges are all walked or closed costs no more
        int active = 0;
        if (lane < R) {
            active = walkable<D>(M, sig, vnew, lane) ? 1 : 0;
            if (active && M.ecnt && ((M.ecnt[v] >> lane) & 1u)) active = 0;  // both end points known
        }
        if (__ballot_sync(FULL, active) == 0u) continue;
        const int a = sig[0];
        float xa[DP], xal[DP], rho[DP];
        load_pt32<D>(M, a, xa);
        load_pt32lo<D>(M, a, xal);
        {
            const float4* pr = reinterpret_cast<const float4*>(M.vrho32 + (size_t)v * DP);
#pragma unroll
            for (int h = 0; h < DP / 4; ++h) {
                float4 f = pr[h];
                rho[4 * h] = f.x; rho[4 * h + 1] = f.y; rho[4 * h + 2] = f.z; rho[4 * h + 3] = f.w;
            }
        }
        // ---- the vertex's inverse (FP64 solve rounded to FP32, written by k_centers)
        for (int x = lane; x < D * D; x += 32) (&sInv[wib][0][0])[x] = M.vinv32[(size_t)v * D * D + x];
        if (lane == 0) sCond[wib] = M.vcond[v];
        __syncwarp();
        // ---- ray directions (lane m < R)
        if (lane < R) {
            const int m = lane;
            if (active) {
                float u[D], db[D];
#pragma unroll
                for (int k = 0; k < D; ++k) { u[k] = 0.f; db[k] = 0.f; }
                if (m >= 1) {
#pragma unroll
                    for (int k = 0; k < D; ++k) u[k] = -sInv[wib][k][m - 1];
                } else {
                    int b = -1;
#pragma unroll
                    for (int c = 0; c < D; ++c) {
                        if (sig[c + 1] < M.n) {
#pragma unroll
                            for (int k = 0; k < D; ++k) u[k] += sInv[wib][k][c];
                            if (b < 0) b = sig[c + 1];
                        }
                    }
                    float xb[DP], xbl[DP];
                    load_pt32<D>(M, b, xb);
                    load_pt32lo<D>(M, b, xbl);
#pragma unroll
                    for (int k = 0; k < D; ++k) { db[k] = (xb[k] - xa[k]) + (xbl[k] - xal[k]); sDb[wib][k] = db[k]; }
                }
                float nu = 0.f;
#pragma unroll
                for (int k = 0; k < D; ++k) nu = fmaf(u[k], u[k], nu);
                nu = rsqrtf(nu);
                float lam = 0.f, lb = 0.f;
#pragma unroll
                for (int k = 0; k < D; ++k) { u[k] *= nu; lam = fmaf(u[k], db[k], lam); lb += fabsf(db[k]); sU[wib][m][k] = u[k]; }
                sLam[wib][m] = lam;
                sLb[wib][m] = lb;
            }
        }
        const unsigned rmask = __ballot_sync(FULL, active) & ((1u << R) - 1u);
        __syncwarp();
        const float cond = sCond[wib];
        // directions come from the FP64 inverse rounded to FP32: relative error
        // (2D+6) 2^-24 from the rounding and normalisation, plus the FP64
        // solve's own error ~ D cond 2^-53
        const float relu = (2.f * D + 6.f) * S32 + 8.f * D * cond * 1.1102230e-16f;
        if (!(cond < 1e7f)) {  // too ill-conditioned for an FP32 decision: all rays exact
            if (lane < R && active) {
                count_add(M.cnt + C_RAYS);
                const unsigned slot = atomicAdd(nfx, 1u);
                if (slot < fxcap) fx[slot] = ((unsigned long long)v << 4) | (unsigned)lane;
                else set_status(M, ST_QUEUE);
            }
            continue;
        }
        float R1 = 0.f, rmax = 0.f;
#pragma unroll
        for (int k = 0; k < D; ++k) { R1 += fabsf(rho[k]); rmax = fmaxf(rmax, fabsf(rho[k])); }
        const float erho = 2.f * S32 * rmax;  // rho is the rounded FP64 centre offset
        // |u|_1 of every open ray (error bound of its denominators)
        if (lane < R && ((rmask >> lane) & 1u)) {
            float a1 = 0.f;
#pragma unroll
            for (int k = 0; k < D; ++k) a1 += fabsf(sU[wib][lane][k]);
            sU1[wib][lane] = a1;
        }
        __syncwarp();
        const float CN = (4.f * D + 20.f) * S32, CD = (4.f * D + 16.f) * S32;
        const float TINY = M.tiny32;
        const int K = M.K;
        // candidate list: the real generator of the vertex with the largest
        // complete radius (every generator is on the current sphere, so any
        // of their lists covers the same neighbourhood; the widest one makes
        // the security test pass most often)
        int own = a;
        float sec_own = -1.f;
        {
            float sv = -1.f;
            int it = -1;
            if (lane < R && sig[lane < R ? lane : 0] < M.n) { it = sig[lane]; sv = __ldg(M.sec + it); }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const float osv = __shfl_xor_sync(FULL, sv, off);
                const int oit = __shfl_xor_sync(FULL, it, off);
                if (osv > sv || (osv == sv && oit >= 0 && (it < 0 || oit < it))) { sv = osv; it = oit; }
            }
            own = it;
            sec_own = sv;
        }
        const int* lst = M.knn + (size_t)own * K;
        float dow[D];  // x_own - x_a (split coordinates), for the security tests
        {
            float xo[DP], xol[DP];
            load_pt32<D>(M, own, xo);
            load_pt32lo<D>(M, own, xol);
#pragma unroll
            for (int k = 0; k < D; ++k) dow[k] = (xo[k] - xa[k]) + (xol[k] - xal[k]);
        }
        // ---- the candidates' ray-independent quantities, once per vertex, into this
        // warp's records (structure of arrays; lane c owns entries c, c+32, ...):
        // dl = x_j - x_a (split), A1 = |dl|_1, num = |dl|^2 - 2 dl.rho and its error
        // bound; item -1 marks a generator of the vertex (on the sphere)
        float* cr = sCand + (size_t)wib * CW * K;
        if constexpr (fast_staged(D)) {
            int jn = lane < K ? __ldg(lst + lane) : -1;
            int jnn = lane + 32 < K ? __ldg(lst + lane + 32) : -1;
            float xn[DP], xnl[DP];
#pragma unroll
            for (int k = 0; k < DP; ++k) { xn[k] = 0.f; xnl[k] = 0.f; }
            if (jn >= 0) { load_pt32<D>(M, jn, xn); load_pt32lo<D>(M, jn, xnl); }
            for (int c = lane; c < K; c += 32) {
                int j = jn;
                float xj[DP], xjl[DP];
#pragma unroll
                for (int k = 0; k < DP; ++k) { xj[k] = xn[k]; xjl[k] = xnl[k]; }
                jn = jnn;
                jnn = c + 64 < K ? __ldg(lst + c + 64) : -1;
                if (jn >= 0) { load_pt32<D>(M, jn, xn); load_pt32lo<D>(M, jn, xnl); }
                bool skip = j < 0;
#pragma unroll
                for (int q = 0; q < R; ++q) skip |= (j == sig[q]);
                float A1 = 0.f, A2 = 0.f, A3 = 0.f, dr = 0.f;
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    const float dl = (xj[k] - xa[k]) + (xjl[k] - xal[k]);
                    A1 += fabsf(dl);
                    A2 = fmaf(dl, dl, A2);
                    A3 = fmaf(fabsf(dl), fabsf(rho[k]), A3);
                    dr = fmaf(dl, rho[k], dr);
                    cr[k * K + c] = dl;
                }
                cr[D * K + c] = A1;
                cr[(D + 1) * K + c] = fmaf(-2.f, dr, A2);
                cr[(D + 2) * K + c] = CN * (A2 + 2.f * A3) + 2.f * A1 * erho + TINY * (A1 + R1);
                cr[(D + 3) * K + c] = __int_as_float(skip ? -1 : j);
            }
        }
        if constexpr (!fast_staged(D)) {
            // ---- 6D: passes over the candidate list, each for two open rays (the list is
            // read once per pass instead of once per ray)
            unsigned todo = rmask;
            while (todo) {
                int mr[2];
                mr[0] = __ffs(todo) - 1;
                todo &= todo - 1;
                mr[1] = todo ? __ffs(todo) - 1 : -1;
                if (todo) todo &= todo - 1;
                const int nr = mr[1] >= 0 ? 2 : 1;
                float eden[2], lmq[2];
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int m = q < nr ? mr[q] : mr[0];
                    lmq[q] = sLam[wib][m];
                    eden[q] = CD * fabsf(lmq[q]) + 2.f * relu * sLb[wib][m] + TINY * sU1[wib][m];
                }
                float lo1[2], hi1[2], lo2[2];
                int j1[2];
#pragma unroll
                for (int q = 0; q < 2; ++q) { lo1[q] = INFINITY; hi1[q] = INFINITY; lo2[q] = INFINITY; j1[q] = -1; }
                int jn = lane < K ? __ldg(lst + lane) : -1;
                int jnn = lane + 32 < K ? __ldg(lst + lane + 32) : -1;
                float xn[DP], xnl[DP];
#pragma unroll
                for (int k = 0; k < DP; ++k) { xn[k] = 0.f; xnl[k] = 0.f; }
                if (jn >= 0) { load_pt32<D>(M, jn, xn); load_pt32lo<D>(M, jn, xnl); }
                for (int c = lane; c < K; c += 32) {
                    const int j = jn;
                    float xj[DP], xjl[DP];
#pragma unroll
                    for (int k = 0; k < DP; ++k) { xj[k] = xn[k]; xjl[k] = xnl[k]; }
                    jn = jnn;
                    jnn = c + 64 < K ? __ldg(lst + c + 64) : -1;
                    if (jn >= 0) { load_pt32<D>(M, jn, xn); load_pt32lo<D>(M, jn, xnl); }
                    if (j < 0) continue;
                    bool insig = false;
#pragma unroll
                    for (int q = 0; q < R; ++q) insig |= (j == sig[q]);
                    if (insig) continue;
                    float dl[D], A1 = 0.f, A2 = 0.f, A3 = 0.f, dr = 0.f;
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        dl[k] = (xj[k] - xa[k]) + (xjl[k] - xal[k]);
                        A1 += fabsf(dl[k]);
                        A2 = fmaf(dl[k], dl[k], A2);
                        A3 = fmaf(fabsf(dl[k]), fabsf(rho[k]), A3);
                        dr = fmaf(dl[k], rho[k], dr);
                    }
                    const float num = fmaf(-2.f, dr, A2);
                    const float e_num = CN * (A2 + 2.f * A3) + 2.f * A1 * erho + TINY * (A1 + R1);
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        if (q >= nr) break;
                        const int m = mr[q];
                        float du = 0.f, B = 0.f;
#pragma unroll
                        for (int k = 0; k < D; ++k) {
                            const float um = sU[wib][m][k];
                            du = fmaf(dl[k], um, du);
                            B = fmaf(fabsf(dl[k]), fabsf(um), B);
                        }
                        float lo, hi;
                        if (!cand_t32(num, e_num, 2.f * (du - lmq[q]), CD * B + 2.f * relu * A1 + eden[q], lo, hi))
                            continue;
                        if (lo < lo1[q] || (lo == lo1[q] && j < j1[q])) { lo2[q] = lo1[q]; lo1[q] = lo; hi1[q] = hi; j1[q] = j; }
                        else if (lo < lo2[q]) lo2[q] = lo;
                    }
                }
#pragma unroll
                for (int q = 0; q < 2; ++q) {
                    if (q >= nr) break;
                    float l1 = lo1[q], h1 = hi1[q], l2 = lo2[q];
                    int jj = j1[q];
#pragma unroll
                    for (int off = 16; off > 0; off >>= 1) {
                        const float olo1 = __shfl_xor_sync(FULL, l1, off);
                        const float ohi1 = __shfl_xor_sync(FULL, h1, off);
                        const float olo2 = __shfl_xor_sync(FULL, l2, off);
                        const int oj1 = __shfl_xor_sync(FULL, jj, off);
                        const bool take = (olo1 < l1) || (olo1 == l1 && oj1 >= 0 && (jj < 0 || oj1 < jj));
                        if (take) { l2 = fminf(l1, olo2); l1 = olo1; h1 = ohi1; jj = oj1; }
                        else { l2 = fminf(l2, olo1); }
                    }
                    if (lane == 0) {
                        const int m = mr[q];
                        sRlo1[wib][m] = l1; sRhi1[wib][m] = h1; sRlo2[wib][m] = l2; sRj1[wib][m] = jj;
                    }
                }
            }
        } else {
        // ---- one pass over the records per open ray (the lane reads back only its own
        // entries: no synchronisation needed)
        unsigned todo = rmask;
        while (todo) {
            const int m = __ffs(todo) - 1;
            todo &= todo - 1;
            float um[D];
#pragma unroll
            for (int k = 0; k < D; ++k) um[k] = sU[wib][m][k];
            const float lm = sLam[wib][m], lbm = sLb[wib][m], u1m = sU1[wib][m];
            const float eden0 = CD * fabsf(lm) + 2.f * relu * lbm + TINY * u1m;
            float lo1 = INFINITY, hi1 = INFINITY, lo2 = INFINITY;
            int j1 = -1;
            if constexpr (!fast_staged(D)) {
                // software pipeline: list entries two iterations ahead, coordinates one ahead
                int jn = lane < K ? __ldg(lst + lane) : -1;
                int jnn = lane + 32 < K ? __ldg(lst + lane + 32) : -1;
                float xn[DP], xnl[DP];
#pragma unroll
                for (int k = 0; k < DP; ++k) { xn[k] = 0.f; xnl[k] = 0.f; }
                if (jn >= 0) { load_pt32<D>(M, jn, xn); load_pt32lo<D>(M, jn, xnl); }
                for (int c = lane; c < K; c += 32) {
                    const int j = jn;
                    float xj[DP], xjl[DP];
#pragma unroll
                    for (int k = 0; k < DP; ++k) { xj[k] = xn[k]; xjl[k] = xnl[k]; }
                    jn = jnn;
                    jnn = c + 64 < K ? __ldg(lst + c + 64) : -1;
                    if (jn >= 0) { load_pt32<D>(M, jn, xn); load_pt32lo<D>(M, jn, xnl); }
                    if (j < 0) continue;
                    bool insig = false;
#pragma unroll
                    for (int q = 0; q < R; ++q) insig |= (j == sig[q]);
                    if (insig) continue;
                    float A1 = 0.f, A2 = 0.f, A3 = 0.f, dr = 0.f, du = 0.f, B = 0.f;
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        const float dl = (xj[k] - xa[k]) + (xjl[k] - xal[k]);
                        A1 += fabsf(dl);
                        A2 = fmaf(dl, dl, A2);
                        A3 = fmaf(fabsf(dl), fabsf(rho[k]), A3);
                        dr = fmaf(dl, rho[k], dr);
                        du = fmaf(dl, um[k], du);
                        B = fmaf(fabsf(dl), fabsf(um[k]), B);
                    }
                    const float num = fmaf(-2.f, dr, A2);
                    const float e_num = CN * (A2 + 2.f * A3) + 2.f * A1 * erho + TINY * (A1 + R1);
                    float lo, hi;
                    if (!cand_t32(num, e_num, 2.f * (du - lm), CD * B + 2.f * relu * A1 + eden0, lo, hi)) continue;
                    if (lo < lo1 || (lo == lo1 && j < j1)) { lo2 = lo1; lo1 = lo; hi1 = hi; j1 = j; }
                    else if (lo < lo2) lo2 = lo;
                }
            } else {
                for (int c = lane; c < K; c += 32) {
                    const int j = __float_as_int(cr[(D + 3) * K + c]);
                    if (j < 0) continue;
                    float du = 0.f, B = 0.f;
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        const float dl = cr[k * K + c];
                        du = fmaf(dl, um[k], du);
                        B = fmaf(fabsf(dl), fabsf(um[k]), B);
                    }
                    const float A1 = cr[D * K + c];
                    const float num = cr[(D + 1) * K + c];
                    const float e_num = cr[(D + 2) * K + c];
                    float lo, hi;
                    if (!cand_t32(num, e_num, 2.f * (du - lm), CD * B + 2.f * relu * A1 + eden0, lo, hi)) continue;
                    if (lo < lo1 || (lo == lo1 && j < j1)) { lo2 = lo1; lo1 = lo; hi1 = hi; j1 = j; }
                    else if (lo < lo2) lo2 = lo;
                }
            }
            // warp reduction of the ray's top-2
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const float olo1 = __shfl_xor_sync(FULL, lo1, off);
                const float ohi1 = __shfl_xor_sync(FULL, hi1, off);
                const float olo2 = __shfl_xor_sync(FULL, lo2, off);
                const int oj1 = __shfl_xor_sync(FULL, j1, off);
                const bool take = (olo1 < lo1) || (olo1 == lo1 && oj1 >= 0 && (j1 < 0 || oj1 < j1));
                if (take) { lo2 = fminf(lo1, olo2); lo1 = olo1; hi1 = ohi1; j1 = oj1; }
                else { lo2 = fminf(lo2, olo1); }
            }
            if (lane == 0) { sRlo1[wib][m] = lo1; sRhi1[wib][m] = hi1; sRlo2[wib][m] = lo2; sRj1[wib][m] = j1; }
        }
        }
        __syncwarp();
        // In a cuboid, every face is at least bdist (its rounding bound emax
        // included) from the centre, so a crossing interval starts at t >=
        // bdist (1 - 1e-5) - 1e-5 emax: a ray whose best candidate ends well
        // below that cannot meet a face first, and neither its decision nor its
        // certification depends on the faces
        float bdist = -INFINITY, emax = 0.f;
        if (M.box) {
            bdist = INFINITY;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                const float ck = xa[k] + (xal[k] + rho[k]);
                const float hk = M.hi32[k], lk = M.lo32[k];
                const float e = 4.f * S32 * (fabsf(hk) + fabsf(lk) + fabsf(xa[k]) + fabsf(rho[k])) + erho + TINY;
                bdist = fminf(bdist, fminf(hk - ck, ck - lk) - e);
                emax = fmaxf(emax, e);
            }
        }
        // ---- per-ray decision on lane m
        int dwin = -1;  // winner of this lane's ray when decided here
        if (lane < R && ((rmask >> lane) & 1u)) {
            const int m = lane;
            count_add(M.cnt + C_RAYS);
            float u[D];
#pragma unroll
            for (int k = 0; k < D; ++k) u[k] = sU[wib][m][k];
            const float clo1 = sRlo1[wib][m], chi1 = sRhi1[wib][m], clo2 = sRlo2[wib][m];
            const int cj1 = sRj1[wib][m];
            // boundary planes in FP32 with the same error model
            float plo1 = INFINITY, phi1 = INFINITY, plo2 = INFINITY;
            int pj1 = -1;
            if (!(cj1 >= 0 && fmaf(1.02f, chi1, emax) < 0.98f * bdist)) planes32<D>(
                M, xa, xal, rho, u, erho, relu, TINY,
                [&](int it) {
                    bool ex = false;
#pragma unroll
                    for (int s = 0; s < R; ++s) ex |= (sig[s] == it);
                    return ex;
                },
                [&](int it, float lo, float hi) {
                    if (lo < plo1) { plo2 = plo1; plo1 = lo; phi1 = hi; pj1 = it; }
                    else if (lo < plo2) plo2 = lo;
                });
            int win;
            float blo, bhi, second;
            if (cj1 >= 0 && clo1 <= plo1) { win = cj1; blo = clo1; bhi = chi1; second = fminf(clo2, plo1); }
            else { win = pj1; blo = plo1; bhi = phi1; second = fminf(plo2, clo1); }
            const bool certified = (win >= 0) && (bhi < second);
            if (!certified) count_add(M.cnt + C_UNCERT);
            // security: the empty sphere at the winner's upper bound must lie inside the
            // complete radius of the list; then every generator outside the list has
            // t above that bound and the list holds every possible winner
            bool secure = false;
            if (win >= 0 && isfinite(bhi)) {
                const float t = certified ? 0.5f * (blo + bhi) : bhi;
                const float et = certified ? 0.5f * (bhi - blo) : 0.f;
                float c2 = 0.f, r2 = 0.f, cm = 0.f;
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    const float db = m == 0 ? sDb[wib][k] : 0.f;
                    const float cc = fmaf(t, u[k], rho[k]);
                    const float co = cc - dow[k];
                    c2 = fmaf(co, co, c2);
                    const float wv = db - cc;
                    r2 = fmaf(wv, wv, r2);
                    cm = fmaxf(cm, fabsf(cc));
                }
                const float ec = erho + fabsf(t) * relu + et + 4.f * S32 * (rmax + fabsf(t)) + 3.f * TINY;
                const float lhs = sqrtf(c2) + sqrtf(r2) + 4.f * sqrtf((float)D) * ec + 4.f * S32 * cm;
                secure = (t > 0.f) && (lhs < sec_own * (1.f - 1e-5f));
            }
            if (certified && !secure) count_add(M.cnt + C_INSECURE);
            if (!(certified && secure)) {
                // bit 3: the list holds every possible winner (no tree pass needed)
                const unsigned slot = atomicAdd(nfq, 1u);
                if (slot < fqcap) {
                    fq[slot] = ((unsigned long long)v << 4) | ((unsigned)secure << 3) | (unsigned)m;
                    if (fqh) fqh[slot] = win >= 0 ? bhi : INFINITY;
                } else {
                    set_status(M, ST_QUEUE);
                }
            } else {
                dwin = win;
            }
        }
        // decided rays: one range of the insert queue per warp, so the warp does not
        // wait on the vertex hash (k_insert_decided inserts them; a full queue is a
        // capacity retry like a full ray queue)
        const unsigned dm = __ballot_sync(FULL, dwin >= 0);
        if (dm) {
            unsigned base = 0;
            if (lane == 0) base = atomicAdd(M.ndq, (unsigned)__popc(dm));
            base = __shfl_sync(FULL, base, 0);
            if (dwin >= 0) {
                const unsigned slot = base + __popc(dm & ((1u << lane) - 1u));
                if (slot < M.dqcap) M.dq[slot] = make_uint2((v << 3) | (unsigned)lane, (unsigned)dwin);
                else set_status(M, ST_QUEUE);
            }
        }
        __syncwarp();
    }
}

// Vertex-hash inserts of the rays the expansion decided, one thread per ray:
// many inserts in flight hide the round trips of the claim, the id and the
// publication that a warp of the expansion would otherwise wait for.
template <int D>
__global__ void __launch_bounds__(256) k_insert_decided(DevMesh M) {
    const unsigned n = min(*M.ndq, M.dqcap);  // past the capacity: a capacity retry follows
    for (unsigned r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const uint2 e = M.dq[r];
        const unsigned v = e.x >> 3;
        int sig[D + 1];
#pragma unroll
        for (int k = 0; k <= D; ++k) sig[k] = M.vsig[(size_t)v * (D + 1) + k];
        int ns[D + 1];
        make_sig<D>(sig, (int)(e.x & 7u), (int)e.y, ns);
        bool is_new;
        vertex_insert<D>(M, ns, (int)e.y, is_new);
    }
}

// ---------------------------------------------------------------------------
// warp fallback: one warp per ray whose new sphere left the list's complete
// radius.  The ray is re-run in FP32 over the candidate list and then over
// the whole tree (warp-uniform traversal, one leaf point per lane), with the
// same per-candidate error bounds; the tree pass is exhaustive up to the
// conservative box test, so no security test is needed.  Rays that remain
// uncertified go to the FP64 kernel.
// ---------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void cand32(const DevMesh& M, int j, const float* xa, const float* xal, const float* rho,
                                       float R1, float erho, const float* u, float lam, float U1, float LB,
                                       float relu, float& lo, float& hi, bool& valid) {
    constexpr int DP = (D <= 4) ? 4 : 8;
    const float S32 = 5.9604645e-08f;
    const float CN = (4.f * D + 20.f) * S32, CD = (4.f * D + 16.f) * S32;
    const float TINY = M.tiny32;
    float xj[DP], xjl[DP];
    load_pt32<D>(M, j, xj);
    load_pt32lo<D>(M, j, xjl);
    float A1 = 0.f, A2 = 0.f, A3 = 0.f, dr = 0.f, du = 0.f, B = 0.f;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        const float dl = (xj[k] - xa[k]) + (xjl[k] - xal[k]);
        A1 += fabsf(dl);
        A2 = fmaf(dl, dl, A2);
        A3 = fmaf(fabsf(dl), fabsf(rho[k]), A3);
        dr = fmaf(dl, rho[k], dr);
        du = fmaf(dl, u[k], du);
        B = fmaf(fabsf(dl), fabsf(u[k]), B);
    }
    const float num = fmaf(-2.f, dr, A2);
    const float e_num = CN * (A2 + 2.f * A3) + 2.f * A1 * erho + TINY * (A1 + R1);
    const float den = 2.f * (du - lam);
    const float e_den = CD * (B + fabsf(lam)) + 2.f * relu * (A1 + LB) + TINY * U1;
    valid = true;
    if (den > e_den) {
        const float r = __fdividef(1.f, den);
        const float t = num * r;
        float et;
        if (e_den < 1e-3f * den) et = (e_num + fabsf(t) * e_den) * r * 1.0021f;
        else et = __fdividef(e_num + fabsf(t) * e_den, den - e_den) * 1.00001f;
        et += 8.f * S32 * fabsf(t);
        lo = t - et; hi = t + et;
    } else if (den < -e_den) {
        valid = false;
    } else if (num - e_num > 0.f) {
        if (!(den + e_den > 0.f)) { valid = false; return; }
        lo = __fdividef(num - e_num, den + e_den) * 0.99999f; hi = INFINITY;
    } else {
        lo = -INFINITY; hi = INFINITY;
    }
}

__device__ __forceinline__ void top2_merge(float& lo1, float& hi1, int& j1, float& lo2, float olo1, float ohi1,
                                           int oj1, float olo2) {
    // the same candidate met by two lanes (list and tree): one entry, not a rival
    if (oj1 >= 0 && oj1 == j1) { lo2 = fminf(lo2, olo2); return; }
    const bool take = (olo1 < lo1) || (olo1 == lo1 && oj1 >= 0 && (j1 < 0 || oj1 < j1));
    if (take) { lo2 = fminf(lo1, olo2); lo1 = olo1; hi1 = ohi1; j1 = oj1; }
    else { lo2 = fminf(lo2, olo1); }
}

__device__ __forceinline__ void top2_warp(float& lo1, float& hi1, int& j1, float& lo2) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float a = __shfl_xor_sync(0xFFFFFFFFu, lo1, off);
        const float b = __shfl_xor_sync(0xFFFFFFFFu, hi1, off);
        const float c = __shfl_xor_sync(0xFFFFFFFFu, lo2, off);
        const int e = __shfl_xor_sync(0xFFFFFFFFu, j1, off);
        top2_merge(lo1, hi1, j1, lo2, a, b, e, c);
    }
}

__device__ __forceinline__ void top2_add(float& lo1, float& hi1, int& j1, float& lo2, float lo, float hi, int j) {
    if (j == j1) return;
    if (lo < lo1 || (lo == lo1 && (j1 < 0 || j < j1))) { lo2 = lo1; lo1 = lo; hi1 = hi; j1 = j; }
    else if (lo < lo2) lo2 = lo;
}

constexpr int FB_WPB = 4;
constexpr int FB_AMB = 4;      // ambiguous candidates kept per lane
constexpr int FB_AMB_MAX = AMB_SET; // ambiguous set re-scored in FP64
constexpr int FB_STK = 1024;   // tree stack entries per warp
constexpr int FB_LQ = 64;      // queued leaves per warp

// FP64 decision of a walk restricted to the candidate set `items` (every
// possible winner is in it): forward-bounded FP64 first, double-double if the
// FP64 intervals still overlap.  Returns the winning item or -1.
template <int D>
__device__ int exact_decide_set(const DevMesh& M, const int (&sig)[D + 1], int m, const int* items, int nitems) {
    Query<D> q;
    if (!setup_walk<D>(M, sig, m, q)) return -1;
    SearchOut R;
    R.best = Cand{-1, INFINITY, INFINITY, INFINITY};
    R.second_lo = INFINITY;
    R.namb = 0;
    R.overflow = false;
    bool planes = false;
    for (int c = 0; c < nitems; ++c) {
        if (items[c] < M.n) eval_point<D>(M, q, items[c], R);
        else planes = true;
    }
    if (planes) eval_planes<D>(M, q, R);
    if (R.best.item < 0) return -1;
    if (R.best.hi < R.second_lo) return R.best.item;
    if (R.overflow) return -1;  // more near-ties than the set holds: the exact tree search decides
    count_add(M.cnt + C_DD);
    int its[HV_NAMB + 1];
    its[0] = R.best.item;
    int w = 1;
    for (int k = 0; k < R.namb; ++k)
        if (R.amb[k].lo <= R.best.hi) its[w++] = R.amb[k].item;
    bool degen = false;
    const int win = dd_rescore_walk<D>(M, sig, m, its, w, degen);
    if (degen) { count_add(M.cnt + C_DEGEN); set_status(M, ST_DEGEN); }
    return win;
}

template <int D>
__global__ void __launch_bounds__(FB_WPB * 32, 4) k_fallback_warp(DevMesh M, const unsigned long long* fq,
                                                               const unsigned* nfq, unsigned fqcap,
                                                               unsigned long long* fx, unsigned* nfx,
                                                               unsigned fxcap, AmbQueue aq) {
    constexpr int R = D + 1;
    constexpr int DP = (D <= 4) ? 4 : 8;
    __shared__ int sstack[FB_WPB][FB_STK];
    __shared__ int sleaf[FB_WPB][FB_LQ];
    __shared__ int scq[FB_WPB][64];
    __shared__ int samb[FB_WPB][FB_AMB_MAX];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned FULL = 0xFFFFFFFFu;
    const float S32 = 5.9604645e-08f;
    const float* fqh = M.fqh;
    if (M.G.lvl) {  // graph-driven levels: the queues of the previous level
        const int p = (M.G.lvl[2] + 1) & 1;
        fq = M.G.fq[p]; nfq = M.G.qc + 2 * p;
        fx = M.G.fx[p]; nfx = M.G.qc + 2 * p + 1;
        fqh = M.G.fqh[p];
    }
    const unsigned nq = min(*nfq, fqcap);
    int* stk = sstack[wib];
    int* lq = sleaf[wib];
    int* cq = scq[wib];
    for (unsigned w = blockIdx.x * FB_WPB + wib; w < nq; w += gridDim.x * FB_WPB) {
        const unsigned long long e = fq[w];
        const unsigned v = (unsigned)(e >> 4);
        const bool complete = ((e >> 3) & 1ull) != 0;
        const int m = (int)(e & 7);
        if (lane == 0) count_add(M.cnt + C_FALLBACK);
        int sig[R];
#pragma unroll
        for (int k = 0; k < R; ++k) sig[k] = M.vsig[(size_t)v * R + k];
        const int a = sig[0];
        float xa[DP], xal[DP], rho[DP];
        load_pt32<D>(M, a, xa);
        load_pt32lo<D>(M, a, xal);
        {
            const float4* pr = reinterpret_cast<const float4*>(M.vrho32 + (size_t)v * DP);
#pragma unroll
            for (int h = 0; h < DP / 4; ++h) {
                float4 f = pr[h];
                rho[4 * h] = f.x; rho[4 * h + 1] = f.y; rho[4 * h + 2] = f.z; rho[4 * h + 3] = f.w;
            }
        }
        const float* inv = M.vinv32 + (size_t)v * D * D;
        float u[D], db[D];
#pragma unroll
        for (int k = 0; k < D; ++k) { u[k] = 0.f; db[k] = 0.f; }
        if (m >= 1) {
#pragma unroll
            for (int k = 0; k < D; ++k) u[k] = -inv[k * D + (m - 1)];
        } else {
            int b = -1;
#pragma unroll
            for (int c = 0; c < D; ++c) {
                if (sig[c + 1] < M.n) {
#pragma unroll
                    for (int k = 0; k < D; ++k) u[k] += inv[k * D + c];
                    if (b < 0) b = sig[c + 1];
                }
            }
            float xb[DP], xbl[DP];
            load_pt32<D>(M, b, xb);
            load_pt32lo<D>(M, b, xbl);
#pragma unroll
            for (int k = 0; k < D; ++k) db[k] = (xb[k] - xa[k]) + (xbl[k] - xal[k]);
        }
        float nu = 0.f;
#pragma unroll
        for (int k = 0; k < D; ++k) nu = fmaf(u[k], u[k], nu);
        nu = rsqrtf(nu);
        float lam = 0.f, LB = 0.f, U1 = 0.f, R1 = 0.f, rmax = 0.f;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            u[k] *= nu;
            lam = fmaf(u[k], db[k], lam);
            LB += fabsf(db[k]);
            U1 += fabsf(u[k]);
            R1 += fabsf(rho[k]);
            rmax = fmaxf(rmax, fabsf(rho[k]));
        }
        const float cond = M.vcond[v];
        const float relu = (2.f * D + 6.f) * S32 + 8.f * D * cond * 1.1102230e-16f;
        const float erho = 2.f * S32 * rmax;
        // the list the fast kernel used: the signature's generator of widest radius
        int own = a;
        {
            float sv = -1.f;
            int it = -1;
            if (lane < R && sig[lane < R ? lane : 0] < M.n) { it = sig[lane]; sv = __ldg(M.sec + it); }
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const float osv = __shfl_xor_sync(FULL, sv, off);
                const int oit = __shfl_xor_sync(FULL, it, off);
                if (osv > sv || (osv == sv && oit >= 0 && (it < 0 || oit < it))) { sv = osv; it = oit; }
            }
            own = it;
        }
        float lo1 = INFINITY, hi1 = INFINITY, lo2 = INFINITY, H = INFINITY;
        int j1 = -1;
        int amb_j[FB_AMB];
        float amb_lo[FB_AMB];
        int namb = 0;
        bool amb_over = false;
        auto push_amb = [&](int j, float lo) {
            if (!(lo <= H)) return;
            if (namb == FB_AMB) {  // drop what the bound already excludes
                int w2 = 0;
                for (int q = 0; q < FB_AMB; ++q)
                    if (amb_lo[q] <= H) { amb_j[w2] = amb_j[q]; amb_lo[w2] = amb_lo[q]; ++w2; }
                namb = w2;
            }
            if (namb < FB_AMB) { amb_j[namb] = j; amb_lo[namb] = lo; ++namb; }
            else amb_over = true;
        };
        auto take = [&](int j, float lo, float hi) {
            H = fminf(H, hi);
            top2_add(lo1, hi1, j1, lo2, lo, hi, j);
            push_amb(j, lo);
        };
        // planes (lane 0)
        if (lane == 0) {
            const float TINY = M.tiny32;
            planes32<D>(
                M, xa, xal, rho, u, erho, relu, TINY,
                [&](int it) {
                    bool ex = false;
#pragma unroll
                    for (int q = 0; q < R; ++q) ex |= (sig[q] == it);
                    return ex;
                },
                [&](int it, float lo, float hi) { take(it, lo, hi); });
        }
        // the candidate list -- unless a tree pass follows and the expansion left a
        // finite bound: its best candidate's upper bound is then the starting bound,
        // and the exhaustive tree pass meets every list candidate inside that ball
        const float H0 = fqh ? fqh[w] : INFINITY;
        const bool list_pass = M.K > 0 && (complete || !isfinite(H0));
        if (!list_pass) H = fminf(H, H0);
        if (list_pass) {
            const int* lst = M.knn + (size_t)own * M.K;
            for (int c = lane; c < M.K; c += 32) {
                const int j = __ldg(lst + c);
                if (j < 0) continue;
                bool insig = false;
#pragma unroll
                for (int q = 0; q < R; ++q) insig |= (j == sig[q]);
                if (insig) continue;
                float lo, hi;
                bool ok;
                cand32<D>(M, j, xa, xal, rho, R1, erho, u, lam, U1, LB, relu, lo, hi, ok);
                if (ok) take(j, lo, hi);
            }
        }
        top2_warp(lo1, hi1, j1, lo2);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) H = fminf(H, __shfl_xor_sync(FULL, H, off));
        // exhaustive tree pass with the shrinking ball (only if the list may miss a winner):
        // up to 32 stack nodes are tested per step, one per lane; surviving leaves are
        // queued and evaluated 32 points at a time, after which the bound H shrinks
        bool overflow = false;
        if (!complete || M.K == 0) {
            long long nnodes = 0, nleaves_seen = 0, npoints_in = 0;
            // start at the (at most 32) nodes of depth min(5, log2 P): one step instead of five
            const int lv0 = min(5, 31 - __clz(M.P));
            int sp = 1 << lv0, nl = 0;
            if (lane < sp) stk[lane] = (1 << lv0) + lane;
            __syncwarp();
            const int L = M.leaf;
            const int lsh = (L & (L - 1)) == 0 ? __ffs(L) - 1 : -1;  // leaf size as a shift when a power of two
            while (sp > 0 || nl > 0) {
                if (nl >= 2 || (sp == 0 && nl > 0)) {
                    const int tot = nl * L;
                    nleaves_seen += nl;
                    // a point can beat the bound H only inside the ball of parameter H (the
                    // node test for a single point, same margins); the survivors, compacted
                    // into full warps, get the interval evaluation
                    const float tp = H;
                    float cH[D];
                    float rr2 = INFINITY;
                    if (isfinite(tp)) {
                        float r2 = 0.f;
#pragma unroll
                        for (int k = 0; k < D; ++k) {
                            const float off = fmaf(tp, u[k], rho[k]);
                            const float w2 = db[k] - off;
                            r2 = fmaf(w2, w2, r2);
                            cH[k] = xa[k] + (xal[k] + off);
                        }
                        const float rr = sqrtf(r2) * 1.0001f + 1e-6f * M.xs32 + 1e-4f * fabsf(tp);
                        rr2 = rr * rr;
                    }
                    int nc = 0;
                    for (int base = 0; base < tot; base += 32) {
                        const int qq = base + lane;
                        int j = -1;
                        if (qq < tot) {
                            j = lsh >= 0 ? (lq[qq >> lsh] << lsh) + (qq & (L - 1)) : lq[qq / L] * L + (qq % L);
                            if (j >= M.n) j = -1;
                        }
                        if (j >= 0) {
#pragma unroll
                            for (int q = 0; q < R; ++q) if (j == sig[q]) j = -1;
                        }
                        if (j >= 0 && rr2 < INFINITY) {
                            float xj[DP];
                            load_pt32<D>(M, j, xj);
                            float d2 = 0.f;
#pragma unroll
                            for (int k = 0; k < D; ++k) { const float e = xj[k] - cH[k]; d2 = fmaf(e, e, d2); }
                            if (d2 > rr2) j = -1;
                        }
                        const unsigned bj = __ballot_sync(FULL, j >= 0);
                        if (j >= 0) cq[nc + __popc(bj & ((1u << lane) - 1u))] = j;
                        nc += __popc(bj);
                        npoints_in += __popc(bj);
                        __syncwarp();
                        if (nc >= 32 || (base + 32 >= tot && nc > 0)) {
                            for (int b2 = 0; b2 < nc; b2 += 32) {
                                if (b2 + lane < nc) {
                                    const int jj = cq[b2 + lane];
                                    float lo, hi;
                                    bool ok;
                                    cand32<D>(M, jj, xa, xal, rho, R1, erho, u, lam, U1, LB, relu, lo, hi, ok);
                                    if (ok) take(jj, lo, hi);
                                }
                            }
                            nc = 0;
                            __syncwarp();
                        }
                    }
                    top2_warp(lo1, hi1, j1, lo2);
#pragma unroll
                    for (int off = 16; off > 0; off >>= 1) H = fminf(H, __shfl_xor_sync(FULL, H, off));
                    nl = 0;
                    __syncwarp();
                    continue;
                }
                const int nt = min(sp, 32);
                const int node = lane < nt ? stk[sp - nt + lane] : 0;
                sp -= nt;
                nnodes += nt;
                __syncwarp();
                bool keep = lane < nt;
                const float tp = H;
                if (keep && isfinite(tp)) {
                    float r2 = 0.f, bd2 = 0.f;
                    float bl[DP], bh[DP];
                    load_f4<DP>(M.blo + (size_t)node * DP, bl);
                    load_f4<DP>(M.bhi + (size_t)node * DP, bh);
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        const float off = fmaf(tp, u[k], rho[k]);
                        const float w2 = db[k] - off;
                        r2 = fmaf(w2, w2, r2);
                        const float ck = xa[k] + (xal[k] + off);
                        const float l = bl[k], h = bh[k];
                        const float ex = ck < l ? l - ck : (ck > h ? ck - h : 0.f);
                        bd2 = fmaf(ex, ex, bd2);
                    }
                    const float rr = sqrtf(r2) * 1.0001f + 1e-6f * M.xs32 + 1e-4f * fabsf(tp);
                    keep = !(bd2 > rr * rr);
                }
                const bool isleaf = node >= M.P;
                const bool lv = keep && isleaf && (node - M.P) < M.nleaves;
                const bool in = keep && !isleaf;
                const unsigned bl = __ballot_sync(FULL, lv), bi = __ballot_sync(FULL, in);
                const unsigned lt = (1u << lane) - 1u;
                if (sp + 2 * __popc(bi) > FB_STK) { overflow = true; break; }
                if (lv) lq[nl + __popc(bl & lt)] = node - M.P;
                if (in) {
                    const int p = sp + 2 * __popc(bi & lt);
                    stk[p] = 2 * node + 1;
                    stk[p + 1] = 2 * node;
                }
                nl += __popc(bl);
                sp += 2 * __popc(bi);
                __syncwarp();
            }
            if (lane == 0) {
                count_add(M.cnt + C_FBTREE);
                atomicAdd(M.cnt + C_FBNODES, (unsigned long long)nnodes);
                atomicAdd(M.cnt + C_FBLEAVES, (unsigned long long)nleaves_seen);
                atomicAdd(M.cnt + C_FBPOINTS, (unsigned long long)npoints_in);
            }
        }
        const bool certified = !overflow && j1 >= 0 && hi1 < lo2;
        if (certified) {
            if (lane == 0) {
                int ns[R];
                make_sig<D>(sig, m, j1, ns);
                bool is_new;
                vertex_insert<D>(M, ns, j1, is_new);
            }
        } else {
            // every possible winner has lo <= H: gather that set and decide it in FP64
            int keep = 0;
            for (int q = 0; q < namb; ++q) keep += (amb_lo[q] <= H) ? 1 : 0;
            const bool over = __any_sync(FULL, amb_over) || overflow;
            int pos = keep;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int y = __shfl_up_sync(FULL, pos, off);
                if (lane >= off) pos += y;
            }
            const int total = __shfl_sync(FULL, pos, 31);
            pos -= keep;
            if (!over && total <= FB_AMB_MAX) {
                for (int q = 0; q < namb; ++q)
                    if (amb_lo[q] <= H) samb[wib][pos++] = amb_j[q];
            }
            __syncwarp();
            // the set goes to the FP64 decision kernel (k_decide_sets); without a usable
            // set, or with its queue full, the ray is redone by the exact tree search
            unsigned slot = 0xFFFFFFFFu;
            if (lane == 0 && !over && total <= FB_AMB_MAX && total > 0) {
                slot = atomicAdd(aq.count, 1u);
                if (slot >= aq.cap) slot = 0xFFFFFFFFu;
            }
            slot = __shfl_sync(FULL, slot, 0);
            if (slot != 0xFFFFFFFFu) {
                if (lane < total) aq.ids[(size_t)slot * AMB_SET + lane] = samb[wib][lane];
                if (lane == 0) { aq.e[slot] = e; aq.n[slot] = total; }
            } else if (lane == 0) {
                const unsigned fs = atomicAdd(nfx, 1u);
                if (fs < fxcap) fx[fs] = e;
                else set_status(M, ST_QUEUE);
            }
        }
        __syncwarp();
    }
}

// FP64 (then double-double) decision of the queued ambiguous sets.  Many sets:
// one per thread.  Few sets (latency-bound): one per warp -- lane 0 sets the ray
// up, every lane evaluates one candidate in FP64, lane 0 folds them in the order
// of the set (the same decisions as the serial pass) and re-scores the rest in
// double-double if needed.  An undecided ray is redone by the exact tree search
// (k_fallback).
constexpr int DS_WPB = 4;

template <int D>
__global__ void __launch_bounds__(DS_WPB * 32) k_decide_sets(DevMesh M, AmbQueue aq, unsigned long long* fx,
                                                             unsigned* nfx, unsigned fxcap) {
    constexpr int R = D + 1;
    __shared__ Query<D> sq[DS_WPB];
    __shared__ Cand sc[DS_WPB][AMB_SET];
    __shared__ int sok[DS_WPB];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned FULL = 0xFFFFFFFFu;
    if (M.G.lvl) {  // graph-driven levels: the exact queue of the previous level
        const int p = (M.G.lvl[2] + 1) & 1;
        fx = M.G.fx[p]; nfx = M.G.qc + 2 * p + 1;
    }
    const unsigned nq = min(*aq.count, aq.cap);
    if (nq > 2u * gridDim.x * DS_WPB) {  // many sets: one per thread (throughput)
        for (unsigned w = blockIdx.x * blockDim.x + threadIdx.x; w < nq; w += gridDim.x * blockDim.x) {
            count_add(M.cnt + C_AMBSET);
            const unsigned long long e = aq.e[w];
            const unsigned v = (unsigned)(e >> 4);
            const int m = (int)(e & 7);
            int sig[R];
#pragma unroll
            for (int k = 0; k < R; ++k) sig[k] = M.vsig[(size_t)v * R + k];
            const int win = exact_decide_set<D>(M, sig, m, aq.ids + (size_t)w * AMB_SET, aq.n[w]);
            if (win >= 0) {
                int ns[R];
                make_sig<D>(sig, m, win, ns);
                bool is_new;
                vertex_insert<D>(M, ns, win, is_new);
            } else {
                const unsigned fs = atomicAdd(nfx, 1u);
                if (fs < fxcap) fx[fs] = e;
                else set_status(M, ST_QUEUE);
            }
        }
        return;
    }
    for (unsigned w = blockIdx.x * DS_WPB + wib; w < nq; w += gridDim.x * DS_WPB) {  // few sets: one per warp
        const unsigned long long e = aq.e[w];
        const unsigned v = (unsigned)(e >> 4);
        const int m = (int)(e & 7);
        const int nitems = aq.n[w];
        const int* items = aq.ids + (size_t)w * AMB_SET;
        int sig[R];
#pragma unroll
        for (int k = 0; k < R; ++k) sig[k] = M.vsig[(size_t)v * R + k];
        if (lane == 0) {
            count_add(M.cnt + C_AMBSET);
            sok[wib] = setup_walk<D>(M, sig, m, sq[wib]) ? 1 : 0;
        }
        __syncwarp();
        int win = -1;
        if (sok[wib]) {
            const Query<D>& q = sq[wib];
            Cand c;
            c.item = -1;
            c.t = c.lo = c.hi = INFINITY;
            if (lane < nitems && items[lane] < M.n) {
                SearchOut Rl;
                Rl.best = Cand{-1, INFINITY, INFINITY, INFINITY};
                Rl.second_lo = INFINITY;
                Rl.namb = 0;
                Rl.overflow = false;
                eval_point<D>(M, q, items[lane], Rl);
                c = Rl.best;
            }
            sc[wib][lane] = c;
            const bool planes = __any_sync(FULL, lane < nitems && items[lane] >= M.n);
            __syncwarp();
            if (lane == 0) {
                SearchOut Rs;
                Rs.best = Cand{-1, INFINITY, INFINITY, INFINITY};
                Rs.second_lo = INFINITY;
                Rs.namb = 0;
                Rs.overflow = false;
                for (int k = 0; k < nitems; ++k)
                    if (sc[wib][k].item >= 0) consider(Rs, sc[wib][k]);
                if (planes) eval_planes<D>(M, q, Rs);
                if (Rs.best.item >= 0) {
                    if (Rs.best.hi < Rs.second_lo) {
                        win = Rs.best.item;
                    } else if (Rs.overflow) {
                        win = -1;  // more near-ties than the set holds: the exact tree search decides
                    } else {
                        count_add(M.cnt + C_DD);
                        int its[HV_NAMB + 1];
                        its[0] = Rs.best.item;
                        int n2 = 1;
                        for (int k = 0; k < Rs.namb; ++k)
                            if (Rs.amb[k].lo <= Rs.best.hi) its[n2++] = Rs.amb[k].item;
                        bool degen = false;
                        win = dd_rescore_walk<D>(M, sig, m, its, n2, degen);
                        if (degen) { count_add(M.cnt + C_DEGEN); set_status(M, ST_DEGEN); }
                    }
                }
            }
        }
        if (lane == 0) {
            if (win >= 0) {
                int ns[R];
                make_sig<D>(sig, m, win, ns);
                bool is_new;
                vertex_insert<D>(M, ns, win, is_new);
            } else {
                const unsigned fs = atomicAdd(nfx, 1u);
                if (fs < fxcap) fx[fs] = e;
                else set_status(M, ST_QUEUE);
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// warp descent: one warp per seed generator; every step is an FP32 ray over
// the seed's candidate list with the same certified bounds and security test
// as the wavefront.  A seed with an undecided step is queued for the FP64
// descent (k_descent with a seed list).
// ---------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(FB_WPB * 32) k_descent_warp(DevMesh M, int stride, int nseeds,
                                                              unsigned long long seed, int* failed,
                                                              unsigned* nfailed) {
    constexpr int DP = (D <= 4) ? 4 : 8;
    __shared__ double sU[FB_WPB][D];
    __shared__ double sRho[FB_WPB][D];
    __shared__ int sOk[FB_WPB];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned FULL = 0xFFFFFFFFu;
    const float S32 = 5.9604645e-08f;
    for (int w = blockIdx.x * FB_WPB + wib; w < nseeds; w += gridDim.x * FB_WPB) {
        const int i = M.own0 + w * stride;
        if (i >= M.own1) continue;
        if (M.own_from >= 0 && __ldg(M.perm + i) < M.own_from) continue;  // refinement: new cells only
        if (lane == 0) count_add(M.cnt + C_DESCENT);
        int T[D + 1];
#pragma unroll
        for (int k = 0; k <= D; ++k) T[k] = -1;
        T[0] = i;
        int nT = 1;
        float xa[DP], xal[DP];
        load_pt32<D>(M, i, xa);
        load_pt32lo<D>(M, i, xal);
        double xi[D];
#pragma unroll
        for (int k = 0; k < D; ++k) xi[k] = __ldg(M.pts + (size_t)i * D + k);
        if (lane < D) sRho[wib][lane] = 0.0;
        const float seci = M.K > 0 ? __ldg(M.sec + i) : 0.f;
        bool ok = M.K > 0;
        for (int step = 1; step <= D && ok; ++step) {
            // direction: Philox Gaussian projected off the constraint rows (FP64, lane 0)
            if (lane == 0) {
                double g[D], B[D][D];
                gauss_dir<D>(seed, (unsigned)(16 + step), (unsigned long long)i, g);
                int nb = 0;
                bool good = true;
                for (int s2 = 1; s2 < nT && good; ++s2) {
                    double row[D], rh;
                    con_row<D, double>(M, xi, T[s2], row, rh);
                    for (int t2 = 0; t2 < nb; ++t2) {
                        double pr = 0;
#pragma unroll
                        for (int k = 0; k < D; ++k) pr = fma(row[k], B[t2][k], pr);
#pragma unroll
                        for (int k = 0; k < D; ++k) row[k] -= pr * B[t2][k];
                    }
                    double nn = 0;
#pragma unroll
                    for (int k = 0; k < D; ++k) nn = fma(row[k], row[k], nn);
                    nn = sqrt(nn);
                    if (!(nn > 1e-300)) { good = false; break; }
                    const double inn = 1.0 / nn;
#pragma unroll
                    for (int k = 0; k < D; ++k) B[nb][k] = row[k] * inn;
                    ++nb;
                }
                for (int rep = 0; rep < 2 && good; ++rep) {
                    for (int t2 = 0; t2 < nb; ++t2) {
                        double pr = 0;
#pragma unroll
                        for (int k = 0; k < D; ++k) pr = fma(g[k], B[t2][k], pr);
#pragma unroll
                        for (int k = 0; k < D; ++k) g[k] -= pr * B[t2][k];
                    }
                }
                double nn = 0;
#pragma unroll
                for (int k = 0; k < D; ++k) nn = fma(g[k], g[k], nn);
                nn = sqrt(nn);
                if (!(nn > 1e-12)) good = false;
                const double inn = 1.0 / nn;
#pragma unroll
                for (int k = 0; k < D; ++k) sU[wib][k] = good ? g[k] * inn : 0.0;
                sOk[wib] = good ? 1 : 0;
            }
            __syncwarp();
            if (!sOk[wib]) { ok = false; break; }
            float u[D], rho[D];
            float U1 = 0.f, R1 = 0.f, rmax = 0.f;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                u[k] = (float)sU[wib][k];
                rho[k] = (float)sRho[wib][k];
                U1 += fabsf(u[k]);
                R1 += fabsf(rho[k]);
                rmax = fmaxf(rmax, fabsf(rho[k]));
            }
            const float relu = 4.f * S32;
            const float erho = 2.f * S32 * rmax + M.e13_32;
            float lo1 = INFINITY, hi1 = INFINITY, lo2 = INFINITY, H = INFINITY;
            int j1 = -1;
            // planes (lane 0)
            if (lane == 0) {
                const float TINY = M.tiny32;
                planes32<D>(
                    M, xa, xal, rho, u, erho, relu, TINY,
                    [&](int it) {
                        bool ex = false;
#pragma unroll
                        for (int q = 0; q <= D; ++q) ex |= (T[q] == it);
                        return ex;
                    },
                    [&](int it, float lo, float hi) {
                        H = fminf(H, hi);
                        top2_add(lo1, hi1, j1, lo2, lo, hi, it);
                    });
            }
            const int* lst = M.knn + (size_t)i * M.K;
            for (int c = lane; c < M.K; c += 32) {
                const int j = __ldg(lst + c);
                if (j < 0) continue;
                bool inT = false;
#pragma unroll
                for (int q = 0; q <= D; ++q) inT |= (j == T[q]);
                if (inT) continue;
                float lo, hi;
                bool okc;
                cand32<D>(M, j, xa, xal, rho, R1, erho, u, 0.f, U1, 0.f, relu, lo, hi, okc);
                if (okc) { H = fminf(H, hi); top2_add(lo1, hi1, j1, lo2, lo, hi, j); }
            }
            top2_warp(lo1, hi1, j1, lo2);
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) H = fminf(H, __shfl_xor_sync(FULL, H, off));
            bool good = j1 >= 0 && hi1 < lo2 && isfinite(hi1) && lo1 > 0.f;
            if (good) {
                // security of the sphere at the winner's upper bound (x_i is on it)
                float c2 = 0.f;
#pragma unroll
                for (int k = 0; k < D; ++k) { const float cc = fmaf(hi1, u[k], rho[k]); c2 = fmaf(cc, cc, c2); }
                const float ec = erho + hi1 * relu + 4.f * S32 * (rmax + hi1) + M.e12_32;
                good = 2.f * sqrtf(c2) + 4.f * sqrtf((float)D) * ec < seci * (1.f - 1e-5f);
            }
            if (!good) { ok = false; break; }
            // FP64 step length of the winner and the new point (lane 0)
            if (lane == 0) {
                double tt;
                if (j1 < M.n) {
                    double nd = 0, dr = 0, du = 0;
#pragma unroll
                    for (int k = 0; k < D; ++k) {
                        const double dl = __ldg(M.pts + (size_t)j1 * D + k) - xi[k];
                        nd = fma(dl, dl, nd); dr = fma(dl, sRho[wib][k], dr); du = fma(dl, sU[wib][k], du);
                    }
                    tt = (nd - 2.0 * dr) / (2.0 * du);
                } else {
                    const DevPlane& P = M.planes[j1 - M.n];
                    if (P.axis >= 0) {  // n = +-e_k: exact dot products
                        double nc = 0, nu = 0;
#pragma unroll
                        for (int k = 0; k < D; ++k) {
                            nc = fma(P.n[k], xi[k] + sRho[wib][k], nc);
                            nu = fma(P.n[k], sU[wib][k], nu);
                        }
                        tt = (P.off - nc) / nu;
                    } else {
                        const dd sx = plane_rhs_dd<D>(P, xi);
                        double nr = 0, nu = 0;
#pragma unroll
                        for (int k = 0; k < D; ++k) { nr = fma(P.n[k], sRho[wib][k], nr); nu = fma(P.n[k], sU[wib][k], nu); }
                        tt = ((sx.hi + sx.lo) - nr) / nu;
                    }
                }
#pragma unroll
                for (int k = 0; k < D; ++k) sRho[wib][k] = fma(tt, sU[wib][k], sRho[wib][k]);
            }
            __syncwarp();
#pragma unroll
            for (int q = 0; q <= D; ++q) if (q == nT) T[q] = j1;
            ++nT;
        }
        if (lane == 0) {
            if (ok) {
                int S[D + 1];
#pragma unroll
                for (int q = 0; q <= D; ++q) S[q] = T[q];
#pragma unroll
                for (int s2 = 1; s2 <= D; ++s2) {
#pragma unroll
                    for (int t2 = s2; t2 > 0; --t2)
                        if (S[t2] < S[t2 - 1]) { const int x = S[t2]; S[t2] = S[t2 - 1]; S[t2 - 1] = x; }
                }
                bool is_new;
                vertex_insert<D>(M, S, -1, is_new);
            } else {
                failed[atomicAdd(nfailed, 1u)] = i;
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
template <int D>
static void launch_register_t(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st) {
    const unsigned long long total = (unsigned long long)(v1 - v0) * (D + 1);
    if (!total) return;
    unsigned long long blocks = (total + 255) / 256;
    if (blocks > (unsigned long long)nsm * 32) blocks = (unsigned long long)nsm * 32;
    k_register_edges<D><<<(unsigned)blocks, 256, 0, st>>>(M, v0, v1);
}
template <int D>
static void launch_refine_t(const DevMesh& M, unsigned V, int nsm, cudaStream_t st) {
    if (!V || !M.vcond) return;
    unsigned blocks = (V + 127) / 128;
    if (blocks > (unsigned)nsm * 16) blocks = (unsigned)nsm * 16;
    k_refine_centers<D><<<blocks, 128, 0, st>>>(M, V);
}
template <int D>
static void launch_centers_t(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st) {
    if (v1 <= v0) return;
    unsigned blocks = (v1 - v0 + 127) / 128;
    if (blocks > (unsigned)nsm * 16) blocks = (unsigned)nsm * 16;
    k_centers<D><<<blocks, 128, 0, st>>>(M, v0, v1);
}
template <int D>
static void launch_descent_t(const DevMesh& M, int stride, int nseeds, unsigned long long seed, int* failed,
                             unsigned* nfailed, int nsm, cudaStream_t st) {
    if (nseeds <= 0) return;
    if (M.K > 0 && failed) {
        // FP32 warp descent; seeds whose step cannot be decided are only listed:
        // any seed reaches the whole (connected) vertex graph, so the exact
        // descent runs on that list only when no seed at all succeeded
        // (launch_descent_exact)
        int blocks = (nseeds + FB_WPB - 1) / FB_WPB;
        if (blocks > nsm * 32) blocks = nsm * 32;
        k_descent_warp<D><<<blocks, FB_WPB * 32, 0, st>>>(M, stride, nseeds, seed, failed, nfailed);
    } else {
        k_descent<D><<<(nseeds + 127) / 128, 128, 0, st>>>(M, stride, nseeds, seed, nullptr, nullptr);
    }
}
template <int D>
static void launch_descent_exact_t(const DevMesh& M, int maxn, unsigned long long seed, int* failed,
                                   unsigned* nfailed, int nsm, cudaStream_t st) {
    if (maxn <= 0) return;
    k_descent<D><<<(maxn + 127) / 128, 128, 0, st>>>(M, 1, maxn, seed, failed, nfailed);
}
template <int D>
static void launch_plain_t(const DevMesh& M, unsigned f0, unsigned f1, int nsm, cudaStream_t st) {
    unsigned long long total = (unsigned long long)(f1 - f0) * (D + 1);
    if (!total) return;
    unsigned long long blocks = (total + 127) / 128;
    blocks = blocks > (unsigned long long)nsm * 64 ? (unsigned long long)nsm * 64 : blocks;
    k_expand_plain<D><<<(unsigned)blocks, 128, 0, st>>>(M, f0, f1);
}
template <int D>
static void launch_fast_t(const DevMesh& M, unsigned f0, unsigned f1, unsigned long long* fq, unsigned* nfq,
                          unsigned fqcap, unsigned long long* fx, unsigned* nfx, unsigned fxcap, int nsm,
                          cudaStream_t st) {
    const size_t sm = fast_smem_bytes(D, M.K);
    if (sm > 48 * 1024) {
        // once per instantiation, for the largest list length (thread-safe static
        // init; an empty launch sets it up ahead of a stream capture)
        static const bool set = [] {
            return cudaFuncSetAttribute(k_expand_fast<D>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)fast_smem_bytes(D, 480)) == cudaSuccess;
        }();
        (void)set;
    }
    unsigned nf = f1 - f0;
    if (!nf) return;
    unsigned blocks = (nf + FAST_WPB - 1) / FAST_WPB;
    if (blocks > (unsigned)nsm * 32) blocks = (unsigned)nsm * 32;
    cudaMemsetAsync(M.ndq, 0, sizeof(unsigned), st);
    k_expand_fast<D><<<blocks, FAST_WPB * 32, sm, st>>>(M, f0, f1, fq, nfq, fqcap, fx, nfx, fxcap);
    k_insert_decided<D><<<nsm * 8, 256, 0, st>>>(M);
}
template <int D>
static void launch_fallback_warp_t(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq,
                                   unsigned fqcap, unsigned maxq, unsigned long long* fx, unsigned* nfx,
                                   unsigned fxcap, const AmbQueue& aq, int nsm, cudaStream_t st) {
    if (!maxq) return;
    // grid-stride over the queue: a few resident waves, so empty levels cost little
    unsigned blocks = (maxq + FB_WPB - 1) / FB_WPB;
    if (blocks > (unsigned)nsm * 8) blocks = (unsigned)nsm * 8;
    k_fallback_warp<D><<<blocks, FB_WPB * 32, 0, st>>>(M, fq, nfq, fqcap, fx, nfx, fxcap, aq);
    unsigned b2 = (min(maxq, aq.cap) + DS_WPB - 1) / DS_WPB;
    if (b2 > (unsigned)nsm * 4) b2 = (unsigned)nsm * 4;
    if (b2 < 1) b2 = 1;
    k_decide_sets<D><<<b2, DS_WPB * 32, 0, st>>>(M, aq, fx, nfx, fxcap);
}
template <int D>
static void launch_fallback_t(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned maxq,
                              int nsm, cudaStream_t st) {
    if (!maxq) return;
    unsigned blocks = (maxq + 127) / 128;
    if (blocks > (unsigned)nsm * 4) blocks = (unsigned)nsm * 4;
    k_fallback<D><<<blocks, 128, 0, st>>>(M, fq, nfq, maxq);
}

}  // namespace hv
