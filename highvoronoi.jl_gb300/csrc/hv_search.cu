// hv_search.cu -- Voronoi vertex search on the GPU.
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
#include "hv_internal.cuh"
#include "hv_host.h"

namespace hv {

constexpr double EPS64 = 1.1102230246251565e-16;

// ---------------------------------------------------------------------------
// vertex hash
// ---------------------------------------------------------------------------
template <int D>
__device__ unsigned vertex_insert(const DevMesh& M, const int (&s)[D + 1], int newitem, bool& is_new) {
    is_new = false;
    const unsigned long long h = hash_items(s, D + 1);
    const unsigned fp = ((unsigned)(h >> 32) & 0x7FFFFFFFu) | 1u;
    unsigned long long slot = h & M.vhmask;
    for (unsigned long long probe = 0; probe <= M.vhmask; ++probe) {
        unsigned long long e = *(volatile unsigned long long*)&M.vhash[slot];
        if (e == HASH_EMPTY) {
            unsigned long long prev = atomicCAS(&M.vhash[slot], HASH_EMPTY, HASH_BUSY);
            if (prev == HASH_EMPTY) {
                unsigned vid = atomicAdd(M.vcount, 1u);
                if (vid >= M.vcap) {
                    set_status(M, ST_VCAP);
                    atomicExch(&M.vhash[slot], ((unsigned long long)fp << 32) | INVALID_ID);
                    return INVALID_ID;
                }
#pragma unroll
                for (int k = 0; k <= D; ++k) M.vsig[(size_t)vid * (D + 1) + k] = s[k];
                M.vnew[vid] = newitem;
                __threadfence();
                atomicExch(&M.vhash[slot], ((unsigned long long)fp << 32) | vid);
                is_new = true;
                return vid;
            }
            e = prev;
        }
        int spins = 0;
        while (e == HASH_BUSY) {
            if (++spins > SPIN_LIMIT) { set_status(M, ST_TIMEOUT); return INVALID_ID; }
            __nanosleep(32);
            e = *(volatile unsigned long long*)&M.vhash[slot];
        }
        if ((unsigned)(e >> 32) == fp) {
            unsigned id = (unsigned)e;
            if (id != INVALID_ID) {
                __threadfence();
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

template <int D>
__device__ __forceinline__ void eval_point(const DevMesh& M, const Query<D>& q, int j, SearchOut& R) {
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
    Cand c; c.item = j;
    if (den > e_den) {
        c.t = num / den;
        double et = (e_num + fabs(c.t) * e_den) / (den - e_den) + 4.0 * EPS64 * fabs(c.t);
        c.lo = c.t - et; c.hi = c.t + et;
    } else if (den < -e_den) {
        return;
    } else {
        if (num - e_num > 0) {
            if (!(den + e_den > 0)) return;
            c.lo = (num - e_num) / (den + e_den); c.hi = INFINITY; c.t = c.lo;
        } else {
            c.lo = -INFINITY; c.hi = INFINITY; c.t = 0;
        }
    }
    if (c.lo < R.best.hi || c.lo < R.second_lo) consider(R, c);
}

template <int D>
__device__ __forceinline__ void eval_planes(const DevMesh& M, const Query<D>& q, SearchOut& R) {
#pragma unroll
    for (int p = 0; p < 2 * D; ++p) {
        const int it = M.n + p;
        if (q_excluded<D>(q, it)) continue;
        const int k = p >> 1;
        const bool upper = (p & 1) == 0;
        double uk = upper ? q.u[k] : -q.u[k];
        double ck = q.xa[k] + q.rho[k];
        double num = upper ? (M.hi[k] - ck) : (ck - M.lo[k]);
        double e_num = 4.0 * EPS64 * (fabs(M.hi[k]) + fabs(M.lo[k]) + fabs(q.xa[k]) + fabs(q.rho[k])) + q.erho;
        double e_den = q.eu + 2.0 * EPS64 * fabs(uk);
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
        consider(R, c);
    }
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
            const int p = it - M.n, k0 = p >> 1;
            const bool upper = (p & 1) == 0;
            dd uk = mk(0.0), ck = mk(0.0);
#pragma unroll
            for (int k = 0; k < D; ++k) if (k == k0) { uk = upper ? u[k] : -u[k]; ck = mk(xa[k]) + rho[k]; }
            if (!(uk.hi > 0)) continue;
            dd num = upper ? (mk(M.hi[k0]) - ck) : (ck - mk(M.lo[k0]));
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
            const int p = it - M.n, k0 = p >> 1;
            const bool upper = (p & 1) == 0;
            double uk = upper ? q.u[k0] : -q.u[k0];
            if (!(uk > 0)) continue;
            dd ck = mk(q.xa[k0]) + mk(q.rho[k0]);
            dd num = upper ? (mk(M.hi[k0]) - ck) : (ck - mk(M.lo[k0]));
            t = num / mk(uk);
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
        if (R.overflow) set_status(M, ST_AMB);
        int items[HV_NAMB + 1];
        items[0] = R.best.item;
        for (int k = 0; k < R.namb; ++k) items[k + 1] = R.amb[k].item;
        bool degen = false;
        win = dd_rescore_walk<D>(M, sig, m, items, R.namb + 1, degen);
        if (degen) { count_add(M.cnt + C_DEGEN); set_status(M, ST_DEGEN); }
        if (win < 0) { set_status(M, ST_NUMERIC); return; }
    }
    int ns[D + 1];
    make_sig<D>(sig, m, win, ns);
    bool is_new;
    vertex_insert<D>(M, ns, win, is_new);
}

// Edge sig \ {sig[m]} is walkable if it is not the edge the vertex was found
// through and if it still contains a real generator.
template <int D>
__device__ __forceinline__ bool walkable(const DevMesh& M, const int (&sig)[D + 1], int vnew, int m) {
    if (sig[m] == vnew) return false;
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
        count_add(M.cnt + C_RAYS);
        exact_walk<D>(M, v, m);
    }
}

template <int D>
__global__ void __launch_bounds__(128) k_fallback(DevMesh M, const unsigned long long* fq, const unsigned* nfq,
                                                  unsigned fqcap) {
    const unsigned n = min(*nfq, fqcap);  // entries past the capacity were never written
    for (unsigned r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const unsigned long long e = fq[r];
        count_add(M.cnt + C_FALLBACK);
        exact_walk<D>(M, (unsigned)(e >> 3), (int)(e & 7));
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
            double u1 = ((double)c[2 * p] + 0.5) * 2.3283064365386963e-10;
            double u2 = ((double)c[2 * p + 1] + 0.5) * 2.3283064365386963e-10;
            double rr = sqrt(-2.0 * log(u1));
            double sn, cs;
            sincospi(2.0 * u2, &sn, &cs);
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
__global__ void __launch_bounds__(128) k_descent(DevMesh M, int stride, int nseeds, unsigned long long seed) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nseeds) return;
    const int i = idx * stride;
    if (i >= M.n) return;
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
                    double tol = 1e-12 * (1.0 + fabs(M.hi[k]) + fabs(M.lo[k]));
                    if (c[k] < M.lo[k] - tol || c[k] > M.hi[k] + tol) good = false;
                    double e = __ldg(p0 + k) - c[k];
                    r2 = fma(e, e, r2);
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
// FP64 circumcentres of new vertices, one thread per vertex (full-warp FP64)
// ---------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(128) k_centers(DevMesh M, unsigned v0, unsigned v1) {
    constexpr int DP = (D <= 4) ? 4 : 8;
    for (unsigned v = v0 + blockIdx.x * blockDim.x + threadIdx.x; v < v1; v += gridDim.x * blockDim.x) {
        int s[D + 1];
#pragma unroll
        for (int k = 0; k <= D; ++k) s[k] = M.vsig[(size_t)v * (D + 1) + k];
        double c[D];
        const double* pa = M.pts + (size_t)s[0] * D;
        if (!vertex_center<D>(M, s, c)) {
            set_status(M, ST_NUMERIC);
#pragma unroll
            for (int k = 0; k < D; ++k) c[k] = __ldg(pa + k);
        }
        float r32[DP];
#pragma unroll
        for (int k = 0; k < DP; ++k) r32[k] = 0.f;
#pragma unroll
        for (int k = 0; k < D; ++k) {
            M.vc[(size_t)v * D + k] = c[k];
            r32[k] = (float)(c[k] - __ldg(pa + k));
        }
        float4* dst = reinterpret_cast<float4*>(M.vrho32 + (size_t)v * DP);
#pragma unroll
        for (int h = 0; h < DP / 4; ++h) dst[h] = make_float4(r32[4 * h], r32[4 * h + 1], r32[4 * h + 2], r32[4 * h + 3]);
    }
}

// ---------------------------------------------------------------------------
// fast kernel: one warp expands one vertex entirely in FP32
// ---------------------------------------------------------------------------
constexpr int FAST_WPB = 4;  // warps per block

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
__global__ void __launch_bounds__(FAST_WPB * 32) k_expand_fast(DevMesh M, unsigned f0, unsigned f1,
                                                               unsigned long long* fq, unsigned* nfq,
                                                               unsigned fqcap) {
    constexpr int R = D + 1;
    constexpr int DP = (D <= 4) ? 4 : 8;
    __shared__ float sInv[FAST_WPB][D][D];
    __shared__ float sU[FAST_WPB][R][D];
    __shared__ float sLam[FAST_WPB][R];
    __shared__ float sLb[FAST_WPB][R];
    __shared__ float sCond[FAST_WPB];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned FULL = 0xFFFFFFFFu;
    const unsigned nf = f1 - f0;
    const float S32 = 5.9604645e-08f;                          // 2^-24
    const float EX = (float)(2.0 * M.xscale * 5.9604645e-08);  // rounding of a coordinate difference
    for (unsigned w = blockIdx.x * FAST_WPB + wib; w < nf; w += gridDim.x * FAST_WPB) {
        const unsigned v = f0 + w;
        int sig[R];
#pragma unroll
        for (int k = 0; k < R; ++k) sig[k] = M.vsig[(size_t)v * R + k];
        const int vnew = M.vnew[v];
        const int a = sig[0];
        float xa[DP], rho[DP];
        load_pt32<D>(M, a, xa);
        {
            const float4* pr = reinterpret_cast<const float4*>(M.vrho32 + (size_t)v * DP);
#pragma unroll
            for (int h = 0; h < DP / 4; ++h) {
                float4 f = pr[h];
                rho[4 * h] = f.x; rho[4 * h + 1] = f.y; rho[4 * h + 2] = f.z; rho[4 * h + 3] = f.w;
            }
        }
        // ---- FP32 constraint system; lanes 0..D-1 each produce one column of the inverse
        float A[D][D];
        float nrm = 0.f;
#pragma unroll
        for (int r = 0; r < D; ++r) {
            const int it = sig[r + 1];
            if (it < M.n) {
                float xg[DP];
                load_pt32<D>(M, it, xg);
#pragma unroll
                for (int k = 0; k < D; ++k) A[r][k] = xg[k] - xa[k];
            } else {
                const int p = it - M.n;
#pragma unroll
                for (int k = 0; k < D; ++k) A[r][k] = (k == (p >> 1)) ? (((p & 1) == 0) ? 1.f : -1.f) : 0.f;
            }
            float s = 0.f;
#pragma unroll
            for (int k = 0; k < D; ++k) s += fabsf(A[r][k]);
            nrm = fmaxf(nrm, s);
        }
        int okv = 1;
        if (lane < D) {
            int piv[D];
            okv = lu_factor<D, float>(A, piv) ? 1 : 0;
            if (okv) {
                float col[D];
#pragma unroll
                for (int k = 0; k < D; ++k) col[k] = (k == lane) ? 1.f : 0.f;
                lu_solve<D, float>(A, piv, col);
#pragma unroll
                for (int k = 0; k < D; ++k) sInv[wib][k][lane] = col[k];
            }
        }
        okv = __shfl_sync(FULL, okv, 0);
        __syncwarp();
        if (!okv) {
            if (lane == 0) set_status(M, ST_NUMERIC);
            continue;
        }
        if (lane == 0) {
            float ninv = 0.f;
#pragma unroll
            for (int r = 0; r < D; ++r) {
                float s = 0.f;
#pragma unroll
                for (int k = 0; k < D; ++k) s += fabsf(sInv[wib][r][k]);
                ninv = fmaxf(ninv, s);
            }
            sCond[wib] = nrm * ninv;
        }
        // ---- ray directions (lane m < R)
        int active = 0;
        if (lane < R) {
            const int m = lane;
            active = walkable<D>(M, sig, vnew, m) ? 1 : 0;
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
                    float xb[DP];
                    load_pt32<D>(M, b, xb);
#pragma unroll
                    for (int k = 0; k < D; ++k) db[k] = xb[k] - xa[k];
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
        // relative error of the FP32 directions: conditioning x (input rounding + LU rounding)
        const float cond = sCond[wib];
        const float relu = 4.f * cond * (D * EX / fmaxf(nrm, 1e-30f) + (D + 2) * S32) + 2.f * S32;
        if (!(relu < 1e-3f)) {  // too ill-conditioned for an FP32 decision: all rays exact
            if (lane < R && active) {
                count_add(M.cnt + C_RAYS);
                const unsigned slot = atomicAdd(nfq, 1u);
                if (slot < fqcap) fq[slot] = ((unsigned long long)v << 3) | (unsigned)lane;
                else set_status(M, ST_QUEUE);
            }
            continue;
        }
        float R1 = 0.f, rmax = 0.f;
#pragma unroll
        for (int k = 0; k < D; ++k) { R1 += fabsf(rho[k]); rmax = fmaxf(rmax, fabsf(rho[k])); }
        const float erho = 2.f * S32 * rmax;  // rho is the rounded FP64 centre offset
        float u32[R][D], lam32[R], U1[R], LB[R];
        float lo1[R], hi1[R], lo2[R];
        int j1[R];
#pragma unroll
        for (int m = 0; m < R; ++m) {
            U1[m] = 0.f; lam32[m] = 0.f; LB[m] = 0.f;
#pragma unroll
            for (int k = 0; k < D; ++k) u32[m][k] = 0.f;
            if ((rmask >> m) & 1u) {
#pragma unroll
                for (int k = 0; k < D; ++k) { u32[m][k] = sU[wib][m][k]; U1[m] += fabsf(u32[m][k]); }
                lam32[m] = sLam[wib][m];
                LB[m] = sLb[wib][m];
            }
            lo1[m] = INFINITY; hi1[m] = INFINITY; lo2[m] = INFINITY; j1[m] = -1;
        }
        const float CN = (4.f * D + 8.f) * S32, CD = (4.f * D + 16.f) * S32;
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
        for (int c = lane; c < K; c += 32) {
            const int j = __ldg(lst + c);
            if (j < 0) continue;
            bool insig = false;
#pragma unroll
            for (int s = 0; s < R; ++s) insig |= (j == sig[s]);
            if (insig) continue;
            float xj[DP];
            load_pt32<D>(M, j, xj);
            float dl[D], A1 = 0.f, A2 = 0.f, A3 = 0.f, dr = 0.f;
#pragma unroll
            for (int k = 0; k < D; ++k) {
                dl[k] = xj[k] - xa[k];
                A1 += fabsf(dl[k]);
                A2 = fmaf(dl[k], dl[k], A2);
                A3 = fmaf(fabsf(dl[k]), fabsf(rho[k]), A3);
                dr = fmaf(dl[k], rho[k], dr);
            }
            const float num = fmaf(-2.f, dr, A2);
            const float e_num = 4.f * EX * (A1 + R1) + CN * (A2 + 2.f * A3) + 2.f * A1 * erho;
#pragma unroll
            for (int m = 0; m < R; ++m) {
                if (!((rmask >> m) & 1u)) continue;
                float du = 0.f, B = 0.f;
#pragma unroll
                for (int k = 0; k < D; ++k) { du = fmaf(dl[k], u32[m][k], du); B = fmaf(fabsf(dl[k]), fabsf(u32[m][k]), B); }
                const float den = 2.f * (du - lam32[m]);
                const float e_den = 4.f * EX * U1[m] + CD * (B + fabsf(lam32[m])) + 2.f * relu * (A1 + LB[m]);
                float lo, hi;
                if (den > e_den) {
                    const float r = __fdividef(1.f, den);
                    const float t = num * r;
                    float et;
                    if (e_den < 1e-3f * den) et = (e_num + fabsf(t) * e_den) * r * 1.0021f;
                    else et = __fdividef(e_num + fabsf(t) * e_den, den - e_den) * 1.00001f;
                    et += 8.f * S32 * fabsf(t);
                    lo = t - et; hi = t + et;
                } else if (den < -e_den) {
                    continue;
                } else {
                    if (num - e_num > 0.f) {
                        if (!(den + e_den > 0.f)) continue;
                        lo = __fdividef(num - e_num, den + e_den) * 0.99999f; hi = INFINITY;
                    } else {
                        lo = -INFINITY; hi = INFINITY;
                    }
                }
                if (lo < lo1[m] || (lo == lo1[m] && j < j1[m])) { lo2[m] = lo1[m]; lo1[m] = lo; hi1[m] = hi; j1[m] = j; }
                else if (lo < lo2[m]) lo2[m] = lo;
            }
        }
        // ---- warp reduction of the per-ray top-2
#pragma unroll
        for (int m = 0; m < R; ++m) {
            if (!((rmask >> m) & 1u)) continue;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const float olo1 = __shfl_xor_sync(FULL, lo1[m], off);
                const float ohi1 = __shfl_xor_sync(FULL, hi1[m], off);
                const float olo2 = __shfl_xor_sync(FULL, lo2[m], off);
                const int oj1 = __shfl_xor_sync(FULL, j1[m], off);
                const bool take = (olo1 < lo1[m]) || (olo1 == lo1[m] && oj1 >= 0 && (j1[m] < 0 || oj1 < j1[m]));
                if (take) { lo2[m] = fminf(lo1[m], olo2); lo1[m] = olo1; hi1[m] = ohi1; j1[m] = oj1; }
                else { lo2[m] = fminf(lo2[m], olo1); }
            }
        }
        // ---- per-ray decision on lane m
        if (lane < R && ((rmask >> lane) & 1u)) {
            const int m = lane;
            count_add(M.cnt + C_RAYS);
            float u[D];
#pragma unroll
            for (int k = 0; k < D; ++k) u[k] = sU[wib][m][k];
            float clo1 = 0.f, chi1 = 0.f, clo2 = 0.f;
            int cj1 = -1;
#pragma unroll
            for (int mm = 0; mm < R; ++mm)
                if (mm == m) { clo1 = lo1[mm]; chi1 = hi1[mm]; clo2 = lo2[mm]; cj1 = j1[mm]; }
            // boundary planes in FP32 with the same error model
            float plo1 = INFINITY, phi1 = INFINITY, plo2 = INFINITY;
            int pj1 = -1;
#pragma unroll
            for (int p = 0; p < 2 * D; ++p) {
                const int it = M.n + p;
                bool ex = false;
#pragma unroll
                for (int s = 0; s < R; ++s) ex |= (sig[s] == it);
                if (ex) continue;
                const int k = p >> 1;
                const bool upper = (p & 1) == 0;
                const float uk = upper ? u[k] : -u[k];
                const float hk = (float)M.hi[k], lk = (float)M.lo[k];
                const float ck = xa[k] + rho[k];
                const float num = upper ? (hk - ck) : (ck - lk);
                const float e_num = 4.f * S32 * (fabsf(hk) + fabsf(lk) + fabsf(xa[k]) + fabsf(rho[k])) + erho + EX;
                const float e_den = relu + 2.f * S32 * fabsf(uk);
                float lo, hi;
                if (uk > e_den) {
                    const float t = __fdividef(num, uk);
                    const float et = __fdividef(e_num + fabsf(t) * e_den, uk - e_den) * 1.00001f + 8.f * S32 * fabsf(t);
                    lo = t - et; hi = t + et;
                } else if (uk < -e_den) {
                    continue;
                } else {
                    if (num - e_num > 0.f) { lo = __fdividef(num - e_num, fabsf(uk) + e_den) * 0.99999f; hi = INFINITY; }
                    else { lo = -INFINITY; hi = INFINITY; }
                }
                if (lo < plo1) { plo2 = plo1; plo1 = lo; phi1 = hi; pj1 = it; }
                else if (lo < plo2) plo2 = lo;
            }
            int win;
            float blo, bhi, second;
            if (cj1 >= 0 && clo1 <= plo1) { win = cj1; blo = clo1; bhi = chi1; second = fminf(clo2, plo1); }
            else { win = pj1; blo = plo1; bhi = phi1; second = fminf(plo2, clo1); }
            bool queue = false;
            if (!(win >= 0 && bhi < second)) {
                count_add(M.cnt + C_UNCERT);
                queue = true;
            } else {
                // security: the new empty sphere must lie inside the complete radius of the list
                const float t = 0.5f * (blo + bhi), et = 0.5f * (bhi - blo);
                float db[D];
#pragma unroll
                for (int k = 0; k < D; ++k) db[k] = 0.f;
                if (m == 0) {
                    int b = -1;
#pragma unroll
                    for (int s = 1; s <= D; ++s) if (b < 0 && sig[s] < M.n) b = sig[s];
                    float xb[DP];
                    load_pt32<D>(M, b, xb);
#pragma unroll
                    for (int k = 0; k < D; ++k) db[k] = xb[k] - xa[k];
                }
                float xo[DP];
                load_pt32<D>(M, own, xo);
                float c2 = 0.f, r2 = 0.f, cm = 0.f;
#pragma unroll
                for (int k = 0; k < D; ++k) {
                    const float cc = fmaf(t, u[k], rho[k]);
                    const float co = cc - (xo[k] - xa[k]);
                    c2 = fmaf(co, co, c2);
                    const float wv = db[k] - cc;
                    r2 = fmaf(wv, wv, r2);
                    cm = fmaxf(cm, fabsf(cc));
                }
                const float ec = erho + fabsf(t) * relu + et + 4.f * S32 * (rmax + fabsf(t)) + 3.f * EX;
                const float lhs = sqrtf(c2) + sqrtf(r2) + 4.f * sqrtf((float)D) * ec + 4.f * S32 * cm;
                const float seco = sec_own;
                if (!(t > 0.f) || !(lhs < seco * (1.f - 1e-5f))) {
                    count_add(M.cnt + C_INSECURE);
                    queue = true;
                }
            }
            if (queue) {
                const unsigned slot = atomicAdd(nfq, 1u);
                if (slot < fqcap) fq[slot] = ((unsigned long long)v << 3) | (unsigned)m;
                else set_status(M, ST_QUEUE);
            } else {
                int ns[R];
                make_sig<D>(sig, m, win, ns);
                bool is_new;
                vertex_insert<D>(M, ns, win, is_new);
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
template <int D>
static void launch_centers_t(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st) {
    if (v1 <= v0) return;
    unsigned blocks = (v1 - v0 + 127) / 128;
    if (blocks > (unsigned)nsm * 16) blocks = (unsigned)nsm * 16;
    k_centers<D><<<blocks, 128, 0, st>>>(M, v0, v1);
}
template <int D>
static void launch_descent_t(const DevMesh& M, int stride, int nseeds, unsigned long long seed, cudaStream_t st) {
    if (nseeds <= 0) return;
    k_descent<D><<<(nseeds + 127) / 128, 128, 0, st>>>(M, stride, nseeds, seed);
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
                          unsigned fqcap, int nsm, cudaStream_t st) {
    unsigned nf = f1 - f0;
    if (!nf) return;
    unsigned blocks = (nf + FAST_WPB - 1) / FAST_WPB;
    if (blocks > (unsigned)nsm * 32) blocks = (unsigned)nsm * 32;
    k_expand_fast<D><<<blocks, FAST_WPB * 32, 0, st>>>(M, f0, f1, fq, nfq, fqcap);
}
template <int D>
static void launch_fallback_t(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned maxq,
                              int nsm, cudaStream_t st) {
    if (!maxq) return;
    unsigned blocks = (maxq + 127) / 128;
    if (blocks > (unsigned)nsm * 16) blocks = (unsigned)nsm * 16;
    k_fallback<D><<<blocks, 128, 0, st>>>(M, fq, nfq, maxq);
}

#define HV_DISPATCH(d, CALL)                      \
    switch (d) {                                  \
        case 2: { constexpr int DD = 2; CALL; } break; \
        case 3: { constexpr int DD = 3; CALL; } break; \
        case 4: { constexpr int DD = 4; CALL; } break; \
        case 5: { constexpr int DD = 5; CALL; } break; \
        case 6: { constexpr int DD = 6; CALL; } break; \
        default: break;                           \
    }

void launch_centers(const DevMesh& M, unsigned v0, unsigned v1, int nsm, cudaStream_t st) {
    HV_DISPATCH(M.d, (launch_centers_t<DD>(M, v0, v1, nsm, st)));
}
void launch_descent(const DevMesh& M, int stride, int nseeds, unsigned long long seed, cudaStream_t st) {
    HV_DISPATCH(M.d, (launch_descent_t<DD>(M, stride, nseeds, seed, st)));
}
void launch_expand_plain(const DevMesh& M, unsigned f0, unsigned f1, int nsm, cudaStream_t st) {
    HV_DISPATCH(M.d, (launch_plain_t<DD>(M, f0, f1, nsm, st)));
}
void launch_expand_fast(const DevMesh& M, unsigned f0, unsigned f1, unsigned long long* fq, unsigned* nfq,
                        unsigned fqcap, int nsm, cudaStream_t st) {
    HV_DISPATCH(M.d, (launch_fast_t<DD>(M, f0, f1, fq, nfq, fqcap, nsm, st)));
}
void launch_fallback(const DevMesh& M, const unsigned long long* fq, const unsigned* nfq, unsigned maxq, int nsm,
                     cudaStream_t st) {
    HV_DISPATCH(M.d, (launch_fallback_t<DD>(M, fq, nfq, maxq, nsm, st)));
}

}  // namespace hv
