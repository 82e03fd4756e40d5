// hv_domain.cu -- the convex domain: boundary planes and their bounding box.
//
// A domain is the intersection of half-spaces {x : n_p . x <= off_p}, one per
// boundary plane p, with n_p the outer unit normal.  The reference describes a
// plane by a base point b and a normal n (Plane, src/boundary.jl:22-29) and
// tests membership with dot(b - x, n) >= 0 (src/boundary.jl:427-435); its
// mirror image of a generator, x + 2 n (n . (b - x)) (src/boundary.jl:206-211),
// is a reflection only for |n| = 1, so normals are scaled to unit length here
// and off = n . b is formed in double-double and rounded once.
//
// cuboid(d, periodic=[]) (src/boundary.jl:510-534) lists for axis k the upper
// face (normal +e_k, base lo + (hi-lo) e_k) before the lower face (normal
// -e_k, base lo): planes 2k and 2k+1, generator ids n+2k and n+2k+1.
//
// The bounding box of the domain bounds every vertex coordinate (the FP32
// error models scale with it) and normalises the Morton codes.  For a cuboid
// it is the box itself; otherwise it comes from linear programs: a Chebyshev
// centre (largest inscribed ball) proves a non-empty interior and gives an
// interior start, then max and min of each coordinate.  Those use a dense
// simplex with Bland's rule over at most 64 planes and 6 coordinates.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "hv_internal.cuh"
#include "hv_host.h"

namespace hv {

namespace {

// sum a_k b_k in double-double, rounded once
double dot_dd(const double* a, const double* b, int d) {
    double hi = 0, lo = 0;
    for (int k = 0; k < d; ++k) {
        const double p = a[k] * b[k];
        const double pe = std::fma(a[k], b[k], -p);
        const double s = hi + p;
        const double bb = s - hi;
        const double se = (hi - (s - bb)) + (p - bb);
        hi = s;
        lo += se + pe;
    }
    return hi + lo;
}

// max c.z subject to A z <= b, z >= 0, with b >= 0 (z = 0 feasible).  A is
// m x nv row-major.  Returns 0 and the optimum in *val (and z if given), 1 if
// unbounded, 2 if the pivot budget ran out.
int lp_max(int m, int nv, const std::vector<double>& A, const std::vector<double>& b, const std::vector<double>& c,
           double* val, std::vector<double>* z) {
    const int W = nv + m + 1;  // columns: z, slacks, rhs
    std::vector<double> T((size_t)(m + 1) * W, 0.0);
    std::vector<int> basis(m);
    for (int i = 0; i < m; ++i) {
        for (int j = 0; j < nv; ++j) T[(size_t)i * W + j] = A[(size_t)i * nv + j];
        T[(size_t)i * W + nv + i] = 1.0;
        T[(size_t)i * W + W - 1] = b[i];
        basis[i] = nv + i;
    }
    double* obj = &T[(size_t)m * W];  // reduced costs: obj row = -c
    for (int j = 0; j < nv; ++j) obj[j] = -c[j];
    const double eps = 1e-12;
    for (int it = 0; it < 5000; ++it) {
        int e = -1;  // Bland: lowest index with negative reduced cost
        for (int j = 0; j < nv + m; ++j)
            if (obj[j] < -eps) { e = j; break; }
        if (e < 0) {
            *val = obj[W - 1];
            if (z) {
                z->assign(nv, 0.0);
                for (int i = 0; i < m; ++i)
                    if (basis[i] < nv) (*z)[basis[i]] = T[(size_t)i * W + W - 1];
            }
            return 0;
        }
        int r = -1;
        double best = 0;
        for (int i = 0; i < m; ++i) {
            const double a = T[(size_t)i * W + e];
            if (a > eps) {
                const double q = T[(size_t)i * W + W - 1] / a;
                if (r < 0 || q < best || (q == best && basis[i] < basis[r])) { r = i; best = q; }
            }
        }
        if (r < 0) return 1;
        const double pv = T[(size_t)r * W + e];
        for (int j = 0; j < W; ++j) T[(size_t)r * W + j] /= pv;
        for (int i = 0; i <= m; ++i) {
            if (i == r) continue;
            const double f = T[(size_t)i * W + e];
            if (f == 0) continue;
            for (int j = 0; j < W; ++j) T[(size_t)i * W + j] -= f * T[(size_t)r * W + j];
        }
        basis[r] = e;
    }
    return 2;
}

}  // namespace

void box_planes(int d, const double* lo, const double* hi, DevPlane* out) {
    for (int k = 0; k < d; ++k)
        for (int s = 0; s < 2; ++s) {
            DevPlane& P = out[2 * k + s];
            std::memset(&P, 0, sizeof(P));
            P.n[k] = s == 0 ? 1.0 : -1.0;
            P.off = s == 0 ? hi[k] : -lo[k];
            P.axis = k;
            P.sgn = s == 0 ? 1 : -1;
            for (int q = 0; q < HV_MAXD; ++q) P.n32[q] = (float)P.n[q];
            P.off32 = (float)P.off;
        }
}

std::string make_planes(int d, int np, const double* base, const double* normal, DevPlane* out) {
    if (np < 1 || np > HV_MAXP) return "plane count must be between 1 and 64";
    for (int p = 0; p < np; ++p) {
        const double* b = base + (size_t)p * d;
        const double* nv = normal + (size_t)p * d;
        double s = 0;
        int nz = 0, ax = -1;
        for (int k = 0; k < d; ++k) {
            if (!std::isfinite(b[k]) || !std::isfinite(nv[k])) return "plane base and normal must be finite";
            s += nv[k] * nv[k];
            if (nv[k] != 0) { ++nz; ax = k; }
        }
        if (!(s > 0)) return "plane normal must be non-zero";
        DevPlane& P = out[p];
        std::memset(&P, 0, sizeof(P));
        if (nz == 1) {  // axis plane: exact +-e_k and off = +-b_k
            P.axis = ax;
            P.sgn = nv[ax] > 0 ? 1 : -1;
            P.n[ax] = (double)P.sgn;
            P.off = P.sgn > 0 ? b[ax] : -b[ax];
        } else {
            const double inv = 1.0 / std::sqrt(s);
            for (int k = 0; k < d; ++k) P.n[k] = nv[k] * inv;
            P.off = dot_dd(P.n, b, d);
            P.axis = -1;
            P.sgn = 0;
        }
        for (int q = 0; q < HV_MAXD; ++q) P.n32[q] = (float)P.n[q];
        P.off32 = (float)P.off;
    }
    return std::string();
}

std::string planes_bbox(int d, int np, const DevPlane* P, double* lo, double* hi) {
    // pure cuboid (one upper and one lower axis plane per coordinate, any order)
    {
        bool hl[HV_MAXD] = {}, hh[HV_MAXD] = {};
        double l[HV_MAXD], h[HV_MAXD];
        bool axis_only = true;
        for (int p = 0; p < np; ++p) {
            if (P[p].axis < 0) { axis_only = false; break; }
            const int k = P[p].axis;
            if (P[p].sgn > 0) { h[k] = hh[k] ? std::min(h[k], P[p].off) : P[p].off; hh[k] = true; }
            else { l[k] = hl[k] ? std::max(l[k], -P[p].off) : -P[p].off; hl[k] = true; }
        }
        if (axis_only) {
            for (int k = 0; k < d; ++k) {
                if (!hl[k] || !hh[k]) return "domain is unbounded";
                if (!(l[k] < h[k])) return "domain has an empty interior";
                lo[k] = l[k]; hi[k] = h[k];
            }
            return std::string();
        }
    }
    // Chebyshev centre: max r subject to n_p.x + r <= off_p, with x = x+ - x-
    // and r = r0 + r+ - r- (r0 = min off - 1 makes the origin strictly feasible).
    double r0 = 0;
    for (int p = 0; p < np; ++p) r0 = p == 0 ? P[p].off : std::min(r0, P[p].off);
    r0 -= 1.0;
    const int nv = 2 * d + 2;
    std::vector<double> A((size_t)np * nv), b(np), c(nv, 0.0);
    for (int p = 0; p < np; ++p) {
        for (int k = 0; k < d; ++k) { A[(size_t)p * nv + 2 * k] = P[p].n[k]; A[(size_t)p * nv + 2 * k + 1] = -P[p].n[k]; }
        A[(size_t)p * nv + 2 * d] = 1.0;
        A[(size_t)p * nv + 2 * d + 1] = -1.0;
        b[p] = P[p].off - r0;
    }
    c[2 * d] = 1.0; c[2 * d + 1] = -1.0;
    double val = 0;
    std::vector<double> z;
    int rc = lp_max(np, nv, A, b, c, &val, &z);
    if (rc == 1) return "domain is unbounded";
    if (rc != 0) return "domain linear program did not converge";
    const double r = r0 + val;
    double xc[HV_MAXD] = {}, scale = 0;
    for (int k = 0; k < d; ++k) { xc[k] = z[2 * k] - z[2 * k + 1]; scale = std::max(scale, std::fabs(xc[k])); }
    for (int p = 0; p < np; ++p) scale = std::max(scale, std::fabs(P[p].off));
    if (!(r > 1e-12 * (1.0 + scale))) return "domain has an empty interior";
    // bounding box from the centre: y = x - xc, n_p.y <= off_p - n_p.xc (>= r > 0)
    const int nv2 = 2 * d;
    std::vector<double> A2((size_t)np * nv2), b2(np), c2(nv2);
    for (int p = 0; p < np; ++p) {
        double s = P[p].off;
        for (int k = 0; k < d; ++k) {
            A2[(size_t)p * nv2 + 2 * k] = P[p].n[k];
            A2[(size_t)p * nv2 + 2 * k + 1] = -P[p].n[k];
            s -= P[p].n[k] * xc[k];
        }
        b2[p] = std::max(s, 0.0);
    }
    for (int k = 0; k < d; ++k)
        for (int sg = 0; sg < 2; ++sg) {
            std::fill(c2.begin(), c2.end(), 0.0);
            c2[2 * k] = sg == 0 ? 1.0 : -1.0;
            c2[2 * k + 1] = -c2[2 * k];
            rc = lp_max(np, nv2, A2, b2, c2, &val, nullptr);
            if (rc == 1) return "domain is unbounded";
            if (rc != 0) return "domain linear program did not converge";
            if (sg == 0) hi[k] = xc[k] + val; else lo[k] = xc[k] - val;
        }
    // widen by a relative margin: the box must contain the domain
    for (int k = 0; k < d; ++k) {
        const double m = 1e-9 * (1.0 + std::fabs(lo[k]) + std::fabs(hi[k]));
        lo[k] -= m; hi[k] += m;
    }
    return std::string();
}

}  // namespace hv
