// hv_api.cu -- host orchestration and the C ABI of libhvgpu (include/hvgpu.h).
//
// hv_mesh_build replaces voronoi(mesh; searcher) (src/sysvoronoi.jl:21-39):
//   prepare   Morton sort, tree, candidate lists
//   seeds     descent from every seed_stride-th generator (src/raycast.jl:45-109)
//   wavefront level k expands the vertices found at level k-1; every level is
//             one expansion launch (+ the exact fallback and the FP64 centres);
//             the reference repeats its cell loop until nothing new is found
//             (src/sysvoronoi.jl:152-215), here until a level finds nothing new
//   canonical vertices renumbered in lexicographic signature order
// All device memory comes from the device's stream-ordered pool; the pool
// keeps freed blocks cached so repeated builds make no CUDA allocation calls.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <map>
#include <functional>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "hv_host.h"
#include "hv_degen.h"
#include "hv_integrate.h"
#include "hv_internal.cuh"
#include "hv_periodic.h"
#include "hvgpu.h"

struct hv_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;  // the fallback ladder of a level, beside the next level's expansion
    cudaStream_t stream3 = nullptr;  // the edge registry of a frontier, beside its circumcentres
    cudaEvent_t ovl_ev[6] = {};      // expansion, fallback (two parities), registry, lists of the non-seeds; no timing
    int nsm = 1;
    std::string err;
    unsigned* h_stat = nullptr;  // pinned: vcount, status, queue length, pad
    std::vector<cudaEvent_t> evpool;  // timing events, reused across builds
    std::map<std::pair<int, int>, hv_params> tuned;  // autotuner results per (d, log2 n)
};

struct hv_mesh {
    hv_ctx* ctx = nullptr;
    int d = 0;
    int n = 0;
    double lo[HV_MAXD], hi[HV_MAXD];  // bounding box of the domain
    int np = 0;                       // boundary planes, generator ids n .. n+np-1
    hv::DevPlane planes[hv::HV_MAXP];
    hv::DevPlane* d_planes = nullptr;
    hv_params prm;
    double* d_in = nullptr;  // points in original order (n x d)
    unsigned V = 0;
    int* osig = nullptr;     // V x (d+1) original 0-based items, canonical order
    double* oc = nullptr;    // V x d
    long long* inc_off = nullptr;
    int* inc = nullptr;
    long long* nbr_off = nullptr;
    int* nbr = nullptr;
    long long nnbr = -1;
    hv_stats st;
    // periodic cuboid: the public view above is reduced from the mesh of the
    // generators and their images in the widened box
    int pmask = 0;
    hv_mesh* ext = nullptr;
    int nimg = 0;
    double delta[HV_MAXD] = {};
    int* img_ref = nullptr;            // nimg originals
    short* img_code = nullptr;         // nimg shift codes sum (s_k + 1) 3^k
    signed char* pshift = nullptr;     // nnbr x d lattice shifts of the neighbours
    int* pperm = nullptr;              // nnbr: position in the extended row
    // shard of a mesh split over ranks: generators own0 .. own1-1 of the
    // internal (Morton) order (-1: the whole mesh)
    int own0 = -1, own1 = -1;
    // incremental refinement: generators own_from .. n-1 are new (-1: none)
    int own_from = -1;
    // integrand quadrature of VI_POLYGON (hv_quad.cu), built on first use
    long long* q_foff = nullptr;  // nnbr + 1: incidence range of each facet slot (lower cells)
    int* q_slot = nullptr;        // nnbr: cell of each slot
    unsigned* q_v = nullptr;      // facet vertices in id order
    double* q_w = nullptr;        // their flag weights
    double* q_a = nullptr;        // nnbr: flag sums
    double* q_c = nullptr;        // nnbr x d: facet centres
    double* q_af = nullptr;       // nnbr: facet areas
    bool q_weights = false;       // the flag weights are in q_w (not only lists and centres)
    // vertices with more than d+1 generators (hv_degen.cu): every vertex's
    // generator list as a CSR in canonical order; osig is then null
    int g_max = 0;                // longest list (0: the fixed-width osig holds the vertices)
    long long* g_off = nullptr;   // V + 1
    int* g_sig = nullptr;         // g_off[V] original 0-based items, ascending per vertex
    int* g_fcell = nullptr;       // nnbr: cell of each neighbour slot
    long long* g_fbeg = nullptr;  // nnbr: the facet's vertices are g_fvert[g_fbeg .. g_fend)
    long long* g_fend = nullptr;
    int* g_fvert = nullptr;
    bool allow_generic = false;   // a search that meets co-spherical generators walks them here
    // the search's kd-tree, kept for hv_mesh_verify: points in Morton order,
    // internal -> original ids, node boxes (2P x DP floats each)
    double* t_pts = nullptr;
    int* t_perm = nullptr;
    float* t_blo = nullptr;
    float* t_bhi = nullptr;
    int t_leaf = 0, t_nleaves = 0, t_P = 0;
};

namespace {

struct HvError : std::runtime_error {
    int code;
    HvError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CK(x)                                                                                      \
    do {                                                                                           \
        cudaError_t e_ = (x);                                                                      \
        if (e_ != cudaSuccess) {                                                                   \
            throw HvError(e_ == cudaErrorMemoryAllocation ? HV_E_OOM : HV_E_CUDA,                  \
                          std::string(#x) + ": " + cudaGetErrorString(e_));                        \
        }                                                                                          \
    } while (0)

// Stream-ordered scratch allocations released when the scope ends.
struct Scratch {
    cudaStream_t st;
    std::vector<void*> ptrs;
    explicit Scratch(cudaStream_t s) : st(s) {}
    template <class T>
    T* get(size_t count) {
        void* p = nullptr;
        CK(cudaMallocAsync(&p, std::max<size_t>(count * sizeof(T), 16), st));
        ptrs.push_back(p);
        return (T*)p;
    }
    void release_all() {
        for (void* p : ptrs) cudaFreeAsync(p, st);
        ptrs.clear();
    }
    ~Scratch() { release_all(); }
};

template <class T>
T* dalloc(cudaStream_t st, size_t count) {
    void* p = nullptr;
    CK(cudaMallocAsync(&p, std::max<size_t>(count * sizeof(T), 16), st));
    return (T*)p;
}

void dfree(cudaStream_t st, void* p) {
    if (p) cudaFreeAsync(p, st);
}

__global__ void k_iota(int* a, unsigned n) {
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = (int)i;
}

unsigned next_pow2(unsigned long long x) {
    unsigned long long p = 1;
    while (p < x) p <<= 1;
    return (unsigned)p;
}

// Candidate list length per dimension, measured on GB300 (sweeps over 2D/1k,
// 3D/100k, 4D/20k, 5D/20k uniform and 50k clustered, 6D/10k): shorter lists
// trade kNN and scan work for more rays that leave the list's complete radius.
int default_knn(int d) {
    static const int k[7] = {0, 0, 24, 64, 128, 256, 384};
    return k[d];
}

// One descent seed per `stride` generators (measured with the list lengths
// above): every seed costs d dependent rays, fewer seeds cost wavefront levels.
int default_seed_stride(long long n) { return n <= 4096 ? 1 : (n < 65536 ? 8 : 16); }

// Expected vertices per generator for uniform points in the cube (the
// reference's own counts, docs/src/index.md:93-96, extrapolated to 2, 3, 6).
double vertices_per_point(int d) {
    static const double c[7] = {0, 0, 2.2, 7.0, 30.0, 150.0, 1400.0};
    return c[d];
}

double ms_between(cudaEvent_t a, cudaEvent_t b) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

struct Events {
    cudaEvent_t e[4];
    Events() { for (auto& x : e) cudaEventCreate(&x); }
    ~Events() { for (auto& x : e) cudaEventDestroy(x); }
};

// Device time per kernel family: events recorded on the context's stream
// around every launch, summed once the build has synchronised.
enum Fam { F_KNN, F_DESCENT, F_EXPAND, F_FALLBACK, F_CENTERS, F_CANON, F_OTHER, F_N };
struct KTimer {
    hv_ctx* ctx;
    std::vector<std::pair<int, int>> spans;  // (family, first event index)
    size_t used = 0;
    long long launches = 0;
    explicit KTimer(hv_ctx* c) : ctx(c) {}
    cudaEvent_t next() {
        if (used == ctx->evpool.size()) {
            cudaEvent_t e;
            CK(cudaEventCreate(&e));
            ctx->evpool.push_back(e);
        }
        return ctx->evpool[used++];
    }
    template <class F>
    void run(int fam, int nlaunch, F&& f) { run_on(ctx->stream, fam, nlaunch, f); }
    template <class F>
    void run_on(cudaStream_t s, int fam, int nlaunch, F&& f) {
        const int i0 = (int)used;
        CK(cudaEventRecord(next(), s));
        f();
        CK(cudaEventRecord(next(), s));
        spans.emplace_back(fam, i0);
        launches += nlaunch;
    }
    void totals(double* ms) const {  // after synchronisation
        for (int f = 0; f < F_N; ++f) ms[f] = 0;
        for (auto& sp : spans) {
            float t = 0.f;
            cudaEventElapsedTime(&t, ctx->evpool[sp.second], ctx->evpool[sp.second + 1]);
            ms[sp.first] += t;
        }
    }
};

// vertex count and status word into h_stat[0..1] (h_stat[2..3] are the caller's)
// Queued rays per SM above which a level's fallback ladder is not overlapped with
// the next expansion (HV_OVERLAP_RAYS_PER_SM overrides, for tuning).
int overlap_rays_per_sm() {
    static const int v = [] {
        const char* e = std::getenv("HV_OVERLAP_RAYS_PER_SM");
        const int x = e ? std::atoi(e) : 0;
        return x > 0 ? x : 128;
    }();
    return v;
}

// HV_GRAPH=1 runs the wavefront's levels as one CUDA graph launch (device-side
// level loop), HV_GRAPH=0 from the host (one synchronisation per level).
bool use_graph(long long n) {
    const char* e = std::getenv("HV_GRAPH");
    (void)n;
    return e && std::atoi(e) == 1;
}

void read_stat(hv_ctx* ctx, const unsigned* dstat) {
    CK(cudaMemcpyAsync(ctx->h_stat, dstat, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
}

void check_fatal(unsigned status) {
    using namespace hv;
    if (status & ST_BADINPUT) throw HvError(HV_E_INVALID_ARG, "points must lie strictly inside the domain and be finite");
    if (status & ST_TIMEOUT) throw HvError(HV_E_TIMEOUT, "a bounded device wait gave up");
    if (status & (ST_NUMERIC | ST_STACK | ST_AMB | ST_DESCENT))
        throw HvError(HV_E_INTERNAL, "device search failed (status " + std::to_string(status) + ")");
}

// A corner of the domain: the first d planes (in id order) whose hyperplanes
// meet in one point inside all the others; the walk starts at its Voronoi
// vertex (the corner, its planes and its nearest generators).
bool domain_corner(const hv_mesh* mesh, double* v) {
    const int d = mesh->d, np = mesh->np;
    int idx[HV_MAXD];
    for (int q = 0; q < d; ++q) idx[q] = q;
    if (np < d) return false;
    for (;;) {
        double A[HV_MAXD][HV_MAXD], b[HV_MAXD];
        for (int r = 0; r < d; ++r) {
            for (int k = 0; k < d; ++k) A[r][k] = mesh->planes[idx[r]].n[k];
            b[r] = mesh->planes[idx[r]].off;
        }
        bool ok = true;
        for (int c = 0; c < d && ok; ++c) {  // Gaussian elimination, partial pivoting
            int p = c;
            for (int r = c + 1; r < d; ++r) if (std::fabs(A[r][c]) > std::fabs(A[p][c])) p = r;
            if (!(std::fabs(A[p][c]) > 1e-12)) { ok = false; break; }
            std::swap(A[p], A[c]);
            std::swap(b[p], b[c]);
            for (int r = c + 1; r < d; ++r) {
                const double f = A[r][c] / A[c][c];
                for (int k = c; k < d; ++k) A[r][k] -= f * A[c][k];
                b[r] -= f * b[c];
            }
        }
        if (ok) {
            for (int r = d - 1; r >= 0; --r) {
                double t = b[r];
                for (int k = r + 1; k < d; ++k) t -= A[r][k] * v[k];
                v[r] = t / A[r][r];
            }
            bool inside = true;
            for (int p = 0; p < np && inside; ++p) {
                double h = mesh->planes[p].off;
                double sc = std::fabs(mesh->planes[p].off);
                for (int k = 0; k < d; ++k) { h -= mesh->planes[p].n[k] * v[k]; sc += std::fabs(v[k]); }
                inside = h >= -1e-12 * (sc + 1.0);
            }
            if (inside) return true;
        }
        int q = d - 1;
        while (q >= 0 && idx[q] == np - d + q) --q;
        if (q < 0) return false;
        ++idx[q];
        for (int r = q + 1; r < d; ++r) idx[r] = idx[r - 1] + 1;
    }
}

// Vertices with more than d+1 generators: the search met co-spherical
// generators (or HV_METHOD_GENERIC asked for this walk).  The vertex graph is
// walked from a corner of the domain with every vertex keeping all generators
// on its sphere (hv_degen.cu); the result is a CSR of generator lists in place
// of the fixed-width vertex list, and the neighbour lists keep the pairs that
// share a full interface.  The device tree, points and planes of the search
// (M) are reused; the walk starts from the search's vertices (seed_sig,
// nseed x (d+1) internal ids) when there are any, else from a domain corner.
void generic_build(hv_ctx* ctx, hv_mesh* mesh, const hv::DevMesh& M, const int* seed_sig = nullptr,
                   unsigned nseed = 0) {
    using namespace hv;
    cudaStream_t st = ctx->stream;
    const int d = mesh->d, n = mesh->n;
    double corner[HV_MAXD];
    const bool have_corner = domain_corner(mesh, corner);
    if (nseed == 0 && !have_corner) throw HvError(HV_E_INTERNAL, "degenerate walk: no corner of the domain found");
    int W = std::min(GMAX, std::max(2 * (d + 1), (1 << d) + 2 * d));
    const unsigned long long vest = (unsigned long long)(vertices_per_point(d) * n) + (1ull << d) + 1024;
    for (int attempt = 0;; ++attempt) {
        if (attempt > 6) throw HvError(HV_E_CAPACITY, "degenerate walk: capacity retries exhausted");
        const unsigned long long vcap64 = vest << std::min(attempt, 5);
        if (vcap64 > 0x7FFFFFF0ull) throw HvError(HV_E_CAPACITY, "degenerate walk: vertex count beyond 31-bit ids");
        Scratch s(st);
        GenRun R{};
        R.M = M;
        R.x = mesh->d_in;
        R.W = W;
        R.vcap = (unsigned)vcap64;
        R.vsig = s.get<int>((size_t)R.vcap * W);
        R.vlen = s.get<int>(R.vcap);
        R.vc = s.get<double>((size_t)R.vcap * d);
        const unsigned long long hsize = next_pow2(2ull * R.vcap);
        R.hmask = hsize - 1;
        R.htab = s.get<unsigned long long>(hsize);
        CK(cudaMemsetAsync(R.htab, 0xFF, sizeof(unsigned long long) * hsize, st));
        unsigned* cnt = s.get<unsigned>(4);  // vertices, records, edges, status
        CK(cudaMemsetAsync(cnt, 0, 4 * sizeof(unsigned), st));
        R.vcnt = cnt; R.rcnt = cnt + 1; R.e_cnt = cnt + 2; R.status = cnt + 3;
        unsigned hc[4] = {0, 0, 0, 0};
        auto read = [&] {
            CK(cudaMemcpyAsync(hc, cnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
        };
        std::unique_ptr<Scratch> es;
        auto grow_edges = [&](unsigned need) {
            es.reset(new Scratch(st));
            R.e_cap = std::max(need, 4096u);
            R.e_vert = es->get<unsigned>(R.e_cap);
            R.e_F = es->get<unsigned long long>(R.e_cap);
            R.e_u = es->get<double>((size_t)R.e_cap * d);
            R.rcap = R.e_cap;
            R.rsig = es->get<int>((size_t)R.rcap * W);
            R.rlen = es->get<int>(R.rcap);
            R.rc = es->get<double>((size_t)R.rcap * d);
            R.rwin = es->get<unsigned>(R.rcap);
        };
        grow_edges(std::max(64u * (d + 1), nseed));
        if (nseed > 0) {  // many starting points: the levels span the gaps between them
            launch_gen_seeds(R, seed_sig, nseed, ctx->nsm, st);
            CK(cudaGetLastError());
            read();
            launch_gen_insert(R, hc[1], st);
            launch_gen_commit(R, hc[1], st);
            CK(cudaGetLastError());
            read();
        }
        if (hc[0] == 0 && have_corner && !hc[3]) {  // no seed survived (or none given): the corner
            double* dcorner = s.get<double>(d);
            CK(cudaMemcpyAsync(dcorner, corner, sizeof(double) * d, cudaMemcpyHostToDevice, st));
            launch_gen_seed(R, dcorner, st);
        }
        CK(cudaGetLastError());
        read();
        unsigned f0 = 0, f1 = hc[0];
        long long levels = 0;
        while (!hc[3] && f1 > f0) {
            for (;;) {
                CK(cudaMemsetAsync(R.e_cnt, 0, sizeof(unsigned), st));
                CK(cudaMemsetAsync(R.rcnt, 0, sizeof(unsigned), st));
                launch_gen_edges(R, f0, f1, ctx->nsm, st);
                CK(cudaGetLastError());
                read();
                if (hc[2] <= R.e_cap || hc[3]) break;
                grow_edges(hc[2] + hc[2] / 2);
            }
            if (hc[3]) break;
            launch_gen_walk(R, hc[2], ctx->nsm, st);
            CK(cudaGetLastError());
            read();
            if (hc[3]) break;
            launch_gen_insert(R, hc[1], st);
            launch_gen_commit(R, hc[1], st);
            CK(cudaGetLastError());
            read();
            f0 = f1;
            f1 = std::min(hc[0], R.vcap);
            ++levels;
        }
        es.reset();
        if (hc[3] & (GS_CAP | GS_HASH)) continue;
        if (hc[3] & GS_WIDE) {
            if (W == GMAX) throw HvError(HV_E_CAPACITY, "a degenerate vertex has more than 64 generators");
            W = GMAX;
            continue;
        }
        if (hc[3] & GS_SUBSETS)
            throw HvError(HV_E_CAPACITY, "a degenerate vertex has too many generators to enumerate its edges");
        if (hc[3]) throw HvError(HV_E_INTERNAL, "degenerate walk: singular vertex system or an edge without end");
        // ---- canonical order and the generator-list CSR
        const unsigned V = f1;
        int* order = s.get<int>(std::max(V, 1u));
        {
            const size_t tb = gen_sort_temp(V);
            void* tmp = s.get<char>(tb);
            gen_sort(R, V, order, tmp, tb, st);
        }
        long long* lens = s.get<long long>((size_t)V + 1);
        unsigned* dmax = s.get<unsigned>(1);
        CK(cudaMemsetAsync(lens + V, 0, sizeof(long long), st));
        CK(cudaMemsetAsync(dmax, 0, sizeof(unsigned), st));
        launch_gen_lens(R, V, order, lens, dmax, st);
        long long* goff = dalloc<long long>(st, (size_t)V + 1);
        {
            const size_t tb = scan_temp((int)V + 1);
            void* tmp = s.get<char>(tb);
            exclusive_scan_i64(tmp, tb, lens, goff, (int)V + 1, st);
        }
        long long total = 0;
        unsigned gmax = 0;
        CK(cudaMemcpyAsync(&total, goff + V, sizeof(long long), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(&gmax, dmax, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        int* gsig = dalloc<int>(st, (size_t)std::max(total, 1ll));
        double* oc = dalloc<double>(st, (size_t)std::max(V, 1u) * d);
        launch_gen_fill(R, V, order, goff, gsig, oc, st);
        dfree(st, mesh->osig);
        dfree(st, mesh->oc);
        mesh->osig = nullptr;
        mesh->oc = oc;
        mesh->g_off = goff;
        mesh->g_sig = gsig;
        mesh->g_max = (int)gmax;
        mesh->V = V;
        // ---- neighbours sharing a full interface, and each facet's vertices
        long long* pc = s.get<long long>((size_t)V + 1);
        long long* poff = s.get<long long>((size_t)V + 1);
        CK(cudaMemsetAsync(pc + V, 0, sizeof(long long), st));
        launch_gen_pair_count(n, V, goff, gsig, pc, st);
        {
            const size_t tb = scan_temp((int)V + 1);
            void* tmp = s.get<char>(tb);
            exclusive_scan_i64(tmp, tb, pc, poff, (int)V + 1, st);
        }
        long long np = 0;
        CK(cudaMemcpyAsync(&np, poff + V, sizeof(long long), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (np > 0x7FFFFFF0ll) throw HvError(HV_E_CAPACITY, "degenerate walk: too many generator pairs");
        unsigned long long* keys = s.get<unsigned long long>((size_t)std::max(np, 1ll));
        unsigned long long* keys2 = s.get<unsigned long long>((size_t)std::max(np, 1ll));
        int* vals = s.get<int>((size_t)std::max(np, 1ll));
        int* vals2 = dalloc<int>(st, (size_t)std::max(np, 1ll));
        mesh->g_fvert = vals2;
        launch_gen_pair_emit(n, V, goff, gsig, poff, keys, vals, st);
        if (np > 0) {
            const size_t tb = sort_pairs_u64_i32_temp((int)np);
            void* tmp = s.get<char>(tb);
            sort_pairs_u64_i32(tmp, tb, keys, keys2, vals, vals2, (int)np, 64, st);
        }
        long long* keep = s.get<long long>((size_t)np + 1);
        long long* kpos = s.get<long long>((size_t)np + 1);
        long long* qend = s.get<long long>((size_t)std::max(np, 1ll));
        CK(cudaMemsetAsync(keep + np, 0, sizeof(long long), st));
        launch_gen_heads(d, np, keys2, vals2, goff, oc, keep, qend, st);
        {
            const size_t tb = scan_temp((int)np + 1);
            void* tmp = s.get<char>(tb);
            exclusive_scan_i64(tmp, tb, keep, kpos, (int)np + 1, st);
        }
        long long nn = 0;
        CK(cudaMemcpyAsync(&nn, kpos + np, sizeof(long long), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        mesh->nbr = dalloc<int>(st, (size_t)std::max(nn, 1ll));
        mesh->g_fcell = dalloc<int>(st, (size_t)std::max(nn, 1ll));
        mesh->g_fbeg = dalloc<long long>(st, (size_t)std::max(nn, 1ll));
        mesh->g_fend = dalloc<long long>(st, (size_t)std::max(nn, 1ll));
        long long* ncnt = s.get<long long>((size_t)n + 1);
        CK(cudaMemsetAsync(ncnt, 0, sizeof(long long) * (n + 1), st));
        launch_gen_slots(np, keys2, keep, kpos, qend, mesh->nbr, mesh->g_fcell, mesh->g_fbeg, mesh->g_fend, ncnt, st);
        mesh->nbr_off = dalloc<long long>(st, (size_t)n + 1);
        {
            const size_t tb = scan_temp(n + 1);
            void* tmp = s.get<char>(tb);
            exclusive_scan_i64(tmp, tb, ncnt, mesh->nbr_off, n + 1, st);
        }
        // ---- cell -> vertex incidence
        unsigned long long* ik = s.get<unsigned long long>((size_t)std::max(total, 1ll));
        unsigned long long* ik2 = s.get<unsigned long long>((size_t)std::max(total, 1ll));
        long long* icnt = s.get<long long>((size_t)n + 1);
        CK(cudaMemsetAsync(icnt, 0, sizeof(long long) * (n + 1), st));
        launch_gen_inc_emit(n, V, goff, gsig, ik, icnt, st);
        if (total > 0) {
            const size_t tb = sort_keys_u64_temp(total);
            void* tmp = s.get<char>(tb);
            sort_keys_u64(tmp, tb, ik, ik2, total, st);
        }
        mesh->inc_off = dalloc<long long>(st, (size_t)n + 1);
        {
            const size_t tb = scan_temp(n + 1);
            void* tmp = s.get<char>(tb);
            exclusive_scan_i64(tmp, tb, icnt, mesh->inc_off, n + 1, st);
        }
        long long ninc = 0;
        CK(cudaMemcpyAsync(&ninc, mesh->inc_off + n, sizeof(long long), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        mesh->inc = dalloc<int>(st, (size_t)std::max(ninc, 1ll));
        launch_inc_split((unsigned long long)ninc, ik2, mesh->inc, st);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(st));
        mesh->nnbr = nn;
        mesh->st.vertices = V;
        mesh->st.levels += levels;
        return;
    }
}

void build_impl(hv_ctx* ctx, hv_mesh* mesh, const double* d_src, bool src_on_device, const double* h_src) {
    using namespace hv;
    const int d = mesh->d, n = mesh->n;
    const int DP = d <= 4 ? 4 : 8;
    cudaStream_t st = ctx->stream;
    Events ev;
    auto t0 = std::chrono::steady_clock::now();
    CK(cudaEventRecord(ev.e[0], st));
    mesh->d_in = dalloc<double>(st, (size_t)n * d);
    mesh->d_planes = dalloc<DevPlane>(st, (size_t)mesh->np);
    CK(cudaMemcpyAsync(mesh->d_planes, mesh->planes, sizeof(DevPlane) * mesh->np, cudaMemcpyHostToDevice, st));
    if (n > 0) {
        if (src_on_device)
            CK(cudaMemcpyAsync(mesh->d_in, d_src, sizeof(double) * n * d, cudaMemcpyDeviceToDevice, st));
        else
            CK(cudaMemcpyAsync(mesh->d_in, h_src, sizeof(double) * n * d, cudaMemcpyHostToDevice, st));
    }
    hv_stats& S = mesh->st;
    std::memset(&S, 0, sizeof(S));
    if (n == 0) {
        mesh->V = 0;
        CK(cudaStreamSynchronize(st));
        return;
    }
    Scratch prep(st);
    // the side streams' kernels use the mesh build's scratch: drain them before it is
    // freed (also when an error unwinds the build)
    struct Drain {
        cudaStream_t s2, s3;
        ~Drain() {
            cudaStreamSynchronize(s2);
            cudaStreamSynchronize(s3);
        }
    } drain{ctx->stream2, ctx->stream3};
    unsigned* dstat = prep.get<unsigned>(8);  // vcount, status, insecure queue, exact queue, ambiguous sets
    unsigned long long* dcnt = prep.get<unsigned long long>(C_NCOUNT);
    CK(cudaMemsetAsync(dstat, 0, 8 * sizeof(unsigned), st));
    CK(cudaMemsetAsync(dcnt, 0, C_NCOUNT * sizeof(unsigned long long), st));
    // ---- Morton order
    unsigned long long* codes = prep.get<unsigned long long>(n);
    unsigned long long* codes2 = prep.get<unsigned long long>(n);
    int* idx = prep.get<int>(n);
    // the tree (Morton-ordered points, permutation, boxes) stays with the mesh
    // for hv_mesh_verify
    int* perm = dalloc<int>(st, n);
    mesh->t_perm = perm;
    KTimer kt(ctx);
    kt.run(F_OTHER, 1, [&] { launch_morton(d, mesh->d_in, n, mesh->lo, mesh->hi, mesh->d_planes, mesh->np, codes, idx, dstat + 1, st); });
    {
        size_t tb = sort_pairs_u64_i32_temp(n);
        void* tmp = prep.get<char>(tb);
        sort_pairs_u64_i32(tmp, tb, codes, codes2, idx, perm, n, d * morton_bits(d, n), st);
    }
    double* pts = dalloc<double>(st, (size_t)n * d);
    mesh->t_pts = pts;
    float* pts32 = prep.get<float>((size_t)n * DP);
    float* pts32lo = prep.get<float>((size_t)n * DP);
    kt.run(F_OTHER, 1, [&] { launch_gather(d, mesh->d_in, perm, n, pts, pts32, pts32lo, st); });
    // ---- tree
    DevMesh M;
    std::memset(&M, 0, sizeof(M));
    M.d = d; M.n = n; M.dp = DP;
    const bool shard = mesh->own0 >= 0;
    M.own0 = shard ? mesh->own0 : 0;
    M.own1 = shard ? mesh->own1 : n;
    M.own_from = mesh->own_from;
    const bool restricted = shard || mesh->own_from >= 0;
    double xs = 0;
    for (int k = 0; k < d; ++k) {
        M.lo[k] = mesh->lo[k]; M.hi[k] = mesh->hi[k];
        xs = std::max(xs, std::max(std::fabs(mesh->lo[k]), std::fabs(mesh->hi[k])));
    }
    M.xscale = xs;
    M.np = mesh->np;
    M.planes = mesh->d_planes;
    M.box = mesh->np == 2 * d;
    for (int p = 0; p < mesh->np && M.box; ++p)
        M.box = mesh->planes[p].axis == p / 2 && mesh->planes[p].sgn == ((p & 1) == 0 ? 1 : -1);
    if (M.box)
        for (int k = 0; k < d; ++k) {
            M.lo32[k] = (float)(-mesh->planes[2 * k + 1].off);
            M.hi32[k] = (float)mesh->planes[2 * k].off;
        }
    M.xs32 = (float)xs;
    M.tiny32 = (float)(4e-14 * xs);
    M.e13_32 = (float)(1e-13 * xs);
    M.e12_32 = (float)(1e-12 * xs);
    M.ulp32 = (float)(xs * 5.9604645e-08);
    M.leaf = mesh->prm.leaf_size > 0 ? mesh->prm.leaf_size : 16;
    M.nleaves = (n + M.leaf - 1) / M.leaf;
    M.P = (int)next_pow2((unsigned long long)M.nleaves);
    M.pts = pts; M.pts32 = pts32; M.pts32lo = pts32lo; M.perm = perm;
    float* blo = dalloc<float>(st, (size_t)2 * M.P * DP);
    float* bhi = dalloc<float>(st, (size_t)2 * M.P * DP);
    mesh->t_blo = blo;
    mesh->t_bhi = bhi;
    mesh->t_leaf = M.leaf;
    mesh->t_nleaves = M.nleaves;
    mesh->t_P = M.P;
    unsigned* flags = prep.get<unsigned>((size_t)2 * M.P);
    CK(cudaMemsetAsync(flags, 0, sizeof(unsigned) * 2 * M.P, st));
    M.blo = blo; M.bhi = bhi;
    M.status = dstat + 1;
    M.cnt = dcnt;
    kt.run(F_OTHER, 1, [&] { launch_bvh(M, blo, bhi, flags, st); });
    // ---- candidate lists
    const bool fast = mesh->prm.method != HV_METHOD_PLAIN;  // HV_METHOD_GENERIC: its walk starts from the descent
    int K = mesh->prm.knn > 0 ? mesh->prm.knn : default_knn(d);
    K = std::min(K, std::max(n - 1, 0));
    K = std::min(K, 480);
    M.K = fast ? K : 0;
    // a shard seeds every one of its generators: its cells need not be connected
    // to each other through shared vertices
    const int stride = restricted ? 1 : (mesh->prm.seed_stride > 0 ? mesh->prm.seed_stride : default_seed_stride(n));
    bool knn_side = false;
    if (fast) {
        int* knn = prep.get<int>((size_t)n * std::max(K, 1));
        float* sec = prep.get<float>(n);
        M.knn = knn; M.sec = sec;
        // the descent needs only the seeds' lists: the other generators' lists are
        // computed on the second stream beside it and awaited before the first level
        knn_side = stride > 1;
        if (knn_side) {
            CK(cudaEventRecord(ctx->ovl_ev[4], st));
            CK(cudaStreamWaitEvent(ctx->stream2, ctx->ovl_ev[4], 0));
            kt.run_on(ctx->stream2, F_KNN, 1, [&] { launch_knn(M, knn, sec, stride, 1, ctx->stream2); });
            CK(cudaEventRecord(ctx->ovl_ev[5], ctx->stream2));
        }
        kt.run(F_KNN, 1, [&] { launch_knn(M, knn, sec, stride, 0, st); });
    }
    CK(cudaGetLastError());
    read_stat(ctx, dstat);
    check_fatal(ctx->h_stat[1]);
    CK(cudaEventRecord(ev.e[1], st));
    // ---- search with capacity retry
    double factor = mesh->prm.capacity_factor > 0 ? mesh->prm.capacity_factor : 1.3;
    unsigned long long est = (unsigned long long)(vertices_per_point(d) * n) + (1ull << d) + 1024;
    if (mesh->own_from >= 0)  // refinement: only the vertices of the new cells (d+1 cells share a vertex)
        est = std::min(est, (unsigned long long)(vertices_per_point(d) * (d + 1) * (n - mesh->own_from)) + 1024);
    const int nseeds = (M.own1 - M.own0 + stride - 1) / stride;
    // a tie that survives double-double: box and plane-domain builds stop the
    // search and walk the vertex graph with vertices of any size instead
    bool degen_abort = false;
    auto fatal = [&](unsigned stt) -> bool {
        if (mesh->allow_generic && (stt & ST_DEGEN) && !(stt & (ST_BADINPUT | ST_TIMEOUT))) {
            degen_abort = true;
            return true;
        }
        check_fatal(stt);
        return false;
    };
    std::unique_ptr<Scratch> srch;
    unsigned V = 0;
    unsigned nseed = 0;  // vertices found before a hand-over to the generic walk
    for (int attempt = 0;; ++attempt) {
        if (attempt > 4) throw HvError(HV_E_CAPACITY, "vertex capacity retries exhausted");
        unsigned long long vcap64 = (unsigned long long)(est * factor * (double)(1ull << attempt));
        if (vcap64 > 0xFFFFFFF0ull / 8) throw HvError(HV_E_CAPACITY, "vertex count beyond 32-bit ids");
        const unsigned vcap = (unsigned)vcap64;
        srch.reset();
        srch.reset(new Scratch(st));
        M.vcap = vcap;
        M.vsig = srch->get<int>((size_t)vcap * (d + 1));
        M.vc = srch->get<double>((size_t)vcap * d);
        M.vrho32 = srch->get<float>((size_t)vcap * DP);
        M.vinv32 = fast ? srch->get<float>((size_t)vcap * d * d) : nullptr;
        M.vcond = fast ? srch->get<float>(vcap) : nullptr;
        M.vnew = srch->get<int>(vcap);
        const unsigned hsize = next_pow2(2ull * vcap);
        M.vhmask = hsize - 1;
        M.vhash = srch->get<unsigned long long>(hsize);
        CK(cudaMemsetAsync(M.vhash, 0, sizeof(unsigned long long) * hsize, st));
        const bool dedup = mesh->prm.edge_dedup >= 0;
        M.ecnt = nullptr; M.ehash = nullptr; M.ehmask = 0;
        if (dedup) {
            M.ecnt = srch->get<unsigned>(vcap);
            CK(cudaMemsetAsync(M.ecnt, 0, sizeof(unsigned) * vcap, st));
            const unsigned esize = next_pow2((unsigned long long)vcap * (d + 1));
            M.ehmask = esize - 1;
            M.ehash = srch->get<unsigned long long>(esize);
            CK(cudaMemsetAsync(M.ehash, 0, sizeof(unsigned long long) * esize, st));
        }
        const unsigned fqcap = std::max(65536u, vcap / 2);
        // insecure rays (fq) and rays for the exact search (fx), one pair per level
        // parity: the ladder of level L drains its pair while level L+1 fills the other
        unsigned long long* fqs[2] = {nullptr, nullptr};
        unsigned long long* fxs[2] = {nullptr, nullptr};
        float* fqhs[2] = {nullptr, nullptr};  // the expansion's bound of every insecure ray
        if (fast)
            for (int p = 0; p < 2; ++p) {
                fqs[p] = srch->get<unsigned long long>(fqcap);
                fxs[p] = srch->get<unsigned long long>(fqcap);
                fqhs[p] = srch->get<float>(fqcap);
            }
        unsigned* qc = fast ? srch->get<unsigned>(4) : nullptr;  // nfq, nfx per parity
        // rays the expansion decided, inserted into the vertex hash by their own kernel
        // (a level decides fewer rays than the build has vertices)
        M.dq = nullptr; M.ndq = nullptr; M.dqcap = 0;
        if (fast) {
            M.dqcap = vcap;
            M.dq = srch->get<uint2>(M.dqcap);
            M.ndq = srch->get<unsigned>(1);
        }
        hv::AmbQueue aq{};  // ambiguous candidate sets of the FP32 tree search
        if (fast) {
            aq.cap = fqcap;
            aq.e = srch->get<unsigned long long>(aq.cap);
            aq.n = srch->get<int>(aq.cap);
            aq.ids = srch->get<int>((size_t)aq.cap * hv::AMB_SET);
            aq.count = dstat + 4;
        }
        M.vcount = dstat;
        CK(cudaMemsetAsync(dstat, 0, 8 * sizeof(unsigned), st));
        CK(cudaMemsetAsync(dcnt, 0, C_NCOUNT * sizeof(unsigned long long), st));
        int* dfail = fast ? srch->get<int>((size_t)nseeds) : nullptr;
        unsigned* ndfail = fast ? srch->get<unsigned>(1) : nullptr;
        if (fast) CK(cudaMemsetAsync(ndfail, 0, sizeof(unsigned), st));
        const unsigned long long dseed = mesh->prm.seed ? mesh->prm.seed : 0x5EEDull;
        kt.run(F_DESCENT, 1, [&] { launch_descent(M, stride, nseeds, dseed, dfail, ndfail, ctx->nsm, st); });
        CK(cudaGetLastError());
        read_stat(ctx, dstat);
        unsigned nundecided = 0;
        if (fast && d == 2 && mesh->allow_generic && ctx->h_stat[0] != 0 && !restricted) {
            CK(cudaMemcpyAsync(&nundecided, ndfail, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
        }
        // a quarter of the seeds undecided in FP32: ties everywhere (lattice points),
        // and the seeds' vertices will start the generic walk -- find them all.
        // In 2D only: there the exact descent of tied seeds is cheap (200^2
        // lattice: 34 ms, walk levels 401 -> 5), in 3D and 4D each tied descent
        // costs more than the levels it saves (32^3: 66 ms -> 1.9 s)
        const bool tied = d == 2 && 4ull * nundecided > (unsigned long long)nseeds;
        if (fast && (ctx->h_stat[0] == 0 || restricted || tied) && !(ctx->h_stat[1] & (ST_VCAP | ST_HASH))) {
            // no FP32 seed was decided (or a shard, whose every cell needs its
            // seed): the exact descent on the undecided ones
            kt.run(F_DESCENT, 1, [&] { launch_descent_exact(M, nseeds, dseed, dfail, ndfail, ctx->nsm, st); });
            CK(cudaGetLastError());
            read_stat(ctx, dstat);
        }
        const unsigned overflow_bits = ST_VCAP | ST_HASH | ST_QUEUE | ST_ECAP;
        bool overflow = (ctx->h_stat[1] & overflow_bits) != 0;
        // seeds that tie in every direction may find no vertex at all: with the
        // generic walk ahead, the others start it
        if (!overflow && tied && mesh->allow_generic && (ctx->h_stat[1] & ST_DESCENT)) degen_abort = true;
        if (!overflow && !degen_abort) fatal(ctx->h_stat[1]);
        if (!overflow && mesh->prm.method == HV_METHOD_GENERIC) degen_abort = true;  // the walk from the seeds
        unsigned f0 = 0, f1 = std::min(ctx->h_stat[0], vcap);
        if (degen_abort) f1 = 0;
        if (!overflow && !degen_abort) kt.run(F_CENTERS, 1, [&] { launch_centers(M, 0, f1, ctx->nsm, st); });
        long long levels = 0;
        if (fast) {
            // Level L expands [f0, f1) on the context's stream; its fallback ladder
            // (tree search, set decisions, exact search) runs on the second stream
            // beside the expansion of level L+1.  The vertices that ladder finds join
            // the frontier of level L+2, whose range is read once it has finished.
            // Overlap pays while a ladder is latency-bound (a few rays per SM); a
            // ladder of more than 128 rays per SM (clustered data) is work-bound and
            // would only contend with the expansion, so the next level waits for it.
            cudaStream_t st2 = ctx->stream2, st3 = ctx->stream3;
            cudaEvent_t ev_exp = ctx->ovl_ev[0], ev_reg = ctx->ovl_ev[3];
            if (knn_side) CK(cudaStreamWaitEvent(st, ctx->ovl_ev[5], 0));  // every generator's list
            bool pend = false;
            int pend_par = 0;
            // a new frontier [a, b): circumcentres on the main stream, the edge registry
            // beside them (both read only the signatures); the expansion waits for both
            static const bool side_registry = [] {
                const char* e = std::getenv("HV_EDGE_STREAM");
                return !(e && e[0] == '0');
            }();
            auto prepare = [&](unsigned a, unsigned b, bool centers) {
                if (centers) kt.run(F_CENTERS, 1, [&] { launch_centers(M, a, b, ctx->nsm, st); });
                if (dedup && !side_registry) {
                    kt.run(F_OTHER, 1, [&] { launch_register_edges(M, a, b, ctx->nsm, st); });
                } else if (dedup) {
                    kt.run_on(st3, F_OTHER, 1, [&] { launch_register_edges(M, a, b, ctx->nsm, st3); });
                    CK(cudaEventRecord(ev_reg, st3));
                    CK(cudaStreamWaitEvent(st, ev_reg, 0));
                }
            };
            if (!overflow && !degen_abort) prepare(f0, f1, false);  // the seeds' centres are queued already
            if (!overflow && !degen_abort && use_graph(n)) {
                // every level in one launch of a CUDA graph: a WHILE node whose body is
                // [ladder of the previous level | expansion] -> advance -> [centres | edge
                // registry]; the frontier and the level live in device memory
                unsigned* lvl = srch->get<unsigned>(4);
                const unsigned hl[4] = {f0, f1, 0, 0};
                CK(cudaMemcpyAsync(lvl, hl, sizeof(hl), cudaMemcpyHostToDevice, st));
                CK(cudaMemsetAsync(qc, 0, 4 * sizeof(unsigned), st));
                DevMesh G = M;
                G.G.lvl = lvl;
                G.G.qc = qc;
                for (int p = 0; p < 2; ++p) { G.G.fq[p] = fqs[p]; G.G.fx[p] = fxs[p]; G.G.fqh[p] = fqhs[p]; }
                G.fqh = nullptr;
                const unsigned stop_bits = overflow_bits | ST_BADINPUT | ST_TIMEOUT | ST_NUMERIC | ST_STACK |
                                           ST_AMB | ST_DESCENT;
                cudaGraph_t graph = nullptr;
                cudaGraphExec_t exec = nullptr;
                struct GraphFree {
                    cudaGraph_t* g; cudaGraphExec_t* e;
                    ~GraphFree() { if (*e) cudaGraphExecDestroy(*e); if (*g) cudaGraphDestroy(*g); }
                } gfree{&graph, &exec};
                launch_expand_fast(G, 0, 0, nullptr, nullptr, fqcap, nullptr, nullptr, fqcap, ctx->nsm, st);
                CK(cudaGraphCreate(&graph, 0));
                cudaGraphConditionalHandle handle;
                CK(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
                cudaGraphNodeParams cp = {};
                cp.type = cudaGraphNodeTypeConditional;
                cp.conditional.handle = handle;
                cp.conditional.type = cudaGraphCondTypeWhile;
                cp.conditional.size = 1;
                cudaGraphNode_t node;
                CK(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp));
                cudaGraph_t body = cp.conditional.phGraph_out[0];
                CK(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
                const unsigned qmax = fqcap;
                launch_level_begin(G, st);
                CK(cudaEventRecord(ctx->ovl_ev[0], st));
                CK(cudaStreamWaitEvent(st2, ctx->ovl_ev[0], 0));
                CK(cudaMemsetAsync(aq.count, 0, sizeof(unsigned), st2));
                launch_fallback_warp(G, nullptr, nullptr, fqcap, qmax, nullptr, nullptr, fqcap, aq, ctx->nsm, st2);
                launch_fallback(G, nullptr, nullptr, qmax, ctx->nsm, st2);
                CK(cudaEventRecord(ctx->ovl_ev[1], st2));
                launch_expand_fast(G, 0, vcap, nullptr, nullptr, fqcap, nullptr, nullptr, fqcap, ctx->nsm, st);
                CK(cudaStreamWaitEvent(st, ctx->ovl_ev[1], 0));
                launch_level_advance(G, handle, stop_bits, st);
                if (dedup) {
                    CK(cudaEventRecord(ctx->ovl_ev[2], st));
                    CK(cudaStreamWaitEvent(st3, ctx->ovl_ev[2], 0));
                    launch_register_edges(G, 0, vcap, ctx->nsm, st3);
                    CK(cudaEventRecord(ev_reg, st3));
                }
                launch_centers(G, 0, vcap, ctx->nsm, st);
                if (dedup) CK(cudaStreamWaitEvent(st, ev_reg, 0));
                CK(cudaStreamEndCapture(st, &body));
                CK(cudaGraphInstantiate(&exec, graph, 0));
                kt.run(F_EXPAND, 1, [&] { CK(cudaGraphLaunch(exec, st)); });
                unsigned hl2[4];
                CK(cudaMemcpyAsync(hl2, lvl, sizeof(hl2), cudaMemcpyDeviceToHost, st));
                read_stat(ctx, dstat);
                if (ctx->h_stat[1] & overflow_bits) overflow = true;
                else fatal(ctx->h_stat[1]);
                f0 = f1 = std::min(ctx->h_stat[0], vcap);
                levels = hl2[2];
            }
            for (int L = 0; !overflow && !degen_abort && !use_graph(n); ++L) {
                if (f1 == f0) {
                    if (!pend) break;
                    CK(cudaStreamWaitEvent(st, ctx->ovl_ev[1 + pend_par], 0));
                    pend = false;
                    read_stat(ctx, dstat);
                    if (ctx->h_stat[1] & overflow_bits) { overflow = true; break; }
                    if (fatal(ctx->h_stat[1])) break;
                    const unsigned e = std::min(ctx->h_stat[0], vcap);
                    if (e == f1) break;
                    prepare(f1, e, true);
                    f0 = f1; f1 = e;
                    continue;
                }
                const int p = L & 1;
                M.fqh = fqhs[p];  // the expansion and the ladder of this level share the parity
                CK(cudaMemsetAsync(qc + 2 * p, 0, 2 * sizeof(unsigned), st));
                kt.run(F_EXPAND, 2, [&] {
                    launch_expand_fast(M, f0, f1, fqs[p], qc + 2 * p, fqcap, fxs[p], qc + 2 * p + 1, fqcap,
                                       ctx->nsm, st);
                });
                CK(cudaEventRecord(ev_exp, st));
                CK(cudaStreamWaitEvent(st2, ev_exp, 0));
                const unsigned long long maxq =
                    std::min<unsigned long long>(fqcap, (unsigned long long)(f1 - f0) * (d + 1));
                CK(cudaMemsetAsync(aq.count, 0, sizeof(unsigned), st2));
                kt.run_on(st2, F_FALLBACK, 3, [&] {
                    launch_fallback_warp(M, fqs[p], qc + 2 * p, fqcap, (unsigned)maxq, fxs[p], qc + 2 * p + 1,
                                         fqcap, aq, ctx->nsm, st2);
                    launch_fallback(M, fxs[p], qc + 2 * p + 1, (unsigned)maxq, ctx->nsm, st2);
                });
                CK(cudaEventRecord(ctx->ovl_ev[1 + p], st2));
                CK(cudaGetLastError());
                if (pend) CK(cudaStreamWaitEvent(st, ctx->ovl_ev[1 + pend_par], 0));
                CK(cudaMemcpyAsync(ctx->h_stat + 2, qc + 2 * p, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
                read_stat(ctx, dstat);
                if (ctx->h_stat[1] & overflow_bits) { overflow = true; break; }
                if (fatal(ctx->h_stat[1])) break;
                if (ctx->h_stat[2] > (unsigned)overlap_rays_per_sm() * (unsigned)ctx->nsm) {  // work-bound: no overlap
                    CK(cudaStreamWaitEvent(st, ctx->ovl_ev[1 + p], 0));
                    read_stat(ctx, dstat);
                    if (ctx->h_stat[1] & overflow_bits) { overflow = true; break; }
                    if (fatal(ctx->h_stat[1])) break;
                }
                const unsigned e = std::min(ctx->h_stat[0], vcap);
                prepare(f1, e, true);
                f0 = f1; f1 = e;
                pend = true;
                pend_par = p;
                ++levels;
            }
            CK(cudaStreamSynchronize(st2));
            CK(cudaStreamSynchronize(st3));
        }
        while (!fast && !overflow && !degen_abort && f1 > f0) {
            if (dedup) kt.run(F_OTHER, 1, [&] { launch_register_edges(M, f0, f1, ctx->nsm, st); });
            kt.run(F_EXPAND, 1, [&] { launch_expand_plain(M, f0, f1, ctx->nsm, st); });
            CK(cudaGetLastError());
            read_stat(ctx, dstat);
            if (ctx->h_stat[1] & overflow_bits) { overflow = true; break; }
            if (fatal(ctx->h_stat[1])) break;
            const unsigned f2 = std::min(ctx->h_stat[0], vcap);
            kt.run(F_CENTERS, 1, [&] { launch_centers(M, f1, f2, ctx->nsm, st); });
            f0 = f1; f1 = f2;
            ++levels;
        }
        if (degen_abort) {
            // the vertices found so far start the generic walk (read at the last level check)
            read_stat(ctx, dstat);
            nseed = std::min(ctx->h_stat[0], vcap);
            break;
        }
        if (overflow) { S.capacity_retries++; continue; }
        V = f1;
        S.levels = levels;
        if (fast) kt.run(F_CENTERS, 1, [&] { launch_refine_centers(M, V, ctx->nsm, st); });
        break;
    }
    CK(cudaEventRecord(ev.e[2], st));
    if (degen_abort) {
        unsigned long long hc[C_NCOUNT];
        CK(cudaMemcpyAsync(hc, dcnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        S.rays = (int64_t)hc[C_RAYS];
        S.degenerate = (int64_t)hc[C_DEGEN];
        S.descents = (int64_t)hc[C_DESCENT];
        generic_build(ctx, mesh, M, M.vsig, nseed);
        srch.reset();
        S.ms_prepare = ms_between(ev.e[0], ev.e[1]);
        S.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return;
    }
    // ---- canonical order
    mesh->V = V;
    CK(cudaEventRecord(kt.next(), st));
    const int canon_ev = (int)kt.used - 1;
    bool packed = false;  // canonical order from one packed sort (else d + 1 sorts)
    {
        Scratch cs(st);
        unsigned* keys = cs.get<unsigned>((size_t)V * (d + 1));
        unsigned* kt = cs.get<unsigned>(V);
        unsigned* kt2 = cs.get<unsigned>(V);
        int* order = cs.get<int>(V);
        int* order2 = cs.get<int>(V);
        launch_canon_keys(M, V, keys, st);
        if (V) k_iota<<<std::min<unsigned>((V + 255) / 256, 65535u), 256, 0, st>>>(order, V);
        int end_bit = 1;
        while ((1ull << end_bit) < (unsigned long long)(n + mesh->np + 1)) ++end_bit;
        if (d * end_bit <= 64) {
            // one sort by the first d items packed in 64 bits; ties (the two end points
            // of an edge) ordered by the last item
            unsigned long long* k64 = cs.get<unsigned long long>(V);
            unsigned long long* k64s = cs.get<unsigned long long>(V);
            size_t tb = sort_pairs_u64_i32_temp((int)std::max(V, 1u));
            void* tmp = cs.get<char>(tb);
            launch_pack_keys(keys, V, d, end_bit, k64, st);
            if (V) sort_pairs_u64_i32(tmp, tb, k64, k64s, order, order2, (int)V, d * end_bit, st);
            std::swap(order, order2);
            launch_fix_runs(k64s, keys + (size_t)d * V, V, order, st);
            packed = true;
        } else {
            // least significant item first, stable sorts
            size_t tb = sort_pairs_u32_i32_temp((int)std::max(V, 1u));
            void* tmp = cs.get<char>(tb);
            for (int pos = d; pos >= 0; --pos) {
                launch_gather_keys(keys + (size_t)pos * V, order, V, kt, st);
                if (V) sort_pairs_u32_i32(tmp, tb, kt, kt2, order, order2, (int)V, end_bit, st);
                std::swap(order, order2);
            }
        }
        mesh->osig = dalloc<int>(st, (size_t)V * (d + 1));
        mesh->oc = dalloc<double>(st, (size_t)V * d);
        launch_canon_gather(M, V, keys, order, mesh->osig, mesh->oc, st);
        CK(cudaGetLastError());
    }
    CK(cudaEventRecord(kt.next(), st));
    kt.spans.emplace_back(F_CANON, canon_ev);
    kt.launches += packed ? 6 : 3 + 2 * (d + 1);
    CK(cudaEventRecord(ev.e[3], st));
    unsigned long long hc[C_NCOUNT];
    CK(cudaMemcpyAsync(hc, dcnt, sizeof(hc), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    srch.reset();
    S.vertices = V;
    S.rays = (int64_t)hc[C_RAYS];
    S.fallback_rays = (int64_t)hc[C_FALLBACK];
    S.uncertified = (int64_t)hc[C_UNCERT];
    S.insecure = (int64_t)hc[C_INSECURE];
    S.dd_rescores = (int64_t)hc[C_DD];
    S.degenerate = (int64_t)hc[C_DEGEN];
    S.descents = (int64_t)hc[C_DESCENT];
    S.descent_retries = (int64_t)hc[C_DRETRY];
    S.edges_closed = (int64_t)hc[C_EDGECLOSED];
    S.fallback_tree_rays = (int64_t)hc[C_FBTREE];
    S.fallback_nodes = (int64_t)hc[C_FBNODES];
    S.fallback_leaves = (int64_t)hc[C_FBLEAVES];
    S.fallback_points = (int64_t)hc[C_FBPOINTS];
    S.ambiguous_sets = (int64_t)hc[C_AMBSET];
    if (shard) {  // the vertices the shard owns sort first
        mesh->V = (unsigned)hc[C_OWNED];
        S.vertices = mesh->V;
    }
    double fam[F_N];
    kt.totals(fam);
    S.ms_knn = fam[F_KNN];
    S.ms_descent = fam[F_DESCENT];
    S.ms_expand = fam[F_EXPAND];
    S.ms_fallback = fam[F_FALLBACK];
    S.ms_centers = fam[F_CENTERS];
    S.ms_canonical = fam[F_CANON];
    S.launches = kt.launches;
    S.ms_prepare = ms_between(ev.e[0], ev.e[1]);
    S.ms_search = ms_between(ev.e[1], ev.e[2]);
    S.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    // A tie that double-double cannot break means generators in degenerate
    // position (more than d+1 on one empty sphere, e.g. lattice points): the
    // reference stores such a vertex with all of them, and so does the generic
    // walk of a box or plane-domain build.  This search broke the tie by index,
    // so a periodic image set, a shard or a refinement refuses the mesh.
    if (S.degenerate > 0 && mesh->allow_generic) {  // a tie the level checks did not see
        dfree(st, mesh->osig);
        dfree(st, mesh->oc);
        mesh->osig = nullptr;
        mesh->oc = nullptr;
        generic_build(ctx, mesh, M);
        S.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        return;
    }
    if (S.degenerate > 0)
        throw HvError(HV_E_DEGENERATE, "generators in degenerate position (" + std::to_string(S.degenerate) +
                                           " exact ties, e.g. more than d+1 points on one empty sphere); "
                                           "the GPU search needs general position -- perturb the points");
}

void ensure_neighbors(hv_mesh* m) {
    using namespace hv;
    if (m->nnbr >= 0) return;
    hv_ctx* ctx = m->ctx;
    cudaStream_t st = ctx->stream;
    const int d = m->d, n = m->n;
    const unsigned V = m->V;
    m->inc_off = dalloc<long long>(st, (size_t)n + 1);
    m->nbr_off = dalloc<long long>(st, (size_t)n + 1);
    if (n == 0) {
        CK(cudaMemsetAsync(m->inc_off, 0, sizeof(long long), st));
        CK(cudaMemsetAsync(m->nbr_off, 0, sizeof(long long), st));
        m->inc = dalloc<int>(st, 1);
        m->nbr = dalloc<int>(st, 1);
        m->nnbr = 0;
        return;
    }
    Scratch s(st);
    const unsigned long long np = (unsigned long long)V * (d + 1);
    unsigned long long* pairs = s.get<unsigned long long>(np);
    unsigned long long* pairs2 = s.get<unsigned long long>(np);
    long long* cnt = s.get<long long>((size_t)n + 1);
    CK(cudaMemsetAsync(cnt, 0, sizeof(long long) * (n + 1), st));
    launch_inc_pairs(d, n, V, m->osig, pairs, cnt, st);
    if (np) {
        size_t tb = sort_keys_u64_temp((long long)np);
        void* tmp = s.get<char>(tb);
        sort_keys_u64(tmp, tb, pairs, pairs2, (long long)np, st);
    }
    {
        size_t tb = scan_temp(n + 1);
        void* tmp = s.get<char>(tb);
        exclusive_scan_i64(tmp, tb, cnt, m->inc_off, n + 1, st);
    }
    long long ninc = 0;
    CK(cudaMemcpyAsync(&ninc, m->inc_off + n, sizeof(long long), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    m->inc = dalloc<int>(st, (size_t)std::max(ninc, 1ll));
    launch_inc_split((unsigned long long)ninc, pairs2, m->inc, st);
    long long* nn = s.get<long long>((size_t)n + 1);
    unsigned* dstat = s.get<unsigned>(1);
    CK(cudaMemsetAsync(nn, 0, sizeof(long long) * (n + 1), st));
    CK(cudaMemsetAsync(dstat, 0, sizeof(unsigned), st));
    launch_nbr_count(d, n, m->inc_off, m->inc, m->osig, nn, dstat, st);
    {
        size_t tb = scan_temp(n + 1);
        void* tmp = s.get<char>(tb);
        exclusive_scan_i64(tmp, tb, nn, m->nbr_off, n + 1, st);
    }
    long long tot = 0;
    unsigned hst = 0;
    CK(cudaMemcpyAsync(&tot, m->nbr_off + n, sizeof(long long), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&hst, dstat, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (hst) throw HvError(HV_E_CAPACITY, "a cell has more neighbours than the neighbour table holds");
    m->nbr = dalloc<int>(st, (size_t)std::max(tot, 1ll));
    launch_nbr_fill(d, n, m->inc_off, m->inc, m->osig, m->nbr_off, m->nbr, st);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(st));
    m->nnbr = tot;
}

int fail(hv_ctx* ctx, const HvError& e) {
    if (ctx) ctx->err = e.what();
    return e.code;
}

int validate_common(hv_ctx* ctx, int d, int64_t n, const double* lo, const double* hi, hv_mesh** out,
                    bool box = true) {
    if (!ctx || !out || (box && (!lo || !hi))) return HV_E_INVALID_ARG;
    if (d < 2 || d > HV_MAXD) { ctx->err = "dimension must be between 2 and 6"; return HV_E_INVALID_ARG; }
    if (n < 0 || n > (1ll << 30)) { ctx->err = "point count out of range"; return HV_E_INVALID_ARG; }
    for (int k = 0; box && k < d; ++k)
        if (!(lo[k] < hi[k]) || !std::isfinite(lo[k]) || !std::isfinite(hi[k])) {
            ctx->err = "box bounds must be finite with lo < hi";
            return HV_E_INVALID_ARG;
        }
    return HV_OK;
}

// The domain: a box [lo, hi] (cuboid planes), or np planes given by base
// points and normals (P x d each) with optional boundary conditions.
struct DomainSpec {
    const double* lo = nullptr;
    const double* hi = nullptr;
    int np = 0;
    const double* base = nullptr;
    const double* normal = nullptr;
    const int16_t* bc = nullptr;
    bool generic_ok = true;  // co-spherical generators: walk vertices of any size (not for periodic images)
};

int build_entry(hv_ctx* ctx, int d, int64_t n, const double* src, bool on_device, const DomainSpec& dom,
                const hv_params* params, hv_mesh** out) {
    if (!ctx || !out) return HV_E_INVALID_ARG;
    int rc = HV_OK;
    if (dom.lo || dom.hi) {
        rc = validate_common(ctx, d, n, dom.lo, dom.hi, out);
    } else {
        rc = validate_common(ctx, d, n, nullptr, nullptr, out, false);
        if (rc == HV_OK && (!dom.base || !dom.normal)) { ctx->err = "null plane array"; rc = HV_E_INVALID_ARG; }
        if (rc == HV_OK && dom.bc)
            for (int p = 0; p < dom.np; ++p)
                if (dom.bc[p] > 0) {
                    ctx->err = "periodic boundary planes are not supported";
                    rc = HV_E_INVALID_ARG;
                    break;
                }
    }
    if (rc != HV_OK) return rc;
    if (n > 0 && !src) { ctx->err = "null point array"; return HV_E_INVALID_ARG; }
    std::unique_ptr<hv_mesh> mp(new hv_mesh());
    hv_mesh* m = mp.get();
    m->ctx = ctx; m->d = d; m->n = (int)n;
    if (dom.lo) {
        for (int k = 0; k < d; ++k) { m->lo[k] = dom.lo[k]; m->hi[k] = dom.hi[k]; }
        m->np = 2 * d;
        hv::box_planes(d, dom.lo, dom.hi, m->planes);
    } else {
        std::string e = hv::make_planes(d, dom.np, dom.base, dom.normal, m->planes);
        if (e.empty()) e = hv::planes_bbox(d, dom.np, m->planes, m->lo, m->hi);
        if (!e.empty()) { ctx->err = e; return HV_E_INVALID_ARG; }
        m->np = dom.np;
    }
    mp.release();
    if (params) m->prm = *params; else hv_params_default(&m->prm);
    {
        int nb = 0;
        while ((1ll << (nb + 1)) <= std::max<int64_t>(n, 1)) ++nb;
        auto it = ctx->tuned.find({d, nb});
        if (it != ctx->tuned.end() && m->prm.method == HV_METHOD_FAST) {
            if (m->prm.knn == 0) m->prm.knn = it->second.knn;
            if (m->prm.leaf_size == 0) m->prm.leaf_size = it->second.leaf_size;
            if (m->prm.seed_stride == 0) m->prm.seed_stride = it->second.seed_stride;
            if (m->prm.rays_per_warp == 0) m->prm.rays_per_warp = it->second.rays_per_warp;
        }
    }
    if (m->prm.method != HV_METHOD_FAST && m->prm.method != HV_METHOD_PLAIN && m->prm.method != HV_METHOD_GENERIC) {
        delete m;
        ctx->err = "unknown method";
        return HV_E_INVALID_ARG;
    }
    m->allow_generic = dom.generic_ok;
    if (m->prm.method == HV_METHOD_GENERIC && !dom.generic_ok) {
        delete m;
        ctx->err = "the generic walk takes box and plane-domain meshes";
        return HV_E_INVALID_ARG;
    }
    try {
        CK(cudaSetDevice(ctx->device));
        build_impl(ctx, m, src, on_device, src);
    } catch (const HvError& e) {
        hv_mesh_free(m);
        return fail(ctx, e);
    } catch (const std::bad_alloc&) {
        hv_mesh_free(m);
        ctx->err = "host allocation failed";
        return HV_E_OOM;
    }
    *out = m;
    return HV_OK;
}

// One shard of the box mesh split over nranks ranks: the generators of range
// `rank` of the internal (Morton) order, the vertices whose smallest generator
// lies in that range.
int shard_entry(hv_ctx* ctx, int d, int64_t n, const double* src, bool on_device, const double* lo,
                const double* hi, int rank, int nranks, const hv_params* params, hv_mesh** out) {
    if (!ctx || !out) return HV_E_INVALID_ARG;
    if (nranks < 1 || rank < 0 || rank >= nranks) { ctx->err = "rank outside 0 .. nranks-1"; return HV_E_INVALID_ARG; }
    int rc = validate_common(ctx, d, n, lo, hi, out);
    if (rc != HV_OK) return rc;
    if (n > 0 && !src) { ctx->err = "null point array"; return HV_E_INVALID_ARG; }
    hv_params p;
    if (params) p = *params; else hv_params_default(&p);
    if (p.method != HV_METHOD_FAST) { ctx->err = "shards use the fast method"; return HV_E_INVALID_ARG; }
    std::unique_ptr<hv_mesh> mp(new hv_mesh());
    hv_mesh* m = mp.get();
    m->ctx = ctx; m->d = d; m->n = (int)n;
    for (int k = 0; k < d; ++k) { m->lo[k] = lo[k]; m->hi[k] = hi[k]; }
    m->np = 2 * d;
    hv::box_planes(d, lo, hi, m->planes);
    m->prm = p;
    m->own0 = (int)((n * rank) / nranks);
    m->own1 = (int)((n * (rank + 1)) / nranks);
    mp.release();
    try {
        CK(cudaSetDevice(ctx->device));
        build_impl(ctx, m, src, on_device, src);
    } catch (const HvError& e) {
        hv_mesh_free(m);
        return fail(ctx, e);
    } catch (const std::bad_alloc&) {
        hv_mesh_free(m);
        ctx->err = "host allocation failed";
        return HV_E_OOM;
    }
    *out = m;
    return HV_OK;
}

// Incremental refinement (refine!, src/meshrefine.jl:183, src/geometry.jl:404-438):
// the mesh of the old generators plus k new ones.  The search runs only over
// the new generators' cells (every vertex holding a new generator); an old
// vertex survives unless a new generator lies strictly inside its
// circumsphere; both sorted lists merge into the canonical order.  A new
// point within rounding of an old sphere makes the whole enlarged set be
// searched again instead.
int refine_entry(hv_mesh* old, int64_t k, const double* src, bool on_device, hv_mesh** out) {
    using namespace hv;
    if (!old || !out || k < 0 || (k > 0 && !src)) return HV_E_INVALID_ARG;
    hv_ctx* ctx = old->ctx;
    if (old->ext || old->pmask || old->own0 >= 0) {
        ctx->err = "refinement takes a box or plane-domain mesh, not a periodic one or a shard";
        return HV_E_INVALID_ARG;
    }
    if (old->prm.method != HV_METHOD_FAST) { ctx->err = "refinement uses the fast method"; return HV_E_INVALID_ARG; }
    if (old->g_max) { ctx->err = "refinement needs vertices of d+1 generators"; return HV_E_DEGENERATE; }
    const int d = old->d, n_old = old->n;
    if ((int64_t)n_old + k > (1ll << 30)) { ctx->err = "point count out of range"; return HV_E_INVALID_ARG; }
    const int n = n_old + (int)k;
    cudaStream_t st = ctx->stream;
    std::unique_ptr<hv_mesh> mp(new hv_mesh());
    hv_mesh* m = mp.get();
    m->ctx = ctx; m->d = d; m->n = n;
    for (int q = 0; q < d; ++q) { m->lo[q] = old->lo[q]; m->hi[q] = old->hi[q]; }
    m->np = old->np;
    std::memcpy(m->planes, old->planes, sizeof(DevPlane) * old->np);
    m->prm = old->prm;
    m->own_from = n_old;
    const auto t0 = std::chrono::steady_clock::now();
    try {
        CK(cudaSetDevice(ctx->device));
        double* all = dalloc<double>(st, (size_t)n * d);
        struct Free { cudaStream_t s; double* p; ~Free() { dfree(s, p); } } fr{st, all};
        if (n_old > 0) CK(cudaMemcpyAsync(all, old->d_in, sizeof(double) * n_old * d, cudaMemcpyDeviceToDevice, st));
        if (k > 0)
            CK(cudaMemcpyAsync(all + (size_t)n_old * d, src, sizeof(double) * k * d,
                               on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
        mp.release();
        build_impl(ctx, m, all, true, nullptr);  // the new generators' cells
        // old vertices: kept unless a new point invades their sphere
        const unsigned Vo = old->V, Vn = m->V;
        Scratch sc(st);
        long long* keep = sc.get<long long>((size_t)Vo + 1);
        long long* rank = sc.get<long long>((size_t)Vo + 1);
        unsigned* unsure = sc.get<unsigned>(1);
        CK(cudaMemsetAsync(keep, 0, sizeof(long long) * (Vo + 1), st));
        CK(cudaMemsetAsync(unsure, 0, sizeof(unsigned), st));
        launch_refine_keep(d, n_old, (int)k, Vo, old->osig, old->oc, old->d_in, m->d_in + (size_t)n_old * d, keep,
                           unsure, st);
        const size_t tb = scan_temp((int)Vo + 1);
        void* tmp = sc.get<char>(tb);
        exclusive_scan_i64(tmp, tb, keep, rank, (int)Vo + 1, st);
        long long kept = 0;
        unsigned hu = 0;
        CK(cudaMemcpyAsync(&kept, rank + Vo, sizeof(long long), cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(&hu, unsure, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (hu) {
            // a new point within rounding of an old sphere: search the whole set
            sc.release_all();
            hv_mesh* fm = new hv_mesh();
            fm->ctx = ctx; fm->d = d; fm->n = n;
            for (int q = 0; q < d; ++q) { fm->lo[q] = old->lo[q]; fm->hi[q] = old->hi[q]; }
            fm->np = old->np;
            std::memcpy(fm->planes, old->planes, sizeof(DevPlane) * old->np);
            fm->prm = old->prm;
            fm->st = m->st;
            hv_mesh_free(m);
            m = fm;
            build_impl(ctx, m, all, true, nullptr);
            m->st.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            *out = m;
            return HV_OK;
        }
        const unsigned V = (unsigned)kept + Vn;
        int* osig = dalloc<int>(st, (size_t)std::max(V, 1u) * (d + 1));
        double* oc = dalloc<double>(st, (size_t)std::max(V, 1u) * d);
        launch_refine_merge(d, n_old, (int)k, Vo, old->osig, old->oc, keep, rank, Vn, m->osig, m->oc, osig, oc, st);
        CK(cudaGetLastError());
        dfree(st, m->osig);
        dfree(st, m->oc);
        m->osig = osig;
        m->oc = oc;
        m->V = V;
        m->st.vertices = V;
        CK(cudaStreamSynchronize(st));
        m->st.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    } catch (const HvError& e) {
        hv_mesh_free(m);
        return fail(ctx, e);
    } catch (const std::bad_alloc&) {
        hv_mesh_free(m);
        ctx->err = "host allocation failed";
        return HV_E_OOM;
    }
    *out = m;
    return HV_OK;
}

// Periodic cuboid [lo, hi] with periodic axes pmask.  The margin starts at
// 1.5 mean spacings and grows by 1.5 until every vertex of an original cell is
// certified (at most 0.999 of a side).
int periodic_entry(hv_ctx* ctx, int d, int64_t n, const double* src, bool on_device, const double* lo,
                   const double* hi, int pmask, const hv_params* params, hv_mesh** out) {
    using namespace hv;
    int rc = validate_common(ctx, d, n, lo, hi, out);
    if (rc != HV_OK) return rc;
    if (n > 0 && !src) { ctx->err = "null point array"; return HV_E_INVALID_ARG; }
    if (n < 1) { ctx->err = "a periodic mesh needs at least one generator"; return HV_E_INVALID_ARG; }
    std::unique_ptr<hv_mesh> mp(new hv_mesh());
    hv_mesh* m = mp.get();
    m->ctx = ctx; m->d = d; m->n = (int)n; m->pmask = pmask;
    for (int k = 0; k < d; ++k) { m->lo[k] = lo[k]; m->hi[k] = hi[k]; }
    m->np = 2 * d;
    box_planes(d, lo, hi, m->planes);
    if (params) m->prm = *params; else hv_params_default(&m->prm);
    try {
        CK(cudaSetDevice(ctx->device));
        cudaStream_t st = ctx->stream;
        m->d_in = dalloc<double>(st, (size_t)n * d);
        CK(cudaMemcpyAsync(m->d_in, src, sizeof(double) * n * d,
                           on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
        m->d_planes = dalloc<DevPlane>(st, (size_t)m->np);
        CK(cudaMemcpyAsync(m->d_planes, m->planes, sizeof(DevPlane) * m->np, cudaMemcpyHostToDevice, st));
        PerBox B{};
        B.d = d; B.pmask = pmask;
        double vol = 1.0, scale = 0.0;
        for (int k = 0; k < d; ++k) {
            B.lo[k] = lo[k]; B.hi[k] = hi[k]; B.L[k] = hi[k] - lo[k];
            vol *= B.L[k];
        }
        const double spacing = std::pow(vol / (double)n, 1.0 / d);
        double grow = 1.5;
        Scratch ps(st);
        unsigned* dbad = ps.get<unsigned>(2);
        CK(cudaMemsetAsync(dbad, 0, 2 * sizeof(unsigned), st));
        launch_in_box(B, m->d_in, (int)n, dbad, st);
        unsigned hb[2] = {0, 0};
        CK(cudaMemcpyAsync(hb, dbad, sizeof(hb), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (hb[0]) throw HvError(HV_E_INVALID_ARG, "points must lie strictly inside the box and be finite");
        long long* cnt = ps.get<long long>((size_t)n + 1);
        long long* off = ps.get<long long>((size_t)n + 1);
        size_t stb = scan_temp((int)n + 1);
        void* stmp = ps.get<char>(stb);
        for (int attempt = 0;; ++attempt) {
            bool capped = true;
            scale = 0.0;
            for (int k = 0; k < d; ++k) {
                B.delta[k] = 0.0;
                if ((pmask >> k) & 1) {
                    B.delta[k] = std::min(grow * spacing, 0.999 * B.L[k]);
                    capped &= B.delta[k] >= 0.999 * B.L[k];
                }
                scale = std::max(scale, std::max(std::fabs(lo[k] - B.delta[k]), std::fabs(hi[k] + B.delta[k])));
            }
            B.scale = scale;
            CK(cudaMemsetAsync(cnt, 0, sizeof(long long) * (n + 1), st));
            launch_img_count(B, m->d_in, (int)n, cnt, st);
            exclusive_scan_i64(stmp, stb, cnt, off, (int)n + 1, st);
            long long nimg = 0;
            CK(cudaMemcpyAsync(&nimg, off + n, sizeof(long long), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            if (n + nimg > (1ll << 30)) throw HvError(HV_E_CAPACITY, "too many periodic images");
            const long long n_ext = n + nimg;
            dfree(st, m->img_ref); dfree(st, m->img_code);
            m->img_ref = dalloc<int>(st, (size_t)std::max(nimg, 1ll));
            m->img_code = dalloc<short>(st, (size_t)std::max(nimg, 1ll));
            Scratch es(st);
            double* ext_pts = es.get<double>((size_t)n_ext * d);
            CK(cudaMemcpyAsync(ext_pts, m->d_in, sizeof(double) * n * d, cudaMemcpyDeviceToDevice, st));
            launch_img_fill(B, m->d_in, (int)n, off, ext_pts, m->img_ref, m->img_code, st);
            CK(cudaGetLastError());
            double elo[HV_MAXD], ehi[HV_MAXD];
            for (int k = 0; k < d; ++k) { elo[k] = lo[k] - B.delta[k]; ehi[k] = hi[k] + B.delta[k]; }
            DomainSpec dom;
            dom.lo = elo; dom.hi = ehi;
            dom.generic_ok = true;  // co-spherical images: the public view takes lists of any length
            hv_mesh* ext = nullptr;
            int r = build_entry(ctx, d, n_ext, ext_pts, true, dom, &m->prm, &ext);
            if (r != HV_OK) throw HvError(r, ctx->err);
            ensure_neighbors(ext);
            CK(cudaMemsetAsync(dbad, 0, sizeof(unsigned), st));
            launch_per_validate(B, ext->g_max ? ext->g_off : nullptr, ext->g_max ? ext->g_sig : ext->osig, ext->oc,
                                ext->V, (int)n, (int)n_ext, ext->d_in, dbad, st);
            CK(cudaMemcpyAsync(hb, dbad, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            if (hb[0] == 0) {
                m->ext = ext;
                m->nimg = (int)nimg;
                for (int k = 0; k < d; ++k) m->delta[k] = B.delta[k];
                break;
            }
            hv_mesh_free(ext);
            if (capped || attempt >= 12)
                throw HvError(HV_E_CAPACITY, "too few generators for the periodic image margin");
            grow *= 1.5;
        }
        // the public view
        hv_mesh* e = m->ext;
        const int n_ext = e->n;
        const unsigned Ve = e->V;
        {
            Scratch vs(st);
            long long* flag = vs.get<long long>((size_t)Ve + 1);
            long long* pos = vs.get<long long>((size_t)Ve + 1);
            int* ext2pub = vs.get<int>((size_t)std::max(Ve, 1u));
            const bool gen = e->g_max > 0;  // vertices with more than d+1 generators: CSR rows
            const long long* eoff = gen ? e->g_off : nullptr;
            const int* esig = gen ? e->g_sig : e->osig;
            long long* len = gen ? vs.get<long long>((size_t)Ve + 1) : nullptr;
            long long* rowpos = gen ? vs.get<long long>((size_t)Ve + 1) : nullptr;
            launch_pub_flag(d, eoff, esig, Ve, (int)n, flag, len, st);
            size_t tb = scan_temp((int)Ve + 1);
            void* tmp = vs.get<char>(tb);
            exclusive_scan_i64(tmp, tb, flag, pos, (int)Ve + 1, st);
            if (gen) exclusive_scan_i64(tmp, tb, len, rowpos, (int)Ve + 1, st);
            long long Vp = 0, Sp = 0;
            CK(cudaMemcpyAsync(&Vp, pos + Ve, sizeof(long long), cudaMemcpyDeviceToHost, st));
            if (gen) CK(cudaMemcpyAsync(&Sp, rowpos + Ve, sizeof(long long), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            m->V = (unsigned)Vp;
            if (gen) {
                m->g_max = e->g_max;
                m->g_off = dalloc<long long>(st, (size_t)Vp + 1);
                m->g_sig = dalloc<int>(st, (size_t)std::max(Sp, 1ll));
                CK(cudaMemcpyAsync(m->g_off + Vp, &Sp, sizeof(long long), cudaMemcpyHostToDevice, st));
            } else {
                m->osig = dalloc<int>(st, (size_t)std::max(Vp, 1ll) * (d + 1));
            }
            m->oc = dalloc<double>(st, (size_t)std::max(Vp, 1ll) * d);
            launch_pub_fill(d, eoff, esig, e->oc, Ve, (int)n, n_ext, m->img_ref, m->img_code, pos, rowpos,
                            gen ? m->g_off : nullptr, gen ? m->g_sig : m->osig, m->oc, ext2pub, st);
            long long tot = 0, ninc = 0;
            CK(cudaMemcpyAsync(&tot, e->nbr_off + n, sizeof(long long), cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(&ninc, e->inc_off + n, sizeof(long long), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            m->nbr_off = dalloc<long long>(st, (size_t)n + 1);
            m->inc_off = dalloc<long long>(st, (size_t)n + 1);
            CK(cudaMemcpyAsync(m->nbr_off, e->nbr_off, sizeof(long long) * (n + 1), cudaMemcpyDeviceToDevice, st));
            CK(cudaMemcpyAsync(m->inc_off, e->inc_off, sizeof(long long) * (n + 1), cudaMemcpyDeviceToDevice, st));
            m->nbr = dalloc<int>(st, (size_t)std::max(tot, 1ll));
            m->pshift = dalloc<signed char>(st, (size_t)std::max(tot, 1ll) * d);
            m->pperm = dalloc<int>(st, (size_t)std::max(tot, 1ll));
            launch_pub_nbr(d, (int)n, n_ext, e->nbr_off, e->nbr, m->img_ref, m->img_code, m->nbr, m->pshift,
                           m->pperm, st);
            m->inc = dalloc<int>(st, (size_t)std::max(ninc, 1ll));
            launch_pub_inc(ninc, e->inc, ext2pub, m->inc, st);
            CK(cudaGetLastError());
            CK(cudaStreamSynchronize(st));
            m->nnbr = tot;
        }
        m->st = e->st;
        m->st.vertices = m->V;
    } catch (const HvError& e) {
        hv_mesh_free(mp.release());
        return fail(ctx, e);
    } catch (const std::bad_alloc&) {
        hv_mesh_free(mp.release());
        ctx->err = "host allocation failed";
        return HV_E_OOM;
    }
    *out = mp.release();
    return HV_OK;
}

}  // namespace

extern "C" {

int hv_version(void) { return HV_VERSION; }

void hv_params_default(hv_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->method = HV_METHOD_FAST;
    p->seed = 0x5EEDull;
}

int hv_ctx_create(int device, hv_ctx** out) {
    if (!out) return HV_E_INVALID_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return HV_E_CUDA;
    hv_ctx* c = new hv_ctx();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess) { delete c; return HV_E_CUDA; }
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { delete c; return HV_E_CUDA; }
    if (cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->stream3, cudaStreamNonBlocking) != cudaSuccess) {
        cudaStreamDestroy(c->stream);
        if (c->stream2) cudaStreamDestroy(c->stream2);
        delete c;
        return HV_E_CUDA;
    }
    for (auto& e : c->ovl_ev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device);
    if (cudaMallocHost((void**)&c->h_stat, 4 * sizeof(unsigned)) != cudaSuccess) {
        cudaStreamDestroy(c->stream);
        cudaStreamDestroy(c->stream2);
        cudaStreamDestroy(c->stream3);
        delete c;
        return HV_E_CUDA;
    }
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    *out = c;
    return HV_OK;
}

int hv_ctx_destroy(hv_ctx* ctx) {
    if (!ctx) return HV_E_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cudaFreeHost(ctx->h_stat);
    for (cudaEvent_t e : ctx->evpool) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->ovl_ev)
        if (e) cudaEventDestroy(e);
    cudaStreamSynchronize(ctx->stream2);
    cudaStreamSynchronize(ctx->stream3);
    cudaStreamDestroy(ctx->stream2);
    cudaStreamDestroy(ctx->stream3);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return HV_OK;
}

const char* hv_last_error(hv_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void* hv_ctx_stream(hv_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int hv_mesh_build(hv_ctx* ctx, int d, int64_t n, const double* pts, const double* lo, const double* hi,
                  const hv_params* params, hv_mesh** out) {
    DomainSpec dom;
    dom.lo = lo; dom.hi = hi;
    if (!lo || !hi) return HV_E_INVALID_ARG;
    return build_entry(ctx, d, n, pts, false, dom, params, out);
}

int hv_mesh_build_device(hv_ctx* ctx, int d, int64_t n, const double* d_pts, const double* lo, const double* hi,
                         const hv_params* params, hv_mesh** out) {
    DomainSpec dom;
    dom.lo = lo; dom.hi = hi;
    if (!lo || !hi) return HV_E_INVALID_ARG;
    return build_entry(ctx, d, n, d_pts, true, dom, params, out);
}

int hv_mesh_build_planes(hv_ctx* ctx, int d, int64_t n, const double* pts, int nplanes, const double* base,
                         const double* normal, const int16_t* bc, const hv_params* params, hv_mesh** out) {
    DomainSpec dom;
    dom.np = nplanes; dom.base = base; dom.normal = normal; dom.bc = bc;
    return build_entry(ctx, d, n, pts, false, dom, params, out);
}

int hv_mesh_build_planes_device(hv_ctx* ctx, int d, int64_t n, const double* d_pts, int nplanes,
                                const double* base, const double* normal, const int16_t* bc,
                                const hv_params* params, hv_mesh** out) {
    DomainSpec dom;
    dom.np = nplanes; dom.base = base; dom.normal = normal; dom.bc = bc;
    return build_entry(ctx, d, n, d_pts, true, dom, params, out);
}

int hv_autotune(hv_ctx* ctx, int d, int64_t n, const double* pts, const double* lo, const double* hi,
                hv_params* out) {
    int rc = validate_common(ctx, d, n, lo, hi, (hv_mesh**)&out);
    if (rc != HV_OK || !out) return rc != HV_OK ? rc : HV_E_INVALID_ARG;
    if (n < 2) { hv_params_default(out); return HV_OK; }
    std::vector<double> synth;
    if (!pts) {  // uniform points in the box (SplitMix64, seed 0x7a11)
        synth.resize((size_t)n * d);
        uint64_t st = 0x7a11;
        for (size_t q = 0; q < synth.size(); ++q) {
            uint64_t z = (st += 0x9E3779B97F4A7C15ull);
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            z ^= z >> 31;
            const double u01 = ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
            const int k = (int)(q % d);
            synth[q] = lo[k] + (hi[k] - lo[k]) * u01;
        }
        pts = synth.data();
    }
    const int K0 = default_knn(d);
    std::vector<int> ks = {std::max(16, K0 / 2), K0, std::min(480, K0 * 3 / 2)};
    std::vector<int> leaves = {8, 16};
    std::vector<int> strides = {1, 4, 8, 16};
    hv_params best;
    hv_params_default(&best);
    double best_ms = 1e300;
    for (int K : ks)
        for (int L : leaves)
            for (int S : strides) {
                hv_params p;
                hv_params_default(&p);
                p.knn = K; p.leaf_size = L; p.seed_stride = S; p.rays_per_warp = 1;
                double ms = 1e300;
                for (int rep = 0; rep < 2; ++rep) {  // the first build warms caches and the pool
                    hv_mesh* m = nullptr;
                    int r = hv_mesh_build(ctx, d, n, pts, lo, hi, &p, &m);
                    if (r != HV_OK) { ms = 1e300; break; }
                    hv_stats stt;
                    hv_mesh_stats(m, &stt);
                    ms = std::min(ms, stt.ms_total);
                    hv_mesh_free(m);
                }
                if (ms < best_ms) { best_ms = ms; best = p; }
            }
    if (best_ms >= 1e300) return HV_E_INTERNAL;
    int nb = 0;
    while ((1ll << (nb + 1)) <= n) ++nb;
    ctx->tuned[{d, nb}] = best;
    *out = best;
    return HV_OK;
}

int hv_mesh_counts(hv_mesh* m, int64_t* nverts, int64_t* nnbr_total) {
    if (!m) return HV_E_INVALID_ARG;
    try {
        CK(cudaSetDevice(m->ctx->device));
        if (nnbr_total) { ensure_neighbors(m); *nnbr_total = m->nnbr; }
        if (nverts) *nverts = m->V;
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

int hv_mesh_vertices(hv_mesh* m, int64_t* sig, double* r) {
    if (!m || (m->V && (!sig || !r))) return HV_E_INVALID_ARG;
    if (m->g_max > m->d + 1) {
        m->ctx->err = "the mesh has vertices with more than d+1 generators: read them with hv_mesh_vertices_csr";
        return HV_E_DEGENERATE;
    }
    try {
        CK(cudaSetDevice(m->ctx->device));
        cudaStream_t st = m->ctx->stream;
        if (m->V) {
            Scratch s(st);
            const size_t ns = (size_t)m->V * (m->d + 1);
            int64_t* dsig = s.get<int64_t>(ns);
            if (m->g_max) hv::launch_out_nbr((long long)ns, m->g_sig, dsig, st);  // every list has d+1 items
            else hv::launch_out_vertices(m->d, m->V, m->osig, dsig, st);
            CK(cudaMemcpyAsync(sig, dsig, ns * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(r, m->oc, (size_t)m->V * m->d * sizeof(double), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
        }
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

int hv_mesh_signature_total(hv_mesh* m, int64_t* total, int* max_len) {
    if (!m || !total) return HV_E_INVALID_ARG;
    try {
        CK(cudaSetDevice(m->ctx->device));
        long long t = (long long)m->V * (m->d + 1);
        if (m->g_max && m->V) {
            CK(cudaMemcpyAsync(&t, m->g_off + m->V, sizeof(long long), cudaMemcpyDeviceToHost, m->ctx->stream));
            CK(cudaStreamSynchronize(m->ctx->stream));
        }
        *total = t;
        if (max_len) *max_len = m->g_max ? m->g_max : (m->V ? m->d + 1 : 0);
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

int hv_mesh_vertices_csr(hv_mesh* m, int64_t* offs, int64_t* sig, double* r) {
    if (!m || !offs || (m->V && (!sig || !r))) return HV_E_INVALID_ARG;
    try {
        CK(cudaSetDevice(m->ctx->device));
        cudaStream_t st = m->ctx->stream;
        const unsigned V = m->V;
        if (m->g_max) {
            CK(cudaMemcpyAsync(offs, m->g_off, sizeof(int64_t) * (V + 1), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
        } else {
            for (unsigned v = 0; v <= V; ++v) offs[v] = (int64_t)v * (m->d + 1);
        }
        const long long total = offs[V];
        if (V) {
            Scratch s(st);
            int64_t* dsig = s.get<int64_t>((size_t)total);
            if (m->g_max) hv::launch_out_nbr(total, m->g_sig, dsig, st);
            else hv::launch_out_vertices(m->d, V, m->osig, dsig, st);
            CK(cudaMemcpyAsync(sig, dsig, sizeof(int64_t) * total, cudaMemcpyDeviceToHost, st));
            CK(cudaMemcpyAsync(r, m->oc, sizeof(double) * V * m->d, cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
        }
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

int hv_mesh_verify(hv_mesh* m, int64_t* inside, int64_t* ties, double* max_dev) {
    if (!m || !inside) return HV_E_INVALID_ARG;
    if (!m->t_pts && m->n > 0) {
        m->ctx->err = "verification needs the search tree (a box, plane-domain or refined mesh)";
        return HV_E_INVALID_ARG;
    }
    try {
        CK(cudaSetDevice(m->ctx->device));
        cudaStream_t st = m->ctx->stream;
        unsigned long long h[3] = {0, 0, 0};
        if (m->V) {
            Scratch s(st);
            unsigned long long* dc = s.get<unsigned long long>(3);
            CK(cudaMemsetAsync(dc, 0, 3 * sizeof(unsigned long long), st));
            hv::DevMesh M;
            std::memset(&M, 0, sizeof(M));
            M.d = m->d; M.n = m->n; M.np = m->np; M.planes = m->d_planes;
            M.pts = m->t_pts; M.perm = m->t_perm; M.blo = m->t_blo; M.bhi = m->t_bhi;
            M.leaf = m->t_leaf; M.nleaves = m->t_nleaves; M.P = m->t_P; M.dp = m->d <= 4 ? 4 : 8;
            hv::launch_verify(M, m->d_in, m->V, m->g_max ? m->g_off : nullptr, m->g_max ? m->g_sig : m->osig, m->oc,
                              dc, dc + 2, st);
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(h, dc, sizeof(h), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
        }
        *inside = (int64_t)h[0];
        if (ties) *ties = (int64_t)h[1];
        if (max_dev) { double dv; std::memcpy(&dv, &h[2], sizeof(dv)); *max_dev = dv; }
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

int hv_mesh_neighbors(hv_mesh* m, int64_t* offs, int64_t* nbr) {
    if (!m || !offs) return HV_E_INVALID_ARG;
    try {
        CK(cudaSetDevice(m->ctx->device));
        ensure_neighbors(m);
        if (m->nnbr > 0 && !nbr) return HV_E_INVALID_ARG;
        cudaStream_t st = m->ctx->stream;
        CK(cudaMemcpyAsync(offs, m->nbr_off, sizeof(int64_t) * (m->n + 1), cudaMemcpyDeviceToHost, st));
        if (m->nnbr > 0) {
            Scratch s(st);
            int64_t* dn = s.get<int64_t>((size_t)m->nnbr);
            hv::launch_out_nbr(m->nnbr, m->nbr, dn, st);
            CK(cudaMemcpyAsync(nbr, dn, sizeof(int64_t) * m->nnbr, cudaMemcpyDeviceToHost, st));
        }
        CK(cudaStreamSynchronize(st));
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

}  // extern "C"

namespace {

// VI_POLYGON; vol/area are host arrays, or (dev_out) device arrays that receive
// the results in place, stream-ordered on the context's stream.
int polygon_impl(hv_mesh* m, double* vol, double* area, bool dev_out);
int mc_impl(hv_mesh* m, int ndir, uint64_t seed, double* vol, double* area, bool dev_out);

// A periodic mesh integrates its extended mesh and gathers the original cells:
// volumes are the first n, areas follow the public neighbour order.
template <class F>
int periodic_integrate(hv_mesh* m, double* vol, double* area, bool dev_out, F&& run_ext) {
    try {
        CK(cudaSetDevice(m->ctx->device));
        cudaStream_t st = m->ctx->stream;
        hv_mesh* e = m->ext;
        long long ne = 0;
        CK(cudaMemcpyAsync(&ne, e->nbr_off + e->n, sizeof(long long), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        Scratch s(st);
        double* evol = s.get<double>((size_t)e->n);
        double* earea = s.get<double>((size_t)std::max(ne, 1ll));
        int r = run_ext(e, evol, earea);
        if (r != HV_OK) { m->ctx->err = e->ctx->err; return r; }
        double* pvol = dev_out ? vol : s.get<double>((size_t)m->n);
        double* parea = dev_out ? area : s.get<double>((size_t)std::max(m->nnbr, 1ll));
        CK(cudaMemcpyAsync(pvol, evol, sizeof(double) * m->n, cudaMemcpyDeviceToDevice, st));
        if (m->nnbr > 0) hv::launch_pub_area(m->n, m->nbr_off, m->pperm, earea, parea, st);
        if (!dev_out) {
            CK(cudaMemcpyAsync(vol, pvol, sizeof(double) * m->n, cudaMemcpyDeviceToHost, st));
            if (m->nnbr > 0) CK(cudaMemcpyAsync(area, parea, sizeof(double) * m->nnbr, cudaMemcpyDeviceToHost, st));
        }
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(st));
        m->st.poly_big_facets = e->st.poly_big_facets;
        m->st.ms_poly_incidence = e->st.ms_poly_incidence;
        m->st.ms_poly_facets = e->st.ms_poly_facets;
        m->st.ms_poly_big = e->st.ms_poly_big;
        m->st.ms_poly_total = e->st.ms_poly_total;
        m->st.poly_faces = e->st.poly_faces;
        m->st.poly_terms = e->st.poly_terms;
        m->st.poly_term_flops = e->st.poly_term_flops;
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

// VI_POLYGON of a mesh with vertices of more than d+1 generators: the area of
// every facet by the pulling decomposition over its faces (hv_degen.cu).
int generic_polygon(hv_mesh* m, double* vol, double* area, bool dev_out) {
    if (m->nnbr > 0 && !area) return HV_E_INVALID_ARG;
    try {
        CK(cudaSetDevice(m->ctx->device));
        cudaStream_t st = m->ctx->stream;
        Scratch s(st);
        double* dvol = dev_out ? vol : s.get<double>((size_t)std::max(m->n, 1));
        double* darea = dev_out ? area : s.get<double>((size_t)std::max(m->nnbr, 1ll));
        unsigned* dst = s.get<unsigned>(1);
        CK(cudaMemsetAsync(dst, 0, sizeof(unsigned), st));
        hv::GenPoly P{};
        P.d = m->d; P.n = m->n; P.planes = m->d_planes; P.pts = m->d_in;
        P.off = m->g_off; P.sig = m->g_sig; P.oc = m->oc;
        P.nbr_off = m->nbr_off; P.nbr = m->nbr; P.fcell = m->g_fcell; P.fbeg = m->g_fbeg; P.fend = m->g_fend;
        P.fvert = m->g_fvert; P.nslots = m->nnbr; P.status = dst;
        hv::launch_gen_polygon(P, darea, dvol, m->ctx->nsm, st);
        CK(cudaGetLastError());
        unsigned hs = 0;
        CK(cudaMemcpyAsync(&hs, dst, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        if (!dev_out) {
            if (m->n) CK(cudaMemcpyAsync(vol, dvol, sizeof(double) * m->n, cudaMemcpyDeviceToHost, st));
            if (m->nnbr > 0) CK(cudaMemcpyAsync(area, darea, sizeof(double) * m->nnbr, cudaMemcpyDeviceToHost, st));
        }
        CK(cudaStreamSynchronize(st));
        if (hs) throw HvError(HV_E_CAPACITY, "a facet has more than 64 vertices or faces (degenerate polygon)");
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

// HV_POLY_FLAGS=1: VI_POLYGON areas from every vertex's signed flag terms
// (hv_polyflag.cu) instead of the face-lattice kernels (slower on this GPU:
// the subset solves are latency-bound; kept as an independent second method).
bool use_poly_flags(int d) {
    const char* e = std::getenv("HV_POLY_FLAGS");
    return d >= 3 && e && e[0] == '1';
}

// VI_POLYGON over the face lattice of the whole mesh (hv_polylat.cu) for
// d >= 3 (HV_POLY_LATTICE=0 selects the per-facet kernels of hv_poly.cu); its
// tables are indexed by 32-bit entries, so larger meshes take the per-facet
// kernels.
bool use_poly_lattice(int d, unsigned V, long long nslots) {
    int from = 3;
    if (const char* e = std::getenv("HV_POLY_LATTICE")) from = e[0] == '0' ? 99 : from;
    if (d < std::max(from, 3) || d > 6) return false;
    long long emax = 0;
    for (int c = 1; c < d; ++c) emax = std::max(emax, (long long)hv::lat_subsets(d, c));
    return (long long)V * emax < (1ll << 31) - 2 && nslots < (1ll << 31) - 2;
}

// The faces of levels 1 .. d-1 of a mesh of simple vertices (hv_polylat.cu):
// counts, reference vertices and masks per level, the edges' second vertices,
// and (when kept) the per-vertex face tables F[c][rank * V + v].
struct Lattice {
    std::vector<long long> nf;
    std::vector<unsigned*> fref;
    std::vector<unsigned char*> fmask;
    unsigned* fref2 = nullptr;
    std::vector<int*> F;
};

// on_level(c, F of level c-1, F of level c, entries, sorted entry ids, run starts)
// runs after level c is numbered, while its sorted entries still exist.
using LevelFn = std::function<void(int, const int*, const int*, long long, const int*, const long long*)>;

hv::LatIn lat_input(hv_mesh* m, unsigned* dstat) {
    hv::LatIn L{};
    L.d = m->d; L.n = m->n; L.V = m->V; L.planes = m->d_planes; L.pts = m->d_in; L.osig = m->osig; L.oc = m->oc;
    L.nbr_off = m->nbr_off; L.nbr = m->nbr; L.status = dstat;
    return L;
}

void lattice_levels(hv_mesh* m, const hv::LatIn& L, int* slot_cell, Scratch& s, KTimer& kt, bool keep, bool starts,
                    Lattice& T, const LevelFn& on_level) {
    cudaStream_t st = m->ctx->stream;
    const int d = m->d, n = m->n;
    const unsigned V = m->V;
    const long long ns = m->nnbr;
    auto sync_read = [&](const void* dev, void* host, size_t b) {
        CK(cudaMemcpyAsync(host, dev, b, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    };
    int gbits = 1;
    while ((1ll << gbits) <= (long long)n + m->np + 1) ++gbits;
    T.nf.assign(d + 1, 0);
    T.fref.assign(d + 1, nullptr);
    T.fmask.assign(d + 1, nullptr);
    T.F.assign(d + 1, nullptr);
    // level 1: facet slots
    std::unique_ptr<Scratch> fprev(new Scratch(st));
    int* Fp = (keep ? s : *fprev).get<int>((size_t)V * hv::lat_subsets(d, 1));
    T.F[1] = keep ? Fp : nullptr;
    T.fref[1] = s.get<unsigned>((size_t)std::max(ns, 1ll));
    T.nf[1] = ns;
    CK(cudaMemsetAsync(T.fref[1], 0xFF, sizeof(unsigned) * std::max(ns, 1ll), st));
    kt.run(0, 2, [&] { hv::launch_lat_facets(L, Fp, T.fref[1], slot_cell, st); });
    CK(cudaGetLastError());
    long long emax = 1;
    for (int c = 2; c < d; ++c) emax = std::max(emax, (long long)V * hv::lat_subsets(d, c));
    Scratch ws(st);  // the sort's buffers
    auto* keys = ws.get<unsigned long long>((size_t)emax + 1);
    auto* keys2 = ws.get<unsigned long long>((size_t)emax + 1);
    int* vals = ws.get<int>((size_t)emax);
    int* vals2 = ws.get<int>((size_t)emax);
    const size_t sort_tb = hv::sort_pairs_u64_i32_temp((int)emax);
    void* sort_tmp = ws.get<char>(sort_tb);
    const size_t scan_tb = hv::scan_temp((int)emax + 1);
    void* scan_tmp = ws.get<char>(scan_tb);
    auto* nvalid = ws.get<unsigned long long>(1);
    for (int c = 2; c < d; ++c) {
        const long long E = (long long)V * hv::lat_subsets(d, c);
        std::unique_ptr<Scratch> fcur(new Scratch(st));
        int* Fc = nullptr;  // no level reads the edges' table unless it is kept
        if (keep) Fc = s.get<int>((size_t)std::max(E, 1ll));
        else if (c < d - 1) Fc = fcur->get<int>((size_t)std::max(E, 1ll));
        T.F[c] = keep ? Fc : nullptr;
        int fbits = 1;
        while ((1ll << fbits) < T.nf[c - 1]) ++fbits;
        CK(cudaMemsetAsync(nvalid, 0, sizeof(unsigned long long), st));
        kt.run(0, 2, [&] {
            hv::launch_lat_entries(L, c, gbits, Fp, keys, vals, Fc, nvalid, st);
            hv::sort_pairs_u64_i32(sort_tmp, sort_tb, keys, keys2, vals, vals2, (int)E, std::min(64, gbits + fbits), st);
        });
        CK(cudaGetLastError());
        unsigned long long nval = 0;
        sync_read(nvalid, &nval, sizeof(nval));
        long long* heads = (long long*)keys;  // the unsorted keys are spent
        long long* fidx = (long long*)keys2;  // and the sorted ones once the heads are marked
        kt.run(0, 2, [&] {
            hv::launch_lat_heads((long long)nval, keys2, heads, st);
            hv::exclusive_scan_i64(scan_tmp, scan_tb, heads, fidx, (int)nval + 1, st);
        });
        sync_read(fidx + nval, &T.nf[c], sizeof(long long));
        T.fref[c] = s.get<unsigned>((size_t)std::max(T.nf[c], 1ll));
        T.fmask[c] = s.get<unsigned char>((size_t)std::max(T.nf[c], 1ll));
        if (c == d - 1) T.fref2 = s.get<unsigned>((size_t)std::max(T.nf[c], 1ll));
        long long* hstart = starts ? heads : nullptr;  // the head flags are spent once scanned
        kt.run(0, 1, [&] {
            hv::launch_lat_scatter(L, c, (long long)nval, fidx, vals2, Fc, T.fref[c], T.fmask[c],
                                   c == d - 1 ? T.fref2 : nullptr, hstart, st);
        });
        CK(cudaGetLastError());
        on_level(c, Fp, Fc, (long long)nval, vals2, hstart);
        if (!keep) fprev = std::move(fcur);
        Fp = Fc;
    }
}

// The interface areas of a mesh of simple vertices through the mesh-wide face
// lattice into area (nslots, zeroed); build time in kt family 0, terms in 1.
void poly_lattice(hv_mesh* m, double* area, int* slot_cell, unsigned* dstat, Scratch& s, KTimer& kt) {
    cudaStream_t st = m->ctx->stream;
    const int d = m->d;
    const long long ns = m->nnbr;
    const hv::LatIn L = lat_input(m, dstat);
    auto sync_read = [&](const void* dev, void* host, size_t b) {
        CK(cudaMemcpyAsync(host, dev, b, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    };
    Lattice T;
    std::vector<long long*> off(d + 1, nullptr);
    std::vector<int*> child(d + 1, nullptr), lgen(d + 1, nullptr), par(d + 1, nullptr);
    std::vector<long long> npairs(d + 1, 0);
    long long emax = 1;
    for (int c = 2; c < d; ++c) emax = std::max(emax, (long long)m->V * hv::lat_subsets(d, c));
    auto* cnt = s.get<unsigned long long>((size_t)std::max(emax, ns) + 1);
    const size_t scan_tb = hv::scan_temp((int)std::max(emax, ns) + 1);
    void* scan_tmp = s.get<char>(scan_tb);
    // the child lists of the parents at level c - 1 (children at level c)
    lattice_levels(m, L, slot_cell, s, kt, false, false, T,
                   [&](int cc, const int* Fprev, const int*, long long, const int*, const long long*) {
        const int c = cc - 1;
        const long long nG = T.nf[c];
        CK(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (nG + 1), st));
        off[c] = s.get<long long>((size_t)nG + 1);
        kt.run(0, 2, [&] {
            hv::launch_lat_pairs(L, c, T.nf[c + 1], T.fref[c + 1], T.fmask[c + 1], Fprev, T.fref[c], cnt, nullptr,
                                 nullptr, nullptr, nullptr, false, st);
            hv::exclusive_scan_i64(scan_tmp, scan_tb, (const long long*)cnt, off[c], (int)nG + 1, st);
        });
        long long np = 0;
        sync_read(off[c] + nG, &np, sizeof(long long));
        npairs[c] = np;
        child[c] = s.get<int>((size_t)std::max(np, 1ll));
        lgen[c] = s.get<int>((size_t)std::max(np, 1ll));
        par[c] = s.get<int>((size_t)std::max(np, 1ll));
        CK(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (nG + 1), st));
        kt.run(0, 1, [&] {
            hv::launch_lat_pairs(L, c, T.nf[c + 1], T.fref[c + 1], T.fmask[c + 1], Fprev, T.fref[c], cnt, off[c],
                                 child[c], lgen[c], par[c], true, st);
        });
        CK(cudaGetLastError());
    });
    // volumes, bottom-up
    std::vector<double*> vol(d + 1, nullptr);
    for (int c = d - 2; c >= 1; --c) {
        vol[c] = c == 1 ? area : s.get<double>((size_t)std::max(T.nf[c], 1ll));
        Scratch lv(st);  // this level's frames and terms
        double* frame = c < d - 2 ? lv.get<double>((size_t)std::max(T.nf[c], 1ll) * (c + 1) * d) : nullptr;
        double* term = lv.get<double>((size_t)std::max(npairs[c], 1ll));
        kt.run(0, 1, [&] {
            hv::launch_lat_prep(L, c, T.nf[c], off[c], child[c], lgen[c], T.fref[c], T.fmask[c], slot_cell, frame,
                                st);
        });
        kt.run(1, 1, [&] {
            hv::launch_lat_terms(L, c, npairs[c], par[c], child[c], lgen[c], T.fref[c], frame, T.fref[c + 1],
                                 c + 1 == d - 1 ? T.fref2 : nullptr, vol[c + 1], term, st);
        });
        kt.run(0, 1, [&] { hv::launch_lat_sum(L, c, T.nf[c], off[c], term, T.fref[c], slot_cell, vol[c], st); });
        CK(cudaGetLastError());
    }
    m->st.poly_faces = 0;
    m->st.poly_terms = 0;
    m->st.poly_term_flops = 0;
    for (int c = 1; c <= d - 2; ++c) {
        m->st.poly_terms += npairs[c];
        m->st.poly_term_flops += npairs[c] * hv::lat_term_flops(d, c);
    }
    for (int c = 2; c < d; ++c) m->st.poly_faces += T.nf[c];
}

// The integrand quadrature's flag weights through the face lattice: qw for the
// facets' sorted vertex lists (qv, foff), the flag sums into qa; the facet
// centres qc must exist.
void quad_lattice(hv_mesh* m, const hv::QuadRun& Q, unsigned* dstat) {
    hv_ctx* ctx = m->ctx;
    cudaStream_t st = ctx->stream;
    const int d = m->d;
    KTimer kt(ctx);
    Scratch s(st);
    const hv::LatIn L = lat_input(m, dstat);
    int* slot_cell = s.get<int>((size_t)std::max(m->nnbr, 1ll));
    Lattice T;
    std::vector<double*> cen(d + 1, nullptr);
    cen[1] = Q.qc;  // the facet centres, by slot
    lattice_levels(m, L, slot_cell, s, kt, true, true, T,
                   [&](int c, const int*, const int*, long long nval, const int* sv, const long long* hstart) {
        if (c > d - 2) return;
        cen[c] = s.get<double>((size_t)std::max(T.nf[c], 1ll) * d);
        hv::launch_lat_centroid(L, T.nf[c], nval, hstart, sv, cen[c], st);
        CK(cudaGetLastError());
    });
    // frames of the levels 1 .. d-3 (the parents of the phi levels)
    std::vector<double*> frame(d + 1, nullptr);
    for (int c = 1; c <= d - 3; ++c) {
        frame[c] = s.get<double>((size_t)std::max(T.nf[c], 1ll) * (c + 1) * d);
        hv::launch_lat_prep(L, c, T.nf[c], nullptr, nullptr, nullptr, T.fref[c], T.fmask[c], slot_cell, frame[c], st);
    }
    // phi, top-down over the levels 2 .. d-2
    std::vector<double*> phi(d + 1, nullptr);
    for (int c = 2; c <= d - 2; ++c) {
        phi[c] = s.get<double>((size_t)std::max(T.nf[c], 1ll) * hv::lat_subsets(c, 1));
        hv::launch_lat_phi(L, c, T.nf[c], T.fref[c], T.fmask[c], T.F[c - 1], frame[c - 1], cen[c - 1], phi[c - 1],
                           phi[c], st);
    }
    // the edges' sums per generator pair, then the (facet, vertex) weights
    const long long nE = T.nf[d - 1];
    double* pe = s.get<double>((size_t)std::max(nE, 1ll) * hv::lat_subsets(d - 1, 1));
    hv::launch_lat_edgew(L, nE, T.fref[d - 1], T.fref2, T.fmask[d - 1], T.F[d - 2], cen[d - 2], phi[d - 2], pe, st);
    hv::launch_lat_qweights(L, m->nnbr, Q.foff, Q.qv, slot_cell, T.F[d - 1], pe, Q.qw, Q.qa, st);
    CK(cudaGetLastError());
}

// The integrand quadrature through the face lattice from d = 4 on
// (HV_QUAD_LATTICE=1 / 0 turns it on for every d >= 3 / off); the flag walk of
// hv_quad.cu otherwise (cheap in 3D: a facet's flags are its edges).
bool use_quad_lattice(int d, unsigned V) {
    int from = 4;
    if (const char* e = std::getenv("HV_QUAD_LATTICE")) from = e[0] == '0' ? 99 : e[0] == '1' ? 3 : from;
    if (d < std::max(from, 3) || d > 6) return false;
    long long emax = 0;
    for (int c = 1; c < d; ++c) emax = std::max(emax, (long long)V * hv::lat_subsets(d, c));
    return emax < (1ll << 31) - 2;
}

int polygon_impl(hv_mesh* m, double* vol, double* area, bool dev_out) {
    if (m && m->own0 >= 0) {  // a shard holds only its own vertices
        m->ctx->err = "integrate the merged mesh, not a shard";
        return HV_E_INVALID_ARG;
    }
    if (!m || (m->n > 0 && !vol)) return HV_E_INVALID_ARG;
    if (m->ext) {
        if (m->nnbr > 0 && !area) return HV_E_INVALID_ARG;
        return periodic_integrate(m, vol, area, dev_out, [&](hv_mesh* e, double* ev, double* ea) {
            return polygon_impl(e, ev, ea, true);
        });
    }
    if (m->g_max) return generic_polygon(m, vol, area, dev_out);
    try {
        CK(cudaSetDevice(m->ctx->device));
        ensure_neighbors(m);
        if (m->nnbr > 0 && !area) return HV_E_INVALID_ARG;
        if (m->n == 0) return HV_OK;
        hv_ctx* ctx = m->ctx;
        cudaStream_t st = ctx->stream;
        const int d = m->d, n = m->n;
        const long long ns = m->nnbr;
        const auto t0 = std::chrono::steady_clock::now();
        KTimer kt(ctx);
        Scratch s(st);
        hv::PolyRun R{};
        R.d = d; R.n = n; R.V = m->V; R.planes = m->d_planes;
        R.pts = m->d_in; R.osig = m->osig; R.oc = m->oc; R.nbr_off = m->nbr_off; R.nbr = m->nbr;
        R.nslots = ns; R.nsm = ctx->nsm; R.stream = st;
        R.cnt = s.get<unsigned long long>((size_t)ns + 1);
        long long* foff = s.get<long long>((size_t)ns + 1);
        R.foff = foff;
        R.slot_cell = s.get<int>((size_t)std::max(ns, 1ll));
        R.area = dev_out && ns > 0 ? area : s.get<double>((size_t)std::max(ns, 1ll));
        R.vol = dev_out ? vol : s.get<double>(n);
        // status, big facets (count, largest vertex count), huge facets (count, largest vertex count)
        unsigned* dstat = s.get<unsigned>(8);
        R.status = dstat; R.nbig = dstat + 1; R.maxnv = dstat + 2; R.nbig2 = dstat + 3; R.maxnv2 = dstat + 4;
        R.next = s.get<unsigned long long>(1);
        R.big = s.get<long long>((size_t)std::max(ns, 1ll));
        R.big2 = s.get<long long>((size_t)std::max(ns, 1ll));
        CK(cudaMemsetAsync(R.cnt, 0, sizeof(unsigned long long) * (ns + 1), st));
        CK(cudaMemsetAsync(dstat, 0, 8 * sizeof(unsigned), st));
        CK(cudaMemsetAsync(R.next, 0, sizeof(unsigned long long), st));
        CK(cudaMemsetAsync(R.area, 0, sizeof(double) * std::max(ns, 1ll), st));
        auto run = [&](int pass) {
            R.pass = pass;
            if (hv::launch_poly(R) != 0) throw HvError(HV_E_CUDA, "polygon integrator launch failed");
            CK(cudaGetLastError());
        };
        if (use_poly_lattice(d, m->V, ns) && !use_poly_flags(d)) {
            poly_lattice(m, R.area, R.slot_cell, dstat, s, kt);
            unsigned h0 = 0;
            CK(cudaMemcpyAsync(&h0, dstat, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            if (h0 & 8u) throw HvError(HV_E_INTERNAL, "a face is not a simple polytope (degenerate vertex)");
            run(4);
            if (!dev_out) {
                CK(cudaMemcpyAsync(vol, R.vol, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
                if (ns > 0) CK(cudaMemcpyAsync(area, R.area, sizeof(double) * ns, cudaMemcpyDeviceToHost, st));
            }
            CK(cudaStreamSynchronize(st));
            double fam[F_N];
            kt.totals(fam);
            m->st.poly_big_facets = 0;
            m->st.ms_poly_incidence = fam[0];
            m->st.ms_poly_facets = fam[1];
            m->st.ms_poly_big = 0;
            m->st.ms_poly_total =
                std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            return HV_OK;
        }
        // facet -> vertex incidences
        size_t scan_tb = hv::scan_temp((int)(ns + 1));
        void* scan_tmp = s.get<char>(scan_tb);
        kt.run(0, 2, [&] {
            run(0);
            hv::exclusive_scan_i64(scan_tmp, scan_tb, (const long long*)R.cnt, foff, (int)(ns + 1), st);
        });
        long long ninc = 0;
        CK(cudaMemcpyAsync(&ninc, foff + ns, sizeof(long long), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        R.fvert = s.get<unsigned>((size_t)std::max(ninc, 1ll));
        CK(cudaMemsetAsync(R.cnt, 0, sizeof(unsigned long long) * (ns + 1), st));
        kt.run(0, 1, [&] { run(1); });
        // tier A: shared-memory work areas
        static const int capA[7] = {0, 0, 2, 32, 64, 128, 256};
        int smax = 0;
        cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
        // HV_POLY_CAPS="a,b" lowers the tier-A and shared-memory tier-B vertex caps
        // (powers of two) so that small meshes exercise every tier
        int cap_a = capA[d], cap_b = 1 << 30;
        if (const char* e = std::getenv("HV_POLY_CAPS")) {
            int a = 0, b = 0;
            if (std::sscanf(e, "%d,%d", &a, &b) == 2 && a >= 2 && b >= 2) {
                cap_a = std::min(cap_a, (int)next_pow2((unsigned)a));
                cap_b = (int)next_pow2((unsigned)b);
            }
        }
        unsigned hs[3] = {0, 0, 0};
        bool flags = use_poly_flags(d);
        if (flags) {
            // every vertex's share of its facets, summed per cell in vertex order;
            // facets whose signed terms cancel go to the face-lattice kernels
            hv::FlagRun F{};
            F.d = d; F.n = n; F.V = m->V; F.planes = m->d_planes; F.pts = m->d_in; F.osig = m->osig; F.oc = m->oc;
            F.nbr_off = m->nbr_off; F.nbr = m->nbr; F.inc_off = m->inc_off; F.inc = m->inc; F.foff = foff;
            const size_t nsh = (size_t)std::max(m->V, 1u) * hv::flag_pairs(d);
            F.share = s.get<double>(nsh);
            F.sabs = s.get<float>(nsh);
            F.area = R.area; F.big = R.big; F.nbig = R.nbig; F.maxnv = R.maxnv; F.status = dstat;
            kt.run(1, 2, [&] {
                hv::launch_vertex_flags(F, ctx->nsm, st);
                hv::launch_cell_flags(F, ctx->nsm, st);
            });
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(hs, dstat, sizeof(hs), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            if (hs[0] & 2u) {  // a singular generator subset: the face lattice for every facet
                flags = false;
                CK(cudaMemsetAsync(dstat, 0, 8 * sizeof(unsigned), st));
                CK(cudaMemsetAsync(R.area, 0, sizeof(double) * std::max(ns, 1ll), st));
            }
        }
        if (!flags) {
            R.capV = cap_a;
            while (R.capV > 4 && hv::poly_area_bytes(d, R.capV, 1, false) > (size_t)smax) R.capV /= 2;
            kt.run(1, 1, [&] { run(2); });
            CK(cudaMemcpyAsync(hs, dstat, sizeof(hs), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
        }
        if (hs[0] & 8u) throw HvError(HV_E_INTERNAL, "a facet is not a simple polytope (degenerate vertex)");
        const unsigned nbig = hs[1];
        if (hs[1] > 0) {  // tier B: facets over the tier-A caps, one block each, shared memory
            R.nbig_host = hs[1];
            // the largest vertex cap that keeps two blocks per SM
            R.capV = 16;
            while (R.capV * 2 <= cap_b && hv::poly_area_bytes(d, R.capV * 2, 1, true) <= (size_t)smax / 2)
                R.capV *= 2;
            CK(cudaMemsetAsync(R.next, 0, sizeof(unsigned long long), st));
            kt.run(2, 1, [&] { run(3); });
            unsigned h2[5] = {0, 0, 0, 0, 0};
            CK(cudaMemcpyAsync(h2, dstat, sizeof(h2), cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
            if (h2[0] & 8u) throw HvError(HV_E_INTERNAL, "a facet is not a simple polytope (degenerate vertex)");
            if (h2[3] > 0) {  // the largest facets: global-memory work areas
                R.nbig_host = h2[3];
                R.capV = (int)next_pow2(h2[4]);
                R.blocks = (int)std::min<long long>(h2[3], 2ll * ctx->nsm);
                for (R.widen = 1;; R.widen *= 2) {
                    Scratch gs(st);
                    R.slab = gs.get<unsigned char>(hv::poly_area_bytes(d, R.capV, R.widen, true) * R.blocks);
                    CK(cudaMemsetAsync(R.next, 0, sizeof(unsigned long long), st));
                    CK(cudaMemsetAsync(dstat, 0, sizeof(unsigned), st));
                    kt.run(2, 1, [&] { run(5); });
                    CK(cudaMemcpyAsync(hs, dstat, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
                    CK(cudaStreamSynchronize(st));
                    if (hs[0] & 8u) throw HvError(HV_E_INTERNAL, "a facet is not a simple polytope (degenerate vertex)");
                    if (hs[0] == 0) break;
                    if (R.widen >= 8)
                        throw HvError(HV_E_CAPACITY, "facet structure beyond the polygon integrator's capacity");
                }
            }
        }
        run(4);
        if (!dev_out) {
            CK(cudaMemcpyAsync(vol, R.vol, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
            if (ns > 0) CK(cudaMemcpyAsync(area, R.area, sizeof(double) * ns, cudaMemcpyDeviceToHost, st));
        }
        CK(cudaStreamSynchronize(st));
        double fam[F_N];
        kt.totals(fam);
        m->st.poly_big_facets = nbig;
        m->st.poly_faces = m->st.poly_terms = m->st.poly_term_flops = 0;
        m->st.ms_poly_incidence = fam[0];
        m->st.ms_poly_facets = fam[1];
        m->st.ms_poly_big = fam[2];
        m->st.ms_poly_total =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

// The quadrature of the integrand path: facet -> vertex lists (the polygon
// integrator's incidence passes), then the flag weights and facet centres.
hv::QuadRun quad_run(hv_mesh* m) {
    hv::QuadRun Q{};
    Q.d = m->d; Q.n = m->n; Q.planes = m->d_planes; Q.pts = m->d_in; Q.osig = m->osig; Q.oc = m->oc;
    Q.nbr_off = m->nbr_off; Q.nbr = m->nbr; Q.nslots = m->nnbr; Q.foff = m->q_foff; Q.slot_cell = m->q_slot;
    Q.qv = m->q_v; Q.qw = m->q_w; Q.qa = m->q_a; Q.qc = m->q_c; Q.af = m->q_af;
    return Q;
}

void ensure_quad(hv_mesh* m, bool weights) {
    if (m->q_foff && (m->q_weights || !weights)) return;
    if (m->q_foff) {  // lists and centres exist: the flag weights on top
        for (void* p : {(void*)m->q_foff, (void*)m->q_slot, (void*)m->q_v, (void*)m->q_w, (void*)m->q_a,
                        (void*)m->q_c, (void*)m->q_af}) dfree(m->ctx->stream, p);
        m->q_foff = nullptr; m->q_slot = nullptr; m->q_v = nullptr; m->q_w = nullptr;
        m->q_a = nullptr; m->q_c = nullptr; m->q_af = nullptr;
    }
    ensure_neighbors(m);
    hv_ctx* ctx = m->ctx;
    cudaStream_t st = ctx->stream;
    const long long ns = m->nnbr;
    Scratch s(st);
    hv::PolyRun R{};
    R.d = m->d; R.n = m->n; R.V = m->V; R.planes = m->d_planes;
    R.pts = m->d_in; R.osig = m->osig; R.oc = m->oc; R.nbr_off = m->nbr_off; R.nbr = m->nbr;
    R.nslots = ns; R.nsm = ctx->nsm; R.stream = st;
    R.cnt = s.get<unsigned long long>((size_t)ns + 1);
    m->q_foff = dalloc<long long>(st, (size_t)ns + 1);
    m->q_slot = dalloc<int>(st, (size_t)std::max(ns, 1ll));
    R.foff = m->q_foff;
    R.slot_cell = m->q_slot;
    CK(cudaMemsetAsync(R.cnt, 0, sizeof(unsigned long long) * (ns + 1), st));
    auto run = [&](int pass) {
        R.pass = pass;
        if (hv::launch_poly(R) != 0) throw HvError(HV_E_CUDA, "quadrature incidence launch failed");
        CK(cudaGetLastError());
    };
    run(0);
    size_t tb = hv::scan_temp((int)(ns + 1));
    void* tmp = s.get<char>(tb);
    hv::exclusive_scan_i64(tmp, tb, (const long long*)R.cnt, m->q_foff, (int)(ns + 1), st);
    long long ninc = 0;
    CK(cudaMemcpyAsync(&ninc, m->q_foff + ns, sizeof(long long), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    unsigned* fvert = s.get<unsigned>((size_t)std::max(ninc, 1ll));
    R.fvert = fvert;
    CK(cudaMemsetAsync(R.cnt, 0, sizeof(unsigned long long) * (ns + 1), st));
    run(1);
    m->q_v = dalloc<unsigned>(st, (size_t)std::max(ninc, 1ll));
    m->q_w = dalloc<double>(st, (size_t)std::max(ninc, 1ll));
    m->q_a = dalloc<double>(st, (size_t)std::max(ns, 1ll));
    m->q_c = dalloc<double>(st, (size_t)std::max(ns, 1ll) * m->d);
    m->q_af = dalloc<double>(st, (size_t)std::max(ns, 1ll));
    unsigned* dstat = s.get<unsigned>(1);
    CK(cudaMemsetAsync(dstat, 0, sizeof(unsigned), st));
    CK(cudaMemsetAsync(m->q_a, 0, sizeof(double) * std::max(ns, 1ll), st));
    hv::QuadRun Q = quad_run(m);
    Q.fvert = fvert;
    Q.status = dstat;
    const bool lat = weights && use_quad_lattice(m->d, m->V);
    hv::launch_poly_quad(Q, weights && !lat, ctx->nsm, st);  // the sorted lists and the centres at least
    if (lat) quad_lattice(m, Q, dstat);
    m->q_weights = weights;
    hv::launch_quad_copy(Q, m->d, m->q_c, st);  // centres of the higher cells' slots
    CK(cudaGetLastError());
    unsigned hs = 0;
    CK(cudaMemcpyAsync(&hs, dstat, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (hs) {
        for (void* p : {(void*)m->q_foff, (void*)m->q_slot, (void*)m->q_v, (void*)m->q_w, (void*)m->q_a,
                        (void*)m->q_c, (void*)m->q_af}) dfree(st, p);
        m->q_foff = nullptr; m->q_slot = nullptr; m->q_v = nullptr; m->q_w = nullptr;
        m->q_a = nullptr; m->q_c = nullptr; m->q_af = nullptr;
        if (hs & 1u) throw HvError(HV_E_CAPACITY, "a facet has more vertices than the quadrature holds");
        throw HvError(HV_E_INTERNAL, "a facet is not a simple polytope (degenerate vertex)");
    }
}

int quad_check(hv_mesh* m) {
    if (!m) return HV_E_INVALID_ARG;
    if (m->g_max) {
        m->ctx->err = "the integrand quadrature needs vertices of d+1 generators";
        return HV_E_DEGENERATE;
    }
    if (m->ext || m->own0 >= 0) {
        m->ctx->err = "the integrand quadrature takes box and plane-domain meshes";
        return HV_E_INVALID_ARG;
    }
    return HV_OK;
}

int mc_impl(hv_mesh* m, int ndir, uint64_t seed, double* vol, double* area, bool dev_out) {
    if (m && m->own0 >= 0) {  // a shard holds only its own vertices
        m->ctx->err = "integrate the merged mesh, not a shard";
        return HV_E_INVALID_ARG;
    }
    if (!m || ndir <= 0 || (m->n > 0 && !vol)) return HV_E_INVALID_ARG;
    if (m->ext) {
        if (m->nnbr > 0 && !area) return HV_E_INVALID_ARG;
        return periodic_integrate(m, vol, area, dev_out, [&](hv_mesh* e, double* ev, double* ea) {
            return mc_impl(e, ndir, seed, ev, ea, true);
        });
    }
    try {
        CK(cudaSetDevice(m->ctx->device));
        ensure_neighbors(m);
        if (m->nnbr > 0 && !area) return HV_E_INVALID_ARG;
        if (m->n == 0) return HV_OK;
        cudaStream_t st = m->ctx->stream;
        const int d = m->d, n = m->n;
        std::vector<long long> no(n + 1);
        CK(cudaMemcpyAsync(no.data(), m->nbr_off, sizeof(long long) * (n + 1), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        long long maxdeg = 1;
        for (int i = 0; i < n; ++i) maxdeg = std::max(maxdeg, no[i + 1] - no[i]);
        const int capN = (int)((maxdeg + 7) / 8 * 8);
        int smax = 0;
        cudaDeviceGetAttribute(&smax, cudaDevAttrMaxSharedMemoryPerBlockOptin, m->ctx->device);
        const size_t sm = hv::mc_smem_bytes(d, capN);
        if ((long long)sm > smax) throw HvError(HV_E_CAPACITY, "cell degree too large for the MC integrator");
        Scratch s(st);
        const size_t E = (size_t)std::max(m->nnbr, 1ll);
        double* rawV = s.get<double>(n);
        double* varV = s.get<double>(n);
        double* dvol = dev_out ? vol : s.get<double>(n);
        double* rawA = s.get<double>(E);
        double* outA = dev_out && m->nnbr > 0 ? area : s.get<double>(E);
        unsigned* dstat = s.get<unsigned>(1);
        CK(cudaMemsetAsync(dstat, 0, sizeof(unsigned), st));
        hv::IntegrateInput in{d, n, m->lo, m->hi, m->np, m->d_planes, m->d_in, m->osig, m->oc, m->inc_off, m->inc, m->nbr_off, m->nbr, dstat};
        const double cvol = std::pow(M_PI, d / 2.0) / std::tgamma(1.0 + d / 2.0);
        if (hv::launch_heuristic_mc(in, ndir, seed, capN, cvol, rawV, rawA, varV, outA, dvol, m->ctx->nsm, st) != 0)
            throw HvError(HV_E_CUDA, "MC integrator launch failed");
        CK(cudaGetLastError());
        unsigned hs = 0;
        CK(cudaMemcpyAsync(&hs, dstat, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        if (!dev_out) {
            CK(cudaMemcpyAsync(vol, dvol, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
            if (m->nnbr > 0) CK(cudaMemcpyAsync(area, outA, sizeof(double) * m->nnbr, cudaMemcpyDeviceToHost, st));
        }
        CK(cudaStreamSynchronize(st));
        if (hs & 4u) throw HvError(HV_E_CAPACITY, "cell degree beyond the MC integrator's capacity");
        if (hs) throw HvError(HV_E_INTERNAL, "neighbour lists inconsistent (status " + std::to_string(hs) + ")");
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

}  // namespace

extern "C" {

int hv_integrate_polygon(hv_mesh* m, double* vol, double* area) { return polygon_impl(m, vol, area, false); }

int hv_mesh_facet_centers(hv_mesh* m, double* centers) {
    int rc = quad_check(m);
    if (rc != HV_OK) return rc;
    try {
        CK(cudaSetDevice(m->ctx->device));
        ensure_quad(m, false);
        if (m->nnbr > 0) {
            if (!centers) return HV_E_INVALID_ARG;
            CK(cudaMemcpyAsync(centers, m->q_c, sizeof(double) * m->nnbr * m->d, cudaMemcpyDeviceToHost,
                               m->ctx->stream));
        }
        CK(cudaStreamSynchronize(m->ctx->stream));
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

int hv_integrate_polygon_functions(hv_mesh* m, int p, const double* fv, const double* fc, const double* fx,
                                   double* iface, double* bulk) {
    int rc = quad_check(m);
    if (rc != HV_OK) return rc;
    if (p < 1 || (m->V > 0 && !fv) || !fx) return HV_E_INVALID_ARG;
    try {
        CK(cudaSetDevice(m->ctx->device));
        ensure_quad(m, true);
        const long long ns = m->nnbr;
        if (ns > 0 && (!fc || !iface)) return HV_E_INVALID_ARG;
        cudaStream_t st = m->ctx->stream;
        Scratch s(st);
        double* dfv = s.get<double>((size_t)std::max(m->V, 1u) * p);
        double* dfc = s.get<double>((size_t)std::max(ns, 1ll) * p);
        double* dfx = s.get<double>((size_t)m->n * p);
        double* dif = s.get<double>((size_t)std::max(ns, 1ll) * p);
        double* dbk = bulk ? s.get<double>((size_t)m->n * p) : nullptr;
        if (m->V) CK(cudaMemcpyAsync(dfv, fv, sizeof(double) * m->V * p, cudaMemcpyHostToDevice, st));
        if (ns) CK(cudaMemcpyAsync(dfc, fc, sizeof(double) * ns * p, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(dfx, fx, sizeof(double) * m->n * p, cudaMemcpyHostToDevice, st));
        hv::launch_quad_integrals(quad_run(m), p, dfv, dfc, dfx, dif, dbk, st);
        CK(cudaGetLastError());
        if (ns) CK(cudaMemcpyAsync(iface, dif, sizeof(double) * ns * p, cudaMemcpyDeviceToHost, st));
        if (bulk) CK(cudaMemcpyAsync(bulk, dbk, sizeof(double) * m->n * p, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

int hv_integrate_polygon_device(hv_mesh* m, double* d_vol, double* d_area) {
    return polygon_impl(m, d_vol, d_area, true);
}

int hv_integrate_heuristic_functions(hv_mesh* m, int p, const double* area, const double* fv, const double* fc,
                                     const double* fx, double* iface, double* bulk) {
    int rc = quad_check(m);
    if (rc != HV_OK) return rc;
    if (p < 1 || (m->V > 0 && !fv) || !fx) return HV_E_INVALID_ARG;
    try {
        CK(cudaSetDevice(m->ctx->device));
        ensure_quad(m, false);
        const long long ns = m->nnbr;
        if (ns > 0 && (!fc || !iface || !area)) return HV_E_INVALID_ARG;
        cudaStream_t st = m->ctx->stream;
        Scratch s(st);
        double* dar = s.get<double>((size_t)std::max(ns, 1ll));
        double* dfv = s.get<double>((size_t)std::max(m->V, 1u) * p);
        double* dfc = s.get<double>((size_t)std::max(ns, 1ll) * p);
        double* dfx = s.get<double>((size_t)m->n * p);
        double* dif = s.get<double>((size_t)std::max(ns, 1ll) * p);
        double* dbk = bulk ? s.get<double>((size_t)m->n * p) : nullptr;
        if (ns) CK(cudaMemcpyAsync(dar, area, sizeof(double) * ns, cudaMemcpyHostToDevice, st));
        if (m->V) CK(cudaMemcpyAsync(dfv, fv, sizeof(double) * m->V * p, cudaMemcpyHostToDevice, st));
        if (ns) CK(cudaMemcpyAsync(dfc, fc, sizeof(double) * ns * p, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(dfx, fx, sizeof(double) * m->n * p, cudaMemcpyHostToDevice, st));
        hv::launch_heur_integrals(quad_run(m), p, dar, dfv, dfc, dfx, dif, dbk, st);
        CK(cudaGetLastError());
        if (ns) CK(cudaMemcpyAsync(iface, dif, sizeof(double) * ns * p, cudaMemcpyDeviceToHost, st));
        if (bulk) CK(cudaMemcpyAsync(bulk, dbk, sizeof(double) * m->n * p, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

int hv_integrate_heuristic_mc(hv_mesh* m, int ndir, uint64_t seed, double* vol, double* area) {
    return mc_impl(m, ndir, seed, vol, area, false);
}

int hv_integrate_heuristic_mc_device(hv_mesh* m, int ndir, uint64_t seed, double* d_vol, double* d_area) {
    return mc_impl(m, ndir, seed, d_vol, d_area, true);
}

int hv_mesh_refine(hv_mesh* old, int64_t k, const double* pts, hv_mesh** out) {
    return refine_entry(old, k, pts, false, out);
}

int hv_mesh_refine_device(hv_mesh* old, int64_t k, const double* d_pts, hv_mesh** out) {
    return refine_entry(old, k, d_pts, true, out);
}

int hv_mesh_build_shard(hv_ctx* ctx, int d, int64_t n, const double* pts, const double* lo, const double* hi,
                        int rank, int nranks, const hv_params* params, hv_mesh** out) {
    return shard_entry(ctx, d, n, pts, false, lo, hi, rank, nranks, params, out);
}

int hv_mesh_build_shard_device(hv_ctx* ctx, int d, int64_t n, const double* d_pts, const double* lo,
                               const double* hi, int rank, int nranks, const hv_params* params, hv_mesh** out) {
    return shard_entry(ctx, d, n, d_pts, true, lo, hi, rank, nranks, params, out);
}

int hv_mesh_build_periodic(hv_ctx* ctx, int d, int64_t n, const double* pts, const double* lo, const double* hi,
                           const int* periodic, const hv_params* params, hv_mesh** out) {
    if (!ctx || !periodic || d < 2 || d > HV_MAXD) return HV_E_INVALID_ARG;
    int pmask = 0;
    for (int k = 0; k < d; ++k) pmask |= (periodic[k] ? 1 : 0) << k;
    if (!pmask) return hv_mesh_build(ctx, d, n, pts, lo, hi, params, out);
    return periodic_entry(ctx, d, n, pts, false, lo, hi, pmask, params, out);
}

int hv_mesh_build_periodic_device(hv_ctx* ctx, int d, int64_t n, const double* d_pts, const double* lo,
                                  const double* hi, const int* periodic, const hv_params* params, hv_mesh** out) {
    if (!ctx || !periodic || d < 2 || d > HV_MAXD) return HV_E_INVALID_ARG;
    int pmask = 0;
    for (int k = 0; k < d; ++k) pmask |= (periodic[k] ? 1 : 0) << k;
    if (!pmask) return hv_mesh_build_device(ctx, d, n, d_pts, lo, hi, params, out);
    return periodic_entry(ctx, d, n, d_pts, true, lo, hi, pmask, params, out);
}

int hv_mesh_periodic_shifts(hv_mesh* m, int8_t* shift) {
    if (!m || !shift) return HV_E_INVALID_ARG;
    try {
        CK(cudaSetDevice(m->ctx->device));
        ensure_neighbors(m);
        if (m->nnbr <= 0) return HV_OK;
        if (!m->pshift) {
            std::memset(shift, 0, (size_t)m->nnbr * m->d);
            return HV_OK;
        }
        CK(cudaMemcpyAsync(shift, m->pshift, (size_t)m->nnbr * m->d, cudaMemcpyDeviceToHost, m->ctx->stream));
        CK(cudaStreamSynchronize(m->ctx->stream));
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

int hv_mesh_periodic_images(hv_mesh* m, int64_t* nimages, double* delta, int64_t* ref, int8_t* shift) {
    if (!m || !nimages) return HV_E_INVALID_ARG;
    *nimages = m->nimg;
    if (delta)
        for (int k = 0; k < m->d; ++k) delta[k] = m->delta[k];
    if (m->nimg == 0 || (!ref && !shift)) return HV_OK;
    try {
        CK(cudaSetDevice(m->ctx->device));
        std::vector<int> r(m->nimg);
        std::vector<short> c(m->nimg);
        CK(cudaMemcpyAsync(r.data(), m->img_ref, sizeof(int) * m->nimg, cudaMemcpyDeviceToHost, m->ctx->stream));
        CK(cudaMemcpyAsync(c.data(), m->img_code, sizeof(short) * m->nimg, cudaMemcpyDeviceToHost, m->ctx->stream));
        CK(cudaStreamSynchronize(m->ctx->stream));
        for (int i = 0; i < m->nimg; ++i) {
            if (ref) ref[i] = (int64_t)r[i] + 1;
            int code = c[i];
            for (int k = 0; k < m->d; ++k) {
                if (shift) shift[(size_t)i * m->d + k] = (int8_t)(code % 3 - 1);
                code /= 3;
            }
        }
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

int hv_mesh_cell_vertices(hv_mesh* m, int64_t* offs, int64_t* vtx) {
    if (!m || !offs) return HV_E_INVALID_ARG;
    try {
        CK(cudaSetDevice(m->ctx->device));
        ensure_neighbors(m);
        cudaStream_t st = m->ctx->stream;
        CK(cudaMemcpyAsync(offs, m->inc_off, sizeof(int64_t) * (m->n + 1), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        const long long tot = offs[m->n];
        if (vtx && tot > 0) {
            Scratch s(st);
            int64_t* dv = s.get<int64_t>((size_t)tot);
            hv::launch_out_nbr(tot, m->inc, dv, st);  // 1-based vertex rows
            CK(cudaMemcpyAsync(vtx, dv, sizeof(int64_t) * tot, cudaMemcpyDeviceToHost, st));
            CK(cudaStreamSynchronize(st));
        }
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

int hv_mesh_device_views(hv_mesh* m, hv_device_views* out) {
    if (!m || !out) return HV_E_INVALID_ARG;
    try {
        CK(cudaSetDevice(m->ctx->device));
        ensure_neighbors(m);
        cudaStream_t st = m->ctx->stream;
        long long ninc = 0;
        CK(cudaMemcpyAsync(&ninc, m->inc_off + m->n, sizeof(long long), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        out->d = m->d;
        out->n = m->n;
        out->nverts = m->V;
        out->nnbr = m->nnbr;
        out->ncell_vertices = ninc;
        out->sig = m->g_max ? (m->g_max == m->d + 1 ? m->g_sig : nullptr) : m->osig;
        out->r = m->oc;
        out->nbr_off = (const int64_t*)m->nbr_off;
        out->nbr = m->nbr;
        out->vtx_off = (const int64_t*)m->inc_off;
        out->vtx = m->inc;
        out->pts = m->d_in;
        out->stream = (void*)st;
    } catch (const HvError& e) {
        return fail(m->ctx, e);
    }
    return HV_OK;
}

int hv_mesh_stats(hv_mesh* m, hv_stats* s) {
    if (!m || !s) return HV_E_INVALID_ARG;
    *s = m->st;
    return HV_OK;
}

int hv_mesh_free(hv_mesh* m) {
    if (!m) return HV_E_INVALID_ARG;
    cudaStream_t st = m->ctx->stream;
    cudaSetDevice(m->ctx->device);
    dfree(st, m->d_in);
    dfree(st, m->d_planes);
    dfree(st, m->osig);
    dfree(st, m->oc);
    dfree(st, m->inc_off);
    dfree(st, m->inc);
    dfree(st, m->nbr_off);
    dfree(st, m->nbr);
    dfree(st, m->img_ref);
    dfree(st, m->img_code);
    dfree(st, m->pshift);
    dfree(st, m->pperm);
    dfree(st, m->q_foff);
    dfree(st, m->q_slot);
    dfree(st, m->q_v);
    dfree(st, m->q_w);
    dfree(st, m->q_a);
    dfree(st, m->q_c);
    dfree(st, m->q_af);
    dfree(st, m->g_off);
    dfree(st, m->g_sig);
    dfree(st, m->g_fcell);
    dfree(st, m->g_fbeg);
    dfree(st, m->g_fend);
    dfree(st, m->g_fvert);
    dfree(st, m->t_pts);
    dfree(st, m->t_perm);
    dfree(st, m->t_blo);
    dfree(st, m->t_bhi);
    cudaStreamSynchronize(st);
    if (m->ext) hv_mesh_free(m->ext);
    delete m;
    return HV_OK;
}

}  // extern "C"
