/*
 * hv_oracle.h -- C API of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a CPU restatement of
 * HighVoronoi.jl's mesh-generation hot path (vertex search by raycasting,
 * neighbour extraction, VI_POLYGON and VI_HEURISTIC_MC integration).  It is
 * used by tests/ as the parity checker, by __graft_entry__.smoke() and by the
 * CPU-baseline leg of bench.py.  The product (libhvgpu) never links or calls it.
 *
 * Index conventions follow the reference: generators are 1-based, boundary
 * plane p (1-based, cuboid order of src/boundary.jl:518-534: plane 2k-1 is the
 * upper face x_k = hi_k, plane 2k the lower face x_k = lo_k; or the p-th plane
 * given to the *_planes entry points) is generator N+p.
 * Point arrays are d x n column-major (Julia layout), i.e. point i occupies
 * pts[d*i .. d*i+d-1].
 */
#ifndef HV_ORACLE_H
#define HV_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct hvo_mesh hvo_mesh;

/* Counters of rare events and work (rays, quad-precision re-scores, ...). */
typedef struct {
    int64_t rays;            /* incircle searches issued (descent + edge walks) */
    int64_t descents;        /* descent attempts */
    int64_t descent_retries; /* descents rejected by the empty-sphere check */
    int64_t quad_rescores;   /* rays whose FP64 decision was not certified */
    int64_t degenerate;      /* ties that survived quad precision */
    int64_t cell_vertices;   /* sum over cells of vertices found */
    int64_t chains;          /* polyintegrator simplices evaluated */
} hvo_stats;

/* Build the mesh.  mode 0: every cell enumerates its own polytope (OpenMP over
 * cells); mode 1: the reference's sequential rule (cells in index order, edges
 * walked only from their minimal generator).  integrate: 0 none, 1 polygon.
 * Returns 0 on success, <0 on error. */
int hvo_build(int d, int64_t n, const double* pts, const double* lo, const double* hi,
              uint64_t seed, int nthreads, int mode, int integrate, hvo_mesh** out);
/* Same inside the convex domain of np planes (base, normal: d x np column-major;
 * the domain is (x - base_p) . normal_p < 0 for every p, normals scaled to unit
 * length). */
int hvo_build_planes(int d, int64_t n, const double* pts, int np, const double* base, const double* normal,
                     uint64_t seed, int nthreads, int mode, int integrate, hvo_mesh** out);

int64_t hvo_num_vertices(const hvo_mesh* m);
int64_t hvo_num_neighbors(const hvo_mesh* m);
/* Vertices sorted lexicographically by their 1-based signature. */
void hvo_vertices(const hvo_mesh* m, int64_t* sig, double* r);
void hvo_neighbors(const hvo_mesh* m, int64_t* offs, int64_t* nbr);
/* Volumes (n) and interface areas aligned with hvo_neighbors.  Needs integrate=1. */
int hvo_polygon(const hvo_mesh* m, double* vol, double* area);
/* Heuristic Monte-Carlo volumes/areas with ndir Philox directions per cell.
 * vol_var / area_var (optional, may be NULL) receive the variance of the
 * per-cell estimators (sample variance / ndir) before two-sided averaging. */
int hvo_heuristic_mc(const hvo_mesh* m, int ndir, uint64_t seed, int nthreads,
                     double* vol, double* area, double* vol_var, double* area_var);
/* recycle > 0: hvo_heuristic_mc uses the reference's direction batches instead
 * of i.i.d. directions -- one vector for every sample of `recycle` consecutive
 * cells (new_directions! never resets its rejection flag,
 * src/mcintegrator.jl:82-95).  0 restores the i.i.d. estimator. */
void hvo_set_mc_reference_directions(int recycle);
/* A mesh holding only the given neighbour CSR (offs n+1, nbr 1-based, planes
 * n+p of the box [lo, hi]): hvo_heuristic_mc runs on it (phase timing). */
int hvo_mesh_from_csr(int d, int64_t n, const double* pts, const double* lo, const double* hi,
                      const int64_t* offs, const int64_t* nbr, hvo_mesh** out);
void hvo_get_stats(const hvo_mesh* m, hvo_stats* st);
const char* hvo_last_error(void);
void hvo_free(hvo_mesh* m);

/* CPU-baseline sample: run the per-cell search for the listed cells (0-based)
 * and report the number of vertices they own (minimal generator) and the
 * wall time.  Returns 0 on success. */
int hvo_sample_cells(int d, int64_t n, const double* pts, const double* lo, const double* hi,
                     uint64_t seed, int nthreads, int64_t ncells, const int64_t* cells,
                     int64_t* owned_vertices, int64_t* rays, double* seconds);

/* Brute-force verification of a vertex list: empty open circumsphere w.r.t.
 * every generator and equidistance to the signature.  Returns the number of
 * violating vertices (0 = all verified). */
int64_t hvo_verify_vertices(int d, int64_t n, const double* pts, const double* lo, const double* hi,
                            int64_t nv, const int64_t* sig, const double* r, double rel_tol);
int64_t hvo_verify_vertices_planes(int d, int64_t n, const double* pts, int np, const double* base,
                                   const double* normal, int64_t nv, const int64_t* sig, const double* r,
                                   double rel_tol);

/* VI_POLYGON volumes (ncells) and interface areas of the listed cells (0-based),
 * each computed from the cell's own polytope, in a CSR of capacity cap:
 * offs (ncells+1), items (1-based neighbours, sorted), area.  Returns -4 if
 * cap is too small (offs[ncells] then holds the size needed). */
int hvo_polygon_cells(int d, int64_t n, const double* pts, const double* lo, const double* hi, uint64_t seed,
                      int nthreads, int64_t ncells, const int64_t* cells, int64_t cap, double* vol, int64_t* offs,
                      int64_t* items, double* area);

/* Certificate of a vertex list independent of the oracle's search (box
 * [lo, hi] when np == 0, else the np planes base/normal): out[0] vertices with
 * a generator strictly inside their circumsphere or a centre beyond a plane, out[1]
 * exact ties, out[2] invalid signatures, out[3] edges without exactly two end
 * points, out[4] duplicate signatures, out[5] binary128 re-decisions;
 * *maxdev = largest coordinate deviation from the FP64 circumcentre. */
int hvo_certify_mesh(int d, int64_t n, const double* pts, const double* lo, const double* hi, int np,
                     const double* base, const double* normal, int64_t nv, const int64_t* sig, const double* r,
                     int nthreads, int64_t* out, double* maxdev);

/* Integrals of tabulated functions (p components) with the reference's
 * polygon quadrature: fv at the vertices (hvo_vertices rows), fc at the facet
 * centres (hvo_facet_centers), fx at the generators; interface integrals
 * aligned with hvo_neighbors (nnbr x p) and, if bulk, cell integrals (n x p).
 * Needs integrate=1. */
int hvo_polygon_functions(const hvo_mesh* m, int p, const double* fv, const double* fc, const double* fx, int bulk,
                          double* iface, double* bulkint);
int hvo_facet_centers(const hvo_mesh* m, double* centers);
/* The heuristic integrand rule on given interface areas (aligned with
 * hvo_neighbors); needs integrate=1. */
int hvo_heuristic_functions(const hvo_mesh* m, int p, const double* area, const double* fv, const double* fc,
                            const double* fx, int bulk, double* iface, double* bulkint);

/* Raw Philox4x32-10 block (for known-answer tests of the generator). */
void hvo_philox4x32(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Philox4x32-10 unit directions shared with the GPU MC kernel (for tests). */
void hvo_mc_directions(int d, int64_t cell, int ndir, uint64_t seed, double* dirs);

/* Vertices with more than d+1 generators (lattices, co-spherical points): the
 * vertex graph of the box [lo, hi] walked from the corner lo in binary128;
 * every vertex keeps all generators on its sphere, neighbours share a full
 * interface, integrate=1 adds the polygon volumes and areas. */
int hvo_build_generic(int d, int64_t n, const double* pts, const double* lo, const double* hi, int integrate,
                      hvo_mesh** out);
/* Total signature length over the vertices, and the vertices as a CSR:
 * offs (V+1), sig (1-based, sorted per vertex), r (V x d). */
int64_t hvo_sig_total(const hvo_mesh* m);
void hvo_vertices_csr(const hvo_mesh* m, int64_t* offs, int64_t* sig, double* r);

#ifdef __cplusplus
}
#endif
#endif
