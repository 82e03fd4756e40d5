/*
 * hvgpu.h -- C ABI of libhvgpu, the GB300 (sm_103a) implementation of
 * HighVoronoi.jl's mesh-generation hot path.
 *
 * The library replaces, behind a `search_settings=(method=RCGPU,)` switch,
 * the whole-mesh vertex search and the per-cell integrators of HighVoronoi.jl:
 *
 *   hv_mesh_build          voronoi(mesh; searcher)                src/sysvoronoi.jl:21-39
 *                          (_voronoi / __voronoi / systematic_explore_cell /
 *                          walkray / raycast_des2, src/sysvoronoi.jl:41-552,
 *                          src/raycast.jl:45-1049), called from
 *                          VoronoiGeometry, src/geometry.jl:153-156
 *   hv_mesh_vertices       the vertex database the search fills    src/abstractmesh.jl:111-127
 *                          (push!(mesh, sig=>r)); read back as VoronoiData
 *                          vertices, src/voronoidata.jl:545-700
 *   hv_mesh_neighbors      neighbors_of_cell                       src/neighbors.jl:219-258
 *   hv_integrate_polygon   integrate_geo with VI_POLYGON           src/geometry.jl:203-263,
 *                          src/polyintegrator.jl:80-468, src/cleanup_cell.jl:174-204
 *   hv_integrate_heuristic_mc  integrate_geo with VI_HEURISTIC_MC  src/heuristic_mc.jl:1-56,
 *                          src/mcintegrator.jl:98-226
 *   hv_mesh_stats          the rare-event counters SRI_*          src/raycast-types.jl:497-539
 *
 * Conventions (identical to the reference): generators are 1-based; the
 * domain is the non-periodic cuboid [lo, hi] (cuboid(d, dimensions=hi-lo,
 * offset=lo, periodic=[]), src/boundary.jl:518-534) whose plane p (1-based,
 * 2k-1 = upper face of axis k, 2k = lower face) is generator n+p, or (the
 * *_planes builds) a convex domain of Dirichlet/Neumann planes given by base
 * points and normals (Boundary(planes...), src/boundary.jl:94-131) whose plane
 * p is generator n+p; every vertex signature is sorted ascending.  Point arrays are d x n column-major doubles
 * (Julia layout): point i occupies pts[d*i .. d*i+d-1].
 *
 * Ownership: the caller owns all host arrays; device memory belongs to the
 * library and is released by hv_mesh_free / hv_ctx_destroy.
 * Errors: every call returns HV_OK (0) or a negative HV_E_* code; the text of
 * the last error of a context is returned by hv_last_error.
 * Threading: one hv_ctx per host thread (each context owns one CUDA stream).
 */
#ifndef HVGPU_H
#define HVGPU_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define HV_VERSION 10000 /* 1.0.0 */

#define HV_OK 0
#define HV_E_INVALID_ARG (-1)
#define HV_E_OOM (-2)
#define HV_E_CAPACITY (-3)
#define HV_E_DEGENERATE (-4)
#define HV_E_TIMEOUT (-5)
#define HV_E_CUDA (-6)
#define HV_E_INTERNAL (-7)

/* Raycast method, the GPU counterpart of the reference's method singletons
 * (src/raycast-types.jl:244-285). */
#define HV_METHOD_FAST 0  /* batched split-precision raycast (FP32 filter, FP64 verify) */
#define HV_METHOD_PLAIN 1 /* one ray per thread, FP64, exact tree search */
/* vertices of any number of generators (lattices): the fast search, then a
 * walk of the vertex graph in which every vertex keeps all generators on its
 * sphere.  A FAST build switches to it by itself when it meets co-spherical
 * generators (box and plane domains). */
#define HV_METHOD_GENERIC 2

typedef struct hv_ctx hv_ctx;
typedef struct hv_mesh hv_mesh;

/* Search settings (the GPU part of the reference's RaycastParameter,
 * src/raycast-types.jl:312-349).  Zero means "choose automatically". */
typedef struct {
    int method;           /* HV_METHOD_FAST, HV_METHOD_PLAIN or HV_METHOD_GENERIC */
    int knn;              /* candidate-list length per generator */
    int leaf_size;        /* points per tree leaf */
    int rays_per_warp;    /* vertices expanded per warp in the fast kernel (1 or 2) */
    int seed_stride;      /* run a descent from every k-th generator */
    int edge_dedup;       /* 0/1: skip edges whose both end points are known (edge table, default); -1: walk all */
    uint64_t seed;        /* seed of the descent directions */
    double capacity_factor; /* vertex capacity headroom over the per-dimension estimate */
} hv_params;

typedef struct {
    int64_t vertices;       /* unique Voronoi vertices */
    int64_t rays;           /* incircle searches issued (edge walks) */
    int64_t fallback_rays;  /* rays redone by the exact FP64 tree search */
    int64_t uncertified;    /* FP32 decisions that needed FP64 */
    int64_t insecure;       /* candidate list did not cover the new sphere */
    int64_t dd_rescores;    /* FP64 decisions redone in double-double */
    int64_t degenerate;     /* ties that survived double-double */
    int64_t descents;       /* descent seeds */
    int64_t descent_retries;
    int64_t levels;         /* wavefront levels */
    int64_t edges_closed;   /* edges skipped because both end points were known */
    int64_t capacity_retries;
    int64_t launches;       /* kernels launched by this mesh build */
    double ms_prepare;      /* upload, sort, tree, candidate lists */
    double ms_search;       /* descent + wavefront */
    double ms_total;        /* whole hv_mesh_build (host wall clock) */
    /* device time per kernel family, CUDA events on the context's stream */
    double ms_knn;          /* candidate lists */
    double ms_descent;      /* seed vertices */
    double ms_expand;       /* wavefront expansion (fast or plain kernel) */
    double ms_fallback;     /* exact re-walks of uncertified/insecure rays */
    double ms_centers;      /* FP64 circumcentres of new vertices */
    double ms_canonical;    /* canonical renumbering */
    /* last hv_integrate_polygon on this mesh */
    int64_t poly_big_facets;   /* facets redone with global-memory work areas */
    double ms_poly_incidence;  /* facet -> vertex lists (device; the face lattice: see below) */
    double ms_poly_facets;     /* shared-memory facet kernel (device; the face lattice: its terms) */
    double ms_poly_big;        /* global-memory facet kernel (device) */
    double ms_poly_total;      /* whole call (host wall clock) */
    /* tree pass of the FP32 fallback (rays whose candidate list may miss the winner) */
    int64_t fallback_tree_rays;
    int64_t fallback_nodes;    /* tree nodes tested */
    int64_t fallback_leaves;   /* leaves scanned */
    int64_t fallback_points;   /* points inside the bounding ball (interval-evaluated) */
    int64_t ambiguous_sets;    /* candidate sets decided in FP64 after the FP32 tree search */
    /* last hv_integrate_polygon through the mesh-wide face lattice (d >= 3; zero
     * for the per-facet kernels): ms_poly_incidence is then the lattice build,
     * the children's order, the frames and the sums, ms_poly_facets the terms */
    int64_t poly_faces;        /* faces of codimension 2 .. d-1 */
    int64_t poly_terms;        /* (face, sub-face) terms of the pulling decomposition */
    int64_t poly_term_flops;   /* FP64 operations of those terms (algorithmic count, FMA = 2) */
} hv_stats;

int hv_version(void);
void hv_params_default(hv_params* p);

int hv_ctx_create(int device, hv_ctx** out);
int hv_ctx_destroy(hv_ctx* ctx);
const char* hv_last_error(hv_ctx* ctx);
/* The CUDA stream (cudaStream_t) on which the context runs all its work, for
 * callers that order their own work or timing events against it. */
void* hv_ctx_stream(hv_ctx* ctx);

/* Vertex search of the Voronoi mesh of n points (host array, d x n) inside the
 * cuboid [lo, hi] (host arrays of length d).  2 <= d <= 6. */
int hv_mesh_build(hv_ctx* ctx, int d, int64_t n, const double* pts, const double* lo, const double* hi,
                  const hv_params* params, hv_mesh** out);
/* Same with pts already in device memory (d x n doubles on the context's device). */
int hv_mesh_build_device(hv_ctx* ctx, int d, int64_t n, const double* d_pts, const double* lo,
                         const double* hi, const hv_params* params, hv_mesh** out);
/* Vertex search inside the convex domain {x : (x - base_p) . normal_p <= 0
 * for every p} of nplanes (1..64) boundary planes (Plane(base, normal, BC),
 * src/boundary.jl:22-29; membership test src/boundary.jl:427-435).  base and
 * normal are d x nplanes column-major host arrays (plane p at [d*p .. d*p+d-1]);
 * normals are scaled to unit length (the reference's reflection,
 * src/boundary.jl:206-211, assumes unit normals).  bc (nplanes entries, may be
 * NULL) takes the reference's codes: Dirichlet and Neumann planes are accepted,
 * periodic ones (bc > 0) are HV_E_INVALID_ARG.  An unbounded domain or one
 * with an empty interior is HV_E_INVALID_ARG.  Plane p (0-based) is generator
 * n+p+1 in the 1-based output. */
int hv_mesh_build_planes(hv_ctx* ctx, int d, int64_t n, const double* pts, int nplanes, const double* base,
                         const double* normal, const int16_t* bc, const hv_params* params, hv_mesh** out);
/* Same with pts already in device memory (base, normal and bc stay host arrays). */
int hv_mesh_build_planes_device(hv_ctx* ctx, int d, int64_t n, const double* d_pts, int nplanes,
                                const double* base, const double* normal, const int16_t* bc,
                                const hv_params* params, hv_mesh** out);

/* Autotuner: times hv_mesh_build over a small grid of knn x leaf_size x
 * seed_stride (x rays_per_warp) on the given points (pts == NULL: uniform
 * points in the box) and writes the fastest settings to *out.  The result is
 * cached in the context per (d, round(log2 n)); later builds on the context
 * whose params leave those fields at 0 use the cached values. */
int hv_autotune(hv_ctx* ctx, int d, int64_t n, const double* pts, const double* lo, const double* hi,
                hv_params* out);

/* Sizes of the caller's buffers: vertices, and the total neighbour count. */
int hv_mesh_counts(hv_mesh* mesh, int64_t* nverts, int64_t* nnbr_total);
/* Vertex records sorted lexicographically by signature: sig is (d+1) x V
 * (1-based, sorted), r is d x V.  HV_E_DEGENERATE if a vertex has more than
 * d+1 generators (read those with hv_mesh_vertices_csr). */
int hv_mesh_vertices(hv_mesh* mesh, int64_t* sig, double* r);
/* Vertices of any number of generators -- the reference's vertex database
 * holds every generator on a vertex's sphere (push!(mesh, sig => r),
 * src/abstractmesh.jl:111-127; lattices put 2^d points on one sphere).
 * hv_mesh_signature_total sizes the buffers: the summed signature length and
 * the longest one.  hv_mesh_vertices_csr writes offs (V+1, 0-based), sig (the
 * 1-based ascending signatures back to back) and r (d x V), in lexicographic
 * order of the signatures (a shorter signature before its extensions). */
int hv_mesh_signature_total(hv_mesh* mesh, int64_t* total, int* max_len);
int hv_mesh_vertices_csr(hv_mesh* mesh, int64_t* offs, int64_t* sig, double* r);
/* Vertex verification on the device, the check of the reference's
 * verify_vertex / fraud_vertex (src/raycast.jl:477-502,
 * src/sysvoronoi.jl:527-552): *inside = vertices with a generator strictly
 * inside their sphere or a centre beyond a boundary plane (0 for a correct
 * mesh); *ties = vertices with a generator outside their signature on their
 * sphere (relative 1e-10; 0 unless generators are co-spherical and the
 * vertex list is fixed-width); *max_dev = largest relative deviation of a
 * vertex's own generators from its sphere (and of its planes).  Box,
 * plane-domain, refined and generic meshes (the search's tree stays with the
 * mesh); periodic meshes are HV_E_INVALID_ARG. */
int hv_mesh_verify(hv_mesh* mesh, int64_t* inside, int64_t* ties, double* max_dev);
/* Neighbour CSR: offs[n+1] (0-based offsets), nbr (1-based, sorted per cell,
 * planes as n+p). */
int hv_mesh_neighbors(hv_mesh* mesh, int64_t* offs, int64_t* nbr);
/* Exact cell volumes (n) and interface areas aligned with hv_mesh_neighbors. */
int hv_integrate_polygon(hv_mesh* mesh, double* vol, double* area);
/* Integrals of a user function with VI_POLYGON's quadrature, the
 * reference's Polygon_Integrator with an integrand (integrand= of
 * VoronoiGeometry, src/polyintegrator.jl:80-123,174-330).  The library cannot
 * call the function, so the caller evaluates it at the quadrature nodes:
 *   the vertices (rows of hv_mesh_vertices), the facet centres (the mean of
 *   each facet's vertices, nnbr x d aligned with hv_mesh_neighbors, from
 *   hv_mesh_facet_centers) and the generators;
 * and hv_integrate_polygon_functions forms, for p function components, the
 * interface integrals (nnbr x p, aligned with the neighbour lists, the lower
 * cell's value for both directions) and, if bulk is not NULL, the cell
 * integrals (n x p) with the reference's rule: along each facet's flag
 * simplices the edge average (f(r1)+f(r2))/2 with weight (d-1)/d and the
 * facet centre with weight 1/d; bulk_i = sum_k V_ik f(x_i)/(d+1) +
 * I_ik h_ik/(d+1).  A constant function gives the areas and volumes.  Box
 * and plane-domain meshes; in 2D and 3D facets of up to 1024 vertices
 * (HV_E_CAPACITY; from 4D the weights come from the mesh's face lattice, with
 * no per-facet cap). */
int hv_mesh_facet_centers(hv_mesh* m, double* centers);
int hv_integrate_polygon_functions(hv_mesh* m, int p, const double* fv, const double* fc, const double* fx,
                                   double* iface, double* bulk);
/* Integrals of a user function with the reference's heuristic rule of
 * VI_HEURISTIC_MC (Heuristic_Integrator, src/heuristic.jl:105-166) on given
 * interface areas (nnbr, aligned with hv_mesh_neighbors; normally those of
 * hv_integrate_heuristic_mc): I = A ((d-1)/d mean of f over the facet's
 * vertices + f(c_F)/d), bulk_i = sum_k h_ik/d (A_ik f(x_i)/(d+1) +
 * d/(d+1) I_ik).  Nodes and arguments as hv_integrate_polygon_functions.  Every
 * facet uses all its vertices (the reference keeps a single vertex for facets
 * toward lower-numbered neighbours, which depends on its storage order). */
int hv_integrate_heuristic_functions(hv_mesh* m, int p, const double* area, const double* fv, const double* fc,
                                     const double* fx, double* iface, double* bulk);
/* Monte-Carlo volumes and areas, ndir Philox directions per cell. */
int hv_integrate_heuristic_mc(hv_mesh* mesh, int ndir, uint64_t seed, double* vol, double* area);
/* Periodic cuboid [lo, hi] (cuboid(d, periodic=...), src/boundary.jl:510-534):
 * periodic[k] != 0 makes axis k periodic, the other faces stay Dirichlet.
 * The mesh of the generators and of their periodic images in a widened box is
 * searched (the reference's periodize!, src/domain.jl:139-213) and reduced to
 * the periodic tessellation: every accessor below then reports the n original
 * cells, naming a neighbour image by its original (1-based) id and its lattice
 * shift (hv_mesh_periodic_shifts); vertex signatures list original ids (a
 * generator may appear twice through two of its images), coordinates are the
 * true positions (a vertex on a periodic seam appears once per translate that
 * touches an original cell); non-periodic faces keep the ids n+p.
 * HV_E_CAPACITY when the generators are too few for any image margin. */
int hv_mesh_build_periodic(hv_ctx* ctx, int d, int64_t n, const double* pts, const double* lo, const double* hi,
                           const int* periodic, const hv_params* params, hv_mesh** out);
int hv_mesh_build_periodic_device(hv_ctx* ctx, int d, int64_t n, const double* d_pts, const double* lo,
                                  const double* hi, const int* periodic, const hv_params* params, hv_mesh** out);
/* Incremental refinement (refine!, src/meshrefine.jl:183,
 * src/geometry.jl:404-438): the mesh of old's generators plus k new points
 * (host array d x k; the _device form takes them in device memory), numbered
 * n+1 .. n+k after the old ones, boundary plane p becoming generator n+k+p.
 * Only the new generators' cells are searched; an old vertex stays unless a
 * new point lies inside its circumsphere; the vertex records come out in the
 * same canonical order as hv_mesh_build of all points gives (if a new point
 * lies on an old circumsphere within rounding, the whole set is searched).
 * old stays valid; box and plane domains, fast method; not periodic meshes
 * or shards (HV_E_INVALID_ARG). */
int hv_mesh_refine(hv_mesh* old, int64_t k, const double* pts, hv_mesh** out);
int hv_mesh_refine_device(hv_mesh* old, int64_t k, const double* d_pts, hv_mesh** out);
/* One shard of the box mesh split over nranks GPUs (one rank each), the
 * GPU form of the reference's cell split between threads
 * (_voronoi(::MultiThread), src/sysvoronoi.jl:50-76).  Every rank passes all
 * points; the generators are ordered along the library's Morton curve and
 * rank r takes the r-th of nranks contiguous ranges of that order (sizes
 * differ by at most one).  The shard searches the vertices of its own cells
 * only and keeps those whose first generator in that order is its own, so
 * every vertex of the mesh belongs to exactly one shard.  hv_mesh_counts /
 * hv_mesh_vertices / hv_mesh_stats report the kept vertices (1-based
 * original ids, sorted signatures, lexicographic order); all-gathering them
 * and sorting the union gives hv_mesh_build's vertex records, from which the
 * neighbour lists follow.  The integrators refuse a shard (HV_E_INVALID_ARG):
 * they run on the merged mesh.  Fast method only. */
int hv_mesh_build_shard(hv_ctx* ctx, int d, int64_t n, const double* pts, const double* lo, const double* hi,
                        int rank, int nranks, const hv_params* params, hv_mesh** out);
int hv_mesh_build_shard_device(hv_ctx* ctx, int d, int64_t n, const double* d_pts, const double* lo,
                               const double* hi, int rank, int nranks, const hv_params* params, hv_mesh** out);
/* Lattice shift s (nnbr x d, entries -1, 0, 1) of every neighbour entry: the
 * neighbour of cell i is the image x_j + s * (hi - lo).  Zeros for
 * non-periodic meshes. */
int hv_mesh_periodic_shifts(hv_mesh* m, int8_t* shift);
/* The images the periodic search added (the reference's references /
 * reference_shifts, src/voronoidata.jl:9-15): their count, the margin delta
 * (d) of the widened box and, if the arrays are given, the 1-based original
 * (nimages) and the lattice shift (nimages x d) of every image. */
int hv_mesh_periodic_images(hv_mesh* m, int64_t* nimages, double* delta, int64_t* ref, int8_t* shift);

/* Cell -> vertex incidences: offs (n+1) and, when vtx is not NULL, the
 * 1-based row indices (into the hv_mesh_vertices order) of the vertices of
 * every cell, ascending (the reference's VoronoiData.vertices,
 * src/voronoidata.jl:545-700).  Call with vtx == NULL to size vtx by offs[n]. */
int hv_mesh_cell_vertices(hv_mesh* m, int64_t* offs, int64_t* vtx);

/* Zero-copy hand-off: device pointers into the mesh's own arrays (valid until
 * hv_mesh_free; read-only; on the context's device).  Indices are 0-based,
 * boundary plane p (0-based) is n+p; signature rows are sorted and the rows
 * are in the hv_mesh_vertices order.  Julia can wrap them with
 * unsafe_wrap(CuArray, ...), Python through __cuda_array_interface__. */
typedef struct {
    int d;
    int64_t n, nverts, nnbr, ncell_vertices;
    const int32_t* sig;       /* nverts x (d+1); NULL if a vertex has more than d+1 generators */
    const double* r;          /* nverts x d */
    const int64_t* nbr_off;   /* n+1 */
    const int32_t* nbr;       /* nnbr, sorted per cell, planes last */
    const int64_t* vtx_off;   /* n+1 */
    const int32_t* vtx;       /* ncell_vertices vertex rows, ascending per cell */
    const double* pts;        /* n x d generators, original order */
    void* stream;             /* cudaStream_t the arrays are ordered on */
} hv_device_views;
int hv_mesh_device_views(hv_mesh* m, hv_device_views* out);

/* The integrators with outputs in caller device memory (vol: n doubles,
 * area: nnbr doubles aligned with the neighbour CSR); complete on return. */
int hv_integrate_polygon_device(hv_mesh* m, double* d_vol, double* d_area);
int hv_integrate_heuristic_mc_device(hv_mesh* m, int ndir, uint64_t seed, double* d_vol, double* d_area);

int hv_mesh_stats(hv_mesh* mesh, hv_stats* stats);
int hv_mesh_free(hv_mesh* mesh);

/* Heuristic Monte-Carlo volumes and areas for callers that cannot allocate
 * device memory: an application that has already committed the whole device
 * memory budget, a loop where allocator calls are not allowed, or a framework
 * that hands out fixed buffers.  It computes what hv_integrate_heuristic_mc
 * computes, but every input and output is a caller-owned device buffer and the
 * scratch lives in a static device array of HV_NOALLOC_SCRATCH_BYTES that this
 * library holds on every GPU that loads it.  No counterpart in the reference.
 *   domain     the cuboid [lo, hi] only (host arrays of length d); its faces
 *              are the items n .. n+2d-1 in hv_mesh_build's order: n+2k is
 *              the upper face x_k = hi_k, n+2k+1 the lower face x_k = lo_k
 *   d_pts      n x d doubles (device), d_nbr_off n+1 int64 and d_nbr nnbr int32
 *              (device): neighbour CSR with 0-based generators, every row
 *              sorted ascending and the relation symmetric (j in row i iff i
 *              in row j), as hv_mesh_neighbors returns it minus one for a box
 *              mesh; max_degree >= every row length
 *   d_vol      n doubles (device), d_area nnbr doubles (device), stream a
 *              cudaStream_t (NULL: legacy default stream); returns synchronised
 * Limits: HV_NOALLOC_FIXED_BYTES + 8 (2 n + nnbr) bytes must fit the scratch
 * (else HV_E_CAPACITY, checked before any device work).  HV_E_INVALID_ARG if
 * a row is longer than max_degree, an item lies outside 0 .. n+2d-1 (or a
 * cell lists itself), or a row k does not list i while row i lists k.
 * The first call on a device looks up the scratch address on that device
 * (call it once before any stream capture).  Calls share the scratch: calls
 * that overlap on the GPU race. */
#define HV_NOALLOC_SCRATCH_BYTES (16u << 20)
/* Fixed part of the scratch: a 256-byte status block and the 2d box planes. */
#define HV_NOALLOC_FIXED_BYTES 1536u
int hv_integrate_heuristic_mc_noalloc(int d, int64_t n, const double* d_pts, const double* lo, const double* hi,
                                      const int64_t* d_nbr_off, const int32_t* d_nbr, int64_t nnbr, int max_degree,
                                      int ndir, uint64_t seed, double* d_vol, double* d_area, void* stream);

/* ------------------------------------------------------------------------
 * Serving: continuous batching of mesh requests on one device.
 *
 * The server owns `slots` contexts (one CUDA stream and one worker thread
 * each).  Requests are admitted in arrival order as soon as a slot is free and
 * the HBM estimate of the request fits into the remaining budget next to the
 * requests already running; the running requests' kernels overlap on the
 * device.  Results do not depend on what else is running (every result is a
 * pure function of its request).  There is no reference counterpart: the
 * reference builds one mesh per call.
 * ------------------------------------------------------------------------ */
typedef struct hv_server hv_server;

#define HV_INTEGRATOR_NONE 0
#define HV_INTEGRATOR_POLYGON 1
#define HV_INTEGRATOR_HEURISTIC_MC 2

typedef struct {
    int device;
    int slots;               /* concurrent requests (worker threads / streams) */
    double hbm_budget_bytes; /* admission budget; 0 = 80% of free device memory */
} hv_server_config;

typedef struct {
    int d;
    int64_t n;
    const double* pts;       /* d x n, copied at submission */
    const double* lo;
    const double* hi;
    int integrator;          /* HV_INTEGRATOR_* */
    int ndir;                /* directions per cell for HV_INTEGRATOR_HEURISTIC_MC */
    uint64_t mc_seed;
    hv_params params;
    /* Domains beyond the box (a zero-initialised tail keeps the box [lo, hi]):
     * periodic != NULL: d flags, the periodic cuboid of hv_mesh_build_periodic;
     * nplanes > 0: the convex domain of hv_mesh_build_planes (lo, hi unused). */
    const int* periodic;
    int nplanes;
    const double* base;      /* d x nplanes */
    const double* normal;    /* d x nplanes */
    const int16_t* bc;       /* nplanes boundary conditions, or NULL */
} hv_request;

typedef struct {
    int status;              /* HV_OK or the HV_E_* code of the failed request */
    int d;
    int64_t n, nverts, nnbr;
    const int64_t* sig;      /* (d+1) x nverts, owned by the server until hv_server_release */
    const double* r;         /* d x nverts */
    const int64_t* offs;     /* n+1 */
    const int64_t* nbr;      /* nnbr */
    const double* vol;       /* n (NULL without integrator) */
    const double* area;      /* nnbr (NULL without integrator) */
    double queue_ms;         /* submission -> start of service */
    double service_ms;       /* start of service -> result ready */
    double latency_ms;       /* submission -> result ready */
    hv_stats stats;
    const int8_t* shift;     /* d x nnbr lattice shifts of the neighbours (periodic requests), else NULL */
    const int64_t* sig_offs; /* nverts+1 row offsets of sig when a vertex has more than d+1 generators
                                (co-spherical generators, hv_mesh_vertices_csr); NULL: sig is (d+1) wide */
} hv_result;

int hv_server_start(const hv_server_config* cfg, hv_server** out);
/* Copies the request and returns a ticket; HV_E_OOM if it can never fit the budget. */
int hv_server_submit(hv_server* s, const hv_request* req, int64_t* ticket);
/* done = 1 once the ticket's result is ready. */
int hv_server_poll(hv_server* s, int64_t ticket, int* done);
/* Blocks until the result is ready (timeout_ms < 0: no limit; HV_E_TIMEOUT on expiry). */
int hv_server_wait(hv_server* s, int64_t ticket, double timeout_ms, hv_result* out);
/* Frees the result buffers of a ticket. */
int hv_server_release(hv_server* s, int64_t ticket);
/* Drains running requests, stops the workers and frees the server. */
int hv_server_stop(hv_server* s);

#ifdef __cplusplus
}
#endif
#endif
