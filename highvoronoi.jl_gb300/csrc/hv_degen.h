// hv_degen.h -- vertices with more than d+1 generators (hv_degen.cu).
#pragma once
#include <cuda_runtime.h>

#include "hv_internal.cuh"

namespace hv {

constexpr int GMAX = 64;  // generators of one vertex record (bit masks of 64)

enum : unsigned {
    GS_CAP = 1u,     // vertex store full (the host retries larger)
    GS_WIDE = 4u,    // a vertex with more than W generators (the host retries with GMAX)
    GS_SUBSETS = 64u, // a vertex with too many d-subsets to enumerate
    GS_NUMERIC = 8u, // singular centre system / no crossing along an edge
    GS_HASH = 16u,   // vertex table full
    GS_FACET = 32u,  // a facet with more than GMAX vertices (polygon)
};

// One walk of the vertex graph.  A vertex is (sorted original generator ids,
// count, FP64 centre), W ids a row.  Each level's walks write records; an
// insert pass keeps the first record of every generator set (open addressing
// on its FNV hash: a slot holds REC_TAG | record of this level or a vertex)
// and a commit pass appends the kept records to the vertices.
constexpr unsigned long long REC_TAG = 1ull << 62;
constexpr unsigned long long SLOT_EMPTY = ~0ull;
struct GenRun {
    DevMesh M;          // tree over the points (internal order), planes
    const double* x;    // n x d points, original order
    int W;              // ids per row (<= GMAX)
    int* vsig;          // vcap x W
    int* vlen;          // vcap
    double* vc;         // vcap x d
    unsigned vcap;
    unsigned* vcnt;
    int* rsig;          // records of the current level: rcap x W, count, centre
    int* rlen;
    double* rc;
    unsigned* rwin;     // hash slot + 1 of a kept record, else 0
    unsigned rcap;
    unsigned* rcnt;
    unsigned long long* htab;
    unsigned long long hmask;
    unsigned* e_vert;   // frontier edges: vertex, generator-slot mask, direction
    unsigned long long* e_F;
    double* e_u;
    unsigned e_cap;
    unsigned* e_cnt;
    unsigned* status;
};

// Vertex 0: the domain corner (d doubles, device), the planes through it and
// its nearest generators.
void launch_gen_seed(const GenRun& R, const double* corner, cudaStream_t st);
// Level-0 records from the search's vertices (vsig: nseed x (d+1) internal
// ids), each completed with every generator on its sphere (rcap >= nseed).
void launch_gen_seeds(const GenRun& R, const int* vsig, unsigned nseed, int nsm, cudaStream_t st);
void launch_gen_edges(const GenRun& R, unsigned f0, unsigned f1, int nsm, cudaStream_t st);
void launch_gen_walk(const GenRun& R, unsigned ne, int nsm, cudaStream_t st);
void launch_gen_insert(const GenRun& R, unsigned nrec, cudaStream_t st);
void launch_gen_commit(const GenRun& R, unsigned nrec, cudaStream_t st);

// Output: canonical order (lexicographic generator lists), CSR of the lists,
// centres; then the neighbour pairs and the cell -> vertex incidence.
size_t gen_sort_temp(unsigned V);
void gen_sort(const GenRun& R, unsigned V, int* order, void* temp, size_t temp_bytes, cudaStream_t st);
void launch_gen_lens(const GenRun& R, unsigned V, const int* order, long long* lens, unsigned* maxlen,
                     cudaStream_t st);
void launch_gen_fill(const GenRun& R, unsigned V, const int* order, const long long* off, int* sig, double* oc,
                     cudaStream_t st);
// pairs (i, j) of every vertex o with i a cell: count per vertex, then keys i << 32 | j with value o
void launch_gen_pair_count(int n, unsigned V, const long long* off, const int* sig, long long* cnt,
                           cudaStream_t st);
void launch_gen_pair_emit(int n, unsigned V, const long long* off, const int* sig, const long long* poff,
                          unsigned long long* keys, int* vals, cudaStream_t st);
// heads of the sorted pair runs: keep[q] = 1 if the run's cells share a full
// interface (a vertex of exactly d+1 generators, or vertices of affine rank
// d-1); qend[q] = end of the run
void launch_gen_heads(int d, long long npairs, const unsigned long long* keys, const int* vals, const long long* off,
                      const double* oc, long long* keep, long long* qend, cudaStream_t st);
void launch_gen_slots(long long npairs, const unsigned long long* keys, const long long* keep,
                      const long long* kpos, const long long* qend, int* nbr, int* fcell, long long* fbeg,
                      long long* fend, long long* ncnt, cudaStream_t st);
// cell -> vertex incidence: key i << 32 | o for every cell i of vertex o at
// position off[o] + slot (planes: ~0), cnt[i] += 1
void launch_gen_inc_emit(int n, unsigned V, const long long* off, const int* sig, unsigned long long* keys,
                         long long* cnt, cudaStream_t st);

// VI_POLYGON of such a mesh: the area of every facet by the pulling
// decomposition over its faces, copied to the higher cell, then the volumes.
struct GenPoly {
    int d, n;
    const DevPlane* planes;
    const double* pts;        // original order
    const long long* off;     // vertex -> generator list
    const int* sig;
    const double* oc;
    const long long* nbr_off;
    const int* nbr;
    const int* fcell;         // slot -> cell
    const long long* fbeg;    // slot -> range of its vertices in fvert
    const long long* fend;
    const int* fvert;
    long long nslots;
    unsigned* status;
};
void launch_gen_polygon(const GenPoly& P, double* area, double* vol, int nsm, cudaStream_t st);

// Vertex verification: cnt[0] += vertices with a generator strictly inside
// their sphere (or their centre beyond a plane), cnt[1] += vertices with a
// generator outside their signature on the sphere (relative 1e-10); maxdev =
// bits of the largest relative deviation of a vertex's own generators.  Rows
// of sig: off (CSR) or d+1 wide when off is null.
void launch_verify(const DevMesh& M, const double* x, unsigned V, const long long* off, const int* sig,
                   const double* oc, unsigned long long* cnt, unsigned long long* maxdev, cudaStream_t st);

}  // namespace hv
