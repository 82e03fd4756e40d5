// hv_integrate.h -- launchers of the per-cell integrators (hv_integrate.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace hv {

struct DevPlane;

struct IntegrateInput {
    int d, n;
    const double* lo;         // host arrays: bounding box of the domain
    const double* hi;
    int np;                   // boundary planes (device array), generator ids n + p
    const DevPlane* planes;
    const double* pts;        // original order, n x d
    const int* osig;          // V x (d+1), original 0-based items
    const double* oc;         // V x d
    const long long* inc_off; // cell -> vertex CSR
    const int* inc;
    const long long* nbr_off; // cell -> neighbour CSR (sorted items, planes n+p)
    const int* nbr;
    unsigned* status;         // 1: cell over capacity, 2: facet over capacity, 4: degree over capacity
};

// VI_POLYGON (hv_poly.cu).  pass 0: count facet-vertex incidences per
// neighbour slot and fill slot_cell; pass 1: fill fvert (cnt re-zeroed, foff
// = exclusive scan of the counts); pass 2: tier-A facet kernel (shared-memory
// work areas, facets of up to capV vertices; the others are listed in big);
// pass 3: tier-B facet kernel with a shared-memory work area over the
// nbig_host facets in big (over its caps: listed in big2); pass 5: tier-B
// kernel with global-memory work areas over the nbig_host facets in big2
// (caps from capV and widen); pass 4: cell volumes.
struct PolyRun {
    int d, n, pass;
    unsigned V;
    const DevPlane* planes;    // device array of boundary planes
    const double* pts;
    const int* osig;
    const double* oc;
    const long long* nbr_off;
    const int* nbr;
    long long nslots;
    unsigned long long* cnt;   // nslots + 1
    const long long* foff;
    unsigned* fvert;
    int* slot_cell;
    double* area;
    double* vol;
    unsigned* status;
    unsigned long long* next;  // work counter
    long long* big;
    unsigned* nbig;
    unsigned* maxnv;
    long long* big2;
    unsigned* nbig2;
    unsigned* maxnv2;
    long long nbig_host;
    int capV, widen, blocks, nsm;
    unsigned char* slab;
    cudaStream_t stream;
};
int launch_poly(const PolyRun& R);

// VI_POLYGON over the face lattice of the whole mesh (hv_polylat.cu), d >= 3.
// Level 1: F1[rank * V + v] = the facet slot of each generator pair of vertex
// v (-1 when its smaller generator is a plane), fref1[t] = the facet's smallest
// vertex (0xFFFFFFFF: no vertex, a slot of the higher cell).  Level c >= 2:
// entries (key, entry index rank * V + v) for every (c+1)-subset of every
// signature (lat_subsets(d, c) per vertex), sorted over the key's low bits;
// heads -> exclusive scan -> face index per entry (Fc), first vertex and mask
// per face (fref, fmask; fref2 = the second vertex of an edge).  Pairs: the
// child faces of level c+1 listed under their parents of level c.  Volumes:
// bottom-up; level 1 writes A_ik into both slots.  status bit 8: a face that is
// not simple or a signature pair that is not a neighbour pair.
struct LatIn {
    int d, n;
    unsigned V;
    const DevPlane* planes;
    const double* pts;
    const int* osig;
    const double* oc;
    const long long* nbr_off;
    const int* nbr;
    unsigned* status;
};
int lat_subsets(int d, int c);  // C(d+1, c+1): the (c+1)-subsets of a signature
void launch_lat_facets(const LatIn& L, int* F1, unsigned* fref1, int* slot_cell, cudaStream_t st);
void launch_lat_entries(const LatIn& L, int c, int gbits, const int* Fp, unsigned long long* keys, int* vals, int* Fc,
                        unsigned long long* nvalid, cudaStream_t st);
void launch_lat_heads(long long nval, const unsigned long long* sk, long long* flags, cudaStream_t st);
// hstart (optional): each face's first position in the sorted entries
void launch_lat_scatter(const LatIn& L, int c, long long nval, const long long* fidx, const int* sv, int* Fc,
                        unsigned* fref, unsigned char* fmask, unsigned* fref2, long long* hstart, cudaStream_t st);
void launch_lat_pairs(const LatIn& L, int c, long long nH, const unsigned* frefH, const unsigned char* fmaskH,
                      const int* Fc, const unsigned* frefG, unsigned long long* cnt, const long long* off, int* child,
                      int* lgen, int* par, bool fill, cudaStream_t st);
// volumes of level c from level c+1: prep (each parent's children in index
// order and, for c < d - 2, its frame of (c + 1) * d doubles), one term per
// pair, then each parent's sum (level 1: both slots of the interface)
void launch_lat_prep(const LatIn& L, int c, long long nG, const long long* off, int* child, int* lgen,
                     const unsigned* frefG, const unsigned char* fmaskG, const int* slot_cell, double* frame,
                     cudaStream_t st);
void launch_lat_terms(const LatIn& L, int c, long long npairs, const int* par, const int* child, const int* lgen,
                      const unsigned* frefG, const double* frame, const unsigned* frefH, const unsigned* fref2H,
                      const double* volH, double* term, cudaStream_t st);
void launch_lat_sum(const LatIn& L, int c, long long nG, const long long* off, const double* term,
                    const unsigned* frefG, const int* slot_cell, double* volG, cudaStream_t st);
long long lat_term_flops(int d, int c);  // FP64 operations of one term at level c
// Integrand quadrature over the same lattice (the reference's flag |det| as a
// product of centroid heights): face centroids of a level from its sorted
// entries; phi (C(c+1, 2) chain sums per face of level c, from level c-1's
// frames (launch_lat_prep with off = nullptr), centroids and phi); per edge
// C(d, 2) sums over its 2-faces; the (facet, vertex) weights into qw and each
// facet's flag sum into qa (foff / qv: the facets' sorted vertex lists).
void launch_lat_centroid(const LatIn& L, long long nf, long long nval, const long long* hstart, const int* sv,
                         double* cen, cudaStream_t st);
void launch_lat_phi(const LatIn& L, int c, long long nQ, const unsigned* frefQ, const unsigned char* fmaskQ,
                    const int* Fp, const double* frameP, const double* cenP, const double* phiP, double* phiQ,
                    cudaStream_t st);
void launch_lat_edgew(const LatIn& L, long long nE, const unsigned* frefE, const unsigned* fref2E,
                      const unsigned char* fmaskE, const int* Fp, const double* cenP, const double* phiP, double* pe,
                      cudaStream_t st);
void launch_lat_qweights(const LatIn& L, long long ns, const long long* foff, const unsigned* qv,
                         const int* slot_cell, const int* Fe, const double* pe, double* qw, double* qa,
                         cudaStream_t st);

// VI_POLYGON areas from the vertices alone (hv_polyflag.cu): every vertex's
// share of the facets through it (signed flag terms over the circumcentres of
// its generator subsets), then per cell the shares in vertex order.  Facets
// whose terms cancel go to big (the exact tier-B kernels); status bit 2: a
// singular generator subset (the host then runs the face-lattice kernels).
struct FlagRun {
    int d, n;
    unsigned V;
    const DevPlane* planes;
    const double* pts;
    const int* osig;
    const double* oc;
    const long long* nbr_off;
    const int* nbr;
    const long long* inc_off;  // cell -> vertex rows, ascending
    const int* inc;
    const long long* foff;     // facet slot -> its vertex range (the incidence passes)
    double* share;             // V x d(d+1)/2
    float* sabs;               // V x d(d+1)/2: sum of the shares' |terms|
    double* area;
    long long* big;
    unsigned* nbig;
    unsigned* maxnv;
    unsigned* status;
};
int flag_pairs(int d);
void launch_vertex_flags(const FlagRun& F, int nsm, cudaStream_t st);
void launch_cell_flags(const FlagRun& F, int nsm, cudaStream_t st);

// Integrand quadrature of VI_POLYGON (hv_quad.cu): per facet of a lower cell
// (slot t with a non-empty incidence range foff[t] .. foff[t+1]) the facet's
// vertices in id order (qv), their flag weights (qw), the flag sum (qa) and the
// facet centre (qc, slots x d); af receives the facet areas of every slot.
struct QuadRun {
    int d, n;
    const DevPlane* planes;
    const double* pts;        // n x d, original order
    const int* osig;          // V x (d+1), original items, planes n+p
    const double* oc;         // V x d
    const long long* nbr_off;
    const int* nbr;
    long long nslots;
    const long long* foff;
    const unsigned* fvert;
    const int* slot_cell;
    unsigned* qv;
    double* qw;
    double* qa;
    double* qc;
    double* af;
    unsigned* status;         // 1: facet over QUAD_MAXV vertices, 8: facet not simple
};
void launch_poly_quad(const QuadRun& Q, bool weights, int nsm, cudaStream_t st);
void launch_heur_integrals(const QuadRun& Q, int p, const double* area, const double* fv, const double* fc,
                           const double* fx, double* iface, double* bulk, cudaStream_t st);
// per-slot values a (slots x p) of the higher cells copied from the lower cell's slot
void launch_quad_copy(const QuadRun& Q, int p, double* a, cudaStream_t st);
void launch_quad_integrals(const QuadRun& Q, int p, const double* fv, const double* fc, const double* fx,
                           double* iface, double* bulk, cudaStream_t st);
// Work-area bytes: per block for tier A, per block (one group) for tier B.
size_t poly_area_bytes(int d, int capV, int widen, bool tier_b);
// dynamic shared memory of the MC cell kernel for cells of up to capN neighbours
size_t mc_smem_bytes(int d, int capN);
int launch_heuristic_mc(const IntegrateInput& in, int ndir, unsigned long long seed, int capN, double cvol,
                        double* rawV, double* rawA, double* varV, double* outA, double* vol, int nsm,
                        cudaStream_t st);

}  // namespace hv
