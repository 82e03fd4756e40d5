// hv_integrate.h -- launchers of the per-cell integrators (hv_integrate.cu).
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>

namespace hv {

struct IntegrateInput {
    int d, n;
    const double* lo;
    const double* hi;
    const double* pts;        // original order, n x d
    const int* osig;          // V x (d+1), original 0-based items
    const double* oc;         // V x d
    const long long* inc_off; // cell -> vertex CSR
    const int* inc;
    const long long* nbr_off; // cell -> neighbour CSR (sorted items, planes n+p)
    const int* nbr;
    unsigned* status;         // 1: cell over capacity, 2: facet over capacity, 4: degree over capacity
};

struct PolyCaps {
    int capC, capV, capF, capE, capI;  // cell vertices, facet vertices, faces, edges, local items (powers of two)
};

size_t poly_smem_bytes(int d, int capC, int capV, int capF, int capE, int capI);
// pass 0: shared-memory kernel over all cells (big cells appended to `big`),
// pass 1: global-memory kernel over the big cells, pass 2: volumes.
int launch_polygon(const IntegrateInput& in, const PolyCaps& cs, const PolyCaps& cg, int* big, unsigned* nbig,
                   unsigned nbig_host, unsigned char* gbase, int gblocks, double* area, double* vol, int pass,
                   int nsm, cudaStream_t st);
int launch_heuristic_mc(const IntegrateInput& in, int ndir, unsigned long long seed, int capN, double cvol,
                        double* rawV, double* rawA, double* varV, double* outA, double* vol, int nsm,
                        cudaStream_t st);

}  // namespace hv
