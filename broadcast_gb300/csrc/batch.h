// Residual (+ K-direction tangent) of many independent grids of uneven size
// in one set of launches.
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <vector>
#include "dnc5.cuh"

namespace bcg {

struct BatchPlan;

// ngrid grids (gh = 3), phys holds 11 values per grid (cp cv prandtl gam rgaz
// cs muref tref s_suth k2 k4); ndir = 0, 1, 2 or 4 directions per grid.
int batch_create(int ngrid, const int* im, const int* jm, const double* phys, int ndir, BatchPlan** out);
// device addresses per grid: w, wd (ndir planes of 5*np), nx, ny, vol, volf, res, resd
int batch_set_arrays(BatchPlan* p, const unsigned long long* w, const unsigned long long* wd,
                     const unsigned long long* nx, const unsigned long long* ny, const unsigned long long* vol,
                     const unsigned long long* volf, const unsigned long long* res, const unsigned long long* resd);
// tile (threads per CTA) of the face pass and of the cell passes, and CTAs
// per SM of the persistent grids; drops a captured graph
int batch_configure(BatchPlan* p, int tile_faces, int tile_cells, int ctas_per_sm);
// tile shapes of the chunk plans of host-array runs (batch_run_host) alone
int batch_configure_host(BatchPlan* p, int tile_faces, int tile_cells, int ctas_per_sm);
int batch_run(BatchPlan* p, int use_graph, cudaStream_t st);
// one pass alone (0 primitives, 1 gradients, 2 interpolation rows, 3 viscous
// point values, 4 faces, 5 balance), for timing each kernel of a run
int batch_run_pass(BatchPlan* p, int pass, cudaStream_t st);
// one evaluation with host arrays: uploads, graph replays and interior
// downloads of nchunk chunks of grids overlap; returns when the outputs are
// in the host arrays
int batch_run_host(BatchPlan* p, int nchunk, const unsigned long long* w, const unsigned long long* wd,
                   const unsigned long long* nx, const unsigned long long* ny, const unsigned long long* vol,
                   const unsigned long long* volf, const unsigned long long* res, const unsigned long long* resd,
                   cudaStream_t st);
void batch_destroy(BatchPlan* p);
size_t batch_device_bytes(const BatchPlan* p);

}  // namespace bcg
