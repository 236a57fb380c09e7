// Learned proposal of the simplex start (rlf_proposal.cu): what the pipeline calls.
#pragma once
#include <cuda_runtime.h>

namespace rlf {

int cnn_param_count();
// nonzero once rlf_proposal_set_params has loaded a network
int proposal_ready();
// proposals (e1, e2, step) of n galaxies from their packed facets (the fit's layout: cells of
// galaxy i at offset[i], count[i] of them, facet side facet[i], cell arrays of double or, with
// as_float, float); flux of galaxy i at flux[i * flux_stride]; start[3 i .. 3 i + 2] written on the
// device, ordered after the work queued on st and before the work queued on st afterwards
int propose_starts(int n, const int* offset, const int* count, const int* facet, const void* gu, const void* gv,
                   const void* dre, const void* dim, const void* sig2, int as_float, const double* flux,
                   int flux_stride, double len, double* start, cudaStream_t st);

}  // namespace rlf
