// Launchers of the visibility-weighting kernels (ingest.cpp).
#pragma once
#include <cuda_runtime_api.h>

#include <cstdint>

namespace pg {

// Blocks of the first stage of the deterministic sums.
constexpr int kIngestBlocks = 256;

// counts[p * Nu + q] += 1 with q = mod(floor(u * scale), Nu), p likewise
// (utilities.cc:583-587); integer atomics, so the counts are exact.
cudaError_t launch_weights_histogram(const double *u, const double *v, int64_t M, double scale,
                                     int Nu, int Nv, uint32_t *counts, cudaStream_t s);
// sums[0..1] = sum w^2 (complex, FP64, fixed reduction order), sums[2] =
// sum count^2 (exact, then converted); sums[4..] is scratch.
cudaError_t launch_weights_sums(const double *w, int64_t M, const uint32_t *counts,
                                int64_t ncells, double *sums, cudaStream_t s);
// out = w / sqrt(count) (uniform) or w / sqrt(1 + robust_scale * count)
// (robust) at each visibility's cell (utilities.cc:592-601).
cudaError_t launch_weights_apply(const double *u, const double *v, const double *w, int64_t M,
                                 double scale, int Nu, int Nv, const uint32_t *counts, bool robust,
                                 double rs_re, double rs_im, double *out, cudaStream_t s);

}  // namespace pg
