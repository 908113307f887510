// kernels.cuh -- launch wrappers of the device kernels.
#pragma once
#include <cuda_runtime.h>

#include "tk_internal.hpp"

namespace tk {

// FP64 grouped segmented GEMM over a tile list (one CTA per 64x64 tile).
constexpr int kF64TileM = 64;
constexpr int kF64TileN = 64;
// C = amul * alpha * A B (+ beta C, or + C when `accumulate`), per task.
cudaError_t launch_gemm_f64(const GemmTile* tiles, int n_tiles, const GemmTask* tasks, const GemmSeg* segs,
                            const double* A, const double* B, double* C, cudaStream_t s, double amul = 1.0,
                            bool accumulate = false);
// The same tables on planar complex operands (four launches): C = A B, or
// conj(A) B with conj_a; the tasks must overwrite their output (beta = 0).
cudaError_t launch_gemm_c64(const GemmTile* tiles, int n_tiles, const GemmTask* tasks, const GemmSeg* segs,
                            const double* Ar, const double* Ai, const double* Br, const double* Bi, double* Cr,
                            double* Ci, bool conj_a, cudaStream_t s);

// Channel combine: one CTA per job.
cudaError_t launch_combine_f64(const CombJob* jobs, int n_jobs, const CombTerm* terms, const double* in,
                               double* out, cudaStream_t s);

// Vector kernels used by the device Lanczos.
cudaError_t launch_fill_start_vector(double* v, int64_t n, cudaStream_t s);

}  // namespace tk
