// tc_gemm.cuh -- split-precision (bf16x3) sector-GEMM path on tcgen05 tensor cores.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <string>

#include "tk_internal.hpp"

namespace tk {

struct TcPlan;
struct TcPlanDeleter {
    void operator()(TcPlan* p) const;
};

// Builds the split operands of L and R (constant across matvecs) and the
// tile tables of both GEMM stages.
tk_status tc_plan_create(const Heff2Tables& host, const double* d_lbuf, const double* d_rbuf,
                         std::unique_ptr<TcPlan, TcPlanDeleter>& out, std::string& err);

// One split-precision matvec, stream-ordered.
cudaError_t tc_apply(TcPlan& tc, const Heff2Tables& host, const CombJob* d_jobs, int n_jobs,
                     const CombTerm* d_terms, const double* x, double* y, cudaStream_t s, std::string& err);

// One stage of the split-precision matvec (0: L x psi, 1: combine, 2: x R), for profiling.
cudaError_t tc_apply_stage(TcPlan& tc, const Heff2Tables& host, const CombJob* d_jobs, int n_jobs,
                           const CombTerm* d_terms, const double* x, double* y, cudaStream_t s, int stage,
                           std::string& err);

}  // namespace tk

namespace tk {
// Adds to *bad (device) the number of inputs where the split kernels' integer
// fp64 -> fp32 conversion differs from the hardware conversion.
cudaError_t tc_conversion_check(const double* x, int64_t n, unsigned long long* bad, cudaStream_t s);
// Device error word of the tensor-core kernels (0 = no bounded wait ran out).
int* tc_error_word(TcPlan& tc);
// Kernel launches of one split-precision matvec (tc_apply).
int tc_launches(const TcPlan& tc);
// True (and the split point) when stage 1 can run as two launches, the first
// reading psi only below *x_split: every stack splits psi in the GEMM kernel.
bool tc_psi_halves(const TcPlan& tc, int64_t* x_split);
// Stage-1 tiles of one psi half (0: those reading below the split only; 1: the rest).
cudaError_t tc_stage1_half(TcPlan& tc, const double* x, int half, cudaStream_t s);
// Synchronises `s`, reads and clears the error word: TK_ERR_TIMEOUT if set.
tk_status tc_check_error(TcPlan& tc, cudaStream_t s);
}  // namespace tk
