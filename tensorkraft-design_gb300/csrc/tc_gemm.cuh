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
// The launch forms of a built plan (combine form, persistent or narrow stage
// 1): the options that do not shape the split tables, applied in place.
tk_status tc_set_launch_forms(TcPlan& p, const TcOptions& o, std::string& err);

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
// True when stage 1 can run as k launches over psi in k pieces (k divides
// kTcPsiPieces; every stack splits psi in the GEMM kernel): x_cut[0..k] are the
// piece boundaries in psi, and tiles1[n1_cut[j], n1_cut[j + 1]) read psi only
// below x_cut[j + 1].
bool tc_psi_pieces(const TcPlan& tc, int k, int64_t* x_cut, int32_t* n1_cut);
// Stage-1 tiles [first, first + count) of the in-kernel-split list.
cudaError_t tc_stage1_range(TcPlan& tc, const double* x, int first, int count, cudaStream_t s);
// Synchronises `s`, reads and clears the error word: TK_ERR_TIMEOUT if set.
tk_status tc_check_error(TcPlan& tc, cudaStream_t s);
}  // namespace tk
