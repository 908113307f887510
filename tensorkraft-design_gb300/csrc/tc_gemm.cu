// tc_gemm.cu -- split-precision (bf16x3) sector-GEMM path on tcgen05 tensor cores.
#include "tc_gemm.cuh"

namespace tk {

struct TcPlan {
    int unused = 0;
};

void TcPlanDeleter::operator()(TcPlan* p) const { delete p; }

tk_status tc_plan_create(const Heff2Tables&, const double*, const double*, std::unique_ptr<TcPlan, TcPlanDeleter>&,
                         std::string& err) {
    err = "split-precision path not built";
    return TK_ERR_UNSUPPORTED;
}

cudaError_t tc_apply(TcPlan&, const Heff2Tables&, const CombJob*, int, const CombTerm*, const double*, double*,
                     cudaStream_t, std::string& err) {
    err = "split-precision path not built";
    return cudaErrorNotSupported;
}

cudaError_t tc_apply_stage(TcPlan&, const Heff2Tables&, const CombJob*, int, const CombTerm*, const double*, double*,
                           cudaStream_t, int, std::string& err) {
    err = "split-precision path not built";
    return cudaErrorNotSupported;
}

}  // namespace tk
