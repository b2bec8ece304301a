// Mixed-precision FMM (FP32 far and near field) used inside FP64 iterative refinement.
#include "fmm_common.cuh"

namespace ibim {

void fmm_prepare_operators_mixed(Plan &, const KParams &) {
    throw Error(IBIM_ERR_INVALID_ARGUMENT, "mixed precision is not available in this build");
}

void fmm_run_mixed(Plan &, int, const ibim_kernel_params &, const double *, double *) {
    throw Error(IBIM_ERR_INVALID_ARGUMENT, "mixed precision is not available in this build");
}

}  // namespace ibim
