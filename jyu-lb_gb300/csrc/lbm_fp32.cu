// lbm_fp32.cu -- time step with FP32 storage of shifted populations
// (f_q - w_q) and FP32 arithmetic (physics in lbm_shifted.cuh).
#include "lbm_shifted.cuh"

namespace jlb {

int launch_step_fp32(const StepArgs &a, int scheme, bool pstep, bool accf, int blocks, cudaStream_t st) {
    return launch_step_impl<StoreF32, PhysSh>(a, scheme, pstep, accf, blocks, st);
}

} // namespace jlb
