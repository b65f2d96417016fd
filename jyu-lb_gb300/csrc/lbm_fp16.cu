// lbm_fp16.cu -- time step with FP16 storage of 2^12 (f_q/w_q - 1) and FP32
// arithmetic (physics in lbm_shifted.cuh).
#include "lbm_shifted.cuh"

namespace jlb {

int launch_step_fp16(const StepArgs &a, int scheme, bool pstep, bool accf, int blocks, cudaStream_t st) {
    return launch_step_impl<StoreF16, PhysSh>(a, scheme, pstep, accf, blocks, st);
}

} // namespace jlb
