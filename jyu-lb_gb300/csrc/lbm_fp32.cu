// lbm_fp32.cu -- time step with FP32 storage of shifted populations
// (f_q - w_q) and FP32 arithmetic (physics in lbm_shifted.cuh): the direct
// kernel and the bulk-copy staged kernel.
#include "lbm_shifted.cuh"
#include "lbm_step_tma.cuh"

namespace jlb {

int launch_step_fp32(const StepArgs &a, int scheme, bool pstep, bool accf, int blocks, cudaStream_t st) {
    return launch_step_impl<StoreF32, PhysSh>(a, scheme, pstep, accf, blocks, st);
}

int launch_step_tma_fp32(const StepArgs &a, int scheme, bool pstep, bool accf, int grid, int ntiles, int nsb,
                         int *err, cudaStream_t st) {
    return launch_step_tma_impl<StoreF32, PhysSh>(a, scheme, pstep, accf, grid, ntiles, nsb, err, st);
}

int tma_blocks_per_sm_fp32(int scheme) {
    int nb = 0;
    const size_t smem = 2 * (size_t)TmaGeom<float>::STAGE * sizeof(float);
    cudaError_t e;
    if (scheme == SCH_BGK) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, lbm_step_tma_kernel<StoreF32, PhysSh<SCH_BGK>, true, false>, 128, smem);
    else if (scheme == SCH_TRT) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, lbm_step_tma_kernel<StoreF32, PhysSh<SCH_TRT>, true, false>, 128, smem);
    else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, lbm_step_tma_kernel<StoreF32, PhysSh<SCH_REG>, true, false>, 128, smem);
    return e == cudaSuccess ? nb : 0;
}

int launch_step_sparse_fp32(const StepArgs &a, int scheme, bool pstep, bool accf, int blocks, cudaStream_t st) {
    return launch_step_sparse_impl<StoreF32, PhysSh>(a, scheme, pstep, accf, blocks, st);
}

} // namespace jlb
