// lbm_fp16.cu -- time step with FP16 storage of 2^12 (f_q/w_q - 1) and FP32
// arithmetic (physics in lbm_shifted.cuh): direct and bulk-copy staged kernels.
#include "lbm_shifted.cuh"
#include "lbm_step_tma.cuh"

namespace jlb {

int launch_step_fp16(const StepArgs &a, int scheme, bool pstep, bool accf, int blocks, cudaStream_t st) {
    return launch_step_impl<StoreF16, PhysH16>(a, scheme, pstep, accf, blocks, st);
}

int launch_step_tma_fp16(const StepArgs &a, int scheme, bool pstep, bool accf, int grid, int ntiles, int nsb,
                         int *err, cudaStream_t st) {
    return launch_step_tma_impl<StoreF16, PhysH16>(a, scheme, pstep, accf, grid, ntiles, nsb, err, st);
}

int launch_step_tma_h2_fp16(const StepArgs &a, int scheme, bool accf, int grid, int ntiles, int kb2, int nsb,
                            int *err, cudaStream_t st) {
    return launch_step_tma_h2_impl<PhysH16>(a, scheme, accf, grid, ntiles, kb2, nsb, err, st);
}

int tma_h2_blocks_per_sm_fp16(int scheme) { return tma_h2_blocks_per_sm<PhysH16>(scheme); }

int tma_blocks_per_sm_fp16(int scheme) {
    int nb = 0;
    const size_t smem = 2 * (size_t)TmaGeom<__half>::STAGE * sizeof(__half);
    cudaError_t e;
    if (scheme == SCH_BGK) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, lbm_step_tma_kernel<StoreF16, PhysH16<SCH_BGK>, true, false>, 128, smem);
    else if (scheme == SCH_TRT) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, lbm_step_tma_kernel<StoreF16, PhysH16<SCH_TRT>, true, false>, 128, smem);
    else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, lbm_step_tma_kernel<StoreF16, PhysH16<SCH_REG>, true, false>, 128, smem);
    return e == cudaSuccess ? nb : 0;
}

// the fluid-only layout keeps the decoded physics: its kernel holds the 18
// neighbour indices in registers, and the stored-value collision would spill
int launch_step_sparse_fp16(const StepArgs &a, int scheme, bool pstep, bool accf, int blocks, cudaStream_t st) {
    return launch_step_sparse_impl<StoreF16, PhysSh>(a, scheme, pstep, accf, blocks, st);
}

} // namespace jlb
