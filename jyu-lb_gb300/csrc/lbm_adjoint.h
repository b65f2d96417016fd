// lbm_adjoint.h -- arguments and launcher of the adjoint step kernel
// (lbm_adjoint.cu).
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>
#include "lbm_common.h"

namespace jlb {

struct AdjArgs {
    StepArgs s;            // the forward step's geometry, tables and parameters
    const void *gin;       // collision inputs of this step, [19][Np] (storage type)
    void *lam;             // adjoint AA array, [19][Np] (storage type)
    int seed;              // 1 on the step whose stored velocity enters the loss
    int plane;             // x index of the loss plane
    const double *target;  // (ny, nz, 3) target velocity on the plane
    double *grad;          // [5] d/d we, d/d wo, d/d a_x, a_y, a_z (accumulated)
    double *grad_uin;      // [ny*nz] d/d u_x of the FIXED_VEL face 1X (accumulated)
};

int launch_adjoint_step(const AdjArgs &A, int prec, int scheme, bool pstep, int blocks, cudaStream_t st);

} // namespace jlb
