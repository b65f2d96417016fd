// lbm_adjoint.h -- arguments and launcher of the adjoint step kernels
// (lbm_adjoint.cu).
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>
#include "lbm_common.h"

namespace jlb {

struct AdjArgs {
    StepArgs s;            // the forward step's geometry, tables and parameters
    const void *snap;      // AA state before this step, [19][Np] (storage type)
    const void *sp_in;     // collision inputs of the boundary sites, [19][M]
    void *lam;             // adjoint AA array, [19][Np] (storage type)
    int seed;              // 1 on the step whose stored velocity enters the loss
    int plane;             // x index of the loss plane
    const double *target;  // (ny, nz, 3) target velocity on the plane
    double *part;          // [adjoint_blocks][5] per-block sums of d/d we, d/d wo,
                           // d/d a_x, a_y, a_z (accumulated over the sweep)
    double *grad_bc;       // [4][M] d/d (den, ux, uy, uz) of each boundary site's Zou-He
                           // data (accumulated), or NULL
    uint32_t param_faces;  // faces (bit f = face f) whose Zou-He data are parameters
    void *lam_den;         // [M] adjoint of each boundary site's density of the step
                           // (compute type; read by the next step's moving-wall
                           // links), or NULL when no link moves
};

// one step of the reverse sweep (one launch)
int launch_adjoint_step(const AdjArgs &A, int prec, int scheme, bool pstep, cudaStream_t st);
// number of per-block sensitivity slots the launches use
int adjoint_blocks(const StepArgs &a);

} // namespace jlb
