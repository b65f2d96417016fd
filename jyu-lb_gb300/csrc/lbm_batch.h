// lbm_batch.h -- device-side description of a batched ensemble of domains
// (lbm_batch.cu) and its launchers.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>
#include "lbm_common.h"

namespace jlb {

// node classes of the packed ensemble (uint8 per node)
constexpr uint8_t BCLS_PLAIN = 0;  // fluid, no bounce-back link
constexpr uint8_t BCLS_WALL = 1;   // fluid with bounce-back links to resting solids
constexpr uint8_t BCLS_MOVING = 2; // fluid with links to moving solids (Ladd)
constexpr uint8_t BCLS_SOLID = 3;  // not a fluid node
constexpr uint8_t BCLS_SPECIAL = 4; // boundary node (Zou-He / symmetric face): table path

struct BatchDomain {
    int32_t off;        // first packed node (multiple of 128)
    int32_t n;          // nx * ny * nz
    int32_t nx, ny, nz;
    int32_t first_tile; // first tile of this domain in the tile table
    float we, wo;       // relaxation rates
    float g[3];         // body force
    float uw[3];        // velocity of the domain's moving solids
    float inv_syz, inv_nz; // 1/(ny*nz), 1/nz for the site -> (i,j,k) split
    int32_t bc[6];         // face kinds (Zou-He kind of the boundary nodes)
};

struct BatchArgs {
    float *f;              // 19 * Np, f - w
    int64_t Np;            // slot stride (multiple of 128)
    float *fq[19];         // f + q * Np: population rows, indexed by 32-bit site
    const BatchDomain *dom;
    const int32_t *tile_dom;
    const uint8_t *ncls;
    const uint32_t *nmask; // bounce-back links (WALL / MOVING nodes)
    const uint32_t *mmask; // links whose source moves (MOVING nodes)
    float *dprev;          // previous-step rho - 1 (MOVING nodes)
    float *den, *ux, *uy, *uz;
    int write_moments;
    int ntiles;            // tiles of the launch
    int pf;                // L2 prefetch distance in tiles: the block of tile t
                           // prefetches the rows tile t + pf reads (0: none)
    // boundary nodes of the domains with Zou-He or symmetric faces, in the
    // single-domain table layout ([19][Msp] element indices into f, Zou-He
    // data fixed at set-up) with the domain of each
    int Msp;
    const int32_t *sp_dom;
    const int64_t *sp_node, *sp_rd, *sp_wr;
    const uint32_t *sp_info;
    const double *sp_lw, *sp_bc;
    float *sp_den;
};

int launch_batch_step(const BatchArgs &a, int scheme, bool pstep, int block, int ntiles, cudaStream_t st);
int launch_batch_pack(const float *src, int64_t Np_d, int32_t n_d, float *dst, int64_t Np, int32_t off,
                      cudaStream_t st);
// boundary nodes [t0, t1) are domain d's
int launch_batch_readout(const BatchArgs &a, int d, int n_d, int parity, int t0, int t1, double *out,
                         cudaStream_t st);
// the boundary nodes' step (after the dense launch of the same step)
int launch_batch_special(const BatchArgs &a, int scheme, bool pstep, cudaStream_t st);

} // namespace jlb
