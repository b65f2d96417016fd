// lbm_common.h -- types shared by the host runtime and the CUDA kernels of
// the D3Q19 engine.
//
// Lattice: the reference's D3Q19 enumeration (jyulb/D3Q19.pxd:59-79),
//   q : 0(-1,-1,0) 1(-1,0,-1) 2(-1,0,0) 3(-1,0,1) 4(-1,1,0) 5(0,-1,-1)
//       6(0,-1,0) 7(0,-1,1) 8(0,0,-1) 9(0,0,0) 10(0,0,1) 11(0,1,-1)
//       12(0,1,0) 13(0,1,1) 14(1,-1,0) 15(1,0,-1) 16(1,0,0) 17(1,0,1) 18(1,1,0)
// with opp(q) = 18 - q and weights w0 = 1/3 (q=9), w1 = 1/18 (one nonzero
// component), w2 = 1/36 (two nonzero components).
//
// Device layout (one lattice, in place, AA pattern):
//   f[q * Np + n], n = (i*ny + j)*nz + k over the interior nodes (no halo),
//   Np = n_nodes rounded up to a multiple of 128.  Two step kinds alternate:
//   "P" (pull-push) gathers f_q from A[opp(q)][x - c_q] and scatters f*_q to
//   A[q][x + c_q]; "L" (local) reads A[q][x] and writes f*_q to A[opp(q)][x].
//   Before a P step the array holds post-collision populations in reversed
//   slots (A[opp(q)][x] = f*_q(x)); after it, the streamed populations
//   (A[q][x] = incoming f_q(x)).
#pragma once
#include <stdint.h>
#include <cmath>
#include <cuda_runtime.h>

namespace jlb {

constexpr int Q = 19;

// node-mask bits (uint32 per node)
constexpr uint32_t MASK_LINKS = 0x7FFFFu;      // bit q: link q bounces back
constexpr uint32_t MASK_SPECIAL = 1u << 30;    // handled by the boundary-node path
constexpr uint32_t MASK_SOLID = 1u << 31;      // not a fluid node
constexpr uint32_t MASK_SKIP = MASK_SPECIAL | MASK_SOLID;

// node classes (uint8 per node); the dense sweep reads the 32-bit mask only
// for CLS_WALL nodes
constexpr uint8_t CLS_PLAIN = 0;   // fluid, no bounce-back link
constexpr uint8_t CLS_WALL = 1;    // fluid with bounce-back links
constexpr uint8_t CLS_SPECIAL = 2; // boundary-node path
constexpr uint8_t CLS_SOLID = 3;   // not a fluid node

// boundary-node info bits
constexpr uint32_t SP_LADD_SHIFT = 0;  // bits 0..18: link has a moving-wall term
constexpr uint32_t SP_FACE_SHIFT = 20; // bits 20..25: node lies on fixed face f

enum Precision { PREC_FP64 = 0, PREC_FP32 = 1, PREC_FP16 = 2 };
enum Scheme { SCH_BGK = 0, SCH_TRT = 1, SCH_REG = 2 };
enum Bc { BC_WALL = 0, BC_PERIODIC = 1, BC_FIXED_DEN = 2, BC_FIXED_VEL = 3, BC_SYMMETRIC = 4 };

// Unsigned 32-bit division by a divisor fixed at launch, as a multiply-high
// and two shifts (Granlund & Montgomery, "Division by invariant integers
// using multiplication", PLDI 1994, unsigned case with N = 32): for
// l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, s1 = min(l, 1),
// s2 = max(l - 1, 0) and t = mulhi(m, n), n / d = (t + ((n - t) >> s1)) >> s2
// for every n < 2^32.
struct UDiv {
    uint32_t m, s1, s2;
};

inline UDiv make_udiv(uint32_t d) {
    uint32_t l = 0;
    while (l < 32 && ((uint64_t)1 << l) < d) ++l;
    UDiv u;
    u.m = (uint32_t)((((uint64_t)1 << 32) * (((uint64_t)1 << l) - d)) / d + 1);
    u.s1 = l < 1 ? l : 1;
    u.s2 = l > 1 ? l - 1 : 0;
    return u;
}

// Relaxation rates for the FP32 / FP16-storage kernels: the nearest values
// to (we, wo) on a grid 2^-p, with p as fine as the FP32 operations of the
// collision allow exactly (1 - we, we + wo, we - wo, 1 - (we + wo)/2, and
// (we - wo)/2).  With those exact, the relaxation passes mass and momentum
// through with unbiased rounding only; rounded coefficients would bias them
// by ~1e-8 of their value at every step.  scheme_trt = false uses we alone.
inline bool f32_exact(double x) { return (double)(float)x == x; }
inline void float_exact_rates(bool scheme_trt, double we, double wo, double &wef, double &wof) {
    for (int p = 40; p >= 16; --p) {
        const double q = std::ldexp(1.0, p);
        const double a = std::nearbyint(we * q) / q;
        const double b = scheme_trt ? std::nearbyint(wo * q) / q : a;
        if (a <= 0.0 || b <= 0.0) continue;
        bool ok = f32_exact(a) && f32_exact(b) && f32_exact(1.0 - a);
        if (scheme_trt)
            ok = ok && f32_exact(a + b) && f32_exact(a - b) && f32_exact(1.0 - 0.5 * (a + b)) &&
                 f32_exact(0.5 * (a - b));
        if (ok) { wef = a; wof = b; return; }
    }
    wef = (double)(float)we;  // not reached for rates in (0, 2)
    wof = (double)(float)wo;
}

#ifdef __CUDACC__
__device__ __forceinline__ uint32_t udiv(uint32_t n, UDiv d) {
    const uint32_t t = __umulhi(n, d.m);
    return (t + ((n - t) >> d.s1)) >> d.s2;
}
#endif

struct StepArgs {
    void *f;              // populations, 19 * Np elements of the storage type
    int64_t Np;           // slot stride
    int nx, ny, nz;
    const uint32_t *nmask;
    const uint8_t *ncls;  // per-node class: CLS_* below (1 byte read per node)
    void *den, *ux, *uy, *uz; // moments (compute type); den holds rho-1 for shifted storage
    const void *acc;      // optional acceleration field, 3 * Np (compute type), SoA
    double g[3];          // uniform gravity
    double w_e, w_o;      // relaxation rates 1/tau (even / odd)
    float gf[3];          // g, w_e and w_o rounded to float once by the host:
    float w_ef, w_of;     // the float kernels read these (a per-thread double
                          // conversion runs on the narrow FP64 pipe)
    int write_moments;
    // dense-node grid
    int bx, by, kblocks;  // block shape and k-blocks per row-block
    int nb_dense;         // number of dense blocks; the rest are boundary blocks
    int b0;               // first dense block of this launch (a launch may cover a slab)
    int pf;               // L2 prefetch distance in dense blocks (0: none): block b
                          // prefetches the rows block b + pf will read
    // linear mapping, used when nz is not a multiple of 32 (a warp along k
    // alone would leave lanes idle): dense block b takes the sites
    // [128 b, 128 b + 128) of n = (i*ny + j)*nz + k, with blocks of (128, 1)
    int lin;
    uint32_t nsite;       // nx*ny*nz (lin only; below 2^32)
    UDiv div_nz, div_ny;  // division by nz (lin only) and by ny
    // fluid-only ("sparse") population layout, used on lattices with many
    // solid sites: populations f[q * Npc + m] over the fluid sites m only
    const int32_t *csite; // [Nc] lattice site n of fluid site m
    const int32_t *cidx;  // [N] fluid index m of lattice site n (-1: solid)
    int64_t Nc, Npc;      // fluid sites, their slot stride (multiple of 128)
    float inv_syz, inv_nz; // 1/(ny*nz), 1/nz for the site -> (i,j,k) split; 0: use integer division
    const int64_t *sp_cnode; // [M] fluid index of each boundary node (sparse layout), else NULL
    // boundary (special) nodes
    int M;                // number of boundary nodes
    const int64_t *sp_node;
    const uint32_t *sp_info;
    const int64_t *sp_rd; // [19][M] P-step read element index
    const int64_t *sp_wr; // [19][M] P-step write element index
    const double *sp_lw;  // [19][M] c_q . u_wall of moving links
    const double *sp_bc;  // [8][M] Zou-He data (den, ux, uy, uz) x 2 faces
    void *sp_den;         // [M] previous-step density (compute type; rho-1 if shifted)
    int bc[6];            // face kinds (for the Zou-He variant)
    void *fout;           // if set: the step writes its outputs here instead of
                          // back into f (same element indices; adjoint recompute)
    void *sp_tee;         // if set: collision inputs (after Zou-He) of the
                          // boundary nodes, [19][M] in the storage type
};

// Blocks of the boundary-node path in a launch of the direct step kernel (or
// the adjoint's reverse kernel), whose blocks have a.bx * a.by threads: 96
// when nz = 96 (row blocks of one 96-site row), 128 otherwise.  The staged and
// fluid-only kernels use 128-thread blocks.
inline int special_blocks(const StepArgs &a) {
    const int T = a.bx * a.by;
    return (a.M + T - 1) / T;
}

// options of the C++-executable collision model (lbm_cxx.cu)
constexpr int CXX_LINEAR_EQ = 1; // linear ("Stokes") equilibrium instead of the quadratic one
constexpr int CXX_FORCE2 = 2;    // second-order forcing term instead of the first-order one

// launch entry points, one per precision translation unit
// grid: `blocks` blocks of (a.bx, a.by) threads; returns a cudaError_t value
int launch_step_fp64(const StepArgs &a, int scheme, bool pstep, bool accf, int blocks, cudaStream_t st);
// FP64 with contracted, regrouped arithmetic (lbm_fp64fast.cu)
int launch_step_fp64fast(const StepArgs &a, int scheme, bool pstep, bool accf, int blocks, cudaStream_t st);
int launch_step_fp32(const StepArgs &a, int scheme, bool pstep, bool accf, int blocks, cudaStream_t st);
int launch_step_fp16(const StepArgs &a, int scheme, bool pstep, bool accf, int blocks, cudaStream_t st);
// the same step on the fluid-only layout (a.csite/a.cidx set): blocks of 128
// fluid sites, then the boundary-node blocks
int launch_step_sparse_fp32(const StepArgs &a, int scheme, bool pstep, bool accf, int blocks, cudaStream_t st);
int launch_step_sparse_fp16(const StepArgs &a, int scheme, bool pstep, bool accf, int blocks, cudaStream_t st);
// the C++-executable collision model (lbm_cxx.cu), FP64; opts: CXX_* flags
int launch_step_cxx(const StepArgs &a, int scheme, int opts, bool pstep, bool accf, int blocks, cudaStream_t st);
// bulk-copy staged variants (lbm_step_tma.cuh): persistent grid over
// `ntiles` row tiles of 128 sites, then `nsb` boundary-node blocks; a
// timed-out mbarrier wait sets *err
int launch_step_tma_fp32(const StepArgs &a, int scheme, bool pstep, bool accf, int grid, int ntiles, int nsb,
                         int *err, cudaStream_t st);
int launch_step_tma_fp16(const StepArgs &a, int scheme, bool pstep, bool accf, int grid, int ntiles, int nsb,
                         int *err, cudaStream_t st);
int tma_blocks_per_sm_fp32(int scheme);
// FP16 storage, staged local step with two sites per thread (256-site tiles,
// nz a multiple of 256; kb2 = nz / 256 tiles per row)
int launch_step_tma_h2_fp16(const StepArgs &a, int scheme, bool accf, int grid, int ntiles, int kb2, int nsb,
                            int *err, cudaStream_t st);
int tma_h2_blocks_per_sm_fp16(int scheme);
int tma_blocks_per_sm_fp16(int scheme);

} // namespace jlb
