// lbm_aux.h -- host-callable launchers of the set-up / read-out / reduction
// kernels (lbm_aux.cu).  All return a cudaError_t value.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace jlb {

struct AuxGeom {
    int nx, ny, nz;       // interior sizes
    int NI, NJ, NK;       // halo-padded sizes of the host arrays
    int64_t N, Np;        // interior node count, population slot stride
};

// initial populations from halo-padded phase/den/vel (device-accessible)
int aux_init(int prec, const AuxGeom &g, const uint8_t *phase, const double *den, const double *vel, double w_e,
             void *f, void *mden, void *mux, void *muy, void *muz, cudaStream_t st);
// post-collision populations, FP64 (19, N); parity 0: post-collision slots,
// 1: streamed slots
int aux_readout(int prec, const AuxGeom &g, const void *f, const uint32_t *nmask, int parity, int M,
                const int64_t *sp_node, const int64_t *sp_wr, double *out, cudaStream_t st);
int aux_restore(int prec, const AuxGeom &g, void *f, const uint32_t *nmask, const double *in, cudaStream_t st);
// moments of fluid nodes into device-accessible halo-padded host arrays
// fluid-only layout: copies the 19 slots of each fluid site between the
// lattice layout (stride Np) and the fluid-only one (stride Npc); to_comp
// selects the direction
int aux_sparse_pack(int elem_bytes, void *dense, void *comp, const int32_t *csite, int64_t Nc, int64_t Np,
                    int64_t Npc, int to_comp, cudaStream_t st);
// boundary-node element tables (q * Np + n) -> fluid-only (q * Npc + m)
int aux_sparse_tables(const int64_t *rd, const int64_t *wr, const int64_t *node, int M, const int32_t *cidx,
                      int64_t Np, int64_t Npc, int64_t *rdc, int64_t *wrc, int64_t *nodec, cudaStream_t st);
// *flag = 1 (device-accessible int) when vel (device-accessible halo-padded
// host array) differs from known (3 per position) at any of the nwall
// positions
int aux_wall_check(const int64_t *pos, const double *known, int64_t nwall, const double *vel, int *flag,
                   cudaStream_t st);
// boundary nodes' per-call density and Zou-He data from device-accessible
// halo-padded host den/vel (faces in refresh_mask are read, the others get
// den = 1, vel = 0); dbuf: double (f64) or float (rho - 1)
int aux_fill_dynamic(const AuxGeom &g, int M, const int64_t *sp_node, const uint32_t *sp_info, unsigned refresh_mask,
                     int f64, const double *den, const double *vel, double *bc, void *dbuf, cudaStream_t st);
// rows [row0, row0 + nrows) of (i, j) rows only
int aux_download_rows(int prec, const AuxGeom &g, const uint32_t *nmask, const void *den, const void *ux,
                      const void *uy, const void *uz, double *hden, double *hvel, int64_t row0, int64_t nrows,
                      cudaStream_t st);
int aux_download(int prec, const AuxGeom &g, const uint32_t *nmask, const void *den, const void *ux,
                 const void *uy, const void *uz, double *hden, double *hvel, cudaStream_t st);
// fluid sites of the first and last interior layers of the axes in `axes`
// (bit 0 x, 1 y, 2 z) only: the sources of the periodic / symmetric halo rules
int aux_download_layers(int prec, const AuxGeom &g, unsigned axes, const uint32_t *nmask, const void *den,
                        const void *ux, const void *uy, const void *uz, double *hden, double *hvel, cudaStream_t st);
// interior of a device-accessible halo-padded (NI,NJ,NK,3) array -> SoA field
int aux_acc_upload(int prec, const AuxGeom &g, const double *hacc, void *acc, cudaStream_t st);
// initial state of the C++-executable model (lbm_cxx.cu); facc: SoA force
// density field or NULL, gv: gravity, tau: relaxation time
int aux_init_cxx(const AuxGeom &g, int scheme, int opts, const uint8_t *phase, const double *den,
                 const double *vel, const double *facc, const double gv[3], double tau, double we, double wo,
                 double *f, double *mden, double *mux, double *muy, double *muz, cudaStream_t st);
int aux_reduce_blocks(int64_t N);
// partial must hold 8 * nblocks doubles; out 8 doubles (device)
int aux_reduce(int prec, const AuxGeom &g, const uint32_t *nmask, const void *den, const void *ux,
               const void *uy, const void *uz, double *partial, int nblocks, double *out, cudaStream_t st);
// convergence residual: out[0] = sum |u - prev|^2, out[1] = sum |u|^2 over
// fluid sites (FP64); prev (3 * Np, compute type) then holds u.  partial as
// for aux_reduce
int aux_residual(int prec, const AuxGeom &g, const uint32_t *nmask, const void *ux, const void *uy,
                 const void *uz, void *prev, double *partial, int nblocks, double *out, cudaStream_t st);
// flow information: partial must hold 12 * nblocks doubles; out 12 doubles
// (device): sums den, jx, jy, jz, |j|, ux, uy, uz, |u|; max den, min den, max |u|
int aux_flow_info(int prec, const AuxGeom &g, const uint32_t *nmask, const void *den, const void *ux,
                  const void *uy, const void *uz, double ref_den, double *partial, int nblocks, double *out,
                  cudaStream_t st);

} // namespace jlb
