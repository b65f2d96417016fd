// lbm_aux.cu -- set-up, read-out and reduction kernels around the time step:
//   * initial populations (jyulb/isothermal.pyx:958-1105), FP64 with the
//     reference's arithmetic (this unit is compiled with -fmad=false);
//   * post-collision population read-out / restore for any AA parity;
//   * moment download straight into mapped host arrays;
//   * acceleration-field upload;
//   * FP64 mass / momentum reductions (two passes, deterministic order).
#include <algorithm>

#include "lbm_aux.h"
#include "lbm_step.cuh"

namespace jlb {

__device__ __forceinline__ int64_t full_idx(const AuxGeom &g, int I, int J, int K) {
    return ((int64_t)I * g.NJ + J) * g.NK + K;
}

// ---------------------------------------------------------------------------
// initial populations
// ---------------------------------------------------------------------------
__device__ void init_project(const double *h, double *f) {
    const double c = 1.0 / 72.0;
    double exy = 2.0 * h[0] + 6.0 * h[4] + 6.0 * h[7] - 3.0 * h[9];
    double a0 = exy + 18.0 * h[5], o0 = -6.0 * h[1] - 6.0 * h[2];
    double a4 = exy - 18.0 * h[5], o4 = -6.0 * h[1] + 6.0 * h[2];
    double exz = 2.0 * h[0] + 6.0 * h[4] - 3.0 * h[7] + 6.0 * h[9];
    double a1 = exz + 18.0 * h[6], o1 = -6.0 * h[1] - 6.0 * h[3];
    double a3 = exz - 18.0 * h[6], o3 = -6.0 * h[1] + 6.0 * h[3];
    double eyz = 2.0 * h[0] - 3.0 * h[4] + 6.0 * h[7] + 6.0 * h[9];
    double a5 = eyz + 18.0 * h[8], o5 = -6.0 * h[2] - 6.0 * h[3];
    double a7 = eyz - 18.0 * h[8], o7 = -6.0 * h[2] + 6.0 * h[3];
    double ex = 4.0 * h[0] + 12.0 * h[4] - 6.0 * h[7] - 6.0 * h[9];
    double ey = 4.0 * h[0] - 6.0 * h[4] + 12.0 * h[7] - 6.0 * h[9];
    double ez = 4.0 * h[0] - 6.0 * h[4] - 6.0 * h[7] + 12.0 * h[9];
    f[0] = c * (a0 + o0);  f[18] = c * (a0 - o0);
    f[1] = c * (a1 + o1);  f[17] = c * (a1 - o1);
    f[2] = c * (ex - 12.0 * h[1]); f[16] = c * (ex + 12.0 * h[1]);
    f[3] = c * (a3 + o3);  f[15] = c * (a3 - o3);
    f[4] = c * (a4 + o4);  f[14] = c * (a4 - o4);
    f[5] = c * (a5 + o5);  f[13] = c * (a5 - o5);
    f[6] = c * (ey - 12.0 * h[2]); f[12] = c * (ey + 12.0 * h[2]);
    f[7] = c * (a7 + o7);  f[11] = c * (a7 - o7);
    f[8] = c * (ez - 12.0 * h[3]); f[10] = c * (ez + 12.0 * h[3]);
    f[9] = (1.0 / 3.0) * h[0] - 0.5 * (h[4] + h[7] + h[9]);
}

// finite-difference velocity gradient along the face normal direction dir
// (jyulb/isothermal.pyx:958-1023)
__device__ void init_der_vel(const AuxGeom &g, const uint8_t *phase, const double *vel, int I, int J, int K,
                             int dir, const double *v, double *dv) {
    // lattice vectors with +1 along dir, in the reference's FDIR order
    const int L[3][5] = {{14, 15, 16, 17, 18}, {4, 11, 12, 13, 18}, {3, 7, 10, 13, 17}};
    dv[0] = 0.0; dv[1] = 0.0; dv[2] = 0.0;
#pragma unroll
    for (int m = 0; m < 5; ++m) {
        const int l = L[dir][m];
        const int cx = l < 5 ? -1 : (l >= 14 ? 1 : 0);
        const int cy = (l == 0 || l == 5 || l == 6 || l == 7 || l == 14) ? -1
                     : (l == 4 || l == 11 || l == 12 || l == 13 || l == 18) ? 1 : 0;
        const int cz = (l == 1 || l == 5 || l == 8 || l == 11 || l == 15) ? -1
                     : (l == 3 || l == 7 || l == 10 || l == 13 || l == 17) ? 1 : 0;
        const int64_t nn = full_idx(g, I + cx, J + cy, K + cz);
        const int64_t no = full_idx(g, I - cx, J - cy, K - cz);
        double c1 = 0.5, c2 = 0.0, c3 = -0.5;
        if (phase[nn] == 0) {
            if (phase[no] == 0) { c1 = 1.0; c3 = -1.0; }
            else { c1 = 4.0 / 3.0; c2 = -1.0; c3 = -1.0 / 3.0; }
        } else if (phase[no] == 0) {
            c1 = 1.0 / 3.0; c2 = 1.0; c3 = -4.0 / 3.0;
        }
        const double w = (l == 16 || l == 12 || l == 10) ? (2.0 / 36.0) : (1.0 / 36.0);
        const double c0 = 2.0 * w * 3.0;
#pragma unroll
        for (int d = 0; d < 3; ++d)
            dv[d] = dv[d] + c0 * (c1 * vel[3 * nn + d] + c2 * v[d] + c3 * vel[3 * no + d]);
    }
}

template <class ST>
__global__ void init_kernel(AuxGeom g, const uint8_t *phase, const double *den, const double *vel, double w_e,
                            typename ST::S *f, typename ST::C *mden, typename ST::C *mux,
                            typename ST::C *muy, typename ST::C *muz) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const int i = (int)(n / ((int64_t)g.ny * g.nz));
    const int rem = (int)(n - (int64_t)i * g.ny * g.nz);
    const int j = rem / g.nz, k = rem - (rem / g.nz) * g.nz;
    const int I = i + 1, J = j + 1, K = k + 1;
    const int64_t fn = full_idx(g, I, J, K);
    if (phase[fn] == 0) return;
    const double d = den[fn];
    const double v[3] = {vel[3 * fn], vel[3 * fn + 1], vel[3 * fn + 2]};
    double h[10], dx[3], dy[3], dz[3], fq[Q];
    {
        double jx = d * v[0], jy = d * v[1], jz = d * v[2];
        h[0] = d; h[1] = jx; h[2] = jy; h[3] = jz;
        h[4] = jx * v[0]; h[5] = jx * v[1]; h[6] = jx * v[2];
        h[7] = jy * v[1]; h[8] = jy * v[2]; h[9] = jz * v[2];
    }
    init_der_vel(g, phase, vel, I, J, K, 0, v, dx);
    init_der_vel(g, phase, vel, I, J, K, 1, v, dy);
    init_der_vel(g, phase, vel, I, J, K, 2, v, dz);
    const double tau = 1.0 / w_e, rc = 1.0 - w_e;
    const double m2 = -2.0 * tau * (1.0 / 3.0) * d;
    h[4] = h[4] + rc * m2 * dx[0];
    h[5] = h[5] + rc * m2 * 0.5 * (dx[1] + dy[0]);
    h[6] = h[6] + rc * m2 * 0.5 * (dx[2] + dz[0]);
    h[7] = h[7] + rc * m2 * dy[1];
    h[8] = h[8] + rc * m2 * 0.5 * (dy[2] + dz[1]);
    h[9] = h[9] + rc * m2 * dz[2];
    init_project(h, fq);
    // post-collision state: A[opp(q)][x] = f_q(x)
    Unroll<0, Q>::run([&]<int q>() {
        typename ST::C val;
        if (ST::shifted) {
            constexpr double w = WCLASS(q) == 0 ? (12.0 / 36.0) : WCLASS(q) == 1 ? (2.0 / 36.0) : (1.0 / 36.0);
            val = (typename ST::C)(fq[q] - w);
        } else {
            val = (typename ST::C)fq[q];
        }
        ST::template st<OPP(q)>(f + OPP(q) * g.Np + n, val);
    });
    mden[n] = ST::shifted ? (typename ST::C)(d - 1.0) : (typename ST::C)d;
    mux[n] = (typename ST::C)v[0];
    muy[n] = (typename ST::C)v[1];
    muz[n] = (typename ST::C)v[2];
}

// ---------------------------------------------------------------------------
// population read-out / restore
// ---------------------------------------------------------------------------
template <class ST>
__device__ __forceinline__ double dec_pop(typename ST::C v, double w) {
    return ST::shifted ? (double)v + w : (double)v;
}

// post-collision population f*_q(x) for dense nodes, any parity
template <class ST>
__global__ void readout_dense_kernel(AuxGeom g, const typename ST::S *f, const uint32_t *nmask, int parity,
                                     double *out) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const uint32_t m = nmask[n];
    if (m & MASK_SOLID) {
#pragma unroll
        for (int q = 0; q < Q; ++q) out[(int64_t)q * g.N + n] = 0.0;
        return;
    }
    if (m & MASK_SPECIAL) return;
    const int i = (int)(n / ((int64_t)g.ny * g.nz));
    const int rem = (int)(n - (int64_t)i * g.ny * g.nz);
    const int j = rem / g.nz, k = rem - (rem / g.nz) * g.nz;
    Unroll<0, Q>::run([&]<int q>() {
        constexpr double w = WCLASS(q) == 0 ? (12.0 / 36.0) : WCLASS(q) == 1 ? (2.0 / 36.0) : (1.0 / 36.0);
        int64_t addr;
        if (parity == 0 || q == 9) {
            addr = (int64_t)OPP(q) * g.Np + n;
        } else if (m & (1u << OPP(q))) {
            addr = (int64_t)OPP(q) * g.Np + n;
        } else {
            int ii = i + CX(q), jj = j + CY(q), kk = k + CZ(q);
            ii = ii < 0 ? g.nx - 1 : (ii >= g.nx ? 0 : ii);
            jj = jj < 0 ? g.ny - 1 : (jj >= g.ny ? 0 : jj);
            kk = kk < 0 ? g.nz - 1 : (kk >= g.nz ? 0 : kk);
            addr = (int64_t)q * g.Np + ((int64_t)ii * g.ny + jj) * g.nz + kk;
        }
        out[(int64_t)q * g.N + n] = dec_pop<ST>(ST::template ld<q>(f + addr), w);
    });
}

template <class ST>
__global__ void readout_special_kernel(AuxGeom g, const typename ST::S *f, int M, const int64_t *sp_node,
                                       const int64_t *sp_wr, int parity, double *out) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= M) return;
    const int64_t n = sp_node[t];
    Unroll<0, Q>::run([&]<int q>() {
        constexpr double w = WCLASS(q) == 0 ? (12.0 / 36.0) : WCLASS(q) == 1 ? (2.0 / 36.0) : (1.0 / 36.0);
        const int64_t addr = parity == 0 ? (int64_t)OPP(q) * g.Np + n : sp_wr[(int64_t)q * M + t];
        out[(int64_t)q * g.N + n] = dec_pop<ST>(ST::template ld<q>(f + addr), w);
    });
}

// restore: writes the post-collision state A[opp(q)][x] = f_q(x)
template <class ST>
__global__ void restore_kernel(AuxGeom g, typename ST::S *f, const uint32_t *nmask, const double *in) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    if (nmask[n] & MASK_SOLID) return;
    Unroll<0, Q>::run([&]<int q>() {
        constexpr double w = WCLASS(q) == 0 ? (12.0 / 36.0) : WCLASS(q) == 1 ? (2.0 / 36.0) : (1.0 / 36.0);
        const double v = in[(int64_t)q * g.N + n];
        ST::template st<OPP(q)>(f + OPP(q) * g.Np + n,
                                (typename ST::C)(ST::shifted ? v - w : v));
    });
}

// ---------------------------------------------------------------------------
// moments -> host arrays (mapped memory), acceleration upload
// ---------------------------------------------------------------------------
// One block per chunk of DL_TILE sites of a k-row.  The (NI,NJ,NK,3) velocity
// layout is assembled in shared memory first so that every warp store to the
// host covers 256 contiguous bytes: NVLink-C2C writes run ~3.5x faster that
// way than with one strided 8-byte store per component.  Solid sites keep
// their host values (the caller's wall velocities).
constexpr int DL_TILE = 256;

template <class C, bool SHIFTED>
__global__ void __launch_bounds__(DL_TILE) download_kernel(AuxGeom g, int kchunks, const uint32_t *nmask,
                                                           const C *den, const C *ux, const C *uy, const C *uz,
                                                           double *hden, double *hvel, int64_t row0) {
    __shared__ double sv[3 * DL_TILE];
    __shared__ unsigned char sfl[DL_TILE];
    const int64_t rowc = blockIdx.x + row0 * kchunks;
    const int64_t row = rowc / kchunks;
    const int k0 = (int)(rowc - row * kchunks) * DL_TILE;
    const int i = (int)(row / g.ny), j = (int)(row - (int64_t)i * g.ny);
    const int cnt = min(DL_TILE, g.nz - k0);
    const int t = threadIdx.x;
    const int64_t n = row * g.nz + k0 + t;
    const int64_t fn0 = full_idx(g, i + 1, j + 1, k0 + 1);
    bool fl = false;
    if (t < cnt) {
        fl = !(nmask[n] & MASK_SOLID);
        if (fl) {
            hden[fn0 + t] = SHIFTED ? 1.0 + (double)den[n] : (double)den[n];
            sv[3 * t] = (double)ux[n];
            sv[3 * t + 1] = (double)uy[n];
            sv[3 * t + 2] = (double)uz[n];
        }
        sfl[t] = fl;
    }
    __syncthreads();
    double *hv = hvel + 3 * fn0;
    for (int w = t; w < 3 * cnt; w += DL_TILE)
        if (sfl[w / 3]) hv[w] = sv[w];
}

template <class C>
__global__ void acc_upload_kernel(AuxGeom g, const double *hacc, C *acc) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const int i = (int)(n / ((int64_t)g.ny * g.nz));
    const int rem = (int)(n - (int64_t)i * g.ny * g.nz);
    const int j = rem / g.nz, k = rem - (rem / g.nz) * g.nz;
    const int64_t fn = full_idx(g, i + 1, j + 1, k + 1);
    acc[n] = (C)hacc[3 * fn];
    acc[g.Np + n] = (C)hacc[3 * fn + 1];
    acc[2 * g.Np + n] = (C)hacc[3 * fn + 2];
}

// ---------------------------------------------------------------------------
// reductions: per-block partial sums in FP64, then one block adds the
// partials in index order (the result does not depend on scheduling)
// ---------------------------------------------------------------------------
constexpr int RED_THREADS = 256;

template <class C, bool SHIFTED>
__global__ void __launch_bounds__(RED_THREADS) reduce_partial_kernel(AuxGeom g, const uint32_t *nmask,
                                                                     const C *den, const C *ux, const C *uy,
                                                                     const C *uz, double *partial) {
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < g.N;
         n += (int64_t)gridDim.x * blockDim.x) {
        if (nmask[n] & MASK_SOLID) continue;
        const double d = SHIFTED ? 1.0 + (double)den[n] : (double)den[n];
        const double u0 = (double)ux[n], u1 = (double)uy[n], u2 = (double)uz[n];
        acc[0] += d;
        acc[1] += d * u0; acc[2] += d * u1; acc[3] += d * u2;
        acc[4] += u0; acc[5] += u1; acc[6] += u2;
        if (!isfinite(d) || !isfinite(u0) || !isfinite(u1) || !isfinite(u2)) acc[7] += 1.0;
    }
    __shared__ double sm[8][RED_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        double v = acc[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sm[c][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        double v = 0.0;
        for (int w = 0; w < RED_THREADS / 32; ++w) v += sm[threadIdx.x][w];
        partial[(int64_t)blockIdx.x * 8 + threadIdx.x] = v;
    }
}

__global__ void reduce_final_kernel(const double *partial, int nblocks, double *out) {
    // one warp per component; lanes stride over the partials, then a fixed
    // shuffle tree
    const int c = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (c >= 8) return;
    double v = 0.0;
    for (int b = lane; b < nblocks; b += 32) v += partial[(int64_t)b * 8 + c];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) out[c] = v;
}

// steady-state convergence residual: over fluid sites, FP64 sums of
// |u - u_prev|^2 (slot 0) and |u|^2 (slot 1) against the velocity kept at
// the previous call, which the same pass replaces by the current one;
// reduce_final_kernel combines the per-block partials (8 slots per block)
template <class C>
__global__ void __launch_bounds__(RED_THREADS) residual_partial_kernel(AuxGeom g, const uint32_t *nmask,
                                                                       const C *ux, const C *uy, const C *uz,
                                                                       C *prev, double *partial) {
    double d2 = 0.0, u2 = 0.0;
    for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < g.N;
         n += (int64_t)gridDim.x * blockDim.x) {
        if (nmask[n] & MASK_SOLID) continue;
        const C v[3] = {ux[n], uy[n], uz[n]};
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double u = (double)v[c], d = u - (double)prev[c * g.Np + n];
            d2 += d * d;
            u2 += u * u;
            prev[c * g.Np + n] = v[c];
        }
    }
    __shared__ double sm[2][RED_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        d2 += __shfl_down_sync(0xffffffffu, d2, o);
        u2 += __shfl_down_sync(0xffffffffu, u2, o);
    }
    if (lane == 0) { sm[0][wid] = d2; sm[1][wid] = u2; }
    __syncthreads();
    if (threadIdx.x < 8) {
        double v = 0.0;
        if (threadIdx.x < 2)
            for (int w = 0; w < RED_THREADS / 32; ++w) v += sm[threadIdx.x][w];
        partial[(int64_t)blockIdx.x * 8 + threadIdx.x] = v;
    }
}

// ---------------------------------------------------------------------------
// flow information (the C++ executable's IsothermalSolver::calc_flow_info,
// include/solver/solver.cpp:64-129): over fluid sites, sums of den, j = den u,
// |j| = den |u|, u and |u|, and the extremes max den, min den, max |u|.  The
// extremes start from the reference density and 0 as there.  Per-block
// partials, then one block combines them in index order.
// partial layout per block: [0..8] sums (den, jx, jy, jz, |j|, ux, uy, uz,
// |u|), [9] max den, [10] min den, [11] max |u|
// ---------------------------------------------------------------------------
constexpr int FI_VALUES = 12;

template <class C, bool SHIFTED>
__global__ void __launch_bounds__(RED_THREADS) flowinfo_partial_kernel(AuxGeom g, const uint32_t *nmask,
                                                                       const C *den, const C *ux, const C *uy,
                                                                       const C *uz, double ref_den,
                                                                       double *partial) {
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    double dmax = ref_den, dmin = ref_den, umax = 0.0;
    for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < g.N;
         n += (int64_t)gridDim.x * blockDim.x) {
        if (nmask[n] & MASK_SOLID) continue;
        const double d = SHIFTED ? 1.0 + (double)den[n] : (double)den[n];
        const double u0 = (double)ux[n], u1 = (double)uy[n], u2 = (double)uz[n];
        const double um = sqrt(u0 * u0 + u1 * u1 + u2 * u2);
        acc[0] += d;
        acc[1] += d * u0; acc[2] += d * u1; acc[3] += d * u2;
        acc[4] += d * um;
        acc[5] += u0; acc[6] += u1; acc[7] += u2;
        acc[8] += um;
        dmax = fmax(dmax, d);
        dmin = fmin(dmin, d);
        umax = fmax(umax, um);
    }
    __shared__ double sm[FI_VALUES][RED_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int c = 0; c < 9; ++c) {
        double v = acc[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sm[c][wid] = v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dmax = fmax(dmax, __shfl_down_sync(0xffffffffu, dmax, o));
        dmin = fmin(dmin, __shfl_down_sync(0xffffffffu, dmin, o));
        umax = fmax(umax, __shfl_down_sync(0xffffffffu, umax, o));
    }
    if (lane == 0) { sm[9][wid] = dmax; sm[10][wid] = dmin; sm[11][wid] = umax; }
    __syncthreads();
    if (threadIdx.x < FI_VALUES) {
        const int c = threadIdx.x;
        double v = sm[c][0];
        for (int w = 1; w < RED_THREADS / 32; ++w) {
            const double x = sm[c][w];
            v = c < 9 ? v + x : (c == 10 ? fmin(v, x) : fmax(v, x));
        }
        partial[(int64_t)blockIdx.x * FI_VALUES + c] = v;
    }
}

__global__ void flowinfo_final_kernel(const double *partial, int nblocks, double *out) {
    const int c = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (c >= FI_VALUES) return;
    const bool is_sum = c < 9, is_min = c == 10;
    double v = is_sum ? 0.0 : partial[c];
    for (int b = lane; b < nblocks; b += 32) {
        const double x = partial[(int64_t)b * FI_VALUES + c];
        v = is_sum ? v + x : (is_min ? fmin(v, x) : fmax(v, x));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double x = __shfl_down_sync(0xffffffffu, v, o);
        v = is_sum ? v + x : (is_min ? fmin(v, x) : fmax(v, x));
    }
    if (lane == 0) out[c] = v;
}

// ---------------------------------------------------------------------------
// fluid-only population layout: gather / scatter of the 19 slots of every
// fluid site between the lattice layout (stride Np) and the fluid-only one
// (stride Npc), and translation of the boundary-node element tables
// ---------------------------------------------------------------------------
template <class T>
__global__ void sparse_pack_kernel(T *dense, T *comp, const int32_t *csite, int64_t Nc, int64_t Np,
                                   int64_t Npc, int to_comp) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= Nc) return;
    const int64_t n = csite[m];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        if (to_comp) comp[q * Npc + m] = dense[q * Np + n];
        else dense[q * Np + n] = comp[q * Npc + m];
    }
}

__global__ void sparse_tables_kernel(const int64_t *rd, const int64_t *wr, const int64_t *node, int M,
                                     const int32_t *cidx, int64_t Np, int64_t Npc, int64_t *rdc, int64_t *wrc,
                                     int64_t *nodec) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e < (int64_t)Q * M) {
        const int64_t r = rd[e], w = wr[e];
        rdc[e] = (r / Np) * Npc + cidx[r % Np];
        wrc[e] = (w / Np) * Npc + cidx[w % Np];
    }
    if (e < M) nodec[e] = cidx[node[e]];
}

// velocities of the solid positions next to fluid (halo-padded host vel,
// read in place) against their values at the last classification: *flag
// becomes 1 when any component differs (a NaN counts as a change)
__global__ void wall_check_kernel(const int64_t *pos, const double *known, int64_t nwall, const double *vel,
                                  int *flag) {
    for (int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; w < nwall;
         w += (int64_t)gridDim.x * blockDim.x) {
        const double *u = vel + 3 * pos[w];
        if (u[0] != known[3 * w] || u[1] != known[3 * w + 1] || u[2] != known[3 * w + 2]) *flag = 1;
    }
}

// per-call data of the boundary nodes read in place from the halo-padded
// host den/vel: the node's density (Ladd's term; FP32 storage keeps rho - 1)
// and the Zou-He (den, vel) of each fixed face it lies on; faces outside
// refresh_mask keep den = 1, vel = 0
__global__ void fill_dynamic_kernel(AuxGeom g, int M, const int64_t *sp_node, const uint32_t *sp_info,
                                    unsigned refresh_mask, int f64, const double *den, const double *vel,
                                    double *bc, void *dbuf) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= M) return;
    const int64_t n = sp_node[t];
    const int64_t syz = (int64_t)g.ny * g.nz;
    const int i = (int)(n / syz);
    const int j = (int)((n / g.nz) % g.ny);
    const int k = (int)(n % g.nz);
    const int64_t fn = ((int64_t)(i + 1) * g.NJ + (j + 1)) * g.NK + (k + 1);
    if (f64) ((double *)dbuf)[t] = den[fn];
    else ((float *)dbuf)[t] = (float)(den[fn] - 1.0);
    const uint32_t faces = (sp_info[t] >> SP_FACE_SHIFT) & 0x3Fu;
    int slot = 0;
    for (int face = 0; face < 6 && faces; ++face) {
        if (!(faces & (1u << face))) continue;
        double d = 1.0, u0 = 0.0, u1 = 0.0, u2 = 0.0;
        if (refresh_mask & (1u << face)) { d = den[fn]; u0 = vel[3 * fn]; u1 = vel[3 * fn + 1]; u2 = vel[3 * fn + 2]; }
        bc[(size_t)(4 * slot) * M + t] = d;
        bc[(size_t)(4 * slot + 1) * M + t] = u0;
        bc[(size_t)(4 * slot + 2) * M + t] = u1;
        bc[(size_t)(4 * slot + 3) * M + t] = u2;
        slot = 1;
    }
}

// ---------------------------------------------------------------------------
// host-callable launchers
// ---------------------------------------------------------------------------
static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

int aux_init(int prec, const AuxGeom &g, const uint8_t *phase, const double *den, const double *vel, double w_e,
             void *f, void *mden, void *mux, void *muy, void *muz, cudaStream_t st) {
    const unsigned b = nblk(g.N, 128);
    if (prec == PREC_FP64)
        init_kernel<StoreF64><<<b, 128, 0, st>>>(g, phase, den, vel, w_e, (double *)f, (double *)mden,
                                                 (double *)mux, (double *)muy, (double *)muz);
    else if (prec == PREC_FP32)
        init_kernel<StoreF32><<<b, 128, 0, st>>>(g, phase, den, vel, w_e, (float *)f, (float *)mden,
                                                 (float *)mux, (float *)muy, (float *)muz);
    else
        init_kernel<StoreF16><<<b, 128, 0, st>>>(g, phase, den, vel, w_e, (__half *)f, (float *)mden,
                                                 (float *)mux, (float *)muy, (float *)muz);
    return (int)cudaGetLastError();
}

int aux_readout(int prec, const AuxGeom &g, const void *f, const uint32_t *nmask, int parity, int M,
                const int64_t *sp_node, const int64_t *sp_wr, double *out, cudaStream_t st) {
    const unsigned b = nblk(g.N, 128), bs = nblk(M, 128);
#define JLB_RO(ST, T)                                                                                   \
    readout_dense_kernel<ST><<<b, 128, 0, st>>>(g, (const T *)f, nmask, parity, out);                  \
    if (M > 0) readout_special_kernel<ST><<<bs, 128, 0, st>>>(g, (const T *)f, M, sp_node, sp_wr, parity, out);
    if (prec == PREC_FP64) { JLB_RO(StoreF64, double) }
    else if (prec == PREC_FP32) { JLB_RO(StoreF32, float) }
    else { JLB_RO(StoreF16, __half) }
#undef JLB_RO
    return (int)cudaGetLastError();
}

int aux_restore(int prec, const AuxGeom &g, void *f, const uint32_t *nmask, const double *in, cudaStream_t st) {
    const unsigned b = nblk(g.N, 128);
    if (prec == PREC_FP64) restore_kernel<StoreF64><<<b, 128, 0, st>>>(g, (double *)f, nmask, in);
    else if (prec == PREC_FP32) restore_kernel<StoreF32><<<b, 128, 0, st>>>(g, (float *)f, nmask, in);
    else restore_kernel<StoreF16><<<b, 128, 0, st>>>(g, (__half *)f, nmask, in);
    return (int)cudaGetLastError();
}

int aux_sparse_pack(int elem_bytes, void *dense, void *comp, const int32_t *csite, int64_t Nc, int64_t Np,
                    int64_t Npc, int to_comp, cudaStream_t st) {
    const unsigned b = nblk(Nc, 256);
    if (b == 0) return 0;
    if (elem_bytes == 8)
        sparse_pack_kernel<uint64_t><<<b, 256, 0, st>>>((uint64_t *)dense, (uint64_t *)comp, csite, Nc, Np, Npc, to_comp);
    else if (elem_bytes == 4)
        sparse_pack_kernel<uint32_t><<<b, 256, 0, st>>>((uint32_t *)dense, (uint32_t *)comp, csite, Nc, Np, Npc, to_comp);
    else
        sparse_pack_kernel<uint16_t><<<b, 256, 0, st>>>((uint16_t *)dense, (uint16_t *)comp, csite, Nc, Np, Npc, to_comp);
    return (int)cudaGetLastError();
}

int aux_wall_check(const int64_t *pos, const double *known, int64_t nwall, const double *vel, int *flag,
                   cudaStream_t st) {
    if (nwall <= 0) return 0;
    const unsigned b = (unsigned)std::min<int64_t>(nblk(nwall, 256), 4096);
    wall_check_kernel<<<b, 256, 0, st>>>(pos, known, nwall, vel, flag);
    return (int)cudaGetLastError();
}

int aux_fill_dynamic(const AuxGeom &g, int M, const int64_t *sp_node, const uint32_t *sp_info, unsigned refresh_mask,
                     int f64, const double *den, const double *vel, double *bc, void *dbuf, cudaStream_t st) {
    if (M <= 0) return 0;
    fill_dynamic_kernel<<<nblk(M, 128), 128, 0, st>>>(g, M, sp_node, sp_info, refresh_mask, f64, den, vel, bc, dbuf);
    return (int)cudaGetLastError();
}

int aux_sparse_tables(const int64_t *rd, const int64_t *wr, const int64_t *node, int M, const int32_t *cidx,
                      int64_t Np, int64_t Npc, int64_t *rdc, int64_t *wrc, int64_t *nodec, cudaStream_t st) {
    if (M <= 0) return 0;
    sparse_tables_kernel<<<nblk((int64_t)Q * M, 256), 256, 0, st>>>(rd, wr, node, M, cidx, Np, Npc, rdc, wrc, nodec);
    return (int)cudaGetLastError();
}

int aux_download_rows(int prec, const AuxGeom &g, const uint32_t *nmask, const void *den, const void *ux,
                      const void *uy, const void *uz, double *hden, double *hvel, int64_t row0, int64_t nrows,
                      cudaStream_t st) {
    const int kchunks = (g.nz + DL_TILE - 1) / DL_TILE;
    const unsigned b = (unsigned)(nrows * kchunks);
    if (b == 0) return 0;
    if (prec == PREC_FP64)
        download_kernel<double, false><<<b, DL_TILE, 0, st>>>(g, kchunks, nmask, (const double *)den,
                                                              (const double *)ux, (const double *)uy,
                                                              (const double *)uz, hden, hvel, row0);
    else
        download_kernel<float, true><<<b, DL_TILE, 0, st>>>(g, kchunks, nmask, (const float *)den,
                                                            (const float *)ux, (const float *)uy,
                                                            (const float *)uz, hden, hvel, row0);
    return (int)cudaGetLastError();
}

// FP64 den / vel of the fluid sites on the first and last interior layers of
// the axes in `axes` (bit 0 x, 1 y, 2 z), written into the halo-padded host
// arrays; one thread per site, the others return at once
template <class C, bool SHIFTED>
__global__ void __launch_bounds__(256) layers_kernel(AuxGeom g, unsigned axes, const uint32_t *nmask, const C *den,
                                                    const C *ux, const C *uy, const C *uz, double *hden,
                                                    double *hvel) {
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const int64_t syz = (int64_t)g.ny * g.nz;
    const int i = (int)(n / syz);
    const int64_t r = n - (int64_t)i * syz;
    const int j = (int)(r / g.nz), k = (int)(r - (int64_t)j * g.nz);
    const bool on = ((axes & 1u) && (i == 0 || i == g.nx - 1)) || ((axes & 2u) && (j == 0 || j == g.ny - 1)) ||
                    ((axes & 4u) && (k == 0 || k == g.nz - 1));
    if (!on || (nmask[n] & MASK_SOLID)) return;
    const int64_t fn = full_idx(g, i + 1, j + 1, k + 1);
    hden[fn] = SHIFTED ? 1.0 + (double)den[n] : (double)den[n];
    hvel[3 * fn] = (double)ux[n];
    hvel[3 * fn + 1] = (double)uy[n];
    hvel[3 * fn + 2] = (double)uz[n];
}

int aux_download_layers(int prec, const AuxGeom &g, unsigned axes, const uint32_t *nmask, const void *den,
                        const void *ux, const void *uy, const void *uz, double *hden, double *hvel, cudaStream_t st) {
    const unsigned b = nblk(g.N, 256);
    if (prec == PREC_FP64)
        layers_kernel<double, false><<<b, 256, 0, st>>>(g, axes, nmask, (const double *)den, (const double *)ux,
                                                        (const double *)uy, (const double *)uz, hden, hvel);
    else
        layers_kernel<float, true><<<b, 256, 0, st>>>(g, axes, nmask, (const float *)den, (const float *)ux,
                                                      (const float *)uy, (const float *)uz, hden, hvel);
    return (int)cudaGetLastError();
}

int aux_download(int prec, const AuxGeom &g, const uint32_t *nmask, const void *den, const void *ux,
                 const void *uy, const void *uz, double *hden, double *hvel, cudaStream_t st) {
    return aux_download_rows(prec, g, nmask, den, ux, uy, uz, hden, hvel, 0, (int64_t)g.nx * g.ny, st);
}

int aux_acc_upload(int prec, const AuxGeom &g, const double *hacc, void *acc, cudaStream_t st) {
    const unsigned b = nblk(g.N, 256);
    if (prec == PREC_FP64) acc_upload_kernel<double><<<b, 256, 0, st>>>(g, hacc, (double *)acc);
    else acc_upload_kernel<float><<<b, 256, 0, st>>>(g, hacc, (float *)acc);
    return (int)cudaGetLastError();
}

int aux_reduce_blocks(int64_t N) {
    int64_t b = (N + RED_THREADS - 1) / RED_THREADS;
    return (int)(b < 1216 ? (b < 1 ? 1 : b) : 1216); // 8 blocks per SM on 152 SMs
}

int aux_reduce(int prec, const AuxGeom &g, const uint32_t *nmask, const void *den, const void *ux,
               const void *uy, const void *uz, double *partial, int nblocks, double *out, cudaStream_t st) {
    if (prec == PREC_FP64)
        reduce_partial_kernel<double, false><<<nblocks, RED_THREADS, 0, st>>>(
            g, nmask, (const double *)den, (const double *)ux, (const double *)uy, (const double *)uz, partial);
    else
        reduce_partial_kernel<float, true><<<nblocks, RED_THREADS, 0, st>>>(
            g, nmask, (const float *)den, (const float *)ux, (const float *)uy, (const float *)uz, partial);
    reduce_final_kernel<<<1, 256, 0, st>>>(partial, nblocks, out);
    return (int)cudaGetLastError();
}

int aux_residual(int prec, const AuxGeom &g, const uint32_t *nmask, const void *ux, const void *uy,
                 const void *uz, void *prev, double *partial, int nblocks, double *out, cudaStream_t st) {
    if (prec == PREC_FP64)
        residual_partial_kernel<double><<<nblocks, RED_THREADS, 0, st>>>(
            g, nmask, (const double *)ux, (const double *)uy, (const double *)uz, (double *)prev, partial);
    else
        residual_partial_kernel<float><<<nblocks, RED_THREADS, 0, st>>>(
            g, nmask, (const float *)ux, (const float *)uy, (const float *)uz, (float *)prev, partial);
    reduce_final_kernel<<<1, 256, 0, st>>>(partial, nblocks, out);
    return (int)cudaGetLastError();
}

int aux_flow_info(int prec, const AuxGeom &g, const uint32_t *nmask, const void *den, const void *ux,
                  const void *uy, const void *uz, double ref_den, double *partial, int nblocks, double *out,
                  cudaStream_t st) {
    if (prec == PREC_FP64)
        flowinfo_partial_kernel<double, false><<<nblocks, RED_THREADS, 0, st>>>(
            g, nmask, (const double *)den, (const double *)ux, (const double *)uy, (const double *)uz, ref_den,
            partial);
    else
        flowinfo_partial_kernel<float, true><<<nblocks, RED_THREADS, 0, st>>>(
            g, nmask, (const float *)den, (const float *)ux, (const float *)uy, (const float *)uz, ref_den,
            partial);
    flowinfo_final_kernel<<<1, 32 * FI_VALUES, 0, st>>>(partial, nblocks, out);
    return (int)cudaGetLastError();
}

} // namespace jlb
