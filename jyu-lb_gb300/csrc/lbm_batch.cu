// lbm_batch.cu -- one launch advances many independent D3Q19 domains.
//
// The domains' nodes are packed into one index space (each domain starts at
// a multiple of 128), populations are stored SoA over that space in FP32 as
// f - w (the shifted storage of lbm_fp32.cu), and the launch walks a tile
// table: tile t covers BLOCK consecutive nodes of domain tile_dom[t].  Per
// domain the kernel reads its relaxation rates, body force, sizes (for the
// periodic wrap) and the velocity of its moving solids.  Supported
// boundaries are those of a channel ensemble: periodic faces, bounce-back
// walls and solids (node link masks), and Ladd's moving-wall term for solids
// that move with the domain's wall velocity.  The AA pair and the physics
// are the single-domain kernels' (lbm_step.cuh, lbm_shifted.cuh).
#include "lbm_batch.h"
#include "lbm_shifted.cuh"

namespace jlb {

// resident warps per SM asked of the register allocator: the P step is
// latency-bound, and 32 warps beat 24 on the 512-channel ensemble although
// the P step then spills a few registers
#ifndef JLB_BATCH_WARPS
#define JLB_BATCH_WARPS 32
#endif
// lane l of warp 0 prefetches lines l, l + 32, ... of the 19 population rows
// tile t reads (slot opp(q) at x - c_q in the pull-push step, slot q at x in
// the local step), clamped to the tile's domain; the periodic wrap is ignored
template <bool PSTEP, int BLOCK>
__device__ __forceinline__ void batch_prefetch(const BatchArgs &a, int t, int lane) {
    const BatchDomain &D = a.dom[__ldg(a.tile_dom + t)];
    const int32_t l0 = (t - D.first_tile) * BLOCK;
    const int32_t syz = D.ny * D.nz;
    constexpr int LPR = BLOCK * (int)sizeof(float) / 128 + 1; // 128-byte lines per row
#pragma unroll 1
    for (int idx = lane; idx < Q * LPR; idx += 32) {
        const int q = idx / LPR, line = idx - q * LPR;
        const int32_t dq = PSTEP ? CX(q) * syz + CY(q) * D.nz + CZ(q) : 0;
        int32_t e = l0 - dq - 1 + line * (128 / (int)sizeof(float));
        if (e < 0) e = 0;
        if (e >= D.n) continue;
        prefetch_line(a.fq[PSTEP ? OPP(q) : q] + D.off + e);
    }
}

// IDX32: every element index q * Np + n fits 32 unsigned bits (19 Np < 2^32),
// so an address is one select of two 32-bit indices and one widening
// multiply-add; otherwise each population row has its own 64-bit pointer
template <int SCH, bool PSTEP, int BLOCK, bool IDX32>
__global__ void __launch_bounds__(BLOCK, JLB_BATCH_WARPS * 32 / BLOCK)
    lbm_batch_kernel(const BatchArgs a) {
    using ST = StoreF32;
    using PH = PhysSh<SCH>;
    using C = float;
    const int t = (int)blockIdx.x;
    if (a.pf && threadIdx.x < 32 && t + a.pf < a.ntiles) batch_prefetch<PSTEP, BLOCK>(a, t + a.pf, (int)threadIdx.x);
    const int d = __ldg(a.tile_dom + t);
    const BatchDomain &D = a.dom[d];
    const int32_t l = (t - D.first_tile) * BLOCK + (int)threadIdx.x;
    if (l >= D.n) return;
    const int32_t n = D.off + l;
    const uint8_t cls = __ldg(a.ncls + n);
    if (cls >= BCLS_SOLID) return;
    // rows of 19 * Np exceed 2^31 elements for large ensembles; each row
    // itself is indexed by a 32-bit site
    const uint32_t m = (PSTEP && cls != BCLS_PLAIN) ? __ldg(a.nmask + n) : 0u;
    const uint32_t mv = (cls == BCLS_MOVING) ? __ldg(a.mmask + n) : 0u;
    C fv[Q];
    int32_t dI[3], dJ[3], dK[3];
    if (PSTEP) {
        const int32_t nx = D.nx, ny = D.ny, nz = D.nz, syz = ny * nz;
        int32_t i, j, k, r;
        if (D.n < (1 << 23)) {
            i = split_div(l, syz, D.inv_syz, r);
            j = split_div(r, nz, D.inv_nz, k);
        } else {
            i = l / syz; r = l - i * syz; j = r / nz; k = r - j * nz;
        }
        dI[0] = (i == 0 ? (nx - 1) : -1) * syz; dI[1] = 0; dI[2] = (i + 1 == nx ? (1 - nx) : 1) * syz;
        dJ[0] = (j == 0 ? (ny - 1) : -1) * nz; dJ[1] = 0; dJ[2] = (j + 1 == ny ? (1 - ny) : 1) * nz;
        dK[0] = k == 0 ? (nz - 1) : -1; dK[1] = 0; dK[2] = k + 1 == nz ? (1 - nz) : 1;
    }
    const uint32_t Npu = (uint32_t)a.Np;
    Unroll<0, Q>::run([&]<int q>() {
        const float *p;
        if constexpr (IDX32) {
            uint32_t e;
            if (!PSTEP || q == 9) {
                e = (uint32_t)q * Npu + (uint32_t)n;
            } else {
                const int32_t src = n + dI[1 - CX(q)] + dJ[1 - CY(q)] + dK[1 - CZ(q)];
                e = (m & (1u << q)) ? (uint32_t)q * Npu + (uint32_t)n : (uint32_t)OPP(q) * Npu + (uint32_t)src;
            }
            p = a.f + e;
        } else {
            if (!PSTEP || q == 9) {
                p = a.fq[q] + n;
            } else {
                const int32_t src = n + dI[1 - CX(q)] + dJ[1 - CY(q)] + dK[1 - CZ(q)];
                p = (m & (1u << q)) ? (a.fq[q] + n) : (a.fq[OPP(q)] + src);
            }
        }
        fv[q] = ST::template ld<q>(p);
    });
    if (mv) {
        // Ladd's term on links to moving solids: 6 w_q rho_prev (c_q . U)
        const float dprev = a.dprev[n];
        Unroll<0, Q>::run([&]<int q>() {
            if (q == 9 || !(mv & (1u << q))) return;
            constexpr int cx = CX(q), cy = CY(q), cz = CZ(q);
            const float s = (float)cx * D.uw[0] + (float)cy * D.uw[1] + (float)cz * D.uw[2];
            fv[q] = PH::template ladd<q>(fv[q], dprev, s);
        });
    }
    C ux, uy, uz;
    const C dd = PH::collide(fv, D.g[0], D.g[1], D.g[2], D.we, D.wo, ux, uy, uz);
    Unroll<0, Q>::run([&]<int q>() {
        float *p;
        if constexpr (IDX32) {
            uint32_t e;
            if (!PSTEP || q == 9) {
                e = (uint32_t)OPP(q) * Npu + (uint32_t)n;
            } else {
                const int32_t dst = n + dI[1 + CX(q)] + dJ[1 + CY(q)] + dK[1 + CZ(q)];
                e = (m & (1u << OPP(q))) ? (uint32_t)OPP(q) * Npu + (uint32_t)n : (uint32_t)q * Npu + (uint32_t)dst;
            }
            p = a.f + e;
        } else {
            if (!PSTEP) {
                p = a.fq[OPP(q)] + n;
            } else if (q == 9) {
                p = a.fq[9] + n;
            } else {
                const int32_t dst = n + dI[1 + CX(q)] + dJ[1 + CY(q)] + dK[1 + CZ(q)];
                p = (m & (1u << OPP(q))) ? (a.fq[OPP(q)] + n) : (a.fq[q] + dst);
            }
        }
        ST::template st<q>(p, fv[q]);
    });
    if (mv) a.dprev[n] = dd;
    if (a.write_moments) {
        a.den[n] = dd;
        a.ux[n] = ux;
        a.uy[n] = uy;
        a.uz[n] = uz;
    }
}

int launch_batch_step(const BatchArgs &a, int scheme, bool pstep, int block, int ntiles, cudaStream_t st) {
    const bool idx32 = 19 * a.Np < (int64_t(1) << 32);
#define JLB_B(SCH, P, B)                                                                 \
    if (idx32) lbm_batch_kernel<SCH, P, B, true><<<ntiles, B, 0, st>>>(a);               \
    else lbm_batch_kernel<SCH, P, B, false><<<ntiles, B, 0, st>>>(a)
#define JLB_BB(SCH, B) if (pstep) JLB_B(SCH, true, B); else JLB_B(SCH, false, B);
#define JLB_BS(SCH)                               \
    if (block == 64) { JLB_BB(SCH, 64) }          \
    else if (block == 256) { JLB_BB(SCH, 256) }   \
    else { JLB_BB(SCH, 128) }
    if (scheme == SCH_BGK) { JLB_BS(SCH_BGK) }
    else if (scheme == SCH_TRT) { JLB_BS(SCH_TRT) }
    else { JLB_BS(SCH_REG) }
#undef JLB_BS
#undef JLB_BB
#undef JLB_B
    return (int)cudaGetLastError();
}

// Boundary nodes: the single-domain boundary-node step with the relaxation
// rates, body force and face kinds of each node's domain.
template <int SCH, bool PSTEP>
__global__ void __launch_bounds__(128) lbm_batch_special_kernel(const BatchArgs a) {
    const int t = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t >= a.Msp) return;
    const BatchDomain &D = a.dom[__ldg(a.sp_dom + t)];
    StepArgs s{};
    s.f = a.f;
    s.Np = a.Np;
    s.M = a.Msp;
    s.sp_node = a.sp_node;
    s.sp_info = a.sp_info;
    s.sp_rd = a.sp_rd;
    s.sp_wr = a.sp_wr;
    s.sp_lw = a.sp_lw;
    s.sp_bc = a.sp_bc;
    s.sp_den = a.sp_den;
    s.den = a.den; s.ux = a.ux; s.uy = a.uy; s.uz = a.uz;
    s.write_moments = a.write_moments;
    s.w_e = D.we;
    s.w_o = D.wo;
    s.w_ef = D.we;
    s.w_of = D.wo;
    for (int c = 0; c < 3; ++c) {
        s.g[c] = D.g[c];
        s.gf[c] = D.g[c];
    }
    for (int f = 0; f < 6; ++f) s.bc[f] = D.bc[f];
    special_node<StoreF32, PhysSh<SCH>, PSTEP, false>(s, (int)blockIdx.x);
}

int launch_batch_special(const BatchArgs &a, int scheme, bool pstep, cudaStream_t st) {
    if (a.Msp <= 0) return 0;
    const unsigned blocks = (unsigned)((a.Msp + 127) / 128);
#define JLB_BS2(SCH) \
    if (pstep) lbm_batch_special_kernel<SCH, true><<<blocks, 128, 0, st>>>(a); \
    else lbm_batch_special_kernel<SCH, false><<<blocks, 128, 0, st>>>(a);
    if (scheme == SCH_BGK) { JLB_BS2(SCH_BGK) }
    else if (scheme == SCH_TRT) { JLB_BS2(SCH_TRT) }
    else { JLB_BS2(SCH_REG) }
#undef JLB_BS2
    return (int)cudaGetLastError();
}

// gathers one domain's initial populations (single-domain S_post layout,
// stride Np_d) into the packed array (stride Np)
__global__ void batch_pack_kernel(const float *src, int64_t Np_d, int32_t n_d, float *dst, int64_t Np,
                                  int32_t off) {
    const int32_t l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= n_d) return;
#pragma unroll
    for (int q = 0; q < Q; ++q) dst[(int64_t)q * Np + off + l] = src[(int64_t)q * Np_d + l];
}

int launch_batch_pack(const float *src, int64_t Np_d, int32_t n_d, float *dst, int64_t Np, int32_t off,
                      cudaStream_t st) {
    batch_pack_kernel<<<(n_d + 255) / 256, 256, 0, st>>>(src, Np_d, n_d, dst, Np, off);
    return (int)cudaGetLastError();
}

// post-collision populations of one domain (any parity) as FP64 (19, n_d)
__global__ void batch_readout_kernel(BatchArgs a, int d, int parity, double *out) {
    const BatchDomain &D = a.dom[d];
    const int32_t l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= D.n) return;
    const int32_t n = D.off + l;
    const uint8_t cls = a.ncls[n];
    if (cls == BCLS_SOLID) {
        for (int q = 0; q < Q; ++q) out[(int64_t)q * D.n + l] = 0.0;
        return;
    }
    const uint32_t m = cls != BCLS_PLAIN ? a.nmask[n] : 0u;
    const int32_t syz = D.ny * D.nz;
    const int i = l / syz, r = l - (l / syz) * syz, j = r / D.nz, k = r - (r / D.nz) * D.nz;
    Unroll<0, Q>::run([&]<int q>() {
        constexpr double w = WCLASS(q) == 0 ? (12.0 / 36.0) : WCLASS(q) == 1 ? (2.0 / 36.0) : (1.0 / 36.0);
        int64_t e;
        if (parity == 0 || q == 9 || (m & (1u << OPP(q)))) {
            e = (int64_t)OPP(q) * a.Np + n;
        } else {
            int ii = i + CX(q), jj = j + CY(q), kk = k + CZ(q);
            ii = ii < 0 ? D.nx - 1 : (ii >= D.nx ? 0 : ii);
            jj = jj < 0 ? D.ny - 1 : (jj >= D.ny ? 0 : jj);
            kk = kk < 0 ? D.nz - 1 : (kk >= D.nz ? 0 : kk);
            e = (int64_t)q * a.Np + D.off + (ii * D.ny + jj) * D.nz + kk;
        }
        out[(int64_t)q * D.n + l] = (double)a.f[e] + w;
    });
}

// boundary nodes [t0, t1) of domain d: their streamed slots come from the
// tables (mirrors and Zou-He faces), overwriting what the kernel above wrote
__global__ void batch_readout_special_kernel(BatchArgs a, int d, int t0, int t1, int parity, double *out) {
    const int t = t0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (t >= t1) return;
    const BatchDomain &D = a.dom[d];
    const int64_t n = a.sp_node[t];
    const int64_t l = n - D.off;
    Unroll<0, Q>::run([&]<int q>() {
        constexpr double w = WCLASS(q) == 0 ? (12.0 / 36.0) : WCLASS(q) == 1 ? (2.0 / 36.0) : (1.0 / 36.0);
        const int64_t e = parity == 0 ? (int64_t)OPP(q) * a.Np + n : a.sp_wr[(int64_t)q * a.Msp + t];
        out[(int64_t)q * D.n + l] = (double)a.f[e] + w;
    });
}

int launch_batch_readout(const BatchArgs &a, int d, int n_d, int parity, int t0, int t1, double *out,
                         cudaStream_t st) {
    batch_readout_kernel<<<(n_d + 255) / 256, 256, 0, st>>>(a, d, parity, out);
    if (t1 > t0) batch_readout_special_kernel<<<(t1 - t0 + 127) / 128, 128, 0, st>>>(a, d, t0, t1, parity, out);
    return (int)cudaGetLastError();
}

} // namespace jlb
