// lbm_step_tma.cuh -- the fused step with bulk-copy (TMA) staging of the
// population rows.
//
// Same physics and AA addressing as lbm_step.cuh, organised for memory-level
// parallelism: a persistent grid walks "tiles" (TW consecutive k of one
// (i,j) row).  For each tile one elected thread issues 19 cp.async.bulk
// copies (one per population slot) from HBM into shared memory, completing
// on an mbarrier, while the block computes the previous tile from the other
// buffer.  Loads therefore occupy shared memory instead of registers, and a
// block keeps a whole tile (~10 KB for FP32) in flight.
//
// Pull-push (P) step: slot q of the tile is read from row (i - c_x, j - c_y)
// (periodic wrap in i/j) over the window [k0 - PAD, k0 + TW + PAD) clipped to
// the row, so the k +/- 1 shift of a population is a fixed offset into the
// staged row.  Lanes whose source wraps in k, or whose link bounces back,
// read global memory directly.  Stores go straight from registers.
// Local (L) step: slot q is staged from the tile's own row.
//
// Requirements checked by the host: nz a multiple of PAD (16-byte aligned
// rows and copy sizes), 19 * Np < 2^31.  Waits on the mbarrier are bounded;
// a timeout sets *err and the block stops.
#pragma once
#include "lbm_step.cuh"

namespace jlb {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// bounded wait: ~1e8 polls (seconds) before giving up
constexpr uint32_t TMA_WAIT_LIMIT = 1u << 27;

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
    for (uint32_t it = 0; it < TMA_WAIT_LIMIT; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

template <class S> struct TmaGeom {
    static constexpr int TW = 128;                    // sites per tile (= threads)
    static constexpr int PAD = 16 / (int)sizeof(S);   // elements per 16 bytes
    static constexpr int SEG = TW + 2 * PAD;          // staged elements per slot
    static constexpr int STAGE = Q * SEG;             // elements per buffer
};

// Issues the 19 copies of tile `tile` into buffer `buf` (one thread).
template <class S, bool PSTEP>
__device__ __forceinline__ void tma_issue(const StepArgs &a, int tile, S *buf, uint64_t *bar) {
    using G = TmaGeom<S>;
    const int row = tile / a.kblocks;
    const int k0 = (tile - row * a.kblocks) * G::TW;
    const int i = row / a.ny, j = row - (row / a.ny) * a.ny;
    const S *f = (const S *)a.f;
    uint32_t bytes = 0;
    // window of staged k in the row, clipped to [0, nz)
    const int lo = PSTEP ? max(0, k0 - G::PAD) : k0;
    const int hi = PSTEP ? min(a.nz, k0 + G::TW + G::PAD) : min(a.nz, k0 + G::TW);
    const uint32_t nb = (uint32_t)(hi - lo) * (uint32_t)sizeof(S);
    const int off = lo - (k0 - G::PAD); // staged element of k is k - (k0 - PAD)
    int64_t rowbase[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        int si = i, sj = j, slot = q;
        if (PSTEP) {
            si = i - CX(q); si = si < 0 ? a.nx - 1 : (si >= a.nx ? 0 : si);
            sj = j - CY(q); sj = sj < 0 ? a.ny - 1 : (sj >= a.ny ? 0 : sj);
            slot = OPP(q);
        }
        rowbase[q] = (int64_t)slot * a.Np + ((int64_t)si * a.ny + sj) * a.nz;
        bytes += nb;
    }
    mbar_arrive_tx(bar, bytes);
#pragma unroll
    for (int q = 0; q < Q; ++q) bulk_g2s(buf + q * G::SEG + off, f + rowbase[q] + lo, nb, bar);
}

template <class ST, class PH, bool PSTEP, bool ACCF>
__global__ void __launch_bounds__(128, JLB_MIN_BLOCKS_TMA) lbm_step_tma_kernel(const StepArgs a, int ntiles,
                                                                            int nspecial_blocks, int *err) {
    using S = typename ST::S;
    using C = typename ST::C;
    using G = TmaGeom<S>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    S *buf0 = (S *)smem_raw;
    S *buf1 = buf0 + G::STAGE;
    __shared__ __align__(8) uint64_t bar[2];
    const int t = threadIdx.x;
    if (t == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();

    S *__restrict__ f = (S *)a.f;
    const int32_t Np = (int32_t)a.Np;
    int tile = blockIdx.x;
    int it = 0;
    if (tile < ntiles && t == 0) tma_issue<S, PSTEP>(a, tile, buf0, &bar[0]);
    for (; tile < ntiles; tile += gridDim.x, ++it) {
        S *cur = (it & 1) ? buf1 : buf0;
        const int next = tile + gridDim.x;
        if (next < ntiles && t == 0) {
            fence_proxy_async_smem();
            tma_issue<S, PSTEP>(a, next, (it & 1) ? buf0 : buf1, &bar[(it + 1) & 1]);
        }
        const int row = tile / a.kblocks;
        const int k0 = (tile - row * a.kblocks) * G::TW;
        const int k = k0 + t;
        const int32_t n = row * a.nz + k;
        uint8_t cls = CLS_SOLID;
        uint32_t m = 0;
        if (k < a.nz) {
            cls = __ldg(a.ncls + n);
            if (PSTEP && cls == CLS_WALL) m = __ldg(a.nmask + n);
        }
        // every thread polls; the block leaves together if any poll timed out
        const bool ok = mbar_wait_bounded(&bar[it & 1], (uint32_t)(it >> 1) & 1u);
        if (__syncthreads_or(!ok)) {
            if (t == 0) {
                atomicExch(err, 1);
                // let the copies this block already issued land before
                // leaving: those of this tile (bounded again) and of the next
                (void)mbar_wait_bounded(&bar[it & 1], (uint32_t)(it >> 1) & 1u);
                if (next < ntiles) (void)mbar_wait_bounded(&bar[(it + 1) & 1], (uint32_t)((it + 1) >> 1) & 1u);
            }
            __syncthreads();
            return;
        }
        if (cls < CLS_SPECIAL) {
            const int i = row / a.ny, j = row - (row / a.ny) * a.ny;
            C fv[Q];
            int32_t dI[3], dJ[3], dK[3];
            if (PSTEP) {
                const int32_t sI = a.ny * a.nz, sJ = a.nz;
                dI[0] = (i == 0 ? (a.nx - 1) : -1) * sI; dI[1] = 0; dI[2] = (i + 1 == a.nx ? (1 - a.nx) : 1) * sI;
                dJ[0] = (j == 0 ? (a.ny - 1) : -1) * sJ; dJ[1] = 0; dJ[2] = (j + 1 == a.ny ? (1 - a.ny) : 1) * sJ;
                dK[0] = k == 0 ? (a.nz - 1) : -1; dK[1] = 0; dK[2] = k + 1 == a.nz ? (1 - a.nz) : 1;
            }
            // every lane takes its value from the staged rows (the index stays
            // inside the slot's segment even where it is not the right value)
            Unroll<0, Q>::run([&]<int q>() {
                constexpr int sh = (PSTEP && q != 9) ? CZ(q) : 0;
                fv[q] = bulk_ldv<ST, PH, q>(cur[q * G::SEG + G::PAD + t - sh]);
            });
            // rare lanes fix theirs up from global memory: links that bounce
            // back read their own opposite slot; sources that wrap in k
            // (periodic) lie outside the staged window
            if (PSTEP && (m != 0u || k == 0 || k == a.nz - 1)) {
                Unroll<0, Q>::run([&]<int q>() {
                    if (q == 9) return;
                    const int kk = k - CZ(q);
                    if (m & (1u << q)) {
                        fv[q] = bulk_ld<ST, PH, q>(f + ((int32_t)q * Np + n));
                    } else if (kk < 0 || kk >= a.nz) {
                        const int32_t src = n + dI[1 - CX(q)] + dJ[1 - CY(q)] + dK[1 - CZ(q)];
                        fv[q] = bulk_ld<ST, PH, q>(f + ((int32_t)OPP(q) * Np + src));
                    }
                });
            }
            C ax, ay, az;
            if (ACCF) {
                const C *acc = (const C *)a.acc;
                ax = arg_g<C>(a, 0) + __ldg(acc + n);
                ay = arg_g<C>(a, 1) + __ldg(acc + Np + n);
                az = arg_g<C>(a, 2) + __ldg(acc + 2 * Np + n);
            } else {
                ax = arg_g<C>(a, 0); ay = arg_g<C>(a, 1); az = arg_g<C>(a, 2);
            }
            C ux, uy, uz;
            const C rho = bulk_collide<ST, PH>(fv, ax, ay, az, arg_we<C>(a), arg_wo<C>(a), ux, uy, uz);
            Unroll<0, Q>::run([&]<int q>() {
                if (!PSTEP) {
                    bulk_st<ST, PH, OPP(q)>(f + ((int32_t)OPP(q) * Np + n), fv[q]);
                    return;
                }
                int32_t e;
                if (q == 9) {
                    e = 9 * Np + n;
                } else {
                    const int32_t dst = n + dI[1 + CX(q)] + dJ[1 + CY(q)] + dK[1 + CZ(q)];
                    e = (m & (1u << OPP(q))) ? ((int32_t)OPP(q) * Np + n) : ((int32_t)q * Np + dst);
                }
                bulk_st<ST, PH, q>(f + e, fv[q]);
            });
            if (a.write_moments) {
                ((C *)a.den)[n] = rho;
                ((C *)a.ux)[n] = ux;
                ((C *)a.uy)[n] = uy;
                ((C *)a.uz)[n] = uz;
            }
        }
        __syncthreads(); // buffer `cur` is free for the copies issued next round
    }
    // boundary nodes after the tiles
    for (int sb = blockIdx.x; sb < nspecial_blocks; sb += gridDim.x) special_node<ST, PH, PSTEP, ACCF>(a, sb);
}

// ---------------------------------------------------------------------------
// FP16 storage, local step, two consecutive sites per thread.  One 2-byte
// population per load keeps only half the bytes in flight per register that
// FP32 does; here each thread takes sites (k, k+1) of a 256-site tile, reads
// each population of both as one aligned 32-bit word from the staged rows,
// collides site k and then site k+1 on the stored values (PhysH16), and
// writes both results of a population with one 32-bit store (one
// cvt.rn.f16x2.f32 for the pair).  A site that is a boundary node or solid
// keeps its half: the other half goes out as a 16-bit store.  The rows are
// staged as in lbm_step_tma_kernel (19 copies of 512 bytes per tile, two
// buffers, bounded mbarrier waits).  Requires nz a multiple of 256.
// ---------------------------------------------------------------------------
struct H2Geom {
    static constexpr int TW = 256;          // sites per tile (2 per thread)
    static constexpr int PAD = 8;           // 16 bytes of halves
    static constexpr int SEG = TW + 2 * PAD; // staged halves per slot
    static constexpr int STAGE = Q * SEG;   // halves per buffer
};
#ifndef JLB_MIN_BLOCKS_H2
#define JLB_MIN_BLOCKS_H2 6
#endif

__device__ __forceinline__ void h2_issue(const StepArgs &a, int tile, int kb2, __half *buf, uint64_t *bar) {
    using G = H2Geom;
    const int row = tile / kb2;
    const int k0 = (tile - row * kb2) * G::TW;
    const __half *f = (const __half *)a.f;
    constexpr uint32_t nb = G::TW * 2;
    mbar_arrive_tx(bar, nb * (uint32_t)Q);
    const int64_t base = (int64_t)row * a.nz + k0;
#pragma unroll
    for (int q = 0; q < Q; ++q) bulk_g2s(buf + q * G::SEG + G::PAD, f + (int64_t)q * a.Np + base, nb, bar);
}

__device__ __forceinline__ void st_h16(__half *p, float v) {
    *p = __float2half_rn(v);
}

template <class PH, bool ACCF>
__global__ void __launch_bounds__(128, JLB_MIN_BLOCKS_H2) lbm_step_tma_h2_kernel(const StepArgs a, int ntiles, int kb2,
                                                                              int nspecial_blocks, int *err) {
    using G = H2Geom;
    using C = float;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __half *buf0 = (__half *)smem_raw;
    __half *buf1 = buf0 + G::STAGE;
    __shared__ __align__(8) uint64_t bar[2];
    const int t = threadIdx.x;
    if (t == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    __half *__restrict__ f = (__half *)a.f;
    const int32_t Np = (int32_t)a.Np;
    int tile = blockIdx.x;
    int it = 0;
    if (tile < ntiles && t == 0) h2_issue(a, tile, kb2, buf0, &bar[0]);
    for (; tile < ntiles; tile += gridDim.x, ++it) {
        const __half *cur = (it & 1) ? buf1 : buf0;
        const int next = tile + gridDim.x;
        if (next < ntiles && t == 0) {
            fence_proxy_async_smem();
            h2_issue(a, next, kb2, (it & 1) ? buf0 : buf1, &bar[(it + 1) & 1]);
        }
        const int row = tile / kb2;
        const int kA = (tile - row * kb2) * G::TW + 2 * t;
        const int32_t nA = row * a.nz + kA;
        // class bytes of both sites in one 16-bit load (nA is even)
        const uint32_t cl = __ldg((const unsigned short *)(a.ncls + nA));
        const bool actA = (cl & 0xFFu) < CLS_SPECIAL, actB = (cl >> 8) < CLS_SPECIAL;
        const bool ok = mbar_wait_bounded(&bar[it & 1], (uint32_t)(it >> 1) & 1u);
        if (__syncthreads_or(!ok)) {
            if (t == 0) {
                atomicExch(err, 1);
                (void)mbar_wait_bounded(&bar[it & 1], (uint32_t)(it >> 1) & 1u);
                if (next < ntiles) (void)mbar_wait_bounded(&bar[(it + 1) & 1], (uint32_t)((it + 1) >> 1) & 1u);
            }
            __syncthreads();
            return;
        }
        if (actA || actB) {
            uint32_t w[Q];
            Unroll<0, Q>::run([&]<int q>() { w[q] = *(const uint32_t *)(cur + q * G::SEG + G::PAD + 2 * t); });
            C axA, ayA, azA, axB, ayB, azB;
            if (ACCF) {
                const C *acc = (const C *)a.acc;
                axA = arg_g<C>(a, 0) + __ldg(acc + nA); axB = arg_g<C>(a, 0) + __ldg(acc + nA + 1);
                ayA = arg_g<C>(a, 1) + __ldg(acc + Np + nA); ayB = arg_g<C>(a, 1) + __ldg(acc + Np + nA + 1);
                azA = arg_g<C>(a, 2) + __ldg(acc + 2 * Np + nA); azB = arg_g<C>(a, 2) + __ldg(acc + 2 * Np + nA + 1);
            } else {
                axA = axB = arg_g<C>(a, 0); ayA = ayB = arg_g<C>(a, 1); azA = azB = arg_g<C>(a, 2);
            }
            C hA[Q], hB[Q];
            Unroll<0, Q>::run([&]<int q>() { hA[q] = __low2float(*(const __half2 *)&w[q]); });
            C uxA, uyA, uzA;
            const C rhoA = PH::collide_h(hA, axA, ayA, azA, arg_we<C>(a), arg_wo<C>(a), uxA, uyA, uzA);
            Unroll<0, Q>::run([&]<int q>() { hB[q] = __high2float(*(const __half2 *)&w[q]); });
            C uxB, uyB, uzB;
            const C rhoB = PH::collide_h(hB, axB, ayB, azB, arg_we<C>(a), arg_wo<C>(a), uxB, uyB, uzB);
            // local step: population q of both sites goes to slot opp(q)
            Unroll<0, Q>::run([&]<int q>() {
                __half *p = f + ((int32_t)OPP(q) * Np + nA);
                if (actA && actB) *(__half2 *)p = __floats2half2_rn(hA[q], hB[q]);
                else if (actA) st_h16(p, hA[q]);
                else st_h16(p + 1, hB[q]);
            });
            if (a.write_moments) {
                C *den = (C *)a.den, *ux = (C *)a.ux, *uy = (C *)a.uy, *uz = (C *)a.uz;
                if (actA) { den[nA] = rhoA; ux[nA] = uxA; uy[nA] = uyA; uz[nA] = uzA; }
                if (actB) { den[nA + 1] = rhoB; ux[nA + 1] = uxB; uy[nA + 1] = uyB; uz[nA + 1] = uzB; }
            }
        }
        __syncthreads(); // buffer `cur` is free for the copies issued next round
    }
    for (int sb = blockIdx.x; sb < nspecial_blocks; sb += gridDim.x) special_node<StoreF16, PH, false, ACCF>(a, sb);
}

template <template <int> class PH>
int launch_step_tma_h2_impl(const StepArgs &a, int scheme, bool accf, int grid, int ntiles, int kb2,
                            int nspecial_blocks, int *err, cudaStream_t st) {
    const size_t smem = 2 * (size_t)H2Geom::STAGE * sizeof(__half);
#define JLB_H(SCH, A) lbm_step_tma_h2_kernel<PH<SCH>, A><<<grid, 128, smem, st>>>(a, ntiles, kb2, nspecial_blocks, err)
#define JLB_HS(SCH) if (accf) JLB_H(SCH, true); else JLB_H(SCH, false);
    if (scheme == SCH_BGK) { JLB_HS(SCH_BGK) }
    else if (scheme == SCH_TRT) { JLB_HS(SCH_TRT) }
    else { JLB_HS(SCH_REG) }
#undef JLB_HS
#undef JLB_H
    return (int)cudaGetLastError();
}

template <template <int> class PH> int tma_h2_blocks_per_sm(int scheme) {
    const size_t smem = 2 * (size_t)H2Geom::STAGE * sizeof(__half);
    int nb = 0;
    cudaError_t e;
    if (scheme == SCH_BGK) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, lbm_step_tma_h2_kernel<PH<SCH_BGK>, false>, 128, smem);
    else if (scheme == SCH_TRT) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, lbm_step_tma_h2_kernel<PH<SCH_TRT>, false>, 128, smem);
    else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, lbm_step_tma_h2_kernel<PH<SCH_REG>, false>, 128, smem);
    return e == cudaSuccess ? nb : 0;
}

template <class ST, template <int> class PH>
int launch_step_tma_impl(const StepArgs &a, int scheme, bool pstep, bool accf, int grid, int ntiles,
                         int nspecial_blocks, int *err, cudaStream_t st) {
    using G = TmaGeom<typename ST::S>;
    const size_t smem = 2 * (size_t)G::STAGE * sizeof(typename ST::S);
    static_assert(2 * G::STAGE * sizeof(typename ST::S) <= 48 * 1024, "staging must fit the default smem limit");
#define JLB_T(SCH, P, A) lbm_step_tma_kernel<ST, PH<SCH>, P, A><<<grid, 128, smem, st>>>(a, ntiles, nspecial_blocks, err)
#define JLB_TS(SCH)                                                                                      \
    if (pstep) { if (accf) JLB_T(SCH, true, true); else JLB_T(SCH, true, false); }                       \
    else { if (accf) JLB_T(SCH, false, true); else JLB_T(SCH, false, false); }
    if (scheme == SCH_BGK) { JLB_TS(SCH_BGK) }
    else if (scheme == SCH_TRT) { JLB_TS(SCH_TRT) }
    else { JLB_TS(SCH_REG) }
#undef JLB_TS
#undef JLB_T
    return (int)cudaGetLastError();
}

} // namespace jlb
