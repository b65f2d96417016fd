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
                ax = (C)a.g[0] + __ldg(acc + n);
                ay = (C)a.g[1] + __ldg(acc + Np + n);
                az = (C)a.g[2] + __ldg(acc + 2 * Np + n);
            } else {
                ax = (C)a.g[0]; ay = (C)a.g[1]; az = (C)a.g[2];
            }
            C ux, uy, uz;
            const C rho = bulk_collide<ST, PH>(fv, ax, ay, az, (C)a.w_e, (C)a.w_o, ux, uy, uz);
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
