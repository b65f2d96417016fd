// lbm_step.cuh -- the fused D3Q19 time step (stream + bounce-back + Zou-He +
// collide + moments) for one AA half-pair, generic over the storage policy
// and the collision physics.
//
// One launch per time step.  Blocks [0, nb_dense) sweep the lattice in
// (k-fastest) rows: every fluid node that is not a boundary node streams with
// plain neighbour arithmetic (periodic wrap for free) and halfway bounce-back
// from its 19-bit link mask.  Blocks [nb_dense, grid) handle the boundary
// nodes from a precomputed list: Zou-He faces, links that cross a symmetric
// face, and links to moving solids (Ladd's term), each with explicit per-link
// read/write element indices.  The two sets are disjoint and the AA pattern
// makes every slot written by exactly the node that reads it, so both halves
// run in one launch without synchronisation.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <type_traits>
#include "lbm_common.h"

namespace jlb {

// lattice tables as constexpr functions of q (resolved at compile time in the
// unrolled loops)
__host__ __device__ constexpr int CX(int q) { return q < 5 ? -1 : (q >= 14 ? 1 : 0); }
__host__ __device__ constexpr int CY(int q) {
    return (q == 0 || q == 5 || q == 6 || q == 7 || q == 14) ? -1
         : (q == 4 || q == 11 || q == 12 || q == 13 || q == 18) ? 1 : 0;
}
__host__ __device__ constexpr int CZ(int q) {
    return (q == 1 || q == 5 || q == 8 || q == 11 || q == 15) ? -1
         : (q == 3 || q == 7 || q == 10 || q == 13 || q == 17) ? 1 : 0;
}
__host__ __device__ constexpr int OPP(int q) { return 18 - q; }
__host__ __device__ constexpr int NNZ(int q) {
    return (CX(q) != 0) + (CY(q) != 0) + (CZ(q) != 0);
}
// weight class of q: 0 rest, 1 axis, 2 diagonal
__host__ __device__ constexpr int WCLASS(int q) { return NNZ(q); }

// ---------------------------------------------------------------------------
// storage policies
// ---------------------------------------------------------------------------
struct StoreF64 {
    using S = double;
    using C = double;
    static constexpr bool shifted = false;
    template <int q> __device__ static C ld(const S *p) { return __ldg(p); }
    template <int q> __device__ static C ldv(S v) { return v; }
    template <int q> __device__ static void st(S *p, C v) { *p = v; }
};

// read-only population loads with the L2::256B hint: each miss fills two
// 128-byte lines of the stream (+1.3% on the 256^3 cavity for FP32)
__device__ __forceinline__ float ld_pop(const float *p) {
    float v;
    asm("ld.global.nc.L2::256B.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ __half ld_pop(const __half *p) {
    unsigned short v;
    asm("ld.global.nc.L2::256B.b16 %0, [%1];" : "=h"(v) : "l"(p));
    return __ushort_as_half(v);
}

struct StoreF32 {
    using S = float;
    using C = float;
    static constexpr bool shifted = true; // holds f_q - w_q
    template <int q> __device__ static C ld(const S *p) { return ld_pop(p); }
    template <int q> __device__ static C ldv(S v) { return v; }
    template <int q> __device__ static void st(S *p, C v) { *p = v; }
};

// FP16 holds 2^12 * (f_q - w_q) / w_q
struct StoreF16 {
    using S = __half;
    using C = float;
    static constexpr bool shifted = true;
    template <int q> __device__ static constexpr float dec() {
        return WCLASS(q) == 0 ? (1.0f / 12288.0f) : WCLASS(q) == 1 ? (1.0f / 73728.0f) : (1.0f / 147456.0f);
    }
    template <int q> __device__ static constexpr float enc() {
        return WCLASS(q) == 0 ? 12288.0f : WCLASS(q) == 1 ? 73728.0f : 147456.0f;
    }
    template <int q> __device__ static C ld(const S *p) {
        return __half2float(ld_pop(p)) * dec<q>();
    }
    template <int q> __device__ static C ldv(S v) { return __half2float(v) * dec<q>(); }
    template <int q> __device__ static void st(S *p, C v) { *p = __float2half_rn(v * enc<q>()); }
    // the stored value itself, for physics that works on it directly
    template <int q> __device__ static C ldr(const S *p) { return __half2float(ld_pop(p)); }
    template <int q> __device__ static C ldvr(S v) { return __half2float(v); }
    template <int q> __device__ static void str(S *p, C v) { *p = __float2half_rn(v); }
};

// physics policies whose forcing takes a force density F = F_field + rho g
// (the C++ executable's model) declare force_density = true; the others
// take an acceleration a = g + a_field
template <class PH, class = void> struct uses_force_density {
    static constexpr bool value = false;
};
template <class PH> struct uses_force_density<PH, std::void_t<decltype(PH::force_density)>> {
    static constexpr bool value = PH::force_density;
};

// physics policies that collide the stored FP16 values directly (the scale
// of each weight class folded into the moments and the projection) declare
// h_space = true and provide collide_h; the bulk of the sites then skips the
// per-population decode and encode.  Boundary nodes keep the decoded path.
template <class PH, class = void> struct uses_h_space {
    static constexpr bool value = false;
};
template <class PH> struct uses_h_space<PH, std::void_t<decltype(PH::h_space)>> {
    static constexpr bool value = PH::h_space;
};
template <class ST, class PH, int q> __device__ __forceinline__ typename ST::C bulk_ld(const typename ST::S *p) {
    if constexpr (uses_h_space<PH>::value) return ST::template ldr<q>(p);
    else return ST::template ld<q>(p);
}
template <class ST, class PH, int q> __device__ __forceinline__ typename ST::C bulk_ldv(typename ST::S v) {
    if constexpr (uses_h_space<PH>::value) return ST::template ldvr<q>(v);
    else return ST::template ldv<q>(v);
}
template <class ST, class PH, int q> __device__ __forceinline__ void bulk_st(typename ST::S *p, typename ST::C v) {
    if constexpr (uses_h_space<PH>::value) ST::template str<q>(p, v);
    else ST::template st<q>(p, v);
}
template <class ST, class PH, class C>
__device__ __forceinline__ C bulk_collide(C *fv, C ax, C ay, C az, C we, C wo, C &ux, C &uy, C &uz) {
    if constexpr (uses_h_space<PH>::value) return PH::collide_h(fv, ax, ay, az, we, wo, ux, uy, uz);
    else return PH::collide(fv, ax, ay, az, we, wo, ux, uy, uz);
}

// a double kernel parameter in the compute type: float kernels take the
// host-rounded copy, double kernels the value itself
template <class C> __device__ __forceinline__ C par(double d, float f) {
    if constexpr (sizeof(C) == sizeof(float)) return (C)f;
    else return (C)d;
}
template <class C> __device__ __forceinline__ C arg_g(const StepArgs &a, int d) { return par<C>(a.g[d], a.gf[d]); }
template <class C> __device__ __forceinline__ C arg_we(const StepArgs &a) { return par<C>(a.w_e, a.w_ef); }
template <class C> __device__ __forceinline__ C arg_wo(const StepArgs &a) { return par<C>(a.w_o, a.w_of); }

// compile-time loop
template <int I, int N> struct Unroll {
    template <class F> __device__ __forceinline__ static void run(F &&f) {
        f.template operator()<I>();
        Unroll<I + 1, N>::run(f);
    }
};
template <int N> struct Unroll<N, N> {
    template <class F> __device__ __forceinline__ static void run(F &&) {}
};

// floor(l / d) and the remainder from a float reciprocal inv = 1/d, for
// 0 <= l < 2^31, 0 < d < 2^30 and a quotient below 2^21: the three roundings
// (l, inv, product) keep the estimate within 1 of l/d, so one correction
// step either way is exact (the trial remainder lies in (-d, 2d))
__device__ __forceinline__ int32_t split_div(int32_t l, int32_t d, float inv, int32_t &rem) {
    int32_t q = (int32_t)((float)l * inv);
    int32_t r = (int32_t)((uint32_t)l - (uint32_t)q * (uint32_t)d);
    if (r < 0) { --q; r += d; }
    else if (r >= d) { ++q; r -= d; }
    rem = r;
    return q;
}

// ---------------------------------------------------------------------------
// dense (interior / plain bounce-back / periodic) nodes
// ---------------------------------------------------------------------------
template <class ST, class PH, bool PSTEP, bool ACCF, class IT>
__device__ __forceinline__ void dense_node(const StepArgs &a, int b) {
    using S = typename ST::S;
    using C = typename ST::C;
    int row, k;
    if (a.lin) {
        // blocks of (128, 1) over consecutive sites
        const uint32_t site = (uint32_t)b * 128u + threadIdx.x;
        if (site >= a.nsite) return;
        row = (int)udiv(site, a.div_nz);
        k = (int)(site - (uint32_t)row * (uint32_t)a.nz);
    } else {
        const int kb = b % a.kblocks;
        const int rb = b / a.kblocks;
        row = rb * a.by + (int)threadIdx.y;
        k = kb * a.bx + (int)threadIdx.x;
        if (row >= a.nx * a.ny || k >= a.nz) return;
    }
    // element indices fit IT (int32 when 19 * Np < 2^31, chosen by the host)
    const IT n = (IT)row * a.nz + k;
    const uint8_t cls = __ldg(a.ncls + n);
    if (cls >= CLS_SPECIAL) return;
    // the link mask matters only to the pull-push step of wall nodes
    const uint32_t m = (PSTEP && cls == CLS_WALL) ? __ldg(a.nmask + n) : 0u;

    S *__restrict__ f = (S *)a.f;
    const IT Np = (IT)a.Np;
    C fv[Q];

    // relative offsets of the (periodically wrapped) neighbours along each
    // axis; index 0 -> -1, 1 -> 0, 2 -> +1
    IT dI[3], dJ[3], dK[3];
    if (PSTEP) {
        const int i = (int)udiv((uint32_t)row, a.div_ny);
        const int j = row - i * a.ny;
        const IT sI = (IT)a.ny * a.nz, sJ = (IT)a.nz;
        dI[0] = (i == 0 ? (IT)(a.nx - 1) : (IT)-1) * sI;
        dI[1] = 0;
        dI[2] = (i + 1 == a.nx ? (IT)(1 - a.nx) : (IT)1) * sI;
        dJ[0] = (j == 0 ? (IT)(a.ny - 1) : (IT)-1) * sJ;
        dJ[1] = 0;
        dJ[2] = (j + 1 == a.ny ? (IT)(1 - a.ny) : (IT)1) * sJ;
        dK[0] = k == 0 ? (IT)(a.nz - 1) : (IT)-1;
        dK[1] = 0;
        dK[2] = k + 1 == a.nz ? (IT)(1 - a.nz) : (IT)1;
    }

    // gather: a bounce-back link reads its own opposite slot; the choice is a
    // select, not a branch
    Unroll<0, Q>::run([&]<int q>() {
        IT e;
        if (!PSTEP || q == 9) {
            e = (IT)q * Np + n;
        } else {
            const IT src = n + dI[1 - CX(q)] + dJ[1 - CY(q)] + dK[1 - CZ(q)];
            const IT e_reg = (IT)OPP(q) * Np + src;
            const IT e_bb = (IT)q * Np + n;
            e = (m & (1u << q)) ? e_bb : e_reg;
        }
        fv[q] = bulk_ld<ST, PH, q>(f + e);
    });

    C ux, uy, uz, rho;
    if constexpr (uses_force_density<PH>::value) {
        C fx = 0, fy = 0, fz = 0;
        if (ACCF) {
            const C *acc = (const C *)a.acc;
            fx = __ldg(acc + n); fy = __ldg(acc + Np + n); fz = __ldg(acc + 2 * Np + n);
        }
        rho = PH::collide_fd(fv, arg_g<C>(a, 0), arg_g<C>(a, 1), arg_g<C>(a, 2), fx, fy, fz, arg_we<C>(a),
                             arg_wo<C>(a), ux, uy, uz);
    } else {
        C ax, ay, az;
        if (ACCF) {
            const C *acc = (const C *)a.acc;
            ax = arg_g<C>(a, 0) + __ldg(acc + n);
            ay = arg_g<C>(a, 1) + __ldg(acc + Np + n);
            az = arg_g<C>(a, 2) + __ldg(acc + 2 * Np + n);
        } else {
            ax = arg_g<C>(a, 0); ay = arg_g<C>(a, 1); az = arg_g<C>(a, 2);
        }
        rho = bulk_collide<ST, PH>(fv, ax, ay, az, arg_we<C>(a), arg_wo<C>(a), ux, uy, uz);
    }

    // scatter: a population heading into a solid is stored back into this
    // node's opposite slot
    S *fo = a.fout ? (S *)a.fout : f;
    Unroll<0, Q>::run([&]<int q>() {
        IT e;
        if (!PSTEP) {
            bulk_st<ST, PH, OPP(q)>(fo + ((IT)OPP(q) * Np + n), fv[q]);
            return;
        }
        if (q == 9) {
            e = (IT)9 * Np + n;
        } else {
            const IT dst = n + dI[1 + CX(q)] + dJ[1 + CY(q)] + dK[1 + CZ(q)];
            const IT e_reg = (IT)q * Np + dst;
            const IT e_bb = (IT)OPP(q) * Np + n;
            e = (m & (1u << OPP(q))) ? e_bb : e_reg;
        }
        bulk_st<ST, PH, q>(fo + e, fv[q]);
    });

    if (a.write_moments) {
        ((C *)a.den)[n] = rho;
        ((C *)a.ux)[n] = ux;
        ((C *)a.uy)[n] = uy;
        ((C *)a.uz)[n] = uz;
    }
}

// ---------------------------------------------------------------------------
// boundary nodes (Zou-He, symmetric faces, moving solids)
// ---------------------------------------------------------------------------
template <class ST, class PH, bool PSTEP, bool ACCF>
__device__ __forceinline__ void special_node(const StepArgs &a, int b) {
    using S = typename ST::S;
    using C = typename ST::C;
    const int t = b * (int)(blockDim.x * blockDim.y) + (int)(threadIdx.y * blockDim.x + threadIdx.x);
    const int M = a.M;
    if (t >= M) return;
    const int64_t n = __ldg(a.sp_node + t);
    const uint32_t info = __ldg(a.sp_info + t);
    S *__restrict__ f = (S *)a.f;
    const int64_t Np = a.Np;
    // population slots of the node: lattice layout, or the fluid-only layout
    const int64_t pn = a.sp_cnode ? __ldg(a.sp_cnode + t) : n;
    const int64_t PNp = a.sp_cnode ? a.Npc : Np;
    C *spden = (C *)a.sp_den;
    const C dprev = spden[t];
    C fv[Q];

    Unroll<0, Q>::run([&]<int q>() {
        const int64_t addr = PSTEP ? __ldg(a.sp_rd + (int64_t)q * M + t) : (int64_t)q * PNp + pn;
        // the value read may belong to any slot; decode with the slot of q's
        // source population (same weight class: mirrors and opposites keep it)
        C v = ST::template ld<q>(f + addr);
        if (q != 9 && (info & (1u << q)))
            v = PH::template ladd<q>(v, dprev, (C)__ldg(a.sp_lw + (int64_t)q * M + t));
        fv[q] = v;
    });

    const uint32_t faces = (info >> SP_FACE_SHIFT) & 0x3Fu;
    if (faces) {
        int slot = 0;
#pragma unroll
        for (int fc = 0; fc < 6; ++fc) {
            if (faces & (1u << fc)) {
                const double *bcd = a.sp_bc + (int64_t)(4 * slot) * M + t;
                PH::zou_he(fc, a.bc[fc], bcd[0], bcd[M], bcd[2 * (int64_t)M], bcd[3 * (int64_t)M], fv);
                slot = 1;
            }
        }
    }
    if (a.sp_tee) {
        S *tee = (S *)a.sp_tee;
        Unroll<0, Q>::run([&]<int q>() { ST::template st<q>(tee + ((int64_t)q * M + t), fv[q]); });
    }

    C ux, uy, uz, rho;
    if constexpr (uses_force_density<PH>::value) {
        C fx = 0, fy = 0, fz = 0;
        if (ACCF) {
            const C *acc = (const C *)a.acc;
            fx = __ldg(acc + n); fy = __ldg(acc + Np + n); fz = __ldg(acc + 2 * Np + n);
        }
        rho = PH::collide_fd(fv, arg_g<C>(a, 0), arg_g<C>(a, 1), arg_g<C>(a, 2), fx, fy, fz, arg_we<C>(a),
                             arg_wo<C>(a), ux, uy, uz);
    } else {
        C ax, ay, az;
        if (ACCF) {
            const C *acc = (const C *)a.acc;
            ax = arg_g<C>(a, 0) + __ldg(acc + n);
            ay = arg_g<C>(a, 1) + __ldg(acc + Np + n);
            az = arg_g<C>(a, 2) + __ldg(acc + 2 * Np + n);
        } else {
            ax = arg_g<C>(a, 0); ay = arg_g<C>(a, 1); az = arg_g<C>(a, 2);
        }
        rho = PH::collide(fv, ax, ay, az, arg_we<C>(a), arg_wo<C>(a), ux, uy, uz);
    }

    S *fo = a.fout ? (S *)a.fout : f;
    Unroll<0, Q>::run([&]<int q>() {
        if (PSTEP) {
            const int64_t addr = __ldg(a.sp_wr + (int64_t)q * M + t);
            ST::template st<q>(fo + addr, fv[q]);
        } else {
            ST::template st<OPP(q)>(fo + OPP(q) * PNp + pn, fv[q]);
        }
    });
    spden[t] = rho;
    if (a.write_moments) {
        ((C *)a.den)[n] = rho;
        ((C *)a.ux)[n] = ux;
        ((C *)a.uy)[n] = uy;
        ((C *)a.uz)[n] = uz;
    }
}

// ---------------------------------------------------------------------------
// fluid sites on the fluid-only layout.  On porous lattices a lattice-ordered
// sweep fetches whole population lines that are partly solid slots; here the
// populations of fluid sites are packed (f[q * Npc + m]) and a neighbour's
// slot is found through the lattice-to-fluid index map (cidx, 4 bytes per
// lattice site, cached), so only fluid populations move.  Same arithmetic and
// AA pattern as dense_node.  Element indices are 32-bit unsigned: the host
// uses this layout only when 19 * Npc < 2^32.
// ---------------------------------------------------------------------------
template <class ST, class PH, bool PSTEP, bool ACCF>
__device__ __forceinline__ void sparse_node(const StepArgs &a, int b) {
    using S = typename ST::S;
    using C = typename ST::C;
    const uint32_t m = (uint32_t)b * (blockDim.x * blockDim.y) + (threadIdx.y * blockDim.x + threadIdx.x);
    if (m >= (uint64_t)a.Nc) return;
    const int32_t n = __ldg(a.csite + m);
    const uint8_t cls = __ldg(a.ncls + n);
    if (cls >= CLS_SPECIAL) return;
    const uint32_t mk = (PSTEP && cls == CLS_WALL) ? __ldg(a.nmask + n) : 0u;
    S *__restrict__ f = (S *)a.f;
    const uint32_t Npc = (uint32_t)a.Npc; // 19 * Npc < 2^32 (checked by the host)
    int32_t dI[3], dJ[3], dK[3];
    if (PSTEP) {
        const int32_t syz = a.ny * a.nz;
        int32_t i, r, j, k;
        if (a.inv_syz != 0.0f) {
            i = split_div(n, syz, a.inv_syz, r);
            j = split_div(r, a.nz, a.inv_nz, k);
        } else {
            i = n / syz; r = n - i * syz; j = r / a.nz; k = r - j * a.nz;
        }
        dI[0] = (i == 0 ? (a.nx - 1) : -1) * syz; dI[1] = 0; dI[2] = (i + 1 == a.nx ? (1 - a.nx) : 1) * syz;
        dJ[0] = (j == 0 ? (a.ny - 1) : -1) * a.nz; dJ[1] = 0; dJ[2] = (j + 1 == a.ny ? (1 - a.ny) : 1) * a.nz;
        dK[0] = k == 0 ? (a.nz - 1) : -1; dK[1] = 0; dK[2] = k + 1 == a.nz ? (1 - a.nz) : 1;
    }
    // fluid index of the neighbour across link q (site x + c_q); only asked
    // for links that do not bounce back, whose neighbour is fluid
    // the fluid indices of the 18 neighbours, looked up once for the gather
    // and the scatter (links that bounce back do not use theirs)
    uint32_t nb[Q];
    if (PSTEP) {
        Unroll<0, Q>::run([&]<int q>() {
            if (q != 9) nb[q] = (uint32_t)__ldg(a.cidx + (n + dI[1 + CX(q)] + dJ[1 + CY(q)] + dK[1 + CZ(q)]));
        });
    }
    auto nbr = [&]<int q>() -> uint32_t { return nb[q]; };
    C fv[Q];
    Unroll<0, Q>::run([&]<int q>() {
        uint32_t e;
        if (!PSTEP || q == 9) e = (uint32_t)q * Npc + m;
        else if (mk & (1u << q)) e = (uint32_t)q * Npc + m;
        else e = (uint32_t)OPP(q) * Npc + nbr.template operator()<OPP(q)>();
        fv[q] = bulk_ld<ST, PH, q>(f + e);
    });
    C ux, uy, uz;
    C ax, ay, az;
    if (ACCF) {
        const C *acc = (const C *)a.acc;
        ax = arg_g<C>(a, 0) + __ldg(acc + n);
        ay = arg_g<C>(a, 1) + __ldg(acc + a.Np + n);
        az = arg_g<C>(a, 2) + __ldg(acc + 2 * a.Np + n);
    } else {
        ax = arg_g<C>(a, 0); ay = arg_g<C>(a, 1); az = arg_g<C>(a, 2);
    }
    const C rho = bulk_collide<ST, PH>(fv, ax, ay, az, arg_we<C>(a), arg_wo<C>(a), ux, uy, uz);
    Unroll<0, Q>::run([&]<int q>() {
        if (!PSTEP) {
            bulk_st<ST, PH, OPP(q)>(f + ((uint32_t)OPP(q) * Npc + m), fv[q]);
            return;
        }
        uint32_t e;
        if (q == 9) e = 9u * Npc + m;
        else if (mk & (1u << OPP(q))) e = (uint32_t)OPP(q) * Npc + m;
        else e = (uint32_t)q * Npc + nbr.template operator()<q>();
        bulk_st<ST, PH, q>(f + e, fv[q]);
    });
    if (a.write_moments) {
        ((C *)a.den)[n] = rho;
        ((C *)a.ux)[n] = ux;
        ((C *)a.uy)[n] = uy;
        ((C *)a.uz)[n] = uz;
    }
}

// ---------------------------------------------------------------------------
// L2 prefetch of a dense block's source rows.  The direct kernels hold their
// 19 loads per site in registers, which caps the loads in flight per SM; line
// prefetches into L2 (one warp, no registers held) issued one resident wave
// ahead let the later loads hit L2.  Block b covers one contiguous run
// of sites [n0, n0 + cnt) under both mappings; the P step reads slot opp(q)
// at n - c_q (wraps aside), the L step slot q at n.  Ranges are clamped to
// the slot's sites and widened to 16-byte boundaries.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void prefetch_line(const void *p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// called by all 32 lanes of one warp: lane l prefetches lines l, l + 32, ...
// of the block's 19 source rows
template <class S, bool PSTEP>
__device__ __forceinline__ void prefetch_block(const StepArgs &a, int b, int lane) {
    int64_t n0, cnt;
    const int64_t N = (int64_t)a.nx * a.ny * a.nz;
    if (a.lin) {
        n0 = (int64_t)b * 128;
        cnt = 128;
    } else {
        const int kb = b % a.kblocks, rb = b / a.kblocks;
        const int k0 = kb * a.bx;
        n0 = (int64_t)rb * a.by * a.nz + k0;
        cnt = a.kblocks == 1 ? (int64_t)a.by * a.nz : (int64_t)min(a.bx, a.nz - k0);
    }
    if (n0 >= N) return;
    if (n0 + cnt > N) cnt = N - n0;
    const char *f = (const char *)a.f;
    const int64_t syz = (int64_t)a.ny * a.nz;
    constexpr int LPR = 128 * (int)sizeof(S) / 128 + 1; // 128-byte lines per source row
#pragma unroll 1
    for (int idx = lane; idx < Q * LPR; idx += 32) {
        const int q = idx / LPR, line = idx - q * LPR;
        const int64_t d = PSTEP ? (int64_t)CX(q) * syz + (int64_t)CY(q) * a.nz + CZ(q) : 0;
        int64_t e = n0 - d - 1 + (int64_t)line * (128 / (int)sizeof(S));
        if (e < 0) e = 0;
        if (e >= N) continue;
        const int slot = PSTEP ? OPP(q) : q;
        prefetch_line(f + (slot * a.Np + e) * (int64_t)sizeof(S));
    }
}

// resident 128-thread blocks per SM asked of the register allocator, per
// kernel kind (the build sets them per storage type)
#ifndef JLB_MIN_BLOCKS
#define JLB_MIN_BLOCKS 1
#endif
#ifndef JLB_MIN_BLOCKS_STEP
#define JLB_MIN_BLOCKS_STEP JLB_MIN_BLOCKS
#endif
#ifndef JLB_MIN_BLOCKS_TMA
#define JLB_MIN_BLOCKS_TMA JLB_MIN_BLOCKS
#endif
#ifndef JLB_MIN_BLOCKS_SPARSE
#define JLB_MIN_BLOCKS_SPARSE JLB_MIN_BLOCKS
#endif
#ifndef JLB_MIN_BLOCKS_SPARSE_L
#define JLB_MIN_BLOCKS_SPARSE_L JLB_MIN_BLOCKS_SPARSE
#endif
template <class ST, class PH, bool PSTEP, bool ACCF, class IT>
__global__ void __launch_bounds__(128, JLB_MIN_BLOCKS_STEP) lbm_step_kernel(const StepArgs a) {
    const int b = (int)blockIdx.x;
    if (b < a.nb_dense) {
        if (a.pf && threadIdx.y == 0 && threadIdx.x < 32 && b + a.pf < a.nb_dense)
            prefetch_block<typename ST::S, PSTEP>(a, b + a.pf + a.b0, (int)threadIdx.x);
        dense_node<ST, PH, PSTEP, ACCF, IT>(a, b + a.b0);
    } else {
        special_node<ST, PH, PSTEP, ACCF>(a, b - a.nb_dense);
    }
}

template <class ST, class PH, bool PSTEP, bool ACCF>
__global__ void __launch_bounds__(128, PSTEP ? JLB_MIN_BLOCKS_SPARSE : JLB_MIN_BLOCKS_SPARSE_L)
    lbm_step_sparse_kernel(const StepArgs a) {
    const int b = (int)blockIdx.x;
    const int nbc = (int)((a.Nc + 127) / 128);
    if (b < nbc) sparse_node<ST, PH, PSTEP, ACCF>(a, b);
    else special_node<ST, PH, PSTEP, ACCF>(a, b - nbc);
}

template <class ST, template <int> class PH>
int launch_step_sparse_impl(const StepArgs &a, int scheme, bool pstep, bool accf, int blocks, cudaStream_t st) {
#define JLB_SL(SCH, P, A) lbm_step_sparse_kernel<ST, PH<SCH>, P, A><<<blocks, 128, 0, st>>>(a)
#define JLB_SS(SCH)                                                          \
    if (pstep) { if (accf) JLB_SL(SCH, true, true); else JLB_SL(SCH, true, false); } \
    else { if (accf) JLB_SL(SCH, false, true); else JLB_SL(SCH, false, false); }
    if (scheme == SCH_BGK) { JLB_SS(SCH_BGK) }
    else if (scheme == SCH_TRT) { JLB_SS(SCH_TRT) }
    else { JLB_SS(SCH_REG) }
#undef JLB_SS
#undef JLB_SL
    return (int)cudaGetLastError();
}

template <class ST, template <int> class PH>
int launch_step_impl(const StepArgs &a, int scheme, bool pstep, bool accf, int blocks, cudaStream_t st) {
    dim3 blk(a.bx, a.by), grd(blocks);
    const bool i64 = a.Np * 19 > 0x7fffffffLL;
#define JLB_L(SCH, P, A)                                                                 \
    do {                                                                                 \
        if (i64) lbm_step_kernel<ST, PH<SCH>, P, A, int64_t><<<grd, blk, 0, st>>>(a);    \
        else lbm_step_kernel<ST, PH<SCH>, P, A, int32_t><<<grd, blk, 0, st>>>(a);        \
    } while (0)
#define JLB_S(SCH)                                   \
    if (pstep) { if (accf) JLB_L(SCH, true, true); else JLB_L(SCH, true, false); } \
    else { if (accf) JLB_L(SCH, false, true); else JLB_L(SCH, false, false); }
    if (scheme == SCH_BGK) { JLB_S(SCH_BGK) }
    else if (scheme == SCH_TRT) { JLB_S(SCH_TRT) }
    else { JLB_S(SCH_REG) }
#undef JLB_S
#undef JLB_L
    return (int)cudaGetLastError();
}

} // namespace jlb
