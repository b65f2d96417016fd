// lbm_adjoint.cu -- discrete adjoint of the fused D3Q19 step (reverse AA
// sweep).
//
// For a step that maps the AA array F_t to F_{t+1}, node x reads its inputs
// from the address set R_x and writes its outputs to W_x; in the AA pattern
// R_x and W_x are the same set and no other node touches it.  The adjoint
// Lam_t = (dF_{t+1}/dF_t)^T Lam_{t+1} is therefore computed in place, node by
// node: read Lam at the addresses the forward step wrote, apply the
// transposed collision and Zou-He Jacobians, write Lam at the addresses the
// forward step read.  Bounce-back links are part of the address maps, so
// their transpose comes for free.  The collision inputs of the step are
// gathered again from the state before the step, which the recompute of the
// segment wrote out of place (StepArgs::fout); boundary sites, whose inputs
// pass through Zou-He, read a copy the recompute kept (StepArgs::sp_tee).
//
// Collision (BGK / TRT with forcing, jyulb/D3Q19.pyx:655-853):
//   rho = sum g, j = sum c g, s = j + rho a / 2,
//   H0 = we rho, H1 = wo s + c1 rho a, H2 = we s s / rho + c2 (a s + s a),
//   f*_q = c3 g_q - c4 g_opp(q) + P_q(H),  f*_rest = (1 - we) g_rest + P_rest(H),
// with c1 = 1 - wo/2, c2 = 1 - we/2, c3 = 1 - (we + wo)/2, c4 = (we - wo)/2
// (BGK: wo = we) and P_q(H) = w_q (H0 + 3 c.H1 + 4.5 (c c - I/3):H2).
// Regularized (jyulb/D3Q19.pyx:859-940): f* = P(H) with
//   H0 = rho, H1 = j + rho a, H2 = (1 - we) (Pi - rho I/3) + we s s / rho + c2 (a s + s a),
// Pi = sum c c g the second moment of the inputs.
// Their transposes and the local sensitivities to we, wo and a are written
// out below.  Zou-He is affine in the populations and in j, so its transpose
// is read off the forward assignment applied to unit vectors.
#include "lbm_adjoint.h"
#include "lbm_step.cuh"

namespace jlb {

template <int q> __device__ constexpr double WQ() {
    return WCLASS(q) == 0 ? (12.0 / 36.0) : WCLASS(q) == 1 ? (2.0 / 36.0) : (1.0 / 36.0);
}

// unknown-population assignment of the Zou-He scheme (jyulb/bcs.pyx:487-716);
// linear in g and j
template <class C> __device__ void zh_assign(int fc, C jx, C jy, C jz, C *g) {
    const C s6 = (C)(1.0 / 6.0), s3 = (C)(1.0 / 3.0), h = (C)0.5;
    C t;
    switch (fc) {
    case 0:
        t = g[11] + g[12] + g[13] - g[5] - g[6] - g[7];
        g[14] = g[4] + s6 * jx + h * t - h * jy;
        g[18] = g[0] + s6 * jx - h * t + h * jy;
        t = g[7] + g[10] + g[13] - g[5] - g[8] - g[11];
        g[15] = g[3] + s6 * jx + h * t - h * jz;
        g[17] = g[1] + s6 * jx - h * t + h * jz;
        g[16] = g[2] + s3 * jx;
        break;
    case 1:
        t = g[11] + g[12] + g[13] - g[5] - g[6] - g[7];
        g[0] = g[18] - s6 * jx + h * t - h * jy;
        g[4] = g[14] - s6 * jx - h * t + h * jy;
        t = g[7] + g[10] + g[13] - g[5] - g[8] - g[11];
        g[1] = g[17] - s6 * jx + h * t - h * jz;
        g[3] = g[15] - s6 * jx - h * t + h * jz;
        g[2] = g[16] - s3 * jx;
        break;
    case 2:
        t = g[15] + g[16] + g[17] - g[1] - g[2] - g[3];
        g[4] = g[14] + s6 * jy + h * t - h * jx;
        g[18] = g[0] + s6 * jy - h * t + h * jx;
        t = g[17] + g[10] + g[3] - g[15] - g[8] - g[1];
        g[11] = g[7] + s6 * jy + h * t - h * jz;
        g[13] = g[5] + s6 * jy - h * t + h * jz;
        g[12] = g[6] + s3 * jy;
        break;
    case 3:
        t = g[15] + g[16] + g[17] - g[1] - g[2] - g[3];
        g[0] = g[18] - s6 * jy + h * t - h * jx;
        g[14] = g[4] - s6 * jy - h * t + h * jx;
        t = g[17] + g[10] + g[3] - g[15] - g[8] - g[1];
        g[5] = g[13] - s6 * jy + h * t - h * jz;
        g[7] = g[11] - s6 * jy - h * t + h * jz;
        g[6] = g[12] - s3 * jy;
        break;
    case 4:
        t = g[18] + g[16] + g[14] - g[4] - g[2] - g[0];
        g[3] = g[15] + s6 * jz + h * t - h * jx;
        g[17] = g[1] + s6 * jz - h * t + h * jx;
        t = g[18] + g[12] + g[4] - g[14] - g[6] - g[0];
        g[7] = g[11] + s6 * jz + h * t - h * jy;
        g[13] = g[5] + s6 * jz - h * t + h * jy;
        g[10] = g[8] + s3 * jz;
        break;
    default:
        t = g[18] + g[16] + g[14] - g[4] - g[2] - g[0];
        g[1] = g[17] - s6 * jz + h * t - h * jx;
        g[15] = g[3] - s6 * jz - h * t + h * jx;
        t = g[18] + g[12] + g[4] - g[14] - g[6] - g[0];
        g[5] = g[13] - s6 * jz + h * t - h * jy;
        g[11] = g[7] - s6 * jz - h * t + h * jy;
        g[8] = g[10] - s3 * jz;
        break;
    }
}

__device__ __forceinline__ int axcomp(int q, int ax) { return ax == 0 ? CX(q) : ax == 1 ? CY(q) : CZ(q); }

// Transposed Zou-He at a face node.  gp: the populations after Zou-He (the
// known ones equal the pre-Zou-He values), mu: adjoint w.r.t. gp; returns in
// mu the adjoint w.r.t. the pre-Zou-He populations and adds the adjoint of the
// face data: du (boundary velocity; a FIXED_DEN face uses its tangential
// components) and dden (density of a FIXED_DEN face).
template <class C, bool SHIFTED>
__device__ void zh_adjoint(int fc, int kind, double den, double ux, double uy, double uz, const C *gp, C *mu,
                           double *du, double &dden) {
    const int ax = fc >> 1;
    const bool high = fc & 1;
    const int in_sign = high ? -1 : 1; // normal component of the unknown populations
    // S = sum of populations with zero normal component + 2 * sum leaving
    C S = SHIFTED ? (C)1 : (C)0;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int cn = axcomp(q, ax);
        if (cn == 0) S += gp[q];
        else if (cn == -in_sign) S += (C)2 * gp[q];
    }
    const double u[3] = {ux, uy, uz};
    // adjoint through the assignment: lam_known = A^T mu, dj = B^T mu
    C lam[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        C e[Q];
#pragma unroll
        for (int p = 0; p < Q; ++p) e[p] = (p == q) ? (C)1 : (C)0;
        zh_assign<C>(fc, (C)0, (C)0, (C)0, e);
        C acc = 0;
#pragma unroll
        for (int p = 0; p < Q; ++p) acc += mu[p] * e[p];
        lam[q] = acc;
    }
    C dj[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        C e[Q];
#pragma unroll
        for (int p = 0; p < Q; ++p) e[p] = (C)0;
        zh_assign<C>(fc, a == 0 ? (C)1 : (C)0, a == 1 ? (C)1 : (C)0, a == 2 ? (C)1 : (C)0, e);
        C acc = 0;
#pragma unroll
        for (int p = 0; p < Q; ++p) acc += mu[p] * e[p];
        dj[a] = acc;
    }
    C dS;
    if (kind == BC_FIXED_VEL) {
        // j = rho_bc u, rho_bc = S / (1 -/+ u_n)
        const double un = u[ax];
        const double denom = high ? 1.0 + un : 1.0 - un;
        const double rho_bc = (double)S / denom;
        const double dju = (double)dj[0] * ux + (double)dj[1] * uy + (double)dj[2] * uz;
        dS = (C)(dju / denom);
        for (int a = 0; a < 3; ++a) du[a] += rho_bc * (double)dj[a];
        du[ax] += dju * (high ? -rho_bc / denom : rho_bc / denom);
    } else {
        // j_n = den - S on a low face, S - den on a high one; j_t = den u_t
        dS = high ? dj[ax] : -dj[ax];
        dden += high ? -(double)dj[ax] : (double)dj[ax];
        for (int t = 0; t < 3; ++t) {
            if (t == ax) continue;
            dden += (double)dj[t] * u[t];
            du[t] += den * (double)dj[t];
        }
    }
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int cn = axcomp(q, ax);
        C v = lam[q];
        if (cn == 0) v += dS;
        else if (cn == -in_sign) v += (C)2 * dS;
        mu[q] = v;
    }
}

// Transposed collision, in two phases so that the inputs g need not stay
// live: AdjSums accumulates, population by population, the moments of the
// inputs (rho, j), the moments of the output adjoint lo (L0, L1, L2) and the
// input-weighted sums the relaxation-rate sensitivities need; adj_finish then
// forms the adjoint of every input li_q (handed to `put`) and adds the local
// sensitivities to we, wo, ax, ay, az into pg.  On the loss step a site of the
// loss plane adds the seed dL/du of its stored velocity u = j/rho + a/2.
template <class C, bool SHIFTED, bool PI = false> struct AdjSums {
    C rho = SHIFTED ? (C)1 : (C)0, jx = 0, jy = 0, jz = 0;
    C pxx = 0, pyy = 0, pzz = 0, pxy = 0, pxz = 0, pyz = 0; // sum c c g (PI: regularized)
    C L0 = 0, L1x = 0, L1y = 0, L1z = 0, Lxx = 0, Lyy = 0, Lzz = 0, Lxy = 0, Lxz = 0, Lyz = 0;
    C sum_pair = 0; // sum_q lo_q (f_q + f_opp(q)), q != rest
    C dif_pair = 0; // sum_q lo_q (f_opp(q) - f_q)
    C rest = 0;     // lo_rest f_rest
    // input g (shifted by w when SHIFTED) and output adjoint l of population q
    template <int q> __device__ __forceinline__ void add(C g, C l) {
        constexpr C w = (C)WQ<q>();
        constexpr int cx = CX(q), cy = CY(q), cz = CZ(q);
        rho += g;
        if (cx) jx += (C)cx * g;
        if (cy) jy += (C)cy * g;
        if (cz) jz += (C)cz * g;
        if constexpr (PI) {
            if (cx) pxx += g;
            if (cy) pyy += g;
            if (cz) pzz += g;
            if (cx * cy) pxy += (C)(cx * cy) * g;
            if (cx * cz) pxz += (C)(cx * cz) * g;
            if (cy * cz) pyz += (C)(cy * cz) * g;
        }
        const C wl = w * l;
        L0 += wl;
        if (cx) L1x += (C)(3 * cx) * wl;
        if (cy) L1y += (C)(3 * cy) * wl;
        if (cz) L1z += (C)(3 * cz) * wl;
        Lxx += (C)(4.5 * (cx * cx - 1.0 / 3.0)) * wl;
        Lyy += (C)(4.5 * (cy * cy - 1.0 / 3.0)) * wl;
        Lzz += (C)(4.5 * (cz * cz - 1.0 / 3.0)) * wl;
        if (cx * cy) Lxy += (C)(4.5 * cx * cy) * wl;
        if (cx * cz) Lxz += (C)(4.5 * cx * cz) * wl;
        if (cy * cz) Lyz += (C)(4.5 * cy * cz) * wl;
        if (q == 9) rest = l * (g + (SHIFTED ? w : (C)0));
    }
    // the pair (q, OPP(q)), q < 9, once both populations were added
    template <int q> __device__ __forceinline__ void pair(C gq, C go, C lq, C lo) {
        constexpr C w2 = SHIFTED ? (C)(2.0 * WQ<q>()) : (C)0;
        sum_pair += (lq + lo) * (gq + go + w2);
        dif_pair += (lq - lo) * (go - gq);
    }
};

// adds the population pair sums once all 19 inputs and adjoints are at hand
template <class C, bool SHIFTED, bool PI>
__device__ __forceinline__ void adj_accumulate(AdjSums<C, SHIFTED, PI> &S, const C *g, const C *lo) {
    Unroll<0, Q>::run([&]<int q>() { S.template add<q>(g[q], lo[q]); });
    Unroll<0, 9>::run([&]<int q>() { S.template pair<q>(g[q], g[OPP(q)], lo[q], lo[OPP(q)]); });
}

template <class C, bool SHIFTED, int SCH, bool SEED, bool PI, class PUT>
__device__ __forceinline__ void adj_finish(const AdjSums<C, SHIFTED, PI> &S, const C *lo, C ax, C ay, C az, C we,
                                           C wo, C *pg, bool on_plane, const double *tg, double gx, double gy,
                                           double gz, PUT &&put) {
    if (SCH == SCH_BGK) wo = we;
    const C rho = S.rho, jx = S.jx, jy = S.jy, jz = S.jz;
    const C c1 = (C)1 - (C)0.5 * wo, c2 = (C)1 - (C)0.5 * we;
    const C c3 = (C)1 - (C)0.5 * (we + wo), c4 = (C)0.5 * (we - wo);
    const C sx = jx + (C)0.5 * rho * ax, sy = jy + (C)0.5 * rho * ay, sz = jz + (C)0.5 * rho * az;
    const C Lsx = S.Lxx * sx + S.Lxy * sy + S.Lxz * sz;
    const C Lsy = S.Lxy * sx + S.Lyy * sy + S.Lyz * sz;
    const C Lsz = S.Lxz * sx + S.Lyz * sy + S.Lzz * sz;
    const C Lax = S.Lxx * ax + S.Lxy * ay + S.Lxz * az;
    const C Lay = S.Lxy * ax + S.Lyy * ay + S.Lyz * az;
    const C Laz = S.Lxz * ax + S.Lyz * ay + S.Lzz * az;
    const C ir = (C)1 / rho;
    const C dsx = wo * S.L1x + (C)2 * we * Lsx * ir + (C)2 * c2 * Lax;
    const C dsy = wo * S.L1y + (C)2 * we * Lsy * ir + (C)2 * c2 * Lay;
    const C dsz = wo * S.L1z + (C)2 * we * Lsz * ir + (C)2 * c2 * Laz;
    const C sLs = sx * Lsx + sy * Lsy + sz * Lsz;
    const C L1a = S.L1x * ax + S.L1y * ay + S.L1z * az;
    // the loss's own dependence on this site's rho and j (seeding step)
    C sd_rho = 0, sd_jx = 0, sd_jy = 0, sd_jz = 0;
    C dax_seed = 0, day_seed = 0, daz_seed = 0;
    if (SEED && on_plane) {
        // L = sum |u - target|^2 over the plane
        const C ux = jx * ir, uy = jy * ir, uz = jz * ir;
        const C d0 = (C)(2.0 * ((double)ux + 0.5 * gx - tg[0]));
        const C d1 = (C)(2.0 * ((double)uy + 0.5 * gy - tg[1]));
        const C d2 = (C)(2.0 * ((double)uz + 0.5 * gz - tg[2]));
        sd_jx = d0 * ir; sd_jy = d1 * ir; sd_jz = d2 * ir;
        sd_rho = -(d0 * ux + d1 * uy + d2 * uz) * ir;
        dax_seed = (C)0.5 * d0; day_seed = (C)0.5 * d1; daz_seed = (C)0.5 * d2;
    }
    const C drho = we * S.L0 + c1 * L1a - we * sLs * ir * ir + (C)0.5 * (ax * dsx + ay * dsy + az * dsz) + sd_rho;
    const C djx = dsx + sd_jx, djy = dsy + sd_jy, djz = dsz + sd_jz;
    if constexpr (SCH == SCH_REG) {
        // lam_q = K + d . c_q + (1 - we) c_q.M.c_q with M the output-adjoint
        // second moments (Lxx .. Lyz); no relaxation term (the projection
        // drops the non-hydrodynamic part)
        const C c1r = (C)1 - we;
        const C trM = S.Lxx + S.Lyy + S.Lzz;
        const C aLs = ax * Lsx + ay * Lsy + az * Lsz;
        const C aLa = ax * Lax + ay * Lay + az * Laz;
        const C K = S.L0 + L1a - c1r * trM * (C)(1.0 / 3.0) + we * (aLs * ir - sLs * ir * ir) + c2 * aLa + sd_rho;
        const C dx = S.L1x + (C)2 * we * Lsx * ir + (C)2 * c2 * Lax + sd_jx;
        const C dy = S.L1y + (C)2 * we * Lsy * ir + (C)2 * c2 * Lay + sd_jy;
        const C dz = S.L1z + (C)2 * we * Lsz * ir + (C)2 * c2 * Laz + sd_jz;
        Unroll<0, Q>::run([&]<int q>() {
            constexpr int cx = CX(q), cy = CY(q), cz = CZ(q);
            C v = K;
            if (cx) v += (C)cx * dx;
            if (cy) v += (C)cy * dy;
            if (cz) v += (C)cz * dz;
            C cmc = 0;
            if (cx) cmc += S.Lxx;
            if (cy) cmc += S.Lyy;
            if (cz) cmc += S.Lzz;
            if (cx * cy) cmc += (C)(2 * cx * cy) * S.Lxy;
            if (cx * cz) cmc += (C)(2 * cx * cz) * S.Lxz;
            if (cy * cz) cmc += (C)(2 * cy * cz) * S.Lyz;
            v += c1r * cmc;
            put.template operator()<q>(v);
        });
        // M:(Pi - rho I/3), the input's second moment (shifted populations
        // carry rho - 1 in rho - 1 and the same deviatoric moments)
        const C r3 = (SHIFTED ? (S.rho - (C)1) : S.rho) * (C)(1.0 / 3.0);
        const C MP = S.Lxx * (S.pxx - r3) + S.Lyy * (S.pyy - r3) + S.Lzz * (S.pzz - r3) +
                     (C)2 * (S.Lxy * S.pxy + S.Lxz * S.pxz + S.Lyz * S.pyz);
        pg[0] += -MP + sLs * ir - aLs;
        pg[2] += rho * S.L1x + (we + (C)2 * c2) * Lsx + c2 * rho * Lax + dax_seed;
        pg[3] += rho * S.L1y + (we + (C)2 * c2) * Lsy + c2 * rho * Lay + day_seed;
        pg[4] += rho * S.L1z + (we + (C)2 * c2) * Lsz + c2 * rho * Laz + daz_seed;
        return;
    }
    Unroll<0, Q>::run([&]<int q>() {
        constexpr int cx = CX(q), cy = CY(q), cz = CZ(q);
        C v;
        if (q == 9) v = ((C)1 - we) * lo[9];
        else v = c3 * lo[q] - c4 * lo[OPP(q)];
        v += drho;
        if (cx) v += (C)cx * djx;
        if (cy) v += (C)cy * djy;
        if (cz) v += (C)cz * djz;
        put.template operator()<q>(v);
    });
    const C aLs = ax * Lsx + ay * Lsy + az * Lsz;
    pg[0] += rho * S.L0 + sLs * ir - aLs - (C)0.5 * S.sum_pair - S.rest;
    pg[1] += S.L1x * sx + S.L1y * sy + S.L1z * sz - (C)0.5 * rho * L1a + (C)0.5 * S.dif_pair;
    pg[2] += (C)0.5 * rho * dsx + c1 * rho * S.L1x + (C)2 * c2 * Lsx + dax_seed;
    pg[3] += (C)0.5 * rho * dsy + c1 * rho * S.L1y + (C)2 * c2 * Lsy + day_seed;
    pg[4] += (C)0.5 * rho * dsz + c1 * rho * S.L1z + (C)2 * c2 * Lsz + daz_seed;
}

// block sum of the five sensitivities, added by one thread into this block's
// own double slot (slots are summed on the host after the sweep: no atomics,
// and the result does not depend on scheduling)
template <class C> __device__ __forceinline__ void block_sensitivities(C *pg, double *slot) {
    __shared__ C sm[5][4];
    const int tid = (int)(threadIdx.y * blockDim.x + threadIdx.x);
    const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        C v = pg[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sm[c][wid] = v;
    }
    __syncthreads();
    // blocks have 3 warps (96-site rows, nz = 96) or 4
    const int nw = (int)(blockDim.x * blockDim.y + 31) >> 5;
    if (tid < 5) {
        double v = 0.0;
        for (int w = 0; w < nw; ++w) v += (double)sm[tid][w];
        slot[tid] += v;
    }
}

// resident 128-thread blocks per SM asked of the register allocator (the
// seeding launch, which also forms the loss gradient, gets one fewer)
#ifndef JLB_ADJ_MIN_BLOCKS
#define JLB_ADJ_MIN_BLOCKS 6
#endif
#ifndef JLB_ADJ_MIN_BLOCKS_SEED
#define JLB_ADJ_MIN_BLOCKS_SEED 5
#endif
template <class ST, bool SEED> constexpr int adj_min_blocks() {
    return ST::shifted ? (SEED ? JLB_ADJ_MIN_BLOCKS_SEED : JLB_ADJ_MIN_BLOCKS) : 1;
}

// Dense sites.  Their collision inputs are gathered from the state before the
// step (A.snap) exactly as the forward step gathers them; the adjoint of the
// outputs sits where the forward step wrote (same address maps).
template <class ST, int SCH, bool PSTEP, bool SEED, class IT>
__device__ __forceinline__ void adjoint_dense_sites(const AdjArgs &A, int b, typename ST::C *pg) {
    using S = typename ST::S;
    using C = typename ST::C;
    const StepArgs &a = A.s;
    const int kb = b % a.kblocks, rb = b / a.kblocks;
    const int row = rb * a.by + (int)threadIdx.y;
    const int k = kb * a.bx + (int)threadIdx.x;
    if (row < a.nx * a.ny && k < a.nz) {
        const IT n = (IT)row * a.nz + k;
        const uint8_t cls = __ldg(a.ncls + n);
        if (cls < CLS_SPECIAL) {
            const uint32_t m = (PSTEP && cls == CLS_WALL) ? __ldg(a.nmask + n) : 0u;
            const IT Np = (IT)a.Np;
            const int i = row / a.ny, j = row - i * a.ny;
            IT dI[3], dJ[3], dK[3];
            if (PSTEP) {
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
            const S *snap = (const S *)A.snap;
            S *lam = (S *)A.lam;
            // forward read (r) and write (w) element of population q
            auto rd = [&]<int q>() -> IT {
                if (!PSTEP || q == 9) return (IT)q * Np + n;
                const IT src = n + dI[1 - CX(q)] + dJ[1 - CY(q)] + dK[1 - CZ(q)];
                return (m & (1u << q)) ? (IT)q * Np + n : (IT)OPP(q) * Np + src;
            };
            auto wr = [&]<int q>() -> IT {
                if (!PSTEP) return (IT)OPP(q) * Np + n;
                if (q == 9) return (IT)9 * Np + n;
                const IT dst = n + dI[1 + CX(q)] + dJ[1 + CY(q)] + dK[1 + CZ(q)];
                return (m & (1u << OPP(q))) ? (IT)OPP(q) * Np + n : (IT)q * Np + dst;
            };
            AdjSums<C, ST::shifted, SCH == SCH_REG> sums;
            C lo[Q];
            {
                C g[Q];
                Unroll<0, Q>::run([&]<int q>() {
                    g[q] = ST::template ld<q>(snap + rd.template operator()<q>());
                    lo[q] = (C)lam[wr.template operator()<q>()];
                });
                adj_accumulate(sums, g, lo);
            }
            const double *tg = nullptr;
            const bool on_plane = SEED && i == A.plane;
            if (on_plane) tg = A.target + 3 * ((int64_t)j * a.nz + k);
            adj_finish<C, ST::shifted, SCH, SEED>(sums, lo, arg_g<C>(a, 0), arg_g<C>(a, 1),
                                                 arg_g<C>(a, 2), arg_we<C>(a),
                                                 arg_wo<C>(a), pg, on_plane, tg, a.g[0], a.g[1], a.g[2],
                                                 [&]<int q>(C v) { lam[rd.template operator()<q>()] = (S)v; });
        }
    }
}

// Boundary sites: collision inputs from the recompute's copy (A.sp_in),
// transposed Zou-He after the transposed collision.
template <class ST, int SCH, bool PSTEP, bool SEED>
__device__ __forceinline__ void adjoint_boundary_sites(const AdjArgs &A, int b, typename ST::C *pg) {
    using S = typename ST::S;
    using C = typename ST::C;
    const StepArgs &a = A.s;
    const int tid = (int)(threadIdx.y * blockDim.x + threadIdx.x);
    const int t = b * (int)(blockDim.x * blockDim.y) + tid;
    const int M = a.M;
    if (t < M) {
        const int64_t Np = a.Np;
        const int64_t n = __ldg(a.sp_node + t);
        const int i = (int)(n / ((int64_t)a.ny * a.nz));
        const int j = (int)((n / a.nz) % a.ny), k = (int)(n % a.nz);
        const S *gin = (const S *)A.sp_in;
        S *lam = (S *)A.lam;
        C g[Q], lo[Q], li[Q];
        Unroll<0, Q>::run([&]<int q>() {
            g[q] = ST::template ld<q>(gin + (int64_t)q * M + t);
            const int64_t w = PSTEP ? __ldg(a.sp_wr + (int64_t)q * M + t) : (int64_t)OPP(q) * Np + n;
            lo[q] = (C)lam[w];
        });
        const double *tg = nullptr;
        const bool on_plane = SEED && i == A.plane;
        if (on_plane) tg = A.target + 3 * ((int64_t)j * a.nz + k);
        AdjSums<C, ST::shifted, SCH == SCH_REG> sums;
        adj_accumulate(sums, g, lo);
        adj_finish<C, ST::shifted, SCH, SEED>(sums, lo, arg_g<C>(a, 0), arg_g<C>(a, 1),
                                             arg_g<C>(a, 2), arg_we<C>(a), arg_wo<C>(a),
                                             pg, on_plane, tg, a.g[0], a.g[1], a.g[2],
                                             [&]<int q>(C v) { li[q] = v; });
        C *lam_den = (C *)A.lam_den;
        if (lam_den) {
            // the density this step stored for the next step's moving-wall
            // links is the sum of the collision inputs
            const C ld = lam_den[t];
            Unroll<0, Q>::run([&]<int q>() { li[q] += ld; });
        }
        const uint32_t info = __ldg(a.sp_info + t);
        const uint32_t faces = (info >> SP_FACE_SHIFT) & 0x3Fu;
        // faces were applied in increasing order, so transpose in decreasing
        int slots[6], nf = 0;
        for (int fc = 0; fc < 6; ++fc)
            if (faces & (1u << fc)) slots[fc] = nf++;
        for (int fc = 5; fc >= 0; --fc) {
            if (!(faces & (1u << fc))) continue;
            const double *bcd = a.sp_bc + (int64_t)(4 * slots[fc]) * M + t;
            double du[3] = {0, 0, 0}, dden = 0.0;
            zh_adjoint<C, ST::shifted>(fc, a.bc[fc], bcd[0], bcd[M], bcd[2 * (int64_t)M], bcd[3 * (int64_t)M], g,
                                       li, du, dden);
            // one thread per boundary site: plain adds are race-free
            if (A.grad_bc && ((A.param_faces >> fc) & 1u)) {
                A.grad_bc[t] += dden;
                for (int c = 0; c < 3; ++c) A.grad_bc[(int64_t)(1 + c) * M + t] += du[c];
            }
        }
        if (lam_den) {
            // Ladd's term of a moving link, g_q = f + 6 w_q den_prev (c_q . u_wall),
            // passes its adjoint to the density of the previous step
            C ld = 0;
            Unroll<0, Q>::run([&]<int q>() {
                if (q != 9 && (info & (1u << q)))
                    ld += li[q] * (C)(6.0 * WQ<q>()) * (C)__ldg(a.sp_lw + (int64_t)q * M + t);
            });
            lam_den[t] = ld;
        }
        Unroll<0, Q>::run([&]<int q>() {
            const int64_t r = PSTEP ? __ldg(a.sp_rd + (int64_t)q * M + t) : (int64_t)q * Np + n;
            lam[r] = (S)li[q];
        });
    }
}

int adjoint_blocks(const StepArgs &a) { return a.nb_dense + special_blocks(a); }

// One step of the reverse sweep: blocks [0, nb_dense) take the dense sites,
// the rest the boundary sites (disjoint address sets, as in the forward step).
template <class ST, int SCH, bool PSTEP, bool SEED, class IT>
__global__ void __launch_bounds__(128, adj_min_blocks<ST, SEED>()) adjoint_step_kernel(const AdjArgs A) {
    using C = typename ST::C;
    C pg[5] = {0, 0, 0, 0, 0};
    const int b = (int)blockIdx.x;
    if (b < A.s.nb_dense) adjoint_dense_sites<ST, SCH, PSTEP, SEED, IT>(A, b, pg);
    else adjoint_boundary_sites<ST, SCH, PSTEP, SEED>(A, b - A.s.nb_dense, pg);
    block_sensitivities<C>(pg, A.part + 5 * (int64_t)b);
}

template <class ST, int SCH, bool PSTEP, bool SEED>
int launch_adjoint_typed(const AdjArgs &A, cudaStream_t st) {
    const StepArgs &a = A.s;
    const int blocks = adjoint_blocks(a);
    if (blocks == 0) return 0;
    const dim3 blk(a.bx, a.by), grd(blocks);
    if (a.Np * 19 > 0x7fffffffLL) adjoint_step_kernel<ST, SCH, PSTEP, SEED, int64_t><<<grd, blk, 0, st>>>(A);
    else adjoint_step_kernel<ST, SCH, PSTEP, SEED, int32_t><<<grd, blk, 0, st>>>(A);
    return (int)cudaGetLastError();
}

template <class ST, int SCH>
int launch_adjoint_scheme(const AdjArgs &A, bool pstep, bool seed, cudaStream_t st) {
    if (pstep) return seed ? launch_adjoint_typed<ST, SCH, true, true>(A, st) : launch_adjoint_typed<ST, SCH, true, false>(A, st);
    return seed ? launch_adjoint_typed<ST, SCH, false, true>(A, st) : launch_adjoint_typed<ST, SCH, false, false>(A, st);
}

int launch_adjoint_step(const AdjArgs &A, int prec, int scheme, bool pstep, cudaStream_t st) {
    const bool seed = A.seed != 0;
    if (prec == PREC_FP64)
        return scheme == SCH_TRT   ? launch_adjoint_scheme<StoreF64, SCH_TRT>(A, pstep, seed, st)
               : scheme == SCH_REG ? launch_adjoint_scheme<StoreF64, SCH_REG>(A, pstep, seed, st)
                                   : launch_adjoint_scheme<StoreF64, SCH_BGK>(A, pstep, seed, st);
    return scheme == SCH_TRT   ? launch_adjoint_scheme<StoreF32, SCH_TRT>(A, pstep, seed, st)
           : scheme == SCH_REG ? launch_adjoint_scheme<StoreF32, SCH_REG>(A, pstep, seed, st)
                               : launch_adjoint_scheme<StoreF32, SCH_BGK>(A, pstep, seed, st);
}

} // namespace jlb
