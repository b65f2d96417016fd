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
// their transpose comes for free.  The collision inputs of the step (after
// Zou-He) come from the forward recompute (StepArgs::tee).
//
// Collision (BGK / TRT with forcing, jyulb/D3Q19.pyx:655-853):
//   rho = sum g, j = sum c g, s = j + rho a / 2,
//   H0 = we rho, H1 = wo s + c1 rho a, H2 = we s s / rho + c2 (a s + s a),
//   f*_q = c3 g_q - c4 g_opp(q) + P_q(H),  f*_rest = (1 - we) g_rest + P_rest(H),
// with c1 = 1 - wo/2, c2 = 1 - we/2, c3 = 1 - (we + wo)/2, c4 = (we - wo)/2
// (BGK: wo = we) and P_q(H) = w_q (H0 + 3 c.H1 + 4.5 (c c - I/3):H2).
// Its transpose and the local sensitivities to we, wo and a are written out
// below.  Zou-He is affine in the populations and in j, so its transpose is
// read off the forward assignment applied to unit vectors.
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
// mu the adjoint w.r.t. the pre-Zou-He populations and adds du (adjoint of the
// boundary velocity) for a FIXED_VEL face.
template <class C, bool SHIFTED>
__device__ void zh_adjoint(int fc, int kind, double den, double ux, double uy, double uz, const C *gp, C *mu,
                           double *du) {
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
        // j_n = +/-(S - den), j_t = den u_t
        dS = high ? dj[ax] : -dj[ax];
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

// transposed collision; g: collision inputs (shifted by w when SHIFTED),
// lo: adjoint of the outputs, li: adjoint of the inputs (out), pg: local
// sensitivities to we, wo, ax, ay, az (accumulated), and the stored-velocity
// seed of the loss (du_loss, or nullptr)
template <class C, bool SHIFTED, int SCH>
__device__ void coll_adjoint(const C *g, const C *lo, C ax, C ay, C az, C we, C wo, C *li, double *pg,
                             const double *du_loss) {
    if (SCH == SCH_BGK) wo = we;
    C rho = SHIFTED ? (C)1 : (C)0, jx = 0, jy = 0, jz = 0;
    C L0 = 0, L1x = 0, L1y = 0, L1z = 0;
    C Lxx = 0, Lyy = 0, Lzz = 0, Lxy = 0, Lxz = 0, Lyz = 0;
    Unroll<0, Q>::run([&]<int q>() {
        constexpr C w = (C)WQ<q>();
        constexpr int cx = CX(q), cy = CY(q), cz = CZ(q);
        rho += g[q];
        if (cx) jx += (C)cx * g[q];
        if (cy) jy += (C)cy * g[q];
        if (cz) jz += (C)cz * g[q];
        const C wl = w * lo[q];
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
    });
    const C c1 = (C)1 - (C)0.5 * wo, c2 = (C)1 - (C)0.5 * we;
    const C c3 = (C)1 - (C)0.5 * (we + wo), c4 = (C)0.5 * (we - wo);
    const C sx = jx + (C)0.5 * rho * ax, sy = jy + (C)0.5 * rho * ay, sz = jz + (C)0.5 * rho * az;
    const C Lsx = Lxx * sx + Lxy * sy + Lxz * sz;
    const C Lsy = Lxy * sx + Lyy * sy + Lyz * sz;
    const C Lsz = Lxz * sx + Lyz * sy + Lzz * sz;
    const C Lax = Lxx * ax + Lxy * ay + Lxz * az;
    const C Lay = Lxy * ax + Lyy * ay + Lyz * az;
    const C Laz = Lxz * ax + Lyz * ay + Lzz * az;
    const C ir = (C)1 / rho;
    const C dsx = wo * L1x + (C)2 * we * Lsx * ir + (C)2 * c2 * Lax;
    const C dsy = wo * L1y + (C)2 * we * Lsy * ir + (C)2 * c2 * Lay;
    const C dsz = wo * L1z + (C)2 * we * Lsz * ir + (C)2 * c2 * Laz;
    const C sLs = sx * Lsx + sy * Lsy + sz * Lsz;
    C drho = we * L0 + c1 * (L1x * ax + L1y * ay + L1z * az) - we * sLs * ir * ir +
             (C)0.5 * (ax * dsx + ay * dsy + az * dsz);
    C djx = dsx, djy = dsy, djz = dsz;
    // loss seed: stored u = j/rho + a/2
    double dax_seed = 0, day_seed = 0, daz_seed = 0;
    if (du_loss) {
        const C ux = jx * ir, uy = jy * ir, uz = jz * ir;
        const C d0 = (C)du_loss[0], d1 = (C)du_loss[1], d2 = (C)du_loss[2];
        djx += d0 * ir; djy += d1 * ir; djz += d2 * ir;
        drho -= (d0 * ux + d1 * uy + d2 * uz) * ir;
        dax_seed = 0.5 * du_loss[0]; day_seed = 0.5 * du_loss[1]; daz_seed = 0.5 * du_loss[2];
    }
    C sum_pair = 0, dif_pair = 0;
    Unroll<0, Q>::run([&]<int q>() {
        constexpr int cx = CX(q), cy = CY(q), cz = CZ(q);
        C v;
        if (q == 9) v = ((C)1 - we) * lo[9];
        else v = c3 * lo[q] - c4 * lo[OPP(q)];
        v += drho;
        if (cx) v += (C)cx * djx;
        if (cy) v += (C)cy * djy;
        if (cz) v += (C)cz * djz;
        li[q] = v;
        if (q != 9) {
            constexpr C w = (C)WQ<q>();
            const C fq = g[q] + (SHIFTED ? w : (C)0), fo = g[OPP(q)] + (SHIFTED ? w : (C)0);
            sum_pair += lo[q] * (fq + fo);
            dif_pair += lo[q] * (fo - fq);
        }
    });
    const C f9 = g[9] + (SHIFTED ? (C)WQ<9>() : (C)0);
    const C aLs = ax * Lsx + ay * Lsy + az * Lsz;
    const double dwe = (double)(rho * L0 + sLs * ir - aLs - (C)0.5 * sum_pair - lo[9] * f9);
    const double dwo = (double)(L1x * sx + L1y * sy + L1z * sz - (C)0.5 * rho * (L1x * ax + L1y * ay + L1z * az) +
                                (C)0.5 * dif_pair);
    pg[0] += dwe;
    pg[1] += dwo;
    pg[2] += (double)((C)0.5 * rho * dsx + c1 * rho * L1x + (C)2 * c2 * Lsx) + dax_seed;
    pg[3] += (double)((C)0.5 * rho * dsy + c1 * rho * L1y + (C)2 * c2 * Lsy) + day_seed;
    pg[4] += (double)((C)0.5 * rho * dsz + c1 * rho * L1z + (C)2 * c2 * Lsz) + daz_seed;
}

template <class ST, int SCH>
__device__ __forceinline__ void adj_node(const AdjArgs &A, bool pstep, bool special, int64_t n, int t_sp,
                                         uint32_t m, int i, int j, int k, double *pg) {
    using S = typename ST::S;
    using C = typename ST::C;
    const StepArgs &a = A.s;
    const int64_t Np = a.Np;
    S *lam = (S *)A.lam;
    const S *gin = (const S *)A.gin;
    C g[Q], lo[Q], li[Q];
    // dense-node neighbour offsets (periodic wrap), as in the forward step
    int64_t dI[3] = {0, 0, 0}, dJ[3] = {0, 0, 0}, dK[3] = {0, 0, 0};
    if (pstep && !special) {
        const int64_t sI = (int64_t)a.ny * a.nz, sJ = a.nz;
        dI[0] = (i == 0 ? (int64_t)(a.nx - 1) : -1) * sI; dI[2] = (i + 1 == a.nx ? (int64_t)(1 - a.nx) : 1) * sI;
        dJ[0] = (j == 0 ? (int64_t)(a.ny - 1) : -1) * sJ; dJ[2] = (j + 1 == a.ny ? (int64_t)(1 - a.ny) : 1) * sJ;
        dK[0] = k == 0 ? (int64_t)(a.nz - 1) : -1;         dK[2] = k + 1 == a.nz ? (int64_t)(1 - a.nz) : 1;
    }
    const int M = a.M;
    Unroll<0, Q>::run([&]<int q>() {
        g[q] = ST::template ld<q>(gin + (int64_t)q * Np + n);
        // adjoint of output q sits where the forward step wrote f*_q
        int64_t w;
        if (!pstep) w = (int64_t)OPP(q) * Np + n;
        else if (special) w = __ldg(a.sp_wr + (int64_t)q * M + t_sp);
        else if (q == 9) w = 9 * Np + n;
        else if (m & (1u << OPP(q))) w = (int64_t)OPP(q) * Np + n;
        else w = (int64_t)q * Np + n + dI[1 + CX(q)] + dJ[1 + CY(q)] + dK[1 + CZ(q)];
        lo[q] = (C)lam[w];
    });
    const double *du_loss = nullptr;
    double dl[3];
    if (A.seed && i == A.plane) {
        const double *tg = A.target + 3 * ((int64_t)j * a.nz + k);
        // stored velocity of the collision input
        C rho = ST::shifted ? (C)1 : (C)0, jx = 0, jy = 0, jz = 0;
        Unroll<0, Q>::run([&]<int q>() {
            rho += g[q];
            if (CX(q)) jx += (C)CX(q) * g[q];
            if (CY(q)) jy += (C)CY(q) * g[q];
            if (CZ(q)) jz += (C)CZ(q) * g[q];
        });
        const double u0 = (double)(jx / rho) + 0.5 * a.g[0], u1 = (double)(jy / rho) + 0.5 * a.g[1],
                     u2 = (double)(jz / rho) + 0.5 * a.g[2];
        dl[0] = 2.0 * (u0 - tg[0]); dl[1] = 2.0 * (u1 - tg[1]); dl[2] = 2.0 * (u2 - tg[2]);
        du_loss = dl;
    }
    coll_adjoint<C, ST::shifted, SCH>(g, lo, (C)a.g[0], (C)a.g[1], (C)a.g[2], (C)a.w_e, (C)a.w_o, li, pg, du_loss);
    if (special) {
        const uint32_t info = __ldg(a.sp_info + t_sp);
        const uint32_t faces = (info >> SP_FACE_SHIFT) & 0x3Fu;
        // faces were applied in increasing order, so transpose in decreasing
        int slots[6], nf = 0;
        for (int fc = 0; fc < 6; ++fc)
            if (faces & (1u << fc)) slots[fc] = nf++;
        for (int fc = 5; fc >= 0; --fc) {
            if (!(faces & (1u << fc))) continue;
            const double *bcd = a.sp_bc + (int64_t)(4 * slots[fc]) * M + t_sp;
            double du[3] = {0, 0, 0};
            zh_adjoint<C, ST::shifted>(fc, a.bc[fc], bcd[0], bcd[M], bcd[2 * (int64_t)M], bcd[3 * (int64_t)M], g,
                                       li, du);
            if (fc == 0 && a.bc[0] == BC_FIXED_VEL && A.grad_uin) A.grad_uin[(int64_t)j * a.nz + k] += du[0];
        }
    }
    Unroll<0, Q>::run([&]<int q>() {
        // adjoint of input q goes where the forward step read g_q
        int64_t r;
        if (!pstep) r = (int64_t)q * Np + n;
        else if (special) r = __ldg(a.sp_rd + (int64_t)q * M + t_sp);
        else if (q == 9) r = 9 * Np + n;
        else if (m & (1u << q)) r = (int64_t)q * Np + n;
        else r = (int64_t)OPP(q) * Np + n + dI[1 - CX(q)] + dJ[1 - CY(q)] + dK[1 - CZ(q)];
        lam[r] = (S)li[q];
    });
}

template <class ST, int SCH>
__global__ void __launch_bounds__(128) adjoint_step_kernel(const AdjArgs A, int pstep) {
    const StepArgs &a = A.s;
    double pg[5] = {0, 0, 0, 0, 0};
    const int b = (int)blockIdx.x;
    const int tid = (int)(threadIdx.y * blockDim.x + threadIdx.x);
    if (b < a.nb_dense) {
        const int kb = b % a.kblocks, rb = b / a.kblocks;
        const int row = rb * a.by + (int)threadIdx.y;
        const int k = kb * a.bx + (int)threadIdx.x;
        if (row < a.nx * a.ny && k < a.nz) {
            const int64_t n = (int64_t)row * a.nz + k;
            const uint32_t m = a.nmask[n];
            if (!(m & MASK_SKIP)) adj_node<ST, SCH>(A, pstep != 0, false, n, 0, m, row / a.ny, row % a.ny, k, pg);
        }
    } else {
        const int t = (b - a.nb_dense) * (int)(blockDim.x * blockDim.y) + tid;
        if (t < a.M) {
            const int64_t n = a.sp_node[t];
            const int i = (int)(n / ((int64_t)a.ny * a.nz));
            const int j = (int)((n / a.nz) % a.ny), k = (int)(n % a.nz);
            adj_node<ST, SCH>(A, pstep != 0, true, n, t, 0u, i, j, k, pg);
        }
    }
    // block sums of the parameter sensitivities, one atomic per block and component
    __shared__ double sm[5][4];
    const int lane = tid & 31, wid = tid >> 5;
#pragma unroll
    for (int c = 0; c < 5; ++c) {
        double v = pg[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) sm[c][wid] = v;
    }
    __syncthreads();
    if (tid < 5) {
        const double v = sm[tid][0] + sm[tid][1] + sm[tid][2] + sm[tid][3];
        if (v != 0.0) atomicAdd(A.grad + tid, v);
    }
}

int launch_adjoint_step(const AdjArgs &A, int prec, int scheme, bool pstep, int blocks, cudaStream_t st) {
    dim3 blk(A.s.bx, A.s.by), grd(blocks);
    if (prec == PREC_FP64) {
        if (scheme == SCH_TRT) adjoint_step_kernel<StoreF64, SCH_TRT><<<grd, blk, 0, st>>>(A, pstep);
        else adjoint_step_kernel<StoreF64, SCH_BGK><<<grd, blk, 0, st>>>(A, pstep);
    } else {
        if (scheme == SCH_TRT) adjoint_step_kernel<StoreF32, SCH_TRT><<<grd, blk, 0, st>>>(A, pstep);
        else adjoint_step_kernel<StoreF32, SCH_BGK><<<grd, blk, 0, st>>>(A, pstep);
    }
    return (int)cudaGetLastError();
}

} // namespace jlb
