// lbm_cxx.cu -- the reference C++ executable's collision model as a physics
// policy of the fused step, with its initial state.
//
// The executable (include/kernel/kernel.cpp:410-550) computes, per fluid
// site: moments rho, j (include/dvs/D3Q19.h:480-509), the force density
// F = F_ext + rho g, the velocity u = j/rho + F/(2 rho), a forcing term
// (first order, D3Q19.h:370-410, or second order with u, D3Q19.h:414-475),
// an equilibrium (linear "Stokes", D3Q19.h:257-299, or quadratic, :303-365)
// and relaxes with BGK or TRT (include/collision/collision.cpp:26-232).
// Its directions are named (B/T = -z/+z, S/N = -y/+y, W/E = -x/+x); below
// they are mapped onto this engine's lattice order.  The unit is compiled
// with -fmad=false and every expression keeps the executable's evaluation
// order, so FP64 results match the executable's bit for bit.  Only resting
// solids and periodic / wall faces exist in that model; the host rejects
// anything that would need Zou-He or moving-wall terms.
#include "lbm_step.cuh"
#include "lbm_aux.h"

namespace jlb {

namespace cxx {
// the executable's direction names -> this engine's q
constexpr int BS = 5, BW = 1, B = 8, BE = 15, BN = 11, SW = 0, S = 6, SE = 14, W = 2, C0 = 9, E = 16, NW = 4,
              N = 12, NE = 18, TS = 7, TW = 3, T = 10, TE = 17, TN = 13;
// the nine pairs in the executable's order; the first member carries the
// sign of the odd part
constexpr int PAIR_FIRST[9] = {BS, BW, B, BE, BN, SW, S, SE, W};
constexpr double WEQ0 = 12.0 / 36.0, WEQ1 = 2.0 / 36.0, WEQ2 = 1.0 / 36.0;

struct Consts {
    double ct2, inv_ct2, cff2;
};
__device__ __forceinline__ Consts consts() {
    // CT = 1/sqrt(3) and its square as the executable forms them
    // (D3Q19.h:206-208): CT2 is not exactly 1/3, nor INV_CT2 exactly 3
    const double ct = 1.0 / sqrt(3.0);
    Consts k;
    k.ct2 = ct * ct;
    k.inv_ct2 = 1.0 / k.ct2;
    k.cff2 = 0.5 * k.inv_ct2 * k.inv_ct2;
    return k;
}

template <int q> __device__ constexpr double wq() {
    return NNZ(q) == 0 ? WEQ0 : (NNZ(q) == 1 ? WEQ1 : WEQ2);
}

// c_q . v for a first pair member, as a single signed sum of the nonzero
// components in x, y, z order (a negated sum is exact, so this equals the
// executable's (-w/cs^2)(a + b) and (w/cs^2)(a - b) forms bit for bit)
template <int q> __device__ __forceinline__ double cdot(double x, double y, double z) {
    constexpr int cx = CX(q), cy = CY(q), cz = CZ(q);
    double s = 0.0;
    bool first = true;
    auto add = [&](int c, double v) {
        if (!c) return;
        const double t = c > 0 ? v : -v;
        s = first ? t : s + t;
        first = false;
    };
    add(cx, x);
    add(cy, y);
    add(cz, z);
    return s;
}

// even part of a pair for the second-order terms: w (cmmn + m_aa + m_bb
// +- 2 m_ab), components in x, y, z order
template <int q> __device__ __forceinline__ double even2(double cmmn, const double *m2) {
    // m2: xx, yy, zz, xy, xz, yz
    constexpr int cx = CX(q), cy = CY(q), cz = CZ(q);
    constexpr double w = wq<q>();
    if (cx && cy) return w * (cmmn + m2[0] + m2[1] + (cx * cy > 0 ? 2.0 * m2[3] : -(2.0 * m2[3])));
    if (cx && cz) return w * (cmmn + m2[0] + m2[2] + (cx * cz > 0 ? 2.0 * m2[4] : -(2.0 * m2[4])));
    if (cy && cz) return w * (cmmn + m2[1] + m2[2] + (cy * cz > 0 ? 2.0 * m2[5] : -(2.0 * m2[5])));
    if (cx) return w * (cmmn + m2[0]);
    if (cy) return w * (cmmn + m2[1]);
    return w * (cmmn + m2[2]);
}
}  // namespace cxx

// EQ2: quadratic equilibrium (else linear); FRC2: second-order forcing
// (else first order)
template <int SCH, bool EQ2, bool FRC2> struct PhysCxx {
    using C = double;
    static constexpr bool force_density = true;

    // never reached: the host admits no boundary node in this model
    template <int q> __device__ static C ladd(C v, C, C) { return v; }
    __device__ static void zou_he(int, int, double, double, double, double, C *) {}

    __device__ static C moments(const C *f, C &ux, C &uy, C &uz, C &inv_den) {
        using namespace cxx;
        const C neg_z = f[BS] + f[BW] + f[B] + f[BE] + f[BN];
        const C pos_z = f[TS] + f[TW] + f[T] + f[TE] + f[TN];
        const C neg_y = f[SW] + f[S] + f[SE];
        const C pos_y = f[NW] + f[N] + f[NE];
        const C den = neg_z + neg_y + pos_y + pos_z + f[W] + f[C0] + f[E];
        inv_den = 1.0 / den;
        ux = inv_den * ((f[BE] + f[SE] + f[E] + f[NE] + f[TE]) - (f[BW] + f[SW] + f[W] + f[NW] + f[TW]));
        uy = inv_den * ((pos_y + f[BN] + f[TN]) - (neg_y + f[BS] + f[TS]));
        uz = inv_den * (pos_z - neg_z);
        return den;
    }

    __device__ static void equilibrium(const cxx::Consts &k, C den, C ux, C uy, C uz, C *feq) {
        using namespace cxx;
        const C jx = den * ux, jy = den * uy, jz = den * uz;
        if (EQ2) {
            C m2[6];
            m2[0] = k.cff2 * jx * ux; m2[1] = k.cff2 * jy * uy; m2[2] = k.cff2 * jz * uz;
            m2[3] = k.cff2 * jx * uy; m2[4] = k.cff2 * jx * uz; m2[5] = k.cff2 * jy * uz;
            const C cmmn = den - k.ct2 * (m2[0] + m2[1] + m2[2]);
            Unroll<0, 9>::run([&]<int p>() {
                constexpr int q = PAIR_FIRST[p];
                const C o = (wq<q>() * k.inv_ct2) * cdot<q>(jx, jy, jz);
                const C e = even2<q>(cmmn, m2);
                feq[q] = e + o;
                feq[OPP(q)] = e - o;
            });
            feq[C0] = WEQ0 * cmmn;
        } else {
            const C c1 = WEQ1 * den, c2 = WEQ2 * den;
            Unroll<0, 9>::run([&]<int p>() {
                constexpr int q = PAIR_FIRST[p];
                const C o = (wq<q>() * k.inv_ct2) * cdot<q>(jx, jy, jz);
                const C e = NNZ(q) == 1 ? c1 : c2;
                feq[q] = e + o;
                feq[OPP(q)] = e - o;
            });
            feq[C0] = WEQ0 * den;
        }
    }

    __device__ static void forcing(const cxx::Consts &k, C ux, C uy, C uz, C fx, C fy, C fz, C *fe) {
        using namespace cxx;
        if (FRC2) {
            C m2[6];
            const C c2 = k.cff2 * 2.0;
            m2[0] = c2 * fx * ux; m2[1] = c2 * fy * uy; m2[2] = c2 * fz * uz;
            m2[3] = k.cff2 * (fx * uy + fy * ux);
            m2[4] = k.cff2 * (fx * uz + fz * ux);
            m2[5] = k.cff2 * (fy * uz + fz * uy);
            const C cmmn = -k.ct2 * (m2[0] + m2[1] + m2[2]);
            Unroll<0, 9>::run([&]<int p>() {
                constexpr int q = PAIR_FIRST[p];
                const C o = (wq<q>() * k.inv_ct2) * cdot<q>(fx, fy, fz);
                const C e = even2<q>(cmmn, m2);
                fe[q] = e + o;
                fe[OPP(q)] = e - o;
            });
            fe[C0] = WEQ0 * cmmn;
        } else {
            Unroll<0, 9>::run([&]<int p>() {
                constexpr int q = PAIR_FIRST[p];
                const C o = (wq<q>() * k.inv_ct2) * cdot<q>(fx, fy, fz);
                fe[q] = o;
                fe[OPP(q)] = -o;
            });
            fe[C0] = 0.0;
        }
    }

    // collision.cpp:26-58 (BGK) and :77-232 (TRT)
    __device__ static void relax(C *f, const C *feq, const C *fe, C we, C wo) {
        using namespace cxx;
        if (SCH == SCH_BGK) {
            const C r = 1.0 - 0.5 * we;
#pragma unroll
            for (int q = 0; q < Q; ++q) f[q] = f[q] - we * (f[q] - feq[q]) + r * fe[q];
        } else {
            const C re = 1.0 - 0.5 * we, ro = 1.0 - 0.5 * wo;
            Unroll<0, 9>::run([&]<int p>() {
                constexpr int q = PAIR_FIRST[p], o = OPP(PAIR_FIRST[p]);
                const C nq = f[q] - feq[q], no = f[o] - feq[o];
                const C ev = 0.5 * (nq + no), od = 0.5 * (nq - no);
                const C fev = 0.5 * (fe[q] + fe[o]), fod = 0.5 * (fe[q] - fe[o]);
                const C rl_e = we * ev - re * fev, rl_o = wo * od - ro * fod;
                f[q] = f[q] - rl_e - rl_o;
                f[o] = f[o] - rl_e + rl_o;
            });
            f[C0] = f[C0] - we * (f[C0] - feq[C0]) + re * fe[C0];
        }
    }

    // kernel.cpp:480-506: returns rho; u is the stored velocity j/rho + F/(2 rho)
    __device__ static C collide_fd(C *f, C gx, C gy, C gz, C fx, C fy, C fz, C we, C wo, C &ux, C &uy, C &uz) {
        const cxx::Consts k = cxx::consts();
        C inv_den;
        const C den = moments(f, ux, uy, uz, inv_den);
        fx = fx + den * gx; fy = fy + den * gy; fz = fz + den * gz;
        ux = ux + 0.5 * inv_den * fx; uy = uy + 0.5 * inv_den * fy; uz = uz + 0.5 * inv_den * fz;
        C fe[Q], feq[Q];
        forcing(k, ux, uy, uz, fx, fy, fz, fe);
        equilibrium(k, den, ux, uy, uz, feq);
        relax(f, feq, fe, we, wo);
        return den;
    }
};

template <int SCH, bool EQ2, bool FRC2>
int launch_cxx_typed(const StepArgs &a, bool pstep, bool accf, int blocks, cudaStream_t st) {
    dim3 blk(a.bx, a.by), grd(blocks);
    const bool i64 = a.Np * 19 > 0x7fffffffLL;
    using PH = PhysCxx<SCH, EQ2, FRC2>;
#define JLB_CX(P, A)                                                                             \
    do {                                                                                         \
        if (i64) lbm_step_kernel<StoreF64, PH, P, A, int64_t><<<grd, blk, 0, st>>>(a);           \
        else lbm_step_kernel<StoreF64, PH, P, A, int32_t><<<grd, blk, 0, st>>>(a);               \
    } while (0)
    if (pstep) { if (accf) JLB_CX(true, true); else JLB_CX(true, false); }
    else { if (accf) JLB_CX(false, true); else JLB_CX(false, false); }
#undef JLB_CX
    return (int)cudaGetLastError();
}

int launch_step_cxx(const StepArgs &a, int scheme, int opts, bool pstep, bool accf, int blocks, cudaStream_t st) {
    const bool eq2 = !(opts & CXX_LINEAR_EQ), frc2 = (opts & CXX_FORCE2) != 0;
#define JLB_CS(SCH)                                                                              \
    if (eq2) return frc2 ? launch_cxx_typed<SCH, true, true>(a, pstep, accf, blocks, st)         \
                         : launch_cxx_typed<SCH, true, false>(a, pstep, accf, blocks, st);       \
    return frc2 ? launch_cxx_typed<SCH, false, true>(a, pstep, accf, blocks, st)                 \
                : launch_cxx_typed<SCH, false, false>(a, pstep, accf, blocks, st);
    if (scheme == SCH_BGK) { JLB_CS(SCH_BGK) }
    JLB_CS(SCH_TRT)
#undef JLB_CS
}

// ---------------------------------------------------------------------------
// initial state (kernel.cpp:239-408): equilibrium of the given rho, u plus
// the non-equilibrium part -2 tau cs^2 rho S from finite-difference velocity
// gradients (one-sided next to solids, zero between two solids), then one
// relaxation with the forcing term of F = F_ext + rho g at the unshifted u.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int64_t cxx_full_idx(const AuxGeom &g, int I, int J, int K) {
    return ((int64_t)I * g.NJ + J) * g.NK + K;
}

// kernel.cpp:261-316 for one axis: d/d_axis of u at (I,J,K)
__device__ void cxx_der(const AuxGeom &g, const uint8_t *phase, const double *vel, int I, int J, int K, int ax,
                        const double *u, double *du) {
    const int dI = ax == 0, dJ = ax == 1, dK = ax == 2;
    const int64_t nf = cxx_full_idx(g, I + dI, J + dJ, K + dK);
    const int64_t nb = cxx_full_idx(g, I - dI, J - dJ, K - dK);
    const bool sf = phase[nf] == 0, sb = phase[nb] == 0;
    for (int d = 0; d < 3; ++d) {
        if (sf) {
            du[d] = sb ? 0.0 : (1.0 / 3.0) * (4.0 * 0.0 - 3.0 * u[d] - vel[3 * nb + d]);
        } else if (sb) {
            du[d] = (1.0 / 3.0) * (vel[3 * nf + d] + 3.0 * u[d] - 4.0 * 0.0);
        } else {
            du[d] = 0.5 * (vel[3 * nf + d] - vel[3 * nb + d]);
        }
    }
}

template <int SCH, bool EQ2, bool FRC2>
__global__ void cxx_init_kernel(AuxGeom g, const uint8_t *phase, const double *den, const double *vel,
                                const double *facc, double gx, double gy, double gz, double tau, double we,
                                double wo, double *f, double *mden, double *mux, double *muy, double *muz) {
    using PH = PhysCxx<SCH, EQ2, FRC2>;
    const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= g.N) return;
    const int i = (int)(n / ((int64_t)g.ny * g.nz));
    const int rem = (int)(n - (int64_t)i * g.ny * g.nz);
    const int j = rem / g.nz, k = rem - (rem / g.nz) * g.nz;
    const int64_t fn = cxx_full_idx(g, i + 1, j + 1, k + 1);
    if (phase[fn] == 0) return;
    const cxx::Consts kc = cxx::consts();
    const double d = den[fn];
    const double u[3] = {vel[3 * fn], vel[3 * fn + 1], vel[3 * fn + 2]};
    double fx = facc ? facc[n] : 0.0, fy = facc ? facc[g.Np + n] : 0.0, fz = facc ? facc[2 * g.Np + n] : 0.0;
    fx = fx + d * gx; fy = fy + d * gy; fz = fz + d * gz;
    double fe[Q], feq[Q], fi[Q];
    PH::forcing(kc, u[0], u[1], u[2], fx, fy, fz, fe);
    PH::equilibrium(kc, d, u[0], u[1], u[2], feq);
    double dx[3], dy[3], dz[3];
    cxx_der(g, phase, vel, i + 1, j + 1, k + 1, 0, u, dx);
    cxx_der(g, phase, vel, i + 1, j + 1, k + 1, 1, u, dy);
    cxx_der(g, phase, vel, i + 1, j + 1, k + 1, 2, u, dz);
    // tau is the relaxation time itself (0.5 + cs^-2 nu), not 1/we
    const double pab = -2.0 * tau * kc.ct2;
    const double pxx = pab * d * dx[0], pxy = pab * d * 0.5 * (dx[1] + dy[0]), pxz = pab * d * 0.5 * (dx[2] + dz[0]);
    const double pyy = pab * d * dy[1], pyz = pab * d * 0.5 * (dy[2] + dz[1]), pzz = pab * d * dz[2];
    Unroll<0, Q>::run([&]<int q>() {
        constexpr double cx = CX(q), cy = CY(q), cz = CZ(q);
        const double w = cxx::wq<q>() * 0.5 * kc.inv_ct2 * kc.inv_ct2;
        const double kxx = w * (cx * cx - kc.ct2), kyy = w * (cy * cy - kc.ct2), kzz = w * (cz * cz - kc.ct2);
        const double kxy = w * (cx * cy), kxz = w * (cx * cz), kyz = w * (cy * cz);
        const double fneq = kxx * pxx + kyy * pyy + kzz * pzz + 2.0 * (kxy * pxy + kxz * pxz + kyz * pyz);
        fi[q] = feq[q] + fneq;
    });
    PH::relax(fi, feq, fe, we, wo);
    // post-collision state: A[opp(q)][x] = f_q(x)
#pragma unroll
    for (int q = 0; q < Q; ++q) f[(int64_t)OPP(q) * g.Np + n] = fi[q];
    mden[n] = d;
    mux[n] = u[0];
    muy[n] = u[1];
    muz[n] = u[2];
}

int aux_init_cxx(const AuxGeom &g, int scheme, int opts, const uint8_t *phase, const double *den,
                 const double *vel, const double *facc, const double gv[3], double tau, double we, double wo,
                 double *f, double *mden, double *mux, double *muy, double *muz, cudaStream_t st) {
    const unsigned b = (unsigned)((g.N + 127) / 128);
    const bool eq2 = !(opts & CXX_LINEAR_EQ), frc2 = (opts & CXX_FORCE2) != 0;
#define JLB_CI(SCH, E2, F2)                                                                                  \
    cxx_init_kernel<SCH, E2, F2><<<b, 128, 0, st>>>(g, phase, den, vel, facc, gv[0], gv[1], gv[2], tau, we, wo, \
                                                   f, mden, mux, muy, muz)
    if (scheme == SCH_BGK) {
        if (eq2) { if (frc2) JLB_CI(SCH_BGK, true, true); else JLB_CI(SCH_BGK, true, false); }
        else { if (frc2) JLB_CI(SCH_BGK, false, true); else JLB_CI(SCH_BGK, false, false); }
    } else {
        if (eq2) { if (frc2) JLB_CI(SCH_TRT, true, true); else JLB_CI(SCH_TRT, true, false); }
        else { if (frc2) JLB_CI(SCH_TRT, false, true); else JLB_CI(SCH_TRT, false, false); }
    }
#undef JLB_CI
    return (int)cudaGetLastError();
}

}  // namespace jlb
