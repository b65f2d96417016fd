// lbm_fp64.cuh -- FP64 helpers of the reference's arithmetic shared by the
// parity step (lbm_fp64.cu, compiled with -fmad=false: every operation a
// separately rounded IEEE add/mul/div in the reference's order) and the fast
// FP64 step (lbm_fp64fast.cu, compiled with contraction): Ladd's moving-wall
// term, the moments, the H10 projection and the Zou-He faces
// (jyulb/D3Q19.pyx:348-940, jyulb/bcs.pyx:31-716,
// jyulb/isothermal.pyx:1112-1248).
#pragma once
#include "lbm_step.cuh"

namespace jlb {

struct Phys64Base {
    using C = double;

    // Ladd's moving-wall term added to a bounced population
    // (jyulb/isothermal.pyx:1117-1119): f + ((2 den) w) 3 * (c . u_wall)
    template <int q> __device__ static C ladd(C v, C den, C s) {
        constexpr double w = NNZ(q) == 1 ? (2.0 / 36.0) : (1.0 / 36.0);
        const C cff = 2.0 * den * w * 3.0;
        return v + cff * s;
    }

    __device__ static C f_to_den_vel(const C *f, C &vx, C &vy, C &vz) {
        C d1x = f[0] + f[1] + f[2] + f[3] + f[4];
        C dx1 = f[14] + f[15] + f[16] + f[17] + f[18];
        C d01y = f[5] + f[6] + f[7];
        C d0y1 = f[11] + f[12] + f[13];
        C den = d1x + dx1 + d01y + d0y1 + f[8] + f[9] + f[10];
        C jx = dx1 - d1x;
        C jy = f[4] + d0y1 + f[18] - f[0] - d01y - f[14];
        C jz = f[3] + f[7] + f[10] + f[13] + f[17] - f[1] - f[5] - f[8] - f[11] - f[15];
        C inv = 1.0 / den;
        vx = inv * jx; vy = inv * jy; vz = inv * jz;
        return den;
    }

    // kinetic projection of the H10 moments; ADD accumulates into f
    template <bool ADD> __device__ static void project(const C *h, C *f) {
        const C c = 1.0 / 72.0;
        C exy = 2.0 * h[0] + 6.0 * h[4] + 6.0 * h[7] - 3.0 * h[9];
        C a0 = exy + 18.0 * h[5], o0 = -6.0 * h[1] - 6.0 * h[2];
        C a4 = exy - 18.0 * h[5], o4 = -6.0 * h[1] + 6.0 * h[2];
        C exz = 2.0 * h[0] + 6.0 * h[4] - 3.0 * h[7] + 6.0 * h[9];
        C a1 = exz + 18.0 * h[6], o1 = -6.0 * h[1] - 6.0 * h[3];
        C a3 = exz - 18.0 * h[6], o3 = -6.0 * h[1] + 6.0 * h[3];
        C eyz = 2.0 * h[0] - 3.0 * h[4] + 6.0 * h[7] + 6.0 * h[9];
        C a5 = eyz + 18.0 * h[8], o5 = -6.0 * h[2] - 6.0 * h[3];
        C a7 = eyz - 18.0 * h[8], o7 = -6.0 * h[2] + 6.0 * h[3];
        C ex = 4.0 * h[0] + 12.0 * h[4] - 6.0 * h[7] - 6.0 * h[9];
        C ey = 4.0 * h[0] - 6.0 * h[4] + 12.0 * h[7] - 6.0 * h[9];
        C ez = 4.0 * h[0] - 6.0 * h[4] - 6.0 * h[7] + 12.0 * h[9];
        C p[Q];
        p[0] = c * (a0 + o0);  p[18] = c * (a0 - o0);
        p[1] = c * (a1 + o1);  p[17] = c * (a1 - o1);
        p[2] = c * (ex - 12.0 * h[1]); p[16] = c * (ex + 12.0 * h[1]);
        p[3] = c * (a3 + o3);  p[15] = c * (a3 - o3);
        p[4] = c * (a4 + o4);  p[14] = c * (a4 - o4);
        p[5] = c * (a5 + o5);  p[13] = c * (a5 - o5);
        p[6] = c * (ey - 12.0 * h[2]); p[12] = c * (ey + 12.0 * h[2]);
        p[7] = c * (a7 + o7);  p[11] = c * (a7 - o7);
        p[8] = c * (ez - 12.0 * h[3]); p[10] = c * (ez + 12.0 * h[3]);
        p[9] = (1.0 / 3.0) * h[0] - 0.5 * (h[4] + h[7] + h[9]);
#pragma unroll
        for (int q = 0; q < Q; ++q) f[q] = ADD ? f[q] + p[q] : p[q];
    }

    __device__ static void heq(C den, C vx, C vy, C vz, C *h) {
        C jx = den * vx, jy = den * vy, jz = den * vz;
        h[0] = den; h[1] = jx; h[2] = jy; h[3] = jz;
        h[4] = jx * vx; h[5] = jx * vy; h[6] = jx * vz;
        h[7] = jy * vy; h[8] = jy * vz; h[9] = jz * vz;
    }

    __device__ static void force_h2(C *h, C c2, C ax, C ay, C az, C jx, C jy, C jz) {
        h[4] = h[4] + 2.0 * c2 * ax * jx;
        h[5] = h[5] + c2 * (ax * jy + ay * jx);
        h[6] = h[6] + c2 * (ax * jz + az * jx);
        h[7] = h[7] + 2.0 * c2 * ay * jy;
        h[8] = h[8] + c2 * (ay * jz + az * jy);
        h[9] = h[9] + 2.0 * c2 * az * jz;
    }

    // Zou-He unknown populations for face fc (jyulb/bcs.pyx:487-716)
    __device__ static void zh_assign(int fc, C jx, C jy, C jz, C *f) {
        const C s6 = 1.0 / 6.0, s3 = 1.0 / 3.0;
        C t;
        switch (fc) {
        case 0:
            t = f[11] + f[12] + f[13] - f[5] - f[6] - f[7];
            f[14] = f[4] + s6 * jx + 0.5 * t - 0.5 * jy;
            f[18] = f[0] + s6 * jx - 0.5 * t + 0.5 * jy;
            t = f[7] + f[10] + f[13] - f[5] - f[8] - f[11];
            f[15] = f[3] + s6 * jx + 0.5 * t - 0.5 * jz;
            f[17] = f[1] + s6 * jx - 0.5 * t + 0.5 * jz;
            f[16] = f[2] + s3 * jx;
            break;
        case 1:
            t = f[11] + f[12] + f[13] - f[5] - f[6] - f[7];
            f[0] = f[18] - s6 * jx + 0.5 * t - 0.5 * jy;
            f[4] = f[14] - s6 * jx - 0.5 * t + 0.5 * jy;
            t = f[7] + f[10] + f[13] - f[5] - f[8] - f[11];
            f[1] = f[17] - s6 * jx + 0.5 * t - 0.5 * jz;
            f[3] = f[15] - s6 * jx - 0.5 * t + 0.5 * jz;
            f[2] = f[16] - s3 * jx;
            break;
        case 2:
            t = f[15] + f[16] + f[17] - f[1] - f[2] - f[3];
            f[4] = f[14] + s6 * jy + 0.5 * t - 0.5 * jx;
            f[18] = f[0] + s6 * jy - 0.5 * t + 0.5 * jx;
            t = f[17] + f[10] + f[3] - f[15] - f[8] - f[1];
            f[11] = f[7] + s6 * jy + 0.5 * t - 0.5 * jz;
            f[13] = f[5] + s6 * jy - 0.5 * t + 0.5 * jz;
            f[12] = f[6] + s3 * jy;
            break;
        case 3:
            t = f[15] + f[16] + f[17] - f[1] - f[2] - f[3];
            f[0] = f[18] - s6 * jy + 0.5 * t - 0.5 * jx;
            f[14] = f[4] - s6 * jy - 0.5 * t + 0.5 * jx;
            t = f[17] + f[10] + f[3] - f[15] - f[8] - f[1];
            f[5] = f[13] - s6 * jy + 0.5 * t - 0.5 * jz;
            f[7] = f[11] - s6 * jy - 0.5 * t + 0.5 * jz;
            f[6] = f[12] - s3 * jy;
            break;
        case 4:
            t = f[18] + f[16] + f[14] - f[4] - f[2] - f[0];
            f[3] = f[15] + s6 * jz + 0.5 * t - 0.5 * jx;
            f[17] = f[1] + s6 * jz - 0.5 * t + 0.5 * jx;
            t = f[18] + f[12] + f[4] - f[14] - f[6] - f[0];
            f[7] = f[11] + s6 * jz + 0.5 * t - 0.5 * jy;
            f[13] = f[5] + s6 * jz - 0.5 * t + 0.5 * jy;
            f[10] = f[8] + s3 * jz;
            break;
        default:
            t = f[18] + f[16] + f[14] - f[4] - f[2] - f[0];
            f[1] = f[17] - s6 * jz + 0.5 * t - 0.5 * jx;
            f[15] = f[3] - s6 * jz - 0.5 * t + 0.5 * jx;
            t = f[18] + f[12] + f[4] - f[14] - f[6] - f[0];
            f[5] = f[13] - s6 * jz + 0.5 * t - 0.5 * jy;
            f[11] = f[7] - s6 * jz - 0.5 * t + 0.5 * jy;
            f[8] = f[10] - s3 * jz;
            break;
        }
    }

    // Zou-He fixed density / velocity (jyulb/bcs.pyx:31-482); the sums run in
    // the reference's literal order for each face
    __device__ static void zou_he(int fc, int kind, double den, double vx, double vy, double vz, C *f) {
        C kn, out;
        switch (fc) {
        case 0:
            kn = f[9] + f[2] + f[6] + f[12] + f[8] + f[5] + f[11] + f[1] + f[0] + f[4] + f[10] + f[7] + f[13] + f[3];
            out = f[2] + f[1] + f[0] + f[4] + f[3];
            break;
        case 1:
            kn = f[9] + f[16] + f[6] + f[12] + f[8] + f[5] + f[11] + f[15] + f[14] + f[18] + f[10] + f[7] + f[13] + f[17];
            out = f[16] + f[15] + f[14] + f[18] + f[17];
            break;
        case 2:
            kn = f[9] + f[2] + f[16] + f[6] + f[8] + f[5] + f[1] + f[15] + f[0] + f[14] + f[10] + f[7] + f[3] + f[17];
            out = f[6] + f[5] + f[0] + f[14] + f[7];
            break;
        case 3:
            kn = f[9] + f[2] + f[16] + f[12] + f[8] + f[11] + f[1] + f[15] + f[4] + f[18] + f[10] + f[13] + f[3] + f[17];
            out = f[12] + f[11] + f[4] + f[18] + f[13];
            break;
        case 4:
            kn = f[9] + f[2] + f[16] + f[6] + f[12] + f[8] + f[5] + f[11] + f[1] + f[15] + f[0] + f[18] + f[14] + f[4];
            out = f[8] + f[5] + f[11] + f[1] + f[15];
            break;
        default:
            kn = f[9] + f[2] + f[16] + f[6] + f[12] + f[10] + f[7] + f[13] + f[3] + f[17] + f[0] + f[18] + f[14] + f[4];
            out = f[10] + f[7] + f[13] + f[3] + f[17];
            break;
        }
        const int ax = fc >> 1;
        const bool high = fc & 1;
        const C v[3] = {vx, vy, vz};
        C j[3];
        if (kind == BC_FIXED_DEN) {
            j[0] = den * vx; j[1] = den * vy; j[2] = den * vz;
            j[ax] = high ? (out - (den - kn)) : ((den - kn) - out);
        } else {
            const C dbc = high ? (kn + out) / (1.0 + v[ax]) : (kn + out) / (1.0 - v[ax]);
            j[0] = dbc * vx; j[1] = dbc * vy; j[2] = dbc * vz;
        }
        zh_assign(fc, j[0], j[1], j[2], f);
    }
};

} // namespace jlb
