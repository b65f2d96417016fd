// lbm_fp64.cu -- FP64 time step with the reference's arithmetic.
//
// This translation unit is compiled with -fmad=false: every FP64 operation
// below is a separately rounded IEEE add/mul/div written in the order the
// reference evaluates it (jyulb/D3Q19.pyx:348-940, jyulb/bcs.pyx:31-716,
// jyulb/isothermal.pyx:1112-1248), so the GPU reproduces the reference's
// populations and moments bit for bit on x86-64 builds of the reference.
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

template <int SCH> struct Phys64 : Phys64Base {
    // forward-Euler update; returns den, writes the stored velocity
    // u = j/den + a/2 (jyulb/D3Q19.pyx:655-940)
    __device__ static C collide(C *f, C ax, C ay, C az, C we, C wo, C &ux, C &uy, C &uz) {
        C h[10];
        if (SCH == SCH_BGK) {
            const C c1 = 1.0 - we, c2 = 1.0 - 0.5 * we;
            const C den = f_to_den_vel(f, ux, uy, uz);
            ux = ux + 0.5 * ax; uy = uy + 0.5 * ay; uz = uz + 0.5 * az;
            heq(den, ux, uy, uz, h);
#pragma unroll
            for (int m = 0; m < 10; ++m) h[m] = h[m] * we;
            const C jx = den * ux, jy = den * uy, jz = den * uz;
            h[1] = h[1] + c2 * ax * den; h[2] = h[2] + c2 * ay * den; h[3] = h[3] + c2 * az * den;
            force_h2(h, c2, ax, ay, az, jx, jy, jz);
#pragma unroll
            for (int q = 0; q < Q; ++q) f[q] = f[q] * c1;
            project<true>(h, f);
            return den;
        } else if (SCH == SCH_TRT) {
            const C c1 = 1.0 - 0.5 * wo, c2 = 1.0 - 0.5 * we;
            const C c3 = 1.0 - 0.5 * (we + wo), c4 = 0.5 * (we - wo);
            const C den = f_to_den_vel(f, ux, uy, uz);
            ux = ux + 0.5 * ax; uy = uy + 0.5 * ay; uz = uz + 0.5 * az;
            heq(den, ux, uy, uz, h);
            h[0] = h[0] * we; h[1] = h[1] * wo; h[2] = h[2] * wo; h[3] = h[3] * wo;
#pragma unroll
            for (int m = 4; m < 10; ++m) h[m] = h[m] * we;
            const C jx = den * ux, jy = den * uy, jz = den * uz;
            h[1] = h[1] + c1 * ax * den; h[2] = h[2] + c1 * ay * den; h[3] = h[3] + c1 * az * den;
            force_h2(h, c2, ax, ay, az, jx, jy, jz);
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                const C fa = f[q], fb = f[18 - q];
                f[q] = c3 * fa - c4 * fb;
                f[18 - q] = c3 * fb - c4 * fa;
            }
            f[9] = f[9] * (1.0 - we);
            project<true>(h, f);
            return den;
        } else {
            const C c1 = 1.0 - we, c2 = 1.0 - 0.5 * we;
            C he[10];
            // f_to_h (jyulb/D3Q19.pyx:395-452)
            C d1x = f[0] + f[1] + f[2] + f[3] + f[4];
            C dx1 = f[14] + f[15] + f[16] + f[17] + f[18];
            C d01y = f[5] + f[6] + f[7];
            C d0y1 = f[11] + f[12] + f[13];
            C d1y = f[0] + d01y + f[14];
            C dy1 = f[4] + d0y1 + f[18];
            C d1z = f[1] + f[5] + f[8] + f[11] + f[15];
            C dz1 = f[3] + f[7] + f[10] + f[13] + f[17];
            C den = d1x + dx1 + d01y + d0y1 + f[8] + f[9] + f[10];
            h[0] = den; h[1] = dx1 - d1x; h[2] = dy1 - d1y; h[3] = dz1 - d1z;
            h[4] = (d1x + dx1) - (1.0 / 3.0) * den;
            h[5] = f[0] + f[18] - f[4] - f[14];
            h[6] = f[1] + f[17] - f[3] - f[15];
            h[7] = (d1y + dy1) - (1.0 / 3.0) * den;
            h[8] = f[5] + f[13] - f[7] - f[11];
            h[9] = (d1z + dz1) - (1.0 / 3.0) * den;
            const C inv = 1.0 / den;
            const C jx = h[1] + 0.5 * ax * den, jy = h[2] + 0.5 * ay * den, jz = h[3] + 0.5 * az * den;
            ux = inv * jx; uy = inv * jy; uz = inv * jz;
            heq(den, ux, uy, uz, he);
#pragma unroll
            for (int m = 0; m < 10; ++m) h[m] = h[m] * c1;
#pragma unroll
            for (int m = 0; m < 10; ++m) h[m] = h[m] + we * he[m];
            h[1] = h[1] + c2 * ax * den; h[2] = h[2] + c2 * ay * den; h[3] = h[3] + c2 * az * den;
            force_h2(h, c2, ax, ay, az, jx, jy, jz);
            project<false>(h, f);
            return den;
        }
    }
};

int launch_step_fp64(const StepArgs &a, int scheme, bool pstep, bool accf, int blocks, cudaStream_t st) {
    return launch_step_impl<StoreF64, Phys64>(a, scheme, pstep, accf, blocks, st);
}

} // namespace jlb
