// lbm_fp64.cu -- FP64 time step with the reference's arithmetic.
//
// This translation unit is compiled with -fmad=false: every FP64 operation
// below is a separately rounded IEEE add/mul/div written in the order the
// reference evaluates it (jyulb/D3Q19.pyx:348-940, jyulb/bcs.pyx:31-716,
// jyulb/isothermal.pyx:1112-1248), so the GPU reproduces the reference's
// populations and moments bit for bit on x86-64 builds of the reference.
#include "lbm_fp64.cuh"

namespace jlb {

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
