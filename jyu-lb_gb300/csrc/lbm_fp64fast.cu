// lbm_fp64fast.cu -- FP64 time step with contracted, regrouped arithmetic
// (precision JLB_FP64_FAST).
//
// Same storage, layout, boundary handling and physics as the parity step
// (lbm_fp64.cu): BGK / TRT / regularized collision of the reference
// (jyulb/D3Q19.pyx:655-940) with its forcing and stored velocity
// u = j/den + a/2.  The arithmetic is reorganised for GB300, whose FP64 rate
// (not HBM) bounds the parity step at ~276 separately rounded operations per
// TRT site:
//   * den, j and u in the reference's order and rounding,
//   * the projection of the H10 moments grouped per pair of opposite
//     populations (even part e, odd part o) and merged with the TRT pair
//     relaxation: f_q <- fma(c3, f_q, fma(-c4, f_opp, e + o)),
//   * den u formed as j + den a/2 directly,
// and the unit is compiled with FMA contraction.  Boundary nodes use the
// reference's Zou-He and Ladd expressions (lbm_fp64.cuh), contracted.
// Results differ from the parity step by rounding only: within 1e-12
// relative of the reference on every golden case, at up to 1000 steps.
#include "lbm_fp64.cuh"

namespace jlb {

struct Phys64FBase : Phys64Base {
    // returns den and j with the reference's sums in the reference's order
    // (jyulb/D3Q19.pyx:348-390; no multiply, so contraction cannot change
    // them): the stored den and u then equal the parity step's whenever the
    // populations do, and slow flows keep the reference's velocity rounding
    __device__ static C moments(const C *f, C &jx, C &jy, C &jz) {
        const C d1x = f[0] + f[1] + f[2] + f[3] + f[4];
        const C dx1 = f[14] + f[15] + f[16] + f[17] + f[18];
        const C d01y = f[5] + f[6] + f[7];
        const C d0y1 = f[11] + f[12] + f[13];
        jx = dx1 - d1x;
        jy = f[4] + d0y1 + f[18] - f[0] - d01y - f[14];
        jz = f[3] + f[7] + f[10] + f[13] + f[17] - f[1] - f[5] - f[8] - f[11] - f[15];
        return d1x + dx1 + d01y + d0y1 + f[8] + f[9] + f[10];
    }

    // P(H) for H = (H0, H1[3], H2[6]): the reference's 1/72 projection
    // (jyulb/D3Q19.pyx:532-599) regrouped by weight class and merged with
    // the pair relaxation: each population becomes
    //   f_q <- c3 f_q - c4 f_opp + (e +/- o)
    // as fma(c3, f_q, fma(-c4, f_opp, e +/- o)), one operation fewer per
    // population than relaxing first and adding the projection after
    // (BGK: c3 = 1 - w_e, c4 = 0; regularized: c3 = c4 = 0)
    template <bool PAIR, bool RELAX>
    __device__ static void relax_project(const C c3, const C c4, const C r9, const C H0, const C hx, const C hy,
                                         const C hz, const C hxx, const C hxy, const C hxz, const C hyy, const C hyz,
                                         const C hzz, C *f) {
        const C tr = hxx + hyy + hzz;
        const C A0 = fma(-1.5, tr, H0);
        const C k18 = 1.0 / 18.0, k36 = 1.0 / 36.0, k6 = 1.0 / 6.0, k12 = 1.0 / 12.0;
        f[9] = RELAX ? fma(A0, 1.0 / 3.0, r9 * f[9]) : A0 * (1.0 / 3.0);
        auto put = [&](int q, C e, C o) {
            const C a = f[q], b = f[18 - q];
            if (!RELAX) {
                f[q] = e + o;
                f[18 - q] = e - o;
            } else if (PAIR) {
                f[q] = fma(c3, a, fma(-c4, b, e + o));
                f[18 - q] = fma(c3, b, fma(-c4, a, e - o));
            } else {
                f[q] = fma(c3, a, e + o);
                f[18 - q] = fma(c3, b, e - o);
            }
        };
        C e, o;
        e = fma(4.5, hxx, A0) * k18; o = hx * k6; put(16, e, o);
        e = fma(4.5, hyy, A0) * k18; o = hy * k6; put(12, e, o);
        e = fma(4.5, hzz, A0) * k18; o = hz * k6; put(10, e, o);
        const C bxy = fma(4.5, hxx + hyy, A0), bxz = fma(4.5, hxx + hzz, A0), byz = fma(4.5, hyy + hzz, A0);
        e = fma(9.0, hxy, bxy) * k36; o = (hx + hy) * k12; put(18, e, o);
        e = fma(-9.0, hxy, bxy) * k36; o = (hx - hy) * k12; put(14, e, o);
        e = fma(9.0, hxz, bxz) * k36; o = (hx + hz) * k12; put(17, e, o);
        e = fma(-9.0, hxz, bxz) * k36; o = (hx - hz) * k12; put(15, e, o);
        e = fma(9.0, hyz, byz) * k36; o = (hy + hz) * k12; put(13, e, o);
        e = fma(-9.0, hyz, byz) * k36; o = (hy - hz) * k12; put(11, e, o);
    }
};

template <int SCH> struct Phys64F : Phys64FBase {
    // returns den, writes the stored velocity u = j/den + a/2
    __device__ static C collide(C *f, C ax, C ay, C az, C we, C wo, C &ux, C &uy, C &uz) {
        C jx, jy, jz;
        C hx, hy, hz, hxx, hxy, hxz, hyy, hyz, hzz, H0;
        const C den = moments(f, jx, jy, jz);
        const C inv = 1.0 / den;
        if (SCH == SCH_REG) {
            // H10 second moments of f (jyulb/D3Q19.pyx:395-452), relaxed
            // towards equilibrium; the projection drops the rest
            const C pxx = ((f[0] + f[1]) + (f[2] + f[3]) + f[4]) + ((f[14] + f[15]) + (f[16] + f[17]) + f[18]);
            const C pyy = ((f[0] + f[5]) + (f[6] + f[7]) + f[14]) + ((f[4] + f[11]) + (f[12] + f[13]) + f[18]);
            const C pzz = ((f[1] + f[5]) + (f[8] + f[11]) + f[15]) + ((f[3] + f[7]) + (f[10] + f[13]) + f[17]);
            const C pxy = (f[0] + f[18]) - (f[4] + f[14]);
            const C pxz = (f[1] + f[17]) - (f[3] + f[15]);
            const C pyz = (f[5] + f[13]) - (f[7] + f[11]);
            const C d3 = den * (1.0 / 3.0);
            const C c1 = 1.0 - we, c2 = 1.0 - 0.5 * we;
            // j + den a/2 and u as the reference rounds them (no contraction)
            const C sx = __dadd_rn(jx, __dmul_rn(0.5 * ax, den)), sy = __dadd_rn(jy, __dmul_rn(0.5 * ay, den)),
                    sz = __dadd_rn(jz, __dmul_rn(0.5 * az, den));
            ux = __dmul_rn(inv, sx); uy = __dmul_rn(inv, sy); uz = __dmul_rn(inv, sz);
            H0 = den;
            hx = fma(c1, jx, fma(we, sx, c2 * ax * den));
            hy = fma(c1, jy, fma(we, sy, c2 * ay * den));
            hz = fma(c1, jz, fma(we, sz, c2 * az * den));
            hxx = fma(c1, pxx - d3, fma(we, sx * ux, 2.0 * c2 * ax * sx));
            hyy = fma(c1, pyy - d3, fma(we, sy * uy, 2.0 * c2 * ay * sy));
            hzz = fma(c1, pzz - d3, fma(we, sz * uz, 2.0 * c2 * az * sz));
            hxy = fma(c1, pxy, fma(we, sx * uy, c2 * (ax * sy + ay * sx)));
            hxz = fma(c1, pxz, fma(we, sx * uz, c2 * (ax * sz + az * sx)));
            hyz = fma(c1, pyz, fma(we, sy * uz, c2 * (ay * sz + az * sy)));
            relax_project<false, false>(0.0, 0.0, 0.0, H0, hx, hy, hz, hxx, hxy, hxz, hyy, hyz, hzz, f);
            return den;
        }
        // u = j/den + a/2 as the reference rounds it (no contraction)
        ux = __dadd_rn(__dmul_rn(inv, jx), 0.5 * ax);
        uy = __dadd_rn(__dmul_rn(inv, jy), 0.5 * ay);
        uz = __dadd_rn(__dmul_rn(inv, jz), 0.5 * az);
        const C wodd = (SCH == SCH_TRT) ? wo : we;
        const C c1 = 1.0 - 0.5 * wodd, c2 = 1.0 - 0.5 * we;
        // momentum including a/2 (= den u)
        const C sx = fma(0.5 * ax, den, jx), sy = fma(0.5 * ay, den, jy), sz = fma(0.5 * az, den, jz);
        H0 = we * den;
        hx = fma(wodd, sx, c1 * ax * den);
        hy = fma(wodd, sy, c1 * ay * den);
        hz = fma(wodd, sz, c1 * az * den);
        const C f2 = 2.0 * c2;
        hxx = fma(we * sx, ux, f2 * ax * sx);
        hyy = fma(we * sy, uy, f2 * ay * sy);
        hzz = fma(we * sz, uz, f2 * az * sz);
        hxy = fma(we * sx, uy, c2 * (ax * sy + ay * sx));
        hxz = fma(we * sx, uz, c2 * (ax * sz + az * sx));
        hyz = fma(we * sy, uz, c2 * (ay * sz + az * sy));
        if (SCH == SCH_BGK) {
            const C r = 1.0 - we;
            relax_project<false, true>(r, 0.0, r, H0, hx, hy, hz, hxx, hxy, hxz, hyy, hyz, hzz, f);
        } else {
            const C c3 = 1.0 - 0.5 * (we + wo), c4 = 0.5 * (we - wo);
            relax_project<true, true>(c3, c4, 1.0 - we, H0, hx, hy, hz, hxx, hxy, hxz, hyy, hyz, hzz, f);
        }
        return den;
    }
};

int launch_step_fp64fast(const StepArgs &a, int scheme, bool pstep, bool accf, int blocks, cudaStream_t st) {
    return launch_step_impl<StoreF64, Phys64F>(a, scheme, pstep, accf, blocks, st);
}

} // namespace jlb
