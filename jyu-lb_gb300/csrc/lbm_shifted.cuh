// lbm_shifted.cuh -- FP32 collision physics on shifted populations
// g_q = f_q - w_q.
//
// The physics is the reference's (jyulb/D3Q19.pyx:655-940, jyulb/bcs.pyx),
// rewritten for FP32 accuracy: every quantity that is ~1 in the FP64 form
// (f_q, den, the zeroth moment) is carried as its deviation from the rest
// state, so no FP32 value ever holds 1 + small.  Identities used:
//   den - 1 = sum_q g_q,  j = sum_q c_q g_q,  P(h) - w = P(h with h0 -> h0 - 1),
//   and the Zou-He formulas are invariant under the shift because the weights
//   of paired populations are equal.
// The collision returns den - 1; velocities are the reference's stored ones,
// u = j/den + a/2.
//
// Conservation in FP32.  Rounding that is the same at every step adds up: a
// relaxation that multiplies the momentum by 1 - 1e-8 per step leaves a
// relative error near 1e-4 after 10^4 steps.  So the coefficients are exact
// where the conserved moments pass through them: the host gives the kernels
// relaxation rates (jlb::float_exact_rates) for which 1 - w_e and the TRT pair
// coefficients 1 - (w_e + w_o)/2 and (w_e - w_o)/2 are exact in FP32, so the
// pair relaxation plus the projection return the momentum and mass they were
// given up to unbiased rounding.
#pragma once
#include "lbm_step.cuh"

namespace jlb {

struct PhysShBase {
    using C = float;

    template <int q> __device__ static C ladd(C v, C dden, C s) {
        constexpr float w6 = NNZ(q) == 1 ? (6.0f / 18.0f) : (6.0f / 36.0f);
        return fmaf(w6 * (1.0f + dden), s, v);
    }

    // moments of shifted populations: returns den - 1
    __device__ static C moments(const C *g, C &jx, C &jy, C &jz) {
        const C d1x = (g[0] + g[1]) + (g[2] + g[3]) + g[4];
        const C dx1 = (g[14] + g[15]) + (g[16] + g[17]) + g[18];
        const C d01y = g[5] + g[6] + g[7];
        const C d0y1 = g[11] + g[12] + g[13];
        const C dz = g[8] + g[9] + g[10];
        jx = dx1 - d1x;
        jy = (g[4] + g[18] + d0y1) - (g[0] + g[14] + d01y);
        jz = ((g[3] + g[7]) + (g[10] + g[13]) + g[17]) - ((g[1] + g[5]) + (g[8] + g[11]) + g[15]);
        return ((d1x + dx1) + (d01y + d0y1)) + dz;
    }

    // P(H) for H = (H0 (shifted), H1[3], H2[6]) added to the relaxed g
    // (g[q] already holds the relaxed part).  The first-moment weights k6 and
    // k12 are FP32 values whose real sum 2 k6 + 8 k12 is exactly 1 (k6 is one
    // ulp below the nearest float to 1/6): with the nearest floats the
    // projection would return (1 + 3e-8) H1, a bias of the momentum that
    // repeats identically every step and accumulates.
    __device__ static void project_add(const C H0, const C hx, const C hy, const C hz, const C hxx,
                                       const C hxy, const C hxz, const C hyy, const C hyz, const C hzz,
                                       C *g) {
        const C tr = hxx + hyy + hzz;
        const C A0 = fmaf(-1.5f, tr, H0);
        const C k18 = 1.0f / 18.0f, k36 = 1.0f / 36.0f;
        const C k6 = 0x1.555554p-3f, k12 = 0x1.555556p-4f; // 11184810 * 2^-26, 11184811 * 2^-27
        g[9] += A0 * (1.0f / 3.0f);
        C e, o;
        e = fmaf(4.5f, hxx, A0) * k18; o = hx * k6; g[16] += e + o; g[2] += e - o;
        e = fmaf(4.5f, hyy, A0) * k18; o = hy * k6; g[12] += e + o; g[6] += e - o;
        e = fmaf(4.5f, hzz, A0) * k18; o = hz * k6; g[10] += e + o; g[8] += e - o;
        const C bxy = fmaf(4.5f, hxx + hyy, A0), bxz = fmaf(4.5f, hxx + hzz, A0), byz = fmaf(4.5f, hyy + hzz, A0);
        e = fmaf(9.0f, hxy, bxy) * k36; o = (hx + hy) * k12; g[18] += e + o; g[0] += e - o;
        e = fmaf(-9.0f, hxy, bxy) * k36; o = (hx - hy) * k12; g[14] += e + o; g[4] += e - o;
        e = fmaf(9.0f, hxz, bxz) * k36; o = (hx + hz) * k12; g[17] += e + o; g[1] += e - o;
        e = fmaf(-9.0f, hxz, bxz) * k36; o = (hx - hz) * k12; g[15] += e + o; g[3] += e - o;
        e = fmaf(9.0f, hyz, byz) * k36; o = (hy + hz) * k12; g[13] += e + o; g[5] += e - o;
        e = fmaf(-9.0f, hyz, byz) * k36; o = (hy - hz) * k12; g[11] += e + o; g[7] += e - o;
    }

    // Zou-He (jyulb/bcs.pyx:31-716) on shifted populations; den_bc is the
    // full density (FP64 on input), converted to its deviation here
    __device__ static void zou_he(int fc, int kind, double den, double vx, double vy, double vz, C *g) {
        C kn, out;
        switch (fc) {
        case 0:
            kn = (g[9] + g[6] + g[12] + g[8] + g[10]) + (g[5] + g[11] + g[7] + g[13]);
            out = g[2] + g[1] + g[0] + g[4] + g[3];
            break;
        case 1:
            kn = (g[9] + g[6] + g[12] + g[8] + g[10]) + (g[5] + g[11] + g[7] + g[13]);
            out = g[16] + g[15] + g[14] + g[18] + g[17];
            break;
        case 2:
            kn = (g[9] + g[2] + g[16] + g[8] + g[10]) + (g[1] + g[15] + g[3] + g[17]);
            out = g[6] + g[5] + g[0] + g[14] + g[7];
            break;
        case 3:
            kn = (g[9] + g[2] + g[16] + g[8] + g[10]) + (g[1] + g[15] + g[3] + g[17]);
            out = g[12] + g[11] + g[4] + g[18] + g[13];
            break;
        case 4:
            kn = (g[9] + g[2] + g[16] + g[6] + g[12]) + (g[0] + g[18] + g[14] + g[4]);
            out = g[8] + g[5] + g[11] + g[1] + g[15];
            break;
        default:
            kn = (g[9] + g[2] + g[16] + g[6] + g[12]) + (g[0] + g[18] + g[14] + g[4]);
            out = g[10] + g[7] + g[13] + g[3] + g[17];
            break;
        }
        // kn above holds the 9 populations with zero normal component; the
        // known set of the reference (14 values) is those plus `out`
        const int ax = fc >> 1;
        const bool high = fc & 1;
        const C S = kn + 2.0f * out;  // (sum of known) + out, shifted
        C j[3];
        const float v[3] = {(float)vx, (float)vy, (float)vz};
        if (kind == BC_FIXED_DEN) {
            const C dd = (C)(den - 1.0);
            const C d = 1.0f + dd;
            j[0] = d * v[0]; j[1] = d * v[1]; j[2] = d * v[2];
            j[ax] = high ? (S - dd) : (dd - S);
        } else {
            const C dbc = high ? (1.0f + S) / (1.0f + v[ax]) : (1.0f + S) / (1.0f - v[ax]);
            j[0] = dbc * v[0]; j[1] = dbc * v[1]; j[2] = dbc * v[2];
        }
        const C jx = j[0], jy = j[1], jz = j[2];
        const C s6 = 1.0f / 6.0f, s3 = 1.0f / 3.0f;
        C t;
        switch (fc) {
        case 0:
            t = (g[11] + g[12] + g[13]) - (g[5] + g[6] + g[7]);
            g[14] = g[4] + s6 * jx + 0.5f * (t - jy);
            g[18] = g[0] + s6 * jx - 0.5f * (t - jy);
            t = (g[7] + g[10] + g[13]) - (g[5] + g[8] + g[11]);
            g[15] = g[3] + s6 * jx + 0.5f * (t - jz);
            g[17] = g[1] + s6 * jx - 0.5f * (t - jz);
            g[16] = g[2] + s3 * jx;
            break;
        case 1:
            t = (g[11] + g[12] + g[13]) - (g[5] + g[6] + g[7]);
            g[0] = g[18] - s6 * jx + 0.5f * (t - jy);
            g[4] = g[14] - s6 * jx - 0.5f * (t - jy);
            t = (g[7] + g[10] + g[13]) - (g[5] + g[8] + g[11]);
            g[1] = g[17] - s6 * jx + 0.5f * (t - jz);
            g[3] = g[15] - s6 * jx - 0.5f * (t - jz);
            g[2] = g[16] - s3 * jx;
            break;
        case 2:
            t = (g[15] + g[16] + g[17]) - (g[1] + g[2] + g[3]);
            g[4] = g[14] + s6 * jy + 0.5f * (t - jx);
            g[18] = g[0] + s6 * jy - 0.5f * (t - jx);
            t = (g[17] + g[10] + g[3]) - (g[15] + g[8] + g[1]);
            g[11] = g[7] + s6 * jy + 0.5f * (t - jz);
            g[13] = g[5] + s6 * jy - 0.5f * (t - jz);
            g[12] = g[6] + s3 * jy;
            break;
        case 3:
            t = (g[15] + g[16] + g[17]) - (g[1] + g[2] + g[3]);
            g[0] = g[18] - s6 * jy + 0.5f * (t - jx);
            g[14] = g[4] - s6 * jy - 0.5f * (t - jx);
            t = (g[17] + g[10] + g[3]) - (g[15] + g[8] + g[1]);
            g[5] = g[13] - s6 * jy + 0.5f * (t - jz);
            g[7] = g[11] - s6 * jy - 0.5f * (t - jz);
            g[6] = g[12] - s3 * jy;
            break;
        case 4:
            t = (g[18] + g[16] + g[14]) - (g[4] + g[2] + g[0]);
            g[3] = g[15] + s6 * jz + 0.5f * (t - jx);
            g[17] = g[1] + s6 * jz - 0.5f * (t - jx);
            t = (g[18] + g[12] + g[4]) - (g[14] + g[6] + g[0]);
            g[7] = g[11] + s6 * jz + 0.5f * (t - jy);
            g[13] = g[5] + s6 * jz - 0.5f * (t - jy);
            g[10] = g[8] + s3 * jz;
            break;
        default:
            t = (g[18] + g[16] + g[14]) - (g[4] + g[2] + g[0]);
            g[1] = g[17] - s6 * jz + 0.5f * (t - jx);
            g[15] = g[3] - s6 * jz - 0.5f * (t - jx);
            t = (g[18] + g[12] + g[4]) - (g[14] + g[6] + g[0]);
            g[5] = g[13] - s6 * jz + 0.5f * (t - jy);
            g[11] = g[7] - s6 * jz - 0.5f * (t - jy);
            g[8] = g[10] - s3 * jz;
            break;
        }
    }
};

template <int SCH> struct PhysSh : PhysShBase {
    __device__ static C collide(C *g, C ax, C ay, C az, C we, C wo, C &ux, C &uy, C &uz) {
        C jx, jy, jz;
        C hx, hy, hz, hxx, hxy, hxz, hyy, hyz, hzz, H0;
        if (SCH == SCH_REG) {
            // H10 moments of g: den-1, j, and the second moment minus den/3
            const C dd = moments(g, jx, jy, jz);
            const C pxx = ((g[0] + g[1]) + (g[2] + g[3]) + g[4]) + ((g[14] + g[15]) + (g[16] + g[17]) + g[18]);
            const C pyy = ((g[0] + g[5]) + (g[6] + g[7]) + g[14]) + ((g[4] + g[11]) + (g[12] + g[13]) + g[18]);
            const C pzz = ((g[1] + g[5]) + (g[8] + g[11]) + g[15]) + ((g[3] + g[7]) + (g[10] + g[13]) + g[17]);
            const C pxy = (g[0] + g[18]) - (g[4] + g[14]);
            const C pxz = (g[1] + g[17]) - (g[3] + g[15]);
            const C pyz = (g[5] + g[13]) - (g[7] + g[11]);
            const C d3 = dd * (1.0f / 3.0f);
            const C den = 1.0f + dd, inv = 1.0f / den;
            const C c1 = 1.0f - we, c2 = 1.0f - 0.5f * we;
            const C sx = fmaf(0.5f * ax, den, jx), sy = fmaf(0.5f * ay, den, jy), sz = fmaf(0.5f * az, den, jz);
            ux = sx * inv; uy = sy * inv; uz = sz * inv;
            // den u = s exactly: no round trip through u
            const C rx = sx, ry = sy, rz = sz;
            H0 = dd;
            hx = fmaf(c1, jx, fmaf(we, rx, c2 * ax * den));
            hy = fmaf(c1, jy, fmaf(we, ry, c2 * ay * den));
            hz = fmaf(c1, jz, fmaf(we, rz, c2 * az * den));
            hxx = fmaf(c1, pxx - d3, fmaf(we, rx * ux, 2.0f * c2 * ax * sx));
            hyy = fmaf(c1, pyy - d3, fmaf(we, ry * uy, 2.0f * c2 * ay * sy));
            hzz = fmaf(c1, pzz - d3, fmaf(we, rz * uz, 2.0f * c2 * az * sz));
            hxy = fmaf(c1, pxy, fmaf(we, rx * uy, c2 * (ax * sy + ay * sx)));
            hxz = fmaf(c1, pxz, fmaf(we, rx * uz, c2 * (ax * sz + az * sx)));
            hyz = fmaf(c1, pyz, fmaf(we, ry * uz, c2 * (ay * sz + az * sy)));
#pragma unroll
            for (int q = 0; q < Q; ++q) g[q] = 0.0f;
            project_add(H0, hx, hy, hz, hxx, hxy, hxz, hyy, hyz, hzz, g);
            return dd;
        }
        const C dd = moments(g, jx, jy, jz);
        const C den = 1.0f + dd, inv = 1.0f / den;
        ux = fmaf(jx, inv, 0.5f * ax);
        uy = fmaf(jy, inv, 0.5f * ay);
        uz = fmaf(jz, inv, 0.5f * az);
        const C wodd = (SCH == SCH_TRT) ? wo : we;
        const C c1 = 1.0f - 0.5f * wodd, c2 = 1.0f - 0.5f * we;
        // momentum incl. a/2 (= den u), formed without the round trip through u
        const C sx = fmaf(0.5f * ax, den, jx), sy = fmaf(0.5f * ay, den, jy), sz = fmaf(0.5f * az, den, jz);
        H0 = we * dd;
        hx = fmaf(wodd, sx, c1 * ax * den);
        hy = fmaf(wodd, sy, c1 * ay * den);
        hz = fmaf(wodd, sz, c1 * az * den);
        const C f2 = 2.0f * c2;
        hxx = fmaf(we * sx, ux, f2 * ax * sx);
        hyy = fmaf(we * sy, uy, f2 * ay * sy);
        hzz = fmaf(we * sz, uz, f2 * az * sz);
        hxy = fmaf(we * sx, uy, c2 * (ax * sy + ay * sx));
        hxz = fmaf(we * sx, uz, c2 * (ax * sz + az * sx));
        hyz = fmaf(we * sy, uz, c2 * (ay * sz + az * sy));
        if (SCH == SCH_BGK) {
            const C r = 1.0f - we;
#pragma unroll
            for (int q = 0; q < Q; ++q) g[q] *= r;
        } else {
            const C c3 = 1.0f - 0.5f * (we + wo), c4 = 0.5f * (we - wo);
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                const C a = g[q], b = g[18 - q];
                g[q] = c3 * a - c4 * b;
                g[18 - q] = c3 * b - c4 * a;
            }
            g[9] *= (1.0f - we);
        }
        project_add(H0, hx, hy, hz, hxx, hxy, hxz, hyy, hyz, hzz, g);
        return dd;
    }
};

// The same physics on the stored FP16 values h_q = 2^12 (f_q - w_q) / w_q
// (StoreF16), used for the bulk of the sites: g_q = w_q 2^-12 h_q enters the
// moments as weighted class sums, relaxation pairs q with opp(q) of equal
// weight, and the projection P(H)_q = w_q poly_q(H) adds poly_q(2^12 H) to
// h_q, so the per-population scale of decode and encode disappears.
template <int SCH> struct PhysH16 : PhysSh<SCH> {
    using C = float;
    static constexpr bool h_space = true;

    __device__ static void project_h(C H0, C hx, C hy, C hz, C hxx, C hxy, C hxz, C hyy, C hyz, C hzz, C *h) {
        constexpr C K = 4096.0f;
        H0 *= K; hx *= K; hy *= K; hz *= K;
        hxx *= K; hxy *= K; hxz *= K; hyy *= K; hyz *= K; hzz *= K;
        const C tr = hxx + hyy + hzz;
        const C A0 = fmaf(-1.5f, tr, H0);
        h[9] += A0;
        C e, o;
        e = fmaf(4.5f, hxx, A0); o = 3.0f * hx; h[16] += e + o; h[2] += e - o;
        e = fmaf(4.5f, hyy, A0); o = 3.0f * hy; h[12] += e + o; h[6] += e - o;
        e = fmaf(4.5f, hzz, A0); o = 3.0f * hz; h[10] += e + o; h[8] += e - o;
        const C bxy = fmaf(4.5f, hxx + hyy, A0), bxz = fmaf(4.5f, hxx + hzz, A0), byz = fmaf(4.5f, hyy + hzz, A0);
        e = fmaf(9.0f, hxy, bxy); o = 3.0f * (hx + hy); h[18] += e + o; h[0] += e - o;
        e = fmaf(-9.0f, hxy, bxy); o = 3.0f * (hx - hy); h[14] += e + o; h[4] += e - o;
        e = fmaf(9.0f, hxz, bxz); o = 3.0f * (hx + hz); h[17] += e + o; h[1] += e - o;
        e = fmaf(-9.0f, hxz, bxz); o = 3.0f * (hx - hz); h[15] += e + o; h[3] += e - o;
        e = fmaf(9.0f, hyz, byz); o = 3.0f * (hy + hz); h[13] += e + o; h[5] += e - o;
        e = fmaf(-9.0f, hyz, byz); o = 3.0f * (hy - hz); h[11] += e + o; h[7] += e - o;
    }

    // returns den - 1, like collide
    __device__ static C collide_h(C *h, C ax, C ay, C az, C we, C wo, C &ux, C &uy, C &uz) {
        constexpr C s0 = 1.0f / 4096.0f;
        constexpr C w0 = s0 / 3.0f, w1 = s0 / 18.0f, w2 = s0 / 36.0f;
        const C axis = ((h[2] + h[16]) + (h[6] + h[12])) + (h[8] + h[10]);
        const C diag = (((h[0] + h[1]) + (h[3] + h[4])) + ((h[14] + h[15]) + (h[17] + h[18]))) +
                       ((h[5] + h[7]) + (h[11] + h[13]));
        const C dd = fmaf(w0, h[9], fmaf(w1, axis, w2 * diag));
        const C jx = fmaf(w1, h[16] - h[2], w2 * (((h[14] + h[15]) + (h[17] + h[18])) - ((h[0] + h[1]) + (h[3] + h[4]))));
        const C jy = fmaf(w1, h[12] - h[6], w2 * (((h[4] + h[11]) + (h[13] + h[18])) - ((h[0] + h[5]) + (h[7] + h[14]))));
        const C jz = fmaf(w1, h[10] - h[8], w2 * (((h[3] + h[7]) + (h[13] + h[17])) - ((h[1] + h[5]) + (h[11] + h[15]))));
        const C den = 1.0f + dd, inv = 1.0f / den;
        C hx, hy, hz, hxx, hxy, hxz, hyy, hyz, hzz, H0;
        if (SCH == SCH_REG) {
            const C dx = ((h[0] + h[1]) + (h[3] + h[4])) + ((h[14] + h[15]) + (h[17] + h[18]));
            const C dy = ((h[0] + h[4]) + (h[5] + h[7])) + ((h[11] + h[13]) + (h[14] + h[18]));
            const C dz = ((h[1] + h[3]) + (h[5] + h[7])) + ((h[11] + h[13]) + (h[15] + h[17]));
            const C pxx = fmaf(w1, h[2] + h[16], w2 * dx);
            const C pyy = fmaf(w1, h[6] + h[12], w2 * dy);
            const C pzz = fmaf(w1, h[8] + h[10], w2 * dz);
            const C pxy = w2 * ((h[0] + h[18]) - (h[4] + h[14]));
            const C pxz = w2 * ((h[1] + h[17]) - (h[3] + h[15]));
            const C pyz = w2 * ((h[5] + h[13]) - (h[7] + h[11]));
            const C d3 = dd * (1.0f / 3.0f);
            const C c1 = 1.0f - we, c2 = 1.0f - 0.5f * we;
            const C sx = fmaf(0.5f * ax, den, jx), sy = fmaf(0.5f * ay, den, jy), sz = fmaf(0.5f * az, den, jz);
            ux = sx * inv; uy = sy * inv; uz = sz * inv;
            // den u = s exactly: no round trip through u
            const C rx = sx, ry = sy, rz = sz;
            H0 = dd;
            hx = fmaf(c1, jx, fmaf(we, rx, c2 * ax * den));
            hy = fmaf(c1, jy, fmaf(we, ry, c2 * ay * den));
            hz = fmaf(c1, jz, fmaf(we, rz, c2 * az * den));
            hxx = fmaf(c1, pxx - d3, fmaf(we, rx * ux, 2.0f * c2 * ax * sx));
            hyy = fmaf(c1, pyy - d3, fmaf(we, ry * uy, 2.0f * c2 * ay * sy));
            hzz = fmaf(c1, pzz - d3, fmaf(we, rz * uz, 2.0f * c2 * az * sz));
            hxy = fmaf(c1, pxy, fmaf(we, rx * uy, c2 * (ax * sy + ay * sx)));
            hxz = fmaf(c1, pxz, fmaf(we, rx * uz, c2 * (ax * sz + az * sx)));
            hyz = fmaf(c1, pyz, fmaf(we, ry * uz, c2 * (ay * sz + az * sy)));
#pragma unroll
            for (int q = 0; q < Q; ++q) h[q] = 0.0f;
            project_h(H0, hx, hy, hz, hxx, hxy, hxz, hyy, hyz, hzz, h);
            return dd;
        }
        ux = fmaf(jx, inv, 0.5f * ax);
        uy = fmaf(jy, inv, 0.5f * ay);
        uz = fmaf(jz, inv, 0.5f * az);
        const C wodd = (SCH == SCH_TRT) ? wo : we;
        const C c1 = 1.0f - 0.5f * wodd, c2 = 1.0f - 0.5f * we;
        const C sx = fmaf(0.5f * ax, den, jx), sy = fmaf(0.5f * ay, den, jy), sz = fmaf(0.5f * az, den, jz);
        H0 = we * dd;
        hx = fmaf(wodd, sx, c1 * ax * den);
        hy = fmaf(wodd, sy, c1 * ay * den);
        hz = fmaf(wodd, sz, c1 * az * den);
        const C f2 = 2.0f * c2;
        hxx = fmaf(we * sx, ux, f2 * ax * sx);
        hyy = fmaf(we * sy, uy, f2 * ay * sy);
        hzz = fmaf(we * sz, uz, f2 * az * sz);
        hxy = fmaf(we * sx, uy, c2 * (ax * sy + ay * sx));
        hxz = fmaf(we * sx, uz, c2 * (ax * sz + az * sx));
        hyz = fmaf(we * sy, uz, c2 * (ay * sz + az * sy));
        if (SCH == SCH_BGK) {
            const C r = 1.0f - we;
#pragma unroll
            for (int q = 0; q < Q; ++q) h[q] *= r;
        } else {
            const C c3 = 1.0f - 0.5f * (we + wo), c4 = 0.5f * (we - wo);
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                const C a = h[q], b = h[18 - q];
                h[q] = c3 * a - c4 * b;
                h[18 - q] = c3 * b - c4 * a;
            }
            h[9] *= (1.0f - we);
        }
        project_h(H0, hx, hy, hz, hxx, hxy, hxz, hyy, hyz, hzz, h);
        return dd;
    }
};

} // namespace jlb
