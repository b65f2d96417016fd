/*
 * lbm_oracle.c -- CPU restatement of the jyulb D3Q19 isothermal time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA engine:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * it.  The product never links or calls it.
 *
 * It restates, in plain C99 and FP64, the reference's pull-scheme two-lattice
 * solver so that results can be compared number-for-number:
 *   - halo-padded (NI,NJ,NK) = (nx+2,ny+2,nz+2) fields, k fastest
 *     (jyulb/isothermal.pyx:234-248);
 *   - periodic / symmetric halo fills for phase, den/vel and populations,
 *     in the order x -> y -> z with the reference's index coverage
 *     (jyulb/isothermal.pyx:509-577, 582-686, 691-837);
 *   - pull streaming with Ladd's moving-wall halfway bounce-back
 *     (jyulb/isothermal.pyx:1112-1248);
 *   - Zou-He fixed density / velocity faces (jyulb/bcs.pyx:31-716) with the
 *     bc data copied from the den/vel face layers at every evolve call,
 *     including the reference's Z1 condition (jyulb/isothermal.pyx:476-502);
 *   - BGK / TRT / regularized forward-Euler collisions in the H10 moment
 *     space (jyulb/D3Q19.pyx:348-630, 655-940);
 *   - initial populations with the finite-difference non-equilibrium part
 *     (jyulb/isothermal.pyx:958-1105).
 * Floating-point operations are written in the same order as the reference
 * so that, built with -ffp-contract=off, the result is bit-identical to the
 * reference compiled for x86-64.  Populations are stored q-major
 * f[q*ncnt + n] rather than in the reference's Bundle-C interleave; storage
 * order does not change any arithmetic.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define Q 19
enum { SOLID = 0, FLUID = 1 };
enum { BGK = 0, TRT = 1, REG = 2 };
enum { WALL = 0, PERIODIC = 1, FIXED_DEN = 2, FIXED_VEL = 3, SYMMETRIC = 4 };
enum { F1X = 0, FX1 = 1, F1Y = 2, FY1 = 3, F1Z = 4, FZ1 = 5 };

/* lattice vectors in the reference enumeration (jyulb/D3Q19.pxd:59-79) */
static const int CI[Q] = {-1,-1,-1,-1,-1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1};
static const int CJ[Q] = {-1, 0, 0, 0, 1,-1,-1,-1, 0, 0, 0, 1, 1, 1,-1, 0, 0, 0, 1};
static const int CK[Q] = { 0,-1, 0, 1, 0,-1, 0, 1,-1, 0, 1,-1, 0, 1, 0,-1, 0, 1, 0};
#define W0 (12.0/36.0)
#define W1 ( 2.0/36.0)
#define W2 ( 1.0/36.0)
#define AS2 3.0
#define INV_AS2 (1.0/3.0)
#define OPP(q) (18 - (q))

typedef struct {
    int nx, ny, nz, NI, NJ, NK;
    long ncnt;
    int scheme;
    double kvisc, prm0, prm1;
    double g[3];
    int bc[6];
    uint8_t *phase;          /* (NI,NJ,NK)   */
    double *den, *vel, *acc; /* (NI,NJ,NK[,3]) */
    double *f1, *f2;         /* [Q][ncnt]    */
    double *bcden[6], *bcvel[6];
    long *fluid;             /* linear indices of fluid nodes, x-major */
    long nfluid;
    int init_done;
    unsigned tot_tsteps;
} orc_t;

static inline long NIDX(const orc_t *o, int i, int j, int k) {
    return ((long)i * o->NJ + j) * o->NK + k;
}

/* ------------------------------------------------------------------------ */
/* Moments and projections (jyulb/D3Q19.pyx:348-630)                         */
/* ------------------------------------------------------------------------ */
static double f_to_den_vel(const double *f, double *v) {
    double d1x = f[0] + f[1] + f[2] + f[3] + f[4];
    double dx1 = f[14] + f[15] + f[16] + f[17] + f[18];
    double d01y = f[5] + f[6] + f[7];
    double d0y1 = f[11] + f[12] + f[13];
    double den = d1x + dx1 + d01y + d0y1 + f[8] + f[9] + f[10];
    double jx = dx1 - d1x;
    double jy = f[4] + d0y1 + f[18] - f[0] - d01y - f[14];
    double jz = f[3] + f[7] + f[10] + f[13] + f[17] - f[1] - f[5] - f[8] - f[11] - f[15];
    double inv = 1.0 / den;
    v[0] = inv * jx; v[1] = inv * jy; v[2] = inv * jz;
    return den;
}

static void f_to_h(const double *f, double *h) {
    double d1x = f[0] + f[1] + f[2] + f[3] + f[4];
    double dx1 = f[14] + f[15] + f[16] + f[17] + f[18];
    double d01y = f[5] + f[6] + f[7];
    double d0y1 = f[11] + f[12] + f[13];
    double d1y = f[0] + d01y + f[14];
    double dy1 = f[4] + d0y1 + f[18];
    double d1z = f[1] + f[5] + f[8] + f[11] + f[15];
    double dz1 = f[3] + f[7] + f[10] + f[13] + f[17];
    double den = d1x + dx1 + d01y + d0y1 + f[8] + f[9] + f[10];
    double mxx = d1x + dx1, myy = d1y + dy1, mzz = d1z + dz1;
    double mxy = f[0] + f[18] - f[4] - f[14];
    double mxz = f[1] + f[17] - f[3] - f[15];
    double myz = f[5] + f[13] - f[7] - f[11];
    h[0] = den; h[1] = dx1 - d1x; h[2] = dy1 - d1y; h[3] = dz1 - d1z;
    h[4] = mxx - INV_AS2 * den; h[5] = mxy; h[6] = mxz;
    h[7] = myy - INV_AS2 * den; h[8] = myz; h[9] = mzz - INV_AS2 * den;
}

/* kinetic projection; add != 0 accumulates into f */
static void project(const double *h, double *f, int add) {
    const double c = 1.0 / 72.0;
    double exy = 2.0*h[0] + 6.0*h[4] + 6.0*h[7] - 3.0*h[9];
    double e_mm_xy = exy + 18.0*h[5], o_mm_xy = -6.0*h[1] - 6.0*h[2];
    double e_mp_xy = exy - 18.0*h[5], o_mp_xy = -6.0*h[1] + 6.0*h[2];
    double exz = 2.0*h[0] + 6.0*h[4] - 3.0*h[7] + 6.0*h[9];
    double e_mm_xz = exz + 18.0*h[6], o_mm_xz = -6.0*h[1] - 6.0*h[3];
    double e_mp_xz = exz - 18.0*h[6], o_mp_xz = -6.0*h[1] + 6.0*h[3];
    double eyz = 2.0*h[0] - 3.0*h[4] + 6.0*h[7] + 6.0*h[9];
    double e_mm_yz = eyz + 18.0*h[8], o_mm_yz = -6.0*h[2] - 6.0*h[3];
    double e_mp_yz = eyz - 18.0*h[8], o_mp_yz = -6.0*h[2] + 6.0*h[3];
    double ex = 4.0*h[0] + 12.0*h[4] - 6.0*h[7] - 6.0*h[9];
    double ey = 4.0*h[0] - 6.0*h[4] + 12.0*h[7] - 6.0*h[9];
    double ez = 4.0*h[0] - 6.0*h[4] - 6.0*h[7] + 12.0*h[9];
    double p[Q];
    p[0]  = c*(e_mm_xy + o_mm_xy); p[18] = c*(e_mm_xy - o_mm_xy);
    p[1]  = c*(e_mm_xz + o_mm_xz); p[17] = c*(e_mm_xz - o_mm_xz);
    p[2]  = c*(ex - 12.0*h[1]);    p[16] = c*(ex + 12.0*h[1]);
    p[3]  = c*(e_mp_xz + o_mp_xz); p[15] = c*(e_mp_xz - o_mp_xz);
    p[4]  = c*(e_mp_xy + o_mp_xy); p[14] = c*(e_mp_xy - o_mp_xy);
    p[5]  = c*(e_mm_yz + o_mm_yz); p[13] = c*(e_mm_yz - o_mm_yz);
    p[6]  = c*(ey - 12.0*h[2]);    p[12] = c*(ey + 12.0*h[2]);
    p[7]  = c*(e_mp_yz + o_mp_yz); p[11] = c*(e_mp_yz - o_mp_yz);
    p[8]  = c*(ez - 12.0*h[3]);    p[10] = c*(ez + 12.0*h[3]);
    p[9]  = (1.0/3.0)*h[0] - 0.5*(h[4] + h[7] + h[9]);
    for (int q = 0; q < Q; ++q) f[q] = add ? f[q] + p[q] : p[q];
}

static void den_vel_to_heq(double den, const double *v, double *h) {
    double jx = den*v[0], jy = den*v[1], jz = den*v[2];
    h[0] = den; h[1] = jx; h[2] = jy; h[3] = jz;
    h[4] = jx*v[0]; h[5] = jx*v[1]; h[6] = jx*v[2];
    h[7] = jy*v[1]; h[8] = jy*v[2]; h[9] = jz*v[2];
}

/* force moments shared by the three schemes (jyulb/D3Q19.pyx:694-708) */
static void add_force_h2(double *h, double c2, const double *a,
                         double jx, double jy, double jz) {
    h[4] += 2.0*c2*a[0]*jx;
    h[5] += c2*(a[0]*jy + a[1]*jx);
    h[6] += c2*(a[0]*jz + a[2]*jx);
    h[7] += 2.0*c2*a[1]*jy;
    h[8] += c2*(a[1]*jz + a[2]*jy);
    h[9] += 2.0*c2*a[2]*jz;
}

/* BGK, jyulb/D3Q19.pyx:655-740 */
static double coll_bgk(double *f, const double *a, double w, double *v) {
    double c1 = 1.0 - w, c2 = 1.0 - 0.5*w, h[10];
    double den = f_to_den_vel(f, v);
    v[0] += 0.5*a[0]; v[1] += 0.5*a[1]; v[2] += 0.5*a[2];
    den_vel_to_heq(den, v, h);
    for (int m = 0; m < 10; ++m) h[m] *= w;
    double jx = den*v[0], jy = den*v[1], jz = den*v[2];
    h[1] += c2*a[0]*den; h[2] += c2*a[1]*den; h[3] += c2*a[2]*den;
    add_force_h2(h, c2, a, jx, jy, jz);
    for (int q = 0; q < Q; ++q) f[q] *= c1;
    project(h, f, 1);
    return den;
}

/* TRT, jyulb/D3Q19.pyx:745-853 */
static double coll_trt(double *f, const double *a, double we, double wo, double *v) {
    double c1 = 1.0 - 0.5*wo, c2 = 1.0 - 0.5*we;
    double c3 = 1.0 - 0.5*(we + wo), c4 = 0.5*(we - wo), h[10];
    double den = f_to_den_vel(f, v);
    v[0] += 0.5*a[0]; v[1] += 0.5*a[1]; v[2] += 0.5*a[2];
    den_vel_to_heq(den, v, h);
    h[0] *= we; h[1] *= wo; h[2] *= wo; h[3] *= wo;
    for (int m = 4; m < 10; ++m) h[m] *= we;
    double jx = den*v[0], jy = den*v[1], jz = den*v[2];
    h[1] += c1*a[0]*den; h[2] += c1*a[1]*den; h[3] += c1*a[2]*den;
    add_force_h2(h, c2, a, jx, jy, jz);
    for (int q = 0; q < 9; ++q) {
        double fa = f[q], fb = f[OPP(q)];
        f[q] = c3*fa - c4*fb;
        f[OPP(q)] = c3*fb - c4*fa;
    }
    f[9] *= (1.0 - we);
    project(h, f, 1);
    return den;
}

/* regularized, jyulb/D3Q19.pyx:859-940 */
static double coll_reg(double *f, const double *a, double w, double *v) {
    double c1 = 1.0 - w, c2 = 1.0 - 0.5*w, h[10], he[10];
    f_to_h(f, h);
    double den = h[0], inv = 1.0/den;
    double jx = h[1] + 0.5*a[0]*den, jy = h[2] + 0.5*a[1]*den, jz = h[3] + 0.5*a[2]*den;
    v[0] = inv*jx; v[1] = inv*jy; v[2] = inv*jz;
    den_vel_to_heq(den, v, he);
    for (int m = 0; m < 10; ++m) h[m] *= c1;
    for (int m = 0; m < 10; ++m) h[m] += w*he[m];
    h[1] += c2*a[0]*den; h[2] += c2*a[1]*den; h[3] += c2*a[2]*den;
    add_force_h2(h, c2, a, jx, jy, jz);
    project(h, f, 0);
    return den;
}

/* ------------------------------------------------------------------------ */
/* Zou-He (jyulb/bcs.pyx).  `ax` is the face axis, `s` = -1 for the low face */
/* (outward normal -e_ax) and +1 for the high face.                          */
/* ------------------------------------------------------------------------ */
/* The reference writes each face with its own literal sums; the summation   */
/* orders below reproduce them exactly.                                       */
static const int ZH_KN[6][14] = {
    /* 1X */ {9, 2, 6, 12, 8, 5, 11, 1, 0, 4, 10, 7, 13, 3},
    /* X1 */ {9, 16, 6, 12, 8, 5, 11, 15, 14, 18, 10, 7, 13, 17},
    /* 1Y */ {9, 2, 16, 6, 8, 5, 1, 15, 0, 14, 10, 7, 3, 17},
    /* Y1 */ {9, 2, 16, 12, 8, 11, 1, 15, 4, 18, 10, 13, 3, 17},
    /* 1Z */ {9, 2, 16, 6, 12, 8, 5, 11, 1, 15, 0, 18, 14, 4},
    /* Z1 */ {9, 2, 16, 6, 12, 10, 7, 13, 3, 17, 0, 18, 14, 4},
};
/* populations leaving through the face (known), in the reference's order */
static const int ZH_OUT[6][5] = {
    /* 1X */ {2, 1, 0, 4, 3},
    /* X1 */ {16, 15, 14, 18, 17},
    /* 1Y */ {6, 5, 0, 14, 7},
    /* Y1 */ {12, 11, 4, 18, 13},
    /* 1Z */ {8, 5, 11, 1, 15},
    /* Z1 */ {10, 7, 13, 3, 17},
};

static double sum_idx(const double *f, const int *idx, int n) {
    double s = f[idx[0]];
    for (int m = 1; m < n; ++m) s = s + f[idx[m]];
    return s;
}

/* unknown-population assignment, jyulb/bcs.pyx:487-716 */
static void zh_assign(int face, double jx, double jy, double jz, double *f) {
    const double s6 = 1.0/6.0, s3 = 1.0/3.0;
    double t;
    switch (face) {
    case F1X:
        t = f[11] + f[12] + f[13] - f[5] - f[6] - f[7];
        f[14] = f[4] + s6*jx + 0.5*t - 0.5*jy;
        f[18] = f[0] + s6*jx - 0.5*t + 0.5*jy;
        t = f[7] + f[10] + f[13] - f[5] - f[8] - f[11];
        f[15] = f[3] + s6*jx + 0.5*t - 0.5*jz;
        f[17] = f[1] + s6*jx - 0.5*t + 0.5*jz;
        f[16] = f[2] + s3*jx;
        break;
    case FX1:
        t = f[11] + f[12] + f[13] - f[5] - f[6] - f[7];
        f[0] = f[18] - s6*jx + 0.5*t - 0.5*jy;
        f[4] = f[14] - s6*jx - 0.5*t + 0.5*jy;
        t = f[7] + f[10] + f[13] - f[5] - f[8] - f[11];
        f[1] = f[17] - s6*jx + 0.5*t - 0.5*jz;
        f[3] = f[15] - s6*jx - 0.5*t + 0.5*jz;
        f[2] = f[16] - s3*jx;
        break;
    case F1Y:
        t = f[15] + f[16] + f[17] - f[1] - f[2] - f[3];
        f[4] = f[14] + s6*jy + 0.5*t - 0.5*jx;
        f[18] = f[0] + s6*jy - 0.5*t + 0.5*jx;
        t = f[17] + f[10] + f[3] - f[15] - f[8] - f[1];
        f[11] = f[7] + s6*jy + 0.5*t - 0.5*jz;
        f[13] = f[5] + s6*jy - 0.5*t + 0.5*jz;
        f[12] = f[6] + s3*jy;
        break;
    case FY1:
        t = f[15] + f[16] + f[17] - f[1] - f[2] - f[3];
        f[0] = f[18] - s6*jy + 0.5*t - 0.5*jx;
        f[14] = f[4] - s6*jy - 0.5*t + 0.5*jx;
        t = f[17] + f[10] + f[3] - f[15] - f[8] - f[1];
        f[5] = f[13] - s6*jy + 0.5*t - 0.5*jz;
        f[7] = f[11] - s6*jy - 0.5*t + 0.5*jz;
        f[6] = f[12] - s3*jy;
        break;
    case F1Z:
        t = f[18] + f[16] + f[14] - f[4] - f[2] - f[0];
        f[3] = f[15] + s6*jz + 0.5*t - 0.5*jx;
        f[17] = f[1] + s6*jz - 0.5*t + 0.5*jx;
        t = f[18] + f[12] + f[4] - f[14] - f[6] - f[0];
        f[7] = f[11] + s6*jz + 0.5*t - 0.5*jy;
        f[13] = f[5] + s6*jz - 0.5*t + 0.5*jy;
        f[10] = f[8] + s3*jz;
        break;
    default: /* FZ1 */
        t = f[18] + f[16] + f[14] - f[4] - f[2] - f[0];
        f[1] = f[17] - s6*jz + 0.5*t - 0.5*jx;
        f[15] = f[3] - s6*jz - 0.5*t + 0.5*jx;
        t = f[18] + f[12] + f[4] - f[14] - f[6] - f[0];
        f[5] = f[13] - s6*jz + 0.5*t - 0.5*jy;
        f[11] = f[7] - s6*jz - 0.5*t + 0.5*jy;
        f[8] = f[10] - s3*jz;
        break;
    }
}

/* jyulb/bcs.pyx:31-482: fixed density (kind=FIXED_DEN) or velocity */
static void zou_he(int face, int kind, double den, const double *vel, double *f) {
    int ax = face >> 1;            /* 0,1,2 */
    int high = face & 1;           /* 0: low face, 1: high face */
    double kn = sum_idx(f, ZH_KN[face], 14);
    double out = sum_idx(f, ZH_OUT[face], 5);
    double j[3];
    if (kind == FIXED_DEN) {
        /* normal momentum from the density; tangential from vel */
        double jn = high ? (out - (den - kn)) : ((den - kn) - out);
        for (int d = 0; d < 3; ++d) j[d] = den * vel[d];
        j[ax] = jn;
    } else {
        double dbc = high ? (kn + out) / (1.0 + vel[ax]) : (kn + out) / (1.0 - vel[ax]);
        for (int d = 0; d < 3; ++d) j[d] = dbc * vel[d];
    }
    zh_assign(face, j[0], j[1], j[2], f);
}

/* ------------------------------------------------------------------------ */
/* Halo fills (jyulb/isothermal.pyx:509-837)                                 */
/* ------------------------------------------------------------------------ */
/* axis ax (0,1,2), low face (side 0) or high face (side 1)                  */
static void halo_pos(const orc_t *o, int ax, int side, int *rd, int *wr, int per) {
    int N = ax == 0 ? o->NI : ax == 1 ? o->NJ : o->NK;
    if (side == 0) { *rd = 1;     *wr = per ? N - 1 : 0; }
    else           { *rd = N - 2; *wr = per ? 0 : N - 1; }
}

/* iterate the face plane with the reference's coverage: x faces interior j,k;
 * y faces all i, interior k; z faces all i,j */
#define FACE_LOOP(o, ax, ...)                                               \
    do {                                                                    \
        int a0 = (ax == 0) ? 1 : 0;                                          \
        int b0 = (ax == 2) ? 0 : 1;                                          \
        int A = (ax == 0) ? (o)->NJ - 1 : (o)->NI;                           \
        int B = (ax == 2) ? (o)->NJ : (o)->NK - 1;                           \
        for (int ua = a0; ua < A; ++ua)                                      \
            for (int ub = b0; ub < B; ++ub) { __VA_ARGS__ }                  \
    } while (0)

static void plane_idx(int ax, int c, int ua, int ub, int *i, int *j, int *k) {
    if (ax == 0) { *i = c; *j = ua; *k = ub; }
    else if (ax == 1) { *i = ua; *j = c; *k = ub; }
    else { *i = ua; *j = ub; *k = c; }
}

static void enforce_phase(orc_t *o) {
    for (int face = 0; face < 6; ++face) {
        int b = o->bc[face], ax = face >> 1, side = face & 1;
        if (b != PERIODIC && b != SYMMETRIC) continue;
        int rd, wr;
        halo_pos(o, ax, side, &rd, &wr, b == PERIODIC);
        FACE_LOOP(o, ax, {
            int i, j, k, i2, j2, k2;
            plane_idx(ax, rd, ua, ub, &i, &j, &k);
            plane_idx(ax, wr, ua, ub, &i2, &j2, &k2);
            o->phase[NIDX(o, i2, j2, k2)] = o->phase[NIDX(o, i, j, k)];
        });
    }
}

static void enforce_den_vel(orc_t *o) {
    for (int face = 0; face < 6; ++face) {
        int b = o->bc[face], ax = face >> 1, side = face & 1;
        if (b != PERIODIC && b != SYMMETRIC) continue;
        int rd, wr;
        halo_pos(o, ax, side, &rd, &wr, b == PERIODIC);
        FACE_LOOP(o, ax, {
            int i, j, k, i2, j2, k2;
            plane_idx(ax, rd, ua, ub, &i, &j, &k);
            plane_idx(ax, wr, ua, ub, &i2, &j2, &k2);
            long r = NIDX(o, i, j, k), w = NIDX(o, i2, j2, k2);
            o->den[w] = o->den[r];
            for (int d = 0; d < 3; ++d) {
                double v = o->vel[3*r + d];
                o->vel[3*w + d] = (b == SYMMETRIC && d == ax) ? -v : v;
            }
        });
    }
}

/* mirror of direction q across the plane normal to axis ax */
static int mirror_q(int q, int ax) {
    int c[3] = {CI[q], CJ[q], CK[q]};
    c[ax] = -c[ax];
    for (int p = 0; p < Q; ++p)
        if (CI[p] == c[0] && CJ[p] == c[1] && CK[p] == c[2]) return p;
    return -1;
}

static void enforce_distr(orc_t *o) {
    for (int face = 0; face < 6; ++face) {
        int b = o->bc[face], ax = face >> 1, side = face & 1;
        if (b != PERIODIC && b != SYMMETRIC) continue;
        int rd, wr;
        halo_pos(o, ax, side, &rd, &wr, b == PERIODIC);
        /* the five populations leaving through this face */
        int leave[5], nl = 0;
        for (int q = 0; q < Q; ++q) {
            int c = ax == 0 ? CI[q] : ax == 1 ? CJ[q] : CK[q];
            if (c == (side ? 1 : -1)) leave[nl++] = q;
        }
        FACE_LOOP(o, ax, {
            int i, j, k, i2, j2, k2;
            plane_idx(ax, rd, ua, ub, &i, &j, &k);
            long r = NIDX(o, i, j, k);
            if (o->phase[r] == SOLID) continue;
            plane_idx(ax, wr, ua, ub, &i2, &j2, &k2);
            long w = NIDX(o, i2, j2, k2);
            for (int m = 0; m < 5; ++m) {
                int q = leave[m];
                int qw = (b == SYMMETRIC) ? mirror_q(q, ax) : q;
                o->f1[qw * o->ncnt + w] = o->f1[q * o->ncnt + r];
            }
        });
    }
}

/* ------------------------------------------------------------------------ */
/* Pull streaming with Ladd bounce-back (jyulb/isothermal.pyx:1112-1248)     */
/* ------------------------------------------------------------------------ */
static void stream_node(const orc_t *o, int i, int j, int k, long n, double *f) {
    double den = o->den[n];
    double cff1 = 2.0*den*W1*AS2, cff2 = 2.0*den*W2*AS2;
    for (int q = 0; q < Q; ++q) {
        if (q == 9) { f[9] = o->f1[9*o->ncnt + n]; continue; }
        long s = NIDX(o, i - CI[q], j - CJ[q], k - CK[q]);
        if (o->phase[s] != SOLID) { f[q] = o->f1[q*o->ncnt + s]; continue; }
        /* c_q . u_solid evaluated as the reference does: the first nonzero
         * component's sign times (u_a +/- u_b) */
        const double *u = o->vel + 3*s;
        int c[3] = {CI[q], CJ[q], CK[q]};
        int a = -1, bb = -1;
        for (int d = 0; d < 3; ++d) if (c[d]) { if (a < 0) a = d; else bb = d; }
        double t;
        if (bb < 0) t = u[a];
        else t = (c[a] == c[bb]) ? (u[a] + u[bb]) : (u[a] - u[bb]);
        if (c[a] < 0) t = -t;
        double cff = (bb < 0) ? cff1 : cff2;
        f[q] = o->f1[OPP(q)*o->ncnt + n] + cff*t;
    }
}

/* ------------------------------------------------------------------------ */
/* Public API (ctypes)                                                       */
/* ------------------------------------------------------------------------ */
orc_t *orc_create(int nx, int ny, int nz, int scheme, double kvisc,
                  const double *g, const int *bc, double trt_magic) {
    orc_t *o = (orc_t *)calloc(1, sizeof(orc_t));
    o->nx = nx; o->ny = ny; o->nz = nz;
    o->NI = nx + 2; o->NJ = ny + 2; o->NK = nz + 2;
    o->ncnt = (long)o->NI * o->NJ * o->NK;
    o->scheme = scheme; o->kvisc = kvisc;
    for (int d = 0; d < 3; ++d) o->g[d] = g ? g[d] : 0.0;
    for (int s = 0; s < 6; ++s) o->bc[s] = bc ? bc[s] : PERIODIC;
    o->phase = (uint8_t *)calloc(o->ncnt, 1);
    o->den = (double *)malloc(sizeof(double) * o->ncnt);
    for (long n = 0; n < o->ncnt; ++n) o->den[n] = 1.0;
    o->vel = (double *)calloc(3 * o->ncnt, sizeof(double));
    o->acc = (double *)calloc(3 * o->ncnt, sizeof(double));
    o->f1 = (double *)calloc((size_t)Q * o->ncnt, sizeof(double));
    o->f2 = (double *)calloc((size_t)Q * o->ncnt, sizeof(double));
    for (int s = 0; s < 6; ++s) {
        int ax = s >> 1;
        size_t np = (ax == 0) ? (size_t)o->NJ * o->NK : ax == 1 ? (size_t)o->NI * o->NK
                                                        : (size_t)o->NI * o->NJ;
        o->bcden[s] = (double *)malloc(sizeof(double) * np);
        for (size_t m = 0; m < np; ++m) o->bcden[s][m] = 1.0;
        o->bcvel[s] = (double *)calloc(3 * np, sizeof(double));
    }
    /* tau = 1/2 + 3 nu; TRT odd rate from the magic parameter
     * (jyulb/isothermal.pyx:274-287; trt_magic <= 0 selects the reference's
     * fixed expression 8(2-w)/(8-w), i.e. magic 3/16) */
    double tau_e = 0.5 + AS2 * kvisc;
    o->prm0 = 1.0 / tau_e;
    if (scheme == TRT) {
        if (trt_magic > 0.0) o->prm1 = 1.0 / (trt_magic / (tau_e - 0.5) + 0.5);
        else o->prm1 = 8.0 * (2.0 - o->prm0) / (8.0 - o->prm0);
    }
    return o;
}

void orc_destroy(orc_t *o) {
    if (!o) return;
    free(o->phase); free(o->den); free(o->vel); free(o->acc);
    free(o->f1); free(o->f2); free(o->fluid);
    for (int s = 0; s < 6; ++s) { free(o->bcden[s]); free(o->bcvel[s]); }
    free(o);
}

/* raw access to the halo-padded arrays (tests wrap them as numpy arrays) */
uint8_t *orc_phase(orc_t *o) { return o->phase; }
double *orc_den(orc_t *o) { return o->den; }
double *orc_vel(orc_t *o) { return o->vel; }
double *orc_acc(orc_t *o) { return o->acc; }
double *orc_f(orc_t *o) { return o->f1; }
void orc_set_gravity(orc_t *o, const double *g) { for (int d = 0; d < 3; ++d) o->g[d] = g[d]; }
double orc_prm(orc_t *o, int m) { return m ? o->prm1 : o->prm0; }
long orc_nfluid(orc_t *o) { return o->nfluid; }

/* velocity gradient by (biased) central differences,
 * jyulb/isothermal.pyx:958-1023 */
static const int FDIR[3][5] = {{14, 15, 16, 17, 18}, {4, 11, 12, 13, 18}, {3, 7, 10, 13, 17}};
static const double LWQ[Q] = {W2, W2, W1, W2, W2, W2, W1, W2, W1, W0, W1, W2, W1, W2, W2, W2, W1, W2, W2};

static void der_vel(const orc_t *o, int i, int j, int k, int dir, const double *v, double *dv) {
    dv[0] = dv[1] = dv[2] = 0.0;
    for (int m = 0; m < 5; ++m) {
        int l = FDIR[dir][m];
        long nn = NIDX(o, i + CI[l], j + CJ[l], k + CK[l]);
        long no = NIDX(o, i - CI[l], j - CJ[l], k - CK[l]);
        double c1 = 0.5, c2 = 0.0, c3 = -0.5;
        if (o->phase[nn] == SOLID) {
            if (o->phase[no] == SOLID) { c1 = 1.0; c3 = -1.0; }
            else { c1 = 4.0/3.0; c2 = -1.0; c3 = -1.0/3.0; }
        } else if (o->phase[no] == SOLID) {
            c1 = 1.0/3.0; c2 = 1.0; c3 = -4.0/3.0;
        }
        double c0 = 2.0*LWQ[l]*AS2;
        for (int d = 0; d < 3; ++d)
            dv[d] += c0*(c1*o->vel[3*nn + d] + c2*v[d] + c3*o->vel[3*no + d]);
    }
}

/* finalize_init: fluid list, halo fills, initial populations
 * (jyulb/isothermal.pyx:1333-1365, 1028-1105) */
long orc_finalize(orc_t *o) {
    long cnt = 0;
    for (int i = 1; i < o->NI - 1; ++i)
        for (int j = 1; j < o->NJ - 1; ++j)
            for (int k = 1; k < o->NK - 1; ++k)
                if (o->phase[NIDX(o, i, j, k)] != SOLID) ++cnt;
    o->nfluid = cnt;
    if (cnt > 0) {
        o->fluid = (long *)malloc(sizeof(long) * cnt);
        long m = 0;
        for (int i = 1; i < o->NI - 1; ++i)
            for (int j = 1; j < o->NJ - 1; ++j)
                for (int k = 1; k < o->NK - 1; ++k) {
                    long n = NIDX(o, i, j, k);
                    if (o->phase[n] != SOLID) o->fluid[m++] = n;
                }
        enforce_phase(o);
        enforce_den_vel(o);
        double inv_tau = o->prm0, tau = 1.0 / inv_tau, rc = 1.0 - inv_tau;
        for (long m2 = 0; m2 < cnt; ++m2) {
            long n = o->fluid[m2];
            int i = (int)(n / ((long)o->NJ * o->NK));
            int j = (int)((n / o->NK) % o->NJ);
            int k = (int)(n % o->NK);
            double den = o->den[n], v[3] = {o->vel[3*n], o->vel[3*n+1], o->vel[3*n+2]};
            double h[10], dx[3], dy[3], dz[3], f[Q];
            den_vel_to_heq(den, v, h);
            der_vel(o, i, j, k, 0, v, dx);
            der_vel(o, i, j, k, 1, v, dy);
            der_vel(o, i, j, k, 2, v, dz);
            double m2c = -2.0*tau*INV_AS2*den;
            h[4] += rc*m2c*dx[0];
            h[5] += rc*m2c*0.5*(dx[1] + dy[0]);
            h[6] += rc*m2c*0.5*(dx[2] + dz[0]);
            h[7] += rc*m2c*dy[1];
            h[8] += rc*m2c*0.5*(dy[2] + dz[1]);
            h[9] += rc*m2c*dz[2];
            project(h, f, 0);
            for (int q = 0; q < Q; ++q) o->f1[q*o->ncnt + n] = f[q];
        }
    }
    o->init_done = 1;
    return cnt;
}

/* bc data from the den/vel face layers, jyulb/isothermal.pyx:476-502 */
static void set_bc_data(orc_t *o) {
    for (int s = 0; s < 6; ++s) {
        int fixed = o->bc[s] == FIXED_DEN || o->bc[s] == FIXED_VEL;
        /* the reference tests bc[FACE_1Z] for the velocity case of face Z1 */
        if (s == FZ1) fixed = o->bc[FZ1] == FIXED_DEN || o->bc[F1Z] == FIXED_VEL;
        if (!fixed) continue;
        int ax = s >> 1;
        int N = ax == 0 ? o->NI : ax == 1 ? o->NJ : o->NK;
        int c = (s & 1) ? N - 2 : 1;
        long m = 0;
        int A = ax == 0 ? o->NJ : o->NI, B = ax == 2 ? o->NJ : o->NK;
        for (int ua = 0; ua < A; ++ua)
            for (int ub = 0; ub < B; ++ub, ++m) {
                int i, j, k;
                plane_idx(ax, c, ua, ub, &i, &j, &k);
                long n = NIDX(o, i, j, k);
                o->bcden[s][m] = o->den[n];
                for (int d = 0; d < 3; ++d) o->bcvel[s][3*m + d] = o->vel[3*n + d];
            }
    }
}

static void face_bc(orc_t *o, int s, int i, int j, int k, double *f) {
    int ax = s >> 1;
    long m = ax == 0 ? (long)j * o->NK + k : ax == 1 ? (long)i * o->NK + k
                                                     : (long)i * o->NJ + j;
    zou_he(s, o->bc[s], o->bcden[s][m], o->bcvel[s] + 3*m, f);
}

/* evolve(tsteps), jyulb/isothermal.pyx:1370-1418; returns total steps or
 * (unsigned)-1 when called before finalize */
unsigned orc_evolve(orc_t *o, unsigned tsteps) {
    if (!o->init_done) return (unsigned)-1;
    set_bc_data(o);
    if (o->nfluid < 1) return o->tot_tsteps;
    for (unsigned t = 0; t < tsteps; ++t) {
        enforce_distr(o);
        enforce_den_vel(o);
        for (long m = 0; m < o->nfluid; ++m) {
            long n = o->fluid[m];
            int i = (int)(n / ((long)o->NJ * o->NK));
            int j = (int)((n / o->NK) % o->NJ);
            int k = (int)(n % o->NK);
            double f[Q], a[3], v[3], den;
            stream_node(o, i, j, k, n, f);
            int fx = (o->bc[F1X] == FIXED_DEN || o->bc[F1X] == FIXED_VEL);
            if (i == 1 && fx) face_bc(o, F1X, i, j, k, f);
            if (i == o->NI - 2 && (o->bc[FX1] == FIXED_DEN || o->bc[FX1] == FIXED_VEL)) face_bc(o, FX1, i, j, k, f);
            if (j == 1 && (o->bc[F1Y] == FIXED_DEN || o->bc[F1Y] == FIXED_VEL)) face_bc(o, F1Y, i, j, k, f);
            if (j == o->NJ - 2 && (o->bc[FY1] == FIXED_DEN || o->bc[FY1] == FIXED_VEL)) face_bc(o, FY1, i, j, k, f);
            if (k == 1 && (o->bc[F1Z] == FIXED_DEN || o->bc[F1Z] == FIXED_VEL)) face_bc(o, F1Z, i, j, k, f);
            if (k == o->NK - 2 && (o->bc[FZ1] == FIXED_DEN || o->bc[FZ1] == FIXED_VEL)) face_bc(o, FZ1, i, j, k, f);
            for (int d = 0; d < 3; ++d) a[d] = o->g[d] + o->acc[3*n + d];
            if (o->scheme == BGK) den = coll_bgk(f, a, o->prm0, v);
            else if (o->scheme == TRT) den = coll_trt(f, a, o->prm0, o->prm1, v);
            else den = coll_reg(f, a, o->prm0, v);
            o->den[n] = den;
            for (int d = 0; d < 3; ++d) o->vel[3*n + d] = v[d];
            for (int q = 0; q < Q; ++q) o->f2[q*o->ncnt + n] = f[q];
        }
        double *sw = o->f1; o->f1 = o->f2; o->f2 = sw;
    }
    o->tot_tsteps += tsteps;
    return o->tot_tsteps;
}
