/*
 * jyulb_gb300.h -- C ABI of the GB300 D3Q19 isothermal lattice-Boltzmann
 * engine (libjyulb_gb300.so).
 *
 * The reference exposes this path only as the Cython class
 * jyulb.isothermal.Solver (jyulb/isothermal.pxd:38-114); it has no C ABI.
 * Each entry point below replaces one step of that class's life cycle and
 * cites it.  Conventions:
 *   - plain pointers and sizes only; every host array uses the reference's
 *     halo-padded C-order layout, (NI,NJ,NK) = (nx+2, ny+2, nz+2) with k
 *     fastest, and (NI,NJ,NK,3) for vectors (jyulb/isothermal.pyx:234-248);
 *   - functions return JLB_OK (0) or a negative status, never exit or trap;
 *     jlb_last_error() gives the message for the last failure;
 *   - a solver runs on one CUDA stream (its own unless one is supplied);
 *     calls on one solver must not overlap (the same rule as the reference's
 *     single Python object).
 */
#ifndef JYULB_GB300_H
#define JYULB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define JLB_OK 0
#define JLB_ERR_INVALID_ARG (-1) /* ValueError in the reference          */
#define JLB_ERR_STATE (-2)       /* RuntimeError in the reference        */
#define JLB_ERR_CUDA (-3)        /* CUDA runtime failure                 */
#define JLB_ERR_NOMEM (-4)       /* device or host allocation failure    */
#define JLB_ERR_UNSUPPORTED (-5) /* valid request this build cannot run  */
#define JLB_ERR_NUMERIC (-6)     /* NaN/Inf found by a reduction         */

/* enumerations, values as in jyulb/defs.pxd:17-103 */
#define JLB_BGK 0
#define JLB_TRT 1
#define JLB_REGULARIZATION 2
#define JLB_WALL 0
#define JLB_PERIODIC 1
#define JLB_FIXED_DEN 2
#define JLB_FIXED_VEL 3
#define JLB_SYMMETRIC 4
#define JLB_SOLID 0
#define JLB_FLUID 1

/* collision model of the time step */
#define JLB_KERNEL_JYULB 0 /* the Python reference's (jyulb/D3Q19.pyx:655-940)  */
#define JLB_KERNEL_CXX 1   /* the reference C++ executable's
                              (include/kernel/kernel.cpp:410-550): FP64, BGK
                              or TRT, periodic/wall faces, resting solids      */
/* kernel_opts of JLB_KERNEL_CXX (its flow type and forcing switches,
 * include/kernel/kernel.cpp:423-427) */
#define JLB_CXX_LINEAR_EQ 1 /* linear ("Stokes flow") equilibrium            */
#define JLB_CXX_FORCE2 2    /* second-order forcing ("external forcing")     */

/* population storage / arithmetic of the time step */
#define JLB_FP64 0 /* FP64 storage and arithmetic (parity path)          */
#define JLB_FP32 1 /* FP32 storage of f_i - w_i, FP32 arithmetic          */
#define JLB_FP16 2 /* FP16 storage of 2^12 (f_i/w_i - 1), FP32 arithmetic */
#define JLB_FP64_FAST 3 /* FP64 storage and arithmetic, regrouped and FMA-
                           contracted: within 1e-12 relative of JLB_FP64,
                           not bit for bit (the reference has no such mode) */

typedef struct jlb_solver jlb_solver;

typedef struct jlb_config {
    int32_t lat_size[3]; /* interior lattice sites per axis (>= 1)          */
    int32_t rlx_scheme;  /* JLB_BGK / JLB_TRT / JLB_REGULARIZATION           */
    double kvisc;        /* kinematic viscosity, > 0                         */
    double g[3];         /* uniform gravity                                  */
    int32_t bc[6];       /* per face 1X,X1,1Y,Y1,1Z,Z1: JLB_WALL..SYMMETRIC  */
    int32_t precision;   /* JLB_FP64 / JLB_FP32 / JLB_FP16 / JLB_FP64_FAST   */
    double trt_magic;    /* TRT magic parameter; <= 0 selects the reference's
                            fixed 8(2-w)/(8-w) odd rate (magic 3/16)         */
    int32_t kernel;      /* JLB_KERNEL_JYULB (0) or JLB_KERNEL_CXX           */
    int32_t kernel_opts; /* JLB_CXX_* flags for JLB_KERNEL_CXX               */
    void *stream;        /* cudaStream_t to run on, or NULL                  */
} jlb_config;
/* With JLB_KERNEL_CXX, kvisc is the executable's dimensionless viscosity
 * (tau = 0.5 + nu / c_s^2 with its c_s^2 = (1/sqrt 3)^2), g is its
 * dimensionless gravity and the per-site acc field holds a dimensionless
 * force density F_ext (the executable's F = F_ext + rho g) instead of an
 * acceleration. */

/* Argument validation of Solver.__cinit__ / _check_bc
 * (jyulb/isothermal.pyx:196-206, 378-426).  Writes the reference's message
 * into msg (if not NULL) and returns JLB_ERR_INVALID_ARG on failure.  One
 * check has no reference counterpart: nx * ny must stay below 2^31. */
int jlb_check_config(const jlb_config *cfg, char *msg, size_t msg_len);

/* Solver.__cinit__ (jyulb/isothermal.pyx:156-298): validate, derive the
 * relaxation rates, allocate device state.  Needs a CUDA device. */
int jlb_create(const jlb_config *cfg, jlb_solver **out);

/* releases device state; NULL is ignored */
void jlb_destroy(jlb_solver *s);

/* Solver.finalize_init (jyulb/isothermal.pyx:1333-1365): applies the
 * periodic/symmetric halo rules to phase, den and vel in place (as the
 * reference does to its own arrays), classifies nodes, and sets the initial
 * populations from den, vel and their finite-difference gradients
 * (jyulb/isothermal.pyx:958-1105).  *nfluid receives the fluid-site count. */
int jlb_finalize_init(jlb_solver *s, uint8_t *phase, double *den, double *vel,
                      uint64_t *nfluid);

/* Solver.evolve (jyulb/isothermal.pyx:1370-1418): re-reads the per-call
 * inputs from the host arrays (Zou-He face data from the den/vel face layers,
 * velocities of solid sites, den of sites next to moving solids, acc when
 * acc != NULL), advances tsteps steps on the GPU, and writes the
 * pre-collision density and velocity back into den and vel.  g is the
 * gravity for this call (Solver.gravity).  *tot receives the total step
 * count.  The halo layers of den/vel are refreshed from the boundary layers
 * at the start of the call. */
int jlb_evolve(jlb_solver *s, uint32_t tsteps, const double g[3], double *den,
               double *vel, const double *acc, uint32_t *tot);

/* With on != 0 the caller promises not to write den/vel in the halo cells of
 * WALL, FIXED_DEN and FIXED_VEL faces after jlb_finalize_init, as with the
 * reference's Solver, whose getters reach the interior only
 * (jyulb/isothermal.pyx:1465-1511).  jlb_evolve then re-reads solid
 * velocities only in the interior and in the halo cells of periodic and
 * symmetric faces, which its halo rules refresh from the interior.  Off by
 * default; no reference counterpart. */
int jlb_set_static_halo(jlb_solver *s, int on);

/* Uploads the per-site field of the halo-padded (NI,NJ,NK,3) array acc
 * (acceleration, or force density with JLB_KERNEL_CXX) now, so that
 * jlb_finalize_init uses it: the C++ executable's initial state includes the
 * forcing term (include/kernel/kernel.cpp:339-345).  jlb_evolve with a
 * non-NULL acc re-reads it as before; an all-zero or NULL acc switches the
 * field off. */
int jlb_set_acc(jlb_solver *s, const double *acc);

/* Device-only stepping with the inputs of the last jlb_evolve call: no host
 * synchronisation, no host arrays.  write_moments != 0 stores den/vel of the
 * last step on the device (read them with jlb_download_moments).  A step
 * kernel whose bounded wait on its bulk copies ran out is reported by the
 * next jlb_evolve, jlb_download_moments or jlb_get_populations call; the
 * solver keeps reporting it until jlb_finalize_init or jlb_set_populations
 * gives it a whole state again. */
int jlb_step(jlb_solver *s, uint32_t tsteps, int write_moments);

/* copies the device den/vel of the last moment-writing step into the
 * interior of the host arrays (layout as above) */
int jlb_download_moments(jlb_solver *s, double *den, double *vel);

/* Post-collision populations of the latest step as FP64, shape
 * (19, nx, ny, nz) in the reference's lattice-vector order
 * (jyulb/D3Q19.pxd:59-79); the reference keeps the same values in Solver.f1
 * (Bundle-C order, jyulb/isothermal.pyx:1532-1704).  Solid sites read 0. */
int jlb_get_populations(jlb_solver *s, double *f);

/* overwrites the populations (same layout); used to restore a saved state */
int jlb_set_populations(jlb_solver *s, const double *f);

/* FP64 reductions over fluid sites of the last moment-writing step:
 * out[0] = sum den, out[1..3] = sum den*u (stored u), out[4..6] = sum u,
 * out[7] = number of non-finite den/u values found. */
int jlb_reduce(jlb_solver *s, double out[8]);

/* Steady-state convergence residual of the last moment-writing step:
 * *res = ||u - u_prev|| / ||u|| over fluid sites (L2 norms, FP64 sums on the
 * GPU), where u_prev is the velocity at the previous call (zero before the
 * first one, which therefore returns 1 unless u = 0).  No reference
 * counterpart; the examples track convergence through printed sums. */
int jlb_residual(jlb_solver *s, double *res);

/* Flow information of the last moment-writing step, as the C++ executable's
 * IsothermalSolver::calc_flow_info (include/solver/solver.cpp:64-129)
 * computes it over fluid sites, in the column order of its .evol file
 * (source/isothermal/jyu_lb_isothermal.cpp:21-56):
 *   out[0] sum den, out[1..3] sum den*u, out[4] sum den*|u|,
 *   out[5..7] mean u, out[8] mean |u|, out[9] max |u|, out[10] max den,
 *   out[11] min den.
 * The extremes start from ref_den (density) and 0 (speed), as there.  Sums
 * are FP64 on the GPU in a fixed order. */
int jlb_flow_info(jlb_solver *s, double ref_den, double out[12]);

/* Allocation-free variant of jlb_reduce, for callers that cannot call
 * cudaMalloc (code inside another framework's memory pool, hosts that forbid
 * allocation after start-up, drivers that budget device memory themselves).
 * It has no counterpart in the reference.
 *   nmask            n_sites node masks; sites with bit 31 set are skipped
 *   den, ux, uy, uz  n_sites moments: double for JLB_FP64, float holding
 *                    den - 1 (and u) for JLB_FP32 / JLB_FP16
 *   out              8 doubles in device-writable memory, same meaning as
 *                    jlb_reduce's out
 *   stream           cudaStream_t (NULL: legacy default stream); the call
 *                    only enqueues work, synchronise before reading out
 * All pointers are device-accessible.  n_sites may be at most 2^28 (268435456)
 * sites; larger or non-positive sizes return JLB_ERR_INVALID_ARG.  Scratch is
 * a static device array of 256 KiB that every GPU loading the library keeps
 * until the process exits; the first call on each device looks up its address
 * and should therefore come before any stream capture (a lookup that failed is
 * retried by the next call).  All calls share that array (each call writes
 * every partial it reads), so calls that overlap on the GPU race: serialise
 * them, e.g. on one stream.  The call clears the CUDA runtime's last-error
 * slot on entry, so that an error left there by an earlier launch is not
 * reported as its own. */
int jlb_reduce_moments_noalloc(const uint32_t *nmask, const void *den, const void *ux, const void *uy,
                               const void *uz, int64_t n_sites, int32_t precision, double *out, void *stream);

/* ---------------------------------------------------------------------
 * Batched ensemble: many independent domains advanced by one launch per
 * step over a packed node index.  The reference advances one Solver at a
 * time (jyulb/isothermal.pyx:1370-1418); an ensemble of its channels is a
 * loop over Solver objects, which these calls replace.  Populations are
 * FP32 shifted.  Domains whose faces are all WALL or PERIODIC and whose
 * moving solids share one velocity (Ladd's term,
 * jyulb/isothermal.pyx:1117-1119) run entirely in the packed step kernel;
 * domains with Zou-He or symmetric faces, or with several solid velocities,
 * run their boundary nodes through a second launch per step over a
 * boundary-node list, as the single-domain solver does.
 * --------------------------------------------------------------------- */
typedef struct jlb_batch jlb_batch;

typedef struct jlb_domain {
    int32_t lat_size[3];  /* interior sites per axis                         */
    double kvisc;         /* kinematic viscosity                             */
    double g[3];          /* body force                                      */
    int32_t bc[6];        /* JLB_WALL .. JLB_SYMMETRIC per face; Zou-He data
                             come from den / vel at jlb_batch_create          */
    double trt_magic;     /* as in jlb_config                                */
    const uint8_t *phase; /* (nx,ny,nz) interior phase, k fastest, 0 = solid */
    const double *den;    /* (nx,ny,nz) initial density or NULL (1)          */
    const double *vel;    /* (nx,ny,nz,3) initial velocity / solid velocity, or NULL */
} jlb_domain;

/* Sets up all domains (the single-domain halo rules, masks and initial
 * populations of each, jyulb/isothermal.pyx:1333-1365) and picks the block
 * size with a timing autotuner (JLB_BATCH_BLOCK=64/128/256 fixes it). */
int jlb_batch_create(int32_t rlx_scheme, const jlb_domain *doms, int32_t ndom, void *stream, jlb_batch **out);
void jlb_batch_destroy(jlb_batch *b);
/* advances every domain tsteps steps (one launch per step, graph-replayed);
 * moments of the last step are stored */
int jlb_batch_step(jlb_batch *b, uint32_t tsteps);
/* Zou-He data of domain d from den (nx,ny,nz) / vel (nx,ny,nz,3) at its
 * boundary sites, as Solver.evolve re-reads them at every call
 * (jyulb/isothermal.pyx:476-502, :1398): the fixed faces; Z1 only when
 * bc[Z1] is FIXED_DEN or bc[1Z] is FIXED_VEL (:500).  When den is given, the
 * domain's sites also take it as their previous-step density (Ladd's term of
 * moving solids), as Solver.evolve does.  Solid velocities stay as created.
 * Either pointer may be NULL (that field keeps its current values). */
int jlb_batch_set_bc(jlb_batch *b, int32_t d, const double *den, const double *vel);
/* den (nx,ny,nz) and vel (nx,ny,nz,3) of domain d on its fluid sites */
int jlb_batch_moments(jlb_batch *b, int32_t d, double *den, double *vel);
/* post-collision populations of domain d, (19, nx, ny, nz) FP64 */
int jlb_batch_populations(jlb_batch *b, int32_t d, double *f);
/* out: total packed sites, fluid sites, block size, tiles, launches, and the
 * autotuner's per-step times (microseconds) for blocks of 64, 128, 256 */
int jlb_batch_info(const jlb_batch *b, int64_t out[8]);
int32_t jlb_batch_domain_fluid(const jlb_batch *b, int32_t d);
const char *jlb_batch_last_error(const jlb_batch *b);

/* ---------------------------------------------------------------------
 * Discrete adjoint of the time step (no counterpart in the reference, which
 * has no derivatives).  A problem is a domain described by a jlb_config:
 * BGK, TRT or regularized, FP64 or FP32, started from rest, with immobile or
 * moving solids; its parameters are the relaxation time tau, the body force g
 * and the Zou-He data of its fixed faces (jlb_adj_forward: the u_x of each
 * site of a FIXED_VEL face 1X; jlb_adj_forward_fields: den and vel of every
 * boundary site of any fixed face).
 * The loss is sum |u - target|^2 of the stored velocity on the plane
 * x = loss_plane after the last step.  The forward run keeps checkpoints
 * every checkpoint_every steps; the backward run recomputes each segment and
 * sweeps the adjoint step back through it.
 * --------------------------------------------------------------------- */
typedef struct jlb_adjoint jlb_adjoint;

int jlb_adj_create(const jlb_config *cfg, const uint8_t *phase, int32_t loss_plane, int32_t checkpoint_every,
                   jlb_adjoint **out);
void jlb_adj_destroy(jlb_adjoint *a);
/* uin: (ny,nz) inlet u_x; target: (ny,nz,3) or NULL; u_plane: (ny,nz,3) out
 * or NULL; rho_out: density of FIXED_DEN faces */
int jlb_adj_forward(jlb_adjoint *a, double tau, const double g[3], const double *uin, double rho_out,
                    uint32_t steps, const double *target, double *loss, double *u_plane);
/* gradients of the last forward run's loss; duin: (ny,nz) */
int jlb_adj_backward(jlb_adjoint *a, double *dtau, double dg[3], double *duin);
/* As jlb_adj_create, with moving solids: solid_vel (nx,ny,nz,3) is read at
 * the solid sites, like Solver.vel at phase == SOLID, and enters the links
 * into them through Ladd's term 6 w_q den_prev (c_q . u_wall)
 * (jyulb/isothermal.pyx:1112-1248); the reverse sweep carries the adjoint of
 * each boundary site's previous-step density. */
int jlb_adj_create_moving(const jlb_config *cfg, const uint8_t *phase, const double *solid_vel, int32_t loss_plane,
                          int32_t checkpoint_every, jlb_adjoint **out);
/* Forward run from rest whose inputs come from den (nx,ny,nz) and vel
 * (nx,ny,nz,3) where Solver.evolve reads them at its call: the Zou-He data of
 * the boundary sites (jyulb/isothermal.pyx:476-502), on every FIXED_VEL and
 * FIXED_DEN face, any of the six (Z1 only when bc[Z1] is FIXED_DEN or bc[1Z]
 * is FIXED_VEL, :500; the others keep den 1, vel 0), and the first step's
 * previous-step density of the sites next to moving solids (Ladd's term).
 * NULL den or vel: 1 or 0 everywhere. */
int jlb_adj_forward_fields(jlb_adjoint *a, double tau, const double g[3], const double *den, const double *vel,
                           uint32_t steps, const double *target, double *loss, double *u_plane);
/* gradients of the last forward run's loss w.r.t. tau, g and the den / vel
 * values it read (zero elsewhere); dden (nx,ny,nz), dvel (nx,ny,nz,3), either
 * may be NULL.  After jlb_adj_forward, the face-1X u_x entries carry duin and
 * the rest is zero. */
int jlb_adj_backward_fields(jlb_adjoint *a, double *dtau, double dg[3], double *dden, double *dvel);
/* device time (ms, CUDA events on the problem's stream) of the last runs:
 * out[0] forward, out[1] recomputation, out[2] reverse sweep, out[3] the
 * whole backward run */
int jlb_adj_timers(const jlb_adjoint *a, double out[4]);
const char *jlb_adj_last_error(const jlb_adjoint *a);

/* Solver.bc_data_den_face_* / bc_data_vel_face_* (jyulb/isothermal.pxd:159-171):
 * the face layer of den (and vel) for face `face` (0..5 = 1X, X1, 1Y, Y1, 1Z,
 * Z1) as the last jlb_evolve call read it.  Like Solver._set_bc_data
 * (jyulb/isothermal.pyx:476-502), jlb_evolve copies the whole first or last
 * interior layer, halo rows included, at its start (before its checks and
 * halo rules) for the faces the reference refreshes: the fixed faces, and Z1
 * when bc[Z1] is FIXED_DEN or bc[1Z] is FIXED_VEL (:500).  Other faces, and
 * every face before the first call, give den = 1 and vel = 0
 * (jyulb/isothermal.pyx:253-265).  Shapes, C order: x faces (NJ,NK), y faces
 * (NI,NK), z faces (NI,NJ); vel adds a last axis of 3.  den or vel may be
 * NULL.  A host copy; no device work. */
int jlb_bc_data(const jlb_solver *s, int32_t face, double *den, double *vel);

/* number of steps taken since finalize (Solver.tot_tsteps) */
uint32_t jlb_tot_tsteps(const jlb_solver *s);

/* relaxation rates (Solver.rlx_prm): out[0] = 1/tau_even, out[1] = 1/tau_odd */
void jlb_rlx_prm(const jlb_solver *s, double out[2]);

/* number of kernel launches issued by this solver so far */
uint64_t jlb_kernel_launches(const jlb_solver *s);

/* cumulative wall-clock seconds of jlb_evolve's phases: out[0] bc-data copy,
 * halo rules and solid-velocity check, out[1] Zou-He / boundary-node inputs, out[2]
 * acceleration field, out[3] step launches, out[4] step completion and the
 * den/vel download, out[5] whole calls */
void jlb_host_timers(const jlb_solver *s, double out[6]);

/* host<->device bytes moved by this solver so far: out[0] host to device,
 * out[1] device to host (copies and in-place access to page-locked arrays) */
void jlb_transfer_bytes(const jlb_solver *s, uint64_t out[2]);

/* message of the last failure on s (or of the last failed jlb_create when s is
 * NULL); never NULL */
const char *jlb_last_error(const jlb_solver *s);

/* static description of the build (architecture, kernels) */
const char *jlb_build_info(void);

#ifdef __cplusplus
}
#endif
#endif /* JYULB_GB300_H */
