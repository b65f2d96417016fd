// lbm_host.cpp -- host runtime behind the C ABI (include/jyulb_gb300.h).
//
// Owns the device state of one D3Q19 solver, turns the reference's per-call
// semantics (jyulb/isothermal.pyx:1370-1418) into device work, and keeps the
// host-side bookkeeping the kernels need:
//   * halo rules for phase/den/vel (periodic copy, symmetric mirror; x, y, z in
//     the reference's order and index coverage, jyulb/isothermal.pyx:509-686);
//   * the node mask (19 bounce-back bits per fluid node) and the boundary-node
//     tables (Zou-He faces, symmetric-face links, moving solids);
//   * the per-call inputs: Zou-He data from the den/vel face layers (with the
//     reference's Z1 condition, jyulb/isothermal.pyx:500), solid velocities,
//     previous-step density next to moving solids, acceleration field;
//   * step sequencing of the AA pair, captured into CUDA graphs.
// The solver's state (struct jlb_solver) and the helpers the ensemble and
// adjoint host units reuse are declared in lbm_solver.h.
#include <cuda_runtime.h>
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "jyulb_gb300.h"
#include "lbm_aux.h"
#include "lbm_common.h"
#include "lbm_solver.h"

using namespace jlb;
using namespace jlb_host;

namespace jlb_host {

// lattice vectors (reference order)
const int CI[19] = {-1, -1, -1, -1, -1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1};
const int CJ[19] = {-1, 0, 0, 0, 1, -1, -1, -1, 0, 0, 0, 1, 1, 1, -1, 0, 0, 0, 1};
const int CK[19] = {0, -1, 0, 1, 0, -1, 0, 1, -1, 0, 1, -1, 0, 1, 0, -1, 0, 1, 0};

int find_q(int cx, int cy, int cz) {
    for (int q = 0; q < 19; ++q)
        if (CI[q] == cx && CJ[q] == cy && CK[q] == cz) return q;
    return -1;
}

thread_local std::string g_create_error;

int fail(jlb_solver *s, int code, const std::string &msg) {
    if (s) s->err = msg;
    else g_create_error = msg;
    return code;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess)                                                                    \
            return fail(s, e_ == cudaErrorMemoryAllocation ? JLB_ERR_NOMEM : JLB_ERR_CUDA,        \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                      \
    } while (0)

#define CKR(expr)                                                                                 \
    do {                                                                                          \
        int r_ = (expr);                                                                          \
        if (r_ != 0) return fail(s, JLB_ERR_CUDA, std::string(#expr) + ": " +                    \
                                 cudaGetErrorString((cudaError_t)r_));                            \
    } while (0)

bool is_fixed(int b) { return b == BC_FIXED_DEN || b == BC_FIXED_VEL; }

// face-plane iteration with the reference's coverage (x faces: interior j,k;
// y faces: all i, interior k; z faces: all i, j)
template <class F> void face_loop(const jlb_solver *s, int ax, F &&fn) {
    int a0, A, b0, B;
    if (ax == 0) { a0 = 1; A = s->NJ - 1; b0 = 1; B = s->NK - 1; }
    else if (ax == 1) { a0 = 0; A = s->NI; b0 = 1; B = s->NK - 1; }
    else { a0 = 0; A = s->NI; b0 = 0; B = s->NJ; }
    for (int ua = a0; ua < A; ++ua)
        for (int ub = b0; ub < B; ++ub) fn(ua, ub);
}

void plane(int ax, int c, int ua, int ub, int &I, int &J, int &K) {
    if (ax == 0) { I = c; J = ua; K = ub; }
    else if (ax == 1) { I = ua; J = c; K = ub; }
    else { I = ua; J = ub; K = c; }
}

void halo_rw(const jlb_solver *s, int face, int &rd, int &wr) {
    const int ax = face >> 1, side = face & 1;
    const int n = ax == 0 ? s->NI : ax == 1 ? s->NJ : s->NK;
    const bool per = s->cfg.bc[face] == BC_PERIODIC;
    if (side == 0) { rd = 1; wr = per ? n - 1 : 0; }
    else { rd = n - 2; wr = per ? 0 : n - 1; }
}

// jyulb/isothermal.pyx:509-577
void enforce_phase(const jlb_solver *s, uint8_t *phase) {
    for (int face = 0; face < 6; ++face) {
        const int b = s->cfg.bc[face];
        if (b != BC_PERIODIC && b != BC_SYMMETRIC) continue;
        const int ax = face >> 1;
        int rd, wr;
        halo_rw(s, face, rd, wr);
        face_loop(s, ax, [&](int ua, int ub) {
            int I, J, K, I2, J2, K2;
            plane(ax, rd, ua, ub, I, J, K);
            plane(ax, wr, ua, ub, I2, J2, K2);
            phase[fidx(s, I2, J2, K2)] = phase[fidx(s, I, J, K)];
        });
    }
}

// extents (na, nb) of the face arrays of face `face`: x faces (NJ, NK), y
// faces (NI, NK), z faces (NI, NJ) (jyulb/isothermal.pyx:253-265)
void face_extent(const jlb_solver *s, int face, int &na, int &nb) {
    const int ax = face >> 1;
    na = ax == 0 ? s->NJ : s->NI;
    nb = ax == 2 ? s->NJ : s->NK;
}

// faces whose bc data the reference refreshes at every evolve call: the
// fixed faces, with Z1 refreshed when bc[Z1] is FIXED_DEN or bc[1Z] is
// FIXED_VEL (jyulb/isothermal.pyx:476-502, the condition at :500)
bool bc_refreshed(const jlb_solver *s, int face) {
    const int *bc = s->cfg.bc;
    return face == 5 ? (bc[5] == BC_FIXED_DEN || bc[4] == BC_FIXED_VEL) : is_fixed(bc[face]);
}

// Solver._set_bc_data (jyulb/isothermal.pyx:476-502): copies the whole first
// or last interior layer of den / vel (halo rows included) for every
// refreshed face; called at the start of evolve, before the halo rules
void snapshot_bc_data(jlb_solver *s, const double *den, const double *vel) {
    for (int face = 0; face < 6; ++face) {
        if (!bc_refreshed(s, face)) continue;
        const int ax = face >> 1;
        const int layer = (face & 1) ? (ax == 0 ? s->NI : ax == 1 ? s->NJ : s->NK) - 2 : 1;
        int na, nb;
        face_extent(s, face, na, nb);
        std::vector<double> &bd = s->bcd_den[face], &bv = s->bcd_vel[face];
        bd.resize((size_t)na * nb);
        bv.resize((size_t)3 * na * nb);
#pragma omp parallel for schedule(static) if ((int64_t)na * nb > 65536)
        for (int a = 0; a < na; ++a) {
            for (int b = 0; b < nb; ++b) {
                int I, J, K;
                plane(ax, layer, a, b, I, J, K);
                const int64_t n = fidx(s, I, J, K);
                const size_t o = (size_t)a * nb + b;
                bd[o] = den[n];
                bv[3 * o] = vel[3 * n];
                bv[3 * o + 1] = vel[3 * n + 1];
                bv[3 * o + 2] = vel[3 * n + 2];
            }
        }
    }
}

// jyulb/isothermal.pyx:582-686
void enforce_den_vel(const jlb_solver *s, double *den, double *vel) {
    for (int face = 0; face < 6; ++face) {
        const int b = s->cfg.bc[face];
        if (b != BC_PERIODIC && b != BC_SYMMETRIC) continue;
        const int ax = face >> 1;
        int rd, wr;
        halo_rw(s, face, rd, wr);
        face_loop(s, ax, [&](int ua, int ub) {
            int I, J, K, I2, J2, K2;
            plane(ax, rd, ua, ub, I, J, K);
            plane(ax, wr, ua, ub, I2, J2, K2);
            const int64_t r = fidx(s, I, J, K), w = fidx(s, I2, J2, K2);
            den[w] = den[r];
            for (int d = 0; d < 3; ++d) {
                const double v = vel[3 * r + d];
                vel[3 * w + d] = (b == BC_SYMMETRIC && d == ax) ? -v : v;
            }
        });
    }
}

// Halo positions outside a wall / Zou-He face are solid for the time step.
// The reference leaves them SOLID unless a caller writes the halo directly;
// forcing them keeps every fluid halo position mappable to an interior node.
void solidify_closed_halo(const jlb_solver *s, std::vector<uint8_t> &phase) {
    const int n[3] = {s->nx, s->ny, s->nz};
#pragma omp parallel for schedule(static)
    for (int I = 0; I < s->NI; ++I)
        for (int J = 0; J < s->NJ; ++J)
            for (int K = 0; K < s->NK; ++K) {
                const int p[3] = {I - 1, J - 1, K - 1};
                bool closed = false;
                for (int ax = 0; ax < 3; ++ax) {
                    if (p[ax] >= 0 && p[ax] < n[ax]) continue;
                    const int b = s->cfg.bc[2 * ax + (p[ax] < 0 ? 0 : 1)];
                    if (b != BC_PERIODIC && b != BC_SYMMETRIC) closed = true;
                }
                if (closed) phase[fidx(s, I, J, K)] = 0;
            }
}

// c_q . u evaluated as the reference does (jyulb/isothermal.pyx:1122-1248):
// sign of the first nonzero component times (u_a + u_b) or (u_a - u_b)
double ladd_proj(int q, const double *u) {
    const int c[3] = {CI[q], CJ[q], CK[q]};
    int a = -1, b = -1;
    for (int d = 0; d < 3; ++d)
        if (c[d]) { if (a < 0) a = d; else b = d; }
    double t;
    if (b < 0) t = u[a];
    else t = (c[a] == c[b]) ? (u[a] + u[b]) : (u[a] - u[b]);
    return c[a] < 0 ? -t : t;
}

// Maps a halo-padded position that lies outside the interior through the
// periodic / symmetric rules.  Returns the interior node index and updates q
// to the mirrored direction; returns -1 if an axis has no such rule.
int64_t map_halo(const jlb_solver *s, int I, int J, int K, int &q) {
    int c[3] = {CI[q], CJ[q], CK[q]};
    int p[3] = {I - 1, J - 1, K - 1};
    const int n[3] = {s->nx, s->ny, s->nz};
    for (int ax = 0; ax < 3; ++ax) {
        if (p[ax] >= 0 && p[ax] < n[ax]) continue;
        const bool low = p[ax] < 0;
        const int b = s->cfg.bc[2 * ax + (low ? 0 : 1)];
        if (b == BC_PERIODIC) p[ax] = low ? n[ax] - 1 : 0;
        else if (b == BC_SYMMETRIC) { p[ax] = low ? 0 : n[ax] - 1; c[ax] = -c[ax]; }
        else return -1;
    }
    q = find_q(c[0], c[1], c[2]);
    return ((int64_t)p[0] * s->ny + p[1]) * s->nz + p[2];
}

int ensure_pinned(jlb_solver *s, size_t bytes) {
    if (bytes <= s->pinned_bytes) return JLB_OK;
    if (s->pinned) cudaFreeHost(s->pinned);
    s->pinned = nullptr;
    s->pinned_bytes = 0;
    CK(cudaHostAlloc(&s->pinned, bytes, cudaHostAllocDefault));
    s->pinned_bytes = bytes;
    return JLB_OK;
}

// device address of a host array when the GPU can read/write it in place
void *dev_view(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return const_cast<void *>(p);
    if (at.type == cudaMemoryTypeHost && at.devicePointer) return at.devicePointer;
    return nullptr;
}

// ---------------------------------------------------------------------------
// classification
// ---------------------------------------------------------------------------
void build_mask(jlb_solver *s) {
    s->hmask.assign((size_t)s->Np, MASK_SOLID);
    uint64_t cnt = 0;
#pragma omp parallel for reduction(+ : cnt) schedule(static)
    for (int i = 0; i < s->nx; ++i) {
        for (int j = 0; j < s->ny; ++j)
            for (int k = 0; k < s->nz; ++k) {
                const int64_t n = ((int64_t)i * s->ny + j) * s->nz + k;
                const int I = i + 1, J = j + 1, K = k + 1;
                if (s->phase[fidx(s, I, J, K)] == 0) continue;
                uint32_t m = 0;
                for (int q = 0; q < 19; ++q) {
                    if (q == 9) continue;
                    if (s->phase[fidx(s, I - CI[q], J - CJ[q], K - CK[q])] == 0) m |= 1u << q;
                }
                s->hmask[n] = m;
                ++cnt;
            }
    }
    s->nfluid = cnt;
}

// halo positions that the halo rules of jlb_evolve rewrite from the
// interior (periodic and symmetric faces, jyulb/isothermal.pyx:582-686)
std::vector<uint8_t> halo_refreshed(const jlb_solver *s) {
    std::vector<uint8_t> m((size_t)s->NCNT, 0);
    for (int face = 0; face < 6; ++face) {
        const int b = s->cfg.bc[face];
        if (b != BC_PERIODIC && b != BC_SYMMETRIC) continue;
        const int ax = face >> 1;
        int rd, wr;
        halo_rw(s, face, rd, wr);
        face_loop(s, ax, [&](int ua, int ub) {
            int I, J, K;
            plane(ax, wr, ua, ub, I, J, K);
            m[fidx(s, I, J, K)] = 1;
        });
    }
    return m;
}

// the wall positions whose velocities jlb_evolve re-reads: all of them, or
// with a static halo all but the halo cells that neither the caller nor the
// halo rules write (those of wall and Zou-He faces)
void select_checked_walls(jlb_solver *s) {
    s->wall_chk.clear();
    std::vector<uint8_t> refreshed;
    if (s->static_halo) refreshed = halo_refreshed(s);
    for (size_t w = 0; w < s->wall_pos.size(); ++w) {
        const int64_t p = s->wall_pos[w];
        if (s->static_halo) {
            const int I = (int)(p / ((int64_t)s->NJ * s->NK));
            const int J = (int)((p / s->NK) % s->NJ);
            const int K = (int)(p % s->NK);
            const bool halo = I == 0 || J == 0 || K == 0 || I == s->NI - 1 || J == s->NJ - 1 || K == s->NK - 1;
            if (halo && !refreshed[p]) continue;
        }
        s->wall_chk.push_back((int64_t)w);
    }
    s->wall_dev_dirty = true;
}

// solid positions that are the source of a bounce-back link
void build_wall_list(jlb_solver *s) {
    std::vector<uint8_t> flag((size_t)s->NCNT, 0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < s->nx; ++i)
        for (int j = 0; j < s->ny; ++j)
            for (int k = 0; k < s->nz; ++k) {
                const int64_t n = ((int64_t)i * s->ny + j) * s->nz + k;
                const uint32_t m = s->hmask[n];
                if ((m & MASK_SOLID) || !(m & MASK_LINKS)) continue;
                for (int q = 0; q < 19; ++q)
                    if (m & (1u << q)) flag[fidx(s, i + 1 - CI[q], j + 1 - CJ[q], k + 1 - CK[q])] = 1;
            }
    s->wall_pos.clear();
    for (int64_t p = 0; p < s->NCNT; ++p)
        if (flag[p]) s->wall_pos.push_back(p);
    select_checked_walls(s);
}

// boundary-node tables from the current wall velocities (vel: halo-padded,
// after the halo rules)
void build_special(jlb_solver *s, const double *vel) {
    const int64_t N = s->N;
    std::vector<uint8_t> special((size_t)N, 0);
    const int *bc = s->cfg.bc;
    // Zou-He faces and symmetric faces: first / last interior layers
    for (int face = 0; face < 6; ++face) {
        const bool zh = is_fixed(bc[face]);
        const bool sym = bc[face] == BC_SYMMETRIC;
        if (!zh && !sym) continue;
        const int ax = face >> 1;
        const int lim = ax == 0 ? s->nx : ax == 1 ? s->ny : s->nz;
        const int c = (face & 1) ? lim - 1 : 0;
        const int A = ax == 0 ? s->ny : s->nx, B = ax == 2 ? s->ny : s->nz;
        for (int a = 0; a < A; ++a)
            for (int b2 = 0; b2 < B; ++b2) {
                int i, j, k;
                if (ax == 0) { i = c; j = a; k = b2; }
                else if (ax == 1) { i = a; j = c; k = b2; }
                else { i = a; j = b2; k = c; }
                const int64_t n = ((int64_t)i * s->ny + j) * s->nz + k;
                if (!(s->hmask[n] & MASK_SOLID)) special[n] = 1;
            }
    }
    // moving solids: a bounce-back link with a nonzero Ladd projection
    s->wall_vel.resize(3 * s->wall_pos.size());
    s->wall_dev_dirty = true;
    for (size_t w = 0; w < s->wall_pos.size(); ++w) {
        const int64_t p = s->wall_pos[w];
        const double *u = vel + 3 * p;
        s->wall_vel[3 * w] = u[0]; s->wall_vel[3 * w + 1] = u[1]; s->wall_vel[3 * w + 2] = u[2];
        if (u[0] == 0.0 && u[1] == 0.0 && u[2] == 0.0) continue;
        const int I = (int)(p / ((int64_t)s->NJ * s->NK));
        const int J = (int)((p / s->NK) % s->NJ);
        const int K = (int)(p % s->NK);
        for (int q = 0; q < 19; ++q) {
            if (q == 9) continue;
            const int i = I + CI[q] - 1, j = J + CJ[q] - 1, k = K + CK[q] - 1;
            if (i < 0 || j < 0 || k < 0 || i >= s->nx || j >= s->ny || k >= s->nz) continue;
            const int64_t n = ((int64_t)i * s->ny + j) * s->nz + k;
            if (s->hmask[n] & MASK_SOLID) continue;
            if (ladd_proj(q, u) != 0.0) special[n] = 1;
        }
    }
    // mark and build tables
    for (int64_t n = 0; n < N; ++n) {
        if (s->hmask[n] & MASK_SOLID) continue;
        s->hmask[n] = special[n] ? (s->hmask[n] | MASK_SPECIAL) : (s->hmask[n] & ~MASK_SPECIAL);
    }
    s->sp_node.clear();
    for (int64_t n = 0; n < N; ++n)
        if (special[n]) s->sp_node.push_back(n);
    const int M = (int)s->sp_node.size();
    s->M = M;
    s->sp_info.assign(M, 0);
    s->sp_rd.assign((size_t)19 * M, 0);
    s->sp_wr.assign((size_t)19 * M, 0);
    s->sp_lw.assign((size_t)19 * M, 0.0);
    const int64_t Np = s->Np;
    int slots = 0;
#pragma omp parallel for schedule(static) reduction(max : slots) if (M > 4096)
    for (int t = 0; t < M; ++t) {
        const int64_t n = s->sp_node[t];
        const int i = (int)(n / ((int64_t)s->ny * s->nz));
        const int j = (int)((n / s->nz) % s->ny);
        const int k = (int)(n % s->nz);
        const int I = i + 1, J = j + 1, K = k + 1;
        uint32_t info = 0;
        for (int q = 0; q < 19; ++q) {
            int64_t rd, wr;
            if (q == 9) {
                rd = wr = 9 * Np + n;
            } else {
                // read: source x - c_q
                const int SI = I - CI[q], SJ = J - CJ[q], SK = K - CK[q];
                const int64_t sp = fidx(s, SI, SJ, SK);
                if (s->phase[sp] == 0) {
                    rd = (int64_t)q * Np + n;
                    const double lw = ladd_proj(q, vel + 3 * sp);
                    if (lw != 0.0) {
                        info |= 1u << q;
                        s->sp_lw[(size_t)q * M + t] = lw;
                    }
                } else if (SI >= 1 && SI <= s->nx && SJ >= 1 && SJ <= s->ny && SK >= 1 && SK <= s->nz) {
                    rd = (int64_t)(18 - q) * Np + (((int64_t)(SI - 1) * s->ny + (SJ - 1)) * s->nz + (SK - 1));
                } else {
                    int p = q;
                    const int64_t m = map_halo(s, SI, SJ, SK, p);
                    rd = m >= 0 ? (int64_t)(18 - p) * Np + m : (int64_t)q * Np + n;
                }
                // write: destination x + c_q
                const int DI = I + CI[q], DJ = J + CJ[q], DK = K + CK[q];
                const int64_t dp = fidx(s, DI, DJ, DK);
                if (s->phase[dp] == 0) {
                    wr = (int64_t)(18 - q) * Np + n;
                } else if (DI >= 1 && DI <= s->nx && DJ >= 1 && DJ <= s->ny && DK >= 1 && DK <= s->nz) {
                    wr = (int64_t)q * Np + (((int64_t)(DI - 1) * s->ny + (DJ - 1)) * s->nz + (DK - 1));
                } else {
                    int p = q;
                    const int64_t m = map_halo(s, DI, DJ, DK, p);
                    wr = m >= 0 ? (int64_t)p * Np + m : (int64_t)(18 - q) * Np + n;
                }
            }
            s->sp_rd[(size_t)q * M + t] = rd;
            s->sp_wr[(size_t)q * M + t] = wr;
        }
        // Zou-He faces of this node
        const int at[6] = {i == 0, i == s->nx - 1, j == 0, j == s->ny - 1, k == 0, k == s->nz - 1};
        int nf = 0;
        for (int face = 0; face < 6; ++face)
            if (at[face] && is_fixed(bc[face])) { info |= 1u << (SP_FACE_SHIFT + face); ++nf; }
        s->sp_info[t] = info;
        slots = std::max(slots, nf);
    }
    s->bc_slots = slots; // Zou-He data sets per boundary node (0, 1 or 2)
}

// per-call Zou-He data and previous-step density of the boundary nodes
// Per-call inputs of the boundary nodes, written straight into the
// page-locked staging buffer: Zou-He data (bc_slots x 4 doubles per node,
// slot-major) followed by the previous-step density in the compute type.
void fill_dynamic(jlb_solver *s, const double *den, const double *vel, double *bcbuf, void *denbuf) {
    const int M = s->M;
    const int *bc = s->cfg.bc;
    const bool f64 = s->prec == PREC_FP64;
#pragma omp parallel for schedule(static) if (M > 4096)
    for (int t = 0; t < M; ++t) {
        const int64_t n = s->sp_node[t];
        const int i = (int)(n / ((int64_t)s->ny * s->nz));
        const int j = (int)((n / s->nz) % s->ny);
        const int k = (int)(n % s->nz);
        const int64_t fn = fidx(s, i + 1, j + 1, k + 1);
        if (f64) ((double *)denbuf)[t] = den[fn];
        else ((float *)denbuf)[t] = (float)(den[fn] - 1.0);
        const uint32_t faces = (s->sp_info[t] >> SP_FACE_SHIFT) & 0x3Fu;
        int slot = 0;
        for (int face = 0; face < 6 && faces; ++face) {
            if (!(faces & (1u << face))) continue;
            // the reference refreshes face Z1's data when bc[Z1] is FIXED_DEN
            // or bc[1Z] is FIXED_VEL (jyulb/isothermal.pyx:500); otherwise it
            // keeps its initial den = 1, vel = 0
            bool refresh = is_fixed(bc[face]);
            if (face == 5) refresh = bc[5] == BC_FIXED_DEN || bc[4] == BC_FIXED_VEL;
            double d = 1.0, u0 = 0.0, u1 = 0.0, u2 = 0.0;
            if (refresh) { d = den[fn]; u0 = vel[3 * fn]; u1 = vel[3 * fn + 1]; u2 = vel[3 * fn + 2]; }
            bcbuf[(size_t)(4 * slot) * M + t] = d;
            bcbuf[(size_t)(4 * slot + 1) * M + t] = u0;
            bcbuf[(size_t)(4 * slot + 2) * M + t] = u1;
            bcbuf[(size_t)(4 * slot + 3) * M + t] = u2;
            slot = 1;
        }
    }
}

template <class T> int dev_alloc(jlb_solver *s, T *&p, size_t count) {
    if (p) cudaFree(p);
    p = nullptr;
    if (count == 0) count = 1;
    CK(cudaMalloc((void **)&p, count * sizeof(T)));
    return JLB_OK;
}

void drop_graphs(jlb_solver *s) {
    for (int p = 0; p < 2; ++p) {
        if (s->gexec[p]) cudaGraphExecDestroy(s->gexec[p]);
        s->gexec[p] = nullptr;
        s->graph_version[p] = 0;
    }
}

// uploads the static boundary tables (after build_special)
int upload_tables(jlb_solver *s) {
    const int M = s->M;
    s->sp_tables_dirty = true;
    if (M > s->Mcap) {
        const size_t cap = (size_t)M + M / 4 + 64;
        int r;
        if ((r = dev_alloc(s, s->d_sp_node, cap)) || (r = dev_alloc(s, s->d_sp_info, cap)) ||
            (r = dev_alloc(s, s->d_sp_rd, 19 * cap)) || (r = dev_alloc(s, s->d_sp_wr, 19 * cap)) ||
            (r = dev_alloc(s, s->d_sp_lw, 19 * cap)) || (r = dev_alloc(s, s->d_sp_bc, 8 * cap)))
            return r;
        if (s->d_sp_den) cudaFree(s->d_sp_den);
        s->d_sp_den = nullptr;
        CK(cudaMalloc(&s->d_sp_den, cap * s->csz));
        s->Mcap = (int)cap;
    }
    if (M > 0) {
        CK(cudaMemcpyAsync(s->d_sp_node, s->sp_node.data(), M * sizeof(int64_t), cudaMemcpyHostToDevice, s->st));
        CK(cudaMemcpyAsync(s->d_sp_info, s->sp_info.data(), M * sizeof(uint32_t), cudaMemcpyHostToDevice, s->st));
        CK(cudaMemcpyAsync(s->d_sp_rd, s->sp_rd.data(), 19 * (size_t)M * sizeof(int64_t), cudaMemcpyHostToDevice, s->st));
        CK(cudaMemcpyAsync(s->d_sp_wr, s->sp_wr.data(), 19 * (size_t)M * sizeof(int64_t), cudaMemcpyHostToDevice, s->st));
        CK(cudaMemcpyAsync(s->d_sp_lw, s->sp_lw.data(), 19 * (size_t)M * sizeof(double), cudaMemcpyHostToDevice, s->st));
    }
    CK(cudaMemcpyAsync(s->nmask, s->hmask.data(), (size_t)s->Np * sizeof(uint32_t), cudaMemcpyHostToDevice, s->st));
    s->hcls.resize((size_t)s->Np);
#pragma omp parallel for schedule(static)
    for (int64_t n = 0; n < s->Np; ++n) {
        const uint32_t m = s->hmask[n];
        s->hcls[n] = (m & MASK_SOLID) ? CLS_SOLID : (m & MASK_SPECIAL) ? CLS_SPECIAL
                                                  : (m & MASK_LINKS) ? CLS_WALL : CLS_PLAIN;
    }
    CK(cudaMemcpyAsync(s->ncls, s->hcls.data(), (size_t)s->Np, cudaMemcpyHostToDevice, s->st));
    s->h2d_bytes += (uint64_t)s->Np * 5 + (uint64_t)M * (8 + 4 + 3 * 19 * 8);
    CK(cudaStreamSynchronize(s->st)); // host vectors may be rebuilt right after
    ++s->args_version;
    return JLB_OK;
}

// uploads bc data and previous-step density of the boundary nodes
int upload_dynamic(jlb_solver *s, const double *den, const double *vel) {
    const int M = s->M;
    if (M == 0) return JLB_OK;
    const size_t bc_bytes = 4 * (size_t)s->bc_slots * M * sizeof(double);
    const size_t den_bytes = (size_t)M * s->csz;
    const double *dden = (const double *)dev_view(den), *dvel = (const double *)dev_view(vel);
    if (dden && dvel) {
        // page-locked host arrays: a kernel reads the face layers in place
        // (stream-ordered after the previous steps, no host pass, no staging)
        const int *bc = s->cfg.bc;
        unsigned refresh = 0;
        for (int face = 0; face < 6; ++face) {
            // the reference refreshes face Z1's data when bc[Z1] is FIXED_DEN
            // or bc[1Z] is FIXED_VEL (jyulb/isothermal.pyx:500)
            const bool r = face == 5 ? (bc[5] == BC_FIXED_DEN || bc[4] == BC_FIXED_VEL) : is_fixed(bc[face]);
            if (r) refresh |= 1u << face;
        }
        CKR(aux_fill_dynamic(s->geom, M, s->d_sp_node, s->d_sp_info, refresh, s->prec == PREC_FP64, dden, dvel,
                             s->d_sp_bc, s->d_sp_den, s->st));
        ++s->launches;
        s->h2d_bytes += bc_bytes + den_bytes;
        return JLB_OK;
    }
    int r = ensure_pinned(s, bc_bytes + den_bytes + 64);
    if (r) return r;
    CK(cudaStreamSynchronize(s->st)); // staging buffer may still be in flight
    char *pin = (char *)s->pinned;
    fill_dynamic(s, den, vel, (double *)pin, pin + bc_bytes);
    if (bc_bytes) CK(cudaMemcpyAsync(s->d_sp_bc, pin, bc_bytes, cudaMemcpyHostToDevice, s->st));
    CK(cudaMemcpyAsync(s->d_sp_den, pin + bc_bytes, den_bytes, cudaMemcpyHostToDevice, s->st));
    s->h2d_bytes += bc_bytes + den_bytes;
    return JLB_OK;
}

// the linear site mapping of the dense sweep: wherever the row blocks would
// leave lanes idle (nz not a multiple of 32, or above 128 and not a multiple
// of 128), on the direct kernel (the staged kernel and the adjoint's reverse
// kernel tile rows) and below 2^32 sites; JLB_LIN=0 keeps the row blocks
bool use_lin(const jlb_solver *s) {
    const char *e = std::getenv("JLB_LIN");
    if (e && e[0] == '0') return false;
    const int nzr = ((s->nz + 31) / 32) * 32;
    const int bx = nzr >= 128 ? 128 : nzr;
    const bool idle = (s->nz + bx - 1) / bx * bx != s->nz;
    return idle && !s->use_tma && !s->no_lin && s->N < ((int64_t)1 << 32);
}

StepArgs make_args(const jlb_solver *s, int write_moments) {
    StepArgs a{};
    a.f = s->f;
    a.Np = s->Np;
    a.nx = s->nx; a.ny = s->ny; a.nz = s->nz;
    a.nmask = s->nmask;
    a.ncls = s->ncls;
    a.den = s->mom[0]; a.ux = s->mom[1]; a.uy = s->mom[2]; a.uz = s->mom[3];
    a.acc = s->accf ? s->acc : nullptr;
    for (int d = 0; d < 3; ++d) a.g[d] = s->g[d];
    a.w_e = s->we; a.w_o = s->wo;
    if (s->prec != PREC_FP64 && s->cfg.kernel == JLB_KERNEL_JYULB)
        float_exact_rates(s->cfg.rlx_scheme == JLB_TRT, s->we, s->wo, a.w_e, a.w_o);
    for (int d = 0; d < 3; ++d) a.gf[d] = (float)a.g[d];
    a.w_ef = (float)a.w_e;
    a.w_of = (float)a.w_o;
    a.write_moments = write_moments;
    const int nzr = ((s->nz + 31) / 32) * 32;
    a.bx = nzr >= 128 ? 128 : nzr;
    a.by = 128 / a.bx;
    a.kblocks = (s->nz + a.bx - 1) / a.bx;
    const int64_t rows = (int64_t)s->nx * s->ny;
    a.nb_dense = (int)(a.kblocks * ((rows + a.by - 1) / a.by));
    a.div_ny = make_udiv((uint32_t)s->ny);
    if (use_lin(s)) {
        // nz = 4 would use 4 of 32 lanes, nz = 40 40 of 64: consecutive
        // sites instead, with (i, j, k) from divisions by nz and ny
        a.lin = 1;
        a.bx = 128; a.by = 1; a.kblocks = 1;
        a.nsite = (uint32_t)s->N;
        a.div_nz = make_udiv((uint32_t)s->nz);
        a.nb_dense = (int)((s->N + 127) / 128);
    }
    a.pf = s->pf_blocks;
    a.M = s->M;
    a.sp_node = s->d_sp_node; a.sp_info = s->d_sp_info;
    a.sp_rd = s->d_sp_rd; a.sp_wr = s->d_sp_wr;
    a.sp_lw = s->d_sp_lw; a.sp_bc = s->d_sp_bc;
    a.sp_den = s->d_sp_den;
    for (int f = 0; f < 6; ++f) a.bc[f] = s->cfg.bc[f];
    if (s->sparse && s->fc) {
        a.f = s->fc;
        a.csite = s->d_csite;
        a.cidx = s->d_cidx;
        a.Nc = s->Nc;
        a.Npc = s->Npc;
        // float-reciprocal split when every quotient (i < nx, j < ny) stays
        // below 2^21 and the divisors below 2^30
        if (s->nx < (1 << 21) && s->ny < (1 << 21) && (int64_t)s->ny * s->nz < (1 << 30)) {
            a.inv_syz = 1.0f / (float)((int64_t)s->ny * s->nz);
            a.inv_nz = 1.0f / (float)s->nz;
        }
        a.sp_rd = s->d_sp_rd_c;
        a.sp_wr = s->d_sp_wr_c;
        a.sp_cnode = s->d_sp_cnode;
    }
    return a;
}

int launch_one(jlb_solver *s, const StepArgs &a, bool pstep) {
    const int blocks = a.nb_dense + special_blocks(a); // direct kernel: blocks of bx * by threads
    const int nsb = (a.M + 127) / 128;                  // staged / fluid-only kernels: 128
    int r;
    if (a.csite) {
        const int nb = (int)((a.Nc + 127) / 128) + nsb;
        if (s->prec == PREC_FP32) r = launch_step_sparse_fp32(a, s->cfg.rlx_scheme, pstep, s->accf, nb, s->st);
        else r = launch_step_sparse_fp16(a, s->cfg.rlx_scheme, pstep, s->accf, nb, s->st);
    } else if (s->use_h2 && !pstep && !a.fout && !a.sp_tee) {
        const int kb2 = s->nz / 256;
        r = launch_step_tma_h2_fp16(a, s->cfg.rlx_scheme, s->accf, s->h2_grid, s->nx * s->ny * kb2, kb2, nsb, s->d_err,
                                    s->st);
    } else if (s->use_tma && !a.fout && !a.sp_tee && (s->tma_p || !pstep)) {
        const int ntiles = a.nb_dense; // one 128-site tile per dense block (bx = 128, by = 1)
        if (s->prec == PREC_FP32)
            r = launch_step_tma_fp32(a, s->cfg.rlx_scheme, pstep, s->accf, s->tma_grid, ntiles, nsb, s->d_err, s->st);
        else
            r = launch_step_tma_fp16(a, s->cfg.rlx_scheme, pstep, s->accf, s->tma_grid, ntiles, nsb, s->d_err, s->st);
    } else if (s->cfg.kernel == JLB_KERNEL_CXX) {
        r = launch_step_cxx(a, s->cfg.rlx_scheme, s->cfg.kernel_opts, pstep, s->accf, blocks, s->st);
    } else if (s->prec == PREC_FP64) {
        r = s->fast64 ? launch_step_fp64fast(a, s->cfg.rlx_scheme, pstep, s->accf, blocks, s->st)
                      : launch_step_fp64(a, s->cfg.rlx_scheme, pstep, s->accf, blocks, s->st);
    }
    else if (s->prec == PREC_FP32) r = launch_step_fp32(a, s->cfg.rlx_scheme, pstep, s->accf, blocks, s->st);
    else r = launch_step_fp16(a, s->cfg.rlx_scheme, pstep, s->accf, blocks, s->st);
    if (r) return fail(s, JLB_ERR_CUDA, std::string("step launch: ") + cudaGetErrorString((cudaError_t)r));
    ++s->launches;
    return JLB_OK;
}

// The staged kernel needs 16-byte aligned rows, whole 128-site tiles per
// row (nz a multiple of 128) and 32-bit element
// indices; it only makes sense when most staged sites are fluid.  By default
// it runs the local (L) step, whose reads are aligned whole rows, and the
// direct kernel runs the pull-push (P) step: on the 256^3 cavity that split
// measured 81% of HBM, direct-only 79%, staged-only 74%.  JLB_TMA=0 disables
// staging, JLB_TMA=1 stages both steps.
void choose_kernel(jlb_solver *s) {
    s->use_tma = false;
    s->use_h2 = false;
    // L2 line prefetch 6 blocks per SM ahead (of the 8 resident) on the
    // direct FP32 kernels: 38.8 -> 39.8 GLUPS on the 256^3 cavity, flat from
    // 5 to 8 blocks per SM, worse beyond.  FP16 storage is issue-bound and
    // loses (50.8 -> 48.5), FP64 is bound by its arithmetic.  JLB_PF=<blocks>
    // sets the distance for any precision, 0 switches it off
    {
        int dev = 0, sms = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
            cudaGetLastError();
            sms = 0;
        }
        // only where the populations do not stay in L2 between steps (a
        // lattice that fits gains nothing and pays for the instructions)
        int l2 = 0;
        if (cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) != cudaSuccess) {
            cudaGetLastError();
            l2 = 0;
        }
        const bool big = (double)19 * (double)s->Np * (double)s->ssz > 2.0 * (double)l2;
        const char *ep = std::getenv("JLB_PF");
        s->pf_blocks = (ep && ep[0]) ? std::max(0, std::atoi(ep)) : (s->prec == PREC_FP32 && big ? 6 * sms : 0);
        ++s->args_version;
    }
    // fluid-only layout for FP32 / FP16 storage when under 80% of the sites
    // are fluid: a lattice-ordered sweep then fetches population lines that
    // are partly solid slots (1.6x the fluid bytes at porosity 0.6).
    // JLB_SPARSE=0 keeps the lattice layout, JLB_SPARSE=1 forces the other.
    const char *es = std::getenv("JLB_SPARSE");
    // (32-bit element indices: 19 * Npc < 2^32)
    const int64_t npc = (((int64_t)s->nfluid + 127) / 128) * 128;
    s->sparse = !s->no_sparse && s->prec != PREC_FP64 && s->cfg.kernel == JLB_KERNEL_JYULB &&
                s->N < (int64_t)1 << 31 && 19 * npc < ((int64_t)1 << 32) &&
                ((es && es[0]) ? es[0] == '1' : (double)s->nfluid < 0.8 * (double)s->N);
    s->c_current = false;
    if (s->sparse) { ++s->args_version; return; }
    const char *e = std::getenv("JLB_TMA");
    if (e && e[0] == '0') return;
    s->tma_p = e && e[0] == '1';
    if (s->prec == PREC_FP64) return;
    const int pad = (int)(16 / s->ssz);
    // whole 128-site tiles per row (other nz take the direct kernel with
    // blocks of consecutive sites)
    if (s->nz % 128 != 0 || s->nz % pad != 0 || s->Np * 19 > 0x7fffffffLL) return;
    if ((double)s->nfluid < 0.85 * (double)s->N) return;
    const int per_sm = s->prec == PREC_FP32 ? tma_blocks_per_sm_fp32(s->cfg.rlx_scheme)
                                            : tma_blocks_per_sm_fp16(s->cfg.rlx_scheme);
    int dev = 0, sms = 0;
    if (per_sm <= 0 || cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
        cudaGetLastError();
        return;
    }
    s->tma_grid = per_sm * sms;
    s->use_tma = true;
    // FP16 storage with nz a multiple of 256: the staged local step takes two
    // sites per thread (JLB_H2=0 keeps one)
    const char *eh = std::getenv("JLB_H2");
    if (s->prec == PREC_FP16 && s->nz % 256 == 0 && !(eh && eh[0] == '0')) {
        const int h2_sm = tma_h2_blocks_per_sm_fp16(s->cfg.rlx_scheme);
        if (h2_sm > 0) {
            s->use_h2 = true;
            s->h2_grid = h2_sm * sms;
        }
    }
    ++s->args_version;
}

// reports a kernel-side timeout recorded in d_err
int check_kernel_error(jlb_solver *s) {
    int h = 0;
    CK(cudaMemcpyAsync(&h, s->d_err, sizeof(int), cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    if (h) return fail(s, JLB_ERR_CUDA, "a step kernel's bounded wait on its bulk copies timed out");
    return JLB_OK;
}

// JLB_OVERLAP_DOWNLOAD=0 keeps the last step and the download in sequence
bool overlap_off() {
    const char *e = std::getenv("JLB_OVERLAP_DOWNLOAD");
    return e && e[0] == '0';
}

bool graphs_enabled() {
    static int en = -1;
    if (en < 0) {
        const char *e = std::getenv("JLB_NO_GRAPH");
        en = (e && e[0] && e[0] != '0') ? 0 : 1;
    }
    return en == 1;
}

// runs n steps; the last one writes moments when write_last
// builds the fluid-only layout on first use: site lists from the node mask
int sparse_setup(jlb_solver *s) {
    if (s->fc) return JLB_OK;
    std::vector<uint32_t> mask((size_t)s->N);
    CK(cudaMemcpy(mask.data(), s->nmask, (size_t)s->N * sizeof(uint32_t), cudaMemcpyDeviceToHost));
    std::vector<int32_t> cidx((size_t)s->N, -1), csite;
    csite.reserve((size_t)s->nfluid);
    for (int64_t n = 0; n < s->N; ++n)
        if (!(mask[n] & MASK_SOLID)) { cidx[n] = (int32_t)csite.size(); csite.push_back((int32_t)n); }
    s->Nc = (int64_t)csite.size();
    s->Npc = ((s->Nc + 127) / 128) * 128;
    if (cudaMalloc(&s->fc, (size_t)19 * s->Npc * s->ssz) != cudaSuccess ||
        cudaMalloc(&s->d_csite, std::max<size_t>(1, csite.size()) * sizeof(int32_t)) != cudaSuccess ||
        cudaMalloc(&s->d_cidx, (size_t)s->N * sizeof(int32_t)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(s->fc); cudaFree(s->d_csite); cudaFree(s->d_cidx);
        s->fc = nullptr; s->d_csite = s->d_cidx = nullptr;
        s->sparse = false;  // not enough device memory: lattice layout
        ++s->args_version;
        return JLB_OK;
    }
    CK(cudaMemcpy(s->d_csite, csite.data(), csite.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(s->d_cidx, cidx.data(), cidx.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    s->sp_tables_dirty = true;
    ++s->args_version;
    return JLB_OK;
}

// makes the fluid-only copy current (gathering the lattice copy if needed)
// and its boundary tables up to date
int sparse_enter(jlb_solver *s) {
    int r = sparse_setup(s);
    if (r || !s->sparse) return r;
    if (s->sp_tables_dirty && s->M > 0) {
        if (s->M > s->sp_c_cap) {
            cudaFree(s->d_sp_rd_c); cudaFree(s->d_sp_wr_c); cudaFree(s->d_sp_cnode);
            const int cap = s->M + s->M / 4 + 64;
            s->d_sp_rd_c = s->d_sp_wr_c = s->d_sp_cnode = nullptr;
            CK(cudaMalloc(&s->d_sp_rd_c, (size_t)19 * cap * sizeof(int64_t)));
            CK(cudaMalloc(&s->d_sp_wr_c, (size_t)19 * cap * sizeof(int64_t)));
            CK(cudaMalloc(&s->d_sp_cnode, (size_t)cap * sizeof(int64_t)));
            s->sp_c_cap = cap;
            ++s->args_version;
        }
        CKR(aux_sparse_tables(s->d_sp_rd, s->d_sp_wr, s->d_sp_node, s->M, s->d_cidx, s->Np, s->Npc, s->d_sp_rd_c,
                              s->d_sp_wr_c, s->d_sp_cnode, s->st));
        ++s->launches;
    }
    s->sp_tables_dirty = false;
    if (!s->c_current) {
        CKR(aux_sparse_pack((int)s->ssz, s->f, s->fc, s->d_csite, s->Nc, s->Np, s->Npc, 1, s->st));
        ++s->launches;
        s->c_current = true;
    }
    return JLB_OK;
}

// makes the lattice-layout copy current (for population read-out / writes)
int sparse_leave(jlb_solver *s) {
    if (!s->sparse || !s->fc || !s->c_current) return JLB_OK;
    CKR(aux_sparse_pack((int)s->ssz, s->f, s->fc, s->d_csite, s->Nc, s->Np, s->Npc, 0, s->st));
    ++s->launches;
    s->c_current = false;
    return JLB_OK;
}

int run_steps(jlb_solver *s, uint32_t n, bool write_last) {
    if (n == 0) return JLB_OK;
    if (s->sparse) {
        int r = sparse_enter(s);
        if (r) return r;
    }
    const StepArgs a0 = make_args(s, 0);
    uint32_t plain = write_last ? n - 1 : n;
    if (graphs_enabled() && plain >= (uint32_t)s->GK) {
        while (plain >= (uint32_t)s->GK) {
            const int p = s->parity;
            if (!s->gexec[p] || s->graph_version[p] != s->args_version) {
                if (s->gexec[p]) cudaGraphExecDestroy(s->gexec[p]);
                s->gexec[p] = nullptr;
                cudaGraph_t graph;
                CK(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeThreadLocal));
                int par = p;
                int rr = JLB_OK;
                for (int t = 0; t < s->GK && rr == JLB_OK; ++t) {
                    rr = launch_one(s, a0, par == 0);
                    par ^= 1;
                }
                cudaError_t ce = cudaStreamEndCapture(s->st, &graph);
                if (rr) return rr;
                if (ce != cudaSuccess) return fail(s, JLB_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
                s->launches -= s->GK; // capture does not launch
                ce = cudaGraphInstantiate(&s->gexec[p], graph, 0);
                cudaGraphDestroy(graph);
                if (ce != cudaSuccess) return fail(s, JLB_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ce));
                s->graph_version[p] = s->args_version;
            }
            CK(cudaGraphLaunch(s->gexec[p], s->st));
            s->launches += s->GK;
            plain -= s->GK;
            if (s->GK & 1) s->parity ^= 1;
        }
    }
    for (uint32_t t = 0; t < plain; ++t) {
        int r = launch_one(s, a0, s->parity == 0);
        if (r) return r;
        s->parity ^= 1;
    }
    if (write_last) {
        const StepArgs a1 = make_args(s, 1);
        int r = launch_one(s, a1, s->parity == 0);
        if (r) return r;
        s->parity ^= 1;
    }
    return JLB_OK;
}

// solid velocities changed since the last classification?  A kernel reads
// the page-locked host vel in place at the wall positions (the host loop
// over them is latency-bound: ~1.2 ms single-threaded, ~0.14 ms on 16
// threads for the 256^3 cavity's 330 K positions)
int wall_check_device(jlb_solver *s, const double *dvel, int &changed) {
    const int64_t nwall = (int64_t)s->wall_chk.size();
    if (!s->wall_flag) {
        CK(cudaHostAlloc((void **)&s->wall_flag, sizeof(int), cudaHostAllocMapped));
    }
    if (s->wall_dev_dirty) {
        std::vector<int64_t> pos((size_t)nwall);
        std::vector<double> known(3 * (size_t)nwall);
        for (int64_t c = 0; c < nwall; ++c) {
            const int64_t w = s->wall_chk[c];
            pos[c] = s->wall_pos[w];
            for (int d = 0; d < 3; ++d) known[3 * c + d] = s->wall_vel[3 * w + d];
        }
        cudaFree(s->d_wall_pos);
        cudaFree(s->d_wall_vel);
        s->d_wall_pos = nullptr;
        s->d_wall_vel = nullptr;
        CK(cudaMalloc(&s->d_wall_pos, nwall * sizeof(int64_t)));
        CK(cudaMalloc(&s->d_wall_vel, 3 * nwall * sizeof(double)));
        CK(cudaMemcpy(s->d_wall_pos, pos.data(), nwall * sizeof(int64_t), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(s->d_wall_vel, known.data(), 3 * nwall * sizeof(double), cudaMemcpyHostToDevice));
        s->wall_dev_dirty = false;
    }
    int *dflag = nullptr;
    CK(cudaHostGetDevicePointer((void **)&dflag, s->wall_flag, 0));
    *(volatile int *)s->wall_flag = 0;
    CKR(aux_wall_check(s->d_wall_pos, s->d_wall_vel, nwall, dvel, dflag, s->st));
    ++s->launches;
    CK(cudaStreamSynchronize(s->st));
    changed = *(volatile int *)s->wall_flag;
    return JLB_OK;
}

// copies planes [i0, i1) of the interior box of a halo-padded host array
// (comps doubles per site) from its device copy with one pitched 3-D copy
cudaError_t copy_interior(const jlb_solver *s, const double *src, double *dst, int comps, int i0, int i1,
                          cudaStream_t st) {
    cudaMemcpy3DParms p{};
    const size_t pitch = (size_t)s->NK * comps * sizeof(double);
    p.srcPtr = make_cudaPitchedPtr((void *)src, pitch, (size_t)s->NK * comps * sizeof(double), s->NJ);
    p.dstPtr = make_cudaPitchedPtr((void *)dst, pitch, (size_t)s->NK * comps * sizeof(double), s->NJ);
    p.srcPos = make_cudaPos((size_t)comps * sizeof(double), 1, 1 + (size_t)i0);
    p.dstPos = p.srcPos;
    p.extent = make_cudaExtent((size_t)s->nz * comps * sizeof(double), s->ny, (size_t)(i1 - i0));
    p.kind = cudaMemcpyDeviceToHost;
    return cudaMemcpy3DAsync(&p, st);
}

// The copy-engine download applies when every interior site is fluid (the
// host values of solid sites must stay untouched, so they cannot be
// overwritten by a box copy) and den/vel are page-locked; it needs a device
// copy of the host layout (allocated on first use).  JLB_DMA_DOWNLOAD=0
// keeps the kernel path.
bool dma_ready(jlb_solver *s, double *den, double *vel) {
    const char *de = std::getenv("JLB_DMA_DOWNLOAD");
    const bool dma_off = de && de[0] == '0';
    if (dma_off || s->stg_failed || s->nfluid != (uint64_t)s->N || !dev_view(den) || !dev_view(vel)) return false;
    if (!s->stg_den) {
        const size_t nb = (size_t)s->NCNT * sizeof(double);
        if (cudaMalloc(&s->stg_den, nb) != cudaSuccess || cudaMalloc(&s->stg_vel, 3 * nb) != cudaSuccess) {
            cudaGetLastError();
            cudaFree(s->stg_den);
            s->stg_den = s->stg_vel = nullptr;
            s->stg_failed = true;  // not enough device memory: kernel path from now on
            return false;
        }
    }
    return true;
}

// Moments into the caller's page-locked den/vel.  On the copy-engine path
// the FP64 rows are assembled in a device copy of the host layout and moved
// in one pitched copy per array (~190 GB/s over NVLink-C2C against ~145 GB/s
// for kernel stores to host memory); otherwise the kernel writes the fluid
// sites straight into host memory.
int download(jlb_solver *s, double *den, double *vel) {
    const size_t nb = (size_t)s->NCNT * sizeof(double);
    double *dd = (double *)dev_view(den);
    double *dv = (double *)dev_view(vel);
    if (dma_ready(s, den, vel)) {
        CKR(aux_download(s->prec, s->geom, s->nmask, s->mom[0], s->mom[1], s->mom[2], s->mom[3], s->stg_den,
                         s->stg_vel, s->st));
        CK(copy_interior(s, s->stg_den, den, 1, 0, s->nx, s->st));
        CK(copy_interior(s, s->stg_vel, vel, 3, 0, s->nx, s->st));
        s->d2h_bytes += s->nfluid * 4 * sizeof(double);
        ++s->launches;
        CK(cudaStreamSynchronize(s->st));
        return JLB_OK;
    }
    if (dd && dv) {
        CKR(aux_download(s->prec, s->geom, s->nmask, s->mom[0], s->mom[1], s->mom[2], s->mom[3], dd, dv, s->st));
        s->d2h_bytes += s->nfluid * 4 * sizeof(double);
        ++s->launches;
        CK(cudaStreamSynchronize(s->st));
        return JLB_OK;
    }
    // host arrays the GPU cannot address: round trip through device copies
    double *tden = nullptr, *tvel = nullptr;
    CK(cudaMalloc(&tden, nb));
    cudaError_t e = cudaMalloc(&tvel, 3 * nb);
    if (e != cudaSuccess) { cudaFree(tden); return fail(s, JLB_ERR_NOMEM, "download staging allocation"); }
    int r = JLB_OK;
    if (cudaMemcpyAsync(tden, den, nb, cudaMemcpyHostToDevice, s->st) != cudaSuccess ||
        cudaMemcpyAsync(tvel, vel, 3 * nb, cudaMemcpyHostToDevice, s->st) != cudaSuccess ||
        aux_download(s->prec, s->geom, s->nmask, s->mom[0], s->mom[1], s->mom[2], s->mom[3], tden, tvel, s->st) ||
        cudaMemcpyAsync(den, tden, nb, cudaMemcpyDeviceToHost, s->st) != cudaSuccess ||
        cudaMemcpyAsync(vel, tvel, 3 * nb, cudaMemcpyDeviceToHost, s->st) != cudaSuccess ||
        cudaStreamSynchronize(s->st) != cudaSuccess)
        r = fail(s, JLB_ERR_CUDA, std::string("staged download: ") + cudaGetErrorString(cudaGetLastError()));
    ++s->launches;
    cudaFree(tden);
    cudaFree(tvel);
    return r;
}

// Halo rules of den / vel (enforce_den_vel) applied to the moments of the
// last moment-writing step: the fluid sites of the layers they read are
// written into the host arrays first (in place for page-locked arrays, else
// by a full download)
int halo_from_moments(jlb_solver *s, double *den, double *vel, unsigned axes) {
    double *dd = (double *)dev_view(den), *dv = (double *)dev_view(vel);
    if (dd && dv) {
        CKR(aux_download_layers(s->prec, s->geom, axes, s->nmask, s->mom[0], s->mom[1], s->mom[2], s->mom[3], dd, dv,
                                s->st));
        ++s->launches;
        CK(cudaStreamSynchronize(s->st));
    } else {
        int r = download(s, den, vel);
        if (r) return r;
    }
    enforce_den_vel(s, den, vel);
    return JLB_OK;
}

// The last step of an evolve call with its download overlapped: the
// boundary nodes first, then the dense sweep in slabs of i-planes, each slab
// followed by its FP64 assembly and (on a second stream) its pitched copy to
// the host while the next slab computes.  The direct step kernel runs this
// step (the staged kernel's persistent grid does not split into slabs).
// Used on the copy-engine download path.
int final_step_overlapped(jlb_solver *s, double *den, double *vel) {
    const bool pstep = s->parity == 0;
    StepArgs a = make_args(s, 1);
    // a dense block covers block_units of one i-plane's plane_units: rows of
    // k-lines (times kmul blocks along k), or sites under the linear mapping
    const int64_t plane_units = a.lin ? (int64_t)s->ny * s->nz : s->ny;
    const int64_t block_units = a.lin ? 128 : a.by;
    const int64_t kmul = a.lin ? 1 : a.kblocks;
    auto direct = [&](const StepArgs &x, int blocks) {
        int r;
        if (s->cfg.kernel == JLB_KERNEL_CXX) r = launch_step_cxx(x, s->cfg.rlx_scheme, s->cfg.kernel_opts, pstep, s->accf, blocks, s->st);
        else if (s->prec == PREC_FP64 && s->fast64) r = launch_step_fp64fast(x, s->cfg.rlx_scheme, pstep, s->accf, blocks, s->st);
        else if (s->prec == PREC_FP64) r = launch_step_fp64(x, s->cfg.rlx_scheme, pstep, s->accf, blocks, s->st);
        else if (s->prec == PREC_FP32) r = launch_step_fp32(x, s->cfg.rlx_scheme, pstep, s->accf, blocks, s->st);
        else r = launch_step_fp16(x, s->cfg.rlx_scheme, pstep, s->accf, blocks, s->st);
        if (r) return fail(s, JLB_ERR_CUDA, std::string("step launch: ") + cudaGetErrorString((cudaError_t)r));
        ++s->launches;
        return JLB_OK;
    };
    if (!s->st2) CK(cudaStreamCreateWithFlags(&s->st2, cudaStreamNonBlocking));
    const int nslab = std::min(8, s->nx);
    while ((int)s->slab_ev.size() < nslab + 1) {
        cudaEvent_t e;
        CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        s->slab_ev.push_back(e);
    }
    int r;
    if (a.M > 0) {
        StepArgs sp = a;
        sp.nb_dense = 0;
        if ((r = direct(sp, special_blocks(a)))) return r;
    }
    // a thin first slab lets the copies start early; the rest split evenly.
    // Slab boundaries fall on whole blocks: plane i starts a block when
    // i * plane_units is a multiple of block_units
    const int step = (int)(block_units / std::gcd(block_units, plane_units));
    auto snap_i = [&](int i) { return std::min(s->nx, ((i + step - 1) / step) * step); };
    const int first = std::max(1, s->nx / 32);
    auto bound = [&](int k) -> int {
        if (k == 0) return 0;
        return snap_i(first + (int)((int64_t)(s->nx - first) * (k - 1) / (nslab - 1)));
    };
    for (int k = 0; k < nslab; ++k) {
        const int i0 = bound(k), i1 = k + 1 == nslab ? s->nx : bound(k + 1);
        if (i1 <= i0) continue;
        StepArgs sl = a;
        sl.M = 0;
        sl.b0 = (int)((int64_t)i0 * plane_units / block_units * kmul);
        // the last slab may end in a partial block
        sl.nb_dense = (int)(((int64_t)(i1 - i0) * plane_units + block_units - 1) / block_units * kmul);
        if ((r = direct(sl, sl.nb_dense))) return r;
        // the slab's FP64 assembly follows its step on the compute stream, so
        // that the copy stream carries nothing but back-to-back copies
        CKR(aux_download_rows(s->prec, s->geom, s->nmask, s->mom[0], s->mom[1], s->mom[2], s->mom[3], s->stg_den,
                              s->stg_vel, (int64_t)i0 * s->ny, (int64_t)(i1 - i0) * s->ny, s->st));
        CK(cudaEventRecord(s->slab_ev[k], s->st));
        CK(cudaStreamWaitEvent(s->st2, s->slab_ev[k], 0));
        CK(copy_interior(s, s->stg_den, den, 1, i0, i1, s->st2));
        CK(copy_interior(s, s->stg_vel, vel, 3, i0, i1, s->st2));
        ++s->launches;
    }
    s->parity ^= 1;
    CK(cudaEventRecord(s->slab_ev[nslab], s->st2));
    CK(cudaStreamWaitEvent(s->st, s->slab_ev[nslab], 0));
    CK(cudaStreamSynchronize(s->st));
    s->d2h_bytes += s->nfluid * 4 * sizeof(double);
    return JLB_OK;
}

} // namespace jlb_host

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int jlb_check_config(const jlb_config *cfg, char *msg, size_t msg_len) {
    auto bad = [&](const char *m) {
        if (msg && msg_len) { std::snprintf(msg, msg_len, "%s", m); }
        return JLB_ERR_INVALID_ARG;
    };
    if (!cfg) return bad("Invalid configuration (NULL).");
    if (cfg->lat_size[0] < 1 || cfg->lat_size[1] < 1 || cfg->lat_size[2] < 1)
        return bad("Invalid lattice size input.");
    // the step kernels index rows of k-lines (i * ny + j) with 32-bit integers
    if ((int64_t)cfg->lat_size[0] * cfg->lat_size[1] >= ((int64_t)1 << 31))
        return bad("Lattice too large: nx * ny must stay below 2^31.");
    if (cfg->rlx_scheme != JLB_BGK && cfg->rlx_scheme != JLB_TRT && cfg->rlx_scheme != JLB_REGULARIZATION)
        return bad("Invalid relaxation scheme input.");
    if (!(cfg->kvisc > 0.0)) return bad("Invalid kinematic viscosity input.");
    const int32_t *bc = cfg->bc;
    for (int f = 0; f < 6; ++f)
        if (bc[f] < JLB_WALL || bc[f] > JLB_SYMMETRIC) return bad("Invalid boundary condition input.");
    const char *dirs[3] = {"Invalid periodic bc setup (in x-dir.).", "Invalid periodic bc setup (in y-dir.).",
                           "Invalid periodic bc setup (in z-dir.)."};
    for (int ax = 0; ax < 3; ++ax) {
        const int a = bc[2 * ax], b = bc[2 * ax + 1];
        if ((a == JLB_PERIODIC || b == JLB_PERIODIC) && a != b) return bad(dirs[ax]);
    }
    bool fx[3];
    for (int ax = 0; ax < 3; ++ax) fx[ax] = is_fixed(bc[2 * ax]) || is_fixed(bc[2 * ax + 1]);
    if ((fx[0] && (fx[1] || fx[2])) || (fx[1] && (fx[0] || fx[2])) || (fx[2] && (fx[0] || fx[1])))
        return bad("Invalid fixed variable bc setup.");
    if (cfg->precision < JLB_FP64 || cfg->precision > JLB_FP64_FAST) return bad("Invalid precision input.");
    if (std::isnan(cfg->trt_magic)) return bad("Invalid TRT magic parameter input.");
    for (int d = 0; d < 3; ++d)
        if (!std::isfinite(cfg->g[d])) return bad("Invalid gravity input.");
    if (cfg->kernel != JLB_KERNEL_JYULB && cfg->kernel != JLB_KERNEL_CXX) return bad("Invalid collision kernel input.");
    if (cfg->kernel == JLB_KERNEL_CXX) {
        if (cfg->rlx_scheme == JLB_REGULARIZATION)
            return bad("The C++-executable kernel supports the BGK and TRT schemes.");
        if (cfg->precision != JLB_FP64) return bad("The C++-executable kernel runs in FP64.");
        for (int f = 0; f < 6; ++f)
            if (bc[f] != JLB_PERIODIC && bc[f] != JLB_WALL)
                return bad("The C++-executable kernel supports periodic and wall faces.");
        if (cfg->kernel_opts & ~(JLB_CXX_LINEAR_EQ | JLB_CXX_FORCE2)) return bad("Invalid kernel options input.");
    } else if (cfg->kernel_opts != 0) {
        return bad("Invalid kernel options input.");
    }
    return JLB_OK;
}

int jlb_create(const jlb_config *cfg, jlb_solver **out) {
    jlb_solver *s = nullptr;
    if (!out) return fail(nullptr, JLB_ERR_INVALID_ARG, "out is NULL");
    *out = nullptr;
    char msg[256];
    if (jlb_check_config(cfg, msg, sizeof msg) != JLB_OK) return fail(nullptr, JLB_ERR_INVALID_ARG, msg);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        cudaGetLastError();
        return fail(nullptr, JLB_ERR_CUDA, "no CUDA device available");
    }
    s = new jlb_solver();
    s->cfg = *cfg;
    s->nx = cfg->lat_size[0]; s->ny = cfg->lat_size[1]; s->nz = cfg->lat_size[2];
    s->NI = s->nx + 2; s->NJ = s->ny + 2; s->NK = s->nz + 2;
    s->N = (int64_t)s->nx * s->ny * s->nz;
    s->Np = ((s->N + 127) / 128) * 128;
    s->NCNT = (int64_t)s->NI * s->NJ * s->NK;
    // JLB_FP64_FAST keeps the FP64 state and host paths; only the step
    // kernel differs
    s->fast64 = cfg->precision == JLB_FP64_FAST;
    s->prec = s->fast64 ? PREC_FP64 : cfg->precision;
    s->ssz = s->prec == PREC_FP64 ? 8 : s->prec == PREC_FP32 ? 4 : 2;
    s->csz = s->prec == PREC_FP64 ? 8 : 4;
    for (int d = 0; d < 3; ++d) s->g[d] = cfg->g[d];
    if (cfg->kernel == JLB_KERNEL_CXX) {
        // the executable's rates (include/collision/collision.cpp:14-24,
        // :64-76) with its c_s^2 = (1/sqrt 3)^2
        const double ct = 1.0 / std::sqrt(3.0), ct2 = ct * ct, inv_ct2 = 1.0 / ct2;
        s->tau = 0.5 + inv_ct2 * cfg->kvisc;
        s->we = 1.0 / s->tau;
        s->wo = cfg->rlx_scheme == JLB_TRT ? 8.0 * ((2.0 - s->we) / (8.0 - s->we)) : s->we;
    } else {
        // relaxation rates (jyulb/isothermal.pyx:274-287)
        const double tau_e = 0.5 + 3.0 * cfg->kvisc;
        s->we = 1.0 / tau_e;
        if (cfg->rlx_scheme == JLB_TRT) {
            if (cfg->trt_magic > 0.0) s->wo = 1.0 / (cfg->trt_magic / (tau_e - 0.5) + 0.5);
            else s->wo = 8.0 * (2.0 - s->we) / (8.0 - s->we);
        }
    }
    s->geom = AuxGeom{s->nx, s->ny, s->nz, s->NI, s->NJ, s->NK, s->N, s->Np};
    int r = JLB_OK;
    auto bail = [&](int code) {
        std::string m = s->err;
        jlb_destroy(s);
        fail(nullptr, code, m);
        return code;
    };
    if (cfg->stream) {
        s->st = (cudaStream_t)cfg->stream;
    } else {
        if (cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking) != cudaSuccess) {
            s->err = "cudaStreamCreate failed";
            return bail(JLB_ERR_CUDA);
        }
        s->own_stream = true;
    }
    auto alloc = [&](void **p, size_t bytes) {
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            s->err = std::string("device allocation of ") + std::to_string(bytes) + " bytes failed: " +
                     cudaGetErrorString(e);
            return JLB_ERR_NOMEM;
        }
        return JLB_OK;
    };
    if ((r = alloc(&s->f, (size_t)19 * s->Np * s->ssz))) return bail(r);
    if ((r = alloc((void **)&s->nmask, (size_t)s->Np * sizeof(uint32_t)))) return bail(r);
    if ((r = alloc((void **)&s->ncls, (size_t)s->Np))) return bail(r);
    for (int c = 0; c < 4; ++c)
        if ((r = alloc(&s->mom[c], (size_t)s->Np * s->csz))) return bail(r);
    s->red_blocks = aux_reduce_blocks(s->N);
    if ((r = alloc((void **)&s->red_partial, (size_t)8 * s->red_blocks * sizeof(double)))) return bail(r);
    if ((r = alloc((void **)&s->red_out, 8 * sizeof(double)))) return bail(r);
    if ((r = alloc((void **)&s->d_err, sizeof(int)))) return bail(r);
    if (cudaMemset(s->d_err, 0, sizeof(int)) != cudaSuccess) {
        s->err = "cudaMemset failed";
        return bail(JLB_ERR_CUDA);
    }
    *out = s;
    return JLB_OK;
}

void jlb_destroy(jlb_solver *s) {
    if (!s) return;
    if (s->st) cudaStreamSynchronize(s->st);
    drop_graphs(s);
    void *bufs[] = {s->f, s->nmask, s->ncls, s->mom[0], s->mom[1], s->mom[2], s->mom[3], s->acc, s->red_partial,
                    s->red_out, s->d_sp_node, s->d_sp_info, s->d_sp_rd, s->d_sp_wr, s->d_sp_lw, s->d_sp_bc,
                    s->d_sp_den, s->d_err, s->fi_partial, s->fi_out, s->stg_den, s->stg_vel,
                    s->fc, s->d_csite, s->d_cidx, s->d_sp_rd_c, s->d_sp_wr_c, s->d_sp_cnode,
                    s->d_wall_pos, s->d_wall_vel, s->res_prev};
    for (void *p : bufs)
        if (p) cudaFree(p);
    if (s->pinned) cudaFreeHost(s->pinned);
    if (s->wall_flag) cudaFreeHost(s->wall_flag);
    for (cudaEvent_t e : s->slab_ev) cudaEventDestroy(e);
    if (s->st2) { cudaStreamSynchronize(s->st2); cudaStreamDestroy(s->st2); }
    if (s->own_stream && s->st) cudaStreamDestroy(s->st);
    delete s;
}

int jlb_finalize_init(jlb_solver *s, uint8_t *phase, double *den, double *vel, uint64_t *nfluid) {
    if (!s || !phase || !den || !vel) return fail(s, JLB_ERR_INVALID_ARG, "NULL argument");
    // fluid sites of the interior (jyulb/isothermal.pyx:1354-1356)
    uint64_t cnt = 0;
    for (int I = 1; I < s->NI - 1; ++I)
        for (int J = 1; J < s->NJ - 1; ++J)
            for (int K = 1; K < s->NK - 1; ++K) cnt += phase[fidx(s, I, J, K)] != 0;
    drop_graphs(s);
    s->M = 0;
    if (cnt >= 1) {
        enforce_phase(s, phase);
        enforce_den_vel(s, den, vel);
        s->phase.assign(phase, phase + s->NCNT);
        solidify_closed_halo(s, s->phase);
        build_mask(s);
        build_wall_list(s);
        build_special(s, vel);
        int r = upload_tables(s);
        if (r) return r;
        // initial populations: the kernel reads the halo-padded arrays
        const size_t nb = (size_t)s->NCNT;
        uint8_t *dph = nullptr;
        double *dden = nullptr, *dvel = nullptr;
        CK(cudaMalloc(&dph, nb));
        cudaError_t e1 = cudaMalloc(&dden, nb * sizeof(double));
        cudaError_t e2 = cudaMalloc(&dvel, 3 * nb * sizeof(double));
        if (e1 != cudaSuccess || e2 != cudaSuccess) {
            cudaFree(dph); cudaFree(dden); cudaFree(dvel);
            return fail(s, JLB_ERR_NOMEM, "initialisation staging allocation");
        }
        CK(cudaMemcpyAsync(dph, phase, nb, cudaMemcpyHostToDevice, s->st));
        CK(cudaMemcpyAsync(dden, den, nb * sizeof(double), cudaMemcpyHostToDevice, s->st));
        CK(cudaMemcpyAsync(dvel, vel, 3 * nb * sizeof(double), cudaMemcpyHostToDevice, s->st));
        CK(cudaMemsetAsync(s->f, 0, (size_t)19 * s->Np * s->ssz, s->st));
        for (int c = 0; c < 4; ++c) CK(cudaMemsetAsync(s->mom[c], 0, (size_t)s->Np * s->csz, s->st));
        // a new state clears a timed-out wait recorded by earlier steps
        CK(cudaMemsetAsync(s->d_err, 0, sizeof(int), s->st));
        if (s->cfg.kernel == JLB_KERNEL_CXX)
            r = aux_init_cxx(s->geom, s->cfg.rlx_scheme, s->cfg.kernel_opts, dph, dden, dvel,
                             s->accf ? (const double *)s->acc : nullptr, s->g, s->tau, s->we, s->wo, (double *)s->f,
                             (double *)s->mom[0], (double *)s->mom[1], (double *)s->mom[2], (double *)s->mom[3],
                             s->st);
        else
            r = aux_init(s->prec, s->geom, dph, dden, dvel, s->we, s->f, s->mom[0], s->mom[1], s->mom[2],
                         s->mom[3], s->st);
        ++s->launches;
        cudaError_t es = cudaStreamSynchronize(s->st);
        cudaFree(dph); cudaFree(dden); cudaFree(dvel);
        if (r) return fail(s, JLB_ERR_CUDA, std::string("init kernel: ") + cudaGetErrorString((cudaError_t)r));
        CK(es);
        choose_kernel(s);
    } else {
        s->nfluid = 0;
    }
    s->parity = 0;
    s->init_done = true;
    if (nfluid) *nfluid = cnt;
    return JLB_OK;
}

// per-site field from a halo-padded (NI,NJ,NK,3) host array; an all-zero or
// NULL array switches the field off
static int set_acc_field(jlb_solver *s, const double *acc) {
    bool accf = false;
    if (acc) {
        for (int I = 1; I < s->NI - 1 && !accf; ++I)
            for (int J = 1; J < s->NJ - 1 && !accf; ++J)
                for (int K = 1; K < s->NK - 1; ++K) {
                    const double *a = acc + 3 * fidx(s, I, J, K);
                    if (a[0] != 0.0 || a[1] != 0.0 || a[2] != 0.0) { accf = true; break; }
                }
    }
    if (accf) {
        if (!s->acc) CK(cudaMalloc(&s->acc, (size_t)3 * s->Np * s->csz));
        const double *da = (const double *)dev_view(acc);
        if (da) {
            CKR(aux_acc_upload(s->prec, s->geom, da, s->acc, s->st));
            s->h2d_bytes += (uint64_t)s->N * 3 * sizeof(double);
        } else {
            double *tmp = nullptr;
            CK(cudaMalloc(&tmp, (size_t)3 * s->NCNT * sizeof(double)));
            cudaMemcpyAsync(tmp, acc, (size_t)3 * s->NCNT * sizeof(double), cudaMemcpyHostToDevice, s->st);
            int rr = aux_acc_upload(s->prec, s->geom, tmp, s->acc, s->st);
            cudaStreamSynchronize(s->st);
            cudaFree(tmp);
            CKR(rr);
        }
        ++s->launches;
    }
    if (accf != s->accf) { s->accf = accf; ++s->args_version; }
    return JLB_OK;
}

int jlb_set_acc(jlb_solver *s, const double *acc) {
    if (!s) return fail(s, JLB_ERR_INVALID_ARG, "NULL solver");
    int r = set_acc_field(s, acc);
    if (r) return r;
    CK(cudaStreamSynchronize(s->st));
    return JLB_OK;
}

int jlb_set_static_halo(jlb_solver *s, int on) {
    if (!s) return fail(s, JLB_ERR_INVALID_ARG, "NULL solver");
    s->static_halo = on != 0;
    if (s->init_done) select_checked_walls(s);
    return JLB_OK;
}

int jlb_evolve(jlb_solver *s, uint32_t tsteps, const double g[3], double *den, double *vel, const double *acc,
               uint32_t *tot) {
    if (!s) return fail(s, JLB_ERR_INVALID_ARG, "NULL solver");
    if (!den || !vel) return fail(s, JLB_ERR_INVALID_ARG, "NULL den/vel");
    // the reference copies the bc data first, before its own checks and halo
    // rules (jyulb/isothermal.pyx:1398); counted in host phase 0
    {
        const auto t_bc = std::chrono::steady_clock::now();
        snapshot_bc_data(s, den, vel);
        s->host_t[0] += std::chrono::duration<double>(std::chrono::steady_clock::now() - t_bc).count();
    }
    if (!s->init_done)
        return fail(s, JLB_ERR_STATE, "Finalize solver initialization before calling evolve\n"
                                      "(i.e. call first the method finalize_init)!");
    if (g) {
        for (int d = 0; d < 3; ++d) {
            if (!std::isfinite(g[d])) return fail(s, JLB_ERR_INVALID_ARG, "Invalid gravity input.");
            if (g[d] != s->g[d]) { s->g[d] = g[d]; ++s->args_version; }
        }
    }
    if (s->nfluid < 1 || tsteps == 0) {
        if (tot) *tot = s->tot;
        return JLB_OK;
    }
    using clk = std::chrono::steady_clock;
    auto since = [](clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); };
    const auto t_start = clk::now();
    enforce_den_vel(s, den, vel);
    // solid velocities: reclassify when any of them changed since the last call
    int changed = 0;
    const int64_t nchk = (int64_t)s->wall_chk.size();
    const double *dvel = (const double *)dev_view(vel);
    if (nchk > 0 && dvel) {
        int r = wall_check_device(s, dvel, changed);
        if (r) return r;
    } else {
#pragma omp parallel for schedule(static) reduction(| : changed) if (nchk > 16384)
        for (int64_t c = 0; c < nchk; ++c) {
            const int64_t w = s->wall_chk[c];
            const double *u = vel + 3 * s->wall_pos[w];
            changed |= (u[0] != s->wall_vel[3 * w]) | (u[1] != s->wall_vel[3 * w + 1]) | (u[2] != s->wall_vel[3 * w + 2]);
        }
    }
    if (changed) {
        build_special(s, vel);
        int r = upload_tables(s);
        if (r) return r;
    }
    s->host_t[0] += since(t_start);
    auto t1 = clk::now();
    int r = upload_dynamic(s, den, vel);
    s->host_t[1] += since(t1);
    t1 = clk::now();
    if (r) return r;
    // acceleration field (read every step by the reference, jyulb/isothermal.pyx:1293-1295)
    if ((r = set_acc_field(s, acc))) return r;
    s->host_t[2] += since(t1);
    t1 = clk::now();
    if (s->cfg.kernel == JLB_KERNEL_CXX && s->M > 0)
        return fail(s, JLB_ERR_UNSUPPORTED, "the C++-executable kernel has no moving solids");
    const bool overlap = !overlap_off() && !s->sparse && dma_ready(s, den, vel);
    // The reference refreshes the periodic / symmetric halos of den and vel
    // at the start of every step (jyulb/isothermal.pyx:1408-1411), so after
    // evolve(n) they hold the images of step n-1's moments: run n-1 steps with
    // moments, bring the layers the halo rules read into the host arrays,
    // apply the rules, then the last step (whose download rewrites the fluid
    // sites of those layers)
    unsigned halo_axes = 0;
    for (int face = 0; face < 6; ++face)
        if (s->cfg.bc[face] == BC_PERIODIC || s->cfg.bc[face] == BC_SYMMETRIC) halo_axes |= 1u << (face >> 1);
    uint32_t remaining = tsteps;
    if (halo_axes && tsteps >= 2) {
        if ((r = run_steps(s, tsteps - 1, true))) return r;
        if ((r = halo_from_moments(s, den, vel, halo_axes))) return r;
        remaining = 1;
    }
    r = run_steps(s, overlap ? remaining - 1 : remaining, !overlap);
    if (r) return r;
    s->host_t[3] += since(t1);
    t1 = clk::now();
    r = overlap ? final_step_overlapped(s, den, vel) : download(s, den, vel);
    if (r) return r;
    if (s->use_tma && (r = check_kernel_error(s))) return r;
    s->host_t[4] += since(t1);
    s->host_t[5] += since(t_start);
    s->tot += tsteps;
    if (tot) *tot = s->tot;
    return JLB_OK;
}

int jlb_step(jlb_solver *s, uint32_t tsteps, int write_moments) {
    if (!s) return fail(s, JLB_ERR_INVALID_ARG, "NULL solver");
    if (!s->init_done) return fail(s, JLB_ERR_STATE, "finalize_init has not been called");
    if (s->nfluid < 1) return JLB_OK;
    if (s->cfg.kernel == JLB_KERNEL_CXX && s->M > 0)
        return fail(s, JLB_ERR_UNSUPPORTED, "the C++-executable kernel has no moving solids");
    int r = run_steps(s, tsteps, write_moments != 0);
    if (r) return r;
    s->tot += tsteps;
    return JLB_OK;
}

int jlb_download_moments(jlb_solver *s, double *den, double *vel) {
    if (!s || !den || !vel) return fail(s, JLB_ERR_INVALID_ARG, "NULL argument");
    if (!s->init_done) return fail(s, JLB_ERR_STATE, "finalize_init has not been called");
    int r = download(s, den, vel);
    // steps run by jlb_step are checked here, the first synchronising call
    if (r == JLB_OK && s->use_tma) r = check_kernel_error(s);
    return r;
}

int jlb_get_populations(jlb_solver *s, double *f) {
    if (!s || !f) return fail(s, JLB_ERR_INVALID_ARG, "NULL argument");
    if (!s->init_done) return fail(s, JLB_ERR_STATE, "finalize_init has not been called");
    const size_t nb = (size_t)19 * s->N * sizeof(double);
    int r0 = sparse_leave(s);
    if (r0) return r0;
    double *tmp = nullptr;
    CK(cudaMalloc(&tmp, nb));
    int r = aux_readout(s->prec, s->geom, s->f, s->nmask, s->parity, s->M, s->d_sp_node, s->d_sp_wr, tmp, s->st);
    s->launches += 1 + (s->M > 0);
    cudaError_t e = r ? (cudaError_t)r : cudaMemcpyAsync(f, tmp, nb, cudaMemcpyDeviceToHost, s->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    cudaFree(tmp);
    CK(e);
    // steps run by jlb_step are checked here, the first synchronising call
    return s->use_tma ? check_kernel_error(s) : JLB_OK;
}

int jlb_set_populations(jlb_solver *s, const double *f) {
    if (!s || !f) return fail(s, JLB_ERR_INVALID_ARG, "NULL argument");
    if (!s->init_done) return fail(s, JLB_ERR_STATE, "finalize_init has not been called");
    const size_t nb = (size_t)19 * s->N * sizeof(double);
    double *tmp = nullptr;
    CK(cudaMalloc(&tmp, nb));
    cudaError_t e = cudaMemcpyAsync(tmp, f, nb, cudaMemcpyHostToDevice, s->st);
    if (e == cudaSuccess) e = (cudaError_t)aux_restore(s->prec, s->geom, s->f, s->nmask, tmp, s->st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_err, 0, sizeof(int), s->st); // the restored state is whole
    s->c_current = false;  // the lattice copy is current again
    ++s->launches;
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->st);
    cudaFree(tmp);
    CK(e);
    s->parity = 0;
    return JLB_OK;
}

int jlb_reduce(jlb_solver *s, double out[8]) {
    if (!s || !out) return fail(s, JLB_ERR_INVALID_ARG, "NULL argument");
    if (!s->init_done) return fail(s, JLB_ERR_STATE, "finalize_init has not been called");
    CKR(aux_reduce(s->prec, s->geom, s->nmask, s->mom[0], s->mom[1], s->mom[2], s->mom[3], s->red_partial,
                   s->red_blocks, s->red_out, s->st));
    s->launches += 2;
    CK(cudaMemcpyAsync(out, s->red_out, 8 * sizeof(double), cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    if (out[7] != 0.0) return fail(s, JLB_ERR_NUMERIC, "non-finite density or velocity found");
    return JLB_OK;
}

int jlb_residual(jlb_solver *s, double *res) {
    if (!s || !res) return fail(s, JLB_ERR_INVALID_ARG, "NULL argument");
    if (!s->init_done) return fail(s, JLB_ERR_STATE, "finalize_init has not been called");
    if (!s->res_prev) {
        const size_t nb = (size_t)3 * s->Np * s->csz;
        CK(cudaMalloc(&s->res_prev, nb));
        CK(cudaMemsetAsync(s->res_prev, 0, nb, s->st));
    }
    CKR(aux_residual(s->prec, s->geom, s->nmask, s->mom[1], s->mom[2], s->mom[3], s->res_prev, s->red_partial,
                     s->red_blocks, s->red_out, s->st));
    s->launches += 2;
    double v[2];
    CK(cudaMemcpyAsync(v, s->red_out, sizeof(v), cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    if (!std::isfinite(v[0]) || !std::isfinite(v[1])) return fail(s, JLB_ERR_NUMERIC, "non-finite velocity found");
    *res = v[1] > 0.0 ? std::sqrt(v[0] / v[1]) : (v[0] > 0.0 ? 1.0 : 0.0);
    return JLB_OK;
}

int jlb_flow_info(jlb_solver *s, double ref_den, double out[12]) {
    if (!s || !out) return fail(s, JLB_ERR_INVALID_ARG, "NULL argument");
    if (!s->init_done) return fail(s, JLB_ERR_STATE, "finalize_init has not been called");
    if (!s->fi_partial) {
        CK(cudaMalloc(&s->fi_partial, (size_t)12 * s->red_blocks * sizeof(double)));
        CK(cudaMalloc(&s->fi_out, 12 * sizeof(double)));
    }
    CKR(aux_flow_info(s->prec, s->geom, s->nmask, s->mom[0], s->mom[1], s->mom[2], s->mom[3], ref_den,
                      s->fi_partial, s->red_blocks, s->fi_out, s->st));
    s->launches += 2;
    double v[12];
    CK(cudaMemcpyAsync(v, s->fi_out, sizeof(v), cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    // order of the .evol columns 3-14 (source/isothermal/jyu_lb_isothermal.cpp:21-56)
    out[0] = v[0];
    out[1] = v[1]; out[2] = v[2]; out[3] = v[3];
    out[4] = v[4];
    const double cff = s->nfluid > 0 ? 1.0 / (double)s->nfluid : 0.0;
    out[5] = cff * v[5]; out[6] = cff * v[6]; out[7] = cff * v[7];
    out[8] = cff * v[8];
    out[9] = v[11];
    out[10] = v[9];
    out[11] = v[10];
    return JLB_OK;
}

int jlb_bc_data(const jlb_solver *s, int32_t face, double *den, double *vel) {
    if (!s || face < 0 || face > 5) return JLB_ERR_INVALID_ARG;
    int na, nb;
    face_extent(s, face, na, nb);
    const size_t n = (size_t)na * nb;
    const std::vector<double> &bd = s->bcd_den[face], &bv = s->bcd_vel[face];
    if (den) {
        if (bd.size() == n) std::memcpy(den, bd.data(), n * sizeof(double));
        else std::fill(den, den + n, 1.0);
    }
    if (vel) {
        if (bv.size() == 3 * n) std::memcpy(vel, bv.data(), 3 * n * sizeof(double));
        else std::fill(vel, vel + 3 * n, 0.0);
    }
    return JLB_OK;
}

uint32_t jlb_tot_tsteps(const jlb_solver *s) { return s ? s->tot : 0; }

void jlb_rlx_prm(const jlb_solver *s, double out[2]) {
    if (!s || !out) return;
    out[0] = s->we;
    out[1] = s->wo;
}

uint64_t jlb_kernel_launches(const jlb_solver *s) { return s ? s->launches : 0; }

void jlb_host_timers(const jlb_solver *s, double out[6]) {
    if (!out) return;
    for (int k = 0; k < 6; ++k) out[k] = s ? s->host_t[k] : 0.0;
}

void jlb_transfer_bytes(const jlb_solver *s, uint64_t out[2]) {
    if (!out) return;
    out[0] = s ? s->h2d_bytes : 0;
    out[1] = s ? s->d2h_bytes : 0;
}

const char *jlb_last_error(const jlb_solver *s) {
    if (!s) return g_create_error.c_str();
    return s->err.c_str();
}

const char *jlb_build_info(void) {
    return "libjyulb_gb300: D3Q19 AA-pattern fused step for sm_103a; FP64 (reference arithmetic, no FMA), "
           "FP32 shifted, FP16 storage; BGK/TRT/regularized; bounce-back, Ladd moving walls, Zou-He, "
           "periodic, symmetric";
}

} // extern "C"
