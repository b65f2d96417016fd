// lbm_adjoint_host.cpp -- host driver of the discrete adjoint (jlb_adj_*):
// forward run with checkpoints, segment recomputation on a second stream,
// and the reverse sweep of the adjoint step kernel (lbm_adjoint.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "jyulb_gb300.h"
#include "lbm_common.h"
#include "lbm_adjoint.h"
#include "lbm_solver.h"

using namespace jlb;
using namespace jlb_host;

struct jlb_adjoint {
    jlb_solver *s = nullptr;
    int K = 50;               // checkpoint interval
    int plane = 0;
    double magic = 0.0;       // TRT magic parameter (<= 0: reference's 3/16)
    void *f0 = nullptr;       // initial populations
    std::vector<void *> ckpt; // populations before steps 0, K, 2K, ...
    // recompute buffers, nsets sets of K: set p holds the states before the
    // steps of a segment in snap[p*K + 1 .. p*K + K-1] (snap[p*K] is scratch)
    // and their boundary-site collision inputs in sp_in[p][K][19][M]; with two
    // sets the recompute of one segment overlaps the reverse sweep of the next
    std::vector<void *> snap;
    void *sp_in = nullptr;
    int nsets = 0;
    cudaStream_t st2 = nullptr; // recompute stream
    void *lam = nullptr;
    double *d_target = nullptr, *d_part = nullptr;
    double *d_gbc = nullptr;      // [4][M] d/d (den, ux, uy, uz) of the boundary sites' Zou-He data
    // previous-step density of the boundary sites (compute type; den - 1 when
    // shifted), which the moving-wall links read: at rest, at each checkpoint
    // ([segment][M]), and the recompute's working copy
    void *spd0 = nullptr, *ckpt_spd = nullptr, *spd_scratch = nullptr;
    int ckpt_spd_cap = 0;         // segments ckpt_spd holds
    void *lam_den = nullptr;      // [M] adjoint of the boundary sites' density
    bool moving = false;          // some boundary site has a moving-wall link
    bool den_param = false;       // the last forward run took den as a parameter
    uint32_t param_faces = 0;     // faces whose Zou-He data the last forward run took as parameters
    int nparts = 0;           // per-block sensitivity slots
    uint32_t steps = 0;
    double tau = 1.0;
    bool have_forward = false;
    size_t fbytes = 0;
    std::vector<cudaEvent_t> ev; // forward pair, backward pair, then 4 per backward segment
    double ms[4] = {0, 0, 0, 0};  // forward, recompute, reverse sweep, whole backward
    std::string err;
};

namespace {

int afail(jlb_adjoint *A, int code, const std::string &m) {
    if (A) A->err = m;
    else g_create_error = m;
    return code;
}

#define ACK(call)                                                                                  \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return afail(A, e_ == cudaErrorMemoryAllocation ? JLB_ERR_NOMEM : JLB_ERR_CUDA,        \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                      \
    } while (0)

// the first n timing events, created on first use
cudaError_t adj_events(jlb_adjoint *A, size_t n) {
    while (A->ev.size() < n) {
        cudaEvent_t e;
        const cudaError_t r = cudaEventCreate(&e);
        if (r != cudaSuccess) return r;
        A->ev.push_back(e);
    }
    return cudaSuccess;
}

float adj_elapsed(const jlb_adjoint *A, size_t i, size_t j) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, A->ev[i], A->ev[j]);
    return ms;
}

// relaxation rates of relaxation time tau (jyulb/isothermal.pyx:274-287)
void adj_rates(const jlb_adjoint *A, double tau, double &we, double &wo) {
    we = 1.0 / tau;
    wo = we;
    if (A->s->cfg.rlx_scheme == JLB_TRT)
        wo = A->magic > 0.0 ? 1.0 / (A->magic / (tau - 0.5) + 0.5) : 8.0 * (2.0 - we) / (8.0 - we);
}

} // namespace

extern "C" {

void jlb_adj_destroy(jlb_adjoint *A) {
    if (!A) return;
    if (A->s) cudaStreamSynchronize(A->s->st);
    if (A->st2) { cudaStreamSynchronize(A->st2); cudaStreamDestroy(A->st2); }
    for (void *p : A->ckpt) if (p) cudaFree(p);
    for (void *p : A->snap) if (p) cudaFree(p);
    for (cudaEvent_t e : A->ev) cudaEventDestroy(e);
    void *bufs[] = {A->f0, A->lam, A->sp_in, A->d_target, A->d_part, A->d_gbc,
                    A->spd0, A->ckpt_spd, A->spd_scratch, A->lam_den};
    for (void *p : bufs) if (p) cudaFree(p);
    if (A->s) jlb_destroy(A->s);
    delete A;
}

}  // extern "C"

namespace {

int adj_create(const jlb_config *cfg, const uint8_t *phase, const double *solid_vel, int32_t loss_plane,
               int32_t checkpoint_every, jlb_adjoint **out) {
    jlb_adjoint *A = nullptr;
    if (!cfg || !phase || !out) return afail(nullptr, JLB_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    if (cfg->precision != JLB_FP64 && cfg->precision != JLB_FP32)
        return afail(nullptr, JLB_ERR_UNSUPPORTED, "adjoint supports FP64 and FP32");
    if (checkpoint_every < 1) return afail(nullptr, JLB_ERR_INVALID_ARG, "checkpoint interval must be >= 1");
    if (cfg->kernel != JLB_KERNEL_JYULB)
        return afail(nullptr, JLB_ERR_UNSUPPORTED, "adjoint supports the jyulb collision kernel");
    if (loss_plane < 0 || loss_plane >= cfg->lat_size[0]) return afail(nullptr, JLB_ERR_INVALID_ARG, "loss plane out of range");
    A = new jlb_adjoint();
    A->K = checkpoint_every;
    A->plane = loss_plane;
    A->magic = cfg->trt_magic;
    int r = jlb_create(cfg, &A->s);
    if (r) { std::string m = g_create_error; delete A; return afail(nullptr, r, m); }
    jlb_solver *s = A->s;
    s->no_sparse = true;  // checkpoints and recomputation work on the lattice layout
    s->no_lin = true;
    // rest state: den = 1, vel = 0 at the fluid sites, so the initial
    // populations do not depend on the parameters; solid sites carry their
    // wall velocity (moving bounce-back with Ladd's term)
    std::vector<uint8_t> ph((size_t)s->NCNT, 0);
    std::vector<double> den((size_t)s->NCNT, 1.0), vel(3 * (size_t)s->NCNT, 0.0);
    for (int i = 0; i < s->nx; ++i)
        for (int j = 0; j < s->ny; ++j)
            for (int k = 0; k < s->nz; ++k) {
                const size_t n = ((size_t)i * s->ny + j) * s->nz + k;
                const int64_t fn = fidx(s, i + 1, j + 1, k + 1);
                ph[fn] = phase[n];
                if (solid_vel && phase[n] == 0)
                    for (int c = 0; c < 3; ++c) vel[3 * fn + c] = solid_vel[3 * n + c];
            }
    uint64_t nf = 0;
    if ((r = jlb_finalize_init(s, ph.data(), den.data(), vel.data(), &nf))) {
        std::string m = s->err;
        jlb_adj_destroy(A);
        return afail(nullptr, r, m);
    }
    A->fbytes = (size_t)19 * s->Np * s->ssz;
    auto bail = [&](const char *m) { jlb_adj_destroy(A); return afail(nullptr, JLB_ERR_NOMEM, m); };
    if (cudaMalloc(&A->f0, A->fbytes) != cudaSuccess || cudaMalloc(&A->lam, A->fbytes) != cudaSuccess ||
        cudaMalloc(&A->d_target, 3 * sizeof(double) * (size_t)s->ny * s->nz) != cudaSuccess) {
        cudaGetLastError();
        return bail("adjoint state allocation failed");
    }
    A->nparts = adjoint_blocks(make_args(s, 0));
    const size_t M1 = (size_t)std::max(s->M, 1);
    if (cudaMalloc(&A->d_part, 5 * sizeof(double) * (size_t)A->nparts) != cudaSuccess ||
        (s->M > 0 && cudaMalloc(&A->sp_in, (size_t)2 * A->K * 19 * s->M * s->ssz) != cudaSuccess) ||
        cudaMalloc(&A->d_gbc, 4 * sizeof(double) * M1) != cudaSuccess ||
        cudaMalloc(&A->spd0, M1 * s->csz) != cudaSuccess || cudaMalloc(&A->spd_scratch, M1 * s->csz) != cudaSuccess ||
        cudaMalloc(&A->lam_den, M1 * s->csz) != cudaSuccess ||
        cudaStreamCreateWithFlags(&A->st2, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        return bail("adjoint state allocation failed");
    }
    // density 1 at rest: 1.0 in FP64, den - 1 = 0 in the shifted FP32 form
    if (s->prec == PREC_FP64) {
        std::vector<double> one(M1, 1.0);
        cudaMemcpy(A->spd0, one.data(), M1 * sizeof(double), cudaMemcpyHostToDevice);
    } else {
        cudaMemset(A->spd0, 0, M1 * s->csz);
    }
    for (int t = 0; t < s->M; ++t)
        if (s->sp_info[t] & ((1u << 19) - 1u)) A->moving = true;
    cudaMemcpy(A->f0, s->f, A->fbytes, cudaMemcpyDeviceToDevice);
    *out = A;
    return JLB_OK;
}

// Zou-He data of boundary site t on face `face`: out = (den, ux, uy, uz)
using BcFill = std::function<void(int t, int face, int64_t n, double *out)>;

// den_field (nx,ny,nz) or NULL: the boundary sites' previous-step density
// for the first step, as Solver.evolve reads it from den; NULL: 1 (rest)
int adj_forward(jlb_adjoint *A, double tau, const double g[3], const BcFill &fill, uint32_t param_faces,
                const double *den_field, uint32_t steps, const double *target, double *loss, double *u_plane) {
    if (!A || !g || steps < 1) return afail(A, JLB_ERR_INVALID_ARG, "bad argument");
    if (!(tau > 0.5)) return afail(A, JLB_ERR_INVALID_ARG, "tau must exceed 1/2");
    jlb_solver *s = A->s;
    double we, wo;
    adj_rates(A, tau, we, wo);
    s->we = we;
    s->wo = wo;
    for (int d = 0; d < 3; ++d) s->g[d] = g[d];
    ++s->args_version;
    // Zou-He data of the boundary sites, in the forward step's slot order
    const int M = s->M;
    const size_t nb = 4 * (size_t)std::max(s->bc_slots, 1) * M;
    std::vector<double> bc(nb, 0.0);
    for (int t = 0; t < M; ++t) {
        const int64_t n = s->sp_node[t];
        const uint32_t faces = (s->sp_info[t] >> SP_FACE_SHIFT) & 0x3Fu;
        int slot = 0;
        for (int face = 0; face < 6; ++face) {
            if (!(faces & (1u << face))) continue;
            double d[4] = {1.0, 0.0, 0.0, 0.0};
            fill(t, face, n, d);
            for (int c = 0; c < 4; ++c) bc[(size_t)(4 * slot + c) * M + t] = d[c];
            slot = 1;
        }
    }
    const int nseg = (int)((steps + A->K - 1) / A->K);
    if (M > 0) {
        ACK(cudaMemcpyAsync(s->d_sp_bc, bc.data(), nb * sizeof(double), cudaMemcpyHostToDevice, s->st));
        if (den_field) {
            std::vector<double> d64(M);
            std::vector<float> d32(M);
            for (int t = 0; t < M; ++t) {
                d64[t] = den_field[s->sp_node[t]];
                d32[t] = (float)(d64[t] - 1.0);
            }
            ACK(cudaMemcpyAsync(s->d_sp_den, s->prec == PREC_FP64 ? (const void *)d64.data() : (const void *)d32.data(),
                                (size_t)M * s->csz, cudaMemcpyHostToDevice, s->st));
            ACK(cudaStreamSynchronize(s->st));
        } else {
            ACK(cudaMemcpyAsync(s->d_sp_den, A->spd0, (size_t)M * s->csz, cudaMemcpyDeviceToDevice, s->st));
        }
        if (A->ckpt_spd_cap < nseg) {
            ACK(cudaStreamSynchronize(s->st));
            if (A->ckpt_spd) cudaFree(A->ckpt_spd);
            A->ckpt_spd = nullptr;
            A->ckpt_spd_cap = 0;
            ACK(cudaMalloc(&A->ckpt_spd, (size_t)nseg * M * s->csz));
            A->ckpt_spd_cap = nseg;
        }
    }
    A->param_faces = param_faces;
    A->den_param = den_field != nullptr;
    // forward with checkpoints
    ACK(adj_events(A, 2));
    ACK(cudaEventRecord(A->ev[0], s->st));
    ACK(cudaMemcpyAsync(s->f, A->f0, A->fbytes, cudaMemcpyDeviceToDevice, s->st));
    s->parity = 0;
    while ((int)A->ckpt.size() < nseg) {
        void *p = nullptr;
        ACK(cudaMalloc(&p, A->fbytes));
        A->ckpt.push_back(p);
    }
    for (int seg = 0; seg < nseg; ++seg) {
        ACK(cudaMemcpyAsync(A->ckpt[seg], s->f, A->fbytes, cudaMemcpyDeviceToDevice, s->st));
        if (M > 0)
            ACK(cudaMemcpyAsync((char *)A->ckpt_spd + (size_t)seg * M * s->csz, s->d_sp_den, (size_t)M * s->csz,
                                cudaMemcpyDeviceToDevice, s->st));
        const uint32_t t0 = (uint32_t)seg * A->K, t1 = std::min<uint32_t>(steps, t0 + A->K);
        int r = run_steps(s, t1 - t0, t1 == steps);
        if (r) return afail(A, r, s->err);
    }
    ACK(cudaEventRecord(A->ev[1], s->st));
    // stored velocity on the loss plane, and the loss
    const size_t plane_n = (size_t)s->ny * s->nz;
    const int64_t p0 = (int64_t)A->plane * s->ny * s->nz;
    std::vector<double> up(3 * plane_n);
    std::vector<uint32_t> pm(plane_n);
    ACK(cudaMemcpyAsync(pm.data(), s->nmask + p0, plane_n * 4, cudaMemcpyDeviceToHost, s->st));
    for (int c = 0; c < 3; ++c) {
        if (s->prec == PREC_FP64) {
            ACK(cudaMemcpyAsync(up.data() + c * plane_n, (double *)s->mom[1 + c] + p0, plane_n * 8,
                                cudaMemcpyDeviceToHost, s->st));
        } else {
            std::vector<float> tmp(plane_n);
            ACK(cudaMemcpyAsync(tmp.data(), (float *)s->mom[1 + c] + p0, plane_n * 4, cudaMemcpyDeviceToHost, s->st));
            ACK(cudaStreamSynchronize(s->st));
            for (size_t m = 0; m < plane_n; ++m) up[c * plane_n + m] = tmp[m];
        }
    }
    ACK(cudaStreamSynchronize(s->st));
    A->ms[0] = adj_elapsed(A, 0, 1);
    double L = 0.0;
    for (size_t m = 0; m < plane_n; ++m) {
        if (pm[m] & MASK_SOLID) continue;
        for (int c = 0; c < 3; ++c) {
            const double u = up[c * plane_n + m];
            if (u_plane) u_plane[3 * m + c] = u;
            if (target) { const double d = u - target[3 * m + c]; L += d * d; }
        }
    }
    std::vector<double> tg(3 * plane_n, 0.0);
    if (target)
        for (size_t m = 0; m < plane_n; ++m)
            if (!(pm[m] & MASK_SOLID)) for (int c = 0; c < 3; ++c) tg[3 * m + c] = target[3 * m + c];
    ACK(cudaMemcpy(A->d_target, tg.data(), tg.size() * sizeof(double), cudaMemcpyHostToDevice));
    if (loss) *loss = L;
    A->steps = steps;
    A->tau = tau;
    A->have_forward = true;
    return JLB_OK;
}

// the reverse sweep; leaves d/d (den, ux, uy, uz) of the boundary sites'
// Zou-He data in gbc ([4][M], host)
int adj_backward(jlb_adjoint *A, double *dtau, double dg[3], std::vector<double> &gbc) {
    if (!A) return afail(A, JLB_ERR_INVALID_ARG, "NULL adjoint");
    if (!A->have_forward) return afail(A, JLB_ERR_STATE, "run jlb_adj_forward first");
    jlb_solver *s = A->s;
    const uint32_t steps = A->steps;
    const int K = A->K;
    const int nseg = (int)((steps + K - 1) / K);
    // one buffer set, a second when memory allows (and there is a next segment)
    const int want = nseg > 1 ? 2 : 1;
    while (A->nsets < want) {
        std::vector<void *> set;
        bool ok = true;
        for (int i = 0; i < K && ok; ++i) {
            void *p = nullptr;
            ok = cudaMalloc(&p, A->fbytes) == cudaSuccess;
            if (ok) set.push_back(p);
        }
        if (!ok) {
            cudaGetLastError();
            for (void *p : set) cudaFree(p);
            if (A->nsets == 0) return afail(A, JLB_ERR_NOMEM, "adjoint recompute buffers");
            break;
        }
        A->snap.insert(A->snap.end(), set.begin(), set.end());
        ++A->nsets;
    }
    const int nsets = std::min(A->nsets, want);
    ACK(adj_events(A, 4 + 4 * (size_t)nseg));
    cudaEvent_t *ev = A->ev.data();
    cudaStream_t st = s->st, st2 = A->st2;
    ACK(cudaEventRecord(ev[2], st));
    ACK(cudaMemsetAsync(A->lam, 0, A->fbytes, st));
    ACK(cudaMemsetAsync(A->d_part, 0, 5 * sizeof(double) * (size_t)A->nparts, st));
    const size_t M1 = (size_t)std::max(s->M, 1);
    ACK(cudaMemsetAsync(A->d_gbc, 0, 4 * sizeof(double) * M1, st));
    ACK(cudaMemsetAsync(A->lam_den, 0, M1 * s->csz, st));
    ACK(cudaStreamWaitEvent(st2, ev[2], 0)); // checkpoints of the forward run are complete
    const size_t sp_step = (size_t)19 * s->M * s->ssz; // bytes of one step's boundary-site inputs
    auto seg_ev = [&](int seg) { return ev + 4 + 4 * (size_t)seg; }; // rc start, rc end, rv start, rv end
    auto range = [&](int seg, uint32_t &t0, uint32_t &t1) {
        t0 = (uint32_t)seg * K;
        t1 = std::min<uint32_t>(steps, t0 + K);
    };
    auto state_before = [&](int seg, uint32_t t) -> void * {
        const uint32_t t0 = (uint32_t)seg * K;
        return t == t0 ? A->ckpt[seg] : A->snap[(size_t)(seg % nsets) * K + (t - t0)];
    };
    auto sp_in_of = [&](int seg, uint32_t t) -> void * {
        if (s->M == 0) return nullptr;
        return (char *)A->sp_in + ((size_t)(seg % nsets) * K + (t - (uint32_t)seg * K)) * sp_step;
    };
    // recompute a segment out of place on st2; its last step's outputs are not
    // needed, so that step runs the boundary sites only (into the scratch slot)
    auto recompute = [&](int seg) -> int {
        uint32_t t0, t1;
        range(seg, t0, t1);
        ACK(cudaEventRecord(seg_ev(seg)[0], st2));
        if (s->M > 0)
            ACK(cudaMemcpyAsync(A->spd_scratch, (char *)A->ckpt_spd + (size_t)seg * s->M * s->csz,
                                (size_t)s->M * s->csz, cudaMemcpyDeviceToDevice, st2));
        for (uint32_t t = t0; t < t1; ++t) {
            StepArgs a = make_args(s, 0);
            a.sp_den = A->spd_scratch;
            a.f = state_before(seg, t);
            a.fout = t + 1 < t1 ? state_before(seg, t + 1) : A->snap[(size_t)(seg % nsets) * K];
            a.sp_tee = sp_in_of(seg, t);
            if (t + 1 == t1) a.nb_dense = 0;
            if (a.nb_dense == 0 && a.M == 0) continue;
            const int blocks = a.nb_dense + special_blocks(a);
            const bool pstep = (t & 1u) == 0;
            const int r = s->prec == PREC_FP64 ? launch_step_fp64(a, s->cfg.rlx_scheme, pstep, s->accf, blocks, st2)
                                               : launch_step_fp32(a, s->cfg.rlx_scheme, pstep, s->accf, blocks, st2);
            if (r) return afail(A, JLB_ERR_CUDA, std::string("recompute step: ") + cudaGetErrorString((cudaError_t)r));
            ++s->launches;
        }
        ACK(cudaEventRecord(seg_ev(seg)[1], st2));
        return JLB_OK;
    };
    int r = recompute(nseg - 1);
    if (r) return r;
    for (int seg = nseg - 1; seg >= 0; --seg) {
        uint32_t t0, t1;
        range(seg, t0, t1);
        ACK(cudaStreamWaitEvent(st, seg_ev(seg)[1], 0));
        ACK(cudaEventRecord(seg_ev(seg)[2], st));
        for (int64_t t = (int64_t)t1 - 1; t >= (int64_t)t0; --t) {
            AdjArgs a{};
            a.s = make_args(s, 0);
            a.snap = state_before(seg, (uint32_t)t);
            a.sp_in = sp_in_of(seg, (uint32_t)t);
            a.lam = A->lam;
            a.seed = (uint32_t)t == steps - 1;
            a.plane = A->plane;
            a.target = A->d_target;
            a.part = A->d_part;
            a.grad_bc = A->d_gbc;
            a.param_faces = A->param_faces;
            a.lam_den = A->moving ? A->lam_den : nullptr;
            r = launch_adjoint_step(a, s->prec, s->cfg.rlx_scheme, (t & 1) == 0, st);
            if (r) return afail(A, JLB_ERR_CUDA, std::string("adjoint step: ") + cudaGetErrorString((cudaError_t)r));
            s->launches += 2;
        }
        ACK(cudaEventRecord(seg_ev(seg)[3], st));
        if (seg > 0) {
            // the buffer set of segment seg-1 was last read by the sweep of
            // segment seg-1+nsets
            if (seg - 1 + nsets < nseg) ACK(cudaStreamWaitEvent(st2, seg_ev(seg - 1 + nsets)[3], 0));
            if ((r = recompute(seg - 1))) return r;
        }
    }
    ACK(cudaEventRecord(ev[3], st));
    std::vector<double> part(5 * (size_t)A->nparts);
    ACK(cudaMemcpyAsync(part.data(), A->d_part, part.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    gbc.assign(4 * M1, 0.0);
    ACK(cudaMemcpyAsync(gbc.data(), A->d_gbc, 4 * sizeof(double) * M1, cudaMemcpyDeviceToHost, st));
    // the adjoint of the first step's previous-step density is the gradient
    // of den at the boundary sites, when den was a parameter
    std::vector<double> lam0;
    if (A->den_param && A->moving) {
        lam0.resize(M1);
        if (s->prec == PREC_FP64) {
            ACK(cudaMemcpyAsync(lam0.data(), A->lam_den, M1 * sizeof(double), cudaMemcpyDeviceToHost, st));
        } else {
            std::vector<float> l32(M1);
            ACK(cudaMemcpyAsync(l32.data(), A->lam_den, M1 * sizeof(float), cudaMemcpyDeviceToHost, st));
            ACK(cudaStreamSynchronize(st));
            for (size_t t = 0; t < M1; ++t) lam0[t] = l32[t];
        }
    }
    ACK(cudaStreamSynchronize(st));
    for (size_t t = 0; t < lam0.size(); ++t) gbc[t] += lam0[t];
    double gr[5] = {0, 0, 0, 0, 0};
    for (int b = 0; b < A->nparts; ++b)
        for (int c = 0; c < 5; ++c) gr[c] += part[5 * (size_t)b + c];
    A->ms[1] = A->ms[2] = 0.0;
    for (int seg = 0; seg < nseg; ++seg) {
        A->ms[1] += adj_elapsed(A, 4 + 4 * (size_t)seg, 5 + 4 * (size_t)seg);
        A->ms[2] += adj_elapsed(A, 6 + 4 * (size_t)seg, 7 + 4 * (size_t)seg);
    }
    A->ms[3] = adj_elapsed(A, 2, 3);
    // chain rule to tau: we = 1/tau, wo(tau) from the magic parameter
    double we, wo;
    adj_rates(A, A->tau, we, wo);
    double dwo_dtau = 0.0;
    if (s->cfg.rlx_scheme == JLB_TRT) {
        const double magic = A->magic > 0.0 ? A->magic : 3.0 / 16.0;
        dwo_dtau = wo * wo * magic / ((A->tau - 0.5) * (A->tau - 0.5));
    }
    if (dtau) {
        if (s->cfg.rlx_scheme == JLB_TRT) *dtau = gr[0] * (-we * we) + gr[1] * dwo_dtau;
        else *dtau = (gr[0] + gr[1]) * (-we * we);
    }
    if (dg) for (int d = 0; d < 3; ++d) dg[d] = gr[2 + d];
    return JLB_OK;
}

// faces whose data the solver refreshes from the den / vel fields at every
// call (the fixed faces; Z1 only when bc[Z1] is FIXED_DEN or bc[1Z] is
// FIXED_VEL, jyulb/isothermal.pyx:500)
uint32_t refreshed_faces(const jlb_solver *s) {
    uint32_t m = 0;
    for (int f = 0; f < 6; ++f) {
        bool r = s->cfg.bc[f] == JLB_FIXED_VEL || s->cfg.bc[f] == JLB_FIXED_DEN;
        if (f == 5) r = s->cfg.bc[5] == JLB_FIXED_DEN || s->cfg.bc[4] == JLB_FIXED_VEL;
        if (r) m |= 1u << f;
    }
    return m;
}

} // namespace

extern "C" {

int jlb_adj_create(const jlb_config *cfg, const uint8_t *phase, int32_t loss_plane, int32_t checkpoint_every,
                   jlb_adjoint **out) {
    return adj_create(cfg, phase, nullptr, loss_plane, checkpoint_every, out);
}

int jlb_adj_create_moving(const jlb_config *cfg, const uint8_t *phase, const double *solid_vel, int32_t loss_plane,
                          int32_t checkpoint_every, jlb_adjoint **out) {
    if (!solid_vel) return afail(nullptr, JLB_ERR_INVALID_ARG, "NULL solid velocity");
    return adj_create(cfg, phase, solid_vel, loss_plane, checkpoint_every, out);
}

int jlb_adj_forward(jlb_adjoint *A, double tau, const double g[3], const double *uin, double rho_out, uint32_t steps,
                    const double *target, double *loss, double *u_plane) {
    if (!A || !uin) return afail(A, JLB_ERR_INVALID_ARG, "bad argument");
    const jlb_solver *s = A->s;
    for (int f = 1; f < 6; ++f)
        if (s->cfg.bc[f] == JLB_FIXED_VEL)
            return afail(A, JLB_ERR_UNSUPPORTED, "jlb_adj_forward: FIXED_VEL on a face other than 1X needs jlb_adj_forward_fields");
    // inlet 1X velocity (uin[j*nz+k], 0, 0), density rho_out on FIXED_DEN faces
    const BcFill fill = [&](int, int face, int64_t n, double *d) {
        if (s->cfg.bc[face] == JLB_FIXED_VEL) {
            d[1] = uin[(size_t)(n % ((int64_t)s->ny * s->nz))];
        } else {
            d[0] = rho_out;
        }
    };
    const uint32_t pf = s->cfg.bc[0] == JLB_FIXED_VEL ? 1u : 0u;
    return adj_forward(A, tau, g, fill, pf, nullptr, steps, target, loss, u_plane);
}

int jlb_adj_forward_fields(jlb_adjoint *A, double tau, const double g[3], const double *den, const double *vel,
                           uint32_t steps, const double *target, double *loss, double *u_plane) {
    if (!A) return afail(A, JLB_ERR_INVALID_ARG, "NULL adjoint");
    const jlb_solver *s = A->s;
    const uint32_t pf = refreshed_faces(s);
    const BcFill fill = [&](int, int face, int64_t n, double *d) {
        if (!((pf >> face) & 1u)) return; // den 1, vel 0
        if (den) d[0] = den[n];
        if (vel) for (int c = 0; c < 3; ++c) d[1 + c] = vel[3 * n + c];
    };
    return adj_forward(A, tau, g, fill, pf, den, steps, target, loss, u_plane);
}

int jlb_adj_backward(jlb_adjoint *A, double *dtau, double dg[3], double *duin) {
    std::vector<double> gbc;
    const int r = adj_backward(A, dtau, dg, gbc);
    if (r || !duin) return r;
    const jlb_solver *s = A->s;
    const size_t M1 = (size_t)std::max(s->M, 1);
    std::fill(duin, duin + (size_t)s->ny * s->nz, 0.0);
    if (s->cfg.bc[0] == JLB_FIXED_VEL)
        for (int t = 0; t < s->M; ++t)
            if ((s->sp_info[t] >> SP_FACE_SHIFT) & 1u) {
                const int64_t n = s->sp_node[t];
                duin[(size_t)(n % ((int64_t)s->ny * s->nz))] += gbc[M1 + t];
            }
    return JLB_OK;
}

int jlb_adj_backward_fields(jlb_adjoint *A, double *dtau, double dg[3], double *dden, double *dvel) {
    std::vector<double> gbc;
    const int r = adj_backward(A, dtau, dg, gbc);
    if (r) return r;
    const jlb_solver *s = A->s;
    const size_t M1 = (size_t)std::max(s->M, 1);
    if (dden) std::fill(dden, dden + (size_t)s->N, 0.0);
    if (dvel) std::fill(dvel, dvel + 3 * (size_t)s->N, 0.0);
    for (int t = 0; t < s->M; ++t) {
        const int64_t n = s->sp_node[t];
        if (dden) dden[n] += gbc[t];
        if (dvel) for (int c = 0; c < 3; ++c) dvel[3 * n + c] += gbc[(1 + c) * M1 + t];
    }
    return JLB_OK;
}

int jlb_adj_timers(const jlb_adjoint *A, double out[4]) {
    if (!A || !out) return JLB_ERR_INVALID_ARG;
    for (int i = 0; i < 4; ++i) out[i] = A->ms[i];
    return JLB_OK;
}

const char *jlb_adj_last_error(const jlb_adjoint *A) { return A ? A->err.c_str() : g_create_error.c_str(); }

} // extern "C"
