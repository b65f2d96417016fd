// lbm_batch_host.cpp -- host runtime of the batched ensemble (jlb_batch_*):
// packs many independent domains, each set up by a single-domain solver,
// into one population array and drives the packed step kernel
// (lbm_batch.cu), its boundary-node launch and their CUDA graphs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "jyulb_gb300.h"
#include "lbm_common.h"
#include "lbm_batch.h"
#include "lbm_solver.h"

using namespace jlb;
using namespace jlb_host;

struct jlb_batch {
    int scheme = 0;
    int ndom = 0;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    std::vector<BatchDomain> dom;
    std::vector<int32_t> nfluid_dom;
    int64_t Np = 0, ntot = 0, nfluid = 0;
    int block = 128, ntiles = 0;
    // device
    float *f = nullptr, *dprev = nullptr, *mom[4] = {nullptr, nullptr, nullptr, nullptr};
    uint8_t *ncls = nullptr;
    uint32_t *nmask = nullptr, *mmask = nullptr;
    BatchDomain *d_dom = nullptr;
    int32_t *tile_dom = nullptr;
    int parity = 0;
    uint32_t tot = 0;
    uint64_t launches = 0;
    double tune_ms[3] = {0, 0, 0}; // per-step time of blocks 64 / 128 / 256
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    int GK = 32;
    // boundary nodes of domains with Zou-He or symmetric faces (device
    // tables in the single-domain layout, element indices into f)
    int Msp = 0;
    std::vector<int> sp_first;    // [ndom + 1]: domain d owns boundary nodes [sp_first[d], sp_first[d+1])
    int32_t *d_sp_dom = nullptr;
    int64_t *d_sp_node = nullptr, *d_sp_rd = nullptr, *d_sp_wr = nullptr;
    uint32_t *d_sp_info = nullptr;
    double *d_sp_lw = nullptr, *d_sp_bc = nullptr;
    float *d_sp_den = nullptr;
    int pf = 0;                      // L2 prefetch distance in tiles of the current block size
    int pf_tiles = -1;               // JLB_BATCH_PF: fixed distance in tiles (0: none)
    bool pf_big = false;             // populations larger than twice the L2
    int sms = 0;                     // multiprocessors of the device
    std::vector<int64_t> h_sp_node;  // [Msp] packed node of each boundary node
    std::vector<uint32_t> h_sp_info; // [Msp] its link / face bits
    std::string err;
};

namespace {

int bfail(jlb_batch *b, int code, const std::string &m) {
    if (b) b->err = m;
    else g_create_error = m;
    return code;
}

#define BCK(call)                                                                                  \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return bfail(b, e_ == cudaErrorMemoryAllocation ? JLB_ERR_NOMEM : JLB_ERR_CUDA,        \
                         std::string(#call) + ": " + cudaGetErrorString(e_));                      \
    } while (0)

BatchArgs batch_args(const jlb_batch *b, int write_moments) {
    BatchArgs a{};
    a.f = b->f;
    a.Np = b->Np;
    for (int q = 0; q < 19; ++q) a.fq[q] = b->f + (size_t)q * b->Np;
    a.dom = b->d_dom;
    a.tile_dom = b->tile_dom;
    a.ncls = b->ncls;
    a.nmask = b->nmask;
    a.mmask = b->mmask;
    a.dprev = b->dprev;
    a.den = b->mom[0]; a.ux = b->mom[1]; a.uy = b->mom[2]; a.uz = b->mom[3];
    a.write_moments = write_moments;
    a.ntiles = b->ntiles;
    a.pf = b->pf;
    a.Msp = b->Msp;
    a.sp_dom = b->d_sp_dom;
    a.sp_node = b->d_sp_node; a.sp_rd = b->d_sp_rd; a.sp_wr = b->d_sp_wr;
    a.sp_info = b->d_sp_info;
    a.sp_lw = b->d_sp_lw; a.sp_bc = b->d_sp_bc;
    a.sp_den = b->d_sp_den;
    return a;
}

// tile table for block size `block`; also sets first_tile of every domain
int batch_tiles(jlb_batch *b, int block) {
    std::vector<int32_t> td;
    for (int d = 0; d < b->ndom; ++d) {
        b->dom[d].first_tile = (int32_t)td.size();
        const int nt = (b->dom[d].n + block - 1) / block;
        for (int t = 0; t < nt; ++t) td.push_back(d);
    }
    b->ntiles = (int)td.size();
    b->block = block;
    // L2 prefetch distance: 3/4 of a wave of resident tiles (the launch
    // bounds ask for 32 warps per SM, so 1024 / block tiles per SM) where the
    // populations exceed twice the L2, or JLB_BATCH_PF tiles.  On the
    // 512-channel ensemble (14.5 GB): 37.2 GLUPS without, 40.6 / 41.1 / 41.0 /
    // 40.9 / 40.8 at 1/2, 3/4, 1, 5/4, 3/2 of a wave
    b->pf = b->pf_tiles >= 0 ? b->pf_tiles
                             : b->pf_big ? (int)std::lround(0.75 * b->sms * (1024.0 / block)) : 0;
    if (b->tile_dom) cudaFree(b->tile_dom);
    b->tile_dom = nullptr;
    BCK(cudaMalloc(&b->tile_dom, td.size() * sizeof(int32_t)));
    BCK(cudaMemcpyAsync(b->tile_dom, td.data(), td.size() * sizeof(int32_t), cudaMemcpyHostToDevice, b->st));
    BCK(cudaMemcpyAsync(b->d_dom, b->dom.data(), b->dom.size() * sizeof(BatchDomain), cudaMemcpyHostToDevice,
                        b->st));
    BCK(cudaStreamSynchronize(b->st));
    for (int p = 0; p < 2; ++p) {
        if (b->gexec[p]) cudaGraphExecDestroy(b->gexec[p]);
        b->gexec[p] = nullptr;
    }
    return JLB_OK;
}

int batch_launch(jlb_batch *b, bool pstep, int write_moments) {
    const BatchArgs a = batch_args(b, write_moments);
    int r = launch_batch_step(a, b->scheme, pstep, b->block, b->ntiles, b->st);
    if (r) return bfail(b, JLB_ERR_CUDA, std::string("batch step: ") + cudaGetErrorString((cudaError_t)r));
    ++b->launches;
    if (b->Msp > 0) {
        r = launch_batch_special(a, b->scheme, pstep, b->st);
        if (r) return bfail(b, JLB_ERR_CUDA, std::string("batch boundary nodes: ") + cudaGetErrorString((cudaError_t)r));
        ++b->launches;
    }
    return JLB_OK;
}

int batch_run(jlb_batch *b, uint32_t n, bool write_last) {
    uint32_t plain = write_last && n > 0 ? n - 1 : n;
    while (graphs_enabled() && plain >= (uint32_t)b->GK) {
        const int p = b->parity;
        if (!b->gexec[p]) {
            cudaGraph_t g;
            BCK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
            int par = p, rr = JLB_OK;
            for (int t = 0; t < b->GK && rr == JLB_OK; ++t) {
                rr = batch_launch(b, par == 0, 0);
                par ^= 1;
            }
            cudaError_t ce = cudaStreamEndCapture(b->st, &g);
            if (rr) return rr;
            if (ce != cudaSuccess) return bfail(b, JLB_ERR_CUDA, "batch graph capture failed");
            b->launches -= (uint64_t)b->GK * (1 + (b->Msp > 0));
            ce = cudaGraphInstantiate(&b->gexec[p], g, 0);
            cudaGraphDestroy(g);
            if (ce != cudaSuccess) return bfail(b, JLB_ERR_CUDA, "batch graph instantiate failed");
        }
        BCK(cudaGraphLaunch(b->gexec[p], b->st));
        b->launches += (uint64_t)b->GK * (1 + (b->Msp > 0));
        plain -= b->GK;
        if (b->GK & 1) b->parity ^= 1;
    }
    for (uint32_t t = 0; t < plain; ++t) {
        int r = batch_launch(b, b->parity == 0, 0);
        if (r) return r;
        b->parity ^= 1;
    }
    if (write_last && n > 0) {
        int r = batch_launch(b, b->parity == 0, 1);
        if (r) return r;
        b->parity ^= 1;
    }
    return JLB_OK;
}

// times 2 warm-up + 4 steps for each block size on the current state, then
// restores the state; keeps the fastest block size
int batch_autotune(jlb_batch *b) {
    const size_t fb = (size_t)19 * b->Np * sizeof(float), db = (size_t)b->Np * sizeof(float);
    float *fsave = nullptr, *dsave = nullptr;
    if (cudaMalloc(&fsave, fb) != cudaSuccess || cudaMalloc(&dsave, db) != cudaSuccess) {
        cudaGetLastError();
        if (fsave) cudaFree(fsave);
        return batch_tiles(b, 128); // no room for a scratch copy: keep the default
    }
    BCK(cudaMemcpyAsync(fsave, b->f, fb, cudaMemcpyDeviceToDevice, b->st));
    BCK(cudaMemcpyAsync(dsave, b->dprev, db, cudaMemcpyDeviceToDevice, b->st));
    std::vector<float> spsave((size_t)b->Msp);
    if (b->Msp > 0)
        BCK(cudaMemcpyAsync(spsave.data(), b->d_sp_den, spsave.size() * sizeof(float), cudaMemcpyDeviceToHost, b->st));
    const int cand[3] = {64, 128, 256};
    int best = 128;
    double best_ms = 1e30;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int c = 0; c < 3; ++c) {
        int r = batch_tiles(b, cand[c]);
        if (r) return r;
        for (int t = 0; t < 2; ++t) if ((r = batch_launch(b, t == 0, 0))) return r;
        cudaEventRecord(e0, b->st);
        for (int t = 0; t < 4; ++t) if ((r = batch_launch(b, t % 2 == 0, 0))) return r;
        cudaEventRecord(e1, b->st);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        b->tune_ms[c] = ms / 4.0;
        if (ms < best_ms) { best_ms = ms; best = cand[c]; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->launches -= 18 * (1 + (b->Msp > 0)); // tuning steps are not part of the run
    BCK(cudaMemcpyAsync(b->f, fsave, fb, cudaMemcpyDeviceToDevice, b->st));
    BCK(cudaMemcpyAsync(b->dprev, dsave, db, cudaMemcpyDeviceToDevice, b->st));
    if (b->Msp > 0)
        BCK(cudaMemcpyAsync(b->d_sp_den, spsave.data(), spsave.size() * sizeof(float), cudaMemcpyHostToDevice, b->st));
    BCK(cudaStreamSynchronize(b->st));
    cudaFree(fsave);
    cudaFree(dsave);
    return batch_tiles(b, best);
}

} // namespace

extern "C" {

void jlb_batch_destroy(jlb_batch *b) {
    if (!b) return;
    if (b->st) cudaStreamSynchronize(b->st);
    for (int p = 0; p < 2; ++p)
        if (b->gexec[p]) cudaGraphExecDestroy(b->gexec[p]);
    void *bufs[] = {b->f, b->dprev, b->mom[0], b->mom[1], b->mom[2], b->mom[3], b->ncls, b->nmask, b->mmask,
                    b->d_dom, b->tile_dom, b->d_sp_dom, b->d_sp_node, b->d_sp_rd, b->d_sp_wr, b->d_sp_info,
                    b->d_sp_lw, b->d_sp_bc, b->d_sp_den};
    for (void *p : bufs)
        if (p) cudaFree(p);
    if (b->own_stream && b->st) cudaStreamDestroy(b->st);
    delete b;
}

int jlb_batch_create(int32_t scheme, const jlb_domain *doms, int32_t ndom, void *stream, jlb_batch **out) {
    jlb_batch *b = nullptr;
    if (!out || !doms || ndom < 1) return bfail(nullptr, JLB_ERR_INVALID_ARG, "no domains");
    *out = nullptr;
    if (scheme < JLB_BGK || scheme > JLB_REGULARIZATION) return bfail(nullptr, JLB_ERR_INVALID_ARG, "Invalid relaxation scheme input.");
    b = new jlb_batch();
    b->scheme = scheme;
    b->ndom = ndom;
    auto bail = [&](int code) {
        std::string m = b->err;
        jlb_batch_destroy(b);
        bfail(nullptr, code, m);
        return code;
    };
    if (stream) b->st = (cudaStream_t)stream;
    else {
        if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess) {
            b->err = "cudaStreamCreate failed";
            return bail(JLB_ERR_CUDA);
        }
        b->own_stream = true;
    }
    // layout
    int64_t off = 0;
    b->dom.resize(ndom);
    for (int d = 0; d < ndom; ++d) {
        const jlb_domain &D = doms[d];
        jlb_config cfg{};
        for (int a = 0; a < 3; ++a) cfg.lat_size[a] = D.lat_size[a];
        cfg.rlx_scheme = scheme;
        cfg.kvisc = D.kvisc;
        for (int a = 0; a < 3; ++a) cfg.g[a] = D.g[a];
        for (int f = 0; f < 6; ++f) cfg.bc[f] = D.bc[f];
        cfg.precision = JLB_FP32;
        cfg.trt_magic = D.trt_magic;
        char msg[256];
        if (jlb_check_config(&cfg, msg, sizeof msg) != JLB_OK) {
            b->err = "domain " + std::to_string(d) + ": " + msg;
            return bail(JLB_ERR_INVALID_ARG);
        }

        if (!D.phase) { b->err = "domain " + std::to_string(d) + ": phase is NULL"; return bail(JLB_ERR_INVALID_ARG); }
        BatchDomain &B = b->dom[d];
        B.nx = D.lat_size[0]; B.ny = D.lat_size[1]; B.nz = D.lat_size[2];
        const int64_t n = (int64_t)B.nx * B.ny * B.nz;
        if (off + n >= 0x7fffff00LL) { b->err = "ensemble exceeds 2^31 sites"; return bail(JLB_ERR_UNSUPPORTED); }
        B.off = (int32_t)off;
        B.n = (int32_t)n;
        B.inv_syz = 1.0f / (float)(B.ny * B.nz);
        B.inv_nz = 1.0f / (float)B.nz;
        for (int f = 0; f < 6; ++f) B.bc[f] = D.bc[f];
        off += ((n + 127) / 128) * 128;
        const double tau_e = 0.5 + 3.0 * D.kvisc;
        const double we = 1.0 / tau_e;
        double wo = we;
        if (scheme == JLB_TRT)
            wo = D.trt_magic > 0.0 ? 1.0 / (D.trt_magic / (tau_e - 0.5) + 0.5) : 8.0 * (2.0 - we) / (8.0 - we);
        double wef, wof;
        float_exact_rates(scheme == JLB_TRT, we, wo, wef, wof);
        B.we = (float)wef; B.wo = (float)wof;
        for (int a = 0; a < 3; ++a) { B.g[a] = (float)D.g[a]; B.uw[a] = 0.0f; }
    }
    b->ntot = off;
    b->Np = off;
    auto alloc = [&](void **p, size_t bytes) {
        if (cudaMalloc(p, bytes) != cudaSuccess) {
            cudaGetLastError();
            b->err = "device allocation of " + std::to_string(bytes) + " bytes failed";
            return JLB_ERR_NOMEM;
        }
        return JLB_OK;
    };
    int r;
    if ((r = alloc((void **)&b->f, (size_t)19 * b->Np * sizeof(float)))) return bail(r);
    if ((r = alloc((void **)&b->dprev, (size_t)b->Np * sizeof(float)))) return bail(r);
    for (int c = 0; c < 4; ++c)
        if ((r = alloc((void **)&b->mom[c], (size_t)b->Np * sizeof(float)))) return bail(r);
    if ((r = alloc((void **)&b->ncls, (size_t)b->Np))) return bail(r);
    if ((r = alloc((void **)&b->nmask, (size_t)b->Np * sizeof(uint32_t)))) return bail(r);
    if ((r = alloc((void **)&b->mmask, (size_t)b->Np * sizeof(uint32_t)))) return bail(r);
    if ((r = alloc((void **)&b->d_dom, (size_t)ndom * sizeof(BatchDomain)))) return bail(r);
    cudaMemsetAsync(b->ncls, BCLS_SOLID, (size_t)b->Np, b->st);
    cudaMemsetAsync(b->dprev, 0, (size_t)b->Np * sizeof(float), b->st);
    // per domain: halo rules, masks and initial populations of a single-domain
    // FP32 solver, packed into the ensemble arrays
    std::vector<uint8_t> cls;
    std::vector<uint32_t> mm, lm;
    std::vector<float> dp;
    b->nfluid_dom.assign(ndom, 0);
    // boundary nodes of domains with Zou-He or symmetric faces, per node:
    // domain, packed node, info, 19 read / write elements, 19 c.u_wall, 2 x 4
    // Zou-He values, previous density
    std::vector<int32_t> g_dom;
    std::vector<int64_t> g_node;
    std::vector<uint32_t> g_info;
    std::vector<int64_t> g_rd, g_wr;   // node-major [t][19] until the upload
    std::vector<double> g_lw, g_bc;    // [t][19], [t][8]
    std::vector<float> g_den;
    b->sp_first.assign(ndom + 1, 0);
    for (int d = 0; d < ndom; ++d) {
        const jlb_domain &D = doms[d];
        BatchDomain &B = b->dom[d];
        jlb_config cfg{};
        for (int a = 0; a < 3; ++a) cfg.lat_size[a] = D.lat_size[a];
        cfg.rlx_scheme = scheme;
        cfg.kvisc = D.kvisc;
        for (int a = 0; a < 3; ++a) cfg.g[a] = D.g[a];
        for (int f = 0; f < 6; ++f) cfg.bc[f] = D.bc[f];
        cfg.precision = JLB_FP32;
        cfg.trt_magic = D.trt_magic;
        cfg.stream = b->st;
        jlb_solver *s = nullptr;
        if ((r = jlb_create(&cfg, &s))) { b->err = "domain " + std::to_string(d) + ": " + g_create_error; return bail(r); }
        const int NI = B.nx + 2, NJ = B.ny + 2, NK = B.nz + 2;
        const size_t ncnt = (size_t)NI * NJ * NK;
        std::vector<uint8_t> ph(ncnt, 0);
        std::vector<double> den(ncnt, 1.0), vel(3 * ncnt, 0.0);
        for (int i = 0; i < B.nx; ++i)
            for (int j = 0; j < B.ny; ++j)
                for (int k = 0; k < B.nz; ++k) {
                    const size_t li = ((size_t)i * B.ny + j) * B.nz + k;
                    const size_t fi = ((size_t)(i + 1) * NJ + (j + 1)) * NK + (k + 1);
                    ph[fi] = D.phase[li];
                    if (D.den) den[fi] = D.den[li];
                    if (D.vel) for (int a = 0; a < 3; ++a) vel[3 * fi + a] = D.vel[3 * li + a];
                }
        uint64_t nf = 0;
        r = jlb_finalize_init(s, ph.data(), den.data(), vel.data(), &nf);
        if (r) { b->err = "domain " + std::to_string(d) + ": " + s->err; jlb_destroy(s); return bail(r); }
        b->nfluid_dom[d] = (int32_t)nf;
        b->nfluid += (int64_t)nf;
        if (nf > 0) {
            r = launch_batch_pack((const float *)s->f, s->Np, B.n, b->f, b->Np, B.off, b->st);
            if (r) { b->err = "pack kernel failed"; jlb_destroy(s); return bail(JLB_ERR_CUDA); }
        }
        // boundary nodes of a domain with Zou-He or symmetric faces take the
        // table path (with their moving-wall links); the tables translate the
        // single-domain element indices q * Np_d + m into the packed array
        bool routed = false;
        for (int f = 0; f < 6; ++f)
            routed |= D.bc[f] == JLB_FIXED_DEN || D.bc[f] == JLB_FIXED_VEL || D.bc[f] == JLB_SYMMETRIC;
        // so do domains whose moving solids have more than one velocity (the
        // packed kernel's Ladd term takes one velocity per domain)
        if (!routed && D.vel) {
            const double *v0 = nullptr;
            for (int64_t l = 0; l < B.n && !routed; ++l) {
                if (D.phase[l] != 0) continue;
                const double *u = D.vel + 3 * l;
                if (u[0] == 0.0 && u[1] == 0.0 && u[2] == 0.0) continue;
                if (!v0) v0 = u;
                else routed = u[0] != v0[0] || u[1] != v0[1] || u[2] != v0[2];
            }
        }
        b->sp_first[d] = (int)g_node.size();
        if (routed && nf > 0 && s->M > 0) {
            const int M = s->M;
            std::vector<double> bcbuf((size_t)8 * M, 0.0);
            std::vector<float> denbuf((size_t)M, 0.0f);
            fill_dynamic(s, den.data(), vel.data(), bcbuf.data(), denbuf.data());
            const int64_t Npd = s->Np;
            auto tr = [&](int64_t e) { return (e / Npd) * b->Np + B.off + (e % Npd); };
            for (int t = 0; t < M; ++t) {
                g_dom.push_back(d);
                g_node.push_back(B.off + s->sp_node[t]);
                g_info.push_back(s->sp_info[t]);
                for (int q = 0; q < 19; ++q) {
                    g_rd.push_back(tr(s->sp_rd[(size_t)q * M + t]));
                    g_wr.push_back(tr(s->sp_wr[(size_t)q * M + t]));
                    g_lw.push_back(s->sp_lw[(size_t)q * M + t]);
                }
                for (int c = 0; c < 8; ++c) g_bc.push_back(c < 4 * s->bc_slots ? bcbuf[(size_t)c * M + t] : 0.0);
                g_den.push_back(denbuf[t]);
            }
        }
        b->sp_first[d + 1] = (int)g_node.size();
        // node classes and masks; the moving solids of a domain share one velocity
        cls.assign(B.n, BCLS_SOLID);
        lm.assign(B.n, 0);
        mm.assign(B.n, 0);
        dp.assign(B.n, 0.0f);
        bool have_uw = false;
        double uw[3] = {0, 0, 0};
        for (int64_t l = 0; l < B.n && nf > 0; ++l) {
            const uint32_t m = s->hmask[l];
            if (m & MASK_SOLID) continue;
            const int i = (int)(l / ((int64_t)B.ny * B.nz)), j = (int)((l / B.nz) % B.ny), k = (int)(l % B.nz);
            if (routed && (m & MASK_SPECIAL)) {
                lm[l] = m & MASK_LINKS;
                cls[l] = BCLS_SPECIAL;
                continue;
            }
            uint32_t mv = 0;
            for (int q = 0; q < 19; ++q) {
                if (!(m & (1u << q))) continue;
                const size_t sp = ((size_t)(i + 1 - CI[q]) * NJ + (j + 1 - CJ[q])) * NK + (k + 1 - CK[q]);
                const double *u = vel.data() + 3 * sp;
                if (u[0] == 0.0 && u[1] == 0.0 && u[2] == 0.0) continue;
                if (!have_uw) { uw[0] = u[0]; uw[1] = u[1]; uw[2] = u[2]; have_uw = true; }
                else if (u[0] != uw[0] || u[1] != uw[1] || u[2] != uw[2]) {
                    b->err = "domain " + std::to_string(d) + ": moving solids of one batched domain must share one velocity";
                    jlb_destroy(s);
                    return bail(JLB_ERR_UNSUPPORTED);
                }
                mv |= 1u << q;
            }
            lm[l] = m & MASK_LINKS;
            mm[l] = mv;
            cls[l] = mv ? BCLS_MOVING : (m & MASK_LINKS) ? BCLS_WALL : BCLS_PLAIN;
            const size_t fi = ((size_t)(i + 1) * NJ + (j + 1)) * NK + (k + 1);
            dp[l] = (float)(den[fi] - 1.0);
        }
        for (int a = 0; a < 3; ++a) B.uw[a] = (float)uw[a];
        cudaError_t e1 = cudaMemcpyAsync(b->ncls + B.off, cls.data(), B.n, cudaMemcpyHostToDevice, b->st);
        cudaError_t e2 = cudaMemcpyAsync(b->nmask + B.off, lm.data(), (size_t)B.n * 4, cudaMemcpyHostToDevice, b->st);
        cudaError_t e3 = cudaMemcpyAsync(b->mmask + B.off, mm.data(), (size_t)B.n * 4, cudaMemcpyHostToDevice, b->st);
        cudaError_t e4 = cudaMemcpyAsync(b->dprev + B.off, dp.data(), (size_t)B.n * 4, cudaMemcpyHostToDevice, b->st);
        cudaError_t e5 = cudaStreamSynchronize(b->st); // host vectors are reused next domain
        jlb_destroy(s);
        if (e1 || e2 || e3 || e4 || e5) { b->err = "domain upload failed"; return bail(JLB_ERR_CUDA); }
    }
    b->Msp = (int)g_node.size();
    b->h_sp_node = g_node;
    b->h_sp_info = g_info;
    if (b->Msp > 0) {
        const int M = b->Msp;
        // node-major [t][19] -> [19][M] as the boundary-node path reads them
        std::vector<int64_t> rd((size_t)19 * M), wr((size_t)19 * M);
        std::vector<double> lw((size_t)19 * M), bcd((size_t)8 * M);
        for (int t = 0; t < M; ++t) {
            for (int q = 0; q < 19; ++q) {
                rd[(size_t)q * M + t] = g_rd[(size_t)t * 19 + q];
                wr[(size_t)q * M + t] = g_wr[(size_t)t * 19 + q];
                lw[(size_t)q * M + t] = g_lw[(size_t)t * 19 + q];
            }
            for (int c = 0; c < 8; ++c) bcd[(size_t)c * M + t] = g_bc[(size_t)t * 8 + c];
        }
        if ((r = alloc((void **)&b->d_sp_dom, (size_t)M * 4)) || (r = alloc((void **)&b->d_sp_node, (size_t)M * 8)) ||
            (r = alloc((void **)&b->d_sp_info, (size_t)M * 4)) || (r = alloc((void **)&b->d_sp_rd, rd.size() * 8)) ||
            (r = alloc((void **)&b->d_sp_wr, wr.size() * 8)) || (r = alloc((void **)&b->d_sp_lw, lw.size() * 8)) ||
            (r = alloc((void **)&b->d_sp_bc, bcd.size() * 8)) || (r = alloc((void **)&b->d_sp_den, (size_t)M * 4)))
            return bail(r);
        cudaError_t e = cudaSuccess;
        auto up = [&](void *dst, const void *src, size_t n) {
            if (e == cudaSuccess) e = cudaMemcpy(dst, src, n, cudaMemcpyHostToDevice);
        };
        up(b->d_sp_dom, g_dom.data(), (size_t)M * 4);
        up(b->d_sp_node, g_node.data(), (size_t)M * 8);
        up(b->d_sp_info, g_info.data(), (size_t)M * 4);
        up(b->d_sp_rd, rd.data(), rd.size() * 8);
        up(b->d_sp_wr, wr.data(), wr.size() * 8);
        up(b->d_sp_lw, lw.data(), lw.size() * 8);
        up(b->d_sp_bc, bcd.data(), bcd.size() * 8);
        up(b->d_sp_den, g_den.data(), (size_t)M * 4);
        if (e != cudaSuccess) { b->err = "boundary-node table upload failed"; return bail(JLB_ERR_CUDA); }
    }
    {
        int dev = 0, l2 = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev) != cudaSuccess) {
            cudaGetLastError();
            b->sms = 0;
            l2 = 0;
        }
        b->pf_big = 19.0 * (double)b->Np * sizeof(float) > 2.0 * (double)l2;
        const char *e = std::getenv("JLB_BATCH_PF");
        if (e && e[0]) b->pf_tiles = std::max(0, std::atoi(e));
    }
    const char *tune = std::getenv("JLB_BATCH_BLOCK");
    if (tune && tune[0]) r = batch_tiles(b, std::atoi(tune));
    else r = batch_autotune(b);
    if (r) return bail(r);
    *out = b;
    return JLB_OK;
}

int jlb_batch_step(jlb_batch *b, uint32_t tsteps) {
    if (!b) return bfail(b, JLB_ERR_INVALID_ARG, "NULL batch");
    int r = batch_run(b, tsteps, true);
    if (r) return r;
    b->tot += tsteps;
    return JLB_OK;
}

int jlb_batch_set_bc(jlb_batch *b, int32_t d, const double *den, const double *vel) {
    if (!b || d < 0 || d >= b->ndom) return bfail(b, JLB_ERR_INVALID_ARG, "bad argument");
    if (!den && !vel) return JLB_OK;
    const BatchDomain &B = b->dom[d];
    const int t0 = b->sp_first[d], t1 = b->sp_first[d + 1], Md = t1 - t0, M = b->Msp;
    // Zou-He data, slot by slot in face order as at creation: the fixed faces
    // read den / vel at the node; Z1 only when bc[Z1] is FIXED_DEN or bc[1Z]
    // is FIXED_VEL (jyulb/isothermal.pyx:500), else den 1, vel 0
    if (Md > 0) {
        std::vector<double> bcd((size_t)8 * Md, 0.0);
        std::vector<float> dp(Md, 0.0f);
        for (int c = 0; c < 8; ++c)
            BCK(cudaMemcpyAsync(bcd.data() + (size_t)c * Md, b->d_sp_bc + (size_t)c * M + t0, (size_t)Md * 8,
                                cudaMemcpyDeviceToHost, b->st));
        BCK(cudaStreamSynchronize(b->st));
        for (int u = 0; u < Md; ++u) {
            const int64_t l = b->h_sp_node[t0 + u] - B.off;
            const uint32_t faces = (b->h_sp_info[t0 + u] >> SP_FACE_SHIFT) & 0x3Fu;
            int slot = 0;
            for (int face = 0; face < 6; ++face) {
                if (!(faces & (1u << face))) continue;
                bool refresh = B.bc[face] == BC_FIXED_DEN || B.bc[face] == BC_FIXED_VEL;
                if (face == 5) refresh = B.bc[5] == BC_FIXED_DEN || B.bc[4] == BC_FIXED_VEL;
                double *row = bcd.data() + (size_t)(4 * slot) * Md + u;
                if (refresh) {
                    if (den) row[0] = den[l];
                    if (vel) for (int c = 0; c < 3; ++c) row[(size_t)(1 + c) * Md] = vel[3 * l + c];
                }
                slot = 1;
            }
            if (den) dp[u] = (float)(den[l] - 1.0);
        }
        for (int c = 0; c < 8; ++c)
            BCK(cudaMemcpyAsync(b->d_sp_bc + (size_t)c * M + t0, bcd.data() + (size_t)c * Md, (size_t)Md * 8,
                                cudaMemcpyHostToDevice, b->st));
        if (den) BCK(cudaMemcpyAsync(b->d_sp_den + t0, dp.data(), (size_t)Md * 4, cudaMemcpyHostToDevice, b->st));
        BCK(cudaStreamSynchronize(b->st));
    }
    // previous-step density of the dense moving-wall nodes
    if (den) {
        std::vector<float> dp((size_t)B.n);
        BCK(cudaMemcpyAsync(dp.data(), b->dprev + B.off, (size_t)B.n * 4, cudaMemcpyDeviceToHost, b->st));
        std::vector<uint8_t> cl(B.n);
        BCK(cudaMemcpyAsync(cl.data(), b->ncls + B.off, B.n, cudaMemcpyDeviceToHost, b->st));
        BCK(cudaStreamSynchronize(b->st));
        for (int32_t l = 0; l < B.n; ++l)
            if (cl[l] != BCLS_SOLID) dp[l] = (float)(den[l] - 1.0);
        BCK(cudaMemcpyAsync(b->dprev + B.off, dp.data(), (size_t)B.n * 4, cudaMemcpyHostToDevice, b->st));
        BCK(cudaStreamSynchronize(b->st));
    }
    return JLB_OK;
}

int jlb_batch_moments(jlb_batch *b, int32_t d, double *den, double *vel) {
    if (!b || d < 0 || d >= b->ndom || !den || !vel) return bfail(b, JLB_ERR_INVALID_ARG, "bad argument");
    const BatchDomain &B = b->dom[d];
    std::vector<float> h((size_t)4 * B.n);
    for (int c = 0; c < 4; ++c)
        BCK(cudaMemcpyAsync(h.data() + (size_t)c * B.n, b->mom[c] + B.off, (size_t)B.n * 4, cudaMemcpyDeviceToHost,
                            b->st));
    std::vector<uint8_t> cl(B.n);
    BCK(cudaMemcpyAsync(cl.data(), b->ncls + B.off, B.n, cudaMemcpyDeviceToHost, b->st));
    BCK(cudaStreamSynchronize(b->st));
    for (int32_t l = 0; l < B.n; ++l) {
        if (cl[l] == BCLS_SOLID) continue; // solid sites keep the caller's values
        den[l] = 1.0 + (double)h[l];
        for (int a = 0; a < 3; ++a) vel[3 * (size_t)l + a] = (double)h[(size_t)(a + 1) * B.n + l];
    }
    return JLB_OK;
}

int jlb_batch_populations(jlb_batch *b, int32_t d, double *f) {
    if (!b || d < 0 || d >= b->ndom || !f) return bfail(b, JLB_ERR_INVALID_ARG, "bad argument");
    const BatchDomain &B = b->dom[d];
    double *tmp = nullptr;
    BCK(cudaMalloc(&tmp, (size_t)19 * B.n * sizeof(double)));
    int r = launch_batch_readout(batch_args(b, 0), d, B.n, b->parity, b->sp_first[d], b->sp_first[d + 1], tmp,
                                 b->st);
    cudaError_t e = r ? (cudaError_t)r
                      : cudaMemcpyAsync(f, tmp, (size_t)19 * B.n * sizeof(double), cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    cudaFree(tmp);
    BCK(e);
    return JLB_OK;
}

int jlb_batch_info(const jlb_batch *b, int64_t out[8]) {
    if (!b || !out) return JLB_ERR_INVALID_ARG;
    out[0] = b->ntot;
    out[1] = b->nfluid;
    out[2] = b->block;
    out[3] = b->ntiles;
    out[4] = (int64_t)b->launches;
    out[5] = (int64_t)(b->tune_ms[0] * 1e3);
    out[6] = (int64_t)(b->tune_ms[1] * 1e3);
    out[7] = (int64_t)(b->tune_ms[2] * 1e3);
    return JLB_OK;
}

int32_t jlb_batch_domain_fluid(const jlb_batch *b, int32_t d) {
    return (b && d >= 0 && d < b->ndom) ? b->nfluid_dom[d] : -1;
}

const char *jlb_batch_last_error(const jlb_batch *b) { return b ? b->err.c_str() : g_create_error.c_str(); }

} // extern "C"
