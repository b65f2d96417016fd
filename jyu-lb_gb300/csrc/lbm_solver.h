// lbm_solver.h -- state of one single-domain solver and the host helpers
// that the ensemble (lbm_batch_host.cpp) and adjoint (lbm_adjoint_host.cpp)
// host units share with the single-domain runtime (lbm_host.cpp).  Internal
// to the library: not part of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <stdint.h>
#include <string>
#include <vector>

#include "jyulb_gb300.h"
#include "lbm_aux.h"
#include "lbm_common.h"


struct jlb_solver {
    jlb_config cfg{};
    int nx = 0, ny = 0, nz = 0, NI = 0, NJ = 0, NK = 0;
    int64_t N = 0, Np = 0, NCNT = 0;
    int prec = 0;
    bool fast64 = false;  // JLB_FP64_FAST: FP64 state, the contracted step kernel
    size_t ssz = 8, csz = 8;  // storage / compute element sizes
    double we = 0, wo = 0;
    double tau = 0;       // relaxation time of the C++-executable model
    jlb::AuxGeom geom{};
    cudaStream_t st = nullptr;
    bool own_stream = false;

    // device state
    void *f = nullptr;
    uint32_t *nmask = nullptr;
    uint8_t *ncls = nullptr;
    void *mom[4] = {nullptr, nullptr, nullptr, nullptr};
    void *acc = nullptr;
    double *red_partial = nullptr, *red_out = nullptr;
    int red_blocks = 0;
    double *fi_partial = nullptr, *fi_out = nullptr; // flow information (allocated on first use)
    void *res_prev = nullptr;        // velocity at the last residual call (3 * Np, compute type)
    double *stg_den = nullptr, *stg_vel = nullptr;   // device copies of the host den/vel layout (DMA download)
    bool stg_failed = false;
    cudaStream_t st2 = nullptr;          // download stream of the overlapped last step
    // fluid-only population layout (lattices with many solid sites)
    bool sparse = false;                 // chosen at finalize_init
    bool no_sparse = false;              // the adjoint driver keeps the lattice layout
    bool no_lin = false;                 // and the row-block mapping of its reverse kernel
    bool c_current = false;              // the fluid-only copy holds the current state
    bool sp_tables_dirty = true;         // boundary tables changed since their translation
    void *fc = nullptr;                  // [19][Npc] populations of the fluid sites
    int32_t *d_csite = nullptr, *d_cidx = nullptr;
    int64_t *d_sp_rd_c = nullptr, *d_sp_wr_c = nullptr, *d_sp_cnode = nullptr;
    int sp_c_cap = 0;
    int64_t Nc = 0, Npc = 0;
    std::vector<cudaEvent_t> slab_ev;    // its slab events
    // boundary-node tables (device)
    int M = 0, Mcap = 0;
    int64_t *d_sp_node = nullptr, *d_sp_rd = nullptr, *d_sp_wr = nullptr;
    uint32_t *d_sp_info = nullptr;
    double *d_sp_lw = nullptr, *d_sp_bc = nullptr;
    void *d_sp_den = nullptr;

    // host bookkeeping
    std::vector<uint8_t> phase;      // halo-padded snapshot after the halo rules
    std::vector<uint32_t> hmask;     // Np entries
    std::vector<uint8_t> hcls;       // Np node classes derived from hmask
    std::vector<int64_t> wall_pos;   // solid positions next to fluid (halo-padded index)
    std::vector<double> wall_vel;    // their velocities at the last classification
    // the reference's bc_data_den_face_* / bc_data_vel_face_* arrays: the
    // face layers of den / vel as the last evolve call read them (empty:
    // never refreshed, den = 1 and vel = 0)
    std::vector<double> bcd_den[6], bcd_vel[6];
    std::vector<int64_t> wall_chk;   // indices into wall_pos re-read at every evolve call
    bool static_halo = false;        // halo cells of closed faces are not written by the caller
    int64_t *d_wall_pos = nullptr;   // device copies of the checked wall_pos / wall_vel
    double *d_wall_vel = nullptr;
    bool wall_dev_dirty = true;      // wall_pos / wall_vel changed since their upload
    int *wall_flag = nullptr;        // mapped host int set by the check kernel
    std::vector<int64_t> sp_node;
    std::vector<uint32_t> sp_info;
    std::vector<int64_t> sp_rd, sp_wr;
    std::vector<double> sp_lw;
    int bc_slots = 0;                // Zou-He data sets per boundary node
    void *pinned = nullptr;          // staging for per-call uploads
    size_t pinned_bytes = 0;

    uint64_t nfluid = 0;
    bool init_done = false;
    uint32_t tot = 0;
    int parity = 0;                  // 0: next step is P, 1: next step is L
    bool accf = false;
    double g[3] = {0, 0, 0};
    uint64_t launches = 0;
    uint64_t h2d_bytes = 0, d2h_bytes = 0; // host<->device traffic issued by the runtime
    double host_t[6] = {0, 0, 0, 0, 0, 0};  // cumulative seconds per jlb_evolve phase
    std::string err;

    // graphs of GK consecutive steps without moment output, one per parity
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    int GK = 32;
    // bulk-copy staged step (FP32/FP16 on aligned, mostly fluid domains)
    bool use_tma = false;
    bool tma_p = true; // also for the pull-push step
    int tma_grid = 0;
    bool use_h2 = false;  // FP16: staged local step with two sites per thread
    int h2_grid = 0;
    int *d_err = nullptr; // set by a kernel whose bounded wait timed out
    int pf_blocks = 0;    // L2 prefetch distance of the direct step kernel (dense blocks)
    uint64_t args_version = 1, graph_version[2] = {0, 0};
};

namespace jlb_host {

// lattice vectors (reference order, jyulb/D3Q19.pxd:59-79)
extern const int CI[19], CJ[19], CK[19];
// message of the last failed create call (jlb_last_error(NULL) and friends)
extern thread_local std::string g_create_error;

// records msg on s (or as the create error when s is NULL); returns code
int fail(jlb_solver *s, int code, const std::string &msg);

// index of halo-padded site (I, J, K) in the host arrays
inline int64_t fidx(const jlb_solver *s, int I, int J, int K) {
    return ((int64_t)I * s->NJ + J) * s->NK + K;
}

// per-call Zou-He data (bc_slots x 4 doubles per boundary node, slot-major)
// and previous-step density of the boundary nodes, from host den/vel
void fill_dynamic(jlb_solver *s, const double *den, const double *vel, double *bcbuf, void *denbuf);

// CUDA graphs of the step loop are on unless JLB_NO_GRAPH is set
bool graphs_enabled();

// kernel arguments of the solver's current state
jlb::StepArgs make_args(const jlb_solver *s, int write_moments);

// runs n steps on the solver's stream; the last writes moments if write_last
int run_steps(jlb_solver *s, uint32_t n, bool write_last);

} // namespace jlb_host
