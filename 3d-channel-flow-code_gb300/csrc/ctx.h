// Library context: device-resident state of one solver instance.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <string>
#include <vector>

#include "dev.cuh"
#include "layout.h"

struct nsmp_ctx {
    nsmp_params prm{};
    nsmp::HostLayout L;
    nsmp::Mesh mesh{};
    cudaStream_t stream = nullptr;
    int device = 0;
    int num_sms = 0;
    std::string err;

    // device tables
    nsmp::ColPPE* d_ppe = nullptr;
    nsmp::ColGeo* d_geo = nullptr;
    int *d_vptr = nullptr, *d_vcell = nullptr;
    double *d_vcoef = nullptr, *d_lev = nullptr;
    int *d_gather = nullptr;      // (N_CELL) -> column, for downloads/uploads
    int *d_vgather = nullptr;     // (N_VERT) -> vertex class

    // state: three buffers per cell field, indexed by time level
    double* lvl[3][4] = {};       // [buffer][u,v,w,p]
    int ln = 0, lknown = 0, lnp = 1;
    double* face[5] = {};         // U1FACE..UBFACE
    double* hist[3] = {};         // rhsuf, rhsvf, rhswf
    double* eddy = nullptr;
    double* ustar[3] = {};
    double* rhsp = nullptr;
    double* vtx[4] = {};          // vertex u, v, w, p (tagdir 2, interior layers)
    // Krylov work vectors
    double *x = nullptr, *r = nullptr, *r0 = nullptr, *pk = nullptr, *vk = nullptr, *sk = nullptr,
           *tk = nullptr, *invD = nullptr;
    double* ahat[5] = {};         // Jacobi-scaled PPE couplings (A D^-1 off-diagonals)
    // mixed precision (NSMP_MIXED): FP64 refinement vectors + FP32 inner Krylov vectors
    double *b64 = nullptr, *xa = nullptr, *xb = nullptr;
    float *r32 = nullptr, *r032 = nullptr, *p32[2] = {}, *v32[2] = {}, *s32 = nullptr, *t32 = nullptr,
          *e32 = nullptr, *invD32 = nullptr, *lev32 = nullptr;
    // double-float (hi, lo) copies of the PPE coefficients for the FP64
    // hand-over: per column {kA1..3, area}, per level {dsigv, aT, aB, 0}
    float *ddcol = nullptr, *ddlev = nullptr;
    nsmp::ColPPE32* d_ppe32 = nullptr;
    nsmp::ColGeo32* d_geo32 = nullptr;  // FP32 stage tables (NSMP_MIXED_F32)
    int stage32 = 0;              // 1: stage right-hand side in FP32 arithmetic
    int fp64_spmv_mf = 0;         // 1: FP64 BiCGSTAB regenerates its couplings instead of reading them
    int l2_limit_set = 0;         // 1: this context raised the persisting-L2 limit (restored by the last such context)
    double inner_tol = 3e-2;      // FP32 residual reduction that triggers an FP64 update
    int inner_cap = 80;           // most FP32 iterations between two FP64 updates
    int restart_every = 300;      // most FP32 iterations of one Krylov process
    int last_outer = 0;
    double* stage_buf = nullptr;  // (N_CELL,NZ) staging for transfers
    double* fx = nullptr;         // body force on u (cell layout), null when unset
    // pressure tape of the adjoint: when tape_x is set a stage copies its
    // PPE solution there; when replay_x is set a stage uses that solution
    // instead of solving (recomputation of a checkpointed segment)
    double* tape_x = nullptr;
    const double* replay_x = nullptr;
    struct AdjScratch* adj = nullptr;  // discrete-adjoint work buffers (lazily allocated)
    struct StatState* stats = nullptr; // turbulence-statistics sums (lazily allocated)
    // reductions and scalars
    nsmp::RedScratch red{}, red2{};
    nsmp::Scal* d_scal = nullptr;
    nsmp::Scal* h_scal = nullptr;  // pinned
    int flag_ab = 0;
    int last_iters = 16;
    int precision = NSMP_FP64;
    nsmp_stage_info last{};
    std::vector<void*> allocs;
    // launch accounting and optional per-kernel event timing
    long long launches = 0;
    long long bicg_iters = 0;
    long long fp64_updates = 0;   // NSMP_MIXED: FP64 hand-overs (refinements) executed since creation
    int prof_on = 0;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    std::vector<std::pair<int, int>> ev_pending;  // (kernel id, first event index)
    std::map<const void*, int> occ_cache;  // kernel -> resident blocks per SM
    long long prof_count[NSMP_K_COUNT] = {};
    double prof_ms[NSMP_K_COUNT] = {};
};

namespace nsmp {

int ctx_init_device(nsmp_ctx* c);
void ctx_free(nsmp_ctx* c);
int run_stage(nsmp_ctx* c, int fin_rk, nsmp_stage_info* info);
int run_user_initial(nsmp_ctx* c);
int run_fill_ghosts(nsmp_ctx* c, int buf);
int run_combine(nsmp_ctx* c, double a, double b);
int run_gather(nsmp_ctx* c, const double* dfield, int ghost_mode, int rows, double* host);
int run_scatter(nsmp_ctx* c, const double* host, double* dfield, int rows = 0, bool sync = true);
int run_mass_diag(nsmp_ctx* c, double out[4]);
int run_cfl_diag(nsmp_ctx* c, double out[NSMP_CFL_COUNT]);
int run_mass_diag_noalloc(nsmp_ctx* c, double out[4]);
int run_download_pv(nsmp_ctx* c, double* host);
int cuda_fail(nsmp_ctx* c, cudaError_t e, const char* where);
int mixed_alloc(nsmp_ctx* c);
int stage32_alloc(nsmp_ctx* c);
int fp64_setup(nsmp_ctx* c);
// FP64 pressure solve of one stage; on return *x_final points at the solution
// (compact layout, before the Glob_Norm mean removal).
int run_pressure_fp64(nsmp_ctx* c, const double* pf, const double** x_final);
// Pressure solve of one stage in mixed precision; on return *x_final points
// at the FP64 solution (before the Glob_Norm mean removal).
int run_pressure_mixed(nsmp_ctx* c, const double* pf, const double** x_final);
int run_adjoint(nsmp_ctx* c, int nsteps, int ckpt_every, const double* fx, double* grad, double* J);
int run_apply_A(nsmp_ctx* c, int transpose, const double* x, double* y);
int run_set_body_force(nsmp_ctx* c, const double* fx);
int run_wall_shear(nsmp_ctx* c, double* tau);
void adj_free(nsmp_ctx* c);
void l2_limit_release(nsmp_ctx* c);
void stats_free(nsmp_ctx* c);
int adj_ensure(nsmp_ctx* c);
int prof_begin(nsmp_ctx* c, int kid);   // returns event slot or -1
void prof_end(nsmp_ctx* c, int slot);
int prof_resolve(nsmp_ctx* c);

// Makes the context's device current for the duration of an entry point and
// gives the caller's current device back on return, so contexts on several
// devices can be driven from one host thread.
struct DeviceGuard {
    int prev = -1;
    int dev = 0;
    cudaError_t err = cudaSuccess;
    explicit DeviceGuard(int d) : dev(d) {
        if (cudaGetDevice(&prev) != cudaSuccess) {
            prev = -1;
            cudaGetLastError();
        }
        if (prev != dev) {
            err = cudaSetDevice(dev);
            if (err != cudaSuccess) cudaGetLastError();
        }
    }
    ~DeviceGuard() {
        if (prev >= 0 && prev != dev && cudaSetDevice(prev) != cudaSuccess) cudaGetLastError();
    }
    DeviceGuard(const DeviceGuard&) = delete;
    DeviceGuard& operator=(const DeviceGuard&) = delete;
};

}  // namespace nsmp

#define NSMP_DEVICE_GUARD(ctx)                                                    \
    nsmp::DeviceGuard nsmp_guard_((ctx)->device);                                 \
    if (nsmp_guard_.err != cudaSuccess) return nsmp::cuda_fail((ctx), nsmp_guard_.err, "cudaSetDevice")
