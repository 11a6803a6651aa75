/*
 * nsmp3D GB300 library -- C-ABI for the per-time-step hot path.
 *
 * Drop-in for the Fortran driver of techi28/3D-channel-flow-code: the driver
 * keeps its setup, I/O and statistics and calls these entry points (through
 * an ISO_C_BINDING interface block) where it used to call `hydro` and copy
 * time levels.  Fields stay resident on one GPU between calls.
 *
 * Conventions (those of the reference's Fortran arrays):
 *   - every array argument is a plain host pointer, column-major, with the
 *     reference's shapes: cell fields (N_CELL,NZ), face fluxes (N0,NZ),
 *     vertex fields (N_VERT,NZ-1), mesh tables (N0,3);
 *   - index values inside No_vp/No_cp are 1-based, No_cp = 0 marks a lateral
 *     boundary edge (data.txt convention, Main/input.F90:150-196);
 *   - N_CELL = N0 + number of ghost cells (one per lateral boundary edge),
 *     query it with nsmp_ncell after nsmp_create.
 * Every entry point returns an int status: 0 ok, > 0 warning (e.g. BiCGSTAB
 * hit MaxIters), < 0 error.  No host exception crosses the ABI; the text of
 * the last error is available from nsmp_last_error.  A context is used from
 * one host thread at a time and owns one CUDA stream.
 */
#ifndef NSMP_H
#define NSMP_H
#ifdef __cplusplus
extern "C" {
#endif

#define NSMP_OK 0
#define NSMP_WARN_MAXITER 1      /* BiCGSTAB stopped at MaxIters (bicgstab.F90:562-566) */
#define NSMP_WARN_BREAKDOWN 2    /* |rho|,|omega| or |r0.v| < 1e-30 (bicgstab.F90:479-517) */
#define NSMP_ERR_ARG -1          /* bad argument                                        */
#define NSMP_ERR_MESH -2         /* malformed mesh / periodic pairing failed            */
#define NSMP_ERR_CUDA -3         /* CUDA runtime error                                  */
#define NSMP_ERR_NAN -4          /* non-finite residual detected                        */
#define NSMP_ERR_UNSUPPORTED -5  /* configuration outside the supported key set         */
#define NSMP_ERR_NOMEM -6        /* device allocation failed                            */
#define NSMP_ERR_RANGE -7        /* size beyond a documented limit                      */

#define NSMP_FP64 0              /* plain form: FP64 throughout                         */
#define NSMP_MIXED 1             /* FP32 stencils/Krylov + FP64 iterative refinement    */
#define NSMP_MIXED_F32 2         /* NSMP_MIXED + the stage right-hand side (fluxes,
                                    gradients, Smagorinsky, diffusion) in FP32; the
                                    state, predictor update and AB2 history stay FP64 */

/* Runtime parameters: dataParameters.txt (input_parameters.F90:240-442) and
 * the compile-time constants of common.mpf:59-113 that the path reads. */
typedef struct nsmp_params {
    int n0;            /* N_CELL0: interior triangles                          */
    int nvert;         /* N_VERT                                                */
    int nz;            /* NZglobal = layers + 2                                 */
    double xdini, xdfin, ydini, ydfin; /* lateral box (common.mpf:66-69)      */
    double sigini, sigfin;             /* vertical range (common.mpf:64-65)   */
    int grid_kind;     /* 0 uniform sigma (calcul_geometry.F90:263-283), 1 tanh */
    double grid_beta;  /* tanh clustering factor (grid_kind = 1)                */
    int top_bc;        /* TopBC: 0 no-slip, 1 free-slip                         */
    int bot_bc;        /* BotBC: 0 no-slip, 1 free-slip                         */
    double dt, re, bdx, bdy, bdz;
    double eps;        /* BiCGSTAB tolerance                                    */
    int max_iters;     /* BiCGSTAB iteration cap                                */
    int les;           /* 1: Smagorinsky (KeyLES, Iturbu = 1)                   */
    int les_van;       /* 1: van Driest damping (KeyLESVan), 0: Mason           */
    int ref_bug_compat;/* 1: reproduce the reference's arithmetic quirks        */
    int precision;     /* NSMP_FP64, NSMP_MIXED or NSMP_MIXED_F32               */
    int device;        /* CUDA device ordinal                                   */
} nsmp_params;

/* Mesh as read from data.txt (the caller keeps ownership; nothing is
 * retained after nsmp_create returns). */
typedef struct nsmp_mesh {
    const int* No_vp;  /* (N0,3) vertex numbers, counter-clockwise             */
    const int* No_cp;  /* (N0,3) neighbour across edge j (v_j -> v_j+1), 0 = bd */
    const int* nbe;    /* (N0) cell tag, != 0 for cells touching the boundary  */
    const int* nbev;   /* (N_VERT) vertex tag, != 0 on the boundary            */
    const double* xv;  /* (N_VERT)                                             */
    const double* yv;  /* (N_VERT)                                             */
} nsmp_mesh;

typedef struct nsmp_stage_info {
    int iters;         /* BiCGSTAB iterations                                   */
    double e1norm;     /* final relative L1 residual                            */
    double e2norm;     /* final relative L2 residual                            */
    int converged;     /* 1 if min(e1norm, e2norm) < eps                        */
    double max_eddy;   /* max nu_t (0 without LES)                              */
    int status;        /* status of the stage                                   */
    int refinements;   /* NSMP_MIXED: FP64 refinement cycles (0 in NSMP_FP64)   */
} nsmp_stage_info;

typedef struct nsmp_ctx nsmp_ctx;

/* Field ids for nsmp_download / nsmp_upload_field. */
enum {
    NSMP_F_U = 0, NSMP_F_V, NSMP_F_W, NSMP_F_P,        /* level n, (N_CELL,NZ)    */
    NSMP_F_U1FACE, NSMP_F_U2FACE, NSMP_F_U3FACE,       /* (N0,NZ)                 */
    NSMP_F_UTFACE, NSMP_F_UBFACE,
    NSMP_F_RHSU, NSMP_F_RHSV, NSMP_F_RHSW,             /* AB2 history (N_CELL,NZ) */
    NSMP_F_EDDY,                                       /* nu_t (N_CELL,NZ)        */
    NSMP_F_UNP, NSMP_F_VNP, NSMP_F_WNP, NSMP_F_PNP,    /* level n+1 (N_CELL,NZ)   */
    NSMP_F_PV,                                         /* pfv after the stage, (N_VERT,NZ-1) */
    NSMP_NFIELDS
};

/* ---- setup: replaces nsmp3D.F90:232-249 device-side ------------------- */

/* Builds the geometry (calcul_geometry, adjust_bc, PDE_center restated),
 * renumbers columns (reverse Cuthill-McKee) and uploads everything.  The
 * floating-point geometry is computed on the context's device (the same bits
 * as the host restatement of nsmp_geometry), the integer topology on the
 * host. */
int nsmp_create(const nsmp_params* prm, const nsmp_mesh* mesh, nsmp_ctx** out);
int nsmp_destroy(nsmp_ctx* ctx);
const char* nsmp_last_error(const nsmp_ctx* ctx);
/* N_CELL = N0 + ghosts, for sizing (N_CELL,NZ) host arrays. */
int nsmp_ncell(const nsmp_ctx* ctx, int* n_cell);

/* ---- state ------------------------------------------------------------ */

/* user_initial.F90:166-238: level-n cell values in, ghosts filled, face
 * fluxes from interpolateU, AB2 history zeroed, flag_ab = 0. */
int nsmp_user_initial(nsmp_ctx* ctx, const double* u, const double* v,
                      const double* w, const double* p);
/* Full state upload (restart): cell fields (N_CELL,NZ) at level n, face
 * fluxes (N0,NZ), AB2 history (N_CELL,NZ). */
int nsmp_upload_state(nsmp_ctx* ctx, const double* u, const double* v,
                      const double* w, const double* p, const double* u1f,
                      const double* u2f, const double* u3f, const double* utf,
                      const double* ubf, const double* rhsu, const double* rhsv,
                      const double* rhsw, int flag_ab);
int nsmp_download(nsmp_ctx* ctx, int field, double* host);
/* Optional: page-lock (cudaHostRegister, portable) a host array that the
 * driver passes to the uploads and downloads above, so their copies run as
 * direct DMA instead of through the CUDA driver's pageable staging buffer;
 * nsmp_host_unregister undoes it before the array is deallocated.  Both are
 * host-memory bookkeeping only: results are the same either way.  Uploads
 * return after their copies have completed and downloads after the data has
 * arrived, so registered or not, an array may be reused at once. */
int nsmp_host_register(nsmp_ctx* ctx, void* host, size_t bytes);
int nsmp_host_unregister(nsmp_ctx* ctx, void* host);

/* ---- time loop: nsmp3D.F90:394-564 ------------------------------------ */

int nsmp_copy_known_from_n(nsmp_ctx* ctx);   /* nsmp3D.F90:419-441 */
/* One hydro() stage (Main/hydro.F90:8-501).  *flag_ab in/out. */
int nsmp_hydro_stage(nsmp_ctx* ctx, int* flag_ab, int fin_rk, nsmp_stage_info* info);
int nsmp_copy_known_from_np(nsmp_ctx* ctx);  /* nsmp3D.F90:480-504 */
int nsmp_rk2_finalize(nsmp_ctx* ctx);        /* nsmp3D.F90:531-546 */
/* u,v,w(n+1) = a*u(n) + b*u(n+1) over all cells (SSP-RK3 combinations). */
int nsmp_rk_combine(nsmp_ctx* ctx, double a, double b);
int nsmp_time_update(nsmp_ctx* ctx);         /* LoopTimeUpdate.F90:228-250 */
/* Convenience: nsteps full steps; fin_rk 1 = Euler->AB2, 2 = RK2, 3 = SSP-RK3.
 * *flag_ab is read before the first stage and written after the last one
 * (the switch of hydro.F90:469-478); NULL keeps the context's flag. */
int nsmp_step(nsmp_ctx* ctx, int fin_rk, int nsteps, int* flag_ab, nsmp_stage_info* last);

/* Indices of the values nsmp_cfl_diag returns. */
enum {
    NSMP_CFL_UMAX = 0,      /* signed u of largest |u| (first in loop order)    cfl.F90:99     */
    NSMP_CFL_VMAX,          /* signed v of largest |v|                          cfl.F90:100    */
    NSMP_CFL_WMAX,          /* signed w of largest |w|                          cfl.F90:101    */
    NSMP_CFL_AVEU,          /* sum u area h / (TotalVolume (SigFin-SigIni)), the meanuv.dat columns */
    NSMP_CFL_AVEV,          /*                                                  cfl.F90:108-110, 186-189 */
    NSMP_CFL_AVEW,
    NSMP_CFL_MAX,           /* max CFL, 0.5 dt sum|face flux| / (area h)        cfl.F90:140-166 */
    NSMP_CFL_FLUX_TOTAL,    /* "Total flux": sum of the cells' net outflow      cfl.F90:138-165 */
    NSMP_CFL_FLUX_MAX,      /* "Maxim flux": signed net outflow of largest modulus  cfl.F90:167-168 */
    NSMP_CFL_FLUX_BC,       /* "BC flux" = BOT + TOP + Side                     cfl.F90:215    */
    NSMP_CFL_FLUX_BOT,      /* sum UBFACE area at k = 2                         cfl.F90:171-175 */
    NSMP_CFL_FLUX_TOP,      /* sum UTFACE area at k = NZ-1                      cfl.F90:177-181 */
    NSMP_CFL_FLUX_SIDE,     /* face flux through the lateral boundary edges     cfl.F90:141-150 */
    NSMP_CFL_ABS_DIV,       /* sum of |net outflow| (not printed by glob_cfl)   */
    NSMP_CFL_COUNT
};
/* glob_cfl (Main/cfl.F90:7-269) on the level-n velocities and the face
 * fluxes, FP64 on the device, out[NSMP_CFL_COUNT].  With ref_bug_compat the
 * lateral fluxes of the divergence are weighted by dsig(k-1) and everything
 * else by dsig(k), as shipped (cfl.F90:108-110, 139-140); without it both use
 * the cell height dsigv(k-1).  Maxima equal the reference's exactly; sums
 * differ from its running accumulators by summation order only. */
int nsmp_cfl_diag(nsmp_ctx* ctx, double* out);
/* The four mass-flux figures of nsmp_cfl_diag: out[0] = sum|div|,
 * out[1] = max|div| (= |Maxim flux|), out[2] = sum div (Total flux),
 * out[3] = max CFL. */
int nsmp_mass_diag(nsmp_ctx* ctx, double out[4]);
int nsmp_set_precision(nsmp_ctx* ctx, int mode);
/* The four figures of nsmp_mass_diag without any allocation (no counterpart
 * in the reference).  For callers that cannot allocate device memory after
 * setup -- a driver that reserves a fixed device-memory budget before its
 * time loop, or one that forbids allocation inside the loop because it can
 * synchronise the device -- the reduction scratch lives in a static device
 * array of the library instead of in context buffers.  Limit: contexts of at
 * most 16,777,216 prisms (65536 blocks of 256); larger ones get
 * NSMP_ERR_RANGE.  The array (about 2 MB) stays on every GPU that loaded the
 * library until exit.  All calls share it, so calls that overlap on the GPU
 * race.  The call copies its four results to `out` and waits for the
 * context's stream before returning.  The first call on a device resolves
 * the array's address and should come before any stream capture. */
int nsmp_mass_diag_noalloc(nsmp_ctx* ctx, double out[4]);
/* NSMP_MIXED pressure solver.  The FP32 BiCGSTAB hands its correction e to
 * FP64 when its residual fell by inner_tol since the last hand-over (default
 * 3e-2) or after inner_cap iterations (default 80): x += e, and the FP32
 * residual is replaced by the FP64 residual b - A x.  A correction that
 * raised |b - A x|_2 more than 2x is cut to the step that minimises it and
 * the Krylov process restarts with a perturbed shadow residual; it also
 * restarts after restart_every iterations (default 300).  The FP64 stopping
 * test (eps) is unaffected: these trade hand-overs against iterations, not
 * accuracy.  The mixed mode needs an even number of interior layers. */
int nsmp_set_inner_solver(nsmp_ctx* ctx, double inner_tol, int inner_cap, int restart_every);
/* NSMP_FP64 pressure solver: 0 (default) applies A D^-1 with the Jacobi-
 * scaled couplings stored once per prism (five FP64 arrays read by each
 * product); 1 regenerates them matrix-free from the column and layer factors
 * and D^-1 (five fewer arrays, ten more FP64 multiplies a prism).  The two
 * give the same bits. */
int nsmp_set_fp64_spmv(nsmp_ctx* ctx, int matrix_free);
/* Stream used by the context (cudaStream_t as void*). */
void* nsmp_stream(nsmp_ctx* ctx);

/* ---- output path (Save/*.F90) ------------------------------------------- */

/* Vertex values of a level-n field (NSMP_F_U .. NSMP_F_P) in the reference's
 * vertex numbering, (N_VERT,NZ-1): tagdir 2 = the cell-layer vertex values
 * of interpolation2D, tagdir 3 = blended to the vertex layers sigv(k) with
 * the wall values of BCvelvertex3D (interpolation3D.F90:151-220,
 * BC.F90:603-807, periodic copies averaged as bc_periodic does). */
int nsmp_download_vertex(nsmp_ctx* ctx, int field, int tagdir, double* host);

/* ---- turbulence statistics (Stats/stats.F90) ---------------------------- */

/* Sums accumulated by nsmp_stats_sample, for nsmp_stats_download. */
enum {
    NSMP_S_U = 0, NSMP_S_V, NSMP_S_W, NSMP_S_P, NSMP_S_U2, NSMP_S_V2, NSMP_S_W2,
    NSMP_S_UV, NSMP_S_VW, NSMP_S_WU, NSMP_S_P2, NSMP_S_EDDY, NSMP_NSTATS
};
/* sm_init (stats.F90:34-84): zero the sums and the sample count. */
int nsmp_stats_reset(nsmp_ctx* ctx);
/* glob_sample (stats.F90:91-197) on level n, to be called after
 * nsmp_time_update where nsmp3D.F90:580-583 calls glob_sample(ufnp,...):
 * adds u, v, w, p, their squares and cross products and nu_t (LES) of every
 * interior cell and layer to the device sums. */
int nsmp_stats_sample(nsmp_ctx* ctx);
int nsmp_stats_count(nsmp_ctx* ctx, int* n);
/* One sum as an (N_CELL,NZ) array (ghost rows zero), e.g. for SavetecStats. */
int nsmp_stats_download(nsmp_ctx* ctx, int which, double* host);
/* glob_put_plane_mm (stats.F90:204-384): for k = 2..NZ-1 a row of out
 * ((NZ-2) rows x 10, row-major): yplus, mean u, v, w, rms u, v, w, and
 * uv, vw, wu shear stresses (mean product minus product of means, as the
 * reference writes them); *tke = the plane-averaged turbulent kinetic
 * energy summed over layers / (NZ-2). */
int nsmp_stats_plane(nsmp_ctx* ctx, double* out, double* tke);

/* ---- discrete adjoint (an extension: the reference has none) ------------ */

/* Body force on u per cell, (N0,NZ) column-major in the original cell
 * numbering (the ghost layers k = 1 and NZ are ignored), added to the u
 * right-hand side of every stage next to bdx (hydro.F90:322-333).  NULL
 * removes it. */
int nsmp_set_body_force(nsmp_ctx* ctx, const double* fx);
/* Wall shear stress of level n averaged over both walls:
 * sum_c area_c nu (u(c,2)/h_2 + u(c,NZ-1)/h_NZ-1) / (2 sum_c area_c), with
 * h the half height of the layer next to the wall and nu = 1/re. */
int nsmp_wall_shear(nsmp_ctx* ctx, double* tau);
/* From the current state: nsteps SSP-RK3 steps with body force fx (as
 * nsmp_set_body_force), J = mean over steps 1..nsteps of nsmp_wall_shear,
 * and the gradient dJ/dfx, (N0,NZ) like fx, by the discrete adjoint of the
 * steps.  The state is checkpointed every ckpt_every steps and each segment
 * is recomputed once during the reverse sweep, replaying the pressure
 * solutions recorded by the forward sweep instead of solving again.  Device
 * memory: 9 cell fields per checkpoint, 3 interior fields per step for the
 * recorded pressures, and the stage inputs of a segment (24 cell fields per
 * step) -- or, when those exceed the budget of nsmp_set_adjoint_budget,
 * inner checkpoints every ~sqrt(ckpt_every) steps of the segment plus the
 * stage inputs of one step.  The adjoint pressure solves run in the
 * context's precision mode.  The context ends at the state after the nsteps
 * steps with fx still set.  Returns the worst status of the forward and
 * adjoint pressure solves. */
int nsmp_adjoint(nsmp_ctx* ctx, int nsteps, int ckpt_every, const double* fx,
                 double* grad_out, double* J_out);
/* Bytes nsmp_adjoint may use for the stage inputs of a segment; 0 (the
 * default) means 80 % of the free device memory at the call. */
int nsmp_set_adjoint_budget(nsmp_ctx* ctx, double bytes);
/* y = A x and y = A^T x for the PPE operator (PDE.F90:69-121) on interior
 * fields (N0,NZ): the hooks of the dot-product test <A v, w> = <v, A^T w>. */
int nsmp_apply_A(nsmp_ctx* ctx, const double* x, double* y);
int nsmp_apply_AT(nsmp_ctx* ctx, const double* x, double* y);

/* ---- instrumentation ---------------------------------------------------- */

/* Kernel ids for nsmp_prof_read.  NSMP_K_BICG_P .. NSMP_K_BICG_X are the FP64
 * solver's passes; NSMP_K_IN_PV .. NSMP_K_MIX_SCALE the mixed solver's (FP32
 * p/v and s/t passes, FP64 update and rescale). */
enum {
    NSMP_K_VERTEX4 = 0, NSMP_K_STAGE_RHS, NSMP_K_FACES_DIV, NSMP_K_BICG_INIT, NSMP_K_BICG_P,
    NSMP_K_BICG_SPMV_V, NSMP_K_BICG_S, NSMP_K_BICG_SPMV_T, NSMP_K_BICG_X, NSMP_K_PMEAN,
    NSMP_K_VERTEX1, NSMP_K_PROJECT, NSMP_K_IN_PV, NSMP_K_IN_ST, NSMP_K_MIX_UPDATE,
    NSMP_K_MIX_SCALE, NSMP_K_OTHER, NSMP_K_COUNT
};
/* on = 1 records a CUDA event pair around every kernel launch on the
 * context's stream and accumulates per-kernel device time; on = 0 stops.
 * Enabling also clears the accumulators. */
int nsmp_prof_enable(nsmp_ctx* ctx, int on);
int nsmp_prof_read(nsmp_ctx* ctx, int kernel_id, long long* launches, double* total_ms);
/* NSMP_MIXED diagnostics of the last stage's pressure solve, for its last
 * (at most 48) FP64 updates, oldest first: FP32 iterations since the previous
 * update, the FP32 relative residual reached, the FP64 relative residual
 * after the update, and flags (bit 0: correction accepted, bit 1: Krylov
 * process restarted).  Returns the number of updates written. */
int nsmp_solver_log(nsmp_ctx* ctx, int max_cycles, int* inner_iters, double* inner_res,
                    double* outer_res, int* accepted);
/* Kernels launched and BiCGSTAB iterations executed since creation. */
int nsmp_counters(nsmp_ctx* ctx, long long* launches, long long* bicg_iters);
/* BiCGSTAB iterations and, in NSMP_MIXED, FP64 hand-overs (refinement
 * updates) executed since creation. */
int nsmp_solver_counters(nsmp_ctx* ctx, long long* bicg_iters, long long* fp64_updates);
/* Measured FP64 FMA issue rate of a device: every thread of a full-device
 * grid runs `chains` independent chains of `iters` dependent fused
 * multiply-adds, timed with CUDA events; *tflops = 2 x FMAs / time.  No
 * context needed.  The roof for the FP64 kernels that are bound by FP64
 * issue rather than by HBM. */
int nsmp_probe_fp64_fma(int device, int iters, double* tflops, double* ms);

/* ---- synthetic inputs (host only, no GPU needed) ------------------------ */

/* Periodic nx x ny quad mesh, each quad split along a seeded diagonal,
 * interior vertices jittered by +-jitter*spacing.  N0 = 2*nx*ny,
 * N_VERT = (nx+1)*(ny+1) (boundary vertices duplicated as in the reference). */
int nsmp_mesh_size(int nx, int ny, int* n0, int* nvert);
int nsmp_mesh_generate(int nx, int ny, double x0, double x1, double y0,
                       double y1, double jitter, unsigned long long seed,
                       int* No_vp, int* No_cp, int* nbe, int* nbev,
                       double* xv, double* yv);
/* Seeded channel initial state on the (N_CELL,NZ) grid: u = umax*z*(2-z),
 * plus uniform noise of half-width amp on u, v, w; p = 0.  The noise of an
 * interior cell depends only on (seed, original cell number, layer,
 * component).  Ghost entries are 0 (filled by nsmp_user_initial). */
int nsmp_initial_channel(const nsmp_params* prm, int n_cell, double umax,
                         double amp, unsigned long long seed, double* u,
                         double* v, double* w, double* p);
/* Sigma grid of the parameters: sig(NZ), dsig(NZ), sigv(NZ-1), dsigv(NZ-1). */
int nsmp_sigma_grid(const nsmp_params* prm, double* sig, double* dsig,
                    double* sigv, double* dsigv);

/* Geometry arrays as the setup computes them (calcul_geometry.F90 shapes),
 * for diagnostics; host only.  `out` must hold 3*N_CELL doubles (N_CELL =
 * N0 + number of lateral boundary edges); *count receives the length. */
enum {
    NSMP_G_XC = 0, NSMP_G_YC, NSMP_G_AREA,                /* (N_CELL)   */
    NSMP_G_DLVV, NSMP_G_DLCC, NSMP_G_DLE1, NSMP_G_DLE2,   /* (N0,3)     */
    NSMP_G_DOE, NSMP_G_XNN, NSMP_G_YNN, NSMP_G_DXCC, NSMP_G_DYCC,
    NSMP_G_SUMXC2, NSMP_G_SUMYC2, NSMP_G_SUMXCYC,         /* (N0)       */
    NSMP_G_SIG, NSMP_G_DSIG, NSMP_G_SIGV, NSMP_G_DSIGV,   /* sigma grid */
    NSMP_G_DLVSUM,                                        /* (N_VERT)   */
    NSMP_G_NOCP,                                          /* (N_CELL,3) */
    NSMP_G_PERM                                           /* (N0) device column -> cell */
};
int nsmp_geometry(const nsmp_params* prm, const nsmp_mesh* mesh, int which,
                  double* out, int* count);
/* The same arrays from the setup nsmp_create runs: the floating-point
 * geometry (calcul_geometry's cell, edge and vertex-weight formulas) computed
 * on device prm->device, the topology (ghosts, periodic images, vertex
 * classes, renumbering) on the host.  Equal to nsmp_geometry bit for bit;
 * needs a GPU. */
int nsmp_geometry_device(const nsmp_params* prm, const nsmp_mesh* mesh, int which,
                         double* out, int* count);

#ifdef __cplusplus
}
#endif
#endif
