/*
 * CPU oracle for the nsmp3D per-time-step hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A C++ restatement of the Fortran reference (techi28/3D-channel-flow-code,
 * serial branches, shipped key set KeyKimChoi + KeyPPECenter + KeyPPERHS +
 * KeyTESTpBC + KeyTESTChannel, optionally KeyLES/KeyLESVan).  It is used only
 * by tests/, by __graft_entry__.smoke() as the checker and by bench.py's CPU
 * baseline leg.  The product (the CUDA library) never links or calls it.
 *
 * Parity status: the reference ships no tests, golden vectors or input decks
 * and no Fortran compiler exists in this image, so parity with the reference
 * binary is UNPINNED.  The oracle is pinned only by the reference's own
 * known answers (Functions.F90 Taylor-Green fields) and the invariants the
 * reference asserts (PPE coefficient checks, periodic pairing checks,
 * mass-flux divergence).
 *
 * Arrays crossing this interface use the reference's Fortran conventions:
 * column-major (N_CELL,NZ) / (N0,NZ) / (N_VERT,NZ-1), 1-based index values.
 */
#ifndef NSMP_ORACLE_H
#define NSMP_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_params {
    int n0, nvert, nz;            /* N_CELL0, N_VERT, NZ (= layers + 2)          */
    double xdini, xdfin;          /* common.mpf:66-67                            */
    double ydini, ydfin;          /* common.mpf:68-69                            */
    double sigini, sigfin;        /* common.mpf:64-65                            */
    int grid_kind;                /* 0 uniform (calcul_geometry.F90:263-283), 1 tanh */
    double grid_beta;             /* tanh stretching factor                      */
    int top_bc, bot_bc;           /* 0 no-slip, 1 free-slip (common.mpf:77-78)   */
    double dt, re, bdx, bdy, bdz; /* dataParameters.txt                          */
    double eps;                   /* BiCGSTAB tolerance                          */
    int max_iters;                /* BiCGSTAB iteration cap                      */
    int les, les_van;             /* KeyLES, KeyLESVan                           */
    int ref_bug_compat;           /* 1: keep reference quirks                    */
    int nthreads;                 /* OpenMP threads (0 = runtime default)        */
} orc_params;

typedef struct orc_info {
    int iters;          /* BiCGSTAB iterations of the last stage     */
    double e1norm;      /* final relative L1 residual                */
    double e2norm;      /* final relative L2 residual                */
    int converged;      /* 1 if min(e1,e2) < eps                     */
    double max_eddy;    /* max nu_t of the last stage (0 without LES)*/
    int iters_total;    /* BiCGSTAB iterations of all stages of a step */
    int iters_stage[3]; /* BiCGSTAB iterations of each stage of a step */
} orc_info;

typedef struct orc_ctx orc_ctx;

/* Field ids for orc_get/orc_set. */
enum {
    ORC_U = 0, ORC_V, ORC_W, ORC_P,          /* level n, (N_CELL,NZ)           */
    ORC_U1F, ORC_U2F, ORC_U3F, ORC_UTF, ORC_UBF, /* face fluxes (N0,NZ)      */
    ORC_RHSU, ORC_RHSV, ORC_RHSW,            /* AB2 history (N_CELL,NZ)        */
    ORC_EDDY,                                 /* nu_t (N_CELL,NZ)               */
    ORC_UV, ORC_VV, ORC_WV, ORC_PV,          /* vertex outputs (N_VERT,NZ-1)   */
    ORC_NFIELDS
};

/* Geometry array ids for orc_geom (N0 x 3 arrays unless noted). */
enum {
    ORCG_XC = 0, ORCG_YC, ORCG_AREA,          /* (N_CELL)                       */
    ORCG_DLVV, ORCG_DLCC, ORCG_DLE1, ORCG_DLE2, ORCG_DOE,
    ORCG_XNN, ORCG_YNN, ORCG_DXCC, ORCG_DYCC,
    ORCG_SUMXC2, ORCG_SUMYC2, ORCG_SUMXCYC,   /* (N0)                           */
    ORCG_SIG, ORCG_DSIG,                      /* (NZ)                           */
    ORCG_SIGV, ORCG_DSIGV,                    /* (NZ-1)                         */
    ORCG_AMC0, ORCG_AMC1, ORCG_AMC2, ORCG_AMC3, ORCG_AMCT, ORCG_AMCB, /* (N0,NZ)*/
    ORCG_DLVSUM,                              /* (N_VERT)                       */
    ORCG_NARR
};

/* Build geometry from the mesh (data.txt contents).  No_vp, No_cp are
 * (N0,3) column-major, 1-based; No_cp = 0 marks a boundary edge.
 * Returns NULL on a malformed mesh; *err gets a negative code. */
orc_ctx* orc_create(const orc_params* prm, const int* No_vp, const int* No_cp,
                    const int* nbe, const int* nbev, const double* xv,
                    const double* yv, int* err);
void orc_destroy(orc_ctx* c);
int orc_ncell(const orc_ctx* c);                 /* N_CELL = N0 + ghosts        */
int orc_ghost_image(const orc_ctx* c, int* img); /* No_cp(ghost,3) per ghost    */
int orc_no_cp(const orc_ctx* c, int* out);       /* (N_CELL,3) after ghosting  */
int orc_geom(const orc_ctx* c, int which, double* out);

/* user_initial.F90:166-238 analogue: take level-n interior values (N_CELL,NZ),
 * fill ghosts, build face fluxes (interpolateU) and zero the AB2 history. */
int orc_user_initial(orc_ctx* c, const double* u, const double* v,
                     const double* w, const double* p);

int orc_get(const orc_ctx* c, int field, double* out);
int orc_set(orc_ctx* c, int field, const double* in);
int orc_get_flag_ab(const orc_ctx* c);
/* 1: add the per-layer partial sums of every global sum in reverse layer
 * order (an equally valid order; for measuring the sensitivity of BiCGSTAB's
 * iteration count to the rounding of its dot products), 0: layer order. */
void orc_set_sum_order(orc_ctx* c, int reverse);
void orc_set_flag_ab(orc_ctx* c, int f);

/* One full time step (nsmp3D.F90:394-564): fin_rk 1 = Euler->AB2,
 * 2 = reference RK2 (Heun), 3 = SSP-RK3 composed from the same stage. */
int orc_step(orc_ctx* c, int fin_rk, orc_info* info);

/* Operator hooks for unit parity tests. */
int orc_set_body_force(orc_ctx* c, const double* fx);      /* (N0,NZ), NULL: none */
int orc_stats_reset(orc_ctx* c);                           /* sm_init              */
int orc_stats_sample(orc_ctx* c);                          /* glob_sample on level n */
int orc_stats_get(const orc_ctx* c, int which, double* out);  /* (N_CELL,NZ)       */
int orc_stats_plane(const orc_ctx* c, double* out, double* tke); /* (NZ-2) x 10    */
int orc_apply_A(orc_ctx* c, const double* x, double* y);   /* (N_CELL,NZ) -> (N0..)*/
int orc_predictor(orc_ctx* c, double* us, double* vs, double* ws); /* u* of a stage from level n */
int orc_gradient_lsm(orc_ctx* c, const double* f, double* dfdx, double* dfdy,
                     double* dfds);                         /* (N_CELL,NZ) each   */
int orc_vertex_interp(orc_ctx* c, const double* f, int is_pressure, int tagBC,
                      int tagdir, double* fv);              /* cell -> vertex     */
/* glob_cfl (cfl.F90:84-215), out[ORC_CFL_COUNT] in the order of nsmp_cfl_diag. */
enum {
    ORC_CFL_UMAX = 0, ORC_CFL_VMAX, ORC_CFL_WMAX, ORC_CFL_AVEU, ORC_CFL_AVEV, ORC_CFL_AVEW,
    ORC_CFL_MAX, ORC_CFL_FLUX_TOTAL, ORC_CFL_FLUX_MAX, ORC_CFL_FLUX_BC, ORC_CFL_FLUX_BOT,
    ORC_CFL_FLUX_TOP, ORC_CFL_FLUX_SIDE, ORC_CFL_ABS_DIV, ORC_CFL_COUNT
};
int orc_cfl_diag(orc_ctx* c, double* out);
/* out[0] = sum |div|, out[1] = max |div|, out[2] = sum div, out[3] = max CFL. */
int orc_mass_diag(orc_ctx* c, double* out);

/* Synthetic inputs (the oracle's own copy, for the CPU baseline): the
 * periodic jittered mesh in data.txt layout and the seeded channel state on
 * the (N_CELL,NZ) grid of a context. */
int orc_mesh_generate(int nx, int ny, double x0, double x1, double y0, double y1, double jitter,
                      unsigned long long seed, int* No_vp, int* No_cp, int* nbe, int* nbev,
                      double* xv, double* yv);
int orc_initial_channel(const orc_ctx* c, double umax, double amp, unsigned long long seed,
                        double* u, double* v, double* w, double* p);

#ifdef __cplusplus
}
#endif
#endif
