// C-ABI entry points (include/nsmp.h).  Every function catches host
// exceptions and returns a status; nothing throws across the boundary.
#include <algorithm>
#include <cstring>
#include <new>

#include "ctx.h"

using nsmp::HostLayout;

namespace {

int set_err(nsmp_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

bool valid_field(int f) { return f >= 0 && f < NSMP_NFIELDS; }

}  // namespace

extern "C" {

int nsmp_create(const nsmp_params* prm, const nsmp_mesh* mesh, nsmp_ctx** out) {
    if (!prm || !mesh || !out || !mesh->No_vp || !mesh->No_cp || !mesh->nbe || !mesh->nbev || !mesh->xv ||
        !mesh->yv)
        return NSMP_ERR_ARG;
    *out = nullptr;
    nsmp_ctx* c = new (std::nothrow) nsmp_ctx();
    if (!c) return NSMP_ERR_NOMEM;
    try {
        c->prm = *prm;
        c->device = prm->device;
        if (prm->precision != NSMP_FP64 && prm->precision != NSMP_MIXED && prm->precision != NSMP_MIXED_F32) {
            delete c;
            return NSMP_ERR_ARG;
        }
        c->precision = (prm->precision == NSMP_FP64) ? NSMP_FP64 : NSMP_MIXED;
        c->stage32 = prm->precision == NSMP_MIXED_F32;
        // the setup makes the context's device current; the caller's
        // current device is given back when nsmp_create returns
        nsmp::DeviceGuard guard(c->device);
        std::string err;
        // the floating-point geometry on the context's device, the topology on the host
        int rc = nsmp::build_layout_device(*prm, *mesh, c->L, err);
        if (rc != 0) {
            delete c;
            return rc;
        }
        rc = nsmp::ctx_init_device(c);
        if (rc != 0) {
            nsmp::ctx_free(c);
            delete c;
            return rc;
        }
    } catch (const std::bad_alloc&) {
        delete c;
        return NSMP_ERR_NOMEM;
    } catch (...) {
        delete c;
        return NSMP_ERR_ARG;
    }
    *out = c;
    return NSMP_OK;
}

int nsmp_destroy(nsmp_ctx* c) {
    if (!c) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    nsmp::ctx_free(c);
    delete c;
    return NSMP_OK;
}

const char* nsmp_last_error(const nsmp_ctx* c) { return c ? c->err.c_str() : "null context"; }

int nsmp_ncell(const nsmp_ctx* c, int* n_cell) {
    if (!c || !n_cell) return NSMP_ERR_ARG;
    *n_cell = c->L.NC;
    return NSMP_OK;
}

void* nsmp_stream(nsmp_ctx* c) { return c ? (void*)c->stream : nullptr; }

int nsmp_host_register(nsmp_ctx* c, void* host, size_t bytes) {
    if (!c || !host || bytes == 0) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    const cudaError_t e = cudaHostRegister(host, bytes, cudaHostRegisterPortable);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(c, NSMP_ERR_CUDA, std::string("nsmp_host_register: ") + cudaGetErrorString(e));
    }
    return NSMP_OK;
}

int nsmp_host_unregister(nsmp_ctx* c, void* host) {
    if (!c || !host) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    const cudaError_t e = cudaHostUnregister(host);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(c, NSMP_ERR_CUDA, std::string("nsmp_host_unregister: ") + cudaGetErrorString(e));
    }
    return NSMP_OK;
}

int nsmp_user_initial(nsmp_ctx* c, const double* u, const double* v, const double* w, const double* p) {
    if (!c || !u || !v || !w || !p) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    const double* in[4] = {u, v, w, p};
    for (int f = 0; f < 4; ++f) {
        int rc = nsmp::run_scatter(c, in[f], c->lvl[c->ln][f]);
        if (rc) return rc;
    }
    c->flag_ab = 0;
    c->lknown = c->ln;
    return nsmp::run_user_initial(c);
}

int nsmp_upload_state(nsmp_ctx* c, const double* u, const double* v, const double* w, const double* p,
                      const double* u1f, const double* u2f, const double* u3f, const double* utf,
                      const double* ubf, const double* rhsu, const double* rhsv, const double* rhsw, int flag_ab) {
    if (!c || !u || !v || !w || !p || !u1f || !u2f || !u3f || !utf || !ubf || !rhsu || !rhsv || !rhsw)
        return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    // one contiguous copy and a scatter per array, one synchronisation at the
    // end (the host arrays are free for reuse when this returns)
    const double* cells[4] = {u, v, w, p};
    for (int f = 0; f < 4; ++f) {
        int rc = nsmp::run_scatter(c, cells[f], c->lvl[c->ln][f], c->L.NC, false);
        if (rc) return rc;
    }
    int rc = nsmp::run_fill_ghosts(c, c->ln);
    if (rc) return rc;
    // face fluxes are (N0,NZ)
    const double* faces[5] = {u1f, u2f, u3f, utf, ubf};
    for (int f = 0; f < 5; ++f) {
        rc = nsmp::run_scatter(c, faces[f], c->face[f], c->L.N0, false);
        if (rc) return rc;
    }
    const double* hs[3] = {rhsu, rhsv, rhsw};
    for (int f = 0; f < 3; ++f) {
        rc = nsmp::run_scatter(c, hs[f], c->hist[f], c->L.NC, false);
        if (rc) return rc;
    }
    const cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return set_err(c, NSMP_ERR_CUDA, std::string("upload_state: ") + cudaGetErrorString(e));
    c->flag_ab = flag_ab;
    c->lknown = c->ln;
    return NSMP_OK;
}

int nsmp_download(nsmp_ctx* c, int field, double* host) {
    if (!c || !host || !valid_field(field)) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    const int NC = c->L.NC, N0 = c->L.N0;
    switch (field) {
        case NSMP_F_U: case NSMP_F_V: case NSMP_F_W: case NSMP_F_P:
            return nsmp::run_gather(c, c->lvl[c->ln][field - NSMP_F_U], 0, NC, host);
        case NSMP_F_UNP: case NSMP_F_VNP: case NSMP_F_WNP: case NSMP_F_PNP:
            return nsmp::run_gather(c, c->lvl[c->lnp][field - NSMP_F_UNP], 0, NC, host);
        case NSMP_F_U1FACE: case NSMP_F_U2FACE: case NSMP_F_U3FACE: case NSMP_F_UTFACE: case NSMP_F_UBFACE:
            return nsmp::run_gather(c, c->face[field - NSMP_F_U1FACE], 0, N0, host);
        case NSMP_F_RHSU: case NSMP_F_RHSV: case NSMP_F_RHSW:
            return nsmp::run_gather(c, c->hist[field - NSMP_F_RHSU], 1, NC, host);
        case NSMP_F_EDDY:
            return nsmp::run_gather(c, c->eddy, 0, NC, host);
        case NSMP_F_PV:
            return nsmp::run_download_pv(c, host);
    }
    return NSMP_ERR_ARG;
}

int nsmp_copy_known_from_n(nsmp_ctx* c) {
    if (!c) return NSMP_ERR_ARG;
    c->lknown = c->ln;
    return NSMP_OK;
}

int nsmp_hydro_stage(nsmp_ctx* c, int* flag_ab, int fin_rk, nsmp_stage_info* info) {
    if (!c || !flag_ab || fin_rk < 1 || fin_rk > 3) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    c->flag_ab = *flag_ab;
    int rc;
    try {
        rc = nsmp::run_stage(c, fin_rk, info);
    } catch (...) {
        return set_err(c, NSMP_ERR_CUDA, "host exception in stage");
    }
    *flag_ab = c->flag_ab;
    return rc;
}

int nsmp_copy_known_from_np(nsmp_ctx* c) {
    if (!c) return NSMP_ERR_ARG;
    c->lknown = c->lnp;
    return NSMP_OK;
}

int nsmp_rk2_finalize(nsmp_ctx* c) {
    if (!c) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    return nsmp::run_combine(c, 0.5, 0.5);
}

int nsmp_rk_combine(nsmp_ctx* c, double a, double b) {
    if (!c) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    return nsmp::run_combine(c, a, b);
}

int nsmp_time_update(nsmp_ctx* c) {
    if (!c) return NSMP_ERR_ARG;
    c->ln = c->lnp;
    c->lknown = c->ln;
    return NSMP_OK;
}

// nsmp3D.F90:394-564 for fin_rk 1 and 2; fin_rk 3 is the SSP-RK3
// composition u1 = S(u^n), u2 = 3/4 u^n + 1/4 S(u1), u^n+1 = 1/3 u^n + 2/3 S(u2)
// of the same stage (pressure and face fluxes taken from the last stage,
// as the reference's RK2 does).
int nsmp_step(nsmp_ctx* c, int fin_rk, int nsteps, int* flag_ab, nsmp_stage_info* last) {
    if (!c || fin_rk < 1 || fin_rk > 3 || nsteps < 0) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    if (flag_ab) c->flag_ab = *flag_ab;
    int worst = 0;
    for (int s = 0; s < nsteps; ++s) {
        nsmp_copy_known_from_n(c);
        const int nst = fin_rk;
        nsmp_stage_info inf{};
        for (int st = 1; st <= nst; ++st) {
            int fab = c->flag_ab;
            int rc = nsmp_hydro_stage(c, &fab, fin_rk, &inf);
            if (rc < 0) return rc;
            if (rc > worst) worst = rc;
            if (fin_rk == 3 && st == 2) {
                rc = nsmp::run_combine(c, 0.75, 0.25);
                if (rc) return rc;
            }
            if (st < nst) nsmp_copy_known_from_np(c);
        }
        if (fin_rk == 2) {
            int rc = nsmp::run_combine(c, 0.5, 0.5);
            if (rc) return rc;
        } else if (fin_rk == 3) {
            int rc = nsmp::run_combine(c, 1.0 / 3.0, 2.0 / 3.0);
            if (rc) return rc;
        }
        nsmp_time_update(c);
        if (last) *last = inf;
    }
    if (flag_ab) *flag_ab = c->flag_ab;
    return worst;
}

int nsmp_mass_diag(nsmp_ctx* c, double out[4]) {
    if (!c || !out) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    return nsmp::run_mass_diag(c, out);
}

int nsmp_set_precision(nsmp_ctx* c, int mode) {
    if (!c || (mode != NSMP_FP64 && mode != NSMP_MIXED && mode != NSMP_MIXED_F32)) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    if (mode != NSMP_FP64 && !c->b64) {
        int rc = nsmp::mixed_alloc(c);
        if (rc) return rc;
    }
    if (mode == NSMP_MIXED_F32) {
        int rc = nsmp::stage32_alloc(c);
        if (rc) return rc;
    }
    c->precision = (mode == NSMP_FP64) ? NSMP_FP64 : NSMP_MIXED;
    c->stage32 = mode == NSMP_MIXED_F32;
    c->prm.precision = mode;
    return NSMP_OK;
}

int nsmp_set_fp64_spmv(nsmp_ctx* c, int matrix_free) {
    if (!c || (matrix_free != 0 && matrix_free != 1)) return NSMP_ERR_ARG;
    c->fp64_spmv_mf = matrix_free;
    return NSMP_OK;
}

int nsmp_set_inner_solver(nsmp_ctx* c, double inner_tol, int inner_cap, int restart_every) {
    if (!c || !(inner_tol > 0.0) || !(inner_tol < 1.0) || inner_cap < 1 || restart_every < 1) return NSMP_ERR_ARG;
    c->inner_tol = inner_tol;
    c->inner_cap = inner_cap;
    c->restart_every = restart_every;
    return NSMP_OK;
}

int nsmp_prof_enable(nsmp_ctx* c, int on) {
    if (!c) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    if (c->stream) cudaStreamSynchronize(c->stream);
    nsmp::prof_resolve(c);
    c->prof_on = on ? 1 : 0;
    if (on)
        for (int k = 0; k < NSMP_K_COUNT; ++k) { c->prof_count[k] = 0; c->prof_ms[k] = 0.0; }
    return NSMP_OK;
}

int nsmp_prof_read(nsmp_ctx* c, int kid, long long* launches, double* total_ms) {
    if (!c || kid < 0 || kid >= NSMP_K_COUNT || !launches || !total_ms) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    if (c->stream) cudaStreamSynchronize(c->stream);
    nsmp::prof_resolve(c);
    *launches = c->prof_count[kid];
    *total_ms = c->prof_ms[kid];
    return NSMP_OK;
}

int nsmp_solver_log(nsmp_ctx* c, int max_cycles, int* inner_iters, double* inner_res, double* outer_res,
                    int* accepted) {
    if (!c || max_cycles < 0 || !inner_iters || !inner_res || !outer_res || !accepted) return NSMP_ERR_ARG;
    const nsmp::Scal& s = *c->h_scal;
    const int n = std::min(std::min(max_cycles, s.outer), nsmp::Scal::kCycLog);
    for (int k = 0; k < n; ++k) {  // the last n updates, oldest first
        const int q = (s.outer - n + k) % nsmp::Scal::kCycLog;
        inner_iters[k] = s.cyc_it[q];
        inner_res[k] = s.cyc_in[q];
        outer_res[k] = s.cyc_out[q];
        accepted[k] = s.cyc_acc[q];
    }
    return n;
}

int nsmp_counters(nsmp_ctx* c, long long* launches, long long* bicg_iters) {
    if (!c || !launches || !bicg_iters) return NSMP_ERR_ARG;
    *launches = c->launches;
    *bicg_iters = c->bicg_iters;
    return NSMP_OK;
}

int nsmp_solver_counters(nsmp_ctx* c, long long* bicg_iters, long long* fp64_updates) {
    if (!c || !bicg_iters || !fp64_updates) return NSMP_ERR_ARG;
    *bicg_iters = c->bicg_iters;
    *fp64_updates = c->fp64_updates;
    return NSMP_OK;
}

namespace {

// Geometry array `which` as the host setup (device = -1) or the device setup
// on ordinal `device` computes it.
int geometry_of(const nsmp_params* prm, const nsmp_mesh* mesh, int which, double* out, int* count, int device) {
    if (!prm || !mesh || !out || !count) return NSMP_ERR_ARG;
    try {
        HostLayout L;
        std::string err;
        int rc;
        if (device >= 0) {
            nsmp::DeviceGuard guard(device);
            if (guard.err != cudaSuccess) return NSMP_ERR_CUDA;
            rc = nsmp::build_layout_device(*prm, *mesh, L, err);
        } else {
            rc = nsmp::build_layout(*prm, *mesh, L, err);
        }
        if (rc) return rc;
        const std::vector<double>* src = nullptr;
        switch (which) {
            case NSMP_G_XC: src = &L.ref_xc; break;
            case NSMP_G_YC: src = &L.ref_yc; break;
            case NSMP_G_AREA: src = &L.ref_area; break;
            case NSMP_G_DLVV: src = &L.ref_dlVV; break;
            case NSMP_G_DLCC: src = &L.ref_dlCC; break;
            case NSMP_G_DLE1: src = &L.ref_dle1; break;
            case NSMP_G_DLE2: src = &L.ref_dle2; break;
            case NSMP_G_DOE: src = &L.ref_doe; break;
            case NSMP_G_XNN: src = &L.ref_xnn; break;
            case NSMP_G_YNN: src = &L.ref_ynn; break;
            case NSMP_G_DXCC: src = &L.ref_dxCC; break;
            case NSMP_G_DYCC: src = &L.ref_dyCC; break;
            case NSMP_G_SUMXC2: src = &L.ref_sxx; break;
            case NSMP_G_SUMYC2: src = &L.ref_syy; break;
            case NSMP_G_SUMXCYC: src = &L.ref_sxy; break;
            case NSMP_G_SIG: src = &L.sig; break;
            case NSMP_G_DSIG: src = &L.dsig; break;
            case NSMP_G_SIGV: src = &L.sigv; break;
            case NSMP_G_DSIGV: src = &L.dsigv; break;
            case NSMP_G_DLVSUM: src = &L.ref_dlVsum; break;
            case NSMP_G_NOCP: {
                for (size_t q = 0; q < L.ref_No_cp.size(); ++q) out[q] = (double)L.ref_No_cp[q];
                *count = (int)L.ref_No_cp.size();
                return NSMP_OK;
            }
            case NSMP_G_PERM: {
                for (size_t q = 0; q < L.perm.size(); ++q) out[q] = (double)L.perm[q];
                *count = (int)L.perm.size();
                return NSMP_OK;
            }
            default: return NSMP_ERR_ARG;
        }
        std::memcpy(out, src->data(), src->size() * sizeof(double));
        *count = (int)src->size();
        return NSMP_OK;
    } catch (...) {
        return NSMP_ERR_NOMEM;
    }
}

}  // namespace

// Host-only diagnostic: geometry exactly as the host setup computes it.
int nsmp_geometry(const nsmp_params* prm, const nsmp_mesh* mesh, int which, double* out, int* count) {
    return geometry_of(prm, mesh, which, out, count, -1);
}

int nsmp_geometry_device(const nsmp_params* prm, const nsmp_mesh* mesh, int which, double* out, int* count) {
    if (!prm) return NSMP_ERR_ARG;
    return geometry_of(prm, mesh, which, out, count, prm->device);
}

}  // extern "C"
