// FP64 pressure solve: the reference's Jacobi-preconditioned BiCGSTAB
// (Main/bicgstab.F90:303-591) on the 7-point PPE of PDE_center
// (AdvectionDiffusion/PDE.F90:69-121), one kernel per vector pass with the
// dot products fused into the pass that produces their operands.
//
// Vectors use the compact interior layout (index = the prism's thread index,
// no wall layers), so the streaming passes are plain double2 streams.  The
// operator A D^-1 is applied with the Jacobi-scaled couplings
// ahat_j = A_ij / A_jj precomputed once (its diagonal is 1): five FMAs per row,
// which matters because FP64 issue rate, not HBM, bounds this part on GB300.
#include "kern_common.cuh"

namespace nsmp {
namespace {

struct KryArgs {
    const double* rhsp;   // compact
    const double* pf;     // cell layout (initial guess, hydro.F90:388-392)
    double *x, *r, *r0, *p, *v, *s, *t;
    const double* invD;
    const double* ah[5];  // couplings to nb 1..3, top, bottom (0 at the walls)
};

// Jacobi diagonal 1/Am0 (diag_precdt, bicgstab.F90:831-836), once at setup.
__global__ void k_inv_diag(Mesh m, double* invD) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const ColPPE& P = m.ppe[c];
        const double dsv = lev(m, LV_DSV, k0);
        const double AAB = P.area * lev(m, LV_IDSB, k0) * lev(m, LV_WB, k0);
        const double AAT = P.area * lev(m, LV_IDST, k0) * lev(m, LV_WT, k0);
        const double AA0 = -1.0 * (AAT + AAB + P.kA[0] * dsv + P.kA[1] * dsv + P.kA[2] * dsv);
        invD[g] = 1.0 / AA0;
    }
}

__global__ void k_scaled_coefs(Mesh m, const double* __restrict__ invD, double* a1, double* a2, double* a3,
                               double* aT, double* aB) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const ColPPE& P = m.ppe[c];
        const double dsv = lev(m, LV_DSV, k0);
        a1[g] = (P.kA[0] * dsv) * invD[ICg(m, P.nb[0], k0)];
        a2[g] = (P.kA[1] * dsv) * invD[ICg(m, P.nb[1], k0)];
        a3[g] = (P.kA[2] * dsv) * invD[ICg(m, P.nb[2], k0)];
        aT[g] = (k0 < m.NZ - 2) ? (P.area * lev(m, LV_IDST, k0)) * invD[g + 1] : 0.0;
        aB[g] = (k0 > 1) ? (P.area * lev(m, LV_IDSB, k0)) * invD[g - 1] : 0.0;
    }
}

// Glob_Norm(rhs, 1) + initial residual and norms (bicgstab.F90:107-109,
// 403-451); x = pf.
__global__ void __launch_bounds__(kBlock) k_bicg_init(Mesh m, KryArgs a, RedScratch rs, Scal* sc) {
    const double avec = sc->sum_rhs / m.tv_lsig;
    double part[4] = {0.0, 0.0, 0.0, 0.0};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const ColPPE& P = m.ppe[c];
        const size_t q = cell_of(g, c);
        const double b = a.rhsp[g] - avec * P.area * lev(m, LV_HMEAN, k0);
        const double x0 = a.pf[q];
        const double Ax = ppe_row(m, P, k0, x0, a.pf[IX(m, P.nb[0], k0)], a.pf[IX(m, P.nb[1], k0)],
                                  a.pf[IX(m, P.nb[2], k0)], a.pf[q + 1], a.pf[q - 1]);
        const double r = b - Ax;
        a.x[g] = x0;
        a.r[g] = r;
        a.r0[g] = r;
        part[0] += b * b; part[1] += r * r; part[2] += fabs(b); part[3] += fabs(r);
    }
    double tot[4];
    if (grid_reduce<4, false>(part, rs, tot) && threadIdx.x == 0) {
        double b2 = sqrt(tot[0]), r2 = sqrt(tot[1]), b1 = tot[2], r1 = tot[3];
        if (b2 == 0.0) b2 = 1.0;
        if (b1 == 0.0) b1 = 1.0;
        sc->b1 = b1; sc->b2 = b2; sc->r1 = r1; sc->r2 = r2;
        sc->e1 = r1 / b1; sc->e2 = r2 / b2;
        sc->rho = tot[1];
        sc->rho_prev = 1.0; sc->alpha = 1.0; sc->omega = 1.0;
        sc->iter = 0; sc->status = 0; sc->converged = 0; sc->done = 0;
        if (!(r2 == r2)) { sc->status = NSMP_ERR_NAN; sc->done = 1; }
        else if (sc->e1 < sc->eps || sc->e2 < sc->eps) { sc->converged = 1; sc->done = 1; }
    }
}

// update_pk (bicgstab.F90:726-773), two prisms per thread.
__global__ void __launch_bounds__(kBlock) k_bicg_p(Mesh m, KryArgs a, const Scal* sc) {
    pdl_enter();
    if (sc->done) return;
    const int it = sc->iter;
    const double beta = (sc->rho / sc->rho_prev) * (sc->alpha / sc->omega), om = sc->omega;
    const int n2 = m.nprism >> 1;
    const double2* r = reinterpret_cast<const double2*>(a.r);
    const double2* v = reinterpret_cast<const double2*>(a.v);
    double2* p = reinterpret_cast<double2*>(a.p);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
        const double2 rr = r[i];
        if (it == 0) {
            p[i] = rr;
        } else {
            const double2 pp = p[i], vv = v[i];
            p[i] = make_double2(fma(beta, fma(-om, vv.x, pp.x), rr.x), fma(beta, fma(-om, vv.y, pp.y), rr.y));
        }
    }
    if ((m.nprism & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const int g = m.nprism - 1;
        a.p[g] = (it == 0) ? a.r[g] : fma(beta, fma(-om, a.v[g], a.p[g]), a.r[g]);
    }
}

// out = A D^-1 in (diag_precdt then get_Apk, bicgstab.F90:976-997) and the
// fused dots.  MODE 0: v = A D^-1 p, (r0, v);  MODE 1: t = A D^-1 s, (t, s), (t, t).
template <int MODE>
__global__ void __launch_bounds__(kBlock) k_bicg_spmv(Mesh m, KryArgs a, RedScratch rs, Scal* sc) {
    pdl_enter();
    if (sc->done) return;
    const double* __restrict__ in = (MODE == 0) ? a.p : a.s;
    double* __restrict__ out = (MODE == 0) ? a.v : a.t;
    const int NZI = m.NZI;
    double part[2] = {0.0, 0.0};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        const int c = g / NZI;
        const int kk = g - c * NZI;  // k0 - 1
        const ColPPE& P = m.ppe[c];
        const double x0 = in[g];
        double o = x0;
        o = fma(a.ah[0][g], in[g + (P.nb[0] - c) * NZI], o);
        o = fma(a.ah[1][g], in[g + (P.nb[1] - c) * NZI], o);
        o = fma(a.ah[2][g], in[g + (P.nb[2] - c) * NZI], o);
        // wall couplings are zero (AmT(i,NZ-1) = AmB(i,2) = 0)
        if (kk < NZI - 1) o = fma(a.ah[3][g], in[g + 1], o);
        if (kk > 0) o = fma(a.ah[4][g], in[g - 1], o);
        out[g] = o;
        if (MODE == 0) {
            part[0] = fma(a.r0[g], o, part[0]);
        } else {
            part[0] = fma(o, x0, part[0]);
            part[1] = fma(o, o, part[1]);
        }
    }
    if (MODE == 0) {
        double p1[1] = {part[0]}, t1[1];
        if (grid_reduce<1, false>(p1, rs, t1) && threadIdx.x == 0) {
            sc->r0v = t1[0];
            if (fabs(t1[0]) < 1.0e-30) { sc->done = 1; sc->status = NSMP_WARN_BREAKDOWN; }
            else sc->alpha = sc->rho / t1[0];
        }
    } else {
        double tot[2];
        if (grid_reduce<2, false>(part, rs, tot) && threadIdx.x == 0) {
            sc->ts = tot[0];
            sc->tt = tot[1];
            sc->omega = tot[0] / tot[1];
        }
    }
}

// The same product matrix-free: each coupling A_ij D^-1_j is regenerated from
// the column's kA_j (or area), the layer factor and D^-1 of the neighbour,
// with the operations k_scaled_coefs uses, so the result is bitwise that of
// the stored form.  It moves 5 fewer FP64 words a prism and issues 10 more
// FP64 multiplies (nsmp_set_fp64_spmv selects it).
template <int MODE>
__global__ void __launch_bounds__(kBlock) k_bicg_spmv_mf(Mesh m, KryArgs a, RedScratch rs, Scal* sc) {
    pdl_enter();
    if (sc->done) return;
    const double* __restrict__ in = (MODE == 0) ? a.p : a.s;
    double* __restrict__ out = (MODE == 0) ? a.v : a.t;
    const double* __restrict__ id = a.invD;
    const int NZI = m.NZI;
    double part[2] = {0.0, 0.0};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        const int c = g / NZI;
        const int kk = g - c * NZI;  // k0 - 1
        const int k0 = kk + 1;
        const ColPPE& P = m.ppe[c];
        const double dsv = lev(m, LV_DSV, k0);
        const double x0 = in[g];
        double o = x0;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int gn = g + (P.nb[j] - c) * NZI;
            o = fma((P.kA[j] * dsv) * id[gn], in[gn], o);
        }
        if (kk < NZI - 1) o = fma((P.area * lev(m, LV_IDST, k0)) * id[g + 1], in[g + 1], o);
        if (kk > 0) o = fma((P.area * lev(m, LV_IDSB, k0)) * id[g - 1], in[g - 1], o);
        out[g] = o;
        if (MODE == 0) {
            part[0] = fma(a.r0[g], o, part[0]);
        } else {
            part[0] = fma(o, x0, part[0]);
            part[1] = fma(o, o, part[1]);
        }
    }
    if (MODE == 0) {
        double p1[1] = {part[0]}, t1[1];
        if (grid_reduce<1, false>(p1, rs, t1) && threadIdx.x == 0) {
            sc->r0v = t1[0];
            if (fabs(t1[0]) < 1.0e-30) { sc->done = 1; sc->status = NSMP_WARN_BREAKDOWN; }
            else sc->alpha = sc->rho / t1[0];
        }
    } else {
        double tot[2];
        if (grid_reduce<2, false>(part, rs, tot) && threadIdx.x == 0) {
            sc->ts = tot[0];
            sc->tt = tot[1];
            sc->omega = tot[0] / tot[1];
        }
    }
}

// update_sk (bicgstab.F90:1007-1041)
__global__ void __launch_bounds__(kBlock) k_bicg_s(Mesh m, KryArgs a, const Scal* sc) {
    pdl_enter();
    if (sc->done) return;
    const double al = sc->alpha;
    const int n2 = m.nprism >> 1;
    const double2* r = reinterpret_cast<const double2*>(a.r);
    const double2* v = reinterpret_cast<const double2*>(a.v);
    double2* s = reinterpret_cast<double2*>(a.s);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
        const double2 rr = r[i], vv = v[i];
        s[i] = make_double2(fma(-al, vv.x, rr.x), fma(-al, vv.y, rr.y));
    }
    if ((m.nprism & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const int g = m.nprism - 1;
        a.s[g] = fma(-al, a.v[g], a.r[g]);
    }
}

// update_xkrk (bicgstab.F90:1047-1111), the next rho = (r0, r) and the
// stopping test of bicgstab.F90:543-566.
__device__ __forceinline__ void xr_one(double id, double al, double om, double p, double s, double t, double r0,
                                       double& x, double& r, double (&part)[3]) {
    x = fma(id, fma(om, s, al * p), x);
    r = fma(-om, t, s);
    part[0] = fma(r, r, part[0]);
    part[1] += fabs(r);
    part[2] = fma(r0, r, part[2]);
}

__global__ void __launch_bounds__(kBlock) k_bicg_x(Mesh m, KryArgs a, RedScratch rs, Scal* sc) {
    pdl_enter();
    if (sc->done) return;
    const double al = sc->alpha, om = sc->omega;
    double part[3] = {0.0, 0.0, 0.0};
    const int n2 = m.nprism >> 1;
    const double2* id2 = reinterpret_cast<const double2*>(a.invD);
    const double2* p2 = reinterpret_cast<const double2*>(a.p);
    const double2* s2 = reinterpret_cast<const double2*>(a.s);
    const double2* t2 = reinterpret_cast<const double2*>(a.t);
    const double2* q2 = reinterpret_cast<const double2*>(a.r0);
    double2* x2 = reinterpret_cast<double2*>(a.x);
    double2* r2 = reinterpret_cast<double2*>(a.r);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += gridDim.x * blockDim.x) {
        const double2 id = id2[i], pp = p2[i], ss = s2[i], tt = t2[i], rq = q2[i];
        double2 xx = x2[i], rr;
        xr_one(id.x, al, om, pp.x, ss.x, tt.x, rq.x, xx.x, rr.x, part);
        xr_one(id.y, al, om, pp.y, ss.y, tt.y, rq.y, xx.y, rr.y, part);
        x2[i] = xx;
        r2[i] = rr;
    }
    if ((m.nprism & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const int g = m.nprism - 1;
        double xx = a.x[g], rr;
        xr_one(a.invD[g], al, om, a.p[g], a.s[g], a.t[g], a.r0[g], xx, rr, part);
        a.x[g] = xx;
        a.r[g] = rr;
    }
    double tot[3];
    if (grid_reduce<3, false>(part, rs, tot) && threadIdx.x == 0) {
        const double r2n = sqrt(tot[0]), r1n = tot[1];
        sc->r1 = r1n; sc->r2 = r2n;
        sc->e2 = r2n / sc->b2;
        sc->e1 = r1n / sc->b1;
        sc->rho_prev = sc->rho;
        sc->rho = tot[2];
        sc->iter = sc->iter + 1;
        double en = 1.0e10;
        if (en > sc->e1) en = sc->e1;
        if (en > sc->e2) en = sc->e2;
        if (!(r2n == r2n)) { sc->status = NSMP_ERR_NAN; sc->done = 1; }
        else if (en < sc->eps) { sc->converged = 1; sc->done = 1; }
        else if (sc->iter > sc->max_iters) { sc->status = NSMP_WARN_MAXITER; sc->done = 1; }
        else if (fabs(sc->rho_prev) < 1.0e-30 || fabs(sc->omega) < 1.0e-30) {
            sc->status = NSMP_WARN_BREAKDOWN; sc->done = 1;
        }
    }
}

}  // namespace

int fp64_setup(nsmp_ctx* c) {
    const Mesh& m = c->mesh;
    k_inv_diag<<<grid_for(c, m.nprism), kBlock, 0, c->stream>>>(m, c->invD);
    CKL("k_inv_diag");
    k_scaled_coefs<<<grid_for(c, m.nprism), kBlock, 0, c->stream>>>(m, c->invD, c->ahat[0], c->ahat[1], c->ahat[2],
                                                                   c->ahat[3], c->ahat[4]);
    CKL("k_scaled_coefs");
    return 0;
}

int run_pressure_fp64(nsmp_ctx* c, const double* pf, const double** x_final) {
    const Mesh& m = c->mesh;
    cudaStream_t st = c->stream;
    KryArgs ka{c->rhsp, pf, c->x, c->r, c->r0, c->pk, c->vk, c->sk, c->tk, c->invD,
               {c->ahat[0], c->ahat[1], c->ahat[2], c->ahat[3], c->ahat[4]}};
    const int g_init = grid_occ(c, k_bicg_init, m.nprism);
    const int g_p = grid_occ(c, k_bicg_p, (m.nprism + 1) / 2);
    const bool mf = c->fp64_spmv_mf != 0;
    const int g_v = mf ? grid_occ(c, k_bicg_spmv_mf<0>, m.nprism) : grid_occ(c, k_bicg_spmv<0>, m.nprism);
    const int g_s = grid_occ(c, k_bicg_s, (m.nprism + 1) / 2);
    const int g_t = mf ? grid_occ(c, k_bicg_spmv_mf<1>, m.nprism) : grid_occ(c, k_bicg_spmv<1>, m.nprism);
    const int g_x = grid_occ(c, k_bicg_x, (m.nprism + 1) / 2);
    LAUNCH(NSMP_K_BICG_INIT, k_bicg_init<<<g_init, kBlock, 0, st>>>(m, ka, c->red, c->d_scal));
    CKL("k_bicg_init");
    // BiCGSTAB iterations, enqueued in chunks; every kernel returns at once
    // after the device-side stopping test has fired.
    int chunk = c->last_iters > 2 ? c->last_iters - 1 : 2;
    int launched = 0;
    for (;;) {
        for (int it = 0; it < chunk; ++it) {
            LAUNCH(NSMP_K_BICG_P, CK(launch_pdl(k_bicg_p, g_p, st, m, ka, c->d_scal)));
            if (mf) LAUNCH(NSMP_K_BICG_SPMV_V, CK(launch_pdl(k_bicg_spmv_mf<0>, g_v, st, m, ka, c->red, c->d_scal)));
            else LAUNCH(NSMP_K_BICG_SPMV_V, CK(launch_pdl(k_bicg_spmv<0>, g_v, st, m, ka, c->red, c->d_scal)));
            LAUNCH(NSMP_K_BICG_S, CK(launch_pdl(k_bicg_s, g_s, st, m, ka, c->d_scal)));
            if (mf) LAUNCH(NSMP_K_BICG_SPMV_T, CK(launch_pdl(k_bicg_spmv_mf<1>, g_t, st, m, ka, c->red, c->d_scal)));
            else LAUNCH(NSMP_K_BICG_SPMV_T, CK(launch_pdl(k_bicg_spmv<1>, g_t, st, m, ka, c->red, c->d_scal)));
            LAUNCH(NSMP_K_BICG_X, CK(launch_pdl(k_bicg_x, g_x, st, m, ka, c->red, c->d_scal)));
        }
        CKL("bicgstab iteration");
        launched += chunk;
        CK(cudaMemcpyAsync(c->h_scal, c->d_scal, sizeof(Scal), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        prof_resolve(c);
        if (c->h_scal->done) break;
        if (launched > c->prm.max_iters + 8) {  // cannot happen: the device test stops at MaxIters
            c->err = "BiCGSTAB did not stop";
            return NSMP_ERR_CUDA;
        }
        chunk = 4;
    }
    *x_final = c->x;
    return 0;
}

}  // namespace nsmp
