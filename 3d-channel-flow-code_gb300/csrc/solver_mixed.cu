// Mixed-precision pressure solve (NSMP_MIXED).
//
// The PPE of one stage, A x = b with the reference's 7-point operator
// (PDE.F90:69-121) and stopping test min(|r|_1/|b|_1, |r|_2/|b|_2) < eps
// (bicgstab.F90:543-566), is solved by FP64 iterative refinement:
//
//   r = b - A x               FP64 operator, FP64 norms       k_mix_refine
//   solve A e = r             FP32 Jacobi-BiCGSTAB to 1e-4    k_in_pv / k_in_st / k_in_upd
//   x = x + e                 FP64 accumulation               k_mix_refine
//
// The inner solver is the reference's right-preconditioned BiCGSTAB
// (bicgstab.F90:477-575) with FP32 vectors and a matrix-free FP32 operator.
// Its passes are fused: the p update is evaluated at the seven stencil points
// inside the first SpMV, the s update inside the second, so one inner
// iteration is three passes.  Dot products are formed per thread in FP32
// over the thread's few prisms and reduced across threads and blocks in FP64.
#include <algorithm>
#include <cmath>

#include "kern_common.cuh"

namespace nsmp {
namespace {

struct MixArgs {
    const double* rhsp;
    const double* pf;
    double* b;          // mean-removed right-hand side
    double *xa, *xb;    // FP64 iterate, double-buffered across refinements
    float *r, *r0, *p0, *p1, *v0, *v1, *s, *t, *e;
    const float* invD;
    const ColPPE32* ppe32;
    const float* lev32; // rows: dsigv(k-1), wT/dsig(k), wB/dsig(k-1)
};

__device__ __forceinline__ float lv32(const MixArgs& a, int nz, int row, int k0) { return __ldg(a.lev32 + row * nz + k0); }

// FP32 operator row: A y at one prism (same coefficients as ppe_row).
__device__ __forceinline__ float a_row32(const MixArgs& a, int nz, const ColPPE32& P, int k0, float y0, float y1,
                                         float y2, float y3, float yT, float yB) {
    const float dsv = lv32(a, nz, 0, k0);
    const float AA1 = P.kA[0] * dsv, AA2 = P.kA[1] * dsv, AA3 = P.kA[2] * dsv;
    const float AAT = P.area * lv32(a, nz, 1, k0), AAB = P.area * lv32(a, nz, 2, k0);
    const float AA0 = -(AAT + AAB + AA1 + AA2 + AA3);
    return AA0 * y0 + AA1 * y1 + AA2 * y2 + AA3 * y3 + AAT * yT + AAB * yB;
}

// Glob_Norm(rhs, 1) + x = pf + FP64 residual and norms; seeds the first
// inner solve with r32 = r.
__global__ void __launch_bounds__(kBlock) k_mix_init(Mesh m, MixArgs a, RedScratch rs, Scal* sc) {
    const double avec = sc->sum_rhs / m.tv_lsig;
    double part[4] = {0.0, 0.0, 0.0, 0.0};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const ColPPE& P = m.ppe[c];
        const size_t q = IX(m, c, k0);
        const double b = a.rhsp[q] - avec * P.area * lev(m, LV_HMEAN, k0);
        const double x0 = a.pf[q];
        const double Ax = ppe_row(m, P, k0, x0, a.pf[IX(m, P.nb[0], k0)], a.pf[IX(m, P.nb[1], k0)],
                                  a.pf[IX(m, P.nb[2], k0)], a.pf[q + 1], a.pf[q - 1]);
        const double r = b - Ax;
        a.b[q] = b;
        a.xa[q] = x0;
        const float rf = (float)r;
        a.r[q] = rf;
        a.r0[q] = rf;
        part[0] += b * b; part[1] += r * r; part[2] += fabs(b); part[3] += fabs(r);
    }
    double tot[4];
    if (grid_reduce<4, false>(part, rs, tot) && threadIdx.x == 0) {
        double b2 = sqrt(tot[0]), r2 = sqrt(tot[1]), b1 = tot[2], r1 = tot[3];
        if (b2 == 0.0) b2 = 1.0;
        if (b1 == 0.0) b1 = 1.0;
        sc->b1 = b1; sc->b2 = b2; sc->r1 = r1; sc->r2 = r2;
        sc->e1 = r1 / b1; sc->e2 = r2 / b2;
        sc->iter = 0; sc->status = 0; sc->converged = 0; sc->done = 0; sc->outer = 0;
        sc->ib1 = (r1 > 0.0) ? r1 : 1.0; sc->ib2 = (r2 > 0.0) ? r2 : 1.0;
        sc->irho = tot[1]; sc->irho_prev = 1.0; sc->ialpha = 1.0; sc->iomega = 1.0;
        sc->iiter = 0; sc->idone = 0;
        if (!(r2 == r2)) { sc->status = NSMP_ERR_NAN; sc->done = 1; }
        else if (sc->e1 < sc->eps || sc->e2 < sc->eps) { sc->converged = 1; sc->done = 1; }
    }
}

// Inner pass 1: p = r + beta (p - omega v) at the stencil points,
// v = A D^-1 p, dot (r0, v).
__global__ void __launch_bounds__(kBlock) k_in_pv(Mesh m, MixArgs a, RedScratch rs, Scal* sc) {
    if (sc->done || sc->idone) return;
    const int it = sc->iiter, nz = m.NZ;
    const float beta = (float)((sc->irho / sc->irho_prev) * (sc->ialpha / sc->iomega));
    const float om = (float)sc->iomega;
    const float* pin = (it & 1) ? a.p1 : a.p0;
    const float* vin = (it & 1) ? a.v1 : a.v0;
    float* pout = (it & 1) ? a.p0 : a.p1;
    float* vout = (it & 1) ? a.v0 : a.v1;
    float acc = 0.f;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const ColPPE32& P = a.ppe32[c];
        const size_t q = IX(m, c, k0);
        auto pn = [&](size_t i) { return (it == 0) ? a.r[i] : fmaf(beta, fmaf(-om, vin[i], pin[i]), a.r[i]); };
        auto y = [&](size_t i) { return pn(i) * a.invD[i]; };
        const float p0 = pn(q);
        const float y0 = p0 * a.invD[q];
        const float yT = (k0 < nz - 2) ? y(q + 1) : 0.f;
        const float yB = (k0 > 1) ? y(q - 1) : 0.f;
        const float v = a_row32(a, nz, P, k0, y0, y(IX(m, P.nb[0], k0)), y(IX(m, P.nb[1], k0)),
                                y(IX(m, P.nb[2], k0)), yT, yB);
        pout[q] = p0;
        vout[q] = v;
        acc = fmaf(a.r0[q], v, acc);
    }
    double part[1] = {(double)acc}, tot[1];
    if (grid_reduce<1, false>(part, rs, tot) && threadIdx.x == 0) {
        sc->ir0v = tot[0];
        if (fabs(tot[0]) < 1.0e-30) sc->idone = 1;  // breakdown: restart from the FP64 residual
        else sc->ialpha = sc->irho / tot[0];
    }
}

// Inner pass 2: s = r - alpha v at the stencil points, t = A D^-1 s,
// dots (t, s) and (t, t).
__global__ void __launch_bounds__(kBlock) k_in_st(Mesh m, MixArgs a, RedScratch rs, Scal* sc) {
    if (sc->done || sc->idone) return;
    const int it = sc->iiter, nz = m.NZ;
    const float al = (float)sc->ialpha;
    const float* v = (it & 1) ? a.v0 : a.v1;
    float ts = 0.f, tt = 0.f;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const ColPPE32& P = a.ppe32[c];
        const size_t q = IX(m, c, k0);
        auto sn = [&](size_t i) { return fmaf(-al, v[i], a.r[i]); };
        auto z = [&](size_t i) { return sn(i) * a.invD[i]; };
        const float s0 = sn(q);
        const float zT = (k0 < nz - 2) ? z(q + 1) : 0.f;
        const float zB = (k0 > 1) ? z(q - 1) : 0.f;
        const float t = a_row32(a, nz, P, k0, s0 * a.invD[q], z(IX(m, P.nb[0], k0)), z(IX(m, P.nb[1], k0)),
                                z(IX(m, P.nb[2], k0)), zT, zB);
        a.s[q] = s0;
        a.t[q] = t;
        ts = fmaf(t, s0, ts);
        tt = fmaf(t, t, tt);
    }
    double part[2] = {(double)ts, (double)tt}, tot[2];
    if (grid_reduce<2, false>(part, rs, tot) && threadIdx.x == 0) {
        if (tot[1] > 0.0) sc->iomega = tot[0] / tot[1];
        else sc->idone = 1;
    }
}

// Inner pass 3: e += D^-1 (alpha p + omega s), r = s - omega t, norms and
// the next rho; inner stopping test relative to the refinement residual.
__global__ void __launch_bounds__(kBlock) k_in_upd(Mesh m, MixArgs a, RedScratch rs, Scal* sc) {
    if (sc->done || sc->idone) return;
    const int it = sc->iiter;
    const float al = (float)sc->ialpha, om = (float)sc->iomega;
    const float* p = (it & 1) ? a.p0 : a.p1;
    float s1 = 0.f, s2 = 0.f, s3 = 0.f;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const size_t q = IX(m, c, k0);
        const float sv = a.s[q];
        const float de = a.invD[q] * fmaf(om, sv, al * p[q]);
        a.e[q] = (it == 0) ? de : a.e[q] + de;
        const float rn = fmaf(-om, a.t[q], sv);
        a.r[q] = rn;
        s1 += fabsf(rn);
        s2 = fmaf(rn, rn, s2);
        s3 = fmaf(a.r0[q], rn, s3);
    }
    double part[3] = {(double)s1, (double)s2, (double)s3}, tot[3];
    if (grid_reduce<3, false>(part, rs, tot) && threadIdx.x == 0) {
        const double r1 = tot[0], r2 = sqrt(tot[1]);
        sc->ir1 = r1; sc->ir2 = r2;
        sc->irho_prev = sc->irho;
        sc->irho = tot[2];
        sc->iiter += 1;
        sc->iter += 1;
        const double en = fmin(r1 / sc->ib1, r2 / sc->ib2);
        if (!(r2 == r2)) { sc->status = NSMP_ERR_NAN; sc->done = 1; }
        else if (en < sc->inner_tol) sc->idone = 1;
        else if (sc->iter > sc->max_iters) sc->idone = 1;
        else if (fabs(sc->irho_prev) < 1.0e-30 || fabs(sc->iomega) < 1.0e-30) sc->idone = 1;
    }
}

// Refinement: x <- x + e, r = b - A x in FP64, norms and the outer test;
// restarts the inner solver from r.  Acts only after an inner solve ended.
__global__ void __launch_bounds__(kBlock) k_mix_refine(Mesh m, MixArgs a, RedScratch rs, Scal* sc) {
    if (sc->done || !sc->idone) return;
    const int o = sc->outer;
    // an inner solve that broke down before its first update left e stale
    const float use_e = (sc->iiter > 0) ? 1.f : 0.f;
    const double* xin = (o & 1) ? a.xb : a.xa;
    double* xout = (o & 1) ? a.xa : a.xb;
    double part[3] = {0.0, 0.0, 0.0};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const ColPPE& P = m.ppe[c];
        const size_t q = IX(m, c, k0);
        auto xn = [&](size_t i) { return xin[i] + (double)(use_e * a.e[i]); };
        const double x0 = xn(q);
        const double xT = (k0 < m.NZ - 2) ? xn(q + 1) : 0.0;
        const double xB = (k0 > 1) ? xn(q - 1) : 0.0;
        const double Ax = ppe_row(m, P, k0, x0, xn(IX(m, P.nb[0], k0)), xn(IX(m, P.nb[1], k0)),
                                  xn(IX(m, P.nb[2], k0)), xT, xB);
        const double r = a.b[q] - Ax;
        xout[q] = x0;
        const float rf = (float)r;
        a.r[q] = rf;
        a.r0[q] = rf;
        part[0] += r * r;
        part[1] += fabs(r);
        part[2] += (double)rf * (double)rf;
    }
    double tot[3];
    if (grid_reduce<3, false>(part, rs, tot) && threadIdx.x == 0) {
        const double r2 = sqrt(tot[0]), r1 = tot[1];
        sc->r1 = r1; sc->r2 = r2;
        sc->e1 = r1 / sc->b1; sc->e2 = r2 / sc->b2;
        sc->outer = o + 1;
        double en = 1.0e10;
        if (en > sc->e1) en = sc->e1;
        if (en > sc->e2) en = sc->e2;
        if (!(r2 == r2)) { sc->status = NSMP_ERR_NAN; sc->done = 1; }
        else if (en < sc->eps) { sc->converged = 1; sc->done = 1; }
        else if (sc->iter > sc->max_iters) { sc->status = NSMP_WARN_MAXITER; sc->done = 1; }
        else if (o + 1 >= 200) { sc->status = NSMP_WARN_BREAKDOWN; sc->done = 1; }
        else {
            sc->ib1 = (r1 > 0.0) ? r1 : 1.0; sc->ib2 = (r2 > 0.0) ? r2 : 1.0;
            sc->irho = tot[2]; sc->irho_prev = 1.0; sc->ialpha = 1.0; sc->iomega = 1.0;
            sc->iiter = 0; sc->idone = 0;
        }
    }
}

__global__ void k_mix_setup(Mesh m, const double* __restrict__ invD, float* __restrict__ invD32) {
    const size_t n = (size_t)m.N0 * m.NZ;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        invD32[i] = (float)invD[i];
}

}  // namespace

int mixed_alloc(nsmp_ctx* c) {
    const HostLayout& L = c->L;
    const size_t ncf = (size_t)L.N0 * L.NZ;
    auto dalloc = [&](void** p, size_t bytes) -> cudaError_t {
        cudaError_t e = cudaMalloc(p, bytes > 0 ? bytes : 16);
        if (e == cudaSuccess) {
            c->allocs.push_back(*p);
            e = cudaMemsetAsync(*p, 0, bytes, c->stream);
        }
        return e;
    };
    for (double** p : {&c->b64, &c->xa, &c->xb}) CK(dalloc((void**)p, ncf * sizeof(double)));
    for (float** p : {&c->r32, &c->r032, &c->p32[0], &c->p32[1], &c->v32[0], &c->v32[1], &c->s32, &c->t32,
                      &c->e32, &c->invD32})
        CK(dalloc((void**)p, ncf * sizeof(float)));
    CK(dalloc((void**)&c->d_ppe32, sizeof(ColPPE32) * L.N0));
    CK(dalloc((void**)&c->lev32, sizeof(float) * 3 * L.NZ));
    std::vector<ColPPE32> p32(L.N0);
    for (int q = 0; q < L.N0; ++q) {
        for (int j = 0; j < 3; ++j) {
            p32[q].nb[j] = L.ppe[q].nb[j];
            p32[q].kA[j] = (float)L.ppe[q].kA[j];
        }
        p32[q].area = (float)L.ppe[q].area;
        p32[q].pad = 0.f;
    }
    std::vector<float> lv(3 * (size_t)L.NZ, 0.f);
    for (int k = 1; k <= L.NZ - 2; ++k) {
        lv[k] = (float)L.lev.dsv[k];
        lv[L.NZ + k] = (float)(L.lev.idsT[k] * L.lev.wT[k]);
        lv[2 * L.NZ + k] = (float)(L.lev.idsB[k] * L.lev.wB[k]);
    }
    CK(cudaMemcpyAsync(c->d_ppe32, p32.data(), sizeof(ColPPE32) * L.N0, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->lev32, lv.data(), sizeof(float) * lv.size(), cudaMemcpyHostToDevice, c->stream));
    k_mix_setup<<<grid_for(c, (long long)ncf), kBlock, 0, c->stream>>>(c->mesh, c->invD, c->invD32);
    CKL("k_mix_setup");
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

int run_pressure_mixed(nsmp_ctx* c, const double* pf, const double** x_final) {
    const Mesh& m = c->mesh;
    cudaStream_t st = c->stream;
    const int gp = grid_for(c, m.nprism);
    MixArgs a{c->rhsp, pf, c->b64, c->xa, c->xb, c->r32, c->r032, c->p32[0], c->p32[1], c->v32[0], c->v32[1],
              c->s32, c->t32, c->e32, c->invD32, c->d_ppe32, c->lev32};
    // inner tolerance lives in the scalars
    CK(cudaMemcpyAsync(&c->d_scal->inner_tol, &c->inner_tol, sizeof(double), cudaMemcpyHostToDevice, st));
    LAUNCH(NSMP_K_BICG_INIT, k_mix_init<<<gp, kBlock, 0, st>>>(m, a, c->red, c->d_scal));
    CKL("k_mix_init");
    int chunk = c->last_inner_chunk > 4 ? c->last_inner_chunk : 4;
    long long launched = 0;
    int seen_outer = 0;
    for (;;) {
        for (int it = 0; it < chunk; ++it) {
            LAUNCH(NSMP_K_BICG_SPMV_V, k_in_pv<<<gp, kBlock, 0, st>>>(m, a, c->red, c->d_scal));
            LAUNCH(NSMP_K_BICG_SPMV_T, k_in_st<<<gp, kBlock, 0, st>>>(m, a, c->red, c->d_scal));
            LAUNCH(NSMP_K_BICG_X, k_in_upd<<<gp, kBlock, 0, st>>>(m, a, c->red, c->d_scal));
        }
        LAUNCH(NSMP_K_OTHER, k_mix_refine<<<gp, kBlock, 0, st>>>(m, a, c->red, c->d_scal));
        CKL("mixed inner chunk");
        launched += chunk;
        CK(cudaMemcpyAsync(c->h_scal, c->d_scal, sizeof(Scal), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        prof_resolve(c);
        if (c->h_scal->done) break;
        if (launched > (long long)c->prm.max_iters + 400) {
            c->err = "mixed solver did not stop";
            return NSMP_ERR_CUDA;
        }
        // a refinement started a new inner solve: enqueue about as many
        // iterations as the last one took; otherwise top up in small chunks
        if (c->h_scal->outer != seen_outer) {
            seen_outer = c->h_scal->outer;
            chunk = std::max(4, c->h_scal->iter / std::max(1, seen_outer) - 2);
        } else {
            chunk = 8;
        }
    }
    const Scal& s = *c->h_scal;
    if (s.outer > 0) c->last_inner_chunk = (int)(s.iter / s.outer);
    c->last_outer = s.outer;
    *x_final = (s.outer & 1) ? c->xb : c->xa;
    return 0;
}

}  // namespace nsmp
