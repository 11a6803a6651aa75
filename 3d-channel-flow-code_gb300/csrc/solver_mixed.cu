// Mixed-precision pressure solve (NSMP_MIXED).
//
// The PPE of one stage, A x = b with the reference's 7-point operator
// (PDE.F90:69-121) and stopping test min(|r|_1/|b|_1, |r|_2/|b|_2) < eps
// (bicgstab.F90:543-566) on the FP64 residual, is solved by the reference's
// right-preconditioned Jacobi BiCGSTAB (bicgstab.F90:477-575) run in FP32,
// wrapped in FP64 iterative refinement by reliable updates (Sleijpen and
// van der Vorst 1996; Clark et al. 2010 for mixed precision):
//
//   FP32 BiCGSTAB iterations on A e = r, e accumulated     k_in_pv / k_in_st / k_in_upd
//   when the FP32 residual fell by inner_tol (or after
//   inner_cap iterations):
//     x = x + e,  r = b - A x          FP64, FP64 norms     k_mix_update
//     FP32 r <- r (true residual)       Krylov state kept   k_mix_scale
//
// Replacing the drifting FP32 recursive residual by the FP64 truth, while
// keeping p, v, the shadow residual and rho, lets one Krylov process run to
// 1e-10 instead of restarting (a restarted FP32 cycle gains only about
// log10(1/(eps32 * cond A)) decades on a smooth residual).  FP32 values are
// the FP64 residual divided by its RMS at the start of the solve.
//
// The PPE is singular (periodic + Neumann: A 1 = 0).  Its FP32 copy has an
// eigenvalue of order 1e-7 |A| along the constant vector instead of 0, so the
// FP32 iteration can grow a large constant in e; added to the FP64 x that
// constant costs rounding in A x.  The FP32 residual therefore starts with its
// plain mean removed and e is added with its mean removed (the pressure level
// is fixed afterwards by Glob_Norm anyway).
//
// The two stencil passes fuse the p and s vector updates (evaluated at the
// seven stencil points); dot products are formed per thread in FP32 over the
// thread's few prisms and reduced across threads and blocks in FP64.
#include <algorithm>
#include <cmath>

#include "kern_common.cuh"

namespace nsmp {
namespace {

struct MixArgs {
    const double* rhsp;
    const double* pf;
    double* b;          // mean-removed right-hand side
    double *r64a, *r64b;// FP64 residual, double-buffered with x (index = refinement parity)
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

// Glob_Norm(rhs, 1) (bicgstab.F90:107-109) + x = pf; norms of b.  The
// first k_mix_update then forms the initial residual.
__global__ void __launch_bounds__(kBlock) k_mix_init(Mesh m, MixArgs a, RedScratch rs, Scal* sc) {
    const double avec = sc->sum_rhs / m.tv_lsig;
    double part[2] = {0.0, 0.0};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const double b = a.rhsp[g] - avec * m.ppe[c].area * lev(m, LV_HMEAN, k0);
        a.b[g] = b;
        a.xa[g] = a.pf[cell_of(g, c)];
        part[0] += b * b;
        part[1] += fabs(b);
    }
    double tot[2];
    if (grid_reduce<2, false>(part, rs, tot) && threadIdx.x == 0) {
        double b2 = sqrt(tot[0]), b1 = tot[1];
        if (b2 == 0.0) b2 = 1.0;
        if (b1 == 0.0) b1 = 1.0;
        sc->b1 = b1; sc->b2 = b2;
        sc->iter = 0; sc->status = 0; sc->converged = 0; sc->done = 0; sc->outer = 0;
        sc->iiter = 0; sc->ksince = 0; sc->pending = 1; sc->restart = 1; sc->cur = 0;
        sc->efresh = 1; sc->has_e = 0;
        sc->iscale = 0.0;  // set from the first residual
        sc->r2_upd = INFINITY;
    }
}

// The two stencil passes process two consecutive layers of one column per
// thread (the compact layout and an even layer count make the pair 8-byte
// aligned), so vertical neighbours are shared and column loads are float2.
__device__ __forceinline__ float2 ld2(const float* p, size_t i) { return *reinterpret_cast<const float2*>(p + i); }

// Inner pass 1: p = r + beta (p - omega v) at the stencil points,
// v = A D^-1 p, dot (r0, v).
__global__ void __launch_bounds__(kBlock) k_in_pv(Mesh m, MixArgs a, RedScratch rs, Scal* sc) {
    if (sc->done || sc->pending) return;
    const int it = sc->iiter, nz = m.NZ, NZI = m.NZI;
    const float beta = (float)((sc->irho / sc->irho_prev) * (sc->ialpha / sc->iomega));
    const float om = (float)sc->iomega;
    const float* pin = (it & 1) ? a.p1 : a.p0;
    const float* vin = (it & 1) ? a.v1 : a.v0;
    float* pout = (it & 1) ? a.p0 : a.p1;
    float* vout = (it & 1) ? a.v0 : a.v1;
    const int npair = m.nprism >> 1;
    float acc = 0.f;
    auto pn1 = [&](size_t i) { return (it == 0) ? a.r[i] : fmaf(beta, fmaf(-om, vin[i], pin[i]), a.r[i]); };
    auto y2 = [&](size_t i) {  // y = D^-1 p at layers i, i+1
        const float2 rr = ld2(a.r, i), dd = ld2(a.invD, i);
        if (it == 0) return make_float2(rr.x * dd.x, rr.y * dd.y);
        const float2 pp = ld2(pin, i), vv = ld2(vin, i);
        return make_float2(fmaf(beta, fmaf(-om, vv.x, pp.x), rr.x) * dd.x, fmaf(beta, fmaf(-om, vv.y, pp.y), rr.y) * dd.y);
    };
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < npair; h += gridDim.x * blockDim.x) {
        const int g = 2 * h;
        const int c = g / NZI, kk = g - c * NZI;  // kk even: layers k0 = kk+1, kk+2
        const int k0 = kk + 1;
        const ColPPE32& P = a.ppe32[c];
        const float2 rr = ld2(a.r, g), dd = ld2(a.invD, g);
        float2 p0 = rr;
        if (it != 0) {
            const float2 pp = ld2(pin, g), vv = ld2(vin, g);
            p0 = make_float2(fmaf(beta, fmaf(-om, vv.x, pp.x), rr.x), fmaf(beta, fmaf(-om, vv.y, pp.y), rr.y));
        }
        const float y0a = p0.x * dd.x, y0b = p0.y * dd.y;
        const float yB = (kk > 0) ? pn1(g - 1) * a.invD[g - 1] : 0.f;
        const float yT = (kk + 2 < NZI) ? pn1(g + 2) * a.invD[g + 2] : 0.f;
        const float2 n1 = y2(g + (size_t)(P.nb[0] - c) * NZI);
        const float2 n2 = y2(g + (size_t)(P.nb[1] - c) * NZI);
        const float2 n3 = y2(g + (size_t)(P.nb[2] - c) * NZI);
        const float va = a_row32(a, nz, P, k0, y0a, n1.x, n2.x, n3.x, y0b, yB);
        const float vb = a_row32(a, nz, P, k0 + 1, y0b, n1.y, n2.y, n3.y, yT, y0a);
        *reinterpret_cast<float2*>(pout + g) = p0;
        *reinterpret_cast<float2*>(vout + g) = make_float2(va, vb);
        const float2 q0 = ld2(a.r0, g);
        acc = fmaf(q0.x, va, acc);
        acc = fmaf(q0.y, vb, acc);
    }
    double part[1] = {(double)acc}, tot[1];
    if (grid_reduce<1, false>(part, rs, tot) && threadIdx.x == 0) {
        sc->ir0v = tot[0];
        if (fabs(tot[0]) < 1.0e-30) { sc->pending = 1; sc->restart = 1; }  // breakdown: restart
        else sc->ialpha = sc->irho / tot[0];
    }
}

// Inner pass 2: s = r - alpha v at the stencil points, t = A D^-1 s,
// dots (t, s) and (t, t).
__global__ void __launch_bounds__(kBlock) k_in_st(Mesh m, MixArgs a, RedScratch rs, Scal* sc) {
    if (sc->done || sc->pending) return;
    const int it = sc->iiter, nz = m.NZ, NZI = m.NZI;
    const float al = (float)sc->ialpha;
    const float* v = (it & 1) ? a.v0 : a.v1;
    const int npair = m.nprism >> 1;
    float ts = 0.f, tt = 0.f;
    auto z2 = [&](size_t i) {
        const float2 rr = ld2(a.r, i), vv = ld2(v, i), dd = ld2(a.invD, i);
        return make_float2(fmaf(-al, vv.x, rr.x) * dd.x, fmaf(-al, vv.y, rr.y) * dd.y);
    };
    auto z1 = [&](size_t i) { return fmaf(-al, v[i], a.r[i]) * a.invD[i]; };
    for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < npair; h += gridDim.x * blockDim.x) {
        const int g = 2 * h;
        const int c = g / NZI, kk = g - c * NZI;
        const int k0 = kk + 1;
        const ColPPE32& P = a.ppe32[c];
        const float2 rr = ld2(a.r, g), vv = ld2(v, g), dd = ld2(a.invD, g);
        const float s0a = fmaf(-al, vv.x, rr.x), s0b = fmaf(-al, vv.y, rr.y);
        const float z0a = s0a * dd.x, z0b = s0b * dd.y;
        const float zB = (kk > 0) ? z1(g - 1) : 0.f;
        const float zT = (kk + 2 < NZI) ? z1(g + 2) : 0.f;
        const float2 n1 = z2(g + (size_t)(P.nb[0] - c) * NZI);
        const float2 n2 = z2(g + (size_t)(P.nb[1] - c) * NZI);
        const float2 n3 = z2(g + (size_t)(P.nb[2] - c) * NZI);
        const float ta = a_row32(a, nz, P, k0, z0a, n1.x, n2.x, n3.x, z0b, zB);
        const float tb = a_row32(a, nz, P, k0 + 1, z0b, n1.y, n2.y, n3.y, zT, z0a);
        *reinterpret_cast<float2*>(a.s + g) = make_float2(s0a, s0b);
        *reinterpret_cast<float2*>(a.t + g) = make_float2(ta, tb);
        ts = fmaf(ta, s0a, ts); ts = fmaf(tb, s0b, ts);
        tt = fmaf(ta, ta, tt); tt = fmaf(tb, tb, tt);
    }
    double part[2] = {(double)ts, (double)tt}, tot[2];
    if (grid_reduce<2, false>(part, rs, tot) && threadIdx.x == 0) {
        if (tot[1] > 0.0) sc->iomega = tot[0] / tot[1];
        else { sc->pending = 1; sc->restart = 1; }
    }
}

// Inner pass 3: e += D^-1 (alpha p + omega s), r = s - omega t, norms and
// the next rho; inner stopping test relative to the cycle's start.
__device__ __forceinline__ void upd_one(int fresh, float id, float al, float om, float p, float s, float t, float r0,
                                        float& e, float& r, float& s1, float& s2, float& s3, float& s4) {
    const float de = id * fmaf(om, s, al * p);
    e = fresh ? de : e + de;
    r = fmaf(-om, t, s);
    s1 += fabsf(r);
    s2 = fmaf(r, r, s2);
    s3 = fmaf(r0, r, s3);
    s4 += e;
}

__global__ void __launch_bounds__(kBlock) k_in_upd(Mesh m, MixArgs a, RedScratch rs, Scal* sc) {
    if (sc->done || sc->pending) return;
    const int it = sc->iiter;
    const int fresh = sc->efresh;
    const float al = (float)sc->ialpha, om = (float)sc->iomega;
    const float* p = (it & 1) ? a.p0 : a.p1;
    float s1 = 0.f, s2 = 0.f, s3 = 0.f, s4 = 0.f;
    const int n4 = m.nprism >> 2;
    const float4* id4 = reinterpret_cast<const float4*>(a.invD);
    const float4* p4 = reinterpret_cast<const float4*>(p);
    const float4* sv4 = reinterpret_cast<const float4*>(a.s);
    const float4* t4 = reinterpret_cast<const float4*>(a.t);
    const float4* q4 = reinterpret_cast<const float4*>(a.r0);
    float4* e4 = reinterpret_cast<float4*>(a.e);
    float4* r4 = reinterpret_cast<float4*>(a.r);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        const float4 id = id4[i], pp = p4[i], ss = sv4[i], tt = t4[i], rq = q4[i];
        float4 ee = fresh ? make_float4(0.f, 0.f, 0.f, 0.f) : e4[i], rr;
        upd_one(fresh, id.x, al, om, pp.x, ss.x, tt.x, rq.x, ee.x, rr.x, s1, s2, s3, s4);
        upd_one(fresh, id.y, al, om, pp.y, ss.y, tt.y, rq.y, ee.y, rr.y, s1, s2, s3, s4);
        upd_one(fresh, id.z, al, om, pp.z, ss.z, tt.z, rq.z, ee.z, rr.z, s1, s2, s3, s4);
        upd_one(fresh, id.w, al, om, pp.w, ss.w, tt.w, rq.w, ee.w, rr.w, s1, s2, s3, s4);
        e4[i] = ee;
        r4[i] = rr;
    }
    for (int g = 4 * n4 + blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        float ee = fresh ? 0.f : a.e[g], rr;
        upd_one(fresh, a.invD[g], al, om, p[g], a.s[g], a.t[g], a.r0[g], ee, rr, s1, s2, s3, s4);
        a.e[g] = ee;
        a.r[g] = rr;
    }
    double part[4] = {(double)s1, (double)s2, (double)s3, (double)s4}, tot[4];
    if (grid_reduce<4, false>(part, rs, tot) && threadIdx.x == 0) {
        const double r1 = tot[0], r2 = sqrt(tot[1]);
        sc->ir1 = r1; sc->ir2 = r2;
        sc->emean = tot[3] / (double)m.nprism;
        sc->irho_prev = sc->irho;
        sc->irho = tot[2];
        sc->iiter += 1;
        sc->ksince += 1;
        sc->iter += 1;
        sc->efresh = 0;
        sc->has_e = 1;
        const double rel = fmin(r1 / sc->ib1, r2 / sc->ib2);                  // since the last update
        const double est = fmin(r1 * sc->iscale / sc->b1, r2 * sc->iscale / sc->b2);  // outer estimate
        if (!(r2 == r2)) { sc->pending = 1; sc->restart = 1; sc->has_e = 0; }
        else if (est < sc->eps || rel < sc->inner_tol || sc->ksince >= sc->inner_cap) sc->pending = 1;
        if (sc->pending && sc->iiter >= sc->restart_every) sc->restart = 1;
        else if (sc->iter > sc->max_iters) sc->pending = 1;
        else if (fabs(sc->irho_prev) < 1.0e-30 || fabs(sc->iomega) < 1.0e-30) { sc->pending = 1; sc->restart = 1; }
    }
}

__device__ __forceinline__ bool o_log(int k) { return k >= 0 && k < Scal::kCycLog; }

// FP64 update: x <- x + iscale (e - mean e), r = b - A x, norms, the outer
// stopping test.  Acts only when an update is pending.
__global__ void __launch_bounds__(kBlock) k_mix_update(Mesh m, MixArgs a, RedScratch rs, Scal* sc) {
    if (sc->done || !sc->pending) return;
    const int cur = sc->cur;
    const double scale = sc->has_e ? sc->iscale : 0.0;
    const float em = (float)sc->emean;
    const double* xin = cur ? a.xb : a.xa;
    double* xout = cur ? a.xa : a.xb;
    double* rout = cur ? a.r64a : a.r64b;
    double part[3] = {0.0, 0.0, 0.0};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const ColPPE& P = m.ppe[c];
        const size_t q = g;
        auto xn = [&](size_t i) { return fma(scale, (double)(a.e[i] - em), xin[i]); };
        const double x0 = xn(q);
        const double xT = (k0 < m.NZ - 2) ? xn(q + 1) : 0.0;
        const double xB = (k0 > 1) ? xn(q - 1) : 0.0;
        const double Ax = ppe_row(m, P, k0, x0, xn(ICg(m, P.nb[0], k0)), xn(ICg(m, P.nb[1], k0)),
                                  xn(ICg(m, P.nb[2], k0)), xT, xB);
        const double r = a.b[q] - Ax;
        xout[q] = x0;
        rout[q] = r;
        part[0] += r * r;
        part[1] += fabs(r);
        part[2] += r;
    }
    double tot[3];
    if (grid_reduce<3, false>(part, rs, tot) && threadIdx.x == 0) {
        const double r2 = sqrt(tot[0]), r1 = tot[1];
        if (o_log(sc->outer)) {
            const int k = sc->outer;
            sc->cyc_it[k] = sc->ksince;
            sc->cyc_in[k] = (sc->ib1 > 0.0 && sc->ksince > 0) ? (float)fmin(sc->ir1 / sc->ib1, sc->ir2 / sc->ib2) : 1.f;
            sc->cyc_out[k] = (float)(r2 / sc->b2);
            sc->cyc_acc[k] = sc->restart;
        }
        sc->outer += 1;
        sc->has_e = 0;
        if (!(r2 == r2) || r2 > 2.0 * sc->r2_upd) {
            // the FP32 process diverged: drop this correction (x and r stay in
            // buffer `cur`) and restart the Krylov process from the truth
            sc->restart = 1;
            if (sc->outer >= 2000) { sc->status = NSMP_WARN_BREAKDOWN; sc->done = 1; }
            else if (sc->iter > sc->max_iters) { sc->status = NSMP_WARN_MAXITER; sc->done = 1; }
            return;
        }
        sc->cur = cur ^ 1;
        sc->r1 = r1; sc->r2 = r2;
        sc->e1 = r1 / sc->b1; sc->e2 = r2 / sc->b2;
        sc->rmean = tot[2] / (double)m.nprism;
        if (sc->iscale == 0.0) sc->iscale = (r2 > 0.0) ? r2 / sqrt((double)m.nprism) : 1.0;
        sc->r2_upd = r2;
        double en = 1.0e10;
        if (en > sc->e1) en = sc->e1;
        if (en > sc->e2) en = sc->e2;
        if (!(r2 == r2)) { sc->status = NSMP_ERR_NAN; sc->done = 1; }
        else if (en < sc->eps) { sc->converged = 1; sc->done = 1; }
        else if (sc->iter > sc->max_iters) { sc->status = NSMP_WARN_MAXITER; sc->done = 1; }
        else if (sc->outer >= 2000) { sc->status = NSMP_WARN_BREAKDOWN; sc->done = 1; }
    }
}

// After an FP64 update: FP32 r <- (r - mean r) / iscale, recompute the norms
// the next update is measured against and rho = (r0, r); on a restart also
// r0 = r and a fresh Krylov process.
__global__ void __launch_bounds__(kBlock) k_mix_scale(Mesh m, MixArgs a, RedScratch rs, Scal* sc) {
    if (sc->done || !sc->pending) return;
    const double inv = 1.0 / sc->iscale, rm = sc->rmean;
    const int rst = sc->restart;
    const double* r64 = sc->cur ? a.r64b : a.r64a;
    double part[3] = {0.0, 0.0, 0.0};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        const float rf = (float)((r64[g] - rm) * inv);
        a.r[g] = rf;
        float q0 = rf;
        if (rst) a.r0[g] = rf;
        else q0 = a.r0[g];
        const double rd = (double)rf;
        part[0] += fabs(rd);
        part[1] += rd * rd;
        part[2] += (double)q0 * rd;
    }
    double tot[3];
    if (grid_reduce<3, false>(part, rs, tot) && threadIdx.x == 0) {
        sc->ib1 = (tot[0] > 0.0) ? tot[0] : 1.0;
        sc->ib2 = (tot[1] > 0.0) ? sqrt(tot[1]) : 1.0;
        sc->irho = tot[2];
        if (rst) { sc->irho_prev = 1.0; sc->ialpha = 1.0; sc->iomega = 1.0; sc->iiter = 0; }
        sc->ksince = 0; sc->pending = 0; sc->restart = 0; sc->efresh = 1;
    }
}

__global__ void k_mix_setup(Mesh m, const double* __restrict__ invD, float* __restrict__ invD32) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x)
        invD32[g] = (float)invD[g];
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
    if (m.NZI & 1) {
        c->err = "mixed precision needs an even number of layers";
        return NSMP_ERR_UNSUPPORTED;
    }
    const int g_pv = grid_occ(c, k_in_pv, m.nprism / 2), g_st = grid_occ(c, k_in_st, m.nprism / 2);
    const int g_up = grid_occ(c, k_in_upd, (m.nprism + 3) / 4);
    const int g_in = grid_occ(c, k_mix_init, m.nprism), g_u = grid_occ(c, k_mix_update, m.nprism);
    const int g_sc = grid_occ(c, k_mix_scale, m.nprism);
    MixArgs a{c->rhsp, pf, c->b64, c->r, c->x, c->xa, c->xb, c->r32, c->r032, c->p32[0], c->p32[1], c->v32[0],
              c->v32[1], c->s32, c->t32, c->e32, c->invD32, c->d_ppe32, c->lev32};
    CK(cudaMemcpyAsync(&c->d_scal->inner_tol, &c->inner_tol, sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(&c->d_scal->inner_cap, &c->inner_cap, sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(&c->d_scal->restart_every, &c->restart_every, sizeof(int), cudaMemcpyHostToDevice, st));
    LAUNCH(NSMP_K_BICG_INIT, k_mix_init<<<g_in, kBlock, 0, st>>>(m, a, c->red, c->d_scal));
    LAUNCH(NSMP_K_OTHER, k_mix_update<<<g_u, kBlock, 0, st>>>(m, a, c->red, c->d_scal));
    LAUNCH(NSMP_K_OTHER, k_mix_scale<<<g_sc, kBlock, 0, st>>>(m, a, c->red, c->d_scal));
    CKL("k_mix_init");
    // FP32 iterations in chunks, an FP64 update slot after every few
    // iterations (it only acts when one was requested); the host polls for
    // the FP64 stopping test once per chunk.
    const int per_update = 8;
    int chunk = std::max(per_update, c->last_iters);
    long long launched = 0;
    for (;;) {
        for (int it = 0; it < chunk; it += per_update) {
            for (int j = 0; j < per_update; ++j) {
                LAUNCH(NSMP_K_BICG_SPMV_V, k_in_pv<<<g_pv, kBlock, 0, st>>>(m, a, c->red, c->d_scal));
                LAUNCH(NSMP_K_BICG_SPMV_T, k_in_st<<<g_st, kBlock, 0, st>>>(m, a, c->red, c->d_scal));
                LAUNCH(NSMP_K_BICG_X, k_in_upd<<<g_up, kBlock, 0, st>>>(m, a, c->red, c->d_scal));
            }
            LAUNCH(NSMP_K_OTHER, k_mix_update<<<g_u, kBlock, 0, st>>>(m, a, c->red, c->d_scal));
            LAUNCH(NSMP_K_OTHER, k_mix_scale<<<g_sc, kBlock, 0, st>>>(m, a, c->red, c->d_scal));
        }
        CKL("mixed inner chunk");
        launched += chunk;
        CK(cudaMemcpyAsync(c->h_scal, c->d_scal, sizeof(Scal), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        prof_resolve(c);
        if (c->h_scal->done) break;
        if (launched > 4 * ((long long)c->prm.max_iters + 2000 * 8)) {
            c->err = "mixed solver did not stop";
            return NSMP_ERR_CUDA;
        }
        chunk = 4 * per_update;
    }
    const Scal& s = *c->h_scal;
    c->last_iters = s.iter > 0 ? s.iter : per_update;
    c->last_outer = s.outer;
    *x_final = s.cur ? c->xb : c->xa;
    return 0;
}

}  // namespace nsmp
