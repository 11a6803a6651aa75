// Mixed-precision pressure solve (NSMP_MIXED).
//
// The PPE of one stage, A x = b with the reference's 7-point operator
// (PDE.F90:69-121) and stopping test min(|r|_1/|b|_1, |r|_2/|b|_2) < eps
// (bicgstab.F90:543-566) on the FP64 residual, is solved by the reference's
// right-preconditioned Jacobi BiCGSTAB (bicgstab.F90:477-575) run in FP32,
// wrapped in FP64 iterative refinement by reliable updates (Sleijpen and
// van der Vorst 1996; Clark et al. 2010 for mixed precision):
//
//   FP32 BiCGSTAB iterations on A e = r, e accumulated     k_in_pv / k_in_st
//   when the FP32 residual fell by inner_tol (or after
//   inner_cap iterations):
//     x1 = x + e, r1 = r - A e           FP64 updates, A e   k_mix_update
//                                        double-float FP32
//     x, r <- x + theta (x1 - x), r + theta (r1 - r) with the minimal-residual
//     theta; stopping test on the FP64 norms               k_mix_scale
//     FP32 r <- r (true residual)       Krylov state kept   k_mix_scale
//   convergence is declared only after an update that forms r1 = b - A x1
//   from scratch in FP64 passes the test again.
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
// An iteration is two stencil passes that fuse the vector updates (evaluated
// at the seven stencil points) with the operator; it moves 17 FP32 vectors.
// The p/v pass forms A D^-1 p from the two products already stored (see
// pv_in1), which halves its lateral-neighbour loads.
// Dot products are formed in FP32 per thread and warp and summed across
// warps and blocks in FP64.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>

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
    // The level factors dsigv(k-1), wT/dsig(k), wB/dsig(k-1) of the operator
    // in two layouts.  lev32: three rows of nzp floats indexed by the interior
    // layer kk = k0 - 1, so a thread's L layers are one aligned vector per row
    // (3 loads a group; the s/t pass).  lev4: one float4 per level k0, loaded
    // where each layer's row is formed (fewer live registers; the p/v pass,
    // which runs at its register cap).
    const float* lev32;
    int nzp;
    const float4* lev4;
    // double-float PPE coefficients, two float4 each: per column
    // {kA1 h,l, kA2 h,l}, {kA3 h,l, area h,l}; per level k0
    // {dsigv h,l, aT h,l}, {aB h,l, 0, 0}
    const float4* ddcol;
    const float4* ddlev;
};

// The 32-byte column record as two 16-byte loads.
__device__ __forceinline__ ColPPE32 ld_col(const ColPPE32* p) {
    const int4 q0 = __ldg(reinterpret_cast<const int4*>(p));
    const float4 q1 = __ldg(reinterpret_cast<const float4*>(p) + 1);
    ColPPE32 P;
    P.nb[0] = q0.x; P.nb[1] = q0.y; P.nb[2] = q0.z;
    P.kA[0] = __int_as_float(q0.w); P.kA[1] = q1.x; P.kA[2] = q1.y;
    P.area = q1.z; P.pad = q1.w;
    return P;
}

// FP32 operator row: A y at one prism (same coefficients as ppe_row), from
// the level factors dsv, aT, aB of its layer.
__device__ __forceinline__ float a_row32(const ColPPE32& P, float dsv, float aT, float aB, float y0, float y1, float y2,
                                         float y3, float yT, float yB) {
    const float AA1 = P.kA[0] * dsv, AA2 = P.kA[1] * dsv, AA3 = P.kA[2] * dsv;
    const float AAT = P.area * aT, AAB = P.area * aB;
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
        sc->has_e = 0; sc->einc = 0; sc->rfresh = 1;
        sc->iscale = 0.0;  // set from the first residual
        sc->r2sq = 0.0; sc->rsum = 0.0; sc->theta = 1.0; sc->perturb = 0; sc->verify = 0;
    }
}

// Both passes process L consecutive layers of one column per thread (L = 4
// when the interior layer count allows it, else 2): the compact layout makes
// the group 4L-byte aligned, vertical neighbours inside the group come from
// registers, and every column load is one float4 (float2) per thread.
template <int L>
struct FV {
    float v[L];
    __device__ __forceinline__ float& operator[](int l) { return v[l]; }
    __device__ __forceinline__ float operator[](int l) const { return v[l]; }
};
template <int L>
__device__ __forceinline__ FV<L> ldv(const float* p, size_t i) {
    FV<L> o;
    if constexpr (L == 4) {
        const float4 q = *reinterpret_cast<const float4*>(p + i);
        o.v[0] = q.x; o.v[1] = q.y; o.v[2] = q.z; o.v[3] = q.w;
    } else {
        const float2 q = *reinterpret_cast<const float2*>(p + i);
        o.v[0] = q.x; o.v[1] = q.y;
    }
    return o;
}
template <int L>
__device__ __forceinline__ void stv(float* p, size_t i, const FV<L>& o) {
    if constexpr (L == 4) *reinterpret_cast<float4*>(p + i) = make_float4(o.v[0], o.v[1], o.v[2], o.v[3]);
    else *reinterpret_cast<float2*>(p + i) = make_float2(o.v[0], o.v[1]);
}

// One BiCGSTAB iteration is two passes.  The p/v pass of iteration i carries
// the tail of iteration i-1 (r = s - omega t and the correction increment
// e += D^-1 (alpha p + omega s)) and forms the norms of that r; the s/t pass
// forms the dots from which omega and the next rho follow:
//   rho_new = (r0, s) - omega (r0, t).
// Inputs of the p/v pass by mode:
//   0: first iteration of a Krylov process:  p = r
//   1: first iteration after an FP64 update: p = r + beta (p - omega v), r stored
//   2: otherwise:                            r = s - omega t, p = r + beta (p - omega v)
// The FP32 Krylov vectors are stored scaled by D^-1 (r~ = D^-1 r, p~, v~,
// s~, t~; the shadow residual as r^0 = D r0): a change of variables that
// leaves the right-preconditioned iteration unchanged in exact arithmetic,
// while the operator's input D^-1 p is then p~ itself, so a stencil point
// needs no D^-1 load.  D^-1 is read only at the centre, where v~ = D^-1 A p~
// is formed and the unscaled values the dots need are recovered.
//
// In modes 0 and 1, v~ = M p~ (M = D^-1 A) is formed from p~ at the seven
// stencil points.  In mode 2 the same product follows from the two stored
// ones, M s~ = t~ (s/t pass) and M p~ = v~ (previous p/v pass), by linearity:
//   M p~' = M (s~ - om t~ + beta (p~ - om v~)) = w - om M w,  w = t~ + beta v~,
// so a lateral neighbour contributes two loads (t~, v~) instead of four
// (s~, t~, p~, v~).  The recurrence carries the rounding of the earlier v~
// forward; every FP64 update is followed by a mode-1 pass (mode 0 after a
// restart), which forms M p~ directly again, so the recurrence spans at most
// inner_cap iterations.
template <int MODE>
__device__ __forceinline__ float pv_in1(const MixArgs& a, const float* pin, const float* vin, float beta, float om,
                                        size_t i) {  // operator input at one point: p~ (modes 0, 1) or w (mode 2)
    if (MODE == 0) return a.r[i];
    if (MODE == 2) return fmaf(beta, vin[i], a.t[i]);
    return fmaf(beta, fmaf(-om, vin[i], pin[i]), a.r[i]);
}

template <int MODE, int L>
__device__ __forceinline__ FV<L> pv_in(const MixArgs& a, const float* pin, const float* vin, float beta, float om,
                                       size_t i) {  // the same at layers i .. i+L-1
    FV<L> y;
    if (MODE == 2) {
        const FV<L> tt = ldv<L>(a.t, i), vv = ldv<L>(vin, i);
#pragma unroll
        for (int l = 0; l < L; ++l) y[l] = fmaf(beta, vv[l], tt[l]);
        return y;
    }
    const FV<L> r = ldv<L>(a.r, i);
    if (MODE == 0) return r;
    const FV<L> pp = ldv<L>(pin, i), vv = ldv<L>(vin, i);
#pragma unroll
    for (int l = 0; l < L; ++l) y[l] = fmaf(beta, fmaf(-om, vv[l], pp[l]), r[l]);
    return y;
}

// p/v pass over the thread's layer groups; f = {(r0, v), sum e, sum D^-1 p,
// |r|_1, |r|_2^2} (e and the norms of r only in mode 2, where r is formed).
template <int MODE, int L>
__device__ __forceinline__ void pv_cells(const Mesh& m, const MixArgs& a, int it, float beta, float om, float al,
                                         float (&f)[5]) {
    const int NZI = m.NZI;
    const float* pin = (it & 1) ? a.p1 : a.p0;
    const float* vin = (it & 1) ? a.v1 : a.v0;
    float* pout = (it & 1) ? a.p0 : a.p1;
    float* vout = (it & 1) ? a.v0 : a.v1;
    const int ngrp = m.nprism / L;
    const int lane = threadIdx.x & 31;
    // warp-uniform trip count: the vertical neighbours of a group are the
    // end layers of the adjacent lanes' groups (shuffled, not reloaded).
    // Every load of a group (centre, column ends, lateral neighbours, r^0)
    // is issued before the shuffle and before any store of the group, so all
    // are in flight together; lanes past the end repeat the warp's first
    // group and store nothing.
    for (int hw = blockIdx.x * blockDim.x + (threadIdx.x & ~31); hw < ngrp; hw += gridDim.x * blockDim.x) {
        const int h = hw + lane;
        const bool act = h < ngrp;
        const int g = L * (act ? h : hw);
        const int c = g / NZI, kk = g - c * NZI;  // layers k0 = kk+1 .. kk+L
        const ColPPE32 P = ld_col(a.ppe32 + c);
        const FV<L> dd = ldv<L>(a.invD, g), q0 = ldv<L>(a.r0, g);
        const bool ldT = act && kk + L < NZI && (lane == 31 || h + 1 >= ngrp);
        const bool ldB = act && kk > 0 && lane == 0;
        const float eT = ldT ? pv_in1<MODE>(a, pin, vin, beta, om, g + L) : 0.f;
        const float eB = ldB ? pv_in1<MODE>(a, pin, vin, beta, om, g - 1) : 0.f;
        FV<L> r, p, e, y;  // y: the operator input (p~, or w in mode 2)
        if (MODE == 2) {
            const FV<L> ss = ldv<L>(a.s, g), tt = ldv<L>(a.t, g), pp = ldv<L>(pin, g), vv = ldv<L>(vin, g);
            e = ldv<L>(a.e, g);
#pragma unroll
            for (int l = 0; l < L; ++l) {
                r[l] = fmaf(-om, tt[l], ss[l]);
                p[l] = fmaf(beta, fmaf(-om, vv[l], pp[l]), r[l]);
                y[l] = fmaf(beta, vv[l], tt[l]);
                // increment of the previous iteration: e += D^-1 (alpha p + omega s)
                e[l] = e[l] + fmaf(om, ss[l], al * pp[l]);
            }
        } else {
            r = ldv<L>(a.r, g);
            p = r;
            if (MODE == 1) {
                const FV<L> pp = ldv<L>(pin, g), vv = ldv<L>(vin, g);
#pragma unroll
                for (int l = 0; l < L; ++l) p[l] = fmaf(beta, fmaf(-om, vv[l], pp[l]), r[l]);
            }
            y = p;
        }
        const FV<L> n1 = pv_in<MODE, L>(a, pin, vin, beta, om, g + (size_t)(P.nb[0] - c) * NZI);
        const FV<L> n2 = pv_in<MODE, L>(a, pin, vin, beta, om, g + (size_t)(P.nb[1] - c) * NZI);
        const FV<L> n3 = pv_in<MODE, L>(a, pin, vin, beta, om, g + (size_t)(P.nb[2] - c) * NZI);
        float yT = __shfl_down_sync(0xffffffffu, y[0], 1);
        float yB = __shfl_up_sync(0xffffffffu, y[L - 1], 1);
        if (!act) continue;
        if (kk + L >= NZI) yT = 0.f;
        else if (ldT) yT = eT;
        if (kk == 0) yB = 0.f;
        else if (ldB) yB = eB;
        FV<L> v;
#pragma unroll
        for (int l = 0; l < L; ++l) {
            const float4 q = __ldg(a.lev4 + kk + 1 + l);
            const float my = a_row32(P, q.x, q.y, q.z, y[l], n1[l], n2[l], n3[l], (l + 1 < L) ? y[l + 1] : yT,
                                     (l > 0) ? y[l - 1] : yB) * dd[l];  // M y = D^-1 A y
            v[l] = (MODE == 2) ? fmaf(-om, my, y[l]) : my;                // v~ = M p~
        }
        if (MODE == 2) {
#pragma unroll
            for (int l = 0; l < L; ++l) {
                f[1] += e[l];
                const float ru = r[l] * __frcp_rn(dd[l]);  // unscaled r
                f[3] += fabsf(ru);
                f[4] = fmaf(ru, ru, f[4]);
            }
            stv<L>(a.e, g, e);
            stv<L>(a.r, g, r);
        }
        stv<L>(pout, g, p);
        stv<L>(vout, g, v);
#pragma unroll
        for (int l = 0; l < L; ++l) {
            f[0] = fmaf(q0[l], v[l], f[0]);  // (r0, v) = (r^0, v~)
            f[2] += p[l];
        }
    }
}

// Pass 1: the previous iteration's tail, p update, v = A D^-1 p, (r0, v).
// In mode 2 it also forms the norms of r and takes the hand-over test: when
// it fires, alpha is left as it was, so that the pass repeated after the FP64
// update (mode 1, same iteration index) continues the same Krylov process.
// Three blocks of 256 per SM (80 registers): with the recurrence of mode 2 a
// 64-register cap (four blocks) spills twice as much and runs 16 % slower
// at 6.3M prisms.
template <int L>
__global__ void __launch_bounds__(kBlock, 3) k_in_pv(Mesh m, MixArgs a, RedScratch rs, Scal* sc) {
    pdl_enter();
    if (sc->done || sc->pending) return;
    const int it = sc->iiter;
    const int mode = (it == 0) ? 0 : (sc->rfresh ? 1 : 2);
    const float beta = it ? (float)((sc->irho / sc->irho_prev) * (sc->ialpha / sc->iomega)) : 0.f;
    const float om = (float)sc->iomega, al = (float)sc->ialpha;
    float f[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    if (mode == 2) pv_cells<2, L>(m, a, it, beta, om, al, f);
    else if (mode == 1) pv_cells<1, L>(m, a, it, beta, om, al, f);
    else pv_cells<0, L>(m, a, it, beta, om, al, f);
    double tot[5];
    if (grid_reduce_f<5>(f, rs, tot) && threadIdx.x == 0) {
        sc->ir0v = tot[0];
        sc->ise = tot[1];
        sc->isy = tot[2];
        sc->rfresh = 0;
        sc->einc = 0;
        if (mode == 2) {
            const double r1 = tot[3], r2 = sqrt(tot[4]);
            sc->ir1 = r1; sc->ir2 = r2;
            const double rel = fmin(r1 / sc->ib1, r2 / sc->ib2);                       // since the last update
            const double est = fmin(r1 * sc->iscale / sc->b1, r2 * sc->iscale / sc->b2);  // outer estimate
            if (!(r2 == r2)) { sc->pending = 1; sc->restart = 1; sc->has_e = 0; }
            else if (est < sc->eps || rel < sc->inner_tol) sc->pending = 1;
            if (sc->pending) {
                if (sc->iiter >= sc->restart_every) sc->restart = 1;
                return;
            }
        }
        if (fabs(tot[0]) < 1.0e-30) { sc->pending = 1; sc->restart = 1; }  // breakdown: restart
        else sc->ialpha = sc->irho / tot[0];
    }
}

// Pass 2: s = r - alpha v at the stencil points, t = A D^-1 s, the dots
// (t, s), (t, t), (r0, s), (r0, t) and sum D^-1 s; then omega, the next rho,
// the mean of e after this iteration and the iteration-count tests.  The
// residual tests wait for the next pass, which forms r = s - omega t
// explicitly: |r|^2 = (s, s) - omega (t, s) cancels badly when t is nearly
// parallel to s, as it is for smooth residuals.
template <int L>
__global__ void __launch_bounds__(kBlock) k_in_st(Mesh m, MixArgs a, RedScratch rs, Scal* sc) {
    pdl_enter();
    if (sc->done || sc->pending) return;
    const int it = sc->iiter, NZI = m.NZI;
    const float al = (float)sc->ialpha;
    const float* v = (it & 1) ? a.v0 : a.v1;
    const int ngrp = m.nprism / L;
    float f[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    auto zv = [&](size_t i) {  // s~ = r~ - alpha v~ = D^-1 s
        const FV<L> rr = ldv<L>(a.r, i), vv = ldv<L>(v, i);
        FV<L> z;
#pragma unroll
        for (int l = 0; l < L; ++l) z[l] = fmaf(-al, vv[l], rr[l]);
        return z;
    };
    auto z1 = [&](size_t i) { return fmaf(-al, v[i], a.r[i]); };
    const int lane = threadIdx.x & 31;
    for (int hw = blockIdx.x * blockDim.x + (threadIdx.x & ~31); hw < ngrp; hw += gridDim.x * blockDim.x) {
        const int h = hw + lane;
        const bool act = h < ngrp;
        const int g = L * (act ? h : hw);
        const int c = g / NZI, kk = g - c * NZI;
        // all loads of the group before the shuffle and the stores
        const ColPPE32 P = ld_col(a.ppe32 + c);
        const FV<L> rr = ldv<L>(a.r, g), vv = ldv<L>(v, g), dd = ldv<L>(a.invD, g), q0 = ldv<L>(a.r0, g);
        const FV<L> ls = ldv<L>(a.lev32, kk), lt = ldv<L>(a.lev32, a.nzp + kk), lb = ldv<L>(a.lev32, 2 * a.nzp + kk);
        const bool ldT = act && kk + L < NZI && (lane == 31 || h + 1 >= ngrp);
        const bool ldB = act && kk > 0 && lane == 0;
        const float eT = ldT ? z1(g + L) : 0.f;
        const float eB = ldB ? z1(g - 1) : 0.f;
        const FV<L> n1 = zv(g + (size_t)(P.nb[0] - c) * NZI);
        const FV<L> n2 = zv(g + (size_t)(P.nb[1] - c) * NZI);
        const FV<L> n3 = zv(g + (size_t)(P.nb[2] - c) * NZI);
        FV<L> z0;
#pragma unroll
        for (int l = 0; l < L; ++l) z0[l] = fmaf(-al, vv[l], rr[l]);
        float zT = __shfl_down_sync(0xffffffffu, z0[0], 1);
        float zB = __shfl_up_sync(0xffffffffu, z0[L - 1], 1);
        if (!act) continue;
        if (kk + L >= NZI) zT = 0.f;
        else if (ldT) zT = eT;
        if (kk == 0) zB = 0.f;
        else if (ldB) zB = eB;
        FV<L> t;
#pragma unroll
        for (int l = 0; l < L; ++l)
            t[l] = a_row32(P, ls[l], lt[l], lb[l], z0[l], n1[l], n2[l], n3[l], (l + 1 < L) ? z0[l + 1] : zT,
                           (l > 0) ? z0[l - 1] : zB);
        FV<L> tt;
#pragma unroll
        for (int l = 0; l < L; ++l) tt[l] = t[l] * dd[l];
        stv<L>(a.s, g, z0);
        stv<L>(a.t, g, tt);
#pragma unroll
        for (int l = 0; l < L; ++l) {
            const float su = __fdividef(z0[l], dd[l]);  // unscaled s (2 ulp: it only enters omega)
            f[0] = fmaf(t[l], su, f[0]);       // (t, s)
            f[1] = fmaf(t[l], t[l], f[1]);     // (t, t)
            f[2] = fmaf(q0[l], z0[l], f[2]);   // (r0, s) = (r^0, s~)
            f[3] = fmaf(q0[l], tt[l], f[3]);   // (r0, t) = (r^0, t~)
            f[4] += z0[l];
        }
    }
    double tot[5];
    if (grid_reduce_f<5>(f, rs, tot) && threadIdx.x == 0) {
        const double ts = tot[0], tt = tot[1];
        if (!(tt > 0.0)) {  // t = 0 or not finite: restart from the FP64 truth
            sc->pending = 1; sc->restart = 1; sc->einc = 0;
            if (!(tt == tt)) sc->has_e = 0;
            return;
        }
        const double om = ts / tt;
        sc->iomega = om;
        sc->emean = (sc->ise + sc->ialpha * sc->isy + om * tot[4]) / (double)m.nprism;
        sc->irho_prev = sc->irho;
        sc->irho = tot[2] - om * tot[3];  // (r0, s - omega t)
        sc->iiter += 1;
        sc->ksince += 1;
        sc->iter += 1;
        sc->has_e = 1;
        sc->einc = 1;
        if (!(om == om)) { sc->pending = 1; sc->restart = 1; sc->has_e = 0; sc->einc = 0; }
        else if (sc->ksince >= sc->inner_cap) sc->pending = 1;
        if (sc->pending && sc->iiter >= sc->restart_every) sc->restart = 1;
        else if (sc->iter > sc->max_iters) sc->pending = 1;
        else if (fabs(sc->irho_prev) < 1.0e-30 || fabs(om) < 1.0e-30) { sc->pending = 1; sc->restart = 1; }
    }
}

// FP64 update, first half: x1 = x + iscale (e - mean e) and r1 = b - A x1
// into the buffers not holding the current x and r.  The correction is taken
// whole (theta = 1, which keeps the FP32 Krylov state consistent with the
// new residual) unless it raised |r|_2 more than 2x.  Then the FP32 process
// went astray: the step is cut to the minimal-residual length
//   theta = argmin |r + theta (r1 - r)|_2 = (r, r - r1) / |r - r1|^2 in [0, 1]
// and the Krylov process restarts with a perturbed shadow residual.  (Simply
// dropping the correction and restarting from the same residual would retrace
// the same FP32 iterations, deterministically, forever.)
__global__ void __launch_bounds__(kBlock) k_mix_update(Mesh m, MixArgs a, RedScratch rs, Scal* sc) {
    pdl_enter();
    if (sc->done || !sc->pending) return;
    const int cur = sc->cur;
    const int has_e = sc->has_e;
    const int first = (sc->iscale == 0.0);
    const int full = first || sc->verify;
    const int einc = has_e && sc->einc;
    const double scale = sc->iscale;
    const float em = (float)sc->emean;
    const float al = (float)sc->ialpha, om = (float)sc->iomega;
    const float* pl = (sc->iiter & 1) ? a.p1 : a.p0;  // p of the last iteration
    const double* xin = cur ? a.xb : a.xa;
    const double* rin = cur ? a.r64b : a.r64a;
    double* xout = cur ? a.xa : a.xb;
    double* rout = cur ? a.r64a : a.r64b;
    double part[3] = {0.0, 0.0, 0.0};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const ColPPE& P = m.ppe[c];
        const size_t q = g;
        double x0, r;
        if (full) {  // b - A x from scratch: the initial residual, or the check of a converged one
            x0 = xin[q];
            const double xT = (k0 < m.NZ - 2) ? xin[q + 1] : 0.0;
            const double xB = (k0 > 1) ? xin[q - 1] : 0.0;
            r = a.b[q] - ppe_row(m, P, k0, x0, xin[ICg(m, P.nb[0], k0)], xin[ICg(m, P.nb[1], k0)],
                                 xin[ICg(m, P.nb[2], k0)], xT, xB);
        } else if (!has_e) {
            x0 = xin[q];
            r = rin[q];
        } else {
            // x1 = x + iscale c with c = e - mean e exactly as stored (FP32),
            // and r1 = r - iscale A c from the differences of c (A 1 = 0): the
            // residual of the stored x1.  A c is formed in double-float FP32
            // arithmetic (about 2^-44 relative): the differences are exact
            // (TwoSum) and the coefficients are hi/lo splits of the FP64
            // ones, so FP64 is left with the x and r updates and the norms
            // (about 9 FP64 instructions a prism instead of 28).
            auto cf = [&](size_t i) {
                float e = a.e[i];
                if (einc) e = e + fmaf(om, a.s[i], al * pl[i]);  // D^-1 (alpha p + omega s)
                return e - em;
            };
            const float c0 = cf(q);
            const F2 zero = {0.f, 0.f};
            const F2 dT = (k0 < m.NZ - 2) ? two_sum(cf(q + 1), -c0) : zero;
            const F2 dB = (k0 > 1) ? two_sum(cf(q - 1), -c0) : zero;
            const F2 d1 = two_sum(cf(ICg(m, P.nb[0], k0)), -c0), d2 = two_sum(cf(ICg(m, P.nb[1], k0)), -c0),
                     d3 = two_sum(cf(ICg(m, P.nb[2], k0)), -c0);
            const float4 ca = __ldg(a.ddcol + 2 * c), cb = __ldg(a.ddcol + 2 * c + 1);
            const float4 la = __ldg(a.ddlev + 2 * k0), lb = __ldg(a.ddlev + 2 * k0 + 1);
            F2 hz = df_add(df_add(df_mul({ca.x, ca.y}, d1), df_mul({ca.z, ca.w}, d2)), df_mul({cb.x, cb.y}, d3));
            hz = df_mul({la.x, la.y}, hz);
            F2 vt = df_add(df_mul({la.z, la.w}, dT), df_mul({lb.x, lb.y}, dB));
            vt = df_mul({cb.z, cb.w}, vt);
            const F2 Ac = df_add(hz, vt);
            x0 = fma(scale, (double)c0, xin[q]);
            r = fma(-scale, (double)Ac.h + (double)Ac.l, rin[q]);
        }
        xout[q] = x0;
        rout[q] = r;
        part[0] += r * r;
        part[1] += r;
        if (!first && has_e) part[2] += rin[q] * r;
    }
    double tot[3];
    if (grid_reduce<3, false>(part, rs, tot) && threadIdx.x == 0) {
        const double R1 = tot[0], C = tot[2], R0 = sc->r2sq;
        double theta = 1.0;
        if (!(R1 == R1)) {  // non-finite correction: drop it
            theta = 0.0;
            sc->restart = 1; sc->perturb = 1;
        } else if (!first && has_e && R1 > 4.0 * R0) {
            const double dd = R0 - 2.0 * C + R1, num = R0 - C;
            theta = (dd > 0.0) ? num / dd : 0.0;
            theta = fmin(fmax(theta, 0.0), 1.0);
            sc->restart = 1; sc->perturb = 1;
        }
        sc->theta = theta;
        if (first) sc->iscale = (R1 > 0.0) ? sqrt(R1 / (double)m.nprism) : 1.0;
        const double sum1 = (R1 == R1) ? tot[1] : 0.0;
        sc->rmean = ((1.0 - theta) * sc->rsum + theta * sum1) / (double)m.nprism;
        const int k = sc->outer % Scal::kCycLog;  // ring buffer of the last updates
        sc->cyc_it[k] = sc->ksince;
        sc->cyc_in[k] = (sc->ib1 > 0.0 && sc->ksince > 0 && sc->ir1 >= 0.0)
                            ? (float)fmin(sc->ir1 / sc->ib1, sc->ir2 / sc->ib2) : 1.f;
        sc->outer += 1;
        sc->has_e = 0;
        sc->einc = 0;
    }
}

// Cheap hash in [-1, 1) of a prism index and the update count: the shadow
// residual of a Krylov restart after a stalled cycle is perturbed by it so
// the next cycle does not retrace the stalled one.
__device__ __forceinline__ float shadow_jitter(unsigned int g, unsigned int k) {
    unsigned int h = g * 2654435761u ^ (k * 40503u + 0x9e3779b9u);
    h ^= h >> 15; h *= 0x2c1b3c6du; h ^= h >> 12; h *= 0x297a2d39u; h ^= h >> 15;
    return (float)(h & 0xffffu) * (1.0f / 32768.0f) - 1.0f;
}

// FP64 update, second half: x, r <- x + theta (x1 - x), r + theta (r1 - r)
// (only when theta != 1), the outer stopping test on that residual, and the
// FP32 residual (r - mean r) / iscale with e <- 0, the norms the next update
// is measured against and rho = (r0, r).  On a restart also r0 = r and a
// fresh Krylov process.
__global__ void __launch_bounds__(kBlock) k_mix_scale(Mesh m, MixArgs a, RedScratch rs, Scal* sc) {
    pdl_enter();
    if (sc->done || !sc->pending) return;
    const int cur = sc->cur;
    const double th = sc->theta;
    const int blend = (th != 1.0);
    const double inv = 1.0 / sc->iscale, rm = sc->rmean;
    const double* xo = cur ? a.xb : a.xa;
    const double* ro = cur ? a.r64b : a.r64a;
    double* xn = cur ? a.xa : a.xb;
    double* rn = cur ? a.r64a : a.r64b;
    // the FP64 residual's norms for the stopping test and the next update are
    // taken from its FP32 image r = iscale (rf + rm / iscale), to FP32
    // accuracy, so the pass costs three FP64 instructions a prism
    const float rmi = (float)(rm * inv);
    // the shadow residual of the next FP32 cycle and rho = (r0, r) are formed
    // in the same pass; they take effect only if no check of b - A x is
    // pending (see the end), and a pending check rewrites them from the
    // checked residual before the next FP32 iteration
    const int rst = sc->restart, jit = sc->perturb;
    const unsigned int salt = (unsigned int)sc->outer;
    float part[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    auto fp64_r = [&](int g) {  // the new FP64 residual, blended when theta != 1
        double r = rn[g];
        if (blend) {
            r = fma(th, r - ro[g], ro[g]);
            rn[g] = r;
            xn[g] = fma(th, xn[g] - xo[g], xo[g]);
        }
        return r;
    };
    // one prism: r~ = D^-1 (r - mean r) / iscale, r^0 on a restart, partials
    auto one = [&](int g, double r, float id, float q0in, float& rt, float& q0out) {
        const float rf = (float)((r - rm) * inv);
        rt = rf * id;  // r~ = D^-1 r
        if (rst) {  // restart: r^0 = D r0 with r0 = r, perturbed after a stalled cycle
            const float d = __frcp_rn(id);
            const float ru = rt * d;
            const float q0 = jit ? ru * (1.0f + 0.5f * shadow_jitter((unsigned int)g, salt)) : ru;
            q0out = q0 * d;
            part[5] = fmaf(q0, ru, part[5]);
        } else {
            part[5] = fmaf(q0in, rt, part[5]);  // (r0, r) = (r^0, r~)
        }
        const float ra = rf + rmi;
        part[0] += fabsf(ra);
        part[1] = fmaf(ra, ra, part[1]);
        part[2] += ra;
        part[3] += fabsf(rf);
        part[4] = fmaf(rf, rf, part[4]);
    };
    // four prisms a thread with 16- and 32-byte loads (the pass is latency-
    // bound with one prism a thread), then the remainder one by one
    const int n4 = m.nprism >> 2;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        const int g = 4 * i;
        double r[4];
        if (blend) {
#pragma unroll
            for (int l = 0; l < 4; ++l) r[l] = fp64_r(g + l);
        } else {
            const double2 r01 = reinterpret_cast<const double2*>(rn)[2 * i];
            const double2 r23 = reinterpret_cast<const double2*>(rn)[2 * i + 1];
            r[0] = r01.x; r[1] = r01.y; r[2] = r23.x; r[3] = r23.y;
        }
        const float4 id = reinterpret_cast<const float4*>(a.invD)[i];
        const float4 qi = rst ? make_float4(0.f, 0.f, 0.f, 0.f) : reinterpret_cast<const float4*>(a.r0)[i];
        float4 rt, qo;
        one(g, r[0], id.x, qi.x, rt.x, qo.x);
        one(g + 1, r[1], id.y, qi.y, rt.y, qo.y);
        one(g + 2, r[2], id.z, qi.z, rt.z, qo.z);
        one(g + 3, r[3], id.w, qi.w, rt.w, qo.w);
        reinterpret_cast<float4*>(a.r)[i] = rt;
        reinterpret_cast<float4*>(a.e)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (rst) reinterpret_cast<float4*>(a.r0)[i] = qo;
    }
    for (int g = 4 * n4 + blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        float rt, qo = 0.f;
        one(g, fp64_r(g), a.invD[g], rst ? 0.f : a.r0[g], rt, qo);
        a.r[g] = rt;
        a.e[g] = 0.f;
        if (rst) a.r0[g] = qo;
    }
    double tot[6];
    if (grid_reduce_f<6>(part, rs, tot) && threadIdx.x == 0) {
        const double is = sc->iscale;
        const double r1 = is * tot[0], r2 = is * sqrt(tot[1]);
        const int k = (sc->outer - 1) % Scal::kCycLog;
        sc->cyc_out[k] = (float)(r2 / sc->b2);
        sc->cur = cur ^ 1;
        sc->r1 = r1; sc->r2 = r2;
        sc->r2sq = is * is * tot[1];
        sc->rsum = is * tot[2];
        sc->e1 = r1 / sc->b1; sc->e2 = r2 / sc->b2;
        sc->cyc_acc[k] = (th == 1.0 ? 1 : 0) | (sc->restart ? 2 : 0);
        sc->ib1 = (tot[3] > 0.0) ? tot[3] : 1.0;
        sc->ib2 = (tot[4] > 0.0) ? sqrt(tot[4]) : 1.0;
        const double en = fmin(sc->e1, sc->e2);
        // the incremental residual drifts from b - A x by FP64 rounding over
        // the updates: when it passes the test, the next update recomputes
        // b - A x from scratch and the test is taken again on that
        if (!(r2 == r2)) { sc->status = NSMP_ERR_NAN; sc->done = 1; }
        else if (en < sc->eps && sc->verify) { sc->converged = 1; sc->done = 1; }
        else if (en < sc->eps) { sc->verify = 1; }
        else if (sc->iter > sc->max_iters) { sc->status = NSMP_WARN_MAXITER; sc->done = 1; }
        else if (sc->outer >= 2000) { sc->status = NSMP_WARN_BREAKDOWN; sc->done = 1; }
        if (!(en < sc->eps)) sc->verify = 0;
        // the next FP32 cycle starts from this residual unless the solve
        // ended or a check of b - A x is pending
        if (!sc->done && !sc->verify) {
            sc->irho = tot[5];
            if (rst) { sc->irho_prev = 1.0; sc->ialpha = 1.0; sc->iomega = 1.0; sc->iiter = 0; }
            sc->ksince = 0; sc->pending = 0; sc->restart = 0; sc->perturb = 0; sc->rfresh = 1; sc->einc = 0;
        }
    }
}

__global__ void k_mix_setup(Mesh m, const double* __restrict__ invD, float* __restrict__ invD32) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x)
        invD32[g] = (float)invD[g];
}

}  // namespace

// Offset of the shadow residual in the block that starts with D^-1: both are
// loaded as float4 at 4-aligned compact indices, so r^0 starts on a 16-byte
// boundary.
static size_t r0_offset(size_t nprism) { return (nprism + 3) / 4 * 4; }

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
    for (float** p : {&c->r32, &c->p32[0], &c->p32[1], &c->v32[0], &c->v32[1], &c->s32, &c->t32, &c->e32})
        CK(dalloc((void**)p, ncf * sizeof(float)));
    // D^-1 and the shadow residual are read by both passes of every
    // iteration and never written inside a Krylov process: one block, so a
    // single L2 access-policy window can keep them resident
    const size_t np = (size_t)L.N0 * (L.NZ - 2);
    CK(dalloc((void**)&c->invD32, (r0_offset(np) + np) * sizeof(float)));
    c->r032 = c->invD32 + r0_offset(np);
    CK(dalloc((void**)&c->d_ppe32, sizeof(ColPPE32) * L.N0));
    const int nzp = (L.NZ - 2 + 3) / 4 * 4;  // interior layers, rounded up to a float4
    CK(dalloc((void**)&c->lev32, sizeof(float) * (3 * nzp + 4 * (size_t)L.NZ)));
    std::vector<ColPPE32> p32(L.N0);
    for (int q = 0; q < L.N0; ++q) {
        for (int j = 0; j < 3; ++j) {
            p32[q].nb[j] = L.ppe[q].nb[j];
            p32[q].kA[j] = (float)L.ppe[q].kA[j];
        }
        p32[q].area = (float)L.ppe[q].area;
        p32[q].pad = 0.f;
    }
    // rows indexed by the interior layer k0 - 1, then one float4 per level k0
    std::vector<float> lv(3 * (size_t)nzp + 4 * (size_t)L.NZ, 0.f);
    float* l4 = lv.data() + 3 * nzp;
    for (int k = 1; k <= L.NZ - 2; ++k) {
        const float f[3] = {(float)L.lev.dsv[k], (float)(L.lev.idsT[k] * L.lev.wT[k]),
                            (float)(L.lev.idsB[k] * L.lev.wB[k])};
        for (int j = 0; j < 3; ++j) {
            lv[j * nzp + k - 1] = f[j];
            l4[4 * k + j] = f[j];
        }
    }
    // double-float splits v = hi + lo of the FP64 coefficients (the values the
    // FP64 operator uses), hi = fl32(v), lo = fl32(v - hi)
    auto split = [](double v, float* out) {
        out[0] = (float)v;
        out[1] = (float)(v - (double)out[0]);
    };
    std::vector<float> dc(8 * (size_t)L.N0, 0.f), dl(8 * (size_t)L.NZ, 0.f);
    for (int q = 0; q < L.N0; ++q) {
        for (int j = 0; j < 3; ++j) split(L.ppe[q].kA[j], &dc[8 * (size_t)q + 2 * j]);
        split(L.ppe[q].area, &dc[8 * (size_t)q + 6]);
    }
    for (int k = 0; k < L.NZ; ++k) {
        split(L.lev.dsv[k], &dl[8 * (size_t)k]);
        split(L.lev.idsT[k] * L.lev.wT[k], &dl[8 * (size_t)k + 2]);
        split(L.lev.idsB[k] * L.lev.wB[k], &dl[8 * (size_t)k + 4]);
    }
    CK(dalloc((void**)&c->ddcol, sizeof(float) * dc.size()));
    CK(dalloc((void**)&c->ddlev, sizeof(float) * dl.size()));
    CK(cudaMemcpyAsync(c->ddcol, dc.data(), sizeof(float) * dc.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->ddlev, dl.data(), sizeof(float) * dl.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_ppe32, p32.data(), sizeof(ColPPE32) * L.N0, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->lev32, lv.data(), sizeof(float) * lv.size(), cudaMemcpyHostToDevice, c->stream));
    k_mix_setup<<<grid_for(c, (long long)ncf), kBlock, 0, c->stream>>>(c->mesh, c->invD, c->invD32);
    CKL("k_mix_setup");
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

// The persisting-L2 set-aside is a limit of the whole CUDA context on a
// device, shared by every nsmp_ctx there and by the caller.  The first
// context that raises it records the value it had; the last such context to
// be destroyed puts that value back.
namespace {
struct L2Limit {
    int users = 0;
    size_t before = 0;
};
std::mutex g_l2_mu;
std::map<int, L2Limit> g_l2;
}  // namespace

static bool l2_limit_raise(nsmp_ctx* c, size_t want) {
    std::lock_guard<std::mutex> lk(g_l2_mu);
    L2Limit& L = g_l2[c->device];
    size_t cur = 0;
    if (cudaDeviceGetLimit(&cur, cudaLimitPersistingL2CacheSize) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (cur >= want) return true;
    if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (!c->l2_limit_set) {
        if (L.users == 0) L.before = cur;
        L.users += 1;
        c->l2_limit_set = 1;
    }
    return true;
}

void l2_limit_release(nsmp_ctx* c) {
    if (!c->l2_limit_set) return;
    std::lock_guard<std::mutex> lk(g_l2_mu);
    L2Limit& L = g_l2[c->device];
    c->l2_limit_set = 0;
    if (--L.users > 0) return;
    cudaCtxResetPersistingL2Cache();
    cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, L.before);
    cudaGetLastError();
}

// L2 residency of D^-1 and r0 (the contiguous block of mixed_alloc) for the
// kernels of one mixed solve, only when the whole block fits the persisting
// set-aside the device allows.  A partial window (hit ratio below 1) on a
// block larger than that carves persisting lines out of the L2 that the
// neighbour gathers of both passes rely on: at 33.5M prisms (a 268 MB block)
// it made the FP32 iteration 1.8x slower.  The destructor returns the stream
// to normal use and resets the persisting lines of the CUDA context
// (cudaCtxResetPersistingL2Cache), which also demotes persisting lines that
// the caller's own streams may have set.
struct L2Window {
    nsmp_ctx* c;
    bool on = false;
    L2Window(nsmp_ctx* cc, size_t bytes) : c(cc) {
        int dev = 0, maxwin = 0, maxpers = 0;
        if (cudaGetDevice(&dev) != cudaSuccess) return;
        cudaDeviceGetAttribute(&maxwin, cudaDevAttrMaxAccessPolicyWindowSize, dev);
        cudaDeviceGetAttribute(&maxpers, cudaDevAttrMaxPersistingL2CacheSize, dev);
        if (maxwin <= 0 || maxpers <= 0) return;
        if (bytes > (size_t)maxwin || bytes > (size_t)maxpers) return;
        const size_t win = bytes;
        size_t lim = 0;
        if (cudaDeviceGetLimit(&lim, cudaLimitPersistingL2CacheSize) != cudaSuccess) return;
        if (lim < std::min(win, (size_t)maxpers) && !l2_limit_raise(c, std::min(win, (size_t)maxpers))) return;
        cudaDeviceGetLimit(&lim, cudaLimitPersistingL2CacheSize);
        cudaStreamAttrValue v{};
        v.accessPolicyWindow.base_ptr = c->invD32;
        v.accessPolicyWindow.num_bytes = win;
        v.accessPolicyWindow.hitRatio = (float)std::min(1.0, (double)lim / (double)win);
        v.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
        v.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
        on = cudaStreamSetAttribute(c->stream, cudaStreamAttributeAccessPolicyWindow, &v) == cudaSuccess;
        cudaGetLastError();  // an unsupported window is not an error of the solve
    }
    ~L2Window() {
        if (!on) return;
        cudaStreamAttrValue v{};
        v.accessPolicyWindow.num_bytes = 0;
        cudaStreamSetAttribute(c->stream, cudaStreamAttributeAccessPolicyWindow, &v);
        cudaCtxResetPersistingL2Cache();
        cudaGetLastError();
    }
};

int run_pressure_mixed(nsmp_ctx* c, const double* pf, const double** x_final) {
    const Mesh& m = c->mesh;
    cudaStream_t st = c->stream;
    L2Window l2win(c, (r0_offset((size_t)m.nprism) + (size_t)m.nprism) * sizeof(float));
    if (m.NZI & 1) {
        c->err = "mixed precision needs an even number of layers";
        return NSMP_ERR_UNSUPPORTED;
    }
    // four layers per thread when the interior layer count allows it
    const bool quad = (m.NZI % 4) == 0;
    const int L = quad ? 4 : 2;
    const int g_pv = quad ? grid_occ(c, k_in_pv<4>, m.nprism / L) : grid_occ(c, k_in_pv<2>, m.nprism / L);
    const int g_st = quad ? grid_occ(c, k_in_st<4>, m.nprism / L) : grid_occ(c, k_in_st<2>, m.nprism / L);
    const int g_in = grid_occ(c, k_mix_init, m.nprism), g_u = grid_occ(c, k_mix_update, m.nprism);
    const int g_sc = grid_occ(c, k_mix_scale, (m.nprism + 3) / 4);
    MixArgs a{c->rhsp, pf, c->b64, c->r, c->x, c->xa, c->xb, c->r32, c->r032, c->p32[0], c->p32[1], c->v32[0],
              c->v32[1], c->s32, c->t32, c->e32, c->invD32, c->d_ppe32, c->lev32,
              (m.NZI + 3) / 4 * 4, reinterpret_cast<const float4*>(c->lev32 + 3 * ((m.NZI + 3) / 4 * 4)),
              reinterpret_cast<const float4*>(c->ddcol), reinterpret_cast<const float4*>(c->ddlev)};
    CK(cudaMemcpyAsync(&c->d_scal->inner_tol, &c->inner_tol, sizeof(double), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(&c->d_scal->inner_cap, &c->inner_cap, sizeof(int), cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(&c->d_scal->restart_every, &c->restart_every, sizeof(int), cudaMemcpyHostToDevice, st));
    LAUNCH(NSMP_K_BICG_INIT, k_mix_init<<<g_in, kBlock, 0, st>>>(m, a, c->red, c->d_scal));
    LAUNCH(NSMP_K_MIX_UPDATE, CK(launch_pdl(k_mix_update, g_u, st, m, a, c->red, c->d_scal)));
    LAUNCH(NSMP_K_MIX_SCALE, CK(launch_pdl(k_mix_scale, g_sc, st, m, a, c->red, c->d_scal)));
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
                if (quad) {
                    LAUNCH(NSMP_K_IN_PV, CK(launch_pdl(k_in_pv<4>, g_pv, st, m, a, c->red, c->d_scal)));
                    LAUNCH(NSMP_K_IN_ST, CK(launch_pdl(k_in_st<4>, g_st, st, m, a, c->red, c->d_scal)));
                } else {
                    LAUNCH(NSMP_K_IN_PV, CK(launch_pdl(k_in_pv<2>, g_pv, st, m, a, c->red, c->d_scal)));
                    LAUNCH(NSMP_K_IN_ST, CK(launch_pdl(k_in_st<2>, g_st, st, m, a, c->red, c->d_scal)));
                }
            }
            LAUNCH(NSMP_K_MIX_UPDATE, CK(launch_pdl(k_mix_update, g_u, st, m, a, c->red, c->d_scal)));
            LAUNCH(NSMP_K_MIX_SCALE, CK(launch_pdl(k_mix_scale, g_sc, st, m, a, c->red, c->d_scal)));
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
