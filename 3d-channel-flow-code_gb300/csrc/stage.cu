// FP64 kernels of one hydro() stage (Main/hydro.F90:197-478) and their
// orchestration.  Thread mapping of every per-prism kernel: one thread per
// interior prism (column c, layer k0), layer fastest, so the loads of a warp
// along a column and along each neighbour column are contiguous.
//
// Kernel list of a stage (fused passes, dead reference work dropped):
//   k_vertex4      cell -> vertex (tagdir 2) of u, v, w and p      BC.F90:202-363
//   k_stage_rhs    Smagorinsky nu_t + Kim-Choi advection/diffusion
//                  + Euler/AB2 predictor + wall ghosts of u*       hydro.F90:258-342
//   k_faces_div    face normal velocities, divergence/dt, PPE
//                  cross-diffusion RHS, sum for Glob_Norm          source3D.F90:92-127,255-288
//   k_bicg_init    mean removal, x = pf, r = b - A x, norms        bicgstab.F90:107-451
//   k_bicg_{p,v,s,t,x}  one BiCGSTAB iteration, dots fused         bicgstab.F90:477-575
//   k_pmean        volume mean of the solution                     bicgstab.F90:598-666
//   k_vertex1      cell -> vertex of the corrected pressure        newu3D.F90:119
//   k_project      LSQ grad p, u = u* - dt grad p, face fluxes      hydro.F90:420-466, newu3D.F90:119-239
#include <cmath>
#include <cstdio>

#include "kern_common.cuh"

namespace nsmp {
namespace {

// ---------------------------------------------------------------------------
// Vertex interpolation: interpolation2D (interpolation2D.F90:120-135) with
// the periodic averaging of bc_periodic (BC.F90:1243-1300) folded into one
// stencil per vertex class; tagdir 2 keeps the value at the cell layer.
// ---------------------------------------------------------------------------
template <int NF>
__global__ void __launch_bounds__(kBlock) k_vertex(Mesh m, const double* __restrict__ f0,
                                                   const double* __restrict__ f1, const double* __restrict__ f2,
                                                   const double* __restrict__ f3, double* __restrict__ o0,
                                                   double* __restrict__ o1, double* __restrict__ o2,
                                                   double* __restrict__ o3, double shift) {
    const int n = m.nclass * m.NZI;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) {
        const int v = g / m.NZI, k0 = 1 + (g - v * m.NZI);
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
        const int s1 = __ldg(m.vptr + v + 1);
        for (int s = __ldg(m.vptr + v); s < s1; ++s) {
            const double w = __ldg(m.vcoef + s);
            const size_t q = IX(m, __ldg(m.vcell + s), k0);
            a0 += w * (f0[q] - shift);
            if (NF > 1) a1 += w * f1[q];
            if (NF > 2) a2 += w * f2[q];
            if (NF > 3) a3 += w * f3[q];
        }
        const size_t o = IV(m, v, k0);
        o0[o] = a0;
        if (NF > 1) o1[o] = a1;
        if (NF > 2) o2[o] = a2;
        if (NF > 3) o3[o] = a3;
    }
}

struct StageArgs {
    const double *u, *v, *w;            // known level (ghost layers valid)
    const double *uv, *vv, *wv;         // vertex values, tagdir 2
    const double *f1, *f2, *f3, *fT, *fB; // face fluxes U?FACE
    double *hu, *hv, *hw;               // AB2 history in/out
    double *us, *vs, *ws;               // predictor out
    double* eddy;
    const double* fx;                   // body force on u per cell, or null
    double c1, c2, dt, inv_re, bdx, bdy, bdz;
    int les, les_van;
};

// The arithmetic type R of the stage right-hand side: FP64 (the plain form)
// or FP32 (the mixed form's flux, gradient and Smagorinsky arithmetic).  Its
// column and level tables come in the same type; the state, the predictor
// update and the AB2 history stay FP64 either way.
template <typename R>
struct StageTables;
template <>
struct StageTables<double> {
    static __device__ __forceinline__ const ColGeo& col(const Mesh& m, int c) { return m.geo[c]; }
    static __device__ __forceinline__ double lv(const Mesh& m, int row, int k0) { return lev(m, row, k0); }
};
template <>
struct StageTables<float> {
    static __device__ __forceinline__ const ColGeo32& col(const Mesh& m, int c) { return m.geo32[c]; }
    static __device__ __forceinline__ float lv(const Mesh& m, int row, int k0) {
        return __ldg(m.levf + row * m.NZ + k0);
    }
};

// Kim-Choi face value (interpolationFace.F90:85-111).
template <typename R>
__device__ __forceinline__ R face_val(R phi, R phinb, R kE, R fa, R fb) {
    return phinb * R(0.5) + phi * R(0.5) + kE * (fb - fa);
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_stage_rhs(Mesh m, StageArgs a, RedScratch rs, Scal* sc) {
    using T = StageTables<R>;
    const R half = R(0.5);
    double emax[1] = {0.0};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const auto& G = T::col(m, c);
        const size_t q = IX(m, c, k0);
        const R dsv = T::lv(m, LV_DSV, k0), idsT = T::lv(m, LV_IDST, k0), idsB = T::lv(m, LV_IDSB, k0);
        const double u64 = a.u[q], v64 = a.v[q], w64 = a.w[q];
        const R u = R(u64), v = R(v64), w = R(w64);
        const R uT = R(a.u[q + 1]), vT = R(a.v[q + 1]), wT = R(a.w[q + 1]);
        const R uB = R(a.u[q - 1]), vB = R(a.v[q - 1]), wB = R(a.w[q - 1]);
        R unb[3], vnb[3], wnb[3], fu[3], fv[3], fw[3];
        int nb[3], vx[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            nb[j] = G.nb[j];
            vx[j] = G.vtx[j];
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const size_t qn = IX(m, nb[j], k0);
            unb[j] = R(a.u[qn]); vnb[j] = R(a.v[qn]); wnb[j] = R(a.w[qn]);
            const size_t qv = IV(m, vx[j], k0);
            fu[j] = R(a.uv[qv]); fv[j] = R(a.vv[qv]); fw[j] = R(a.wv[qv]);
        }
        // face values of the three components (advection and LES gradient)
        R Uf[3], Vf[3], Wf[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int jj = (j + 1) % 3;
            Uf[j] = face_val<R>(u, unb[j], G.kE[j], fu[j], fu[jj]);
            Vf[j] = face_val<R>(v, vnb[j], G.kE[j], fv[j], fv[jj]);
            Wf[j] = face_val<R>(w, wnb[j], G.kE[j], fw[j], fw[jj]);
        }
        const R UT = half * (u + uT), UB = half * (u + uB);
        const R VT = half * (v + vT), VB = half * (v + vB);
        const R WT = half * (w + wT), WB = half * (w + wB);
        // Smagorinsky eddy viscosity (sgm_les.F90:208-250 with fvm_gradient
        // sgm_les.F90:437-473 and van Driest/Mason damping sgdamp)
        R gam = R(a.inv_re), nut = R(0);
        if (a.les) {
            R dudx = 0, dudy = 0, dvdx = 0, dvdy = 0, dwdx = 0, dwdy = 0;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                dudx += Uf[j] * G.lxu[j]; dudy += Uf[j] * G.lyu[j];
                dvdx += Vf[j] * G.lxv[j]; dvdy += Vf[j] * G.lyv[j];
                dwdx += Wf[j] * G.lxu[j]; dwdy += Wf[j] * G.lyu[j];
            }
            const R ihz = T::lv(m, LV_IHZ, k0);
            const R dudz = (UT - UB) * ihz, dvdz = (VT - VB) * ihz, dwdz = (WT - WB) * ihz;
            const R sxy = half * (dudy + dvdx), sxz = half * (dudz + dwdx), syz = half * (dvdz + dwdy);
            const R sij = sqrt(R(2) * (dudx * dudx + dvdy * dvdy + dwdz * dwdz) +
                               R(4) * (sxy * sxy + sxz * sxz + syz * syz));
            const R dd = G.cbrt_area * T::lv(m, LV_DD, k0);
            R lw = T::lv(m, LV_KD, k0), l2;
            if (a.les_van) {
                if (lw > dd) lw = dd;
                const R l = lw * T::lv(m, LV_DAMP, k0);
                l2 = l * l;
            } else {
                l2 = R(1) / (R(1) / (dd * dd) + R(1) / (lw * lw));
            }
            nut = l2 * sij;
            gam = nut + R(a.inv_re);
            emax[0] = fmax(emax[0], double(nut));
        }
        // diffusion (diffusion3D.F90:110-191; the dle3 term is identically 0)
        R su = 0, sv = 0, sw = 0;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int jj = (j + 1) % 3;
            su += (unb[j] - u) * G.kA[j] + (fu[jj] - fu[j]) * G.dle2[j];
            sv += (vnb[j] - v) * G.kA[j] + (fv[jj] - fv[j]) * G.dle2[j];
            sw += (wnb[j] - w) * G.kA[j] + (fw[jj] - fw[j]) * G.dle2[j];
        }
        const R ar = G.area;
        su = su * dsv + ((uT - u) * idsT + (uB - u) * idsB) * ar;
        sv = sv * dsv + ((vT - v) * idsT + (vB - v) * idsB) * ar;
        sw = sw * dsv + ((wT - w) * idsT + (wB - w) * idsB) * ar;
        // advection (advection3D.F90:112-284)
        const R F1 = R(a.f1[q]) * G.L[0] * dsv, F2 = R(a.f2[q]) * G.L[1] * dsv, F3 = R(a.f3[q]) * G.L[2] * dsv;
        const R FT = R(a.fT[q]) * ar, FB = R(a.fB[q]) * ar;
        const R au = Uf[0] * F1 + Uf[1] * F2 + Uf[2] * F3 + UT * FT + UB * FB;
        const R av = Vf[0] * F1 + Vf[1] * F2 + Vf[2] * F3 + VT * FT + VB * FB;
        const R aw = Wf[0] * F1 + Wf[1] * F2 + Wf[2] * F3 + WT * FT + WB * FB;
        const R ivol = G.inv_area * T::lv(m, LV_IDSV, k0);
        const double bu = a.fx ? a.bdx + a.fx[q] : a.bdx;
        double ru, rv, rw;
        if constexpr (sizeof(R) == sizeof(double)) {  // the reference's order: rhs = b + diffusion - advection
            ru = bu + gam * su * ivol - au * ivol;
            rv = a.bdy + gam * sv * ivol - av * ivol;
            rw = a.bdz + gam * sw * ivol - aw * ivol;
        } else {  // the O(1) forcing is added in FP64 to the FP32 flux balance
            ru = bu + double(gam * su * ivol - au * ivol);
            rv = a.bdy + double(gam * sv * ivol - av * ivol);
            rw = a.bdz + double(gam * sw * ivol - aw * ivol);
        }
        // predictor (hydro.F90:322-333), FP64
        double pu = a.c1 * ru, pv = a.c1 * rv, pw = a.c1 * rw;
        if (a.c2 != 0.0) {
            pu += a.c2 * a.hu[q];
            pv += a.c2 * a.hv[q];
            pw += a.c2 * a.hw[q];
        }
        const double us = u64 + a.dt * pu, vs = v64 + a.dt * pv, ws = w64 + a.dt * pw;
        a.us[q] = us; a.vs[q] = vs; a.ws[q] = ws;
        a.hu[q] = ru; a.hv[q] = rv; a.hw[q] = rw;
        if (a.les) a.eddy[q] = double(nut);
        // wall ghost layers (BCvelcenter3D, BC.F90:459-527; BCpcenter for nu_t)
        if (k0 == 1) {
            a.us[q - 1] = m.sgn_bot[0] * us; a.vs[q - 1] = m.sgn_bot[1] * vs; a.ws[q - 1] = m.sgn_bot[2] * ws;
            if (a.les) a.eddy[q - 1] = double(nut);
        }
        if (k0 == m.NZ - 2) {
            a.us[q + 1] = m.sgn_top[0] * us; a.vs[q + 1] = m.sgn_top[1] * vs; a.ws[q + 1] = m.sgn_top[2] * ws;
            if (a.les) a.eddy[q + 1] = double(nut);
        }
    }
    if (a.les) {
        double tot[1];
        if (grid_reduce<1, true>(emax, rs, tot) && threadIdx.x == 0) sc->max_eddy = tot[0];
    }
}

struct FaceArgs {
    const double *us, *vs, *ws;
    const double* pv;                 // vertex pressure (tagdir 2 of pf)
    double *f1, *f2, *f3, *fT, *fB;
    double* rhsp;
    double inv_dt;
    int with_div;
};

// interpolateU (interpolationU.F90:122-160) + source3D divergence
// (source3D.F90:105-127) + rhsp/dt (hydro.F90:365-373) + update_rhsp
// (source3D.F90:255-288).
__global__ void __launch_bounds__(kBlock) k_faces_div(Mesh m, FaceArgs a, RedScratch rs, Scal* sc) {
    double part[1] = {0.0};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const ColGeo& G = m.geo[c];
        const size_t q = IX(m, c, k0);
        const double u = a.us[q], v = a.vs[q], w = a.ws[q];
        double U[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const size_t qn = IX(m, G.nb[j], k0);
            U[j] = (0.5 * (u + a.us[qn])) * G.xn[j] + (0.5 * (v + a.vs[qn])) * G.yn[j];
        }
        const double UT = 0.5 * (w + a.ws[q + 1]);
        const double UB = -1.0 * (0.5 * (w + a.ws[q - 1]));
        a.f1[q] = U[0]; a.f2[q] = U[1]; a.f3[q] = U[2]; a.fT[q] = UT; a.fB[q] = UB;
        if (a.with_div) {
            const double dsv = lev(m, LV_DSV, k0);
            double div = 0.0;
            div = div + U[0] * G.L[0] * dsv;
            div = div + U[1] * G.L[1] * dsv;
            div = div + U[2] * G.L[2] * dsv;
            div = div + UT * G.area;
            div = div + UB * G.area;
            double r = div * a.inv_dt;
            double src = 0.0;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const double pa = a.pv[IV(m, G.vtx[j], k0)], pb = a.pv[IV(m, G.vtx[(j + 1) % 3], k0)];
                src += (pb - pa) * G.dle2[j];
            }
            r = r - src * dsv;
            a.rhsp[g] = r;
            part[0] += r;
        }
    }
    if (a.with_div) {
        double tot[1];
        if (grid_reduce<1, false>(part, rs, tot) && threadIdx.x == 0) sc->sum_rhs = tot[0];
    }
}

// Glob_Norm(phi, 0) sum (bicgstab.F90:617-640)
__global__ void __launch_bounds__(kBlock) k_pmean(Mesh m, const double* __restrict__ x, RedScratch rs, Scal* sc) {
    double part[1] = {0.0};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        part[0] += x[g] * (m.ppe[c].area * lev(m, LV_HMEAN, k0));
    }
    double tot[1];
    if (grid_reduce<1, false>(part, rs, tot) && threadIdx.x == 0) sc->avec_p = tot[0] / m.tv_lsig;
}

__global__ void k_vertex1(Mesh m, const double* __restrict__ x, const Scal* sc, double* __restrict__ pv) {
    const double sh = sc->avec_p;
    const int n = m.nclass * m.NZI;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) {
        const int v = g / m.NZI, k0 = 1 + (g - v * m.NZI);
        double acc = 0.0;
        const int s1 = __ldg(m.vptr + v + 1);
        for (int s = __ldg(m.vptr + v); s < s1; ++s) acc += __ldg(m.vcoef + s) * (x[ICg(m, __ldg(m.vcell + s), k0)] - sh);
        pv[IV(m, v, k0)] = acc;
    }
}

struct ProjArgs {
    const double* x;      // BiCGSTAB solution before mean removal
    const double* pv;     // vertex pressure of the corrected solution
    const double *us, *vs, *ws;
    double *f1, *f2, *f3, *fT, *fB;
    double *un, *vn, *wn, *pn;
    double dt;
};

// gradientP(pfnp) (gradientLSM.F90:153-188) + cell correction
// (hydro.F90:440-448) + newu3D face correction (newu3D.F90:119-239).
__global__ void __launch_bounds__(kBlock) k_project(Mesh m, ProjArgs a, const Scal* sc) {
    const double avec = sc->avec_p;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const ColGeo& G = m.geo[c];
        const size_t q = IX(m, c, k0);
        const double p = a.x[g] - avec;
        // wall ghost layers of p are Neumann copies (BCpcenter, BC.F90:869-888)
        const double pT = (k0 < m.NZ - 2) ? a.x[g + 1] - avec : p;
        const double pB = (k0 > 1) ? a.x[g - 1] - avec : p;
        double dpdx = 0.0, dpdy = 0.0, dn[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const double pn = a.x[ICg(m, G.nb[j], k0)] - avec;
            const double d = pn - p;
            dpdx += G.gx[j] * d;
            dpdy += G.gy[j] * d;
            const double va = a.pv[IV(m, G.vtx[j], k0)], vb = a.pv[IV(m, G.vtx[(j + 1) % 3], k0)];
            dn[j] = d * G.cA[j] + (vb - va) * G.cB[j];
        }
        const double dpds = (pT - p) * lev(m, LV_GZP, k0) + (pB - p) * lev(m, LV_GZM, k0);
        const double un = a.us[q] - a.dt * dpdx, vn = a.vs[q] - a.dt * dpdy, wn = a.ws[q] - a.dt * dpds;
        a.un[q] = un; a.vn[q] = vn; a.wn[q] = wn; a.pn[q] = p;
        if (k0 == 1) {
            a.un[q - 1] = m.sgn_bot[0] * un; a.vn[q - 1] = m.sgn_bot[1] * vn; a.wn[q - 1] = m.sgn_bot[2] * wn;
            a.pn[q - 1] = p;
        }
        if (k0 == m.NZ - 2) {
            a.un[q + 1] = m.sgn_top[0] * un; a.vn[q + 1] = m.sgn_top[1] * vn; a.wn[q + 1] = m.sgn_top[2] * wn;
            a.pn[q + 1] = p;
        }
        const double dT = (pT - p) * lev(m, LV_IDST, k0);
        const double dB = (pB - p) * lev(m, LV_IDSBU, k0);
        a.f1[q] = a.f1[q] - dn[0] * a.dt;
        a.f2[q] = a.f2[q] - dn[1] * a.dt;
        a.f3[q] = a.f3[q] - dn[2] * a.dt;
        a.fT[q] = a.fT[q] - dT * a.dt;
        a.fB[q] = a.fB[q] - dB * a.dt;
    }
}

// Wall ghost layers of a level from its first/last interior layers
// (BCvelcenter3D/BCpcenter vertical parts).
__global__ void k_fill_ghosts(Mesh m, double* u, double* v, double* w, double* p) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m.N0; c += gridDim.x * blockDim.x) {
        const size_t b = (size_t)c * m.NZ, t = b + m.NZ - 1;
        u[b] = m.sgn_bot[0] * u[b + 1]; v[b] = m.sgn_bot[1] * v[b + 1]; w[b] = m.sgn_bot[2] * w[b + 1];
        u[t] = m.sgn_top[0] * u[t - 1]; v[t] = m.sgn_top[1] * v[t - 1]; w[t] = m.sgn_top[2] * w[t - 1];
        p[b] = p[b + 1]; p[t] = p[t - 1];
    }
}

__global__ void k_combine(size_t n, double a, double b, const double* __restrict__ un, double* __restrict__ unp) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        unp[i] = a * un[i] + b * unp[i];
}

// (N_CELL,NZ) Fortran order <-> device columns.  ghost_mode 0: ghost rows
// copy the periodic image; 1: ghost rows are 0.
// Device columns <-> the reference's (rows, NZ) Fortran arrays.  The two
// layouts are transposes of each other, so both directions go through a
// 32 x 32 shared-memory tile: a column's layers are read (written)
// contiguously on the device side and a layer's rows written (read)
// contiguously on the host-array side.
constexpr int kTile = 32, kTileRows = 8;  // tile edge, thread rows of a block

// out(cell, k) = f(col[cell], k + kofs) for cell < ncell, k < layers; rows
// cell >= n0 are zero when ghost_mode = 1.
__global__ void __launch_bounds__(kTile * kTileRows) k_gather(int ncell, int nz, int layers, int kofs,
                                                             const int* __restrict__ col,
                                                             const double* __restrict__ f, int ghost_mode, int n0,
                                                             double* __restrict__ out) {
    __shared__ double tile[kTile][kTile + 1];
    const int c0 = blockIdx.x * kTile, k0 = blockIdx.y * kTile, tx = threadIdx.x;
    for (int j = threadIdx.y; j < kTile; j += kTileRows) {
        const int cell = c0 + j, k = k0 + tx;
        if (cell < ncell && k < layers) {
            const double v = f[(size_t)col[cell] * nz + k + kofs];
            tile[j][tx] = (ghost_mode == 1 && cell >= n0) ? 0.0 : v;
        }
    }
    __syncthreads();
    for (int j = threadIdx.y; j < kTile; j += kTileRows) {
        const int cell = c0 + tx, k = k0 + j;
        if (cell < ncell && k < layers) out[(size_t)cell + (size_t)k * ncell] = tile[tx][j];
    }
}

// f(col[cell], k) = in(cell, k) for cell < n0, k < nz; in is (rows, nz).
__global__ void __launch_bounds__(kTile * kTileRows) k_scatter(int n0, int nz, int rows, const int* __restrict__ col,
                                                              const double* __restrict__ in,
                                                              double* __restrict__ f) {
    __shared__ double tile[kTile][kTile + 1];
    const int c0 = blockIdx.x * kTile, k0 = blockIdx.y * kTile, tx = threadIdx.x;
    for (int j = threadIdx.y; j < kTile; j += kTileRows) {
        const int cell = c0 + tx, k = k0 + j;
        if (cell < n0 && k < nz) tile[j][tx] = in[(size_t)cell + (size_t)k * rows];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < kTile; j += kTileRows) {
        const int cell = c0 + j, k = k0 + tx;
        if (cell < n0 && k < nz) f[(size_t)col[cell] * nz + k] = tile[tx][j];
    }
}

// Vertex pressure (N_VERT,NZ-1): layer 1 equals layer 2 because the wall
// ghost layer of p is a Neumann copy.
__global__ void k_gather_pv(int nvert, int nzi, const int* __restrict__ vcls, const double* __restrict__ pv,
                            double* __restrict__ out) {
    const size_t n = (size_t)nvert * (nzi + 1);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const int nv = (int)(i % nvert), k = (int)(i / nvert);  // k = 0..nzi (reference layer k+1)
        const int kk = (k == 0) ? 0 : k - 1;
        out[i] = pv[(size_t)vcls[nv] * nzi + kk];
    }
}

}  // namespace

int cuda_fail(nsmp_ctx* c, cudaError_t e, const char* where) {
    c->err = std::string(where) + ": " + cudaGetErrorString(e);
    // clear the runtime's last-error slot: a recoverable failure (an
    // allocation that did not fit) must not be reported again by the next
    // launch check of a later, correct call
    cudaGetLastError();
    return NSMP_ERR_CUDA;
}

int occupancy_grid(nsmp_ctx* c, const void* kernel, long long n) {
    int per_sm = 0;
    auto it = c->occ_cache.find(kernel);
    if (it != c->occ_cache.end()) {
        per_sm = it->second;
    } else {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, 0) != cudaSuccess || per_sm < 1)
            per_sm = 1;
        if (per_sm > 8) per_sm = 8;  // reduction scratch holds 8 blocks per SM
        c->occ_cache[kernel] = per_sm;
    }
    long long b = (n + kBlock - 1) / kBlock;
    const long long cap = (long long)c->num_sms * per_sm;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

int prof_begin(nsmp_ctx* c, int kid) {
    if (!c->prof_on) return -1;
    if (c->ev_used + 2 > c->ev_pool.size()) {
        for (int q = 0; q < 256; ++q) {
            cudaEvent_t e;
            if (cudaEventCreate(&e) != cudaSuccess) return -1;
            c->ev_pool.push_back(e);
        }
    }
    const int slot = (int)c->ev_used;
    c->ev_used += 2;
    cudaEventRecord(c->ev_pool[slot], c->stream);
    c->ev_pending.push_back({kid, slot});
    return slot;
}

void prof_end(nsmp_ctx* c, int slot) {
    if (slot < 0) return;
    cudaEventRecord(c->ev_pool[slot + 1], c->stream);
}

// Call after the stream has been synchronised.
int prof_resolve(nsmp_ctx* c) {
    for (auto& pe : c->ev_pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, c->ev_pool[pe.second], c->ev_pool[pe.second + 1]) == cudaSuccess) {
            c->prof_count[pe.first] += 1;
            c->prof_ms[pe.first] += ms;
        }
    }
    c->ev_pending.clear();
    c->ev_used = 0;
    return 0;
}

int run_user_initial(nsmp_ctx* c) {
    const Mesh& m = c->mesh;
    double** L = c->lvl[c->ln];
    const int gb = grid_for(c, m.N0);
    LAUNCH(NSMP_K_OTHER, k_fill_ghosts<<<gb, kBlock, 0, c->stream>>>(m, L[0], L[1], L[2], L[3]));
    CKL("k_fill_ghosts");
    FaceArgs fa{L[0], L[1], L[2], nullptr, c->face[0], c->face[1], c->face[2], c->face[3], c->face[4],
                nullptr, 0.0, 0};
    LAUNCH(NSMP_K_OTHER, k_faces_div<<<grid_for(c, m.nprism), kBlock, 0, c->stream>>>(m, fa, c->red, c->d_scal));
    CKL("k_faces_div(init)");
    const size_t n = (size_t)m.N0 * m.NZ;
    for (int q = 0; q < 3; ++q) CK(cudaMemsetAsync(c->hist[q], 0, n * sizeof(double), c->stream));
    return 0;
}

int run_fill_ghosts(nsmp_ctx* c, int buf) {
    double** L = c->lvl[buf];
    LAUNCH(NSMP_K_OTHER, k_fill_ghosts<<<grid_for(c, c->mesh.N0), kBlock, 0, c->stream>>>(c->mesh, L[0], L[1], L[2], L[3]));
    CKL("k_fill_ghosts");
    return 0;
}

int run_combine(nsmp_ctx* c, double a, double b) {
    const size_t n = (size_t)c->mesh.N0 * c->mesh.NZ;
    for (int f = 0; f < 3; ++f) {
        LAUNCH(NSMP_K_OTHER, k_combine<<<grid_for(c, (long long)n), kBlock, 0, c->stream>>>(n, a, b, c->lvl[c->ln][f], c->lvl[c->lnp][f]));
        CKL("k_combine");
    }
    return 0;
}

int run_stage(nsmp_ctx* c, int fin_rk, nsmp_stage_info* info) {
    const Mesh& m = c->mesh;
    const nsmp_params& P = c->prm;
    cudaStream_t st = c->stream;
    // pick the output buffer: neither the known level nor level n
    int np = 0;
    while (np == c->lknown || np == c->ln) ++np;
    c->lnp = np;
    double** K = c->lvl[c->lknown];
    double** N = c->lvl[np];
    LAUNCH(NSMP_K_VERTEX4, k_vertex<4><<<grid_occ(c, k_vertex<4>, (long long)m.nclass * m.NZI), kBlock, 0, st>>>(m, K[0], K[1], K[2], K[3], c->vtx[0], c->vtx[1], c->vtx[2], c->vtx[3], 0.0));
    CKL("k_vertex4");
    StageArgs sa;
    sa.u = K[0]; sa.v = K[1]; sa.w = K[2];
    sa.uv = c->vtx[0]; sa.vv = c->vtx[1]; sa.wv = c->vtx[2];
    sa.f1 = c->face[0]; sa.f2 = c->face[1]; sa.f3 = c->face[2]; sa.fT = c->face[3]; sa.fB = c->face[4];
    sa.hu = c->hist[0]; sa.hv = c->hist[1]; sa.hw = c->hist[2];
    sa.us = c->ustar[0]; sa.vs = c->ustar[1]; sa.ws = c->ustar[2];
    sa.eddy = c->eddy;
    sa.c1 = (c->flag_ab == 1) ? 1.55 : 1.0;
    sa.c2 = (c->flag_ab == 1) ? -0.55 : 0.0;
    sa.dt = P.dt; sa.inv_re = 1.0 / P.re; sa.bdx = P.bdx; sa.bdy = P.bdy; sa.bdz = P.bdz;
    sa.les = P.les; sa.les_van = P.les_van;
    sa.fx = c->fx;
    if (c->stage32)
        LAUNCH(NSMP_K_STAGE_RHS, k_stage_rhs<float><<<grid_occ(c, k_stage_rhs<float>, m.nprism), kBlock, 0, st>>>(m, sa, c->red, c->d_scal));
    else
        LAUNCH(NSMP_K_STAGE_RHS, k_stage_rhs<double><<<grid_occ(c, k_stage_rhs<double>, m.nprism), kBlock, 0, st>>>(m, sa, c->red, c->d_scal));
    CKL("k_stage_rhs");
    FaceArgs fa{c->ustar[0], c->ustar[1], c->ustar[2], c->vtx[3], c->face[0], c->face[1], c->face[2],
                c->face[3], c->face[4], c->rhsp, 1.0 / P.dt, 1};
    LAUNCH(NSMP_K_FACES_DIV, k_faces_div<<<grid_occ(c, k_faces_div, m.nprism), kBlock, 0, st>>>(m, fa, c->red, c->d_scal));
    CKL("k_faces_div");
    const double* xsol = nullptr;
    const bool replay = c->replay_x != nullptr;
    if (replay) {
        xsol = c->replay_x;
    } else {
        const int rcp = (c->precision == NSMP_MIXED) ? run_pressure_mixed(c, K[3], &xsol)
                                                     : run_pressure_fp64(c, K[3], &xsol);
        if (rcp) return rcp;
        if (c->tape_x)
            CK(cudaMemcpyAsync(c->tape_x, xsol, sizeof(double) * m.nprism, cudaMemcpyDeviceToDevice, st));
    }
    LAUNCH(NSMP_K_PMEAN, k_pmean<<<grid_occ(c, k_pmean, m.nprism), kBlock, 0, st>>>(m, xsol, c->red, c->d_scal));
    CKL("k_pmean");
    LAUNCH(NSMP_K_VERTEX1, k_vertex1<<<grid_occ(c, k_vertex1, (long long)m.nclass * m.NZI), kBlock, 0, st>>>(m, xsol, c->d_scal, c->vtx[3]));
    CKL("k_vertex1");
    ProjArgs pa{xsol, c->vtx[3], c->ustar[0], c->ustar[1], c->ustar[2], c->face[0], c->face[1], c->face[2],
                c->face[3], c->face[4], N[0], N[1], N[2], N[3], P.dt};
    LAUNCH(NSMP_K_PROJECT, k_project<<<grid_occ(c, k_project, m.nprism), kBlock, 0, st>>>(m, pa, c->d_scal));
    CKL("k_project");
    CK(cudaMemcpyAsync(c->h_scal, c->d_scal, sizeof(Scal), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    prof_resolve(c);
    if (replay) {  // the solve was replayed from the tape: no solver statistics
        nsmp_stage_info inf{};
        inf.converged = 1;
        inf.max_eddy = P.les ? c->h_scal->max_eddy : 0.0;
        c->last = inf;
        if (info) *info = inf;
        return 0;
    }
    const Scal& s = *c->h_scal;
    c->last_iters = s.iter > 0 ? s.iter : 1;
    c->bicg_iters += s.iter;
    if (c->precision == NSMP_MIXED) c->fp64_updates += s.outer;
    nsmp_stage_info inf{};
    inf.iters = s.iter;
    inf.e1norm = s.e1;
    inf.e2norm = s.e2;
    inf.converged = s.converged;
    inf.max_eddy = P.les ? s.max_eddy : 0.0;
    inf.status = s.status;
    inf.refinements = (c->precision == NSMP_MIXED) ? s.outer : 0;
    c->last = inf;
    if (s.status == NSMP_ERR_NAN) {
        char buf[512];
        snprintf(buf, sizeof buf,
                 "non-finite residual: iter %d inner %d refinements %d | rho %.3e rho_prev %.3e alpha %.3e "
                 "omega %.3e r0v %.3e | inner r1 %.3e r2 %.3e b1 %.3e b2 %.3e | outer e1 %.3e e2 %.3e",
                 s.iter, s.iiter, s.outer, s.irho, s.irho_prev, s.ialpha, s.iomega, s.ir0v, s.ir1, s.ir2, s.ib1,
                 s.ib2, s.e1, s.e2);
        c->err = buf;
    }
    if (info) *info = inf;
    if (fin_rk == 1 && c->flag_ab != 1) c->flag_ab = 1;  // hydro.F90:469-478
    return s.status;
}

int run_gather(nsmp_ctx* c, const double* dfield, int ghost_mode, int rows, double* host) {
    const int ncell = rows;
    const int layers = c->mesh.NZ;
    const size_t n = (size_t)ncell * layers;
    const dim3 tiles((ncell + kTile - 1) / kTile, (layers + kTile - 1) / kTile), tb(kTile, kTileRows);
    k_gather<<<tiles, tb, 0, c->stream>>>(ncell, c->mesh.NZ, layers, 0, c->d_gather, dfield, ghost_mode, c->L.N0,
                                          c->stage_buf);
    CKL("k_gather");
    CK(cudaMemcpyAsync(host, c->stage_buf, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

int run_download_pv(nsmp_ctx* c, double* host) {
    const size_t n = (size_t)c->L.NV * (c->mesh.NZI + 1);
    k_gather_pv<<<grid_for(c, (long long)n), kBlock, 0, c->stream>>>(c->L.NV, c->mesh.NZI, c->d_vgather,
                                                                     c->vtx[3], c->stage_buf);
    CKL("k_gather_pv");
    CK(cudaMemcpyAsync(host, c->stage_buf, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

// Host (rows,NZ) Fortran array -> device columns, rows = N_CELL (cell
// fields, ghost rows ignored) or N0 (face fluxes): one contiguous copy into
// the staging buffer and a scatter of the interior rows.  Without sync the
// caller synchronises the stream before the host array may change; copies
// of consecutive calls are ordered behind the previous scatter on the stream.
int run_scatter(nsmp_ctx* c, const double* host, double* dfield, int rows, bool sync) {
    const int n0 = c->L.N0, nz = c->mesh.NZ;
    if (rows <= 0) rows = c->L.NC;
    if (rows < n0 || rows > c->L.NC) {
        c->err = "run_scatter: rows out of range";
        return NSMP_ERR_ARG;
    }
    CK(cudaMemcpyAsync(c->stage_buf, host, (size_t)rows * nz * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    const dim3 tiles((n0 + kTile - 1) / kTile, (nz + kTile - 1) / kTile), tb(kTile, kTileRows);
    k_scatter<<<tiles, tb, 0, c->stream>>>(n0, nz, rows, c->d_gather, c->stage_buf, dfield);
    CKL("k_scatter");
    if (sync) CK(cudaStreamSynchronize(c->stream));
    return 0;
}

// The per-layer factor table of the kernels (lev[row * NZ + k0]).
std::vector<double> level_table(const HostLayout& L) {
    std::vector<double> lv((size_t)LV_COUNT * L.NZ, 0.0);
    const Levels& V = L.lev;
    const std::vector<double>* rows[LV_COUNT] = {&V.dsv, nullptr, &V.idsT, &V.idsB, &V.idsBu, &V.wT, &V.wB,
                                                 &V.gzp, &V.gzm, &V.hmean, &V.les_dd, &V.les_kd, &V.les_damp, &V.ihz,
                                                 nullptr, nullptr, &V.cfl_div, &V.cfl_h};
    for (int r = 0; r < LV_COUNT; ++r)
        for (int k = 0; k < L.NZ; ++k) {
            double val;
            if (r == LV_IDSV) val = (V.dsv[k] != 0.0) ? 1.0 / V.dsv[k] : 0.0;
            else if (r == LV_ATOP) val = V.idsT[k] * V.wT[k];  // PPE coupling / area to the layer above
            else if (r == LV_ABOT) val = V.idsB[k] * V.wB[k];  // and below (0 at the walls)
            else val = (*rows[r])[k];
            lv[(size_t)r * L.NZ + k] = val;
        }
    return lv;
}

// FP32 column and level tables of the FP32 stage arithmetic, once.
int stage32_alloc(nsmp_ctx* c) {
    if (c->d_geo32) return 0;
    const HostLayout& L = c->L;
    std::vector<ColGeo32> g32(L.N0);
    for (int q = 0; q < L.N0; ++q) {
        const ColGeo& G = L.geo[q];
        ColGeo32& H = g32[q];
        for (int j = 0; j < 3; ++j) {
            H.nb[j] = G.nb[j]; H.vtx[j] = G.vtx[j];
            H.kA[j] = (float)G.kA[j]; H.dle2[j] = (float)G.dle2[j]; H.kE[j] = (float)G.kE[j]; H.L[j] = (float)G.L[j];
            H.lxu[j] = (float)G.lxu[j]; H.lyu[j] = (float)G.lyu[j];
            H.lxv[j] = (float)G.lxv[j]; H.lyv[j] = (float)G.lyv[j];
        }
        H.area = (float)G.area; H.inv_area = (float)G.inv_area; H.cbrt_area = (float)G.cbrt_area; H.pad = 0.f;
    }
    const std::vector<double> lv = level_table(L);
    std::vector<float> lvf(lv.begin(), lv.end());
    ColGeo32* dg = nullptr;
    float* dl = nullptr;
    CK(cudaMalloc((void**)&dg, sizeof(ColGeo32) * g32.size()));
    c->allocs.push_back(dg);
    CK(cudaMalloc((void**)&dl, sizeof(float) * lvf.size()));
    c->allocs.push_back(dl);
    CK(cudaMemcpyAsync(dg, g32.data(), sizeof(ColGeo32) * g32.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(dl, lvf.data(), sizeof(float) * lvf.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->d_geo32 = dg;
    c->mesh.geo32 = dg;
    c->mesh.levf = dl;
    return 0;
}

int ctx_init_device(nsmp_ctx* c) {
    CK(cudaSetDevice(c->device));
    CK(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device));
    CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    const HostLayout& L = c->L;
    auto dalloc = [&](void** p, size_t bytes) -> cudaError_t {
        cudaError_t e = cudaMalloc(p, bytes > 0 ? bytes : 16);
        if (e == cudaSuccess) c->allocs.push_back(*p);
        return e;
    };
    const size_t ncf = (size_t)L.N0 * L.NZ;
    const size_t nvf = (size_t)L.nclass * L.NZI;
    CK(dalloc((void**)&c->d_ppe, sizeof(ColPPE) * L.N0));
    CK(dalloc((void**)&c->d_geo, sizeof(ColGeo) * L.N0));
    CK(dalloc((void**)&c->d_vptr, sizeof(int) * L.vptr.size()));
    CK(dalloc((void**)&c->d_vcell, sizeof(int) * L.vcell.size()));
    CK(dalloc((void**)&c->d_vcoef, sizeof(double) * L.vcoef.size()));
    CK(dalloc((void**)&c->d_lev, sizeof(double) * LV_COUNT * L.NZ));
    CK(dalloc((void**)&c->d_gather, sizeof(int) * L.NC));
    CK(dalloc((void**)&c->d_vgather, sizeof(int) * L.NV));
    for (int b = 0; b < 3; ++b)
        for (int f = 0; f < 4; ++f) CK(dalloc((void**)&c->lvl[b][f], ncf * sizeof(double)));
    for (auto** p : {&c->face[0], &c->face[1], &c->face[2], &c->face[3], &c->face[4], &c->hist[0], &c->hist[1],
                     &c->hist[2], &c->eddy, &c->ustar[0], &c->ustar[1], &c->ustar[2], &c->rhsp, &c->x, &c->r,
                     &c->r0, &c->pk, &c->vk, &c->sk, &c->tk, &c->invD, &c->ahat[0], &c->ahat[1], &c->ahat[2],
                     &c->ahat[3], &c->ahat[4]})
        CK(dalloc((void**)p, ncf * sizeof(double)));
    for (int f = 0; f < 4; ++f) CK(dalloc((void**)&c->vtx[f], nvf * sizeof(double)));
    const size_t stage_n = std::max((size_t)L.NC * L.NZ, (size_t)L.NV * L.NZ);
    CK(dalloc((void**)&c->stage_buf, stage_n * sizeof(double)));
    const int maxblocks = c->num_sms * 8;
    CK(dalloc((void**)&c->red.partials, sizeof(double) * kMaxRed * maxblocks));
    CK(dalloc((void**)&c->red.counter, sizeof(unsigned int)));
    CK(dalloc((void**)&c->red2.partials, sizeof(double) * kMaxRed * maxblocks));
    CK(dalloc((void**)&c->red2.counter, sizeof(unsigned int)));
    CK(dalloc((void**)&c->d_scal, sizeof(Scal)));
    CK(cudaMallocHost((void**)&c->h_scal, sizeof(Scal)));
    // zero everything once (face fluxes at the wall layers stay 0, as in the reference)
    for (int b = 0; b < 3; ++b)
        for (int f = 0; f < 4; ++f) CK(cudaMemsetAsync(c->lvl[b][f], 0, ncf * sizeof(double), c->stream));
    for (auto* p : {c->face[0], c->face[1], c->face[2], c->face[3], c->face[4], c->hist[0], c->hist[1], c->hist[2],
                    c->eddy, c->ustar[0], c->ustar[1], c->ustar[2], c->rhsp, c->x, c->r, c->r0, c->pk, c->vk,
                    c->sk, c->tk, c->invD})
        CK(cudaMemsetAsync(p, 0, ncf * sizeof(double), c->stream));
    CK(cudaMemsetAsync(c->red.counter, 0, sizeof(unsigned int), c->stream));
    CK(cudaMemsetAsync(c->red2.counter, 0, sizeof(unsigned int), c->stream));
    CK(cudaMemsetAsync(c->d_scal, 0, sizeof(Scal), c->stream));
    // tables
    CK(cudaMemcpyAsync(c->d_ppe, L.ppe.data(), sizeof(ColPPE) * L.N0, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_geo, L.geo.data(), sizeof(ColGeo) * L.N0, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_vptr, L.vptr.data(), sizeof(int) * L.vptr.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_vcell, L.vcell.data(), sizeof(int) * L.vcell.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_vcoef, L.vcoef.data(), sizeof(double) * L.vcoef.size(), cudaMemcpyHostToDevice, c->stream));
    const std::vector<double> lv = level_table(L);
    CK(cudaMemcpyAsync(c->d_lev, lv.data(), sizeof(double) * lv.size(), cudaMemcpyHostToDevice, c->stream));
    std::vector<int> gcol(L.NC), vg(L.NV);
    for (int i = 0; i < L.NC; ++i) gcol[i] = (i < L.N0) ? L.iperm[i] : L.iperm[L.ghost_img[i - L.N0]];
    for (int v = 0; v < L.NV; ++v) vg[v] = L.vclass[v];
    CK(cudaMemcpyAsync(c->d_gather, gcol.data(), sizeof(int) * L.NC, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->d_vgather, vg.data(), sizeof(int) * L.NV, cudaMemcpyHostToDevice, c->stream));
    // kernel view of the mesh
    Mesh& m = c->mesh;
    m.N0 = L.N0; m.NZ = L.NZ; m.NZI = L.NZI; m.nclass = L.nclass;
    m.nprism = L.N0 * L.NZI;
    m.ppe = c->d_ppe; m.geo = c->d_geo; m.vptr = c->d_vptr; m.vcell = c->d_vcell; m.vcoef = c->d_vcoef;
    m.lev = c->d_lev;
    for (int q = 0; q < 3; ++q) { m.sgn_bot[q] = L.sgn_bot[q]; m.sgn_top[q] = L.sgn_top[q]; }
    m.tv_lsig = L.total_volume * L.lsig;
    {
        int rc = fp64_setup(c);
        if (rc) return rc;
    }
    m.geo32 = nullptr;
    m.levf = nullptr;
    Scal s0{};
    s0.eps = c->prm.eps;
    s0.max_iters = c->prm.max_iters;
    s0.inner_tol = c->inner_tol;
    CK(cudaMemcpyAsync(c->d_scal, &s0, sizeof(Scal), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (c->precision == NSMP_MIXED) {
        int rc = mixed_alloc(c);
        if (rc) return rc;
    }
    if (c->stage32) return stage32_alloc(c);
    return 0;
}

void ctx_free(nsmp_ctx* c) {
    if (c->stream) cudaStreamSynchronize(c->stream);
    adj_free(c);
    stats_free(c);
    l2_limit_release(c);  // the last context that raised the persisting-L2 limit restores it
    for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
    c->ev_pool.clear();
    for (void* p : c->allocs) cudaFree(p);
    c->allocs.clear();
    if (c->h_scal) cudaFreeHost(c->h_scal);
    c->h_scal = nullptr;
    if (c->stream) cudaStreamDestroy(c->stream);
    c->stream = nullptr;
}

}  // namespace nsmp
