// Discrete adjoint of the SSP-RK3 step of the reference stage.
//
// Objective: the wall shear stress averaged over both walls and over the
// steps n = 1..N,
//   J = 1/N sum_n sum_c area_c nu (u^n(c,1) / h_1 + u^n(c,NZ-2) / h_NZ-2) / (2 A)
// with h = half the height of the first (last) interior layer, A the plan
// area and nu = 1/Re (no-slip walls: the ghost holds -u).  Control: a body
// force f_x per cell added to the u right-hand side of every stage
// (hydro.F90:322-333 with bdx + f_x).  Result: dJ/df_x.
//
// Each kernel here is the transpose of one forward kernel of stage.cu
// (linear parts exactly; advection and the Smagorinsky viscosity linearised
// about the recomputed forward state).  The pressure solve is linear,
//   p = P2 A^+ P1 rhsp   (P1, P2 the Glob_Norm mean removals),
// and A is symmetric, so its adjoint is the same BiCGSTAB solve applied to
// the adjoint pressure (after the transposed mean removals).  Contributions
// to neighbour cells and vertex classes are not scattered with atomics: each
// transposed kernel writes them to slot planes (one value per prism and kind
// of contribution), and gather kernels add, for every destination, the slots
// that point at it in a fixed order (lateral edges 0-2, the layer below, the
// layer above; vertex classes over their incident corners in column order).
// The gradient is therefore the same bit for bit from run to run.
//
// Memory: checkpoints of the state every `ckpt_every` steps and the PPE
// solution of every stage (the pressure tape); during the reverse sweep one
// segment is recomputed from its checkpoint, replaying the taped pressures
// instead of solving again, and the inputs of each of its stages (u, v, w
// with ghost layers and the five face fluxes) are kept -- for the whole
// segment when that fits, else for the step being reversed, re-reached from
// inner checkpoints.  The adjoint pressure solves run in the context's
// precision mode (FP64, or FP32 BiCGSTAB with FP64 refinement).
#include <algorithm>
#include <cmath>
#include <vector>

#include "kern_common.cuh"

struct AdjScratch {
    // adjoint of the input and output of one stage (cell layout, ghost layers
    // folded into the interior between kernels)
    double* A[2][9] = {};   // [set][u, v, w, p, f1, f2, f3, fT, fB]
    double* acc[3] = {};    // RK3: accumulated adjoint of u^n
    double* aus[3] = {};    // adjoint of u*
    double* apc = nullptr;  // adjoint of the new pressure (compact layout)
    double* arhs = nullptr; // adjoint of the PPE right-hand side (compact)
    double* avx[4] = {};    // adjoint of the vertex fields (class layout)
    double* vtx[3] = {};    // recomputed vertex values of the stage input
    double* afx = nullptr;  // gradient accumulator (cell layout)
    double* zero = nullptr; // zero cell field
    double* lamc = nullptr; // last adjoint pressure solution (cell layout, unscaled)
    double* guess = nullptr;// initial guess of the next adjoint solve (cell layout)
    double* fx_host_stage = nullptr;
    int* tptr = nullptr;    // transposed vertex stencil: cell -> (class, weight)
    int* tcls = nullptr;
    double* tcoef = nullptr;
    // deterministic accumulation: a kernel writes each contribution to a
    // neighbour into a slot plane (compact layout, one plane per kind of
    // contribution); gather kernels then add, in a fixed order, the slots
    // that point at each destination
    double* slot = nullptr; // kSlotPlanes x nprism
    int* nbrev = nullptr;   // (N0,3): edge of nb[c][j] that leads back to c
    int* iptr = nullptr;    // vertex class -> incident (column, corner) pairs, column-major order
    int* inc = nullptr;     //   encoded 3 * column + corner
    bool pairing_ok = true; // every edge has exactly one reversed partner
    double tot_area = 0.0, hsum = 0.0;
    double seg_budget = 0.0;  // bytes for the segment's stage inputs; 0: 80 % of free memory
};

namespace nsmp {
namespace {

constexpr int NF_STATE = 9;  // u, v, w, p + five face fluxes
constexpr int kSlotPlanes = 24;  // k_adj_stage: 3 fields x (3 lateral + up + down + 3 corners)

// Slot plane layout of one field's contributions: lateral across edge 0..2,
// to the layer above, to the layer below; corner planes separately.
enum { SL_L0 = 0, SL_UP = 3, SL_DN = 4, SL_CELL = 5 };

// vertex values of u, v, w (the arithmetic of the forward k_vertex, so the
// linearisation point is the forward's)
__global__ void __launch_bounds__(kBlock) k_vtx3(Mesh m, const double* __restrict__ f0,
                                                 const double* __restrict__ f1, const double* __restrict__ f2,
                                                 double* __restrict__ o0, double* __restrict__ o1,
                                                 double* __restrict__ o2) {
    const int n = m.nclass * m.NZI;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) {
        const int v = g / m.NZI, k0 = 1 + (g - v * m.NZI);
        double a0 = 0.0, a1 = 0.0, a2 = 0.0;
        const int s1 = __ldg(m.vptr + v + 1);
        for (int s = __ldg(m.vptr + v); s < s1; ++s) {
            const double w = __ldg(m.vcoef + s);
            const size_t q = IX(m, __ldg(m.vcell + s), k0);
            a0 += w * f0[q];
            a1 += w * f1[q];
            a2 += w * f2[q];
        }
        const size_t o = IV(m, v, k0);
        o0[o] = a0; o1[o] = a1; o2[o] = a2;
    }
}

// ---------------------------------------------------------------------------
// objective
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_wall_shear(Mesh m, const double* __restrict__ u, double wb, double wt,
                                                       RedScratch rs, Scal* sc) {
    double part[1] = {0.0};
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m.N0; c += gridDim.x * blockDim.x) {
        const double ar = m.geo[c].area;
        part[0] += ar * (wb * u[IX(m, c, 1)] + wt * u[IX(m, c, m.NZ - 2)]);
    }
    double tot[1];
    if (grid_reduce<1, false>(part, rs, tot) && threadIdx.x == 0) sc->jval = tot[0];
}

__global__ void k_adj_seed(Mesh m, double* __restrict__ au, double wb, double wt) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m.N0; c += gridDim.x * blockDim.x) {
        const double ar = m.geo[c].area;
        au[IX(m, c, 1)] += ar * wb;
        au[IX(m, c, m.NZ - 2)] += ar * wt;
    }
}

// ---------------------------------------------------------------------------
// ghost layers: the forward writes ghost = sign * interior (velocity) or
// ghost = interior (pressure); the adjoint of a ghost value moves into the
// interior value it was copied from.
// ---------------------------------------------------------------------------
__global__ void k_adj_fold(Mesh m, double* a0, double* a1, double* a2, double* ap) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < m.N0; c += gridDim.x * blockDim.x) {
        const size_t b = (size_t)c * m.NZ, t = b + m.NZ - 1;
        double* a[3] = {a0, a1, a2};
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            if (!a[f]) continue;
            a[f][b + 1] += m.sgn_bot[f] * a[f][b]; a[f][b] = 0.0;
            a[f][t - 1] += m.sgn_top[f] * a[f][t]; a[f][t] = 0.0;
        }
        if (ap) {
            ap[b + 1] += ap[b]; ap[b] = 0.0;
            ap[t - 1] += ap[t]; ap[t] = 0.0;
        }
    }
}

// y = a x + b y over n values
__global__ void k_axpby(size_t n, double a, const double* __restrict__ x, double b, double* __restrict__ y) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        y[i] = a * x[i] + b * y[i];
}

// ---------------------------------------------------------------------------
// transpose of the vertex interpolation (k_vertex / k_vertex1): each cell
// gathers weight * adjoint over the vertex classes whose stencil holds it.
// COMPACT: destination in the compact solver layout, else cell layout.
// ---------------------------------------------------------------------------
template <int NF, bool COMPACT>
__global__ void __launch_bounds__(kBlock) k_adj_vertexT(Mesh m, const int* __restrict__ tptr,
                                                        const int* __restrict__ tcls,
                                                        const double* __restrict__ tcoef, const double* i0,
                                                        const double* i1, const double* i2, double* o0, double* o1,
                                                        double* o2) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        double s0 = 0.0, s1 = 0.0, s2 = 0.0;
        for (int e = tptr[c]; e < tptr[c + 1]; ++e) {
            const double w = tcoef[e];
            const size_t v = IV(m, tcls[e], k0);
            s0 += w * i0[v];
            if (NF > 1) s1 += w * i1[v];
            if (NF > 2) s2 += w * i2[v];
        }
        const size_t q = COMPACT ? (size_t)g : IX(m, c, k0);
        o0[q] += s0;
        if (NF > 1) o1[q] += s1;
        if (NF > 2) o2[q] += s2;
    }
}

// ---------------------------------------------------------------------------
// transpose of k_project (gradientP + cell correction + newu3D faces)
// ---------------------------------------------------------------------------
struct AdjProjArgs {
    const double *au, *av, *aw, *ap;         // adjoint of u, v, w, p of the stage output
    const double *f1, *f2, *f3, *fT, *fB;    // adjoint of the face fluxes (output = input of the face pass)
    double *aus, *avs, *aws;                 // adjoint of u* (written)
    double* apc;                             // adjoint of the new p (compact, accumulated)
    double* apv;                             // adjoint of the vertex p (class layout, accumulated)
    double dt;
};

// Contributions to other prisms go to slot planes 0-4 (lateral across edge
// 0..2, above, below; zero at the walls) and the vertex-pressure
// contributions per corner to planes 5-7; the prism's own part is added in
// place.  k_gather_cells / k_gather_corners sum them in a fixed order.
__global__ void __launch_bounds__(kBlock) k_adj_project(Mesh m, AdjProjArgs a, double* __restrict__ slot) {
    const size_t np = (size_t)m.nprism;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const ColGeo& G = m.geo[c];
        const size_t q = IX(m, c, k0);
        const double ub = a.au[q], vb = a.av[q], wb = a.aw[q];
        a.aus[q] = ub; a.avs[q] = vb; a.aws[q] = wb;
        const double Fb[3] = {a.f1[q], a.f2[q], a.f3[q]};
        double pc = a.ap[q];
        double cv[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            // d = p_nb - p enters dpdx, dpdy and the face correction dn_j
            const double t = -a.dt * (G.gx[j] * ub + G.gy[j] * vb + G.cA[j] * Fb[j]);
            slot[(SL_L0 + j) * np + g] = t;
            pc -= t;
            const double tv = -a.dt * G.cB[j] * Fb[j];   // (vb - va) * cB
            cv[(j + 1) % 3] += tv;
            cv[j] -= tv;
        }
        double up = 0.0, dn = 0.0;
        if (k0 < m.NZ - 2) {  // pT - p (zero at the top wall: Neumann ghost)
            up = -a.dt * (lev(m, LV_GZP, k0) * wb + lev(m, LV_IDST, k0) * a.fT[q]);
            pc -= up;
        }
        if (k0 > 1) {
            dn = -a.dt * (lev(m, LV_GZM, k0) * wb + lev(m, LV_IDSBU, k0) * a.fB[q]);
            pc -= dn;
        }
        slot[SL_UP * np + g] = up;
        slot[SL_DN * np + g] = dn;
        a.apc[g] += pc;
#pragma unroll
        for (int j = 0; j < 3; ++j) slot[(SL_CELL + j) * np + g] = cv[j];
    }
}

// ---------------------------------------------------------------------------
// deterministic gathers of the slot planes
// ---------------------------------------------------------------------------
// Per destination field: the planes of its lateral contributions (lat..lat+2,
// indexed by the SOURCE's edge), of contributions from the layer below
// (`up`, written by the prism below) and from the layer above (`dn`); -1:
// none.  Cell-layout destinations also receive the wall-ghost entries
// (folded into the interior later, as the forward's ghosts are copies).
struct GatherArgs {
    double* out[3];
    int lat[3], up[3], dn[3];
    int nf;
};

template <bool COMPACT>
__global__ void __launch_bounds__(kBlock) k_gather_cells(Mesh m, const int* __restrict__ nbrev,
                                                         const double* __restrict__ slot, GatherArgs ga) {
    const size_t np = (size_t)m.nprism;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const ColGeo& G = m.geo[c];
        for (int f = 0; f < ga.nf; ++f) {
            double s = 0.0;
            if (ga.lat[f] >= 0)
#pragma unroll
                for (int j = 0; j < 3; ++j)
                    s += slot[(size_t)(ga.lat[f] + __ldg(nbrev + 3 * c + j)) * np + ICg(m, G.nb[j], k0)];
            if (ga.up[f] >= 0 && k0 > 1) s += slot[(size_t)ga.up[f] * np + g - 1];
            if (ga.dn[f] >= 0 && k0 < m.NZ - 2) s += slot[(size_t)ga.dn[f] * np + g + 1];
            double* o = ga.out[f];
            if (COMPACT) {
                o[g] += s;
            } else {
                o[IX(m, c, k0)] += s;
                if (ga.dn[f] >= 0 && k0 == 1) o[IX(m, c, 0)] += slot[(size_t)ga.dn[f] * np + g];
                if (ga.up[f] >= 0 && k0 == m.NZ - 2) o[IX(m, c, m.NZ - 1)] += slot[(size_t)ga.up[f] * np + g];
            }
        }
    }
}

// Vertex classes: the corner planes base..base+2 of every (column, corner)
// incident to the class, in ascending column order.
struct CornerArgs {
    double* out[3];
    int base[3];
    int nf;
};

__global__ void __launch_bounds__(kBlock) k_gather_corners(Mesh m, const int* __restrict__ iptr,
                                                           const int* __restrict__ inc,
                                                           const double* __restrict__ slot, CornerArgs ca) {
    const size_t np = (size_t)m.nprism;
    const int n = m.nclass * m.NZI;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int v = i / m.NZI, k0 = 1 + (i - v * m.NZI);
        const int e0 = __ldg(iptr + v), e1 = __ldg(iptr + v + 1);
        for (int f = 0; f < ca.nf; ++f) {
            double s = 0.0;
            for (int e = e0; e < e1; ++e) {
                const int cj = __ldg(inc + e), cc = cj / 3, j = cj - 3 * cc;
                s += slot[(size_t)(ca.base[f] + j) * np + ICg(m, cc, k0)];
            }
            ca.out[f][IV(m, v, k0)] += s;
        }
    }
}

// ---------------------------------------------------------------------------
// transposes of the Glob_Norm mean removals around the solve
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_adj_sum(Mesh m, const double* __restrict__ x, RedScratch rs, Scal* sc) {
    double part[1] = {0.0};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) part[0] += x[g];
    double tot[1];
    if (grid_reduce<1, false>(part, rs, tot) && threadIdx.x == 0) sc->jsum = tot[0];
}

// rhs = P2^T p_bar with its plain mean removed: p_bar - h S / H - (S - S hsum / H) / N,
// S = sum p_bar, h = area * hmean weight, hsum = sum h (so the result sums to 0),
// and |rhs|_2.
__global__ void __launch_bounds__(kBlock) k_adj_solve_rhs(Mesh m, const double* __restrict__ pb,
                                                          double* __restrict__ rhs, double hsum, RedScratch rs,
                                                          Scal* sc) {
    const double S = sc->jsum, H = m.tv_lsig;
    const double cst = (S - S * hsum / H) / (double)m.nprism;
    double part[1] = {0.0};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const double y = pb[g] - m.ppe[c].area * lev(m, LV_HMEAN, k0) * S / H - cst;
        rhs[g] = y;
        part[0] += y * y;
    }
    double tot[1];
    if (grid_reduce<1, false>(part, rs, tot) && threadIdx.x == 0) {
        sc->adjn = sqrt(tot[0]);
        sc->sum_rhs = 0.0;
    }
}

// The solve sees the right-hand side scaled to unit norm: the adjoint
// values are small, and BiCGSTAB's breakdown tests are absolute
// (bicgstab.F90:479-517).
__global__ void k_adj_unit(Mesh m, double* __restrict__ rhs, const Scal* sc) {
    const double n = sc->adjn;
    const double inv = (n > 0.0) ? 1.0 / n : 1.0;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) rhs[g] *= inv;
}

// The adjoint pressure varies slowly from stage to stage, as the forward
// pressure does: the last solution, scaled to the new right-hand side's norm,
// starts the next solve.
__global__ void k_adj_guess(Mesh m, const double* __restrict__ lamc, double* __restrict__ guess, const Scal* sc) {
    const double n = sc->adjn;
    const double inv = (n > 0.0) ? 1.0 / n : 0.0;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const size_t q = cell_of(g, c);
        guess[q] = lamc[q] * inv;
    }
}

__global__ void k_adj_keep(Mesh m, const double* __restrict__ lam, double* __restrict__ lamc, const Scal* sc) {
    const double n = sc->adjn;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        lamc[cell_of(g, c)] = lam[g] * n;
    }
}

// rhs_bar = (lambda - mean(lambda)) * |rhs|_2
__global__ void k_adj_center(Mesh m, const double* __restrict__ lam, double* __restrict__ out, const Scal* sc) {
    const double mean = sc->jsum / (double)m.nprism, n = sc->adjn;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x)
        out[g] = (lam[g] - mean) * n;
}

// ---------------------------------------------------------------------------
// transpose of k_faces_div (interpolateU + divergence/dt + update_rhsp)
// ---------------------------------------------------------------------------
struct AdjFaceArgs {
    const double* arhs;                      // adjoint of rhsp (compact)
    const double *f1, *f2, *f3, *fT, *fB;    // adjoint of the face fluxes after the face pass
    double *aus, *avs, *aws;                 // adjoint of u* (accumulated, cell layout with ghosts)
    double* apv;                             // adjoint of the vertex p of the stage input
    double inv_dt;
};

// Slot planes: u lateral 0-2, v lateral 3-5, w to the layer above 6 and
// below 7, vertex-pressure corners 8-10; the prism's own parts in place.
enum { SF_U = 0, SF_V = 3, SF_WUP = 6, SF_WDN = 7, SF_PC = 8 };

__global__ void __launch_bounds__(kBlock) k_adj_faces(Mesh m, AdjFaceArgs a, double* __restrict__ slot) {
    const size_t np = (size_t)m.nprism;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const ColGeo& G = m.geo[c];
        const size_t q = IX(m, c, k0);
        const double rb = a.arhs[g];
        const double dsv = lev(m, LV_DSV, k0);
        const double Fb[3] = {a.f1[q] + rb * G.L[0] * dsv * a.inv_dt, a.f2[q] + rb * G.L[1] * dsv * a.inv_dt,
                              a.f3[q] + rb * G.L[2] * dsv * a.inv_dt};
        const double FTb = a.fT[q] + rb * G.area * a.inv_dt, FBb = a.fB[q] + rb * G.area * a.inv_dt;
        double ou = 0.0, ov = 0.0;
        double cp[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const double tu = 0.5 * G.xn[j] * Fb[j], tv = 0.5 * G.yn[j] * Fb[j];
            slot[(SF_U + j) * np + g] = tu;
            slot[(SF_V + j) * np + g] = tv;
            ou += tu;
            ov += tv;
            const double tp = -dsv * G.dle2[j] * rb;   // (pb - pa) * dle2, pb = vertex j+1
            cp[(j + 1) % 3] += tp;
            cp[j] -= tp;
        }
        a.aus[q] += ou;
        a.avs[q] += ov;
        a.aws[q] += 0.5 * FTb - 0.5 * FBb;
        slot[SF_WUP * np + g] = 0.5 * FTb;
        slot[SF_WDN * np + g] = -0.5 * FBb;
#pragma unroll
        for (int j = 0; j < 3; ++j) slot[(SF_PC + j) * np + g] = cp[j];
    }
}

// ---------------------------------------------------------------------------
// transpose of k_stage_rhs (Smagorinsky nu_t, Kim-Choi advection and
// diffusion, Euler predictor), linearised about the stage input.
// ---------------------------------------------------------------------------
struct AdjStageArgs {
    const double *u, *v, *w;              // stage input (ghost layers valid)
    const double *uv, *vv, *wv;           // vertex values of the input
    const double *f1, *f2, *f3, *fT, *fB; // input face fluxes
    const double *aus, *avs, *aws;        // adjoint of u* (ghosts folded)
    double *au, *av, *aw;                 // adjoint of the input (accumulated, cell layout with ghosts)
    double *af1, *af2, *af3, *afT, *afB;  // adjoint of the input face fluxes (written)
    double* afx;                          // dJ/df_x (accumulated)
    double* slot;                         // contributions to other prisms and vertex classes
    double c1, dt, inv_re;
    int les, les_van;
};

__global__ void __launch_bounds__(kBlock) k_adj_stage(Mesh m, AdjStageArgs a) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const ColGeo& G = m.geo[c];
        const size_t q = IX(m, c, k0);
        const double dsv = lev(m, LV_DSV, k0), idsT = lev(m, LV_IDST, k0), idsB = lev(m, LV_IDSB, k0);
        // ---- forward values ----
        const double* U[3] = {a.u, a.v, a.w};
        const double* UV[3] = {a.uv, a.vv, a.wv};
        double x0[3], xT[3], xB[3], xn[3][3], fv[3][3], Ff[3][3];
        size_t qn[3], qv[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            qn[j] = IX(m, G.nb[j], k0);
            qv[j] = IV(m, G.vtx[j], k0);
        }
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            x0[f] = U[f][q]; xT[f] = U[f][q + 1]; xB[f] = U[f][q - 1];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                xn[f][j] = U[f][qn[j]];
                fv[f][j] = UV[f][qv[j]];
            }
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int jj = (j + 1) % 3;
                Ff[f][j] = xn[f][j] * 0.5 + x0[f] * 0.5 + G.kE[j] * (fv[f][jj] - fv[f][j]);
            }
        }
        double FT[3], FB[3];  // vertical face values
#pragma unroll
        for (int f = 0; f < 3; ++f) { FT[f] = 0.5 * (x0[f] + xT[f]); FB[f] = 0.5 * (x0[f] + xB[f]); }
        const double ar = G.area;
        const double F[3] = {a.f1[q] * G.L[0] * dsv, a.f2[q] * G.L[1] * dsv, a.f3[q] * G.L[2] * dsv};
        const double FTf = a.fT[q] * ar, FBf = a.fB[q] * ar;
        double gam = a.inv_re;
        double dudx = 0, dudy = 0, dvdx = 0, dvdy = 0, dwdx = 0, dwdy = 0, dudz = 0, dvdz = 0, dwdz = 0;
        double sij = 0.0, l2 = 0.0, ihz = 0.0;
        if (a.les) {
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                dudx += Ff[0][j] * G.lxu[j]; dudy += Ff[0][j] * G.lyu[j];
                dvdx += Ff[1][j] * G.lxv[j]; dvdy += Ff[1][j] * G.lyv[j];
                dwdx += Ff[2][j] * G.lxu[j]; dwdy += Ff[2][j] * G.lyu[j];
            }
            ihz = lev(m, LV_IHZ, k0);
            dudz = (FT[0] - FB[0]) * ihz; dvdz = (FT[1] - FB[1]) * ihz; dwdz = (FT[2] - FB[2]) * ihz;
            const double sxy = 0.5 * (dudy + dvdx), sxz = 0.5 * (dudz + dwdx), syz = 0.5 * (dvdz + dwdy);
            sij = sqrt(2.0 * (dudx * dudx + dvdy * dvdy + dwdz * dwdz) + 4.0 * (sxy * sxy + sxz * sxz + syz * syz));
            const double dd = G.cbrt_area * lev(m, LV_DD, k0);
            double lw = lev(m, LV_KD, k0);
            if (a.les_van) {
                if (lw > dd) lw = dd;
                const double l = lw * lev(m, LV_DAMP, k0);
                l2 = l * l;
            } else {
                l2 = 1.0 / (1.0 / (dd * dd) + 1.0 / (lw * lw));
            }
            gam = l2 * sij + a.inv_re;
        }
        double sd[3];  // diffusion sums
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            double s = 0.0;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int jj = (j + 1) % 3;
                s += (xn[f][j] - x0[f]) * G.kA[j] + (fv[f][jj] - fv[f][j]) * G.dle2[j];
            }
            sd[f] = s * dsv + ((xT[f] - x0[f]) * idsT + (xB[f] - x0[f]) * idsB) * ar;
        }
        const double ivol = G.inv_area * lev(m, LV_IDSV, k0);
        // ---- reverse ----
        const double usb[3] = {a.aus[q], a.avs[q], a.aws[q]};
        double rb[3];
#pragma unroll
        for (int f = 0; f < 3; ++f) rb[f] = a.dt * a.c1 * usb[f];
        a.afx[q] += rb[0];
        double gamb = (rb[0] * sd[0] + rb[1] * sd[1] + rb[2] * sd[2]) * ivol;
        double sdb[3], advb[3];
#pragma unroll
        for (int f = 0; f < 3; ++f) { sdb[f] = rb[f] * gam * ivol; advb[f] = -rb[f] * ivol; }
        // advection: adv = sum_j Ff_j F_j + FT FTf + FB FBf
        double Ffb[3][3], FTb[3], FBb[3];
#pragma unroll
        for (int f = 0; f < 3; ++f) {
#pragma unroll
            for (int j = 0; j < 3; ++j) Ffb[f][j] = advb[f] * F[j];
            FTb[f] = advb[f] * FTf;
            FBb[f] = advb[f] * FBf;
        }
        {
            double fb[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) fb[j] = advb[0] * Ff[0][j] + advb[1] * Ff[1][j] + advb[2] * Ff[2][j];
            a.af1[q] = fb[0] * G.L[0] * dsv;
            a.af2[q] = fb[1] * G.L[1] * dsv;
            a.af3[q] = fb[2] * G.L[2] * dsv;
            a.afT[q] = (advb[0] * FT[0] + advb[1] * FT[1] + advb[2] * FT[2]) * ar;
            a.afB[q] = (advb[0] * FB[0] + advb[1] * FB[1] + advb[2] * FB[2]) * ar;
        }
        // Smagorinsky: nu_t = l2 sqrt(Q)
        if (a.les && sij > 0.0) {
            const double sxy = 0.5 * (dudy + dvdx), sxz = 0.5 * (dudz + dwdx), syz = 0.5 * (dvdz + dwdy);
            const double Qb = gamb * l2 / (2.0 * sij);
            const double dudxb = 4.0 * Qb * dudx, dvdyb = 4.0 * Qb * dvdy, dwdzb = 4.0 * Qb * dwdz;
            const double sxyb = 8.0 * Qb * sxy, sxzb = 8.0 * Qb * sxz, syzb = 8.0 * Qb * syz;
            const double dudyb = 0.5 * sxyb, dvdxb = 0.5 * sxyb, dudzb = 0.5 * sxzb, dwdxb = 0.5 * sxzb;
            const double dvdzb = 0.5 * syzb, dwdyb = 0.5 * syzb;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                Ffb[0][j] += dudxb * G.lxu[j] + dudyb * G.lyu[j];
                Ffb[1][j] += dvdxb * G.lxv[j] + dvdyb * G.lyv[j];
                Ffb[2][j] += dwdxb * G.lxu[j] + dwdyb * G.lyu[j];
            }
            FTb[0] += dudzb * ihz; FBb[0] -= dudzb * ihz;
            FTb[1] += dvdzb * ihz; FBb[1] -= dvdzb * ihz;
            FTb[2] += dwdzb * ihz; FBb[2] -= dwdzb * ihz;
        }
        double* AU[3] = {a.au, a.av, a.aw};
        const size_t np = (size_t)m.nprism;
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            double* sl = a.slot + (size_t)(8 * f) * np;  // field f: lateral 0-2, up 3, down 4, corners 5-7
            double own = usb[f];          // u* = u + dt * r
            double vb[3] = {0.0, 0.0, 0.0};
            const double s = sdb[f] * dsv;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const int jj = (j + 1) % 3;
                // diffusion: (xn - x0) kA + (f_jj - f_j) dle2
                const double tn = s * G.kA[j] + 0.5 * Ffb[f][j];
                sl[(SL_L0 + j) * np + g] = tn;
                own += -s * G.kA[j] + 0.5 * Ffb[f][j];
                const double tv = s * G.dle2[j] + G.kE[j] * Ffb[f][j];
                vb[jj] += tv;
                vb[j] -= tv;
            }
            const double tT = sdb[f] * ar * idsT + 0.5 * FTb[f];
            const double tB = sdb[f] * ar * idsB + 0.5 * FBb[f];
            own += -sdb[f] * ar * idsT - sdb[f] * ar * idsB + 0.5 * FTb[f] + 0.5 * FBb[f];
            sl[SL_UP * np + g] = tT;
            sl[SL_DN * np + g] = tB;
            AU[f][q] += own;
#pragma unroll
            for (int j = 0; j < 3; ++j) sl[(SL_CELL + j) * np + g] = vb[j];
        }
    }
}

// ---------------------------------------------------------------------------
// A and its transpose on interior fields (test hooks for the dot-product test)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_apply_A(Mesh m, int transpose, const double* __restrict__ x,
                                                    double* __restrict__ y) {
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const ColPPE& P = m.ppe[c];
        const size_t q = IX(m, c, k0);
        if (!transpose) {
            y[q] = ppe_row(m, P, k0, x[q], x[IX(m, P.nb[0], k0)], x[IX(m, P.nb[1], k0)], x[IX(m, P.nb[2], k0)],
                           x[q + 1], x[q - 1]);
            continue;
        }
        // (A^T x)_j = sum_i A_ij x_i: row i's coefficient toward this prism
        const double dsv = lev(m, LV_DSV, k0);
        const double AAT = P.area * lev(m, LV_IDST, k0) * lev(m, LV_WT, k0);
        const double AAB = P.area * lev(m, LV_IDSB, k0) * lev(m, LV_WB, k0);
        double acc = -(AAT + AAB + (P.kA[0] + P.kA[1] + P.kA[2]) * dsv) * x[q];
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            const int n = P.nb[j];
            const ColPPE& Q = m.ppe[n];
            double kq = 0.0;
#pragma unroll
            for (int e = 0; e < 3; ++e)
                if (Q.nb[e] == c) kq += Q.kA[e];
            // a column met over two of its edges appears twice in P.nb;
            // share kq between those appearances
            int mult = 0;
#pragma unroll
            for (int e = 0; e < 3; ++e) mult += (P.nb[e] == n);
            acc += kq / mult * dsv * x[IX(m, n, k0)];
        }
        if (k0 < m.NZ - 2)  // row k0+1 couples to k0 through its bottom coefficient
            acc += P.area * lev(m, LV_IDSB, k0 + 1) * lev(m, LV_WB, k0 + 1) * x[q + 1];
        if (k0 > 1)
            acc += P.area * lev(m, LV_IDST, k0 - 1) * lev(m, LV_WT, k0 - 1) * x[q - 1];
        y[q] = acc;
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int adj_alloc(nsmp_ctx* c) {
    if (c->adj) return 0;
    c->adj = new AdjScratch();
    AdjScratch& S = *c->adj;
    const HostLayout& L = c->L;
    const size_t ncf = (size_t)L.N0 * L.NZ, ncmp = (size_t)L.N0 * L.NZI, nvx = (size_t)L.nclass * L.NZI;
    auto dalloc = [&](void** p, size_t bytes) -> cudaError_t {
        cudaError_t e = cudaMalloc(p, bytes > 0 ? bytes : 16);
        if (e == cudaSuccess) {
            c->allocs.push_back(*p);
            e = cudaMemsetAsync(*p, 0, bytes, c->stream);
        }
        return e;
    };
    for (int s = 0; s < 2; ++s)
        for (int f = 0; f < NF_STATE; ++f) CK(dalloc((void**)&S.A[s][f], ncf * sizeof(double)));
    for (int f = 0; f < 3; ++f) {
        CK(dalloc((void**)&S.acc[f], ncf * sizeof(double)));
        CK(dalloc((void**)&S.aus[f], ncf * sizeof(double)));
        CK(dalloc((void**)&S.vtx[f], nvx * sizeof(double)));
    }
    for (int f = 0; f < 4; ++f) CK(dalloc((void**)&S.avx[f], nvx * sizeof(double)));
    CK(dalloc((void**)&S.apc, ncmp * sizeof(double)));
    CK(dalloc((void**)&S.arhs, ncmp * sizeof(double)));
    CK(dalloc((void**)&S.afx, ncf * sizeof(double)));
    CK(dalloc((void**)&S.zero, ncf * sizeof(double)));
    CK(dalloc((void**)&S.lamc, ncf * sizeof(double)));
    CK(dalloc((void**)&S.guess, ncf * sizeof(double)));
    // transposed vertex stencil (cell -> classes), deterministic order
    std::vector<std::vector<std::pair<int, double>>> rows(L.N0);
    for (int v = 0; v < L.nclass; ++v)
        for (int s = L.vptr[v]; s < L.vptr[v + 1]; ++s) rows[L.vcell[s]].push_back({v, L.vcoef[s]});
    std::vector<int> tptr(L.N0 + 1, 0), tcls;
    std::vector<double> tcoef;
    for (int q = 0; q < L.N0; ++q) {
        std::sort(rows[q].begin(), rows[q].end());
        for (auto& e : rows[q]) { tcls.push_back(e.first); tcoef.push_back(e.second); }
        tptr[q + 1] = (int)tcls.size();
    }
    CK(dalloc((void**)&S.tptr, sizeof(int) * tptr.size()));
    CK(dalloc((void**)&S.tcls, sizeof(int) * std::max<size_t>(1, tcls.size())));
    CK(dalloc((void**)&S.tcoef, sizeof(double) * std::max<size_t>(1, tcoef.size())));
    CK(cudaMemcpyAsync(S.tptr, tptr.data(), sizeof(int) * tptr.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(S.tcls, tcls.data(), sizeof(int) * tcls.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(S.tcoef, tcoef.data(), sizeof(double) * tcoef.size(), cudaMemcpyHostToDevice, c->stream));
    // edge pairing of the gathers: edge j of column c runs from vertex class
    // vtx[j] to vtx[j+1]; its neighbour n holds the same edge reversed
    std::vector<int> nbrev(3 * (size_t)L.N0, -1);
    for (int q = 0; q < L.N0; ++q)
        for (int j = 0; j < 3; ++j) {
            const ColGeo& G = L.geo[q];
            const ColGeo& H = L.geo[G.nb[j]];
            int found = -1, count = 0;
            for (int e = 0; e < 3; ++e)
                if (H.nb[e] == q && H.vtx[e] == G.vtx[(j + 1) % 3] && H.vtx[(e + 1) % 3] == G.vtx[j]) {
                    found = e;
                    ++count;
                }
            if (count != 1) S.pairing_ok = false;  // nsmp_adjoint refuses such a mesh
            nbrev[3 * (size_t)q + j] = count == 1 ? found : 0;
        }
    std::vector<int> iptr(L.nclass + 1, 0), inc(3 * (size_t)L.N0);
    for (int q = 0; q < L.N0; ++q)
        for (int j = 0; j < 3; ++j) iptr[L.geo[q].vtx[j] + 1] += 1;
    for (int v = 0; v < L.nclass; ++v) iptr[v + 1] += iptr[v];
    {
        std::vector<int> fill(iptr.begin(), iptr.end() - 1);
        for (int q = 0; q < L.N0; ++q)  // ascending column, then corner: a fixed order
            for (int j = 0; j < 3; ++j) inc[fill[L.geo[q].vtx[j]]++] = 3 * q + j;
    }
    CK(dalloc((void**)&S.nbrev, sizeof(int) * nbrev.size()));
    CK(dalloc((void**)&S.iptr, sizeof(int) * iptr.size()));
    CK(dalloc((void**)&S.inc, sizeof(int) * inc.size()));
    CK(dalloc((void**)&S.slot, sizeof(double) * kSlotPlanes * ncmp));
    CK(cudaMemcpyAsync(S.nbrev, nbrev.data(), sizeof(int) * nbrev.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(S.iptr, iptr.data(), sizeof(int) * iptr.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(S.inc, inc.data(), sizeof(int) * inc.size(), cudaMemcpyHostToDevice, c->stream));
    double ta = 0.0, hs = 0.0;
    for (int q = 0; q < L.N0; ++q) {
        ta += L.ppe[q].area;
        for (int k = 1; k <= L.NZ - 2; ++k) hs += L.ppe[q].area * L.lev.hmean[k];
    }
    S.tot_area = ta;
    S.hsum = hs;
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

// wall-shear weights: nu / (2 A) / (half layer height), per wall
void shear_weights(const nsmp_ctx* c, double& wb, double& wt) {
    const HostLayout& L = c->L;
    const double nu = 1.0 / c->prm.re, A = c->adj ? c->adj->tot_area : 0.0;
    wb = nu / (2.0 * A) / (0.5 * L.lev.dsv[1]);
    wt = nu / (2.0 * A) / (0.5 * L.lev.dsv[L.NZ - 2]);
}

int wall_shear_now(nsmp_ctx* c, double* tau) {
    double wb, wt;
    shear_weights(c, wb, wt);
    const Mesh& m = c->mesh;
    k_wall_shear<<<grid_for(c, m.N0), kBlock, 0, c->stream>>>(m, c->lvl[c->ln][0], wb, wt, c->red, c->d_scal);
    CKL("k_wall_shear");
    CK(cudaMemcpyAsync(c->h_scal, c->d_scal, sizeof(Scal), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *tau = c->h_scal->jval;
    return 0;
}

// state of level n + faces <-> a flat buffer of NF_STATE cell fields
int copy_state(nsmp_ctx* c, double* buf, bool save) {
    const size_t ncf = (size_t)c->L.N0 * c->L.NZ;
    double* f[NF_STATE] = {c->lvl[c->ln][0], c->lvl[c->ln][1], c->lvl[c->ln][2], c->lvl[c->ln][3],
                           c->face[0], c->face[1], c->face[2], c->face[3], c->face[4]};
    for (int q = 0; q < NF_STATE; ++q) {
        if (save) CK(cudaMemcpyAsync(buf + q * ncf, f[q], ncf * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        else CK(cudaMemcpyAsync(f[q], buf + q * ncf, ncf * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    }
    if (!save) c->lknown = c->ln;
    return 0;
}

// One SSP-RK3 step (as nsmp_step composes it); when `keep` is set the input
// of stage s (u, v, w of the known level with ghosts, then the 5 face
// fluxes) is copied to keep + s * 8 * ncf before the stage runs.  With
// `tape` the stage's PPE solution is recorded at tape + s * nprism; with
// `replay` it is taken from there instead of solving.
int rk3_step(nsmp_ctx* c, double* keep, double* tape, const double* replay, int* worst) {
    const size_t ncf = (size_t)c->L.N0 * c->L.NZ;
    c->lknown = c->ln;
    c->flag_ab = 0;
    for (int st = 0; st < 3; ++st) {
        if (keep) {
            double* k = keep + (size_t)st * 8 * ncf;
            for (int f = 0; f < 3; ++f)
                CK(cudaMemcpyAsync(k + f * ncf, c->lvl[c->lknown][f], ncf * sizeof(double), cudaMemcpyDeviceToDevice,
                                   c->stream));
            for (int f = 0; f < 5; ++f)
                CK(cudaMemcpyAsync(k + (3 + f) * ncf, c->face[f], ncf * sizeof(double), cudaMemcpyDeviceToDevice,
                                   c->stream));
        }
        nsmp_stage_info inf{};
        c->tape_x = tape ? tape + (size_t)st * c->mesh.nprism : nullptr;
        c->replay_x = replay ? replay + (size_t)st * c->mesh.nprism : nullptr;
        int rc = run_stage(c, 3, &inf);
        c->tape_x = nullptr;
        c->replay_x = nullptr;
        if (rc < 0) return rc;
        *worst = std::max(*worst, rc);
        if (st == 1) {
            rc = run_combine(c, 0.75, 0.25);
            if (rc) return rc;
        }
        if (st < 2) c->lknown = c->lnp;
    }
    int rc = run_combine(c, 1.0 / 3.0, 2.0 / 3.0);
    if (rc) return rc;
    c->ln = c->lnp;
    c->lknown = c->ln;
    return 0;
}

// Adjoint of one stage.  in: the stage input (u, v, w with ghosts, 5 face
// fluxes); Aout: adjoint of the stage output (u, v, w, p, faces; interior);
// Ain: adjoint of the stage input (overwritten; interior).
int adj_stage(nsmp_ctx* c, const double* in, double* const* Aout, double* const* Ain) {
    AdjScratch& S = *c->adj;
    const Mesh& m = c->mesh;
    const nsmp_params& P = c->prm;
    cudaStream_t st = c->stream;
    const size_t ncf = (size_t)c->L.N0 * c->L.NZ, ncmp = (size_t)m.nprism, nvx = (size_t)m.nclass * m.NZI;
    const double* U[3] = {in, in + ncf, in + 2 * ncf};
    const double* F[5] = {in + 3 * ncf, in + 4 * ncf, in + 5 * ncf, in + 6 * ncf, in + 7 * ncf};
    const int gp = grid_for(c, m.nprism), gc = grid_for(c, m.N0), gv = grid_for(c, (long long)nvx);
    for (int f = 0; f < 4; ++f) CK(cudaMemsetAsync(S.avx[f], 0, nvx * sizeof(double), st));
    CK(cudaMemsetAsync(S.apc, 0, ncmp * sizeof(double), st));
    for (int f = 0; f < NF_STATE; ++f) CK(cudaMemsetAsync(Ain[f], 0, ncf * sizeof(double), st));
    // vertex values of the stage input
    LAUNCH(NSMP_K_OTHER, k_vtx3<<<gv, kBlock, 0, st>>>(m, U[0], U[1], U[2], S.vtx[0], S.vtx[1], S.vtx[2]));
    // projection
    AdjProjArgs pa{Aout[0], Aout[1], Aout[2], Aout[3], Aout[4], Aout[5], Aout[6], Aout[7], Aout[8],
                   S.aus[0], S.aus[1], S.aus[2], S.apc, S.avx[3], P.dt};
    for (int f = 0; f < 3; ++f) CK(cudaMemsetAsync(S.aus[f], 0, ncf * sizeof(double), st));
    LAUNCH(NSMP_K_OTHER, k_adj_project<<<gp, kBlock, 0, st>>>(m, pa, S.slot));
    {
        GatherArgs ga{{S.apc, nullptr, nullptr}, {SL_L0, -1, -1}, {SL_UP, -1, -1}, {SL_DN, -1, -1}, 1};
        LAUNCH(NSMP_K_OTHER, k_gather_cells<true><<<gp, kBlock, 0, st>>>(m, S.nbrev, S.slot, ga));
        CornerArgs ca{{S.avx[3], nullptr, nullptr}, {SL_CELL, 0, 0}, 1};
        LAUNCH(NSMP_K_OTHER, k_gather_corners<<<gv, kBlock, 0, st>>>(m, S.iptr, S.inc, S.slot, ca));
    }
    LAUNCH(NSMP_K_OTHER, (k_adj_vertexT<1, true><<<gp, kBlock, 0, st>>>(m, S.tptr, S.tcls, S.tcoef, S.avx[3], nullptr,
                                                                        nullptr, S.apc, nullptr, nullptr)));
    CK(cudaMemsetAsync(S.avx[3], 0, nvx * sizeof(double), st));
    // mean removals and the solve
    LAUNCH(NSMP_K_OTHER, k_adj_sum<<<gp, kBlock, 0, st>>>(m, S.apc, c->red, c->d_scal));
    LAUNCH(NSMP_K_OTHER, k_adj_solve_rhs<<<gp, kBlock, 0, st>>>(m, S.apc, c->rhsp, S.hsum, c->red, c->d_scal));
    LAUNCH(NSMP_K_OTHER, k_adj_unit<<<gp, kBlock, 0, st>>>(m, c->rhsp, c->d_scal));
    CKL("adjoint pressure right-hand side");
    LAUNCH(NSMP_K_OTHER, k_adj_guess<<<gp, kBlock, 0, st>>>(m, S.lamc, S.guess, c->d_scal));
    const double* lam = nullptr;
    int rc = (c->precision == NSMP_MIXED) ? run_pressure_mixed(c, S.guess, &lam) : run_pressure_fp64(c, S.guess, &lam);
    if (rc < 0) return rc;
    CK(cudaMemcpyAsync(c->h_scal, c->d_scal, sizeof(Scal), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    c->bicg_iters += c->h_scal->iter;
    if (c->h_scal->status < 0) {
        c->err = "adjoint pressure solve: non-finite residual";
        return c->h_scal->status;
    }
    rc = std::max(rc, c->h_scal->status);
    LAUNCH(NSMP_K_OTHER, k_adj_sum<<<gp, kBlock, 0, st>>>(m, lam, c->red, c->d_scal));
    LAUNCH(NSMP_K_OTHER, k_adj_center<<<gp, kBlock, 0, st>>>(m, lam, S.arhs, c->d_scal));
    LAUNCH(NSMP_K_OTHER, k_adj_keep<<<gp, kBlock, 0, st>>>(m, lam, S.lamc, c->d_scal));
    // face pass
    AdjFaceArgs fa{S.arhs, Aout[4], Aout[5], Aout[6], Aout[7], Aout[8], S.aus[0], S.aus[1], S.aus[2], S.avx[3],
                   1.0 / P.dt};
    LAUNCH(NSMP_K_OTHER, k_adj_faces<<<gp, kBlock, 0, st>>>(m, fa, S.slot));
    {
        GatherArgs ga{{S.aus[0], S.aus[1], S.aus[2]}, {SF_U, SF_V, -1}, {-1, -1, SF_WUP}, {-1, -1, SF_WDN}, 3};
        LAUNCH(NSMP_K_OTHER, k_gather_cells<false><<<gp, kBlock, 0, st>>>(m, S.nbrev, S.slot, ga));
        CornerArgs ca{{S.avx[3], nullptr, nullptr}, {SF_PC, 0, 0}, 1};
        LAUNCH(NSMP_K_OTHER, k_gather_corners<<<gv, kBlock, 0, st>>>(m, S.iptr, S.inc, S.slot, ca));
    }
    LAUNCH(NSMP_K_OTHER, k_adj_fold<<<gc, kBlock, 0, st>>>(m, S.aus[0], S.aus[1], S.aus[2], nullptr));
    // stage right-hand side
    AdjStageArgs sa;
    sa.u = U[0]; sa.v = U[1]; sa.w = U[2];
    sa.uv = S.vtx[0]; sa.vv = S.vtx[1]; sa.wv = S.vtx[2];
    sa.f1 = F[0]; sa.f2 = F[1]; sa.f3 = F[2]; sa.fT = F[3]; sa.fB = F[4];
    sa.aus = S.aus[0]; sa.avs = S.aus[1]; sa.aws = S.aus[2];
    sa.au = Ain[0]; sa.av = Ain[1]; sa.aw = Ain[2];
    sa.slot = S.slot;
    sa.af1 = Ain[4]; sa.af2 = Ain[5]; sa.af3 = Ain[6]; sa.afT = Ain[7]; sa.afB = Ain[8];
    sa.afx = S.afx;
    sa.c1 = 1.0; sa.dt = P.dt; sa.inv_re = 1.0 / P.re;
    sa.les = P.les; sa.les_van = P.les_van;
    LAUNCH(NSMP_K_OTHER, k_adj_stage<<<gp, kBlock, 0, st>>>(m, sa));
    {
        GatherArgs ga{{Ain[0], Ain[1], Ain[2]}, {SL_L0, 8 + SL_L0, 16 + SL_L0}, {SL_UP, 8 + SL_UP, 16 + SL_UP},
                      {SL_DN, 8 + SL_DN, 16 + SL_DN}, 3};
        LAUNCH(NSMP_K_OTHER, k_gather_cells<false><<<gp, kBlock, 0, st>>>(m, S.nbrev, S.slot, ga));
        CornerArgs ca{{S.avx[0], S.avx[1], S.avx[2]}, {SL_CELL, 8 + SL_CELL, 16 + SL_CELL}, 3};
        LAUNCH(NSMP_K_OTHER, k_gather_corners<<<gv, kBlock, 0, st>>>(m, S.iptr, S.inc, S.slot, ca));
    }
    LAUNCH(NSMP_K_OTHER, k_adj_fold<<<gc, kBlock, 0, st>>>(m, Ain[0], Ain[1], Ain[2], nullptr));
    // vertex transposes: velocity vertex values and the vertex p of the input
    LAUNCH(NSMP_K_OTHER, (k_adj_vertexT<3, false><<<gp, kBlock, 0, st>>>(m, S.tptr, S.tcls, S.tcoef, S.avx[0],
                                                                         S.avx[1], S.avx[2], Ain[0], Ain[1], Ain[2])));
    LAUNCH(NSMP_K_OTHER, (k_adj_vertexT<1, false><<<gp, kBlock, 0, st>>>(m, S.tptr, S.tcls, S.tcoef, S.avx[3],
                                                                         nullptr, nullptr, Ain[3], nullptr, nullptr)));
    CKL("adjoint stage");
    return rc;
}

struct DevBuf {  // per-call device buffer
    double* p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
};

}  // namespace

int adj_ensure(nsmp_ctx* c) { return adj_alloc(c); }

void adj_free(nsmp_ctx* c) {
    delete c->adj;  // device buffers are in c->allocs
    c->adj = nullptr;
}

int run_set_body_force(nsmp_ctx* c, const double* fx) {
    const size_t ncf = (size_t)c->L.N0 * c->L.NZ;
    if (!fx) {
        c->fx = nullptr;
        return 0;
    }
    if (!c->adj) {
        int rc = adj_alloc(c);
        if (rc) return rc;
    }
    if (!c->adj->fx_host_stage) {
        cudaError_t e = cudaMalloc((void**)&c->adj->fx_host_stage, ncf * sizeof(double));
        if (e != cudaSuccess) return cuda_fail(c, e, "cudaMalloc(body force)");
        c->allocs.push_back(c->adj->fx_host_stage);
    }
    // (N0,NZ) host array -> (N_CELL,NZ)-shaped staging -> device columns
    const int N0 = c->L.N0, NZ = c->L.NZ, NC = c->L.NC;
    std::vector<double> wide((size_t)NC * NZ, 0.0);
    for (int k = 0; k < NZ; ++k)
        std::copy(fx + (size_t)k * N0, fx + (size_t)(k + 1) * N0, wide.begin() + (size_t)k * NC);
    int rc = run_scatter(c, wide.data(), c->adj->fx_host_stage);
    if (rc) return rc;
    // the ghost layers carry no force
    const Mesh& m = c->mesh;
    CK(cudaMemcpy2DAsync(c->adj->fx_host_stage, NZ * sizeof(double), c->adj->zero, NZ * sizeof(double),
                         sizeof(double), m.N0, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemcpy2DAsync(c->adj->fx_host_stage + NZ - 1, NZ * sizeof(double), c->adj->zero, NZ * sizeof(double),
                         sizeof(double), m.N0, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    c->fx = c->adj->fx_host_stage;
    return 0;
}

int run_wall_shear(nsmp_ctx* c, double* tau) {
    if (!c->adj) {
        int rc = adj_alloc(c);
        if (rc) return rc;
    }
    return wall_shear_now(c, tau);
}

int run_apply_A(nsmp_ctx* c, int transpose, const double* x, double* y) {
    if (!c->adj) {
        int rc = adj_alloc(c);
        if (rc) return rc;
    }
    AdjScratch& S = *c->adj;
    const int N0 = c->L.N0, NZ = c->L.NZ, NC = c->L.NC;
    std::vector<double> wide((size_t)NC * NZ, 0.0);
    for (int k = 1; k < NZ - 1; ++k)
        std::copy(x + (size_t)k * N0, x + (size_t)(k + 1) * N0, wide.begin() + (size_t)k * NC);
    int rc = run_scatter(c, wide.data(), S.A[0][0]);
    if (rc) return rc;
    const size_t ncf = (size_t)N0 * NZ;
    CK(cudaMemsetAsync(S.A[0][1], 0, ncf * sizeof(double), c->stream));
    k_apply_A<<<grid_for(c, c->mesh.nprism), kBlock, 0, c->stream>>>(c->mesh, transpose, S.A[0][0], S.A[0][1]);
    CKL("k_apply_A");
    return run_gather(c, S.A[0][1], 0, N0, y);
}

int run_adjoint(nsmp_ctx* c, int nsteps, int ckpt_every, const double* fx, double* grad, double* J) {
    int rc = adj_alloc(c);
    if (rc) return rc;
    AdjScratch& S = *c->adj;
    if (!S.pairing_ok) {
        c->err = "nsmp_adjoint: a column meets a neighbour over two periodic edges (mesh of fewer than 3 quads "
                 "across); the transposed stencils cannot pair its edges";
        return NSMP_ERR_MESH;
    }
    const Mesh& m = c->mesh;
    cudaStream_t st = c->stream;
    const size_t ncf = (size_t)c->L.N0 * c->L.NZ;
    const int nseg = (nsteps + ckpt_every - 1) / ckpt_every;
    rc = run_set_body_force(c, fx);
    if (rc) return rc;
    cudaError_t e = cudaSuccess;
    // checkpoints (state at the start of every segment and at the end), the
    // stage inputs of one segment, and the PPE solution of every stage (the
    // recomputation of a segment replays those instead of solving again)
    DevBuf ck, seg, tape;
    const size_t np3 = (size_t)3 * m.nprism;
    e = cudaMalloc((void**)&tape.p, (size_t)nsteps * np3 * sizeof(double));
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaMalloc(adjoint pressure tape)");
    e = cudaMalloc((void**)&ck.p, (size_t)(nseg + 1) * NF_STATE * ncf * sizeof(double));
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaMalloc(adjoint checkpoints)");
    // The stage inputs of a whole segment (24 cell fields per step) when they
    // fit in 80 % of the free device memory; else inner checkpoints every q
    // steps of the segment (q ~ sqrt(ckpt_every)) and the stage inputs of the
    // one step being reversed, each step re-reached by replaying at most
    // q - 1 steps (replays skip the PPE solve: ~5 % of a step each).
    size_t free_b = 0, total_b = 0;
    CK(cudaMemGetInfo(&free_b, &total_b));
    const size_t seg_all = (size_t)ckpt_every * 3 * 8 * ncf * sizeof(double);
    const double budget = S.seg_budget > 0.0 ? S.seg_budget : 0.8 * (double)free_b;
    const bool inner = (double)seg_all > budget;
    int q = 1;
    while ((long long)q * q < ckpt_every) ++q;
    const int ninner = (ckpt_every + q - 1) / q;
    if (!inner) {
        e = cudaMalloc((void**)&seg.p, seg_all);
    } else {
        e = cudaMalloc((void**)&seg.p, ((size_t)ninner * NF_STATE + 3 * 8) * ncf * sizeof(double));
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaMalloc(adjoint segment)");
    double* inner_ck = inner ? seg.p + (size_t)3 * 8 * ncf : nullptr;
    double wb, wt;
    shear_weights(c, wb, wt);
    // forward sweep
    int worst = 0;
    double jsum = 0.0;
    for (int n = 0; n < nsteps; ++n) {
        if (n % ckpt_every == 0) {
            rc = copy_state(c, ck.p + (size_t)(n / ckpt_every) * NF_STATE * ncf, true);
            if (rc) return rc;
        }
        rc = rk3_step(c, nullptr, tape.p + (size_t)n * np3, nullptr, &worst);
        if (rc) return rc;
        double tau;
        rc = wall_shear_now(c, &tau);
        if (rc) return rc;
        jsum += tau;
    }
    rc = copy_state(c, ck.p + (size_t)nseg * NF_STATE * ncf, true);
    if (rc) return rc;
    if (J) *J = jsum / nsteps;
    // reverse sweep
    double* const* A = S.A[0];
    double* const* B = S.A[1];
    for (int f = 0; f < NF_STATE; ++f) CK(cudaMemsetAsync(A[f], 0, ncf * sizeof(double), st));
    CK(cudaMemsetAsync(S.afx, 0, ncf * sizeof(double), st));
    CK(cudaMemsetAsync(S.lamc, 0, ncf * sizeof(double), st));
    const int gc = grid_for(c, m.N0), ga = grid_for(c, (long long)ncf);
    for (int sgi = nseg - 1; sgi >= 0; --sgi) {
        const int n0 = sgi * ckpt_every, n1 = std::min(nsteps, n0 + ckpt_every);
        rc = copy_state(c, ck.p + (size_t)sgi * NF_STATE * ncf, false);
        if (rc) return rc;
        for (int n = n0; n < n1; ++n) {
            if (inner && (n - n0) % q == 0) {
                rc = copy_state(c, inner_ck + (size_t)((n - n0) / q) * NF_STATE * ncf, true);
                if (rc) return rc;
            }
            double* keep = inner ? nullptr : seg.p + (size_t)(n - n0) * 3 * 8 * ncf;
            rc = rk3_step(c, keep, nullptr, tape.p + (size_t)n * np3, &worst);
            if (rc) return rc;
        }
        for (int n = n1 - 1; n >= n0; --n) {
            const double* keep = seg.p + (size_t)(inner ? 0 : n - n0) * 3 * 8 * ncf;
            if (inner) {  // re-reach step n from the inner checkpoint below it
                const int j = (n - n0) / q;
                rc = copy_state(c, inner_ck + (size_t)j * NF_STATE * ncf, false);
                if (rc) return rc;
                for (int n2 = n0 + j * q; n2 < n; ++n2) {
                    rc = rk3_step(c, nullptr, nullptr, tape.p + (size_t)n2 * np3, &worst);
                    if (rc) return rc;
                }
                rc = rk3_step(c, seg.p, nullptr, tape.p + (size_t)n * np3, &worst);
                if (rc) return rc;
            }
            // objective at u^{n+1}
            k_adj_seed<<<gc, kBlock, 0, st>>>(m, A[0], wb / nsteps, wt / nsteps);
            CKL("k_adj_seed");
            // u^{n+1} = 1/3 u^n + 2/3 S3: split the velocity adjoint
            for (int f = 0; f < 3; ++f) {
                CK(cudaMemcpyAsync(S.acc[f], A[f], ncf * sizeof(double), cudaMemcpyDeviceToDevice, st));
                k_axpby<<<ga, kBlock, 0, st>>>(ncf, 0.0, A[f], 1.0 / 3.0, S.acc[f]);
                k_axpby<<<ga, kBlock, 0, st>>>(ncf, 0.0, A[f], 2.0 / 3.0, A[f]);
            }
            rc = adj_stage(c, keep + 2 * 8 * ncf, A, B);  // stage 3
            if (rc < 0) return rc;
            worst = std::max(worst, rc);
            // u2 = 3/4 u^n + 1/4 S2
            for (int f = 0; f < 3; ++f) {
                k_axpby<<<ga, kBlock, 0, st>>>(ncf, 0.75, B[f], 1.0, S.acc[f]);
                k_axpby<<<ga, kBlock, 0, st>>>(ncf, 0.0, B[f], 0.25, B[f]);
            }
            rc = adj_stage(c, keep + 1 * 8 * ncf, B, A);  // stage 2
            if (rc < 0) return rc;
            worst = std::max(worst, rc);
            rc = adj_stage(c, keep, A, B);                // stage 1
            if (rc < 0) return rc;
            worst = std::max(worst, rc);
            for (int f = 0; f < 3; ++f) k_axpby<<<ga, kBlock, 0, st>>>(ncf, 1.0, S.acc[f], 1.0, B[f]);
            CKL("adjoint step");
            for (int f = 0; f < NF_STATE; ++f)
                CK(cudaMemcpyAsync(A[f], B[f], ncf * sizeof(double), cudaMemcpyDeviceToDevice, st));
        }
    }
    // leave the context at the end of the forward run
    rc = copy_state(c, ck.p + (size_t)nseg * NF_STATE * ncf, false);
    if (rc) return rc;
    if (grad) {
        rc = run_gather(c, S.afx, 0, c->L.N0, grad);
        if (rc) return rc;
    }
    CK(cudaStreamSynchronize(st));
    return worst;
}

}  // namespace nsmp

extern "C" {

int nsmp_set_body_force(nsmp_ctx* c, const double* fx) {
    if (!c) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    return nsmp::run_set_body_force(c, fx);
}

int nsmp_wall_shear(nsmp_ctx* c, double* tau) {
    if (!c || !tau) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    return nsmp::run_wall_shear(c, tau);
}

int nsmp_set_adjoint_budget(nsmp_ctx* c, double bytes) {
    if (!c || bytes < 0.0) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    if (!c->adj) {
        int rc = nsmp::adj_ensure(c);
        if (rc) return rc;
    }
    c->adj->seg_budget = bytes;
    return NSMP_OK;
}

int nsmp_apply_A(nsmp_ctx* c, const double* x, double* y) {
    if (!c || !x || !y) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    return nsmp::run_apply_A(c, 0, x, y);
}

int nsmp_apply_AT(nsmp_ctx* c, const double* x, double* y) {
    if (!c || !x || !y) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    return nsmp::run_apply_A(c, 1, x, y);
}

int nsmp_adjoint(nsmp_ctx* c, int nsteps, int ckpt_every, const double* fx, double* grad_out, double* J_out) {
    if (!c || nsteps < 1 || ckpt_every < 1 || !fx) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    try {
        return nsmp::run_adjoint(c, nsteps, ckpt_every, fx, grad_out, J_out);
    } catch (...) {
        c->err = "host exception in nsmp_adjoint";
        return NSMP_ERR_CUDA;
    }
}

}  // extern "C"
