// Per-prism quantities of glob_cfl (Main/cfl.F90:84-184), shared by the
// allocating diagnostic (diag.cu) and its no-allocation variant (noalloc.cu).
#pragma once
#include "kern_common.cuh"

namespace nsmp {

// One interior prism's contribution to glob_cfl.  Every operation is an
// explicitly rounded intrinsic in the reference's evaluation order, so no
// multiply-add is contracted and each prism's values equal the reference's
// unfused FP64 arithmetic bit for bit; only the order of the global sums
// differs.
struct CflCell {
    double flux;   // net outflow: sum_j U_j dlVV_j h_div + UT area + UB area   (cfl.F90:138-147)
    double cfl;    // 0.5 dt (sum_j |U_j dlVV_j h| + |UB area| + |UT area|) / (area h)  (:140, 149-152)
    double side;   // sum over lateral boundary edges of U_j dlVV_j h           (:141-150)
    double bot;    // UB area at the first interior layer (bcbot = 1), else 0   (:171-175)
    double top;    // UT area at the last interior layer (bctop = 1), else 0    (:177-181)
};

// h_div = dsig(k-1) and h = dsig(k) as shipped, the cell height dsigv(k-1)
// for both when the reference's quirks are off (level rows LV_CFLD, LV_CFLH).
__device__ __forceinline__ CflCell cfl_cell(const Mesh& m, const double* f1, const double* f2, const double* f3,
                                            const double* fT, const double* fB, double dt, int c, int k0) {
    const ColGeo& G = m.geo[c];
    const size_t q = IX(m, c, k0);
    const double hd = lev(m, LV_CFLD, k0), hc = lev(m, LV_CFLH, k0);
    const double uf[3] = {f1[q], f2[q], f3[q]};
    CflCell o;
    double flux = 0.0, fc = 0.0, side = 0.0;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        const double ul = __dmul_rn(uf[j], G.L[j]);
        flux = __dadd_rn(flux, __dmul_rn(ul, hd));
        const double t = __dmul_rn(ul, hc);
        fc = __dadd_rn(fc, fabs(t));
        if ((G.bnd >> j) & 1) side = __dadd_rn(side, t);
    }
    const double ta = __dmul_rn(fT[q], G.area), ba = __dmul_rn(fB[q], G.area);
    flux = __dadd_rn(flux, ta);
    flux = __dadd_rn(flux, ba);
    fc = __dadd_rn(__dadd_rn(fc, fabs(ba)), fabs(ta));
    o.flux = flux;
    o.cfl = __ddiv_rn(__dmul_rn(__dmul_rn(0.5, dt), fc), __dmul_rn(G.area, hc));
    o.side = side;
    o.bot = (k0 == 1) ? ba : 0.0;
    o.top = (k0 == m.NZ - 2) ? ta : 0.0;
    return o;
}

// Position of a prism in the reference's loop order (k outer, original cell
// number inner): the signed maxima keep the first value of largest modulus.
__device__ __forceinline__ unsigned long long cfl_order(const Mesh& m, int c, int k0) {
    return (unsigned long long)(k0 - 1) * (unsigned long long)m.N0 + (unsigned long long)m.geo[c].orig;
}

// Signed value of largest modulus with its loop position.  The reference
// replaces its running value only on a strictly larger modulus, starting
// from 0 (cfl.F90:99-101, 167-168): the result is the first value of largest
// modulus in loop order, 0 when all are 0; NaN never replaces it.
struct ArgAbs {
    double a, v;
    unsigned long long ord;
};
__device__ __forceinline__ ArgAbs argabs_none() { return {0.0, 0.0, ~0ull}; }
__device__ __forceinline__ ArgAbs argabs_of(double v, unsigned long long ord) {
    const double a = fabs(v);
    return (a > 0.0) ? ArgAbs{a, v, ord} : argabs_none();
}
__device__ __forceinline__ ArgAbs argabs_merge(const ArgAbs& x, const ArgAbs& y) {
    const bool take_y = (y.a > x.a) || (y.a == x.a && y.ord < x.ord);
    return take_y ? y : x;
}
__device__ __forceinline__ ArgAbs argabs_shfl_down(const ArgAbs& x, int o) {
    ArgAbs y;
    y.a = __shfl_down_sync(0xffffffffu, x.a, o);
    y.v = __shfl_down_sync(0xffffffffu, x.v, o);
    y.ord = __shfl_down_sync(0xffffffffu, x.ord, o);
    return y;
}

}  // namespace nsmp
