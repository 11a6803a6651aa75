// Device-side data structures and helpers shared by the kernels.
#pragma once
#include <cuda_runtime.h>

#include "layout.h"

namespace nsmp {

constexpr int kBlock = 256;   // threads per block of every per-prism kernel
constexpr int kMaxRed = 8;    // values reduced at once

// Per-layer factor rows of the level table (lev[row*NZ + k0]).
enum LevRow {
    LV_DSV = 0, LV_IDSV, LV_IDST, LV_IDSB, LV_IDSBU, LV_WT, LV_WB, LV_GZP, LV_GZM, LV_HMEAN,
    LV_DD, LV_KD, LV_DAMP, LV_IHZ, LV_ATOP, LV_ABOT, LV_CFLD, LV_CFLH, LV_COUNT
};

// Scalars of one stage kept in device memory between kernels.
struct Scal {
    double sum_rhs;        // sum of the PPE right-hand side (Glob_Norm, tags = 1)
    double avec_p;         // volume mean of the solution (Glob_Norm, tags = 0)
    double max_eddy;
    double rho, rho_prev, alpha, omega, r0v, ts, tt;
    double b1, b2, r1, r2, e1, e2;
    double diag[4];
    double jval, jsum;     // wall-shear objective, adjoint mean-removal sum
    double adjn;           // |rhs|_2 of the adjoint pressure solve
    int iter, done, converged, status;
    int max_iters, pad;
    double eps;
    // mixed precision: FP32 BiCGSTAB with FP64 reliable updates
    double ib1, ib2, ir1, ir2, irho, irho_prev, ialpha, iomega, ir0v;
    double inner_tol;      // reduction of the FP32 residual that triggers an FP64 update
    double iscale;         // residual RMS at the start of the solve (FP32 values are r / iscale)
    double theta;          // minimal-residual step of the last FP64 update
    double r2sq, rsum;     // |r|_2^2 and sum of the current FP64 residual
    double rmean, emean;   // plain means of the FP64 residual and of the FP32 correction
    double ise, isy;       // sum of e and of D^-1 p formed by the p/v pass
    int iiter;             // iterations since the last Krylov restart (0: p = r)
    int ksince;            // iterations since the last FP64 update
    int outer;             // FP64 updates done
    int pending;           // 1: FP64 update requested
    int restart;           // 1: restart the Krylov process at the next update
    int perturb;           // 1: perturb the shadow residual at that restart
    int verify;            // 1: the next FP64 update recomputes b - A x to confirm convergence
    int has_e;             // 1: e holds a correction
    int einc;              // 1: e lacks D^-1 (alpha p + omega s) of the last iteration
    int rfresh;            // 1: r was set by an FP64 update (else r = s - omega t)
    int inner_cap;         // most FP32 iterations between two FP64 updates
    int cur;               // buffer holding the current x and r
    int restart_every;     // most FP32 iterations of one Krylov process
    // per-update record of the last mixed solve (diagnostics)
    static constexpr int kCycLog = 48;
    int cyc_it[kCycLog];
    float cyc_in[kCycLog], cyc_out[kCycLog];
    int cyc_acc[kCycLog];
};

// Everything a kernel needs to address the mesh; passed by value.
struct Mesh {
    int N0, NZ, NZI, nclass;
    int nprism;            // N0*NZI
    const ColPPE* ppe;
    const ColGeo* geo;
    const int* vptr;
    const int* vcell;
    const double* vcoef;
    const double* lev;     // LV_COUNT x NZ
    const ColGeo32* geo32; // FP32 copies for the FP32 stage arithmetic (null until used)
    const float* levf;
    double sgn_bot[3], sgn_top[3];
    double tv_lsig;        // TotalVolume*(SigFin-SigIni)
};

// Reduction scratch: per-block partial values and the arrival counter used to
// elect the last block (which then sums the partials in block order, so the
// result is deterministic for a fixed grid).
struct RedScratch {
    double* partials;      // gridDim.x * kMaxRed
    unsigned int* counter;
};

__device__ __forceinline__ double lev(const Mesh& m, int row, int k0) { return __ldg(m.lev + row * m.NZ + k0); }

__device__ __forceinline__ size_t IX(const Mesh& m, int c, int k0) { return (size_t)c * m.NZ + k0; }
__device__ __forceinline__ size_t IV(const Mesh& m, int v, int k0) { return (size_t)v * m.NZI + (k0 - 1); }

template <int N>
struct Vec {
    double v[N];
};

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    return x;
}
__device__ __forceinline__ double warp_max(double x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_down_sync(0xffffffffu, x, o));
    return x;
}

// Block-wide reduction of N values (sum or max); the result is valid in
// thread 0.  Fixed tree order: deterministic.
template <int N, bool MAX>
__device__ __forceinline__ void block_reduce(double (&x)[N]) {
    __shared__ double sh[kBlock / 32][N];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < N; ++q) x[q] = MAX ? warp_max(x[q]) : warp_sum(x[q]);
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < N; ++q) sh[wid][q] = x[q];
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int q = 0; q < N; ++q) {
            double y = (lane < kBlock / 32) ? sh[lane][q] : (MAX ? -INFINITY : 0.0);
            x[q] = MAX ? warp_max(y) : warp_sum(y);
        }
    }
    __syncthreads();
}

// Last-block part of a grid reduction: x (valid in thread 0) is this block's
// contribution; the last block to arrive gets the totals in `tot` (all its
// threads) and returns true.  The counter is reset by the last block so the
// scratch is reusable by the next launch.
template <int N, bool MAX>
__device__ bool grid_finish(const double (&x)[N], RedScratch rs, double (&tot)[N]) {
    __shared__ bool last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < N; ++q) rs.partials[blockIdx.x * kMaxRed + q] = x[q];
        __threadfence();
        unsigned int prev = atomicAdd(rs.counter, 1u);
        last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double y[N];
#pragma unroll
    for (int q = 0; q < N; ++q) y[q] = MAX ? -INFINITY : 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
#pragma unroll
        for (int q = 0; q < N; ++q) {
            double p = __ldcg(rs.partials + b * kMaxRed + q);
            y[q] = MAX ? fmax(y[q], p) : y[q] + p;
        }
    block_reduce<N, MAX>(y);
    __shared__ double res[N];
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < N; ++q) res[q] = y[q];
        *rs.counter = 0u;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < N; ++q) tot[q] = res[q];
    return true;
}

// Grid reduction of FP64 values (sum or max), fixed order: deterministic for
// a fixed grid.
template <int N, bool MAX>
__device__ bool grid_reduce(double (&x)[N], RedScratch rs, double (&tot)[N]) {
    block_reduce<N, MAX>(x);
    return grid_finish<N, MAX>(x, rs, tot);
}

// Programmatic dependent launch.  A kernel launched with programmatic stream
// serialization (launch_pdl) may be scheduled while its predecessor in the
// stream drains; it waits here until the predecessor has completed and its
// memory is visible, then releases its own dependent launch.  A dependent
// grid is launched only after every block of its predecessor has started, so
// its waiting blocks never hold back a block of the predecessor.  Both
// instructions are no-ops for an ordinary launch.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Double-float arithmetic: a value is an unevaluated sum h + l of two FP32
// numbers with |l| <= ulp(h)/2, about 48 significant bits.  The algorithms
// are the published error-free transformations: TwoSum (Knuth, TAOCP vol. 2),
// Fast2Sum (Dekker 1971), the FMA-based exact product, and the accurate
// double-double addition of Hida, Li and Bailey (2001).  Every operation is
// an explicitly rounded intrinsic, so the compiler cannot contract or
// reorder the error terms away.  Used where FP64 issue rate, not accuracy,
// is the constraint (about 2 FP64 instructions per SM clock on this GPU).
struct F2 {
    float h, l;
};
__device__ __forceinline__ F2 two_sum(float a, float b) {  // exact: a + b = s + e
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
__device__ __forceinline__ F2 fast_two_sum(float a, float b) {  // exact when |a| >= |b| or a == 0
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ F2 df_add(F2 a, F2 b) {
    F2 s = two_sum(a.h, b.h);
    const F2 t = two_sum(a.l, b.l);
    s.l = __fadd_rn(s.l, t.h);
    s = fast_two_sum(s.h, s.l);
    s.l = __fadd_rn(s.l, t.l);
    return fast_two_sum(s.h, s.l);
}
__device__ __forceinline__ F2 df_mul(F2 a, F2 b) {
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);  // exact error of the product
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return fast_two_sum(p, e);
}

// Grid sum of FP32 per-thread values: FP32 inside each warp (a 32-value tree,
// relative error at most 5 units of FP32 rounding), FP64 across warps and
// blocks.  Used by the FP32 inner solver, whose values are formed in FP32
// anyway; it keeps FP64 instructions (a few per SM cycle on this GPU) out of
// the bandwidth-bound passes.
template <int N>
__device__ bool grid_reduce_f(float (&x)[N], RedScratch rs, double (&tot)[N]) {
    __shared__ double sh[kBlock / 32][N];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < N; ++q) {
        float y = x[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) y += __shfl_down_sync(0xffffffffu, y, o);
        if (lane == 0) sh[wid][q] = (double)y;
    }
    __syncthreads();
    double d[N];
#pragma unroll
    for (int q = 0; q < N; ++q) d[q] = 0.0;
    if (wid == 0) {
#pragma unroll
        for (int q = 0; q < N; ++q) {
            double y = (lane < kBlock / 32) ? sh[lane][q] : 0.0;
#pragma unroll
            for (int o = kBlock / 64; o > 0; o >>= 1) y += __shfl_down_sync(0xffffffffu, y, o);
            d[q] = y;
        }
    }
    __syncthreads();
    return grid_finish<N, false>(d, rs, tot);
}

}  // namespace nsmp
