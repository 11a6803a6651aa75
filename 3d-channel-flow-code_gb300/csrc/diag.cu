// Device glob_cfl (Main/cfl.F90:7-269): velocity maxima, volume means,
// CFL number and the mass-flux checks, FP64 on the device.
//
// Two launches and no atomics: k_cfl_diag reduces each block's prisms into
// one record of partials, k_cfl_final (one block) combines the records in
// block order with a fixed tree.  Results are deterministic for a fixed
// grid; maxima and signed maxima equal the reference's exactly, sums differ
// from its single running accumulator by summation order only.
#include "diag.cuh"

namespace nsmp {
namespace {

// Partial record of one block (doubles): 8 sums, the CFL maximum, then
// four (modulus, value, order) triples for u, v, w and the net flux.
enum { CS_ABSDIV = 0, CS_FLUX, CS_MU, CS_MV, CS_MW, CS_BOT, CS_TOP, CS_SIDE, CS_NSUM };
constexpr int kCflRec = 24;  // CS_NSUM sums + 1 max + 4 x 3, padded

struct CflArgs {
    const double *u, *v, *w;               // level-n cell fields
    const double *f1, *f2, *f3, *fT, *fB;  // face fluxes
    double dt;
};

__device__ void argabs_block(ArgAbs (&x)[4]) {
    __shared__ double sa[kBlock / 32][4], sv[kBlock / 32][4];
    __shared__ unsigned long long so[kBlock / 32][4];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x[q] = argabs_merge(x[q], argabs_shfl_down(x[q], o));
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < 4; ++q) { sa[wid][q] = x[q].a; sv[wid][q] = x[q].v; so[wid][q] = x[q].ord; }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            ArgAbs y = argabs_none();
            if (lane < kBlock / 32) y = ArgAbs{sa[lane][q], sv[lane][q], so[lane][q]};
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) y = argabs_merge(y, argabs_shfl_down(y, o));
            x[q] = y;
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kBlock) k_cfl_diag(Mesh m, CflArgs a, double* rec) {
    double s[CS_NSUM];
#pragma unroll
    for (int q = 0; q < CS_NSUM; ++q) s[q] = 0.0;
    double cmax[1] = {0.0};
    ArgAbs am[4] = {argabs_none(), argabs_none(), argabs_none(), argabs_none()};
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < m.nprism; g += gridDim.x * blockDim.x) {
        int c, k0;
        prism_of(m, g, c, k0);
        const CflCell o = cfl_cell(m, a.f1, a.f2, a.f3, a.fT, a.fB, a.dt, c, k0);
        const size_t q = IX(m, c, k0);
        const double u = a.u[q], v = a.v[q], w = a.w[q];
        // sumu = phiu(i,k) areaCell(i) dsig(k) + sumu (cfl.F90:108-110)
        const double ah = lev(m, LV_CFLH, k0);
        const double area = m.geo[c].area;
        s[CS_ABSDIV] += fabs(o.flux);
        s[CS_FLUX] += o.flux;
        s[CS_MU] += __dmul_rn(__dmul_rn(u, area), ah);
        s[CS_MV] += __dmul_rn(__dmul_rn(v, area), ah);
        s[CS_MW] += __dmul_rn(__dmul_rn(w, area), ah);
        s[CS_BOT] += o.bot;
        s[CS_TOP] += o.top;
        s[CS_SIDE] += o.side;
        cmax[0] = fmax(cmax[0], o.cfl);
        const unsigned long long ord = cfl_order(m, c, k0);
        am[0] = argabs_merge(am[0], argabs_of(u, ord));
        am[1] = argabs_merge(am[1], argabs_of(v, ord));
        am[2] = argabs_merge(am[2], argabs_of(w, ord));
        am[3] = argabs_merge(am[3], argabs_of(o.flux, ord));
    }
    block_reduce<CS_NSUM, false>(s);
    block_reduce<1, true>(cmax);
    argabs_block(am);
    if (threadIdx.x == 0) {
        double* r = rec + (size_t)blockIdx.x * kCflRec;
#pragma unroll
        for (int q = 0; q < CS_NSUM; ++q) r[q] = s[q];
        r[CS_NSUM] = cmax[0];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            r[CS_NSUM + 1 + 3 * q] = am[q].a;
            r[CS_NSUM + 2 + 3 * q] = am[q].v;
            r[CS_NSUM + 3 + 3 * q] = __longlong_as_double((long long)am[q].ord);
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_cfl_final(int nblocks, double tv_lsig, const double* rec, double* out) {
    double s[CS_NSUM];
#pragma unroll
    for (int q = 0; q < CS_NSUM; ++q) s[q] = 0.0;
    double cmax[1] = {0.0};
    ArgAbs am[4] = {argabs_none(), argabs_none(), argabs_none(), argabs_none()};
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        const double* r = rec + (size_t)b * kCflRec;
#pragma unroll
        for (int q = 0; q < CS_NSUM; ++q) s[q] += r[q];
        cmax[0] = fmax(cmax[0], r[CS_NSUM]);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const ArgAbs y{r[CS_NSUM + 1 + 3 * q], r[CS_NSUM + 2 + 3 * q],
                           (unsigned long long)__double_as_longlong(r[CS_NSUM + 3 + 3 * q])};
            am[q] = argabs_merge(am[q], y);
        }
    }
    block_reduce<CS_NSUM, false>(s);
    block_reduce<1, true>(cmax);
    argabs_block(am);
    if (threadIdx.x == 0) {
        out[NSMP_CFL_UMAX] = am[0].v;
        out[NSMP_CFL_VMAX] = am[1].v;
        out[NSMP_CFL_WMAX] = am[2].v;
        out[NSMP_CFL_AVEU] = s[CS_MU] / tv_lsig;  // Vol = TotalVolume (SigFin - SigIni)
        out[NSMP_CFL_AVEV] = s[CS_MV] / tv_lsig;
        out[NSMP_CFL_AVEW] = s[CS_MW] / tv_lsig;
        out[NSMP_CFL_MAX] = cmax[0];
        out[NSMP_CFL_FLUX_TOTAL] = s[CS_FLUX];
        out[NSMP_CFL_FLUX_MAX] = am[3].v;
        out[NSMP_CFL_FLUX_BC] = (s[CS_BOT] + s[CS_TOP]) + s[CS_SIDE];
        out[NSMP_CFL_FLUX_BOT] = s[CS_BOT];
        out[NSMP_CFL_FLUX_TOP] = s[CS_TOP];
        out[NSMP_CFL_FLUX_SIDE] = s[CS_SIDE];
        out[NSMP_CFL_ABS_DIV] = s[CS_ABSDIV];
    }
}

}  // namespace

int run_cfl_diag(nsmp_ctx* c, double out[NSMP_CFL_COUNT]) {
    const Mesh& m = c->mesh;
    const int nb = grid_for(c, m.nprism);
    // the records and the result live in the transfer staging buffer, which
    // is free between calls (every use of it is stream-ordered)
    const size_t need = (size_t)nb * kCflRec + NSMP_CFL_COUNT;
    const size_t have = std::max((size_t)c->L.NC * c->L.NZ, (size_t)c->L.NV * c->L.NZ);
    if (need > have) {
        c->err = "nsmp_cfl_diag: staging buffer too small for the reduction records";
        return NSMP_ERR_RANGE;
    }
    double* rec = c->stage_buf;
    double* dres = c->stage_buf + (size_t)nb * kCflRec;
    double** N = c->lvl[c->ln];
    const CflArgs a{N[0], N[1], N[2], c->face[0], c->face[1], c->face[2], c->face[3], c->face[4], c->prm.dt};
    LAUNCH(NSMP_K_OTHER, k_cfl_diag<<<nb, kBlock, 0, c->stream>>>(m, a, rec));
    CKL("k_cfl_diag");
    LAUNCH(NSMP_K_OTHER, k_cfl_final<<<1, kBlock, 0, c->stream>>>(nb, m.tv_lsig, rec, dres));
    CKL("k_cfl_final");
    CK(cudaMemcpyAsync(out, dres, NSMP_CFL_COUNT * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

int run_mass_diag(nsmp_ctx* c, double out[4]) {
    double d[NSMP_CFL_COUNT];
    const int rc = run_cfl_diag(c, d);
    if (rc) return rc;
    out[0] = d[NSMP_CFL_ABS_DIV];
    out[1] = fabs(d[NSMP_CFL_FLUX_MAX]);
    out[2] = d[NSMP_CFL_FLUX_TOTAL];
    out[3] = d[NSMP_CFL_MAX];
    return 0;
}

}  // namespace nsmp

extern "C" int nsmp_cfl_diag(nsmp_ctx* c, double* out) {
    if (!c || !out) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    return nsmp::run_cfl_diag(c, out);
}
