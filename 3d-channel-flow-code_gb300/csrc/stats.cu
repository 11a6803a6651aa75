// Turbulence statistics on the device: the running sums of glob_sample
// (Stats/stats.F90:91-197) accumulated in place every sampling step, and the
// plane averages of glob_put_plane_mm (Stats/stats.F90:204-384), so the
// driver samples without downloading fields.
//
// Sums per cell over all layers k = 1..NZ of the interior cells:
//   u, v, w, p, u^2, v^2, w^2, uv, vw, wu, p^2 and nu_t (KeyLES),
// in the cell layout of the state fields.
#include <cmath>
#include <vector>

#include "kern_common.cuh"

constexpr int kStatFields = 12;  // NSMP_S_U .. NSMP_S_EDDY

constexpr int kPlaneChunks = 64;  // column chunks of the first stage of the plane sums

struct StatState {
    double* sm[kStatFields] = {};
    double* plane = nullptr;
    double* plane_part = nullptr;  // kPlaneChunks x NZ x 9 first-stage sums
    long long n = 0;
};

namespace nsmp {
namespace {

struct StatArgs {
    const double *u, *v, *w, *p, *eddy;
    double* sm[kStatFields];
};

// glob_sample: one thread per cell value (all layers, ghost layers included)
__global__ void k_stats_sample(size_t n, StatArgs a) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double tu = a.u[i], tv = a.v[i], tw = a.w[i], tp = a.p[i];
        a.sm[0][i] += tu;
        a.sm[1][i] += tv;
        a.sm[2][i] += tw;
        a.sm[3][i] += tp;
        a.sm[4][i] += tu * tu;
        a.sm[5][i] += tv * tv;
        a.sm[6][i] += tw * tw;
        a.sm[7][i] += tu * tv;
        a.sm[8][i] += tv * tw;
        a.sm[9][i] += tw * tu;
        a.sm[10][i] += tp * tp;
        if (a.eddy) a.sm[11][i] += a.eddy[i];
    }
}

// glob_put_plane_mm sums over the interior cells of every layer k0 =
// 1..NZ-2, the nine second-order sums divided by the sample count ns;
// out[k0 * 9 + f].  The reference divides every term by ns; here each block
// sum is divided once (the same value up to rounding, and 9 FP64 divisions a
// prism less, which on this GPU's FP64 rate dominated the pass).  Two stages with a fixed order, so the
// result is deterministic: (1) a block takes 32 consecutive layers (one per
// lane, so a warp reads a column's layers contiguously) and one of
// kPlaneChunks contiguous column chunks, its 8 thread rows striding over the
// chunk's columns; the rows are summed in order into part[chunk][k0][f];
// (2) the chunks are summed in order.
struct PlaneArgs {
    const double* sm[9];  // u, v, w, u^2, v^2, w^2, uv, vw, wu
};

__global__ void __launch_bounds__(256) k_stats_plane_part(Mesh m, PlaneArgs a, double ns, double* part) {
    __shared__ double sh[8][9][33];
    const int k0 = 1 + blockIdx.x * 32 + threadIdx.x, chunk = blockIdx.y;
    const int c_beg = (int)((long long)m.N0 * chunk / gridDim.y);
    const int c_end = (int)((long long)m.N0 * (chunk + 1) / gridDim.y);
    double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (k0 <= m.NZ - 2)
        for (int c = c_beg + threadIdx.y; c < c_end; c += blockDim.y) {
            const size_t q = IX(m, c, k0);
#pragma unroll
            for (int f = 0; f < 9; ++f) s[f] += a.sm[f][q];
        }
#pragma unroll
    for (int f = 0; f < 9; ++f) sh[threadIdx.y][f][threadIdx.x] = s[f] / ns;
    __syncthreads();
    if (threadIdx.y == 0 && k0 <= m.NZ - 2)
        for (int f = 0; f < 9; ++f) {
            double t = 0.0;
            for (int y = 0; y < 8; ++y) t += sh[y][f][threadIdx.x];
            part[((size_t)chunk * m.NZ + k0) * 9 + f] = t;
        }
}

__global__ void k_stats_plane_sum(int nz, int nchunks, const double* __restrict__ part, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;  // k0 * 9 + f
    const int k0 = i / 9;
    if (i >= nz * 9 || k0 < 1 || k0 > nz - 2) return;
    double t = 0.0;
    for (int ch = 0; ch < nchunks; ++ch) t += part[(size_t)ch * nz * 9 + i];
    out[i] = t;
}

int stats_alloc(nsmp_ctx* c) {
    if (c->stats) return 0;
    c->stats = new StatState();
    StatState& S = *c->stats;
    const size_t ncf = (size_t)c->L.N0 * c->L.NZ;
    for (int f = 0; f < kStatFields; ++f) {
        CK(cudaMalloc((void**)&S.sm[f], ncf * sizeof(double)));
        c->allocs.push_back(S.sm[f]);
        CK(cudaMemsetAsync(S.sm[f], 0, ncf * sizeof(double), c->stream));
    }
    CK(cudaMalloc((void**)&S.plane, (size_t)c->L.NZ * 9 * sizeof(double)));
    c->allocs.push_back(S.plane);
    CK(cudaMalloc((void**)&S.plane_part, (size_t)kPlaneChunks * c->L.NZ * 9 * sizeof(double)));
    c->allocs.push_back(S.plane_part);
    CK(cudaStreamSynchronize(c->stream));
    return 0;
}

}  // namespace

void stats_free(nsmp_ctx* c) {
    delete c->stats;  // device buffers are in c->allocs
    c->stats = nullptr;
}

}  // namespace nsmp

extern "C" {

int nsmp_stats_reset(nsmp_ctx* c) {
    if (!c) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    int rc = nsmp::stats_alloc(c);
    if (rc) return rc;
    const size_t ncf = (size_t)c->L.N0 * c->L.NZ;
    for (int f = 0; f < kStatFields; ++f)
        if (cudaMemsetAsync(c->stats->sm[f], 0, ncf * sizeof(double), c->stream) != cudaSuccess)
            return nsmp::cuda_fail(c, cudaGetLastError(), "nsmp_stats_reset");
    c->stats->n = 0;
    return NSMP_OK;
}

int nsmp_stats_sample(nsmp_ctx* c) {
    if (!c) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    int rc = nsmp::stats_alloc(c);
    if (rc) return rc;
    nsmp::StatArgs a;
    a.u = c->lvl[c->ln][0]; a.v = c->lvl[c->ln][1]; a.w = c->lvl[c->ln][2]; a.p = c->lvl[c->ln][3];
    a.eddy = c->prm.les ? c->eddy : nullptr;
    for (int f = 0; f < kStatFields; ++f) a.sm[f] = c->stats->sm[f];
    const size_t ncf = (size_t)c->L.N0 * c->L.NZ;
    nsmp::k_stats_sample<<<nsmp::grid_for(c, (long long)ncf), nsmp::kBlock, 0, c->stream>>>(ncf, a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return nsmp::cuda_fail(c, e, "k_stats_sample");
    ++c->launches;
    c->stats->n += 1;
    return NSMP_OK;
}

int nsmp_stats_count(nsmp_ctx* c, int* n) {
    if (!c || !n) return NSMP_ERR_ARG;
    *n = c->stats ? (int)c->stats->n : 0;
    return NSMP_OK;
}

int nsmp_stats_download(nsmp_ctx* c, int which, double* host) {
    if (!c || !host || which < 0 || which >= kStatFields) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    int rc = nsmp::stats_alloc(c);
    if (rc) return rc;
    return nsmp::run_gather(c, c->stats->sm[which], 1, c->L.NC, host);
}

int nsmp_stats_plane(nsmp_ctx* c, double* out, double* tke) {
    if (!c || !out) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    int rc = nsmp::stats_alloc(c);
    if (rc) return rc;
    StatState& S = *c->stats;
    if (S.n <= 0) {
        c->err = "nsmp_stats_plane: no samples";
        return NSMP_ERR_ARG;
    }
    const int NZ = c->L.NZ;
    nsmp::PlaneArgs a;
    const int idx[9] = {0, 1, 2, 4, 5, 6, 7, 8, 9};
    for (int f = 0; f < 9; ++f) a.sm[f] = S.sm[idx[f]];
    const dim3 g1((NZ - 2 + 31) / 32, kPlaneChunks), b1(32, 8);
    nsmp::k_stats_plane_part<<<g1, b1, 0, c->stream>>>(c->mesh, a, (double)S.n, S.plane_part);
    nsmp::k_stats_plane_sum<<<(NZ * 9 + 255) / 256, 256, 0, c->stream>>>(NZ, kPlaneChunks, S.plane_part, S.plane);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return nsmp::cuda_fail(c, e, "k_stats_plane");
    c->launches += 1;
    ++c->launches;
    std::vector<double> sums((size_t)NZ * 9);
    e = cudaMemcpyAsync(sums.data(), S.plane, sums.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return nsmp::cuda_fail(c, e, "nsmp_stats_plane");
    // glob_put_plane_mm (stats.F90:315-364): means, rms, shear stresses
    const double npjx = 1.0 / c->L.N0;
    double tkesum = 0.0;
    for (int k = 2; k <= NZ - 1; ++k) {
        const double* sk = &sums[(size_t)(k - 1) * 9];
        const double yplus = c->prm.re * (2 * k - 3) / (2 * NZ - 4);
        const double u1m = sk[0] * npjx, v1m = sk[1] * npjx, w1m = sk[2] * npjx;
        const double u2m = sk[3] * npjx, v2m = sk[4] * npjx, w2m = sk[5] * npjx;
        const double uvm = sk[6] * npjx, vwm = sk[7] * npjx, wum = sk[8] * npjx;
        const double Tuvm = u1m * v1m - uvm, Tvwm = v1m * w1m - vwm, Twum = w1m * u1m - wum;
        const double xrms = u2m - u1m * u1m, yrms = v2m - v1m * v1m, zrms = w2m - w1m * w1m;
        tkesum = tkesum + 0.5 * (xrms + yrms + zrms);
        double* o = out + (size_t)(k - 2) * 10;
        o[0] = yplus;
        o[1] = u1m; o[2] = v1m; o[3] = w1m;
        o[4] = std::sqrt(xrms); o[5] = std::sqrt(yrms); o[6] = std::sqrt(zrms);
        o[7] = Tuvm; o[8] = Tvwm; o[9] = Twum;
    }
    if (tke) *tke = tkesum / (NZ - 2);
    return NSMP_OK;
}

}  // extern "C"
