// Vertex fields for the output path (SavetecVertex, SavetecCenter's vertex
// variables): the vertex interpolation of a level-n field in the reference's
// vertex numbering, (N_VERT, NZ-1), computed on the device so the driver
// downloads vertex values instead of cell fields.
//
//   tagdir 2: phiv(nv,k) = IDW of phi at cell layer k (interpolation2D,
//             Interpolation/interpolation3D.F90:151-198)
//   tagdir 3: phiv(nv,k) = the IDW values of layers k and k+1 blended to the
//             vertex layer sigv(k) (interpolation3D.F90:200-220), with
//             BCvelvertex3D's wall values for velocity (BC.F90:603-807)
// The periodic averaging of bc_periodic (BC.F90:1243-1300) is the merged
// class stencil; being linear it commutes with the vertical blend.
#include <cmath>
#include <vector>

#include "kern_common.cuh"

namespace nsmp {
namespace {

__device__ __forceinline__ double class_idw(const Mesh& m, const double* __restrict__ f, int v, int k0) {
    double a = 0.0;
    const int s1 = __ldg(m.vptr + v + 1);
    for (int s = __ldg(m.vptr + v); s < s1; ++s) a += __ldg(m.vcoef + s) * f[IX(m, __ldg(m.vcell + s), k0)];
    return a;
}

// out[nv + kv * nvert], kv = 0..NZ-2 (reference vertex layer kv+1).  A block
// computes a tile of 32 vertices x 32 layers: lanes run over layers when the
// stencil cells are read (a column's layers are contiguous, the stencil is the
// same for the warp) and over vertices when the tile is written.
constexpr int kVTile = 32, kVRows = 8;

__global__ void __launch_bounds__(kVTile * kVRows) k_vertex_out(Mesh m, int nvert, const int* __restrict__ vcls,
                                                               const double* __restrict__ f, int tagdir,
                                                               const double* __restrict__ wT,
                                                               const double* __restrict__ wB, int zero_bot,
                                                               int zero_top, double* __restrict__ out) {
    __shared__ double tile[kVTile][kVTile + 1];
    const int nl = m.NZ - 1;
    const int v0 = blockIdx.x * kVTile, kv0 = blockIdx.y * kVTile, tx = threadIdx.x;
    for (int j = threadIdx.y; j < kVTile; j += kVRows) {
        const int nv = v0 + j, kv = kv0 + tx;
        if (nv < nvert && kv < nl) {
            const int v = vcls[nv];
            double val;
            if (tagdir == 2) {
                val = class_idw(m, f, v, kv);
            } else if ((kv == 0 && zero_bot) || (kv == m.NZ - 2 && zero_top)) {
                val = 0.0;
            } else {
                const double a = class_idw(m, f, v, kv), b = class_idw(m, f, v, kv + 1);
                val = (wB[kv] * b + wT[kv] * a) / (wT[kv] + wB[kv]);
            }
            tile[j][tx] = val;
        }
    }
    __syncthreads();
    for (int j = threadIdx.y; j < kVTile; j += kVRows) {
        const int nv = v0 + tx, kv = kv0 + j;
        if (nv < nvert && kv < nl) out[(size_t)nv + (size_t)kv * nvert] = tile[tx][j];
    }
}

}  // namespace
}  // namespace nsmp

extern "C" int nsmp_download_vertex(nsmp_ctx* c, int field, int tagdir, double* host) {
    if (!c || !host || field < NSMP_F_U || field > NSMP_F_P || (tagdir != 2 && tagdir != 3)) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);
    const nsmp::HostLayout& L = c->L;
    const int NZ = L.NZ, NV = L.NV;
    // blend weights of the vertex layers: dzT = |sigv(k) - sig(k+1)|, dzB = |sigv(k) - sig(k)|
    std::vector<double> w(2 * (size_t)(NZ - 1));
    for (int k = 1; k <= NZ - 1; ++k) {
        w[k - 1] = std::fabs(L.sigv[k - 1] - L.sig[k]);
        w[NZ - 1 + k - 1] = std::fabs(L.sigv[k - 1] - L.sig[k - 1]);
    }
    // wall vertex values of BCvelvertex3D with tagdir 3: velocity zero on a
    // no-slip wall, w zero on any wall; pressure untouched (BCpvertex)
    const bool vel = field != NSMP_F_P, is_w = field == NSMP_F_W;
    const int zb = vel && (c->prm.bot_bc == 0 || is_w), zt = vel && (c->prm.top_bc == 0 || is_w);
    const size_t n = (size_t)NV * (NZ - 1);
    double* dw = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&dw, w.size() * sizeof(double), c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dw, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        const dim3 tiles((NV + nsmp::kVTile - 1) / nsmp::kVTile, (NZ - 1 + nsmp::kVTile - 1) / nsmp::kVTile);
        nsmp::k_vertex_out<<<tiles, dim3(nsmp::kVTile, nsmp::kVRows), 0, c->stream>>>(
            c->mesh, NV, c->d_vgather, c->lvl[c->ln][field - NSMP_F_U], tagdir, dw, dw + (NZ - 1), zb, zt,
            c->stage_buf);
        e = cudaGetLastError();
        ++c->launches;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, c->stage_buf, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (dw) cudaFreeAsync(dw, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return nsmp::cuda_fail(c, e, "nsmp_download_vertex");
    return NSMP_OK;
}
