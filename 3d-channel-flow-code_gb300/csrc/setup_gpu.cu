// The floating-point steps of the setup on the GPU: cell centres, areas,
// edges and normals (calcul_geometry.F90:292-367), the inverse-distance
// vertex weights (:1055-1076), the edge midpoint offsets doe (:1343-1387) and
// the LSQ sums and Kim-Choi factors (:1460-1517).  The integer topology --
// ghost cells and periodic images, vertex pairs, classes, the renumbering --
// and the packing of the device tables stay on the host (setup.cpp).
//
// This file is compiled without multiply-add contraction, and every
// expression below is the host step's expression in the same order; division
// and square root are IEEE-rounded on the device as on the host.  The results
// are therefore the host setup's bits (tests/test_gpu_setup.py compares every
// array).
#include <cuda_runtime.h>

#include <vector>

#include "setup_geo.h"

namespace nsmp {
namespace setup {
namespace {

constexpr int kSetupBlock = 256;

// calcul_geometry.F90:292-367, one thread per cell.
__global__ void k_cell_geometry(int N0, const int* __restrict__ vp, const double* __restrict__ xv,
                                const double* __restrict__ yv, double* xc, double* yc, double* area, double* dxVV,
                                double* dyVV, double* dlVV, double* xnn, double* ynn) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N0; i += gridDim.x * blockDim.x) {
        const int v1 = vp[i], v2 = vp[i + N0], v3 = vp[i + 2 * N0];
        xc[i] = (xv[v1] + xv[v2] + xv[v3]) / 3.0;
        yc[i] = (yv[v1] + yv[v2] + yv[v3]) / 3.0;
        area[i] = 0.5 * fabs(xv[v1] * (yv[v2] - yv[v3]) + xv[v2] * (yv[v3] - yv[v1]) + xv[v3] * (yv[v1] - yv[v2]));
        const int vv[4] = {v1, v2, v3, v1};
        for (int j = 0; j < 3; ++j) {
            const int q = i + j * N0;
            const double dx = xv[vv[j + 1]] - xv[vv[j]], dy = yv[vv[j + 1]] - yv[vv[j]];
            const double dl = sqrt(dx * dx + dy * dy);
            dxVV[q] = dx;
            dyVV[q] = dy;
            dlVV[q] = dl;
            xnn[q] = dy / dl;
            ynn[q] = -dx / dl;
        }
    }
}

// calcul_geometry.F90:1055-1076: the weight of every (cell, corner), then per
// vertex their sum in the reference's visiting order (the incidence list).
__global__ void k_vertex_weights(int N0, const int* __restrict__ vp, const double* __restrict__ xv,
                                 const double* __restrict__ yv, const double* __restrict__ xc,
                                 const double* __restrict__ yc, double* w) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < 3 * N0; q += gridDim.x * blockDim.x) {
        const int i = q / 3, j = q - 3 * i;
        const int nv = vp[i + j * N0];
        const double dx = xc[i] - xv[nv], dy = yc[i] - yv[nv];
        w[q] = 1.0 / sqrt(dx * dx + dy * dy);
    }
}

__global__ void k_vertex_sums(int NV, const int* __restrict__ ptr, const int* __restrict__ inc,
                              const double* __restrict__ w, double* dlVsum) {
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < NV; v += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int e = ptr[v]; e < ptr[v + 1]; ++e) s = s + w[inc[e]];
        dlVsum[v] = s;
    }
}

// calcul_geometry.F90:1343-1387 and 1460-1517, one thread per cell; cp holds
// the neighbour (or ghost) of each edge with leading dimension ldc.
__global__ void k_edge_geometry(int N0, size_t ldc, const int* __restrict__ vp, const int* __restrict__ cp,
                                const double* __restrict__ xv, const double* __restrict__ yv,
                                const double* __restrict__ xc, const double* __restrict__ yc,
                                const double* __restrict__ dxVV, const double* __restrict__ dyVV,
                                const double* __restrict__ xnn, const double* __restrict__ ynn, double* doe,
                                double* dxCC, double* dyCC, double* dlCC, double* dle1, double* dle2, double* sxx,
                                double* syy, double* sxy) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N0; i += gridDim.x * blockDim.x) {
        for (int j = 0; j < 3; ++j) {
            const int q = i + j * N0;
            const int jv1 = vp[q], jv2 = vp[i + ((j + 1) % 3) * N0], jc = cp[i + j * ldc];
            const double xme = 0.5 * (xv[jv2] + xv[jv1]), yme = 0.5 * (yv[jv2] + yv[jv1]);
            const double x1 = xc[i], x2 = xc[jc], x3 = xv[jv1], x4 = xv[jv2];
            const double y1 = yc[i], y2 = yc[jc], y3 = yv[jv1], y4 = yv[jv2];
            const double den = (x1 - x2) * (y3 - y4) - (y1 - y2) * (x3 - x4);
            const double xmo = ((x1 * y2 - y1 * x2) * (x3 - x4) - (x1 - x2) * (x3 * y4 - y3 * x4)) / den;
            const double ymo = ((x1 * y2 - y1 * x2) * (y3 - y4) - (y1 - y2) * (x3 * y4 - y3 * x4)) / den;
            const double ex = xme - xmo, ey = yme - ymo;
            double d = sqrt(ex * ex + ey * ey);
            if (ex * dxVV[q] + ey * dyVV[q] < 0.0) d = -d;
            doe[q] = d;
        }
        double sX = 0.0, sY = 0.0, sXY = 0.0;
        for (int j = 0; j < 3; ++j) {
            const int q = i + j * N0, jc = cp[i + j * ldc];
            const double dx = xc[jc] - xc[i], dy = yc[jc] - yc[i];
            const double dl = sqrt(dx * dx + dy * dy);
            dxCC[q] = dx; dyCC[q] = dy; dlCC[q] = dl;
            sX = sX + dx * dx;
            sY = sY + dy * dy;
            sXY = sXY + dx * dy;
            double ux = dx / dl, uy = dy / dl;
            const double cth = ux * xnn[q] + uy * ynn[q];
            ux = ux / cth;
            uy = uy / cth;
            dle1[q] = 1.0 / cth;
            const double tx2 = xnn[q] - ux, ty2 = ynn[q] - uy;
            const double s = tx2 * dxVV[q] + ty2 * dyVV[q];
            dle2[q] = (s < 0.0) ? -1.0 * sqrt(tx2 * tx2 + ty2 * ty2) : sqrt(tx2 * tx2 + ty2 * ty2);
        }
        sxx[i] = sX; syy[i] = sY; sxy[i] = sXY;
    }
}

// Device buffers of one setup, freed on every return path.
struct SetupBuffers {
    std::vector<void*> p;
    cudaError_t err = cudaSuccess;
    template <class T>
    T* get(size_t n) {
        void* q = nullptr;
        if (err == cudaSuccess) err = cudaMalloc(&q, n > 0 ? n * sizeof(T) : 16);
        if (err == cudaSuccess) p.push_back(q);
        return static_cast<T*>(q);
    }
    ~SetupBuffers() {
        for (void* q : p) cudaFree(q);
    }
};

template <class T>
cudaError_t up(T* d, const std::vector<T>& h, cudaStream_t st) {
    return cudaMemcpyAsync(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, st);
}
template <class T>
cudaError_t down(std::vector<T>& h, const T* d, size_t n, cudaStream_t st) {
    h.resize(n);
    return cudaMemcpyAsync(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost, st);
}

int grid_of(long long n) {
    long long b = (n + kSetupBlock - 1) / kSetupBlock;
    return (int)(b < 1 ? 1 : (b > 65535 ? 65535 : b));
}

}  // namespace

int device_steps(const nsmp_params& p, Geo& g, std::string& err) {
    const int N0 = g.N0, NV = g.NV;
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        err = "device setup: cannot create a stream";
        return NSMP_ERR_CUDA;
    }
    int rc = 0;
    {
        SetupBuffers B;
        const size_t e3 = 3 * (size_t)N0;
        int* d_vp = B.get<int>(e3);
        double* d_xv = B.get<double>(NV);
        double* d_yv = B.get<double>(NV);
        // ghost-free sizes first; the centre arrays get the ghosts after the host step
        int nghost = 0;
        for (size_t q = 0; q < e3; ++q) nghost += g.cp[q] < 0;
        const size_t ncmax = (size_t)N0 + nghost;
        double* d_xc = B.get<double>(ncmax);
        double* d_yc = B.get<double>(ncmax);
        double* d_area = B.get<double>(N0);
        double* d_e[5];  // dxVV, dyVV, dlVV, xnn, ynn
        for (auto& a : d_e) a = B.get<double>(e3);
        cudaError_t e = B.err;
        if (e == cudaSuccess) e = up(d_vp, g.vp, st);
        if (e == cudaSuccess) e = up(d_xv, g.xv, st);
        if (e == cudaSuccess) e = up(d_yv, g.yv, st);
        if (e == cudaSuccess) {
            k_cell_geometry<<<grid_of(N0), kSetupBlock, 0, st>>>(N0, d_vp, d_xv, d_yv, d_xc, d_yc, d_area, d_e[0],
                                                                 d_e[1], d_e[2], d_e[3], d_e[4]);
            e = cudaGetLastError();
        }
        // the host needs the centres, areas and edges for the ghost cells
        std::vector<double> xc, yc, area;
        std::vector<double>* ev[5] = {&g.dxVV, &g.dyVV, &g.dlVV, &g.xnn, &g.ynn};
        if (e == cudaSuccess) e = down(xc, d_xc, N0, st);
        if (e == cudaSuccess) e = down(yc, d_yc, N0, st);
        if (e == cudaSuccess) e = down(area, d_area, N0, st);
        for (int k = 0; k < 5 && e == cudaSuccess; ++k) e = down(*ev[k], d_e[k], e3, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            cudaGetLastError();
            err = std::string("device setup (cell geometry): ") + cudaGetErrorString(e);
            rc = NSMP_ERR_CUDA;
        }
        if (rc == 0) {
            g.xc.assign(ncmax, 0.0); g.yc.assign(ncmax, 0.0); g.area.assign(ncmax, 0.0);
            std::copy(xc.begin(), xc.end(), g.xc.begin());
            std::copy(yc.begin(), yc.end(), g.yc.begin());
            std::copy(area.begin(), area.end(), g.area.begin());
            double vol = 0.0;  // TotalVolume in the reference's order
            for (int i = 0; i < N0; ++i) vol = vol + g.area[i];
            g.total_volume = vol;
            rc = ghosts_and_pairs(p, g, err);
        }
        if (rc == 0) {
            // ghost centres and the ghosted neighbour table
            const size_t ldc = g.cp.size() / 3;
            int* d_cp = B.get<int>(g.cp.size());
            double* d_w = B.get<double>(e3);
            double* d_sum = B.get<double>(NV);
            std::vector<int> ptr, inc;
            vertex_incidence(g, ptr, inc);
            int* d_ptr = B.get<int>(ptr.size());
            int* d_inc = B.get<int>(inc.size());
            double* d_f[9];  // doe, dxCC, dyCC, dlCC, dle1, dle2 (3 N0); sxx, syy, sxy (N0)
            for (int k = 0; k < 9; ++k) d_f[k] = B.get<double>(k < 6 ? e3 : (size_t)N0);
            e = B.err;
            if (e == cudaSuccess) e = up(d_cp, g.cp, st);
            if (e == cudaSuccess) e = up(d_xc, g.xc, st);
            if (e == cudaSuccess) e = up(d_yc, g.yc, st);
            if (e == cudaSuccess) e = up(d_ptr, ptr, st);
            if (e == cudaSuccess) e = up(d_inc, inc, st);
            if (e == cudaSuccess) {
                k_vertex_weights<<<grid_of((long long)e3), kSetupBlock, 0, st>>>(N0, d_vp, d_xv, d_yv, d_xc, d_yc, d_w);
                k_vertex_sums<<<grid_of(NV), kSetupBlock, 0, st>>>(NV, d_ptr, d_inc, d_w, d_sum);
                k_edge_geometry<<<grid_of(N0), kSetupBlock, 0, st>>>(
                    N0, ldc, d_vp, d_cp, d_xv, d_yv, d_xc, d_yc, d_e[0], d_e[1], d_e[3], d_e[4], d_f[0], d_f[1], d_f[2],
                    d_f[3], d_f[4], d_f[5], d_f[6], d_f[7], d_f[8]);
                e = cudaGetLastError();
            }
            std::vector<double> w;
            std::vector<double>* fv[9] = {&g.doe, &g.dxCC, &g.dyCC, &g.dlCC, &g.dle1, &g.dle2, &g.sxx, &g.syy, &g.sxy};
            if (e == cudaSuccess) e = down(w, d_w, e3, st);
            if (e == cudaSuccess) e = down(g.dlVsum, d_sum, NV, st);
            for (int k = 0; k < 9 && e == cudaSuccess; ++k) e = down(*fv[k], d_f[k], k < 6 ? e3 : (size_t)N0, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) {
                cudaGetLastError();
                err = std::string("device setup (weights, edges): ") + cudaGetErrorString(e);
                rc = NSMP_ERR_CUDA;
            } else {
                // the stencils in the reference's order: per vertex, its (cell, weight)
                g.stencil.assign(NV, {});
                for (int v = 0; v < NV; ++v)
                    for (int k = ptr[v]; k < ptr[v + 1]; ++k) g.stencil[v].push_back({inc[k] / 3, w[inc[k]]});
            }
        }
    }
    cudaStreamDestroy(st);
    return rc;
}

}  // namespace setup
}  // namespace nsmp
