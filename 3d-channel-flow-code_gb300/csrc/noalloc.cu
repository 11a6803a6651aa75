// nsmp_mass_diag_noalloc: the four glob_cfl mass-flux figures of
// nsmp_mass_diag without any allocation.
//
// Some callers cannot allocate device memory once their setup is done: a
// driver that reserves a fixed device-memory budget before its time loop,
// a code that forbids allocation inside its loop (allocation can synchronise
// the device), or a caller sharing the GPU under an external memory manager.
// This variant keeps its reduction scratch (per-block partial values, the
// arrival counter and the result) in a file-scope static device array of a
// fixed size instead of in context-allocated buffers, and calls no cudaMalloc,
// cudaFree or allocating library routine.  Its per-prism arithmetic is the
// shared glob_cfl restatement of diag.cuh, so its figures are those of
// nsmp_mass_diag: the maxima bit for bit, the sums up to summation order.
//
// Limits and behaviour:
//  * one thread per interior prism, 256 per block; the static array holds the
//    partials of at most kNoAllocMaxBlocks = 65536 blocks, so contexts with
//    more than 65536 * 256 = 16,777,216 prisms are rejected with
//    NSMP_ERR_RANGE;
//  * the array (2 MB plus a small header) is held by every GPU that loads the
//    library until the process exits;
//  * every call shares the array and the array keeps the last call's
//    contents; the arrival counter is cleared before each launch.  Calls that
//    overlap on the GPU (several host threads, or several contexts on the
//    same device using different streams) race on the array;
//  * the call copies its four results to the caller's array and waits for
//    the context's stream before it returns;
//  * the first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (the array's name in host code is only a host-side
//    stand-in, not a device address); make that first call before any
//    stream capture.  The resolved address is cached per device for the life
//    of the process; a cudaDeviceReset by the caller would invalidate it.
#include <mutex>

#include "diag.cuh"

namespace nsmp {
namespace {

constexpr int kNoAllocMaxBlocks = 65536;
constexpr int kNoAllocHeader = 32;  // doubles: [0] counter (as unsigned), [8..11] results
constexpr size_t kNoAllocDoubles = (size_t)kNoAllocHeader + 4 * (size_t)kNoAllocMaxBlocks;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_addr_mu;
double* g_addr[kMaxDevices] = {};

// Per-block partials: sum |div|, sum div, max |div|, max CFL.
__global__ void __launch_bounds__(kBlock) k_mass_diag_noalloc(Mesh m, const double* f1, const double* f2,
                                                              const double* f3, const double* fT,
                                                              const double* fB, double dt, double* scr) {
    unsigned int* counter = reinterpret_cast<unsigned int*>(scr);
    double* res = scr + 8;
    double* partials = scr + kNoAllocHeader;
    __shared__ bool last;
    double s[2] = {0.0, 0.0}, mx[2] = {0.0, 0.0};
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < m.nprism) {
        int c, k0;
        prism_of(m, g, c, k0);
        const CflCell o = cfl_cell(m, f1, f2, f3, fT, fB, dt, c, k0);
        s[0] = fabs(o.flux);
        s[1] = o.flux;
        mx[0] = fabs(o.flux);
        mx[1] = o.cfl;
    }
    block_reduce<2, false>(s);
    block_reduce<2, true>(mx);
    if (threadIdx.x == 0) {
        double* pb = partials + 4 * (size_t)blockIdx.x;
        pb[0] = s[0]; pb[1] = s[1]; pb[2] = mx[0]; pb[3] = mx[1];
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double y[2] = {0.0, 0.0}, z[2] = {0.0, 0.0};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
        const double* pb = partials + 4 * (size_t)b;
        y[0] += __ldcg(pb); y[1] += __ldcg(pb + 1);
        z[0] = fmax(z[0], __ldcg(pb + 2)); z[1] = fmax(z[1], __ldcg(pb + 3));
    }
    block_reduce<2, false>(y);
    block_reduce<2, true>(z);
    if (threadIdx.x == 0) {
        res[0] = y[0]; res[1] = z[0]; res[2] = y[1]; res[3] = z[1];
        *counter = 0u;
    }
}

// Device address of the static scratch on `dev`, resolved once per device
// with that device current.
int scratch_addr(nsmp_ctx* c, int dev, double** out) {
    if (dev < 0 || dev >= kMaxDevices) {
        c->err = "nsmp_mass_diag_noalloc: device ordinal out of range";
        return NSMP_ERR_RANGE;
    }
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return cuda_fail(c, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_addr[dev] = static_cast<double*>(p);
    }
    *out = g_addr[dev];
    return 0;
}

}  // namespace

int run_mass_diag_noalloc(nsmp_ctx* c, double out[4]) {
    const Mesh& m = c->mesh;
    const long long blocks = ((long long)m.nprism + kBlock - 1) / kBlock;
    if (blocks > kNoAllocMaxBlocks) {
        c->err = "nsmp_mass_diag_noalloc: " + std::to_string(m.nprism) + " prisms exceed the static scratch limit of " +
                 std::to_string((long long)kNoAllocMaxBlocks * kBlock) + " prisms";
        return NSMP_ERR_RANGE;
    }
    double* scr = nullptr;
    int rc = scratch_addr(c, c->device, &scr);
    if (rc == 0) {
        cudaError_t e = cudaMemsetAsync(scr, 0, sizeof(unsigned int), c->stream);  // arrival counter
        if (e == cudaSuccess) {
            k_mass_diag_noalloc<<<(unsigned)blocks, kBlock, 0, c->stream>>>(m, c->face[0], c->face[1], c->face[2],
                                                                            c->face[3], c->face[4], c->prm.dt, scr);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(out, scr + 8, 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) rc = cuda_fail(c, e, "nsmp_mass_diag_noalloc");
    }
    return rc;
}

}  // namespace nsmp

extern "C" int nsmp_mass_diag_noalloc(nsmp_ctx* c, double out[4]) {
    if (!c || !out) return NSMP_ERR_ARG;
    NSMP_DEVICE_GUARD(c);  // the scratch address is resolved with the context's device current
    return nsmp::run_mass_diag_noalloc(c, out);
}
