// FP64 fused multiply-add issue rate of the device (instrumentation): the
// roof of the FP64 solver passes, which issue more FP64 instructions per byte
// than this GPU's FP64 pipes retire at HBM speed.
#include "ctx.h"

namespace nsmp {
namespace {

constexpr int kChains = 8;

// Every thread runs kChains independent chains of `iters` dependent FMAs, so
// the FP64 pipes always have independent work; the result is stored so the
// chains are not removed.
__global__ void __launch_bounds__(256) k_fp64_fma(int iters, double a, double b, double* out) {
    double x[kChains];
#pragma unroll
    for (int q = 0; q < kChains; ++q) x[q] = (double)(threadIdx.x + q) * 1e-3;
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int q = 0; q < kChains; ++q) x[q] = fma(x[q], a, b);
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < kChains; ++q) s += x[q];
    if (s == 1.2345e300) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // never true: keeps the chains live
}

}  // namespace
}  // namespace nsmp

extern "C" int nsmp_probe_fp64_fma(int device, int iters, double* tflops, double* ms) {
    if (iters < 1 || !tflops) return NSMP_ERR_ARG;
    nsmp::DeviceGuard guard(device);
    if (guard.err != cudaSuccess) return NSMP_ERR_CUDA;
    int sms = 0, per_sm = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return NSMP_ERR_CUDA;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, nsmp::k_fp64_fma, 256, 0) != cudaSuccess) return NSMP_ERR_CUDA;
    const int blocks = sms * (per_sm > 0 ? per_sm : 1);
    double* out = nullptr;  // never written (see the kernel); a valid address for the compiler's sake
    cudaEvent_t e0, e1;
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return NSMP_ERR_CUDA;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaError_t e = cudaMalloc((void**)&out, sizeof(double) * (size_t)blocks * 256);
    float t = 0.f;
    if (e == cudaSuccess) {
        nsmp::k_fp64_fma<<<blocks, 256, 0, st>>>(iters / 10 + 1, 0.999999, 1e-7, out);  // warm-up
        cudaEventRecord(e0, st);
        nsmp::k_fp64_fma<<<blocks, 256, 0, st>>>(iters, 0.999999, 1e-7, out);
        cudaEventRecord(e1, st);
        e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    }
    if (out) cudaFree(out);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return NSMP_ERR_CUDA;
    }
    const double fmas = (double)blocks * 256.0 * nsmp::kChains * (double)iters;
    *tflops = 2.0 * fmas / (t * 1e-3) / 1e12;
    if (ms) *ms = t;
    return NSMP_OK;
}
