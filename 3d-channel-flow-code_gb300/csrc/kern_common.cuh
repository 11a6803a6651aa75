// Helpers shared by the kernel translation units: prism indexing, the
// FP64 PPE row, grid sizing and the launch/error macros.
#pragma once
#include <utility>

#include "ctx.h"

namespace nsmp {

__device__ __forceinline__ void prism_of(const Mesh& m, int g, int& c, int& k0) {
    c = g / m.NZI;
    k0 = 1 + (g - c * m.NZI);
}

// PPE row (PDE.F90:69-121) applied to a field: returns sum of the six
// coefficient products in the reference's order.
__device__ __forceinline__ double ppe_row(const Mesh& m, const ColPPE& P, int k0, double x0, double x1, double x2,
                                          double x3, double xT, double xB) {
    const double dsv = lev(m, LV_DSV, k0);
    const double AA1 = P.kA[0] * dsv, AA2 = P.kA[1] * dsv, AA3 = P.kA[2] * dsv;
    const double AAB = P.area * lev(m, LV_IDSB, k0) * lev(m, LV_WB, k0);
    const double AAT = P.area * lev(m, LV_IDST, k0) * lev(m, LV_WT, k0);
    const double AA0 = -1.0 * (AAT + AAB + AA1 + AA2 + AA3);
    return AA0 * x0 + AA1 * x1 + AA2 * x2 + AA3 * x3 + AAT * xT + AAB * xB;
}

// Compact interior layout of the solver vectors: index g = c*NZI + k0-1,
// i.e. the prism's own thread index.  Neighbour column nb, same layer:
// g + (nb - c)*NZI; vertical neighbours g +- 1 (inside the column).
__device__ __forceinline__ size_t ICg(const Mesh& m, int c, int k0) { return (size_t)c * m.NZI + (k0 - 1); }

// Cell-layout index of the prism with compact index g in column c.
__device__ __forceinline__ size_t cell_of(int g, int c) { return (size_t)g + 2 * (size_t)c + 1; }

// Blocks that fit on the device at once for a kernel (one full wave).
int occupancy_grid(nsmp_ctx* c, const void* kernel, long long n);
template <class K>
inline int grid_occ(nsmp_ctx* c, K kernel, long long n) { return occupancy_grid(c, (const void*)kernel, n); }

inline int grid_for(const nsmp_ctx* c, long long n) {
    long long b = (n + kBlock - 1) / kBlock;
    long long cap = (long long)c->num_sms * 8;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

// Launch with programmatic stream serialization: the kernel may start while
// the previous kernel of the stream drains, and must begin with pdl_enter().
template <typename... P, typename... A>
cudaError_t launch_pdl(void (*kernel)(P...), int grid, cudaStream_t st, A&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)kBlock);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

}  // namespace nsmp

#define CK(call)                                                  \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, #call);    \
    } while (0)
#define CKL(where)                                                \
    do {                                                          \
        cudaError_t e_ = cudaGetLastError();                      \
        if (e_ != cudaSuccess) return cuda_fail(c, e_, where);    \
    } while (0)

#define LAUNCH(KID, ...)                         \
    do {                                         \
        const int slot_ = prof_begin(c, (KID));  \
        __VA_ARGS__;                             \
        prof_end(c, slot_);                      \
        ++c->launches;                           \
    } while (0)

