// common.cuh -- shared device helpers of libdmftgpu (complex FP64 arithmetic, status codes, launch checks).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "dmftgpu.h"
#include "internal.h"

#define DG_PI 3.1415926535897932384626  // src/dmft_common.h:43

// ---------------------------------------------------------------------------------------------------
// complex double as double2 (x = re, y = im)
// ---------------------------------------------------------------------------------------------------
__host__ __device__ __forceinline__ double2 cmk(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ double2 cadd(double2 a, double2 b) { return cmk(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ double2 csub(double2 a, double2 b) { return cmk(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ double2 cneg(double2 a) { return cmk(-a.x, -a.y); }
__host__ __device__ __forceinline__ double2 cconj(double2 a) { return cmk(a.x, -a.y); }
__host__ __device__ __forceinline__ double2 cscale(double2 a, double s) { return cmk(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return cmk(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__host__ __device__ __forceinline__ double2 cmulc(double2 a, double2 b) {
    return cmk(fma(a.x, b.x, a.y * b.y), fma(a.y, b.x, -a.x * b.y));
}
// acc + a*b
__host__ __device__ __forceinline__ double2 cfma(double2 a, double2 b, double2 acc) {
    return cmk(fma(a.x, b.x, fma(-a.y, b.y, acc.x)), fma(a.x, b.y, fma(a.y, b.x, acc.y)));
}
// acc - a*b
__host__ __device__ __forceinline__ double2 cfms(double2 a, double2 b, double2 acc) {
    return cmk(fma(-a.x, b.x, fma(a.y, b.y, acc.x)), fma(-a.x, b.y, fma(-a.y, b.x, acc.y)));
}
__host__ __device__ __forceinline__ double cabs2(double2 a) { return fma(a.x, a.x, a.y * a.y); }
// 1/a = conj(a)/|a|^2 with a single division (FP64 division is a multi-instruction sequence on this GPU).
// |a| stays within 1e-150..1e150 for every caller (shifted Matsubara frequencies, pivots of well-scaled
// matrices); a zero pivot gives inf/nan, as the reference's division would.
__host__ __device__ __forceinline__ double2 crcp(double2 a) {
    const double r = 1.0 / fma(a.x, a.x, a.y * a.y);
    return cmk(a.x * r, -a.y * r);
}
__host__ __device__ __forceinline__ double2 cdiv(double2 a, double2 b) { return cmul(a, crcp(b)); }
__host__ __device__ __forceinline__ double2 cexpi(double ang) {  // exp(i ang)
    double s, c;
    sincos(ang, &s, &c);
    return cmk(c, s);
}

__device__ __forceinline__ double2 shfl2(double2 v, int src, int width) {
    return cmk(__shfl_sync(0xffffffffu, v.x, src, width), __shfl_sync(0xffffffffu, v.y, src, width));
}
__device__ __forceinline__ void atomic_add_c(double2 *p, double2 v) {
    atomicAdd(&p->x, v.x);
    atomicAdd(&p->y, v.y);
}

// status word written by kernels (never a trap): the host reads it after the launch sequence.
__device__ __forceinline__ void dg_flag(int *status, int code) {
    if (status) atomicMax(status, code);
}

#define DG_CUDA(call)                                                   \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) return dg_set_cuda_error(ctx, e_, #call); \
    } while (0)

static inline int dg_ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }
