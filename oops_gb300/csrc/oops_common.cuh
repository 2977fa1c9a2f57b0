// oops_common.cuh -- shared device helpers and status codes for liboops_gb300.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "oops_expv.h"

// complex128 as double2 (re, im); same layout as std::complex<double>
typedef double2 zd;

__host__ __device__ __forceinline__ zd zmake(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ zd zadd(zd a, zd b) { return zmake(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ zd zsub(zd a, zd b) { return zmake(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ zd zmul(zd a, zd b)
{
    return zmake(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) * b
__host__ __device__ __forceinline__ zd zcmul(zd a, zd b)
{
    return zmake(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ zd zscale(zd a, double s) { return zmake(a.x * s, a.y * s); }
// acc += a * b (four fused multiply-adds)
__device__ __forceinline__ void zfma(zd &acc, zd a, zd b)
{
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}
__host__ __device__ __forceinline__ double zabs(zd a) { return hypot(a.x, a.y); }

// record a failure and return it (host side)
int oops_set_status(int code, const char *msg);

#define OOPS_CUDA_TRY(expr)                                                   \
    do {                                                                      \
        cudaError_t _e = (expr);                                              \
        if (_e != cudaSuccess)                                                \
            return oops_set_status(OOPS_ERR_CUDA, cudaGetErrorString(_e));    \
    } while (0)

// number of SMs on the current device (cached per device)
int oops_sm_count();

// Cluster coherence from n0 = ||B0||_F^2, n1 = ||B1||_F^2, d = ||B0 - B1||_F^2:
//   L = Re Tr(B1^+ B0) / sqrt(n0 n1) = 1 - (d - (sqrt(n0) - sqrt(n1))^2) / (2 sqrt(n0 n1)),
// which is Re Tr(B1^+ B0) / D for unitary B0, B1 (n0 = n1 = D).  The
// normalisation removes any common scale error of the two computed chains
// (tensor-core FP32 accumulation truncates toward zero, so reduced-precision
// products shrink slowly), and the difference form keeps the remaining
// rounding error proportional to sqrt(1 - L).
// The same in FP32 for the mixed-precision kernels, returned as the defect
// x = 1 - L (relative error ~1e-7 of x, i.e. ~1e-7 (1 - L) in L once the
// caller forms 1 - x in FP64): per time point it replaces ~60 FP64
// instructions (square roots, a division, double shuffles), which kept the
// SM's FP64 pipe busier than the FP32 products.
__device__ __forceinline__ float coherence_defect_f(float n0, float n1, float d)
{
    const float s0 = sqrtf(n0), s1 = sqrtf(n1);
    const float ds = (n0 - n1) / (s0 + s1);  // sqrt(n0) - sqrt(n1)
    return (d - ds * ds) / (2.0f * s0 * s1);
}

__device__ __forceinline__ double coherence_from_sums(double n0, double n1, double d)
{
    const double s0 = sqrt(n0), s1 = sqrt(n1);
    const double ds = (n0 - n1) / (s0 + s1);  // sqrt(n0) - sqrt(n1)
    return 1.0 - (d - ds * ds) / (2.0 * s0 * s1);
}

// e^{-2 pi i x} in FP32 for x = frac(i * phi / 2^64) turns.  phi is the phase
// advance of one time step as a 64-bit fixed-point fraction of a turn
// (computed once per cluster in FP64), so time point i needs one integer
// multiply (exact modulo 2^64), the nearest quarter turn taken off exactly
// (a swap and sign changes of the result), and an FP32 sincospi of the
// remaining [-1/8, 1/8) turn: no FP64 instruction per time point (FP64
// issues at 1/64 of the FP32 rate).  The remainder keeps 30 of its bits in
// the conversion to FP32, so the phase error is at most ~5e-8 rad (2^-24 of
// an eighth of a turn) plus sincospi's own rounding.
__device__ __forceinline__ float2 phase_step_f(unsigned long long phi, long long i)
{
    const unsigned long long u = (unsigned long long)i * phi;
    const unsigned q = (unsigned)((u + (1ULL << 61)) >> 62) & 3u;    // nearest quarter turn
    const long long r = (long long)(u - ((unsigned long long)q << 62)); // [-2^61, 2^61)
    const int hi = (int)(r >> 32);                                     // turns * 2^32
    const float x = (float)hi * 0x1p-31f;                              // 2 * turns, |x| <= 1/4
    float s, c;
    sincospif(x, &s, &c);
    // e^{-i pi x} (-i)^q
    switch (q) {
        case 0: return make_float2(c, -s);
        case 1: return make_float2(-s, -c);
        case 2: return make_float2(-c, s);
        default: return make_float2(s, c);
    }
}
