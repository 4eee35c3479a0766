// mdt_fastmath.cuh -- FP32 building blocks of the fast force kernels (mdt_nnf.cu,
// mdt_nnr.cu): the cosine cutoff as a polynomial in s = r^2/rc^2, hardware 2^x / log2 /
// reciprocal approximations, the softplus activation with its derivative from one
// exponential, and shared-memory float reductions.
#pragma once
#include <cstdint>

#include "mdt_common.cuh"

namespace mdt {

// Cosine cutoff fc = (cos(pi r/rc) + 1)/2 = c^2 with c = cos(pi sqrt(s)/2), s = r^2/rc^2.
// c is the Taylor series sum_n (-pi^2 s/4)^n / (2n)! truncated after n = 7 (remainder
// below 1e-10 on [0, 1], alternating terms no larger than 1.24, so FP32 Horner loses
// little), and fc = c^2 keeps the absolute error vanishing at the cutoff.
constexpr double half_cos_sqrt_coef(int n) {
    double c = 1.0;
    for (int k = 1; k <= n; ++k) c *= -(kPi * kPi / 4.0) / ((2.0 * k - 1.0) * (2.0 * k));
    return c;
}
constexpr float kCs0 = (float)half_cos_sqrt_coef(0), kCs1 = (float)half_cos_sqrt_coef(1),
                kCs2 = (float)half_cos_sqrt_coef(2), kCs3 = (float)half_cos_sqrt_coef(3),
                kCs4 = (float)half_cos_sqrt_coef(4), kCs5 = (float)half_cos_sqrt_coef(5),
                kCs6 = (float)half_cos_sqrt_coef(6), kCs7 = (float)half_cos_sqrt_coef(7);

// fc(s)
__device__ __forceinline__ float fc_of_s(float s) {
    float c = kCs7;
    c = fmaf(c, s, kCs6);
    c = fmaf(c, s, kCs5);
    c = fmaf(c, s, kCs4);
    c = fmaf(c, s, kCs3);
    c = fmaf(c, s, kCs2);
    c = fmaf(c, s, kCs1);
    c = fmaf(c, s, kCs0);
    return c * c;
}

// fc(s) and dfc/ds = 2 c c'(s) (Horner with derivative)
__device__ __forceinline__ void fc_of_s_d(float s, float &fc, float &dfds) {
    float c = kCs7, d = 0.f;
#define MDT_STEP(k)        \
    d = fmaf(d, s, c);     \
    c = fmaf(c, s, k);
    MDT_STEP(kCs6) MDT_STEP(kCs5) MDT_STEP(kCs4) MDT_STEP(kCs3) MDT_STEP(kCs2) MDT_STEP(kCs1) MDT_STEP(kCs0)
#undef MDT_STEP
    fc = c * c;
    dfds = 2.f * c * d;
}

// 2^x (hardware approximation, relative error about 2^-22; results below the FP32
// normal range flush to zero, far below any radial function that matters)
__device__ __forceinline__ float ex2a(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// log2(x) for x in [1, 2] (hardware approximation, absolute error about 2^-22)
__device__ __forceinline__ float lg2a(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// 1/x (hardware approximation, about 1 ulp)
__device__ __forceinline__ float rcpa(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

constexpr float kLog2eF = 1.4426950408889634f;
constexpr float kLn2F = 0.6931471805599453f;

// softplus v = log(1 + e^z) and its derivative dv/dz = 1/(1 + e^-z) in the form that
// cannot overflow: v = max(z, 0) + log(1 + e^-|z|), one exponential for both.
__device__ __forceinline__ void softplus_d(float z, float &v, float &dv) {
    const float e = ex2a(-fabsf(z) * kLog2eF);
    const float d = 1.f + e;
    v = fmaf(lg2a(d), kLn2F, fmaxf(z, 0.f));
    const float r = rcpa(d);
    dv = z >= 0.f ? r : e * r;
}

__device__ __forceinline__ void red_shared(float *p, float v) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(p);
    asm volatile("red.shared.add.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}

}  // namespace mdt
