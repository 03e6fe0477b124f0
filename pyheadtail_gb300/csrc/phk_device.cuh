// Device-side building blocks of the turn kernels: exact slice binning,
// IEEE-ordered FP64 element arithmetic (plain form) and FP32 arithmetic with
// float-float phase arguments (precision form).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "phk_internal.h"

namespace phk {

// ---------------------------------------------------------------- helpers
// The plain form reproduces the reference's NumPy evaluation order, so each
// product and sum is rounded on its own (no FMA contraction).
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

// ---------------------------------------------------------------- binning
// Exact reference slice index from the host-built lower-edge table
// e[0..S]: inside iff e[0] <= z < e[S], index k with e[k] <= z < e[k+1].
// The first estimate only seeds the search; both loops stop at the table
// ends whatever the table contents, so no access leaves e[0..S].
template <typename T>
__device__ __forceinline__ int slice_of(T z, int S, int negate, T est_tail,
                                        T est_inv_w, const T* __restrict__ e) {
    const T zz = negate ? -z : z;
    if (!(zz >= e[0]) || !(zz < e[S])) return -1;
    int k = (int)((zz - est_tail) * est_inv_w);
    k = k < 0 ? 0 : (k > S - 1 ? S - 1 : k);
    while (zz < e[k]) --k;
    while (zz >= e[k + 1]) ++k;
    return k;
}

// Reference index int32(floor((z - tail)/width)) for particles outside the
// cuts (rare): IEEE division, NaN and out-of-range map to INT32_MIN as the
// x86 conversion of numpy's astype(int32) does.
__device__ __forceinline__ int32_t outside_index(double z, double tail,
                                                 double width) {
    const double q = floor(dvd(sub(z, tail), width));
    if (!(q >= -2147483648.0) || !(q < 2147483648.0)) return INT32_MIN;
    return (int32_t)q;
}

// ------------------------------------------------------- float-float phase
// sin and cos of 2*pi*(hi + lo + d) for a phase given in turns as the
// unevaluated sum of a float-float base (hi, lo) and a small float d.
// The integer number of turns is removed exactly (Knuth two-sum, then
// t - rint(t) is exact), the remaining fraction f + g is split into a float
// f and its residual g; sincospif(2f) is corrected to first order in g.
// The phase argument thus carries ~2^-46 turns of precision on the FP32
// pipes (GB300's FP64 pipe runs at a small fraction of the FP32 rate).
__device__ __forceinline__ void sincos_turns(float hi, float lo, float d,
                                             float* s, float* c) {
    const float t = hi + d;
    const float bp = t - hi;
    float err = (hi - (t - bp)) + (d - bp);
    err += lo;
    const float r = t - rintf(t);
    const float f = r + err;
    const float g = (r - f) + err;
    float sp, cp;
    sincospif(2.0f * f, &sp, &cp);
    const float dl = 6.28318530717958647692f * g;
    *s = fmaf(dl, cp, sp);
    *c = fmaf(-dl, sp, cp);
}

// sin of 2*pi*(z * (mh + ml) + (oh + ol)) with z exact in float: the
// product's rounding error is recovered with an FMA (two-product).
__device__ __forceinline__ float sin_turns_of_product(float z, float mh,
                                                      float ml, float oh,
                                                      float ol) {
    const float p = z * mh;
    float e = fmaf(z, mh, -p);
    e = fmaf(z, ml, e);
    float s, c;
    sincos_turns(p, e + ol, oh, &s, &c);
    return s;
}

}  // namespace phk
