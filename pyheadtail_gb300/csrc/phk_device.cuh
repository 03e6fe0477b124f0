// Device-side building blocks of the turn kernels: exact slice binning,
// IEEE-ordered FP64 element arithmetic (plain form) and FP32 arithmetic with
// float-float phase arguments (precision form).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "phk_internal.h"

namespace phk {

// ------------------------------------------------- TMA bulk copies, mbarrier
// Thin inline-PTX wrappers: one-dimensional bulk copies global -> shared
// (cp.async.bulk, completion counted on an mbarrier in transaction bytes)
// and the mbarrier operations around them.  Addresses and sizes of every
// bulk copy are multiples of 16 bytes (checked by the callers).
__device__ __forceinline__ unsigned smem_addr(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar,
                                          unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(count)
                 : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar,
                                               unsigned bytes) {
    asm volatile(
        "mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
            smem_addr(bar)),
        "r"(bytes)
        : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src,
                                         unsigned bytes,
                                         unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
// one poll of the barrier phase with the given parity
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar,
                                              unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait: false if the phase did not complete within `limit` polls
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar,
                                          unsigned parity, unsigned limit) {
    for (unsigned i = 0; i < limit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}


// ---------------------------------------------------------------- helpers
// The plain form reproduces the reference's NumPy evaluation order, so each
// product and sum is rounded on its own (no FMA contraction).
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dvd(double a, double b) { return __ddiv_rn(a, b); }

// Correctly rounded a / b for a divisor b known on the host, with
// y = RN(1/b) also from the host: q = RN(a y) is within one ulp of a/b, the
// remainder r = a - b q is exact through an FMA, and RN(q + r y) is the
// correctly rounded quotient (Markstein's theorem, IBM J. Res. Dev. 34,
// 1990; the basis of IA-64 division).  The theorem needs operands and
// quotient away from underflow and overflow; outside a safe exponent window
// the IEEE division is used.  Three FP64 instructions instead of a full
// division on GB300's slow FP64 pipe.
__device__ __forceinline__ double div_by(double a, double b, double y) {
    const double q = mul(a, y);
    const int ea = (__double2hiint(a) >> 20) & 0x7ff;
    const int eq = (__double2hiint(q) >> 20) & 0x7ff;
    if (ea > 64 && ea < 1984 && eq > 64 && eq < 1984) {
        const double r = fma(-b, q, a);
        return fma(r, y, q);
    }
    return dvd(a, b);
}

// sin and cos of phi = phi0 + d for a base phi0 whose sine s0 and cosine c0
// are known (host, correctly rounded): angle addition with the Maclaurin
// series of sin d (to d^11) and cos d (to d^12), whose truncation errors
// are below 3e-18 and 5e-20 for |d| <= 1/4.  d = phi - phi0 is exact when
// phi and phi0 are within a factor two (Sterbenz).  Larger |d| falls back
// to the library sincos.
__device__ __forceinline__ void sincos_about(double phi, double phi0,
                                             double s0, double c0, double* s,
                                             double* c) {
    const double d = phi - phi0;
    if (!(fabs(d) <= 0.25)) {
        sincos(phi, s, c);
        return;
    }
    const double d2 = d * d;
    // sin d = d + d^3 (-1/3! + d^2 (1/5! + d^2 (-1/7! + d^2 (1/9! - d^2/11!))))
    double ps = fma(d2, -1.0 / 39916800.0, 1.0 / 362880.0);
    ps = fma(d2, ps, -1.0 / 5040.0);
    ps = fma(d2, ps, 1.0 / 120.0);
    ps = fma(d2, ps, -1.0 / 6.0);
    const double sd = fma(d * d2, ps, d);
    // cos d = 1 + d^2 (-1/2! + d^2 (1/4! + ... + d^2 / 12!))
    double pc = fma(d2, 1.0 / 479001600.0, -1.0 / 3628800.0);
    pc = fma(d2, pc, 1.0 / 40320.0);
    pc = fma(d2, pc, -1.0 / 720.0);
    pc = fma(d2, pc, 1.0 / 24.0);
    pc = fma(d2, pc, -0.5);
    const double cd = fma(d2, pc, 1.0);
    *s = fma(s0, cd, c0 * sd);
    *c = fma(c0, cd, -(s0 * sd));
}

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

// Order-preserving 64-bit integer key of a double (sign-magnitude to two's
// complement): a < b  <=>  key(a) < key(b) for non-NaN doubles.  NaN keys
// fall beyond the keys of +-inf, i.e. outside any finite slicing range.
__device__ __forceinline__ long long order_key(double v) {
    const long long b = __double_as_longlong(v);
    return b >= 0 ? b : (long long)((unsigned long long)b ^ 0x7fffffffffffffffull);
}

__device__ __forceinline__ double key_to_double(long long k) {
    return __longlong_as_double(
        k >= 0 ? k : (long long)((unsigned long long)k ^ 0x7fffffffffffffffull));
}

// A float close to the double v (20 mantissa bits) built from v's high
// word with integer operations only; magnitudes outside the normal float
// range map to 0 or +-inf.  Only seeds the exact search below.
__device__ __forceinline__ float approx_float(double v) {
    const unsigned hi = (unsigned)__double2hiint(v);
    const unsigned sign = hi & 0x80000000u;
    const int e = (int)((hi >> 20) & 0x7ff) - 1023 + 127;
    unsigned bits;
    if (e <= 0) bits = sign;
    else if (e >= 255) bits = sign | 0x7f800000u;
    else bits = sign | ((unsigned)e << 23) | ((hi & 0xfffffu) << 3);
    return __uint_as_float(bits);
}

// FP64 slice index without FP64 arithmetic: ek[] holds order_key() of the
// exact edge table; the estimate uses FP32 (tail_f, inv_w_f).
__device__ __forceinline__ int slice_of_keys(double z, int S, int negate,
                                             float tail_f, float inv_w_f,
                                             const long long* __restrict__ ek) {
    const double zz = negate ? -z : z;
    const long long kz = order_key(zz);
    if (kz < ek[0] || kz >= ek[S]) return -1;
    int k = (int)((approx_float(zz) - tail_f) * inv_w_f);
    k = k < 0 ? 0 : (k > S - 1 ? S - 1 : k);
    while (kz < ek[k]) --k;
    while (kz >= ek[k + 1]) ++k;
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

// --------------------------------------------------- FP32 sin/cos of 2 pi f
// sin and cos of 2*pi*f for |f| <= 1/2 turn: quadrant q = rint(4 f) and the
// exact remainder r = f - q/4 in [-1/8, 1/8] turn, theta = 2 pi r with 2 pi
// split into a float and its residual (so theta carries no systematic
// scale error), then the Maclaurin series of sin (to theta^11) and cos (to
// theta^10): truncation error below 1e-11 and 2e-10 on |theta| <= pi/4, far
// under the FP32 rounding of the result.  A truncation error of fixed sign
// would make cos^2 + sin^2 drift from 1 the same way every turn, growing the
// betatron amplitude -- and, through amplitude detuning, the phase error --
// secularly.  The quadrant rotates (s, c) by q * 90 degrees.
__device__ __forceinline__ void sincos_2pi(float f, float* s, float* c) {
    const float q = rintf(4.0f * f);
    const float r = fmaf(-0.25f, q, f);
    const float th = fmaf(r, 6.28318548202514648438f, r * -1.7484556e-7f);
    const float t2 = th * th;
    float ps = fmaf(t2, -2.5052108385e-8f, 2.7557319224e-6f);   // -1/11!, 1/9!
    ps = fmaf(t2, ps, -1.9841269841e-4f);                        // -1/7!
    ps = fmaf(t2, ps, 8.3333333333e-3f);                         //  1/5!
    ps = fmaf(t2, ps, -1.6666666667e-1f);                        // -1/3!
    const float sn = fmaf(th * t2, ps, th);
    float pc = fmaf(t2, -2.7557319224e-7f, 2.4801587302e-5f);    // -1/10!, 1/8!
    pc = fmaf(t2, pc, -1.3888888889e-3f);                        // -1/6!
    pc = fmaf(t2, pc, 4.1666666667e-2f);                         //  1/4!
    pc = fmaf(t2, pc, -0.5f);                                    // -1/2!
    const float cs = fmaf(t2, pc, 1.0f);
    const int k = (int)q & 3;
    const float a = (k & 1) ? cs : sn;
    const float b = (k & 1) ? sn : cs;
    *s = (k & 2) ? -a : a;
    *c = ((k + 1) & 2) ? -b : b;
}

// ------------------------------------------------------- float-float phase
// sin and cos of 2*pi*(hi + lo + d) for a phase given in turns as the
// unevaluated sum of a float-float base (hi, lo) and a small float d.
// The integer number of turns is removed exactly (Knuth two-sum, then
// t - rint(t) is exact), the remaining fraction f + g is split into a float
// f and its residual g; sin/cos(2 pi f) is corrected to first order in g.
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
    sincos_2pi(f, &sp, &cp);
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

// ------------------------------------------- packed FP32 pairs (f32x2)
// Two particles per instruction on the sm_100 family's paired FP32 pipes
// (FFMA2 / FADD2 / FMUL2).  Each lane rounds as an IEEE fmaf / + / * and
// the packed operations are never contracted, so the forms below run the
// operation sequence of their scalar counterparts above, lane by lane,
// with every written rounding kept (the scalar forms leave the compiler
// free to fuse a product into a following sum).
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
    return __ffma2_rn(a, b, c);
}
// a - b, one rounding (b * -1 is exact)
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
}
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

// quadrant rotation of sincos_2pi for one lane
__device__ __forceinline__ void quadrant_2pi(float q, float sn, float cs,
                                             float* s, float* c) {
    const int k = (int)q & 3;
    const float a = (k & 1) ? cs : sn;
    const float b = (k & 1) ? sn : cs;
    *s = (k & 2) ? -a : a;
    *c = ((k + 1) & 2) ? -b : b;
}

// sincos_2pi of two lanes
__device__ __forceinline__ void sincos_2pi_x2(float2 f, float2* s, float2* c) {
    const float2 q = make_float2(rintf(4.0f * f.x), rintf(4.0f * f.y));
    const float2 r = fma2(f2(-0.25f), q, f);
    const float2 th = fma2(r, f2(6.28318548202514648438f),
                           mul2(r, f2(-1.7484556e-7f)));
    const float2 t2 = mul2(th, th);
    float2 ps = fma2(t2, f2(-2.5052108385e-8f), f2(2.7557319224e-6f));
    ps = fma2(t2, ps, f2(-1.9841269841e-4f));
    ps = fma2(t2, ps, f2(8.3333333333e-3f));
    ps = fma2(t2, ps, f2(-1.6666666667e-1f));
    const float2 sn = fma2(mul2(th, t2), ps, th);
    float2 pc = fma2(t2, f2(-2.7557319224e-7f), f2(2.4801587302e-5f));
    pc = fma2(t2, pc, f2(-1.3888888889e-3f));
    pc = fma2(t2, pc, f2(4.1666666667e-2f));
    pc = fma2(t2, pc, f2(-0.5f));
    const float2 cs = fma2(t2, pc, f2(1.0f));
    quadrant_2pi(q.x, sn.x, cs.x, &s->x, &c->x);
    quadrant_2pi(q.y, sn.y, cs.y, &s->y, &c->y);
}

// sincos_turns of two lanes, the float-float base given per lane
__device__ __forceinline__ void sincos_turns_x2(float2 hi, float2 lo, float2 d,
                                                float2* s, float2* c) {
    const float2 t = add2(hi, d);
    const float2 bp = sub2(t, hi);
    float2 err = add2(sub2(hi, sub2(t, bp)), sub2(d, bp));
    err = add2(err, lo);
    const float2 r = sub2(t, make_float2(rintf(t.x), rintf(t.y)));
    const float2 f = add2(r, err);
    const float2 g = add2(sub2(r, f), err);
    float2 sp, cp;
    sincos_2pi_x2(f, &sp, &cp);
    const float2 dl = mul2(f2(6.28318530717958647692f), g);
    *s = fma2(dl, cp, sp);
    *c = fma2(neg2(dl), sp, cp);
}

// sin_turns_of_product of two lanes
__device__ __forceinline__ float2 sin_turns_of_product_x2(float2 z, float mh,
                                                          float ml, float oh,
                                                          float ol) {
    const float2 p = mul2(z, f2(mh));
    float2 e = fma2(z, f2(mh), neg2(p));
    e = fma2(z, f2(ml), e);
    float2 s, c;
    sincos_turns_x2(p, add2(e, f2(ol)), f2(oh), &s, &c);
    return s;
}

}  // namespace phk
