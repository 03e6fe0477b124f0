// The fused track kernel and the batched track kernel as templates, with
// their launch helpers.  Included by the per-precision translation units
// (phk_track_f32.cu, phk_track_f64.cu), which instantiate and launch them,
// and by phk_kernels.cu for the host-side planning helpers.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <cooperative_groups.h>

#include <type_traits>

#include "phk_device.cuh"
#include "phk_internal.h"

namespace phk {

// ===================================================================
// particle tiles: VEC particles per thread, one register array per
// coordinate; every op below works op-major / particle-minor, reading its
// parameters once per tile
// ===================================================================

template <typename T, int VEC>
struct Tile {
    T c[6][VEC];
};

// ===================================================================
// element arithmetic, plain FP64 form (reference evaluation order)
// ===================================================================

// ChromaticitySegment detune: Horner with separately rounded steps, lowest
// coefficient first, then the extra dp factors of the order > 3 path.
__device__ __forceinline__ double chroma_poly(const double* c, int n, int z,
                                             double dp) {
    double r = c[n - 1];
    for (int i = n - 2; i >= 0; --i) r = add(c[i], mul(r, dp));
    r = mul(r, dp);
    for (int i = 0; i < z; ++i) r = mul(r, dp);
    return r;
}

// The detuned map below feeds sin / cos of a per-particle phase, which no
// FP64 evaluation reproduces bit for bit anyway; its products and sums are
// therefore fused (one rounding per multiply-add) to save FP64 operations
// on GB300's narrow FP64 pipe.  Maps without per-particle transcendentals
// keep the reference's separately rounded order.
__device__ __forceinline__ double amp_action(double c1, double twoa, double b,
                                             double u, double up) {
    // 1/2 * ((1+a^2)/b * u**2 + 2*a * u*up + b * up**2)
    double s = c1 * u * u;
    if (twoa != 0.0) s = fma(twoa * u, up, s);
    s = fma(b * up, up, s);
    return 0.5 * s;
}

__device__ __forceinline__ double ij_term(double I, double J, bool hi,
                                          bool hj, double cc, double ss) {
    if (hi && hj) return fma(I, cc, J * ss);
    if (hi) return I * cc;
    if (hj) return J * ss;
    return 0.0;
}

// OP0 (unused here): see the FP32 form
template <int VEC, bool OP0 = false>
__device__ __forceinline__ void op_transverse(const phk_op& op,
                                              const phk_program& prog,
                                              Tile<double, VEC>& t) {
    const double* p = op.p;
    const bool disp = op.flags & PHK_FLAG_DISPERSION;
    const double Dx0 = p[16], Dx1 = p[17], Dy0 = p[18], Dy1 = p[19];
    double (&x)[VEC] = t.c[PHK_X];
    double (&xp)[VEC] = t.c[PHK_XP];
    double (&y)[VEC] = t.c[PHK_Y];
    double (&yp)[VEC] = t.c[PHK_YP];
    const double (&dp)[VEC] = t.c[PHK_DP];
    if (!(op.flags & PHK_FLAG_DETUNED)) {
        const double M00 = p[0], M01 = p[1], M10 = p[2], M11 = p[3];
        const double M22 = p[4], M23 = p[5], M32 = p[6], M33 = p[7];
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            if (disp) {
                x[j] = sub(x[j], mul(Dx0, dp[j]));
                y[j] = sub(y[j], mul(Dy0, dp[j]));
            }
            const double nx = add(mul(M00, x[j]), mul(M01, xp[j]));
            const double nxp = add(mul(M10, x[j]), mul(M11, xp[j]));
            const double ny = add(mul(M22, y[j]), mul(M23, yp[j]));
            const double nyp = add(mul(M32, y[j]), mul(M33, yp[j]));
            x[j] = nx; xp[j] = nxp; y[j] = ny; yp[j] = nyp;
            if (disp) {
                x[j] = add(x[j], mul(Dx1, dp[j]));
                y[j] = add(y[j], mul(Dy1, dp[j]));
            }
        }
        return;
    }
    double phx[VEC], phy[VEC];
#pragma unroll
    for (int j = 0; j < VEC; ++j) { phx[j] = p[20]; phy[j] = p[21]; }
    for (int d = 0; d < op.det_count; ++d) {
        const phk_detuner& dt = prog.det[op.det_begin + d];
        if (dt.kind == PHK_DET_CHROMA) {
            const int nx = dt.nx, ny = dt.ny, zx = dt.zx, zy = dt.zy;
#pragma unroll
            for (int j = 0; j < VEC; ++j) {
                phx[j] = add(phx[j], chroma_poly(dt.c, nx, zx, dp[j]));
                phy[j] = add(phy[j], chroma_poly(dt.c + 8, ny, zy, dp[j]));
            }
        } else {
            const double ax = dt.c[0], ay = dt.c[1], axy = dt.c[2], ayx = dt.c[3];
            const double c1x = dt.c[4], tax = dt.c[5], bx = dt.c[6];
            const double c1y = dt.c[7], tay = dt.c[8], by = dt.c[9];
            const double p0 = dt.c[10], ip0 = dt.c[11];
#pragma unroll
            for (int j = 0; j < VEC; ++j) {
                const double Jx = amp_action(c1x, tax, bx, x[j], xp[j]);
                const double Jy = amp_action(c1y, tay, by, y[j], yp[j]);
                phx[j] = add(phx[j], div_by(fma(ax, Jx, axy * Jy), p0, ip0));
                phy[j] = add(phy[j], div_by(fma(ay, Jy, ayx * Jx), p0, ip0));
            }
        }
    }
    const double twopi = p[22];
    const double phx0 = p[23], sx0 = p[24], cx0 = p[25];
    const double phy0 = p[26], sy0 = p[27], cy0 = p[28];
    const int m = op.ij_mask;
    double I[8], J[8];
    bool hI[8], hJ[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        I[e] = p[e]; J[e] = p[8 + e];
        hI[e] = (m >> e) & 1; hJ[e] = (m >> (8 + e)) & 1;
    }
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
        double sx, cx, sy, cy;
        sincos_about(mul(phx[j], twopi), phx0, sx0, cx0, &sx, &cx);
        sincos_about(mul(phy[j], twopi), phy0, sy0, cy0, &sy, &cy);
        const double M00 = ij_term(I[0], J[0], hI[0], hJ[0], cx, sx);
        const double M01 = ij_term(I[1], J[1], hI[1], hJ[1], cx, sx);
        const double M10 = ij_term(I[2], J[2], hI[2], hJ[2], cx, sx);
        const double M11 = ij_term(I[3], J[3], hI[3], hJ[3], cx, sx);
        const double M22 = ij_term(I[4], J[4], hI[4], hJ[4], cy, sy);
        const double M23 = ij_term(I[5], J[5], hI[5], hJ[5], cy, sy);
        const double M32 = ij_term(I[6], J[6], hI[6], hJ[6], cy, sy);
        const double M33 = ij_term(I[7], J[7], hI[7], hJ[7], cy, sy);
        if (disp) {
            x[j] = sub(x[j], mul(Dx0, dp[j]));
            y[j] = sub(y[j], mul(Dy0, dp[j]));
        }
        const double nx = fma(M00, x[j], M01 * xp[j]);
        const double nxp = fma(M10, x[j], M11 * xp[j]);
        const double ny = fma(M22, y[j], M23 * yp[j]);
        const double nyp = fma(M32, y[j], M33 * yp[j]);
        x[j] = nx; xp[j] = nxp; y[j] = ny; yp[j] = nyp;
        if (disp) {
            x[j] = add(x[j], mul(Dx1, dp[j]));
            y[j] = add(y[j], mul(Dy1, dp[j]));
        }
    }
}

template <int VEC>
__device__ __forceinline__ void op_drift(const phk_op& op,
                                         Tile<double, VEC>& t) {
    const double br = op.p[0], eta0 = op.p[1], L = op.p[2];
    const bool shrink = op.flags & PHK_FLAG_SHRINK;
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
        const double z = t.c[PHK_Z][j];
        const double zz = shrink ? mul(br, z) : z;
        t.c[PHK_Z][j] = sub(zz, mul(mul(eta0, t.c[PHK_DP][j]), L));
    }
}

template <int VEC>
__device__ __forceinline__ void op_rfkick(const phk_op& op,
                                          Tile<double, VEC>& t) {
    const double* p = op.p;
    const int f = op.flags;
    const double h = p[0], twopi = p[1], C = p[2], off = p[3], lock = p[4];
    const double A = p[5], p0o = p[6], pinc = p[7], p0n = p[8];
    const double Dx = p[9], Dy = p[10], iC = p[11], ip0n = p[12];
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
        double& dp = t.c[PHK_DP][j];
        if (f & PHK_FLAG_DISPERSION) {
            t.c[PHK_X][j] = sub(t.c[PHK_X][j], mul(Dx, dp));
            t.c[PHK_Y][j] = sub(t.c[PHK_Y][j], mul(Dy, dp));
        }
        double phi = mul(h, div_by(mul(twopi, t.c[PHK_Z][j]), C, iC));
        if (f & PHK_FLAG_PHI_OFFSET) phi = add(phi, off);
        if (f & PHK_FLAG_PHI_LOCK) phi = add(phi, lock);
        double s = mul(A, sin(phi));
        if (f & PHK_FLAG_P_INC) s = sub(s, pinc);
        dp = div_by(add(mul(dp, p0o), s), p0n, ip0n);
        if (f & PHK_FLAG_DISPERSION) {
            t.c[PHK_X][j] = add(t.c[PHK_X][j], mul(Dx, dp));
            t.c[PHK_Y][j] = add(t.c[PHK_Y][j], mul(Dy, dp));
        }
    }
}

// Drift and RF kick of an RFSystems element (Drift, Kick, Drift), plain
// form.  The kick's per-particle sine makes the step inexact whatever the
// evaluation order, so around it the arithmetic is regrouped to save FP64
// operations (GB300 runs FP64 at a small fraction of the FP32 rate): the
// drift is one multiply-add with eta0 * L, the phase one multiply-add with
// h 2 pi / C, and the momentum update
//   dp' = (dp p0_old + A sin(phi) - dp_inc) / p0_new
// is dp (p0_old / p0_new) + (A / p0_new) sin(phi) - dp_inc / p0_new with
// the ratios formed once per thread (the ratio is exactly 1 without
// acceleration).  The separately rounded forms above remain for other
// element sequences.
template <int VEC>
__device__ __forceinline__ void op_drift_rf(const phk_op& op,
                                            Tile<double, VEC>& t) {
    const double br = op.p[0], etaL = op.p[1] * op.p[2];
    const bool shrink = op.flags & PHK_FLAG_SHRINK;
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
        const double z = t.c[PHK_Z][j];
        const double zz = shrink ? mul(br, z) : z;
        t.c[PHK_Z][j] = fma(-etaL, t.c[PHK_DP][j], zz);
    }
}

template <int VEC>
__device__ __forceinline__ void op_rfkick_rf(const phk_op& op,
                                             Tile<double, VEC>& t) {
    const double* p = op.p;
    const int f = op.flags;
    const double hk = p[0] * p[1] * p[11];   // h 2 pi / C
    double off = 0.0;
    if (f & PHK_FLAG_PHI_OFFSET) off = add(off, p[3]);
    if (f & PHK_FLAG_PHI_LOCK) off = add(off, p[4]);
    const double Ar = p[5] * p[12];          // A / p0_new
    const double ratio = p[6] == p[8] ? 1.0 : p[6] * p[12];
    const double pinc = (f & PHK_FLAG_P_INC) ? p[7] * p[12] : 0.0;
    const double Dx = p[9], Dy = p[10];
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
        double& dp = t.c[PHK_DP][j];
        if (f & PHK_FLAG_DISPERSION) {
            t.c[PHK_X][j] = sub(t.c[PHK_X][j], mul(Dx, dp));
            t.c[PHK_Y][j] = sub(t.c[PHK_Y][j], mul(Dy, dp));
        }
        const double s = sin(fma(hk, t.c[PHK_Z][j], off));
        dp = fma(dp, ratio, fma(Ar, s, -pinc));
        if (f & PHK_FLAG_DISPERSION) {
            t.c[PHK_X][j] = add(t.c[PHK_X][j], mul(Dx, dp));
            t.c[PHK_Y][j] = add(t.c[PHK_Y][j], mul(Dy, dp));
        }
    }
}

template <int VEC>
__device__ __forceinline__ void op_linear_long(const phk_op& op,
                                               Tile<double, VEC>& t) {
    const double* p = op.p;
    const double cs = p[0], sn = p[1], lf = p[2], Dx = p[3], Dy = p[4];
    const double ilf = p[5];
    const bool disp = op.flags & PHK_FLAG_DISPERSION;
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
        double& z = t.c[PHK_Z][j];
        double& dp = t.c[PHK_DP][j];
        if (disp) {
            t.c[PHK_X][j] = sub(t.c[PHK_X][j], mul(Dx, dp));
            t.c[PHK_Y][j] = sub(t.c[PHK_Y][j], mul(Dy, dp));
        }
        const double z0 = z, dp0 = dp;
        z = sub(mul(z0, cs), mul(mul(lf, dp0), sn));
        dp = add(mul(dp0, cs), mul(div_by(z0, lf, ilf), sn));
        if (disp) {
            t.c[PHK_X][j] = add(t.c[PHK_X][j], mul(Dx, dp));
            t.c[PHK_Y][j] = add(t.c[PHK_Y][j], mul(Dy, dp));
        }
    }
}

template <int VEC>
__device__ __forceinline__ void op_scale(const phk_op& op,
                                         Tile<double, VEC>& t) {
    const double f = op.p[0];
#pragma unroll
    for (int j = 0; j < VEC; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) t.c[q][j] = mul(t.c[q][j], f);
}

// the device means a damper op reads (phk_stats.means, FP64 then FP32)
__device__ __forceinline__ const double* damper_means(const phk_op& op) {
    unsigned long long bits;
    memcpy(&bits, &op.p[31], sizeof(bits));
    return reinterpret_cast<const double*>(bits);
}

// TransverseDamper.track_all (feedback/transverse_damper.py:64-86): the
// reference's order, xp -= (g sin) <xp>, then xp -= ((g cos) <x>) / beta
template <int VEC>
__device__ __forceinline__ void op_damper(const phk_op& op,
                                          Tile<double, VEC>& t) {
    const double* m = damper_means(op);
    const bool reactive = op.flags & PHK_FLAG_REACTIVE;
#pragma unroll
    for (int pl = 0; pl < 2; ++pl) {
        if (!(op.flags & (pl == 0 ? PHK_FLAG_DAMP_X : PHK_FLAG_DAMP_Y))) continue;
        const int u = pl == 0 ? PHK_X : PHK_Y, up = pl == 0 ? PHK_XP : PHK_YP;
        const double* g = op.p + 3 * pl;
        const double c1 = mul(g[0], __ldg(m + up));
        const double c2 = reactive ? __ddiv_rn(mul(g[1], __ldg(m + u)), g[2]) : 0.0;
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            t.c[up][j] = __dsub_rn(t.c[up][j], c1);
            if (reactive) t.c[up][j] = __dsub_rn(t.c[up][j], c2);
        }
    }
}

// ===================================================================
// element arithmetic, FP32 precision form (parameters packed as floats)
// ===================================================================

__device__ __forceinline__ float chroma_poly_f32(const float* c, int n, int z,
                                                 float dp) {
    float r = c[n - 1];
    for (int i = n - 2; i >= 0; --i) r = fmaf(r, dp, c[i]);
    r *= dp;
    for (int i = 0; i < z; ++i) r *= dp;
    return r;
}

// dq += the chromatic detuning of VEC particles (ChromaticitySegment.detune,
// trackers/detuners.py:64-98): Horner orders 1-3 inline, anything else
// through the general loop.  The branches are uniform.
template <int VEC>
__device__ __forceinline__ void chroma_add_f32(const float* c, int n, int z,
                                               const float (&dp)[VEC],
                                               float (&dq)[VEC]) {
    if (z == 0 && n == 1) {
#pragma unroll
        for (int j = 0; j < VEC; ++j) dq[j] = fmaf(c[0], dp[j], dq[j]);
    } else if (z == 0 && n == 2) {
#pragma unroll
        for (int j = 0; j < VEC; ++j)
            dq[j] = fmaf(fmaf(c[1], dp[j], c[0]), dp[j], dq[j]);
    } else if (z == 0 && n == 3) {
#pragma unroll
        for (int j = 0; j < VEC; ++j)
            dq[j] = fmaf(fmaf(fmaf(c[2], dp[j], c[1]), dp[j], c[0]), dp[j],
                         dq[j]);
    } else {
#pragma unroll
        for (int j = 0; j < VEC; ++j) dq[j] += chroma_poly_f32(c, n, z, dp[j]);
    }
}

// dqx, dqy += the detuning of VEC particles by one detuner
template <int VEC>
__device__ __forceinline__ void detune_f32(const phk_detuner& dt,
                                           const Tile<float, VEC>& t,
                                           float (&dqx)[VEC],
                                           float (&dqy)[VEC]) {
    const float* c = reinterpret_cast<const float*>(dt.c);
    if (dt.kind == PHK_DET_CHROMA) {
        chroma_add_f32<VEC>(c, dt.nx, dt.zx, t.c[PHK_DP], dqx);
        chroma_add_f32<VEC>(c + 8, dt.ny, dt.zy, t.c[PHK_DP], dqy);
    } else {
        // c = dapp_x/p0, dapp_y/p0, dapp_xy/p0, dapp_yx/p0,
        //     (1+ax^2)/bx, 2ax, bx, (1+ay^2)/by, 2ay, by
        const float ax = c[0], ay = c[1], axy = c[2], ayx = c[3];
        const float c1x = c[4], tax = c[5], bx = c[6];
        const float c1y = c[7], tay = c[8], by = c[9];
        const float (&x)[VEC] = t.c[PHK_X];
        const float (&xp)[VEC] = t.c[PHK_XP];
        const float (&y)[VEC] = t.c[PHK_Y];
        const float (&yp)[VEC] = t.c[PHK_YP];
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            const float Jx = 0.5f * fmaf(bx * xp[j], xp[j],
                                         fmaf(tax * x[j], xp[j], c1x * x[j] * x[j]));
            const float Jy = 0.5f * fmaf(by * yp[j], yp[j],
                                         fmaf(tay * y[j], yp[j], c1y * y[j] * y[j]));
            dqx[j] += fmaf(ax, Jx, axy * Jy);
            dqy[j] += fmaf(ay, Jy, ayx * Jx);
        }
    }
}

// OP0: the op is prog.op[0] of a specialised shape, whose detuners start at
// det[0] (program_shape checks it), so the first two are read at
// compile-time offsets of the parameter block.
// detune_f32 of two particles on the paired FP32 pipes
__device__ __forceinline__ void detune_f32_x2(const phk_detuner& dt,
                                              const Tile<float, 2>& t,
                                              float2& dqx, float2& dqy) {
    const float* c = reinterpret_cast<const float*>(dt.c);
    const float2 DP = make_float2(t.c[PHK_DP][0], t.c[PHK_DP][1]);
    if (dt.kind == PHK_DET_CHROMA) {
        const int n[2] = {dt.nx, dt.ny}, z[2] = {dt.zx, dt.zy};
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const float* cq = c + 8 * q;
            float2& dq = q ? dqy : dqx;
            if (z[q] == 0 && n[q] == 1) {
                dq = fma2(f2(cq[0]), DP, dq);
            } else if (z[q] == 0 && n[q] == 2) {
                dq = fma2(fma2(f2(cq[1]), DP, f2(cq[0])), DP, dq);
            } else if (z[q] == 0 && n[q] == 3) {
                dq = fma2(fma2(fma2(f2(cq[2]), DP, f2(cq[1])), DP, f2(cq[0])),
                          DP, dq);
            } else {
                dq.x += chroma_poly_f32(cq, n[q], z[q], DP.x);
                dq.y += chroma_poly_f32(cq, n[q], z[q], DP.y);
            }
        }
    } else {
        const float2 X = make_float2(t.c[PHK_X][0], t.c[PHK_X][1]);
        const float2 XP = make_float2(t.c[PHK_XP][0], t.c[PHK_XP][1]);
        const float2 Y = make_float2(t.c[PHK_Y][0], t.c[PHK_Y][1]);
        const float2 YP = make_float2(t.c[PHK_YP][0], t.c[PHK_YP][1]);
        const float2 Jx = mul2(f2(0.5f),
                               fma2(mul2(f2(c[6]), XP), XP,
                                    fma2(mul2(f2(c[5]), X), XP,
                                         mul2(mul2(f2(c[4]), X), X))));
        const float2 Jy = mul2(f2(0.5f),
                               fma2(mul2(f2(c[9]), YP), YP,
                                    fma2(mul2(f2(c[8]), Y), YP,
                                         mul2(mul2(f2(c[7]), Y), Y))));
        dqx = add2(dqx, fma2(f2(c[0]), Jx, mul2(f2(c[2]), Jy)));
        dqy = add2(dqy, fma2(f2(c[1]), Jy, mul2(f2(c[3]), Jx)));
    }
}

// op_transverse for two particles per thread on the paired FP32 pipes:
// the same operations as the scalar form below, lane for lane
template <bool OP0>
__device__ __forceinline__ void op_transverse_x2(const phk_op& op,
                                                 const phk_program& prog,
                                                 Tile<float, 2>& t) {
    const float* p = reinterpret_cast<const float*>(op.p);
    const bool disp = op.flags & PHK_FLAG_DISPERSION;
    float2 X = make_float2(t.c[PHK_X][0], t.c[PHK_X][1]);
    float2 XP = make_float2(t.c[PHK_XP][0], t.c[PHK_XP][1]);
    float2 Y = make_float2(t.c[PHK_Y][0], t.c[PHK_Y][1]);
    float2 YP = make_float2(t.c[PHK_YP][0], t.c[PHK_YP][1]);
    const float2 DP = make_float2(t.c[PHK_DP][0], t.c[PHK_DP][1]);
    float2 M[8];
    const bool detuned = op.flags & PHK_FLAG_DETUNED;
    if (detuned) {
        float2 dqx = f2(0.f), dqy = f2(0.f);
        const int nd = op.det_count;
        if (OP0) {
            if (nd > 0) detune_f32_x2(prog.det[0], t, dqx, dqy);
            if (nd > 1) detune_f32_x2(prog.det[1], t, dqx, dqy);
            for (int d = 2; d < nd; ++d) detune_f32_x2(prog.det[d], t, dqx, dqy);
        } else {
            for (int d = 0; d < nd; ++d)
                detune_f32_x2(prog.det[op.det_begin + d], t, dqx, dqy);
        }
        float2 sx, cx, sy, cy;
        sincos_turns_x2(f2(p[16]), f2(p[17]), dqx, &sx, &cx);
        sincos_turns_x2(f2(p[18]), f2(p[19]), dqy, &sy, &cy);
        // I and J are float-float (p[40..55] their low parts)
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            M[e] = fma2(f2(p[e]), cx,
                        fma2(f2(p[8 + e]), sx,
                             fma2(f2(p[40 + e]), cx, mul2(f2(p[48 + e]), sx))));
            M[4 + e] = fma2(f2(p[4 + e]), cy,
                            fma2(f2(p[12 + e]), sy,
                                 fma2(f2(p[44 + e]), cy, mul2(f2(p[52 + e]), sy))));
        }
    } else {
#pragma unroll
        for (int e = 0; e < 8; ++e) M[e] = f2(p[e]);
    }
    if (disp) {
        X = fma2(f2(-p[32]), DP, X);
        Y = fma2(f2(-p[34]), DP, Y);
    }
    float2 cxr = f2(0.f), cxp = f2(0.f), cyr = f2(0.f), cyp = f2(0.f);
    if (!detuned) {
        // low parts of the constant matrix
        cxr = fma2(f2(p[40]), X, mul2(f2(p[41]), XP));
        cxp = fma2(f2(p[42]), X, mul2(f2(p[43]), XP));
        cyr = fma2(f2(p[44]), Y, mul2(f2(p[45]), YP));
        cyp = fma2(f2(p[46]), Y, mul2(f2(p[47]), YP));
    }
    const float2 nx = fma2(M[0], X, fma2(M[1], XP, cxr));
    const float2 nxp = fma2(M[2], X, fma2(M[3], XP, cxp));
    const float2 ny = fma2(M[4], Y, fma2(M[5], YP, cyr));
    const float2 nyp = fma2(M[6], Y, fma2(M[7], YP, cyp));
    X = nx; XP = nxp; Y = ny; YP = nyp;
    if (disp) {
        X = fma2(f2(p[33]), DP, X);
        Y = fma2(f2(p[35]), DP, Y);
    }
    t.c[PHK_X][0] = X.x; t.c[PHK_X][1] = X.y;
    t.c[PHK_XP][0] = XP.x; t.c[PHK_XP][1] = XP.y;
    t.c[PHK_Y][0] = Y.x; t.c[PHK_Y][1] = Y.y;
    t.c[PHK_YP][0] = YP.x; t.c[PHK_YP][1] = YP.y;
}

template <int VEC, bool OP0 = false>
__device__ __forceinline__ void op_transverse(const phk_op& op,
                                              const phk_program& prog,
                                              Tile<float, VEC>& t) {
    if constexpr (VEC == 2) {
        op_transverse_x2<OP0>(op, prog, t);
    } else {
        const float* p = reinterpret_cast<const float*>(op.p);
        const bool disp = op.flags & PHK_FLAG_DISPERSION;
        const float Dx0 = p[32], Dx1 = p[33], Dy0 = p[34], Dy1 = p[35];
        float (&x)[VEC] = t.c[PHK_X];
        float (&xp)[VEC] = t.c[PHK_XP];
        float (&y)[VEC] = t.c[PHK_Y];
        float (&yp)[VEC] = t.c[PHK_YP];
        const float (&dp)[VEC] = t.c[PHK_DP];
        float M[8][VEC];
        if (op.flags & PHK_FLAG_DETUNED) {
            float dqx[VEC], dqy[VEC];
    #pragma unroll
            for (int j = 0; j < VEC; ++j) { dqx[j] = 0.f; dqy[j] = 0.f; }
            const int nd = op.det_count;
            if (OP0) {
                if (nd > 0) detune_f32<VEC>(prog.det[0], t, dqx, dqy);
                if (nd > 1) detune_f32<VEC>(prog.det[1], t, dqx, dqy);
                for (int d = 2; d < nd; ++d) detune_f32<VEC>(prog.det[d], t, dqx, dqy);
            } else {
                for (int d = 0; d < nd; ++d)
                    detune_f32<VEC>(prog.det[op.det_begin + d], t, dqx, dqy);
            }
            const float qxh = p[16], qxl = p[17], qyh = p[18], qyl = p[19];
    #pragma unroll
            for (int j = 0; j < VEC; ++j) {
                float sx, cx, sy, cy;
                sincos_turns(qxh, qxl, dqx[j], &sx, &cx);
                sincos_turns(qyh, qyl, dqy[j], &sy, &cy);
                // I and J are float-float (p[40..55] their low parts)
    #pragma unroll
                for (int e = 0; e < 4; ++e) {
                    M[e][j] = fmaf(p[e], cx, fmaf(p[8 + e], sx,
                                                  fmaf(p[40 + e], cx, p[48 + e] * sx)));
                    M[4 + e][j] = fmaf(p[4 + e], cy,
                                       fmaf(p[12 + e], sy,
                                            fmaf(p[44 + e], cy, p[52 + e] * sy)));
                }
            }
        } else {
    #pragma unroll
            for (int j = 0; j < VEC; ++j)
    #pragma unroll
                for (int e = 0; e < 8; ++e) M[e][j] = p[e];
        }
        // low parts of a constant matrix (zero for a per-particle one)
        const bool ml = !(op.flags & PHK_FLAG_DETUNED);
    #pragma unroll
        for (int j = 0; j < VEC; ++j) {
            if (disp) {
                x[j] = fmaf(-Dx0, dp[j], x[j]);
                y[j] = fmaf(-Dy0, dp[j], y[j]);
            }
            float cxr = 0.f, cxp = 0.f, cyr = 0.f, cyp = 0.f;
            if (ml) {
                cxr = fmaf(p[40], x[j], p[41] * xp[j]);
                cxp = fmaf(p[42], x[j], p[43] * xp[j]);
                cyr = fmaf(p[44], y[j], p[45] * yp[j]);
                cyp = fmaf(p[46], y[j], p[47] * yp[j]);
            }
            const float nx = fmaf(M[0][j], x[j], fmaf(M[1][j], xp[j], cxr));
            const float nxp = fmaf(M[2][j], x[j], fmaf(M[3][j], xp[j], cxp));
            const float ny = fmaf(M[4][j], y[j], fmaf(M[5][j], yp[j], cyr));
            const float nyp = fmaf(M[6][j], y[j], fmaf(M[7][j], yp[j], cyp));
            x[j] = nx; xp[j] = nxp; y[j] = ny; yp[j] = nyp;
            if (disp) {
                x[j] = fmaf(Dx1, dp[j], x[j]);
                y[j] = fmaf(Dy1, dp[j], y[j]);
            }
        }
    }
}

template <int VEC>
__device__ __forceinline__ void op_drift(const phk_op& op,
                                         Tile<float, VEC>& t) {
    // p: beta_ratio, eta0 * L (hi, lo), beta_ratio lo
    const float* p = reinterpret_cast<const float*>(op.p);
    const float br = p[0], etaL = p[1], etaLl = p[2], brl = p[3];
    const bool shrink = op.flags & PHK_FLAG_SHRINK;
    if constexpr (VEC == 2) {
        const float2 Z = make_float2(t.c[PHK_Z][0], t.c[PHK_Z][1]);
        const float2 DP = make_float2(t.c[PHK_DP][0], t.c[PHK_DP][1]);
        const float2 zs = shrink ? fma2(f2(br), Z, mul2(f2(brl), Z)) : Z;
        const float2 zn = fma2(f2(-etaL), DP, fma2(f2(-etaLl), DP, zs));
        t.c[PHK_Z][0] = zn.x; t.c[PHK_Z][1] = zn.y;
    } else {
    #pragma unroll
        for (int j = 0; j < VEC; ++j) {
            // z = beta_ratio * z - (eta0 * L) * dp, constants float-float
            const float z = t.c[PHK_Z][j];
            const float dp = t.c[PHK_DP][j];
            const float zs = shrink ? fmaf(br, z, brl * z) : z;
            t.c[PHK_Z][j] = fmaf(-etaL, dp, fmaf(-etaLl, dp, zs));
        }
    }
}

template <int VEC>
__device__ __forceinline__ void op_rfkick(const phk_op& op,
                                          Tile<float, VEC>& t) {
    // p: h/C (hi, lo) turns per metre, (phi_offset+phi_lock)/2pi (hi, lo),
    //    A/p0_new, p0_old/p0_new, p_inc/p0_new, -, D_x, D_y, then the low
    //    parts of A/p0_new and p0_old/p0_new
    const float* p = reinterpret_cast<const float*>(op.p);
    const float mh = p[0], ml = p[1], oh = p[2], ol = p[3];
    const float A = p[4], ratio = p[5], pinc = p[6], Dx = p[8], Dy = p[9];
    const float Al = p[10], ratiol = p[11];
    const bool disp = op.flags & PHK_FLAG_DISPERSION;
    if constexpr (VEC == 2) {
        float2 DP = make_float2(t.c[PHK_DP][0], t.c[PHK_DP][1]);
        float2 X = make_float2(t.c[PHK_X][0], t.c[PHK_X][1]);
        float2 Y = make_float2(t.c[PHK_Y][0], t.c[PHK_Y][1]);
        if (disp) {
            X = fma2(f2(-Dx), DP, X);
            Y = fma2(f2(-Dy), DP, Y);
        }
        const float2 s = sin_turns_of_product_x2(
            make_float2(t.c[PHK_Z][0], t.c[PHK_Z][1]), mh, ml, oh, ol);
        DP = fma2(f2(A), s, fma2(f2(Al), s,
                                 fma2(DP, f2(ratio), fma2(DP, f2(ratiol), f2(-pinc)))));
        if (disp) {
            X = fma2(f2(Dx), DP, X);
            Y = fma2(f2(Dy), DP, Y);
        }
        t.c[PHK_DP][0] = DP.x; t.c[PHK_DP][1] = DP.y;
        t.c[PHK_X][0] = X.x; t.c[PHK_X][1] = X.y;
        t.c[PHK_Y][0] = Y.x; t.c[PHK_Y][1] = Y.y;
    } else {
    #pragma unroll
        for (int j = 0; j < VEC; ++j) {
            float& dp = t.c[PHK_DP][j];
            if (disp) {
                t.c[PHK_X][j] = fmaf(-Dx, dp, t.c[PHK_X][j]);
                t.c[PHK_Y][j] = fmaf(-Dy, dp, t.c[PHK_Y][j]);
            }
            const float s = sin_turns_of_product(t.c[PHK_Z][j], mh, ml, oh, ol);
            dp = fmaf(A, s, fmaf(Al, s, fmaf(dp, ratio, fmaf(dp, ratiol, -pinc))));
            if (disp) {
                t.c[PHK_X][j] = fmaf(Dx, dp, t.c[PHK_X][j]);
                t.c[PHK_Y][j] = fmaf(Dy, dp, t.c[PHK_Y][j]);
            }
        }
    }
}

template <int VEC>
__device__ __forceinline__ void op_linear_long(const phk_op& op,
                                               Tile<float, VEC>& t) {
    // p: cos (hi, lo), longfac*sin (hi, lo), D_x, D_y, sin/longfac (hi, lo)
    const float* p = reinterpret_cast<const float*>(op.p);
    const float cs = p[0], csl = p[1], a = p[2], al = p[3];
    const float b = p[6], bl = p[7];
    const float Dx = p[4], Dy = p[5];
    const bool disp = op.flags & PHK_FLAG_DISPERSION;
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
        float& z = t.c[PHK_Z][j];
        float& dp = t.c[PHK_DP][j];
        if (disp) {
            t.c[PHK_X][j] = fmaf(-Dx, dp, t.c[PHK_X][j]);
            t.c[PHK_Y][j] = fmaf(-Dy, dp, t.c[PHK_Y][j]);
        }
        const float z0 = z, dp0 = dp;
        z = fmaf(z0, cs, fmaf(-a, dp0, fmaf(z0, csl, -al * dp0)));
        dp = fmaf(dp0, cs, fmaf(b, z0, fmaf(dp0, csl, bl * z0)));
        if (disp) {
            t.c[PHK_X][j] = fmaf(Dx, dp, t.c[PHK_X][j]);
            t.c[PHK_Y][j] = fmaf(Dy, dp, t.c[PHK_Y][j]);
        }
    }
}

template <int VEC>
__device__ __forceinline__ void op_scale(const phk_op& op,
                                         Tile<float, VEC>& t) {
    const float f = reinterpret_cast<const float*>(op.p)[0];
#pragma unroll
    for (int j = 0; j < VEC; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) t.c[q][j] *= f;
}

template <int VEC>
__device__ __forceinline__ void op_damper(const phk_op& op,
                                          Tile<float, VEC>& t) {
    const float* m = reinterpret_cast<const float*>(damper_means(op) + 6);
    const float* f = reinterpret_cast<const float*>(op.p);
    const bool reactive = op.flags & PHK_FLAG_REACTIVE;
#pragma unroll
    for (int pl = 0; pl < 2; ++pl) {
        if (!(op.flags & (pl == 0 ? PHK_FLAG_DAMP_X : PHK_FLAG_DAMP_Y))) continue;
        const int u = pl == 0 ? PHK_X : PHK_Y, up = pl == 0 ? PHK_XP : PHK_YP;
        const float* g = f + 3 * pl;
        const float c1 = g[0] * __ldg(m + up);
        const float c2 = reactive ? __fdiv_rn(g[1] * __ldg(m + u), g[2]) : 0.f;
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            t.c[up][j] -= c1;
            if (reactive) t.c[up][j] -= c2;
        }
    }
}

// one dispatch per op per tile (uniform across the CTA)
template <typename T, int VEC>
__device__ __forceinline__ void run_program(const phk_program& prog,
                                            Tile<T, VEC>& t) {
    for (int o = 0; o < prog.n_ops; ++o) {
        const phk_op& op = prog.op[o];
        switch (op.kind) {
            case PHK_OP_TRANSVERSE: op_transverse<VEC>(op, prog, t); break;
            case PHK_OP_DRIFT: op_drift<VEC>(op, t); break;
            case PHK_OP_RF_KICK: op_rfkick<VEC>(op, t); break;
            case PHK_OP_LINEAR_LONG: op_linear_long<VEC>(op, t); break;
            case PHK_OP_SCALE_TRANS: op_scale<VEC>(op, t); break;
            case PHK_OP_DAMPER: op_damper<VEC>(op, t); break;
            default: break;
        }
    }
}

// Element sequences with a compile-time shape: the op parameters are then
// read at fixed offsets of the kernel's parameter block (constant-bank
// operands) instead of through a per-tile dispatch loop.
enum TrackShape {
    SHAPE_GENERIC = 0,   // any program: run_program's loop
    SHAPE_NONE = 1,      // no ops (slicing / kicks only)
    SHAPE_T = 2,         // one transverse segment
    SHAPE_T_RF = 3,      // transverse, drift, RF kick, drift (RFSystems)
    SHAPE_T_LIN = 4,     // transverse, linear longitudinal map
};

template <typename T, int VEC, int SHAPE>
__device__ __forceinline__ void run_program_shape(const phk_program& prog,
                                                  Tile<T, VEC>& t) {
    if constexpr (SHAPE == SHAPE_NONE) {
        return;
    } else if constexpr (SHAPE == SHAPE_T) {
        op_transverse<VEC, true>(prog.op[0], prog, t);
    } else if constexpr (SHAPE == SHAPE_T_RF) {
        op_transverse<VEC, true>(prog.op[0], prog, t);
        if constexpr (std::is_same<T, double>::value) {
            op_drift_rf<VEC>(prog.op[1], t);
            op_rfkick_rf<VEC>(prog.op[2], t);
            op_drift_rf<VEC>(prog.op[3], t);
        } else {
            op_drift<VEC>(prog.op[1], t);
            op_rfkick<VEC>(prog.op[2], t);
            op_drift<VEC>(prog.op[3], t);
        }
    } else if constexpr (SHAPE == SHAPE_T_LIN) {
        op_transverse<VEC, true>(prog.op[0], prog, t);
        op_linear_long<VEC>(prog.op[1], t);
    } else {
        run_program<T, VEC>(prog, t);
    }
}

// ===================================================================
// per-slice accumulation in shared memory
//
// FP64 form and the batched kernels: each warp owns a private histogram
//   (count, sum x, sum y per slice); lanes of a warp holding the same slice
//   are serialised by bids (warp_accumulate), so a bin is updated in a fixed
//   lane order and the sums do not depend on scheduling.  FP64: plain
//   double sums; FP32 (batched kernel): Kahan (1965) compensated float sums,
//   one (sum, compensation) float2 per bin.  When the per-warp copies do not
//   fit the shared-memory plan, warps share copies through atomics; the
//   order of the warps sharing a copy is then not fixed, so those sums can
//   differ in their last bits between launches (FP64 single bunch: beyond
//   511 slices with two kick tables, 573 without).
//
// FP32 single-bunch kernel: exact fixed-point sums (FixHist below), one
//   histogram per CTA updated with 32-bit integer atomics: integer addition
//   is associative, so the sums are bit-identical whatever the order.
// ===================================================================

template <typename T>
struct Hist;

template <>
struct Hist<double> {
    using Word = double;
    static __device__ __forceinline__ void zero(Word* w) { *w = 0.0; }
    static __device__ __forceinline__ void add(Word* w, double v) {
        *w = ::phk::add(*w, v);
    }
    static __device__ __forceinline__ void add_atomic(Word* w, double v) {
        atomicAdd(w, v);
    }
    static __device__ __forceinline__ void merge(Word* dst, const Word* src) {
        *dst = ::phk::add(*dst, *src);
    }
    static __device__ __forceinline__ double value(const Word* w) { return *w; }
};

template <>
struct Hist<float> {
    using Word = float2;  // x: running sum, y: Kahan compensation
    static __device__ __forceinline__ void zero(Word* w) {
        *w = make_float2(0.f, 0.f);
    }
    static __device__ __forceinline__ void add(Word* w, float v) {
        float2 a = *w;
        const float yk = v - a.y;
        const float tk = a.x + yk;
        a.y = (tk - a.x) - yk;
        a.x = tk;
        *w = a;
    }
    static __device__ __forceinline__ void add_atomic(Word* w, float v) {
        atomicAdd(&w->x, v);
    }
    static __device__ __forceinline__ void merge(Word* dst, const Word* src) {
        const float2 b = *src;
        add(dst, b.x - b.y);
    }
    static __device__ __forceinline__ double value(const Word* w) {
        const float2 a = *w;
        return (double)(a.x - a.y);
    }
};

// All 32 lanes of the warp must call this together; s < 0 means "no bin".
// Lanes of a warp that hold the same slice are serialised by bids: in each
// round every pending lane bids atomicMax(tag[s], epoch << 5 | lane) on the
// warp's private tag array; the standing bid (the highest pending lane of
// that slice) updates the bin with plain loads and stores.  A bin is thus
// always updated in descending lane order: the sums are deterministic.
template <typename T>
__device__ __forceinline__ void warp_accumulate(int s, T vx, T vy,
                                                typename Hist<T>::Word* hx,
                                                typename Hist<T>::Word* hy,
                                                int* hc, int* tag,
                                                unsigned& epoch,
                                                bool shared_hist) {
    if (shared_hist) {
        if (s >= 0) {
            atomicAdd(hc + s, 1);
            Hist<T>::add_atomic(hx + s, vx);
            Hist<T>::add_atomic(hy + s, vy);
        }
        return;
    }
    const int lane = threadIdx.x & 31;
    bool pending = s >= 0;
    while (__any_sync(0xffffffffu, pending)) {
        ++epoch;
        const int bid = (int)((epoch << 5) | (unsigned)lane);
        if (pending) atomicMax(tag + s, bid);
        __syncwarp();
        if (pending && tag[s] == bid) {
            hc[s] += 1;
            Hist<T>::add(hx + s, vx);
            Hist<T>::add(hy + s, vy);
            pending = false;
        }
        __syncwarp();
    }
}

// -------------------------------------------------------------------
// FixHist: exact, order-independent per-slice sums of FP32 coordinates.
//
// Every thread-block cluster agrees on one power-of-two scale per
// coordinate, 2^k with k chosen from the largest finite |u| of the
// cluster's first tiles so that it maps to [2^26, 2^27).  A value
// u becomes the integer v = rint(u 2^k) (u 2^k is exact; the rounding is
// the only approximation, at most 2^-27 of that largest value, the order
// of the FP32 rounding of u itself).  Level A, |u 2^k| < 2^30: v is split into two
// 15-bit digits d0 = v & 0x7fff in [0, 2^15) and d1 = v >> 15 (arithmetic)
// in [-2^15, 2^15), added to 32-bit counters with shared-memory atomics
// (two per coordinate, one for the count: five per particle); 2^16 values
// per counter stay inside the int32 range (a CTA adds its counters to level
// B at least every 2^16 values).  Level B, larger
// finite values (2^30 <= |u 2^k| < 2^40, rare): 64-bit atomics at the same
// scale on the cluster's partial column in global memory, zeroed by the
// cluster's rank 0 before the first add.  Level C: NaN, +-inf and
// |u 2^k| >= 2^40 set flag bits of the slice; the slice's sum then becomes
// NaN (NaN, both infinities, or out of range) or +-inf, as a floating-point
// sum would.  At the end rank 0 adds the digits of its cluster's CTAs and
// the level-B sums as 64-bit integers, converts once to FP64 (x 2^-k) and
// writes the partial column.  Every step is integer arithmetic or a fixed
// sequence of FP64 operations: the result is bit-identical on every launch.
// -------------------------------------------------------------------
constexpr float kFixLevelA = 1073741824.0f;        // 2^30
constexpr float kFixLevelB = 1099511627776.0f;     // 2^40
constexpr int64_t kFixMaxPerCta = (int64_t)1 << 16;  // values per counter

// Levels B and C of one value (rare; kept out of line): v = u 2^k.
static __device__ __noinline__ void fix_add_slow(long long* spill,
                                                 unsigned* flag, int shift,
                                                 float u, float v) {
    if (fabsf(v) < kFixLevelB) {
        atomicAdd(reinterpret_cast<unsigned long long*>(spill),
                  (unsigned long long)__float2ll_rn(v));
        return;
    }
    // 1 NaN, 2 +inf, 4 -inf, 8 finite beyond the 64-bit range
    const unsigned b = isnan(u) ? 1u : (isinf(u) ? (u > 0.f ? 2u : 4u) : 8u);
    atomicOr(flag, b << shift);
}

// level-B columns of a CTA's FixHist (read on the rare slow path only):
// element s of coordinate q at spill[q] + s * stride
struct FixSpill {
    long long* spill[2];
    int64_t stride;
};

struct FixHist {
    int* cnt;             // [S] counts
    int* dig;             // [4][S]: x d0 d1, y d0 d1
    unsigned* flag;       // [(S + 3) / 4]: one byte per slice, x low nibble
    const FixSpill* sp;   // in shared memory
    int S;
    float scale[2];       // 2^k of x and y

    __device__ __forceinline__ void add_q(int q, int s, float u) const {
        const float v = u * scale[q];
        if (fabsf(v) < kFixLevelA) {
            const int iv = __float2int_rn(v);
            int* d = dig + 2 * q * S + s;
            atomicAdd(d, iv & 0x7fff);
            atomicAdd(d + S, iv >> 15);
        } else {
            fix_add_slow(sp->spill[q] + (int64_t)s * sp->stride,
                         flag + (s >> 2), 8 * (s & 3) + 4 * q, u, v);
        }
    }
    __device__ __forceinline__ void add(int s, float x, float y) const {
        atomicAdd(cnt + s, 1);
        add_q(0, s, x);
        add_q(1, s, y);
    }
    // the sum held by the two digit counters at d and d + S
    static __device__ __forceinline__ long long total(const int* d, int S) {
        return (long long)d[0] + ((long long)d[S] << 15);
    }
};

// 2^k, the FixHist scale for the largest finite magnitude m (as float bits;
// 0 when there is none): m 2^k in [2^26, 2^27)
__device__ __forceinline__ float fix_scale(unsigned mbits) {
    int k = 40;                         // no finite non-zero value seen
    if (mbits != 0u && mbits < 0x7f800000u) {
        const int e = (int)(mbits >> 23) - 127;   // denormals: e = -127
        k = 26 - e;
    }
    k = k > 100 ? 100 : (k < -100 ? -100 : k);
    return ldexpf(1.0f, k);
}

// the FP64 value of a slice sum from its 64-bit total and flag nibble
__device__ __forceinline__ double fix_value(long long total, unsigned fl,
                                            float scale) {
    if (fl) {
        if ((fl & 9u) || (fl & 6u) == 6u)
            return __longlong_as_double(0x7ff8000000000000ll);
        return (fl & 2u) ? __longlong_as_double(0x7ff0000000000000ll)
                         : __longlong_as_double((long long)0xfff0000000000000ull);
    }
    return (double)total * (1.0 / (double)scale);
}

// ===================================================================
// the fused track kernel
// ===================================================================

template <typename T, int VEC>
struct VecIO;
template <>
struct VecIO<double, 2> {
    static __device__ __forceinline__ void ld(const double* p, double (&o)[2]) {
        const double2 t = *reinterpret_cast<const double2*>(p);
        o[0] = t.x; o[1] = t.y;
    }
    static __device__ __forceinline__ void st(double* p, const double (&v)[2]) {
        *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
    }
};
template <>
struct VecIO<float, 2> {
    static __device__ __forceinline__ void ld(const float* p, float (&o)[2]) {
        const float2 t = *reinterpret_cast<const float2*>(p);
        o[0] = t.x; o[1] = t.y;
    }
    static __device__ __forceinline__ void st(float* p, const float (&v)[2]) {
        *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
    }
};
template <>
struct VecIO<float, 4> {
    static __device__ __forceinline__ void ld(const float* p, float (&o)[4]) {
        const float4 t = *reinterpret_cast<const float4*>(p);
        o[0] = t.x; o[1] = t.y; o[2] = t.z; o[3] = t.w;
    }
    static __device__ __forceinline__ void st(float* p, const float (&v)[4]) {
        *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
};
template <typename T>
struct VecIO<T, 1> {
    static __device__ __forceinline__ void ld(const T* p, T (&o)[1]) { o[0] = *p; }
    static __device__ __forceinline__ void st(T* p, const T (&v)[1]) { *p = v[0]; }
};

struct TrackArgs {
    void* c[6];
    int64_t n;
    int64_t n_tiles;
    int32_t has_pk;
    int32_t has_acc;
    int32_t load_mask;
    int32_t store_mask;
    int32_t n_hist;      // histogram copies per CTA (1 or warps per CTA)
    int32_t kicks_smem;  // kick tables staged in shared memory
    int32_t cluster;     // CTAs per thread-block cluster (accumulation)
    int32_t stages;      // TMA ring stages (0: plain loads)
    int32_t kick_comb;   // kicks staged as one summed table per target
    int32_t comb_slot[3];  // table of target xp, yp, dp (-1: none)
    uint32_t wait_limit;   // polls of a copy wait before giving up
    int32_t n_tables;      // kick tables staged (summed targets or kicks)
    int32_t reserved;
};

template <typename T>
__device__ __forceinline__ T tadd(T a, T b);
template <>
__device__ __forceinline__ double tadd<double>(double a, double b) { return add(a, b); }
template <>
__device__ __forceinline__ float tadd<float>(float a, float b) { return a + b; }
template <typename T>
__device__ __forceinline__ T tmul(T a, T b);
template <>
__device__ __forceinline__ double tmul<double>(double a, double b) { return mul(a, b); }
template <>
__device__ __forceinline__ float tmul<float>(float a, float b) { return a * b; }

// shared memory layout, in this order (every region 16-byte aligned):
//   histogram: bid-serialised words [3][n_hist][Sa] (sum x, sum y as
//              Hist<T>::Word; count as int in the third region), or with
//              `fix` (FP32 single bunch) the FixHist counters: count [Sa],
//              digits [4][Sa], flag bytes [Sa] (ints)
//   accumulation edges [Sa + 1] T, pending-kick edges [Sp + 1] T,
//   kick tables [n_tables][Sp] T (when staged), bid tags [n_hist][Sa] int
//   (none with `fix`), TMA ring [stages][6][tile] T, one mbarrier per stage
__host__ __device__ inline size_t align16(size_t b) { return (b + 15) & ~size_t(15); }

template <typename T>
__host__ __device__ inline size_t track_smem_layout(int Sa, int Sp, int n_hist,
                                                    int n_tables, int kicks_smem,
                                                    int stages, int tile,
                                                    size_t* off, bool fix = false) {
    size_t b = 0;
    if (fix) {
        off[0] = b; b = align16(b + (size_t)4 * Sa);              // count
        off[1] = b; b = align16(b + (size_t)4 * 4 * Sa);          // digits
        off[2] = b; b = align16(b + (size_t)4 * ((Sa + 3) / 4));  // flags
    } else {
        off[0] = b; b = align16(b + (size_t)8 * n_hist * Sa);   // sum x words
        off[1] = b; b = align16(b + (size_t)8 * n_hist * Sa);   // sum y words
        off[2] = b; b = align16(b + (size_t)4 * n_hist * Sa);   // count
    }
    off[3] = b; b = align16(b + sizeof(T) * (Sa > 0 ? Sa + 1 : 0));
    off[4] = b; b = align16(b + sizeof(T) * (Sp > 0 ? Sp + 1 : 0));
    off[5] = b; b = align16(b + (kicks_smem ? sizeof(T) * (size_t)n_tables * Sp : 0));
    off[6] = b; b = align16(b + (fix ? 0 : (size_t)4 * n_hist * Sa));  // bid tags
    off[7] = b; b = align16(b + (size_t)stages * 6 * tile * sizeof(T));
    off[8] = b; b = align16(b + (size_t)8 * stages);         // mbarriers
    return b;
}

// Exact slice lookup against a staged edge table.  FP32: the float edges
// themselves.  FP64: order-preserving int64 keys of the edges, so that the
// lookup needs no FP64 instruction (the first estimate is FP32).
template <typename T>
__device__ __forceinline__ void stage_edge(T* dst, int i, T e);
template <>
__device__ __forceinline__ void stage_edge<float>(float* dst, int i, float e) {
    dst[i] = e;
}
template <>
__device__ __forceinline__ void stage_edge<double>(double* dst, int i,
                                                   double e) {
    reinterpret_cast<long long*>(dst)[i] = order_key(e);
}

template <typename T>
struct Bins;
template <>
struct Bins<float> {
    const float* e;
    int S, neg;
    float tail, iw, mg;   // tail = e[0]
    // mg bounds |u - u_ref|, u = (zz - e0) * iw the FP32 position in slice
    // units and u_ref the reference's (z - tail) / width of the same z.
    // The table's end edges lie within one FP32 ulp of the real cuts, so
    // with A = |e0| + |eS|: |u - u_ref| <= 2^-23 A iw (the cuts) +
    // 4 * 2^-24 (S + 1) (the four roundings of D = eS - e0, S / D,
    // zz - e0 and the product), plus FP64 roundings of order 2^-52 S.
    // mg takes twice that; a margin of 1/4 slice or more switches the fast
    // path off.
    __device__ __forceinline__ void init(const float* edges, int n, int negate) {
        e = edges; S = n; neg = negate;
        const float e0 = e[0], eS = e[S];
        tail = e0;
        const float span = eS - e0;
        iw = span > 0.f ? (float)S / span : 0.f;
        const float m = 4.76837158203125e-7f *      // 2^-21
                        ((fabsf(e0) + fabsf(eS)) * iw + (float)S + 2.f);
        mg = m < 0.25f ? m : 2.f;
    }
    // The fast path also needs every edge within mg of its uniform
    // position: u(e_k) within mg of k.  Then for u at least mg inside
    // slice k (and u monotone in z), e_k <= z < e_{k+1}.  Tables of
    // uniform-bin slicers pass (the bound above); tables of other slicers
    // (uniform charge) fail and keep the search.  u - k is exact here
    // (Sterbenz) whenever it is small.
    __device__ __forceinline__ bool edges_uniform(int tid, int nthreads) const {
        if (mg >= 1.f) return true;
        bool ok = true;
        for (int i = tid; i <= S; i += nthreads)
            ok = ok && fabsf((e[i] - tail) * iw - (float)i) < mg;
        return ok;
    }
    __device__ __forceinline__ void disable_fast() { mg = 2.f; }
    // Exact slice of VEC particles.  Fast path: when u lies at least mg
    // inside a slice of [0, S), floor(u) is the reference's index.  Only
    // particles within mg of a slice edge (or outside the cuts, or NaN)
    // read the edge table: the estimate and both bracketing edges, then
    // corrections that walk at most to the table ends (e0 <= zz < eS holds
    // inside), so no access leaves e[0..S].
    template <int VEC>
    __device__ __forceinline__ void index_vec(const float (&z)[VEC],
                                              int (&out)[VEC]) const {
        float zz[VEC];
        bool slow = false;
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            zz[j] = neg ? -z[j] : z[j];
            const float u = (zz[j] - tail) * iw;
            const float fl = floorf(u);
            const float fr = u - fl;             // exact
            const int ki = (int)fl;              // saturating, NaN -> 0
            const bool ok = fr >= mg && fr <= 1.f - mg &&
                            (unsigned)ki < (unsigned)S;
            out[j] = ok ? ki : -2;
            slow |= !ok;
        }
        if (!slow) return;
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            if (out[j] != -2) continue;
            if (!(zz[j] >= tail) || !(zz[j] < e[S])) { out[j] = -1; continue; }
            int kk = (int)((zz[j] - tail) * iw);
            kk = kk < 0 ? 0 : (kk > S - 1 ? S - 1 : kk);
            float l = e[kk], h = e[kk + 1];
            while (zz[j] < l) { --kk; h = l; l = e[kk]; }
            while (zz[j] >= h) { ++kk; h = e[kk + 1]; }
            out[j] = kk;
        }
    }
    __device__ __forceinline__ int index(float z) const {
        float zv[1] = {z};
        int o[1];
        index_vec<1>(zv, o);
        return o[0];
    }
};
template <>
struct Bins<double> {
    const long long* k;
    int S, neg;
    float tail, iw;
    long long k0, kS;
    __device__ __forceinline__ void init(const double* edges, int n, int negate) {
        k = reinterpret_cast<const long long*>(edges); S = n; neg = negate;
        k0 = k[0]; kS = k[S];
        // undo the key map for the two end edges (keys of finite doubles)
        const float lo = approx_float(key_to_double(k0));
        const float hi = approx_float(key_to_double(kS));
        tail = lo;
        const float span = hi - lo;
        iw = span > 0.f ? (float)S / span : 0.f;
    }
    template <int VEC>
    __device__ __forceinline__ void index_vec(const double (&z)[VEC],
                                              int (&out)[VEC]) const {
        long long kz[VEC], lo[VEC], hi[VEC];
        int b[VEC];
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            const double zz = neg ? -z[j] : z[j];
            kz[j] = order_key(zz);
            int kk = (int)((approx_float(zz) - tail) * iw);
            b[j] = kk < 0 ? 0 : (kk > S - 1 ? S - 1 : kk);
        }
#pragma unroll
        for (int j = 0; j < VEC; ++j) { lo[j] = k[b[j]]; hi[j] = k[b[j] + 1]; }
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            if (kz[j] < k0 || kz[j] >= kS) { out[j] = -1; continue; }
            int kk = b[j];
            long long l = lo[j], h = hi[j];
            while (kz[j] < l) { --kk; h = l; l = k[kk]; }
            while (kz[j] >= h) { ++kk; h = k[kk + 1]; }
            out[j] = kk;
        }
    }
    __device__ __forceinline__ int index(double z) const {
        double zv[1] = {z};
        int o[1];
        index_vec<1>(zv, o);
        return o[0];
    }
    // no table-free path in the FP64 form
    __device__ __forceinline__ bool edges_uniform(int, int) const { return true; }
    __device__ __forceinline__ void disable_fast() {}
};

// After Bins::init over a staged table: the table-free lookup stays on
// only if every edge passes edges_uniform (a block-wide vote; every
// thread of the block calls this, `active` being the same for all).
template <typename T>
__device__ __forceinline__ void vote_fast_path(Bins<T>& b, bool active,
                                               int tid, int nthreads) {
    const bool ok = !active || b.edges_uniform(tid, nthreads);
    if (!__syncthreads_and(ok) && active) b.disable_fast();
}

// Stages the pending kicks' slice edges (as lookup keys) into `epk` and,
// when a.kicks_smem, their tables into `ktab`: one table per kick, or with
// a.kick_comb one summed table per target (slot a.comb_slot[target]).
// Called by all threads of a CTA; a __syncthreads() must follow.
template <typename T>
__device__ __forceinline__ void stage_pending(const phk_kick_set& pk,
                                              const TrackArgs& a, T* epk,
                                              T* ktab, int tid, int nthreads) {
    const int Sp = pk.slicer.n_slices;
    const int nk = pk.n_kicks;
    const T* e = reinterpret_cast<const T*>(pk.slicer.edges);
    for (int i = tid; i <= Sp; i += nthreads) stage_edge<T>(epk, i, e[i]);
    if (a.kick_comb) {
        for (int i = tid; i < Sp; i += nthreads) {
            T v[3] = {T(0), T(0), T(0)};
            for (int k = 0; k < nk; ++k) {
                const int tg = pk.target[k];
                const int q = tg == PHK_XP ? 0 : (tg == PHK_YP ? 1 : 2);
                v[q] = tadd<T>(v[q], reinterpret_cast<const T*>(pk.kick[k])[i]);
            }
            for (int q = 0; q < 3; ++q)
                if (a.comb_slot[q] >= 0) ktab[a.comb_slot[q] * Sp + i] = v[q];
        }
    } else if (a.kicks_smem) {
        for (int i = tid; i < nk * Sp; i += nthreads) {
            const int k = i / Sp;
            ktab[i] = reinterpret_cast<const T*>(pk.kick[k])[i - k * Sp];
        }
    }
}

// Wake kicks left pending by the previous WakeField.track, applied in
// kick order to the VEC particles of a tile in registers
// (DipoleWakeKickX/Y.apply, impedances/wake_kicks.py:207-260, and the
// quadrupolar / constant kicks :185-202, :284-361).  `ktab` holds the
// staged tables (stage_pending); particles outside the cuts or past the
// end are left alone.
template <typename T, int VEC, bool FULL>
__device__ __forceinline__ void apply_pending(const phk_kick_set& pk,
                                              const TrackArgs& a,
                                              const Bins<T>& bpk,
                                              const T* ktab, Tile<T, VEC>& t,
                                              int64_t i0) {
    const int Sp = pk.slicer.n_slices;
    const int nk = pk.n_kicks;
    int sl[VEC];
    bpk.index_vec(t.c[PHK_Z], sl);
    if (a.kick_comb) {
        // FP32 form, dipolar kicks only: one table per target, the
        // kicks of that target summed at staging
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            const bool on = sl[j] >= 0 && (FULL || i0 + j < a.n);
            const int s = on ? sl[j] : 0;
            if (a.comb_slot[0] >= 0)
                t.c[PHK_XP][j] = tadd<T>(t.c[PHK_XP][j], on ? ktab[a.comb_slot[0] * Sp + s] : T(0));
            if (a.comb_slot[1] >= 0)
                t.c[PHK_YP][j] = tadd<T>(t.c[PHK_YP][j], on ? ktab[a.comb_slot[1] * Sp + s] : T(0));
            if (a.comb_slot[2] >= 0)
                t.c[PHK_DP][j] = tadd<T>(t.c[PHK_DP][j], on ? ktab[a.comb_slot[2] * Sp + s] : T(0));
        }
    } else {
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            const int s = sl[j];
            if (s < 0 || (!FULL && i0 + j >= a.n)) continue;
            const T kx = t.c[PHK_X][j], ky = t.c[PHK_Y][j];
            for (int k = 0; k < nk; ++k) {
                T val = a.kicks_smem
                            ? ktab[k * Sp + s]
                            : __ldg(reinterpret_cast<const T*>(pk.kick[k]) + s);
                const int qd = pk.quad[k];
                if (qd == PHK_X) val = tmul<T>(val, kx);
                else if (qd == PHK_Y) val = tmul<T>(val, ky);
                const int tg = pk.target[k];
                if (tg == PHK_XP) t.c[PHK_XP][j] = tadd<T>(t.c[PHK_XP][j], val);
                else if (tg == PHK_YP) t.c[PHK_YP][j] = tadd<T>(t.c[PHK_YP][j], val);
                else t.c[PHK_DP][j] = tadd<T>(t.c[PHK_DP][j], val);
            }
        }
    }
}

// Per-CTA state shared by the tile loops of the track kernel.
template <typename T, int VEC>
struct TrackCtx {
    using W = typename Hist<T>::Word;
    T* cp[6];
    Bins<T> bpk, bac;
    const T* ktab;
    W* hx;
    W* hy;
    int* hc;
    int* tag;
    unsigned epoch;
    bool shared_hist;
    FixHist fix;          // FP32 single-bunch accumulation
};

// One tile of VEC particles per thread, already in registers: pending
// kicks, element program, slice accumulation; then the stores.  All threads
// of the CTA call this together (the accumulation is warp-synchronous);
// lanes whose particles are past the end pass live = false.
template <typename T, int VEC, int SHAPE, bool FULL, bool FIX = false>
__device__ __forceinline__ void run_tile(const phk_program& prog,
                                         const phk_kick_set& pk,
                                         const phk_accum& acc,
                                         const TrackArgs& a,
                                         TrackCtx<T, VEC>& cx, Tile<T, VEC>& t,
                                         int64_t i0, bool full) {
    // 1. wake kicks of the previous WakeField.track, in kick order
    if (a.has_pk) apply_pending<T, VEC, FULL>(pk, a, cx.bpk, cx.ktab, t, i0);
    // 2. element program
    run_program_shape<T, VEC, SHAPE>(prog, t);
    // 3. slice accumulation
    if (a.has_acc) {
        int sl[VEC];
        cx.bac.index_vec(t.c[PHK_Z], sl);
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            const bool live = FULL || i0 + j < a.n;
            const int s = live ? sl[j] : -1;
            if (acc.idx_out && live)
                acc.idx_out[i0 + j] =
                    s >= 0 ? s
                           : outside_index((double)t.c[PHK_Z][j],
                                           acc.slicer.tail, acc.slicer.width);
            if constexpr (FIX) {
                if (s >= 0) cx.fix.add(s, (float)t.c[PHK_X][j], (float)t.c[PHK_Y][j]);
            } else {
                warp_accumulate<T>(s, t.c[PHK_X][j], t.c[PHK_Y][j], cx.hx, cx.hy,
                                   cx.hc, cx.tag, cx.epoch, cx.shared_hist);
            }
        }
    }
    // 4. stores of the coordinates the tile changed
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        if (!((a.store_mask >> q) & 1)) continue;
        if (FULL || full) {
            VecIO<T, VEC>::st(cx.cp[q] + i0, t.c[q]);
        } else {
#pragma unroll
            for (int j = 0; j < VEC; ++j)
                if (i0 + j < a.n) cx.cp[q][i0 + j] = t.c[q][j];
        }
    }
}

template <typename T, int VEC>
__device__ __forceinline__ void load_tile_plain(const TrackArgs& a,
                                                const TrackCtx<T, VEC>& cx,
                                                Tile<T, VEC>& t, int64_t i0,
                                                bool full) {
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        if (!((a.load_mask >> q) & 1)) {
#pragma unroll
            for (int j = 0; j < VEC; ++j) t.c[q][j] = T(0);
            continue;
        }
        if (full) {
            VecIO<T, VEC>::ld(cx.cp[q] + i0, t.c[q]);
        } else {
#pragma unroll
            for (int j = 0; j < VEC; ++j)
                t.c[q][j] = (i0 + j < a.n) ? cx.cp[q][i0 + j] : T(0);
        }
    }
}

// CTAs per thread-block cluster of an accumulating launch
constexpr int kCluster = 4;

// FP32 single-bunch kernel: particles per thread, resident CTAs per SM it
// is compiled for (register cap) and the shared memory a CTA may plan for
constexpr int kF32Vec = 2;
constexpr int kF32MinBlocks = 4;
constexpr size_t kF32SmemBudget = 56 * 1024;
// shared memory a CTA may use at three CTAs per SM
constexpr size_t kF32SmemBudget3 = 75 * 1024;
constexpr size_t kF64SmemBudget = 112 * 1024;

// polls of one mbarrier phase before a kernel gives up (order of a second)
constexpr unsigned kWaitLimit = 1u << 22;
// stages of the TMA ring at most
constexpr int kMaxStages = 4;

// FixHist counters are added to the level-B column after this many tiles
// of a CTA (kFixMaxPerCta values per counter at most)
template <int TILE>
constexpr int64_t fix_flush_tiles() { return kFixMaxPerCta / TILE; }

// Adds the FixHist digits of this CTA to the level-B column and clears them
// (all threads, between two barriers).
__device__ __forceinline__ void fix_flush(const FixHist& f, int tid,
                                          int nthreads) {
    for (int s = tid; s < f.S; s += nthreads) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            int* d = f.dig + 2 * q * f.S + s;
            const long long t = FixHist::total(d, f.S);
            if (t != 0)
                atomicAdd(reinterpret_cast<unsigned long long*>(
                              f.sp->spill[q] + (int64_t)s * f.sp->stride),
                          (unsigned long long)t);
            d[0] = 0; d[f.S] = 0;
        }
    }
}

// FP32 launches aim at four resident CTAs per SM (<= 64 registers), FP64
// ones at two (<= 128 registers; the FP64 pipe needs the warps to hide
// its latency)
template <typename T, int VEC, int SHAPE>
__global__ void __launch_bounds__(kTrackThreads, sizeof(T) == 4 ? kF32MinBlocks : 2)
track_kernel(const __grid_constant__ phk_program prog,
             const __grid_constant__ phk_kick_set pk,
             const __grid_constant__ phk_accum acc, const TrackArgs a) {
    using W = typename Hist<T>::Word;
    // FP32: exact fixed-point slice sums (FixHist); FP64: bid-serialised
    // per-warp histograms
    constexpr bool FIX = std::is_same<T, float>::value;
    namespace cg = cooperative_groups;
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int TILE = kTrackThreads * VEC;
    const int Sa = a.has_acc ? acc.slicer.n_slices : 0;
    const int Sp = a.has_pk ? pk.slicer.n_slices : 0;
    size_t off[9];
    track_smem_layout<T>(Sa, Sp, a.n_hist, a.n_tables, a.kicks_smem, a.stages,
                         TILE, off, FIX);
    W* hsx = reinterpret_cast<W*>(smem + off[0]);
    W* hsy = reinterpret_cast<W*>(smem + off[1]);
    int* hcnt = reinterpret_cast<int*>(smem + (FIX ? off[0] : off[2]));
    int* fdig = reinterpret_cast<int*>(smem + off[1]);
    unsigned* fflag = reinterpret_cast<unsigned*>(smem + off[2]);
    T* eacc = reinterpret_cast<T*>(smem + off[3]);
    T* epk = reinterpret_cast<T*>(smem + off[4]);
    T* ktab = reinterpret_cast<T*>(smem + off[5]);
    int* htag = reinterpret_cast<int*>(smem + off[6]);
    T* ring = reinterpret_cast<T*>(smem + off[7]);
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem + off[8]);
    __shared__ unsigned s_max[2];   // FixHist: largest finite |x|, |y| bits
    __shared__ FixSpill s_spill;
    // TMA ring: warps that finished each stage, the last tile issued into
    // each stage (-1: none), a wait that gave up somewhere in the CTA
    __shared__ int s_rel[kMaxStages], s_last[kMaxStages], s_abort;

    const int tid = threadIdx.x;
    const int64_t full_tiles = a.n / TILE;
    const int64_t mine = (a.stages > 0 && blockIdx.x < full_tiles)
                             ? (full_tiles - blockIdx.x + gridDim.x - 1) / gridDim.x
                             : 0;
    const bool has_partial = a.stages > 0 && a.n % TILE != 0 &&
                             blockIdx.x == (int)(full_tiles % gridDim.x);
    int nq = 0;
    for (int q = 0; q < 6; ++q) nq += (a.load_mask >> q) & 1;
    const unsigned stage_bytes = (unsigned)(nq * TILE * sizeof(T));
    // bulk copies of this CTA's k-th tile into stage st (one thread)
    auto issue = [&](int64_t k, int st) {
        const int64_t tile = blockIdx.x + k * gridDim.x;
        fence_proxy_async_smem();
        mbar_expect_tx(bars + st, stage_bytes);
        for (int q = 0; q < 6; ++q)
            if ((a.load_mask >> q) & 1)
                bulk_g2s(ring + ((size_t)st * 6 + q) * TILE,
                         reinterpret_cast<T*>(a.c[q]) + tile * TILE,
                         TILE * sizeof(T), bars + st);
        s_last[st] = (int)k;
    };
    if (tid == 0) {
        s_max[0] = s_max[1] = 0u;
        s_abort = 0;
        for (int st = 0; st < kMaxStages; ++st) s_rel[st] = 0, s_last[st] = -1;
        for (int st = 0; st < a.stages; ++st) mbar_init(bars + st, 1);
        if (a.stages > 0) {
            mbar_fence_init();
            // the first tiles are on their way while the CTA stages its
            // tables (the ring has shared memory of its own)
            for (int64_t k = 0; k < mine && k < a.stages; ++k) issue(k, (int)k);
        }
    }
    if (a.has_acc) {
        const T* e = reinterpret_cast<const T*>(acc.slicer.edges);
        for (int i = tid; i <= Sa; i += blockDim.x) stage_edge<T>(eacc, i, e[i]);
        if constexpr (FIX) {
            for (int i = tid; i < Sa; i += blockDim.x) hcnt[i] = 0;
            for (int i = tid; i < 4 * Sa; i += blockDim.x) fdig[i] = 0;
            for (int i = tid; i < (Sa + 3) / 4; i += blockDim.x) fflag[i] = 0u;
        } else {
            for (int i = tid; i < a.n_hist * Sa; i += blockDim.x) {
                Hist<T>::zero(hsx + i); Hist<T>::zero(hsy + i);
                hcnt[i] = 0; htag[i] = 0;
            }
        }
    }
    if (a.has_pk) stage_pending<T>(pk, a, epk, ktab, tid, blockDim.x);
    __syncthreads();

    TrackCtx<T, VEC> cx;
#pragma unroll
    for (int q = 0; q < 6; ++q) cx.cp[q] = reinterpret_cast<T*>(a.c[q]);
    if (a.has_pk) cx.bpk.init(epk, Sp, pk.slicer.negate);
    if (a.has_acc) cx.bac.init(eacc, Sa, acc.slicer.negate);
    vote_fast_path<T>(cx.bpk, a.has_pk, tid, blockDim.x);
    vote_fast_path<T>(cx.bac, a.has_acc, tid, blockDim.x);
    cx.ktab = ktab;
    const int h = (a.n_hist > 1) ? (tid >> 5) % a.n_hist : 0;
    cx.hx = hsx + h * Sa;
    cx.hy = hsy + h * Sa;
    cx.hc = hcnt + h * Sa;
    cx.tag = htag + h * Sa;
    cx.epoch = 0;
    cx.shared_hist = a.n_hist < (int)(blockDim.x >> 5);

    // partial column of this CTA's cluster
    const bool clustered = a.has_acc && a.cluster > 1;
    const unsigned crank = clustered ? cg::this_cluster().block_rank() : 0u;
    const int column = clustered ? (int)(blockIdx.x / a.cluster) : (int)blockIdx.x;
    const int G = acc.grid;
    double* P = acc.partials;

    bool bad = false;   // a bounded copy wait of this thread gave up

    if constexpr (FIX) {
        if (a.has_acc) {
            // ---- the cluster's scale: largest finite |x|, |y| of the inputs
            // of every member's first tile (the maps change them by factors
            // of order one; larger values take level B)
            unsigned m[2] = {0u, 0u};
            auto see = [&](float u, int q) {
                const unsigned b = __float_as_uint(u) & 0x7fffffffu;
                if (b < 0x7f800000u && b > m[q]) m[q] = b;
            };
            if (mine > 0) {
                bad = !mbar_wait(bars, 0u, a.wait_limit);
                if (!bad) {
                    const T* src = ring + tid * VEC;
#pragma unroll
                    for (int j = 0; j < VEC; ++j) {
                        see(src[(size_t)PHK_X * TILE + j], 0);
                        see(src[(size_t)PHK_Y * TILE + j], 1);
                    }
                }
            } else {
                const int64_t i0 = (a.stages > 0 ? full_tiles * TILE
                                                 : (int64_t)blockIdx.x * TILE) +
                                   tid * VEC;
                if (a.stages == 0 || has_partial) {
#pragma unroll
                    for (int j = 0; j < VEC; ++j) {
                        if (i0 + j < a.n) {
                            see(cx.cp[PHK_X][i0 + j], 0);
                            see(cx.cp[PHK_Y][i0 + j], 1);
                        }
                    }
                }
            }
            m[0] = __reduce_max_sync(0xffffffffu, m[0]);
            m[1] = __reduce_max_sync(0xffffffffu, m[1]);
            if ((tid & 31) == 0) {
                atomicMax(&s_max[0], m[0]);
                atomicMax(&s_max[1], m[1]);
            }
            if (tid == 0) {
                s_spill.spill[0] = reinterpret_cast<long long*>(P) + (int64_t)Sa * G + column;
                s_spill.spill[1] = reinterpret_cast<long long*>(P) + (int64_t)2 * Sa * G + column;
                s_spill.stride = G;
            }
            // rank 0 clears its column's level-B sums before any member adds
            if (crank == 0) {
                for (int s = tid; s < Sa; s += blockDim.x) {
                    reinterpret_cast<long long*>(P)[(int64_t)(Sa + s) * G + column] = 0;
                    reinterpret_cast<long long*>(P)[(int64_t)(2 * Sa + s) * G + column] = 0;
                }
            }
            unsigned M[2];
            if (clustered) {
                __threadfence();
                cg::cluster_group cl = cg::this_cluster();
                cl.sync();
                M[0] = M[1] = 0u;
                for (unsigned r = 0; r < cl.num_blocks(); ++r) {
                    const unsigned* sm = cl.map_shared_rank(s_max, r);
                    M[0] = max(M[0], sm[0]);
                    M[1] = max(M[1], sm[1]);
                }
            } else {
                __syncthreads();
                M[0] = s_max[0];
                M[1] = s_max[1];
            }
            cx.fix.cnt = hcnt;
            cx.fix.dig = fdig;
            cx.fix.flag = fflag;
            cx.fix.sp = &s_spill;
            cx.fix.S = Sa;
            cx.fix.scale[0] = fix_scale(M[0]);
            cx.fix.scale[1] = fix_scale(M[1]);
        }
    }

    if (a.stages > 0) {
        // ---- full tiles through a TMA ring of `stages` stages.  Warps run
        // decoupled: each waits for a stage's copies, processes its part of
        // the tile and releases the stage; the warp whose release completes
        // the stage issues the copies of the tile `stages` ahead into it.
        // A wait that gives up marks the CTA aborted: no more copies are
        // issued, the remaining tiles are skipped (every warp still takes
        // part in the same barriers), and the copies in flight are drained.
        const int nwarps = (int)(blockDim.x >> 5);
        const int lane = tid & 31;
        volatile int* abort_flag = &s_abort;
        int st = 0;
        unsigned ph = 0u;
        for (int64_t k = 0; k < mine; ++k) {
            bool ok = false;
            if (!bad && !*abort_flag) {
                ok = mbar_wait(bars + st, ph, a.wait_limit);
                if (!ok) {
                    bad = true;
                    *abort_flag = 1;
                }
            }
            if (ok) {
                Tile<T, VEC> t;
                const T* src = ring + (size_t)st * 6 * TILE + tid * VEC;
#pragma unroll
                for (int q = 0; q < 6; ++q) {
                    if ((a.load_mask >> q) & 1) {
                        VecIO<T, VEC>::ld(src + (size_t)q * TILE, t.c[q]);
                    } else {
#pragma unroll
                        for (int j = 0; j < VEC; ++j) t.c[q][j] = T(0);
                    }
                }
                const int64_t i0 = (blockIdx.x + k * gridDim.x) * TILE + tid * VEC;
                run_tile<T, VEC, SHAPE, true, FIX>(prog, pk, acc, a, cx, t, i0, true);
            }
            __syncwarp();                    // this warp's part of stage st read
            if (lane == 0) {
                __threadfence_block();
                if (atomicAdd(&s_rel[st], 1) == nwarps - 1) {
                    s_rel[st] = 0;
                    if (k + a.stages < mine && !*abort_flag) issue(k + a.stages, st);
                }
            }
            if (++st == a.stages) {
                st = 0;
                ph ^= 1u;
            }
            if constexpr (FIX) {
                if (a.has_acc && (k + 1) % fix_flush_tiles<TILE>() == 0) {
                    __syncthreads();
                    fix_flush(cx.fix, tid, blockDim.x);
                    __syncthreads();
                }
            }
        }
        __syncthreads();
        if (s_abort) {
            // report, then wait (bounded) for the last copies issued into
            // each stage so that none lands in shared memory after the CTA
            // has exited (earlier ones completed before their stage was
            // released)
            if (tid == 0) {
                bool drained = true;
                for (int q = 0; q < a.stages; ++q)
                    if (s_last[q] >= 0 &&
                        !mbar_wait(bars + q, (unsigned)((s_last[q] / a.stages) & 1),
                                   kWaitLimit))
                        drained = false;
                if (prog.status)
                    atomicMax(prog.status, drained ? PHK_DEV_TIMEOUT
                                                   : PHK_DEV_TIMEOUT_UNDRAINED);
            }
            __syncthreads();
        } else if (has_partial) {
            // ---- the partial last tile, plain loads
            const int64_t i0 = full_tiles * TILE + tid * VEC;
            const bool full = i0 + VEC <= a.n;
            Tile<T, VEC> t;
            load_tile_plain<T, VEC>(a, cx, t, i0, full);
            run_tile<T, VEC, SHAPE, false, FIX>(prog, pk, acc, a, cx, t, i0, full);
        }
    } else {
        // ---- plain loads; every warp runs whole tiles (lanes past the end
        // carry dead particles) so the warp-level accumulation sees 32 lanes
        const int64_t n_tiles_grid = (a.n_tiles + gridDim.x - 1) / gridDim.x;
        for (int64_t it = 0; it < n_tiles_grid; ++it) {
            const int64_t tile = blockIdx.x + it * gridDim.x;
            const int64_t i0 = (tile * blockDim.x + tid) * VEC;
            const bool full = i0 + VEC <= a.n;
            Tile<T, VEC> t;
            load_tile_plain<T, VEC>(a, cx, t, i0, full);
            run_tile<T, VEC, SHAPE, false, FIX>(prog, pk, acc, a, cx, t, i0, full);
            if constexpr (FIX) {
                if (a.has_acc && (it + 1) % fix_flush_tiles<TILE>() == 0) {
                    __syncthreads();
                    fix_flush(cx.fix, tid, blockDim.x);
                    __syncthreads();
                }
            }
        }
    }

    if (!a.has_acc) return;
    if constexpr (FIX) {
        // ---- rank 0 adds its cluster's counters and level-B sums as 64-bit
        // integers and writes the partial column in FP64
        unsigned nb = 1;
        if (clustered) {
            __threadfence();                 // level-B adds before the barrier
            cg::cluster_group cl = cg::this_cluster();
            cl.sync();
            nb = cl.num_blocks();
        } else {
            __syncthreads();
        }
        if (crank == 0) {
            const long long* lp = reinterpret_cast<const long long*>(P);
            for (int s = tid; s < Sa; s += blockDim.x) {
                long long c = 0, tq[2];
                unsigned fl = 0;
                tq[0] = __ldcg(lp + (int64_t)(Sa + s) * G + column);
                tq[1] = __ldcg(lp + (int64_t)(2 * Sa + s) * G + column);
                // unrolled over the cluster's members, so that the loads of
                // every member are in flight together
#pragma unroll
                for (int r = 0; r < kCluster; ++r) {
                    if (r >= (int)nb) break;
                    const int* rc = hcnt;
                    const int* rd = fdig;
                    const unsigned* rf = fflag;
                    if (clustered) {
                        cg::cluster_group cl = cg::this_cluster();
                        rc = cl.map_shared_rank(hcnt, r);
                        rd = cl.map_shared_rank(fdig, r);
                        rf = cl.map_shared_rank(fflag, r);
                    }
                    c += rc[s];
                    fl |= (rf[s >> 2] >> (8 * (s & 3))) & 0xffu;
#pragma unroll
                    for (int q = 0; q < 2; ++q)
                        tq[q] += FixHist::total(rd + 2 * q * Sa + s, Sa);
                }
                P[(int64_t)s * G + column] = (double)c;
                P[(int64_t)(Sa + s) * G + column] =
                    fix_value(tq[0], fl & 15u, cx.fix.scale[0]);
                P[(int64_t)(2 * Sa + s) * G + column] =
                    fix_value(tq[1], fl >> 4, cx.fix.scale[1]);
            }
        }
        if (clustered) cg::this_cluster().sync();  // members keep their counters until read
        return;
    } else {
        __syncthreads();
        // fold the per-warp copies into copy 0 (fixed order)
        for (int s = tid; s < Sa; s += blockDim.x) {
            int c = hcnt[s];
            for (int k = 1; k < a.n_hist; ++k) {
                c += hcnt[k * Sa + s];
                Hist<T>::merge(hsx + s, hsx + k * Sa + s);
                Hist<T>::merge(hsy + s, hsy + k * Sa + s);
            }
            hcnt[s] = c;
        }
        if (clustered) {
            // fold the CTAs of the thread-block cluster into its rank 0
            // through distributed shared memory
            cg::cluster_group cl = cg::this_cluster();
            cl.sync();
            if (crank == 0) {
                for (int s = tid; s < Sa; s += blockDim.x) {
                    int c = hcnt[s];
                    for (unsigned r = 1; r < cl.num_blocks(); ++r) {
                        c += *cl.map_shared_rank(hcnt + s, r);
                        Hist<T>::merge(hsx + s, cl.map_shared_rank(hsx + s, r));
                        Hist<T>::merge(hsy + s, cl.map_shared_rank(hsy + s, r));
                    }
                    hcnt[s] = c;
                }
            }
            cl.sync();  // members keep their shared memory until read
            if (crank != 0) return;
        } else {
            __syncthreads();
        }
        for (int s = tid; s < Sa; s += blockDim.x) {
            P[(int64_t)s * G + column] = (double)hcnt[s];
            P[(int64_t)(Sa + s) * G + column] = Hist<T>::value(hsx + s);
            P[(int64_t)(2 * Sa + s) * G + column] = Hist<T>::value(hsy + s);
        }
    }
}

// ===================================================================
// launch configuration
// ===================================================================

// Shared-memory plan of a launch: histogram copies (FP64: one private copy
// per warp when they fit, else fewer copies shared with atomics; FP32: the
// one FixHist of the CTA) and TMA ring stages (FP32 aligned launches),
// chosen so that the occupancy the kernel is compiled for is reached
// whenever possible.  n_tables: kick tables staged per CTA.
template <typename T>
static size_t smem_for(int Sa, int Sp, int n_tables, bool tma, int* n_hist,
                       int* kicks_smem, int* stages, size_t budget_in = 0,
                       int forced_stages = -1) {
    constexpr bool fix = sizeof(T) == 4;
    const int warps = kTrackThreads / 32;
    const int tile = kTrackThreads * (sizeof(T) == 8 ? 2 : kF32Vec);
    const size_t budget = budget_in ? budget_in
                                    : (sizeof(T) == 8 ? kF64SmemBudget : kF32SmemBudget);
    *kicks_smem = n_tables > 0 && (size_t)n_tables * Sp * sizeof(T) <= 48 * 1024;
    const int hist_opts[4] = {warps, 4, 2, 1};
    const int n_hist_opts = fix ? 1 : 4;
    // ring stages by default: two (measured fastest at 500 slices; more
    // stages take a launch plan), else plain loads (large slice counts)
    const int stage_opts[2] = {2, 0};
    size_t off[9];
    if (tma && (forced_stages == 0 || (forced_stages >= 2 && forced_stages <= kMaxStages))) {
        const int nh = 1;
        const size_t b = track_smem_layout<T>(Sa, Sp, nh, n_tables, *kicks_smem,
                                              forced_stages, tile, off, fix);
        if (fix && b <= budget) {
            *n_hist = nh;
            *stages = forced_stages;
            return b;
        }
    }
    if (fix && tma && budget_in == 0 && forced_stages < 0) {
        // FP32 default: two ring stages at four CTAs per SM; where they do
        // not fit (about 700 slices and more), two stages at three CTAs
        // per SM, measured faster than plain loads at 1000 slices
        const size_t budgets[2] = {kF32SmemBudget, kF32SmemBudget3};
        for (int bi = 0; bi < 2; ++bi) {
            const size_t b = track_smem_layout<T>(Sa, Sp, 1, n_tables, *kicks_smem,
                                                  2, tile, off, fix);
            if (b <= budgets[bi]) {
                *n_hist = 1;
                *stages = 2;
                return b;
            }
        }
    }
    size_t smallest = 0;
    for (int hi = 0; hi < n_hist_opts; ++hi) {
        for (int si = 0; si < (tma ? 2 : 1); ++si) {
            const int nh = (Sa > 0 && !fix) ? hist_opts[hi] : 1;
            const int st = tma ? stage_opts[si] : 0;
            const size_t b = track_smem_layout<T>(Sa, Sp, nh, n_tables,
                                                  *kicks_smem, st, tile, off,
                                                  fix);
            if (b <= budget) {
                *n_hist = nh;
                *stages = st;
                return b;
            }
            if (smallest == 0 || b < smallest) {
                // nothing fits the occupancy budget yet: keep the smallest
                // plan (fewer resident CTAs per SM)
                *n_hist = nh;
                *stages = st;
                smallest = b;
            }
        }
    }
    return smallest;
}

// Kick tables a launch stages: with dipolar kicks only, the kicks of one
// target are summed once per slice into one table per target (one rounding
// per slice instead of one per kick and particle; quadrupolar kicks keep
// the per-kick loop).  Sets
// a->kicks_smem, a->kick_comb, a->comb_slot and a->n_tables.
template <typename T>
static void plan_kick_tables(const phk_kick_set* pk, TrackArgs* a) {
    a->kick_comb = 0;
    a->comb_slot[0] = a->comb_slot[1] = a->comb_slot[2] = -1;
    a->n_tables = 0;
    a->kicks_smem = 0;
    if (!pk) return;
    const int nk = pk->n_kicks, Sp = pk->slicer.n_slices;
    bool dip = true;
    for (int k = 0; k < nk; ++k) dip = dip && pk->quad[k] < 0;
    int slot[3] = {-1, -1, -1}, n = 0;
    if (dip) {
        for (int k = 0; k < nk; ++k) {
            const int tg = pk->target[k];
            const int q = tg == PHK_XP ? 0 : (tg == PHK_YP ? 1 : 2);
            if (slot[q] < 0) slot[q] = n++;
        }
    }
    const int tables = dip ? n : nk;
    a->kicks_smem = tables > 0 && (size_t)tables * Sp * sizeof(T) <= 48 * 1024;
    if (dip && a->kicks_smem) {
        a->kick_comb = 1;
        for (int q = 0; q < 3; ++q) a->comb_slot[q] = slot[q];
        a->n_tables = n;
    } else {
        a->kicks_smem = nk > 0 && (size_t)nk * Sp * sizeof(T) <= 48 * 1024;
        a->n_tables = nk;
    }
}

// Opt the track kernel into the device's full dynamic shared memory, once
// per instantiation and device (never inside a stream capture's hot path).
template <typename T, int VEC, int SHAPE>
static void prepare_track_kernel() {
    static int done_for[64] = {0};
    const DeviceInfo& d = device_info();
    const int dev = d.device < 64 ? d.device : 63;
    if (done_for[dev]) return;
    // dynamic + static shared memory must stay within the opt-in limit
    cudaFuncAttributes fa;
    size_t static_smem = 0;
    if (cudaFuncGetAttributes(&fa, track_kernel<T, VEC, SHAPE>) == cudaSuccess)
        static_smem = fa.sharedSizeBytes;
    else
        cudaGetLastError();
    if (cudaFuncSetAttribute(track_kernel<T, VEC, SHAPE>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             d.max_smem_optin - (int)static_smem) != cudaSuccess)
        cudaGetLastError();
    done_for[dev] = 1;
}

// largest dynamic shared memory a track launch may request
template <typename T, int VEC, int SHAPE>
static size_t track_dynamic_smem_limit() {
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, track_kernel<T, VEC, SHAPE>) != cudaSuccess) {
        cudaGetLastError();
        return (size_t)device_info().max_smem_optin - 1024;
    }
    return (size_t)device_info().max_smem_optin - fa.sharedSizeBytes;
}


template <typename T, int VEC, int SHAPE>
static int occupancy_blocks(size_t smem) {
    int b = 0;
    prepare_track_kernel<T, VEC, SHAPE>();
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &b, track_kernel<T, VEC, SHAPE>, kTrackThreads, smem) != cudaSuccess)
        b = 1;
    return b < 1 ? 1 : b;
}

// clusters of kCluster CTAs that can be resident at once
template <typename T, int VEC, int SHAPE>
static int occupancy_clusters(size_t smem) {
    prepare_track_kernel<T, VEC, SHAPE>();
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kCluster * device_info().sm_count, 1, 1);
    cfg.blockDim = dim3(kTrackThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeClusterDimension;
    attr.val.clusterDim.x = kCluster;
    attr.val.clusterDim.y = 1;
    attr.val.clusterDim.z = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, track_kernel<T, VEC, SHAPE>, &cfg) !=
            cudaSuccess || n < 1) {
        cudaGetLastError();
        n = device_info().sm_count / kCluster;
    }
    return n < 1 ? 1 : n;
}

template <typename T, int VEC, int SHAPE>
static int launch_track_t(const phk_program* prog, const phk_coords* c,
                          const phk_kick_set* pk, const phk_accum* acc,
                          int load_mask, int store_mask, cudaStream_t st) {
    TrackArgs a;
    memset(&a, 0, sizeof(a));
    a.c[0] = c->x; a.c[1] = c->xp; a.c[2] = c->y;
    a.c[3] = c->yp; a.c[4] = c->z; a.c[5] = c->dp;
    a.n = c->n;
    a.has_pk = pk != nullptr;
    a.has_acc = acc != nullptr;
    a.load_mask = load_mask;
    a.store_mask = store_mask;
    a.cluster = 1;
    a.stages = 0;
    a.kick_comb = 0;
    a.comb_slot[0] = a.comb_slot[1] = a.comb_slot[2] = -1;
    a.wait_limit = wait_limit();
    const int64_t per_tile = (int64_t)kTrackThreads * VEC;
    a.n_tiles = (c->n + per_tile - 1) / per_tile;
    static phk_kick_set zero_pk;
    static phk_accum zero_acc;
    const int Sa = acc ? acc->slicer.n_slices : 0;
    const int Sp = pk ? pk->slicer.n_slices : 0;
    // the TMA ring needs 16-byte aligned coordinates (VEC > 1 launches)
    // and pays off for the memory-bound FP32 form
    const bool tma = VEC > 1 && sizeof(T) == 4;
    plan_kick_tables<T>(pk, &a);
    int kicks_smem = 0;
    const TrackPlan pl = track_plan();
    const bool planned = sizeof(T) == 4;
    const size_t smem = smem_for<T>(
        Sa, Sp, a.n_tables, tma, &a.n_hist, &kicks_smem, &a.stages,
        planned && pl.smem_kb > 0 ? (size_t)pl.smem_kb * 1024 : 0,
        planned ? pl.stages : -1);
    if (kicks_smem != a.kicks_smem)
        return set_error(PHK_EPARAM, "phk_track: inconsistent kick-table plan");
    if (smem > track_dynamic_smem_limit<T, VEC, SHAPE>())
        return set_error(PHK_ESIZE, "phk_track: %zu bytes of shared memory "
                         "needed for %d + %d slices", smem, Sa, Sp);
    prepare_track_kernel<T, VEC, SHAPE>();
    cudaError_t e;
    if (acc) {
        // one partial column per cluster of kCluster CTAs
        a.cluster = kCluster;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)acc->grid * kCluster, 1, 1);
        cfg.blockDim = dim3(kTrackThreads, 1, 1);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cudaLaunchAttribute attr;
        attr.id = cudaLaunchAttributeClusterDimension;
        attr.val.clusterDim.x = kCluster;
        attr.val.clusterDim.y = 1;
        attr.val.clusterDim.z = 1;
        cfg.attrs = &attr;
        cfg.numAttrs = 1;
        e = cudaLaunchKernelEx(&cfg, track_kernel<T, VEC, SHAPE>, *prog, pk ? *pk : zero_pk,
                               *acc, a);
    } else {
        const int bps = occupancy_blocks<T, VEC, SHAPE>(smem);
        int64_t g = (int64_t)device_info().sm_count * bps;
        if (a.n_tiles < g) g = a.n_tiles;
        const int grid = (int)(g < 1 ? 1 : g);
        track_kernel<T, VEC, SHAPE><<<grid, kTrackThreads, smem, st>>>(
            *prog, pk ? *pk : zero_pk, zero_acc, a);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess)
        return set_error(PHK_ECUDA, "phk_track launch: %s", cudaGetErrorString(e));
    count_launches(1);
    note_track_launch(0, a.stages, smem);
    return PHK_OK;
}

static inline int op_mask(const phk_program* prog, int* load, int* store) {
    // which coordinates the program reads / writes
    int ld = 0, stm = 0;
    for (int o = 0; o < prog->n_ops; ++o) {
        const phk_op& op = prog->op[o];
        const bool disp = op.flags & PHK_FLAG_DISPERSION;
        switch (op.kind) {
            case PHK_OP_TRANSVERSE:
                ld |= 0x0F | 0x20;  // x xp y yp dp
                stm |= 0x0F;
                break;
            case PHK_OP_DRIFT:
                ld |= 0x30; stm |= 0x10;
                break;
            case PHK_OP_RF_KICK:
            case PHK_OP_LINEAR_LONG:
                ld |= 0x30; stm |= (op.kind == PHK_OP_RF_KICK ? 0x20 : 0x30);
                if (disp) { ld |= 0x05; stm |= 0x05; }
                break;
            case PHK_OP_SCALE_TRANS:
                ld |= 0x0F; stm |= 0x0F;
                break;
            case PHK_OP_DAMPER:
                if (op.flags & PHK_FLAG_DAMP_X) { ld |= 0x03; stm |= 0x02; }
                if (op.flags & PHK_FLAG_DAMP_Y) { ld |= 0x0C; stm |= 0x08; }
                break;
        }
    }
    *load = ld; *store = stm;
    return 0;
}

// ===================================================================
// batched form: many bunches, one persistent launch
// ===================================================================

struct BatchArgs {
    TrackArgs a;             // coordinates, masks, has_pk / has_acc, n_hist
    const phk_unit* units;
    const int32_t* cta_first;
    const phk_program* programs;
    const void* kicks;
    int32_t* status;
    int32_t n_bunches;
    int32_t n_units;
    int32_t n_columns;
};

constexpr size_t kProgSmem = (sizeof(phk_program) + 15) & ~(size_t)15;

// Per CTA: its units in order.  When the bunch changes, the CTA's per-slice
// sums of the previous bunch go to that bunch's partial column, and the new
// bunch's program and kick tables are staged in shared memory.
template <typename T, int VEC, int THREADS, int SHAPE>
__global__ void __launch_bounds__(THREADS, (sizeof(T) == 4 ? 1024 : 512) / THREADS)
batch_track_kernel(const __grid_constant__ phk_kick_set pk,
                   const __grid_constant__ phk_accum acc, const BatchArgs b) {
    using W = typename Hist<T>::Word;
    extern __shared__ __align__(16) unsigned char smem[];
    constexpr int TILE = THREADS * VEC;
    const TrackArgs& a = b.a;
    const int Sa = a.has_acc ? acc.slicer.n_slices : 0;
    const int Sp = a.has_pk ? pk.slicer.n_slices : 0;
    const int nk = a.has_pk ? pk.n_kicks : 0;
    phk_program* sprog = reinterpret_cast<phk_program*>(smem);
    unsigned char* rest = smem + kProgSmem;
    size_t off[9];
    track_smem_layout<T>(Sa, Sp, a.n_hist, nk, 1, 0, TILE, off);
    W* hsx = reinterpret_cast<W*>(rest + off[0]);
    W* hsy = reinterpret_cast<W*>(rest + off[1]);
    int* hcnt = reinterpret_cast<int*>(rest + off[2]);
    T* eacc = reinterpret_cast<T*>(rest + off[3]);
    T* epk = reinterpret_cast<T*>(rest + off[4]);
    T* ktab = reinterpret_cast<T*>(rest + off[5]);
    int* htag = reinterpret_cast<int*>(rest + off[6]);
    const int tid = threadIdx.x;

    if (a.has_acc) {
        const T* e = reinterpret_cast<const T*>(acc.slicer.edges);
        for (int i = tid; i <= Sa; i += THREADS) stage_edge<T>(eacc, i, e[i]);
        for (int i = tid; i < a.n_hist * Sa; i += THREADS) {
            Hist<T>::zero(hsx + i); Hist<T>::zero(hsy + i);
            hcnt[i] = 0; htag[i] = 0;
        }
    }
    if (a.has_pk) {
        const T* e = reinterpret_cast<const T*>(pk.slicer.edges);
        for (int i = tid; i <= Sp; i += THREADS) stage_edge<T>(epk, i, e[i]);
    }

    TrackCtx<T, VEC> cx;
#pragma unroll
    for (int q = 0; q < 6; ++q) cx.cp[q] = reinterpret_cast<T*>(a.c[q]);
    cx.ktab = ktab;
    const int h = (a.n_hist > 1) ? (tid >> 5) % a.n_hist : 0;
    cx.hx = hsx + h * Sa;
    cx.hy = hsy + h * Sa;
    cx.hc = hcnt + h * Sa;
    cx.tag = htag + h * Sa;
    cx.epoch = 0;
    cx.shared_hist = a.n_hist < THREADS / 32;
    __syncthreads();
    if (a.has_pk) cx.bpk.init(epk, Sp, pk.slicer.negate);
    if (a.has_acc) cx.bac.init(eacc, Sa, acc.slicer.negate);
    vote_fast_path<T>(cx.bpk, a.has_pk, tid, blockDim.x);
    vote_fast_path<T>(cx.bac, a.has_acc, tid, blockDim.x);

    int u0 = b.cta_first[blockIdx.x], u1 = b.cta_first[blockIdx.x + 1];
    if (u0 < 0 || u1 > b.n_units || u0 > u1) {
        if (tid == 0 && b.status) atomicMax(b.status, PHK_DEV_BAD_TABLE);
        u0 = u1 = 0;
    }
    int cur = -1, col = -1;
    // write the CTA's sums of the current bunch to its column, then zero
    auto flush = [&]() {
        __syncthreads();
        for (int s = tid; s < Sa; s += THREADS) {
            int c = hcnt[s];
            for (int k = 1; k < a.n_hist; ++k) {
                c += hcnt[k * Sa + s];
                Hist<T>::merge(hsx + s, hsx + k * Sa + s);
                Hist<T>::merge(hsy + s, hsy + k * Sa + s);
            }
            const int G = b.n_columns;
            double* P = acc.partials;
            P[(int64_t)s * G + col] = (double)c;
            P[(int64_t)(Sa + s) * G + col] = Hist<T>::value(hsx + s);
            P[(int64_t)(2 * Sa + s) * G + col] = Hist<T>::value(hsy + s);
        }
        __syncthreads();
        for (int i = tid; i < a.n_hist * Sa; i += THREADS) {
            Hist<T>::zero(hsx + i); Hist<T>::zero(hsy + i);
            hcnt[i] = 0; htag[i] = 0;
        }
    };
    for (int u = u0; u < u1; ++u) {
        const phk_unit U = b.units[u];
        const bool ok = U.bunch >= 0 && U.bunch < b.n_bunches &&
                        U.start >= 0 && U.start <= U.end && U.end <= a.n &&
                        (U.start & 3) == 0 &&
                        (!a.has_acc || (U.column >= 0 && U.column < b.n_columns));
        if (!ok) {
            if (tid == 0 && b.status) atomicMax(b.status, PHK_DEV_BAD_TABLE);
            continue;
        }
        if (U.bunch != cur) {
            if (cur >= 0 && a.has_acc) flush();
            __syncthreads();       // the previous bunch's program is done
            const int4* src = reinterpret_cast<const int4*>(b.programs + U.bunch);
            int4* dst = reinterpret_cast<int4*>(sprog);
            for (int i = tid; i < (int)(sizeof(phk_program) / 16); i += THREADS)
                dst[i] = src[i];
            if (a.has_pk) {
                const T* kt = reinterpret_cast<const T*>(b.kicks) +
                              (int64_t)U.bunch * nk * Sp;
                if (a.kick_comb) {
                    for (int i = tid; i < Sp; i += THREADS) {
                        T v[3] = {T(0), T(0), T(0)};
                        for (int k = 0; k < nk; ++k) {
                            const int tg = pk.target[k];
                            const int q = tg == PHK_XP ? 0 : (tg == PHK_YP ? 1 : 2);
                            v[q] = tadd<T>(v[q], kt[k * Sp + i]);
                        }
                        for (int q = 0; q < 3; ++q)
                            if (a.comb_slot[q] >= 0) ktab[a.comb_slot[q] * Sp + i] = v[q];
                    }
                } else {
                    for (int i = tid; i < nk * Sp; i += THREADS) ktab[i] = kt[i];
                }
            }
            __syncthreads();
            cur = U.bunch;
            col = U.column;
        }
        TrackArgs ua = a;
        ua.n = U.end;
        for (int64_t base = U.start; base < U.end; base += TILE) {
            const int64_t i0 = base + (int64_t)tid * VEC;
            const bool full = i0 + VEC <= U.end;
            Tile<T, VEC> t;
            load_tile_plain<T, VEC>(ua, cx, t, i0, full);
            run_tile<T, VEC, SHAPE, false>(*sprog, pk, acc, ua, cx, t, i0, full);
        }
    }
    if (cur >= 0 && a.has_acc) flush();
}

static_assert(sizeof(phk_program) % 16 == 0, "program copied as int4");

template <typename T>
static size_t batch_smem(int Sa, int Sp, int nk, int threads, int* n_hist) {
    const int tile = threads * (sizeof(T) == 8 ? 2 : kF32Vec);
    size_t off[9];
    const int warps = threads / 32;
    // one private histogram copy per warp when it stays within 48 KB
    int nh = Sa > 0 ? warps : 1;
    size_t bytes = track_smem_layout<T>(Sa, Sp, nh, nk, 1, 0, tile, off);
    if (bytes > 48 * 1024 && Sa > 0) {
        nh = 1;
        bytes = track_smem_layout<T>(Sa, Sp, nh, nk, 1, 0, tile, off);
    }
    *n_hist = nh;
    return kProgSmem + bytes;
}

template <typename T, int VEC, int THREADS, int SHAPE>
static int batch_occupancy(size_t smem) {
    static int done_for[64] = {0};
    const DeviceInfo& d = device_info();
    const int dev = d.device < 64 ? d.device : 63;
    if (!done_for[dev]) {
        cudaFuncAttributes fa;
        size_t st = 0;
        if (cudaFuncGetAttributes(&fa, batch_track_kernel<T, VEC, THREADS, SHAPE>) ==
            cudaSuccess)
            st = fa.sharedSizeBytes;
        else
            cudaGetLastError();
        if (cudaFuncSetAttribute(batch_track_kernel<T, VEC, THREADS, SHAPE>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 d.max_smem_optin - (int)st) != cudaSuccess)
            cudaGetLastError();
        done_for[dev] = 1;
    }
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &nb, batch_track_kernel<T, VEC, THREADS, SHAPE>, THREADS, smem) !=
        cudaSuccess) {
        cudaGetLastError();
        nb = 0;
    }
    return nb;
}

template <typename T, int VEC, int THREADS, int SHAPE>
static int launch_batch_t(const phk_batch* bt, const phk_coords* c,
                          const phk_kick_set* pk, const phk_accum* acc,
                          int ld, int stm, cudaStream_t st) {
    BatchArgs b;
    memset(&b, 0, sizeof(b));
    TrackArgs& a = b.a;
    a.c[0] = c->x; a.c[1] = c->xp; a.c[2] = c->y;
    a.c[3] = c->yp; a.c[4] = c->z; a.c[5] = c->dp;
    a.n = c->n;
    a.has_pk = pk != nullptr;
    a.has_acc = acc != nullptr;
    a.load_mask = ld;
    a.store_mask = stm;
    a.kicks_smem = 1;
    a.comb_slot[0] = a.comb_slot[1] = a.comb_slot[2] = -1;
    if (sizeof(T) == 4 && pk) {
        // FP32 form, dipolar kicks only: one staged table per target
        bool dip = true;
        for (int k = 0; k < pk->n_kicks; ++k) dip = dip && pk->quad[k] < 0;
        if (dip) {
            a.kick_comb = 1;
            int n = 0;
            for (int k = 0; k < pk->n_kicks; ++k) {
                const int tg = pk->target[k];
                const int q = tg == PHK_XP ? 0 : (tg == PHK_YP ? 1 : 2);
                if (a.comb_slot[q] < 0) a.comb_slot[q] = n++;
            }
        }
    }
    a.cluster = 1;
    a.stages = 0;
    const int Sa = acc ? acc->slicer.n_slices : 0;
    const int Sp = pk ? pk->slicer.n_slices : 0;
    const int nk = pk ? pk->n_kicks : 0;
    const size_t smem = batch_smem<T>(Sa, Sp, nk, THREADS, &a.n_hist);
    if (batch_occupancy<T, VEC, THREADS, SHAPE>(smem) < 1)
        return set_error(PHK_ESIZE, "phk_track_batch: %zu bytes of shared "
                         "memory for %d + %d slices do not fit", smem, Sa, Sp);
    b.units = bt->units;
    b.cta_first = bt->cta_first;
    b.programs = bt->programs;
    b.kicks = bt->kicks;
    b.status = bt->status;
    b.n_bunches = bt->n_bunches;
    b.n_units = bt->n_units;
    b.n_columns = bt->n_columns;
    static phk_kick_set zero_pk;
    static phk_accum zero_acc;
    batch_track_kernel<T, VEC, THREADS, SHAPE><<<bt->grid, THREADS, smem, st>>>(
        pk ? *pk : zero_pk, acc ? *acc : zero_acc, b);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(PHK_ECUDA, "phk_track_batch launch: %s",
                         cudaGetErrorString(e));
    count_launches(1);
    return PHK_OK;
}

static inline void track_masks(const phk_program* prog, const phk_kick_set* pk,
                        const phk_accum* acc, int* ld_out, int* stm_out) {
    int ld, stm;
    op_mask(prog, &ld, &stm);
    if (pk) {
        ld |= 1 << PHK_Z;
        for (int k = 0; k < pk->n_kicks; ++k) {
            ld |= 1 << pk->target[k];
            stm |= 1 << pk->target[k];
            if (pk->quad[k] >= 0) ld |= 1 << pk->quad[k];
        }
    }
    if (acc) ld |= (1 << PHK_Z) | (1 << PHK_X) | (1 << PHK_Y);
    ld |= stm;
    *ld_out = ld;
    *stm_out = stm;
}

// ---- per-precision entry points (phk_track_f32.cu / phk_track_f64.cu)
int program_shape(const phk_program* prog);
int launch_track_f32(const phk_program* prog, const phk_coords* c,
                     const phk_kick_set* pk, const phk_accum* acc, int ld,
                     int stm, bool vec_ok, cudaStream_t st);
int launch_track_f64(const phk_program* prog, const phk_coords* c,
                     const phk_kick_set* pk, const phk_accum* acc, int ld,
                     int stm, bool vec_ok, cudaStream_t st);
int track_clusters_f32(size_t smem);
int track_clusters_f64(size_t smem);
int launch_batch_f32(const phk_batch* bt, const phk_coords* c,
                     const phk_kick_set* pk, const phk_accum* acc, int ld,
                     int stm, cudaStream_t st);
int launch_batch_f64(const phk_batch* bt, const phk_coords* c,
                     const phk_kick_set* pk, const phk_accum* acc, int ld,
                     int stm, cudaStream_t st);
int batch_per_sm_f32(int threads, size_t smem);
int batch_per_sm_f64(int threads, size_t smem);

}  // namespace phk
