// Turn kernels of libphk: the fused track kernel (pending wake kick ->
// element program -> slice accumulation), the fixed-order merge of its
// per-CTA partials, the wake convolution and the per-slice moment kernel.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <type_traits>

#include "phk_device.cuh"
#include "phk_internal.h"

namespace phk {

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

__device__ __forceinline__ double amp_action(double c1, double twoa, double b,
                                             double u, double up) {
    // 1/2 * ((1+a^2)/b * u**2 + 2*a * u*up + b * up**2)
    double s = mul(c1, mul(u, u));
    if (twoa != 0.0) s = add(s, mul(mul(twoa, u), up));
    s = add(s, mul(b, mul(up, up)));
    return mul(0.5, s);
}

__device__ __forceinline__ double ij_term(const double* p, int mask, int bi,
                                          int bj, double cc, double ss) {
    const bool hi = (mask >> bi) & 1, hj = (mask >> bj) & 1;
    if (hi && hj) return add(mul(p[bi], cc), mul(p[bj], ss));
    if (hi) return mul(p[bi], cc);
    if (hj) return mul(p[bj], ss);
    return 0.0;
}

__device__ __forceinline__ void op_transverse_f64(const phk_op& op,
                                                  const phk_program& prog,
                                                  double& x, double& xp,
                                                  double& y, double& yp,
                                                  double dp) {
    const double* p = op.p;
    double M00, M01, M10, M11, M22, M23, M32, M33;
    if (op.flags & PHK_FLAG_DETUNED) {
        double phx = p[20], phy = p[21];
        for (int d = 0; d < op.det_count; ++d) {
            const phk_detuner& dt = prog.det[op.det_begin + d];
            if (dt.kind == PHK_DET_CHROMA) {
                phx = add(phx, chroma_poly(dt.c, dt.nx, dt.zx, dp));
                phy = add(phy, chroma_poly(dt.c + 8, dt.ny, dt.zy, dp));
            } else {
                const double* c = dt.c;
                const double Jx = amp_action(c[4], c[5], c[6], x, xp);
                const double Jy = amp_action(c[7], c[8], c[9], y, yp);
                phx = add(phx, dvd(add(mul(c[0], Jx), mul(c[2], Jy)), c[10]));
                phy = add(phy, dvd(add(mul(c[1], Jy), mul(c[3], Jx)), c[10]));
            }
        }
        phx = mul(phx, p[22]);
        phy = mul(phy, p[22]);
        double sx, cx, sy, cy;
        sincos(phx, &sx, &cx);
        sincos(phy, &sy, &cy);
        const int m = op.ij_mask;
        M00 = ij_term(p, m, 0, 8, cx, sx);
        M01 = ij_term(p, m, 1, 9, cx, sx);
        M10 = ij_term(p, m, 2, 10, cx, sx);
        M11 = ij_term(p, m, 3, 11, cx, sx);
        M22 = ij_term(p, m, 4, 12, cy, sy);
        M23 = ij_term(p, m, 5, 13, cy, sy);
        M32 = ij_term(p, m, 6, 14, cy, sy);
        M33 = ij_term(p, m, 7, 15, cy, sy);
    } else {
        M00 = p[0]; M01 = p[1]; M10 = p[2]; M11 = p[3];
        M22 = p[4]; M23 = p[5]; M32 = p[6]; M33 = p[7];
    }
    if (op.flags & PHK_FLAG_DISPERSION) {
        x = sub(x, mul(p[16], dp));
        y = sub(y, mul(p[18], dp));
    }
    const double nx = add(mul(M00, x), mul(M01, xp));
    const double nxp = add(mul(M10, x), mul(M11, xp));
    const double ny = add(mul(M22, y), mul(M23, yp));
    const double nyp = add(mul(M32, y), mul(M33, yp));
    x = nx; xp = nxp; y = ny; yp = nyp;
    if (op.flags & PHK_FLAG_DISPERSION) {
        x = add(x, mul(p[17], dp));
        y = add(y, mul(p[19], dp));
    }
}

__device__ __forceinline__ void op_drift_f64(const phk_op& op, double& z,
                                             double dp) {
    const double* p = op.p;
    const double zz = (op.flags & PHK_FLAG_SHRINK) ? mul(p[0], z) : z;
    z = sub(zz, mul(mul(p[1], dp), p[2]));
}

__device__ __forceinline__ void op_rfkick_f64(const phk_op& op, double& x,
                                              double& y, double z,
                                              double& dp) {
    const double* p = op.p;
    if (op.flags & PHK_FLAG_DISPERSION) {
        x = sub(x, mul(p[9], dp));
        y = sub(y, mul(p[10], dp));
    }
    double phi = mul(p[0], dvd(mul(p[1], z), p[2]));
    if (op.flags & PHK_FLAG_PHI_OFFSET) phi = add(phi, p[3]);
    if (op.flags & PHK_FLAG_PHI_LOCK) phi = add(phi, p[4]);
    double t = mul(p[5], sin(phi));
    if (op.flags & PHK_FLAG_P_INC) t = sub(t, p[7]);
    dp = dvd(add(mul(dp, p[6]), t), p[8]);
    if (op.flags & PHK_FLAG_DISPERSION) {
        x = add(x, mul(p[9], dp));
        y = add(y, mul(p[10], dp));
    }
}

__device__ __forceinline__ void op_linear_long_f64(const phk_op& op,
                                                   double& x, double& y,
                                                   double& z, double& dp) {
    const double* p = op.p;
    if (op.flags & PHK_FLAG_DISPERSION) {
        x = sub(x, mul(p[3], dp));
        y = sub(y, mul(p[4], dp));
    }
    const double z0 = z, dp0 = dp;
    z = sub(mul(z0, p[0]), mul(mul(p[2], dp0), p[1]));
    dp = add(mul(dp0, p[0]), mul(dvd(z0, p[2]), p[1]));
    if (op.flags & PHK_FLAG_DISPERSION) {
        x = add(x, mul(p[3], dp));
        y = add(y, mul(p[4], dp));
    }
}

__device__ __forceinline__ void apply_op(const phk_op& op,
                                         const phk_program& prog, double& x,
                                         double& xp, double& y, double& yp,
                                         double& z, double& dp) {
    switch (op.kind) {
        case PHK_OP_TRANSVERSE: op_transverse_f64(op, prog, x, xp, y, yp, dp); break;
        case PHK_OP_DRIFT: op_drift_f64(op, z, dp); break;
        case PHK_OP_RF_KICK: op_rfkick_f64(op, x, y, z, dp); break;
        case PHK_OP_LINEAR_LONG: op_linear_long_f64(op, x, y, z, dp); break;
        case PHK_OP_SCALE_TRANS: {
            const double f = op.p[0];
            x = mul(x, f); xp = mul(xp, f); y = mul(y, f); yp = mul(yp, f);
            break;
        }
        default: break;
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

__device__ __forceinline__ void op_transverse_f32(const phk_op& op,
                                                  const phk_program& prog,
                                                  float& x, float& xp,
                                                  float& y, float& yp,
                                                  float dp) {
    const float* p = reinterpret_cast<const float*>(op.p);
    float M00, M01, M10, M11, M22, M23, M32, M33;
    if (op.flags & PHK_FLAG_DETUNED) {
        float dqx = 0.f, dqy = 0.f;
        for (int d = 0; d < op.det_count; ++d) {
            const phk_detuner& dt = prog.det[op.det_begin + d];
            const float* c = reinterpret_cast<const float*>(dt.c);
            if (dt.kind == PHK_DET_CHROMA) {
                dqx += chroma_poly_f32(c, dt.nx, dt.zx, dp);
                dqy += chroma_poly_f32(c + 8, dt.ny, dt.zy, dp);
            } else {
                // c = dapp_x/p0, dapp_y/p0, dapp_xy/p0, dapp_yx/p0,
                //     (1+ax^2)/bx, 2ax, bx, (1+ay^2)/by, 2ay, by
                const float Jx = 0.5f * fmaf(c[6] * xp, xp, fmaf(c[5] * x, xp, c[4] * x * x));
                const float Jy = 0.5f * fmaf(c[9] * yp, yp, fmaf(c[8] * y, yp, c[7] * y * y));
                dqx += fmaf(c[0], Jx, c[2] * Jy);
                dqy += fmaf(c[1], Jy, c[3] * Jx);
            }
        }
        float sx, cx, sy, cy;
        sincos_turns(p[16], p[17], dqx, &sx, &cx);
        sincos_turns(p[18], p[19], dqy, &sy, &cy);
        M00 = fmaf(p[0], cx, p[8] * sx);
        M01 = fmaf(p[1], cx, p[9] * sx);
        M10 = fmaf(p[2], cx, p[10] * sx);
        M11 = fmaf(p[3], cx, p[11] * sx);
        M22 = fmaf(p[4], cy, p[12] * sy);
        M23 = fmaf(p[5], cy, p[13] * sy);
        M32 = fmaf(p[6], cy, p[14] * sy);
        M33 = fmaf(p[7], cy, p[15] * sy);
    } else {
        M00 = p[0]; M01 = p[1]; M10 = p[2]; M11 = p[3];
        M22 = p[4]; M23 = p[5]; M32 = p[6]; M33 = p[7];
    }
    if (op.flags & PHK_FLAG_DISPERSION) {
        x = fmaf(-p[32], dp, x);
        y = fmaf(-p[34], dp, y);
    }
    const float nx = fmaf(M00, x, M01 * xp);
    const float nxp = fmaf(M10, x, M11 * xp);
    const float ny = fmaf(M22, y, M23 * yp);
    const float nyp = fmaf(M32, y, M33 * yp);
    x = nx; xp = nxp; y = ny; yp = nyp;
    if (op.flags & PHK_FLAG_DISPERSION) {
        x = fmaf(p[33], dp, x);
        y = fmaf(p[35], dp, y);
    }
}

__device__ __forceinline__ void apply_op(const phk_op& op,
                                         const phk_program& prog, float& x,
                                         float& xp, float& y, float& yp,
                                         float& z, float& dp) {
    const float* p = reinterpret_cast<const float*>(op.p);
    switch (op.kind) {
        case PHK_OP_TRANSVERSE: op_transverse_f32(op, prog, x, xp, y, yp, dp); break;
        case PHK_OP_DRIFT:
            // z = beta_ratio * z - (eta0 * L) * dp
            z = fmaf(-p[1], dp, (op.flags & PHK_FLAG_SHRINK) ? p[0] * z : z);
            break;
        case PHK_OP_RF_KICK: {
            // p: h/C (hi, lo) turns per metre, (phi_offset+phi_lock)/2pi
            // (hi, lo), A/p0_new, p0_old/p0_new, p_inc/p0_new, D_x, D_y
            if (op.flags & PHK_FLAG_DISPERSION) {
                x = fmaf(-p[8], dp, x);
                y = fmaf(-p[9], dp, y);
            }
            const float s = sin_turns_of_product(z, p[0], p[1], p[2], p[3]);
            dp = fmaf(p[4], s, fmaf(dp, p[5], -p[6]));
            if (op.flags & PHK_FLAG_DISPERSION) {
                x = fmaf(p[8], dp, x);
                y = fmaf(p[9], dp, y);
            }
            break;
        }
        case PHK_OP_LINEAR_LONG: {
            // p: cos, sin, longfac, 1/longfac, D_x, D_y
            if (op.flags & PHK_FLAG_DISPERSION) {
                x = fmaf(-p[4], dp, x);
                y = fmaf(-p[5], dp, y);
            }
            const float z0 = z, dp0 = dp;
            z = fmaf(z0, p[0], -(p[2] * dp0) * p[1]);
            dp = fmaf(dp0, p[0], (z0 * p[3]) * p[1]);
            if (op.flags & PHK_FLAG_DISPERSION) {
                x = fmaf(p[4], dp, x);
                y = fmaf(p[5], dp, y);
            }
            break;
        }
        case PHK_OP_SCALE_TRANS: {
            const float f = p[0];
            x *= f; xp *= f; y *= f; yp *= f;
            break;
        }
        default: break;
    }
}

// ===================================================================
// the fused track kernel
// ===================================================================

template <typename T>
struct AccumType { using type = double; };
template <>
struct AccumType<float> { using type = float; };

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
};

__device__ __forceinline__ double tmul(double a, double b) { return mul(a, b); }
__device__ __forceinline__ double tadd(double a, double b) { return add(a, b); }
__device__ __forceinline__ float tmul(float a, float b) { return a * b; }
__device__ __forceinline__ float tadd(float a, float b) { return a + b; }

template <typename T>
__device__ __forceinline__ T kick_value(const phk_kick_set& pk, int k,
                                        int s) {
    return __ldg(reinterpret_cast<const T*>(pk.kick[k]) + s);
}

template <typename T, int VEC>
__global__ void __launch_bounds__(kTrackThreads)
track_kernel(const __grid_constant__ phk_program prog,
             const __grid_constant__ phk_kick_set pk,
             const __grid_constant__ phk_accum acc, const TrackArgs a) {
    using AccT = typename AccumType<T>::type;
    extern __shared__ __align__(16) unsigned char smem[];
    const int Sa = a.has_acc ? acc.slicer.n_slices : 0;
    const int Sp = a.has_pk ? pk.slicer.n_slices : 0;
    AccT* hsx = reinterpret_cast<AccT*>(smem);
    AccT* hsy = hsx + Sa;
    T* eacc = reinterpret_cast<T*>(hsy + Sa);
    T* epk = eacc + (a.has_acc ? Sa + 1 : 0);
    int* hcnt = reinterpret_cast<int*>(epk + (a.has_pk ? Sp + 1 : 0));

    const int tid = threadIdx.x;
    if (a.has_acc) {
        const T* e = reinterpret_cast<const T*>(acc.slicer.edges);
        for (int i = tid; i <= Sa; i += blockDim.x) eacc[i] = e[i];
        for (int i = tid; i < Sa; i += blockDim.x) {
            hsx[i] = AccT(0); hsy[i] = AccT(0); hcnt[i] = 0;
        }
    }
    if (a.has_pk) {
        const T* e = reinterpret_cast<const T*>(pk.slicer.edges);
        for (int i = tid; i <= Sp; i += blockDim.x) epk[i] = e[i];
    }
    __syncthreads();

    T* cp[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) cp[q] = reinterpret_cast<T*>(a.c[q]);
    const T pk_tail = T(pk.slicer.est_tail), pk_iw = T(pk.slicer.est_inv_w);
    const T ac_tail = T(acc.slicer.est_tail), ac_iw = T(acc.slicer.est_inv_w);

    for (int64_t tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x) {
        const int64_t i0 = (tile * blockDim.x + tid) * VEC;
        if (i0 >= a.n) continue;
        const bool full = i0 + VEC <= a.n;
        T v[6][VEC];
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            if (!((a.load_mask >> q) & 1)) {
#pragma unroll
                for (int j = 0; j < VEC; ++j) v[q][j] = T(0);
                continue;
            }
            if (full) {
                VecIO<T, VEC>::ld(cp[q] + i0, v[q]);
            } else {
#pragma unroll
                for (int j = 0; j < VEC; ++j)
                    v[q][j] = (i0 + j < a.n) ? cp[q][i0 + j] : T(0);
            }
        }
        // 1. wake kicks of the previous WakeField.track, in kick order
        if (a.has_pk) {
#pragma unroll
            for (int j = 0; j < VEC; ++j) {
                const int s = slice_of<T>(v[PHK_Z][j], Sp, pk.slicer.negate,
                                          pk_tail, pk_iw, epk);
                if (s < 0 || i0 + j >= a.n) continue;
                T& kxp = v[PHK_XP][j];
                T& kyp = v[PHK_YP][j];
                T& kdp = v[PHK_DP][j];
                const T kx = v[PHK_X][j], ky = v[PHK_Y][j];
                for (int k = 0; k < pk.n_kicks; ++k) {
                    T val = kick_value<T>(pk, k, s);
                    const int qd = pk.quad[k];
                    if (qd == PHK_X) val = tmul(val, kx);
                    else if (qd == PHK_Y) val = tmul(val, ky);
                    const int tg = pk.target[k];
                    if (tg == PHK_XP) kxp = tadd(kxp, val);
                    else if (tg == PHK_YP) kyp = tadd(kyp, val);
                    else kdp = tadd(kdp, val);
                }
            }
        }
        // 2. element program
        for (int o = 0; o < prog.n_ops; ++o) {
            const phk_op& op = prog.op[o];
#pragma unroll
            for (int j = 0; j < VEC; ++j)
                apply_op(op, prog, v[PHK_X][j], v[PHK_XP][j], v[PHK_Y][j],
                         v[PHK_YP][j], v[PHK_Z][j], v[PHK_DP][j]);
        }
        // 3. slice accumulation
        if (a.has_acc) {
#pragma unroll
            for (int j = 0; j < VEC; ++j) {
                if (i0 + j >= a.n) continue;
                const int s = slice_of<T>(v[PHK_Z][j], Sa, acc.slicer.negate,
                                          ac_tail, ac_iw, eacc);
                if (acc.idx_out)
                    acc.idx_out[i0 + j] =
                        s >= 0 ? s
                               : outside_index((double)v[PHK_Z][j],
                                               acc.slicer.tail,
                                               acc.slicer.width);
                if (s >= 0) {
                    atomicAdd(hcnt + s, 1);
                    atomicAdd(hsx + s, AccT(v[PHK_X][j]));
                    atomicAdd(hsy + s, AccT(v[PHK_Y][j]));
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            if (!((a.store_mask >> q) & 1)) continue;
            if (full) {
                VecIO<T, VEC>::st(cp[q] + i0, v[q]);
            } else {
#pragma unroll
                for (int j = 0; j < VEC; ++j)
                    if (i0 + j < a.n) cp[q][i0 + j] = v[q][j];
            }
        }
    }

    if (a.has_acc) {
        __syncthreads();
        const int G = gridDim.x;
        double* P = acc.partials;
        for (int s = tid; s < Sa; s += blockDim.x) {
            P[(int64_t)s * G + blockIdx.x] = (double)hcnt[s];
            P[(int64_t)(Sa + s) * G + blockIdx.x] = (double)hsx[s];
            P[(int64_t)(2 * Sa + s) * G + blockIdx.x] = (double)hsy[s];
        }
    }
}

// ===================================================================
// launch configuration
// ===================================================================

template <typename T, int VEC>
static size_t smem_bytes(int Sa, int Sp) {
    using AccT = typename AccumType<T>::type;
    size_t b = 0;
    if (Sa > 0) b += 2 * sizeof(AccT) * Sa + sizeof(T) * (Sa + 1) + sizeof(int) * Sa;
    if (Sp > 0) b += sizeof(T) * (Sp + 1);
    return b;
}

size_t track_smem_bytes(int32_t dtype, int32_t Sa, int32_t Sp) {
    return dtype == PHK_F64 ? smem_bytes<double, 2>(Sa, Sp)
                            : smem_bytes<float, 4>(Sa, Sp);
}

// Opt the track kernel into the device's full dynamic shared memory, once
// per instantiation and device (never inside a stream capture's hot path).
template <typename T, int VEC>
static void prepare_track_kernel() {
    static int done_for[64] = {0};
    const DeviceInfo& d = device_info();
    const int dev = d.device < 64 ? d.device : 63;
    if (done_for[dev]) return;
    cudaFuncSetAttribute(track_kernel<T, VEC>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         d.max_smem_optin);
    done_for[dev] = 1;
}

template <typename T, int VEC>
static int occupancy_blocks(size_t smem) {
    int b = 0;
    prepare_track_kernel<T, VEC>();
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
            &b, track_kernel<T, VEC>, kTrackThreads, smem) != cudaSuccess)
        b = 1;
    return b < 1 ? 1 : b;
}

int track_grid(int64_t n, int32_t dtype, int32_t n_slices) {
    const DeviceInfo& d = device_info();
    // size the grid for an accumulation with a pending kick on the same
    // slicing (the largest shared-memory layout of a turn)
    const size_t smem = track_smem_bytes(dtype, n_slices, n_slices);
    const int vec = dtype == PHK_F64 ? 2 : 4;
    const int bps = dtype == PHK_F64 ? occupancy_blocks<double, 2>(smem)
                                     : occupancy_blocks<float, 4>(smem);
    const int64_t tiles = (n + (int64_t)kTrackThreads * vec - 1) /
                          ((int64_t)kTrackThreads * vec);
    int64_t g = (int64_t)d.sm_count * bps;
    if (tiles < g) g = tiles;
    if (g < 1) g = 1;
    return (int)g;
}

template <typename T, int VEC>
static int launch_track_t(const phk_program* prog, const phk_coords* c,
                          const phk_kick_set* pk, const phk_accum* acc,
                          int load_mask, int store_mask, cudaStream_t st) {
    TrackArgs a;
    a.c[0] = c->x; a.c[1] = c->xp; a.c[2] = c->y;
    a.c[3] = c->yp; a.c[4] = c->z; a.c[5] = c->dp;
    a.n = c->n;
    a.has_pk = pk != nullptr;
    a.has_acc = acc != nullptr;
    a.load_mask = load_mask;
    a.store_mask = store_mask;
    const int64_t per_tile = (int64_t)kTrackThreads * VEC;
    a.n_tiles = (c->n + per_tile - 1) / per_tile;
    static phk_kick_set zero_pk;
    static phk_accum zero_acc;
    const int Sa = acc ? acc->slicer.n_slices : 0;
    const int Sp = pk ? pk->slicer.n_slices : 0;
    const size_t smem = smem_bytes<T, VEC>(Sa, Sp);
    if (smem > (size_t)device_info().max_smem_optin)
        return set_error(PHK_ESIZE, "phk_track: %zu bytes of shared memory "
                         "needed for %d + %d slices", smem, Sa, Sp);
    int grid;
    if (acc) {
        grid = acc->grid;
    } else {
        const int bps = occupancy_blocks<T, VEC>(smem);
        int64_t g = (int64_t)device_info().sm_count * bps;
        if (a.n_tiles < g) g = a.n_tiles;
        grid = (int)(g < 1 ? 1 : g);
    }
    prepare_track_kernel<T, VEC>();
    track_kernel<T, VEC><<<grid, kTrackThreads, smem, st>>>(
        *prog, pk ? *pk : zero_pk, acc ? *acc : zero_acc, a);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(PHK_ECUDA, "phk_track launch: %s", cudaGetErrorString(e));
    count_launches(1);
    return PHK_OK;
}

static int op_mask(const phk_program* prog, int* load, int* store) {
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
        }
    }
    *load = ld; *store = stm;
    return 0;
}

int launch_track(const phk_program* prog, const phk_coords* c,
                 const phk_kick_set* pk, const phk_accum* acc,
                 cudaStream_t st) {
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
    // every coordinate the program writes must be read first
    ld |= stm;
    const bool f64 = c->dtype == PHK_F64;
    uintptr_t align = 0;
    void* ptrs[6] = {c->x, c->xp, c->y, c->yp, c->z, c->dp};
    for (int q = 0; q < 6; ++q)
        if ((ld >> q) & 1) align |= reinterpret_cast<uintptr_t>(ptrs[q]);
    const bool vec_ok = (align & 15) == 0;
    if (f64)
        return vec_ok ? launch_track_t<double, 2>(prog, c, pk, acc, ld, stm, st)
                      : launch_track_t<double, 1>(prog, c, pk, acc, ld, stm, st);
    return vec_ok ? launch_track_t<float, 4>(prog, c, pk, acc, ld, stm, st)
                  : launch_track_t<float, 1>(prog, c, pk, acc, ld, stm, st);
}

// ===================================================================
// fixed-order merge of the per-CTA partials (one warp per slice)
// ===================================================================

__global__ void finalize_kernel(const double* __restrict__ P, int S, int G,
                                int32_t* counts, double* mean_x,
                                double* mean_y, double* moments) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= S) return;
    const int s = warp;
    double c = 0.0, sx = 0.0, sy = 0.0;
    for (int g = lane; g < G; g += 32) {
        c += P[(int64_t)s * G + g];
        sx += P[(int64_t)(S + s) * G + g];
        sy += P[(int64_t)(2 * S + s) * G + g];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        c += __shfl_xor_sync(0xffffffffu, c, o);
        sx += __shfl_xor_sync(0xffffffffu, sx, o);
        sy += __shfl_xor_sync(0xffffffffu, sy, o);
    }
    if (lane != 0) return;
    const int32_t n = (int32_t)c;
    // stats.pyx:251-253: divide non-empty slices by their count
    const double mx = n ? dvd(sx, (double)n) : 0.0;
    const double my = n ? dvd(sy, (double)n) : 0.0;
    if (counts) counts[s] = n;
    if (mean_x) mean_x[s] = mx;
    if (mean_y) mean_y[s] = my;
    if (moments) {
        // wake_kicks.py:217-218: n_macroparticles_per_slice * mean
        moments[s] = (double)n;
        moments[S + s] = mul((double)n, mx);
        moments[2 * S + s] = mul((double)n, my);
    }
}

int launch_finalize(const phk_accum* acc, int32_t* counts, double* mean_x,
                    double* mean_y, double* moments, cudaStream_t st) {
    const int S = acc->slicer.n_slices;
    const int threads = 256;
    const int blocks = (S * 32 + threads - 1) / threads;
    finalize_kernel<<<blocks, threads, 0, st>>>(acc->partials, S, acc->grid,
                                                counts, mean_x, mean_y,
                                                moments);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(PHK_ECUDA, "phk_slice_finalize launch: %s",
                         cudaGetErrorString(e));
    count_launches(1);
    return PHK_OK;
}

// ===================================================================
// wake convolution
// ===================================================================

struct WakeArgs {
    phk_wake_set w;
};

// numpy path: one warp per (kick, target slice); lanes split the sources
__global__ void wake_conv_kernel(const __grid_constant__ phk_wake_set w) {
    const int S = w.n_slices;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int k = gw / S;
    const int i = gw - k * S;
    if (k >= w.n_kicks) return;
    const phk_wake_kick& kk = w.kick[k];
    if (kk.dense) return;
    const int L2 = 2 * S - 1;
    double acc = 0.0;
    for (int a = 0; a < kk.n_lags; ++a) {
        const int slot = ((w.head - a) % w.ring_len + w.ring_len) % w.ring_len;
        const double* m = w.moments + ((int64_t)slot * 3 + kk.source) * S;
        const double* v = kk.table + (int64_t)a * L2 + i + S - 1;
        double part = 0.0;
        for (int j = lane; j < S; j += 32) part = fma(m[j], v[-j], part);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            part += __shfl_xor_sync(0xffffffffu, part, o);
        acc = add(acc, part);
    }
    if (lane == 0) {
        const double r = mul(kk.factor, acc);
        if (w.out_dtype == PHK_F64)
            reinterpret_cast<double*>(kk.out)[i] = r;
        else
            reinterpret_cast<float*>(kk.out)[i] = (float)r;
    }
}

// dot-product path: one thread per (kick, target slice); coalesced over i
__global__ void wake_dense_kernel(const __grid_constant__ phk_wake_set w) {
    const int S = w.n_slices;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int k = t / S;
    const int i = t - k * S;
    if (k >= w.n_kicks) return;
    const phk_wake_kick& kk = w.kick[k];
    if (!kk.dense) return;
    double acc = 0.0;
    for (int a = 0; a < kk.n_lags; ++a) {
        const int slot = ((w.head - a) % w.ring_len + w.ring_len) % w.ring_len;
        const double* m = w.moments + ((int64_t)slot * 3 + kk.source) * S;
        const double* W = kk.table + (int64_t)a * S * S;
        double part = 0.0;
        for (int j = 0; j < S; ++j) part = fma(m[j], W[(int64_t)j * S + i], part);
        acc = add(acc, part);
    }
    const double r = mul(kk.factor, acc);
    if (w.out_dtype == PHK_F64)
        reinterpret_cast<double*>(kk.out)[i] = r;
    else
        reinterpret_cast<float*>(kk.out)[i] = (float)r;
}

int launch_wake(const phk_wake_set* w, cudaStream_t st) {
    bool any_dense = false, any_conv = false;
    for (int k = 0; k < w->n_kicks; ++k) {
        if (w->kick[k].dense) any_dense = true; else any_conv = true;
    }
    const int S = w->n_slices;
    if (any_conv) {
        const int warps = w->n_kicks * S;
        const int threads = 256;
        wake_conv_kernel<<<(warps * 32 + threads - 1) / threads, threads, 0,
                           st>>>(*w);
    }
    if (any_dense) {
        const int n = w->n_kicks * S;
        wake_dense_kernel<<<(n + 127) / 128, 128, 0, st>>>(*w);
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(PHK_ECUDA, "phk_wake launch: %s", cudaGetErrorString(e));
    count_launches((int)any_conv + (int)any_dense);
    return PHK_OK;
}

// ===================================================================
// per-slice moments for statistics (two passes, global FP64 atomics)
// ===================================================================

template <typename T>
__global__ void moments_kernel(const __grid_constant__ phk_slicer sl,
                               const T* __restrict__ z, int64_t n,
                               const T* __restrict__ q0,
                               const T* __restrict__ q1,
                               const T* __restrict__ q2, int n_q, int pass,
                               const double* __restrict__ means,
                               double* sums, int32_t* counts) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int S = sl.n_slices;
    T* e = reinterpret_cast<T*>(smem);
    for (int i = threadIdx.x; i <= S; i += blockDim.x)
        e[i] = reinterpret_cast<const T*>(sl.edges)[i];
    __syncthreads();
    const T tail = T(sl.est_tail), iw = T(sl.est_inv_w);
    const T* qs[3] = {q0, q1, q2};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int s = slice_of<T>(z[i], S, sl.negate, tail, iw, e);
        if (s < 0) continue;
        if (pass == 0) {
            atomicAdd(counts + s, 1);
            for (int q = 0; q < n_q; ++q)
                atomicAdd(sums + (int64_t)q * S + s, (double)qs[q][i]);
        } else {
            double d[3];
            for (int q = 0; q < n_q; ++q)
                d[q] = (double)qs[q][i] - means[(int64_t)q * S + s];
            // pairs (0,0) (0,1) (1,1) (0,2) (1,2) (2,2)
            const int pa[6] = {0, 0, 1, 0, 1, 2}, pb[6] = {0, 1, 1, 2, 2, 2};
            for (int p = 0; p < 6; ++p) {
                if (pa[p] >= n_q || pb[p] >= n_q) continue;
                atomicAdd(sums + (int64_t)(3 + p) * S + s, d[pa[p]] * d[pb[p]]);
            }
        }
    }
}

int launch_moments(const phk_slicer* sl, const void* z, int64_t n,
                   int32_t dtype, const void* const* q, int32_t n_q,
                   int32_t pass, const double* means, double* sums,
                   int32_t* counts, cudaStream_t st) {
    const DeviceInfo& d = device_info();
    const int threads = 256;
    int64_t blocks = (n + threads - 1) / threads;
    if (blocks > (int64_t)d.sm_count * 8) blocks = (int64_t)d.sm_count * 8;
    if (blocks < 1) blocks = 1;
    const void* qq[3] = {nullptr, nullptr, nullptr};
    for (int i = 0; i < n_q; ++i) qq[i] = q[i];
    if (dtype == PHK_F64) {
        const size_t smem = sizeof(double) * (sl->n_slices + 1);
        moments_kernel<double><<<(int)blocks, threads, smem, st>>>(
            *sl, (const double*)z, n, (const double*)qq[0],
            (const double*)qq[1], (const double*)qq[2], n_q, pass, means,
            sums, counts);
    } else {
        const size_t smem = sizeof(float) * (sl->n_slices + 1);
        moments_kernel<float><<<(int)blocks, threads, smem, st>>>(
            *sl, (const float*)z, n, (const float*)qq[0], (const float*)qq[1],
            (const float*)qq[2], n_q, pass, means, sums, counts);
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(PHK_ECUDA, "phk_slice_moments launch: %s",
                         cudaGetErrorString(e));
    count_launches(1);
    return PHK_OK;
}

}  // namespace phk
