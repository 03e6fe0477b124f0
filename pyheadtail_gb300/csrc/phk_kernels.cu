// Host-side planning and the small kernels around the fused pass: the
// launch dispatch of the track kernels (instantiated per precision in
// phk_track_f32.cu / phk_track_f64.cu), the fixed-order merge of the
// per-CTA partials, the wake convolution, the per-slice moment kernel and
// the batched merge / wake kernels.
#include "phk_track.cuh"

namespace phk {

size_t track_smem_bytes(int32_t dtype, int32_t Sa, int32_t Sp) {
    int nh, ks, st;
    // a turn's pending kicks: four dipolar kicks (resonator and resistive
    // wall, both planes).  Launches stage one summed table per plane; the
    // FP64 size is taken for all four tables, an upper bound (the launched
    // grid is the caller's column count either way)
    return dtype == PHK_F64 ? smem_for<double>(Sa, Sp, 4, false, &nh, &ks, &st)
                            : smem_for<float>(Sa, Sp, 2, true, &nh, &ks, &st);
}

// Compile-time shape of a program (see TrackShape), from its op kinds.
int program_shape(const phk_program* prog) {
    const int n = prog->n_ops;
    int k[4] = {0, 0, 0, 0};
    for (int i = 0; i < n && i < 4; ++i) k[i] = prog->op[i].kind;
    if (n == 0) return SHAPE_NONE;
    // the shapes read op[0]'s detuners from det[0] on
    if (k[0] == PHK_OP_TRANSVERSE && prog->op[0].det_begin != 0)
        return SHAPE_GENERIC;
    if (n == 1 && k[0] == PHK_OP_TRANSVERSE) return SHAPE_T;
    if (n == 2 && k[0] == PHK_OP_TRANSVERSE && k[1] == PHK_OP_LINEAR_LONG)
        return SHAPE_T_LIN;
    if (n == 4 && k[0] == PHK_OP_TRANSVERSE && k[1] == PHK_OP_DRIFT &&
        k[2] == PHK_OP_RF_KICK && k[3] == PHK_OP_DRIFT)
        return SHAPE_T_RF;
    return SHAPE_GENERIC;
}

// partial columns (= clusters) of an accumulating launch over n particles
int track_grid(int64_t n, int32_t dtype, int32_t n_slices) {
    // size for an accumulation with a pending kick on the same slicing (the
    // largest shared-memory layout of a turn)
    const size_t smem = track_smem_bytes(dtype, n_slices, n_slices);
    const int vec = dtype == PHK_F64 ? 2 : kF32Vec;
    const int nc = dtype == PHK_F64 ? track_clusters_f64(smem)
                                    : track_clusters_f32(smem);
    const int64_t tiles = (n + (int64_t)kTrackThreads * vec - 1) /
                          ((int64_t)kTrackThreads * vec);
    int64_t g = nc;
    const int64_t need = (tiles + kCluster - 1) / kCluster;
    if (need < g) g = need;
    if (g < 1) g = 1;
    return (int)g;
}

int launch_track(const phk_program* prog, const phk_coords* c,
                 const phk_kick_set* pk, const phk_accum* acc,
                 cudaStream_t st) {
    int ld, stm;
    track_masks(prog, pk, acc, &ld, &stm);
    uintptr_t align = 0;
    void* ptrs[6] = {c->x, c->xp, c->y, c->yp, c->z, c->dp};
    for (int q = 0; q < 6; ++q)
        if ((ld >> q) & 1) align |= reinterpret_cast<uintptr_t>(ptrs[q]);
    const bool vec_ok = (align & 15) == 0;
    if (c->dtype == PHK_F64)
        return launch_track_f64(prog, c, pk, acc, ld, stm, vec_ok, st);
    return launch_track_f32(prog, c, pk, acc, ld, stm, vec_ok, st);
}

// ===================================================================
// fixed-order merge of the per-CTA partials (one warp per slice)
// ===================================================================

// Fixed-order sum of the partial columns [g0, g1) of slice s (P laid out
// [3][S][G]) and the finalised outputs; all 32 lanes of the warp call it.
__device__ __forceinline__ void merge_slice(const double* __restrict__ P,
                                            int S, int G, int s, int g0,
                                            int g1, int32_t* counts,
                                            double* mean_x, double* mean_y,
                                            double* moments, int lane) {
    const double* pc = P + (int64_t)s * G;
    const double* px = P + (int64_t)(S + s) * G;
    const double* py = P + (int64_t)(2 * S + s) * G;
    // four independent strided partial sums per lane (loads in flight),
    // combined in a fixed order: the result does not depend on timing
    double c[4] = {0, 0, 0, 0}, sx[4] = {0, 0, 0, 0}, sy[4] = {0, 0, 0, 0};
    int g = g0 + lane;
    for (; g + 96 < g1; g += 128) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            c[u] += pc[g + 32 * u];
            sx[u] += px[g + 32 * u];
            sy[u] += py[g + 32 * u];
        }
    }
    for (; g < g1; g += 32) {
        c[0] += pc[g];
        sx[0] += px[g];
        sy[0] += py[g];
    }
    double tc = (c[0] + c[1]) + (c[2] + c[3]);
    double tx = (sx[0] + sx[1]) + (sx[2] + sx[3]);
    double ty = (sy[0] + sy[1]) + (sy[2] + sy[3]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        tc += __shfl_xor_sync(0xffffffffu, tc, o);
        tx += __shfl_xor_sync(0xffffffffu, tx, o);
        ty += __shfl_xor_sync(0xffffffffu, ty, o);
    }
    if (lane != 0) return;
    const int32_t n = (int32_t)tc;
    // stats.pyx:251-253: divide non-empty slices by their count
    const double mx = n ? dvd(tx, (double)n) : 0.0;
    const double my = n ? dvd(ty, (double)n) : 0.0;
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

__global__ void finalize_kernel(const double* __restrict__ P, int S, int G,
                                int32_t* counts, double* mean_x,
                                double* mean_y, double* moments) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= S) return;
    merge_slice(P, S, G, warp, 0, G, counts, mean_x, mean_y, moments, lane);
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
// compensated column sums of a particle shard (one warp per slice)
// ===================================================================

// Error-free sum: s + e == a + b exactly (Knuth's TwoSum, six operations,
// no branch); symmetric in a and b.
__device__ __forceinline__ void two_sum(double a, double b, double* s,
                                        double* e) {
    const double t = add(a, b);
    const double bb = sub(t, a);
    *e = add(sub(a, sub(t, bb)), sub(b, bb));
    *s = t;
}

// (hi, lo) pairs: hi the running sum, lo the running sum of the exact
// rounding errors; combining two pairs adds their lows and the error of
// the high sum.
__device__ __forceinline__ void dd_combine(double& hi, double& lo, double bh,
                                           double bl) {
    double s, e;
    two_sum(hi, bh, &s, &e);
    lo = add(add(lo, bl), e);
    hi = s;
}

// Per slice s and quantity q (count, sum x, sum y): lane l adds columns
// l, l + 32, ... in order into its (hi, lo) pair, then the lanes combine
// in a fixed butterfly (partner l ^ 16, ^ 8, ^ 4, ^ 2, ^ 1); lane 0 writes
// out[(0 * 3 + q) * S + s] = hi, out[(1 * 3 + q) * S + s] = lo.  hi + lo
// is the sum of the columns to about 2^-106 of the largest partial sum,
// so sums of disjoint column sets merged the same way (phk_slice_merge on
// the pairs of every shard) round to the same double as one fold over
// all columns.
__global__ void slice_sums_kernel(const double* __restrict__ P, int S, int G,
                                  double* __restrict__ out) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= S) return;
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const double* pc = P + ((int64_t)q * S + warp) * G;
        double hi = 0.0, lo = 0.0;
        for (int g = lane; g < G; g += 32) {
            double s, e;
            two_sum(hi, pc[g], &s, &e);
            hi = s;
            lo = add(lo, e);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double bh = __shfl_xor_sync(0xffffffffu, hi, o);
            const double bl = __shfl_xor_sync(0xffffffffu, lo, o);
            dd_combine(hi, lo, bh, bl);
        }
        if (lane == 0) {
            out[(int64_t)q * S + warp] = hi;
            out[(int64_t)(3 + q) * S + warp] = lo;
        }
    }
}

int launch_slice_sums(const phk_accum* acc, double* out, cudaStream_t st) {
    const int S = acc->slicer.n_slices;
    const int threads = 256;
    const int blocks = (S * 32 + threads - 1) / threads;
    slice_sums_kernel<<<blocks, threads, 0, st>>>(acc->partials, S, acc->grid,
                                                  out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(PHK_ECUDA, "phk_slice_sums launch: %s",
                         cudaGetErrorString(e));
    count_launches(1);
    return PHK_OK;
}

// Rank-ordered merge of the (hi, lo) pairs of n_shards shards, laid out
// [n_shards][2][3][S]: shard 0's pair, combined with shard 1's, then 2's,
// ...; then the finalised outputs of phk_slice_finalize from the totals
// hi + lo.  One thread per slice.
__global__ void slice_merge_kernel(const double* __restrict__ sums,
                                   int n_shards, int S, int32_t* counts,
                                   double* mean_x, double* mean_y,
                                   double* moments) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    double t[3];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        double hi = sums[(int64_t)q * S + s];
        double lo = sums[(int64_t)(3 + q) * S + s];
        for (int r = 1; r < n_shards; ++r) {
            const double* b = sums + (int64_t)r * 6 * S;
            dd_combine(hi, lo, b[(int64_t)q * S + s], b[(int64_t)(3 + q) * S + s]);
        }
        t[q] = add(hi, lo);
    }
    const int32_t n = (int32_t)t[0];
    const double mx = n ? dvd(t[1], (double)n) : 0.0;
    const double my = n ? dvd(t[2], (double)n) : 0.0;
    if (counts) counts[s] = n;
    if (mean_x) mean_x[s] = mx;
    if (mean_y) mean_y[s] = my;
    if (moments) {
        moments[s] = (double)n;
        moments[S + s] = mul((double)n, mx);
        moments[2 * S + s] = mul((double)n, my);
    }
}

int launch_slice_merge(const double* sums, int n_shards, int S,
                       int32_t* counts, double* mean_x, double* mean_y,
                       double* moments, cudaStream_t st) {
    const int threads = 128;
    const int blocks = (S + threads - 1) / threads;
    slice_merge_kernel<<<blocks, threads, 0, st>>>(sums, n_shards, S, counts,
                                                   mean_x, mean_y, moments);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(PHK_ECUDA, "phk_slice_merge launch: %s",
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

// numpy path: one warp per (kick, target slice); lanes split the sources.
// Each lane keeps its partial sums over every stored turn and the warp
// reduces once at the end (the reference sums each turn's convolution,
// then the turns: the same terms, regrouped; GB300's FP64 pipe makes the
// per-turn reductions the larger part of the cost otherwise).
__device__ __forceinline__ void wake_conv_one(const phk_wake_set& w, int gw,
                                              int lane) {
    const int S = w.n_slices;
    const int k = gw / S;
    const int i = gw - k * S;
    if (k >= w.n_kicks) return;
    const phk_wake_kick& kk = w.kick[k];
    if (kk.dense) return;
    const int L2 = 2 * S - 1;
    double p0 = 0.0, p1 = 0.0, p2 = 0.0, p3 = 0.0;
    int slot = (w.head % w.ring_len + w.ring_len) % w.ring_len;
    for (int a = 0; a < kk.n_lags; ++a) {
        const double* m = w.moments + ((int64_t)slot * 3 + kk.source) * S;
        const double* v = kk.table + (int64_t)a * L2 + i + S - 1;
        int j = lane;
        for (; j + 96 < S; j += 128) {
            p0 = fma(__ldg(m + j), __ldg(v - j), p0);
            p1 = fma(__ldg(m + j + 32), __ldg(v - j - 32), p1);
            p2 = fma(__ldg(m + j + 64), __ldg(v - j - 64), p2);
            p3 = fma(__ldg(m + j + 96), __ldg(v - j - 96), p3);
        }
        for (; j < S; j += 32) p0 = fma(__ldg(m + j), __ldg(v - j), p0);
        slot = slot == 0 ? w.ring_len - 1 : slot - 1;
    }
    double part = (p0 + p1) + (p2 + p3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane == 0) {
        const double r = mul(kk.factor, part);
        if (w.out_dtype == PHK_F64)
            reinterpret_cast<double*>(kk.out)[i] = r;
        else
            reinterpret_cast<float*>(kk.out)[i] = (float)r;
    }
}

// dot-product path: one thread per (kick, target slice); coalesced over i
__device__ __forceinline__ void wake_dense_one(const phk_wake_set& w, int t) {
    const int S = w.n_slices;
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

// Single-bunch numpy path: one CTA of kConvWarps warps per (kick, target
// slice); warp w takes the stored turns w, w + kConvWarps, ...; the warps'
// partial sums are added in a fixed order.  (One warp per output leaves
// too few warps on GB300 to cover the load latency of a 50-turn history.)
constexpr int kConvWarps = 8;
__global__ void __launch_bounds__(kConvWarps * 32)
wake_conv_kernel(const __grid_constant__ phk_wake_set w) {
    __shared__ double part_w[kConvWarps];
    const int S = w.n_slices;
    const int k = blockIdx.x / S;
    const int i = blockIdx.x - k * S;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (k >= w.n_kicks) return;
    const phk_wake_kick& kk = w.kick[k];
    if (kk.dense) return;
    const int L2 = 2 * S - 1;
    double p0 = 0.0, p1 = 0.0, p2 = 0.0, p3 = 0.0;
    for (int a = warp; a < kk.n_lags; a += kConvWarps) {
        const int slot = ((w.head - a) % w.ring_len + w.ring_len) % w.ring_len;
        const double* m = w.moments + ((int64_t)slot * 3 + kk.source) * S;
        const double* v = kk.table + (int64_t)a * L2 + i + S - 1;
        int j = lane;
        for (; j + 96 < S; j += 128) {
            p0 = fma(__ldg(m + j), __ldg(v - j), p0);
            p1 = fma(__ldg(m + j + 32), __ldg(v - j - 32), p1);
            p2 = fma(__ldg(m + j + 64), __ldg(v - j - 64), p2);
            p3 = fma(__ldg(m + j + 96), __ldg(v - j - 96), p3);
        }
        for (; j < S; j += 32) p0 = fma(__ldg(m + j), __ldg(v - j), p0);
    }
    double part = (p0 + p1) + (p2 + p3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        part += __shfl_xor_sync(0xffffffffu, part, o);
    if (lane == 0) part_w[warp] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
        double acc = part_w[0];
        for (int q = 1; q < kConvWarps; ++q) acc += part_w[q];
        const double r = mul(kk.factor, acc);
        if (w.out_dtype == PHK_F64)
            reinterpret_cast<double*>(kk.out)[i] = r;
        else
            reinterpret_cast<float*>(kk.out)[i] = (float)r;
    }
}

__global__ void wake_dense_kernel(const __grid_constant__ phk_wake_set w) {
    wake_dense_one(w, blockIdx.x * blockDim.x + threadIdx.x);
}

int launch_wake(const phk_wake_set* w, cudaStream_t st) {
    bool any_dense = false, any_conv = false;
    for (int k = 0; k < w->n_kicks; ++k) {
        if (w->kick[k].dense) any_dense = true; else any_conv = true;
    }
    const int S = w->n_slices;
    if (any_conv)
        wake_conv_kernel<<<w->n_kicks * S, kConvWarps * 32, 0, st>>>(*w);
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


// ===================================================================
// batched form: dispatch, merge and wake
// ===================================================================

int launch_track_batch(const phk_batch* bt, const phk_coords* c,
                       const phk_kick_set* pk, const phk_accum* acc,
                       cudaStream_t st) {
    int ld = 0, stm = 0;
    for (int i = 0; i < bt->n_bunches; ++i) {
        int l, s;
        track_masks(bt->programs_host + i, pk, acc, &l, &s);
        ld |= l;
        stm |= s;
    }
    if (c->dtype == PHK_F64) return launch_batch_f64(bt, c, pk, acc, ld, stm, st);
    return launch_batch_f32(bt, c, pk, acc, ld, stm, st);
}

int batch_max_grid(int32_t dtype, int32_t threads, int32_t S, int32_t nk) {
    int nh = 0;
    int per_sm = 0;
    if (dtype == PHK_F64)
        per_sm = batch_per_sm_f64(
            threads, batch_smem<double>(S, nk > 0 ? S : 0, nk, threads, &nh));
    else
        per_sm = batch_per_sm_f32(
            threads, batch_smem<float>(S, nk > 0 ? S : 0, nk, threads, &nh));
    return per_sm * device_info().sm_count;
}

__global__ void batch_finalize_kernel(const double* __restrict__ P, int S,
                                      int G, int nb,
                                      const int32_t* __restrict__ bcols,
                                      int32_t* counts, double* mean_x,
                                      double* mean_y, double* moments,
                                      int64_t mstride, int32_t* status) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int bunch = warp / S;
    const int s = warp - bunch * S;
    if (bunch >= nb) return;
    int g0 = bcols[bunch], g1 = bcols[bunch + 1];
    if (g0 < 0 || g1 > G || g0 > g1) {
        if (lane == 0 && status) atomicMax(status, PHK_DEV_BAD_TABLE);
        g0 = g1 = 0;
    }
    const int64_t o = (int64_t)bunch * S;
    merge_slice(P, S, G, s, g0, g1, counts ? counts + o : nullptr,
                mean_x ? mean_x + o : nullptr, mean_y ? mean_y + o : nullptr,
                moments ? moments + bunch * mstride : nullptr, lane);
}

int launch_batch_finalize(const phk_accum* acc, int nb, const int32_t* bcols,
                          int32_t* counts, double* mean_x, double* mean_y,
                          double* moments, int64_t mstride, int32_t* status,
                          cudaStream_t st) {
    const int S = acc->slicer.n_slices;
    const int64_t warps = (int64_t)nb * S;
    const int threads = 256;
    const int64_t blocks = (warps * 32 + threads - 1) / threads;
    batch_finalize_kernel<<<(unsigned)blocks, threads, 0, st>>>(
        acc->partials, S, acc->grid, nb, bcols, counts, mean_x, mean_y,
        moments, mstride, status);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(PHK_ECUDA, "phk_batch_finalize launch: %s",
                         cudaGetErrorString(e));
    count_launches(1);
    return PHK_OK;
}

// one warp per (bunch, kick, target slice), numpy path; one thread per
// (bunch, kick, target slice), dot-product path
__global__ void batch_wake_kernel(const phk_wake_set* __restrict__ sets,
                                  int nb, int S, int nk) {
    const int64_t gw = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int per = nk * S;
    const int64_t bunch = gw / per;
    if (bunch >= nb) return;
    const phk_wake_set& w = sets[bunch];
    if (w.n_slices != S || w.n_kicks > nk || w.n_kicks < 0 ||
        w.ring_len < 1 || w.head < 0 || w.head >= w.ring_len)
        return;
    const int r = (int)(gw - bunch * per);
    wake_conv_one(w, r, lane);
    // dense kicks: the warp's lanes take target slices r*32+lane of the
    // warp-major numbering (warps [0, per/32] cover all nk*S targets)
    const int t = r * 32 + lane;
    if (t < per) wake_dense_one(w, t);
}

int launch_wake_batch(const phk_wake_set* sets, int nb, int S, int nk,
                      cudaStream_t st) {
    const int64_t warps = (int64_t)nb * nk * S;
    const int threads = 256;
    const int64_t blocks = (warps * 32 + threads - 1) / threads;
    batch_wake_kernel<<<(unsigned)blocks, threads, 0, st>>>(sets, nb, S, nk);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(PHK_ECUDA, "phk_wake_batch launch: %s",
                         cudaGetErrorString(e));
    count_launches(1);
    return PHK_OK;
}

}  // namespace phk
