// Multi-turn wake convolution of the FP32 form as a Toeplitz GEMM on the
// 5th-generation tensor cores (tcgen05), BF16x3 split products accumulated
// in FP32 in tensor memory.
//
// For every kick k (wake_kicks.py:118-139, numpy path :87-116):
//   out_k[i] = factor_k * sum_a sum_j T_g(k)[a][i - j + S - 1] * m_a[src_k][j]
// with T_g the sampled wake of table group g (kicks whose tables are equal,
// e.g. the x and y dipole kicks of a circular source, share one group) and
// m_a the moment ring slot of stored turn a.  Written as D = A B^T:
//   A[i][(g, a, j)] = T_g[a][i - j + S - 1]          (S x K, the Toeplitz
//                                                     rows of every group)
//   B[n][(g, a, j)] = m_a[src_k][j] if g(k) == g    (n = k: high part,
//                                                     n = nk + k: low part)
// Each operand is split into a high and a low bfloat16 part (x ~ hi + lo to
// ~2^-16 relative); D_hi = A_hi B^T and D_lo = A_lo B^T hold all four
// products hi*hi, hi*lo, lo*hi, lo*lo, summed in the epilogue.
//
// A is never stored: a 128 x 64 tile of it is a window of at most two
// rows of a table (191 consecutive samples per lag), so each CTA builds its
// A tiles in shared memory, in the canonical no-swizzle K-major layout of
// the tensor-core operand, from a bfloat16 hi / lo copy of the tables
// (written once per table change; C3: 200 KB, read from L2).  B is built
// in shared memory from the FP64 moment ring for all of a CTA's K chunks
// (at most kTcMaxChunks) before its first MMA.  The K range is
// split across CTAs; a fixed-order FP64 reduction of the split partials
// applies the factors.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "phk_device.cuh"
#include "phk_internal.h"

namespace phk {

constexpr int kTcM = 128;          // rows per tile (TMEM lanes)
constexpr int kTcN = 16;           // B rows: hi and lo parts of <= 8 kicks
constexpr int kTcK = 64;           // K per chunk (4 MMAs of K = 16)
constexpr int kTcStages = 3;
constexpr int kTcMaxChunks = 8;    // K chunks per CTA (B staged up front)
constexpr int kTcThreads = 256;
constexpr unsigned kTcTileBytes = kTcM * kTcK * 2;   // 16 KB per A part
constexpr int kTcBuildRows = kTcThreads / 8;          // rows per build pass

// K columns of one lag: the S source slices padded to a multiple of 8 (so
// that no 8-column segment of a tile row spans two lags); the padding
// columns of B are zero
__host__ __device__ __forceinline__ int lag_cols(int S) { return (S + 7) & ~7; }
// bfloat16 table rows (a_hi / a_lo): 8 zeros, the 2 S - 1 samples, 9 zeros
__host__ __device__ __forceinline__ int row_stride(int S) { return 2 * S + 16; }
constexpr unsigned kTcBBytes = kTcN * kTcK * 2;      // 2 KB
constexpr unsigned kTcWaitLimit = 1u << 22;

// ------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ void tmem_alloc(unsigned* dst, unsigned ncols) {
    asm volatile(
        "tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
            smem_addr(dst)),
        "r"(ncols)
        : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::
                     : "memory");
}
__device__ __forceinline__ void tmem_dealloc(unsigned taddr, unsigned ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(
                     taddr),
                 "r"(ncols)
                 : "memory");
}
// D[tmem] (+)= A[smem] * B[smem]^T, kind::f16 (bf16 in, fp32 accumulate)
__device__ __forceinline__ void umma_bf16(unsigned d, uint64_t a, uint64_t b,
                                          unsigned idesc, unsigned accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
// arrive on the mbarrier once every MMA issued so far has completed
__device__ __forceinline__ void umma_commit(unsigned long long* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 "
        "[%0];" ::"r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ void tc_fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
// 16 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld16(unsigned taddr, float (&v)[16]) {
    unsigned r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
          "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
          "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Shared-memory operand descriptor, canonical K-major layout without
// swizzle: 8-row x 16-byte core matrices of 128 contiguous bytes; `lbo` is
// the byte distance of core matrices adjacent along K, `sbo` along M/N.
__device__ __forceinline__ uint64_t smem_desc(unsigned addr, unsigned lbo,
                                              unsigned sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;   // descriptor version of this architecture
    return d;                 // base offset 0, no swizzle
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N = 16, M = 128.
constexpr unsigned kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) |
                              ((unsigned)(kTcN >> 3) << 17) |
                              ((unsigned)(kTcM >> 4) << 24);

// element (r, k) of a tile of `rows` x 64 in the canonical layout (core
// matrices ordered k-fastest: lbo = 128 B, sbo = 1024 B)
__host__ __device__ __forceinline__ int tile_offset(int r, int k) {
    return ((r >> 3) * 8 + (k >> 3)) * 64 + (r & 7) * 8 + (k & 7);
}

// hi + lo ~ x to ~2^-16 relative; the split runs in FP32 after one
// conversion (the two parts keep 16 of FP32's 24 bits, and GB300's FP64
// pipe would otherwise bound the operand staging)
__device__ __forceinline__ void split_bf16(double x, __nv_bfloat16* hi,
                                           __nv_bfloat16* lo) {
    const float f = (float)x;
    const __nv_bfloat16 h = __float2bfloat16_rn(f);
    *hi = h;
    *lo = __float2bfloat16_rn(f - __bfloat162float(h));
}

// K index -> (group, lag, source slice); false past the groups' columns
// and on the padding columns of a lag
__device__ __forceinline__ bool decode_k(const phk_wake_tc& w, int kg, int* g,
                                         int* a, int* j) {
    const int SC = lag_cols(w.n_slices);
    int gg = w.n_groups - 1;
    while (gg > 0 && kg < w.group_k0[gg]) --gg;
    const int r = kg - w.group_k0[gg];
    if (r < 0) return false;
    const int aa = r / SC;
    if (aa >= w.group_lags[gg]) return false;
    const int jj = r - aa * SC;
    if (jj >= w.n_slices) return false;
    *g = gg;
    *a = aa;
    *j = jj;
    return true;
}

// ------------------------------------------------------------ table split
// bfloat16 hi / lo parts of every table row: sample t of lag a of group g
// at row_stride(S) * R + 8 + t, R = group_k0[g] / lag_cols(S) + a (the
// padding elements are zero)
__global__ void wake_split_kernel(const __grid_constant__ phk_wake_tc w) {
    const int S = w.n_slices, L = 2 * S - 1, Ls = row_stride(S);
    const int SC = lag_cols(S);
    const int rows = w.group_k0[w.n_groups - 1] / SC + w.group_lags[w.n_groups - 1];
    const int64_t total = (int64_t)rows * Ls;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int row = (int)(e / Ls);
        const int t = (int)(e - (int64_t)row * Ls) - 8;
        int g = w.n_groups - 1;
        while (g > 0 && row < w.group_k0[g] / SC) --g;
        const int a = row - w.group_k0[g] / SC;
        const double v = (t >= 0 && t < L) ? w.tables[g][(int64_t)a * L + t] : 0.0;
        __nv_bfloat16 h, l;
        split_bf16(v, &h, &l);
        reinterpret_cast<__nv_bfloat16*>(w.a_hi)[e] = h;
        reinterpret_cast<__nv_bfloat16*>(w.a_lo)[e] = l;
    }
}

// ------------------------------------------------------------ the GEMM
// grid (m_tiles, splits); CTA (mt, sp) multiplies row tile mt over its
// contiguous range of K chunks and writes FP32 partials[sp][k][row].
__global__ void __launch_bounds__(kTcThreads, 1)
wake_gemm_kernel(const __grid_constant__ phk_wake_tc w, unsigned wait_limit) {
    // A stages [A_hi | A_lo], then the B tiles of every chunk (the
    // no-swizzle operand layout needs 16-byte aligned core matrices)
    extern __shared__ __align__(128) unsigned char smem[];
    constexpr unsigned kStage = 2 * kTcTileBytes;
    unsigned char* bsm = smem + kTcStages * kStage;
    unsigned long long* done = reinterpret_cast<unsigned long long*>(
        bsm + kTcMaxChunks * kTcBBytes);
    unsigned long long* fin = done + kTcStages;
    unsigned* s_taddr = reinterpret_cast<unsigned*>(fin + 1);
    __shared__ int s_fail;

    const int tid = threadIdx.x, warp = tid >> 5;
    const int mt = blockIdx.x, sp = blockIdx.y;
    const int n_chunks = w.k_total / kTcK;
    const int c0 = (int)((int64_t)n_chunks * sp / gridDim.y);
    const int c1 = (int)((int64_t)n_chunks * (sp + 1) / gridDim.y);
    const int nc = c1 - c0 < kTcMaxChunks ? c1 - c0 : kTcMaxChunks;
    const int S = w.n_slices, nk = w.n_kicks;

    if (tid == 0) {
        s_fail = 0;
        for (int s = 0; s < kTcStages; ++s) mbar_init(done + s, 1);
        mbar_init(fin, 1);
        mbar_fence_init();
    }
    if (warp == 0) {
        tmem_alloc(s_taddr, 32);   // D_hi: columns 0-15, D_lo: 16-31
        tmem_relinquish();
    }
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();
    const unsigned taddr = *s_taddr;

    // A tile of chunk c0 + it into stage st.  An 8-column segment of a
    // tile row lies within one lag (lag_cols), so its eight elements,
    // sample i - j + S - 1 for j = j0 .. j0 + 7, are eight consecutive
    // samples of one table row in descending order: five aligned 32-bit
    // loads, four byte permutes, one 16-byte store in the canonical
    // layout.  Thread t fills segment t & 7 of rows (t >> 3) + 32 m; rows
    // past the slices and columns past the groups are zero.  The loads of
    // the next chunk are issued right after a tile's stores, so they are
    // in flight while the CTA synchronises and its MMAs are issued.
    const int SC = lag_cols(S), Ls = row_stride(S);
    const int k_valid = w.group_k0[w.n_groups - 1] + w.group_lags[w.n_groups - 1] * SC;
    const unsigned* thi = reinterpret_cast<const unsigned*>(w.a_hi);
    const unsigned* tlo = reinterpret_cast<const unsigned*>(w.a_lo);
    constexpr int kRows = kTcM / kTcBuildRows;
    // the source words of chunk c0 + it (loads only; held in registers so
    // that their latency overlaps the previous chunk's barrier and MMAs)
    auto build_load = [&](int it, unsigned (&h)[kRows][5], unsigned (&l)[kRows][5]) {
        const int c = tid & 7;
        const int kg0 = (c0 + it) * kTcK + 8 * c;
        const int R = kg0 / SC;
        const int j0 = kg0 - R * SC;
        const bool cols = kg0 < k_valid;
#pragma unroll
        for (int m = 0; m < kRows; ++m) {
            const int i = mt * kTcM + (tid >> 3) + kTcBuildRows * m;
            // elements e_q = T[base + 7 - q], q = 0..7
            const int64_t base = (int64_t)R * Ls + 8 + (S - 1 - j0 + i) - 7;
            const int64_t w0 = base >> 1;          // 32-bit word index
            const bool on = cols && i < S;
#pragma unroll
            for (int q = 0; q < 5; ++q) {
                h[m][q] = on ? __ldg(thi + w0 + q) : 0u;
                l[m][q] = on ? __ldg(tlo + w0 + q) : 0u;
            }
        }
    };
    // the permutes and stores of chunk c0 + it into stage st
    auto build_store = [&](int it, int st, const unsigned (&h)[kRows][5],
                           const unsigned (&l)[kRows][5]) {
        const int c = tid & 7;
        const int kg0 = (c0 + it) * kTcK + 8 * c;
        const int R = kg0 / SC;
        const int j0 = kg0 - R * SC;
        unsigned char* dst = smem + st * kStage;
#pragma unroll
        for (int m = 0; m < kRows; ++m) {
            const int r = (tid >> 3) + kTcBuildRows * m;
            const int i = mt * kTcM + r;
            const unsigned sel = ((S - 1 - j0 + i) & 1) ? 0x5476u : 0x7610u;
            const uint4 vh = make_uint4(
                __byte_perm(h[m][4], h[m][3], sel), __byte_perm(h[m][3], h[m][2], sel),
                __byte_perm(h[m][2], h[m][1], sel), __byte_perm(h[m][1], h[m][0], sel));
            const uint4 vl = make_uint4(
                __byte_perm(l[m][4], l[m][3], sel), __byte_perm(l[m][3], l[m][2], sel),
                __byte_perm(l[m][2], l[m][1], sel), __byte_perm(l[m][1], l[m][0], sel));
            const int off = tile_offset(r, 8 * c) * 2;
            *reinterpret_cast<uint4*>(dst + off) = vh;
            *reinterpret_cast<uint4*>(dst + kTcTileBytes + off) = vl;
        }
    };
    unsigned src_h[kRows][5], src_l[kRows][5];
    if (nc > 0) build_load(0, src_h, src_l);    // in flight during B staging

    // B of every chunk of this CTA: one K column per thread and pass,
    // decoded once, then the rows of its kicks (hi rows 0..nk-1, lo rows
    // nk..2nk-1; the rest zero)
    for (int e = tid; e < nc * kTcK; e += kTcThreads) {
        const int c = e / kTcK, kk = e - c * kTcK;
        int g = 0, a = 0, j = 0;
        const bool on = decode_k(w, (c0 + c) * kTcK + kk, &g, &a, &j);
        const int slot = ((w.head - a) % w.ring_len + w.ring_len) % w.ring_len;
        __nv_bfloat16* col = reinterpret_cast<__nv_bfloat16*>(bsm + c * kTcBBytes);
#pragma unroll
        for (int k = 0; k < kTcN / 2; ++k) {
            if (k >= nk) break;
            double v = 0.0;
            if (on && w.group_of[k] == g && a < w.n_lags[k])
                v = w.moments[((int64_t)slot * 3 + w.source[k]) * S + j];
            __nv_bfloat16 h, l;
            split_bf16(v, &h, &l);
            col[tile_offset(k, kk)] = h;
            col[tile_offset(nk + k, kk)] = l;
        }
        for (int n = 2 * nk; n < kTcN; ++n)
            col[tile_offset(n, kk)] = __float2bfloat16_rn(0.f);
    }

    // per chunk: the CTA builds its A tile in a free stage (the MMAs that
    // read the stage before have completed), then one thread issues the
    // MMAs asynchronously, so building the next tile overlaps them
    int it = 0;
    for (; it < nc; ++it) {
        const int st = it % kTcStages;
        bool ok = true;
        if (it >= kTcStages)
            ok = mbar_wait(done + st, (unsigned)((it / kTcStages - 1) & 1),
                           wait_limit);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) s_fail = 1;
            break;
        }
        tc_fence_after_sync();
        build_store(it, st, src_h, src_l);
        if (it + 1 < nc) build_load(it + 1, src_h, src_l);
        fence_proxy_async_smem();      // generic writes -> tensor-core reads
        __syncthreads();
        if (tid == 0) {
            tc_fence_after_sync();
            const unsigned a_hi = smem_addr(smem + st * kStage);
            const unsigned a_lo = a_hi + kTcTileBytes;
            const unsigned b = smem_addr(bsm + it * kTcBBytes);
#pragma unroll
            for (int ks = 0; ks < kTcK / 16; ++ks) {
                const unsigned acc = (it > 0 || ks > 0) ? 1u : 0u;
                const uint64_t db = smem_desc(b + ks * 256, 128, 1024);
                umma_bf16(taddr, smem_desc(a_hi + ks * 256, 128, 1024), db,
                          kTcIdesc, acc);
                umma_bf16(taddr + 16, smem_desc(a_lo + ks * 256, 128, 1024), db,
                          kTcIdesc, acc);
            }
            umma_commit(done + st);
        }
    }

    // completion of every MMA issued (the commit arrives once all are
    // done; bounded)
    if (tid == 0) {
        umma_commit(fin);
        if (!mbar_wait(fin, 0, kTcWaitLimit)) s_fail = 2;
    }
    tc_fence_before_sync();
    __syncthreads();
    tc_fence_after_sync();

    if (!s_fail && warp < 4) {
        // warp q reads TMEM lanes 32q..32q+31: rows of this tile
        float dh[16], dl[16];
        const unsigned lane_base = (unsigned)(warp * 32) << 16;
        if (nc > 0) {
            tmem_ld16(taddr + lane_base, dh);
            tmem_ld16(taddr + lane_base + 16, dl);
        } else {
#pragma unroll
            for (int c = 0; c < 16; ++c) dh[c] = dl[c] = 0.f;
        }
        const int row = mt * kTcM + warp * 32 + (tid & 31);
        const int rows = w.m_tiles * kTcM;
        for (int k = 0; k < nk; ++k) {
            // hi*hi + hi*lo + lo*hi + lo*lo
            const float v = (dh[k] + dh[nk + k]) + (dl[k] + dl[nk + k]);
            w.partials[((int64_t)sp * nk + k) * rows + row] = v;
        }
    }
    // 1: a stage wait gave up and every MMA issued completed; 2: the final
    // wait for them gave up as well
    if (s_fail && tid == 0 && w.status)
        atomicMax(w.status, s_fail == 2 ? PHK_DEV_TIMEOUT_UNDRAINED : PHK_DEV_TIMEOUT);
    tc_fence_before_sync();
    __syncthreads();
    if (warp == 0) tmem_dealloc(taddr, 32);
}

// fixed-order FP64 sum of the split partials, times the kick factor: one
// warp per (kick, slice), lanes over the splits, then a fixed shuffle tree
__global__ void wake_tc_reduce_kernel(const __grid_constant__ phk_wake_tc w) {
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int S = w.n_slices;
    const int k = gw / S, i = gw - k * S;
    if (k >= w.n_kicks) return;
    const int64_t rows = (int64_t)w.m_tiles * kTcM;
    const int64_t stride = (int64_t)w.n_kicks * rows;
    const float* p = w.partials + k * rows + i;
    double acc = 0.0;
    for (int sp = lane; sp < w.splits; sp += 32) acc += (double)p[sp * stride];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane != 0) return;
    const double r = w.factor[k] * acc;
    if (w.out_dtype == PHK_F64)
        reinterpret_cast<double*>(w.out[k])[i] = r;
    else
        reinterpret_cast<float*>(w.out[k])[i] = (float)r;
}

size_t wake_tc_smem() {
    return kTcStages * 2 * kTcTileBytes + kTcMaxChunks * kTcBBytes +
           (kTcStages + 1) * 8 + 16;
}

// K layout, tiles and split of a GEMM (fills k_total, m_tiles, splits and
// group_k0 of w from n_slices, n_groups and group_lags)
int plan_wake_tc(phk_wake_tc* w, int64_t* a_elems, int64_t* partial_elems) {
    int64_t k = 0;
    for (int g = 0; g < w->n_groups; ++g) {
        w->group_k0[g] = (int32_t)k;
        k += (int64_t)w->group_lags[g] * lag_cols(w->n_slices);
    }
    k = (k + kTcK - 1) / kTcK * kTcK;
    if (k > (int64_t)1 << 30)
        return set_error(PHK_ESIZE, "phk_wake_tc_plan: K = %lld too large",
                         (long long)k);
    w->k_total = (int32_t)k;
    w->m_tiles = (w->n_slices + kTcM - 1) / kTcM;
    const int chunks = (int)(k / kTcK);
    // two CTAs per SM, at most kTcMaxChunks chunks per CTA
    int splits = 2 * device_info().sm_count / w->m_tiles;
    if (splits > chunks / 2) splits = chunks / 2;
    const int need = (chunks + kTcMaxChunks - 1) / kTcMaxChunks;
    if (splits < need) splits = need;
    if (splits < 1) splits = 1;
    w->splits = splits;
    int64_t rows = 0;
    for (int g = 0; g < w->n_groups; ++g) rows += w->group_lags[g];
    if (a_elems) *a_elems = rows * row_stride(w->n_slices);
    if (partial_elems)
        *partial_elems = (int64_t)splits * w->n_kicks * w->m_tiles * kTcM;
    return PHK_OK;
}

int launch_wake_tc_expand(const phk_wake_tc* w, cudaStream_t st) {
    int64_t rows = 0;
    for (int g = 0; g < w->n_groups; ++g) rows += w->group_lags[g];
    const int64_t total = rows * row_stride(w->n_slices);
    int64_t blocks = (total + 255) / 256;
    const int64_t cap = (int64_t)device_info().sm_count * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    wake_split_kernel<<<(unsigned)blocks, 256, 0, st>>>(*w);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(PHK_ECUDA, "phk_wake_tc_expand launch: %s",
                         cudaGetErrorString(e));
    count_launches(1);
    return PHK_OK;
}

int launch_wake_tc(const phk_wake_tc* w, cudaStream_t st) {
    static int attr_done[64] = {0};
    const DeviceInfo& d = device_info();
    const int dev = d.device < 64 ? d.device : 63;
    const size_t smem = wake_tc_smem();
    if (!attr_done[dev]) {
        if (cudaFuncSetAttribute(wake_gemm_kernel,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem) != cudaSuccess) {
            cudaGetLastError();
            return set_error(PHK_ECUDA, "phk_wake_tc: shared memory attribute");
        }
        attr_done[dev] = 1;
    }
    wake_gemm_kernel<<<dim3(w->m_tiles, w->splits), kTcThreads, smem, st>>>(
        *w, wait_limit());
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(PHK_ECUDA, "phk_wake_tc launch: %s",
                         cudaGetErrorString(e));
    const int64_t threads = (int64_t)w->n_kicks * w->n_slices * 32;
    wake_tc_reduce_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(*w);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(PHK_ECUDA, "phk_wake_tc reduce launch: %s",
                         cudaGetErrorString(e));
    count_launches(2);
    return PHK_OK;
}

}  // namespace phk
