// Order statistics of z for UniformChargeSlicer (particles/slicing.py:
// 618-686) without sorting the bunch.
//
// The reference argsorts z and cuts the sorted bunch into slices of equal
// particle counts; the slice edges are the z values at given ranks.  Only
// those few (2 per slice) order statistics are needed, so:
//   1. charge_hist_kernel: a coarse histogram of the particles inside the
//      cuts over K uniform bins of [tail, head), and the counts below tail
//      and below head (the reference's searchsorted of the cuts);
//   2. (host) the ranks the reference needs, the coarse bin of each and the
//      rank inside that bin; the bins holding a rank become segments;
//   3. charge_gather_kernel: the order keys of the particles of those bins,
//      each into its segment (a few thousand values per segment);
//   4. charge_select_kernel: one CTA per requested rank: radix select
//      (8-bit digits, shared-memory histogram) over its segment.
// Every step is integer counting on exact keys: the values are the
// reference's z_sorted[rank] exactly (ties included).  No step writes
// outside its buffers: gather positions are checked against the segment
// sizes, digits are 8-bit; an inconsistent table sets the status word.
#include "phk_track.cuh"

namespace phk {

constexpr int kChargeThreads = 256;
constexpr int kChargeMaxSmemBins = 8192;

// coarse bin of a particle inside [tail, head): monotone in z, the same
// arithmetic in the histogram and the gather kernels
__device__ __forceinline__ int charge_bin(double z, double tail, double scale,
                                          int K) {
    const int b = (int)((z - tail) * scale);
    return b < 0 ? 0 : (b >= K ? K - 1 : b);
}

// unsigned radix key of a coordinate: order-preserving over all values
__device__ __forceinline__ unsigned long long radix_key(double v) {
    return (unsigned long long)order_key(v) ^ 0x8000000000000000ull;
}
__device__ __forceinline__ double radix_value(unsigned long long k) {
    return key_to_double((long long)(k ^ 0x8000000000000000ull));
}

template <typename T>
__global__ void __launch_bounds__(kChargeThreads)
charge_hist_kernel(const T* __restrict__ z, int64_t n, double tail,
                   double head, double scale, int K, uint32_t* hist,
                   unsigned long long* below) {
    __shared__ uint32_t sh[kChargeMaxSmemBins];
    __shared__ unsigned long long s_below[2];
    const bool use_smem = K <= kChargeMaxSmemBins;
    if (use_smem)
        for (int i = threadIdx.x; i < K; i += blockDim.x) sh[i] = 0;
    if (threadIdx.x < 2) s_below[threadIdx.x] = 0;
    __syncthreads();
    unsigned int bt = 0, bh = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double v = (double)z[i];
        const bool lt = v < tail, lh = v < head;
        bt += lt;
        bh += lh;
        if (!lt && lh) {
            const int b = charge_bin(v, tail, scale, K);
            if (use_smem) atomicAdd(sh + b, 1u);
            else atomicAdd(hist + b, 1u);
        }
    }
    // warp sums of the below counts, then one atomic per warp
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        bt += __shfl_xor_sync(0xffffffffu, bt, o);
        bh += __shfl_xor_sync(0xffffffffu, bh, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(s_below, (unsigned long long)bt);
        atomicAdd(s_below + 1, (unsigned long long)bh);
    }
    __syncthreads();
    if (use_smem)
        for (int i = threadIdx.x; i < K; i += blockDim.x)
            if (sh[i]) atomicAdd(hist + i, sh[i]);
    if (threadIdx.x < 2) atomicAdd(below + threadIdx.x, s_below[threadIdx.x]);
}

template <typename T>
__global__ void __launch_bounds__(kChargeThreads)
charge_gather_kernel(const T* __restrict__ z, int64_t n, double tail,
                     double head, double scale, int K,
                     const int32_t* __restrict__ seg_of_bin,
                     const int64_t* __restrict__ seg_off,
                     const int32_t* __restrict__ seg_count, uint32_t* fill,
                     unsigned long long* keys, int32_t* status) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double v = (double)z[i];
        if (!(v >= tail) || !(v < head)) continue;
        const int s = seg_of_bin[charge_bin(v, tail, scale, K)];
        if (s < 0) continue;
        const uint32_t pos = atomicAdd(fill + s, 1u);
        if (pos < (uint32_t)seg_count[s]) keys[seg_off[s] + pos] = radix_key(v);
        else if (status) atomicOr(status, PHK_DEV_BAD_TABLE);
    }
}

__global__ void __launch_bounds__(kChargeThreads)
charge_select_kernel(const unsigned long long* __restrict__ keys,
                     const int64_t* __restrict__ seg_off,
                     const int32_t* __restrict__ seg_count,
                     const int32_t* __restrict__ tgt_seg,
                     const int32_t* __restrict__ tgt_rank, double* out,
                     int32_t* status) {
    __shared__ uint32_t hist[256];
    __shared__ unsigned long long s_prefix;
    __shared__ uint32_t s_rank;
    const int t = blockIdx.x;
    const int s = tgt_seg[t];
    const unsigned long long* k = keys + seg_off[s];
    const int m = seg_count[s];
    if (threadIdx.x == 0) {
        s_prefix = 0ull;
        s_rank = (uint32_t)tgt_rank[t];
        if (tgt_rank[t] < 0 || tgt_rank[t] >= m) {
            if (status) atomicOr(status, PHK_DEV_BAD_TABLE);
            s_rank = 0;
        }
    }
    unsigned long long mask = 0ull;
    for (int shift = 56; shift >= 0; shift -= 8) {
        for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[i] = 0;
        __syncthreads();
        const unsigned long long prefix = s_prefix;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            const unsigned long long key = k[i];
            if ((key & mask) == prefix)
                atomicAdd(hist + (int)((key >> shift) & 255ull), 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t r = s_rank, cum = 0;
            int d = -1;
            for (int j = 0; j < 256; ++j) {
                if (r < cum + hist[j]) { d = j; break; }
                cum += hist[j];
            }
            if (d < 0) {            // rank beyond the segment: bad table
                if (status) atomicOr(status, PHK_DEV_BAD_TABLE);
                d = 0;
                cum = 0;
            }
            s_rank = r - cum;
            s_prefix = prefix | ((unsigned long long)d << shift);
        }
        mask |= 255ull << shift;
        __syncthreads();
    }
    if (threadIdx.x == 0) out[t] = radix_value(s_prefix);
}

static int charge_launch_error(const char* who) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(PHK_ECUDA, "%s: %s", who, cudaGetErrorString(e));
    return PHK_OK;
}

static unsigned charge_grid(int64_t n) {
    int64_t g = (n + kChargeThreads - 1) / kChargeThreads;
    const int64_t cap = (int64_t)device_info().sm_count * 8;
    if (g > cap) g = cap;
    return (unsigned)(g < 1 ? 1 : g);
}

int launch_charge_hist(const void* z, int64_t n, int32_t dtype, double tail,
                       double head, int32_t K, uint32_t* hist,
                       unsigned long long* below, cudaStream_t st) {
    const double scale = (double)K / (head - tail);
    const unsigned g = charge_grid(n);
    if (dtype == PHK_F64)
        charge_hist_kernel<double><<<g, kChargeThreads, 0, st>>>(
            reinterpret_cast<const double*>(z), n, tail, head, scale, K, hist,
            below);
    else
        charge_hist_kernel<float><<<g, kChargeThreads, 0, st>>>(
            reinterpret_cast<const float*>(z), n, tail, head, scale, K, hist,
            below);
    int r = charge_launch_error("phk_charge_hist");
    if (!r) count_launches(1);
    return r;
}

int launch_charge_gather(const void* z, int64_t n, int32_t dtype,
                         double tail, double head, int32_t K,
                         const int32_t* seg_of_bin, const int64_t* seg_off,
                         const int32_t* seg_count, uint32_t* fill,
                         unsigned long long* keys, int32_t* status,
                         cudaStream_t st) {
    const double scale = (double)K / (head - tail);
    const unsigned g = charge_grid(n);
    if (dtype == PHK_F64)
        charge_gather_kernel<double><<<g, kChargeThreads, 0, st>>>(
            reinterpret_cast<const double*>(z), n, tail, head, scale, K,
            seg_of_bin, seg_off, seg_count, fill, keys, status);
    else
        charge_gather_kernel<float><<<g, kChargeThreads, 0, st>>>(
            reinterpret_cast<const float*>(z), n, tail, head, scale, K,
            seg_of_bin, seg_off, seg_count, fill, keys, status);
    int r = charge_launch_error("phk_charge_gather");
    if (!r) count_launches(1);
    return r;
}

int launch_charge_select(const unsigned long long* keys,
                         const int64_t* seg_off, const int32_t* seg_count,
                         const int32_t* tgt_seg, const int32_t* tgt_rank,
                         int32_t n_targets, double* out, int32_t* status,
                         cudaStream_t st) {
    charge_select_kernel<<<n_targets, kChargeThreads, 0, st>>>(
        keys, seg_off, seg_count, tgt_seg, tgt_rank, out, status);
    int r = charge_launch_error("phk_charge_select");
    if (!r) count_launches(1);
    return r;
}

}  // namespace phk
