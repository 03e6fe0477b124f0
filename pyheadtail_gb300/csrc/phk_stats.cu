// Bunch statistics in one pass over the coordinates (phk_bunch_stats).
//
// PyHEADTAIL evaluates every statistic of a bunch with its own pass over
// the particles: np.mean for the centroids, and for each of the up to six
// covariances behind one emittance another shifted single pass
// (cobra_functions/stats.pyx:17-45, 73-122).  Here one read-only pass
// produces the sums every statistic is a few scalar operations of:
//
//   order 1: S_q = sum_i u_q,i (plain sums; the centroids need no shift)
//   order 2: S_q = sum_i (u_q,i - u_q,0) and the 13 pair sums
//            S_ab = sum_i (u_a,i - u_a,0)(u_b,i - u_b,0) that some statistic
//            uses (within each plane, and each coordinate with dp), about
//            the reference's shift, particle 0
//
// with the pending wake kicks applied in registers.  Two kernels:
//   * sums_kernel: order 1 without kicks to apply, over the NQ requested
//     coordinates only (NQ a template parameter, so the FP64 form issues
//     one FP64 add per coordinate and particle and nothing else);
//   * stats_kernel: everything else (kicks, order 2, any alignment).
// GB300 runs FP64 at ~1/59 of its FP32 rate (measured), so the FP64 form of both is
// bound by FP64 issue, not by HBM: every FP64 instruction per particle
// costs ~17 us per 1e7 particles.
//
// Each CTA reduces its threads' values with a transposed warp reduction
// (each shuffle step halves the values a lane holds, so a warp needs V-1
// adds per lane for V values instead of 5 V) and then its warps in order;
// the last CTA to finish (ticket counter) merges the CTA rows in CTA
// order.  The record is therefore the same for every CTA schedule.
#include "phk_track.cuh"

namespace phk {

constexpr int kStatsThreads = 256;
constexpr int kStatsWarps = kStatsThreads / 32;
constexpr int kUsedPairs = 13;

// the pair sums a statistic of Particles uses: (x,x) (x,xp) (xp,xp), the
// same for y and for (z, dp), and x, xp, y, yp with dp
// (pairs p = 0..12: a = 0 0 1 2 2 3 4 4 5 0 1 2 3, b = 0 1 1 2 3 3 4 5 5 5 5 5 5)
__host__ __device__ constexpr int pair_a(int p) {
    return p <= 1 ? 0 : p == 2 ? 1 : p <= 4 ? 2 : p == 5 ? 3 : p <= 7 ? 4
         : p == 8 ? 5 : p - 9;
}
__host__ __device__ constexpr int pair_b(int p) {
    return p == 0 ? 0 : p <= 2 ? 1 : p == 3 ? 2 : p <= 5 ? 3 : p == 6 ? 4 : 5;
}

// record entry of the pair sum (a <= b)
__host__ __device__ constexpr int pair_entry(int a, int b) {
    return 13 + a * 6 - a * (a - 1) / 2 + (b - a);
}

struct StatsOut {
    double* partials;   // [grid][PHK_STATS_LEN]
    double* records;    // [capacity][PHK_STATS_LEN]
    double* means;      // optional [6] doubles + [6] floats
    int64_t* cursor;
    uint32_t* ticket;
    int64_t n;
    uint64_t entries;   // bit k: record entry k (7..33) is summed
    int32_t capacity;
    int32_t order;
};

// ------------------------------------------------------------------
// CTA reduction and the last-CTA merge

// Sum V per-thread values (V a power of two <= 32) over the warp: lane l
// ends with the warp's sum of value l >> (5 - log2 V).  Then warps in
// order into s_red[V]; returns after a __syncthreads().
template <int V>
__device__ __forceinline__ void cta_reduce(double (&v)[V], double* s_red,
                                           int lane, int warp) {
    constexpr int M = V == 1 ? 0 : V == 2 ? 1 : V == 4 ? 2 : V == 8 ? 3
                    : V == 16 ? 4 : 5;
    static_assert((1 << M) == V, "V must be a power of two <= 32");
#pragma unroll
    for (int s = 0; s < M; ++s) {
        const int off = 16 >> s;
        const int half = V >> (s + 1);
        const bool up = (lane & off) != 0;
#pragma unroll
        for (int i = 0; i < half; ++i) {
            const double send = up ? v[i] : v[i + half];
            const double keep = up ? v[i + half] : v[i];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
#pragma unroll
    for (int off = 16 >> M; off > 0; off >>= 1)
        v[0] += __shfl_xor_sync(0xffffffffu, v[0], off);
    __shared__ double s_w[kStatsWarps][32];
    if ((lane & ((32 >> M) - 1)) == 0) s_w[warp][lane >> (5 - M)] = v[0];
    __syncthreads();
    if (threadIdx.x < V) {
        double x = 0.0;
#pragma unroll
        for (int w = 0; w < kStatsWarps; ++w) x += s_w[w][threadIdx.x];
        s_red[threadIdx.x] = x;
    }
    __syncthreads();
}

// Write this CTA's row; the last CTA to arrive merges all rows in CTA
// order into the record slot, with `shift` (6 entries) and n.
__device__ __forceinline__ void merge_rows(const StatsOut& o,
                                           const double* s_red,
                                           const int* entry, int nval,
                                           const double* shift) {
    __shared__ int s_last;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid < nval)
        o.partials[(int64_t)blockIdx.x * PHK_STATS_LEN + entry[tid]] = s_red[tid];
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(o.ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const int64_t c = o.cursor ? *o.cursor : 0;
    int64_t slot = c % o.capacity;
    if (slot < 0) slot += o.capacity;
    double* rec = o.records + (int64_t)PHK_STATS_LEN * slot;
    for (int k = 7 + warp; k < PHK_STATS_LEN; k += kStatsWarps) {
        double x = 0.0;
        if ((o.entries >> k) & 1)
            for (int g = lane; g < (int)gridDim.x; g += 32)
                x += __ldcg(o.partials + (int64_t)g * PHK_STATS_LEN + k);
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
            x += __shfl_xor_sync(0xffffffffu, x, off);
        if (lane == 0) rec[k] = x;
    }
    if (tid < 6) rec[1 + tid] = shift[tid];
    if (tid == 0) rec[0] = (double)o.n;
    __syncthreads();
    if (o.means && tid < 6) {
        const double m = ((o.entries >> (7 + tid)) & 1) && o.n > 0
                             ? __dadd_rn(rec[1 + tid], __ddiv_rn(rec[7 + tid], (double)o.n))
                             : 0.0;
        o.means[tid] = m;
        reinterpret_cast<float*>(o.means + 6)[tid] = (float)m;
    }
    if (tid == 0) {
        *o.ticket = 0u;
        if (o.cursor) *o.cursor = c + 1;
    }
}

// ------------------------------------------------------------------
// order 1 over NQ coordinates, no kicks

struct SumsArgs {
    const void* c[6];   // the NQ summed coordinates, in slot order
    int32_t entry[6];   // their record entries (7 + coordinate index)
    StatsOut o;
};

template <typename T, int VEC, int NQ>
__global__ void __launch_bounds__(kStatsThreads, 4)
sums_kernel(const __grid_constant__ SumsArgs a) {
    __shared__ double s_red[8];
    __shared__ int s_entry[6];
    __shared__ double s_zero[6];
    const int tid = threadIdx.x;
    // FP64: plain sums; FP32: compensated (Kahan) sums
    T s[NQ], cmp[NQ];
#pragma unroll
    for (int k = 0; k < NQ; ++k) s[k] = cmp[k] = T(0);
    constexpr int TILE = kStatsThreads * VEC;
    const int64_t n = a.o.n;
    const int64_t n_tiles = (n + TILE - 1) / TILE;
    for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const int64_t i0 = tile * TILE + (int64_t)tid * VEC;
        const bool full = i0 + VEC <= n;
        T u[NQ][VEC];
#pragma unroll
        for (int k = 0; k < NQ; ++k) {
            const T* p = reinterpret_cast<const T*>(a.c[k]);
            if (full) {
                VecIO<T, VEC>::ld(p + i0, u[k]);
            } else {
#pragma unroll
                for (int j = 0; j < VEC; ++j) u[k][j] = i0 + j < n ? p[i0 + j] : T(0);
            }
        }
#pragma unroll
        for (int k = 0; k < NQ; ++k)
#pragma unroll
            for (int j = 0; j < VEC; ++j) {
                if (sizeof(T) == 8) {
                    s[k] += u[k][j];
                } else {
                    const T y = u[k][j] - cmp[k];
                    const T t = s[k] + y;
                    cmp[k] = (t - s[k]) - y;
                    s[k] = t;
                }
            }
    }
    double v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k)
        v[k] = k < NQ ? (double)s[k < NQ ? k : 0] - (double)cmp[k < NQ ? k : 0] : 0.0;
    if (tid < 6) {
        s_entry[tid] = tid < NQ ? a.entry[tid] : 0;
        s_zero[tid] = 0.0;
    }
    cta_reduce<8>(v, s_red, tid & 31, tid >> 5);
    merge_rows(a.o, s_red, s_entry, NQ, s_zero);
}

// ------------------------------------------------------------------
// general pass: pending kicks, masks, order 1 or 2

struct StatsArgs {
    TrackArgs t;        // coordinates, n, pending-kick staging flags
    StatsOut o;
    int32_t mask;       // coordinates summed
};

// dynamic shared memory: pending-kick edges [Sp + 1] T, then the staged
// kick tables [n_tab][Sp] T
template <typename T>
static size_t stats_smem(const phk_kick_set* pk, const TrackArgs& a) {
    if (!pk) return 0;
    const int Sp = pk->slicer.n_slices;
    int n_tab = 0;
    if (a.kick_comb)
        for (int q = 0; q < 3; ++q) n_tab += a.comb_slot[q] >= 0;
    else if (a.kicks_smem)
        n_tab = pk->n_kicks;
    return align16(sizeof(T) * (Sp + 1)) + sizeof(T) * (size_t)n_tab * Sp;
}

template <typename T, int VEC, int ORDER>
__global__ void __launch_bounds__(kStatsThreads, sizeof(T) == 4 ? 3 : 2)
stats_kernel(const __grid_constant__ phk_kick_set pk,
             const __grid_constant__ StatsArgs a) {
    // values per thread: 6 first sums (+ 13 pair sums), padded
    constexpr int NVAL = ORDER == 2 ? 6 + kUsedPairs : 6;
    constexpr int NP = ORDER == 2 ? kUsedPairs : 1;
    constexpr int V = ORDER == 2 ? 32 : 8;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ double s_red[V];
    __shared__ int s_entry[NVAL];
    __shared__ T s_shift[6];
    __shared__ double s_shiftd[6];
    const TrackArgs& ta = a.t;
    const int tid = threadIdx.x;
    const int Sp = ta.has_pk ? pk.slicer.n_slices : 0;
    T* epk = reinterpret_cast<T*>(smem);
    T* ktab = reinterpret_cast<T*>(smem + align16(sizeof(T) * (Sp + 1)));
    if (ta.has_pk) stage_pending<T>(pk, ta, epk, ktab, tid, kStatsThreads);
    __syncthreads();
    Bins<T> bpk;
    if (ta.has_pk) bpk.init(epk, Sp, pk.slicer.negate);
    vote_fast_path<T>(bpk, ta.has_pk, tid, kStatsThreads);
    const T* cp[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) cp[q] = reinterpret_cast<const T*>(ta.c[q]);

    // order 2: the shift is particle 0 as the reference holds it (kicks
    // applied); order 1 sums need none
    if (tid == 0) {
        Tile<T, 1> t0;
#pragma unroll
        for (int q = 0; q < 6; ++q)
            t0.c[q][0] = (ORDER == 2 && ta.n > 0) ? cp[q][0] : T(0);
        if (ORDER == 2 && ta.has_pk && ta.n > 0)
            apply_pending<T, 1, false>(pk, ta, bpk, ktab, t0, 0);
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            s_shift[q] = t0.c[q][0];
            s_shiftd[q] = (double)t0.c[q][0];
        }
    }
    if (tid < NVAL) {
        const int p = tid < 6 ? 0 : tid - 6;
        s_entry[tid] = tid < 6 ? 7 + tid
                               : pair_entry(pair_a(p), pair_b(p));
    }
    __syncthreads();
    T sh[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) sh[q] = s_shift[q];

    const int mask = a.mask;
    T s1[6], c1[6], s2[NP];
#pragma unroll
    for (int q = 0; q < 6; ++q) s1[q] = c1[q] = T(0);
#pragma unroll
    for (int p = 0; p < NP; ++p) s2[p] = T(0);
    constexpr int TILE = kStatsThreads * VEC;
    const int64_t n_tiles = (ta.n + TILE - 1) / TILE;
    for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
        const int64_t i0 = tile * TILE + (int64_t)tid * VEC;
        const bool full = i0 + VEC <= ta.n;
        Tile<T, VEC> t;
#pragma unroll
        for (int q = 0; q < 6; ++q) {
            if (!((ta.load_mask >> q) & 1)) {
#pragma unroll
                for (int j = 0; j < VEC; ++j) t.c[q][j] = sh[q];
            } else if (full) {
                VecIO<T, VEC>::ld(cp[q] + i0, t.c[q]);
            } else {
#pragma unroll
                for (int j = 0; j < VEC; ++j)
                    t.c[q][j] = i0 + j < ta.n ? cp[q][i0 + j] : sh[q];
            }
        }
        if (ta.has_pk) apply_pending<T, VEC, false>(pk, ta, bpk, ktab, t, i0);
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            if (!full && i0 + j >= ta.n) continue;
            T d[6];
#pragma unroll
            for (int q = 0; q < 6; ++q)
                d[q] = ORDER == 2 ? t.c[q][j] - sh[q] : t.c[q][j];
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                if (!((mask >> q) & 1)) continue;
                if (sizeof(T) == 8) {
                    s1[q] += d[q];
                } else {
                    const T y = d[q] - c1[q];
                    const T tt = s1[q] + y;
                    c1[q] = (tt - s1[q]) - y;
                    s1[q] = tt;
                }
            }
            if (ORDER == 2) {
#pragma unroll
                for (int p = 0; p < NP; ++p) {
                    const int qa = pair_a(p), qb = pair_b(p);
                    if ((mask >> qa) & (mask >> qb) & 1)
                        s2[p] = fma(d[qa], d[qb], s2[p]);
                }
            }
        }
    }
    double v[V];
#pragma unroll
    for (int k = 0; k < V; ++k) {
        const int q = k < 6 ? k : 0;
        const int p = (k >= 6 && k < NVAL) ? k - 6 : 0;
        v[k] = k < 6 ? (double)s1[q] - (double)c1[q]
                     : (k < NVAL ? (double)s2[p] : 0.0);
    }
    cta_reduce<V>(v, s_red, tid & 31, tid >> 5);
    merge_rows(a.o, s_red, s_entry, NVAL, s_shiftd);
}

// ------------------------------------------------------------------
// launches

static int opt_in_smem(const void* fn) {
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             device_info().max_smem_optin - 8 * 1024) !=
        cudaSuccess)
        cudaGetLastError();
    return 1;
}

static int finish_launch() {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(PHK_ECUDA, "phk_bunch_stats: %s", cudaGetErrorString(e));
    count_launches(1);
    return PHK_OK;
}

// CTAs of a launch: the caller's grid, at most the resident CTAs, at most
// one per tile
static unsigned launch_grid(const phk_stats* s, int64_t n, int vec,
                            int per_sm) {
    int64_t g = s->grid;
    const int64_t res = (int64_t)device_info().sm_count * per_sm;
    const int64_t tiles = (n + (int64_t)kStatsThreads * vec - 1) /
                          ((int64_t)kStatsThreads * vec);
    if (g > res) g = res;
    if (g > tiles) g = tiles;
    return (unsigned)(g < 1 ? 1 : g);
}

static StatsOut stats_out(const phk_coords* c, const phk_stats* s) {
    StatsOut o;
    o.partials = s->partials;
    o.records = s->records;
    o.means = s->means;
    o.cursor = s->cursor;
    o.ticket = s->ticket;
    o.n = c->n;
    o.capacity = s->capacity;
    o.order = s->order;
    o.entries = 0;
    return o;
}

template <typename T, int VEC, int NQ>
static int launch_sums_nq(const SumsArgs& a, const phk_stats* s,
                          cudaStream_t st) {
    const unsigned g = launch_grid(s, a.o.n, VEC, 4);
    sums_kernel<T, VEC, NQ><<<g, kStatsThreads, 0, st>>>(a);
    return finish_launch();
}

template <typename T, int VEC>
static int launch_sums(const phk_coords* c, const phk_stats* s, int mask,
                       cudaStream_t st) {
    SumsArgs a;
    memset(&a, 0, sizeof(a));
    a.o = stats_out(c, s);
    void* ptrs[6] = {c->x, c->xp, c->y, c->yp, c->z, c->dp};
    int nq = 0;
    for (int q = 0; q < 6; ++q) {
        if (!((mask >> q) & 1)) continue;
        a.c[nq] = ptrs[q];
        a.entry[nq] = 7 + q;
        a.o.entries |= 1ull << (7 + q);
        ++nq;
    }
    switch (nq) {
        case 1: return launch_sums_nq<T, VEC, 1>(a, s, st);
        case 2: return launch_sums_nq<T, VEC, 2>(a, s, st);
        case 3: return launch_sums_nq<T, VEC, 3>(a, s, st);
        case 4: return launch_sums_nq<T, VEC, 4>(a, s, st);
        case 5: return launch_sums_nq<T, VEC, 5>(a, s, st);
        default: return launch_sums_nq<T, VEC, 6>(a, s, st);
    }
}

template <typename T, int VEC, int ORDER>
static int launch_stats_t(const phk_coords* c, const phk_kick_set* pk,
                          const phk_stats* s, int mask, int load_mask,
                          cudaStream_t st) {
    StatsArgs a;
    memset(&a, 0, sizeof(a));
    TrackArgs& t = a.t;
    t.c[0] = c->x; t.c[1] = c->xp; t.c[2] = c->y;
    t.c[3] = c->yp; t.c[4] = c->z; t.c[5] = c->dp;
    t.n = c->n;
    t.has_pk = pk != nullptr;
    t.load_mask = load_mask;
    plan_kick_tables<T>(pk, &t);
    a.o = stats_out(c, s);
    a.mask = mask;
    for (int q = 0; q < 6; ++q)
        if ((mask >> q) & 1) a.o.entries |= 1ull << (7 + q);
    if (ORDER == 2)
        for (int p = 0; p < kUsedPairs; ++p)
            if ((mask >> pair_a(p)) & (mask >> pair_b(p)) & 1)
                a.o.entries |= 1ull << pair_entry(pair_a(p), pair_b(p));
    const size_t smem = stats_smem<T>(pk, t);
    static int opted[64] = {0};
    const int dev = device_info().device < 64 ? device_info().device : 63;
    if (!opted[dev])
        opted[dev] = opt_in_smem((const void*)stats_kernel<T, VEC, ORDER>);
    static phk_kick_set zero_pk;
    const unsigned g = launch_grid(s, c->n, VEC, sizeof(T) == 4 ? 3 : 2);
    stats_kernel<T, VEC, ORDER><<<g, kStatsThreads, smem, st>>>(
        pk ? *pk : zero_pk, a);
    return finish_launch();
}

int stats_grid(int64_t n, int32_t dtype) {
    (void)dtype;
    // the largest grid any of the kernels launches (sums_kernel: 4 per SM,
    // at least 512 particles per CTA)
    const int64_t per_cta = (int64_t)kStatsThreads * 2;
    int64_t g = (int64_t)device_info().sm_count * 4;
    const int64_t need = (n + per_cta - 1) / per_cta;
    if (need < g) g = need;
    return g < 1 ? 1 : (int)g;
}

// Coordinates a stats pass must load: the summed ones, plus z (slice
// lookup) and x, y (quadrupolar kicks) when kicks are applied.
static int stats_load_mask(const phk_kick_set* pk, int mask) {
    int ld = mask;
    if (pk) {
        ld |= 1 << PHK_Z;
        for (int k = 0; k < pk->n_kicks; ++k)
            if (pk->quad[k] >= 0) ld |= (1 << PHK_X) | (1 << PHK_Y);
    }
    return ld;
}

int launch_stats(const phk_coords* c, const phk_kick_set* pk,
                 const phk_stats* s, cudaStream_t st) {
    const int mask = s->mask ? s->mask : 0x3f;
    // kicks that change no summed coordinate need not be applied
    if (pk) {
        int kicked = 0;
        for (int k = 0; k < pk->n_kicks; ++k) kicked |= 1 << pk->target[k];
        if (!(mask & kicked)) pk = nullptr;
    }
    const int ld = stats_load_mask(pk, mask);
    uintptr_t align = 0;
    void* ptrs[6] = {c->x, c->xp, c->y, c->yp, c->z, c->dp};
    for (int q = 0; q < 6; ++q)
        if ((ld >> q) & 1) align |= reinterpret_cast<uintptr_t>(ptrs[q]);
    const bool a16 = (align & 15) == 0;
    if (c->dtype == PHK_F64) {
        if (s->order == 1) {
            if (!pk && a16) return launch_sums<double, 2>(c, s, mask, st);
            return launch_stats_t<double, 1, 1>(c, pk, s, mask, ld, st);
        }
        // one particle at a time: the 19 FP64 sums leave no registers for
        // a second one
        return launch_stats_t<double, 1, 2>(c, pk, s, mask, ld, st);
    }
    const bool a8 = (align & 7) == 0;
    if (s->order == 1) {
        if (!pk && a16) return launch_sums<float, 4>(c, s, mask, st);
        return a8 ? launch_stats_t<float, 2, 1>(c, pk, s, mask, ld, st)
                  : launch_stats_t<float, 1, 1>(c, pk, s, mask, ld, st);
    }
    return a8 ? launch_stats_t<float, 2, 2>(c, pk, s, mask, ld, st)
              : launch_stats_t<float, 1, 2>(c, pk, s, mask, ld, st);
}

}  // namespace phk
