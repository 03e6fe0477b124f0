// extern "C" entry points of libphk: host-side validation of every
// argument before any launch, thread-local error messages, dispatch to the
// launchers in phk_kernels.cu.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "phk_internal.h"

namespace phk {

static thread_local char g_err[512] = "";
static std::atomic<int64_t> g_launches(0);

void count_launches(int n) { g_launches.fetch_add(n); }

static std::atomic<unsigned> g_wait_limit(kDefaultWaitLimit);

unsigned wait_limit() { return g_wait_limit.load(); }

static std::atomic<int> g_plan_variant(-1), g_plan_stages(-1), g_plan_kb(-1);

TrackPlan track_plan() {
    return TrackPlan{g_plan_variant.load(), g_plan_stages.load(), g_plan_kb.load()};
}

static std::atomic<int> g_last_variant(-1), g_last_stages(-1), g_last_smem(-1);

void note_track_launch(int variant, int stages, size_t smem) {
    g_last_variant.store(variant);
    g_last_stages.store(stages);
    g_last_smem.store((int)smem);
}

int set_error(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

const DeviceInfo& device_info() {
    static std::mutex mu;
    static std::vector<DeviceInfo> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(mu);
    for (const DeviceInfo& d : cache)
        if (d.device == dev) return d;
    DeviceInfo d;
    d.device = dev;
    cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&d.max_smem_optin,
                           cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (d.sm_count < 1) d.sm_count = 1;
    if (d.max_smem_optin < 48 * 1024) d.max_smem_optin = 48 * 1024;
    cache.push_back(d);
    return cache.back();
}

static int check_dtype(int32_t dtype, const char* who) {
    if (dtype != PHK_F64 && dtype != PHK_F32)
        return set_error(PHK_EPARAM, "%s: unknown dtype %d", who, dtype);
    return PHK_OK;
}

static size_t dsize(int32_t dtype) { return dtype == PHK_F64 ? 8 : 4; }

static int check_slicer(const phk_slicer* s, const char* who) {
    if (!s->edges) return set_error(PHK_ENULL, "%s: slicer edges is NULL", who);
    if (s->n_slices < 1 || s->n_slices > PHK_MAX_SLICES)
        return set_error(PHK_ESIZE, "%s: n_slices %d outside [1, %d]", who,
                         s->n_slices, PHK_MAX_SLICES);
    if (s->negate != 0 && s->negate != 1)
        return set_error(PHK_EPARAM, "%s: negate must be 0 or 1", who);
    return PHK_OK;
}

// a device pointer that kernels read or write with loads / stores of
// `align` bytes (NULL passes: optional outputs are checked where required)
static int check_aligned(const void* ptr, size_t align, const char* who,
                         const char* what) {
    if (reinterpret_cast<uintptr_t>(ptr) % align)
        return set_error(PHK_EALIGN, "%s: %s not %zu-byte aligned", who, what,
                         align);
    return PHK_OK;
}

// the kernels read the edge table with loads of the coordinate type
static int check_edges(const phk_slicer* s, int32_t dtype, const char* who) {
    if (reinterpret_cast<uintptr_t>(s->edges) % dsize(dtype))
        return set_error(PHK_EALIGN, "%s: slicer edges not %zu-byte aligned",
                         who, dsize(dtype));
    return PHK_OK;
}

static int check_coords(const phk_coords* c, const char* who) {
    if (!c) return set_error(PHK_ENULL, "%s: coords is NULL", who);
    int r = check_dtype(c->dtype, who);
    if (r) return r;
    if (c->n < 0) return set_error(PHK_ESIZE, "%s: n = %lld < 0", who,
                                   (long long)c->n);
    const void* p[6] = {c->x, c->xp, c->y, c->yp, c->z, c->dp};
    const size_t al = dsize(c->dtype);
    for (int q = 0; q < 6; ++q) {
        if (c->n > 0 && !p[q])
            return set_error(PHK_ENULL, "%s: coordinate %d is NULL", who, q);
        if (reinterpret_cast<uintptr_t>(p[q]) % al)
            return set_error(PHK_EALIGN, "%s: coordinate %d not %zu-byte "
                             "aligned", who, q, al);
    }
    return PHK_OK;
}

static int check_program(const phk_program* p, const char* who) {
    if (!p) return set_error(PHK_ENULL, "%s: program is NULL", who);
    if (p->n_ops < 0 || p->n_ops > PHK_MAX_OPS)
        return set_error(PHK_ESIZE, "%s: n_ops %d outside [0, %d]", who,
                         p->n_ops, PHK_MAX_OPS);
    if (p->n_det < 0 || p->n_det > PHK_MAX_DETUNERS)
        return set_error(PHK_ESIZE, "%s: n_det %d outside [0, %d]", who,
                         p->n_det, PHK_MAX_DETUNERS);
    if (reinterpret_cast<uintptr_t>(p->status) % 4)
        return set_error(PHK_EALIGN, "%s: status word not 4-byte aligned", who);
    for (int o = 0; o < p->n_ops; ++o) {
        const phk_op& op = p->op[o];
        if (op.kind < PHK_OP_TRANSVERSE || op.kind > PHK_OP_DAMPER)
            return set_error(PHK_EPARAM, "%s: op %d has unknown kind %d", who,
                             o, op.kind);
        if (op.kind == PHK_OP_DAMPER) {
            uint64_t ptr;
            memcpy(&ptr, &op.p[31], sizeof(ptr));
            if (!ptr || ptr % 8)
                return set_error(PHK_EPARAM, "%s: damper op %d has no aligned "
                                 "means pointer", who, o);
        }
        if (op.kind == PHK_OP_TRANSVERSE && (op.flags & PHK_FLAG_DETUNED)) {
            if (op.det_begin < 0 || op.det_count < 0 ||
                op.det_begin + op.det_count > p->n_det)
                return set_error(PHK_EPARAM, "%s: op %d detuner range "
                                 "[%d, +%d) outside the %d detuners", who, o,
                                 op.det_begin, op.det_count, p->n_det);
        }
    }
    for (int d = 0; d < p->n_det; ++d) {
        const phk_detuner& dt = p->det[d];
        if (dt.kind == PHK_DET_CHROMA) {
            if (dt.nx < 1 || dt.nx > PHK_MAX_POLY || dt.ny < 1 ||
                dt.ny > PHK_MAX_POLY || dt.zx < 0 || dt.zy < 0 ||
                dt.zx > 4096 || dt.zy > 4096)
                return set_error(PHK_EPARAM, "%s: detuner %d has a bad "
                                 "polynomial (nx %d ny %d zx %d zy %d)", who,
                                 d, dt.nx, dt.ny, dt.zx, dt.zy);
        } else if (dt.kind != PHK_DET_AMPLITUDE) {
            return set_error(PHK_EPARAM, "%s: detuner %d has unknown kind %d",
                             who, d, dt.kind);
        }
    }
    return PHK_OK;
}

static int check_kicks(const phk_kick_set* k, int32_t dtype, const char* who) {
    int r = check_slicer(&k->slicer, who);
    if (r) return r;
    if ((r = check_edges(&k->slicer, dtype, who))) return r;
    if (k->n_kicks < 0 || k->n_kicks > PHK_MAX_KICKS)
        return set_error(PHK_ESIZE, "%s: n_kicks %d outside [0, %d]", who,
                         k->n_kicks, PHK_MAX_KICKS);
    for (int i = 0; i < k->n_kicks; ++i) {
        if (!k->kick[i]) return set_error(PHK_ENULL, "%s: kick %d is NULL",
                                          who, i);
        if (reinterpret_cast<uintptr_t>(k->kick[i]) % dsize(dtype))
            return set_error(PHK_EALIGN, "%s: kick %d misaligned", who, i);
        const int t = k->target[i];
        if (t != PHK_XP && t != PHK_YP && t != PHK_DP)
            return set_error(PHK_EPARAM, "%s: kick %d target %d is not xp, "
                             "yp or dp", who, i, t);
        const int q = k->quad[i];
        if (q != -1 && q != PHK_X && q != PHK_Y)
            return set_error(PHK_EPARAM, "%s: kick %d quad %d is not -1, x "
                             "or y", who, i, q);
    }
    return PHK_OK;
}

static int check_accum(const phk_accum* a, const char* who) {
    int r = check_slicer(&a->slicer, who);
    if (r) return r;
    if (!a->partials) return set_error(PHK_ENULL, "%s: partials is NULL", who);
    if ((r = check_aligned(a->partials, 8, who, "partials"))) return r;
    if (a->grid < 1) return set_error(PHK_ESIZE, "%s: grid %d < 1", who,
                                      a->grid);
    const int64_t need = 3LL * a->slicer.n_slices * a->grid;
    if (a->partials_len < need)
        return set_error(PHK_EWORKSPACE, "%s: partials hold %lld doubles, "
                         "%lld needed", who, (long long)a->partials_len,
                         (long long)need);
    return PHK_OK;
}

}  // namespace phk

using namespace phk;

extern "C" {

int phk_abi_version(void) { return PHK_ABI_VERSION; }

int phk_set_wait_limit(int64_t polls) {
    g_wait_limit.store(polls < 0 ? kDefaultWaitLimit
                                 : (unsigned)(polls > 0xffffffffLL ? 0xffffffffLL
                                                                  : polls));
    return PHK_OK;
}

int phk_set_track_plan(int32_t variant, int32_t stages, int32_t smem_kb) {
    if (variant < -1 || variant > 1)
        return set_error(PHK_EPARAM, "phk_set_track_plan: variant %d", variant);
    if (stages < -1 || stages > 4 || stages == 1)
        return set_error(PHK_EPARAM, "phk_set_track_plan: stages %d", stages);
    if (smem_kb != -1 && (smem_kb < 16 || smem_kb > 227))
        return set_error(PHK_EPARAM, "phk_set_track_plan: smem_kb %d", smem_kb);
    g_plan_variant.store(variant);
    g_plan_stages.store(stages);
    g_plan_kb.store(smem_kb);
    return PHK_OK;
}

int phk_last_track_launch(int32_t* variant, int32_t* stages, int32_t* smem_bytes) {
    if (!variant || !stages || !smem_bytes)
        return set_error(PHK_ENULL, "phk_last_track_launch: null pointer");
    *variant = g_last_variant.load();
    *stages = g_last_stages.load();
    *smem_bytes = g_last_smem.load();
    return PHK_OK;
}

int64_t phk_launch_count(void) { return g_launches.load(); }

int phk_last_error(char* buf, int len) {
    const int n = (int)strlen(g_err);
    if (buf && len > 0) {
        strncpy(buf, g_err, (size_t)len - 1);
        buf[len - 1] = '\0';
    }
    return n;
}

int phk_track_grid(int64_t n, int32_t dtype, int32_t n_slices) {
    int r = check_dtype(dtype, "phk_track_grid");
    if (r) return r;
    if (n < 0) return set_error(PHK_ESIZE, "phk_track_grid: n < 0");
    if (n_slices < 1 || n_slices > PHK_MAX_SLICES)
        return set_error(PHK_ESIZE, "phk_track_grid: n_slices %d outside "
                         "[1, %d]", n_slices, PHK_MAX_SLICES);
    return track_grid(n, dtype, n_slices);
}

int phk_track(const phk_program* program, const phk_coords* coords,
              const phk_kick_set* pending, const phk_accum* acc,
              void* stream) {
    int r = check_program(program, "phk_track");
    if (r) return r;
    if ((r = check_coords(coords, "phk_track"))) return r;
    if (pending && (r = check_kicks(pending, coords->dtype, "phk_track")))
        return r;
    if (acc && (r = check_accum(acc, "phk_track"))) return r;
    if (acc && (r = check_edges(&acc->slicer, coords->dtype, "phk_track")))
        return r;
    if (coords->n == 0 && !acc) return PHK_OK;
    return launch_track(program, coords, pending, acc, (cudaStream_t)stream);
}

int phk_slice_finalize(const phk_accum* acc, int32_t* counts, double* mean_x,
                       double* mean_y, double* moments_slot, void* stream) {
    if (!acc) return set_error(PHK_ENULL, "phk_slice_finalize: acc is NULL");
    int r = check_accum(acc, "phk_slice_finalize");
    if (r) return r;
    const char* who = "phk_slice_finalize";
    if ((r = check_aligned(counts, 4, who, "counts")) ||
        (r = check_aligned(mean_x, 8, who, "mean_x")) ||
        (r = check_aligned(mean_y, 8, who, "mean_y")) ||
        (r = check_aligned(moments_slot, 8, who, "moments_slot")))
        return r;
    return launch_finalize(acc, counts, mean_x, mean_y, moments_slot,
                           (cudaStream_t)stream);
}

int phk_slice_sums(const phk_accum* acc, double* sums, void* stream) {
    if (!acc || !sums)
        return set_error(PHK_ENULL, "phk_slice_sums: acc or sums is NULL");
    int r = check_accum(acc, "phk_slice_sums");
    if (r) return r;
    if (reinterpret_cast<uintptr_t>(sums) % 8)
        return set_error(PHK_EALIGN, "phk_slice_sums: sums not 8-byte aligned");
    return launch_slice_sums(acc, sums, (cudaStream_t)stream);
}

int phk_slice_merge(const double* sums, int32_t n_shards, int32_t n_slices,
                    int32_t* counts, double* mean_x, double* mean_y,
                    double* moments_slot, void* stream) {
    if (!sums) return set_error(PHK_ENULL, "phk_slice_merge: sums is NULL");
    if (n_shards < 1 || n_shards > 65536)
        return set_error(PHK_ESIZE, "phk_slice_merge: n_shards %d", n_shards);
    if (n_slices < 1 || n_slices > PHK_MAX_SLICES)
        return set_error(PHK_ESIZE, "phk_slice_merge: n_slices %d outside "
                         "[1, %d]", n_slices, PHK_MAX_SLICES);
    if (reinterpret_cast<uintptr_t>(sums) % 8)
        return set_error(PHK_EALIGN, "phk_slice_merge: sums not 8-byte aligned");
    const char* who = "phk_slice_merge";
    int r;
    if ((r = check_aligned(counts, 4, who, "counts")) ||
        (r = check_aligned(mean_x, 8, who, "mean_x")) ||
        (r = check_aligned(mean_y, 8, who, "mean_y")) ||
        (r = check_aligned(moments_slot, 8, who, "moments_slot")))
        return r;
    return launch_slice_merge(sums, n_shards, n_slices, counts, mean_x, mean_y,
                              moments_slot, (cudaStream_t)stream);
}

int phk_wake(const phk_wake_set* w, void* stream) {
    if (!w) return set_error(PHK_ENULL, "phk_wake: wake set is NULL");
    if (w->n_slices < 1 || w->n_slices > PHK_MAX_SLICES)
        return set_error(PHK_ESIZE, "phk_wake: n_slices %d outside [1, %d]",
                         w->n_slices, PHK_MAX_SLICES);
    if (w->n_kicks < 0 || w->n_kicks > PHK_MAX_KICKS)
        return set_error(PHK_ESIZE, "phk_wake: n_kicks %d", w->n_kicks);
    if (w->ring_len < 1 || w->head < 0 || w->head >= w->ring_len)
        return set_error(PHK_EPARAM, "phk_wake: ring_len %d head %d",
                         w->ring_len, w->head);
    if (!w->moments) return set_error(PHK_ENULL, "phk_wake: moments is NULL");
    int r = check_dtype(w->out_dtype, "phk_wake");
    if (r) return r;
    if ((r = check_aligned(w->moments, 8, "phk_wake", "moments"))) return r;
    for (int k = 0; k < w->n_kicks; ++k) {
        const phk_wake_kick& kk = w->kick[k];
        if (!kk.table || !kk.out)
            return set_error(PHK_ENULL, "phk_wake: kick %d table/out NULL", k);
        if (kk.source < 0 || kk.source > 2)
            return set_error(PHK_EPARAM, "phk_wake: kick %d source %d", k,
                             kk.source);
        if (kk.n_lags < 0 || kk.n_lags > w->ring_len)
            return set_error(PHK_EPARAM, "phk_wake: kick %d uses %d lags of a "
                             "%d-slot ring", k, kk.n_lags, w->ring_len);
        if (kk.dense != 0 && kk.dense != 1)
            return set_error(PHK_EPARAM, "phk_wake: kick %d dense flag", k);
        if ((r = check_aligned(kk.table, 8, "phk_wake", "a kick table")) ||
            (r = check_aligned(kk.out, dsize(w->out_dtype), "phk_wake",
                               "a kick output")))
            return r;
    }
    if (w->n_kicks == 0) return PHK_OK;
    return launch_wake(w, (cudaStream_t)stream);
}

int phk_kick(const phk_coords* coords, const phk_kick_set* kicks,
             void* stream) {
    int r = check_coords(coords, "phk_kick");
    if (r) return r;
    if (!kicks) return set_error(PHK_ENULL, "phk_kick: kicks is NULL");
    if ((r = check_kicks(kicks, coords->dtype, "phk_kick"))) return r;
    if (coords->n == 0 || kicks->n_kicks == 0) return PHK_OK;
    phk_program empty;
    memset(&empty, 0, sizeof(empty));
    return launch_track(&empty, coords, kicks, nullptr, (cudaStream_t)stream);
}

int phk_slice_moments(const phk_slicer* slicer, const void* z, int64_t n,
                      int32_t dtype, const void* const* quantities,
                      int32_t n_q, int32_t pass, const double* means,
                      double* sums, int32_t* counts, void* stream) {
    const char* who = "phk_slice_moments";
    if (!slicer) return set_error(PHK_ENULL, "%s: slicer is NULL", who);
    int r = check_slicer(slicer, who);
    if (r) return r;
    if ((r = check_dtype(dtype, who))) return r;
    if ((r = check_edges(slicer, dtype, who))) return r;
    if (n < 0) return set_error(PHK_ESIZE, "%s: n < 0", who);
    if (n_q < 0 || n_q > 3) return set_error(PHK_ESIZE, "%s: n_q %d", who, n_q);
    if (pass != 0 && pass != 1) return set_error(PHK_EPARAM, "%s: pass", who);
    if (n > 0 && !z) return set_error(PHK_ENULL, "%s: z is NULL", who);
    if (!sums) return set_error(PHK_ENULL, "%s: sums is NULL", who);
    if (pass == 0 && !counts) return set_error(PHK_ENULL, "%s: counts", who);
    if (pass == 1 && !means) return set_error(PHK_ENULL, "%s: means", who);
    if (n_q > 0 && !quantities) return set_error(PHK_ENULL, "%s: quantities", who);
    for (int q = 0; q < n_q; ++q)
        if (n > 0 && !quantities[q])
            return set_error(PHK_ENULL, "%s: quantity %d is NULL", who, q);
    if (reinterpret_cast<uintptr_t>(z) % dsize(dtype))
        return set_error(PHK_EALIGN, "%s: z not %zu-byte aligned", who,
                         dsize(dtype));
    for (int q = 0; q < n_q; ++q)
        if (reinterpret_cast<uintptr_t>(quantities[q]) % dsize(dtype))
            return set_error(PHK_EALIGN, "%s: quantity %d not %zu-byte "
                             "aligned", who, q, dsize(dtype));
    if (n == 0) return PHK_OK;
    return launch_moments(slicer, z, n, dtype, quantities, n_q, pass, means,
                          sums, counts, (cudaStream_t)stream);
}

int phk_track_batch(const phk_batch* batch, const phk_coords* coords,
                    const phk_kick_set* pending, const phk_accum* acc,
                    void* stream) {
    const char* who = "phk_track_batch";
    if (!batch) return set_error(PHK_ENULL, "%s: batch is NULL", who);
    const phk_batch& b = *batch;
    if (b.n_bunches < 1)
        return set_error(PHK_ESIZE, "%s: n_bunches %d < 1", who, b.n_bunches);
    if (b.n_units < 0) return set_error(PHK_ESIZE, "%s: n_units < 0", who);
    if (b.grid < 1) return set_error(PHK_ESIZE, "%s: grid %d < 1", who, b.grid);
    if (b.threads != 128 && b.threads != 256 && b.threads != 512)
        return set_error(PHK_EPARAM, "%s: threads %d is not 128, 256 or 512",
                         who, b.threads);
    if (!b.units || !b.cta_first || !b.programs || !b.programs_host)
        return set_error(PHK_ENULL, "%s: units, cta_first or programs is NULL",
                         who);
    int r = check_coords(coords, who);
    if (r) return r;
    if ((r = check_aligned(b.units, 8, who, "units")) ||
        (r = check_aligned(b.cta_first, 4, who, "cta_first")) ||
        (r = check_aligned(b.programs, 8, who, "programs")) ||
        (r = check_aligned(b.kicks, dsize(coords->dtype), who, "kicks")) ||
        (r = check_aligned(b.status, 4, who, "status")))
        return r;
    const void* p[6] = {coords->x, coords->xp, coords->y, coords->yp,
                        coords->z, coords->dp};
    for (int q = 0; q < 6; ++q)
        if (reinterpret_cast<uintptr_t>(p[q]) % 16)
            return set_error(PHK_EALIGN, "%s: coordinate %d not 16-byte "
                             "aligned", who, q);
    for (int i = 0; i < b.n_bunches; ++i)
        if ((r = check_program(b.programs_host + i, who))) return r;
    if (pending) {
        if (!b.kicks)
            return set_error(PHK_ENULL, "%s: pending kicks without tables", who);
        phk_kick_set k = *pending;
        for (int i = 0; i < k.n_kicks && i < PHK_MAX_KICKS; ++i)
            k.kick[i] = b.kicks;
        if ((r = check_kicks(&k, coords->dtype, who))) return r;
        if ((size_t)k.n_kicks * k.slicer.n_slices * dsize(coords->dtype) >
            48 * 1024)
            return set_error(PHK_ESIZE, "%s: kick tables of one bunch exceed "
                             "48 KB", who);
    }
    if (acc) {
        if ((r = check_accum(acc, who))) return r;
        if ((r = check_edges(&acc->slicer, coords->dtype, who))) return r;
        if (b.n_columns < 1 || acc->grid != b.n_columns)
            return set_error(PHK_EPARAM, "%s: acc->grid %d must equal "
                             "n_columns %d >= 1", who, acc->grid, b.n_columns);
    }
    return launch_track_batch(batch, coords, pending, acc,
                              (cudaStream_t)stream);
}

int phk_batch_max_grid(int32_t dtype, int32_t threads, int32_t n_slices,
                       int32_t n_kicks) {
    const char* who = "phk_batch_max_grid";
    int r = check_dtype(dtype, who);
    if (r) return r;
    if (threads != 128 && threads != 256 && threads != 512)
        return set_error(PHK_EPARAM, "%s: threads %d", who, threads);
    if (n_slices < 1 || n_slices > PHK_MAX_SLICES)
        return set_error(PHK_ESIZE, "%s: n_slices %d", who, n_slices);
    if (n_kicks < 0 || n_kicks > PHK_MAX_KICKS)
        return set_error(PHK_ESIZE, "%s: n_kicks %d", who, n_kicks);
    const int g = batch_max_grid(dtype, threads, n_slices, n_kicks);
    if (g < 1)
        return set_error(PHK_ESIZE, "%s: configuration does not fit on an SM",
                         who);
    return g;
}

int phk_batch_finalize(const phk_accum* acc, int32_t n_bunches,
                       const int32_t* bunch_columns, int32_t* counts,
                       double* mean_x, double* mean_y, double* moments,
                       int64_t moments_stride, void* stream) {
    const char* who = "phk_batch_finalize";
    if (!acc) return set_error(PHK_ENULL, "%s: acc is NULL", who);
    int r = check_accum(acc, who);
    if (r) return r;
    if (n_bunches < 1)
        return set_error(PHK_ESIZE, "%s: n_bunches %d < 1", who, n_bunches);
    if (!bunch_columns)
        return set_error(PHK_ENULL, "%s: bunch_columns is NULL", who);
    if (moments && moments_stride < 3LL * acc->slicer.n_slices)
        return set_error(PHK_EPARAM, "%s: moments_stride %lld < 3 * n_slices",
                         who, (long long)moments_stride);
    if ((r = check_aligned(bunch_columns, 4, who, "bunch_columns")) ||
        (r = check_aligned(counts, 4, who, "counts")) ||
        (r = check_aligned(mean_x, 8, who, "mean_x")) ||
        (r = check_aligned(mean_y, 8, who, "mean_y")) ||
        (r = check_aligned(moments, 8, who, "moments")))
        return r;
    return launch_batch_finalize(acc, n_bunches, bunch_columns, counts, mean_x,
                                 mean_y, moments, moments_stride, nullptr,
                                 (cudaStream_t)stream);
}

int phk_wake_batch(const phk_wake_set* sets, int32_t n_bunches,
                   int32_t n_slices, int32_t n_kicks, void* stream) {
    const char* who = "phk_wake_batch";
    if (!sets) return set_error(PHK_ENULL, "%s: sets is NULL", who);
    if (n_bunches < 1)
        return set_error(PHK_ESIZE, "%s: n_bunches %d < 1", who, n_bunches);
    if (n_slices < 1 || n_slices > PHK_MAX_SLICES)
        return set_error(PHK_ESIZE, "%s: n_slices %d outside [1, %d]", who,
                         n_slices, PHK_MAX_SLICES);
    if (n_kicks < 0 || n_kicks > PHK_MAX_KICKS)
        return set_error(PHK_ESIZE, "%s: n_kicks %d", who, n_kicks);
    if (n_kicks == 0) return PHK_OK;
    int r = check_aligned(sets, 8, who, "sets");
    if (r) return r;
    return launch_wake_batch(sets, n_bunches, n_slices, n_kicks,
                             (cudaStream_t)stream);
}

static int check_wake_tc(const phk_wake_tc* w, const char* who, bool planned) {
    if (!w) return set_error(PHK_ENULL, "%s: w is NULL", who);
    if (w->n_slices < 1 || w->n_slices > PHK_MAX_SLICES)
        return set_error(PHK_ESIZE, "%s: n_slices %d", who, w->n_slices);
    if (w->n_groups < 1 || w->n_groups > PHK_MAX_KICKS)
        return set_error(PHK_ESIZE, "%s: n_groups %d", who, w->n_groups);
    if (w->n_kicks < 1 || w->n_kicks > PHK_MAX_KICKS)
        return set_error(PHK_ESIZE, "%s: n_kicks %d", who, w->n_kicks);
    for (int g = 0; g < w->n_groups; ++g)
        if (w->group_lags[g] < 1 || w->group_lags[g] > 4096)
            return set_error(PHK_ESIZE, "%s: group %d lags %d", who, g,
                             w->group_lags[g]);
    if (reinterpret_cast<uintptr_t>(w->status) % 4)
        return set_error(PHK_EALIGN, "%s: status word not 4-byte aligned", who);
    if (!planned) return PHK_OK;
    phk_wake_tc p = *w;
    int64_t ae = 0, pe = 0;
    int r = plan_wake_tc(&p, &ae, &pe);
    if (r) return r;
    if (p.k_total != w->k_total || p.m_tiles != w->m_tiles ||
        p.splits != w->splits)
        return set_error(PHK_EPARAM, "%s: plan fields do not match "
                         "phk_wake_tc_plan", who);
    for (int g = 0; g < w->n_groups; ++g)
        if (p.group_k0[g] != w->group_k0[g])
            return set_error(PHK_EPARAM, "%s: group_k0 does not match", who);
    if (!w->a_hi || !w->a_lo)
        return set_error(PHK_ENULL, "%s: a_hi / a_lo is NULL", who);
    if ((reinterpret_cast<uintptr_t>(w->a_hi) |
         reinterpret_cast<uintptr_t>(w->a_lo)) & 15)
        return set_error(PHK_EALIGN, "%s: a_hi / a_lo not 16-byte aligned", who);
    return PHK_OK;
}

int phk_wake_tc_plan(phk_wake_tc* w, int64_t* a_elems, int64_t* partial_elems) {
    int r = check_wake_tc(w, "phk_wake_tc_plan", false);
    if (r) return r;
    return plan_wake_tc(w, a_elems, partial_elems);
}

int phk_wake_tc_expand(const phk_wake_tc* w, void* stream) {
    const char* who = "phk_wake_tc_expand";
    int r = check_wake_tc(w, who, true);
    if (r) return r;
    for (int g = 0; g < w->n_groups; ++g)
        if (!w->tables[g])
            return set_error(PHK_ENULL, "%s: table of group %d is NULL", who, g);
    for (int g = 0; g < w->n_groups; ++g)
        if ((r = check_aligned(w->tables[g], 8, who, "a group table")))
            return r;
    return launch_wake_tc_expand(w, (cudaStream_t)stream);
}

int phk_wake_tc_run(const phk_wake_tc* w, void* stream) {
    const char* who = "phk_wake_tc_run";
    int r = check_wake_tc(w, who, true);
    if (r) return r;
    if (!w->moments || !w->partials)
        return set_error(PHK_ENULL, "%s: moments / partials is NULL", who);
    if ((r = check_aligned(w->moments, 8, who, "moments")) ||
        (r = check_aligned(w->partials, 4, who, "partials")))
        return r;
    if (w->ring_len < 1 || w->head < 0 || w->head >= w->ring_len)
        return set_error(PHK_EPARAM, "%s: ring_len %d head %d", who,
                         w->ring_len, w->head);
    if ((r = check_dtype(w->out_dtype, who))) return r;
    for (int k = 0; k < w->n_kicks; ++k) {
        if (!w->out[k]) return set_error(PHK_ENULL, "%s: out %d is NULL", who, k);
        if ((r = check_aligned(w->out[k], dsize(w->out_dtype), who, "an output")))
            return r;
        if (w->group_of[k] < 0 || w->group_of[k] >= w->n_groups)
            return set_error(PHK_EPARAM, "%s: kick %d group %d", who, k,
                             w->group_of[k]);
        if (w->source[k] < 0 || w->source[k] > 2)
            return set_error(PHK_EPARAM, "%s: kick %d source %d", who, k,
                             w->source[k]);
        if (w->n_lags[k] < 0 || w->n_lags[k] > w->ring_len)
            return set_error(PHK_EPARAM, "%s: kick %d n_lags %d", who, k,
                             w->n_lags[k]);
    }
    return launch_wake_tc(w, (cudaStream_t)stream);
}

static int check_charge_range(const void* z, int64_t n, int32_t dtype,
                              double tail, double head, int32_t K,
                              const char* who) {
    int r = check_dtype(dtype, who);
    if (r) return r;
    if (n < 0) return set_error(PHK_ESIZE, "%s: n < 0", who);
    if (n > 0 && !z) return set_error(PHK_ENULL, "%s: z is NULL", who);
    if (reinterpret_cast<uintptr_t>(z) % dsize(dtype))
        return set_error(PHK_EALIGN, "%s: z misaligned", who);
    if (!(head > tail))
        return set_error(PHK_EPARAM, "%s: head %g <= tail %g", who, head, tail);
    if (K < 1 || K > (1 << 24))
        return set_error(PHK_ESIZE, "%s: K %d outside [1, 2^24]", who, K);
    return PHK_OK;
}

int phk_charge_hist(const void* z, int64_t n, int32_t dtype, double tail,
                    double head, int32_t K, uint32_t* hist, uint64_t* below,
                    void* stream) {
    const char* who = "phk_charge_hist";
    int r = check_charge_range(z, n, dtype, tail, head, K, who);
    if (r) return r;
    if (!hist || !below)
        return set_error(PHK_ENULL, "%s: hist / below is NULL", who);
    if ((r = check_aligned(hist, 4, who, "hist")) ||
        (r = check_aligned(below, 8, who, "below")))
        return r;
    if (n == 0) return PHK_OK;
    return launch_charge_hist(z, n, dtype, tail, head, K, hist,
                              reinterpret_cast<unsigned long long*>(below),
                              (cudaStream_t)stream);
}

int phk_charge_gather(const void* z, int64_t n, int32_t dtype, double tail,
                      double head, int32_t K, const int32_t* seg_of_bin,
                      const int64_t* seg_off, const int32_t* seg_count,
                      uint32_t* fill, uint64_t* keys, int32_t* status,
                      void* stream) {
    const char* who = "phk_charge_gather";
    int r = check_charge_range(z, n, dtype, tail, head, K, who);
    if (r) return r;
    if (!seg_of_bin || !seg_off || !seg_count || !fill || !keys)
        return set_error(PHK_ENULL, "%s: a table is NULL", who);
    if ((r = check_aligned(seg_of_bin, 4, who, "seg_of_bin")) ||
        (r = check_aligned(seg_off, 8, who, "seg_off")) ||
        (r = check_aligned(seg_count, 4, who, "seg_count")) ||
        (r = check_aligned(fill, 4, who, "fill")) ||
        (r = check_aligned(keys, 8, who, "keys")) ||
        (r = check_aligned(status, 4, who, "status")))
        return r;
    if (n == 0) return PHK_OK;
    return launch_charge_gather(z, n, dtype, tail, head, K, seg_of_bin,
                                seg_off, seg_count, fill,
                                reinterpret_cast<unsigned long long*>(keys),
                                status, (cudaStream_t)stream);
}

int phk_charge_select(const uint64_t* keys, const int64_t* seg_off,
                      const int32_t* seg_count, const int32_t* tgt_seg,
                      const int32_t* tgt_rank, int32_t n_targets, double* out,
                      int32_t* status, void* stream) {
    const char* who = "phk_charge_select";
    if (n_targets < 0) return set_error(PHK_ESIZE, "%s: n_targets < 0", who);
    if (n_targets == 0) return PHK_OK;
    if (!keys || !seg_off || !seg_count || !tgt_seg || !tgt_rank || !out)
        return set_error(PHK_ENULL, "%s: a table is NULL", who);
    int r;
    if ((r = check_aligned(keys, 8, who, "keys")) ||
        (r = check_aligned(seg_off, 8, who, "seg_off")) ||
        (r = check_aligned(seg_count, 4, who, "seg_count")) ||
        (r = check_aligned(tgt_seg, 4, who, "tgt_seg")) ||
        (r = check_aligned(tgt_rank, 4, who, "tgt_rank")) ||
        (r = check_aligned(out, 8, who, "out")) ||
        (r = check_aligned(status, 4, who, "status")))
        return r;
    return launch_charge_select(
        reinterpret_cast<const unsigned long long*>(keys), seg_off, seg_count,
        tgt_seg, tgt_rank, n_targets, out, status, (cudaStream_t)stream);
}

int phk_bunch_stats_grid(int64_t n, int32_t dtype) {
    int r = check_dtype(dtype, "phk_bunch_stats_grid");
    if (r) return r;
    if (n < 0) return set_error(PHK_ESIZE, "phk_bunch_stats_grid: n < 0");
    return stats_grid(n, dtype);
}

int phk_bunch_stats(const phk_coords* coords, const phk_kick_set* pending,
                    const phk_stats* stats, void* stream) {
    const char* who = "phk_bunch_stats";
    int r = check_coords(coords, who);
    if (r) return r;
    if (pending && (r = check_kicks(pending, coords->dtype, who))) return r;
    if (!stats) return set_error(PHK_ENULL, "%s: stats is NULL", who);
    const phk_stats& s = *stats;
    if (s.order != 1 && s.order != 2)
        return set_error(PHK_EPARAM, "%s: order %d is not 1 or 2", who, s.order);
    if (s.capacity < 1)
        return set_error(PHK_ESIZE, "%s: capacity %d < 1", who, s.capacity);
    if (s.grid < 1) return set_error(PHK_ESIZE, "%s: grid %d < 1", who, s.grid);
    if (s.mask < 0 || s.mask > 0x3f)
        return set_error(PHK_EPARAM, "%s: mask 0x%x has bits beyond dp", who,
                         s.mask);
    if (!s.records || !s.partials || !s.ticket)
        return set_error(PHK_ENULL, "%s: records / partials / ticket is NULL",
                         who);
    if (reinterpret_cast<uintptr_t>(s.records) % 8 ||
        reinterpret_cast<uintptr_t>(s.partials) % 8 ||
        reinterpret_cast<uintptr_t>(s.cursor) % 8 ||
        reinterpret_cast<uintptr_t>(s.ticket) % 4 ||
        reinterpret_cast<uintptr_t>(s.means) % 8)
        return set_error(PHK_EALIGN, "%s: a workspace pointer is misaligned",
                         who);
    return launch_stats(coords, pending, stats, (cudaStream_t)stream);
}

}  // extern "C"
