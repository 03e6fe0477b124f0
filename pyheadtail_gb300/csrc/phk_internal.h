// Internal declarations shared by the translation units of libphk.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pyheadtail_gb300.h"

namespace phk {

// kernels launched by the library (phk_launch_count)
void count_launches(int n);

// polls of a first-level copy or MMA wait before a kernel gives up and
// reports PHK_DEV_TIMEOUT (phk_set_wait_limit); draining waits always use
// the default
constexpr unsigned kDefaultWaitLimit = 1u << 22;
unsigned wait_limit();

// launch plan of the FP32 single-bunch pass (phk_set_track_plan): kernel
// variant (-1 default, 0 track_kernel, 1 streaming kernel), TMA ring stages
// (-1 default) and shared-memory budget per CTA in KB (-1 default)
struct TrackPlan {
    int variant, stages, smem_kb;
};
TrackPlan track_plan();
// records the kernel variant, ring stages and shared memory of the last
// single-bunch pass launched (phk_last_track_launch)
void note_track_launch(int variant, int stages, size_t smem);

// thread-local error message, read back by phk_last_error()
int set_error(int code, const char* fmt, ...);

// device properties of the current device (cached per device)
struct DeviceInfo {
    int device;
    int sm_count;
    int max_smem_optin;
};
const DeviceInfo& device_info();

constexpr int kTrackThreads = 256;

// launchers (phk_kernels.cu); arguments already validated by phk_api.cu
int launch_track(const phk_program* prog, const phk_coords* c,
                 const phk_kick_set* pk, const phk_accum* acc,
                 cudaStream_t stream);
int track_grid(int64_t n, int32_t dtype, int32_t n_slices);
size_t track_smem_bytes(int32_t dtype, int32_t acc_slices, int32_t pk_slices);
int launch_slice_sums(const phk_accum* acc, double* out, cudaStream_t st);
int launch_slice_merge(const double* sums, int n_shards, int S,
                       int32_t* counts, double* mean_x, double* mean_y,
                       double* moments, cudaStream_t st);
int launch_finalize(const phk_accum* acc, int32_t* counts, double* mean_x,
                    double* mean_y, double* moments, cudaStream_t stream);
int launch_wake(const phk_wake_set* w, cudaStream_t stream);
int launch_moments(const phk_slicer* s, const void* z, int64_t n,
                   int32_t dtype, const void* const* q, int32_t n_q,
                   int32_t pass, const double* means, double* sums,
                   int32_t* counts, cudaStream_t stream);

int plan_wake_tc(phk_wake_tc* w, int64_t* a_elems, int64_t* partial_elems);
int launch_wake_tc_expand(const phk_wake_tc* w, cudaStream_t stream);
int launch_wake_tc(const phk_wake_tc* w, cudaStream_t stream);
int launch_track_batch(const phk_batch* b, const phk_coords* c,
                       const phk_kick_set* pk, const phk_accum* acc,
                       cudaStream_t stream);
int batch_max_grid(int32_t dtype, int32_t threads, int32_t n_slices,
                   int32_t n_kicks);
int launch_batch_finalize(const phk_accum* acc, int nb, const int32_t* bcols,
                          int32_t* counts, double* mean_x, double* mean_y,
                          double* moments, int64_t mstride, int32_t* status,
                          cudaStream_t stream);
int launch_wake_batch(const phk_wake_set* sets, int nb, int n_slices,
                      int n_kicks, cudaStream_t stream);
int stats_grid(int64_t n, int32_t dtype);
int launch_charge_hist(const void* z, int64_t n, int32_t dtype, double tail,
                       double head, int32_t K, uint32_t* hist,
                       unsigned long long* below, cudaStream_t stream);
int launch_charge_gather(const void* z, int64_t n, int32_t dtype,
                         double tail, double head, int32_t K,
                         const int32_t* seg_of_bin, const int64_t* seg_off,
                         const int32_t* seg_count, uint32_t* fill,
                         unsigned long long* keys, int32_t* status,
                         cudaStream_t stream);
int launch_charge_select(const unsigned long long* keys,
                         const int64_t* seg_off, const int32_t* seg_count,
                         const int32_t* tgt_seg, const int32_t* tgt_rank,
                         int32_t n_targets, double* out, int32_t* status,
                         cudaStream_t stream);
int launch_stats(const phk_coords* c, const phk_kick_set* pk,
                 const phk_stats* s, cudaStream_t stream);

}  // namespace phk
