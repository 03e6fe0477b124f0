// Slicing pass that needs no caller workspace: the per-cluster partial
// sums live in a file-scope device array owned by the library.
//
// Who needs it: callers that cannot allocate device memory -- for example a
// host program that reaches the library through a foreign-function layer
// holding only raw device pointers handed to it by another runtime, without
// a device allocator of its own to size a workspace, or a process whose
// device memory is owned by another runtime's pool under a fixed budget.
// They pass the coordinates and the output arrays; nothing else.
//
// Limits and sharing: at most kNoAllocMaxSlices slices; the pass uses at most
// kNoAllocMaxColumns partial columns (larger grids are clamped; the kernel's
// tile loop covers any grid).  The array (1.5 MiB) is loaded with the
// library on every device that uses it and stays there until the process
// exits.  Every call on a device shares it and it keeps the last call's
// contents; each call rewrites every column it reads, so nothing needs
// clearing, but calls whose kernels overlap on the GPU (different streams
// without ordering) race on it.
#include <cuda_runtime.h>
#include <string.h>

#include "phk_internal.h"

namespace phk {

constexpr int kNoAllocMaxSlices = 512;
constexpr int kNoAllocMaxColumns = 128;

static __device__ __align__(256) double
    g_noalloc_partials[3 * kNoAllocMaxSlices * kNoAllocMaxColumns];

// Device address of g_noalloc_partials in the current device's context,
// looked up on every call (a cached address would go stale when the context
// is destroyed and recreated, and the lookup costs far less than the pass).
// The host-side symbol is only a stand-in and must never reach a kernel.
static double* noalloc_scratch() {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        return nullptr;
    }
    return static_cast<double*>(p);
}

}  // namespace phk

using namespace phk;

extern "C" int phk_slice_noalloc(const phk_slicer* slicer,
                                 const phk_coords* coords, int32_t* counts,
                                 double* mean_x, double* mean_y,
                                 void* stream) {
    if (!slicer || !coords)
        return set_error(PHK_ENULL, "phk_slice_noalloc: slicer or coords is "
                         "NULL");
    if (slicer->n_slices < 1 || slicer->n_slices > kNoAllocMaxSlices)
        return set_error(PHK_ESIZE, "phk_slice_noalloc: n_slices %d outside "
                         "[1, %d], the capacity of the library-owned scratch",
                         slicer->n_slices, kNoAllocMaxSlices);
    // argument errors are reported before any CUDA call
    if (!slicer->edges)
        return set_error(PHK_ENULL, "phk_slice_noalloc: slicer edges is NULL");
    if (coords->dtype != PHK_F64 && coords->dtype != PHK_F32)
        return set_error(PHK_EPARAM, "phk_slice_noalloc: unknown dtype %d",
                         coords->dtype);
    if (coords->n < 0)
        return set_error(PHK_ESIZE, "phk_slice_noalloc: n = %lld < 0",
                         (long long)coords->n);
    const size_t al = coords->dtype == PHK_F64 ? 8 : 4;
    if (reinterpret_cast<uintptr_t>(slicer->edges) % al)
        return set_error(PHK_EALIGN, "phk_slice_noalloc: slicer edges not "
                         "%zu-byte aligned", al);
    const void* xyz[3] = {coords->x, coords->y, coords->z};
    for (int q = 0; q < 3; ++q) {
        if (coords->n > 0 && !xyz[q])
            return set_error(PHK_ENULL, "phk_slice_noalloc: x, y or z is NULL");
        if (reinterpret_cast<uintptr_t>(xyz[q]) % al)
            return set_error(PHK_EALIGN, "phk_slice_noalloc: x, y or z not "
                             "%zu-byte aligned", al);
    }
    // only x, y, z are read; the momenta may be passed as NULL
    phk_coords c = *coords;
    if (!c.xp) c.xp = c.x;
    if (!c.yp) c.yp = c.y;
    if (!c.dp) c.dp = c.z;
    int grid = c.n > 0 ? track_grid(c.n, c.dtype, slicer->n_slices) : 1;
    if (grid > kNoAllocMaxColumns) grid = kNoAllocMaxColumns;
    if (grid < 1) grid = 1;
    double* scratch = noalloc_scratch();
    if (!scratch)
        return set_error(PHK_ECUDA, "phk_slice_noalloc: no device address for "
                         "the scratch array on the current device");
    phk_accum acc;
    memset(&acc, 0, sizeof(acc));
    acc.slicer = *slicer;
    acc.partials = scratch;
    acc.partials_len = 3LL * kNoAllocMaxSlices * kNoAllocMaxColumns;
    acc.grid = grid;
    phk_program empty;
    memset(&empty, 0, sizeof(empty));
    // the public entry points validate every argument before any launch
    int r = phk_track(&empty, &c, nullptr, &acc, stream);
    if (r) return r;
    return phk_slice_finalize(&acc, counts, mean_x, mean_y, nullptr, stream);
}
