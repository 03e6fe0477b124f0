// Instantiations and launches of the track kernels for double coordinates.
#include "phk_track.cuh"

namespace phk {

int launch_track_f64(const phk_program* prog, const phk_coords* c,
                     const phk_kick_set* pk, const phk_accum* acc, int ld,
                     int stm, bool vec_ok, cudaStream_t st) {
    if (!vec_ok)
        return launch_track_t<double, 1, SHAPE_GENERIC>(prog, c, pk, acc, ld, stm, st);
    switch (program_shape(prog)) {
        case SHAPE_NONE:
            return launch_track_t<double, 2, SHAPE_NONE>(prog, c, pk, acc, ld, stm, st);
        case SHAPE_T:
            return launch_track_t<double, 2, SHAPE_T>(prog, c, pk, acc, ld, stm, st);
        case SHAPE_T_RF:
            return launch_track_t<double, 2, SHAPE_T_RF>(prog, c, pk, acc, ld, stm, st);
        case SHAPE_T_LIN:
            return launch_track_t<double, 2, SHAPE_T_LIN>(prog, c, pk, acc, ld, stm, st);
        default:
            return launch_track_t<double, 2, SHAPE_GENERIC>(prog, c, pk, acc, ld, stm, st);
    }
}

int track_clusters_f64(size_t smem) {
    return occupancy_clusters<double, 2, SHAPE_GENERIC>(smem);
}

// common program shape of every bunch of a batch (GENERIC unless all equal
// a specialised shape)
static int batch_shape(const phk_batch* bt) {
    int sh = -1;
    for (int i = 0; i < bt->n_bunches; ++i) {
        const int s = program_shape(bt->programs_host + i);
        if (sh < 0) sh = s;
        else if (s != sh) return SHAPE_GENERIC;
    }
    return sh == SHAPE_T_RF ? SHAPE_T_RF : SHAPE_GENERIC;
}

template <int THREADS>
static int launch_batch_threads(const phk_batch* bt, const phk_coords* c,
                                const phk_kick_set* pk, const phk_accum* acc,
                                int ld, int stm, cudaStream_t st) {
    if (batch_shape(bt) == SHAPE_T_RF)
        return launch_batch_t<double, 2, THREADS, SHAPE_T_RF>(bt, c, pk, acc, ld, stm, st);
    return launch_batch_t<double, 2, THREADS, SHAPE_GENERIC>(bt, c, pk, acc, ld, stm, st);
}

int launch_batch_f64(const phk_batch* bt, const phk_coords* c,
                     const phk_kick_set* pk, const phk_accum* acc, int ld,
                     int stm, cudaStream_t st) {
    switch (bt->threads) {
        case 128: return launch_batch_threads<128>(bt, c, pk, acc, ld, stm, st);
        case 512: return launch_batch_threads<512>(bt, c, pk, acc, ld, stm, st);
        default: return launch_batch_threads<256>(bt, c, pk, acc, ld, stm, st);
    }
}

// occupancy of the generic instantiation (the launch bounds give every
// shape the same register cap)
int batch_per_sm_f64(int threads, size_t smem) {
    return threads == 128   ? batch_occupancy<double, 2, 128, SHAPE_GENERIC>(smem)
           : threads == 512 ? batch_occupancy<double, 2, 512, SHAPE_GENERIC>(smem)
                            : batch_occupancy<double, 2, 256, SHAPE_GENERIC>(smem);
}

}  // namespace phk
