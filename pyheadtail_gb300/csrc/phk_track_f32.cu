// Instantiations and launches of the track kernels for float coordinates.
#include "phk_track.cuh"

namespace phk {

int launch_track_f32(const phk_program* prog, const phk_coords* c,
                     const phk_kick_set* pk, const phk_accum* acc, int ld,
                     int stm, bool vec_ok, cudaStream_t st) {
    if (!vec_ok)
        return launch_track_t<float, 1, SHAPE_GENERIC>(prog, c, pk, acc, ld, stm, st);
    switch (program_shape(prog)) {
        case SHAPE_NONE:
            return launch_track_t<float, kF32Vec, SHAPE_NONE>(prog, c, pk, acc, ld, stm, st);
        case SHAPE_T:
            return launch_track_t<float, kF32Vec, SHAPE_T>(prog, c, pk, acc, ld, stm, st);
        case SHAPE_T_RF:
            return launch_track_t<float, kF32Vec, SHAPE_T_RF>(prog, c, pk, acc, ld, stm, st);
        case SHAPE_T_LIN:
            return launch_track_t<float, kF32Vec, SHAPE_T_LIN>(prog, c, pk, acc, ld, stm, st);
        default:
            return launch_track_t<float, kF32Vec, SHAPE_GENERIC>(prog, c, pk, acc, ld, stm, st);
    }
}

int track_clusters_f32(size_t smem) {
    return occupancy_clusters<float, kF32Vec, SHAPE_GENERIC>(smem);
}

int launch_batch_f32(const phk_batch* bt, const phk_coords* c,
                     const phk_kick_set* pk, const phk_accum* acc, int ld,
                     int stm, cudaStream_t st) {
    switch (bt->threads) {
        case 128: return launch_batch_t<float, 4, 128>(bt, c, pk, acc, ld, stm, st);
        case 512: return launch_batch_t<float, 4, 512>(bt, c, pk, acc, ld, stm, st);
        default: return launch_batch_t<float, 4, 256>(bt, c, pk, acc, ld, stm, st);
    }
}

int batch_per_sm_f32(int threads, size_t smem) {
    return threads == 128   ? batch_occupancy<float, 4, 128>(smem)
           : threads == 512 ? batch_occupancy<float, 4, 512>(smem)
                            : batch_occupancy<float, 4, 256>(smem);
}

}  // namespace phk
