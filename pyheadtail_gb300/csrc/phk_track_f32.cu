// Instantiations and launches of the track kernels for float coordinates.
#include "phk_stream.cuh"

namespace phk {

template <int SHAPE, bool PK, bool ACC>
static int launch_stream_t(const StreamProg& sp, const phk_coords* c,
                           const phk_kick_set* pk, const phk_accum* acc,
                           StreamArgs a, size_t smem, cudaStream_t st) {
    a.load_mask = stream_load_bits<SHAPE, PK, ACC>();
    static int done_for[64] = {0};
    const DeviceInfo& d = device_info();
    const int dev = d.device < 64 ? d.device : 63;
    auto kern = stream_kernel<SHAPE, PK, ACC>;
    if (!done_for[dev]) {
        cudaFuncAttributes fa;
        size_t static_smem = 0;
        if (cudaFuncGetAttributes(&fa, kern) == cudaSuccess)
            static_smem = fa.sharedSizeBytes;
        else
            cudaGetLastError();
        if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 d.max_smem_optin - (int)static_smem) != cudaSuccess)
            cudaGetLastError();
        done_for[dev] = 1;
    }
    static phk_kick_set zero_pk;
    static phk_accum zero_acc;
    cudaError_t e;
    if (ACC) {
        // one partial column per cluster of kCluster CTAs
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)acc->grid * kCluster, 1, 1);
        cfg.blockDim = dim3(kStreamThreads, 1, 1);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cudaLaunchAttribute attr;
        attr.id = cudaLaunchAttributeClusterDimension;
        attr.val.clusterDim.x = kCluster;
        attr.val.clusterDim.y = 1;
        attr.val.clusterDim.z = 1;
        cfg.attrs = &attr;
        cfg.numAttrs = 1;
        e = cudaLaunchKernelEx(&cfg, kern, sp, pk ? *pk : zero_pk, *acc, a);
    } else {
        const int64_t warp_tiles = (c->n + kStreamTile - 1) / kStreamTile;
        int64_t g = (warp_tiles + kStreamWarps - 1) / kStreamWarps;
        const int64_t cap = (int64_t)d.sm_count * 4;
        if (g > cap) g = cap;
        if (g < 1) g = 1;
        kern<<<(unsigned)g, kStreamThreads, smem, st>>>(sp, pk ? *pk : zero_pk,
                                                        zero_acc, a);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess)
        return set_error(PHK_ECUDA, "phk_track launch: %s", cudaGetErrorString(e));
    count_launches(1);
    note_track_launch(1, a.stages, smem);
    return PHK_OK;
}

template <int SHAPE>
static int launch_stream_shape(const StreamProg& sp, const phk_coords* c,
                               const phk_kick_set* pk, const phk_accum* acc,
                               const StreamArgs& a, size_t smem,
                               cudaStream_t st) {
    if (pk && acc) return launch_stream_t<SHAPE, true, true>(sp, c, pk, acc, a, smem, st);
    if (pk) return launch_stream_t<SHAPE, true, false>(sp, c, pk, acc, a, smem, st);
    if (acc) return launch_stream_t<SHAPE, false, true>(sp, c, pk, acc, a, smem, st);
    return launch_stream_t<SHAPE, false, false>(sp, c, pk, acc, a, smem, st);
}

// The float parameters of a program of a streaming shape; false if its
// detuners are outside the streaming form (more than two, or a chromatic
// polynomial of order above three or with the order > 3 dp factors).
static bool stream_prog(const phk_program* prog, StreamProg* sp) {
    memset(sp, 0, sizeof(*sp));
    for (int o = 0; o < prog->n_ops && o < 4; ++o) {
        memcpy(sp->op[o], prog->op[o].p, sizeof(sp->op[o]));
        sp->flags[o] = prog->op[o].flags;
    }
    if (prog->n_ops > 0 && prog->op[0].kind == PHK_OP_TRANSVERSE) {
        const phk_op& t = prog->op[0];
        if (t.det_count > 2 || (t.det_count > 0 && t.det_begin != 0)) return false;
        sp->n_det = t.det_count;
        for (int d = 0; d < t.det_count; ++d) {
            const phk_detuner& dt = prog->det[d];
            if (dt.kind == PHK_DET_CHROMA &&
                (dt.zx || dt.zy || dt.nx < 1 || dt.nx > 3 || dt.ny < 1 || dt.ny > 3))
                return false;
            if (dt.kind != PHK_DET_CHROMA && dt.kind != PHK_DET_AMPLITUDE) return false;
            memcpy(sp->det[d], dt.c, sizeof(sp->det[d]));
            sp->det_kind[d] = dt.kind;
            sp->det_nx[d] = dt.nx;
            sp->det_ny[d] = dt.ny;
        }
    }
    return true;
}

// The streaming kernel for the cases it covers (see phk_stream.cuh);
// *handled = false leaves the launch to track_kernel.
static int launch_stream_f32(const phk_program* prog, const phk_coords* c,
                             const phk_kick_set* pk, const phk_accum* acc,
                             int ld, cudaStream_t st, bool* handled) {
    *handled = false;
    const int shape = program_shape(prog);
    if (shape == SHAPE_GENERIC) return PHK_OK;
    if (shape == SHAPE_NONE && (pk || !acc)) return PHK_OK;
    if (c->n >= ((int64_t)1 << 31) - kStreamTile) return PHK_OK;
    if (acc && acc->idx_out) return PHK_OK;
    TrackArgs plan;
    plan_kick_tables<float>(pk, &plan);
    if (pk && !plan.kick_comb) return PHK_OK;
    StreamProg sp;
    if (!stream_prog(prog, &sp)) return PHK_OK;
    const int Sa = acc ? acc->slicer.n_slices : 0;
    const int Sp = pk ? pk->slicer.n_slices : 0;
    const TrackPlan pl = track_plan();
    const size_t budget = pl.smem_kb > 0 ? (size_t)pl.smem_kb * 1024 : kStreamSmemBudget;
    size_t off[8], smem = 0;
    int stages = 0;
    if (pl.stages >= 2 && pl.stages <= kStreamMaxStages) {
        smem = stream_smem_layout(Sa, Sp, pk ? plan.n_tables : 0, pl.stages, off);
        if (smem <= budget) stages = pl.stages;
    }
    for (int sg = kStreamMaxStages; !stages && sg >= 2; --sg) {
        smem = stream_smem_layout(Sa, Sp, pk ? plan.n_tables : 0, sg, off);
        if (smem <= budget) stages = sg;
    }
    if (!stages) return PHK_OK;
    StreamArgs a;
    memset(&a, 0, sizeof(a));
    a.c[0] = (float*)c->x; a.c[1] = (float*)c->xp; a.c[2] = (float*)c->y;
    a.c[3] = (float*)c->yp; a.c[4] = (float*)c->z; a.c[5] = (float*)c->dp;
    a.n = c->n;
    a.stages = stages;
    a.cluster = acc ? kCluster : 1;
    a.n_tables = pk ? plan.n_tables : 0;
    for (int q = 0; q < 3; ++q) a.comb_slot[q] = pk ? plan.comb_slot[q] : -1;
    a.load_mask = ld;
    a.status = prog->status;
    a.wait_limit = wait_limit();
    *handled = true;
    switch (shape) {
        case SHAPE_NONE:
            return launch_stream_shape<SHAPE_NONE>(sp, c, pk, acc, a, smem, st);
        case SHAPE_T:
            return launch_stream_shape<SHAPE_T>(sp, c, pk, acc, a, smem, st);
        case SHAPE_T_RF:
            return launch_stream_shape<SHAPE_T_RF>(sp, c, pk, acc, a, smem, st);
        default:
            return launch_stream_shape<SHAPE_T_LIN>(sp, c, pk, acc, a, smem, st);
    }
}

int launch_track_f32(const phk_program* prog, const phk_coords* c,
                     const phk_kick_set* pk, const phk_accum* acc, int ld,
                     int stm, bool vec_ok, cudaStream_t st) {
    if (vec_ok && track_plan().variant == 1) {
        bool handled = false;
        const int r = launch_stream_f32(prog, c, pk, acc, ld, st, &handled);
        if (handled) return r;
    }
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
        return launch_batch_t<float, kF32Vec, THREADS, SHAPE_T_RF>(bt, c, pk, acc, ld, stm, st);
    return launch_batch_t<float, kF32Vec, THREADS, SHAPE_GENERIC>(bt, c, pk, acc, ld, stm, st);
}

int launch_batch_f32(const phk_batch* bt, const phk_coords* c,
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
int batch_per_sm_f32(int threads, size_t smem) {
    return threads == 128   ? batch_occupancy<float, kF32Vec, 128, SHAPE_GENERIC>(smem)
           : threads == 512 ? batch_occupancy<float, kF32Vec, 512, SHAPE_GENERIC>(smem)
                            : batch_occupancy<float, kF32Vec, 256, SHAPE_GENERIC>(smem);
}

}  // namespace phk
