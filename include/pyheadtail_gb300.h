/*
 * pyheadtail_gb300.h -- C ABI of the GB300 (sm_103a) single-bunch turn loop.
 *
 * The library replaces the per-particle arithmetic of PyHEADTAIL's turn loop
 * (v1.16.5) behind plain C entry points: device pointers, sizes and POD
 * parameter blocks, no torch or C++ types.  Every call is asynchronous on the
 * caller's CUDA stream (passed as void*, a cudaStream_t), allocates no
 * device memory at run time (every buffer belongs to the caller, except the
 * fixed scratch array of phk_slice_noalloc, which is loaded with the
 * library) and returns an int status:
 *   0      success
 *   < 0    argument error detected on the host before any launch
 *          (PHK_E* below); the message is available from phk_last_error()
 *   > 0    never returned by a call; device-side errors (PHK_DEV_*) are
 *          written to the optional status word of phk_program.
 *
 * Citations are path:line in the PyHEADTAIL source tree.
 *
 * The reference's own native seam for the GPU path is a ctypes binding of
 * raw device pointers + lengths with no error reporting
 * (PyHEADTAIL/gpu/thrust_interface.py:5-30, 233-269); the entry points below
 * take its place for the hot path, and the PyHEADTAIL-shaped Python classes
 * in pyheadtail_gb300/ drive them.
 */
#ifndef PYHEADTAIL_GB300_H
#define PYHEADTAIL_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PHK_ABI_VERSION 1

/* status codes */
#define PHK_OK 0
#define PHK_ENULL (-1)      /* a required pointer is NULL                  */
#define PHK_ESIZE (-2)      /* a size / count is out of range              */
#define PHK_EALIGN (-3)     /* a pointer is not aligned for its dtype      */
#define PHK_EPARAM (-4)     /* a parameter block is inconsistent           */
#define PHK_ECUDA (-5)      /* the CUDA runtime reported a launch error    */
#define PHK_EWORKSPACE (-6) /* a caller workspace is too small             */

/* coordinate storage types */
#define PHK_F64 0 /* plain form: FP64 coordinates, FP64 arithmetic          */
#define PHK_F32 1 /* precision form: FP32 coordinates, float-float phases */

/* limits of the parameter blocks */
#define PHK_MAX_OPS 12
#define PHK_MAX_DETUNERS 6
#define PHK_MAX_POLY 8
#define PHK_MAX_KICKS 8
#define PHK_MAX_SLICES 4096

/* coordinate indices (phk_kick_set.target / .quad) */
#define PHK_X 0
#define PHK_XP 1
#define PHK_Y 2
#define PHK_YP 3
#define PHK_Z 4
#define PHK_DP 5

/* ---- particle coordinates: Particles SoA, particles/particles.py:16-57,
 *      217-229.  Six device arrays of n elements of `dtype`.             */
typedef struct phk_coords {
    void *x, *xp, *y, *yp, *z, *dp;
    int64_t n;
    int32_t dtype; /* PHK_F64 | PHK_F32 */
    int32_t reserved;
} phk_coords;

/* ---- uniform-bin slicer: UniformBinSlicer.compute_sliceset_kwargs,
 *      particles/slicing.py:599-615.
 * The slice index of a particle is the reference's
 *     int32(floor((z - tail) / width)),  width = (head - tail) / n_slices.
 * `edges` holds, in the coordinate dtype, the n_slices+1 exact lower
 * boundaries e_k = min{ z : floor((z - tail)/width) >= k } (computed by the
 * host from that very formula); a particle is inside the cuts iff
 * e_0 <= z < e_S and its index is the k with e_k <= z < e_{k+1}.  For
 * width < 0 (tail > head, slicing.py:334-337) the tables are built for -z
 * and `negate` is 1.  `tail`/`width` are the reference's unmirrored values,
 * used only for particles outside the cuts when an index array is written.
 */
typedef struct phk_slicer {
    int32_t n_slices;
    int32_t negate;
    double tail;      /* z_cut_tail                                      */
    double width;     /* slice width (may be negative)                   */
    double est_tail;  /* mirrored tail (for the first index estimate)    */
    double est_inv_w; /* 1 / |width|                                     */
    const void *edges; /* device, n_slices + 1 entries of the coords dtype */
} phk_slicer;

/* ---- element programs --------------------------------------------------
 * A program is the element sequence of one (part of a) turn, applied to
 * every particle in one pass.  Parameters are host-computed FP64 scalars
 * following the reference formulas (see each kind).                       */
#define PHK_OP_TRANSVERSE 1   /* TransverseSegmentMap.track, transverse_tracking.py:138-196 */
#define PHK_OP_DRIFT 2        /* Drift.track, longitudinal_tracking.py:107-111            */
#define PHK_OP_RF_KICK 3      /* Kick.track_*, longitudinal_tracking.py:183-203           */
#define PHK_OP_LINEAR_LONG 4  /* LinearMap.track_*, longitudinal_tracking.py:731-759      */
#define PHK_OP_SCALE_TRANS 5  /* RFSystems._shrink_transverse_emittance, :546-554         */
#define PHK_OP_DAMPER 6       /* TransverseDamper.track_*, feedback/transverse_damper.py:64-86 */

/* op flags */
#define PHK_FLAG_DISPERSION 1 /* subtract / add D * dp around the op      */
#define PHK_FLAG_DETUNED 2    /* transverse: per-particle phase advance   */
#define PHK_FLAG_SHRINK 4     /* drift: beta_ratio != 1                   */
#define PHK_FLAG_PHI_OFFSET 8 /* rf kick: add phi_offset                  */
#define PHK_FLAG_PHI_LOCK 16  /* rf kick: add _phi_lock                   */
#define PHK_FLAG_P_INC 32     /* rf kick: subtract p_increment            */
#define PHK_FLAG_DAMP_X 64    /* damper: horizontal plane active          */
#define PHK_FLAG_DAMP_Y 128   /* damper: vertical plane active            */
#define PHK_FLAG_REACTIVE 256 /* damper: local beta given (reactive part) */

/*
 * phk_op.p layout per kind (all FP64):
 *  TRANSVERSE, not detuned: p[0..7]  = M00 M01 M10 M11 M22 M23 M32 M33
 *  TRANSVERSE, detuned:     p[0..7]  = I00 I01 I10 I11 I22 I23 I32 I33
 *                           p[8..15] = J00 J01 J10 J11 J22 J23 J32 J33
 *                           p[20], p[21] = dQ_x, dQ_y;  p[22] = 2*pi
 *                           p[23..25] = phi0_x = dQ_x*2pi, sin, cos of it
 *                           p[26..28] = phi0_y, sin, cos (base of the
 *                           angle-addition evaluation of sin/cos(phase))
 *                           ij_mask bit b set <=> entry b of (I..., J...) != 0
 *                           detuners det[det_begin .. det_begin+det_count)
 *  TRANSVERSE, either:      p[16..19] = D_x_s0 D_x_s1 D_y_s0 D_y_s1
 *  DRIFT:        p[0] = beta_ratio, p[1] = eta0 (alpha_0 - gamma^-2), p[2] = length
 *  RF_KICK:      p[0] = harmonic, p[1] = 2*pi, p[2] = circumference,
 *                p[3] = phi_offset, p[4] = _phi_lock, p[5] = |q| V / (beta c),
 *                p[6] = p0 before, p[7] = p_increment, p[8] = p0 after,
 *                p[9] = D_x, p[10] = D_y, p[11] = 1/circumference,
 *                p[12] = 1/(p0 after)   (reciprocals rounded to nearest)
 *  LINEAR_LONG:  p[0] = cos(2 pi Q_s), p[1] = sin(2 pi Q_s), p[2] = longfac,
 *                p[3] = D_x, p[4] = D_y, p[5] = 1/longfac
 *  SCALE_TRANS:  p[0] = sqrt(betagamma_old / betagamma_new)
 *  DAMPER:       p[0] = gain_x sin(phase), p[1] = gain_x cos(phase),
 *                p[2] = local beta, p[3..5] the same for y; the eight bytes
 *                of p[31] hold a device pointer to the bunch means
 *                (phk_stats.means, written before the pass runs):
 *                xp -= p[0] * <xp>, then (REACTIVE) xp -= p[1] * <x> / p[2];
 *                the same for y, yp
 *
 * With PHK_F32 coordinates the same 256 bytes hold 64 floats; hi/lo pairs
 * are float-float values (hi + lo), fractions in turns have the integer part
 * removed:
 *  TRANSVERSE, not detuned: f[0..7] M hi, f[40..47] M lo
 *  TRANSVERSE, detuned:     f[0..7] I hi, f[8..15] J hi, f[40..47] I lo,
 *                           f[48..55] J lo, f[16..17] frac(dQ_x) hi/lo,
 *                           f[18..19] frac(dQ_y) hi/lo
 *  TRANSVERSE, either:      f[32..35] = D_x_s0 D_x_s1 D_y_s0 D_y_s1
 *  DRIFT:        f[0] beta_ratio hi, f[1..2] eta0 * length hi/lo,
 *                f[3] beta_ratio lo
 *  RF_KICK:      f[0..1] h / circumference hi/lo (turns per metre),
 *                f[2..3] frac((phi_offset + _phi_lock) / 2 pi) hi/lo,
 *                f[4] |q| V / (beta c) / p0_after hi, f[5] p0_before /
 *                p0_after hi, f[6] p_increment / p0_after, f[8..9] D_x, D_y,
 *                f[10..11] the lo parts of f[4] and f[5]
 *  LINEAR_LONG:  f[0..1] cos hi/lo, f[2..3] longfac * sin hi/lo, f[4..5]
 *                D_x, D_y, f[6..7] sin / longfac hi/lo
 *  SCALE_TRANS:  f[0]
 *  DAMPER:       f[0..5] as p[0..5]; p[31] as above (the float means)
 * and phk_detuner.c holds 32 floats: CHROMA as above (x from f[0], y from
 * f[8]); AMPLITUDE f[0..3] = dapp / p0, f[4..9] as above.
 */
typedef struct phk_op {
    int32_t kind;
    int32_t flags;
    int32_t det_begin;
    int32_t det_count;
    int32_t ij_mask;
    int32_t reserved;
    double p[32];
} phk_op;

/* detuners: ChromaticitySegment.detune (trackers/detuners.py:64-98) and
 * AmplitudeDetuningSegment.detune (:128-151).
 *  CHROMA: Horner coefficients c[0..nx-1] (x) and c[8..8+ny-1] (y), lowest
 *          order first, i.e. detune = (c0 + (c1 + ...)*dp)*dp; zx / zy extra
 *          factors of dp (the reference's order > 3 polyval path prepends
 *          one zero coefficient per call, detuners.py:95-97).
 *  AMPLITUDE: c[0..9] = dapp_x, dapp_y, dapp_xy, dapp_yx,
 *             (1+ax^2)/bx, 2 ax, bx, (1+ay^2)/by, 2 ay, by;  c[10] = p0,
 *             c[11] = 1/p0 (rounded to nearest)                            */
#define PHK_DET_CHROMA 1
#define PHK_DET_AMPLITUDE 2
typedef struct phk_detuner {
    int32_t kind;
    int32_t nx, ny;
    int32_t zx, zy;
    int32_t reserved;
    double c[16];
} phk_detuner;

/* status (optional, device int32): a kernel that gives up a bounded wait
 * (a bulk copy that never completed) stores PHK_DEV_TIMEOUT there, stops
 * processing, drains its copies in flight and returns; the caller reads
 * it after synchronising.  If a drain wait gives up as well (default
 * limit), the kernel stores PHK_DEV_TIMEOUT_UNDRAINED instead and returns
 * with a copy or tensor-core operation possibly still in flight: the
 * results of that launch and of later launches in the process are not to
 * be trusted, and the caller should stop using the device from this
 * process.  NULL: no report. */
#define PHK_DEV_TIMEOUT 1
#define PHK_DEV_TIMEOUT_UNDRAINED 4
typedef struct phk_program {
    int32_t n_ops;
    int32_t n_det;
    phk_op op[PHK_MAX_OPS];
    phk_detuner det[PHK_MAX_DETUNERS];
    int32_t *status;
} phk_program;

/* ---- wake kicks applied to particles: DipoleWakeKickX/Y.apply
 *      (impedances/wake_kicks.py:207-260), QuadrupoleWakeKick* (:284-361),
 *      ConstantWakeKickZ (:185-202).  For every particle inside the cuts of
 *      `slicer`, in order k = 0..n_kicks-1:
 *          target += kick_k[idx]            (quad[k] < 0)
 *          target += kick_k[idx] * quad     (quad[k] = PHK_X | PHK_Y)
 *      kick_k are device arrays of n_slices entries of the coords dtype.  */
typedef struct phk_kick_set {
    phk_slicer slicer;
    int32_t n_kicks;
    int32_t target[PHK_MAX_KICKS];
    int32_t quad[PHK_MAX_KICKS];
    const void *kick[PHK_MAX_KICKS];
} phk_kick_set;

/* ---- per-slice accumulation (Slicer.slice + add_statistics for the
 * dipole moments: slicing.py:348-381, 443-470; stats.pyx:192-253).
 * An accumulating phk_track runs `grid` thread-block clusters; each cluster
 * folds its CTAs' histograms through distributed shared memory and writes
 * its per-slice count / sum x / sum y to the partial column
 * partials[q * n_slices * grid + s * grid + column] (q = 0,1,2).  Use
 * phk_track_grid() for `grid`; size partials >= 3 * n_slices * grid.
 * Reproducibility: FP32 values are summed exactly as integers at a
 * power-of-two scale per cluster (each value rounds by at most 2^-27 of
 * the largest |value| of the cluster's first tiles), so the columns are
 * bit-identical on every launch and for every launch plan.  FP64 sums are
 * bit-identical while every warp has a private histogram copy (up to 511
 * slices with two summed kick tables, 573 without kicks, fewer with more
 * tables); beyond that, warps share copies through atomics and the last
 * bits may differ between launches.
 * idx_out (optional, int32[n]) receives the reference's slice index of
 * every particle (outside particles included; NaN -> INT32_MIN).        */
typedef struct phk_accum {
    phk_slicer slicer;
    double *partials;
    int64_t partials_len;
    int32_t *idx_out;
    int32_t grid;
    int32_t reserved;
} phk_accum;

/* ---- wake convolution: WakeKick._accumulate_source_signal + _wake_factor
 *      (wake_kicks.py:66-73, 118-139) with _convolution_numpy (:87-116) or
 *      _convolution_dot_product (:75-85).
 * moments: device ring [ring_len][3][n_slices] FP64 of (count,
 *          count*mean_x, count*mean_y) per stored SliceSet; the set of age
 *          `a` lives in slot (head - a) mod ring_len.
 * For kick k: out_k[i] = factor_k * sum_{a < n_lags_k} conv_a[i] with
 *   numpy path  (dense=0): conv_a[i] = sum_m m_a[m] * table_k[a][i + S-1 - m],
 *                          table_k[a] has 2S-1 entries
 *   dot path    (dense=1): conv_a[i] = sum_j m_a[j] * table_k[a][j][i]
 * where m_a = moments[slot(a)][source_k].  out_k has the dtype out_dtype. */
typedef struct phk_wake_kick {
    int32_t source; /* 0 count, 1 count*mean_x, 2 count*mean_y */
    int32_t n_lags;
    int32_t dense;
    int32_t reserved;
    double factor;
    const double *table;
    void *out;
} phk_wake_kick;

typedef struct phk_wake_set {
    int32_t n_slices;
    int32_t ring_len;
    int32_t head;
    int32_t n_kicks;
    int32_t out_dtype;
    int32_t reserved;
    const double *moments;
    phk_wake_kick kick[PHK_MAX_KICKS];
} phk_wake_set;

/* ---- multi-turn wake on the tensor cores (FP32 form) --------------------
 * The convolution of phk_wake (numpy path) for every kick of one WakeField
 * as one Toeplitz GEMM with split bfloat16 products (hi*hi + hi*lo + lo*hi
 * + lo*lo) accumulated in FP32 (see phk_wake_tc).  Kicks whose sampled
 * tables are equal form one table group and share its K columns.
 * Set n_slices, n_groups, group_lags (rows of each group's table) and
 * n_kicks, then phk_wake_tc_plan() fills group_k0, k_total, m_tiles,
 * splits and the sizes of a_hi / a_lo (uint16 elements each: every table
 * row, sum of group_lags x (2 S - 1)) and partials (float elements).
 * phk_wake_tc_expand() writes the bfloat16 high / low parts of tables[g]
 * (double[group_lags[g]][2 S - 1], the layout of phk_wake_kick.table) to
 * a_hi / a_lo; repeat it whenever a table changes.  Per turn,
 * phk_wake_tc_run() reads the moment ring (as phk_wake_set), builds the
 * Toeplitz operand tiles from a_hi / a_lo in shared memory and writes
 * out[k] = factor[k] * convolution, in out_dtype. */
typedef struct phk_wake_tc {
    int32_t n_slices;
    int32_t ring_len;
    int32_t head;
    int32_t n_kicks;
    int32_t n_groups;
    int32_t k_total;
    int32_t m_tiles;
    int32_t splits;
    int32_t out_dtype;
    int32_t reserved;
    int32_t group_lags[PHK_MAX_KICKS];
    int32_t group_k0[PHK_MAX_KICKS];
    int32_t group_of[PHK_MAX_KICKS];  /* table group of each kick */
    int32_t source[PHK_MAX_KICKS];    /* 0 count, 1 count*mean_x, 2 count*mean_y */
    int32_t n_lags[PHK_MAX_KICKS];    /* stored turns each kick uses */
    double factor[PHK_MAX_KICKS];
    const double *tables[PHK_MAX_KICKS];
    void *out[PHK_MAX_KICKS];
    const double *moments;
    void *a_hi;
    void *a_lo;
    float *partials;
    int32_t *status;
} phk_wake_tc;

/* ---- batched form: many bunches in one persistent launch ---------------
 * No counterpart in the reference, which tracks one bunch per element
 * call.  The coordinates of all bunches are concatenated in one set of six
 * arrays; bunch b owns [offset_b, offset_b + n_b) with offset_b a multiple
 * of 4.  Every bunch runs its own element program (its own chromaticity,
 * detuning, RF parameters) and its own wake kicks; all bunches share one
 * slicing (same cuts and slice count).
 *
 * A work unit is particles [start, end) of one bunch (start a multiple of
 * 4).  CTA g of the persistent launch processes units cta_first[g] ..
 * cta_first[g+1]-1 in order; consecutive units of one bunch accumulate
 * into the partial column of the first of them.  Columns of bunch b are
 * the range bunch_columns[b] .. bunch_columns[b+1]-1 of phk_batch_finalize.
 * The kernel checks every table entry against the sizes below: a unit out
 * of range is skipped and PHK_DEV_BAD_TABLE is stored in *status. */
#define PHK_DEV_BAD_TABLE 2
typedef struct phk_unit {
    int64_t start;
    int64_t end;
    int32_t bunch;
    int32_t column;
} phk_unit;

typedef struct phk_batch {
    int32_t n_bunches;
    int32_t n_units;
    int32_t n_columns;
    int32_t grid;               /* CTAs of the persistent launch */
    int32_t threads;            /* 128, 256 or 512 threads per CTA */
    int32_t reserved;
    const phk_unit *units;      /* device [n_units] */
    const int32_t *cta_first;   /* device [grid + 1] */
    const phk_program *programs;      /* device [n_bunches] */
    const phk_program *programs_host; /* the same programs, host memory */
    const void *kicks;          /* device [n_bunches][n_kicks][n_slices],
                                   coords dtype; NULL without pending kicks */
    int32_t *status;            /* device word or NULL */
} phk_batch;

/* ---- bunch statistics: Particles.mean_* / sigma_* / epsn_* /
 *      dispersion_* / *_Twiss_* (particles/particles.py:311-390) from the
 *      moments of cobra_functions/stats.pyx:17-185, whose cov() is a
 *      shifted single pass with the shift a[0] (stats.pyx:34-45):
 *          cov(a, b) = (S_ab - S_a S_b / n) / (n - 1),
 *          S_a = sum_i (a_i - a_0),  S_ab = sum_i (a_i - a_0)(b_i - b_0).
 * One pass over the coordinates computes the sums every statistic needs,
 * with the pending wake kicks applied to the particles in registers: the
 * statistics of the state after the last WakeField.track while the kicks
 * stay pending for the next phk_track.  A record is PHK_STATS_LEN doubles:
 *   r[0]       n
 *   r[1..6]    shift of x, xp, y, yp, z, dp: particle 0 (kicks applied)
 *              for order 2; 0 for order 1
 *   r[7..12]   S_q = sum_i (u_q,i - shift_q), q = x, xp, y, yp, z, dp
 *   r[13..33]  S_ab for the 21 pairs a <= b in the order (x,x) (x,xp) ...
 *              (x,dp) (xp,xp) ... (dp,dp); order 2 computes the 13 pairs
 *              a statistic uses -- (x,x) (x,xp) (xp,xp), (y,y) (y,yp)
 *              (yp,yp), (z,z) (z,dp) (dp,dp), and x, xp, y, yp with dp --
 *              and writes 0 for the cross-plane ones (and order 1 for all)
 * Entries of coordinates outside `mask` are 0.  The record goes to
 * records + PHK_STATS_LEN * (c % capacity), where c is *cursor (0 when
 * cursor is NULL); the call then increments *cursor, so a captured graph
 * appends one record per replay (a negative counter counts from the end).
 * Per CTA sums are merged in a fixed order: the record is reproducible bit
 * for bit.  Calls that share partials / ticket must not run concurrently
 * (same stream, or ordered streams).  FP64 form: FP64 sums.  FP32 form:
 * per-thread compensated (Kahan) FP32 first sums and FP32 pair sums,
 * merged in FP64. */
#define PHK_STATS_LEN 34
typedef struct phk_stats {
    int32_t order;     /* 1: first sums only; 2: also the 21 pair sums    */
    int32_t capacity;  /* records in `records` (>= 1)                     */
    double *records;   /* device [capacity][PHK_STATS_LEN]                */
    int64_t *cursor;   /* device record counter, or NULL                  */
    double *partials;  /* device workspace [grid][PHK_STATS_LEN]          */
    uint32_t *ticket;  /* device word; zero before the first call, and
                          every call leaves it zero                        */
    double *means;     /* optional device [6] doubles then [6] floats:
                          shift_q + S_q / n of the summed coordinates (0
                          for the others), in FP64 and rounded to FP32   */
    int32_t grid;      /* phk_bunch_stats_grid(n, dtype)                   */
    int32_t mask;      /* coordinates to sum (bit q = PHK_X ... PHK_DP; 0:
                          all six); sums of the others are written as 0  */
} phk_stats;

/* ---------------------------------------------------------------------- */

int phk_abi_version(void);

/* Polls of a kernel's wait for its own bulk copies or tensor-core MMAs
 * before it gives up, stores PHK_DEV_TIMEOUT in its status word, waits
 * (with the default limit) for what it has in flight and returns; if that
 * drain gives up too, the status is PHK_DEV_TIMEOUT_UNDRAINED.  polls < 0
 * restores the default (2^22 polls, of the order of a second); 0 makes every
 * such wait give up at once, which exercises the failure path without any
 * fault.  Process-wide; applies to launches made after the call.  No
 * counterpart in the reference (its kernels have no waits). */
int phk_set_wait_limit(int64_t polls);

/* Launch plan of the FP32 form's single-bunch pass (phk_track with float
 * coordinates), process-wide, for launches made after the call: variant 0
 * runs the tile-shared kernel, 1 the streaming kernel (one TMA ring per
 * warp; used where the program is a transverse segment with or without
 * RFSystems / LinearMap, or no element, with summed dipolar kicks), -1
 * the default (the tile-shared kernel); stages: TMA ring stages (0, 2, 3
 * for the tile-shared kernel, 2..4 for the streaming one; -1 the largest
 * that fits); smem_kb: shared memory a CTA may plan for (16..227 KB; -1:
 * 56 KB, four CTAs per SM).  A plan that does not apply to a launch falls
 * back to the default for it.  Results are identical whatever the plan.
 * Used by the autotuner of the Python layer (pyheadtail_gb300.tuning); no
 * counterpart in the reference. */
int phk_set_track_plan(int32_t variant, int32_t stages, int32_t smem_kb);

/* The kernel variant (0 tile-shared, 1 streaming), TMA ring stages and
 * dynamic shared memory per CTA of the last single-bunch phk_track launch
 * in this process (-1 before the first); lets a caller check that a plan
 * was honoured.  No counterpart in the reference. */
int phk_last_track_launch(int32_t *variant, int32_t *stages,
                          int32_t *smem_bytes);

/* Number of kernels the library has launched in this process (all
 * devices, all threads): lets a caller verify which work ran natively. */
int64_t phk_launch_count(void);

/* Copies the calling thread's last error message (NUL-terminated, at most
 * len bytes) and returns its full length. */
int phk_last_error(char *buf, int len);

/* Number of partial columns (thread-block clusters) an accumulating
 * phk_track() uses for n particles of dtype over n_slices slices; sizes the
 * partials workspace. */
int phk_track_grid(int64_t n, int32_t dtype, int32_t n_slices);

/* The fused turn kernel.  In one pass over the particles:
 *   1. pending (optional): apply the wake kicks left by the previous
 *      WakeField.track (wake_kicks.py:221-223 and siblings);
 *   2. program: apply the element sequence (transverse segments with
 *      chromaticity / amplitude detuning, drifts, RF kicks, linear
 *      longitudinal maps, transverse shrinking);
 *   3. acc (optional): bin the updated z and accumulate per-slice count,
 *      sum x, sum y into acc->partials (and the index array).
 * Coordinates are written back iff pending or program change them.
 * Replaces TransverseSegmentMap.track, RFSystems/Drift/Kick/LinearMap.track
 * and the particle loops of Slicer.slice / mean_per_slice / the kick apply. */
int phk_track(const phk_program *program, const phk_coords *coords,
              const phk_kick_set *pending, const phk_accum *acc,
              void *stream);

/* Merge the per-CTA partials of phk_track in a fixed order into
 * counts (int32[S]), mean_x / mean_y (double[S], 0 for empty slices:
 * stats.pyx:251-253) and, if moments_slot != NULL, the wake moment ring
 * slot double[3][S] = (count, count*mean_x, count*mean_y) as in
 * wake_kicks.py:217-218.  Any output pointer may be NULL. */
int phk_slice_finalize(const phk_accum *acc, int32_t *counts, double *mean_x,
                       double *mean_y, double *moments_slot, void *stream);

/* Sharded bunch (the particles of one bunch split over several GPUs, one
 * phk_track per shard): the column sums of this shard's partials in
 * compensated form, sums = double[2][3][S]: [0][q][s] the high and
 * [1][q][s] the low part of the count (q = 0), sum x (1) and sum y (2) of
 * slice s.  Replaces, per shard, the per-slice sums of the reference's
 * slicing (particles/slicing.py:443-470, cobra_functions/stats.pyx:235-253)
 * that a sharded bunch must combine across shards. */
int phk_slice_sums(const phk_accum *acc, double *sums, void *stream);

/* Rank-ordered merge of the compensated sums of n_shards shards (device
 * double[n_shards][2][3][S], shard 0 first, e.g. gathered over the ranks
 * with an all-gather) into the outputs of phk_slice_finalize.  The totals
 * are the columns' sums to about 2^-106 of the largest partial sum, so the
 * result does not depend on how the columns are split over shards (it
 * equals one shard holding all columns except where an exact sum lies
 * within that distance of a rounding boundary). */
int phk_slice_merge(const double *sums, int32_t n_shards, int32_t n_slices,
                    int32_t *counts, double *mean_x, double *mean_y,
                    double *moments_slot, void *stream);

/* Wake convolution of every kick of `w` (see phk_wake_set). */
int phk_wake(const phk_wake_set *w, void *stream);

/* Standalone wake-kick application (when no element program follows). */
int phk_kick(const phk_coords *coords, const phk_kick_set *kicks, void *stream);

/* Per-slice moments of up to three quantities for Slicer.add_statistics
 * (slicing.py:443-529, stats.pyx:235-425), two passes:
 *   pass 0: sums[q][s] += u_q            (q < n_q), counts[s] += 1
 *   pass 1: sums[3 + pair][s] += (u_a - mean_a[s]) (u_b - mean_b[s])
 *           for the pairs (0,0) (0,1) (1,1) (0,2) (1,2) (2,2), means given
 * quantities are device arrays of the coords dtype (n entries); sums is
 * double[9][S] and counts int32[S], both accumulated (zero them first).  */
int phk_slice_moments(const phk_slicer *slicer, const void *z, int64_t n,
                      int32_t dtype, const void *const *quantities, int32_t n_q,
                      int32_t pass, const double *means, double *sums,
                      int32_t *counts, void *stream);

/* Batched fused pass (see phk_batch): per unit, the pending kicks of its
 * bunch (tables batch->kicks; `pending` gives n_kicks, quad, target and the
 * slicer, its kick[] pointers are ignored), the bunch's program, binning
 * and per-slice sums into acc->partials[3][S][batch->n_columns]
 * (acc->grid must equal n_columns).  acc may be NULL (no slicing). */
int phk_track_batch(const phk_batch *batch, const phk_coords *coords,
                    const phk_kick_set *pending, const phk_accum *acc,
                    void *stream);

/* Largest resident grid of phk_track_batch for a configuration: CTAs per
 * SM at `threads` threads x SM count (sizes the persistent launch). */
int phk_batch_max_grid(int32_t dtype, int32_t threads, int32_t n_slices,
                       int32_t n_kicks);

/* Per bunch b and slice s: fixed-order sum of the bunch's partial columns
 * (bunch_columns: device int32[n_bunches + 1]) into counts[b*S + s],
 * mean_x, mean_y (any may be NULL) and, if moments != NULL, the moment
 * ring slot moments + b * moments_stride, laid out [3][S] as in
 * phk_slice_finalize. */
int phk_batch_finalize(const phk_accum *acc, int32_t n_bunches,
                       const int32_t *bunch_columns, int32_t *counts,
                       double *mean_x, double *mean_y, double *moments,
                       int64_t moments_stride, void *stream);

/* Wake convolution of every bunch: sets is a DEVICE array of n_bunches
 * phk_wake_set (each with n_slices and at most n_kicks kicks); bunch b's
 * convolution is the one phk_wake would compute for sets[b]. */
int phk_wake_batch(const phk_wake_set *sets, int32_t n_bunches,
                   int32_t n_slices, int32_t n_kicks, void *stream);

/* Tensor-core wake (see phk_wake_tc): planning, operand expansion, and the
 * per-turn convolution of every kick. */
int phk_wake_tc_plan(phk_wake_tc *w, int64_t *a_elems, int64_t *partial_elems);
int phk_wake_tc_expand(const phk_wake_tc *w, void *stream);
int phk_wake_tc_run(const phk_wake_tc *w, void *stream);

/* Slicing pass that allocates nothing and takes no workspace; no
 * counterpart in the reference.  Same results as phk_track(empty program,
 * coords, NULL, acc) followed by phk_slice_finalize(acc, counts, mean_x,
 * mean_y, NULL): per-slice counts and centroids of x, y binned on z
 * (slicing.py:96-113, 253-262).  For callers that cannot allocate device
 * memory (a host runtime that holds only device pointers given to it, or
 * whose device memory belongs to another allocator's fixed pool).
 *   - The partial sums live in a library-owned device array of
 *     3 * 512 * 128 doubles (1.5 MiB, loaded with the library): n_slices
 *     must be <= 512, else PHK_ESIZE and nothing runs.
 *   - Its device address is looked up (cudaGetSymbolAddress) on the first
 *     call on each device, with that device current; make that first call
 *     before any stream capture.
 *   - Nothing needs zeroing: every call rewrites the part it reads.
 *   - All calls on a device share the array: calls whose kernels can
 *     overlap (different streams without ordering between them) race.
 *   - coords->xp, yp, dp are not read and may be NULL.
 * counts, mean_x, mean_y: device arrays of n_slices entries (any may be
 * NULL).  Allocates no device or host memory. */
int phk_slice_noalloc(const phk_slicer *slicer, const phk_coords *coords,
                      int32_t *counts, double *mean_x, double *mean_y,
                      void *stream);

/* ---- order statistics of z for UniformChargeSlicer
 *      (particles/slicing.py:618-686): the reference argsorts z and cuts
 *      the sorted bunch into equal-count slices; only the z values at the
 *      slice-edge ranks are needed.  Three steps, all integer counting on
 *      exact order keys (so the values are z_sorted[rank] bit for bit):
 *  phk_charge_hist: hist[b] (uint32[K], zeroed by the caller) counts the
 *    particles with tail <= z < head in bin b = clamp(int((z - tail) *
 *    K / (head - tail)), 0, K-1); below[0] += #(z < tail), below[1] +=
 *    #(z < head) (uint64[2], zeroed by the caller; NaN counts in neither).
 *  phk_charge_gather: for particles inside the cuts whose bin b has
 *    seg_of_bin[b] = s >= 0, their order keys go to keys[seg_off[s] ..
 *    + seg_count[s]) in any order (fill: uint32[n_seg], zeroed).  A
 *    segment that receives more than seg_count[s] keys sets
 *    PHK_DEV_BAD_TABLE in *status and drops the extra keys.
 *  phk_charge_select: out[t] = the tgt_rank[t]-th smallest value (0-based)
 *    of segment tgt_seg[t].
 * No counterpart of the split in the reference (it sorts the whole bunch). */
int phk_charge_hist(const void *z, int64_t n, int32_t dtype, double tail,
                    double head, int32_t K, uint32_t *hist, uint64_t *below,
                    void *stream);
int phk_charge_gather(const void *z, int64_t n, int32_t dtype, double tail,
                      double head, int32_t K, const int32_t *seg_of_bin,
                      const int64_t *seg_off, const int32_t *seg_count,
                      uint32_t *fill, uint64_t *keys, int32_t *status,
                      void *stream);
int phk_charge_select(const uint64_t *keys, const int64_t *seg_off,
                      const int32_t *seg_count, const int32_t *tgt_seg,
                      const int32_t *tgt_rank, int32_t n_targets, double *out,
                      int32_t *status, void *stream);

/* CTAs of a phk_bunch_stats launch over n particles of dtype; sizes the
 * partials workspace (grid * PHK_STATS_LEN doubles). */
int phk_bunch_stats_grid(int64_t n, int32_t dtype);

/* One statistics record of the bunch (see phk_stats): replaces the
 * particle loops of np.mean and stats.pyx cov / std / emittance /
 * dispersion / get_alpha / get_beta / get_gamma behind the Particles
 * statistics methods.  pending (optional) is the kick set that the next
 * phk_track would apply first.  Coordinates are only read. */
int phk_bunch_stats(const phk_coords *coords, const phk_kick_set *pending,
                    const phk_stats *stats, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PYHEADTAIL_GB300_H */
