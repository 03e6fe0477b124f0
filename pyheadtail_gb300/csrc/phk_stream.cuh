// The streaming form of the FP32 fused pass: the common single-bunch cases
// (one transverse segment, alone or followed by RFSystems or a linear
// longitudinal map, or no element at all; summed dipolar kicks pending or
// none; slice accumulation or none) compiled as separate kernels.
//
// Each warp streams its own warp-tiles of 64 particles (two per lane)
// through a private ring of TMA bulk copies: no block-wide barrier and no
// bookkeeping between warps in the loop.  The arithmetic is the FP32 form
// of phk_track.cuh on the paired FP32 pipes (a lane's two particles in one
// instruction, each lane the same IEEE operation in the same order as the
// scalar form, operands from the parameter bank); the partial last
// warp-tile runs the scalar form particle by particle.  The stores are
// evict-first 8-byte stores at 32-bit offsets, and the per-slice sums are
// the exact FixHist sums.  Launches outside these cases run track_kernel.
#pragma once

#include "phk_track.cuh"

namespace phk {

constexpr int kStreamWarps = 8;
constexpr int kStreamThreads = kStreamWarps * 32;
constexpr int kStreamTile = 64;          // particles per warp-tile
constexpr int kStreamMaxStages = 4;
constexpr size_t kStreamSmemBudget = 56 * 1024;


struct StreamArgs {
    float* c[6];
    int64_t n;              // < 2^31
    int32_t* status;        // phk_program.status
    int32_t stages;         // ring stages per warp
    int32_t cluster;        // CTAs per cluster (accumulating launches)
    int32_t n_tables;       // summed kick tables staged
    int32_t comb_slot[3];   // table of target xp, yp, dp (-1: none)
    int32_t load_mask;      // coordinates copied into the ring
    uint32_t wait_limit;
};

// The element program of a streaming launch as float parameters (the FP32
// layout of phk_op.p / phk_detuner.c, copied on the host), so that every
// constant is an operand read from the parameter bank.
struct StreamProg {
    float op[4][64];
    float det[2][32];        // detuners of op 0 (at most two)
    int32_t flags[4];
    int32_t det_kind[2], det_nx[2], det_ny[2];
    int32_t n_det;
    int32_t reserved;
};

// ---- scalar FP32 element arithmetic on parameter-bank operands (the
// operations of the FP32 forms in phk_track.cuh), for the partial last
// warp-tile
template <int OPI>
__device__ __forceinline__ void sp_chroma(const StreamProg& sp, int d, int q,
                                          float dp, float& dq) {
    const int n = q ? sp.det_ny[d] : sp.det_nx[d];
    const float* c = sp.det[d] + 8 * q;
    if (n == 1) dq = fmaf(c[0], dp, dq);
    else if (n == 2) dq = fmaf(fmaf(c[1], dp, c[0]), dp, dq);
    else dq = fmaf(fmaf(fmaf(c[2], dp, c[1]), dp, c[0]), dp, dq);
}

__device__ __forceinline__ void sp_detune(const StreamProg& sp, int d,
                                          const Tile<float, 1>& t, float& dqx,
                                          float& dqy) {
    if (sp.det_kind[d] == PHK_DET_CHROMA) {
        sp_chroma<0>(sp, d, 0, t.c[PHK_DP][0], dqx);
        sp_chroma<0>(sp, d, 1, t.c[PHK_DP][0], dqy);
    } else {
        const float* c = sp.det[d];
        const float x = t.c[PHK_X][0], xp = t.c[PHK_XP][0];
        const float y = t.c[PHK_Y][0], yp = t.c[PHK_YP][0];
        const float Jx = 0.5f * fmaf(c[6] * xp, xp, fmaf(c[5] * x, xp, c[4] * x * x));
        const float Jy = 0.5f * fmaf(c[9] * yp, yp, fmaf(c[8] * y, yp, c[7] * y * y));
        dqx += fmaf(c[0], Jx, c[2] * Jy);
        dqy += fmaf(c[1], Jy, c[3] * Jx);
    }
}

__device__ __forceinline__ void sp_transverse(const StreamProg& sp,
                                              Tile<float, 1>& t) {
    const float* p = sp.op[0];
    const int f = sp.flags[0];
    float& x = t.c[PHK_X][0];
    float& xp = t.c[PHK_XP][0];
    float& y = t.c[PHK_Y][0];
    float& yp = t.c[PHK_YP][0];
    const float dp = t.c[PHK_DP][0];
    float M[8], lx = 0.f, lxp = 0.f, ly = 0.f, lyp = 0.f;
    if (f & PHK_FLAG_DETUNED) {
        float dqx = 0.f, dqy = 0.f;
        if (sp.n_det > 0) sp_detune(sp, 0, t, dqx, dqy);
        if (sp.n_det > 1) sp_detune(sp, 1, t, dqx, dqy);
        float sx, cx, sy, cy;
        sincos_turns(p[16], p[17], dqx, &sx, &cx);
        sincos_turns(p[18], p[19], dqy, &sy, &cy);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            M[e] = fmaf(p[e], cx, fmaf(p[8 + e], sx, fmaf(p[40 + e], cx, p[48 + e] * sx)));
            M[4 + e] = fmaf(p[4 + e], cy, fmaf(p[12 + e], sy,
                                               fmaf(p[44 + e], cy, p[52 + e] * sy)));
        }
    } else {
#pragma unroll
        for (int e = 0; e < 8; ++e) M[e] = p[e];
    }
    if (f & PHK_FLAG_DISPERSION) {
        x = fmaf(-p[32], dp, x);
        y = fmaf(-p[34], dp, y);
    }
    if (!(f & PHK_FLAG_DETUNED)) {
        // low parts of the constant matrix
        lx = fmaf(p[40], x, p[41] * xp);
        lxp = fmaf(p[42], x, p[43] * xp);
        ly = fmaf(p[44], y, p[45] * yp);
        lyp = fmaf(p[46], y, p[47] * yp);
    }
    const float nx = fmaf(M[0], x, fmaf(M[1], xp, lx));
    const float nxp = fmaf(M[2], x, fmaf(M[3], xp, lxp));
    const float ny = fmaf(M[4], y, fmaf(M[5], yp, ly));
    const float nyp = fmaf(M[6], y, fmaf(M[7], yp, lyp));
    x = nx; xp = nxp; y = ny; yp = nyp;
    if (f & PHK_FLAG_DISPERSION) {
        x = fmaf(p[33], dp, x);
        y = fmaf(p[35], dp, y);
    }
}

template <int OPI>
__device__ __forceinline__ void sp_drift(const StreamProg& sp, Tile<float, 1>& t) {
    const float* p = sp.op[OPI];
    const float z = t.c[PHK_Z][0], dp = t.c[PHK_DP][0];
    const float zs = (sp.flags[OPI] & PHK_FLAG_SHRINK) ? fmaf(p[0], z, p[3] * z) : z;
    t.c[PHK_Z][0] = fmaf(-p[1], dp, fmaf(-p[2], dp, zs));
}

__device__ __forceinline__ void sp_rfkick(const StreamProg& sp, Tile<float, 1>& t) {
    const float* p = sp.op[2];
    const bool disp = sp.flags[2] & PHK_FLAG_DISPERSION;
    float& dp = t.c[PHK_DP][0];
    if (disp) {
        t.c[PHK_X][0] = fmaf(-p[8], dp, t.c[PHK_X][0]);
        t.c[PHK_Y][0] = fmaf(-p[9], dp, t.c[PHK_Y][0]);
    }
    const float s = sin_turns_of_product(t.c[PHK_Z][0], p[0], p[1], p[2], p[3]);
    dp = fmaf(p[4], s, fmaf(p[10], s, fmaf(dp, p[5], fmaf(dp, p[11], -p[6]))));
    if (disp) {
        t.c[PHK_X][0] = fmaf(p[8], dp, t.c[PHK_X][0]);
        t.c[PHK_Y][0] = fmaf(p[9], dp, t.c[PHK_Y][0]);
    }
}

__device__ __forceinline__ void sp_linear_long(const StreamProg& sp,
                                               Tile<float, 1>& t) {
    const float* p = sp.op[1];
    const bool disp = sp.flags[1] & PHK_FLAG_DISPERSION;
    float& z = t.c[PHK_Z][0];
    float& dp = t.c[PHK_DP][0];
    if (disp) {
        t.c[PHK_X][0] = fmaf(-p[4], dp, t.c[PHK_X][0]);
        t.c[PHK_Y][0] = fmaf(-p[5], dp, t.c[PHK_Y][0]);
    }
    const float z0 = z, dp0 = dp;
    z = fmaf(z0, p[0], fmaf(-p[2], dp0, fmaf(z0, p[1], -p[3] * dp0)));
    dp = fmaf(dp0, p[0], fmaf(p[6], z0, fmaf(dp0, p[1], p[7] * z0)));
    if (disp) {
        t.c[PHK_X][0] = fmaf(p[4], dp, t.c[PHK_X][0]);
        t.c[PHK_Y][0] = fmaf(p[5], dp, t.c[PHK_Y][0]);
    }
}

template <int SHAPE>
__device__ __forceinline__ void sp_program(const StreamProg& sp, Tile<float, 1>& t) {
    if constexpr (SHAPE == SHAPE_T) {
        sp_transverse(sp, t);
    } else if constexpr (SHAPE == SHAPE_T_RF) {
        sp_transverse(sp, t);
        sp_drift<1>(sp, t);
        sp_rfkick(sp, t);
        sp_drift<3>(sp, t);
    } else if constexpr (SHAPE == SHAPE_T_LIN) {
        sp_transverse(sp, t);
        sp_linear_long(sp, t);
    }
}

// ---- the same element arithmetic for the lane's two particles on the
// paired FP32 pipes (FFMA2 / FADD2 / FMUL2): every lane rounds as the scalar
// forms above, operation for operation
struct Pair {
    float2 c[6];
};

__device__ __forceinline__ void sp_detune_x2(const StreamProg& sp, int d,
                                             const Pair& t, float2& dqx,
                                             float2& dqy) {
    const float* c = sp.det[d];
    const float2 DP = t.c[PHK_DP];
    if (sp.det_kind[d] == PHK_DET_CHROMA) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int n = q ? sp.det_ny[d] : sp.det_nx[d];
            const float* cq = c + 8 * q;
            float2& dq = q ? dqy : dqx;
            if (n == 1) dq = fma2(f2(cq[0]), DP, dq);
            else if (n == 2) dq = fma2(fma2(f2(cq[1]), DP, f2(cq[0])), DP, dq);
            else dq = fma2(fma2(fma2(f2(cq[2]), DP, f2(cq[1])), DP, f2(cq[0])), DP, dq);
        }
    } else {
        const float2 X = t.c[PHK_X], XP = t.c[PHK_XP];
        const float2 Y = t.c[PHK_Y], YP = t.c[PHK_YP];
        const float2 Jx = mul2(f2(0.5f), fma2(mul2(f2(c[6]), XP), XP,
                                              fma2(mul2(f2(c[5]), X), XP,
                                                   mul2(mul2(f2(c[4]), X), X))));
        const float2 Jy = mul2(f2(0.5f), fma2(mul2(f2(c[9]), YP), YP,
                                              fma2(mul2(f2(c[8]), Y), YP,
                                                   mul2(mul2(f2(c[7]), Y), Y))));
        dqx = add2(dqx, fma2(f2(c[0]), Jx, mul2(f2(c[2]), Jy)));
        dqy = add2(dqy, fma2(f2(c[1]), Jy, mul2(f2(c[3]), Jx)));
    }
}

__device__ __forceinline__ void sp_transverse_x2(const StreamProg& sp, Pair& t) {
    const float* p = sp.op[0];
    const int f = sp.flags[0];
    float2 X = t.c[PHK_X], XP = t.c[PHK_XP], Y = t.c[PHK_Y], YP = t.c[PHK_YP];
    const float2 DP = t.c[PHK_DP];
    float2 M[8];
    const bool detuned = f & PHK_FLAG_DETUNED;
    if (detuned) {
        float2 dqx = f2(0.f), dqy = f2(0.f);
        if (sp.n_det > 0) sp_detune_x2(sp, 0, t, dqx, dqy);
        if (sp.n_det > 1) sp_detune_x2(sp, 1, t, dqx, dqy);
        float2 sx, cx, sy, cy;
        sincos_turns_x2(f2(p[16]), f2(p[17]), dqx, &sx, &cx);
        sincos_turns_x2(f2(p[18]), f2(p[19]), dqy, &sy, &cy);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            M[e] = fma2(f2(p[e]), cx, fma2(f2(p[8 + e]), sx,
                                           fma2(f2(p[40 + e]), cx, mul2(f2(p[48 + e]), sx))));
            M[4 + e] = fma2(f2(p[4 + e]), cy, fma2(f2(p[12 + e]), sy,
                                                   fma2(f2(p[44 + e]), cy, mul2(f2(p[52 + e]), sy))));
        }
    } else {
#pragma unroll
        for (int e = 0; e < 8; ++e) M[e] = f2(p[e]);
    }
    if (f & PHK_FLAG_DISPERSION) {
        X = fma2(f2(-p[32]), DP, X);
        Y = fma2(f2(-p[34]), DP, Y);
    }
    float2 cxr = f2(0.f), cxp = f2(0.f), cyr = f2(0.f), cyp = f2(0.f);
    if (!detuned) {
        cxr = fma2(f2(p[40]), X, mul2(f2(p[41]), XP));
        cxp = fma2(f2(p[42]), X, mul2(f2(p[43]), XP));
        cyr = fma2(f2(p[44]), Y, mul2(f2(p[45]), YP));
        cyp = fma2(f2(p[46]), Y, mul2(f2(p[47]), YP));
    }
    const float2 nx = fma2(M[0], X, fma2(M[1], XP, cxr));
    const float2 nxp = fma2(M[2], X, fma2(M[3], XP, cxp));
    const float2 ny = fma2(M[4], Y, fma2(M[5], YP, cyr));
    const float2 nyp = fma2(M[6], Y, fma2(M[7], YP, cyp));
    X = nx; XP = nxp; Y = ny; YP = nyp;
    if (f & PHK_FLAG_DISPERSION) {
        X = fma2(f2(p[33]), DP, X);
        Y = fma2(f2(p[35]), DP, Y);
    }
    t.c[PHK_X] = X; t.c[PHK_XP] = XP; t.c[PHK_Y] = Y; t.c[PHK_YP] = YP;
}

template <int OPI>
__device__ __forceinline__ void sp_drift_x2(const StreamProg& sp, Pair& t) {
    const float* p = sp.op[OPI];
    const float2 Z = t.c[PHK_Z], DP = t.c[PHK_DP];
    const float2 zs = (sp.flags[OPI] & PHK_FLAG_SHRINK)
                          ? fma2(f2(p[0]), Z, mul2(f2(p[3]), Z)) : Z;
    t.c[PHK_Z] = fma2(f2(-p[1]), DP, fma2(f2(-p[2]), DP, zs));
}

__device__ __forceinline__ void sp_rfkick_x2(const StreamProg& sp, Pair& t) {
    const float* p = sp.op[2];
    const bool disp = sp.flags[2] & PHK_FLAG_DISPERSION;
    float2 DP = t.c[PHK_DP];
    if (disp) {
        t.c[PHK_X] = fma2(f2(-p[8]), DP, t.c[PHK_X]);
        t.c[PHK_Y] = fma2(f2(-p[9]), DP, t.c[PHK_Y]);
    }
    const float2 s = sin_turns_of_product_x2(t.c[PHK_Z], p[0], p[1], p[2], p[3]);
    DP = fma2(f2(p[4]), s, fma2(f2(p[10]), s,
                                fma2(DP, f2(p[5]), fma2(DP, f2(p[11]), f2(-p[6])))));
    t.c[PHK_DP] = DP;
    if (disp) {
        t.c[PHK_X] = fma2(f2(p[8]), DP, t.c[PHK_X]);
        t.c[PHK_Y] = fma2(f2(p[9]), DP, t.c[PHK_Y]);
    }
}

__device__ __forceinline__ void sp_linear_long_x2(const StreamProg& sp, Pair& t) {
    const float* p = sp.op[1];
    const bool disp = sp.flags[1] & PHK_FLAG_DISPERSION;
    if (disp) {
        t.c[PHK_X] = fma2(f2(-p[4]), t.c[PHK_DP], t.c[PHK_X]);
        t.c[PHK_Y] = fma2(f2(-p[5]), t.c[PHK_DP], t.c[PHK_Y]);
    }
    const float2 z0 = t.c[PHK_Z], dp0 = t.c[PHK_DP];
    t.c[PHK_Z] = fma2(z0, f2(p[0]), fma2(f2(-p[2]), dp0,
                                         fma2(z0, f2(p[1]), mul2(f2(-p[3]), dp0))));
    t.c[PHK_DP] = fma2(dp0, f2(p[0]), fma2(f2(p[6]), z0,
                                           fma2(dp0, f2(p[1]), mul2(f2(p[7]), z0))));
    if (disp) {
        t.c[PHK_X] = fma2(f2(p[4]), t.c[PHK_DP], t.c[PHK_X]);
        t.c[PHK_Y] = fma2(f2(p[5]), t.c[PHK_DP], t.c[PHK_Y]);
    }
}

template <int SHAPE>
__device__ __forceinline__ void sp_program_x2(const StreamProg& sp, Pair& t) {
    if constexpr (SHAPE == SHAPE_T) {
        sp_transverse_x2(sp, t);
    } else if constexpr (SHAPE == SHAPE_T_RF) {
        sp_transverse_x2(sp, t);
        sp_drift_x2<1>(sp, t);
        sp_rfkick_x2(sp, t);
        sp_drift_x2<3>(sp, t);
    } else if constexpr (SHAPE == SHAPE_T_LIN) {
        sp_transverse_x2(sp, t);
        sp_linear_long_x2(sp, t);
    }
}

// coordinates a shape reads and writes (bit q = coordinate q)
template <int SHAPE, bool PK, bool ACC>
constexpr int stream_load_bits() {
    return SHAPE == SHAPE_NONE ? 0x15
                               : (SHAPE == SHAPE_T ? (0x2F | ((PK || ACC) ? 0x10 : 0)) : 0x3F);
}

// shared memory: FixHist [count Sa | digits 4 Sa | flags], accumulation
// edges [Sa + 1], pending-kick edges [Sp + 1], summed kick tables
// [n_tables][Sp], rings [warps][stages][6][64] floats, mbarriers
// [warps][stages]
__host__ __device__ inline size_t stream_smem_layout(int Sa, int Sp,
                                                     int n_tables, int stages,
                                                     size_t* off) {
    size_t b = 0;
    off[0] = b; b = align16(b + (size_t)4 * Sa);              // FixHist count
    off[1] = b; b = align16(b + (size_t)4 * 4 * Sa);          // digits
    off[2] = b; b = align16(b + (size_t)4 * ((Sa + 3) / 4));
    off[3] = b; b = align16(b + (size_t)4 * (Sa > 0 ? Sa + 1 : 0));
    off[4] = b; b = align16(b + (size_t)4 * (Sp > 0 ? Sp + 1 : 0));
    off[5] = b; b = align16(b + (size_t)4 * n_tables * Sp);
    off[6] = b; b = align16(b + (size_t)4 * kStreamWarps * stages * 6 * kStreamTile);
    off[7] = b; b = align16(b + (size_t)8 * kStreamWarps * stages);
    return b;
}

// coordinates written by a shape (bit q = coordinate q), before the kicks
template <int SHAPE>
constexpr int stream_store_bits() {
    return SHAPE == SHAPE_T ? 0x0F : (SHAPE == SHAPE_NONE ? 0 : 0x3F);
}

// pending kicks, program, accumulation of one particle
template <int SHAPE, bool PK, bool ACC>
__device__ __forceinline__ void stream_particle(const StreamProg& sp,
                                                const StreamArgs& a,
                                                const Bins<float>& bpk,
                                                const Bins<float>& bac,
                                                const float* ktab, int Sp,
                                                const FixHist& fix,
                                                Tile<float, 1>& t) {
    if constexpr (PK) {
        const int s = bpk.index(t.c[PHK_Z][0]);
        if (s >= 0) {
            if (a.comb_slot[0] >= 0) t.c[PHK_XP][0] += ktab[a.comb_slot[0] * Sp + s];
            if (a.comb_slot[1] >= 0) t.c[PHK_YP][0] += ktab[a.comb_slot[1] * Sp + s];
            if (a.comb_slot[2] >= 0) t.c[PHK_DP][0] += ktab[a.comb_slot[2] * Sp + s];
        }
    }
    sp_program<SHAPE>(sp, t);
    if constexpr (ACC) {
        const int s = bac.index(t.c[PHK_Z][0]);
        if (s >= 0) fix.add(s, t.c[PHK_X][0], t.c[PHK_Y][0]);
    }
}

// pending kicks, program and accumulation of the lane's two particles
template <int SHAPE, bool PK, bool ACC>
__device__ __forceinline__ void stream_pair(const StreamProg& sp,
                                            const StreamArgs& a,
                                            const Bins<float>& bpk,
                                            const Bins<float>& bac,
                                            const float* ktab, int Sp,
                                            const FixHist& fix, Pair& t) {
    if constexpr (PK) {
        const float zv[2] = {t.c[PHK_Z].x, t.c[PHK_Z].y};
        int sl[2];
        bpk.index_vec<2>(zv, sl);
        const bool on0 = sl[0] >= 0, on1 = sl[1] >= 0;
        const int s0 = on0 ? sl[0] : 0, s1 = on1 ? sl[1] : 0;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const int slot = a.comb_slot[q];
            if (slot < 0) continue;
            const float* tab = ktab + slot * Sp;
            const int c = q == 0 ? PHK_XP : (q == 1 ? PHK_YP : PHK_DP);
            t.c[c] = add2(t.c[c], make_float2(on0 ? tab[s0] : 0.f, on1 ? tab[s1] : 0.f));
        }
    }
    sp_program_x2<SHAPE>(sp, t);
    if constexpr (ACC) {
        const float zv[2] = {t.c[PHK_Z].x, t.c[PHK_Z].y};
        int sl[2];
        bac.index_vec<2>(zv, sl);
        if (sl[0] >= 0) fix.add(sl[0], t.c[PHK_X].x, t.c[PHK_Y].x);
        if (sl[1] >= 0) fix.add(sl[1], t.c[PHK_X].y, t.c[PHK_Y].y);
    }
}

template <int SHAPE, bool PK, bool ACC>
__global__ void __launch_bounds__(kStreamThreads, 4)
stream_kernel(const __grid_constant__ StreamProg sp,
              const __grid_constant__ phk_kick_set pk,
              const __grid_constant__ phk_accum acc,
              const __grid_constant__ StreamArgs a) {
    namespace cg = cooperative_groups;
    extern __shared__ __align__(16) unsigned char smem[];
    const int Sa = ACC ? acc.slicer.n_slices : 0;
    const int Sp = PK ? pk.slicer.n_slices : 0;
    size_t off[8];
    stream_smem_layout(Sa, Sp, a.n_tables, a.stages, off);
    int* hcnt = reinterpret_cast<int*>(smem + off[0]);
    int* fdig = reinterpret_cast<int*>(smem + off[1]);
    unsigned* fflag = reinterpret_cast<unsigned*>(smem + off[2]);
    float* eacc = reinterpret_cast<float*>(smem + off[3]);
    float* epk = reinterpret_cast<float*>(smem + off[4]);
    float* ktab = reinterpret_cast<float*>(smem + off[5]);
    __shared__ unsigned s_max[2];
    __shared__ FixSpill s_spill;
    __shared__ int s_abort;
    __shared__ int s_undrained;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int stages = a.stages;
    float* ring = reinterpret_cast<float*>(smem + off[6]) +
                  (size_t)warp * stages * 6 * kStreamTile;
    unsigned long long* wb =
        reinterpret_cast<unsigned long long*>(smem + off[7]) + warp * stages;
    // warp-tiles: full ones through the ring, the partial last one (if
    // any) with plain loads by the warp that owns its index
    const int GW = (int)gridDim.x * kStreamWarps;
    const int gw = (int)blockIdx.x * kStreamWarps + warp;
    const int n_full = (int)(a.n / kStreamTile);
    const int mine = gw < n_full ? (n_full - gw + GW - 1) / GW : 0;
    const int w0 = (int)blockIdx.x * kStreamWarps;   // the CTA's first warp
    const int mine_cta = w0 < n_full ? (n_full - w0 + GW - 1) / GW : 0;
    const bool has_partial = a.n % kStreamTile != 0 && gw == n_full % GW;
    int nq = 0;
    for (int q = 0; q < 6; ++q) nq += (a.load_mask >> q) & 1;
    const unsigned stage_bytes = (unsigned)(nq * kStreamTile * 4);
    int last[kStreamMaxStages];      // lane 0: last warp-tile issued per stage
    for (int st = 0; st < kStreamMaxStages; ++st) last[st] = -1;
    auto issue = [&](int k, int st) {
        const int64_t tile = (int64_t)gw + (int64_t)k * GW;
        fence_proxy_async_smem();
        mbar_expect_tx(wb + st, stage_bytes);
        for (int q = 0; q < 6; ++q)
            if ((a.load_mask >> q) & 1)
                bulk_g2s(ring + ((size_t)st * 6 + q) * kStreamTile,
                         a.c[q] + tile * kStreamTile, kStreamTile * 4, wb + st);
        last[st] = k;
    };
    if (tid == 0) {
        s_max[0] = s_max[1] = 0u;
        s_abort = 0;
        s_undrained = 0;
    }
    if (lane == 0) {
        for (int st = 0; st < stages; ++st) mbar_init(wb + st, 1);
        mbar_fence_init();
        // the warp's first tiles are on their way while the CTA stages its
        // tables (each warp's ring has shared memory of its own)
        for (int k = 0; k < mine && k < stages; ++k) issue(k, k);
    }
    if constexpr (ACC) {
        const float* e = reinterpret_cast<const float*>(acc.slicer.edges);
        for (int i = tid; i <= Sa; i += kStreamThreads) eacc[i] = e[i];
        for (int i = tid; i < Sa; i += kStreamThreads) hcnt[i] = 0;
        for (int i = tid; i < 4 * Sa; i += kStreamThreads) fdig[i] = 0;
        for (int i = tid; i < (Sa + 3) / 4; i += kStreamThreads) fflag[i] = 0u;
    }
    if constexpr (PK) {
        TrackArgs ta;
        ta.kick_comb = 1;
        ta.kicks_smem = 1;
        for (int q = 0; q < 3; ++q) ta.comb_slot[q] = a.comb_slot[q];
        stage_pending<float>(pk, ta, epk, ktab, tid, kStreamThreads);
    }
    __syncthreads();
    Bins<float> bpk, bac;
    if constexpr (PK) bpk.init(epk, Sp, pk.slicer.negate);
    if constexpr (ACC) bac.init(eacc, Sa, acc.slicer.negate);
    vote_fast_path<float>(bpk, PK, tid, kStreamThreads);
    vote_fast_path<float>(bac, ACC, tid, kStreamThreads);

    const bool clustered = ACC && a.cluster > 1;
    const unsigned crank = clustered ? cg::this_cluster().block_rank() : 0u;
    const int column = clustered ? (int)(blockIdx.x / a.cluster) : (int)blockIdx.x;
    const int G = acc.grid;
    double* P = acc.partials;
    long long* PL = reinterpret_cast<long long*>(P);

    bool bad = false;

    FixHist fix;
    if constexpr (ACC) {
        // ---- the cluster's fixed-point scale, from each warp's first tile
        unsigned m[2] = {0u, 0u};
        auto see = [&](float u, int q) {
            const unsigned b = __float_as_uint(u) & 0x7fffffffu;
            if (b < 0x7f800000u && b > m[q]) m[q] = b;
        };
        if (mine > 0) {
            bad = !mbar_wait(wb, 0u, a.wait_limit);
            if (!bad) {
                const float* src = ring + lane * 2;
                see(src[PHK_X * kStreamTile], 0);
                see(src[PHK_X * kStreamTile + 1], 0);
                see(src[PHK_Y * kStreamTile], 1);
                see(src[PHK_Y * kStreamTile + 1], 1);
            }
        } else if (has_partial) {
            const int64_t i0 = (int64_t)n_full * kStreamTile + lane * 2;
            for (int j = 0; j < 2; ++j) {
                if (i0 + j < a.n) {
                    see(a.c[PHK_X][i0 + j], 0);
                    see(a.c[PHK_Y][i0 + j], 1);
                }
            }
        }
        m[0] = __reduce_max_sync(0xffffffffu, m[0]);
        m[1] = __reduce_max_sync(0xffffffffu, m[1]);
        if (lane == 0) {
            atomicMax(&s_max[0], m[0]);
            atomicMax(&s_max[1], m[1]);
        }
        if (tid == 0) {
            s_spill.spill[0] = PL + (int64_t)Sa * G + column;
            s_spill.spill[1] = PL + (int64_t)2 * Sa * G + column;
            s_spill.stride = G;
        }
        if (crank == 0) {
            // the level-B sums of the column start at zero
            for (int s = tid; s < Sa; s += kStreamThreads) {
                PL[(int64_t)(Sa + s) * G + column] = 0;
                PL[(int64_t)(2 * Sa + s) * G + column] = 0;
            }
        }
        unsigned M[2];
        if (clustered) {
            __threadfence();
            cg::cluster_group cl = cg::this_cluster();
            cl.sync();
            M[0] = M[1] = 0u;
            for (unsigned r = 0; r < cl.num_blocks(); ++r) {
                const unsigned* sm = cl.map_shared_rank(s_max, r);
                M[0] = max(M[0], sm[0]);
                M[1] = max(M[1], sm[1]);
            }
        } else {
            __syncthreads();
            M[0] = s_max[0];
            M[1] = s_max[1];
        }
        fix.cnt = hcnt;
        fix.dig = fdig;
        fix.flag = fflag;
        fix.sp = &s_spill;
        fix.S = Sa;
        fix.scale[0] = fix_scale(M[0]);
        fix.scale[1] = fix_scale(M[1]);
    }

    // ---- the warp's full tiles.  The loop runs the CTA's count so that
    // every warp reaches the flush barriers of the slice sums; a warp past
    // its own tiles, or after a wait gave up anywhere in the CTA, only keeps
    // pace.
    constexpr int kStore = stream_store_bits<SHAPE>() | (PK ? 0x0A : 0);
    constexpr int kLoad = stream_load_bits<SHAPE, PK, ACC>();
    constexpr int kFlushEvery = (int)(kFixMaxPerCta / (kStreamWarps * kStreamTile));
    volatile int* abort_flag = &s_abort;
    int st = 0;
    unsigned ph = 0u;
    for (int k = 0; k < mine_cta; ++k) {
        bool ok = false;
        if (k < mine && !bad && !*abort_flag) {
            ok = mbar_wait(wb + st, ph, a.wait_limit);
            if (!ok) {
                bad = true;
                *abort_flag = 1;
            }
        }
        if (ok) {
            const float* src = ring + (size_t)st * 6 * kStreamTile + lane * 2;
            Pair t;
#pragma unroll
            for (int q = 0; q < 6; ++q)
                t.c[q] = ((kLoad >> q) & 1)
                             ? *reinterpret_cast<const float2*>(src + q * kStreamTile)
                             : make_float2(0.f, 0.f);
            __syncwarp();                   // the warp's reads of stage st done
            if (lane == 0 && k + stages < mine && !*abort_flag) issue(k + stages, st);
            stream_pair<SHAPE, PK, ACC>(sp, a, bpk, bac, ktab, Sp, fix, t);
            const int off = (gw + k * GW) * kStreamTile + lane * 2;
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const bool w = ((kStore >> q) & 1) ||
                               (PK && q == PHK_DP && a.comb_slot[2] >= 0);
                if (w) __stcs(reinterpret_cast<float2*>(a.c[q] + off), t.c[q]);
            }
        }
        if (++st == stages) {
            st = 0;
            ph ^= 1u;
        }
        if constexpr (ACC) {
            if ((k + 1) % kFlushEvery == 0) {
                __syncthreads();
                fix_flush(fix, tid, kStreamThreads);
                __syncthreads();
            }
        }
    }
    if (has_partial && !*abort_flag) {
        // ---- the partial last warp-tile, plain loads
        const int64_t i0 = (int64_t)n_full * kStreamTile + lane * 2;
        Tile<float, 1> t[2];
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const bool live = i0 + j < a.n;
#pragma unroll
            for (int q = 0; q < 6; ++q)
                t[j].c[q][0] = (live && ((kLoad >> q) & 1)) ? a.c[q][i0 + j] : 0.f;
            if (!live) continue;
            stream_particle<SHAPE, PK, ACC>(sp, a, bpk, bac, ktab, Sp, fix, t[j]);
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                const bool w = ((kStore >> q) & 1) ||
                               (PK && q == PHK_DP && a.comb_slot[2] >= 0);
                if (w) a.c[q][i0 + j] = t[j].c[q][0];
            }
        }
    }
    // copies still in flight after a wait gave up: the last one issued into
    // each stage (bounded waits)
    if (lane == 0 && *abort_flag) {
        for (int q = 0; q < stages; ++q)
            if (last[q] >= 0 &&
                !mbar_wait(wb + q, (unsigned)((last[q] / stages) & 1), kWaitLimit))
                atomicOr(&s_undrained, 1);
    }
    __syncwarp();
    __syncthreads();
    if (tid == 0 && s_abort && a.status)
        atomicMax(a.status, s_undrained ? PHK_DEV_TIMEOUT_UNDRAINED : PHK_DEV_TIMEOUT);
    if constexpr (!ACC) {
        return;
    } else {
        // ---- rank 0 adds its cluster's counters and level-B sums
        unsigned nb = 1;
        if (clustered) {
            __threadfence();
            cg::cluster_group cl = cg::this_cluster();
            cl.sync();
            nb = cl.num_blocks();
        }
        if (crank == 0) {
            for (int s = tid; s < Sa; s += kStreamThreads) {
                long long c = 0;
                long long tq[2];
                unsigned fl = 0;
                tq[0] = __ldcg(PL + (int64_t)(Sa + s) * G + column);
                tq[1] = __ldcg(PL + (int64_t)(2 * Sa + s) * G + column);
                for (unsigned r = 0; r < nb; ++r) {
                    const unsigned* rf = fflag;
                    if (clustered) rf = cg::this_cluster().map_shared_rank(fflag, r);
                    fl |= (rf[s >> 2] >> (8 * (s & 3))) & 0xffu;
                    const int* rc = hcnt;
                    const int* rd = fdig;
                    if (clustered) {
                        cg::cluster_group cl = cg::this_cluster();
                        rc = cl.map_shared_rank(hcnt, r);
                        rd = cl.map_shared_rank(fdig, r);
                    }
                    c += rc[s];
#pragma unroll
                    for (int q = 0; q < 2; ++q)
                        tq[q] += FixHist::total(rd + 2 * q * Sa + s, Sa);
                }
                P[(int64_t)s * G + column] = (double)c;
                P[(int64_t)(Sa + s) * G + column] = fix_value(tq[0], fl & 15u, fix.scale[0]);
                P[(int64_t)(2 * Sa + s) * G + column] = fix_value(tq[1], fl >> 4, fix.scale[1]);
            }
        }
        if (clustered) cg::this_cluster().sync();
    }
}

}  // namespace phk
