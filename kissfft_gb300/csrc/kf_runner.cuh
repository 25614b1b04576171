// Sequencing of one tile: pre phase, the passes of one or two sub-plans,
// post phase.  Written once against an executor X that supplies the thread
// loop and the barriers: the CUDA kernel's executor runs each call on its
// own thread index and places __syncthreads(); the CPU emulator's executor
// loops over all thread indices in order (a pass touches disjoint shared
// locations per group, so sequential order is equivalent).
#pragma once
#include "kf_engine.cuh"

namespace kf {

#if defined(__CUDACC__)
#pragma nv_exec_check_disable
#endif
template <typename S, int MODE, kmask_t KM, class X>
KF_HD void run_sub(X& x, Tile<S>& t, const KSub& sb, const KTab& tb, bool src_first, bool dst_last, int col_in,
                   int col_out) {
#pragma unroll
    for (int pi = 0; pi < sb.npass; ++pi) {
        const KPass& ps = sb.ps[pi];
        const bool first = pi == 0, last = pi == sb.npass - 1;
        t.col = last ? col_out : col_in;
        const bool sg = first && src_first, dg = last && dst_last;
        if constexpr ((KM & KM_RTG) != 0) {
            if (ps.kind == KIND_RT_GENERIC) {
                x.rtg(t, sb, tb, ps, last, sg, dg);
                x.sync();
                if (first && src_first) x.input_consumed();
                continue;
            }
        }
        x.pass(t, sb, tb, ps, last, sg, dg);
        x.sync();
        if (first && src_first) x.input_consumed();
    }
}

// One tile with shapes s0 (and s1 for the fast FIR's inverse plan): the
// generic kernels pass a.sub[0/1]; specialised kernels pass compile-time
// constants.
#if defined(__CUDACC__)
#pragma nv_exec_check_disable
#endif
template <typename S, int MODE, kmask_t KM, class X>
KF_HD void run_tile(X& x, const KRun& a, const KSub& s0, const KSub& s1, Tile<S>& t, int ci, int co) {
    if constexpr (MODE == MODE_C2R) {
        t.col = ci;
        x.c2r_pre(t, s0, a.tab[0]);
        x.sync();
    }
    run_sub<S, MODE, KM>(x, t, s0, a.tab[0], MODE != MODE_C2R, MODE == MODE_C2C || MODE == MODE_C2R, ci, co);
    if constexpr (MODE == MODE_R2C) {
        t.col = co;
        x.r2c_post(t, s0, a.tab[0]);
    }
    if constexpr (MODE == MODE_FIR) {
        t.col = co;
        x.fir_mid(t, s0, a.tab[0], a.tab[1], (const cpx<S>*)a.fir_H);
        x.sync();
        run_sub<S, MODE, KM>(x, t, s1, a.tab[1], false, true, co, co);
    }
}

// Shared-memory layout of a tile: interleaved jobs (column launches) or
// job-major rows.
template <typename S>
KF_HD void tile_layout(const KRun& a, int L, int J, int logJ, int col, Tile<S>& t) {
    t.J = J;
    t.logJ = logJ;
    if (col) {
        t.sA = J;
        t.sJ = 1;
    } else {
        t.sA = 1;
        t.sJ = L;
    }
    t.in = a.in;
    t.out = a.out;
    t.swzm = a.swz;
    t.in_stride = (int)a.in_stride;
    t.out_stride = (int)a.out_stride;
    t.err = a.err;
}

}  // namespace kf
