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
template <typename S, int MODE, int FAM, class X>
KF_HD void run_sub(X& x, Tile<S>& t, const KSub& sb, bool src_first, bool dst_last, int col_in, int col_out) {
    for (int pi = 0; pi < sb.npass; ++pi) {
        const KPass& ps = sb.ps[pi];
        const bool first = pi == 0, last = pi == sb.npass - 1;
        t.col = last ? col_out : col_in;
        const bool sg = first && src_first, dg = last && dst_last;
        if constexpr (FAM >= FAM_GENERAL) {
            if (ps.kind == KIND_RT_GENERIC) {
                x.rtg(t, sb, ps, last, sg, dg);
                x.sync();
                continue;
            }
        }
        x.pass(t, sb, ps, last, sg, dg);
        x.sync();
    }
}

#if defined(__CUDACC__)
#pragma nv_exec_check_disable
#endif
template <typename S, int MODE, int FAM, class X>
KF_HD void run_tile(X& x, const KArgs& a, Tile<S>& t) {
    const int ci = a.col_in, co = a.col_out;
    if constexpr (MODE == MODE_C2R) {
        t.col = ci;
        x.c2r_pre(t, a.sub[0]);
        x.sync();
    }
    run_sub<S, MODE, FAM>(x, t, a.sub[0], MODE != MODE_C2R, MODE == MODE_C2C || MODE == MODE_C2R, ci, co);
    if constexpr (MODE == MODE_R2C) {
        t.col = co;
        x.r2c_post(t, a.sub[0]);
    }
    if constexpr (MODE == MODE_FIR) {
        t.col = co;
        x.fir_mid(t, a.sub[0], a.sub[1], (const cpx<S>*)a.fir_H);
        x.sync();
        run_sub<S, MODE, FAM>(x, t, a.sub[1], false, true, co, co);
    }
}

// Shared-memory layout of a tile: interleaved jobs (column launches) or
// job-major rows.
template <typename S>
KF_HD void tile_layout(const KArgs& a, Tile<S>& t) {
    t.J = a.J;
    t.logJ = a.logJ;
    if (a.col_in || a.col_out) {
        t.sA = a.J;
        t.sJ = 1;
    } else {
        t.sA = 1;
        t.sJ = a.sub[0].L;
    }
    t.in = a.in;
    t.out = a.out;
    t.in_stride = a.in_stride;
    t.out_stride = a.out_stride;
    t.err = a.err;
}

}  // namespace kf
