// CPU emulator of the GPU engine -- test infrastructure.
//
// Runs the library's launch schedules with the very same engine functions
// the CUDA kernels run (kissfft_gb300/csrc/kf_engine.cuh), looping over the
// thread indices of each CTA in order.  The tests compare its output with
// the oracle, bit for bit in fixed point, to validate the plan tables, the
// pass grouping, the digit-reversal addressing and the two-pass splits
// without a GPU.  It is never part of the shipped library.
#include <string.h>

#include <limits>
#include <vector>

// Count the overflows the reference built with CHECK_OVERFLOW would report
// (_kiss_fft_guts.h:57-61), at the operations the engine marks with
// KF_OVF_CHECK (kissfft_gb300/csrc/kf_arith.cuh).
static long long g_overflows = 0;
template <typename S>
static inline void emu_ovf_note(long long v) {
    if (v > (long long)std::numeric_limits<S>::max() || v < (long long)std::numeric_limits<S>::min()) ++g_overflows;
}
#define KF_OVF_NOTE(S, v) emu_ovf_note<S>(v)

// Bounds checking of every access the engine marks with KF_MEM_CHECK
// (kissfft_gb300/csrc/kf_engine.cuh): an access must lie wholly inside one
// of the memory regions the current run owns (the caller's input and
// output, the schedule's scratch, the shared tile of exactly the launch's
// dynamic size, the plan tables, the fast-FIR response).
struct EmuRegion {
    const unsigned char* lo;
    const unsigned char* hi;
};
static std::vector<EmuRegion> g_regions;
static long long g_oob = 0;
static inline void emu_mem_note(const void* p, size_t n) {
    const unsigned char* a = (const unsigned char*)p;
    for (size_t i = g_regions.size(); i-- > 0;)
        if (a >= g_regions[i].lo && a + n <= g_regions[i].hi) return;
    ++g_oob;
}
#define KF_MEM_NOTE(p, n) emu_mem_note(p, n)

// Bytes by which the next runs under-declare the output region (which 1) or
// the shared tile (which 2), to show that the check catches the last
// accesses; the buffers themselves keep their full size.
static long long g_trim_out = 0, g_trim_sm = 0;
static size_t trimmed(size_t n, long long t) { return t > 0 && (size_t)t < n ? n - (size_t)t : n; }

// A region owned for the lifetime of the guard.
struct EmuOwn {
    EmuOwn(const void* p, size_t n) {
        g_regions.push_back({(const unsigned char*)p, (const unsigned char*)p + n});
    }
    ~EmuOwn() { g_regions.pop_back(); }
};

#include "kf_plan.h"
#include "kf_runner.cuh"

using namespace kf;

static int g_force_J = 0, g_force_T = 0, g_force_col = 0, g_force_swz = -1;

template <typename S, int MODE, kmask_t KM>
struct CpuExec {
    int T;
    void sync() {}
    void input_consumed() {}
    void pass(Tile<S>& t, const KSub& sb, const KTab& tb, const KPass& ps, bool last, bool sg, bool dg) {
        for (int tid = 0; tid < T; ++tid) run_pass<S, MODE, KM>(t, sb, tb, ps, last, tid, T, sg, dg);
    }
    void rtg(Tile<S>& t, const KSub& sb, const KTab& tb, const KPass& ps, bool last, bool sg, bool dg) {
        std::vector<cpx<S>> buf((size_t)T * KF_MAXO);
        for (int tid = 0; tid < T; ++tid)
            rtg_compute<S, MODE>(t, sb, tb, ps, last, tid, T, sg, &buf[(size_t)tid * KF_MAXO]);
        for (int tid = 0; tid < T; ++tid)
            rtg_store<S, MODE>(t, sb, tb, ps, last, tid, T, dg, &buf[(size_t)tid * KF_MAXO]);
    }
    void c2r_pre(Tile<S>& t, const KSub& sb, const KTab& tb) {
        for (int tid = 0; tid < T; ++tid) kf::c2r_pre<S>(t, sb, tb, tid, T);
    }
    void r2c_post(Tile<S>& t, const KSub& sb, const KTab& tb) {
        for (int tid = 0; tid < T; ++tid) kf::r2c_post<S>(t, sb, tb, tid, T);
    }
    void fir_mid(Tile<S>& t, const KSub& fw, const KTab& fwt, const KTab& ivt, const cpx<S>* H) {
        std::vector<cpx<S>> buf((size_t)T * KF_MAXO);
        for (int tid = 0; tid < T; ++tid) fir_mid_compute<S>(t, fw, fwt, ivt, H, tid, T, &buf[(size_t)tid * KF_MAXO]);
        for (int tid = 0; tid < T; ++tid) fir_mid_store<S>(t, fw, tid, T, &buf[(size_t)tid * KF_MAXO]);
    }
};

template <typename S, int MODE, int FAM>
static int run_engine_step_f(const Step& st) {
    const KArgs& a = st.args;
    const LaunchCfg& c = st.cfg;
    std::vector<cpx<S>> sm(c.smem / sizeof(cpx<S>) + 1);
    EmuOwn own_sm(sm.data(), trimmed((size_t)c.smem, g_trim_sm));
    long long inb[KF_MAXJ], outb[KF_MAXJ], lin[KF_MAXJ], lout[KF_MAXJ];
    int U[KF_MAXJ];
    int err = 0;
    Tile<S> t;
    memset(&t, 0, sizeof(t));
    tile_layout(a, a.sub[0].L, a.J, a.logJ, a.col_in | a.col_out, t);
    t.sm = sm.data();
    t.T = c.T;
    t.inb = inb;
    t.outb = outb;
    t.U = U;
    t.lim_in = lin;
    t.lim_out = lout;
    t.err = &err;
    CpuExec<S, MODE, family_mask(FAM, is_f32<S>())> x;
    x.T = c.T;
    for (long long tile = 0; tile < a.ntiles; ++tile) {
        for (int j = 0; j < a.J; ++j) job_entry(a, tile, a.J, j, inb[j], outb[j], U[j], lin[j], lout[j]);
        run_tile<S, MODE, family_mask(FAM, is_f32<S>())>(x, a, a.sub[0], a.sub[1], t, a.col_in, a.col_out);
    }
    return err;
}

template <typename S, int MODE>
static int run_engine_step(const Step& st) {
    switch (st.fam) {
        case FAM_POW2: return run_engine_step_f<S, MODE, FAM_POW2>(st);
        case FAM_SMOOTH: return run_engine_step_f<S, MODE, FAM_SMOOTH>(st);
        default: return run_engine_step_f<S, MODE, FAM_GENERAL>(st);
    }
}

template <typename S>
static int run_step_t(const Step& st) {
    if (st.kind == 1) {
        long long items = st.args.G * (st.args.sub[0].L / 2 + 1);
        for (long long it = 0; it < items; ++it) split_item<S>(st.args, it);
        return 0;
    }
    if (st.kind == 2) {
        long long items = st.args.G * (st.args.sub[0].L / 2 + 1);
        for (long long it = 0; it < items; ++it) merge_item<S>(st.args, it);
        return 0;
    }
    switch (st.mode) {
        case MODE_C2C: return run_engine_step<S, MODE_C2C>(st);
        case MODE_R2C: return run_engine_step<S, MODE_R2C>(st);
        case MODE_C2R: return run_engine_step<S, MODE_C2R>(st);
        case MODE_FIR: return run_engine_step<S, MODE_FIR>(st);
    }
    return -1;
}

static int run_schedule(Schedule& s, const void* in, void* out, const void* firH = nullptr) {
    std::vector<uint8_t> tmp(s.scratch[0] + s.scratch[1] + 16);
    EmuOwn own_s0(tmp.data(), s.scratch[0]), own_s1(tmp.data() + s.scratch[0], s.scratch[1]);
    for (auto& st : s.steps) {
        void* roles[4] = {(void*)in, out, tmp.data(), tmp.data() + s.scratch[0]};
        st.args.in = roles[st.in_role];
        st.args.out = roles[st.out_role];
        st.args.fir_H = firH;
        if (g_force_J && st.kind == 0) {
            st.cfg.J = g_force_J;
            st.args.J = g_force_J;
            int lj = 0;
            while ((1 << lj) < g_force_J) ++lj;
            st.args.logJ = lj;
            st.cfg.grid = (st.args.G + g_force_J - 1) / g_force_J;
            st.args.ntiles = st.cfg.grid;
            st.cfg.smem = cfg_smem_bytes(st.args.sub[0], st.dtype, g_force_J);
            st.cfg.T = std::max(st.cfg.T, cfg_min_threads(st.args.sub[0], st.mode, g_force_J));
        }
        if (g_force_T && st.kind == 0) st.cfg.T = std::max(g_force_T, cfg_min_threads(st.args.sub[0], st.mode, st.cfg.J));
        if (g_force_swz >= 0 && st.kind == 0) st.args.swz = g_force_swz;
        if (g_force_col && st.kind == 0 && st.mode != MODE_FIR) {
            st.cfg.col_in = st.cfg.col_out = 1;
            st.args.col_in = st.args.col_out = 1;
        }
        int e = 0;
        switch (st.dtype) {
            case KF_F32: e = run_step_t<float>(st); break;
            case KF_F64: e = run_step_t<double>(st); break;
            case KF_Q15: e = run_step_t<int16_t>(st); break;
            case KF_Q31: e = run_step_t<int32_t>(st); break;
        }
        if (e) return e;
    }
    return 0;
}

extern "C" {

void emu_trim(int which, long long bytes) {
    if (which == 1) g_trim_out = bytes;
    if (which == 2) g_trim_sm = bytes;
}

// out-of-bounds accesses counted since the last call
long long emu_oob_take(void) {
    const long long n = g_oob;
    g_oob = 0;
    return n;
}

// overflows counted since the last call
long long emu_overflows_take(void) {
    const long long n = g_overflows;
    g_overflows = 0;
    return n;
}

void emu_force(int J, int T) {
    g_force_J = J;
    g_force_T = T;
}

// column-layout tiles (jobs fastest) for every engine step
void emu_force_col(int col) { g_force_col = col; }

// shared-tile index map (SWZ_*) of every engine step; -1: the schedule's own
void emu_force_swz(int mode) { g_force_swz = mode; }

int emu_c2c(int dtype, int n, int inverse, int lmax, const void* in, void* out, long long batch, long long in_dist,
            long long in_stride, long long out_dist) {
    Plan p;
    if (!p.build(dtype, n, inverse, lmax)) return -2;
    p.bind(p.blob.data());
    Schedule s;
    if (!schedule_c2c(p, batch, in_dist, in_stride, out_dist, s)) return -3;
    const long long esz = cpx_size(dtype);
    const long long ind = in_dist ? in_dist : (long long)n * in_stride, outd = out_dist ? out_dist : n;
    EmuOwn own_p(p.blob.data(), p.blob.size());
    EmuOwn own_i(in, (size_t)(((batch - 1) * ind + (long long)(n - 1) * in_stride + 1) * esz));
    EmuOwn own_o(out, trimmed((size_t)(((batch - 1) * outd + n) * esz), g_trim_out));
    return run_schedule(s, in, out);
}

int emu_r2c(int dtype, int nfft, int lmax, const void* in, void* out, long long batch) {
    Plan p;
    if (!p.build(dtype, nfft / 2, 0, lmax, nfft)) return -2;
    p.bind(p.blob.data());
    Schedule s;
    if (!schedule_r2c(p, batch, nfft, nfft / 2 + 1, s)) return -3;
    const long long esz = cpx_size(dtype);
    EmuOwn own_p(p.blob.data(), p.blob.size());
    EmuOwn own_i(in, (size_t)(batch * nfft * esz / 2));
    EmuOwn own_o(out, (size_t)(batch * (nfft / 2 + 1) * esz));
    return run_schedule(s, in, out);
}

int emu_c2r(int dtype, int nfft, int lmax, const void* in, void* out, long long batch) {
    Plan p;
    if (!p.build(dtype, nfft / 2, 1, lmax, nfft)) return -2;
    p.bind(p.blob.data());
    Schedule s;
    if (!schedule_c2r(p, batch, nfft / 2 + 1, nfft, s)) return -3;
    const long long esz = cpx_size(dtype);
    EmuOwn own_p(p.blob.data(), p.blob.size());
    EmuOwn own_i(in, (size_t)(batch * (nfft / 2 + 1) * esz));
    EmuOwn own_o(out, (size_t)(batch * nfft * esz / 2));
    return run_schedule(s, in, out);
}

// In-place complex transform along one axis of a row-major array; lmax
// caps the tile length (0: the dtype's default), so small axes can take the
// two-pass route.
int emu_axis_lmax(int dtype, const int* dims, int ndims, int axis, int inverse, int lmax, void* buf) {
    Plan p;
    if (!p.build(dtype, dims[axis], inverse, lmax)) return -2;
    p.bind(p.blob.data());
    Schedule s;
    if (!schedule_axis(p, dims, ndims, axis, 1, 0, 1, s)) return -3;
    long long total = 1;
    for (int i = 0; i < ndims; ++i) total *= dims[i];
    EmuOwn own_p(p.blob.data(), p.blob.size());
    EmuOwn own_b(buf, (size_t)(total * cpx_size(dtype)));
    return run_schedule(s, buf, buf);
}

int emu_axis(int dtype, const int* dims, int ndims, int axis, int inverse, void* buf) {
    Plan p;
    if (!p.build(dtype, dims[axis], inverse)) return -2;
    p.bind(p.blob.data());
    Schedule s;
    if (!schedule_axis(p, dims, ndims, axis, 1, 0, 1, s)) return -3;
    long long total = 1;
    for (int i = 0; i < ndims; ++i) total *= dims[i];
    EmuOwn own_p(p.blob.data(), p.blob.size());
    EmuOwn own_b(buf, (size_t)(total * cpx_size(dtype)));
    return run_schedule(s, buf, buf);
}

// Real fast FIR with the library's block plan (H computed by the caller,
// already scaled by 1/nfft).
int emu_fastfir(const float* H, long long nfft, long long L, const float* x, long long Ns, float* y) {
    Plan fw, iv;
    if (!fw.build(KF_F32, (int)nfft / 2, 0, 0, (int)nfft)) return -2;
    if (!iv.build(KF_F32, (int)nfft / 2, 1, 0, (int)nfft)) return -2;
    fw.bind(fw.blob.data());
    iv.bind(iv.blob.data());
    Schedule s;
    if (!schedule_fastfir(fw, iv, L, Ns, 0, s)) return -3;
    EmuOwn own_f(fw.blob.data(), fw.blob.size()), own_v(iv.blob.data(), iv.blob.size());
    EmuOwn own_h(H, (size_t)(nfft / 2 + 1) * 2 * sizeof(float));
    EmuOwn own_x(x, (size_t)Ns * sizeof(float));
    EmuOwn own_y(y, (size_t)(Ns >= L ? Ns - L + 1 : 0) * sizeof(float));
    return run_schedule(s, x, y, H);
}

int emu_plan_info(int dtype, int n, int lmax, int* out) {
    Plan p;
    if (!p.build(dtype, n, 0, lmax)) return -2;
    out[0] = p.nsub;
    out[1] = p.sub[0].L;
    out[2] = p.nsub > 1 ? p.sub[1].L : 0;
    out[3] = p.sub[0].npass;
    return 0;
}
}
