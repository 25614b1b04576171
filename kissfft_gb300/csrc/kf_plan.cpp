// Host-side plans and launch schedules.  Compiled with -ffp-contract=off:
// the twiddle expressions must round exactly like the reference's.
#include "kf_plan.h"
#include "kf_shape.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>

namespace kf {

int dtype_size(int dtype) {
    switch (dtype) {
        case KF_F32: return 4;
        case KF_F64: return 8;
        case KF_Q15: return 2;
        case KF_Q31: return 4;
    }
    return 0;
}

std::vector<int> factor(int n) {
    int f[64] = {};
    int k = factor_into(n, f);
    if (k > 64) k = 64;
    return std::vector<int>(f, f + k);
}

int next_fast_size(int n) {
    for (;; ++n) {
        int m = n;
        while (m % 2 == 0) m /= 2;
        while (m % 3 == 0) m /= 3;
        while (m % 5 == 0) m /= 5;
        if (m <= 1) return n;
    }
}

// kf_cexp with KISS_FFT_COS/SIN (_kiss_fft_guts.h:127-145) at the plan dtype
static void cexp_at(int dtype, double phase, void* out, size_t i) {
    switch (dtype) {
        case KF_F32: {
            float* o = (float*)out + 2 * i;
            o[0] = (float)cos(phase);
            o[1] = (float)sin(phase);
            break;
        }
        case KF_F64: {
            double* o = (double*)out + 2 * i;
            o[0] = cos(phase);
            o[1] = sin(phase);
            break;
        }
        case KF_Q15: {
            int16_t* o = (int16_t*)out + 2 * i;
            o[0] = (int16_t)floor(.5 + 32767 * cos(phase));
            o[1] = (int16_t)floor(.5 + 32767 * sin(phase));
            break;
        }
        case KF_Q31: {
            int32_t* o = (int32_t*)out + 2 * i;
            o[0] = (int32_t)floor(.5 + 2147483647 * cos(phase));
            o[1] = (int32_t)floor(.5 + 2147483647 * sin(phase));
            break;
        }
    }
}

// The phase expressions of kiss_fft.c:361-367 and kiss_fftr.c:53-59, kept
// verbatim in form so that they round identically.
void make_twiddles(int dtype, int n, int inverse, void* out) {
    for (int i = 0; i < n; ++i) {
        const double pi = 3.141592653589793238462643383279502884197169399375105820974944;
        double phase = -2 * pi * i / n;
        if (inverse) phase *= -1;
        cexp_at(dtype, phase, out, (size_t)i);
    }
}

void make_super_twiddles(int dtype, int ncfft, int inverse, void* out) {
    for (int i = 0; i < ncfft / 2; ++i) {
        double phase = -3.14159265358979323846264338327 * ((double)(i + 1) / ncfft + .5);
        if (inverse) phase *= -1;
        cexp_at(dtype, phase, out, (size_t)i);
    }
}

int max_tile_len(int dtype) { return tile_len_max(dtype); }

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Twiddle slot `slot` of a compact stage table at base: a copy of the full
// table's entry idx, or for Q15 that entry as a sign-extended int32 pair
// (kf_shape.h tw_units)
static void put_tw(int dtype, uint8_t* base, size_t slot, const uint8_t* full, size_t idx) {
    const int esz = cpx_size(dtype);
    if (dtype == KF_Q15) {
        const int16_t* w = (const int16_t*)(full + idx * esz);
        const int32_t pair[2] = {w[0], w[1]};
        memcpy(base + slot * 8, pair, 8);
    } else {
        memcpy(base + slot * esz, full + idx * esz, esz);
    }
}

bool Plan::build(int dtype_, int n_, int inverse_, int lmax, int real_nfft_) {
    dtype = dtype_;
    n = n_;
    inverse = inverse_ ? 1 : 0;
    real_nfft = real_nfft_;
    error.clear();
    if (dtype_size(dtype) == 0) {
        error = "unknown sample type";
        return false;
    }
    const ShapeInfo si = make_shape(dtype, n, inverse, lmax, real_nfft);
    switch (si.error) {
        case 0: break;
        case 1: error = "transform length must be positive"; return false;
        case 2: error = "too many factors"; return false;
        case 3:
            error = "transform length has no split into two tiles of at most " +
                    std::to_string(lmax > 0 ? lmax : max_tile_len(dtype));
            return false;
        default: error = "generic radix tile too long"; return false;
    }
    radix.assign(si.radix, si.radix + si.K);
    nsub = si.nsub;
    split = si.split;
    sub[0] = si.sub[0];
    sub[1] = si.sub[1];
    const int esz = cpx_size(dtype);
    std::vector<uint8_t> twf((size_t)n * esz);
    make_twiddles(dtype, n, inverse, twf.data());
    // compact per-stage tables (layout of kf_shape.h: tw_width(p) entries per u)
    std::vector<uint8_t> tws((size_t)std::max<long long>(si.tw_count, 1) * esz, 0);
    for (int j = 0; j < si.K; ++j) {
        const int p = si.radix[j];
        if (si.twoff[j] < 0) continue;
        if (p > 5) {
            // generic-radix rows (kf_shape.h gen_row)
            const int RP = gen_row(p);
            const long long fs = si.fs[j], m = si.m[j];
            uint8_t* base = tws.data() + (size_t)si.twoff[j] * esz;
            for (long long u = 0; u < m; ++u)
                for (int q1 = 0; q1 < p; ++q1) {
                    const long long step = fs * (u + q1 * m) % n;
                    long long idx = 0;
                    for (int q = 1; q < p; ++q) {
                        idx = (idx + step) % n;
                        put_tw(dtype, base, (size_t)((u * p + q1) * RP + (q - 1)), twf.data(), (size_t)idx);
                    }
                }
            continue;
        }
        const int W = tw_width(p);
        uint8_t* base = tws.data() + (size_t)si.twoff[j] * esz;
        for (int u = 0; u < si.m[j]; ++u)
            for (int q = 1; q < p; ++q) put_tw(dtype, base, (size_t)u * W + (q - 1), twf.data(), (size_t)q * u * si.fs[j]);
        const size_t cst = (size_t)W * si.m[j];
        put_tw(dtype, base, cst, twf.data(), (size_t)si.fs[j] * si.m[j] % n);
        put_tw(dtype, base, cst + 1, twf.data(), (size_t)2 * si.fs[j] * si.m[j] % n);
    }
    // digit-reversal tables at the offsets make_shape assigned
    std::vector<int> rev((size_t)std::max(si.rev_total, 1), 0);
    for (int s = 0; s < nsub; ++s) {
        const KSub& sb = sub[s];
        for (int k = 0; k < sb.npass; ++k) {
            const KPass& p = sb.ps[k];
            if (p.ML <= 1) continue;
            const int b = p.a + p.ns - 1;
            const bool last = (k == sb.npass - 1);
            for (int idx = 0; idx < p.ML; ++idx) {
                int rem = idx, ul = 0;
                for (int j = b + 1; j < sb.nst; ++j) {
                    int d = rem % sb.st[j].p;
                    rem /= sb.st[j].p;
                    ul += d * sb.st[j].mloc;
                }
                // idx is the input-order index of the lower digits, ul their position
                if (last)
                    rev[p.rev_off + ul] = idx;
                else
                    rev[p.rev_off + idx] = ul;
            }
        }
        if (sb.revfull_off >= 0) {
            for (int A = 0; A < sb.L; ++A) {
                int rem = A, pos = 0;
                for (int j = 0; j < sb.nst; ++j) {
                    int d = rem % sb.st[j].p;
                    rem /= sb.st[j].p;
                    pos += d * sb.st[j].mloc;
                }
                rev[sb.revfull_off + pos] = A;
            }
        }
    }
    std::vector<uint8_t> sup;
    if (real_nfft > 0) {
        sup.resize((size_t)std::max(1, n / 2) * esz);
        make_super_twiddles(dtype, n, inverse, sup.data());
    }
    off_tw_full = 0;
    off_tw_stage = align256(twf.size());
    off_super = off_tw_stage + align256(tws.size());
    off_rev = off_super + align256(sup.size());
    blob.assign(off_rev + align256(rev.size() * sizeof(int)), 0);
    memcpy(blob.data() + off_tw_full, twf.data(), twf.size());
    memcpy(blob.data() + off_tw_stage, tws.data(), tws.size());
    if (!sup.empty()) memcpy(blob.data() + off_super, sup.data(), sup.size());
    memcpy(blob.data() + off_rev, rev.data(), rev.size() * sizeof(int));
    tab = KTab{};
    return true;
}

void Plan::bind(const void* base) {
    const uint8_t* b = (const uint8_t*)base;
    tab.tw_full = b + off_tw_full;
    tab.tw_stage = b + off_tw_stage;
    tab.super_tw = real_nfft > 0 ? (const void*)(b + off_super) : nullptr;
    tab.rev = (const int*)(b + off_rev);
}

// ------------------------------------------------------------- launch shapes
int cfg_smem_bytes(const KSub& sb, int dtype, int J) {
    const int esz = cpx_size(dtype);
    const int B = esz == 4 ? 5 : (esz == 8 ? 4 : 3);
    long long e = (long long)J * sb.L;
    e = (e + (1 << B) - 1) >> B << B;
    return (int)(e * esz);
}

static int max_R(const KSub& sb) {
    int r = 1;
    for (int k = 0; k < sb.npass; ++k) r = std::max(r, sb.ps[k].R);
    return r;
}

int cfg_min_threads(const KSub& sb, int mode, int J) {
    long long t = 32;
    for (int k = 0; k < sb.npass; ++k)
        if (sb.ps[k].kind == KIND_RT_GENERIC) t = std::max<long long>(t, ((long long)J * sb.L + KF_MAXO - 1) / KF_MAXO);
    if (mode == MODE_FIR) t = std::max<long long>(t, ((long long)J * (sb.L / 2 + 1) + KF_MAXO / 2 - 1) / (KF_MAXO / 2));
    return (int)((t + 31) / 32 * 32);
}

LaunchCfg default_cfg(const KSub& sb, int dtype, int mode, long long G, int col_in, int col_out, int want_threads) {
    LaunchCfg c;
    c.col_in = col_in;
    c.col_out = col_out;
    const int R = max_R(sb);
    const long long tpj = std::max(1, sb.L / R);
    const int budget = 96 * 1024;
    int J = 1;
    const bool col = col_in || col_out;
    while (J * 2 <= KF_MAXJ && J * 2 <= std::max<long long>(1, G) && cfg_smem_bytes(sb, dtype, J * 2) <= budget &&
           (tpj * J * 2 <= want_threads || (col && J < 16)))
        J *= 2;
    while (J > 1 && cfg_min_threads(sb, mode, J) > KF_MAXT) J /= 2;
    c.J = J;
    long long T = (tpj * J + 31) / 32 * 32;
    T = std::max<long long>(T, cfg_min_threads(sb, mode, J));
    T = std::min<long long>(std::max<long long>(T, 32), KF_MAXT);
    c.T = (int)T;
    c.smem = cfg_smem_bytes(sb, dtype, J);
    c.grid = (G + J - 1) / J;
    return c;
}

// ------------------------------------------------------------- schedules
static void set_shape(Step& st, const Plan& p, int sub) {
    st.shape_n = p.n;
    st.shape_inv = p.inverse;
    st.shape_sub = sub;
}

static KArgs base_args(const Plan& p, int s) {
    KArgs a;
    memset(&a, 0, sizeof(a));
    a.sub[0] = p.sub[s];
    a.tab[0] = p.tab;
    a.nsub = 1;
    return a;
}

int sub_family(const KSub& sb) { return family_of(sb); }

static int g_tma = -1;

void set_tma_enabled(int on) { g_tma = on ? 1 : 0; }

bool tma_enabled() {
    if (g_tma < 0) {
        const char* e = getenv("KISSFFT_GB300_TMA");
        g_tma = (e && e[0] == '0') ? 0 : 1;
    }
    return g_tma == 1;
}

bool enable_tma(Step& st, const void* in) {
    const KArgs& a = st.args;
    if (!tma_enabled() || !st.tma_ok || st.kind != 0 || (st.mode != MODE_C2C && st.mode != MODE_R2C)) return false;
    if (a.col_in || a.col_out || a.in_stride != 1 || a.in_dlo != 0 || a.G_lo != 1 || a.G_mid > 1 || a.in_off)
        return false;
    const long long L = a.sub[0].L, esz = cpx_size(st.dtype);
    if (a.in_dhi != L || (L * esz) % 16 != 0 || ((uintptr_t)in & 15) != 0) return false;
    const long long stage_off = ((long long)st.cfg.smem + 15) / 16 * 16;
    const long long total = stage_off + (long long)st.cfg.J * L * esz;
    if (total > 200 * 1024) return false;
    st.args.tma = 1;
    st.args.stage_off = (int)stage_off;
    st.cfg.smem = (int)total;
    return true;
}

// Column-layout tiles (jobs fastest in shared memory and in the group
// order) for a row-mode engine step: fewer bank conflicts for strides that
// the swizzle does not spread, at the price of shorter global runs (32/J
// elements of each job per warp access).
bool recolumn_step(Step& st) {
    if (st.kind != 0 || st.mode == MODE_FIR || st.args.col_in || st.args.col_out) return false;
    st.cfg.col_in = st.cfg.col_out = 1;
    st.args.col_in = st.args.col_out = 1;
    st.args.tma = 0;
    st.kfn = nullptr;
    return true;
}

static int default_minb(int T, int smem) {
    const int by_threads = 2048 / std::max(T, 32);
    const int by_smem = (227 * 1024) / std::max(smem + 1024, 1);
    const int by_regs = 65536 / (std::max(T, 32) * 64);  // keep >= 64 registers a thread
    return std::max(1, std::min(std::min(by_threads, by_smem), std::min(by_regs, 8)));
}

static void finish(Step& st, const LaunchCfg& c);

// Another thread count for an engine step (same tile): a multiple of 32 at
// least the step's minimum, so a pass's groups fill whole rounds.
bool retarget_threads(Step& st, int T) {
    if (st.kind != 0 || T < 32 || T > KF_MAXT || (T & 31)) return false;
    if (T < cfg_min_threads(st.args.sub[0], st.mode, st.cfg.J)) return false;
    st.cfg.T = T;
    st.cfg.minb = default_minb(T, st.cfg.smem);
    st.kfn = nullptr;
    return true;
}

bool reshape_step(Step& st, int J) {
    if (st.kind != 0 || J < 1 || J > KF_MAXJ || (J & (J - 1))) return false;
    const KSub& sb = st.args.sub[0];
    LaunchCfg c = st.cfg;
    int R = 1;
    for (int k = 0; k < sb.npass; ++k) R = std::max(R, sb.ps[k].R);
    const long long tpj = std::max(1, sb.L / R);
    long long T = (tpj * J + 31) / 32 * 32;
    T = std::max<long long>(T, cfg_min_threads(sb, st.mode, J));
    if (T > KF_MAXT || cfg_smem_bytes(sb, st.dtype, J) > 200 * 1024) return false;
    c.J = J;
    c.T = (int)std::max<long long>(T, 32);
    c.smem = cfg_smem_bytes(sb, st.dtype, J);
    c.grid = (st.args.G + J - 1) / J;
    st.args.tma = 0;
    st.args.stage_off = 0;
    finish(st, c);
    return true;
}

// Default shared-tile index map of a launch (kf_engine.cuh swz): the
// XOR fold for IEEE tiles whose strides are even; none for odd-length
// (generic-radix) tiles and for fixed point, whose integer-issue-bound
// passes gain more from the saved instructions than they lose to bank
// conflicts (measured over the 480/1000/3003/65536 workload).
int default_swz(int dtype, int L) {
    if (dtype == KF_Q15 || dtype == KF_Q31) return SWZ_NONE;
    return (L & 1) ? SWZ_NONE : SWZ_FOLD;
}

static void finish(Step& st, const LaunchCfg& c) {
    st.kfn = nullptr;
    st.args.swz = default_swz(st.dtype, st.args.sub[0].L);
    st.fam = sub_family(st.args.sub[0]);
    if (st.args.nsub > 1) st.fam = std::max(st.fam, sub_family(st.args.sub[1]));
    st.cfg = c;
    st.cfg.minb = default_minb(c.T, c.smem);
    st.args.J = c.J;
    st.args.col_in = c.col_in;
    st.args.col_out = c.col_out;
    int lj = 0;
    while ((1 << lj) < c.J) ++lj;
    st.args.logJ = lj;
    st.args.ntiles = c.grid;
}

// The kernels index one transform's elements as (local offset) * stride in
// 32-bit arithmetic (per-transform bases are 64-bit).  A schedule whose
// strides would leave that range (huge N-D arrays, huge kiss_fft_stride
// strides) is refused here, on the host, instead of addressing wrong memory.
static bool fits(Schedule& s) {
    const long long lim = 0x7fffffffLL;
    for (const Step& st : s.steps) {
        if (st.kind != 0) continue;
        const KArgs& a = st.args;
        long long L = a.sub[0].L;
        if (a.nsub > 1) L = std::max<long long>(L, a.sub[1].L);
        const long long stride = std::max(a.in_stride, a.out_stride);
        if (stride > lim || (L - 1) * stride > lim) {
            s.error = "element strides of this call exceed the kernels' 32-bit in-transform offsets";
            s.steps.clear();
            return false;
        }
    }
    return true;
}

bool schedule_c2c(const Plan& p, long long batch, long long in_dist, long long in_stride, long long out_dist,
                  Schedule& s) {
    s.steps.clear();
    s.scratch[0] = s.scratch[1] = 0;
    const int esz = cpx_size(p.dtype);
    if (p.nsub == 1) {
        Step st;
        st.mode = MODE_C2C;
        st.dtype = p.dtype;
        st.args = base_args(p, 0);
        set_shape(st, p, 0);
        st.args.G = batch;
        st.args.G_lo = 1;
        st.args.in_dhi = in_dist;
        st.args.in_stride = in_stride;
        st.args.out_dhi = out_dist;
        st.args.out_stride = 1;
        finish(st, default_cfg(p.sub[0], p.dtype, MODE_C2C, batch, 0, 0));
        s.steps.push_back(st);
        return fits(s);
    }
    const long long Ps = p.sub[1].L, LA = p.sub[0].L, n = p.n;
    Step a;
    a.mode = MODE_C2C;
    a.dtype = p.dtype;
    a.args = base_args(p, 0);
    set_shape(a, p, 0);
    a.args.G = batch * Ps;
    a.args.G_lo = Ps;
    a.args.in_dhi = in_dist;
    a.args.in_dlo = in_stride;
    a.args.in_stride = Ps * in_stride;
    a.args.out_dhi = n;
    a.args.out_dlo = 1;
    a.args.out_stride = Ps;
    a.in_role = 0;
    a.out_role = 2;
    finish(a, default_cfg(p.sub[0], p.dtype, MODE_C2C, a.args.G, 1, 1));
    Step b;
    b.mode = MODE_C2C;
    b.dtype = p.dtype;
    b.args = base_args(p, 1);
    set_shape(b, p, 1);
    b.args.G = batch * LA;
    b.args.G_lo = LA;
    b.args.in_dhi = n;
    b.args.in_dlo = Ps;
    b.args.in_stride = 1;
    b.args.out_dhi = out_dist;
    b.args.out_dlo = 1;
    b.args.out_stride = LA;
    b.args.use_u = 1;
    b.in_role = 2;
    b.out_role = 1;
    finish(b, default_cfg(p.sub[1], p.dtype, MODE_C2C, b.args.G, 0, 1));
    s.steps.push_back(a);
    s.steps.push_back(b);
    s.scratch[0] = (size_t)batch * n * esz;
    return fits(s);
}

// Real split / merge as separate elementwise launches (two-pass real plans).
static Step elementwise(int kind, const Plan& p, long long batch, long long in_dist, long long out_dist, int in_role,
                        int out_role) {
    Step st;
    st.kind = kind;
    st.dtype = p.dtype;
    st.args = base_args(p, 0);
    set_shape(st, p, 0);
    st.args.sub[0].L = p.n;  // ncfft for the element kernels
    st.args.G = batch;
    st.args.in_dhi = in_dist;
    st.args.out_dhi = out_dist;
    st.in_role = in_role;
    st.out_role = out_role;
    long long items = batch * (p.n / 2 + 1);
    st.cfg.T = 256;
    st.cfg.grid = (items + 255) / 256;
    st.cfg.J = 1;
    st.args.ntiles = st.cfg.grid;
    return st;
}

bool schedule_r2c(const Plan& p, long long batch, long long in_dist, long long out_dist, Schedule& s, int in_role,
                  int out_role) {
    s.steps.clear();
    s.scratch[0] = s.scratch[1] = 0;
    if (p.real_nfft <= 0 || (in_dist & 1)) {
        s.error = "real transform needs a real plan and an even row distance";
        return false;
    }
    const int esz = cpx_size(p.dtype);
    if (p.nsub == 1) {
        Step st;
        st.mode = MODE_R2C;
        st.dtype = p.dtype;
        st.args = base_args(p, 0);
        set_shape(st, p, 0);
        st.args.G = batch;
        st.args.G_lo = 1;
        st.args.in_dhi = in_dist / 2;
        st.args.in_stride = 1;
        st.args.out_dhi = out_dist;
        st.args.out_stride = 1;
        st.in_role = in_role;
        st.out_role = out_role;
        finish(st, default_cfg(p.sub[0], p.dtype, MODE_R2C, batch, 0, 0));
        s.steps.push_back(st);
        return fits(s);
    }
    Schedule c;
    schedule_c2c(p, batch, in_dist / 2, 1, p.n, c);
    c.steps.front().in_role = in_role;
    c.steps.back().out_role = 3;
    for (auto& st : c.steps) s.steps.push_back(st);
    s.steps.push_back(elementwise(1, p, batch, p.n, out_dist, 3, out_role));
    s.scratch[0] = c.scratch[0];
    s.scratch[1] = (size_t)batch * p.n * esz;
    return fits(s);
}

bool schedule_c2r(const Plan& p, long long batch, long long in_dist, long long out_dist, Schedule& s, int in_role,
                  int out_role) {
    s.steps.clear();
    s.scratch[0] = s.scratch[1] = 0;
    if (p.real_nfft <= 0 || (out_dist & 1)) {
        s.error = "real transform needs a real plan and an even row distance";
        return false;
    }
    const int esz = cpx_size(p.dtype);
    if (p.nsub == 1) {
        Step st;
        st.mode = MODE_C2R;
        st.dtype = p.dtype;
        st.args = base_args(p, 0);
        set_shape(st, p, 0);
        st.args.G = batch;
        st.args.G_lo = 1;
        st.args.in_dhi = in_dist;
        st.args.in_stride = 1;
        st.args.out_dhi = out_dist / 2;
        st.args.out_stride = 1;
        st.in_role = in_role;
        st.out_role = out_role;
        finish(st, default_cfg(p.sub[0], p.dtype, MODE_C2R, batch, 0, 0));
        s.steps.push_back(st);
        return fits(s);
    }
    s.steps.push_back(elementwise(2, p, batch, in_dist, p.n, in_role, 3));
    Schedule c;
    schedule_c2c(p, batch, p.n, 1, out_dist / 2, c);
    c.steps.front().in_role = 3;
    c.steps.back().out_role = out_role;
    for (auto& st : c.steps) s.steps.push_back(st);
    s.scratch[0] = c.scratch[0];
    s.scratch[1] = (size_t)batch * p.n * esz;
    return fits(s);
}

bool schedule_axis(const Plan& p, const int* dims, int ndims, int axis, long long batch, int in_role, int out_role,
                   Schedule& s, int tmp_role) {
    s.steps.clear();
    s.scratch[0] = s.scratch[1] = 0;
    long long S = 1, outer = batch;
    for (int i = axis + 1; i < ndims; ++i) S *= dims[i];
    for (int i = 0; i < axis; ++i) outer *= dims[i];
    const long long n = dims[axis];
    if (p.nsub != 1) {
        // An axis longer than one tile: its fibers (outer o, offset s; element
        // m at o*n*S + m*S + s) run as the two HBM passes of schedule_c2c.
        // Pass 1, job (o, s, j < Ps): elements j + k*Ps of the fiber, written
        // to the intermediate with every fiber contiguous (o*n*S + s*n + m);
        // pass 2, job (o, s, j < LA): intermediate elements j*Ps + k, written
        // back to positions j + k*LA of the fiber.
        if (tmp_role != 2 && tmp_role != 3) {
            s.error = "N-D axis: bad intermediate buffer";
            return false;
        }
        const long long Ps = p.sub[1].L, LA = p.sub[0].L;
        const int esz = cpx_size(p.dtype);
        Step a;
        a.mode = MODE_C2C;
        a.dtype = p.dtype;
        a.args = base_args(p, 0);
        set_shape(a, p, 0);
        a.args.G = outer * S * Ps;
        a.args.G_lo = Ps;
        a.args.G_mid = S;
        a.args.in_dhi = n * S;
        a.args.in_dmid = 1;
        a.args.in_dlo = S;
        a.args.in_stride = Ps * S;
        a.args.out_dhi = n * S;
        a.args.out_dmid = n;
        a.args.out_dlo = 1;
        a.args.out_stride = Ps;
        a.in_role = in_role;
        a.out_role = tmp_role;
        finish(a, default_cfg(p.sub[0], p.dtype, MODE_C2C, a.args.G, 1, 1));
        Step b;
        b.mode = MODE_C2C;
        b.dtype = p.dtype;
        b.args = base_args(p, 1);
        set_shape(b, p, 1);
        b.args.G = outer * S * LA;
        b.args.G_lo = LA;
        b.args.G_mid = S;
        b.args.in_dhi = n * S;
        b.args.in_dmid = n;
        b.args.in_dlo = Ps;
        b.args.in_stride = 1;
        b.args.out_dhi = n * S;
        b.args.out_dmid = 1;
        b.args.out_dlo = S;
        b.args.out_stride = LA * S;
        b.args.use_u = 1;
        b.in_role = tmp_role;
        b.out_role = out_role;
        finish(b, default_cfg(p.sub[1], p.dtype, MODE_C2C, b.args.G, 0, 1));
        s.steps.push_back(a);
        s.steps.push_back(b);
        s.scratch[tmp_role - 2] = (size_t)(outer * S * n) * esz;
        return fits(s);
    }
    Step st;
    st.mode = MODE_C2C;
    st.dtype = p.dtype;
    st.args = base_args(p, 0);
    set_shape(st, p, 0);
    st.in_role = in_role;
    st.out_role = out_role;
    if (S == 1) {
        st.args.G = outer;
        st.args.G_lo = 1;
        st.args.in_dhi = n;
        st.args.in_stride = 1;
        st.args.out_dhi = n;
        st.args.out_stride = 1;
        finish(st, default_cfg(p.sub[0], p.dtype, MODE_C2C, st.args.G, 0, 0));
    } else {
        st.args.G = outer * S;
        st.args.G_lo = S;
        st.args.in_dhi = n * S;
        st.args.in_dlo = 1;
        st.args.in_stride = S;
        st.args.out_dhi = n * S;
        st.args.out_dlo = 1;
        st.args.out_stride = S;
        finish(st, default_cfg(p.sub[0], p.dtype, MODE_C2C, st.args.G, 1, 1));
    }
    s.steps.push_back(st);
    return fits(s);
}

bool schedule_fastfir(const Plan& fw, const Plan& iv, long long L, long long Ns, long long, Schedule& s) {
    s.steps.clear();
    s.scratch[0] = s.scratch[1] = 0;
    const long long nfft = fw.real_nfft;
    if (fw.nsub != 1 || iv.nsub != 1 || nfft <= 0) {
        s.error = "fast FIR block does not fit one tile";
        return false;
    }
    if (sub_family(fw.sub[0]) > FAM_SMOOTH) {
        s.error = "fast FIR block size must have only the factors 2, 3 and 5";
        return false;
    }
    const long long ngood = nfft - L + 1, nout = Ns - L + 1;
    if (ngood < 1 || nout < 0) {
        s.error = "bad fast FIR sizes";
        return false;
    }
    Step st;
    st.mode = MODE_FIR;
    st.dtype = fw.dtype;
    st.args = base_args(fw, 0);
    set_shape(st, fw, 0);
    st.args.sub[1] = iv.sub[0];
    st.args.tab[1] = iv.tab;
    st.args.nsub = 2;
    st.args.G = (nout + ngood - 1) / ngood;
    st.args.G_lo = 1;
    st.args.in_dhi = ngood;
    st.args.in_stride = 1;
    st.args.out_dhi = ngood;
    st.args.out_stride = 1;
    st.args.in_limit = Ns;
    st.args.out_limit = nout;
    st.args.fir_ngood = (int)ngood;
    finish(st, default_cfg(fw.sub[0], fw.dtype, MODE_FIR, st.args.G, 0, 0));
    if (st.args.G > 0) s.steps.push_back(st);
    return fits(s);
}

}  // namespace kf
