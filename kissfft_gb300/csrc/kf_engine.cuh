// The register-pass FFT engine (host/device code: the CUDA kernels run it,
// and the CPU emulator used by the tests runs the very same functions).
//
// A sub-plan's stages are grouped into passes of one or two stages.  In a
// pass every thread takes groups of R elements: R = p (one stage) or
// pa*pb (two stages, run on registers without an exchange in between).
// The first pass reads its group straight from HBM (input order is the
// natural order of the input samples, so consecutive threads read
// consecutive samples); the last pass writes its group straight to HBM in
// position order (= output order).  Between passes the tile lives in shared
// memory at index I = A*sA + job*sJ (A = input-order index), XOR-swizzled
// so that both the input-order and the position-order sweeps are
// bank-conflict free for power-of-two strides.
//
// Every function takes the sub-plan shape (KSub, integers only) and its
// device tables (KTab) separately: a specialised kernel passes a
// compile-time constant shape and the compiler folds every stride.
#pragma once

#include "kf_arith.cuh"
#include "kf_desc.h"
#include "kf_shape.h"

#if !defined(__CUDACC__) && !defined(__CUDACC_RTC__)
// host compilers (the CPU emulator): the CUDA vector types used below
struct uint2 {
    unsigned x, y;
};
struct alignas(16) uint4 {
    unsigned x, y, z, w;
};
#endif

namespace kf {

// unrolling of the output-leg loop of the fixed-point generic radix (2 was
// the fastest of 1, 2 and 13 for Q15/Q31 3003)
constexpr int kGenUnroll = 2;

// Read-only (non-coherent cache) loads of tables: twiddles, reverse
// tables.  The raw words go through aligned unions (no memcpy: NVRTC has no
// C library).
template <typename T, typename V>
union KfPun {
    V v;
    T t;
};

// Memory-access hook: every shared-tile, global-buffer and table access of
// the engine is marked with KF_MEM_CHECK(p, bytes).  It expands to nothing
// unless the includer defines KF_MEM_NOTE(p, bytes); the CPU emulator of the
// engine does, and checks each access against the buffers of its run.
#if defined(KF_MEM_NOTE)
#define KF_MEM_CHECK(p, n) KF_MEM_NOTE((const void*)(p), (size_t)(n))
#else
#define KF_MEM_CHECK(p, n) ((void)0)
#endif

template <typename T>
KF_HD T ldro(const T* p) {
    KF_MEM_CHECK(p, sizeof(T));
#if defined(__CUDA_ARCH__)
    if constexpr (sizeof(T) == 4) {
        KfPun<T, unsigned> u;
        u.v = __ldg((const unsigned*)p);
        return u.t;
    } else if constexpr (sizeof(T) == 8) {
        KfPun<T, uint2> u;
        u.v = __ldg((const uint2*)p);
        return u.t;
    } else if constexpr (sizeof(T) == 16) {
        KfPun<T, uint4> u;
        u.v = __ldg((const uint4*)p);
        return u.t;
    } else {
        return *p;
    }
#else
    return *p;
#endif
}
#define KF_LDG(p) ::kf::ldro(p)

template <typename S, int W>
struct KfVec {
    static constexpr int bytes = W * (int)sizeof(cpx<S>);
    static constexpr int nu = bytes >= 16 ? bytes / 16 : 1;
    union U {
        uint4 q[nu];
        uint2 d;
        unsigned w;
        cpx<S> c[W];
    };
};

// W consecutive complex table entries; the caller guarantees alignment to
// min(16, W*sizeof(cpx)) bytes.
template <typename S, int W>
KF_HD void ldro_vec(const cpx<S>* p, cpx<S>* out) {
    KF_MEM_CHECK(p, W * sizeof(cpx<S>));
#if defined(__CUDA_ARCH__)
    typename KfVec<S, W>::U u;
    constexpr int bytes = KfVec<S, W>::bytes;
    if constexpr (bytes >= 16) {
#pragma unroll
        for (int i = 0; i < bytes / 16; ++i) u.q[i] = __ldg((const uint4*)p + i);
    } else if constexpr (bytes == 8) {
        u.d = __ldg((const uint2*)p);
    } else {
        u.w = __ldg((const unsigned*)p);
    }
#pragma unroll
    for (int i = 0; i < W; ++i) out[i] = u.c[i];
#else
    for (int i = 0; i < W; ++i) out[i] = p[i];
#endif
}

// n / d for n * d < 2^40 with M = div_magic(d)
KF_HD int fdiv(int n, unsigned long long M) { return (int)(((unsigned long long)(unsigned)n * M) >> 40); }

template <typename S>
struct SwzBits {
    static constexpr int v = sizeof(cpx<S>) == 4 ? 5 : (sizeof(cpx<S>) == 8 ? 4 : 3);
};

// Shared-tile index map inside aligned blocks of 2^B elements (a bijection):
//   SWZ_FOLD  XOR of the three next digit groups into the low B bits --
//             conflict-free sweeps for power-of-two strides;
//   SWZ_ONE   XOR of the next digit group only (two instructions);
//   SWZ_NONE  identity -- odd strides (generic radices) need no spreading,
//             and integer-issue-bound fixed-point tiles gain more from the
//             saved instructions than they lose to conflicts.
// The launch picks the map (KArgs::swz; the autotuner times all three).
template <typename S>
KF_HD int swz(int I, int mode) {
    constexpr int B = SwzBits<S>::v;
    if (mode == SWZ_NONE) return I;
    if (mode == SWZ_ONE) return I ^ ((I >> B) & ((1 << B) - 1));
    const int f = (I >> B) ^ (I >> (2 * B)) ^ (I >> (3 * B));
    return I ^ (f & ((1 << B) - 1));
}

// Per-tile view: shared tile, job table, global pointers.
template <typename S>
struct Tile {
    typedef cpx<S> C;
    C* sm;
    int sA, sJ;  // shared index strides of the input-order index and of the job
    int J, logJ, col;
    int swzm;    // index map (swz)
    int T;       // threads working on the tile
    int in_stride, out_stride;
    const long long* inb;
    const long long* outb;
    const int* U;
    const long long* lim_in;   // real-input limit (fast FIR)
    const long long* lim_out;  // real-output limit (fast FIR)
    const void* in;
    void* out;
    int* err;

    KF_HD int sidx(int A, int job) const { return swz<S>(A * sA + job * sJ, swzm); }
    KF_HD C sld(int A, int job) const { return (KF_MEM_CHECK(sm + sidx(A, job), sizeof(C)), sm[sidx(A, job)]); }
    KF_HD void sst(int A, int job, C v) const { (KF_MEM_CHECK(sm + sidx(A, job), sizeof(C)), sm[sidx(A, job)] = v); }
    KF_HD bool valid(int job) const { return inb[job] >= 0; }
};

// ------------------------------------------------------------ global access
// A group's HBM base: element k sits at base + off_k * stride.  MODE_FIR
// moves real samples with limits (zero padding on input) instead.
template <typename S, int MODE>
struct GIn {
    const cpx<S>* p;
    const S* r;
    long long lim;
    int stride;
    KF_HD cpx<S> ld(int off) const {
        cpx<S> v;
        if constexpr (MODE == MODE_FIR) {
            const long long i0 = 2LL * off;
            v.r = i0 < lim ? (KF_MEM_CHECK(r + i0, sizeof(S)), r[i0]) : (S)0;
            v.i = i0 + 1 < lim ? (KF_MEM_CHECK(r + i0 + 1, sizeof(S)), r[i0 + 1]) : (S)0;
        } else {
            v = (KF_MEM_CHECK(p + (long long)(off * stride), sizeof(v)), p[(long long)(off * stride)]);
        }
        return v;
    }
};

template <typename S, int MODE>
KF_HD GIn<S, MODE> gin(const Tile<S>& t, int job, int A0) {
    GIn<S, MODE> g;
    g.stride = t.in_stride;
    if constexpr (MODE == MODE_FIR) {
        g.r = (const S*)t.in + t.inb[job] + 2LL * A0;
        g.lim = t.lim_in[job] - 2LL * A0;
        g.p = nullptr;
    } else {
        g.p = (const cpx<S>*)t.in + t.inb[job] + (long long)A0 * t.in_stride;
        g.r = nullptr;
        g.lim = 0;
    }
    return g;
}

template <typename S, int MODE>
struct GOut {
    cpx<S>* p;
    S* r;
    long long lim;
    int stride;
    KF_HD void st(int off, cpx<S> v) const {
        if constexpr (MODE == MODE_FIR) {
            const long long i0 = 2LL * off;
            if (i0 < lim) (KF_MEM_CHECK(r + i0, sizeof(S)), r[i0] = v.r);
            if (i0 + 1 < lim) (KF_MEM_CHECK(r + i0 + 1, sizeof(S)), r[i0 + 1] = v.i);
        } else {
            (KF_MEM_CHECK(p + (long long)(off * stride), sizeof(v)), p[(long long)(off * stride)] = v);
        }
    }
};

template <typename S, int MODE>
KF_HD GOut<S, MODE> gout(const Tile<S>& t, int job, int pos0) {
    GOut<S, MODE> g;
    g.stride = t.out_stride;
    if constexpr (MODE == MODE_FIR) {
        g.r = (S*)t.out + t.outb[job] + 2LL * pos0;
        g.lim = t.lim_out[job] - 2LL * pos0;
        g.p = nullptr;
    } else {
        g.p = (cpx<S>*)t.out + t.outb[job] + (long long)pos0 * t.out_stride;
        g.r = nullptr;
        g.lim = 0;
    }
    return g;
}

// ------------------------------------------------------------ group decode
struct GroupIx {
    int job, A0, pos0, ul;
};

// gidx enumerates the groups of a pass over the whole tile: jobs fastest in
// column mode (coalesced across jobs), digits fastest in row mode.
// Non-last passes enumerate the lower digits in input order (conflict-free
// shared sweeps); the last pass enumerates them in position order
// (coalesced output) and uses the reverse table.
KF_HD GroupIx decode(const KPass& ps, const KTab& tb, int J, int logJ, int col, bool is_last, int gidx) {
    GroupIx g;
    int r;
    if (col) {
        g.job = gidx & (J - 1);
        r = gidx >> logJ;
    } else if (J == 1) {
        g.job = 0;
        r = gidx;
    } else {
        g.job = fdiv(gidx, ps.gdiv);
        r = gidx - g.job * (ps.H * ps.ML);
    }
    int h, ulp, ul;
    if (is_last) {
        h = 0;
        ul = r;
        ulp = ps.ML > 1 ? KF_LDG(tb.rev + ps.rev_off + ul) : 0;
    } else {
        ulp = ps.H > 1 ? fdiv(r, ps.hdiv) : r;
        h = r - ulp * ps.H;
        ul = ps.ML > 1 ? KF_LDG(tb.rev + ps.rev_off + ulp) : 0;
    }
    g.A0 = h + ulp * ps.H * ps.R;
    g.pos0 = ul;
    g.ul = ul;
    return g;
}

// The twiddles of butterfly u of a radix-P stage and the stage's constants,
// as Ar<S>::CW (the compact table's entries; Q15 tables hold them widened).
template <typename S, int P>
KF_HD void stage_tw(const KTab& tb, const KStage& st, int u, typename Ar<S>::CW* w, typename Ar<S>::CW& c0,
                    typename Ar<S>::CW& c1) {
    typedef typename Ar<S>::CW CW;
    typedef typename Ar<S>::W Wt;
    constexpr int W = P == 2 ? 1 : (P == 3 ? 2 : 4);
    const CW* tws = (const CW*)((const cpx<S>*)tb.tw_stage + st.tw_off);
    CW v[W];
    ldro_vec<Wt, W>(tws + u * W, v);
#pragma unroll
    for (int q = 1; q < P; ++q) w[q - 1] = v[q - 1];
    if constexpr (P == 3 || P == 5) c0 = KF_LDG(tws + W * st.m);
    if constexpr (P == 5) c1 = KF_LDG(tws + W * st.m + 1);
}

// ------------------------------------------------------------ group kernels
// One stage of radix P (2..5) on a group of P elements.
template <typename S, int MODE, int P>
KF_HD void group1(const Tile<S>& t, const KSub& sb, const KTab& tb, const KPass& ps, const GroupIx& g, int U,
                  bool src_g, bool dst_g) {
    typedef cpx<S> C;
    const KStage& sa = sb.st[ps.a];
    C x[P];
    if (src_g) {
        const GIn<S, MODE> gi = gin<S, MODE>(t, g.job, g.A0);
#pragma unroll
        for (int q = 0; q < P; ++q) x[q] = gi.ld(q * sa.iloc);
    } else {
#pragma unroll
        for (int q = 0; q < P; ++q) x[q] = t.sld(g.A0 + q * sa.iloc, g.job);
    }
    typename Ar<S>::CW w[P > 1 ? P - 1 : 1], c0, c1;
    stage_tw<S, P>(tb, sa, g.ul * sb.m_low + U, w, c0, c1);
    bfly<S, P, 1>(x, w, c0, c1, sb.inverse != 0);
    if (dst_g) {
        const GOut<S, MODE> go = gout<S, MODE>(t, g.job, g.pos0);
#pragma unroll
        for (int q = 0; q < P; ++q) go.st(q * sa.mloc, x[q]);
    } else {
#pragma unroll
        for (int q = 0; q < P; ++q) t.sst(g.A0 + q * sa.iloc, g.job, x[q]);
    }
}

// Two stages: stage a+1 (radix PB) then stage a (radix PA), element
// (ea, eb) at register k = ea + PA*eb.
template <typename S, int MODE, int PA, int PB>
KF_HD void group2(const Tile<S>& t, const KSub& sb, const KTab& tb, const KPass& ps, const GroupIx& g, int U,
                  bool src_g, bool dst_g) {
    typedef cpx<S> C;
    const KStage& sa = sb.st[ps.a];
    const KStage& sbb = sb.st[ps.a + 1];
    C x[PA * PB];
    if (src_g) {
        const GIn<S, MODE> gi = gin<S, MODE>(t, g.job, g.A0);
#pragma unroll
        for (int eb = 0; eb < PB; ++eb)
#pragma unroll
            for (int ea = 0; ea < PA; ++ea) x[ea + PA * eb] = gi.ld(ea * sa.iloc + eb * sbb.iloc);
    } else {
#pragma unroll
        for (int eb = 0; eb < PB; ++eb)
#pragma unroll
            for (int ea = 0; ea < PA; ++ea) x[ea + PA * eb] = t.sld(g.A0 + ea * sa.iloc + eb * sbb.iloc, g.job);
    }
    {
        typename Ar<S>::CW w[PB - 1], c0, c1;
        stage_tw<S, PB>(tb, sbb, g.ul * sb.m_low + U, w, c0, c1);
#pragma unroll
        for (int ea = 0; ea < PA; ++ea) bfly<S, PB, PA>(x + ea, w, c0, c1, sb.inverse != 0);
    }
#pragma unroll
    for (int eb = 0; eb < PB; ++eb) {
        typename Ar<S>::CW w[PA - 1], c0, c1;
        stage_tw<S, PA>(tb, sa, (eb * sbb.mloc + g.ul) * sb.m_low + U, w, c0, c1);
        bfly<S, PA, 1>(x + PA * eb, w, c0, c1, sb.inverse != 0);
    }
    if (dst_g) {
        const GOut<S, MODE> go = gout<S, MODE>(t, g.job, g.pos0);
#pragma unroll
        for (int eb = 0; eb < PB; ++eb)
#pragma unroll
            for (int ea = 0; ea < PA; ++ea) go.st(ea * sa.mloc + eb * sbb.mloc, x[ea + PA * eb]);
    } else {
#pragma unroll
        for (int eb = 0; eb < PB; ++eb)
#pragma unroll
            for (int ea = 0; ea < PA; ++ea) t.sst(g.A0 + ea * sa.iloc + eb * sbb.iloc, g.job, x[ea + PA * eb]);
    }
}

// Three stages: stage a+2 (radix PC), then a+1 (PB), then a (PA); element
// (ea, eb, ec) at register k = ea + PA*(eb + PB*ec).  Stage s of the group
// takes the twiddle row of u = (sum of the deeper group digits * their mloc
// + ul) * m_low + U, as in group2.
template <typename S, int MODE, int PA, int PB, int PC>
KF_HD void group3(const Tile<S>& t, const KSub& sb, const KTab& tb, const KPass& ps, const GroupIx& g, int U,
                  bool src_g, bool dst_g) {
    typedef cpx<S> C;
    const KStage& sa = sb.st[ps.a];
    const KStage& sbb = sb.st[ps.a + 1];
    const KStage& sc = sb.st[ps.a + 2];
    C x[PA * PB * PC];
    if (src_g) {
        const GIn<S, MODE> gi = gin<S, MODE>(t, g.job, g.A0);
#pragma unroll
        for (int ec = 0; ec < PC; ++ec)
#pragma unroll
            for (int eb = 0; eb < PB; ++eb)
#pragma unroll
                for (int ea = 0; ea < PA; ++ea)
                    x[ea + PA * (eb + PB * ec)] = gi.ld(ea * sa.iloc + eb * sbb.iloc + ec * sc.iloc);
    } else {
#pragma unroll
        for (int ec = 0; ec < PC; ++ec)
#pragma unroll
            for (int eb = 0; eb < PB; ++eb)
#pragma unroll
                for (int ea = 0; ea < PA; ++ea)
                    x[ea + PA * (eb + PB * ec)] = t.sld(g.A0 + ea * sa.iloc + eb * sbb.iloc + ec * sc.iloc, g.job);
    }
    {
        typename Ar<S>::CW w[PC - 1], c0, c1;
        stage_tw<S, PC>(tb, sc, g.ul * sb.m_low + U, w, c0, c1);
#pragma unroll
        for (int k = 0; k < PA * PB; ++k) bfly<S, PC, PA * PB>(x + k, w, c0, c1, sb.inverse != 0);
    }
#pragma unroll
    for (int ec = 0; ec < PC; ++ec) {
        typename Ar<S>::CW w[PB - 1], c0, c1;
        stage_tw<S, PB>(tb, sbb, (ec * sc.mloc + g.ul) * sb.m_low + U, w, c0, c1);
#pragma unroll
        for (int ea = 0; ea < PA; ++ea) bfly<S, PB, PA>(x + ea + PA * PB * ec, w, c0, c1, sb.inverse != 0);
    }
#pragma unroll
    for (int ec = 0; ec < PC; ++ec)
#pragma unroll
        for (int eb = 0; eb < PB; ++eb) {
            typename Ar<S>::CW w[PA - 1], c0, c1;
            stage_tw<S, PA>(tb, sa, (eb * sbb.mloc + ec * sc.mloc + g.ul) * sb.m_low + U, w, c0, c1);
            bfly<S, PA, 1>(x + PA * (eb + PB * ec), w, c0, c1, sb.inverse != 0);
        }
    if (dst_g) {
        const GOut<S, MODE> go = gout<S, MODE>(t, g.job, g.pos0);
#pragma unroll
        for (int ec = 0; ec < PC; ++ec)
#pragma unroll
            for (int eb = 0; eb < PB; ++eb)
#pragma unroll
                for (int ea = 0; ea < PA; ++ea)
                    go.st(ea * sa.mloc + eb * sbb.mloc + ec * sc.mloc, x[ea + PA * (eb + PB * ec)]);
    } else {
#pragma unroll
        for (int ec = 0; ec < PC; ++ec)
#pragma unroll
            for (int eb = 0; eb < PB; ++eb)
#pragma unroll
                for (int ea = 0; ea < PA; ++ea)
                    t.sst(g.A0 + ea * sa.iloc + eb * sbb.iloc + ec * sc.iloc, g.job, x[ea + PA * (eb + PB * ec)]);
    }
}

// Generic radix P (a prime 7..31) on registers.
//
// Fixed point follows kf_bfly_generic (kiss_fft.c:192-233) exactly: output
// leg q1 sums legs q = 0..P-1 in order, each product rounded, with twiddle
// index (q*fstride*k) mod N, k = u + q1*m.  Those P-1 twiddles of every
// (u, q1) are one row of the stage's compact table (kf_shape.h gen_row),
// read with vector loads; the sum is kept untruncated until the store.
//
// IEEE types (no bit-exactness to keep, only the error bound) multiply the
// legs by tw[q*fstride*u] first and then take the size-P DFT on the table's
// P-th roots, pairing legs q and P-q: about a quarter of the flops.
template <typename S, int MODE, int P>
KF_HD void groupg(const Tile<S>& t, const KSub& sb, const KTab& tb, const KPass& ps, const GroupIx& g, int U,
                  bool src_g, bool dst_g) {
    typedef cpx<S> C;
    typedef Ar<S> Arr;
    constexpr bool kFixed = sizeof(typename Arr::W) == 4 && (S)0.5 == (S)0;
    typedef typename Arr::CW CW;
    const KStage& sa = sb.st[ps.a];
    const C* tw = (const C*)tb.tw_full;
    CW x[P];
    if (src_g) {
        const GIn<S, MODE> gi = gin<S, MODE>(t, g.job, g.A0);
#pragma unroll
        for (int q = 0; q < P; ++q) x[q] = Arr::template fixdiv_w<P>(Arr::widen(gi.ld(q * sa.iloc)));
    } else {
#pragma unroll
        for (int q = 0; q < P; ++q) x[q] = Arr::template fixdiv_w<P>(Arr::widen(t.sld(g.A0 + q * sa.iloc, g.job)));
    }
    const int u = g.ul * sb.m_low + U;
    const int N = sb.N;
    const int NP = sa.fs * sa.m;  // N / P
    GOut<S, MODE> go{};
    if (dst_g) go = gout<S, MODE>(t, g.job, g.pos0);
    C y[P];
    if constexpr (kFixed) {
        typedef typename Arr::W W;
        constexpr int RP = gen_row(P);
        // twiddles as W pairs (Q15 rows are pre-widened, kf_shape.h tw_units)
        const CW* row = (const CW*)((const C*)tb.tw_stage + sa.tw_off) + (long long)u * P * RP;
#if defined(__CUDA_ARCH__)
        // Q31: doubled legs for Ar::gen_out_q31
        W x2r[P], x2i[P], x2n[P];
        if constexpr (sizeof(S) == 4) {
#pragma unroll
            for (int q = 1; q < P; ++q) {
                x2r[q] = (W)((unsigned)x[q].r << 1);
                x2i[q] = (W)((unsigned)x[q].i << 1);
                x2n[q] = (W)(0u - ((unsigned)x[q].i << 1));
            }
        }
#endif
#pragma unroll kGenUnroll
        for (int q1 = 0; q1 < P; ++q1) {
            CW w[RP];
            ldro_vec<W, RP>(row + q1 * RP, w);
            C acc;
#if defined(__CUDA_ARCH__)
            if constexpr (sizeof(S) == 4) {
                acc = Arr::template gen_out_q31<P>(x[0], x2r, x2i, x2n, w);
            } else
#endif
            {
                W ar = x[0].r, ai = x[0].i;
#pragma unroll
                for (int q = 1; q < P; ++q) Arr::cmul_acc_w(ar, ai, x[q], w[q - 1]);
                acc.r = Arr::st(ar);
                acc.i = Arr::st(ai);
            }
            if (dst_g)
                go.st(q1 * sa.mloc, acc);
            else
                t.sst(g.A0 + q1 * sa.iloc, g.job, acc);
        }
        (void)tw;
        (void)N;
        (void)NP;
        return;
    } else {
        constexpr int h = (P - 1) / 2;
        if (u != 0) {
            int idx = 0;
            const int step = sa.fs * u;
#pragma unroll
            for (int q = 1; q < P; ++q) {
                idx += step;
                if (idx >= N) idx -= N;
                x[q] = Arr::cmul_w(x[q], KF_LDG(tw + idx));
            }
        }
        C Wr[h + 1];
#pragma unroll
        for (int r = 1; r <= h; ++r) Wr[r] = KF_LDG(tw + r * NP);
        CW a[h + 1], b[h + 1];
        CW y0 = x[0];
#pragma unroll
        for (int q = 1; q <= h; ++q) {
            a[q].r = x[q].r + x[P - q].r;
            a[q].i = x[q].i + x[P - q].i;
            b[q].r = x[q].r - x[P - q].r;
            b[q].i = x[q].i - x[P - q].i;
            y0.r += a[q].r;
            y0.i += a[q].i;
        }
        y[0] = y0;
#pragma unroll
        for (int q1 = 1; q1 <= h; ++q1) {
            CW A = x[0], B;
            B.r = 0;
            B.i = 0;
#pragma unroll
            for (int q = 1; q <= h; ++q) {
                const int k = (q * q1) % P;
                const S c = k <= h ? Wr[k].r : Wr[P - k].r;
                const S sn = k <= h ? Wr[k].i : -Wr[P - k].i;
                A.r += a[q].r * c;
                A.i += a[q].i * c;
                B.r += b[q].r * sn;
                B.i += b[q].i * sn;
            }
            y[q1].r = A.r - B.i;
            y[q1].i = A.i + B.r;
            y[P - q1].r = A.r + B.i;
            y[P - q1].i = A.i - B.r;
        }
    }
    if (dst_g) {
#pragma unroll
        for (int q1 = 0; q1 < P; ++q1) go.st(q1 * sa.mloc, y[q1]);
    } else {
#pragma unroll
        for (int q1 = 0; q1 < P; ++q1) t.sst(g.A0 + q1 * sa.iloc, g.job, y[q1]);
    }
}

// Generic radix of any size, output-parallel: every thread computes up to
// KF_MAXO outputs into registers (reading all p legs of each), then -- after
// a barrier the caller places -- stores them.
template <typename S, int MODE>
KF_HD void rtg_compute(const Tile<S>& t, const KSub& sb, const KTab& tb, const KPass& ps, bool is_last, int tid,
                       int T, bool src_g, cpx<S>* outv) {
    typedef cpx<S> C;
    typedef Ar<S> Arr;
    const KStage& sa = sb.st[ps.a];
    const C* tw = (const C*)tb.tw_full;
    const int p = sa.p, N = sb.N;
    const int NG = t.J * ps.H * ps.ML;
#pragma unroll
    for (int i = 0; i < KF_MAXO; ++i) {
        const int o = tid + i * T;
        if (o >= NG * p) break;
        const int q1 = o / NG, gidx = o - q1 * NG;
        const GroupIx g = decode(ps, tb, t.J, t.logJ, t.col, is_last, gidx);
        if (!t.valid(g.job)) continue;
        const int U = t.U[g.job];
        const int step = sa.fs * (g.ul * sb.m_low + U + q1 * sa.m);
        int twidx = 0;
        GIn<S, MODE> gi{};
        if (src_g) gi = gin<S, MODE>(t, g.job, g.A0);
        C v0 = src_g ? gi.ld(0) : t.sld(g.A0, g.job);
        C acc = Arr::fixdiv_rt(v0, p);
        for (int q = 1; q < p; ++q) {
            C v = src_g ? gi.ld(q * sa.iloc) : t.sld(g.A0 + q * sa.iloc, g.job);
            twidx += step;
            if (twidx >= N) twidx -= N;
            acc = c_add(acc, Arr::cmul(Arr::fixdiv_rt(v, p), KF_LDG(tw + twidx)));
        }
        outv[i] = acc;
    }
}

template <typename S, int MODE>
KF_HD void rtg_store(const Tile<S>& t, const KSub& sb, const KTab& tb, const KPass& ps, bool is_last, int tid,
                     int T, bool dst_g, const cpx<S>* outv) {
    const KStage& sa = sb.st[ps.a];
    const int p = sa.p;
    const int NG = t.J * ps.H * ps.ML;
#pragma unroll
    for (int i = 0; i < KF_MAXO; ++i) {
        const int o = tid + i * T;
        if (o >= NG * p) break;
        const int q1 = o / NG, gidx = o - q1 * NG;
        const GroupIx g = decode(ps, tb, t.J, t.logJ, t.col, is_last, gidx);
        if (!t.valid(g.job)) continue;
        if (dst_g)
            gout<S, MODE>(t, g.job, g.pos0).st(q1 * sa.mloc, outv[i]);
        else
            t.sst(g.A0 + q1 * sa.iloc, g.job, outv[i]);
    }
}

// All groups of one (non runtime-generic) pass handled by thread tid.  KM
// is the mask of pass kinds compiled in (kind_bit): a family kernel covers
// a family of plans, a specialised kernel exactly its own passes.  kf_factor
// emits 4s, at most one 2, then 3s, 5s and larger primes, so only 9 ordered
// radix pairs and 12 ordered triples (up to 64 elements) can occur.
template <typename S, int MODE, kmask_t KM>
KF_HD void run_pass(const Tile<S>& t, const KSub& sb, const KTab& tb, const KPass& ps, bool is_last, int tid, int T,
                    bool src_g, bool dst_g) {
    const int NG = t.J * ps.H * ps.ML;
    for (int gidx = tid; gidx < NG; gidx += T) {
        const GroupIx g = decode(ps, tb, t.J, t.logJ, t.col, is_last, gidx);
        if (!t.valid(g.job)) continue;
        const int U = t.U[g.job];
        switch (ps.kind) {
#define KF_G1(P)                                                                            \
    case P:                                                                                 \
        if constexpr ((KM & kind_bit(P)) != 0) group1<S, MODE, P>(t, sb, tb, ps, g, U, src_g, dst_g); \
        break;
#define KF_G2(PA, PB)                                                                       \
    case 10 * PA + PB:                                                                      \
        if constexpr ((KM & kind_bit(10 * PA + PB)) != 0)                                   \
            group2<S, MODE, PA, PB>(t, sb, tb, ps, g, U, src_g, dst_g);                     \
        break;
#define KF_G3(PA, PB, PC)                                                                   \
    case 1000 + 100 * PA + 10 * PB + PC:                                                    \
        if constexpr ((KM & kind_bit(1000 + 100 * PA + 10 * PB + PC)) != 0)                \
            group3<S, MODE, PA, PB, PC>(t, sb, tb, ps, g, U, src_g, dst_g);                 \
        break;
#define KF_GG(P)                                                                            \
    case 100 + P:                                                                           \
        if constexpr ((KM & kind_bit(100 + P)) != 0) groupg<S, MODE, P>(t, sb, tb, ps, g, U, src_g, dst_g); \
        break;
            KF_G1(2) KF_G1(4) KF_G2(4, 2) KF_G2(4, 4)
            KF_G1(3) KF_G1(5)
            KF_G2(2, 3) KF_G2(2, 5) KF_G2(3, 3) KF_G2(3, 5) KF_G2(4, 3) KF_G2(4, 5) KF_G2(5, 5)
            KF_GG(7) KF_GG(11) KF_GG(13) KF_GG(17) KF_GG(19) KF_GG(23) KF_GG(29) KF_GG(31)
            KF_G3(4, 4, 4) KF_G3(4, 4, 2) KF_G3(4, 4, 3) KF_G3(4, 2, 3) KF_G3(4, 2, 5) KF_G3(4, 3, 3)
            KF_G3(4, 3, 5) KF_G3(2, 3, 3) KF_G3(2, 3, 5) KF_G3(2, 5, 5) KF_G3(3, 3, 3) KF_G3(3, 3, 5)
#undef KF_G3
#undef KF_G1
#undef KF_G2
#undef KF_GG
            default:
                if (t.err) *t.err = 1;
                break;
        }
    }
}

// ------------------------------------------------------------ real-transform phases
// Split of kiss_fftr (kiss_fftr.c:88-116) for work item k = 0..ncfft/2 of
// the half-size complex transform X: from Xk = X[k], Xnk = X[ncfft-k] (for
// k == 0: X[0] twice) to the bins Fk = F[k] and Fnk = F[ncfft-k] (for
// k == 0: F[0] and F[ncfft]).  When k == ncfft-k the reference writes the
// bin twice and Fnk is the value that survives.
template <typename S>
KF_HD void split_vals(const KTab& tb, int k, cpx<S> Xk, cpx<S> Xnk, cpx<S>& Fk, cpx<S>& Fnk) {
    typedef Ar<S> Arr;
    typedef cpx<S> C;
    if (k == 0) {
        C dc = Arr::template fixdiv<2>(Xk);
        KF_OVF_CHECK(S, dc.r, +, dc.i);
        KF_OVF_CHECK(S, dc.r, -, dc.i);
        Fk.r = Arr::st(Arr::add(dc.r, dc.i));
        Fk.i = 0;
        Fnk.r = Arr::st(Arr::sub(dc.r, dc.i));
        Fnk.i = 0;
        return;
    }
    C fpnk;
    fpnk.r = Xnk.r;
    fpnk.i = Arr::st(Arr::neg(Xnk.i));
    C fpk = Arr::template fixdiv<2>(Xk);
    fpnk = Arr::template fixdiv<2>(fpnk);
    C f1k = c_add(fpk, fpnk), f2k = c_sub(fpk, fpnk);
    C tw = Arr::cmul(f2k, KF_LDG((const C*)tb.super_tw + (k - 1)));
    Fk.r = Arr::st(Arr::half(Arr::add(f1k.r, tw.r)));
    Fk.i = Arr::st(Arr::half(Arr::add(f1k.i, tw.i)));
    Fnk.r = Arr::st(Arr::half(Arr::sub(f1k.r, tw.r)));
    Fnk.i = Arr::st(Arr::half(Arr::sub(tw.i, f1k.i)));
}

// The same split reading X from the shared tile (position n lives at
// input-order index revfull[n]).
template <typename S>
KF_HD void r2c_split_pair(const Tile<S>& t, const KSub& sb, const KTab& tb, int job, int k, cpx<S>& Fk,
                          cpx<S>& Fnk) {
    const int* rf = tb.rev + sb.revfull_off;
    cpx<S> Xk = t.sld(KF_LDG(rf + k), job);
    cpx<S> Xnk = k == 0 ? Xk : t.sld(KF_LDG(rf + (sb.L - k)), job);
    split_vals(tb, k, Xk, Xnk, Fk, Fnk);
}

// Merge of kiss_fftri (kiss_fftr.c:131-153) for work item k: from bins
// Gk = G[k] and Gnk = G[ncfft-k] (for k == 0: G[0] and G[ncfft]) to the
// half-size inverse input tmp[k], tmp[ncfft-k].
template <typename S>
KF_HD void c2r_merge_pair(const KTab& tb, int k, cpx<S> Gk, cpx<S> Gnk, cpx<S>& tk, cpx<S>& tnk) {
    typedef Ar<S> Arr;
    typedef cpx<S> C;
    if (k == 0) {
        C t0;
        t0.r = Arr::st(Arr::add(Gk.r, Gnk.r));
        t0.i = Arr::st(Arr::sub(Gk.r, Gnk.r));
        tk = Arr::template fixdiv<2>(t0);
        tnk = tk;
        return;
    }
    C fk = Gk, fnkc;
    fnkc.r = Gnk.r;
    fnkc.i = Arr::st(Arr::neg(Gnk.i));
    fk = Arr::template fixdiv<2>(fk);
    fnkc = Arr::template fixdiv<2>(fnkc);
    C fek = c_add(fk, fnkc), d = c_sub(fk, fnkc);
    C fok = Arr::cmul(d, KF_LDG((const C*)tb.super_tw + (k - 1)));
    tk = c_add(fek, fok);
    tnk = c_sub(fek, fok);
    tnk.i = Arr::st(Arr::neg(tnk.i));
}

KF_HD void item_decode(int J, int logJ, int col, int nk, int it, int& job, int& k) {
    if (col) {
        job = it & (J - 1);
        k = it >> logJ;
    } else {
        job = it / nk;
        k = it - job * nk;
    }
}

// R2C: split from shared memory straight to the output bins in HBM.
template <typename S>
KF_HD void r2c_post(const Tile<S>& t, const KSub& sb, const KTab& tb, int tid, int T) {
    const int ncfft = sb.L, nk = ncfft / 2 + 1;
    for (int it = tid; it < t.J * nk; it += T) {
        int job, k;
        item_decode(t.J, t.logJ, t.col, nk, it, job, k);
        if (!t.valid(job)) continue;
        cpx<S> Fk, Fnk;
        r2c_split_pair(t, sb, tb, job, k, Fk, Fnk);
        cpx<S>* o = (cpx<S>*)t.out + t.outb[job];
        if (k != ncfft - k) (KF_MEM_CHECK(o + (long long)k * t.out_stride, sizeof(Fk)), o[(long long)k * t.out_stride] = Fk);
        (KF_MEM_CHECK(o + (long long)(ncfft - k) * t.out_stride, sizeof(Fnk)), o[(long long)(ncfft - k) * t.out_stride] = Fnk);
    }
}

// C2R: merge from the input bins in HBM into the shared tile (input order).
template <typename S>
KF_HD void c2r_pre(const Tile<S>& t, const KSub& sb, const KTab& tb, int tid, int T) {
    const int ncfft = sb.L, nk = ncfft / 2 + 1;
    for (int it = tid; it < t.J * nk; it += T) {
        int job, k;
        item_decode(t.J, t.logJ, t.col, nk, it, job, k);
        if (!t.valid(job)) continue;
        const cpx<S>* f = (const cpx<S>*)t.in + t.inb[job];
        cpx<S> Gk = (KF_MEM_CHECK(f + (long long)k * t.in_stride, sizeof(cpx<S>)), f[(long long)k * t.in_stride]);
        cpx<S> Gnk = (KF_MEM_CHECK(f + (long long)(ncfft - k) * t.in_stride, sizeof(cpx<S>)),
                      f[(long long)(ncfft - k) * t.in_stride]);
        cpx<S> tk, tnk;
        c2r_merge_pair(tb, k, Gk, Gnk, tk, tnk);
        if (k == 0) {
            t.sst(0, job, tk);
        } else {
            if (k != ncfft - k) t.sst(k, job, tk);
            t.sst(ncfft - k, job, tnk);
        }
    }
}

// Fast FIR middle: split (forward plan), multiply by the filter response,
// merge (inverse plan).  Reads every bin pair before any write: the caller
// places a barrier between fir_mid_compute and fir_mid_store.
template <typename S>
KF_HD void fir_mid_compute(const Tile<S>& t, const KSub& fw, const KTab& fwt, const KTab& ivt, const cpx<S>* H,
                           int tid, int T, cpx<S>* outv) {
    typedef Ar<S> Arr;
    const int ncfft = fw.L, nk = ncfft / 2 + 1;
#pragma unroll
    for (int i = 0; i < KF_MAXO / 2; ++i) {
        int it = tid + i * T;
        if (it >= t.J * nk) break;
        int job, k;
        item_decode(t.J, t.logJ, t.col, nk, it, job, k);
        if (!t.valid(job)) continue;
        cpx<S> Fk, Fnk;
        r2c_split_pair(t, fw, fwt, job, k, Fk, Fnk);
        int kk = k, knk = ncfft - k;
        if (k == 0) kk = 0, knk = ncfft;
        cpx<S> Gk = Arr::cmul(Fk, KF_LDG(H + kk));
        cpx<S> Gnk = Arr::cmul(Fnk, KF_LDG(H + knk));
        if (k != 0 && k == ncfft - k) Gk = Gnk;
        c2r_merge_pair(ivt, k, Gk, Gnk, outv[2 * i], outv[2 * i + 1]);
    }
}

template <typename S>
KF_HD void fir_mid_store(const Tile<S>& t, const KSub& fw, int tid, int T, const cpx<S>* outv) {
    const int ncfft = fw.L, nk = ncfft / 2 + 1;
#pragma unroll
    for (int i = 0; i < KF_MAXO / 2; ++i) {
        int it = tid + i * T;
        if (it >= t.J * nk) break;
        int job, k;
        item_decode(t.J, t.logJ, t.col, nk, it, job, k);
        if (!t.valid(job)) continue;
        if (k == 0) {
            t.sst(0, job, outv[2 * i]);
        } else {
            if (k != ncfft - k) t.sst(k, job, outv[2 * i]);
            t.sst(ncfft - k, job, outv[2 * i + 1]);
        }
    }
}

// Standalone split / merge items for real plans that run as two HBM
// passes: X (or the merged input) sits in HBM in natural order.  Item it
// belongs to transform it / (ncfft/2+1), found at its in_off / out_off entry
// when the launch carries per-transform offsets (batched requests).
template <typename S>
KF_HD void split_item(const KArgs& a, long long it) {
    const int ncfft = a.sub[0].L, nk = ncfft / 2 + 1;
    long long b = it / nk;
    int k = (int)(it - b * nk);
    const cpx<S>* X = (const cpx<S>*)a.in + (a.in_off ? a.in_off[b] : b * a.in_dhi);
    cpx<S>* F = (cpx<S>*)a.out + (a.out_off ? a.out_off[b] : b * a.out_dhi);
    cpx<S> Fk, Fnk;
    KF_MEM_CHECK(X + k, sizeof(Fk));
    KF_MEM_CHECK(X + (k == 0 ? 0 : ncfft - k), sizeof(Fk));
    split_vals(a.tab[0], k, X[k], k == 0 ? X[0] : X[ncfft - k], Fk, Fnk);
    if (k != ncfft - k) (KF_MEM_CHECK(F + k, sizeof(Fk)), F[k] = Fk);
    (KF_MEM_CHECK(F + ncfft - k, sizeof(Fnk)), F[ncfft - k] = Fnk);
}

template <typename S>
KF_HD void merge_item(const KArgs& a, long long it) {
    const int ncfft = a.sub[0].L, nk = ncfft / 2 + 1;
    long long b = it / nk;
    int k = (int)(it - b * nk);
    const cpx<S>* G = (const cpx<S>*)a.in + (a.in_off ? a.in_off[b] : b * a.in_dhi);
    cpx<S>* X = (cpx<S>*)a.out + (a.out_off ? a.out_off[b] : b * a.out_dhi);
    cpx<S> tk, tnk;
    KF_MEM_CHECK(G + k, sizeof(tk));
    KF_MEM_CHECK(G + ncfft - k, sizeof(tk));
    c2r_merge_pair(a.tab[0], k, G[k], G[ncfft - k], tk, tnk);
    if (k == 0) {
        (KF_MEM_CHECK(X, sizeof(tk)), X[0] = tk);
    } else {
        if (k != ncfft - k) (KF_MEM_CHECK(X + k, sizeof(tk)), X[k] = tk);
        (KF_MEM_CHECK(X + ncfft - k, sizeof(tnk)), X[ncfft - k] = tnk);
    }
}

// Job table entries for tile slot j (any thread may fill one).
KF_HD void job_entry(const KRun& a, long long tile, int J, int j, long long& inb, long long& outb, int& U,
                     long long& lin, long long& lout) {
    long long jg = tile * J + j;
    if (jg >= a.G) {
        inb = -1;
        outb = -1;
        U = 0;
        lin = lout = 0;
        return;
    }
    long long ghi = jg / a.G_lo, glo = jg - ghi * a.G_lo, gmid = 0;
    if (a.G_mid > 1) {
        gmid = ghi % a.G_mid;
        ghi /= a.G_mid;
    }
    inb = (a.in_off ? a.in_off[ghi] : ghi * a.in_dhi) + gmid * a.in_dmid + glo * a.in_dlo;
    outb = (a.out_off ? a.out_off[ghi] : ghi * a.out_dhi) + gmid * a.out_dmid + glo * a.out_dlo;
    U = a.use_u ? (int)glo : 0;
    lin = a.in_limit - inb;
    lout = a.out_limit - outb;
    if (a.fir_ngood > 0 && lout > a.fir_ngood) lout = a.fir_ngood;
}

}  // namespace kf
