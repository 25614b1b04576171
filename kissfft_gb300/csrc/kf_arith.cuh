// Sample arithmetic and radix butterflies shared by every GPU kernel.
//
// The arithmetic follows the reference's macros (_kiss_fft_guts.h:43-139)
// per sample type:
//   float/double : IEEE arithmetic; C_FIXDIV is a no-op; HALF_OF multiplies
//                  by 0.5.
//   Q15 / Q31    : values stored in int16/int32 are truncated to that width;
//                  expressions are 32-bit wrapping integers; products are
//                  int32 (Q15) or int64 (Q31) rounded by
//                  sround(x) = (x + 2^(FRACBITS-1)) >> FRACBITS;
//                  C_FIXDIV(c, p) multiplies by the integer SAMP_MAX/p.
// The butterflies perform, per output element, the same operations on the
// same operands as kf_bfly2/3/4/5/generic (kiss_fft.c:15-233), so Q15/Q31
// results are bit-identical to the reference.
#pragma once
#include "kf_stdint.h"

#if defined(__CUDACC__) || defined(__CUDACC_RTC__)
#define KF_HD __host__ __device__ __forceinline__
#else
#define KF_HD inline
#endif

// Overflow hook.  The reference built with CHECK_OVERFLOW warns when a
// fixed-point C_ADD / C_SUB / C_ADDTO / C_SUBFROM component, or one of
// kiss_fftr's two DC sums, leaves [SAMP_MIN, SAMP_MAX] (_kiss_fft_guts.h:57-61,
// kiss_fftr.c:94-95).  The engine marks exactly those operations with
// KF_OVF_CHECK(S, a, op, b).  It expands to nothing unless the includer
// defines KF_OVF_NOTE(S, v) (v: the exact sum as long long); the CPU emulator
// of the engine defines it to count, the CUDA builds do not.
#if defined(KF_OVF_NOTE)
#define KF_OVF_CHECK(S, a, op, b)                                                   \
    do {                                                                            \
        if constexpr ((S)0.5 == (S)0) KF_OVF_NOTE(S, (long long)(a) op (long long)(b)); \
    } while (0)
#else
#define KF_OVF_CHECK(S, a, op, b) ((void)0)
#endif

namespace kf {

// float samples (the only type whose plans use three-stage register groups)
template <typename S>
#if defined(__CUDACC__) || defined(__CUDACC_RTC__)
__host__ __device__
#endif
constexpr bool is_f32() {
    return sizeof(S) == 4 && (S)0.5 != (S)0;
}

template <typename S>
struct alignas(2 * sizeof(S)) cpx {
    S r, i;
};

template <typename S>
struct Ar;

template <typename S>
struct ArIeee {
    typedef S W;  // expression type
    typedef cpx<S> C;
    static KF_HD S st(W x) { return x; }
    static KF_HD W add(W a, W b) { return a + b; }
    static KF_HD W sub(W a, W b) { return a - b; }
    static KF_HD W neg(W a) { return -a; }
    static KF_HD W half(W a) { return a * (S)0.5; }
    static KF_HD S smul(S a, S b) { return a * b; }
    static KF_HD C cmul(C a, C b) {
        C m;
        m.r = a.r * b.r - a.i * b.i;
        m.i = a.r * b.i + a.i * b.r;
        return m;
    }
    template <int P>
    static KF_HD C fixdiv(C c) { return c; }
    static KF_HD C fixdiv_rt(C c, int) { return c; }
    static KF_HD C mulsc(C c, S s) {
        c.r *= s;
        c.i *= s;
        return c;
    }
    // "wide" forms (see ArFixed): for IEEE types they are the plain ones
    typedef cpx<S> CW;
    static KF_HD CW widen(C c) { return c; }
    static KF_HD C narrow(CW c) { return c; }
    static KF_HD W tr(W x) { return x; }
    template <int P>
    static KF_HD CW fixdiv_w(CW c) { return c; }
    static KF_HD CW cmul_w(CW a, CW b) { return cmul(a, b); }
    static KF_HD W smul_w(W a, W b) { return a * b; }
    static KF_HD CW mulsc_w(CW c, W s) { return mulsc(c, s); }
};

template <typename S, typename P, int FB, int64_t SMAX>
struct ArFixed {
    typedef int32_t W;
    typedef cpx<S> C;
    // truncation to the storage width (mod 2^16 for Q15)
    static KF_HD S st(W x) { return (S)x; }
    static KF_HD W add(W a, W b) { return (W)((uint32_t)a + (uint32_t)b); }
    static KF_HD W sub(W a, W b) { return (W)((uint32_t)a - (uint32_t)b); }
    // Negation as a 32-bit word.  For Q15 it is opaque on the device: when
    // the optimizer could see a 16-bit sample being negated and then
    // truncated, it compiled -(-32768) as if it fitted 16 bits (32768
    // instead of the reference's wrap to -32768).
    static KF_HD W neg(W a) {
#if defined(__CUDA_ARCH__)
        if constexpr (sizeof(S) == 2) {
            int r;
            asm("sub.s32 %0, 0, %1;" : "=r"(r) : "r"((int)a));
            return (W)r;
        }
#endif
        return (W)(0u - (uint32_t)a);
    }
    static KF_HD W half(W a) { return a >> 1; }
    static KF_HD S sround(P x) { return (S)((x + ((P)1 << (FB - 1))) >> FB); }
    // sround(a*b + c*d) as an untruncated word (exact: |a*b + c*d| < 2^(2*FB+1))
    static KF_HD W round2(S a, S b, S c, S d) {
#if defined(__CUDA_ARCH__)
        if constexpr (sizeof(P) == 8) {
            // Q31: two signed 32x32+64 multiply-adds, then bits 31..62 of the
            // 64-bit sum (the low word of the arithmetic shift)
            long long t;
            unsigned lo, hi, r;
            asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(t) : "r"((int)a), "r"((int)b), "l"(1ll << (FB - 1)));
            asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(t) : "r"((int)c), "r"((int)d), "l"(t));
            asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "l"(t));
            asm("shf.r.wrap.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(lo), "r"(hi), "r"(FB));
            return (W)r;
        }
#endif
        return (W)(((P)a * (P)b + (P)c * (P)d + ((P)1 << (FB - 1))) >> FB);
    }
    // sround(a*b) as an untruncated word
    static KF_HD W round1(S a, S b) {
#if defined(__CUDA_ARCH__)
        if constexpr (sizeof(P) == 8) {
            long long t;
            unsigned lo, hi, r;
            asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(t) : "r"((int)a), "r"((int)b), "l"(1ll << (FB - 1)));
            asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "l"(t));
            asm("shf.r.wrap.b32 %0, %1, %2, %3;" : "=r"(r) : "r"(lo), "r"(hi), "r"(FB));
            return (W)r;
        }
#endif
        return (W)(((P)a * (P)b + ((P)1 << (FB - 1))) >> FB);
    }
    static KF_HD S smul(S a, S b) { return st(round1(a, b)); }
    // C_MUL(m, a, b) with b a table twiddle (|b| <= SMAX, so -b.i fits S)
    static KF_HD C cmul(C a, C b) {
        C m;
        m.r = st(round2(a.r, b.r, a.i, (S)(0 - b.i)));
        m.i = st(round2(a.r, b.i, a.i, b.r));
        return m;
    }
    template <int Q>
    static KF_HD C fixdiv(C c) {
        constexpr S k = (S)(SMAX / Q);
        c.r = st(round1(c.r, k));
        c.i = st(round1(c.i, k));
        return c;
    }
    static KF_HD C fixdiv_rt(C c, int q) {
        const S k = (S)(SMAX / q);
        c.r = st(round1(c.r, k));
        c.i = st(round1(c.i, k));
        return c;
    }
    static KF_HD C mulsc(C c, S s) {
        c.r = st(round1(c.r, s));
        c.i = st(round1(c.i, s));
        return c;
    }
    // "Wide" forms for the butterflies.  The reference stores every sum in a
    // sample (truncation to the storage width), but truncation commutes with
    // the wrapping adds and subtracts, so a chain of them may keep its
    // values untruncated (CW: complex of W) and truncate once where the
    // stored value feeds a multiply or a shift, and at the butterfly's
    // outputs.  tr(x) is the value the reference would have stored.
    typedef cpx<W> CW;
    static KF_HD CW widen(C c) {
        CW r;
        r.r = c.r;
        r.i = c.i;
        return r;
    }
    static KF_HD C narrow(CW c) {
        C r;
        r.r = st(c.r);
        r.i = st(c.i);
        return r;
    }
    static KF_HD W tr(W x) { return (W)st(x); }
    // sround(a*b + c*d) and sround(a*b - c*d), untruncated, for a and c
    // within the sample range and |b|, |d| <= SMAX (|a*b| + |c*d| < 2^31
    // for Q15, so the int32 expression of the reference is exact; the
    // compiler fuses the shift into the add that consumes the result)
    static KF_HD W rnd_add(W a, W b, W c, W d) {
        if constexpr (sizeof(P) == 4)
            return (a * b + c * d + (1 << (FB - 1))) >> FB;
        else
            return round2((S)a, (S)b, (S)c, (S)d);
    }
    static KF_HD W rnd_sub(W a, W b, W c, W d) {
        if constexpr (sizeof(P) == 4)
            return (a * b - c * d + (1 << (FB - 1))) >> FB;
        else
            return round2((S)a, (S)b, (S)c, (S)(0 - d));
    }
    static KF_HD W rnd1(W a, W b) {
        if constexpr (sizeof(P) == 4)
            return (a * b + (1 << (FB - 1))) >> FB;
        else
            return round1((S)a, (S)b);
    }
    // C_FIXDIV of a sample value: |result| <= SMAX/Q < 2^(FB-1), no truncation
    template <int Q>
    static KF_HD CW fixdiv_w(CW c) {
        constexpr W k = (W)(SMAX / Q);
        CW r;
        r.r = rnd1(c.r, k);
        r.i = rnd1(c.i, k);
        return r;
    }
    // C_MUL(m, a, b), a within the sample range, b a table twiddle held as W
    // (Q15 stage tables store them widened); the result is left untruncated
    static KF_HD CW cmul_w(CW a, CW b) {
        CW m;
        m.r = rnd_sub(a.r, b.r, a.i, b.i);
        m.i = rnd_add(a.r, b.i, a.i, b.r);
        return m;
    }
    // S_MUL / C_MULBYSCALAR: |a*b| < 2^(2*FB), so the result fits the sample type
    static KF_HD W smul_w(W a, W b) { return rnd1(a, b); }
    static KF_HD CW mulsc_w(CW c, W s) {
        CW r;
        r.r = rnd1(c.r, s);
        r.i = rnd1(c.i, s);
        return r;
    }
    // C_MUL(t, a, w) then C_ADDTO(acc, t) of kf_bfly_generic, a within the
    // sample range, w a table twiddle held as W; acc untruncated
    static KF_HD void cmul_acc_w(W& ar, W& ai, CW a, CW w) {
        const W tr_ = rnd_sub(a.r, w.r, a.i, w.i), ti = rnd_add(a.r, w.i, a.i, w.r);
        KF_OVF_CHECK(S, st(ar), +, st(tr_));
        KF_OVF_CHECK(S, st(ai), +, st(ti));
        ar = add(ar, tr_);
        ai = add(ai, ti);
    }
#if defined(__CUDA_ARCH__)
    // Q31 output of kf_bfly_generic on the device:
    //   acc = x0 + sum_{q=1..P-1} C_MUL(x_q, w_q)   (each product rounded).
    // With the legs doubled (x2r = 2*x.r, x2i = 2*x.i, x2n = -2*x.i; they fit
    // since |x| <= SMAX/P) and v = a*b + c*d exact,
    //   acc*2^32 + 2^31 + 2v  (mod 2^64)
    // is two widening multiply-adds, and its high word is acc + sround(v)
    // (mod 2^32): the rounding shift and the accumulation cost nothing.
    template <int P>
    static __device__ __forceinline__ C gen_out_q31(CW x0, const W* x2r, const W* x2i, const W* x2n, const CW* w) {
        unsigned ar = (unsigned)x0.r, ai = (unsigned)x0.i;
#pragma unroll
        for (int q = 1; q < P; ++q) {
            unsigned long long cr, ci;
            unsigned lo;
            asm("mov.b64 %0, {%1, %2};" : "=l"(cr) : "r"(1u << FB), "r"(ar));
            asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(cr) : "r"((int)x2r[q]), "r"((int)w[q - 1].r));
            asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(cr) : "r"((int)x2n[q]), "r"((int)w[q - 1].i));
            asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(ar) : "l"(cr));
            asm("mov.b64 %0, {%1, %2};" : "=l"(ci) : "r"(1u << FB), "r"(ai));
            asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(ci) : "r"((int)x2r[q]), "r"((int)w[q - 1].i));
            asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(ci) : "r"((int)x2i[q]), "r"((int)w[q - 1].r));
            asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(ai) : "l"(ci));
            (void)lo;
        }
        C out;
        out.r = (S)ar;
        out.i = (S)ai;
        return out;
    }
#endif
    // C_MUL(t, a, w) then C_ADDTO(acc, t) of kf_bfly_generic, with acc kept as
    // an untruncated word: truncation to S commutes with the wrapping adds, so
    // the caller truncates once after the whole sum.  Twiddles have
    // |w| <= SMAX, so -w.i fits S and every product is one widening
    // multiply-add; the sums are exact in P (|a*w| < 2^(2*FB)).
    static KF_HD void cmul_acc(W& ar, W& ai, C a, C w) {
        const W tr = round2(a.r, w.r, a.i, (S)(0 - w.i)), ti = round2(a.r, w.i, a.i, w.r);
        // C_ADDTO's check sees the stored (truncated) running sum and product
        KF_OVF_CHECK(S, st(ar), +, st(tr));
        KF_OVF_CHECK(S, st(ai), +, st(ti));
        ar = add(ar, tr);
        ai = add(ai, ti);
    }
};

template <>
struct Ar<float> : ArIeee<float> {};
template <>
struct Ar<double> : ArIeee<double> {};
template <>
struct Ar<int16_t> : ArFixed<int16_t, int32_t, 15, 32767> {};
template <>
struct Ar<int32_t> : ArFixed<int32_t, int64_t, 31, 2147483647> {};

template <typename S>
KF_HD cpx<S> c_add(cpx<S> a, cpx<S> b) {
    typedef Ar<S> A;
    KF_OVF_CHECK(S, a.r, +, b.r);
    KF_OVF_CHECK(S, a.i, +, b.i);
    cpx<S> r;
    r.r = A::st(A::add(a.r, b.r));
    r.i = A::st(A::add(a.i, b.i));
    return r;
}
template <typename S>
KF_HD cpx<S> c_sub(cpx<S> a, cpx<S> b) {
    typedef Ar<S> A;
    KF_OVF_CHECK(S, a.r, -, b.r);
    KF_OVF_CHECK(S, a.i, -, b.i);
    cpx<S> r;
    r.r = A::st(A::sub(a.r, b.r));
    r.i = A::st(A::sub(a.i, b.i));
    return r;
}

// C_ADD / C_SUB on wide values (no truncation; the overflow hook sees the
// values the reference stored)
template <typename S>
KF_HD typename Ar<S>::CW w_add(typename Ar<S>::CW a, typename Ar<S>::CW b) {
    typedef Ar<S> A;
    KF_OVF_CHECK(S, A::tr(a.r), +, A::tr(b.r));
    KF_OVF_CHECK(S, A::tr(a.i), +, A::tr(b.i));
    typename A::CW r;
    r.r = A::add(a.r, b.r);
    r.i = A::add(a.i, b.i);
    return r;
}
template <typename S>
KF_HD typename Ar<S>::CW w_sub(typename Ar<S>::CW a, typename Ar<S>::CW b) {
    typedef Ar<S> A;
    KF_OVF_CHECK(S, A::tr(a.r), -, A::tr(b.r));
    KF_OVF_CHECK(S, A::tr(a.i), -, A::tr(b.i));
    typename A::CW r;
    r.r = A::sub(a.r, b.r);
    r.i = A::sub(a.i, b.i);
    return r;
}

// ---------------------------------------------------------------- butterflies
// v[0], v[VS], ..., v[(P-1)*VS] are the P legs of one butterfly (register
// array, compile-time stride).  w[q-1] is the twiddle of leg q.  The
// constants c0/c1 are epi3 (radix 3) or ya/yb (radix 5).

// kf_bfly2, kiss_fft.c:15-36
// Twiddles and constants arrive as Ar<S>::CW (the plan tables' entries; for
// Q15 widened to 32-bit words).
template <typename S, int VS>
KF_HD void bfly2(cpx<S>* v, const typename Ar<S>::CW* w) {
    typedef Ar<S> A;
    typedef typename A::CW CW;
    CW a = A::template fixdiv_w<2>(A::widen(v[0])), b = A::template fixdiv_w<2>(A::widen(v[VS]));
    CW t = A::cmul_w(b, w[0]);
    v[VS] = A::narrow(w_sub<S>(a, t));
    v[0] = A::narrow(w_add<S>(a, t));
}

// kf_bfly4, kiss_fft.c:38-84
template <typename S, int VS>
KF_HD void bfly4(cpx<S>* v, const typename Ar<S>::CW* w, bool inverse) {
    typedef Ar<S> A;
    typedef typename A::CW CW;
    CW a0 = A::template fixdiv_w<4>(A::widen(v[0])), a1 = A::template fixdiv_w<4>(A::widen(v[VS]));
    CW a2 = A::template fixdiv_w<4>(A::widen(v[2 * VS])), a3 = A::template fixdiv_w<4>(A::widen(v[3 * VS]));
    CW t0 = A::cmul_w(a1, w[0]), t1 = A::cmul_w(a2, w[1]), t2 = A::cmul_w(a3, w[2]);
    CW d02 = w_sub<S>(a0, t1), s02 = w_add<S>(a0, t1);
    CW s13 = w_add<S>(t0, t2), d13 = w_sub<S>(t0, t2);
    v[2 * VS] = A::narrow(w_sub<S>(s02, s13));
    v[0] = A::narrow(w_add<S>(s02, s13));
    cpx<S> o1, o3;
    if (inverse) {
        o1.r = A::st(A::sub(d02.r, d13.i));
        o1.i = A::st(A::add(d02.i, d13.r));
        o3.r = A::st(A::add(d02.r, d13.i));
        o3.i = A::st(A::sub(d02.i, d13.r));
    } else {
        o1.r = A::st(A::add(d02.r, d13.i));
        o1.i = A::st(A::sub(d02.i, d13.r));
        o3.r = A::st(A::sub(d02.r, d13.i));
        o3.i = A::st(A::add(d02.i, d13.r));
    }
    v[VS] = o1;
    v[3 * VS] = o3;
}

// kf_bfly3, kiss_fft.c:86-128 (c0 = epi3 = tw[fstride*m]).  HALF_OF and
// C_MULBYSCALAR act on the stored (truncated) sums.
template <typename S, int VS>
KF_HD void bfly3(cpx<S>* v, const typename Ar<S>::CW* w, typename Ar<S>::CW c0) {
    typedef Ar<S> A;
    typedef typename A::CW CW;
    typedef typename A::W W;
    CW a0 = A::template fixdiv_w<3>(A::widen(v[0])), a1 = A::template fixdiv_w<3>(A::widen(v[VS]));
    CW a2 = A::template fixdiv_w<3>(A::widen(v[2 * VS]));
    CW t1 = A::cmul_w(a1, w[0]), t2 = A::cmul_w(a2, w[1]);
    CW s = w_add<S>(t1, t2), d = w_sub<S>(t1, t2);
    const W o1r = A::sub(a0.r, A::half(A::tr(s.r))), o1i = A::sub(a0.i, A::half(A::tr(s.i)));
    CW dt;
    dt.r = A::tr(d.r);
    dt.i = A::tr(d.i);
    const CW dm = A::mulsc_w(dt, c0.i);
    v[0] = A::narrow(w_add<S>(a0, s));
    cpx<S> o1, o2;
    o2.r = A::st(A::add(o1r, dm.i));
    o2.i = A::st(A::sub(o1i, dm.r));
    o1.r = A::st(A::sub(o1r, dm.i));
    o1.i = A::st(A::add(o1i, dm.r));
    v[VS] = o1;
    v[2 * VS] = o2;
}

// kf_bfly5, kiss_fft.c:130-189 (c0 = ya = tw[fstride*m], c1 = yb = tw[2*fstride*m]).
// S_MUL acts on the stored (truncated) sums and differences.
template <typename S, int VS>
KF_HD void bfly5(cpx<S>* v, const typename Ar<S>::CW* w, typename Ar<S>::CW ya, typename Ar<S>::CW yb) {
    typedef Ar<S> A;
    typedef typename A::CW CW;
    typedef typename A::W W;
    CW a0 = A::template fixdiv_w<5>(A::widen(v[0])), a1 = A::template fixdiv_w<5>(A::widen(v[VS]));
    CW a2 = A::template fixdiv_w<5>(A::widen(v[2 * VS])), a3 = A::template fixdiv_w<5>(A::widen(v[3 * VS]));
    CW a4 = A::template fixdiv_w<5>(A::widen(v[4 * VS]));
    CW t1 = A::cmul_w(a1, w[0]), t2 = A::cmul_w(a2, w[1]), t3 = A::cmul_w(a3, w[2]), t4 = A::cmul_w(a4, w[3]);
    CW s14 = w_add<S>(t1, t4), d14 = w_sub<S>(t1, t4);
    CW s23 = w_add<S>(t2, t3), d23 = w_sub<S>(t2, t3);
    const W s14r = A::tr(s14.r), s14i = A::tr(s14.i), s23r = A::tr(s23.r), s23i = A::tr(s23.i);
    const W d14r = A::tr(d14.r), d14i = A::tr(d14.i), d23r = A::tr(d23.r), d23i = A::tr(d23.i);
    CW o0, b1, e1, b2, e2;
    o0.r = A::add(a0.r, A::add(s14r, s23r));
    o0.i = A::add(a0.i, A::add(s14i, s23i));
    b1.r = A::add(A::add(a0.r, A::smul_w(s14r, ya.r)), A::smul_w(s23r, yb.r));
    b1.i = A::add(A::add(a0.i, A::smul_w(s14i, ya.r)), A::smul_w(s23i, yb.r));
    e1.r = A::add(A::smul_w(d14i, ya.i), A::smul_w(d23i, yb.i));
    e1.i = A::sub(A::neg(A::smul_w(d14r, ya.i)), A::smul_w(d23r, yb.i));
    b2.r = A::add(A::add(a0.r, A::smul_w(s14r, yb.r)), A::smul_w(s23r, ya.r));
    b2.i = A::add(A::add(a0.i, A::smul_w(s14i, yb.r)), A::smul_w(s23i, ya.r));
    e2.r = A::add(A::neg(A::smul_w(d14i, yb.i)), A::smul_w(d23i, ya.i));
    e2.i = A::sub(A::smul_w(d14r, yb.i), A::smul_w(d23r, ya.i));
    v[0] = A::narrow(o0);
    v[VS] = A::narrow(w_sub<S>(b1, e1));
    v[4 * VS] = A::narrow(w_add<S>(b1, e1));
    v[2 * VS] = A::narrow(w_add<S>(b2, e2));
    v[3 * VS] = A::narrow(w_sub<S>(b2, e2));
}

template <typename S, int P, int VS>
KF_HD void bfly(cpx<S>* v, const typename Ar<S>::CW* w, typename Ar<S>::CW c0, typename Ar<S>::CW c1,
                bool inverse) {
    if constexpr (P == 2) bfly2<S, VS>(v, w);
    if constexpr (P == 3) bfly3<S, VS>(v, w, c0);
    if constexpr (P == 4) bfly4<S, VS>(v, w, inverse);
    if constexpr (P == 5) bfly5<S, VS>(v, w, c0, c1);
}

}  // namespace kf
