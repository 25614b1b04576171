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

// ---------------------------------------------------------------- butterflies
// v[0], v[VS], ..., v[(P-1)*VS] are the P legs of one butterfly (register
// array, compile-time stride).  w[q-1] is the twiddle of leg q.  The
// constants c0/c1 are epi3 (radix 3) or ya/yb (radix 5).

// kf_bfly2, kiss_fft.c:15-36
template <typename S, int VS>
KF_HD void bfly2(cpx<S>* v, const cpx<S>* w) {
    typedef Ar<S> A;
    cpx<S> a = A::template fixdiv<2>(v[0]), b = A::template fixdiv<2>(v[VS]);
    cpx<S> t = A::cmul(b, w[0]);
    v[VS] = c_sub(a, t);
    v[0] = c_add(a, t);
}

// kf_bfly4, kiss_fft.c:38-84
template <typename S, int VS>
KF_HD void bfly4(cpx<S>* v, const cpx<S>* w, bool inverse) {
    typedef Ar<S> A;
    cpx<S> a0 = A::template fixdiv<4>(v[0]), a1 = A::template fixdiv<4>(v[VS]);
    cpx<S> a2 = A::template fixdiv<4>(v[2 * VS]), a3 = A::template fixdiv<4>(v[3 * VS]);
    cpx<S> t0 = A::cmul(a1, w[0]), t1 = A::cmul(a2, w[1]), t2 = A::cmul(a3, w[2]);
    cpx<S> d02 = c_sub(a0, t1), s02 = c_add(a0, t1);
    cpx<S> s13 = c_add(t0, t2), d13 = c_sub(t0, t2);
    v[2 * VS] = c_sub(s02, s13);
    v[0] = c_add(s02, s13);
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

// kf_bfly3, kiss_fft.c:86-128 (c0 = epi3 = tw[fstride*m])
template <typename S, int VS>
KF_HD void bfly3(cpx<S>* v, const cpx<S>* w, cpx<S> c0) {
    typedef Ar<S> A;
    cpx<S> a0 = A::template fixdiv<3>(v[0]), a1 = A::template fixdiv<3>(v[VS]);
    cpx<S> a2 = A::template fixdiv<3>(v[2 * VS]);
    cpx<S> t1 = A::cmul(a1, w[0]), t2 = A::cmul(a2, w[1]);
    cpx<S> s = c_add(t1, t2), d = c_sub(t1, t2);
    cpx<S> o1, o2;
    o1.r = A::st(A::sub(a0.r, A::half(s.r)));
    o1.i = A::st(A::sub(a0.i, A::half(s.i)));
    d = A::mulsc(d, c0.i);
    v[0] = c_add(a0, s);
    o2.r = A::st(A::add(o1.r, d.i));
    o2.i = A::st(A::sub(o1.i, d.r));
    o1.r = A::st(A::sub(o1.r, d.i));
    o1.i = A::st(A::add(o1.i, d.r));
    v[VS] = o1;
    v[2 * VS] = o2;
}

// kf_bfly5, kiss_fft.c:130-189 (c0 = ya = tw[fstride*m], c1 = yb = tw[2*fstride*m])
template <typename S, int VS>
KF_HD void bfly5(cpx<S>* v, const cpx<S>* w, cpx<S> ya, cpx<S> yb) {
    typedef Ar<S> A;
    cpx<S> a0 = A::template fixdiv<5>(v[0]), a1 = A::template fixdiv<5>(v[VS]);
    cpx<S> a2 = A::template fixdiv<5>(v[2 * VS]), a3 = A::template fixdiv<5>(v[3 * VS]);
    cpx<S> a4 = A::template fixdiv<5>(v[4 * VS]);
    cpx<S> t1 = A::cmul(a1, w[0]), t2 = A::cmul(a2, w[1]), t3 = A::cmul(a3, w[2]), t4 = A::cmul(a4, w[3]);
    cpx<S> s14 = c_add(t1, t4), d14 = c_sub(t1, t4);
    cpx<S> s23 = c_add(t2, t3), d23 = c_sub(t2, t3);
    cpx<S> o0, b1, e1, b2, e2;
    o0.r = A::st(A::add(a0.r, A::add(s14.r, s23.r)));
    o0.i = A::st(A::add(a0.i, A::add(s14.i, s23.i)));
    b1.r = A::st(A::add(A::add(a0.r, A::smul(s14.r, ya.r)), A::smul(s23.r, yb.r)));
    b1.i = A::st(A::add(A::add(a0.i, A::smul(s14.i, ya.r)), A::smul(s23.i, yb.r)));
    e1.r = A::st(A::add(A::smul(d14.i, ya.i), A::smul(d23.i, yb.i)));
    e1.i = A::st(A::sub(A::neg(A::smul(d14.r, ya.i)), A::smul(d23.r, yb.i)));
    b2.r = A::st(A::add(A::add(a0.r, A::smul(s14.r, yb.r)), A::smul(s23.r, ya.r)));
    b2.i = A::st(A::add(A::add(a0.i, A::smul(s14.i, yb.r)), A::smul(s23.i, ya.r)));
    e2.r = A::st(A::add(A::neg(A::smul(d14.i, yb.i)), A::smul(d23.i, ya.i)));
    e2.i = A::st(A::sub(A::smul(d14.r, yb.i), A::smul(d23.r, ya.i)));
    v[0] = o0;
    v[VS] = c_sub(b1, e1);
    v[4 * VS] = c_add(b1, e1);
    v[2 * VS] = c_add(b2, e2);
    v[3 * VS] = c_sub(b2, e2);
}

template <typename S, int P, int VS>
KF_HD void bfly(cpx<S>* v, const cpx<S>* w, cpx<S> c0, cpx<S> c1, bool inverse) {
    if constexpr (P == 2) bfly2<S, VS>(v, w);
    if constexpr (P == 3) bfly3<S, VS>(v, w, c0);
    if constexpr (P == 4) bfly4<S, VS>(v, w, inverse);
    if constexpr (P == 5) bfly5<S, VS>(v, w, c0, c1);
}

}  // namespace kf
