/*
 * CPU oracle body -- TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the arithmetic of the KISS FFT reference
 * (mborgerding/kissfft) for one sample type.  It is included once per type by
 * kfo.c with these macros defined:
 *     KFO_S      storage scalar (float, double, int16_t, int32_t)
 *     KFO_FIXED  0 for IEEE types, 16 for Q15, 32 for Q31
 *     KFO_SFX    name suffix (f32, f64, q15, q31)
 *
 * It is used only by the test suite, by __graft_entry__.smoke() and by the
 * CPU-baseline leg of bench.py, always as the results to compare against
 * or the timed CPU baseline -- never as part of the shipped GPU path.
 *
 * Fixed-point model (reference _kiss_fft_guts.h:43-82, 100-130): every value
 * stored into a sample variable is truncated to the storage width; every
 * expression is evaluated in 32-bit wrapping int (int16 operands are
 * promoted; int32 adds wrap, as the reference's gcc builds do); products are
 * taken in SAMPPROD (int32 for Q15, int64 for Q31) and rounded by
 * sround(x) = (x + 2^(FRACBITS-1)) >> FRACBITS.
 */

#define KFO_CAT2(a, b) a##_##b
#define KFO_CAT(a, b) KFO_CAT2(a, b)
#define KFN(name) KFO_CAT(name, KFO_SFX)

typedef struct { KFO_S r, i; } KFN(kfo_cpx);
#define CPX KFN(kfo_cpx)

/* ---------------------------------------------------------------- scalar ops */
#if KFO_FIXED
#  if KFO_FIXED == 32
#    define KFO_FRACBITS 31
#    define KFO_SAMP_MAX 2147483647
typedef int64_t KFN(kfo_prod);
#  else
#    define KFO_FRACBITS 15
#    define KFO_SAMP_MAX 32767
typedef int32_t KFN(kfo_prod);
#  endif
#  define PROD KFN(kfo_prod)
/* 32-bit wrapping integer expression arithmetic */
static inline int32_t KFN(w_add)(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t KFN(w_sub)(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
static inline int32_t KFN(w_neg)(int32_t a) { return (int32_t)(0u - (uint32_t)a); }
/* store to the sample width (two's complement truncation) */
static inline KFO_S KFN(st)(int32_t x) { return (KFO_S)x; }
/* sround(x) of _kiss_fft_guts.h:65 */
static inline KFO_S KFN(sround)(PROD x) {
    return (KFO_S)((x + ((PROD)1 << (KFO_FRACBITS - 1))) >> KFO_FRACBITS);
}
/* S_MUL of _kiss_fft_guts.h:67 */
static inline KFO_S KFN(s_mul)(KFO_S a, KFO_S b) { return KFN(sround)((PROD)a * (PROD)b); }
/* C_MUL of _kiss_fft_guts.h:69-71: each component rounded once */
static inline CPX KFN(c_mul)(CPX a, CPX b) {
    CPX m;
    m.r = KFN(sround)((PROD)a.r * (PROD)b.r - (PROD)a.i * (PROD)b.i);
    m.i = KFN(sround)((PROD)a.r * (PROD)b.i + (PROD)a.i * (PROD)b.r);
    return m;
}
/* C_FIXDIV of _kiss_fft_guts.h:73-78: multiply by SAMP_MAX/p (integer quotient) */
static inline CPX KFN(fixdiv)(CPX c, int p) {
    PROD k = (PROD)(KFO_SAMP_MAX / p);
    c.r = KFN(sround)((PROD)c.r * k);
    c.i = KFN(sround)((PROD)c.i * k);
    return c;
}
/* C_MULBYSCALAR of _kiss_fft_guts.h:80-82 */
static inline CPX KFN(mul_scalar)(CPX c, KFO_S s) {
    c.r = KFN(sround)((PROD)c.r * (PROD)s);
    c.i = KFN(sround)((PROD)c.i * (PROD)s);
    return c;
}
/* HALF_OF of _kiss_fft_guts.h:130 (arithmetic shift of the int expression) */
static inline int32_t KFN(half)(int32_t x) { return x >> 1; }
/* CHECK_OVERFLOW_OP of _kiss_fft_guts.h:57-61 in the counting build
 * (KFO_CHECK_OVERFLOW): a sum or difference of two samples, taken in the
 * product type, outside [SAMP_MIN, SAMP_MAX] counts one overflow where the
 * reference built with CHECK_OVERFLOW prints one warning. */
#  ifdef KFO_CHECK_OVERFLOW
#    define KFO_OVF(a, op, b) KFN(ovf_note)((int64_t)(a) op (int64_t)(b))
static inline void KFN(ovf_note)(int64_t v) {
    if (v > KFO_SAMP_MAX || v < -KFO_SAMP_MAX - 1) __atomic_fetch_add(&kfo_overflow_count, 1, __ATOMIC_RELAXED);
}
#  else
#    define KFO_OVF(a, op, b) ((void)0)
#  endif
#  define E_ADD(a, b) KFN(w_add)((int32_t)(a), (int32_t)(b))
#  define E_SUB(a, b) KFN(w_sub)((int32_t)(a), (int32_t)(b))
#  define E_NEG(a) KFN(w_neg)((int32_t)(a))
#  define ST(x) KFN(st)(x)
#  define HALF(x) KFN(half)(x)
#else
static inline KFO_S KFN(s_mul)(KFO_S a, KFO_S b) { return a * b; }
static inline CPX KFN(c_mul)(CPX a, CPX b) {
    CPX m;
    m.r = a.r * b.r - a.i * b.i;
    m.i = a.r * b.i + a.i * b.r;
    return m;
}
static inline CPX KFN(fixdiv)(CPX c, int p) { (void)p; return c; }
static inline CPX KFN(mul_scalar)(CPX c, KFO_S s) { c.r *= s; c.i *= s; return c; }
#  define KFO_OVF(a, op, b) ((void)0)
#  define E_ADD(a, b) ((a) + (b))
#  define E_SUB(a, b) ((a) - (b))
#  define E_NEG(a) (-(a))
#  define ST(x) ((KFO_S)(x))
#  define HALF(x) ((x) * (KFO_S)0.5)
#endif

/* C_ADD / C_ADDTO and C_SUB / C_SUBFROM (_kiss_fft_guts.h:100-124), the
 * macros that carry the reference's overflow checks */
static inline CPX KFN(c_add)(CPX a, CPX b) {
    CPX r;
    KFO_OVF(a.r, +, b.r);
    KFO_OVF(a.i, +, b.i);
    r.r = ST(E_ADD(a.r, b.r));
    r.i = ST(E_ADD(a.i, b.i));
    return r;
}
static inline CPX KFN(c_sub)(CPX a, CPX b) {
    CPX r;
    KFO_OVF(a.r, -, b.r);
    KFO_OVF(a.i, -, b.i);
    r.r = ST(E_SUB(a.r, b.r));
    r.i = ST(E_SUB(a.i, b.i));
    return r;
}

/* ------------------------------------------------------------- twiddles */
/* kf_cexp / KISS_FFT_COS / KISS_FFT_SIN, _kiss_fft_guts.h:127-145 */
static inline CPX KFN(kfo_cexp)(double phase) {
    CPX x;
#if KFO_FIXED
    x.r = (KFO_S)floor(.5 + KFO_SAMP_MAX * cos(phase));
    x.i = (KFO_S)floor(.5 + KFO_SAMP_MAX * sin(phase));
#else
    x.r = (KFO_S)cos(phase);
    x.i = (KFO_S)sin(phase);
#endif
    return x;
}

/* Twiddle table of kiss_fft_alloc, kiss_fft.c:361-367. */
void KFN(kfo_twiddles)(int nfft, int inverse, CPX *tw) {
    for (int i = 0; i < nfft; ++i) {
        const double pi = 3.141592653589793238462643383279502884197169399375105820974944;
        double phase = -2 * pi * i / nfft;
        if (inverse) phase *= -1;
        tw[i] = KFN(kfo_cexp)(phase);
    }
}

/* Super twiddles of kiss_fftr_alloc, kiss_fftr.c:53-59 (ncfft = nfft/2). */
void KFN(kfo_super_twiddles)(int ncfft, int inverse, CPX *stw) {
    for (int i = 0; i < ncfft / 2; ++i) {
        double phase = -3.14159265358979323846264338327 * ((double)(i + 1) / ncfft + .5);
        if (inverse) phase *= -1;
        stw[i] = KFN(kfo_cexp)(phase);
    }
}

/* ------------------------------------------------------------ butterflies */
/* Each butterfly restates one kf_bfly* routine of kiss_fft.c: it combines,
 * for every u < m, the p legs F[u + q*m] (q < p) in place.  Twiddle for leg
 * q at offset u is tw[q*u*fstride]. */

/* kiss_fft.c:15-36 */
static void KFN(bf2)(CPX *F, size_t fs, const CPX *tw, int m) {
    for (int u = 0; u < m; ++u) {
        CPX a = KFN(fixdiv)(F[u], 2), b = KFN(fixdiv)(F[u + m], 2);
        CPX t = KFN(c_mul)(b, tw[u * fs]);
        F[u + m] = KFN(c_sub)(a, t);
        F[u] = KFN(c_add)(a, t);
    }
}

/* kiss_fft.c:38-84 */
static void KFN(bf4)(CPX *F, size_t fs, const CPX *tw, int m, int inverse) {
    for (int u = 0; u < m; ++u) {
        CPX a0 = KFN(fixdiv)(F[u], 4), a1 = KFN(fixdiv)(F[u + m], 4);
        CPX a2 = KFN(fixdiv)(F[u + 2 * m], 4), a3 = KFN(fixdiv)(F[u + 3 * m], 4);
        CPX t0 = KFN(c_mul)(a1, tw[u * fs]);
        CPX t1 = KFN(c_mul)(a2, tw[2 * u * fs]);
        CPX t2 = KFN(c_mul)(a3, tw[3 * u * fs]);
        CPX d02 = KFN(c_sub)(a0, t1);
        CPX s02 = KFN(c_add)(a0, t1);
        CPX s13 = KFN(c_add)(t0, t2);
        CPX d13 = KFN(c_sub)(t0, t2);
        CPX o1, o3;
        F[u + 2 * m] = KFN(c_sub)(s02, s13);
        F[u] = KFN(c_add)(s02, s13);
        if (inverse) {
            o1.r = ST(E_SUB(d02.r, d13.i)); o1.i = ST(E_ADD(d02.i, d13.r));
            o3.r = ST(E_ADD(d02.r, d13.i)); o3.i = ST(E_SUB(d02.i, d13.r));
        } else {
            o1.r = ST(E_ADD(d02.r, d13.i)); o1.i = ST(E_SUB(d02.i, d13.r));
            o3.r = ST(E_SUB(d02.r, d13.i)); o3.i = ST(E_ADD(d02.i, d13.r));
        }
        F[u + m] = o1;
        F[u + 3 * m] = o3;
    }
}

/* kiss_fft.c:86-128; epi3 = tw[fstride*m] */
static void KFN(bf3)(CPX *F, size_t fs, const CPX *tw, int m) {
    CPX epi3 = tw[fs * m];
    for (int u = 0; u < m; ++u) {
        CPX a0 = KFN(fixdiv)(F[u], 3), a1 = KFN(fixdiv)(F[u + m], 3), a2 = KFN(fixdiv)(F[u + 2 * m], 3);
        CPX t1 = KFN(c_mul)(a1, tw[u * fs]);
        CPX t2 = KFN(c_mul)(a2, tw[2 * u * fs]);
        CPX s = KFN(c_add)(t1, t2);
        CPX d = KFN(c_sub)(t1, t2);
        CPX o1, o2;
        o1.r = ST(E_SUB(a0.r, HALF(s.r)));
        o1.i = ST(E_SUB(a0.i, HALF(s.i)));
        d = KFN(mul_scalar)(d, epi3.i);
        F[u] = KFN(c_add)(a0, s);
        o2.r = ST(E_ADD(o1.r, d.i));
        o2.i = ST(E_SUB(o1.i, d.r));
        o1.r = ST(E_SUB(o1.r, d.i));
        o1.i = ST(E_ADD(o1.i, d.r));
        F[u + m] = o1;
        F[u + 2 * m] = o2;
    }
}

/* kiss_fft.c:130-189; ya = tw[fstride*m], yb = tw[2*fstride*m] */
static void KFN(bf5)(CPX *F, size_t fs, const CPX *tw, int m) {
    CPX ya = tw[fs * m], yb = tw[2 * fs * m];
    for (int u = 0; u < m; ++u) {
        CPX a0 = KFN(fixdiv)(F[u], 5), a1 = KFN(fixdiv)(F[u + m], 5), a2 = KFN(fixdiv)(F[u + 2 * m], 5);
        CPX a3 = KFN(fixdiv)(F[u + 3 * m], 5), a4 = KFN(fixdiv)(F[u + 4 * m], 5);
        CPX t1 = KFN(c_mul)(a1, tw[u * fs]);
        CPX t2 = KFN(c_mul)(a2, tw[2 * u * fs]);
        CPX t3 = KFN(c_mul)(a3, tw[3 * u * fs]);
        CPX t4 = KFN(c_mul)(a4, tw[4 * u * fs]);
        CPX s14 = KFN(c_add)(t1, t4), d14 = KFN(c_sub)(t1, t4);
        CPX s23 = KFN(c_add)(t2, t3), d23 = KFN(c_sub)(t2, t3);
        CPX o0, b1, c1, b2, c2;
        o0.r = ST(E_ADD(a0.r, E_ADD(s14.r, s23.r)));
        o0.i = ST(E_ADD(a0.i, E_ADD(s14.i, s23.i)));
        b1.r = ST(E_ADD(E_ADD(a0.r, KFN(s_mul)(s14.r, ya.r)), KFN(s_mul)(s23.r, yb.r)));
        b1.i = ST(E_ADD(E_ADD(a0.i, KFN(s_mul)(s14.i, ya.r)), KFN(s_mul)(s23.i, yb.r)));
        c1.r = ST(E_ADD(KFN(s_mul)(d14.i, ya.i), KFN(s_mul)(d23.i, yb.i)));
        c1.i = ST(E_SUB(E_NEG(KFN(s_mul)(d14.r, ya.i)), KFN(s_mul)(d23.r, yb.i)));
        b2.r = ST(E_ADD(E_ADD(a0.r, KFN(s_mul)(s14.r, yb.r)), KFN(s_mul)(s23.r, ya.r)));
        b2.i = ST(E_ADD(E_ADD(a0.i, KFN(s_mul)(s14.i, yb.r)), KFN(s_mul)(s23.i, ya.r)));
        c2.r = ST(E_ADD(E_NEG(KFN(s_mul)(d14.i, yb.i)), KFN(s_mul)(d23.i, ya.i)));
        c2.i = ST(E_SUB(KFN(s_mul)(d14.r, yb.i), KFN(s_mul)(d23.r, ya.i)));
        F[u] = o0;
        F[u + m] = KFN(c_sub)(b1, c1);
        F[u + 4 * m] = KFN(c_add)(b1, c1);
        F[u + 2 * m] = KFN(c_add)(b2, c2);
        F[u + 3 * m] = KFN(c_sub)(b2, c2);
    }
}

/* kiss_fft.c:192-233: O(p^2) butterfly for any other radix.  The twiddle
 * index for output k and leg q is (q*fstride*k) mod N, accumulated as the
 * reference does; legs are summed in order q = 1..p-1. */
static void KFN(bfg)(CPX *F, size_t fs, const CPX *tw, int m, int p, int N, CPX *scr) {
    for (int u = 0; u < m; ++u) {
        for (int q = 0; q < p; ++q) scr[q] = KFN(fixdiv)(F[u + q * m], p);
        for (int q1 = 0; q1 < p; ++q1) {
            int k = u + q1 * m;
            int twidx = 0;
            CPX acc = scr[0];
            for (int q = 1; q < p; ++q) {
                twidx += (int)(fs * k);
                if (twidx >= N) twidx -= N;
                acc = KFN(c_add)(acc, KFN(c_mul)(scr[q], tw[twidx]));
            }
            F[k] = acc;
        }
    }
}

/* --------------------------------------------------------------- plans */
typedef struct {
    int nfft, inverse;
    int fac[64];
    CPX *tw;
    CPX *scr;   /* scratch for the generic butterfly (the reference mallocs per call) */
} KFN(kfo_plan);
#define PLAN KFN(kfo_plan)

static PLAN *KFN(plan_new)(int nfft, int inverse) {
    PLAN *p = (PLAN *)calloc(1, sizeof(PLAN));
    p->nfft = nfft;
    p->inverse = inverse;
    p->tw = (CPX *)malloc(sizeof(CPX) * (size_t)(nfft > 0 ? nfft : 1));
    p->scr = (CPX *)malloc(sizeof(CPX) * (size_t)(nfft > 0 ? nfft : 1));
    KFN(kfo_twiddles)(nfft, inverse, p->tw);
    kfo_factor(nfft, p->fac);
    return p;
}
static void KFN(plan_free)(PLAN *p) {
    if (!p) return;
    free(p->tw);
    free(p->scr);
    free(p);
}

/* The radix-p butterfly of one stage (the switch at the end of kf_work,
 * kiss_fft.c:293-299); scr holds p elements for the generic radix. */
static void KFN(stage)(CPX *out, size_t fs, int p, int m, const PLAN *pl, CPX *scr) {
    switch (p) {
        case 2: KFN(bf2)(out, fs, pl->tw, m); break;
        case 3: KFN(bf3)(out, fs, pl->tw, m); break;
        case 4: KFN(bf4)(out, fs, pl->tw, m, pl->inverse); break;
        case 5: KFN(bf5)(out, fs, pl->tw, m); break;
        default: KFN(bfg)(out, fs, pl->tw, m, p, pl->nfft, scr); break;
    }
}

/* Depth-first decimation in time, the recursion of kf_work (kiss_fft.c:235-300)
 * without the OpenMP top-level split: the p sub-transforms of length m read
 * the input decimated by fstride*p, then the radix-p butterfly combines them.
 * scr is the generic butterfly's scratch (the reference mallocs it per
 * butterfly call, kiss_fft.c:205). */
static void KFN(work)(CPX *out, const CPX *in, size_t fs, int istride, const int *fac, const PLAN *pl, CPX *scr) {
    const int p = fac[0], m = fac[1];
    if (m == 1) {
        for (int q = 0; q < p; ++q) out[q] = in[(size_t)q * fs * istride];
    } else {
        for (int q = 0; q < p; ++q)
            KFN(work)(out + q * m, in + (size_t)q * fs * istride, fs * p, istride, fac + 2, pl, scr);
    }
    KFN(stage)(out, fs, p, m, pl, scr);
}

/* kiss_fft_stride, kiss_fft.c:375-399 (out-of-place case).  nfft == 1 runs
 * the reference's factor list [1, 1]: a leaf copy and a p = 1 generic
 * butterfly, which in fixed point still scales by SAMP_MAX/1. */
static void KFN(exec)(const PLAN *pl, const CPX *in, int istride, CPX *out) {
    KFN(work)(out, in, 1, istride, pl->fac, pl, pl->scr);
}

/* ------------------------------------------------------------ public API */

/* One complex transform (kiss_fft_stride semantics, out-of-place). */
void KFN(kfo_fft)(int nfft, int inverse, const CPX *in, int istride, CPX *out) {
    PLAN *pl = KFN(plan_new)(nfft, inverse);
    KFN(exec)(pl, in, istride, out);
    KFN(plan_free)(pl);
}

/* A batch of contiguous complex transforms; nthreads > 1 splits the batch
 * over OpenMP threads (one plan per thread: the generic butterfly's scratch
 * lives in the plan). */
void KFN(kfo_fft_batch)(int nfft, int inverse, const CPX *in, CPX *out, long batch, int nthreads) {
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
    {
        PLAN *pl = KFN(plan_new)(nfft, inverse);
#pragma omp for schedule(static)
        for (long b = 0; b < batch; ++b) KFN(exec)(pl, in + b * nfft, 1, out + b * nfft);
        KFN(plan_free)(pl);
    }
#else
    (void)nthreads;
    PLAN *pl = KFN(plan_new)(nfft, inverse);
    for (long b = 0; b < batch; ++b) KFN(exec)(pl, in + b * nfft, 1, out + b * nfft);
    KFN(plan_free)(pl);
#endif
}

/* A batch of contiguous complex transforms, one after the other, each with
 * the reference's KISSFFT_OPENMP split (kf_work, kiss_fft.c:250-272): at the
 * top level (fstride == 1), when p <= 5 and m != 1, the p sub-transforms run
 * as an OpenMP parallel for and the top stage's butterfly follows the join;
 * other plans run on one thread.  This is how the reference's OpenMP build
 * uses the cores (at most p of them per transform); the results equal
 * kfo_fft_batch's bit for bit.  Returns 0, or -1 when scratch allocation
 * fails. */
int KFN(kfo_fft_batch_legs)(int nfft, int inverse, const CPX *in, CPX *out, long batch, int nthreads) {
    PLAN *pl = KFN(plan_new)(nfft, inverse);
    const int p = pl->fac[0], m = pl->fac[1];
    const int split = p <= 5 && m != 1;
    /* one generic-butterfly scratch per leg: the legs run at once */
    CPX *scr = split ? (CPX *)malloc(sizeof(CPX) * (size_t)p * (size_t)nfft) : NULL;
    if (split && !scr) {
        KFN(plan_free)(pl);
        return -1;
    }
    for (long b = 0; b < batch; ++b) {
        const CPX *f = in + b * nfft;
        CPX *F = out + b * nfft;
        if (!split) {
            KFN(exec)(pl, f, 1, F);
            continue;
        }
#ifdef _OPENMP
#pragma omp parallel for num_threads(nthreads > 0 ? nthreads : 1) schedule(static)
#endif
        for (int k = 0; k < p; ++k)
            KFN(work)(F + k * m, f + k, (size_t)p, 1, pl->fac + 2, pl, scr + (size_t)k * nfft);
        KFN(stage)(F, 1, p, m, pl, pl->scr);
    }
#ifndef _OPENMP
    (void)nthreads;
#endif
    free(scr);
    KFN(plan_free)(pl);
    return 0;
}

/* Real forward transform, kiss_fftr.c:63-117.  ncfft = nfft/2. */
static void KFN(fftr_core)(const PLAN *sub, const CPX *stw, const KFO_S *t, CPX *f, CPX *tmp) {
    int ncfft = sub->nfft;
    KFN(exec)(sub, (const CPX *)t, 1, tmp);
    CPX dc = KFN(fixdiv)(tmp[0], 2);
    KFO_OVF(dc.r, +, dc.i);  /* kiss_fftr.c:94-95 */
    KFO_OVF(dc.r, -, dc.i);
    f[0].r = ST(E_ADD(dc.r, dc.i));
    f[ncfft].r = ST(E_SUB(dc.r, dc.i));
    f[0].i = 0;
    f[ncfft].i = 0;
    for (int k = 1; k <= ncfft / 2; ++k) {
        CPX fpk = tmp[k], fpnk;
        fpnk.r = tmp[ncfft - k].r;
        fpnk.i = ST(E_NEG(tmp[ncfft - k].i));
        fpk = KFN(fixdiv)(fpk, 2);
        fpnk = KFN(fixdiv)(fpnk, 2);
        CPX f1k = KFN(c_add)(fpk, fpnk);
        CPX f2k = KFN(c_sub)(fpk, fpnk);
        CPX tw = KFN(c_mul)(f2k, stw[k - 1]);
        f[k].r = ST(HALF(E_ADD(f1k.r, tw.r)));
        f[k].i = ST(HALF(E_ADD(f1k.i, tw.i)));
        f[ncfft - k].r = ST(HALF(E_SUB(f1k.r, tw.r)));
        f[ncfft - k].i = ST(HALF(E_SUB(tw.i, f1k.i)));
    }
}

/* Real inverse transform, kiss_fftr.c:119-155. */
static void KFN(fftri_core)(const PLAN *sub, const CPX *stw, const CPX *f, KFO_S *t, CPX *tmp) {
    int ncfft = sub->nfft;
    tmp[0].r = ST(E_ADD(f[0].r, f[ncfft].r));
    tmp[0].i = ST(E_SUB(f[0].r, f[ncfft].r));
    tmp[0] = KFN(fixdiv)(tmp[0], 2);
    for (int k = 1; k <= ncfft / 2; ++k) {
        CPX fk = f[k], fnkc;
        fnkc.r = f[ncfft - k].r;
        fnkc.i = ST(E_NEG(f[ncfft - k].i));
        fk = KFN(fixdiv)(fk, 2);
        fnkc = KFN(fixdiv)(fnkc, 2);
        CPX fek = KFN(c_add)(fk, fnkc);
        CPX d = KFN(c_sub)(fk, fnkc);
        CPX fok = KFN(c_mul)(d, stw[k - 1]);
        tmp[k] = KFN(c_add)(fek, fok);
        tmp[ncfft - k] = KFN(c_sub)(fek, fok);
        tmp[ncfft - k].i = ST(E_NEG(tmp[ncfft - k].i));
    }
    KFN(exec)(sub, tmp, 1, (CPX *)t);
}

typedef struct {
    PLAN *sub;
    CPX *stw;
    CPX *tmp;
} KFN(kfo_rplan);
#define RPLAN KFN(kfo_rplan)

static RPLAN *KFN(rplan_new)(int nfft, int inverse) {
    RPLAN *r = (RPLAN *)calloc(1, sizeof(RPLAN));
    int ncfft = nfft / 2;
    r->sub = KFN(plan_new)(ncfft, inverse);
    r->stw = (CPX *)malloc(sizeof(CPX) * (size_t)(ncfft / 2 + 1));
    r->tmp = (CPX *)malloc(sizeof(CPX) * (size_t)(ncfft + 1));
    KFN(kfo_super_twiddles)(ncfft, inverse, r->stw);
    return r;
}
static void KFN(rplan_free)(RPLAN *r) {
    if (!r) return;
    KFN(plan_free)(r->sub);
    free(r->stw);
    free(r->tmp);
    free(r);
}

/* Batch of real forward transforms: batch rows of nfft reals -> nfft/2+1 bins. */
int KFN(kfo_fftr_batch)(int nfft, const KFO_S *t, CPX *f, long batch, int nthreads) {
    if (nfft & 1) return -1;
    long nb = nfft / 2 + 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
    {
        RPLAN *r = KFN(rplan_new)(nfft, 0);
#pragma omp for schedule(static)
        for (long b = 0; b < batch; ++b) KFN(fftr_core)(r->sub, r->stw, t + b * nfft, f + b * nb, r->tmp);
        KFN(rplan_free)(r);
    }
#else
    (void)nthreads;
    RPLAN *r = KFN(rplan_new)(nfft, 0);
    for (long b = 0; b < batch; ++b) KFN(fftr_core)(r->sub, r->stw, t + b * nfft, f + b * nb, r->tmp);
    KFN(rplan_free)(r);
#endif
    return 0;
}

/* Batch of real inverse transforms: nfft/2+1 bins -> nfft reals. */
int KFN(kfo_fftri_batch)(int nfft, const CPX *f, KFO_S *t, long batch, int nthreads) {
    if (nfft & 1) return -1;
    long nb = nfft / 2 + 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
    {
        RPLAN *r = KFN(rplan_new)(nfft, 1);
#pragma omp for schedule(static)
        for (long b = 0; b < batch; ++b) KFN(fftri_core)(r->sub, r->stw, f + b * nb, t + b * nfft, r->tmp);
        KFN(rplan_free)(r);
    }
#else
    (void)nthreads;
    RPLAN *r = KFN(rplan_new)(nfft, 1);
    for (long b = 0; b < batch; ++b) KFN(fftri_core)(r->sub, r->stw, f + b * nb, t + b * nfft, r->tmp);
    KFN(rplan_free)(r);
#endif
    return 0;
}

/* Complex transform of every fiber along one axis of a row-major array, in
 * place.  Applying it to axes 0, 1, ..., ndims-1 in that order gives every
 * 1-D transform the same input vector as the reference's transposing passes
 * (kiss_fftnd.c:156-188, each pass transforming the columns of a
 * dims[k] x (dimprod/dims[k]) view). */
static void KFN(axis_pass)(CPX *a, const int *dims, int ndims, int axis, int inverse, CPX *col, CPX *res) {
    long outer = 1, inner = 1;
    for (int i = 0; i < axis; ++i) outer *= dims[i];
    for (int i = axis + 1; i < ndims; ++i) inner *= dims[i];
    int n = dims[axis];
    PLAN *pl = KFN(plan_new)(n, inverse);
    for (long o = 0; o < outer; ++o)
        for (long i = 0; i < inner; ++i) {
            CPX *base = a + o * n * inner + i;
            for (int r = 0; r < n; ++r) col[r] = base[r * inner];
            KFN(exec)(pl, col, 1, res);
            for (int r = 0; r < n; ++r) base[r * inner] = res[r];
        }
    KFN(plan_free)(pl);
}

/* N-D complex transform (kiss_fftnd semantics). */
void KFN(kfo_fftnd)(const int *dims, int ndims, int inverse, const CPX *in, CPX *out) {
    long tot = 1;
    int maxd = 1;
    for (int i = 0; i < ndims; ++i) { tot *= dims[i]; if (dims[i] > maxd) maxd = dims[i]; }
    CPX *col = (CPX *)malloc(sizeof(CPX) * (size_t)maxd), *res = (CPX *)malloc(sizeof(CPX) * (size_t)maxd);
    memmove(out, in, sizeof(CPX) * (size_t)tot);
    for (int k = 0; k < ndims; ++k) KFN(axis_pass)(out, dims, ndims, k, inverse, col, res);
    free(col);
    free(res);
}

/* N-D real forward transform (kiss_fftndr.c:86-110): real transform of each
 * row of the last axis, then the complex axes 0..ndims-2 on the bins. */
void KFN(kfo_fftndr)(const int *dims, int ndims, const KFO_S *t, CPX *f) {
    int dr = dims[ndims - 1];
    long other = 1;
    for (int i = 0; i < ndims - 1; ++i) other *= dims[i];
    KFN(kfo_fftr_batch)(dr, t, f, other, 1);
    int odims[33];
    int maxd = dr / 2 + 1;
    for (int i = 0; i < ndims - 1; ++i) { odims[i] = dims[i]; if (dims[i] > maxd) maxd = dims[i]; }
    odims[ndims - 1] = dr / 2 + 1;
    CPX *col = (CPX *)malloc(sizeof(CPX) * (size_t)maxd), *res = (CPX *)malloc(sizeof(CPX) * (size_t)maxd);
    for (int k = 0; k < ndims - 1; ++k) KFN(axis_pass)(f, odims, ndims, k, 0, col, res);
    free(col);
    free(res);
}

/* N-D real inverse transform (kiss_fftndr.c:112-132): complex inverse axes
 * 0..ndims-2 on the bins, then the real inverse of each row. */
void KFN(kfo_fftndri)(const int *dims, int ndims, const CPX *f, KFO_S *t) {
    int dr = dims[ndims - 1];
    long other = 1;
    for (int i = 0; i < ndims - 1; ++i) other *= dims[i];
    long nb = dr / 2 + 1;
    CPX *w = (CPX *)malloc(sizeof(CPX) * (size_t)(other * nb));
    memcpy(w, f, sizeof(CPX) * (size_t)(other * nb));
    int odims[33];
    int maxd = (int)nb;
    for (int i = 0; i < ndims - 1; ++i) { odims[i] = dims[i]; if (dims[i] > maxd) maxd = dims[i]; }
    odims[ndims - 1] = (int)nb;
    CPX *col = (CPX *)malloc(sizeof(CPX) * (size_t)maxd), *res = (CPX *)malloc(sizeof(CPX) * (size_t)maxd);
    for (int k = 0; k < ndims - 1; ++k) KFN(axis_pass)(w, odims, ndims, k, 1, col, res);
    KFN(kfo_fftri_batch)(dr, w, t, other, 1);
    free(col);
    free(res);
    free(w);
}

#undef CPX
#undef PLAN
#undef RPLAN
#undef E_ADD
#undef E_SUB
#undef E_NEG
#undef ST
#undef HALF
#undef KFO_OVF
#undef PROD
#undef KFO_FRACBITS
#undef KFO_SAMP_MAX
#undef KFN
#undef KFO_CAT
#undef KFO_CAT2
