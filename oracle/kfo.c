/*
 * CPU oracle for the KISS FFT hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's (mborgerding/kissfft) algorithm:
 * kf_factor, the twiddle tables, the depth-first mixed-radix decimation in
 * time with its radix-2/3/4/5/generic butterflies, the real-input split and
 * merge, the N-D and N-D-real axis passes and the overlap-scrap fast FIR.
 * Each function cites the reference file:line it restates.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library, as the results to compare against or the timed CPU
 * baseline.  The GPU library
 * never links or calls it.
 *
 * Build: oracle/Makefile (gcc -O2 -ffp-contract=off -fopenmp); a second
 * build with -DKFO_CHECK_OVERFLOW (libkfo_ovf.so) also counts the overflows
 * the reference's CHECK_OVERFLOW build warns about.  Floating
 * point contraction must stay off: the float and double builds then perform
 * exactly the reference's operation sequence, and the fixed-point twiddle
 * tables (floor(.5 + SAMP_MAX*cos(phase))) round identically at exact ties.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* kf_factor, kiss_fft.c:306-328: pull out 4s, then 2, then odd trial
 * divisors 3, 5, 7, ... while they do not exceed floor(sqrt(original n));
 * once past that bound the remainder is the last factor.  Writes the pairs
 * (p_i, m_i) with m_i = m_{i-1}/p_i and returns the number of stages. */
int kfo_factor(int n, int *fac) {
    int p = 4, k = 0;
    double lim = floor(sqrt((double)n));
    if (n <= 1) {
        fac[0] = n > 0 ? n : 1;
        fac[1] = 1;
        return 1;
    }
    while (n > 1) {
        while (n % p) {
            if (p == 4)
                p = 2;
            else if (p == 2)
                p = 3;
            else
                p += 2;
            if (p > lim) p = n;
        }
        n /= p;
        fac[2 * k] = p;
        fac[2 * k + 1] = n;
        ++k;
    }
    return k;
}

/* kiss_fft_next_fast_size, kiss_fft.c:412-424 */
int kfo_next_fast_size(int n) {
    for (;; ++n) {
        int m = n;
        while (m % 2 == 0) m /= 2;
        while (m % 3 == 0) m /= 3;
        while (m % 5 == 0) m /= 5;
        if (m <= 1) return n;
    }
}

/* Overflows counted by the CHECK_OVERFLOW build of the oracle
 * (libkfo_ovf.so, -DKFO_CHECK_OVERFLOW); always 0 in the plain build. */
long kfo_overflow_count = 0;

long kfo_overflows_take(void) { return __atomic_exchange_n(&kfo_overflow_count, 0, __ATOMIC_RELAXED); }

int kfo_checks_overflow(void) {
#ifdef KFO_CHECK_OVERFLOW
    return 1;
#else
    return 0;
#endif
}

int kfo_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

#define KFO_S float
#define KFO_FIXED 0
#define KFO_SFX f32
#include "kfo_body.h"
#undef KFO_S
#undef KFO_FIXED
#undef KFO_SFX

#define KFO_S double
#define KFO_FIXED 0
#define KFO_SFX f64
#include "kfo_body.h"
#undef KFO_S
#undef KFO_FIXED
#undef KFO_SFX

#define KFO_S int16_t
#define KFO_FIXED 16
#define KFO_SFX q15
#include "kfo_body.h"
#undef KFO_S
#undef KFO_FIXED
#undef KFO_SFX

#define KFO_S int32_t
#define KFO_FIXED 32
#define KFO_SFX q31
#include "kfo_body.h"
#undef KFO_S
#undef KFO_FIXED
#undef KFO_SFX

/* ------------------------------------------------------------ fast FIR */
/* Real overlap-scrap FIR of tools/kiss_fastfir.c (REAL_FASTFIR, float).
 *
 * kfo_fastfir_nfft: the block size rule of kiss_fastfir_alloc
 * (tools/kiss_fastfir.c:75-87): the power of two above 2*(L-1), at least
 * 2048. */
long kfo_fastfir_nfft(long L) {
    long i = L - 1, nfft = 2;
    do {
        nfft <<= 1;
    } while (i >>= 1);
    if (nfft < 2048) nfft = 2048;
    return nfft;
}

/* Frequency response of the filter (tools/kiss_fastfir.c:142-163): the taps
 * are rotated left by L-1 so the scrap lands at the block tail, transformed,
 * and scaled by (float)(1.0/nfft). */
void kfo_fastfir_response_f32(const float *h, long L, long nfft, kfo_cpx_f32 *H) {
    float *tmp = (float *)calloc((size_t)nfft, sizeof(float));
    tmp[0] = h[L - 1];
    for (long i = 0; i < L - 1; ++i) tmp[nfft - L + 1 + i] = h[i];
    kfo_fftr_batch_f32((int)nfft, tmp, H, 1, 1);
    float scale = 1.0 / nfft;
    for (long i = 0; i < nfft / 2 + 1; ++i) {
        H[i].r *= scale;
        H[i].i *= scale;
    }
    free(tmp);
}

/* Whole-signal filter: the result of kiss_fastfir(cfg, x, y, Ns, &offset=0)
 * followed by the flush call kiss_fastfir(cfg, ..., 0, &offset)
 * (tools/kiss_fastfir.c:186-239).  Full blocks of nfft samples advance by
 * ngood = nfft-L+1; the flush block is the tail zero-padded to nfft.
 * Returns the number of outputs, Ns-L+1 (the valid convolution), or -1. */
long kfo_fastfir_f32(const float *h, long L, long nfft, const float *x, long Ns, float *y, int nthreads) {
    if (nfft <= 0) nfft = kfo_fastfir_nfft(L);
    if (Ns < L - 1 || L < 1 || nfft < L) return -1;
    long ngood = nfft - L + 1, nout = Ns - L + 1, nb = nfft / 2 + 1;
    long nblocks = (nout + ngood - 1) / ngood;
    kfo_cpx_f32 *H = (kfo_cpx_f32 *)malloc(sizeof(kfo_cpx_f32) * (size_t)nb);
    kfo_fastfir_response_f32(h, L, nfft, H);
    (void)nthreads;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
#endif
    {
        float *blk = (float *)malloc(sizeof(float) * (size_t)nfft);
        kfo_cpx_f32 *F = (kfo_cpx_f32 *)malloc(sizeof(kfo_cpx_f32) * (size_t)nb);
        kfo_rplan_f32 *fw = rplan_new_f32((int)nfft, 0), *iv = rplan_new_f32((int)nfft, 1);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (long b = 0; b < nblocks; ++b) {
            long o = b * ngood, avail = Ns - o;
            if (avail > nfft) avail = nfft;
            memcpy(blk, x + o, sizeof(float) * (size_t)avail);
            memset(blk + avail, 0, sizeof(float) * (size_t)(nfft - avail));
            fftr_core_f32(fw->sub, fw->stw, blk, F, fw->tmp);
            for (long i = 0; i < nb; ++i) F[i] = c_mul_f32(F[i], H[i]);
            fftri_core_f32(iv->sub, iv->stw, F, blk, iv->tmp);
            long w = nout - o;
            if (w > ngood) w = ngood;
            memcpy(y + o, blk, sizeof(float) * (size_t)w);
        }
        rplan_free_f32(fw);
        rplan_free_f32(iv);
        free(blk);
        free(F);
    }
    free(H);
    return nout;
}

/* Direct time-domain FIR (the -d path of tools/kiss_fastfir.c:247-333): the
 * independent check of the fast FIR.  y[k] = sum_t h[t] * x[k+L-1-t]. */
long kfo_direct_fir_f32(const float *h, long L, const float *x, long Ns, float *y) {
    if (Ns < L - 1 || L < 1) return -1;
    long nout = Ns - L + 1;
    for (long k = 0; k < nout; ++k) {
        double acc = 0;
        for (long t = 0; t < L; ++t) acc += (double)h[t] * (double)x[k + L - 1 - t];
        y[k] = (float)acc;
    }
    return nout;
}
