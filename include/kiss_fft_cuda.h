/*
 * kiss_fft_cuda.h -- drop-in GPU replacements for the KISS FFT calls.
 *
 * Each function below replaces the reference (mborgerding/kissfft) call
 * cited beside it, with the same argument order, the same meaning and the
 * same error behaviour (NULL from an alloc; a message on stderr and an
 * early return from a void call), on NVIDIA GB300 (sm_103a).
 *
 * Sample type.  As in the reference (kiss_fft.h:73-85) it is fixed at
 * compile time: FIXED_POINT=16 selects int16_t (Q15), FIXED_POINT=32
 * int32_t (Q31), otherwise kiss_fft_scalar (default float; -Dkiss_fft_scalar=
 * double for double).  Link the library of the same type:
 *     libkissfft_cuda-float.so   libkissfft_cuda-double.so
 *     libkissfft_cuda-int16_t.so libkissfft_cuda-int32_t.so
 * Q15/Q31 results are bit-identical to the reference's fixed-point builds;
 * float/double results agree with an FP64 transform to within
 * 2e-7*log2(N) (float) and 1e-15*log2(N) (double) relative L2.
 *
 * Buffers.  Device pointers are the fast path: the call is enqueued on the
 * library stream (kiss_fft_cuda_set_stream; default the legacy default
 * stream) and returns at once.  Host pointers are also accepted: they are
 * staged through device memory and the call returns when the result is in
 * host memory, exactly like the reference's synchronous calls.
 *
 * Configs.  A cfg holds device memory, so it must be released with the
 * matching kiss_*_cuda_free call, not with free() (the reference's
 * kiss_fft_free is free, kiss_fft.h:138).  The mem/lenmem placement protocol
 * of kiss_fft_alloc (kiss_fft.h:94-115) is kept for the host handle.  Unlike
 * the reference's real, N-D and fast-FIR configs (which embed a scratch
 * buffer), every cfg here may be shared between threads and streams.
 *
 * If the reference's kiss_fft.h is also included, include it first: the
 * types below are then taken from it.
 */
#ifndef KISS_FFT_CUDA_H
#define KISS_FFT_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifndef KISS_FFT_H
#ifdef FIXED_POINT
#if (FIXED_POINT == 32)
#define kiss_fft_scalar int32_t
#else
#define kiss_fft_scalar int16_t
#endif
#else
#ifndef kiss_fft_scalar
#define kiss_fft_scalar float
#endif
#endif
typedef struct {
    kiss_fft_scalar r;
    kiss_fft_scalar i;
} kiss_fft_cpx;
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- complex 1-D: kiss_fft.h ------------------------------------------- */
typedef struct kiss_fft_cuda_state *kiss_fft_cuda_cfg;

/* kiss_fft_alloc, kiss_fft.h:117 (kiss_fft.c:337-372) */
kiss_fft_cuda_cfg kiss_fft_cuda_alloc(int nfft, int inverse_fft, void *mem, size_t *lenmem);
/* kiss_fft, kiss_fft.h:129 (kiss_fft.c:401-404) */
void kiss_fft_cuda(kiss_fft_cuda_cfg cfg, const kiss_fft_cpx *fin, kiss_fft_cpx *fout);
/* kiss_fft_stride, kiss_fft.h:134 (kiss_fft.c:375-399) */
void kiss_fft_cuda_stride(kiss_fft_cuda_cfg cfg, const kiss_fft_cpx *fin, kiss_fft_cpx *fout, int fin_stride);
/* kiss_fft_free (= free), kiss_fft.h:138; releases the device plan too */
void kiss_fft_cuda_free(void *cfg);
/* kiss_fft_cleanup, kiss_fft.h:144 */
void kiss_fft_cuda_cleanup(void);
/* kiss_fft_next_fast_size, kiss_fft.h:150 */
int kiss_fft_cuda_next_fast_size(int n);

/* The loop `for b < batch: kiss_fft(cfg, fin + b*in_dist, fout + b*out_dist)`
 * (the reference's callers, e.g. tools/fftutil.c:30) as one launch.
 * in_dist/out_dist in complex elements, 0 = nfft.  Returns 0 or a negative
 * status (see kissfft_gb300.h). */
int kiss_fft_cuda_batch(kiss_fft_cuda_cfg cfg, const kiss_fft_cpx *fin, kiss_fft_cpx *fout, long long batch,
                        long long in_dist, long long out_dist);

/* ---- plan cache: kfc.h --------------------------------------------------- */
/* The plan cache of kfc.h (kfc.c:24-83): the first call for a size builds
 * the device plan, later calls reuse it.  Keyed by (nfft, direction) per
 * sample-type library like find_cached_fft, but guarded by a mutex (the
 * reference's list is not thread-safe, kfc.c:21-22).  Buffers as for
 * kiss_fft_cuda. */
/* kfc_fft, kfc.h:43 */
void kfc_cuda_fft(int nfft, const kiss_fft_cpx *fin, kiss_fft_cpx *fout);
/* kfc_ifft, kfc.h:45 */
void kfc_cuda_ifft(int nfft, const kiss_fft_cpx *fin, kiss_fft_cpx *fout);
/* kfc_cleanup, kfc.h:48: waits for the library stream, then frees every
 * cached plan */
void kfc_cuda_cleanup(void);
/* The number of cached plans (the reference's static ncached, kfc.c:22,
 * which its KFC_TEST self-test checks, kfc.c:85-109). */
int kfc_cuda_ncached(void);

/* ---- real 1-D: kiss_fftr.h ---------------------------------------------- */
typedef struct kiss_fft_cuda_state *kiss_fftr_cuda_cfg;

/* kiss_fftr_alloc, kiss_fftr.h:29 (kiss_fftr.c:21-61); NULL for odd nfft */
kiss_fftr_cuda_cfg kiss_fftr_cuda_alloc(int nfft, int inverse_fft, void *mem, size_t *lenmem);
/* kiss_fftr, kiss_fftr.h:37 (kiss_fftr.c:63-117): nfft reals -> nfft/2+1 bins */
void kiss_fftr_cuda(kiss_fftr_cuda_cfg cfg, const kiss_fft_scalar *timedata, kiss_fft_cpx *freqdata);
/* kiss_fftri, kiss_fftr.h:43 (kiss_fftr.c:119-155): nfft/2+1 bins -> nfft reals */
void kiss_fftri_cuda(kiss_fftr_cuda_cfg cfg, const kiss_fft_cpx *freqdata, kiss_fft_scalar *timedata);
/* kiss_fftr_free, kiss_fftr.h:49 */
void kiss_fftr_cuda_free(void *cfg);
/* batched forms (distances in reals / bins, 0 = packed) */
int kiss_fftr_cuda_batch(kiss_fftr_cuda_cfg cfg, const kiss_fft_scalar *timedata, kiss_fft_cpx *freqdata,
                         long long batch, long long in_dist, long long out_dist);
int kiss_fftri_cuda_batch(kiss_fftr_cuda_cfg cfg, const kiss_fft_cpx *freqdata, kiss_fft_scalar *timedata,
                          long long batch, long long in_dist, long long out_dist);

/* ---- complex N-D: kiss_fftnd.h ------------------------------------------- */
typedef struct kiss_fft_cuda_state *kiss_fftnd_cuda_cfg;

/* kiss_fftnd_alloc, kiss_fftnd.h:20 (kiss_fftnd.c:20-92) */
kiss_fftnd_cuda_cfg kiss_fftnd_cuda_alloc(const int *dims, int ndims, int inverse_fft, void *mem, size_t *lenmem);
/* kiss_fftnd, kiss_fftnd.h:21 (kiss_fftnd.c:156-188); fin == fout allowed */
void kiss_fftnd_cuda(kiss_fftnd_cuda_cfg cfg, const kiss_fft_cpx *fin, kiss_fft_cpx *fout);
void kiss_fftnd_cuda_free(void *cfg);

/* ---- real N-D: kiss_fftndr.h --------------------------------------------- */
typedef struct kiss_fft_cuda_state *kiss_fftndr_cuda_cfg;

/* kiss_fftndr_alloc, kiss_fftndr.h:23 (kiss_fftndr.c:30-84); the halved axis
 * is the last one, dims[ndims-1], which must be even */
kiss_fftndr_cuda_cfg kiss_fftndr_cuda_alloc(const int *dims, int ndims, int inverse_fft, void *mem, size_t *lenmem);
/* kiss_fftndr, kiss_fftndr.h:31 (kiss_fftndr.c:86-110) */
void kiss_fftndr_cuda(kiss_fftndr_cuda_cfg cfg, const kiss_fft_scalar *timedata, kiss_fft_cpx *freqdata);
/* kiss_fftndri, kiss_fftndr.h:40 (kiss_fftndr.c:112-132) */
void kiss_fftndri_cuda(kiss_fftndr_cuda_cfg cfg, const kiss_fft_cpx *freqdata, kiss_fft_scalar *timedata);
/* kiss_fftndr_free, kiss_fftndr.h:49 */
void kiss_fftndr_cuda_free(void *cfg);

/* ---- real fast FIR: tools/kiss_fastfir.c (REAL_FASTFIR) -------------------
 * Float builds only, as in the reference ("won't work for fixed point",
 * tools/kiss_fastfir.c:152); other builds return NULL from the alloc. */
typedef struct kiss_fft_cuda_state *kiss_fastfir_cuda_cfg;

/* kiss_fastfir_alloc, tools/kiss_fastfir.c:36 (59-165): *nfft <= 0 picks the
 * block size, which is written back */
kiss_fastfir_cuda_cfg kiss_fastfir_cuda_alloc(const kiss_fft_scalar *imp_resp, size_t n_imp_resp, size_t *nfft,
                                              void *mem, size_t *lenmem);
/* kiss_fastfir, tools/kiss_fastfir.c:40 (222-239): filters *offset + n_new
 * samples of inbuf, returns the number of outputs written, moves the unused
 * tail to the front of inbuf and updates *offset; n_new == 0 flushes */
size_t kiss_fastfir_cuda(kiss_fastfir_cuda_cfg cfg, kiss_fft_scalar *inbuf, kiss_fft_scalar *outbuf, size_t n_new,
                         size_t *offset);
/* Whole signal in one call: the stream call plus its flush; writes
 * nx - n_imp_resp + 1 samples (the valid convolution) and returns that
 * count, or (size_t)-1 on error */
size_t kiss_fastfir_cuda_filter(kiss_fastfir_cuda_cfg cfg, const kiss_fft_scalar *x, size_t nx, kiss_fft_scalar *y);
void kiss_fastfir_cuda_free(void *cfg);

/* ---- execution control (no reference counterpart: the reference is a
 * synchronous CPU library) ---------------------------------------------- */
int kiss_fft_cuda_set_stream(void *cuda_stream);
int kiss_fft_cuda_sync(void);
const char *kiss_fft_cuda_last_error(void);
/* 0 if this thread's last kiss_*_cuda call succeeded, else a negative
 * status of kissfft_gb300.h (the void calls report failures only on stderr,
 * as the reference does) */
int kiss_fft_cuda_status(void);
/* Plan-specialised kernels (kissfft_gb300.h: kfg_set_specialize) and their
 * ahead-of-time preparation for a batch size (kfg_plan_prepare; batch is
 * the signal length for a fast FIR cfg). */
int kiss_fft_cuda_set_specialize(int on);
int kiss_fft_cuda_prepare(void *cfg, long long batch);
/* Autotune the launch shapes of batched calls of this size on cfg
 * (kissfft_gb300.h: kfg_autotune). */
int kiss_fft_cuda_autotune(void *cfg, long long batch);

#ifdef __cplusplus
}
#endif
#endif
