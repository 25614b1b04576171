/*
 * kissfft_gb300 core C API -- GPU KISS FFT plans with the sample type as a
 * run-time tag.
 *
 * This is the layer under the per-type drop-in libraries (kiss_fft_cuda.h):
 * it exposes batched execution, explicit streams and the fast FIR.  The
 * transform calls map onto the reference (mborgerding/kissfft) like this:
 *
 *   kfg_plan_c2c   kiss_fft_alloc      (kiss_fft.h:117,   kiss_fft.c:337-372)
 *   kfg_plan_real  kiss_fftr_alloc     (kiss_fftr.h:29,   kiss_fftr.c:21-61)
 *   kfg_plan_nd    kiss_fftnd_alloc    (kiss_fftnd.h:20,  kiss_fftnd.c:20-92)
 *   kfg_plan_ndr   kiss_fftndr_alloc   (kiss_fftndr.h:23, kiss_fftndr.c:30-84)
 *   kfg_plan_fir   kiss_fastfir_alloc  (tools/kiss_fastfir.c:59-165, REAL_FASTFIR)
 *   kfg_exec       kiss_fft / kiss_fftr / kiss_fftri / kiss_fftnd / kiss_fftndr /
 *                  kiss_fftndri        (one transform per call)
 *   kfg_exec_stride kiss_fft_stride    (kiss_fft.h:134)
 *   kfg_exec_batch  a loop of the above over `batch` transforms, in one launch
 *   kfg_fir_filter  kiss_fastfir over a whole signal plus its flush call
 *                  (tools/kiss_fastfir.c:222-239)
 *   kfg_next_fast_size kiss_fft_next_fast_size (kiss_fft.h:150)
 *
 * Data layout is the reference's: interleaved {r, i} pairs of the sample
 * type (kiss_fft.h:87-90); real transforms take n reals and give n/2+1
 * bins; N-D arrays are row-major; N-D-real halves the last axis.
 * Normalisation is the reference's: none for float/double, 1/N per
 * direction for Q15/Q31 (fixed-point outputs are bit-identical to the
 * reference's fixed-point builds).
 *
 * Pointers may be device pointers (the fast path: the call is enqueued on
 * the stream and returns) or host pointers (staged through device memory;
 * the call returns when the result is in host memory).  There is no CPU
 * fallback: without a usable GPU every call fails with KFG_ECUDA.
 */
#ifndef KISSFFT_GB300_H
#define KISSFFT_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define KFG_FLOAT 0  /* kiss_fft_scalar = float   */
#define KFG_DOUBLE 1 /* kiss_fft_scalar = double  */
#define KFG_INT16 2  /* FIXED_POINT=16 (Q15)      */
#define KFG_INT32 3  /* FIXED_POINT=32 (Q31)      */

#define KFG_OK 0
#define KFG_EINVAL (-1)       /* bad argument or unsupported size           */
#define KFG_ENOMEM (-2)       /* device or host allocation failed           */
#define KFG_ECUDA (-3)        /* a CUDA call failed (no GPU, launch error)  */
#define KFG_EUNSUPPORTED (-4) /* valid in the reference, not built here      */

typedef struct kfg_plan kfg_plan;

kfg_plan *kfg_plan_c2c(int dtype, int nfft, int inverse);
kfg_plan *kfg_plan_real(int dtype, int nfft, int inverse);
kfg_plan *kfg_plan_nd(int dtype, const int *dims, int ndims, int inverse);
kfg_plan *kfg_plan_ndr(int dtype, const int *dims, int ndims, int inverse);
/* Real fast FIR (float).  taps: host array of ntaps floats.  nfft = 0 picks
 * the reference's block size (next power of two above 2*(ntaps-1), at least
 * 2048); the chosen size is returned through *nfft_out when non-null. */
kfg_plan *kfg_plan_fir(const float *taps, size_t ntaps, size_t nfft, size_t *nfft_out);
void kfg_plan_free(kfg_plan *p);

/* stream: a cudaStream_t, or NULL for the library's current stream. */
int kfg_exec(kfg_plan *p, const void *in, void *out, void *stream);
int kfg_exec_stride(kfg_plan *p, const void *in, void *out, int in_stride, void *stream);
/* in_dist / out_dist: element distance between consecutive transforms of the
 * batch (complex elements or real samples, as the side holds); 0 = packed. */
int kfg_exec_batch(kfg_plan *p, const void *in, void *out, long long batch, long long in_dist, long long out_dist,
                   void *stream);
/* kfg_exec_batch for callers that may not allocate device memory while they
 * transform (code inside a custom allocator or memory-pool hook, real-time
 * loops with memory fixed at start-up).  It has no counterpart in the
 * reference, whose transforms run on the host.  Complex 1-D plans and device
 * pointers only.  Scratch of two-pass plans (batch * nfft complex elements)
 * comes from one fixed device array per device of KFG_NOALLOC_SCRATCH_BYTES;
 * a larger batch fails with KFG_EINVAL.  The stream and both buffers must be
 * on the current device (the array used is the current device's); a stream
 * or buffer of another device fails with KFG_EINVAL.  Calls that may overlap
 * on the GPU (other streams or threads) race on that array: issue them on
 * one stream.  The first call in a context looks the array up (and may load
 * the module holding it, which reserves the array's bytes): make it before
 * any stream capture.  The address is kept per context, so calls after a
 * device reset look it up again.  Run-time specialised kernels are not
 * used. */
#define KFG_NOALLOC_SCRATCH_BYTES ((size_t)64 << 20)
int kfg_exec_batch_noalloc(kfg_plan *p, const void *in, void *out, long long batch, long long in_dist,
                           long long out_dist, void *stream);
/* Whole-signal filter: y receives nx - ntaps + 1 samples (the valid
 * convolution); *ny_out gets that count. */
int kfg_fir_filter(kfg_plan *p, const float *x, size_t nx, float *y, size_t *ny_out, void *stream);

/* The packing step of the C++ facade's transform_real (kissfft.hh:154-189):
 * bins[0..n] of a 2n-point real transform (device, float or double) ->
 * dst[0] = (X0, Xn), dst[k] = X[k] (conj != 0: conj(X[k])), k = 1..n-1. */
int kfg_pack_real(int dtype, const void *bins, void *dst, long long n, int conj, void *stream);

/* Power spectrogram of tools/psdpng.c (transform_signal, psdpng.c:116-175;
 * the PNG output is not part of this library): 16-bit samples (stereo != 0:
 * interleaved pairs, summed), frames of nfft with their mean removed when
 * remove_dc != 0, a real forward FFT per frame, and per row of navg frames
 * rows[r][k] = 10*log10(sum |X[k]|^2 / navg + 1), k = 0..nfft/2.  p: a float
 * forward real plan of nfft.  nsamples counts samples per channel; only
 * whole rows are produced (*nrows_out gets their number).  Buffers may be
 * host or device memory. */
int kfg_psd(kfg_plan *p, const short *samples, long long nsamples, int stereo, int remove_dc, int navg, float *rows,
            long long *nrows_out, void *stream);

int kfg_set_stream(void *stream);
void *kfg_get_stream(void);
int kfg_synchronize(void);
const char *kfg_last_error(void);
int kfg_next_fast_size(int n);

/* Plan-specialised kernels.  With specialisation on, every launch uses a
 * kernel compiled for its exact plan shape (all strides and radices
 * constant), compiled at run time with NVRTC on first use and cached on
 * disk (KISSFFT_GB300_CACHE); without it the precompiled kernels that read
 * the shape at run time are used.  Default off; KISSFFT_GB300_SPECIALIZE=1
 * turns it on. */
int kfg_set_specialize(int on);
/* TMA staging of contiguous tiles (bulk copy of the next tile's input into
 * shared memory while the current tile computes).  Default on;
 * KISSFFT_GB300_TMA=0 turns it off. */
int kfg_set_tma(int on);
/* Compile (or load) the specialised kernels a batched call of this shape
 * will use, so that the compile cost is paid here.  For a fast FIR plan,
 * batch is the signal length. */
int kfg_plan_prepare(kfg_plan *p, long long batch, long long in_dist, long long out_dist);
/* Autotuner: for each launch of a batched call of this shape, time the
 * candidate tile shapes (jobs per tile, register budget, TMA staging on or
 * off) on scratch buffers and keep the fastest for later calls with the
 * same (batch, in_dist, out_dist).  Results persist in the cache
 * directory (tune.txt), keyed by plan, shape and GPU. */
int kfg_autotune(kfg_plan *p, long long batch, long long in_dist, long long out_dist);
/* Compile, without loading or a GPU, the specialised kernels of a complex
 * (real = 0) or real (real = 1) plan: a check of the embedded sources. */
int kfg_specialize_check(int dtype, int real, int n, int inverse, long long batch);

/* Device plan cache (the reference's kfc.c: kfc_fft/kfc_ifft keep plans
 * keyed by size and direction): a shared plan per (real, dtype, n,
 * inverse), kept until kfg_cache_clear.  Thread-safe. */
kfg_plan *kfg_plan_cached(int real, int dtype, int n, int inverse);
int kfg_cache_clear(void);

/* Batched uneven mix: transforms of different sizes, sample types and kinds
 * in one submission.  Each request reads at in_off and writes at out_off
 * (bytes, element aligned) of two device arenas given at commit.  Requests
 * are grouped per plan and run as persistent work-queue launches (one per
 * sample type, kind and pass), optionally replayed from a CUDA graph. */
#define KFG_KIND_C2C 1 /* kiss_fft   */
#define KFG_KIND_R2C 2 /* kiss_fftr  */
#define KFG_KIND_C2R 3 /* kiss_fftri */
typedef struct kfg_batch kfg_batch;
kfg_batch *kfg_batch_create(void);
int kfg_batch_add(kfg_batch *b, int kind, int dtype, int n, long long in_off, long long out_off);
/* target_threads: threads per CTA the tiles are widened towards (0 = 256) */
int kfg_batch_commit(kfg_batch *b, void *in_arena, void *out_arena, int target_threads);
int kfg_batch_run(kfg_batch *b, void *stream);
/* capture one run into a CUDA graph; later kfg_batch_run calls replay it */
int kfg_batch_capture(kfg_batch *b, void *stream);
/* the plain per-call form of the same work: one drop-in call per request */
int kfg_batch_run_percall(kfg_batch *b, void *stream);
/* out[0] requests, out[1] launch steps, out[2] kernel launches, out[3] tiles,
 * out[4] bytes of intermediate traffic: requests longer than one shared tile
 * write their intermediate results to device scratch and read them back */
int kfg_batch_info(const kfg_batch *b, long long *out, int nout);
void kfg_batch_free(kfg_batch *b);

/* Serving loop (the served form of the path): requests submitted from any
 * host thread are admitted in arrival order under an HBM budget, batched
 * continuously (everything admitted since the last launch goes out together,
 * up to KFG_SERVE_SLOTS batches in flight on their own streams), and
 * completed asynchronously.  Plans and fast-FIR responses stay cached on the
 * device; their bytes count against the budget and the least recently used
 * plan no request holds is evicted when the budget runs out.  Buffers may be device, pinned host (moved by one zero-copy
 * gather/scatter kernel per batch) or ordinary host memory, and must stay
 * valid until the request is waited for.  Latency = completion - submit. */
#define KFG_SERVE_C2C 1    /* kiss_fft:   n0 points, dtype, inverse        */
#define KFG_SERVE_R2C 2    /* kiss_fftr:  n0 reals -> n0/2+1 bins          */
#define KFG_SERVE_C2R 3    /* kiss_fftri: n0/2+1 bins -> n0 reals          */
#define KFG_SERVE_C2C_2D 4 /* kiss_fftnd: n0 x n1 complex, row-major       */
#define KFG_SERVE_FIR 5    /* kiss_fastfir: n0 float taps, len samples in,
                              len - n0 + 1 samples out (valid part)       */
#define KFG_SERVE_SLOTS 8
typedef struct {
    int kind, dtype, inverse;
    int n0, n1;
    long long len;
    const float *taps;
    const void *in;
    void *out;
} kfg_serve_req;
typedef struct {
    long long completed, failed, batches, max_batch, peak_hbm_bytes;
    double p50_s, p99_s, max_s, mean_s; /* latency, submit to completion */
    double req_per_s, gbs, bytes;       /* over first submit .. last completion */
    double host_s;                      /* host time spent describing and launching batches */
    long long plans, plan_bytes, evictions; /* device plan cache: entries, bytes, LRU evictions */
} kfg_serve_stats;
typedef struct kfg_server kfg_server;
/* hbm_budget: bytes (0 = 40 GiB); slots: batches in flight (0 = 4) */
kfg_server *kfg_server_create(size_t hbm_budget, int slots);
/* returns a request id > 0, or a negative KFG_E* code */
long long kfg_server_submit(kfg_server *s, const kfg_serve_req *req);
/* timeout_s < 0 waits without limit; returns the request's status, or 1 on
 * timeout (the request stays pending and may be waited for again) */
int kfg_server_wait(kfg_server *s, long long id, double timeout_s, double *latency_s);
int kfg_server_drain(kfg_server *s); /* waits for every submitted request */
int kfg_server_stats(kfg_server *s, kfg_serve_stats *out);
int kfg_server_reset_stats(kfg_server *s);
void kfg_server_free(kfg_server *s);

/* Synthetic load for the serving loop: Poisson arrivals at `rate` requests/s
 * for `seconds` (rate <= 0: `count` requests submitted at once), kinds drawn
 * with weights mix[] = {c2c, r2c, 2-D, fast FIR} (float), c2c/r2c lengths
 * log-uniform [c2c_min, c2c_max] moved to the next fast size, 2-D sides
 * log-uniform [d2_min, d2_max], FIR taps log-uniform [fir_taps_min,
 * fir_taps_max] N(0,1) (16 filters) on signals of log-uniform
 * [fir_len_min, fir_len_max] samples.  Inputs are N(0,1) in a pinned pool.
 * Then the first percall_max requests run again through the plain per-call
 * form (one synchronous kfg_exec / kfg_fir_filter each). */
typedef struct {
    double rate, seconds;
    long long count;
    unsigned long long seed;
    double mix[4];
    int c2c_min, c2c_max, d2_min, d2_max, fir_taps_min, fir_taps_max;
    long long fir_len_min, fir_len_max;
    long long percall_max;
    int in_pool_mb, out_pool_mb;
} kfg_loadtest;
typedef struct {
    long long offered;
    double submit_s;
    kfg_serve_stats served;
    long long percall_count;
    double percall_req_per_s, percall_gbs, percall_p50_s, percall_p99_s;
} kfg_loadtest_result;
int kfg_server_loadtest(kfg_server *s, const kfg_loadtest *cfg, kfg_loadtest_result *res);

/* Plan introspection for tests and tools: out[0] = transform kind, out[1] =
 * dtype, out[2] = length, out[3] = number of HBM passes of a 1-D plan,
 * out[4] = kernel family, out[5] = tile length. */
int kfg_plan_info(const kfg_plan *p, int *out, int nout);
/* Reads a table back from a plan's device memory (the bytes the kernels
 * use), for tests that compare it with the reference's: which = 0, the full
 * twiddle table of a complex plan (nfft entries of the sample type,
 * kiss_fft.c:361-367; for a real plan, that of its nfft/2-point complex
 * sub-transform), which = 1, the super twiddles of a real plan (nfft/4
 * entries, kiss_fftr.c:53-59).  Returns the table's byte count and copies
 * min(bytes, count) bytes to host when host != NULL; a negative KFG_E*
 * code on error. */
long long kfg_plan_table(const kfg_plan *p, int which, void *host, size_t bytes);

#ifdef __cplusplus
}
#endif
#endif
