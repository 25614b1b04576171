// The drop-in C ABI of include/kiss_fft_cuda.h for one sample type.
// Compiled once per type (-DKF_DROPIN_DTYPE=0..3 with the matching
// FIXED_POINT / kiss_fft_scalar definition) into libkissfft_cuda-<type>.so,
// each a thin layer over the core library libkissfft_gb300.so.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <map>
#include <mutex>
#include <utility>

#include <cuda_runtime.h>

#include "kiss_fft_cuda.h"
#include "kissfft_gb300.h"

#ifndef KF_DROPIN_DTYPE
#error "KF_DROPIN_DTYPE must be defined"
#endif

namespace {

thread_local int t_status = 0;  // status of this thread's last drop-in call

const uint32_t kMagic = 0x4b464743u;  // "KFGC"
enum { H_C2C = 1, H_REAL = 2, H_ND = 3, H_NDR = 4, H_FIR = 5 };

}  // namespace

struct kiss_fft_cuda_state {
    uint32_t magic;
    int kind;
    int owned;  // 1: allocated by the library (freed by *_free)
    int inverse;
    long long n;      // nfft (1-D), product of dims (N-D), block size (FIR)
    long long ntaps;  // fast FIR
    long long ngood;
    kfg_plan* plan;
};

namespace {

// KISS_FFT_ERROR style report (kiss_fft_log.h:20-29)
void report(const char* where, const char* msg) {
    if (t_status == 0) t_status = KFG_EINVAL;
    fprintf(stderr, "[ERROR] %s: %s\n", where, msg);
}

void report_last(const char* where) { report(where, kfg_last_error()); }

// record a failing core status (report() alone defaults to KFG_EINVAL)
int note(int rc) {
    if (rc != KFG_OK) t_status = rc;
    return rc;
}

// The mem/lenmem protocol of kiss_fft_alloc (kiss_fft.h:94-115) for the host handle.
kiss_fft_cuda_state* place(void* mem, size_t* lenmem, bool* too_small) {
    const size_t need = sizeof(kiss_fft_cuda_state);
    *too_small = false;
    if (lenmem == nullptr) {
        kiss_fft_cuda_state* s = (kiss_fft_cuda_state*)calloc(1, need);
        if (s) s->owned = 1;
        return s;
    }
    kiss_fft_cuda_state* s = nullptr;
    if (mem != nullptr && *lenmem >= need) {
        s = (kiss_fft_cuda_state*)mem;
        memset(s, 0, need);
        s->owned = 0;
    } else {
        *too_small = true;
    }
    *lenmem = need;
    return s;
}

kiss_fft_cuda_state* finish(kiss_fft_cuda_state* s, kfg_plan* plan, int kind, int inverse, long long n) {
    if (!plan) {
        report_last("kiss_fft_cuda alloc");
        if (s->owned) free(s);
        return nullptr;
    }
    s->magic = kMagic;
    s->kind = kind;
    s->inverse = inverse ? 1 : 0;
    s->n = n;
    s->plan = plan;
    return s;
}

bool check(const kiss_fft_cuda_state* s, int kind, const char* where) {
    if (!s || s->magic != kMagic || !s->plan) {
        report(where, "invalid cfg");
        return false;
    }
    if (s->kind != kind) {
        report(where, "kiss fft usage error: improper alloc");
        return false;
    }
    return true;
}

void free_state(void* p) {
    kiss_fft_cuda_state* s = (kiss_fft_cuda_state*)p;
    if (!s || s->magic != kMagic) return;
    kfg_plan_free(s->plan);
    s->plan = nullptr;
    s->magic = 0;
    if (s->owned) free(s);
}

bool is_device(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

extern "C" {

kiss_fft_cuda_cfg kiss_fft_cuda_alloc(int nfft, int inverse_fft, void* mem, size_t* lenmem) {
    t_status = 0;
    bool small;
    if (nfft < 1) return nullptr;
    kiss_fft_cuda_state* s = place(mem, lenmem, &small);
    if (!s) return nullptr;
    return finish(s, kfg_plan_c2c(KF_DROPIN_DTYPE, nfft, inverse_fft), H_C2C, inverse_fft, nfft);
}

void kiss_fft_cuda_stride(kiss_fft_cuda_cfg cfg, const kiss_fft_cpx* fin, kiss_fft_cpx* fout, int fin_stride) {
    t_status = 0;
    if (!check(cfg, H_C2C, "kiss_fft_cuda_stride")) return;
    if (fout == nullptr) {
        report("kiss_fft_cuda_stride", "fout buffer NULL.");
        return;
    }
    if (note(kfg_exec_stride(cfg->plan, fin, fout, fin_stride, nullptr)) != KFG_OK) report_last("kiss_fft_cuda_stride");
}

void kiss_fft_cuda(kiss_fft_cuda_cfg cfg, const kiss_fft_cpx* fin, kiss_fft_cpx* fout) {
    t_status = 0;
    kiss_fft_cuda_stride(cfg, fin, fout, 1);
}

int kiss_fft_cuda_batch(kiss_fft_cuda_cfg cfg, const kiss_fft_cpx* fin, kiss_fft_cpx* fout, long long batch,
                        long long in_dist, long long out_dist) {
    t_status = 0;
    if (!check(cfg, H_C2C, "kiss_fft_cuda_batch")) return KFG_EINVAL;
    int rc = note(kfg_exec_batch(cfg->plan, fin, fout, batch, in_dist, out_dist, nullptr));
    if (rc != KFG_OK) report_last("kiss_fft_cuda_batch");
    return rc;
}

void kiss_fft_cuda_free(void* cfg) { free_state(cfg); }
void kiss_fftr_cuda_free(void* cfg) { free_state(cfg); }
void kiss_fftnd_cuda_free(void* cfg) { free_state(cfg); }
void kiss_fftndr_cuda_free(void* cfg) { free_state(cfg); }
void kiss_fastfir_cuda_free(void* cfg) { free_state(cfg); }

void kiss_fft_cuda_cleanup(void) {}

int kiss_fft_cuda_next_fast_size(int n) { return kfg_next_fast_size(n); }

}  // extern "C"

namespace {

// The kfc cache of this sample type's library: (nfft, inverse) -> device
// plan, like find_cached_fft (kfc.c:24-61) but under a mutex.
std::mutex g_kfc_mu;
std::map<std::pair<int, int>, kfg_plan*> g_kfc;

void kfc_run(int nfft, int inverse, const kiss_fft_cpx* fin, kiss_fft_cpx* fout, const char* where) {
    t_status = 0;
    if (nfft < 1 || !fin || !fout) {
        report(where, "bad arguments");
        return;
    }
    kfg_plan* p = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_kfc_mu);
        auto it = g_kfc.find(std::make_pair(nfft, inverse));
        if (it != g_kfc.end()) {
            p = it->second;
        } else {
            p = kfg_plan_c2c(KF_DROPIN_DTYPE, nfft, inverse);
            if (p) g_kfc[std::make_pair(nfft, inverse)] = p;
        }
    }
    if (!p) {
        t_status = KFG_ECUDA;
        report_last(where);
        return;
    }
    if (note(kfg_exec(p, fin, fout, nullptr)) != KFG_OK) report_last(where);
}

}  // namespace

extern "C" {

void kfc_cuda_fft(int nfft, const kiss_fft_cpx* fin, kiss_fft_cpx* fout) {
    kfc_run(nfft, 0, fin, fout, "kfc_cuda_fft");
}

void kfc_cuda_ifft(int nfft, const kiss_fft_cpx* fin, kiss_fft_cpx* fout) {
    kfc_run(nfft, 1, fin, fout, "kfc_cuda_ifft");
}

void kfc_cuda_cleanup(void) {
    std::lock_guard<std::mutex> lk(g_kfc_mu);
    if (g_kfc.empty()) return;
    // transforms enqueued on device buffers may still read the plans
    kfg_synchronize();
    for (auto& kv : g_kfc) kfg_plan_free(kv.second);
    g_kfc.clear();
}

int kfc_cuda_ncached(void) {
    std::lock_guard<std::mutex> lk(g_kfc_mu);
    return (int)g_kfc.size();
}

kiss_fftr_cuda_cfg kiss_fftr_cuda_alloc(int nfft, int inverse_fft, void* mem, size_t* lenmem) {
    t_status = 0;
    if (nfft & 1) {
        report("kiss_fftr_cuda_alloc", "Real FFT optimization must be even.");
        return nullptr;
    }
    bool small;
    kiss_fft_cuda_state* s = place(mem, lenmem, &small);
    if (!s) return nullptr;
    return finish(s, kfg_plan_real(KF_DROPIN_DTYPE, nfft, inverse_fft), H_REAL, inverse_fft, nfft);
}

void kiss_fftr_cuda(kiss_fftr_cuda_cfg cfg, const kiss_fft_scalar* timedata, kiss_fft_cpx* freqdata) {
    t_status = 0;
    if (!check(cfg, H_REAL, "kiss_fftr_cuda")) return;
    if (cfg->inverse) {
        report("kiss_fftr_cuda", "kiss fft usage error: improper alloc");
        return;
    }
    if (note(kfg_exec(cfg->plan, timedata, freqdata, nullptr)) != KFG_OK) report_last("kiss_fftr_cuda");
}

void kiss_fftri_cuda(kiss_fftr_cuda_cfg cfg, const kiss_fft_cpx* freqdata, kiss_fft_scalar* timedata) {
    t_status = 0;
    if (!check(cfg, H_REAL, "kiss_fftri_cuda")) return;
    if (!cfg->inverse) {
        report("kiss_fftri_cuda", "kiss fft usage error: improper alloc");
        return;
    }
    if (note(kfg_exec(cfg->plan, freqdata, timedata, nullptr)) != KFG_OK) report_last("kiss_fftri_cuda");
}

int kiss_fftr_cuda_batch(kiss_fftr_cuda_cfg cfg, const kiss_fft_scalar* timedata, kiss_fft_cpx* freqdata,
                         long long batch, long long in_dist, long long out_dist) {
    t_status = 0;
    if (!check(cfg, H_REAL, "kiss_fftr_cuda_batch")) return KFG_EINVAL;
    if (cfg->inverse) {
        report("kiss_fftr_cuda_batch", "kiss fft usage error: improper alloc");
        return KFG_EINVAL;
    }
    int rc = note(kfg_exec_batch(cfg->plan, timedata, freqdata, batch, in_dist, out_dist, nullptr));
    if (rc != KFG_OK) report_last("kiss_fftr_cuda_batch");
    return rc;
}

int kiss_fftri_cuda_batch(kiss_fftr_cuda_cfg cfg, const kiss_fft_cpx* freqdata, kiss_fft_scalar* timedata,
                          long long batch, long long in_dist, long long out_dist) {
    t_status = 0;
    if (!check(cfg, H_REAL, "kiss_fftri_cuda_batch")) return KFG_EINVAL;
    if (!cfg->inverse) {
        report("kiss_fftri_cuda_batch", "kiss fft usage error: improper alloc");
        return KFG_EINVAL;
    }
    int rc = note(kfg_exec_batch(cfg->plan, freqdata, timedata, batch, in_dist, out_dist, nullptr));
    if (rc != KFG_OK) report_last("kiss_fftri_cuda_batch");
    return rc;
}

kiss_fftnd_cuda_cfg kiss_fftnd_cuda_alloc(const int* dims, int ndims, int inverse_fft, void* mem, size_t* lenmem) {
    t_status = 0;
    bool small;
    if (!dims || ndims < 1) return nullptr;
    kiss_fft_cuda_state* s = place(mem, lenmem, &small);
    if (!s) return nullptr;
    long long n = 1;
    for (int i = 0; i < ndims; ++i) n *= dims[i];
    return finish(s, kfg_plan_nd(KF_DROPIN_DTYPE, dims, ndims, inverse_fft), H_ND, inverse_fft, n);
}

void kiss_fftnd_cuda(kiss_fftnd_cuda_cfg cfg, const kiss_fft_cpx* fin, kiss_fft_cpx* fout) {
    t_status = 0;
    if (!check(cfg, H_ND, "kiss_fftnd_cuda")) return;
    if (note(kfg_exec(cfg->plan, fin, fout, nullptr)) != KFG_OK) report_last("kiss_fftnd_cuda");
}

kiss_fftndr_cuda_cfg kiss_fftndr_cuda_alloc(const int* dims, int ndims, int inverse_fft, void* mem, size_t* lenmem) {
    t_status = 0;
    if (!dims || ndims < 1) return nullptr;
    if (dims[ndims - 1] & 1) {
        report("kiss_fftndr_cuda_alloc", "Real FFT optimization must be even.");
        return nullptr;
    }
    bool small;
    kiss_fft_cuda_state* s = place(mem, lenmem, &small);
    if (!s) return nullptr;
    long long n = 1;
    for (int i = 0; i < ndims; ++i) n *= dims[i];
    return finish(s, kfg_plan_ndr(KF_DROPIN_DTYPE, dims, ndims, inverse_fft), H_NDR, inverse_fft, n);
}

void kiss_fftndr_cuda(kiss_fftndr_cuda_cfg cfg, const kiss_fft_scalar* timedata, kiss_fft_cpx* freqdata) {
    t_status = 0;
    if (!check(cfg, H_NDR, "kiss_fftndr_cuda")) return;
    if (cfg->inverse) {
        report("kiss_fftndr_cuda", "kiss fft usage error: improper alloc");
        return;
    }
    if (note(kfg_exec(cfg->plan, timedata, freqdata, nullptr)) != KFG_OK) report_last("kiss_fftndr_cuda");
}

void kiss_fftndri_cuda(kiss_fftndr_cuda_cfg cfg, const kiss_fft_cpx* freqdata, kiss_fft_scalar* timedata) {
    t_status = 0;
    if (!check(cfg, H_NDR, "kiss_fftndri_cuda")) return;
    if (!cfg->inverse) {
        report("kiss_fftndri_cuda", "kiss fft usage error: improper alloc");
        return;
    }
    if (note(kfg_exec(cfg->plan, freqdata, timedata, nullptr)) != KFG_OK) report_last("kiss_fftndri_cuda");
}

kiss_fastfir_cuda_cfg kiss_fastfir_cuda_alloc(const kiss_fft_scalar* imp_resp, size_t n_imp_resp, size_t* nfft,
                                              void* mem, size_t* lenmem) {
#if KF_DROPIN_DTYPE != KFG_FLOAT
    (void)imp_resp;
    (void)n_imp_resp;
    (void)nfft;
    (void)mem;
    (void)lenmem;
    report("kiss_fastfir_cuda_alloc", "the fast FIR is built for float samples only");
    return nullptr;
#else
    if (!imp_resp || n_imp_resp < 1) return nullptr;
    bool small;
    kiss_fft_cuda_state* s = place(mem, lenmem, &small);
    if (!s) return nullptr;
    size_t want = nfft ? *nfft : 0, got = 0;
    kfg_plan* plan = kfg_plan_fir(imp_resp, n_imp_resp, want, &got);
    if (nfft) *nfft = got;
    kiss_fft_cuda_state* r = finish(s, plan, H_FIR, 0, (long long)got);
    if (r) {
        r->ntaps = (long long)n_imp_resp;
        r->ngood = (long long)got - (long long)n_imp_resp + 1;
    }
    return r;
#endif
}

size_t kiss_fastfir_cuda_filter(kiss_fastfir_cuda_cfg cfg, const kiss_fft_scalar* x, size_t nx, kiss_fft_scalar* y) {
    t_status = 0;
    if (!check(cfg, H_FIR, "kiss_fastfir_cuda_filter")) return (size_t)-1;
    size_t ny = 0;
    if (note(kfg_fir_filter(cfg->plan, (const float*)x, nx, (float*)y, &ny, nullptr)) != KFG_OK) {
        report_last("kiss_fastfir_cuda_filter");
        return (size_t)-1;
    }
    return ny;
}

size_t kiss_fastfir_cuda(kiss_fastfir_cuda_cfg cfg, kiss_fft_scalar* inbuf, kiss_fft_scalar* outbuf, size_t n_new,
                         size_t* offset) {
    t_status = 0;
    if (!check(cfg, H_FIR, "kiss_fastfir_cuda")) return 0;
    if (!offset) {
        report("kiss_fastfir_cuda", "offset pointer NULL.");
        return 0;
    }
    const size_t ntot = n_new + *offset;
    const long long nfft = cfg->n, ngood = cfg->ngood, L = cfg->ntaps;
    if (n_new == 0) {
        // flush (kff_flush, tools/kiss_fastfir.c:202-220): the remaining
        // samples, zero padded, give ntot - L + 1 outputs
        if ((long long)ntot < L - 1) return 0;
        size_t ny = 0;
        if (note(kfg_fir_filter(cfg->plan, (const float*)inbuf, ntot, (float*)outbuf, &ny, nullptr)) != KFG_OK) {
            report_last("kiss_fastfir_cuda");
            return 0;
        }
        return ny;
    }
    // full blocks only (kff_nocopy, tools/kiss_fastfir.c:186-200)
    long long nfull = (long long)ntot >= nfft ? ((long long)ntot - nfft) / ngood + 1 : 0;
    const size_t nwritten = (size_t)(nfull * ngood);
    if (nfull > 0) {
        size_t ny = 0;
        if (note(kfg_fir_filter(cfg->plan, (const float*)inbuf, nwritten + (size_t)L - 1, (float*)outbuf, &ny,
                                nullptr)) != KFG_OK) {
            report_last("kiss_fastfir_cuda");
            return 0;
        }
    }
    // keep the unused tail at the front of inbuf (tools/kiss_fastfir.c:234-236)
    const size_t keep = ntot - nwritten;
    if (nwritten > 0 && keep > 0) {
        if (is_device(inbuf)) {
            // through a temporary: the kept tail may overlap the front
            void* tmp = nullptr;
            cudaStream_t st = (cudaStream_t)kfg_get_stream();
            bool ok = cudaMallocAsync(&tmp, keep * sizeof(kiss_fft_scalar), st) == cudaSuccess;
            ok = ok && cudaMemcpyAsync(tmp, inbuf + nwritten, keep * sizeof(kiss_fft_scalar), cudaMemcpyDeviceToDevice,
                                       st) == cudaSuccess;
            ok = ok && cudaMemcpyAsync(inbuf, tmp, keep * sizeof(kiss_fft_scalar), cudaMemcpyDeviceToDevice, st) ==
                           cudaSuccess;
            if (tmp) cudaFreeAsync(tmp, st);
            if (!ok) {
                t_status = KFG_ECUDA;
                report("kiss_fastfir_cuda", "device copy of the kept samples failed");
                return 0;
            }
        } else {
            memmove(inbuf, inbuf + nwritten, keep * sizeof(kiss_fft_scalar));
        }
    }
    *offset = keep;
    return nwritten;
}

int kiss_fft_cuda_set_stream(void* cuda_stream) { return kfg_set_stream(cuda_stream); }

int kiss_fft_cuda_sync(void) { return kfg_synchronize(); }

const char* kiss_fft_cuda_last_error(void) { return kfg_last_error(); }

int kiss_fft_cuda_status(void) { return t_status; }

int kiss_fft_cuda_set_specialize(int on) { return kfg_set_specialize(on); }

int kiss_fft_cuda_autotune(void* cfg, long long batch) {
    t_status = 0;
    kiss_fft_cuda_state* s = (kiss_fft_cuda_state*)cfg;
    if (!s || s->magic != kMagic || !s->plan) {
        report("kiss_fft_cuda_autotune", "invalid cfg");
        return KFG_EINVAL;
    }
    int rc = note(kfg_autotune(s->plan, batch, 0, 0));
    if (rc != KFG_OK) report_last("kiss_fft_cuda_autotune");
    return rc;
}

int kiss_fft_cuda_prepare(void* cfg, long long batch) {
    t_status = 0;
    kiss_fft_cuda_state* s = (kiss_fft_cuda_state*)cfg;
    if (!s || s->magic != kMagic || !s->plan) {
        report("kiss_fft_cuda_prepare", "invalid cfg");
        return KFG_EINVAL;
    }
    int rc = note(kfg_plan_prepare(s->plan, batch, 0, 0));
    if (rc != KFG_OK) report_last("kiss_fft_cuda_prepare");
    return rc;
}

}  // extern "C"
