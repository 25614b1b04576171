// CUDA kernels for sm_103a: the engine kernel (one tile of jobs per CTA
// iteration) and the element kernels of two-pass real plans.
#pragma once
#include <cuda_runtime.h>

#include "kf_device.cuh"
#include "kf_plan.h"

#include <atomic>
#include <cstdlib>
#include <string>

namespace kf {

// Identity of the calling thread's current CUDA context (cuCtxGetId; 0 when
// the thread has none).  State that belongs to a context -- kernel
// attributes, the address of a __device__ array -- is cached per context
// and set up again when the id changes (after cudaDeviceReset or a reset
// of the primary context the runtime creates a new context with a new id).
unsigned long long current_context_id();

// Grid of a launch: one CTA per tile, or -- for TMA-staged steps, which
// loop over tiles -- as many CTAs as fit on the GPU at once.
inline long long launch_grid(const void* k, const Step& st) {
    long long grid = st.cfg.grid;
    if (st.args.tma) {
        static const int nsm = [] {
            int dev = 0, n = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
            return n > 0 ? n : 1;
        }();
        // occupancy of the last (kernel, threads, shared memory) this thread asked for
        thread_local const void* ck = nullptr;
        thread_local int cT = 0, cS = 0, cper = 1;
        if (k != ck || st.cfg.T != cT || st.cfg.smem != cS) {
            int per = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, st.cfg.T, (size_t)st.cfg.smem) != cudaSuccess ||
                per <= 0)
                per = 1;
            ck = k;
            cT = st.cfg.T;
            cS = st.cfg.smem;
            cper = per;
        }
        const int per = cper;
        const long long cap = (long long)per * nsm;
        if (grid > cap) grid = cap;
    }
    if (grid > 0x7fffffffLL) grid = 0x7fffffffLL;
    return grid;
}

// Engine launches carry the programmatic-stream-serialization attribute
// (the kernels wait for the previous kernel on entry, kf_pdl_enter), so the
// next launch of a schedule overlaps the tail of the one before it.
// KISSFFT_GB300_PDL=0 launches them plainly.
inline bool pdl_enabled() {
    static const bool on = [] {
        const char* e = getenv("KISSFFT_GB300_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}

inline cudaError_t launch_engine_raw(const void* k, long long grid, const Step& st, void** args, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)st.cfg.T);
    cfg.dynamicSmemBytes = (size_t)st.cfg.smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1] = {};
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl_enabled() ? 1 : 0;
    return cudaLaunchKernelExC(&cfg, k, args);
}

template <typename S, int MODE, int FAM>
static cudaError_t launch_engine_f(const Step& st, cudaStream_t s) {
    auto k = kf_engine_kernel<S, MODE, FAM>;
    static std::atomic<unsigned long long> attr_ctx{0};
    const unsigned long long ctx = current_context_id();
    if (ctx == 0 || attr_ctx.load() != ctx) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e != cudaSuccess) return e;
        attr_ctx.store(current_context_id());
    }
    const long long grid = launch_grid((const void*)k, st);
    if (grid <= 0) return cudaSuccess;
    void* args[] = {(void*)&st.args};
    return launch_engine_raw((const void*)k, grid, st, args, s);
}

template <typename S>
static cudaError_t launch_elem(const Step& st, cudaStream_t s) {
    long long grid = st.cfg.grid;
    if (grid > 0x7fffffffLL) grid = 0x7fffffffLL;
    if (grid <= 0) return cudaSuccess;
    if (st.kind == 1)
        kf_split_kernel<S><<<(unsigned)grid, 256, 0, s>>>(st.args);
    else
        kf_merge_kernel<S><<<(unsigned)grid, 256, 0, s>>>(st.args);
    return cudaGetLastError();
}

// Entry points of the per-(type, family) translation units (kf_inst.cu).
#define KF_DECL_DT(D)                                                   \
    cudaError_t launch_engine_dt##D##_fam0(const Step&, cudaStream_t); \
    cudaError_t launch_engine_dt##D##_fam1(const Step&, cudaStream_t); \
    cudaError_t launch_engine_dt##D##_fam2(const Step&, cudaStream_t); \
    cudaError_t launch_elem_dt##D(const Step&, cudaStream_t);           \
    cudaError_t launch_multi_elem_dt##D(int, const MultiArgs&, cudaStream_t);
KF_DECL_DT(0)
KF_DECL_DT(1)
KF_DECL_DT(2)
KF_DECL_DT(3)
#undef KF_DECL_DT
#define KF_DECL_MULTI(D)                                                                                   \
    cudaError_t launch_multi_dt##D##_fam0(int, const MultiArgs&, int, int, long long, cudaStream_t);       \
    cudaError_t launch_multi_dt##D##_fam1(int, const MultiArgs&, int, int, long long, cudaStream_t);       \
    cudaError_t launch_multi_dt##D##_fam2(int, const MultiArgs&, int, int, long long, cudaStream_t);
KF_DECL_MULTI(0)
KF_DECL_MULTI(1)
KF_DECL_MULTI(2)
KF_DECL_MULTI(3)
#undef KF_DECL_MULTI

// grid <= 0: as many CTAs as fit at once
inline cudaError_t launch_multi(int dtype, int fam, int mode, const MultiArgs& m, int T, int smem, long long grid,
                                cudaStream_t s) {
#define KF_CASE_MULTI(D)                                                                   \
    case D:                                                                               \
        if (fam == FAM_POW2) return launch_multi_dt##D##_fam0(mode, m, T, smem, grid, s);   \
        if (fam == FAM_SMOOTH) return launch_multi_dt##D##_fam1(mode, m, T, smem, grid, s); \
        return launch_multi_dt##D##_fam2(mode, m, T, smem, grid, s);
    switch (dtype) {
        KF_CASE_MULTI(0)
        KF_CASE_MULTI(1)
        KF_CASE_MULTI(2)
        KF_CASE_MULTI(3)
    }
#undef KF_CASE_MULTI
    return cudaErrorInvalidValue;
}

// kind 1: real split, 2: real merge items of many steps (kf_multi_elem_kernel)
inline cudaError_t launch_multi_elem(int dtype, int kind, const MultiArgs& m, cudaStream_t s) {
    switch (dtype) {
        case 0: return launch_multi_elem_dt0(kind, m, s);
        case 1: return launch_multi_elem_dt1(kind, m, s);
        case 2: return launch_multi_elem_dt2(kind, m, s);
        case 3: return launch_multi_elem_dt3(kind, m, s);
    }
    return cudaErrorInvalidValue;
}

// Run-time specialised kernels (kf_jit.cpp).
bool specialize_enabled();
void set_specialize(int on);
const void* spec_kernel(const Step& st, std::string& err);
bool spec_compile_only(const Step& st, std::string& err);

inline cudaError_t launch_spec(const void* k, const Step& st, cudaStream_t s) {
    const long long grid = launch_grid(k, st);
    if (grid <= 0) return cudaSuccess;
    // the specialised kernels take the run-time part only (their shape is compiled in)
    void* args[] = {(void*)static_cast<const KRun*>(&st.args)};
    return launch_engine_raw(k, grid, st, args, s);
}

inline cudaError_t launch_step(const Step& st, cudaStream_t s) {
    if (st.kind == 0 && specialize_enabled()) {
        if (st.kfn) return launch_spec(st.kfn, st, s);
        std::string err;
        const void* k = spec_kernel(st, err);
        if (k) return launch_spec(k, st, s);
    }
#define KF_CASE_DT(D)                                                       \
    case D:                                                                 \
        if (st.kind != 0) return launch_elem_dt##D(st, s);                  \
        if (st.fam == FAM_POW2) return launch_engine_dt##D##_fam0(st, s);   \
        if (st.fam == FAM_SMOOTH) return launch_engine_dt##D##_fam1(st, s); \
        return launch_engine_dt##D##_fam2(st, s);
    switch (st.dtype) {
        KF_CASE_DT(0)
        KF_CASE_DT(1)
        KF_CASE_DT(2)
        KF_CASE_DT(3)
    }
#undef KF_CASE_DT
    return cudaErrorInvalidValue;
}

}  // namespace kf
