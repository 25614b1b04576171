// Kernel instantiations for one (sample type, kernel family, transform mode)
// part, selected at compile time with -DKF_INST_DT=<0..3> -DKF_INST_FAM=<0..2>
// -DKF_INST_MODE=<0..3> (MODE_C2C, MODE_R2C, MODE_C2R, MODE_FIR).  The build
// compiles this file once per part, all parts in parallel: the engine and
// work-queue kernels of one mode are a unit of their own, so the largest
// families (float plans with three-stage register groups, generic radices)
// do not serialise the whole build behind one compiler process.
//
// Part MODE_C2C of each (type, family) also holds the dispatchers over modes
// (launch_engine_dt<D>_fam<F>, launch_multi_dt<D>_fam<F>) and, for family 0,
// the element kernels of two-pass real plans.
#include "kf_kernels.cuh"

#if !defined(KF_INST_DT) || !defined(KF_INST_FAM) || !defined(KF_INST_MODE)
#error "KF_INST_DT, KF_INST_FAM and KF_INST_MODE must be defined"
#endif

#if KF_INST_DT == 0
typedef float kf_inst_s;
#elif KF_INST_DT == 1
typedef double kf_inst_s;
#elif KF_INST_DT == 2
typedef int16_t kf_inst_s;
#else
typedef int32_t kf_inst_s;
#endif

// fast FIR blocks are powers of two by default (tools/kiss_fastfir.c:75-87);
// the fused FIR kernel is built for float and 2/3/5-smooth block sizes
#define KF_HAS_FIR(D, F) ((D) == 0 && (F) < 2)

// (the preprocessor sees the mode as its number: MODE_FIR is 3)
#if KF_INST_MODE == 3 && !KF_HAS_FIR(KF_INST_DT, KF_INST_FAM)
#error "the fast FIR part exists for float families 0 and 1 only"
#endif

#define KF_PASTE6(a, b, c, d, e, f) a##b##c##d##e##f
#define KF_NAME6(a, b, c, d, e, f) KF_PASTE6(a, b, c, d, e, f)
#define KF_PASTE4(a, b, c, d) a##b##c##d
#define KF_NAME(a, b, c, d) KF_PASTE4(a, b, c, d)

// per-mode entry points of this (type, family): engine_m<M>, multi_m<M>
#define KF_ENGINE_M(M) KF_NAME6(launch_engine_dt, KF_INST_DT, _fam, KF_INST_FAM, _m, M)
#define KF_MULTI_M(M) KF_NAME6(launch_multi_dt, KF_INST_DT, _fam, KF_INST_FAM, _m, M)

namespace kf {

cudaError_t KF_ENGINE_M(0)(const Step& st, cudaStream_t s);
cudaError_t KF_ENGINE_M(1)(const Step& st, cudaStream_t s);
cudaError_t KF_ENGINE_M(2)(const Step& st, cudaStream_t s);
cudaError_t KF_ENGINE_M(3)(const Step& st, cudaStream_t s);
cudaError_t KF_MULTI_M(0)(const MultiArgs& m, int T, int smem, long long grid, cudaStream_t s);
cudaError_t KF_MULTI_M(1)(const MultiArgs& m, int T, int smem, long long grid, cudaStream_t s);
cudaError_t KF_MULTI_M(2)(const MultiArgs& m, int T, int smem, long long grid, cudaStream_t s);

// ------------------------------------------------------------ this part's kernels
cudaError_t KF_ENGINE_M(KF_INST_MODE)(const Step& st, cudaStream_t s) {
    return launch_engine_f<kf_inst_s, KF_INST_MODE, KF_INST_FAM>(st, s);
}

#if KF_INST_MODE != 3
cudaError_t KF_MULTI_M(KF_INST_MODE)(const MultiArgs& m, int T, int smem, long long grid, cudaStream_t s) {
    constexpr kmask_t KM = family_mask(KF_INST_FAM, KF_INST_DT == 0);
    const void* k = (const void*)kf_multi_kernel<kf_inst_s, KF_INST_MODE, KM>;
    static std::atomic<unsigned long long> attr_ctx{0};
    const unsigned long long ctx = current_context_id();
    if (ctx == 0 || attr_ctx.load() != ctx) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e != cudaSuccess) return e;
        attr_ctx.store(current_context_id());
    }
    if (grid <= 0) {
        int per = 0, nsm = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, T, (size_t)smem) != cudaSuccess || per < 1) per = 1;
        grid = (long long)per * (nsm > 0 ? nsm : 1);
        if (grid > m.nitems) grid = m.nitems;
    }
    if (grid <= 0) return cudaSuccess;
    void* args[] = {(void*)&m};
    return cudaLaunchKernel(k, dim3((unsigned)grid), dim3(T), args, (size_t)smem, s);
}
#endif

#if KF_INST_MODE == 0
// ------------------------------------------------------------ dispatchers over modes
cudaError_t KF_NAME(launch_engine_dt, KF_INST_DT, _fam, KF_INST_FAM)(const Step& st, cudaStream_t s) {
    switch (st.mode) {
        case MODE_C2C: return KF_ENGINE_M(0)(st, s);
        case MODE_R2C: return KF_ENGINE_M(1)(st, s);
        case MODE_C2R: return KF_ENGINE_M(2)(st, s);
#if KF_HAS_FIR(KF_INST_DT, KF_INST_FAM)
        case MODE_FIR: return KF_ENGINE_M(3)(st, s);
#endif
    }
    return cudaErrorNotSupported;
}

cudaError_t KF_NAME(launch_multi_dt, KF_INST_DT, _fam, KF_INST_FAM)(int mode, const MultiArgs& m, int T, int smem,
                                                                     long long grid, cudaStream_t s) {
    switch (mode) {
        case MODE_C2C: return KF_MULTI_M(0)(m, T, smem, grid, s);
        case MODE_R2C: return KF_MULTI_M(1)(m, T, smem, grid, s);
        case MODE_C2R: return KF_MULTI_M(2)(m, T, smem, grid, s);
    }
    return cudaErrorNotSupported;
}

#if KF_INST_FAM == 0
cudaError_t KF_NAME(launch_elem_dt, KF_INST_DT, , )(const Step& st, cudaStream_t s) {
    return launch_elem<kf_inst_s>(st, s);
}

cudaError_t KF_NAME(launch_multi_elem_dt, KF_INST_DT, , )(int kind, const MultiArgs& m, cudaStream_t s) {
    typedef kf_inst_s S;
    const void* k = kind == 1 ? (const void*)kf_multi_elem_kernel<S, 1> : (const void*)kf_multi_elem_kernel<S, 2>;
    int per = 0, nsm = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, 256, 0) != cudaSuccess || per < 1) per = 1;
    long long grid = (long long)per * (nsm > 0 ? nsm : 1);
    if (grid > m.nitems) grid = m.nitems;
    if (grid <= 0) return cudaSuccess;
    void* args[] = {(void*)&m};
    return cudaLaunchKernel(k, dim3((unsigned)grid), dim3(256), args, 0, s);
}
#endif
#endif

}  // namespace kf
