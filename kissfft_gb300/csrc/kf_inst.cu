// Kernel instantiations for one (sample type, kernel family) pair, selected
// at compile time with -DKF_INST_DT=<0..3> -DKF_INST_FAM=<0..2>.  The build
// compiles this file once per pair, in parallel.
#include "kf_kernels.cuh"

#if !defined(KF_INST_DT) || !defined(KF_INST_FAM)
#error "KF_INST_DT and KF_INST_FAM must be defined"
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

#define KF_PASTE4(a, b, c, d) a##b##c##d
#define KF_NAME(a, b, c, d) KF_PASTE4(a, b, c, d)

namespace kf {

cudaError_t KF_NAME(launch_engine_dt, KF_INST_DT, _fam, KF_INST_FAM)(const Step& st, cudaStream_t s) {
    typedef kf_inst_s S;
    switch (st.mode) {
        case MODE_C2C: return launch_engine_f<S, MODE_C2C, KF_INST_FAM>(st, s);
        case MODE_R2C: return launch_engine_f<S, MODE_R2C, KF_INST_FAM>(st, s);
        case MODE_C2R: return launch_engine_f<S, MODE_C2R, KF_INST_FAM>(st, s);
#if KF_INST_DT == 0 && KF_INST_FAM < 2
        // fast FIR blocks are powers of two by default (tools/kiss_fastfir.c:75-87);
        // the fused FIR kernel is built for 2/3/5-smooth block sizes
        case MODE_FIR: return launch_engine_f<S, MODE_FIR, KF_INST_FAM>(st, s);
#endif
    }
    return cudaErrorNotSupported;
}

cudaError_t KF_NAME(launch_multi_dt, KF_INST_DT, _fam, KF_INST_FAM)(int mode, const MultiArgs& m, int T, int smem,
                                                                     long long grid, cudaStream_t s) {
    typedef kf_inst_s S;
    constexpr kmask_t KM = family_mask(KF_INST_FAM, KF_INST_DT == 0);
    const void* k = nullptr;
    switch (mode) {
        case MODE_C2C: k = (const void*)kf_multi_kernel<S, MODE_C2C, KM>; break;
        case MODE_R2C: k = (const void*)kf_multi_kernel<S, MODE_R2C, KM>; break;
        case MODE_C2R: k = (const void*)kf_multi_kernel<S, MODE_C2R, KM>; break;
        default: return cudaErrorNotSupported;
    }
    static bool attr_done[3] = {false, false, false};
    if (!attr_done[mode]) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e != cudaSuccess) return e;
        attr_done[mode] = true;
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

}  // namespace kf
