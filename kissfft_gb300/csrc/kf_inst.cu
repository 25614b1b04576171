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

#if KF_INST_FAM == 0
cudaError_t KF_NAME(launch_elem_dt, KF_INST_DT, , )(const Step& st, cudaStream_t s) {
    return launch_elem<kf_inst_s>(st, s);
}
#endif

}  // namespace kf
