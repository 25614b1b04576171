// Specialised engine kernels: the plan shape of one (type, size, direction)
// is evaluated at compile time by make_shape, so every stride, pass kind,
// twiddle offset and divisor of the engine is a constant and the pass loop
// unrolls.  Instantiated ahead of time for common sizes (kf_spec_inst.cu)
// and at run time through NVRTC for any other size (kf_jit.cpp).
#pragma once
#include "kf_device.cuh"

namespace kf {

// The shape as a constant of static storage: the engine reads it through a
// reference and the compiler folds every load.
template <int DT, int N, int INV, int LMAX>
__device__ constexpr ShapeInfo kSpecShape = make_shape(DT, N, INV, LMAX, 0);

// MODE/J/COLIN/COLOUT/SWZ fix the launch shape too (J jobs per tile, the
// shared-tile index map); T threads per block and MINB resident blocks per
// SM bound the registers a thread.
template <typename S, int MODE, int DT, int N, int INV, int LMAX, int SUB, int J, int COLIN, int COLOUT, int T,
          int MINB, int SWZ>
__global__ void __launch_bounds__(T, MINB) kf_spec_kernel(const __grid_constant__ KRun a) {
    static_assert(kSpecShape<DT, N, INV, LMAX>.error == 0, "plan shape");
    constexpr kmask_t KM = kind_mask(kSpecShape<DT, N, INV, LMAX>.sub[SUB]);
    if constexpr ((MODE == MODE_C2C || MODE == MODE_R2C) && COLIN == 0 && COLOUT == 0) {
        if (a.tma) {
            engine_body_tma<S, MODE, KM, J, SWZ>(a, kSpecShape<DT, N, INV, LMAX>.sub[SUB]);
            return;
        }
    }
    // the fast FIR's second sub-plan is the inverse of the same size
    engine_body<S, MODE, KM, J, COLIN, COLOUT, SWZ>(a, kSpecShape<DT, N, INV, LMAX>.sub[SUB],
                                                kSpecShape<DT, N, MODE == MODE_FIR ? 1 : INV, LMAX>.sub[SUB]);
}

}  // namespace kf
