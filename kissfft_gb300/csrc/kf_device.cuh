// Device side of the engine kernels (compiled by nvcc and by NVRTC): the
// executor that maps the tile sequencing onto a CUDA block, the engine
// kernel body, and the element kernels of two-pass real plans.
#pragma once
#include "kf_runner.cuh"

namespace kf {

template <typename S, int MODE, unsigned KM>
struct DevExec {
    __device__ void sync() { __syncthreads(); }
    __device__ void pass(Tile<S>& t, const KSub& sb, const KTab& tb, const KPass& ps, bool last, bool sg, bool dg) {
        run_pass<S, MODE, KM>(t, sb, tb, ps, last, threadIdx.x, blockDim.x, sg, dg);
    }
    __device__ void rtg(Tile<S>& t, const KSub& sb, const KTab& tb, const KPass& ps, bool last, bool sg, bool dg) {
        cpx<S> ov[KF_MAXO];
        rtg_compute<S, MODE>(t, sb, tb, ps, last, threadIdx.x, blockDim.x, sg, ov);
        __syncthreads();
        rtg_store<S, MODE>(t, sb, tb, ps, last, threadIdx.x, blockDim.x, dg, ov);
    }
    __device__ void c2r_pre(Tile<S>& t, const KSub& sb, const KTab& tb) {
        kf::c2r_pre<S>(t, sb, tb, threadIdx.x, blockDim.x);
    }
    __device__ void r2c_post(Tile<S>& t, const KSub& sb, const KTab& tb) {
        kf::r2c_post<S>(t, sb, tb, threadIdx.x, blockDim.x);
    }
    __device__ void fir_mid(Tile<S>& t, const KSub& fw, const KTab& fwt, const KTab& ivt, const cpx<S>* H) {
        cpx<S> ov[KF_MAXO];
        fir_mid_compute<S>(t, fw, fwt, ivt, H, threadIdx.x, blockDim.x, ov);
        __syncthreads();
        fir_mid_store<S>(t, fw, threadIdx.x, blockDim.x, ov);
    }
};

// Body shared by the generic and the specialised kernels: one CTA works
// through tiles blockIdx.x, blockIdx.x + gridDim.x, ... of J jobs each; the
// tile lives in dynamic shared memory.  JF/CIF/COF > 0 fix the tile shape at
// compile time (specialised kernels); 0 takes it from the arguments.
template <typename S, int MODE, unsigned KM, int JF = 0, int CIF = -1, int COF = -1>
__device__ __forceinline__ void engine_body(const KArgs& a, const KSub& s0, const KSub& s1) {
    extern __shared__ __align__(16) unsigned char kf_dyn_smem[];
    __shared__ long long s_inb[KF_MAXJ], s_outb[KF_MAXJ], s_lin[KF_MAXJ], s_lout[KF_MAXJ];
    __shared__ int s_U[KF_MAXJ];
    const int J = JF > 0 ? JF : a.J;
    const int logJ = JF > 0 ? (JF >= 64 ? 6 : JF >= 32 ? 5 : JF >= 16 ? 4 : JF >= 8 ? 3 : JF >= 4 ? 2 : JF >= 2 ? 1 : 0)
                            : a.logJ;
    const int ci = CIF >= 0 ? CIF : a.col_in;
    const int co = COF >= 0 ? COF : a.col_out;
    Tile<S> t;
    tile_layout(a, s0.L, J, logJ, ci | co, t);
    t.sm = (cpx<S>*)kf_dyn_smem;
    t.T = blockDim.x;
    t.inb = s_inb;
    t.outb = s_outb;
    t.U = s_U;
    t.lim_in = s_lin;
    t.lim_out = s_lout;
    DevExec<S, MODE, KM> x;
    for (long long tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
        for (int j = threadIdx.x; j < J; j += blockDim.x) job_entry(a, tile, J, j, s_inb[j], s_outb[j], s_U[j], s_lin[j], s_lout[j]);
        __syncthreads();
        run_tile<S, MODE, KM>(x, a, s0, s1, t, ci, co);
        __syncthreads();
    }
}

template <typename S, int MODE, int FAM>
__global__ void __launch_bounds__(KF_MAXT) kf_engine_kernel(const __grid_constant__ KArgs a) {
    engine_body<S, MODE, family_mask(FAM)>(a, a.sub[0], a.sub[1]);
}

template <typename S>
__global__ void __launch_bounds__(256) kf_split_kernel(const __grid_constant__ KArgs a) {
    const long long items = a.G * (a.sub[0].L / 2 + 1);
    for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < items;
         it += (long long)gridDim.x * blockDim.x)
        split_item<S>(a, it);
}

template <typename S>
__global__ void __launch_bounds__(256) kf_merge_kernel(const __grid_constant__ KArgs a) {
    const long long items = a.G * (a.sub[0].L / 2 + 1);
    for (long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x; it < items;
         it += (long long)gridDim.x * blockDim.x)
        merge_item<S>(a, it);
}

}  // namespace kf
