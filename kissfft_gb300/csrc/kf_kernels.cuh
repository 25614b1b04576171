// CUDA kernels for sm_103a: the engine kernel (one tile of jobs per CTA
// iteration) and the element kernels of two-pass real plans.
#pragma once
#include <cuda_runtime.h>

#include "kf_plan.h"
#include "kf_runner.cuh"

namespace kf {

template <typename S, int MODE, int FAM>
struct DevExec {
    __device__ void sync() { __syncthreads(); }
    __device__ void pass(Tile<S>& t, const KSub& sb, const KPass& ps, bool last, bool sg, bool dg) {
        run_pass<S, MODE, FAM>(t, sb, ps, last, threadIdx.x, blockDim.x, sg, dg);
    }
    __device__ void rtg(Tile<S>& t, const KSub& sb, const KPass& ps, bool last, bool sg, bool dg) {
        cpx<S> ov[KF_MAXO];
        rtg_compute<S, MODE>(t, sb, ps, last, threadIdx.x, blockDim.x, sg, ov);
        __syncthreads();
        rtg_store<S, MODE>(t, sb, ps, last, threadIdx.x, blockDim.x, dg, ov);
    }
    __device__ void c2r_pre(Tile<S>& t, const KSub& sb) { kf::c2r_pre<S>(t, sb, threadIdx.x, blockDim.x); }
    __device__ void r2c_post(Tile<S>& t, const KSub& sb) { kf::r2c_post<S>(t, sb, threadIdx.x, blockDim.x); }
    __device__ void fir_mid(Tile<S>& t, const KSub& fw, const KSub& iv, const cpx<S>* H) {
        cpx<S> ov[KF_MAXO];
        fir_mid_compute<S>(t, fw, iv, H, threadIdx.x, blockDim.x, ov);
        __syncthreads();
        fir_mid_store<S>(t, fw, threadIdx.x, blockDim.x, ov);
    }
};

// One CTA works through tiles blockIdx.x, blockIdx.x + gridDim.x, ... of J
// jobs each; the tile lives in dynamic shared memory.
template <typename S, int MODE, int FAM>
__global__ void __launch_bounds__(KF_MAXT) kf_engine_kernel(const __grid_constant__ KArgs a) {
    extern __shared__ __align__(16) unsigned char kf_dyn_smem[];
    __shared__ long long s_inb[KF_MAXJ], s_outb[KF_MAXJ], s_lin[KF_MAXJ], s_lout[KF_MAXJ];
    __shared__ int s_U[KF_MAXJ];
    Tile<S> t;
    tile_layout(a, t);
    t.sm = (cpx<S>*)kf_dyn_smem;
    t.T = blockDim.x;
    t.inb = s_inb;
    t.outb = s_outb;
    t.U = s_U;
    t.lim_in = s_lin;
    t.lim_out = s_lout;
    DevExec<S, MODE, FAM> x;
    for (long long tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
        for (int j = threadIdx.x; j < a.J; j += blockDim.x) job_entry(a, tile, j, s_inb[j], s_outb[j], s_U[j], s_lin[j], s_lout[j]);
        __syncthreads();
        run_tile<S, MODE, FAM>(x, a, t);
        __syncthreads();
    }
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

template <typename S, int MODE, int FAM>
static cudaError_t launch_engine_f(const Step& st, cudaStream_t s) {
    auto k = kf_engine_kernel<S, MODE, FAM>;
    static bool attr_done = false;
    if (!attr_done) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (e != cudaSuccess) return e;
        attr_done = true;
    }
    long long grid = st.cfg.grid;
    if (grid > 0x7fffffffLL) grid = 0x7fffffffLL;
    if (grid <= 0) return cudaSuccess;
    k<<<(unsigned)grid, st.cfg.T, st.cfg.smem, s>>>(st.args);
    return cudaGetLastError();
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
    cudaError_t launch_elem_dt##D(const Step&, cudaStream_t);
KF_DECL_DT(0)
KF_DECL_DT(1)
KF_DECL_DT(2)
KF_DECL_DT(3)
#undef KF_DECL_DT

inline cudaError_t launch_step(const Step& st, cudaStream_t s) {
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
