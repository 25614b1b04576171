// Device side of the engine kernels (compiled by nvcc and by NVRTC): the
// executor that maps the tile sequencing onto a CUDA block, the engine
// kernel body, and the element kernels of two-pass real plans.
#pragma once
#include "kf_runner.cuh"

namespace kf {

// ------------------------------------------------- programmatic dependent launch
// Engine launches may start while the previous kernel in their stream
// finishes (launch attribute programmaticStreamSerialization): every block
// first waits until that kernel has completed and its writes are visible
// (a no-op for a launch without the attribute), then lets the next launch
// in the stream begin to launch.  No global memory is touched before the wait.
__device__ __forceinline__ void kf_pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// ---------------------------------------------------------------- TMA staging
// One-dimensional bulk copies global -> shared completing on an mbarrier
// (cp.async.bulk, sm_90+).  Every wait is bounded: past the limit the kernel
// records bit 1 in the error word and stops using the tile.
__device__ __forceinline__ unsigned kf_smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void kf_mbar_init(unsigned bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void kf_fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void kf_fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void kf_bulk_load(unsigned dst, const void* src, unsigned bytes, unsigned bar) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

__device__ __forceinline__ bool kf_mbar_try_wait(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait for phase `parity`; false after the limit (about seconds)
__device__ __forceinline__ bool kf_mbar_wait(unsigned bar, unsigned parity) {
    for (long long it = 0; it < (1LL << 22); ++it)
        if (kf_mbar_try_wait(bar, parity)) return true;
    return false;
}

template <typename S, int MODE, kmask_t KM>
struct DevExec {
    // TMA staging: thread 0 re-arms the staging buffer once the first pass
    // has read it (next >= 0: the tile to fetch)
    long long next = -1;
    unsigned bar = 0, stage = 0;
    const KRun* args = nullptr;
    int L = 0;
    __device__ void input_consumed() {
        if (next >= 0 && threadIdx.x == 0) {
            kf_fence_proxy_async();
            issue(next);
        }
    }
    __device__ void issue(long long tile) {
        const long long jg0 = tile * args->J;
        long long nj = args->G - jg0;
        if (nj > args->J) nj = args->J;
        const unsigned bytes = (unsigned)(nj * L * (long long)sizeof(cpx<S>));
        const cpx<S>* src = (const cpx<S>*)args->in + jg0 * args->in_dhi;
        kf_bulk_load(stage, src, bytes, bar);
    }
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
template <typename S, int MODE, kmask_t KM, int JF = 0, int CIF = -1, int COF = -1, int SWF = -1>
__device__ __forceinline__ void engine_body(const KRun& a, const KSub& s0, const KSub& s1) {
    kf_pdl_enter();
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
    if (SWF >= 0) t.swzm = SWF;
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

// Tiles of contiguous input (a.tma): persistent CTAs, the next tile's input
// is bulk-copied into a staging buffer while the current tile runs its
// passes; the first pass reads the staged tile through shared memory.
template <typename S, int MODE, kmask_t KM, int JF = 0, int SWF = -1>
__device__ __forceinline__ void engine_body_tma(const KRun& a, const KSub& s0) {
    kf_pdl_enter();
    extern __shared__ __align__(16) unsigned char kf_dyn_smem[];
    __shared__ long long s_inb[KF_MAXJ], s_outb[KF_MAXJ], s_lin[KF_MAXJ], s_lout[KF_MAXJ];
    __shared__ int s_U[KF_MAXJ];
    __shared__ __align__(8) unsigned long long s_bar;
    const int J = JF > 0 ? JF : a.J;
    const int logJ = JF > 0 ? (JF >= 64 ? 6 : JF >= 32 ? 5 : JF >= 16 ? 4 : JF >= 8 ? 3 : JF >= 4 ? 2 : JF >= 2 ? 1 : 0)
                            : a.logJ;
    cpx<S>* stage = (cpx<S>*)(kf_dyn_smem + a.stage_off);
    Tile<S> t;
    tile_layout(a, s0.L, J, logJ, 0, t);
    if (SWF >= 0) t.swzm = SWF;
    t.sm = (cpx<S>*)kf_dyn_smem;
    t.T = blockDim.x;
    t.inb = s_inb;
    t.outb = s_outb;
    t.U = s_U;
    t.lim_in = s_lin;
    t.lim_out = s_lout;
    t.in = stage;  // the first pass reads the staged tile
    t.in_stride = 1;
    DevExec<S, MODE, KM> x;
    x.bar = kf_smem_u32(&s_bar);
    x.stage = kf_smem_u32(stage);
    x.args = &a;
    x.L = s0.L;
    if (threadIdx.x == 0) {
        kf_mbar_init(x.bar, 1);
        kf_fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0 && (long long)blockIdx.x < a.ntiles) x.issue(blockIdx.x);
    unsigned parity = 0;
    for (long long tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x) {
        for (int j = threadIdx.x; j < J; j += blockDim.x) {
            job_entry(a, tile, J, j, s_inb[j], s_outb[j], s_U[j], s_lin[j], s_lout[j]);
            if (s_inb[j] >= 0) s_inb[j] = (long long)j * s0.L;  // offset inside the staging buffer
        }
        const bool ok = kf_mbar_wait(x.bar, parity);
        parity ^= 1u;
        if (!ok) {
            if (threadIdx.x == 0 && a.err) atomicOr(a.err, 2);
            kf_mbar_wait(x.bar, parity ^ 1u);  // give the copy in flight a last chance to land
            return;
        }
        __syncthreads();
        const long long nxt = tile + gridDim.x;
        x.next = nxt < a.ntiles ? nxt : -1;
        run_tile<S, MODE, KM>(x, a, s0, s0, t, 0, 0);
        __syncthreads();
    }
}

template <typename S, int MODE, int FAM>
__global__ void __launch_bounds__(KF_MAXT) kf_engine_kernel(const __grid_constant__ KArgs a) {
    if constexpr (MODE == MODE_C2C || MODE == MODE_R2C) {
        if (a.tma) {
            engine_body_tma<S, MODE, family_mask(FAM, is_f32<S>())>(a, a.sub[0]);
            return;
        }
    }
    engine_body<S, MODE, family_mask(FAM, is_f32<S>())>(a, a.sub[0], a.sub[1]);
}

// Persistent multi-plan kernel: tiles of many plans (one sample type and
// mode) in one launch, pulled from a work queue.  Every step carries its own
// shape (KArgs in global memory); the CTA copies the step's KArgs into shared
// memory when it takes an item, so the passes read the shape with shared
// loads instead of global ones on their address paths.  blockDim and the
// shared tile are sized for the largest step of the launch.
// Registers capped at 80 a thread (up to 512 threads a block): every pass
// kind of a family is compiled in, and without a cap the compiler takes 128
// and leaves the work-queue launches at a quarter of the warps; 80 was the
// fastest of 64/80/96/128 on the uneven mix.
template <typename S, int MODE, kmask_t KM>
__global__ void __maxnreg__(80) kf_multi_kernel(const __grid_constant__ MultiArgs m) {
    extern __shared__ __align__(16) unsigned char kf_dyn_smem[];
    __shared__ long long s_inb[KF_MAXJ], s_outb[KF_MAXJ], s_lin[KF_MAXJ], s_lout[KF_MAXJ];
    __shared__ int s_U[KF_MAXJ];
    __shared__ unsigned long long s_item;
    __shared__ __align__(16) KArgs s_args;
    static_assert(sizeof(KArgs) % 8 == 0, "KArgs copies as 8-byte words");
    DevExec<S, MODE, KM> x;
    int cur = -1;  // step whose arguments s_args holds (the same in every thread)
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(m.counter, 1ull);
        __syncthreads();
        const unsigned long long it = s_item;
        if (it >= (unsigned long long)m.nitems) break;
        const MultiItem w = m.items[it];
        if (w.step != cur) {
            // every thread is past the previous tile (barrier at its end)
            const uint2* src = (const uint2*)(m.steps + w.step);
            uint2* dst = (uint2*)&s_args;
            for (int k = threadIdx.x; k < (int)(sizeof(KArgs) / 8); k += blockDim.x) dst[k] = src[k];
            cur = w.step;
            __syncthreads();
        }
        const KArgs& a = s_args;
        Tile<S> t;
        tile_layout(a, a.sub[0].L, a.J, a.logJ, a.col_in | a.col_out, t);
        t.sm = (cpx<S>*)kf_dyn_smem;
        t.T = blockDim.x;
        t.inb = s_inb;
        t.outb = s_outb;
        t.U = s_U;
        t.lim_in = s_lin;
        t.lim_out = s_lout;
        for (int j = threadIdx.x; j < a.J; j += blockDim.x)
            job_entry(a, w.tile, a.J, j, s_inb[j], s_outb[j], s_U[j], s_lin[j], s_lout[j]);
        __syncthreads();
        run_tile<S, MODE, KM>(x, a, a.sub[0], a.sub[1], t, a.col_in, a.col_out);
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

// Real split / merge items of many two-pass real plans in one launch
// (batched requests): work item w covers elements [w.tile * KF_ELEM_CHUNK,
// (w.tile + 1) * KF_ELEM_CHUNK) of step w.step.  KIND 1 splits, 2 merges.
template <typename S, int KIND>
__global__ void __launch_bounds__(256) kf_multi_elem_kernel(const __grid_constant__ MultiArgs m) {
    __shared__ unsigned long long s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(m.counter, 1ull);
        __syncthreads();
        const unsigned long long it = s_item;
        __syncthreads();  // all threads hold the item before thread 0 takes the next
        if (it >= (unsigned long long)m.nitems) break;
        const MultiItem w = m.items[it];
        const KArgs& a = m.steps[w.step];
        const long long total = a.G * (a.sub[0].L / 2 + 1);
        const long long lo = w.tile * KF_ELEM_CHUNK;
        const long long hi = lo + KF_ELEM_CHUNK < total ? lo + KF_ELEM_CHUNK : total;
        for (long long e = lo + threadIdx.x; e < hi; e += blockDim.x) {
            if constexpr (KIND == 1)
                split_item<S>(a, e);
            else
                merge_item<S>(a, e);
        }
    }
}

}  // namespace kf
