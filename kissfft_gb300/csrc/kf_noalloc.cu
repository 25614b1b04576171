// kfg_exec_batch_noalloc: batched complex 1-D transforms that allocate no
// device memory.
//
// Who needs it: callers that may not allocate device memory while they
// transform.  Examples are code that runs inside a custom device allocator
// or memory-pool hook (an allocation there would re-enter the allocator),
// real-time loops whose memory is fixed at start-up and may not touch the
// driver's allocator afterwards, and hosts that hand all device memory to
// their own pool up front.  kfg_exec_batch serves everyone else: for plans
// longer than one shared-memory tile it allocates stream-ordered scratch
// for the transposed intermediate that the two HBM passes exchange.  This
// entry point runs the same precompiled kernels with that intermediate in
// the fixed device array below instead.
//
// Rules of use:
//  - complex 1-D plans (kfg_plan_c2c) and device pointers for in and out;
//  - a call may need at most KFG_NOALLOC_SCRATCH_BYTES (64 MiB) of scratch:
//    batch * nfft complex elements for a two-pass plan, none for a plan that
//    fits one tile.  A larger batch is rejected with KFG_EINVAL and a
//    message; split it into several calls;
//  - there is one array per device, shared by every call on that device and
//    keeping the last call's data.  Calls whose kernels can run at the same
//    time (on different streams, or from different host threads) race on it
//    and give wrong results: issue them on one stream.  Nothing in it has to
//    start at zero: the first pass writes every element the second pass
//    reads;
//  - the stream and both buffers must belong to the current device: the
//    array used is the current device's.  A stream or buffer of another
//    device is refused with KFG_EINVAL;
//  - the first call in a CUDA context of a device (with that device
//    current) looks up the array's device address with cudaGetSymbolAddress,
//    which loads this module into the context if it is not loaded yet.  Make
//    that first call before any stream capture on that device.  The address
//    is kept per context: after cudaDeviceReset (or a reset of the primary
//    context) the next call finds a new context and looks the address up
//    again;
//  - the array lives in this file's own device module, which holds no
//    kernel.  With lazy module loading (the CUDA default) that module, and
//    its 64 MiB, is loaded by the first call of this entry point in a
//    context; with eager loading (CUDA_MODULE_LOADING=EAGER) every context
//    of a process that loads this library reserves the 64 MiB, whether it
//    calls the entry point or not;
//  - run-time specialised kernels are not used here (their first use
//    compiles and loads a module), so the precompiled kernels run whatever
//    kfg_set_specialize says.
#include <mutex>
#include <string>

#include "kf_kernels.cuh"
#include "kissfft_gb300.h"

using namespace kf;

namespace kf {
int c2c_schedule(kfg_plan* p, long long batch, long long in_dist, long long out_dist, Schedule& s);
int set_error(int code, const std::string& msg);
bool device_pointer(const void* ptr);
cudaStream_t stream_or_default(void* stream);
}  // namespace kf

static __device__ __align__(256) unsigned char kf_noalloc_scratch[KFG_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
// device address of kf_noalloc_scratch per device, and the context it was
// looked up in
struct ScratchAddr {
    unsigned long long ctx = 0;
    void* ptr = nullptr;
};
ScratchAddr g_scratch[kMaxDevices];

// Set-up, once per device and context, with that device current.
int scratch_of_current_device(int dev, void** out) {
    if (dev < 0 || dev >= kMaxDevices) return set_error(KFG_EUNSUPPORTED, "kfg_exec_batch_noalloc: device index too large");
    std::lock_guard<std::mutex> lk(g_setup_mu);
    const unsigned long long ctx = current_context_id();
    ScratchAddr& a = g_scratch[dev];
    if (!a.ptr || ctx == 0 || a.ctx != ctx) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, kf_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return set_error(KFG_ECUDA, std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(e));
        a.ptr = ptr;
        a.ctx = current_context_id();  // the lookup makes the device's primary context current if none was
    }
    *out = a.ptr;
    return KFG_OK;
}

// The device a pointer's memory belongs to, or -1.
int device_of(const void* ptr) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return a.device;
}

// launch_step without the run-time specialised kernels
cudaError_t launch_precompiled(const Step& st, cudaStream_t s) {
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

}  // namespace

extern "C" int kfg_exec_batch_noalloc(kfg_plan* p, const void* in, void* out, long long batch, long long in_dist,
                                      long long out_dist, void* stream) {
    if (!p || !in || !out || batch < 0) return set_error(KFG_EINVAL, "kfg_exec_batch_noalloc: bad arguments");
    if (batch == 0) return KFG_OK;
    if (!device_pointer(in) || !device_pointer(out))
        return set_error(KFG_EINVAL, "kfg_exec_batch_noalloc: in and out must be device pointers");
    Schedule s;
    int rc = c2c_schedule(p, batch, in_dist, out_dist, s);
    if (rc) return rc;
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(KFG_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    const cudaStream_t st = stream_or_default(stream);
    int sdev = -1;
    e = cudaStreamGetDevice(st, &sdev);
    if (e != cudaSuccess) return set_error(KFG_ECUDA, std::string("cudaStreamGetDevice: ") + cudaGetErrorString(e));
    if (sdev != dev || device_of(in) != dev || device_of(out) != dev)
        return set_error(KFG_EINVAL, "kfg_exec_batch_noalloc: the stream and both buffers must be on the current device");
    const size_t off1 = (s.scratch[0] + 255) & ~(size_t)255;
    const size_t need = s.scratch[1] ? off1 + s.scratch[1] : s.scratch[0];
    if (need > KFG_NOALLOC_SCRATCH_BYTES)
        return set_error(KFG_EINVAL, "kfg_exec_batch_noalloc: this batch needs " + std::to_string(need) +
                                         " bytes of scratch, more than the fixed " +
                                         std::to_string((size_t)KFG_NOALLOC_SCRATCH_BYTES) +
                                         "; split it into smaller batches");
    void* scratch = nullptr;
    if (need > 0) {
        rc = scratch_of_current_device(dev, &scratch);
        if (rc) return rc;
    }
    void* roles[4] = {(void*)in, out, scratch, scratch ? (char*)scratch + off1 : nullptr};
    for (auto& step : s.steps) {
        step.args.in = roles[step.in_role];
        step.args.out = roles[step.out_role];
        step.args.fir_H = nullptr;
        enable_tma(step, step.args.in);
        e = launch_precompiled(step, st);
        if (e != cudaSuccess) return set_error(KFG_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
    }
    return KFG_OK;
}
