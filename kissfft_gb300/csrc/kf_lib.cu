// Core library: device plans, launch-schedule execution, host staging and
// the dtype-tagged C API of include/kissfft_gb300.h.
//
// Plans are immutable once built (twiddles, digit-reversal tables and the
// launch schedule templates live in one device allocation), so one plan may
// be used from several threads and streams at once.  Scratch for two-pass
// plans and host staging is stream-ordered (cudaMallocAsync on the call's
// stream), never shared between calls.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include <math.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <fstream>
#include <iterator>
#include <map>
#include <mutex>
#include <sstream>
#include <thread>
#include <memory>
#include <string>
#include <vector>

#include "kf_kernels.cuh"
#include "kissfft_gb300.h"

using namespace kf;

namespace kf {

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry points, so
// that the library needs no link to the driver library itself.
unsigned long long current_context_id() {
    typedef int (*get_current_t)(void**);
    typedef int (*get_id_t)(void*, unsigned long long*);
    static get_current_t get_current = nullptr;
    static get_id_t get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (get_current_t)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (get_id_t)f;
        cudaGetLastError();
    });
    if (!get_current || !get_id) return 0;
    void* ctx = nullptr;
    if (get_current(&ctx) != 0 || !ctx) return 0;
    unsigned long long id = 0;
    if (get_id(ctx, &id) != 0) return 0;
    return id;
}

}  // namespace kf

namespace {

thread_local std::string g_err;
std::atomic<cudaStream_t> g_stream{(cudaStream_t)0};

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

#define KFG_CK(call)                                                                                   \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) return fail(KFG_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

enum { K_C2C = 1, K_REAL = 2, K_ND = 3, K_NDR = 4, K_FIR = 5 };

struct DevPlan {
    Plan p;
    void* d = nullptr;
    ~DevPlan() {
        if (d) cudaFree(d);
    }
};

std::unique_ptr<DevPlan> make_devplan(int dtype, int n, int inverse, int real_nfft) {
    std::unique_ptr<DevPlan> dp(new DevPlan);
    if (!dp->p.build(dtype, n, inverse, 0, real_nfft)) {
        fail(KFG_EINVAL, dp->p.error);
        return nullptr;
    }
    cudaError_t e = cudaMalloc(&dp->d, dp->p.blob.size());
    if (e != cudaSuccess) {
        fail(e == cudaErrorMemoryAllocation ? KFG_ENOMEM : KFG_ECUDA,
             std::string("cudaMalloc(plan): ") + cudaGetErrorString(e));
        dp->d = nullptr;
        return nullptr;
    }
    e = cudaMemcpy(dp->d, dp->p.blob.data(), dp->p.blob.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        fail(KFG_ECUDA, std::string("cudaMemcpy(plan): ") + cudaGetErrorString(e));
        return nullptr;
    }
    dp->p.bind(dp->d);
    return dp;
}

// Pinned (page-locked, device-mapped) host memory: the kernels read and
// write it directly over the host link.
bool is_pinned_host_ptr(const void* ptr) {
    if (!ptr) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost && a.devicePointer == ptr;
}

// large host batches: chunked copy/compute/copy pipeline (default on;
// KISSFFT_GB300_PIPELINE=0 keeps the zero-copy kernels for every size)
bool pipeline_enabled() {
    static int on = -1;
    if (on < 0) {
        const char* e = getenv("KISSFFT_GB300_PIPELINE");
        on = (e && *e == '0') ? 0 : 1;
    }
    return on == 1;
}

bool zero_copy_enabled() {
    static int on = -1;
    if (on < 0) {
        const char* e = getenv("KISSFFT_GB300_ZEROCOPY");
        on = (e && *e == '0') ? 0 : 1;
    }
    return on == 1;
}

bool is_device_ptr(const void* ptr) {
    if (!ptr) return false;
    cudaPointerAttributes a;
    cudaError_t e = cudaPointerGetAttributes(&a, ptr);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

cudaStream_t pick(void* stream) { return stream ? (cudaStream_t)stream : g_stream.load(); }

// kissfft.hh transform_real packing (kissfft.hh:154-189): bins X[0..n] of a
// 2n-point real transform -> dst[0] = (X0, Xn), dst[k] = X[k] (conjugated
// for the facade's inverse flag), k = 1..n-1.  One thread per output.
template <typename T>
__global__ void kf_pack_real_kernel(const T* X, T* dst, long long n, int conj) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    if (k == 0) {
        dst[0] = X[0];
        dst[1] = X[2 * n];
    } else {
        dst[2 * k] = X[2 * k];
        dst[2 * k + 1] = conj ? -X[2 * k + 1] : X[2 * k + 1];
    }
}

// psdpng's frame preparation (tools/psdpng.c:134-155): 16-bit samples
// (stereo: the two channels summed) to float, optionally minus the frame's
// mean.  One CTA per frame.
__global__ void kf_psd_prep_kernel(const short* in, float* t, int nfft, int stereo, int remove_dc) {
    __shared__ float part[32];
    const long long f = blockIdx.x;
    float* tf = t + f * nfft;
    float sum = 0.f;
    for (int i = threadIdx.x; i < nfft; i += blockDim.x) {
        const long long j = f * nfft + i;
        const float v = stereo ? (float)(in[2 * j] + in[2 * j + 1]) : (float)in[j];
        tf[i] = v;
        sum += v;
    }
    if (!remove_dc) return;
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x < 32) {
        float s = threadIdx.x < (blockDim.x + 31) / 32 ? part[threadIdx.x] : 0.f;
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) part[0] = s;
    }
    __syncthreads();
    const float avg = part[0] / nfft;
    for (int i = threadIdx.x; i < nfft; i += blockDim.x) tf[i] -= avg;
}

// psdpng's row (tools/psdpng.c:160-170): 10*log10(sum over navg frames of
// |X|^2 / navg + 1) per frequency.  One thread per (row, frequency).
__global__ void kf_psd_reduce_kernel(const float* bins, float* rows, long long nrows, int nfreqs, int navg) {
    const long long it = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (it >= nrows * nfreqs) return;
    const long long r = it / nfreqs;
    const int k = (int)(it - r * nfreqs);
    float m = 0.f;
    for (int a = 0; a < navg; ++a) {
        const float* b = bins + 2 * ((r * navg + a) * nfreqs + k);
        m += b[0] * b[0] + b[1] * b[1];
    }
    rows[it] = 10.f * log10f(m / navg + 1.f);
}

// scale the fast FIR response by the reference's float(1.0/nfft)
__global__ void kf_scale_kernel(float* H, long long n, float s) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) H[i] *= s;
}

}  // namespace

// A call's launch schedule, tuned and with its specialised kernels resolved,
// kept per plan for the next call of the same shape.
struct CachedSched {
    long long batch, in_dist, in_stride, out_dist;
    Schedule s;
    size_t ib = 0, ob = 0;
    bool multi = false;  // several steps or column tiles (the pinned-host copy pipeline qualifies)
};

struct kfg_plan {
    int kind = 0, dtype = 0, inverse = 0;
    long long n = 0;  // c2c: nfft; real: nfft; nd/ndr: product of dims; fir: nfft
    std::vector<int> dims;
    std::unique_ptr<DevPlan> main, aux;
    std::vector<std::unique_ptr<DevPlan>> axes;  // one per axis (nd), or per leading axis (ndr)
    long long ntaps = 0;
    void* d_H = nullptr;
    // ready launch schedules of recent calls (most recent first)
    std::mutex sched_mu;
    std::vector<std::shared_ptr<const struct CachedSched>> scheds;
    // autotuned launch shapes per (batch, in_dist, out_dist): J, minb, tma per step
    std::mutex tune_mu;
    std::map<std::string, std::vector<std::array<int, 6>>> tuned;
    ~kfg_plan() {
        if (d_H) cudaFree(d_H);
    }
};

namespace {

int run_schedule(Schedule& s, const void* in, void* out, cudaStream_t st, const void* firH = nullptr,
                 bool allow_tma = true) {
    void* scratch = nullptr;
    const size_t off1 = (s.scratch[0] + 255) & ~(size_t)255;
    const size_t tot = off1 + s.scratch[1];
    if (s.scratch[0] + s.scratch[1] > 0) KFG_CK(cudaMallocAsync(&scratch, tot, st));
    int rc = KFG_OK;
    for (auto& step : s.steps) {
        void* roles[4] = {(void*)in, out, scratch, (char*)scratch + off1};
        step.args.in = roles[step.in_role];
        step.args.out = roles[step.out_role];
        step.args.fir_H = firH;
        if (allow_tma) enable_tma(step, step.args.in);
        cudaError_t e = launch_step(step, st);
        if (e != cudaSuccess) {
            rc = fail(KFG_ECUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
            break;
        }
    }
    if (scratch) cudaFreeAsync(scratch, st);
    return rc;
}

int esz_of(int dtype) { return cpx_size(dtype); }

// Build the schedule of one batched call; in/out element counts per
// transform are returned for staging.
int build_schedule(kfg_plan* p, long long batch, long long in_dist, long long in_stride, long long out_dist,
                   Schedule& s, size_t& in_bytes, size_t& out_bytes) {
    const int esz = esz_of(p->dtype), rsz = esz / 2;
    s = Schedule();
    switch (p->kind) {
        case K_C2C: {
            const long long n = p->n;
            if (!in_dist) in_dist = n * in_stride;
            if (!out_dist) out_dist = n;
            if (!schedule_c2c(p->main->p, batch, in_dist, in_stride, out_dist, s)) return fail(KFG_EINVAL, s.error);
            in_bytes = (size_t)((batch - 1) * in_dist + (n - 1) * in_stride + 1) * esz;
            out_bytes = (size_t)((batch - 1) * out_dist + n) * esz;
            return KFG_OK;
        }
        case K_REAL: {
            const long long nfft = p->n, nb = nfft / 2 + 1;
            if (!p->inverse) {
                if (!in_dist) in_dist = nfft;
                if (!out_dist) out_dist = nb;
                if (!schedule_r2c(p->main->p, batch, in_dist, out_dist, s)) return fail(KFG_EINVAL, s.error);
                in_bytes = (size_t)((batch - 1) * in_dist + nfft) * rsz;
                out_bytes = (size_t)((batch - 1) * out_dist + nb) * esz;
            } else {
                if (!in_dist) in_dist = nb;
                if (!out_dist) out_dist = nfft;
                if (!schedule_c2r(p->main->p, batch, in_dist, out_dist, s)) return fail(KFG_EINVAL, s.error);
                in_bytes = (size_t)((batch - 1) * in_dist + nb) * esz;
                out_bytes = (size_t)((batch - 1) * out_dist + nfft) * rsz;
            }
            return KFG_OK;
        }
        case K_ND: {
            const long long tot = p->n;
            if ((in_dist && in_dist != tot) || (out_dist && out_dist != tot))
                return fail(KFG_EINVAL, "N-D batches must be packed");
            const int nd = (int)p->dims.size();
            for (int k = 0; k < nd; ++k) {
                Schedule a;
                if (!schedule_axis(p->axes[k]->p, p->dims.data(), nd, k, batch, k == 0 ? 0 : 1, 1, a))
                    return fail(KFG_EINVAL, a.error);
                for (auto& st : a.steps) s.steps.push_back(st);
                s.scratch[0] = std::max(s.scratch[0], a.scratch[0]);  // two-pass axes, one after the other
            }
            in_bytes = out_bytes = (size_t)(batch * tot) * esz;
            return KFG_OK;
        }
        case K_NDR: {
            const int nd = (int)p->dims.size();
            const long long dr = p->dims[nd - 1], nb = dr / 2 + 1;
            long long other = 1;
            for (int i = 0; i < nd - 1; ++i) other *= p->dims[i];
            if ((in_dist && in_dist != (p->inverse ? other * nb : other * dr)) ||
                (out_dist && out_dist != (p->inverse ? other * dr : other * nb)))
                return fail(KFG_EINVAL, "N-D batches must be packed");
            std::vector<int> bd(p->dims.begin(), p->dims.end());
            bd[nd - 1] = (int)nb;
            if (!p->inverse) {
                if (!schedule_r2c(p->main->p, batch * other, dr, nb, s)) return fail(KFG_EINVAL, s.error);
                for (int k = 0; k < nd - 1; ++k) {
                    Schedule a;
                    if (!schedule_axis(p->axes[k]->p, bd.data(), nd, k, batch, 1, 1, a))
                        return fail(KFG_EINVAL, a.error);
                    for (auto& st : a.steps) s.steps.push_back(st);
                    // the real rows' scratch is free again once the axes run
                    s.scratch[0] = std::max(s.scratch[0], a.scratch[0]);
                }
                in_bytes = (size_t)(batch * other * dr) * rsz;
                out_bytes = (size_t)(batch * other * nb) * esz;
            } else {
                if (nd == 1) {
                    if (!schedule_c2r(p->main->p, batch, nb, dr, s)) return fail(KFG_EINVAL, s.error);
                } else {
                    size_t tmp = 0;
                    for (int k = 0; k < nd - 1; ++k) {
                        Schedule a;
                        // the half spectrum lives in role 2; a two-pass axis keeps its intermediate in role 3
                        if (!schedule_axis(p->axes[k]->p, bd.data(), nd, k, batch, k == 0 ? 0 : 2, 2, a, 3))
                            return fail(KFG_EINVAL, a.error);
                        for (auto& st : a.steps) s.steps.push_back(st);
                        tmp = std::max(tmp, a.scratch[1]);
                    }
                    Schedule c;
                    if (!schedule_c2r(p->main->p, batch * other, nb, dr, c, 2, 1)) return fail(KFG_EINVAL, c.error);
                    for (auto& st : c.steps) s.steps.push_back(st);
                    // role 2: the half spectrum, then (two-pass last axis) the
                    // c2r's own intermediate once its merge has read it;
                    // role 3: two-pass axis intermediates, then the merged rows
                    s.scratch[0] = std::max((size_t)(batch * other * nb) * esz, c.scratch[0]);
                    s.scratch[1] = std::max(tmp, c.scratch[1]);
                }
                in_bytes = (size_t)(batch * other * nb) * esz;
                out_bytes = (size_t)(batch * other * dr) * rsz;
            }
            return KFG_OK;
        }
    }
    return fail(KFG_EINVAL, "plan kind cannot run kfg_exec");
}

// Run a schedule with host-pointer staging where needed.
int exec_staged(Schedule& s, const void* in, void* out, size_t in_bytes, size_t out_bytes, cudaStream_t st,
                const void* firH = nullptr) {
    const bool din = is_device_ptr(in), dout = is_device_ptr(out);
    if (din && dout) return run_schedule(s, in, out, st, firH);
    if (zero_copy_enabled() && (din || is_pinned_host_ptr(in)) && (dout || is_pinned_host_ptr(out))) {
        // pinned host buffers: the passes read and write them in place over
        // the host link (no staging copies); bulk tile copies stay off
        int rc = run_schedule(s, in, out, st, firH, false);
        cudaError_t e = cudaStreamSynchronize(st);
        if (rc == KFG_OK && e != cudaSuccess)
            rc = fail(KFG_ECUDA, std::string("cudaStreamSynchronize: ") + cudaGetErrorString(e));
        return rc;
    }
    void *sin = (void*)in, *sout = out;
    if (!din) {
        KFG_CK(cudaMallocAsync(&sin, in_bytes, st));
        KFG_CK(cudaMemcpyAsync(sin, in, in_bytes, cudaMemcpyHostToDevice, st));
    }
    if (!dout) {
        if (!din && (const void*)out == in && out_bytes <= in_bytes)
            sout = sin;
        else
            KFG_CK(cudaMallocAsync(&sout, out_bytes, st));
    }
    int rc = run_schedule(s, sin, sout, st, firH);
    if (rc == KFG_OK && !dout) {
        cudaError_t e = cudaMemcpyAsync(out, sout, out_bytes, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) rc = fail(KFG_ECUDA, std::string("cudaMemcpyAsync(D2H): ") + cudaGetErrorString(e));
    }
    if (!din) cudaFreeAsync(sin, st);
    if (!dout && sout != sin) cudaFreeAsync(sout, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (rc == KFG_OK && e != cudaSuccess) rc = fail(KFG_ECUDA, std::string("cudaStreamSynchronize: ") + cudaGetErrorString(e));
    return rc;
}

bool valid_dtype(int d) { return d >= KFG_FLOAT && d <= KFG_INT32; }

constexpr size_t kSchedCache = 8;

void apply_tuned(kfg_plan* p, const std::string& key, Schedule& s);
std::string tune_key(long long batch, long long in_dist, long long out_dist);

// The schedule of a call of this shape: from the plan's cache, or built,
// tuned (for unit stride), its specialised kernels resolved, and cached.  A
// plain device-pointer call then costs little more than its launches.
int get_schedule(kfg_plan* p, long long batch, long long in_dist, long long in_stride, long long out_dist,
                 std::shared_ptr<const CachedSched>& out) {
    {
        std::lock_guard<std::mutex> lk(p->sched_mu);
        for (size_t i = 0; i < p->scheds.size(); ++i) {
            const auto& c = p->scheds[i];
            if (c->batch == batch && c->in_dist == in_dist && c->in_stride == in_stride && c->out_dist == out_dist) {
                out = c;
                if (i) std::rotate(p->scheds.begin(), p->scheds.begin() + i, p->scheds.begin() + i + 1);
                return KFG_OK;
            }
        }
    }
    auto c = std::make_shared<CachedSched>();
    c->batch = batch;
    c->in_dist = in_dist;
    c->in_stride = in_stride;
    c->out_dist = out_dist;
    int rc = build_schedule(p, batch, in_dist, in_stride, out_dist, c->s, c->ib, c->ob);
    if (rc) return rc;
    if (in_stride == 1) apply_tuned(p, tune_key(batch, in_dist, out_dist), c->s);
    c->multi = c->s.steps.size() > 1;
    for (auto& st : c->s.steps) {
        c->multi |= st.args.col_in || st.args.col_out;
        if (st.kind == 0 && specialize_enabled()) {
            std::string err;
            st.kfn = spec_kernel(st, err);  // null: the precompiled kernels run
        }
    }
    out = c;
    std::lock_guard<std::mutex> lk(p->sched_mu);
    p->scheds.insert(p->scheds.begin(), c);
    if (p->scheds.size() > kSchedCache) p->scheds.resize(kSchedCache);
    return KFG_OK;
}

void drop_schedules(kfg_plan* p) {
    std::lock_guard<std::mutex> lk(p->sched_mu);
    p->scheds.clear();
}

std::string tune_key(long long batch, long long in_dist, long long out_dist) {
    std::ostringstream o;
    o << batch << "/" << in_dist << "/" << out_dist;
    return o.str();
}

void apply_cfgs(Schedule& s, const std::vector<std::array<int, 6>>& v) {
    size_t k = 0;
    for (auto& st : s.steps) {
        if (st.kind != 0) continue;
        if (k >= v.size()) break;
        const auto& c = v[k++];
        if (c[3] && !st.args.col_in) recolumn_step(st);
        if (c[0] != st.cfg.J) reshape_step(st, c[0]);
        if (c[4] && c[4] != st.cfg.T) retarget_threads(st, c[4]);
        // the tuning file is plain text on disk: take only budgets a launch can have
        if (c[1] >= 1 && c[1] <= 32) st.cfg.minb = c[1];
        st.tma_ok = c[2] != 0;
        if (c[5] >= SWZ_FOLD && c[5] <= SWZ_ONE) st.args.swz = c[5];
        st.kfn = nullptr;
    }
}

void apply_tuned(kfg_plan* p, const std::string& key, Schedule& s) {
    std::lock_guard<std::mutex> lk(p->tune_mu);
    auto it = p->tuned.find(key);
    if (it != p->tuned.end()) apply_cfgs(s, it->second);
}

// Signature of a plan for the on-disk tuning cache.
std::string plan_sig(const kfg_plan* p) {
    std::ostringstream o;
    o << p->kind << ":" << p->dtype << ":" << p->inverse << ":" << p->n;
    for (int d : p->dims) o << "x" << d;
    char name[256] = {0};
    cudaDeviceProp prop;
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaGetDeviceProperties(&prop, dev) == cudaSuccess)
        snprintf(name, sizeof(name), "%s", prop.name);
    for (char* c = name; *c; ++c)
        if (*c == ' ') *c = '_';
    o << ":" << name << ":spec" << (specialize_enabled() ? 1 : 0) << ":v6";
    return o.str();
}

std::string tune_file() {
    const char* e = getenv("KISSFFT_GB300_CACHE");
    std::string d;
    if (e && *e)
        d = e;
    else {
        const char* home = getenv("HOME");
        d = std::string(home && *home ? home : "/tmp") + "/.cache/kissfft_gb300";
    }
    return d + "/tune.txt";
}

bool tune_load(const std::string& key, std::vector<std::array<int, 6>>& v) {
    std::ifstream f(tune_file());
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {
        size_t sp = line.find(' ');
        if (sp == std::string::npos || line.compare(0, sp, key) != 0 || sp != key.size()) continue;
        std::istringstream is(line.substr(sp + 1));
        std::vector<std::array<int, 6>> r;
        std::array<int, 6> c;
        while (is >> c[0] >> c[1] >> c[2] >> c[3] >> c[4] >> c[5]) r.push_back(c);
        v = r;
        found = true;  // the last line for a key wins
    }
    return found;
}

void tune_store(const std::string& key, const std::vector<std::array<int, 6>>& v) {
    std::string path = tune_file();
    std::string dir = path.substr(0, path.rfind('/'));
    std::string cmd;
    for (size_t i = 1; i <= dir.size(); ++i)
        if (i == dir.size() || dir[i] == '/') mkdir(dir.substr(0, i).c_str(), 0755);
    std::ofstream f(path, std::ios::app);
    f << key;
    for (auto& c : v) f << " " << c[0] << " " << c[1] << " " << c[2] << " " << c[3] << " " << c[4] << " " << c[5];
    f << "\n";
}

float time_step(Step& st, void* const roles[4], cudaStream_t strm, cudaEvent_t e0, cudaEvent_t e1, int reps) {
    st.args.in = roles[st.in_role];
    st.args.out = roles[st.out_role];
    st.args.tma = 0;
    enable_tma(st, st.args.in);
    if (launch_step(st, strm) != cudaSuccess) return -1.f;
    float best = -1.f;
    for (int r = 0; r < reps; ++r) {
        cudaEventRecord(e0, strm);
        launch_step(st, strm);
        cudaEventRecord(e1, strm);
        if (cudaEventSynchronize(e1) != cudaSuccess) return -1.f;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (best < 0 || ms < best) best = ms;
    }
    return best;
}

}  // namespace

extern "C" {

kfg_plan* kfg_plan_c2c(int dtype, int nfft, int inverse) {
    if (!valid_dtype(dtype) || nfft < 1) {
        fail(KFG_EINVAL, "kfg_plan_c2c: bad sample type or size");
        return nullptr;
    }
    std::unique_ptr<kfg_plan> p(new kfg_plan);
    p->kind = K_C2C;
    p->dtype = dtype;
    p->inverse = inverse ? 1 : 0;
    p->n = nfft;
    p->main = make_devplan(dtype, nfft, p->inverse, 0);
    if (!p->main) return nullptr;
    return p.release();
}

kfg_plan* kfg_plan_real(int dtype, int nfft, int inverse) {
    if (!valid_dtype(dtype) || nfft < 2 || (nfft & 1)) {
        // kiss_fftr_alloc rejects odd sizes (kiss_fftr.c:29-32)
        fail(KFG_EINVAL, "Real FFT optimization must be even.");
        return nullptr;
    }
    std::unique_ptr<kfg_plan> p(new kfg_plan);
    p->kind = K_REAL;
    p->dtype = dtype;
    p->inverse = inverse ? 1 : 0;
    p->n = nfft;
    p->main = make_devplan(dtype, nfft / 2, p->inverse, nfft);
    if (!p->main) return nullptr;
    return p.release();
}

kfg_plan* kfg_plan_nd(int dtype, const int* dims, int ndims, int inverse) {
    if (!valid_dtype(dtype) || !dims || ndims < 1) {
        fail(KFG_EINVAL, "kfg_plan_nd: bad arguments");
        return nullptr;
    }
    std::unique_ptr<kfg_plan> p(new kfg_plan);
    p->kind = K_ND;
    p->dtype = dtype;
    p->inverse = inverse ? 1 : 0;
    p->n = 1;
    for (int i = 0; i < ndims; ++i) {
        if (dims[i] < 1) {
            fail(KFG_EINVAL, "kfg_plan_nd: dimension < 1");
            return nullptr;
        }
        p->dims.push_back(dims[i]);
        p->n *= dims[i];
        p->axes.push_back(make_devplan(dtype, dims[i], p->inverse, 0));
        if (!p->axes.back()) return nullptr;
    }
    return p.release();
}

kfg_plan* kfg_plan_ndr(int dtype, const int* dims, int ndims, int inverse) {
    if (!valid_dtype(dtype) || !dims || ndims < 1 || dims[ndims - 1] < 2 || (dims[ndims - 1] & 1)) {
        fail(KFG_EINVAL, "kfg_plan_ndr: bad arguments (the last dimension must be even)");
        return nullptr;
    }
    std::unique_ptr<kfg_plan> p(new kfg_plan);
    p->kind = K_NDR;
    p->dtype = dtype;
    p->inverse = inverse ? 1 : 0;
    p->n = 1;
    for (int i = 0; i < ndims; ++i) {
        if (dims[i] < 1) {
            fail(KFG_EINVAL, "kfg_plan_ndr: dimension < 1");
            return nullptr;
        }
        p->dims.push_back(dims[i]);
        p->n *= dims[i];
    }
    p->main = make_devplan(dtype, dims[ndims - 1] / 2, p->inverse, dims[ndims - 1]);
    if (!p->main) return nullptr;
    for (int i = 0; i < ndims - 1; ++i) {
        p->axes.push_back(make_devplan(dtype, dims[i], p->inverse, 0));
        if (!p->axes.back()) return nullptr;
    }
    return p.release();
}

kfg_plan* kfg_plan_fir(const float* taps, size_t ntaps, size_t nfft, size_t* nfft_out) {
    if (!taps || ntaps < 1) {
        fail(KFG_EINVAL, "kfg_plan_fir: no taps");
        return nullptr;
    }
    if (nfft == 0) {
        // block size rule of kiss_fastfir_alloc (tools/kiss_fastfir.c:75-87)
        size_t i = ntaps - 1;
        nfft = 2;
        do {
            nfft <<= 1;
        } while (i >>= 1);
        if (nfft < 2048) nfft = 2048;
    }
    if (nfft_out) *nfft_out = nfft;
    if ((nfft & 1) || nfft < ntaps || nfft > (size_t)1 << 30) {
        fail(KFG_EINVAL, "kfg_plan_fir: block size must be even and at least the filter length");
        return nullptr;
    }
    std::unique_ptr<kfg_plan> p(new kfg_plan);
    p->kind = K_FIR;
    p->dtype = KFG_FLOAT;
    p->n = (long long)nfft;
    p->ntaps = (long long)ntaps;
    p->main = make_devplan(KFG_FLOAT, (int)nfft / 2, 0, (int)nfft);
    if (!p->main) return nullptr;
    p->aux = make_devplan(KFG_FLOAT, (int)nfft / 2, 1, (int)nfft);
    if (!p->aux) return nullptr;
    // taps rotated left by ntaps-1 so the scrap lands at the block tail
    // (tools/kiss_fastfir.c:142-148), transformed, scaled by float(1/nfft)
    std::vector<float> rot(nfft, 0.0f);
    rot[0] = taps[ntaps - 1];
    for (size_t i = 0; i + 1 < ntaps; ++i) rot[nfft - ntaps + 1 + i] = taps[i];
    const size_t nb = nfft / 2 + 1;
    cudaStream_t st = g_stream.load();
    void* d_rot = nullptr;
    if (cudaMalloc(&p->d_H, nb * 8) != cudaSuccess || cudaMalloc(&d_rot, nfft * 4) != cudaSuccess) {
        if (d_rot) cudaFree(d_rot);
        fail(KFG_ENOMEM, "kfg_plan_fir: device allocation failed");
        return nullptr;
    }
    int rc = KFG_OK;
    if (cudaMemcpy(d_rot, rot.data(), nfft * 4, cudaMemcpyHostToDevice) != cudaSuccess) rc = KFG_ECUDA;
    Schedule s;
    if (rc == KFG_OK && !schedule_r2c(p->main->p, 1, (long long)nfft, (long long)nb, s)) rc = fail(KFG_EINVAL, s.error);
    if (rc == KFG_OK) rc = run_schedule(s, d_rot, p->d_H, st);
    if (rc == KFG_OK) {
        float scale = 1.0 / (double)nfft;
        kf_scale_kernel<<<(unsigned)((2 * nb + 255) / 256), 256, 0, st>>>((float*)p->d_H, (long long)(2 * nb), scale);
        if (cudaStreamSynchronize(st) != cudaSuccess) rc = fail(KFG_ECUDA, "kfg_plan_fir: response kernel failed");
    }
    cudaFree(d_rot);
    if (rc != KFG_OK) return nullptr;
    return p.release();
}

void kfg_plan_free(kfg_plan* p) { delete p; }

}  // extern "C"

namespace {

// Streams, events and a ring of device buffers for pipelined host calls,
// one set per host thread.
struct HostPipe {
    static constexpr int kSlots = 3;
    cudaStream_t h2d = nullptr, comp = nullptr, d2h = nullptr;
    cudaEvent_t start = nullptr, ev_in[kSlots] = {}, ev_comp[kSlots] = {}, ev_out[kSlots] = {};
    unsigned char *din = nullptr, *dout = nullptr;  // ring, kept between calls
    size_t din_cap = 0, dout_cap = 0;
    bool ok = false;
    bool reserve(size_t in_bytes, size_t out_bytes) {
        if (in_bytes > din_cap) {
            if (din) cudaFree(din);
            din = nullptr;
            din_cap = 0;
            if (cudaMalloc((void**)&din, in_bytes) != cudaSuccess) return false;
            din_cap = in_bytes;
        }
        if (out_bytes > dout_cap) {
            if (dout) cudaFree(dout);
            dout = nullptr;
            dout_cap = 0;
            if (cudaMalloc((void**)&dout, out_bytes) != cudaSuccess) return false;
            dout_cap = out_bytes;
        }
        return true;
    }
    HostPipe() {
        ok = cudaStreamCreateWithFlags(&h2d, cudaStreamNonBlocking) == cudaSuccess &&
             cudaStreamCreateWithFlags(&comp, cudaStreamNonBlocking) == cudaSuccess &&
             cudaStreamCreateWithFlags(&d2h, cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&start, cudaEventDisableTiming) == cudaSuccess;
        for (int k = 0; k < kSlots && ok; ++k)
            ok = cudaEventCreateWithFlags(&ev_in[k], cudaEventDisableTiming) == cudaSuccess &&
                 cudaEventCreateWithFlags(&ev_comp[k], cudaEventDisableTiming) == cudaSuccess &&
                 cudaEventCreateWithFlags(&ev_out[k], cudaEventDisableTiming) == cudaSuccess;
    }
};

// A large packed 1-D batch on page-locked host buffers, in chunks of about
// 32 MiB: chunk i+1's copy in, chunk i's kernels and chunk i-1's copy out
// run at the same time on three streams (both directions of the host link
// busy at once), through a ring of three device buffers per side kept per
// host thread.  Returns 1 when the call does not qualify (the caller takes
// another path).
int exec_pipelined(kfg_plan* p, const void* in, void* out, long long batch, long long in_dist, long long out_dist,
                   cudaStream_t caller) {
    if (p->kind != K_C2C && p->kind != K_REAL) return 1;
    const long long n = p->n, nb = n / 2 + 1;
    const int esz = esz_of(p->dtype), rsz = esz / 2;
    long long in_frame, out_frame;  // bytes of one transform
    if (p->kind == K_C2C)
        in_frame = out_frame = n * esz;
    else if (!p->inverse)
        in_frame = n * rsz, out_frame = nb * esz;
    else
        in_frame = nb * esz, out_frame = n * rsz;
    const long long in_elem = p->kind == K_C2C || p->inverse ? esz : rsz;
    const long long out_elem = p->kind == K_C2C || !p->inverse ? esz : rsz;
    if ((in_dist && in_dist * in_elem != in_frame) || (out_dist && out_dist * out_elem != out_frame)) return 1;
    const long long cb = std::max(1LL, (32LL << 20) / std::max(in_frame, out_frame));
    const long long nch = (batch + cb - 1) / cb;
    if (nch < 4) return 1;
    thread_local HostPipe pipe;
    if (!pipe.ok) return 1;
    const int S = HostPipe::kSlots;
    // the previous call on this thread has finished (it synchronised), so
    // the ring may be regrown here
    if (!pipe.reserve((size_t)(S * cb * in_frame), (size_t)(S * cb * out_frame)))
        return fail(KFG_ENOMEM, "pipelined host call: device ring");
    unsigned char *din = pipe.din, *dout = pipe.dout;
    KFG_CK(cudaEventRecord(pipe.start, caller));
    KFG_CK(cudaStreamWaitEvent(pipe.h2d, pipe.start, 0));
    KFG_CK(cudaStreamWaitEvent(pipe.comp, pipe.start, 0));
    KFG_CK(cudaStreamWaitEvent(pipe.d2h, pipe.start, 0));
    int rc = KFG_OK;
    for (long long i = 0; i < nch && rc == KFG_OK; ++i) {
        const int k = (int)(i % S);
        const long long b0 = i * cb, nbt = std::min(cb, batch - b0);
        unsigned char* di = din + (size_t)k * cb * in_frame;
        unsigned char* dq = dout + (size_t)k * cb * out_frame;
        Schedule s;
        size_t ib = 0, ob = 0;
        rc = build_schedule(p, nbt, 0, 1, 0, s, ib, ob);
        if (rc) break;
        cudaError_t e = cudaSuccess;
        if (i >= S) e = cudaStreamWaitEvent(pipe.h2d, pipe.ev_comp[k], 0);  // slot's input consumed
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(di, (const unsigned char*)in + b0 * in_frame, (size_t)(nbt * in_frame),
                                cudaMemcpyHostToDevice, pipe.h2d);
        if (e == cudaSuccess) e = cudaEventRecord(pipe.ev_in[k], pipe.h2d);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(pipe.comp, pipe.ev_in[k], 0);
        if (e == cudaSuccess && i >= S) e = cudaStreamWaitEvent(pipe.comp, pipe.ev_out[k], 0);  // output copied out
        if (e != cudaSuccess) {
            rc = fail(KFG_ECUDA, std::string("pipelined copy in: ") + cudaGetErrorString(e));
            break;
        }
        rc = run_schedule(s, di, dq, pipe.comp);
        if (rc) break;
        e = cudaEventRecord(pipe.ev_comp[k], pipe.comp);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(pipe.d2h, pipe.ev_comp[k], 0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync((unsigned char*)out + b0 * out_frame, dq, (size_t)(nbt * out_frame),
                                cudaMemcpyDeviceToHost, pipe.d2h);
        if (e == cudaSuccess) e = cudaEventRecord(pipe.ev_out[k], pipe.d2h);
        if (e != cudaSuccess) rc = fail(KFG_ECUDA, std::string("pipelined copy out: ") + cudaGetErrorString(e));
    }
    cudaError_t e1 = cudaStreamSynchronize(pipe.h2d), e2 = cudaStreamSynchronize(pipe.d2h),
                e3 = cudaStreamSynchronize(pipe.comp);
    if (rc == KFG_OK && (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess))
        rc = fail(KFG_ECUDA, "pipelined host call failed");
    return rc;
}

}  // namespace

extern "C" {

int kfg_exec_batch(kfg_plan* p, const void* in, void* out, long long batch, long long in_dist, long long out_dist,
                   void* stream) {
    if (!p || !in || !out || batch < 0) return fail(KFG_EINVAL, "kfg_exec_batch: bad arguments");
    if (batch == 0) return KFG_OK;
    if (p->kind == K_FIR) return fail(KFG_EINVAL, "use kfg_fir_filter for a fast FIR plan");
    std::shared_ptr<const CachedSched> c;
    int rc = get_schedule(p, batch, in_dist, 1, out_dist, c);
    if (rc) return rc;
    // pinned host buffers: kernels that read whole rows in one pass use
    // them in place (zero-copy); schedules of several steps or column tiles
    // (short runs per row over the host link) take the copy pipeline
    if (c->multi && pipeline_enabled() && is_pinned_host_ptr(in) && is_pinned_host_ptr(out) &&
        (const void*)out != in) {
        rc = exec_pipelined(p, in, out, batch, in_dist, out_dist, pick(stream));
        if (rc != 1) return rc;
    }
    Schedule s = c->s;  // the executor writes buffer pointers into its copy
    return exec_staged(s, in, out, c->ib, c->ob, pick(stream));
}

int kfg_exec(kfg_plan* p, const void* in, void* out, void* stream) { return kfg_exec_batch(p, in, out, 1, 0, 0, stream); }

int kfg_exec_stride(kfg_plan* p, const void* in, void* out, int in_stride, void* stream) {
    if (!p || !in || !out || in_stride < 1) return fail(KFG_EINVAL, "kfg_exec_stride: bad arguments");
    if (p->kind != K_C2C) return fail(KFG_EINVAL, "kfg_exec_stride needs a complex 1-D plan");
    std::shared_ptr<const CachedSched> c;
    int rc = get_schedule(p, 1, 0, in_stride, 0, c);
    if (rc) return rc;
    Schedule s = c->s;
    return exec_staged(s, in, out, c->ib, c->ob, pick(stream));
}

int kfg_fir_filter(kfg_plan* p, const float* x, size_t nx, float* y, size_t* ny_out, void* stream) {
    if (!p || p->kind != K_FIR || !x || !y) return fail(KFG_EINVAL, "kfg_fir_filter: bad arguments");
    if ((long long)nx < p->ntaps - 1) return fail(KFG_EINVAL, "kfg_fir_filter: signal shorter than the filter transient");
    const long long nout = (long long)nx - p->ntaps + 1;
    if (ny_out) *ny_out = (size_t)nout;
    if (nout == 0) return KFG_OK;
    Schedule s;
    if (!schedule_fastfir(p->main->p, p->aux->p, p->ntaps, (long long)nx, 0, s)) return fail(KFG_EINVAL, s.error);
    return exec_staged(s, x, y, nx * sizeof(float), (size_t)nout * sizeof(float), pick(stream), p->d_H);
}

int kfg_pack_real(int dtype, const void* bins, void* dst, long long n, int conj, void* stream) {
    if ((dtype != KFG_FLOAT && dtype != KFG_DOUBLE) || !bins || !dst || n < 1)
        return fail(KFG_EINVAL, "kfg_pack_real: float or double bins and n >= 1");
    if (!is_device_ptr(bins) || !is_device_ptr(dst)) return fail(KFG_EINVAL, "kfg_pack_real: device pointers only");
    const cudaStream_t st = pick(stream);
    const unsigned grid = (unsigned)((n + 255) / 256);
    if (dtype == KFG_FLOAT)
        kf_pack_real_kernel<float><<<grid, 256, 0, st>>>((const float*)bins, (float*)dst, n, conj);
    else
        kf_pack_real_kernel<double><<<grid, 256, 0, st>>>((const double*)bins, (double*)dst, n, conj);
    KFG_CK(cudaGetLastError());
    return KFG_OK;
}

int kfg_psd(kfg_plan* p, const short* samples, long long nsamples, int stereo, int remove_dc, int navg, float* rows,
            long long* nrows_out, void* stream) {
    if (!p || p->kind != K_REAL || p->inverse || p->dtype != KFG_FLOAT || !samples || !rows || navg < 1 || nsamples < 0)
        return fail(KFG_EINVAL, "kfg_psd: a forward float real plan, samples, rows and navg >= 1");
    const long long nfft = p->n, nfreqs = nfft / 2 + 1;
    const long long nrows = nsamples / nfft / navg, nframes = nrows * navg;  // whole rows only
    if (nrows_out) *nrows_out = nrows;
    if (nrows == 0) return KFG_OK;
    const cudaStream_t st = pick(stream);
    const bool din = is_device_ptr(samples), dout = is_device_ptr(rows);
    const size_t in_bytes = (size_t)nframes * nfft * (stereo ? 2 : 1) * sizeof(short);
    const size_t t_bytes = (size_t)nframes * nfft * sizeof(float), b_bytes = (size_t)nframes * nfreqs * 8;
    const size_t r_bytes = (size_t)nrows * nfreqs * sizeof(float);
    void *d_in = (void*)samples, *d_t = nullptr, *d_b = nullptr, *d_rows = rows;
    KFG_CK(cudaMallocAsync(&d_t, t_bytes, st));
    KFG_CK(cudaMallocAsync(&d_b, b_bytes, st));
    if (!din) {
        KFG_CK(cudaMallocAsync(&d_in, in_bytes, st));
        KFG_CK(cudaMemcpyAsync(d_in, samples, in_bytes, cudaMemcpyHostToDevice, st));
    }
    if (!dout) KFG_CK(cudaMallocAsync(&d_rows, r_bytes, st));
    kf_psd_prep_kernel<<<(unsigned)nframes, 256, 0, st>>>((const short*)d_in, (float*)d_t, (int)nfft, stereo ? 1 : 0,
                                                          remove_dc ? 1 : 0);
    int rc = KFG_OK;
    if (cudaGetLastError() != cudaSuccess) rc = fail(KFG_ECUDA, "kfg_psd: frame kernel");
    Schedule s;
    size_t ib = 0, ob = 0;
    if (rc == KFG_OK) rc = build_schedule(p, nframes, 0, 1, 0, s, ib, ob);
    if (rc == KFG_OK) rc = run_schedule(s, d_t, d_b, st);
    if (rc == KFG_OK) {
        const long long items = nrows * nfreqs;
        kf_psd_reduce_kernel<<<(unsigned)((items + 255) / 256), 256, 0, st>>>((const float*)d_b, (float*)d_rows, nrows,
                                                                              (int)nfreqs, navg);
        if (cudaGetLastError() != cudaSuccess) rc = fail(KFG_ECUDA, "kfg_psd: row kernel");
    }
    if (rc == KFG_OK && !dout) {
        cudaError_t e = cudaMemcpyAsync(rows, d_rows, r_bytes, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) rc = fail(KFG_ECUDA, std::string("kfg_psd: D2H: ") + cudaGetErrorString(e));
    }
    cudaFreeAsync(d_t, st);
    cudaFreeAsync(d_b, st);
    if (!din) cudaFreeAsync(d_in, st);
    if (!dout) cudaFreeAsync(d_rows, st);
    if (!din || !dout) {
        cudaError_t e = cudaStreamSynchronize(st);
        if (rc == KFG_OK && e != cudaSuccess) rc = fail(KFG_ECUDA, std::string("kfg_psd: ") + cudaGetErrorString(e));
    }
    return rc;
}

int kfg_set_stream(void* stream) {
    g_stream.store((cudaStream_t)stream);
    return KFG_OK;
}

void* kfg_get_stream(void) { return (void*)g_stream.load(); }

int kfg_synchronize(void) {
    KFG_CK(cudaStreamSynchronize(g_stream.load()));
    return KFG_OK;
}

const char* kfg_last_error(void) { return g_err.c_str(); }

int kfg_next_fast_size(int n) { return next_fast_size(n); }

int kfg_set_tma(int on) {
    set_tma_enabled(on);
    return KFG_OK;
}

int kfg_set_specialize(int on) {
    set_specialize(on);
    return KFG_OK;
}

int kfg_plan_prepare(kfg_plan* p, long long batch, long long in_dist, long long out_dist) {
    if (!p || batch < 1) return fail(KFG_EINVAL, "kfg_plan_prepare: bad arguments");
    if (!specialize_enabled()) return KFG_OK;
    Schedule s;
    size_t ib = 0, ob = 0;
    int rc = KFG_OK;
    if (p->kind == K_FIR) {
        const long long nx = batch;  // signal length for a FIR plan
        if (!schedule_fastfir(p->main->p, p->aux->p, p->ntaps, nx, 0, s)) return fail(KFG_EINVAL, s.error);
    } else {
        rc = build_schedule(p, batch, in_dist, 1, out_dist, s, ib, ob);
        if (rc) return rc;
        apply_tuned(p, tune_key(batch, in_dist, out_dist), s);
    }
    std::vector<std::string> errs(s.steps.size());
    std::vector<std::thread> th;
    for (size_t i = 0; i < s.steps.size(); ++i) {
        if (s.steps[i].kind != 0) continue;
        th.emplace_back([&, i]() {
            if (!spec_kernel(s.steps[i], errs[i]) && errs[i].empty()) errs[i] = "specialised kernel unavailable";
        });
    }
    for (auto& t : th) t.join();
    for (auto& e : errs)
        if (!e.empty()) return fail(KFG_EUNSUPPORTED, e);
    return KFG_OK;
}

int kfg_autotune(kfg_plan* p, long long batch, long long in_dist, long long out_dist) {
    if (!p || batch < 1 || p->kind == K_FIR) return fail(KFG_EINVAL, "kfg_autotune: bad arguments");
    const std::string key = tune_key(batch, in_dist, out_dist);
    const std::string dkey = plan_sig(p) + ":" + key;
    std::vector<std::array<int, 6>> best;
    if (tune_load(dkey, best)) {
        {
            std::lock_guard<std::mutex> lk(p->tune_mu);
            p->tuned[key] = best;
        }
        drop_schedules(p);
        return KFG_OK;
    }
    Schedule s;
    size_t ib = 0, ob = 0;
    int rc = build_schedule(p, batch, in_dist, 1, out_dist, s, ib, ob);
    if (rc) return rc;
    void *din = nullptr, *dout = nullptr, *scr = nullptr;
    const size_t off1 = (s.scratch[0] + 255) & ~(size_t)255;
    if (cudaMalloc(&din, ib) != cudaSuccess || cudaMalloc(&dout, ob) != cudaSuccess ||
        (s.scratch[0] + s.scratch[1] > 0 && cudaMalloc(&scr, off1 + s.scratch[1]) != cudaSuccess)) {
        cudaFree(din);
        cudaFree(dout);
        return fail(KFG_ENOMEM, "kfg_autotune: no room for the tuning buffers");
    }
    cudaMemset(din, 0, ib);
    void* roles[4] = {din, dout, scr, (char*)scr + off1};
    cudaStream_t strm;
    cudaEvent_t e0, e1;
    cudaStreamCreate(&strm);
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int nsm = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    for (auto& st0 : s.steps) {
        if (st0.kind != 0) continue;
        std::vector<Step> cands;
        const int J0 = st0.cfg.J;
        // a launch with few tiles for the SMs (small batches, N-D axes) runs
        // about one wave, as long as one tile's latency: narrower tiles too
        const bool few_tiles = (st0.args.G + J0 - 1) / J0 < 4LL * std::max(nsm, 1);
        // row-mode steps also try column-layout tiles with 2..8 jobs
        Step colst = st0;
        const bool can_col = recolumn_step(colst);
        for (int col = 0; col <= (can_col ? 1 : 0); ++col) {
            const Step& base = col ? colst : st0;
            std::vector<int> Js = col ? std::vector<int>{2, 4, 8} : std::vector<int>{J0 / 2, J0, J0 * 2, J0 * 4};
            if (few_tiles && !col) {
                Js.push_back(J0 / 4);
                Js.push_back(J0 / 8);
            }
            for (int J : Js) {
                Step c = base;
                if (J < 1 || (J != base.cfg.J && !reshape_step(c, J))) continue;
                const int m0 = c.cfg.minb;
                // register budgets: none, the default, a little and a lot
                // tighter, and the occupancy that threads and shared memory allow
                const int maxb = std::max(1, std::min(std::min(2048 / std::max(c.cfg.T, 32),
                                                               (227 * 1024) / std::max(c.cfg.smem + 1024, 1)),
                                                      32));
                for (int mb : {1, m0, m0 + 1, m0 + 2, 2 * m0, maxb}) {
                    if (mb < 1 || mb > maxb) continue;
                    bool dup = false;
                    for (auto& d : cands)
                        dup |= (d.cfg.J == c.cfg.J && d.cfg.T == c.cfg.T && d.cfg.minb == mb &&
                                d.args.col_in == c.args.col_in);
                    if (dup) continue;
                    Step cm = c;
                    cm.cfg.minb = mb;
                    cands.push_back(cm);
                }
                // thread counts that fit one pass's groups in one or two
                // rounds (passes with uneven group counts leave threads idle)
                const KSub& sb = c.args.sub[0];
                for (int pi = 0; pi < sb.npass; ++pi) {
                    const long long G = (long long)c.cfg.J * sb.ps[pi].H * sb.ps[pi].ML;
                    for (int r = 1; r <= 2; ++r) {
                        const int T = (int)(((G + r - 1) / r + 31) / 32 * 32);
                        Step ct = c;
                        if (T == c.cfg.T || !retarget_threads(ct, T)) continue;
                        bool dup = false;
                        for (auto& d : cands)
                            dup |= (d.cfg.J == ct.cfg.J && d.cfg.T == ct.cfg.T && d.cfg.minb == ct.cfg.minb &&
                                    d.args.col_in == ct.args.col_in);
                        if (!dup) cands.push_back(ct);
                    }
                }
            }
        }
        if (specialize_enabled()) {
            // compile the candidates' kernels in parallel
            std::vector<std::thread> th;
            for (auto& c : cands)
                th.emplace_back([&c]() {
                    std::string err;
                    spec_kernel(c, err);
                });
            for (auto& t : th) t.join();
        }
        float bt = -1.f;
        std::array<int, 6> bc = {st0.cfg.J, st0.cfg.minb, 1, st0.args.col_in, st0.cfg.T, st0.args.swz};
        Step bstep = st0;
        for (auto& c : cands) {
            for (int tma = 1; tma >= 0; --tma) {
                Step x = c;
                x.tma_ok = tma;
                const Step untimed = x;  // time_step adds the staging buffer to x's shared memory
                float ms = time_step(x, roles, strm, e0, e1, 3);
                if (ms > 0 && (bt < 0 || ms < bt)) {
                    bt = ms;
                    bc = {c.cfg.J, c.cfg.minb, tma, c.args.col_in, c.cfg.T, c.args.swz};
                    bstep = untimed;
                }
                if (!x.args.tma) break;  // staging not eligible: one timing is enough
            }
        }
        // the winner's shape with the other shared-tile index maps
        if (bt > 0) {
            std::vector<Step> sw;
            for (int m = SWZ_FOLD; m <= SWZ_ONE; ++m) {
                if (m == bstep.args.swz) continue;
                Step x = bstep;
                x.args.swz = m;
                sw.push_back(x);
            }
            if (specialize_enabled()) {
                std::vector<std::thread> th;
                for (auto& c : sw)
                    th.emplace_back([&c]() {
                        std::string err;
                        spec_kernel(c, err);
                    });
                for (auto& t : th) t.join();
            }
            for (auto& x : sw) {
                float ms = time_step(x, roles, strm, e0, e1, 3);
                if (ms > 0 && ms < bt) {
                    bt = ms;
                    bc[5] = x.args.swz;
                }
            }
        }
        best.push_back(bc);
        // later steps read what this one wrote: run it once with the winner
        Step w = st0;
        std::vector<std::array<int, 6>> one = {bc};
        Schedule tmp;
        tmp.steps.push_back(w);
        apply_cfgs(tmp, one);
        time_step(tmp.steps[0], roles, strm, e0, e1, 1);
    }
    cudaStreamSynchronize(strm);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(strm);
    cudaFree(din);
    cudaFree(dout);
    if (scr) cudaFree(scr);
    {
        std::lock_guard<std::mutex> lk(p->tune_mu);
        p->tuned[key] = best;
    }
    drop_schedules(p);
    tune_store(dkey, best);
    return KFG_OK;
}

int kfg_specialize_check(int dtype, int real, int n, int inverse, long long batch) {
    Plan p;
    if (!p.build(dtype, real ? n / 2 : n, inverse, 0, real ? n : 0)) return fail(KFG_EINVAL, p.error);
    Schedule s;
    bool ok = real ? (inverse ? schedule_c2r(p, batch, n / 2 + 1, n, s) : schedule_r2c(p, batch, n, n / 2 + 1, s))
                   : schedule_c2c(p, batch, n, 1, n, s);
    if (!ok) return fail(KFG_EINVAL, s.error);
    for (auto& st : s.steps) {
        if (st.kind != 0) continue;
        std::string err;
        if (!spec_compile_only(st, err)) return fail(KFG_EUNSUPPORTED, err);
    }
    return KFG_OK;
}

int kfg_plan_info(const kfg_plan* p, int* out, int nout) {
    if (!p || !out) return KFG_EINVAL;
    int v[6] = {p->kind, p->dtype, (int)p->n, 0, 0, 0};
    const DevPlan* d = p->main ? p->main.get() : (p->axes.empty() ? nullptr : p->axes[0].get());
    if (d) {
        v[3] = d->p.nsub;
        v[4] = sub_family(d->p.sub[0]);
        v[5] = d->p.sub[0].L;
    }
    for (int i = 0; i < nout && i < 6; ++i) out[i] = v[i];
    return KFG_OK;
}

long long kfg_plan_table(const kfg_plan* p, int which, void* host, size_t bytes) {
    if (!p || !p->main || (p->kind != K_C2C && p->kind != K_REAL) || which < 0 || which > 1)
        return fail(KFG_EINVAL, "kfg_plan_table: needs a complex or real 1-D plan and table 0 or 1");
    const DevPlan& d = *p->main;
    const size_t esz = (size_t)esz_of(p->dtype);
    size_t off = 0, count = 0;
    if (which == 0) {
        off = d.p.off_tw_full;
        count = (size_t)d.p.n * esz;
    } else {
        if (d.p.real_nfft <= 0) return fail(KFG_EINVAL, "kfg_plan_table: super twiddles belong to real plans");
        off = d.p.off_super;
        count = (size_t)(d.p.n / 2) * esz;
    }
    if (host && bytes) {
        const size_t nb = bytes < count ? bytes : count;
        cudaError_t e = cudaMemcpy(host, (const char*)d.d + off, nb, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return fail(KFG_ECUDA, std::string("cudaMemcpy(plan table): ") + cudaGetErrorString(e));
    }
    return (long long)count;
}

}  // extern "C"

// ====================================================================
// Device plan cache (the GPU counterpart of the reference's kfc.c:24-83:
// find_cached_fft keyed by (nfft, inverse)); here keyed by transform kind,
// sample type, size and direction, thread-safe, plans kept until
// kfg_cache_clear().
// ====================================================================
namespace {
std::mutex g_cache_mu;
std::map<std::string, kfg_plan*> g_cache;
}  // namespace

extern "C" kfg_plan* kfg_plan_cached(int real, int dtype, int n, int inverse) {
    std::ostringstream k;
    k << real << ":" << dtype << ":" << n << ":" << (inverse ? 1 : 0);
    std::lock_guard<std::mutex> lk(g_cache_mu);
    auto it = g_cache.find(k.str());
    if (it != g_cache.end()) return it->second;
    kfg_plan* p = real ? kfg_plan_real(dtype, n, inverse) : kfg_plan_c2c(dtype, n, inverse);
    if (p) g_cache[k.str()] = p;
    return p;
}

extern "C" int kfg_cache_clear(void) {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    for (auto& kv : g_cache) kfg_plan_free(kv.second);
    g_cache.clear();
    return KFG_OK;
}

// ====================================================================
// Batched uneven mix: many transforms of different sizes, sample types and
// kinds, their data at byte offsets in two device arenas.  Requests are
// grouped per plan; the tiles of all groups run in persistent multi-plan
// launches (one per sample type, mode and pass), CTAs pulling work items
// from an atomic counter, largest tiles first.  The whole run can be
// captured in a CUDA graph.
// ====================================================================
struct kfg_batch {
    struct Req {
        int kind, dtype, n;
        long long in_off, out_off;
    };
    struct Launch {
        int phase = 0, dtype = 0, mode = 0, fam = 0, T = 32, smem = 0;
        int elem_kind = 0;  // 0: engine tiles; 1 / 2: real split / merge elements
        double cost = 0;
        std::vector<MultiItem> items;
        std::vector<int> groups;  // plan groups with steps in this launch (sorted)
        std::vector<int> deps;    // launches of the previous phase that hold steps of those groups
        cudaEvent_t done = nullptr;
        MultiItem* d_items = nullptr;
        unsigned long long* d_counter = nullptr;
    };
    // launches run on several streams, each after the launches it depends on
    static constexpr int kAux = 7;
    cudaStream_t aux[kAux] = {};
    cudaEvent_t fork = nullptr, join[kAux] = {};
    std::vector<Req> reqs;
    void* in_arena = nullptr;
    void* out_arena = nullptr;
    int target_T = 256;
    bool committed = false;
    std::vector<Step> steps;
    KArgs* d_steps = nullptr;
    std::vector<Launch> launches;
    std::vector<void*> allocs;
    std::vector<kfg_plan*> req_plan;
    long long scratch_bytes = 0;  // intermediates of multi-pass requests (each written once, read once)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;

    void release() {
        if (gexec) cudaGraphExecDestroy(gexec);
        if (graph) cudaGraphDestroy(graph);
        gexec = nullptr;
        graph = nullptr;
        for (void* p : allocs) cudaFree(p);
        allocs.clear();
        for (auto& L : launches)
            if (L.done) cudaEventDestroy(L.done);
        launches.clear();
        steps.clear();
        d_steps = nullptr;
        scratch_bytes = 0;
        committed = false;
    }
    ~kfg_batch() {
        release();
        for (int k = 0; k < kAux; ++k) {
            if (aux[k]) cudaStreamDestroy(aux[k]);
            if (join[k]) cudaEventDestroy(join[k]);
        }
        if (fork) cudaEventDestroy(fork);
    }
};

namespace {

template <typename T>
T* upload(kfg_batch* b, const std::vector<T>& v) {
    if (v.empty()) return nullptr;
    void* d = nullptr;
    if (cudaMalloc(&d, v.size() * sizeof(T)) != cudaSuccess) return nullptr;
    cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    b->allocs.push_back(d);
    return (T*)d;
}

int batch_commit(kfg_batch* b) {
    b->release();
    // group requests per plan
    std::map<std::string, std::vector<int>> groups;
    b->req_plan.assign(b->reqs.size(), nullptr);
    for (size_t i = 0; i < b->reqs.size(); ++i) {
        const auto& r = b->reqs[i];
        std::ostringstream k;
        k << r.kind << ":" << r.dtype << ":" << r.n;
        groups[k.str()].push_back((int)i);
        const bool real = r.kind != KFG_KIND_C2C;
        kfg_plan* p = kfg_plan_cached(real, r.dtype, r.n, r.kind == KFG_KIND_C2R);
        if (!p) return KFG_EINVAL;
        b->req_plan[i] = p;
    }
    std::vector<int> phase_of, group_of;
    int gi = 0;
    for (auto& kv : groups) {
        const auto& idx = kv.second;
        kfg_plan* p = b->req_plan[idx[0]];
        const long long cnt = (long long)idx.size();
        Schedule s;
        size_t ib = 0, ob = 0;
        int rc = build_schedule(p, cnt, 0, 1, 0, s, ib, ob);
        if (rc) return rc;
        const int esz = cpx_size(p->dtype);
        std::vector<long long> io(cnt), oo(cnt);
        for (long long j = 0; j < cnt; ++j) {
            const auto& r = b->reqs[idx[j]];
            if (r.in_off % esz || r.out_off % esz) return fail(KFG_EINVAL, "kfg_batch: offsets must be element aligned");
            io[j] = r.in_off / esz;
            oo[j] = r.out_off / esz;
        }
        long long* d_io = upload(b, io);
        long long* d_oo = upload(b, oo);
        void* scr = nullptr;
        const size_t off1 = (s.scratch[0] + 255) & ~(size_t)255;
        b->scratch_bytes += (long long)(s.scratch[0] + s.scratch[1]);
        if (s.scratch[0] + s.scratch[1] > 0) {
            if (cudaMalloc(&scr, off1 + s.scratch[1]) != cudaSuccess) return fail(KFG_ENOMEM, "kfg_batch: scratch");
            b->allocs.push_back(scr);
        }
        void* roles[4] = {b->in_arena, b->out_arena, scr, (char*)scr + off1};
        int ph = 0;
        for (auto& st : s.steps) {
            if (st.in_role == 0) st.args.in_off = d_io;
            if (st.out_role == 1) st.args.out_off = d_oo;
            st.args.in = roles[st.in_role];
            st.args.out = roles[st.out_role];
            if (st.kind == 0) {
                // widen the tile towards the launch's thread target
                while (st.cfg.T * 2 <= b->target_T) {
                    Step w = st;
                    if (!reshape_step(w, st.cfg.J * 2) || w.cfg.T > b->target_T || w.args.ntiles < 1) break;
                    st = w;
                }
            }
            b->steps.push_back(st);
            phase_of.push_back(ph++);
            group_of.push_back(gi);
        }
        ++gi;
    }
    // launches: engine tiles keyed by (phase, dtype, mode, family, threads
    // class, shared-memory class) -- two classes each (up to 256 threads or
    // more; up to 64 KiB of tile or more), so that small tiles do not run
    // with the block shape of the largest (on the 20,000-request mix: 44
    // launches in 4.96 ms; one class each, 16 launches, took 5.80 ms and one
    // class per power of two, 108 launches, 5.14 ms); split / merge elements
    // keyed by (phase, dtype, kind)
    std::map<std::string, int> lkey;
    for (size_t i = 0; i < b->steps.size(); ++i) {
        const Step& st = b->steps[i];
        std::ostringstream k;
        if (st.kind != 0)
            k << "E" << phase_of[i] << ":" << st.dtype << ":" << st.kind;
        else
            k << phase_of[i] << ":" << st.dtype << ":" << st.mode << ":" << st.fam << ":" << (st.cfg.T > 256) << ":"
              << (st.cfg.smem > 65536);
        auto it = lkey.find(k.str());
        int li;
        if (it == lkey.end()) {
            li = (int)b->launches.size();
            lkey[k.str()] = li;
            kfg_batch::Launch L;
            L.phase = phase_of[i];
            L.dtype = st.dtype;
            L.mode = st.mode;
            L.fam = st.fam;
            L.elem_kind = st.kind;
            b->launches.push_back(L);
        } else {
            li = it->second;
        }
        auto& L = b->launches[li];
        if (L.groups.empty() || L.groups.back() != group_of[i]) L.groups.push_back(group_of[i]);
        if (st.kind != 0) {
            const long long total = st.args.G * (st.args.sub[0].L / 2 + 1);
            for (long long c = 0; c * KF_ELEM_CHUNK < total; ++c) L.items.push_back(MultiItem{(int)i, 0, c});
            L.cost += (double)total;
            continue;
        }
        L.T = std::max(L.T, st.cfg.T);
        L.smem = std::max(L.smem, st.cfg.smem);
        for (long long t = 0; t < st.args.ntiles; ++t) L.items.push_back(MultiItem{(int)i, 0, t});
    }
    // most expensive tiles first (cost ~ J * L * log L)
    std::vector<double> cost(b->steps.size());
    for (size_t i = 0; i < b->steps.size(); ++i) {
        const Step& st = b->steps[i];
        const double L = st.args.sub[0].L;
        cost[i] = st.cfg.J * L * (L > 1 ? std::log2(L) : 1.0);
    }
    for (auto& L : b->launches) {
        if (L.elem_kind == 0) {
            std::stable_sort(L.items.begin(), L.items.end(),
                             [&](const MultiItem& a, const MultiItem& c) { return cost[a.step] > cost[c.step]; });
            for (auto& w : L.items) L.cost += cost[w.step];
        }
        L.d_items = upload(b, L.items);
        void* c = nullptr;
        if (cudaMalloc(&c, sizeof(unsigned long long)) != cudaSuccess) return fail(KFG_ENOMEM, "kfg_batch: counter");
        b->allocs.push_back(c);
        L.d_counter = (unsigned long long*)c;
    }
    // by phase; inside a phase the most expensive launch first
    std::stable_sort(b->launches.begin(), b->launches.end(), [](const kfg_batch::Launch& a, const kfg_batch::Launch& c) {
        return a.phase != c.phase ? a.phase < c.phase : a.cost > c.cost;
    });
    // A launch waits only for the launches of the previous phase that hold
    // steps of its own plan groups (a plan's steps are one phase apart), not
    // for the whole previous phase: long single-pass tiles no longer hold
    // back the second passes of other plans.
    for (auto& L : b->launches) {
        std::sort(L.groups.begin(), L.groups.end());
        L.groups.erase(std::unique(L.groups.begin(), L.groups.end()), L.groups.end());
    }
    for (size_t l = 0; l < b->launches.size(); ++l) {
        auto& L = b->launches[l];
        if (L.phase == 0) continue;
        for (size_t m = 0; m < l; ++m) {
            const auto& M = b->launches[m];
            if (M.phase != L.phase - 1) continue;
            std::vector<int> common;
            std::set_intersection(L.groups.begin(), L.groups.end(), M.groups.begin(), M.groups.end(),
                                  std::back_inserter(common));
            if (!common.empty()) L.deps.push_back((int)m);
        }
    }
    for (auto& L : b->launches) KFG_CK(cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming));
    for (int k = 0; k < kfg_batch::kAux; ++k) {
        if (!b->aux[k]) KFG_CK(cudaStreamCreateWithFlags(&b->aux[k], cudaStreamNonBlocking));
        if (!b->join[k]) KFG_CK(cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming));
    }
    if (!b->fork) KFG_CK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    std::vector<KArgs> ka;
    for (auto& st : b->steps) ka.push_back(st.args);
    b->d_steps = upload(b, ka);
    b->committed = true;
    return KFG_OK;
}

cudaError_t batch_launch(kfg_batch* b, const kfg_batch::Launch& L, cudaStream_t strm) {
    cudaError_t e = cudaMemsetAsync(L.d_counter, 0, sizeof(unsigned long long), strm);
    if (e != cudaSuccess) return e;
    MultiArgs m;
    m.steps = b->d_steps;
    m.items = L.d_items;
    m.nitems = (long long)L.items.size();
    m.counter = L.d_counter;
    if (L.elem_kind != 0) return launch_multi_elem(L.dtype, L.elem_kind, m, strm);
    return launch_multi(L.dtype, L.fam, L.mode, m, L.T, L.smem, 0, strm);
}

// Phases run in order on strm; the launches of one phase fork onto the
// auxiliary streams and join back before the next phase.
int batch_enqueue(kfg_batch* b, cudaStream_t strm) {
    // lanes: strm and the auxiliary streams; each launch goes to the lane
    // that frees up first by the launches' estimated costs, after waiting
    // for the events of the launches it depends on
    const int nl = 1 + kfg_batch::kAux;
    std::vector<double> lane_t(nl, 0.0), fin(b->launches.size(), 0.0);
    KFG_CK(cudaEventRecord(b->fork, strm));
    for (int k = 0; k < kfg_batch::kAux; ++k) KFG_CK(cudaStreamWaitEvent(b->aux[k], b->fork, 0));
    for (size_t l = 0; l < b->launches.size(); ++l) {
        const auto& L = b->launches[l];
        double ready = 0;
        for (int d : L.deps) ready = std::max(ready, fin[d]);
        int best = 0;
        for (int k = 1; k < nl; ++k)
            if (std::max(lane_t[k], ready) < std::max(lane_t[best], ready)) best = k;
        cudaStream_t s = best == 0 ? strm : b->aux[best - 1];
        for (int d : L.deps) KFG_CK(cudaStreamWaitEvent(s, b->launches[d].done, 0));
        cudaError_t e = batch_launch(b, L, s);
        if (e != cudaSuccess) return fail(KFG_ECUDA, std::string("kfg_batch launch: ") + cudaGetErrorString(e));
        KFG_CK(cudaEventRecord(L.done, s));
        fin[l] = lane_t[best] = std::max(lane_t[best], ready) + std::max(L.cost, 1.0);
    }
    for (int k = 0; k < kfg_batch::kAux; ++k) {
        KFG_CK(cudaEventRecord(b->join[k], b->aux[k]));
        KFG_CK(cudaStreamWaitEvent(strm, b->join[k], 0));
    }
    return KFG_OK;
}

}  // namespace

extern "C" {

kfg_batch* kfg_batch_create(void) { return new kfg_batch; }

void kfg_batch_free(kfg_batch* b) { delete b; }

int kfg_batch_add(kfg_batch* b, int kind, int dtype, int n, long long in_off, long long out_off) {
    if (!b || !valid_dtype(dtype) || n < 1 || kind < KFG_KIND_C2C || kind > KFG_KIND_C2R || in_off < 0 || out_off < 0)
        return fail(KFG_EINVAL, "kfg_batch_add: bad arguments");
    if (kind != KFG_KIND_C2C && (n & 1)) return fail(KFG_EINVAL, "Real FFT optimization must be even.");
    b->reqs.push_back(kfg_batch::Req{kind, dtype, n, in_off, out_off});
    b->committed = false;
    return KFG_OK;
}

int kfg_batch_commit(kfg_batch* b, void* in_arena, void* out_arena, int target_threads) {
    if (!b || !in_arena || !out_arena) return fail(KFG_EINVAL, "kfg_batch_commit: bad arguments");
    b->in_arena = in_arena;
    b->out_arena = out_arena;
    if (target_threads > 0) b->target_T = std::min(std::max(target_threads, 32), KF_MAXT);
    return batch_commit(b);
}

int kfg_batch_run(kfg_batch* b, void* stream) {
    if (!b || !b->committed) return fail(KFG_EINVAL, "kfg_batch_run: commit first");
    cudaStream_t s = pick(stream);
    if (b->gexec) {
        KFG_CK(cudaGraphLaunch(b->gexec, s));
        return KFG_OK;
    }
    return batch_enqueue(b, s);
}

int kfg_batch_capture(kfg_batch* b, void* stream) {
    if (!b || !b->committed) return fail(KFG_EINVAL, "kfg_batch_capture: commit first");
    cudaStream_t s = stream ? (cudaStream_t)stream : nullptr;
    bool own = false;
    if (!s) {
        KFG_CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        own = true;
    }
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->gexec = nullptr;
    b->graph = nullptr;
    KFG_CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int rc = batch_enqueue(b, s);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (own) cudaStreamDestroy(s);
    if (rc) return rc;
    if (e != cudaSuccess) return fail(KFG_ECUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
    b->graph = g;
    KFG_CK(cudaGraphInstantiate(&b->gexec, g, 0));
    return KFG_OK;
}

int kfg_batch_run_percall(kfg_batch* b, void* stream) {
    if (!b || !b->in_arena) return fail(KFG_EINVAL, "kfg_batch_run_percall: commit first");
    if (b->req_plan.size() != b->reqs.size()) return fail(KFG_EINVAL, "kfg_batch_run_percall: commit first");
    for (size_t i = 0; i < b->reqs.size(); ++i) {
        const auto& r = b->reqs[i];
        int rc = kfg_exec_batch(b->req_plan[i], (const char*)b->in_arena + r.in_off, (char*)b->out_arena + r.out_off, 1,
                                0, 0, stream);
        if (rc) return rc;
    }
    return KFG_OK;
}

int kfg_batch_info(const kfg_batch* b, long long* out, int nout) {
    if (!b || !out) return KFG_EINVAL;
    long long items = 0;
    for (auto& L : b->launches) items += (long long)L.items.size();
    long long v[5] = {(long long)b->reqs.size(), (long long)b->steps.size(), (long long)b->launches.size(), items,
                      2 * b->scratch_bytes};
    for (int i = 0; i < nout && i < 5; ++i) out[i] = v[i];
    return KFG_OK;
}

}  // extern "C"

// Internal hooks for kf_noalloc.cu (not exported): the schedule of a complex
// 1-D batch, the thread's error message, the pointer test and the stream pick.
namespace kf {
__attribute__((visibility("hidden"))) int c2c_schedule(kfg_plan* p, long long batch, long long in_dist,
                                                       long long out_dist, Schedule& s) {
    if (!p || p->kind != K_C2C) return fail(KFG_EINVAL, "needs a complex 1-D plan (kfg_plan_c2c)");
    size_t ib = 0, ob = 0;
    return build_schedule(p, batch, in_dist, 1, out_dist, s, ib, ob);
}
__attribute__((visibility("hidden"))) int set_error(int code, const std::string& msg) { return fail(code, msg); }
// device bytes a plan holds (tables of every sub-plan, fast-FIR response)
__attribute__((visibility("hidden"))) size_t plan_device_bytes(const kfg_plan* p) {
    if (!p) return 0;
    size_t b = 0;
    if (p->main) b += p->main->p.blob.size();
    if (p->aux) b += p->aux->p.blob.size();
    for (auto& a : p->axes)
        if (a) b += a->p.blob.size();
    if (p->d_H) b += (size_t)(p->n / 2 + 1) * 8;
    return b;
}
__attribute__((visibility("hidden"))) bool device_pointer(const void* ptr) { return is_device_ptr(ptr); }
__attribute__((visibility("hidden"))) cudaStream_t stream_or_default(void* stream) { return pick(stream); }
}  // namespace kf
