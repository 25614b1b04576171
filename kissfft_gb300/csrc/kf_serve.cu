// Serving loop: continuous batching of FFT, real-FFT, 2-D and fast-FIR
// requests under an HBM budget.
//
// A request is submitted from any host thread with its input and output
// buffers (device memory, pinned host memory, or ordinary host memory).  A
// worker thread owns the GPU side:
//
//  1. admission -- pending requests are admitted in arrival order while the
//     device bytes of the admitted-but-unfinished requests (input + output +
//     two-pass scratch) stay within the budget; a request larger than the
//     whole budget fails at once;
//  2. batching -- what was admitted since the last launch (up to 1/(2*slots)
//     of the budget) becomes one batch on a free slot (a stream of its own,
//     up to KFG_SERVE_SLOTS batches in flight), so requests that arrive while
//     others run join the next batch and overlap with them on the device;
//  3. per batch (on the slot's own launcher thread) -- one device allocation (stream-ordered, from the memory
//     pool) holds every request's input and output, laid out by plan; small
//     pinned host inputs are gathered into it by one zero-copy kernel over
//     the host link, large or pageable ones by the copy engines
//     (cudaMemcpyAsync); each plan group runs
//     as one batched launch sequence (kfg_exec_batch), fast-FIR requests as
//     their own block launches, all forked over the slot's sub-streams so
//     the small launches overlap; outputs are scattered back the same way;
//  4. completion -- a host callback at the end of the batch's stream work
//     stamps the completion time; the worker then releases the budget and
//     wakes waiters.
//
// Plans (and fast-FIR filter responses, keyed by the taps' contents) stay
// cached on the device; their bytes count against the budget, and the least
// recently used plan that no pending or admitted request holds is evicted
// when plans + requests would pass it.  Latency = completion
// stamp - submit stamp (steady clock), so p50/p99 include queueing.
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "kissfft_gb300.h"

namespace kf {
int set_error(int code, const std::string& msg);
size_t plan_device_bytes(const kfg_plan* p);
}
using kf::plan_device_bytes;
using kf::set_error;

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

int cpx_bytes_of(int dtype) { return dtype == KFG_DOUBLE ? 16 : (dtype == KFG_INT16 ? 4 : 8); }

// ---------------------------------------------------------------- copies
struct CopyItem {
    const unsigned char* src;
    unsigned char* dst;
    long long bytes;
};

// Item blockIdx.y, its 64 KiB chunks spread over the blockIdx.x CTAs (so a
// large request is copied by many CTAs at once); 16-byte words when both
// ends and the length allow, else 4-byte words, else bytes.  Host-side
// pointers are pinned memory the device reads or writes over the host link.
constexpr long long kChunk = 64 * 1024;
__global__ void kf_copy_items_kernel(const CopyItem* items) {
    const CopyItem c = items[blockIdx.y];
    const unsigned long long a = (unsigned long long)c.src | (unsigned long long)c.dst | (unsigned long long)c.bytes;
    for (long long lo = (long long)blockIdx.x * kChunk; lo < c.bytes; lo += (long long)gridDim.x * kChunk) {
        const long long hi = lo + kChunk < c.bytes ? lo + kChunk : c.bytes;
        if ((a & 15) == 0) {
            // four 16-byte loads in flight per thread across the host link
            const uint4* s = (const uint4*)(c.src + lo);
            uint4* d = (uint4*)(c.dst + lo);
            const long long nw = (hi - lo) / 16;
            long long i = threadIdx.x;
            for (; i + 3 * (long long)blockDim.x < nw; i += 4 * (long long)blockDim.x) {
                const uint4 v0 = s[i], v1 = s[i + blockDim.x], v2 = s[i + 2 * blockDim.x], v3 = s[i + 3 * blockDim.x];
                d[i] = v0;
                d[i + blockDim.x] = v1;
                d[i + 2 * blockDim.x] = v2;
                d[i + 3 * blockDim.x] = v3;
            }
            for (; i < nw; i += blockDim.x) d[i] = s[i];
        } else if ((a & 3) == 0) {
            const unsigned* s = (const unsigned*)(c.src + lo);
            unsigned* d = (unsigned*)(c.dst + lo);
            for (long long i = threadIdx.x; i < (hi - lo) / 4; i += blockDim.x) d[i] = s[i];
        } else {
            for (long long i = lo + threadIdx.x; i < hi; i += blockDim.x) c.dst[i] = c.src[i];
        }
    }
}

cudaError_t copy_items(const CopyItem* d_items, int n, long long max_bytes, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    long long gx = (max_bytes + kChunk - 1) / kChunk;
    if (gx > 64) gx = 64;
    if (gx < 1) gx = 1;
    kf_copy_items_kernel<<<dim3((unsigned)gx, (unsigned)n), 256, 0, st>>>(d_items);
    return cudaGetLastError();
}

enum { MEM_DEVICE = 0, MEM_PINNED = 1, MEM_PAGEABLE = 2 };

int mem_kind(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return MEM_PAGEABLE;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return MEM_DEVICE;
    if (a.type == cudaMemoryTypeHost) return MEM_PINNED;
    return MEM_PAGEABLE;
}

unsigned long long fnv1a(const void* p, size_t n) {
    const unsigned char* b = (const unsigned char*)p;
    unsigned long long h = 1469598103934665603ull;
    for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
    return h;
}

struct Req {
    kfg_serve_req d;
    long long id = 0;
    size_t in_b = 0, out_b = 0, dev_b = 0;
    double t_submit = 0, t_done = 0;
    int rc = 0;
    int in_mem = MEM_PAGEABLE, out_mem = MEM_PAGEABLE;
    std::string key;
    kfg_plan* plan = nullptr;
    std::atomic<int> state{0};  // 0 pending, 1 admitted, 2 done
};

constexpr int kMaxBatch = 8192;
// buffers at least this large move by the copy engines (cudaMemcpyAsync);
// smaller pinned ones by the gather/scatter kernel, one launch per batch
constexpr size_t kDmaBytes = 256 * 1024;

constexpr int kSub = 8;  // compute sub-streams per slot

struct Slot {
    cudaStream_t stream = nullptr;
    cudaStream_t sub[kSub] = {};
    cudaEvent_t fork = nullptr, join[kSub] = {};
    std::vector<Req*> reqs;
    void* dbuf = nullptr;
    CopyItem* h_items = nullptr;  // pinned: gather + scatter descriptors
    CopyItem* d_items = nullptr;
    std::atomic<int> done{0};
    double t_done = 0;
    bool busy = false;       // holds a batch (launching, in flight or waiting to be reaped)
    bool to_launch = false;  // handed to the slot's launcher thread
    size_t dev_bytes = 0;
    std::thread launcher;
};

}  // namespace

struct kfg_server {
    size_t budget = 0;
    int nslots = 0;
    int dev = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_launch;
    std::deque<Req*> pending;
    std::map<long long, std::unique_ptr<Req>> reqs;  // all requests not yet collected
    long long next_id = 1;
    size_t used = 0, peak_used = 0;
    bool stop = false;
    std::thread worker;
    std::vector<std::unique_ptr<Slot>> slots;
    // device plan cache: every plan the loop uses, least recently used
    // evicted first once plans + admitted requests would pass the budget;
    // a plan pinned by a pending or admitted request is never evicted
    struct PlanEntry {
        kfg_plan* plan = nullptr;
        size_t bytes = 0;
        unsigned long long last = 0;
        int pins = 0;
    };
    std::map<std::string, PlanEntry> plans;
    size_t plan_bytes = 0;
    unsigned long long tick = 0;
    long long evictions = 0;
    std::vector<double> lat;                 // completed latencies (s)
    long long completed = 0, failed = 0, batches = 0, max_batch = 0;
    double bytes_done = 0, t_first = 0, t_last = 0;
    double host_s = 0;  // host time spent describing and launching batches

    ~kfg_server();
};

namespace {

// Evict unpinned plans, least recently used first, until plans + admitted
// requests + `extra` fit the budget (or nothing is left to evict).
void evict_lru(kfg_server* s, size_t extra) {
    while (s->used + s->plan_bytes + extra > s->budget) {
        auto victim = s->plans.end();
        for (auto it = s->plans.begin(); it != s->plans.end(); ++it)
            if (it->second.pins == 0 && (victim == s->plans.end() || it->second.last < victim->second.last))
                victim = it;
        if (victim == s->plans.end()) return;
        s->plan_bytes -= victim->second.bytes;
        kfg_plan_free(victim->second.plan);
        s->plans.erase(victim);
        ++s->evictions;
    }
}

// The cached plan of `key` (built by make() on a miss), pinned for one request.
kfg_plan* pin_plan(kfg_server* s, const std::string& key, kfg_plan* (*make)(const kfg_serve_req&),
                   const kfg_serve_req& d) {
    auto it = s->plans.find(key);
    if (it == s->plans.end()) {
        kfg_plan* p = make(d);
        if (!p) return nullptr;
        kfg_server::PlanEntry e;
        e.plan = p;
        e.bytes = plan_device_bytes(p);
        s->plan_bytes += e.bytes;
        it = s->plans.emplace(key, e).first;
        it->second.pins = 1;  // not a victim of its own admission
        evict_lru(s, 0);
        it->second.pins = 0;
    }
    it->second.pins++;
    it->second.last = ++s->tick;
    return it->second.plan;
}

void unpin_plan(kfg_server* s, const std::string& key) {
    auto it = s->plans.find(key);
    if (it != s->plans.end() && it->second.pins > 0) it->second.pins--;
}

kfg_plan* make_c2c(const kfg_serve_req& d) { return kfg_plan_c2c(d.dtype, d.n0, d.inverse ? 1 : 0); }
kfg_plan* make_real(const kfg_serve_req& d) { return kfg_plan_real(d.dtype, d.n0, d.kind == KFG_SERVE_C2R); }
kfg_plan* make_2d(const kfg_serve_req& d) {
    const int dims[2] = {d.n0, d.n1};
    return kfg_plan_nd(d.dtype, dims, 2, d.inverse ? 1 : 0);
}
kfg_plan* make_fir(const kfg_serve_req& d) { return kfg_plan_fir(d.taps, (size_t)d.n0, 0, nullptr); }

// device bytes, plan key and (pinned) plan of a request (called on the worker)
int describe(kfg_server* s, Req* r) {
    const kfg_serve_req& d = r->d;
    const int esz = cpx_bytes_of(d.dtype), rsz = esz / 2;
    char key[160];
    kfg_plan* (*make)(const kfg_serve_req&) = nullptr;
    switch (d.kind) {
        case KFG_SERVE_C2C:
            if (d.n0 < 1) return set_error(KFG_EINVAL, "serve: bad length");
            r->in_b = r->out_b = (size_t)d.n0 * esz;
            snprintf(key, sizeof(key), "c:%d:%d:%d", d.dtype, d.n0, d.inverse ? 1 : 0);
            make = make_c2c;
            break;
        case KFG_SERVE_R2C:
        case KFG_SERVE_C2R: {
            if (d.n0 < 2 || (d.n0 & 1)) return set_error(KFG_EINVAL, "Real FFT optimization must be even.");
            const size_t nb = (size_t)(d.n0 / 2 + 1) * esz, nr = (size_t)d.n0 * rsz;
            r->in_b = d.kind == KFG_SERVE_R2C ? nr : nb;
            r->out_b = d.kind == KFG_SERVE_R2C ? nb : nr;
            snprintf(key, sizeof(key), "r:%d:%d:%d", d.dtype, d.n0, d.kind == KFG_SERVE_C2R);
            make = make_real;
            break;
        }
        case KFG_SERVE_C2C_2D:
            if (d.n0 < 1 || d.n1 < 1) return set_error(KFG_EINVAL, "serve: bad 2-D shape");
            r->in_b = r->out_b = (size_t)d.n0 * d.n1 * esz;
            snprintf(key, sizeof(key), "n:%d:%dx%d:%d", d.dtype, d.n0, d.n1, d.inverse ? 1 : 0);
            make = make_2d;
            break;
        case KFG_SERVE_FIR:
            if (d.dtype != KFG_FLOAT || !d.taps || d.n0 < 1 || d.len < d.n0)
                return set_error(KFG_EINVAL, "serve: fast FIR needs float taps and a signal at least as long");
            r->in_b = (size_t)d.len * 4;
            r->out_b = (size_t)(d.len - d.n0 + 1) * 4;
            snprintf(key, sizeof(key), "f:%d:%016llx", d.n0, fnv1a(d.taps, (size_t)d.n0 * 4));
            make = make_fir;
            break;
        default:
            return set_error(KFG_EINVAL, "serve: unknown request kind");
    }
    r->plan = pin_plan(s, key, make, d);
    if (!r->plan) return KFG_EINVAL;
    r->key = key;
    // two-pass plans allocate scratch of one more copy of the data
    int info[6] = {0};
    kfg_plan_info(r->plan, info, 6);
    const size_t scratch = (d.kind != KFG_SERVE_FIR && info[3] > 1) ? std::max(r->in_b, r->out_b) : 0;
    r->dev_b = ((r->in_b + 255) & ~(size_t)255) + ((r->out_b + 255) & ~(size_t)255) + scratch;
    r->in_mem = mem_kind(d.in);
    r->out_mem = mem_kind(d.out);
    return KFG_OK;
}

void CUDART_CB slot_done(void* p) {
    Slot* sl = (Slot*)p;
    sl->t_done = now_s();
    sl->done.store(1);
}

// Launch one batch on a free slot.  Requests are grouped by plan; each group
// is contiguous in the batch buffer (inputs, then outputs), so a group is one
// packed kfg_exec_batch call.
int launch_batch(kfg_server* s, Slot* sl) {
    std::map<std::string, std::vector<Req*>> groups;
    for (Req* r : sl->reqs) groups[r->key].push_back(r);
    std::vector<std::pair<Req*, size_t>> in_off, out_off;
    size_t off = 0;
    for (auto& g : groups)
        for (Req* r : g.second) {
            in_off.push_back({r, off});
            off += (r->in_b + 255) & ~(size_t)255;
        }
    for (auto& g : groups)
        for (Req* r : g.second) {
            out_off.push_back({r, off});
            off += (r->out_b + 255) & ~(size_t)255;
        }
    cudaError_t e = cudaMallocAsync(&sl->dbuf, std::max<size_t>(off, 256), sl->stream);
    if (e != cudaSuccess) return set_error(KFG_ENOMEM, std::string("serve: batch buffer: ") + cudaGetErrorString(e));
    unsigned char* base = (unsigned char*)sl->dbuf;
    std::map<Req*, size_t> ioff, ooff;
    int nin = 0;
    for (auto& io : in_off) {
        ioff[io.first] = io.second;
        Req* r = io.first;
        if (r->in_mem == MEM_PINNED && r->in_b < kDmaBytes) {
            sl->h_items[nin++] = CopyItem{(const unsigned char*)r->d.in, base + io.second, (long long)r->in_b};
        } else {
            e = cudaMemcpyAsync(base + io.second, r->d.in, r->in_b, cudaMemcpyDefault, sl->stream);
            if (e != cudaSuccess) return set_error(KFG_ECUDA, std::string("serve: input copy: ") + cudaGetErrorString(e));
        }
    }
    int nout = 0;
    for (auto& oo : out_off) {
        ooff[oo.first] = oo.second;
        Req* r = oo.first;
        if (r->out_mem == MEM_PINNED && r->out_b < kDmaBytes)
            sl->h_items[kMaxBatch + nout++] = CopyItem{base + oo.second, (unsigned char*)r->d.out, (long long)r->out_b};
    }
    if (nin > 0)
        e = cudaMemcpyAsync(sl->d_items, sl->h_items, sizeof(CopyItem) * nin, cudaMemcpyHostToDevice, sl->stream);
    if (e == cudaSuccess && nout > 0)
        e = cudaMemcpyAsync(sl->d_items + kMaxBatch, sl->h_items + kMaxBatch, sizeof(CopyItem) * nout,
                            cudaMemcpyHostToDevice, sl->stream);
    if (e != cudaSuccess) return set_error(KFG_ECUDA, std::string("serve: descriptors: ") + cudaGetErrorString(e));
    long long max_in = 0, max_out = 0;
    for (int k = 0; k < nin; ++k) max_in = std::max(max_in, sl->h_items[k].bytes);
    for (int k = 0; k < nout; ++k) max_out = std::max(max_out, sl->h_items[kMaxBatch + k].bytes);
    e = copy_items(sl->d_items, nin, max_in, sl->stream);
    if (e != cudaSuccess) return set_error(KFG_ECUDA, std::string("serve: gather: ") + cudaGetErrorString(e));
    // compute: the plan groups (and fast-FIR requests) are independent, so
    // they fork over the slot's sub-streams and join before the scatter
    e = cudaEventRecord(sl->fork, sl->stream);
    for (int k = 0; k < kSub && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(sl->sub[k], sl->fork, 0);
    if (e != cudaSuccess) return set_error(KFG_ECUDA, std::string("serve: fork: ") + cudaGetErrorString(e));
    int lane = 0;
    for (auto& g : groups) {
        Req* r0 = g.second[0];
        if (r0->d.kind == KFG_SERVE_FIR) {
            for (Req* r : g.second) {
                size_t ny = 0;
                int rc = kfg_fir_filter(r->plan, (const float*)(base + ioff[r]), (size_t)r->d.len,
                                        (float*)(base + ooff[r]), &ny, sl->sub[lane++ % kSub]);
                if (rc) r->rc = rc;
            }
            continue;
        }
        int rc = kfg_exec_batch(r0->plan, base + ioff[r0], base + ooff[r0], (long long)g.second.size(), 0, 0,
                                sl->sub[lane++ % kSub]);
        if (rc)
            for (Req* r : g.second) r->rc = rc;
    }
    for (int k = 0; k < kSub && e == cudaSuccess; ++k) {
        e = cudaEventRecord(sl->join[k], sl->sub[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(sl->stream, sl->join[k], 0);
    }
    if (e != cudaSuccess) return set_error(KFG_ECUDA, std::string("serve: join: ") + cudaGetErrorString(e));
    e = copy_items(sl->d_items + kMaxBatch, nout, max_out, sl->stream);
    if (e != cudaSuccess) return set_error(KFG_ECUDA, std::string("serve: scatter: ") + cudaGetErrorString(e));
    for (auto& oo : out_off) {
        Req* r = oo.first;
        if (r->out_mem != MEM_PINNED || r->out_b >= kDmaBytes) {
            e = cudaMemcpyAsync(r->d.out, base + oo.second, r->out_b, cudaMemcpyDefault, sl->stream);
            if (e != cudaSuccess) r->rc = KFG_ECUDA;
        }
    }
    cudaFreeAsync(sl->dbuf, sl->stream);
    sl->dbuf = nullptr;
    sl->done.store(0);
    e = cudaLaunchHostFunc(sl->stream, slot_done, sl);
    if (e != cudaSuccess) return set_error(KFG_ECUDA, std::string("serve: completion callback: ") + cudaGetErrorString(e));
    return KFG_OK;
}

void finish_req(kfg_server* s, Req* r, double t) {
    r->t_done = t;
    s->used -= r->dev_b;
    unpin_plan(s, r->key);
    if (r->rc == 0) {
        ++s->completed;
        s->lat.push_back(t - r->t_submit);
        s->bytes_done += (double)(r->in_b + r->out_b);
        if (s->t_first == 0 || r->t_submit < s->t_first) s->t_first = r->t_submit;
        s->t_last = std::max(s->t_last, t);
    } else {
        ++s->failed;
    }
    r->state.store(2);
}

// One per slot: turns the batch the worker assigned into stream work, so the
// host cost of launching batches is spread over the slots' threads.
void launcher_main(kfg_server* s, Slot* sl) {
    cudaSetDevice(s->dev);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        s->cv_launch.wait(lk, [&] { return sl->to_launch || s->stop; });
        if (!sl->to_launch) break;  // stopping, nothing assigned
        sl->to_launch = false;
        lk.unlock();
        const double t0 = now_s();
        int rc = launch_batch(s, sl);
        const double dt = now_s() - t0;
        lk.lock();
        s->host_s += dt;
        if (rc) {
            // wait for what was queued before the failure, then fail the batch
            lk.unlock();
            cudaStreamSynchronize(sl->stream);
            lk.lock();
            for (Req* r : sl->reqs) {
                r->rc = rc;
                finish_req(s, r, now_s());
            }
            sl->reqs.clear();
            sl->busy = false;
            s->cv_done.notify_all();
            s->cv_work.notify_all();
        }
    }
}

void worker_main(kfg_server* s) {
    cudaSetDevice(s->dev);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        // reap finished batches
        bool reaped = false;
        for (auto& slp : s->slots) {
            Slot* sl = slp.get();
            if (sl->busy && sl->done.load()) {
                cudaError_t e = cudaStreamSynchronize(sl->stream);  // already complete: returns its status
                for (Req* r : sl->reqs) {
                    if (e != cudaSuccess && r->rc == 0) r->rc = KFG_ECUDA;
                    finish_req(s, r, sl->t_done);
                }
                sl->reqs.clear();
                sl->busy = false;
                reaped = true;
            }
        }
        if (reaped) s->cv_done.notify_all();
        // admit and launch
        Slot* free_slot = nullptr;
        for (auto& slp : s->slots)
            if (!slp->busy) {
                free_slot = slp.get();
                break;
            }
        if (free_slot && !s->pending.empty()) {
            std::vector<Req*> batch;
            // a batch holds at most 1/(2*slots) of the budget, so several
            // batches pipeline (copy in / compute / copy out) across slots
            const size_t cap = std::max<size_t>(s->budget / (2 * (size_t)s->nslots), 1);
            size_t bbytes = 0;
            while (!s->pending.empty() && (int)batch.size() < kMaxBatch && (batch.empty() || bbytes < cap)) {
                Req* r = s->pending.front();
                if (r->dev_b == 0) {
                    const double td = now_s();
                    int rc = describe(s, r);
                    s->host_s += now_s() - td;
                    if (rc) {
                        s->pending.pop_front();
                        r->rc = rc;
                        r->state.store(2);
                        ++s->failed;
                        s->cv_done.notify_all();
                        continue;
                    }
                    const auto pe = s->plans.find(r->key);
                    const size_t own = pe != s->plans.end() ? pe->second.bytes : 0;
                    if (r->dev_b + own > s->budget) {
                        unpin_plan(s, r->key);
                        s->pending.pop_front();
                        r->rc = set_error(KFG_ENOMEM, "serve: request larger than the HBM budget");
                        r->state.store(2);
                        ++s->failed;
                        s->cv_done.notify_all();
                        continue;
                    }
                }
                if (s->used + s->plan_bytes + r->dev_b > s->budget) evict_lru(s, r->dev_b);
                if (s->used + s->plan_bytes + r->dev_b > s->budget) break;  // wait for memory to free up
                s->pending.pop_front();
                s->used += r->dev_b;
                bbytes += r->dev_b;
                r->state.store(1);
                batch.push_back(r);
            }
            s->peak_used = std::max(s->peak_used, s->used);
            if (!batch.empty()) {
                free_slot->reqs = batch;
                free_slot->busy = true;
                free_slot->done.store(0);
                free_slot->to_launch = true;
                ++s->batches;
                s->max_batch = std::max<long long>(s->max_batch, (long long)batch.size());
                s->cv_launch.notify_all();
                continue;
            }
        }
        bool inflight = false;
        for (auto& slp : s->slots) inflight |= slp->busy;
        if (s->stop && s->pending.empty() && !inflight) break;
        // sleep until new work arrives or a batch may have finished
        s->cv_work.wait_for(lk, std::chrono::microseconds(inflight ? 20 : 500));
    }
}

}  // namespace

kfg_server::~kfg_server() {
    {
        std::lock_guard<std::mutex> lk(mu);
        stop = true;
    }
    cv_work.notify_all();
    if (worker.joinable()) worker.join();
    cv_launch.notify_all();
    for (auto& sl : slots)
        if (sl->launcher.joinable()) sl->launcher.join();
    for (auto& sl : slots) {
        for (int k = 0; k < kSub; ++k) {
            if (sl->sub[k]) cudaStreamDestroy(sl->sub[k]);
            if (sl->join[k]) cudaEventDestroy(sl->join[k]);
        }
        if (sl->fork) cudaEventDestroy(sl->fork);
        if (sl->stream) cudaStreamDestroy(sl->stream);
        if (sl->h_items) cudaFreeHost(sl->h_items);
        if (sl->d_items) cudaFree(sl->d_items);
    }
    for (auto& kv : plans) kfg_plan_free(kv.second.plan);
}

extern "C" {

kfg_server* kfg_server_create(size_t hbm_budget, int slots) {
    if (hbm_budget == 0) hbm_budget = (size_t)40 << 30;
    if (slots <= 0) slots = 4;
    if (slots > KFG_SERVE_SLOTS) slots = KFG_SERVE_SLOTS;
    std::unique_ptr<kfg_server> s(new kfg_server);
    s->budget = hbm_budget;
    s->nslots = slots;
    if (cudaGetDevice(&s->dev) != cudaSuccess) {
        set_error(KFG_ECUDA, "serve: no CUDA device");
        return nullptr;
    }
    for (int i = 0; i < slots; ++i) {
        std::unique_ptr<Slot> sl(new Slot);
        if (cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaHostAlloc((void**)&sl->h_items, sizeof(CopyItem) * 2 * kMaxBatch, cudaHostAllocDefault) !=
                cudaSuccess ||
            cudaMalloc((void**)&sl->d_items, sizeof(CopyItem) * 2 * kMaxBatch) != cudaSuccess) {
            set_error(KFG_ECUDA, "serve: slot set-up failed");
            if (sl->stream) cudaStreamDestroy(sl->stream);
            if (sl->h_items) cudaFreeHost(sl->h_items);
            return nullptr;
        }
        bool ok = cudaEventCreateWithFlags(&sl->fork, cudaEventDisableTiming) == cudaSuccess;
        for (int k = 0; k < kSub && ok; ++k)
            ok = cudaStreamCreateWithFlags(&sl->sub[k], cudaStreamNonBlocking) == cudaSuccess &&
                 cudaEventCreateWithFlags(&sl->join[k], cudaEventDisableTiming) == cudaSuccess;
        s->slots.push_back(std::move(sl));
        if (!ok) {
            set_error(KFG_ECUDA, "serve: sub-stream set-up failed");
            return nullptr;
        }
    }
    // keep freed batch buffers in the pool between batches
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, s->dev) == cudaSuccess) {
        unsigned long long thr = (unsigned long long)hbm_budget;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    kfg_server* raw = s.release();
    for (auto& sl : raw->slots) sl->launcher = std::thread(launcher_main, raw, sl.get());
    raw->worker = std::thread(worker_main, raw);
    return raw;
}

long long kfg_server_submit(kfg_server* s, const kfg_serve_req* req) {
    if (!s || !req || !req->in || !req->out) return set_error(KFG_EINVAL, "kfg_server_submit: bad arguments");
    std::unique_ptr<Req> r(new Req);
    r->d = *req;
    r->t_submit = now_s();
    Req* raw = r.get();
    long long id;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        id = s->next_id++;
        raw->id = id;
        s->reqs[id] = std::move(r);
        s->pending.push_back(raw);
    }
    s->cv_work.notify_one();
    return id;
}

int kfg_server_wait(kfg_server* s, long long id, double timeout_s, double* latency_s) {
    if (!s) return KFG_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return set_error(KFG_EINVAL, "kfg_server_wait: unknown or already collected request");
    Req* r = it->second.get();
    const auto until = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
    while (r->state.load() != 2) {
        if (timeout_s >= 0 && s->cv_done.wait_until(lk, until) == std::cv_status::timeout && r->state.load() != 2)
            return 1;  // not finished yet
        if (timeout_s < 0) s->cv_done.wait(lk);
    }
    const int rc = r->rc;
    if (latency_s) *latency_s = r->t_done - r->t_submit;
    s->reqs.erase(it);
    return rc;
}

int kfg_server_drain(kfg_server* s) {
    if (!s) return KFG_EINVAL;
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        bool busy = !s->pending.empty();
        for (auto& sl : s->slots) busy |= sl->busy;
        if (!busy) break;
        s->cv_done.wait_for(lk, std::chrono::milliseconds(1));
    }
    // collect everything finished
    for (auto it = s->reqs.begin(); it != s->reqs.end();)
        if (it->second->state.load() == 2)
            it = s->reqs.erase(it);
        else
            ++it;
    return KFG_OK;
}

int kfg_server_stats(kfg_server* s, kfg_serve_stats* out) {
    if (!s || !out) return KFG_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    memset(out, 0, sizeof(*out));
    out->completed = s->completed;
    out->failed = s->failed;
    out->batches = s->batches;
    out->max_batch = s->max_batch;
    out->peak_hbm_bytes = (long long)s->peak_used;
    std::vector<double> v = s->lat;
    if (!v.empty()) {
        std::sort(v.begin(), v.end());
        auto q = [&](double f) { return v[std::min(v.size() - 1, (size_t)(f * (double)(v.size() - 1) + 0.5))]; };
        out->p50_s = q(0.50);
        out->p99_s = q(0.99);
        out->max_s = v.back();
        double sum = 0;
        for (double x : v) sum += x;
        out->mean_s = sum / (double)v.size();
    }
    const double span = s->t_last - s->t_first;
    if (span > 0) {
        out->req_per_s = (double)s->completed / span;
        out->gbs = s->bytes_done / span / 1e9;
    }
    out->bytes = s->bytes_done;
    out->host_s = s->host_s;
    out->plans = (long long)s->plans.size();
    out->plan_bytes = (long long)s->plan_bytes;
    out->evictions = s->evictions;
    return KFG_OK;
}

int kfg_server_reset_stats(kfg_server* s) {
    if (!s) return KFG_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    s->lat.clear();
    s->completed = s->failed = s->batches = s->max_batch = 0;
    s->bytes_done = s->t_first = s->t_last = 0;
    s->host_s = 0;
    s->peak_used = s->used;
    return KFG_OK;
}

void kfg_server_free(kfg_server* s) { delete s; }

}  // extern "C"

// ====================================================================
// Synthetic load: Poisson arrivals of a request mix against a server, and
// the same requests through the plain per-call form.
namespace {

struct GenReq {
    kfg_serve_req d;
    double t_arrival;
};

int fast_size(int n) { return kfg_next_fast_size(n); }

// nfft of a fast-FIR block for ntaps (tools/kiss_fastfir.c:75-87)
size_t fir_nfft(int ntaps) {
    size_t i = (size_t)ntaps - 1, nfft = 2;
    do {
        nfft <<= 1;
    } while (i >>= 1);
    return nfft < 2048 ? 2048 : nfft;
}

}  // namespace

extern "C" int kfg_server_loadtest(kfg_server* s, const kfg_loadtest* cfg, kfg_loadtest_result* res) {
    if (!s || !cfg || !res) return KFG_EINVAL;
    memset(res, 0, sizeof(*res));
    std::mt19937_64 rng(cfg->seed);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    std::normal_distribution<float> N01(0.0f, 1.0f);
    auto logu = [&](double lo, double hi) { return std::exp(std::log(lo) + U(rng) * (std::log(hi) - std::log(lo))); };
    // pinned pools: inputs (random, shared by requests at random offsets) and
    // an output ring
    const size_t in_pool = (size_t)cfg->in_pool_mb << 20, out_pool = (size_t)cfg->out_pool_mb << 20;
    unsigned char *hin = nullptr, *hout = nullptr;
    if (cudaHostAlloc((void**)&hin, in_pool, cudaHostAllocDefault) != cudaSuccess ||
        cudaHostAlloc((void**)&hout, out_pool, cudaHostAllocDefault) != cudaSuccess) {
        if (hin) cudaFreeHost(hin);
        return set_error(KFG_ENOMEM, "loadtest: pinned pools");
    }
    {
        float* f = (float*)hin;
        const size_t nf = in_pool / 4;
        std::mt19937 r2((unsigned)cfg->seed + 1);
        std::normal_distribution<float> g(0.0f, 1.0f);
        for (size_t i = 0; i < nf; ++i) f[i] = g(r2);
    }
    // a fixed set of filters (taps N(0,1)), so plans are reused
    const int nfilt = 16;
    std::vector<std::vector<float>> filt(nfilt);
    for (auto& h : filt) {
        const int L = (int)std::lround(logu(cfg->fir_taps_min, cfg->fir_taps_max));
        h.resize(L);
        for (auto& v : h) v = N01(rng);
    }
    // the request sequence
    std::vector<GenReq> seq;
    const double wsum = cfg->mix[0] + cfg->mix[1] + cfg->mix[2] + cfg->mix[3];
    const long long nreq = cfg->rate > 0 ? (long long)(cfg->rate * cfg->seconds * 1.2) + 16 : cfg->count;
    size_t oring = 0;
    double t = 0;
    for (long long k = 0; k < nreq; ++k) {
        if (cfg->rate > 0) {
            t += -std::log(1.0 - U(rng)) / cfg->rate;
            if (t > cfg->seconds) break;
        }
        GenReq g;
        memset(&g.d, 0, sizeof(g.d));
        g.t_arrival = t;
        const double u = U(rng) * wsum;
        size_t ib, ob;
        g.d.dtype = KFG_FLOAT;
        if (u < cfg->mix[0]) {
            g.d.kind = KFG_SERVE_C2C;
            g.d.n0 = fast_size((int)logu(cfg->c2c_min, cfg->c2c_max));
            ib = ob = (size_t)g.d.n0 * 8;
        } else if (u < cfg->mix[0] + cfg->mix[1]) {
            g.d.kind = KFG_SERVE_R2C;
            int n = fast_size((int)logu(cfg->c2c_min, cfg->c2c_max));
            while (n & 1) n = fast_size(n + 1);
            g.d.n0 = n;
            ib = (size_t)n * 4;
            ob = (size_t)(n / 2 + 1) * 8;
        } else if (u < cfg->mix[0] + cfg->mix[1] + cfg->mix[2]) {
            g.d.kind = KFG_SERVE_C2C_2D;
            g.d.n0 = fast_size((int)logu(cfg->d2_min, cfg->d2_max));
            g.d.n1 = fast_size((int)logu(cfg->d2_min, cfg->d2_max));
            ib = ob = (size_t)g.d.n0 * g.d.n1 * 8;
        } else {
            g.d.kind = KFG_SERVE_FIR;
            const auto& h = filt[(size_t)(U(rng) * nfilt) % nfilt];
            g.d.n0 = (int)h.size();
            g.d.taps = h.data();
            g.d.len = std::max<long long>((long long)logu((double)cfg->fir_len_min, (double)cfg->fir_len_max),
                                          (long long)fir_nfft(g.d.n0));
            ib = (size_t)g.d.len * 4;
            ob = (size_t)(g.d.len - g.d.n0 + 1) * 4;
        }
        if (ib + 256 > in_pool || ob + 256 > out_pool) continue;
        const size_t span = (in_pool - ib) / 256;
        g.d.in = hin + (size_t)(U(rng) * (double)span) * 256;
        if (oring + ob > out_pool) oring = 0;
        g.d.out = hout + oring;
        oring = (oring + ob + 255) & ~(size_t)255;
        seq.push_back(g);
    }
    res->offered = (long long)seq.size();
    // served: submit at the arrival times (or all at once)
    kfg_server_drain(s);
    kfg_server_reset_stats(s);
    std::vector<long long> ids(seq.size());
    const double t0 = now_s();
    for (size_t k = 0; k < seq.size(); ++k) {
        if (cfg->rate > 0)
            while (now_s() - t0 < seq[k].t_arrival) std::this_thread::yield();
        ids[k] = kfg_server_submit(s, &seq[k].d);
    }
    res->submit_s = now_s() - t0;
    kfg_server_drain(s);
    kfg_server_stats(s, &res->served);
    // per call: the same requests, one synchronous drop-in call each
    const long long npc = std::min<long long>((long long)seq.size(), cfg->percall_max);
    std::vector<double> lat;
    double pc_bytes = 0;
    std::map<std::string, kfg_plan*> pplans;
    const double p0 = now_s();
    for (long long k = 0; k < npc; ++k) {
        const kfg_serve_req& d = seq[k].d;
        const double a = now_s();
        int rc = KFG_OK;
        if (d.kind == KFG_SERVE_C2C) {
            kfg_plan* p = kfg_plan_cached(0, d.dtype, d.n0, 0);
            rc = p ? kfg_exec(p, d.in, d.out, nullptr) : KFG_EINVAL;
            pc_bytes += 16.0 * d.n0;
        } else if (d.kind == KFG_SERVE_R2C) {
            kfg_plan* p = kfg_plan_cached(1, d.dtype, d.n0, 0);
            rc = p ? kfg_exec(p, d.in, d.out, nullptr) : KFG_EINVAL;
            pc_bytes += 4.0 * d.n0 + 8.0 * (d.n0 / 2 + 1);
        } else if (d.kind == KFG_SERVE_C2C_2D) {
            char key[64];
            snprintf(key, sizeof(key), "n%dx%d", d.n0, d.n1);
            kfg_plan*& p = pplans[key];
            const int dims[2] = {d.n0, d.n1};
            if (!p) p = kfg_plan_nd(d.dtype, dims, 2, 0);
            rc = p ? kfg_exec(p, d.in, d.out, nullptr) : KFG_EINVAL;
            pc_bytes += 16.0 * d.n0 * d.n1;
        } else {
            char key[64];
            snprintf(key, sizeof(key), "f%p", (const void*)d.taps);
            kfg_plan*& p = pplans[key];
            if (!p) p = kfg_plan_fir(d.taps, (size_t)d.n0, 0, nullptr);
            size_t ny = 0;
            rc = p ? kfg_fir_filter(p, (const float*)d.in, (size_t)d.len, (float*)d.out, &ny, nullptr) : KFG_EINVAL;
            pc_bytes += 4.0 * d.len + 4.0 * (d.len - d.n0 + 1);
        }
        if (rc == KFG_OK) lat.push_back(now_s() - a);
    }
    const double pspan = now_s() - p0;
    for (auto& kv : pplans)
        if (kv.second) kfg_plan_free(kv.second);
    res->percall_count = (long long)lat.size();
    if (!lat.empty()) {
        res->percall_req_per_s = (double)lat.size() / pspan;
        res->percall_gbs = pc_bytes / pspan / 1e9;
        std::sort(lat.begin(), lat.end());
        res->percall_p50_s = lat[lat.size() / 2];
        res->percall_p99_s = lat[std::min(lat.size() - 1, (size_t)(0.99 * (double)(lat.size() - 1) + 0.5))];
    }
    cudaFreeHost(hin);
    cudaFreeHost(hout);
    return KFG_OK;
}
