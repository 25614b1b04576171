// Host-side plans and launch schedules (no CUDA calls in here).
//
// A Plan is the device-ready form of kiss_fft_alloc's state
// (kiss_fft.c:337-372): the kf_factor radix list, the FP64-built twiddle
// table stored at the plan dtype, per-stage compact copies of the twiddles
// each stage reads, digit-reversal tables, and one or two sub-plans (a
// transform larger than one shared-memory tile runs as two HBM passes:
// the leaf stages, then the remaining stages with the inter-pass twiddles
// built in).  A Schedule is the list of kernel launches for one call.
#pragma once
#include <stddef.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "kf_desc.h"

namespace kf {

int dtype_size(int dtype);  // bytes of one scalar
inline int cpx_size(int dtype) { return 2 * dtype_size(dtype); }

// kf_factor (kiss_fft.c:306-328)
std::vector<int> factor(int n);
// kiss_fft_next_fast_size (kiss_fft.c:412-424)
int next_fast_size(int n);

// Twiddle tables exactly as kiss_fft_alloc / kiss_fftr_alloc build them.
void make_twiddles(int dtype, int n, int inverse, void* out);
void make_super_twiddles(int dtype, int ncfft, int inverse, void* out);

// Largest sub-plan length held in one shared-memory tile for a dtype.
int max_tile_len(int dtype);

struct LaunchCfg {
    int J = 1;        // jobs per tile (power of two)
    int T = 128;      // threads per CTA
    int col_in = 0;   // enumeration of the first pass (1: jobs fastest)
    int col_out = 0;  // enumeration of the last pass
    int smem = 0;     // dynamic shared bytes
    long long grid = 0;
    int minb = 1;     // specialised kernels: blocks per SM the register budget must allow
};

struct Plan {
    int dtype = KF_F32;
    int n = 0;         // complex transform length
    int inverse = 0;
    std::vector<int> radix;
    int nsub = 1;      // 1: one tile pass; 2: two HBM passes
    int split = 0;     // stages [0, split) form sub 1 when nsub == 2
    int real_nfft = 0; // > 0: a real plan of this size (n = real_nfft/2)
    // blob = [tw_full | tw_stage | super_tw | rev ints], 256-byte aligned parts
    std::vector<uint8_t> blob;
    size_t off_tw_full = 0, off_tw_stage = 0, off_super = 0, off_rev = 0;
    KSub sub[2];       // shapes (kf_shape.h)
    KTab tab{};        // device tables, set by bind()
    std::string error;

    // Builds everything; lmax caps the tile length (0 = dtype default).
    bool build(int dtype, int n, int inverse, int lmax = 0, int real_nfft = 0);
    // Point the tables at a copy of the blob at base.
    void bind(const void* base);
    // Length of each sub-plan's tile.
    int sub_len(int s) const { return sub[s].L; }
};

// Default launch shape for a sub-plan of length L and a mode.
LaunchCfg default_cfg(const KSub& sb, int dtype, int mode, long long G, int col_in, int col_out, int want_threads = 256);
int cfg_smem_bytes(const KSub& sb, int dtype, int J);
int cfg_min_threads(const KSub& sb, int mode, int J);
// Default shared-tile index map (SWZ_*) of a launch over tiles of length L.
int default_swz(int dtype, int L);
// Smallest kernel family whose compiled pass kinds cover a sub-plan.
int sub_family(const KSub& sb);

// Stage a step's contiguous tiles by TMA bulk copy when it qualifies: row
// tiles (C2C/R2C) whose inputs are packed transforms, 16-byte aligned, with
// room for the staging buffer.  Returns whether staging was switched on.
struct Step;
bool enable_tma(Step& st, const void* in);
bool recolumn_step(Step& st);
bool retarget_threads(Step& st, int T);
void set_tma_enabled(int on);
bool tma_enabled();

// Re-shape a step: J jobs per tile (T, shared memory and grid follow);
// false if the shape is not valid for the step.
bool reshape_step(Step& st, int J);

// One kernel launch of a schedule.
struct Step {
    int kind = 0;       // 0: engine kernel; 1: real split; 2: real merge
    int mode = MODE_C2C;
    int fam = FAM_GENERAL;  // kernel family covering the sub-plans' pass kinds
    int tma_ok = 1;         // 0: never stage this step by TMA (autotuner's choice)
    // plan shape of a specialised kernel: make_shape(dtype, shape_n, shape_inv, 0).sub[shape_sub]
    int shape_n = 0, shape_inv = 0, shape_sub = 0;
    int dtype = KF_F32;
    KArgs args;
    LaunchCfg cfg;
    // buffer roles resolved by the executor: 0 user in, 1 user out, 2 tmp
    int in_role = 0, out_role = 1;
    // run-time specialised kernel resolved for exactly this launch shape
    // (set by the executor's schedule cache; any change of the shape clears it)
    const void* kfn = nullptr;
};

// Buffer roles of a schedule: 0 the caller's input, 1 the caller's output,
// 2 and 3 scratch the executor provides (scratch[0] and scratch[1] bytes).
struct Schedule {
    std::vector<Step> steps;
    size_t scratch[2] = {0, 0};
    std::string error;
};

// Batched complex transforms: batch transforms, element r of transform b at
// in[b*in_dist + r*in_stride], output contiguous rows at b*out_dist.
bool schedule_c2c(const Plan& p, long long batch, long long in_dist, long long in_stride, long long out_dist,
                  Schedule& s);
// Batched real transforms (plan built with real_nfft): rows of nfft reals
// at b*in_dist -> nfft/2+1 bins at b*out_dist (units: reals / bins).
bool schedule_r2c(const Plan& p, long long batch, long long in_dist, long long out_dist, Schedule& s,
                  int in_role = 0, int out_role = 1);
bool schedule_c2r(const Plan& p, long long batch, long long in_dist, long long out_dist, Schedule& s,
                  int in_role = 0, int out_role = 1);
// Complex transform of every fiber along `axis` of a row-major array of
// `batch` arrays with shape dims (plan length = dims[axis]).  A two-pass
// axis plan keeps its intermediate in scratch role tmp_role (2 or 3).
bool schedule_axis(const Plan& p, const int* dims, int ndims, int axis, long long batch, int in_role, int out_role,
                   Schedule& s, int tmp_role = 2);
// Real overlap-scrap FIR of a signal of Ns samples with fw/iv real plans
// of nfft and filter response H (bound to a device pointer by the caller).
bool schedule_fastfir(const Plan& fw, const Plan& iv, long long L, long long Ns, long long nblocks_first,
                      Schedule& s);

}  // namespace kf
