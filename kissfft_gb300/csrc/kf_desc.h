// Plain-old-data descriptors handed from the host plan to the GPU kernels.
//
// Vocabulary (all follow the reference's recursive decimation in time,
// kiss_fft.c:235-300):
//   stage i      one kf_bfly call level: radix p_i, span m_i = N/(p_0..p_i),
//                twiddle stride fstride_i = p_0..p_{i-1}.  Stages run from the
//                last factor (leaves) to the first.
//   position n   index into the reference's Fout buffer; n = sum d_i*m_i over
//                mixed-radix digits d_i < p_i.  Stage i combines the p_i
//                positions that differ only in digit i.
//   input order  A(n) = sum d_i*fstride_i, the input sample that the leaf
//                copy (kiss_fft.c:274-278) puts at position n.
//   sub-plan     a contiguous range of stages run as one kernel: the whole
//                transform, or one half of a two-pass large transform.
//   pass         one or two consecutive stages of a sub-plan executed on a
//                register tile (group) of R = p_a[*p_b] elements.
#pragma once
#include "kf_stdint.h"

#define KF_MAXST 32
#define KF_MAXJ 64
#define KF_MAXO 32
#define KF_MAXT 512
// real split / merge elements per work item of a batched element launch
#define KF_ELEM_CHUNK 2048

namespace kf {

enum { KF_F32 = 0, KF_F64 = 1, KF_Q15 = 2, KF_Q31 = 3 };
enum { MODE_C2C = 0, MODE_R2C = 1, MODE_C2R = 2, MODE_FIR = 3 };
// pass kinds: 2..5 single stage; 10*pa+pb two stages; 100+p generic p in
// registers (p in 7..31); 99 generic p of any size (output-parallel)
enum { KIND_RT_GENERIC = 99 };
// kernel families: the pass kinds a kernel is compiled for
enum { FAM_POW2 = 0, FAM_SMOOTH = 1, FAM_GENERAL = 2 };
// shared-tile index maps (all bijections inside blocks of 2^B elements):
// three-level XOR fold, identity, one-level XOR
enum { SWZ_FOLD = 0, SWZ_NONE = 1, SWZ_ONE = 2 };

struct KStage {
    int p;       // radix
    int m;       // global span m_i
    int fs;      // global twiddle stride fstride_i
    int tw_off;  // compact table: (q, u) at tw_off + (q-1)*m + u; constants at tw_off + (p-1)*m
    int mloc;    // local position stride (m_i / m_low)
    int iloc;    // local input-order stride (fstride_i / fstride_first)
};

struct KPass {
    int kind;
    int a;        // lowest local stage index in the pass (run last)
    int ns;       // stages in the pass (1 or 2)
    int R;        // elements per group
    int H;        // groups along the higher digits  (= iloc of stage a)
    int ML;       // groups along the lower digits   (= mloc of stage a+ns-1)
    int rev_off;  // digit-reversal table of the lower digits (-1 if ML == 1)
    int pad;
    unsigned long long hdiv;  // magic for n / H   (fdiv)
    unsigned long long gdiv;  // magic for n / (H*ML)
};

// Shape of a sub-plan: integers only, so that a whole shape can also be a
// compile-time constant of a specialised kernel.
struct KSub {
    int N;            // full transform length (generic twiddle modulus)
    int L;            // sub-plan length
    int nst, npass;
    int m_low;        // global span of the last stage in the range (1 for the leaf range)
    int inverse;
    int revfull_off;  // position -> input-order table (L ints) in the reverse tables, or -1
    int pad;
    KStage st[KF_MAXST];
    KPass ps[KF_MAXST];
};

// Device tables of a plan.
struct KTab {
    const void* tw_full;   // N twiddles (plan dtype)
    const void* tw_stage;  // compact per-stage tables
    const int* rev;        // digit-reversal tables
    const void* super_tw;  // real-transform super twiddles (ncfft/2) or null
};

// One launch: G jobs (sub-transforms), J per CTA tile.  Job jg decomposes as
// (g_hi, g_lo) = (jg / G_lo, jg % G_lo); its input base is
// g_hi*in_dhi + g_lo*in_dlo and element A sits at base + A*in_stride
// (units: complex elements, or real samples for the real-input modes).
// With G_mid > 1, g_hi splits once more into (g_hi / G_mid, g_hi % G_mid),
// the second part weighted by in_dmid / out_dmid (the strided fibers of an
// N-D axis that runs as two HBM passes).
// KRun holds everything but the plan shape: the argument of the
// plan-specialised kernels (whose shape is a compile-time constant), a few
// hundred bytes per launch instead of the shapes' kilobytes.
struct KRun {
    KTab tab[2];
    const void* in;
    void* out;
    const void* fir_H;        // fast FIR frequency response (nfft/2+1 bins)
    long long G, G_lo;
    long long G_mid, in_dmid, out_dmid;  // third level of the job index (G_mid <= 1: none)
    long long in_dhi, in_dlo, in_stride;
    long long out_dhi, out_dlo, out_stride;
    long long in_limit;       // fast FIR: signal length (zero padding beyond)
    long long out_limit;      // fast FIR: number of valid outputs
    long long ntiles;
    int J, logJ;
    int col_in, col_out;      // group enumeration of the first / last pass (1: jobs fastest)
    int nsub;
    int fir_ngood;
    int use_u;                // 1: twiddle offset U = g_lo (second half of a two-pass plan)
    const long long* in_off;  // per-transform input base (elements), replaces g_hi*in_dhi when set
    const long long* out_off; // per-transform output base (elements)
    int tma;                  // 1: tiles are contiguous; stage the next tile by TMA bulk copy
    int stage_off;            // byte offset of the staging buffer in dynamic shared memory
    int swz;                  // shared-tile layout: SWZ_FOLD, SWZ_NONE or SWZ_ONE (kf_engine.cuh swz)
    int* err;                 // device error word: bit 0 bad pass kind, bit 1 TMA wait timeout
};

// A launch's full arguments: the run-time part and the sub-plan shapes that
// the precompiled kernels read at run time (sub[1]: inverse plan of the fast FIR).
struct KArgs : KRun {
    KSub sub[2];
};

// A persistent multi-plan launch: CTAs take work items (a step's tile) from
// an atomic counter; every step carries its own plan shape.
struct MultiItem {
    int step;
    int pad;
    long long tile;
};

struct MultiArgs {
    const KArgs* steps;      // device array of step arguments
    const MultiItem* items;  // work items, most expensive first
    long long nitems;
    unsigned long long* counter;  // zeroed before every launch
};

}  // namespace kf
