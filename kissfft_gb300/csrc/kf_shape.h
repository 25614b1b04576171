// Plan shape as a constexpr function: the kf_factor radix list, stage
// spans and strides, the split into one or two tile passes, the register
// pass grouping, and the offsets of every table in the plan's device blob.
//
// The host plan builder (kf_plan.cpp) fills the tables at these offsets;
// specialised kernels evaluate the same function at compile time, so the
// two always agree on the layout.
#pragma once
#include "kf_desc.h"

#if defined(__CUDACC__) || defined(__CUDACC_RTC__)
#define KF_CX __host__ __device__ constexpr
#else
#define KF_CX constexpr
#endif

namespace kf {

struct ShapeInfo {
    int error;        // 0 ok; 1 bad size; 2 too many factors; 3 no two-tile split; 4 generic tile too long
    int K;            // number of stages
    int radix[KF_MAXST];
    int m[KF_MAXST];
    int fs[KF_MAXST];
    int twoff[KF_MAXST];  // -1 for stages that read the full table (IEEE generic radix, p > 31)
    long long tw_count;   // entries of the compact per-stage table
    int nsub, split;
    int rev_total;        // ints of all reverse tables
    KSub sub[2];
};

KF_CX int cpx_bytes(int dtype) { return dtype == KF_F64 ? 16 : (dtype == KF_Q15 ? 4 : 8); }

// largest sub-plan length of one shared-memory tile (128 KiB)
KF_CX int tile_len_max(int dtype) { return (128 * 1024) / cpx_bytes(dtype); }

// Compact per-stage twiddle table of a radix-p stage (p = 2..5): for every
// u < m, tw_width(p) consecutive entries tw[q*u*fstride] (q = 1..p-1, then
// padding), so one butterfly's twiddles are one or two vector loads; the
// radix-3/5 constants (tw[fstride*m], tw[2*fstride*m]) follow the m rows.
// Q15 tables (these and the generic rows below) hold every twiddle as a pair
// of int32, the 16-bit values sign-extended, so the multiplies take them as
// they are: tw_units(dtype) table entries per twiddle.
KF_CX int tw_width(int p) { return p == 2 ? 1 : (p == 3 ? 2 : 4); }
KF_CX int tw_units(int dtype) { return dtype == KF_Q15 ? 2 : 1; }

KF_CX bool small_prime(int p) {
    return p == 7 || p == 11 || p == 13 || p == 17 || p == 19 || p == 23 || p == 29 || p == 31;
}

// Fixed-point generic-radix stages (p = 7..31) read their twiddles from
// rows: for every u < m and output leg q1 < p, gen_row(p) consecutive
// entries tw[(q*fstride*(u + q1*m)) mod N] for q = 1..p-1 (then padding) --
// the exact sequence kf_bfly_generic walks (kiss_fft.c:218-226).
KF_CX int gen_row(int p) { return (p - 1 + 3) & ~3; }

// magic multiplier M with n / d == (n * M) >> 40 for n * d < 2^40
KF_CX unsigned long long div_magic(int d) {
    return d <= 1 ? (1ull << 40) : (((1ull << 40) + (unsigned long long)d - 1) / (unsigned long long)d);
}

KF_CX int isqrt_floor(int n) {
    long long r = 0;
    while ((r + 1) * (r + 1) <= n) ++r;
    return (int)r;
}

// kf_factor (kiss_fft.c:306-328): 4s, then 2, then odd trial divisors up to
// floor(sqrt(n)) of the original n; the remainder is the last factor.
KF_CX int factor_into(int n, int* f) {
    if (n <= 1) {
        f[0] = 1;
        return 1;
    }
    int k = 0, p = 4;
    const int lim = isqrt_floor(n);
    while (n > 1) {
        while (n % p) {
            p = (p == 4) ? 2 : (p == 2 ? 3 : p + 2);
            if (p > lim) p = n;
        }
        n /= p;
        if (k < KF_MAXST) f[k] = p;
        ++k;
    }
    return k;
}

// One sub-plan over global stages [g0, g1); reverse tables are appended at
// *rev_next (ints).
KF_CX void shape_sub(ShapeInfo& si, KSub& sb, int n, int inverse, int g0, int g1, int pair_rmax, int trip_rmax,
                     int& rev_next) {
    const int nst = g1 - g0;
    sb.N = n;
    sb.nst = nst;
    sb.inverse = inverse;
    sb.m_low = si.m[g1 - 1];
    sb.revfull_off = -1;
    long long L = 1;
    for (int j = g0; j < g1; ++j) L *= si.radix[j];
    sb.L = (int)L;
    for (int i = 0; i < nst; ++i) {
        const int j = g0 + i;
        sb.st[i].p = si.radix[j];
        sb.st[i].m = si.m[j];
        sb.st[i].fs = si.fs[j];
        sb.st[i].tw_off = si.twoff[j];
        sb.st[i].mloc = si.m[j] / sb.m_low;
        sb.st[i].iloc = si.fs[j] / si.fs[g0];
    }
    // passes in execution order: from the leaf stage down to stage 0.
    // Adjacent radices 2..5 share a register group of up to three stages;
    // the grouping minimises the number of passes, then the largest group.
    // bpass/bmaxr/bns[i]: best grouping of stages 0..i-1 and its last group.
    int bpass[KF_MAXST + 1]{}, bmaxr[KF_MAXST + 1]{}, bns[KF_MAXST + 1]{};
    for (int i = 1; i <= nst; ++i) {
        bpass[i] = 1 << 20;
        for (int ns = 3; ns >= 1; --ns) {  // ties: the larger group on the leaf side
            if (ns > i) continue;
            int R = 1;
            bool ok = true;
            for (int k = i - ns; k < i; ++k) {
                const int pk = sb.st[k].p;
                if (ns > 1 && (pk < 2 || pk > 5)) ok = false;
                R *= pk;
            }
            if (!ok || (ns == 2 && R > pair_rmax) || (ns == 3 && R > trip_rmax)) continue;
            const int np1 = bpass[i - ns] + 1;
            const int mr = bmaxr[i - ns] > R ? bmaxr[i - ns] : R;
            if (np1 < bpass[i] || (np1 == bpass[i] && mr < bmaxr[i])) {
                bpass[i] = np1;
                bmaxr[i] = mr;
                bns[i] = ns;
            }
        }
    }
    int np = 0, i = nst - 1;
    while (i >= 0) {
        KPass p{};
        const int ns = bns[i + 1];
        p.a = i - ns + 1;
        p.ns = ns;
        p.R = 1;
        for (int k = p.a; k <= i; ++k) p.R *= sb.st[k].p;
        if (ns == 3) {
            p.kind = 1000 + 100 * sb.st[p.a].p + 10 * sb.st[p.a + 1].p + sb.st[p.a + 2].p;
        } else if (ns == 2) {
            p.kind = 10 * sb.st[p.a].p + sb.st[p.a + 1].p;
        } else {
            // p == 1 only for nfft == 1: the reference's p = 1 generic butterfly
            const int pa = sb.st[i].p;
            p.kind = (pa >= 2 && pa <= 5) ? pa : (small_prime(pa) ? 100 + pa : KIND_RT_GENERIC);
        }
        i -= ns;
        const int b = p.a + p.ns - 1;
        p.H = sb.st[p.a].iloc;
        p.ML = sb.st[b].mloc;
        p.rev_off = -1;
        if (p.ML > 1) {
            p.rev_off = rev_next;
            rev_next += p.ML;
        }
        p.hdiv = div_magic(p.H);
        p.gdiv = div_magic(p.H * p.ML);
        sb.ps[np++] = p;
    }
    sb.npass = np;
}

KF_CX ShapeInfo make_shape(int dtype, int n, int inverse, int lmax, int real_nfft) {
    ShapeInfo si{};
    si.error = 0;
    if (n < 1) {
        si.error = 1;
        return si;
    }
    if (lmax <= 0) lmax = tile_len_max(dtype);
    int f[KF_MAXST + 8]{};
    const int K = factor_into(n, f);
    if (K > KF_MAXST) {
        si.error = 2;
        return si;
    }
    si.K = K;
    long long acc = 1, cnt = 0;
    for (int j = 0; j < K; ++j) {
        si.radix[j] = f[j];
        si.fs[j] = (int)acc;
        acc *= f[j];
        si.m[j] = (int)(n / acc);
        if (f[j] >= 2 && f[j] <= 5) {
            cnt = (cnt + 3) & ~3LL;  // 4-entry alignment for vector loads
            si.twoff[j] = (int)cnt;
            cnt += ((long long)tw_width(f[j]) * si.m[j] + 2) * tw_units(dtype);
        } else if ((dtype == KF_Q15 || dtype == KF_Q31) && small_prime(f[j])) {
            cnt = (cnt + 3) & ~3LL;
            si.twoff[j] = (int)cnt;
            cnt += (long long)gen_row(f[j]) * f[j] * si.m[j] * tw_units(dtype);
        } else {
            si.twoff[j] = -1;
        }
    }
    si.tw_count = cnt;
    const int prm = dtype == KF_F64 ? 16 : 25;
    const int trm = dtype == KF_F32 ? 48 : 0;  // three-stage register groups: float only
    int rev_next = 0;
    if (n <= lmax) {
        si.nsub = 1;
        si.split = 0;
        shape_sub(si, si.sub[0], n, inverse, 0, K, prm, trm, rev_next);
    } else {
        int best = -1;
        long long bestv = 0, P = 1;
        for (int s = 1; s < K; ++s) {
            P *= si.radix[s - 1];
            const long long LA = n / P;
            if (P <= lmax && LA <= lmax) {
                const long long v = P > LA ? P : LA;
                if (best < 0 || v < bestv) best = s, bestv = v;
            }
        }
        if (best < 0) {
            si.error = 3;
            return si;
        }
        si.nsub = 2;
        si.split = best;
        shape_sub(si, si.sub[0], n, inverse, best, K, prm, trm, rev_next);
        shape_sub(si, si.sub[1], n, inverse, 0, best, prm, trm, rev_next);
    }
    for (int s = 0; s < si.nsub; ++s) {
        for (int k = 0; k < si.sub[s].npass; ++k)
            if (si.sub[s].ps[k].kind == KIND_RT_GENERIC && si.sub[s].L > KF_MAXO * KF_MAXT) si.error = 4;
        if (si.nsub == 1) {
            si.sub[s].revfull_off = rev_next;
            rev_next += si.sub[s].L;
        }
    }
    si.rev_total = rev_next;
    (void)real_nfft;
    return si;
}

// Bit of a pass kind in a kernel's kind mask (the pass kinds it compiles).
typedef unsigned long long kmask_t;
KF_CX kmask_t kind_bit(int kind) {
    switch (kind) {
        case 2: return 1ull << 0;
        case 4: return 1ull << 1;
        case 42: return 1ull << 2;
        case 44: return 1ull << 3;
        case 3: return 1ull << 4;
        case 5: return 1ull << 5;
        case 23: return 1ull << 6;
        case 25: return 1ull << 7;
        case 33: return 1ull << 8;
        case 35: return 1ull << 9;
        case 43: return 1ull << 10;
        case 45: return 1ull << 11;
        case 55: return 1ull << 12;
        case 107: return 1ull << 13;
        case 111: return 1ull << 14;
        case 113: return 1ull << 15;
        case 117: return 1ull << 16;
        case 119: return 1ull << 17;
        case 123: return 1ull << 18;
        case 129: return 1ull << 19;
        case 131: return 1ull << 20;
        case KIND_RT_GENERIC: return 1ull << 21;
        // three-stage groups (radices of stages a, a+1, a+2), float plans only
        case 1444: return 1ull << 22;
        case 1442: return 1ull << 23;
        case 1443: return 1ull << 24;
        case 1423: return 1ull << 25;
        case 1425: return 1ull << 26;
        case 1433: return 1ull << 27;
        case 1435: return 1ull << 28;
        case 1233: return 1ull << 29;
        case 1235: return 1ull << 30;
        case 1255: return 1ull << 31;
        case 1333: return 1ull << 32;
        case 1335: return 1ull << 33;
    }
    return 0;
}
constexpr kmask_t KM_POW2 = 0xfull;           // kinds 2, 4, 42, 44
constexpr kmask_t KM_SMOOTH = 0x1fffull;      // + 3, 5 and the 2/3/5 pairs
constexpr kmask_t KM_GENERAL = 0x3fffffull;   // + generic primes 7..31 and any p
constexpr kmask_t KM_RTG = 1ull << 21;
constexpr kmask_t KM_TRIP_POW2 = (1ull << 22) | (1ull << 23);  // 444, 442
constexpr kmask_t KM_TRIP = 0xfffull << 22;                     // all twelve triples

KF_CX kmask_t kind_mask(const KSub& sb) {
    kmask_t m = 0;
    for (int k = 0; k < sb.npass; ++k) m |= kind_bit(sb.ps[k].kind);
    return m;
}

// Pass kinds a family kernel compiles; triples only where plans have them.
KF_CX kmask_t family_mask(int fam, bool f32) {
    const kmask_t m = fam == FAM_POW2 ? KM_POW2 : (fam == FAM_SMOOTH ? KM_SMOOTH : KM_GENERAL);
    if (!f32) return m;
    return m | (fam == FAM_POW2 ? KM_TRIP_POW2 : KM_TRIP);
}

// Smallest kernel family whose compiled pass kinds cover a sub-plan.
KF_CX int family_of(const KSub& sb) {
    int f = FAM_POW2;
    for (int k = 0; k < sb.npass; ++k) {
        const int kd = sb.ps[k].kind;
        if (kd == 2 || kd == 4 || kd == 42 || kd == 44 || kd == 1444 || kd == 1442) continue;
        if (kd < 99 || kd > 1000)
            f = f > FAM_SMOOTH ? f : FAM_SMOOTH;
        else
            f = FAM_GENERAL;
    }
    return f;
}

}  // namespace kf
