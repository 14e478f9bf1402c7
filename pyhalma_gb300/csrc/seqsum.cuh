// Exact sequential FP64 sums on GB300 without a chain of FP64 adds.
//
// pyHALMA's per-cell and per-halo sums are numba loops that add one value at a time in FP64;
// reproducing them bit for bit needs the same sequence of roundings.  A chain of dependent
// FP64 adds is the slowest thing GB300 does (its FP64 pipe takes dozens of cycles per warp
// instruction), so the sum is kept as a signed integer count S of ulps of its binade
// [2^e, 2^(e+1)), ulp = 2^(e-52).  While the sum stays inside the binade, __dadd_rn(sum, a)
// is exactly (S +- round(|a| / ulp)) x ulp: |a| / ulp rounded to the nearest integer, the
// sign of a deciding between adding and subtracting, and a remainder of exactly half an ulp
// (a tie) going to the even result.  Away from ties the increment does not depend on the sum,
// so a warp adds 32 values at once: every lane rounds its value, an inclusive scan gives
// the 32 intermediate sums, and the prefix that stays strictly inside the binade (with half an
// ulp of margin) is accepted.  The first step that would leave the binade, change sign, meet a
// tie or a non-finite value is done by lane 0 with one __dadd_rn, after which the binade is
// read from the result and the warp continues with the rest of the values.
#pragma once

#include <math.h>
#include <stdint.h>

namespace halma {

struct SeqSum {
    double c;      // the sum when it is zero, subnormal or not finite (nrm == 0)
    long long S;   // |sum| in ulps of its binade, in [2^52, 2^53), when nrm
    int e;         // binade exponent
    int neg;       // sign of the sum (nrm only)
    int nrm;       // the sum is a normal number
};

constexpr long long kSeqTwo52 = 1ll << 52, kSeqTwo53 = 1ll << 53;
constexpr unsigned long long kSeqMant = (1ull << 52) - 1ull;

__device__ __forceinline__ void seq_init(SeqSum &q) {
    q.c = 0.0;
    q.S = 0;
    q.e = 0;
    q.neg = 0;
    q.nrm = 0;
}

__device__ __forceinline__ void seq_from_double(SeqSum &q, double c) {
    q.c = c;
    const unsigned long long b = (unsigned long long)__double_as_longlong(c);
    const int ef = (int)((b >> 52) & 0x7ff);
    q.nrm = ef != 0 && ef != 0x7ff;
    if (q.nrm) {
        q.e = ef - 1023;
        q.S = (long long)((b & kSeqMant) | (1ull << 52));
        q.neg = (int)(b >> 63);
    }
}

__device__ __forceinline__ double seq_value(const SeqSum &q) {
    if (!q.nrm) return q.c;
    const double v = ldexp((double)q.S, q.e - 52);   // exact
    return q.neg ? -v : v;
}

// |a| / ulp for ulp = 2^(e-52), ab = the bits of a finite |a|: integer part fl and the
// remainder's class (0 none, 3 below half an ulp, 2 exactly half, 1 above half); big when
// |a| / ulp may not fit the binade's range.
__device__ __forceinline__ void seq_ulps(unsigned long long ab, int e, long long &fl, int &code, bool &big) {
    const int ef = (int)(ab >> 52);
    const unsigned long long M = (ab & kSeqMant) | (ef ? (1ull << 52) : 0ull);
    const int d = (e - 52) - (ef ? ef - 1075 : -1074);   // |a| = M * 2^(e - 52 - d)
    big = d < 0;
    if (d <= 0) {
        fl = (long long)M;
        code = 0;
    } else if (d >= 64) {
        fl = 0;
        code = M ? 3 : 0;
    } else {
        fl = (long long)(M >> d);
        const unsigned long long rem = M & ((1ull << d) - 1ull), hb = 1ull << (d - 1);
        code = rem > hb ? 1 : (rem == hb ? 2 : (rem ? 3 : 0));
    }
}

// The signed increment of a to a normal sum with sign neg in binade e (ties and values that
// cannot be taken set bad).
__device__ __forceinline__ long long seq_inc(double a, int e, int neg, bool &bad) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(a);
    if (((b >> 52) & 0x7ff) == 0x7ff) {
        bad = true;
        return 0;
    }
    long long fl;
    int code;
    bool big;
    seq_ulps(b & ~(1ull << 63), e, fl, code, big);
    bad = big || code == 2;
    const long long m = fl + (code == 1 ? 1 : 0);
    const bool same = (int)(b >> 63) == neg || (b << 1) == 0;
    return same ? m : -m;
}

// One value, in order (any lane; the state is the caller's copy).
__device__ __forceinline__ void seq_add(SeqSum &q, double a) {
    if (q.nrm) {
        const unsigned long long ab = (unsigned long long)__double_as_longlong(a);
        if (((ab >> 52) & 0x7ff) != 0x7ff) {
            long long fl;
            int code;
            bool big;
            seq_ulps(ab & ~(1ull << 63), q.e, fl, code, big);
            if (!big) {
                const bool same = (int)(ab >> 63) == q.neg || (ab << 1) == 0;
                long long R;
                bool ok;
                if (same) {
                    const long long base = q.S + fl;
                    R = base + (code == 1 ? 1 : (code == 2 ? (base & 1) : 0));
                    ok = R < kSeqTwo53;
                } else {
                    const long long base = q.S - fl;
                    R = code == 1 ? base - 1 : (code == 2 ? base - (base & 1) : base);
                    ok = R >= kSeqTwo52 + 1;
                }
                if (ok) {
                    q.S = R;
                    return;
                }
            }
        }
        q.c = seq_value(q);
    }
    seq_from_double(q, __dadd_rn(q.c, a));
}

__device__ __forceinline__ void seq_bcast(SeqSum &q, int src) {
    q.c = __shfl_sync(0xffffffffu, q.c, src);
    q.S = __shfl_sync(0xffffffffu, q.S, src);
    q.e = __shfl_sync(0xffffffffu, q.e, src);
    q.neg = __shfl_sync(0xffffffffu, q.neg, src);
    q.nrm = __shfl_sync(0xffffffffu, q.nrm, src);
}

// The values a of lanes 0 .. nb-1 added in lane order to a warp-uniform sum (every lane of the
// warp calls it with the same state and nb).
__device__ __forceinline__ void seq_add_warp(SeqSum &q, double a, int nb, int lane) {
    int start = 0;
    while (start < nb) {
        if (q.nrm) {
            bool bad = false;
            const bool act = lane >= start && lane < nb;
            const long long inc = act ? seq_inc(a, q.e, q.neg, bad) : 0;
            long long P = inc;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const long long u = __shfl_up_sync(0xffffffffu, P, o);
                if (lane >= o) P += u;
            }
            P += q.S;
            const bool fail = act && (bad || P < kSeqTwo52 + 1 || P > kSeqTwo53 - 1);
            const unsigned fm = __ballot_sync(0xffffffffu, fail);
            const int first = fm ? __ffs(fm) - 1 : nb;
            if (first > start) q.S = __shfl_sync(0xffffffffu, P, first - 1);
            if (first >= nb) return;
            start = first;
        }
        // one value with the general step (lane 0), then the warp continues from the result
        const double v = __shfl_sync(0xffffffffu, a, start);
        if (lane == 0) seq_add(q, v);
        seq_bcast(q, 0);
        ++start;
    }
}

}  // namespace halma
