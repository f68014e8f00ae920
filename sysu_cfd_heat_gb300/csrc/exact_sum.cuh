// Deterministic, exactly rounded sums of FP64 values with integer arithmetic.
//
// On GB300 the FP64 pipe issues two lanes per clock per SM and a dependent FP64
// add takes tens of cycles, so a reduction tree of FP64 adds over a 1024-thread
// block and a grid of 152 blocks costs microseconds per dot product.  Here each
// value becomes a 128-bit two's-complement fixed-point number relative to the
// largest exponent of its warp, warps and blocks are aligned to the largest
// exponent of their group, and all additions are 64-bit integer adds with carry
// (the integer pipe).  Integer addition is associative, so the result does not
// depend on the order of the terms; it is the exact sum of the inputs up to
// truncations below 2^-100 of the largest term, rounded once to FP64.
//
// Layout of a fixed-point number: value = S * 2^(E - 1075 - F), S a signed
// 128-bit integer, E the biased FP64 exponent of the largest term, F = 56
// fraction bits below a term's 53-bit significand.  Headroom: a term is below
// 2^109; a warp sum below 2^114; a block sum (32 warps) below 2^119; block sums
// enter the grid sum shifted right by G = 8 more bits, so up to 2^16 blocks fit
// below 2^127.  Inf/NaN inputs are tracked by a flag and give a NaN sum.
#pragma once

#include <cstdint>

#include "device.hpp"

namespace sysu {

#ifdef __CUDACC__

struct I128 {
    unsigned long long lo;
    long long hi;
};

constexpr int XS_F = 56;  // fraction bits below the significand
constexpr int XS_G = 8;   // extra right shift of block sums in the grid sum

__device__ __forceinline__ I128 xs_add(I128 a, I128 b) {
    I128 r;
    asm("add.cc.u64 %0, %2, %4;\n\taddc.s64 %1, %3, %5;"
        : "=l"(r.lo), "=l"(r.hi)
        : "l"(a.lo), "l"(a.hi), "l"(b.lo), "l"(b.hi));
    return r;
}

__device__ __forceinline__ I128 xs_neg(I128 a) {
    I128 r;
    asm("sub.cc.u64 %0, 0, %2;\n\tsubc.s64 %1, 0, %3;" : "=l"(r.lo), "=l"(r.hi) : "l"(a.lo), "l"(a.hi));
    return r;
}

// Arithmetic shift right by s >= 0 (rounds toward minus infinity).
__device__ __forceinline__ I128 xs_sar(I128 a, int s) {
    I128 r;
    if (s <= 0) return a;
    if (s >= 127) {
        r.hi = a.hi >> 63;
        r.lo = (unsigned long long)r.hi;
    } else if (s >= 64) {
        r.lo = (unsigned long long)(a.hi >> (s - 64));
        r.hi = a.hi >> 63;
    } else {
        r.lo = (a.lo >> s) | ((unsigned long long)a.hi << (64 - s));
        r.hi = a.hi >> s;
    }
    return r;
}

__device__ __forceinline__ I128 xs_shfl_xor(I128 a, int o) {
    I128 r;
    r.lo = __shfl_xor_sync(FULL_MASK, a.lo, o);
    r.hi = __shfl_xor_sync(FULL_MASK, a.hi, o);
    return r;
}

// Biased exponent (0 for zero) and significand of |x|; nonfinite -> flag.
__device__ __forceinline__ int xs_split(double x, unsigned long long &m, bool &neg, int &nonfinite) {
    long long bits = __double_as_longlong(x);
    int e = (int)((bits >> 52) & 0x7FF);
    m = (unsigned long long)bits & 0xFFFFFFFFFFFFFull;
    neg = bits < 0;
    if (e == 0x7FF) {
        nonfinite = 1;
        m = 0;
        return 0;
    }
    if (e) m |= 1ull << 52;
    else e = 1;  // subnormal
    return m ? e : 0;
}

// Warp-level exact sum: every lane passes one value; every lane gets the warp's
// (exponent, fixed-point sum, nonfinite flag).
__device__ __forceinline__ void xs_warp(double x, int &E, I128 &S, int &nf) {
    unsigned long long m;
    bool neg;
    int f = 0;
    int e = xs_split(x, m, neg, f);
    E = __reduce_max_sync(FULL_MASK, e);
    int sh = E - e;
    I128 t;
    t.hi = (long long)(m >> (64 - XS_F));
    t.lo = m << XS_F;
    t = (m == 0) ? I128{0ull, 0ll} : xs_sar(t, sh);
    if (neg) t = xs_neg(t);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t = xs_add(t, xs_shfl_xor(t, o));
    S = t;
    nf = __reduce_or_sync(FULL_MASK, f);
}

// Lanes hold (E, S, nf) of up to 32 groups; all lanes get the aligned total.
// guard: extra right shift applied to every group (headroom for the sum).
__device__ __forceinline__ void xs_combine(int e, I128 s, int f, int guard, int &E, I128 &S, int &nf) {
    bool zero = (s.lo == 0 && s.hi == 0);
    int ee = zero ? 0 : e;
    E = __reduce_max_sync(FULL_MASK, ee);
    I128 t = zero ? I128{0ull, 0ll} : xs_sar(s, E - e + guard);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t = xs_add(t, xs_shfl_xor(t, o));
    S = t;
    nf = __reduce_or_sync(FULL_MASK, f);
}

// value = S * 2^(E + extra - 1075 - XS_F), correctly rounded (NaN if nf).
__device__ __forceinline__ double xs_to_double(int E, I128 S, int nf, int extra) {
    if (nf) return __longlong_as_double(0x7FF8000000000000ll);
    bool neg = S.hi < 0;
    if (neg) S = xs_neg(S);
    unsigned long long hi = (unsigned long long)S.hi, lo = S.lo;
    if (hi == 0 && lo == 0) return 0.0;
    int top = hi ? 128 - __clzll((long long)hi) : 64 - __clzll((long long)lo);  // significant bits
    unsigned long long u;
    int sc = E + extra - 1075 - XS_F;
    if (top <= 64) {
        u = lo;  // hi == 0
    } else {
        int s = top - 64;  // 1..63: drop s low bits, keep a sticky bit for the rounding
        u = (lo >> s) | (hi << (64 - s));
        if (lo << (64 - s)) u |= 1ull;
        sc += s;
    }
    double d = __ull2double_rn(u);
    // d * 2^sc in two steps so that neither factor leaves the normal range
    int s1 = sc / 2, s2 = sc - s1;
    d *= __longlong_as_double((long long)(s1 + 1023) << 52);
    d *= __longlong_as_double((long long)(s2 + 1023) << 52);
    return neg ? -d : d;
}

#endif  // __CUDACC__

}  // namespace sysu
