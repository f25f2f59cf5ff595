// deo_fx.cuh -- fixed-point helpers for exact Float64 stencil sums: a double
// decomposed into (e, m) with value = m * 2^(e - 1075 - S), m = +-mantissa << S;
// arithmetic shifts that align mantissas to a common exponent; a signed
// 128-bit accumulator of 64 x 64-bit products; and the 128-bit total rounded
// once to the nearest double (ties to even).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace deo {

template <int S>
__device__ __forceinline__ void decompose_fx(double v, long long& m, short& e) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int ex = (int)((b >> 52) & 0x7ffULL);
    const unsigned long long fr = b & 0xFFFFFFFFFFFFFULL;
    const long long mag = (long long)((ex ? (fr | (1ULL << 52)) : fr) << S);
    m = ((long long)b < 0) ? -mag : mag;
    e = (short)(ex == 0x7ff ? 4095 : (ex ? ex : 1));  // 4095 marks Inf/NaN: forces the fallback
}

// The signed 128-bit integer (hi, lo) rounded to the nearest double, ties to
// even, where a magnitude with lz leading zeros gets the biased exponent
// ebase - lz.  ok = false when the result would be subnormal or overflow.
__device__ __forceinline__ double fx_round(long long hi_s, unsigned long long lo, int ebase, bool& ok) {
    unsigned long long hi = (unsigned long long)hi_s;
    const bool neg = hi_s < 0;
    if (neg) {
        lo = 0ULL - lo;
        hi = ~hi + (lo == 0ULL ? 1ULL : 0ULL);
    }
    if ((hi | lo) == 0ULL) {
        ok = true;
        return 0.0;
    }
    int lz;
    if (hi) {
        lz = __clzll((long long)hi);
        if (lz) {
            hi = (hi << lz) | (lo >> (64 - lz));
            lo <<= lz;
        }
    } else {
        lz = 64 + __clzll((long long)lo);
        hi = lo << (lz - 64);
        lo = 0ULL;
    }
    unsigned long long mant = hi >> 11;
    const unsigned long long rb = hi & 0x7FFULL;
    if (rb > 0x400ULL || (rb == 0x400ULL && (lo != 0ULL || (mant & 1ULL)))) ++mant;
    int be = ebase - lz;
    if (mant >> 53) {
        mant >>= 1;
        ++be;
    }
    if (be <= 0 || be >= 2047) {
        ok = false;
        return 0.0;
    }
    ok = true;
    return __longlong_as_double(
        (long long)(((unsigned long long)neg << 63) | ((unsigned long long)be << 52) | (mant & 0xFFFFFFFFFFFFFULL)));
}

// 128-bit accumulator (hi, lo) += a * b for signed 64-bit a, b: one 64 x 64
// -> 128 product (mul.lo / mul.hi) and a carry-propagating add.
// Arithmetic shift right by d >= 0; PTX clamps shift amounts above 64 to 64
// (the result is then 0 or -1), so no clamp is needed.
__device__ __forceinline__ long long sar64(long long m, int d) {
    long long r;
    asm("shr.s64 %0, %1, %2;" : "=l"(r) : "l"(m), "r"(d));
    return r;
}

struct Acc128 {
    unsigned long long lo;
    long long hi;
};
__device__ __forceinline__ void mad128(Acc128& A, long long a, long long b) {
    const unsigned long long plo = (unsigned long long)(a * b);
    const long long phi = __mul64hi(a, b);
    asm("add.cc.u64 %0, %0, %2;\n\taddc.s64 %1, %1, %3;" : "+l"(A.lo), "+l"(A.hi) : "l"(plo), "l"(phi));
}

}  // namespace deo
