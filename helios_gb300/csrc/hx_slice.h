// Exact splitting of FP64 values into signed base-256 digits for the
// tensor-core GEMM (integer arithmetic; host and device).
#pragma once
#include <cstring>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace tc {

// IEEE-754 bits of a double (host and device).
__host__ __device__ __forceinline__ unsigned long long dbits(double x)
{
#ifdef __CUDA_ARCH__
    return (unsigned long long)__double_as_longlong(x);
#else
    unsigned long long b;
    memcpy(&b, &x, sizeof b);
    return b;
#endif
}

// frexp exponent of the largest magnitude whose bits (sign cleared) are mb:
// max|x| = f 2^e with f in [0.5, 1); mb must be non-zero and finite.
__host__ __device__ __forceinline__ int exp_of_bits(unsigned long long mb)
{
    const int ex = (int)(mb >> 52);
    if (ex) return ex - 1022;
#ifdef __CUDA_ARCH__
    return (64 - __clzll((long long)mb)) - 1074;          // subnormal
#else
    return (64 - __builtin_clzll(mb)) - 1074;
#endif
}

// Signed base-256 digits of a = x 2^(7-e), |a| < 128 (e from exp_of_bits of
// the row): a = s_0 + 2^-8 s_1 + ... + 2^-8(S-1) s_(S-1) + r with |s_p| <= 128
// and |r| <= 2^-8(S-1)-1. Integer arithmetic on the bit pattern: a rounded to
// 8(S-1) fraction bits, then digits peeled off with round-half-up shifts
// (GB300's FP64 rate is a small fraction of its integer and FP32 rates).
template <int S>
__host__ __device__ __forceinline__ void slice_digits(double x, int e, int *s)
{
    constexpr int F = 8 * (S - 1);
    const unsigned long long bits = dbits(x);
    const int ex = (int)((bits >> 52) & 0x7FF);
    const long long mant = (long long)(bits & 0xFFFFFFFFFFFFFull) | (ex ? (1LL << 52) : 0LL);
    const int sh = (ex ? ex : 1) - 1075 + 7 - e + F;       // A = mant 2^sh = a 2^F
    long long A;
    if (mant == 0 || sh < -62) A = 0;
    else if (sh >= 0) A = mant << sh;
    else A = (mant + (1LL << (-sh - 1))) >> (-sh);
    if (bits >> 63) A = -A;
#pragma unroll
    for (int p = 0; p < S - 1; ++p) {
        const int shift = 8 * (S - 1 - p);
        const long long d = (A + (1LL << (shift - 1))) >> shift;
        s[p] = (int)d;
        A -= d << shift;
    }
    s[S - 1] = (int)A;
}

}  // namespace tc
