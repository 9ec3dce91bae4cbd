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

// The same digits with fewer operations. The top-down peel leaves, below
// every digit position 8j, the centered residue L_j of A modulo 2^8j (in
// [-2^(8j-1), 2^(8j-1))), so digit k from the bottom is (L_(k+1) - L_k) 2^-8k
// and the top digit (A - L_(S-1)) 2^-F: one residue per digit from A's
// words (32-bit operations up to 8j = 32) instead of S-1 rounds of 64-bit
// add, shift and subtract.
template <int S>
__host__ __device__ __forceinline__ void slice_digits_fast(double x, int e, int *s)
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
    const unsigned lo = (unsigned)A;
    long long Lprev = 0;
#pragma unroll
    for (int k = 0; k < S - 1; ++k) {
        const int w = 8 * (k + 1);                             // residue modulo 2^w
        long long L;
        if (w < 32) L = (long long)(int)((lo + (1u << (w - 1))) & ((1u << w) - 1u)) - (1LL << (w - 1));
        else if (w == 32) L = (long long)(int)lo;
        else L = ((A + (1LL << (w - 1))) & ((1LL << w) - 1)) - (1LL << (w - 1));
        s[S - 1 - k] = w < 32 ? (int)((int)(L - Lprev) >> (8 * k)) : (int)((L - Lprev) >> (8 * k));
        Lprev = L;
    }
    s[0] = (int)((A - Lprev) >> F);
}

// bf16 bit pattern of s 2^-8p for an integer |s| <= 128 (exact): s is
// placed in the significand of the float 1.5 2^(23-8p), whose unit in the
// last place is 2^-8p, and the offset subtracted -- an integer add and an
// FP32 subtract instead of an int-to-float conversion.
__host__ __device__ __forceinline__ float digit_value(int s, int p)
{
    const unsigned mb = (unsigned)(150 - 8 * p) << 23 | 0x400000u;    // bits of 1.5 2^(23-8p)
    float m, v;
    const unsigned b = mb + (unsigned)s;
#ifdef __CUDA_ARCH__
    m = __uint_as_float(mb);
    v = __uint_as_float(b);
#else
    memcpy(&m, &mb, sizeof m);
    memcpy(&v, &b, sizeof v);
#endif
    return v - m;
}

// FP32 bits, FP64 from bits, leading zeros of a 64-bit word, a right shift
// that gives 0 for shift counts of 32 or more (host and device).
__host__ __device__ __forceinline__ unsigned fbits(float x)
{
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    unsigned b;
    memcpy(&b, &x, sizeof b);
    return b;
#endif
}
__host__ __device__ __forceinline__ double dfrom(unsigned long long b)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double x;
    memcpy(&x, &b, sizeof x);
    return x;
#endif
}
__host__ __device__ __forceinline__ int clz64(unsigned long long x)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}
__host__ __device__ __forceinline__ unsigned shr_clamped(unsigned m, unsigned s)
{
#ifdef __CUDA_ARCH__
    unsigned n;
    asm("shr.b32 %0, %1, %2;" : "=r"(n) : "r"(m), "r"(s));
    return n;
#else
    return s >= 32u ? 0u : m >> s;
#endif
}

// GB300 issues about two FP64 instructions per clock per SM, so a GEMM
// epilogue that converts, scales and stores every output in FP64 costs
// several times the MMAs of a short-K product. The conversions below use
// integer arithmetic on the bit patterns instead.
//
// x 2^k as an FP64 value, exactly, for a normal FP32 x and |k| <= 896 (the
// result stays normal): the exponent rebiased, the significand widened;
// a sign flip by `negmask` (0 or 0x80000000). Zero and FP32 subnormals give
// 0 (a subnormal accumulator is below 2^-126 of its row scale).
__host__ __device__ __forceinline__ double f2d_pow2(float x, int k, unsigned negmask)
{
    const unsigned u = fbits(x);
    const unsigned e = (u >> 23) & 255u;
    const unsigned hi32 = ((u & 0x80000000u) ^ negmask) | ((e + 896u + (unsigned)k) << 20) | ((u >> 3) & 0xFFFFFu);
    const unsigned lo32 = u << 29;
    return e == 0u ? 0.0 : dfrom(((unsigned long long)hi32 << 32) | lo32);
}

// x 2^k for a normal FP64 x whose result stays normal (an exponent add);
// `ok` cleared otherwise.
__host__ __device__ __forceinline__ double pow2_int(double x, int k, bool &ok)
{
    const unsigned long long b = dbits(x);
    const int ex = (int)((b >> 52) & 2047);
    if ((b << 1) == 0ull) return x;
    if (ex == 0 || ex == 2047 || ex + k <= 0 || ex + k >= 2047) { ok = false; return 0.0; }
    return dfrom(b + ((unsigned long long)(long long)k << 52));
}

// The count n of an exact class sum a = n 2^-8q (|n| < 2^24, an integer by
// the chunk rule of the tensor-core GEMM) from its bit pattern: the
// significand shifted right by the exponent's distance from the units
// place (a shift of 32 or more gives 0, which covers a == 0).
__host__ __device__ __forceinline__ int class_count(float a, int q)
{
    const unsigned u = fbits(a);
    const unsigned m = (u & 0x7FFFFFu) | 0x800000u;
    const unsigned n = shr_clamped(m, (unsigned)(150 - 8 * q) - ((u >> 23) & 255u));
    return (u >> 31) ? -(int)n : (int)n;
}

}  // namespace tc
