// Tensor-core backend of the grouped tensor-GEMM: exact-slice BF16 products on tcgen05.
//
// FP64 operands are turned into integer slices (an error-free splitting in
// the spirit of the Ozaki scheme): row r of A is scaled by 2^-e_r so that its
// largest entry is below 1, then a = 2^-7 (s0 + 2^-8 s1 + 2^-16 s2 + ...)
// with S integer digits |s_p| <= 128 (hx_slice.h), stored as s_p 2^-8p, each
// exactly representable in bf16 (the representation error is below 2^-8S+1
// of the row maximum). The product keeps the slice pairs (i, j) with
// i + j <= QMAX. Products of such slices are integers times 2^-8(i+j) with
// at most 15 significant bits, so a tensor-core accumulation of a few hundred
// of them with equal weight is exact in FP32 (checked on the hardware:
// integer inputs give bit-exact sums, while general bf16 inputs lose low bits
// as K grows). Every weight q = i + j gets its own TMEM accumulator block;
// those of the leading weights (q < NX) are exact, the rounding of the others
// is scaled down by 2^-8NX. The blocks of one buffer lie side by side in TMEM
// in the order of q, and the B slices side by side in shared memory, so one
// MMA multiplies slice i of A by slices j = 0..J of B stacked along N into the
// blocks q = i..i+J: one MMA per A slice instead of one per slice pair, which
// divides the shared-memory operand reads (the kernel's bound) by about the
// number of pairs per A slice. Every chunk of KC k-blocks the accumulators are
// summed by TwoSum and added into an FP32 (hi, lo) pair per output, so the
// result carries the accuracy of the splitting relative to the operands' row
// maxima without the tensor core's accumulation error. (A drain in FP64 would
// be exact too, but at GB300's FP64 rate it costs more than the MMAs.)
//
// Per group of TgemmDesc problems:
//   1. row_scale: per row of A and B (through the descriptor's strides) the
//      binary exponent of the largest |entry|, over 32 x 64 tiles staged in
//      shared memory (coalesced along the source's contiguous dimension).
//   2. split_gather: the slices, K-major, zero-padded, from the same tiles:
//      [slice][batch][rows][Kp] (rows to 128 for A, to the tile width for B;
//      Kp to 64). Integer arithmetic only.
//   3. tc_gemm: one CTA per 128 x BN output tile (or per K slice of it).
//      A producer warp streams 64-deep k-blocks of all slices with TMA
//      (cp.async.bulk.tensor, 128-byte swizzle) through a ring of stages; one
//      thread of the MMA warp issues tcgen05.mma (kind::f16, BF16 x BF16 ->
//      FP32, M = 128, N = a multiple of BN, K = 16) into the class accumulators, alternating
//      between two TMEM buffers per chunk; the epilogue warps drain a finished
//      buffer with tcgen05.ld (a TMEM lane is an output row; the warps of a
//      lane quarter split its columns) while the next chunk runs, then stage
//      the (hi, lo) pairs in shared memory and write C = alpha*2^(e_m+f_n-14)*
//      (hi+lo) + beta*C with consecutive threads on consecutive columns, the
//      FP64 value built from the FP32 pair and the power of two by integer
//      arithmetic (GB300's FP64 pipe is a small fraction of its integer rate).
//   Every mbarrier wait is bounded by wall time; a wait that runs out records
//   a code in a device error word and the CTA still frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "hx_common.cuh"
#include "hx_kernels.h"
#include "hx_slice.h"
#include "hx_tc.h"

namespace tc {

// Four precisions of the same kernel. Slice p of an operand is stored as
// s_p 2^-8p (exact in bf16), so the product of slices i and j weighs
// 2^-8(i+j) by itself and a class accumulator needs no further weight.
// Classes q = i + j < NX are kept exact (their partial sums are integers
// times 2^-8q below 2^24 per chunk); the classes q >= NX are accumulated in
// FP32 (error about K * 2^-32 relative for a chunk of depth K) and summed
// in the epilogue, their rounding scaled down by 2^-8NX.
//   LOW:  3 slices, pairs i + j <= 3 (8 products, 4 MMAs per k-step), NX = 1:
//         about 2^-24 of the row maxima; 128 x 64 tiles.
//   MID:  4 slices, pairs i + j <= 3 (10 products, 4 MMAs), NX = 2: about
//         2^-32; 128 x 64.
//   HIGH: 5 slices, pairs i + j <= 4 (15 products, 5 MMAs), NX = 3: about
//         2^-35 of the row maxima (3.3e-11 measured at 6400^3); 128 x 48
//         tiles fed by 32-deep k-blocks (64-byte swizzle). Six slices with
//         pairs i + j <= 5 reached 1.5e-13 but cost 1.7x more, far more
//         accuracy than the phase needs: it hands over to the 7-slice check
//         at 0.1 eps, and the ladder sends any molecule whose residual stalls
//         above that to 7-slice iterations.
//   EXACT: 7 slices (48 fraction bits below the leading digit, past FP64's
//         53-bit mantissa), pairs i + j <= 6 (28 products, 7 MMAs), NX = 5:
//         an emulation of an FP64 GEMM, its error that of the FP64 product
//         itself; 128 x 32 tiles, so that two buffers of seven accumulator
//         blocks fit in TMEM.
// These errors set the residual level a phase can reach (the GEMM outputs
// are ~1e3-1e4 times the residual they cancel down to).
template <int S_, int QMAX_, int NX_, int BN_, int STAGES_, int KC_, int EPIW_, int BK_>
struct Cfg {
    static constexpr int S = S_;                     // integer slices per FP64 operand
    static constexpr int QMAX = QMAX_;               // slice pairs with i + j <= QMAX are multiplied
    static constexpr int NX = NX_;                   // exact classes q = 0 .. NX-1
    static constexpr int NQ = QMAX_ + 1;             // TMEM accumulator blocks per buffer (q = 0..QMAX)
    static constexpr int BM = 128, BN = BN_, BK = BK_;   // BK: k-block depth (64 or 32)
    static constexpr uint64_t SWZ = BK_ == 64 ? 2 : 4;     // smem descriptor layout: 128- or 64-byte swizzle
    static constexpr int SBO = 8 * BK_ * 2;                 // bytes between 8-row core-matrix groups
    static constexpr int KC = KC_;                   // k-blocks per chunk (exact classes stay exact)
    static constexpr int STAGES = STAGES_;
    static constexpr int EPI_WARPS = EPIW_;          // epilogue warps (a multiple of 4)
    static constexpr int NTHREADS = (EPIW_ + 2) * 32; // + TMA producer warp + MMA warp
    static constexpr int EPI_THREADS = EPIW_ * 32;
    static constexpr int ATILE = BM * BK * 2;        // bytes per A slice tile
    static constexpr int BTILE = BN * BK * 2;        // bytes per B slice tile
    static constexpr int STAGE_BYTES = S * (ATILE + BTILE);
    // output staging strip: (hi, lo) pairs of STG_ROWS rows (all 128 where the
    // ring leaves room), row offsets and exponents of C
    static constexpr int RING_BYTES = STAGES * S * (128 * BK * 2 + BN * BK * 2);
    static constexpr int STG_ROWS = [] {
        const int avail = 232448 - 1280 - 128 * 12 - STAGES_ * S_ * (128 * BK_ * 2 + BN_ * BK_ * 2);
        int r = 128;
        while (r > 8 && r * (BN_ + 1) * 8 > avail) r >>= 1;
        return r;
    }();
    static constexpr int STG_BYTES = STG_ROWS * (BN_ + 1) * 8 + 128 * 12;
    static constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + STG_BYTES + 1024 + 256;
    static constexpr int EPI_COLS = BN / (EPIW_ / 4); // columns drained per epilogue thread
    // 7-slice mode: the exact classes are drained into an int64 per element
    // (units of 2^-8(NX-1)); the other modes use an FP32 (hi, lo) pair
    static constexpr bool INT_DRAIN = S_ >= 7;
    static constexpr float DRAIN_SCALE = (float)(1ull << (8 * (NX_ - 1)));
    static constexpr int PRODUCTS = [] { int n = 0; for (int i = 0; i < S_; ++i) for (int j = 0; j < S_; ++j) n += (i + j <= QMAX_); return n; }();
    // pairs in the largest exact class
    static constexpr int XPAIRS = [] { int m = 0; for (int q = 0; q < NX_; ++q) { int n = 0; for (int i = 0; i < S_; ++i) n += (q - i >= 0 && q - i < S_); m = n > m ? n : m; } return m; }();
    // exactness of a chunk: (pairs per exact class) * KC*64 * 2^14 < 2^24
    static_assert((long long)XPAIRS * KC_ * BK_ * 16384LL < (1LL << 24), "chunk too deep for exact sums");
    static_assert(BK_ == 64 || BK_ == 32, "k-block depth");
    static_assert(2 * NQ * BN_ <= 512, "two TMEM buffers must fit in 512 columns");
    static_assert(RING_BYTES + STG_BYTES + 1280 <= 232448, "shared memory");
    static_assert(STG_ROWS * (BN_ + 1) * 8 <= 232448 - 1280 - 128 * 12 - RING_BYTES, "staging strip");
    static_assert(EPIW_ % 4 == 0 && EPI_COLS % 8 == 0, "epilogue split");
    static_assert(EPIW_ * 32 >= 128 && EPIW_ * 32 >= BN_, "epilogue threads cover the tile's rows and columns");
    // int64 drain: a chunk adds below 2^(24 + 8(NX-1) + 1); 32 chunks stay below 2^63
    static_assert(!INT_DRAIN || 24 + 8 * (NX_ - 1) + 1 + 5 < 63, "int64 drain headroom");
};
using Low = Cfg<3, 3, 1, 64, 2, 8, 16, 64>;
using Mid = Cfg<4, 3, 2, 64, 2, 6, 16, 64>;
using High = Cfg<5, 4, 3, 48, 3, 8, 12, 32>;
using Exact = Cfg<7, 6, 5, 32, 3, 6, 16, 32>;
constexpr int TMEM_COLS = 512;
constexpr int BM = 128, KPAD = 64;   // K is padded to KPAD (the slicing tile depth)
constexpr unsigned long long WAIT_NS = 4000000000ull; // a wait longer than 4 s is declared failed

struct TcDesc {
    int batch, M, N, K, Mp, Np, Kp;
    int Mi, Ni;
    long long c[5];
    double alpha, beta;
    int alpha_e, alpha_neg;          // alpha = (-1)^alpha_neg 2^alpha_e when alpha_pow2
    int alpha_pow2, beta_one;        // beta_one: beta == 1 (C += r without a multiply)
    double *C;
    int tiles_m, tiles_n;
    long long tile_start;
    int mol;
    int ksplit;                      // K slices accumulated with FP64 atomics (beta == 1 only)
    int kb_per;                      // k-blocks per slice
    const int *expA, *expB;          // per-row binary exponents ([batch][Mp], [batch][Np])
    CUtensorMap mapA, mapB;          // 2D maps over this desc's scratch
};

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: false (and an error record) if the phase never completes.
__device__ __forceinline__ unsigned long long globaltimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, int *err, int code)
{
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = globaltimer();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (globaltimer() - t0 > WAIT_NS) break;
    }
    if (err) atomicCAS(err, 0, code);
    return false;
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
            smem_u32(dst)),
        "l"(map), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}
// Shared-memory matrix descriptor of a configuration's k-block depth: K-major,
// 128-byte rows (BK = 64, SWIZZLE_128B) or 64-byte rows (BK = 32,
// SWIZZLE_64B), 8-row groups SBO bytes apart, descriptor version 1.
template <class C>
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr)
{
    return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(C::SBO >> 4) << 32) |
           ((uint64_t)1 << 46) | (C::SWZ << 61);
}
// Instruction descriptor: kind::f16, D=F32, A=B=BF16, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
// TMEM loads of eight columns without a wait: several loads in flight, then
// tmem_wait_ld and tmem_tie8 on their registers (the tie names them after the
// wait, so no use moves above it).
__device__ __forceinline__ void tmem_ld8_issue(uint32_t taddr, uint32_t *r)
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_tie8(uint32_t *r)
{
    asm volatile("" : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]));
}

__device__ __forceinline__ long long split_off(int x, int xi, long long s0, long long s1)
{
    return (long long)(x / xi) * s0 + (long long)(x % xi) * s1;
}

// x 2^(ea + eb - 14) for row exponent ea of A and column exponent eb of B:
// the value ldexp gives (one rounding; exact for normal results); zero when
// the row or the column is all zero (exponent INT_MIN: every product is zero)
__device__ __forceinline__ double scale_pow2(double x, int ea, int eb)
{
    if (ea == INT_MIN || eb == INT_MIN) return 0.0;
    const int e = ea + eb - 14;
    if (e >= -1022 && e <= 1023) return x * __longlong_as_double((long long)(e + 1023) << 52);
    return ldexp(x, e);
}

// Slices of eight consecutive values of a row with exponent e, as S
// 16-byte groups of bf16 (s_p 2^-8p, exact): digits from the residue form,
// values by an integer add and an FP32 subtract, packed two at a time.
template <int S>
__device__ __forceinline__ void slice8(const double *v, int e, uint4 *out)
{
    __nv_bfloat162 w[S][4];
#pragma unroll
    for (int q = 0; q < 8; q += 2) {
        int d0[S], d1[S];
        slice_digits_fast<S>(v[q], e, d0);
        slice_digits_fast<S>(v[q + 1], e, d1);
#pragma unroll
        for (int p = 0; p < S; ++p) w[p][q / 2] = __floats2bfloat162_rn(digit_value(d0[p], p), digit_value(d1[p], p));
    }
#pragma unroll
    for (int p = 0; p < S; ++p) out[p] = *reinterpret_cast<const uint4 *>(w[p]);
}

// ------------------------------------------------------------------ split + gather
// Both kernels walk the operand in tiles of PT_R rows x PT_K k staged in
// shared memory: the global reads run along whichever of the two dimensions
// is contiguous in the FP64 source (rfast), the slice writes along k, so
// transposed operands are read as coalesced as plain ones.
constexpr int PT_R = 32, PT_K = 64, PT_THREADS = 256;

struct PrepDesc {
    const double *src;
    __nv_bfloat16 *dst;              // [S][batch][Rp][Kp]
    int *rexp;                       // [batch][Rp] binary exponent of each row's largest entry
    int batch, R, K, Rp, Kp, Ri, Ki;
    long long s[5];                  // r0, r1, k0, k1, batch strides of the FP64 source
    long long work_start;            // prefix of tiles (batch * ceil(Rp/PT_R) * Kp/PT_K) over the launch
    long long row_start;             // prefix of batch*Rp over the launch
    long long band_start;            // prefix of bands (batch * ceil(Rp/rb)) over the launch
    int mol;
    int rfast;                       // rows (1) or k (0) are the contiguous dimension of the source
    int rb;                          // rows per band (slice_band), 0: sliced by row_scale + split_gather
};

// Operands whose padded K is at most BAND_KP are sliced in one pass by
// slice_band: rb rows x the whole K staged in shared memory (at most
// BAND_ELEMS doubles), so the row maxima come from the staged band and the
// FP64 source is read once; wider operands take row_scale + split_gather.
constexpr int BAND_KP = 1024, BAND_ELEMS = 4096;
constexpr int BAND_SMEM = (BAND_ELEMS + 64) * 8 + BAND_KP * 8 + 32 * 8 + 32 * 4 + 16;
__host__ __device__ constexpr int band_rows(int Kp) { return Kp <= 128 ? 32 : Kp <= 256 ? 16 : Kp <= 512 ? 8 : Kp <= BAND_KP ? 4 : 0; }

__device__ __forceinline__ int find_desc(const PrepDesc *pd, int n, long long w)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (pd[mid].work_start <= w) lo = mid; else hi = mid - 1;
    }
    return lo;
}

struct PrepTile {
    double x[PT_R][PT_K + 1];
    long long roff[PT_R], koff[PT_K];
    int desc;
};

// Stage tile `u` of the launch in shared memory (zero outside R x K); returns
// false (uniformly) when its molecule is inactive.
__device__ __forceinline__ bool load_tile(const PrepDesc *__restrict__ pd, int n, long long u, const int *active,
                                          PrepTile &t, int &b, int &r0, int &k0, bool skip_single = false)
{
    if (threadIdx.x == 0) t.desc = find_desc(pd, n, u);
    __syncthreads();
    const PrepDesc &d = pd[t.desc];
    if (active && !active[d.mol]) return false;
    if (d.rb) return false;                              // sliced by slice_band (holds no tiles)
    if (skip_single && d.Kp == PT_K) return false;      // split_gather scales these rows itself
    long long local = u - d.work_start;
    const int tk = d.Kp / PT_K, tr = (d.Rp + PT_R - 1) / PT_R;
    k0 = (int)(local % tk) * PT_K;
    local /= tk;
    r0 = (int)(local % tr) * PT_R;
    b = (int)(local / tr);
    for (int e = threadIdx.x; e < PT_R + PT_K; e += PT_THREADS) {
        if (e < PT_R) t.roff[e] = split_off(r0 + e, d.Ri, d.s[0], d.s[1]) + (long long)b * d.s[4];
        else t.koff[e - PT_R] = split_off(k0 + e - PT_R, d.Ki, d.s[2], d.s[3]);
    }
    __syncthreads();
    const int rlim = d.R - r0, klim = d.K - k0;
    // the tile's eight loads per thread all in flight before their shared-memory stores
    constexpr int NL = PT_R * PT_K / PT_THREADS;
    double v[NL];
#pragma unroll
    for (int j = 0; j < NL; ++j) {
        const int e = threadIdx.x + j * PT_THREADS;
        const int rr = d.rfast ? e % PT_R : e / PT_K, kk = d.rfast ? e / PT_R : e % PT_K;
        v[j] = (rr < rlim && kk < klim) ? __ldg(d.src + t.roff[rr] + t.koff[kk]) : 0.0;
    }
#pragma unroll
    for (int j = 0; j < NL; ++j) {
        const int e = threadIdx.x + j * PT_THREADS;
        const int rr = d.rfast ? e % PT_R : e / PT_K, kk = d.rfast ? e / PT_R : e % PT_K;
        t.x[rr][kk] = v[j];
    }
    __syncthreads();
    return true;
}

// Every row exponent of the launch's operands starts at INT_MIN.
__global__ void rexp_init(const PrepDesc *__restrict__ pd, int n, long long rows, const int *__restrict__ active)
{
    for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < rows; w += (long long)gridDim.x * blockDim.x) {
        int lo = 0, hi = n - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (pd[mid].row_start <= w) lo = mid; else hi = mid - 1;
        }
        const PrepDesc &d = pd[lo];
        if ((active && !active[d.mol]) || d.rb) continue;   // slice_band writes its own exponents
        d.rexp[w - d.row_start] = INT_MIN;
    }
}

// Row exponents: e with max|row| < 2^e (frexp), combined over the k tiles of a row by
// atomicMax (the list's exponents start at INT_MIN; a row that stays there is
// all zero and is treated as e = 0). Operands with one k tile per row are left
// to split_gather, which scales them from the tile it slices.
__global__ void __launch_bounds__(PT_THREADS) row_scale(const PrepDesc *__restrict__ pd, int n, long long units,
                                                        const int *__restrict__ active)
{
    __shared__ PrepTile t;
    const int rr = threadIdx.x >> 3, part = threadIdx.x & 7;
    for (long long u = blockIdx.x; u < units; u += gridDim.x) {
        int b, r0, k0;
        if (load_tile(pd, n, u, active, t, b, r0, k0, true)) {
            const PrepDesc &d = pd[t.desc];
            // magnitudes compare as their bit patterns with the sign cleared
            unsigned long long mb = 0;
#pragma unroll
            for (int kk = part; kk < PT_K; kk += 8) {
                const unsigned long long v = dbits(t.x[rr][kk]) & 0x7FFFFFFFFFFFFFFFull;
                mb = v > mb ? v : mb;
            }
#pragma unroll
            for (int o = 1; o < 8; o <<= 1) {
                const unsigned long long v = __shfl_xor_sync(0xffffffffu, mb, o);
                mb = v > mb ? v : mb;
            }
            if (part == 0 && mb != 0 && r0 + rr < d.R)
                atomicMax(&d.rexp[(long long)b * d.Rp + r0 + rr], exp_of_bits(mb));
        }
        __syncthreads();
    }
}

// Slices of each tile, K-major: the digits of x 2^(7-e) (slice_digits),
// stored as s_p 2^-8p (exact in bf16); thread = (row, 8-wide k chunk), one
// 16-byte store per slice.
template <int S>
__global__ void __launch_bounds__(PT_THREADS) split_gather(const PrepDesc *__restrict__ pd, int n, long long units,
                                                           const int *__restrict__ active)
{
    __shared__ PrepTile t;
    const int rr = threadIdx.x >> 3, c8 = (threadIdx.x & 7) * 8;
    for (long long u = blockIdx.x; u < units; u += gridDim.x) {
        int b, r0, k0;
        if (load_tile(pd, n, u, active, t, b, r0, k0)) {
            const PrepDesc &d = pd[t.desc];
            const bool in_rows = r0 + rr < d.Rp;  // a partial last row tile has rows beyond Rp: they write nothing
            int e;
            if (d.Kp == PT_K) {
                // one k tile per row (K <= 64): the row's scale from this tile,
                // so these operands skip row_scale (all lanes join the shuffle)
                unsigned long long mb = 0;
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const unsigned long long v = dbits(t.x[rr][c8 + q]) & 0x7FFFFFFFFFFFFFFFull;
                    mb = v > mb ? v : mb;
                }
#pragma unroll
                for (int o = 1; o < 8; o <<= 1) {
                    const unsigned long long v = __shfl_xor_sync(0xffffffffu, mb, o);
                    mb = v > mb ? v : mb;
                }
                if ((threadIdx.x & 7) == 0 && mb != 0 && r0 + rr < d.R)
                    d.rexp[(long long)b * d.Rp + r0 + rr] = exp_of_bits(mb);
                e = mb != 0 ? exp_of_bits(mb) : 0;
            } else {
                e = in_rows ? d.rexp[(long long)b * d.Rp + r0 + rr] : 0;
                if (e == INT_MIN) e = 0;
            }
            if (in_rows) {
                uint4 out[S];
                if (r0 + rr < d.R && k0 + c8 < d.K) {
                    double v[8];
#pragma unroll
                    for (int q = 0; q < 8; ++q) v[q] = t.x[rr][c8 + q];
                    slice8<S>(v, e, out);
                } else {                                         // zero padding: no digits to compute
#pragma unroll
                    for (int p = 0; p < S; ++p) out[p] = make_uint4(0u, 0u, 0u, 0u);
                }
                const long long plane = (long long)d.batch * d.Rp * d.Kp;
                const long long off = ((long long)b * d.Rp + r0 + rr) * d.Kp + k0 + c8;
#pragma unroll
                for (int p = 0; p < S; ++p) *reinterpret_cast<uint4 *>(d.dst + p * plane + off) = out[p];
            }
        }
        __syncthreads();
    }
}

// One pass for operands with Kp <= BAND_KP: each unit is a band of rb rows
// over the whole K, staged in shared memory (reads coalesced along the
// source's contiguous dimension); a warp per row takes the row's largest
// magnitude (bit patterns, sign cleared) and its exponent, then the slices
// are written for every (row, 8-k chunk) of the band, each slice of the
// band one contiguous run of [rb][Kp] bf16.
__device__ __forceinline__ int find_band(const PrepDesc *pd, int n, long long w)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (pd[mid].band_start <= w) lo = mid; else hi = mid - 1;
    }
    return lo;
}

template <int S>
__global__ void __launch_bounds__(PT_THREADS, 4) slice_band(const PrepDesc *__restrict__ pd, int n, long long units,
                                                         const int *__restrict__ active)
{
    extern __shared__ __align__(16) unsigned char band_raw[];
    double *x = (double *)band_raw;                                   // [rb][Kp + 2] (rows padded: fewer bank conflicts)
    long long *koff = (long long *)(x + BAND_ELEMS + 64);             // [Kp]
    long long *roff = koff + BAND_KP;                                 // [rb]
    int *rexp_s = (int *)(roff + 32);                                 // [rb]
    int *sdesc = rexp_s + 32;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (long long u = blockIdx.x; u < units; u += gridDim.x) {
        if (threadIdx.x == 0) *sdesc = find_band(pd, n, u);
        __syncthreads();
        const PrepDesc &d = pd[*sdesc];
        if (d.rb == 0 || (active && !active[d.mol])) { __syncthreads(); continue; }
        const int rb = d.rb, Kp = d.Kp, ld = Kp + 2;
        const int nb = (d.Rp + rb - 1) / rb;
        const long long local = u - d.band_start;
        const int b = (int)(local / nb), r0 = (int)(local % nb) * rb;
        for (int k = threadIdx.x; k < Kp; k += PT_THREADS) koff[k] = k < d.K ? split_off(k, d.Ki, d.s[2], d.s[3]) : 0;
        if (threadIdx.x < rb) roff[threadIdx.x] = split_off(r0 + threadIdx.x, d.Ri, d.s[0], d.s[1]) + (long long)b * d.s[4];
        __syncthreads();
        const int rlim = min(rb, d.R - r0), total = rb * Kp, K = d.K;
        const double *__restrict__ src = d.src;
        // element e of the band: rows contiguous in the source (rfast): row e % rb,
        // k e / rb (consecutive threads on consecutive rows); else row e / Kp, k
        // e % Kp. Walked by the block size without divisions, the loads of
        // eight steps in flight before their values go to shared memory.
        {
            const int lrb = rb == 32 ? 5 : rb == 16 ? 4 : rb == 8 ? 3 : 2;
            int r = d.rfast ? (threadIdx.x & (rb - 1)) : threadIdx.x / Kp;
            int k = d.rfast ? (threadIdx.x >> lrb) : threadIdx.x % Kp;
            const int dr = d.rfast ? 0 : PT_THREADS / Kp, dk = d.rfast ? (PT_THREADS >> lrb) : PT_THREADS % Kp;
            for (int e0 = 0; e0 < total; e0 += 8 * PT_THREADS) {
                double buf[8];
                int at[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const bool in = e0 + j * PT_THREADS + (int)threadIdx.x < total;
                    at[j] = in ? r * ld + k : -1;
                    buf[j] = (in && r < rlim && k < K) ? __ldg(src + roff[r] + koff[k]) : 0.0;
                    r += dr;
                    k += dk;
                    if (!d.rfast && k >= Kp) { k -= Kp; ++r; }
                }
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    if (at[j] >= 0) x[at[j]] = buf[j];
            }
        }
        __syncthreads();
        for (int r = warp; r < rb; r += PT_THREADS / 32) {
            unsigned long long mb = 0;
            for (int k = lane; k < Kp; k += 32) {
                const unsigned long long v = dbits(x[r * ld + k]) & 0x7FFFFFFFFFFFFFFFull;
                mb = v > mb ? v : mb;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long v = __shfl_xor_sync(0xffffffffu, mb, o);
                mb = v > mb ? v : mb;
            }
            if (lane == 0) {
                rexp_s[r] = mb ? exp_of_bits(mb) : 0;
                if (r < rlim) d.rexp[(long long)b * d.Rp + r0 + r] = mb ? exp_of_bits(mb) : INT_MIN;
            }
        }
        __syncthreads();
        // (row, 8-k chunk) c of the band, walked without divisions: c advances by
        // the block size, its row and k by the block size's quotient and rest
        const int cpr = Kp / 8, rows_band = min(rb, d.Rp - r0);
        const int dr = PT_THREADS / cpr, dk = (PT_THREADS % cpr) * 8;
        const long long plane = (long long)d.batch * d.Rp * Kp;
        __nv_bfloat16 *__restrict__ dst = d.dst + ((long long)b * d.Rp + r0) * Kp;
        int r = threadIdx.x / cpr, k8 = (threadIdx.x % cpr) * 8;
        const int rlive = min(rows_band, rlim);                 // rows past R and k past K are zero padding
        while (r < rows_band) {
            uint4 out[S];
            if (r < rlive && k8 < K) {
                double v[8];
#pragma unroll
                for (int q = 0; q < 8; q += 2) {
                    const double2 w2 = *reinterpret_cast<const double2 *>(x + r * ld + k8 + q);
                    v[q] = w2.x;
                    v[q + 1] = w2.y;
                }
                slice8<S>(v, rexp_s[r], out);
            } else {
#pragma unroll
                for (int p = 0; p < S; ++p) out[p] = make_uint4(0u, 0u, 0u, 0u);
            }
#pragma unroll
            for (int p = 0; p < S; ++p) *reinterpret_cast<uint4 *>(dst + p * plane + (long long)r * Kp + k8) = out[p];
            r += dr;
            k8 += dk;
            if (k8 >= Kp) { k8 -= Kp; ++r; }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ the GEMM
// Work of one output tile: its problem, batch entry, tile row and column,
// k-block range and chunks (grouped rasterisation: 16 tile-rows per group
// keep A and B blocks L2-resident).
struct TileWork {
    int di, bt, tm, tn, kb0, nkb, nchunk;
};
template <class C>
__device__ __forceinline__ TileWork tile_work(const TcDesc *__restrict__ descs, int ndesc, long long tile)
{
    TileWork w;
    int lo = 0, hi = ndesc - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (descs[mid].tile_start <= tile) lo = mid; else hi = mid - 1;
    }
    w.di = lo;
    const TcDesc &d = descs[lo];
    // a problem's tiles number below 2^31: 32-bit divisions (64-bit ones are
    // emulated, and every epilogue thread does this for every tile)
    int local = (int)(tile - d.tile_start);
    const int ks = local % d.ksplit;
    local /= d.ksplit;
    const int per_batch = d.tiles_m * d.tiles_n;
    w.bt = local / per_batch;
    local -= w.bt * per_batch;
    const int GM = 16;
    const int group = local / (GM * d.tiles_n);
    const int first_m = group * GM;
    const int gsz = min(d.tiles_m - first_m, GM);
    const int in_g = local % (GM * d.tiles_n);
    w.tm = first_m + in_g % gsz;
    w.tn = in_g / gsz;
    w.kb0 = ks * d.kb_per;
    w.nkb = min(d.Kp / C::BK - w.kb0, d.kb_per);  // >= 1 by construction
    w.nchunk = (w.nkb + C::KC - 1) / C::KC;
    return w;
}

// AND of v over the epilogue threads (named barrier 1), so that they leave
// the tile loop together and never wait at a named barrier for one another
template <int NT>
__device__ __forceinline__ bool epilogue_all(bool v)
{
    uint32_t r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.and.pred q, 1, %2, p;\n\t"
                 "selp.u32 %0, 1, 0, q;\n\t}" : "=r"(r) : "r"((uint32_t)v), "n"(NT) : "memory");
    return r != 0;
}

// Persistent: CTA b computes tiles b, b + gridDim.x, ... The producer warp
// streams k-blocks through the TMA ring and the MMA warp fills the two TMEM
// buffers with one running count each across tiles, so loads and MMAs of the
// next tile overlap the epilogue of the previous one; the epilogue stages the
// tile's (hi, lo) pairs in its own shared-memory strip and stores C with
// consecutive threads on consecutive columns.
template <class C>
__global__ void __launch_bounds__(C::NTHREADS, 1) tc_gemm(const TcDesc *__restrict__ descs, int ndesc, long long ntiles,
                                                        const int *__restrict__ active, int *err)
{
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    constexpr int LD = C::BN + 1;
    float2 *strip = (float2 *)(smem + C::STAGES * C::STAGE_BYTES);   // [STG_ROWS][BN + 1] (hi, lo) of the outputs
    double *dstrip = (double *)strip;                                 // the same, 7-slice values
    long long *srow = (long long *)(strip + C::STG_ROWS * LD);       // [BM] row offsets into C
    int *sexp = (int *)(srow + BM);                                   // [BM] row exponents of A
    uint64_t *full = (uint64_t *)(sexp + BM);
    uint64_t *empty = full + C::STAGES;
    uint64_t *acc_full = empty + C::STAGES;      // [2] MMA -> epilogue: chunk done in buffer b
    uint64_t *acc_empty = acc_full + 2;       // [2] epilogue -> MMA: buffer b drained
    uint32_t *tmem_slot = (uint32_t *)(acc_empty + 2);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < C::STAGES; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(&acc_full[b], 1); mbar_init(&acc_empty[b], C::EPI_THREADS); }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    constexpr int WP = C::EPI_WARPS, WM = C::EPI_WARPS + 1;   // producer and MMA warps
    if (warp == WM) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    bool ok = true;

    if (warp == WP) {
        if (lane == 0) {
            long long g = 0;                                  // k-blocks loaded so far
            for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
                const TileWork w = tile_work<C>(descs, ndesc, tile);
                const TcDesc &d = descs[w.di];
                if (active && !active[d.mol]) continue;
                const int arow0 = w.bt * d.Mp + w.tm * BM, brow0 = w.bt * d.Np + w.tn * C::BN;
                const int aplane = d.batch * d.Mp, bplane = d.batch * d.Np;
                for (int kb = 0; kb < w.nkb && ok; ++kb, ++g) {
                    const int st = (int)(g % C::STAGES);
                    const uint32_t ph = (uint32_t)((g / C::STAGES) & 1);
                    ok = mbar_wait(&empty[st], ph ^ 1, err, 1);
                    if (!ok) break;
                    uint8_t *sa = smem + st * C::STAGE_BYTES;
                    uint8_t *sb = sa + C::S * C::ATILE;
                    mbar_expect_tx(&full[st], C::STAGE_BYTES);
                    for (int p = 0; p < C::S; ++p) {
                        tma_load_2d(sa + p * C::ATILE, &d.mapA, &full[st], (w.kb0 + kb) * C::BK, p * aplane + arow0);
                        tma_load_2d(sb + p * C::BTILE, &d.mapB, &full[st], (w.kb0 + kb) * C::BK, p * bplane + brow0);
                    }
                }
            }
        }
    } else if (warp == WM) {
        if (lane == 0) {
            long long g = 0, gc = 0;                          // k-blocks and chunks consumed so far
            for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
                const TileWork w = tile_work<C>(descs, ndesc, tile);
                if (active && !active[descs[w.di].mol]) continue;
                for (int c = 0; c < w.nchunk && ok; ++c, ++gc) {
                    const int buf = (int)(gc & 1);
                    const uint32_t use = (uint32_t)(gc >> 1);
                    ok = mbar_wait(&acc_empty[buf], (use & 1) ^ 1, err, 4);
                    if (!ok) break;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t dbase = tmem + (uint32_t)(buf * C::NQ * C::BN);
                    const int kend = min(w.nkb, (c + 1) * C::KC);
                    for (int kb = c * C::KC; kb < kend && ok; ++kb, ++g) {
                        const int st = (int)(g % C::STAGES);
                        const uint32_t ph = (uint32_t)((g / C::STAGES) & 1);
                        ok = mbar_wait(&full[st], ph, err, 2);
                        if (!ok) break;
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        const uint32_t sa = smem_u32(smem + st * C::STAGE_BYTES);
                        const uint32_t sb = sa + C::S * C::ATILE;
                        const bool chunk_start = kb == c * C::KC;
                        // descriptors of the stage's first slices; the others differ
                        // only in the start-address field (address / 16, 14 bits:
                        // shared memory stays below 256 KB, so adding never carries)
                        const uint64_t a0 = smem_desc<C>(sa), b0 = smem_desc<C>(sb);
                        // per k-step, for each A slice i: B slices j = 0..J_i (J_i =
                        // min(S-1, QMAX-i)) stacked along N into blocks q = i..i+J_i.
                        // Blocks 0..covered were written earlier in this k-step (the
                        // ranges issued so far cover a prefix of the blocks) and
                        // accumulate; the MMA of the new blocks overwrites them at
                        // the chunk's first k-step.
#pragma unroll
                        for (int kk = 0; kk < C::BK / 16; ++kk) {
                            int covered = -1;
#pragma unroll
                            for (int i = 0; i < C::S; ++i) {
                                const int jmax = min(C::S - 1, C::QMAX - i);
                                if (jmax < 0) continue;
                                const uint64_t ad = a0 + (uint64_t)((i * C::ATILE + kk * 32) >> 4);
                                const int jold = min(jmax, covered - i);        // j = 0..jold accumulate
                                if (jold >= 0)
                                    mma_bf16(dbase + i * C::BN, ad, b0 + (uint64_t)((kk * 32) >> 4),
                                             idesc_bf16(BM, (jold + 1) * C::BN), 1u);
                                const int jnew = max(0, covered - i + 1);       // j = jnew..jmax are new
                                if (jnew <= jmax)
                                    mma_bf16(dbase + (i + jnew) * C::BN, ad,
                                             b0 + (uint64_t)((jnew * C::BTILE + kk * 32) >> 4),
                                             idesc_bf16(BM, (jmax - jnew + 1) * C::BN),
                                             (chunk_start && kk == 0) ? 0u : 1u);
                                covered = max(covered, i + jmax);
                            }
                        }
                        mma_commit(&empty[st]);
                    }
                    mma_commit(&acc_full[buf]);
                }
            }
        }
    } else {
        // epilogue: warps 0 .. EPI_WARPS-1; warp w drains TMEM lanes 32*(w%4)..
        // (output rows) and the column block w/4 of the tile
        const int row = (warp & 3) * 32 + lane;
        const int col0 = (warp >> 2) * C::EPI_COLS;
        const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
        // store: one fixed column per thread (consecutive threads on
        // consecutive n), rows RSTEP apart; all of a thread's rows of a strip
        // pass (up to 32) read from C before any is stored, so the reads of
        // C cost one round trip per pass (the drain's registers are free then)
        constexpr int RSTEP = C::EPI_THREADS / C::BN;
        constexpr int U = (C::STG_ROWS + RSTEP - 1) / RSTEP < 32 ? (C::STG_ROWS + RSTEP - 1) / RSTEP : 32;
        const int nn = threadIdx.x % C::BN, rr = threadIdx.x / C::BN;
        long long gc = 0;                                     // chunks drained so far
        for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
            const TileWork w = tile_work<C>(descs, ndesc, tile);
            const TcDesc &d = descs[w.di];
            if (active && !active[d.mol]) continue;
            float hi[C::EPI_COLS], lo[C::EPI_COLS];
            // INT_DRAIN: each exact class of a chunk is an integer count of
            // 2^-8q below 2^24, so a[q] 2^8(NX-1) is an integer below 2^56 and
            // one int64 sums every exact class of up to 32 chunks without
            // rounding; every 32 chunks it moves into an FP64 sum. The merged
            // class (about 2^-8NX of the value) is summed in FP32.
            long long iacc[C::EPI_COLS];
            double dacc[C::EPI_COLS];
            float macc[C::EPI_COLS];
#pragma unroll
            for (int e = 0; e < C::EPI_COLS; ++e) { hi[e] = 0.f; lo[e] = 0.f; iacc[e] = 0; dacc[e] = 0.0; macc[e] = 0.f; }
            for (int c = 0; c < w.nchunk; ++c, ++gc) {
                const int buf = (int)(gc & 1);
                const uint32_t use = (uint32_t)(gc >> 1);
                if (ok) ok = mbar_wait(&acc_full[buf], use & 1, err, 3);
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
                for (int c0 = 0; c0 < C::EPI_COLS; c0 += 8) {
                    // chunk value of 8 columns: the classes (exact ones first) summed
                    // by TwoSum, then added into (hi, lo); rounding errors go to lo
                    // all classes of the 8 columns in flight, one wait
                    uint32_t ra[C::NQ][8];
#pragma unroll
                    for (int q = 0; q < C::NQ; ++q)
                        tmem_ld8_issue(tmem + lane_base + (uint32_t)(buf * C::NQ * C::BN + q * C::BN + col0 + c0), ra[q]);
                    tmem_wait_ld();
                    float a[C::NQ][8];
#pragma unroll
                    for (int q = 0; q < C::NQ; ++q) {
                        tmem_tie8(ra[q]);
#pragma unroll
                        for (int e = 0; e < 8; ++e) a[q][e] = __uint_as_float(ra[q][e]);
                    }
                    if constexpr (C::INT_DRAIN) {
#pragma unroll
                        for (int e = 0; e < 8; ++e) {
                            // sum of n_q 2^8(NX-1-q) (Horner), integer arithmetic only
                            long long v = class_count(a[0][e], 0);
#pragma unroll
                            for (int q = 1; q < C::NX; ++q) v = v * 256 + class_count(a[q][e], q);
                            iacc[c0 + e] += v;
#pragma unroll
                            for (int q = C::NX; q < C::NQ; ++q) macc[c0 + e] += a[q][e];
                        }
                    } else {
#pragma unroll
                        for (int e = 0; e < 8; ++e) {
                            float x = a[0][e], err = 0.f;
#pragma unroll
                            for (int q = 1; q < C::NQ; ++q) {
                                const float sq = x + a[q][e];
                                const float bq = sq - x;
                                err += (x - (sq - bq)) + (a[q][e] - bq);
                                x = sq;
                            }
                            const float sh = hi[c0 + e] + x;
                            const float bh = sh - hi[c0 + e];
                            lo[c0 + e] += ((hi[c0 + e] - (sh - bh)) + (x - bh)) + err;
                            hi[c0 + e] = sh;
                        }
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                mbar_arrive(&acc_empty[buf]);
                if constexpr (C::INT_DRAIN) {
                    if ((c & 31) == 31) {
#pragma unroll
                        for (int e = 0; e < C::EPI_COLS; ++e) { dacc[e] += (double)iacc[e]; iacc[e] = 0; }
                    }
                }
            }
            // the tile is drained: the (hi, lo) pairs go through a shared-memory
            // strip (STG_ROWS rows at a time, all 128 where the ring leaves room)
            // so that consecutive threads store consecutive columns of C;
            // C = alpha 2^(e_m + f_n - 14) x + beta C with the power of two and
            // a power-of-two alpha applied by exponent arithmetic
            const int mv = min(BM, d.M - w.tm * BM), nv = min(C::BN, d.N - w.tn * C::BN);
            if (threadIdx.x < mv) {
                const int m = w.tm * BM + threadIdx.x;
                srow[threadIdx.x] = split_off(m, d.Mi, d.c[0], d.c[1]);
                sexp[threadIdx.x] = d.expA[(long long)w.bt * d.Mp + m];
            }
            int eb = INT_MIN;
            double *Cn = nullptr;
            if (rr < RSTEP && nn < nv) {
                const int n = w.tn * C::BN + nn;
                eb = d.expB[(long long)w.bt * d.Np + n];
                Cn = d.C + (long long)w.bt * d.c[4] + split_off(n, d.Ni, d.c[2], d.c[3]);
            }
            const bool load_c = d.ksplit == 1 && d.beta != 0.0;
            const uint32_t negmask = d.alpha_neg ? 0x80000000u : 0u;
            for (int r0 = 0; r0 < mv; r0 += C::STG_ROWS) {
                if (row >= r0 && row < r0 + C::STG_ROWS) {
#pragma unroll
                    for (int e = 0; e < C::EPI_COLS; ++e) {
                        if constexpr (C::INT_DRAIN)
                            dstrip[(row - r0) * LD + col0 + e] =
                                (dacc[e] + (double)iacc[e]) * (1.0 / (double)C::DRAIN_SCALE) + (double)macc[e];
                        else
                            strip[(row - r0) * LD + col0 + e] = make_float2(hi[e], lo[e]);
                    }
                }
                asm volatile("bar.sync 1, %0;" ::"r"(C::EPI_THREADS) : "memory");
                const int rend = min(r0 + C::STG_ROWS, mv);
                if (ok && Cn) {
                    for (int m0 = r0 + rr; m0 < rend; m0 += RSTEP * U) {
                        double old[U];
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            const int mm = m0 + u * RSTEP;
                            old[u] = (load_c && mm < rend) ? Cn[srow[mm]] : 0.0;
                        }
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            const int mm = m0 + u * RSTEP;
                            if (mm >= rend) break;
                            const int ea = sexp[mm];
                            double r = 0.0;
                            if (ea != INT_MIN && eb != INT_MIN) {
                                const int k = ea + eb - 14 + d.alpha_e;
                                bool fast = d.alpha_pow2 != 0 && k >= -896 && k <= 896;
                                if constexpr (C::INT_DRAIN) {
                                    const double v = dstrip[(mm - r0) * LD + nn];
                                    if (fast) {
                                        r = pow2_int(v, k, fast);
                                        if (d.alpha_neg) r = -r;
                                    }
                                    if (!fast) r = d.alpha * scale_pow2(v, ea, eb);
                                } else {
                                    const float2 v = strip[(mm - r0) * LD + nn];
                                    if (fast) r = f2d_pow2(v.x, k, negmask) + f2d_pow2(v.y, k, negmask);
                                    else r = d.alpha * scale_pow2((double)v.x + (double)v.y, ea, eb);
                                }
                            }
                            double *p = Cn + srow[mm];
                            if (d.ksplit > 1) atomicAdd(p, r);
                            else *p = load_c ? (d.beta_one ? r + old[u] : fma(d.beta, old[u], r)) : r;
                        }
                    }
                }
                asm volatile("bar.sync 1, %0;" ::"r"(C::EPI_THREADS) : "memory");
            }
            ok = epilogue_all<C::EPI_THREADS>(ok);
            if (!ok) break;
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == WM) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

// ------------------------------------------------------------------ tile-shape candidates
// Every precision mode has a few configurations that differ only in the
// output tile width BN (with the pipeline depth and epilogue
// warps that fit it); slices, slice pairs, exact classes, k-block depth and
// chunk length are the mode's own, so every candidate forms the same sums.
// Narrow tiles waste less on the thin operands of small molecules; wide ones
// reuse each A tile over more columns. The autotuner (choose_variant) picks one
// per plan group, precision mode and size class.
using Low32 = Cfg<3, 3, 1, 32, 3, 8, 8, 64>;
using LowS3 = Cfg<3, 3, 1, 64, 3, 8, 16, 64>;      // three stages
using Mid48 = Cfg<4, 3, 2, 48, 2, 6, 12, 64>;
using Mid32 = Cfg<4, 3, 2, 32, 2, 6, 8, 64>;
using High32 = Cfg<5, 4, 3, 32, 3, 8, 8, 32>;
using Exact16 = Cfg<7, 6, 5, 16, 3, 6, 8, 32>;
struct Variant {
    int S, BN, BK, products, smem;
    cudaError_t (*attr)();
    void (*launch)(unsigned grid, cudaStream_t s, const TcDesc *d, int nd, long long tiles, const int *act, int *err);
};
template <class C>
static cudaError_t attr_tc()
{
    return cudaFuncSetAttribute(tc_gemm<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
}
template <class C>
static void launch_tc(unsigned grid, cudaStream_t s, const TcDesc *d, int nd, long long tiles, const int *act, int *err)
{
    tc_gemm<C><<<grid, C::NTHREADS, C::SMEM_BYTES, s>>>(d, nd, tiles, act, err);
}
template <class C>
static Variant variant()
{
    return Variant{C::S, C::BN, C::BK, C::PRODUCTS, C::SMEM_BYTES, &attr_tc<C>, &launch_tc<C>};
}
constexpr int MAX_VARIANTS = 3;
static const int kNumVariants[4] = {3, 3, 2, 2};
static const Variant &variant_of(int mode, int k)
{
    static const Variant table[4][MAX_VARIANTS] = {{variant<Low>(), variant<Low32>(), variant<LowS3>()},
                                                   {variant<Mid>(), variant<Mid48>(), variant<Mid32>()},
                                                   {variant<High>(), variant<High32>(), variant<High32>()},
                                                   {variant<Exact>(), variant<Exact16>(), variant<Exact16>()}};
    return table[mode][k];
}

// ------------------------------------------------------------------ host side
struct PrepList {                    // operands sliced by one set of launches
    std::vector<PrepDesc> h;
    PrepDesc *d = nullptr;
    long long work = 0, rows = 0, bands = 0;
};

struct SubGroup {                    // one plan group in one precision mode and tile variant
    int var = 0;
    std::vector<TcDesc> tcd;         // tensor-core problems
    TcDesc *d_tcd = nullptr;
    PrepList var_ops, fixed;         // operands sliced every run / once per initialisation
    __nv_bfloat16 *fixed_buf = nullptr;   // slices of the constant operands (persistent)
    int *fixed_rexp = nullptr;
    int fixed_gen = -1;              // generation the fixed slices were made for
    long long tiles = 0;
    Group fp64;                      // problems too small for the tensor cores
};

struct Mode {                        // one precision: one SubGroup per plan group, same order
    std::vector<SubGroup> groups;
};

struct Engine {
    __nv_bfloat16 *scratch = nullptr;   // slices of the variable operands (shared by groups and modes)
    size_t scratch_elems = 0;
    int *rexp = nullptr;
    int *d_err = nullptr;
    Mode mode[4];                        // 0 = LOW, 1 = MID, 2 = HIGH, 3 = EXACT (3, 4, 5, 7 slices)
    std::vector<const Group *> keys;
    bool profile = false;
    int generation = 0;
    struct Pending { cudaEvent_t a, b; double flops, hwflops; };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> pool;
    double tot[4] = {0, 0, 0, 0};
    int nsm = 152;                       // SMs of the device: CTAs of a persistent launch
    double tune_ms = 0.0;                // time spent timing candidates at creation
};

static cudaEvent_t take_event(Engine *e)
{
    if (!e->pool.empty()) { cudaEvent_t x = e->pool.back(); e->pool.pop_back(); return x; }
    cudaEvent_t x;
    cudaEventCreate(&x);
    return x;
}

void set_profile(Engine *e, bool on) { if (e) e->profile = on; }

void invalidate(Engine *e) { if (e) ++e->generation; }

void collect(Engine *e, double out[4])
{
    if (!e) return;
    for (auto &p : e->pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
            e->tot[0] += 1; e->tot[1] += ms; e->tot[2] += p.flops; e->tot[3] += p.hwflops;
        }
        e->pool.push_back(p.a);
        e->pool.push_back(p.b);
    }
    e->pending.clear();
    if (out) for (int k = 0; k < 4; ++k) out[k] = e->tot[k];
}

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

// 2D map over slices [rows][kp] bf16: boxes of bk x box_rows, swizzled to the
// k-block's row length (128 bytes for bk = 64, 64 bytes for bk = 32).
static int make_map(CUtensorMap *map, void *base, long long rows, int kp, int box_rows, int bk)
{
    auto fn = encode_fn();
    if (!fn) { hx_set_error("cuTensorMapEncodeTiled is unavailable"); return HX_ERR_CUDA; }
    cuuint64_t dims[2] = {(cuuint64_t)kp, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)kp * 2};
    cuuint32_t box[2] = {(cuuint32_t)bk, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, base, dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, bk == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { hx_set_error("cuTensorMapEncodeTiled failed (%d)", (int)r); return HX_ERR_CUDA; }
    return HX_OK;
}

static inline long long rup(long long x, long long m) { return (x + m - 1) / m * m; }

// alpha and beta of a descriptor, with the flags of the epilogue's integer
// route: alpha = +-2^e (every coefficient of the CCSD plan) and beta == 1.
static void set_scalars(TcDesc &d, double alpha, double beta)
{
    d.alpha = alpha;
    d.beta = beta;
    int e = 0;
    const double f = std::frexp(std::fabs(alpha), &e);
    d.alpha_pow2 = (alpha != 0.0 && f == 0.5) ? 1 : 0;
    d.alpha_e = d.alpha_pow2 ? e - 1 : 0;
    d.alpha_neg = alpha < 0.0 ? 1 : 0;
    d.beta_one = beta == 1.0 ? 1 : 0;
}

// Which dimension of a source is contiguous: the one whose consecutive
// elements are closer in memory.
static int prep_rfast(const PrepDesc &p)
{
    const long long rs = p.Ri > 1 ? p.s[1] : p.s[0], ks = p.Ki > 1 ? p.s[3] : p.s[2];
    return std::llabs(rs) < std::llabs(ks) ? 1 : 0;
}

template <int S>
static cudaError_t band_attr()
{
    return cudaFuncSetAttribute(slice_band<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, BAND_SMEM);
}
// shared memory of every slice_band instance (once per device)
static cudaError_t band_attrs()
{
    cudaError_t r = band_attr<Low::S>();
    if (r == cudaSuccess) r = band_attr<Mid::S>();
    if (r == cudaSuccess) r = band_attr<High::S>();
    if (r == cudaSuccess) r = band_attr<Exact::S>();
    return r;
}

// Slices of one list of operands (n descriptors): the banded ones in one
// pass (`bands` units), the others by row exponents then slices (`tiles`
// PT_R x PT_K tiles, `rows` padded rows).
static cudaError_t prep_launch(const PrepDesc *d, int n, long long tiles, long long rows, long long bands, int S,
                               const int *active, cudaStream_t s, int nsm = 152)
{
    if (n == 0) return cudaSuccess;
    if (tiles > 0) {
        const unsigned rb = (unsigned)std::min<long long>((rows + 255) / 256, 1 << 14);
        const unsigned tb = (unsigned)std::min<long long>(tiles, 1 << 16);
        rexp_init<<<rb, 256, 0, s>>>(d, n, rows, active);
        row_scale<<<tb, PT_THREADS, 0, s>>>(d, n, tiles, active);
        if (S == Low::S) split_gather<Low::S><<<tb, PT_THREADS, 0, s>>>(d, n, tiles, active);
        else if (S == Mid::S) split_gather<Mid::S><<<tb, PT_THREADS, 0, s>>>(d, n, tiles, active);
        else if (S == High::S) split_gather<High::S><<<tb, PT_THREADS, 0, s>>>(d, n, tiles, active);
        else split_gather<Exact::S><<<tb, PT_THREADS, 0, s>>>(d, n, tiles, active);
        hx_count_launches(3);
    }
    if (bands > 0) {
        // four bands of up to 32 KB per SM
        const unsigned g = (unsigned)std::min<long long>(bands, 4LL * nsm);
        if (S == Low::S) slice_band<Low::S><<<g, PT_THREADS, BAND_SMEM, s>>>(d, n, bands, active);
        else if (S == Mid::S) slice_band<Mid::S><<<g, PT_THREADS, BAND_SMEM, s>>>(d, n, bands, active);
        else if (S == High::S) slice_band<High::S><<<g, PT_THREADS, BAND_SMEM, s>>>(d, n, bands, active);
        else slice_band<Exact::S><<<g, PT_THREADS, BAND_SMEM, s>>>(d, n, bands, active);
        hx_count_launches(1);
    }
    return cudaGetLastError();
}

// Problems below this many multiply-adds stay on the FP64 CUDA-core kernel.
// GB300's FP64 rate is about a thousandth of its BF16 tensor rate, so even
// the small contractions of 8..64-site molecules (padded to 128-row tiles)
// are faster on the tensor cores; only the tiniest stay on FP64.
static const double kMinTcWork = 1.0e4;

static bool on_tc(const TgemmDesc &t) { return (double)t.batch * t.M * t.N * t.K >= kMinTcWork; }


static void free_sub(SubGroup &sg)
{
    cudaFree(sg.d_tcd);
    cudaFree(sg.var_ops.d);
    cudaFree(sg.fixed.d);
    cudaFree(sg.fp64.d);
    cudaFree(sg.fixed_buf);
    cudaFree(sg.fixed_rexp);
    sg = SubGroup();
}

// Slice elements (and padded rows) of a group's variable operands in one variant.
static void var_need(const Group &g, const Variant &V, size_t &elems, size_t &rows)
{
    elems = rows = 0;
    for (const TgemmDesc &t : g.h) {
        if (!on_tc(t)) continue;
        const size_t Kp = rup(t.K, KPAD), Ma = rup(t.M, BM), Nb = rup(t.N, V.BN);
        if (!t.a_const) { elems += (size_t)V.S * t.batch * Ma * Kp; rows += (size_t)t.batch * Ma; }
        if (!t.b_const) { elems += (size_t)V.S * t.batch * Nb * Kp; rows += (size_t)t.batch * Nb; }
    }
}

// Descriptors, tensor maps and constant-slice storage of one plan group in
// one precision mode and tile variant.
static int build_sub(Engine *e, int mode, int var, const Group &g, SubGroup &sg)
{
    const Variant &V = variant_of(mode, var);
    const int S = V.S, BN = V.BN;
    sg = SubGroup();
    sg.var = var;
    size_t fneed = 0, frows = 0;
    for (const TgemmDesc &t : g.h) {
        if (!on_tc(t)) continue;
        const size_t Kp = rup(t.K, KPAD), Ma = rup(t.M, BM), Nb = rup(t.N, BN);
        if (t.a_const) { fneed += (size_t)S * t.batch * Ma * Kp; frows += (size_t)t.batch * Ma; }
        if (t.b_const) { fneed += (size_t)S * t.batch * Nb * Kp; frows += (size_t)t.batch * Nb; }
    }
    if ((fneed && cudaMalloc(&sg.fixed_buf, fneed * sizeof(__nv_bfloat16)) != cudaSuccess) ||
        (frows && cudaMalloc(&sg.fixed_rexp, frows * sizeof(int)) != cudaSuccess)) {
        hx_set_error("cudaMalloc of %zu bytes of constant slices failed", fneed * 2 + frows * 4);
        return HX_ERR_NOMEM;
    }
    size_t off = 0, roff = 0, foff = 0, froff = 0;
    long long tiles = 0;
    for (const TgemmDesc &t : g.h) {
        if (!on_tc(t)) { sg.fp64.h.push_back(t); continue; }
        TcDesc d;
        memset(&d, 0, sizeof(d));
        d.batch = t.batch; d.M = t.M; d.N = t.N; d.K = t.K;
        d.Mp = (int)rup(t.M, BM); d.Np = (int)rup(t.N, BN); d.Kp = (int)rup(t.K, KPAD);
        d.Mi = t.Mi; d.Ni = t.Ni;
        for (int k = 0; k < 5; ++k) d.c[k] = t.c[k];
        set_scalars(d, t.alpha, t.beta);
        d.C = t.C; d.mol = t.mol;
        d.tiles_m = d.Mp / BM; d.tiles_n = d.Np / BN;
        // long K over few output tiles: cut K into slices that fill the GPU
        const int nkb = d.Kp / V.BK, n64 = d.Kp / KPAD;
        const long long out_tiles = (long long)d.batch * d.tiles_m * d.tiles_n;
        int ks = 1;
        if (t.beta == 1.0 && out_tiles < e->nsm && n64 >= 16)
            ks = (int)std::min<long long>((e->nsm + out_tiles - 1) / out_tiles, n64 / 8);
        d.kb_per = (nkb + ks - 1) / ks;
        d.ksplit = (nkb + d.kb_per - 1) / d.kb_per;
        d.tile_start = tiles;
        tiles += out_tiles * d.ksplit;
        const size_t asz = (size_t)S * d.batch * d.Mp * d.Kp;
        const size_t bsz = (size_t)S * d.batch * d.Np * d.Kp;
        __nv_bfloat16 *abuf, *bbuf;
        int *aexp, *bexp;
        if (t.a_const) { abuf = sg.fixed_buf + foff; foff += asz; aexp = sg.fixed_rexp + froff; froff += (size_t)t.batch * d.Mp; }
        else { abuf = e->scratch + off; off += asz; aexp = e->rexp + roff; roff += (size_t)t.batch * d.Mp; }
        if (t.b_const) { bbuf = sg.fixed_buf + foff; foff += bsz; bexp = sg.fixed_rexp + froff; froff += (size_t)t.batch * d.Np; }
        else { bbuf = e->scratch + off; off += bsz; bexp = e->rexp + roff; roff += (size_t)t.batch * d.Np; }
        if (off > e->scratch_elems) { hx_set_error("tensor-core scratch overflow"); return HX_ERR_STATE; }
        int rc = make_map(&d.mapA, abuf, (long long)S * d.batch * d.Mp, d.Kp, BM, V.BK);
        if (rc == HX_OK) rc = make_map(&d.mapB, bbuf, (long long)S * d.batch * d.Np, d.Kp, BN, V.BK);
        if (rc < 0) return rc;
        PrepDesc pa, pb;
        memset(&pa, 0, sizeof(pa));
        pa.src = t.A; pa.dst = abuf; pa.batch = t.batch; pa.R = t.M; pa.K = t.K;
        pa.Rp = d.Mp; pa.Kp = d.Kp; pa.Ri = t.Mi; pa.Ki = t.Ki; pa.mol = t.mol;
        pa.s[0] = t.a[0]; pa.s[1] = t.a[1]; pa.s[2] = t.a[2]; pa.s[3] = t.a[3]; pa.s[4] = t.a[4];
        pa.rexp = aexp;
        d.expA = aexp;
        pb = pa;
        pb.src = t.B; pb.dst = bbuf; pb.R = t.N; pb.Rp = d.Np; pb.Ri = t.Ni;
        pb.s[0] = t.b[0]; pb.s[1] = t.b[1]; pb.s[2] = t.b[2]; pb.s[3] = t.b[3]; pb.s[4] = t.b[4];
        pb.rexp = bexp;
        d.expB = bexp;
        auto add = [&](PrepList &L, PrepDesc p) {
            p.work_start = L.work;
            p.row_start = L.rows;
            p.band_start = L.bands;
            p.rfast = prep_rfast(p);
            p.rb = band_rows(p.Kp);
            if (p.rb) L.bands += (long long)p.batch * ((p.Rp + p.rb - 1) / p.rb);
            else L.work += (long long)p.batch * ((p.Rp + PT_R - 1) / PT_R) * (p.Kp / PT_K);
            L.rows += (long long)p.batch * p.Rp;
            L.h.push_back(p);
        };
        add(t.a_const ? sg.fixed : sg.var_ops, pa);
        add(t.b_const ? sg.fixed : sg.var_ops, pb);
        sg.tcd.push_back(d);
    }
    sg.tiles = tiles;
    if (!sg.tcd.empty()) {
        if (cudaMalloc(&sg.d_tcd, sizeof(TcDesc) * sg.tcd.size()) != cudaSuccess) {
            hx_set_error("descriptor allocation failed");
            return HX_ERR_NOMEM;
        }
        cudaMemcpy(sg.d_tcd, sg.tcd.data(), sizeof(TcDesc) * sg.tcd.size(), cudaMemcpyHostToDevice);
        for (PrepList *L : {&sg.var_ops, &sg.fixed}) {
            if (L->h.empty()) continue;
            if (cudaMalloc(&L->d, sizeof(PrepDesc) * L->h.size()) != cudaSuccess) {
                hx_set_error("descriptor allocation failed");
                return HX_ERR_NOMEM;
            }
            cudaMemcpy(L->d, L->h.data(), sizeof(PrepDesc) * L->h.size(), cudaMemcpyHostToDevice);
        }
    }
    if (!sg.fp64.h.empty()) {
        sg.fp64.tiles = hx_tgemm_f64_prepare(sg.fp64.h.data(), (int)sg.fp64.h.size());
        if (cudaMalloc(&sg.fp64.d, sizeof(TgemmDesc) * sg.fp64.h.size()) != cudaSuccess) {
            hx_set_error("descriptor allocation failed");
            return HX_ERR_NOMEM;
        }
        cudaMemcpy(sg.fp64.d, sg.fp64.h.data(), sizeof(TgemmDesc) * sg.fp64.h.size(), cudaMemcpyHostToDevice);
    }
    return HX_OK;
}

// One plan group in its mode and variant: slice the operands (the constant
// ones once per initialisation), then the persistent tcgen05 GEMM.
static cudaError_t run_sub(Engine *e, SubGroup &sg, int mode, const int *d_active, cudaStream_t s)
{
    const Variant &V = variant_of(mode, sg.var);
    if (sg.fp64.tiles > 0) {
        cudaError_t r = hx_tgemm_f64_launch(sg.fp64.d, (int)sg.fp64.h.size(), sg.fp64.tiles, d_active, s);
        if (r != cudaSuccess) return r;
    }
    if (sg.tiles == 0) return cudaSuccess;
    cudaError_t r = cudaSuccess;
    // constant slices are made once per initialisation, for every molecule
    // (molecules enter a mode at different iterations)
    if (sg.fixed_gen != e->generation) {
        if ((r = prep_launch(sg.fixed.d, (int)sg.fixed.h.size(), sg.fixed.work, sg.fixed.rows, sg.fixed.bands, V.S,
                             nullptr, s, e->nsm)) != cudaSuccess)
            return r;
        sg.fixed_gen = e->generation;
    }
    if ((r = prep_launch(sg.var_ops.d, (int)sg.var_ops.h.size(), sg.var_ops.work, sg.var_ops.rows, sg.var_ops.bands,
                         V.S, d_active, s, e->nsm)) != cudaSuccess)
        return r;
    hx_count_launches(1);
    Engine::Pending pend{};
    if (e->profile) {
        pend.a = take_event(e);
        pend.b = take_event(e);
        for (const TcDesc &d : sg.tcd) {
            pend.flops += 2.0 * d.batch * (double)d.M * d.N * d.K;
            pend.hwflops += 2.0 * d.batch * (double)d.Mp * d.Np * d.Kp * V.products;
        }
        cudaEventRecord(pend.a, s);
    }
    // persistent: one CTA per SM (shared memory allows one), each looping over tiles
    const unsigned grid = (unsigned)std::min<long long>(sg.tiles, e->nsm);
    V.launch(grid, s, sg.d_tcd, (int)sg.tcd.size(), sg.tiles, d_active, e->d_err);
    r = cudaGetLastError();
    if (e->profile) {
        cudaEventRecord(pend.b, s);
        e->pending.push_back(pend);
    }
    return r;
}

// ------------------------------------------------------------------ autotuner
// The tile variant of each (precision mode, plan group, size class): size
// class = (ceil log2 of the widest output column count N, floor log2 of the
// group's multiply-adds). Choices live in one process-wide table, filled from
// a shipped table (hx_tile_table_load) or by timing every candidate on the
// handle's own contraction shapes at creation (tuning = 1, on a table miss).
using TileKey = std::array<int, 4>;
static std::mutex g_tile_mu;
static std::map<TileKey, int> g_tile_table;

static TileKey tile_key(int mode, int gi, const Group &g)
{
    long long maxn = 0;
    double work = 0.0;
    for (const TgemmDesc &t : g.h) {
        if (!on_tc(t)) continue;
        maxn = std::max<long long>(maxn, t.N);
        work += (double)t.batch * t.M * t.N * t.K;
    }
    int nb = 0;
    while ((1LL << nb) < maxn) ++nb;
    return TileKey{mode, gi, nb, work > 0.0 ? (int)std::floor(std::log2(work)) : 0};
}

// Time every candidate of one group (one warm-up run that also slices the
// constant operands, then the mean of three runs, CUDA events on s) and
// return the fastest; *ms gets the time spent.
static int tune_group(Engine *e, int mode, const Group &g, cudaStream_t s, int *best, double *spent)
{
    *best = 0;
    float best_ms = 1e30f;
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
        hx_set_error("autotuner: cudaEventCreate failed");
        return HX_ERR_CUDA;
    }
    const auto t0 = std::chrono::steady_clock::now();
    int rc = HX_OK;
    for (int v = 0; v < kNumVariants[mode] && rc == HX_OK; ++v) {
        SubGroup sg;
        rc = build_sub(e, mode, v, g, sg);
        if (rc == HX_OK && sg.tiles == 0) { free_sub(sg); break; }
        cudaError_t ce = cudaSuccess;
        if (rc == HX_OK) ce = run_sub(e, sg, mode, nullptr, s);
        if (rc == HX_OK && ce == cudaSuccess) ce = cudaEventRecord(a, s);
        for (int r = 0; r < 3 && rc == HX_OK && ce == cudaSuccess; ++r) ce = run_sub(e, sg, mode, nullptr, s);
        if (rc == HX_OK && ce == cudaSuccess) ce = cudaEventRecord(b, s);
        if (rc == HX_OK && ce == cudaSuccess) ce = cudaEventSynchronize(b);
        float ms = 0.f;
        if (rc == HX_OK && ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, a, b);
        free_sub(sg);
        if (rc == HX_OK && ce != cudaSuccess) { hx_set_error("autotuner: %s", cudaGetErrorString(ce)); rc = HX_ERR_CUDA; }
        if (rc == HX_OK && error_word(e) != 0) { hx_set_error("autotuner: a tensor-core wait timed out"); rc = HX_ERR_KERNEL; }
        if (rc == HX_OK && ms < best_ms) { best_ms = ms; *best = v; }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    *spent += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

static int choose_variant(Engine *e, int mode, int gi, const Group &g, cudaStream_t s, int tuning, int force)
{
    if (force >= 0) return std::min(force, kNumVariants[mode] - 1);
    const TileKey key = tile_key(mode, gi, g);
    if (tuning != 2) {
        std::lock_guard<std::mutex> lock(g_tile_mu);
        auto it = g_tile_table.find(key);
        if (it != g_tile_table.end()) return std::min(it->second, kNumVariants[mode] - 1);
    }
    if (tuning != 1) return 0;
    int best = 0;
    const int rc = tune_group(e, mode, g, s, &best, &e->tune_ms);
    if (rc < 0) return rc;
    std::lock_guard<std::mutex> lock(g_tile_mu);
    g_tile_table[key] = best;
    return best;
}

int create(Engine **out, const std::vector<Group> &plan, cudaStream_t s, int tuning, int force, int only_mode)
{
    *out = nullptr;
    Engine *e = new Engine();
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&e->nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || e->nsm < 1) {
        delete e;
        hx_set_error("cannot query the device's multiprocessor count");
        return HX_ERR_CUDA;
    }
    // variable operands share one scratch: the largest group of any mode and variant
    size_t need = 0, need_rows = 0;
    for (int md = 0; md < 4; ++md)
        for (int v = 0; v < kNumVariants[md] && (only_mode < 0 || md == only_mode); ++v)
            for (const Group &g : plan) {
                size_t ge, gr;
                var_need(g, variant_of(md, v), ge, gr);
                need = std::max(need, ge);
                need_rows = std::max(need_rows, gr);
            }
    if ((need && cudaMalloc(&e->scratch, need * sizeof(__nv_bfloat16)) != cudaSuccess) ||
        (need_rows && cudaMalloc(&e->rexp, need_rows * sizeof(int)) != cudaSuccess) ||
        cudaMalloc(&e->d_err, sizeof(int)) != cudaSuccess) {
        hx_set_error("cudaMalloc of %zu bytes of tensor-core scratch failed", need * 2 + need_rows * 4);
        destroy(e);
        return HX_ERR_NOMEM;
    }
    e->scratch_elems = need;
    cudaMemsetAsync(e->d_err, 0, sizeof(int), s);
    for (int md = 0; md < 4; ++md)
        for (int v = 0; v < kNumVariants[md]; ++v)
            if (variant_of(md, v).attr() != cudaSuccess) {
                destroy(e);
                hx_set_error("cannot reserve shared memory for tc_gemm");
                return HX_ERR_CUDA;
            }
    if (band_attrs() != cudaSuccess) {
        destroy(e);
        hx_set_error("cannot reserve shared memory for slice_band");
        return HX_ERR_CUDA;
    }
    for (int md = 0; md < 4; ++md)
        for (size_t gi = 0; gi < plan.size(); ++gi) {
            if (only_mode >= 0 && md != only_mode) { e->mode[md].groups.emplace_back(); continue; }
            int var = choose_variant(e, md, (int)gi, plan[gi], s, tuning, force);
            if (var < 0) { destroy(e); return var; }
            SubGroup sg;
            int rc = build_sub(e, md, var, plan[gi], sg);
            e->mode[md].groups.push_back(std::move(sg));
            if (rc < 0) { destroy(e); return rc; }
        }
    for (const Group &g : plan) e->keys.push_back(&g);
    ++e->generation;                  // tuning runs made constant slices of zeros: make them again
    *out = e;
    return HX_OK;
}

cudaError_t run_group(Engine *e, const TgemmDesc *descs, int n, const int *d_active, cudaStream_t s, int mode)
{
    int gi = -1;
    for (size_t k = 0; k < e->keys.size(); ++k)
        if (e->keys[k]->h.data() == descs) { gi = (int)k; break; }
    if (gi < 0 || mode < 0 || mode > 3) return cudaErrorInvalidValue;
    (void)n;
    return run_sub(e, e->mode[mode].groups[gi], mode, d_active, s);
}

cudaError_t prepare_fixed(Engine *e, cudaStream_t s)
{
    if (!e) return cudaSuccess;
    for (int md = 0; md < 4; ++md)
        for (SubGroup &sg : e->mode[md].groups) {
            if (sg.tiles == 0 || sg.fixed_gen == e->generation) continue;
            const cudaError_t r = prep_launch(sg.fixed.d, (int)sg.fixed.h.size(), sg.fixed.work, sg.fixed.rows,
                                              sg.fixed.bands, variant_of(md, sg.var).S, nullptr, s, e->nsm);
            if (r != cudaSuccess) return r;
            sg.fixed_gen = e->generation;
        }
    return cudaSuccess;
}

int error_word(Engine *e)
{
    int v = 0;
    if (e && e->d_err) cudaMemcpy(&v, e->d_err, sizeof(int), cudaMemcpyDeviceToHost);
    return v;
}

int choices(Engine *e, int *var, int cap)
{
    const int ng = e ? (int)e->keys.size() : 0;
    for (int md = 0; md < 4; ++md)
        for (int gi = 0; gi < ng; ++gi)
            if (var && md * ng + gi < cap) var[md * ng + gi] = e->mode[md].groups[gi].var;
    return 4 * ng;
}

double tune_ms(Engine *e) { return e ? e->tune_ms : 0.0; }

void destroy(Engine *e)
{
    if (!e) return;
    for (Mode &md : e->mode)
        for (auto &g : md.groups) free_sub(g);
    for (auto &p : e->pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    for (auto x : e->pool) cudaEventDestroy(x);
    cudaFree(e->scratch);
    cudaFree(e->rexp);
    cudaFree(e->d_err);
    delete e;
}

int table_get(int *entries, int cap)
{
    std::lock_guard<std::mutex> lock(g_tile_mu);
    int k = 0;
    for (const auto &kv : g_tile_table) {
        if (entries && k < cap)
            for (int c = 0; c < 4; ++c) entries[5 * k + c] = kv.first[c];
        if (entries && k < cap) entries[5 * k + 4] = kv.second;
        ++k;
    }
    return k;
}

int table_load(const int *entries, int n)
{
    std::lock_guard<std::mutex> lock(g_tile_mu);
    for (int k = 0; k < n; ++k) {
        const int *x = entries + 5 * k;
        if (x[0] < 0 || x[0] > 3 || x[4] < 0 || x[4] >= kNumVariants[x[0]]) {
            hx_set_error("tile table entry %d: mode %d, variant %d out of range", k, x[0], x[4]);
            return HX_ERR_ARG;
        }
        g_tile_table[TileKey{x[0], x[1], x[2], x[3]}] = x[4];
    }
    return HX_OK;
}

int variants(int mode, int *bn, int cap)
{
    if (mode < 0 || mode > 3) return HX_ERR_ARG;
    for (int k = 0; k < kNumVariants[mode] && bn && k < cap; ++k) bn[k] = variant_of(mode, k).BN;
    return kNumVariants[mode];
}
}  // namespace tc

// ------------------------------------------------------------------ allocation-free single GEMM
// hx_gemm_noalloc: one C = A B^T on the tensor cores with every piece of
// scratch (operand slices, row exponents, the error word, the descriptors) in
// one file-scope device array, so that a call allocates no memory: for hosts
// whose device memory belongs to their own pool allocator, or that must not
// let a cudaFree synchronise the device. Every GPU that loads the library
// holds the array until exit; its size bounds the problem: M, N, K <=
// HX_NOALLOC_MAX_DIM (512), about 5.3 MB.
namespace tc {
namespace {

constexpr size_t na_rup(size_t x, size_t m) { return (x + m - 1) / m * m; }
constexpr int NA_DIM = HX_NOALLOC_MAX_DIM;
constexpr int na_max(int a, int b) { return a > b ? a : b; }
// padded rows of A (to 128) and of B (to either mode's tile width), padded K
constexpr int NA_AROWS = (int)na_rup(NA_DIM, BM);
constexpr int NA_BROWS = na_max((int)na_rup(NA_DIM, Low::BN), (int)na_rup(NA_DIM, High::BN));
constexpr int NA_KP = (int)na_rup(NA_DIM, KPAD);
constexpr size_t NA_A_BYTES = (size_t)na_max(Low::S, High::S) * NA_AROWS * NA_KP * sizeof(__nv_bfloat16);
constexpr size_t NA_B_BYTES = (size_t)na_max(Low::S * (int)na_rup(NA_DIM, Low::BN), High::S * (int)na_rup(NA_DIM, High::BN)) *
                              NA_KP * sizeof(__nv_bfloat16);
constexpr size_t NA_OFF_A = 0;
constexpr size_t NA_OFF_B = na_rup(NA_OFF_A + NA_A_BYTES, 1024);
constexpr size_t NA_OFF_REXP = na_rup(NA_OFF_B + NA_B_BYTES, 256);          // int[NA_AROWS + NA_BROWS]
constexpr size_t NA_OFF_ERR = NA_OFF_REXP + (size_t)(NA_AROWS + NA_BROWS) * sizeof(int);
constexpr size_t NA_OFF_TCD = na_rup(NA_OFF_ERR + sizeof(int), 256);
constexpr size_t NA_OFF_PREP = na_rup(NA_OFF_TCD + sizeof(TcDesc), 256);
constexpr size_t NA_BYTES = na_rup(NA_OFF_PREP + 2 * sizeof(PrepDesc), 256);

static __device__ __align__(256) unsigned char g_na_scratch[NA_BYTES];

constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mutex;
unsigned char *g_na_base[NA_MAX_DEVICES] = {};

// Address of the static scratch on the current device, looked up once per
// device (the first call on a device must not be inside a stream capture) and
// kept for the life of the library: a device reset while it is loaded would
// leave a stale address, and is not supported.
int na_setup(unsigned char **base)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) {
        hx_set_error("hx_gemm_noalloc: no usable current device");
        return HX_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_base[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_na_scratch);
        if (e != cudaSuccess || !p) {
            hx_set_error("hx_gemm_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return HX_ERR_CUDA;
        }
        if (cudaFuncSetAttribute(tc_gemm<Low>, cudaFuncAttributeMaxDynamicSharedMemorySize, Low::SMEM_BYTES) != cudaSuccess ||
            cudaFuncSetAttribute(tc_gemm<High>, cudaFuncAttributeMaxDynamicSharedMemorySize, High::SMEM_BYTES) != cudaSuccess ||
            band_attrs() != cudaSuccess) {
            hx_set_error("hx_gemm_noalloc: cannot reserve shared memory for tc_gemm");
            return HX_ERR_CUDA;
        }
        g_na_base[dev] = (unsigned char *)p;
    }
    *base = g_na_base[dev];
    return HX_OK;
}

}  // namespace
}  // namespace tc

extern "C" int hx_gemm_noalloc(const double *dA, const double *dB, double *dC, int32_t M, int32_t N, int32_t K,
                               int32_t precision, void *stream)
{
    using namespace tc;
    if (!dA || !dB || !dC || M <= 0 || N <= 0 || K <= 0) { hx_set_error("hx_gemm_noalloc: bad arguments"); return HX_ERR_ARG; }
    if (M > HX_NOALLOC_MAX_DIM || N > HX_NOALLOC_MAX_DIM || K > HX_NOALLOC_MAX_DIM) {
        hx_set_error("hx_gemm_noalloc: M=%d N=%d K=%d exceeds the static scratch limit of %d per dimension", M, N, K,
                     HX_NOALLOC_MAX_DIM);
        return HX_ERR_ARG;
    }
    if (precision != HX_PRECISION_MIXED && precision != 2) {
        hx_set_error("hx_gemm_noalloc: precision must be 1 (3 slices) or 2 (5 slices)");
        return HX_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    // the call ends with a read-back and a stream synchronisation, neither of
    // which a capture may record: refuse before touching the stream
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
        hx_set_error("hx_gemm_noalloc: the stream is being captured (the call synchronises its stream)");
        return HX_ERR_ARG;
    }
    unsigned char *base = nullptr;
    int rc = na_setup(&base);
    if (rc != HX_OK) return rc;
    const bool high = precision == 2;
    const int S = high ? High::S : Low::S, BN = high ? High::BN : Low::BN;

    __nv_bfloat16 *abuf = (__nv_bfloat16 *)(base + NA_OFF_A), *bbuf = (__nv_bfloat16 *)(base + NA_OFF_B);
    int *aexp = (int *)(base + NA_OFF_REXP), *bexp = aexp + NA_AROWS;
    int *err = (int *)(base + NA_OFF_ERR);
    TcDesc *d_tcd = (TcDesc *)(base + NA_OFF_TCD);
    PrepDesc *d_prep = (PrepDesc *)(base + NA_OFF_PREP);

    // the descriptor of hx_gemm's single problem: C = 1 * A B^T + 1 * C on a zeroed C
    TcDesc d;
    memset(&d, 0, sizeof(d));
    d.batch = 1; d.M = M; d.N = N; d.K = K;
    const int BK = high ? High::BK : Low::BK;
    d.Mp = (int)rup(M, BM); d.Np = (int)rup(N, BN); d.Kp = (int)rup(K, KPAD);
    d.Mi = M; d.Ni = N;
    d.c[0] = 0; d.c[1] = N; d.c[2] = 0; d.c[3] = 1; d.c[4] = 0;
    set_scalars(d, 1.0, 1.0);
    d.C = dC; d.mol = 0;
    d.tiles_m = d.Mp / BM; d.tiles_n = d.Np / BN;
    d.kb_per = d.Kp / BK;            // K <= 512: at most 16 k-blocks, never split
    d.ksplit = 1;
    d.tile_start = 0;
    d.expA = aexp; d.expB = bexp;
    if ((rc = make_map(&d.mapA, abuf, (long long)S * d.Mp, d.Kp, BM, BK)) != HX_OK) return rc;
    if ((rc = make_map(&d.mapB, bbuf, (long long)S * d.Np, d.Kp, BN, BK)) != HX_OK) return rc;
    PrepDesc p[2];
    memset(p, 0, sizeof(p));
    p[0].src = dA; p[0].dst = abuf; p[0].rexp = aexp; p[0].batch = 1; p[0].R = M; p[0].K = K;
    p[0].Rp = d.Mp; p[0].Kp = d.Kp; p[0].Ri = M; p[0].Ki = K;
    p[0].s[0] = 0; p[0].s[1] = K; p[0].s[2] = 0; p[0].s[3] = 1; p[0].s[4] = 0;
    p[1] = p[0];
    p[1].src = dB; p[1].dst = bbuf; p[1].rexp = bexp; p[1].R = N; p[1].Rp = d.Np; p[1].Ri = N;
    p[0].rfast = prep_rfast(p[0]);
    p[1].rfast = prep_rfast(p[1]);
    // K <= 512: both operands are sliced in one pass, in bands of rb rows
    const int rb = band_rows(d.Kp);
    p[0].rb = p[1].rb = rb;
    p[1].band_start = (d.Mp + rb - 1) / rb;
    p[1].row_start = d.Mp;
    const long long rows = (long long)d.Mp + d.Np;
    const long long bands = p[1].band_start + (d.Np + rb - 1) / rb;
    const long long tiles = (long long)d.tiles_m * d.tiles_n;

    // what must start at zero: the error word and C (accumulated with beta = 1)
    cudaError_t ce = cudaMemsetAsync(err, 0, sizeof(int), s);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(dC, 0, sizeof(double) * (size_t)M * N, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_tcd, &d, sizeof(d), cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(d_prep, p, sizeof(p), cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess) {
        ce = prep_launch(d_prep, 2, 0, rows, bands, S, nullptr, s);
        // one CTA per tile (the kernel's tile loop then runs once per CTA)
        if (ce == cudaSuccess && high) tc_gemm<High><<<(unsigned)tiles, High::NTHREADS, High::SMEM_BYTES, s>>>(d_tcd, 1, tiles, nullptr, err);
        else if (ce == cudaSuccess) tc_gemm<Low><<<(unsigned)tiles, Low::NTHREADS, Low::SMEM_BYTES, s>>>(d_tcd, 1, tiles, nullptr, err);
        hx_count_launches(1);
        if (ce == cudaSuccess) ce = cudaGetLastError();
    }
    int werr = 0;
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&werr, err, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) { hx_set_error("hx_gemm_noalloc: %s", cudaGetErrorString(ce)); return HX_ERR_CUDA; }
    if (werr) { hx_set_error("hx_gemm_noalloc: tensor-core wait timed out (code %d)", werr); return HX_ERR_KERNEL; }
    return HX_OK;
}
