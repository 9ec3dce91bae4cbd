// Learned T2 initial guess: a 4-layer MLP (8 -> 256 -> 256 -> 256 -> 1, SiLU)
// that predicts, per amplitude, t2(converged) - t2(reference guess).
//
// Inputs of the amplitude t2(i,a,j,b) with (ia) <= (jb):
//   the reference guess L(iajb)/D(iajb) (guessCC), e_i, e_j, e_a, e_b (MO Fock
//   diagonal), (ia|jb), (ib|ja) and 8/N (molecule size).
// Only canonical pairs are evaluated and the result is written to both t2
// entries of the pair, so the guess keeps the pair symmetry of t2 exactly.
//
// Inference (mlp_infer, one CTA per SM looping over 128-row tiles): layer 1
// runs on the CUDA cores and writes bf16 activations straight into shared
// memory in the 128-byte-swizzled K-major layout the tensor core reads;
// layers 2 and 3 are tcgen05.mma (kind::f16, BF16 x BF16 -> FP32, M = 128,
// N = 256, K = 256) with the bf16 weights brought in by TMA and the
// accumulator in 256 TMEM columns; their epilogues (tcgen05.ld, bias, SiLU,
// bf16) feed the next layer through shared memory; the output layer is a dot
// product in the last epilogue. In the engine the features are computed from
// the molecule's device state inside the kernel and the result goes straight
// into t2.
//
// Training (hx_mlp_grad / hx_mlp_train): the six 256-wide products of a step
// (layers 2 and 3 forward, their weight gradients and the gradients of their
// inputs) on the tensor cores (bgemm: bf16 operands brought in by TMA, FP32
// accumulation in TMEM), with the same bf16 roundings as inference (W2, W3
// and the activations entering layers 2 and 3) plus the loss gradients
// entering those products (straight-through in the backward pass); the
// 8-wide first layer, the output unit and the bias sums on the CUDA cores.
// Mean-squared error in units of y_scale, Adam with a cosine learning-rate
// decay. The gradients are those of the CPU reference in oracle/mlp.py.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "hx_common.cuh"
#include "hx_mlp.h"

namespace mlp {

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z)
{
    const float s = 1.f / (1.f + __expf(-z));
    return s * (1.f + z * (1.f - s));
}
__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// ------------------------------------------------------------------ features
// canonical pair index r -> (p, q), p <= q, rows of the upper triangle of an n x n matrix
__device__ __forceinline__ void tri_index(long long r, long long n, long long &p, long long &q)
{
    const double nn = (double)n + 0.5;
    long long pp = (long long)(nn - sqrt(fmax(nn * nn - 2.0 * (double)r, 0.0)));
    if (pp < 0) pp = 0;
    if (pp > n - 1) pp = n - 1;
    while (pp > 0 && pp * n - pp * (pp - 1) / 2 > r) --pp;
    while (pp + 1 < n && (pp + 1) * n - (pp + 1) * pp / 2 <= r) ++pp;
    p = pp;
    q = pp + (r - (pp * n - pp * (pp - 1) / 2));
}

// features of canonical pair (p, q); returns the flat pair index p*ov + q
__device__ long long pair_features(const CCMol &m, long long p, long long q, float *f, double &guess)
{
    const int o = m.o, v = m.v, n = m.N;
    const long long ov = (long long)o * v;
    const int i = (int)(p / v), a = (int)(p % v), j = (int)(q / v), b = (int)(q % v);
    const long long pq = p * ov + q;
    const long long p2 = (long long)i * v + b, q2 = (long long)j * v + a;
    guess = m.Lov[pq] / m.D2[pq];
    f[0] = (float)guess;
    f[1] = (float)m.Fmo[(long long)i * n + i];
    f[2] = (float)m.Fmo[(long long)j * n + j];
    f[3] = (float)m.Fmo[(long long)(o + a) * n + o + a];
    f[4] = (float)m.Fmo[(long long)(o + b) * n + o + b];
    f[5] = (float)m.gov[pq];
    f[6] = (float)m.gov[(p2 < q2 ? p2 : q2) * ov + (p2 < q2 ? q2 : p2)];
    f[7] = 8.f / (float)n;
    return pq;
}

// training rows: features and target t2 - guess of the given canonical pairs
__global__ void k_sample(const CCMol *mols, int mol, const long long *rows, int n, float *X, float *T)
{
    const CCMol &m = mols[mol];
    const long long ov = (long long)m.o * m.v;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        long long p, q;
        tri_index(rows[k], ov, p, q);
        double g;
        const long long pq = pair_features(m, p, q, X + (long long)k * F, g);
        T[k] = (float)(m.t2[pq] - g);
    }
}

// ------------------------------------------------------------------ tcgen05 inference
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// bounded wait (4 s): false and an error code if the phase never completes
__device__ __forceinline__ bool wait_bar(uint64_t *bar, uint32_t parity, int *err, int code)
{
    const unsigned long long t0 = gtimer();
    for (;;) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
        if (gtimer() - t0 > 4000000000ull) {
            if (err) atomicCAS(err, 0, code);
            return false;
        }
    }
}
// shared-memory descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr)
{
    return (uint64_t)((addr & 0x3FFFF) >> 4) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
           ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}
// byte offset of the 16-byte chunk c (elements 8c..8c+7) of row `row` in a [rows x 64] bf16 K-block
__device__ __forceinline__ uint32_t sw128_chunk(int row, int c) { return (uint32_t)(row * 128 + (((c ^ row) & 7) << 4)); }

constexpr int TILE = 128;
constexpr int A_KB = TILE * 128;               // one K-block of activations: 128 rows x 64 bf16
constexpr int B_KB = H * 128;                  // one K-block of weights: 256 rows x 64 bf16
constexpr int A_BYTES = 4 * A_KB;              // 64 KB
constexpr int B_BYTES = 4 * B_KB;              // 128 KB
constexpr int MLP_THREADS = 256;
constexpr int MLP_SMEM = 1024 + A_BYTES + B_BYTES + (H * F + 4 * H + TILE) * 4;

struct InferArgs {
    const float *X;          // [n x F] features (hx_mlp_predict) or NULL (engine)
    float *Y;                // [n] predictions (hx_mlp_predict)
    const CCMol *mols;       // engine: molecules, the one used, first canonical pair
    int mol;
    long long row0;
    long long n;
    const float *P;
    int *err;
};

// one row's input and the pair it belongs to
__device__ __forceinline__ void load_row(const InferArgs &a, long long gr, float *x, long long &pq, long long &qp,
                                         double &guess)
{
    pq = qp = -1;
    guess = 0.0;
    if (gr >= a.n) {
#pragma unroll
        for (int f = 0; f < F; ++f) x[f] = 0.f;
        return;
    }
    if (a.X) {
#pragma unroll
        for (int f = 0; f < F; ++f) x[f] = a.X[gr * F + f];
        return;
    }
    const CCMol &m = a.mols[a.mol];
    const long long ov = (long long)m.o * m.v;
    long long p, q;
    tri_index(a.row0 + gr, ov, p, q);
    pq = pair_features(m, p, q, x, guess);
    qp = q * ov + p;
}

__global__ void __launch_bounds__(MLP_THREADS, 1) mlp_infer(InferArgs a, const __grid_constant__ CUtensorMap mapW2,
                                                            const __grid_constant__ CUtensorMap mapW3)
{
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *sA = smem, *sB = smem + A_BYTES;
    float *sW1 = (float *)(sB + B_BYTES);       // [H x F]
    float *sb1 = sW1 + H * F;                   // [H] biases of layers 1, 2, 3
    float *sb2 = sb1 + H;
    float *sb3 = sb2 + H;
    float *sw4 = sb3 + H;                       // [H] output weights
    float *sred = sw4 + H;                      // [TILE] half-row dot products
    __shared__ __align__(8) uint64_t bar_full, bar_done;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int row = (warp & 3) * 32 + lane;     // TMEM lane = tile row of this thread
    const int half = warp >> 2;                 // column half [128*half, +128) of this thread
    for (int k = tid; k < H * F; k += MLP_THREADS) sW1[k] = a.P[O_W1 + k];
    for (int k = tid; k < H; k += MLP_THREADS) {
        sb1[k] = a.P[O_B1 + k];
        sb2[k] = a.P[O_B2 + k];
        sb3[k] = a.P[O_B3 + k];
        sw4[k] = a.P[O_W4 + k];
    }
    float xs[F], xc[F];
#pragma unroll
    for (int f = 0; f < F; ++f) { xs[f] = a.P[O_XS + f]; xc[f] = a.P[O_XC + f]; }
    const float b4 = a.P[O_B4], ys = a.P[O_YS];
    if (tid == 0) {
        s_abort = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar_full)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar_done)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(H));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(H >> 3) << 17) | ((uint32_t)(TILE >> 4) << 24);
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    uint32_t ph_full = 0, ph_done = 0;
    const long long ntiles = (a.n + TILE - 1) / TILE;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long gr = tile * TILE + row;
        float x[F];
        long long pq, qp;
        double guess;
        load_row(a, gr, x, pq, qp, guess);
#pragma unroll
        for (int f = 0; f < F; ++f) x[f] = (x[f] - xs[f]) * xc[f];
        // layer 1: hidden units [128*half, +128) of this row, 8 per 16-byte store
        for (int c = half * 16; c < half * 16 + 16; ++c) {
            __align__(16) __nv_bfloat16 h8[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int j = c * 8 + e;
                float z = sb1[j];
#pragma unroll
                for (int f = 0; f < F; ++f) z = fmaf(sW1[j * F + f], x[f], z);
                h8[e] = __float2bfloat16_rn(silu(z));
            }
            *reinterpret_cast<uint4 *>(sA + (c >> 3) * A_KB + sw128_chunk(row, c & 7)) = *reinterpret_cast<uint4 *>(h8);
        }
        float dot = 0.f;
        for (int layer = 0; layer < 2; ++layer) {
            const float *sb = layer == 0 ? sb2 : sb3;
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // generic smem writes -> tensor core
            __syncthreads();
            if (tid == 0) {
                const CUtensorMap *map = layer == 0 ? &mapW2 : &mapW3;
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&bar_full)),
                             "r"(B_BYTES)
                             : "memory");
                for (int kb = 0; kb < 4; ++kb)
                    asm volatile(
                        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
                            smem_u32(sB + kb * B_KB)),
                        "l"(map), "r"(smem_u32(&bar_full)), "r"(kb * 64), "r"(0)
                        : "memory");
                if (!wait_bar(&bar_full, ph_full, a.err, 11)) {
                    s_abort = 1;
                } else {
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    for (int kb = 0; kb < 4; ++kb)
                        for (int kk = 0; kk < 4; ++kk) {
                            const uint64_t ad = sw128_desc(smem_u32(sA + kb * A_KB) + kk * 32);
                            const uint64_t bd = sw128_desc(smem_u32(sB + kb * B_KB) + kk * 32);
                            const uint32_t acc = (kb | kk) ? 1u : 0u;
                            asm volatile(
                                "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                                "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
                        }
                }
                // arrives once the MMAs issued above (if any) have completed
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_u32(&bar_done))
                             : "memory");
            }
            ph_full ^= 1;
            if (!wait_bar(&bar_done, ph_done, a.err, 12)) s_abort = 1;
            ph_done ^= 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            __syncthreads();
            if (s_abort) break;
            // epilogue: this row, columns [128*half, +128)
            for (int c0 = half * 128; c0 < half * 128 + 128; c0 += 16) {
                uint32_t r[16];
                asm volatile(
                    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                    : "r"(tmem + lane_base + (uint32_t)c0));
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                if (layer == 0) {
                    __align__(16) __nv_bfloat16 h8[16];
#pragma unroll
                    for (int e = 0; e < 16; ++e) h8[e] = __float2bfloat16_rn(silu(__uint_as_float(r[e]) + sb[c0 + e]));
                    const int c = c0 >> 3;
                    *reinterpret_cast<uint4 *>(sA + (c >> 3) * A_KB + sw128_chunk(row, c & 7)) = *reinterpret_cast<uint4 *>(h8);
                    *reinterpret_cast<uint4 *>(sA + ((c + 1) >> 3) * A_KB + sw128_chunk(row, (c + 1) & 7)) =
                        *reinterpret_cast<uint4 *>(h8 + 8);
                } else {
#pragma unroll
                    for (int e = 0; e < 16; ++e) dot = fmaf(silu(__uint_as_float(r[e]) + sb[c0 + e]), sw4[c0 + e], dot);
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        }
        if (half == 1) sred[row] = dot;
        __syncthreads();
        if (s_abort) break;
        if (half == 0 && gr < a.n) {
            const float y = (dot + sred[row] + b4) * ys;
            if (a.X) {
                a.Y[gr] = y;
            } else {
                const CCMol &m = a.mols[a.mol];
                const double t = guess + (double)y;
                m.t2[pq] = t;
                m.t2[qp] = t;
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(H));
}

// ------------------------------------------------------------------ tcgen05 training GEMM
// C[M x 256] = A[M x K] B[256 x K]^T (+ bias[n]) from bf16 operands, both
// K-major (row m of A, row n of B, K contiguous), FP32 accumulation in 256
// TMEM columns. CTA (x, y) = 128-row tile x a split of kb_per 64-deep
// K-blocks; with more than one split the CTAs add into C with atomics (C
// cleared first). Thread 0 streams the K-blocks with TMA through two
// stages and issues the MMAs (M = 128, N = 256, K = 16); the four warps
// then drain TMEM (a lane per row). Every wait is bounded; a CTA that gives
// up records a code, waits (bounded) for the loads it issued and still
// frees its TMEM.
constexpr int BG_STAGE = A_KB + B_KB;                 // 16 KB of A + 32 KB of B per K-block
constexpr int BG_SMEM = 1024 + 2 * BG_STAGE;
constexpr int BG_THREADS = 128;

__global__ void __launch_bounds__(BG_THREADS, 1) bgemm(const __grid_constant__ CUtensorMap mapA,
                                                       const __grid_constant__ CUtensorMap mapB, float *C, int ldc,
                                                       const float *bias, int nkb, int kb_per, int *err)
{
    extern __shared__ __align__(1024) uint8_t bg_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)bg_raw + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t full[2], freed[2], done;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.x * TILE;
    const int kb0 = blockIdx.y * kb_per, n = min(nkb, kb0 + kb_per) - kb0;
    if (tid == 0) {
        s_abort = 0;
        for (int q = 0; q < 2; ++q) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full[q])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&freed[q])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&done)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(H));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    if (tid == 0) {
        const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(H >> 3) << 17) | ((uint32_t)(TILE >> 4) << 24);
        auto load = [&](int i) {
            uint8_t *sa = smem + (i & 1) * BG_STAGE, *sb = sa + A_KB;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&full[i & 1])),
                         "r"(BG_STAGE)
                         : "memory");
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
                    smem_u32(sa)),
                "l"(&mapA), "r"(smem_u32(&full[i & 1])), "r"((kb0 + i) * 64), "r"(m0)
                : "memory");
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
                    smem_u32(sb)),
                "l"(&mapB), "r"(smem_u32(&full[i & 1])), "r"((kb0 + i) * 64), "r"(0)
                : "memory");
        };
        int issued = 0, consumed = 0;
        for (; issued < n && issued < 2; ++issued) load(issued);
        bool ok = true;
        for (int i = 0; i < n && ok; ++i) {
            ok = wait_bar(&full[i & 1], (uint32_t)((i >> 1) & 1), err, 21);
            if (!ok) break;
            ++consumed;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = smem_u32(smem + (i & 1) * BG_STAGE), sb = sa + A_KB;
            for (int kk = 0; kk < 4; ++kk) {
                const uint64_t ad = sw128_desc(sa + kk * 32), bd = sw128_desc(sb + kk * 32);
                const uint32_t acc = (i | kk) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&freed[i & 1]))
                         : "memory");
            if (issued < n) {                  // stage i & 1 is free once these MMAs complete
                ok = wait_bar(&freed[i & 1], (uint32_t)((i >> 1) & 1), err, 22);
                if (ok) load(issued++);
            }
        }
        if (!ok) {
            s_abort = 1;
            for (int j = consumed; j < issued; ++j) wait_bar(&full[j & 1], (uint32_t)((j >> 1) & 1), nullptr, 0);
        }
        // arrives once every MMA issued above has completed
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(&done))
                     : "memory");
    }
    const bool fin = wait_bar(&done, 0u, err, 23);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    if (fin && !s_abort) {
        const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
        float *crow = C + (long long)(m0 + tid) * ldc;
        const bool atomic = gridDim.y > 1;
        for (int c0 = 0; c0 < H; c0 += 16) {
            uint32_t r[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                : "r"(tmem + lane_base + (uint32_t)c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            float v[16];
#pragma unroll
            for (int e = 0; e < 16; ++e) v[e] = __uint_as_float(r[e]) + (bias ? bias[c0 + e] : 0.f);
            if (atomic) {
#pragma unroll
                for (int e = 0; e < 16; ++e) atomicAdd(crow + c0 + e, v[e]);
            } else {
#pragma unroll
                for (int e = 0; e < 16; e += 4) *reinterpret_cast<float4 *>(crow + c0 + e) = make_float4(v[e], v[e + 1], v[e + 2], v[e + 3]);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(H));
}

// bf16 copies of an FP32 [rows x cols] matrix (cols a multiple of 32): row-major
// (dst) and transposed (dstT, [cols x rows]), through 32 x 32 shared tiles so
// that both are written coalesced.
__global__ void k_bf16_copies(const float *src, int rows, int cols, __nv_bfloat16 *dst, __nv_bfloat16 *dstT)
{
    __shared__ float t[32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;          // 32 x 8 threads
    const int ct = cols / 32, tiles = ((rows + 31) / 32) * ct;
    for (int u = blockIdx.x; u < tiles; u += gridDim.x) {
        const int r0 = (u / ct) * 32, c0 = (u % ct) * 32;
        for (int y = ty; y < 32; y += 8) {
            const int r = r0 + y;
            const float v = r < rows ? src[(long long)r * cols + c0 + tx] : 0.f;
            t[y][tx] = v;
            if (dst && r < rows) dst[(long long)r * cols + c0 + tx] = __float2bfloat16_rn(v);
        }
        __syncthreads();
        if (dstT)
            for (int y = ty; y < 32; y += 8)
                if (r0 + tx < rows) dstT[(long long)(c0 + y) * rows + r0 + tx] = __float2bfloat16_rn(t[tx][y]);
        __syncthreads();
    }
}

__global__ void k_to_bf16(const float *src, __nv_bfloat16 *dst, int n)
{
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) dst[k] = __float2bfloat16_rn(src[k]);
}

// ------------------------------------------------------------------ SIMT training kernels
// C[M x N] = alpha * sum_k A(m,k) B(k,n) (+ bias[n]) + beta C, with
// A(m,k) = A[m*ar + k*ac], B(k,n) = B[k*br + n*bc] (a stride of 0 broadcasts),
// C row-major with leading dimension ldc; optional bf16 rounding of B.
__global__ void __launch_bounds__(256) sgemm(int M, int N, int K, float alpha, const float *A, long long ar,
                                              long long ac, const float *B, long long br, long long bc, float beta,
                                              float *C, int ldc, const float *bias, int round_b)
{
    __shared__ float As[16][65], Bs[16][65];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += 16) {
        for (int e = threadIdx.x; e < 64 * 16; e += 256) {
            const int kk = e % 16, mm = e / 16;
            const int m = m0 + mm, k = k0 + kk;
            As[kk][mm] = (m < M && k < K) ? A[m * ar + k * ac] : 0.f;
            const int nn = e % 64, kb = e / 64;
            const int n = n0 + nn, k2 = k0 + kb;
            const float vb = (n < N && k2 < K) ? B[k2 * br + n * bc] : 0.f;
            Bs[kb][nn] = round_b ? bf16r(vb) : vb;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            float av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + ty + 16 * i;
        if (m >= M) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int n = n0 + tx + 16 * j;
            if (n >= N) continue;
            float r = alpha * acc[i][j] + (bias ? bias[n] : 0.f);
            if (beta != 0.f) r += beta * C[(long long)m * ldc + n];
            C[(long long)m * ldc + n] = r;
        }
    }
}

// x = (X[idx] - shift) * scale and t = T[idx] for the rows of one batch (idx NULL = identity)
__global__ void k_gather_norm(const float *X, const float *T, const long long *idx, const float *P, float *x,
                              float *t, int n)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n * F; e += gridDim.x * blockDim.x) {
        const int r = e / F, f = e % F;
        const long long src = idx ? idx[r] : r;
        x[e] = (X[src * F + f] - P[O_XS + f]) * P[O_XC + f];
        if (f == 0) t[r] = T[src];
    }
}
// h = silu(z), rounded to bf16 when it feeds a bf16 layer
__global__ void k_silu(const float *z, float *h, long long n, int round)
{
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const float s = silu(z[e]);
        h[e] = round ? bf16r(s) : s;
    }
}
// residual in network units r = y + b4 - T / y_scale; dy = 2 r / M; loss += mean r^2
__global__ void k_loss(const float *y, const float *T, const float *P, float *dy, float *loss, int n)
{
    __shared__ float sh[256];
    float acc = 0.f;
    const float s = P[O_YS], b4 = P[O_B4];
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const float r = y[e] + b4 - T[e] / s;
        dy[e] = 2.f * r / n;
        acc += r * r;
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, sh[0] / n);
}
// dz = dh * silu'(z), with dh[m][j] = dy[m] * w4[j] when w4 is given
__global__ void k_dsilu(const float *dh, const float *dy, const float *w4, const float *z, float *dz, int M)
{
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < (long long)M * H;
         e += (long long)gridDim.x * blockDim.x) {
        const int m = (int)(e / H), j = (int)(e % H);
        const float g = w4 ? dy[m] * w4[j] : dh[e];
        dz[e] = g * dsilu(z[e]);
    }
}
// Adam on the trainable prefix of the blob
__global__ void k_adam(float *P, const float *G, float *m1, float *m2, int n, float lr, float b1, float b2, float eps,
                       float c1, float c2)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const float g = G[e];
        m1[e] = b1 * m1[e] + (1.f - b1) * g;
        m2[e] = b2 * m2[e] + (1.f - b2) * g * g;
        P[e] -= lr * (m1[e] / c1) / (sqrtf(m2[e] / c2) + eps);
    }
}

// ------------------------------------------------------------------ host helpers
static inline unsigned nblocks(long long n, int t = 256)
{
    long long b = (n + t - 1) / t;
    return (unsigned)std::max(1LL, std::min(b, 65535LL));
}

static void gemm(cudaStream_t s, int M, int N, int K, const float *A, long long ar, long long ac, const float *B,
                 long long br, long long bc, float *C, int ldc, const float *bias = nullptr, int round_b = 0)
{
    dim3 g((N + 63) / 64, (M + 63) / 64);
    sgemm<<<g, 256, 0, s>>>(M, N, K, 1.f, A, ar, ac, B, br, bc, 0.f, C, ldc, bias, round_b);
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

// 2D map over a bf16 [rows x cols] matrix: 64 x box_rows boxes, 128-byte swizzle
static int map_bf16(CUtensorMap *map, const void *base, long long rows, int cols, int box_rows)
{
    auto fn = encode_fn();
    if (!fn) { hx_set_error("cuTensorMapEncodeTiled is unavailable"); return HX_ERR_CUDA; }
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
    cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { hx_set_error("cuTensorMapEncodeTiled failed (%d)", (int)r); return HX_ERR_CUDA; }
    return HX_OK;
}

// device workspace for batches of up to M rows (padded to Mp, a multiple of
// the 128-row tile: the padded rows have zero inputs and zero loss gradient)
struct Work {
    int M = 0, Mp = 0;
    float *x = nullptr, *t = nullptr, *z1 = nullptr, *h1 = nullptr, *z2 = nullptr, *h2 = nullptr, *z3 = nullptr,
          *h3 = nullptr, *y = nullptr, *dy = nullptr, *dz = nullptr, *dh = nullptr, *G = nullptr, *loss = nullptr,
          *ones = nullptr;
    // bf16 operands of the tensor-core GEMMs: activations and gradients (and
    // their transposes, [H x Mp]) and the two hidden weight matrices
    __nv_bfloat16 *h1b = nullptr, *h2b = nullptr, *h1T = nullptr, *h2T = nullptr, *dzb = nullptr, *dzT = nullptr,
                  *W2b = nullptr, *W3b = nullptr, *W2T = nullptr, *W3T = nullptr;
    CUtensorMap mH1b, mH2b, mW2b, mW3b, mDzT, mH1T, mH2T, mDzb, mW2T, mW3T;
    int *err = nullptr;
    int alloc(int m)
    {
        M = m;
        Mp = (m + TILE - 1) / TILE * TILE;
        const size_t act = (size_t)Mp * H * 4, actb = (size_t)Mp * H * 2, wb = (size_t)H * H * 2;
        float **big[] = {&z1, &h1, &z2, &h2, &z3, &h3, &dz, &dh};
        for (float **b : big)
            if (cudaMalloc(b, act) != cudaSuccess) return HX_ERR_NOMEM;
        __nv_bfloat16 **bb[] = {&h1b, &h2b, &h1T, &h2T, &dzb, &dzT};
        for (__nv_bfloat16 **b : bb)
            if (cudaMalloc(b, actb) != cudaSuccess) return HX_ERR_NOMEM;
        __nv_bfloat16 **wbs[] = {&W2b, &W3b, &W2T, &W3T};
        for (__nv_bfloat16 **b : wbs)
            if (cudaMalloc(b, wb) != cudaSuccess) return HX_ERR_NOMEM;
        if (cudaMalloc(&x, (size_t)Mp * F * 4) != cudaSuccess || cudaMalloc(&t, (size_t)Mp * 4) != cudaSuccess ||
            cudaMalloc(&y, (size_t)Mp * 4) != cudaSuccess || cudaMalloc(&dy, (size_t)Mp * 4) != cudaSuccess ||
            cudaMalloc(&G, (size_t)NPARAM * 4) != cudaSuccess || cudaMalloc(&loss, 4) != cudaSuccess ||
            cudaMalloc(&ones, (size_t)Mp * 4) != cudaSuccess || cudaMalloc(&err, 4) != cudaSuccess)
            return HX_ERR_NOMEM;
        // padded rows: zero inputs and targets, and a zero loss gradient (k_loss writes the first M only)
        if (cudaMemset(x, 0, (size_t)Mp * F * 4) != cudaSuccess || cudaMemset(t, 0, (size_t)Mp * 4) != cudaSuccess ||
            cudaMemset(dy, 0, (size_t)Mp * 4) != cudaSuccess || cudaMemset(err, 0, 4) != cudaSuccess)
            return HX_ERR_CUDA;
        int rc = HX_OK;
        if (rc == HX_OK) rc = map_bf16(&mH1b, h1b, Mp, H, TILE);
        if (rc == HX_OK) rc = map_bf16(&mH2b, h2b, Mp, H, TILE);
        if (rc == HX_OK) rc = map_bf16(&mDzb, dzb, Mp, H, TILE);
        if (rc == HX_OK) rc = map_bf16(&mDzT, dzT, H, Mp, TILE);
        if (rc == HX_OK) rc = map_bf16(&mH1T, h1T, H, Mp, H);
        if (rc == HX_OK) rc = map_bf16(&mH2T, h2T, H, Mp, H);
        if (rc == HX_OK) rc = map_bf16(&mW2b, W2b, H, H, H);
        if (rc == HX_OK) rc = map_bf16(&mW3b, W3b, H, H, H);
        if (rc == HX_OK) rc = map_bf16(&mW2T, W2T, H, H, H);
        if (rc == HX_OK) rc = map_bf16(&mW3T, W3T, H, H, H);
        if (rc != HX_OK) return rc;
        if (cudaFuncSetAttribute(bgemm, cudaFuncAttributeMaxDynamicSharedMemorySize, BG_SMEM) != cudaSuccess) {
            hx_set_error("cannot reserve shared memory for the training GEMM");
            return HX_ERR_CUDA;
        }
        std::vector<float> one(Mp, 1.f);
        return cudaMemcpy(ones, one.data(), (size_t)Mp * 4, cudaMemcpyHostToDevice) == cudaSuccess ? HX_OK : HX_ERR_CUDA;
    }
    int error_word() const
    {
        int v = 0;
        if (err) cudaMemcpy(&v, err, 4, cudaMemcpyDeviceToHost);
        return v;
    }
    ~Work()
    {
        float *all[] = {x, t, z1, h1, z2, h2, z3, h3, y, dy, dz, dh, G, loss, ones};
        for (float *b : all) cudaFree(b);
        __nv_bfloat16 *allb[] = {h1b, h2b, h1T, h2T, dzb, dzT, W2b, W3b, W2T, W3T};
        for (__nv_bfloat16 *b : allb) cudaFree(b);
        cudaFree(err);
    }
};

// bf16 copies (row-major and transposed) of an FP32 [rows x H] matrix
static void copies(cudaStream_t s, const float *src, int rows, __nv_bfloat16 *dst, __nv_bfloat16 *dstT)
{
    k_bf16_copies<<<nblocks((long long)((rows + 31) / 32) * (H / 32), 1), 256, 0, s>>>(src, rows, H, dst, dstT);
}
// tensor-core GEMM C[rows x H] = A B^T (+ bias) over nkb 64-deep K-blocks; splits > 1
// add into C (cleared first) from that many K ranges
static void bf16_gemm(cudaStream_t s, const CUtensorMap &a, const CUtensorMap &b, int rows, int nkb, int splits,
                    float *C, const float *bias, int *err)
{
    const int kb_per = (nkb + splits - 1) / splits;
    const dim3 grid(rows / TILE, (nkb + kb_per - 1) / kb_per);
    if (grid.y > 1) cudaMemsetAsync(C, 0, (size_t)rows * H * 4, s);
    bgemm<<<grid, BG_THREADS, BG_SMEM, s>>>(a, b, C, H, bias, nkb, kb_per, err);
}

// forward + backward of one batch already normalised in w.x / w.t (M rows);
// gradients into w.G (overwritten), mean squared error added to w.loss. The
// six 256-wide products (layers 2 and 3 forward, their weight gradients and
// the gradients of their inputs) run on the tensor cores in BF16 with FP32
// accumulation (bgemm); the 8-wide first layer, the 1-wide output and the
// bias sums stay on the CUDA cores. The loss gradient dz entering a bf16
// product is rounded to bf16 (oracle/mlp.py applies the same roundings).
static void fwd_bwd(cudaStream_t s, Work &w, const float *P, int M)
{
    const int Mp = w.Mp, nk = H / 64, nkm = Mp / 64;
    const long long MH = (long long)Mp * H;
    k_bf16_copies<<<64, 256, 0, s>>>(P + O_W2, H, H, w.W2b, w.W2T);
    k_bf16_copies<<<64, 256, 0, s>>>(P + O_W3, H, H, w.W3b, w.W3T);
    gemm(s, Mp, H, F, w.x, F, 1, P + O_W1, 1, F, w.z1, H, P + O_B1);
    k_silu<<<nblocks(MH), 256, 0, s>>>(w.z1, w.h1, MH, 1);
    copies(s, w.h1, Mp, w.h1b, w.h1T);
    bf16_gemm(s, w.mH1b, w.mW2b, Mp, nk, 1, w.z2, P + O_B2, w.err);
    k_silu<<<nblocks(MH), 256, 0, s>>>(w.z2, w.h2, MH, 1);
    copies(s, w.h2, Mp, w.h2b, w.h2T);
    bf16_gemm(s, w.mH2b, w.mW3b, Mp, nk, 1, w.z3, P + O_B3, w.err);
    k_silu<<<nblocks(MH), 256, 0, s>>>(w.z3, w.h3, MH, 0);
    gemm(s, Mp, 1, H, w.h3, H, 1, P + O_W4, 1, 0, w.y, 1);
    k_loss<<<nblocks(M), 256, 0, s>>>(w.y, w.t, P, w.dy, w.loss, M);
    // output layer
    gemm(s, 1, H, Mp, w.dy, 0, 1, w.h3, H, 1, w.G + O_W4, H);             // dw4 = h3^T dy
    gemm(s, 1, 1, Mp, w.dy, 0, 1, w.ones, 1, 0, w.G + O_B4, 1);            // db4 = sum dy
    k_dsilu<<<nblocks(MH), 256, 0, s>>>(nullptr, w.dy, P + O_W4, w.z3, w.dz, Mp);
    copies(s, w.dz, Mp, w.dzb, w.dzT);
    // layer 3
    bf16_gemm(s, w.mDzT, w.mH2T, H, nkm, std::max(1, nkm / 4), w.G + O_W3, nullptr, w.err);   // dW3 = bf16(dz3)^T h2
    gemm(s, 1, H, Mp, w.ones, 0, 1, w.dz, H, 1, w.G + O_B3, H);            // db3
    bf16_gemm(s, w.mDzb, w.mW3T, Mp, nk, 1, w.dh, nullptr, w.err);          // dh2 = bf16(dz3) bf16(W3)
    k_dsilu<<<nblocks(MH), 256, 0, s>>>(w.dh, nullptr, nullptr, w.z2, w.dz, Mp);
    copies(s, w.dz, Mp, w.dzb, w.dzT);
    // layer 2
    bf16_gemm(s, w.mDzT, w.mH1T, H, nkm, std::max(1, nkm / 4), w.G + O_W2, nullptr, w.err);
    gemm(s, 1, H, Mp, w.ones, 0, 1, w.dz, H, 1, w.G + O_B2, H);
    bf16_gemm(s, w.mDzb, w.mW2T, Mp, nk, 1, w.dh, nullptr, w.err);
    k_dsilu<<<nblocks(MH), 256, 0, s>>>(w.dh, nullptr, nullptr, w.z1, w.dz, Mp);
    // layer 1
    gemm(s, H, F, Mp, w.dz, 1, H, w.x, F, 1, w.G + O_W1, F);
    gemm(s, 1, H, Mp, w.ones, 0, 1, w.dz, H, 1, w.G + O_B1, H);
    hx_count_launches(30);
}


int Model::load(const float *host_blob)
{
    release();
    if (cudaMalloc(&P, (size_t)NPARAM * 4) != cudaSuccess || cudaMalloc(&W2, (size_t)H * H * 2) != cudaSuccess ||
        cudaMalloc(&W3, (size_t)H * H * 2) != cudaSuccess || cudaMalloc(&err, 4) != cudaSuccess) {
        hx_set_error("learned guess: device allocation failed");
        return HX_ERR_NOMEM;
    }
    if (cudaMemcpy(P, host_blob, (size_t)NPARAM * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(err, 0, 4) != cudaSuccess) {
        hx_set_error("learned guess: upload failed");
        return HX_ERR_CUDA;
    }
    k_to_bf16<<<64, 256>>>(P + O_W2, W2, H * H);
    k_to_bf16<<<64, 256>>>(P + O_W3, W3, H * H);
    auto fn = encode_fn();
    if (!fn) { hx_set_error("cuTensorMapEncodeTiled is unavailable"); return HX_ERR_CUDA; }
    for (int k = 0; k < 2; ++k) {
        cuuint64_t dims[2] = {(cuuint64_t)H, (cuuint64_t)H};
        cuuint64_t strides[1] = {(cuuint64_t)H * 2};
        cuuint32_t box[2] = {64, (cuuint32_t)H};
        cuuint32_t es[2] = {1, 1};
        CUresult r = fn(k == 0 ? &mapW2 : &mapW3, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, k == 0 ? (void *)W2 : (void *)W3,
                        dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) { hx_set_error("cuTensorMapEncodeTiled failed (%d)", (int)r); return HX_ERR_CUDA; }
    }
    if (cudaFuncSetAttribute(mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, MLP_SMEM) != cudaSuccess) {
        hx_set_error("cannot reserve shared memory for mlp_infer");
        return HX_ERR_CUDA;
    }
    hx_count_launches(2);
    return cudaDeviceSynchronize() == cudaSuccess ? HX_OK : HX_ERR_CUDA;
}

void Model::release()
{
    cudaFree(P);
    cudaFree(W2);
    cudaFree(W3);
    cudaFree(err);
    P = nullptr;
    W2 = W3 = nullptr;
    err = nullptr;
}

int Model::error_word() const
{
    int v = 0;
    if (err) cudaMemcpy(&v, err, 4, cudaMemcpyDeviceToHost);
    return v;
}

static cudaError_t launch_infer(const InferArgs &a, const Model &m, cudaStream_t s)
{
    if (a.n <= 0) return cudaSuccess;
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const long long tiles = (a.n + TILE - 1) / TILE;
    const unsigned grid = (unsigned)std::min<long long>(tiles, nsm > 0 ? nsm : 1);
    mlp_infer<<<grid, MLP_THREADS, MLP_SMEM, s>>>(a, m.mapW2, m.mapW3);
    hx_count_launches(1);
    return cudaGetLastError();
}

cudaError_t Model::apply(const CCMol *d_mols, int mol, long long npairs, cudaStream_t s) const
{
    InferArgs a{nullptr, nullptr, d_mols, mol, 0, npairs, P, err};
    return launch_infer(a, *this, s);
}

}  // namespace mlp

// ------------------------------------------------------------------ C ABI
using namespace mlp;

extern "C" {

int hx_mlp_nparam(void) { return NPARAM; }

int hx_mlp_predict(const float *params, const float *X, int64_t n, float *Y)
{
    if (!params || n < 0 || (n > 0 && (!X || !Y))) { hx_set_error("hx_mlp_predict: bad arguments"); return HX_ERR_ARG; }
    if (n == 0) return HX_OK;
    Model m;
    int rc = m.load(params);
    float *dX = nullptr, *dY = nullptr;
    if (rc == HX_OK && (cudaMalloc(&dX, (size_t)n * F * 4) != cudaSuccess || cudaMalloc(&dY, (size_t)n * 4) != cudaSuccess)) {
        hx_set_error("hx_mlp_predict: allocation failed");
        rc = HX_ERR_NOMEM;
    }
    if (rc == HX_OK) {
        cudaError_t e = cudaMemcpy(dX, X, (size_t)n * F * 4, cudaMemcpyHostToDevice);
        InferArgs a{dX, dY, nullptr, 0, 0, n, m.P, m.err};
        if (e == cudaSuccess) e = launch_infer(a, m, 0);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e != cudaSuccess) { hx_set_error("hx_mlp_predict: %s", cudaGetErrorString(e)); rc = HX_ERR_CUDA; }
        else if (int w = m.error_word()) { hx_set_error("hx_mlp_predict: a tensor-core wait timed out (%d)", w); rc = HX_ERR_KERNEL; }
        else if (cudaMemcpy(Y, dY, (size_t)n * 4, cudaMemcpyDeviceToHost) != cudaSuccess) rc = HX_ERR_CUDA;
    }
    cudaFree(dX);
    cudaFree(dY);
    m.release();
    return rc;
}

int hx_mlp_grad(const float *params, const float *X, const float *T, int32_t n, float *loss, float *grad)
{
    if (!params || !X || !T || n <= 0) { hx_set_error("hx_mlp_grad: bad arguments"); return HX_ERR_ARG; }
    Work w;
    float *dP = nullptr, *dX = nullptr, *dT = nullptr;
    int rc = w.alloc(n);
    if (rc == HX_OK && (cudaMalloc(&dP, (size_t)NPARAM * 4) != cudaSuccess || cudaMalloc(&dX, (size_t)n * F * 4) != cudaSuccess ||
                        cudaMalloc(&dT, (size_t)n * 4) != cudaSuccess))
        rc = HX_ERR_NOMEM;
    if (rc == HX_ERR_NOMEM) hx_set_error("hx_mlp_grad: allocation failed");
    if (rc == HX_OK) {
        cudaMemcpy(dP, params, (size_t)NPARAM * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(dX, X, (size_t)n * F * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(dT, T, (size_t)n * 4, cudaMemcpyHostToDevice);
        cudaMemset(w.loss, 0, 4);
        k_gather_norm<<<nblocks((long long)n * F), 256>>>(dX, dT, nullptr, dP, w.x, w.t, n);
        fwd_bwd(0, w, dP, n);
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) { hx_set_error("hx_mlp_grad: %s", cudaGetErrorString(e)); rc = HX_ERR_CUDA; }
        else if (int we = w.error_word()) { hx_set_error("hx_mlp_grad: a tensor-core wait timed out (%d)", we); rc = HX_ERR_KERNEL; }
        else {
            if (loss) cudaMemcpy(loss, w.loss, 4, cudaMemcpyDeviceToHost);
            if (grad) {
                cudaMemcpy(grad, w.G, (size_t)O_XS * 4, cudaMemcpyDeviceToHost);
                for (int k = O_XS; k < NPARAM; ++k) grad[k] = 0.f;     // normalisation constants are not trained
            }
        }
    }
    cudaFree(dP);
    cudaFree(dX);
    cudaFree(dT);
    return rc;
}

int hx_mlp_train(float *params, const float *X, const float *T, int64_t n, int32_t epochs, int32_t batch, float lr,
                 uint64_t seed, float *epoch_loss)
{
    if (!params || !X || !T || batch <= 0 || n < batch || epochs <= 0 || !(lr > 0.f)) {
        hx_set_error("hx_mlp_train: bad arguments");
        return HX_ERR_ARG;
    }
    Work w;
    float *dP = nullptr, *dX = nullptr, *dT = nullptr, *m1 = nullptr, *m2 = nullptr;
    long long *dperm = nullptr;
    const int ntrain = O_XS;          // W1 .. b4; the normalisation constants stay fixed
    int rc = w.alloc(batch);
    if (rc == HX_OK &&
        (cudaMalloc(&dP, (size_t)NPARAM * 4) != cudaSuccess || cudaMalloc(&dX, (size_t)n * F * 4) != cudaSuccess ||
         cudaMalloc(&dT, (size_t)n * 4) != cudaSuccess || cudaMalloc(&m1, (size_t)ntrain * 4) != cudaSuccess ||
         cudaMalloc(&m2, (size_t)ntrain * 4) != cudaSuccess || cudaMalloc(&dperm, (size_t)n * 8) != cudaSuccess))
        rc = HX_ERR_NOMEM;
    if (rc == HX_ERR_NOMEM) hx_set_error("hx_mlp_train: allocation failed");
    if (rc == HX_OK) {
        cudaMemcpy(dP, params, (size_t)NPARAM * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(dX, X, (size_t)n * F * 4, cudaMemcpyHostToDevice);
        cudaMemcpy(dT, T, (size_t)n * 4, cudaMemcpyHostToDevice);
        cudaMemset(m1, 0, (size_t)ntrain * 4);
        cudaMemset(m2, 0, (size_t)ntrain * 4);
        std::mt19937_64 rng(seed);
        std::vector<long long> perm(n);
        std::iota(perm.begin(), perm.end(), 0LL);
        const long long nb = n / batch;
        const long long total = nb * epochs;
        long long step = 0;
        const float b1 = 0.9f, b2 = 0.999f;
        for (int ep = 0; ep < epochs && rc == HX_OK; ++ep) {
            std::shuffle(perm.begin(), perm.end(), rng);
            cudaMemcpy(dperm, perm.data(), (size_t)n * 8, cudaMemcpyHostToDevice);
            cudaMemset(w.loss, 0, 4);
            for (long long b = 0; b < nb; ++b) {
                k_gather_norm<<<nblocks((long long)batch * F), 256>>>(dX, dT, dperm + b * batch, dP, w.x, w.t, batch);
                fwd_bwd(0, w, dP, batch);
                ++step;
                const float lr_t = 0.5f * lr * (1.f + cosf(3.14159265f * (float)(step - 1) / (float)total));
                k_adam<<<nblocks(ntrain), 256>>>(dP, w.G, m1, m2, ntrain, lr_t, b1, b2, 1e-8f,
                                                 1.f - powf(b1, (float)step), 1.f - powf(b2, (float)step));
                hx_count_launches(2);
            }
            float l = 0.f;
            cudaError_t e = cudaMemcpy(&l, w.loss, 4, cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) { hx_set_error("hx_mlp_train: %s", cudaGetErrorString(e)); rc = HX_ERR_CUDA; }
            else if (int we = w.error_word()) { hx_set_error("hx_mlp_train: a tensor-core wait timed out (%d)", we); rc = HX_ERR_KERNEL; }
            if (epoch_loss) epoch_loss[ep] = l / (float)(nb > 0 ? nb : 1);
        }
        if (rc == HX_OK && cudaMemcpy(params, dP, (size_t)ntrain * 4, cudaMemcpyDeviceToHost) != cudaSuccess) rc = HX_ERR_CUDA;
    }
    cudaFree(dP);
    cudaFree(dX);
    cudaFree(dT);
    cudaFree(m1);
    cudaFree(m2);
    cudaFree(dperm);
    return rc;
}

}  // extern "C"

// training rows of a solved molecule (engine side, declared in hx_engine.cu)
cudaError_t hx_mlp_sample(const CCMol *d_mols, int mol, const long long *d_rows, int n, float *dX, float *dT,
                          cudaStream_t s)
{
    k_sample<<<nblocks(n), 256, 0, s>>>(d_mols, mol, d_rows, n, dX, dT);
    hx_count_launches(1);
    return cudaGetLastError();
}
