// FP64 grouped tensor-GEMM on the CUDA cores (the plain-FP64 contraction backend).
//
// One launch runs a whole group of TgemmDesc problems (e.g. the same
// contraction for every molecule of a batch): CTAs are laid out over the
// concatenated tile lists and each finds its problem by binary search on
// tile_start. Tiles of molecules whose `active` flag is 0 exit at once.
//
// Tile 64x64x16, 256 threads, 4x4 outputs per thread. Operand tiles are
// gathered through the descriptor's split strides, so any index permutation
// of a 4-index tensor is read in place; the loader walks the operand's
// contiguous dimension first so the warp's loads coalesce.
#include <algorithm>
#include "hx_common.cuh"

namespace {
constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

__device__ __forceinline__ long long split_off(int x, int xi, long long s0, long long s1)
{
    return (long long)(x / xi) * s0 + (long long)(x % xi) * s1;
}

__global__ void __launch_bounds__(NT) tgemm_f64_kernel(const TgemmDesc *__restrict__ descs, int ndesc,
                                                        const int *__restrict__ active)
{
    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BN + 1];
    __shared__ int s_d;
    const long long tile = blockIdx.x;
    if (threadIdx.x == 0) {
        int lo = 0, hi = ndesc - 1;
        while (lo < hi) {                      // last desc with tile_start <= tile
            int mid = (lo + hi + 1) >> 1;
            if (descs[mid].tile_start <= tile) lo = mid; else hi = mid - 1;
        }
        s_d = lo;
    }
    __syncthreads();
    const TgemmDesc &d = descs[s_d];
    if (active && !active[d.mol]) return;
    long long local = tile - d.tile_start;
    const int ks = (int)(local % d.ksplit);
    local /= d.ksplit;
    const int per_batch = d.tiles_m * d.tiles_n;
    const int bt = (int)(local / per_batch);
    local -= (long long)bt * per_batch;
    const int tm = (int)(local / d.tiles_n), tn = (int)(local % d.tiles_n);
    // K slice of this CTA (multiples of BK)
    const int kslice = ((d.K + d.ksplit - 1) / d.ksplit + BK - 1) / BK * BK;
    const int kbeg = ks * kslice, kend = min(d.K, kbeg + kslice);
    const int m0 = tm * BM, n0 = tn * BN;
    const double *A = d.A + (long long)bt * d.a[4];
    const double *B = d.B + (long long)bt * d.b[4];
    double *C = d.C + (long long)bt * d.c[4];
    // K is contiguous for an operand when its inner k stride is 1 and it is the fast axis.
    const bool a_kfast = (d.a[3] == 1) || (d.a[1] != 1);
    const bool b_kfast = (d.b[3] == 1) || (d.b[1] != 1);

    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

    for (int k0 = kbeg; k0 < kend; k0 += BK) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            int e = threadIdx.x + NT * r;
            int mm, kk;
            if (a_kfast) { kk = e % BK; mm = e / BK; } else { mm = e % BM; kk = e / BM; }
            int m = m0 + mm, k = k0 + kk;
            double val = 0.0;
            if (m < d.M && k < kend)
                val = A[split_off(m, d.Mi, d.a[0], d.a[1]) + split_off(k, d.Ki, d.a[2], d.a[3])];
            As[kk][mm] = val;
            int nn;
            if (b_kfast) { kk = e % BK; nn = e / BK; } else { nn = e % BN; kk = e / BN; }
            int n = n0 + nn;
            k = k0 + kk;
            val = 0.0;
            if (n < d.N && k < kend)
                val = B[split_off(n, d.Ni, d.b[0], d.b[1]) + split_off(k, d.Ki, d.b[2], d.b[3])];
            Bs[kk][nn] = val;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            double av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int m = m0 + ty + 16 * i;
        if (m >= d.M) continue;
        long long offm = split_off(m, d.Mi, d.c[0], d.c[1]);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int n = n0 + tx + 16 * j;
            if (n >= d.N) continue;
            double *p = C + offm + split_off(n, d.Ni, d.c[2], d.c[3]);
            double r = d.alpha * acc[i][j];
            if (d.ksplit > 1) { atomicAdd(p, r); continue; }
            if (d.beta != 0.0) r += d.beta * *p;
            *p = r;
        }
    }
}
}  // namespace

// Fill tiles/tile_start of the group on the host; returns the total tile count.
long long hx_tgemm_f64_prepare(TgemmDesc *descs, int n)
{
    long long start = 0;
    for (int i = 0; i < n; ++i) {
        TgemmDesc &d = descs[i];
        d.tiles_m = (d.M + BM - 1) / BM;
        d.tiles_n = (d.N + BN - 1) / BN;
        // split K when the output has few tiles but K is long (accumulating problems only)
        d.ksplit = 1;
        const long long out_tiles = (long long)d.batch * d.tiles_m * d.tiles_n;
        if (d.beta == 1.0 && d.K >= 4 * BK * 8 && out_tiles < 304) {
            long long want = (304 + out_tiles - 1) / out_tiles;
            long long maxk = d.K / (BK * 8);
            d.ksplit = (int)std::max(1LL, std::min(want, maxk));
        }
        d.tile_start = start;
        if (d.M > 0 && d.N > 0 && d.batch > 0) start += out_tiles * d.ksplit;
    }
    return start;
}

cudaError_t hx_tgemm_f64_launch(const TgemmDesc *d_descs, int n, long long total_tiles,
                                const int *d_active, cudaStream_t s)
{
    if (total_tiles <= 0) return cudaSuccess;
    tgemm_f64_kernel<<<(unsigned)total_tiles, NT, 0, s>>>(d_descs, n, d_active);
    hx_count_launches(1);
    return cudaGetLastError();
}
