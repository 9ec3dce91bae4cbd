// Shared declarations of the GB300 PPP-CCSD engine (device kernels + host plan).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

#define HX_MAX_MOL_N 256      // largest PPP system (sites) one handle accepts

// Status / error codes (HX_OK, HX_CONVERGED, HX_ERR_*) are those of the public header.
#include "../../include/helios_cc.h"

// One (optionally batched) tensor contraction
//   C[m,n] = alpha * sum_k A[m,k] * B[n,k] + beta * C[m,n]
// Each of m, n, k is split into (outer, inner) = (x / xi, x % xi) so that a
// 4-index tensor reached through any two of its indices has a plain offset:
//   off_A(m,k) = (m/Mi)*a[0] + (m%Mi)*a[1] + (k/Ki)*a[2] + (k%Ki)*a[3] + batch*a[4]
// (B and C alike with their own strides). A plain matrix sets Mi=M, Ni=N, Ki=K
// and puts its strides in slots 1 and 3.
struct TgemmDesc {
    const double *A, *B;
    double *C;
    int batch, M, N, K;
    int Mi, Ni, Ki;
    long long a[5], b[5], c[5];
    double alpha, beta;
    int mol;            // molecule index (skipped when that molecule is inactive)
    int ksplit;         // K is cut into ksplit slices accumulated atomically (needs beta == 1)
    int a_const, b_const;   // operand unchanged between hx_ccsd_init calls (prepared once)
    int tiles_m, tiles_n;
    long long tile_start;   // prefix sum of batch*tiles_m*tiles_n over the group
};

#define HX_CUDA(call)                                                                  \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            hx_set_error("%s:%d CUDA error %s: %s", __FILE__, __LINE__, #call,          \
                         cudaGetErrorString(e_));                                      \
            return HX_ERR_CUDA;                                                        \
        }                                                                              \
    } while (0)

void hx_set_error(const char *fmt, ...);
// Count kernel launches of the engine (read back through hx_ccsd_timing).
void hx_count_launches(int n);
