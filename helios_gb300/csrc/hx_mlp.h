// Learned T2 initial guess: device copy of the network and its application
// to the molecules of a handle.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include "hx_plan.h"

namespace mlp {

constexpr int H = 256, F = 8;
// parameter blob (float32): W1 [H x F], b1 [H], W2 [H x H], b2 [H], W3 [H x H],
// b3 [H], w4 [H], b4, x_shift [F], x_scale [F], y_scale
constexpr int O_W1 = 0, O_B1 = O_W1 + H * F, O_W2 = O_B1 + H, O_B2 = O_W2 + H * H, O_W3 = O_B2 + H,
              O_B3 = O_W3 + H * H, O_W4 = O_B3 + H, O_B4 = O_W4 + H, O_XS = O_B4 + 1, O_XC = O_XS + F,
              O_YS = O_XC + F, NPARAM = O_YS + 1;

struct Model {
    float *P = nullptr;                 // the blob
    __nv_bfloat16 *W2 = nullptr, *W3 = nullptr;
    int *err = nullptr;                 // device error word of the inference kernel
    CUtensorMap mapW2, mapW3;           // TMA maps of the bf16 weights (256 x 256, 128-byte swizzle)
    int load(const float *host_blob);   // HX_OK or an error code (message set)
    void release();
    // t2 <- guess + prediction for every canonical pair (ia) <= (jb) of
    // molecule mol (both t2 entries of the pair), after the reference guess.
    cudaError_t apply(const CCMol *d_mols, int mol, long long npairs, cudaStream_t s) const;
    int error_word() const;
};

}  // namespace mlp
