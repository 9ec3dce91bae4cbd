// Tensor-core (tcgen05, BF16x3 split precision) backend of the grouped tensor-GEMM.
#pragma once
#include <vector>
#include "hx_plan.h"

namespace tc {
struct Engine;
// Build the backend for the GEMM groups of a plan (scratch sized to the largest operand).
int create(Engine **out, const std::vector<Group> &plan, cudaStream_t s);
// Run one plan group on the tensor cores: slice the operands, tcgen05 GEMM,
// FP64 epilogue. mode 0 = LOW (3 slices, about 2^-24 of the row maxima),
// 1 = MID (4 slices, about 2^-32), 2 = HIGH (5 slices, about 2^-35), 3 =
// EXACT (7 slices: an FP64 GEMM emulated, as accurate as the FP64 product).
cudaError_t run_group(Engine *e, const TgemmDesc *descs, int n, const int *d_active, cudaStream_t s, int mode);
void destroy(Engine *e);
// Device error word of the tensor-core kernels (0 = no wait timed out).
int error_word(Engine *e);
// Live timing of the tcgen05 GEMM launches (CUDA events on the launching
// stream): enable/disable, then collect after the stream has synchronised.
void set_profile(Engine *e, bool on);
// The constant operands changed (new orbitals): slice them again on next use.
void invalidate(Engine *e);
// Adds the finished launches to totals: out[0] launches, [1] ms, [2]
// algorithmic flops (2*M*N*K per problem), [3] tensor-core flops issued.
void collect(Engine *e, double out[4]);
}  // namespace tc
