// Tensor-core (tcgen05, BF16x3 split precision) backend of the grouped tensor-GEMM.
#pragma once
#include <vector>
#include "hx_plan.h"

struct Group;
namespace tc {
struct Engine;
// Build the backend for the GEMM groups of a plan (scratch sized to the largest operand).
int create(Engine **out, const std::vector<Group> &plan, cudaStream_t s);
// Run one group: gather + split the operands to BF16 hi/lo, tcgen05 GEMM, FP64 epilogue.
cudaError_t run_group(Engine *e, const TgemmDesc *descs, int n, const int *active_host, cudaStream_t s);
void destroy(Engine *e);
}  // namespace tc
