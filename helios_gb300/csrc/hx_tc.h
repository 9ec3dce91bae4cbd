// Tensor-core (tcgen05, BF16x3 split precision) backend of the grouped tensor-GEMM.
#pragma once
#include <vector>
#include "hx_plan.h"

namespace tc {
struct Engine;
// Build the backend for the GEMM groups of a plan (scratch sized to the largest
// operand). Tile variants: force >= 0 takes candidate `force` of every mode;
// otherwise tuning 0 looks each (mode, group, size class) up in the tile
// table and takes the default on a miss, 1 times every candidate on a miss
// (and records the winner), 2 takes the defaults. only_mode >= 0 builds that
// precision mode alone (the others have no groups to run).
int create(Engine **out, const std::vector<Group> &plan, cudaStream_t s, int tuning = 2, int force = -1,
           int only_mode = -1);
// Run one plan group on the tensor cores: slice the operands, tcgen05 GEMM,
// FP64 epilogue. mode 0 = LOW (3 slices, about 2^-24 of the row maxima),
// 1 = MID (4 slices, about 2^-32), 2 = HIGH (5 slices, about 2^-35), 3 =
// EXACT (7 slices: an FP64 GEMM emulated, as accurate as the FP64 product).
cudaError_t run_group(Engine *e, const TgemmDesc *descs, int n, const int *d_active, cudaStream_t s, int mode);
void destroy(Engine *e);
// Slice the constant operands of every group and mode now (they are
// otherwise sliced on a group's first run after an initialisation), so that
// a captured iteration holds no one-off work.
cudaError_t prepare_fixed(Engine *e, cudaStream_t s);
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
// Chosen variant of every (mode, plan group), var[mode * groups + group];
// returns 4 * groups.
int choices(Engine *e, int *var, int cap);
// Milliseconds spent timing candidates when the backend was built.
double tune_ms(Engine *e);
// The process-wide tile table: entries of 5 ints (mode, group, size class
// N, size class work, variant). table_get copies up to cap entries and
// returns the count; table_load merges n entries.
int table_get(int *entries, int cap);
int table_load(const int *entries, int n);
// Output tile widths of a mode's candidates (returns their number).
int variants(int mode, int *bn, int cap);
}  // namespace tc
