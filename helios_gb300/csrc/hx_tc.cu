// Tensor-core backend placeholder: the BF16x3 tcgen05 GEMM lands in this file.
#include "hx_common.cuh"
#include "hx_tc.h"

namespace tc {
struct Engine { int unused; };
int create(Engine **out, const std::vector<Group> &, cudaStream_t)
{
    *out = nullptr;
    hx_set_error("mixed precision is not available in this build");
    return HX_ERR_UNSUPPORTED;
}
cudaError_t run_group(Engine *, const TgemmDesc *, int, const int *, cudaStream_t) { return cudaErrorNotSupported; }
void destroy(Engine *) {}
}  // namespace tc
