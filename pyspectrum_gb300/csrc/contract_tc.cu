// tcgen05 split-BF16 triangle contraction (placeholder until the kernel lands).
#include "contract.cuh"

namespace pyspec {
size_t contract_tc_ws(int64_t, int, int) { return 0; }
int contract_tc_impl(const float*, int64_t, int, const int32_t*, int, double*, void*, size_t, cudaStream_t) {
    set_error("the BF16x3 tensor-core contraction is not built in this version");
    return PYSPEC_E_UNSUPPORTED;
}
}  // namespace pyspec
