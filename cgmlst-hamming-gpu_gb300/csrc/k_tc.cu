// Tensor-core contraction (tcgen05) — not compiled in yet.
#include "tch_internal.cuh"

namespace tch {

bool tc_kernel_compiled(int) { return false; }

cudaError_t launch_tc_stripe(int, const ByteOperands&, const uint8_t*, const RareCSR&, const StripeArgs&, int,
                             cudaStream_t) {
    return cudaErrorNotSupported;
}

}  // namespace tch
