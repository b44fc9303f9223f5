// isf_tc.cu -- F(q,tau) slice correlation on the tensor cores (tcgen05).
#include "pgb_device.cuh"

namespace pgb {

bool isf_tc_supported(int M) { return false; }
size_t isf_tc_scratch_bytes(int nq, int M) { return 0; }
cudaError_t launch_isf_tc(const float2*, int, int, double, double*, void*, cudaStream_t) {
    return cudaErrorNotSupported;
}

}  // namespace pgb
