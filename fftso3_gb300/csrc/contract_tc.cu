// Tensor-core beta-sum contraction (placeholder until the tcgen05 kernels land).
#include "../../include/fftso3_gb300.h"
#include "tc.cuh"

namespace fftso3 {

struct TCState {
    int dummy;
};

int tc_create(TCState** out, int, int, int, const double*, const std::vector<long long>&, long long, const double*,
              const double*, const FFTFactors&, bool, std::string& err)
{
    *out = nullptr;
    err = "tensor-core precision not built yet";
    return FFTSO3_ERR_UNSUPPORTED;
}
void tc_destroy(TCState* s) { delete s; }
long long tc_device_bytes(const TCState*) { return 0; }
int tc_forward(TCState*, const void*, void*, cudaStream_t, std::string& err)
{
    err = "tensor-core precision not built yet";
    return FFTSO3_ERR_UNSUPPORTED;
}
int tc_inverse(TCState*, const void*, void*, cudaStream_t, std::string& err)
{
    err = "tensor-core precision not built yet";
    return FFTSO3_ERR_UNSUPPORTED;
}

}  // namespace fftso3
