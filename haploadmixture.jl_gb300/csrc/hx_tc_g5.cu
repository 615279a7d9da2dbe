// hx_tc_g5.cu -- tensor-core pass instantiations for K = 12.
#include "hx_tc_impl.cuh"

namespace hx {
cudaError_t tc_run_g5(TcCall& c) {
    switch (c.K) {
        case 12: return tc_run<12>(c);
    }
    return cudaErrorInvalidValue;
}
}  // namespace hx
