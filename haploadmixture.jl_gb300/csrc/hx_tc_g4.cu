// hx_tc_g4.cu -- tensor-core pass instantiations for K = 11.
#include "hx_tc_impl.cuh"

namespace hx {
cudaError_t tc_run_g4(TcCall& c) {
    switch (c.K) {
        case 11: return tc_run<11>(c);
    }
    return cudaErrorInvalidValue;
}
}  // namespace hx
