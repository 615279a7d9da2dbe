// hx_tc_g3.cu -- tensor-core pass instantiations for K = 10.
#include "hx_tc_impl.cuh"

namespace hx {
cudaError_t tc_run_g3(TcCall& c) {
    switch (c.K) {
        case 10: return tc_run<10>(c);
    }
    return cudaErrorInvalidValue;
}
}  // namespace hx
