// hx_tc_g2.cu -- tensor-core pass instantiations for K = 8, 9.
#include "hx_tc_impl.cuh"

namespace hx {
cudaError_t tc_run_g2(TcCall& c) {
    switch (c.K) {
        case 8: return tc_run<8>(c);
        case 9: return tc_run<9>(c);
    }
    return cudaErrorInvalidValue;
}
}  // namespace hx
