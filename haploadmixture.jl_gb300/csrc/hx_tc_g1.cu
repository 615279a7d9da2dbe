// hx_tc_g1.cu -- tensor-core pass instantiations for K = 1, 2, 3, 4, 5, 6, 7.
#include "hx_tc_impl.cuh"

namespace hx {
cudaError_t tc_run_g1(TcCall& c) {
    switch (c.K) {
        case 1: return tc_run<1>(c);
        case 2: return tc_run<2>(c);
        case 3: return tc_run<3>(c);
        case 4: return tc_run<4>(c);
        case 5: return tc_run<5>(c);
        case 6: return tc_run<6>(c);
        case 7: return tc_run<7>(c);
    }
    return cudaErrorInvalidValue;
}
}  // namespace hx
