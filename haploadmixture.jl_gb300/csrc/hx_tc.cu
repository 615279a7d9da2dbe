// hx_tc.cu -- dispatch of the tensor-core passes on K.  The kernels live in
// hx_tc_impl.cuh and are instantiated a few K at a time by hx_tc_g*.cu, so
// that the units compile in parallel.
#include "hx_ops.cuh"

namespace hx {
namespace {
cudaError_t tc_run_any(TcCall& c) {
    if (c.K < 1 || c.K > 12) return cudaErrorInvalidValue;
    if (c.K <= 7) return tc_run_g1(c);
    if (c.K <= 9) return tc_run_g2(c);
    if (c.K == 10) return tc_run_g3(c);
    if (c.K == 11) return tc_run_g4(c);
    return tc_run_g5(c);
}
}  // namespace

cudaError_t init_tc_attrs() {
    for (int K = 1; K <= 12; ++K) {
        TcCall c{TC_ATTRS, K, true, nullptr, nullptr, 0, 0, 0};
        const cudaError_t e = tc_run_any(c);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

int tc_resident(int K, bool p_side) {
    TcCall c{p_side ? TC_RESIDENT_P : TC_RESIDENT_Q, K, true, nullptr, nullptr, 0, 0, 0};
    return tc_run_any(c) == cudaSuccess ? (int)c.bytes : 1;
}

size_t tc_image_bytes(int K, int64_t I, int64_t J) {
    TcCall c{TC_IMG_BYTES, K, true, nullptr, nullptr, I, J, 0};
    return tc_run_any(c) == cudaSuccess ? c.bytes : 0;
}

cudaError_t launch_accum_q_tc(int K, bool hess, const PassArgs& a, cudaStream_t st) {
    TcCall c{TC_Q, K, hess, &a, st, a.I, a.J, 0};
    return tc_run_any(c);
}

cudaError_t launch_accum_p_tc(int K, bool hess, const PassArgs& a, cudaStream_t st) {
    TcCall c{TC_P, K, hess, &a, st, a.I, a.J, 0};
    return tc_run_any(c);
}

}  // namespace hx
