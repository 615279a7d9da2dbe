// hx_loglik_f32.cu -- instantiations of the mixed method's log-likelihood pass.
#include "hx_ops.cuh"

#define HX_FOR_K(X) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12)

namespace hx {

int loglik_f32x2_blocks(int64_t Ipad) { return (int)((Ipad + 2 * ACC_THREADS - 1) / (2 * ACC_THREADS)); }

cudaError_t launch_loglik_f32x2(int K, const PassArgs& a, cudaStream_t st) {
    dim3 grid((unsigned)loglik_f32x2_blocks(a.Ipad), (unsigned)a.S);
#define HX_CASE(KK) case KK: k_loglik2<KK><<<grid, ACC_THREADS, 0, st>>>(a); break;
    switch (K) { HX_FOR_K(HX_CASE) default: return cudaErrorInvalidValue; }
#undef HX_CASE
    return cudaGetLastError();
}

}  // namespace hx
