// hx_loglik_f32.cu -- instantiations of the mixed method's log-likelihood pass.
#include "hx_ops.cuh"

#define HX_FOR_K(X) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12)

namespace hx {

// individuals per thread (4 measured slower at K = 8: 155 registers cut the
// resident warps from 20 to 12 per SM)
inline int loglik_nu(int) { return 2; }
int loglik_f32x2_blocks(int64_t Ipad, int K) {
    const int64_t per = (int64_t)loglik_nu(K) * ACC_THREADS;
    return (int)((Ipad + per - 1) / per);
}

int loglik_f32x2_resident(int K) {
#define HX_CASE(KK) case KK: return resident_ctas((const void*)k_loglik2<KK, 2>, ACC_THREADS, 0, 0);
    switch (K) { HX_FOR_K(HX_CASE) default: return 1; }
#undef HX_CASE
}

cudaError_t launch_loglik_f32x2(int K, const PassArgs& a, cudaStream_t st) {
    dim3 grid((unsigned)loglik_f32x2_blocks(a.Ipad, K), (unsigned)a.S);
#define HX_CASE(KK) case KK: k_loglik2<KK, 2><<<grid, ACC_THREADS, 0, st>>>(a); break;
    switch (K) { HX_FOR_K(HX_CASE) default: return cudaErrorInvalidValue; }
#undef HX_CASE
    return cudaGetLastError();
}

}  // namespace hx
