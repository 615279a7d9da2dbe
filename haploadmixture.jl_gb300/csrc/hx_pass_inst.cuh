// hx_pass_inst.cuh -- instantiates the pass kernels for one arithmetic type.
// Included by hx_pass_f64.cu (HX_T = double) and hx_pass_f32.cu (HX_T = float)
// so that the two precisions compile as separate translation units.
#pragma once
#include "hx_ops.cuh"

#define HX_CAT2(a, b) a##_##b
#define HX_CAT(a, b) HX_CAT2(a, b)
#define HX_FOR_K(X) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12)

namespace hx {

cudaError_t HX_CAT(launch_accum_q, HX_SUF)(int K, bool hess, const PassArgs& a, cudaStream_t st) {
    dim3 grid((unsigned)(a.Ipad / ACC_THREADS), (unsigned)a.S);
#define HX_CASE(KK) \
    case KK: if (hess) k_accum_q<KK, HX_T, true><<<grid, ACC_THREADS, 0, st>>>(a); \
             else k_accum_q<KK, HX_T, false><<<grid, ACC_THREADS, 0, st>>>(a); break;
    switch (K) { HX_FOR_K(HX_CASE) default: return cudaErrorInvalidValue; }
#undef HX_CASE
    return cudaGetLastError();
}

cudaError_t HX_CAT(launch_accum_p, HX_SUF)(int K, bool hess, const PassArgs& a, cudaStream_t st) {
    dim3 grid((unsigned)((a.J + 31) / 32), (unsigned)a.S);
#define HX_CASE(KK) \
    case KK: if (hess) k_accum_p<KK, HX_T, true><<<grid, ACC_THREADS, 0, st>>>(a); \
             else k_accum_p<KK, HX_T, false><<<grid, ACC_THREADS, 0, st>>>(a); break;
    switch (K) { HX_FOR_K(HX_CASE) default: return cudaErrorInvalidValue; }
#undef HX_CASE
    return cudaGetLastError();
}

cudaError_t HX_CAT(launch_loglik, HX_SUF)(int K, const PassArgs& a, cudaStream_t st) {
    dim3 grid((unsigned)(a.Ipad / ACC_THREADS), (unsigned)a.S);
#define HX_CASE(KK) case KK: k_loglik<KK, HX_T><<<grid, ACC_THREADS, 0, st>>>(a); break;
    switch (K) { HX_FOR_K(HX_CASE) default: return cudaErrorInvalidValue; }
#undef HX_CASE
    return cudaGetLastError();
}

}  // namespace hx
