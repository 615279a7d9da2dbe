// hx_ops.cuh -- declarations of the non-pass kernels and launchers (hx_ops.cu)
// and of the pass launchers (hx_pass_f64.cu / hx_pass_f32.cu).
#pragma once
#include "hx_pass.cuh"

namespace hx {

// Slots of the per-context device scalar block (double[HX_NSLOT]).
enum Slot {
    S_LL_NEW = 0, S_LL_PREV = 1, S_LL_BASIC = 2, S_LL_QN = 3, S_RELDIFF = 4, S_ACCEPT_QN = 5,
    S_ITER = 6, S_TMP = 7, S_QP_FAIL = 8, S_NAN = 9, S_TC_TIMEOUT = 10, HX_NSLOT = 16
};

// pass launchers: precision-specific translation units
cudaError_t launch_accum_q_f64(int K, bool hess, const PassArgs& a, cudaStream_t st);
cudaError_t launch_accum_p_f64(int K, bool hess, const PassArgs& a, cudaStream_t st);
cudaError_t launch_loglik_f64(int K, const PassArgs& a, cudaStream_t st);
cudaError_t launch_accum_q_f32(int K, bool hess, const PassArgs& a, cudaStream_t st);
cudaError_t launch_accum_p_f32(int K, bool hess, const PassArgs& a, cudaStream_t st);
cudaError_t launch_loglik_f32(int K, const PassArgs& a, cudaStream_t st);
cudaError_t launch_loglik_f32x2(int K, const PassArgs& a, cudaStream_t st);   // several individuals per thread
int loglik_f32x2_blocks(int64_t Ipad, int K);
int loglik_f32x2_resident(int K);   // CTAs of launch_loglik_f32x2 resident on one SM
// CTAs of a kernel resident on one SM of the current device, from its
// registers (8-register steps per thread, 256-register steps per warp, a
// quarter of the file per SM sub-partition), its shared memory (static +
// dynamic + the driver's reserve), its threads and, for kernels that
// allocate them, TMEM columns (512 per SM).  The runtime's occupancy
// calculator reports one CTA for the tensor-core passes where the hardware
// holds two, so the limits are applied here.
int resident_ctas(const void* kernel, int threads, size_t dyn_smem, int tmem_cols);

// tensor-core (tcgen05) Hessian+gradient passes of the mixed method (hx_tc.cu)
// Host operations on the tensor-core instantiation of one K (hx_tc_impl.cuh);
// each hx_tc_g*.cu unit serves a few values of K.
enum TcOp { TC_ATTRS, TC_IMG_BYTES, TC_Q, TC_P, TC_RESIDENT_Q, TC_RESIDENT_P };
struct TcCall {
    TcOp op;
    int K;
    bool hess;
    const PassArgs* a;
    cudaStream_t st;
    int64_t I, J;
    size_t bytes;
};
cudaError_t tc_run_g1(TcCall& c);   // K = 1..7
cudaError_t tc_run_g2(TcCall& c);   // K = 8, 9
cudaError_t tc_run_g3(TcCall& c);   // K = 10
cudaError_t tc_run_g4(TcCall& c);   // K = 11
cudaError_t tc_run_g5(TcCall& c);   // K = 12
cudaError_t init_tc_attrs();
// CTAs of the Hessian tensor-core pass resident on one SM (registers, shared
// memory and TMEM columns), after init_tc_attrs
int tc_resident(int K, bool p_side);

cudaError_t launch_f2d(const float* a, int64_t n, double* out, cudaStream_t st);
cudaError_t launch_d2f(const double* a, int64_t n, float* out, cudaStream_t st);

// learned warm start (hx_lws.cu)
cudaError_t lws_attrs();
cudaError_t lws_features(int K, const PassArgs& a, const unsigned long long* dm, const double* Xtz, float* feat,
                         cudaStream_t st);
cudaError_t lws_forward(const float* feat, int64_t n, int K, const float* P, float* q, cudaStream_t st);
cudaError_t lws_grad(const float* feat, const float* target, const int64_t* idx, int64_t ns, int K, const float* P,
                     float* part, double* loss_part, float* grad, double* loss, cudaStream_t st);
cudaError_t lws_train(const float* feat, const float* target, int64_t n, int K, float* P, float* m, float* v,
                      int steps, int64_t bs, float lr, uint64_t seed, int step0, int64_t* idx, float* part,
                      double* loss_part, float* grad, double* losses, cudaStream_t st);
constexpr int LWS_MAX_BLOCKS = 304;   // CTA partials of lws_grad
cudaError_t launch_accum_q_tc(int K, bool hess, const PassArgs& a, cudaStream_t st);
cudaError_t launch_accum_p_tc(int K, bool hess, const PassArgs& a, cudaStream_t st);
size_t tc_image_bytes(int K, int64_t I, int64_t J);

// decode / checks / synthetic data
cudaError_t launch_pack(const uint8_t* bed, int64_t bps, int64_t I, int64_t J, int64_t Ipad, int JW, uint32_t* G,
                        cudaStream_t st);
cudaError_t launch_census(const uint32_t* G, int64_t Ipad, int64_t I, int64_t J, int JW,
                          unsigned long long* counts, cudaStream_t st);
cudaError_t launch_double_missing(const uint8_t* bed, int64_t bps, int64_t I, int64_t nsnp,
                                  unsigned long long* dm, cudaStream_t st);
cudaError_t launch_synth(uint64_t seed, int64_t I, int64_t J, int K, const uint64_t* thrQ, const uint64_t* thrP,
                         double miss, uint8_t* bed, cudaStream_t st);

// reductions of pass partials
cudaError_t launch_reduce_sym(const double* part, int S, int K, bool hess, int64_t rows, int64_t ld,
                              double* XtX, double* Xtz, cudaStream_t st);
cudaError_t launch_reduce_sum(const double* part, int64_t n, double* out, cudaStream_t st);

// EM normalisation + projection (algorithms_inner.jl:66-76)
cudaError_t launch_em_q(const double* q, const double* Xtz, const unsigned long long* dm, int64_t J, int K,
                        int64_t I, double eps, double* q_next, cudaStream_t st);
cudaError_t launch_em_p(const double* p, const double* Xtz, int K, int64_t J, double eps, double* p_next,
                        cudaStream_t st);
// q_next = project(q + d) per column / quartet; d may be null (plain projection)
cudaError_t launch_step_q(const double* q, const double* d, int K, int64_t ncol, double eps, double* out,
                          cudaStream_t st, double factor = 1.0);
cudaError_t launch_step_p(const double* p, const double* d, int K, int64_t J, double eps, double* out,
                          cudaStream_t st, double factor = 1.0);
// batched QP (init_kernel_attrs: once per device, before the first launch)
cudaError_t init_kernel_attrs();
cudaError_t launch_qp_q(int K, int64_t n, const double* XtX, const double* Xtz, const double* q, double* qdiff,
                        double* slots, cudaStream_t st, double pen_rho = -1.0);
// eq: the equality form (K equalities per block, rho and ws unused)
cudaError_t launch_qp_p(int K, int64_t n, const double* XtX, const double* Xtz, const double* p, double rho,
                        double* pdiff, double* slots, int8_t* ws, cudaStream_t st, bool eq = false);
// quasi-Newton point (ZAL or LBQN)
int qn_dots_blocks(int64_t n);
// mode 0: ZAL, 1: LBQN (the limited-memory Broyden step)
cudaError_t launch_qn(int64_t n, const double* x, const double* xn, const double* xn2, double* U, double* V,
                      int Qs, double* part, double* coef, double* xt, double* slots, cudaStream_t st, int mode = 0);
// outer-iteration bookkeeping
cudaError_t launch_iter_begin(double* slots, cudaStream_t st);
cudaError_t launch_accept(int64_t n, double* x, const double* xt, const double* xn2, double* slots,
                          cudaStream_t st);
cudaError_t launch_copy_slot(double* slots, int dst, int src, cudaStream_t st);
cudaError_t launch_nan_check(const double* a, int64_t n, double* slots, cudaStream_t st);

}  // namespace hx
