/* haplo_gb300.h -- C ABI of the GB300 (sm_103a) HaploADMIXTURE fitting path.
 *
 * One context (hx_ctx) owns, for its whole lifetime, all device memory of one
 * fit on one GPU: the decoded genotype classes, the Q/P iterates of
 * AdmixData2 (x, x_next, x_next2, x_tmp; K x (I+4J) FP64, Julia column-major),
 * the gradient/Hessian buffers, the ZAL secant matrices U/V and the scratch of
 * the reductions.  Host buffers are owned by the caller; the library copies
 * them in or out during the call and never keeps a host pointer.
 *
 * Layouts follow the reference's Julia arrays (column-major, 0-based here):
 *   bed   : PLINK 1 .bed data bytes after the 3-byte magic, SNP-major,
 *           bytes_per_snp = ceil(N_file/4) bytes per SNP (SnpArray.data)
 *   q     : K x I            q[k + K*i]
 *   p     : K x 4J           p[k + K*m], m = 4j + h, h in {00,01,10,11}
 *   XtX_q : K x K x I        XtX[k2 + K*k + K*K*i]      Xtz_q : K x I
 *   XtX_p : K x K x 4J       XtX[k2 + K*k + K*K*m]      Xtz_p : K x 4J
 *
 * Every entry point returns an int status (HX_OK = 0).  hx_last_error()
 * returns the context's last message.  No C++ exception crosses the ABI.
 * A context is used by one host thread at a time; distinct contexts are
 * independent.  There is no CPU fallback: without a usable CUDA device
 * hx_create returns HX_ECUDA.
 */
#ifndef HAPLO_GB300_H
#define HAPLO_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HX_OK 0
#define HX_EINVAL 1        /* bad argument or size */
#define HX_ECUDA 2         /* CUDA runtime error, or no device */
#define HX_ENAN 3          /* NaN in a gradient/Hessian (src/algorithms_inner.jl:132-133) */
#define HX_ETIMEOUT 4      /* an iteration cap was hit, or a tensor-core pipeline wait ran out
                              (hx_set_wait_budget); the context stays usable */
#define HX_ENOMEM 5        /* device allocation failed */
#define HX_ESTATE 6        /* call out of order (e.g. no Q/P set yet) */
#define HX_EUNSUPPORTED 7  /* K outside 1..HX_KMAX, or secant count outside 1..HX_QMAX */

#define HX_KMAX 12
#define HX_QMAX 6

#define HX_PREC_FP64 0     /* plain method: every pass in FP64 */
#define HX_PREC_MIXED 1    /* FP32 per-pair arithmetic, FP64 totals, FP64 QP/QN */

typedef struct hx_ctx hx_ctx;

#define HX_PATH_AUTO 0     /* mixed method: Hessian passes on the tensor cores (tcgen05) */
#define HX_PATH_CUDA_CORES 1  /* mixed method: every pass on the CUDA cores */

typedef struct hx_opts {
    int32_t precision;     /* HX_PREC_FP64 (default) or HX_PREC_MIXED */
    int32_t device;        /* CUDA device ordinal (default 0) */
    int32_t Qsec;          /* secant pairs of the QN step, AdmixData2.Q (default 3; driver.jl:50) */
    int32_t verbose;       /* 1: one JSON line per outer iteration on stderr */
    double rho;            /* P-step penalty (default 1e7; algorithms_inner.jl:225) */
    double pseudocount;    /* projection floor (default 1e-5; utils.jl:20) */
    int32_t path;          /* HX_PATH_AUTO (default) or HX_PATH_CUDA_CORES */
    int32_t reserved;
} hx_opts;

typedef struct hx_iter_info {
    int32_t iter;          /* outer iteration number (1-based) */
    int32_t accepted_qn;   /* 1 if the ZAL point was kept (algorithms_outer.jl:154-160) */
    double ll_prev, ll_basic, ll_qn, ll_new, reldiff;
    double seconds;        /* device time of the iteration */
} hx_iter_info;

typedef struct hx_fit_info {
    int32_t iters;         /* outer iterations run */
    int32_t converged;     /* reldiff < rtol reached */
    int32_t em_iters;      /* EM iterations run before the QN loop */
    int32_t pad_;
    double ll;             /* final log-likelihood (d.ll_new) */
    double seconds;        /* wall time of the call */
} hx_fit_info;

/* Loop options of admixture_qn! / init_em! (src/algorithms_outer.jl:1-3,
 * 38-41; src/driver.jl:54-55).  Set per context with hx_set_loop_opts; they
 * apply to hx_init_em, hx_update_q/p, hx_qn_iteration, hx_admixture_qn and
 * hx_fit. */
typedef struct hx_loop_opts {
    int32_t fix_q;               /* 1: Q stays unchanged (q_next = q) */
    int32_t fix_p;               /* 1: P stays unchanged */
    int32_t guarantee_increase;  /* 1: halve each update's step until the log-likelihood does not drop
                                    (src/algorithms_inner.jl:169-199 Q with >=, :313-343 P with >) */
    int32_t penalty;             /* -1 (default, penalty=nothing): P penalty form, Q equality form;
                                    1: penalty form for both (rho * 1 1' on each Q block);
                                    0: equality form for both (P: sum_h d[k,h] = 0 for every k,
                                       src/algorithms_inner.jl:307-310) */
    int32_t mode;                /* admixture_qn!'s mode (src/algorithms_outer.jl:128-138): 0 = :ZAL
                                    (default), 1 = :LBQN, the limited-memory Broyden step
                                    x_next - V ((U-V)'(U-V))^-1 (U-V)'(x - x_next) */
} hx_loop_opts;

/* Defaults: precision FP64, device 0, Qsec 3, rho 1e7, pseudocount 1e-5. */
int hx_opts_default(hx_opts* opts);
/* Defaults: no fixed factor, no step control, penalty -1, mode 0 (ZAL). */
int hx_loop_opts_default(hx_loop_opts* opts);
int hx_set_loop_opts(hx_ctx* ctx, const hx_loop_opts* opts);
const char* hx_status_string(int status);
const char* hx_last_error(const hx_ctx* ctx);

/* Replaces _cu_admixture_base / CuAdmixData (src/cuda/structs.jl:16-44,
 * src/driver.jl:203-205): uploads the first I individuals x first 2J SNPs of
 * the BED matrix (host memory), decodes them once into class words, counts
 * double-missing blocks over all n_snp SNPs (src/utils.jl:1-18).  Q/P are
 * unset until hx_set_qp. */
int hx_create(const uint8_t* bed, int64_t bytes_per_snp, int64_t n_snp, int64_t I, int64_t J, int32_t K,
              const hx_opts* opts, hx_ctx** out);
/* Same, with the BED matrix already in device memory of opts->device. */
int hx_create_device(const uint8_t* d_bed, int64_t bytes_per_snp, int64_t n_snp, int64_t I, int64_t J,
                     int32_t K, const hx_opts* opts, hx_ctx** out);
int hx_destroy(hx_ctx* ctx);
int hx_dims(const hx_ctx* ctx, int64_t* I, int64_t* J, int32_t* K);

/* State (AdmixData2.q / .p, src/structs.jl:36-46).  which: 0 x, 1 x_next,
 * 2 x_next2, 3 x_tmp.  q/p may be NULL to skip one of them. */
int hx_set_qp(hx_ctx* ctx, const double* q, const double* p);
int hx_set_qp_device(hx_ctx* ctx, const double* d_q, const double* d_p);
int hx_get_qp(hx_ctx* ctx, int32_t which, double* q, double* p);
/* d.ll_new (NaN until computed) */
int hx_get_ll(hx_ctx* ctx, double* ll_new);

/* Genotype checks: 16-class census, index g1*4+g2 with missing = 3 (bit-exact
 * integer counts over the I x J pairs), and double-missing counts per individual. */
int hx_census(hx_ctx* ctx, uint64_t counts[16]);
int hx_double_missing(hx_ctx* ctx, int64_t* dm);

/* ---- the reference's GPU runners (src/cuda/runners.jl), on host arrays ---- */
/* loglikelihood(d_cu, g_cu, q, p) (runners.jl:13-16).  q/p NULL -> device x. */
int hx_loglikelihood(hx_ctx* ctx, const double* q, const double* p, double* ll);
/* em!(d_cu, g_cu) raw numerators (runners.jl:45-49; kernels.jl:42-73). */
int hx_em_accum(hx_ctx* ctx, const double* q, const double* p, double* q_next, double* p_next);
/* update_q_cuda!(d_cu, g_cu) (runners.jl:71-74; kernels.jl:104-138). */
int hx_update_q_accum(hx_ctx* ctx, const double* q, const double* p, double* XtX, double* Xtz);
/* update_p_cuda!(d_cu, g_cu) (runners.jl:89-92; kernels.jl:140-175). */
int hx_update_p_accum(hx_ctx* ctx, const double* q, const double* p, double* XtX, double* Xtz);
/* em_p!(d_cu, g_cu) raw P numerators only (runners.jl:51-55; kernels.jl:75-102). */
int hx_em_p_accum(hx_ctx* ctx, const double* q, const double* p, double* p_next);

/* Bound on any one pipeline wait of the tensor-core passes, in SM clock
 * cycles (clock64).  No reference counterpart (CUDA.jl kernels never wait on
 * one another).  A wait that runs out makes the pass stop early: it drains the
 * copies and MMAs it issued (each such wait allowed HX_WAIT_BUDGET_DEFAULT
 * cycles), releases its tensor memory, and the call returns HX_ETIMEOUT with
 * the context still usable.  cycles <= 0 restores the default. */
#define HX_WAIT_BUDGET_DEFAULT 4000000000LL
int hx_set_wait_budget(hx_ctx* ctx, int64_t cycles);

/* ---- batched QP / projection (CPU-only in the reference) on host arrays ---- */
/* Per individual: argmin 0.5 d'Hd - g'd, sum d = 0, 0 <= q+d <= 1 with
 * H = XtX[:,:,i], g = Xtz[:,i] (algorithms_inner.jl:134-168). n individuals.
 * With loop option penalty = 1: H + rho 1 1' and no equality (:158-162). */
int hx_qp_q(hx_ctx* ctx, int64_t n, const double* XtX, const double* Xtz, const double* q, double* qdiff);
/* Per block: 4K variables, H = blockdiag(XtX[:,:,4j+h]) + rho on the
 * (h,h2,k) pattern, 0 <= p+d <= 1 (algorithms_inner.jl:264-305). n blocks.
 * With loop option penalty = 0: no rho and sum_h d[k,h] = 0 for every k (:307-310). */
int hx_qp_p(hx_ctx* ctx, int64_t n, const double* XtX, const double* Xtz, const double* p, double* pdiff);
/* OpenADMIXTURE.project_q! per column / project_p! per (k, block) quartet. */
int hx_project_q(hx_ctx* ctx, int64_t ncol, double* q);
int hx_project_p(hx_ctx* ctx, int64_t nblocks, double* p);
/* ZAL quasi-Newton point (update_UV! + update_QN!, algorithms_outer.jl:129-133)
 * on host vectors of length n = K(I+4J): U/V are n x Qsec and are updated. */
int hx_zal(hx_ctx* ctx, const double* x, const double* x_next, const double* x_next2, double* U, double* V,
           int32_t iter, double* x_tmp);

/* ---- device-resident algorithm steps (algorithms_inner.jl / _outer.jl) ---- */
/* em! (algorithms_inner.jl:29-84): x -> x_next (normalised, projected). */
int hx_em_step(hx_ctx* ctx);
/* init_em! (algorithms_outer.jl:1-22): iters EM steps; sets d.ll_new. */
int hx_init_em(hx_ctx* ctx, int32_t iters);
/* update_q!(d, g, update2) / update_p!(d, g, update2) (algorithms_inner.jl:97-355). */
int hx_update_q(hx_ctx* ctx, int32_t update2);
int hx_update_p(hx_ctx* ctx, int32_t update2);
/* One outer iteration of admixture_qn! (algorithms_outer.jl:65-171, :ZAL). */
int hx_qn_iteration(hx_ctx* ctx, hx_iter_info* info);
/* admixture_qn!(d, g, n_iter, rtol; iter_count_offset) (algorithms_outer.jl:38-172). */
int hx_admixture_qn(hx_ctx* ctx, int32_t n_iter, double rtol, int32_t iter_offset, hx_fit_info* info);
/* _admixture_base's fit sequence (driver.jl:181-197): init_em! (em_iters) then
 * admixture_qn!.  Starts from the current x. */
int hx_fit(hx_ctx* ctx, int32_t n_iter, double rtol, int32_t em_iters, hx_fit_info* info);

/* Batched fits for the K sweep with random restarts (README.md:9 names AIC
 * model selection; run_admixture fits one K per call, src/driver.jl:38-79).
 * No reference counterpart: the reference runs such sweeps as separate
 * run_admixture calls.
 *
 * hx_create_shared: a context for K ancestries that shares the parent's
 * decoded genotype classes and double-missing counts (no second upload or
 * decode).  The parent must outlive it.  opts->device is ignored (the
 * parent's device is used).
 *
 * hx_fit_many: hx_fit on each of n contexts, up to `threads` at a time (0 =
 * all) from host threads, each context on its own CUDA stream, so that the
 * fits' kernels overlap on the GPU.  Each context gives the same result as
 * hx_fit alone.  status (optional, n entries) receives each fit's status;
 * the return value is the first non-OK status, or HX_OK. */
int hx_create_shared(const hx_ctx* parent, int32_t K, const hx_opts* opts, hx_ctx** out);
/* Learned warm start of Q (no reference counterpart).
 * Features of (individual i, ancestry k), two FP32 values each, feat[i][k][2]:
 *   f1 = a_k - max_k' a_k', a_k = (1/n_i) sum_j log L_ij(Q_i = e_k)
 *   f2 = (g - 1) sqrt(n_i), g = Xtz_q[k,i] / (2 n_i) (Q gradient per block),
 *   n_i = J - dm_i.
 * Network, permutation-equivariant over k, FP16 weights and FP32 accumulation:
 *   h1_k = relu(W1 x_k + b1), m = mean_k h1_k, h2_k = relu(W2 h1_k + U2 m + b2),
 *   z_k = w3.h2_k + b3, q = softmax(z).  Parameters: FP32 master copy, layout
 *   W1[64][2], b1[64], W2[64][64], U2[64][64], b2[64], w3[64], b3 (HX_LWS_NPARAM
 *   floats, zero-padded).  Loss: cross-entropy against converged Q.
 * Device pointers unless stated; stream may be NULL. */
#define HX_LWS_HIDDEN 64
#define HX_LWS_NPARAM 8516
/* Features at the context's current state (device, I*K*2 floats). */
int hx_lws_features(hx_ctx* ctx, float* d_feat);
/* q[i][k] for n samples of K ancestries. */
int hx_lws_forward(const float* d_feat, int64_t n, int32_t K, const float* d_params, float* d_q, void* stream);
/* Mean loss and its gradient over all n samples (d_grad: HX_LWS_NPARAM floats). */
int hx_lws_grad(const float* d_feat, const float* d_target, int64_t n, int32_t K, const float* d_params,
                float* d_grad, double* d_loss, void* stream);
/* `steps` Adam steps (lr, beta 0.9/0.999) on mini-batches of `batch` samples
 * drawn with replacement by a counter-based hash of (seed, step0 + s, slot);
 * d_m, d_v: Adam moments (HX_LWS_NPARAM floats each, zero at the start);
 * d_losses (optional): mean loss of each step's batch, before the update. */
int hx_lws_train(const float* d_feat, const float* d_target, int64_t n, int32_t K, float* d_params, float* d_m,
                 float* d_v, int32_t steps, int64_t batch, float lr, uint64_t seed, int32_t step0, double* d_losses,
                 void* stream);
/* Warm start: Q' = project(network(features of the current state)); with
 * p_step, P' = one P step (update_p!) at (Q', P), else P' = P.  (Q', P')
 * replaces the state if it raises the log-likelihood; then the QN history is
 * reset (hx_set_qp semantics).  params: host, HX_LWS_NPARAM floats.
 * *accepted (optional) = 1 if the state was replaced. */
int hx_lws_warm_start(hx_ctx* ctx, const float* params, int32_t p_step, int32_t* accepted);
int hx_fit_many(hx_ctx* const* ctxs, int32_t n, int32_t n_iter, double rtol, int32_t em_iters, int32_t threads,
                hx_fit_info* infos, int32_t* status);

/* AIM selection before the fit (run_admixture's `sparsity` branch,
 * src/driver.jl:60-73, 84-105): sparse k-means with feature ranking (SKFR1 of
 * Zhang, Lange and Xu 2020; the reference calls SparseKmeansFeatureRanking
 * 0.1.2's sparsekmeans1 on blocks of 2 SNPs) over the first I individuals of
 * the SNP-major BED matrix (host memory, bytes_per_snp bytes per SNP, n_snp
 * SNPs; an odd last SNP is ignored).  Genotypes are standardised per SNP
 * (missing -> mean), the start is k-means++ with uniform draws
 * SplitMix64(seed + t), and `sparsity` blocks are kept.  Outputs: clusters
 * (I entries, 0..K-1), aims (2 * sparsity sorted SNP indices), *iters and
 * *objective (optional: the within-cluster sum of squares over the kept SNPs,
 * which sparsekmeans_repeat compares across tries).  HX_EINVAL for K > I or
 * sparsity outside 1..n_snp/2. */
int hx_skfr(const uint8_t* bed, int64_t bytes_per_snp, int64_t n_snp, int64_t I, int32_t K, int64_t sparsity,
            int32_t max_iter, uint64_t seed, int32_t device, int32_t* clusters, int64_t* aims, int32_t* iters,
            double* objective);

/* Tile-shape autotuner of the mixed method (no reference counterpart): times
 * the Q and P tensor-core passes and the FP32 log-likelihood pass at the
 * context's current Q/P for chunk counts (grid splits along the reduction)
 * from half to twice the planned ones, keeps the fastest for this context,
 * and applies it to every later context of the same device, K, I and J in
 * this process (hx_create, hx_create_shared).  A different chunking only
 * reorders the FP32/FP64 partial sums.  chunks (optional, 3 entries)
 * receives the chosen chunk counts (Q pass, P pass, log-likelihood).  No-op
 * (HX_OK) for the plain FP64 method and the CUDA-core path. */
int hx_autotune(hx_ctx* ctx, int32_t* chunks);

/* ---- launch accounting (no counterpart in the reference, which prints
 * @time per phase, src/algorithms_inner.jl:114,135,241,259) ---- */
#define HX_KIND_ACCUM_Q 0  /* Q-side gradient+Hessian pass */
#define HX_KIND_ACCUM_P 1  /* P-side gradient+Hessian pass */
#define HX_KIND_LOGLIK 2   /* log-likelihood pass */
#define HX_KIND_QP_Q 3     /* batched per-individual QP */
#define HX_KIND_QP_P 4     /* batched per-block QP */
#define HX_KIND_QN 5       /* ZAL secant update, solve and step */
#define HX_KIND_OTHER 6    /* reductions, projections, bookkeeping */
#define HX_KIND_EM_Q 7     /* Q-side gradient-only pass (EM numerators) */
#define HX_KIND_EM_P 8     /* P-side gradient-only pass (EM numerators) */
#define HX_NKIND 9
/* on != 0: record CUDA events around every launch on the context's stream. */
int hx_set_profiling(hx_ctx* ctx, int32_t on);
/* Launches issued (always counted) and device ms (while profiling) of a kind. */
int hx_kernel_stats(hx_ctx* ctx, int32_t kind, int64_t* launches, double* ms);
int hx_reset_stats(hx_ctx* ctx);

/* ---- synthetic cohorts ---- */
/* Writes the SNP-major BED matrix (ceil(I/4) bytes per SNP, 2J SNPs) of a
 * synthetic admixed cohort into device memory d_bed: per (i, j) two haplotype
 * copies with ancestry z ~ Cat(Q_i) and haplotype h ~ Cat(P_{z,j}); missing at
 * rate miss per (i, SNP).  thrQ (K x I) and thrP (K x 4J) are the cumulative
 * probabilities as integer thresholds ceil(cum * 2^53) (last entry may be any
 * value >= 2^53).  Counter-based SplitMix64 draws: the bytes equal those of the
 * CPU generator bit for bit. */
int hx_synth_bed_device(uint64_t seed, int64_t I, int64_t J, int32_t K, const uint64_t* thrQ,
                        const uint64_t* thrP, double miss, uint8_t* d_bed, int32_t device);

/* ---- log-likelihood without device allocation ----
 * No counterpart in the reference.  For callers that must not allocate
 * device memory at call time: frameworks that hand out all device memory
 * from their own pool (CUDA.jl, the PyTorch caching allocator) and forbid side
 * allocations, or latency-critical loops where cudaMalloc/cudaFree would
 * synchronise the device.  Evaluates the same log-likelihood as
 * hx_loglikelihood (src/loops.jl:236-258) straight from caller-owned device
 * buffers: d_bed (first I individuals x first 2J SNPs of the SNP-major BED
 * matrix, bytes_per_snp bytes per SNP), d_q (K x I) and d_p (K x 4J), FP64,
 * column-major; writes one double to d_ll.  Kernels are enqueued on `stream`
 * (a cudaStream_t, NULL = legacy default stream); the call does not
 * synchronise.
 *
 * Its only scratch is a file-scope device array of HX_NOALLOC_SCRATCH doubles
 * (256 KB), held by every GPU that loads this library until the process exits.
 * Every call looks up that array's device address in the current device's
 * context (cudaGetSymbolAddress, which allocates nothing), so a device reset
 * between calls is safe; the first call in a context also loads the module,
 * so make that first call before any stream capture.  Q and P may hold any
 * values in [0, 1]; in the mixed method a pair whose FP32 likelihood falls
 * below the smallest normal float is evaluated in FP64.  Every call shares the
 * array and leaves its partial sums
 * in it; each call overwrites all the partials it reads, so nothing needs to
 * start at zero.  Calls that overlap on the GPU (different streams, or other
 * host threads) race on the array and must be serialised by the caller.
 * Returns HX_EUNSUPPORTED when ceil(I/128) exceeds HX_NOALLOC_SCRATCH
 * (I > 4,194,304) or K is outside 1..HX_KMAX, HX_EINVAL for bad arguments, and
 * HX_ECUDA on a CUDA error.  Calls no cudaMalloc, cudaFree or allocating
 * library routine. */
#define HX_NOALLOC_SCRATCH 32768
int hx_loglikelihood_noalloc(const uint8_t* d_bed, int64_t bytes_per_snp, int64_t I, int64_t J, int32_t K,
                             const double* d_q, const double* d_p, int32_t precision, double* d_ll, void* stream);

#ifdef __cplusplus
}
#endif
#endif
