// hx_api.cu -- context, device-resident fitting loop and the C ABI
// (include/haplo_gb300.h).  One context = one fit on one GPU, one CUDA stream;
// all iterates, gradients, Hessians and secants stay in HBM for the whole fit
// (the reference copies Q/P in and XtX/Xtz out on every half-step,
// src/algorithms_inner.jl:121-127, 247-253; here only two scalars per outer
// iteration cross PCIe/C2C).
#include "hx_ops.cuh"
#include "../../include/haplo_gb300.h"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>
#include <atomic>
#include <thread>
#include <map>
#include <mutex>
#include <tuple>

using namespace hx;

struct hx_ctx {
    int device = 0, prec = HX_PREC_FP64, Qs = 3, verbose = 0;
    double rho = 1e7, eps = 1e-5;
    int64_t I = 0, J = 0, nsnp = 0, bps = 0;
    int K = 0;
    int64_t Ipad = 0;
    int JW = 0;
    int64_t nx = 0;        // K * (I + 4J)
    cudaStream_t st = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    uint32_t* G = nullptr;
    unsigned long long* dm = nullptr;
    double *x = nullptr, *xn = nullptr, *xn2 = nullptr, *xt = nullptr, *xio = nullptr;
    double *U = nullptr, *V = nullptr;
    double *XtXq = nullptr, *Xtzq = nullptr, *XtXp = nullptr, *Xtzp = nullptr;
    double *part_q = nullptr, *part_p = nullptr, *part_ll = nullptr, *part_qn = nullptr, *coef = nullptr;
    float* pf = nullptr;                     // mixed: FP32 copy of the pass's p (K x 4J)
    double* slots = nullptr;
    double* h_slots = nullptr;   // pinned
    uint8_t* img = nullptr;      // B-operand image of the tensor-core passes
    int8_t* qp_ws = nullptr;     // P-side QP working sets, warm start of the next solve
    hx_loop_opts lo{0, 0, 0, -1};  // admixture_qn!/init_em! options
    double ll_tmp = NAN;         // d.ll_tmp of the step control
    bool shared_geno = false;    // G and dm belong to the parent context (hx_create_shared)
    int S_q = 1, wpc_q = 1, S_p = 1, ipc_p = 1;
    int S_ll = 1, wpc_ll = 1;                // FP32 log-likelihood pass
    bool tc = false;                         // Hessian passes on the tensor cores
    int S_qt = 1, wpc_qt = 2, S_pt = 1, ipc_pt = 64;
    // chunk counts the partial buffers hold: twice the plan's, the range the
    // autotuner tries (hx_autotune)
    int Sq_cap = 1, Sp_cap = 1, Sll_cap = 1;
    bool have_qp = false;
    long long wait_budget = HX_WAIT_BUDGET_DEFAULT;   // tensor-core pipeline waits (clock64 cycles)
    std::string err;
    // launch accounting: per kind, kernel launches issued and (when profiling
    // is on) device milliseconds from CUDA events recorded on this stream
    bool profiling = false;
    int64_t launches[HX_NKIND] = {0};
    double kms[HX_NKIND] = {0};
    struct Pending { int kind; cudaEvent_t a, b; };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> pool;
    cudaEvent_t open_ev = nullptr;
};

namespace {

int fail(hx_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}
int cuda_fail(hx_ctx* c, const char* what, cudaError_t e) {
    return fail(c, e == cudaErrorMemoryAllocation ? HX_ENOMEM : HX_ECUDA,
                std::string(what) + ": " + cudaGetErrorString(e));
}
#define HX_CK(expr)                                              \
    do {                                                         \
        cudaError_t e_ = (expr);                                 \
        if (e_ != cudaSuccess) return cuda_fail(c, #expr, e_);   \
    } while (0)
#define HX_ST(expr)                      \
    do {                                 \
        int s_ = (expr);                 \
        if (s_ != HX_OK) return s_;      \
    } while (0)

cudaEvent_t pool_get(hx_ctx* c) {
    if (!c->pool.empty()) {
        cudaEvent_t e = c->pool.back();
        c->pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
void prof_begin(hx_ctx* c) {
    if (!c->profiling) return;
    c->open_ev = pool_get(c);
    cudaEventRecord(c->open_ev, c->st);
}
void prof_end(hx_ctx* c, int kind, int n) {
    c->launches[kind] += n;
    if (!c->profiling || !c->open_ev) return;
    cudaEvent_t e = pool_get(c);
    cudaEventRecord(e, c->st);
    c->pending.push_back({kind, c->open_ev, e});
    c->open_ev = nullptr;
}
// after a stream synchronisation: fold the recorded intervals into kms[]
void prof_resolve(hx_ctx* c) {
    for (auto& p : c->pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) c->kms[p.kind] += ms;
        c->pool.push_back(p.a);
        c->pool.push_back(p.b);
    }
    c->pending.clear();
}
// one kernel launch (or n) of a kind, timed when profiling is on
#define HX_LAUNCH(kind, n, expr) \
    do {                         \
        prof_begin(c);           \
        HX_CK(expr);             \
        prof_end(c, kind, n);    \
    } while (0)

inline double* qof(double* x) { return x; }
inline double* pof(hx_ctx* c, double* x) { return x + (int64_t)c->K * c->I; }

// Chunks per tile for a pass of `tiles` independent tiles, each splitting
// `units` (word columns or 32-individual stages) into chunks, on `slots`
// resident CTAs: at least `waves` waves, and among up to twice that many
// chunks the count whose last wave is fullest (a part-filled last wave idles
// SMs for a whole CTA lifetime).  Returns the chunk length in units.
int64_t pick_chunk(int64_t tiles, int64_t units, int64_t slots, int64_t waves) {
    const int64_t s0 = std::min(units, std::max<int64_t>(1, (waves * slots + tiles - 1) / tiles));
    int64_t best = (units + s0 - 1) / s0;
    double beff = -1.0;
    for (int64_t s = s0; s <= std::min(units, 2 * s0); ++s) {
        const int64_t per = (units + s - 1) / s;
        const int64_t sa = (units + per - 1) / per;            // chunks formed
        const double w = (double)(tiles * sa) / (double)slots;
        const double eff = w / std::ceil(w);
        if (eff > beff + 1e-9) { beff = eff; best = per; }
    }
    return best;
}

// Chunk lengths (grid.y splits) of the mixed method's three pass kernels that
// hx_autotune measured fastest, per device, K, I and J, for the whole process.
struct TuneVal { int wpc_qt, spc_pt, wpc_ll; };
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int64_t, int64_t>, TuneVal> g_tune;

bool tune_lookup(const hx_ctx* c, TuneVal& v) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_tune.find(std::make_tuple(c->device, c->K, c->I, c->J));
    if (it == g_tune.end()) return false;
    v = it->second;
    return true;
}
void tune_store(const hx_ctx* c, const TuneVal& v) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune[std::make_tuple(c->device, c->K, c->I, c->J)] = v;
}
void apply_tuned(hx_ctx* c, const TuneVal& v) {
    const int64_t nst = (c->I + 31) / 32;
    c->wpc_qt = v.wpc_qt;
    c->S_qt = (c->JW + v.wpc_qt - 1) / v.wpc_qt;
    c->ipc_pt = v.spc_pt * 32;
    c->S_pt = (int)((nst + v.spc_pt - 1) / v.spc_pt);
    c->wpc_ll = v.wpc_ll;
    c->S_ll = (c->JW + v.wpc_ll - 1) / v.wpc_ll;
}

void plan(hx_ctx* c) {
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess || nsm < 1) nsm = 1;
    const int64_t target = 2048;
    const int64_t tilesQ = c->Ipad / ACC_THREADS;
    int64_t S = std::max<int64_t>(1, (target + tilesQ - 1) / tilesQ);
    S = std::min<int64_t>(S, c->JW);
    c->wpc_q = (int)((c->JW + S - 1) / S);
    c->S_q = (c->JW + c->wpc_q - 1) / c->wpc_q;
    const int64_t tilesP = (c->J + 31) / 32;
    int64_t Sp = std::max<int64_t>(1, (target + tilesP - 1) / tilesP);
    Sp = std::min<int64_t>(Sp, (c->I + PSTAGE_IND - 1) / PSTAGE_IND);
    int64_t ipc = (c->I + Sp - 1) / Sp;
    ipc = (ipc + PSTAGE_IND - 1) / PSTAGE_IND * PSTAGE_IND;
    c->ipc_p = (int)ipc;
    c->S_p = (int)((c->I + ipc - 1) / ipc);
    // tensor-core passes (stages of one word column, Q, or 32 individuals, P)
    // and the FP32 log-likelihood pass: >= 8 waves with a full last wave
    const int64_t wpc = pick_chunk(tilesQ, c->JW, (int64_t)nsm * tc_resident(c->K, false), 8);
    c->wpc_qt = (int)wpc;
    c->S_qt = (int)((c->JW + wpc - 1) / wpc);
    const int64_t nst = (c->I + 31) / 32;
    const int64_t spc = pick_chunk(tilesP, nst, (int64_t)nsm * tc_resident(c->K, true), 8);
    c->ipc_pt = (int)(spc * 32);
    c->S_pt = (int)((nst + spc - 1) / spc);
    const int64_t tilesL = loglik_f32x2_blocks(c->Ipad, c->K);
    c->wpc_ll = (int)pick_chunk(tilesL, c->JW, (int64_t)nsm * loglik_f32x2_resident(c->K), 8);
    c->S_ll = (c->JW + c->wpc_ll - 1) / c->wpc_ll;
    c->Sq_cap = std::min(c->JW, 2 * c->S_qt);
    c->Sp_cap = (int)std::min<int64_t>(nst, 2 * (int64_t)c->S_pt);
    c->Sll_cap = std::min(c->JW, 2 * c->S_ll);
    // chunk lengths an earlier hx_autotune chose for this shape (always
    // within the caps above, which depend on the shape only)
    TuneVal tv;
    if (c->tc && tune_lookup(c, tv)) apply_tuned(c, tv);
}

PassArgs pass_args(hx_ctx* c, const double* q, const double* p) {
    PassArgs a;
    a.G = c->G; a.Ipad = c->Ipad; a.I = c->I; a.J = c->J; a.JW = c->JW;
    a.q = q; a.p = p; a.S = 1; a.per_chunk = 1;
    a.part = nullptr; a.XtX = nullptr; a.Xtz = nullptr;
    a.slots = c->slots;
    a.img = c->img;
    a.pf = nullptr;
    a.budget = c->wait_budget;
    return a;
}

// The FP32 passes that stage p per CTA read this FP32 copy of it.
int stage_pf(hx_ctx* c, const double* p, PassArgs& a) {
    HX_LAUNCH(HX_KIND_OTHER, 1, launch_d2f(p, (int64_t)c->K * 4 * c->J, c->pf, c->st));
    a.pf = c->pf;
    return HX_OK;
}

int pass_q(hx_ctx* c, const double* q, const double* p, bool hess, double* XtX, double* Xtz) {
    PassArgs a = pass_args(c, q, p);
    // the gradient-only (EM) Q pass is as fast on the CUDA cores (measured
    // again after the pipeline changes: 6.91 vs 6.90 s of Q passes per C3 fit)
    if (c->tc && hess) {
        a.S = c->S_qt; a.per_chunk = c->wpc_qt; a.part = c->part_q;
        HX_LAUNCH(HX_KIND_ACCUM_Q, 2, launch_accum_q_tc(c->K, hess, a, c->st));
        HX_LAUNCH(HX_KIND_OTHER, 1, launch_reduce_sym(c->part_q, c->S_qt, c->K, hess, c->I, c->Ipad, XtX, Xtz, c->st));
        return HX_OK;
    }
    a.S = c->S_q; a.per_chunk = c->wpc_q; a.part = c->part_q;
    if (c->prec != HX_PREC_FP64) HX_ST(stage_pf(c, p, a));
    HX_LAUNCH(hess ? HX_KIND_ACCUM_Q : HX_KIND_EM_Q, 1,
              c->prec == HX_PREC_FP64 ? launch_accum_q_f64(c->K, hess, a, c->st)
                                      : launch_accum_q_f32(c->K, hess, a, c->st));
    HX_LAUNCH(HX_KIND_OTHER, 1, launch_reduce_sym(c->part_q, c->S_q, c->K, hess, c->I, c->Ipad, XtX, Xtz, c->st));
    return HX_OK;
}

int pass_p(hx_ctx* c, const double* q, const double* p, bool hess, double* XtX, double* Xtz) {
    PassArgs a = pass_args(c, q, p);
    if (c->tc) {
        a.S = c->S_pt; a.per_chunk = c->ipc_pt; a.part = c->part_p; a.XtX = XtX; a.Xtz = Xtz;
        HX_LAUNCH(hess ? HX_KIND_ACCUM_P : HX_KIND_EM_P, 2, launch_accum_p_tc(c->K, hess, a, c->st));
        if (c->S_pt > 1)
            HX_LAUNCH(HX_KIND_OTHER, 1,
                      launch_reduce_sym(c->part_p, c->S_pt, c->K, hess, 4 * c->J, 4 * c->J, XtX, Xtz, c->st));
        return HX_OK;
    }
    a.S = c->S_p; a.per_chunk = c->ipc_p; a.part = c->part_p; a.XtX = XtX; a.Xtz = Xtz;
    HX_LAUNCH(hess ? HX_KIND_ACCUM_P : HX_KIND_EM_P, 1,
              c->prec == HX_PREC_FP64 ? launch_accum_p_f64(c->K, hess, a, c->st)
                                      : launch_accum_p_f32(c->K, hess, a, c->st));
    if (c->S_p > 1)
        HX_LAUNCH(HX_KIND_OTHER, 1,
                  launch_reduce_sym(c->part_p, c->S_p, c->K, hess, 4 * c->J, 4 * c->J, XtX, Xtz, c->st));
    return HX_OK;
}

int loglik_to_slot(hx_ctx* c, const double* q, const double* p, int slot) {
    PassArgs a = pass_args(c, q, p);
    a.S = c->S_q; a.per_chunk = c->wpc_q; a.part = c->part_ll;
    if (c->prec == HX_PREC_FP64) {
        HX_LAUNCH(HX_KIND_LOGLIK, 1, launch_loglik_f64(c->K, a, c->st));
        HX_LAUNCH(HX_KIND_OTHER, 1,
                  launch_reduce_sum(c->part_ll, (c->Ipad / ACC_THREADS) * c->S_q, c->slots + slot, c->st));
    } else {
        a.S = c->S_ll; a.per_chunk = c->wpc_ll;
        HX_ST(stage_pf(c, p, a));
        HX_LAUNCH(HX_KIND_LOGLIK, 1, launch_loglik_f32x2(c->K, a, c->st));
        HX_LAUNCH(HX_KIND_OTHER, 1,
                  launch_reduce_sum(c->part_ll, (int64_t)loglik_f32x2_blocks(c->Ipad, c->K) * c->S_ll, c->slots + slot,
                                    c->st));
    }
    return HX_OK;
}

int read_slots(hx_ctx* c) {
    HX_CK(cudaMemcpyAsync(c->h_slots, c->slots, HX_NSLOT * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    HX_CK(cudaStreamSynchronize(c->st));
    prof_resolve(c);
    return HX_OK;
}
int write_slot(hx_ctx* c, int slot, double v) {
    HX_CK(cudaStreamSynchronize(c->st));
    c->h_slots[slot] = v;
    HX_CK(cudaMemcpyAsync(c->slots + slot, c->h_slots + slot, sizeof(double), cudaMemcpyHostToDevice, c->st));
    HX_CK(cudaStreamSynchronize(c->st));
    return HX_OK;
}

// After a call's work: HX_ETIMEOUT if a tensor-core pipeline wait ran out
// since the last check.  The slot is cleared, so the context stays usable (the
// kernel that timed out drained its copies and MMAs before it exited).
int take_timeout(hx_ctx* c) {
    HX_ST(read_slots(c));
    if (c->h_slots[S_TC_TIMEOUT] == 0.0) return HX_OK;
    HX_ST(write_slot(c, S_TC_TIMEOUT, 0.0));
    return fail(c, HX_ETIMEOUT, "tensor-core pass wait timed out");
}

// em! (src/algorithms_inner.jl:29-84): x -> x_next.  With fix_q / fix_p the
// fixed factor is copied unchanged (the reference rescales a fixed q before
// projecting it and rebinds p_next to p, :45-52; the intended "keep" is used).
int em_step(hx_ctx* c) {
    const size_t nq = (size_t)c->K * c->I * sizeof(double), np = (size_t)c->K * 4 * c->J * sizeof(double);
    if (!c->lo.fix_q) {
        HX_ST(pass_q(c, qof(c->x), pof(c, c->x), false, c->XtXq, c->Xtzq));
        HX_LAUNCH(HX_KIND_OTHER, 1,
                  launch_em_q(qof(c->x), c->Xtzq, c->dm, c->J, c->K, c->I, c->eps, qof(c->xn), c->st));
    } else {
        HX_CK(cudaMemcpyAsync(qof(c->xn), qof(c->x), nq, cudaMemcpyDeviceToDevice, c->st));
    }
    if (!c->lo.fix_p) {
        HX_ST(pass_p(c, qof(c->x), pof(c, c->x), false, c->XtXp, c->Xtzp));
        HX_LAUNCH(HX_KIND_OTHER, 1, launch_em_p(pof(c, c->x), c->Xtzp, c->K, c->J, c->eps, pof(c, c->xn), c->st));
    } else {
        HX_CK(cudaMemcpyAsync(pof(c, c->xn), pof(c, c->x), np, cudaMemcpyDeviceToDevice, c->st));
    }
    return HX_OK;
}

// Step control of update_q!/update_p! with guarantee_increase
// (src/algorithms_inner.jl:169-199, 313-343): x_next = project(x + f d) for
// f = 1, 1/2, ..., accepted once ll(x_next) >= ll_tmp (Q) or > ll_tmp (P);
// below f = 1e-3 the loop stops and keeps the last trial.
template <class STEP>
int step_control(hx_ctx* c, const double* q_eval, const double* p_eval, bool strict, STEP&& step) {
    double factor = 1.0;
    for (;;) {
        HX_ST(step(factor));
        HX_ST(loglik_to_slot(c, q_eval, p_eval, S_TMP));
        HX_ST(read_slots(c));
        const double ll_new = c->h_slots[S_TMP];
        if (strict ? ll_new > c->ll_tmp : ll_new >= c->ll_tmp) {
            c->ll_tmp = ll_new;
            return HX_OK;
        }
        factor /= 2.0;
        if (factor < 1e-3) factor = 0.0;
        if (factor == 0.0) return HX_OK;
    }
}

// update_q! (src/algorithms_inner.jl:97-211): equality form by default,
// penalty form (rho 1 1' on each block, no equality) with penalty = 1.
int update_q(hx_ctx* c, bool update2) {
    double* q = update2 ? qof(c->xn) : qof(c->x);
    double* p = update2 ? pof(c, c->xn) : pof(c, c->x);
    double* out = update2 ? qof(c->xn2) : qof(c->xn);
    if (c->lo.fix_q) {
        HX_CK(cudaMemcpyAsync(out, q, (size_t)c->K * c->I * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
        return HX_OK;
    }
    HX_ST(pass_q(c, q, p, true, c->XtXq, c->Xtzq));
    HX_LAUNCH(HX_KIND_OTHER, 1, launch_nan_check(c->XtXq, (int64_t)c->K * c->K * c->I, c->slots, c->st));
    HX_LAUNCH(HX_KIND_OTHER, 1, launch_nan_check(c->Xtzq, (int64_t)c->K * c->I, c->slots, c->st));
    HX_LAUNCH(HX_KIND_QP_Q, 1, launch_qp_q(c->K, c->I, c->XtXq, c->Xtzq, q, qof(c->xt), c->slots, c->st,
                                           c->lo.penalty == 1 ? c->rho : -1.0));
    auto step = [&](double f) {
        HX_LAUNCH(HX_KIND_OTHER, 1, launch_step_q(q, qof(c->xt), c->K, c->I, c->eps, out, c->st, f));
        return HX_OK;
    };
    if (!c->lo.guarantee_increase) return step(1.0);
    return step_control(c, out, p, false, step);
}

// update_p! (src/algorithms_inner.jl:224-355): penalty branch by default, the
// equality branch (K equalities per block, :307-310) with penalty = 0.
int update_p(hx_ctx* c, bool update2) {
    double* q = update2 ? qof(c->xn2) : qof(c->xn);
    double* p = update2 ? pof(c, c->xn) : pof(c, c->x);
    double* out = update2 ? pof(c, c->xn2) : pof(c, c->xn);
    if (c->lo.fix_p) {
        HX_CK(cudaMemcpyAsync(out, p, (size_t)c->K * 4 * c->J * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
        return HX_OK;
    }
    HX_ST(pass_p(c, q, p, true, c->XtXp, c->Xtzp));
    HX_LAUNCH(HX_KIND_QP_P, 1,
              launch_qp_p(c->K, c->J, c->XtXp, c->Xtzp, p, c->rho, pof(c, c->xt), c->slots, c->qp_ws, c->st,
                          c->lo.penalty == 0));
    auto step = [&](double f) {
        HX_LAUNCH(HX_KIND_OTHER, 1, launch_step_p(p, pof(c, c->xt), c->K, c->J, c->eps, out, c->st, f));
        return HX_OK;
    };
    if (!c->lo.guarantee_increase) return step(1.0);
    return step_control(c, q, out, true, step);
}

// One outer iteration of admixture_qn! (src/algorithms_outer.jl:65-171).
int qn_iteration(hx_ctx* c) {
    if (c->lo.guarantee_increase) {   // d.ll_tmp = d.ll_new (:69-70)
        HX_ST(read_slots(c));
        c->ll_tmp = c->h_slots[S_LL_NEW];
    }
    HX_LAUNCH(HX_KIND_OTHER, 1, launch_iter_begin(c->slots, c->st));
    HX_ST(update_q(c, false));
    HX_ST(update_p(c, false));
    HX_ST(update_q(c, true));
    HX_ST(update_p(c, true));
    HX_ST(loglik_to_slot(c, qof(c->xn2), pof(c, c->xn2), S_LL_BASIC));
    HX_LAUNCH(HX_KIND_QN, 3,
              launch_qn(c->nx, c->x, c->xn, c->xn2, c->U, c->V, c->Qs, c->part_qn, c->coef, c->xt, c->slots, c->st,
                        c->lo.mode));
    HX_LAUNCH(HX_KIND_OTHER, 1, launch_step_p(pof(c, c->xt), nullptr, c->K, c->J, c->eps, pof(c, c->xt), c->st));
    HX_LAUNCH(HX_KIND_OTHER, 1, launch_step_q(qof(c->xt), nullptr, c->K, c->I, c->eps, qof(c->xt), c->st));
    HX_ST(loglik_to_slot(c, qof(c->xt), pof(c, c->xt), S_LL_QN));
    HX_LAUNCH(HX_KIND_OTHER, 1, launch_accept(c->nx, c->x, c->xt, c->xn2, c->slots, c->st));
    return HX_OK;
}

int check_qp(hx_ctx* c) {
    if (!c) return HX_EINVAL;
    if (!c->have_qp) return fail(c, HX_ESTATE, "Q/P not set (call hx_set_qp first)");
    return HX_OK;
}

template <class T>
int dalloc(hx_ctx* c, T** p, size_t n) {
    cudaError_t e = cudaMalloc((void**)p, std::max<size_t>(n, 1) * sizeof(T));
    if (e != cudaSuccess) return cuda_fail(c, "cudaMalloc", e);
    return HX_OK;
}

int create_common(const uint8_t* bed, bool bed_on_device, int64_t bps, int64_t nsnp, int64_t I, int64_t J,
                  int32_t K, const hx_opts* opts, hx_ctx** out, const hx_ctx* parent = nullptr) {
    if (!out) return HX_EINVAL;
    *out = nullptr;
    hx_opts o;
    hx_opts_default(&o);
    if (opts) o = *opts;
    if (parent && o.device != parent->device) return HX_EINVAL;
    if ((!bed && !parent) || I <= 0 || J <= 0 || bps < (I + 3) / 4 || nsnp < 2 * J) return HX_EINVAL;
    if (K < 1 || K > HX_KMAX || o.Qsec < 1 || o.Qsec > HX_QMAX) return HX_EUNSUPPORTED;
    if (o.precision != HX_PREC_FP64 && o.precision != HX_PREC_MIXED) return HX_EINVAL;
    hx_ctx* c = new hx_ctx();
    *out = c;
    c->device = o.device; c->prec = o.precision; c->Qs = o.Qsec; c->verbose = o.verbose;
    c->rho = o.rho; c->eps = o.pseudocount;
    c->tc = (o.precision == HX_PREC_MIXED) && (o.path == HX_PATH_AUTO);
    c->I = I; c->J = J; c->K = K; c->nsnp = nsnp; c->bps = bps;
    c->Ipad = (I + HX_IPAD - 1) / HX_IPAD * HX_IPAD;
    c->JW = (int)((J + 7) / 8);
    c->nx = (int64_t)K * (I + 4 * J);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= c->device || c->device < 0)
        return fail(c, HX_ECUDA, "no usable CUDA device");
    HX_CK(cudaSetDevice(c->device));
    HX_CK(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
    HX_CK(cudaEventCreate(&c->ev0));
    HX_CK(cudaEventCreate(&c->ev1));
    HX_CK(init_kernel_attrs());
    HX_CK(init_tc_attrs());
    plan(c);
    if (c->verbose)
        fprintf(stderr,
                "{\"plan\": {\"chunks_q\": %d, \"chunks_p\": %d, \"chunks_q_tc\": %d, \"chunks_p_tc\": %d, "
                "\"chunks_loglik\": %d, \"resident_q_tc\": %d, \"resident_p_tc\": %d, \"resident_loglik\": %d}}\n",
                c->S_q, c->S_p, c->S_qt, c->S_pt, c->S_ll, tc_resident(K, false), tc_resident(K, true),
                loglik_f32x2_resident(K));
    const int NVmax = K + K * (K + 1) / 2;
    if (parent) {
        c->G = parent->G;
        c->dm = parent->dm;
        c->shared_geno = true;
    } else {
        HX_ST(dalloc(c, &c->G, (size_t)c->JW * c->Ipad));
        HX_ST(dalloc(c, &c->dm, (size_t)I));
    }
    for (double** b : {&c->x, &c->xn, &c->xn2, &c->xt, &c->xio}) HX_ST(dalloc(c, b, (size_t)c->nx));
    HX_ST(dalloc(c, &c->U, (size_t)c->nx * c->Qs));
    HX_ST(dalloc(c, &c->V, (size_t)c->nx * c->Qs));
    HX_ST(dalloc(c, &c->XtXq, (size_t)K * K * I));
    HX_ST(dalloc(c, &c->Xtzq, (size_t)K * I));
    HX_ST(dalloc(c, &c->XtXp, (size_t)K * K * 4 * J));
    HX_ST(dalloc(c, &c->Xtzp, (size_t)K * 4 * J));
    HX_ST(dalloc(c, &c->part_q, (size_t)std::max(c->S_q, c->tc ? c->Sq_cap : 1) * NVmax * c->Ipad));
    const int Sp_max = std::max(c->S_p, c->tc ? c->Sp_cap : 1);
    if (Sp_max > 1) HX_ST(dalloc(c, &c->part_p, (size_t)Sp_max * NVmax * 4 * J));
    HX_ST(dalloc(c, &c->part_ll, (size_t)std::max<int64_t>((c->Ipad / ACC_THREADS) * c->S_q,
                                                            (int64_t)loglik_f32x2_blocks(c->Ipad, K) *
                                                                std::max(c->S_ll, c->Sll_cap))));
    HX_ST(dalloc(c, &c->part_qn, (size_t)qn_dots_blocks(c->nx) * (2 * HX_QMAX * HX_QMAX + HX_QMAX)));
    HX_ST(dalloc(c, &c->coef, HX_QMAX));
    HX_ST(dalloc(c, &c->slots, HX_NSLOT));
    if (c->tc) HX_ST(dalloc(c, &c->img, tc_image_bytes(K, I, J)));
    if (c->prec != HX_PREC_FP64) HX_ST(dalloc(c, &c->pf, (size_t)K * 4 * J));
    HX_ST(dalloc(c, &c->qp_ws, (size_t)4 * K * J));
    HX_CK(cudaMemsetAsync(c->qp_ws, 0, (size_t)4 * K * J, c->st));
    HX_CK(cudaMallocHost((void**)&c->h_slots, HX_NSLOT * sizeof(double)));
    HX_CK(cudaMemsetAsync(c->U, 0, (size_t)c->nx * c->Qs * sizeof(double), c->st));
    HX_CK(cudaMemsetAsync(c->V, 0, (size_t)c->nx * c->Qs * sizeof(double), c->st));
    for (int s = 0; s < HX_NSLOT; ++s) c->h_slots[s] = 0.0;
    c->h_slots[S_LL_NEW] = NAN;
    HX_CK(cudaMemcpyAsync(c->slots, c->h_slots, HX_NSLOT * sizeof(double), cudaMemcpyHostToDevice, c->st));
    if (parent) {
        HX_CK(cudaStreamSynchronize(c->st));
        return HX_OK;
    }
    HX_CK(cudaMemsetAsync(c->dm, 0, (size_t)I * sizeof(unsigned long long), c->st));
    // stage the BED matrix (first 2J SNPs used by the fit; all n_snp SNPs for
    // the double-missing count, as count_double_missing! reads the whole file)
    const uint8_t* dbed = bed;
    uint8_t* tmp = nullptr;
    if (!bed_on_device) {
        HX_ST(dalloc(c, &tmp, (size_t)bps * nsnp));
        HX_CK(cudaMemcpyAsync(tmp, bed, (size_t)bps * nsnp, cudaMemcpyHostToDevice, c->st));
        dbed = tmp;
    }
    HX_CK(launch_pack(dbed, bps, I, J, c->Ipad, c->JW, c->G, c->st));
    HX_CK(launch_double_missing(dbed, bps, I, nsnp, c->dm, c->st));
    HX_CK(cudaStreamSynchronize(c->st));
    if (tmp) HX_CK(cudaFree(tmp));
    return HX_OK;
}

int upload_x(hx_ctx* c, const double* q, const double* p, bool device, double* dst) {
    const cudaMemcpyKind kind = device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (q) HX_CK(cudaMemcpyAsync(qof(dst), q, (size_t)c->K * c->I * sizeof(double), kind, c->st));
    if (p) HX_CK(cudaMemcpyAsync(pof(c, dst), p, (size_t)c->K * 4 * c->J * sizeof(double), kind, c->st));
    return HX_OK;
}

int reset_state(hx_ctx* c) {
    // a new trajectory starts from cold QP working sets, so that a fit from
    // given Q, P is reproducible regardless of earlier calls
    HX_CK(cudaMemsetAsync(c->qp_ws, 0, (size_t)4 * c->K * c->J, c->st));
    HX_CK(cudaMemsetAsync(c->U, 0, (size_t)c->nx * c->Qs * sizeof(double), c->st));
    HX_CK(cudaMemsetAsync(c->V, 0, (size_t)c->nx * c->Qs * sizeof(double), c->st));
    HX_CK(cudaStreamSynchronize(c->st));
    for (int s = 0; s < HX_NSLOT; ++s) c->h_slots[s] = 0.0;
    c->h_slots[S_LL_NEW] = NAN;
    HX_CK(cudaMemcpyAsync(c->slots, c->h_slots, HX_NSLOT * sizeof(double), cudaMemcpyHostToDevice, c->st));
    HX_CK(cudaStreamSynchronize(c->st));
    return HX_OK;
}

struct Tmp {  // temporary device buffers of the host-array entry points
    std::vector<void*> ptrs;
    ~Tmp() { for (void* p : ptrs) cudaFree(p); }
    template <class T> T* get(hx_ctx* c, size_t n, int* st) {
        T* p = nullptr;
        cudaError_t e = cudaMalloc((void**)&p, std::max<size_t>(n, 1) * sizeof(T));
        if (e != cudaSuccess) { *st = cuda_fail(c, "cudaMalloc", e); return nullptr; }
        ptrs.push_back(p);
        return p;
    }
};

}  // namespace

// ====================================================================== C ABI
extern "C" {

int hx_loop_opts_default(hx_loop_opts* o) {
    if (!o) return HX_EINVAL;
    o->fix_q = 0;
    o->fix_p = 0;
    o->guarantee_increase = 0;
    o->penalty = -1;
    o->mode = 0;
    return HX_OK;
}

int hx_set_loop_opts(hx_ctx* c, const hx_loop_opts* o) {
    if (!c || !o) return HX_EINVAL;
    if (o->penalty < -1 || o->penalty > 1) return fail(c, HX_EINVAL, "penalty must be -1, 0 or 1");
    if (o->mode < 0 || o->mode > 1) return fail(c, HX_EINVAL, "mode must be 0 (ZAL) or 1 (LBQN)");
    c->lo = *o;
    return HX_OK;
}

int hx_opts_default(hx_opts* o) {
    if (!o) return HX_EINVAL;
    o->precision = HX_PREC_FP64;
    o->device = 0;
    o->Qsec = 3;
    o->verbose = 0;
    o->rho = 1e7;
    o->pseudocount = 1e-5;
    o->path = HX_PATH_AUTO;
    o->reserved = 0;
    return HX_OK;
}

const char* hx_status_string(int s) {
    switch (s) {
        case HX_OK: return "ok";
        case HX_EINVAL: return "invalid argument";
        case HX_ECUDA: return "CUDA error";
        case HX_ENAN: return "NaN in gradient or Hessian";
        case HX_ETIMEOUT: return "iteration cap reached, or a device pipeline wait timed out";
        case HX_ENOMEM: return "device out of memory";
        case HX_ESTATE: return "call out of order";
        case HX_EUNSUPPORTED: return "unsupported size";
        default: return "unknown status";
    }
}

const char* hx_last_error(const hx_ctx* c) { return c ? c->err.c_str() : "null context"; }

int hx_create(const uint8_t* bed, int64_t bps, int64_t nsnp, int64_t I, int64_t J, int32_t K, const hx_opts* opts,
              hx_ctx** out) {
    return create_common(bed, false, bps, nsnp, I, J, K, opts, out);
}
int hx_create_device(const uint8_t* d_bed, int64_t bps, int64_t nsnp, int64_t I, int64_t J, int32_t K,
                     const hx_opts* opts, hx_ctx** out) {
    return create_common(d_bed, true, bps, nsnp, I, J, K, opts, out);
}

int hx_destroy(hx_ctx* c) {
    if (!c) return HX_OK;
    if (c->st) cudaStreamSynchronize(c->st);
    void* bufs[] = {c->shared_geno ? nullptr : (void*)c->G, c->shared_geno ? nullptr : (void*)c->dm, c->x, c->xn, c->xn2, c->xt, c->xio, c->U, c->V, c->XtXq, c->Xtzq, c->XtXp,
                    c->Xtzp, c->part_q, c->part_p, c->part_ll, c->part_qn, c->coef, c->slots, c->img, c->qp_ws,
                    c->pf};
    for (void* b : bufs) if (b) cudaFree(b);
    prof_resolve(c);
    for (cudaEvent_t e : c->pool) cudaEventDestroy(e);
    if (c->h_slots) cudaFreeHost(c->h_slots);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->st) cudaStreamDestroy(c->st);
    delete c;
    return HX_OK;
}

int hx_dims(const hx_ctx* c, int64_t* I, int64_t* J, int32_t* K) {
    if (!c) return HX_EINVAL;
    if (I) *I = c->I;
    if (J) *J = c->J;
    if (K) *K = c->K;
    return HX_OK;
}

int hx_set_qp(hx_ctx* c, const double* q, const double* p) {
    if (!c || (!q && !p)) return HX_EINVAL;
    if ((!q || !p) && !c->have_qp) return fail(c, HX_ESTATE, "first hx_set_qp needs both q and p");
    HX_CK(cudaSetDevice(c->device));
    HX_ST(upload_x(c, q, p, false, c->x));
    HX_ST(reset_state(c));
    c->have_qp = true;
    return HX_OK;
}
int hx_set_qp_device(hx_ctx* c, const double* q, const double* p) {
    if (!c || (!q && !p)) return HX_EINVAL;
    if ((!q || !p) && !c->have_qp) return fail(c, HX_ESTATE, "first hx_set_qp needs both q and p");
    HX_CK(cudaSetDevice(c->device));
    HX_ST(upload_x(c, q, p, true, c->x));
    HX_ST(reset_state(c));
    c->have_qp = true;
    return HX_OK;
}

int hx_get_qp(hx_ctx* c, int32_t which, double* q, double* p) {
    HX_ST(check_qp(c));
    double* src = which == 0 ? c->x : which == 1 ? c->xn : which == 2 ? c->xn2 : which == 3 ? c->xt : nullptr;
    if (!src) return HX_EINVAL;
    if (q) HX_CK(cudaMemcpyAsync(q, qof(src), (size_t)c->K * c->I * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    if (p)
        HX_CK(cudaMemcpyAsync(p, pof(c, src), (size_t)c->K * 4 * c->J * sizeof(double), cudaMemcpyDeviceToHost,
                              c->st));
    HX_CK(cudaStreamSynchronize(c->st));
    return HX_OK;
}

int hx_get_ll(hx_ctx* c, double* ll) {
    if (!c || !ll) return HX_EINVAL;
    HX_ST(read_slots(c));
    *ll = c->h_slots[S_LL_NEW];
    return HX_OK;
}

int hx_census(hx_ctx* c, uint64_t counts[16]) {
    if (!c || !counts) return HX_EINVAL;
    int st = HX_OK;
    Tmp t;
    unsigned long long* d = t.get<unsigned long long>(c, 16, &st);
    if (!d) return st;
    HX_CK(cudaMemsetAsync(d, 0, 16 * sizeof(unsigned long long), c->st));
    HX_CK(launch_census(c->G, c->Ipad, c->I, c->J, c->JW, d, c->st));
    HX_CK(cudaMemcpyAsync(counts, d, 16 * sizeof(uint64_t), cudaMemcpyDeviceToHost, c->st));
    HX_CK(cudaStreamSynchronize(c->st));
    return HX_OK;
}

int hx_double_missing(hx_ctx* c, int64_t* dm) {
    if (!c || !dm) return HX_EINVAL;
    HX_CK(cudaMemcpyAsync(dm, c->dm, (size_t)c->I * sizeof(int64_t), cudaMemcpyDeviceToHost, c->st));
    HX_CK(cudaStreamSynchronize(c->st));
    return HX_OK;
}

int hx_loglikelihood(hx_ctx* c, const double* q, const double* p, double* ll) {
    if (!c || !ll) return HX_EINVAL;
    const double* dq;
    const double* dp;
    if (q || p) {
        if (!q || !p) return HX_EINVAL;
        HX_ST(upload_x(c, q, p, false, c->xio));
        dq = qof(c->xio);
        dp = pof(c, c->xio);
    } else {
        HX_ST(check_qp(c));
        dq = qof(c->x);
        dp = pof(c, c->x);
    }
    HX_ST(loglik_to_slot(c, dq, dp, S_TMP));
    HX_ST(read_slots(c));
    *ll = c->h_slots[S_TMP];
    return HX_OK;
}

int hx_em_accum(hx_ctx* c, const double* q, const double* p, double* q_next, double* p_next) {
    if (!c || !q || !p) return HX_EINVAL;
    HX_ST(upload_x(c, q, p, false, c->xio));
    HX_ST(pass_q(c, qof(c->xio), pof(c, c->xio), false, c->XtXq, c->Xtzq));
    HX_ST(pass_p(c, qof(c->xio), pof(c, c->xio), false, c->XtXp, c->Xtzp));
    HX_ST(take_timeout(c));
    // numerators q .* Xtz_q and p .* Xtz_p, formed on the host from the copies
    std::vector<double> g((size_t)c->K * std::max<int64_t>(c->I, 4 * c->J));
    if (q_next) {
        HX_CK(cudaMemcpy(g.data(), c->Xtzq, (size_t)c->K * c->I * sizeof(double), cudaMemcpyDeviceToHost));
        for (int64_t a = 0; a < (int64_t)c->K * c->I; ++a) q_next[a] = q[a] * g[a];
    }
    if (p_next) {
        HX_CK(cudaMemcpy(g.data(), c->Xtzp, (size_t)c->K * 4 * c->J * sizeof(double), cudaMemcpyDeviceToHost));
        for (int64_t a = 0; a < (int64_t)c->K * 4 * c->J; ++a) p_next[a] = p[a] * g[a];
    }
    return HX_OK;
}

int hx_update_q_accum(hx_ctx* c, const double* q, const double* p, double* XtX, double* Xtz) {
    if (!c || !q || !p) return HX_EINVAL;
    HX_ST(upload_x(c, q, p, false, c->xio));
    HX_ST(pass_q(c, qof(c->xio), pof(c, c->xio), true, c->XtXq, c->Xtzq));
    if (XtX) HX_CK(cudaMemcpyAsync(XtX, c->XtXq, (size_t)c->K * c->K * c->I * sizeof(double),
                                   cudaMemcpyDeviceToHost, c->st));
    if (Xtz) HX_CK(cudaMemcpyAsync(Xtz, c->Xtzq, (size_t)c->K * c->I * sizeof(double), cudaMemcpyDeviceToHost,
                                   c->st));
    HX_CK(cudaStreamSynchronize(c->st));
    return take_timeout(c);
}

int hx_update_p_accum(hx_ctx* c, const double* q, const double* p, double* XtX, double* Xtz) {
    if (!c || !q || !p) return HX_EINVAL;
    HX_ST(upload_x(c, q, p, false, c->xio));
    HX_ST(pass_p(c, qof(c->xio), pof(c, c->xio), true, c->XtXp, c->Xtzp));
    if (XtX) HX_CK(cudaMemcpyAsync(XtX, c->XtXp, (size_t)c->K * c->K * 4 * c->J * sizeof(double),
                                   cudaMemcpyDeviceToHost, c->st));
    if (Xtz) HX_CK(cudaMemcpyAsync(Xtz, c->Xtzp, (size_t)c->K * 4 * c->J * sizeof(double),
                                   cudaMemcpyDeviceToHost, c->st));
    HX_CK(cudaStreamSynchronize(c->st));
    return take_timeout(c);
}

// em_p!(d_cu, g_cu) (src/cuda/runners.jl:51-55; kernels.jl:75-102): the P
// part of the EM numerators only, p_next[k,m] = p[k,m] Xtz_p[k,m].
int hx_em_p_accum(hx_ctx* c, const double* q, const double* p, double* p_next) {
    if (!c || !q || !p || !p_next) return HX_EINVAL;
    HX_ST(upload_x(c, q, p, false, c->xio));
    HX_ST(pass_p(c, qof(c->xio), pof(c, c->xio), false, c->XtXp, c->Xtzp));
    HX_ST(take_timeout(c));
    std::vector<double> g((size_t)c->K * 4 * c->J);
    HX_CK(cudaMemcpy(g.data(), c->Xtzp, g.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (size_t a = 0; a < g.size(); ++a) p_next[a] = p[a] * g[a];
    return HX_OK;
}

int hx_set_wait_budget(hx_ctx* c, int64_t cycles) {
    if (!c) return HX_EINVAL;
    c->wait_budget = cycles > 0 ? (long long)cycles : (long long)HX_WAIT_BUDGET_DEFAULT;
    return HX_OK;
}

int hx_qp_q(hx_ctx* c, int64_t n, const double* XtX, const double* Xtz, const double* q, double* qdiff) {
    if (!c || n <= 0 || !XtX || !Xtz || !q || !qdiff) return HX_EINVAL;
    const int K = c->K;
    int st = HX_OK;
    Tmp t;
    double* dX = t.get<double>(c, (size_t)K * K * n, &st);
    double* dz = t.get<double>(c, (size_t)K * n, &st);
    double* dq = t.get<double>(c, (size_t)K * n, &st);
    double* dd = t.get<double>(c, (size_t)K * n, &st);
    if (st != HX_OK) return st;
    HX_CK(cudaMemcpyAsync(dX, XtX, (size_t)K * K * n * 8, cudaMemcpyHostToDevice, c->st));
    HX_CK(cudaMemcpyAsync(dz, Xtz, (size_t)K * n * 8, cudaMemcpyHostToDevice, c->st));
    HX_CK(cudaMemcpyAsync(dq, q, (size_t)K * n * 8, cudaMemcpyHostToDevice, c->st));
    HX_CK(launch_qp_q(K, n, dX, dz, dq, dd, c->slots, c->st, c->lo.penalty == 1 ? c->rho : -1.0));
    HX_CK(cudaMemcpyAsync(qdiff, dd, (size_t)K * n * 8, cudaMemcpyDeviceToHost, c->st));
    HX_CK(cudaStreamSynchronize(c->st));
    return HX_OK;
}

int hx_qp_p(hx_ctx* c, int64_t n, const double* XtX, const double* Xtz, const double* p, double* pdiff) {
    if (!c || n <= 0 || !XtX || !Xtz || !p || !pdiff) return HX_EINVAL;
    const int K = c->K;
    int st = HX_OK;
    Tmp t;
    double* dX = t.get<double>(c, (size_t)K * K * 4 * n, &st);
    double* dz = t.get<double>(c, (size_t)K * 4 * n, &st);
    double* dp = t.get<double>(c, (size_t)K * 4 * n, &st);
    double* dd = t.get<double>(c, (size_t)K * 4 * n, &st);
    if (st != HX_OK) return st;
    HX_CK(cudaMemcpyAsync(dX, XtX, (size_t)K * K * 4 * n * 8, cudaMemcpyHostToDevice, c->st));
    HX_CK(cudaMemcpyAsync(dz, Xtz, (size_t)K * 4 * n * 8, cudaMemcpyHostToDevice, c->st));
    HX_CK(cudaMemcpyAsync(dp, p, (size_t)K * 4 * n * 8, cudaMemcpyHostToDevice, c->st));
    HX_CK(launch_qp_p(K, n, dX, dz, dp, c->rho, dd, c->slots, nullptr, c->st, c->lo.penalty == 0));
    HX_CK(cudaMemcpyAsync(pdiff, dd, (size_t)K * 4 * n * 8, cudaMemcpyDeviceToHost, c->st));
    HX_CK(cudaStreamSynchronize(c->st));
    return HX_OK;
}

int hx_project_q(hx_ctx* c, int64_t ncol, double* q) {
    if (!c || ncol <= 0 || !q) return HX_EINVAL;
    int st = HX_OK;
    Tmp t;
    double* d = t.get<double>(c, (size_t)c->K * ncol, &st);
    if (!d) return st;
    HX_CK(cudaMemcpyAsync(d, q, (size_t)c->K * ncol * 8, cudaMemcpyHostToDevice, c->st));
    HX_CK(launch_step_q(d, nullptr, c->K, ncol, c->eps, d, c->st));
    HX_CK(cudaMemcpyAsync(q, d, (size_t)c->K * ncol * 8, cudaMemcpyDeviceToHost, c->st));
    HX_CK(cudaStreamSynchronize(c->st));
    return HX_OK;
}

int hx_project_p(hx_ctx* c, int64_t nb, double* p) {
    if (!c || nb <= 0 || !p) return HX_EINVAL;
    int st = HX_OK;
    Tmp t;
    double* d = t.get<double>(c, (size_t)c->K * 4 * nb, &st);
    if (!d) return st;
    HX_CK(cudaMemcpyAsync(d, p, (size_t)c->K * 4 * nb * 8, cudaMemcpyHostToDevice, c->st));
    HX_CK(launch_step_p(d, nullptr, c->K, nb, c->eps, d, c->st));
    HX_CK(cudaMemcpyAsync(p, d, (size_t)c->K * 4 * nb * 8, cudaMemcpyDeviceToHost, c->st));
    HX_CK(cudaStreamSynchronize(c->st));
    return HX_OK;
}

int hx_zal(hx_ctx* c, const double* x, const double* x_next, const double* x_next2, double* U, double* V,
           int32_t iter, double* x_tmp) {
    if (!c || !x || !x_next || !x_next2 || !U || !V || !x_tmp || iter < 1) return HX_EINVAL;
    const int64_t n = c->nx;
    const int Qs = c->Qs;
    int st = HX_OK;
    Tmp t;
    double* dx = t.get<double>(c, n, &st);
    double* dxn = t.get<double>(c, n, &st);
    double* dxn2 = t.get<double>(c, n, &st);
    double* dU = t.get<double>(c, (size_t)n * Qs, &st);
    double* dV = t.get<double>(c, (size_t)n * Qs, &st);
    double* dxt = t.get<double>(c, n, &st);
    double* part = t.get<double>(c, (size_t)qn_dots_blocks(n) * (2 * HX_QMAX * HX_QMAX + HX_QMAX), &st);
    double* coef = t.get<double>(c, HX_QMAX, &st);
    double* slots = t.get<double>(c, HX_NSLOT, &st);
    if (st != HX_OK) return st;
    HX_CK(cudaMemcpyAsync(dx, x, n * 8, cudaMemcpyHostToDevice, c->st));
    HX_CK(cudaMemcpyAsync(dxn, x_next, n * 8, cudaMemcpyHostToDevice, c->st));
    HX_CK(cudaMemcpyAsync(dxn2, x_next2, n * 8, cudaMemcpyHostToDevice, c->st));
    HX_CK(cudaMemcpyAsync(dU, U, (size_t)n * Qs * 8, cudaMemcpyHostToDevice, c->st));
    HX_CK(cudaMemcpyAsync(dV, V, (size_t)n * Qs * 8, cudaMemcpyHostToDevice, c->st));
    std::vector<double> hs(HX_NSLOT, 0.0);
    hs[S_ITER] = iter;
    HX_CK(cudaMemcpyAsync(slots, hs.data(), HX_NSLOT * 8, cudaMemcpyHostToDevice, c->st));
    HX_CK(launch_qn(n, dx, dxn, dxn2, dU, dV, Qs, part, coef, dxt, slots, c->st));
    HX_CK(cudaMemcpyAsync(U, dU, (size_t)n * Qs * 8, cudaMemcpyDeviceToHost, c->st));
    HX_CK(cudaMemcpyAsync(V, dV, (size_t)n * Qs * 8, cudaMemcpyDeviceToHost, c->st));
    HX_CK(cudaMemcpyAsync(x_tmp, dxt, n * 8, cudaMemcpyDeviceToHost, c->st));
    HX_CK(cudaStreamSynchronize(c->st));
    return HX_OK;
}

int hx_em_step(hx_ctx* c) {
    HX_ST(check_qp(c));
    HX_ST(em_step(c));
    return take_timeout(c);
}

// init_em! (src/algorithms_outer.jl:1-22).  The log-likelihood of every EM
// iteration is only reported there; the last one seeds the QN loop.  So it is
// evaluated after the last iteration, and after every one only when verbose.
int hx_init_em(hx_ctx* c, int32_t iters) {
    HX_ST(check_qp(c));
    for (int e = 0; e < iters; ++e) {
        HX_ST(em_step(c));
        HX_CK(cudaMemcpyAsync(c->x, c->xn, (size_t)c->nx * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
        if (c->verbose || e + 1 == iters) HX_ST(loglik_to_slot(c, qof(c->x), pof(c, c->x), S_LL_NEW));
        HX_LAUNCH(HX_KIND_OTHER, 1, launch_step_p(pof(c, c->x), nullptr, c->K, c->J, c->eps, pof(c, c->x), c->st));
        HX_LAUNCH(HX_KIND_OTHER, 1, launch_step_q(qof(c->x), nullptr, c->K, c->I, c->eps, qof(c->x), c->st));
        if (c->verbose) {
            HX_ST(read_slots(c));
            fprintf(stderr, "{\"em_iter\": %d, \"ll\": %.17g}\n", e + 1, c->h_slots[S_LL_NEW]);
        }
    }
    return take_timeout(c);
}

int hx_update_q(hx_ctx* c, int32_t update2) {
    HX_ST(check_qp(c));
    HX_ST(update_q(c, update2 != 0));
    HX_ST(take_timeout(c));     // a pass that timed out leaves garbage sums: report the cause first
    if (c->h_slots[S_NAN] != 0.0) return fail(c, HX_ENAN, "NaN in XtX_q/Xtz_q");
    return HX_OK;
}

int hx_update_p(hx_ctx* c, int32_t update2) {
    HX_ST(check_qp(c));
    HX_ST(update_p(c, update2 != 0));
    return take_timeout(c);
}

int hx_qn_iteration(hx_ctx* c, hx_iter_info* info) {
    HX_ST(check_qp(c));
    HX_ST(read_slots(c));
    if (std::isnan(c->h_slots[S_LL_NEW])) HX_ST(loglik_to_slot(c, qof(c->x), pof(c, c->x), S_LL_NEW));
    HX_CK(cudaEventRecord(c->ev0, c->st));
    HX_ST(qn_iteration(c));
    HX_CK(cudaEventRecord(c->ev1, c->st));
    HX_ST(read_slots(c));
    float ms = 0.f;
    HX_CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    const double* s = c->h_slots;
    if (info) {
        info->iter = (int32_t)s[S_ITER];
        info->accepted_qn = s[S_ACCEPT_QN] != 0.0;
        info->ll_prev = s[S_LL_PREV];
        info->ll_basic = s[S_LL_BASIC];
        info->ll_qn = s[S_LL_QN];
        info->ll_new = s[S_LL_NEW];
        info->reldiff = s[S_RELDIFF];
        info->seconds = ms * 1e-3;
    }
    if (c->verbose)
        fprintf(stderr,
                "{\"iter\": %d, \"ll\": %.17g, \"reldiff\": %.6e, \"ll_basic\": %.17g, \"ll_qn\": %.17g, "
                "\"qn\": %d, \"ms\": %.3f}\n",
                (int)s[S_ITER], s[S_LL_NEW], s[S_RELDIFF], s[S_LL_BASIC], s[S_LL_QN], (int)s[S_ACCEPT_QN], ms);
    HX_ST(take_timeout(c));
    if (s[S_NAN] != 0.0) return fail(c, HX_ENAN, "NaN in XtX_q/Xtz_q");
    return HX_OK;
}

// admixture_qn! (src/algorithms_outer.jl:38-172), mode = :ZAL.
int hx_admixture_qn(hx_ctx* c, int32_t n_iter, double rtol, int32_t iter_offset, hx_fit_info* info) {
    HX_ST(check_qp(c));
    auto t0 = std::chrono::steady_clock::now();
    HX_ST(read_slots(c));
    if (std::isnan(c->h_slots[S_LL_NEW])) HX_ST(loglik_to_slot(c, qof(c->x), pof(c, c->x), S_LL_NEW));
    HX_ST(write_slot(c, S_ITER, (double)iter_offset));
    int run = 0;
    bool conv = false;
    for (int it = iter_offset + 1; it <= n_iter; ++it) {
        hx_iter_info ii;
        HX_ST(hx_qn_iteration(c, &ii));
        ++run;
        if (ii.reldiff < rtol) { conv = true; break; }
    }
    HX_ST(read_slots(c));
    if (info) {
        info->iters = run;
        info->converged = conv;
        info->ll = c->h_slots[S_LL_NEW];
        info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return HX_OK;
}

int hx_create_shared(const hx_ctx* parent, int32_t K, const hx_opts* opts, hx_ctx** out) {
    if (!parent || !out) return HX_EINVAL;
    hx_opts o;
    hx_opts_default(&o);
    if (opts) o = *opts;
    o.device = parent->device;
    return create_common(nullptr, true, parent->bps, parent->nsnp, parent->I, parent->J, K, &o, out, parent);
}

int hx_fit_many(hx_ctx* const* ctxs, int32_t n, int32_t n_iter, double rtol, int32_t em_iters, int32_t threads,
                hx_fit_info* infos, int32_t* status) {
    if (!ctxs || n < 0 || !infos) return HX_EINVAL;
    for (int32_t a = 0; a < n; ++a)
        if (!ctxs[a]) return HX_EINVAL;
    const int nt = std::max(1, std::min<int>(threads > 0 ? threads : n, n));
    std::atomic<int> next(0);
    std::vector<int> st(n, HX_OK);
    auto worker = [&]() {
        for (int a = next++; a < n; a = next++) {
            if (cudaSetDevice(ctxs[a]->device) != cudaSuccess) { st[a] = HX_ECUDA; continue; }
            st[a] = hx_fit(ctxs[a], n_iter, rtol, em_iters, &infos[a]);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
    int first = HX_OK;
    for (int32_t a = 0; a < n; ++a) {
        if (status) status[a] = st[a];
        if (first == HX_OK && st[a] != HX_OK) first = st[a];
    }
    return first;
}

// ------------------------------------------------------------ learned warm start
namespace {
struct LwsScratch {   // temporary device buffers of one training or gradient call
    float* part = nullptr;
    double* loss_part = nullptr;
    float* grad = nullptr;
    int64_t* idx = nullptr;
    ~LwsScratch() {
        if (part) cudaFree(part);
        if (loss_part) cudaFree(loss_part);
        if (grad) cudaFree(grad);
        if (idx) cudaFree(idx);
    }
    cudaError_t alloc(int64_t nidx) {
        cudaError_t e = cudaMalloc((void**)&part, (size_t)LWS_MAX_BLOCKS * HX_LWS_NPARAM * sizeof(float));
        if (e == cudaSuccess) e = cudaMalloc((void**)&loss_part, LWS_MAX_BLOCKS * sizeof(double));
        if (e == cudaSuccess) e = cudaMalloc((void**)&grad, HX_LWS_NPARAM * sizeof(float));
        if (e == cudaSuccess && nidx > 0) e = cudaMalloc((void**)&idx, (size_t)nidx * sizeof(int64_t));
        return e;
    }
};
int cuda_status(cudaError_t e) {
    return e == cudaSuccess ? HX_OK : (e == cudaErrorMemoryAllocation ? HX_ENOMEM : HX_ECUDA);
}
}  // namespace

int hx_lws_features(hx_ctx* c, float* d_feat) {
    HX_ST(check_qp(c));
    if (!d_feat) return HX_EINVAL;
    HX_CK(cudaSetDevice(c->device));
    HX_ST(pass_q(c, qof(c->x), pof(c, c->x), false, c->XtXq, c->Xtzq));
    PassArgs a = pass_args(c, qof(c->x), pof(c, c->x));
    HX_LAUNCH(HX_KIND_OTHER, 1, lws_features(c->K, a, c->dm, c->Xtzq, d_feat, c->st));
    HX_CK(cudaStreamSynchronize(c->st));
    return HX_OK;
}

int hx_lws_forward(const float* d_feat, int64_t n, int32_t K, const float* d_params, float* d_q, void* stream) {
    if (!d_feat || !d_params || !d_q || n < 0 || K < 1 || K > HX_KMAX) return HX_EINVAL;
    if (n == 0) return HX_OK;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = lws_forward(d_feat, n, K, d_params, d_q, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return cuda_status(e);
}

int hx_lws_grad(const float* d_feat, const float* d_target, int64_t n, int32_t K, const float* d_params,
                float* d_grad, double* d_loss, void* stream) {
    if (!d_feat || !d_target || !d_params || !d_grad || n <= 0 || K < 1 || K > HX_KMAX) return HX_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = lws_attrs();
    LwsScratch sc;
    if (e == cudaSuccess) e = sc.alloc(0);
    if (e == cudaSuccess) e = lws_grad(d_feat, d_target, nullptr, n, K, d_params, sc.part, sc.loss_part, d_grad, d_loss, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return cuda_status(e);
}

int hx_lws_train(const float* d_feat, const float* d_target, int64_t n, int32_t K, float* d_params, float* d_m,
                 float* d_v, int32_t steps, int64_t batch, float lr, uint64_t seed, int32_t step0, double* d_losses,
                 void* stream) {
    if (!d_feat || !d_target || !d_params || !d_m || !d_v || n <= 0 || K < 1 || K > HX_KMAX || steps < 0 ||
        batch <= 0 || step0 < 0)
        return HX_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = lws_attrs();
    LwsScratch sc;
    if (e == cudaSuccess) e = sc.alloc(batch);
    if (e == cudaSuccess)
        e = lws_train(d_feat, d_target, n, K, d_params, d_m, d_v, steps, batch, lr, seed, step0, sc.idx, sc.part,
                      sc.loss_part, sc.grad, d_losses, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return cuda_status(e);
}

int hx_lws_warm_start(hx_ctx* c, const float* params, int32_t p_step, int32_t* accepted) {
    HX_ST(check_qp(c));
    if (!params) return HX_EINVAL;
    if (accepted) *accepted = 0;
    HX_CK(cudaSetDevice(c->device));
    const int64_t nq = (int64_t)c->K * c->I;
    Tmp t;
    int st = HX_OK;
    float* dP = t.get<float>(c, HX_LWS_NPARAM, &st);
    float* feat = t.get<float>(c, (size_t)nq * 2, &st);
    float* qf = t.get<float>(c, (size_t)nq, &st);
    if (st != HX_OK) return st;
    HX_CK(cudaMemcpyAsync(dP, params, HX_LWS_NPARAM * sizeof(float), cudaMemcpyHostToDevice, c->st));
    HX_ST(hx_lws_features(c, feat));
    HX_CK(lws_forward(feat, c->I, c->K, dP, qf, c->st));
    // x_tmp = [project(q') | p]
    HX_LAUNCH(HX_KIND_OTHER, 1, launch_f2d(qf, nq, qof(c->xt), c->st));
    HX_LAUNCH(HX_KIND_OTHER, 1, launch_step_q(qof(c->xt), nullptr, c->K, c->I, c->eps, qof(c->xt), c->st));
    if (p_step) {
        // x_tmp.p = one P step at (q', p) (update_p!, src/algorithms_inner.jl:224-355);
        // x_next.p holds the QP's step (x_next is rewritten by the next iteration)
        HX_ST(pass_p(c, qof(c->xt), pof(c, c->x), true, c->XtXp, c->Xtzp));
        HX_LAUNCH(HX_KIND_QP_P, 1,
                  launch_qp_p(c->K, c->J, c->XtXp, c->Xtzp, pof(c, c->x), c->rho, pof(c, c->xn), c->slots, c->qp_ws,
                              c->st, c->lo.penalty == 0));
        HX_LAUNCH(HX_KIND_OTHER, 1,
                  launch_step_p(pof(c, c->x), pof(c, c->xn), c->K, c->J, c->eps, pof(c, c->xt), c->st));
    } else {
        HX_CK(cudaMemcpyAsync(pof(c, c->xt), pof(c, c->x), (size_t)c->K * 4 * c->J * sizeof(double),
                              cudaMemcpyDeviceToDevice, c->st));
    }
    HX_ST(loglik_to_slot(c, qof(c->x), pof(c, c->x), S_TMP));
    HX_ST(read_slots(c));
    const double ll0 = c->h_slots[S_TMP];
    HX_ST(loglik_to_slot(c, qof(c->xt), pof(c, c->xt), S_TMP));
    HX_ST(read_slots(c));
    const double ll1 = c->h_slots[S_TMP];
    if (ll1 > ll0) {
        HX_CK(cudaMemcpyAsync(c->x, c->xt, (size_t)c->nx * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
        HX_ST(reset_state(c));
        if (accepted) *accepted = 1;
    }
    return HX_OK;
}

int hx_fit(hx_ctx* c, int32_t n_iter, double rtol, int32_t em_iters, hx_fit_info* info) {
    HX_ST(check_qp(c));
    auto t0 = std::chrono::steady_clock::now();
    HX_ST(hx_init_em(c, em_iters));
    HX_ST(hx_admixture_qn(c, n_iter, rtol, 0, info));
    if (info) {
        info->em_iters = em_iters;
        info->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return HX_OK;
}

// Measures each of the mixed method's pass kernels (Q and P tensor-core
// passes with their reductions, FP32 log-likelihood) at the current state
// for chunk counts from half to twice the plan's, keeps the fastest, and
// remembers it for every later context of the same device and shape.
namespace {
int autotune(hx_ctx* c, TuneVal& best) {
    HX_CK(cudaSetDevice(c->device));
    const double* q = qof(c->x);
    const double* p = pof(c, c->x);
    auto elapsed = [&](auto&& run, float& best) -> int {
        best = 1e30f;
        for (int rep = 0; rep < 2; ++rep) {
            HX_CK(cudaEventRecord(c->ev0, c->st));
            HX_ST(run());
            HX_CK(cudaEventRecord(c->ev1, c->st));
            HX_CK(cudaEventSynchronize(c->ev1));
            float ms = 0.f;
            HX_CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
            best = std::min(best, ms);
        }
        return HX_OK;
    };
    // candidate chunk lengths: chunk counts S0 * f for f in [1/2, 2], within the cap
    auto candidates = [](int64_t units, int S0, int cap) {
        std::vector<int64_t> per;
        for (double f : {0.5, 2.0 / 3.0, 0.75, 1.0, 4.0 / 3.0, 1.5, 2.0}) {
            int64_t S = std::max<int64_t>(1, std::min<int64_t>(cap, (int64_t)std::lround(S0 * f)));
            const int64_t len = (units + S - 1) / S;
            if (std::find(per.begin(), per.end(), len) == per.end()) per.push_back(len);
        }
        return per;
    };
    const int64_t nst = (c->I + 31) / 32;
    float t_best = 0.f, t = 0.f;
    // Q side
    {
        const TuneVal keep = best;
        HX_ST(elapsed([&] { return pass_q(c, q, p, true, c->XtXq, c->Xtzq); }, t_best));
        for (int64_t len : candidates(c->JW, c->S_qt, c->Sq_cap)) {
            apply_tuned(c, TuneVal{(int)len, keep.spc_pt, keep.wpc_ll});
            HX_ST(elapsed([&] { return pass_q(c, q, p, true, c->XtXq, c->Xtzq); }, t));
            if (t < t_best) { t_best = t; best.wpc_qt = (int)len; }
        }
        apply_tuned(c, best);
    }
    // P side
    {
        HX_ST(elapsed([&] { return pass_p(c, q, p, true, c->XtXp, c->Xtzp); }, t_best));
        const TuneVal keep = best;
        for (int64_t len : candidates(nst, c->S_pt, c->Sp_cap)) {
            apply_tuned(c, TuneVal{keep.wpc_qt, (int)len, keep.wpc_ll});
            HX_ST(elapsed([&] { return pass_p(c, q, p, true, c->XtXp, c->Xtzp); }, t));
            if (t < t_best) { t_best = t; best.spc_pt = (int)len; }
        }
        apply_tuned(c, best);
    }
    // log-likelihood
    {
        HX_ST(elapsed([&] { return loglik_to_slot(c, q, p, S_TMP); }, t_best));
        const TuneVal keep = best;
        for (int64_t len : candidates(c->JW, c->S_ll, c->Sll_cap)) {
            apply_tuned(c, TuneVal{keep.wpc_qt, keep.spc_pt, (int)len});
            HX_ST(elapsed([&] { return loglik_to_slot(c, q, p, S_TMP); }, t));
            if (t < t_best) { t_best = t; best.wpc_ll = (int)len; }
        }
        apply_tuned(c, best);
    }
    return HX_OK;
}
}  // namespace

int hx_autotune(hx_ctx* c, int32_t* chunks) {
    HX_ST(check_qp(c));
    if (!c->tc) return HX_OK;
    const TuneVal planned{c->wpc_qt, c->ipc_pt / 32, c->wpc_ll};
    TuneVal best = planned;
    int st = autotune(c, best);
    if (st == HX_OK) st = take_timeout(c);
    if (st != HX_OK) {          // keep the context on its planned splits
        apply_tuned(c, planned);
        return st;
    }
    tune_store(c, best);
    if (chunks) { chunks[0] = c->S_qt; chunks[1] = c->S_pt; chunks[2] = c->S_ll; }
    return HX_OK;
}

int hx_set_profiling(hx_ctx* c, int32_t on) {
    if (!c) return HX_EINVAL;
    HX_CK(cudaStreamSynchronize(c->st));
    prof_resolve(c);
    c->profiling = on != 0;
    return HX_OK;
}

int hx_kernel_stats(hx_ctx* c, int32_t kind, int64_t* launches, double* ms) {
    if (!c || kind < 0 || kind >= HX_NKIND) return HX_EINVAL;
    HX_CK(cudaStreamSynchronize(c->st));
    prof_resolve(c);
    if (launches) *launches = c->launches[kind];
    if (ms) *ms = c->kms[kind];
    return HX_OK;
}

int hx_reset_stats(hx_ctx* c) {
    if (!c) return HX_EINVAL;
    HX_CK(cudaStreamSynchronize(c->st));
    prof_resolve(c);
    for (int k = 0; k < HX_NKIND; ++k) { c->launches[k] = 0; c->kms[k] = 0.0; }
    return HX_OK;
}

int hx_synth_bed_device(uint64_t seed, int64_t I, int64_t J, int32_t K, const uint64_t* thrQ, const uint64_t* thrP,
                        double miss, uint8_t* d_bed, int32_t device) {
    if (I <= 0 || J <= 0 || K < 1 || !thrQ || !thrP || !d_bed) return HX_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return HX_ECUDA;
    uint64_t *dQ = nullptr, *dP = nullptr;
    if (cudaMalloc((void**)&dQ, (size_t)K * I * 8) != cudaSuccess) return HX_ENOMEM;
    if (cudaMalloc((void**)&dP, (size_t)K * 4 * J * 8) != cudaSuccess) { cudaFree(dQ); return HX_ENOMEM; }
    int rc = HX_OK;
    if (cudaMemcpy(dQ, thrQ, (size_t)K * I * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(dP, thrP, (size_t)K * 4 * J * 8, cudaMemcpyHostToDevice) != cudaSuccess ||
        launch_synth(seed, I, J, K, dQ, dP, miss, d_bed, 0) != cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess)
        rc = HX_ECUDA;
    cudaFree(dQ);
    cudaFree(dP);
    return rc;
}

}  // extern "C"
