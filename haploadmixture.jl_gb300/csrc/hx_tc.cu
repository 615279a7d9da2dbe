// hx_tc.cu -- tensor-core (tcgen05) gradient/Hessian passes of the mixed method.
//
// Both accumulations are GEMMs whose A operand is generated on the fly from the
// genotype classes:
//   Q side (src/loops.jl:328-365):  H_i = sum_m W[i,m] PP[m,:],  g_i = sum_m U[i,m] P[m,:]
//   P side (src/loops.jl:367-403):  H_m = sum_i W[i,m] QQ[i,:],  g_m = sum_i U[i,m] Q[i,:]
// with m = 4j+h, U = c_h/qp_h, W = c_h/qp_h^2, PP[m,(k,k2)] = p[k,m] p[k2,m]
// (upper triangle) and QQ[i,(k,k2)] = q[k,i] q[k2,i].  The CUDA cores evaluate
// each (individual, block) pair once (qp, class, U, W) and write 16-bit hi/lo
// splits of U and W into shared memory; one thread issues
// tcgen05.mma kind::f16 (16-bit x 16-bit -> fp32 in TMEM) for hi*hi + hi*lo + lo*hi.
// The Hessian operands use BF16 (8-bit exponent) because W spans ~1 .. 2e10,
// beyond FP16's range: hi+lo carries 16 significant bits.  The gradient
// operands use IEEE FP16 hi/lo (22 bits) under exact power-of-two scaling,
// since the gradient fixes the optimum and the Hessian only the step.
// TMEM accumulates FP32 over windows of TC_FLUSH stages; each window is folded
// into registers (the gradient Kahan-compensated), and chunk partials are
// summed in FP64 by the same reduction as the CUDA-core pass.
//
// Pipeline per stage (32 reduction indices): the next stage's global inputs
// are prefetched into registers; [wait MMA of stage s-2] -> stage inputs to
// shared memory -> generate A and B tiles (double-buffered) -> barrier -> one
// thread issues the MMAs and commits to an mbarrier -> the previous TMEM window
// is folded while the tensor core runs.  ~100 KB of shared memory per CTA, so
// two CTAs (16 warps) share an SM and cover each other's barrier and load
// stalls.  Every wait is bounded (TC_BUDGET cycles); a timeout sets
// slots[S_TC_TIMEOUT] and the CTA drains and exits.
#include "hx_ops.cuh"
#include "hx_tc.cuh"

namespace hx {
namespace {
using namespace tc;

constexpr int TC_THREADS = 256;
constexpr int TC_FLUSH = 8;                // stages per TMEM window (256 reduction indices)
constexpr long long TC_BUDGET = 4000000000LL;
constexpr int KD = 32;                     // reduction indices per stage
constexpr int LBO_STD = 128;
constexpr int SBO_STD = (KD / 8) * LBO_STD;      // 512
constexpr int LBO_PAD = 144;               // P-side A: padded for conflict-free generator stores
constexpr int SBO_PAD = (KD / 8) * LBO_PAD;      // 576
constexpr int A_TILE_STD = 16 * SBO_STD;   // 128 rows x 32 x 2 B = 8 KB
constexpr int A_TILE_PAD = 16 * SBO_PAD;
// Gradient operands: IEEE FP16 hi/lo under exact power-of-two scaling that keeps
// them in FP16's normal range: U * 2^-2 <= 5e4 (U = c/qp <= 2/1e-5); P or Q * 2^12
// in [0.04, 4096].
constexpr float U_SCALE = 0.25f;
constexpr float GB_SCALE = 4096.0f;
constexpr double G_UNSCALE = 1.0 / 1024.0;

template <int K> struct TcDims {
    static constexpr int NH = K * (K + 1) / 2;
    static constexpr int NHP = (NH + 15) / 16 * 16;
    static constexpr int NG = 16;
    static constexpr int NT = NHP + NG;
    static constexpr int TCOLS = (2 * NT <= 32) ? 32 : (2 * NT <= 64) ? 64 : (2 * NT <= 128) ? 128 : 256;
    static constexpr int HALF = NT / 2;
    static constexpr int B_TILE = (NT / 8) * SBO_STD;    // NT rows x 32 x 2 B
    static constexpr int VPT = (KD * K + TC_THREADS - 1) / TC_THREADS;   // staged values per thread
    // CTAs per SM: 2 while the generators fit in 128 registers, else 1
    static constexpr int MINB = K <= 8 ? 2 : 1;
};

struct Sync {
    uint64_t mma_done[2];
    uint64_t flush_done[2];
    uint64_t qp_done[2];
    uint32_t tslot;
    int bad;
    int issued;     // stages whose MMAs have been issued
    uint32_t arrived[2];   // generator threads done with stage buffer b
};

// Arrival on the stage buffer: returns true for the last of the TC_THREADS
// generator threads.  Release/acquire ordering (after each writer's
// fence.proxy.async) makes every thread's tile stores visible to the MMAs
// that the last arriver issues.
__device__ __forceinline__ bool arrive_last(uint32_t* ctr, uint32_t total) {
    uint32_t old;
    asm volatile("atom.acq_rel.cta.shared::cta.add.u32 %0, [%1], 1;" : "=r"(old) : "r"(smem_u32(ctr)) : "memory");
    return old == total - 1;
}

__device__ __forceinline__ void set_bad(Sync* sy, double* slots) {
    sy->bad = 1;
    if (slots) slots[S_TC_TIMEOUT] = 1.0;
}

// After a timeout: wait (bounded) until the MMAs of the last two issued stages
// have completed, so that TMEM is not released under an MMA in flight.
__device__ __forceinline__ void drain(Sync* sy) {
    __syncthreads();
    const int n = sy->issued;
    if (!sy->bad || n == 0) return;
    for (int s = (n >= 2 ? n - 2 : 0); s < n; ++s) mbar_wait(&sy->mma_done[s & 1], (s >> 1) & 1, TC_BUDGET);
}

// TMEM window fold: this thread's lane, columns [HF*HALF, HF*HALF + HALF) of the
// accumulator at column base dcol.  Hessian columns add plainly; gradient
// columns (>= NHP) use Kahan compensation in comp[col - NHP].
template <int K, int HF>
__device__ __forceinline__ void fold(uint32_t taddr_lane, int dcol, float* acc, float* comp) {
    using D = TcDims<K>;
#pragma unroll
    for (int c = 0; c < D::HALF / 8; ++c) {
        float v[8];
        tmem_ld8(taddr_lane + (uint32_t)(dcol + HF * D::HALF + 8 * c), v);
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int col = HF * D::HALF + 8 * c + t;
            if (col >= D::NHP) {
                const float y = v[t] - comp[col - D::NHP];
                const float s = acc[8 * c + t] + y;
                comp[col - D::NHP] = (s - acc[8 * c + t]) - y;
                acc[8 * c + t] = s;
            } else {
                acc[8 * c + t] += v[t];
            }
        }
    }
}
template <int K>
__device__ __forceinline__ void fold_half(int hf, uint32_t taddr_lane, int dcol, float* acc, float* comp) {
    if (hf == 0) fold<K, 0>(taddr_lane, dcol, acc, comp);
    else fold<K, 1>(taddr_lane, dcol, acc, comp);
}
// Applies the Kahan compensation to the gradient columns: acc then holds the sums.
template <int K, int HF>
__device__ __forceinline__ void compensate(float* acc, const float* comp) {
    using D = TcDims<K>;
#pragma unroll
    for (int c = 0; c < D::HALF; ++c) {
        const int col = HF * D::HALF + c;
        if (col >= D::NHP) acc[c] -= comp[col - D::NHP];
    }
}

// Issues the 3 split products of one 32-deep stage into D (TMEM cols dcol..):
// Hessian (N = NHP, bf16) and gradient (N = 16, fp16).  A tiles W_hi, W_lo,
// U_hi, U_lo at aBase + t*aStride; B tiles: hi at bBase, lo at bBase + B_TILE.
template <int K>
__device__ __forceinline__ void issue_stage(uint32_t tmem, int dcol, uint32_t aBase, int aStride, int aLBO, int aSBO,
                                            uint32_t bBase, bool first) {
    using D = TcDims<K>;
    constexpr uint32_t idH = idesc_bf16(D::NHP);
    constexpr uint32_t idG = idesc_f16(D::NG);
    const uint32_t dH = tmem + dcol;
    const uint32_t dG = tmem + dcol + D::NHP;
    const uint32_t bPPh = bBase, bPPl = bBase + D::B_TILE;
    const uint32_t bPh = bBase + (D::NHP / 8) * SBO_STD, bPl = bPh + D::B_TILE;
#pragma unroll
    for (int ks = 0; ks < KD / 16; ++ks) {
        const uint32_t ao = ks * 2 * aLBO, bo = ks * 2 * LBO_STD;
        const uint32_t acc0 = (first && ks == 0) ? 0u : 1u;
        const uint64_t aWh = sdesc(aBase + ao, aLBO, aSBO), aWl = sdesc(aBase + aStride + ao, aLBO, aSBO);
        const uint64_t aUh = sdesc(aBase + 2 * aStride + ao, aLBO, aSBO), aUl = sdesc(aBase + 3 * aStride + ao, aLBO, aSBO);
        mma_bf16(dH, aWh, sdesc(bPPh + bo, LBO_STD, SBO_STD), idH, acc0);
        mma_bf16(dH, aWh, sdesc(bPPl + bo, LBO_STD, SBO_STD), idH, 1u);
        mma_bf16(dH, aWl, sdesc(bPPh + bo, LBO_STD, SBO_STD), idH, 1u);
        mma_bf16(dG, aUh, sdesc(bPh + bo, LBO_STD, SBO_STD), idG, acc0);
        mma_bf16(dG, aUh, sdesc(bPl + bo, LBO_STD, SBO_STD), idG, 1u);
        mma_bf16(dG, aUl, sdesc(bPh + bo, LBO_STD, SBO_STD), idG, 1u);
    }
}

// B tile item: row n (PP column for n < NHP, P/Q column for n >= NHP), 8
// consecutive reduction indices whose K-vectors start at vec0[e * K].
template <int K, int VS>
__device__ __forceinline__ void b_item(const float* vec0, int n, uint32_t dst_hi, uint32_t dst_lo) {
    using D = TcDims<K>;
    float v[8];
    uint32_t h[4], l[4];
    if (n >= D::NHP) {
        const int kk = n - D::NHP;
#pragma unroll
        for (int e = 0; e < 8; ++e) v[e] = kk < K ? vec0[e * VS + kk] * GB_SCALE : 0.f;
#pragma unroll
        for (int e = 0; e < 4; ++e) split2_f16(v[2 * e], v[2 * e + 1], h[e], l[e]);
    } else {
        if (n < D::NH) {
            int k, k2;
            tri_pair<K>(n, k, k2);
#pragma unroll
            for (int e = 0; e < 8; ++e) v[e] = vec0[e * VS + k] * vec0[e * VS + k2];
        } else {
#pragma unroll
            for (int e = 0; e < 8; ++e) v[e] = 0.f;
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) split2(v[2 * e], v[2 * e + 1], h[e], l[e]);
    }
    sts128(dst_hi, h[0], h[1], h[2], h[3]);
    sts128(dst_lo, l[0], l[1], l[2], l[3]);
}

// One (individual, block) pair: qp from q and p (4K values), then U (scaled)
// and W.
template <int K>
__device__ __forceinline__ void gen_pair(unsigned nib, const float* qv, const float* pb, float* U4, float* W4,
                                         const float4* tab) {
    float qp[4];
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        float sm = 0.f;
#pragma unroll
        for (int k = 0; k < K; ++k) sm = fmaf(qv[k], pb[h * K + k], sm);
        qp[h] = sm;
    }
    float L, u[4];
    pair_eval_tab(nib, qp, L, u, tab);
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        U4[h] = u[h] * U_SCALE;
        W4[h] = u[h] * rcp_approx(qp[h]);
    }
}

__device__ __forceinline__ void init_sync(Sync* sy, int tid) {
    if (tid == 0) {
        mbar_init(&sy->mma_done[0], 1); mbar_init(&sy->mma_done[1], 1);
        mbar_init(&sy->flush_done[0], 1); mbar_init(&sy->flush_done[1], 1);
        mbar_init(&sy->qp_done[0], 1); mbar_init(&sy->qp_done[1], 1);
        sy->bad = 0;
        sy->issued = 0;
        sy->arrived[0] = 0;
        sy->arrived[1] = 0;
        mbar_fence_init();
    }
}

// Shared tail of the main loop: MMA issue for stage s and the fold of the
// previous TMEM window.
template <int K>
__device__ __forceinline__ void issue_and_fold(Sync* sy, double* slots, int tid, int hf, int s, int ns, int b,
                                               uint32_t tmem, uint32_t taddr_lane, uint32_t aB, int aStride, int aLBO,
                                               int aSBO, uint32_t bB, float* acc, float* comp) {
    using D = TcDims<K>;
    const int win = s / TC_FLUSH;
    const int d = win & 1;
    (void)tid;
    if (arrive_last(&sy->arrived[b], TC_THREADS)) {
        sy->arrived[b] = 0;          // next touched at stage s+2, after two barriers
        fence_after();
        issue_stage<K>(tmem, d * D::NT, aB, aStride, aLBO, aSBO, bB, (s % TC_FLUSH) == 0);
        commit(&sy->mma_done[b]);
        if ((s % TC_FLUSH) == TC_FLUSH - 1 || s == ns - 1) commit(&sy->flush_done[d]);
        sy->issued = s + 1;
    }
    if ((s % TC_FLUSH) == 0 && s > 0) {
        const int wp = win - 1;
        const bool ok = __all_sync(0xffffffffu, mbar_wait(&sy->flush_done[wp & 1], (wp >> 1) & 1, TC_BUDGET));
        if (!ok) set_bad(sy, slots);
        else {
            fence_after();
            fold_half<K>(hf, taddr_lane, (wp & 1) * D::NT, acc, comp);
        }
        fence_before();
    }
}

template <int K>
__device__ __forceinline__ void final_fold(Sync* sy, double* slots, int hf, int ns, uint32_t taddr_lane, float* acc,
                                           float* comp) {
    using D = TcDims<K>;
    __syncthreads();
    if (ns > 0 && !sy->bad) {
        const int wl = (ns - 1) / TC_FLUSH;
        const bool ok = __all_sync(0xffffffffu, mbar_wait(&sy->flush_done[wl & 1], (wl >> 1) & 1, TC_BUDGET));
        if (!ok) set_bad(sy, slots);
        else {
            fence_after();
            fold_half<K>(hf, taddr_lane, (wl & 1) * D::NT, acc, comp);
        }
    }
    drain(sy);
    fence_before();
    __syncthreads();
    if (hf == 0) compensate<K, 0>(acc, comp);
    else compensate<K, 1>(acc, comp);
}

// ------------------------------------------------------------------ Q side
// CTA: 128 individuals (TMEM lanes) x a chunk of class words; stage = 1 word
// (8 blocks, 32 haplotype columns).  Thread (r, hf): row r, blocks 4hf..4hf+3.
// qp[i, m] = sum_k q[k,i] p[k,m] also comes from the tensor core: kind::tf32
// MMAs (hi*hi + hi*lo + lo*hi of TF32-rounded splits, ~2^-21 relative) of the
// CTA's q tile by the stage's p tile into a double-buffered 32-column TMEM
// tile, issued one stage ahead; each thread reads its row's 16 values.
template <int K> struct QpDims {
    static constexpr int KP = K <= 8 ? 8 : 16;        // reduction padded to tf32 steps of 8
    static constexpr int SBO = (KP / 4) * 128;        // 4 tf32 per 16-byte core row
    static constexpr int A_T = 16 * SBO;              // 128 rows
    static constexpr int B_T = 4 * SBO;               // 32 rows
    static constexpr int NCOL = 2 * TcDims<K>::NT + 64;
    static constexpr int TCOLS = NCOL <= 32 ? 32 : NCOL <= 64 ? 64 : NCOL <= 128 ? 128 : 256;
};

template <int K>
__device__ __forceinline__ void issue_qp(uint32_t tmem_col, uint32_t sAq, uint32_t sBq_buf) {
    using QD = QpDims<K>;
    constexpr uint32_t id = idesc_tf32(32);
#pragma unroll
    for (int ks = 0; ks < QD::KP / 8; ++ks) {
        const uint32_t o = ks * 256;
        const uint64_t ah = sdesc(sAq + o, 128, QD::SBO), al = sdesc(sAq + QD::A_T + o, 128, QD::SBO);
        const uint64_t bh = sdesc(sBq_buf + o, 128, QD::SBO), bl = sdesc(sBq_buf + QD::B_T + o, 128, QD::SBO);
        mma_tf32(tmem_col, ah, bh, id, ks > 0 ? 1u : 0u);
        mma_tf32(tmem_col, ah, bl, id, 1u);
        mma_tf32(tmem_col, al, bh, id, 1u);
    }
}

// Stage t's p values (this thread's VPT of the 32K) into P32 (fp32, for the
// PP tile) and into the tf32 hi/lo B tile of the qp MMA.
template <int K>
__device__ __forceinline__ void stage_p(int tid, const float* pv, float* P, uint32_t sBq_buf) {
    using D = TcDims<K>;
    using QD = QpDims<K>;
#pragma unroll
    for (int v = 0; v < D::VPT; ++v) {
        const int t = tid + v * TC_THREADS;
        if (t < KD * K) {
            P[t] = pv[v];
            const int m = t / K, k = t - (t / K) * K;
            const float hi = tf32_round(pv[v]);
            const float lo = tf32_round(pv[v] - hi);
            const uint32_t off = (m >> 3) * QD::SBO + (k >> 2) * 128 + (m & 7) * 16 + (k & 3) * 4;
            asm volatile("st.shared.b32 [%0], %1;" :: "r"(sBq_buf + off), "f"(hi) : "memory");
            asm volatile("st.shared.b32 [%0], %1;" :: "r"(sBq_buf + QD::B_T + off), "f"(lo) : "memory");
        }
    }
}

template <int K>
__device__ __forceinline__ void load_p(int tid, int64_t word, int64_t plimit, const double* p, float* pv) {
    using D = TcDims<K>;
#pragma unroll
    for (int v = 0; v < D::VPT; ++v) {
        const int t = tid + v * TC_THREADS;
        const int64_t g = word * 8 * 4 * K + t;
        pv[v] = (t < KD * K && g < plimit) ? (float)p[g] : 0.25f;
    }
}

// One pair from its qp: U (scaled) and W.
__device__ __forceinline__ void gen_pair_qp(unsigned nib, const float* qp, float* U4, float* W4, const float4* tab) {
    float L, u[4];
    pair_eval_tab(nib, qp, L, u, tab);
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        U4[h] = u[h] * U_SCALE;
        W4[h] = u[h] * rcp_approx(qp[h]);
    }
}

template <int K>
__global__ void __launch_bounds__(TC_THREADS, TcDims<K>::MINB) k_accum_q_tc(PassArgs a) {
    using D = TcDims<K>;
    using QD = QpDims<K>;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sA = smem_u32(smem);                              // [2][4][A_TILE_STD]
    const uint32_t sB = sA + 2 * 4 * A_TILE_STD;                     // [2][2][B_TILE]
    const uint32_t sAq = sB + 2 * 2 * D::B_TILE;                     // [2 hi/lo][A_T]
    const uint32_t sBq = sAq + 2 * QD::A_T;                          // [2 buf][2 hi/lo][B_T]
    float* P32 = (float*)(smem + (sBq - sA) + 4 * QD::B_T);          // [2][KD * K]
    Sync* sy = (Sync*)(P32 + 2 * KD * K);
    __shared__ float4 s_snp[4];

    const int tid = threadIdx.x, warp = tid >> 5;
    const int r = tid & 127, hf = tid >> 7;
    snp_table_init(s_snp, tid);
    const int64_t i = (int64_t)blockIdx.x * 128 + r;
    const bool active = i < a.I;
    const int w0 = blockIdx.y * a.per_chunk;
    const int ns = min(a.JW, w0 + a.per_chunk) - w0;     // one word per stage
    const int64_t plimit = a.J * 4 * K;

    if (warp == 0) tmem_alloc<QD::TCOLS>(&sy->tslot);
    init_sync(sy, tid);
    // zero the tf32 operand tiles (reduction padding k >= K stays zero)
    for (int t = tid; t < (2 * QD::A_T + 4 * QD::B_T) / 4; t += TC_THREADS)
        asm volatile("st.shared.b32 [%0], %1;" :: "r"(sAq + 4 * t), "r"(0u) : "memory");
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = sy->tslot;
    const uint32_t tq = tmem + 2 * D::NT;                 // qp tiles: columns [2NT, 2NT + 64)
    const uint32_t taddr_lane = tmem + ((uint32_t)(32 * (warp & 3)) << 16);

    // q tile (tf32 hi/lo), once per CTA
    if (hf == 0) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const float x = active ? (float)a.q[(int64_t)K * i + k] : 1.f / K;
            const float hi = tf32_round(x), lo = tf32_round(x - hi);
            const uint32_t off = (r >> 3) * QD::SBO + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4;
            asm volatile("st.shared.b32 [%0], %1;" :: "r"(sAq + off), "f"(hi) : "memory");
            asm volatile("st.shared.b32 [%0], %1;" :: "r"(sAq + QD::A_T + off), "f"(lo) : "memory");
        }
    }
    float acc[D::HALF], comp[D::NG];
#pragma unroll
    for (int c = 0; c < D::HALF; ++c) acc[c] = 0.f;
#pragma unroll
    for (int c = 0; c < D::NG; ++c) comp[c] = 0.f;

    // stage 0 inputs, then the qp MMA of stage 0
    float pv[D::VPT];
    uint32_t word_cur = HX_PAD_WORD, word_nx = HX_PAD_WORD;
    if (ns > 0) {
        load_p<K>(tid, w0, plimit, a.p, pv);
        stage_p<K>(tid, pv, P32, sBq);
        word_cur = a.G[(int64_t)w0 * a.Ipad + i];
    }
    if (ns > 1) load_p<K>(tid, w0 + 1, plimit, a.p, pv);
    fence_async_smem();
    fence_before();
    __syncthreads();
    if (tid == 0 && ns > 0) {
        fence_after();
        issue_qp<K>(tq, sAq, sBq);
        commit(&sy->qp_done[0]);
    }

    for (int s = 0; s < ns; ++s) {
        const int b = s & 1, bn = b ^ 1;
        const uint32_t word = word_cur;
        // main tile buffer b was last read by the MMAs of stage s-2
        if (s >= 2 && !sy->bad) {
            if (!mbar_wait(&sy->mma_done[b], ((s - 2) >> 1) & 1, TC_BUDGET)) set_bad(sy, a.slots);
        }
        __syncthreads();
        if (sy->bad) break;
        // the next stage's inputs (its qp MMA is issued by this stage's last arriver)
        if (s + 1 < ns) {
            stage_p<K>(tid, pv, P32 + bn * KD * K, sBq + bn * 2 * QD::B_T);
            word_nx = a.G[(int64_t)(w0 + s + 1) * a.Ipad + i];
            if (s + 2 < ns) load_p<K>(tid, w0 + s + 2, plimit, a.p, pv);
        }
        const float* P = P32 + b * KD * K;
        const uint32_t bB = sB + b * 2 * D::B_TILE;
        for (int it = tid; it < D::NT * (KD / 8); it += TC_THREADS) {
            const int n = it % D::NT, kg = it / D::NT;
            const uint32_t off = (n >> 3) * SBO_STD + kg * LBO_STD + (n & 7) * 16;
            b_item<K, K>(P + kg * 8 * K, n, bB + off, bB + D::B_TILE + off);
        }
        // this stage's qp: 16 columns of this thread's row
        float qpv[16];
        {
            const bool ok = __all_sync(0xffffffffu, mbar_wait(&sy->qp_done[b], (s >> 1) & 1, TC_BUDGET));
            if (!ok) set_bad(sy, a.slots);
            fence_after();
            tmem_ld8(taddr_lane + (uint32_t)(2 * D::NT + b * 32 + hf * 16), qpv);
            tmem_ld8(taddr_lane + (uint32_t)(2 * D::NT + b * 32 + hf * 16 + 8), qpv + 8);
        }
        const uint32_t aB = sA + b * 4 * A_TILE_STD;
#pragma unroll
        for (int t2 = 0; t2 < 2; ++t2) {
            float W[8], U[8];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int bb = 2 * t2 + e;                    // block within this thread's half
                gen_pair_qp((word >> (4 * (hf * 4 + bb))) & 0xFu, qpv + 4 * bb, U + 4 * e, W + 4 * e, s_snp);
            }
            const uint32_t off = (r >> 3) * SBO_STD + (hf * 2 + t2) * LBO_STD + (r & 7) * 16;
            uint32_t wh[4], wl[4], uh[4], ul[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                split2(W[2 * e], W[2 * e + 1], wh[e], wl[e]);
                split2_f16(U[2 * e], U[2 * e + 1], uh[e], ul[e]);
            }
            sts128(aB + off, wh[0], wh[1], wh[2], wh[3]);
            sts128(aB + A_TILE_STD + off, wl[0], wl[1], wl[2], wl[3]);
            sts128(aB + 2 * A_TILE_STD + off, uh[0], uh[1], uh[2], uh[3]);
            sts128(aB + 3 * A_TILE_STD + off, ul[0], ul[1], ul[2], ul[3]);
        }
        fence_async_smem();
        fence_before();
        {
            const int win = s / TC_FLUSH;
            const int d = win & 1;
            if (arrive_last(&sy->arrived[b], TC_THREADS)) {
                sy->arrived[b] = 0;
                fence_after();
                issue_stage<K>(tmem, d * D::NT, aB, A_TILE_STD, LBO_STD, SBO_STD, bB, (s % TC_FLUSH) == 0);
                if (s + 1 < ns) issue_qp<K>(tq + bn * 32, sAq, sBq + bn * 2 * QD::B_T);
                // mma_done also covers the qp MMA, so that draining it covers every MMA in flight
                commit(&sy->mma_done[b]);
                if (s + 1 < ns) commit(&sy->qp_done[bn]);
                if ((s % TC_FLUSH) == TC_FLUSH - 1 || s == ns - 1) commit(&sy->flush_done[d]);
                sy->issued = s + 1;
            }
            if ((s % TC_FLUSH) == 0 && s > 0) {
                const int wp = win - 1;
                const bool ok = __all_sync(0xffffffffu, mbar_wait(&sy->flush_done[wp & 1], (wp >> 1) & 1, TC_BUDGET));
                if (!ok) set_bad(sy, a.slots);
                else {
                    fence_after();
                    fold_half<K>(hf, taddr_lane, (wp & 1) * D::NT, acc, comp);
                }
                fence_before();
            }
        }
        word_cur = word_nx;
    }
    final_fold<K>(sy, a.slots, hf, ns, taddr_lane, acc, comp);
    // write partials: v < K gradient, v = K + tri index Hessian
    constexpr int NV = K + D::NH;
    double* out = a.part + (int64_t)blockIdx.y * NV * a.Ipad;
#pragma unroll
    for (int c = 0; c < D::HALF; ++c) {
        const int col = hf * D::HALF + c;
        if (col < D::NH) {
            out[(int64_t)(K + col) * a.Ipad + i] = (double)acc[c];
        } else if (col >= D::NHP && col < D::NHP + K) {
            out[(int64_t)(col - D::NHP) * a.Ipad + i] = (double)acc[c] * G_UNSCALE;
        }
    }
    if (warp == 0) {
        fence_after();
        tmem_dealloc<QD::TCOLS>(tmem);
    }
}

// ------------------------------------------------------------------ P side
// CTA: 32 blocks (128 haplotype columns = TMEM lanes) x a chunk of individuals;
// stage = 32 individuals.  Thread (jl, ig): block jl, individuals 4ig..4ig+3.
// Staged q rows have stride QSTR floats (an odd number of 16-byte units), so
// the 8 individual groups of a warp read 8 distinct bank quads.
template <int K> constexpr int qstr() { return K <= 4 ? 4 : 12; }

template <int K>
__global__ void __launch_bounds__(TC_THREADS, TcDims<K>::MINB) k_accum_p_tc(PassArgs a) {
    using D = TcDims<K>;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sA = smem_u32(smem);                              // [2][4][A_TILE_PAD]
    const uint32_t sB = sA + 2 * 4 * A_TILE_PAD;                     // [2][2][B_TILE]
    constexpr int QSTR = qstr<K>();
    float* Q32 = (float*)(smem + 2 * 4 * A_TILE_PAD + 2 * 2 * D::B_TILE);   // [2][KD * QSTR]
    uint32_t* SW = (uint32_t*)(Q32 + 2 * KD * QSTR);                 // [2][4][KD]
    Sync* sy = (Sync*)(SW + 2 * 4 * KD);
    __shared__ float4 s_snp[4];

    const int tid = threadIdx.x, warp = tid >> 5;
    snp_table_init(s_snp, tid);
    const int jl = tid >> 3, ig = tid & 7;
    const int hf = tid >> 7;
    const int64_t j = (int64_t)blockIdx.x * 32 + jl;
    const bool valid = j < a.J;
    const int64_t i0 = (int64_t)blockIdx.y * a.per_chunk;
    const int64_t i1 = min(a.I, i0 + (int64_t)a.per_chunk);
    const int ns = (int)((i1 - i0 + KD - 1) / KD);

    if (warp == 0) tmem_alloc<D::TCOLS>(&sy->tslot);
    init_sync(sy, tid);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = sy->tslot;
    const uint32_t taddr_lane = tmem + ((uint32_t)(32 * (warp & 3)) << 16);

    float pr[4 * K];
#pragma unroll
    for (int t = 0; t < 4 * K; ++t) pr[t] = valid ? (float)a.p[(int64_t)K * 4 * j + t] : 0.25f;
    float acc[D::HALF], comp[D::NG];
#pragma unroll
    for (int c = 0; c < D::HALF; ++c) acc[c] = 0.f;
#pragma unroll
    for (int c = 0; c < D::NG; ++c) comp[c] = 0.f;
    const int bsh = 4 * (jl & 7);

    // staging roles: q values (VPT per thread) and class words (threads < 4*KD)
    const int sw_w = tid / KD, sw_i = tid % KD;                      // word column, individual
    const int64_t sw_jw = (int64_t)blockIdx.x * 4 + sw_w;
    float qv_nx[D::VPT];
    uint32_t w_nx = HX_PAD_WORD;
    {
        const int64_t n0 = min((int64_t)KD, i1 - i0);
        if (tid < 4 * KD && sw_i < n0 && sw_jw < a.JW) w_nx = a.G[sw_jw * a.Ipad + i0 + sw_i];
#pragma unroll
        for (int v = 0; v < D::VPT; ++v) {
            const int t = tid + v * TC_THREADS;
            qv_nx[v] = (t < (int)n0 * K) ? (float)a.q[(int64_t)K * i0 + t] : 1.f / K;
        }
    }

    for (int s = 0; s < ns; ++s) {
        const int b = s & 1;
        float* Qs = Q32 + b * KD * QSTR;
        uint32_t* Ws = SW + b * 4 * KD;
        if (s >= 2 && !sy->bad) {
            if (!mbar_wait(&sy->mma_done[b], ((s - 2) >> 1) & 1, TC_BUDGET)) set_bad(sy, a.slots);
        }
#pragma unroll
        for (int v = 0; v < D::VPT; ++v) {
            const int t = tid + v * TC_THREADS;
            if (t < KD * K) Qs[(t / K) * QSTR + t % K] = qv_nx[v];
        }
        if (tid < 4 * KD) Ws[tid] = w_nx;
        if (s + 1 < ns) {
            const int64_t isn = i0 + (int64_t)KD * (s + 1);
            const int64_t nn = min((int64_t)KD, i1 - isn);
            w_nx = (tid < 4 * KD && sw_i < nn && sw_jw < a.JW) ? a.G[sw_jw * a.Ipad + isn + sw_i] : HX_PAD_WORD;
#pragma unroll
            for (int v = 0; v < D::VPT; ++v) {
                const int t = tid + v * TC_THREADS;
                qv_nx[v] = (t < (int)nn * K) ? (float)a.q[(int64_t)K * isn + t] : 1.f / K;
            }
        }
        __syncthreads();
        if (sy->bad) break;
        const uint32_t bB = sB + b * 2 * D::B_TILE;
        for (int it = tid; it < D::NT * (KD / 8); it += TC_THREADS) {
            const int nn = it % D::NT, kg = it / D::NT;
            const uint32_t off = (nn >> 3) * SBO_STD + kg * LBO_STD + (nn & 7) * 16;
            b_item<K, QSTR>(Qs + kg * 8 * QSTR, nn, bB + off, bB + D::B_TILE + off);
        }
        // A = W^T tile: rows m = 4*jl + h, reduction over the stage's individuals
        float W[4][4], U[4][4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int ii = ig * 4 + e;
            const unsigned nib = (Ws[(jl >> 3) * KD + ii] >> bsh) & 0xFu;
            float qv[(K + 3) / 4 * 4];
            const float4* q4 = reinterpret_cast<const float4*>(Qs + ii * QSTR);
#pragma unroll
            for (int c = 0; c < (K + 3) / 4; ++c) {
                const float4 x = q4[c];
                qv[4 * c] = x.x; qv[4 * c + 1] = x.y; qv[4 * c + 2] = x.z; qv[4 * c + 3] = x.w;
            }
            float u4[4], w4[4];
            gen_pair<K>(nib, qv, pr, u4, w4, s_snp);
#pragma unroll
            for (int h = 0; h < 4; ++h) { U[h][e] = u4[h]; W[h][e] = w4[h]; }
        }
        const uint32_t aB = sA + b * 4 * A_TILE_PAD;
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            const int m = 4 * jl + h;
            const uint32_t off = (m >> 3) * SBO_PAD + (ig >> 1) * LBO_PAD + (m & 7) * 16 + (ig & 1) * 8;
            uint32_t wh[2], wl[2], uh[2], ul[2];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                split2(W[h][2 * e], W[h][2 * e + 1], wh[e], wl[e]);
                split2_f16(U[h][2 * e], U[h][2 * e + 1], uh[e], ul[e]);
            }
            asm volatile("st.shared.v2.b32 [%0], {%1, %2};" :: "r"(aB + off), "r"(wh[0]), "r"(wh[1]) : "memory");
            asm volatile("st.shared.v2.b32 [%0], {%1, %2};" :: "r"(aB + A_TILE_PAD + off), "r"(wl[0]), "r"(wl[1]) : "memory");
            asm volatile("st.shared.v2.b32 [%0], {%1, %2};" :: "r"(aB + 2 * A_TILE_PAD + off), "r"(uh[0]), "r"(uh[1]) : "memory");
            asm volatile("st.shared.v2.b32 [%0], {%1, %2};" :: "r"(aB + 3 * A_TILE_PAD + off), "r"(ul[0]), "r"(ul[1]) : "memory");
        }
        fence_async_smem();
        fence_before();
        issue_and_fold<K>(sy, a.slots, tid, hf, s, ns, b, tmem, taddr_lane, aB, A_TILE_PAD, LBO_PAD, SBO_PAD, bB, acc,
                          comp);
    }
    final_fold<K>(sy, a.slots, hf, ns, taddr_lane, acc, comp);
    // rows m of this CTA: TMEM lane r
    const int r = tid & 127;
    const int64_t m = (int64_t)blockIdx.x * 128 + r;
    if (m < 4 * a.J) {
        constexpr int NV = K + D::NH;
        const int64_t rows = 4 * a.J;
#pragma unroll
        for (int c = 0; c < D::HALF; ++c) {
            const int col = hf * D::HALF + c;
            if (col < D::NH) {
                const double val = (double)acc[c];
                if (a.S == 1) {
                    int k, k2;
                    tri_pair<K>(col, k, k2);
                    a.XtX[(int64_t)K * K * m + k2 + K * k] = val;
                    a.XtX[(int64_t)K * K * m + k + K * k2] = val;
                } else {
                    a.part[((int64_t)blockIdx.y * NV + K + col) * rows + m] = val;
                }
            } else if (col >= D::NHP && col < D::NHP + K) {
                const double val = (double)acc[c] * G_UNSCALE;
                if (a.S == 1) a.Xtz[(int64_t)K * m + (col - D::NHP)] = val;
                else a.part[((int64_t)blockIdx.y * NV + (col - D::NHP)) * rows + m] = val;
            }
        }
    }
    if (warp == 0) {
        fence_after();
        tmem_dealloc<D::TCOLS>(tmem);
    }
}

template <int K> constexpr size_t smem_q() {
    using D = TcDims<K>;
    using QD = QpDims<K>;
    return 1024 + 2 * 4 * A_TILE_STD + 2 * 2 * D::B_TILE + 2 * QD::A_T + 4 * QD::B_T + 2 * KD * K * 4 + sizeof(Sync);
}
template <int K> constexpr size_t smem_p() {
    using D = TcDims<K>;
    return 1024 + 2 * 4 * A_TILE_PAD + 2 * 2 * D::B_TILE + 2 * KD * qstr<K>() * 4 + 2 * 4 * KD * 4 + sizeof(Sync);
}

#define HX_FOR_K(X) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12)

}  // namespace

cudaError_t init_tc_attrs() {
    cudaError_t e = cudaSuccess;
#define HX_ATTR(KK)                                                                                   \
    if (e == cudaSuccess)                                                                             \
        e = cudaFuncSetAttribute(k_accum_q_tc<KK>, cudaFuncAttributeMaxDynamicSharedMemorySize,       \
                                 (int)smem_q<KK>());                                                  \
    if (e == cudaSuccess)                                                                             \
        e = cudaFuncSetAttribute(k_accum_p_tc<KK>, cudaFuncAttributeMaxDynamicSharedMemorySize,       \
                                 (int)smem_p<KK>());
    HX_FOR_K(HX_ATTR)
#undef HX_ATTR
    return e;
}

cudaError_t launch_accum_q_tc(int K, const PassArgs& a, cudaStream_t st) {
    dim3 grid((unsigned)(a.Ipad / 128), (unsigned)a.S);
#define HX_CASE(KK) case KK: k_accum_q_tc<KK><<<grid, TC_THREADS, smem_q<KK>(), st>>>(a); break;
    switch (K) { HX_FOR_K(HX_CASE) default: return cudaErrorInvalidValue; }
#undef HX_CASE
    return cudaGetLastError();
}

cudaError_t launch_accum_p_tc(int K, const PassArgs& a, cudaStream_t st) {
    dim3 grid((unsigned)((a.J + 31) / 32), (unsigned)a.S);
#define HX_CASE(KK) case KK: k_accum_p_tc<KK><<<grid, TC_THREADS, smem_p<KK>(), st>>>(a); break;
    switch (K) { HX_FOR_K(HX_CASE) default: return cudaErrorInvalidValue; }
#undef HX_CASE
    return cudaGetLastError();
}

}  // namespace hx
