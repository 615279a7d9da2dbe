// hx_tc_impl.cuh -- tensor-core (tcgen05) gradient/Hessian passes of the mixed method.
//
// Included by the hx_tc_g*.cu translation units, each of which instantiates
// the kernels for a few values of K (see tc_run); hx_tc.cu dispatches on K.
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
// Operand images.  The B operands depend only on p (Q side) or only on q (P
// side), so a small kernel writes them once per pass into global memory, in the
// exact shared-memory core-matrix layout of one stage: for each word column
// (8 blocks) the PP/P hi/lo tile and the tf32 p tile of the qp MMA; for each
// group of 32 individuals the QQ/Q hi/lo tile and the FP32 q rows.  The main
// kernels stream one image slice plus the stage's class words per stage with
// 1-D bulk copies (TMA engine) into a RING-deep shared-memory ring, completing
// on an mbarrier with a transaction count.
//
// Pipeline per stage, with no CTA-wide barrier in the loop: every thread waits
// for the stage's ring slot and until the MMAs that last read its A buffer
// (stage s-2) are done; the first warp to get there refills the ring slot of
// stage s-2 with stage s-2+RING; every warp generates its part of the A tiles and arrives on
// a shared counter; the last arriving warp issues the stage's MMAs and commits
// them to an mbarrier.  Warps therefore run up to two stages apart, and two CTAs (16 warps)
// share an SM.  Every wait is bounded (PassArgs::budget cycles, by default
// TC_BUDGET; the drain after a timeout always allows TC_BUDGET); a timeout sets
// slots[S_TC_TIMEOUT] and the CTA drains and exits.
#pragma once
#include <algorithm>
#include "hx_ops.cuh"
#include "hx_tc.cuh"

namespace hx {
namespace {
using namespace tc;

constexpr int TC_THREADS = 256;
constexpr int TC_FLUSH = 8;                // stages per TMEM window (256 reduction indices)
constexpr long long TC_BUDGET = 4000000000LL;
constexpr int RING = 3;                    // stage-input ring depth
constexpr int QRING = 4;                   // Q side: ring of the qp MMA's p tiles, loaded 4 stages ahead
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
// The generators form U * U_SCALE directly and W * U_SCALE beside it (one
// factor fewer per pair); the Hessian's B rows carry the exact inverse factor.
constexpr float W_UNDO = 1.0f / U_SCALE;
constexpr float GB_SCALE = 4096.0f;
constexpr double G_UNSCALE = 1.0 / 1024.0;

template <int K> struct TcDims {
    static constexpr int NH = K * (K + 1) / 2;
    static constexpr int NHP = (NH + 15) / 16 * 16;
    static constexpr int NG = 16;
    static constexpr int NT = NHP + NG;
    static constexpr int TCOLS = (2 * NT <= 32) ? 32 : (2 * NT <= 64) ? 64 : (2 * NT <= 128) ? 128 : 256;
    static constexpr int HALF = NT / 2;
    // Q side: one TMEM window = [Hessian NHP | gradient hi.hi NG | gradient
    // hi.lo + lo.hi NG].  Every MMA write rounds the accumulator it adds to,
    // not to nearest, so the small lo products get columns of their own:
    // the large hi.hi sums are written a third as often.
    static constexpr int WQ = NT + NG;
    static constexpr int B_TILE = (NT / 8) * SBO_STD;    // NT rows x 32 x 2 B
    // P side, stacked operands: one TMEM window holds hi.hi (+ lo.hi) and hi.lo
    // of the Hessian side by side, then the same for the gradient
    static constexpr int WS = 2 * NHP + 2 * NG;
    static constexpr int TCOLS_S = (2 * WS <= 32) ? 32 : (2 * WS <= 64) ? 64 : (2 * WS <= 128) ? 128 : (2 * WS <= 256) ? 256 : 512;
    // CTAs per SM: 2 while the generators fit in 128 registers, else 1
    static constexpr int MINB = K <= 8 ? 2 : 1;
};

// qp of the Q side from the tensor core (kind::tf32), see k_accum_q_tc.
template <int K> struct QpDims {
    static constexpr int KP = K <= 8 ? 8 : 16;        // reduction padded to tf32 steps of 8
    static constexpr int SBO = (KP / 4) * 128;        // 4 tf32 per 16-byte core row
    static constexpr int A_T = 16 * SBO;              // 128 rows
    static constexpr int B_T = 4 * SBO;               // 32 rows
    static constexpr int NCOL = 2 * TcDims<K>::WQ + 64;
    static constexpr int TCOLS = NCOL <= 32 ? 32 : NCOL <= 64 ? 64 : NCOL <= 128 ? 128 : NCOL <= 256 ? 256 : 512;
    static_assert(NCOL <= TCOLS && TCOLS <= 512, "Q-side TMEM columns");
};

// P side: staged q rows hold each q[k] twice, (q_k, q_k), as the first operand
// of packed f32x2 FMAs; rows have stride QSTR floats (an odd number of 16-byte
// units) and individual ii = 4*ig + e sits in row slot 8e + ig, so the 8
// individual groups ig of a warp read 8 distinct bank quads.
template <int K> constexpr int qstr() { return 4 * ((((2 * K + 3) / 4) | 1)); }
__host__ __device__ constexpr int qrow_slot(int ii) { return 8 * (ii & 3) + (ii >> 2); }

// Image bytes per stage: Q side per word column, P side per 32 individuals.
template <int K> constexpr int qimg_bytes() { return 2 * TcDims<K>::B_TILE + 2 * QpDims<K>::B_T; }
template <int K> constexpr int pimg_bytes() { return 2 * TcDims<K>::B_TILE + KD * qstr<K>() * 4; }

struct Sync {
    uint64_t full[RING];   // stage inputs landed (transaction-count barrier)
    uint64_t fullq[QRING]; // Q side: p tile of the qp MMA landed
    uint64_t mma_done[2];
    uint64_t flush_done[2];
    uint64_t qp_done[2];
    uint64_t gen_full[2];  // the 8 generator warps have written stage buffer b (one arrival per warp)
    uint32_t tslot;
    int bad;
    int issued;            // stages whose MMAs have been issued
    int loaded;            // stages whose input copies have been issued
    int loadedq;           // Q side: stages whose qp p tile copy has been issued
    uint32_t arrived[2];   // generator arrivals on stage buffer b (monotonic)
    uint32_t started[2];   // warps past the waits of a stage, by stage parity (the first one refills)
    // stage-input sources, read only by the thread that issues a refill
    const uint8_t* img0;   // image slice of stage 0
    const uint32_t* g0;    // class words of stage 0
    int64_t gstride;       // words between word columns (Ipad)
    int nwc;               // word columns (P side)
    uint32_t tx;           // bytes per stage
};

__device__ __forceinline__ bool is_bad(const Sync* sy) { return *(volatile const int*)&sy->bad != 0; }

// Arrival on the stage buffer, one atomic per warp: after __syncwarp (which
// orders the warp's tile stores, each already fenced to the async proxy), lane
// 0 adds to the buffer's counter; the lane 0 of the last of the TC_THREADS/32
// warps of this use of the buffer returns true (the counter only grows, so no
// reset races with the next use).  Release/acquire ordering of the atomic makes
// every warp's stores visible to the MMAs that the last arriver issues.
__device__ __forceinline__ bool arrive_last(uint32_t* ctr) {
    __syncwarp();
    bool last = false;
    if ((threadIdx.x & 31) == 0) {
        uint32_t old;
        asm volatile("atom.acq_rel.cta.shared::cta.add.u32 %0, [%1], 1;" : "=r"(old) : "r"(smem_u32(ctr)) : "memory");
        last = (old % (TC_THREADS / 32)) == TC_THREADS / 32 - 1;
    }
    return last;
}

// True in lane 0 of the first warp of the CTA to reach this point of a stage
// (one atomic per warp).  Counted by stage parity like arrive_last: a warp
// reaches stage s+2 only after every warp has passed this point of stage s.
__device__ __forceinline__ bool first_at_stage(uint32_t* ctr) {
    __syncwarp();
    bool first = false;
    if ((threadIdx.x & 31) == 0) {
        uint32_t old;
        asm volatile("atom.relaxed.cta.shared::cta.add.u32 %0, [%1], 1;" : "=r"(old) : "r"(smem_u32(ctr)) : "memory");
        first = (old % (TC_THREADS / 32)) == 0;
    }
    return first;
}

__device__ __forceinline__ void set_bad(Sync* sy, double* slots) {
    *(volatile int*)&sy->bad = 1;
    if (slots) slots[S_TC_TIMEOUT] = 1.0;
}

// After a timeout: wait (bounded) until the MMAs of the last two issued stages
// and the bulk copies of the last RING loaded stages have completed, so that
// TMEM and shared memory are not released under them.  Only operations that
// were issued are waited for, so each wait ends as soon as the hardware does.
__device__ __forceinline__ void drain(Sync* sy) {
    __syncthreads();
    if (!is_bad(sy)) return;
    const int n = sy->issued, l = sy->loaded, lq = sy->loadedq;
    for (int s = (n >= 2 ? n - 2 : 0); s < n; ++s) mbar_wait(&sy->mma_done[s & 1], (s >> 1) & 1, TC_BUDGET);
    for (int s = (l >= RING ? l - RING : 0); s < l; ++s) mbar_wait(&sy->full[s % RING], (s / RING) & 1, TC_BUDGET);
    for (int s = (lq >= QRING ? lq - QRING : 0); s < lq; ++s)
        mbar_wait(&sy->fullq[s % QRING], (s / QRING) & 1, TC_BUDGET);
}

// TMEM window fold: this thread's lane, columns [HF*HALF, HF*HALF + HALF) of the
// accumulator at column base dcol.  Hessian columns add plainly; gradient
// columns (>= NHP) use Kahan compensation in comp[col - NHP].
// With STACK (P side) logical column c sums two physical columns: c and
// NHP + c for the Hessian, 2NHP + g and 2NHP + NG + g for gradient column g.
template <int K, int HF, bool STACK>
__device__ __forceinline__ void fold(uint32_t taddr_lane, int dcol, float* acc, float* comp) {
    using D = TcDims<K>;
    uint32_t raw[D::HALF];
    if (!STACK) {
#pragma unroll
        for (int c = 0; c < D::HALF / 8; ++c)
            tmem_ld8_async(taddr_lane + (uint32_t)(dcol + HF * D::HALF + 8 * c), raw + 8 * c);
        tmem_wait_ld();
        // gradient columns: add their lo-product columns [NT, NT + NG)
#pragma unroll
        for (int c = 0; c < D::HALF / 8; ++c) {
            const int col = HF * D::HALF + 8 * c;     // chunks never straddle NHP (a multiple of 16)
            if (col >= D::NHP) {
                uint32_t r2[8];
                tmem_ld8_async(taddr_lane + (uint32_t)(dcol + D::NT + (col - D::NHP)), r2);
                tmem_wait_ld();
#pragma unroll
                for (int t = 0; t < 8; ++t)
                    raw[8 * c + t] = __float_as_uint(__uint_as_float(raw[8 * c + t]) + __uint_as_float(r2[t]));
            }
        }
    } else {
#pragma unroll
        for (int c = 0; c < D::HALF / 8; ++c) {
            const int col = HF * D::HALF + 8 * c;     // chunks never straddle NHP (a multiple of 16)
            const int p0 = col < D::NHP ? col : 2 * D::NHP + (col - D::NHP);
            tmem_ld8_async(taddr_lane + (uint32_t)(dcol + p0), raw + 8 * c);
        }
        tmem_wait_ld();
#pragma unroll
        for (int c = 0; c < D::HALF / 8; ++c) {
            const int col = HF * D::HALF + 8 * c;
            const int p1 = col < D::NHP ? D::NHP + col : 2 * D::NHP + D::NG + (col - D::NHP);
            uint32_t r2[8];
            tmem_ld8_async(taddr_lane + (uint32_t)(dcol + p1), r2);
            tmem_wait_ld();
#pragma unroll
            for (int t = 0; t < 8; ++t)
                raw[8 * c + t] = __float_as_uint(__uint_as_float(raw[8 * c + t]) + __uint_as_float(r2[t]));
        }
    }
#pragma unroll
    for (int c = 0; c < D::HALF / 8; ++c) {
        float v[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) v[t] = __uint_as_float(raw[8 * c + t]);
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
template <int K, bool STACK>
__device__ __forceinline__ void fold_half(int hf, uint32_t taddr_lane, int dcol, float* acc, float* comp) {
    if (hf == 0) fold<K, 0, STACK>(taddr_lane, dcol, acc, comp);
    else fold<K, 1, STACK>(taddr_lane, dcol, acc, comp);
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

// The 3 split products of one 32-deep stage into D (TMEM cols dcol..):
// Hessian (N = NHP, bf16) and gradient (N = 16, fp16).  A tiles W_hi, W_lo,
// U_hi, U_lo at aBase + t*aStride; B tiles: hi at bBase, lo at bBase + B_TILE.
// Issued in two groups with disjoint accumulator columns, by two issuers: the
// Hessian's (HG = 0) and the gradient's (HG = 1).  Each column keeps one
// issuer, issuing in stage order, so the FP32 accumulation order is fixed
// (bit-reproducible).
template <int K, int HG>
__device__ __forceinline__ void issue_stage_group(uint32_t tmem, int dcol, uint32_t aBase, int aStride, int aLBO,
                                                  int aSBO, uint32_t bBase, bool first) {
    using D = TcDims<K>;
    constexpr uint32_t idH = idesc_bf16(D::NHP);
    constexpr uint32_t idG = idesc_f16(D::NG);
    const uint32_t dH = tmem + dcol;
    const uint32_t dG = tmem + dcol + D::NHP;
    const uint64_t dA = sdesc(aBase, aLBO, aSBO), dB = sdesc(bBase, LBO_STD, SBO_STD);
    const uint64_t oS = (uint64_t)(aStride >> 4), oBl = (uint64_t)(D::B_TILE >> 4);
    const uint64_t oPh = (uint64_t)(((D::NHP / 8) * SBO_STD) >> 4);
#pragma unroll
    for (int ks = 0; ks < KD / 16; ++ks) {
        const uint64_t ao = (uint64_t)((ks * 2 * aLBO) >> 4), bo = (uint64_t)((ks * 2 * LBO_STD) >> 4);
        const uint32_t acc0 = (first && ks == 0) ? 0u : 1u;
        const uint64_t aWh = dA + ao, aWl = aWh + oS, aUh = aWh + 2 * oS, aUl = aWh + 3 * oS;
        if (HG == 0) {
            mma_bf16(dH, aWh, dB + bo, idH, acc0);
            mma_bf16(dH, aWh, dB + oBl + bo, idH, 1u);
            mma_bf16(dH, aWl, dB + bo, idH, 1u);
        } else {
            mma_bf16(dG, aUh, dB + oPh + bo, idG, acc0);
            mma_bf16(dG + D::NG, aUh, dB + oPh + oBl + bo, idG, acc0);   // lo products: own columns
            mma_bf16(dG + D::NG, aUl, dB + oPh + bo, idG, 1u);
        }
    }
}

// P side with stacked B rows [hi_H | lo_H | hi_G | lo_G] (one tile of 2 NT rows):
// the hi.hi and hi.lo products come from one MMA each for the Hessian (N = 2NHP)
// and the gradient (N = 2NG), into side-by-side TMEM columns; lo.hi adds into
// the hi.hi columns.  Eight MMAs per 32-deep stage instead of twelve.
template <int K, bool HESS>
__device__ __forceinline__ void issue_stage_stacked(uint32_t tmem, int dcol, uint32_t aBase, int aStride, int aLBO,
                                                    int aSBO, uint32_t bBase, bool first) {
    using D = TcDims<K>;
    constexpr uint32_t idH2 = idesc_bf16(2 * D::NHP), idH = idesc_bf16(D::NHP);
    constexpr uint32_t idG2 = idesc_f16(2 * D::NG), idG = idesc_f16(D::NG);
    const uint32_t dH = tmem + dcol;
    const uint32_t dG = tmem + dcol + 2 * D::NHP;
    const uint64_t dA = sdesc(aBase, aLBO, aSBO), dB = sdesc(bBase, LBO_STD, SBO_STD);
    const uint64_t oS = (uint64_t)(aStride >> 4);
    const uint64_t oG = (uint64_t)(((2 * D::NHP / 8) * SBO_STD) >> 4);
#pragma unroll
    for (int ks = 0; ks < KD / 16; ++ks) {
        const uint64_t ao = (uint64_t)((ks * 2 * aLBO) >> 4), bo = (uint64_t)((ks * 2 * LBO_STD) >> 4);
        const uint32_t acc0 = (first && ks == 0) ? 0u : 1u;
        const uint64_t aWh = dA + ao, aWl = aWh + oS, aUh = aWh + 2 * oS, aUl = aWh + 3 * oS;
        // lo.hi adds into the hi.lo columns, so that the large hi.hi sums are
        // written once per k-step (every MMA write rounds its accumulator,
        // not to nearest)
        if (HESS) {
            mma_bf16(dH, aWh, dB + bo, idH2, acc0);
            mma_bf16(dH + D::NHP, aWl, dB + bo, idH, 1u);
        }
        mma_bf16(dG, aUh, dB + oG + bo, idG2, acc0);
        mma_bf16(dG + D::NG, aUl, dB + oG + bo, idG, 1u);
    }
}

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

// ------------------------------------------------------------------ images
// B tile rows of one 8-deep reduction group kg from the 8 K-vectors v[e]
// (e = reduction index within the group): rows n < NH are the products
// v[k] v[k2] (bf16 hi/lo), rows NHP.. NHP+K-1 the scaled vector (fp16 hi/lo),
// other rows zero.  Row n's 16-byte hi chunk goes to
// base + (n/8)*SBO + kg*LBO + (n%8)*16, the lo chunk B_TILE further.
// STACK (P side): physical rows [hi_H (NHP) | lo_H (NHP) | hi_G (NG) | lo_G (NG)]
// in one tile of 2 NT rows instead of a hi tile and a lo tile.
template <int K, bool STACK>
__device__ __forceinline__ void put_b_row(uint8_t* base, int kg, int n, const uint32_t (&h)[4], const uint32_t (&l)[4]) {
    using D = TcDims<K>;
    int ph = n, pl = n;
    if (STACK) {
        ph = n < D::NHP ? n : 2 * D::NHP + (n - D::NHP);
        pl = n < D::NHP ? D::NHP + n : 2 * D::NHP + D::NG + (n - D::NHP);
    }
    uint8_t* dh = base + (ph >> 3) * SBO_STD + kg * LBO_STD + (ph & 7) * 16;
    uint8_t* dl = STACK ? base + (pl >> 3) * SBO_STD + kg * LBO_STD + (pl & 7) * 16 : dh + D::B_TILE;
    *reinterpret_cast<uint4*>(dh) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4*>(dl) = make_uint4(l[0], l[1], l[2], l[3]);
}

template <int K, bool STACK>
__device__ __forceinline__ void write_b_rows(const float (&v)[8][K], uint8_t* base, int kg) {
    using D = TcDims<K>;
#pragma unroll
    for (int k = 0; k < K; ++k) {
#pragma unroll
        for (int k2 = k; k2 < K; ++k2) {
            uint32_t h[4], l[4];
#pragma unroll
            for (int e = 0; e < 4; ++e)
                split2(W_UNDO * (v[2 * e][k] * v[2 * e][k2]), W_UNDO * (v[2 * e + 1][k] * v[2 * e + 1][k2]), h[e],
                       l[e]);
            put_b_row<K, STACK>(base, kg, tri_idx<K>(k, k2), h, l);
        }
    }
    const uint32_t z[4] = {0u, 0u, 0u, 0u};
    for (int n = D::NH; n < D::NHP; ++n) put_b_row<K, STACK>(base, kg, n, z, z);
#pragma unroll
    for (int kk = 0; kk < D::NG; ++kk) {
        uint32_t h[4], l[4];
        const int kc = kk < K ? kk : 0;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float a0 = kk < K ? v[2 * e][kc] * GB_SCALE : 0.f;
            const float a1 = kk < K ? v[2 * e + 1][kc] * GB_SCALE : 0.f;
            split2_f16(a0, a1, h[e], l[e]);
        }
        put_b_row<K, STACK>(base, kg, D::NHP + kk, h, l);
    }
}

// Q-side image of word column jw (blocks 8jw..8jw+7, haplotype columns
// m = 32jw..32jw+31); thread (jw, kg) covers columns 8kg..8kg+7 of it.
// Columns past 4J read p = 0.25 (their class nibbles are padding).
template <int K>
__global__ void __launch_bounds__(128) k_qimg(const double* __restrict__ p, int64_t J, int JW, uint8_t* __restrict__ img) {
    using QD = QpDims<K>;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)JW * 4) return;
    const int64_t jw = t >> 2;
    const int kg = (int)(t & 3);
    uint8_t* base = img + jw * qimg_bytes<K>();
    const int64_t plimit = J * 4 * K;
    float v[8][K];
#pragma unroll
    for (int e = 0; e < 8; ++e)
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int64_t g = (32 * jw + 8 * kg + e) * K + k;
            v[e][k] = g < plimit ? (float)p[g] : 0.25f;
        }
    write_b_rows<K, false>(v, base, kg);
    // tf32 hi/lo p tile of the qp MMA: rows m (32), reduction k (KP, zero-padded)
    uint8_t* bq = base + 2 * TcDims<K>::B_TILE;
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const int m = 8 * kg + e;
#pragma unroll
        for (int k = 0; k < QD::KP; ++k) {
            const float x = k < K ? v[e][k < K ? k : 0] : 0.f;
            const float hi = tf32_round(x), lo = tf32_round(x - hi);
            const int off = (m >> 3) * QD::SBO + (k >> 2) * 128 + (m & 7) * 16 + (k & 3) * 4;
            *reinterpret_cast<float*>(bq + off) = hi;
            *reinterpret_cast<float*>(bq + QD::B_T + off) = lo;
        }
    }
}

// P-side image of the 32 individuals of group g; thread (g, kg) covers
// individuals 32g + 8kg .. +7.  Individuals past I read q = 1/K (their class
// nibbles are padding).
template <int K>
__global__ void __launch_bounds__(128) k_pimg(const double* __restrict__ q, int64_t I, uint8_t* __restrict__ img) {
    constexpr int QSTR = qstr<K>();
    const int64_t ng = (I + KD - 1) / KD;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ng * 4) return;
    const int64_t g = t >> 2;
    const int kg = (int)(t & 3);
    uint8_t* base = img + g * pimg_bytes<K>();
    float v[8][K];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const int64_t i = KD * g + 8 * kg + e;
#pragma unroll
        for (int k = 0; k < K; ++k) v[e][k] = i < I ? (float)q[(int64_t)K * i + k] : 1.f / K;
    }
    write_b_rows<K, true>(v, base, kg);
    float* rows = reinterpret_cast<float*>(base + 2 * TcDims<K>::B_TILE);
#pragma unroll
    for (int e = 0; e < 8; ++e)
#pragma unroll
        for (int k = 0; k < QSTR; ++k)
            rows[qrow_slot(8 * kg + e) * QSTR + k] = (k >> 1) < K ? v[e][(k >> 1) < K ? (k >> 1) : 0] : 0.f;
}

// ------------------------------------------------------------------ shared helpers
// n_mma: issuers that commit each stage to mma_done; n_flush: those that
// commit each accumulator window to flush_done
__device__ __forceinline__ void init_sync(Sync* sy, int tid, int n_mma, int n_flush) {
    if (tid == 0) {
        for (int r = 0; r < RING; ++r) mbar_init(&sy->full[r], 1);
        for (int r = 0; r < QRING; ++r) mbar_init(&sy->fullq[r], 1);
        sy->loadedq = 0;
        mbar_init(&sy->mma_done[0], n_mma); mbar_init(&sy->mma_done[1], n_mma);
        mbar_init(&sy->flush_done[0], n_flush); mbar_init(&sy->flush_done[1], n_flush);
        mbar_init(&sy->gen_full[0], TC_THREADS / 32); mbar_init(&sy->gen_full[1], TC_THREADS / 32);
        mbar_init(&sy->qp_done[0], 1); mbar_init(&sy->qp_done[1], 1);
        sy->bad = 0;
        sy->issued = 0;
        sy->loaded = 0;
        sy->arrived[0] = 0;
        sy->arrived[1] = 0;
        sy->started[0] = 0;
        sy->started[1] = 0;
        mbar_fence_init();
    }
}

__device__ __forceinline__ void expect_tx(uint64_t* mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(smem_u32(mbar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_copy(uint32_t dst, const void* src, uint32_t bytes, uint64_t* mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(dst), "l"(src), "r"(bytes), "r"(smem_u32(mbar)) : "memory");
}

// Window bookkeeping after a stage's MMAs were issued by this thread.
__device__ __forceinline__ void commit_stage(Sync* sy, int s, int ns, int b, bool window = true) {
    const int d = (s / TC_FLUSH) & 1;
    commit(&sy->mma_done[b]);
    if (window && ((s % TC_FLUSH) == TC_FLUSH - 1 || s == ns - 1)) commit(&sy->flush_done[d]);
    atomicMax(&sy->issued, s + 1);
}

// Every generator warp has written its part of stage s's A tiles (buffer b):
// one arrival per warp, after the tiles are made visible to the tensor core.
__device__ __forceinline__ void arrive_generated(Sync* sy, int b) {
    fence_async_smem();
    fence_before();
    __syncwarp();
    if ((threadIdx.x & 31) == 0) mbar_arrive(&sy->gen_full[b]);
}
// An issuer (lane 0 of a fixed warp) waits until the whole stage is generated.
__device__ __forceinline__ bool wait_generated(Sync* sy, int s, int b, double* slots, long long budget) {
    if (!mbar_wait(&sy->gen_full[b], (s >> 1) & 1, budget)) { set_bad(sy, slots); return false; }
    fence_after();
    return true;
}

// Fold of TMEM window w at stage (w+1)*TC_FLUSH + FOLD_OFF: half a window
// after its last MMAs were issued, so that they are done and no warp waits,
// and before window w+2 reuses its columns (issued at stage (w+2)*TC_FLUSH,
// once every thread has arrived there).
constexpr int FOLD_OFF = TC_FLUSH / 2;
template <int K, bool STACK>
__device__ __forceinline__ void maybe_fold(Sync* sy, double* slots, long long budget, int hf, int s, uint32_t taddr_lane, float* acc,
                                           float* comp) {
    using D = TcDims<K>;
    constexpr int WC = STACK ? D::WS : D::WQ;   // TMEM columns per window
    if (s >= TC_FLUSH + FOLD_OFF && (s - FOLD_OFF) % TC_FLUSH == 0) {
        const int wp = (s - FOLD_OFF) / TC_FLUSH - 1;
        const bool ok = __all_sync(0xffffffffu, mbar_wait(&sy->flush_done[wp & 1], (wp >> 1) & 1, budget));
        if (!ok) set_bad(sy, slots);
        else {
            fence_after();
            fold_half<K, STACK>(hf, taddr_lane, (wp & 1) * WC, acc, comp);
        }
        fence_before();
    }
}

template <int K, bool STACK>
__device__ __forceinline__ void final_fold(Sync* sy, double* slots, long long budget, int hf, int ns, uint32_t taddr_lane, float* acc,
                                           float* comp) {
    using D = TcDims<K>;
    constexpr int WC = STACK ? D::WS : D::WQ;
    __syncthreads();
    if (ns > 0 && !is_bad(sy)) {
        // windows not folded in the loop: the last one and possibly the one before
        const int wl = (ns - 1) / TC_FLUSH;
        const int nf = ns - 1 >= FOLD_OFF ? (ns - 1 - FOLD_OFF) / TC_FLUSH : 0;
        for (int w = nf; w <= wl; ++w) {
            const bool ok = __all_sync(0xffffffffu, mbar_wait(&sy->flush_done[w & 1], (w >> 1) & 1, budget));
            if (!ok) { set_bad(sy, slots); break; }
            fence_after();
            fold_half<K, STACK>(hf, taddr_lane, (w & 1) * WC, acc, comp);
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
// tile, issued two stages ahead; each thread reads its row's 16 values.

// One pair from its qp: U and W, both times U_SCALE.
template <bool HESS>
__device__ __forceinline__ void gen_pair_qp(unsigned nib, const float* qp, float* U4, float* W4, const float4* tab) {
    pair_u_tab(nib, qp, U4, tab, U_SCALE);          // U * U_SCALE
#pragma unroll
    for (int h = 0; h < 4; ++h)
        if (HESS) W4[h] = U4[h] * rcp_approx(qp[h]);   // W * U_SCALE
}

template <int K, bool HESS>
__global__ void __launch_bounds__(TC_THREADS, TcDims<K>::MINB) k_accum_q_tc(PassArgs a) {
    using D = TcDims<K>;
    using QD = QpDims<K>;
    constexpr int GB = qimg_bytes<K>();
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const uint32_t sA = smem_u32(smem);                              // [2][4][A_TILE_STD]
    constexpr int GBM = 2 * D::B_TILE;                               // main ring slot: the B tile
    constexpr int GBQ = 2 * QD::B_T;                                 // qp ring slot: tf32 p tile
    const uint32_t sAq = sA + 2 * 4 * A_TILE_STD;                    // [2 hi/lo][A_T]
    const uint32_t sR = sAq + 2 * QD::A_T;                           // ring [RING][GBM]
    const uint32_t sRq = sR + RING * GBM;                            // ring [QRING][GBQ]
    uint32_t* SW = (uint32_t*)(smem + (sRq - sA) + QRING * GBQ);     // [RING][128]
    Sync* sy = (Sync*)(SW + RING * 128);
    __shared__ float4 s_snp[4];
    const long long budget = a.budget;

    const int tid = threadIdx.x, warp = tid >> 5;
    const int r = tid & 127, hf = tid >> 7;
    const int64_t i = (int64_t)blockIdx.x * 128 + r;
    const bool active = i < a.I;
    const int w0 = blockIdx.y * a.per_chunk;
    const int ns = min(a.JW, w0 + a.per_chunk) - w0;     // one word per stage
    const int64_t i0 = (int64_t)blockIdx.x * 128;
    snp_table_init(s_snp, tid);

    // stage t's inputs: the word column's B tile and the CTA's 128 class words;
    // separately, 4 stages ahead, the tf32 p tile of its qp MMA
    auto load_stage = [&](int t) {
        const int slot = t % RING;
        expect_tx(&sy->full[slot], (uint32_t)(GBM + 512));
        bulk_copy(sR + slot * GBM, sy->img0 + (int64_t)t * GB, GBM, &sy->full[slot]);
        bulk_copy(smem_u32(SW + slot * 128), sy->g0 + (int64_t)t * sy->gstride, 512, &sy->full[slot]);
        atomicMax(&sy->loaded, t + 1);   // refills come from different warps
    };
    auto load_qtile = [&](int t) {
        const int slot = t % QRING;
        expect_tx(&sy->fullq[slot], (uint32_t)GBQ);
        bulk_copy(sRq + slot * GBQ, sy->img0 + (int64_t)t * GB + GBM, GBQ, &sy->fullq[slot]);
        atomicMax(&sy->loadedq, t + 1);
    };

    if (warp == 0) tmem_alloc<QD::TCOLS>(&sy->tslot);
    init_sync(sy, tid, HESS ? 3 : 2, HESS ? 2 : 1);   // issuers: Hessian, gradient, qp
    if (tid == 0) {
        sy->img0 = a.img + (int64_t)w0 * GB;
        sy->g0 = a.G + (int64_t)w0 * a.Ipad + i0;
        sy->gstride = a.Ipad;
    }
    // zero the q tile (reduction padding k >= K stays zero)
    for (int t = tid; t < (2 * QD::A_T) / 4; t += TC_THREADS)
        asm volatile("st.shared.b32 [%0], %1;" :: "r"(sAq + 4 * t), "r"(0u) : "memory");
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = sy->tslot;
    const uint32_t tq = tmem + 2 * D::WQ;                 // qp tiles: columns [2WQ, 2WQ + 64)
    const uint32_t taddr_lane = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
    if (tid == 0) {
        for (int t = 0; t < RING && t < ns; ++t) load_stage(t);
        for (int t = 0; t < QRING && t < ns; ++t) load_qtile(t);
    }

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

    fence_async_smem();
    fence_before();
    __syncthreads();
    // qp of stages 0 and 1; stage t's qp is then issued at stage t-2
    if (tid == 0) {
        for (int t = 0; t < 2 && t < ns; ++t) {
            if (!mbar_wait(&sy->fullq[t], 0, budget)) { set_bad(sy, a.slots); break; }
            fence_after();
            issue_qp<K>(tq + t * 32, sAq, sRq + t * GBQ);
            commit(&sy->qp_done[t]);
        }
    }

    for (int s = 0; s < ns; ++s) {
        const int b = s & 1, slot = s % RING;
        if (!mbar_wait(&sy->full[slot], (s / RING) & 1, budget)) set_bad(sy, a.slots);
        // A buffer b was last read by the MMAs of stage s-2
        if (s >= 2 && !is_bad(sy))
            if (!mbar_wait(&sy->mma_done[b], ((s - 2) >> 1) & 1, budget)) set_bad(sy, a.slots);
        if (is_bad(sy)) break;
        // ring refill: the slot of stage s-2 is free (its MMAs are done -- just
        // waited for -- and they were issued after every thread had read it).
        // The first warp here loads it, which keeps the refill off the last
        // arriving warp of stage s-1 (the MMA issuer, still issuing).
        // The qp tile slot of stage s is free too: its MMA (issued with the
        // MMAs of stage s-2) is done.
        if (s >= 2 && first_at_stage(&sy->started[b])) {
            if (s - 2 + RING < ns) load_stage(s - 2 + RING);
            if (s + QRING < ns) load_qtile(s + QRING);
        }
        // this stage's qp: 16 columns of this thread's row.  From stage 2 on it
        // was issued with the MMAs of stage s-2 and is covered by their
        // mma_done, just waited for; stages 0 and 1 wait for the prologue's.
        // Both loads go out before one wait, with the class word read between.
        float qpv[16];
        uint32_t word;
        {
            if (s < 2) {
                const bool ok = __all_sync(0xffffffffu, mbar_wait(&sy->qp_done[b], 0, budget));
                if (!ok) { set_bad(sy, a.slots); break; }
            }
            fence_after();
            uint32_t raw[16];
            tmem_ld8_async(taddr_lane + (uint32_t)(2 * D::WQ + b * 32 + hf * 16), raw);
            tmem_ld8_async(taddr_lane + (uint32_t)(2 * D::WQ + b * 32 + hf * 16 + 8), raw + 8);
            word = SW[slot * 128 + r];
            tmem_wait_ld();
#pragma unroll
            for (int t = 0; t < 16; ++t) qpv[t] = __uint_as_float(raw[t]);
        }
        const uint32_t aB = sA + b * 4 * A_TILE_STD;
#pragma unroll
        for (int t2 = 0; t2 < 2; ++t2) {
            float W[8], U[8];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int bb = 2 * t2 + e;                    // block within this thread's half
                gen_pair_qp<HESS>((word >> (4 * (hf * 4 + bb))) & 0xFu, qpv + 4 * bb, U + 4 * e, W + 4 * e, s_snp);
            }
            const uint32_t off = (r >> 3) * SBO_STD + (hf * 2 + t2) * LBO_STD + (r & 7) * 16;
            uint32_t wh[4], wl[4], uh[4], ul[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                if (HESS) split2(W[2 * e], W[2 * e + 1], wh[e], wl[e]);
                split2_f16(U[2 * e], U[2 * e + 1], uh[e], ul[e]);
            }
            if (HESS) {
                sts128(aB + off, wh[0], wh[1], wh[2], wh[3]);
                sts128(aB + A_TILE_STD + off, wl[0], wl[1], wl[2], wl[3]);
            }
            sts128(aB + 2 * A_TILE_STD + off, uh[0], uh[1], uh[2], uh[3]);
            sts128(aB + 3 * A_TILE_STD + off, ul[0], ul[1], ul[2], ul[3]);
        }
        arrive_generated(sy, b);
        // Three issuers, lane 0 of warps 0, 2 and 4, each with its own TMEM
        // columns: the Hessian MMAs, the gradient MMAs, and the qp MMA of stage
        // s+2 into this stage's qp columns (every thread has read them).  Each
        // commits to mma_done, which therefore also covers the qp MMA.
        if ((tid & 31) == 0 && (warp == 2 || warp == 4 || (HESS && warp == 0))) {
            if (wait_generated(sy, s, b, a.slots, budget)) {
                const int d = (s / TC_FLUSH) & 1;
                if (warp == 4) {
                    if (s + 2 < ns) {
                        const int qs = (s + 2) % QRING;
                        if (!mbar_wait(&sy->fullq[qs], ((s + 2) / QRING) & 1, budget)) set_bad(sy, a.slots);
                        else issue_qp<K>(tq + b * 32, sAq, sRq + qs * GBQ);
                    }
                    commit_stage(sy, s, ns, b, false);
                    // the qp tile slots of stages 0 and 1 (their MMAs came from the
                    // prologue, every thread waited for them); later ones are
                    // refilled by the first warp of the stage
                    if (s < 2 && s + QRING < ns) load_qtile(s + QRING);
                } else {
                    const bool first = (s % TC_FLUSH) == 0;
                    if (warp == 0)
                        issue_stage_group<K, 0>(tmem, d * D::WQ, aB, A_TILE_STD, LBO_STD, SBO_STD, sR + slot * GBM, first);
                    else
                        issue_stage_group<K, 1>(tmem, d * D::WQ, aB, A_TILE_STD, LBO_STD, SBO_STD, sR + slot * GBM, first);
                    commit_stage(sy, s, ns, b);
                }
            }
        }
        maybe_fold<K, false>(sy, a.slots, budget, hf, s, taddr_lane, acc, comp);
    }
    final_fold<K, false>(sy, a.slots, budget, hf, ns, taddr_lane, acc, comp);
    // write partials: v < K gradient, v = K + tri index Hessian
    constexpr int NV = K + (HESS ? D::NH : 0);
    double* out = a.part + (int64_t)blockIdx.y * NV * a.Ipad;
#pragma unroll
    for (int c = 0; c < D::HALF; ++c) {
        const int col = hf * D::HALF + c;
        if (col < D::NH) {
            if (HESS) out[(int64_t)(K + col) * a.Ipad + i] = (double)acc[c];
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

// One (individual, block) pair: qp from q and p (4K values), then U and W,
// both times U_SCALE.  qd[k] = (q_k, q_k); pr2[2k] = (p[k,4j], p[k,4j+1]),
// pr2[2k+1] = (p[k,4j+2], p[k,4j+3]): the packed FMAs form qp_h for h pairs
// in the order of the fmaf chain sum_k q_k p[k,m].
template <int K, bool HESS>
__device__ __forceinline__ void gen_pair(unsigned nib, const uint64_t* qd, const uint64_t* pr2, float* U4, float* W4,
                                         const float4* tab) {
    uint64_t z01 = 0ull, z23 = 0ull;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        z01 = f2_fma(qd[k], pr2[2 * k], z01);
        z23 = f2_fma(qd[k], pr2[2 * k + 1], z23);
    }
    float qp[4];
    f2_split(z01, qp[0], qp[1]);
    f2_split(z23, qp[2], qp[3]);
    pair_u_tab(nib, qp, U4, tab, U_SCALE);          // U * U_SCALE
#pragma unroll
    for (int h = 0; h < 4; ++h)
        if (HESS) W4[h] = U4[h] * rcp_approx(qp[h]);   // W * U_SCALE
}

template <int K, bool HESS>
__global__ void __launch_bounds__(TC_THREADS, TcDims<K>::MINB) k_accum_p_tc(PassArgs a) {
    using D = TcDims<K>;
    constexpr int QSTR = qstr<K>();
    constexpr int GB = pimg_bytes<K>();
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // aligned by an offset from the shared array (no integer round trip), so
    // that the compiler keeps every derived pointer in the shared space:
    // 32-bit shared loads instead of generic ones (fewer registers, no spills)
    uint8_t* smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const uint32_t sA = smem_u32(smem);                              // [2][4][A_TILE_PAD]
    const uint32_t sR = sA + 2 * 4 * A_TILE_PAD;                     // ring [RING][GB]
    uint32_t* SW = (uint32_t*)(smem + (sR - sA) + RING * GB);        // [RING][4][KD]
    Sync* sy = (Sync*)(SW + RING * 4 * KD);
    __shared__ float4 s_snp[4];
    const long long budget = a.budget;

    const int tid = threadIdx.x, warp = tid >> 5;
    const int jl = tid >> 3, ig = tid & 7;
    const int hf = tid >> 7;
    const int64_t j = (int64_t)blockIdx.x * 32 + jl;
    const bool valid = j < a.J;
    const int64_t i0 = (int64_t)blockIdx.y * a.per_chunk;
    const int64_t i1 = min(a.I, i0 + (int64_t)a.per_chunk);
    const int ns = (int)((i1 - i0 + KD - 1) / KD);
    const int64_t g0 = i0 / KD;
    const int64_t jw0 = (int64_t)blockIdx.x * 4;
    const int nwc = (int)min((int64_t)4, (int64_t)a.JW - jw0);     // word columns inside the matrix
    snp_table_init(s_snp, tid);

    // stage t's inputs: the 32 individuals' image and their class words of the
    // CTA's word columns (columns past JW are never read: their blocks are
    // past J and evaluate as padding)
    auto load_stage = [&](int t) {
        const int slot = t % RING;
        expect_tx(&sy->full[slot], sy->tx);
        bulk_copy(sR + slot * GB, sy->img0 + (int64_t)t * GB, GB, &sy->full[slot]);
        for (int w = 0; w < sy->nwc; ++w)
            bulk_copy(smem_u32(SW + (slot * 4 + w) * KD), sy->g0 + w * sy->gstride + (int64_t)KD * t, 128,
                      &sy->full[slot]);
        atomicMax(&sy->loaded, t + 1);   // refills come from different warps
    };

    if (warp == 0) tmem_alloc<D::TCOLS_S>(&sy->tslot);
    init_sync(sy, tid, 1, 1);
    if (tid == 0) {
        sy->img0 = a.img + g0 * GB;
        sy->g0 = a.G + jw0 * a.Ipad + i0;
        sy->gstride = a.Ipad;
        sy->nwc = nwc;
        sy->tx = (uint32_t)(GB + 128 * nwc);
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = sy->tslot;
    const uint32_t taddr_lane = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
    if (tid == 0)
        for (int t = 0; t < RING && t < ns; ++t) load_stage(t);

    uint64_t pr2[2 * K];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const double* pj = a.p + (int64_t)K * 4 * j + k;
        pr2[2 * k] = valid ? f2_pack((float)pj[0], (float)pj[K]) : f2_dup(0.25f);
        pr2[2 * k + 1] = valid ? f2_pack((float)pj[2 * K], (float)pj[3 * K]) : f2_dup(0.25f);
    }
    float acc[D::HALF], comp[D::NG];
#pragma unroll
    for (int c = 0; c < D::HALF; ++c) acc[c] = 0.f;
#pragma unroll
    for (int c = 0; c < D::NG; ++c) comp[c] = 0.f;
    const int bsh = 4 * (jl & 7);

    for (int s = 0; s < ns; ++s) {
        const int b = s & 1, slot = s % RING;
        if (!mbar_wait(&sy->full[slot], (s / RING) & 1, budget)) set_bad(sy, a.slots);
        if (s >= 2 && !is_bad(sy))
            if (!mbar_wait(&sy->mma_done[b], ((s - 2) >> 1) & 1, budget)) set_bad(sy, a.slots);
        if (is_bad(sy)) break;
        // ring refill by the first warp here (see the Q side)
        if (s >= 2 && s - 2 + RING < ns && first_at_stage(&sy->started[b])) load_stage(s - 2 + RING);
        const float* Qs = reinterpret_cast<const float*>(smem + (sR - sA) + slot * GB + 2 * D::B_TILE);
        const uint32_t* Ws = SW + slot * 4 * KD + (jl >> 3) * KD;
        // A = W^T tile: rows m = 4*jl + h, reduction over the stage's individuals
        float W[4][4], U[4][4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int ii = ig * 4 + e;
            const unsigned nib = valid ? (Ws[ii] >> bsh) & 0xFu : HX_PAD_NIBBLE;
            uint64_t qd[(K + 1) / 2 * 2];
            const ulonglong2* q2 = reinterpret_cast<const ulonglong2*>(Qs + qrow_slot(ii) * QSTR);
#pragma unroll
            for (int c = 0; c < (K + 1) / 2; ++c) {
                const ulonglong2 x = q2[c];
                qd[2 * c] = x.x;
                qd[2 * c + 1] = x.y;
            }
            float u4[4], w4[4];
            gen_pair<K, HESS>(nib, qd, pr2, u4, w4, s_snp);
#pragma unroll
            for (int h = 0; h < 4; ++h) { U[h][e] = u4[h]; if (HESS) W[h][e] = w4[h]; }
        }
        const uint32_t aB = sA + b * 4 * A_TILE_PAD;
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            const int m = 4 * jl + h;
            const uint32_t off = (m >> 3) * SBO_PAD + (ig >> 1) * LBO_PAD + (m & 7) * 16 + (ig & 1) * 8;
            uint32_t wh[2], wl[2], uh[2], ul[2];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                if (HESS) split2(W[h][2 * e], W[h][2 * e + 1], wh[e], wl[e]);
                split2_f16(U[h][2 * e], U[h][2 * e + 1], uh[e], ul[e]);
            }
            if (HESS) {
                asm volatile("st.shared.v2.b32 [%0], {%1, %2};" :: "r"(aB + off), "r"(wh[0]), "r"(wh[1]) : "memory");
                asm volatile("st.shared.v2.b32 [%0], {%1, %2};" :: "r"(aB + A_TILE_PAD + off), "r"(wl[0]), "r"(wl[1]) : "memory");
            }
            asm volatile("st.shared.v2.b32 [%0], {%1, %2};" :: "r"(aB + 2 * A_TILE_PAD + off), "r"(uh[0]), "r"(uh[1]) : "memory");
            asm volatile("st.shared.v2.b32 [%0], {%1, %2};" :: "r"(aB + 3 * A_TILE_PAD + off), "r"(ul[0]), "r"(ul[1]) : "memory");
        }
        // One issuer, the last warp to arrive: on this side two issuers were
        // measured slower (the SM's MMA issue rate, not one thread, is the
        // limit, and the fixed issuer warps fall behind on generation)
        fence_async_smem();
        fence_before();
        if (arrive_last(&sy->arrived[b])) {
            fence_after();
            const int d = (s / TC_FLUSH) & 1;
            issue_stage_stacked<K, HESS>(tmem, d * D::WS, aB, A_TILE_PAD, LBO_PAD, SBO_PAD, sR + slot * GB,
                                         (s % TC_FLUSH) == 0);
            commit_stage(sy, s, ns, b);
        }
        maybe_fold<K, true>(sy, a.slots, budget, hf, s, taddr_lane, acc, comp);
    }
    final_fold<K, true>(sy, a.slots, budget, hf, ns, taddr_lane, acc, comp);
    // rows m of this CTA: TMEM lane r
    const int r = tid & 127;
    const int64_t m = (int64_t)blockIdx.x * 128 + r;
    if (m < 4 * a.J) {
        constexpr int NV = K + (HESS ? D::NH : 0);
        const int64_t rows = 4 * a.J;
#pragma unroll
        for (int c = 0; c < D::HALF; ++c) {
            const int col = hf * D::HALF + c;
            if (col < D::NH) {
                if (!HESS) continue;
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
        tmem_dealloc<D::TCOLS_S>(tmem);
    }
}

template <int K> constexpr size_t smem_q() {
    using QD = QpDims<K>;
    return 1024 + 2 * 4 * A_TILE_STD + 2 * QD::A_T + RING * 2 * TcDims<K>::B_TILE + QRING * 2 * QD::B_T +
           RING * 128 * 4 + sizeof(Sync);
}
template <int K> constexpr size_t smem_p() {
    return 1024 + 2 * 4 * A_TILE_PAD + RING * pimg_bytes<K>() + RING * 4 * KD * 4 + sizeof(Sync);
}

// One entry for every host-side operation on the K instantiation.
template <int K>
cudaError_t tc_run(TcCall& c) {
    switch (c.op) {
    case TC_ATTRS: {
        cudaError_t e = cudaFuncSetAttribute(k_accum_q_tc<K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem_q<K>());
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_accum_q_tc<K, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem_q<K>());
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_accum_p_tc<K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem_p<K>());
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_accum_p_tc<K, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem_p<K>());
        return e;
    }
    case TC_RESIDENT_Q:
        c.bytes = (size_t)resident_ctas((const void*)k_accum_q_tc<K, true>, TC_THREADS, smem_q<K>(), QpDims<K>::TCOLS);
        return cudaSuccess;
    case TC_RESIDENT_P:
        c.bytes = (size_t)resident_ctas((const void*)k_accum_p_tc<K, true>, TC_THREADS, smem_p<K>(), TcDims<K>::TCOLS_S);
        return cudaSuccess;
    case TC_IMG_BYTES: {
        const int64_t JW = (c.J + 7) / 8, ng = (c.I + KD - 1) / KD;
        c.bytes = std::max((size_t)JW * qimg_bytes<K>(), (size_t)ng * pimg_bytes<K>());
        return cudaSuccess;
    }
    case TC_Q: {   // two launches: the operand image, then the pass
        const PassArgs& a = *c.a;
        const unsigned gi = (unsigned)(((int64_t)a.JW * 4 + 127) / 128);
        dim3 grid((unsigned)(a.Ipad / 128), (unsigned)a.S);
        k_qimg<K><<<gi, 128, 0, c.st>>>(a.p, a.J, a.JW, a.img);
        if (c.hess) k_accum_q_tc<K, true><<<grid, TC_THREADS, smem_q<K>(), c.st>>>(a);
        else k_accum_q_tc<K, false><<<grid, TC_THREADS, smem_q<K>(), c.st>>>(a);
        return cudaGetLastError();
    }
    case TC_P: {
        const PassArgs& a = *c.a;
        const unsigned gi = (unsigned)((((a.I + KD - 1) / KD) * 4 + 127) / 128);
        dim3 grid((unsigned)((a.J + 31) / 32), (unsigned)a.S);
        k_pimg<K><<<gi, 128, 0, c.st>>>(a.q, a.I, a.img);
        if (c.hess) k_accum_p_tc<K, true><<<grid, TC_THREADS, smem_p<K>(), c.st>>>(a);
        else k_accum_p_tc<K, false><<<grid, TC_THREADS, smem_p<K>(), c.st>>>(a);
        return cudaGetLastError();
    }
    }
    return cudaErrorInvalidValue;
}

}  // namespace
}  // namespace hx
