// hx_pass.cuh -- the streaming passes over the genotype classes (CUDA cores).
//
// Three kernels, templated on the number of ancestries K (register-resident
// accumulators) and on the arithmetic type T:
//   T = double : the plain FP64 method (the reference's arithmetic class),
//   T = float  : the mixed method (FP32 products, FP64 cross-chunk totals and
//                FP64 stage-level promotion of the gradient).
//
//   k_accum_q  : per individual i over a chunk of blocks (src/loops.jl:328-365,
//                src/cuda/kernels.jl:104-138):
//                Xtz_q[k,i]    = sum_{j,h} c_h p[k,m] / qp_h
//                XtX_q[k2,k,i] = sum_{j,h} c_h p[k,m] p[k2,m] / qp_h^2
//   k_accum_p  : per haplotype column m = 4j+h over a chunk of individuals
//                (src/loops.jl:367-403, src/cuda/kernels.jl:140-175):
//                Xtz_p[k,m]    = sum_i c_h q[k,i] / qp_h
//                XtX_p[k2,k,m] = sum_i c_h q[k,i] q[k2,i] / qp_h^2
//   k_loglik   : sum over pairs of log L (src/loops.jl:236-258,
//                src/cuda/kernels.jl:16-40), as the log of an exponent-
//                renormalised running product (one log per thread).
//
// The EM numerators of em_loop!/em_kernel! (src/loops.jl:260-295,
// src/cuda/kernels.jl:42-73) are q[k,i] * Xtz_q[k,i] and p[k,m] * Xtz_p[k,m],
// so EM runs the gradient-only instances of the two accumulation kernels.
//
// No atomics: each output element has exactly one owner thread per chunk and
// chunks are combined by a fixed-order FP64 reduction, so every pass is
// bit-reproducible run to run.
#pragma once
#include "hx_common.cuh"

namespace hx {

constexpr int ACC_THREADS = 128;
constexpr int QSTAGE_WORDS = 8;     // words (x8 blocks) of p staged per Q-side stage
constexpr int PSTAGE_IND = 128;     // individuals staged per P-side stage

struct PassArgs {
    const uint32_t* G;      // class words [JW][Ipad]
    int64_t Ipad, I, J;
    int JW;
    const double* q;        // K x I
    const double* p;        // K x 4J
    int S;                  // number of chunks (grid.y)
    int per_chunk;          // words (Q side) or individuals (P side) per chunk
    double* part;           // [S][NV][rows] partials, or null when S == 1 (P side)
    double* XtX;            // direct outputs when S == 1 (P side)
    double* Xtz;
    double* slots;          // per-context scalar block (tensor-core kernels record timeouts there)
    uint8_t* img;           // tensor-core passes: B-operand image of the pass (written by the pass)
    const float* pf;        // FP32 copy of p for the FP32 passes that stage p (or null): GB300's
                            // FP64 unit is narrow, and converting in every CTA kept it busy
    long long budget;       // tensor-core passes: clock64 cycles any one pipeline wait may take
};

template <int K> __device__ __forceinline__ constexpr int tri(int k, int k2) {
    return k * K - (k * (k - 1)) / 2 + (k2 - k);
}

// ------------------------------------------------------------------ Q side
template <int K, typename T, bool HESS>
__global__ void __launch_bounds__(ACC_THREADS)
k_accum_q(PassArgs a) {
    constexpr int NH = K * (K + 1) / 2;
    constexpr int NV = K + (HESS ? NH : 0);
    __shared__ T sp[QSTAGE_WORDS * 8 * 4 * K];
    __shared__ float4 s_snp[4];
    const int tid = threadIdx.x;
    snp_table_init(s_snp, tid);
    const int64_t i = (int64_t)blockIdx.x * ACC_THREADS + tid;
    const int w0 = blockIdx.y * a.per_chunk;
    const int w1 = min(a.JW, w0 + a.per_chunk);
    const bool active = i < a.I;
    T qi[K];
#pragma unroll
    for (int k = 0; k < K; ++k) qi[k] = active ? (T)a.q[(int64_t)K * i + k] : T(1) / T(K);
    T gin[K];
    double gout[K];
    T H[HESS ? NH : 1];
#pragma unroll
    for (int k = 0; k < K; ++k) { gin[k] = T(0); gout[k] = 0.0; }
#pragma unroll
    for (int v = 0; v < (HESS ? NH : 1); ++v) H[v] = T(0);

    for (int ws = w0; ws < w1; ws += QSTAGE_WORDS) {
        const int nw = min(QSTAGE_WORDS, w1 - ws);
        uint32_t words[QSTAGE_WORDS];
#pragma unroll
        for (int w = 0; w < QSTAGE_WORDS; ++w)
            words[w] = (w < nw) ? a.G[(int64_t)(ws + w) * a.Ipad + i] : HX_PAD_WORD;
        __syncthreads();
        const int nval = nw * 8 * 4 * K;
        const int64_t base = (int64_t)ws * 8 * 4 * K;
        const int64_t limit = a.J * 4 * K;
        for (int t = tid; t < nval; t += ACC_THREADS)
            sp[t] = (base + t < limit) ? ((sizeof(T) == 4 && a.pf) ? (T)a.pf[base + t] : (T)a.p[base + t]) : T(0.25);
        __syncthreads();
        if (active) {
            for (int w = 0; w < nw; ++w) {
                const uint32_t word = words[w];
#pragma unroll 1
                for (int b = 0; b < 8; ++b) {
                    const unsigned nib = (word >> (4 * b)) & 0xFu;
                    if (nib == NIB_MM) continue;
                    const T* pb = sp + (w * 8 + b) * 4 * K;
                    T qp[4];
#pragma unroll
                    for (int h = 0; h < 4; ++h) {
                        T s = T(0);
#pragma unroll
                        for (int k = 0; k < K; ++k) s = fma(qi[k], pb[h * K + k], s);
                        qp[h] = s;
                    }
                    T L, u[4];
                    pair_eval_t(nib, qp, L, u, s_snp);
#pragma unroll
                    for (int k = 0; k < K; ++k) {
                        T g = gin[k];
                        g = fma(u[0], pb[k], g);
                        g = fma(u[1], pb[K + k], g);
                        g = fma(u[2], pb[2 * K + k], g);
                        g = fma(u[3], pb[3 * K + k], g);
                        gin[k] = g;
                    }
                    if (HESS) {
#pragma unroll
                        for (int h = 0; h < 4; ++h) {
                            const T wh = u[h] * rcp<T>(qp[h]);
                            T t[K];
#pragma unroll
                            for (int k = 0; k < K; ++k) t[k] = wh * pb[h * K + k];
#pragma unroll
                            for (int k = 0; k < K; ++k)
#pragma unroll
                                for (int k2 = k; k2 < K; ++k2)
                                    H[tri<K>(k, k2)] = fma(t[k], pb[h * K + k2], H[tri<K>(k, k2)]);
                        }
                    }
                }
            }
        }
        // promote the stage's gradient partial to FP64 (exact for T = double)
#pragma unroll
        for (int k = 0; k < K; ++k) { gout[k] += (double)gin[k]; gin[k] = T(0); }
    }
    if (i < a.Ipad) {
        double* out = a.part + (int64_t)blockIdx.y * NV * a.Ipad;
#pragma unroll
        for (int k = 0; k < K; ++k) out[(int64_t)k * a.Ipad + i] = gout[k];
        if (HESS) {
#pragma unroll
            for (int v = 0; v < (HESS ? NH : 1); ++v) out[(int64_t)(K + v) * a.Ipad + i] = (double)H[v];
        }
    }
}

// ------------------------------------------------------------------ P side
// Thread (b, h) of a CTA owns haplotype column m = 4*(32*blockIdx.x + b) + h;
// the 4 threads of a block exchange their qp_h by warp shuffles.
template <int K, typename T, bool HESS>
__global__ void __launch_bounds__(ACC_THREADS)
k_accum_p(PassArgs a) {
    constexpr int NH = K * (K + 1) / 2;
    constexpr int NV = K + (HESS ? NH : 0);
    __shared__ T sq[PSTAGE_IND * K];
    __shared__ uint32_t sg[4 * PSTAGE_IND];
    __shared__ float4 s_snp[4];
    const int tid = threadIdx.x;
    snp_table_init(s_snp, tid);
    const int lane = tid & 31, warp = tid >> 5;
    const int b = tid >> 2, h = tid & 3;
    const int64_t j = (int64_t)blockIdx.x * 32 + b;
    const bool valid = j < a.J;
    const int64_t m = 4 * j + h;
    T pr[K];
#pragma unroll
    for (int k = 0; k < K; ++k) pr[k] = valid ? (T)a.p[(int64_t)K * m + k] : T(0.25);
    const int64_t i0 = (int64_t)blockIdx.y * a.per_chunk;
    const int64_t i1 = min(a.I, i0 + (int64_t)a.per_chunk);
    const int bsh = 4 * (b & 7);
    T gin[K];
    double gout[K];
    T H[HESS ? NH : 1];
#pragma unroll
    for (int k = 0; k < K; ++k) { gin[k] = T(0); gout[k] = 0.0; }
#pragma unroll
    for (int v = 0; v < (HESS ? NH : 1); ++v) H[v] = T(0);

    for (int64_t is = i0; is < i1; is += PSTAGE_IND) {
        const int n = (int)min((int64_t)PSTAGE_IND, i1 - is);
        __syncthreads();
        for (int t = tid; t < n * K; t += ACC_THREADS) sq[t] = (T)a.q[(int64_t)K * is + t];
        for (int t = tid; t < 4 * PSTAGE_IND; t += ACC_THREADS) {
            const int w = t / PSTAGE_IND, r = t % PSTAGE_IND;
            const int64_t jw = (int64_t)blockIdx.x * 4 + w;
            sg[t] = (r < n && jw < a.JW) ? a.G[jw * a.Ipad + is + r] : HX_PAD_WORD;
        }
        __syncthreads();
#pragma unroll 1
        for (int r = 0; r < n; ++r) {
            const unsigned nib = (sg[warp * PSTAGE_IND + r] >> bsh) & 0xFu;
            const T* qr = sq + r * K;
            T own = T(0);
#pragma unroll
            for (int k = 0; k < K; ++k) own = fma(qr[k], pr[k], own);
            T qp[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) qp[t] = __shfl_sync(0xffffffffu, own, (lane & ~3) | t);
            T L, u[4];
            pair_eval_t(nib, qp, L, u, s_snp);
            const T uh = h == 0 ? u[0] : (h == 1 ? u[1] : (h == 2 ? u[2] : u[3]));
#pragma unroll
            for (int k = 0; k < K; ++k) gin[k] = fma(uh, qr[k], gin[k]);
            if (HESS) {
                const T wh = uh * rcp<T>(own);
                T t[K];
#pragma unroll
                for (int k = 0; k < K; ++k) t[k] = wh * qr[k];
#pragma unroll
                for (int k = 0; k < K; ++k)
#pragma unroll
                    for (int k2 = k; k2 < K; ++k2) H[tri<K>(k, k2)] = fma(t[k], qr[k2], H[tri<K>(k, k2)]);
            }
        }
#pragma unroll
        for (int k = 0; k < K; ++k) { gout[k] += (double)gin[k]; gin[k] = T(0); }
    }
    if (!valid) return;
    if (a.S == 1) {
        double* X = a.XtX + (int64_t)K * K * m;
#pragma unroll
        for (int k = 0; k < K; ++k) a.Xtz[(int64_t)K * m + k] = gout[k];
        if (HESS) {
#pragma unroll
            for (int k = 0; k < K; ++k)
#pragma unroll
                for (int k2 = 0; k2 < K; ++k2)
                    X[k2 + K * k] = (double)H[k <= k2 ? tri<K>(k, k2) : tri<K>(k2, k)];
        }
    } else {
        const int64_t rows = 4 * a.J;
        double* out = a.part + (int64_t)blockIdx.y * NV * rows;
#pragma unroll
        for (int k = 0; k < K; ++k) out[(int64_t)k * rows + m] = gout[k];
        if (HESS) {
#pragma unroll
            for (int v = 0; v < (HESS ? NH : 1); ++v) out[(int64_t)(K + v) * rows + m] = (double)H[v];
        }
    }
}

// ------------------------------------------------------------------ loglik
template <int K, typename T>
__global__ void __launch_bounds__(ACC_THREADS)
k_loglik(PassArgs a) {
    __shared__ T sp[QSTAGE_WORDS * 8 * 4 * K];
    __shared__ double red[ACC_THREADS];
    __shared__ float4 s_snp[4];
    const int tid = threadIdx.x;
    snp_table_init(s_snp, tid);
    const int64_t i = (int64_t)blockIdx.x * ACC_THREADS + tid;
    const int w0 = blockIdx.y * a.per_chunk;
    const int w1 = min(a.JW, w0 + a.per_chunk);
    const bool active = i < a.I;
    T qi[K];
#pragma unroll
    for (int k = 0; k < K; ++k) qi[k] = active ? (T)a.q[(int64_t)K * i + k] : T(1) / T(K);
    T mant = T(1);
    int ex = 0;
    bool zero = false, bad = false;
    for (int ws = w0; ws < w1; ws += QSTAGE_WORDS) {
        const int nw = min(QSTAGE_WORDS, w1 - ws);
        uint32_t words[QSTAGE_WORDS];
#pragma unroll
        for (int w = 0; w < QSTAGE_WORDS; ++w)
            words[w] = (w < nw) ? a.G[(int64_t)(ws + w) * a.Ipad + i] : HX_PAD_WORD;
        __syncthreads();
        const int nval = nw * 8 * 4 * K;
        const int64_t base = (int64_t)ws * 8 * 4 * K;
        const int64_t limit = a.J * 4 * K;
        for (int t = tid; t < nval; t += ACC_THREADS)
            sp[t] = (base + t < limit) ? ((sizeof(T) == 4 && a.pf) ? (T)a.pf[base + t] : (T)a.p[base + t]) : T(0.25);
        __syncthreads();
        if (active) {
            for (int w = 0; w < nw; ++w) {
                const uint32_t word = words[w];
#pragma unroll 2
                for (int b = 0; b < 8; ++b) {
                    const unsigned nib = (word >> (4 * b)) & 0xFu;
                    if (nib == NIB_MM) continue;
                    const T* pb = sp + (w * 8 + b) * 4 * K;
                    T qp[4];
#pragma unroll
                    for (int hh = 0; hh < 4; ++hh) {
                        T s = T(0);
#pragma unroll
                        for (int k = 0; k < K; ++k) s = fma(qi[k], pb[hh * K + k], s);
                        qp[hh] = s;
                    }
                    T L = pair_lik_t(nib, qp, s_snp);
                    if (!(L > T(0))) {
                        if (L == T(0)) zero = true; else bad = true;
                        L = T(1);
                    }
                    mant = renorm(mant * L, ex);
                }
            }
        }
    }
    double v = 0.0;
    if (active) {
        v = log((double)mant) + (double)ex * 0.69314718055994530942;
        if (zero) v = -INFINITY;
        if (bad) v = NAN;
    }
    red[tid] = v;
    __syncthreads();
    for (int s = ACC_THREADS / 2; s > 0; s >>= 1) {
        if (tid < s) red[tid] += red[tid + s];
        __syncthreads();
    }
    if (tid == 0) a.part[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = red[0];
}

// ------------------------------------------------------------------ loglik, FP32
// The mixed method's log-likelihood pass (same sums as k_loglik<K, float>):
// each thread carries NU individuals (i + u ACC_THREADS) that share every
// staged p row, and forms qp for haplotype pairs (h, h+1) with packed FP32x2
// FMAs (fma.rn.f32x2: two IEEE FMAs per instruction, the same results and
// order as fmaf).  Stage rows are transposed to [block][k][h] so that one
// 16-byte load gives p[k, 4j..4j+3].

template <int K, int NU>
__global__ void __launch_bounds__(ACC_THREADS)
k_loglik2(PassArgs a) {
    __shared__ __align__(16) float spt[QSTAGE_WORDS * 8 * 4 * K];
    __shared__ double red[ACC_THREADS];
    __shared__ float4 s_snp[4];
    const int tid = threadIdx.x;
    snp_table_init(s_snp, tid);
    int64_t ii[NU];
#pragma unroll
    for (int u = 0; u < NU; ++u) ii[u] = (int64_t)blockIdx.x * NU * ACC_THREADS + u * ACC_THREADS + tid;
    const int w0 = blockIdx.y * a.per_chunk;
    const int w1 = min(a.JW, w0 + a.per_chunk);
    uint64_t qd[NU][K];
    // lmin: smallest pair likelihood (0 -> log 0 = -inf, < 0 -> NaN); chk
    // turns NaN once any likelihood is NaN or infinite (L * 0).  Flagged
    // products are replaced at the end, so no per-pair branch is needed.
    float mant[NU], lmin[NU], chk[NU];
    int ex[NU];
#pragma unroll
    for (int u = 0; u < NU; ++u) { mant[u] = 1.f; ex[u] = 0; lmin[u] = 1.f; chk[u] = 0.f; }
#pragma unroll
    for (int u = 0; u < NU; ++u)
#pragma unroll
        for (int k = 0; k < K; ++k)
            qd[u][k] = f2_dup(ii[u] < a.I ? (float)a.q[(int64_t)K * ii[u] + k] : 1.f / K);
    for (int ws = w0; ws < w1; ws += QSTAGE_WORDS) {
        const int nw = min(QSTAGE_WORDS, w1 - ws);
        uint32_t words[NU][QSTAGE_WORDS];
#pragma unroll
        for (int u = 0; u < NU; ++u)
#pragma unroll
            for (int w = 0; w < QSTAGE_WORDS; ++w)
                words[u][w] = (w < nw && ii[u] < a.Ipad) ? a.G[(int64_t)(ws + w) * a.Ipad + ii[u]] : HX_PAD_WORD;
        __syncthreads();
        const int nval = nw * 8 * 4 * K;
        const int64_t base = (int64_t)ws * 8 * 4 * K;
        const int64_t limit = a.J * 4 * K;
        for (int t = tid; t < nval; t += ACC_THREADS) {
            const int blk = t / (4 * K), r = t - blk * 4 * K, h = r / K, k = r - h * K;
            spt[blk * 4 * K + k * 4 + h] = (base + t < limit) ? (a.pf ? a.pf[base + t] : (float)a.p[base + t]) : 0.25f;
        }
        __syncthreads();
        for (int w = 0; w < nw; ++w) {
#pragma unroll 2
            for (int b = 0; b < 8; ++b) {
                const ulonglong2* pb = reinterpret_cast<const ulonglong2*>(spt + (w * 8 + b) * 4 * K);
                uint64_t z01[NU], z23[NU];
#pragma unroll
                for (int u = 0; u < NU; ++u) { z01[u] = 0ull; z23[u] = 0ull; }
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    const ulonglong2 pk = pb[k];
#pragma unroll
                    for (int u = 0; u < NU; ++u) {
                        z01[u] = f2_fma(qd[u][k], pk.x, z01[u]);
                        z23[u] = f2_fma(qd[u][k], pk.y, z23[u]);
                    }
                }
#pragma unroll
                for (int u = 0; u < NU; ++u) {
                    const unsigned nib = (words[u][w] >> (4 * b)) & 0xFu;
                    float qp[4];
                    f2_split(z01[u], qp[0], qp[1]);
                    f2_split(z23[u], qp[2], qp[3]);
                    const float L = pair_lik_tab(nib, qp, s_snp);
                    lmin[u] = fminf(lmin[u], L);
                    chk[u] = fmaf(L, 0.f, chk[u]);
                    mant[u] = renorm(mant[u] * L, ex[u]);
                }
            }
        }
    }
    double v = 0.0;
#pragma unroll
    for (int u = 0; u < NU; ++u) {
        if (ii[u] < a.I) {
            double x = log((double)mant[u]) + (double)ex[u] * 0.69314718055994530942;
            if (lmin[u] == 0.f) x = -INFINITY;
            if (lmin[u] < 0.f || chk[u] != chk[u]) x = NAN;
            v += x;
        }
    }
    red[tid] = v;
    __syncthreads();
    for (int s = ACC_THREADS / 2; s > 0; s >>= 1) {
        if (tid < s) red[tid] += red[tid + s];
        __syncthreads();
    }
    if (tid == 0) a.part[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = red[0];
}

}  // namespace hx
