// hx_lws.cu -- learned warm start of Q: features, network forward/backward,
// Adam, and the in-fit warm start.
//
// Features of individual i and ancestry k (two per pair (i, k)):
//   a[i,k] = (1/n_i) sum_j log L_ij(e_k)   -- the block log-likelihood if i
//            were entirely of ancestry k (qp_h = p[k, 4j+h]), n_i = J - dm_i
//   f1[i,k] = a[i,k] - max_k' a[i,k']     (<= 0)
//   f2[i,k] = (g[i,k] - 1) sqrt(n_i), g = Xtz_q[k,i] / (2 n_i) -- the Q
//            gradient per block at the current state (sum_k q_k g_k = 1 for
//            every i), centred and scaled by sqrt(n_i)
// Network (permutation-equivariant over k, H = 64 hidden units, FP16 weights,
// FP32 accumulation):
//   h1_k = relu(W1 x_k + b1),  m = mean_k h1_k,
//   h2_k = relu(W2 h1_k + U2 m + b2),  z_k = w3 . h2_k + b3,  q = softmax_k(z).
// Training minimises the cross-entropy -sum_k t_k log q_k against converged
// Q (soft targets); dL/dz_k = q_k - t_k.
//
// One warp per sample: lane l owns hidden units l and l + 32 of every layer.
// Weight matrices sit in shared memory as FP16 (W2 and U2 row-major [u][v]
// and transposed [v][u], so that both products read consecutive halves per
// lane).  Gradients of W2 and U2 accumulate in warp-private shared memory
// (each lane owns two rows: no atomics); the CTA's warps are summed in a fixed
// order and CTA partials are reduced in a fixed order, so every gradient is
// bit-reproducible.
#include "hx_ops.cuh"
#include "../../include/haplo_gb300.h"

#include <cuda_fp16.h>

namespace hx {
namespace {

constexpr int H = HX_LWS_HIDDEN;   // 64
// parameter layout (FP32 master copy)
constexpr int O_W1 = 0;                 // [H][2]
constexpr int O_B1 = O_W1 + 2 * H;      // [H]
constexpr int O_W2 = O_B1 + H;          // [H][H]  (row u: output unit)
constexpr int O_U2 = O_W2 + H * H;      // [H][H]
constexpr int O_B2 = O_U2 + H * H;      // [H]
constexpr int O_W3 = O_B2 + H;          // [H]
constexpr int O_B3 = O_W3 + H;          // [1]
static_assert(O_B3 + 1 <= HX_LWS_NPARAM, "parameter layout");
constexpr int LWS_WARPS = 4;
constexpr unsigned FULL = 0xffffffffu;

struct LwsSmem {
    __half W2[H * H], W2t[H * H], U2[H * H], U2t[H * H];
    float W1[2 * H], b1[H], b2[H], w3[H], b3;
};

__device__ __forceinline__ float h16(float x) { return __half2float(__float2half_rn(x)); }

__device__ void load_weights(LwsSmem* s, const float* __restrict__ P) {
    for (int t = threadIdx.x; t < H * H; t += blockDim.x) {
        const int u = t / H, v = t % H;
        const __half w = __float2half_rn(P[O_W2 + t]), uu = __float2half_rn(P[O_U2 + t]);
        s->W2[t] = w;
        s->W2t[v * H + u] = w;
        s->U2[t] = uu;
        s->U2t[v * H + u] = uu;
    }
    for (int t = threadIdx.x; t < 2 * H; t += blockDim.x) s->W1[t] = h16(P[O_W1 + t]);
    for (int t = threadIdx.x; t < H; t += blockDim.x) {
        s->b1[t] = h16(P[O_B1 + t]);
        s->b2[t] = h16(P[O_B2 + t]);
        s->w3[t] = h16(P[O_W3 + t]);
    }
    if (threadIdx.x == 0) s->b3 = h16(P[O_B3]);
}

// x[k] = (f1, f2) of one sample; fills h1, h2 (this lane's two units), q.
__device__ __forceinline__ void lws_forward(const LwsSmem* s, int K, const float* f, int lane, float (*h1)[2],
                                            float* mm, float (*h2)[2], float* q) {
    const int u0 = lane, u1 = lane + 32;
    float m0 = 0.f, m1 = 0.f;
    for (int k = 0; k < K; ++k) {
        const float x0 = f[2 * k], x1 = f[2 * k + 1];
        h1[k][0] = fmaxf(fmaf(s->W1[2 * u0], x0, fmaf(s->W1[2 * u0 + 1], x1, s->b1[u0])), 0.f);
        h1[k][1] = fmaxf(fmaf(s->W1[2 * u1], x0, fmaf(s->W1[2 * u1 + 1], x1, s->b1[u1])), 0.f);
        m0 += h1[k][0];
        m1 += h1[k][1];
    }
    const float inv = 1.f / (float)K;
    mm[0] = m0 * inv;
    mm[1] = m1 * inv;
    // context c = U2 m + b2
    float c0 = s->b2[u0], c1 = s->b2[u1];
    for (int v = 0; v < H; ++v) {
        const float mv = __shfl_sync(FULL, v < 32 ? mm[0] : mm[1], v & 31);
        c0 = fmaf(__half2float(s->U2t[v * H + u0]), mv, c0);
        c1 = fmaf(__half2float(s->U2t[v * H + u1]), mv, c1);
    }
    float zmax = -INFINITY;
    for (int k = 0; k < K; ++k) {
        float a0 = c0, a1 = c1;
        for (int v = 0; v < H; ++v) {
            const float hv = __shfl_sync(FULL, v < 32 ? h1[k][0] : h1[k][1], v & 31);
            a0 = fmaf(__half2float(s->W2t[v * H + u0]), hv, a0);
            a1 = fmaf(__half2float(s->W2t[v * H + u1]), hv, a1);
        }
        h2[k][0] = fmaxf(a0, 0.f);
        h2[k][1] = fmaxf(a1, 0.f);
        float z = fmaf(s->w3[u0], h2[k][0], s->w3[u1] * h2[k][1]);
        for (int o = 16; o > 0; o >>= 1) z += __shfl_xor_sync(FULL, z, o);
        q[k] = z + s->b3;
        zmax = fmaxf(zmax, q[k]);
    }
    float den = 0.f;
    for (int k = 0; k < K; ++k) {
        q[k] = __expf(q[k] - zmax);
        den += q[k];
    }
    const float rd = 1.f / den;
    for (int k = 0; k < K; ++k) q[k] *= rd;
}

__global__ void __launch_bounds__(32 * LWS_WARPS) k_lws_forward(const float* __restrict__ feat, int64_t n, int K,
                                                                const float* __restrict__ P, float* __restrict__ qout) {
    __shared__ LwsSmem s;
    load_weights(&s, P);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t w0 = (int64_t)blockIdx.x * LWS_WARPS + (threadIdx.x >> 5);
    const int64_t nw = (int64_t)gridDim.x * LWS_WARPS;
    float f[2 * HX_KMAX], h1[HX_KMAX][2], h2[HX_KMAX][2], mm[2], q[HX_KMAX];
    for (int64_t b = w0; b < n; b += nw) {
        for (int t = 0; t < 2 * K; ++t) f[t] = feat[(int64_t)2 * K * b + t];
        lws_forward(&s, K, f, lane, h1, mm, h2, q);
        if (lane < K) {
            float v = q[0];
            for (int k = 1; k < K; ++k) v = lane == k ? q[k] : v;
            qout[(int64_t)K * b + lane] = v;
        }
    }
}

// Samples of one training step: idx[s] (or s itself when idx is null).
// Writes per-CTA gradient partials part[blockIdx.x][NPARAM] and loss partials.
__global__ void __launch_bounds__(32 * LWS_WARPS) k_lws_grad(const float* __restrict__ feat,
                                                             const float* __restrict__ target, const int64_t* idx,
                                                             int64_t ns, int K, const float* __restrict__ P,
                                                             float* __restrict__ part, double* __restrict__ loss_part) {
    extern __shared__ __align__(16) float gacc[];   // [LWS_WARPS][2][H v][H u] (dW2, dU2 transposed)
    __shared__ LwsSmem s;
    __shared__ float small[LWS_WARPS][2 * H + 3 * H + 1];   // dW1, db1, db2, dw3, db3
    __shared__ double lsum[LWS_WARPS];
    load_weights(&s, P);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float* gW2 = gacc + (size_t)warp * 2 * H * H;
    float* gU2 = gW2 + H * H;
    for (int t = lane; t < 2 * H * H; t += 32) gW2[t] = 0.f;
    __syncthreads();
    const int u0 = lane, u1 = lane + 32;
    float dW1[2][2] = {{0.f, 0.f}, {0.f, 0.f}}, db1[2] = {0.f, 0.f}, db2[2] = {0.f, 0.f}, dw3[2] = {0.f, 0.f};
    float db3 = 0.f;
    double loss = 0.0;
    const int64_t w0 = (int64_t)blockIdx.x * LWS_WARPS + warp;
    const int64_t nw = (int64_t)gridDim.x * LWS_WARPS;
    float f[2 * HX_KMAX], h1[HX_KMAX][2], h2[HX_KMAX][2], mm[2], q[HX_KMAX], dz[HX_KMAX];
    float dh2[HX_KMAX][2];
    for (int64_t sidx = w0; sidx < ns; sidx += nw) {
        const int64_t b = idx ? idx[sidx] : sidx;
        for (int t = 0; t < 2 * K; ++t) f[t] = feat[(int64_t)2 * K * b + t];
        lws_forward(&s, K, f, lane, h1, mm, h2, q);
        float l = 0.f;
        for (int k = 0; k < K; ++k) {
            const float t = target[(int64_t)K * b + k];
            dz[k] = q[k] - t;
            l -= t * __logf(fmaxf(q[k], 1e-30f));
        }
        loss += (double)l;
        float s0 = 0.f, s1 = 0.f;
        for (int k = 0; k < K; ++k) {
            dw3[0] = fmaf(dz[k], h2[k][0], dw3[0]);
            dw3[1] = fmaf(dz[k], h2[k][1], dw3[1]);
            db3 += dz[k];
            dh2[k][0] = h2[k][0] > 0.f ? dz[k] * s.w3[u0] : 0.f;
            dh2[k][1] = h2[k][1] > 0.f ? dz[k] * s.w3[u1] : 0.f;
            s0 += dh2[k][0];
            s1 += dh2[k][1];
        }
        db2[0] += s0;
        db2[1] += s1;
        // dW2[u][v] += sum_k dh2_k[u] h1_k[v];  dU2[u][v] += s[u] m[v]
        for (int v = 0; v < H; ++v) {
            float a0 = 0.f, a1 = 0.f;
            for (int k = 0; k < K; ++k) {
                const float hv = __shfl_sync(FULL, v < 32 ? h1[k][0] : h1[k][1], v & 31);
                a0 = fmaf(dh2[k][0], hv, a0);
                a1 = fmaf(dh2[k][1], hv, a1);
            }
            gW2[v * H + u0] += a0;
            gW2[v * H + u1] += a1;
            const float mv = __shfl_sync(FULL, v < 32 ? mm[0] : mm[1], v & 31);
            gU2[v * H + u0] = fmaf(s0, mv, gU2[v * H + u0]);
            gU2[v * H + u1] = fmaf(s1, mv, gU2[v * H + u1]);
        }
        // dh1_k[v] = sum_u W2[u][v] dh2_k[u] + (1/K) sum_u U2[u][v] s[u]; this lane's v = u0, u1
        float e0 = 0.f, e1 = 0.f;
        for (int u = 0; u < H; ++u) {
            const float su = __shfl_sync(FULL, u < 32 ? s0 : s1, u & 31);
            e0 = fmaf(__half2float(s.U2[u * H + u0]), su, e0);
            e1 = fmaf(__half2float(s.U2[u * H + u1]), su, e1);
        }
        const float invK = 1.f / (float)K;
        e0 *= invK;
        e1 *= invK;
        for (int k = 0; k < K; ++k) {
            float g0 = e0, g1 = e1;
            for (int u = 0; u < H; ++u) {
                const float du = __shfl_sync(FULL, u < 32 ? dh2[k][0] : dh2[k][1], u & 31);
                g0 = fmaf(__half2float(s.W2[u * H + u0]), du, g0);
                g1 = fmaf(__half2float(s.W2[u * H + u1]), du, g1);
            }
            // through m = mean_k h1_k the context term reaches every h1_k
            g0 = h1[k][0] > 0.f ? g0 : 0.f;
            g1 = h1[k][1] > 0.f ? g1 : 0.f;
            db1[0] += g0;
            db1[1] += g1;
            dW1[0][0] = fmaf(g0, f[2 * k], dW1[0][0]);
            dW1[0][1] = fmaf(g0, f[2 * k + 1], dW1[0][1]);
            dW1[1][0] = fmaf(g1, f[2 * k], dW1[1][0]);
            dW1[1][1] = fmaf(g1, f[2 * k + 1], dW1[1][1]);
        }
    }
    // small gradients of this warp
    float* sm = small[warp];
    sm[2 * u0] = dW1[0][0]; sm[2 * u0 + 1] = dW1[0][1];
    sm[2 * u1] = dW1[1][0]; sm[2 * u1 + 1] = dW1[1][1];
    sm[2 * H + u0] = db1[0]; sm[2 * H + u1] = db1[1];
    sm[3 * H + u0] = db2[0]; sm[3 * H + u1] = db2[1];
    sm[4 * H + u0] = dw3[0]; sm[4 * H + u1] = dw3[1];
    if (lane == 0) {
        sm[5 * H] = db3;
        lsum[warp] = loss;
    }
    __syncthreads();
    // CTA partial: warps summed in a fixed order
    float* out = part + (size_t)blockIdx.x * HX_LWS_NPARAM;
    for (int t = threadIdx.x; t < H * H; t += blockDim.x) {
        const int u = t / H, v = t % H;
        float a = 0.f, c = 0.f;
        for (int w = 0; w < LWS_WARPS; ++w) {
            a += gacc[(size_t)w * 2 * H * H + v * H + u];
            c += gacc[(size_t)w * 2 * H * H + H * H + v * H + u];
        }
        out[O_W2 + t] = a;
        out[O_U2 + t] = c;
    }
    for (int t = threadIdx.x; t < 2 * H; t += blockDim.x) {
        float a = 0.f;
        for (int w = 0; w < LWS_WARPS; ++w) a += small[w][t];
        out[O_W1 + t] = a;
    }
    for (int t = threadIdx.x; t < H; t += blockDim.x) {
        float a = 0.f, c = 0.f, e = 0.f;
        for (int w = 0; w < LWS_WARPS; ++w) {
            a += small[w][2 * H + t];
            c += small[w][3 * H + t];
            e += small[w][4 * H + t];
        }
        out[O_B1 + t] = a;
        out[O_B2 + t] = c;
        out[O_W3 + t] = e;
    }
    if (threadIdx.x == 0) {
        float a = 0.f;
        double l = 0.0;
        for (int w = 0; w < LWS_WARPS; ++w) {
            a += small[w][5 * H];
            l += lsum[w];
        }
        out[O_B3] = a;
        for (int t = O_B3 + 1; t < HX_LWS_NPARAM; ++t) out[t] = 0.f;
        loss_part[blockIdx.x] = l;
    }
}

// Fixed-order sum of the CTA partials, scaled by 1/ns: grad and mean loss.
__global__ void k_lws_reduce(const float* __restrict__ part, const double* __restrict__ loss_part, int nb,
                             int64_t ns, float* __restrict__ grad, double* __restrict__ loss) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < HX_LWS_NPARAM) {
        double a = 0.0;
        for (int b = 0; b < nb; ++b) a += (double)part[(size_t)b * HX_LWS_NPARAM + t];
        grad[t] = (float)(a / (double)ns);
    }
    if (t == 0 && loss) {
        double l = 0.0;
        for (int b = 0; b < nb; ++b) l += loss_part[b];
        *loss = l / (double)ns;
    }
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters.
__global__ void k_lws_adam(float* __restrict__ P, const float* __restrict__ g, float* __restrict__ m,
                           float* __restrict__ v, float lr, float b1, float b2, float eps, int step) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= HX_LWS_NPARAM) return;
    const float gt = g[t];
    const float mt = b1 * m[t] + (1.f - b1) * gt;
    const float vt = b2 * v[t] + (1.f - b2) * gt * gt;
    m[t] = mt;
    v[t] = vt;
    const float mh = mt / (1.f - powf(b1, (float)step));
    const float vh = vt / (1.f - powf(b2, (float)step));
    P[t] -= lr * mh / (sqrtf(vh) + eps);
}

// SplitMix64 finaliser (Steele, Lea & Flood 2014), for sample indices.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
__global__ void k_lws_batch(uint64_t seed, int step, int64_t n, int64_t bs, int64_t* __restrict__ idx) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= bs) return;
    const uint64_t r = mix64(seed * 0x9E3779B97F4A7C15ULL + ((uint64_t)step << 32) + (uint64_t)t);
    idx[t] = (int64_t)(r % (uint64_t)n);
}

// Features of every individual (see the top of the file).  Thread per
// individual over all blocks; p of QSTAGE_WORDS words staged in shared memory
// as [block][k][h].  The K log-likelihood sums are exponent-renormalised FP32
// products (one log per (i, k)).
template <int K>
__global__ void __launch_bounds__(ACC_THREADS) k_lws_feat(PassArgs a, const unsigned long long* __restrict__ dm,
                                                          const double* __restrict__ Xtz, float* __restrict__ feat) {
    __shared__ __align__(16) float sp[QSTAGE_WORDS * 8 * 4 * K];
    __shared__ float4 s_snp[4];
    const int tid = threadIdx.x;
    snp_table_init(s_snp, tid);
    const int64_t i = (int64_t)blockIdx.x * ACC_THREADS + tid;
    float mant[K];
    int ex[K];
#pragma unroll
    for (int k = 0; k < K; ++k) { mant[k] = 1.f; ex[k] = 0; }
    for (int ws = 0; ws < a.JW; ws += QSTAGE_WORDS) {
        const int nw = min(QSTAGE_WORDS, a.JW - ws);
        uint32_t words[QSTAGE_WORDS];
#pragma unroll
        for (int w = 0; w < QSTAGE_WORDS; ++w)
            words[w] = (w < nw && i < a.Ipad) ? a.G[(int64_t)(ws + w) * a.Ipad + i] : HX_PAD_WORD;
        __syncthreads();
        const int nval = nw * 8 * 4 * K;
        const int64_t base = (int64_t)ws * 8 * 4 * K;
        const int64_t limit = a.J * 4 * K;
        for (int t = tid; t < nval; t += ACC_THREADS) {
            const int blk = t / (4 * K), r = t - blk * 4 * K, h = r / K, k = r - h * K;
            sp[blk * 4 * K + k * 4 + h] = (base + t < limit) ? (float)a.p[base + t] : 0.25f;
        }
        __syncthreads();
        for (int w = 0; w < nw; ++w) {
            for (int b = 0; b < 8; ++b) {
                const unsigned nib = (words[w] >> (4 * b)) & 0xFu;
                const float4* pb = reinterpret_cast<const float4*>(sp + (w * 8 + b) * 4 * K);
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    const float4 pk = pb[k];
                    const float qp[4] = {pk.x, pk.y, pk.z, pk.w};
                    mant[k] = renorm(mant[k] * pair_lik_tab(nib, qp, s_snp), ex[k]);
                }
            }
        }
    }
    if (i >= a.I) return;
    const int64_t nobs = (int64_t)a.J - (int64_t)dm[i];   // blocks that are not double missing
    const double n = nobs > 0 ? (double)nobs : 1.0;
    double av[K], amax = -INFINITY;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        av[k] = (log((double)mant[k]) + (double)ex[k] * 0.69314718055994530942) / n;
        amax = fmax(amax, av[k]);
    }
#pragma unroll
    for (int k = 0; k < K; ++k) {
        feat[((int64_t)K * i + k) * 2] = (float)(av[k] - amax);
        feat[((int64_t)K * i + k) * 2 + 1] = (float)((Xtz[(int64_t)K * i + k] / (2.0 * n) - 1.0) * sqrt(n));
    }
}

size_t grad_smem() { return (size_t)LWS_WARPS * 2 * H * H * sizeof(float); }
int grad_blocks(int64_t ns) {
    int64_t b = (ns + LWS_WARPS * 8 - 1) / (LWS_WARPS * 8);
    return (int)(b < 1 ? 1 : (b > 304 ? 304 : b));
}

}  // namespace

cudaError_t lws_attrs() {
    return cudaFuncSetAttribute(k_lws_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)grad_smem());
}

cudaError_t lws_features(int K, const PassArgs& a, const unsigned long long* dm, const double* Xtz, float* feat,
                         cudaStream_t st) {
    dim3 grid((unsigned)(a.Ipad / ACC_THREADS));
#define HX_CASE(KK) case KK: k_lws_feat<KK><<<grid, ACC_THREADS, 0, st>>>(a, dm, Xtz, feat); break;
    switch (K) {
        HX_CASE(1) HX_CASE(2) HX_CASE(3) HX_CASE(4) HX_CASE(5) HX_CASE(6)
        HX_CASE(7) HX_CASE(8) HX_CASE(9) HX_CASE(10) HX_CASE(11) HX_CASE(12)
        default: return cudaErrorInvalidValue;
    }
#undef HX_CASE
    return cudaGetLastError();
}

cudaError_t lws_forward(const float* feat, int64_t n, int K, const float* P, float* q, cudaStream_t st) {
    int64_t nb = (n + LWS_WARPS - 1) / LWS_WARPS;
    if (nb > 65535 * 8) nb = 65535 * 8;
    k_lws_forward<<<(unsigned)nb, 32 * LWS_WARPS, 0, st>>>(feat, n, K, P, q);
    return cudaGetLastError();
}

// Gradient of the mean loss over samples idx[0..ns) (or 0..ns), into grad;
// scratch: part (304 x NPARAM floats), loss_part (304 doubles).
cudaError_t lws_grad(const float* feat, const float* target, const int64_t* idx, int64_t ns, int K, const float* P,
                     float* part, double* loss_part, float* grad, double* loss, cudaStream_t st) {
    const int nb = grad_blocks(ns);
    k_lws_grad<<<nb, 32 * LWS_WARPS, grad_smem(), st>>>(feat, target, idx, ns, K, P, part, loss_part);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_lws_reduce<<<(HX_LWS_NPARAM + 255) / 256, 256, 0, st>>>(part, loss_part, nb, ns, grad, loss);
    return cudaGetLastError();
}

cudaError_t lws_train(const float* feat, const float* target, int64_t n, int K, float* P, float* m, float* v,
                      int steps, int64_t bs, float lr, uint64_t seed, int step0, int64_t* idx, float* part,
                      double* loss_part, float* grad, double* losses, cudaStream_t st) {
    for (int s = 0; s < steps; ++s) {
        k_lws_batch<<<(unsigned)((bs + 255) / 256), 256, 0, st>>>(seed, step0 + s, n, bs, idx);
        cudaError_t e = lws_grad(feat, target, idx, bs, K, P, part, loss_part, grad, losses ? losses + s : nullptr,
                                 st);
        if (e != cudaSuccess) return e;
        k_lws_adam<<<(HX_LWS_NPARAM + 255) / 256, 256, 0, st>>>(P, grad, m, v, lr, 0.9f, 0.999f, 1e-8f,
                                                                step0 + s + 1);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace hx
