// hx_skfr.cu -- AIM selection by sparse k-means with feature ranking (SKFR).
//
// The reference optionally selects ancestry-informative markers before the fit
// (src/driver.jl:60-73, 84-105): SparseKmeansFeatureRanking.sparsekmeans1 on an
// ImputedSnpMatrix with blocks of 2 SNPs, then SnpArrays.filter to the sorted
// AIMs.  That package is not part of the reference tree; this is the published
// method (Zhang, Lange and Xu 2020, SKFR1) on the GPU:
//   features   x = (g - mean) / sd per SNP over observed genotypes (n-1 sd),
//              missing -> 0; a SNP with < 2 observations or no variance -> 0;
//   start      k-means++ over all SNPs, uniform draws from SplitMix64(seed + t);
//   iteration  cluster means (an empty cluster keeps its centre), SNP score
//              sum_j n_j theta_jl^2, the `sparsity` best blocks of 2 SNPs kept
//              (higher score first, lower index on ties), centres zero elsewhere,
//              reassignment to the nearest centre over the kept SNPs (lower
//              cluster index on ties), until no assignment changes or max_iter.
// A SNP's standardised value depends only on its 2-bit code, so features are a
// 4-entry table per SNP read through the packed bytes, and cluster sums are
// integer code counts times that table.  All FP64 arithmetic uses explicit
// round-to-nearest operations in a fixed order (no contraction), so results do
// not depend on the thread schedule.
#include "hx_ops.cuh"
#include "../../include/haplo_gb300.h"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

namespace hx {
namespace {

constexpr int SK_THREADS = 256;
constexpr int SK_WARPS = SK_THREADS / 32;

__device__ __forceinline__ unsigned sk_code(const uint8_t* __restrict__ bed, int64_t bps, int64_t l, int64_t i) {
    return (bed[l * bps + (i >> 2)] >> (2 * (int)(i & 3))) & 3u;
}

// Per SNP (one warp each): counts of the four codes over the first I
// individuals, then (lane 0) the standardised value of each code.
__global__ void __launch_bounds__(SK_THREADS)
k_sk_tables(const uint8_t* __restrict__ bed, int64_t bps, int64_t I, int64_t M, double* __restrict__ T) {
    const int lane = threadIdx.x & 31;
    const int64_t l = (int64_t)blockIdx.x * SK_WARPS + (threadIdx.x >> 5);
    if (l >= M) return;
    unsigned n[4] = {0u, 0u, 0u, 0u};
    for (int64_t i = lane; i < I; i += 32) n[sk_code(bed, bps, l, i)]++;
#pragma unroll
    for (int c = 0; c < 4; ++c)
        for (int o = 16; o > 0; o >>= 1) n[c] += __shfl_xor_sync(0xffffffffu, n[c], o);
    if (lane != 0) return;
    double t0 = 0.0, t2 = 0.0, t3 = 0.0;
    const double n0 = (double)n[0], n1 = (double)n[2], n2 = (double)n[3];
    const double nobs = __dadd_rn(__dadd_rn(n0, n1), n2);
    if (nobs >= 2.0) {
        const double mu = __ddiv_rn(__dadd_rn(__dmul_rn(n1, 1.0), __dmul_rn(n2, 2.0)), nobs);
        const double a = __dsub_rn(1.0, mu), b = __dsub_rn(2.0, mu);
        const double ss = __dadd_rn(__dadd_rn(__dmul_rn(n0, __dmul_rn(mu, mu)), __dmul_rn(n1, __dmul_rn(a, a))),
                                    __dmul_rn(n2, __dmul_rn(b, b)));
        const double var = __ddiv_rn(ss, __dsub_rn(nobs, 1.0));
        if (var > 0.0) {
            const double sd = __dsqrt_rn(var);
            t0 = __ddiv_rn(__dsub_rn(0.0, mu), sd);
            t2 = __ddiv_rn(a, sd);
            t3 = __ddiv_rn(b, sd);
        }
    }
    T[4 * l + 0] = t0;
    T[4 * l + 1] = 0.0;   // missing: the mean
    T[4 * l + 2] = t2;
    T[4 * l + 3] = t3;
}

// Column t of the centres (theta[l*K + t]) = individual c's features.
__global__ void k_sk_row(const uint8_t* __restrict__ bed, int64_t bps, int64_t c, const double* __restrict__ T,
                         int64_t M, int K, int t, double* __restrict__ theta) {
    for (int64_t l = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; l < M; l += (int64_t)gridDim.x * blockDim.x)
        theta[l * K + t] = T[4 * l + sk_code(bed, bps, l, c)];
}

// Squared distances of every individual to KK centres (columns col0 .. col0+KK-1
// of theta, row stride ldt) over the SNPs sel[0..nsel), summed in that order.
// With d_out (KK = 1 only) the distance is written there; otherwise the
// nearest centre goes to assign and, with dmin, its distance to dmin.
template <int KK>
__global__ void __launch_bounds__(SK_THREADS)
k_sk_dist(const uint8_t* __restrict__ bed, int64_t bps, int64_t I, const double* __restrict__ T,
          const double* __restrict__ theta, int ldt, int col0, const int64_t* __restrict__ sel, int64_t nsel,
          int* __restrict__ assign, double* __restrict__ d_out, double* __restrict__ dmin) {
    const int64_t i = (int64_t)blockIdx.x * SK_THREADS + threadIdx.x;
    if (i >= I) return;
    double acc[KK];
#pragma unroll
    for (int j = 0; j < KK; ++j) acc[j] = 0.0;
    for (int64_t s = 0; s < nsel; ++s) {
        const int64_t l = sel[s];
        const double x = T[4 * l + sk_code(bed, bps, l, i)];
        const double* th = theta + l * ldt + col0;
#pragma unroll
        for (int j = 0; j < KK; ++j) {
            const double d = __dsub_rn(x, th[j]);
            acc[j] = __dadd_rn(acc[j], __dmul_rn(d, d));
        }
    }
    if (d_out) {
        d_out[i] = acc[0];
        return;
    }
    int best = 0;
#pragma unroll
    for (int j = 1; j < KK; ++j)
        if (acc[j] < acc[best]) best = j;
    assign[i] = best;
    if (dmin) dmin[i] = acc[best];
}

// Per SNP (one warp each): counts of codes 0, 2, 3 per cluster, then the
// cluster means (clusters with n_j = 0 keep their centre) and the SNP's score
// sum_j n_j theta_jl^2.
__global__ void __launch_bounds__(SK_THREADS)
k_sk_centers(const uint8_t* __restrict__ bed, int64_t bps, int64_t I, int64_t M, int K, const int* __restrict__ assign,
             const double* __restrict__ n, const double* __restrict__ T, double* __restrict__ theta,
             double* __restrict__ score) {
    __shared__ unsigned cnt[SK_WARPS][HX_KMAX][3];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t l = (int64_t)blockIdx.x * SK_WARPS + w;
    for (int e = lane; e < HX_KMAX * 3; e += 32) (&cnt[w][0][0])[e] = 0u;
    __syncwarp();
    if (l < M) {
        for (int64_t i = lane; i < I; i += 32) {
            const unsigned c = sk_code(bed, bps, l, i);
            if (c != 1u) atomicAdd(&cnt[w][assign[i]][c == 0u ? 0 : (int)c - 1], 1u);
        }
    }
    __syncwarp();
    if (l >= M || lane != 0) return;
    const double t0 = T[4 * l + 0], t2 = T[4 * l + 2], t3 = T[4 * l + 3];
    double sc = 0.0;
    for (int j = 0; j < K; ++j) {
        if (n[j] > 0.0) {
            const double s = __dadd_rn(__dadd_rn(__dmul_rn((double)cnt[w][j][0], t0), __dmul_rn((double)cnt[w][j][1], t2)),
                                       __dmul_rn((double)cnt[w][j][2], t3));
            theta[l * K + j] = __ddiv_rn(s, n[j]);
        }
        const double th = theta[l * K + j];
        sc = __dadd_rn(sc, __dmul_rn(n[j], __dmul_rn(th, th)));
    }
    score[l] = sc;
}

// Centres are zero off the kept SNPs (keep[l] == 0).
__global__ void k_sk_mask(double* __restrict__ theta, const uint8_t* __restrict__ keep, int64_t M, int K) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < M * K; e += (int64_t)gridDim.x * blockDim.x)
        if (!keep[e / K]) theta[e] = 0.0;
}

cudaError_t launch_dist(int K, int64_t I, const uint8_t* bed, int64_t bps, const double* T, const double* theta,
                        int ldt, int col0, const int64_t* sel, int64_t nsel, int* assign, double* d_out,
                        double* dmin = nullptr) {
    // exactly one output: a distance (one centre) or an assignment
    if ((d_out != nullptr) == (assign != nullptr) || (d_out && K != 1)) return cudaErrorInvalidValue;
    const unsigned g = (unsigned)((I + SK_THREADS - 1) / SK_THREADS);
#define HX_SK_CASE(KK)                                                                                         \
    case KK:                                                                                                   \
        k_sk_dist<KK><<<g, SK_THREADS>>>(bed, bps, I, T, theta, ldt, col0, sel, nsel, assign, d_out, dmin);    \
        break;
    switch (K) {
        HX_SK_CASE(1) HX_SK_CASE(2) HX_SK_CASE(3) HX_SK_CASE(4) HX_SK_CASE(5) HX_SK_CASE(6)
        HX_SK_CASE(7) HX_SK_CASE(8) HX_SK_CASE(9) HX_SK_CASE(10) HX_SK_CASE(11) HX_SK_CASE(12)
        default: return cudaErrorInvalidValue;
    }
#undef HX_SK_CASE
    return cudaGetLastError();
}

// The seed's t-th uniform draw in [0, 1): 53 bits of SplitMix64(seed + t).
double sk_uniform(uint64_t seed, uint64_t t) {
    uint64_t z = seed + t + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

struct SkBuf {   // device buffers of one call, freed on every exit
    std::vector<void*> p;
    ~SkBuf() { for (void* x : p) cudaFree(x); }
    template <class T> cudaError_t get(T** out, size_t n) {
        cudaError_t e = cudaMalloc((void**)out, std::max<size_t>(n, 1) * sizeof(T));
        if (e == cudaSuccess) p.push_back(*out);
        return e;
    }
};

int sk_status(cudaError_t e) {
    return e == cudaSuccess ? HX_OK : (e == cudaErrorMemoryAllocation ? HX_ENOMEM : HX_ECUDA);
}

}  // namespace
}  // namespace hx

#define HX_SK_CK(expr)                          \
    do {                                        \
        cudaError_t e_ = (expr);                \
        if (e_ != cudaSuccess) return hx::sk_status(e_); \
    } while (0)

extern "C" int hx_skfr(const uint8_t* bed, int64_t bytes_per_snp, int64_t n_snp, int64_t I, int32_t K,
                       int64_t sparsity, int32_t max_iter, uint64_t seed, int32_t device, int32_t* clusters,
                       int64_t* aims, int32_t* iters, double* objective) {
    using namespace hx;
    const int64_t M = n_snp - n_snp % 2, nb = M / 2;
    if (!bed || !clusters || !aims || I < 1 || bytes_per_snp < (I + 3) / 4 || n_snp < 2 || max_iter < 1)
        return HX_EINVAL;
    if (K < 1 || K > HX_KMAX) return HX_EUNSUPPORTED;
    if (K > I || sparsity < 1 || sparsity > nb) return HX_EINVAL;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return HX_ECUDA;
    HX_SK_CK(cudaSetDevice(device));
    SkBuf b;
    uint8_t* d_bed = nullptr;
    double *T = nullptr, *theta = nullptr, *score = nullptr, *d2 = nullptr, *n = nullptr;
    int* assign = nullptr;
    int64_t* sel = nullptr;
    uint8_t* keep = nullptr;
    HX_SK_CK(b.get(&d_bed, (size_t)bytes_per_snp * M));
    HX_SK_CK(b.get(&T, (size_t)4 * M));
    HX_SK_CK(b.get(&theta, (size_t)M * K));
    HX_SK_CK(b.get(&score, (size_t)M));
    HX_SK_CK(b.get(&d2, (size_t)I));
    HX_SK_CK(b.get(&n, (size_t)K));
    HX_SK_CK(b.get(&assign, (size_t)I));
    HX_SK_CK(b.get(&sel, (size_t)M));
    HX_SK_CK(b.get(&keep, (size_t)M));
    HX_SK_CK(cudaMemcpy(d_bed, bed, (size_t)bytes_per_snp * M, cudaMemcpyHostToDevice));
    HX_SK_CK(cudaMemset(theta, 0, (size_t)M * K * sizeof(double)));
    const unsigned gw = (unsigned)((M + SK_WARPS - 1) / SK_WARPS);
    k_sk_tables<<<gw, SK_THREADS>>>(d_bed, bytes_per_snp, I, M, T);
    HX_SK_CK(cudaGetLastError());
    std::vector<int64_t> all(M);
    std::iota(all.begin(), all.end(), (int64_t)0);
    HX_SK_CK(cudaMemcpy(sel, all.data(), (size_t)M * sizeof(int64_t), cudaMemcpyHostToDevice));
    const unsigned gr = (unsigned)std::min<int64_t>((M + 255) / 256, 4096);

    // k-means++ start over all SNPs
    std::vector<double> hd(I), ht(I);
    int64_t c = std::min<int64_t>((int64_t)(sk_uniform(seed, 0) * (double)I), I - 1);
    k_sk_row<<<gr, 256>>>(d_bed, bytes_per_snp, c, T, M, K, 0, theta);
    HX_SK_CK(launch_dist(1, I, d_bed, bytes_per_snp, T, theta, K, 0, sel, M, nullptr, d2));
    HX_SK_CK(cudaMemcpy(hd.data(), d2, (size_t)I * sizeof(double), cudaMemcpyDeviceToHost));
    for (int t = 1; t < K; ++t) {
        std::vector<double> cs(I);
        double acc = 0.0;
        for (int64_t i = 0; i < I; ++i) { acc += hd[i]; cs[i] = acc; }
        const double target = sk_uniform(seed, (uint64_t)t) * acc;
        c = I - 1;
        for (int64_t i = 0; i < I; ++i)
            if (cs[i] > target) { c = i; break; }
        k_sk_row<<<gr, 256>>>(d_bed, bytes_per_snp, c, T, M, K, t, theta);
        HX_SK_CK(launch_dist(1, I, d_bed, bytes_per_snp, T, theta, K, t, sel, M, nullptr, d2));
        HX_SK_CK(cudaMemcpy(ht.data(), d2, (size_t)I * sizeof(double), cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < I; ++i)
            if (ht[i] < hd[i]) hd[i] = ht[i];
    }
    HX_SK_CK(launch_dist(K, I, d_bed, bytes_per_snp, T, theta, K, 0, sel, M, assign, nullptr));
    std::vector<int> ha(I), hn_assign(I);
    HX_SK_CK(cudaMemcpy(ha.data(), assign, (size_t)I * sizeof(int), cudaMemcpyDeviceToHost));

    std::vector<double> hs(M), bs(nb), hn(K);
    std::vector<int64_t> order(nb), kept;
    std::vector<uint8_t> hk(M);
    int it = 0;
    for (it = 1; it <= max_iter; ++it) {
        std::fill(hn.begin(), hn.end(), 0.0);
        for (int64_t i = 0; i < I; ++i) hn[ha[i]] += 1.0;
        HX_SK_CK(cudaMemcpy(n, hn.data(), (size_t)K * sizeof(double), cudaMemcpyHostToDevice));
        k_sk_centers<<<gw, SK_THREADS>>>(d_bed, bytes_per_snp, I, M, K, assign, n, T, theta, score);
        HX_SK_CK(cudaGetLastError());
        HX_SK_CK(cudaMemcpy(hs.data(), score, (size_t)M * sizeof(double), cudaMemcpyDeviceToHost));
        for (int64_t k = 0; k < nb; ++k) bs[k] = hs[2 * k] + hs[2 * k + 1];
        std::iota(order.begin(), order.end(), (int64_t)0);
        std::sort(order.begin(), order.end(),
                  [&](int64_t x, int64_t y) { return bs[x] > bs[y] || (bs[x] == bs[y] && x < y); });
        std::vector<int64_t> kb(order.begin(), order.begin() + sparsity);
        std::sort(kb.begin(), kb.end());
        kept.clear();
        for (int64_t k : kb) { kept.push_back(2 * k); kept.push_back(2 * k + 1); }
        std::fill(hk.begin(), hk.end(), (uint8_t)0);
        for (int64_t l : kept) hk[l] = 1;
        HX_SK_CK(cudaMemcpy(keep, hk.data(), (size_t)M, cudaMemcpyHostToDevice));
        k_sk_mask<<<(unsigned)std::min<int64_t>((M * K + 255) / 256, 4096), 256>>>(theta, keep, M, K);
        HX_SK_CK(cudaGetLastError());
        HX_SK_CK(cudaMemcpy(sel, kept.data(), kept.size() * sizeof(int64_t), cudaMemcpyHostToDevice));
        HX_SK_CK(launch_dist(K, I, d_bed, bytes_per_snp, T, theta, K, 0, sel, (int64_t)kept.size(), assign, nullptr,
                             d2));
        HX_SK_CK(cudaMemcpy(hn_assign.data(), assign, (size_t)I * sizeof(int), cudaMemcpyDeviceToHost));
        const bool changed = hn_assign != ha;
        ha.swap(hn_assign);
        if (!changed) break;
    }
    if (it > max_iter) it = max_iter;
    if (objective) {   // within-cluster sum of squares over the kept SNPs, summed in individual order
        HX_SK_CK(cudaMemcpy(hd.data(), d2, (size_t)I * sizeof(double), cudaMemcpyDeviceToHost));
        double w = 0.0;
        for (int64_t i = 0; i < I; ++i) w += hd[i];
        *objective = w;
    }
    std::copy(ha.begin(), ha.end(), clusters);
    std::copy(kept.begin(), kept.end(), aims);
    if (iters) *iters = it;
    return HX_OK;
}
