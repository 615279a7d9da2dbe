// hx_noalloc.cu -- log-likelihood entry point that allocates no device memory.
//
// Some callers cannot or must not allocate device memory at call time.
// Examples: a host framework that hands out all device memory from its own
// pool (the Julia CUDA.jl or PyTorch caching allocators) and forbids side
// allocations; a latency-critical loop where cudaMalloc/cudaFree would
// synchronise the device.  hx_loglikelihood_noalloc evaluates the
// log-likelihood of src/loops.jl:236-258 directly from caller-owned device
// buffers (raw BED bytes, Q, P, output).  Its only scratch (one partial sum
// per CTA) lives in the file-scope array below, which every GPU that loads
// this library holds until the process exits.
#include "hx_ops.cuh"
#include "../../include/haplo_gb300.h"

#include <algorithm>

namespace hx {
namespace {

constexpr int NA_THREADS = 128;

// Scratch of the no-allocation entry point: one FP64 partial per CTA.
__device__ __align__(256) double g_noalloc_scratch[HX_NOALLOC_SCRATCH];

// One individual per thread over a chunk of blocks, decoding the two SNP codes
// of each block straight from the BED bytes (src/loops.jl:55-71); pair
// likelihoods multiply into an exponent-renormalised product (one log per
// thread).  Writes one partial per CTA into scratch[blockIdx.y * gridDim.x + blockIdx.x].
template <int K, typename T>
__global__ void __launch_bounds__(NA_THREADS)
k_loglik_bed(const uint8_t* __restrict__ bed, int64_t bps, int64_t I, int64_t J, const double* __restrict__ q,
             const double* __restrict__ p, int64_t per_chunk, double* __restrict__ scratch) {
    __shared__ double red[NA_THREADS];
    const int tid = threadIdx.x;
    const int64_t i = (int64_t)blockIdx.x * NA_THREADS + tid;
    const bool active = i < I;
    const int64_t j0 = (int64_t)blockIdx.y * per_chunk;
    const int64_t j1 = min(J, j0 + per_chunk);
    T qi[K];
#pragma unroll
    for (int k = 0; k < K; ++k) qi[k] = active ? (T)q[(int64_t)K * i + k] : T(1) / T(K);
    T mant = T(1);
    int ex = 0;
    bool zero = false, bad = false;
    if (active) {
        const int64_t byte = i >> 2;
        const int sh = 2 * (int)(i & 3);
        for (int64_t j = j0; j < j1; ++j) {
            const unsigned c1 = (bed[(2 * j) * bps + byte] >> sh) & 3u;
            const unsigned c2 = (bed[(2 * j + 1) * bps + byte] >> sh) & 3u;
            const unsigned nib = c1 | (c2 << 2);
            if (nib == NIB_MM) continue;
            const double* pj = p + (int64_t)K * 4 * j;
            T qp[4];
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                T s = T(0);
#pragma unroll
                for (int k = 0; k < K; ++k) s = fma(qi[k], (T)pj[h * K + k], s);
                qp[h] = s;
            }
            T L, u[4];
            pair_eval<T>(nib, qp, L, u);
            if (sizeof(T) == 4 && L < T(1.17549435e-38f) && L == L) {
                // FP32 pair likelihood below the smallest normal float (caller
                // Q/P entries far below the fit's 1e-5 floor): the renormaliser
                // reads the exponent field, so redo this pair in FP64 and fold
                // its mantissa and exponent in separately
                double qd[4], Ld, ud[4];
#pragma unroll
                for (int h = 0; h < 4; ++h) {
                    double s = 0.0;
#pragma unroll
                    for (int k = 0; k < K; ++k) s = fma((double)q[(int64_t)K * i + k], pj[h * K + k], s);
                    qd[h] = s;
                }
                pair_eval<double>(nib, qd, Ld, ud);
                if (!(Ld > 0.0)) {
                    if (Ld == 0.0) zero = true; else bad = true;
                    continue;
                }
                mant = renorm(mant * (T)renorm(Ld, ex), ex);
                continue;
            }
            if (!(L > T(0))) {
                if (L == T(0)) zero = true; else bad = true;
                L = T(1);
            }
            mant = renorm(mant * L, ex);
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
    for (int s = NA_THREADS / 2; s > 0; s >>= 1) {
        if (tid < s) red[tid] += red[tid + s];
        __syncthreads();
    }
    if (tid == 0) scratch[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = red[0];
}

// Sums the n partials in a fixed order into *out (one CTA).
__global__ void k_sum_partials(const double* __restrict__ scratch, int64_t n, double* __restrict__ out) {
    __shared__ double red[256];
    double s = 0.0;
    for (int64_t a = threadIdx.x; a < n; a += 256) s += scratch[a];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

#define HX_NA_FOR_K(X) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12)

template <typename T>
cudaError_t launch_bed(int K, dim3 grid, cudaStream_t st, const uint8_t* bed, int64_t bps, int64_t I, int64_t J,
                       const double* q, const double* p, int64_t per_chunk, double* scratch) {
#define HX_CASE(KK) \
    case KK: k_loglik_bed<KK, T><<<grid, NA_THREADS, 0, st>>>(bed, bps, I, J, q, p, per_chunk, scratch); break;
    switch (K) { HX_NA_FOR_K(HX_CASE) default: return cudaErrorInvalidValue; }
#undef HX_CASE
    return cudaGetLastError();
}

}  // namespace
}  // namespace hx

extern "C" int hx_loglikelihood_noalloc(const uint8_t* d_bed, int64_t bytes_per_snp, int64_t I, int64_t J, int32_t K,
                                        const double* d_q, const double* d_p, int32_t precision, double* d_ll,
                                        void* stream) {
    using namespace hx;
    if (!d_bed || !d_q || !d_p || !d_ll || I <= 0 || J <= 0 || bytes_per_snp < (I + 3) / 4) return HX_EINVAL;
    if (K < 1 || K > HX_KMAX) return HX_EUNSUPPORTED;
    if (precision != HX_PREC_FP64 && precision != HX_PREC_MIXED) return HX_EINVAL;
    // one partial per CTA: (individual tiles) x (block chunks) must fit the static scratch
    const int64_t tiles = (I + NA_THREADS - 1) / NA_THREADS;
    if (tiles > HX_NOALLOC_SCRATCH) return HX_EUNSUPPORTED;
    // The device address of the scratch array in the current device's
    // context (host code may not use the symbol itself as an address).  It is
    // looked up on every call, not cached: after a device or primary-context
    // reset the module is loaded again at another address.  The lookup
    // allocates nothing; the first call in a context also loads the module,
    // so make that first call before any stream capture.
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return HX_ECUDA;
    double* scratch = (double*)ptr;
    const int64_t target = 2048;
    int64_t S = std::max<int64_t>(1, std::min<int64_t>(J, (target + tiles - 1) / tiles));
    S = std::min<int64_t>(S, HX_NOALLOC_SCRATCH / tiles);
    const int64_t per_chunk = (J + S - 1) / S;
    S = (J + per_chunk - 1) / per_chunk;
    dim3 grid((unsigned)tiles, (unsigned)S);
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = precision == HX_PREC_FP64
                        ? launch_bed<double>(K, grid, st, d_bed, bytes_per_snp, I, J, d_q, d_p, per_chunk, scratch)
                        : launch_bed<float>(K, grid, st, d_bed, bytes_per_snp, I, J, d_q, d_p, per_chunk, scratch);
    if (e != cudaSuccess) return HX_ECUDA;
    k_sum_partials<<<1, 256, 0, st>>>(scratch, tiles * S, d_ll);
    if (cudaGetLastError() != cudaSuccess) return HX_ECUDA;
    return HX_OK;
}
