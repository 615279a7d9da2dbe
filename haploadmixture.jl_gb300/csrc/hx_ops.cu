// hx_ops.cu -- decode, checks, synthetic data, reductions, EM normalisation,
// projection, batched QP and ZAL quasi-Newton kernels (all FP64 where the
// arithmetic is floating point).
#include "hx_ops.cuh"
#include <climits>

namespace hx {

namespace {
constexpr unsigned FULL = 0xffffffffu;

// ------------------------------------------------------------------ decode
// One thread per (word column jw, BED byte column c): reads the 16 SNP rows of
// the word column at byte c (4 individuals) and writes 4 class words.
__global__ void k_pack(const uint8_t* __restrict__ bed, int64_t bps, int64_t I, int64_t J, int64_t Ipad,
                       uint32_t* __restrict__ G) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t jw = blockIdx.y;
    if (c >= Ipad / 4) return;
    uint32_t w[4] = {0u, 0u, 0u, 0u};
#pragma unroll
    for (int t = 0; t < 16; ++t) {
        const int64_t s = 16 * jw + t;
        const int64_t j = s >> 1;
        const uint8_t byte = (j < J && c < bps) ? bed[s * bps + c] : (uint8_t)0x55;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            uint32_t code = (byte >> (2 * r)) & 3u;
            if (4 * c + r >= I) code = 1u;
            w[r] |= code << (4 * (t >> 1) + 2 * (t & 1));
        }
    }
    uint4 v = make_uint4(w[0], w[1], w[2], w[3]);
    *reinterpret_cast<uint4*>(G + jw * Ipad + 4 * c) = v;
}

__global__ void k_census(const uint32_t* __restrict__ G, int64_t Ipad, int64_t I, int64_t J,
                         unsigned long long* __restrict__ counts) {
    __shared__ unsigned hist[16];
    if (threadIdx.x < 16) hist[threadIdx.x] = 0u;
    __syncthreads();
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t jw = blockIdx.y;
    if (i < I) {
        const uint32_t word = G[jw * Ipad + i];
        for (int b = 0; b < 8; ++b) {
            if (8 * jw + b >= J) break;
            const unsigned nib = (word >> (4 * b)) & 0xFu;
            const int g1 = code_g(nib & 3), g2 = code_g(nib >> 2);
            atomicAdd(&hist[g1 * 4 + g2], 1u);
        }
    }
    __syncthreads();
    if (threadIdx.x < 16 && hist[threadIdx.x]) atomicAdd(counts + threadIdx.x, (unsigned long long)hist[threadIdx.x]);
}

// src/utils.jl:1-18: per individual, blocks (over the whole SNP range) whose
// two SNPs are both missing.  Thread per (byte column, chunk of blocks).
__global__ void k_double_missing(const uint8_t* __restrict__ bed, int64_t bps, int64_t I, int64_t Jf, int64_t chunk,
                                 unsigned long long* __restrict__ dm) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= bps) return;
    const int64_t j0 = (int64_t)blockIdx.y * chunk, j1 = min(Jf, j0 + chunk);
    unsigned cnt[4] = {0u, 0u, 0u, 0u};
    for (int64_t j = j0; j < j1; ++j) {
        const uint8_t b1 = bed[(2 * j) * bps + c], b2 = bed[(2 * j + 1) * bps + c];
#pragma unroll
        for (int r = 0; r < 4; ++r) cnt[r] += (((b1 >> (2 * r)) & 3) == 1 && ((b2 >> (2 * r)) & 3) == 1) ? 1u : 0u;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r)
        if (4 * c + r < I && cnt[r]) atomicAdd(dm + 4 * c + r, (unsigned long long)cnt[r]);
}

// ------------------------------------------------------------------ synthetic
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t draw53(uint64_t key, uint64_t idx) {
    return mix64(key + (idx + 1) * 0x9E3779B97F4A7C15ULL) >> 11;
}

__global__ void k_synth(uint64_t seed, int64_t I, int64_t J, int K, const uint64_t* __restrict__ thrQ,
                        const uint64_t* __restrict__ thrP, uint64_t thr_miss, uint8_t* __restrict__ bed) {
    const int64_t bps = (I + 3) / 4;
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= bps) return;
    const uint64_t k0 = mix64(seed ^ (0ULL * 0x9E3779B97F4A7C15ULL));
    const uint64_t k1 = mix64(seed ^ (1ULL * 0x9E3779B97F4A7C15ULL));
    const uint64_t k2 = mix64(seed ^ (2ULL * 0x9E3779B97F4A7C15ULL));
    for (int64_t j = blockIdx.y; j < J; j += gridDim.y) {
        unsigned o1 = 0, o2 = 0;
        for (int r = 0; r < 4; ++r) {
            const int64_t i = 4 * c + r;
            if (i >= I) break;
            int a1 = 0, a2 = 0;
            for (int cp = 0; cp < 2; ++cp) {
                const uint64_t idx = ((uint64_t)i * (uint64_t)J + (uint64_t)j) * 2 + cp;
                const uint64_t u = draw53(k0, idx);
                int z = K - 1;
                for (int k = 0; k < K; ++k)
                    if (u < thrQ[(int64_t)K * i + k]) { z = k; break; }
                const uint64_t u2 = draw53(k1, idx);
                int h = 3;
                for (int l = 0; l < 4; ++l)
                    if (u2 < thrP[(int64_t)K * (4 * j + l) + z]) { h = l; break; }
                a1 += h >> 1;
                a2 += h & 1;
            }
            unsigned c1 = a1 == 0 ? 0u : (a1 == 1 ? 2u : 3u);
            unsigned c2 = a2 == 0 ? 0u : (a2 == 1 ? 2u : 3u);
            if (draw53(k2, (uint64_t)i * (uint64_t)(2 * J) + (uint64_t)(2 * j)) < thr_miss) c1 = 1u;
            if (draw53(k2, (uint64_t)i * (uint64_t)(2 * J) + (uint64_t)(2 * j + 1)) < thr_miss) c2 = 1u;
            o1 |= c1 << (2 * r);
            o2 |= c2 << (2 * r);
        }
        bed[(2 * j) * bps + c] = (uint8_t)o1;
        bed[(2 * j + 1) * bps + c] = (uint8_t)o2;
    }
}

// ------------------------------------------------------------------ reductions
__global__ void k_reduce_sym(const double* __restrict__ part, int S, int K, int NV, int64_t rows, int64_t ld,
                             double* __restrict__ XtX, double* __restrict__ Xtz) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    for (int k = 0; k < K; ++k) {
        double s = 0.0;
        for (int c = 0; c < S; ++c) s += part[((int64_t)c * NV + k) * ld + r];
        Xtz[(int64_t)K * r + k] = s;
    }
    if (NV == K) return;
    int v = K;
    for (int k = 0; k < K; ++k)
        for (int k2 = k; k2 < K; ++k2, ++v) {
            double s = 0.0;
            for (int c = 0; c < S; ++c) s += part[((int64_t)c * NV + v) * ld + r];
            XtX[(int64_t)K * K * r + k2 + K * k] = s;
            XtX[(int64_t)K * K * r + k + K * k2] = s;
        }
}

__global__ void k_reduce_sum(const double* __restrict__ part, int64_t n, double* __restrict__ out) {
    __shared__ double red[256];
    double s = 0.0;
    for (int64_t a = threadIdx.x; a < n; a += 256) s += part[a];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

// ------------------------------------------------------------------ projection
// OpenADMIXTURE.project_q! contract restated (Chen & Ye 2011): Euclidean
// projection of v onto {x >= eps, sum x = 1}; same operation order as the oracle.
__device__ void project_simplex(double* v, int n, double eps) {
    double y[HX_KMAX > 4 ? HX_KMAX : 4];
    int idx[HX_KMAX > 4 ? HX_KMAX : 4];
    for (int a = 0; a < n; ++a) { y[a] = v[a] - eps; idx[a] = a; }
    for (int a = 1; a < n; ++a) {
        const int t = idx[a];
        int b = a - 1;
        while (b >= 0 && y[idx[b]] < y[t]) { idx[b + 1] = idx[b]; --b; }
        idx[b + 1] = t;
    }
    const double target = 1.0 - n * eps;
    double tsum = 0.0, tmax = 0.0;
    bool found = false;
    for (int a = 0; a < n - 1; ++a) {
        tsum = tsum + y[idx[a]];
        tmax = (tsum - target) / (a + 1);
        if (tmax >= y[idx[a + 1]]) { found = true; break; }
    }
    if (!found) tmax = (tsum + y[idx[n - 1]] - target) / n;
    for (int a = 0; a < n; ++a) {
        const double t = y[a] - tmax;
        v[a] = (t > 0.0 ? t : 0.0) + eps;
    }
}

// src/algorithms_inner.jl:66,75: q_next = project(q .* Xtz ./ 2(J - dm)).
__global__ void k_em_q(const double* __restrict__ q, const double* __restrict__ Xtz,
                       const unsigned long long* __restrict__ dm, int64_t J, int K, int64_t I, double eps,
                       double* __restrict__ qn) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= I) return;
    double v[HX_KMAX];
    const double den = 2.0 * (double)(J - (int64_t)dm[i]);
    for (int k = 0; k < K; ++k) v[k] = (q[(int64_t)K * i + k] * Xtz[(int64_t)K * i + k]) / den;
    project_simplex(v, K, eps);
    for (int k = 0; k < K; ++k) qn[(int64_t)K * i + k] = v[k];
}

// src/algorithms_inner.jl:67-76: p_next = project(normalise(p .* Xtz)) per (k, quartet).
__global__ void k_em_p(const double* __restrict__ p, const double* __restrict__ Xtz, int K, int64_t J, double eps,
                       double* __restrict__ pn) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)K * J) return;
    const int64_t j = t / K;
    const int k = (int)(t % K);
    double v[4];
    for (int h = 0; h < 4; ++h) {
        const int64_t a = (int64_t)K * (4 * j + h) + k;
        v[h] = p[a] * Xtz[a];
    }
    const double s = v[0] + v[1] + v[2] + v[3];
    for (int h = 0; h < 4; ++h) v[h] /= s;
    project_simplex(v, 4, eps);
    for (int h = 0; h < 4; ++h) pn[(int64_t)K * (4 * j + h) + k] = v[h];
}

__global__ void k_step_q(const double* __restrict__ q, const double* __restrict__ d, int K, int64_t ncol, double eps,
                         double* __restrict__ out, double factor) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ncol) return;
    double v[HX_KMAX];
    for (int k = 0; k < K; ++k) v[k] = q[(int64_t)K * i + k] + (d ? factor * d[(int64_t)K * i + k] : 0.0);
    project_simplex(v, K, eps);
    for (int k = 0; k < K; ++k) out[(int64_t)K * i + k] = v[k];
}

__global__ void k_step_p(const double* __restrict__ p, const double* __restrict__ d, int K, int64_t J, double eps,
                         double* __restrict__ out, double factor) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)K * J) return;
    const int64_t j = t / K;
    const int k = (int)(t % K);
    double v[4];
    for (int h = 0; h < 4; ++h) {
        const int64_t a = (int64_t)K * (4 * j + h) + k;
        v[h] = p[a] + (d ? factor * d[a] : 0.0);
    }
    project_simplex(v, 4, eps);
    for (int h = 0; h < 4; ++h) out[(int64_t)K * (4 * j + h) + k] = v[h];
}

// ------------------------------------------------------------------ QP
// One warp per problem: exact minimiser of 0.5 d'Hd - z'd subject to
// lo <= d <= hi and G equality groups (G = 0: none; G = 1: sum d = 0;
// G >= 2: the variables a with a % G == k sum to 0, for every k), by the
// primal active-set method of the oracle (same working-set rules, tie-breaks
// and tolerance).  The free
// block of H is factorised by a warp-parallel right-looking Cholesky in
// shared memory.  Restates OpenADMIXTURE's create_tableau!/quadratic_program!
// contract as called at src/algorithms_inner.jl:160-166, :303-305 and
// :307-310 (the P quartets' K equalities).  With G >= 2 the multipliers come
// from the G x G Schur system S nu = E_F y1 + E_X d_X, S = E_F H_FF^-1 E_F',
// and a group's last free variable (fixed by its equality) never blocks.
// GB300's FP64 unit is narrow and every lane's FP64 operation costs issue
// slots on it, so each scalar step (square root, pivot reciprocal, the
// solved unknown of a triangular sweep) is computed by lane 0 alone and
// broadcast; rows then scale by the reciprocal.  The working set may start
// from a previous solve's final set (box-only problems, where any set is a
// feasible start): the method converges to the same unique minimiser.
enum { QF = 0, QL = 1, QH = 2 };

struct QPWork {
    double* A;
    double *d, *z, *lo, *hi, *r, *y1, *y2, *ds, *g, *iv;
    double *Y, *S, *nu, *rhs;   // G >= 2 only: nF x G, G x G, G, G
    int *st, *F;
};

__device__ __forceinline__ double wsum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}
__device__ __forceinline__ double wmax(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

// L L' x = b in place (L lower, iv[a] = 1 / L[a,a]).
__device__ void tri_solve(const double* A, const double* iv, int nF, double* x, int lane) {
    for (int a = 0; a < nF; ++a) {
        __syncwarp();
        double xa = 0.0;
        if (lane == 0) {
            xa = x[a] * iv[a];
            x[a] = xa;
        }
        xa = __shfl_sync(FULL, xa, 0);
        for (int rr = a + 1 + lane; rr < nF; rr += 32) x[rr] -= A[rr + nF * a] * xa;
    }
    for (int a = nF - 1; a >= 0; --a) {
        __syncwarp();
        double xa = 0.0;
        if (lane == 0) {
            xa = x[a] * iv[a];
            x[a] = xa;
        }
        xa = __shfl_sync(FULL, xa, 0);
        for (int rr = lane; rr < a; rr += 32) x[rr] -= A[a + nF * rr] * xa;
    }
    __syncwarp();
}

// L L' X = B in place for the ncol columns of X (nF x ncol, column-major).
__device__ void tri_solve_cols(const double* A, const double* iv, int nF, double* X, int ncol, int lane) {
    for (int a = 0; a < nF; ++a) {
        __syncwarp();
        for (int c = lane; c < ncol; c += 32) X[a + nF * c] *= iv[a];
        __syncwarp();
        const int m = nF - a - 1;
        for (int e = lane; e < m * ncol; e += 32) {
            const int rr = a + 1 + e % m, c = e / m;
            X[rr + nF * c] -= A[rr + nF * a] * X[a + nF * c];
        }
    }
    for (int a = nF - 1; a >= 0; --a) {
        __syncwarp();
        for (int c = lane; c < ncol; c += 32) X[a + nF * c] *= iv[a];
        __syncwarp();
        for (int e = lane; e < a * ncol; e += 32) {
            const int rr = e % a, c = e / a;
            X[rr + nF * c] -= A[a + nF * rr] * X[a + nF * c];
        }
    }
    __syncwarp();
}

// GROUPS: the G-group path (G >= 2, instantiated apart so that the other
// forms keep their register allocation); otherwise G is 0 or 1.
template <bool GROUPS, class HF>
__device__ int warp_qp(int n, int G, const HF& H, const QPWork& w) {
    const int lane = threadIdx.x & 31;
    double zs = 1.0;
    for (int a = lane; a < n; a += 32) zs = fmax(zs, fabs(w.z[a]));
    zs = wmax(zs);
    const double tol = 1e-12 * zs;
    const int max_iter = 4 * n + 20;
    if (GROUPS)
        for (int k = lane; k < G; k += 32) w.nu[k] = 0.0;
    for (int it = 0; it < max_iter; ++it) {
        __syncwarp();
        int nF = 0;
        for (int a = 0; a < n; ++a)
            if (w.st[a] == QF) {
                if (lane == 0) w.F[nF] = a;
                ++nF;
            }
        __syncwarp();
        double nu = 0.0;
        if (nF > 0) {
            for (int a = lane; a < nF; a += 32) {
                const int fa = w.F[a];
                double s = w.z[fa];
                for (int b = 0; b < n; ++b)
                    if (w.st[b] != QF) s -= H(fa, b) * w.d[b];
                w.r[a] = s;
                for (int b = 0; b < nF; ++b) w.A[a + nF * b] = H(fa, w.F[b]);
            }
            __syncwarp();
            double md = 0.0;
            for (int a = lane; a < nF; a += 32) md = fmax(md, fabs(w.A[a + nF * a]));
            md = wmax(md);
            const double fl = 1e-300 + 1e-14 * md;
            for (int c = 0; c < nF; ++c) {
                __syncwarp();
                double inv = 0.0;
                if (lane == 0) {
                    double s = w.A[c + nF * c];
                    if (!(s > fl)) s = fl;
                    const double lcc = sqrt(s);
                    inv = 1.0 / lcc;
                    w.A[c + nF * c] = lcc;
                    w.iv[c] = inv;
                }
                inv = __shfl_sync(FULL, inv, 0);
                for (int rr = c + 1 + lane; rr < nF; rr += 32) w.A[rr + nF * c] *= inv;
                __syncwarp();
                for (int rr = c + 1 + lane; rr < nF; rr += 32) {
                    const double lrc = w.A[rr + nF * c];
                    for (int s2 = c + 1; s2 <= rr; ++s2) w.A[rr + nF * s2] -= lrc * w.A[s2 + nF * c];
                }
            }
            __syncwarp();
            for (int a = lane; a < nF; a += 32) w.y1[a] = w.r[a];
            tri_solve(w.A, w.iv, nF, w.y1, lane);
            if (GROUPS) {
                for (int e = lane; e < nF * G; e += 32) {
                    const int a = e % nF, k = e / nF;
                    w.Y[e] = (w.F[a] % G == k) ? 1.0 : 0.0;
                }
                tri_solve_cols(w.A, w.iv, nF, w.Y, G, lane);
                for (int e = lane; e < G * G; e += 32) {
                    const int k = e % G, l = e / G;
                    double s = 0.0;
                    for (int a = 0; a < nF; ++a)
                        if (w.F[a] % G == k) s += w.Y[a + nF * l];
                    w.S[e] = s;
                }
                for (int k = lane; k < G; k += 32) {
                    double s = 0.0;
                    for (int a = 0; a < nF; ++a)
                        if (w.F[a] % G == k) s += w.y1[a];
                    for (int b = 0; b < n; ++b)
                        if (w.st[b] != QF && b % G == k) s += w.d[b];
                    w.rhs[k] = s;
                }
                __syncwarp();
                if (lane == 0) {   // G x G Cholesky and the two sweeps, as the oracle
                    double* S = w.S;
                    double smax = 0.0;
                    for (int k = 0; k < G; ++k) smax = fmax(smax, fabs(S[k + G * k]));
                    const double sfl = 1e-300 + 1e-14 * smax;
                    for (int c = 0; c < G; ++c) {
                        double s = S[c + G * c];
                        for (int k = 0; k < c; ++k) s -= S[c + G * k] * S[c + G * k];
                        if (!(s > sfl)) s = sfl;
                        const double lcc = sqrt(s);
                        S[c + G * c] = lcc;
                        for (int rr = c + 1; rr < G; ++rr) {
                            double t = S[rr + G * c];
                            for (int k = 0; k < c; ++k) t -= S[rr + G * k] * S[c + G * k];
                            S[rr + G * c] = t / lcc;
                        }
                    }
                    for (int a = 0; a < G; ++a) {
                        double t = w.rhs[a];
                        for (int k = 0; k < a; ++k) t -= S[a + G * k] * w.nu[k];
                        w.nu[a] = t / S[a + G * a];
                    }
                    for (int a = G - 1; a >= 0; --a) {
                        double t = w.nu[a];
                        for (int k = a + 1; k < G; ++k) t -= S[k + G * a] * w.nu[k];
                        w.nu[a] = t / S[a + G * a];
                    }
                }
                __syncwarp();
                for (int a = lane; a < nF; a += 32) {
                    double t = w.y1[a];
                    for (int l = 0; l < G; ++l) t -= w.Y[a + nF * l] * w.nu[l];
                    w.ds[a] = t;
                }
            } else if (G == 1) {
                for (int a = lane; a < nF; a += 32) w.y2[a] = 1.0;
                tri_solve(w.A, w.iv, nF, w.y2, lane);
                double cf = 0.0;
                for (int b = lane; b < n; b += 32)
                    if (w.st[b] != QF) cf -= w.d[b];
                cf = wsum(cf);
                double s1 = 0.0, s2 = 0.0;
                for (int a = lane; a < nF; a += 32) { s1 += w.y1[a]; s2 += w.y2[a]; }
                s1 = wsum(s1);
                s2 = wsum(s2);
                nu = (s1 - cf) / s2;
                for (int a = lane; a < nF; a += 32) w.ds[a] = w.y1[a] - nu * w.y2[a];
            } else {
                for (int a = lane; a < nF; a += 32) w.ds[a] = w.y1[a];
            }
            __syncwarp();
        }
        // ratio test: smallest step ratio < 1, lowest variable index on ties
        double best = 1.0;
        int bidx = INT_MAX, bto = QF;
        for (int a = lane; a < nF; a += 32) {
            const int fa = w.F[a];
            if (GROUPS) {   // a group's last free variable is fixed by its equality
                int cnt = 0;
                for (int b = 0; b < nF; ++b) cnt += (w.F[b] % G == fa % G);
                if (cnt == 1) continue;
            }
            const double s = w.ds[a] - w.d[fa];
            double ra = 2.0;
            int to = QF;
            if (s < 0.0) { ra = (w.lo[fa] - w.d[fa]) / s; to = QL; }
            else if (s > 0.0) { ra = (w.hi[fa] - w.d[fa]) / s; to = QH; }
            if (ra < best) { best = ra; bidx = fa; bto = to; }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double ob = __shfl_xor_sync(FULL, best, o);
            const int oi = __shfl_xor_sync(FULL, bidx, o);
            const int ot = __shfl_xor_sync(FULL, bto, o);
            if (ob < best || (ob == best && oi < bidx)) { best = ob; bidx = oi; bto = ot; }
        }
        if (bidx == INT_MAX) {
            for (int a = lane; a < nF; a += 32) w.d[w.F[a]] = w.ds[a];
            __syncwarp();
            for (int a = lane; a < n; a += 32) {
                double s = -w.z[a];
                for (int b = 0; b < n; ++b) s += H(a, b) * w.d[b];
                w.g[a] = s + (GROUPS ? w.nu[a % G] : nu);
            }
            __syncwarp();
            double wv = tol;
            int rel = INT_MAX;
            for (int a = lane; a < n; a += 32) {
                if (w.lo[a] >= 0.0 && w.hi[a] <= 0.0) continue;
                double v = 0.0;
                if (w.st[a] == QL) v = -w.g[a];
                else if (w.st[a] == QH) v = w.g[a];
                if (v > wv) { wv = v; rel = a; }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const double ov = __shfl_xor_sync(FULL, wv, o);
                const int oi = __shfl_xor_sync(FULL, rel, o);
                if (ov > wv || (ov == wv && oi < rel)) { wv = ov; rel = oi; }
            }
            if (rel == INT_MAX) return it + 1;
            __syncwarp();
            if (lane == 0) w.st[rel] = QF;
        } else {
            const double al = best < 0.0 ? 0.0 : best;
            for (int a = lane; a < nF; a += 32) {
                const int fa = w.F[a];
                w.d[fa] = w.d[fa] + al * (w.ds[a] - w.d[fa]);
            }
            __syncwarp();
            if (lane == 0) {
                w.d[bidx] = (bto == QL) ? w.lo[bidx] : w.hi[bidx];
                w.st[bidx] = bto;
            }
        }
    }
    return -1;
}

constexpr int QP_WARPS = 4;

// Per-warp workspace for problems of up to nmax variables and gmax >= 2
// equality groups (gmax = 0 when the problems have at most one equality).
__device__ QPWork carve(double* base, int nmax, int gmax = 0) {
    QPWork w;
    w.A = base;
    double* v = base + nmax * nmax;
    w.d = v; w.z = v + nmax; w.lo = v + 2 * nmax; w.hi = v + 3 * nmax; w.r = v + 4 * nmax;
    w.y1 = v + 5 * nmax; w.y2 = v + 6 * nmax; w.ds = v + 7 * nmax; w.g = v + 8 * nmax; w.iv = v + 9 * nmax;
    double* e = v + 10 * nmax;
    w.Y = e; w.S = e + nmax * gmax; w.nu = w.S + gmax * gmax; w.rhs = w.nu + gmax;
    w.st = reinterpret_cast<int*>(w.rhs + gmax);
    w.F = w.st + nmax;
    return w;
}
__host__ __device__ constexpr size_t qp_warp_bytes(int nmax, int gmax = 0) {
    return (size_t)(nmax * nmax + 10 * nmax + nmax * gmax + gmax * gmax + 2 * gmax) * sizeof(double) +
           (size_t)(2 * nmax) * sizeof(int);
}

struct HQ {
    const double* X;
    int K;
    double pen;   // penalty form: rho on every entry (rho * 1 1'); 0 in the equality form
    __device__ double operator()(int r, int c) const { return X[r + K * c] + pen; }
};
struct HP {
    const double* X;   // XtX_p + K*K*4j
    int K;
    double rho;
    __device__ double operator()(int r, int c) const {
        const int l = r / K, k2 = r - l * K, l2 = c / K, k = c - l2 * K;
        return (l == l2 ? X[(int64_t)K * K * l + k2 + K * k] : 0.0) + (k2 == k ? rho : 0.0);
    }
};

__global__ void __launch_bounds__(32 * QP_WARPS)
k_qp_q(int K, int64_t n, const double* __restrict__ XtX, const double* __restrict__ Xtz,
       const double* __restrict__ q, double* __restrict__ qdiff, double* slots, double pen_rho) {
    extern __shared__ double smem_qp[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t pidx = (int64_t)blockIdx.x * QP_WARPS + warp;
    if (pidx >= n) return;
    QPWork w = carve(smem_qp + warp * (qp_warp_bytes(K) / sizeof(double)), K);
    for (int a = lane; a < K; a += 32) {
        const double qa = q[(int64_t)K * pidx + a];
        w.d[a] = 0.0;
        w.z[a] = Xtz[(int64_t)K * pidx + a];
        w.lo[a] = 0.0 - qa;
        w.hi[a] = 1.0 - qa;
        w.st[a] = (w.lo[a] >= 0.0 && w.hi[a] <= 0.0) ? QL : QF;
    }
    __syncwarp();
    HQ H{XtX + (int64_t)K * K * pidx, K, pen_rho >= 0.0 ? pen_rho : 0.0};
    const int it = warp_qp<false>(K, pen_rho < 0.0 ? 1 : 0, H, w);
    __syncwarp();
    for (int a = lane; a < K; a += 32) qdiff[(int64_t)K * pidx + a] = w.d[a];
    if (it < 0 && lane == 0) atomicAdd(slots + S_QP_FAIL, 1.0);
}

// G = 0: penalty form (rho, warm-started working set); G >= 1: equality form
// with G = K groups (no rho, cold start: a warm-started working set would
// break the equalities); GROUPS when G >= 2.
template <bool GROUPS>
__global__ void __launch_bounds__(32 * QP_WARPS)
k_qp_p(int K, int64_t n, const double* __restrict__ XtX, const double* __restrict__ Xtz,
       const double* __restrict__ p, double rho, double* __restrict__ pdiff, double* slots, int8_t* __restrict__ ws,
       int G) {
    extern __shared__ double smem_qp[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t j = (int64_t)blockIdx.x * QP_WARPS + warp;
    if (j >= n) return;
    const int nv = 4 * K;
    const int gmax = GROUPS ? G : 0;
    if (G > 0) ws = nullptr;
    QPWork w = carve(smem_qp + warp * (qp_warp_bytes(nv, gmax) / sizeof(double)), nv, gmax);
    for (int a = lane; a < nv; a += 32) {
        const double pa = p[(int64_t)nv * j + a];
        w.d[a] = 0.0;
        w.z[a] = Xtz[(int64_t)nv * j + a];
        w.lo[a] = 0.0 - pa;
        w.hi[a] = 1.0 - pa;
        // warm start from the previous solve's working set (bounds only: feasible)
        int s0 = ws ? (int)ws[(int64_t)nv * j + a] : QF;
        if (w.lo[a] >= 0.0 && w.hi[a] <= 0.0) s0 = QL;
        w.st[a] = s0;
        w.d[a] = s0 == QL ? w.lo[a] : (s0 == QH ? w.hi[a] : 0.0);
    }
    __syncwarp();
    HP H{XtX + (int64_t)K * K * 4 * j, K, G > 0 ? 0.0 : rho};
    const int it = warp_qp<GROUPS>(nv, G, H, w);
    __syncwarp();
    for (int a = lane; a < nv; a += 32) {
        pdiff[(int64_t)nv * j + a] = w.d[a];
        if (ws) ws[(int64_t)nv * j + a] = (int8_t)w.st[a];
    }
    if (it < 0 && lane == 0) atomicAdd(slots + S_QP_FAIL, 1.0);
}

// ------------------------------------------------------------------ ZAL QN
constexpr int QN_THREADS = 256;

// Secant-pair update and the dot products of the QN point: for ZAL UtU (full),
// UtV and Utd with d = x - x_next; for LB (the LBQN step) YtY and Ytd with
// Y = U - V formed per element (a short Y, v close to u, keeps its accuracy).
template <int QS, bool LB>
__global__ void __launch_bounds__(QN_THREADS)
k_qn_dots(int64_t n, const double* __restrict__ x, const double* __restrict__ xn, const double* __restrict__ xn2,
          double* __restrict__ U, double* __restrict__ V, const double* __restrict__ slots, double* __restrict__ part) {
    constexpr int NV = LB ? QS * QS + QS : QS * QS * 2 + QS;
    __shared__ double red[QN_THREADS / 32][NV];
    const int it = (int)slots[S_ITER];
    const int col = (it > 0 ? it - 1 : 0) % QS;
    double acc[NV];
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[v] = 0.0;
    for (int64_t a = (int64_t)blockIdx.x * QN_THREADS + threadIdx.x; a < n; a += (int64_t)gridDim.x * QN_THREADS) {
        const double xa = x[a], xna = xn[a];
        const double ua = xna - xa, va = xn2[a] - xna;
        U[a + n * col] = ua;
        V[a + n * col] = va;
        double u[QS], v[QS];
#pragma unroll
        for (int r = 0; r < QS; ++r) {
            u[r] = (r == col) ? ua : U[a + n * r];
            v[r] = (r == col) ? va : V[a + n * r];
        }
        const double dxa = xa - xna;
        if (LB) {
            double y[QS];
#pragma unroll
            for (int r = 0; r < QS; ++r) y[r] = u[r] - v[r];
#pragma unroll
            for (int r = 0; r < QS; ++r) {
#pragma unroll
                for (int s = 0; s < QS; ++s) acc[r * QS + s] += y[r] * y[s];
                acc[QS * QS + r] += y[r] * dxa;
            }
        } else {
#pragma unroll
            for (int r = 0; r < QS; ++r) {
#pragma unroll
                for (int s = 0; s < QS; ++s) {
                    acc[r * QS + s] += u[r] * u[s];
                    acc[QS * QS + r * QS + s] += u[r] * v[s];
                }
                acc[2 * QS * QS + r] += u[r] * dxa;
            }
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        double s = acc[v];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(FULL, s, o);
        if (lane == 0) red[warp][v] = s;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0.0;
        for (int w = 0; w < QN_THREADS / 32; ++w) s += red[w][threadIdx.x];
        part[(int64_t)blockIdx.x * NV + threadIdx.x] = s;
    }
}

// Sums the block partials in block order, then solves (U'U - U'V) c = U'(x - x_next)
// on the first m = min(iter, QS) secant pairs (Gaussian elimination with
// partial pivoting, as Julia's `\`).
// The Q x Q system of the QN point, solved as Julia's `\` (Gaussian
// elimination with partial pivoting): ZAL (lb = 0) (U'U - U'V) c = U'd;
// LBQN (lb = 1) (U-V)'(U-V) c = (U-V)'d.
__global__ void k_qn_solve(const double* __restrict__ part, int nblk, int QS, const double* __restrict__ slots,
                           double* __restrict__ coef, int lb) {
    __shared__ double tot[2 * HX_QMAX_DEV * HX_QMAX_DEV + HX_QMAX_DEV];
    const int NV = lb ? QS * QS + QS : QS * QS * 2 + QS;
    for (int v = threadIdx.x; v < NV; v += blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < nblk; ++b) s += part[(int64_t)b * NV + v];
        tot[v] = s;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    const int it = (int)slots[S_ITER];
    const int m = it < QS ? it : QS;
    double A[HX_QMAX_DEV * HX_QMAX_DEV], b[HX_QMAX_DEV];
    for (int r = 0; r < m; ++r) {
        for (int s = 0; s < m; ++s)
            A[r + m * s] = lb ? tot[r * QS + s] : tot[r * QS + s] - tot[QS * QS + r * QS + s];
        b[r] = lb ? tot[QS * QS + r] : tot[2 * QS * QS + r];
    }
    for (int c = 0; c < m; ++c) {
        int piv = c;
        for (int r = c + 1; r < m; ++r)
            if (fabs(A[r + m * c]) > fabs(A[piv + m * c])) piv = r;
        if (piv != c) {
            for (int k = 0; k < m; ++k) { double t = A[c + m * k]; A[c + m * k] = A[piv + m * k]; A[piv + m * k] = t; }
            double t = b[c]; b[c] = b[piv]; b[piv] = t;
        }
        const double dc = A[c + m * c];
        for (int r = c + 1; r < m; ++r) {
            const double f = A[r + m * c] / dc;
            for (int k = c; k < m; ++k) A[r + m * k] -= f * A[c + m * k];
            b[r] -= f * b[c];
        }
    }
    for (int r = m - 1; r >= 0; --r) {
        double t = b[r];
        for (int k = r + 1; k < m; ++k) t -= A[r + m * k] * b[k];
        b[r] = t / A[r + m * r];
    }
    for (int r = 0; r < QS; ++r) coef[r] = r < m ? b[r] : 0.0;
}

__global__ void k_qn_apply(int64_t n, const double* __restrict__ xn, const double* __restrict__ V, int QS,
                           const double* __restrict__ coef, double* __restrict__ xt) {
    for (int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x) {
        double t = 0.0;
        for (int r = 0; r < QS; ++r) t += V[a + n * r] * coef[r];
        xt[a] = xn[a] - t;
    }
}

// ------------------------------------------------------------------ bookkeeping
__global__ void k_iter_begin(double* slots) {
    slots[S_ITER] += 1.0;
    slots[S_LL_PREV] = slots[S_LL_NEW];
}

// src/algorithms_outer.jl:154-161: keep the ZAL point only if ll_basic < ll_qn.
__global__ void k_accept(int64_t n, double* __restrict__ x, const double* __restrict__ xt,
                         const double* __restrict__ xn2, double* slots) {
    const double lb = slots[S_LL_BASIC], lq = slots[S_LL_QN];
    const bool qn = lb < lq;
    const double* src = qn ? xt : xn2;
    for (int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x)
        x[a] = src[a];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const double ll = qn ? lq : lb;
        const double prev = slots[S_LL_PREV];
        slots[S_LL_NEW] = ll;
        slots[S_RELDIFF] = fabs((ll - prev) / prev);
        slots[S_ACCEPT_QN] = qn ? 1.0 : 0.0;
    }
}

__global__ void k_copy_slot(double* slots, int dst, int src) { slots[dst] = slots[src]; }

__global__ void k_nan_check(const double* __restrict__ a, int64_t n, double* slots) {
    bool bad = false;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        bad |= isnan(a[t]);
    if (__any_sync(FULL, bad) && (threadIdx.x & 31) == 0) slots[S_NAN] = 1.0;
}

inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// ================================================================== launchers
cudaError_t launch_pack(const uint8_t* bed, int64_t bps, int64_t I, int64_t J, int64_t Ipad, int JW, uint32_t* G,
                        cudaStream_t st) {
    dim3 grid(nblk(Ipad / 4, 256), JW);
    k_pack<<<grid, 256, 0, st>>>(bed, bps, I, J, Ipad, G);
    return cudaGetLastError();
}
cudaError_t launch_census(const uint32_t* G, int64_t Ipad, int64_t I, int64_t J, int JW, unsigned long long* counts,
                          cudaStream_t st) {
    dim3 grid(nblk(I, 256), JW);
    k_census<<<grid, 256, 0, st>>>(G, Ipad, I, J, counts);
    return cudaGetLastError();
}
cudaError_t launch_double_missing(const uint8_t* bed, int64_t bps, int64_t I, int64_t nsnp, unsigned long long* dm,
                                  cudaStream_t st) {
    const int64_t Jf = nsnp / 2;
    if (Jf == 0) return cudaSuccess;
    const int64_t chunk = 512;
    dim3 grid(nblk(bps, 256), (unsigned)((Jf + chunk - 1) / chunk));
    k_double_missing<<<grid, 256, 0, st>>>(bed, bps, I, Jf, chunk, dm);
    return cudaGetLastError();
}
cudaError_t launch_synth(uint64_t seed, int64_t I, int64_t J, int K, const uint64_t* thrQ, const uint64_t* thrP,
                         double miss, uint8_t* bed, cudaStream_t st) {
    const int64_t bps = (I + 3) / 4;
    const double tm = ceil(miss * 9007199254740992.0);
    const uint64_t thr_miss = tm <= 0.0 ? 0ULL : (uint64_t)tm;
    dim3 grid(nblk(bps, 128), (unsigned)(J < 65535 ? J : 65535));
    k_synth<<<grid, 128, 0, st>>>(seed, I, J, K, thrQ, thrP, thr_miss, bed);
    return cudaGetLastError();
}
cudaError_t launch_reduce_sym(const double* part, int S, int K, bool hess, int64_t rows, int64_t ld, double* XtX,
                              double* Xtz, cudaStream_t st) {
    const int NV = K + (hess ? K * (K + 1) / 2 : 0);
    k_reduce_sym<<<nblk(rows, 256), 256, 0, st>>>(part, S, K, NV, rows, ld, XtX, Xtz);
    return cudaGetLastError();
}
cudaError_t launch_reduce_sum(const double* part, int64_t n, double* out, cudaStream_t st) {
    k_reduce_sum<<<1, 256, 0, st>>>(part, n, out);
    return cudaGetLastError();
}
cudaError_t launch_em_q(const double* q, const double* Xtz, const unsigned long long* dm, int64_t J, int K, int64_t I,
                        double eps, double* q_next, cudaStream_t st) {
    k_em_q<<<nblk(I, 128), 128, 0, st>>>(q, Xtz, dm, J, K, I, eps, q_next);
    return cudaGetLastError();
}
cudaError_t launch_em_p(const double* p, const double* Xtz, int K, int64_t J, double eps, double* p_next,
                        cudaStream_t st) {
    k_em_p<<<nblk((int64_t)K * J, 128), 128, 0, st>>>(p, Xtz, K, J, eps, p_next);
    return cudaGetLastError();
}
cudaError_t launch_step_q(const double* q, const double* d, int K, int64_t ncol, double eps, double* out,
                          cudaStream_t st, double factor) {
    k_step_q<<<nblk(ncol, 128), 128, 0, st>>>(q, d, K, ncol, eps, out, factor);
    return cudaGetLastError();
}
cudaError_t launch_step_p(const double* p, const double* d, int K, int64_t J, double eps, double* out,
                          cudaStream_t st, double factor) {
    k_step_p<<<nblk((int64_t)K * J, 128), 128, 0, st>>>(p, d, K, J, eps, out, factor);
    return cudaGetLastError();
}
__global__ void k_f2d(const float* __restrict__ a, int64_t n, double* __restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = (double)a[t];
}
cudaError_t launch_f2d(const float* a, int64_t n, double* out, cudaStream_t st) {
    k_f2d<<<nblk(n, 256), 256, 0, st>>>(a, n, out);
    return cudaGetLastError();
}
__global__ void k_d2f(const double* __restrict__ a, int64_t n, float* __restrict__ out) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = (float)a[t];
}
cudaError_t launch_d2f(const double* a, int64_t n, float* out, cudaStream_t st) {
    k_d2f<<<nblk(n, 256), 256, 0, st>>>(a, n, out);
    return cudaGetLastError();
}
int resident_ctas(const void* kernel, int threads, size_t dyn_smem, int tmem_cols) {
    cudaFuncAttributes at{};
    int dev = 0, regs_sm = 0, smem_sm = 0, resv = 0, thr_sm = 0, blk_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaFuncGetAttributes(&at, kernel) != cudaSuccess) return 1;
    cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
    cudaDeviceGetAttribute(&blk_sm, cudaDevAttrMaxBlocksPerMultiprocessor, dev);
    const int warps = (threads + 31) / 32;
    int n = std::min(blk_sm, thr_sm / (32 * warps));
    const int rwarp = ((at.numRegs + 7) / 8 * 8 * 32 + 255) / 256 * 256;   // registers of one warp
    if (rwarp > 0) {
        const int wsub = (regs_sm / 4) / rwarp;                               // warps per sub-partition
        n = std::min(n, 4 * wsub / warps);
    }
    const size_t per = at.sharedSizeBytes + dyn_smem + (size_t)resv;
    if (per > 0) n = std::min(n, (int)((size_t)smem_sm / per));
    if (tmem_cols > 0) n = std::min(n, 512 / tmem_cols);
    return std::max(n, 1);
}

cudaError_t init_kernel_attrs() {
    cudaError_t e = cudaFuncSetAttribute(k_qp_p<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)(QP_WARPS * qp_warp_bytes(4 * HX_KMAX)));
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_qp_p<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(QP_WARPS * qp_warp_bytes(4 * HX_KMAX, HX_KMAX)));
}
cudaError_t launch_qp_q(int K, int64_t n, const double* XtX, const double* Xtz, const double* q, double* qdiff,
                        double* slots, cudaStream_t st, double pen_rho) {
    const size_t smem = QP_WARPS * qp_warp_bytes(K);
    k_qp_q<<<nblk(n, QP_WARPS), 32 * QP_WARPS, smem, st>>>(K, n, XtX, Xtz, q, qdiff, slots, pen_rho);
    return cudaGetLastError();
}
cudaError_t launch_qp_p(int K, int64_t n, const double* XtX, const double* Xtz, const double* p, double rho,
                        double* pdiff, double* slots, int8_t* ws, cudaStream_t st, bool eq) {
    const bool groups = eq && K >= 2;
    const size_t smem = QP_WARPS * qp_warp_bytes(4 * K, groups ? K : 0);
    if (groups)
        k_qp_p<true><<<nblk(n, QP_WARPS), 32 * QP_WARPS, smem, st>>>(K, n, XtX, Xtz, p, rho, pdiff, slots, ws, K);
    else
        k_qp_p<false><<<nblk(n, QP_WARPS), 32 * QP_WARPS, smem, st>>>(K, n, XtX, Xtz, p, rho, pdiff, slots, ws,
                                                                      eq ? 1 : 0);
    return cudaGetLastError();
}
int qn_dots_blocks(int64_t n) {
    int64_t b = (n + QN_THREADS * 8 - 1) / (QN_THREADS * 8);
    return (int)(b < 1 ? 1 : (b > 1216 ? 1216 : b));
}
cudaError_t launch_qn(int64_t n, const double* x, const double* xn, const double* xn2, double* U, double* V, int Qs,
                      double* part, double* coef, double* xt, double* slots, cudaStream_t st, int mode) {
    const int nb = qn_dots_blocks(n);
#define HX_QN(QQ)                                                                                       \
    case QQ:                                                                                            \
        if (mode == 1) k_qn_dots<QQ, true><<<nb, QN_THREADS, 0, st>>>(n, x, xn, xn2, U, V, slots, part);  \
        else k_qn_dots<QQ, false><<<nb, QN_THREADS, 0, st>>>(n, x, xn, xn2, U, V, slots, part);          \
        break;
    switch (Qs) {
        HX_QN(1) HX_QN(2) HX_QN(3) HX_QN(4) HX_QN(5) HX_QN(6)
        default: return cudaErrorInvalidValue;
    }
#undef HX_QN
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_qn_solve<<<1, 128, 0, st>>>(part, nb, Qs, slots, coef, mode == 1 ? 1 : 0);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_qn_apply<<<nblk(n, 256) < 2432 ? nblk(n, 256) : 2432, 256, 0, st>>>(n, xn, V, Qs, coef, xt);
    return cudaGetLastError();
}
cudaError_t launch_iter_begin(double* slots, cudaStream_t st) {
    k_iter_begin<<<1, 1, 0, st>>>(slots);
    return cudaGetLastError();
}
cudaError_t launch_accept(int64_t n, double* x, const double* xt, const double* xn2, double* slots, cudaStream_t st) {
    unsigned nb = nblk(n, 256);
    k_accept<<<nb < 2432 ? nb : 2432, 256, 0, st>>>(n, x, xt, xn2, slots);
    return cudaGetLastError();
}
cudaError_t launch_copy_slot(double* slots, int dst, int src, cudaStream_t st) {
    k_copy_slot<<<1, 1, 0, st>>>(slots, dst, src);
    return cudaGetLastError();
}
cudaError_t launch_nan_check(const double* a, int64_t n, double* slots, cudaStream_t st) {
    unsigned nb = nblk(n, 256);
    k_nan_check<<<nb < 1216 ? nb : 1216, 256, 0, st>>>(a, n, slots);
    return cudaGetLastError();
}

}  // namespace hx
