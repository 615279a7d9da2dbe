// hx_common.cuh -- shared definitions of the GB300 HaploADMIXTURE fitting path.
//
// Genotype layout in HBM ("class words"): after hx_create the PLINK BED bytes
// are decoded once into one 32-bit word per (individual, group of 8 two-SNP
// blocks): word G[jw * Ipad + i] holds in nibble b (bits 4b..4b+3) the class
// of block j = 8*jw + b for individual i, as code(SNP 2j) | code(SNP 2j+1) << 2
// with the raw 2-bit BED codes (0b00 hom A1, 0b01 missing, 0b10 het, 0b11 hom
// A2; src/loops.jl:55-71).  Padding individuals (i >= I) and padding blocks
// (j >= J) carry nibble 0x5 (both SNPs missing), whose likelihood factor is 1
// and whose expected counts are 0, so padding never contributes.  The layout
// keeps the BED's 4 bits per (i, j) pair and turns every pass into fully
// coalesced word loads along individuals.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define HX_KMAX 12
#define HX_QMAX_DEV 6
#define HX_IPAD 128
#define HX_PAD_NIBBLE 0x5u
#define HX_PAD_WORD 0x55555555u

namespace hx {

// Genotype value of a raw BED code (src/loops.jl:64-71): 0->0, 1->missing(3), 2->1, 3->2.
__host__ __device__ constexpr int code_g(int c) { return c == 0 ? 0 : (c == 1 ? 3 : (c == 2 ? 1 : 2)); }

// Haplotype-set masks of a class (bit h for haplotype h = 2*allele(SNP1)+allele(SNP2)).
// The pair likelihood is L = F1 * F2 with F_s = sum_{h in S_s} qp_h, except the
// double heterozygote (L = qp00 qp11 + qp01 qp10, both phases) and the
// double-missing class (L = 1).  This is the factored form of
// @coefs_likelihood (src/loops.jl:85-104): F1 = a1 + a2 and F2 = b1 + b2.
__host__ __device__ constexpr unsigned class_m1(unsigned nib) {
    int g1 = code_g(nib & 3), g2 = code_g((nib >> 2) & 3);
    if (g1 == 3 && g2 == 3) return 0;
    if (g1 == 1 && g2 == 1) return 0;
    if (g1 == 3) return g2 == 2 ? 0xAu : 0x5u;          // {01,11} : {00,10}
    if (g2 == 3) return g1 == 2 ? 0xCu : 0x3u;          // {10,11} : {00,01}
    int s1 = g1 == 2 ? 1 : 0, s2 = g2 == 2 ? 1 : 0;     // first copy
    return 1u << (2 * s1 + s2);
}
__host__ __device__ constexpr unsigned class_m2(unsigned nib) {
    int g1 = code_g(nib & 3), g2 = code_g((nib >> 2) & 3);
    if (g1 == 3 && g2 == 3) return 0;
    if (g1 == 1 && g2 == 1) return 0;
    if (g1 == 3) return g2 == 0 ? 0x5u : 0xAu;          // second copy's SNP2 allele
    if (g2 == 3) return g1 == 0 ? 0x3u : 0xCu;
    int s1 = g1 >= 1 ? 1 : 0, s2 = g2 >= 1 ? 1 : 0;     // second copy
    return 1u << (2 * s1 + s2);
}
__host__ __device__ constexpr uint64_t make_tab(bool second) {
    uint64_t t = 0;
    for (unsigned n = 0; n < 16; ++n) t |= (uint64_t)(second ? class_m2(n) : class_m1(n)) << (4 * n);
    return t;
}
constexpr uint64_t TAB_M1 = make_tab(false);
constexpr uint64_t TAB_M2 = make_tab(true);
constexpr unsigned NIB_HH = 2u | (2u << 2);   // het / het
constexpr unsigned NIB_MM = 1u | (1u << 2);   // missing / missing

template <typename T> __device__ __forceinline__ T rcp(T x);
template <> __device__ __forceinline__ float rcp<float>(float x) { return __frcp_rn(x); }
template <> __device__ __forceinline__ double rcp<double>(double x) { return 1.0 / x; }

// Per-pair evaluation.  Given the class nibble and the mixed haplotype
// frequencies qp[h] = sum_k q[k,i] p[k,4j+h] it returns
//   L    : the pair likelihood (src/loops.jl:85-104, 254),
//   u[h] : c_h / qp_h = d log L / d qp_h, with c_h the E-step expected
//          haplotype counts of @coefs (src/loops.jl:114-155).
// Branch-free: the class only selects operands.
template <typename T>
__device__ __forceinline__ void pair_eval(unsigned nib, const T qp[4], T& L, T u[4]) {
    const unsigned m1 = (unsigned)(TAB_M1 >> (4 * nib)) & 0xFu;
    const unsigned m2 = (unsigned)(TAB_M2 >> (4 * nib)) & 0xFu;
    T F1 = ((((m1 & 1u) ? qp[0] : T(0)) + ((m1 & 2u) ? qp[1] : T(0))) + ((m1 & 4u) ? qp[2] : T(0))) +
           ((m1 & 8u) ? qp[3] : T(0));
    T F2 = ((((m2 & 1u) ? qp[0] : T(0)) + ((m2 & 2u) ? qp[1] : T(0))) + ((m2 & 4u) ? qp[2] : T(0))) +
           ((m2 & 8u) ? qp[3] : T(0));
    const bool hh = nib == NIB_HH;
    const bool mm = nib == NIB_MM;
    T den = qp[0] * qp[3] + qp[1] * qp[2];
    F1 = hh ? den : F1;
    F1 = mm ? T(1) : F1;
    F2 = (hh || mm) ? T(1) : F2;
    const T r1 = rcp<T>(F1), r2 = rcp<T>(F2);
    L = F1 * F2;
#pragma unroll
    for (int h = 0; h < 4; ++h) {
        T a = ((m1 >> h) & 1u) ? r1 : T(0);
        T b = ((m2 >> h) & 1u) ? r2 : T(0);
        T v = a + b;
        u[h] = hh ? qp[3 - h] * r1 : v;
    }
}

// Copy-level allele indicators of a raw SNP code, as FP32 0/1 values
// {copy 1 may carry allele 0, copy 1 allele 1, copy 2 allele 0, copy 2 allele 1}:
// hom A1 (code 0) {0}{0}; missing (1) {0,1}{0,1}; het (2) {0}{1}; hom A2 (3) {1}{1}.
// With M[a][b] = qp_{2a+b}, F_s = sum_{a in A_s, b in B_s} M[a][b] over the
// copy-s sets of the block's two SNPs, which is the class_m1/class_m2 factor
// for every class except the double heterozygote and double missing.
// A kernel keeps the table in shared memory (snp_table_init by its first 16
// threads, then a barrier) and reads one 16-byte row per SNP: the four rows
// occupy distinct banks, so a warp's lookups never conflict.
__device__ __forceinline__ void snp_table_init(float4* tab, int tid) {
    if (tid < 16) {
        const int c = tid >> 2, e = tid & 3;
        const int bits = c == 0 ? 0x5 : c == 1 ? 0xF : c == 2 ? 0x9 : 0xA;   // bit e: indicator e
        reinterpret_cast<float*>(tab)[tid] = (bits >> e) & 1 ? 1.f : 0.f;
    }
}

// FP32 pair evaluation for the mixed method: same results as pair_eval<float>
// (L identical; u to the last bit of an approximate reciprocal), with the class
// turned into arithmetic on indicator rows instead of per-haplotype selects.
__device__ __forceinline__ void pair_eval_tab(unsigned nib, const float qp[4], float& L, float u[4], const float4* tab) {
    const float4 ta = tab[nib & 3u], tb = tab[(nib >> 2) & 3u];
    const float v10 = fmaf(tb.y, qp[1], tb.x * qp[0]), v11 = fmaf(tb.y, qp[3], tb.x * qp[2]);
    const float v20 = fmaf(tb.w, qp[1], tb.z * qp[0]), v21 = fmaf(tb.w, qp[3], tb.z * qp[2]);
    float F1 = fmaf(ta.y, v11, ta.x * v10);
    float F2 = fmaf(ta.w, v21, ta.z * v20);
    const bool hh = nib == NIB_HH;
    const bool mm = nib == NIB_MM;
    const float den = fmaf(qp[1], qp[2], qp[0] * qp[3]);
    F1 = hh ? den : F1;
    F1 = mm ? 1.f : F1;
    F2 = (hh || mm) ? 1.f : F2;
    L = F1 * F2;
    float r1, r2;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r1) : "f"(F1));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r2) : "f"(F2));
    const float hr = hh ? r1 : 0.f;
    r1 = (hh || mm) ? 0.f : r1;
    r2 = (hh || mm) ? 0.f : r2;
    const float x10 = ta.x * r1, x11 = ta.y * r1, x20 = ta.z * r2, x21 = ta.w * r2;
    u[0] = fmaf(hr, qp[3], fmaf(x10, tb.x, x20 * tb.z));
    u[1] = fmaf(hr, qp[2], fmaf(x10, tb.y, x20 * tb.w));
    u[2] = fmaf(hr, qp[1], fmaf(x11, tb.x, x21 * tb.z));
    u[3] = fmaf(hr, qp[0], fmaf(x11, tb.y, x21 * tb.w));
}

// scale * u of pair_eval_tab (scale a power of two, e.g. 1/4), without the
// likelihood: the scale is folded into the two reciprocals, and since every
// later operation is a product or a sum of scaled terms the result has the
// same bits as u * scale, two multiplications cheaper than scaling u.
__device__ __forceinline__ void pair_u_tab(unsigned nib, const float qp[4], float u[4], const float4* tab,
                                           float scale) {
    const float4 ta = tab[nib & 3u], tb = tab[(nib >> 2) & 3u];
    const float v10 = fmaf(tb.y, qp[1], tb.x * qp[0]), v11 = fmaf(tb.y, qp[3], tb.x * qp[2]);
    const float v20 = fmaf(tb.w, qp[1], tb.z * qp[0]), v21 = fmaf(tb.w, qp[3], tb.z * qp[2]);
    float F1 = fmaf(ta.y, v11, ta.x * v10);
    float F2 = fmaf(ta.w, v21, ta.z * v20);
    const bool hh = nib == NIB_HH;
    const bool mm = nib == NIB_MM;
    const float den = fmaf(qp[1], qp[2], qp[0] * qp[3]);
    F1 = hh ? den : F1;
    F1 = mm ? 1.f : F1;
    F2 = (hh || mm) ? 1.f : F2;
    float r1, r2;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r1) : "f"(F1));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r2) : "f"(F2));
    r1 *= scale;
    r2 *= scale;
    const float hr = hh ? r1 : 0.f;
    r1 = (hh || mm) ? 0.f : r1;
    r2 = (hh || mm) ? 0.f : r2;
    const float x10 = ta.x * r1, x11 = ta.y * r1, x20 = ta.z * r2, x21 = ta.w * r2;
    u[0] = fmaf(hr, qp[3], fmaf(x10, tb.x, x20 * tb.z));
    u[1] = fmaf(hr, qp[2], fmaf(x10, tb.y, x20 * tb.w));
    u[2] = fmaf(hr, qp[1], fmaf(x11, tb.x, x21 * tb.z));
    u[3] = fmaf(hr, qp[0], fmaf(x11, tb.y, x21 * tb.w));
}

// Likelihood only (log-likelihood passes).
__device__ __forceinline__ float pair_lik_tab(unsigned nib, const float qp[4], const float4* tab) {
    const float4 ta = tab[nib & 3u], tb = tab[(nib >> 2) & 3u];
    const float v10 = fmaf(tb.y, qp[1], tb.x * qp[0]), v11 = fmaf(tb.y, qp[3], tb.x * qp[2]);
    const float v20 = fmaf(tb.w, qp[1], tb.z * qp[0]), v21 = fmaf(tb.w, qp[3], tb.z * qp[2]);
    float F1 = fmaf(ta.y, v11, ta.x * v10);
    float F2 = fmaf(ta.w, v21, ta.z * v20);
    const bool hh = nib == NIB_HH;
    const bool mm = nib == NIB_MM;
    const float den = fmaf(qp[1], qp[2], qp[0] * qp[3]);
    F1 = hh ? den : F1;
    F1 = mm ? 1.f : F1;
    F2 = (hh || mm) ? 1.f : F2;
    return F1 * F2;
}

// Type-generic entry: FP32 uses the indicator table, FP64 the exact select form.
__device__ __forceinline__ void pair_eval_t(unsigned nib, const float qp[4], float& L, float u[4], const float4* tab) {
    pair_eval_tab(nib, qp, L, u, tab);
}
__device__ __forceinline__ void pair_eval_t(unsigned nib, const double qp[4], double& L, double u[4], const float4*) {
    pair_eval<double>(nib, qp, L, u);
}

__device__ __forceinline__ float pair_lik_t(unsigned nib, const float qp[4], const float4* tab) {
    return pair_lik_tab(nib, qp, tab);
}
__device__ __forceinline__ double pair_lik_t(unsigned nib, const double qp[4], const float4*) {
    const unsigned m1 = (unsigned)(TAB_M1 >> (4 * nib)) & 0xFu;
    const unsigned m2 = (unsigned)(TAB_M2 >> (4 * nib)) & 0xFu;
    double F1 = ((((m1 & 1u) ? qp[0] : 0.0) + ((m1 & 2u) ? qp[1] : 0.0)) + ((m1 & 4u) ? qp[2] : 0.0)) +
                ((m1 & 8u) ? qp[3] : 0.0);
    double F2 = ((((m2 & 1u) ? qp[0] : 0.0) + ((m2 & 2u) ? qp[1] : 0.0)) + ((m2 & 4u) ? qp[2] : 0.0)) +
                ((m2 & 8u) ? qp[3] : 0.0);
    const bool hh = nib == NIB_HH;
    const bool mm = nib == NIB_MM;
    const double den = qp[0] * qp[3] + qp[1] * qp[2];
    F1 = hh ? den : F1;
    F1 = mm ? 1.0 : F1;
    F2 = (hh || mm) ? 1.0 : F2;
    return F1 * F2;
}

// Packed FP32x2 arithmetic (sm_100+): fma.rn.f32x2 performs two IEEE FMAs,
// lane by lane, with the results of two fmaf calls.
__device__ __forceinline__ uint64_t f2_dup(float x) {
    uint64_t d;
    asm("mov.b64 %0, {%1, %1};" : "=l"(d) : "f"(x));
    return d;
}
__device__ __forceinline__ uint64_t f2_pack(float lo, float hi) {
    uint64_t d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
    return d;
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ void f2_split(uint64_t v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}

// Exact exponent/mantissa split used to accumulate products of likelihoods
// without underflow (one log per thread instead of two per pair).
__device__ __forceinline__ float renorm(float m, int& e) {
    unsigned b = __float_as_uint(m);
    e += (int)((b >> 23) & 0xFFu) - 127;
    return __uint_as_float((b & 0x007FFFFFu) | 0x3F800000u);
}
__device__ __forceinline__ double renorm(double m, int& e) {
    unsigned long long b = (unsigned long long)__double_as_longlong(m);
    e += (int)((b >> 52) & 0x7FFull) - 1023;
    return __longlong_as_double((long long)((b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull));
}

}  // namespace hx
