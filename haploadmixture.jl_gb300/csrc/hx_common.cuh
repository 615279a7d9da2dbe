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
