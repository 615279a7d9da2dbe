// haplo_oracle.cpp -- CPU oracle for the HaploADMIXTURE fitting hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the FP64 CPU restatement that the
// parity tests, the smoke check and the CPU-baseline leg of bench.py use as
// the checker.  The product (libhaplo_gb300.so) never links, loads or calls it.
//
// Parity status: the reference (pure Julia, HaploADMIXTURE.jl) cannot run in
// this environment (no Julia, no OpenADMIXTURE / SnpArrays packages, and the
// EUR_subset.bed fixture of test/runtests.jl is not shipped), so this oracle is
// "parity unpinned" against reference outputs.  It is pinned instead by
//   * a literal transcription of the reference's mask arithmetic
//     (src/loops.jl:55-155), cross-checked by an independent exact-rational
//     transcription in tests/golden/make_golden.py (committed fixtures),
//   * the two independent likelihood formulas of the reference
//     (src/loops.jl:157-212 vs 214-258), which must agree per pair,
//   * analytic identities (gradient = finite difference of the log-likelihood,
//     EM monotonicity, KKT conditions of the QP, projection optimality).
//
// Arithmetic follows the reference expression order where the reference fixes
// it (compile with -ffp-contract=off: Julia does not contract a*b+c into FMA).
// Third-party routines that the reference calls but does not contain
// (OpenADMIXTURE v0.1.0: project_q!, create_tableau!/quadratic_program!,
// update_UV!/update_QN!) are restated from their published mathematics:
//   * projection onto {x >= eps, sum x = 1}: Chen & Ye (2011), "Projection
//     onto a simplex", applied to x - eps with target sum 1 - n*eps;
//   * QP: exact minimiser of the strictly convex QP by a primal active-set
//     method (the minimiser is unique, so any exact solver agrees to rounding);
//   * quasi-Newton: Zhou, Alexander & Lange (2011), Stat. Comput. 21:261-273,
//     x_qn = F(x) - V (U'U - U'V)^{-1} U'(x - F(x)).
//
// Layouts (Julia column-major, 0-based here):
//   bed    : SNP-major PLINK 1 data bytes (no 3-byte magic); SNP s occupies
//            bytes [s*bps, (s+1)*bps); individual i sits in byte i>>2 at bit
//            offset 2*(i&3).
//   q      : K x I        q[k + K*i]
//   p      : K x 4J       p[k + K*m], m = 4*j + h, h in {00,01,10,11}
//   XtX_q  : K x K x I    XtX[k2 + K*k + K*K*i]
//   XtX_p  : K x K x 4J   XtX[k2 + K*k + K*K*m]

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <thread>
#include <algorithm>
#include <functional>
#include <atomic>

namespace {

// ---------------------------------------------------------------- threading
void parallel_for(int64_t n, int nthreads, const std::function<void(int64_t, int64_t)>& body) {
    if (nthreads <= 1 || n < 2) { body(0, n); return; }
    int nt = (int)std::min<int64_t>(nthreads, n);
    std::vector<std::thread> th;
    std::atomic<int64_t> next(0);
    const int64_t grain = std::max<int64_t>(1, n / (int64_t)(nt * 8));
    for (int t = 0; t < nt; ++t) {
        th.emplace_back([&]() {
            for (;;) {
                int64_t a = next.fetch_add(grain);
                if (a >= n) break;
                body(a, std::min(n, a + grain));
            }
        });
    }
    for (auto& x : th) x.join();
}

// ---------------------------------------------------------------- BED decode
// src/loops.jl:55-71 (@gcoefs_snparray): code 0b00->0, 0b01->missing(3),
// 0b10->1, 0b11->2.
inline int bed_code(const uint8_t* bed, int64_t bps, int64_t i, int64_t snp) {
    uint8_t blk = bed[snp * bps + (i >> 2)];
    return (blk >> ((i & 3) << 1)) & 3;
}
inline double code_to_g(int c) {
    return c == 0 ? 0.0 : (c == 1 ? 3.0 : (c == 2 ? 1.0 : 2.0));
}

struct GMask {  // src/loops.jl:72-81
    double g1, g2;
    double g11, g12, g10, g1M, g1B, g21, g22, g20, g2M, g2B;
};
inline GMask gmask(double g1, double g2) {
    GMask m;
    m.g1 = g1; m.g2 = g2;
    m.g11 = g1 == 1; m.g12 = g1 == 2; m.g10 = g1 == 0; m.g1M = g1 == 3; m.g1B = g1 != 3;
    m.g21 = g2 == 1; m.g22 = g2 == 2; m.g20 = g2 == 0; m.g2M = g2 == 3; m.g2B = g2 != 3;
    return m;
}

// src/loops.jl:85-104 (@coefs_likelihood), literal operation order.
inline void coefs_likelihood(const GMask& g, double qp00, double qp01, double qp10, double qp11,
                             double& a1, double& a2, double& b1, double& b2) {
    a1 = g.g1M * g.g2M + g.g11 * g.g21 * qp00 * qp11 +
         ((g.g1M + g.g10) * (g.g20 + g.g21) + g.g2M * (g.g10 + g.g11) + g.g11 * g.g20) * qp00 +
         ((g.g1M + g.g10 + g.g11) * g.g22) * qp01 +
         (g.g12 * (g.g2M + g.g20 + g.g21)) * qp10 +
         (g.g12 * g.g22) * qp11;
    a2 = g.g11 * g.g21 * qp01 * qp10 + g.g1M * (g.g20 + g.g21) * qp10 +
         g.g2M * (g.g10 + g.g11) * qp01 + (g.g1M * g.g22 + g.g12 * g.g2M) * qp11;
    b1 = g.g1M * g.g2M + g.g11 * g.g21 +
         (g.g10 * g.g20 + g.g1M * g.g20 + g.g10 * g.g2M) * qp00 +
         (g.g1M + g.g10) * (g.g21 + g.g22) * qp01 +
         (g.g11 + g.g12) * (g.g2M + g.g20) * qp10 +
         (g.g11 * g.g22 + g.g12 * (g.g21 + g.g22)) * qp11;
    b2 = (g.g1M * g.g21 + g.g1M * g.g22 + g.g11 * g.g2M + g.g12 * g.g2M) * qp11 +
         g.g1M * g.g20 * qp10 + g.g10 * g.g2M * qp01;
}

// src/loops.jl:114-155 (@coefs), literal operation order.
inline void coefs(const GMask& g, double qp00, double qp01, double qp10, double qp11,
                  double& c00, double& c01, double& c10, double& c11) {
    double a0001 = qp00 / (qp00 + qp01);
    double a0010 = qp00 / (qp00 + qp10);
    double a0100 = qp01 / (qp01 + qp00);
    double a0111 = qp01 / (qp01 + qp11);
    double a1000 = qp10 / (qp10 + qp00);
    double a1011 = qp10 / (qp10 + qp11);
    double a1101 = qp11 / (qp11 + qp01);
    double a1110 = qp11 / (qp11 + qp10);
    double ahet0011 = qp00 * qp11 / (qp00 * qp11 + qp01 * qp10);
    double ahet0110 = qp01 * qp10 / (qp00 * qp11 + qp01 * qp10);
    c00 = 0.0;
    c00 += g.g11 * g.g21 * ahet0011;
    c00 += g.g1M * g.g2B * (2.0 - g.g2) * a0010;
    c00 += g.g1B * g.g2M * (2.0 - g.g1) * a0001;
    c00 += g.g10 * g.g2B * (2.0 - g.g2);
    c00 += g.g11 * g.g20;
    c01 = 0.0;
    c01 += g.g11 * g.g21 * ahet0110;
    c01 += g.g1M * g.g2B * g.g2 * a0111;
    c01 += g.g1B * g.g2M * (2.0 - g.g1) * a0100;
    c01 += g.g10 * g.g2B * g.g2;
    c01 += g.g11 * g.g22;
    c10 = 0.0;
    c10 += g.g11 * g.g21 * ahet0110;
    c10 += g.g1M * g.g2B * (2.0 - g.g2) * a1000;
    c10 += g.g1B * g.g2M * g.g1 * a1011;
    c10 += g.g12 * g.g2B * (2.0 - g.g2);
    c10 += g.g11 * g.g20;
    c11 = 0.0;
    c11 += g.g11 * g.g21 * ahet0011;
    c11 += g.g1M * g.g2B * g.g2 * a1101;
    c11 += g.g1B * g.g2M * g.g1 * a1110;
    c11 += g.g12 * g.g2B * g.g2;
    c11 += g.g11 * g.g22;
}

// src/loops.jl:15-36 (qp_block!): k ascending, no fused multiply-add.
inline void qp4(const double* q, const double* p, int K, int64_t i, int64_t j, double qp[4]) {
    qp[0] = qp[1] = qp[2] = qp[3] = 0.0;
    const double* qi = q + (int64_t)K * i;
    const double* pj = p + (int64_t)K * 4 * j;
    for (int k = 0; k < K; ++k) {
        qp[0] += qi[k] * pj[k];
        qp[1] += qi[k] * pj[K + k];
        qp[2] += qi[k] * pj[2 * K + k];
        qp[3] += qi[k] * pj[3 * K + k];
    }
}

inline GMask pair_mask(const uint8_t* bed, int64_t bps, int64_t i, int64_t j) {
    return gmask(code_to_g(bed_code(bed, bps, i, 2 * j)), code_to_g(bed_code(bed, bps, i, 2 * j + 1)));
}

// src/loops.jl:157-212 (loglikelihood_full_loop): the branchy formula.
inline double ll_formula1(double g1, double g2, const double qp[4]) {
    double qp00 = qp[0], qp01 = qp[1], qp10 = qp[2], qp11 = qp[3];
    if (g1 == 0 && g2 == 0) return 2 * std::log(qp00);
    if (g1 == 0 && g2 == 2) return 2 * std::log(qp01);
    if (g1 == 2 && g2 == 0) return 2 * std::log(qp10);
    if (g1 == 2 && g2 == 2) return 2 * std::log(qp11);
    if (g1 == 3 && g2 == 0) return 2 * std::log(qp00 + qp10);
    if (g1 == 3 && g2 == 2) return 2 * std::log(qp01 + qp11);
    if (g1 == 0 && g2 == 3) return 2 * std::log(qp00 + qp01);
    if (g1 == 2 && g2 == 3) return 2 * std::log(qp10 + qp11);
    if (g1 == 3 && g2 == 1) return std::log(qp00 + qp10) + std::log(qp01 + qp11);
    if (g1 == 1 && g2 == 3) return std::log(qp00 + qp01) + std::log(qp10 + qp11);
    if (g1 == 0 && g2 == 1) return std::log(qp00) + std::log(qp01);
    if (g1 == 2 && g2 == 1) return std::log(qp10) + std::log(qp11);
    if (g1 == 1 && g2 == 0) return std::log(qp00) + std::log(qp10);
    if (g1 == 1 && g2 == 2) return std::log(qp01) + std::log(qp11);
    if (g1 == 1 && g2 == 1) return std::log(qp00 * qp11 + qp01 * qp10);
    return 0.0;
}

// ---------------------------------------------------------------- projection
// OpenADMIXTURE.project_q! contract (called at src/utils.jl:24 and
// src/algorithms_inner.jl:75,178,206; src/algorithms_outer.jl:16,144):
// Euclidean projection of v (n entries, stride st) onto {x >= eps, sum x = 1},
// by Chen & Ye (2011) on y = v - eps with target sum 1 - n*eps.
void project_simplex(double* v, int n, int64_t st, double eps) {
    double y[64];
    int idx[64];
    for (int a = 0; a < n; ++a) { y[a] = v[a * st] - eps; idx[a] = a; }
    // descending order (stable insertion sort)
    for (int a = 1; a < n; ++a) {
        int t = idx[a];
        int b = a - 1;
        while (b >= 0 && y[idx[b]] < y[t]) { idx[b + 1] = idx[b]; --b; }
        idx[b + 1] = t;
    }
    double target = 1.0 - n * eps;
    double tsum = 0.0, tmax = 0.0;
    bool found = false;
    for (int a = 0; a < n - 1; ++a) {
        tsum = tsum + y[idx[a]];
        tmax = (tsum - target) / (a + 1);
        if (tmax >= y[idx[a + 1]]) { found = true; break; }
    }
    if (!found) tmax = (tsum + y[idx[n - 1]] - target) / n;
    for (int a = 0; a < n; ++a) {
        double t = y[a] - tmax;
        v[a * st] = (t > 0.0 ? t : 0.0) + eps;
    }
}

// ---------------------------------------------------------------- QP
// Exact minimiser of 0.5 d'Hd - z'd subject to lo <= d <= hi and ngrp
// equality groups: ngrp = 0, none; ngrp = 1, sum(d) = 0; ngrp = G >= 2,
// sum over {a : a % G == k} of d_a = 0 for every k < G.  Primal active-set
// method from the feasible start d = 0; H is n x n column-major, SPD on the
// subspaces visited.  This restates the contract of OpenADMIXTURE's
// create_tableau!/quadratic_program! pair as used at
// src/algorithms_inner.jl:160-166 (K variables, one equality), :303-305
// (4K variables, penalty form, no equality) and :307-310 (4K variables, K
// equalities: the P quartets of each ancestry sum to zero, variable h*K + k
// in group k).  With G >= 2 groups the multipliers solve the G x G Schur
// system S nu = E_F H_FF^-1 r + E_X d_X with S = E_F H_FF^-1 E_F'; a group's
// last free variable is determined by its equality and never blocks the
// ratio test, so every group keeps a free variable and S stays definite.
// Returns iterations used, or -1 when the iteration cap was hit (d is then
// the last feasible iterate).
int qp_active_set(int n, const double* H, const double* z, const double* lo, const double* hi,
                  int ngrp, double* d) {
    enum { FREE = 0, AT_LO = 1, AT_HI = 2 };
    const int G = ngrp;
    std::vector<int> st(n, FREE);
    std::vector<double> A(n * n), r(n), y1(n), y2(n), g(n);
    std::vector<double> Y((size_t)n * std::max(G, 1)), S((size_t)G * G), nug(std::max(G, 1), 0.0);
    std::vector<int> F(n), nfree(std::max(G, 1));
    for (int a = 0; a < n; ++a) {
        d[a] = 0.0;
        if (lo[a] >= 0.0 && hi[a] <= 0.0) st[a] = AT_LO;  // degenerate box: pinned at 0
    }
    double zscale = 1.0;
    for (int a = 0; a < n; ++a) zscale = std::max(zscale, std::fabs(z[a]));
    const double tol = 1e-12 * zscale;
    const int max_iter = 4 * n + 20;
    for (int it = 0; it < max_iter; ++it) {
        int nF = 0;
        for (int a = 0; a < n; ++a) if (st[a] == FREE) F[nF++] = a;
        double nu = 0.0;
        std::vector<double> dstar(nF);
        if (nF > 0) {
            // r = z_F - H_{F,X} d_X
            for (int a = 0; a < nF; ++a) {
                int fa = F[a];
                double s = z[fa];
                for (int b = 0; b < n; ++b) if (st[b] != FREE) s -= H[fa + (int64_t)n * b] * d[b];
                r[a] = s;
                for (int b = 0; b < nF; ++b) A[a + nF * b] = H[fa + (int64_t)n * F[b]];
            }
            // Cholesky A = L L' (lower, in place)
            double maxdiag = 0.0;
            for (int a = 0; a < nF; ++a) maxdiag = std::max(maxdiag, std::fabs(A[a + nF * a]));
            const double floor_piv = 1e-300 + 1e-14 * maxdiag;
            for (int c = 0; c < nF; ++c) {
                double s = A[c + nF * c];
                for (int k = 0; k < c; ++k) s -= A[c + nF * k] * A[c + nF * k];
                if (!(s > floor_piv)) s = floor_piv;
                double lcc = std::sqrt(s);
                A[c + nF * c] = lcc;
                for (int rr = c + 1; rr < nF; ++rr) {
                    double t = A[rr + nF * c];
                    for (int k = 0; k < c; ++k) t -= A[rr + nF * k] * A[c + nF * k];
                    A[rr + nF * c] = t / lcc;
                }
            }
            auto solve = [&](std::vector<double>& x) {
                for (int a = 0; a < nF; ++a) {
                    double t = x[a];
                    for (int k = 0; k < a; ++k) t -= A[a + nF * k] * x[k];
                    x[a] = t / A[a + nF * a];
                }
                for (int a = nF - 1; a >= 0; --a) {
                    double t = x[a];
                    for (int k = a + 1; k < nF; ++k) t -= A[k + nF * a] * x[k];
                    x[a] = t / A[a + nF * a];
                }
            };
            for (int a = 0; a < nF; ++a) y1[a] = r[a];
            solve(y1);
            if (G >= 2) {
                // Y = H_FF^-1 E_F' (column k: indicator of group k), S = E_F Y
                for (int k = 0; k < G; ++k) {
                    for (int a = 0; a < nF; ++a) y2[a] = (F[a] % G == k) ? 1.0 : 0.0;
                    solve(y2);
                    for (int a = 0; a < nF; ++a) Y[a + (size_t)nF * k] = y2[a];
                }
                std::vector<double> rhs(G, 0.0);
                for (int k = 0; k < G; ++k)
                    for (int l = 0; l < G; ++l) S[k + G * l] = 0.0;
                for (int a = 0; a < nF; ++a) {
                    const int k = F[a] % G;
                    rhs[k] += y1[a];
                    for (int l = 0; l < G; ++l) S[k + G * l] += Y[a + (size_t)nF * l];
                }
                for (int b = 0; b < n; ++b)
                    if (st[b] != FREE) rhs[b % G] += d[b];
                // Cholesky of the G x G Schur complement, then S nu = rhs
                double smax = 0.0;
                for (int k = 0; k < G; ++k) smax = std::max(smax, std::fabs(S[k + G * k]));
                const double sfl = 1e-300 + 1e-14 * smax;
                for (int c = 0; c < G; ++c) {
                    double s = S[c + G * c];
                    for (int k = 0; k < c; ++k) s -= S[c + G * k] * S[c + G * k];
                    if (!(s > sfl)) s = sfl;
                    const double lcc = std::sqrt(s);
                    S[c + G * c] = lcc;
                    for (int rr = c + 1; rr < G; ++rr) {
                        double t = S[rr + G * c];
                        for (int k = 0; k < c; ++k) t -= S[rr + G * k] * S[c + G * k];
                        S[rr + G * c] = t / lcc;
                    }
                }
                for (int a = 0; a < G; ++a) {
                    double t = rhs[a];
                    for (int k = 0; k < a; ++k) t -= S[a + G * k] * nug[k];
                    nug[a] = t / S[a + G * a];
                }
                for (int a = G - 1; a >= 0; --a) {
                    double t = nug[a];
                    for (int k = a + 1; k < G; ++k) t -= S[k + G * a] * nug[k];
                    nug[a] = t / S[a + G * a];
                }
                for (int a = 0; a < nF; ++a) {
                    double t = y1[a];
                    for (int l = 0; l < G; ++l) t -= Y[a + (size_t)nF * l] * nug[l];
                    dstar[a] = t;
                }
            } else if (G == 1) {
                for (int a = 0; a < nF; ++a) y2[a] = 1.0;
                solve(y2);
                double cfix = 0.0;
                for (int b = 0; b < n; ++b) if (st[b] != FREE) cfix -= d[b];
                double s1 = 0.0, s2 = 0.0;
                for (int a = 0; a < nF; ++a) { s1 += y1[a]; s2 += y2[a]; }
                nu = (s1 - cfix) / s2;
                for (int a = 0; a < nF; ++a) dstar[a] = y1[a] - nu * y2[a];
            } else {
                for (int a = 0; a < nF; ++a) dstar[a] = y1[a];
            }
        }
        // ratio test along s = dstar - d_F
        double alpha = 1.0;
        int blk = -1, blk_to = FREE;
        if (G >= 2) {
            for (int k = 0; k < G; ++k) nfree[k] = 0;
            for (int a = 0; a < nF; ++a) nfree[F[a] % G]++;
        }
        for (int a = 0; a < nF; ++a) {
            int fa = F[a];
            if (G >= 2 && nfree[fa % G] == 1) continue;   // fixed by its group's equality
            double s = dstar[a] - d[fa];
            if (s < 0.0) {
                double ra = (lo[fa] - d[fa]) / s;
                if (ra < alpha) { alpha = ra; blk = fa; blk_to = AT_LO; }
            } else if (s > 0.0) {
                double ra = (hi[fa] - d[fa]) / s;
                if (ra < alpha) { alpha = ra; blk = fa; blk_to = AT_HI; }
            }
        }
        if (blk < 0) {
            for (int a = 0; a < nF; ++a) d[F[a]] = dstar[a];
            // multipliers of the fixed bounds
            for (int a = 0; a < n; ++a) {
                double s = -z[a];
                for (int b = 0; b < n; ++b) s += H[a + (int64_t)n * b] * d[b];
                g[a] = s + (G >= 2 ? nug[a % G] : nu);
            }
            int rel = -1;
            double worst = tol;
            for (int a = 0; a < n; ++a) {
                if (lo[a] >= 0.0 && hi[a] <= 0.0) continue;
                double v = 0.0;
                if (st[a] == AT_LO) v = -g[a];
                else if (st[a] == AT_HI) v = g[a];
                if (v > worst) { worst = v; rel = a; }
            }
            if (rel < 0) return it + 1;
            st[rel] = FREE;
        } else {
            if (alpha < 0.0) alpha = 0.0;
            for (int a = 0; a < nF; ++a) {
                int fa = F[a];
                d[fa] = d[fa] + alpha * (dstar[a] - d[fa]);
            }
            d[blk] = (blk_to == AT_LO) ? lo[blk] : hi[blk];
            st[blk] = blk_to;
        }
    }
    return -1;
}

struct Dims {
    const uint8_t* bed;
    int64_t bps, nsnp, I, J;
    int K;
};

// ---------------------------------------------------------------- passes
// src/loops.jl:236-258 (formula 2) and 157-212 (formula 1).  The total is
// summed per block j over i ascending, then over j ascending (a fixed order,
// so the value does not depend on the thread count).
double loglik(const Dims& D, const double* q, const double* p, int formula, int nthreads) {
    std::vector<double> per_j(D.J, 0.0);
    parallel_for(D.J, nthreads, [&](int64_t j0, int64_t j1) {
        for (int64_t j = j0; j < j1; ++j) {
            double r = 0.0;
            for (int64_t i = 0; i < D.I; ++i) {
                double qp[4];
                qp4(q, p, D.K, i, j, qp);
                GMask g = pair_mask(D.bed, D.bps, i, j);
                if (formula == 1) {
                    r += ll_formula1(g.g1, g.g2, qp);
                } else {
                    double a1, a2, b1, b2;
                    coefs_likelihood(g, qp[0], qp[1], qp[2], qp[3], a1, a2, b1, b2);
                    r += std::log(a1 + a2) + std::log(b1 + b2);
                }
            }
            per_j[j] = r;
        }
    });
    double s = 0.0;
    for (int64_t j = 0; j < D.J; ++j) s += per_j[j];
    return s;
}

// src/loops.jl:260-295 (em_loop!): raw EM numerators.  q_next summed over j
// ascending per individual; p_next summed over i ascending per haplotype column.
void em_accum(const Dims& D, const double* q, const double* p, double* qn, double* pn, int nthreads) {
    const int K = D.K;
    parallel_for(D.I, nthreads, [&](int64_t i0, int64_t i1) {
        for (int64_t i = i0; i < i1; ++i) {
            double* out = qn + (int64_t)K * i;
            for (int k = 0; k < K; ++k) out[k] = 0.0;
            const double* qi = q + (int64_t)K * i;
            for (int64_t j = 0; j < D.J; ++j) {
                double qp[4], c[4];
                qp4(q, p, K, i, j, qp);
                GMask g = pair_mask(D.bed, D.bps, i, j);
                coefs(g, qp[0], qp[1], qp[2], qp[3], c[0], c[1], c[2], c[3]);
                const double* pj = p + (int64_t)K * 4 * j;
                for (int k = 0; k < K; ++k) {
                    out[k] += c[0] * qi[k] * pj[k] / qp[0];
                    out[k] += c[1] * qi[k] * pj[K + k] / qp[1];
                    out[k] += c[2] * qi[k] * pj[2 * K + k] / qp[2];
                    out[k] += c[3] * qi[k] * pj[3 * K + k] / qp[3];
                }
            }
        }
    });
    parallel_for(D.J, nthreads, [&](int64_t j0, int64_t j1) {
        for (int64_t j = j0; j < j1; ++j) {
            double* out = pn + (int64_t)K * 4 * j;
            for (int a = 0; a < 4 * K; ++a) out[a] = 0.0;
            const double* pj = p + (int64_t)K * 4 * j;
            for (int64_t i = 0; i < D.I; ++i) {
                double qp[4], c[4];
                qp4(q, p, K, i, j, qp);
                GMask g = pair_mask(D.bed, D.bps, i, j);
                coefs(g, qp[0], qp[1], qp[2], qp[3], c[0], c[1], c[2], c[3]);
                const double* qi = q + (int64_t)K * i;
                for (int k = 0; k < K; ++k) {
                    for (int h = 0; h < 4; ++h)
                        out[h * K + k] += c[h] * qi[k] * pj[h * K + k] / qp[h];
                }
            }
        }
    });
}

// src/loops.jl:328-365 (update_q_loop!): Xtz_q, XtX_q; j ascending per i.
void accum_q(const Dims& D, const double* q, const double* p, double* XtX, double* Xtz, int nthreads) {
    const int K = D.K;
    parallel_for(D.I, nthreads, [&](int64_t i0, int64_t i1) {
        for (int64_t i = i0; i < i1; ++i) {
            double* H = XtX + (int64_t)K * K * i;
            double* g = Xtz + (int64_t)K * i;
            for (int a = 0; a < K * K; ++a) H[a] = 0.0;
            for (int k = 0; k < K; ++k) g[k] = 0.0;
            for (int64_t j = 0; j < D.J; ++j) {
                double qp[4], c[4];
                qp4(q, p, K, i, j, qp);
                GMask gm = pair_mask(D.bed, D.bps, i, j);
                coefs(gm, qp[0], qp[1], qp[2], qp[3], c[0], c[1], c[2], c[3]);
                const double* pj = p + (int64_t)K * 4 * j;
                for (int k = 0; k < K; ++k) {
                    for (int h = 0; h < 4; ++h) g[k] += c[h] * pj[h * K + k] / qp[h];
                    for (int k2 = 0; k2 < K; ++k2) {
                        for (int h = 0; h < 4; ++h)
                            H[k2 + K * k] += c[h] * pj[h * K + k] * pj[h * K + k2] / (qp[h] * qp[h]);
                    }
                }
            }
        }
    });
}

// src/loops.jl:367-403 (update_p_loop!): Xtz_p, XtX_p; i ascending per block.
void accum_p(const Dims& D, const double* q, const double* p, double* XtX, double* Xtz, int nthreads) {
    const int K = D.K;
    parallel_for(D.J, nthreads, [&](int64_t j0, int64_t j1) {
        for (int64_t j = j0; j < j1; ++j) {
            for (int h = 0; h < 4; ++h) {
                int64_t m = 4 * j + h;
                for (int a = 0; a < K * K; ++a) XtX[(int64_t)K * K * m + a] = 0.0;
                for (int k = 0; k < K; ++k) Xtz[(int64_t)K * m + k] = 0.0;
            }
            for (int64_t i = 0; i < D.I; ++i) {
                double qp[4], c[4];
                qp4(q, p, K, i, j, qp);
                GMask gm = pair_mask(D.bed, D.bps, i, j);
                coefs(gm, qp[0], qp[1], qp[2], qp[3], c[0], c[1], c[2], c[3]);
                const double* qi = q + (int64_t)K * i;
                for (int k = 0; k < K; ++k) {
                    for (int h = 0; h < 4; ++h) Xtz[(int64_t)K * (4 * j + h) + k] += c[h] * qi[k] / qp[h];
                    for (int k2 = 0; k2 < K; ++k2)
                        for (int h = 0; h < 4; ++h)
                            XtX[(int64_t)K * K * (4 * j + h) + k2 + K * k] +=
                                c[h] * qi[k] * qi[k2] / (qp[h] * qp[h]);
                }
            }
        }
    });
}

void project_q_all(double* q, int K, int64_t ncol, double eps, int nthreads) {
    parallel_for(ncol, nthreads, [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b; ++i) project_simplex(q + (int64_t)K * i, K, 1, eps);
    });
}
// src/utils.jl:20-28 (project_p!): each (k, block) quartet p[k, 4j:4j+3].
void project_p_all(double* p, int K, int64_t J, double eps, int nthreads) {
    parallel_for(J, nthreads, [&](int64_t a, int64_t b) {
        for (int64_t j = a; j < b; ++j)
            for (int k = 0; k < K; ++k) project_simplex(p + (int64_t)K * 4 * j + k, 4, K, eps);
    });
}

// src/algorithms_inner.jl:134-168 (non-penalty branch) for every individual.
// Xtz is the gradient as accumulated (before the reference's `Xtz .*= -1`).
// pen_rho < 0: the default equality form (sum d = 0, src/algorithms_inner.jl:
// 163-166).  pen_rho >= 0: the penalty form of :158-162, H + rho 1 1' and no
// equality (the reference adds rho to the whole XtX array inside the loop over
// i, algorithms_inner.jl:159; the intended per-individual penalty is used).
int qp_q_batch(int K, int64_t I, const double* XtX, const double* Xtz, const double* q, double* qdiff,
               int nthreads, double pen_rho = -1.0) {
    std::atomic<int> fails(0);
    parallel_for(I, nthreads, [&](int64_t a, int64_t b) {
        std::vector<double> lo(K), hi(K), H((size_t)K * K);
        for (int64_t i = a; i < b; ++i) {
            const double* qi = q + (int64_t)K * i;
            for (int k = 0; k < K; ++k) { lo[k] = 0.0 - qi[k]; hi[k] = 1.0 - qi[k]; }
            const double* Hi = XtX + (int64_t)K * K * i;
            if (pen_rho >= 0.0) {
                for (int e = 0; e < K * K; ++e) H[e] = Hi[e] + pen_rho;
                Hi = H.data();
            }
            int it = qp_active_set(K, Hi, Xtz + (int64_t)K * i, lo.data(), hi.data(), pen_rho < 0.0,
                                   qdiff + (int64_t)K * i);
            if (it < 0) fails++;
        }
    });
    return fails.load();
}

// src/algorithms_inner.jl:264-310: block-diagonal 4K x 4K Hessian (274-283).
// eq = 0: the penalty branch (the default), + rho on the (l,l2,k) pattern
// (295-305).  eq = 1: the equality branch (307-310), no penalty and the K
// equalities sum_h d[k, h] = 0.  Variable v = h*K + k <-> p[k, 4j+h].
int qp_p_batch(int K, int64_t J, const double* XtX, const double* Xtz, const double* p, double rho,
               double* pdiff, int nthreads, int eq = 0) {
    std::atomic<int> fails(0);
    const int n = 4 * K;
    parallel_for(J, nthreads, [&](int64_t a, int64_t b) {
        std::vector<double> H(n * n), lo(n), hi(n);
        for (int64_t j = a; j < b; ++j) {
            std::fill(H.begin(), H.end(), 0.0);
            for (int l = 0; l < 4; ++l)
                for (int k = 0; k < K; ++k)
                    for (int k2 = 0; k2 < K; ++k2)
                        H[(l * K + k2) + n * (l * K + k)] = XtX[(int64_t)K * K * (4 * j + l) + k2 + K * k];
            if (!eq)
                for (int l2 = 0; l2 < 4; ++l2)
                    for (int l = 0; l < 4; ++l)
                        for (int k = 0; k < K; ++k) H[(l * K + k) + n * (l2 * K + k)] += rho;
            const double* pj = p + (int64_t)n * j;
            for (int v = 0; v < n; ++v) { lo[v] = 0.0 - pj[v]; hi[v] = 1.0 - pj[v]; }
            int it = qp_active_set(n, H.data(), Xtz + (int64_t)n * j, lo.data(), hi.data(), eq ? K : 0,
                                   pdiff + (int64_t)n * j);
            if (it < 0) fails++;
        }
    });
    return fails.load();
}

// Dense (UtU - UtV) \ rhs by Gaussian elimination with partial pivoting
// (Julia's `\` on a square matrix).
void solve_small(int m, std::vector<double> A, std::vector<double>& b) {
    for (int c = 0; c < m; ++c) {
        int piv = c;
        for (int r = c + 1; r < m; ++r) if (std::fabs(A[r + m * c]) > std::fabs(A[piv + m * c])) piv = r;
        if (piv != c) {
            for (int k = 0; k < m; ++k) std::swap(A[c + m * k], A[piv + m * k]);
            std::swap(b[c], b[piv]);
        }
        double dc = A[c + m * c];
        for (int r = c + 1; r < m; ++r) {
            double f = A[r + m * c] / dc;
            for (int k = c; k < m; ++k) A[r + m * k] -= f * A[c + m * k];
            b[r] -= f * b[c];
        }
    }
    for (int r = m - 1; r >= 0; --r) {
        double t = b[r];
        for (int k = r + 1; k < m; ++k) t -= A[r + m * k] * b[k];
        b[r] = t / A[r + m * r];
    }
}

}  // namespace

// ============================================================== C interface
extern "C" {

int orc_bed_code(const uint8_t* bed, int64_t bps, int64_t i, int64_t snp) { return bed_code(bed, bps, i, snp); }

// Census of the 16 genotype-pair classes, index g1*4 + g2 with missing = 3.
void orc_census(const uint8_t* bed, int64_t bps, int64_t I, int64_t J, uint64_t* counts) {
    for (int a = 0; a < 16; ++a) counts[a] = 0;
    for (int64_t j = 0; j < J; ++j)
        for (int64_t i = 0; i < I; ++i) {
            int g1 = (int)code_to_g(bed_code(bed, bps, i, 2 * j));
            int g2 = (int)code_to_g(bed_code(bed, bps, i, 2 * j + 1));
            counts[g1 * 4 + g2]++;
        }
}

// src/utils.jl:1-18 (count_double_missing!): blocks of the whole SNP range
// (ceil(nsnp/2) blocks; an odd trailing SNP has no partner and is skipped).
void orc_count_double_missing(const uint8_t* bed, int64_t bps, int64_t I, int64_t nsnp, int64_t* dm) {
    int64_t Jf = nsnp / 2;
    for (int64_t i = 0; i < I; ++i) {
        int64_t c = 0;
        for (int64_t j = 0; j < Jf; ++j)
            if (bed_code(bed, bps, i, 2 * j) == 1 && bed_code(bed, bps, i, 2 * j + 1) == 1) c++;
        dm[i] = c;
    }
}

// Per-pair terms for one class (g1, g2 in {0,1,2,3=missing}) at given qp:
// out[0] = log-likelihood term by formula 2, out[1] = by formula 1,
// out[2..5] = c00,c01,c10,c11.
void orc_pair_terms(int g1, int g2, const double* qp, double* out) {
    GMask g = gmask(g1, g2);
    double a1, a2, b1, b2;
    coefs_likelihood(g, qp[0], qp[1], qp[2], qp[3], a1, a2, b1, b2);
    out[0] = std::log(a1 + a2) + std::log(b1 + b2);
    out[1] = ll_formula1(g1, g2, qp);
    coefs(g, qp[0], qp[1], qp[2], qp[3], out[2], out[3], out[4], out[5]);
}

double orc_loglik(const uint8_t* bed, int64_t bps, int64_t I, int64_t J, int K, const double* q,
                  const double* p, int formula, int nthreads) {
    Dims D{bed, bps, 0, I, J, K};
    return loglik(D, q, p, formula, nthreads);
}

void orc_em_accum(const uint8_t* bed, int64_t bps, int64_t I, int64_t J, int K, const double* q,
                  const double* p, double* q_next, double* p_next, int nthreads) {
    Dims D{bed, bps, 0, I, J, K};
    em_accum(D, q, p, q_next, p_next, nthreads);
}

void orc_accum_q(const uint8_t* bed, int64_t bps, int64_t I, int64_t J, int K, const double* q,
                 const double* p, double* XtX, double* Xtz, int nthreads) {
    Dims D{bed, bps, 0, I, J, K};
    accum_q(D, q, p, XtX, Xtz, nthreads);
}

void orc_accum_p(const uint8_t* bed, int64_t bps, int64_t I, int64_t J, int K, const double* q,
                 const double* p, double* XtX, double* Xtz, int nthreads) {
    Dims D{bed, bps, 0, I, J, K};
    accum_p(D, q, p, XtX, Xtz, nthreads);
}

void orc_project_q(double* q, int K, int64_t ncol, double eps) { project_q_all(q, K, ncol, eps, 1); }
void orc_project_p(double* p, int K, int64_t J, double eps) { project_p_all(p, K, J, eps, 1); }

int orc_qp_dense(int n, const double* H, const double* z, const double* lo, const double* hi, int eq, double* d) {
    return qp_active_set(n, H, z, lo, hi, eq, d);
}
int orc_qp_q(int K, int64_t I, const double* XtX, const double* Xtz, const double* q, double* qdiff, int nthreads) {
    return qp_q_batch(K, I, XtX, Xtz, q, qdiff, nthreads);
}
int orc_qp_p(int K, int64_t J, const double* XtX, const double* Xtz, const double* p, double rho, double* pdiff,
             int nthreads) {
    return qp_p_batch(K, J, XtX, Xtz, p, rho, pdiff, nthreads);
}
int orc_qp_p_eq(int K, int64_t J, const double* XtX, const double* Xtz, const double* p, double* pdiff,
                int nthreads) {
    return qp_p_batch(K, J, XtX, Xtz, p, 0.0, pdiff, nthreads, 1);
}

// src/algorithms_inner.jl:29-84 (em!, CPU branch): q_next ./= 2(J - dm);
// p_next normalised per (k, quartet); project both.
void orc_em_step(const uint8_t* bed, int64_t bps, int64_t I, int64_t J, int K, const int64_t* dm,
                 const double* q, const double* p, double* q_next, double* p_next, int nthreads) {
    Dims D{bed, bps, 0, I, J, K};
    em_accum(D, q, p, q_next, p_next, nthreads);
    for (int64_t i = 0; i < I; ++i) {
        double den = 2.0 * (double)(J - dm[i]);
        for (int k = 0; k < K; ++k) q_next[(int64_t)K * i + k] /= den;
    }
    for (int64_t j = 0; j < J; ++j)
        for (int k = 0; k < K; ++k) {
            double* c = p_next + (int64_t)K * 4 * j + k;
            double s = c[0] + c[K] + c[2 * K] + c[3 * K];
            for (int l = 0; l < 4; ++l) c[l * K] /= s;
        }
    project_q_all(q_next, K, I, 1e-5, nthreads);
    project_p_all(p_next, K, J, 1e-5, nthreads);
}

// src/algorithms_inner.jl:97-211 (update_q!, default branch): q_next =
// project(q + QP step).  Returns the number of QP problems that hit the cap.
int orc_update_q(const uint8_t* bed, int64_t bps, int64_t I, int64_t J, int K, const double* q, const double* p,
                 double* q_next, double* XtX_out, double* Xtz_out, int nthreads) {
    Dims D{bed, bps, 0, I, J, K};
    std::vector<double> XtX((size_t)K * K * I), Xtz((size_t)K * I), qd((size_t)K * I);
    accum_q(D, q, p, XtX.data(), Xtz.data(), nthreads);
    if (XtX_out) std::memcpy(XtX_out, XtX.data(), XtX.size() * sizeof(double));
    if (Xtz_out) std::memcpy(Xtz_out, Xtz.data(), Xtz.size() * sizeof(double));
    int f = qp_q_batch(K, I, XtX.data(), Xtz.data(), q, qd.data(), nthreads);
    for (int64_t a = 0; a < (int64_t)K * I; ++a) q_next[a] = q[a] + qd[a];
    project_q_all(q_next, K, I, 1e-5, nthreads);
    return f;
}

// src/algorithms_inner.jl:224-355 (update_p!, default penalty branch).
int orc_update_p(const uint8_t* bed, int64_t bps, int64_t I, int64_t J, int K, const double* q, const double* p,
                 double rho, double* p_next, double* XtX_out, double* Xtz_out, int nthreads) {
    Dims D{bed, bps, 0, I, J, K};
    std::vector<double> XtX((size_t)K * K * 4 * J), Xtz((size_t)K * 4 * J), pd((size_t)K * 4 * J);
    accum_p(D, q, p, XtX.data(), Xtz.data(), nthreads);
    if (XtX_out) std::memcpy(XtX_out, XtX.data(), XtX.size() * sizeof(double));
    if (Xtz_out) std::memcpy(Xtz_out, Xtz.data(), Xtz.size() * sizeof(double));
    int f = qp_p_batch(K, J, XtX.data(), Xtz.data(), p, rho, pd.data(), nthreads);
    for (int64_t a = 0; a < (int64_t)K * 4 * J; ++a) p_next[a] = p[a] + pd[a];
    project_p_all(p_next, K, J, 1e-5, nthreads);
    return f;
}

// The quasi-Newton point of admixture_qn! (src/algorithms_outer.jl:128-138):
// column c = (it-1) mod Qs of U/V gets x_next - x and x_next2 - x_next; with
// m = min(it, Qs) columns and d = x - x_next,
//   mode 0, ZAL (update_UV!/update_QN!, Zhou, Alexander & Lange 2011):
//     x_tmp = x_next - V (U'U - U'V)^{-1} U' d   (the multi-secant "good"
//     Broyden inverse with H0 = -I, secant pairs s = u, y = v - u);
//   mode 1, LBQN (update_UV_LBQN!/update_QN_LBQN!, the limited-memory Broyden
//     method of Agarwal & Xu): the multi-secant "bad" Broyden inverse
//     H = -I + V (Y'Y)^{-1} Y', Y = V - U, which satisfies H Y = U, giving
//     x_tmp = x_next - V ((U-V)'(U-V))^{-1} (U-V)' d.
// OpenADMIXTURE's LBQN code is not available here: this restates the
// published method, so its trajectory is not pinned to the reference's.
void qn_point(int64_t n, const double* x, const double* x_next, const double* x_next2, double* U, double* V,
              int Qs, int it, int mode, double* x_tmp) {
    int c = (it - 1) % Qs;
    for (int64_t a = 0; a < n; ++a) {
        U[a + n * c] = x_next[a] - x[a];
        V[a + n * c] = x_next2[a] - x_next[a];
    }
    int m = it < Qs ? it : Qs;
    std::vector<double> A(m * m), b(m);
    // ZAL: (U'U - U'V) c = U'd.  LBQN: Y'Y c = Y'd with Y = U - V formed per
    // element, so that a short Y (v close to u, slow EM) keeps its accuracy.
    for (int r = 0; r < m; ++r) {
        for (int s = 0; s < m; ++s) {
            double uu = 0.0, uv = 0.0, yy = 0.0;
            for (int64_t a = 0; a < n; ++a) {
                uu += U[a + n * r] * U[a + n * s];
                uv += U[a + n * r] * V[a + n * s];
                yy += (U[a + n * r] - V[a + n * r]) * (U[a + n * s] - V[a + n * s]);
            }
            A[r + m * s] = mode == 1 ? yy : uu - uv;
        }
        double t = 0.0, ty = 0.0;
        for (int64_t a = 0; a < n; ++a) {
            t += U[a + n * r] * (x[a] - x_next[a]);
            ty += (U[a + n * r] - V[a + n * r]) * (x[a] - x_next[a]);
        }
        b[r] = mode == 1 ? ty : t;
    }
    solve_small(m, A, b);
    for (int64_t a = 0; a < n; ++a) {
        double t = 0.0;
        for (int r = 0; r < m; ++r) t += V[a + n * r] * b[r];
        x_tmp[a] = x_next[a] - t;
    }
}
void orc_zal(int64_t n, const double* x, const double* x_next, const double* x_next2, double* U, double* V,
             int Qs, int it, double* x_tmp) {
    qn_point(n, x, x_next, x_next2, U, V, Qs, it, 0, x_tmp);
}
void orc_qn(int64_t n, const double* x, const double* x_next, const double* x_next2, double* U, double* V,
            int Qs, int it, int mode, double* x_tmp) {
    qn_point(n, x, x_next, x_next2, U, V, Qs, it, mode, x_tmp);
}

// Loop options of admixture_qn!/init_em! (src/algorithms_outer.jl:1-3, 38-41):
// fix_q / fix_p keep Q or P; guarantee_increase halves each update's step
// until the log-likelihood does not drop (src/algorithms_inner.jl:169-199 for
// Q with >=, :313-343 for P with >); penalty -1 is the default (P penalty
// form, Q equality form), 1 the penalty form for both, 0 the equality form
// for both (src/algorithms_outer.jl:58-64).
struct LoopOpts {
    int fix_q = 0, fix_p = 0, gi = 0, penalty = -1;
};

namespace {
// update_q! with the loop options; ll_tmp is d.ll_tmp.
void update_q_opts(const Dims& D, const double* q, const double* p, double* q_next, const LoopOpts& o, double rho,
                   double& ll_tmp, int nthreads) {
    const int K = D.K;
    const int64_t n = (int64_t)K * D.I;
    if (o.fix_q) { std::memcpy(q_next, q, n * sizeof(double)); return; }
    std::vector<double> XtX((size_t)K * K * D.I), Xtz((size_t)n), qd((size_t)n);
    accum_q(D, q, p, XtX.data(), Xtz.data(), nthreads);
    qp_q_batch(K, D.I, XtX.data(), Xtz.data(), q, qd.data(), nthreads, o.penalty == 1 ? rho : -1.0);
    double factor = 1.0;
    for (;;) {
        for (int64_t a = 0; a < n; ++a) q_next[a] = q[a] + factor * qd[a];
        project_q_all(q_next, K, D.I, 1e-5, nthreads);
        if (!o.gi) break;
        const double ll_new = loglik(D, q_next, p, 2, nthreads);
        if (ll_new >= ll_tmp) { ll_tmp = ll_new; break; }
        factor /= 2.0;
        if (factor < 1e-3) factor = 0.0;
        if (factor == 0.0) break;
    }
}
void update_p_opts(const Dims& D, const double* q, const double* p, double* p_next, const LoopOpts& o, double rho,
                   double& ll_tmp, int nthreads) {
    const int K = D.K;
    const int64_t n = (int64_t)K * 4 * D.J;
    if (o.fix_p) { std::memcpy(p_next, p, n * sizeof(double)); return; }
    std::vector<double> XtX((size_t)K * K * 4 * D.J), Xtz((size_t)n), pd((size_t)n);
    accum_p(D, q, p, XtX.data(), Xtz.data(), nthreads);
    qp_p_batch(K, D.J, XtX.data(), Xtz.data(), p, rho, pd.data(), nthreads, o.penalty == 0);
    double factor = 1.0;
    for (;;) {
        for (int64_t a = 0; a < n; ++a) p_next[a] = p[a] + factor * pd[a];
        project_p_all(p_next, K, D.J, 1e-5, nthreads);
        if (!o.gi) break;
        const double ll_new = loglik(D, q, p_next, 2, nthreads);
        if (ll_new > ll_tmp) { ll_tmp = ll_new; break; }
        factor /= 2.0;
        if (factor < 1e-3) factor = 0.0;
        if (factor == 0.0) break;
    }
}
}  // namespace

// src/algorithms_outer.jl:1-22 (init_em!) followed by :38-172 (admixture_qn!,
// mode = :ZAL, or :LBQN with mode 1) with the loop options above.  x (K x (I+4J)) holds the initial
// [q | p] and receives the final one; trace (optional, n_iter entries)
// receives ll after every outer iteration.  EM with fix_q / fix_p keeps that
// factor unchanged (the reference's em! rescales a fixed q before projecting
// it and rebinds p_next to p, algorithms_inner.jl:45-52, which is not
// restated).  Returns 0.
int orc_fit_ex(const uint8_t* bed, int64_t bps, int64_t nsnp, int64_t I, int64_t J, int K, int Qs, double* x,
               int n_iter, double rtol, int em_iters, double rho, int nthreads, double* ll_out, int* iters_out,
               double* trace, int fix_q, int fix_p, int guarantee_increase, int penalty, int mode) {
    LoopOpts o;
    o.fix_q = fix_q; o.fix_p = fix_p; o.gi = guarantee_increase; o.penalty = penalty;
    Dims D{bed, bps, nsnp, I, J, K};
    const int64_t n = (int64_t)K * (I + 4 * J);
    std::vector<int64_t> dm(I);
    orc_count_double_missing(bed, bps, I, nsnp, dm.data());
    std::vector<double> xn(n), xn2(n), xt(n), U(n * Qs, 0.0), V(n * Qs, 0.0);
    double* q = x;
    double* p = x + (int64_t)K * I;
    double ll_new = NAN;
    for (int e = 0; e < em_iters; ++e) {
        orc_em_step(bed, bps, I, J, K, dm.data(), q, p, xn.data(), xn.data() + (int64_t)K * I, nthreads);
        if (o.fix_q) std::memcpy(xn.data(), q, (size_t)K * I * sizeof(double));
        if (o.fix_p) std::memcpy(xn.data() + (int64_t)K * I, p, (size_t)K * 4 * J * sizeof(double));
        std::memcpy(x, xn.data(), n * sizeof(double));
        ll_new = loglik(D, q, p, 2, nthreads);
        project_p_all(p, K, J, 1e-5, nthreads);
        project_q_all(q, K, I, 1e-5, nthreads);
    }
    if (std::isnan(ll_new)) ll_new = loglik(D, q, p, 2, nthreads);
    int it = 0;
    for (it = 1; it <= n_iter; ++it) {
        double ll_prev = ll_new;
        double ll_tmp = ll_new;
        double* qn = xn.data();
        double* pn = xn.data() + (int64_t)K * I;
        double* qn2 = xn2.data();
        double* pn2 = xn2.data() + (int64_t)K * I;
        update_q_opts(D, q, p, qn, o, rho, ll_tmp, nthreads);
        update_p_opts(D, qn, p, pn, o, rho, ll_tmp, nthreads);
        update_q_opts(D, qn, pn, qn2, o, rho, ll_tmp, nthreads);
        update_p_opts(D, qn2, pn, pn2, o, rho, ll_tmp, nthreads);
        double ll_basic = loglik(D, qn2, pn2, 2, nthreads);
        qn_point(n, x, xn.data(), xn2.data(), U.data(), V.data(), Qs, it, mode, xt.data());
        project_p_all(xt.data() + (int64_t)K * I, K, J, 1e-5, nthreads);
        project_q_all(xt.data(), K, I, 1e-5, nthreads);
        double ll_qn = loglik(D, xt.data(), xt.data() + (int64_t)K * I, 2, nthreads);
        if (ll_basic < ll_qn) {
            std::memcpy(x, xt.data(), n * sizeof(double));
            ll_new = ll_qn;
        } else {
            std::memcpy(x, xn2.data(), n * sizeof(double));
            ll_new = ll_basic;
        }
        if (trace) trace[it - 1] = ll_new;
        double reldiff = std::fabs((ll_new - ll_prev) / ll_prev);
        if (reldiff < rtol) break;
    }
    if (ll_out) *ll_out = ll_new;
    if (iters_out) *iters_out = it > n_iter ? n_iter : it;
    return 0;
}

// The default options (src/driver.jl:38-58 defaults).
int orc_fit(const uint8_t* bed, int64_t bps, int64_t nsnp, int64_t I, int64_t J, int K, int Qs, double* x,
            int n_iter, double rtol, int em_iters, double rho, int nthreads, double* ll_out, int* iters_out,
            double* trace) {
    return orc_fit_ex(bed, bps, nsnp, I, J, K, Qs, x, n_iter, rtol, em_iters, rho, nthreads, ll_out, iters_out,
                      trace, 0, 0, 0, -1, 0);
}

// ---------------------------------------------------------------- synthetic
// Counter-based generator shared bit-for-bit with the device generator:
// SplitMix64 (Steele, Lea & Flood 2014) output at position idx of the stream
// keyed by (seed, stream); uniform double = top 53 bits * 2^-53.
static inline uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
static inline double unif(uint64_t seed, uint64_t stream, uint64_t idx) {
    uint64_t key = mix64(seed ^ (stream * 0x9E3779B97F4A7C15ULL));
    uint64_t r = mix64(key + (idx + 1) * 0x9E3779B97F4A7C15ULL);
    return (double)(r >> 11) * (1.0 / 9007199254740992.0);
}

// Genotypes of a synthetic admixed cohort: per (i, j) two haplotype copies,
// ancestry z ~ Cat(Q_i) by cumQ (K x I cumulative sums), haplotype
// h ~ Cat(P_zj) by cumP (K x 4J cumulative over each quartet); missing code
// 0b01 at rate miss per (i, SNP).  Writes the SNP-major BED matrix
// (bps = ceil(I/4) bytes per SNP, 2J SNPs, padding bits zero).
void orc_synth(uint64_t seed, int64_t I, int64_t J, int K, const double* cumQ, const double* cumP, double miss,
               uint8_t* bed, int nthreads) {
    const int64_t bps = (I + 3) / 4;
    std::memset(bed, 0, (size_t)bps * 2 * J);
    parallel_for(J, nthreads, [&](int64_t j0, int64_t j1) {
        for (int64_t j = j0; j < j1; ++j) {
            for (int64_t i = 0; i < I; ++i) {
                int a1 = 0, a2 = 0;
                for (int c = 0; c < 2; ++c) {
                    uint64_t idx = ((uint64_t)i * (uint64_t)J + (uint64_t)j) * 2 + c;
                    double u = unif(seed, 0, idx);
                    int z = K - 1;
                    for (int k = 0; k < K; ++k) if (u < cumQ[(int64_t)K * i + k]) { z = k; break; }
                    double u2 = unif(seed, 1, idx);
                    int h = 3;
                    for (int l = 0; l < 4; ++l) if (u2 < cumP[(int64_t)K * (4 * j + l) + z]) { h = l; break; }
                    a1 += h >> 1;
                    a2 += h & 1;
                }
                int cnt[2] = {a1, a2};
                for (int s = 0; s < 2; ++s) {
                    int64_t snp = 2 * j + s;
                    int code = cnt[s] == 0 ? 0 : (cnt[s] == 1 ? 2 : 3);
                    if (unif(seed, 2, (uint64_t)i * (uint64_t)(2 * J) + (uint64_t)snp) < miss) code = 1;
                    bed[snp * bps + (i >> 2)] |= (uint8_t)(code << ((i & 3) << 1));
                }
            }
        }
    });
}

}  // extern "C"
