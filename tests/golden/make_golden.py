"""Generates tests/golden/golden_small.json: known answers for the per-pair
terms and for the passes on a tiny cohort.

This is an independent, exact-rational transcription of the reference's
mask arithmetic (src/loops.jl:38-155: @gcoefs, @coefs_likelihood, @coefs)
and of its loops (src/loops.jl:236-258, 260-295, 328-403), written with
Python Fractions so that no floating-point summation order enters the
expected values.  Only the final log() is taken in floating point.

    python tests/golden/make_golden.py
"""
import json
import math
import os
from fractions import Fraction as Fr

HERE = os.path.dirname(os.path.abspath(__file__))


def masks(g1, g2):
    m = {}
    m["g11"], m["g12"], m["g10"], m["g1M"], m["g1B"] = (int(g1 == 1), int(g1 == 2), int(g1 == 0), int(g1 == 3),
                                                          int(g1 != 3))
    m["g21"], m["g22"], m["g20"], m["g2M"], m["g2B"] = (int(g2 == 1), int(g2 == 2), int(g2 == 0), int(g2 == 3),
                                                          int(g2 != 3))
    return m


def coefs_likelihood(g1, g2, qp00, qp01, qp10, qp11):
    # src/loops.jl:85-104
    m = masks(g1, g2)
    g11, g12, g10, g1M = m["g11"], m["g12"], m["g10"], m["g1M"]
    g21, g22, g20, g2M = m["g21"], m["g22"], m["g20"], m["g2M"]
    a1 = (g1M * g2M + g11 * g21 * qp00 * qp11 +
          ((g1M + g10) * (g20 + g21) + g2M * (g10 + g11) + g11 * g20) * qp00 +
          ((g1M + g10 + g11) * g22) * qp01 + (g12 * (g2M + g20 + g21)) * qp10 + (g12 * g22) * qp11)
    a2 = g11 * g21 * qp01 * qp10 + g1M * (g20 + g21) * qp10 + g2M * (g10 + g11) * qp01 + (g1M * g22 + g12 * g2M) * qp11
    b1 = (g1M * g2M + g11 * g21 + (g10 * g20 + g1M * g20 + g10 * g2M) * qp00 + (g1M + g10) * (g21 + g22) * qp01 +
          (g11 + g12) * (g2M + g20) * qp10 + (g11 * g22 + g12 * (g21 + g22)) * qp11)
    b2 = (g1M * g21 + g1M * g22 + g11 * g2M + g12 * g2M) * qp11 + g1M * g20 * qp10 + g10 * g2M * qp01
    return a1 + a2, b1 + b2


def coefs(g1, g2, qp00, qp01, qp10, qp11):
    # src/loops.jl:114-155
    m = masks(g1, g2)
    g11, g12, g10, g1M, g1B = m["g11"], m["g12"], m["g10"], m["g1M"], m["g1B"]
    g21, g22, g20, g2M, g2B = m["g21"], m["g22"], m["g20"], m["g2M"], m["g2B"]
    a0001 = qp00 / (qp00 + qp01)
    a0010 = qp00 / (qp00 + qp10)
    a0100 = qp01 / (qp01 + qp00)
    a0111 = qp01 / (qp01 + qp11)
    a1000 = qp10 / (qp10 + qp00)
    a1011 = qp10 / (qp10 + qp11)
    a1101 = qp11 / (qp11 + qp01)
    a1110 = qp11 / (qp11 + qp10)
    ahet0011 = qp00 * qp11 / (qp00 * qp11 + qp01 * qp10)
    ahet0110 = qp01 * qp10 / (qp00 * qp11 + qp01 * qp10)
    c00 = (g11 * g21 * ahet0011 + g1M * g2B * (2 - g2) * a0010 + g1B * g2M * (2 - g1) * a0001 +
           g10 * g2B * (2 - g2) + g11 * g20)
    c01 = (g11 * g21 * ahet0110 + g1M * g2B * g2 * a0111 + g1B * g2M * (2 - g1) * a0100 + g10 * g2B * g2 +
           g11 * g22)
    c10 = (g11 * g21 * ahet0110 + g1M * g2B * (2 - g2) * a1000 + g1B * g2M * g1 * a1011 +
           g12 * g2B * (2 - g2) + g11 * g20)
    c11 = (g11 * g21 * ahet0011 + g1M * g2B * g2 * a1101 + g1B * g2M * g1 * a1110 + g12 * g2B * g2 + g11 * g22)
    return c00, c01, c10, c11


def code_to_g(c):
    return {0: 0, 1: 3, 2: 1, 3: 2}[c]


def lcg(state):
    state = (state * 6364136223846793005 + 1442695040888963407) % (1 << 64)
    return state, state >> 33


def main():
    out = {"pair_terms": [], "cohort": {}}
    qps = [[Fr(1, 10), Fr(2, 10), Fr(3, 10), Fr(4, 10)], [Fr(7, 13), Fr(1, 29), Fr(3, 17), Fr(5, 11)],
           [Fr(1, 100000), Fr(1, 2), Fr(1, 3), Fr(99, 1000)]]
    for qp in qps:
        for g1 in range(4):
            for g2 in range(4):
                A, B = coefs_likelihood(g1, g2, *qp)
                c = coefs(g1, g2, *qp)
                out["pair_terms"].append({"g1": g1, "g2": g2, "qp": [float(v) for v in qp],
                                          "ll": math.log(A) + math.log(B), "L": float(A * B),
                                          "c": [float(v) for v in c]})
    # tiny cohort: I individuals, J blocks, K populations; deterministic bytes
    I, J, K = 7, 5, 2
    bps = (I + 3) // 4
    st = 12345
    data = []
    for s in range(2 * J):
        row = []
        for b in range(bps):
            st, r = lcg(st)
            byte = r & 0xFF
            if b == bps - 1 and I % 4:   # zero padding bits
                byte &= (1 << (2 * (I % 4))) - 1
            row.append(byte)
        data.append(row)
    # rational q (K x I) and p (K x 4J) on the simplex
    q = [[None] * I for _ in range(K)]
    for i in range(I):
        a = Fr(i + 1, I + 3)
        q[0][i], q[1][i] = a, 1 - a
    p = [[None] * (4 * J) for _ in range(K)]
    for k in range(K):
        for j in range(J):
            w = [Fr(1 + ((3 * j + 5 * k + h * (k + 2)) % 7), 1) for h in range(4)]
            s = sum(w)
            for h in range(4):
                p[k][4 * j + h] = w[h] / s

    def geno(i, snp):
        byte = data[snp][i >> 2]
        return code_to_g((byte >> (2 * (i & 3))) & 3)

    ll = 0.0
    Xtz_q = [[Fr(0)] * I for _ in range(K)]
    XtX_q = [[[Fr(0)] * I for _ in range(K)] for _ in range(K)]   # [k2][k][i]
    Xtz_p = [[Fr(0)] * (4 * J) for _ in range(K)]
    XtX_p = [[[Fr(0)] * (4 * J) for _ in range(K)] for _ in range(K)]
    em_q = [[Fr(0)] * I for _ in range(K)]
    em_p = [[Fr(0)] * (4 * J) for _ in range(K)]
    for j in range(J):
        for i in range(I):
            qp = [sum(q[k][i] * p[k][4 * j + h] for k in range(K)) for h in range(4)]
            g1, g2 = geno(i, 2 * j), geno(i, 2 * j + 1)
            A, B = coefs_likelihood(g1, g2, *qp)
            ll += math.log(A) + math.log(B)
            c = coefs(g1, g2, *qp)
            for k in range(K):
                for h in range(4):
                    m = 4 * j + h
                    Xtz_q[k][i] += c[h] * p[k][m] / qp[h]
                    Xtz_p[k][m] += c[h] * q[k][i] / qp[h]
                    em_q[k][i] += c[h] * q[k][i] * p[k][m] / qp[h]
                    em_p[k][m] += c[h] * q[k][i] * p[k][m] / qp[h]
                    for k2 in range(K):
                        XtX_q[k2][k][i] += c[h] * p[k][m] * p[k2][m] / qp[h] ** 2
                        XtX_p[k2][k][m] += c[h] * q[k][i] * q[k2][i] / qp[h] ** 2
    fl = lambda M: [[float(v) for v in row] for row in M]  # noqa: E731
    out["cohort"] = {
        "I": I, "J": J, "K": K, "bytes_per_snp": bps, "bed": data,
        "q": fl(q), "p": fl(p), "loglik": ll,
        "Xtz_q": fl(Xtz_q), "XtX_q": [fl(M) for M in XtX_q],
        "Xtz_p": fl(Xtz_p), "XtX_p": [fl(M) for M in XtX_p],
        "em_q": fl(em_q), "em_p": fl(em_p),
    }
    with open(os.path.join(HERE, "golden_small.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
