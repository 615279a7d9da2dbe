"""Test infrastructure: CPU restatement (numpy, FP64) of the learned warm
start -- its features and its network's forward pass, loss and gradient --
the checker of the hx_lws_* kernels.  Nothing in the product imports it.

Features of (individual i, ancestry k):
  a[i,k] = (1/n_i) sum_j log L_ij(e_k), with L from the reference likelihood
           (src/loops.jl:236-258, through orc_pair_terms) at qp = p[k, 4j..4j+3],
  f1 = a - max_k a,  f2 = (g - 1) sqrt(n_i), g = Xtz_q[k,i] / (2 n_i),
  n_i = J - dm_i.
Network: h1_k = relu(W1 x_k + b1), m = mean_k h1_k,
h2_k = relu(W2 h1_k + U2 m + b2), z_k = w3.h2_k + b3, q = softmax(z);
loss = -sum_k t_k log q_k, averaged over samples.  Weights are rounded to
FP16 (round16=True) as the kernels use them.
"""
import numpy as np

from . import oracle as O

H = 64
NPARAM = 8516
_O = dict(W1=(0, (H, 2)), b1=(2 * H, (H,)), W2=(3 * H, (H, H)), U2=(3 * H + H * H, (H, H)),
          b2=(3 * H + 2 * H * H, (H,)), w3=(4 * H + 2 * H * H, (H,)), b3=(5 * H + 2 * H * H, ()))
CODE_G = np.array([0, 3, 1, 2])   # BED code -> genotype (3 = missing), src/loops.jl:64-71


def unpack(params, round16=True):
    if round16:
        p = np.asarray(params, dtype=np.float32).astype(np.float16).astype(np.float64)
    else:
        p = np.asarray(params, dtype=np.float64)
    out = {}
    for name, (off, shape) in _O.items():
        n = int(np.prod(shape)) if shape else 1
        out[name] = p[off:off + n].reshape(shape) if shape else p[off]
    return out


def genotypes(b):
    """(2J, I) genotype codes 0/1/2/3=missing of the first 2J SNPs."""
    bed = np.asarray(b.data).reshape(-1, b.bps)[:2 * b.J]
    i = np.arange(b.I)
    codes = (bed[:, i >> 2] >> (2 * (i & 3))) & 3
    return CODE_G[codes]


def features(b, K, q, p):
    """float64 (I, K, 2)."""
    g = genotypes(b)
    g1, g2 = g[0::2], g[1::2]                      # (J, I)
    cls = g1 * 4 + g2
    p = np.asarray(p, dtype=np.float64).reshape(K, 4 * b.J)
    term = np.zeros((b.J, K, 16))
    for j in range(b.J):
        for k in range(K):
            qp = np.ascontiguousarray(p[k, 4 * j:4 * j + 4])
            for c in np.unique(cls[j]):
                term[j, k, c] = O.pair_terms(int(c) // 4, int(c) % 4, qp)[0] if c != 15 else 0.0
    a = np.zeros((b.I, K))
    for j in range(b.J):
        a += term[j][:, cls[j]].T
    n = (b.J - O.double_missing(b)).astype(np.float64)
    n[n <= 0] = 1.0
    a /= n[:, None]
    _, Xtz = O.accum_q(b, K, q, p)
    f = np.zeros((b.I, K, 2))
    f[:, :, 0] = a - a.max(axis=1, keepdims=True)
    g = np.asarray(Xtz).reshape(K, b.I).T / (2.0 * n[:, None])
    f[:, :, 1] = (g - 1.0) * np.sqrt(n)[:, None]
    return f


def forward(feat, params, round16=True):
    """q (n, K) and the activations."""
    w = unpack(params, round16)
    x = np.asarray(feat, dtype=np.float64)                       # (n, K, 2)
    a1 = x @ w["W1"].T + w["b1"]                                  # (n, K, H)
    h1 = np.maximum(a1, 0.0)
    m = h1.mean(axis=1)                                           # (n, H)
    c = m @ w["U2"].T + w["b2"]                                   # (n, H)
    a2 = h1 @ w["W2"].T + c[:, None, :]
    h2 = np.maximum(a2, 0.0)
    z = h2 @ w["w3"] + w["b3"]                                    # (n, K)
    z = z - z.max(axis=1, keepdims=True)
    q = np.exp(z)
    q /= q.sum(axis=1, keepdims=True)
    return q, dict(x=x, h1=h1, m=m, h2=h2, w=w)


def loss_grad(feat, target, params, round16=True):
    """Mean cross-entropy and its gradient (NPARAM, float64)."""
    q, s = forward(feat, params, round16)
    t = np.asarray(target, dtype=np.float64)
    n, K = q.shape
    loss = -(t * np.log(np.maximum(q, 1e-30))).sum() / n
    w, x, h1, m, h2 = s["w"], s["x"], s["h1"], s["m"], s["h2"]
    dz = (q - t) / n                                              # (n, K)
    g = {}
    g["w3"] = np.einsum("nk,nkh->h", dz, h2)
    g["b3"] = dz.sum()
    dh2 = dz[:, :, None] * w["w3"][None, None, :] * (h2 > 0)
    g["b2"] = dh2.sum(axis=(0, 1))
    g["W2"] = np.einsum("nku,nkv->uv", dh2, h1)
    sdh = dh2.sum(axis=1)                                         # (n, H)
    g["U2"] = sdh.T @ m
    dh1 = dh2 @ w["W2"] + (sdh @ w["U2"])[:, None, :] / K
    dh1 = dh1 * (h1 > 0)
    g["b1"] = dh1.sum(axis=(0, 1))
    g["W1"] = np.einsum("nkh,nkc->hc", dh1, x)
    flat = np.zeros(NPARAM)
    for name, (off, shape) in _O.items():
        v = np.asarray(g[name], dtype=np.float64).reshape(-1)
        flat[off:off + v.size] = v
    return loss, flat
