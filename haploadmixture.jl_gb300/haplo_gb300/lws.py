"""Learned warm start of Q (no reference counterpart).

A small permutation-equivariant network maps, for each individual, the
per-ancestry block log-likelihood sums and the Q gradient at the current state
to a point on the simplex.  It is trained on (features, converged Q) pairs that
the fit itself produces on simulated cohorts, by the library's own CUDA
kernels (hx_lws_* in include/haplo_gb300.h: warp-per-sample forward and
backward, FP16 weights, FP32 accumulation, Adam).  In a fit it is applied after
a few plain outer iterations and kept only when it raises the log-likelihood;
the fit then converges to the plain method's optimum, so the converged
log-likelihood judges the network's error.

    python -m haplo_gb300.lws train --out lws_params.npy   # needs a GPU
"""
import ctypes as C
import os
import time

import numpy as np

from . import _lib
from .admix import GB300Admix, random_init

NPARAM = 8516
H = 64
PARAMS_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lws_params.npy")
_O = dict(W1=(0, (H, 2)), b1=(2 * H, (H,)), W2=(3 * H, (H, H)), U2=(3 * H + H * H, (H, H)),
          b2=(3 * H + 2 * H * H, (H,)), w3=(4 * H + 2 * H * H, (H,)), b3=(5 * H + 2 * H * H, ()))


def unpack(params):
    """Named views of a flat parameter vector (layout of hx_lws_*)."""
    out = {}
    for name, (off, shape) in _O.items():
        n = int(np.prod(shape)) if shape else 1
        out[name] = params[off:off + n].reshape(shape) if shape else params[off]
    return out


def init_params(seed=0):
    """He-style initialisation, FP32."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, dtype=np.float32)
    v = unpack(p)
    v["W1"][:] = rng.normal(0, 1.0, (H, 2))
    v["W2"][:] = rng.normal(0, np.sqrt(1.0 / H), (H, H))
    v["U2"][:] = rng.normal(0, np.sqrt(1.0 / H), (H, H))
    v["w3"][:] = rng.normal(0, np.sqrt(1.0 / H), H)
    return p


def load_params(path=PARAMS_PATH):
    return np.load(path).astype(np.float32)


def _torch():
    import torch
    return torch


def _dptr(t):
    return C.c_void_p(t.data_ptr())


def features(d):
    """Features at the context's current state: float32 array (I, K, 2)."""
    torch = _torch()
    f = torch.empty(d.I * d.K * 2, dtype=torch.float32, device="cuda")
    d._ck(d.lib.hx_lws_features(d._h, _dptr(f)))
    return f.cpu().numpy().reshape(d.I, d.K, 2)


def forward(feat, params):
    """Network output q (n, K) on the GPU (hx_lws_forward)."""
    torch = _torch()
    feat = np.ascontiguousarray(feat, dtype=np.float32)
    n, K = feat.shape[0], feat.shape[1]
    f = torch.from_numpy(feat.reshape(-1)).cuda()
    P = torch.from_numpy(np.ascontiguousarray(params, dtype=np.float32)).cuda()
    q = torch.empty(n * K, dtype=torch.float32, device="cuda")
    _lib.check(_lib.load().hx_lws_forward(_dptr(f), n, K, _dptr(P), _dptr(q), None))
    return q.cpu().numpy().reshape(n, K)


def grad(feat, target, params):
    """Mean cross-entropy and its gradient on the GPU (hx_lws_grad)."""
    torch = _torch()
    feat = np.ascontiguousarray(feat, dtype=np.float32)
    n, K = feat.shape[0], feat.shape[1]
    f = torch.from_numpy(feat.reshape(-1)).cuda()
    t = torch.from_numpy(np.ascontiguousarray(target, dtype=np.float32).reshape(-1)).cuda()
    P = torch.from_numpy(np.ascontiguousarray(params, dtype=np.float32)).cuda()
    g = torch.empty(NPARAM, dtype=torch.float32, device="cuda")
    loss = torch.empty(1, dtype=torch.float64, device="cuda")
    _lib.check(_lib.load().hx_lws_grad(_dptr(f), _dptr(t), n, K, _dptr(P), _dptr(g), _dptr(loss), None))
    return float(loss.item()), g.cpu().numpy()


def train(feat, target, params=None, steps=2000, batch=8192, lr=2e-3, seed=1, log_every=0):
    """Adam on random mini-batches with the library's kernels; returns
    (params, per-step batch losses)."""
    torch = _torch()
    feat = np.ascontiguousarray(feat, dtype=np.float32)
    n, K = feat.shape[0], feat.shape[1]
    f = torch.from_numpy(feat.reshape(-1)).cuda()
    t = torch.from_numpy(np.ascontiguousarray(target, dtype=np.float32).reshape(-1)).cuda()
    P = torch.from_numpy(np.ascontiguousarray(init_params() if params is None else params, dtype=np.float32)).cuda()
    m = torch.zeros(NPARAM, dtype=torch.float32, device="cuda")
    v = torch.zeros(NPARAM, dtype=torch.float32, device="cuda")
    losses = torch.empty(max(steps, 1), dtype=torch.float64, device="cuda")
    chunk = log_every or steps
    done = 0
    while done < steps:
        s = min(chunk, steps - done)
        _lib.check(_lib.load().hx_lws_train(_dptr(f), _dptr(t), n, K, _dptr(P), _dptr(m), _dptr(v), s, batch, lr,
                                            seed, done, C.c_void_p(losses.data_ptr() + 8 * done), None))
        done += s
        if log_every:
            print("step %d  loss %.5f" % (done, float(losses[done - 1].item())), flush=True)
    return P.cpu().numpy(), losses[:steps].cpu().numpy()


def warm_start(d, params, p_step=False):
    """Replaces Q by the network's prediction (and, with p_step, P by one P
    step at that Q) when that raises the log-likelihood
    (hx_lws_warm_start); returns True if it did."""
    acc = C.c_int32()
    P = np.ascontiguousarray(params, dtype=np.float32)
    d._ck(d.lib.hx_lws_warm_start(d._h, P.ctypes.data_as(C.c_void_p), int(p_step), C.byref(acc)))
    return bool(acc.value)


def fit(d, params=None, n_iter=1000, rtol=1e-7, em_iters=5, plain_iters=1, p_step=True):
    """The warm-started fit: init_em!, `plain_iters` outer iterations, the warm
    start (the network's Q and, with p_step, one P step at it, kept only if
    that raises the log-likelihood), then admixture_qn! to convergence (from a
    fresh QN history when the warm start was kept, else continuing the plain
    loop unchanged).  Returns the fit info with the total outer iterations,
    'warm_start_accepted' and the wall time.

    Without the P step the network's Q is judged at the current P, where the
    current Q (just optimised for that P by the Q step) is hard to beat, and
    after 3 outer iterations it was never kept; one iteration in, with the P
    step, it is kept on most cohorts."""
    t0 = time.time()
    d.init_em(em_iters)
    i1 = d.admixture_qn(n_iter=plain_iters, rtol=rtol) if plain_iters > 0 else {"converged": 0, "iters": 0}
    accepted = False
    if not i1["converged"]:
        accepted = warm_start(d, load_params() if params is None else params, p_step=p_step)
        if accepted:
            i2 = d.admixture_qn(n_iter=n_iter - i1["iters"], rtol=rtol)
        else:
            i2 = d.admixture_qn(n_iter=n_iter, rtol=rtol, iter_count_offset=i1["iters"])
        info = dict(i2)
        info["iters"] = i1["iters"] + i2["iters"]
    else:
        info = dict(i1)
    info.update(warm_start_accepted=accepted, seconds=time.time() - t0)
    return info


def align_labels(p_now, p_conv):
    """Ancestry permutation perm with p_conv[perm[k]] closest to p_now[k]
    (least total L1 distance between the K x 4J haplotype-frequency rows; an
    assignment problem, solved exactly).  The fit's labelling of ancestries is
    arbitrary and can still change after the point where features are taken,
    so a converged Q is only a target once its rows are put in the labelling
    of that point: target[k] = q_conv[perm[k]]."""
    from scipy.optimize import linear_sum_assignment
    cost = np.abs(p_now[:, None, :] - p_conv[None, :, :]).sum(axis=2)
    rows, cols = linear_sum_assignment(cost)
    perm = np.empty(p_now.shape[0], dtype=np.int64)
    perm[rows] = cols
    return perm


def training_set(cohorts=50, I=20000, J=5000, K=6, seed=20261209, em_iters=5, plain_iters=1, rtol=1e-7,
                 precision="mixed", align=True, verbose=False, stats=None, q_now_out=None):
    """(features, converged Q) pairs from the method's own fits on simulated
    cohorts: alpha in [0.1, 1], differentiation mix in [0.05, 0.5]; features
    are taken where the warm start applies (after init_em! and plain_iters
    outer iterations).  With align, each converged Q is permuted into the
    ancestry labelling of that point (align_labels on P).  stats (a list), if
    given, receives per cohort the share of individuals whose largest Q entry
    is the same ancestry at that point and at convergence, before and after
    the alignment."""
    torch = _torch()
    from . import synth
    rng = np.random.default_rng(seed)
    feats, targets = [], []
    bps = (I + 3) // 4
    for c in range(cohorts):
        alpha = float(rng.uniform(0.1, 1.0))
        mix = float(rng.uniform(0.05, 0.5))
        Q, P = synth.draw_params(I, J, K, alpha, "shared", seed + 17 * c, mix=mix)
        bed = torch.empty(bps * 2 * J, dtype=torch.uint8, device="cuda")
        synth.synth_device(seed + 31 * c, Q, P, 0.01, bed.data_ptr())
        torch.cuda.synchronize()
        d = GB300Admix(bed.data_ptr(), I, J, K, bytes_per_snp=bps, n_snp=2 * J, precision=precision,
                       bed_on_device=True)
        d.set_qp(*random_init(I, J, K, np.random.default_rng(seed + 7 * c)))
        d.init_em(em_iters)
        if plain_iters > 0:
            d.admixture_qn(n_iter=plain_iters, rtol=rtol)
        f = features(d)
        q_now, p_now = d.get_qp()
        d.admixture_qn(n_iter=1000, rtol=rtol, iter_count_offset=plain_iters)
        q_conv, p_conv = d.get_qp()
        perm = align_labels(p_now, p_conv) if align else np.arange(K)
        q = q_conv[perm].T.astype(np.float32)        # (I, K), labelling of the feature point
        if q_now_out is not None:
            q_now_out.append(q_now.T.astype(np.float32))
        if stats is not None:
            a_now = q_now.argmax(axis=0)
            stats.append({"agree_unaligned": float(np.mean(a_now == q_conv.argmax(axis=0))),
                          "agree_aligned": float(np.mean(a_now == q.argmax(axis=1))),
                          "perm": perm.tolist()})
        feats.append(f)
        targets.append(q)
        if verbose:
            print("cohort %d alpha %.2f mix %.2f ll %.6e" % (c, alpha, mix, d.ll_new), flush=True)
        d.close()
    return np.concatenate(feats), np.concatenate(targets)


def _evaluate(a):
    """Plain mixed fit vs the chosen fit (warm start) on a synthetic cohort of
    the named configuration, from the same random start: one JSON line."""
    import json
    torch = _torch()
    from . import synth
    cfg = synth.config(a.config)
    I, J, K = cfg["I"], cfg["J"], cfg["K"]
    bps = (I + 3) // 4
    bed = torch.empty(bps * 2 * J, dtype=torch.uint8, device="cuda")
    synth.synth_device(cfg["seed"], cfg["Q"], cfg["P"], cfg["miss"], bed.data_ptr())
    torch.cuda.synchronize()
    q0, p0 = random_init(I, J, K, np.random.default_rng(cfg["seed"] + 7))
    params = load_params(a.params)
    out = {"config": a.config, "I": I, "J": J, "K": K, "rtol": a.rtol}
    for name in ("plain", "chosen"):
        d = GB300Admix(bed.data_ptr(), I, J, K, bytes_per_snp=bps, n_snp=2 * J, precision="mixed",
                       bed_on_device=True)
        d.set_qp(q0, p0)
        torch.cuda.synchronize()
        t0 = time.time()
        info = d.fit(n_iter=1000, rtol=a.rtol, em_iters=5) if name == "plain" else fit(d, params, rtol=a.rtol)
        torch.cuda.synchronize()
        out[name] = {"seconds": time.time() - t0, "outer_iters": info["iters"], "ll": info["ll"],
                     "warm_start_accepted": info.get("warm_start_accepted")}
        d.close()
    out["ll_rel_diff"] = abs(out["chosen"]["ll"] - out["plain"]["ll"]) / abs(out["plain"]["ll"])
    out["speedup"] = out["plain"]["seconds"] / out["chosen"]["seconds"]
    print(json.dumps(out))


def _main():
    import argparse
    import json
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--cohorts", type=int, default=50)
    t.add_argument("--I", type=int, default=20000)
    t.add_argument("--J", type=int, default=5000)
    t.add_argument("--K", type=int, default=6)
    t.add_argument("--steps", type=int, default=3000)
    t.add_argument("--batch", type=int, default=8192)
    t.add_argument("--lr", type=float, default=2e-3)
    t.add_argument("--plain-iters", type=int, default=1)
    t.add_argument("--out", default=PARAMS_PATH)
    e = sub.add_parser("eval")
    e.add_argument("--config", default="C5")
    e.add_argument("--params", default=PARAMS_PATH)
    e.add_argument("--rtol", type=float, default=1e-8)
    a = ap.parse_args()
    if a.cmd == "eval":
        _evaluate(a)
        return
    t0 = time.time()
    X, T = training_set(cohorts=a.cohorts, I=a.I, J=a.J, K=a.K, plain_iters=a.plain_iters, verbose=True)
    t1 = time.time()
    params, losses = train(X, T, steps=a.steps, batch=a.batch, lr=a.lr, log_every=max(a.steps // 10, 1))
    t2 = time.time()
    np.save(a.out, params)
    print(json.dumps({"samples": int(X.shape[0]), "data_s": t1 - t0, "train_s": t2 - t1,
                      "loss_first": float(losses[0]), "loss_last": float(np.mean(losses[-50:])), "out": a.out}))


if __name__ == "__main__":
    _main()
