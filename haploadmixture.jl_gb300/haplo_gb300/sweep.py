"""K sweep with random restarts on one GPU (for example K = 2..10 x 4
restarts on one cohort of I = 20,000 individuals x 40,000 SNPs).

The reference fits one K per run_admixture call (src/driver.jl:38-79) and
names AIC-based model selection only in its README (README.md:9).  Here all
fits share one decoded genotype matrix (hx_create_shared) and run
concurrently (hx_fit_many): each fit has its own context and CUDA stream, so
the small fits' kernels overlap on the GPU.  Every fit returns exactly what
it returns when run alone.
"""
import ctypes as C

import numpy as np

from . import _lib
from .admix import GB300Admix, random_init


def aic(ll, I, J, K):
    """AIC = 2 [(K-1) I + 3 K J] - 2 ll: K-1 free Q entries per individual and
    3 free haplotype frequencies per (ancestry, block)."""
    return 2.0 * ((K - 1) * I + 3 * K * J) - 2.0 * ll


def fit_many(ctxs, n_iter=1000, rtol=1e-7, em_iters=5, threads=0):
    """hx_fit on every context concurrently; returns one info dict per context."""
    lib = _lib.load()
    n = len(ctxs)
    hs = (C.c_void_p * n)(*[c._h for c in ctxs])
    infos = (_lib.HxFitInfo * n)()
    status = (C.c_int32 * n)()
    st = lib.hx_fit_many(hs, n, n_iter, rtol, em_iters, threads, infos, status)
    if st != _lib.HX_OK:
        bad = [a for a in range(n) if status[a] != _lib.HX_OK]
        raise _lib.HxError(st, "fit %d failed: %s" % (bad[0], lib.hx_last_error(hs[bad[0]]).decode()))
    return [{f: getattr(infos[a], f) for f, _ in infos[a]._fields_ if f != "pad_"} for a in range(n)]


def k_sweep(bed, I, J, Ks, restarts=4, seed=0, precision="mixed", n_iter=1000, rtol=1e-7, em_iters=5,
            threads=0, keep=False, autotune=False, **create):
    """Fits every K in Ks from `restarts` random starts (random_init with seed
    seed + 1000 K + r).  Returns a list of dicts (K, restart, ll, aic, iters,
    converged, and q, p when keep=True), in (K, restart) order.  With
    autotune (mixed method), the first fit of each K tunes the grid splits of
    that K's passes at its start (hx_autotune) before the other restarts of
    the K are created, so they start with the same splits."""
    Ks = [int(k) for k in Ks]
    parent = GB300Admix(bed, I, J, Ks[0], precision=precision, **create)
    ctxs, specs = [], []
    for K in Ks:
        for r in range(restarts):
            d = parent if (K == Ks[0] and r == 0) else GB300Admix.shared(parent, K, precision=precision)
            q0, p0 = random_init(I, J, K, np.random.default_rng(seed + 1000 * K + r))
            d.set_qp(q0, p0)
            if autotune and r == 0 and precision == "mixed":
                d.autotune()
                d.set_qp(q0, p0)
            ctxs.append(d)
            specs.append((K, r))
    infos = fit_many(ctxs, n_iter=n_iter, rtol=rtol, em_iters=em_iters, threads=threads)
    out = []
    for (K, r), d, info in zip(specs, ctxs, infos):
        row = dict(K=K, restart=r, ll=info["ll"], aic=aic(info["ll"], I, J, K), iters=info["iters"],
                   converged=bool(info["converged"]), seconds=info["seconds"])
        if keep:
            row["q"], row["p"] = d.get_qp()
        out.append(row)
    for d in ctxs:
        if d is not parent:
            d.close()
    parent.close()
    return out


def _main():
    """python -m haplo_gb300.sweep [--config C4] [--Ks 2-10] [--restarts 4]:
    the synthetic K sweep; prints one JSON line per fit and a summary line."""
    import argparse
    import json
    import time
    from . import synth
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="C4")
    ap.add_argument("--Ks", default="2-10")
    ap.add_argument("--restarts", type=int, default=4)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--rtol", type=float, default=1e-7)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--sequential", action="store_true", help="also time the fits one after another")
    ap.add_argument("--autotune", action="store_true", help="tune each K's grid splits on its first fit")
    a = ap.parse_args()
    lo, hi = (int(x) for x in a.Ks.split("-"))
    Ks = list(range(lo, hi + 1))
    cfg = synth.config(a.config)
    import torch
    I, J = cfg["I"], cfg["J"]
    bps = (I + 3) // 4
    dev = torch.empty(bps * 2 * J, dtype=torch.uint8, device="cuda")
    synth.synth_device(cfg["seed"], cfg["Q"], cfg["P"], cfg["miss"], dev.data_ptr())
    bed = dev.cpu().numpy().reshape(2 * J, bps)
    t0 = time.time()
    rows = k_sweep(bed, I, J, Ks, restarts=a.restarts, precision=a.precision, rtol=a.rtol, threads=a.threads,
                   autotune=a.autotune)
    t_batch = time.time() - t0
    for r in rows:
        print(json.dumps(r))
    summary = {"config": a.config, "I": I, "J": J, "Ks": a.Ks, "restarts": a.restarts, "fits": len(rows),
               "autotune": a.autotune, "outer_iters": sum(r["iters"] for r in rows),
               "seconds_concurrent": t_batch, "best_K_by_aic": min(rows, key=lambda r: r["aic"])["K"]}
    if a.sequential:
        t0 = time.time()
        k_sweep(bed, I, J, Ks, restarts=a.restarts, precision=a.precision, rtol=a.rtol, threads=1)
        summary["seconds_one_at_a_time"] = time.time() - t0
    print(json.dumps(summary))


if __name__ == "__main__":
    _main()
