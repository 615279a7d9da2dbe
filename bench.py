#!/usr/bin/env python
"""Time to converge of the HaploADMIXTURE fit on GB300.

Workload: synthetic admixed cohort of I=100,000 individuals x 200,000 SNPs
(100,000 two-SNP blocks), K=8, Q ~ Dirichlet(0.3), 1% missing (seeded; no
public dataset).  One step = one complete fit from the same random start:
init_em! (5 EM iterations) then admixture_qn! (ZAL) until
|dll/ll| < 1e-8, through the C ABI.  The genotype input (5 GB) is larger than
L2 (129 MB), so no flush is needed between steps.

  value : seconds per fit (lower is better), chosen method = mixed precision
          (FP32 per-pair arithmetic, FP64 totals/QP/QN), inputs resident in HBM
  e2e   : the same fit through the public API from host buffers, including
          the H2D copy of the .bed matrix and initial Q/P and the D2H of the
          fitted Q/P and log-likelihood
  roofline : dominant kernel, algorithmic bytes per launch / CUDA-event time
  plain_fp64 : the plain FP64 GPU method fitted to convergence once from the
          same start (the metric's comparison), with the chosen fit's
          log-likelihood and Q/P differences against it
  cpu_baseline : CPU oracle (C++ restatement, all host cores): each piece of
          the fit timed on a bounded slice or at full size, summed with the
          fit's iteration counts (extrapolated, labelled)

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "haploadmixture.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "s to converge (rel Δloglik<1e-8), I=1e5×2e5 SNPs K=8: chosen vs plain GPU"
# outer iterations of the I=1e5, J=1e5, K=8 fit measured on GB300 (26 at rtol
# 1e-8); used only to extrapolate the CPU reference arm, whose full fit takes
# hours
REF_ITERS_DEFAULT = 26


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="C3")
    ap.add_argument("--I", type=int, default=0, help="override the config's individuals (profiling)")
    ap.add_argument("--J", type=int, default=0, help="override the config's 2-SNP blocks (profiling)")
    ap.add_argument("--K", type=int, default=0, help="override the config's ancestral populations")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--rtol", type=float, default=1e-8)
    ap.add_argument("--n-iter", type=int, default=1000)
    ap.add_argument("--em-iters", type=int, default=5)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--plain-estimate", action="store_true",
                    help="time one EM and one outer iteration of the plain FP64 method instead of fitting it "
                         "to convergence (the default, about 11 minutes at I=1e5, J=1e5, K=8)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the planned grid splits (no hx_autotune)")
    ap.add_argument("--skfr", type=int, default=0, metavar="SPARSITY",
                    help="also time the AIM selection (hx_skfr) of SPARSITY blocks on the cohort, with the CPU "
                         "oracle on the same input beside it (oracle memory grows as I x SNPs: small configs)")
    ap.add_argument("--cpu-full-fit", action="store_true",
                    help="also fit the whole cohort with the CPU oracle from the same start (measured, not "
                         "extrapolated; hours at I=1e5, J=1e5; minutes at I=1e4, J=5e4)")
    ap.add_argument("--ref-iters", type=int, default=REF_ITERS_DEFAULT)
    ap.add_argument("--cpu-slice-blocks", type=int, default=0)
    return ap.parse_args(argv)


def load_peaks():
    """(hbm GB/s, bf16 TFLOP/s burst, bf16 TFLOP/s sustained, source)."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return (d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), d.get("bf16_tflops_sustained", 1700.0),
                "measured")
    return 6800.0, 1900.0, 1700.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def pass_bytes(kind, I, J, K):
    """Algorithmic HBM bytes of one launch of a pass kernel: genotype classes
    (4 bits per (individual, block) pair) + Q and P reads + outputs."""
    geno = I * J / 2.0
    qp = 8.0 * K * I + 32.0 * K * J
    if kind == "accum_q":
        return geno + qp + 8.0 * (K + K * (K + 1) / 2) * I
    if kind == "accum_p":
        return geno + qp + 8.0 * (K + K * K) * 4 * J
    if kind == "loglik":
        return geno + qp
    return None


def pass_flops(I, J, K):
    """Algorithmic FLOPs of one accumulation pass: the Hessian contraction
    F_H = 2 N 4 K(K+1)/2 (symmetric part) and the gradient 2 N 4K, N = I J pairs."""
    n = float(I) * J
    return 2.0 * n * 4 * K * (K + 1) / 2, 2.0 * n * 4 * K


# DRAM bytes (read + write) per (individual, block) pair of the tensor-core
# Hessian passes, from one-pass ncu captures (dram__bytes_read.sum +
# dram__bytes_write.sum) of one launch each at I=100,000, J=100,000, K=8:
# P 5.65 GB, Q 5.83 GB per launch over 1e10 pairs.
TRAFFIC_PER_PAIR = {"accum_q": 0.592, "accum_p": 0.588}

# Warp instructions per (individual, block) pair that the mixed method's pass
# kernels execute at K=8 (ncu smsp__inst_executed.sum over one launch at
# I=100,000, J=5,000, divided by the 5e8 pairs).  These passes are bound by
# instruction issue (the CUDA cores generate the tensor core's A operand), so
# their third roofline is the issue rate: one warp instruction per clock in
# each of an SM's 4 sub-partitions.
ISSUE_INST_PER_PAIR = {("accum_q", 8): 4.12, ("accum_p", 8): 5.22, ("loglik", 8): 1.96}
SMS = 152


def workload(name, cfg):
    return ("%s synthetic cohort I=%d x %d SNPs (J=%d blocks), K=%d, alpha=%g, %g%% missing, seed %d"
            % (name, cfg["I"], 2 * cfg["J"], cfg["J"], cfg["K"], cfg["alpha"], 100 * cfg["miss"], cfg["seed"]))


def load_config(args):
    from haplo_gb300 import synth
    return synth.config(args.config, I=args.I, J=args.J, K=args.K)


def cpu_info():
    """Host cores and CPU model, as nproc and lscpu report them."""
    info = {"nproc": os.cpu_count() or 1}
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            k, _, v = ln.partition(":")
            if k.strip() in ("Model name", "Architecture", "Socket(s)", "Core(s) per socket", "Thread(s) per core"):
                info[k.strip()] = v.strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return info


def cpu_components(cfg, slice_blocks, j0, threads, seed):
    """Seconds of the CPU oracle's pieces of the fit, timed on an I x
    slice_blocks slice of the cohort (blocks j0 .. j0+slice_blocks-1 of P) for
    the work that grows with J, and at full size for the rest:
      per slice: em (both gradient-only passes), ll, accum_q, accum_p (Hessian
        passes), qp_p (per-block QPs), proj_p (quartet projections);
      full size: qp_q (the I per-individual QPs), proj_q, qn (ZAL point on
        vectors of K (I + 4J))."""
    from oracle import oracle as O
    from haplo_gb300 import synth
    I, J, K = cfg["I"], cfg["J"], cfg["K"]
    Js = slice_blocks
    P = cfg["P"][:, 4 * j0:4 * (j0 + Js)]
    cq, cp = synth.cumulative(cfg["Q"], P)
    bed = O.synth(cfg["seed"] + j0, I, Js, cq, cp, cfg["miss"], threads=threads)
    b = O.Bed(bed, I, Js)
    rng = np.random.default_rng(seed)
    x = rng.random((K, I + 4 * Js))
    q = np.asfortranarray(x[:, :I] / x[:, :I].sum(axis=0, keepdims=True))
    p4 = x[:, I:].reshape(K, Js, 4)
    p = np.asfortranarray((p4 / p4.sum(axis=2, keepdims=True)).reshape(K, 4 * Js))
    t = {}

    def timed(name, f, *a, **kw):
        t0 = time.perf_counter()
        r = f(*a, **kw)
        t[name] = time.perf_counter() - t0
        return r

    timed("em", O.em_accum, b, K, q, p, threads=threads)
    timed("ll", O.loglik, b, K, q, p, threads=threads)
    XtXq, Xtzq = timed("accum_q", O.accum_q, b, K, q, p, threads=threads)
    XtXp, Xtzp = timed("accum_p", O.accum_p, b, K, q, p, threads=threads)
    timed("qp_p", O.qp_p, XtXp, Xtzp, p, threads=threads)
    timed("proj_p", O.project_p, p)
    timed("qp_q", O.qp_q, XtXq, Xtzq, q, threads=threads)
    timed("proj_q", O.project_q, q)
    n = K * (I + 4 * J)
    v = rng.random((3, n))
    U, V = np.zeros((n, 3)), np.zeros((n, 3))
    for it in (1, 2, 3):
        timed("qn", O.zal, v[0], v[1], v[2], U, V, it)
    return t


def cpu_fit_model(t, J, slice_blocks, em_iters, outer_iters):
    """Seconds of the reference's fit from per-piece times (cpu_components):
    the slice pieces scaled by J / slice_blocks, the rest as measured.
      EM iteration (src/algorithms_outer.jl:4-18): em + ll + projections;
      outer iteration (src/algorithms_outer.jl:65-171): 2 x (accum_q + qp_q +
      proj_q) + 2 x (accum_p + qp_p + proj_p) + 2 ll + qn + proj of the QN point."""
    s = J / float(slice_blocks)
    em = (t["em"] + t["ll"] + t["proj_p"]) * s + t["proj_q"]
    outer = (2 * (t["accum_q"] + t["accum_p"] + t["qp_p"] + t["proj_p"]) + 2 * t["ll"] + t["proj_p"]) * s \
        + 2 * (t["qp_q"] + t["proj_q"]) + t["qn"] + t["proj_q"]
    return em_iters * em + outer_iters * outer, em, outer


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def max_over_ranks(v, world, device=None):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def bench_config(args, cfg):
    """The workload description both arms print as "config"."""
    return {"workload": workload(args.config, cfg), "rtol": args.rtol, "em_iters": args.em_iters,
            "n_iter_cap": args.n_iter,
            "l2": "inputs (class words: I*J/2 bytes, 5 GB at I=1e5, J=1e5) larger than L2; no flush"}


def run_reference(args, world, rank):
    """CPU reference arm: the oracle port (C++ restatement of the reference's
    CPU loops, all host threads).  Each step times the fit's pieces on an
    I x slice_blocks slice of the blocks (a different slice each step) and at
    full size for the I-only work, then adds them up with the fit's iteration
    counts (cpu_fit_model)."""
    if rank != 0:
        return
    cfg = load_config(args)
    threads = os.cpu_count() or 1
    Js = min(args.cpu_slice_blocks or 500, cfg["J"])
    vals, sample_s = [], []
    for s in range(args.warmup + args.steps):
        j0 = (s * Js) % max(1, cfg["J"] - Js + 1)
        t0 = time.perf_counter()
        t = cpu_components(cfg, Js, j0, threads, seed=cfg["seed"] + s)
        sample_s.append(time.perf_counter() - t0)
        v, _, _ = cpu_fit_model(t, cfg["J"], Js, args.em_iters, args.ref_iters)
        if s >= args.warmup:
            vals.append(v)
    value = float(np.mean(vals))
    sample = ("oracle port, %d host threads: per step, the J-proportional pieces (EM and Hessian passes, "
              "log-likelihood, per-block QPs and projections) timed on an I=%d x %d-block slice (%.1f%% of "
              "the blocks; a different slice each step) and scaled by J/%d, the I-only pieces (per-individual "
              "QPs, projections) and the ZAL point timed at full size; summed with %d EM + %d outer iterations "
              "(the GB300 fit's count): extrapolated, %.1f s of CPU work per step"
              % (threads, cfg["I"], Js, 100.0 * Js / cfg["J"], Js, args.em_iters, args.ref_iters,
                 float(np.mean(sample_s[args.warmup:])) if args.steps else 0.0))
    line = {"metric": METRIC, "value": value, "unit": "s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(args, cfg),
            "cpu_baseline": {"value": value, "unit": "s", "cores": threads, "kind": "port", "sample": sample,
                             "host": cpu_info(), "extrapolated": True,
                             "measured_s_per_step": float(np.mean(sample_s[args.warmup:])) if args.steps else 0.0},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def issue_roofline(kind, I, J, K, per_launch_ms, sm_mhz):
    """Achieved warp-instruction issue rate of one launch against the SMs' peak."""
    ipp = ISSUE_INST_PER_PAIR.get((kind, K))
    if ipp is None or not sm_mhz:
        return None
    achieved = ipp * float(I) * J / (per_launch_ms * 1e-3)
    peak = SMS * 4 * sm_mhz * 1e6
    return {"achieved": achieved, "peak": peak, "unit": "warp instructions/s", "frac": achieved / peak,
            "warp_inst_per_pair": ipp, "sm_mhz": sm_mhz,
            "source": "instructions per pair from ncu smsp__inst_executed.sum at I=1e5, J=5e3, K=8 (the same "
                      "kernel); peak = 152 SMs x 4 issue slots per clock at the median SM clock of this run"}


def roofline_of(stats, ms_fit, steps, I, J, K, precision, sm_mhz=None):
    """Roofline of the dominant kernel from the launch accounting of the timed
    fits.  A tensor-core pass is two launches (operand image, pass), both
    timed; Hessian passes and gradient-only (EM) passes are counted apart."""
    peak_hbm, peak_bf16, peak_bf16_sus, peak_src = load_peaks()
    top = max(("accum_q", "accum_p", "loglik"), key=lambda k: stats[k][1])
    n_top, ms_top = stats[top]
    per = 2 if (precision == "mixed" and top in ("accum_q", "accum_p")) else 1
    launches = max(n_top / per, 1)
    per_launch_ms = ms_top / launches
    alg = pass_bytes(top, I, J, K)
    hbm_gbs = alg / (per_launch_ms * 1e-3) / 1e9
    share = ms_top / (ms_fit * steps)
    if top in ("accum_q", "accum_p"):
        fh, fg = pass_flops(I, J, K)
        achieved = fh / (per_launch_ms * 1e-3) / 1e12
        traffic = TRAFFIC_PER_PAIR[top] * I * J if precision == "mixed" else None
        issue = issue_roofline(top, I, J, K, per_launch_ms, sm_mhz) if precision == "mixed" else None
        return {"bound": "tensor", "kernel": top, "achieved": achieved, "peak": peak_bf16_sus,
                "unit": "TFLOP/s", "frac": achieved / peak_bf16_sus, "traffic": traffic,
                "traffic_source": "ncu one-pass capture (dram__bytes_read.sum + dram__bytes_write.sum) of one "
                                  "launch at I=1e5, J=1e5, K=8, per pair x I*J; not measured in this run",
                "peak_source": peak_src + " (bf16 sustained)", "flops_hessian_per_launch": fh,
                "flops_gradient_per_launch": fg, "ms_per_launch": per_launch_ms, "launches": int(launches),
                "secondary_hbm": {"achieved": hbm_gbs, "peak": peak_hbm, "unit": "GB/s",
                                  "frac": hbm_gbs / peak_hbm, "algorithmic_bytes_per_launch": alg},
                "issue": issue,
                "note": "the pass is bound by instruction issue (CUDA-core generation of the A operand), "
                        "not by the tensor pipe or HBM: 'issue' is the roofline that describes it",
                "share_of_timed": share}
    return {"bound": "hbm", "kernel": top, "achieved": hbm_gbs, "peak": peak_hbm, "unit": "GB/s",
            "frac": hbm_gbs / peak_hbm, "traffic": None, "peak_source": peak_src,
            "algorithmic_bytes_per_launch": alg, "ms_per_launch": per_launch_ms, "launches": int(launches),
            "issue": issue_roofline(top, I, J, K, per_launch_ms, sm_mhz) if precision == "mixed" else None,
            "share_of_timed": share}


def run_ours(args, world, rank, local):
    import torch
    import haplo_gb300 as hx
    from haplo_gb300 import synth
    from haplo_gb300.admix import random_init
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    cfg = load_config(args)
    I, J, K = cfg["I"], cfg["J"], cfg["K"]
    bps = (I + 3) // 4
    n_snp = 2 * J
    bed_dev = torch.empty(bps * n_snp, dtype=torch.uint8, device=dev)
    synth.synth_device(cfg["seed"], cfg["Q"], cfg["P"], cfg["miss"], bed_dev.data_ptr(), device=local)
    torch.cuda.synchronize()
    q0, p0 = random_init(I, J, K, np.random.default_rng(cfg["seed"] + 7))
    q0_dev = torch.from_numpy(np.ascontiguousarray(q0.T)).to(dev)   # memory = column-major K x I
    p0_dev = torch.from_numpy(np.ascontiguousarray(p0.T)).to(dev)
    d = hx.GB300Admix(bed_dev.data_ptr(), I, J, K, bytes_per_snp=bps, n_snp=n_snp, precision=args.precision,
                      device=local, bed_on_device=True)

    def step():
        d.set_qp_device(q0_dev.data_ptr(), p0_dev.data_ptr())
        return d.fit(n_iter=args.n_iter, rtol=args.rtol, em_iters=args.em_iters)

    # grid splits of the pass kernels, measured once for this shape (outside
    # the timed region, like the plan itself; later contexts of the shape reuse them)
    chunks = None
    if args.precision == "mixed" and not args.no_autotune:
        d.set_qp_device(q0_dev.data_ptr(), p0_dev.data_ptr())
        t0 = time.time()
        chunks = d.autotune()
        t_tune = time.time() - t0

    for _ in range(args.warmup):
        step()
    d.reset_stats()
    d.set_profiling(True)
    clocks = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    timed = [step() for _ in range(args.steps)]
    e1.record()
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    d.set_profiling(False)
    ms = e0.elapsed_time(e1) / args.steps
    ms = max_over_ranks(ms, world, dev)
    stats = d.kernel_stats()
    launches = int(sum(n for n, _ in stats.values()))
    iters = timed[-1]["iters"]
    ll = timed[-1]["ll"]
    q_c, p_c = d.get_qp()
    roofline = roofline_of(stats, ms, args.steps, I, J, K, args.precision, sm_mhz=clk.get("sm_mhz"))
    kernels = {k: {"launches": n, "ms": round(t, 3)} for k, (n, t) in stats.items()}
    # every pass kind against its own roofline (per launch, CUDA events of the timed fits)
    per = {}
    for kind in ("accum_q", "accum_p", "loglik", "em_q", "em_p"):
        n, t = stats[kind]
        if n == 0:
            continue
        lpp = 2 if (args.precision == "mixed" and kind in ("accum_q", "accum_p", "em_p")) else 1
        ms_l = t / (n / lpp)
        row = {"ms_per_launch": ms_l, "launches": int(n / lpp)}
        base = {"em_q": "accum_q", "em_p": "accum_p"}.get(kind, kind)
        b_alg = pass_bytes(base, I, J, K)
        row["hbm_frac"] = b_alg / (ms_l * 1e-3) / 1e9 / load_peaks()[0]
        if kind in ("accum_q", "accum_p"):
            row["tensor_frac"] = pass_flops(I, J, K)[0] / (ms_l * 1e-3) / 1e12 / load_peaks()[2]
        if args.precision == "mixed":
            iss = issue_roofline(kind, I, J, K, ms_l, clk.get("sm_mhz"))
            row["issue_frac"] = iss["frac"] if iss else None
        per[kind] = row
    roofline["per_kernel"] = per

    line = {"metric": METRIC, "value": ms / 1e3, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64" if args.precision == "mixed" else "f64",
            "data": "synthetic", "config": bench_config(args, cfg),
            "fit": {"method": args.precision, "outer_iters": iters, "loglik": ll,
                    "autotuned_chunks": ({"q_pass": chunks[0], "p_pass": chunks[1], "loglik": chunks[2],
                                          "tuning_s": round(t_tune, 3)} if chunks else None),
                    "parallelism": "replicas" if world > 1 else "1 GPU",
                    "init_em_loglik": "evaluated after the last of the EM iterations only; the reference "
                                      "evaluates it after each (src/algorithms_outer.jl:8-12) but only logs "
                                      "the others, so results are unchanged"},
            "gpu_launches": launches, "kernels": kernels, "roofline": roofline, "clocks": clk}

    # the plain FP64 method from the same start: to convergence (default), or
    # per-iteration timings only (--plain-estimate)
    if not args.no_plain and rank == 0:
        dp = hx.GB300Admix.shared(d, K, precision="fp64")
        dp.set_qp_device(q0_dev.data_ptr(), p0_dev.data_ptr())
        torch.cuda.synchronize()
        if args.plain_estimate:
            t0 = time.time()
            dp.init_em(1)
            t_em = time.time() - t0          # one EM step + its log-likelihood
            t0 = time.time()
            dp.loglikelihood()
            t_ll = time.time() - t0
            t0 = time.time()
            dp.qn_iteration()
            t_it = time.time() - t0
            est = args.em_iters * (t_em - t_ll) + t_ll + iters * t_it
            line["plain_fp64"] = {"s_per_em_iter": t_em, "s_per_loglik": t_ll, "s_per_outer_iter": t_it,
                                  "est_s_to_converge": est, "est_speedup_chosen_vs_plain": est / (ms / 1e3),
                                  "note": "extrapolated: measured EM and outer-iteration times x the chosen "
                                          "fit's iteration counts"}
        else:
            e0.record()
            pinfo = dp.fit(n_iter=args.n_iter, rtol=args.rtol, em_iters=args.em_iters)
            e1.record()
            torch.cuda.synchronize()
            t_full = e0.elapsed_time(e1) / 1e3
            q_f, p_f = dp.get_qp()
            rel_ll = abs(ll - pinfo["ll"]) / abs(pinfo["ll"])
            dq = float(np.abs(q_c - q_f).max())
            line["plain_fp64"] = {
                "measured_s_to_converge": t_full, "outer_iters": pinfo["iters"], "loglik": pinfo["ll"],
                "measured_speedup_chosen_vs_plain": t_full / (ms / 1e3),
                "chosen_vs_plain": {"ll_rel_diff": rel_ll, "q_max_abs_diff": dq,
                                    "p_max_abs_diff": float(np.abs(p_c - p_f).max()),
                                    "meets_1e-8_ll_and_1e-5_q": bool(rel_ll <= 1e-8 and dq <= 1e-5)},
                "note": "plain FP64 GPU method fitted to convergence once in this run from the same start "
                        "(CUDA events); not part of the timed steps"}
        dp.close()

    # end to end through the public API from host buffers
    if not args.no_e2e:
        host_bed = torch.empty(bps * n_snp, dtype=torch.uint8, pin_memory=True)
        host_bed.copy_(bed_dev)
        hb = host_bed.numpy().reshape(n_snp, bps)
        torch.cuda.synchronize()
        barrier(world)
        t0 = time.time()
        de = hx.GB300Admix(hb, I, J, K, bytes_per_snp=bps, n_snp=n_snp, precision=args.precision, device=local)
        de.set_qp(q0, p0)
        info = de.fit(n_iter=args.n_iter, rtol=args.rtol, em_iters=args.em_iters)
        q_out, p_out = de.get_qp()
        ll_e = de.ll_new
        de.close()
        t_e2e = max_over_ranks(time.time() - t0, world, dev)
        line["e2e"] = {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": int(bps * n_snp + 8 * K * (I + 4 * J)),
                       "d2h_bytes_per_step": int(8 * K * (I + 4 * J) + 8), "outer_iters": info["iters"],
                       "loglik": ll_e}

    if not args.no_cpu and rank == 0:
        threads = os.cpu_count() or 1
        Js = min(args.cpu_slice_blocks or 2000, J)
        t0 = time.perf_counter()
        t = cpu_components(cfg, Js, 0, threads, seed=cfg["seed"])
        spent = time.perf_counter() - t0
        v, em, outer = cpu_fit_model(t, J, Js, args.em_iters, iters)
        line["cpu_baseline"] = {
            "value": v, "unit": "s", "cores": threads, "kind": "port", "host": cpu_info(), "extrapolated": True,
            "s_per_em_iter": em, "s_per_outer_iter": outer, "measured_s": spent,
            "pieces_s": {k: round(x, 4) for k, x in t.items()},
            "sample": "oracle port, %d host threads: J-proportional pieces timed on an I=%d x %d-block slice and "
                      "scaled by J/%d; I-only pieces (per-individual QPs, projections) and the ZAL point at full "
                      "size; summed with this fit's %d EM + %d outer iterations (extrapolated)"
                      % (threads, I, Js, Js, args.em_iters, iters)}
    if args.skfr and rank == 0:
        from haplo_gb300 import skfr
        hb = bed_dev.cpu().numpy().reshape(n_snp, bps)
        t0 = time.perf_counter()
        cl, aims, sit = skfr.select_aims(hb, I, K, args.skfr, seed=0, device=local)
        t_gpu = time.perf_counter() - t0
        row = {"sparsity_blocks": args.skfr, "K": K, "iterations": sit, "gpu_s": t_gpu,
               "note": "wall time of hx_skfr from host bytes (upload, k-means++ start, iterations)"}
        if not args.no_cpu:
            from oracle import skfr_oracle
            t0 = time.perf_counter()
            oc, oa, oit = skfr_oracle.select(hb, I, K, args.skfr, seed=0)
            row.update({"cpu_s": time.perf_counter() - t0, "cpu_kind": "port (numpy oracle, one host thread "
                        "for the per-SNP loops)", "identical_to_oracle": bool(np.array_equal(oa, aims) and
                                                                             np.array_equal(oc, cl) and oit == sit)})
        line["skfr"] = row
    if args.cpu_full_fit and rank == 0:
        from oracle import oracle as O
        threads = os.cpu_count() or 1
        hb = bed_dev.cpu().numpy().reshape(n_snp, bps)
        b = O.Bed(hb, I, J)
        t0 = time.perf_counter()
        oq, op, oll, oit, _ = O.fit(b, K, q0, p0, n_iter=args.n_iter, rtol=args.rtol, em_iters=args.em_iters,
                                    threads=threads)
        t_cpu = time.perf_counter() - t0
        line["cpu_full_fit"] = {
            "value": t_cpu, "unit": "s", "cores": threads, "kind": "port", "host": cpu_info(), "extrapolated": False,
            "outer_iters": oit, "loglik": oll, "speedup_chosen_vs_cpu": t_cpu / (ms / 1e3),
            "chosen_vs_cpu": {"ll_rel_diff": abs(ll - oll) / abs(oll), "q_max_abs_diff": float(np.abs(q_c - oq).max())},
            "sample": "oracle port: the whole fit (init_em! + admixture_qn! to rtol) from the GPU fits' start"}
    d.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
