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
  cpu_baseline : CPU oracle (C++ restatement, all host cores) on a bounded
          slice, extrapolated to the full fit (labelled)

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
# outer iterations of the C3 fit measured on GB300 (26 at rtol 1e-8); used
# only to extrapolate the CPU reference arm, whose full fit takes hours
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
    ap.add_argument("--plain-full", action="store_true",
                    help="run the plain FP64 fit to convergence (minutes) and compare it with the chosen fit")
    ap.add_argument("--no-cpu", action="store_true")
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
# Hessian passes, from one-pass ncu captures of one launch each at I=100,000,
# J=100,000, K=8 (profiles/k_accum_tc_c3_dram.md): P 5.65 GB, Q 5.83 GB per
# launch over 1e10 pairs.
TRAFFIC_PER_PAIR = {"accum_q": 0.592, "accum_p": 0.588}


def workload(name, cfg):
    return ("%s synthetic cohort I=%d x %d SNPs (J=%d blocks), K=%d, alpha=%g, %g%% missing, seed %d"
            % (name, cfg["I"], 2 * cfg["J"], cfg["J"], cfg["K"], cfg["alpha"], 100 * cfg["miss"], cfg["seed"]))


def load_config(args):
    from haplo_gb300 import synth
    return synth.config(args.config, I=args.I, J=args.J, K=args.K)


def cpu_oracle_sample(cfg, slice_blocks, threads):
    """Times the CPU oracle on an I x slice_blocks slice: one EM step and one
    outer QN iteration (4 accumulations + QPs + 2 log-likelihoods + ZAL)."""
    from oracle import oracle as O
    from haplo_gb300 import synth
    from haplo_gb300.admix import random_init
    I, K = cfg["I"], cfg["K"]
    Js = slice_blocks
    Q = cfg["Q"]
    P = cfg["P"][:, :4 * Js]
    cq, cp = synth.cumulative(Q, P)
    bed = O.synth(cfg["seed"], I, Js, cq, cp, cfg["miss"], threads=threads)
    b = O.Bed(bed, I, Js)
    q0, p0 = random_init(I, Js, K, np.random.default_rng(7))
    t0 = time.time()
    q1, p1 = O.em_step(b, K, q0, p0, threads=threads)
    O.loglik(b, K, q1, p1, threads=threads)
    t_em = time.time() - t0
    t0 = time.time()
    O.fit(b, K, q1, p1, n_iter=1, rtol=0.0, em_iters=0, threads=threads)
    t_it = time.time() - t0
    return t_em, t_it


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


def run_reference(args, world, rank):
    """CPU reference arm: the oracle port (C++ restatement of the reference's
    CPU loops, all host threads) on bounded slices of the workload."""
    if rank != 0:
        return
    cfg = load_config(args)
    threads = os.cpu_count() or 1
    Js = args.cpu_slice_blocks or 200
    vals = []
    for s in range(args.warmup + args.steps):
        t_em, t_it = cpu_oracle_sample(cfg, Js, threads)
        scale = cfg["J"] / Js
        v = (args.em_iters * t_em + args.ref_iters * t_it) * scale
        if s >= args.warmup:
            vals.append(v)
    value = float(np.mean(vals))
    sample = ("oracle port on I=%d x %d-block slices (%.2f%% of the blocks): %d EM steps + %d outer "
              "iterations, per-block time scaled by J/%d; iteration count %d from the GB300 fit (extrapolated)"
              % (cfg["I"], Js, 100.0 * Js / cfg["J"], args.em_iters, args.ref_iters, Js, args.ref_iters))
    line = {"metric": METRIC, "value": value, "unit": "s", "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload(args.config, cfg), "rtol": args.rtol, "em_iters": args.em_iters},
            "cpu_baseline": {"value": value, "unit": "s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


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

    infos = []
    for _ in range(args.warmup):
        infos.append(step())
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

    # roofline of the dominant pass kernel.  The accumulation passes are
    # contractions on the tensor cores: their roofline is the tensor pipe
    # (achieved = Hessian FLOPs / time against the measured sustained bf16
    # peak, the kernel running inside a long fit), with the HBM floor as the
    # secondary bound.  The log-likelihood pass streams the class words (HBM).
    peak_hbm, peak_bf16, peak_bf16_sus, peak_src = load_peaks()
    top = max(("accum_q", "accum_p", "loglik"), key=lambda k: stats[k][1])
    n_top, ms_top = stats[top]
    # passes of the top kind: in the mixed method a tensor-core pass is two
    # launches (operand image, pass); the gradient-only EM Q passes run on the
    # CUDA cores (one launch each)
    passes = n_top
    if args.precision == "mixed" and top == "accum_p":
        passes = n_top / 2
    elif args.precision == "mixed" and top == "accum_q":
        em = args.em_iters * args.steps
        passes = (n_top - em) / 2 + em
    per_launch_ms = ms_top / max(passes, 1)
    alg = pass_bytes(top, I, J, K)
    hbm_gbs = alg / (per_launch_ms * 1e-3) / 1e9
    if top in ("accum_q", "accum_p"):
        fh, fg = pass_flops(I, J, K)
        achieved = fh / (per_launch_ms * 1e-3) / 1e12
        traffic = TRAFFIC_PER_PAIR[top] * I * J if args.precision == "mixed" else None
        roofline = {"bound": "tensor", "kernel": top, "achieved": achieved, "peak": peak_bf16_sus,
                    "unit": "TFLOP/s", "frac": achieved / peak_bf16_sus, "traffic": traffic,
                    "peak_source": peak_src + " (bf16 sustained)", "flops_hessian_per_launch": fh,
                    "flops_gradient_per_launch": fg, "ms_per_launch": per_launch_ms,
                    "secondary_hbm": {"achieved": hbm_gbs, "peak": peak_hbm, "unit": "GB/s",
                                      "frac": hbm_gbs / peak_hbm, "algorithmic_bytes_per_launch": alg},
                    "share_of_timed": ms_top / (ms * args.steps)}
    else:
        roofline = {"bound": "hbm", "kernel": top, "achieved": hbm_gbs, "peak": peak_hbm, "unit": "GB/s",
                    "frac": hbm_gbs / peak_hbm, "traffic": None, "peak_source": peak_src,
                    "algorithmic_bytes_per_launch": alg, "ms_per_launch": per_launch_ms,
                    "share_of_timed": ms_top / (ms * args.steps)}
    kernels = {k: {"launches": n, "ms": round(t, 3)} for k, (n, t) in stats.items()}

    line = {"metric": METRIC, "value": ms / 1e3, "unit": "s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64" if args.precision == "mixed" else "f64",
            "data": "synthetic",
            "config": {"workload": workload(args.config, cfg),
                       "method": args.precision, "rtol": args.rtol, "em_iters": args.em_iters,
                       "outer_iters": iters, "loglik": ll, "parallelism": "replicas" if world > 1 else "1 GPU",
                       "l2": "inputs (5 GB class words) larger than L2; no flush"},
            "gpu_launches": launches, "kernels": kernels, "roofline": roofline, "clocks": clk}

    # plain FP64 method, per-iteration sample (its full fit takes minutes)
    if not args.no_plain and rank == 0:
        dp = hx.GB300Admix(bed_dev.data_ptr(), I, J, K, bytes_per_snp=bps, n_snp=n_snp, precision="fp64",
                           device=local, bed_on_device=True)
        dp.set_qp_device(q0_dev.data_ptr(), p0_dev.data_ptr())
        t0 = time.time()
        dp.init_em(1)
        t_em = time.time() - t0          # one EM step + its log-likelihood
        t0 = time.time()
        dp.loglikelihood()
        t_ll = time.time() - t0
        t0 = time.time()
        dp.qn_iteration()
        t_it = time.time() - t0
        # init_em evaluates the log-likelihood after its last step only
        est = args.em_iters * (t_em - t_ll) + t_ll + iters * t_it
        line["plain_fp64"] = {"s_per_em_iter": t_em, "s_per_loglik": t_ll, "s_per_outer_iter": t_it,
                              "est_s_to_converge": est, "est_speedup_chosen_vs_plain": est / (ms / 1e3),
                              "note": "extrapolated: measured EM and outer-iteration times x the chosen "
                                      "fit's iteration counts"}
        if args.plain_full:
            # the plain fit to convergence from the same start, against the
            # chosen fit's result (ll relative, Q and P largest absolute)
            q_c, p_c = d.get_qp()
            dp.set_qp_device(q0_dev.data_ptr(), p0_dev.data_ptr())
            torch.cuda.synchronize()
            t0 = time.time()
            pinfo = dp.fit(n_iter=args.n_iter, rtol=args.rtol, em_iters=args.em_iters)
            t_full = time.time() - t0
            q_f, p_f = dp.get_qp()
            line["plain_fp64"].update({
                "measured_s_to_converge": t_full, "measured_outer_iters": pinfo["iters"], "ll": pinfo["ll"],
                "measured_speedup_chosen_vs_plain": t_full / (ms / 1e3),
                "chosen_vs_plain": {"ll_rel_diff": abs(ll - pinfo["ll"]) / abs(pinfo["ll"]),
                                    "q_max_abs_diff": float(np.abs(q_c - q_f).max()),
                                    "p_max_abs_diff": float(np.abs(p_c - p_f).max())}})
        dp.close()

    # end to end through the public API from host buffers
    if not args.no_e2e:
        host_bed = torch.empty(bps * n_snp, dtype=torch.uint8, pin_memory=True)
        host_bed.copy_(bed_dev)
        hb = host_bed.numpy().reshape(n_snp, bps)
        q_out = np.empty((K, I), order="F")
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
        Js = args.cpu_slice_blocks or 200
        t_em, t_it = cpu_oracle_sample(cfg, Js, threads)
        v = (args.em_iters * t_em + iters * t_it) * J / Js
        line["cpu_baseline"] = {"value": v, "unit": "s", "cores": threads, "kind": "port",
                                "sample": "oracle port, I=%d x %d blocks: 1 EM step + 1 outer iteration, "
                                          "scaled by J/%d and by this fit's %d EM + %d outer iterations "
                                          "(extrapolated)" % (I, Js, Js, args.em_iters, iters)}
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
