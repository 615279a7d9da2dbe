"""bench.py's CPU reference arm: the piecewise model of the CPU fit (slice
pieces scaled by J / slice, I-only pieces at full size) and the JSON line
of `--impl reference` on a tiny case.  CPU only."""
import json

import pytest


def test_cpu_fit_model_scales_only_block_pieces():
    import bench
    t = {"em": 1.0, "ll": 0.5, "accum_q": 2.0, "accum_p": 3.0, "qp_p": 0.25, "proj_p": 0.125,
         "qp_q": 7.0, "proj_q": 0.0625, "qn": 0.03125}
    total, em, outer = bench.cpu_fit_model(t, J=1000, slice_blocks=100, em_iters=5, outer_iters=10)
    s = 10.0
    assert em == pytest.approx((1.0 + 0.5 + 0.125) * s + 0.0625)
    assert outer == pytest.approx((2 * (2.0 + 3.0 + 0.25 + 0.125) + 2 * 0.5 + 0.125) * s
                                  + 2 * (7.0 + 0.0625) + 0.03125 + 0.0625)
    assert total == pytest.approx(5 * em + 10 * outer)
    # the per-individual QPs are not multiplied by J / slice
    t2 = dict(t, qp_q=8.0)
    _, _, outer2 = bench.cpu_fit_model(t2, J=1000, slice_blocks=100, em_iters=5, outer_iters=10)
    assert outer2 - outer == pytest.approx(2.0)


def test_reference_arm_line(capsys):
    import bench
    args = bench.parse(["--impl", "reference", "--config", "C1", "--I", "64", "--J", "40", "--K", "2",
                        "--cpu-slice-blocks", "10", "--steps", "2", "--warmup", "1"])
    bench.run_reference(args, 1, 0)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "s" and line["higher_is_better"] is False
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["extrapolated"] and cb["cores"] >= 1 and "nproc" in cb["host"]
    # the same "config" as the GPU arm prints
    cfg = bench.load_config(args)
    assert line["config"] == bench.bench_config(args, cfg)
