"""Host-side arithmetic of bench.py (no GPU): the algorithmic byte models of
the roofline lines and the two-size extrapolation of the CPU baselines."""

import math
from types import SimpleNamespace

import pytest

import bench


def test_level0_byte_models():
    dm = SimpleNamespace(d=3, n_blocks=1000, n_dofs=300)
    # FP32 pass: 9 values of 4 bytes and a 4-byte column per block, x and y once
    assert bench.spmv_bytes(dm, 4) == 1000 * 40 + 2 * 4 * 300
    # FP16 smoothing copy: 9 values of 2 bytes
    assert bench.spmv_bytes(dm, 2) == 1000 * 22 + 2 * 4 * 300
    # four smoothing passes on the FP16 copy and one FP32 product per iteration
    mean = bench.level0_launch_bytes(dm, "fp16")
    assert mean == pytest.approx((4 * bench.spmv_bytes(dm, 2) + bench.spmv_bytes(dm, 4)) / 5)
    assert bench.level0_launch_bytes(dm, "fp32") == bench.spmv_bytes(dm, 4)


def test_cpu_baseline_extrapolates_by_measured_iteration_growth(monkeypatch):
    """Set-up scales with DOF and CG with DOF x iterations, the iteration
    count grown as n^alpha with alpha fitted between the two samples."""
    samples = {16: (2.0, 1.0, 3 * 17**3, 500), 24: (6.0, 4.0, 3 * 25**3, 750)}
    monkeypatch.setattr(bench, "_port_step", lambda n: samples[n])
    out = bench.cpu_baseline(24, 70)
    alpha = math.log(750 / 500) / math.log(24 / 16)
    dofs_t = 3 * 71**3
    it_t = 750 * (70 / 24) ** alpha
    t_t = (6.0 - 4.0) * dofs_t / (3 * 25**3) + 4.0 * dofs_t / (3 * 25**3) * it_t / 750
    assert out["value"] == pytest.approx(t_t / (dofs_t / 1e6))
    assert out["samples"]["iteration_exponent"] == pytest.approx(alpha)
    assert out["kind"] == "port" and out["unit"] == bench.UNIT


def test_heat_and_assembly_baselines_use_the_same_rule(monkeypatch):
    monkeypatch.setattr(bench, "_heat_port_step", lambda n: {20: (1.0, 0.5, 21**3, 200),
                                                              30: (3.0, 2.0, 31**3, 300)}[n])
    h = bench.heat_cpu_baseline(30, 100)
    alpha = math.log(300 / 200) / math.log(30 / 20)
    dofs_t = 101**3
    it_t = 300 * (100 / 30) ** alpha
    assert h["value"] == pytest.approx(((3.0 - 2.0) * dofs_t / 31**3 + 2.0 * dofs_t / 31**3 * it_t / 300)
                                       / (dofs_t / 1e6))
    monkeypatch.setattr(bench, "_assembly_port_step", lambda n: {8: (1.0, 0.4, 4380, 400),
                                                                  12: (3.0, 1.6, 13188, 600)}[n])
    a = bench.assembly_cpu_baseline(12, 40)
    assert a["value"] > 0 and a["samples"]["n"] == [8, 12]


def test_reference_arm_line(monkeypatch, capsys):
    """`--impl reference` prints one line whose value and step time are the
    mean of the timed runs' extrapolations (warm-up runs dropped)."""
    import json

    samples = {16: (2.0, 1.0, 3 * 17**3, 500), 24: (6.0, 4.0, 3 * 25**3, 750)}
    monkeypatch.setattr(bench, "_port_step", lambda n: samples[n])
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    args = SimpleNamespace(gpus=1, steps=2, warmup=3, cpu_n=24, n=70)
    bench.run_reference(args)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    ref = bench.cpu_baseline(24, 70)
    assert line["impl"] == "reference" and line["higher_is_better"] is False
    assert line["value"] == pytest.approx(ref["value"])
    assert line["ms_per_step"] == pytest.approx(1e3 * ref["samples"]["predicted_seconds"])
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port"
