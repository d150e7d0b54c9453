"""Host logic of bench.py (no GPU): the algorithmic-bytes model, the CFL dt,
the FP64 peak and the replica rate."""
from math import pi

import numpy as np
import pytest


def test_fields_per_launch_at_512():
    import bench
    fpl = bench.fields_per_launch(512, 512, 512)
    assert set(fpl) == set(bench.KINDS)
    fx, fy = 171 / 257, 341 / 512
    # the x pass reads the six kept-x rows and writes three
    assert fpl["x_product"] == pytest.approx(9 * fx)
    assert fpl["inv_y"] == pytest.approx(6 * fx * fy + 6 * fx)
    # one spectral field at 512^3 FP32: 512 * 512 * 257 complex64
    field = 512 * 512 * 257 * 8
    step = 4 * sum(fpl.values()) * field
    assert step == pytest.approx(51.13e9, rel=2e-3)  # bytes per RK4 step
    assert fpl["x_product"] * field == pytest.approx(3.2275e9, rel=1e-3)


def test_cfl_dt_rule():
    import bench
    n = 64
    dx = 2 * pi / n
    # dt = cfl / sum(max|v_i| / dx), capped by dtmax
    assert bench.cfl_dt([1.0, 2.0, 0.5], n) == pytest.approx(0.5 / (3.5 / dx))
    assert bench.cfl_dt([0.0, 0.0, 0.0], n) == 0.2
    assert bench.cfl_dt([1e-9, 0, 0], n, dtmax=0.1) == 0.1


def test_fp64_peak_and_flops():
    import bench
    # 152 SMs x 2 FP64 FMA per clock x 2 flops x 2070 MHz
    assert bench.fp64_peak_tflops(2070.0) == pytest.approx(152 * 2 * 2 * 2.07e9 / 1e12)
    f = bench.fp64_flops_per_step(512, 512, 512)
    assert 1e11 < f < 1e12
    # more points, more flops
    assert bench.fp64_flops_per_step(256, 256, 256) < f


def test_replica_rate_single_process():
    import bench
    rate, ms = bench.replica_rate(1000.0, 20, 1)
    assert rate == pytest.approx(20.0) and ms == 1000.0
    rate, _ = bench.replica_rate(500.0, 10, 4)
    assert rate == pytest.approx(80.0)


def test_workload_config_names_the_workload():
    import bench
    cfg = bench.workload_config(512, 512, 512, 1e-3, 1)
    assert "512^3" in cfg["workload"] and cfg["nx"] == 512
    assert cfg["parallelism"] == "replicas x1"
