"""The 512-point kernels of the ns3d 512^3 benchmark step against the oracle.

The benchmark runs the compile-time-size kernels instantiated for 512-point
lines: the curl + inverse z pass and the forward z pass on 512-point z
columns, both y passes on 512-point y columns, and the x pass on 512-point
rows.  These cases run each of them against the float64 CPU oracle, first on
small boxes where one axis or two are 512 long, then on the full 512^3
benchmark workload itself (seeded isotropic field, nu_2 = 5e-4, dt from the
CFL rule): the first tendency and two RK4 steps, FP64 within 1e-12 and FP32
within 1e-5 relative L2 per state variable.
"""
from math import pi

import numpy as np
import pytest

from test_fast_path_gpu import rel, run_3d

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [(512, 512, 32), (32, 32, 512)])
def test_512_point_lines_fp64(cuda, shape):
    sim, orc = run_3d(shape, "float64", 3, USE_CFL=True, cfl_coef=0.5, L=(2 * pi,) * 3)
    assert rel(sim.state.state_spect.cpu().numpy(), orc.state_spect) < 1e-12
    assert abs(sim.time_stepping.deltat - orc.deltat) <= 1e-12 * orc.deltat


@pytest.mark.parametrize("shape", [(512, 512, 32)])
def test_512_point_columns_fp32(cuda, shape):
    sim, orc = run_3d(shape, "float32", 3, USE_CFL=True, cfl_coef=0.5, L=(2 * pi,) * 3)
    got = sim.state.state_spect.cpu().numpy().astype(np.complex128)
    assert rel(got, orc.state_spect) < 1e-5


@pytest.fixture(scope="module")
def workload_512():
    """The benchmark's 512^3 initial field, its dt, and the oracle's first
    tendency and state after two RK4 steps."""
    import bench
    n = 512
    v0 = bench.initial_state(n)
    dt = bench.initial_dt(v0, n)
    orc = bench.oracle_sim(n, v0, dt)
    tend0 = orc.tendencies_nonlin()
    orc.one_time_step()
    orc.one_time_step()
    return {"v0": v0, "dt": dt, "tend0": tend0, "state2": orc.state_spect.copy()}


@pytest.mark.parametrize("precision,tol", [("float64", 1e-12), ("float32", 1e-5)])
def test_benchmark_workload_512_cubed(cuda, workload_512, precision, tol):
    import torch
    import bench
    w = workload_512
    sim = bench.make_sim(512, precision, w["v0"])
    sim.time_stepping.deltat = w["dt"]
    tend = sim.tendencies_nonlin().cpu().numpy().astype(np.complex128)
    assert rel(tend, w["tend0"]) < tol
    sim.time_stepping.one_time_step()
    sim.time_stepping.one_time_step()
    got = sim.state.state_spect.cpu().numpy().astype(np.complex128)
    assert rel(got, w["state2"]) < tol
    del sim
    torch.cuda.empty_cache()
