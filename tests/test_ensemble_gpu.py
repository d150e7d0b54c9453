"""Batched ns2d ensembles against individually solved runs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_ensemble_matches_individual_runs(cuda):
    from fluidsim_gb300.ensemble import EnsembleNS2D, make_group, reference_run
    groups = [make_group(128, 3, seed=1), make_group(256, 2, seed=2)]
    ens = EnsembleNS2D(groups)
    ens.autotune(steps=1, candidates=[(8, 2, 8), (16, 4, 4)])
    ens.run(20)
    assert not ens.nan_flag()
    for gi, g in enumerate(groups):
        got = ens.groups[gi]["S"].cpu().numpy()
        for i in range(len(g["nu2"])):
            ref = reference_run(g, i, 20)
            assert np.linalg.norm(got[i] - ref) / np.linalg.norm(ref) < 2e-5
            ref32 = reference_run(g, i, 20, precision="float32")
            # same kernels, same order of operations as a single float32 run
            assert np.linalg.norm(got[i] - ref32) / np.linalg.norm(ref32) < 1e-6


def test_graph_replay_equals_direct_launch(cuda):
    from fluidsim_gb300.ensemble import EnsembleNS2D, make_group
    groups = [make_group(128, 2, seed=5), make_group(256, 2, seed=6)]
    ens = EnsembleNS2D(groups)
    ens.run(6)
    direct = [g["S"].clone() for g in ens.groups]
    ens.reset()
    ens.capture(3)
    ens.reset()
    ens.run(6)
    for g, d in zip(ens.groups, direct):
        assert np.array_equal(g["S"].cpu().numpy(), d.cpu().numpy())


def test_single_launch_mode_equals_per_group_streams(cuda):
    """One launch per pass for all sizes gives the per-group results to
    rounding (same operations per line; the compiler may contract a few
    products differently inside the multi-size kernel: ~1e-8 relative after
    5 steps), and its graph replay equals its direct launch bit for bit."""
    from fluidsim_gb300.ensemble import EnsembleNS2D, make_group
    groups = [make_group(128, 3, seed=7), make_group(512, 2, seed=8), make_group(256, 2, seed=9)]
    ens = EnsembleNS2D(groups)
    ens.mixed = False
    ens.step(5)
    per_group = [g["S"].cpu().numpy() for g in ens.groups]
    ens.reset()
    ens.mixed = True
    ens.step(5)
    mixed = [g["S"].cpu().numpy() for g in ens.groups]
    for a, b in zip(mixed, per_group):
        for i in range(len(b)):
            assert np.linalg.norm(a[i] - b[i]) / np.linalg.norm(b[i]) < 1e-6
    ens.reset()
    ens.capture(5)
    ens.reset()
    ens.run(5)
    for g, d in zip(ens.groups, mixed):
        assert np.array_equal(g["S"].cpu().numpy(), d)
    assert not ens.nan_flag()


def test_persistent_mode_equals_per_group_streams(cuda):
    """All steps in one persistent launch (device work queue, per-run
    dependency counters) give the per-group results to rounding, for both
    thread counts, and its graph replay equals its direct launch."""
    from fluidsim_gb300.ensemble import EnsembleNS2D, make_group
    groups = [make_group(128, 3, seed=7), make_group(512, 2, seed=8), make_group(256, 2, seed=9)]
    ens = EnsembleNS2D(groups)
    ens.step(1)  # from here on the states are dealiased
    start = [g["S"].clone() for g in ens.groups]
    ens.step(5)
    per_group = [g["S"].cpu().numpy() for g in ens.groups]
    for th in (256, 512):
        for g, s in zip(ens.groups, start):
            g["S"].copy_(s)
        ens.persistent, ens.persist_threads = True, th
        ens.step(5)
        ens.check_status()
        got = [g["S"].cpu().numpy() for g in ens.groups]
        for a, b in zip(got, per_group):
            for i in range(len(b)):
                assert np.linalg.norm(a[i] - b[i]) / np.linalg.norm(b[i]) < 1e-6, th
    for g, s in zip(ens.groups, start):
        g["S"].copy_(s)
    ens.capture(5)
    for g, s in zip(ens.groups, start):
        g["S"].copy_(s)
    ens.run(5)
    for g, d in zip(ens.groups, got):
        assert np.array_equal(g["S"].cpu().numpy(), d)
    assert not ens.nan_flag()


def test_persistent_wait_that_runs_out_returns_error_status(cuda):
    """A dependency wait that can never be satisfied (test hook: one wait
    needs an item that does not exist) gives up after its time limit: the
    launch ends, the status reads GBS_ETIMEDOUT, and the context stays usable
    (the next persistent call runs normally)."""
    import ctypes
    import torch
    from fluidsim_gb300 import _lib
    from fluidsim_gb300.ensemble import EnsembleNS2D, make_group
    groups = [make_group(128, 2, seed=3), make_group(256, 1, seed=4)]
    ens = EnsembleNS2D(groups)
    ens.step(1)
    start = [g["S"].clone() for g in ens.groups]
    ens.persistent, ens.persist_timeout_s = True, 1e-3
    ens.step(2, flags=_lib.GBS_STEP_DEALIASED | _lib.GBS_STEP_TEST_STALL)
    torch.cuda.synchronize()
    st = ctypes.c_int()
    rc = ens.lib.gbs_ens2d_persistent_status(ens._mix, ctypes.byref(st))
    assert rc == _lib.GBS_ETIMEDOUT and st.value == 1
    # status cleared; a normal call works and matches the per-group path
    for g, s in zip(ens.groups, start):
        g["S"].copy_(s)
    ens.persist_timeout_s = 1.0
    ens.step(2)
    ens.check_status()
    got = [g["S"].cpu().numpy() for g in ens.groups]
    for g, s in zip(ens.groups, start):
        g["S"].copy_(s)
    ens.persistent = False
    ens.step(2)
    for g, a in zip(ens.groups, got):
        b = g["S"].cpu().numpy()
        for i in range(len(b)):
            assert np.linalg.norm(a[i] - b[i]) / np.linalg.norm(b[i]) < 1e-6


def test_ensemble_runs_match_the_oracle(cuda):
    """Runs of a batched group against the float64 oracle solving each run
    alone (IF-RK4, per-run nu_2, nu_8, dt): float32 within 1e-5 after 20
    steps."""
    from math import pi
    from fluidsim_gb300.ensemble import EnsembleNS2D, make_group
    from oracle.solvers import NS2DOracle
    from oracle.spectral import OperNumpy2D
    groups = [make_group(128, 2, seed=11), make_group(256, 2, seed=12)]
    ens = EnsembleNS2D(groups)
    ens.step(20, flags=0)
    for gi, g in enumerate(groups):
        got = ens.groups[gi]["S"].cpu().numpy()
        n, L = g["n"], g["L"]
        for i in range(len(g["nu2"])):
            orc = NS2DOracle(OperNumpy2D(n, n, L, L), nu_2=float(g["nu2"][i]),
                             nu_8=float(g["nu8"][i]), deltat0=float(g["dt"][i]))
            orc.init_from_rotfft(g["rot0"][i])
            orc.run(it_end=20)
            ref = orc.state_spect[0]
            assert np.linalg.norm(got[i] - ref) / np.linalg.norm(ref) < 1e-5
