"""The oracle restatement reproduces the fixtures made by the reference code.

Fixtures (``tests/golden/*.npz``) come from the reference's own time-scheme
(RK4, RK2, RK2_trapezoid, Euler, the phase-shift schemes including the random
ones) / CFL / tendency code (``oracle/refshim.py``, see
``golden/make_golden.py``).
"""
import random

import numpy as np
import pytest

from golden_cases import (CASES_2D, CASES_3D, KEY_NAMES, forcing_config, lengths, load,
                          projection_kwargs, solver_kwargs)
from oracle.forcing import CoarseForcingOracle
from oracle.spectral import OperNumpy2D, OperNumpy3D
from oracle.solvers import NS2DOracle, NS2DStratOracle, NS3DOracle, NS3DStratOracle
from oracle.turb import smagorinsky_forcing


def make_oracle(name):
    d, p = load(name)
    if p.get("phase_seed") is not None:  # the random phase schemes draw with `random`
        random.seed(int(p["phase_seed"]))
    if name.startswith("ns2d"):
        oper = OperNumpy2D(int(p["nx"]), int(p["ny"]), *lengths(p, 2))
        if p.get("N") is not None or p.get("bouss"):
            orc = NS2DStratOracle(oper, N=p.get("N") or 0.0, **solver_kwargs(p))
        else:
            orc = NS2DOracle(oper, beta=p.get("beta") or 0.0, **solver_kwargs(p))
    else:
        oper = OperNumpy3D(int(p["nx"]), int(p["ny"]), int(p["nz"]), *lengths(p, 3))
        turb = None
        if p.get("smagorinsky_C") is not None:
            C = p["smagorinsky_C"]

            def turb(o, vx, vy, vz):
                return smagorinsky_forcing(o, vx, vy, vz, C=C)
        if p.get("N") is not None:
            orc = NS3DStratOracle(oper, N=p["N"], f=p.get("f"), bouss=bool(p.get("bouss")),
                                  **projection_kwargs(p), **solver_kwargs(p))
        else:
            orc = NS3DOracle(oper, f=p.get("f"), turb_model=turb, **projection_kwargs(p),
                             **solver_kwargs(p))
    orc.state_spect[:] = d["S_init"]
    orc.state_phys[:] = d["phys_init"]
    fc = forcing_config(p)
    if fc is not None:  # drawn from np.random seeded as the reference run was
        np.random.seed(fc["np_seed"])
        orc.forcing = CoarseForcingOracle(
            orc.oper, orc.nvar, [KEY_NAMES.index(k) for k in fc["key_forced"]], fc["type"],
            fc["nkmin_forcing"], fc["nkmax_forcing"], fc["forcing_rate"],
            fc["time_correlation"])
    return orc, d, p


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("name", CASES_2D + CASES_3D)
def test_oracle_tendency_matches_reference(name):
    orc, d, _ = make_oracle(name)
    tend = orc.tendencies_nonlin(orc.state_spect.copy())
    assert rel(tend, d["tend0"]) < 1e-13


@pytest.mark.parametrize("name", CASES_2D + CASES_3D)
def test_oracle_steps_match_reference(name):
    orc, d, p = make_oracle(name)
    steps = int(p["steps"])
    for it in range(steps):
        orc.one_time_step()
        assert orc.deltat == d["dts"][it]
        if it == 0:
            assert rel(orc.state_spect, d["S_1"]) < 1e-13
    assert rel(orc.state_spect, d["S_end"]) < 1e-13
    np.testing.assert_allclose([orc.compute_energy()], d["E"][-1:], rtol=1e-13)


@pytest.mark.parametrize("name", CASES_2D + CASES_3D)
def test_reference_tendency_conserves_energy(name):
    """``ns2d/test_solver.py:49-69`` and ``ns3d/test_solver.py:73-96``."""
    if "tgv" in name:
        pytest.skip("Taylor-Green at t=0: the tendency is round-off only")
    if "smag" in name:
        pytest.skip("with a turbulence model the tendency dissipates energy")
    if "toroidal" in name or "poloidal" in name:
        pytest.skip("the projected tendency acts on an unprojected initial state")
    orc, d, p = make_oracle(name)
    S, F = d["S_init"], d["tend0"]
    T = np.real(np.conj(F) * S)
    if p.get("bouss"):
        # the bouss equations exchange kinetic energy with b (the buoyancy
        # force does work) and have no N^2 term to close a quadratic budget
        pytest.skip("bouss: no conserved quadratic energy")
    if p.get("N") is not None and name.startswith("ns2d"):
        # ns2d/strat/solver.py:212-240 (check_energy_conservation): kinetic
        # energy from the vorticity (1 / k^2, 0 at k = 0) plus b / N^2
        inv_k2 = orc.oper.inv_K_square_nozero
        T = 0.5 * inv_k2 * T[0] + T[1] / (2 * p["N"] ** 2)
        T = T[None]
    elif p.get("N") is not None:  # ns3d/strat/test_solver.py:34-58: b weighted by 1/N^2
        T[3] /= p["N"] ** 2
    T = T.sum(axis=0)
    ratio = orc.oper.sum_wavenumbers(T) / orc.oper.sum_wavenumbers(np.abs(T))
    assert abs(ratio) < 1e-14


def test_parseval_normalisation():
    """``fluidsim/base/state.py:385-392``: sum_k |v_k|^2/2 == <v^2>/2."""
    oper = OperNumpy3D(12, 10, 8, 3.0, 2.0, 1.0)
    v = np.random.default_rng(0).standard_normal(oper.shapeX)
    vk = oper.fft(v)
    assert np.isclose(oper.sum_wavenumbers(np.abs(vk) ** 2 / 2), np.mean(v**2) / 2)
    assert np.allclose(oper.ifft(vk), v)


def test_index_layout():
    """``fluidsim/operators/test/test_operators3d.py:226-301`` layout."""
    oper = OperNumpy3D(16, 12, 8)
    assert oper.shapeK == (8, 12, 9)
    assert oper.get_dimX_K() == (0, 1, 2)
    kz, ky, kx = oper.get_k_adim_loc()
    assert list(kx) == list(range(9))
    assert list(ky) == [0, 1, 2, 3, 4, 5, 6, -5, -4, -3, -2, -1]
    assert list(kz) == [0, 1, 2, 3, 4, -3, -2, -1]
