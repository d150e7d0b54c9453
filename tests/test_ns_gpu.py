"""GPU parity of the fused ns2d / ns3d time step against the reference fixtures.

FP64: relative L2 <= 1e-12 on every state variable after 10 steps (and on
the first tendency); FP32: relative L2 <= 1e-5 after 10 steps.
"""
import random

import numpy as np
import pytest

from golden_cases import (CASES_2D, CASES_3D, forcing_config, lengths, load, projection_kwargs,
                          scheme)

pytestmark = pytest.mark.gpu

TOL_F64 = 1e-12
TOL_F32 = 1e-5


def make_sim(name, precision="float64"):
    import torch
    from fluidsim_gb300.solvers import (SimulNS2D, SimulNS2DBouss, SimulNS2DStrat, SimulNS3D,
                                        SimulNS3DBouss, SimulNS3DStrat)
    d, p = load(name)
    ndim = 2 if name.startswith("ns2d") else 3
    strat = p.get("N") is not None
    if ndim == 2:
        Simul = SimulNS2DBouss if p.get("bouss") else (SimulNS2DStrat if strat else SimulNS2D)
    else:
        Simul = SimulNS3DBouss if p.get("bouss") else (SimulNS3DStrat if strat else SimulNS3D)
    params = Simul.create_default_params()
    if p.get("N") is not None:
        params.N = p["N"]
    params.precision = precision
    params.oper.nx, params.oper.ny = int(p["nx"]), int(p["ny"])
    L = lengths(p, ndim)
    params.oper.Lx, params.oper.Ly = L[0], L[1]
    if ndim == 3:
        params.oper.nz = int(p["nz"])
        params.oper.Lz = L[2]
        params.f = p.get("f")
        for k, v in projection_kwargs(p).items():
            setattr(params, k, v)
        if p.get("smagorinsky_C") is not None:
            params.turb_model.enable = True
            params.turb_model.type = "smagorinsky"
            params.turb_model.smagorinsky.C = p["smagorinsky_C"]
    else:
        params.beta = p.get("beta") or 0.0
    for k in ("nu_2", "nu_4", "nu_8", "nu_m4"):
        if p.get(k) is not None:
            setattr(params, k, p[k])
    ts = params.time_stepping
    ts.USE_CFL = bool(p["USE_CFL"])
    ts.deltat0 = p["deltat0"]
    if p.get("deltat_max") is not None:
        ts.deltat_max = p["deltat_max"]
    ts.cfl_coef = p.get("cfl_coef")
    ts.type_time_scheme = scheme(p)
    ts.USE_T_END = False
    ts.it_end = int(p["steps"])
    if p.get("phase_seed") is not None:  # the random phase schemes draw with `random`
        random.seed(int(p["phase_seed"]))
    fc = forcing_config(p)
    if fc is not None:  # the reference's forcing maker, seeded as the fixture's run
        pf = params.forcing
        pf.enable, pf.type, pf.key_forced = True, fc["type"], fc["key_forced"]
        pf.nkmin_forcing, pf.nkmax_forcing = fc["nkmin_forcing"], fc["nkmax_forcing"]
        pf.forcing_rate = fc["forcing_rate"]
        pf.tcrandom.time_correlation = fc["time_correlation"]
        pf.seed = fc["np_seed"]
    sim = Simul(params)
    sim.state.init_statespect_from(**{k: torch.from_numpy(d["S_init"][i])
                                      for i, k in enumerate(sim.state.keys_state_spect)})
    return sim, d, p


def rel_l2_per_var(a, b):
    """Largest per-variable relative L2 error (absolute where the reference
    variable is identically zero, as vz under the toroidal projection)."""
    out = []
    for i in range(len(b)):
        nb = np.linalg.norm(b[i])
        d = np.linalg.norm(a[i] - b[i])
        out.append(d / nb if nb > 0 else d)
    return max(out)


@pytest.mark.parametrize("name", CASES_2D + CASES_3D)
def test_tendencies_fp64(cuda, name):
    sim, d, _ = make_sim(name)
    tend = sim.tendencies_nonlin(sim.state.state_spect).cpu().numpy()
    if "tgv" in name:  # round-off-only tendency: absolute check
        assert np.abs(tend - d["tend0"]).max() < 1e-14
    else:
        assert rel_l2_per_var(tend, d["tend0"]) < TOL_F64


@pytest.mark.parametrize("name", CASES_2D + CASES_3D)
def test_ten_steps_fp64(cuda, name):
    sim, d, p = make_sim(name)
    ts = sim.time_stepping
    ts.one_time_step()
    assert rel_l2_per_var(sim.state.state_spect.cpu().numpy(), d["S_1"]) < TOL_F64
    dts = [ts.deltat]
    while ts.it < int(p["steps"]):
        ts.one_time_step()
        dts.append(ts.deltat)
    np.testing.assert_allclose(dts, d["dts"], rtol=1e-12)
    assert rel_l2_per_var(sim.state.state_spect.cpu().numpy(), d["S_end"]) < TOL_F64
    np.testing.assert_allclose(sim.output.compute_energy(), d["E"][-1], rtol=1e-12)
    phys = sim.state.state_phys.cpu().numpy()
    assert rel_l2_per_var(phys, d["phys_end"]) < TOL_F64


@pytest.mark.parametrize("name", ["ns2d_256_c1", "ns3d_iso_24x16x32_f", "ns3d_tgv_32",
                                  "ns2d_40x32_rk2", "ns3d_heun_24x16x32_f", "ns2d_32_rk2ps",
                                  "ns3d_eulerps_32", "ns3d_rk2psx_16x24x32_f",
                                  "ns3d_strat_64_f_rk2", "ns3d_rk2psr_24x16x32_f",
                                  "ns2d_32_eulerpsr", "ns2d_strat_64_rk2", "ns3d_tcrandom_32"])
def test_ten_steps_fp32(cuda, name):
    sim, d, p = make_sim(name, "float32")
    sim.time_stepping.start()
    err = rel_l2_per_var(sim.state.state_spect.cpu().numpy().astype(np.complex128), d["S_end"])
    assert err < TOL_F32, err


@pytest.mark.parametrize("name", ["ns2d_48x40_beta", "ns3d_iso_24x16x32_f",
                                  "ns3d_strat_64x32x32", "ns2d_strat_64x32"])
def test_spatial_means_match_oracle(cuda, name):
    from test_oracle_golden import make_oracle
    sim, d, _ = make_sim(name)
    orc, _, _ = make_oracle(name)
    got = sim.output.compute_spatial_means()
    ref = orc.spatial_means()
    for k, v in ref.items():
        assert np.isclose(got[k], v, rtol=1e-12, atol=1e-300), k
    k, E = sim.output.compute_spectrum()  # kinetic energy spectrum
    assert np.isclose(E.sum() * (k[1] - k[0]), got.get("EK", got["E"]), rtol=1e-12)


def test_tendency_conserves_energy_gpu(cuda):
    """``ns3d/test_solver.py:73-96`` on the GPU path (20 x 15 x 10 grid)."""
    sim, d, _ = make_sim("ns3d_20x15x10")
    S = sim.state.state_spect
    F = sim.tendencies_nonlin(S)
    T = (F.conj() * S).real.sum(dim=0)
    ratio = sim.oper.sum_wavenumbers(T) / sim.oper.sum_wavenumbers(T.abs())
    assert abs(ratio) < 1e-14


def test_strat_tendency_conserves_energy_gpu(cuda):
    """``ns3d/strat/test_solver.py:34-58`` on the GPU path: kinetic plus
    potential (b weighted by 1 / N^2) energy transfer sums to zero."""
    sim, d, p = make_sim("ns3d_strat_64x32x32")
    S = sim.state.state_spect
    F = sim.tendencies_nonlin(S)
    T = (F.conj() * S).real
    T[3] /= p["N"] ** 2
    T = T.sum(dim=0)
    ratio = sim.oper.sum_wavenumbers(T) / sim.oper.sum_wavenumbers(T.abs())
    assert abs(ratio) < 1e-14


def test_strat2d_tendency_conserves_energy_gpu(cuda):
    """``ns2d/strat/solver.py:212-240`` (check_energy_conservation) on the
    GPU path: kinetic (from the vorticity) plus potential energy transfer."""
    sim, d, p = make_sim("ns2d_strat_64x32")
    S = sim.state.state_spect
    F = sim.tendencies_nonlin(S)
    T = (F.conj() * S).real
    k2 = sim.oper.K2.clone()
    k2[0, 0] = 1.0
    TK = 0.5 * T[0] / k2
    TK[0, 0] = 0.0
    T = TK + T[1] / (2 * p["N"] ** 2)
    ratio = sim.oper.sum_wavenumbers(T) / sim.oper.sum_wavenumbers(T.abs())
    assert abs(ratio) < 1e-14


def test_nan_raises_value_error(cuda):
    sim, d, _ = make_sim("ns2d_32_cfl")
    sim.params.time_stepping.USE_CFL = False
    sim.state.state_spect[0, 3, 2] = float("nan")
    with pytest.raises(ValueError, match="nan at it = 0"):
        sim.time_stepping.one_time_step()


def test_max_velocity_matches_state_phys(cuda):
    sim, d, _ = make_sim("ns3d_iso_24x16x32_f")
    vmax = sim.max_velocity()
    phys = sim.state.state_phys.cpu().numpy()
    np.testing.assert_allclose(vmax, np.abs(phys).reshape(3, -1).max(axis=1), rtol=1e-14)


def test_set_state_spect_rotation_matches_in_place(cuda):
    """Steps on rotated state buffers (set_state_spect) give the same states
    as steps on one buffer; a tensor of another shape or dtype is refused."""
    import torch
    sim_a, d, _ = make_sim("ns3d_iso_24x16x32_f")
    sim_b, _, _ = make_sim("ns3d_iso_24x16x32_f")
    S0 = sim_a.state.state_spect.clone()
    bufs = [torch.empty_like(S0) for _ in range(3)]
    for i in range(4):
        sim_a.time_stepping.one_time_step()
        nxt = bufs[i % 3]
        nxt.copy_(sim_b.state.state_spect)
        sim_b.state.set_state_spect(nxt)
        sim_b.time_stepping.one_time_step()
        assert sim_b.state.state_spect.data_ptr() == nxt.data_ptr()
        assert torch.equal(sim_a.state.state_spect, nxt)
    with pytest.raises(ValueError):
        sim_b.state.set_state_spect(S0[:2].clone())
    with pytest.raises(ValueError):
        sim_b.state.set_state_spect(S0.to(torch.complex64 if S0.dtype == torch.complex128
                                          else torch.complex128))
