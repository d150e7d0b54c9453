"""Generate the golden fixtures from the reference's own Python code.

Usage (needs the fluidsim 0.8.3 sources; writes ``tests/golden/*.npz``)::

    python tests/golden/make_golden.py <fluidsim source root> [case ...]

Each case builds a reference ns2d / ns3d ``Simul`` with ``oracle.refshim``
(the reference's ``TimeSteppingPseudoSpectral`` RK4, CFL logic,
``tendencies_nonlin``, ``compute_freq_diss`` and state classes, unmodified,
on top of the numpy fluidfft restatement), runs it from a seeded initial
state and stores the inputs, the first tendency and the states/time steps
after 1 and 10 steps.  The oracle restatement is run beside it and must
agree to 1e-13 before anything is written.
"""

import random
import sys
from math import pi
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle import refshim  # noqa: E402
from oracle.spectral import OperNumpy2D, OperNumpy3D  # noqa: E402
from oracle.solvers import NS2DOracle, NS2DStratOracle, NS3DOracle, NS3DStratOracle  # noqa: E402
from oracle.turb import smagorinsky_forcing  # noqa: E402
from oracle.forcing import CoarseForcingOracle  # noqa: E402
from fluidsim_gb300.init_fields import (  # noqa: E402
    isotropic_3d, noise_rot_2d, taylor_green_3d)

CASES_2D = [
    dict(name="ns2d_32_cfl", nx=32, ny=32, Lx=6.0, Ly=6.0, nu_8=2e-5,
         USE_CFL=True, deltat0=0.2, deltat_max=0.2, cfl_coef=None,
         init=dict(kmin=2.0, kmax=6.0, seed=1), steps=10),
    dict(name="ns2d_48x40_beta", nx=48, ny=40, Lx=2 * pi, Ly=2 * pi * 40 / 48,
         nu_2=1e-3, nu_m4=1e-3, beta=1.0, USE_CFL=False, deltat0=0.01,
         init=dict(kmin=2.0, kmax=9.0, seed=2), steps=10),
    dict(name="ns2d_256_c1", nx=256, ny=256, Lx=2 * pi, Ly=2 * pi, nu_2=1e-4,
         USE_CFL=False, deltat0=1e-3, init=dict(kmin=4.0, kmax=8.0, seed=2024),
         steps=10),
    dict(name="ns2d_32_euler", nx=32, ny=32, Lx=6.0, Ly=6.0, nu_2=1e-3,
         USE_CFL=True, deltat0=0.2, deltat_max=0.2, cfl_coef=None,
         type_time_scheme="Euler", init=dict(kmin=2.0, kmax=6.0, seed=5), steps=10),
    dict(name="ns2d_40x32_rk2", nx=40, ny=32, Lx=2 * pi, Ly=2 * pi * 32 / 40,
         nu_2=1e-3, beta=0.5, USE_CFL=True, deltat0=0.2, deltat_max=0.2, cfl_coef=None,
         type_time_scheme="RK2", init=dict(kmin=2.0, kmax=8.0, seed=7), steps=10),
    dict(name="ns2d_32_rk2ps", nx=32, ny=32, Lx=6.0, Ly=6.0, nu_2=1e-3,
         USE_CFL=True, deltat0=0.2, deltat_max=0.2, cfl_coef=None,
         type_time_scheme="RK2_phaseshift", init=dict(kmin=2.0, kmax=10.0, seed=11),
         steps=10),
    dict(name="ns2d_36x32_eulerps", nx=36, ny=32, Lx=2 * pi, Ly=5.0, nu_2=2e-3,
         USE_CFL=False, deltat0=5e-3, type_time_scheme="Euler_phaseshift",
         init=dict(kmin=2.0, kmax=9.0, seed=12), steps=10),
    dict(name="ns2d_32_eulerpsr", nx=32, ny=32, Lx=6.0, Ly=6.0, nu_2=1e-3,
         USE_CFL=False, deltat0=5e-3, type_time_scheme="Euler_phaseshift_random",
         phase_seed=101, init=dict(kmin=2.0, kmax=10.0, seed=13), steps=10),
    dict(name="ns2d_40x32_rk2psr", nx=40, ny=32, Lx=2 * pi, Ly=5.0, nu_2=1e-3, beta=0.5,
         USE_CFL=True, deltat0=0.2, deltat_max=0.2, cfl_coef=None,
         type_time_scheme="RK2_phaseshift_random", phase_seed=102,
         init=dict(kmin=2.0, kmax=9.0, seed=14), steps=10),
    dict(name="ns2d_strat_64x32", nx=64, ny=32, Lx=2 * pi, Ly=pi, nu_2=1e-3, N=1.5,
         USE_CFL=True, deltat0=0.2, deltat_max=0.2, cfl_coef=None,
         init=dict(kmin=2.0, kmax=8.0, seed=15), b_init=dict(kmin=2.0, kmax=6.0, seed=16),
         steps=10),
    dict(name="ns2d_bouss_64x32", nx=64, ny=32, Lx=2 * pi, Ly=pi, nu_2=1e-3, bouss=True,
         USE_CFL=True, deltat0=0.2, deltat_max=0.2, cfl_coef=None,
         init=dict(kmin=2.0, kmax=8.0, seed=19), b_init=dict(kmin=2.0, kmax=6.0, seed=20),
         steps=10),
    dict(name="ns2d_strat_64_rk2", nx=64, ny=64, Lx=6.0, Ly=6.0, nu_8=1e-9, N=3.0,
         USE_CFL=False, deltat0=5e-3, type_time_scheme="RK2",
         init=dict(kmin=2.0, kmax=10.0, seed=17), b_init=dict(kmin=3.0, kmax=9.0, seed=18),
         steps=10),
]

CASES_3D = [
    dict(name="ns3d_20x15x10", nx=20, ny=15, nz=10, Lx=6.0, Ly=4.5, Lz=3.0,
         nu_2=1e-2, USE_CFL=True, deltat0=0.2, deltat_max=0.2,
         cfl_coef=None, init="iso", seed=3, steps=10),
    dict(name="ns3d_tgv_32", nx=32, ny=32, nz=32, nu_2=1 / 1600, USE_CFL=True,
         deltat0=0.2, deltat_max=0.2, cfl_coef=0.5, init="tgv", steps=10),
    dict(name="ns3d_iso_24x16x32_f", nx=24, ny=16, nz=32, nu_2=5e-3, f=1.0,
         USE_CFL=False, deltat0=5e-3, init="iso", seed=4, steps=10),
    dict(name="ns3d_smag_20x24x16", nx=20, ny=24, nz=16, nu_2=1e-3,
         smagorinsky_C=0.18, USE_CFL=True, deltat0=0.2, deltat_max=0.2,
         cfl_coef=0.5, init="iso", seed=6, steps=10),
    dict(name="ns3d_rk2_20x15x10", nx=20, ny=15, nz=10, Lx=6.0, Ly=4.5, Lz=3.0,
         nu_2=1e-2, USE_CFL=True, deltat0=0.2, deltat_max=0.2, cfl_coef=None,
         type_time_scheme="RK2", init="iso", seed=8, steps=10),
    dict(name="ns3d_heun_24x16x32_f", nx=24, ny=16, nz=32, nu_2=5e-3, f=1.0,
         USE_CFL=False, deltat0=5e-3, type_time_scheme="RK2_trapezoid", init="iso",
         seed=9, steps=10),
    dict(name="ns3d_euler_tgv_32", nx=32, ny=32, nz=32, nu_2=1 / 1600, USE_CFL=True,
         deltat0=0.2, deltat_max=0.2, cfl_coef=None, type_time_scheme="Euler",
         init="tgv", steps=10),
    dict(name="ns3d_rk2ps_20x15x10", nx=20, ny=15, nz=10, Lx=6.0, Ly=4.5, Lz=3.0,
         nu_2=1e-2, USE_CFL=True, deltat0=0.2, deltat_max=0.2, cfl_coef=None,
         type_time_scheme="RK2_phaseshift", init="iso", seed=13, steps=10),
    dict(name="ns3d_rk2psx_16x24x32_f", nx=16, ny=24, nz=32, nu_2=5e-3, f=0.5,
         USE_CFL=True, deltat0=0.2, deltat_max=0.2, cfl_coef=None,
         type_time_scheme="RK2_phaseshift_exact", init="iso", seed=14, steps=10),
    dict(name="ns3d_eulerps_32", nx=32, ny=32, nz=32, nu_2=2e-3, USE_CFL=False,
         deltat0=2e-3, type_time_scheme="Euler_phaseshift", init="iso", seed=15,
         steps=10),
    dict(name="ns3d_rk2psr_24x16x32_f", nx=24, ny=16, nz=32, nu_2=5e-3, f=0.5,
         USE_CFL=True, deltat0=0.2, deltat_max=0.2, cfl_coef=None,
         type_time_scheme="RK2_phaseshift_random", phase_seed=103, init="iso", seed=22,
         steps=10),
    dict(name="ns3d_eulerpsr_32", nx=32, ny=32, nz=32, nu_2=2e-3, USE_CFL=False,
         deltat0=2e-3, type_time_scheme="Euler_phaseshift_random", phase_seed=104,
         init="iso", seed=23, steps=10),
    dict(name="ns3d_toroidal_24x20x16", nx=24, ny=20, nz=16, nu_2=5e-3, f=1.0,
         USE_CFL=True, deltat0=0.2, deltat_max=0.2, cfl_coef=0.5, projection="toroidal",
         init="iso", seed=16, steps=10),
    dict(name="ns3d_poloidal_32_novz", nx=32, ny=32, nz=32, nu_2=5e-3, USE_CFL=True,
         deltat0=0.2, deltat_max=0.2, cfl_coef=0.5, projection="poloidal", no_vz_kz0=True,
         init="iso", seed=17, steps=10),
    dict(name="ns3d_strat_64x32x32", nx=64, ny=32, nz=32, Lx=2 * pi, Ly=pi, Lz=pi,
         nu_2=2e-3, N=2.0, USE_CFL=True, deltat0=0.2, deltat_max=0.2, cfl_coef=0.5,
         init="iso", seed=18, b_seed=19, steps=10),
    dict(name="ns3d_bouss_32x32x64", nx=64, ny=32, nz=32, Lx=2 * pi, Ly=pi, Lz=pi,
         nu_2=2e-3, N=1.0, bouss=True, USE_CFL=True, deltat0=0.2, deltat_max=0.2,
         cfl_coef=0.5, init="iso", seed=24, b_seed=25, steps=10),
    dict(name="ns3d_strat_64_f_rk2", nx=64, ny=64, nz=64, nu_2=1e-3, N=4.0, f=0.5,
         USE_CFL=True, deltat0=0.2, deltat_max=0.2, cfl_coef=None, type_time_scheme="RK2",
         init="iso", seed=20, b_seed=21, steps=10),
]

# coarse normalized forcings (the reference's forcing makers of
# fluidsim/base/forcing/specific.py run through refshim); np_seed seeds the
# global np.random before the forcing is created
CASES_3D += [
    dict(name="ns3d_tcrandom_32", nx=32, ny=32, nz=32, nu_2=1e-2, USE_CFL=True,
         deltat0=0.2, deltat_max=0.2, cfl_coef=0.5, init="iso", seed=30, steps=10,
         np_seed=31, forcing=dict(type="tcrandom", key_forced=["vx_fft", "vy_fft", "vz_fft"],
                                  nkmin_forcing=2, nkmax_forcing=3, forcing_rate=0.3,
                                  time_correlation=0.02)),
    dict(name="ns3d_tcrandom_vx_24x32x16", nx=24, ny=32, nz=16, Lx=2 * pi, Ly=4 * pi,
         Lz=pi, nu_2=5e-3, USE_CFL=False, deltat0=5e-3, init="iso", seed=32, steps=10,
         np_seed=33, forcing=dict(type="tcrandom", key_forced="vx_fft", nkmin_forcing=1,
                                  nkmax_forcing=2, forcing_rate=1.0)),
    dict(name="ns3d_random_32", nx=32, ny=32, nz=32, nu_2=5e-3, USE_CFL=False,
         deltat0=4e-3, init="iso", seed=34, steps=10, np_seed=35,
         forcing=dict(type="random", key_forced=["vz_fft"], nkmin_forcing=3, nkmax_forcing=4,
                      forcing_rate=0.5)),
    dict(name="ns3d_proportional_32", nx=32, ny=32, nz=32, nu_2=5e-3, USE_CFL=False,
         deltat0=4e-3, init="iso", seed=36, steps=10, np_seed=37,
         forcing=dict(type="proportional", key_forced="vy_fft", nkmin_forcing=2,
                      nkmax_forcing=4, forcing_rate=0.2)),
]

FORCING_CODES = {"tcrandom": 0, "random": 1, "proportional": 2}
KEY_BITS = {"vx_fft": 1, "vy_fft": 2, "vz_fft": 4}

PROJECTION_CODES = {None: 0, "toroidal": 1, "vortical": 1, "poloidal": 2}

SCHEME_CODES = {"RK4": 0, "Euler": 1, "RK2": 2, "RK2_trapezoid": 3, "Euler_phaseshift": 4,
                "RK2_phaseshift": 5, "RK2_phaseshift_exact": 6, "Euler_phaseshift_random": 7,
                "RK2_phaseshift_random": 8}


class _PhaseRNG:
    """The random phase schemes draw with the global ``random`` module and the
    forcings with the global ``np.random``; the reference solver and the
    oracle each get the sequences of ``random.seed(phase_seed)`` and
    ``np.random.seed(np_seed)``, kept apart while their steps alternate."""

    def __init__(self, seed, np_seed=None):
        self.states = {}
        self.np_states = {}
        self.seed = seed
        self.np_seed = np_seed

    def run(self, who, fn):
        if self.seed is not None:
            if who in self.states:
                random.setstate(self.states[who])
            else:
                random.seed(self.seed)
        if self.np_seed is not None:
            if who in self.np_states:
                np.random.set_state(self.np_states[who])
            else:
                np.random.seed(self.np_seed)
        try:
            return fn()
        finally:
            if self.seed is not None:
                self.states[who] = random.getstate()
            if self.np_seed is not None:
                self.np_states[who] = np.random.get_state()


def _kw(case, keys):
    return {k: case[k] for k in keys if k in case}


def run_2d(mods, case):
    oper = OperNumpy2D(case["nx"], case["ny"], case["Lx"], case["Ly"])
    rot0 = noise_rot_2d(case["nx"], case["ny"], case["Lx"], case["Ly"],
                        **case["init"])
    kw = _kw(case, ["nu_2", "nu_4", "nu_8", "nu_m4", "USE_CFL", "deltat0",
                    "deltat_max", "cfl_coef", "type_time_scheme"])
    rng = _PhaseRNG(case.get("phase_seed"))
    bouss = bool(case.get("bouss"))
    strat = case.get("N") is not None or bouss
    sim = rng.run("ref", lambda: refshim.make_ns2d(mods, oper, beta=case.get("beta", 0.0),
                                                    N=case.get("N"), bouss=bouss, **kw))
    if strat:  # rot and b, dealiased, then the phys/spect round trip
        b0 = noise_rot_2d(case["nx"], case["ny"], case["Lx"], case["Ly"], **case["b_init"])
        r, b = rot0.copy(), b0.copy()
        oper.dealiasing(r)
        oper.dealiasing(b)
        sim.state.state_spect.set_var("rot_fft", r)
        sim.state.state_spect.set_var("b_fft", b)
        sim.state.statephys_from_statespect()
    else:
        sim.state.init_from_rotfft(rot0.copy())
    S_init = np.array(sim.state.state_spect)
    phys_init = np.array(sim.state.state_phys)
    tend0 = np.array(sim.tendencies_nonlin(state_spect=sim.state.state_spect))
    if strat:  # (ns2d.bouss: the strat equations with N = 0)
        orc = NS2DStratOracle(oper, N=case.get("N") or 0.0, **kw)
        orc.init_from_rotbfft(rot0.copy(), b0.copy())
    else:
        orc = rng.run("orc", lambda: NS2DOracle(oper, beta=case.get("beta", 0.0), **kw))
        orc.init_from_rotfft(rot0.copy())
    assert np.abs(orc.state_spect - S_init).max() <= 1e-15 * np.abs(S_init).max()
    np.testing.assert_allclose(orc.tendencies_nonlin(orc.state_spect), tend0,
                               rtol=0, atol=1e-13 * np.abs(tend0).max())
    out = dict(S_init=S_init, phys_init=phys_init, tend0=tend0, dts=[], E=[])
    for it in range(case["steps"]):
        rng.run("ref", sim.time_stepping.one_time_step)
        rng.run("orc", orc.one_time_step)
        out["dts"].append(sim.time_stepping.deltat)
        S = np.array(sim.state.state_spect)
        err = np.abs(orc.state_spect - S).max() / np.abs(S).max()
        assert err < 1e-13, (case["name"], it, err)
        assert orc.deltat == sim.time_stepping.deltat
        out["E"].append(orc.compute_energy())
        if it == 0:
            out["S_1"] = S
    out["S_end"] = np.array(sim.state.state_spect)
    out["phys_end"] = np.array(sim.state.state_phys)
    if case.get("phase_seed") is not None:  # (alpha, beta) of every step
        out["phase_pairs"] = np.asarray(orc.phase_pairs_used)
    return out


def run_3d(mods, case):
    nx, ny, nz = case["nx"], case["ny"], case["nz"]
    L = (case.get("Lx", 2 * pi), case.get("Ly", 2 * pi), case.get("Lz", 2 * pi))
    oper = OperNumpy3D(nx, ny, nz, *L)
    if case["init"] == "tgv":
        v0 = taylor_green_3d(nx, ny, nz, *L)
    else:
        v0 = isotropic_3d(nx, ny, nz, *L, seed=case["seed"])
    kw = _kw(case, ["nu_2", "nu_4", "nu_8", "nu_m4", "USE_CFL", "deltat0",
                    "deltat_max", "cfl_coef", "type_time_scheme"])
    proj = dict(projection=case.get("projection"), no_vz_kz0=case.get("no_vz_kz0", False))
    strat = case.get("N") is not None
    rng = _PhaseRNG(case.get("phase_seed"), case.get("np_seed"))
    sim = rng.run("ref", lambda: refshim.make_ns3d(
        mods, oper, f=case.get("f"), smagorinsky_C=case.get("smagorinsky_C"),
        N=case.get("N"), bouss=bool(case.get("bouss")), forcing=case.get("forcing"),
        **proj, **kw))
    sim.state.init_from_vxvyvzfft(*[c.copy() for c in v0])
    if strat:  # a buoyancy field as well (set after the velocity round trip)
        b0 = isotropic_3d(nx, ny, nz, *L, seed=case["b_seed"])[0]
        sim.state.state_spect.set_var("b_fft", b0)
        sim.state.statephys_from_statespect()
    S_init = np.array(sim.state.state_spect)
    phys_init = np.array(sim.state.state_phys)
    tend0 = np.array(sim.tendencies_nonlin(state_spect=sim.state.state_spect))
    turb = None
    if case.get("smagorinsky_C") is not None:
        C = case["smagorinsky_C"]

        def turb(o, vx, vy, vz):
            return smagorinsky_forcing(o, vx, vy, vz, C=C)
    if strat:
        orc = NS3DStratOracle(oper, N=case["N"], f=case.get("f"), bouss=bool(case.get("bouss")),
                              **proj, **kw)
    else:
        orc = rng.run("orc", lambda: NS3DOracle(oper, f=case.get("f"), turb_model=turb,
                                                **proj, **kw))
    orc.init_from_vxvyvzfft(*[c.copy() for c in v0])
    if strat:
        orc.state_spect[3] = b0
        orc.statephys_from_statespect()
    if case.get("forcing") is not None:
        orc.forcing = rng.run("orc", lambda: oracle_forcing(orc, case["forcing"]))
    assert np.abs(orc.state_spect - S_init).max() <= 1e-15 * np.abs(S_init).max()
    np.testing.assert_allclose(orc.tendencies_nonlin(orc.state_spect), tend0,
                               rtol=0, atol=1e-13 * np.abs(tend0).max())
    out = dict(S_init=S_init, phys_init=phys_init, tend0=tend0, dts=[], E=[])
    for it in range(case["steps"]):
        rng.run("ref", sim.time_stepping.one_time_step)
        rng.run("orc", orc.one_time_step)
        out["dts"].append(sim.time_stepping.deltat)
        S = np.array(sim.state.state_spect)
        err = np.abs(orc.state_spect - S).max() / np.abs(S).max()
        assert err < 1e-13, (case["name"], it, err)
        assert orc.deltat == sim.time_stepping.deltat
        out["E"].append(orc.compute_energy())
        if it == 0:
            out["S_1"] = S
    out["S_end"] = np.array(sim.state.state_spect)
    out["phys_end"] = np.array(sim.state.state_phys)
    if case.get("phase_seed") is not None:  # (alpha, beta) of every step
        out["phase_pairs"] = np.asarray(orc.phase_pairs_used)
    return out


def oracle_forcing(orc, fc):
    """The oracle's restatement of the forcing maker ``fc`` describes."""
    keys = fc["key_forced"]
    keys = [keys] if isinstance(keys, str) else keys
    names = ["vx_fft", "vy_fft", "vz_fft"]
    return CoarseForcingOracle(
        orc.oper, orc.nvar, [names.index(k) for k in keys], fc["type"],
        fc["nkmin_forcing"], fc["nkmax_forcing"], fc["forcing_rate"],
        fc.get("time_correlation", "based_on_forcing_rate"))


def _params_array(case):
    keys = ["nx", "ny", "nz", "Lx", "Ly", "Lz", "nu_2", "nu_4", "nu_8", "nu_m4",
            "beta", "f", "USE_CFL", "deltat0", "deltat_max", "cfl_coef", "steps",
            "smagorinsky_C", "N", "phase_seed", "bouss"]
    out = {("p_" + k): np.asarray(case[k] if case.get(k) is not None else np.nan,
                                  dtype=np.float64)
           for k in keys if k in case}
    out["p_scheme"] = np.asarray(SCHEME_CODES[case.get("type_time_scheme", "RK4")],
                                 dtype=np.float64)
    out["p_projection"] = np.asarray(PROJECTION_CODES[case.get("projection")], dtype=np.float64)
    out["p_no_vz_kz0"] = np.asarray(float(case.get("no_vz_kz0", False)))
    fc = case.get("forcing")
    if fc is not None:
        keys = fc["key_forced"]
        keys = [keys] if isinstance(keys, str) else keys
        tc = fc.get("time_correlation", "based_on_forcing_rate")
        for k, v in {"forcing_type": FORCING_CODES[fc["type"]],
                     "forced_keys": sum(KEY_BITS[k] for k in keys),
                     "nkmin_forcing": fc["nkmin_forcing"],
                     "nkmax_forcing": fc["nkmax_forcing"],
                     "forcing_rate": fc["forcing_rate"],
                     "time_correlation": np.nan if tc == "based_on_forcing_rate" else tc,
                     "np_seed": case["np_seed"]}.items():
            out["p_" + k] = np.asarray(v, dtype=np.float64)
    return out


def main(ref_root, only=None):
    mods = refshim.load_reference(ref_root)
    for case in CASES_2D:
        if only and case["name"] not in only:
            continue
        out = run_2d(mods, case)
        np.savez_compressed(HERE / f"{case['name']}.npz", **_params_array(case),
                            **{k: np.asarray(v) for k, v in out.items()})
        print(case["name"], "ok", out["dts"][-1], out["E"][-1])
    for case in CASES_3D:
        if only and case["name"] not in only:
            continue
        out = run_3d(mods, case)
        np.savez_compressed(HERE / f"{case['name']}.npz", **_params_array(case),
                            **{k: np.asarray(v) for k, v in out.items()})
        print(case["name"], "ok", out["dts"][-1], out["E"][-1])


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: python tests/golden/make_golden.py <fluidsim source root> [case ...]")
    main(sys.argv[1], sys.argv[2:])
