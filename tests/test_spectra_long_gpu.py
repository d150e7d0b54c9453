"""Long runs where chaos decorrelates pointwise fields: spectra still agree.

ns2d decaying turbulence (config C1's initial field: band-passed Gaussian
noise vorticity, k in [4, 8], rms velocity 1) with CFL time steps is run on
the float64 CPU oracle and on the GPU in FP64 and FP32.  Rounding
differences grow exponentially, so after a few eddy turnovers the pointwise
fields of the runs differ at order one, while the energy E(t), enstrophy
Z(t) and the time-averaged energy and enstrophy spectra E(k), Z(k) must
still agree: the reference's own comparison for long runs
(``fluidsim/solvers/ns2d/output/spectra.py:16-27``,
``ns2d/output/spatial_means.py:23-36``).

``long_run_ns2d`` is shared with ``tests/validation/spectra_long.py``.
"""
from math import pi

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def octave_bands(k, spec, kmax):
    """Sums of a spectrum over the bands [1, 2), [2, 4), ... up to kmax."""
    edges = [1.0]
    while edges[-1] < kmax:
        edges.append(min(2 * edges[-1], kmax))
    return np.array([spec[(k >= a) & (k < b)].sum() for a, b in zip(edges[:-1], edges[1:])])


def long_run_ns2d(n=128, nu_2=5e-4, t_end=20.0, t_avg=10.0, every=0.5, seed=3,
                  precisions=("float64", "float32")):
    """Runs of the oracle and the GPU; returns time series, time-averaged
    spectra over t >= t_avg and pointwise errors against the oracle."""
    import torch
    from fluidsim_gb300.init_fields import noise_rot_2d
    from fluidsim_gb300.solvers import SimulNS2D
    from oracle.solvers import NS2DOracle
    from oracle.spectral import OperNumpy2D
    rot0 = noise_rot_2d(n, n, kmin=4.0, kmax=8.0, seed=seed, urms=1.0)
    samples = np.arange(0.0, t_end + 1e-9, every)

    def record(series, t, e_rot):
        """e_rot = 0.5 |rot_fft|^2 on the half spectrum (numpy, float64)"""
        series["t"].append(t)
        series["e_rot"].append(e_rot)

    def drive(step, get_t, get_erot):
        series = {"t": [], "e_rot": []}
        for ts in samples:
            while get_t() < ts - 1e-12:
                step()
            record(series, get_t(), get_erot())
        return series

    orc = NS2DOracle(OperNumpy2D(n, n), nu_2=nu_2, USE_CFL=True, cfl_coef=0.5,
                     deltat0=0.01, deltat_max=0.05)
    orc.init_from_rotfft(rot0)
    runs = {"oracle": drive(orc.one_time_step, lambda: orc.t,
                            lambda: 0.5 * np.abs(orc.state_spect[0]) ** 2)}
    finals = {"oracle": orc.state_spect[0].copy()}
    oper_np = orc.oper
    for prec in precisions:
        p = SimulNS2D.create_default_params()
        p.precision = prec
        p.oper.nx = p.oper.ny = n
        p.oper.Lx = p.oper.Ly = 2 * pi  # the ns2d default box is 8 x 8
        p.nu_2 = nu_2
        ts = p.time_stepping
        ts.USE_CFL, ts.cfl_coef, ts.deltat0, ts.deltat_max = True, 0.5, 0.01, 0.05
        ts.USE_T_END = False
        sim = SimulNS2D(p)
        sim.state.init_statespect_from(rot_fft=torch.from_numpy(rot0))
        runs[prec] = drive(
            sim.time_stepping.one_time_step, lambda: sim.time_stepping.t,
            lambda: (0.5 * sim.state.state_spect[0].to(torch.complex128).abs() ** 2)
            .cpu().numpy())
        finals[prec] = sim.state.state_spect[0].cpu().numpy().astype(np.complex128)
        del sim
        torch.cuda.empty_cache()

    inv_k2 = oper_np.inv_K_square_nozero
    k = min(oper_np.deltakx, oper_np.deltaky) * np.arange(10 ** 6)
    out = {"config": {"n": n, "nu_2": nu_2, "t_end": t_end, "t_avg": t_avg, "cfl": 0.5,
                      "init": f"noise_rot_2d k in [4, 8], urms 1, seed {seed}"}}
    kmax = None
    for name, s in runs.items():
        E = [oper_np.sum_wavenumbers(e * inv_k2) for e in s["e_rot"]]
        Z = [oper_np.sum_wavenumbers(e) for e in s["e_rot"]]
        keep = [i for i, t in enumerate(s["t"]) if t >= t_avg - 1e-12]
        Ek = np.mean([oper_np.compute_2dspectrum(s["e_rot"][i] * inv_k2) for i in keep], 0)
        Zk = np.mean([oper_np.compute_2dspectrum(s["e_rot"][i]) for i in keep], 0)
        kmax = (n // 3) if kmax is None else kmax
        out[name] = {"t": s["t"], "E": E, "Z": Z, "Ek": Ek.tolist(), "Zk": Zk.tolist(),
                     "Ek_bands": octave_bands(k[:len(Ek)], Ek, kmax).tolist(),
                     "Zk_bands": octave_bands(k[:len(Zk)], Zk, kmax).tolist()}
    ref = out["oracle"]
    for prec in precisions:
        r = out[prec]
        f, fo = finals[prec], finals["oracle"]
        r["pointwise_rel_l2_end"] = float(np.linalg.norm(f - fo) / np.linalg.norm(fo))
        r["E_max_rel_diff"] = float(np.max(np.abs(np.array(r["E"]) - ref["E"]) / ref["E"]))
        r["Z_max_rel_diff"] = float(np.max(np.abs(np.array(r["Z"]) - ref["Z"]) / ref["Z"]))
        r["Ek_bands_rel_diff"] = (np.abs(np.array(r["Ek_bands"]) - ref["Ek_bands"])
                                  / np.array(ref["Ek_bands"])).tolist()
        r["Zk_bands_rel_diff"] = (np.abs(np.array(r["Zk_bands"]) - ref["Zk_bands"])
                                  / np.array(ref["Zk_bands"])).tolist()
    return out


def test_long_run_spectra_match_oracle_after_decorrelation(cuda):
    """128^2, nu_2 = 5e-4, CFL 0.5, to t = 20 (about 4000 steps).  FP64 keeps
    pointwise parity with the oracle (round-off amplified by the chaos:
    ~2e-11 at t = 20); the FP32 run has decorrelated (~0.2 pointwise at
    t = 20) while E(t), Z(t) and the octave bands of the time-averaged E(k)
    and Z(k) over t in [10, 20] stay within 1e-4, 0.5 % and 0.5 % of the
    oracle's (measured on GB300; the bounds below leave a factor ~10)."""
    out = long_run_ns2d()
    r = out["float64"]
    assert r["pointwise_rel_l2_end"] < 1e-9, r["pointwise_rel_l2_end"]
    assert r["E_max_rel_diff"] < 1e-12 and r["Z_max_rel_diff"] < 1e-10
    assert max(r["Ek_bands_rel_diff"] + r["Zk_bands_rel_diff"]) < 1e-10
    r = out["float32"]
    assert r["pointwise_rel_l2_end"] > 0.05, r["pointwise_rel_l2_end"]  # decorrelated
    assert r["E_max_rel_diff"] < 1e-3, r["E_max_rel_diff"]
    assert r["Z_max_rel_diff"] < 0.02, r["Z_max_rel_diff"]
    assert max(r["Ek_bands_rel_diff"]) < 0.05, r["Ek_bands_rel_diff"]
    assert max(r["Zk_bands_rel_diff"]) < 0.05, r["Zk_bands_rel_diff"]
