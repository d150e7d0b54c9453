"""Helpers to read the golden fixtures written by ``golden/make_golden.py``."""
import math
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES_2D = ["ns2d_32_cfl", "ns2d_48x40_beta", "ns2d_256_c1", "ns2d_32_euler", "ns2d_40x32_rk2",
            "ns2d_32_rk2ps", "ns2d_36x32_eulerps", "ns2d_32_eulerpsr", "ns2d_40x32_rk2psr",
            "ns2d_strat_64x32", "ns2d_strat_64_rk2", "ns2d_bouss_64x32"]
CASES_3D = ["ns3d_20x15x10", "ns3d_tgv_32", "ns3d_iso_24x16x32_f", "ns3d_smag_20x24x16",
            "ns3d_rk2_20x15x10", "ns3d_heun_24x16x32_f", "ns3d_euler_tgv_32",
            "ns3d_rk2ps_20x15x10", "ns3d_rk2psx_16x24x32_f", "ns3d_eulerps_32",
            "ns3d_toroidal_24x20x16", "ns3d_poloidal_32_novz", "ns3d_strat_64x32x32",
            "ns3d_strat_64_f_rk2", "ns3d_rk2psr_24x16x32_f", "ns3d_eulerpsr_32",
            "ns3d_bouss_32x32x64"]
CASES_FORCING = ["ns3d_tcrandom_32", "ns3d_tcrandom_vx_24x32x16", "ns3d_random_32",
                 "ns3d_proportional_32"]
CASES_3D = CASES_3D + CASES_FORCING
FORCING_TYPES = {0: "tcrandom", 1: "random", 2: "proportional"}
KEY_NAMES = ("vx_fft", "vy_fft", "vz_fft")
PROJECTIONS = {0: None, 1: "toroidal", 2: "poloidal"}
SCHEME_NAMES = {0: "RK4", 1: "Euler", 2: "RK2", 3: "RK2_trapezoid", 4: "Euler_phaseshift",
                5: "RK2_phaseshift", 6: "RK2_phaseshift_exact", 7: "Euler_phaseshift_random",
                8: "RK2_phaseshift_random"}


def load(name):
    d = dict(np.load(GOLDEN / f"{name}.npz"))
    p = {k[2:]: float(v) for k, v in d.items() if k.startswith("p_")}
    for k in list(p):
        if math.isnan(p[k]):
            p[k] = None
    return d, p


def scheme(p):
    """type_time_scheme of a fixture (RK4 when it records none)."""
    return SCHEME_NAMES[int(p["scheme"])] if p.get("scheme") is not None else "RK4"


def projection_kwargs(p):
    """params.projection / no_vz_kz0 of an ns3d fixture."""
    return {"projection": PROJECTIONS[int(p.get("projection") or 0)],
            "no_vz_kz0": bool(p.get("no_vz_kz0") or 0)}


def solver_kwargs(p):
    kw = {"type_time_scheme": scheme(p)}
    for k in ("nu_2", "nu_4", "nu_8", "nu_m4", "deltat0", "deltat_max", "cfl_coef"):
        if p.get(k) is not None:
            kw[k] = p[k]
    kw["USE_CFL"] = bool(p.get("USE_CFL"))
    return kw


def lengths(p, ndim):
    keys = ("Lx", "Ly", "Lz")[:ndim]
    return tuple(p.get(k) if p.get(k) is not None else 2 * math.pi for k in keys)


def forcing_config(p):
    """(type, keys, nkmin, nkmax, rate, time_correlation, np_seed) of a forcing
    fixture, or None."""
    if p.get("forcing_type") is None:
        return None
    bits = int(p["forced_keys"])
    keys = [k for i, k in enumerate(KEY_NAMES) if bits & (1 << i)]
    tc = p.get("time_correlation")
    return {"type": FORCING_TYPES[int(p["forcing_type"])], "key_forced": keys,
            "nkmin_forcing": p["nkmin_forcing"], "nkmax_forcing": p["nkmax_forcing"],
            "forcing_rate": p["forcing_rate"],
            "time_correlation": "based_on_forcing_rate" if tc is None else tc,
            "np_seed": int(p["np_seed"])}
