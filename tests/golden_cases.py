"""Helpers to read the golden fixtures written by ``golden/make_golden.py``."""
import math
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES_2D = ["ns2d_32_cfl", "ns2d_48x40_beta", "ns2d_256_c1"]
CASES_3D = ["ns3d_20x15x10", "ns3d_tgv_32", "ns3d_iso_24x16x32_f", "ns3d_smag_20x24x16"]


def load(name):
    d = dict(np.load(GOLDEN / f"{name}.npz"))
    p = {k[2:]: float(v) for k, v in d.items() if k.startswith("p_")}
    for k in list(p):
        if math.isnan(p[k]):
            p[k] = None
    return d, p


def solver_kwargs(p):
    kw = {}
    for k in ("nu_2", "nu_4", "nu_8", "nu_m4", "deltat0", "deltat_max", "cfl_coef"):
        if p.get(k) is not None:
            kw[k] = p[k]
    kw["USE_CFL"] = bool(p.get("USE_CFL"))
    return kw


def lengths(p, ndim):
    keys = ("Lx", "Ly", "Lz")[:ndim]
    return tuple(p.get(k) if p.get(k) is not None else 2 * math.pi for k in keys)
