"""Taylor-Green vortex runs on the GPU: FP64 and FP32 to t_end.

Configuration: 256^3 periodic box L = 2 pi, u = sin x cos y cos z,
v = -cos x sin y cos z, w = 0 (``doc/test_cases/Taylor_Green_vortices/
run_simul.py:40-54``), nu = 1/1600, RK4 with exact integrating factor, CFL
0.5, 2/3 dealiasing, run to t = 10.

FP64 and FP32 GPU runs to ``t_end``: dissipation rate
eps(t) = sum 2 nu k^2 E(k) (FP64 reductions) every ``every`` steps, and the
FP32 state's relative L2 against FP64 at the end.

``python -m fluidsim_gb300.tgv`` prints one JSON line.
"""

import argparse
import json
import time

import numpy as np
import torch

from .init_fields import taylor_green_3d
from .solvers import SimulNS3D


def make(n, precision, nu=1.0 / 1600, cfl=0.5):
    p = SimulNS3D.create_default_params()
    p.precision = precision
    p.oper.nx = p.oper.ny = p.oper.nz = n
    p.nu_2 = nu
    ts = p.time_stepping
    ts.USE_CFL, ts.cfl_coef, ts.deltat0, ts.deltat_max = True, cfl, 0.2, 0.2
    sim = SimulNS3D(p)
    v0 = taylor_green_3d(n, n, n)
    sim.init_from_vxvyvzfft(*v0)
    return sim


def rel_l2(a, b):
    return [float(np.linalg.norm(a[i] - b[i]) / np.linalg.norm(b[i])) for i in range(len(b))
            if np.linalg.norm(b[i]) > 0]


def run_curve(sim, t_end, every):
    ts = sim.time_stepping
    curve = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    while ts.t < t_end:
        if ts.it % every == 0:
            m = sim.output.compute_spatial_means()
            curve.append((ts.t, m["E"], m["epsK"]))
        ts.one_time_step()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    m = sim.output.compute_spatial_means()
    curve.append((ts.t, m["E"], m["epsK"]))
    return np.array(curve), wall


def compare_precisions(n, t_end, every):
    """FP64 and FP32 runs to ``t_end``: their eps(t) curves and the FP32
    state's relative L2 against FP64 at the end."""
    out = {}
    curves = {}
    finals = {}
    for prec in ("float64", "float32"):
        sim = make(n, prec)
        curve, wall = run_curve(sim, t_end, every)
        curves[prec] = curve
        finals[prec] = sim.state.state_spect.cpu().numpy().astype(np.complex128)
        out[prec] = {"steps": sim.time_stepping.it, "wall_s": wall,
                     "steps_per_s": sim.time_stepping.it / wall, "t": sim.time_stepping.t}
        del sim
        torch.cuda.empty_cache()
    c64, c32 = curves["float64"], curves["float32"]
    m = min(len(c64), len(c32))
    eps64, eps32 = c64[:m, 2], c32[:m, 2]
    out["fp32_vs_fp64"] = {
        "rel_l2_final": rel_l2(finals["float32"], finals["float64"]),
        "eps_max_rel_diff": float(np.max(np.abs(eps32 - eps64)) / np.max(np.abs(eps64))),
        "eps_peak_fp64": float(eps64.max()), "t_eps_peak_fp64": float(c64[np.argmax(eps64), 0]),
        "eps_peak_fp32": float(eps32.max()), "t_eps_peak_fp32": float(c32[np.argmax(eps32), 0]),
    }
    out["eps_curve_fp64"] = c64[:, [0, 2]].round(8).tolist()
    out["eps_curve_fp32"] = c32[:, [0, 2]].round(8).tolist()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--t-end", type=float, default=10.0)
    ap.add_argument("--every", type=int, default=10)
    a = ap.parse_args()
    out = {"config": {"workload": f"Taylor-Green vortex {a.n}^3", "nu": 1 / 1600, "cfl": 0.5,
                      "t_end": a.t_end}}
    out.update(compare_precisions(a.n, a.t_end, a.every))
    print(json.dumps(out))


if __name__ == "__main__":
    main()
