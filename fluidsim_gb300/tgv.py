"""Taylor-Green vortex: FP64 GPU vs the FP64 CPU oracle, FP32 vs FP64 on GPU.

Configuration: 256^3 periodic box L = 2 pi, u = sin x cos y cos z,
v = -cos x sin y cos z, w = 0 (``doc/test_cases/Taylor_Green_vortices/
run_simul.py:40-54``), nu = 1/1600, RK4 with exact integrating factor, CFL
0.5, 2/3 dealiasing, run to t = 10.

* ``oracle_steps`` first steps: FP64 GPU state against the FP64 CPU oracle
  (relative L2 per velocity component), same time steps;
* FP64 and FP32 GPU runs to ``t_end``: dissipation rate
  eps(t) = sum 2 nu k^2 E(k) (FP64 reductions) every ``every`` steps, and
  the FP32 state's relative L2 against FP64 at the end.

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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--t-end", type=float, default=10.0)
    ap.add_argument("--oracle-steps", type=int, default=20)
    ap.add_argument("--every", type=int, default=10)
    a = ap.parse_args()
    n = a.n
    out = {"config": {"workload": f"Taylor-Green vortex {n}^3", "nu": 1 / 1600, "cfl": 0.5,
                      "t_end": a.t_end}}

    # 1. FP64 GPU vs FP64 CPU oracle over the first steps
    from oracle.solvers import NS3DOracle
    from oracle.spectral import OperNumpy3D
    sim = make(n, "float64")
    orc = NS3DOracle(OperNumpy3D(n, n, n), nu_2=1 / 1600, USE_CFL=True, cfl_coef=0.5,
                     deltat0=0.2, deltat_max=0.2)
    v0 = taylor_green_3d(n, n, n)
    orc.init_from_vxvyvzfft(*v0)
    t0 = time.perf_counter()
    for _ in range(a.oracle_steps):
        orc.one_time_step()
    cpu_s = (time.perf_counter() - t0) / a.oracle_steps
    for _ in range(a.oracle_steps):
        sim.time_stepping.one_time_step()
    out["fp64_vs_oracle"] = {"steps": a.oracle_steps,
                             "rel_l2": rel_l2(sim.state.state_spect.cpu().numpy(),
                                              orc.state_spect),
                             "dt_gpu": sim.time_stepping.deltat, "dt_oracle": orc.deltat,
                             "oracle_s_per_step": cpu_s}
    del sim, orc

    # 2. FP64 and FP32 GPU runs to t_end with the dissipation curve
    curves = {}
    finals = {}
    for prec in ("float64", "float32"):
        sim = make(n, prec)
        curve, wall = run_curve(sim, a.t_end, a.every)
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
    print(json.dumps(out))


if __name__ == "__main__":
    main()
