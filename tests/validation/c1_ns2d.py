"""Config C1: ns2d 256^2, band-passed noise, 200 IF-RK4 steps: GPU against the oracle.

Doubly periodic box 2 pi x 2 pi, float64, initial vorticity Gaussian white
noise (seeded) band-passed to k in [4, 8] and scaled to rms velocity 1,
nu_2 = 1e-4, fixed dt = 1e-3, 2/3 dealiasing, 200 steps.  Runs the FP64 and
FP32 GPU solvers and the float64 CPU oracle from the same field, records
the energy and enstrophy time series of each and compares the final
vorticity fields.  Prints one JSON line (with the clocks sampled during the
GPU runs).

    python tests/validation/c1_ns2d.py [--n 256] [--steps 200]
"""
import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def gpu_run(n, precision, rot0, steps, nu):
    import torch
    from fluidsim_gb300.solvers import SimulNS2D
    p = SimulNS2D.create_default_params()
    p.precision = precision
    p.oper.nx = p.oper.ny = n
    p.oper.Lx = p.oper.Ly = 2 * np.pi  # (the ns2d default box is 8 x 8)
    p.nu_2 = nu
    ts = p.time_stepping
    ts.USE_CFL, ts.deltat0, ts.USE_T_END, ts.it_end = False, 1e-3, False, steps
    sim = SimulNS2D(p)
    sim.state.init_statespect_from(rot_fft=rot0)
    series = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        m = sim.output.compute_spatial_means()
        series.append((m["E"], m["Z"]))
        sim.time_stepping.one_time_step()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    m = sim.output.compute_spatial_means()
    series.append((m["E"], m["Z"]))
    rot = sim.state.state_spect[0].cpu().numpy().astype(np.complex128)
    # step rate without the per-step means (steps past the compared ones)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        sim.time_stepping.one_time_step()
    torch.cuda.synchronize()
    rate = steps / (time.perf_counter() - t0)
    return rot, np.array(series), wall, rate


def main():
    import torch
    import bench
    from fluidsim_gb300.init_fields import noise_rot_2d
    from oracle.solvers import NS2DOracle
    from oracle.spectral import OperNumpy2D
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--steps", type=int, default=200)
    a = ap.parse_args()
    n, steps, nu = a.n, a.steps, 1e-4
    rot0 = noise_rot_2d(n, n, kmin=4.0, kmax=8.0, seed=0, urms=1.0)
    out = {"config": {"workload": f"ns2d {n}^2 band-passed noise k in [4, 8], urms 1",
                      "nu_2": nu, "dt": 1e-3, "steps": steps, "scheme": "RK4 exact IF"}}

    orc = NS2DOracle(OperNumpy2D(n, n), nu_2=nu, USE_CFL=False, deltat0=1e-3)
    orc.init_from_rotfft(rot0)
    s_orc = []
    t0 = time.perf_counter()
    for _ in range(steps):
        s_orc.append((orc.compute_energy(), orc.compute_enstrophy()))
        orc.one_time_step()
    cpu_s = time.perf_counter() - t0
    s_orc.append((orc.compute_energy(), orc.compute_enstrophy()))
    s_orc = np.array(s_orc)
    ref = orc.state_spect[0]

    torch.cuda.set_device(0)
    with bench.ClockSampler(0) as clocks:
        r64, s64, w64, rate64 = gpu_run(n, "float64", rot0, steps, nu)
        r32, s32, w32, rate32 = gpu_run(n, "float32", rot0, steps, nu)

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    def series_err(s):
        return {"E": float(np.max(np.abs(s[:, 0] - s_orc[:, 0]) / s_orc[:, 0])),
                "Z": float(np.max(np.abs(s[:, 1] - s_orc[:, 1]) / s_orc[:, 1]))}

    out["oracle"] = {"s_per_step": cpu_s / steps, "E0": float(s_orc[0, 0]),
                     "E_end": float(s_orc[-1, 0]), "Z0": float(s_orc[0, 1]),
                     "Z_end": float(s_orc[-1, 1])}
    out["fp64"] = {"rel_l2_rot": rel(r64, ref), "series_max_rel_err": series_err(s64),
                   "steps_per_s": rate64}
    out["fp32"] = {"rel_l2_rot": rel(r32, ref), "series_max_rel_err": series_err(s32),
                   "steps_per_s": rate32}
    out["clocks"] = clocks.summary()
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
