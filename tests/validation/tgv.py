"""Taylor-Green vortex (256^3, nu = 1/1600, CFL 0.5): GPU against the oracle.

1. ``--oracle-steps`` first steps with CFL time steps: FP64 GPU state
   against the float64 CPU oracle (relative L2 per velocity component) and
   the two dt sequences;
2. FP64 and FP32 GPU runs to ``--t-end`` (``fluidsim_gb300.tgv``): the
   dissipation curve eps(t) and the FP32 state against FP64 at the end.

Prints one JSON line (with the clocks sampled during the GPU runs).

    python tests/validation/tgv.py [--n 256] [--t-end 10] [--oracle-steps 20]
"""
import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def main():
    import torch
    import bench
    from fluidsim_gb300.init_fields import taylor_green_3d
    from fluidsim_gb300.tgv import compare_precisions, make, rel_l2
    from oracle.solvers import NS3DOracle
    from oracle.spectral import OperNumpy3D
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--t-end", type=float, default=10.0)
    ap.add_argument("--oracle-steps", type=int, default=20)
    ap.add_argument("--every", type=int, default=10)
    a = ap.parse_args()
    n = a.n
    out = {"config": {"workload": f"Taylor-Green vortex {n}^3", "nu": 1 / 1600, "cfl": 0.5,
                      "t_end": a.t_end}}
    torch.cuda.set_device(0)

    orc = NS3DOracle(OperNumpy3D(n, n, n), nu_2=1 / 1600, USE_CFL=True, cfl_coef=0.5,
                     deltat0=0.2, deltat_max=0.2)
    orc.init_from_vxvyvzfft(*taylor_green_3d(n, n, n))
    dts_orc = []
    t0 = time.perf_counter()
    for _ in range(a.oracle_steps):
        orc.one_time_step()
        dts_orc.append(orc.deltat)
    cpu_s = (time.perf_counter() - t0) / a.oracle_steps

    with bench.ClockSampler(0) as clocks:
        sim = make(n, "float64")
        dts_gpu = []
        for _ in range(a.oracle_steps):
            sim.time_stepping.one_time_step()
            dts_gpu.append(sim.time_stepping.deltat)
        out["fp64_vs_oracle"] = {
            "steps": a.oracle_steps,
            "rel_l2": rel_l2(sim.state.state_spect.cpu().numpy(), orc.state_spect),
            "dt_max_rel_diff": float(np.max(np.abs(np.array(dts_gpu) - dts_orc)
                                            / np.array(dts_orc))),
            "oracle_s_per_step": cpu_s}
        del sim, orc
        torch.cuda.empty_cache()
        out.update(compare_precisions(n, a.t_end, a.every))
    out["clocks"] = clocks.summary()
    print(json.dumps(out), flush=True)
    return 0 if max(out["fp64_vs_oracle"]["rel_l2"]) <= 1e-12 else 1


if __name__ == "__main__":
    sys.exit(main())
