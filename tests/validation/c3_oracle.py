"""ns3d 512^3 benchmark workload: GPU FP64 / FP32 against the FP64 oracle.

The workload of ``bench.py`` (seeded solenoidal random phases,
E(k) ~ k^4 exp(-2 (k/4)^2), E = 0.5, nu_2 = 5e-4, IF-RK4, dt fixed by the
CFL rule with coefficient 0.5, 2/3 dealiasing) run for ``--steps`` steps
three times: float64 CPU oracle (scipy.fft and slab-parallel numpy on all
host cores), GPU FP64 and GPU FP32.  Prints one JSON line with the relative
L2 error of each GPU state variable against the oracle.

    python tests/validation/c3_oracle.py [--n 512] [--steps 10]
"""
import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def rel_l2(a, b):
    return [float(np.linalg.norm(a[i] - b[i]) / np.linalg.norm(b[i])) for i in range(len(b))]


def main():
    import torch
    import bench
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--steps", type=int, default=10)
    a = ap.parse_args()
    n = a.n
    v0 = bench.initial_state(n)
    dt = bench.initial_dt(v0, n)
    out = {"config": bench.workload_config(n, n, n, dt, 1), "steps": a.steps}

    t0 = time.perf_counter()
    orc = bench.oracle_sim(n, v0, dt)
    for _ in range(a.steps):
        orc.one_time_step()
    out["oracle_s_per_step"] = (time.perf_counter() - t0) / a.steps
    ref = orc.state_spect.copy()
    out["oracle_E"] = orc.compute_energy()
    del orc

    torch.cuda.set_device(0)
    with bench.ClockSampler(0) as clocks:
        for prec in ("float64", "float32"):
            sim = bench.make_sim(n, prec, v0)
            sim.time_stepping.deltat = dt
            for _ in range(a.steps):
                sim.time_stepping.one_time_step()
            got = sim.state.state_spect.cpu().numpy().astype(np.complex128)
            out[prec] = {"rel_l2_vs_oracle": rel_l2(got, ref),
                         "E": sim.output.compute_spatial_means()["E"]}
            del sim
            torch.cuda.empty_cache()
    out["clocks"] = clocks.summary()
    out["fp64_max_rel_l2"] = max(out["float64"]["rel_l2_vs_oracle"])
    out["fp32_max_rel_l2"] = max(out["float32"]["rel_l2_vs_oracle"])
    out["pass"] = out["fp64_max_rel_l2"] <= 1e-12 and out["fp32_max_rel_l2"] <= 1e-5
    print(json.dumps(out), flush=True)
    return 0 if out["pass"] else 1


if __name__ == "__main__":
    sys.exit(main())
