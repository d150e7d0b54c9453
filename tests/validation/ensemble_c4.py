"""Config C4: the batched ns2d ensemble against individually solved oracle runs.

96 runs (32 each at 128^2, 256^2, 512^2), float32, seeded noise vorticity in
k in [3, 10], nu_2 log-uniform in [1e-5, 1e-3], nu_8 = 2 dx^8, 500 IF-RK4
steps replayed from CUDA graphs in the mode the autotuner picks
(``fluidsim_gb300.ensemble.benchmark``).  Then ``--check`` runs of each size
are solved alone by the float64 CPU oracle (same initial field, viscosities
and dt) and compared with the ensemble's final states.  Prints one JSON line.

    python tests/validation/ensemble_c4.py [--steps 500] [--check 2]
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
    from fluidsim_gb300.ensemble import EnsembleNS2D, make_group
    from oracle.solvers import NS2DOracle
    from oracle.spectral import OperNumpy2D
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--runs-per-size", type=int, default=32)
    ap.add_argument("--check", type=int, default=2)
    a = ap.parse_args()
    torch.cuda.set_device(0)
    sizes = (128, 256, 512)
    groups = [make_group(n, a.runs_per_size, k) for k, n in enumerate(sizes)]
    ens = EnsembleNS2D(groups)
    tuning = ens.autotune()
    ens.capture(10)
    ens.reset()
    ens.run(10)
    ens.reset()
    with bench.ClockSampler(0) as clocks:
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ens.run(a.steps)
        e1.record()
        torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1000
    nruns = a.runs_per_size * len(sizes)
    out = {"workload": f"{nruns} ns2d runs ({a.runs_per_size} each at 128^2, 256^2, 512^2), "
                       f"float32, {a.steps} RK4 steps",
           "runs_per_s": nruns / sec, "seconds": sec, "tuning": tuning,
           "nan": ens.nan_flag(), "clocks": clocks.summary(), "vs_oracle": {}}
    for gi, g in enumerate(groups):
        got = ens.groups[gi]["S"].cpu().numpy()
        n, L = g["n"], g["L"]
        errs, secs = [], []
        for i in range(a.check):
            orc = NS2DOracle(OperNumpy2D(n, n, L, L), nu_2=float(g["nu2"][i]),
                             nu_8=float(g["nu8"][i]), deltat0=float(g["dt"][i]))
            orc.init_from_rotfft(g["rot0"][i])
            t0 = time.perf_counter()
            orc.run(it_end=a.steps)
            secs.append(time.perf_counter() - t0)
            ref = orc.state_spect[0]
            errs.append(float(np.linalg.norm(got[i] - ref) / np.linalg.norm(ref)))
        out["vs_oracle"][n] = {"runs_checked": a.check, "rel_l2": errs,
                               "oracle_s_per_run": float(np.mean(secs))}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
