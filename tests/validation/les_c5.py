"""Config C5: the learned subgrid closure, end to end, with the clocks.

Runs ``fluidsim_gb300.les.pipeline`` (forced 512^3 FP32 DNS, box-filtered
snapshots on the 128^3 LES grid, training with the project's tensor-core
forward/backward kernels, 2000-step LES with no model, Smagorinsky and the
learned closure) and prints one JSON line with the clocks sampled during
the run.

    python tests/validation/les_c5.py [--n-dns 512] [--n-les 128]
"""
import argparse
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def main():
    import torch
    import bench
    from fluidsim_gb300 import les
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-dns", type=int, default=512)
    ap.add_argument("--n-les", type=int, default=128)
    ap.add_argument("--train-steps", type=int, default=3000)
    ap.add_argument("--les-steps", type=int, default=2000)
    a = ap.parse_args()
    torch.cuda.set_device(0)
    with bench.ClockSampler(0) as clocks:
        out = les.pipeline(a.n_dns, a.n_les, nu=3e-4, t_coarse=6.0, t_fine=1.5, n_snap=4,
                           t_between=0.25, train_steps=a.train_steps, les_steps=a.les_steps,
                           lambda_pi=1.0)
    out["clocks"] = clocks.summary()
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
