"""Long ns2d runs: GPU FP64 / FP32 against the float64 oracle, spectra.

Runs ``long_run_ns2d`` of ``tests/test_spectra_long_gpu.py`` (oracle, GPU
FP64 and FP32 from the same seeded band-passed vorticity, CFL 0.5) and prints
one JSON line: E(t), Z(t), pointwise error at the end, time-averaged E(k) and
Z(k) and their octave-band differences against the oracle.

    python tests/validation/spectra_long.py [--n 256] [--t-end 40] [--t-avg 20]
"""
import argparse
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))


def main():
    import torch
    import bench
    from test_spectra_long_gpu import long_run_ns2d
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--nu", type=float, default=2e-4)
    ap.add_argument("--t-end", type=float, default=40.0)
    ap.add_argument("--t-avg", type=float, default=20.0)
    ap.add_argument("--every", type=float, default=0.5)
    a = ap.parse_args()
    torch.cuda.set_device(0)
    with bench.ClockSampler(0) as clocks:
        out = long_run_ns2d(a.n, a.nu, a.t_end, a.t_avg, a.every)
    out["clocks"] = clocks.summary()
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
