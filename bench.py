"""Benchmark: ns3d 512^3 IF-RK4 steps/s on GB300 (FP32, with FP64 beside it).

Workload (decaying isotropic turbulence): 512^3 periodic box L = 2 pi,
seeded solenoidal random-phase velocity with E(k) ~ k^4 exp(-2 (k/4)^2),
total energy 0.5, nu_2 = 5e-4, RK4 with exact integrating factor, 2/3
dealiasing, dt fixed once from the CFL rule with coefficient 0.5.  A step is
one full RK4 step (4 tendency evaluations + projection + dealiasing + NaN
check).  The working set (~10 GB in FP32) is far larger than the 129 MB L2,
so no explicit L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Under torchrun (N > 1) each rank runs an independent replica on its own GPU
(one simulation per GPU: no data-path exchange); value = steps of all ranks
divided by the slowest rank's time.  The reference arm times whole RK4
steps of the CPU restatement of the reference algorithm (float64, scipy.fft
and slab-parallel numpy on all host cores) on the same workload, honouring
--steps and --warmup.
"""

import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time
from math import pi
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "ns3d 512^3 RK4 steps/s"
KINDS = ("inv_z_curl", "inv_y", "x_product", "fwd_y", "fwd_z_rk")


def fields_per_launch(nx, ny, nz, coef=2.0 / 3):
    """Algorithmic HBM traffic per launch of each pass of a pruned step, in
    units of one spectral field (nz*ny*(nx/2+1) complex): what the pass must
    read and write given the 2/3 truncation (kept fractions fx, fy, fz)."""
    from fluidsim_gb300.init_fields import cubic_dealias_cutoff
    nkx = nx // 2 + 1
    fx = min(cubic_dealias_cutoff(nx, 2 * pi, coef), nkx) / nkx
    cy = cubic_dealias_cutoff(ny, 2 * pi, coef)
    cz = cubic_dealias_cutoff(nz, 2 * pi, coef)
    fy = min(2 * cy - 1, ny) / ny
    fz = min(2 * cz - 1, nz) / nz
    # stage average of the RK state traffic: reads+writes of S, tmp, tmp1
    rk_state = ((3 + 6) + (6 + 6) + (6 + 6) + (3 + 3)) / 4
    return {"inv_z_curl": 3 * fx * fy * fz + 6 * fx * fy,
            "inv_y": 6 * fx * fy + 6 * fx,
            "x_product": 6 * fx + 3 * fx,
            "fwd_y": 3 * fx + 3 * fx * fy,
            "fwd_z_rk": 3 * fx * fy + rk_state * fx * fy * fz}


def fp64_flops_per_step(nx, ny, nz, coef=2.0 / 3):
    """Floating-point operations of the FFT butterflies of one pruned RK4
    step (4 tendency evaluations), counting 5 n log2 n per complex n-point
    line and 2.5 n log2 n per real line, over the lines each pass actually
    transforms given the 2/3 truncation: per evaluation 5 inverse and 3
    forward z transforms on the kept (kx, ky) columns, 6 inverse and 3
    forward y transforms on the kept kx columns, 6 C2R and 3 R2C x rows."""
    from math import log2
    from fluidsim_gb300.init_fields import cubic_dealias_cutoff
    kx = min(cubic_dealias_cutoff(nx, 2 * pi, coef), nx // 2 + 1)
    ky = min(2 * cubic_dealias_cutoff(ny, 2 * pi, coef) - 1, ny)
    z_lines, y_lines, x_lines = kx * ky, kx * nz, ny * nz
    per_eval = ((5 + 3) * z_lines * 5 * nz * log2(nz)
                + (6 + 3) * y_lines * 5 * ny * log2(ny)
                + (6 + 3) * x_lines * 2.5 * nx * log2(nx))
    return 4 * per_eval


def fp64_peak_tflops(sm_mhz, sms=152):
    """FP64 FMA peak: 2 FP64 FMA (4 flops) per clock per SM."""
    return sms * 4 * sm_mhz * 1e6 / 1e12


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 100; 20 for --impl reference)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--ny", type=int, default=None, help="override ny (profiling cases)")
    ap.add_argument("--nz", type=int, default=None, help="override nz (profiling cases)")
    ap.add_argument("--no-fft", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    return ap.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def replica_rate(elapsed_ms, steps, world, dist=None, device="cpu"):
    """Whole-job steps/s of ``world`` independent replicas that each ran
    ``steps`` steps: all ranks' steps over the slowest rank's time (max over
    ranks through ``dist``).  Returns (steps/s, slowest elapsed ms)."""
    if dist is not None and world > 1:
        import torch
        t = torch.tensor([float(elapsed_ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
    return world * steps / (elapsed_ms / 1000.0), elapsed_ms


def initial_state(n, ny=None, nz=None):
    from fluidsim_gb300.init_fields import isotropic_3d
    ny, nz = ny or n, nz or n
    return isotropic_3d(n, ny, nz, 2 * pi, 2 * pi * ny / n, 2 * pi * nz / n,
                        k0=4.0, energy=0.5, seed=0)


def cfl_dt(vmax, n, cfl=0.5, dtmax=0.2):
    """dt from the CFL rule of fluidsim/base/time_stepping/base.py:320-354."""
    dx = 2 * pi / n
    tmp = sum(v / dx for v in vmax)
    return min(cfl / tmp, dtmax) if tmp > 0 else dtmax


def initial_dt(v0, n):
    """The workload's fixed dt: the CFL rule (coefficient 0.5) applied once
    to the initial field, with max|v_i| taken in float64 on the host, so both
    arms step with the same dt."""
    import scipy.fft as sfft
    nz, ny = v0.shape[1], v0.shape[2]
    shape = (nz, ny, n)
    vmax = []
    for c in range(3):
        x = sfft.irfftn(v0[c], s=shape, workers=os.cpu_count()) * (n * ny * nz)
        vmax.append(float(max(abs(x.min()), abs(x.max()))))
    return cfl_dt(vmax, n)


def workload_config(n, ny, nz, dt, world):
    size = f"{n}^3" if n == ny == nz else f"{n}x{ny}x{nz}"
    return {"workload": f"ns3d decaying isotropic turbulence {size}", "nx": n,
            "ny": ny, "nz": nz, "L": "2pi", "nu_2": 5e-4, "dt": dt,
            "scheme": "RK4 exact integrating factor", "dealiasing": "2/3 cubic",
            "initial": "seeded solenoidal random phases, E(k)~k^4 exp(-2(k/4)^2), E=0.5",
            "l2_flush": "none needed: working set ~10 GB >> 129 MB L2",
            "parallelism": f"replicas x{world}"}


def make_sim(n, precision, v0):
    import torch
    from fluidsim_gb300.solvers import SimulNS3D
    p = SimulNS3D.create_default_params()
    p.precision = precision
    nz, ny = v0.shape[1], v0.shape[2]
    p.oper.nx, p.oper.ny, p.oper.nz = n, ny, nz
    p.oper.Ly, p.oper.Lz = 2 * pi * ny / n, 2 * pi * nz / n
    p.nu_2 = 5e-4
    p.time_stepping.USE_CFL = False
    p.time_stepping.USE_T_END = False
    sim = SimulNS3D(p)
    sim.state.init_statespect_from(**{k: torch.from_numpy(v0[i]) for i, k in
                                      enumerate(sim.state.keys_state_spect)})
    return sim


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for name, val in zip(names, r[5:9]):
                if val.strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kind, n):
    """dram read+write bytes per launch from the committed ncu summary."""
    f = ROOT / "profiles" / "ncu_traffic.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        parts = line.split()
        if len(parts) >= 3 and parts[0] == kind and parts[1] == f"{n}^3":
            return float(parts[2])
    return None


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the
    platform string)."""
    import platform
    import subprocess
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                key = line.split(":")[0].strip().lower()
                if key in ("model name", "cpu part", "hardware"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def oracle_sim(n, v0, dt):
    """The float64 CPU oracle set up on the workload (untimed)."""
    from oracle.solvers import NS3DOracle
    from oracle.spectral import OperNumpy3D
    orc = NS3DOracle(OperNumpy3D(n, n, n), nu_2=5e-4, deltat0=dt, USE_CFL=False)
    orc.state_spect[:] = v0
    orc.statephys_from_statespect()
    orc._coefs()  # exp(-dt sigma) tables, computed once per dt
    return orc


def cpu_sample(n, v0, dt, steps=1):
    """Oracle (float64, scipy.fft and slab-parallel numpy on all host cores):
    ``steps`` whole RK4 steps (4 tendency evaluations, the stage updates,
    projection, dealiasing, the inverse transforms of the state, NaN check)."""
    from oracle.spectral import WORKERS
    orc = oracle_sim(n, v0, dt)
    t0 = time.perf_counter()
    for _ in range(steps):
        orc.one_time_step()
    el = time.perf_counter() - t0
    return {"value": steps / el, "unit": "steps/s", "cores": WORKERS, "kind": "port",
            "cpu_model": cpu_model(),
            "sample": (f"{steps} whole RK4 step(s) of the float64 oracle at {n}^3 "
                       f"(one_time_step: 4 tendency evaluations, stage updates, "
                       f"projection, dealiasing, state_phys, NaN check), "
                       f"{el / steps:.2f} s each")}


def run_reference(args):
    """Reference arm: the CPU restatement of the reference's algorithm,
    whole RK4 steps on the same workload, ``--warmup`` untimed then exactly
    ``--steps`` timed (the method of fluidsim/util/console/util.py:329-390:
    fixed dt, it_end steps, outputs off)."""
    rank, _, world = dist_env()
    if rank != 0:
        return
    from oracle.spectral import WORKERS
    n = args.n
    steps = args.steps if args.steps is not None else 20
    v0 = initial_state(n)
    dt = initial_dt(v0, n)
    orc = oracle_sim(n, v0, dt)
    for _ in range(args.warmup):
        orc.one_time_step()
    t0 = time.perf_counter()
    for _ in range(steps):
        orc.one_time_step()
    el = time.perf_counter() - t0
    value = steps / el
    base = {"value": value, "unit": "steps/s", "cores": WORKERS, "kind": "port",
            "cpu_model": cpu_model(),
            "sample": (f"{steps} timed whole RK4 steps after {args.warmup} warm-up steps "
                       f"of the float64 oracle at {n}^3, {el / steps:.2f} s each")}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "steps/s",
            "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * el / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(n, n, n, dt, world),
            "cpu_baseline": base,
            "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def e2e_run(ts, S, host_in, host_out, steps, world, dist, pipelined):
    """Steps through the public API with host buffers: each step's input
    state is copied from pinned host memory and its result copied back.

    serial: H2D, step, D2H on one stream.  pipelined: three device state
    buffers in rotation (``state.set_state_spect``): the H2D of the next
    step's input into one and the D2H of the previous step's result from
    another run on their own streams while the current step computes on the
    third.  The timed region includes the first input's H2D and the last
    result's D2H, which nothing overlaps.  Leaves the simulation on S."""
    import torch
    state = ts.sim.state
    cs = torch.cuda.current_stream()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if not pipelined:
        e0.record()
        for _ in range(steps):
            S.copy_(host_in, non_blocking=True)
            ts.one_time_step()
            host_out.copy_(S, non_blocking=True)
        e1.record()
    else:
        h2d, d2h = torch.cuda.Stream(), torch.cuda.Stream()
        bufs = [S, torch.empty_like(S), torch.empty_like(S)]
        staged = [torch.cuda.Event() for _ in range(steps)]
        copied = [torch.cuda.Event() for _ in range(steps)]
        e0.record()
        h2d.wait_stream(cs)
        with torch.cuda.stream(h2d):
            bufs[0].copy_(host_in, non_blocking=True)
            staged[0].record()
        for i in range(steps):
            cur = bufs[i % 3]
            if i + 1 < steps:  # input i + 1 into the buffer result i - 2 has left
                if i >= 2:
                    h2d.wait_event(copied[i - 2])
                with torch.cuda.stream(h2d):
                    bufs[(i + 1) % 3].copy_(host_in, non_blocking=True)
                    staged[i + 1].record()
            cs.wait_event(staged[i])
            state.set_state_spect(cur)
            ts.one_time_step()
            d2h.wait_stream(cs)
            with torch.cuda.stream(d2h):
                host_out.copy_(cur, non_blocking=True)
                copied[i].record()
        cs.wait_stream(d2h)
        e1.record()
        torch.cuda.synchronize()
        S.copy_(state.state_spect)
        state.set_state_spect(S)
    torch.cuda.synchronize()
    rate, _ = replica_rate(e0.elapsed_time(e1), steps, world, dist, "cuda")
    return rate


def fft_throughput(n, reps=20):
    """FP32 512^3 R2C + C2R through the plugin class (HBM GB/s), cuFFT beside it."""
    import torch
    from fluidsim_gb300 import FFT3DGB300
    op = FFT3DGB300(n, n, n, precision="float32")
    x = torch.randn((n, n, n), dtype=torch.float32, device="cuda")
    k = op.create_arrayK()
    x2 = torch.empty_like(x)
    for _ in range(3):
        op.fft_as_arg(x, k)
        op.ifft_as_arg(k, x2)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    torch.cuda.synchronize()
    ev[0].record()
    for _ in range(reps):
        op.fft_as_arg(x, k)
    ev[1].record()
    for _ in range(reps):
        op.ifft_as_arg(k, x2)
    ev[2].record()
    torch.cuda.synchronize()
    r2c_ms = ev[0].elapsed_time(ev[1]) / reps
    c2r_ms = ev[1].elapsed_time(ev[2]) / reps
    sr = x.numel() * 4
    sk = k.numel() * 8
    # x pass reads S_r writes S_k; y and z passes read and write S_k
    alg = sr + 5 * sk
    out = {"r2c_ms": r2c_ms, "c2r_ms": c2r_ms,
           "r2c_hbm_gbs": alg / r2c_ms / 1e6, "c2r_hbm_gbs": alg / c2r_ms / 1e6,
           "alg_bytes_per_transform": alg}
    # comparison only: cuFFT through torch (not part of the product); both
    # directions warmed up (plan creation) before either is timed
    for _ in range(3):
        torch.fft.rfftn(x)
        torch.fft.irfftn(k, s=x.shape)
    torch.cuda.synchronize()
    ev[0].record()
    for _ in range(reps):
        torch.fft.rfftn(x)
    ev[1].record()
    torch.cuda.synchronize()
    ev[2].record()
    for _ in range(reps):
        torch.fft.irfftn(k, s=x.shape)
    ev[3].record()
    torch.cuda.synchronize()
    out["cufft_compare"] = {"rfftn_ms": ev[0].elapsed_time(ev[1]) / reps,
                            "irfftn_ms": ev[2].elapsed_time(ev[3]) / reps}
    return out


MLP_FLOPS_PER_POINT = 2 * (9 * 64 + 64 * 64 + 64 * 6)  # 9 -> 64 -> 64 -> 6 network


def mlp_throughput(n_points=128**3, reps=20):
    """The learned closure's 9 -> 64 -> 64 -> 6 network (BF16 tensor-core
    MMAs, FP32 accumulation) on n_points gradient tensors through
    gbs_mlp_forward, the evaluation the 128^3 LES runs four times a step."""
    import torch
    from fluidsim_gb300.closure import ClosureMLP, predict
    net = ClosureMLP(seed=0)
    G = torch.randn((9, n_points), dtype=torch.float32, device="cuda")
    for _ in range(3):
        predict(net, G)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    torch.cuda.synchronize()
    ev[0].record()
    for _ in range(reps):
        predict(net, G)
    ev[1].record()
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[1]) / reps
    for _ in range(3):
        predict(net, G, precision="bf16")
    torch.cuda.synchronize()
    ev[0].record()
    for _ in range(reps):
        predict(net, G, precision="bf16")
    ev[1].record()
    torch.cuda.synchronize()
    ms_bf16 = ev[0].elapsed_time(ev[1]) / reps
    # one training gradient (forward + backward on the tensor cores, then the
    # weight-gradient reduction) of a 65536-sample batch
    from fluidsim_gb300.closure import ClosureTrainer
    batch = 65536
    tr = ClosureTrainer(net, batch=batch)
    Tau = torch.randn((6, n_points), dtype=torch.float32, device="cuda")
    idx = torch.randint(0, n_points, (batch,), device="cuda", dtype=torch.int64)
    for _ in range(3):
        tr.gradient(G, Tau, idx)
    torch.cuda.synchronize()
    ev[0].record()
    for _ in range(reps):
        tr.gradient(G, Tau, idx)
    ev[1].record()
    torch.cuda.synchronize()
    grad_ms = ev[0].elapsed_time(ev[1]) / reps
    alg = MLP_FLOPS_PER_POINT * n_points
    return {"points": n_points, "ms": ms, "ms_bf16": ms_bf16, "train_gradient_ms": grad_ms,
            "train_batch": batch, "alg_flops": alg,
            "alg_tflops": alg / ms / 1e9,
            "tensor_flops_issued": 3 * 2 * n_points * (16 * 64 + 64 * 64 + 64 * 8),
            "bytes": n_points * 15 * 4, "hbm_gbs": n_points * 15 * 4 / ms / 1e6,
            "alg_tflops_bf16": alg / ms_bf16 / 1e9,
            "note": "mma.sync m16n8k16 BF16 x FP32-accumulate, weights exact BF16; ms: "
                    "FP32 activations as 3 BF16 terms (3 MMAs per tile); ms_bf16: "
                    "activations rounded to BF16, hardware tanh (1 MMA per tile)"}


def rel_l2(a, b):
    return max(float(np.linalg.norm(a[i] - b[i]) / np.linalg.norm(b[i])) for i in range(len(b)))


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    from fluidsim_gb300 import _lib

    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    n = args.n
    steps = args.steps if args.steps is not None else 100
    v0 = initial_state(n, args.ny, args.nz)
    dt = initial_dt(v0, n)
    sim = make_sim(n, "float32", v0)
    sim.time_stepping.deltat = dt
    lib = sim._lib
    ts = sim.time_stepping
    for _ in range(args.warmup):
        ts.one_time_step()
    torch.cuda.synchronize()

    launches0 = ctypes.c_int64()
    _lib.check(lib.gbs_ns_timing_report(sim._solver, None, None, 0, ctypes.byref(launches0)))
    _lib.check(lib.gbs_ns_timing(sim._solver, 1))
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clocks:
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        start.record()
        for _ in range(steps):
            ts.one_time_step()
        stop.record()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
    elapsed_ms = start.elapsed_time(stop)
    ms = (ctypes.c_double * 5)()
    cnt = (ctypes.c_int64 * 5)()
    launches = ctypes.c_int64()
    _lib.check(lib.gbs_ns_timing_report(sim._solver, ms, cnt, 5, ctypes.byref(launches)))
    _lib.check(lib.gbs_ns_timing(sim._solver, 0))
    steps_per_s, elapsed_ms = replica_rate(elapsed_ms, steps, world, dist, "cuda")

    # roofline of the dominant kernel (largest share of the timed region)
    field_bytes = v0.shape[1] * v0.shape[2] * (n // 2 + 1) * 8  # complex64
    kinds = {k: {"ms": ms[i], "launches": cnt[i]} for i, k in enumerate(KINDS)}
    dom = max(kinds, key=lambda k: kinds[k]["ms"])
    avg_s = kinds[dom]["ms"] / max(kinds[dom]["launches"], 1) / 1000.0
    fpl = fields_per_launch(n, v0.shape[2], v0.shape[1])
    alg_bytes = fpl[dom] * field_bytes
    peak, peak_src = measured_peak()
    achieved = alg_bytes / avg_s / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_src,
                "traffic": ncu_traffic(dom, n), "alg_bytes_per_launch": alg_bytes,
                "kernel_gbs": {k: fpl[k] * field_bytes / (v["ms"] / max(v["launches"], 1)) / 1e6
                               for k, v in kinds.items() if v["ms"] > 0},
                "kernel_ms": {k: v["ms"] / max(v["launches"], 1) for k, v in kinds.items()},
                "kernel_share": {k: v["ms"] / sum(x["ms"] for x in kinds.values())
                                 for k, v in kinds.items()}}
    # whole pruned step: the algorithmic bytes of its 20 launches against
    # the peak at the measured step rate
    step_bytes = 4 * sum(fpl.values()) * field_bytes
    step_gbs = step_bytes * steps_per_s / world / 1e9
    roofline["step"] = {"alg_bytes_per_step": step_bytes, "achieved": step_gbs,
                        "frac": step_gbs / peak, "unit": "GB/s"}

    # end to end: host state in pinned memory, copied in and out every step
    S = sim.state.state_spect
    host_in = torch.empty(S.shape, dtype=S.dtype, pin_memory=True)
    host_in.copy_(S)
    host_out = torch.empty_like(host_in, pin_memory=True)
    e_steps = max(3, steps)
    e2e_serial = e2e_run(ts, S, host_in, host_out, e_steps, world, dist, pipelined=False)
    e2e_run(ts, S, host_in, host_out, 2, world, dist, pipelined=True)  # warm-up
    e2e_rate = e2e_run(ts, S, host_in, host_out, e_steps, world, dist, pipelined=True)
    state_bytes = S.numel() * S.element_size()

    line = {"metric": METRIC, "value": steps_per_s, "unit": "steps/s", "n_gpus": world,
            "steps": steps, "warmup": args.warmup,
            "ms_per_step": elapsed_ms / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(n, v0.shape[2], v0.shape[1], dt, world),
            "precision": "fp32 FFT/products, fp64 twiddles and reductions",
            "gpu_launches": int(launches.value - launches0.value),
            "roofline": roofline,
            "e2e": {"value": e2e_rate, "unit": "steps/s", "h2d_bytes_per_step": state_bytes,
                    "d2h_bytes_per_step": state_bytes,
                    "note": "every step: its input state copied host->device, its result "
                            "device->host (pinned buffers); the copies run on two copy "
                            "streams into and out of three device state buffers in "
                            "rotation (state.set_state_spect), overlapping the "
                            "neighbouring steps' compute; each step checks its copied-in "
                            "state for dealiasing",
                    "serial": e2e_serial},
            "clocks": clocks.summary()}

    if not args.no_fft and args.ny is None and args.nz is None:
        line["fft"] = fft_throughput(n)
        line["mlp_closure"] = mlp_throughput()

    if not args.no_fp64:
        sim32 = make_sim(n, "float32", v0)
        sim32.time_stepping.deltat = dt
        for _ in range(10):
            sim32.time_stepping.one_time_step()
        s32 = sim32.state.state_spect.cpu().numpy()
        del sim32, sim
        torch.cuda.empty_cache()
        sim64 = make_sim(n, "float64", v0)
        sim64.time_stepping.deltat = dt
        sim64.time_stepping.one_time_step()
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record()
        for _ in range(9):
            sim64.time_stepping.one_time_step()
        f1.record()
        torch.cuda.synchronize()
        fp64_rate = 9 / (f0.elapsed_time(f1) / 1000.0)
        s64 = sim64.state.state_spect.cpu().numpy()
        flops = fp64_flops_per_step(n, v0.shape[2], v0.shape[1])
        sm_mhz = line["clocks"].get("sm_mhz") or 2070.0
        peak64 = fp64_peak_tflops(sm_mhz)
        line["fp64"] = {"steps_per_s": fp64_rate, "ms_per_step": 1000.0 / fp64_rate,
                        "roofline": {"bound": "fp64", "flops_per_step": flops,
                                     "achieved": flops * fp64_rate / 1e12, "unit": "TFLOP/s",
                                     "peak": peak64, "frac": flops * fp64_rate / 1e12 / peak64,
                                     "peak_source": (f"derived: 152 SMs x 2 FP64 FMA/clk x 2 "
                                                     f"flops x {sm_mhz:.0f} MHz (median SM "
                                                     "clock of the timed FP32 region)")}}
        line["fp32_over_fp64_speedup"] = steps_per_s / world / fp64_rate
        line["fp32_vs_fp64_rel_l2_10_steps"] = rel_l2(s32.astype(np.complex128), s64)

    if rank == 0 and world == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_sample(n, v0, dt)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
