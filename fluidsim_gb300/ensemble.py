"""Batched ensembles of independent ns2d runs of uneven grid sizes.

Runs of one size are advanced together by ``gbs_ens2d_step`` (one launch
per pass for the whole group, per-run nu_2, nu_8 and dt).  The groups of
different sizes either run on their own streams, or all together through
``gbs_ens2d_mixed_step``: one launch per pass covers every run of every
size, or through ``gbs_ens2d_persistent_step``: all the steps of a call in
one persistent cooperative launch whose CTAs take (stage, pass, group, run,
tile) items from a device queue and wait, with a time limit, only on the
items of their own run that they read.  ``capture`` records
``steps_per_graph`` RK4 steps of every group into one CUDA graph; ``run``
replays it.  ``autotune`` times the compiled tile shapes of each group
(column width of the y passes, rows per CTA of the x pass), keeps the
fastest, then times the three modes (per-group streams, one launch per
pass, persistent) and keeps the fastest.

``python -m fluidsim_gb300.ensemble`` runs the 96-run configuration (32 each
at 128^2, 256^2, 512^2, float32, 500 steps) and prints one JSON line with
runs/s and the per-run error against individually solved float64 runs.
"""

import argparse
import ctypes
import itertools
import json
import time
from math import pi

import numpy as np
import torch

from . import _lib
from .init_fields import cubic_dealias_cutoff, noise_rot_2d

TUNING_CANDIDATES = list(itertools.product((4, 8, 16), (1, 2, 4), (4, 8, 16)))


def _kadim(n):
    ik = np.arange(n)
    return np.where(ik <= n // 2, ik, ik - n)


def cfl_dt(rot_fft, n, L=2 * pi, cfl=0.5, dtmax=0.2):
    """dt of the CFL rule (fluidsim/base/time_stepping/base.py:341-366) for
    the initial field (host, initialisation only)."""
    kx = (2 * pi / L) * np.arange(n // 2 + 1)[None, :]
    ky = (2 * pi / L) * _kadim(n)[:, None]
    k2 = kx**2 + ky**2
    k2[0, 0] = 1.0
    ux = np.fft.irfft2(1j * ky * rot_fft / k2, s=(n, n)) * n * n
    uy = np.fft.irfft2(-1j * kx * rot_fft / k2, s=(n, n)) * n * n
    dx = L / n
    tmp = np.abs(ux).max() / dx + np.abs(uy).max() / dx
    return min(cfl / tmp, dtmax)


def make_group(n, nruns, seed, L=2 * pi, kmin=3.0, kmax=10.0):
    rng = np.random.default_rng(seed)
    nu2 = 10 ** rng.uniform(-5, -3, nruns)
    dx = L / n
    nu8 = np.full(nruns, 2.0 * dx**8)  # as the reference's ns2d example
    rot = np.stack([noise_rot_2d(n, n, L, L, kmin, kmax, seed=seed * 1000 + i)
                    for i in range(nruns)])
    dt = np.array([cfl_dt(r, n, L) for r in rot])
    return {"n": n, "rot0": rot, "nu2": nu2, "nu8": nu8, "dt": dt, "L": L}


class EnsembleNS2D:
    def __init__(self, groups, beta=0.0, coef_dealiasing=2.0 / 3):
        self.lib = _lib.load()
        self.groups = []
        for g in groups:
            n, L = g["n"], g["L"]
            h = ctypes.c_void_p()
            kc = cubic_dealias_cutoff(n, L, coef_dealiasing)
            _lib.check(self.lib.gbs_ens2d_create(n, n, L, L, len(g["nu2"]), kc, kc, beta,
                                                 ctypes.byref(h)), "gbs_ens2d_create")
            arr = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(
                ctypes.POINTER(ctypes.c_double))
            _lib.check(self.lib.gbs_ens2d_set_params(h, arr(g["nu2"]), arr(g["nu8"]),
                                                     arr(g["dt"])))
            S = torch.from_numpy(np.ascontiguousarray(g["rot0"])).to("cuda", torch.complex64)
            self.groups.append({"h": h, "S": S, "S0": S.clone(), "n": n, "tuning": (8, 2, 8),
                                "stream": torch.cuda.Stream()})
        self.graph = None
        self.steps_per_graph = 0
        # single-launch mode: the groups, largest first (their CTAs start first)
        order = sorted(range(len(self.groups)), key=lambda k: -self.groups[k]["n"])
        self._mix_order = order
        hs = (ctypes.c_void_p * len(order))(*[self.groups[k]["h"].value for k in order])
        self._mix = ctypes.c_void_p()
        _lib.check(self.lib.gbs_ens2d_mixed_create(hs, len(order), ctypes.byref(self._mix)),
                   "gbs_ens2d_mixed_create")
        self._mix_states = (ctypes.c_void_p * len(order))(
            *[self.groups[k]["S"].data_ptr() for k in order])
        self.mixed = False
        # persistent mode: all steps of a call in one cooperative launch
        self.persistent = False
        self.persist_threads = 512
        self.persist_timeout_s = 1.0
        self.persist_chunk = 4  # work items a CTA takes from the queue at a time

    def __del__(self):
        if getattr(self, "_mix", None):
            self.lib.gbs_ens2d_mixed_destroy(self._mix)
        for g in getattr(self, "groups", []):
            self.lib.gbs_ens2d_destroy(g["h"])

    def reset(self):
        for g in self.groups:
            g["S"].copy_(g["S0"])

    def _step_group(self, g, nsteps, stream):
        _lib.check(self.lib.gbs_ens2d_step(g["h"], ctypes.c_void_p(g["S"].data_ptr()), nsteps,
                                           _lib.GBS_STEP_DEALIASED,
                                           ctypes.c_void_p(stream.cuda_stream)), "ens2d_step")

    def step(self, nsteps=1, flags=_lib.GBS_STEP_DEALIASED):
        cur = torch.cuda.current_stream()
        if self.persistent:
            _lib.check(self.lib.gbs_ens2d_persistent_set_chunk(self._mix, self.persist_chunk))
            _lib.check(self.lib.gbs_ens2d_persistent_step(
                self._mix, self._mix_states, nsteps, self.persist_threads,
                self.persist_timeout_s, flags, ctypes.c_void_p(cur.cuda_stream)),
                "ens2d_persistent_step")
            return
        if self.mixed:
            _lib.check(self.lib.gbs_ens2d_mixed_step(self._mix, self._mix_states, nsteps,
                                                     _lib.GBS_STEP_DEALIASED,
                                                     ctypes.c_void_p(cur.cuda_stream)),
                       "ens2d_mixed_step")
            return
        for g in self.groups:
            g["stream"].wait_stream(cur)
            self._step_group(g, nsteps, g["stream"])
        for g in self.groups:
            cur.wait_stream(g["stream"])

    def autotune(self, steps=4, candidates=None):
        """Time every compiled tile shape per group; keep the fastest."""
        candidates = candidates or TUNING_CANDIDATES
        table = {}
        for g in self.groups:
            best = None
            for cand in candidates:
                _lib.check(self.lib.gbs_ens2d_set_tuning(g["h"], *cand))
                self._step_group(g, 1, torch.cuda.current_stream())  # warm
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                self._step_group(g, steps, torch.cuda.current_stream())
                e1.record()
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / steps
                if best is None or ms < best[0]:
                    best = (ms, cand)
            g["tuning"] = best[1]
            _lib.check(self.lib.gbs_ens2d_set_tuning(g["h"], *best[1]))
            table[g["n"]] = {"ms_per_step": best[0], "tx_inverse": best[1][0],
                             "rows_x": best[1][1], "tx_forward": best[1][2]}
        # all groups per step: their own streams, or one launch per pass with
        # the fastest threads per CTA of each pass
        def time_all(steps):
            self.step(1)  # warm
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            self.step(steps)
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / steps

        self.mixed = False
        mode_ms = {"per_group_streams": time_all(steps)}
        self.mixed = True
        best_mix = None
        for th in itertools.product((128, 256, 512), repeat=3):
            if self.lib.gbs_ens2d_mixed_set_tuning(self._mix, *th) != _lib.GBS_OK:
                continue  # some group has no tile at these thread counts
            ms = time_all(steps)
            if best_mix is None or ms < best_mix[0]:
                best_mix = (ms, th)
        _lib.check(self.lib.gbs_ens2d_mixed_set_tuning(self._mix, *best_mix[1]))
        mode_ms["single_launch"] = best_mix[0]
        self.mixed = False
        self.persistent = True
        best_p = None
        for th, chunk in itertools.product((256, 512), (1, 4, 16)):
            self.persist_threads, self.persist_chunk = th, chunk
            try:
                ms = time_all(steps)
            except ValueError:  # a group has no tile at this thread count
                continue
            self.check_status()
            if best_p is None or ms < best_p[0]:
                best_p = (ms, th, chunk)
        self.persistent = False
        if best_p is not None:
            self.persist_threads, self.persist_chunk = best_p[1], best_p[2]
            mode_ms["persistent"] = best_p[0]
        mode = min(mode_ms, key=mode_ms.get)
        self.mixed = mode == "single_launch"
        self.persistent = mode == "persistent"
        table["all_groups_ms_per_step"] = mode_ms
        table["single_launch_threads"] = dict(zip(("inverse", "x", "forward"), best_mix[1]))
        table["persistent_threads"] = best_p[1] if best_p else None
        table["persistent_chunk"] = best_p[2] if best_p else None
        table["mode"] = mode
        self.reset()
        return table

    def check_status(self):
        """Raise RuntimeError if a bounded wait of the persistent launch ran out
        (the states are then undefined); clears the status word."""
        st = ctypes.c_int()
        _lib.check(self.lib.gbs_ens2d_persistent_status(self._mix, ctypes.byref(st)),
                   "persistent ensemble step")

    def capture(self, steps_per_graph=10):
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, capture_error_mode="relaxed"):
            self.step(steps_per_graph)
        self.steps_per_graph = steps_per_graph

    def run(self, nsteps):
        if self.graph is None or nsteps % self.steps_per_graph:
            self.step(nsteps)
            return
        for _ in range(nsteps // self.steps_per_graph):
            self.graph.replay()

    def nan_flag(self):
        self.check_status()
        flags = []
        for g in self.groups:
            f = ctypes.c_int()
            _lib.check(self.lib.gbs_ens2d_nan_flag(g["h"], ctypes.byref(f)))
            flags.append(f.value)
        return any(flags)


def reference_run(group, i, nsteps, precision="float64"):
    """Run i of a group solved alone with SimulNS2D (same init and params)."""
    from .solvers import SimulNS2D
    n, L = group["n"], group["L"]
    p = SimulNS2D.create_default_params()
    p.precision = precision
    p.oper.nx = p.oper.ny = n
    p.oper.Lx = p.oper.Ly = L
    p.nu_2, p.nu_8 = float(group["nu2"][i]), float(group["nu8"][i])
    ts = p.time_stepping
    ts.USE_CFL, ts.deltat0, ts.USE_T_END, ts.it_end = False, float(group["dt"][i]), False, nsteps
    sim = SimulNS2D(p)
    sim.init_from_rotfft(group["rot0"][i])
    sim.time_stepping.start()
    return sim.state.state_spect[0].cpu().numpy()


def benchmark(sizes=(128, 256, 512), runs_per_size=32, nsteps=500, steps_per_graph=10,
              n_check=None, seed=0):
    groups = [make_group(n, runs_per_size, seed + k) for k, n in enumerate(sizes)]
    ens = EnsembleNS2D(groups)
    tuning = ens.autotune()
    ens.capture(steps_per_graph)
    ens.reset()
    ens.run(steps_per_graph)  # warm the graph
    ens.reset()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    ens.run(nsteps)
    e1.record()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1000
    nruns = runs_per_size * len(sizes)
    out = {"metric": "batched ns2d ensemble runs/s", "value": nruns / sec, "unit": "runs/s",
           "runs": nruns, "sizes": list(sizes), "steps": nsteps, "seconds": sec,
           "steps_per_graph": steps_per_graph, "tuning": tuning, "nan": ens.nan_flag()}
    errs = {}
    n_check = runs_per_size if n_check is None else n_check
    for gi, g in enumerate(groups):
        got = ens.groups[gi]["S"].cpu().numpy()
        e = []
        for i in range(n_check):
            ref = reference_run(g, i, nsteps)
            e.append(float(np.linalg.norm(got[i] - ref) / np.linalg.norm(ref)))
        errs[g["n"]] = {"max_rel_l2": max(e), "median_rel_l2": float(np.median(e)),
                        "runs_checked": n_check}
    out["error_vs_fp64"] = errs
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--runs-per-size", type=int, default=32)
    ap.add_argument("--check", type=int, default=None)
    a = ap.parse_args()
    print(json.dumps(benchmark(runs_per_size=a.runs_per_size, nsteps=a.steps, n_check=a.check)))


if __name__ == "__main__":
    main()
