"""Learned subgrid closure for coarse-grid LES, end to end on one GB300.

1. ``forced_dns``: ns3d DNS (FP32) forced by the ``tcrandom`` forcing of
   ``fluidsim_gb300.forcing`` on the three velocity components (1/3 each) in
   the shells ``k in [2, 3]``, total power 1, brought to its statistically steady
   state (coarse-grid spin-up, prolongation, fine-grid spin-up); snapshots
   of the spectral state.
2. ``filtered_data``: for each snapshot, top-hat filter of width
   Delta = L / n_les and resampling to the LES grid; targets
   ``tau_ij = filt(u_i u_j) - filt(u_i) filt(u_j)`` and inputs
   ``d_j filt(u_i)`` (the LES-dealiased filtered field), as 9 / 6 float32
   fields on the LES grid.
3. ``train_closure``: the 9 -> 64 -> 64 -> 6 network trained with the
   hand-written gradient and Adam kernels (``closure.ClosureTrainer``).
4. ``run_les``: forced LES on the coarse grid with no model, Smagorinsky or
   the learned closure; time-averaged shell energy spectrum and wall time.
5. ``spectral_error``: relative error of E(k) against the filtered DNS
   spectrum over the LES-resolved shells.

``python -m fluidsim_gb300.les --n-dns 512 --n-les 128`` runs the whole
pipeline and prints one JSON line.
"""

import argparse
import ctypes
import json
import time
from math import pi

import numpy as np
import torch

from . import _lib
from .closure import ClosureMLP, ClosureTrainer
from .fft import FFT3DGB300, current_stream_handle
from .init_fields import cubic_dealias_cutoff, isotropic_3d
from .solvers import SimulNS3D


def make_sim(n, nu, cfl=0.5, precision="float32", turb=None, forcing=True, seed=0,
             closure_precision="fp32"):
    p = SimulNS3D.create_default_params()
    p.precision = precision
    p.oper.nx = p.oper.ny = p.oper.nz = n
    p.nu_2 = nu
    ts = p.time_stepping
    ts.USE_CFL, ts.cfl_coef, ts.deltat0, ts.USE_T_END = True, cfl, 1e-3, False
    if forcing:
        # tcrandom on the three velocity components in shells k in [2, 3]; each
        # component is normalized to 1/3, a total injection rate of 1
        pf = p.forcing
        pf.enable, pf.type, pf.seed = True, "tcrandom", seed
        pf.nkmin_forcing, pf.nkmax_forcing = 2, 3
        pf.key_forced = ["vx_fft", "vy_fft", "vz_fft"]
        pf.forcing_rate = 1.0 / 3
        pf.tcrandom.time_correlation = 1.0
    if turb == "smagorinsky":
        p.turb_model.enable, p.turb_model.type = True, "smagorinsky"
    elif turb is not None:
        p.turb_model.enable, p.turb_model.type = True, "mlp_closure"
    sim = SimulNS3D(p)
    if turb is not None and turb != "smagorinsky":
        sim.set_closure(turb, precision=closure_precision)
    return sim


def shell_spectrum(sim):
    k, E = sim.output.compute_spectrum()
    return k, E


def run_until(sim, t_end):
    ts = sim.time_stepping
    n0 = ts.it
    while ts.t < t_end:
        ts.one_time_step()
    return ts.it - n0


def prolong(S, n_in, n_out, precision="float32"):
    """Spectral prolongation of a (3, ...) state from n_in^3 to n_out^3
    (zero padding; the wavenumbers are grid independent)."""
    lib = _lib.load()
    L = (ctypes.c_double * 3)(2 * pi, 2 * pi, 2 * pi)
    sin_ = (ctypes.c_int64 * 3)(n_in, n_in, n_in)
    sout = (ctypes.c_int64 * 3)(n_out, n_out, n_out)
    out = torch.empty((3, n_out, n_out, n_out // 2 + 1), dtype=S.dtype, device=S.device)
    dt = _lib.GBS_F32 if S.dtype == torch.complex64 else _lib.GBS_F64
    _lib.check(lib.gbs_spectral_resample(sin_, sout, 3, L, 0.0, dt,
                                         ctypes.c_void_p(S.contiguous().data_ptr()),
                                         ctypes.c_void_p(out.data_ptr()),
                                         current_stream_handle()))
    return out


def forced_dns(n, nu=3e-4, t_coarse=6.0, t_fine=1.5, n_snap=4, t_between=0.25, seed=0):
    """Forced DNS in its statistically steady state.

    1. Spin-up of the large scales on the n/2 grid with the Smagorinsky
       model for ``t_coarse`` (several large-eddy turnover times at 1/16 of
       the cost of the full grid);
    2. spectral prolongation to n^3 and ``t_fine`` of plain DNS, in which the
       small scales fill in (their turnover times are short);
    3. ``n_snap`` snapshots of the spectral state ``t_between`` apart.

    Returns (snapshots on the device, mean shell spectrum, stats)."""
    nc = n // 2
    simc = make_sim(nc, nu, turb="smagorinsky", seed=seed)
    v0 = isotropic_3d(nc, nc, nc, k0=3.0, energy=0.5, seed=seed)
    simc.state.init_statespect_from(vx_fft=v0[0], vy_fft=v0[1], vz_fft=v0[2])
    t0 = time.perf_counter()
    steps_c = run_until(simc, t_coarse)
    torch.cuda.synchronize()
    t_spin_c = time.perf_counter() - t0
    S = prolong(simc.state.state_spect, nc, n)
    E_coarse = simc.output.compute_energy()
    del simc
    torch.cuda.empty_cache()

    sim = make_sim(n, nu, seed=seed + 1)
    sim.state.init_statespect_from(vx_fft=S[0], vy_fft=S[1], vz_fft=S[2])
    del S
    ts = sim.time_stepping
    ts.t = t_coarse
    t0 = time.perf_counter()
    steps_f = run_until(sim, t_coarse + t_fine)
    torch.cuda.synchronize()
    t_spin_f = time.perf_counter() - t0
    snaps, spectra, energies = [], [], []
    t0 = time.perf_counter()
    t_sim0 = ts.t
    nsteps = 0
    for i in range(n_snap):
        if i:
            nsteps += run_until(sim, t_sim0 + i * t_between)
        snaps.append(sim.state.state_spect.clone())
        spectra.append(shell_spectrum(sim)[1])
        energies.append(sim.output.compute_energy())
    torch.cuda.synchronize()
    t_run = time.perf_counter() - t0
    k = shell_spectrum(sim)[0]
    stats = {"n": n, "coarse_spinup": {"n": nc, "model": "smagorinsky", "t": t_coarse,
                                       "steps": steps_c, "wall_s": t_spin_c, "E": E_coarse},
             "steps_fine": steps_f + nsteps, "t_spinup_fine_s": t_spin_f,
             "dt_last": ts.deltat, "s_per_step": t_run / max(nsteps, 1),
             "wall_per_time_unit_s": t_run / max(ts.t - t_sim0, 1e-30),
             "E_snapshots": energies, "t": ts.t}
    return snaps, (k, np.mean(spectra, axis=0)), stats


def filtered_data(snaps, n_dns, n_les):
    """(G (9, N) float32, Tau (6, N) float32) on the LES grid, and the mean
    shell spectrum of the filtered velocity."""
    lib = _lib.load()
    st = current_stream_handle()
    delta = 2 * pi / n_les
    L = (ctypes.c_double * 3)(2 * pi, 2 * pi, 2 * pi)
    sin_ = (ctypes.c_int64 * 3)(n_dns, n_dns, n_dns)
    sout = (ctypes.c_int64 * 3)(n_les, n_les, n_les)
    dns = FFT3DGB300(n_dns, n_dns, n_dns, precision="float32")
    les = FFT3DGB300(n_les, n_les, n_les, precision="float32")
    kc = cubic_dealias_cutoff(n_les, 2 * pi)
    kcut = (ctypes.c_int64 * 3)(kc, kc, kc)
    Gs, Ts, specs = [], [], []
    first = None
    sim_les = make_sim(n_les, 1e-3, forcing=False)
    for S in snaps:
        u = torch.empty((3,) + dns.shapeX, dtype=torch.float32, device="cuda")
        dns.ifft_as_arg(S.contiguous(), u)
        uu = torch.empty((6,) + dns.shapeX, dtype=torch.float32, device="cuda")
        _lib.check(lib.gbs_products6(ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(uu.data_ptr()),
                                     u[0].numel(), None, _lib.GBS_F32, st))
        del u
        uu_k = torch.empty((6,) + dns.shapeK, dtype=torch.complex64, device="cuda")
        dns.fft_as_arg(uu, uu_k)
        del uu
        ub_k = torch.empty((3,) + les.shapeK, dtype=torch.complex64, device="cuda")
        uub_k = torch.empty((6,) + les.shapeK, dtype=torch.complex64, device="cuda")
        for src, dst, nf in ((S, ub_k, 3), (uu_k, uub_k, 6)):
            _lib.check(lib.gbs_spectral_resample(sin_, sout, nf, L, delta, _lib.GBS_F32,
                                                 ctypes.c_void_p(src.data_ptr()),
                                                 ctypes.c_void_p(dst.data_ptr()), st))
        del uu_k
        # the LES represents only |k| < kcut: the effective filter is the box
        # filter followed by the sharp truncation, applied to both terms of tau
        sim_les.oper.dealiasing(ub_k)
        sim_les.oper.dealiasing(uub_k)
        ub = torch.empty((3,) + les.shapeX, dtype=torch.float32, device="cuda")
        les.ifft_as_arg(ub_k, ub)
        uub = torch.empty((6,) + les.shapeX, dtype=torch.float32, device="cuda")
        les.ifft_as_arg_destroy(uub_k, uub)
        tau = torch.empty_like(uub)
        _lib.check(lib.gbs_products6(ctypes.c_void_p(ub.data_ptr()), ctypes.c_void_p(tau.data_ptr()),
                                     ub[0].numel(), ctypes.c_void_p(uub.data_ptr()),
                                     _lib.GBS_F32, st))
        gk = torch.empty((9,) + les.shapeK, dtype=torch.complex64, device="cuda")
        _lib.check(lib.gbs_velocity_gradients(sout, L, kcut, _lib.GBS_F32,
                                              ctypes.c_void_p(ub_k.data_ptr()),
                                              ctypes.c_void_p(gk.data_ptr()), st))
        g = torch.empty((9,) + les.shapeX, dtype=torch.float32, device="cuda")
        les.ifft_as_arg_destroy(gk, g)
        Gs.append(g.reshape(9, -1))
        Ts.append(tau.reshape(6, -1))
        sim_les.state.state_spect.copy_(ub_k)
        specs.append(shell_spectrum(sim_les)[1])
        if first is None:
            first = ub_k.cpu().numpy()
    k = shell_spectrum(sim_les)[0]
    return torch.cat(Gs, dim=1).contiguous(), torch.cat(Ts, dim=1).contiguous(), (
        k, np.mean(specs, axis=0)), first


def train_closure(G, Tau, steps=3000, batch=65536, lr=2e-3, lr_final=1e-4, seed=0,
                  lambda_pi=1.0):
    net = ClosureMLP(seed=seed)
    tr = ClosureTrainer(net, batch=batch, lr=lr, seed=seed, lambda_pi=lambda_pi)
    tr.set_scales(G, Tau)
    t0 = time.perf_counter()
    hist = tr.train(G, Tau, steps, log_every=max(steps // 10, 1), lr_final=lr_final)
    torch.cuda.synchronize()
    return net, {"history": hist, "train_s": time.perf_counter() - t0, "steps": steps,
                 "batch": batch, "samples": int(G.shape[1]), "lambda_pi": lambda_pi}


def run_les(n, model, nu=3e-4, steps=2000, avg_last=1000, init=None, seed=0,
            closure_precision="bf16"):
    """Forced LES; returns ((k, time-averaged E(k)), stats).  A run that
    produces NaN stops there and reports ``"nan": true`` (its spectrum is
    then the average of what was collected)."""
    sim = make_sim(n, nu, turb=model, seed=seed, closure_precision=closure_precision)
    if init is None:
        init = isotropic_3d(n, n, n, k0=3.0, energy=0.5, seed=seed)
    sim.state.init_statespect_from(**{k: init[i] for i, k in enumerate(sim.state.keys_state_spect)})
    ts = sim.time_stepping
    specs = []
    nan = False
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    done = 0
    for it in range(steps):
        try:
            ts.one_time_step()
        except ValueError:
            nan = True
            break
        done += 1
        if it >= steps - avg_last and (it - (steps - avg_last)) % 50 == 0:
            specs.append(shell_spectrum(sim)[1])
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    k = shell_spectrum(sim)[0]
    E_k = np.mean(specs, axis=0) if specs else np.full(len(k), np.nan)
    return (k, E_k), {"n": n, "steps": done, "wall_s": wall, "nan": nan,
                      "s_per_step": wall / max(done, 1), "dt_last": ts.deltat,
                      "wall_per_time_unit_s": wall / max(ts.t, 1e-30),
                      "E": sim.output.compute_energy() if not nan else float("nan"),
                      "t": ts.t}


def spectral_error(k_les, E_les, k_ref, E_ref, kmin=1.0, kmax=None, reduce=np.mean):
    """Mean (or ``reduce``) relative error of E(k) over shells
    kmin <= k <= kmax."""
    n = min(len(E_les), len(E_ref))
    k = k_les[:n]
    sel = (k >= kmin) & (k <= (kmax if kmax is not None else k[n - 1]))
    return float(reduce(np.abs(E_les[:n][sel] - E_ref[:n][sel]) / E_ref[:n][sel]))


def pipeline(n_dns=512, n_les=128, nu=3e-4, t_coarse=6.0, t_fine=1.5, n_snap=4,
             t_between=0.25, train_steps=3000, les_steps=2000, lambda_pi=1.0, seed=0,
             closure_precision="bf16"):
    out = {"config": {"n_dns": n_dns, "n_les": n_les, "nu": nu, "forcing": "tcrandom k in [2,3], P=1",
                      "closure": "MLP 9-64-64-6 tanh, BF16 weights, FP32 accumulation",
                      "closure_precision_in_les": closure_precision,
                      "filter": "top-hat width L/n_les, then the LES grid's 2/3 truncation"}}
    snaps, (k_dns, E_dns), st_dns = forced_dns(n_dns, nu, t_coarse=t_coarse, t_fine=t_fine,
                                              n_snap=n_snap, t_between=t_between, seed=seed)
    out["dns"] = st_dns
    G, Tau, (k_f, E_f), init_les = filtered_data(snaps, n_dns, n_les)
    del snaps
    torch.cuda.empty_cache()
    net, st_train = train_closure(G, Tau, steps=train_steps, seed=seed, lambda_pi=lambda_pi)
    out["train"] = st_train
    from .closure import predict
    pred = predict(net, G)
    out["train"]["rel_mse"] = float(((pred - Tau) ** 2).mean() / (Tau**2).mean())
    from .closure import subgrid_dissipation
    pi_t, pi_p = subgrid_dissipation(G, Tau), subgrid_dissipation(G, pred)
    out["train"]["mean_dissipation_target"] = float(pi_t.double().mean())
    out["train"]["mean_dissipation_learned"] = float(pi_p.double().mean())
    out["train"]["dissipation_corr"] = float(torch.corrcoef(torch.stack([pi_t, pi_p]).double())[0, 1])
    del G, Tau
    kc = cubic_dealias_cutoff(n_les, 2 * pi) - 1
    res = {}
    for name, model in (("none", None), ("smagorinsky", "smagorinsky"), ("learned", net)):
        (k_l, E_l), st = run_les(n_les, model, nu=nu, steps=les_steps, avg_last=les_steps // 2,
                                 closure_precision=closure_precision,
                                 init=init_les, seed=seed)
        st["spectral_error"] = spectral_error(k_l, E_l, k_f, E_f, kmin=1.0, kmax=kc)
        st["spectral_error_k_ge_4"] = spectral_error(k_l, E_l, k_f, E_f, kmin=4.0, kmax=kc)
        st["spectral_error_max"] = spectral_error(k_l, E_l, k_f, E_f, kmin=1.0, kmax=kc,
                                                  reduce=np.max)
        res[name] = st
        res[name]["E_k"] = [float(x) for x in E_l[:kc + 1]]
    out["les"] = res
    out["filtered_dns_E_k"] = [float(x) for x in E_f[:kc + 1]]
    out["wall_time_ratio_dns_over_les_per_unit_time"] = (
        st_dns["wall_per_time_unit_s"] / res["learned"]["wall_per_time_unit_s"])
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-dns", type=int, default=512)
    ap.add_argument("--n-les", type=int, default=128)
    ap.add_argument("--t-coarse", type=float, default=6.0)
    ap.add_argument("--t-fine", type=float, default=1.5)
    ap.add_argument("--n-snap", type=int, default=4)
    ap.add_argument("--t-between", type=float, default=0.25)
    ap.add_argument("--train-steps", type=int, default=3000)
    ap.add_argument("--les-steps", type=int, default=2000)
    ap.add_argument("--nu", type=float, default=3e-4)
    ap.add_argument("--lambda-pi", type=float, default=1.0)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    out = pipeline(a.n_dns, a.n_les, nu=a.nu, t_coarse=a.t_coarse, t_fine=a.t_fine,
                   n_snap=a.n_snap, t_between=a.t_between, train_steps=a.train_steps,
                   les_steps=a.les_steps, lambda_pi=a.lambda_pi)
    line = json.dumps(out)
    print(line)
    if a.out:
        with open(a.out, "w") as f:
            f.write(line + "\n")


if __name__ == "__main__":
    main()
