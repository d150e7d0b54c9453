"""Time-correlated random forcing normalized to a constant injection rate.

Restates fluidsim's ``tcrandom`` forcing with the ``2nd_degree_eq``
normalization (``fluidsim/base/forcing/specific.py:428-727`` and
``768-868``) for ns3d on the GB300 solver:

* forced modes: ``nkmin <= |k| / deltak <= nkmax`` (all three velocity
  components), raw forcing = complex Gaussian values made solenoidal and
  Hermitian on the ``kx = 0`` plane;
* time correlation: ``f = f1 - (cos((t - t_last) pi / T) + 1) (f1 - f0) / 2``
  with a new ``f1`` every ``T = forcing_rate**(-1/3)``;
* normalization once per time step (``sim.forcing.compute()``): ``f = R f``
  with R the root of smaller magnitude of
  ``(dt/2 sum|f|^2) R^2 + (sum Re(v* f)) R - P = 0`` (Hermitian-weighted sums).

The few forced modes are gathered to the host for the normalization (the
reference computes its forcing on rank 0 as well); the forcing field lives
on the device and the solver adds it to the tendencies in every stage
(``gbs_ns_set_forcing``).  The random draws are this module's own (seeded
numpy generator), not the reference's ``np.random`` sequence.
"""

import ctypes
from math import cos, pi

import numpy as np
import torch

from . import _lib


class TCRandomForcing3D:
    def __init__(self, sim, nkmin=2.0, nkmax=3.0, forcing_rate=1.0, seed=0,
                 time_correlation=None):
        self.sim = sim
        oper = sim.oper
        self.P = float(forcing_rate)
        self.period = (forcing_rate ** (-1.0 / 3) if time_correlation is None
                       else float(time_correlation))
        kz, ky, kx = oper.opfft.get_k_adim_loc()
        KX = oper.deltakx * kx[None, None, :]
        KY = oper.deltaky * ky[None, :, None]
        KZ = oper.deltakz * kz[:, None, None]
        kmod = np.sqrt(KX**2 + KY**2 + KZ**2)
        dk = min(oper.deltakx, oper.deltaky, oper.deltakz)
        sel = (kmod >= nkmin * dk) & (kmod <= nkmax * dk)
        flat = np.flatnonzero(sel)
        self.flat = flat
        iz, iy, ix = np.unravel_index(flat, oper.shapeK)
        self.k = np.stack([np.broadcast_to(KX, oper.shapeK).ravel()[flat],
                           np.broadcast_to(KY, oper.shapeK).ravel()[flat],
                           np.broadcast_to(KZ, oper.shapeK).ravel()[flat]])
        self.w = np.where(ix == 0, 1.0, 2.0)
        if oper.nx % 2 == 0:
            self.w[ix == oper.nx // 2] = 1.0
        # Hermitian partners on the kx = 0 plane
        pos = {int(f): n for n, f in enumerate(flat)}
        self.partner = np.full(len(flat), -1)
        for n, (a, b, c) in enumerate(zip(iz, iy, ix)):
            if c == 0:
                q = np.ravel_multi_index(((-a) % oper.nz, (-b) % oper.ny, 0), oper.shapeK)
                self.partner[n] = pos.get(int(q), -1)
        self.rng = np.random.default_rng(seed)
        self.t_last = 0.0
        self.f0 = self._raw()
        self.f1 = self._raw()
        self.idx = torch.from_numpy(flat).to(oper.device)
        self.dense = torch.zeros((3,) + oper.shapeK, dtype=oper.cdtype, device=oper.device)
        self.forcing = np.zeros((3, len(flat)), np.complex128)
        _lib.check(sim._lib.gbs_ns_set_forcing(sim._solver,
                                               ctypes.c_void_p(self.dense.data_ptr())))

    def _raw(self):
        n = self.k.shape[1]
        f = self.rng.standard_normal((3, n)) + 1j * self.rng.standard_normal((3, n))
        k2 = (self.k**2).sum(0)
        f -= self.k * ((self.k * f).sum(0) / k2)  # solenoidal
        for n_, p in enumerate(self.partner):
            if p > n_:
                f[:, p] = np.conj(f[:, n_])
            elif p == n_:
                f[:, n_] = f[:, n_].real
        return f

    def compute(self):
        """Normalized forcing for the coming step (reads the current state)."""
        ts = self.sim.time_stepping
        t, dt = ts.t, ts.deltat
        if t - self.t_last >= self.period:
            self.t_last = t
            self.f0 = self.f1
            self.f1 = self._raw()
        fr = self.f1 - 0.5 * (cos((t - self.t_last) * pi / self.period) + 1) * (self.f1 - self.f0)
        S = self.sim.state.state_spect.reshape(3, -1)[:, self.idx].cpu().numpy()
        S = S.astype(np.complex128)
        a = dt / 2 * float((self.w * (np.abs(fr) ** 2).sum(0)).sum())
        b = float((self.w * (np.conj(S) * fr).real.sum(0)).sum())
        c = -self.P
        R = _minabs_root(a, b, c)
        self.forcing = R * fr
        f = torch.from_numpy(self.forcing).to(self.dense.device, self.dense.dtype)
        self.dense.view(3, -1)[:, self.idx] = f
        return self.forcing

    def injection_rate(self):
        """sum Re(v* f) + dt/2 sum |f|^2 at the last compute (= P)."""
        S = self.sim.state.state_spect.reshape(3, -1)[:, self.idx].cpu().numpy()
        dt = self.sim.time_stepping.deltat
        return float((self.w * ((np.conj(S) * self.forcing).real.sum(0)
                                + dt / 2 * (np.abs(self.forcing) ** 2).sum(0))).sum())


def _minabs_root(a, b, c):
    """``coef_normalization_from_abc`` with which_root = "minabs"."""
    if a == 0.0:
        return -c / b if b != 0.0 else 0.0
    disc = b * b - 4 * a * c
    if disc < 0:
        return 0.0
    sq = disc**0.5
    r1, r2 = (-b + sq) / (2 * a), (-b - sq) / (2 * a)
    return r2 if abs(r2) < abs(r1) else r1
