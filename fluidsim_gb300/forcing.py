"""fluidsim's coarse normalized forcings on the GB300 solver (ns3d).

Restates, for the ns3d solvers, the forcing types ``tcrandom``
(``TimeCorrelatedRandomPseudoSpectral``), ``random``
(``RandomSimplePseudoSpectral``) and ``proportional`` of
``fluidsim/base/forcing/specific.py`` with the same steps in the same order,
so that a run seeded like a reference run draws the same forcing:

* coarse grid (``specific.py:164-246``): ``nc = 2**i``, the smallest power
  of two ``>= 2 nkmax_forcing`` (the reference's choice when ``pulp`` is
  absent, as in a default fluidsim installation), same box lengths, no
  truncation; forced modes ``deltak nkmin <= |k| <= deltak nkmax`` with
  ``deltak`` the largest of the ``deltak_i`` (the coarse Nyquist planes
  excluded, ``_compute_cond_no_forcing``);
* raw random forcing (``compute_forcingc_raw``, 840-850):
  ``create_arrayK_random(min_val)`` drawn with the global ``np.random``,
  zeroed outside the forced modes, projected on real fields
  (``project_fft_on_realX`` = ``fft(ifft(f))``, ``operators3d.py:1051-1052``;
  the round trip runs on the GPU FFT);
* ``tcrandom`` (``__init__`` 784-822, ``forcingc_raw_each_time`` 824-840,
  ``forcingc_from_f0f1`` 852-868): two seeds ``np.random.randint(0, 2**31)``,
  ``f0``/``f1`` drawn after ``np.random.seed`` of each, a new ``f1`` every
  ``period = forcing_rate**(-1/3)`` (or ``time_correlation``), and
  ``f = f1 - (cos((t - t_last) pi / period) + 1) (f1 - f0) / 2``;
* 2nd-degree normalization of each forced variable
  (``normalize_forcingc_2nd_degree_eq``, 587-676, ``coef_normalization_from_abc``
  678-727) and the ``proportional`` rule (346-425): on the device, by
  ``gbs_forcing_coarse`` (one kernel launch per step, no host
  synchronisation), into the dense forcing array the solver adds to its
  tendencies before projection and dealiasing (``gbs_ns_set_forcing``).

``create_arrayK_random`` belongs to fluidfft, which is not part of the
reference; it is restated here as: real parts, then imaginary parts, each
``np.random.random(shapeK)`` scaled to ``[min_val, max_val)`` (defaults 0 and
1).  The oracle's numpy operator uses the same definition.
"""

import ctypes
from math import pi

import numpy as np
import torch

from . import _lib

FORCING_TYPES = ("tcrandom", "random", "proportional")
_ROOTS = {"minabs": 0, "positive": 1}


def coarse_fft_size(nkmax_forcing):
    """Coarse points per axis, ``specific.py:190-201`` without ``pulp``."""
    i = 0
    while 2 * nkmax_forcing > 2**i:
        i += 1
    return 2**i


def create_arrayK_random(shapeK, min_val=None, max_val=None):
    """Uniform random complex array drawn with the global ``np.random``:
    real parts then imaginary parts, each scaled to ``[min_val, max_val)``."""
    lo = 0.0 if min_val is None else float(min_val)
    hi = 1.0 if max_val is None else float(max_val)
    re = lo + (hi - lo) * np.random.random(shapeK)
    im = lo + (hi - lo) * np.random.random(shapeK)
    return re + 1j * im


def _kadim(n):
    ik = np.arange(n)
    return np.where(ik <= n // 2, ik, ik - n)


class CoarseForcing3D:
    """``sim.forcing`` of the ns3d GB300 solvers: ``compute()`` once per
    step (after the CFL update, ``base.py:208-213``) fills ``forcing_fft``
    for the coming step."""

    def __init__(self, sim):
        self.sim = sim
        pf = sim.params.forcing
        self.type = pf.type
        if self.type not in FORCING_TYPES:
            raise NotImplementedError(
                f"forcing type {self.type!r} on GB300 (available: {FORCING_TYPES})")
        if pf.nkmax_forcing < pf.nkmin_forcing:
            raise ValueError(f"params.forcing.nkmax_forcing = {pf.nkmax_forcing} < "
                             f"params.forcing.nkmin_forcing = {pf.nkmin_forcing}")
        norm = pf.normalized
        if self.type != "proportional":
            if norm.type != "2nd_degree_eq" or norm.constant_rate_of is not None:
                raise NotImplementedError("normalized forcing on GB300: type '2nd_degree_eq' "
                                          "without constant_rate_of")
            if norm.which_root not in _ROOTS:
                raise NotImplementedError(f"which_root {norm.which_root!r} on GB300 "
                                          f"(available: {sorted(_ROOTS)})")
        oper = sim.oper
        keys = pf.key_forced
        if keys is None:
            raise ValueError("params.forcing.key_forced must name state variables of "
                             f"{sim.state.keys_state_spect} (the reference's default "
                             "'rot_fft' is not an ns3d state variable)")
        keys = [keys] if isinstance(keys, str) else list(keys)
        names = list(sim.state.keys_state_spect)
        for k in keys:
            if k not in names:
                raise NotImplementedError(f"forced key {k!r} on GB300: only state variables "
                                          f"{names}")
        if self.type == "proportional" and len(keys) > 1:
            raise ValueError("proportional forcing takes one key_forced")
        self.keys = keys
        self.forcing_rate = float(pf.forcing_rate)

        # coarse grid and forced modes (specific.py:164-246)
        deltak = max(oper.deltakx, oper.deltaky, oper.deltakz)
        kmax, kmin = deltak * pf.nkmax_forcing, deltak * pf.nkmin_forcing
        nc = coarse_fft_size(pf.nkmax_forcing)
        if any(nc > n for n in oper.shapeX):
            raise NotImplementedError(
                "The resolution is too small for the required forcing: "
                f"any(np.greater({[nc]}, {oper.shapeX}))")
        self.nc = nc
        self.shapeK_coarse = (nc, nc, nc // 2 + 1)
        kx = oper.deltakx * np.arange(nc // 2 + 1)
        ky = oper.deltaky * _kadim(nc)
        kz = oper.deltakz * _kadim(nc)
        Kx = np.broadcast_to(kx[None, None, :], self.shapeK_coarse)
        Ky = np.broadcast_to(ky[None, :, None], self.shapeK_coarse)
        Kz = np.broadcast_to(kz[:, None, None], self.shapeK_coarse)
        K = np.sqrt(Kx**2 + Ky**2 + Kz**2)
        no_f = np.logical_or(K > kmax, K < kmin)
        no_f[nc // 2, :, :] = True
        no_f[:, nc // 2, :] = True
        no_f[:, :, nc // 2] = True
        self.COND_NO_F = no_f
        self.nb_forced_modes = int(no_f.size - no_f.sum())
        if not self.nb_forced_modes:
            raise ValueError("0 modes forced.")

        dev = oper.device
        self.forcing_fft = torch.zeros(sim.state.state_spect.shape, dtype=oper.cdtype,
                                       device=dev)
        self._no_f = torch.from_numpy(no_f.astype(np.uint8)).to(dev)
        self._coef = torch.zeros(len(keys), dtype=torch.float64, device=dev)
        self._params = _lib.ForcingParams()
        p = self._params
        p.ndim = 3
        p.nx, p.ny, p.nz = oper.nx, oper.ny, oper.nz
        p.nc = nc
        p.nvar = len(names)
        p.nkeys = len(keys)
        for i, k in enumerate(keys):
            p.keys[i] = names.index(k)
        p.type = 1 if self.type == "proportional" else 0
        p.which_root = _ROOTS.get(norm.which_root, 0)
        p.forcing_rate = self.forcing_rate
        p.dtype = _lib.GBS_F64 if oper.cdtype == torch.complex128 else _lib.GBS_F32
        self._fft = None
        self.min_val = None if pf.random.only_positive else -1

        if getattr(pf, "seed", None) is not None:
            np.random.seed(pf.seed)
        if self.type == "tcrandom":
            self.t_last_change = sim.time_stepping.t
            self._seed0 = np.random.randint(0, 2**31)
            self._seed1 = np.random.randint(0, 2**31)
            np.random.seed(self._seed0)
            self.forcing0 = self.compute_forcingc_raw()
            np.random.seed(self._seed1)
            self.forcing1 = self.compute_forcingc_raw()
            tc = pf.tcrandom.time_correlation
            self.period_change_f0f1 = (self.forcing_rate ** (-1.0 / 3)
                                       if tc == "based_on_forcing_rate" else float(tc))
            self._f0 = self._upload(self.forcing0)
            self._f1 = self._upload(self.forcing1)
        _lib.check(sim._lib.gbs_ns_set_forcing(sim._solver,
                                               ctypes.c_void_p(self.forcing_fft.data_ptr())))

    def _upload(self, f):
        return torch.from_numpy(np.ascontiguousarray(f, dtype=np.complex128)).to(
            self.sim.oper.device)

    def project_fft_on_realX(self, f_fft):
        """``fft(ifft(f_fft))`` on the coarse grid (operators3d.py:1051-1052)."""
        if self._fft is None:
            from .fft import FFT3DGB300
            self._fft = FFT3DGB300(self.nc, self.nc, self.nc, precision="float64",
                                   device=self.sim.oper.device)
        return self._fft.fft(self._fft.ifft(np.ascontiguousarray(f_fft)))

    def compute_forcingc_raw(self):
        """``RandomSimplePseudoSpectral.compute_forcingc_raw``."""
        f_fft = create_arrayK_random(self.shapeK_coarse, min_val=self.min_val)
        f_fft[self.COND_NO_F] = 0.0
        return self.project_fft_on_realX(f_fft)

    def compute(self):
        """The forcing of the coming step (reads the current state)."""
        ts = self.sim.time_stepping
        tsim = ts.t
        mix = 0.0
        if self.type == "tcrandom":
            if tsim - self.t_last_change >= self.period_change_f0f1:
                self.t_last_change = tsim
                self._seed0 = self._seed1
                self.forcing0 = self.forcing1
                self._seed1 = np.random.randint(0, 2**31)
                np.random.seed(self._seed1)
                self.forcing1 = self.compute_forcingc_raw()
                self._f0 = self._f1
                self._f1 = self._upload(self.forcing1)
            omega = pi / self.period_change_f0f1
            mix = float(0.5 * (np.cos((tsim - self.t_last_change) * omega) + 1))
            f0, f1 = self._f0, self._f1
        elif self.type == "random":
            f1 = f0 = self._upload(self.compute_forcingc_raw())
        else:
            f0 = f1 = None
        from .fft import current_stream_handle
        S = self.sim.state.state_spect
        ptr = (lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None)
        _lib.check(self.sim._lib.gbs_forcing_coarse(
            ctypes.byref(self._params), ptr(S), ptr(f0), ptr(f1), ptr(self._no_f),
            mix, ts.deltat, ptr(self.forcing_fft), ptr(self._coef),
            current_stream_handle()), "forcing")
        self._last = (f0, f1)  # keep the uploaded arrays alive until the kernel ran
        return self.forcing_fft

    def get_forcing(self):
        return self.forcing_fft

    def injection_rate(self):
        """Per forced variable: sum Re(v* f) + dt/2 sum |f|^2 over the whole
        spectrum at the current state (= forcing_rate for the normalized
        types, ``verify_injection_rate``, specific.py:269-287)."""
        S = self.sim.state.state_spect.to(torch.complex128)
        F = self.forcing_fft.to(torch.complex128)
        dt = self.sim.time_stepping.deltat
        names = list(self.sim.state.keys_state_spect)
        out = []
        for k in self.keys:
            i = names.index(k)
            p1 = self.sim.oper.sum_wavenumbers((F[i].conj() * S[i]).real)
            p2 = dt / 2 * self.sim.oper.sum_wavenumbers(F[i].abs() ** 2)
            out.append(p1 + p2)
        return out
