"""ns2d / ns3d solvers whose time step runs in libgbspec on one GB300.

The class layout follows fluidsim's (``Simul`` with ``create_default_params``
and ``tendencies_nonlin``, ``State`` with ``state_spect`` / ``state_phys``,
``TimeSteppingPseudoSpectral`` with ``start`` / ``one_time_step``, ``Output``
with the spatial means), so solver scripts written for
``fluidsim.solvers.ns2d`` / ``ns3d`` run unchanged on the parts listed here:

* ``fluidsim/solvers/ns2d/solver.py:111-194`` / ``ns3d/solver.py:180-263``
  -> ``Simul.tendencies_nonlin`` (fused kernels, ``gbs_ns_tendencies``);
* ``fluidsim/base/time_stepping/pseudo_spect.py`` time schemes with exact
  integrating factor (RK4 798-984, Euler 245-280, RK2 469-517,
  RK2_trapezoid 519-569) + ``one_time_step_computation`` (236-243, ns3d
  ``time_stepping.py:8-20``) -> ``gbs_ns_step``;
* ``fluidsim/base/time_stepping/base.py:182-354`` (loop, CFL with the 2 %
  hysteresis, ``max_elapsed``, SIGUSR2 stop) -> ``TimeSteppingPseudoSpectral``;
* spatial means / spectra (FP64 device reductions).

State arrays are CUDA tensors in the sequential fluidfft layout; the
precision is chosen with ``params.precision`` ("float64" or "float32").
"""

import ctypes
import random
import signal
from datetime import datetime, timedelta
from math import pi
from time import time

import numpy as np
import torch

from . import _lib
from .fft import current_stream_handle
from .operators import OperatorsPseudoSpectral2D, OperatorsPseudoSpectral3D
from .params import Parameters


class StatePseudoSpectral:
    """``fluidsim/base/state.py:209-392`` on device tensors."""

    def __init__(self, sim):
        self.sim = sim
        self.oper = sim.oper
        self.keys_state_spect = list(sim.keys_state_spect)
        self.keys_state_phys = list(sim.keys_state_phys)
        self.state_spect = torch.zeros((len(self.keys_state_spect),) + self.oper.shapeK,
                                       dtype=self.oper.cdtype, device=self.oper.device)
        self._phys = None
        self._phys_stamp = None
        self.is_initialized = False

    # state_phys is regenerated lazily from state_spect (3 C2R transforms)
    def _stamp(self):
        return (self.sim.time_stepping.it, self.state_spect._version)

    @property
    def state_phys(self):
        if self._phys is None or self._phys_stamp != self._stamp():
            self._phys = self.sim._statephys_from_statespect(self.state_spect)
            self._phys_stamp = self._stamp()
        return self._phys

    def statephys_from_statespect(self):
        self._phys = None
        return self.state_phys

    def get_var(self, key):
        if key in self.keys_state_spect:
            return self.state_spect[self.keys_state_spect.index(key)]
        if key in self.keys_state_phys:
            return self.state_phys[self.keys_state_phys.index(key)]
        raise ValueError(f'Do not know how to compute "{key}".')

    def has_vars(self, *keys):
        return set(keys).issubset(set(self.keys_state_spect + self.keys_state_phys))

    def set_state_spect(self, tensor):
        """Make the device tensor ``tensor`` (shape, dtype and device of
        ``state_spect``, contiguous) the spectral state, without a copy: the
        next steps read and update it in place.  Lets a caller rotate state
        buffers, e.g. fill one from the host while a step runs on another."""
        s = self.state_spect
        if (not isinstance(tensor, torch.Tensor) or tensor.shape != s.shape
                or tensor.dtype != s.dtype or tensor.device != s.device
                or not tensor.is_contiguous()):
            raise ValueError("set_state_spect: a contiguous tensor of shape "
                             f"{tuple(s.shape)}, dtype {s.dtype} on {s.device} is required")
        self.state_spect = tensor
        self._phys = None
        self.sim.time_stepping._dealiased_version = None

    def init_statespect_from(self, **kwargs):
        """``fluidsim/base/state.py:345-382``: other keys are set to zero."""
        self.state_spect.zero_()
        for key, value in kwargs.items():
            if key not in self.keys_state_spect:
                raise ValueError(f"Do not know how to initialize with key '{key}'.")
            v = value if isinstance(value, torch.Tensor) else torch.from_numpy(np.asarray(value))
            self.state_spect[self.keys_state_spect.index(key)].copy_(v)
        self._phys = None
        self.is_initialized = True


class _PhaseShiftPairs:
    """The (alpha, beta) shift pairs of the ``*_phaseshift_random`` schemes,
    drawn exactly as the reference does, with the global ``random`` module
    (so ``random.seed`` before building the simulation repeats a reference
    run): ``get_phases_random`` (operators3d.py:1128-1146,
    operators2d.py:618-631) and the pair rotation of
    ``TimeSteppingPseudoSpectral._init_phaseshift_random`` /
    ``_get_phaseshift_random`` (pseudo_spect.py:302-372).  A pair holds the
    shifts in grid spacings per axis (x, y[, z])."""

    def __init__(self, ndim, nb_pairs, nb_steps_compute_new_pair):
        self.ndim = ndim
        if nb_steps_compute_new_pair is None:
            nb_steps_compute_new_pair = 2 if nb_pairs == 1 else 4 * nb_pairs
        self.nb_pairs = nb_pairs
        self.nb_new = nb_steps_compute_new_pair
        self._index = 1
        self._previous_index_pair = 0
        self._previous_index_flip = 0
        self._pairs = [self._draw() for _ in range(nb_pairs)]

    def _draw(self):
        alpha = tuple(random.uniform(-0.5, 0.5) for _ in range(self.ndim))
        beta = tuple(a + 0.5 if a < 0 else a - 0.5 for a in alpha)
        return alpha, beta

    def next(self):
        if self.nb_pairs == 1 and self.nb_new == 1:
            alpha, beta = self._pairs[0]
        elif self.nb_pairs == 1 and self.nb_new == 2:
            pair = self._pairs[0]
            alpha, beta = pair if self._index == 1 else pair[::-1]
        else:
            index_pair = random.randint(0, self.nb_pairs - 1)
            pair = self._pairs[index_pair]
            index_flip = random.randint(0, 1)
            if (index_pair == self._previous_index_pair
                    and index_flip == self._previous_index_flip):
                index_flip = 0 if index_flip else 1
            self._previous_index_pair = index_pair
            self._previous_index_flip = index_flip
            alpha, beta = pair if index_flip else pair[::-1]
        if self._index == self.nb_new:
            self._index = 1
            new_pair = self._draw()
            self._pairs.pop(0)
            self._pairs.append(new_pair)
        else:
            self._index += 1
        return alpha, beta


class TimeSteppingPseudoSpectral:
    """Pseudo-spectral time stepping (RK4, RK2, RK2_trapezoid, Euler and the
    phase-shift schemes) with the reference loop semantics."""

    @staticmethod
    def _complete_params_with_default(params):
        # base.py:33-46 + pseudo_spect.py:159-167 (USE_CFL = True)
        params._set_child("time_stepping", attribs={
            "USE_T_END": True, "t_end": 10.0, "it_end": 10, "USE_CFL": True,
            "type_time_scheme": "RK4", "deltat0": 0.2, "deltat_max": 0.2,
            "cfl_coef": None, "max_elapsed": None})
        params.time_stepping._set_child(
            "phaseshift_random", attribs={"nb_pairs": 1, "nb_steps_compute_new_pair": None})

    def __init__(self, sim):
        self.sim = sim
        self.params = sim.params
        pts = self.params.time_stepping
        self.it = 0
        self.t = 0.0
        self._has_to_stop = False
        self._stop_signal_received = False
        if pts.type_time_scheme not in _lib.SCHEMES:
            raise NotImplementedError(
                f"type_time_scheme {pts.type_time_scheme!r}: GB300 runs "
                + ", ".join(_lib.SCHEMES))
        self._scheme = _lib.SCHEMES[pts.type_time_scheme]
        self._phase_pairs = None
        if pts.type_time_scheme.endswith("_random"):
            pr = pts.phaseshift_random
            self._phase_pairs = _PhaseShiftPairs(len(sim.oper.shapeX), pr.nb_pairs,
                                                 pr.nb_steps_compute_new_pair)
        if pts.USE_CFL:
            # base.py:249-260: default coefficient 0.4 for RK2*/Euler*, 1 for RK4
            if pts.cfl_coef is not None:
                self.CFL = pts.cfl_coef
            else:
                self.CFL = 1.0 if pts.type_time_scheme.startswith("RK4") else 0.4
        self.deltat = pts.deltat0
        self.deltat_max = pts.deltat_max
        if hasattr(sim, "deltat_cap"):  # ns2d.strat: dispersion-relation time
            self.deltat_max = min(self.deltat_max, sim.deltat_cap())
        self._nan_check = True
        # (address, _version) of state_spect right after our last step:
        # while both are unchanged the state is the dealiased output of it
        self._dealiased_version = None

        def handler(signum, stack):
            self._stop_signal_received = signum

        try:
            signal.signal(signal.SIGUSR2, handler)
        except (ValueError, AttributeError):
            pass
        self.max_elapsed = None
        if pts.max_elapsed is not None:
            try:
                self.max_elapsed = float(pts.max_elapsed)
            except ValueError:
                tt = datetime.strptime(pts.max_elapsed, "%H:%M:%S")
                self.max_elapsed = timedelta(
                    hours=tt.hour, minutes=tt.minute, seconds=tt.second).total_seconds()
            self._time_should_stop = time() + self.max_elapsed

    def start(self):
        self.main_loop()

    def main_loop(self, print_begin=False, save_init_field=False):
        pts = self.params.time_stepping
        if pts.USE_T_END:
            while self.t < pts.t_end and not self._has_to_stop:
                self.one_time_step()
        else:
            while self.it < pts.it_end and not self._has_to_stop:
                self.one_time_step()

    def one_time_step(self):
        """``fluidsim/base/time_stepping/base.py:208-244``."""
        forcing = getattr(self.sim, "forcing", None)
        if forcing is not None:
            # CFL first, then sim.forcing.compute() with that dt (base.py:210-213)
            if self.params.time_stepping.USE_CFL:
                vmax = self.sim.max_velocity()
                o = self.sim.oper
                tmp = sum(v / d for v, d in zip(vmax, (o.deltax, o.deltay, o.deltaz)))
                self.deltat = self.sim._lib.gbs_cfl_update(self.deltat, tmp, self.CFL,
                                                           self.deltat_max)
            forcing.compute()
        if self.max_elapsed is not None and time() > self._time_should_stop:
            self._has_to_stop = True
        if self._stop_signal_received:
            self._has_to_stop = True
        self.sim.output.one_time_step()
        self.one_time_step_computation()
        self.t += self.deltat
        self.it += 1

    def one_time_step_computation(self):
        """One step of the scheme + projection (ns3d) + dealiasing + NaN
        check, one library call."""
        pts = self.params.time_stepping
        dt = ctypes.c_double(self.deltat)
        cfl = (ctypes.c_double * 2)(self.CFL, self.deltat_max) if pts.USE_CFL else None
        if getattr(self.sim, "forcing", None) is not None:
            cfl = None  # dt already updated before the forcing was computed
        S = self.sim.state.state_spect
        flags = _lib.GBS_STEP_CHECK_NAN if self._nan_check else 0
        if self._dealiased_version == (S.data_ptr(), S._version):
            flags |= _lib.GBS_STEP_DEALIASED
        else:
            # a state set through torch: prune only if it is exactly zero
            # outside the 2/3 box (then the pruned step is bit-identical)
            ok = ctypes.c_int()
            _lib.check(self.sim._lib.gbs_ns_is_dealiased(
                self.sim._solver, ctypes.c_void_p(S.data_ptr()), ctypes.byref(ok),
                current_stream_handle()), "gbs_ns_is_dealiased")
            if ok.value:
                flags |= _lib.GBS_STEP_DEALIASED
        if self._phase_pairs is not None:
            alpha, beta = self._phase_pairs.next()
            pad = (0.0,) * (3 - len(alpha))
            _lib.check(self.sim._lib.gbs_ns_set_phase_shifts(
                self.sim._solver, (ctypes.c_double * 3)(*alpha, *pad),
                (ctypes.c_double * 3)(*beta, *pad)), "gbs_ns_set_phase_shifts")
        rc = self.sim._lib.gbs_ns_step(
            self.sim._solver, self._scheme, ctypes.c_void_p(S.data_ptr()), ctypes.byref(dt),
            cfl, flags, current_stream_handle())
        self.deltat = dt.value
        self._dealiased_version = (S.data_ptr(), S._version)
        self.sim.state._phys = None
        if rc == _lib.GBS_ENAN:
            raise ValueError(f"nan at it = {self.it}, t = {self.t:.4f}")
        _lib.check(rc, "gbs_ns_step_rk4")


class Output:
    """Spatial means and spectra (FP64 device reductions)."""

    @staticmethod
    def _complete_params_with_default(params):
        params._set_child("output", attribs={"HAS_TO_SAVE": False, "sub_directory": ""})
        params.output._set_child("periods_save", attribs={"spatial_means": 0.0})

    def __init__(self, sim):
        self.sim = sim
        self.spatial_means_series = []
        self._t_last = -np.inf

    def one_time_step(self):
        period = self.sim.params.output.periods_save.spatial_means
        ts = self.sim.time_stepping
        if period and ts.t >= self._t_last + period:
            self._t_last = ts.t
            self.spatial_means_series.append({"t": ts.t, **self.compute_spatial_means()})

    def compute_spatial_means(self):
        out = (ctypes.c_double * 9)()
        sim = self.sim
        _lib.check(sim._lib.gbs_ns_spatial_means(
            sim._solver, ctypes.c_void_p(sim.state.state_spect.data_ptr()), out,
            current_stream_handle()), "gbs_ns_spatial_means")
        means = dict(zip(sim._means_keys, list(out)))
        if "EA" in means:  # ns3d.strat: kinetic + potential
            means["E"] = means["EK"] + means["EA"]
        return means

    def compute_energy(self):
        return self.compute_spatial_means()["E"]

    def compute_spectrum(self):
        """(k, E(k)) shell spectrum, bins round(|k|/dk_min)."""
        sim = self.sim
        nk = ctypes.c_int64()
        _lib.check(sim._lib.gbs_ns_spectrum_size(sim._solver, ctypes.byref(nk)))
        spec = torch.empty(nk.value, dtype=torch.float64, device=sim.oper.device)
        _lib.check(sim._lib.gbs_ns_spectrum(
            sim._solver, ctypes.c_void_p(sim.state.state_spect.data_ptr()),
            ctypes.c_void_p(spec.data_ptr()), current_stream_handle()))
        dk = min(sim.oper.deltakx, sim.oper.deltaky,
                 getattr(sim.oper, "deltakz", np.inf))
        return dk * np.arange(nk.value), spec.cpu().numpy()

    def print_stdout(self, *args, **kwargs):
        print(*args, **kwargs)


class _SimulBase:
    Operators = None
    ndim = None

    @classmethod
    def create_default_params(cls):
        params = Parameters("params", {
            "short_name_type_run": "", "NEW_DIR_RESULTS": True, "ONLY_COARSE_OPER": False,
            "nu_2": 0.0, "nu_4": 0.0, "nu_8": 0.0, "nu_m4": 0.0,
            "precision": "float64"})
        cls.Operators._complete_params_with_default(params)
        params.oper._set_attribs({"type_fft": "default"})
        TimeSteppingPseudoSpectral._complete_params_with_default(params)
        Output._complete_params_with_default(params)
        params._set_child("init_fields", attribs={"type": "in_script"})
        # fluidsim/base/forcing/base.py:55-90 and specific.py:440-455,
        # 736-745, 775-782 (defaults of ForcingBasePseudoSpectral, normalized,
        # random, tcrandom); `seed` (None: the global np.random state, as the
        # reference) is this build's addition
        params._set_child("forcing", attribs={
            "enable": False, "type": "", "forcing_rate": 1.0, "key_forced": None,
            "nkmin_forcing": 4, "nkmax_forcing": 5, "seed": None})
        params.forcing._set_child("normalized", attribs={
            "type": "2nd_degree_eq", "which_root": "minabs", "constant_rate_of": None})
        params.forcing._set_child("random", attribs={"only_positive": False})
        params.forcing._set_child("tcrandom", attribs={
            "time_correlation": "based_on_forcing_rate"})
        cls._complete_params_with_default(params)
        return params

    @staticmethod
    def _complete_params_with_default(params):
        pass

    def __init__(self, params):
        self.params = params
        if params.forcing.enable:
            from .forcing import FORCING_TYPES
            if self.ndim != 3 or params.forcing.type not in FORCING_TYPES:
                raise NotImplementedError(f"forcing on GB300: ns3d with a type of "
                                          f"{FORCING_TYPES}")
        if params.init_fields.type != "in_script":
            raise NotImplementedError("only init_fields.type = 'in_script' is supported")
        self._lib = _lib.load()
        self.oper = self.Operators(params, precision=params.precision)
        self.state = StatePseudoSpectral(self)
        self.output = Output(self)
        self._solver = ctypes.c_void_p()
        p = self._ns_params()
        with torch.cuda.device(self.oper.device):
            _lib.check(self._lib.gbs_ns_create(ctypes.byref(p), ctypes.byref(self._solver)),
                       "gbs_ns_create")
        self.time_stepping = TimeSteppingPseudoSpectral(self)
        self.is_forcing_enabled = False
        self.forcing = None

    def __del__(self):
        lib = getattr(self, "_lib", None)
        solver = getattr(self, "_solver", None)
        if lib is not None and solver:
            lib.gbs_ns_destroy(solver)
            self._solver = None

    def _ns_params(self):
        prm = self.params
        o = self.oper
        p = _lib.NSParams()
        p.ndim = self.ndim
        p.nx, p.ny = o.nx, o.ny
        p.nz = o.nz if self.ndim == 3 else 1
        p.Lx, p.Ly = o.Lx, o.Ly
        p.Lz = o.Lz if self.ndim == 3 else 1.0
        p.nu_2, p.nu_4, p.nu_8, p.nu_m4 = prm.nu_2, prm.nu_4, prm.nu_8, prm.nu_m4
        p.kcut_x = o.kcut[-1]
        p.kcut_y = o.kcut[-2]
        p.kcut_z = o.kcut[0] if self.ndim == 3 else 1
        p.dtype = _lib.GBS_F64 if prm.precision == "float64" else _lib.GBS_F32
        return p

    def tendencies_nonlin(self, state_spect=None, old=None):
        """Dealiased nonlinear tendencies of ``state_spect`` (default: the state)."""
        S = self.state.state_spect if state_spect is None else state_spect
        if not isinstance(S, torch.Tensor):
            S = torch.from_numpy(np.ascontiguousarray(S)).to(self.oper.device, self.oper.cdtype)
        if old is None:
            old = torch.empty_like(self.state.state_spect)
        _lib.check(self._lib.gbs_ns_tendencies(
            self._solver, ctypes.c_void_p(S.contiguous().data_ptr()),
            ctypes.c_void_p(old.data_ptr()), current_stream_handle()), "tendencies_nonlin")
        return old

    def max_velocity(self):
        out = (ctypes.c_double * 3)()
        _lib.check(self._lib.gbs_ns_max_velocity(
            self._solver, ctypes.c_void_p(self.state.state_spect.data_ptr()), out,
            current_stream_handle()))
        return list(out)[: self.ndim]


class SimulNS2D(_SimulBase):
    """``fluidsim.solvers.ns2d.solver.Simul`` on GB300 (state: rot_fft)."""

    Operators = OperatorsPseudoSpectral2D
    ndim = 2
    keys_state_spect = ("rot_fft",)
    keys_state_phys = ("ux", "uy", "rot")  # ns2d/state.py:31
    _means_keys = ("E", "Z", "epsK", "epsK_hypo", "epsZ", "epsZ_hypo")

    @staticmethod
    def _complete_params_with_default(params):
        params._set_attribs({"beta": 0.0})

    def _ns_params(self):
        p = super()._ns_params()
        p.beta = self.params.beta
        return p

    def _statephys_from_statespect(self, S):
        """``ns2d/state.py:95-106``: (ux, uy, rot)."""
        rot_fft = S[0]
        ux_fft, uy_fft = self.oper.vecfft_from_rotfft(rot_fft)
        K = torch.stack([ux_fft, uy_fft, rot_fft])
        X = torch.empty((3,) + self.oper.shapeX, dtype=self.oper.rdtype, device=self.oper.device)
        self.oper.opfft.ifft_as_arg_destroy(K, X)
        return X

    def init_from_rotfft(self, rot_fft):
        """``ns2d/state.py:115-119``: dealiased, then state_phys."""
        r = rot_fft if isinstance(rot_fft, torch.Tensor) else torch.from_numpy(np.asarray(rot_fft))
        r = r.to(self.oper.device, self.oper.cdtype).clone()
        self.oper.dealiasing(r)
        self.state.init_statespect_from(rot_fft=r)


class SimulNS2DStrat(SimulNS2D):
    """``fluidsim.solvers.ns2d.strat.solver.Simul`` on GB300: state
    (rot_fft, b_fft), tendencies ``-u.grad(rot) + d_x b`` and
    ``-u.grad(b) - N^2 u_y`` (``ns2d/strat/solver.py:27-32,143-192``); the
    CFL time is also capped by the dispersion-relation time 2 pi / max(N kx
    / |k|) (``ns2d/strat/time_stepping.py:31-70,158-198``; the optional
    group-velocity cap is not implemented).  Power-of-two grids only."""

    keys_state_spect = ("rot_fft", "b_fft")
    keys_state_phys = ("ux", "uy", "rot", "b")  # ns2d/strat/state.py:31-34
    _means_keys = ("EK", "Z", "epsK", "epsK_hypo", "epsZ", "epsZ_hypo", "EA", "epsA",
                   "epsA_hypo")

    @staticmethod
    def _complete_params_with_default(params):
        SimulNS2D._complete_params_with_default(params)
        params._set_attribs({"N": 1.0})  # ns2d/strat/solver.py:95-99

    def __init__(self, params):
        pts = params.time_stepping
        if getattr(pts, "cfl_coef_group", None):
            raise NotImplementedError("the group-velocity time of ns2d.strat")
        if params.beta:
            raise ValueError("ns2d.strat has no beta term")
        super().__init__(params)

    def _ns_params(self):
        p = super()._ns_params()
        p.strat = 1
        p.N = float(self.params.N)
        return p

    def deltat_cap(self):
        """``time_stepping.py:55-70`` with ``compute_dispersion_relation``
        (``solver.py:215-225``): 2 pi / max(N KX / K_not0)."""
        if not float(self.params.N):
            return np.inf
        o = self.oper
        kx = o.deltakx * np.arange(o.nx // 2 + 1)
        ky = o.deltaky * np.fft.fftfreq(o.ny, 1.0 / o.ny)
        KX, KY = np.meshgrid(kx, ky)
        K2 = KX**2 + KY**2
        K2[0, 0] = 1e-14
        freq = (float(self.params.N) * (KX / np.sqrt(K2))).max()
        return 2.0 * np.pi / freq

    def _statephys_from_statespect(self, S):
        """``ns2d/strat/state.py:137-151``: (ux, uy, rot, b)."""
        rot_fft = S[0]
        ux_fft, uy_fft = self.oper.vecfft_from_rotfft(rot_fft)
        K = torch.stack([ux_fft, uy_fft, rot_fft, S[1]])
        X = torch.empty((4,) + self.oper.shapeX, dtype=self.oper.rdtype, device=self.oper.device)
        self.oper.opfft.ifft_as_arg_destroy(K, X)
        return X

    def init_from_rotbfft(self, rot_fft, b_fft):
        """Dealiased rot and b (``ns2d/strat/init_fields.py``)."""
        fields = []
        for a in (rot_fft, b_fft):
            t = a if isinstance(a, torch.Tensor) else torch.from_numpy(np.asarray(a))
            t = t.to(self.oper.device, self.oper.cdtype).clone()
            self.oper.dealiasing(t)
            fields.append(t)
        self.state.init_statespect_from(rot_fft=fields[0], b_fft=fields[1])


class SimulNS2DBouss(SimulNS2DStrat):
    """``fluidsim.solvers.ns2d.bouss.solver.Simul`` on GB300: Boussinesq
    with the buoyancy along y, tendencies ``-u.grad(rot) + d_x b`` and
    ``-u.grad(b)`` (``ns2d/bouss/solver.py:22-27,60-160``): the ns2d.strat
    equations with N = 0, the plain ns2d time stepping and energy."""

    _means_keys = SimulNS2DStrat._means_keys

    @staticmethod
    def _complete_params_with_default(params):
        SimulNS2D._complete_params_with_default(params)

    def __init__(self, params):
        params._set_attribs({"N": 0.0})
        super().__init__(params)

    def _ns_params(self):
        p = super()._ns_params()
        p.N = 0.0
        p.bouss = 1
        return p


class SimulNS3D(_SimulBase):
    """``fluidsim.solvers.ns3d.solver.Simul`` on GB300 (vx_fft, vy_fft, vz_fft)."""

    Operators = OperatorsPseudoSpectral3D
    ndim = 3
    keys_state_spect = ("vx_fft", "vy_fft", "vz_fft")
    keys_state_phys = ("vx", "vy", "vz")  # ns3d/state.py:20
    _means_keys = ("E", "Ex", "Ey", "Ez", "epsK", "epsK_hypo")

    @staticmethod
    def _complete_params_with_default(params):
        params._set_attribs({"f": None, "no_vz_kz0": False, "projection": None})
        # fluidsim/base/turb_model/base.py:36-70 (+ smagorinsky.py:46-47)
        tm = params._set_child("turb_model", attribs={"enable": False, "type": ""})
        tm._set_child("smagorinsky", attribs={"C": 0.18})

    _PROJECTIONS = {None: 0, "toroidal": 1, "vortical": 1, "poloidal": 2}

    def __init__(self, params):
        if params.projection not in self._PROJECTIONS:
            # ns3d/solver.py:171-174
            raise ValueError("No known projection for params.projection = "
                             f"{params.projection}")
        super().__init__(params)
        # ns3d/solver.py:147-175: projection of the tendencies and the state
        _lib.check(self._lib.gbs_ns_set_projection(
            self._solver, self._PROJECTIONS[params.projection], int(bool(params.no_vz_kz0))),
            "gbs_ns_set_projection")
        self.is_turb_model_enabled = False
        self._closure = None
        if params.forcing.enable:
            from .forcing import CoarseForcing3D
            self.forcing = CoarseForcing3D(self)
            self.is_forcing_enabled = True
        tm = params.turb_model
        if tm.enable:
            if tm.type == "smagorinsky":
                _lib.check(self._lib.gbs_ns_set_turb_model(
                    self._solver, 1, float(tm.smagorinsky.C), None), "turb_model")
                self.is_turb_model_enabled = True
            elif tm.type != "mlp_closure":
                raise ValueError(
                    f"Wrong value ('{tm.type}') of params.turb_model.type. "
                    "It should be in ('smagorinsky', 'mlp_closure')")

    def set_closure(self, closure, precision="fp32"):
        """Use a trained ``fluidsim_gb300.closure.ClosureMLP`` as turb model
        (precision "fp32" or "bf16", as ``closure.predict``)."""
        from .closure import PRECISIONS
        if precision not in PRECISIONS:
            raise ValueError(f"precision {precision!r} not in {PRECISIONS}")
        self._closure = closure  # keeps the device weights alive
        w = closure.c_weights()
        _lib.check(self._lib.gbs_ns_set_turb_model(
            self._solver, 2 if precision == "fp32" else 3, 0.0, ctypes.byref(w)), "turb_model")
        self.is_turb_model_enabled = True

    def _ns_params(self):
        p = super()._ns_params()
        if self.params.f is not None:
            p.has_f = 1
            p.f = float(self.params.f)
        return p

    def _statephys_from_statespect(self, S):
        X = torch.empty((3,) + self.oper.shapeX, dtype=self.oper.rdtype, device=self.oper.device)
        self.oper.opfft.ifft_as_arg(S.contiguous(), X)
        return X

    def init_from_vxvyvzfft(self, vx_fft, vy_fft, vz_fft):
        """``ns3d/state.py:124-130``: set, then phys -> spect round trip."""
        self.state.init_statespect_from(vx_fft=vx_fft, vy_fft=vy_fft, vz_fft=vz_fft)
        X = self.state.state_phys
        self.oper.opfft.fft_as_arg(X.contiguous(), self.state.state_spect)
        self.state._phys = None


class SimulNS3DStrat(SimulNS3D):
    """``fluidsim.solvers.ns3d.strat.solver.Simul`` on GB300: Boussinesq
    equations with a constant Brunt-Vaisala frequency ``params.N``; state
    (vx_fft, vy_fft, vz_fft, b_fft), tendencies
    ``P(v x omega) + b e_z`` and ``-div(v b) - N^2 v_z``
    (``ns3d/strat/solver.py:138-216``).  Power-of-two grids only."""

    keys_state_spect = ("vx_fft", "vy_fft", "vz_fft", "b_fft")
    keys_state_phys = ("vx", "vy", "vz", "b")  # ns3d/strat/state.py:18-24
    _means_keys = ("EK", "EKx", "EKy", "EKz", "epsK", "epsK_hypo", "EA", "epsA",
                   "epsA_hypo")

    @staticmethod
    def _complete_params_with_default(params):
        SimulNS3D._complete_params_with_default(params)
        params._set_attribs({"N": 1.0})  # ns3d/strat/solver.py:124-128

    def _ns_params(self):
        p = super()._ns_params()
        p.strat = 1
        p.N = float(self.params.N)
        return p

    def _statephys_from_statespect(self, S):
        X = torch.empty((4,) + self.oper.shapeX, dtype=self.oper.rdtype, device=self.oper.device)
        self.oper.opfft.ifft_as_arg(S.contiguous(), X)
        return X

    def init_from_vxvyvzfft(self, vx_fft, vy_fft, vz_fft):
        """``ns3d/strat/state.py:26-32``: b = 0, then phys -> spect round trip."""
        self.state.init_statespect_from(vx_fft=vx_fft, vy_fft=vy_fft, vz_fft=vz_fft)
        X = self.state.state_phys
        self.oper.opfft.fft_as_arg(X.contiguous(), self.state.state_spect)
        self.state._phys = None


class SimulNS3DBouss(SimulNS3DStrat):
    """``fluidsim.solvers.ns3d.bouss.solver.Simul`` on GB300: the ns3d.strat
    tendencies without the -N^2 v_z term (``ns3d/bouss/solver.py:48-160``);
    params.N (default 1) only weights the potential energy of the outputs,
    as in the reference, whose bouss solver keeps the strat output."""

    def _ns_params(self):
        p = super()._ns_params()
        p.bouss = 1
        return p
