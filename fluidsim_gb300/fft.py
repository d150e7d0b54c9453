"""fluidfft-compatible FFT classes backed by libgbspec (GB300, sm_103a).

``FFT2DGB300(n0, n1)`` and ``FFT3DGB300(n0, n1, n2)`` present the fluidfft
``fft2d`` / ``fft3d`` class API used by fluidsim (constructor with the
physical shape in C order, ``fft_as_arg``, ``ifft_as_arg``,
``ifft_as_arg_destroy``, ``fft``, ``ifft``, ``get_shapeX_loc`` ...,
``get_k_adim_loc``, ``sum_wavenumbers``; fluidfft 0.4.2, selected by
``params.oper.type_fft`` at ``fluidsim/operators/operators3d.py:222-231``).

Arrays are CUDA ``torch.Tensor`` (zero copy) or numpy arrays (copied to the
device and back).  Layout: physical ``shapeX`` real, spectral
``shapeX[:-1] + (nx//2+1,)`` complex, sequential (``dimX_K == (0, 1, 2)``),
forward transform divided by the number of points.
"""

import ctypes

import numpy as np
import torch

from . import _lib

_PRECISIONS = {
    "float64": (torch.float64, torch.complex128, _lib.GBS_F64),
    "float32": (torch.float32, torch.complex64, _lib.GBS_F32),
}


def current_stream_handle():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _kadim(n):
    ik = np.arange(n)
    return np.where(ik <= n // 2, ik, ik - n)


class _FFTGB300:
    ndim = None

    def __init__(self, *shapeX, precision="float64", device=None):
        if len(shapeX) != self.ndim:
            raise ValueError(f"expected {self.ndim} sizes, got {shapeX}")
        if precision not in _PRECISIONS:
            raise ValueError(f"precision must be one of {list(_PRECISIONS)}")
        self._lib = _lib.load()
        if not torch.cuda.is_available():
            raise RuntimeError("a CUDA device is required (no CPU fallback)")
        self.shapeX = tuple(int(n) for n in shapeX)
        nx = self.shapeX[-1]
        if nx % 2:
            raise ValueError("nx (last axis) must be even")
        self.shapeK = self.shapeX[:-1] + (nx // 2 + 1,)
        self.precision = precision
        self.rdtype, self.cdtype, self._code = _PRECISIONS[precision]
        self.device = torch.device(device) if device is not None else torch.device(
            "cuda", torch.cuda.current_device())
        self.npoints = int(np.prod(self.shapeX))
        self._plans = {}
        self._plan(1)

    # ------------------------------------------------------------- plans
    def _plan(self, batch):
        plan = self._plans.get(batch)
        if plan is None:
            shape = (ctypes.c_int64 * self.ndim)(*self.shapeX)
            handle = ctypes.c_void_p()
            with torch.cuda.device(self.device):
                _lib.check(self._lib.gbs_fft_plan_create(
                    self.ndim, shape, self._code, batch, ctypes.byref(handle)),
                    "gbs_fft_plan_create")
            plan = self._plans[batch] = handle
        return plan

    def __del__(self):
        lib = getattr(self, "_lib", None)
        for handle in getattr(self, "_plans", {}).values():
            if lib is not None and handle:
                lib.gbs_fft_plan_destroy(handle)
        self._plans = {}

    # ---------------------------------------------------------- geometry
    def get_short_name(self):
        return self.__class__.__name__.lower()

    def get_shapeX_loc(self):
        return self.shapeX

    def get_shapeX_seq(self):
        return self.shapeX

    def get_shapeK_loc(self):
        return self.shapeK

    def get_shapeK_seq(self):
        return self.shapeK

    def get_local_size_X(self):
        return self.npoints

    def get_dimX_K(self):
        return tuple(range(self.ndim))

    def get_seq_indices_first_K(self):
        return (0,) * self.ndim

    def get_seq_indices_first_X(self):
        return (0,) * self.ndim

    def get_is_transposed(self):
        return False

    def get_k_adim_loc(self):
        """Integer wavenumbers per spectral axis (x non-negative)."""
        ks = [_kadim(n) for n in self.shapeX[:-1]]
        ks.append(np.arange(self.shapeX[-1] // 2 + 1))
        return tuple(ks)

    def create_arrayX(self, value=None, shape="loc"):
        a = torch.empty(self.shapeX, dtype=self.rdtype, device=self.device)
        if value is not None:
            a.fill_(value)
        return a

    def create_arrayK(self, value=None, shape="loc"):
        a = torch.empty(self.shapeK, dtype=self.cdtype, device=self.device)
        if value is not None:
            a.fill_(value)
        return a

    def gather_Xspace(self, ff, root=None):
        return ff

    def scatter_Xspace(self, ff_seq, root=None):
        return ff_seq

    # -------------------------------------------------------- transforms
    def _check(self, t, shape, dtype, name):
        if t.shape[-len(shape):] != torch.Size(shape) or t.dtype != dtype:
            raise ValueError(
                f"{name}: expected (..., {shape}) {dtype}, got {tuple(t.shape)} {t.dtype}")
        if not t.is_contiguous():
            raise ValueError(f"{name} must be C-contiguous")
        if t.device != self.device:
            raise ValueError(f"{name} must live on {self.device}")
        batch = int(np.prod(t.shape[:-len(shape)])) if t.dim() > len(shape) else 1
        return batch

    def _to_device(self, arr, dtype):
        if isinstance(arr, torch.Tensor):
            return arr, False
        a = np.ascontiguousarray(arr)
        return torch.from_numpy(a).to(self.device, dtype), True

    def fft_as_arg(self, fieldX, fieldK):
        """fieldK[...] = rfftn(fieldX) / N."""
        x, xh = self._to_device(fieldX, self.rdtype)
        k, kh = (fieldK, False) if isinstance(fieldK, torch.Tensor) else (
            torch.empty(np.shape(fieldK), dtype=self.cdtype, device=self.device), True)
        batch = self._check(x, self.shapeX, self.rdtype, "fieldX")
        if self._check(k, self.shapeK, self.cdtype, "fieldK") != batch:
            raise ValueError("fieldX and fieldK hold different numbers of fields")
        with torch.cuda.device(self.device):
            _lib.check(self._lib.gbs_fft_r2c(self._plan(batch), ctypes.c_void_p(x.data_ptr()),
                                             ctypes.c_void_p(k.data_ptr()),
                                             current_stream_handle()), "fft")
        if kh:
            np.copyto(fieldK, k.cpu().numpy())
        return fieldK

    def _c2r(self, fieldK, fieldX, destroy):
        k, kh = self._to_device(fieldK, self.cdtype)
        x, xh = (fieldX, False) if isinstance(fieldX, torch.Tensor) else (
            torch.empty(np.shape(fieldX), dtype=self.rdtype, device=self.device), True)
        batch = self._check(k, self.shapeK, self.cdtype, "fieldK")
        if self._check(x, self.shapeX, self.rdtype, "fieldX") != batch:
            raise ValueError("fieldX and fieldK hold different numbers of fields")
        with torch.cuda.device(self.device):
            _lib.check(self._lib.gbs_fft_c2r(self._plan(batch), ctypes.c_void_p(k.data_ptr()),
                                             ctypes.c_void_p(x.data_ptr()), int(destroy),
                                             current_stream_handle()), "ifft")
        if xh:
            np.copyto(fieldX, x.cpu().numpy())
        return fieldX

    def ifft_as_arg(self, fieldK, fieldX):
        """fieldX[...] = irfftn(fieldK) * N; fieldK is preserved."""
        return self._c2r(fieldK, fieldX, False)

    def ifft_as_arg_destroy(self, fieldK, fieldX):
        """Same as ``ifft_as_arg`` but fieldK may be overwritten."""
        return self._c2r(fieldK, fieldX, True)

    def fft(self, fieldX):
        host = not isinstance(fieldX, torch.Tensor)
        x, _ = self._to_device(fieldX, self.rdtype)
        k = torch.empty(x.shape[:-self.ndim] + self.shapeK, dtype=self.cdtype,
                        device=self.device)
        self.fft_as_arg(x, k)
        return k.cpu().numpy() if host else k

    def ifft(self, fieldK):
        host = not isinstance(fieldK, torch.Tensor)
        k, _ = self._to_device(fieldK, self.cdtype)
        x = torch.empty(k.shape[:-self.ndim] + self.shapeX, dtype=self.rdtype,
                        device=self.device)
        self.ifft_as_arg(k, x)
        return x.cpu().numpy() if host else x

    # -------------------------------------------------------- reductions
    def sum_wavenumbers(self, arrK):
        """Sum over the full spectrum of a real array of shapeK (FP64)."""
        a = arrK if isinstance(arrK, torch.Tensor) else torch.from_numpy(np.asarray(arrK))
        a = a.to(torch.float64)
        nx = self.shapeX[-1]
        last = nx // 2
        s = a[..., 0].sum() + 2 * a[..., 1:last].sum() + a[..., last].sum()
        return float(s)

    def compute_energy_from_X(self, fieldX):
        x = fieldX if isinstance(fieldX, torch.Tensor) else torch.from_numpy(np.asarray(fieldX))
        return float((x.to(torch.float64) ** 2).mean() / 2)

    def compute_energy_from_K(self, fieldK):
        k = fieldK if isinstance(fieldK, torch.Tensor) else torch.from_numpy(np.asarray(fieldK))
        return self.sum_wavenumbers(k.abs().to(torch.float64) ** 2 / 2)


class FFT2DGB300(_FFTGB300):
    """``fluidfft.fft2d`` plugin class: ``FFT2DGB300(ny, nx)``."""

    ndim = 2


class FFT3DGB300(_FFTGB300):
    """``fluidfft.fft3d`` plugin class: ``FFT3DGB300(nz, ny, nx)``."""

    ndim = 3


# fluidfft method name -> plugin module (the `fluidfft.plugins` entry points
# that pyproject.toml declares)
PLUGIN_MODULES = {
    "fft2d.with_gb300": "fluidsim_gb300.plugins.fft2d_with_gb300",
    "fft3d.with_gb300": "fluidsim_gb300.plugins.fft3d_with_gb300",
}


def import_fft_class(name, dim=None):
    """Resolve a ``params.oper.type_fft`` string to an FFT class, as
    fluidfft's ``import_fft_class`` does for a plugin: strip a leading
    ``fluidfft.``, import the module the method's entry point names and
    return its ``FFTclass``.  ``"default"``/``"sequential"``/``"gb300"``
    select this plugin's class of dimension ``dim``."""
    import importlib
    if name in (None, "default", "sequential", "gb300", "with_gb300"):
        if dim is None:
            raise ValueError("dim is required for the default FFT class")
        name = "fft2d.with_gb300" if dim == 2 else "fft3d.with_gb300"
    method = name[len("fluidfft."):] if name.startswith("fluidfft.") else name
    try:
        module = PLUGIN_MODULES[method]
    except KeyError:
        raise ValueError(f"unknown FFT class {name!r} (this plugin provides "
                         f"{sorted(PLUGIN_MODULES)})") from None
    return importlib.import_module(module).FFTclass
