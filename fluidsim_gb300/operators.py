"""Operators on device arrays with the fluidsim operator-class surface.

``OperatorsPseudoSpectral2D`` / ``OperatorsPseudoSpectral3D`` mirror the
attributes and methods of ``fluidsim/operators/operators2d.py:85-259`` and
``fluidsim/operators/operators3d.py:116-342`` that the ns2d/ns3d hot path
and its outputs use (wavenumber arrays, ``where_dealiased``, ``dealiasing``,
curl / gradient / projection helpers, ``sum_wavenumbers``), over CUDA
tensors.  The transforms go through the GB300 FFT plugin; the fused time
step does not call these helpers (it recomputes k on the fly inside its
kernels), they serve user scripts and outputs.

Wavenumber conventions: ``k_adim = ik`` if ``ik <= n//2`` else ``ik - n``
(``operators3d.py:1196-1199``), x non-negative; cubic truncation removes
``|k_adim| >= kcut`` on any axis, kcut from ``init_fields.cubic_dealias_cutoff``.
"""

from math import pi

import numpy as np
import torch

from .fft import FFT2DGB300, FFT3DGB300, import_fft_class
from .init_fields import cubic_dealias_cutoff
from .params import Parameters


def _kadim(n):
    ik = np.arange(n)
    return np.where(ik <= n // 2, ik, ik - n)


class _OperBase:
    is_sequential = True
    SAME_SIZE_IN_ALL_PROC = True

    def _finish_init(self):
        self._has_to_dealiase = self.coef_dealiasing < 1.0
        mask = np.zeros(self.shapeK, dtype=bool)
        for axis, (n, L, cut) in enumerate(zip(self.shapeX, self._lengths, self.kcut)):
            ks = np.abs(_kadim(n)) if axis < self.ndim - 1 else np.arange(n // 2 + 1)
            shape = [1] * self.ndim
            shape[axis] = -1
            mask = mask | (ks >= cut).reshape(shape)
        self._where_dealiased_np = mask.astype(np.uint8)
        self.where_dealiased = torch.from_numpy(self._where_dealiased_np).to(self.device)
        self._keep = (self.where_dealiased == 0).to(self.rdtype)

    # ----- transforms (fluidfft operator API) -----
    def fft(self, fieldX):
        return self.opfft.fft(fieldX)

    def ifft(self, fieldK):
        return self.opfft.ifft(fieldK)

    def fft_as_arg(self, fieldX, fieldK):
        return self.opfft.fft_as_arg(fieldX, fieldK)

    def ifft_as_arg(self, fieldK, fieldX):
        return self.opfft.ifft_as_arg(fieldK, fieldX)

    def ifft_as_arg_destroy(self, fieldK, fieldX):
        return self.opfft.ifft_as_arg_destroy(fieldK, fieldX)

    def create_arrayX(self, value=None, shape="loc"):
        return self.opfft.create_arrayX(value)

    def create_arrayK(self, value=None, shape="loc"):
        return self.opfft.create_arrayK(value)

    def get_shapeX_loc(self):
        return self.shapeX

    def get_shapeK_loc(self):
        return self.shapeK

    def get_k_adim_loc(self):
        return self.opfft.get_k_adim_loc()

    def sum_wavenumbers(self, arrK):
        return self.opfft.sum_wavenumbers(arrK)

    def mean_space(self, arr):
        return float(arr.to(torch.float64).mean()) if isinstance(arr, torch.Tensor) else float(np.mean(arr))

    # ----- dealiasing (operators3d.py:336-342, operators2d.py:200-220) -----
    def dealiasing_variable(self, ff_fft):
        if self._has_to_dealiase:
            ff_fft.mul_(self._keep)

    def dealiasing_setofvar(self, sov):
        if self._has_to_dealiase:
            sov.mul_(self._keep)

    def dealiasing(self, *args):
        for thing in args:
            if isinstance(thing, torch.Tensor):
                if self._has_to_dealiase:
                    thing.mul_(self._keep)
            else:
                arr = np.asarray(thing)
                if self._has_to_dealiase:
                    arr[..., self._where_dealiased_np.astype(bool)] = 0.0


    # ----- spectra (FP64 accumulation on the device) -----
    # Definitions from the mathematics (fluidfft's own binning is not
    # available to compare against): an energy array over the half spectrum
    # (x non-negative) is summed with the Hermitian weights (x modes other
    # than 0 and nx/2 count twice) and divided by the bin width; a mode goes
    # to bin round(|k| / dk).
    def _deltak(self):
        return (self.deltakx, self.deltaky, getattr(self, "deltakz", 1.0))[: self.ndim]

    def _spectra(self, energy_fft, kx=False, ky=False, kz=False, shell=False, kzkh=False):
        """FP64 spectra of ``energy_fft`` (real, shapeK) by the ``gbs_spectra``
        kernel; returns the requested outputs, in (kx, ky, kz, shell, kzkh)
        order, as float64 device tensors."""
        import ctypes

        from . import _lib
        from .fft import current_stream_handle
        e = energy_fft if isinstance(energy_fft, torch.Tensor) else torch.from_numpy(
            np.ascontiguousarray(energy_fft))
        e = e.to(self.device)
        if e.dtype not in (torch.float32, torch.float64):
            e = e.to(torch.float64)
        e = e.contiguous()
        if tuple(e.shape) != tuple(self.shapeK):
            raise ValueError(f"energy array of shape {tuple(e.shape)}, expected {self.shapeK}")
        lib = self.opfft._lib
        shape = (ctypes.c_int64 * self.ndim)(*self.shapeX)
        dk = (ctypes.c_double * self.ndim)(*self._deltak())
        sizes = (ctypes.c_int64 * 5)()
        _lib.check(lib.gbs_spectra_sizes(self.ndim, shape, dk, sizes), "spectra")
        want = (kx, ky, kz, shell, kzkh)
        lens = (sizes[0], sizes[1], sizes[2], sizes[3], sizes[2] * sizes[4])
        outs = [torch.empty(n, dtype=torch.float64, device=self.device) if w else None
                for w, n in zip(want, lens)]
        ptrs = [ctypes.c_void_p(o.data_ptr()) if o is not None else None for o in outs]
        dtype = _lib.GBS_F64 if e.dtype == torch.float64 else _lib.GBS_F32
        with torch.cuda.device(self.device):
            _lib.check(lib.gbs_spectra(self.ndim, shape, dk, dtype, ctypes.c_void_p(e.data_ptr()),
                                       *ptrs, current_stream_handle()), "spectra")
        if kzkh:
            outs[4] = outs[4].reshape(int(sizes[2]), int(sizes[4]))
        return [o for o in outs if o is not None]

    def create_arrayX_random(self, min_val=None, max_val=None, shape="loc"):
        """Uniform random real array (``min_val`` 0, ``max_val`` 1 by default)."""
        lo = 0.0 if min_val is None else float(min_val)
        hi = 1.0 if max_val is None else float(max_val)
        return lo + (hi - lo) * torch.rand(self.shapeX, dtype=self.rdtype, device=self.device)

    def create_arrayK_random(self, min_val=None, max_val=None, shape="loc"):
        """Complex array with uniform random real and imaginary parts."""
        lo = 0.0 if min_val is None else float(min_val)
        hi = 1.0 if max_val is None else float(max_val)
        re = lo + (hi - lo) * torch.rand(self.shapeK, dtype=self.rdtype, device=self.device)
        im = lo + (hi - lo) * torch.rand(self.shapeK, dtype=self.rdtype, device=self.device)
        return torch.complex(re, im)


class OperatorsPseudoSpectral2D(_OperBase):
    ndim = 2

    @staticmethod
    def _complete_params_with_default(params):
        """Same defaults as ``operators2d.py:100-112``."""
        params._set_child("oper", attribs={
            "type_fft": "default", "coef_dealiasing": 2.0 / 3, "nx": 48, "ny": 48,
            "Lx": 8, "Ly": 8, "truncation_shape": "cubic", "NO_SHEAR_MODES": False,
            "NO_KY0": False})

    def __init__(self, params, precision="float64", device=None):
        self.params = params
        po = params.oper
        if po.truncation_shape != "cubic" or po.NO_SHEAR_MODES or po.NO_KY0:
            raise NotImplementedError("only the cubic truncation is implemented on GB300")
        self.nx, self.ny = int(po.nx), int(po.ny)
        self.Lx = self.lx = float(po.Lx)
        self.Ly = self.ly = float(po.Ly)
        self.coef_dealiasing = po.coef_dealiasing
        cls = import_fft_class(po.type_fft, 2)
        self.opfft = self.oper_fft = cls(self.ny, self.nx, precision=precision, device=device)
        self.device = self.opfft.device
        self.rdtype, self.cdtype = self.opfft.rdtype, self.opfft.cdtype
        self.shapeX = self.shapeX_seq = self.shapeX_loc = (self.ny, self.nx)
        self.shapeK = self.shapeK_seq = self.shapeK_loc = (self.ny, self.nx // 2 + 1)
        self.deltax, self.deltay = self.Lx / self.nx, self.Ly / self.ny
        self.deltakx, self.deltaky = 2 * pi / self.Lx, 2 * pi / self.Ly
        self._lengths = (self.Ly, self.Lx)
        self.kcut = (cubic_dealias_cutoff(self.ny, self.Ly, self.coef_dealiasing),
                     cubic_dealias_cutoff(self.nx, self.Lx, self.coef_dealiasing))
        kx = torch.tensor(self.deltakx * np.arange(self.nx // 2 + 1), dtype=self.rdtype,
                          device=self.device)
        ky = torch.tensor(self.deltaky * _kadim(self.ny), dtype=self.rdtype, device=self.device)
        self.kx, self.ky = kx, ky
        self.KX = kx[None, :].expand(self.shapeK)
        self.KY = ky[:, None].expand(self.shapeK)
        self.K2 = self.KX**2 + self.KY**2
        self.K4 = self.K2**2
        self.K8 = self.K4**2
        self.K2_not0 = self.K2.clone()
        self.K2_not0[0, 0] = 1e-14
        self.inv_K_square_nozero = 1.0 / self.K2_not0
        self.inv_K_square_nozero[0, 0] = 0.0
        self.K_not0 = torch.sqrt(self.K2_not0)
        x = torch.arange(self.nx, dtype=torch.float64) * self.deltax
        y = torch.arange(self.ny, dtype=torch.float64) * self.deltay
        self.x = self.x_seq = self.x_loc = x
        self.y = self.y_seq = self.y_loc = y
        self._finish_init()

    def vecfft_from_rotfft(self, rot_fft):
        ux = 1j * self.KY * self.inv_K_square_nozero * rot_fft
        uy = -1j * self.KX * self.inv_K_square_nozero * rot_fft
        return ux, uy

    def rotfft_from_vecfft(self, vecx_fft, vecy_fft):
        return 1j * (self.KX * vecy_fft - self.KY * vecx_fft)

    def divfft_from_vecfft(self, vecx_fft, vecy_fft):
        return 1j * (self.KX * vecx_fft + self.KY * vecy_fft)

    def gradfft_from_fft(self, f_fft):
        return 1j * self.KX * f_fft, 1j * self.KY * f_fft

    def laplacian_fft(self, a_fft, order=2):
        return a_fft * self.K2 ** (order // 2)

    def invlaplacian_fft(self, a_fft, order=2):
        r = a_fft / self.K2_not0 ** (order // 2)
        r[0, 0] = 0.0
        return r

    def get_XY_loc(self):
        Y, X = torch.meshgrid(self.y, self.x, indexing="ij")
        return X, Y

    def projection_perp(self, fx_fft, fy_fft):
        """In place: remove the part of (fx, fy) parallel to k (k = 0 kept)."""
        tmp = (self.KX * fx_fft + self.KY * fy_fft) * self.inv_K_square_nozero
        fx_fft.sub_(self.KX * tmp)
        fy_fft.sub_(self.KY * tmp)

    def compute_1dspectra(self, energy_fft):
        """(E(kx), E(ky)) of an energy array: Hermitian-weighted sums over the
        other axis, |ky| binned, divided by the bin width (FP64)."""
        return tuple(self._spectra(energy_fft, kx=True, ky=True))

    def compute_2dspectrum(self, energy_fft):
        """Shell-summed spectrum, bins floor(|k| / dk + 0.5), dk = min(dkx, dky)."""
        return self._spectra(energy_fft, shell=True)[0]

    # names fluidsim's ns2d outputs bind (fluidsim/base/output/spectra.py:373-374)
    spectra1D_from_fft = compute_1dspectra
    spectrum2D_from_fft = compute_2dspectrum

    def produce_str_describing_oper(self):
        return f"{self.nx}x{self.ny}"


class OperatorsPseudoSpectral3D(_OperBase):
    ndim = 3

    @staticmethod
    def _complete_params_with_default(params):
        """Same defaults as ``operators3d.py:152-168``."""
        params._set_child("oper", attribs={
            "type_fft": "default", "type_fft2d": "sequential", "coef_dealiasing": 2.0 / 3,
            "nx": 48, "ny": 48, "nz": 48, "Lx": 2 * pi, "Ly": 2 * pi, "Lz": 2 * pi,
            "truncation_shape": "cubic", "NO_SHEAR_MODES": False})

    def __init__(self, params, precision="float64", device=None):
        self.params = params
        po = params.oper
        if po.truncation_shape != "cubic" or po.NO_SHEAR_MODES:
            raise NotImplementedError("only the cubic truncation is implemented on GB300")
        self.axes = ("z", "y", "x")
        self.nx, self.ny, self.nz = int(po.nx), int(po.ny), int(po.nz)
        self.Lx, self.Ly, self.Lz = float(po.Lx), float(po.Ly), float(po.Lz)
        self.coef_dealiasing = po.coef_dealiasing
        cls = import_fft_class(po.type_fft, 3)
        self.opfft = self.oper_fft = cls(self.nz, self.ny, self.nx, precision=precision,
                                         device=device)
        self.device = self.opfft.device
        self.rdtype, self.cdtype = self.opfft.rdtype, self.opfft.cdtype
        self.shapeX = self.shapeX_seq = self.shapeX_loc = (self.nz, self.ny, self.nx)
        self.shapeK = self.shapeK_seq = self.shapeK_loc = (self.nz, self.ny, self.nx // 2 + 1)
        self.seq_indices_first_K = (0, 0, 0)
        self.dimX_K = (0, 1, 2)
        self.deltax, self.deltay, self.deltaz = (self.Lx / self.nx, self.Ly / self.ny,
                                                 self.Lz / self.nz)
        self.deltakx, self.deltaky, self.deltakz = (2 * pi / self.Lx, 2 * pi / self.Ly,
                                                    2 * pi / self.Lz)
        self._lengths = (self.Lz, self.Ly, self.Lx)
        self.kcut = (cubic_dealias_cutoff(self.nz, self.Lz, self.coef_dealiasing),
                     cubic_dealias_cutoff(self.ny, self.Ly, self.coef_dealiasing),
                     cubic_dealias_cutoff(self.nx, self.Lx, self.coef_dealiasing))
        dev, rd = self.device, self.rdtype
        self.kx = torch.tensor(self.deltakx * np.arange(self.nx // 2 + 1), dtype=rd, device=dev)
        self.ky = torch.tensor(self.deltaky * _kadim(self.ny), dtype=rd, device=dev)
        self.kz = torch.tensor(self.deltakz * _kadim(self.nz), dtype=rd, device=dev)
        self.Kx = self.kx[None, None, :].expand(self.shapeK)
        self.Ky = self.ky[None, :, None].expand(self.shapeK)
        self.Kz = self.kz[:, None, None].expand(self.shapeK)
        self._finish_init()

    # full-size arrays are built on demand (a 512^3 float64 K2 is 0.5 GB)
    @property
    def K2(self):
        return self.Kx**2 + self.Ky**2 + self.Kz**2

    @property
    def K4(self):
        return self.K2**2

    @property
    def K8(self):
        return self.K4**2

    @property
    def K2_not0(self):
        K2 = self.K2
        K2[0, 0, 0] = 1e-14
        return K2

    @property
    def inv_K_square_nozero(self):
        return 1.0 / self.K2_not0

    def rotfft_from_vecfft(self, vx_fft, vy_fft, vz_fft):
        return (1j * (self.Ky * vz_fft - self.Kz * vy_fft),
                1j * (self.Kz * vx_fft - self.Kx * vz_fft),
                1j * (self.Kx * vy_fft - self.Ky * vx_fft))

    def rotfft_from_vecfft_outin(self, vx_fft, vy_fft, vz_fft, rx, ry, rz):
        ox, oy, oz = self.rotfft_from_vecfft(vx_fft, vy_fft, vz_fft)
        rx.copy_(ox)
        ry.copy_(oy)
        rz.copy_(oz)

    def divfft_from_vecfft(self, vx_fft, vy_fft, vz_fft):
        return 1j * (self.Kx * vx_fft + self.Ky * vy_fft + self.Kz * vz_fft)

    def gradfft_from_fft(self, f_fft):
        return 1j * self.Kx * f_fft, 1j * self.Ky * f_fft, 1j * self.Kz * f_fft

    def get_XYZ_loc(self):
        z = torch.arange(self.nz, dtype=torch.float64, device=self.device) * self.deltaz
        y = torch.arange(self.ny, dtype=torch.float64, device=self.device) * self.deltay
        x = torch.arange(self.nx, dtype=torch.float64, device=self.device) * self.deltax
        Z, Y, X = torch.meshgrid(z, y, x, indexing="ij")
        return X, Y, Z

    @staticmethod
    def vector_product(ax, ay, az, bx, by, bz):
        """a x b of physical fields."""
        return ay * bz - az * by, az * bx - ax * bz, ax * by - ay * bx

    def urudfft_from_vxvyfft(self, vx_fft, vy_fft):
        """Toroidal (r) and poloidal (d) horizontal velocities,
        ``operators3d.py:713-730``."""
        kh2 = self.Kx**2 + self.Ky**2
        kh2 = torch.where(kh2 == 0, torch.full_like(kh2, 1e-14), kh2)
        inv = 1.0 / kh2
        kdotu = self.Kx * vx_fft + self.Ky * vy_fft
        udx = kdotu * self.Kx * inv
        udy = kdotu * self.Ky * inv
        return vx_fft - udx, vy_fft - udy, udx, udy

    def build_invariant_arrayX_from_2d_indices12X(self, arr2d, oper2d=None):
        """3D array constant along z from a (ny, nx) array."""
        a = arr2d if isinstance(arr2d, torch.Tensor) else torch.from_numpy(np.asarray(arr2d))
        return a.to(self.device).unsqueeze(0).expand((self.nz,) + tuple(a.shape)).contiguous()

    def build_invariant_arrayK_from_2d_indices12X(self, arr2d):
        """Spectral array of a field constant along z: the (ny, nx/2+1)
        spectrum of the 2D field on the kz = 0 plane (the forward transform
        is normalised by the number of points, so the plane carries the 2D
        coefficients unchanged)."""
        a = arr2d if isinstance(arr2d, torch.Tensor) else torch.from_numpy(np.asarray(arr2d))
        out = torch.zeros(self.shapeK, dtype=self.cdtype, device=self.device)
        out[0].copy_(a.to(self.device))
        return out

    def compute_1dspectra(self, energy_fft):
        """(E(kx), E(ky), E(kz)) of an energy array: Hermitian-weighted sums
        over the other axes, |ky| and |kz| binned, divided by the bin width."""
        return tuple(self._spectra(energy_fft, kx=True, ky=True, kz=True))

    def compute_3dspectrum(self, energy_fft):
        """Shell-summed spectrum, bins floor(|k| / dk + 0.5), dk = min(dkx, dky, dkz)."""
        return self._spectra(energy_fft, shell=True)[0]

    def compute_spectrum_kzkh(self, energy_fft):
        """2D spectrum over (|kz|, kh), kh = sqrt(kx^2 + ky^2): rows |kz_adim|,
        columns floor(kh / dkh + 0.5), dkh = min(dkx, dky), divided by
        dkz dkh."""
        return self._spectra(energy_fft, kzkh=True)[0]

    def project_perpk3d(self, vx_fft, vy_fft, vz_fft):
        tmp = (self.Kx * vx_fft + self.Ky * vy_fft + self.Kz * vz_fft) * self.inv_K_square_nozero
        vx_fft.sub_(self.Kx * tmp)
        vy_fft.sub_(self.Ky * tmp)
        vz_fft.sub_(self.Kz * tmp)

    def produce_str_describing_oper(self):
        return f"{self.nx}x{self.ny}x{self.nz}"
