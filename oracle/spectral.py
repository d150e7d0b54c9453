"""numpy / scipy.fft restatement of the fluidfft operator subset (ORACLE).

Test infrastructure only (see ``oracle/__init__.py``).

The reference delegates these operations to fluidfft 0.4.2 (pinned at
``pdm.lock:920-923``; not vendored).  What is restated here is the
mathematics the reference relies on, with the conventions its own code and
tests pin:

* layout, sequential plan: physical ``(nz, ny, nx)`` / ``(ny, nx)``; spectral
  ``(nz, ny, nx//2+1)`` / ``(ny, nx//2+1)``, C order, ``dimX_K == (0, 1, 2)``
  (``fluidsim/operators/test/test_operators3d.py:226-301``,
  ``fluidsim/operators/operators3d.py:1108-1121``);
* index -> adimensional wavenumber: ``ik`` if ``ik <= n//2`` else ``ik - n``;
  non-negative along x only (``fluidsim/operators/operators3d.py:1196-1199``);
* forward transform divided by the number of points, inverse not
  normalised: Parseval check ``sum_wavenumbers(|v_k|^2/2) == mean(v^2)/2``
  (``fluidsim/base/state.py:385-392``);
* Hermitian-weighted sums over the half spectrum (``sum_wavenumbers``);
* cubic 2/3 truncation mask ``where_dealiased`` with the ``>=`` comparison
  against ``coef * deltak * n / 2`` used for the other truncation shapes in
  ``fluidsim/operators/base.py:47-72`` and
  ``fluidsim/operators/operators3d.py:272-280``;
* the ``K2_not0`` convention (``fluidsim/operators/operators3d.py:290-295``).
"""

import os
from concurrent.futures import ThreadPoolExecutor
from math import pi

import numpy as np
import scipy.fft as sfft

WORKERS = os.cpu_count() or 1
_POOL = None


def slabs(n, parts=None):
    """Split ``range(n)`` into at most ``parts`` (default: all host cores)
    contiguous slices."""
    parts = max(1, min(n, parts or WORKERS))
    b = [n * i // parts for i in range(parts + 1)]
    return [slice(b[i], b[i + 1]) for i in range(parts)]


def slab_map(fn, n):
    """Run ``fn(sl)`` over slabs ``sl`` of a leading axis of length ``n`` on
    all host cores (numpy ufuncs release the GIL).  Each element gets the same
    operations as one whole-array expression, so results do not depend on the
    number of slabs."""
    global _POOL
    if WORKERS == 1 or n < 2:
        fn(slice(None))
        return
    if _POOL is None:
        _POOL = ThreadPoolExecutor(WORKERS)
    for _ in _POOL.map(fn, slabs(n)):
        pass


def kadim_from_ik(ik, n):
    """``fluidsim/operators/operators3d.py:1196-1199`` (vectorised)."""
    ik = np.asarray(ik)
    return np.where(ik <= n // 2, ik, ik - n)


def k_adim_seq(n, halved=False):
    """Per-axis integer wavenumbers in storage order."""
    if halved:
        return np.arange(n // 2 + 1)
    return kadim_from_ik(np.arange(n), n)


def dealias_cutoff(n, length, coef):
    """Smallest ``|k_adim|`` removed by the cubic truncation along one axis.

    Mode ``k`` is removed when ``abs(deltak * k) >= coef * deltak * n / 2``
    (same float64 evaluation order as ``fluidsim/operators/base.py:56`` and
    ``operators3d.py:273``).  Returns ``n`` (nothing removed along this
    axis) when ``coef >= 1``, which matches ``_has_to_dealiase`` being false.
    """
    if coef >= 1.0:
        return n
    deltak = 2 * pi / length
    kmax = coef * deltak * n / 2
    for k in range(n + 1):
        if abs(deltak * k) >= kmax:
            return k
    return n


def _rfftn(x):
    return sfft.rfftn(x, workers=WORKERS)


def _irfftn(k, shape):
    return sfft.irfftn(k, s=shape, workers=WORKERS)


class OperNumpy3D:
    """fluidfft ``OperatorsPseudoSpectral3D`` subset used by ns3d."""

    is_sequential = True

    def __init__(self, nx, ny, nz, Lx=2 * pi, Ly=2 * pi, Lz=2 * pi,
                 coef_dealiasing=2.0 / 3, truncation_shape="cubic"):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.axes = ("z", "y", "x")
        self.Lx, self.Ly, self.Lz = float(Lx), float(Ly), float(Lz)
        self.coef_dealiasing = coef_dealiasing
        self.deltax = self.Lx / nx
        self.deltay = self.Ly / ny
        self.deltaz = self.Lz / nz
        self.deltakx = 2 * pi / self.Lx
        self.deltaky = 2 * pi / self.Ly
        self.deltakz = 2 * pi / self.Lz
        self.shapeX = self.shapeX_seq = self.shapeX_loc = (nz, ny, nx)
        self.shapeK = self.shapeK_seq = self.shapeK_loc = (nz, ny, nx // 2 + 1)
        self.seq_indices_first_K = (0, 0, 0)
        self.dimX_K = (0, 1, 2)
        self.npoints = nx * ny * nz

        kx = self.deltakx * k_adim_seq(nx, halved=True)
        ky = self.deltaky * k_adim_seq(ny)
        kz = self.deltakz * k_adim_seq(nz)
        self.kx, self.ky, self.kz = kx, ky, kz
        self.Kx = np.broadcast_to(kx[None, None, :], self.shapeK)
        self.Ky = np.broadcast_to(ky[None, :, None], self.shapeK)
        self.Kz = np.broadcast_to(kz[:, None, None], self.shapeK)
        self.K2 = self.Kx**2 + self.Ky**2 + self.Kz**2
        self.K4 = self.K2**2
        self.K8 = self.K4**2
        self.K2_not0 = np.copy(self.K2)
        self.K2_not0[0, 0, 0] = 1e-14
        self.inv_K_square_nozero = 1.0 / self.K2_not0

        self.kcut = (
            dealias_cutoff(nz, self.Lz, coef_dealiasing),
            dealias_cutoff(ny, self.Ly, coef_dealiasing),
            dealias_cutoff(nx, self.Lx, coef_dealiasing),
        )
        if truncation_shape != "cubic":
            raise NotImplementedError(truncation_shape)
        akz = np.abs(k_adim_seq(nz))[:, None, None]
        aky = np.abs(k_adim_seq(ny))[None, :, None]
        akx = np.abs(k_adim_seq(nx, True))[None, None, :]
        self.where_dealiased = np.array(
            (akx >= self.kcut[2]) | (aky >= self.kcut[1]) | (akz >= self.kcut[0]),
            dtype=np.uint8,
        )
        self._has_to_dealiase = coef_dealiasing < 1.0

    # -- geometry (fluidfft fft3d class API) --------------------------------
    def get_shapeX_loc(self):
        return self.shapeX

    get_shapeX_seq = get_shapeX_loc

    def get_shapeK_loc(self):
        return self.shapeK

    get_shapeK_seq = get_shapeK_loc

    def get_k_adim_loc(self):
        return (k_adim_seq(self.nz), k_adim_seq(self.ny),
                k_adim_seq(self.nx, halved=True))

    def get_dimX_K(self):
        return self.dimX_K

    def get_seq_indices_first_K(self):
        return self.seq_indices_first_K

    # -- transforms -----------------------------------------------------------
    def fft(self, fieldX):
        out = _rfftn(fieldX)

        def norm(sl):
            out[sl] /= self.npoints
        slab_map(norm, out.shape[0])
        return out

    def ifft(self, fieldK):
        out = _irfftn(fieldK, self.shapeX)

        def norm(sl):
            out[sl] *= self.npoints
        slab_map(norm, out.shape[0])
        return out

    def fft_as_arg(self, fieldX, fieldK):
        fieldK[...] = self.fft(fieldX)

    def ifft_as_arg(self, fieldK, fieldX):
        fieldX[...] = self.ifft(fieldK)

    ifft_as_arg_destroy = ifft_as_arg
    fft3d = fft
    ifft3d = ifft

    def create_arrayX(self, value=None):
        a = np.empty(self.shapeX)
        if value is not None:
            a.fill(value)
        return a

    def create_arrayK(self, value=None):
        a = np.empty(self.shapeK, dtype=np.complex128)
        if value is not None:
            a.fill(value)
        return a

    def create_arrayK_random(self, min_val=None, max_val=None):
        """Uniform random complex array drawn with the global ``np.random``:
        real parts, then imaginary parts, each scaled to ``[min_val,
        max_val)`` (defaults 0 and 1).  fluidfft's method is not in the
        reference; this definition is the oracle's and the GPU forcing's."""
        lo = 0.0 if min_val is None else float(min_val)
        hi = 1.0 if max_val is None else float(max_val)
        re = lo + (hi - lo) * np.random.random(self.shapeK)
        im = lo + (hi - lo) * np.random.random(self.shapeK)
        return re + 1j * im

    # -- spectral operators ---------------------------------------------------
    def rotfft_from_vecfft(self, vx, vy, vz):
        out = np.empty((3,) + np.shape(vx), np.complex128)

        def curl(sl):
            Kx, Ky, Kz = self.Kx[sl], self.Ky[sl], self.Kz[sl]
            x, y, z = vx[sl], vy[sl], vz[sl]
            out[0][sl] = 1j * (Ky * z - Kz * y)
            out[1][sl] = 1j * (Kz * x - Kx * z)
            out[2][sl] = 1j * (Kx * y - Ky * x)
        slab_map(curl, out.shape[1])
        return out[0], out[1], out[2]

    def rotfft_from_vecfft_outin(self, vx, vy, vz, rx, ry, rz):
        ox, oy, oz = self.rotfft_from_vecfft(vx, vy, vz)
        rx[...] = ox
        ry[...] = oy
        rz[...] = oz

    def divfft_from_vecfft(self, vx, vy, vz):
        return 1j * (self.Kx * vx + self.Ky * vy + self.Kz * vz)

    def grad_fft_from_arr_fft(self, arr_fft):
        """fluidfft gradient used by ``turb_model/stress_tensor.py:22-26``."""
        return 1j * self.Kx * arr_fft, 1j * self.Ky * arr_fft, 1j * self.Kz * arr_fft

    def project_perpk3d(self, vx, vy, vz):
        """In place ``v -= k (k.v)/|k|^2``; the k=0 mode is unchanged."""
        def proj(sl):
            Kx, Ky, Kz = self.Kx[sl], self.Ky[sl], self.Kz[sl]
            x, y, z = vx[sl], vy[sl], vz[sl]
            tmp = (Kx * x + Ky * y + Kz * z) * self.inv_K_square_nozero[sl]
            x -= Kx * tmp
            y -= Ky * tmp
            z -= Kz * tmp
        slab_map(proj, np.shape(vx)[0])

    def div_vb_fft_from_vb(self, vx, vy, vz, b):
        """Spectral divergence of v b for physical fields (fluidfft's
        ``div_vb_fft_from_vb``, restated from its definition:
        i (kx FFT(vx b) + ky FFT(vy b) + kz FFT(vz b)))."""
        return 1j * (self.Kx * self.fft(vx * b) + self.Ky * self.fft(vy * b)
                     + self.Kz * self.fft(vz * b))

    def project_toroidal(self, vx, vy, vz):
        """In place v = (e_phi . v) e_phi, e_phi = (-sin phi_k, cos phi_k, 0)
        (``fluidsim/operators/operators3d.py:911-959``)."""
        kh2 = self.Kx**2 + self.Ky**2
        kh2 = np.where(kh2 == 0, 1e-14, kh2)
        t = np.sqrt(1.0 / kh2)
        cp, sp = self.Kx * t, self.Ky * t
        tmp = -sp * vx + cp * vy
        vx[...] = -sp * tmp
        vy[...] = cp * tmp
        vz[...] = 0.0

    def project_poloidal(self, vx, vy, vz):
        """In place v = (e_theta . v) e_theta, e_theta = (cos theta cos phi,
        cos theta sin phi, -sin theta) (``operators3d.py:788-855``)."""
        kh2 = self.Kx**2 + self.Ky**2
        k2n = kh2 + self.Kz**2
        kh2n = np.where(kh2 == 0, 1e-14, kh2)
        k2n = np.where(k2n == 0, 1e-14, k2n)
        inv_kh2, inv_k2 = 1.0 / kh2n, 1.0 / k2n
        ct = self.Kz * np.sqrt(inv_k2)
        st = np.sqrt(kh2 * inv_k2)
        cp, sp = self.Kx * np.sqrt(inv_kh2), self.Ky * np.sqrt(inv_kh2)
        tmp = ct * cp * vx + ct * sp * vy - st * vz
        vx[...] = ct * cp * tmp
        vy[...] = ct * sp * tmp
        vz[...] = -st * tmp

    def dealiasing_variable(self, arr):
        if self._has_to_dealiase:
            mask = self.where_dealiased.astype(bool)

            def zero(sl):
                arr[sl][mask[sl]] = 0.0
            slab_map(zero, arr.shape[0])

    def dealiasing(self, *args):
        for thing in args:
            thing = np.asarray(thing)
            if thing.ndim == 4:
                for a in thing:
                    self.dealiasing_variable(a)
            else:
                self.dealiasing_variable(thing)

    # -- reductions -----------------------------------------------------------
    def sum_wavenumbers(self, arr):
        """Sum over the full spectrum from the x-halved array."""
        nx = self.nx
        arr = np.asarray(arr)
        s = arr[..., 0].sum()
        last = nx // 2
        if nx % 2 == 0:
            s += 2 * arr[..., 1:last].sum() + arr[..., last].sum()
        else:
            s += 2 * arr[..., 1:last + 1].sum()
        return float(s)

    def mean_space(self, arr):
        return float(np.mean(arr))

    # -- spectra ------------------------------------------------------------
    # fluidfft's compute_1dspectra / compute_3dspectrum / compute_spectrum_kzkh
    # (called by fluidsim/solvers/ns3d/output/spectra.py:15-100) are not in
    # the reference; restated from their definitions: Hermitian weights over
    # the half spectrum, sums binned by |k_adim| (1D), floor(|k|/dk + 0.5)
    # (shells, dk = min of the deltak) and floor(kh/dkh + 0.5) (kh columns,
    # dkh = min(dkx, dky)), each divided by its bin width.
    def hermitian_weights(self):
        w = np.full(self.shapeK[-1], 2.0)
        w[0] = 1.0
        if self.nx % 2 == 0:
            w[-1] = 1.0
        return w

    def compute_1dspectra(self, energy_fft):
        e = np.asarray(energy_fft, dtype=np.float64) * self.hermitian_weights()
        skx = e.sum(axis=(0, 1)) / self.deltakx
        iky = np.abs(k_adim_seq(self.ny))
        ikz = np.abs(k_adim_seq(self.nz))
        sky = np.bincount(iky, weights=e.sum(axis=(0, 2)), minlength=self.ny // 2 + 1)
        skz = np.bincount(ikz, weights=e.sum(axis=(1, 2)), minlength=self.nz // 2 + 1)
        return skx, sky / self.deltaky, skz / self.deltakz

    def compute_3dspectrum(self, energy_fft):
        dk = min(self.deltakx, self.deltaky, self.deltakz)
        ik = np.floor(np.sqrt(self.K2) / dk + 0.5).astype(np.int64)
        e = np.asarray(energy_fft, dtype=np.float64) * self.hermitian_weights()
        return np.bincount(ik.ravel(), weights=e.ravel(), minlength=int(ik.max()) + 1) / dk

    def compute_spectrum_kzkh(self, energy_fft):
        dkh = min(self.deltakx, self.deltaky)
        kh = np.sqrt(self.Kx**2 + self.Ky**2)
        ih = np.floor(kh / dkh + 0.5).astype(np.int64)
        nkh = int(ih.max()) + 1
        nzb = self.nz // 2 + 1
        iz = np.broadcast_to(np.abs(k_adim_seq(self.nz))[:, None, None], self.shapeK)
        e = np.asarray(energy_fft, dtype=np.float64) * self.hermitian_weights()
        flat = np.bincount((iz * nkh + ih).ravel(), weights=e.ravel(), minlength=nzb * nkh)
        return flat.reshape(nzb, nkh) / (self.deltakz * dkh)


class OperNumpy2D:
    """fluidfft ``OperatorsPseudoSpectral2D`` subset used by ns2d."""

    is_sequential = True

    def __init__(self, nx, ny, Lx=2 * pi, Ly=2 * pi, coef_dealiasing=2.0 / 3,
                 truncation_shape="cubic"):
        self.nx, self.ny = nx, ny
        self.axes = ("y", "x")
        self.Lx, self.Ly = float(Lx), float(Ly)
        self.coef_dealiasing = coef_dealiasing
        self.deltax = self.Lx / nx
        self.deltay = self.Ly / ny
        self.deltakx = 2 * pi / self.Lx
        self.deltaky = 2 * pi / self.Ly
        self.shapeX = self.shapeX_seq = self.shapeX_loc = (ny, nx)
        self.shapeK = self.shapeK_seq = self.shapeK_loc = (ny, nx // 2 + 1)
        self.seq_indices_first_K = (0, 0)
        self.npoints = nx * ny
        kx = self.deltakx * k_adim_seq(nx, halved=True)
        ky = self.deltaky * k_adim_seq(ny)
        self.kx, self.ky = kx, ky
        self.KX = np.broadcast_to(kx[None, :], self.shapeK)
        self.KY = np.broadcast_to(ky[:, None], self.shapeK)
        self.K2 = self.KX**2 + self.KY**2
        self.K4 = self.K2**2
        self.K8 = self.K4**2
        self.K2_not0 = np.copy(self.K2)
        self.K2_not0[0, 0] = 1e-14
        self.K_not0 = np.sqrt(self.K2_not0)  # fluidfft's K_not0 (|k|, 1e-7 at k = 0)
        self.inv_K_square_nozero = 1.0 / self.K2_not0
        self.inv_K_square_nozero[0, 0] = 0.0
        self.kcut = (
            dealias_cutoff(ny, self.Ly, coef_dealiasing),
            dealias_cutoff(nx, self.Lx, coef_dealiasing),
        )
        if truncation_shape != "cubic":
            raise NotImplementedError(truncation_shape)
        aky = np.abs(k_adim_seq(ny))[:, None]
        akx = np.abs(k_adim_seq(nx, True))[None, :]
        self.where_dealiased = np.array(
            (akx >= self.kcut[1]) | (aky >= self.kcut[0]), dtype=np.uint8)
        self._has_to_dealiase = coef_dealiasing < 1.0

    def get_shapeX_loc(self):
        return self.shapeX

    get_shapeX_seq = get_shapeX_loc

    def get_shapeK_loc(self):
        return self.shapeK

    get_shapeK_seq = get_shapeK_loc

    def get_k_adim_loc(self):
        return (k_adim_seq(self.ny), k_adim_seq(self.nx, halved=True))

    def fft(self, fieldX):
        return _rfftn(fieldX) / self.npoints

    def ifft(self, fieldK):
        return _irfftn(fieldK, self.shapeX) * self.npoints

    fft2 = fft
    ifft2 = ifft

    def fft_as_arg(self, fieldX, fieldK):
        fieldK[...] = self.fft(fieldX)

    def ifft_as_arg(self, fieldK, fieldX):
        fieldX[...] = self.ifft(fieldK)

    ifft_as_arg_destroy = ifft_as_arg

    def create_arrayX(self, value=None):
        a = np.empty(self.shapeX)
        if value is not None:
            a.fill(value)
        return a

    def create_arrayK(self, value=None):
        a = np.empty(self.shapeK, dtype=np.complex128)
        if value is not None:
            a.fill(value)
        return a

    def vecfft_from_rotfft(self, rot_fft):
        """``u = (i ky, -i kx) rot / k^2`` with the k=0 mode set to 0."""
        ux = 1j * self.KY * self.inv_K_square_nozero * rot_fft
        uy = -1j * self.KX * self.inv_K_square_nozero * rot_fft
        return ux, uy

    def rotfft_from_vecfft(self, ux_fft, uy_fft):
        return 1j * (self.KX * uy_fft - self.KY * ux_fft)

    def gradfft_from_fft(self, f_fft):
        return 1j * self.KX * f_fft, 1j * self.KY * f_fft

    def dealiasing_variable(self, arr):
        if self._has_to_dealiase:
            arr[self.where_dealiased.astype(bool)] = 0.0

    def dealiasing(self, *args):
        for thing in args:
            thing = np.asarray(thing)
            if thing.ndim == 3:
                for a in thing:
                    self.dealiasing_variable(a)
            else:
                self.dealiasing_variable(thing)

    def sum_wavenumbers(self, arr):
        nx = self.nx
        arr = np.asarray(arr)
        s = arr[..., 0].sum()
        last = nx // 2
        if nx % 2 == 0:
            s += 2 * arr[..., 1:last].sum() + arr[..., last].sum()
        else:
            s += 2 * arr[..., 1:last + 1].sum()
        return float(s)

    def mean_space(self, arr):
        return float(np.mean(arr))

    # fluidfft's spectra1D_from_fft / spectrum2D_from_fft (bound at
    # fluidsim/base/output/spectra.py:373-374), restated as in the 3D case
    def hermitian_weights(self):
        w = np.full(self.shapeK[-1], 2.0)
        w[0] = 1.0
        if self.nx % 2 == 0:
            w[-1] = 1.0
        return w

    def compute_1dspectra(self, energy_fft):
        e = np.asarray(energy_fft, dtype=np.float64) * self.hermitian_weights()
        iky = np.abs(k_adim_seq(self.ny))
        sky = np.bincount(iky, weights=e.sum(axis=1), minlength=self.ny // 2 + 1)
        return e.sum(axis=0) / self.deltakx, sky / self.deltaky

    def compute_2dspectrum(self, energy_fft):
        dk = min(self.deltakx, self.deltaky)
        ik = np.floor(np.sqrt(self.K2) / dk + 0.5).astype(np.int64)
        e = np.asarray(energy_fft, dtype=np.float64) * self.hermitian_weights()
        return np.bincount(ik.ravel(), weights=e.ravel(), minlength=int(ik.max()) + 1) / dk

    spectra1D_from_fft = compute_1dspectra
    spectrum2D_from_fft = compute_2dspectrum
