"""Seeded initial conditions for the ns2d / ns3d workloads (host side).

These play the role of fluidsim's ``init_fields`` "in_script" plugins
(``fluidsim/base/init_fields.py:435-443``): they build a complex128 spectral
state on the host, in the sequential fluidfft layout, which is then copied
once to the device.  They are not part of the time step.

All spectra use the forward-normalised convention of the solver
(``fft = rfftn / N``) and Hermitian-weighted sums over the x-halved
spectrum.
"""

from math import pi

import numpy as np


def _kadim(n, halved=False):
    if halved:
        return np.arange(n // 2 + 1)
    ik = np.arange(n)
    return np.where(ik <= n // 2, ik, ik - n)


def _hermitian_weights(nx):
    w = np.full(nx // 2 + 1, 2.0)
    w[0] = 1.0
    if nx % 2 == 0:
        w[-1] = 1.0
    return w


def _symmetrize_plane(plane):
    """Make a ``kx = 0`` (or Nyquist) plane Hermitian: ``P(-k) = conj P(k)``."""
    flipped = plane
    for axis in range(plane.ndim):
        flipped = np.roll(np.flip(flipped, axis=axis), 1, axis=axis)
    return 0.5 * (plane + np.conj(flipped))


def _make_realizable(fk, nx):
    """Hermitian-symmetrise the kx=0 and (even nx) Nyquist planes in place."""
    fk[..., 0] = _symmetrize_plane(fk[..., 0])
    if nx % 2 == 0:
        fk[..., -1] = _symmetrize_plane(fk[..., -1])
    return fk


def cubic_dealias_cutoff(n, length, coef=2.0 / 3):
    """Smallest ``|k_adim|`` removed by the cubic truncation along one axis.

    Mode ``k`` is removed when ``abs(deltak*k) >= coef*deltak*n/2`` (the
    float64 comparison used for fluidsim's truncation shapes,
    ``fluidsim/operators/base.py:56``).  ``coef >= 1`` removes nothing.
    """
    if coef >= 1.0:
        return n
    deltak = 2 * pi / length
    kmax = coef * deltak * n / 2
    for k in range(n + 1):
        if abs(deltak * k) >= kmax:
            return k
    return n


def noise_rot_2d(nx, ny, Lx=2 * pi, Ly=2 * pi, kmin=4.0, kmax=8.0, seed=0,
                 urms=1.0, coef_dealiasing=2.0 / 3):
    """Band-passed Gaussian white-noise vorticity, ``rot_fft`` (ny, nx//2+1).

    White noise is drawn in physical space (``default_rng(seed)``), Fourier
    transformed, restricted to ``kmin <= |k| <= kmax`` and scaled so that
    ``sqrt(<ux^2 + uy^2>) == urms``.
    """
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((ny, nx))
    rot_fft = np.fft.rfft2(w) / (nx * ny)
    KX = (2 * pi / Lx) * _kadim(nx, True)[None, :]
    KY = (2 * pi / Ly) * _kadim(ny)[:, None]
    K2 = KX**2 + KY**2
    kmod = np.sqrt(K2)
    rot_fft[(kmod < kmin) | (kmod > kmax)] = 0.0
    cy = cubic_dealias_cutoff(ny, Ly, coef_dealiasing)
    cx = cubic_dealias_cutoff(nx, Lx, coef_dealiasing)
    rot_fft[(np.abs(_kadim(ny))[:, None] >= cy) | (np.abs(_kadim(nx, True))[None, :] >= cx)] = 0.0
    K2_not0 = K2.copy()
    K2_not0[0, 0] = 1.0
    energy_fft = 0.5 * np.abs(rot_fft) ** 2 / K2_not0
    energy = float((energy_fft * _hermitian_weights(nx)[None, :]).sum())
    if energy > 0:
        rot_fft *= urms / np.sqrt(2 * energy)
    return np.ascontiguousarray(rot_fft)


def taylor_green_3d(nx, ny, nz, Lx=2 * pi, Ly=2 * pi, Lz=2 * pi):
    """``u = sin x cos y cos z, v = -cos x sin y cos z, w = 0`` (spectral).

    Same initial condition as the reference's Taylor-Green example
    (``doc/test_cases/Taylor_Green_vortices/run_simul.py:40-54``).
    """
    x = Lx / nx * np.arange(nx)
    y = Ly / ny * np.arange(ny)
    z = Lz / nz * np.arange(nz)
    Z, Y, X = np.meshgrid(z, y, x, indexing="ij")
    vx = np.sin(X) * np.cos(Y) * np.cos(Z)
    vy = -np.cos(X) * np.sin(Y) * np.cos(Z)
    n = nx * ny * nz
    out = np.zeros((3, nz, ny, nx // 2 + 1), np.complex128)
    out[0] = np.fft.rfftn(vx) / n
    out[1] = np.fft.rfftn(vy) / n
    return out


def isotropic_3d(nx, ny, nz, Lx=2 * pi, Ly=2 * pi, Lz=2 * pi, k0=4.0,
                 energy=0.5, seed=0, coef_dealiasing=2.0 / 3):
    """Solenoidal random-phase velocity with ``E(k) ~ k^4 exp(-2 (k/k0)^2)``.

    Built directly in spectral space: complex Gaussian modes
    (``default_rng(seed)``), projected perpendicular to ``k``, made
    Hermitian on the ``kx = 0`` / Nyquist planes, dealiased, then each
    integer shell is rescaled to the target spectrum and the total energy
    ``sum_k |v_k|^2 / 2`` is set to ``energy``.
    """
    rng = np.random.default_rng(seed)
    nkx = nx // 2 + 1
    shape = (nz, ny, nkx)
    v = rng.standard_normal((3,) + shape) + 1j * rng.standard_normal((3,) + shape)
    kx = (2 * pi / Lx) * _kadim(nx, True)
    ky = (2 * pi / Ly) * _kadim(ny)
    kz = (2 * pi / Lz) * _kadim(nz)
    KX = kx[None, None, :]
    KY = ky[None, :, None]
    KZ = kz[:, None, None]
    K2 = KX**2 + KY**2 + KZ**2
    K2_not0 = K2.copy()
    K2_not0[0, 0, 0] = 1.0
    kdotv = (KX * v[0] + KY * v[1] + KZ * v[2]) / K2_not0
    v[0] -= KX * kdotv
    v[1] -= KY * kdotv
    v[2] -= KZ * kdotv
    for c in range(3):
        _make_realizable(v[c], nx)
    v[:, 0, 0, 0] = 0.0
    cz = cubic_dealias_cutoff(nz, Lz, coef_dealiasing)
    cy = cubic_dealias_cutoff(ny, Ly, coef_dealiasing)
    cx = cubic_dealias_cutoff(nx, Lx, coef_dealiasing)
    mask = ((np.abs(_kadim(nz))[:, None, None] >= cz)
            | (np.abs(_kadim(ny))[None, :, None] >= cy)
            | (np.abs(_kadim(nx, True))[None, None, :] >= cx))
    v[:, mask] = 0.0
    w = _hermitian_weights(nx)[None, None, :]
    kmod = np.sqrt(K2)
    dk = min(2 * pi / Lx, 2 * pi / Ly, 2 * pi / Lz)
    shell = np.floor(kmod / dk + 0.5).astype(np.int64)
    e_mode = 0.5 * (np.abs(v) ** 2).sum(axis=0) * w
    nsh = int(shell.max()) + 1
    e_shell = np.bincount(shell.ravel(), weights=e_mode.ravel(), minlength=nsh)
    ks = dk * np.arange(nsh)
    target = ks**4 * np.exp(-2.0 * (ks / k0) ** 2)
    scale = np.zeros(nsh)
    nz_shell = e_shell > 0
    scale[nz_shell] = np.sqrt(target[nz_shell] / e_shell[nz_shell])
    v *= scale[shell][None]
    e_tot = float((0.5 * (np.abs(v) ** 2).sum(axis=0) * w).sum())
    if e_tot > 0:
        v *= np.sqrt(energy / e_tot)
    return np.ascontiguousarray(v)
