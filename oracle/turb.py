"""Turbulence-model forcings for the ns3d tendencies (ORACLE).

Test infrastructure only (see ``oracle/__init__.py``).

* ``smagorinsky_forcing``: ``fluidsim/base/turb_model/smagorinsky.py:56-110``
  with ``stress_tensor.py:28-43`` (float64, same expression order, including
  the ``2j`` factor of the reference's divergence).
* ``MLPClosure``: the learned subgrid-stress closure, a pointwise MLP
  9 -> 64 -> 64 -> 6 (tanh) on the velocity-gradient tensor
  ``g[3*i + j] = d_j u_i`` giving the symmetric stress
  ``tau = (xx, yy, zz, xy, xz, yz)``; its forcing is ``-d_j tau_ij``.
  Forward and backward in float64 numpy, used to check the GPU kernels'
  outputs and gradients.  The training loss may add a term on the
  pointwise subgrid dissipation ``tau_ij S_ij`` (no reference counterpart).
"""

from math import sqrt

import numpy as np

TAU_INDEX = ((0, 3, 4), (3, 1, 5), (4, 5, 2))  # tau_ij -> component of (xx,yy,zz,xy,xz,yz)


def grad_phys(oper, v_fft):
    """9 physical gradient fields g[3*i + j] = d_j u_i."""
    out = []
    for i in range(3):
        for gk in oper.grad_fft_from_arr_fft(v_fft[i]):
            out.append(oper.ifft(gk))
    return np.array(out)


def smagorinsky_forcing(oper, vx_fft, vy_fft, vz_fft, C=0.18, Lx=None, nx=None):
    Lx = oper.Lx if Lx is None else Lx
    nx = oper.nx if nx is None else nx
    C_nu_T = C * (Lx / nx) ** 2 * sqrt(2)
    g = grad_phys(oper, (vx_fft, vy_fft, vz_fft))
    dx_ux, dy_ux, dz_ux, dx_uy, dy_uy, dz_uy, dx_uz, dy_uz, dz_uz = g
    Sxx, Syy, Szz = dx_ux, dy_uy, dz_uz
    Syx = 0.5 * (dy_ux + dx_uy)
    Szx = 0.5 * (dz_ux + dx_uz)
    Szy = 0.5 * (dz_uy + dy_uz)
    norm = np.sqrt(Sxx**2 + Syy**2 + Szz**2 + 2 * (Syx**2 + Szx**2 + Szy**2))
    nu_T_2 = 2 * C_nu_T * norm
    fft = oper.fft
    t_xx, t_yy, t_zz = fft(nu_T_2 * Sxx), fft(nu_T_2 * Syy), fft(nu_T_2 * Szz)
    t_yx, t_zx, t_zy = fft(nu_T_2 * Syx), fft(nu_T_2 * Szx), fft(nu_T_2 * Szy)
    Kx, Ky, Kz = oper.Kx, oper.Ky, oper.Kz
    fx = 2j * (Kx * t_xx + Ky * t_yx + Kz * t_zx)
    fy = 2j * (Kx * t_yx + Ky * t_yy + Kz * t_zy)
    fz = 2j * (Kx * t_zx + Ky * t_zy + Kz * t_zz)
    return np.array([fx, fy, fz])


class MLPClosure:
    """float64 reference of the 9 -> 64 -> 64 -> 6 tanh MLP."""

    def __init__(self, W1, b1, W2, b2, W3, b3, in_scale, out_scale):
        # W: (out, in) row-major, like the device layout
        self.W1, self.b1 = np.asarray(W1, float), np.asarray(b1, float)
        self.W2, self.b2 = np.asarray(W2, float), np.asarray(b2, float)
        self.W3, self.b3 = np.asarray(W3, float), np.asarray(b3, float)
        self.in_scale = np.asarray(in_scale, float)
        self.out_scale = np.asarray(out_scale, float)

    def forward(self, g, keep=False):
        """g: (npts, 9) physical gradients -> tau (npts, 6)."""
        x = g * self.in_scale
        z1 = x @ self.W1.T + self.b1
        h1 = np.tanh(z1)
        z2 = h1 @ self.W2.T + self.b2
        h2 = np.tanh(z2)
        y = h2 @ self.W3.T + self.b3
        if keep:
            self._cache = (x, h1, h2)
        return y * self.out_scale

    def loss_and_grads(self, g, target, pi_weight=0.0):
        """Mean squared error on the scaled outputs, plus ``pi_weight`` times
        the mean squared error of the subgrid dissipation tau_ij S_ij, and
        the gradients."""
        y = self.forward(g, keep=True) / self.out_scale
        t = target / self.out_scale
        x, h1, h2 = self._cache
        n = g.shape[0]
        d = y - t
        # tau_ij S_ij = sum_o sw_o tau_o (off-diagonal terms counted twice)
        sw = np.stack([g[:, 0], g[:, 4], g[:, 8], g[:, 1] + g[:, 3], g[:, 2] + g[:, 6],
                       g[:, 5] + g[:, 7]], axis=1)
        dpi = (sw * (y * self.out_scale - target)).sum(1)
        loss = float((d**2).sum() / (n * 6) + pi_weight * (dpi**2).sum() / n)
        dy = 2 * d / (n * 6) + 2 * pi_weight / n * dpi[:, None] * sw * self.out_scale
        gW3 = dy.T @ h2
        gb3 = dy.sum(0)
        dh2 = dy @ self.W3
        dz2 = dh2 * (1 - h2**2)
        gW2 = dz2.T @ h1
        gb2 = dz2.sum(0)
        dh1 = dz2 @ self.W2
        dz1 = dh1 * (1 - h1**2)
        gW1 = dz1.T @ x
        gb1 = dz1.sum(0)
        return loss, dict(W1=gW1, b1=gb1, W2=gW2, b2=gb2, W3=gW3, b3=gb3)


def closure_forcing(oper, v_fft, mlp):
    """-d_j tau_ij from the MLP stress (spectral, 3 components)."""
    g = grad_phys(oper, v_fft)
    npts = g[0].size
    tau = mlp.forward(g.reshape(9, npts).T).T.reshape((6,) + g.shape[1:])
    tau_fft = [oper.fft(t) for t in tau]
    K = (oper.Kx, oper.Ky, oper.Kz)
    out = []
    for i in range(3):
        acc = 0
        for j in range(3):
            acc = acc + K[j] * tau_fft[TAU_INDEX[i][j]]
        out.append(-1j * acc)
    return np.array(out)
