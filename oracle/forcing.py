"""Coarse normalized forcings restated in numpy (ORACLE, test infrastructure).

``fluidsim/base/forcing/specific.py``: coarse grid and forced modes
(137-246), ``Proportional`` (346-425), ``NormalizedForcing`` with the
2nd-degree normalization (428-727), ``RandomSimplePseudoSpectral`` (729-768)
and ``TimeCorrelatedRandomPseudoSpectral`` (770-868), for ns3d state
variables.  Random draws use the global ``np.random`` in the reference's
order; ``create_arrayK_random`` (fluidfft, not in the reference) is the
oracle operator's restatement.  Forcing arrays are float64 / complex128.
"""

import numpy as np

from .spectral import OperNumpy3D, k_adim_seq


def coarse_fft_size(nkmax_forcing):
    """``specific.py:190-201`` when ``pulp`` is absent (power of two)."""
    i = 0
    while 2 * nkmax_forcing > 2**i:
        i += 1
    return 2**i


def _ik_from_ikc(ikc, nkc, nk):
    """``operators3d.py:1183-1193``."""
    return ikc if ikc <= nkc / 2.0 else ikc - nkc + nk


class CoarseForcingOracle:
    """``compute(sim)`` once per step returns the (nvar, *shapeK) forcing."""

    def __init__(self, oper: OperNumpy3D, nvar, keys, forcing_type="tcrandom",
                 nkmin_forcing=4, nkmax_forcing=5, forcing_rate=1.0,
                 time_correlation="based_on_forcing_rate", which_root="minabs",
                 only_positive=False, t0=0.0):
        self.oper = oper
        self.nvar = nvar
        self.keys = list(keys)
        self.type = forcing_type
        self.forcing_rate = forcing_rate
        self.which_root = which_root
        deltak = max(oper.deltakx, oper.deltaky, oper.deltakz)
        kmax, kmin = deltak * nkmax_forcing, deltak * nkmin_forcing
        nc = coarse_fft_size(nkmax_forcing)
        self.oper_coarse = OperNumpy3D(nc, nc, nc, oper.Lx, oper.Ly, oper.Lz,
                                       coef_dealiasing=1.0)
        K = np.sqrt(self.oper_coarse.K2)
        no_f = np.logical_or(K > kmax, K < kmin)
        nkzc, nkyc, nkxc = self.oper_coarse.shapeK
        no_f[nkzc // 2, :, :] = True
        no_f[:, nkyc // 2, :] = True
        no_f[:, :, nkxc - 1] = True
        self.COND_NO_F = no_f
        self.min_val = None if only_positive else -1
        # fine-grid indices of the coarse modes (coarse_seq_from_fft_loc)
        iz = np.array([_ik_from_ikc(i, nkzc, oper.nz) for i in range(nkzc)])
        iy = np.array([_ik_from_ikc(i, nkyc, oper.ny) for i in range(nkyc)])
        self._ix = np.ix_(iz, iy, np.arange(nkxc))
        self.forcing_fft = np.zeros((nvar,) + oper.shapeK, np.complex128)
        if forcing_type == "tcrandom":
            self.t_last_change = t0
            self._seed0 = np.random.randint(0, 2**31)
            self._seed1 = np.random.randint(0, 2**31)
            np.random.seed(self._seed0)
            self.forcing0 = self.compute_forcingc_raw()
            np.random.seed(self._seed1)
            self.forcing1 = self.compute_forcingc_raw()
            self.period_change_f0f1 = (forcing_rate ** (-1.0 / 3)
                                       if time_correlation == "based_on_forcing_rate"
                                       else time_correlation)

    def compute_forcingc_raw(self):
        """``specific.py:840-850``; project_fft_on_realX = fft(ifft())."""
        oc = self.oper_coarse
        f_fft = oc.create_arrayK_random(min_val=self.min_val)
        f_fft[self.COND_NO_F] = 0.0
        return oc.fft(oc.ifft(f_fft))

    def forcingc_raw_each_time(self, t):
        if self.type == "random":
            return self.compute_forcingc_raw()
        if t - self.t_last_change >= self.period_change_f0f1:  # 824-840
            self.t_last_change = t
            self._seed0 = self._seed1
            self.forcing0 = self.forcing1
            self._seed1 = np.random.randint(0, 2**31)
            np.random.seed(self._seed1)
            self.forcing1 = self.compute_forcingc_raw()
        omega = np.pi / self.period_change_f0f1  # 852-868
        deltaf = self.forcing1 - self.forcing0
        return self.forcing1 - 0.5 * (np.cos((t - self.t_last_change) * omega) + 1) * deltaf

    def _root(self, a, b, c):
        """``coef_normalization_from_abc`` (678-727)."""
        try:
            alpha1, alpha2 = np.roots([a, b, c])
        except ValueError:
            return 0.0
        if self.which_root == "minabs":
            return alpha2 if abs(alpha2) < abs(alpha1) else alpha1
        if self.which_root == "positive":
            return alpha2 if alpha2 > 0.0 else alpha1
        raise NotImplementedError(self.which_root)

    def compute(self, state_spect, t, dt):
        oc = self.oper_coarse
        coarse = np.zeros((self.nvar,) + oc.shapeK, np.complex128)
        for key in self.keys:
            vc = np.asarray(state_spect[key])[self._ix]
            if self.type == "proportional":  # 403-425
                fvc = vc.copy()
                fvc[self.COND_NO_F] = 0.0
                Z = oc.sum_wavenumbers(abs(fvc) ** 2 / 2.0)
                fvc = (np.sqrt(1 + dt * self.forcing_rate / Z) - 1.0) / dt * fvc
            else:  # 484-507 and 587-676
                fvc = self.forcingc_raw_each_time(t)
                a = dt / 2 * oc.sum_wavenumbers(abs(fvc) ** 2)
                b = oc.sum_wavenumbers((vc.conj() * fvc).real)
                fvc *= self._root(a, b, -self.forcing_rate)
            coarse[key] += fvc
        for key in range(self.nvar):  # put_forcingc_in_forcing
            self.forcing_fft[key][self._ix] = coarse[key]
        return self.forcing_fft
