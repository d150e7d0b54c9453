"""Restatement of the ns2d / ns3d pseudo-spectral time step (ORACLE).

Test infrastructure only (see ``oracle/__init__.py``).  Every function cites
the reference lines it follows; all arithmetic is float64 / complex128.
"""

import random

import numpy as np

from .spectral import OperNumpy2D, OperNumpy3D, slab_map


def max_abs(arr):
    """``fluidsim/base/time_stepping/base.py:24-25``."""
    return max(abs(arr.min()), abs(arr.max()))


def compute_freq_diss(oper, nu_2=0.0, nu_4=0.0, nu_8=0.0, nu_m4=0.0):
    """``fluidsim/base/solvers/pseudo_spect.py:134-191``."""
    if nu_2 > 0:
        f_d = nu_2 * oper.K2
    else:
        f_d = np.zeros_like(oper.K2)
    if nu_4 > 0.0:
        f_d = f_d + nu_4 * oper.K4
    if nu_8 > 0.0:
        f_d = f_d + nu_8 * oper.K8
    if nu_m4 != 0.0:
        f_d_hypo = nu_m4 / oper.K2_not0**2
        if f_d_hypo.ndim == 2:
            f_d_hypo[0, 0] = f_d_hypo[0, 1]
        else:
            f_d_hypo[0, 0, 0] = f_d_hypo[0, 0, 1]
    else:
        f_d_hypo = 0.0
    return f_d, f_d_hypo


class _SolverBase:
    """IF-RK4 driver shared by ns2d/ns3d.

    ``TimeSteppingPseudoSpectral`` (``fluidsim/base/time_stepping/pseudo_spect.py``):
    ``ExactLinearCoefs`` 103-152, ``_time_step_RK4`` 798-984; CFL logic
    ``fluidsim/base/time_stepping/base.py:248-354``; loop 182-244.
    """

    SCHEMES = ("RK4", "RK2", "Euler", "RK2_trapezoid", "Euler_phaseshift",
               "RK2_phaseshift", "RK2_phaseshift_exact", "Euler_phaseshift_random",
               "RK2_phaseshift_random")

    def __init__(self, oper, nu_2=0.0, nu_4=0.0, nu_8=0.0, nu_m4=0.0,
                 deltat0=0.2, deltat_max=0.2, USE_CFL=False, cfl_coef=None,
                 type_time_scheme="RK4", nb_pairs=1, nb_steps_compute_new_pair=None):
        if type_time_scheme not in self.SCHEMES:
            raise ValueError(f"time scheme {type_time_scheme!r} not in the oracle")
        self.type_time_scheme = type_time_scheme
        self.oper = oper
        self.nu_2, self.nu_4, self.nu_8, self.nu_m4 = nu_2, nu_4, nu_8, nu_m4
        f_d, f_d_hypo = compute_freq_diss(oper, nu_2, nu_4, nu_8, nu_m4)
        self.freq_lin = f_d + f_d_hypo
        self.USE_CFL = USE_CFL
        # base.py:249-260: default coefficient 0.4 for RK2*/Euler*, 1 for RK4
        if cfl_coef is not None:
            self.CFL = cfl_coef
        else:
            self.CFL = 1.0 if type_time_scheme.startswith("RK4") else 0.4
        self.deltat = deltat0
        self.deltat_max = deltat_max
        self.dt_old = None
        self.t = 0.0
        self.it = 0
        self.state_spect = np.zeros((self.nvar,) + oper.shapeK, np.complex128)
        self.state_phys = np.zeros((len(self.keys_phys),) + oper.shapeX)
        # sim.forcing (oracle.forcing.CoarseForcingOracle), computed once per
        # step after the CFL update (base.py:208-213)
        self.forcing = None
        self._forcing_fft = None
        if type_time_scheme.endswith("_random"):
            self._init_phaseshift_random(nb_pairs, nb_steps_compute_new_pair)

    # ExactLinearCoefs.compute / get_updated_coefs_CLF (pseudo_spect.py:125-146)
    def _coefs(self):
        dt = self.deltat
        if self.dt_old != dt:
            self.exact = np.exp(-dt * self.freq_lin)
            self.exact2 = np.exp(-dt / 2 * self.freq_lin)
            self.dt_old = dt
        return self.exact, self.exact2

    # base.py:334-354
    def _cfl_from_tmp(self, tmp):
        if tmp > 0:
            deltat_CFL = self.CFL / tmp
        else:
            deltat_CFL = self.deltat_max
        maybe_new_dt = min(deltat_CFL, self.deltat_max)
        normalize_diff = abs(self.deltat - maybe_new_dt) / maybe_new_dt
        if normalize_diff > 0.02:
            self.deltat = maybe_new_dt

    def time_step_RK4(self):
        """``pseudo_spect.py:798-984`` line for line (each expression run over
        slabs of the first spatial axis on all host cores)."""
        dt = self.deltat
        diss, diss2 = self._coefs()
        S = self.state_spect
        tmp = np.empty_like(S)
        tmp1 = np.empty_like(S)
        nslab = S.shape[1]
        N0 = self.tendencies_nonlin()

        def stage1(sl):
            s = (slice(None), sl)
            tmp[s] = (S[s] + dt / 6 * N0[s]) * diss[sl]
            tmp1[s] = (S[s] + dt / 2 * N0[s]) * diss2[sl]
        slab_map(stage1, nslab)
        N1 = self.tendencies_nonlin(tmp1)

        def stage2(sl):
            s = (slice(None), sl)
            tmp[s] += dt / 3 * diss2[sl] * N1[s]
            tmp1[s] = S[s] * diss2[sl] + dt / 2 * N1[s]
        slab_map(stage2, nslab)
        N2 = self.tendencies_nonlin(tmp1)

        def stage3(sl):
            s = (slice(None), sl)
            tmp[s] += dt / 3 * diss2[sl] * N2[s]
            tmp1[s] = S[s] * diss[sl] + dt * diss2[sl] * N2[s]
        slab_map(stage3, nslab)
        N3 = self.tendencies_nonlin(tmp1)

        def stage4(sl):
            s = (slice(None), sl)
            S[s] = tmp[s] + dt / 6 * N3[s]
        slab_map(stage4, nslab)

    def time_step_Euler(self):
        """``pseudo_spect.py:245-280`` (``step_Euler_inplace``, 51-60)."""
        dt = self.deltat
        diss = self._coefs()[0]
        S = self.state_spect
        N0 = self.tendencies_nonlin()
        S[:] = (S + dt * N0) * diss

    def time_step_RK2(self):
        """``pseudo_spect.py:469-517`` (``step_Euler`` 51-56, ``step_like_RK2``
        63-67)."""
        dt = self.deltat
        diss, diss2 = self._coefs()
        S = self.state_spect
        N0 = self.tendencies_nonlin()
        S12 = (S + dt / 2 * N0) * diss2
        N12 = self.tendencies_nonlin(S12)
        S[:] = S * diss + dt * diss2 * N12

    def time_step_RK2_trapezoid(self):
        """``pseudo_spect.py:519-569``."""
        dt = self.deltat
        diss = self._coefs()[0]
        S = self.state_spect
        N0 = self.tendencies_nonlin()
        S1 = (S + dt * N0) * diss
        N1 = self.tendencies_nonlin(S1)
        S[:] = (S + dt / 2 * N0) * diss + dt / 2 * N1

    def _phaseshift(self):
        """exp(i phi), phi = (dx kx + dy ky (+ dz kz)) / 2,
        ``pseudo_spect.py:282-300``."""
        o = self.oper
        if len(o.axes) == 3:
            phase = 0.5 * (o.deltax * o.Kx + o.deltay * o.Ky + o.deltaz * o.Kz)
        else:
            phase = 0.5 * (o.deltax * o.KX + o.deltay * o.KY)
        return np.exp(1j * phase)

    def get_phases_random(self):
        """``operators3d.py:1128-1146`` / ``operators2d.py:618-631``: one
        ``random.uniform(-0.5, 0.5)`` per axis (x, y, z order), beta from
        alpha by +- 1/2; returns the coefficients (a_x, a_y[, a_z]) of
        phase = a_x dx Kx + a_y dy Ky (+ a_z dz Kz)."""
        alpha = tuple(random.uniform(-0.5, 0.5) for _ in self.oper.axes)
        beta = tuple(a + 0.5 if a < 0 else a - 0.5 for a in alpha)
        return alpha, beta

    def _phase_from(self, coefs):
        o = self.oper
        if len(o.axes) == 3:
            phase = (coefs[0] * o.deltax * o.Kx + coefs[1] * o.deltay * o.Ky
                     + coefs[2] * o.deltaz * o.Kz)
        else:
            phase = coefs[0] * o.deltax * o.KX + coefs[1] * o.deltay * o.KY
        return np.exp(1j * phase)

    def _init_phaseshift_random(self, nb_pairs, nb_steps_compute_new_pair):
        """``pseudo_spect.py:302-327`` (pairs kept as coefficient tuples)."""
        if nb_steps_compute_new_pair is None:
            nb_steps_compute_new_pair = 2 if nb_pairs == 1 else 4 * nb_pairs
        self.nb_pairs = nb_pairs
        self.nb_steps_compute_new_pair = nb_steps_compute_new_pair
        self._index_phaseshift = 1
        self._previous_index_pair = 0
        self._previous_index_flip = 0
        self._pairs_phaseshift = [self.get_phases_random() for _ in range(nb_pairs)]
        self.phase_pairs_used = []

    def _get_phaseshift_random(self):
        """``pseudo_spect.py:329-372``: the (alpha, beta) coefficients of
        this step."""
        nb_pairs, nb_new = self.nb_pairs, self.nb_steps_compute_new_pair
        if nb_pairs == 1 and nb_new == 1:
            alpha, beta = self._pairs_phaseshift[0]
        elif nb_pairs == 1 and nb_new == 2:
            pair = self._pairs_phaseshift[0]
            if self._index_phaseshift == 1:
                alpha, beta = pair
            else:
                beta, alpha = pair
        else:
            index_pair = random.randint(0, nb_pairs - 1)
            pair = self._pairs_phaseshift[index_pair]
            index_flip = random.randint(0, 1)
            if (index_pair == self._previous_index_pair
                    and index_flip == self._previous_index_flip):
                index_flip = 0 if index_flip else 1
            self._previous_index_pair = index_pair
            self._previous_index_flip = index_flip
            if index_flip:
                alpha, beta = pair
            else:
                beta, alpha = pair
        if self._index_phaseshift == nb_new:
            self._index_phaseshift = 1
            new_pair = self.get_phases_random()
            self._pairs_phaseshift.pop(0)
            self._pairs_phaseshift.append(new_pair)
        else:
            self._index_phaseshift += 1
        self.phase_pairs_used.append((alpha, beta))
        return self._phase_from(alpha), self._phase_from(beta)

    def time_step_Euler_phaseshift_random(self):
        """``pseudo_spect.py:421-467``."""
        dt = self.deltat
        diss = self._coefs()[0]
        S = self.state_spect
        pa, pb = self._get_phaseshift_random()
        Na = self.tendencies_nonlin(pa * S) / pa
        Nb = self.tendencies_nonlin(pb * S) / pb
        Nd = 0.5 * (Na + Nb)
        S[:] = (S + dt * Nd) * diss

    def time_step_RK2_phaseshift_random(self):
        """``pseudo_spect.py:641-710``."""
        dt = self.deltat
        diss, diss2 = self._coefs()
        pa, pb = self._get_phaseshift_random()
        S = self.state_spect
        N0 = self.tendencies_nonlin(pa * S) / pa
        S1 = (S + dt * N0) * diss
        N1s = self.tendencies_nonlin(pb * S1)
        Nd = 0.5 * (N0 + N1s / pb)
        S[:] = S * diss + dt * diss2 * Nd

    def time_step_Euler_phaseshift(self):
        """``pseudo_spect.py:374-419``."""
        dt = self.deltat
        diss = self._coefs()[0]
        S = self.state_spect
        N0 = self.tendencies_nonlin()
        ph = self._phaseshift()
        Ns = self.tendencies_nonlin(ph * S) / ph
        Nd = 0.5 * (N0 + Ns)
        S[:] = (S + dt * Nd) * diss

    def time_step_RK2_phaseshift(self):
        """``pseudo_spect.py:571-639``."""
        dt = self.deltat
        diss, diss2 = self._coefs()
        S = self.state_spect
        N0 = self.tendencies_nonlin()
        S1 = (S + dt * N0) * diss
        ph = self._phaseshift()
        N1s = self.tendencies_nonlin(ph * S1)
        Nd = 0.5 * (N0 + N1s / ph)
        S[:] = S * diss + dt * diss2 * Nd

    def time_step_RK2_phaseshift_exact(self):
        """``pseudo_spect.py:712-796``."""
        dt = self.deltat
        diss, diss2 = self._coefs()
        ph = self._phaseshift()
        S = self.state_spect
        N0 = self.tendencies_nonlin(S)
        N0s = self.tendencies_nonlin(ph * S)
        Nd0 = 0.5 * (N0 + N0s / ph)
        S1 = (S + dt * Nd0) * diss
        N1 = self.tendencies_nonlin(S1)
        N1s = self.tendencies_nonlin(ph * S1)
        Nd = 0.5 * (Nd0 + 0.5 * (N1 + N1s / ph))
        S[:] = S * diss + dt * diss2 * Nd

    def time_step(self):
        """``_init_time_scheme`` dispatch, ``pseudo_spect.py:191-231``."""
        getattr(self, "time_step_" + self.type_time_scheme)()

    def one_time_step(self):
        """``base.py:208-244`` without outputs or signals."""
        if self.USE_CFL:
            self.compute_time_increment_CLF()
        if self.forcing is not None:
            self._forcing_fft = self.forcing.compute(self.state_spect, self.t, self.deltat)
        self.one_time_step_computation()
        self.t += self.deltat
        self.it += 1

    def run(self, it_end=None, t_end=None):
        if t_end is not None:
            while self.t < t_end:
                self.one_time_step()
        else:
            while self.it < it_end:
                self.one_time_step()


class NS2DOracle(_SolverBase):
    """ns2d: ``fluidsim/solvers/ns2d/solver.py`` + ``state.py``."""

    nvar = 1
    keys_phys = ("ux", "uy", "rot")  # ns2d/state.py:31

    def __init__(self, oper: OperNumpy2D, beta=0.0, **kw):
        self.beta = beta
        super().__init__(oper, **kw)

    def statephys_from_statespect(self):
        """``ns2d/state.py:95-106``."""
        rot_fft = self.state_spect[0]
        ux_fft, uy_fft = self.oper.vecfft_from_rotfft(rot_fft)
        self.state_phys[2] = self.oper.ifft(rot_fft)
        self.state_phys[0] = self.oper.ifft(ux_fft)
        self.state_phys[1] = self.oper.ifft(uy_fft)

    def init_from_rotfft(self, rot_fft):
        """``ns2d/state.py:115-119``."""
        rot_fft = np.array(rot_fft, dtype=np.complex128)
        self.oper.dealiasing(rot_fft)
        self.state_spect[0] = rot_fft
        self.statephys_from_statespect()

    def tendencies_nonlin(self, state_spect=None):
        """``ns2d/solver.py:111-194`` with ``compute_Frot`` 33-39."""
        oper = self.oper
        if state_spect is None:
            rot_fft = self.state_spect[0]
            ux = self.state_phys[0]
            uy = self.state_phys[1]
        else:
            rot_fft = state_spect[0]
            ux_fft, uy_fft = oper.vecfft_from_rotfft(rot_fft)
            ux = oper.ifft(ux_fft)
            uy = oper.ifft(uy_fft)
        px_rot_fft, py_rot_fft = oper.gradfft_from_fft(rot_fft)
        px_rot = oper.ifft(px_rot_fft)
        py_rot = oper.ifft(py_rot_fft)
        if self.beta == 0:
            Frot = -ux * px_rot - uy * py_rot
        else:
            Frot = -ux * px_rot - uy * (py_rot + self.beta)
        F = np.empty_like(self.state_spect)
        F[0] = oper.fft(Frot)
        oper.dealiasing(F[0])
        return F

    def one_time_step_computation(self):
        """``pseudo_spect.py:236-243``."""
        self.time_step()
        self.oper.dealiasing(self.state_spect[0])
        self.statephys_from_statespect()
        if np.isnan(np.sum(self.state_spect[0])):
            raise ValueError(f"nan at it = {self.it}, t = {self.t:.4f}")

    def compute_time_increment_CLF(self):
        """``base.py:356-366`` (``_compute_time_increment_CLF_uxuy``)."""
        ux, uy = self.state_phys[0], self.state_phys[1]
        tmp = max_abs(ux) / self.oper.deltax + max_abs(uy) / self.oper.deltay
        self._cfl_from_tmp(tmp)

    # outputs: ns2d/output/__init__.py:110-129, spatial_means.py:23-36
    def energy_fft(self):
        ux_fft, uy_fft = self.oper.vecfft_from_rotfft(self.state_spect[0])
        return (np.abs(ux_fft) ** 2 + np.abs(uy_fft) ** 2) / 2.0

    def enstrophy_fft(self):
        return np.abs(self.state_spect[0]) ** 2 / 2.0

    def compute_energy(self):
        return self.oper.sum_wavenumbers(self.energy_fft())

    def compute_enstrophy(self):
        return self.oper.sum_wavenumbers(self.enstrophy_fft())

    def spatial_means(self):
        f_d, f_d_hypo = compute_freq_diss(self.oper, self.nu_2, self.nu_4,
                                          self.nu_8, self.nu_m4)
        e_fft, z_fft = self.energy_fft(), self.enstrophy_fft()
        s = self.oper.sum_wavenumbers
        return {
            "E": s(e_fft), "Z": s(z_fft),
            "epsK": s(f_d * 2 * e_fft), "epsK_hypo": s(f_d_hypo * 2 * e_fft),
            "epsZ": s(f_d * 2 * z_fft), "epsZ_hypo": s(f_d_hypo * 2 * z_fft),
        }


class NS2DStratOracle(NS2DOracle):
    """ns2d.strat: ``fluidsim/solvers/ns2d/strat/solver.py`` (tendencies
    101-210), ``state.py`` (keys), ``time_stepping.py`` (CFL with the
    dispersion-relation time, 31-70, 158-198)."""

    nvar = 2
    keys_phys = ("ux", "uy", "rot", "b")  # ns2d/strat/state.py:33

    def __init__(self, oper: OperNumpy2D, N=1.0, cfl_coef_group=None, **kw):
        self.N = N
        if cfl_coef_group:
            raise NotImplementedError("the group-velocity time of ns2d.strat")
        super().__init__(oper, beta=0.0, **kw)
        # time_stepping.py:55-70 and solver.py:215-225 (compute_dispersion_relation);
        # N = 0 (ns2d.bouss: the plain ns2d time stepping) caps nothing
        freq_disp = (N * (oper.KX / oper.K_not0)).max()
        self.deltat_dispersion_relation = (1.0 * (2.0 * np.pi / freq_disp) if freq_disp > 0
                                           else np.inf)

    def statephys_from_statespect(self):
        super().statephys_from_statespect()
        self.state_phys[3] = self.oper.ifft(self.state_spect[1])

    def init_from_rotbfft(self, rot_fft, b_fft):
        rot_fft = np.array(rot_fft, dtype=np.complex128)
        b_fft = np.array(b_fft, dtype=np.complex128)
        self.oper.dealiasing(rot_fft)
        self.oper.dealiasing(b_fft)
        self.state_spect[0] = rot_fft
        self.state_spect[1] = b_fft
        self.statephys_from_statespect()

    def tendencies_nonlin(self, state_spect=None):
        """``ns2d/strat/solver.py:143-192`` and
        ``tendencies_nonlin_ns2dstrat`` 27-32."""
        oper = self.oper
        if state_spect is None:
            rot_fft, b_fft = self.state_spect[0], self.state_spect[1]
            ux, uy = self.state_phys[0], self.state_phys[1]
        else:
            rot_fft, b_fft = state_spect[0], state_spect[1]
            ux_fft, uy_fft = oper.vecfft_from_rotfft(rot_fft)
            ux = oper.ifft(ux_fft)
            uy = oper.ifft(uy_fft)
        px_rot_fft, py_rot_fft = oper.gradfft_from_fft(rot_fft)
        px_b_fft, py_b_fft = oper.gradfft_from_fft(b_fft)
        px_rot, py_rot = oper.ifft(px_rot_fft), oper.ifft(py_rot_fft)
        px_b, py_b = oper.ifft(px_b_fft), oper.ifft(py_b_fft)
        f_rot = -ux * px_rot - uy * py_rot
        f_b = -ux * px_b - uy * py_b - self.N**2 * uy
        F = np.empty_like(self.state_spect)
        F[1] = oper.fft(f_b)
        F[0] = oper.fft(f_rot)
        F[0] += px_b_fft
        oper.dealiasing(F[0])
        oper.dealiasing(F[1])
        return F

    def one_time_step_computation(self):
        """``pseudo_spect.py:236-243`` (dealiasing of every variable)."""
        self.time_step()
        self.oper.dealiasing(self.state_spect[0])
        self.oper.dealiasing(self.state_spect[1])
        self.statephys_from_statespect()
        if np.isnan(np.sum(self.state_spect[0])):
            raise ValueError(f"nan at it = {self.it}, t = {self.t:.4f}")

    def compute_time_increment_CLF(self):
        """``time_stepping.py:158-198`` (``_compute_time_increment_CFL_uxuyb``,
        no group-velocity term, no forcing)."""
        ux, uy = self.state_phys[0], self.state_phys[1]
        freq_CFL = abs(ux).max() / self.oper.deltax + abs(uy).max() / self.oper.deltay
        deltat_CFL = self.CFL / freq_CFL if freq_CFL > 0 else self.deltat_max
        maybe_new_dt = min(deltat_CFL, self.deltat_dispersion_relation, self.deltat_max)
        normalize_diff = abs(self.deltat - maybe_new_dt) / maybe_new_dt
        if normalize_diff > 0.02:
            self.deltat = maybe_new_dt

    # ns2d/strat/output/__init__.py:85-109 (compute_energies_fft)
    def energyA_fft(self):
        if self.N == 0:
            return np.zeros(self.oper.shapeK)
        return ((np.abs(self.state_spect[1]) / self.N) ** 2) / 2

    def compute_energy(self):
        return self.oper.sum_wavenumbers(self.energy_fft() + self.energyA_fft())

    def spatial_means(self):
        """``ns2d/strat/output/spatial_means.py:23-55`` (no forcing)."""
        f_d, f_d_hypo = compute_freq_diss(self.oper, self.nu_2, self.nu_4,
                                          self.nu_8, self.nu_m4)
        ek, ea, z = self.energy_fft(), self.energyA_fft(), self.enstrophy_fft()
        s = self.oper.sum_wavenumbers
        return {
            "E": s(ek + ea), "EK": s(ek), "EA": s(ea), "Z": s(z),
            "epsK": s(f_d * 2.0 * ek), "epsK_hypo": s(f_d_hypo * 2.0 * ek),
            "epsA": s(f_d * 2.0 * ea), "epsA_hypo": s(f_d_hypo * 2.0 * ea),
            "epsZ": s(f_d * 2.0 * z), "epsZ_hypo": s(f_d_hypo * 2.0 * z),
        }


class NS3DOracle(_SolverBase):
    """ns3d: ``fluidsim/solvers/ns3d/solver.py``, ``time_stepping.py``."""

    nvar = 3
    keys_phys = ("vx", "vy", "vz")  # ns3d/state.py:20

    def __init__(self, oper: OperNumpy3D, f=None, turb_model=None, projection=None,
                 no_vz_kz0=False, **kw):
        self.f = f
        # ns3d/solver.py:147-175
        self._projector = {None: oper.project_perpk3d, "toroidal": oper.project_toroidal,
                           "vortical": oper.project_toroidal,
                           "poloidal": oper.project_poloidal}[projection]
        self.no_vz_kz0 = no_vz_kz0
        # callable (oper, vx_fft, vy_fft, vz_fft) -> forcing (3, *shapeK)
        self.turb_model = turb_model
        super().__init__(oper, **kw)

    def statephys_from_statespect(self):
        """``fluidsim/base/state.py:326-333``."""
        for ik in range(self.nvar):
            self.state_phys[ik] = self.oper.ifft(self.state_spect[ik])

    def statespect_from_statephys(self):
        """``fluidsim/base/state.py:318-325``."""
        for ik in range(self.nvar):
            self.state_spect[ik] = self.oper.fft(self.state_phys[ik])

    def init_from_vxvyvzfft(self, vx_fft, vy_fft, vz_fft):
        """``ns3d/state.py:124-130``."""
        self.state_spect[0] = vx_fft
        self.state_spect[1] = vy_fft
        self.state_spect[2] = vz_fft
        self.statephys_from_statespect()
        self.statespect_from_statephys()

    def project_state_spect(self, S):
        """``ns3d/solver.py:255-263``."""
        self._projector(S[0], S[1], S[2])
        if self.no_vz_kz0:
            S[2][self.oper.Kz == 0] = 0.0
            if self.nvar == 4:  # b_fft
                S[3][self.oper.Kz == 0] = 0.0

    def tendencies_nonlin(self, state_spect=None):
        """``ns3d/solver.py:180-253``."""
        oper = self.oper
        S = self.state_spect if state_spect is None else state_spect
        vx_fft, vy_fft, vz_fft = S[0], S[1], S[2]
        ox_fft, oy_fft, oz_fft = oper.rotfft_from_vecfft(vx_fft, vy_fft, vz_fft)
        if self.f is not None:
            oz_fft = oz_fft.copy()
            oz_fft[0, 0, 0] += self.f
        ox, oy, oz = oper.ifft(ox_fft), oper.ifft(oy_fft), oper.ifft(oz_fft)
        if state_spect is None:
            vx, vy, vz = self.state_phys[:3]
        else:
            vx, vy, vz = oper.ifft(vx_fft), oper.ifft(vy_fft), oper.ifft(vz_fft)
        # fluidfft vector_product(v, omega) = v x omega
        fx, fy, fz = np.empty((3,) + vx.shape)

        def product(sl):
            fx[sl] = vy[sl] * oz[sl] - vz[sl] * oy[sl]
            fy[sl] = vz[sl] * ox[sl] - vx[sl] * oz[sl]
            fz[sl] = vx[sl] * oy[sl] - vy[sl] * ox[sl]
        slab_map(product, vx.shape[0])
        F = np.empty_like(self.state_spect)
        F[0] = oper.fft(fx)
        F[1] = oper.fft(fy)
        F[2] = oper.fft(fz)
        if self._forcing_fft is not None:  # ns3d/solver.py:243-244
            F += self._forcing_fft
        if self.turb_model is not None:  # ns3d/solver.py:246-249
            F += self.turb_model(oper, vx_fft, vy_fft, vz_fft)
        self.project_state_spect(F)
        oper.dealiasing(F)
        return F

    def one_time_step_computation(self):
        """``ns3d/time_stepping.py:8-20``."""
        self.time_step()
        self.project_state_spect(self.state_spect)
        self.oper.dealiasing(self.state_spect)
        self.statephys_from_statespect()
        if np.isnan(np.sum(self.state_spect[0])):
            raise ValueError(f"nan at it = {self.it}, t = {self.t:.4f}")

    def compute_time_increment_CLF(self):
        """``base.py:320-339`` (``_compute_time_increment_CLF_uxuyuz``)."""
        vx, vy, vz = self.state_phys[:3]
        o = self.oper
        tmp = (max_abs(vx) / o.deltax + max_abs(vy) / o.deltay
               + max_abs(vz) / o.deltaz)
        self._cfl_from_tmp(tmp)

    # outputs: ns3d/output/__init__.py:101-117, spatial_means.py:23-40
    def energy_fft(self):
        S = self.state_spect
        return 0.5 * (np.abs(S[0]) ** 2 + np.abs(S[1]) ** 2 + np.abs(S[2]) ** 2)

    def compute_energy(self):
        return self.oper.sum_wavenumbers(self.energy_fft())

    def spatial_means(self):
        f_d, f_d_hypo = compute_freq_diss(self.oper, self.nu_2, self.nu_4,
                                          self.nu_8, self.nu_m4)
        e_fft = self.energy_fft()
        s = self.oper.sum_wavenumbers
        return {"E": s(e_fft), "epsK": s(f_d * 2 * e_fft),
                "epsK_hypo": s(f_d_hypo * 2 * e_fft)}


class NS3DStratOracle(NS3DOracle):
    """ns3d.strat: ``fluidsim/solvers/ns3d/strat/solver.py`` + ``state.py``."""

    nvar = 4
    keys_phys = ("vx", "vy", "vz", "b")  # ns3d/strat/state.py:18-24

    def __init__(self, oper: OperNumpy3D, N=1.0, bouss=False, **kw):
        """bouss: ns3d.bouss (``ns3d/bouss/solver.py:48-160``), the same
        tendencies without the -N^2 vz term (its output still weights EA by
        the strat class's params.N)."""
        self.N = N
        self.bouss = bouss
        super().__init__(oper, **kw)

    def init_from_vxvyvzfft(self, vx_fft, vy_fft, vz_fft):
        """``ns3d/strat/state.py:26-32``: b = 0, then the phys/spect round trip."""
        self.state_spect[3] = 0.0
        super().init_from_vxvyvzfft(vx_fft, vy_fft, vz_fft)

    def tendencies_nonlin(self, state_spect=None):
        """``ns3d/strat/solver.py:138-216``."""
        oper = self.oper
        S = self.state_spect if state_spect is None else state_spect
        vx_fft, vy_fft, vz_fft, b_fft = S[0], S[1], S[2], S[3]
        ox_fft, oy_fft, oz_fft = oper.rotfft_from_vecfft(vx_fft, vy_fft, vz_fft)
        if self.f is not None:
            oz_fft = oz_fft.copy()
            oz_fft[0, 0, 0] += self.f
        ox, oy, oz = oper.ifft(ox_fft), oper.ifft(oy_fft), oper.ifft(oz_fft)
        if state_spect is None:
            vx, vy, vz, b = self.state_phys
        else:
            vx, vy, vz = oper.ifft(vx_fft), oper.ifft(vy_fft), oper.ifft(vz_fft)
            b = oper.ifft(b_fft)
        F = np.empty_like(self.state_spect)
        F[0] = oper.fft(vy * oz - vz * oy)
        F[1] = oper.fft(vz * ox - vx * oz)
        F[2] = oper.fft(vx * oy - vy * ox)
        F[2] += b_fft
        div_vb_fft = oper.div_vb_fft_from_vb(vx, vy, vz, b)
        if self.bouss:  # ns3d/bouss/solver.py:150-152
            F[3] = -div_vb_fft
        else:
            F[3] = -div_vb_fft - self.N**2 * vz_fft  # compute_fb_fft, solver.py:19-23
        self.project_state_spect(F)
        oper.dealiasing(F)
        return F

    def energy_fft(self):
        """Kinetic + potential, ``ns3d/strat/output/__init__.py:74-84``."""
        S = self.state_spect
        return 0.5 * (np.abs(S[0]) ** 2 + np.abs(S[1]) ** 2 + np.abs(S[2]) ** 2
                      + np.abs(S[3]) ** 2 / self.N**2)

    def spatial_means(self):
        """``ns3d/strat/output/spatial_means.py:27-61`` (EK, EA, dissipations)."""
        f_d, f_d_hypo = compute_freq_diss(self.oper, self.nu_2, self.nu_4,
                                          self.nu_8, self.nu_m4)
        S = self.state_spect
        ek = 0.5 * (np.abs(S[0]) ** 2 + np.abs(S[1]) ** 2 + np.abs(S[2]) ** 2)
        ea = 0.5 * np.abs(S[3]) ** 2 / self.N**2
        s = self.oper.sum_wavenumbers
        return {"E": s(ek) + s(ea), "EK": s(ek), "EA": s(ea), "epsK": s(f_d * 2 * ek),
                "epsK_hypo": s(f_d_hypo * 2 * ek), "epsA": s(f_d * 2 * ea),
                "epsA_hypo": s(f_d_hypo * 2 * ea)}
