"""Compile-time-size kernels (power-of-two grids) against the oracle.

The golden fixtures mostly use odd or small grids (generic kernels); these
cases use sizes served by the fast path.  Step 1 runs unpruned (the state was
set from outside), later steps run pruned (state known to be dealiased), so
both variants are compared with the float64 oracle run live.
"""
from math import pi

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return max(np.linalg.norm(a[i] - b[i]) / np.linalg.norm(b[i]) for i in range(len(b)))


def run_3d(shape, precision, steps, **kw):
    import torch
    from fluidsim_gb300.init_fields import isotropic_3d
    from fluidsim_gb300.solvers import SimulNS3D
    from oracle.solvers import NS3DOracle
    from oracle.spectral import OperNumpy3D
    nz, ny, nx = shape
    L = kw.get("L", (2 * pi, 2 * pi * ny / nx, 2 * pi * nz / nx))
    p = SimulNS3D.create_default_params()
    p.precision = precision
    p.oper.nx, p.oper.ny, p.oper.nz = nx, ny, nz
    p.oper.Lx, p.oper.Ly, p.oper.Lz = L
    p.nu_2 = kw.get("nu_2", 2e-3)
    p.nu_4 = kw.get("nu_4", 0.0)
    p.nu_m4 = kw.get("nu_m4", 0.0)
    p.f = kw.get("f")
    ts = p.time_stepping
    ts.USE_CFL = kw.get("USE_CFL", False)
    ts.cfl_coef = kw.get("cfl_coef")
    ts.deltat0 = kw.get("dt", 5e-3)
    ts.type_time_scheme = kw.get("type_time_scheme", "RK4")
    ts.USE_T_END = False
    ts.it_end = steps
    sim = SimulNS3D(p)
    v0 = isotropic_3d(nx, ny, nz, *L, seed=11)
    sim.state.init_statespect_from(vx_fft=v0[0], vy_fft=v0[1], vz_fft=v0[2])
    sim.time_stepping.start()
    orc = NS3DOracle(OperNumpy3D(nx, ny, nz, *L), f=kw.get("f"), nu_2=p.nu_2,
                     nu_4=p.nu_4, nu_m4=p.nu_m4, USE_CFL=ts.USE_CFL,
                     cfl_coef=ts.cfl_coef, deltat0=ts.deltat0,
                     type_time_scheme=ts.type_time_scheme)
    orc.state_spect[:] = v0
    orc.statephys_from_statespect()
    orc.run(it_end=steps)
    return sim, orc


@pytest.mark.parametrize("shape,kw", [
    ((64, 64, 64), {}),
    ((32, 64, 128), {"USE_CFL": True, "cfl_coef": 0.5, "f": 0.7}),
    ((64, 32, 64), {"nu_4": 1e-6, "nu_m4": 1e-3}),
    ((32, 64, 64), {"type_time_scheme": "RK2", "USE_CFL": True}),
    ((64, 64, 32), {"type_time_scheme": "RK2_trapezoid", "f": 0.3}),
    ((32, 32, 64), {"type_time_scheme": "Euler", "dt": 2e-3}),
    ((32, 64, 64), {"type_time_scheme": "RK2_phaseshift", "USE_CFL": True}),
    ((64, 32, 32), {"type_time_scheme": "RK2_phaseshift_exact", "f": 0.4}),
    ((32, 32, 32), {"type_time_scheme": "Euler_phaseshift", "dt": 2e-3}),
])
def test_ns3d_fast_fp64_matches_oracle(cuda, shape, kw):
    sim, orc = run_3d(shape, "float64", 4, **kw)
    got = sim.state.state_spect.cpu().numpy()
    assert rel(got, orc.state_spect) < 1e-12
    assert abs(sim.time_stepping.deltat - orc.deltat) <= 1e-12 * orc.deltat
    # pruned steps keep the state dealiased
    assert np.abs(got[:, orc.oper.where_dealiased.astype(bool)]).max() == 0


def test_ns3d_fast_fp32_error(cuda):
    sim, orc = run_3d((64, 64, 64), "float32", 6)
    got = sim.state.state_spect.cpu().numpy().astype(np.complex128)
    assert rel(got, orc.state_spect) < 1e-5


def test_ns3d_fast_fp32_nx512_error(cuda):
    """nx = 512 in FP32 runs the register x pass (kf3_xr: the six fields of a
    row pair by one group of 64 threads, named barriers; CFL maxima and f
    included)."""
    # a 2 pi cube: the energetic modes (|k| ~ 4) vary along y and z too
    sim, orc = run_3d((32, 32, 512), "float32", 6, USE_CFL=True, cfl_coef=0.5, f=0.7,
                      L=(2 * pi,) * 3)
    got = sim.state.state_spect.cpu().numpy().astype(np.complex128)
    assert rel(got, orc.state_spect) < 1e-5
    assert abs(sim.time_stepping.deltat - orc.deltat) <= 1e-5 * orc.deltat


def test_ns3d_fast_fp32_nx256_error(cuda):
    """nx = 256 in FP32: the register x pass on 256-point lines inside one
    warp (8 row pairs per CTA), CFL maxima included."""
    sim, orc = run_3d((32, 32, 256), "float32", 5, USE_CFL=True, cfl_coef=0.5,
                      L=(2 * pi,) * 3)
    got = sim.state.state_spect.cpu().numpy().astype(np.complex128)
    assert rel(got, orc.state_spect) < 1e-5
    assert abs(sim.time_stepping.deltat - orc.deltat) <= 1e-5 * orc.deltat


def test_ns3d_fast_fp32_nx1024_error(cuda):
    """nx = 1024 in FP32: rows in pairs on 1024-point lines of four warps
    (named barriers of 128 threads), CFL maxima included."""
    sim, orc = run_3d((32, 32, 1024), "float32", 4, USE_CFL=True, cfl_coef=0.5,
                      L=(2 * pi,) * 3)
    got = sim.state.state_spect.cpu().numpy().astype(np.complex128)
    assert rel(got, orc.state_spect) < 1e-5
    assert abs(sim.time_stepping.deltat - orc.deltat) <= 1e-5 * orc.deltat


def test_ns3d_strat_fast_fp32_nx512_error(cuda):
    """ns3d.strat with nx = 512 in FP32 (the 7-field 16 x 16 x pass)."""
    import torch
    from fluidsim_gb300.init_fields import isotropic_3d
    from fluidsim_gb300.solvers import SimulNS3DStrat
    from oracle.solvers import NS3DStratOracle
    from oracle.spectral import OperNumpy3D
    nz, ny, nx = 32, 32, 512
    L = (2 * pi,) * 3
    p = SimulNS3DStrat.create_default_params()
    p.precision = "float32"
    p.N = 2.0
    p.oper.nx, p.oper.ny, p.oper.nz = nx, ny, nz
    p.oper.Lx, p.oper.Ly, p.oper.Lz = L
    p.nu_2 = 2e-3
    ts = p.time_stepping
    ts.USE_CFL, ts.deltat0, ts.USE_T_END, ts.it_end = False, 5e-3, False, 5
    sim = SimulNS3DStrat(p)
    v0 = isotropic_3d(nx, ny, nz, *L, seed=11)
    b0 = isotropic_3d(nx, ny, nz, *L, seed=12)[0]
    sim.state.init_statespect_from(vx_fft=v0[0], vy_fft=v0[1], vz_fft=v0[2], b_fft=b0)
    sim.time_stepping.start()
    orc = NS3DStratOracle(OperNumpy3D(nx, ny, nz, *L), N=2.0, nu_2=2e-3, deltat0=5e-3)
    orc.state_spect[:3] = v0
    orc.state_spect[3] = b0
    orc.statephys_from_statespect()
    orc.run(it_end=5)
    got = sim.state.state_spect.cpu().numpy().astype(np.complex128)
    assert rel(got, orc.state_spect) < 1e-5


def test_ns3d_fast_tendency_matches_oracle(cuda):
    import torch
    from fluidsim_gb300.init_fields import isotropic_3d
    from fluidsim_gb300.solvers import SimulNS3D
    from oracle.solvers import NS3DOracle
    from oracle.spectral import OperNumpy3D
    n = 64
    p = SimulNS3D.create_default_params()
    p.oper.nx = p.oper.ny = p.oper.nz = n
    sim = SimulNS3D(p)
    v0 = isotropic_3d(n, n, n, seed=5, coef_dealiasing=1.0)  # not dealiased
    S = torch.from_numpy(v0).cuda()
    tend = sim.tendencies_nonlin(S).cpu().numpy()
    orc = NS3DOracle(OperNumpy3D(n, n, n))
    ref = orc.tendencies_nonlin(v0.copy())
    assert rel(tend, ref) < 1e-12


@pytest.mark.parametrize("shape,beta,cfl,scheme", [
    ((128, 128), 0.0, False, "RK4"), ((64, 256), 2.0, True, "RK4"),
    ((512, 512), 0.0, False, "RK4"), ((128, 64), 1.0, True, "RK2_phaseshift"),
    ((64, 128), 0.0, False, "RK2_trapezoid"), ((128, 128), 0.5, False, "Euler_phaseshift")])
def test_ns2d_fast_fp64_matches_oracle(cuda, shape, beta, cfl, scheme):
    from fluidsim_gb300.init_fields import noise_rot_2d
    from fluidsim_gb300.solvers import SimulNS2D
    from oracle.solvers import NS2DOracle
    from oracle.spectral import OperNumpy2D
    ny, nx = shape
    L = (2 * pi, 2 * pi * ny / nx)
    p = SimulNS2D.create_default_params()
    p.oper.nx, p.oper.ny = nx, ny
    p.oper.Lx, p.oper.Ly = L
    p.nu_2, p.nu_8, p.beta = 1e-3, 1e-14, beta
    ts = p.time_stepping
    ts.USE_CFL, ts.cfl_coef, ts.deltat0 = cfl, 0.5, 2e-3
    ts.type_time_scheme = scheme
    ts.USE_T_END, ts.it_end = False, 5
    sim = SimulNS2D(p)
    rot = noise_rot_2d(nx, ny, *L, kmin=3, kmax=10, seed=4)
    sim.init_from_rotfft(rot)
    sim.time_stepping.start()
    orc = NS2DOracle(OperNumpy2D(nx, ny, *L), beta=beta, nu_2=1e-3, nu_8=1e-14,
                     USE_CFL=cfl, cfl_coef=0.5, deltat0=2e-3, type_time_scheme=scheme)
    orc.init_from_rotfft(rot)
    orc.run(it_end=5)
    assert rel(sim.state.state_spect.cpu().numpy(), orc.state_spect) < 1e-12


@pytest.mark.parametrize("shape,beta,cfl", [
    ((64, 256), 2.0, True),     # 6 rows per CTA: 3 pairs of 256-point lines
    ((128, 512), 0.0, False),   # 3 rows per CTA: half-length real transforms
    ((32, 1024), 1.0, True),    # 1 row per CTA
    ((64, 64), 0.5, True)])     # 24 rows per CTA: 12 pairs of 64-point lines
def test_ns2d_fast_fp32_matches_oracle(cuda, shape, beta, cfl):
    """The ns2d FP32 x pass with and without rows in pairs."""
    from fluidsim_gb300.init_fields import noise_rot_2d
    from fluidsim_gb300.solvers import SimulNS2D
    from oracle.solvers import NS2DOracle
    from oracle.spectral import OperNumpy2D
    ny, nx = shape
    L = (2 * pi, 2 * pi * ny / nx)
    p = SimulNS2D.create_default_params()
    p.precision = "float32"
    p.oper.nx, p.oper.ny = nx, ny
    p.oper.Lx, p.oper.Ly = L
    p.nu_2, p.beta = 1e-3, beta
    ts = p.time_stepping
    ts.USE_CFL, ts.cfl_coef, ts.deltat0 = cfl, 0.5, 2e-3
    ts.USE_T_END, ts.it_end = False, 5
    sim = SimulNS2D(p)
    rot = noise_rot_2d(nx, ny, *L, kmin=3, kmax=10, seed=6)
    sim.init_from_rotfft(rot)
    sim.time_stepping.start()
    orc = NS2DOracle(OperNumpy2D(nx, ny, *L), beta=beta, nu_2=1e-3, USE_CFL=cfl,
                     cfl_coef=0.5, deltat0=2e-3)
    orc.init_from_rotfft(rot)
    orc.run(it_end=5)
    got = sim.state.state_spect.cpu().numpy().astype(np.complex128)
    assert rel(got, orc.state_spect) < 1e-5


@pytest.mark.parametrize("precision,shape", [("float32", (64, 64, 64)),
                                             ("float64", (64, 64, 64)),
                                             ("float32", (32, 32, 512))])
def test_pruned_step_is_bit_identical_and_detected(cuda, precision, shape):
    """gbs_ns_is_dealiased accepts only states that are +0 outside the 2/3
    box; on such a state the pruned step equals the unpruned one bit for
    bit."""
    import ctypes
    import torch
    from fluidsim_gb300 import _lib
    from fluidsim_gb300.fft import current_stream_handle
    from fluidsim_gb300.init_fields import isotropic_3d
    from fluidsim_gb300.solvers import SimulNS3D
    nz, ny, nx = shape
    L = (2 * pi,) * 3
    p = SimulNS3D.create_default_params()
    p.precision = precision
    p.oper.nx, p.oper.ny, p.oper.nz = nx, ny, nz
    p.oper.Lx, p.oper.Ly, p.oper.Lz = L
    p.nu_2 = 1e-3
    sim = SimulNS3D(p)
    v0 = isotropic_3d(nx, ny, nz, *L, seed=5)
    sim.state.init_statespect_from(vx_fft=v0[0], vy_fft=v0[1], vz_fft=v0[2])
    sim.oper.dealiasing(sim.state.state_spect)
    lib, h = sim._lib, sim._solver

    def is_dealiased(S):
        ok = ctypes.c_int()
        _lib.check(lib.gbs_ns_is_dealiased(h, ctypes.c_void_p(S.data_ptr()), ctypes.byref(ok),
                                           current_stream_handle()))
        return ok.value

    def step(S, flags):
        dt = ctypes.c_double(2e-3)
        _lib.check(lib.gbs_ns_step_rk4(h, ctypes.c_void_p(S.data_ptr()), ctypes.byref(dt),
                                       None, flags, current_stream_handle()))

    S = sim.state.state_spect
    assert is_dealiased(S) == 1
    a, b = S.clone(), S.clone()
    step(a, 0)
    step(b, _lib.GBS_STEP_DEALIASED)
    torch.cuda.synchronize()
    assert torch.equal(torch.view_as_real(a), torch.view_as_real(b))
    # a removed mode that is not +0 (a value, or -0.0) is detected
    kc = sim.oper.kcut[2]
    c = S.clone()
    c[1, 0, 0, kc] = 1e-30
    assert is_dealiased(c) == 0
    c[1, 0, 0, kc] = complex(-0.0, 0.0)
    assert is_dealiased(c) == 0
    c[1, 0, 0, kc] = 0
    assert is_dealiased(c) == 1


def test_x_pass_staging_timeout_is_reported(cuda):
    """The FP32 x pass at nx = 512 stages each field's rows by a bulk copy
    awaited on an mbarrier with a bounded wait.  The test hook withholds one
    copy: the wait runs out (1 ms), the step returns GBS_ETIMEDOUT once, the
    context stays usable and the next steps equal those of a fresh solver."""
    import ctypes
    import torch
    from fluidsim_gb300 import _lib
    from fluidsim_gb300.fft import current_stream_handle
    from fluidsim_gb300.init_fields import isotropic_3d
    from fluidsim_gb300.solvers import SimulNS3D
    nz, ny, nx = 32, 32, 512
    L = (2 * pi,) * 3

    def make():
        p = SimulNS3D.create_default_params()
        p.precision = "float32"
        p.oper.nx, p.oper.ny, p.oper.nz = nx, ny, nz
        p.oper.Lx, p.oper.Ly, p.oper.Lz = L
        p.nu_2 = 1e-3
        sim = SimulNS3D(p)
        v0 = isotropic_3d(nx, ny, nz, *L, seed=5)
        sim.state.init_statespect_from(vx_fft=v0[0], vy_fft=v0[1], vz_fft=v0[2])
        sim.oper.dealiasing(sim.state.state_spect)
        return sim

    def step(sim, S, flags):
        dt = ctypes.c_double(2e-3)
        return sim._lib.gbs_ns_step_rk4(sim._solver, ctypes.c_void_p(S.data_ptr()),
                                        ctypes.byref(dt), None, flags, current_stream_handle())

    base = _lib.GBS_STEP_CHECK_NAN | _lib.GBS_STEP_DEALIASED
    sim, ref = make(), make()
    S0 = sim.state.state_spect.clone()
    S = sim.state.state_spect
    assert step(sim, S, base | _lib.GBS_STEP_TEST_STALL) == _lib.GBS_ETIMEDOUT
    assert "staging copy" in _lib.load().gbs_last_error().decode()
    S.copy_(S0)
    for _ in range(2):
        assert step(sim, S, base) == _lib.GBS_OK
        assert step(ref, ref.state.state_spect, base) == _lib.GBS_OK
    torch.cuda.synchronize()
    assert torch.equal(torch.view_as_real(S), torch.view_as_real(ref.state.state_spect))
