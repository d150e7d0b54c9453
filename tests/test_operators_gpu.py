"""Operator helpers outside the fused step: spectra, projections, grids.

Properties the reference's operator tests check (``test_operators3d.py``,
``test_operators2d.py``): sums of spectra equal the energy (Parseval, the
``base/state.py:385-392`` normalisation), projections leave a divergence-free
field, z-invariant arrays transform to the kz = 0 plane.
"""
from math import pi

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _oper3d(nx=24, ny=20, nz=16, L=(2 * pi, 3.0, 2.5)):
    from fluidsim_gb300.operators import OperatorsPseudoSpectral3D
    from fluidsim_gb300.params import Parameters
    p = Parameters("params")
    OperatorsPseudoSpectral3D._complete_params_with_default(p)
    p.oper.nx, p.oper.ny, p.oper.nz = nx, ny, nz
    p.oper.Lx, p.oper.Ly, p.oper.Lz = L
    return OperatorsPseudoSpectral3D(p, precision="float64")


def _oper2d(nx=32, ny=24):
    from fluidsim_gb300.operators import OperatorsPseudoSpectral2D
    from fluidsim_gb300.params import Parameters
    p = Parameters("params")
    OperatorsPseudoSpectral2D._complete_params_with_default(p)
    p.oper.nx, p.oper.ny = nx, ny
    return OperatorsPseudoSpectral2D(p, precision="float64")


def test_spectra_3d_sum_to_energy(cuda):
    import torch
    op = _oper3d()
    torch.manual_seed(0)
    u = op.create_arrayX_random(-1, 1)
    u_fft = op.fft(u)
    e_fft = 0.5 * u_fft.abs() ** 2
    E = 0.5 * float((u.double() ** 2).mean())
    assert abs(op.sum_wavenumbers(e_fft) - E) < 1e-12 * E
    skx, sky, skz = op.compute_1dspectra(e_fft)
    assert abs(float(skx.sum()) * op.deltakx - E) < 1e-12 * E
    assert abs(float(sky.sum()) * op.deltaky - E) < 1e-12 * E
    assert abs(float(skz.sum()) * op.deltakz - E) < 1e-12 * E
    dk = min(op.deltakx, op.deltaky, op.deltakz)
    assert abs(float(op.compute_3dspectrum(e_fft).sum()) * dk - E) < 1e-12 * E
    kzkh = op.compute_spectrum_kzkh(e_fft)
    assert abs(float(kzkh.sum()) * op.deltakz * min(op.deltakx, op.deltaky) - E) < 1e-12 * E


def test_shell_spectrum_bins(cuda):
    """A single mode lands in bin round(|k| / dk) with its Hermitian weight."""
    import torch
    op = _oper3d(16, 16, 16, (2 * pi,) * 3)
    e = torch.zeros(op.shapeK, dtype=torch.float64, device="cuda")
    e[2, 3, 1] = 1.0  # kz = 2, ky = 3, kx = 1: |k| = sqrt(14) -> bin 4, weight 2
    e[0, 0, 8] = 1.0  # Nyquist x column: weight 1, |k| = 8
    s = op.compute_3dspectrum(e).cpu().numpy()
    assert s[4] == 2.0 and s[8] == 1.0 and s.sum() == 3.0


def test_projections_and_curl_identities(cuda):
    import torch
    op = _oper3d()
    torch.manual_seed(1)
    v = [op.fft(op.create_arrayX_random(-1, 1)) for _ in range(3)]
    op.project_perpk3d(*v)
    div = op.divfft_from_vecfft(*v)
    assert float(div.abs().max()) < 1e-13 * float(v[0].abs().max())
    g = op.gradfft_from_fft(v[0])
    rot = op.rotfft_from_vecfft(*g)
    assert max(float(r.abs().max()) for r in rot) < 1e-13 * float(g[0].abs().max())
    urx, ury, udx, udy = op.urudfft_from_vxvyfft(v[0], v[1])
    assert torch.allclose(urx + udx, v[0]) and torch.allclose(ury + udy, v[1])
    kh_div = op.Kx * urx + op.Ky * ury
    assert float(kh_div.abs().max()) < 1e-12 * float(v[0].abs().max())

    op2 = _oper2d()
    fx = op2.fft(op2.create_arrayX_random(-1, 1))
    fy = op2.fft(op2.create_arrayX_random(-1, 1))
    op2.projection_perp(fx, fy)
    assert float(op2.divfft_from_vecfft(fx, fy).abs().max()) < 1e-13 * float(fx.abs().max())
    e2 = 0.5 * (fx.abs() ** 2 + fy.abs() ** 2)
    E2 = op2.sum_wavenumbers(e2)
    skx, sky = op2.compute_1dspectra(e2)
    assert abs(float(skx.sum()) * op2.deltakx - E2) < 1e-12 * E2
    assert abs(float(sky.sum()) * op2.deltaky - E2) < 1e-12 * E2
    assert abs(float(op2.compute_2dspectrum(e2).sum()) * min(op2.deltakx, op2.deltaky)
               - E2) < 1e-12 * E2


def test_invariant_arrays_and_grids(cuda):
    import torch
    op = _oper3d()
    a2 = torch.rand((op.ny, op.nx), dtype=torch.float64, device="cuda")
    a3 = op.build_invariant_arrayX_from_2d_indices12X(a2)
    assert a3.shape == op.shapeX and torch.equal(a3[5], a2)
    k3 = op.fft(a3)
    a2_fft = torch.fft.rfft2(a2) / (op.nx * op.ny)
    assert torch.allclose(op.build_invariant_arrayK_from_2d_indices12X(a2_fft), k3, atol=1e-14)
    X, Y, Z = op.get_XYZ_loc()
    assert X.shape == op.shapeX
    assert float(X[0, 0, 1]) == pytest.approx(op.deltax)
    assert float(Y[0, 1, 0]) == pytest.approx(op.deltay)
    assert float(Z[1, 0, 0]) == pytest.approx(op.deltaz)
    ax, ay, az = (torch.rand(op.shapeX, dtype=torch.float64, device="cuda") for _ in range(3))
    px, py, pz = op.vector_product(ax, ay, az, ax, ay, az)
    assert float(max(px.abs().max(), py.abs().max(), pz.abs().max())) == 0.0
