"""FP64 spectra on the GPU against the oracle's restatement.

fluidsim's spectra outputs call the operator methods compute_1dspectra,
compute_3dspectrum and compute_spectrum_kzkh (3D,
``fluidsim/solvers/ns3d/output/spectra.py:15-100``) and spectra1D_from_fft /
spectrum2D_from_fft (2D, ``fluidsim/solvers/ns2d/output/spectra.py:16-27``).
The GPU computes them with the ``gbs_spectra`` kernel (FP64 accumulation for
FP32 or FP64 inputs); ``oracle/spectral.py`` restates the same definitions in
numpy.  Random energy arrays on cubic and non-cubic boxes, and the energy and
enstrophy spectra of solver states, must agree within 1e-12 (relative to the
largest bin of each spectrum).
"""
from math import pi

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


def close(got, ref):
    got = got.cpu().numpy() if hasattr(got, "cpu") else np.asarray(got)
    assert got.shape == ref.shape, (got.shape, ref.shape)
    return np.abs(got - ref).max() <= TOL * np.abs(ref).max()


def oper3d(nz, ny, nx, L):
    from fluidsim_gb300.operators import OperatorsPseudoSpectral3D
    from fluidsim_gb300.params import Parameters
    p = Parameters("params")
    OperatorsPseudoSpectral3D._complete_params_with_default(p)
    p.oper.nx, p.oper.ny, p.oper.nz = nx, ny, nz
    p.oper.Lx, p.oper.Ly, p.oper.Lz = L
    return OperatorsPseudoSpectral3D(p, precision="float64")


def oper2d(ny, nx, L):
    from fluidsim_gb300.operators import OperatorsPseudoSpectral2D
    from fluidsim_gb300.params import Parameters
    p = Parameters("params")
    OperatorsPseudoSpectral2D._complete_params_with_default(p)
    p.oper.nx, p.oper.ny = nx, ny
    p.oper.Lx, p.oper.Ly = L
    return OperatorsPseudoSpectral2D(p, precision="float64")


@pytest.mark.parametrize("shape,L", [((16, 20, 24), (2 * pi, 2 * pi, 2 * pi)),
                                     ((32, 32, 64), (4 * pi, 2 * pi, 3.0)),
                                     ((64, 48, 40), (1.0, 2.0, 1.5)),
                                     ((128, 128, 128), (2 * pi,) * 3)])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_spectra_3d_match_oracle(cuda, shape, L, dtype):
    import torch
    from oracle.spectral import OperNumpy3D
    nz, ny, nx = shape
    op = oper3d(nz, ny, nx, L)
    orc = OperNumpy3D(nx, ny, nz, *L)
    e = np.random.default_rng(sum(shape)).random(orc.shapeK).astype(dtype)
    e[np.random.default_rng(1).random(orc.shapeK) < 0.2] = 0.0  # some empty modes
    ref_e = e.astype(np.float64)
    dev = torch.from_numpy(e).cuda()
    for got, ref in zip(op.compute_1dspectra(dev), orc.compute_1dspectra(ref_e)):
        assert close(got, ref)
    assert close(op.compute_3dspectrum(dev), orc.compute_3dspectrum(ref_e))
    assert close(op.compute_spectrum_kzkh(dev), orc.compute_spectrum_kzkh(ref_e))


@pytest.mark.parametrize("shape,L", [((40, 48), (2 * pi, 2 * pi)), ((64, 30), (3.0, 5.0)),
                                     ((512, 512), (2 * pi, 2 * pi))])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_spectra_2d_match_oracle(cuda, shape, L, dtype):
    import torch
    from oracle.spectral import OperNumpy2D
    ny, nx = shape
    op = oper2d(ny, nx, L)
    orc = OperNumpy2D(nx, ny, *L)
    e = np.random.default_rng(sum(shape)).random(orc.shapeK).astype(dtype)
    ref_e = e.astype(np.float64)
    dev = torch.from_numpy(e).cuda()
    for got, ref in zip(op.spectra1D_from_fft(dev), orc.spectra1D_from_fft(ref_e)):
        assert close(got, ref)
    assert close(op.spectrum2D_from_fft(dev), orc.spectrum2D_from_fft(ref_e))


def test_energy_spectra_of_a_state_match_oracle(cuda):
    """The spectra fluidsim's ns3d output computes from a state
    (``ns3d/output/spectra.py:17-41``): per-component energy arrays
    0.5 |v_i|^2 -> 1D spectra and shells; the benchmark workload's initial field at 64^3."""
    import torch
    import bench
    from oracle.spectral import OperNumpy3D
    n = 64
    v0 = bench.initial_state(n)
    op = oper3d(n, n, n, (2 * pi,) * 3)
    orc = OperNumpy3D(n, n, n)
    V = torch.from_numpy(v0).cuda()
    for i in range(3):
        e_dev = 0.5 * V[i].abs() ** 2
        e_ref = 0.5 * np.abs(v0[i]) ** 2
        for got, ref in zip(op.compute_1dspectra(e_dev), orc.compute_1dspectra(e_ref)):
            assert close(got, ref)
        assert close(op.compute_3dspectrum(e_dev), orc.compute_3dspectrum(e_ref))
