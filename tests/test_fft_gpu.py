"""GPU parity of the R2C / C2R plugin classes against numpy / scipy."""
import numpy as np
import pytest
import scipy.fft as sfft

pytestmark = pytest.mark.gpu

SHAPES = [(16, 16), (40, 48), (15, 20), (256, 256), (8, 12, 10), (10, 15, 20),
          (32, 32, 32), (64, 48, 40), (128, 128, 128), (4, 6, 2), (1, 8, 8),
          # the 512-point column and row kernels of the 512^3 benchmark step
          (512, 512), (512, 512, 16), (16, 16, 512), (512, 512, 512),
          # 1024-point columns (one exchange slot)
          (1024, 64), (1024, 64, 32), (32, 1024, 64)]
TOL = {"float64": 1e-13, "float32": 3e-6}


def _cls(shape):
    from fluidsim_gb300 import FFT2DGB300, FFT3DGB300
    return FFT2DGB300 if len(shape) == 2 else FFT3DGB300


def relmax(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("precision", ["float64", "float32"])
def test_forward_and_inverse(cuda, shape, precision):
    import torch
    op = _cls(shape)(*shape, precision=precision)
    rng = np.random.default_rng(sum(shape))
    x = rng.standard_normal(shape)
    N = np.prod(shape)
    ref = sfft.rfftn(x) / N
    X = torch.from_numpy(x).cuda().to(op.rdtype)
    K = op.fft(X)
    assert relmax(K.cpu().numpy(), ref) < TOL[precision] * (1 + np.log2(N))
    back = op.ifft(K)
    assert relmax(back.cpu().numpy(), x) < TOL[precision] * (1 + np.log2(N))


@pytest.mark.parametrize("shape", [(12, 16), (8, 12, 10), (32, 32, 32)])
def test_c2r_non_hermitian_input_matches_scipy(cuda, shape):
    """C2R keeps only the real part of the kx = 0 / Nyquist columns, like irfftn."""
    import torch
    op = _cls(shape)(*shape)
    rng = np.random.default_rng(1)
    K = rng.standard_normal(op.shapeK) + 1j * rng.standard_normal(op.shapeK)
    ref = sfft.irfftn(K, s=shape) * np.prod(shape)
    Kd = torch.from_numpy(K).cuda()
    keep = Kd.clone()
    X = op.create_arrayX()
    op.ifft_as_arg(Kd, X)
    assert torch.equal(Kd, keep)  # ifft_as_arg preserves its input
    assert relmax(X.cpu().numpy(), ref) < 1e-12
    op.ifft_as_arg_destroy(Kd, X)
    assert relmax(X.cpu().numpy(), ref) < 1e-12


@pytest.mark.parametrize("shape", [(24, 32), (16, 12, 8)])
def test_batched_fields_and_host_arrays(cuda, shape):
    import torch
    op = _cls(shape)(*shape)
    rng = np.random.default_rng(2)
    x = rng.standard_normal((3,) + shape)
    ref = sfft.rfftn(x, axes=tuple(range(1, len(shape) + 1))) / np.prod(shape)
    K = torch.empty((3,) + op.shapeK, dtype=torch.complex128, device="cuda")
    op.fft_as_arg(torch.from_numpy(x).cuda(), K)
    assert relmax(K.cpu().numpy(), ref) < 1e-13
    # numpy in, numpy out (host path)
    k1 = np.empty(op.shapeK, np.complex128)
    op.fft_as_arg(x[1], k1)
    assert relmax(k1, ref[1]) < 1e-13
    x1 = np.empty(shape)
    op.ifft_as_arg(k1, x1)
    assert relmax(x1, x[1]) < 1e-13


def test_parseval_and_sum_wavenumbers(cuda):
    import torch
    from fluidsim_gb300 import FFT3DGB300
    op = FFT3DGB300(12, 10, 16)
    v = torch.randn(op.shapeX, dtype=torch.float64, device="cuda")
    vk = op.fft(v)
    assert np.isclose(op.sum_wavenumbers(vk.abs() ** 2 / 2), float((v**2).mean() / 2))


def test_bad_arguments_raise(cuda):
    import torch
    from fluidsim_gb300 import FFT3DGB300
    op = FFT3DGB300(8, 8, 8)
    with pytest.raises(ValueError):
        op.fft_as_arg(torch.zeros((8, 8, 9), dtype=torch.float64, device="cuda"),
                      op.create_arrayK())
    with pytest.raises(ValueError):
        op.fft_as_arg(op.create_arrayX().to(torch.float32), op.create_arrayK())
