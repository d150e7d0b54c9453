"""Host emulation of the CUDA FFT core (no GPU): index arithmetic check.

``tests/cpu/core_harness.cpp`` compiles the ``__host__ __device__`` stage
functions of ``gbs_core.cuh`` with g++ and drives every thread id of the CTA
in turn between the barriers, so the Stockham stage / direct-DFT indexing of
the interleaved tile layout is checked against numpy.fft on the CPU.
"""
import ctypes
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    out = tmp_path_factory.mktemp("core") / "core_harness.so"
    cmd = ["g++", "-O1", "-std=c++17", "-shared", "-fPIC",
           "-I/usr/local/cuda/include", str(HERE / "cpu" / "core_harness.cpp"),
           "-o", str(out)]
    try:
        subprocess.run(cmd, check=True, capture_output=True)
    except (OSError, subprocess.CalledProcessError) as e:  # pragma: no cover
        pytest.skip(f"cannot build the host harness: {e}")
    lib = ctypes.CDLL(str(out))
    lib.emulate_fft_tile.restype = ctypes.c_int
    return lib


def _twiddles(n):
    k = np.arange(n)
    return np.exp(-2j * np.pi * k / n).astype(np.complex128)


@pytest.mark.parametrize("n", [2, 3, 5, 8, 10, 15, 16, 32, 64, 128, 256, 512, 1024])
@pytest.mark.parametrize("dir_", [-1, 1])
def test_fft_tile_matches_numpy(harness, n, dir_):
    rng = np.random.default_rng(n)
    nlines, LP = 5, 7
    nthreads = max(64, ((nlines * max(n // 8, 1) + 1) // 2 + 31) // 32 * 32)
    x = rng.standard_normal((n, nlines)) + 1j * rng.standard_normal((n, nlines))
    buf = np.zeros((n, LP), np.complex128)
    buf[:, :nlines] = x
    buf = np.ascontiguousarray(buf)
    tw = _twiddles(n)
    rc = harness.emulate_fft_tile(
        n, nlines, LP, dir_, nthreads,
        buf.ctypes.data_as(ctypes.c_void_p), tw.ctypes.data_as(ctypes.c_void_p), 1)
    assert rc == 0
    ref = np.fft.fft(x, axis=0) if dir_ < 0 else np.fft.ifft(x, axis=0) * n
    err = np.abs(buf[:, :nlines] - ref).max() / np.abs(ref).max()
    assert err < 1e-14 * max(1, np.log2(n)), err


def test_twiddle_stride_half_length(harness):
    """The x pass runs an M = nx/2 point FFT on the nx-entry table (stride 2)."""
    nx, nlines = 64, 3
    M = nx // 2
    rng = np.random.default_rng(0)
    x = rng.standard_normal((M, nlines)) + 1j * rng.standard_normal((M, nlines))
    buf = np.ascontiguousarray(x.copy())
    tw = _twiddles(nx)
    rc = harness.emulate_fft_tile(
        M, nlines, nlines, -1, 64,
        buf.ctypes.data_as(ctypes.c_void_p), tw.ctypes.data_as(ctypes.c_void_p), 2)
    assert rc == 0
    assert np.allclose(buf, np.fft.fft(x, axis=0), rtol=0, atol=1e-13)
