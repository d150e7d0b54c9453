"""The packaged fluidfft plugin: entry points and class resolution (CPU).

fluidfft resolves ``params.oper.type_fft`` through the ``fluidfft.plugins``
entry-point group (``Makefile:13-14``, ``operators/test/test_operators3d.py:
16-31``); each entry point names a module that exposes ``FFTclass``.
"""
import importlib
import tomllib

import pytest

from conftest import ROOT


def entry_points():
    meta = tomllib.loads((ROOT / "pyproject.toml").read_text())
    return meta["project"]["entry-points"]["fluidfft.plugins"]


def test_pyproject_declares_both_plugin_modules():
    from fluidsim_gb300.fft import PLUGIN_MODULES
    assert entry_points() == PLUGIN_MODULES


@pytest.mark.parametrize("method,cls", [("fft2d.with_gb300", "FFT2DGB300"),
                                        ("fft3d.with_gb300", "FFT3DGB300")])
def test_entry_point_modules_expose_fftclass(method, cls):
    import fluidsim_gb300
    mod = importlib.import_module(entry_points()[method])
    assert mod.FFTclass is getattr(fluidsim_gb300, cls)
    for name in (method, "fluidfft." + method):
        assert fluidsim_gb300.import_fft_class(name) is mod.FFTclass


def test_default_names_and_unknown_method():
    from fluidsim_gb300 import FFT2DGB300, FFT3DGB300, import_fft_class
    assert import_fft_class("default", dim=2) is FFT2DGB300
    assert import_fft_class("sequential", dim=3) is FFT3DGB300
    with pytest.raises(ValueError, match="unknown FFT class"):
        import_fft_class("fft3d.with_fftw3d")
