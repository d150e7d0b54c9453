"""C ABI and host logic checks that need no GPU."""
import ctypes
import re
import subprocess
from math import pi
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "gbspec.h"


@pytest.fixture(scope="module")
def lib():
    from fluidsim_gb300 import _lib
    try:
        return _lib.load()
    except (OSError, RuntimeError, ImportError) as e:  # pragma: no cover
        pytest.fail(f"libgbspec.so cannot be built/loaded: {e}")


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+(gbs_\w+)\s*\(", text, re.M)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name
    from fluidsim_gb300 import _lib
    assert set(_lib.EXPORTED) == set(names)


def test_version(lib):
    assert b"sm_103a" in lib.gbs_version()


def test_cfl_update_matches_reference_rule(lib):
    """``fluidsim/base/time_stepping/base.py:334-354`` through the oracle."""
    from oracle.solvers import _SolverBase

    class Probe(_SolverBase):
        nvar = 1
        keys_phys = ("a",)

        def __init__(self, dt, cfl, dtmax):
            self.deltat, self.CFL, self.deltat_max = dt, cfl, dtmax

    rng = np.random.default_rng(0)
    for _ in range(2000):
        dt = rng.uniform(1e-4, 0.3)
        tmp = rng.choice([0.0, rng.uniform(0.1, 100.0)])
        cfl = rng.choice([0.5, 1.0, 0.4])
        dtmax = rng.choice([0.2, 0.01, 1.0])
        if rng.random() < 0.3:  # land near the 2 % hysteresis edge
            tmp = cfl / (dt * rng.choice([1.0199, 1.0201, 0.9801, 0.98]))
        probe = Probe(dt, cfl, dtmax)
        probe._cfl_from_tmp(tmp)
        assert lib.gbs_cfl_update(dt, tmp, cfl, dtmax) == probe.deltat


def test_ns_params_struct_layout(tmp_path):
    """ctypes mirror of gbs_ns_params has the C layout (sizes and offsets)."""
    from fluidsim_gb300._lib import NSParams
    src = tmp_path / "layout.c"
    fields = [f[0] for f in NSParams._fields_]
    body = "".join(f'printf("%zu ", offsetof(gbs_ns_params, {f}));' for f in fields)
    src.write_text(
        "#include <stdio.h>\n#include <stddef.h>\n#include \"gbspec.h\"\n"
        f"int main(void){{{body}printf(\"%zu\\n\", sizeof(gbs_ns_params));return 0;}}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    offs = [getattr(NSParams, f).offset for f in fields]
    assert out[:-1] == offs
    assert out[-1] == ctypes.sizeof(NSParams)


def test_invalid_arguments_are_rejected_without_gpu(lib):
    h = ctypes.c_void_p()
    shape = (ctypes.c_int64 * 3)(8, 8, 7)  # odd nx
    assert lib.gbs_fft_plan_create(3, shape, 1, 1, ctypes.byref(h)) == -22
    assert b"nx must be even" in lib.gbs_last_error()
    assert lib.gbs_fft_r2c(None, None, None, None) == -22
    assert lib.gbs_ns_step_rk4(None, None, None, None, 1, None) == -22


def test_dealias_cutoff_matches_oracle():
    from fluidsim_gb300.init_fields import cubic_dealias_cutoff
    from oracle.spectral import dealias_cutoff
    for n in list(range(2, 80)) + [128, 256, 512, 1024]:
        for L in (2 * pi, 6.0, 1.0, 4.5):
            for coef in (2.0 / 3, 0.5, 1.0, 0.8):
                assert cubic_dealias_cutoff(n, L, coef) == dealias_cutoff(n, L, coef)


def test_params_container():
    from fluidsim_gb300.params import Parameters
    p = Parameters("params", {"a": 1})
    p._set_child("oper", {"nx": 4})
    p.oper.nx = 8
    assert p.oper.nx == 8 and p["a"] == 1
    with pytest.raises(AttributeError):
        p.oper.nz = 3


def test_default_params_mirror_reference():
    from fluidsim_gb300.solvers import SimulNS2D, SimulNS3D
    p3 = SimulNS3D.create_default_params()
    assert p3.oper.coef_dealiasing == 2.0 / 3 and p3.oper.Lx == 2 * pi
    assert p3.time_stepping.USE_CFL is True and p3.time_stepping.type_time_scheme == "RK4"
    assert p3.f is None and p3.nu_8 == 0.0
    p2 = SimulNS2D.create_default_params()
    assert p2.oper.Lx == 8 and p2.beta == 0.0


def test_import_fft_class():
    from fluidsim_gb300 import FFT2DGB300, FFT3DGB300, import_fft_class
    assert import_fft_class("fluidfft.fft3d.with_gb300") is FFT3DGB300
    assert import_fft_class("default", 2) is FFT2DGB300
    with pytest.raises(ValueError):
        import_fft_class("fft3d.with_fftw3d")
