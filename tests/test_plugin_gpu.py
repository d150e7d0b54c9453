"""Drop-in check: the restated reference solvers with the plugin as their FFT.

A fluidsim operator calls its fluidfft object through ``fft_as_arg`` /
``ifft_as_arg`` on host numpy arrays (``ns3d/solver.py:210-241``,
``ns2d/solver.py:161-181``, ``base/state.py:318-333``).  Here the numpy
operator under the oracle's ns2d / ns3d solvers (the reference's tendencies
and IF-RK4 restated, pinned to fixtures that the reference's own code made)
gets ``FFTclass`` of the packaged entry-point module as its transform, and the
fixtures' 10-step states must come out within 1e-12.
"""
import importlib

import numpy as np
import pytest

from test_oracle_golden import make_oracle, rel

pytestmark = pytest.mark.gpu


def plug_in(oper, method):
    from fluidsim_gb300.fft import PLUGIN_MODULES
    fft_obj = importlib.import_module(PLUGIN_MODULES[method]).FFTclass(*oper.shapeX)
    assert fft_obj.get_shapeK_seq() == oper.shapeK

    def fft(fieldX):
        fieldK = np.empty(oper.shapeK, np.complex128)
        fft_obj.fft_as_arg(np.ascontiguousarray(fieldX), fieldK)
        return fieldK

    def ifft(fieldK):
        fieldX = np.empty(oper.shapeX)
        fft_obj.ifft_as_arg(np.ascontiguousarray(fieldK), fieldX)
        return fieldX
    oper.fft, oper.ifft = fft, ifft
    return fft_obj


@pytest.mark.parametrize("name", ["ns2d_32_cfl", "ns2d_256_c1", "ns3d_20x15x10",
                                  "ns3d_tgv_32", "ns3d_iso_24x16x32_f"])
def test_oracle_solver_on_plugin_fft_matches_fixture(cuda, name):
    orc, d, p = make_oracle(name)
    plug_in(orc.oper, "fft2d.with_gb300" if name.startswith("ns2d") else "fft3d.with_gb300")
    for it in range(int(p["steps"])):
        orc.one_time_step()
        assert abs(orc.deltat - d["dts"][it]) <= 1e-12 * d["dts"][it]
    assert rel(orc.state_spect, d["S_end"]) < 1e-12
