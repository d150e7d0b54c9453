"""fluidsim_gb300 — fluidsim's pseudo-spectral time step on one GB300.

The R2C/C2R transforms (fluidfft ``fft2d`` / ``fft3d`` plugin classes), the
ns2d / ns3d nonlinear tendencies and the exponential-integrating-factor RK4
step run as hand-written sm_103a CUDA kernels in ``libgbspec.so``, called
through the C ABI declared in ``include/gbspec.h``.  There is no CPU
fallback: without the library (or a GPU) the classes raise.
"""

from .fft import FFT2DGB300, FFT3DGB300, import_fft_class
from .params import Parameters

__all__ = ["FFT2DGB300", "FFT3DGB300", "import_fft_class", "Parameters",
           "SimulNS2D", "SimulNS2DStrat", "SimulNS2DBouss", "SimulNS3D", "SimulNS3DStrat",
           "SimulNS3DBouss"]


def __getattr__(name):
    if name in __all__[4:]:
        from . import solvers
        return getattr(solvers, name)
    raise AttributeError(name)
