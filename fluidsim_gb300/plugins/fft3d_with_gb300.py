"""fluidfft method ``fft3d.with_gb300``: 3D R2C/C2R on one GB300."""
from ..fft import FFT3DGB300 as FFTclass

__all__ = ["FFTclass"]
