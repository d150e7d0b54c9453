"""fluidfft method ``fft2d.with_gb300``: 2D R2C/C2R on one GB300."""
from ..fft import FFT2DGB300 as FFTclass

__all__ = ["FFTclass"]
