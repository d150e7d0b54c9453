"""fluidfft plugin modules: one module per FFT class, each exposing it as
``FFTclass``, the attribute fluidfft's ``import_fft_class`` reads from the
module an entry point of the ``fluidfft.plugins`` group names."""
