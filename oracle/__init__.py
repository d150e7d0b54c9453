"""CPU float64 oracle for the pseudo-spectral time step (TEST INFRASTRUCTURE).

This package is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline / reference arm
may import it.  The GPU product path (``fluidsim_gb300``) never calls into it
and fails loudly when its CUDA library is missing.

Contents
--------
``spectral``  numpy/scipy.fft restatement of the fluidfft 0.4.2 operator
              subset the fluidsim hot path calls (R2C/C2R normalisation,
              wavenumber arrays, cubic 2/3 dealiasing, curl, vector product,
              perpendicular projection, Hermitian-weighted sums, spectra).
``solvers``   restatement of ns2d/ns3d ``tendencies_nonlin``, the
              exponential-integrating-factor RK4 of
              ``TimeSteppingPseudoSpectral`` and the CFL time increment.
``refshim``   loads the reference's *own* Python files for the RK4 loop and
              the ns2d/ns3d tendencies (fluidsim 0.8.3) on top of small
              shims, so golden fixtures come from the reference's code
              itself.  Only usable where the reference sources exist.

Parity status
-------------
The RK4 / tendency / CFL logic is pinned against the reference's own code
through ``refshim`` (fixtures under ``tests/golden``).  The FFT-library
arithmetic lives in fluidfft 0.4.2, which is not vendored: the restated
mathematics (DFT, curl, projection, cubic mask with ``>=``, Hermitian sums)
is pinned by the identities the reference tests assert (Parseval, energy
and enstrophy conservation of the tendencies, curl/vecfft round trips,
index layout), not by bit-level fluidfft outputs.
"""
