"""CPU f64 oracle for the optics-studio propagation hot path.

TEST INFRASTRUCTURE ONLY.  This package restates, in numpy float64, the
algorithms of the reference Rust crates (optics-core ``src/`` and
``crates/optics-inverse/src/``) so that the CUDA product can be checked
against them.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` may import it; the product path
(``optics_studio_gb300``) never does.

Every function cites the reference ``file:line`` it follows.  The FFT in
the reference is the third-party crate ``rustfft`` 6.4.1 (Cargo.lock:6500),
which is not vendored; its published algorithm is the unnormalised DFT with
kernel e^{-2 pi i k n / N}.  The reference wraps it in the NumPy scaling
convention (``src/propagation/fft.rs:1-33``: unnormalised forward, 1/N
inverse, unshifted bins), so ``numpy.fft`` (pocketfft) computes the same
transform; the convention pins of ``fft.rs:159-259`` are re-run against it
in ``tests/test_oracle_pins.py``.

Parity pins (see ``tests/test_oracle_pins.py``):
  * the reference's own known-answer tests for this path
    (``src/propagation/*.rs`` test modules, ``tests/asm.rs``,
    ``crates/optics-inverse/src/{gs,adjoint}.rs`` test modules);
  * the only external golden vector of the reference,
    ``crates/optics-inverse/tests/data/hypercam/forward.npy`` (copied to
    ``tests/golden/hypercam/`` by ``tests/golden/make_hypercam.py``), which
    pins ASM + sampled PhaseMask + ThinLens relay + Gaussian source + scene
    finite-difference channels to 1e-6 of peak
    (``crates/optics-inverse/tests/hypercam_forward.rs:89-207``).
"""

from . import fft, field, asm, fresnel, fraunhofer, rs, element, beamline  # noqa: F401
from . import carrier, observe, merit, gs, adjoint, adam, analysis  # noqa: F401
