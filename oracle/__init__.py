"""ORACLE — test infrastructure only.

CPU restatement of the reference's LDL hot path (CIC paint/readout in C,
FFT conventions over numpy, the FP64 LDL pipeline and both gradient
conventions).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline use it, always to check results against.  The product
(jerald_gb300) never imports it.  The CIC loops are pinned to the
reference's own code: build.build_ref() compiles the reference's CIC header
with a world-size-one MPI stand-in into oracle/_ref/, and
tests/test_ref_pin.py requires bit-equal outputs.  The FFT conventions and
the model math stay unpinned (the reference needs FFTW-MPI and JAX, neither
present); the known-answer tests in tests/test_oracle.py and the committed
fixtures in tests/golden/ hold them.
"""
from . import cic, fft  # noqa: F401
from .ldl import LDLOracle  # noqa: F401
