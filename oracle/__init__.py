"""ORACLE — test infrastructure only.

CPU restatement of the reference's LDL hot path (CIC paint/readout in C,
FFT conventions over numpy, the FP64 LDL pipeline and both gradient
conventions).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline use it, always as the checker.  The product (jerald_gb300) never
imports it.  Parity unpinned against the reference binary, which cannot be
built here (it needs MPI and FFTW); pinned instead by the known-answer tests
in tests/test_oracle.py and the committed fixtures in tests/golden/.
"""
from . import cic, fft  # noqa: F401
from .ldl import LDLOracle  # noqa: F401
