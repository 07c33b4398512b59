"""ORACLE — test infrastructure only.  Builds the oracle's C libraries.

build(): liborc.so from cic_oracle.c.  gcc -O2 -ffp-contract=off keeps every
product and sum separately rounded, as in the reference's x86-64 build (no
FMA).  Output goes to oracle/_build/.

build_ref(): libjldref.so from the reference's own CIC header
(lib/parops_fast.h of maurorigo/JERALD, read where it lies under the
reference checkout) through ref_shim.cc, with ref_stub/mpi.h for MPI at world
size one.  Output goes to oracle/_ref/.  It returns None when the reference
checkout is absent (the GPU hosts have none): the tests that need the
library skip, and the hash fixtures made from it stay the link to the
reference there.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "cic_oracle.c"
OUT = HERE / "_build" / "liborc.so"

REF_ROOT = Path(os.environ.get("JLD_REFERENCE_ROOT", "/root/reference"))
REF_HEADER = REF_ROOT / "lib" / "parops_fast.h"
REF_SHIM = HERE / "ref_shim.cc"
REF_STUB = HERE / "ref_stub"
REF_OUT = HERE / "_ref" / "libjldref.so"


def build() -> Path:
    OUT.parent.mkdir(exist_ok=True)
    if OUT.exists() and OUT.stat().st_mtime >= SRC.stat().st_mtime:
        return OUT
    cc = shutil.which("gcc") or "cc"
    cmd = [cc, "-O2", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC",
           str(SRC), "-o", str(OUT), "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return OUT


def build_ref() -> Path | None:
    """Compiles the reference's CIC loops into oracle/_ref/libjldref.so, or
    returns the existing library (None when neither it nor the reference
    source is there)."""
    if not REF_HEADER.exists():
        return REF_OUT if REF_OUT.exists() else None
    REF_OUT.parent.mkdir(exist_ok=True)
    deps = [REF_HEADER, REF_SHIM, REF_STUB / "mpi.h"]
    if REF_OUT.exists() and REF_OUT.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return REF_OUT
    cxx = shutil.which("g++") or "c++"
    cmd = [cxx, "-O2", "-ffp-contract=off", "-fno-fast-math", "-std=c++17", "-w", "-shared", "-fPIC",
           "-I", str(REF_STUB), "-I", str(REF_HEADER.parent), str(REF_SHIM), "-o", str(REF_OUT)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference CIC build failed:\n{r.stdout}\n{r.stderr}")
    return REF_OUT


if __name__ == "__main__":
    print(build())
    print(build_ref())
