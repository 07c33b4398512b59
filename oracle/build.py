"""ORACLE — test infrastructure only.  Builds liborc.so from cic_oracle.c.

gcc -O2 -ffp-contract=off keeps every product and sum separately rounded, as
in the reference's x86-64 build (no FMA).  Output goes to oracle/_build/.
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "cic_oracle.c"
OUT = HERE / "_build" / "liborc.so"


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


if __name__ == "__main__":
    print(build())
