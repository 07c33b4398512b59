"""Writes tests/golden/ref_hashes.json: sha256 digests of the reference's own
CIC outputs (oracle/_ref/libjldref.so, compiled from the reference's
lib/parops_fast.h by oracle/build.py) on the seeded cases of
oracle/pin_inputs.py.

The inputs regenerate bit for bit on any host, so a digest stands for the
whole output array: the GPU tests compare the digests of the CUDA readouts
with these directly (bit-exact), and the digests of the oracle's paints with
them before comparing the CUDA paints with the oracle's within tolerance.

Run from the repository root where the reference checkout is present:
    python tests/golden/make_ref_hashes.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import pin_inputs, ref  # noqa: E402

OUT = Path(__file__).resolve().parent / "ref_hashes.json"


def main() -> None:
    if not ref.available():
        raise SystemExit("the reference checkout is needed to make these fixtures")
    table = {}
    for name in pin_inputs.CASES:
        outs = pin_inputs.outputs(ref, name)
        table[name] = {k: pin_inputs.digest(v) for k, v in outs.items()}
        table[name]["nparts"] = int(len(pin_inputs.positions(name)))
        print(name, table[name]["nparts"], flush=True)
    OUT.write_text(json.dumps({"source": "reference lib/parops_fast.h via oracle/_ref, world size one",
                               "cases": table}, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    main()
