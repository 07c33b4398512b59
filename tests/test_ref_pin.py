"""The oracle against the reference's own CIC code (CPU).

oracle/_ref/libjldref.so is the reference's lib/parops_fast.h compiled from
its source (world size one, oracle/build.py).  Where it is present the
oracle's C restatement must equal it bit for bit: on the committed CIC
fixtures (with their edge cases: grid points, box edges, tiny negatives that
round to L) and on the seeded pin cases.  Everywhere, the oracle must
reproduce the digests that the reference's outputs left in
tests/golden/ref_hashes.json, which carries the pin to hosts without the
reference checkout.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import cic, pin_inputs, ref

G = Path(__file__).resolve().parent / "golden"
HASHES = json.loads((G / "ref_hashes.json").read_text())["cases"]
SMALL = [n for n in pin_inputs.CASES if not n.startswith("clustered_256")]

needs_ref = pytest.mark.skipif(not ref.available(), reason="reference checkout absent: oracle/_ref not built")


@pytest.fixture(autouse=True)
def _serial_oracle():
    # the digests are of the reference's serial loops: paint in particle order
    cic.set_threads(1)
    yield


@needs_ref
@pytest.mark.parametrize("name", ["cic_f32.npz", "cic_f64.npz"])
def test_oracle_equals_reference_on_fixtures(name):
    f = np.load(G / name)
    nm, box = tuple(int(v) for v in f["nmesh"]), tuple(f["box"])
    pm = f["mesh_pos"]
    np.testing.assert_array_equal(cic.paint(pm, f["mass"], nm), ref.paint(pm, f["mass"], nm))
    np.testing.assert_array_equal(cic.paint3d(pm, f["mass3"], nm), ref.paint3d(pm, f["mass3"], nm))
    for d in (-1, 0, 1, 2):
        np.testing.assert_array_equal(cic.readout(pm, f["field"], nm, box, d),
                                      ref.readout(pm, f["field"], nm, box, d))
    np.testing.assert_array_equal(cic.readout3d(pm, f["field3"], nm, box, False),
                                  ref.readout3d(pm, f["field3"], nm, box, False))
    np.testing.assert_array_equal(cic.readout3d(pm, f["field"], nm, box, True),
                                  ref.readout3d(pm, f["field"], nm, box, True))


@needs_ref
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_oracle_equals_reference_on_edges(dt):
    # positions at and just below N (float32 rounds them to N: the reference
    # then drops the lower corner), exact grid points and the origin
    nm, box = (8, 6, 4), (8.0, 3.0, 2.0)
    vals = np.array([0.0, 1.0, 3.5, 7.999999, 8.0 - 1e-9, 5.0], dtype=np.float64)
    grid = np.stack(np.meshgrid(vals, vals * 0.75, vals * 0.5, indexing="ij"), -1).reshape(-1, 3)
    pm = np.minimum(grid, np.asarray(nm, dtype=np.float64)).astype(dt)
    rng = np.random.default_rng(4)
    mass = rng.random(len(pm)).astype(dt)
    field = rng.random(nm).astype(dt)
    np.testing.assert_array_equal(cic.paint(pm, mass, nm), ref.paint(pm, mass, nm))
    for d in (-1, 0, 1, 2):
        np.testing.assert_array_equal(cic.readout(pm, field, nm, box, d), ref.readout(pm, field, nm, box, d))


@needs_ref
@pytest.mark.parametrize("name", SMALL)
def test_oracle_equals_reference_on_pin_cases(name):
    a = pin_inputs.outputs(cic, name)
    b = pin_inputs.outputs(ref, name)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("name", SMALL)
def test_oracle_reproduces_reference_digests(name):
    outs = pin_inputs.outputs(cic, name)
    assert pin_inputs.CASES[name] and len(pin_inputs.positions(name)) == HASHES[name]["nparts"]
    for k, v in outs.items():
        assert pin_inputs.digest(v) == HASHES[name][k], k
