"""GPU CIC ops against the reference's own code, through the C ABI.

The seeded cases of oracle/pin_inputs.py regenerate bit for bit on any
host, and tests/golden/ref_hashes.json holds the sha256 digests of the
reference's outputs on them (lib/parops_fast.h compiled from source at world
size one; tests/golden/make_ref_hashes.py).  Readouts must hash to the
reference's digests (bit-exact).  Paints are compared with the oracle's
serial paint within 1e-5 (float32) or 1e-12 (float64) of the mesh scale,
after checking that the oracle's paint hashes to the reference's digest on
this host: the atomic summation order of the GPU differs from the
reference's particle order, so bit equality is not expected there.
"""
import ctypes as ct
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import cic, pin_inputs  # noqa: E402

HASHES = json.loads((Path(__file__).resolve().parent / "golden" / "ref_hashes.json").read_text())["cases"]


@pytest.fixture(scope="module")
def jl():
    from jerald_gb300 import _lib, build
    build.build()
    cic.set_threads(1)
    return _lib


def _st():
    return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return ct.c_void_p(t.data_ptr())


def _tdt(dt):
    return torch.float32 if dt == np.float32 else torch.float64


@pytest.mark.parametrize("name", list(pin_inputs.CASES))
def test_readouts_hash_to_reference(jl, name):
    pos, _, _, field, field3, nm, box, dt = pin_inputs.operands(name)
    sfx = "f32" if dt == np.float32 else "f64"
    b = np.ascontiguousarray(np.asarray(box, dtype=dt))
    bp = b.ctypes.data_as(ct.c_void_p)
    dpos = torch.from_numpy(pos).cuda()
    dfield = torch.from_numpy(field).cuda()
    dfield3 = torch.from_numpy(field3).cuda()
    out = torch.empty(len(pos), dtype=_tdt(dt), device="cuda")
    for v in (-1, 0, 1, 2):
        jl.call(f"jld_preadout_{sfx}", _st(), _p(dpos), len(pos), _p(dfield), *nm, bp, v, _p(out))
        assert pin_inputs.digest(out.cpu().numpy()) == HASHES[name][f"readout{v}"], f"vjpdim {v}"
    out3 = torch.empty((len(pos), 3), dtype=_tdt(dt), device="cuda")
    jl.call(f"jld_preadout3d_{sfx}", _st(), _p(dpos), len(pos), _p(dfield3), *nm, bp, 0, _p(out3))
    assert pin_inputs.digest(out3.cpu().numpy()) == HASHES[name]["readout3d"]
    jl.call(f"jld_preadout3d_{sfx}", _st(), _p(dpos), len(pos), _p(dfield), *nm, bp, 1, _p(out3))
    assert pin_inputs.digest(out3.cpu().numpy()) == HASHES[name]["readout3d_vjp"]
    torch.cuda.synchronize()


@pytest.mark.parametrize("name", list(pin_inputs.CASES))
def test_paints_match_reference(jl, name):
    pos, mass, mass3, _, _, nm, _, dt = pin_inputs.operands(name)
    sfx = "f32" if dt == np.float32 else "f64"
    o_paint = cic.paint(pos, mass, nm)
    o_paint3 = cic.paint3d(pos, mass3, nm)
    # the oracle's serial paint is the reference's paint, bit for bit, here too
    assert pin_inputs.digest(o_paint) == HASHES[name]["paint"]
    assert pin_inputs.digest(o_paint3) == HASHES[name]["paint3d"]
    rel = 1e-5 if dt == np.float32 else 1e-12
    dpos = torch.from_numpy(pos).cuda()
    out = torch.empty(nm, dtype=_tdt(dt), device="cuda")
    jl.call(f"jld_ppaint_{sfx}", _st(), _p(dpos), len(pos), _p(torch.from_numpy(mass).cuda()), *nm, _p(out))
    got = out.cpu().numpy()
    assert np.abs(got - o_paint).max() <= rel * max(1.0, float(np.abs(o_paint).max()))
    out3 = torch.empty((3,) + tuple(nm), dtype=_tdt(dt), device="cuda")
    jl.call(f"jld_ppaint3d_{sfx}", _st(), _p(dpos), len(pos), _p(torch.from_numpy(mass3).cuda()), *nm, _p(out3))
    got3 = out3.cpu().numpy()
    assert np.abs(got3 - o_paint3).max() <= rel * max(1.0, float(np.abs(o_paint3).max()))
    # keys: int(p) % N per axis (the reference's decomposition key)
    keys = torch.empty(len(pos), dtype=torch.int32, device="cuda")
    jl.call(f"jld_cell_keys_{sfx}", _st(), _p(dpos), len(pos), *nm, None, _p(keys))
    np.testing.assert_array_equal(keys.cpu().numpy(), cic.cell_keys(pos, nm))
    torch.cuda.synchronize()
