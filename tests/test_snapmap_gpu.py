"""GPU snapshot ingestion (makemap, JERALD/snaputils.py:253-406) against the
oracle's restatement: every map kind, chunked streaming with a ragged last
chunk, positions outside the box, and the saved bigfile map.  Bar: 1e-5 of
the map scale (float32 atomics in another order; weights rounded once)."""
import types

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

from oracle import snapmap as osm  # noqa: E402


def _snapshot(seed=0, n=40000, box=25.0):
    from jerald_gb300.snapmap import ArraySnapshot
    rng = np.random.default_rng(seed)
    parts = {}
    for t in (0, 1, 4):
        # kpc/h, a few outside [0, box) to exercise the wrap
        coords = rng.uniform(-0.1, 1.1, (n, 3)) * box * 1000.0
        coords[:64] = rng.normal(0.5 * box * 1000.0, 30.0, (64, 3))   # a clump
        parts[t] = {"Coordinates": coords.astype(np.float32),
                    "Masses": rng.uniform(1e-4, 2e-3, n).astype(np.float32),
                    "ElectronAbundance": rng.uniform(0.0, 1.2, n).astype(np.float32),
                    "InternalEnergy": rng.uniform(10.0, 1e4, n).astype(np.float32),
                    "NeutralHydrogenAbundance": rng.uniform(0.0, 1.0, n).astype(np.float32),
                    "Velocities": rng.normal(0.0, 300.0, (n, 3)).astype(np.float32)}
    return ArraySnapshot(redshift=2.3, parts=parts), box


@pytest.mark.parametrize("kind", ["dm", "Mstar", "ne", "nT", "nHI", "neVz", "MstarVz", "XHI"])
def test_makemap_matches_oracle(kind):
    from jerald_gb300 import snapmap
    snap, box = _snapshot()
    nm = (32, 32, 32)
    pm = types.SimpleNamespace(Nmesh=np.asarray(nm), BoxSize=np.asarray([box] * 3), device="cuda", fftss=(0, 32))
    out = snapmap.makemap(snap, kind, pm, save=False, chunk=7001, h=0.7, XH=0.76)
    pt = snapmap.mapPartNum(kind)
    fields = dict(snap.parts[pt])
    fields["Velocities"] = fields["Velocities"][:, 2]
    ref = osm.makemap(fields, kind, nm, [box] * 3, 2.3, h=0.7, XH=0.76)
    scale = np.abs(ref).max()
    assert scale > 0
    assert np.abs(out - ref).max() <= 1e-5 * scale, (kind, np.abs(out - ref).max() / scale)
    if kind == "dm":
        assert abs(out.sum() / np.prod(nm) - 1.0) < 1e-5


def test_makemap_saves_a_loadable_field(tmp_path):
    from jerald_gb300 import fieldio, snapmap
    snap, box = _snapshot(seed=3, n=5000)
    nm = (16, 16, 16)
    pm = types.SimpleNamespace(Nmesh=np.asarray(nm), BoxSize=np.asarray([box] * 3), device="cuda", fftss=(0, 16))
    out = snapmap.makemap(snap, "nHI", pm, save=True, outpath=str(tmp_path), chunk=1 << 20)
    back, Nmesh, BoxSize = fieldio.loadfield(tmp_path / "nHImap_Nmesh16", verify=True)
    np.testing.assert_array_equal(back, out)
    assert list(Nmesh) == list(nm) and list(BoxSize) == [box] * 3
    one = snapmap.makemap(snap, "nHI", pm, save=False, chunk=1 << 20, return_tensor=True)
    assert one.is_cuda and one.dtype == torch.float32
    # a second run adds in another atomic order
    assert np.abs(one.cpu().numpy() - out).max() <= 1e-5 * np.abs(out).max()


@pytest.mark.parametrize("kind", ["Mstar", "ne", "nT", "nHI", "neVz", "MstarVz", "XHI"])
def test_particle_weights_bit_exact(kind):
    """The per-particle weights of jld_snap_prep_f32 equal NumPy's
    (snaputils.py:360-376 under NumPy 2 promotion, cast to float32) bit for
    bit, and the wrapped positions equal pos / 1000 % BoxSize."""
    import ctypes as ct

    from jerald_gb300 import _lib
    from jerald_gb300.snapmap import KINDS
    snap, box = _snapshot(seed=5, n=20000)
    fields = dict(snap.parts[{"Mstar": 4, "MstarVz": 4}.get(kind, 0)])
    vz = np.ascontiguousarray(fields["Velocities"][:, 2])
    a, c1, c2 = osm.coefficients(2.3, [box] * 3, (32, 32, 32), h=0.7, XH=0.76)
    want = np.asarray(osm.weights(kind, dict(fields, Velocities=vz), a, c1, c2, 0.76)).astype(np.float32)
    want_pos = osm.positions(fields["Coordinates"], [box] * 3)
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in fields.items()}
    dvz = torch.from_numpy(vz).cuda()
    n = len(want)
    pos_out = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    w = torch.empty(n, dtype=torch.float32, device="cuda")
    P = lambda t: ct.c_void_p(t.data_ptr())  # noqa: E731
    box64 = np.asarray([box] * 3, dtype=np.float64)
    _lib.call("jld_snap_prep_f32", ct.c_void_p(torch.cuda.current_stream().cuda_stream), P(dev["Coordinates"]), n,
              ct.c_float(1000.0), box64.ctypes.data_as(ct.c_void_p), KINDS[kind], P(dev["Masses"]),
              P(dev["ElectronAbundance"]), P(dev["InternalEnergy"]), P(dev["NeutralHydrogenAbundance"]), P(dvz), 1,
              float(c1), float(c2), 0.76, float(a ** 0.5), P(pos_out), P(w))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(w.cpu().numpy().view(np.uint32), want.view(np.uint32))
    np.testing.assert_array_equal(pos_out.cpu().numpy(), want_pos)
