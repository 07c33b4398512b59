"""Bigfile-layout mesh files (maputils.savefield / loadfield restated without
the bigfile module) and the host logic of the snapshot ingestion: CPU only."""
import types

import numpy as np
import pytest

from jerald_gb300 import fieldio


def _pm(nm, box):
    return types.SimpleNamespace(Nmesh=np.asarray(nm, dtype=np.int64), BoxSize=np.asarray(box, dtype=np.float64),
                                 fftss=(0, nm[0]))


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("nfile", [1, 3])
def test_field_roundtrip(tmp_path, dt, nfile):
    nm, box = (6, 5, 4), (10.0, 12.5, 8.0)
    data = np.random.default_rng(0).standard_normal(nm).astype(dt)
    fieldio.savefield(data, tmp_path / "m", _pm(nm, box), nfile=nfile)
    out, Nmesh, BoxSize = fieldio.loadfield(tmp_path / "m", verify=True)
    assert out.dtype == dt and out.shape == nm
    np.testing.assert_array_equal(out, data)
    np.testing.assert_array_equal(Nmesh, nm)
    np.testing.assert_array_equal(BoxSize, box)
    loc, _, _ = fieldio.loadfield(tmp_path / "m", local=True, pm=_pm(nm, box))
    np.testing.assert_array_equal(loc, data)


def test_block_layout_and_attributes(tmp_path):
    data = np.arange(10, dtype=np.float32)
    fieldio.savefield(data.reshape(1, 2, 5), tmp_path / "f", _pm((1, 2, 5), (3.0, 4.0, 5.0)), nfile=2)
    d = tmp_path / "f" / "Field"
    assert sorted(p.name for p in d.iterdir()) == ["000000", "000001", "attr-v2", "header"]
    lines = (d / "header").read_text().splitlines()
    assert lines[:3] == ["DTYPE: <f4", "NMEMB: 1", "NFILE: 2"]
    ck, sv = fieldio.sysv_checksums(data[:5].tobytes())
    assert lines[3] == f"000000: 5 : {ck} : {sv}"
    attrs = fieldio.read_attrs(tmp_path / "f", "Field")
    assert set(attrs) == {"ndarray.shape", "BoxSize", "Nmesh"}
    assert attrs["Nmesh"].dtype == np.dtype("<i8") and list(attrs["Nmesh"]) == [1, 2, 5]
    assert attrs["BoxSize"].dtype == np.dtype("<f8") and list(attrs["BoxSize"]) == [3.0, 4.0, 5.0]
    first = (d / "attr-v2").read_text().splitlines()[0]
    assert first.startswith("ndarray.shape <i8 3 0100000000000000") and "#HUMANE [ 1 2 5 ]" in first


def test_sysv_checksum_known_values():
    assert fieldio.sysv_checksums(b"abc") == (294, 294)
    s, sv = fieldio.sysv_checksums(bytes([255]) * 1000)
    assert s == 255000 and sv == ((255000 & 0xFFFF) + (255000 >> 16))


def test_corruption_is_detected(tmp_path):
    data = np.ones((2, 2, 2), dtype=np.float32)
    fieldio.savefield(data, tmp_path / "c", _pm((2, 2, 2), (1.0, 1.0, 1.0)))
    p = tmp_path / "c" / "Field" / "000000"
    raw = bytearray(p.read_bytes())
    raw[0] ^= 1
    p.write_bytes(bytes(raw))
    with pytest.raises(ValueError, match="checksum"):
        fieldio.loadfield(tmp_path / "c", verify=True)
    (tmp_path / "c" / "Field" / "header").write_text("DTYPE: <f4\nNMEMB: 1\nNFILE: 2\n000000: 8 : 0 : 0\n")
    with pytest.raises(ValueError, match="incomplete"):
        fieldio.loadfield(tmp_path / "c")


def test_snapshot_host_logic(tmp_path):
    from jerald_gb300 import snapmap
    assert [snapmap.mapPartNum(k) for k in ("dm", "Mstar", "MstarVz", "ne", "nT", "nHI", "neVz", "XHI")] == \
        [1, 4, 4, 0, 0, 0, 0, 0]
    with pytest.raises(ValueError):
        snapmap.mapPartNum("gas")
    f, mdi = snapmap.map_fields("neVz")
    assert f == ["Coordinates", "Masses", "ElectronAbundance", "Velocities"] and mdi == [None, None, None, 2]
    assert snapmap.map_fields("nT")[0] == ["Coordinates", "ElectronAbundance", "InternalEnergy", "Masses"]
    a, c1, c2 = snapmap.map_coefficients(2.0, [25.0] * 3, [64] * 3, h=0.7, XH=0.76)
    assert a == 1 / 3 and c2 == 323.06014
    assert c1 == 4.0475e-07 * 0.7 ** 2 / (1 / 3) ** 3 * 0.76 / 25.0 ** 3 * 64 ** 3
    # snapshot path resolution (snaputils.fname)
    (tmp_path / "snap_004.0.hdf5").write_bytes(b"")
    (tmp_path / "snap_004.1.hdf5").write_bytes(b"")
    base = str(tmp_path / "snap_004")
    assert snapmap.fname(base) == base + ".0.hdf5"
    assert snapmap.fname(base + ".1") == base + ".0.hdf5"
    assert snapmap.fname(base + ".1.hdf5") == base + ".1.hdf5"
    with pytest.raises(FileNotFoundError):
        snapmap.fname(str(tmp_path / "nothing"))
    snap = snapmap.ArraySnapshot(0.5, {0: {"Coordinates": np.zeros((10, 3), np.float32),
                                           "Velocities": np.arange(30, dtype=np.float32).reshape(10, 3)}})
    assert list(snap.nall) == [10, 0, 0, 0, 0, 0]
    ch = list(snap.chunks(0, ["Coordinates", "Velocities"], [None, 2], 4))
    assert [len(c["Coordinates"]) for c in ch] == [4, 4, 2]
    np.testing.assert_array_equal(np.concatenate([c["Velocities"] for c in ch]), np.arange(2, 30, 3))


def test_snapmap_oracle_known_answers():
    """The oracle's makemap on single particles: a particle on a grid point
    puts its whole weight in that cell; coordinates in kpc/h wrap into the
    box; each kind's weight follows snaputils.py:360-376."""
    from oracle import snapmap as osm
    nm, box, z = (8, 8, 8), 4.0, 1.0
    a, c1, c2 = osm.coefficients(z, [box] * 3, nm, h=0.7, XH=0.76)
    assert a == 0.5 and c1 == 4.0475e-07 * 0.7 ** 2 / 0.5 ** 3 * 0.76 / box ** 3 * 8 ** 3
    cell = box / 8
    # grid point (3, 1, 6) given once inside and once a box length away
    for shift in (0.0, box, -box):
        coords = np.array([[(3 * cell + shift) * 1000.0, 1 * cell * 1000.0, 6 * cell * 1000.0]], np.float32)
        f = {"Coordinates": coords, "Masses": np.array([2e-3], np.float32),
             "ElectronAbundance": np.array([1.1], np.float32), "InternalEnergy": np.array([500.0], np.float32),
             "NeutralHydrogenAbundance": np.array([0.25], np.float32), "Velocities": np.array([-120.0], np.float32)}
        expect = {"ne": c1 * np.float32(2e-3) * np.float32(1.1),
                  "nT": c1 * np.float32(2e-3) * np.float32(1.1) * c2 * np.float32(500.0)
                  / (1 + 3 * 0.76 + 4 * 0.76 * np.float32(1.1)),
                  "nHI": c1 * np.float32(2e-3) * np.float32(0.25),
                  "MstarVz": np.float32(2e-3) * np.float32(-120.0) * a ** 0.5,
                  "XHI": np.float32(0.25), "Mstar": np.float32(2e-3), "dm": 8.0 ** 3}
        for kind, w in expect.items():
            m = osm.makemap(f, kind, nm, [box] * 3, z, h=0.7, XH=0.76)
            assert np.count_nonzero(m) == 1, (kind, shift)
            assert m[3, 1, 6] == pytest.approx(float(np.float32(w)), rel=1e-6), kind


def test_hdf5_snapshot_reader_logic_with_a_stub(tmp_path, monkeypatch):
    """HDF5Snapshot against an in-memory stand-in for h5py (absent here):
    header attributes, files walked in order, files without the particle type
    skipped, chunks split at max_particles, Velocities reduced to vz."""
    import sys
    import types as _types
    from jerald_gb300 import snapmap
    base = tmp_path / "snap_007"
    nfile = 3
    rng = np.random.default_rng(4)
    files = {}
    for i in range(nfile):
        n = [5, 0, 7][i]
        parts = {} if n == 0 else {"PartType0": {"Coordinates": rng.random((n, 3)) * 1e4,
                                                  "Masses": rng.random(n),
                                                  "Velocities": rng.standard_normal((n, 3))}}
        npart = [n, 0, 0, 0, 0, 0]
        files[f"{base}.{i}.hdf5"] = {"Header": {"Time": 0.5, "Redshift": 1.0, "BoxSize": 10000.0,
                                                "NumFilesPerSnapshot": nfile, "Omega0": 0.3, "OmegaLambda": 0.7,
                                                "HubbleParam": 0.7, "MassTable": [0.0] * 6,
                                                "NumPart_ThisFile": npart, "NumPart_Total": [12, 0, 0, 0, 0, 0],
                                                "Flag_Cooling": 1}, **parts}
        (tmp_path / f"snap_007.{i}.hdf5").write_bytes(b"")

    class _Group(dict):
        pass

    class _File:
        def __init__(self, path, mode="r"):
            d = files[str(path)]
            self._d = {k: v for k, v in d.items() if k != "Header"}
            self._h = _types.SimpleNamespace(attrs=d["Header"])

        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False

        def close(self):
            pass

        def __contains__(self, k):
            return k == "Header" or k in self._d

        def __getitem__(self, k):
            return self._h if k == "Header" else _Group(self._d[k])

    monkeypatch.setitem(sys.modules, "h5py", _types.SimpleNamespace(File=_File))
    snap = snapmap.HDF5Snapshot(str(base))
    assert snap.redshift == 1.0 and list(snap.nall) == [12, 0, 0, 0, 0, 0]
    fields, mdi = snapmap.map_fields("neVz")[0][:2] + ["Velocities"], [None, None, 2]
    got = list(snap.chunks(0, fields, mdi, 4))
    assert [len(c["Coordinates"]) for c in got] == [4, 1, 4, 3]
    want_v = np.concatenate([files[f"{base}.{i}.hdf5"]["PartType0"]["Velocities"][:, 2] for i in (0, 2)])
    np.testing.assert_allclose(np.concatenate([c["Velocities"] for c in got]), want_v.astype(np.float32))
    assert all(c["Masses"].dtype == np.float32 for c in got)
