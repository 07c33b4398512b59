"""The C-ABI library loads and exports every entry point include/jld.h declares,
and the Python binding covers all of them (no compute calls: CPU only)."""
import ctypes as ct
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_names():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(jld_\w+)\s*\(", txt))
    return sorted(names)


@pytest.fixture(scope="module")
def libjld():
    from jerald_gb300 import build
    path = build.build()
    return ct.CDLL(str(path))


def test_header_declares_entry_points():
    names = declared_names()
    assert "jld_ppaint_f32" in names and "jld_pfft_f32" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(libjld):
    missing = [n for n in declared_names() if not hasattr(libjld, n)]
    assert not missing, f"symbols declared in include/*.h but not exported: {missing}"


def test_python_binding_covers_header():
    from jerald_gb300 import _lib
    assert set(declared_names()) == set(_lib.exported_names())


def test_host_only_entry_points(libjld):
    libjld.jld_version.restype = ct.c_char_p
    assert b"sm_103a" in libjld.jld_version()
    libjld.jld_status_string.restype = ct.c_char_p
    assert libjld.jld_status_string(3) == b"workspace too small"
    libjld.jld_fft_workspace_f32.restype = ct.c_size_t
    libjld.jld_fft_workspace_f32.argtypes = [ct.c_int32] * 3
    assert libjld.jld_fft_workspace_f32(8, 8, 8) == 8 * 8 * 5 * 8
    # layout bookkeeping validates like the reference (lyidx 0..4, world size 1)
    assert libjld.jld_init_layout(1, 0) == 0
    assert libjld.jld_init_layout(1, 5) == 1
    assert libjld.jld_init_layout(2, 0) == 2
    assert libjld.jld_clean(7) == 1


def test_exports_are_c_symbols_only(libjld):
    # hidden visibility: no C++ internals leak into the dynamic symbol table
    import subprocess
    out = subprocess.run(["nm", "-D", "--defined-only", str(Path(libjld._name))],
                         capture_output=True, text=True).stdout
    syms = [l.split()[-1] for l in out.splitlines() if " T " in l]
    ours = [s for s in syms if s.startswith("jld_")]
    assert set(declared_names()) <= set(ours)


def test_argument_errors_before_any_launch(libjld):
    """Argument checks of the newer entry points return a status and a
    message before they touch the GPU (no device needed)."""
    libjld.jld_last_error.restype = ct.c_char_p
    box = (ct.c_double * 3)(25.0, 25.0, 25.0)
    f = ct.c_void_p(16)  # never dereferenced: every call below fails first
    sp = libjld.jld_snap_prep_f32
    sp.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_int64, ct.c_float, ct.c_void_p, ct.c_int32] + \
        [ct.c_void_p] * 5 + [ct.c_int64, ct.c_double, ct.c_double, ct.c_double, ct.c_double, ct.c_void_p,
                             ct.c_void_p]
    args = lambda kind, n=10, masses=f, unit=1000.0, b=box: (None, f, n, unit, b, kind, masses, f, f, f, f, 3,  # noqa
                                                              1.0, 1.0, 0.76, 1.0, f, f)
    assert sp(*args(8)) == 1 and b"kind" in libjld.jld_last_error()
    assert sp(*args(2, masses=None)) == 1 and b"NULL" in libjld.jld_last_error()
    assert sp(*args(2, n=-1)) == 1
    assert sp(*args(2, unit=0.0)) == 1 and b"unit" in libjld.jld_last_error()
    assert sp(*args(2, b=None)) == 1 and b"box" in libjld.jld_last_error()
    assert sp(*args(2, n=0)) == 0  # nothing to do
    ext = libjld.jld_ldl_step_ext_f32
    ext.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_int64, ct.c_int32, ct.c_int32, ct.c_int32, ct.c_void_p,
                    ct.c_int32, ct.c_int32, ct.c_int32, ct.c_int32, ct.c_int32, ct.c_void_p, ct.c_void_p,
                    ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_size_t, ct.c_void_p]
    fbox = (ct.c_float * 3)(1.0, 1.0, 1.0)
    assert ext(None, f, 8, 4, 4, 4, fbox, 2, 0, 1, 0, 0, f, f, None, None, f, 1 << 30, f) == 1
    assert b"ext is NULL" in libjld.jld_last_error()
    acc = libjld.jld_ppaint_box_acc_f32
    acc.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_int64, ct.c_void_p, ct.c_float, ct.c_int32, ct.c_int32,
                    ct.c_int32, ct.c_void_p, ct.c_void_p]
    assert acc(None, f, 8, None, ct.c_float(1.0), 4, 4, 4, None, f) == 1 and b"box" in libjld.jld_last_error()
    ws = libjld.jld_wait_selftest
    ws.argtypes = [ct.c_void_p, ct.c_int32, ct.c_void_p]
    assert ws(None, 0, None) == 1 and b"polls" in libjld.jld_last_error()
    assert ws(None, (1 << 22) + 1, None) == 1
    cs = libjld.jld_cell_sort_f32
    cs.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_int64, ct.c_int32, ct.c_int32, ct.c_int32, ct.c_void_p,
                   ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_size_t]
    assert cs(None, f, 10, 4, 4, 4, fbox, f, f, None, 0) == 3 and b"workspace" in libjld.jld_last_error()
    assert cs(None, f, 10, 4, 4, 4, None, f, f, f, 1 << 20) == 1 and b"box" in libjld.jld_last_error()
    assert cs(None, f, 10, 4, 4, 4, fbox, f, None, f, 1 << 20) == 1 and b"order" in libjld.jld_last_error()
    libjld.jld_cell_sort_workspace.restype = ct.c_size_t
    libjld.jld_cell_sort_workspace.argtypes = [ct.c_int64]
    assert libjld.jld_cell_sort_workspace(1) == 0 and libjld.jld_cell_sort_workspace(5000) > 40000
    bs = libjld.jld_ppaint_box_sorted_f32
    bs.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_int64, ct.c_void_p, ct.c_float, ct.c_int32, ct.c_int32,
                   ct.c_int32, ct.c_void_p, ct.c_void_p, ct.c_void_p, ct.c_size_t]
    assert bs(None, f, 10, None, ct.c_float(1.0), 4, 4, 4, fbox, f, f, 16) == 3
    hi = libjld.jld_ldl_step_hi_f32
    hi.argtypes = [ct.c_void_p, ct.c_void_p, ct.c_int64, ct.c_int32, ct.c_int32, ct.c_int32, ct.c_void_p,
                   ct.c_int32, ct.c_int32, ct.c_int32, ct.c_int32, ct.c_void_p, ct.c_void_p, ct.c_void_p,
                   ct.c_void_p, ct.c_void_p, ct.c_size_t, ct.c_void_p]
    assert hi(None, f, 8, 4, 4, 4, fbox, 2, 1, 0, 0, f, f, None, None, f, 1 << 30, f) == 1
    assert b"star map" in libjld.jld_last_error()
    for fn in (libjld.jld_ldl_workspace_hi_f32, libjld.jld_ldl_workspace_opt_f32):
        fn.restype = ct.c_size_t
        fn.argtypes = [ct.c_int32] * 3 + [ct.c_int64, ct.c_int32, ct.c_int32]
    # the HI workspace adds nstep + 1 half spectra and two real meshes
    extra = libjld.jld_ldl_workspace_hi_f32(32, 32, 32, 1000, 2, 0) - \
        libjld.jld_ldl_workspace_opt_f32(32, 32, 32, 1000, 2, 0)
    assert extra == 3 * 8 * 32 * 32 * 17 + 2 * 4 * 32 ** 3
    assert hi(None, f, 8, 4, 4, 4, fbox, 2, 1, 0, 0, f, f, None, f, f, 16, f) == 3


def _c_examples():
    txt = (ROOT / "INTEGRATION.md").read_text()
    return re.findall(r"```c\n(.*?)```", txt, flags=re.S)


def test_integration_c_examples_compile_and_link(libjld, tmp_path):
    """The C examples of INTEGRATION.md build against include/jld.h with
    -Wall -Werror and link against libjld and cudart with no undefined
    symbol (compiled only, never run)."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    nvcc = shutil.which("nvcc")
    cuda = Path(nvcc).resolve().parents[1] if nvcc else Path("/usr/local/cuda")
    if not gcc or not (cuda / "include" / "cuda_runtime.h").exists():
        pytest.skip("gcc or the CUDA runtime headers are absent")
    blocks = _c_examples()
    assert len(blocks) >= 2
    lib = Path(libjld._name).parent
    for i, src in enumerate(blocks):
        c = tmp_path / f"example{i}.c"
        c.write_text(src)
        cmd = [gcc, "-std=c11", "-Wall", "-Werror", "-shared", "-fPIC", "-I", str(ROOT / "include"),
               "-I", str(cuda / "include"), str(c), "-o", str(tmp_path / f"example{i}.so"),
               "-L", str(lib), "-ljld", "-L", str(cuda / "lib64"), "-lcudart", "-Wl,--no-undefined"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, f"example {i}:\n{r.stderr}"
