"""CPU checks of the C ABI: the library builds and loads, exports every
entry point include/lbm_gb300.h declares, and the ctypes mirror of
lbm_geometry has the C layout.  No kernel is launched."""
import ctypes
import os
import re
import shutil
import subprocess

import pytest

from lattice_boltzmann_parallel_solver_gb300 import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "lbm_gb300.h")


def declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*[a-z_0-9 ]+[ *](lbm_[a-z_0-9]+)\(", text, re.M)))


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = declared()
    assert "lbm_step_f64" in names and "lbm_lattice_run" in names
    assert len(names) >= 15


def test_every_declared_symbol_is_exported_and_bound(lib):
    for name in declared():
        assert hasattr(lib, name), name
        assert name in _lib.SIGNATURES, "no ctypes signature for " + name


def test_version_and_error_string(lib):
    assert lib.lbm_version() >= 10000
    assert isinstance(lib.lbm_last_error(), bytes)


def test_argument_errors_without_gpu(lib):
    # argument checks run before any CUDA call and map to AssertionError
    g = _lib.Geometry()
    g.nx, g.ny = 0, 4
    with pytest.raises(AssertionError):
        _lib.check(lib.lbm_lattice_read(ctypes.byref(g), 0, None, 32, None, None, None, None, None))
    g.nx = 8
    with pytest.raises(AssertionError, match="omega"):
        _lib.check(lib.lbm_lattice_run(ctypes.byref(g), 0, 1, 2, 32, None, None, 2.5, 1, None, None, 0, 0, None))
    with pytest.raises(AssertionError, match="pitch"):
        _lib.check(lib.lbm_lattice_run(ctypes.byref(g), 0, 1, 2, 7, None, None, 1.0, 1, None, None, 0, 0, None))


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
@pytest.mark.parametrize("cname,pyname", [("lbm_geometry", "Geometry"), ("lbm_batch_lattice", "BatchLattice"),
                                          ("lbm_run_options", "RunOptions")])
def test_struct_layout_matches_c(tmp_path, cname, pyname):
    cls = getattr(_lib, pyname)
    src = tmp_path / ("%s.c" % cname)
    fields = [f[0] for f in cls._fields_]
    body = "".join('printf("%s %%zu\\n", offsetof(%s, %s));' % (n, cname, n) for n in fields)
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "lbm_gb300.h"\n'
                   'int main(void){printf("size %%zu\\n", sizeof(%s));%s return 0;}\n' % (cname, body))
    exe = tmp_path / cname
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = dict(line.split() for line in subprocess.check_output([str(exe)]).decode().splitlines())
    assert int(out["size"]) == ctypes.sizeof(cls)
    for n in fields:
        assert int(out[n]) == getattr(cls, n).offset, n


def test_integration_stub_geometry_matches_binding():
    """The ctypes stub a maintainer copies from INTEGRATION.md has the binding's
    fields, sizes and offsets (so the documented struct cannot drift)."""
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    m = re.search(r"```python\n(import ctypes as C\n.*?)```", text, re.S)
    assert m, "no ctypes stub in INTEGRATION.md"
    code = m.group(1).replace('lib = C.CDLL("liblbm_gb300.so")', "lib = None")
    code = code[:code.index("lib.lbm_step_f64.argtypes")]
    ns = {}
    exec(compile(code, "INTEGRATION.md", "exec"), ns)
    stub = ns["Geometry"]
    assert [f[0] for f in stub._fields_] == [f[0] for f in _lib.Geometry._fields_]
    assert ctypes.sizeof(stub) == ctypes.sizeof(_lib.Geometry)
    for name, _ in _lib.Geometry._fields_:
        assert getattr(stub, name).offset == getattr(_lib.Geometry, name).offset, name


def test_run_options_argument_errors_without_gpu(lib):
    g = _lib.Geometry()
    g.nx, g.ny = 8, 4
    o = _lib.RunOptions()
    o.probe_buf, o.probe_count, o.probe_cap = 4096, 8192, 10
    o.probe_x, o.probe_y = 8, 0
    with pytest.raises(AssertionError, match="probe"):
        _lib.check(lib.lbm_lattice_run_opts(ctypes.byref(g), 0, 1, 2, 32, None, None, 1.0, 1, None, None, 0, 0,
                                            ctypes.byref(o), None))
    o.probe_x, o.probe_count = 0, None
    with pytest.raises(AssertionError, match="probe_count"):
        _lib.check(lib.lbm_lattice_run_opts(ctypes.byref(g), 0, 1, 2, 32, None, None, 1.0, 1, None, None, 0, 0,
                                            ctypes.byref(o), None))


def test_batch_argument_errors_without_gpu(lib):
    # the batch table builder checks its arguments before any CUDA call
    assert lib.lbm_batch_table_bytes(8) > lib.lbm_batch_table_bytes(4) > lib.lbm_batch_table_bytes(1) > 0
    g = _lib.Geometry()
    g.nx, g.ny = 64, 16
    arr = (_lib.BatchLattice * 1)()
    arr[0].g = ctypes.addressof(g)
    arr[0].pop_a, arr[0].pop_b, arr[0].pitch, arr[0].omega = 1024, 2048, 64, 1.0
    size = int(lib.lbm_batch_table_bytes(1))
    table = ctypes.create_string_buffer(size + 16)
    ptr = (ctypes.addressof(table) + 15) // 16 * 16
    tiles, chunks = ctypes.c_int32(0), ctypes.c_int32(0)

    def build(n=1, npt=4, threads=64, nbytes=size, with_chunks=True):
        return lib.lbm_batch_build(arr, n, npt, threads, ptr, nbytes, ctypes.byref(tiles),
                                   ctypes.byref(chunks) if with_chunks else None, None)

    with pytest.raises(AssertionError, match="bad batch arguments"):
        _lib.check(build(n=0))
    with pytest.raises(AssertionError, match="bad batch arguments"):
        _lib.check(build(with_chunks=False))
    with pytest.raises(AssertionError, match="too small"):
        _lib.check(build(nbytes=size - 1))
    with pytest.raises(AssertionError, match="npt"):
        _lib.check(build(npt=3))
    arr[0].omega = 2.0
    with pytest.raises(AssertionError, match="omega"):
        _lib.check(build())
    arr[0].omega, arr[0].pitch = 1.0, 60
    with pytest.raises(AssertionError, match="pitch"):
        _lib.check(build())
    arr[0].pitch, g.nx = 64, 5  # narrower than npt + 2 nodes
    with pytest.raises(NotImplementedError):
        _lib.check(build())
    with pytest.raises(AssertionError, match="batch run"):
        _lib.check(lib.lbm_batch_run(ptr, 1, 10, -1, 2, 4, 64, None, 1, 0, None))


def test_storage_constants_match_header():
    text = open(HEADER).read()
    defs = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define LBM_STORE_(\w+) (\d+)", text)}
    assert defs == {"F64": _lib.STORE_F64, "F32": _lib.STORE_F32, "F16S": _lib.STORE_F16S,
                    "BF16S": _lib.STORE_BF16S, "FX64": _lib.STORE_FX64, "F16R": _lib.STORE_F16R,
                    "BF16R": _lib.STORE_BF16R}


def test_reference_velocity_range_checked_without_gpu(lib):
    g = _lib.Geometry()
    g.nx, g.ny = 8, 4
    for ux, uy in ((0.5, 0.0), (0.0, -0.7), (float("nan"), 0.0)):
        g.dev_ref_ux, g.dev_ref_uy = ux, uy
        with pytest.raises(AssertionError, match="reference velocity"):
            _lib.check(lib.lbm_lattice_run(ctypes.byref(g), _lib.STORE_F16R, 1, 2, 32, None, None, 1.0, 1, None,
                                           None, 0, 0, None))
