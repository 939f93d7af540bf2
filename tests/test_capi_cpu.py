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
def test_geometry_struct_layout_matches_c(tmp_path):
    src = tmp_path / "layout.c"
    fields = [f[0] for f in _lib.Geometry._fields_]
    body = "".join('printf("%s %%zu\\n", offsetof(lbm_geometry, %s));' % (n, n) for n in fields)
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "lbm_gb300.h"\n'
                   'int main(void){printf("size %%zu\\n", sizeof(lbm_geometry));%s return 0;}\n' % body)
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = dict(line.split() for line in subprocess.check_output([str(exe)]).decode().splitlines())
    assert int(out["size"]) == ctypes.sizeof(_lib.Geometry)
    for n in fields:
        assert int(out[n]) == getattr(_lib.Geometry, n).offset, n
