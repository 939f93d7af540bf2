"""The .npy snapshot writer against the layout save_mpiio writes
(parallelization_utils.py:203-253, one rank): format 1.0, header padded to a
16-byte boundary with spaces and a newline, C-order data; numpy.load reads it
back unchanged."""
import numpy as np
import pytest


def reference_layout(arr):
    """save_mpiio's bytes for a single-rank 2-D array, written out from its steps."""
    magic_str = b"\x93NUMPY\x01\x00"
    d = str({'descr': np.lib.format.dtype_to_descr(arr.dtype), 'fortran_order': False,
             'shape': (arr.shape[0], arr.shape[1])})
    while (len(d) + len(magic_str) + 2) % 16 != 15:
        d += ' '
    d += '\n'
    return magic_str + np.int16(len(d)).tobytes() + d.encode('latin-1') + np.ascontiguousarray(arr).tobytes()


@pytest.mark.parametrize("shape,dtype", [((420, 180), np.float64), ((7, 3), np.float64), ((64, 64), np.float32)])
def test_npy_bytes_match_save_mpiio_layout(tmp_path, shape, dtype):
    from lattice_boltzmann_parallel_solver_gb300.analysis import npy_bytes, save_field_npy
    arr = np.random.default_rng(1).normal(size=shape).astype(dtype)
    assert npy_bytes(arr) == reference_layout(arr)
    p = tmp_path / "field.npy"
    save_field_npy(str(p), arr)
    assert p.read_bytes() == reference_layout(arr)
    back = np.load(str(p))
    assert back.dtype == arr.dtype and np.array_equal(back, arr)
    # the data starts on a 16-byte boundary
    assert (len(reference_layout(arr)) - arr.nbytes) % 16 == 0
