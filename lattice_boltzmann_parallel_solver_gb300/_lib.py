"""ctypes binding of ``liblbm_gb300.so`` (declarations in include/lbm_gb300.h).

There is no CPU fallback: when the library is missing or no CUDA device is
present, every compute entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblbm_gb300.so")

LBM_OK = 0
LBM_ERR_ARG = -1
LBM_ERR_OMEGA = -2
LBM_ERR_CUDA = -3
LBM_ERR_UNSUPPORTED = -4

SRC_PULL, SRC_BOUNCE, SRC_CONST, SRC_OUTLET = 0, 1, 2, 3
KSET_SHIFT, CSET_SHIFT = 18, 22
MAX_SETS = 16

STORE_F64, STORE_F32, STORE_F16S, STORE_BF16S, STORE_FX64, STORE_F16R, STORE_BF16R = 0, 1, 2, 3, 4, 5, 6
FLAG_EXACT = 1
FLAG_GENERIC = 2
FLAG_NPT_SHIFT = 4
FLAG_STOCHASTIC = 256
FLAG_BC_INLINE = 1024
FLAG_BC_SPLIT = 2048

vp = C.c_void_p
i32 = C.c_int32
i64 = C.c_int64
f64 = C.c_double


class Geometry(C.Structure):
    _fields_ = [
        ("nx", i32), ("ny", i32),
        ("bcmask", vp), ("desc", vp),
        ("n_kset", i32), ("n_cset", i32),
        ("kconst", (f64 * 9) * MAX_SETS),
        ("cconst", (f64 * 9) * MAX_SETS),
        ("pressure", i32),
        ("pressure_in_dirs", C.c_uint32), ("pressure_out_dirs", C.c_uint32),
        ("rho_in", f64), ("rho_out", f64),
        ("outlet", i32),
        ("bcnodes", vp), ("n_bcnodes", i32),
        ("edge_inlet_desc", C.c_uint32), ("edge_outlet_desc", C.c_uint32), ("n_bcnodes_edge", i32),
        ("dev_ref_ux", f64), ("dev_ref_uy", f64),
    ]


GP = C.POINTER(Geometry)


class BatchLattice(C.Structure):
    """lbm_batch_lattice in include/lbm_gb300.h"""
    _fields_ = [("g", vp), ("pop_a", vp), ("pop_b", vp), ("aux_a", vp), ("aux_b", vp), ("pitch", i64),
                ("omega", f64), ("s0", i32), ("s_end", i32), ("probe_x", i32), ("probe_y", i32),
                ("probe_cap", i32), ("probe_buf", vp), ("probe_count", vp), ("seed", C.c_uint32),
                ("flags", i32), ("rows", i32)]


class RunOptions(C.Structure):
    """lbm_run_options in include/lbm_gb300.h"""
    _fields_ = [("step_counter", vp), ("probe_x", i32), ("probe_y", i32), ("probe_cap", i32),
                ("probe_buf", vp), ("probe_count", vp)]


# name: (restype, argtypes)
SIGNATURES = {
    "lbm_version": (C.c_int, []),
    "lbm_last_error": (C.c_char_p, []),
    "lbm_launch_count": (i64, [C.c_int]),
    "lbm_density_f64": (C.c_int, [vp, vp, i64, vp]),
    "lbm_velocity_f64": (C.c_int, [vp, vp, vp, i64, vp]),
    "lbm_equilibrium_f64": (C.c_int, [vp, vp, vp, i64, vp]),
    "lbm_streaming_f64": (C.c_int, [vp, vp, i32, i32, vp]),
    "lbm_collide_f64": (C.c_int, [vp, vp, vp, f64, vp, i64, i32, vp]),
    "lbm_apply_boundary_f64": (C.c_int, [GP, vp, vp, vp, vp]),
    "lbm_pressure_prestream_f64": (C.c_int, [GP, vp, vp, vp, vp]),
    "lbm_halo_fill_f64": (C.c_int, [vp, i32, i32, vp]),
    "lbm_step_scratch_bytes": (C.c_size_t, [i32, i32]),
    "lbm_step_f64": (C.c_int, [GP, vp, vp, vp, f64, vp, vp, vp, vp, i32, vp]),
    "lbm_step_host_scratch_bytes": (C.c_size_t, [i32, i32]),
    "lbm_step_f64_host": (C.c_int, [GP, vp, vp, vp, f64, vp, vp, vp, vp, C.c_size_t, i32, i32, vp]),
    "lbm_step_f64_noalloc": (C.c_int, [GP, vp, vp, vp, f64, vp, vp, vp, i32, vp]),
    "lbm_lattice_pop_bytes": (C.c_size_t, [i32, i32, i64, i32]),
    "lbm_lattice_init": (C.c_int, [GP, i32, vp, vp, vp, f64, vp, i64, vp, i32, vp]),
    "lbm_lattice_run": (C.c_int, [GP, i32, vp, vp, i64, vp, vp, f64, i32, vp, vp, i32, C.c_uint32, vp]),
    "lbm_lattice_run_opts": (C.c_int, [GP, i32, vp, vp, i64, vp, vp, f64, i32, vp, vp, i32, C.c_uint32,
                                       C.POINTER(RunOptions), vp]),
    "lbm_lattice_read": (C.c_int, [GP, i32, vp, i64, vp, vp, vp, vp, vp]),
    "lbm_reduce_scratch_bytes": (C.c_size_t, [i64]),
    "lbm_reduce_moments_f64": (C.c_int, [vp, i64, vp, C.c_size_t, vp, vp]),
    "lbm_batch_table_bytes": (C.c_size_t, [i32]),
    "lbm_batch_build": (C.c_int, [C.POINTER(BatchLattice), i32, i32, i32, vp, C.c_size_t, C.POINTER(i32),
                                  C.POINTER(i32), vp]),
    "lbm_batch_run": (C.c_int, [vp, i32, i32, i32, i32, i32, i32, vp, i32, i32, vp]),
}

_lib = None


def load():
    """Load the library (once) and declare every signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            "liblbm_gb300.so is not built (expected at %s); run "
            "`python -c \"import __graft_entry__ as g; g.build()\"` first" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, what: str = "") -> None:
    """Map a status code to the exception the reference raises for it."""
    if status == LBM_OK:
        return
    msg = load().lbm_last_error().decode(errors="replace")
    text = "%s: %s" % (what, msg) if what else msg
    if status in (LBM_ERR_ARG, LBM_ERR_OMEGA):
        raise AssertionError(text)
    if status == LBM_ERR_UNSUPPORTED:
        raise NotImplementedError(text)
    raise RuntimeError(text)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)


def launches(reset: bool = False) -> int:
    return int(load().lbm_launch_count(1 if reset else 0))
