"""The C ABI library builds, loads and exports every declared symbol
(no compute calls: this runs without a GPU)."""
import ctypes as C
import subprocess

import pytest

from pplacer_gb300 import lib as L


@pytest.fixture(scope="module")
def so():
    from pplacer_gb300 import build
    return build.build()


def test_every_header_symbol_is_exported(so):
    syms = L.header_symbols()
    assert len(syms) >= 30
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    lib = L.load()
    for s in syms:
        assert getattr(lib, s) is not None


def test_dropin_surface_covers_linear_c():
    """One drop-in entry point per external of pplacer_src/linear.ml:13-89
    (the two print functions stay in the OCaml stub: host-side debug output)."""
    externals = ["gemmish", "dediagonalize", "mat_log_like3", "mat_pairwise_prod", "mat_statd_pairwise_prod",
                 "mat_masked_logdot", "mat_bounded_logdot", "ten_log_like3", "ten_pairwise_prod",
                 "ten_statd_pairwise_prod", "ten_masked_logdot", "ten_bounded_logdot", "vec_pairwise_prod",
                 "int_vec_tot", "int_vec_pairwise_prod", "float_mat_int_vec_mul"]
    syms = set(L.header_symbols())
    assert all("pgb_" + e in syms for e in externals)


def test_argument_errors_before_any_device_work(so):
    lib = L.load()
    h = C.c_void_p()
    assert lib.pgb_engine_create(None, None, C.byref(h)) == 1  # PGB_ERR_ARG
    assert b"null" in lib.pgb_last_error()
    md = L.ModelDesc(5, 4, 0, 100, None, None, None, None, None, None)  # 5 states: unsupported
    td = L.TreeDesc(3, None, None)
    assert lib.pgb_engine_create(C.byref(md), C.byref(td), C.byref(h)) == 1
    assert b"unsupported" in lib.pgb_last_error()
    # the tensor-core evolve checks its shapes before touching a device
    import numpy as np
    a = np.zeros((4, 20), np.float32)
    b = np.zeros((70, 20), np.float32)
    o = np.zeros((4, 70), np.float32)
    assert lib.pgb_tc_evolve(a.ctypes.data, b.ctypes.data, o.ctypes.data, 4, 20, 70) == 1
    assert b"tc_evolve" in lib.pgb_last_error()
    assert lib.pgb_tc_evolve(a.ctypes.data, b.ctypes.data, o.ctypes.data, 4, 25, 8) == 1
    assert lib.pgb_tc_evolve(a.ctypes.data, b.ctypes.data, o.ctypes.data, 0, 20, 8) == 0  # nothing to do
