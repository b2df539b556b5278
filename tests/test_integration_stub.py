"""The OCaml stub file integration/linear_gpu_stubs.c -- pplacer's Linear
externals (linear.ml:13-89) over the GPU library -- compiled the way pplacer
would compile it, against a stand-in for the OCaml runtime headers
(oracle/shim), and called through its value-typed CAMLprim symbols with
OCaml-shaped bigarrays.

CPU: it compiles, links against the library and exports every external the
reference's linear.ml binds.  GPU: gemmish_c, ten_log_like3_c,
ten_masked_logdot_c (and the other numeric stubs) against the FP64 oracle.
"""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
STUB = os.path.join(ROOT, "integration", "linear_gpu_stubs.c")
REF_LINEAR_ML = "/root/reference/pplacer_src/linear.ml"

# the externals of linear.ml:13-89
EXTERNALS = ["gemmish_c", "dediagonalize", "mat_print_c", "mat_log_like3_c", "mat_pairwise_prod_c",
             "mat_statd_pairwise_prod_c", "mat_masked_logdot_c", "mat_bounded_logdot_c", "ten_print_c",
             "ten_log_like3_c", "ten_pairwise_prod_c", "ten_statd_pairwise_prod_c", "ten_masked_logdot_c",
             "ten_bounded_logdot_c", "vec_pairwise_prod_c", "int_vec_tot_c", "int_vec_pairwise_prod_c",
             "float_mat_int_vec_mul_c"]


def _build_stub(out_dir):
    from pplacer_gb300 import build as B
    lib = B.build()
    so = os.path.join(str(out_dir), "liblinear_gpu_stubs.so")
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-Wall", "-Werror", "-I", os.path.join(ROOT, "oracle", "shim"),
           "-I", os.path.join(ROOT, "include"), STUB, "-o", so, "-L", os.path.dirname(lib), "-lpplacer_gb300",
           "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return so


def test_stub_compiles_and_exports_every_external(tmp_path):
    so = _build_stub(tmp_path)
    names = EXTERNALS
    if os.path.exists(REF_LINEAR_ML):  # the names the reference binds, read from its source
        text = open(REF_LINEAR_ML).read()
        names = re.findall(r'external\s+\w+\s*:[^=]*=\s*"(\w+)"', text)
        assert sorted(names) == sorted(EXTERNALS)
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT\s+(\w+)", out))
    assert not [n for n in names if n not in exported]


class _Ba(C.Structure):  # struct caml_ba_array of the shim
    _fields_ = [("data", C.c_void_p), ("num_dims", C.c_ssize_t), ("flags", C.c_ssize_t), ("proxy", C.c_void_p),
                ("dim", C.c_ssize_t * 4)]


def _val(arr, keep):
    ba = _Ba()
    ba.data = arr.ctypes.data
    ba.num_dims = arr.ndim
    for i, n in enumerate(arr.shape):
        ba.dim[i] = n
    keep.append((ba, arr))
    return C.addressof(ba)


def _int_val(n):
    return (n << 1) + 1


@pytest.mark.gpu
def test_stub_calls_match_oracle(tmp_path, oracle_lib):
    O = oracle_lib
    so = C.CDLL(_build_stub(tmp_path))
    for n in EXTERNALS:
        getattr(so, n).restype = C.c_ssize_t
    rng = np.random.default_rng(5)
    keep = []
    R, S, K = 4, 333, 4
    unit = _int_val(0)
    # gemmish_c: dst[s] = a b[s]
    a = np.ascontiguousarray(rng.random((K, K)))
    b = np.ascontiguousarray(rng.random((S, K)))
    dst = np.zeros((S, K))
    assert so.gemmish_c(C.c_ssize_t(_val(dst, keep)), C.c_ssize_t(_val(a, keep)), C.c_ssize_t(_val(b, keep))) == unit
    want = np.zeros((S, K))
    O.lib().orc_gemmish(want, a, b, S, K)
    np.testing.assert_allclose(dst, want, rtol=1e-14)
    # ten_log_like3_c and ten_masked_logdot_c return a boxed double
    statd = np.ascontiguousarray(rng.dirichlet(np.ones(K)))
    x, y, z = (np.ascontiguousarray(rng.random((R, S, K)) + 0.01) for _ in range(3))
    util = np.zeros(S)
    box = so.ten_log_like3_c(*(C.c_ssize_t(_val(v, keep)) for v in (statd, x, y, z, util)))
    got = C.cast(C.c_void_p(box), C.POINTER(C.c_double))[0]
    want = O.lib().orc_ten_log_like3(statd, x, y, z, np.zeros(S), R, S, K)
    assert abs(got - want) <= 1e-12 * abs(want), (got, want)
    mask = np.ascontiguousarray((rng.random(S) < 0.7).astype(np.uint16))
    box = so.ten_masked_logdot_c(*(C.c_ssize_t(_val(v, keep)) for v in (x, y, mask, util)))
    got = C.cast(C.c_void_p(box), C.POINTER(C.c_double))[0]
    want = O.lib().orc_ten_masked_logdot(x, y, mask, np.zeros(S), R, S, K)
    assert abs(got - want) <= 1e-12 * abs(want), (got, want)
    # dediagonalize and the integer helpers
    u, uit = (np.ascontiguousarray(rng.random((K, K))) for _ in range(2))
    lam = np.ascontiguousarray(rng.random(K))
    pm = np.zeros((K, K))
    assert so.dediagonalize(*(C.c_ssize_t(_val(v, keep)) for v in (pm, u, lam, uit))) == unit
    np.testing.assert_allclose(pm, (u * lam) @ uit.T, rtol=1e-13)
    iv = np.ascontiguousarray(rng.integers(0, 9, size=50).astype(np.uint16))
    assert so.int_vec_tot_c(C.c_ssize_t(_val(iv, keep))) == _int_val(int(iv.sum()))
    fv = np.zeros(K)
    mat = np.ascontiguousarray(rng.random((50, K)))
    assert so.float_mat_int_vec_mul_c(*(C.c_ssize_t(_val(v, keep)) for v in (fv, mat, iv))) == unit
    np.testing.assert_allclose(fv, iv.astype(np.float64) @ mat, rtol=1e-13)
