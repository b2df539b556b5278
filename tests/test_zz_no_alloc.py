"""The allocation-free entry point pgb_ten_log_like3_noalloc.

It exists for callers that cannot allocate device memory when they need a
likelihood (their device memory belongs to another runtime's pool, or they
allocate only at start-up): they pass device buffers, and the function's
scratch is a fixed array inside the library.  This test owns the device
buffers (through torch), calls the entry point through the C ABI twice in a
row on different inputs, and checks each result against the host-pointer
drop-in pgb_ten_log_like3 and against the FP64 oracle (oracle.cpp's
restatement of linear_c.c's ten_log_like3_c) at the drop-in tolerance.  The file is named so
pytest collects it last.
"""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lib():
    from pplacer_gb300 import lib as L
    lib = L.load()
    f = lib.pgb_ten_log_like3_noalloc
    f.argtypes = [C.c_void_p] * 4 + [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return L, lib, f


def test_noalloc_matches_dropin_twice(oracle_lib):
    import torch
    from pplacer_gb300 import linear
    L, lib, f = _lib()
    rng = np.random.default_rng(21)
    dev = torch.device("cuda:0")
    for call, (R, S, K) in enumerate(((4, 1500, 4), (3, 777, 20))):
        statd = rng.dirichlet(np.ones(K))
        x, y, z = (rng.random((R, S, K)) + 0.01 for _ in range(3))
        want = linear.ten_log_like3(statd, x, y, z, np.zeros(S))
        want_orc = oracle_lib.lib().orc_ten_log_like3(statd, x, y, z, np.zeros(S), R, S, K)
        t = [torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (statd, x, y, z)]
        out = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        st = f(t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), t[3].data_ptr(), R, S, K, out.data_ptr(), None)
        assert st == 0, lib.pgb_last_error()
        torch.cuda.synchronize()
        got = float(out.item())
        assert math.isclose(got, want, rel_tol=1e-12), (call, got, want)
        assert math.isclose(got, want_orc, rel_tol=1e-12), (call, got, want_orc)


def test_noalloc_rejects_oversized_input():
    import torch
    L, lib, f = _lib()
    dev = torch.device("cuda:0")
    big = 1 << 16
    buf = torch.zeros(4 * (big + 1) * 4 + 4, dtype=torch.float64, device=dev)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    p = buf.data_ptr()
    st = f(p, p, p, p, 1, big + 1, 4, out.data_ptr(), None)
    assert st == 1 and b"exceed" in lib.pgb_last_error()
