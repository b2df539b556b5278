"""Python mirror of pplacer's ``Linear`` module (pplacer_src/linear.ml:13-89)
over the GPU drop-in of include/pplacer_gb300.h.

Same function names, argument order and meaning as the OCaml externals:
arrays are C-contiguous float64 (matrices [site][state], tensors
[rate][site][state]) and uint16 masks; results are written in place into
``dst`` / ``util`` or returned as floats.  Like linear_c.c, mismatched sizes
only print a warning.  A failing GPU raises ``PgbError``.
"""
import math

import numpy as np

from . import lib as _L


def _f64(a):
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous):
        raise TypeError("expected a C-contiguous float64 array")
    return a


def _u16(a):
    if not (isinstance(a, np.ndarray) and a.dtype == np.uint16 and a.flags.c_contiguous):
        raise TypeError("expected a C-contiguous uint16 array")
    return a


def _status(st, what):
    _L.check(st, what)


def _value(v, what):
    if isinstance(v, float) and math.isnan(v):
        msg = _L.load().pgb_last_error().decode(errors="replace")
        if msg:
            raise _L.PgbError("%s failed: %s" % (what, msg))
    return v


def gemmish(dst, a, b):
    """dst = a * b^T per site (linear_c.c:29-90)."""
    _f64(dst), _f64(a), _f64(b)
    n_states, n_sites = a.shape[0], b.shape[0]
    if a.shape[1] != n_states or dst.shape != (n_sites, n_states):
        print("bad input dimensions!")
    _status(_L.load().pgb_gemmish(dst.ctypes.data, a.ctypes.data, b.ctypes.data, n_sites, n_states), "gemmish")


def dediagonalize(dst, u, lam, uit):
    """dst_ij = sum_k lam_k u_ik uit_jk (linear_c.c:92-146)."""
    _f64(dst), _f64(u), _f64(lam), _f64(uit)
    _status(_L.load().pgb_dediagonalize(dst.ctypes.data, u.ctypes.data, lam.ctypes.data, uit.ctypes.data, len(lam)),
            "dediagonalize")


def mat_log_like3(statd, x, y, z):
    for a in (statd, x, y, z):
        _f64(a)
    n_sites, n_states = x.shape
    return _value(_L.load().pgb_mat_log_like3(statd.ctypes.data, x.ctypes.data, y.ctypes.data, z.ctypes.data,
                                              n_sites, n_states), "mat_log_like3")


def mat_pairwise_prod(dst, x, y):
    for a in (dst, x, y):
        _f64(a)
    n_sites, n_states = x.shape
    _status(_L.load().pgb_mat_pairwise_prod(dst.ctypes.data, x.ctypes.data, y.ctypes.data, n_sites, n_states),
            "mat_pairwise_prod")


def mat_statd_pairwise_prod(statd, dst, a, b):
    for v in (statd, dst, a, b):
        _f64(v)
    n_sites, n_states = a.shape
    _status(_L.load().pgb_mat_statd_pairwise_prod(statd.ctypes.data, dst.ctypes.data, a.ctypes.data, b.ctypes.data,
                                                  n_sites, n_states), "mat_statd_pairwise_prod")


def mat_masked_logdot(x, y, mask):
    _f64(x), _f64(y), _u16(mask)
    n_sites, n_states = x.shape
    if n_sites != mask.shape[0]:
        print("mat_masked_logdot_c: Mask length doesn't match!")
    return _value(_L.load().pgb_mat_masked_logdot(x.ctypes.data, y.ctypes.data, mask.ctypes.data, n_sites, n_states),
                  "mat_masked_logdot")


def mat_bounded_logdot(x, y, first, last):
    _f64(x), _f64(y)
    n_sites, n_states = x.shape
    return _value(_L.load().pgb_mat_bounded_logdot(x.ctypes.data, y.ctypes.data, first, last, n_sites, n_states),
                  "mat_bounded_logdot")


def ten_log_like3(statd, x, y, z, util):
    for a in (statd, x, y, z, util):
        _f64(a)
    n_rates, n_sites, n_states = x.shape
    return _value(_L.load().pgb_ten_log_like3(statd.ctypes.data, x.ctypes.data, y.ctypes.data, z.ctypes.data,
                                              util.ctypes.data, n_rates, n_sites, n_states), "ten_log_like3")


def ten_pairwise_prod(dst, x, y):
    for a in (dst, x, y):
        _f64(a)
    n_rates, n_sites, n_states = x.shape
    _status(_L.load().pgb_ten_pairwise_prod(dst.ctypes.data, x.ctypes.data, y.ctypes.data, n_rates, n_sites,
                                            n_states), "ten_pairwise_prod")


def ten_statd_pairwise_prod(statd, dst, a, b):
    for v in (statd, dst, a, b):
        _f64(v)
    n_rates, n_sites, n_states = a.shape
    _status(_L.load().pgb_ten_statd_pairwise_prod(statd.ctypes.data, dst.ctypes.data, a.ctypes.data, b.ctypes.data,
                                                  n_rates, n_sites, n_states), "ten_statd_pairwise_prod")


def ten_masked_logdot(x, y, mask, util):
    _f64(x), _f64(y), _u16(mask), _f64(util)
    n_rates, n_sites, n_states = x.shape
    if n_sites != mask.shape[0]:
        print("ten_masked_logdot_c: Mask length doesn't match!")
    if n_sites != util.shape[0]:
        print("ten_masked_logdot_c: Util length doesn't match!")
    return _value(_L.load().pgb_ten_masked_logdot(x.ctypes.data, y.ctypes.data, mask.ctypes.data, util.ctypes.data,
                                                  n_rates, n_sites, n_states), "ten_masked_logdot")


def ten_bounded_logdot(x, y, first, last, util):
    _f64(x), _f64(y), _f64(util)
    n_rates, n_sites, n_states = x.shape
    return _value(_L.load().pgb_ten_bounded_logdot(x.ctypes.data, y.ctypes.data, first, last, util.ctypes.data,
                                                   n_rates, n_sites, n_states), "ten_bounded_logdot")


def vec_pairwise_prod(dst, x, y):
    for a in (dst, x, y):
        _f64(a)
    _status(_L.load().pgb_vec_pairwise_prod(dst.ctypes.data, x.ctypes.data, y.ctypes.data, x.shape[0]),
            "vec_pairwise_prod")


def int_vec_tot(x):
    _u16(x)
    v = _L.load().pgb_int_vec_tot(x.ctypes.data, x.shape[0])
    msg = _L.load().pgb_last_error().decode(errors="replace")
    if v == 0 and msg:
        raise _L.PgbError("int_vec_tot failed: " + msg)
    return v


def int_vec_pairwise_prod(dst, x, y):
    for a in (dst, x, y):
        _u16(a)
    _status(_L.load().pgb_int_vec_pairwise_prod(dst.ctypes.data, x.ctypes.data, y.ctypes.data, dst.shape[0]),
            "int_vec_pairwise_prod")


def float_mat_int_vec_mul(dst, mat, vec):
    _f64(dst), _f64(mat), _u16(vec)
    n, k = mat.shape
    if vec.shape[0] != n:
        raise ValueError("dim_0 vec != dim_0 mat")
    if dst.shape[0] != k:
        raise ValueError("dim_0 dst != dim_1 mat")
    _status(_L.load().pgb_float_mat_int_vec_mul(dst.ctypes.data, mat.ctypes.data, vec.ctypes.data, n, k),
            "float_mat_int_vec_mul")
