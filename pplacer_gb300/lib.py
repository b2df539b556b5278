"""ctypes binding of the C ABI in include/pplacer_gb300.h.

The shared library is built in-tree (pplacer_gb300/_build/libpplacer_gb300.so,
see pplacer_gb300/build.py).  There is no fallback: if the library is missing
or the GPU is unusable, the calls raise.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpplacer_gb300.so")

PGB_OK = 0


class PgbError(RuntimeError):
    pass


class ModelDesc(C.Structure):
    _fields_ = [("n_states", C.c_int), ("n_rates", C.c_int), ("gcat", C.c_int), ("n_sites", C.c_int),
                ("statd", C.c_void_p), ("x", C.c_void_p), ("lambda_", C.c_void_p), ("xit", C.c_void_p),
                ("rates", C.c_void_p), ("site_categories", C.c_void_p)]


class TreeDesc(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("parent", C.c_void_p), ("bl", C.c_void_p)]


class Prefs(C.Structure):
    _fields_ = [("start_pend", C.c_double), ("max_pend", C.c_double), ("initial_tolerance", C.c_double),
                ("max_strikes", C.c_int), ("strike_box", C.c_double), ("max_pitches", C.c_int),
                ("keep_at_most", C.c_int), ("keep_factor", C.c_double), ("optimizer", C.c_int),
                ("calc_pp", C.c_int), ("prior", C.c_int), ("pp_rel_err", C.c_double), ("prior_lower", C.c_double),
                ("pp_rule", C.c_int)]


class Placement(C.Structure):
    _fields_ = [("edge", C.c_int), ("pad", C.c_int), ("like", C.c_double), ("lwr", C.c_double),
                ("dist", C.c_double), ("pend", C.c_double), ("marginal_like", C.c_double), ("post_prob", C.c_double)]


class Trial(C.Structure):
    _fields_ = [("query", C.c_int), ("edge", C.c_int), ("pend0", C.c_double), ("dist0", C.c_double),
                ("tol", C.c_double)]


class TrialOut(C.Structure):
    _fields_ = [("like", C.c_double), ("pend", C.c_double), ("dist", C.c_double), ("derivs", C.c_double * 6),
                ("status", C.c_int), ("n_evals", C.c_int)]


_lib = None


def load(build_if_missing=True):
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise PgbError("pplacer_gb300 library not built: %s" % LIB_PATH)
        from . import build
        build.build()
    L = C.CDLL(LIB_PATH)
    dp, vp, i, d = C.c_void_p, C.c_void_p, C.c_int, C.c_double
    L.pgb_last_error.restype = C.c_char_p
    L.pgb_kernel_launch_count.restype = C.c_uint64
    for name, args in [("pgb_gemmish", [dp, dp, dp, i, i]), ("pgb_dediagonalize", [dp, dp, dp, dp, i]),
                       ("pgb_mat_pairwise_prod", [dp, dp, dp, i, i]),
                       ("pgb_mat_statd_pairwise_prod", [dp, dp, dp, dp, i, i]),
                       ("pgb_ten_pairwise_prod", [dp, dp, dp, i, i, i]),
                       ("pgb_ten_statd_pairwise_prod", [dp, dp, dp, dp, i, i, i]),
                       ("pgb_vec_pairwise_prod", [dp, dp, dp, i]),
                       ("pgb_int_vec_pairwise_prod", [vp, vp, vp, i]),
                       ("pgb_float_mat_int_vec_mul", [dp, dp, vp, i, i]),
                       ("pgb_tc_evolve", [vp, vp, vp, i, i, i])]:
        getattr(L, name).argtypes = args
        getattr(L, name).restype = i
    for name, args in [("pgb_mat_log_like3", [dp, dp, dp, dp, i, i]),
                       ("pgb_mat_masked_logdot", [dp, dp, vp, i, i]),
                       ("pgb_mat_bounded_logdot", [dp, dp, i, i, i, i]),
                       ("pgb_ten_log_like3", [dp, dp, dp, dp, dp, i, i, i]),
                       ("pgb_ten_masked_logdot", [dp, dp, vp, dp, i, i, i]),
                       ("pgb_ten_bounded_logdot", [dp, dp, i, i, dp, i, i, i])]:
        getattr(L, name).argtypes = args
        getattr(L, name).restype = d
    L.pgb_int_vec_tot.argtypes = [vp, i]
    L.pgb_int_vec_tot.restype = i
    L.pgb_engine_create.argtypes = [C.POINTER(ModelDesc), C.POINTER(TreeDesc), C.POINTER(C.c_void_p)]
    L.pgb_engine_destroy.argtypes = [vp]
    L.pgb_engine_precompute.argtypes = [vp, vp, C.c_char_p, i]
    L.pgb_engine_refine_categories.argtypes = [vp, vp, C.c_char_p, i, vp]
    L.pgb_engine_set_glvs.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    L.pgb_engine_get_glv.argtypes = [vp, i, i, vp, vp]
    L.pgb_prefs_default.argtypes = [C.POINTER(Prefs)]
    L.pgb_prefs_default.restype = None
    L.pgb_place.argtypes = [vp, C.POINTER(Prefs), i, C.c_char_p, vp, vp, vp]
    L.pgb_place_batch.argtypes = [vp, C.POINTER(Prefs), i, vp, i, vp, vp, vp]
    L.pgb_host_alloc.argtypes = [C.c_size_t, C.POINTER(C.c_void_p)]
    L.pgb_host_free.argtypes = [vp]
    L.pgb_queries_load.argtypes = [vp, i, C.c_char_p]
    L.pgb_queries_run.argtypes = [vp, C.POINTER(Prefs)]
    L.pgb_queries_fetch.argtypes = [vp, vp, vp, vp]
    L.pgb_queries_stage1.argtypes = [vp, C.POINTER(Prefs), vp]
    L.pgb_queries_rank.argtypes = [vp, C.POINTER(Prefs), i, vp]
    L.pgb_queries_trials.argtypes = [vp, C.POINTER(Prefs), i, i, i, vp, vp]
    L.pgb_engine_timings.argtypes = [vp, vp, vp]
    L.pgb_engine_autotune.argtypes = [vp, C.POINTER(Prefs)]
    L.pgb_engine_get_tuning.argtypes = [vp, vp, vp]
    L.pgb_engine_set_tuning.argtypes = [vp, vp, vp]
    for name in ["pgb_engine_create", "pgb_engine_destroy", "pgb_engine_precompute", "pgb_engine_refine_categories",
                 "pgb_engine_set_glvs",
                 "pgb_engine_get_glv", "pgb_place", "pgb_place_batch", "pgb_queries_load", "pgb_queries_run", "pgb_queries_fetch",
                 "pgb_queries_stage1", "pgb_queries_rank", "pgb_queries_trials", "pgb_engine_timings", "pgb_engine_autotune",
                 "pgb_engine_get_tuning", "pgb_engine_set_tuning", "pgb_host_alloc", "pgb_host_free"]:
        getattr(L, name).restype = i
    _lib = L
    return L


def check(status, what=""):
    if status != PGB_OK:
        msg = load().pgb_last_error().decode(errors="replace")
        raise PgbError("%s failed (status %d): %s" % (what, status, msg))


def ptr(a):
    return None if a is None else a.ctypes.data


def header_symbols():
    """Every function the public header declares."""
    import re
    hdr = os.path.join(os.path.dirname(HERE), "include", "pplacer_gb300.h")
    text = re.sub(r"/\*.*?\*/", "", open(hdr).read(), flags=re.S)
    return sorted(set(re.findall(r"\b(pgb_[a-z0-9_]+)\s*\(", text)))


class HostBuffer:
    """Page-locked host memory from pgb_host_alloc, freed on close / deletion."""

    def __init__(self, nbytes):
        self.ptr = C.c_void_p()
        self.nbytes = int(nbytes)
        check(load().pgb_host_alloc(self.nbytes, C.byref(self.ptr)), "pgb_host_alloc")

    @property
    def address(self):
        return self.ptr.value

    def array(self, dtype, count):
        """A numpy view of the first count elements of dtype."""
        import numpy as np
        dt = np.dtype(dtype)
        assert count * dt.itemsize <= self.nbytes
        buf = (C.c_char * (count * dt.itemsize)).from_address(self.ptr.value)
        return np.frombuffer(buf, dtype=dt, count=count)

    def close(self):
        if self.ptr and self.ptr.value:
            load().pgb_host_free(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
