"""Build and load the oracle's C arithmetic (``clv.c``) as a shared library.

Test infrastructure only. Output goes to ``oracle/_build/`` (git-ignored).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")


SOURCES = ["clv.c", "sweep.c"]


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    if (not force and os.path.exists(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in srcs)):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O3", "-fPIC", "-shared", "-fopenmp",
                           "-std=c99"] + srcs + ["-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        dp = ctypes.POINTER(ctypes.c_double)
        up = ctypes.POINTER(ctypes.c_uint32)
        _lib.oracle_update_partial.argtypes = [
            ctypes.c_int64, ctypes.c_int, ctypes.c_int, dp, up, dp, up, dp,
            dp, up, dp]
        _lib.oracle_update_partial.restype = None
        _lib.oracle_root_logl.argtypes = [
            ctypes.c_int64, ctypes.c_int, ctypes.c_int, dp, up, dp, dp, dp, dp, ctypes.c_double, dp]
        _lib.oracle_root_logl.restype = ctypes.c_double
        _lib.oracle_num_threads.restype = ctypes.c_int
    return _lib


def _dp(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _up(a):
    if a is None:
        return None
    assert a.dtype == np.uint32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


def update_partial(parent, parent_scaler, left, left_scaler, pl,
                   right, right_scaler, pr):
    n, R, S = parent.shape
    lib().oracle_update_partial(n, R, S, _dp(parent), _up(parent_scaler),
                                _dp(left), _up(left_scaler), _dp(pl),
                                _dp(right), _up(right_scaler), _dp(pr))


def root_logl(clv, scaler, freqs, rate_weights, weights, persite=None, gamma_frac=1.0, inv_term=None):
    n, R, S = clv.shape
    return lib().oracle_root_logl(n, R, S, _dp(clv), _up(scaler), _dp(freqs),
                                  _dp(rate_weights), _dp(weights),
                                  _dp(persite), float(gamma_frac), _dp(inv_term))
