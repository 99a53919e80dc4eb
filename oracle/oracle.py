"""ctypes front end of the CPU oracle (test infrastructure only).

Builds oracle/_build/liboracle.so from trans_oracle.cpp when needed and drives it through
the same Python driver as the GPU library (the two export the same ABI under different
prefixes).  Only tests, the smoke check and the CPU-baseline leg of bench.py use this.
"""
import ctypes as C
import os
import subprocess

from trans_gb300 import abi
from trans_gb300.solver import Solver

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build(force=False):
    src = os.path.join(HERE, "trans_oracle.cpp")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(LIB)
        vp = C.c_void_p
        lib.oracle_create.argtypes = [C.POINTER(abi.TransParams), C.c_int, C.POINTER(abi.TransBlock), C.POINTER(vp)]
        lib.oracle_destroy.argtypes = [vp]
        lib.oracle_set_field.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_double)]
        lib.oracle_get_field.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_double)]
        lib.oracle_iterate.argtypes = [vp, C.c_int, C.POINTER(abi.TransNorms)]
        lib.oracle_run_stage.argtypes = [vp, C.c_int, C.c_int, C.c_int]
        lib.oracle_get_norms.argtypes = [vp, C.POINTER(abi.TransNorms)]
        lib.oracle_set_threads.argtypes = [C.c_int]
        lib.oracle_set_threads.restype = C.c_int
        lib.oracle_alimiter.argtypes = [C.c_double, C.c_double]
        lib.oracle_alimiter.restype = C.c_double
        lib.oracle_muscl2_limiter.argtypes = [C.c_double, C.c_double]
        lib.oracle_muscl2_limiter.restype = C.c_double
        dp = C.POINTER(C.c_double)
        lib.oracle_ausmpw.argtypes = [C.POINTER(abi.TransParams), dp, dp]
        lib.oracle_roe.argtypes = [C.POINTER(abi.TransParams), dp, dp]
        lib.oracle_mdcd.argtypes = [dp, C.c_double, dp]
        for f in ("exp", "expm1", "tanh", "log", "atan"):
            fn = getattr(lib, "oracle_tm_" + f)
            fn.argtypes = [C.c_double]
            fn.restype = C.c_double
        lib.oracle_tm_pow.argtypes = [C.c_double, C.c_double]
        lib.oracle_tm_pow.restype = C.c_double
        _lib = lib
    return _lib


def OracleSolver(case, conns, geo, state, params=None):
    return Solver(case, conns, geo, state, lib=load(), prefix="oracle_", params=params)
