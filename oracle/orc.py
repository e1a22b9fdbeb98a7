"""Python loader of the CPU oracle (oracle/sps_oracle.c).  TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
PARITY UNPINNED: no Fortran compiler exists to run the reference itself; the oracle is
pinned by its own known-answer and invariant tests.
"""
import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "build")
LIB = os.path.join(BUILD, "libsps_oracle.so")
SRC = os.path.join(HERE, "sps_oracle.c")
HDRS = [os.path.join(HERE, "sps_oracle.h"), os.path.join(HERE, "..", "include", "sps.h")]

_LIB = None


def build(force=False):
    """Compile the oracle with -ffp-contract=off (no fused multiply-add, as gfortran -O3 on
    x86-64 produces for the reference)."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [SRC] + HDRS
    if not force and os.path.exists(LIB) and all(
            os.path.getmtime(s) <= os.path.getmtime(LIB) for s in srcs):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-Wall", "-o", LIB, SRC, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def lib():
    global _LIB
    if _LIB is None:
        import sps_gb300._abi as abi
        L = C.CDLL(build())
        abi.declare_step_api(L, "orc")
        P = C.POINTER
        L.orc_kernel.argtypes = [C.c_int32, C.c_double, C.c_double, P(C.c_double), C.c_double,
                                 P(C.c_double), P(C.c_double)]
        L.orc_kernel.restype = None
        L.orc_adapt_stress.argtypes = [C.c_double, C.c_double, P(C.c_double)]
        L.orc_adapt_stress.restype = None
        L.orc_drucker_prager.argtypes = [P(C.c_double), C.c_double, P(C.c_double),
                                         P(C.c_double), P(C.c_double), P(C.c_double),
                                         P(C.c_double)]
        L.orc_drucker_prager.restype = None
        L.orc_viscoplastic.argtypes = [P(C.c_double), C.c_int, P(C.c_double), C.c_double,
                                       P(C.c_double), P(C.c_double)]
        L.orc_viscoplastic.restype = None
        L.orc_artificial_force.argtypes = [C.c_void_p, P(C.c_double)]
        L.orc_artificial_force.restype = None
        _LIB = L
    return _LIB


def context(params):
    """An oracle StepContext with the same API as the GPU Solver's context."""
    from sps_gb300.context import StepContext
    return StepContext(lib(), "orc", params)
