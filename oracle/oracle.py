"""ORACLE -- test infrastructure only. Loads the CPU restatement (refcpu.c) and exposes it
behind the same facade as the product, so tests can run a scene through both and compare.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

from neofiz_gb300 import _abi
from neofiz_gb300.batch import BatchSolver
from neofiz_gb300.solver import ExplicitSolver

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIBRARY = os.path.join(BUILD, "liboracle.so")
SOURCES = [os.path.join(HERE, "refcpu.c")]
CFLAGS = ["-O2", "-std=gnu11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
          "-pthread"]


def build(force: bool = False) -> str:
    """Compiles refcpu.c with contraction off (bitwise Java evaluation order)."""
    os.makedirs(BUILD, exist_ok=True)
    csrc = os.path.join(HERE, "..", "neofiz_gb300", "csrc")
    deps = SOURCES + [os.path.join(HERE, "..", "include", "neofiz.h"),
                      os.path.join(csrc, "nf_math.h"), os.path.join(csrc, "nf_math_tables.h"),
                      os.path.join(csrc, "nf_adjoint.h")]
    if not force and os.path.exists(LIBRARY):
        t = os.path.getmtime(LIBRARY)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIBRARY
    tmp = LIBRARY + ".tmp"
    subprocess.check_call(["gcc", *CFLAGS, *SOURCES, "-o", tmp, "-lm"])
    os.replace(tmp, LIBRARY)
    return LIBRARY


_api = None


def api():
    global _api
    if _api is None:
        lib = ctypes.CDLL(build())
        _api = _abi.bind(lib, "nfo_")
        lib.nfo_jc_flow_stress.restype = ctypes.c_double
        lib.nfo_jc_flow_stress.argtypes = [ctypes.POINTER(_abi.MaterialC), ctypes.c_double,
                                           ctypes.c_double, ctypes.c_double]
        lib.nfo_math.restype = ctypes.c_double
        lib.nfo_math.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double]
    return _api


class OracleSolver(ExplicitSolver):
    """The reference algorithm on the CPU, behind the product's facade."""

    @classmethod
    def _binding(cls):
        return api()


class OracleBatch(BatchSolver):
    """The reference's sweep (one CPU solver per instance, a thread pool over instances)
    behind the product's batch facade. NFO_THREADS sets the pool size."""

    @classmethod
    def _binding(cls):
        return api()


def math_fn(which: str, x: float, y: float = 0.0) -> float:
    idx = ["log", "exp", "pow", "atan2", "sin", "cos", "hypot"].index(which)
    return api().lib.nfo_math(idx, x, y)


def jc_flow_stress(material, eps, rate, temperature) -> float:
    return api().lib.nfo_jc_flow_stress(ctypes.byref(_abi.material_struct(material)), eps,
                                        rate, temperature)
