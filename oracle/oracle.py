"""Python handle on the CPU oracle (oracle/esf_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline legs as the checker; never by eulersf_gb300.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libesf_oracle.so")
SRC = os.path.join(HERE, "esf_oracle.c")

_lib = None


def build(force: bool = False) -> str:
    """Compile the restatement (gcc, no FMA contraction so x86 and aarch64
    give the same bits)."""
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "esf_oracle.h"))):
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fopenmp", "-fPIC",
                               "-shared", "-o", tmp, SRC, "-lm"])
        os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        from eulersf_gb300 import abi
        build()
        lib = C.CDLL(LIB)
        abi.declare(lib, "esfo_", device_pointer_ops=False)
        lib.esfo_create.argtypes = [C.POINTER(abi.Grid), C.POINTER(abi.Params)]
        dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
        lib.esfo_pressure_apply.argtypes = [C.POINTER(abi.Grid), dp, dp, dp]
        lib.esfo_pressure_solve.argtypes = [C.POINTER(abi.Grid), dp, dp, dp, dp, C.c_double,
                                            C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]
        lib.esfo_mt19937.argtypes = [C.c_uint32, np.ctypeslib.ndpointer(dtype=np.uint32),
                                     C.c_long]
        _lib = lib
    return _lib


def scene(desc, noise=True):
    """Oracle integrator for a synthetic scene (same set-up as the product)."""
    from eulersf_gb300.integrator import build_from_scene
    return build_from_scene(load(), "esfo_", desc, noise=noise)


def grid(res, dh):
    from eulersf_gb300 import abi
    return abi.Grid(res, res, res, dh, (C.c_double * 3)(0, 0, 0))


def pressure_apply(g, mass_inv_node, x):
    out = np.zeros((g.xRes - 1) * (g.yRes - 1) * (g.zRes - 1))
    st = load().esfo_pressure_apply(C.byref(g), np.ascontiguousarray(mass_inv_node, np.float64),
                                    np.ascontiguousarray(x, np.float64), out)
    assert st == 0
    return out


def pressure_residual(I):
    """||J M^-1 J^T lambda1 - b1|| / ||b1|| of an integrator's last pressure
    solve (getMatVecMult, COUPLED_INTEGRATOR_3D.cpp:638-660, applied by the
    oracle on the CPU): an independent check of a solve's answer. I is any
    CoupledIntegrator3D (the CUDA library's or the oracle's)."""
    dof = I.get("gridIdxToSolutionIdx")
    mv = I.get("nzMassVecInv").reshape(-1, 3)
    assert np.array_equal(mv[:, 0], mv[:, 1]) and np.array_equal(mv[:, 0], mv[:, 2])
    minv = np.zeros(len(dof))
    minv[dof >= 0] = mv[dof[dof >= 0], 0]
    from eulersf_gb300 import abi
    g = abi.Grid(I.xRes(), I.yRes(), I.zRes(), I.dh(), (C.c_double * 3)(*I.origin()))
    b = I.get("b1")
    r = pressure_apply(g, minv, I.get("lambda1")) - b
    return float(np.linalg.norm(r) / np.linalg.norm(b))


def pressure_solve(g, mass_inv_node, diag, b, x0, eps, max_it):
    x = np.array(x0, dtype=np.float64, copy=True)
    it, rr = C.c_int(), C.c_double()
    st = load().esfo_pressure_solve(C.byref(g), np.ascontiguousarray(mass_inv_node, np.float64),
                                    np.ascontiguousarray(diag, np.float64),
                                    np.ascontiguousarray(b, np.float64), x, eps, max_it,
                                    C.byref(it), C.byref(rr))
    return x, it.value, rr.value, st


def mt19937(seed, n):
    out = np.empty(n, dtype=np.uint32)
    load().esfo_mt19937(seed, out, n)
    return out
