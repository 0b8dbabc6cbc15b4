"""ctypes binding of the FP64 CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: a restatement of the reference algorithm
(konsim83/MPI-MSFEC) used as the checker in tests/, in
``__graft_entry__.smoke()`` and as the timed CPU baseline in ``bench.py``. The
product library never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

LOAD_ZERO, LOAD_CONSTANT, LOAD_SIN_PRODUCT = 0, 1, 2
SOLVER_DIRECT, SOLVER_CG_SSOR = 0, 1
COEF_SCALAR, COEF_TENSOR, COEF_GAUSS = 0, 1, 2

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build() -> str:
    """Compile the oracle with its Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        L.oracle_q1_build.restype = ctypes.c_int
        L.oracle_q1_build.argtypes = [ctypes.c_int, _dp, _dp, _ip, _dp, _dp, ctypes.c_int, _dp,
                                      ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp, _dp, _dp,
                                      _ip, ctypes.c_int]
        L.oracle_q1_assemble.restype = ctypes.c_int
        L.oracle_q1_assemble.argtypes = [_dp, _dp, ctypes.c_int, _dp, _dp, ctypes.c_int, _dp,
                                         _ip, _ip, _dp, _dp]
        L.oracle_q1_build_coef.restype = ctypes.c_int
        L.oracle_q1_build_coef.argtypes = [ctypes.c_int, _dp, _dp, _ip, ctypes.c_int, _dp, _dp, ctypes.c_int,
                                           _dp, ctypes.c_int, ctypes.c_double, ctypes.c_int, _dp, _dp, _dp,
                                           _ip, ctypes.c_int]
        L.oracle_q1_assemble_coef.restype = ctypes.c_int
        L.oracle_q1_assemble_coef.argtypes = [_dp, _dp, ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_int, _dp,
                                              _ip, _ip, _dp, _dp]
        L.oracle_nedelec_dof_values_unit_cube.restype = ctypes.c_int
        L.oracle_nedelec_dof_values_unit_cube.argtypes = [ctypes.c_int, _dp, _dp, ctypes.c_int]
        _lib = L
    return _lib


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _i(a):
    return None if a is None else a.ctypes.data_as(_ip)


def q1_build(origin, size, depth, a, r=None, load_kind=LOAD_ZERO, load_params=(0, 0, 0, 0),
             solver=SOLVER_DIRECT, tol=1e-12, max_iter=1000, want_phi=True, nthreads=0, coef_mode=0):
    """Q1 basis build (reference QBasis::run, source/Q/q_basis.cc:518-603).

    coef_mode: COEF_SCALAR (a: one value per fine cell), COEF_TENSOR (6 per
    fine cell: a00 a11 a22 a01 a02 a12), COEF_GAUSS (48 per fine cell: the 6
    at each 2x2x2 Gauss point, x fastest).
    Returns dict with KH [c,8,8], FH [c,8], Phi (flat, per cell 8 planes of
    (n+1)^3 nodes) and iters [c,8]."""
    origin = np.ascontiguousarray(origin, dtype=np.float64).reshape(-1, 3)
    size = np.ascontiguousarray(size, dtype=np.float64).reshape(-1, 3)
    depth = np.ascontiguousarray(depth, dtype=np.int32).reshape(-1)
    nc = depth.shape[0]
    a = np.ascontiguousarray(a, dtype=np.float64)
    r = None if r is None else np.ascontiguousarray(r, dtype=np.float64)
    lp = np.ascontiguousarray(load_params, dtype=np.float64)
    n = (1 << depth.astype(np.int64))
    nphi = int(np.sum(8 * (n + 1) ** 3))
    Phi = np.zeros(nphi) if want_phi else None
    KH = np.zeros((nc, 8, 8))
    FH = np.zeros((nc, 8))
    iters = np.zeros((nc, 8), dtype=np.int32)
    st = lib().oracle_q1_build_coef(nc, _d(origin), _d(size), _i(depth), int(coef_mode), _d(a), _d(r),
                                    int(load_kind), _d(lp), int(solver), float(tol), int(max_iter), _d(Phi),
                                    _d(KH), _d(FH), _i(iters), int(nthreads))
    return {"status": st, "KH": KH, "FH": FH, "Phi": Phi, "iters": iters}


def q1_assemble(origin, size, depth, a, r=None, load_kind=LOAD_ZERO, load_params=(0, 0, 0, 0), coef_mode=0):
    """Unconstrained fine K (scipy CSR) and load b of one coarse cell."""
    import scipy.sparse as sp
    n = 1 << int(depth)
    nn = (n + 1) ** 3
    rows = np.zeros(27 * nn, dtype=np.int32)
    cols = np.zeros(27 * nn, dtype=np.int32)
    vals = np.zeros(27 * nn)
    b = np.zeros(nn)
    o = np.ascontiguousarray(origin, dtype=np.float64)
    s = np.ascontiguousarray(size, dtype=np.float64)
    a = np.ascontiguousarray(a, dtype=np.float64)
    r = None if r is None else np.ascontiguousarray(r, dtype=np.float64)
    lp = np.ascontiguousarray(load_params, dtype=np.float64)
    st = lib().oracle_q1_assemble_coef(_d(o), _d(s), int(depth), int(coef_mode), _d(a), _d(r), int(load_kind),
                                       _d(lp), _i(rows), _i(cols), _d(vals), _d(b))
    assert st == 0
    K = sp.coo_matrix((vals, (rows, cols)), shape=(nn, nn)).tocsr()
    return K, b


def nedelec_dof_values_unit_cube(depth, c):
    n = 1 << int(depth)
    cap = 3 * n * (n + 1) ** 2
    out = np.zeros(cap)
    cc = np.ascontiguousarray(c, dtype=np.float64)
    cnt = lib().oracle_nedelec_dof_values_unit_cube(int(depth), _d(cc), _d(out), cap)
    assert cnt == cap
    return out
