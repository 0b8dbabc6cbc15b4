"""CPU checks of the host-side coarse Q1 and Ned_RT assembly/solve (consumers
of K_H, F_H) and of the C++ shim library build."""
import ctypes
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import workloads

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def host_lib():
    import msfec_build
    msfec_build.build()
    L = ctypes.CDLL(msfec_build.HOSTLIB)
    dp = ctypes.POINTER(ctypes.c_double)
    L.msfec_host_q1_coarse_solve.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_double, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_int)]
    L.msfec_host_q1_coarse_solve.restype = ctypes.c_int
    for name in ("msfec_host_nedrt_coarse_solve", "msfec_host_nedrt_coarse_solve_essential"):
        getattr(L, name).argtypes = L.msfec_host_q1_coarse_solve.argtypes
        getattr(L, name).restype = ctypes.c_int
    return L


def coarse_solve(m, KH, FH):
    L = host_lib()
    U = np.zeros((m + 1) ** 3)
    it = ctypes.c_int(0)
    dp = ctypes.POINTER(ctypes.c_double)
    KH = np.ascontiguousarray(KH, dtype=np.float64)
    FH = np.ascontiguousarray(FH, dtype=np.float64)
    st = L.msfec_host_q1_coarse_solve(m, KH.ctypes.data_as(dp), FH.ctypes.data_as(dp), U.ctypes.data_as(dp),
                                      1e-14, 20000, ctypes.byref(it))
    assert st == 0
    return U


def scipy_coarse(m, KH, FH):
    M1 = m + 1
    rows, cols, vals = [], [], []
    b = np.zeros(M1 ** 3)
    for c in range(m ** 3):
        i, j, k = c % m, (c // m) % m, c // (m * m)
        nodes = [(i + (v & 1)) + M1 * ((j + ((v >> 1) & 1)) + M1 * (k + (v >> 2))) for v in range(8)]
        for u in range(8):
            b[nodes[u]] += FH[c, u]
            for v in range(8):
                rows.append(nodes[u]); cols.append(nodes[v]); vals.append(KH[c, u, v])
    K = sp.coo_matrix((vals, (rows, cols)), shape=(M1 ** 3, M1 ** 3)).tocsr()
    idx = np.arange(M1 ** 3)
    i, j, k = idx % M1, (idx // M1) % M1, idx // (M1 * M1)
    I = np.where((i > 0) & (j > 0) & (k > 0) & (i < m) & (j < m) & (k < m))[0]
    U = np.zeros(M1 ** 3)
    U[I] = spla.spsolve(K[I][:, I].tocsc(), b[I])
    return U


def test_coarse_solver_matches_scipy(oracle_lib):
    cells, a, r, load = workloads.q1_lognormal(m=3, depth=2, seed=21, reaction=False)
    res = oracle_lib.q1_build(cells["origin"], cells["size"], cells["depth"], a, r, load_kind=load.kind,
                              load_params=list(load.params), want_phi=False)
    U = coarse_solve(3, res["KH"], res["FH"])
    Us = scipy_coarse(3, res["KH"], res["FH"])
    assert np.abs(U - Us).max() <= 1e-11 * np.abs(Us).max()


def test_shim_library_and_example_build():
    import msfec_build
    msfec_build.build()
    assert os.path.exists(msfec_build.HOSTLIB) and os.path.exists(msfec_build.EXAMPLE)
    for ex in (msfec_build.EXAMPLE_NR, msfec_build.EXAMPLE_PAIR, msfec_build.EXAMPLE_STD):
        assert os.path.exists(ex), ex
    L = ctypes.CDLL(msfec_build.HOSTLIB)
    assert hasattr(L, "msfec_host_q1_coarse_solve") and hasattr(L, "msfec_host_nedrt_coarse_solve")


def nedrt_coarse_solve(m, KH, FH, rtol=1e-13, essential=False):
    """Host coarse Ned_RT solve: natural conditions (the reference's
    NedRTMultiscale) by default, or boundary DoFs fixed at 0."""
    L = host_lib()
    from oracle import nedrt_oracle as N
    NE, NF = N.counts(m)
    U = np.zeros(NE + NF)
    it = ctypes.c_int(0)
    dp = ctypes.POINTER(ctypes.c_double)
    KH = np.ascontiguousarray(KH, dtype=np.float64)
    FH = np.ascontiguousarray(FH, dtype=np.float64)
    f = L.msfec_host_nedrt_coarse_solve_essential if essential else L.msfec_host_nedrt_coarse_solve
    st = f(m, KH.ctypes.data_as(dp), FH.ctypes.data_as(dp), U.ctypes.data_as(dp), rtol, 50000, ctypes.byref(it))
    assert st == 0, (st, it.value)
    return U


def scipy_nedrt_coarse(m, KH, FH, essential=False):
    """Independent assembly (global maps of the oracle) and sparse direct solve."""
    from oracle import nedrt_adjoint as NA
    g, bnd = NA.coarse_maps(m)
    if not essential:
        bnd = np.zeros_like(bnd)
    n = bnd.size
    K = sp.coo_matrix((np.asarray(KH).ravel(), (np.repeat(g, 18, axis=1).ravel(), np.tile(g, (1, 18)).ravel())),
                      shape=(n, n)).tocsr()
    F = np.zeros(n)
    np.add.at(F, g.ravel(), np.asarray(FH).ravel())
    I = np.where(~bnd)[0]
    U = np.zeros(n)
    U[I] = spla.spsolve(K[I][:, I].tocsc(), F[I])
    return U


@pytest.mark.parametrize("essential", [False, True])
@pytest.mark.parametrize("m", [2, 3])
def test_nedrt_coarse_solver_matches_scipy(m, essential):
    from oracle import nedrt_adjoint as NA
    from oracle import nedrt_oracle as N
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=m, depth=1, seed=8)
    res = N.build(cells, N.sym6_to_ainv(ainv6), bdiv, load.kind, list(load.params), want_phi=False)
    rng = np.random.default_rng(m)
    # the trig load of the workload and a generic face load on top of it
    for FH in (res["FH"], res["FH"] + np.concatenate([np.zeros((m ** 3, 12)), rng.standard_normal((m ** 3, 6))], 1)):
        U = nedrt_coarse_solve(m, res["KH"], FH, essential=essential)
        Us = scipy_nedrt_coarse(m, res["KH"], FH, essential=essential)
        assert np.abs(U - Us).max() <= 1e-10 * np.abs(Us).max()
        if not essential:  # natural conditions: the boundary DoFs carry the solution too
            _, bnd = NA.coarse_maps(m)
            assert np.abs(Us[bnd]).max() > 1e-3 * np.abs(Us).max()


def test_q1_multiscale_converges_to_analytic_solution(oracle_lib):
    """Known answer for the Q1 multiscale pipeline (oracle basis, 8x8
    Galerkin, host coarse solve): constant a = 0.8 and the sin-product load
    have the exact solution u = f / (3 a pi^2); the coarse nodal values
    converge at O(H^2) (measured 47.8 %, 10.8 %, 2.6 % for coarse 2^3, 4^3, 8^3
    at depth 2)."""
    a0, depth = 0.8, 2
    err = []
    for m in (2, 4, 8):
        cells = workloads.coarse_grid(m, depth)
        nf = len(cells) * (1 << depth) ** 3
        res = oracle_lib.q1_build(cells["origin"], cells["size"], cells["depth"], np.full(nf, a0), None,
                                  load_kind=oracle_lib.LOAD_SIN_PRODUCT, load_params=[1.0, 1.0, 0.0, 0.0],
                                  want_phi=False)
        U = coarse_solve(m, res["KH"], res["FH"])
        M1 = m + 1
        idx = np.arange(M1 ** 3)
        i, j, k = idx % M1, (idx // M1) % M1, idx // (M1 * M1)
        ue = np.sin(np.pi * i / m) * np.sin(np.pi * j / m) * np.sin(np.pi * k / m) / (3 * a0 * np.pi ** 2)
        err.append(np.abs(U - ue).max() / np.abs(ue).max())
    assert err[-1] < 0.03 and err[0] / err[1] > 3.5 and err[1] / err[2] > 3.5, err
