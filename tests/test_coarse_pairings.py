"""CPU checks of the host-side coarse Q_Ned and RT_DQ assembly/solve
(mpi-msfec_gb300/host/coarse_pairings.cpp), the consumers of the 20x20 and
7x7 element matrices: element matrices from the FP64 oracles on a 2^3 coarse
grid, solved by the host MINRES and by an independent scipy assembly (global
maps restated below) with a sparse direct solve."""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import workloads
from oracle import nedrt_oracle as NR
from oracle import qned_oracle as Q
from oracle import rtdq_oracle as RQ

LINES = [(1, 0, 0), (1, 1, 0), (0, 0, 0), (0, 1, 0), (1, 0, 1), (1, 1, 1), (0, 0, 1), (0, 1, 1),
         (2, 0, 0), (2, 1, 0), (2, 0, 1), (2, 1, 1)]  # GeometryInfo<3> lines: direction, two positions


def host_lib():
    import msfec_build
    msfec_build.build()
    L = ctypes.CDLL(msfec_build.HOSTLIB)
    dp = ctypes.POINTER(ctypes.c_double)
    for name in ("msfec_host_qned_coarse_solve", "msfec_host_rtdq_coarse_solve"):
        f = getattr(L, name)
        f.argtypes = [ctypes.c_int, dp, dp, dp, ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        f.restype = ctypes.c_int
    for name in ("msfec_host_qned_cell_dofs", "msfec_host_rtdq_cell_dofs"):
        f = getattr(L, name)
        f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        f.restype = ctypes.c_int
    return L


def qned_maps(m):
    N1 = m + 1
    NV, Ex = N1 ** 3, m * N1 * N1
    g = np.zeros((m ** 3, 20), dtype=np.int64)
    for c in range(m ** 3):
        i, j, k = c % m, (c // m) % m, c // (m * m)
        for v in range(8):
            g[c, v] = (i + (v & 1)) + N1 * ((j + ((v >> 1) & 1)) + N1 * (k + (v >> 2)))
        for l, (d, p, q) in enumerate(LINES):
            if d == 0:
                g[c, 8 + l] = NV + i + m * ((j + p) + N1 * (k + q))
            elif d == 1:
                g[c, 8 + l] = NV + Ex + (i + p) + N1 * (j + m * (k + q))
            else:
                g[c, 8 + l] = NV + 2 * Ex + (i + p) + N1 * ((j + q) + N1 * k)
    fixed = np.zeros(NV + 3 * Ex, dtype=bool)
    t = np.arange(NV)
    vi, vj, vk = t % N1, (t // N1) % N1, t // (N1 * N1)
    fixed[:NV] = (vi == 0) | (vi == m) | (vj == 0) | (vj == m) | (vk == 0) | (vk == m)
    fixed[NV:] = NR.boundary_mask(m)[:3 * Ex]
    return g, fixed


def rtdq_maps(m):
    Fx, NF = (m + 1) * m * m, 3 * (m + 1) * m * m
    g = np.zeros((m ** 3, 7), dtype=np.int64)
    for c in range(m ** 3):
        i, j, k = c % m, (c // m) % m, c // (m * m)
        g[c] = [i + (m + 1) * (j + m * k), i + 1 + (m + 1) * (j + m * k), Fx + i + m * (j + (m + 1) * k),
                Fx + i + m * (j + 1 + (m + 1) * k), 2 * Fx + i + m * (j + m * k), 2 * Fx + i + m * (j + m * (k + 1)),
                NF + c]
    return g, np.zeros(NF + m ** 3, dtype=bool)


def scipy_solve(g, fixed, KH, FH):
    nb = g.shape[1]
    n = fixed.size
    K = sp.coo_matrix((np.asarray(KH).ravel(), (np.repeat(g, nb, axis=1).ravel(), np.tile(g, (1, nb)).ravel())),
                      shape=(n, n)).tocsr()
    F = np.zeros(n)
    np.add.at(F, g.ravel(), np.asarray(FH).ravel())
    I = np.where(~fixed)[0]
    U = np.zeros(n)
    U[I] = spla.spsolve(K[I][:, I].tocsc(), F[I])
    return U


def host_solve(name, n, KH, FH, m):
    L = host_lib()
    dp = ctypes.POINTER(ctypes.c_double)
    U = np.zeros(n)
    it = ctypes.c_int(0)
    KH = np.ascontiguousarray(KH, dtype=np.float64)
    FH = np.ascontiguousarray(FH, dtype=np.float64)
    st = getattr(L, name)(m, KH.ctypes.data_as(dp), FH.ctypes.data_as(dp), U.ctypes.data_as(dp), 1e-12, 50000,
                          ctypes.byref(it))
    assert st == 0, (st, it.value)
    return U


def check_maps(name, g):
    L = host_lib()
    out = (ctypes.c_int * g.shape[1])()
    for c in range(g.shape[0]):
        assert getattr(L, name)(round(g.shape[0] ** (1 / 3)), c, out) == 0
        assert list(out) == list(g[c])


@pytest.mark.parametrize("depth", [1, 2])
def test_qned_coarse_solver_matches_scipy(depth):
    m = 2
    cells, a6, binv, load = workloads.qned_tensor(m=m, depth=depth, seed=12)
    res = Q.build(cells, binv, NR.sym6_to_ainv(a6), load.kind, list(load.params), want_phi=False)
    g, fixed = qned_maps(m)
    check_maps("msfec_host_qned_cell_dofs", g)
    rng = np.random.default_rng(depth)
    for FH in (res["FH"], res["FH"] + np.concatenate([np.zeros((m ** 3, 8)), rng.standard_normal((m ** 3, 12))], 1)):
        U = host_solve("msfec_host_qned_coarse_solve", fixed.size, res["KH"], FH, m)
        Us = scipy_solve(g, fixed, res["KH"], FH)
        assert np.abs(Us).max() > 0
        assert np.abs(U - Us).max() <= 1e-9 * np.abs(Us).max()


@pytest.mark.parametrize("depth", [1, 2])
def test_rtdq_coarse_solver_matches_scipy(depth):
    m = 2
    cells, ainv6, load = workloads.rtdq_tensor(m=m, depth=depth, seed=13)
    res = RQ.build(cells, NR.sym6_to_ainv(ainv6), load.kind, list(load.params), want_phi=False)
    g, fixed = rtdq_maps(m)
    check_maps("msfec_host_rtdq_cell_dofs", g)
    rng = np.random.default_rng(depth)
    for FH in (res["FH"], res["FH"] + np.concatenate([np.zeros((m ** 3, 6)), rng.standard_normal((m ** 3, 1))], 1)):
        U = host_solve("msfec_host_rtdq_coarse_solve", fixed.size, res["KH"], FH, m)
        Us = scipy_solve(g, fixed, res["KH"], FH)
        assert np.abs(Us).max() > 0
        assert np.abs(U - Us).max() <= 1e-9 * np.abs(Us).max()
