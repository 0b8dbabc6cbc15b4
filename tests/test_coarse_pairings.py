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


def _sin_int(s0, s1):
    """Integral of sin(pi s) over [s0, s1]."""
    return (np.cos(np.pi * s0) - np.cos(np.pi * s1)) / np.pi


def rtdq_exact(m, a):
    """Known answer of the RT_DQ problem (A^-1 sigma + grad u = 0, div sigma = f,
    u = 0 on the boundary through the natural condition) with A = a I and
    f = sin(pi x) sin(pi y) sin(pi z): u = f / (3 a pi^2), sigma = -a grad u.
    Returns the coarse face fluxes (+axis) and the coarse cell means of u."""
    H = 1.0 / m
    Fx = (m + 1) * m * m
    t = np.arange(Fx)
    fl = np.zeros(3 * Fx)
    i, j, k = t % (m + 1), (t // (m + 1)) % m, t // ((m + 1) * m)
    fl[:Fx] = -np.cos(np.pi * i * H) * _sin_int(j * H, j * H + H) * _sin_int(k * H, k * H + H) / (3 * np.pi)
    i, j, k = t % m, (t // m) % (m + 1), t // (m * (m + 1))
    fl[Fx:2 * Fx] = -np.cos(np.pi * j * H) * _sin_int(i * H, i * H + H) * _sin_int(k * H, k * H + H) / (3 * np.pi)
    i, j, k = t % m, (t // m) % m, t // (m * m)
    fl[2 * Fx:] = -np.cos(np.pi * k * H) * _sin_int(i * H, i * H + H) * _sin_int(j * H, j * H + H) / (3 * np.pi)
    c = np.arange(m ** 3)
    ci, cj, ck = c % m, (c // m) % m, c // (m * m)
    um = (_sin_int(ci * H, ci * H + H) * _sin_int(cj * H, cj * H + H) * _sin_int(ck * H, ck * H + H) / H ** 3
          / (3 * a * np.pi ** 2))
    return fl, um


def qned_exact_edges(m, a):
    """Known answer of the Q_Ned problem (B^-1 sigma + div u = 0,
    grad sigma + curl(A curl u) = f, sigma = 0 and u x n = 0 on the boundary)
    with A = a I and the divergence-free vector trig load (w = pi):
    u = f / (2 a w^2), sigma = 0. Returns the line integrals of u along the
    coarse edges (x-, y-, z-edges in the coarse numbering)."""
    w, H, N1 = np.pi, 1.0 / m, m + 1
    Ex = m * N1 * N1
    t = np.arange(Ex)
    out = np.zeros(3 * Ex)
    i, j, k = t % m, (t // m) % N1, t // (m * N1)
    out[:Ex] = np.sin(w * j * H) * np.sin(w * k * H)
    i, j, k = t % N1, (t // N1) % m, t // (N1 * m)
    out[Ex:2 * Ex] = np.sin(w * k * H) * np.sin(w * i * H)
    i, j, k = t % N1, (t // N1) % N1, t // (N1 * N1)
    out[2 * Ex:] = np.sin(w * i * H) * np.sin(w * j * H)
    return out * H / (2 * a * w * w)


def test_rtdq_multiscale_converges_to_analytic_solution():
    """Oracle multiscale RT_DQ (local solves, 7x7 Galerkin, coarse solve):
    coarse cell values converge to the exact cell means at O(H^2) (measured
    17.8 %, 5.0 % for coarse 2^3, 4^3 at depth 2); the coarse face fluxes equal
    the exact fluxes up to the fine-scale quadrature of f (1.7e-5, 1.0e-6)."""
    a, depth = 0.8, 2
    n = 1 << depth
    err = []
    for m in (2, 4):
        cells = workloads.coarse_grid(m, depth)
        nfc = len(cells) * n ** 3
        res = RQ.build(cells, np.tile(np.eye(3) / a, (nfc, 1, 1)), RQ.LOAD_SIN_PRODUCT, [1.0, 1.0, 0.0, 0.0],
                       want_phi=False)
        g, fixed = rtdq_maps(m)
        U = scipy_solve(g, fixed, res["KH"], res["FH"])
        fl, um = rtdq_exact(m, a)
        NF = fl.size
        err.append((np.linalg.norm(U[NF:] - um) / np.linalg.norm(um), np.linalg.norm(U[:NF] - fl) / np.linalg.norm(fl)))
    (u2, f2), (u4, f4) = err
    assert u2 < 0.2 and u4 < 0.06 and u2 / u4 > 3.0, err
    assert f2 < 1e-4 and f4 < 1e-5, err


def test_qned_multiscale_converges_to_analytic_solution():
    """Oracle multiscale Q_Ned (local solves, 20x20 Galerkin, coarse solve with
    the reference's Dirichlet conditions): coarse edge DoFs converge to the
    exact line integrals of u at O(H^2) (measured 21.6 %, 5.2 % for coarse 2^3,
    4^3 at depth 2) and the vertex (sigma) DoFs vanish to rounding (sigma = 0)."""
    a, depth = 0.8, 2
    n = 1 << depth
    err = []
    for m in (2, 4):
        cells = workloads.coarse_grid(m, depth)
        nfc = len(cells) * n ** 3
        res = Q.build(cells, np.full(nfc, 1.7), np.tile(np.eye(3) * a, (nfc, 1, 1)), Q.LOAD_VEC_TRIG,
                      [1.0, 1.0, 0.0, 0.0], want_phi=False)
        g, fixed = qned_maps(m)
        U = scipy_solve(g, fixed, res["KH"], res["FH"])
        ue = qned_exact_edges(m, a)
        NV = (m + 1) ** 3
        assert np.abs(U[:NV]).max() <= 1e-12 * np.abs(ue).max()
        err.append(np.linalg.norm(U[NV:] - ue) / np.linalg.norm(ue))
    assert err[0] < 0.25 and err[1] < 0.06 and err[0] / err[1] > 3.0, err
