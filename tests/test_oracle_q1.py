"""CPU checks of the FP64 oracle (Q1 pairing) against known answers.

The reference (deal.II/Trilinos) cannot be built here; the oracle is pinned by
mathematical known-answer tests, an independent numpy/scipy restatement and
the committed seeded fixtures.
"""
import os

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import workloads

HERE = os.path.dirname(os.path.abspath(__file__))


def trilinear_planes(n):
    t = np.arange(n + 1) / n
    z, y, x = np.meshgrid(t, t, t, indexing="ij")
    out = []
    for v in range(8):
        f = np.ones_like(x)
        for d, T in enumerate((x, y, z)):
            f = f * (T if (v >> d) & 1 else 1 - T)
        out.append(f.ravel())
    return np.array(out)


def q1_element(h):
    """Q1 element stiffness (unit coefficient) and mass on a box, by tensor products."""
    K = np.zeros((8, 8))
    M = np.zeros((8, 8))
    k1 = [np.array([[1, -1], [-1, 1]]) / hd for hd in h]
    m1 = [hd * np.array([[1 / 3, 1 / 6], [1 / 6, 1 / 3]]) for hd in h]
    for u in range(8):
        for v in range(8):
            a = [(u >> d) & 1 for d in range(3)]
            b = [(v >> d) & 1 for d in range(3)]
            K[u, v] = (k1[0][a[0], b[0]] * m1[1][a[1], b[1]] * m1[2][a[2], b[2]]
                       + m1[0][a[0], b[0]] * k1[1][a[1], b[1]] * m1[2][a[2], b[2]]
                       + m1[0][a[0], b[0]] * m1[1][a[1], b[1]] * k1[2][a[2], b[2]])
            M[u, v] = m1[0][a[0], b[0]] * m1[1][a[1], b[1]] * m1[2][a[2], b[2]]
    return K, M


def numpy_assemble(n, size, a, r):
    """Independent sparse assembly of the fine Q1 matrix (numpy/scipy)."""
    h = np.asarray(size) / n
    K, M = q1_element(h)
    N1 = n + 1
    e = np.arange(n ** 3)
    i, j, k = e % n, (e // n) % n, e // (n * n)
    rows, cols, vals = [], [], []
    for u in range(8):
        nu = (i + (u & 1)) + N1 * ((j + ((u >> 1) & 1)) + N1 * (k + (u >> 2)))
        for v in range(8):
            nv = (i + (v & 1)) + N1 * ((j + ((v >> 1) & 1)) + N1 * (k + (v >> 2)))
            rows.append(nu)
            cols.append(nv)
            vals.append(a * K[u, v] + (r * M[u, v] if r is not None else 0.0))
    return sp.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                         shape=(N1 ** 3, N1 ** 3)).tocsr()


def boundary_mask(n):
    N1 = n + 1
    idx = np.arange(N1 ** 3)
    i, j, k = idx % N1, (idx // N1) % N1, idx // (N1 * N1)
    return (i == 0) | (j == 0) | (k == 0) | (i == n) | (j == n) | (k == n)


def test_constant_coefficient_gives_trilinear_basis(oracle_lib):
    # KAT: for constant A the trilinear coarse functions are A-harmonic and lie
    # in the fine Q1 space, so the basis is their interpolant and K_H is the
    # coarse Q1 element stiffness.
    for L in (1, 2, 3):
        n = 1 << L
        H = [0.25, 0.5, 0.125]
        res = oracle_lib.q1_build([0, 0, 0], H, [L], np.full(n ** 3, 2.5))
        assert res["status"] == 0
        Phi = res["Phi"].reshape(8, -1)
        assert np.abs(Phi - trilinear_planes(n)).max() < 1e-13
        Kc, _ = q1_element(H)
        assert np.allclose(res["KH"][0], 2.5 * Kc, rtol=1e-12, atol=1e-14)


def test_partition_of_unity_and_symmetry(oracle_lib):
    rng = np.random.default_rng(11)
    L = 3
    n = 1 << L
    a = np.exp(rng.standard_normal(n ** 3))
    res = oracle_lib.q1_build([0.5, 0, 0.25], [0.25] * 3, [L], a)
    KH = res["KH"][0]
    Phi = res["Phi"].reshape(8, -1)
    assert np.abs(Phi.sum(axis=0) - 1).max() < 1e-12  # sum_v phi_v == 1 (R = 0)
    assert np.abs(KH.sum(axis=1)).max() < 1e-12 * np.abs(KH).max()
    assert np.allclose(KH, KH.T, rtol=0, atol=1e-14 * np.abs(KH).max())
    assert np.linalg.eigvalsh(KH).min() > -1e-12 * np.abs(KH).max()


def test_oracle_matches_independent_scipy_solve(oracle_lib):
    rng = np.random.default_rng(5)
    for L, react in ((2, True), (3, False)):
        n = 1 << L
        size = [0.25, 0.25, 0.25]
        a = np.exp(rng.standard_normal(n ** 3))
        r = np.ones(n ** 3) if react else None
        res = oracle_lib.q1_build([0, 0, 0], size, [L], a, r, load_kind=2, load_params=[1, 1, 0, 0])
        K = numpy_assemble(n, size, a, r)
        Ko, bo = oracle_lib.q1_assemble([0, 0, 0], size, L, a, r, 2, [1, 1, 0, 0])
        assert abs(K - Ko).max() < 1e-15 * abs(K).max() * 10
        bnd = boundary_mask(n)
        I, B = np.where(~bnd)[0], np.where(bnd)[0]
        G = trilinear_planes(n)
        Phi = np.zeros_like(G)
        for v in range(8):
            Phi[v, B] = G[v, B]
            Phi[v, I] = spla.spsolve(K[I][:, I].tocsc(), -K[I][:, B] @ G[v, B])
        assert np.abs(Phi - res["Phi"].reshape(8, -1)).max() < 1e-12
        KH = Phi @ (K @ Phi.T)
        assert np.allclose(res["KH"][0], KH, rtol=1e-11, atol=1e-15)
        assert np.allclose(res["FH"][0], Phi @ bo, rtol=1e-11, atol=1e-16)


def test_reference_iterative_mode_agrees_with_direct(oracle_lib):
    cells, a, r, load = workloads.q1_lognormal(m=2, depth=3, seed=2, reaction=True)
    kw = dict(load_kind=load.kind, load_params=list(load.params))
    d = oracle_lib.q1_build(cells["origin"], cells["size"], cells["depth"], a, r, **kw)
    it = oracle_lib.q1_build(cells["origin"], cells["size"], cells["depth"], a, r,
                             solver=oracle_lib.SOLVER_CG_SSOR, tol=1e-12, max_iter=1000, **kw)
    assert it["status"] == 0
    assert (it["iters"] > 0).all() and (it["iters"] < 1000).all()
    assert np.abs(d["KH"] - it["KH"]).max() < 1e-9 * np.abs(d["KH"]).max()


def test_committed_q1_fixtures_reproduce(oracle_lib):
    g = np.load(os.path.join(HERE, "golden", "q1_lognormal_m4_L3_seed1.npz"))
    cells, a, r, load = workloads.q1_lognormal(m=4, depth=3, seed=1, reaction=True)
    res = oracle_lib.q1_build(cells["origin"], cells["size"], cells["depth"], a, r,
                              load_kind=load.kind, load_params=list(load.params), want_phi=False)
    assert np.abs(res["KH"] - g["KH"]).max() <= 1e-13 * np.abs(g["KH"]).max()
    assert np.abs(res["FH"] - g["FH"]).max() <= 1e-13 * np.abs(g["FH"]).max()


def test_invalid_depth_rejected(oracle_lib):
    res = oracle_lib.q1_build([0, 0, 0], [1, 1, 1], [0], np.ones(1))
    assert res["status"] != 0


def test_fine_problem_converges_to_analytic_solution(oracle_lib):
    """Known answer for the standard fine-scale Q1 problem (the system the fine
    solve and the local problems discretise): constant a and r with the
    sin-product load f = sin(pi x) sin(pi y) sin(pi z) have the exact solution
    u = f / (3 a pi^2 + r), which vanishes on the boundary (homogeneous
    Dirichlet data). The nodal error falls at O(h^2) (measured: 11.3 %, 2.7 %,
    0.67 % at depths 2-4)."""
    a0, r0 = 0.8, 2.0
    err = []
    for depth in (2, 3, 4):
        n = 1 << depth
        nf = n ** 3
        K, b = oracle_lib.q1_assemble(np.zeros(3), np.ones(3), depth, np.full(nf, a0), np.full(nf, r0),
                                      oracle_lib.LOAD_SIN_PRODUCT, [1.0, 1.0, 0.0, 0.0])
        K = K.tocsr()
        N1 = n + 1
        idx = np.arange(N1 ** 3)
        i, j, k = idx % N1, (idx // N1) % N1, idx // (N1 * N1)
        I = np.where((i > 0) & (j > 0) & (k > 0) & (i < n) & (j < n) & (k < n))[0]
        u = np.zeros(N1 ** 3)
        u[I] = spla.spsolve(K[I][:, I].tocsc(), b[I])
        ue = np.sin(np.pi * i / n) * np.sin(np.pi * j / n) * np.sin(np.pi * k / n) / (3 * a0 * np.pi ** 2 + r0)
        err.append(np.abs(u - ue).max() / np.abs(ue).max())
    assert err[-1] < 2e-2, err
    assert err[0] / err[1] > 3.5 and err[1] / err[2] > 3.5, err
