"""CPU checks of the Ned_RT FP64 oracle and of the closed-form element tables
the CUDA kernel uses (restated here in Python from the kernel's formulas)."""
import os

import numpy as np

from oracle import nedrt_oracle as N
import workloads

HERE = os.path.dirname(os.path.abspath(__file__))


def _m1(a, b):
    return 1.0 / 3.0 if a == b else 1.0 / 6.0


def _sgn(a):
    return 1.0 if a else -1.0


def _other(p):
    return (1 if p == 0 else 0), (1 if p == 2 else 2)


def _edge_pos(p, l4, ax):
    o1, o2 = _other(p)
    return (l4 & 1) if ax == o1 else (l4 >> 1)


def kernel_table_G(h, p, q, l4, m4):
    """Same closed form as table_G in csrc/nedrt_solve.cu."""
    if p == q:
        o1, o2 = _other(p)
        return h[o1] * h[o2] / h[p] * _m1(l4 & 1, m4 & 1) * _m1(l4 >> 1, m4 >> 1)
    r = 3 - p - q
    return 0.25 * h[r] * _m1(_edge_pos(p, l4, r), _edge_pos(q, m4, r))


def kernel_table_C(h, l, f):
    """Same closed form as table_C in csrc/nedrt_solve.cu."""
    p, l4 = l >> 2, l & 3
    fd, fa = f >> 1, f & 1
    if fd == p:
        return 0.0
    hx, hy, hz = h
    a0, a1 = l4 & 1, l4 >> 1
    if p == 0:
        return _sgn(a1) * hy * _m1(a0, fa) / (hx * hz) if fd == 1 else -_sgn(a0) * hz * _m1(a1, fa) / (hx * hy)
    if p == 1:
        return -_sgn(a1) * hx * _m1(a0, fa) / (hy * hz) if fd == 0 else _sgn(a0) * hz * _m1(a1, fa) / (hx * hy)
    return _sgn(a1) * hx * _m1(a0, fa) / (hy * hz) if fd == 0 else -_sgn(a0) * hy * _m1(a1, fa) / (hx * hz)


def test_kernel_closed_form_tables_match_quadrature():
    h = np.array([0.3, 0.17, 0.55])
    for p in range(3):
        for q in range(3):
            ainv = np.zeros((1, 3, 3))
            ainv[0, p, q] = ainv[0, q, p] = 1.0
            Me, Ce, _ = N.element_matrices(h, ainv, np.ones(1))
            G = np.array([[kernel_table_G(h, p, q, l4, m4) for m4 in range(4)] for l4 in range(4)])
            blk = Me[0][4 * p:4 * p + 4, 4 * q:4 * q + 4]
            assert np.allclose(blk, G, rtol=1e-13, atol=1e-15), (p, q)
    C = np.array([[kernel_table_C(h, l, f) for f in range(6)] for l in range(12)])
    assert np.allclose(Ce, C, rtol=1e-13, atol=1e-14)


def kernel_edge_mass_form(h, ai, x, y):
    """Same factored form as edge_mass_form in csrc/nedrt_solve.cu (the A part of
    the adjoint gradient): x^T M_e y without the 12 x 12 table."""
    A = np.array([[ai[0], ai[3], ai[4]], [ai[3], ai[1], ai[5]], [ai[4], ai[5], ai[2]]])
    my = np.zeros(12)
    for p in range(3):
        o1, o2 = _other(p)
        k = A[p, p] * h[o1] * h[o2] / (36.0 * h[p])
        t = [2.0 * y[4 * p + l] + y[4 * p + (l ^ 1)] for l in range(4)]
        for l in range(4):
            my[4 * p + l] = k * (2.0 * t[l] + t[l ^ 2])
    for p in range(3):
        for q in range(3):
            if q == p:
                continue
            r = 3 - p - q
            s1 = sum(y[4 * q + m] for m in range(4) if _edge_pos(q, m, r))
            s0 = sum(y[4 * q + m] for m in range(4) if not _edge_pos(q, m, r))
            k = A[p, q] * h[r] / 24.0
            for l in range(4):
                my[4 * p + l] += k * (s0 + 2.0 * s1 if _edge_pos(p, l, r) else 2.0 * s0 + s1)
    return float(np.dot(x, my))


def test_kernel_edge_mass_form_matches_quadrature():
    rng = np.random.default_rng(4)
    for _ in range(5):
        h = rng.uniform(0.05, 0.6, 3)
        G = rng.standard_normal((3, 3))
        ainv = G @ G.T + 0.5 * np.eye(3)
        ai = [ainv[0, 0], ainv[1, 1], ainv[2, 2], ainv[0, 1], ainv[0, 2], ainv[1, 2]]
        Me, _, _ = N.element_matrices(h, ainv[None], np.ones(1))
        x, y = rng.standard_normal(12), rng.standard_normal(12)
        ref = x @ Me[0] @ y
        scale = np.abs(x) @ np.abs(Me[0]) @ np.abs(y)
        assert abs(kernel_edge_mass_form(h, ai, x, y) - ref) <= 1e-13 * scale


def test_standard_basis_galerkin_is_refinement_invariant():
    # The reference's set_to_std sanity path (ned_rt_basis.cc:1312-1335): with
    # constant coefficients the coarse functions' Galerkin matrix does not
    # depend on the local refinement.
    H = [0.25, 0.5, 0.125]
    ref = None
    for L in (0, 1, 2):
        n = 1 << L
        ainv = np.tile(np.array([[2.0, 0.3, 0.1], [0.3, 1.0, -0.2], [0.1, -0.2, 1.5]]), (n ** 3, 1, 1))
        _, KH, _ = N.build_cell([0, 0, 0], H, L, ainv, np.full(n ** 3, 0.7), basis="std")
        if ref is None:
            ref = KH
        assert np.abs(KH - ref).max() <= 1e-12 * np.abs(ref).max()


def test_solution_satisfies_the_saddle_point_system():
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=1, depth=2, seed=5)
    n = 4
    ainv = N.sym6_to_ainv(ainv6)
    Phi, KH, FH = N.build_cell(cells["origin"][0], cells["size"][0], 2, ainv, bdiv, load.kind,
                               list(load.params))
    A = N.assemble(n, cells["size"][0], ainv, bdiv)
    bnd = N.boundary_mask(n)
    NE, NF = N.counts(n)
    for b in range(18):
        f = np.zeros(NE + NF)
        if b < 12:
            f[NE:] = N.coarse_curl_rhs(n, cells["size"][0], b)
            g = N.coarse_edge_dofs(n, b)
            assert np.array_equal(Phi[b][:NE][bnd[:NE]], g[bnd[:NE]])
        r = f - A @ Phi[b]
        assert np.abs(r[~bnd]).max() <= 1e-10 * max(np.abs(A @ Phi[b]).max(), 1e-300)
    # block structure of K_H: K_ef = -K_fe^T, ee and ff symmetric
    assert np.abs(KH[:12, 12:] + KH[12:, :12].T).max() <= 1e-12 * np.abs(KH).max()
    assert np.abs(KH[:12, :12] - KH[:12, :12].T).max() <= 1e-12 * np.abs(KH).max()
    assert np.all(FH[:12] == 0.0)


def test_committed_nedrt_fixture_reproduces():
    g = np.load(os.path.join(HERE, "golden", "nedrt_tensor_m2_L2_seed2.npz"))
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=2, depth=2, seed=2)
    res = N.build(cells, N.sym6_to_ainv(ainv6), bdiv, load.kind, list(load.params), want_phi=False)
    assert np.abs(res["KH"] - g["KH"]).max() <= 1e-9 * np.abs(g["KH"]).max()
    assert np.abs(res["FH"] - g["FH"]).max() <= 1e-9 * np.abs(g["FH"]).max()


def _edge_index(n, d, i, j, k):
    Ex = n * (n + 1) ** 2
    return [i + n * (j + (n + 1) * k), Ex + i + (n + 1) * (j + n * k),
            2 * Ex + i + (n + 1) * (j + (n + 1) * k)][d]


def _face_index(n, d, i, j, k):
    Fx = (n + 1) * n * n
    return [i + (n + 1) * (j + n * k), Fx + i + n * (j + (n + 1) * k), 2 * Fx + i + n * (j + n * k)][d]


def cyclic_image(n):
    """DoF map of the rotation (x, y, z) -> (z, x, y) of the unit cube: the DoF
    of direction d at lattice position (i, j, k) goes to direction d+1 at
    (k, i, j) (tangential line integrals and normal fluxes keep their sign)."""
    NE, NF = N.counts(n)
    img = np.zeros(NE + NF, dtype=np.int64)
    off = 0
    for d, i, j, k in N.edge_geometry(n):
        img[off:off + len(i)] = _edge_index(n, (d + 1) % 3, k, i, j)
        off += len(i)
    for d, i, j, k in N.face_geometry(n):
        img[off:off + len(i)] = NE + _face_index(n, (d + 1) % 3, k, i, j)
        off += len(i)
    return img


def test_standard_solve_natural_boundary():
    """NedRTStd restatement: every DoF free (no Dirichlet rows), residual of the
    full system at rounding, the boundary fluxes and tangential fields nonzero."""
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=1, depth=2, seed=5)
    c = cells[0]
    x = N.standard_solve(c["origin"], c["size"], 2, N.sym6_to_ainv(ainv6), bdiv, load.kind, list(load.params))
    n = 4
    NE, NF = N.counts(n)
    A = N.assemble(n, c["size"], N.sym6_to_ainv(ainv6), bdiv)
    rhs = np.zeros(NE + NF)
    rhs[NE:] = N.face_load(n, c["origin"], c["size"], load.kind, list(load.params))
    assert np.linalg.norm(A @ x - rhs) <= 1e-12 * np.linalg.norm(rhs)
    bnd = N.boundary_mask(n)
    assert np.abs(x[bnd]).max() > 1e-3 * np.abs(x).max()


def test_standard_solve_cyclic_symmetry():
    """Isotropic constant coefficients and the cyclic vector trig load on the unit
    cube: the solution is invariant under the rotation (x, y, z) -> (z, x, y)."""
    depth, n = 3, 8
    ainv = np.tile(np.eye(3) * 0.7, (n ** 3, 1, 1))
    bdiv = np.full(n ** 3, 1.3)
    x = N.standard_solve(np.zeros(3), np.ones(3), depth, ainv, bdiv, N.LOAD_VEC_TRIG, [1.0, 1.0, 0.0, 0.0])
    img = cyclic_image(n)
    y = np.empty_like(x)
    y[img] = x
    assert np.abs(x).max() > 0
    assert np.abs(y - x).max() <= 1e-10 * np.abs(x).max()


def _global_fine_field(m, n, cells_vec):
    """Scatter per-coarse-cell fine vectors (edges, faces of an n^3 lattice) into
    the global (m n)^3 lattice; shared interface DoFs agree (conforming basis)."""
    D = m * n
    GE, GF = N.counts(D)
    x = np.zeros(GE + GF)
    for c in range(m ** 3):
        ci, cj, ck = c % m, (c // m) % m, c // (m * m)
        sig, u = cells_vec(c)
        off = 0
        for d, a, b, q in N.edge_geometry(n):
            x[_edge_index(D, d, ci * n + a, cj * n + b, ck * n + q)] = sig[off:off + len(a)]
            off += len(a)
        off = 0
        for d, a, b, q in N.face_geometry(n):
            x[GE + _face_index(D, d, ci * n + a, cj * n + b, ck * n + q)] = u[off:off + len(a)]
            off += len(a)
    return x


def _multiscale_vs_standard(m, depth, seed):
    from oracle import nedrt_adjoint as NA
    from test_coarse_solve import scipy_nedrt_coarse
    n = 1 << depth
    D = m * n
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=m, depth=depth, seed=seed)
    ainv = N.sym6_to_ainv(ainv6)
    ref = N.build(cells, ainv, bdiv, load.kind, list(load.params))
    U = scipy_nedrt_coarse(m, ref["KH"], ref["FH"])  # natural conditions, as NedRTMultiscale
    g, _ = NA.coarse_maps(m)
    NE, _ = N.counts(n)
    Phi = np.array(ref["Phi"])
    # set_global_weights: sigma from the edge bases' sigma blocks, u from the face bases' u blocks
    x = _global_fine_field(m, n, lambda c: (U[g[c, :12]] @ Phi[c, :12, :NE], U[g[c, 12:]] @ Phi[c, 12:, NE:]))
    nf = n ** 3
    ga, gb = np.zeros((D ** 3, 3, 3)), np.zeros(D ** 3)
    t = np.arange(nf)
    i, j, k = t % n, (t // n) % n, t // (n * n)
    for c in range(m ** 3):
        ci, cj, ck = c % m, (c // m) % m, c // (m * m)
        G = (ci * n + i) + D * ((cj * n + j) + D * (ck * n + k))
        ga[G] = ainv[c * nf:(c + 1) * nf]
        gb[G] = bdiv[c * nf:(c + 1) * nf]
    xs = N.standard_solve(np.zeros(3), np.ones(3), int(np.log2(D)), ga, gb, load.kind, list(load.params))
    GE, _ = N.counts(D)
    es = np.linalg.norm(x[:GE] - xs[:GE]) / np.linalg.norm(xs[:GE])
    eu = np.linalg.norm(x[GE:] - xs[GE:]) / np.linalg.norm(xs[GE:])
    return es, eu


def test_multiscale_vs_standard_solution():
    """Error of the Ned_RT multiscale solution (coarse solve with the reference's
    natural conditions, fine reconstruction by set_global_weights) against the
    standard fine-scale solution (NedRTStd) on the same fine grid and rough
    coefficient: bounded, and smaller on the finer coarse grid."""
    es2, eu2 = _multiscale_vs_standard(2, 2, 3)  # coarse 2^3 x depth 2 vs fine 8^3
    es4, eu4 = _multiscale_vs_standard(4, 2, 3)  # coarse 4^3 x depth 2 vs fine 16^3
    print(f"multiscale vs standard Ned_RT: 2^3 sigma {es2:.3e} u {eu2:.3e}; 4^3 sigma {es4:.3e} u {eu4:.3e}")
    assert max(es2, eu2) < 0.7 and max(es4, eu4) < 0.55
    assert es4 < es2 and eu4 < eu2


def test_standard_solve_converges_to_analytic_solution():
    """Known answer: A = a I and the vector trig load with w = pi have the exact
    solution u = f / (2 a w^2), sigma = curl f / (2 w^2) under the natural
    conditions (N.vec_trig_exact_dofs). The discrete solution's DoFs converge
    to the exact ones: face DoFs O(h^2), edge DoFs O(h^4) (measured ratios
    3.9-4.0 and 16)."""
    a, B = 1.0 / 0.7, 1.3
    err = []
    for depth in (2, 3, 4):
        n = 1 << depth
        ainv = np.tile(np.eye(3) / a, (n ** 3, 1, 1))
        xs = N.standard_solve(np.zeros(3), np.ones(3), depth, ainv, np.full(n ** 3, B), N.LOAD_VEC_TRIG,
                              [1.0, 1.0, 0.0, 0.0])
        xe = N.vec_trig_exact_dofs(n, 1.0, 1.0, a)
        NE, _ = N.counts(n)
        err.append((np.linalg.norm(xs[:NE] - xe[:NE]) / np.linalg.norm(xe[:NE]),
                    np.linalg.norm(xs[NE:] - xe[NE:]) / np.linalg.norm(xe[NE:])))
    assert err[-1][0] < 1e-6 and err[-1][1] < 5e-3
    for (s0, u0), (s1, u1) in zip(err, err[1:]):
        assert s0 / s1 > 12.0 and u0 / u1 > 3.5, err


def test_multiscale_solution_converges_to_analytic_solution():
    """The whole multiscale Ned_RT pipeline of the oracle (local basis solves,
    block Galerkin, coarse solve with the reference's natural conditions,
    set_global_weights reconstruction) against the analytic solution of the
    constant-coefficient problem (N.vec_trig_exact_dofs): the error falls at
    first order in the coarse mesh size H (measured: sigma 45.7 % -> 22.3 %,
    u 58.9 % -> 30.8 % from coarse 2^3 to 4^3 at depth 2)."""
    from oracle import nedrt_adjoint as NA
    from test_coarse_solve import scipy_nedrt_coarse
    a, B, depth = 1.0 / 0.7, 1.3, 2
    n = 1 << depth
    err = []
    for m in (2, 4):
        cells = workloads.coarse_grid(m, depth)
        nfc = len(cells) * n ** 3
        ref = N.build(cells, np.tile(np.eye(3) / a, (nfc, 1, 1)), np.full(nfc, B), N.LOAD_VEC_TRIG,
                      [1.0, 1.0, 0.0, 0.0])
        U = scipy_nedrt_coarse(m, ref["KH"], ref["FH"])
        g, _ = NA.coarse_maps(m)
        NE, _ = N.counts(n)
        Phi = np.array(ref["Phi"])
        x = _global_fine_field(m, n, lambda c: (U[g[c, :12]] @ Phi[c, :12, :NE], U[g[c, 12:]] @ Phi[c, 12:, NE:]))
        xe = N.vec_trig_exact_dofs(m * n, 1.0, 1.0, a)
        GE, _ = N.counts(m * n)
        err.append((np.linalg.norm(x[:GE] - xe[:GE]) / np.linalg.norm(xe[:GE]),
                    np.linalg.norm(x[GE:] - xe[GE:]) / np.linalg.norm(xe[GE:])))
    (s2, u2), (s4, u4) = err
    assert max(s2, u2) < 0.65 and max(s4, u4) < 0.35, err
    assert s2 / s4 > 1.7 and u2 / u4 > 1.7, err


def test_constant_diagonal_coefficients_give_the_standard_basis():
    """Known answer (the Ned_RT analogue of Q1's trilinear basis): with a
    constant diagonal A^-1 and constant B the coarse Nedelec / RT functions
    solve the local problems, so the multiscale basis (primary blocks) equals
    the standard functions of the set_to_std path and K_H its Galerkin matrix,
    on any box. A full constant tensor breaks it (edge bases differ by ~7 %)."""
    n, size = 4, np.array([1.0, 0.8, 1.3])
    NE, _ = N.counts(n)
    for A3, holds in ((np.diag([0.5, 1.0, 2.0]), True),
                      (np.array([[1.0, 0.3, 0.1], [0.3, 0.8, -0.2], [0.1, -0.2, 1.5]]), False)):
        ainv = np.tile(A3, (n ** 3, 1, 1))
        bdiv = np.full(n ** 3, 1.7)
        P, KH, _ = N.build_cell(np.zeros(3), size, 2, ainv, bdiv, basis="solve")
        S, KHs, _ = N.build_cell(np.zeros(3), size, 2, ainv, bdiv, basis="std")
        de = max(np.abs(P[b, :NE] - S[b, :NE]).max() / np.abs(S[b, :NE]).max() for b in range(12))
        if holds:
            df = max(np.abs(P[b, NE:] - S[b, NE:]).max() / np.abs(S[b, NE:]).max() for b in range(12, 18))
            assert de <= 1e-12 and df <= 1e-12
            assert np.abs(KH - KHs).max() <= 1e-12 * np.abs(KHs).max()
        else:
            assert de > 1e-3
