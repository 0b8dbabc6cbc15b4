"""CPU checks of the multilevel (BPX) face preconditioner of the Ned_RT
solver, restated in Python from the kernel's index maps (csrc/nedrt_solve.cu:
ml_index / ml_parents / ml_code, nr_ml_setup_kernel's probing colours,
ml_coarse_block's cascade) against explicit matrices built from the oracle:
  - the level functions nest (level m = 1/8, 1/4, 1/8 combination of the
    level-2m functions at planes 2P-1, 2P, 2P+1 of its four child patches);
  - one application of S = D + C^T diag(M)^-1 C to the sum of the functions of
    one colour (normal, P mod 3, patch parity) gives their exact diagonal
    entries of P_m^T S P_m (no two functions of a colour interact);
  - the restriction / exact level-2 solve / prolongation cascade equals the
    explicit operator sum_m P_m X_m P_m^T."""
import numpy as np
import pytest
import scipy.sparse as sp

import workloads
from oracle import nedrt_oracle as N


def ml_count(m):
    return 3 * (m - 1) * m * m


def ml_index(lm, d, P, a, b):
    m = 1 << lm
    return ((d * (m - 1) + P - 1) << (2 * lm)) + (b << lm) + a


def ml_parents(lm, d, p, x, y):
    m = 1 << lm
    a, b = x >> 1, y >> 1
    if p % 2 == 0:
        P = p >> 1
        return [(ml_index(lm, d, P, a, b), 0.25)] if 1 <= P <= m - 1 else []
    P0 = p >> 1
    out = []
    if P0 >= 1:
        out.append((ml_index(lm, d, P0, a, b), 0.125))
    if P0 + 1 <= m - 1:
        out.append((ml_index(lm, d, P0 + 1, a, b), 0.125))
    return out


def ml_decode(lm, J):
    m = 1 << lm
    per = (m - 1) << (2 * lm)
    d = int(J >= per) + int(J >= 2 * per)
    rem = J - d * per
    return d, (rem >> (2 * lm)) + 1, rem & (m - 1), (rem >> lm) & (m - 1)


def face_geometry(n):
    """(normal, plane, x, y) of every fine face in the kernel's numbering."""
    Fx = (n + 1) * n * n
    out = []
    for u in range(3 * Fx):
        d, t = divmod(u, Fx)
        if d == 0:
            i, j, k = t % (n + 1), (t // (n + 1)) % n, t // ((n + 1) * n)
            out.append((0, i, j, k))
        elif d == 1:
            i, j, k = t % n, (t // n) % (n + 1), t // (n * (n + 1))
            out.append((1, j, i, k))
        else:
            i, j, k = t % n, (t // n) % n, t // (n * n)
            out.append((2, k, i, j))
    return out


def fine_weights(L, k, d, q, x, y):
    """Values of the level-2^(L-k) functions at fine face (d, q, x, y) (ml_fine_weights)."""
    lm, r = L - k, 1 << k
    m = 1 << lm
    a, b, P0, rem = x >> k, y >> k, q >> k, q & (r - 1)
    out = []
    if 1 <= P0 <= m - 1:
        out.append((ml_index(lm, d, P0, a, b), (r - rem) / r / (r * r), P0))
    if rem and 1 <= P0 + 1 <= m - 1:
        out.append((ml_index(lm, d, P0 + 1, a, b), rem / r / (r * r), P0 + 1))
    return out


@pytest.fixture(scope="module")
def system():
    depth = 3
    cells, ainv6, bdiv, _ = workloads.nedrt_tensor(m=1, depth=depth, seed=3)
    n = 1 << depth
    A = N.assemble(n, cells["size"][0], N.sym6_to_ainv(ainv6), bdiv).tocsr()
    NE, NF = N.counts(n)
    bnd = N.boundary_mask(n)
    I = np.where(~bnd)[0]
    Ie, If = I[I < NE], I[I >= NE]
    M, C, D = A[Ie][:, Ie], -A[Ie][:, If], A[If][:, If]
    S = (D + C.T @ sp.diags(1.0 / M.diagonal()) @ C).tocsr()
    geo = face_geometry(n)
    pos = {u: t for t, u in enumerate(If - NE)}
    return depth, n, S, geo, pos, If - NE


def level_matrix(system, k):
    L, n, S, geo, pos, uI = system
    m = 1 << (L - k)
    rows, cols, vals = [], [], []
    for u in uI:
        d, q, x, y = geo[u]
        for j, w, _ in fine_weights(L, k, d, q, x, y):
            rows.append(pos[u]); cols.append(j); vals.append(w)
    return sp.csr_matrix((vals, (rows, cols)), shape=(len(uI), ml_count(m)))


def test_levels_nest(system):
    L = system[0]
    P1, P2 = level_matrix(system, 1), level_matrix(system, 2)
    R = np.zeros((ml_count(2), ml_count(4)))  # level 2 from level 4 (ml_restrict_one weights)
    for J in range(ml_count(2)):
        d, P, a, b = ml_decode(1, J)
        for q in (-1, 0, 1):
            for yy in (0, 1):
                for xx in (0, 1):
                    R[J, ml_index(2, d, 2 * P + q, 2 * a + xx, 2 * b + yy)] += 0.25 if q == 0 else 0.125
    assert np.abs((P1 @ R.T) - P2.toarray()).max() < 1e-15


def test_probing_colours_give_exact_diagonals(system):
    L, n, S, geo, pos, uI = system
    k = 1  # level n/2 = 4
    P1 = level_matrix(system, k)
    ref = (P1.T @ S @ P1).diagonal()
    got = np.zeros_like(ref)
    for col in range(36):
        cd, cP, ca, cb = col // 12, (col >> 2) % 3, (col >> 1) & 1, col & 1
        x = np.zeros(len(uI))
        members = []
        for u in uI:
            d, q, xx, yy = geo[u]
            for j, w, P in fine_weights(L, k, d, q, xx, yy):
                if d == cd and P % 3 == cP and (xx >> k) & 1 == ca and (yy >> k) & 1 == cb:
                    x[pos[u]] += w
                    members.append((pos[u], j, w))
        s = S @ x
        for t, j, w in members:
            got[j] += w * s[t]
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    # a parity-only colouring (P mod 2) would not separate the functions: S reaches two planes
    G = (P1.T @ S @ P1).toarray()
    assert abs(G[ml_index(2, 0, 1, 0, 0), ml_index(2, 0, 3, 0, 0)]) > 1e-6 * G.diagonal().max()


def test_cascade_equals_explicit_bpx(system):
    L, n, S, geo, pos, uI = system
    P1, P2 = level_matrix(system, 1), level_matrix(system, 2)
    D1 = (P1.T @ S @ P1).diagonal()
    S2inv = np.linalg.inv((P2.T @ S @ P2).toarray())
    v = np.random.default_rng(0).standard_normal(len(uI))
    explicit = P1 @ (P1.T @ v / D1) + P2 @ (S2inv @ (P2.T @ v))
    # the kernel's path: fine -> level 4 (face codes), level 4 -> 2, exact, level 2 -> 4 (codes), level 4 -> fine
    r1 = np.zeros(ml_count(4))
    for u in uI:
        d, p, x, y = geo[u]
        for j, w in ml_parents(2, d, p, x, y):
            r1[j] += w * v[pos[u]]
    r2 = np.zeros(ml_count(2))
    for j in range(ml_count(4)):
        d, P, a, b = ml_decode(2, j)
        for J, w in ml_parents(1, d, P, a, b):
            r2[J] += w * r1[j]
    y2 = S2inv @ r2
    y1 = np.array([r1[j] / D1[j] + sum(w * y2[J] for J, w in ml_parents(1, *ml_decode(2, j)))
                   for j in range(ml_count(4))])
    z = np.zeros(len(uI))
    for u in uI:
        d, p, x, y = geo[u]
        z[pos[u]] = sum(w * y1[j] for j, w in ml_parents(2, d, p, x, y))
    assert np.abs(z - explicit).max() <= 1e-12 * np.abs(explicit).max()
    # and the coarse share of gamma^2
    assert abs(v @ z - (r1 @ (r1 / D1) + r2 @ y2)) <= 1e-12 * abs(v @ z)


def test_fine_face_probing_gives_assembled_diagonal(system):
    """The setup kernel's 36 single-face colours (normal, plane mod 3, x and y
    parity): one application of S per colour returns S_ff for all its faces."""
    L, n, S, geo, pos, uI = system
    got = np.zeros(len(uI))
    for col in range(36):
        cd, cP, ca, cb = col // 12, (col >> 2) % 3, (col >> 1) & 1, col & 1
        sel = [pos[u] for u in uI if geo[u][0] == cd and geo[u][1] % 3 == cP and geo[u][2] % 2 == ca
               and geo[u][3] % 2 == cb]
        x = np.zeros(len(uI))
        x[sel] = 1.0
        s = S @ x
        got[sel] = s[sel]
    ref = S.diagonal()
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
