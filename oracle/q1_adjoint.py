"""FP64 CPU oracle of the Q1 adjoint gradient (TEST INFRASTRUCTURE ONLY).

dJ/d log a_e for J = 1/2 sum_k (u_H(x_k) - d_k)^2 of the coarse multiscale
solution (structured m^3 coarse grid of the unit cube, homogeneous Dirichlet),
from the FP64 oracle basis:
  dJ/d log a_e = -a_e [ (mu + psi_U)_e^T Khat psi_l,e + eta_e^T Khat psi_U,e ]
psi_U = Phi U_e, psi_l = Phi lambda_e (lambda = K_H^-1 dJ/dU), mu = K_II^-1 b_I,
eta = K_II^-1 (sum_k g_k E_k)_I (sparse direct solves). The reference has no
adjoint; this restates the derivative of its Q1 path (QBasis,
source/Q/q_basis.cc; QMultiscale, source/Q/q_global.cc).
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import oracle as O


def _cell_nodes(m):
    M1 = m + 1
    out = np.zeros((m ** 3, 8), dtype=np.int64)
    for c in range(m ** 3):
        i, j, k = c % m, (c // m) % m, c // (m * m)
        out[c] = [(i + (v & 1)) + M1 * ((j + ((v >> 1) & 1)) + M1 * (k + (v >> 2))) for v in range(8)]
    return out


def _coarse(m, KH):
    M1 = m + 1
    nodes = _cell_nodes(m)
    rows = np.repeat(nodes, 8, axis=1).ravel()
    cols = np.tile(nodes, (1, 8)).ravel()
    K = sp.coo_matrix((KH.ravel(), (rows, cols)), shape=(M1 ** 3, M1 ** 3)).tocsr()
    idx = np.arange(M1 ** 3)
    i, j, k = idx % M1, (idx // M1) % M1, idx // (M1 * M1)
    I = np.where((i > 0) & (j > 0) & (k > 0) & (i < m) & (j < m) & (k < m))[0]
    return K, I, nodes


def _interp(t, n):
    """Fine nodes and trilinear weights of a point with cell-local coordinates t in [0,1]^3."""
    N1 = n + 1
    s = np.asarray(t) * n
    f = np.minimum(np.floor(s).astype(int), n - 1)
    xi = s - f
    out = []
    for c in range(8):
        cx, cy, cz = c & 1, (c >> 1) & 1, c >> 2
        w = (xi[0] if cx else 1 - xi[0]) * (xi[1] if cy else 1 - xi[1]) * (xi[2] if cz else 1 - xi[2])
        out.append(((f[0] + cx) + N1 * ((f[1] + cy) + N1 * (f[2] + cz)), w))
    return out


def _element(h):
    K = np.zeros((8, 8))
    k1 = [np.array([[1.0, -1.0], [-1.0, 1.0]]) / hd for hd in h]
    m1 = [hd * np.array([[1 / 3, 1 / 6], [1 / 6, 1 / 3]]) for hd in h]
    for u in range(8):
        for v in range(8):
            a = [(u >> d) & 1 for d in range(3)]
            b = [(v >> d) & 1 for d in range(3)]
            K[u, v] = (k1[0][a[0], b[0]] * m1[1][a[1], b[1]] * m1[2][a[2], b[2]]
                       + m1[0][a[0], b[0]] * k1[1][a[1], b[1]] * m1[2][a[2], b[2]]
                       + m1[0][a[0], b[0]] * m1[1][a[1], b[1]] * k1[2][a[2], b[2]])
    return K


def element_tensor(h, A6, gauss):
    """Element stiffness sum_q grad psi_u . A_q grad psi_v JxW of every fine cell
    (the reference's quadrature loop, q_basis.cc:222-231). A6: [ne, 6] (one
    tensor per cell) or [ne, 48] (at the 2x2x2 Gauss points, x fastest).
    Returns [ne, 8, 8]."""
    g = 0.5 / np.sqrt(3.0)
    qp = np.array([0.5 - g, 0.5 + g])
    G = np.zeros((8, 8, 3))  # [gauss point, vertex, direction], physical gradient
    for q in range(8):
        t = [qp[q & 1], qp[(q >> 1) & 1], qp[q >> 2]]
        for u in range(8):
            b = [(u >> d) & 1 for d in range(3)]
            val = [t[d] if b[d] else 1 - t[d] for d in range(3)]
            der = [(1.0 if b[d] else -1.0) / h[d] for d in range(3)]
            G[q, u] = [der[0] * val[1] * val[2], val[0] * der[1] * val[2], val[0] * val[1] * der[2]]
    A6 = np.asarray(A6).reshape(len(A6), 8 if gauss else 1, 6)
    A6 = np.broadcast_to(A6, (len(A6), 8, 6))
    A = np.stack([np.stack([A6[..., 0], A6[..., 3], A6[..., 4]], -1),
                  np.stack([A6[..., 3], A6[..., 1], A6[..., 5]], -1),
                  np.stack([A6[..., 4], A6[..., 5], A6[..., 2]], -1)], -2)  # [ne, 8, 3, 3]
    return np.einsum("qud,eqdk,qvk->euv", G, A, G) * (h[0] * h[1] * h[2] / 8.0)


def misfit(cells, m, theta, load, cell_of, points, data, gradient=True, coef_mode=0, base=None):
    """Returns (J, grad or None) for a uniform-depth batch on the m^3 coarse grid.
    coef_mode 0: a = exp(theta) per fine cell; 1 / 2 (tensor per fine cell / at
    the Gauss points): A_e = exp(theta_e) base_e, grad = dJ/dtheta."""
    depth = int(cells["depth"][0])
    n = 1 << depth
    N1 = n + 1
    a = np.exp(theta) if coef_mode == 0 else np.asarray(base) * np.exp(theta)[:, None]
    res = O.q1_build(cells["origin"], cells["size"], cells["depth"], a, None, load_kind=load.kind,
                     load_params=list(load.params), coef_mode=coef_mode)
    KH, FH = res["KH"], res["FH"]
    Phi = res["Phi"].reshape(m ** 3, 8, -1)
    K, I, nodes = _coarse(m, KH)
    b = np.zeros((m + 1) ** 3)
    np.add.at(b, nodes.ravel(), FH.ravel())
    lu = spla.splu(K[I][:, I].tocsc())
    U = np.zeros_like(b)
    U[I] = lu.solve(b[I])
    tloc = (np.asarray(points) - cells["origin"][cell_of]) / cells["size"][cell_of]
    u = np.zeros(len(points))
    for p in range(len(points)):
        psi = U[nodes[cell_of[p]]] @ Phi[cell_of[p]]
        u[p] = sum(w * psi[q] for q, w in _interp(tloc[p], n))
    g = u - data
    J = 0.5 * float(np.sum(g ** 2))
    if not gradient:
        return J, None
    cvec = np.zeros_like(b)
    for p in range(len(points)):
        c = cell_of[p]
        for v in range(8):
            cvec[nodes[c, v]] += g[p] * sum(w * Phi[c, v, q] for q, w in _interp(tloc[p], n))
    lam = np.zeros_like(b)
    lam[I] = lu.solve(cvec[I])
    grad = np.zeros_like(theta)
    bidx = np.arange(N1 ** 3)
    bi, bj, bk = bidx % N1, (bidx // N1) % N1, bidx // (N1 * N1)
    Iin = np.where(~((bi == 0) | (bj == 0) | (bk == 0) | (bi == n) | (bj == n) | (bk == n)))[0]
    e = np.arange(n ** 3)
    ei, ej, ek = e % n, (e // n) % n, e // (n * n)
    enodes = np.stack([(ei + (v & 1)) + N1 * ((ej + ((v >> 1) & 1)) + N1 * (ek + (v >> 2))) for v in range(8)], 1)
    for c in range(m ** 3):
        sl = slice(c * n ** 3, (c + 1) * n ** 3)
        Kf, bf = O.q1_assemble(cells["origin"][c], cells["size"][c], depth, a[sl], None, load.kind,
                               list(load.params), coef_mode=coef_mode)
        Kf = Kf.tocsr()
        flu = spla.splu(Kf[Iin][:, Iin].tocsc())
        mu = np.zeros(N1 ** 3)
        mu[Iin] = flu.solve(bf[Iin])
        src = np.zeros(N1 ** 3)
        for p in np.where(cell_of == c)[0]:
            for q, w in _interp(tloc[p], n):
                src[q] += g[p] * w
        eta = np.zeros(N1 ** 3)
        eta[Iin] = flu.solve(src[Iin])
        psiU = U[nodes[c]] @ Phi[c]
        psiL = lam[nodes[c]] @ Phi[c]
        A_ = (mu + psiU)[enodes]
        B_ = psiL[enodes]
        C_ = eta[enodes]
        D_ = psiU[enodes]
        if coef_mode == 0:
            Kh = _element(np.asarray(cells["size"][c]) / n)
            grad[sl] = -a[sl] * (np.einsum("eu,uv,ev->e", A_, Kh, B_) + np.einsum("eu,uv,ev->e", C_, Kh, D_))
        else:  # d K_e / d theta_e = K_e(A_e)
            Ke = element_tensor(np.asarray(cells["size"][c]) / n, a[sl], coef_mode == 2)
            grad[sl] = -(np.einsum("eu,euv,ev->e", A_, Ke, B_) + np.einsum("eu,euv,ev->e", C_, Ke, D_))
    return J, grad
