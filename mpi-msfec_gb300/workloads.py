"""Seeded synthetic inputs of the MsFEC basis-build workloads.

The reference measures on no public dataset; every input here is synthetic
and seeded (numpy PCG64), identical on x86_64 and aarch64:

  q1_lognormal   coarse m^3 cells of the unit cube, depth L, log a ~ N(0,1)
                 i.i.d. per fine cell, optional reaction r, f = sin(pi x)
                 sin(pi y) sin(pi z)         (coarse 4^3, L = 3: the small
                 Q1 case; coarse 8^3, L = 4: the adjoint case)
  q1_uneven      coarse 16^3, L ~ U{2,3,4,5} per cell, a = (1 + 0.9
                 sin(2 pi x/eps) sin(2 pi y/eps) sin(2 pi z/eps)) exp(0.5 xi_c),
                 eps = 1/64, xi_c ~ N(0,1) per coarse cell, sampled at
                 fine-cell centres                     (batched uneven Q1)
  nedrt_tensor   coarse m^3 cells, depth L, A_e = R_e diag(e^g1, e^g2, e^g3) R_e^T
                 per fine cell, g ~ N(0,1), R_e Haar-random rotation (QR of a
                 Gaussian 3x3, sign-fixed, det +1); B = 1 - 0.9 sin(2 pi 14 x)
                 at fine-cell centres (the reference's example div-div
                 coefficient, example_parameters/prm_ned_rt_test-01.prm);
                 f = (sin pi y sin pi z, sin pi z sin pi x, sin pi x sin pi y)
                 (coarse 8^3, L = 3: the small mixed case; 16^3, L = 4: large)
Coarse cells are listed lexicographically (x fastest); fine-cell arrays per
coarse cell are lexicographic too.
"""
from __future__ import annotations

import numpy as np

from msfec import CELL_DTYPE, LOAD_SIN_PRODUCT, LOAD_VEC_TRIG, make_load


def coarse_grid(m, depths, lo=0.0, hi=1.0):
    """m^3 coarse cells of [lo, hi]^3 (x fastest); depths scalar or per cell."""
    H = (hi - lo) / m
    idx = np.arange(m ** 3)
    ci, cj, ck = idx % m, (idx // m) % m, idx // (m * m)
    cells = np.zeros(m ** 3, dtype=CELL_DTYPE)
    cells["origin"] = lo + H * np.stack([ci, cj, ck], axis=1)
    cells["size"] = H
    cells["depth"] = np.broadcast_to(np.asarray(depths, dtype=np.int32), (m ** 3,))
    return cells


def fine_counts(cells):
    n = 1 << cells["depth"].astype(np.int64)
    return n ** 3, (n + 1) ** 3


def work_dof_rhs(cells, rhs=8):
    """Fine DoF x RHS of a Q1 build: sum over cells of (n+1)^3 * 8."""
    return int(np.sum(fine_counts(cells)[1]) * rhs)


def fine_centres(cells):
    """Fine-cell centres (x, y, z) concatenated over cells, per-cell lexicographic."""
    out = []
    for c in cells:
        n = 1 << int(c["depth"])
        h = c["size"] / n
        t = np.arange(n) + 0.5
        z, y, x = np.meshgrid(t, t, t, indexing="ij")
        out.append(np.stack([c["origin"][0] + x.ravel() * h[0], c["origin"][1] + y.ravel() * h[1],
                             c["origin"][2] + z.ravel() * h[2]], axis=1))
    return np.concatenate(out, axis=0)


def q1_lognormal(m=4, depth=3, seed=1, reaction=True):
    rng = np.random.default_rng(seed)
    cells = coarse_grid(m, depth)
    nf = int(np.sum(fine_counts(cells)[0]))
    a = np.exp(rng.standard_normal(nf))
    r = np.ones(nf) if reaction else None
    load = make_load(LOAD_SIN_PRODUCT, (1.0, 1.0, 0.0, 0.0))
    return cells, a, r, load


def q1_uneven(m=16, seed=3, eps=1.0 / 64.0, depths=(2, 3, 4, 5)):
    rng = np.random.default_rng(seed)
    cells = coarse_grid(m, 2)
    cells["depth"] = rng.choice(np.asarray(depths, dtype=np.int32), size=m ** 3)
    xi = rng.standard_normal(m ** 3)
    a_parts = []
    for c in range(m ** 3):
        n = 1 << int(cells["depth"][c])
        h = cells["size"][c][0] / n
        t = (np.arange(n) + 0.5) * h
        sx = np.sin(2 * np.pi * (cells["origin"][c][0] + t) / eps)
        sy = np.sin(2 * np.pi * (cells["origin"][c][1] + t) / eps)
        sz = np.sin(2 * np.pi * (cells["origin"][c][2] + t) / eps)
        osc = 1.0 + 0.9 * sz[:, None, None] * sy[None, :, None] * sx[None, None, :]
        a_parts.append((osc * np.exp(0.5 * xi[c])).ravel())
    a = np.concatenate(a_parts)
    load = make_load(LOAD_SIN_PRODUCT, (1.0, 1.0, 0.0, 0.0))
    return cells, a, None, load


GAUSS_2 = np.array([0.5 - 0.5 / np.sqrt(3.0), 0.5 + 0.5 / np.sqrt(3.0)])


def gauss_points(cells):
    """The 2x2x2 Gauss points (x fastest) of every fine cell: [sum n^3, 8, 3]."""
    out = []
    for c in cells:
        n = 1 << int(c["depth"])
        h = c["size"] / n
        t = np.arange(n)
        k, j, i = np.meshgrid(t, t, t, indexing="ij")
        base = np.stack([i.ravel(), j.ravel(), k.ravel()], 1).astype(np.float64)
        q = np.array([[GAUSS_2[g & 1], GAUSS_2[(g >> 1) & 1], GAUSS_2[g >> 2]] for g in range(8)])
        out.append(c["origin"][None, None, :] + (base[:, None, :] + q[None, :, :]) * h[None, None, :])
    return np.concatenate(out, axis=0)


def euler_rotation(alpha=np.pi / 3, beta=np.pi / 6, gamma=np.pi / 4):
    """The fixed rotation of the reference's Diffusion_A
    (source/equation_data/eqn_coeff_A.cc:25-42; Euler angles pi/3, pi/6, pi/4)."""
    ca, sa, cb, sb, cg, sg = np.cos(alpha), np.sin(alpha), np.cos(beta), np.sin(beta), np.cos(gamma), np.sin(gamma)
    return np.array([[ca * cg - sa * cb * sg, -ca * sg - sa * cb * cg, sa * sb],
                     [sa * cg + ca * cb * sg, -sa * sg + ca * cb * cg, -ca * sb],
                     [sb * sg, sb * cg, cb]])


def reference_diffusion(points, freq=(17, 16, 15), alpha=(0.9, 0.9, 0.9), scale=(1.0, 1.0, 1.0), rotate=True):
    """The reference's Q1 diffusion tensor at points [..., 3]
    (Diffusion_A::value_list, eqn_coeff_A.cc:162-191): diag(scale_d (1 - alpha_d
    sin(2 pi k_d x_d))), rotated by R . R^T; defaults of
    example_parameters/prm_q_test-01.prm (frequencies 17/16/15, alpha 0.9,
    rotate = true). Returns [..., 6] (a00 a11 a22 a01 a02 a12)."""
    x = np.asarray(points, dtype=np.float64)
    d = np.stack([scale[q] * (1.0 - alpha[q] * np.sin(2.0 * np.pi * freq[q] * x[..., q])) for q in range(3)], -1)
    R = euler_rotation() if rotate else np.eye(3)
    A = np.einsum("ij,...j,kj->...ik", R, d, R)
    return np.stack([A[..., 0, 0], A[..., 1, 1], A[..., 2, 2], A[..., 0, 1], A[..., 0, 2], A[..., 1, 2]], -1)


def q1_reference_tensor(m=2, depth=3, gauss=True, freq=(17, 16, 15)):
    """Q1 workload with the reference's example coefficient (rotated
    oscillatory Diffusion_A of prm_q_test-01.prm) on coarse m^3 cells of the
    unit cube: the tensor at each fine cell's Gauss points (gauss=True, 48 per
    fine cell) or at its centre (6 per fine cell); no reaction; the
    example's load f = sin(2 pi x) sin(2 pi y) sin(2 pi z)."""
    cells = coarse_grid(m, depth)
    if gauss:
        a = reference_diffusion(gauss_points(cells), freq=freq).reshape(-1, 48)
    else:
        a = reference_diffusion(fine_centres(cells), freq=freq)
    load = make_load(LOAD_SIN_PRODUCT, (1.0, 2.0, 0.0, 0.0))
    return cells, a, None, load


def haar_rotations(rng, count):
    """Haar-random rotations: QR of Gaussian 3x3 with the sign of diag(R) fixed, det +1."""
    G = rng.standard_normal((count, 3, 3))
    Q, Rm = np.linalg.qr(G)
    d = np.sign(np.diagonal(Rm, axis1=1, axis2=2))
    d[d == 0] = 1.0
    Q = Q * d[:, None, :]
    det = np.linalg.det(Q)
    Q[:, :, 0] *= np.sign(det)[:, None]
    return Q


def nedrt_tensor(m=8, depth=3, seed=2, kb=14.0):
    """Ned_RT workload; returns cells, A^-1 as [fine, 6] (a00 a11 a22 a01 a02 a12), B, load."""
    rng = np.random.default_rng(seed)
    cells = coarse_grid(m, depth)
    nf = int(np.sum(fine_counts(cells)[0]))
    g = rng.standard_normal((nf, 3))
    ainv6 = np.empty((nf, 6))
    chunk = 1 << 20  # rotations drawn in chunks: the same stream as one draw, less memory
    for lo in range(0, nf, chunk):
        hi = min(nf, lo + chunk)
        Rr = haar_rotations(rng, hi - lo)
        ainv = np.einsum("cij,cj,ckj->cik", Rr, np.exp(-g[lo:hi]), Rr)
        ainv6[lo:hi] = np.stack([ainv[:, 0, 0], ainv[:, 1, 1], ainv[:, 2, 2], ainv[:, 0, 1], ainv[:, 0, 2],
                                 ainv[:, 1, 2]], 1)
    x = fine_centres(cells)[:, 0]
    bdiv = 1.0 - 0.9 * np.sin(2 * np.pi * kb * x)
    load = make_load(LOAD_VEC_TRIG, (1.0, 1.0, 0.0, 0.0))
    return cells, ainv6, bdiv, load


def qned_tensor(m=8, depth=3, seed=2, kb=14.0):
    """Q_Ned workload; returns cells, A as [fine, 6] (a00 a11 a22 a01 a02 a12; A = R diag(e^g) R^T,
    g ~ N(0, 1/4), R Haar), B^-1 = 1 / (1 - 0.9 sin(2 pi 14 x)), vector trig load."""
    rng = np.random.default_rng(seed)
    cells = coarse_grid(m, depth)
    nf = int(np.sum(fine_counts(cells)[0]))
    g = 0.5 * rng.standard_normal((nf, 3))
    Rr = haar_rotations(rng, nf)
    A = np.einsum("cij,cj,ckj->cik", Rr, np.exp(g), Rr)
    a6 = np.stack([A[:, 0, 0], A[:, 1, 1], A[:, 2, 2], A[:, 0, 1], A[:, 0, 2], A[:, 1, 2]], 1)
    x = fine_centres(cells)[:, 0]
    binv = 1.0 / (1.0 - 0.9 * np.sin(2 * np.pi * kb * x))
    load = make_load(LOAD_VEC_TRIG, (1.0, 1.0, 0.0, 0.0))
    return cells, a6, binv, load


def rtdq_tensor(m=8, depth=3, seed=2):
    """RT_DQ workload; returns cells, A^-1 as [fine, 6] (A^-1 = R diag(e^-g) R^T, g ~ N(0, 1),
    R Haar: the Ned_RT coefficient law), scalar sin-product load."""
    cells, ainv6, _, _ = nedrt_tensor(m, depth, seed)
    load = make_load(LOAD_SIN_PRODUCT, (1.0, 1.0, 0.0, 0.0))
    return cells, ainv6, load


def rtdq_work_dof_rhs(cells):
    n = 1 << cells["depth"].astype(np.int64)
    return int(np.sum(3 * n * n * (n + 1) + n ** 3) * 6)


def qned_work_dof_rhs(cells):
    n = 1 << cells["depth"].astype(np.int64)
    return int(np.sum((n + 1) ** 3 + 3 * n * (n + 1) ** 2) * 20)


def nedrt_work_dof_rhs(cells):
    n = 1 << cells["depth"].astype(np.int64)
    return int(np.sum(3 * n * (n + 1) ** 2 + 3 * n * n * (n + 1)) * 18)
