"""GPU parity of the Q1 build with a tensor diffusion coefficient (the handle's
q1_coefficient TENSOR / GAUSS layouts) against the FP64 oracle (C ABI).

The reference's only Q1 example (example_parameters/prm_q_test-01.prm) uses
the rotated oscillatory Diffusion_A (frequencies 17/16/15, alpha 0.9,
rotate = true) evaluated at the 2x2x2 Gauss points of every fine cell
(source/equation_data/eqn_coeff_A.cc:162-191, q_basis.cc:218-231); the GAUSS
layout takes exactly those values, so the reference's own Q1 problem is
reproduced. Tolerances (both precisions), as for the scalar layout:
  K_H, F_H         max abs error <= 1e-10 * max |entry| of the cell
  basis functions  max |phi - phi_oracle| <= 1e-10 * max |phi_oracle| per function
"""
import numpy as np
import pytest

import workloads

pytestmark = pytest.mark.gpu
TOL = 1e-10
PRECISIONS = ("mixed", "fp64")


def _handle(gpu, precision, layout):
    p = gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64
    return gpu.Handle(precision=p, q1_coefficient=layout)


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _check(gpu, oracle_lib, precision, layout, cells, a, r, load, basis=True):
    h = _handle(gpu, precision, layout)
    KH, FH, rep, st = h.q1_build(cells, a, r, load)
    assert st == gpu.SUCCESS and rep["converged"].all(), rep
    ref = oracle_lib.q1_build(cells["origin"], cells["size"], cells["depth"], a, r, load_kind=load.kind,
                              load_params=list(load.params), want_phi=basis, coef_mode=layout)
    assert ref["status"] == 0
    ek = max(_rel(KH[c], ref["KH"][c]) for c in range(len(cells)))
    ef = max(_rel(FH[c], ref["FH"][c]) for c in range(len(cells)) if np.abs(ref["FH"][c]).max() > 0)
    ep = 0.0
    if basis:
        n1 = (1 << cells["depth"].astype(np.int64)) + 1
        off = np.concatenate([[0], np.cumsum(8 * n1 ** 3)])
        for c, pg in enumerate(h.q1_basis_cells(cells, 0, len(cells))):
            po = ref["Phi"][off[c]:off[c + 1]].reshape(8, -1)
            ep = max(ep, max(_rel(pg[v], po[v]) for v in range(8)))
    print(f"{precision} layout {layout}: K_H {ek:.2e}, F_H {ef:.2e}, Phi {ep:.2e}, "
          f"max iterations {int(rep['iterations'].max())}")
    assert ek <= TOL and ef <= TOL and ep <= TOL, (ek, ef, ep)
    return KH, FH, rep


@pytest.mark.parametrize("precision", PRECISIONS)
def test_reference_diffusion_at_gauss_points(gpu, oracle_lib, precision):
    """The reference's own Q1 coefficient (rotated, oscillatory, varying inside
    every fine cell) at the Gauss points, coarse 2^3 x depth 3."""
    cells, a, r, load = workloads.q1_reference_tensor(m=2, depth=3, gauss=True)
    _check(gpu, oracle_lib, precision, gpu.Q1_COEF_GAUSS, cells, a, r, load)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_tensor_per_cell_mixed_depths_with_reaction(gpu, oracle_lib, precision):
    """A Haar-rotated log-normal tensor per fine cell (the Ned_RT law), depths
    1-4 in one batch, reaction 1: shared-memory and global element data."""
    cells = workloads.coarse_grid(2, [1, 2, 3, 4, 4, 3, 2, 1])
    nf = int(np.sum(workloads.fine_counts(cells)[0]))
    rng = np.random.default_rng(12)
    g = rng.standard_normal((nf, 3))
    R = workloads.haar_rotations(rng, nf)
    A = np.einsum("cij,cj,ckj->cik", R, np.exp(g), R)
    a6 = np.stack([A[:, 0, 0], A[:, 1, 1], A[:, 2, 2], A[:, 0, 1], A[:, 0, 2], A[:, 1, 2]], 1)
    load = gpu.make_load(gpu.LOAD_SIN_PRODUCT, (1.0, 1.0, 0.0, 0.0))
    _check(gpu, oracle_lib, precision, gpu.Q1_COEF_TENSOR, cells, a6, np.ones(nf), load)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_depth5_gauss_global_workspace(gpu, oracle_lib, precision):
    """A depth-5 cell (35937 nodes: vectors in the global workspace) with the
    reference's coefficient at the Gauss points."""
    cells, a, r, load = workloads.q1_reference_tensor(m=1, depth=5, gauss=True)
    _check(gpu, oracle_lib, precision, gpu.Q1_COEF_GAUSS, cells, a, r, load, basis=True)


def test_isotropic_tensor_equals_scalar_layout(gpu):
    """A I per fine cell through the tensor solver gives the scalar solver's
    K_H (two independent operator applies)."""
    cells, a, r, load = workloads.q1_lognormal(m=2, depth=3, seed=4, reaction=True)
    hs = gpu.Handle()
    KH0, FH0, rep0, _ = hs.q1_build(cells, a, r, load)
    a6 = np.zeros((a.size, 6))
    a6[:, :3] = a[:, None]
    ht = gpu.Handle(q1_coefficient=gpu.Q1_COEF_TENSOR)
    KH1, FH1, rep1, _ = ht.q1_build(cells, a6, r, load)
    for c in range(len(cells)):
        assert _rel(KH1[c], KH0[c]) <= TOL and _rel(FH1[c], FH0[c]) <= TOL


def test_tensor_layout_rejects_non_spd(gpu):
    """A non-SPD tensor is rejected before any launch (MSFEC_ERROR_NUMERICAL)."""
    cells, a, r, load = workloads.q1_reference_tensor(m=1, depth=1, gauss=False)
    bad = a.copy()
    bad[3, 3] = 10.0  # |a01| > sqrt(a00 a11)
    h = gpu.Handle(q1_coefficient=gpu.Q1_COEF_TENSOR)
    with pytest.raises(gpu.MsfecError) as e:
        h.q1_build(cells, bad, r, load)
    assert e.value.status == gpu.ERROR_NUMERICAL


def _tensor_misfit(gpu, precision, m=2, depth=2, npts=24, seed=21, rtol=None):
    """Misfit of the coarse solution for A_e = exp(theta_e) A_ref at the Gauss
    points (the reference's coefficient), data from a perturbed theta."""
    from adjoint_harness import MisfitProblem
    cells, base, _, load = workloads.q1_reference_tensor(m=m, depth=depth, gauss=True)
    rng = np.random.default_rng(seed)
    cell_of = rng.integers(0, len(cells), npts)
    pts = cells["origin"][cell_of] + rng.random((npts, 3)) * cells["size"][cell_of]
    theta = 0.3 * rng.standard_normal(base.shape[0])
    prec = gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64
    p2 = MisfitProblem(gpu, cells, m, load, cell_of, pts, np.zeros(npts), prec, base=base, layout=gpu.Q1_COEF_GAUSS)
    _, st2 = p2.forward(theta + 0.5 * rng.standard_normal(theta.shape))
    prob = MisfitProblem(gpu, cells, m, load, cell_of, pts, st2["u"], prec, rtol=rtol, base=base,
                         layout=gpu.Q1_COEF_GAUSS)
    return prob, theta


@pytest.mark.parametrize("precision", PRECISIONS)
def test_tensor_adjoint_matches_central_differences(gpu, precision):
    """dJ/dtheta for A_e -> exp(theta_e) A_e (Gauss-point layout) against
    central differences of the GPU forward (h = 1e-6, 4 seeded directions;
    tolerance as the scalar adjoint's: 1e-6 of sum |g_i d_i|)."""
    prob, theta = _tensor_misfit(gpu, precision, rtol=1e-14)
    J, state = prob.forward(theta)
    grad = prob.gradient(theta, state)
    rng = np.random.default_rng(5)
    h = 1e-6
    for t in range(4):
        d = rng.standard_normal(theta.shape)
        fd = (prob.forward(theta + h * d)[0] - prob.forward(theta - h * d)[0]) / (2 * h)
        ad = float(grad @ d)
        scale = float(np.abs(grad * d).sum())
        assert abs(fd - ad) <= 1e-6 * scale, (t, fd, ad, scale)


def test_tensor_adjoint_matches_oracle(gpu, oracle_lib):
    """The GPU tensor-layout gradient against the FP64 oracle's (quadrature
    element matrices, sparse direct adjoint solves) to 1e-8."""
    from oracle import q1_adjoint
    prob, theta = _tensor_misfit(gpu, "mixed")
    g_gpu = prob.gradient(theta)
    J_o, g_or = q1_adjoint.misfit(prob.cells, prob.m, theta, prob.load, prob.cell_of, prob.points, prob.data,
                                  coef_mode=2, base=prob.base)
    J_g, _ = prob.forward(theta)
    assert abs(J_g - J_o) <= 1e-9 * abs(J_o)
    assert np.abs(g_gpu - g_or).max() <= 1e-8 * np.abs(g_or).max()
