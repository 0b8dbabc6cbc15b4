"""GPU parity of the Q_Ned (Q1 sigma x Nedelec u) basis build against the FP64
oracle (C ABI). Stated tolerances (both precisions; mixed = FP32 MINRES +
FP64 refinement): K_H, F_H max abs error <= 1e-10 * max |entry| of the cell;
basis max|phi - phi_oracle| <= 1e-10 * max|phi_oracle| per function."""
import numpy as np
import pytest

import workloads
from oracle import nedrt_oracle as NR
from oracle import qned_oracle as Q

pytestmark = pytest.mark.gpu
TOL_KH = 1e-10
TOL_PHI = 1e-10


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _coefs(cells, seed):
    """A (SPD tensor, from the Ned_RT workload's A^-1) and B^-1 per fine cell."""
    cen = workloads.fine_centres(cells)
    rng = np.random.default_rng(seed)
    nf = cen.shape[0]
    g = rng.standard_normal((nf, 3))
    R = workloads.haar_rotations(rng, nf)
    A = np.einsum("cij,cj,ckj->cik", R, np.exp(0.5 * g), R)
    a6 = NR.ainv_to_sym6(A)
    binv = 1.0 / (1.0 - 0.9 * np.sin(2 * np.pi * 14.0 * cen[:, 0]))
    return A, a6, binv


@pytest.mark.parametrize("precision", ("mixed", "fp64"))
@pytest.mark.parametrize("m,depth", [(1, 2), (1, 3)])
def test_qned_basis_matches_oracle(gpu, precision, m, depth):
    cells = workloads.coarse_grid(m, depth)
    A, a6, binv = _coefs(cells, seed=7 + depth)
    load = gpu.make_load(gpu.LOAD_VEC_TRIG, (1.0, 1.0, 0.0, 0.0))
    h = gpu.Handle(precision=gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64)
    KH, FH, rep, st = h.qned_build(cells, a6, binv, load)
    assert st == gpu.SUCCESS and rep["converged"].all(), rep
    ref = Q.build(cells, binv, A, load.kind, list(load.params))
    for c in range(len(cells)):
        assert _rel(KH[c], ref["KH"][c]) <= TOL_KH, (c, _rel(KH[c], ref["KH"][c]))
        assert _rel(FH[c], ref["FH"][c]) <= TOL_KH
    phi = h.qned_basis()
    off = 0
    for c, po in enumerate(ref["Phi"]):
        pg = phi[off:off + po.size].reshape(po.shape)
        off += po.size
        for b in range(20):
            assert _rel(pg[b], po[b]) <= TOL_PHI, (c, b, _rel(pg[b], po[b]))
    print(f"{precision} depth {depth}: max K_H rel err {max(_rel(KH[c], ref['KH'][c]) for c in range(len(cells))):.2e}, "
          f"max iterations {rep['iterations'].max()}")


@pytest.mark.parametrize("precision", ("mixed", "fp64"))
def test_qned_matches_golden(gpu, precision):
    """GPU build against the committed oracle fixture (coarse 2^3 x depth 2,
    tests/golden/make_golden.py), same per-cell tolerance as above."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "qned_tensor_m2_L2_seed4.npz"))
    cells, a6, binv, load = workloads.qned_tensor(m=2, depth=2, seed=4)
    h = gpu.Handle(precision=gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64)
    KH, FH, rep, st = h.qned_build(cells, a6, binv, load)
    assert st == gpu.SUCCESS and rep["converged"].all(), rep
    for c in range(len(cells)):
        assert _rel(KH[c], g["KH"][c]) <= TOL_KH, (c, _rel(KH[c], g["KH"][c]))
        assert _rel(FH[c], g["FH"][c]) <= TOL_KH, (c, _rel(FH[c], g["FH"][c]))


def test_qned_mixed_depth_batch(gpu):
    """Ragged batch: depths 2 and 3 in one persistent launch (deepest items
    first, workspace sized by the deepest cell), per cell against the oracle."""
    cells = workloads.coarse_grid(2, 2)
    cells["depth"] = [3, 2, 2, 3, 2, 3, 3, 2]
    A, a6, binv = _coefs(cells, seed=21)
    load = gpu.make_load(gpu.LOAD_VEC_TRIG, (1.0, 1.0, 0.0, 0.0))
    h = gpu.Handle()
    KH, FH, rep, st = h.qned_build(cells, a6, binv, load)
    assert st == gpu.SUCCESS and rep["converged"].all(), rep
    ref = Q.build(cells, binv, A, load.kind, list(load.params), want_phi=False)
    for c in range(len(cells)):
        assert _rel(KH[c], ref["KH"][c]) <= TOL_KH, (c, _rel(KH[c], ref["KH"][c]))
        assert _rel(FH[c], ref["FH"][c]) <= TOL_KH, (c, _rel(FH[c], ref["FH"][c]))


def test_qned_rejects_bad_input(gpu):
    """Host-side validation (no kernel runs): scalar load, B^-1 <= 0, A not SPD,
    depth 5; an empty batch succeeds with empty outputs."""
    cells = workloads.coarse_grid(1, 2)
    A, a6, binv = _coefs(cells, seed=3)
    h = gpu.Handle()
    with pytest.raises(gpu.MsfecError):
        h.qned_build(cells, a6, binv, gpu.make_load(gpu.LOAD_SIN_PRODUCT, (1.0, 1.0, 0.0, 0.0)))
    bad = binv.copy()
    bad[3] = -1.0
    with pytest.raises(gpu.MsfecError):
        h.qned_build(cells, a6, bad, gpu.make_load())
    nspd = a6.copy()
    nspd[5, 0] = -1.0
    with pytest.raises(gpu.MsfecError):
        h.qned_build(cells, nspd, binv, gpu.make_load())
    deep = cells.copy()
    deep["depth"] = 5
    with pytest.raises(gpu.MsfecError):
        h.qned_build(deep, np.tile(a6, (512, 1)), np.tile(binv, 512), gpu.make_load())
    KH, FH, rep, st = h.qned_build(cells[:0], a6[:0], binv[:0], gpu.make_load())
    assert st == gpu.SUCCESS and KH.shape == (0, 20, 20) and FH.shape == (0, 20)


@pytest.mark.parametrize("precision", ("mixed", "fp64"))
def test_qned_constant_diagonal_gives_the_standard_basis(gpu, precision):
    """Known answer: constant diagonal A, constant B^-1, non-cubic box; the
    vertex bases' sigma is trilinear, the edge bases' u the coarse Nedelec
    function."""
    depth, n = 3, 8
    cells = workloads.coarse_grid(1, depth)
    cells["size"] = [[1.0, 0.8, 1.3]]
    a6 = np.tile([0.5, 1.0, 2.0, 0.0, 0.0, 0.0], (n ** 3, 1))
    h = gpu.Handle(precision=gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64)
    KH, FH, rep, st = h.qned_build(cells, a6, np.full(n ** 3, 1.7), gpu.make_load())
    assert st == gpu.SUCCESS and rep["converged"].all(), rep
    NV, NE = Q.counts(n)
    phi = h.qned_basis().reshape(20, NV + NE)
    for v in range(8):
        assert _rel(phi[v, :NV], Q.coarse_vertex_values(n, v)) <= TOL_PHI, v
    for l in range(12):
        std = NR.coarse_edge_dofs(n, l)
        assert _rel(phi[8 + l, NV:], std) <= TOL_PHI, (l, _rel(phi[8 + l, NV:], std))
