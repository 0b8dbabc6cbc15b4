"""GPU parity of the Ned_RT basis build against the FP64 oracle (C ABI).

Tolerances, the 1e-10 bar of the FP64 path, for both precisions (mixed =
FP32 MINRES + FP64 refinement); the oracle's sparse-direct solves are refined
in FP64 to well below it:
  K_H, F_H   max abs error <= 1e-10 * max |entry| of the cell
  basis      max|phi - phi_oracle| <= 1e-10 * max|phi_oracle| per function
"""
import os

import numpy as np
import pytest

import workloads
from oracle import nedrt_oracle as N

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
TOL_KH = 1e-10
TOL_PHI = 1e-10
PRECISIONS = ("mixed", "fp64")


def _handle(gpu, precision, **kw):
    return gpu.Handle(precision=gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64, **kw)


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _check(gpu, precision, cells, ainv6, bdiv, load, basis=True, **kw):
    h = _handle(gpu, precision, **kw)
    KH, FH, rep, st = h.nedrt_build(cells, ainv6, bdiv, load)
    assert st == gpu.SUCCESS and rep["converged"].all(), rep
    ref = N.build(cells, N.sym6_to_ainv(ainv6), bdiv, load.kind, list(load.params), want_phi=basis)
    errs = []
    for c in range(len(cells)):
        e = _rel(KH[c], ref["KH"][c])
        errs.append(e)
        assert e <= TOL_KH, (c, e)
        if np.abs(ref["FH"][c]).max() > 0:
            assert _rel(FH[c], ref["FH"][c]) <= TOL_KH
    if basis:
        phi = h.nedrt_basis()
        off = 0
        for c, po in enumerate(ref["Phi"]):
            pg = phi[off:off + po.size].reshape(po.shape)
            off += po.size
            for b in range(18):
                assert _rel(pg[b], po[b]) <= TOL_PHI, (c, b, _rel(pg[b], po[b]))
    print(f"{precision}: max K_H rel err {max(errs):.2e}, max iterations {rep['iterations'].max()}")
    return KH, FH, rep


@pytest.mark.parametrize("precision", PRECISIONS)
def test_small_tensor_matches_golden(gpu, precision):
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=2, depth=2, seed=2)
    g = np.load(os.path.join(HERE, "golden", "nedrt_tensor_m2_L2_seed2.npz"))
    h = _handle(gpu, precision)
    KH, FH, rep, st = h.nedrt_build(cells, ainv6, bdiv, load)
    assert st == gpu.SUCCESS and rep["converged"].all()
    for c in range(len(cells)):
        assert _rel(KH[c], g["KH"][c]) <= TOL_KH
        assert _rel(FH[c], g["FH"][c]) <= TOL_KH


@pytest.mark.parametrize("precision", PRECISIONS)
def test_depth3_basis_matches_oracle(gpu, precision):
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=1, depth=3, seed=3)
    cells2, a2, b2, _ = workloads.nedrt_tensor(m=1, depth=1, seed=4)
    _check(gpu, precision, np.concatenate([cells, cells2]), np.concatenate([ainv6, a2]),
           np.concatenate([bdiv, b2]), load)


@pytest.mark.parametrize("precision,ctas_per_sm", [("mixed", 1), ("fp64", 0), ("mixed", 2)])
def test_depth4_global_workspace(gpu, precision, ctas_per_sm):
    """Depth 4 (MINRES workspace in a per-CTA global slot): one 512-thread CTA
    per SM, or (mixed) two 256-thread CTAs per SM."""
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=1, depth=4, seed=6)
    _check(gpu, precision, cells, ainv6, bdiv, load, basis=False, nedrt_ctas_per_sm=ctas_per_sm)


def test_invalid_tensor_rejected(gpu):
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=1, depth=1, seed=1)
    h = gpu.Handle()
    bad = ainv6.copy()
    bad[0, 0] = -1.0
    with pytest.raises(gpu.MsfecError) as e:
        h.nedrt_build(cells, bad, bdiv, load)
    assert e.value.status == gpu.ERROR_NUMERICAL
    c5 = cells.copy()
    c5["depth"] = 5
    with pytest.raises(gpu.MsfecError) as e:
        h.nedrt_build(c5, ainv6, bdiv, load)
    assert e.value.status == gpu.ERROR_INVALID_ARGUMENT


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("depth", [2, 3, 4])
def test_multilevel_preconditioner_matches_diagonal(gpu, precision, depth):
    """The multilevel face preconditioner (default) and the diagonal one give the
    same K_H to the stated tolerance; the multilevel one needs fewer iterations."""
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=1 if depth == 4 else 2, depth=depth, seed=11 + depth)
    out = {}
    for pc in (0, 1):
        h = gpu.Handle(precision=gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64,
                       nedrt_precond=pc)
        KH, FH, rep, st = h.nedrt_build(cells, ainv6, bdiv, load)
        assert st == gpu.SUCCESS and rep["converged"].all(), (pc, rep)
        out[pc] = (KH, FH, rep)
    for c in range(len(cells)):
        assert _rel(out[0][0][c], out[1][0][c]) <= TOL_KH
    if depth <= 3:
        ref = N.build(cells, N.sym6_to_ainv(ainv6), bdiv, load.kind, list(load.params), want_phi=False)
        for c in range(len(cells)):
            assert _rel(out[0][0][c], ref["KH"][c]) <= TOL_KH
    it_ml, it_d = out[0][2]["iterations"].max(), out[1][2]["iterations"].max()
    print(f"{precision} depth {depth}: iterations multilevel {it_ml}, diagonal {it_d}")
    assert it_ml < it_d


def test_multilevel_mixed_depth_batch(gpu):
    """One launch over cells of depths 1-4: every item picks its own level count
    (diagonal only at depth 1) inside the shared multilevel region sized for the
    deepest cell; K_H equals the diagonal-preconditioner build."""
    parts = [workloads.nedrt_tensor(m=1, depth=d, seed=20 + d) for d in (2, 4, 1, 3, 2)]
    cells = np.concatenate([p[0] for p in parts])
    ainv6 = np.concatenate([p[1] for p in parts])
    bdiv = np.concatenate([p[2] for p in parts])
    load = parts[0][3]
    out = {}
    for pc in (0, 1):
        h = gpu.Handle(nedrt_precond=pc)
        KH, FH, rep, st = h.nedrt_build(cells, ainv6, bdiv, load)
        assert st == gpu.SUCCESS and rep["converged"].all(), (pc, rep)
        out[pc] = (KH, FH)
    for c in range(len(cells)):
        assert _rel(out[0][0][c], out[1][0][c]) <= TOL_KH, c
        assert _rel(out[0][1][c], out[1][1][c]) <= TOL_KH, c


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("depth", [2, 3])
def test_constant_diagonal_coefficients_give_the_standard_basis(gpu, precision, depth):
    """Known answer: constant diagonal A^-1 and constant B on a non-cubic box;
    the multiscale basis (primary blocks) is the standard coarse Nedelec / RT
    functions and K_H their Galerkin matrix (the oracle's set_to_std path)."""
    n = 1 << depth
    cells = workloads.coarse_grid(1, depth)
    cells["size"] = [[1.0, 0.8, 1.3]]
    ainv6 = np.tile([0.5, 1.0, 2.0, 0.0, 0.0, 0.0], (n ** 3, 1))
    bdiv = np.full(n ** 3, 1.7)
    h = _handle(gpu, precision)
    KH, FH, rep, st = h.nedrt_build(cells, ainv6, bdiv, gpu.make_load())
    assert st == gpu.SUCCESS and rep["converged"].all(), rep
    S, KHs, _ = N.build_cell(cells["origin"][0], cells["size"][0], depth, N.sym6_to_ainv(ainv6), bdiv, basis="std")
    assert _rel(KH[0], KHs) <= 1e-10, _rel(KH[0], KHs)
    NE, NF = N.counts(n)
    phi = h.nedrt_basis().reshape(18, NE + NF)
    for b in range(18):
        blk = slice(0, NE) if b < 12 else slice(NE, NE + NF)
        assert _rel(phi[b, blk], S[b, blk]) <= TOL_PHI, (b, _rel(phi[b, blk], S[b, blk]))


def test_staged_coefficient_tiles_match_plain_loads(gpu):
    """Cells with the global MINRES workspace (a depth-4 cell in the batch,
    mixed precision): the apply that reads its coefficient tiles from shared
    memory, put there by bulk copies (nedrt_stage 1), gives the plain-load
    build's K_H and F_H up to the rounding of the apply's atomics, on depths
    4, 3, 2, 1 (full, single-round and partly empty warps)."""
    parts = [workloads.nedrt_tensor(m=1, depth=d, seed=40 + d) for d in (4, 3, 2, 1)]
    cells = np.concatenate([p[0] for p in parts])
    ainv6 = np.concatenate([p[1] for p in parts])
    bdiv = np.concatenate([p[2] for p in parts])
    load = parts[0][3]
    out = {}
    for st in (0, 1):
        h = gpu.Handle(nedrt_stage=st)
        KH, FH, rep, status = h.nedrt_build(cells, ainv6, bdiv, load)
        assert status == gpu.SUCCESS and rep["converged"].all(), (st, rep)
        out[st] = (KH, FH, rep)
    for c in range(len(cells)):
        assert _rel(out[1][0][c], out[0][0][c]) <= 1e-11, c
        assert _rel(out[1][1][c], out[0][1][c]) <= 1e-11, c
    print(f"staged: iterations {out[1][2]['iterations'].max()} (plain {out[0][2]['iterations'].max()})")


def test_two_ctas_per_sm_global_workspace_match_one(gpu):
    """A batch whose deepest cell has depth 4 runs every item from a global
    workspace slot; two 256-thread CTAs per SM (nedrt_ctas_per_sm 2) give the
    512-thread build's K_H, F_H and basis up to the rounding of the apply's
    atomics, on depths 4, 3, 2, 1 (full, single-round and partly empty warps)."""
    parts = [workloads.nedrt_tensor(m=1, depth=d, seed=50 + d) for d in (4, 3, 2, 1)]
    cells = np.concatenate([p[0] for p in parts])
    ainv6 = np.concatenate([p[1] for p in parts])
    bdiv = np.concatenate([p[2] for p in parts])
    load = parts[0][3]
    out = {}
    for cps in (1, 2):
        h = gpu.Handle(nedrt_ctas_per_sm=cps)
        KH, FH, rep, status = h.nedrt_build(cells, ainv6, bdiv, load)
        assert status == gpu.SUCCESS and rep["converged"].all(), (cps, rep)
        out[cps] = (KH, FH, rep, h.nedrt_basis())
    for c in range(len(cells)):
        assert _rel(out[2][0][c], out[1][0][c]) <= 1e-11, c
        assert _rel(out[2][1][c], out[1][1][c]) <= 1e-11, c
    assert np.abs(out[2][3] - out[1][3]).max() <= 1e-10 * np.abs(out[1][3]).max()
    print(f"2 CTAs/SM: iterations {out[2][2]['iterations'].max()} (1 CTA/SM {out[1][2]['iterations'].max()})")


@pytest.mark.parametrize("precision", PRECISIONS)
def test_patch_edge_preconditioner_matches_diagonal_edges(gpu, precision):
    """Cells with a global MINRES workspace (depth 4 in the batch, or the FP64
    path at depth 3): the cell-patch edge preconditioner (nedrt_precond 0, the
    default) and diag(M)^-1 on the edges (nedrt_precond 2) give the same K_H,
    F_H and basis, on depths 4, 3, 2, 1, and the patch version needs fewer
    MINRES iterations on the deepest cell."""
    parts = [workloads.nedrt_tensor(m=1, depth=d, seed=60 + d) for d in (4, 3, 2, 1)]
    cells = np.concatenate([p[0] for p in parts])
    ainv6 = np.concatenate([p[1] for p in parts])
    bdiv = np.concatenate([p[2] for p in parts])
    load = parts[0][3]
    out = {}
    for pc in (2, 0):
        h = _handle(gpu, precision, nedrt_precond=pc)
        KH, FH, rep, status = h.nedrt_build(cells, ainv6, bdiv, load)
        assert status == gpu.SUCCESS and rep["converged"].all(), (pc, rep)
        out[pc] = (KH, FH, rep, h.nedrt_basis())
    for c in range(len(cells)):
        assert _rel(out[0][0][c], out[2][0][c]) <= 1e-11, c
        assert _rel(out[0][1][c], out[2][1][c]) <= 1e-11, c
    assert np.abs(out[0][3] - out[2][3]).max() <= 1e-10 * np.abs(out[2][3]).max()
    it0, it2 = out[0][2]["iterations_sum"][0], out[2][2]["iterations_sum"][0]
    print(f"{precision} patch edge block: depth-4 iterations {it0} (diagonal edges {it2})")
    assert it0 < it2


def test_zt_in_shared_memory_matches_global_slot(gpu):
    """Mixed path, depths 4, 3, 2, 1 in one batch (global workspace, multilevel,
    patch edge block): z~ in shared memory (nedrt_zt_place 1) and in the CTA's
    global slot (2) give the same K_H, F_H and basis (to the order of the
    floating-point sums) and the same iteration counts within a few, and the
    shared-memory placement matches the FP64 oracle on the depth-3 cell."""
    parts = [workloads.nedrt_tensor(m=1, depth=d, seed=70 + d) for d in (4, 3, 2, 1)]
    cells = np.concatenate([p[0] for p in parts])
    ainv6 = np.concatenate([p[1] for p in parts])
    bdiv = np.concatenate([p[2] for p in parts])
    load = parts[0][3]
    out = {}
    for zp in (2, 1):
        h = _handle(gpu, "mixed", nedrt_zt_place=zp)
        KH, FH, rep, status = h.nedrt_build(cells, ainv6, bdiv, load)
        assert status == gpu.SUCCESS and rep["converged"].all(), (zp, rep)
        out[zp] = (KH, FH, rep, h.nedrt_basis())
    for c in range(len(cells)):
        assert _rel(out[1][0][c], out[2][0][c]) <= 1e-11, c
        assert _rel(out[1][1][c], out[2][1][c]) <= 1e-11, c
    assert np.abs(out[1][3] - out[2][3]).max() <= 1e-10 * np.abs(out[2][3]).max()
    it1, it2 = out[1][2]["iterations_sum"], out[2][2]["iterations_sum"]
    assert np.abs(it1.astype(np.int64) - it2.astype(np.int64)).max() <= 0.02 * it2.max() + 4, (it1, it2)
    # the depth-3 cell ran through the same launch (z~ in shared memory, sized for depth 4)
    f0 = 8 ** 4
    ref = N.build(cells[1:2], N.sym6_to_ainv(ainv6[f0:f0 + 8 ** 3]), bdiv[f0:f0 + 8 ** 3], load.kind,
                  list(load.params), want_phi=False)
    assert _rel(out[1][0][1], ref["KH"][0]) <= TOL_KH
