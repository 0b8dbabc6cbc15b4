"""GPU parity of the RT_DQ (RT0 sigma x DQ0 u) basis build against the FP64
oracle (C ABI). Stated tolerances (both precisions; mixed = FP32 MINRES +
FP64 refinement): K_H, F_H max abs error <= 1e-10 * max |entry| of the cell;
sigma of every basis max|phi - phi_oracle| <= 1e-8 * max|phi_oracle|; the
stored u block is exactly 1 (the reference's set_u_to_std)."""

import numpy as np
import pytest

import workloads
from oracle import nedrt_oracle as NR
from oracle import rtdq_oracle as RQ

pytestmark = pytest.mark.gpu
TOL_KH = 1e-10
TOL_PHI = 1e-10


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _check(gpu, h, cells, ainv6, load, KH, FH):
    ref = RQ.build(cells, NR.sym6_to_ainv(ainv6), load.kind, list(load.params))
    for c in range(len(cells)):
        assert _rel(KH[c], ref["KH"][c]) <= TOL_KH, (c, _rel(KH[c], ref["KH"][c]))
        assert _rel(FH[c], ref["FH"][c]) <= TOL_KH, (c, FH[c], ref["FH"][c])
    phi = h.rtdq_basis()
    off = 0
    for c, po in enumerate(ref["Phi"]):
        n = 1 << int(cells["depth"][c])
        NF, _ = RQ.counts(n)
        pg = phi[off:off + po.size].reshape(po.shape)
        off += po.size
        for b in range(6):
            assert _rel(pg[b, :NF], po[b, :NF]) <= TOL_PHI, (c, b, _rel(pg[b, :NF], po[b, :NF]))
            assert np.all(pg[b, NF:] == 1.0)
    assert off == phi.size
    return max(_rel(KH[c], ref["KH"][c]) for c in range(len(cells)))


@pytest.mark.parametrize("precision", ("mixed", "fp64"))
@pytest.mark.parametrize("m,depth", [(1, 1), (2, 2), (1, 3)])
def test_rtdq_basis_matches_oracle(gpu, precision, m, depth):
    cells, ainv6, load = workloads.rtdq_tensor(m=m, depth=depth, seed=3 + depth)
    h = gpu.Handle(precision=gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64)
    KH, FH, rep, st = h.rtdq_build(cells, ainv6, load)
    assert st == gpu.SUCCESS and rep["converged"].all(), rep
    err = _check(gpu, h, cells, ainv6, load, KH, FH)
    print(f"{precision} depth {depth}: max K_H rel err {err:.2e}, max iterations {rep['iterations'].max()}")


def test_rtdq_mixed_depths_constant_load(gpu):
    cells, ainv6, _ = workloads.rtdq_tensor(m=2, depth=2, seed=9)
    cells["depth"] = np.array([1, 3, 2, 2, 3, 1, 2, 2], dtype=np.int32)
    nf = int(np.sum((1 << cells["depth"].astype(np.int64)) ** 3))
    rng = np.random.default_rng(9)
    Rr = workloads.haar_rotations(rng, nf)
    ainv = np.einsum("cij,cj,ckj->cik", Rr, np.exp(rng.standard_normal((nf, 3))), Rr)
    ainv6 = NR.ainv_to_sym6(ainv)
    load = gpu.make_load(gpu.LOAD_CONSTANT, (2.5, 0.0, 0.0, 0.0))
    h = gpu.Handle()
    KH, FH, rep, st = h.rtdq_build(cells, ainv6, load)
    assert st == gpu.SUCCESS and rep["converged"].all(), rep
    _check(gpu, h, cells, ainv6, load, KH, FH)
    vol = np.prod(cells["size"], axis=1)
    assert np.allclose(FH[:, 6], 2.5 * vol, rtol=1e-13)


def test_rtdq_device_entry_matches_host(gpu):
    import torch
    cells, ainv6, load = workloads.rtdq_tensor(m=2, depth=2, seed=4)
    h = gpu.Handle()
    KH, FH, rep, st = h.rtdq_build(cells, ainv6, load)
    nc = len(cells)
    d_a = torch.from_numpy(ainv6).cuda()
    d_KH = torch.zeros((nc, 7, 7), dtype=torch.float64, device="cuda")
    d_FH = torch.zeros((nc, 7), dtype=torch.float64, device="cuda")
    h.rtdq_build_device(cells, d_a.data_ptr(), load, d_KH.data_ptr(), d_FH.data_ptr(), 0)
    torch.cuda.synchronize()
    assert _rel(d_KH.cpu().numpy(), KH) <= TOL_KH
    assert _rel(d_FH.cpu().numpy(), FH) <= TOL_KH


def test_rtdq_rejects_bad_input(gpu):
    cells, ainv6, _ = workloads.rtdq_tensor(m=1, depth=2, seed=1)
    h = gpu.Handle()
    vec = gpu.make_load(gpu.LOAD_VEC_TRIG, (1.0, 1.0, 0.0, 0.0))
    with pytest.raises(gpu.MsfecError):
        h.rtdq_build(cells, ainv6, vec)
    bad = ainv6.copy()
    bad[5, 0] = -1.0
    with pytest.raises(gpu.MsfecError):
        h.rtdq_build(cells, bad, gpu.make_load(gpu.LOAD_ZERO, (0, 0, 0, 0)))
    deep = cells.copy()
    deep["depth"] = 5
    with pytest.raises(gpu.MsfecError):
        h.rtdq_build(deep, np.tile(ainv6, (64, 1)), gpu.make_load(gpu.LOAD_ZERO, (0, 0, 0, 0)))
    KH, FH, rep, st = h.rtdq_build(cells[:0], ainv6[:0], gpu.make_load(gpu.LOAD_ZERO, (0, 0, 0, 0)))
    assert st == gpu.SUCCESS and KH.shape == (0, 7, 7)


@pytest.mark.parametrize("precision", ("mixed", "fp64"))
def test_rtdq_matches_golden(gpu, precision):
    """GPU build against the committed oracle fixture (coarse 2^3 x depth 2,
    tests/golden/make_golden.py), same per-cell tolerance as above."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rtdq_tensor_m2_L2_seed6.npz"))
    cells, ainv6, load = workloads.rtdq_tensor(m=2, depth=2, seed=6)
    h = gpu.Handle(precision=gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64)
    KH, FH, rep, st = h.rtdq_build(cells, ainv6, load)
    assert st == gpu.SUCCESS and rep["converged"].all(), rep
    for c in range(len(cells)):
        assert _rel(KH[c], g["KH"][c]) <= TOL_KH, (c, _rel(KH[c], g["KH"][c]))
        assert _rel(FH[c], g["FH"][c]) <= TOL_KH, (c, _rel(FH[c], g["FH"][c]))


@pytest.mark.parametrize("precision", ("mixed", "fp64"))
def test_rtdq_constant_diagonal_gives_the_standard_basis(gpu, precision):
    """Known answer: constant diagonal A^-1 on a non-cubic box; sigma of every
    basis is the standard coarse RT function."""
    depth, n = 3, 8
    cells = workloads.coarse_grid(1, depth)
    cells["size"] = [[1.0, 0.8, 1.3]]
    ainv6 = np.tile([0.5, 1.0, 2.0, 0.0, 0.0, 0.0], (n ** 3, 1))
    h = gpu.Handle(precision=gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64)
    KH, FH, rep, st = h.rtdq_build(cells, ainv6, gpu.make_load(gpu.LOAD_ZERO, (0, 0, 0, 0)))
    assert st == gpu.SUCCESS and rep["converged"].all(), rep
    NF, NC = RQ.counts(n)
    phi = h.rtdq_basis().reshape(6, NF + NC)
    for f in range(6):
        std = NR.coarse_face_dofs(n, f)
        assert _rel(phi[f, :NF], std) <= TOL_PHI, (f, _rel(phi[f, :NF], std))
