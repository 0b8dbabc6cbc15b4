"""GPU parity of the Q1 basis build against the FP64 oracle (through the C ABI).

Tolerances (FP64 path and mixed FP32-PCG + FP64 refinement path alike):
  basis functions  max|phi - phi_oracle| <= 1e-10 * max|phi_oracle| per function
  K_H, F_H         max abs error <= 1e-10 * max |entry| of the cell
"""
import os

import numpy as np
import pytest

import workloads

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
TOL = 1e-10
PRECISIONS = ("mixed", "fp64")


def _handle(gpu, precision):
    p = gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64
    return gpu.Handle(precision=p)


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _split_phi(phi, cells):
    out, off = [], 0
    for c in cells:
        n = 1 << int(c["depth"])
        sz = 8 * (n + 1) ** 3
        out.append(phi[off:off + sz].reshape(8, -1))
        off += sz
    return out


def _check_against_oracle(gpu, oracle_lib, precision, cells, a, r, load, basis=True):
    h = _handle(gpu, precision)
    KH, FH, rep, st = h.q1_build(cells, a, r, load)
    assert st == gpu.SUCCESS
    assert rep["converged"].all()
    ref = oracle_lib.q1_build(cells["origin"], cells["size"], cells["depth"], a, r,
                              load_kind=load.kind, load_params=list(load.params), want_phi=basis)
    assert ref["status"] == 0
    for c in range(len(cells)):
        assert _rel(KH[c], ref["KH"][c]) <= TOL, (c, _rel(KH[c], ref["KH"][c]))
        if np.abs(ref["FH"][c]).max() > 0:
            assert _rel(FH[c], ref["FH"][c]) <= TOL
    if basis:
        phi = h.q1_basis()
        for c, (pg, po) in enumerate(zip(_split_phi(phi, cells), _split_phi(ref["Phi"], cells))):
            for v in range(8):
                assert _rel(pg[v], po[v]) <= TOL, (c, v, _rel(pg[v], po[v]))
    return KH, FH, rep


@pytest.mark.parametrize("precision", PRECISIONS)
def test_small_lognormal_with_reaction_matches_golden(gpu, oracle_lib, precision):
    cells, a, r, load = workloads.q1_lognormal(m=4, depth=3, seed=1, reaction=True)
    g = np.load(os.path.join(HERE, "golden", "q1_lognormal_m4_L3_seed1.npz"))
    h = _handle(gpu, precision)
    KH, FH, rep, st = h.q1_build(cells, a, r, load)
    assert st == gpu.SUCCESS and rep["converged"].all()
    for c in range(len(cells)):
        assert _rel(KH[c], g["KH"][c]) <= TOL
        assert _rel(FH[c], g["FH"][c]) <= TOL


@pytest.mark.parametrize("precision", PRECISIONS)
def test_basis_functions_match_oracle(gpu, oracle_lib, precision):
    cells, a, r, load = workloads.q1_lognormal(m=2, depth=3, seed=4, reaction=True)
    _check_against_oracle(gpu, oracle_lib, precision, cells, a, r, load)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_mixed_depths_1_to_4(gpu, oracle_lib, precision):
    g = np.load(os.path.join(HERE, "golden", "q1_mixed_depths_seed7.npz"))
    cells, _, _, load = workloads.q1_lognormal(m=2, depth=1, seed=7, reaction=False)
    cells["depth"] = g["depth"]
    rng = np.random.default_rng(7)
    a = np.exp(rng.standard_normal(int(np.sum(workloads.fine_counts(cells)[0]))))
    h = _handle(gpu, precision)
    KH, FH, rep, st = h.q1_build(cells, a, None, load)
    assert st == gpu.SUCCESS and rep["converged"].all()
    for c in range(len(cells)):
        assert _rel(KH[c], g["KH"][c]) <= TOL, (c, cells["depth"][c], _rel(KH[c], g["KH"][c]))
        assert _rel(FH[c], g["FH"][c]) <= TOL


@pytest.mark.parametrize("precision", PRECISIONS)
def test_depth5_cluster_slabs(gpu, oracle_lib, precision):
    # depth-5 cells run as z-slabs over a cluster of 8 CTAs (DSMEM halos)
    cells, a, r, load = workloads.q1_lognormal(m=1, depth=5, seed=9, reaction=False)
    cells2, a2, _, _ = workloads.q1_lognormal(m=1, depth=4, seed=10, reaction=False)
    allc = np.concatenate([cells, cells2])
    alla = np.concatenate([a, a2])
    _check_against_oracle(gpu, oracle_lib, precision, allc, alla, None, load)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_constant_coefficient_known_answer(gpu, precision):
    cells = workloads.coarse_grid(2, [1, 2, 3, 4, 5, 3, 2, 1])
    nf = int(np.sum(workloads.fine_counts(cells)[0]))
    h = _handle(gpu, precision)
    KH, FH, rep, st = h.q1_build(cells, np.full(nf, 3.0), None, gpu.make_load())
    assert st == gpu.SUCCESS
    H = 0.5
    Kc = np.zeros((8, 8))
    for u in range(8):
        for v in range(8):
            d = bin(u ^ v).count("1")
            Kc[u, v] = {0: H / 3, 1: 0.0, 2: -H / 12, 3: -H / 12}[d]
    for c in range(len(cells)):
        assert np.abs(KH[c] - 3.0 * Kc).max() <= TOL * H
    phi = h.q1_basis()
    for c, pg in enumerate(_split_phi(phi, cells)):
        n = 1 << int(cells["depth"][c])
        t = np.arange(n + 1) / n
        z, y, x = np.meshgrid(t, t, t, indexing="ij")
        for v in range(8):
            f = np.ones_like(x)
            for d, T in enumerate((x, y, z)):
                f = f * (T if (v >> d) & 1 else 1 - T)
            assert np.abs(pg[v] - f.ravel()).max() < 1e-12


@pytest.mark.parametrize("precision", PRECISIONS)
def test_partition_of_unity(gpu, precision):
    cells, a, _, load = workloads.q1_lognormal(m=2, depth=4, seed=12, reaction=False)
    h = _handle(gpu, precision)
    KH, FH, rep, st = h.q1_build(cells, a, None, load)
    for c in range(len(cells)):
        assert np.abs(KH[c].sum(axis=1)).max() <= TOL * np.abs(KH[c]).max()
        assert np.abs(KH[c] - KH[c].T).max() <= TOL * np.abs(KH[c]).max()


def test_device_entry_point_matches_host_entry_point(gpu):
    import torch
    cells, a, r, load = workloads.q1_lognormal(m=2, depth=3, seed=3, reaction=True)
    h = gpu.Handle(precision=gpu.PRECISION_MIXED)
    KH, FH, rep, _ = h.q1_build(cells, a, r, load)
    da = torch.from_numpy(a).cuda()
    dr = torch.from_numpy(r).cuda()
    dK = torch.zeros((len(cells), 8, 8), dtype=torch.float64, device="cuda")
    dF = torch.zeros((len(cells), 8), dtype=torch.float64, device="cuda")
    drep = torch.zeros(len(cells) * gpu.REPORT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    h.set_stream(s.cuda_stream)
    h.q1_build_device(cells, da.data_ptr(), dr.data_ptr(), load, dK.data_ptr(), dF.data_ptr(),
                      drep.data_ptr())
    s.synchronize()
    assert np.array_equal(dK.cpu().numpy(), KH)
    assert np.array_equal(dF.cpu().numpy(), FH)
    rep2 = np.frombuffer(drep.cpu().numpy().tobytes(), dtype=gpu.REPORT_DTYPE)
    assert (rep2["converged"] == 1).all()


def test_eval_fine_reconstruction(gpu):
    cells, a, r, load = workloads.q1_lognormal(m=2, depth=2, seed=8, reaction=False)
    h = gpu.Handle()
    h.q1_build(cells, a, None, load)
    phi = _split_phi(h.q1_basis(), cells)
    rng = np.random.default_rng(0)
    U = rng.standard_normal((len(cells), 8))
    npts = 200
    cell_of = rng.integers(0, len(cells), npts).astype(np.int32)
    t = rng.random((npts, 3))
    pts = cells["origin"][cell_of] + t * cells["size"][cell_of]
    vals = h.q1_eval_fine(U, cell_of, pts)
    for p in range(npts):
        c = cell_of[p]
        n = 1 << int(cells["depth"][c])
        u = U[c] @ phi[c]  # fine nodal values
        s = t[p] * n
        f = np.minimum(np.floor(s).astype(int), n - 1)
        xi = s - f
        acc = 0.0
        for corner in range(8):
            cx, cy, cz = corner & 1, (corner >> 1) & 1, corner >> 2
            w = (xi[0] if cx else 1 - xi[0]) * (xi[1] if cy else 1 - xi[1]) * (xi[2] if cz else 1 - xi[2])
            acc += w * u[(f[0] + cx) + (n + 1) * ((f[1] + cy) + (n + 1) * (f[2] + cz))]
        assert abs(vals[p] - acc) < 1e-12


def test_invalid_inputs_are_reported_not_trapped(gpu):
    cells, a, r, load = workloads.q1_lognormal(m=1, depth=2, seed=1, reaction=False)
    h = gpu.Handle()
    bad = a.copy()
    bad[3] = -1.0
    with pytest.raises(gpu.MsfecError) as e:
        h.q1_build(cells, bad, None, load)
    assert e.value.status == gpu.ERROR_NUMERICAL
    bad[3] = np.nan
    with pytest.raises(gpu.MsfecError) as e:
        h.q1_build(cells, bad, None, load)
    assert e.value.status == gpu.ERROR_NUMERICAL
    cz = cells.copy()
    cz["depth"] = 0
    with pytest.raises(gpu.MsfecError) as e:
        h.q1_build(cz, a, None, load)
    assert e.value.status == gpu.ERROR_INVALID_ARGUMENT
    # a valid call afterwards still works on the same handle
    KH, FH, rep, st = h.q1_build(cells, a, None, load)
    assert st == gpu.SUCCESS
