"""GPU parity at the benchmark's scale: the full seeded batches of the
workloads, built on the GPU through the C ABI in one call each, against the
FP64 oracle on a stratified sample of their cells (every refinement depth
represented; oracle.parity).

Workloads (seeded, the benchmark's generators):
  Ned_RT coarse 8^3 x depth 3 (512 cells, seed 2): 32 cells spread over the batch
  Q1 uneven coarse 16^3, depth U{2..5} (4096 cells, seed 3): 3 cells of each
     of depths 2-4 and 2 of depth 5 (the depth-5 cells run as cluster z-slabs)
  Q1 coarse 8^3 x depth 4, log a ~ N(0,1) (512 cells, seed 4): 4 cells
  Ned_RT coarse 16^3 x depth 4 (4096 cells, seed 5; 1.99e9 basis values, so
     64-bit offsets): first, middle and last cell. The mixed path builds the
     whole batch; the FP64 path builds the three sampled cells as a batch of
     their own (the whole batch would take minutes in FP64).
Tolerances, stated in the test (relative to the largest entry of the cell /
of the basis function):
  FP64 path:  K_H, F_H, every basis function <= 1e-10
  mixed path (FP32 Krylov + FP64 refinement to the same residual): <= 1e-10
"""
import numpy as np
import pytest

import workloads
from oracle import parity

pytestmark = pytest.mark.gpu
TOL = {"fp64": 1e-10, "mixed": 1e-10}
PRECISIONS = ("mixed", "fp64")

_CACHE = {}


def _handle(gpu, precision):
    return gpu.Handle(precision=gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64)


def _nedrt_case(name):
    """(cells, ainv6, bdiv, load, sample) with the oracle started asynchronously."""
    if name not in _CACHE:
        if name == "nedrt_8x3":
            cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=8, depth=3, seed=2)
            sel = parity.stratified_sample(cells, 32)
        else:
            cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=16, depth=4, seed=5)
            sel = parity.stratified_sample(cells, 3)
        _CACHE[name] = (cells, ainv6, bdiv, load, parity.OracleSample("nedrt", cells, sel, (ainv6, bdiv), load))
    return _CACHE[name]


def _q1_case(name):
    if name not in _CACHE:
        if name == "q1_uneven":
            cells, a, r, load = workloads.q1_uneven(m=16, seed=3)
            sel = parity.stratified_sample(cells, {2: 3, 3: 3, 4: 3, 5: 2})
        else:
            cells, a, r, load = workloads.q1_lognormal(m=8, depth=4, seed=4, reaction=False)
            sel = parity.stratified_sample(cells, 4)
        _CACHE[name] = (cells, a, r, load, parity.OracleSample("q1", cells, sel, (a, r), load))
    return _CACHE[name]


def _report(tag, precision, err, rep):
    print(f"{tag} {precision}: {err['cells']} cells, max rel K_H {err['KH_max_rel']:.2e}, "
          f"F_H {err['FH_max_rel']:.2e}, Phi {err['Phi_max_rel']:.2e}, max iterations "
          f"{int(rep['iterations'].max())}")


def _assert_within(err, tol):
    for pc in err["per_cell"]:
        assert pc["KH"] <= tol and pc["FH"] <= tol, pc
        if pc["Phi"] is not None:
            assert pc["Phi"] <= tol, pc


@pytest.mark.parametrize("precision", PRECISIONS)
def test_nedrt_8x3_batch_sample(gpu, precision):
    cells, ainv6, bdiv, load, sample = _nedrt_case("nedrt_8x3")
    h = _handle(gpu, precision)
    KH, FH, rep, st = h.nedrt_build(cells, ainv6, bdiv, load)
    assert st == gpu.SUCCESS and rep["converged"].all()
    err = parity.compare(sample, KH, FH, lambda c: h.nedrt_basis_cells(cells, c, 1)[0])
    _report("Ned_RT 8^3 x L3", precision, err, rep)
    _assert_within(err, TOL[precision])


@pytest.mark.parametrize("precision", PRECISIONS)
def test_q1_uneven_batch_sample(gpu, precision):
    cells, a, r, load, sample = _q1_case("q1_uneven")
    assert (cells["depth"][sample.sel] == 5).sum() >= 2
    h = _handle(gpu, precision)
    KH, FH, rep, st = h.q1_build(cells, a, r, load)
    assert st == gpu.SUCCESS and rep["converged"].all()
    err = parity.compare(sample, KH, FH, lambda c: h.q1_basis_cells(cells, c, 1)[0])
    _report("Q1 uneven 16^3 x L2-5", precision, err, rep)
    _assert_within(err, TOL[precision])


@pytest.mark.parametrize("precision", PRECISIONS)
def test_q1_8x4_batch_sample(gpu, precision):
    cells, a, r, load, sample = _q1_case("q1_8x4")
    h = _handle(gpu, precision)
    KH, FH, rep, st = h.q1_build(cells, a, r, load)
    assert st == gpu.SUCCESS and rep["converged"].all()
    err = parity.compare(sample, KH, FH, lambda c: h.q1_basis_cells(cells, c, 1)[0])
    _report("Q1 8^3 x L4", precision, err, rep)
    _assert_within(err, TOL[precision])


def test_nedrt_16x4_full_batch_mixed(gpu):
    """The whole coarse 16^3 x depth 4 batch in one build (mixed precision)."""
    cells, ainv6, bdiv, load, sample = _nedrt_case("nedrt_16x4")
    h = _handle(gpu, "mixed")
    KH, FH, rep, st = h.nedrt_build(cells, ainv6, bdiv, load)
    assert st == gpu.SUCCESS and rep["converged"].all()
    err = parity.compare(sample, KH, FH, lambda c: h.nedrt_basis_cells(cells, c, 1)[0])
    _report("Ned_RT 16^3 x L4 (whole batch)", "mixed", err, rep)
    _assert_within(err, TOL["mixed"])


def test_nedrt_16x4_sampled_cells_fp64(gpu):
    """The sampled cells of the coarse 16^3 x depth 4 batch as a batch of their
    own, plain FP64 path."""
    cells, ainv6, bdiv, load, sample = _nedrt_case("nedrt_16x4")
    sl = parity.fine_slices(cells, sample.sel)
    sub = cells[sample.sel]
    a = np.concatenate([ainv6[f0:f1] for f0, f1 in sl])
    b = np.concatenate([bdiv[f0:f1] for f0, f1 in sl])
    h = _handle(gpu, "fp64")
    KHs, FHs, rep, st = h.nedrt_build(sub, a, b, load)
    assert st == gpu.SUCCESS and rep["converged"].all()
    KH = np.zeros((len(cells), 18, 18))
    FH = np.zeros((len(cells), 18))
    KH[sample.sel], FH[sample.sel] = KHs, FHs
    pos = {int(c): i for i, c in enumerate(sample.sel)}
    err = parity.compare(sample, KH, FH, lambda c: h.nedrt_basis_cells(sub, pos[c], 1)[0])
    _report("Ned_RT 16^3 x L4 (sampled cells)", "fp64", err, rep)
    _assert_within(err, TOL["fp64"])
