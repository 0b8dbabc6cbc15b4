"""msfec_nedrt_build_noalloc against msfec_nedrt_build_device (C ABI).

The allocation-free entry point serves callers that cannot allocate device
memory mid-build (a pooling allocator that already holds HBM, streams that a
cudaMalloc would stall). It runs the same plan, launch shape, preconditioner,
kernels and item order as the handle-owned build, with every internal buffer
in the library's static per-device pool, so its K_H, F_H and reports must
agree with the existing entry point on the same device inputs. Tolerance: max |diff| <= 1e-11 * max
|entry| per cell. The cell apply accumulates with shared-memory atomics, so
two runs of either entry point differ in the last bits and in the Krylov
iteration counts; both meet nedrt_rtol = 1e-14, which puts K_H within ~1e-14
relative of the converged value. Two calls in a row must both agree, and the
second must leave the device's free memory unchanged. This file is collected
last so that it also runs after every other GPU test.
"""
import numpy as np
import pytest

import workloads

pytestmark = pytest.mark.gpu
TOL = 1e-11
POOL_BYTES = 32 << 20


def _batch(parts):
    cells, ainv6, bdiv = [], [], []
    load = None
    for m, depth, seed in parts:
        c, a, b, load = workloads.nedrt_tensor(m=m, depth=depth, seed=seed)
        cells.append(c)
        ainv6.append(a)
        bdiv.append(b)
    return np.concatenate(cells), np.concatenate(ainv6), np.concatenate(bdiv), load


def _device_inputs(ainv6, bdiv):
    import torch
    return (torch.from_numpy(np.ascontiguousarray(ainv6)).cuda(),
            torch.from_numpy(np.ascontiguousarray(bdiv)).cuda())


def _outputs(ncells):
    import torch
    return (torch.zeros(ncells * 324, dtype=torch.float64, device="cuda"),
            torch.zeros(ncells * 18, dtype=torch.float64, device="cuda"),
            torch.zeros(ncells * 24, dtype=torch.uint8, device="cuda"))


def _host(gpu, out, ncells):
    KH, FH, rep = (t.cpu().numpy() for t in out)
    return KH.reshape(ncells, 18, 18), FH.reshape(ncells, 18), rep.view(gpu.REPORT_DTYPE)


def _agree(a, b):
    for c in range(a.shape[0]):
        scale = max(np.abs(b[c]).max(), 1e-300)
        assert np.abs(a[c] - b[c]).max() <= TOL * scale, c


@pytest.mark.parametrize("precision,parts", [
    # a depth-4 cell takes the global MINRES workspace path (workspace in the pool)
    ("mixed", [(1, 4, 6), (1, 3, 3), (1, 1, 4)]),
    ("fp64", [(1, 3, 3), (2, 2, 2), (1, 1, 4)]),
])
def test_noalloc_matches_device_build(gpu, precision, parts):
    import torch
    cells, ainv6, bdiv, load = _batch(parts)
    n = len(cells)
    h = gpu.Handle(precision=gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64)
    h.set_stream(torch.cuda.current_stream().cuda_stream)
    d_a, d_b = _device_inputs(ainv6, bdiv)
    ref_out = _outputs(n)
    h.nedrt_build_device(cells, d_a.data_ptr(), d_b.data_ptr(), load, *(t.data_ptr() for t in ref_out))
    torch.cuda.synchronize()
    KH0, FH0, rep0 = _host(gpu, ref_out, n)
    assert rep0["converged"].all(), rep0
    outs = [_outputs(n), _outputs(n)]
    free = []
    for out in outs:  # two calls in a row
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        h.nedrt_build_noalloc(cells, d_a.data_ptr(), d_b.data_ptr(), load, *(t.data_ptr() for t in out))
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
    assert free[2] == free[3], f"second call changed free device memory by {free[2] - free[3]} bytes"
    for out in outs:
        KH, FH, rep = _host(gpu, out, n)
        assert rep["converged"].all(), rep
        _agree(KH, KH0)
        _agree(FH, FH0)
        d = max(np.abs(KH[c] - KH0[c]).max() / np.abs(KH0[c]).max() for c in range(n))
        print(f"{precision}: max K_H rel diff {d:.2e}, iterations {rep['iterations'].max()} "
              f"(device build {rep0['iterations'].max()})")


def _high_contrast(ncells, depth, seed, sigma=2.0):
    """Depth-`depth` cells with A^-1 = R diag(e^-g) R^T, g ~ N(0, sigma^2): a
    contrast of e^(+-3 sigma) per axis, harder than the benchmark law."""
    cells, _, bdiv, load = workloads.nedrt_tensor(m=1, depth=depth, seed=seed)
    cells = np.repeat(cells, ncells)
    cells["origin"][:, 0] = np.arange(ncells)  # side by side along x
    rng = np.random.default_rng(seed)
    nf = ncells * 8 ** depth
    g = sigma * rng.standard_normal((nf, 3))
    R = workloads.haar_rotations(rng, nf)
    ainv = np.einsum("cij,cj,ckj->cik", R, np.exp(-g), R)
    ainv6 = np.stack([ainv[:, 0, 0], ainv[:, 1, 1], ainv[:, 2, 2], ainv[:, 0, 1], ainv[:, 0, 2], ainv[:, 1, 2]], 1)
    return cells, ainv6, np.tile(bdiv, ncells), load


def test_noalloc_high_contrast_depth4_converges(gpu):
    """Three depth-4 cells at contrast e^+-6: the multilevel face
    preconditioner converges, iteration counts close to the device build's
    with the same preconditioner (diagonal edge block: nedrt_precond 2), K_H
    within the tolerance."""
    import torch
    cells, ainv6, bdiv, load = _high_contrast(3, 4, seed=11)
    n = len(cells)
    h = gpu.Handle(precision=gpu.PRECISION_MIXED, nedrt_precond=2)
    h.set_stream(torch.cuda.current_stream().cuda_stream)
    d_a, d_b = _device_inputs(ainv6, bdiv)
    ref_out, out = _outputs(n), _outputs(n)
    h.nedrt_build_device(cells, d_a.data_ptr(), d_b.data_ptr(), load, *(t.data_ptr() for t in ref_out))
    h.nedrt_build_noalloc(cells, d_a.data_ptr(), d_b.data_ptr(), load, *(t.data_ptr() for t in out))
    torch.cuda.synchronize()
    KH0, FH0, rep0 = _host(gpu, ref_out, n)
    KH, FH, rep = _host(gpu, out, n)
    assert rep0["converged"].all() and rep["converged"].all(), (rep0, rep)
    _agree(KH, KH0)
    _agree(FH, FH0)
    it0, it1 = int(rep0["iterations"].max()), int(rep["iterations"].max())
    assert it1 <= 1.2 * it0 + 20, (it1, it0)
    print(f"high contrast depth 4: iterations {it1} (device build {it0})")


def test_noalloc_rejects_oversize(gpu):
    import torch
    h = gpu.Handle()
    # five depth-4 cells: Phi and Y alone take 38.8 MB
    cells, ainv6, bdiv, load = _batch([(1, 4, 6)] * 5)
    d_a, d_b = _device_inputs(ainv6, bdiv)
    out = _outputs(len(cells))
    with pytest.raises(gpu.MsfecError) as e:
        h.nedrt_build_noalloc(cells, d_a.data_ptr(), d_b.data_ptr(), load, *(t.data_ptr() for t in out))
    assert e.value.status == gpu.ERROR_INVALID_ARGUMENT
    assert str(POOL_BYTES) in str(e.value) and "split the batch" in str(e.value)
    # more cells than the static cell limit
    many = np.repeat(cells[:1], 4097)
    many["depth"] = 1
    with pytest.raises(gpu.MsfecError) as e:
        h.nedrt_build_noalloc(many, d_a.data_ptr(), d_b.data_ptr(), load, *(t.data_ptr() for t in out))
    assert "4096" in str(e.value)
    torch.cuda.synchronize()
