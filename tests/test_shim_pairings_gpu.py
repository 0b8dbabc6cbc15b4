"""QNedBasis / RTDQBasis-compatible host shim (mpi-msfec_gb300/host/): the C++
driver example_pairings builds Q_Ned and RT_DQ element matrices per coarse cell
through the shim classes (std::map of basis objects, run(), getters,
set_global_weights, fine solution) and prints checksums; they must equal the
same builds made through the C ABI directly (relative 1e-9: both are GPU
builds of the same inputs; shared-memory atomics make the last bits vary)."""
import json
import subprocess

import numpy as np
import pytest

import workloads

pytestmark = pytest.mark.gpu
M, DEPTH = 2, 2


def _coefs(cells):
    x = workloads.fine_centres(cells)
    a = 1.0 + 0.5 * np.sin(20.0 * x[:, 0]) * np.sin(17.0 * x[:, 1])
    z = np.zeros_like(a)
    return a, z, 1.0 / (1.0 - 0.9 * np.sin(2.0 * np.pi * 14.0 * x[:, 0]))


def _close(a, b, tol=1e-9):
    return abs(a - b) <= tol * max(abs(b), 1e-300)


def test_pairings_shim_matches_c_abi(gpu):
    import msfec_build
    out = subprocess.run([msfec_build.EXAMPLE_PAIR, str(M), str(DEPTH)], capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr
    got = json.loads(out.stdout.strip().splitlines()[-1])
    cells = workloads.coarse_grid(M, DEPTH)
    a, z, binv = _coefs(cells)
    n = 1 << DEPTH
    h = gpu.Handle()
    # Q_Ned: A = a I (curl-curl weight), B^-1 from the sin law, vector trig load
    a6 = np.stack([a, a, a, z, z, z], 1)
    KH, FH, rep, st = h.qned_build(cells, a6, binv, gpu.make_load(gpu.LOAD_VEC_TRIG, (1.0, 1.0, 0.0, 0.0)))
    assert st == gpu.SUCCESS
    phi = h.qned_basis()
    NV, NE = (n + 1) ** 3, 3 * n * (n + 1) ** 2
    P = phi.reshape(len(cells), 20, NV + NE)
    sig = P[:, :8, :NV].sum(1)
    u = P[:, 8:, NV:].sum(1)
    q = got["qned"]
    assert _close(q["KH_abs"], np.abs(KH).sum())
    assert abs(q["KH_sum"] - KH.sum()) <= 1e-9 * np.abs(KH).sum()
    assert abs(q["FH_sum"] - FH.sum()) <= 1e-9 * max(np.abs(FH).sum(), 1e-300)
    assert _close(q["sigma_norm"], np.linalg.norm(sig))
    assert _close(q["u_norm"], np.linalg.norm(u))
    # RT_DQ: A^-1 = I / a, sin-product scalar load
    ainv6 = np.stack([1 / a, 1 / a, 1 / a, z, z, z], 1)
    KH, FH, rep, st = h.rtdq_build(cells, ainv6, gpu.make_load(gpu.LOAD_SIN_PRODUCT, (1.0, 1.0, 0.0, 0.0)))
    assert st == gpu.SUCCESS
    phi = h.rtdq_basis()
    NF, NC = 3 * n * n * (n + 1), n ** 3
    P = phi.reshape(len(cells), 6, NF + NC)
    sig = P[:, :6, :NF].sum(1)
    u = P[:, 0, NF:]  # weight 6 times basis 0's u block (= 1)
    r = got["rtdq"]
    assert _close(r["KH_abs"], np.abs(KH).sum())
    assert abs(r["FH_sum"] - FH.sum()) <= 1e-9 * max(np.abs(FH).sum(), 1e-300)
    assert _close(r["sigma_norm"], np.linalg.norm(sig))
    assert _close(r["u_norm"], np.linalg.norm(u))
    assert np.all(u == 1.0)
