"""QStd / NedRTStd-compatible host shim (mpi-msfec_gb300/host/): the C++
driver example_std runs both standard fine-scale solves on the unit cube
through the shim classes and prints solution norms and point values; they must
equal the same solves made through the C ABI directly (relative 1e-9: both are
GPU solves of the same inputs; shared-memory atomics make the last bits vary),
and the point values the trilinear (Q1) / lowest-order RT (Ned_RT)
interpolation of those solutions."""
import json
import subprocess

import numpy as np
import pytest

import workloads

pytestmark = pytest.mark.gpu
RQ, RN = 4, 3  # n_refine of the Q1 and Ned_RT solves
PROBE = np.array([0.3, 0.55, 0.7])


def _a(x):
    return 1.0 + 0.5 * np.sin(20.0 * x[:, 0]) * np.sin(17.0 * x[:, 1])


def _lattice(n):
    s = PROBE * n
    c = np.minimum(s.astype(int), n - 1)
    return c, s - c


def test_std_shim_matches_c_abi(gpu):
    import msfec_build
    out = subprocess.run([msfec_build.EXAMPLE_STD, str(RQ), str(RN)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    got = json.loads(out.stdout.strip().splitlines()[-1])
    h = gpu.Handle()
    # Q1: a from the sin law, sin-product load, homogeneous Dirichlet data
    dom = workloads.coarse_grid(1, RQ)
    u, rep, st = h.q1_fine_solve(dom, _a(workloads.fine_centres(dom)), None,
                                 gpu.make_load(gpu.LOAD_SIN_PRODUCT, (1.0, 1.0, 0.0, 0.0)))
    assert st == gpu.SUCCESS
    assert abs(got["q_u_norm"] - np.linalg.norm(u)) <= 1e-9 * np.linalg.norm(u)
    n = 1 << RQ
    c, t = _lattice(n)
    U = u.reshape(n + 1, n + 1, n + 1)  # [k][j][i]
    val = sum((t[0] if a else 1 - t[0]) * (t[1] if b else 1 - t[1]) * (t[2] if e else 1 - t[2]) *
              U[c[2] + e, c[1] + b, c[0] + a] for a in (0, 1) for b in (0, 1) for e in (0, 1))
    assert abs(got["q_u_probe"] - val) <= 1e-9 * np.abs(u).max()
    # Ned_RT: A^-1 = I / a, B from the sin law, vector trig load, natural conditions
    dom = workloads.coarse_grid(1, RN)
    x = workloads.fine_centres(dom)
    ai = 1.0 / _a(x)
    z = np.zeros_like(ai)
    bdiv = 1.0 - 0.9 * np.sin(2.0 * np.pi * 14.0 * x[:, 0])
    xs, rep, st = h.nedrt_fine_solve(dom, np.stack([ai, ai, ai, z, z, z], 1), bdiv,
                                     gpu.make_load(gpu.LOAD_VEC_TRIG, (1.0, 1.0, 0.0, 0.0)))
    assert st == gpu.SUCCESS
    n = 1 << RN
    NE = 3 * n * (n + 1) ** 2
    sig, uf = xs[:NE], xs[NE:]
    assert abs(got["nedrt_sigma_norm"] - np.linalg.norm(sig)) <= 1e-9 * np.linalg.norm(sig)
    assert abs(got["nedrt_u_norm"] - np.linalg.norm(uf)) <= 1e-9 * np.linalg.norm(uf)
    Fx = (n + 1) * n * n
    c, t = _lattice(n)

    def face(d, i, j, k):
        return [i + (n + 1) * (j + n * k), Fx + i + n * (j + (n + 1) * k), 2 * Fx + i + n * (j + n * k)][d]

    area = 1.0 / (n * n)
    for d in range(3):
        hi = c.copy()
        hi[d] += 1
        v = ((1 - t[d]) * uf[face(d, *c)] + t[d] * uf[face(d, *hi)]) / area
        assert abs(got["nedrt_u_probe"][d] - v) <= 1e-9 * np.abs(uf).max() / area
