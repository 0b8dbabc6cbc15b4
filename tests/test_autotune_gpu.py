"""Launch-shape autotuner (msfec_autotune) and the split Q1 launch.

The split launch (cluster kernel for z-slab items, non-cluster kernel for the
rest, concurrently on two streams) runs the same per-item solver, so its K_H,
F_H and reports equal the fused launch bit for bit (the Q1 solver is
deterministic). The autotuner must return a valid candidate with positive
times, and builds after tuning must equal the defaults (Q1 bit for bit,
Ned_RT within 1e-11 relative: shared-memory atomics).
"""
import numpy as np
import pytest

import workloads

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_q1_split_launch_equals_fused(gpu, precision):
    prec = gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64
    cells, a, r, load = workloads.q1_uneven(m=3, seed=4)
    assert set(np.unique(cells["depth"])) >= {4, 5}
    out = {}
    for launch in (1, 2):
        h = gpu.Handle(precision=prec, q1_launch=launch)
        KH, FH, rep, st = h.q1_build(cells, a, None, load)
        assert st == gpu.SUCCESS and rep["converged"].all()
        out[launch] = (KH, FH, rep)
        assert h.timings()["kernel_launches"] == (3 if launch == 1 else 4)
    assert np.array_equal(out[1][0], out[2][0]) and np.array_equal(out[1][1], out[2][1])
    assert np.array_equal(out[1][2]["iterations"], out[2][2]["iterations"])


def test_q1_autotune_then_build(gpu):
    cells, a, _, load = workloads.q1_uneven(m=3, seed=4)
    h = gpu.Handle()
    choice, ncand, times = h.autotune(gpu.KIND_Q1, cells, a, None, load)
    assert ncand == 2 and choice in (0, 1) and all(t > 0 for t in times), (choice, times)
    print(f"q1 autotune: fused {times[0]:.2f} ms, split {times[1]:.2f} ms -> {['fused', 'split'][choice]}")
    KH, FH, rep, st = h.q1_build(cells, a, None, load)
    KH0, FH0, _, _ = gpu.Handle(q1_launch=1).q1_build(cells, a, None, load)
    assert np.array_equal(KH, KH0) and np.array_equal(FH, FH0)
    assert h.timings()["kernel_launches"] == (4 if choice == 1 else 3)


def test_nedrt_autotune_global_workspace(gpu):
    # FP64 depth 3: the workspace lives in global memory, so CTA counts are tuned
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=2, depth=3, seed=2)
    h = gpu.Handle(precision=gpu.PRECISION_FP64)
    choice, ncand, times = h.autotune(gpu.KIND_NEDRT, cells, ainv6, bdiv, load)
    assert ncand == 5 and 0 <= choice < 5 and all(t > 0 for t in times), (choice, times)
    print("nedrt autotune (fp64, depth 3):", [f"{t:.1f}" for t in times], "->", choice)
    KH, FH, rep, st = h.nedrt_build(cells, ainv6, bdiv, load)
    assert st == gpu.SUCCESS and rep["converged"].all()
    KH0, _, _, _ = gpu.Handle(precision=gpu.PRECISION_FP64).nedrt_build(cells, ainv6, bdiv, load)
    for c in range(len(cells)):
        assert _rel(KH[c], KH0[c]) <= 1e-11
    # mixed depth 3 (shared workspace): one 512-thread CTA or two 256-thread CTAs per SM
    h2 = gpu.Handle()
    choice, ncand, times = h2.autotune(gpu.KIND_NEDRT, cells, ainv6, bdiv, load)
    assert ncand == 2 and choice in (0, 1) and all(t > 0 for t in times), (choice, times)
    print("nedrt autotune (mixed, depth 3): 512x1 %.1f ms, 256x2 %.1f ms -> %d" % (times[0], times[1], choice))
    KH2, _, rep2, st2 = h2.nedrt_build(cells, ainv6, bdiv, load)
    KH20, _, _, _ = gpu.Handle().nedrt_build(cells, ainv6, bdiv, load)
    assert st2 == gpu.SUCCESS and rep2["converged"].all()
    for c in range(len(cells)):
        assert _rel(KH2[c], KH20[c]) <= 1e-11


def test_nedrt_autotune_depth4_ctas_and_staging(gpu):
    """Mixed depth 4 (global MINRES workspace): 11 candidates, resident
    512-thread CTAs x coefficient staging, then two 256-thread CTAs per SM; the
    tuned build's K_H equals the default build's."""
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=1, depth=4, seed=6)
    h = gpu.Handle()
    choice, ncand, times = h.autotune(gpu.KIND_NEDRT, cells, ainv6, bdiv, load)
    assert ncand == 11 and 0 <= choice < 11 and all(t > 0 for t in times[:11]), (choice, times)
    print("nedrt autotune (mixed, depth 4): plain", [f"{t:.1f}" for t in times[:5]], "staged",
          [f"{t:.1f}" for t in times[5:10]], "2 CTAs/SM", f"{times[10]:.1f}", "->", choice)
    KH, FH, rep, st = h.nedrt_build(cells, ainv6, bdiv, load)
    assert st == gpu.SUCCESS and rep["converged"].all()
    KH0, FH0, _, _ = gpu.Handle().nedrt_build(cells, ainv6, bdiv, load)
    assert _rel(KH[0], KH0[0]) <= 1e-11 and _rel(FH[0], FH0[0]) <= 1e-11


@pytest.mark.parametrize("kind", ["qned", "rtdq"])
def test_mixed_pairings_autotune_cta_shape(gpu, kind):
    """Q_Ned and RT_DQ (mixed, depth 3): one 512-thread CTA or two 256-thread
    CTAs per SM; both shapes give the same K_H (shared-memory atomics aside)."""
    if kind == "qned":
        cells, a6, binv, load = workloads.qned_tensor(m=2, depth=3, seed=2)
        c0, c1, k = a6, binv, gpu.KIND_QNED
        build = lambda h: h.qned_build(cells, a6, binv, load)  # noqa: E731
    else:
        cells, ainv6, load = workloads.rtdq_tensor(m=2, depth=3, seed=2)
        c0, c1, k = ainv6, None, gpu.KIND_RTDQ
        build = lambda h: h.rtdq_build(cells, ainv6, load)  # noqa: E731
    h = gpu.Handle()
    choice, ncand, times = h.autotune(k, cells, c0, c1, load)
    assert ncand == 2 and choice in (0, 1) and all(t > 0 for t in times), (choice, times)
    print(f"{kind} autotune: 512x1 {times[0]:.1f} ms, 256x2 {times[1]:.1f} ms -> {choice}")
    KH, FH, rep, st = build(h)
    KH0, FH0, _, _ = build(gpu.Handle())
    assert st == gpu.SUCCESS and rep["converged"].all()
    for c in range(len(cells)):
        assert _rel(KH[c], KH0[c]) <= 1e-11
