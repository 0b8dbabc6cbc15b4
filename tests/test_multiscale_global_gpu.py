"""Global multiscale Q1 and Ned_RT solutions from GPU-built K_H/F_H vs the
FP64 oracle's (coarse assembly + solve on the host, the reference's
QMultiscale / NedRTMultiscale flow), and the C++ QBasis-compatible shim driver
on the GPU. Tolerance (stated): relative L2 difference <= 1e-9 of the coarse
solution, and for Ned_RT also of the fine reconstruction sigma_h, u_h."""
import json
import subprocess

import numpy as np
import pytest

import workloads
from test_coarse_solve import coarse_solve, nedrt_coarse_solve

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ("mixed", "fp64"))
def test_global_multiscale_solution_matches_oracle(gpu, oracle_lib, precision):
    m = 4
    cells, a, r, load = workloads.q1_lognormal(m=m, depth=3, seed=1, reaction=True)
    h = gpu.Handle(precision=gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64)
    KH, FH, rep, st = h.q1_build(cells, a, r, load)
    ref = oracle_lib.q1_build(cells["origin"], cells["size"], cells["depth"], a, r, load_kind=load.kind,
                              load_params=list(load.params), want_phi=False)
    U = coarse_solve(m, KH, FH)
    Ur = coarse_solve(m, ref["KH"], ref["FH"])
    rel = np.linalg.norm(U - Ur) / np.linalg.norm(Ur)
    assert rel <= 1e-9, rel


@pytest.mark.parametrize("precision", ("mixed", "fp64"))
def test_global_nedrt_solution_matches_oracle(gpu, precision):
    from oracle import nedrt_adjoint as NA
    from oracle import nedrt_oracle as N
    m, depth = 3, 2
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=m, depth=depth, seed=12)
    h = gpu.Handle(precision=gpu.PRECISION_MIXED if precision == "mixed" else gpu.PRECISION_FP64)
    KH, FH, rep, st = h.nedrt_build(cells, ainv6, bdiv, load)
    assert st == gpu.SUCCESS and rep["converged"].all()
    ref = N.build(cells, N.sym6_to_ainv(ainv6), bdiv, load.kind, list(load.params))
    rng = np.random.default_rng(5)
    # the workload's trig load and a generic face load on top of it; the coarse
    # solve has the reference's natural conditions (every coarse DoF free)
    extra = np.concatenate([np.zeros((m ** 3, 12)), rng.standard_normal((m ** 3, 6))], 1)
    g, _ = NA.coarse_maps(m)
    n = 1 << depth
    NE, NF = N.counts(n)
    phi = h.nedrt_basis().reshape(m ** 3, 18, NE + NF)
    for F_add in (0.0, extra):
        U = nedrt_coarse_solve(m, KH, FH + F_add)
        Ur = nedrt_coarse_solve(m, ref["KH"], ref["FH"] + F_add)
        assert np.linalg.norm(U - Ur) <= 1e-9 * np.linalg.norm(Ur)
        # fine reconstruction (set_global_weights): sigma from edge bases, u from face bases
        sig = np.einsum("ce,ced->cd", U[g[:, :12]], phi[:, :12, :NE])
        sig_r = np.einsum("ce,ced->cd", Ur[g[:, :12]], np.array(ref["Phi"])[:, :12, :NE])
        u = np.einsum("cf,cfd->cd", U[g[:, 12:]], phi[:, 12:, NE:])
        u_r = np.einsum("cf,cfd->cd", Ur[g[:, 12:]], np.array(ref["Phi"])[:, 12:, NE:])
        assert np.linalg.norm(u - u_r) <= 1e-9 * np.linalg.norm(u_r)
        if np.linalg.norm(sig_r) > 1e-12 * np.linalg.norm(u_r):
            assert np.linalg.norm(sig - sig_r) <= 1e-9 * np.linalg.norm(sig_r)


def test_qbasis_shim_example_driver(gpu):
    import msfec_build
    out = subprocess.run([msfec_build.EXAMPLE, "3", "2"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    res = json.loads(out.stdout.strip().splitlines()[-1])
    # the same build through the Python view of the ABI
    cells = workloads.coarse_grid(3, 2)
    cen = workloads.fine_centres(cells)
    acoef = 1.0 + 0.5 * np.sin(20.0 * cen[:, 0]) * np.sin(17.0 * cen[:, 1])
    h = gpu.Handle()
    KH, FH, rep, st = h.q1_build(cells, acoef, None, gpu.make_load(gpu.LOAD_SIN_PRODUCT, (1, 1, 0, 0)))
    assert abs(res["KH0_00"] - KH[0, 0, 0]) <= 1e-12 * abs(KH[0, 0, 0])
    assert res["coarse_cg_iterations"] > 0 and np.isfinite(res["u_centre"])


def test_qbasis_shim_reference_tensor_coefficient(gpu, oracle_lib):
    """The shim driver with the reference's own Q1 coefficient (rotated
    Diffusion_A of prm_q_test-01.prm as a tensor callback, evaluated by the
    shim at the Gauss points): its K_H equals the C ABI's GAUSS-layout build
    and the oracle's quadrature assembly to 1e-10."""
    import msfec_build
    out = subprocess.run([msfec_build.EXAMPLE, "2", "2", "reference"], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    res = json.loads(out.stdout.strip().splitlines()[-1])
    KHs = np.array(res["KH"]).reshape(-1, 8, 8)
    cells, a, r, load = workloads.q1_reference_tensor(m=2, depth=2, gauss=True)
    h = gpu.Handle(q1_coefficient=gpu.Q1_COEF_GAUSS)
    KH, FH, rep, st = h.q1_build(cells, a, r, load)
    ref = oracle_lib.q1_build(cells["origin"], cells["size"], cells["depth"], a, r, load_kind=load.kind,
                              load_params=list(load.params), want_phi=False, coef_mode=oracle_lib.COEF_GAUSS)
    for c in range(len(cells)):
        scale = np.abs(ref["KH"][c]).max()
        assert np.abs(KHs[c] - KH[c]).max() <= 1e-10 * scale
        assert np.abs(KH[c] - ref["KH"][c]).max() <= 1e-10 * scale


def test_nedrtbasis_shim_example_driver(gpu):
    """The C++ NedRTBasis-compatible shim driver (run, getters, host coarse
    solve, set_global_weights, fine sigma/u) against the same build through the
    Python view of the ABI and the host coarse solver."""
    import msfec_build
    m, depth = 2, 2
    out = subprocess.run([msfec_build.EXAMPLE_NR, str(m), str(depth)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    res = json.loads(out.stdout.strip().splitlines()[-1])
    cells = workloads.coarse_grid(m, depth)
    cen = workloads.fine_centres(cells)
    a = 1.0 / (1.0 + 0.5 * np.sin(20.0 * cen[:, 0]) * np.sin(17.0 * cen[:, 1]))
    ainv6 = np.stack([a, a, a, 0 * a, 0 * a, 0 * a], 1)
    bdiv = 1.0 - 0.9 * np.sin(2 * np.pi * 14.0 * cen[:, 0])
    load = gpu.make_load(gpu.LOAD_VEC_TRIG, (1, 1, 0, 0))
    KH, FH, rep, st = gpu.Handle().nedrt_build(cells, ainv6, bdiv, load)
    assert st == gpu.SUCCESS and rep["converged"].all()
    assert abs(res["KH0_1212"] - KH[0, 12, 12]) <= 1e-12 * abs(KH[0, 12, 12])
    U = nedrt_coarse_solve(m, KH, FH, rtol=1e-12)
    assert abs(res["U_norm"] - np.linalg.norm(U)) <= 1e-9 * np.linalg.norm(U)
    assert res["coarse_minres_iterations"] > 0 and res["fine_u_norm"] > 0
