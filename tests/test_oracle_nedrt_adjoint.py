"""CPU check of the Ned_RT adjoint oracle (oracle/nedrt_adjoint.py) against
central finite differences of its own forward misfit, on a coarse 3^3 grid
where the coarse solution has an edge part, so that dJ/d log A does not
vanish (on the 2^3 grid of the GPU adjoint tests it vanishes to rounding).
Tolerance (stated): |fd - g.d| <= 1e-6 * sum_i |g_i d_i| (h = 1e-5)."""
import numpy as np

import workloads
from oracle import nedrt_adjoint as NA
from oracle import nedrt_oracle as N


def test_nedrt_adjoint_oracle_matches_finite_differences():
    m, depth = 3, 1
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=m, depth=depth, seed=5)
    ainv = N.sym6_to_ainv(ainv6)
    rng = np.random.default_rng(1)
    pts = rng.uniform(0.02, 0.98, (30, 3))
    ci = np.minimum((pts * m).astype(int), m - 1)
    cell_of = ci[:, 0] + m * (ci[:, 1] + m * ci[:, 2])
    data = rng.standard_normal((30, 3)) * 0.1
    nf = len(bdiv)
    ta, tb = np.zeros(nf), np.zeros(nf)
    args = (load.kind, list(load.params), cell_of, pts, data)
    _, ga, gb = NA.misfit(cells, m, ainv, bdiv, ta, tb, *args)
    assert np.abs(ga).max() > 1e-2 * np.abs(gb).max()  # the A gradient is not trivially zero here
    h = 1e-5
    for _ in range(3):
        for which in ("a", "b"):
            d = rng.standard_normal(nf)
            da, db = (d, 0 * d) if which == "a" else (0 * d, d)
            g = ga if which == "a" else gb
            Jp = NA.misfit(cells, m, ainv, bdiv, ta + h * da, tb + h * db, *args, gradient=False)[0]
            Jm = NA.misfit(cells, m, ainv, bdiv, ta - h * da, tb - h * db, *args, gradient=False)[0]
            fd = (Jp - Jm) / (2 * h)
            assert abs(fd - g @ d) <= 1e-6 * np.abs(g * d).sum(), (which, fd, g @ d)
