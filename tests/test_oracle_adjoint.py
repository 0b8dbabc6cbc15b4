"""The oracle's Q1 adjoint gradient against central finite differences of the
oracle's own J (CPU, FP64 direct solves)."""
import numpy as np

import workloads
from oracle import q1_adjoint


def test_oracle_adjoint_matches_finite_differences(oracle_lib):
    m = 2
    cells, a, _, load = workloads.q1_lognormal(m=m, depth=2, seed=3, reaction=False)
    rng = np.random.default_rng(1)
    npts = 20
    cell_of = rng.integers(0, m ** 3, npts)
    pts = cells["origin"][cell_of] + rng.random((npts, 3)) * cells["size"][cell_of]
    data = 0.01 * rng.standard_normal(npts)
    theta = np.log(a)
    J, grad = q1_adjoint.misfit(cells, m, theta, load, cell_of, pts, data)
    h = 1e-6
    for t in range(3):
        d = rng.standard_normal(theta.shape)
        Jp, _ = q1_adjoint.misfit(cells, m, theta + h * d, load, cell_of, pts, data, gradient=False)
        Jm, _ = q1_adjoint.misfit(cells, m, theta - h * d, load, cell_of, pts, data, gradient=False)
        fd = (Jp - Jm) / (2 * h)
        assert abs(fd - grad @ d) <= 1e-6 * abs(fd)
