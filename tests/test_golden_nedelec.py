"""The reference's only golden vector: Nedelec L2 projection of (1, 2, 3).

test/test_fe_projection_nedelec_mpi.cc projects the constant field (1, 2, 3)
onto FE_Nedelec(0) on the unit cube refined 3 times and prints the DoF values
(golden outputs for 1 and 2 MPI ranks). The oracle restates the lowest-order
edge functional (line integral of the tangential component, tangent along the
positive axis) and deal.II's enumeration (Morton-ordered active cells,
GeometryInfo<3> line order, first-encounter numbering); both golden files
must be reproduced exactly.
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden(k):
    path = os.path.join(HERE, "golden", f"ref_nedelec_projection_mpirun{k}.txt")
    return np.array([float(x) for x in open(path).read().split("\n")[1:] if x.strip()])


def test_nedelec_projection_golden_single_rank(oracle_lib):
    vals = oracle_lib.nedelec_dof_values_unit_cube(3, [1.0, 2.0, 3.0])
    gold = _golden(1)
    assert vals.shape == gold.shape == (1944,)
    assert np.array_equal(vals, gold)


def test_nedelec_projection_golden_two_ranks_prefix(oracle_lib):
    # rank 0 of 2 owns the first half of the Morton-ordered cells: its DoFs are
    # the first 1044 of the global enumeration
    vals = oracle_lib.nedelec_dof_values_unit_cube(3, [1.0, 2.0, 3.0])
    gold = _golden(2)
    assert gold.shape == (1044,)
    assert np.array_equal(vals[:1044], gold)
