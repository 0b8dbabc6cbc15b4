"""Regenerate the committed golden fixtures under tests/golden/.

1. ref_nedelec_projection_mpirun{1,2}.txt: the values printed by the
   reference's only test (test/test_fe_projection_nedelec_mpi.cc, golden
   outputs test/test_fe_projection_nedelec_mpi.mpirun=1.output / =2.output),
   copied verbatim from the reference checkout (needs the checkout; run here,
   not on the GPU machine).
2. q1_*.npz: FP64 oracle (banded-Cholesky mode) K_H / F_H of seeded Q1
   workloads, the parity target of the CUDA path.
3. nedrt_*.npz: FP64 oracle (sparse direct, SuperLU) K_H / F_H of a seeded
   Ned_RT workload.
4. qned_*.npz, rtdq_*.npz: the same for seeded Q_Ned and RT_DQ workloads.

Usage: python tests/golden/make_golden.py [--reference DIR]
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "mpi-msfec_gb300"))
sys.path.insert(0, REPO)

from oracle import oracle  # noqa: E402
from oracle import nedrt_oracle  # noqa: E402
from oracle import qned_oracle  # noqa: E402
from oracle import rtdq_oracle  # noqa: E402
import workloads  # noqa: E402


def copy_reference_golden(refdir):
    for k in (1, 2):
        src = os.path.join(refdir, "test", f"test_fe_projection_nedelec_mpi.mpirun={k}.output")
        lines = open(src).read().splitlines()
        vals = [ln.strip() for ln in lines if ln.strip() and ln.strip()[0].isdigit()]
        with open(os.path.join(HERE, f"ref_nedelec_projection_mpirun{k}.txt"), "w") as f:
            f.write("# values printed by test/test_fe_projection_nedelec_mpi.cc "
                    f"(reference golden output mpirun={k}), one per line\n")
            f.write("\n".join(vals) + "\n")


def q1_case(name, cells, a, r, load):
    res = oracle.q1_build(cells["origin"], cells["size"], cells["depth"], a, r,
                          load_kind=load.kind, load_params=list(load.params),
                          solver=oracle.SOLVER_DIRECT, want_phi=False)
    assert res["status"] == 0
    np.savez_compressed(os.path.join(HERE, name), KH=res["KH"], FH=res["FH"],
                        depth=cells["depth"])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("MSFEC_REFERENCE_DIR"),
                    help="checkout of konsim83/MPI-MSFEC whose test outputs are copied "
                         "(default: $MSFEC_REFERENCE_DIR; skipped when neither is given)")
    args = ap.parse_args()
    oracle.build()
    if args.reference and os.path.isdir(args.reference):
        copy_reference_golden(args.reference)
    # small Q1 case: coarse 4^3, depth 3, log-normal a, reaction 1, sin load (seed 1)
    q1_case("q1_lognormal_m4_L3_seed1.npz", *workloads.q1_lognormal(m=4, depth=3, seed=1, reaction=True))
    # mixed depths 1..4, no reaction (seed 7)
    cells, a, r, load = workloads.q1_lognormal(m=2, depth=1, seed=7, reaction=False)
    cells["depth"] = [1, 2, 3, 4, 4, 3, 2, 1]
    rng = np.random.default_rng(7)
    nf = int(np.sum(workloads.fine_counts(cells)[0]))
    a = np.exp(rng.standard_normal(nf))
    q1_case("q1_mixed_depths_seed7.npz", cells, a, None, load)
    # Ned_RT: coarse 2^3, depth 2, Haar-rotated log-normal tensor (seed 2)
    cells, ainv6, bdiv, load = workloads.nedrt_tensor(m=2, depth=2, seed=2)
    res = nedrt_oracle.build(cells, nedrt_oracle.sym6_to_ainv(ainv6), bdiv, load.kind, list(load.params),
                             want_phi=False)
    np.savez_compressed(os.path.join(HERE, "nedrt_tensor_m2_L2_seed2.npz"), KH=res["KH"], FH=res["FH"])
    # Q_Ned: coarse 2^3, depth 2, seeded tensor A and B^-1 (seed 4)
    cells, a6, binv, load = workloads.qned_tensor(m=2, depth=2, seed=4)
    res = qned_oracle.build(cells, binv, nedrt_oracle.sym6_to_ainv(a6), load.kind, list(load.params),
                            want_phi=False)
    np.savez_compressed(os.path.join(HERE, "qned_tensor_m2_L2_seed4.npz"), KH=res["KH"], FH=res["FH"])
    # RT_DQ: coarse 2^3, depth 2, seeded tensor A^-1 (seed 6)
    cells, ainv6, load = workloads.rtdq_tensor(m=2, depth=2, seed=6)
    res = rtdq_oracle.build(cells, nedrt_oracle.sym6_to_ainv(ainv6), load.kind, list(load.params), want_phi=False)
    np.savez_compressed(os.path.join(HERE, "rtdq_tensor_m2_L2_seed6.npz"), KH=res["KH"], FH=res["FH"])


if __name__ == "__main__":
    main()
