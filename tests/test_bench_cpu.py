"""CPU checks of bench.py's host logic: the autotuner candidate names match the
candidate counts msfec_autotune reports (include/msfec_cuda.h), and the CPU
baseline sample of the depth-4 headline workload is whole rounds of one cell
per worker, every depth represented."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_shape_names_match_candidate_counts():
    assert bench.shape_names("q1", 2) == ["fused", "split"]
    assert bench.shape_names("qned", 2) == ["152x512", "304x256"]
    assert bench.shape_names("nedrt", 2) == ["152x512", "304x256"]
    assert len(bench.shape_names("nedrt", 5)) == 5  # FP64 global workspace: resident CTAs
    names = bench.shape_names("nedrt", 11)  # mixed global workspace
    assert len(names) == 11 and len(set(names)) == 11
    assert names[0] == "152x512" and names[5] == "152x512+stage" and names[10] == "304x256"
    assert bench.shape_names("rtdq", 1) == ["default"]


class _Cells:
    """The fields of a benchmark workload that cpu_sample reads."""

    def __init__(self, kind, depths):
        import workloads
        self.kind = kind
        self.cells = workloads.coarse_grid(round(len(depths) ** (1 / 3)), list(depths))


def test_cpu_sample_whole_rounds():
    wl = _Cells("nedrt", [4] * 512)  # a batch of the depth-4 headline workload (~10 s per cell)
    for target, workers in ((10.0, 16), (20.0, 16), (10.0, 8)):
        sel = bench.cpu_sample(wl, target, workers, 0, 512)
        assert len(sel) % workers == 0 and len(sel) >= workers, (target, workers, len(sel))
        assert np.all((sel >= 0) & (sel < 512))
    mixed = _Cells("q1", [2, 3, 4, 5] * 128)
    sel = bench.cpu_sample(mixed, 10.0, 16)
    assert set(int(d) for d in mixed.cells["depth"][sel]) == {2, 3, 4, 5}
