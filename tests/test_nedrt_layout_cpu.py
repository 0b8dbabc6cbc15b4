"""CPU checks of the Ned_RT workspace arithmetic in csrc/nedrt_common.cuh,
compiled as host code (the header's __host__ __device__ functions):
  - every cell's shared prep block (nr_prep_floats) is a multiple of 64 floats,
    so each cell's block, and its patch-factor region (nr_prep_patch_offset),
    start on a 16-byte boundary for the solver's uint4 factor loads;
  - the patch-factor word map (word t of fine cell c at (t / 4 * n^3 + c) * 4
    + t % 4, kNRPatchFloats words per cell) is a bijection onto the region and
    fits inside the prep block;
  - with z~ in shared memory (mixed, depth 4) the dynamic shared memory (the
    multilevel region, then z~ at a 128-byte aligned offset) stays within the
    224 KB the host allows one 512-thread CTA (capi.cu, kNRSmemTotalLimit)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "mpi-msfec_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "nedrt_common.cuh"
using namespace msfec;
int main() {
  for (int n = 4; n <= 16; n *= 2) {
    const size_t nc = (size_t)n * n * n;
    const size_t pf = nr_prep_floats(n), po = nr_prep_patch_offset(n);
    std::vector<unsigned char> hit(kNRPatchFloats * nc, 0);
    long bad = 0;
    for (size_t c = 0; c < nc; ++c)
      for (int t = 0; t < kNRPatchFloats; ++t) {
        const size_t w = ((size_t)(t / 4) * nc + c) * 4 + t % 4;
        if (w >= hit.size() || hit[w]++) ++bad;
      }
    int NEx, NFx, NE, NF;
    nr_counts(n, NEx, NFx, NE, NF);
    const size_t Np = ((size_t)NE + NF + 63) / 64 * 64;
    const size_t ml = nr_ml_layout(n, 4).bytes;
    const size_t zt_off = (ml + 127) / 128 * 128;
    printf("%d %zu %zu %zu %d %ld %zu %zu\n", n, pf, po, nc, kNRPatchFloats, bad, zt_off, zt_off + Np * 4);
  }
  return 0;
}
"""


def test_prep_patch_layout_and_zt_shared_memory(tmp_path):
    cxx = shutil.which("g++")
    cuda_inc = None
    for root in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if root and os.path.exists(os.path.join(root, "include", "cuda_runtime.h")):
            cuda_inc = os.path.join(root, "include")
            break
    if cxx is None or cuda_inc is None:
        pytest.skip("no g++ or CUDA headers")
    src = tmp_path / "layout.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "layout"
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-I", CSRC, "-I", cuda_inc, "-I", os.path.join(HERE, "..", "include"),
                        str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    rows = [list(map(int, l.split())) for l in lines if l.strip()]
    assert [row[0] for row in rows] == [4, 8, 16]
    for n, pf, po, nc, words, bad, zt_off, smem in rows:
        assert pf % 64 == 0, n  # every cell's block starts 256-byte aligned
        assert po % 4 == 0, n  # the patch region starts 16-byte aligned
        assert words % 4 == 0 and bad == 0, n  # whole uint4 groups, a bijection
        assert po + words * nc <= pf, n  # inside the cell's block
        assert zt_off % 16 == 0, n  # float4 access to z~
        assert smem <= 224 * 1024, (n, smem)  # one 512-thread CTA at nmax = n
