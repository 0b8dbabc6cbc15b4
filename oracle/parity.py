"""Parity of a batched GPU build against the FP64 oracle on a stratified
sample of its cells.

TEST INFRASTRUCTURE ONLY: used by tests/ and by the parity check that
bench.py runs after its timed region; the product library never imports it.

A batch of the benchmark's size (512 to 4096 coarse cells, up to 1.6e10
basis values) is far beyond what the oracle solves in seconds, but its cells
are independent: the GPU builds the whole batch in one launch sequence, and a
sample of cells that represents every refinement depth of the batch is
rebuilt cell by cell by the oracle (sparse direct / banded Cholesky, FP64) in
a spawn-started process pool. The comparison is per cell and per basis
function, relative to the largest entry:
  K_H, F_H  max |gpu - oracle| / max |oracle|   (F_H: cells with a nonzero load)
  Phi       max over the basis functions b of max |phi_b - phi_b^oracle| / max |phi_b^oracle|
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
PKG = os.path.join(REPO, "mpi-msfec_gb300")


def stratified_sample(cells, per_depth, spread=True):
    """Indices of up to per_depth[d] cells of every depth d present in the batch
    (sorted). spread: evenly spaced over the batch's cells of that depth (first,
    ..., last); otherwise the first ones."""
    depth = np.asarray(cells["depth"])
    out = []
    for d in sorted(set(int(x) for x in depth)):
        cand = np.where(depth == d)[0]
        k = min(len(cand), int(per_depth.get(d, per_depth.get("default", 1))
                               if isinstance(per_depth, dict) else per_depth))
        if k <= 0:
            continue
        pick = cand[np.round(np.linspace(0, len(cand) - 1, k)).astype(int)] if spread else cand[:k]
        out.extend(int(c) for c in pick)
    return np.array(sorted(set(out)), dtype=np.int64)


def fine_slices(cells, sel):
    """(start, stop) of every selected cell's n^3 fine-cell values."""
    n = 1 << np.asarray(cells["depth"]).astype(np.int64)
    off = np.concatenate([[0], np.cumsum(n ** 3)])
    return [(int(off[c]), int(off[c + 1])) for c in sel]


def _paths():
    for p in (PKG, REPO):
        if p not in sys.path:
            sys.path.insert(0, p)


def _oracle_cell(args):
    """One cell through the oracle (worker process): returns (KH, FH, Phi [nb, ndof])."""
    _paths()
    kind, cell, coef, load_kind, load_params = args
    cells = cell.reshape(1)
    if kind == "q1":
        from oracle import oracle
        a, r = coef
        res = oracle.q1_build(cells["origin"], cells["size"], cells["depth"], a, r, load_kind=load_kind,
                              load_params=list(load_params), want_phi=True, nthreads=1)
        if res["status"] != 0:
            raise RuntimeError(f"Q1 oracle status {res['status']}")
        return res["KH"][0], res["FH"][0], res["Phi"].reshape(8, -1)
    from oracle import nedrt_oracle as N
    if kind == "nedrt":
        ainv6, bdiv = coef
        phi, kh, fh = N.build_cell(cells["origin"][0], cells["size"][0], int(cells["depth"][0]),
                                   N.sym6_to_ainv(ainv6), bdiv, load_kind, load_params)
        return kh, fh, phi
    raise ValueError(f"unknown pairing {kind!r}")


class OracleSample:
    """Oracle results of the sampled cells, computed asynchronously in a
    spawn-started pool (start it before the GPU work so that both overlap;
    a pool forked after the first CUDA call would hang)."""

    def __init__(self, kind, cells, sel, coef_arrays, load, processes=None):
        self.kind, self.sel = kind, np.asarray(sel, dtype=np.int64)
        sl = fine_slices(cells, self.sel)
        jobs = []
        for c, (f0, f1) in zip(self.sel, sl):
            coef = tuple(None if a is None else np.ascontiguousarray(a[f0:f1]) for a in coef_arrays)
            jobs.append((kind, np.array(cells[c]), coef, int(load.kind), tuple(float(p) for p in load.params)))
        nproc = max(1, min(len(jobs), processes or os.cpu_count() or 1))
        saved = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")}
        for k in saved:
            os.environ[k] = "1"
        try:
            self._pool = mp.get_context("spawn").Pool(nproc)
        finally:
            for k, v in saved.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
        # largest cells first: the pool's tail is then short
        order = np.argsort([-(f1 - f0) for f0, f1 in sl], kind="stable")
        self._async = {int(i): self._pool.apply_async(_oracle_cell, (jobs[int(i)],)) for i in order}
        self._res = None

    def results(self, timeout=None):
        """[(KH, FH, Phi)] in sample order."""
        if self._res is None:
            self._res = [self._async[i].get(timeout) for i in range(len(self.sel))]
            self._pool.close()
            self._pool.join()
        return self._res

    def close(self):
        self._pool.terminate()
        self._pool.join()


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def compare(sample, KH, FH, phi_of):
    """Errors of the GPU outputs on the sampled cells. KH, FH: the whole batch's
    arrays ([ncells, nb, nb], [ncells, nb]); phi_of(c) -> [nb, ndof] GPU basis of
    batch cell c, or None to skip the basis. Returns the maxima and the
    per-cell values."""
    kh, fh, ph, per = [], [], [], []
    for c, (rk, rf, rp) in zip(sample.sel, sample.results()):
        ek = rel(KH[c], rk)
        ef = rel(FH[c], rf) if np.abs(rf).max() > 0 else 0.0
        ep = 0.0
        pg = phi_of(int(c)) if phi_of is not None else None
        if pg is not None:
            pg = np.asarray(pg).reshape(rp.shape)
            ep = max(rel(pg[b], rp[b]) for b in range(rp.shape[0]))
            ph.append(ep)
        kh.append(ek)
        fh.append(ef)
        per.append({"cell": int(c), "KH": ek, "FH": ef, "Phi": ep if pg is not None else None})
    return {"cells": len(kh), "KH_max_rel": max(kh), "FH_max_rel": max(fh),
            "Phi_max_rel": max(ph) if ph else None, "per_cell": per}
