"""ctypes binding of libmsfec_cuda.so (C ABI in include/msfec_cuda.h).

Python-side view of the C ABI used by tests, the benchmark and
``__graft_entry__``; the product interface for C++ callers is the header
itself and the QBasis-compatible shim under host/. Loading fails loudly when
the library has not been built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libmsfec_cuda.so")

SUCCESS = 0
ERROR_INVALID_ARGUMENT = 1
ERROR_CUDA = 2
ERROR_OUT_OF_MEMORY = 3
ERROR_NOT_CONVERGED = 4
ERROR_NOT_SUPPORTED = 5
ERROR_NUMERICAL = 6
ERROR_INVALID_STATE = 7
KIND_Q1, KIND_NEDRT, KIND_QNED, KIND_RTDQ = 1, 2, 3, 4
Q1_COEF_SCALAR, Q1_COEF_TENSOR, Q1_COEF_GAUSS = 0, 1, 2  # msfec_config.q1_coefficient

PRECISION_FP64 = 0
PRECISION_MIXED = 1

LOAD_ZERO, LOAD_CONSTANT, LOAD_SIN_PRODUCT, LOAD_VEC_TRIG = 0, 1, 2, 3

# Every symbol the public header declares (checked by the CPU test suite).
EXPORTED = [
    "msfec_config_default", "msfec_create", "msfec_destroy", "msfec_status_string",
    "msfec_last_error", "msfec_set_stream", "msfec_set_precision", "msfec_q1_build",
    "msfec_q1_build_device", "msfec_q1_basis_size", "msfec_q1_get_basis",
    "msfec_q1_basis_device", "msfec_q1_eval_fine", "msfec_set_timing", "msfec_get_timings",
    "msfec_nedrt_build", "msfec_nedrt_build_device", "msfec_nedrt_basis_size",
    "msfec_nedrt_get_basis", "msfec_q1_backward", "msfec_nedrt_build_noalloc",
    "msfec_q1_get_basis_cells", "msfec_nedrt_get_basis_cells",
    "msfec_set_graph", "msfec_autotune", "msfec_q1_fine_solve", "msfec_nedrt_backward",
    "msfec_qned_build", "msfec_qned_build_device", "msfec_qned_basis_size", "msfec_qned_get_basis",
    "msfec_rtdq_build", "msfec_rtdq_build_device", "msfec_rtdq_basis_size", "msfec_rtdq_get_basis",
    "msfec_nedrt_fine_solve",
]


class Config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("precision", ctypes.c_int32), ("rtol", ctypes.c_double),
                ("inner_rtol", ctypes.c_double), ("max_iter", ctypes.c_int32),
                ("max_refine", ctypes.c_int32), ("verbose", ctypes.c_int32),
                ("q1_launch", ctypes.c_int32), ("nedrt_rtol", ctypes.c_double),
                ("nedrt_precond", ctypes.c_int32), ("q1_coefficient", ctypes.c_int32),
                ("nedrt_stage", ctypes.c_int32), ("nedrt_ctas_per_sm", ctypes.c_int32),
                ("nedrt_zt_place", ctypes.c_int32), ("nedrt_inner_rtol", ctypes.c_double)]


class Cell(ctypes.Structure):
    _fields_ = [("origin", ctypes.c_double * 3), ("size", ctypes.c_double * 3),
                ("depth", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Load(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("params", ctypes.c_double * 4)]


class CellReport(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("refinements", ctypes.c_int32),
                ("converged", ctypes.c_int32), ("iterations_sum", ctypes.c_int32),
                ("residual", ctypes.c_double)]


class Timings(ctypes.Structure):
    _fields_ = [("solve_ms", ctypes.c_float), ("galerkin_ms", ctypes.c_float),
                ("total_ms", ctypes.c_float), ("solve_launches", ctypes.c_int32),
                ("kernel_launches", ctypes.c_int32), ("graph", ctypes.c_int32),
                ("setup_ms", ctypes.c_float)]


CELL_DTYPE = np.dtype([("origin", "<f8", (3,)), ("size", "<f8", (3,)), ("depth", "<i4"),
                       ("reserved", "<i4")])
REPORT_DTYPE = np.dtype([("iterations", "<i4"), ("refinements", "<i4"), ("converged", "<i4"),
                         ("iterations_sum", "<i4"), ("residual", "<f8")])
assert CELL_DTYPE.itemsize == ctypes.sizeof(Cell)
assert REPORT_DTYPE.itemsize == ctypes.sizeof(CellReport)

_lib = None
_vp = ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)


def load_library(path: str = LIB_PATH):
    """Load the CUDA library; raises if it is missing (build it first)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libmsfec_cuda.so not built ({path}); run __graft_entry__.build()")
    L = ctypes.CDLL(path)
    L.msfec_config_default.argtypes = [ctypes.POINTER(Config)]
    L.msfec_config_default.restype = None
    L.msfec_create.argtypes = [ctypes.POINTER(_vp), ctypes.POINTER(Config)]
    L.msfec_create.restype = ctypes.c_int
    L.msfec_destroy.argtypes = [_vp]
    L.msfec_destroy.restype = None
    L.msfec_status_string.argtypes = [ctypes.c_int]
    L.msfec_status_string.restype = ctypes.c_char_p
    L.msfec_last_error.argtypes = [_vp]
    L.msfec_last_error.restype = ctypes.c_char_p
    L.msfec_set_stream.argtypes = [_vp, _vp]
    L.msfec_set_stream.restype = ctypes.c_int
    L.msfec_set_precision.argtypes = [_vp, ctypes.c_int32]
    L.msfec_set_precision.restype = ctypes.c_int
    L.msfec_q1_build.argtypes = [_vp, ctypes.c_int32, _vp, _dp, _dp, ctypes.POINTER(Load), _dp, _dp, _vp]
    L.msfec_q1_build.restype = ctypes.c_int
    L.msfec_q1_build_device.argtypes = [_vp, ctypes.c_int32, _vp, _vp, _vp, ctypes.POINTER(Load), _vp,
                                        _vp, _vp]
    L.msfec_q1_build_device.restype = ctypes.c_int
    L.msfec_q1_basis_size.argtypes = [_vp]
    L.msfec_q1_basis_size.restype = ctypes.c_int64
    L.msfec_q1_get_basis.argtypes = [_vp, _dp, ctypes.c_int64]
    L.msfec_q1_get_basis.restype = ctypes.c_int
    L.msfec_q1_basis_device.argtypes = [_vp]
    L.msfec_q1_basis_device.restype = _vp
    L.msfec_q1_eval_fine.argtypes = [_vp, _dp, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32), _dp, _dp]
    L.msfec_q1_eval_fine.restype = ctypes.c_int
    L.msfec_nedrt_build.argtypes = [_vp, ctypes.c_int32, _vp, _dp, _dp, ctypes.POINTER(Load), _dp, _dp,
                                    _vp]
    L.msfec_nedrt_build.restype = ctypes.c_int
    L.msfec_nedrt_build_device.argtypes = [_vp, ctypes.c_int32, _vp, _vp, _vp, ctypes.POINTER(Load), _vp,
                                           _vp, _vp]
    L.msfec_nedrt_build_device.restype = ctypes.c_int
    L.msfec_nedrt_basis_size.argtypes = [_vp]
    L.msfec_nedrt_basis_size.restype = ctypes.c_int64
    L.msfec_nedrt_get_basis.argtypes = [_vp, _dp, ctypes.c_int64]
    L.msfec_nedrt_get_basis.restype = ctypes.c_int
    for name in ("msfec_q1_get_basis_cells", "msfec_nedrt_get_basis_cells"):
        getattr(L, name).argtypes = [_vp, ctypes.c_int32, ctypes.c_int32, _dp, ctypes.c_int64]
        getattr(L, name).restype = ctypes.c_int
    L.msfec_q1_backward.argtypes = [_vp, ctypes.c_int32, _vp, _dp, _dp, ctypes.POINTER(Load), ctypes.c_int32,
                                    _dp, _dp, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32), _dp, _dp, _dp]
    L.msfec_q1_backward.restype = ctypes.c_int
    L.msfec_set_timing.argtypes = [_vp, ctypes.c_int32]
    L.msfec_set_timing.restype = ctypes.c_int
    L.msfec_get_timings.argtypes = [_vp, ctypes.POINTER(Timings)]
    L.msfec_get_timings.restype = ctypes.c_int
    L.msfec_autotune.argtypes = [_vp, ctypes.c_int32, ctypes.c_int32, _vp, _vp, _vp, ctypes.POINTER(Load),
                                 ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_float)]
    L.msfec_autotune.restype = ctypes.c_int
    L.msfec_q1_fine_solve.argtypes = [_vp, _vp, _dp, _dp, ctypes.POINTER(Load), _dp, _vp]
    L.msfec_q1_fine_solve.restype = ctypes.c_int
    L.msfec_nedrt_fine_solve.argtypes = [_vp, _vp, _dp, _dp, ctypes.POINTER(Load), _dp, _vp]
    L.msfec_nedrt_fine_solve.restype = ctypes.c_int
    L.msfec_nedrt_backward.argtypes = [_vp, ctypes.c_int32, _vp, _dp, _dp, ctypes.POINTER(Load), ctypes.c_int32,
                                       _dp, _dp, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32), _dp, _dp, _dp, _dp]
    L.msfec_nedrt_backward.restype = ctypes.c_int
    L.msfec_qned_build.argtypes = [_vp, ctypes.c_int32, _vp, _dp, _dp, ctypes.POINTER(Load), _dp, _dp, _vp]
    L.msfec_qned_build.restype = ctypes.c_int
    L.msfec_qned_basis_size.argtypes = [_vp]
    L.msfec_qned_basis_size.restype = ctypes.c_int64
    L.msfec_qned_get_basis.argtypes = [_vp, _dp, ctypes.c_int64]
    L.msfec_qned_get_basis.restype = ctypes.c_int
    L.msfec_rtdq_build.argtypes = [_vp, ctypes.c_int32, _vp, _dp, ctypes.POINTER(Load), _dp, _dp, _vp]
    L.msfec_rtdq_build.restype = ctypes.c_int
    L.msfec_rtdq_build_device.argtypes = [_vp, ctypes.c_int32, _vp, _vp, ctypes.POINTER(Load), _vp, _vp, _vp]
    L.msfec_rtdq_build_device.restype = ctypes.c_int
    L.msfec_rtdq_basis_size.argtypes = [_vp]
    L.msfec_rtdq_basis_size.restype = ctypes.c_int64
    L.msfec_rtdq_get_basis.argtypes = [_vp, _dp, ctypes.c_int64]
    L.msfec_rtdq_get_basis.restype = ctypes.c_int
    L.msfec_set_graph.argtypes = [_vp, ctypes.c_int32]
    L.msfec_set_graph.restype = ctypes.c_int
    _lib = L
    return L


class MsfecError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"msfec status {status}: {msg}")
        self.status = status


def make_cells(origins, sizes, depths):
    origins = np.asarray(origins, dtype=np.float64).reshape(-1, 3)
    sizes = np.asarray(sizes, dtype=np.float64).reshape(-1, 3)
    depths = np.asarray(depths, dtype=np.int32).reshape(-1)
    cells = np.zeros(depths.shape[0], dtype=CELL_DTYPE)
    cells["origin"] = origins
    cells["size"] = sizes
    cells["depth"] = depths
    return cells


def make_load(kind=LOAD_ZERO, params=(0.0, 0.0, 0.0, 0.0)):
    ld = Load()
    ld.kind = int(kind)
    for i, p in enumerate(list(params) + [0.0] * (4 - len(params))):
        ld.params[i] = float(p)
    return ld


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


class Handle:
    """One msfec handle (device buffers + stream)."""

    def __init__(self, precision=PRECISION_MIXED, device=0, rtol=None, inner_rtol=None,
                 max_iter=None, max_refine=None, verbose=0, nedrt_rtol=None, q1_launch=0, nedrt_precond=0,
                 q1_coefficient=0, nedrt_stage=None, nedrt_ctas_per_sm=0, nedrt_zt_place=0,
                 nedrt_inner_rtol=None):
        L = load_library()
        cfg = Config()
        L.msfec_config_default(ctypes.byref(cfg))
        cfg.device = device
        cfg.precision = precision
        if rtol is not None:
            cfg.rtol = rtol
        if inner_rtol is not None:
            cfg.inner_rtol = inner_rtol
        if max_iter is not None:
            cfg.max_iter = max_iter
        if max_refine is not None:
            cfg.max_refine = max_refine
        if nedrt_rtol is not None:
            cfg.nedrt_rtol = nedrt_rtol
        cfg.verbose = int(verbose or os.environ.get("MSFEC_VERBOSE", "0"))
        cfg.q1_launch = int(q1_launch)
        cfg.nedrt_precond = int(nedrt_precond)
        cfg.q1_coefficient = int(q1_coefficient)
        if nedrt_stage is not None:
            cfg.nedrt_stage = int(nedrt_stage)
        cfg.nedrt_ctas_per_sm = int(nedrt_ctas_per_sm)
        cfg.nedrt_zt_place = int(nedrt_zt_place)
        if nedrt_inner_rtol is not None:
            cfg.nedrt_inner_rtol = nedrt_inner_rtol
        self.cfg = cfg
        h = _vp()
        st = L.msfec_create(ctypes.byref(h), ctypes.byref(cfg))
        if st != SUCCESS:
            raise MsfecError(st, L.msfec_status_string(st).decode())
        self._h = h
        self._lib = L

    @property
    def ptr(self):
        return self._h

    def close(self):
        if self._h:
            self._lib.msfec_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def last_error(self):
        return self._lib.msfec_last_error(self._h).decode()

    def check(self, st, allow=()):
        if st != SUCCESS and st not in allow:
            raise MsfecError(st, self._lib.msfec_status_string(st).decode() + ": " + self.last_error())
        return st

    def set_stream(self, stream_handle):
        return self.check(self._lib.msfec_set_stream(self._h, _vp(stream_handle or 0)))

    def set_precision(self, precision):
        return self.check(self._lib.msfec_set_precision(self._h, int(precision)))

    def q1_build(self, cells, a, reaction=None, load=None, allow_unconverged=False):
        """Host-buffer Q1 build. Returns (KH [c,8,8], FH [c,8], reports, status)."""
        cells = np.ascontiguousarray(cells, dtype=CELL_DTYPE)
        nc = cells.shape[0]
        a = np.ascontiguousarray(a, dtype=np.float64)
        reaction = None if reaction is None else np.ascontiguousarray(reaction, dtype=np.float64)
        KH = np.zeros((nc, 8, 8))
        FH = np.zeros((nc, 8))
        rep = np.zeros(nc, dtype=REPORT_DTYPE)
        ld = load if load is not None else make_load()
        st = self._lib.msfec_q1_build(self._h, nc, cells.ctypes.data_as(_vp), _d(a), _d(reaction),
                                      ctypes.byref(ld), _d(KH), _d(FH), rep.ctypes.data_as(_vp))
        self.check(st, allow=(ERROR_NOT_CONVERGED,) if allow_unconverged else ())
        return KH, FH, rep, st

    def q1_build_device(self, cells, d_a, d_reaction, load, d_KH, d_FH, d_reports):
        """Device-pointer Q1 build (asynchronous on the handle's stream)."""
        cells = np.ascontiguousarray(cells, dtype=CELL_DTYPE)
        st = self._lib.msfec_q1_build_device(self._h, cells.shape[0], cells.ctypes.data_as(_vp),
                                             _vp(d_a), _vp(d_reaction or 0), ctypes.byref(load),
                                             _vp(d_KH), _vp(d_FH), _vp(d_reports or 0))
        return self.check(st)

    def set_timing(self, enable=True):
        return self.check(self._lib.msfec_set_timing(self._h, 1 if enable else 0))

    def nedrt_backward(self, cells, ainv6, bdiv, load, U, lam, cell_of, points, dJ_du, reuse_basis=True):
        """(dJ/d log A, dJ/d log B) per fine cell (msfec_nedrt_backward)."""
        cells = np.ascontiguousarray(cells, dtype=CELL_DTYPE)
        ainv6 = np.ascontiguousarray(ainv6, dtype=np.float64)
        bdiv = np.ascontiguousarray(bdiv, dtype=np.float64)
        U = np.ascontiguousarray(U, dtype=np.float64)
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        cell_of = np.ascontiguousarray(cell_of, dtype=np.int32)
        points = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        dJ_du = np.ascontiguousarray(dJ_du, dtype=np.float64).reshape(-1, 3)
        ga = np.zeros(bdiv.size)
        gb = np.zeros(bdiv.size)
        st = self._lib.msfec_nedrt_backward(self._h, cells.shape[0], cells.ctypes.data_as(_vp), _d(ainv6), _d(bdiv),
                                            ctypes.byref(load), 1 if reuse_basis else 0, _d(U), _d(lam),
                                            points.shape[0], cell_of.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                            _d(points), _d(dJ_du), _d(ga), _d(gb))
        self.check(st)
        return ga, gb

    def q1_fine_solve(self, domain, a, reaction, load):
        """msfec_q1_fine_solve: standard fine-scale solve on one box; returns (u, report, status)."""
        domain = np.ascontiguousarray(domain, dtype=CELL_DTYPE).reshape(1)
        a = np.ascontiguousarray(a, dtype=np.float64)
        reaction = None if reaction is None else np.ascontiguousarray(reaction, dtype=np.float64)
        n = 1 << int(domain["depth"][0])
        u = np.zeros((n + 1) ** 3)
        rep = np.zeros(1, dtype=REPORT_DTYPE)
        st = self._lib.msfec_q1_fine_solve(self._h, domain.ctypes.data_as(_vp), _d(a),
                                           None if reaction is None else _d(reaction), ctypes.byref(load),
                                           _d(u), rep.ctypes.data_as(_vp))
        self.check(st, allow=(ERROR_NOT_CONVERGED,))
        return u, rep[0], st

    def nedrt_fine_solve(self, domain, ainv6, bdiv, load):
        """msfec_nedrt_fine_solve: standard fine-scale Ned_RT solve (natural boundary
        conditions) on one box; returns (x = [sigma edges, u faces], report, status)."""
        domain = np.ascontiguousarray(domain, dtype=CELL_DTYPE).reshape(1)
        ainv6 = np.ascontiguousarray(ainv6, dtype=np.float64)
        bdiv = np.ascontiguousarray(bdiv, dtype=np.float64)
        n = 1 << int(domain["depth"][0])
        x = np.zeros(3 * n * (n + 1) ** 2 + 3 * (n + 1) * n * n)
        rep = np.zeros(1, dtype=REPORT_DTYPE)
        ld = load if load is not None else make_load()
        st = self._lib.msfec_nedrt_fine_solve(self._h, domain.ctypes.data_as(_vp), _d(ainv6), _d(bdiv),
                                              ctypes.byref(ld), _d(x), rep.ctypes.data_as(_vp))
        self.check(st, allow=(ERROR_NOT_CONVERGED,))
        return x, rep[0], st

    def autotune(self, kind, cells, coef0, coef1, load):
        """msfec_autotune on a sample batch; returns (choice, n_candidates, times_ms)."""
        cells = np.ascontiguousarray(cells, dtype=CELL_DTYPE)
        c0 = np.ascontiguousarray(coef0, dtype=np.float64)
        c1 = None if coef1 is None else np.ascontiguousarray(coef1, dtype=np.float64)
        ch = (ctypes.c_int32 * 2)()
        tm = (ctypes.c_float * 16)()
        st = self._lib.msfec_autotune(self._h, int(kind), cells.shape[0], cells.ctypes.data_as(_vp),
                                      c0.ctypes.data_as(_vp), None if c1 is None else c1.ctypes.data_as(_vp),
                                      ctypes.byref(load), ch, tm)
        self.check(st)
        return int(ch[0]), int(ch[1]), [float(tm[k]) for k in range(int(ch[1]))]

    def set_graph(self, enable=True):
        """msfec_set_graph: capture / replay the build's launch sequence as a CUDA graph."""
        return self.check(self._lib.msfec_set_graph(self._h, 1 if enable else 0))

    def timings(self):
        t = Timings()
        self.check(self._lib.msfec_get_timings(self._h, ctypes.byref(t)))
        return {"solve_ms": t.solve_ms, "galerkin_ms": t.galerkin_ms, "total_ms": t.total_ms,
                "solve_launches": t.solve_launches, "kernel_launches": t.kernel_launches,
                "graph": t.graph, "setup_ms": t.setup_ms}

    def q1_backward(self, cells, a, reaction, load, U, lam, cell_of, points, dJ_du, reuse_basis=True):
        """dJ/d log a per fine cell (msfec_q1_backward)."""
        cells = np.ascontiguousarray(cells, dtype=CELL_DTYPE)
        a = np.ascontiguousarray(a, dtype=np.float64)
        reaction = None if reaction is None else np.ascontiguousarray(reaction, dtype=np.float64)
        U = np.ascontiguousarray(U, dtype=np.float64)
        lam = np.ascontiguousarray(lam, dtype=np.float64)
        cell_of = np.ascontiguousarray(cell_of, dtype=np.int32)
        points = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        dJ_du = np.ascontiguousarray(dJ_du, dtype=np.float64)
        grad = np.zeros(a.shape[0])
        st = self._lib.msfec_q1_backward(self._h, cells.shape[0], cells.ctypes.data_as(_vp), _d(a), _d(reaction),
                                         ctypes.byref(load), 1 if reuse_basis else 0, _d(U), _d(lam),
                                         points.shape[0], cell_of.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                         _d(points), _d(dJ_du), _d(grad))
        self.check(st)
        return grad

    def nedrt_build(self, cells, ainv6, bdiv, load=None, allow_unconverged=False):
        """Host-buffer Ned_RT build. Returns (KH [c,18,18], FH [c,18], reports, status)."""
        cells = np.ascontiguousarray(cells, dtype=CELL_DTYPE)
        nc = cells.shape[0]
        ainv6 = np.ascontiguousarray(ainv6, dtype=np.float64)
        bdiv = np.ascontiguousarray(bdiv, dtype=np.float64)
        KH = np.zeros((nc, 18, 18))
        FH = np.zeros((nc, 18))
        rep = np.zeros(nc, dtype=REPORT_DTYPE)
        ld = load if load is not None else make_load()
        st = self._lib.msfec_nedrt_build(self._h, nc, cells.ctypes.data_as(_vp), _d(ainv6), _d(bdiv),
                                         ctypes.byref(ld), _d(KH), _d(FH), rep.ctypes.data_as(_vp))
        self.check(st, allow=(ERROR_NOT_CONVERGED,) if allow_unconverged else ())
        return KH, FH, rep, st

    def nedrt_build_device(self, cells, d_ainv6, d_bdiv, load, d_KH, d_FH, d_reports):
        cells = np.ascontiguousarray(cells, dtype=CELL_DTYPE)
        st = self._lib.msfec_nedrt_build_device(self._h, cells.shape[0], cells.ctypes.data_as(_vp),
                                                _vp(d_ainv6), _vp(d_bdiv), ctypes.byref(load),
                                                _vp(d_KH), _vp(d_FH), _vp(d_reports or 0))
        return self.check(st)

    def nedrt_build_noalloc(self, cells, d_ainv6, d_bdiv, load, d_KH, d_FH, d_reports):
        """msfec_nedrt_build_noalloc: msfec_nedrt_build_device with every internal
        buffer in the library's static per-device pool (no device allocation)."""
        cells = np.ascontiguousarray(cells, dtype=CELL_DTYPE)
        st = self._lib.msfec_nedrt_build_noalloc(self._h, cells.shape[0], cells.ctypes.data_as(_vp),
                                                 _vp(d_ainv6), _vp(d_bdiv), ctypes.byref(load),
                                                 _vp(d_KH), _vp(d_FH), _vp(d_reports or 0))
        return self.check(st)

    def qned_build(self, cells, a6, binv, load):
        """Q_Ned basis build from host arrays; returns (KH [c,20,20], FH [c,20], reports, status)."""
        cells = np.ascontiguousarray(cells, dtype=CELL_DTYPE)
        a6 = np.ascontiguousarray(a6, dtype=np.float64)
        binv = np.ascontiguousarray(binv, dtype=np.float64)
        nc = cells.shape[0]
        KH = np.zeros((nc, 20, 20))
        FH = np.zeros((nc, 20))
        rep = np.zeros(nc, dtype=REPORT_DTYPE)
        st = self._lib.msfec_qned_build(self._h, nc, cells.ctypes.data_as(_vp), _d(a6), _d(binv),
                                        ctypes.byref(load), _d(KH), _d(FH), rep.ctypes.data_as(_vp))
        self.check(st, allow=(ERROR_NOT_CONVERGED,))
        return KH, FH, rep, st

    def qned_build_device(self, cells, d_a6, d_binv, load, d_KH, d_FH, d_reports):
        cells = np.ascontiguousarray(cells, dtype=CELL_DTYPE)
        st = self._lib.msfec_qned_build_device(self._h, cells.shape[0], cells.ctypes.data_as(_vp),
                                               _vp(d_a6), _vp(d_binv), ctypes.byref(load),
                                               _vp(d_KH), _vp(d_FH), _vp(d_reports or 0))
        return self.check(st)

    def qned_basis(self):
        n = self._lib.msfec_qned_basis_size(self._h)
        out = np.zeros(n)
        self.check(self._lib.msfec_qned_get_basis(self._h, _d(out), n))
        return out

    def rtdq_build(self, cells, ainv6, load):
        """RT_DQ basis build from host arrays; returns (KH [c,7,7], FH [c,7], reports, status)."""
        cells = np.ascontiguousarray(cells, dtype=CELL_DTYPE)
        ainv6 = np.ascontiguousarray(ainv6, dtype=np.float64)
        nc = cells.shape[0]
        KH = np.zeros((nc, 7, 7))
        FH = np.zeros((nc, 7))
        rep = np.zeros(nc, dtype=REPORT_DTYPE)
        st = self._lib.msfec_rtdq_build(self._h, nc, cells.ctypes.data_as(_vp), _d(ainv6), ctypes.byref(load),
                                        _d(KH), _d(FH), rep.ctypes.data_as(_vp))
        self.check(st, allow=(ERROR_NOT_CONVERGED,))
        return KH, FH, rep, st

    def rtdq_build_device(self, cells, d_ainv6, load, d_KH, d_FH, d_reports):
        cells = np.ascontiguousarray(cells, dtype=CELL_DTYPE)
        st = self._lib.msfec_rtdq_build_device(self._h, cells.shape[0], cells.ctypes.data_as(_vp),
                                               _vp(d_ainv6), ctypes.byref(load),
                                               _vp(d_KH), _vp(d_FH), _vp(d_reports or 0))
        return self.check(st)

    def rtdq_basis(self):
        n = self._lib.msfec_rtdq_basis_size(self._h)
        out = np.zeros(n)
        self.check(self._lib.msfec_rtdq_get_basis(self._h, _d(out), n))
        return out

    def nedrt_basis(self):
        n = self._lib.msfec_nedrt_basis_size(self._h)
        out = np.zeros(n)
        self.check(self._lib.msfec_nedrt_get_basis(self._h, _d(out), n))
        return out

    def q1_basis(self):
        n = self._lib.msfec_q1_basis_size(self._h)
        out = np.zeros(n)
        self.check(self._lib.msfec_q1_get_basis(self._h, _d(out), n))
        return out

    def q1_basis_cells(self, cells, first, count):
        """Basis of cells [first, first + count) of the last Q1 build `cells`:
        a list of [8, (n+1)^3] arrays."""
        n1 = (1 << cells["depth"][first:first + count].astype(np.int64)) + 1
        out = np.zeros(int(np.sum(8 * n1 ** 3)))
        self.check(self._lib.msfec_q1_get_basis_cells(self._h, first, count, _d(out), out.size))
        sizes = np.cumsum(np.concatenate([[0], 8 * n1 ** 3]))
        return [out[sizes[i]:sizes[i + 1]].reshape(8, -1) for i in range(count)]

    def nedrt_basis_cells(self, cells, first, count):
        """Basis of cells [first, first + count) of the last Ned_RT build
        `cells`: a list of [18, NE + NF] arrays."""
        n = 1 << cells["depth"][first:first + count].astype(np.int64)
        nd = 3 * n * (n + 1) ** 2 + 3 * n * n * (n + 1)
        out = np.zeros(int(np.sum(18 * nd)))
        self.check(self._lib.msfec_nedrt_get_basis_cells(self._h, first, count, _d(out), out.size))
        sizes = np.cumsum(np.concatenate([[0], 18 * nd]))
        return [out[sizes[i]:sizes[i + 1]].reshape(18, -1) for i in range(count)]

    def q1_eval_fine(self, weights, cell_of, points):
        weights = np.ascontiguousarray(weights, dtype=np.float64)
        cell_of = np.ascontiguousarray(cell_of, dtype=np.int32)
        points = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(points.shape[0])
        st = self._lib.msfec_q1_eval_fine(self._h, _d(weights), points.shape[0],
                                          cell_of.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                          _d(points), _d(out))
        self.check(st)
        return out
