"""doug_gb300 -- GB300-native solve path of DOUG (Domain decomposition On
Unstructured Grids): PCG with a two-level additive Schwarz preconditioner
(overlapping subdomain solves + smoothed-aggregation coarse grid).

The Python side is a thin host mirror of the reference's solver entry over the
C ABI in ``include/doug_gpu.h`` (``doug_gb300/_build/libdouggpu.so``):

* control words and control files as in ``doug_aggr -f DOUG.ctl``
  (src/utils/DOUG_utils.F90:629-1150),
* assembled input (src/datatypes/SpMtx/SpMtx_class.F90:410-617),
* ``setup()`` = aggregation + coarse space + subdomains (src/main/aggr.F90:131-226),
* ``solve()`` = ``pcg_weigs`` (src/solvers/pcg.F90:289-462) on the GPU.

There is no CPU fallback: without the built library or without a CUDA device
the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from .build import LIB as _LIB_PATH, build as build_library

__all__ = ["DougSolver", "DougError", "SolveStats", "load_library", "build_library", "residual_csr",
           "DG_OK", "DG_NOT_CONVERGED", "DG_BREAKDOWN", "DG_SINGULAR", "DG_BAD_INPUT",
           "DG_CUDA_ERROR", "DG_NO_DEVICE", "DG_NOT_READY", "EXPORTED_SYMBOLS"]

DG_OK, DG_NOT_CONVERGED, DG_BREAKDOWN, DG_SINGULAR = 0, 1, 2, 3
DG_BAD_INPUT, DG_CUDA_ERROR, DG_NO_DEVICE, DG_NOT_READY = 4, 5, 6, 7
_STATUS_NAMES = {0: "DG_OK", 1: "DG_NOT_CONVERGED", 2: "DG_BREAKDOWN", 3: "DG_SINGULAR",
                 4: "DG_BAD_INPUT", 5: "DG_CUDA_ERROR", 6: "DG_NO_DEVICE", 7: "DG_NOT_READY"}

EXPORTED_SYMBOLS = [
    "dg_create", "dg_destroy", "dg_last_error", "dg_set_option", "dg_load_ctl",
    "dg_set_matrix_coo", "dg_set_rhs", "dg_set_partition", "dg_setup", "dg_solve",
    "dg_solve_device", "dg_write_solution", "dg_get_sizes", "dg_get_aggregates",
    "dg_get_subdomains", "dg_get_restriction", "dg_get_coarse_matrix", "dg_residual_csr",
    "dg_set_elements", "dg_get_input", "dg_grad_matrix", "dg_grad_elements",
    "dg_residual_csr_noalloc", "dg_autotune", "dg_set_systems", "dg_get_system_stats",
    "dg_solve_multi", "dg_solve_multi_device", "dg_set_node_geometry", "dg_get_coarse_coords",
    "dg_get_setup_phases",
]


class DougError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class _Stats(C.Structure):
    _fields_ = [("iterations", C.c_int), ("init_norm", C.c_double), ("final_norm", C.c_double),
                ("true_rel_residual", C.c_double), ("cond_num", C.c_double),
                ("t_setup_s", C.c_double), ("t_factor_s", C.c_double), ("t_iterate_s", C.c_double),
                ("t_total_s", C.c_double), ("n", C.c_int), ("nsubdomains", C.c_int),
                ("ncoarse", C.c_int), ("gpu_launches", C.c_int), ("factor_nnz", C.c_longlong),
                ("factor_gflop", C.c_double), ("t_subsolve_s", C.c_double),
                ("subsolve_bytes", C.c_double), ("t_coarse_s", C.c_double),
                ("coarse_bytes", C.c_double), ("t_spmv_s", C.c_double), ("spmv_bytes", C.c_double)]


@dataclass
class SolveStats:
    status: int
    iterations: int
    init_norm: float
    final_norm: float
    true_rel_residual: float
    cond_num: float
    t_setup_s: float
    t_factor_s: float
    t_iterate_s: float
    t_total_s: float
    n: int
    nsubdomains: int
    ncoarse: int
    gpu_launches: int
    factor_nnz: int
    factor_gflop: float
    t_subsolve_s: float = 0.0
    subsolve_bytes: float = 0.0
    t_coarse_s: float = 0.0
    coarse_bytes: float = 0.0
    t_spmv_s: float = 0.0
    spmv_bytes: float = 0.0


_lib = None


def load_library(path: str | None = None):
    """Load libdouggpu.so (built in-tree by ``build_library()``)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or _LIB_PATH
    if not os.path.exists(p):
        raise DougError(DG_CUDA_ERROR, f"{p} is missing: run doug_gb300.build_library() "
                                       "(there is no CPU fallback)")
    L = C.CDLL(p)
    P = C.POINTER
    vp = C.c_void_p
    L.dg_create.argtypes = [P(vp)]
    L.dg_destroy.argtypes = [vp]
    L.dg_last_error.argtypes = [vp]
    L.dg_last_error.restype = C.c_char_p
    L.dg_set_option.argtypes = [vp, C.c_char_p, C.c_char_p]
    L.dg_load_ctl.argtypes = [vp, C.c_char_p]
    L.dg_set_matrix_coo.argtypes = [vp, C.c_int, C.c_int, P(C.c_int), P(C.c_int), P(C.c_double)]
    L.dg_set_rhs.argtypes = [vp, P(C.c_double)]
    L.dg_grad_matrix.argtypes = [vp, vp, vp, vp, vp]
    L.dg_grad_elements.argtypes = [vp, vp, vp, vp, vp]
    L.dg_autotune.argtypes = [vp, P(C.c_double), P(C.c_int)]
    L.dg_set_systems.argtypes = [vp, C.c_int, P(C.c_int), P(C.c_longlong), P(C.c_int), P(C.c_int),
                                 P(C.c_double), P(C.c_double)]
    L.dg_get_system_stats.argtypes = [vp, P(C.c_int), P(C.c_int), P(C.c_double), P(C.c_double)]
    L.dg_solve_multi.argtypes = [vp, C.c_int, P(C.c_double), P(C.c_double), P(_Stats)]
    L.dg_solve_multi_device.argtypes = [vp, C.c_int, vp, vp, P(_Stats), vp]
    L.dg_set_elements.argtypes = [vp, C.c_int, C.c_int, P(C.c_int), P(C.c_int), P(C.c_double), P(C.c_double)]
    L.dg_set_node_geometry.argtypes = [vp, C.c_int, C.c_int, P(C.c_double), P(C.c_int)]
    L.dg_get_setup_phases.argtypes = [vp, P(C.c_double), P(C.c_double), P(C.c_int), P(C.c_double)]
    L.dg_get_coarse_coords.argtypes = [vp, P(C.c_int), P(C.c_int), P(C.c_double)]
    L.dg_get_input.argtypes = [vp, P(C.c_int), P(C.c_int), P(C.c_int), P(C.c_int), P(C.c_double),
                               P(C.c_double)]
    L.dg_set_partition.argtypes = [vp, P(C.c_int), C.c_int]
    L.dg_setup.argtypes = [vp]
    L.dg_solve.argtypes = [vp, P(C.c_double), P(C.c_double), P(_Stats)]
    L.dg_solve_device.argtypes = [vp, vp, vp, P(_Stats), vp]
    L.dg_write_solution.argtypes = [vp, P(C.c_double)]
    L.dg_get_sizes.argtypes = [vp, P(C.c_int), P(C.c_int), P(C.c_int), P(C.c_int), P(C.c_longlong),
                               P(C.c_int), P(C.c_int)]
    L.dg_get_aggregates.argtypes = [vp, P(C.c_int), P(C.c_int)]
    L.dg_get_subdomains.argtypes = [vp, P(C.c_longlong), P(C.c_int)]
    L.dg_get_restriction.argtypes = [vp, P(C.c_int), P(C.c_int), P(C.c_double)]
    L.dg_get_coarse_matrix.argtypes = [vp, P(C.c_int), P(C.c_int), P(C.c_double)]
    L.dg_residual_csr.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp, vp, vp]
    L.dg_residual_csr_noalloc.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp, vp, vp]
    for nm in EXPORTED_SYMBOLS:
        if nm not in ("dg_destroy", "dg_last_error"):
            getattr(L, nm).restype = C.c_int
    if path is None:
        _lib = L
    return L


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def residual_csr(rowptr, col, val, x, b, stream: int = 0):
    """r = b - A x and ||r||^2 on the GPU for torch CUDA tensors (CSR with
    int64 row pointers, int32 columns, float64 values).  Returns (r, norm2)."""
    import torch
    L = load_library()
    n = x.numel()
    r = torch.empty_like(x)
    nrm = torch.empty(1, dtype=torch.float64, device=x.device)
    rc = L.dg_residual_csr(n, rowptr.data_ptr(), col.data_ptr(), val.data_ptr(), x.data_ptr(),
                           b.data_ptr(), r.data_ptr(), nrm.data_ptr(), stream)
    if rc != DG_OK:
        raise DougError(rc, "dg_residual_csr failed")
    return r, nrm


class DougSolver:
    """One linear system and its preconditioner on one GPU (a ``dg_handle``)."""

    def __init__(self, options: dict | None = None, ctl: str | None = None):
        self._L = load_library()
        self._h = C.c_void_p()
        self._check(self._L.dg_create(C.byref(self._h)))
        if ctl is not None:
            self.load_ctl(ctl)
        for k, v in (options or {}).items():
            self.set_option(k, v)

    def __del__(self):
        try:
            if self._h:
                self._L.dg_destroy(self._h)
                self._h = C.c_void_p()
        except Exception:
            pass

    def _check(self, rc, allow=()):
        if rc != DG_OK and rc not in allow:
            msg = self._L.dg_last_error(self._h) if self._h else b""
            raise DougError(rc, (msg or b"").decode(errors="replace"))
        return rc

    # --- inputs -----------------------------------------------------------
    def set_option(self, name: str, value) -> None:
        if isinstance(value, bool):
            value = "T" if value else "F"
        self._check(self._L.dg_set_option(self._h, name.encode(), str(value).encode()))

    def load_ctl(self, path: str) -> None:
        self._check(self._L.dg_load_ctl(self._h, path.encode()))

    def set_matrix_coo(self, n: int, rows1, cols1, vals) -> None:
        r = np.ascontiguousarray(rows1, dtype=np.int32)
        c = np.ascontiguousarray(cols1, dtype=np.int32)
        v = np.ascontiguousarray(vals, dtype=np.float64)
        self._check(self._L.dg_set_matrix_coo(self._h, int(n), len(v), _ip(r), _ip(c), _dp(v)))

    def set_elements(self, ngf: int, eptr, efree, emat, erhs) -> None:
        """Elemental input (the in-memory form of DOUG's input_type 1 files):
        element e has the 1-based freedoms efree[eptr[e]:eptr[e+1]], its
        matrix column by column in emat and its right-hand side in erhs."""
        ep = np.ascontiguousarray(eptr, dtype=np.int32)
        ef = np.ascontiguousarray(efree, dtype=np.int32)
        em = np.ascontiguousarray(emat, dtype=np.float64)
        er = np.ascontiguousarray(erhs, dtype=np.float64)
        self._check(self._L.dg_set_elements(self._h, len(ep) - 1, int(ngf), _ip(ep), _ip(ef), _dp(em), _dp(er)))

    def set_node_geometry(self, coords, freemap) -> None:
        """Node coordinates (nnode x nsd, nsd 2 or 3) and the 1-based node of
        every global freedom, after set_elements: the input of doug_geom's
        geometric coarse grid (control word executable geom, levels 2)."""
        xyz = np.ascontiguousarray(coords, dtype=np.float64)
        fm = np.ascontiguousarray(freemap, dtype=np.int32)
        self._check(self._L.dg_set_node_geometry(self._h, xyz.shape[1], xyz.shape[0], _dp(xyz), _ip(fm)))

    def coarse_coords(self):
        """Coordinates of the geometric coarse grid's coarse freedoms, one row each."""
        nsd, nc = C.c_int(), C.c_int()
        self._check(self._L.dg_get_coarse_coords(self._h, C.byref(nsd), C.byref(nc), None))
        buf = np.zeros(nsd.value * nc.value, dtype=np.float64)
        self._check(self._L.dg_get_coarse_coords(self._h, None, None, _dp(buf)))
        return buf.reshape(nc.value, nsd.value)

    def grad_matrix(self, d_lambda: int, d_x: int, d_grad: int, stream: int = 0) -> None:
        """d_grad[k] = -lambda[row_k] x[col_k] per input triplet (device pointers)."""
        self._check(self._L.dg_grad_matrix(self._h, C.c_void_p(d_lambda), C.c_void_p(d_x), C.c_void_p(d_grad),
                                           C.c_void_p(stream)))

    def grad_elements(self, d_lambda: int, d_x: int, d_grad: int, stream: int = 0) -> None:
        """d_grad[e] = dL/ds_e for a factor scaling element e's matrix (device pointers)."""
        self._check(self._L.dg_grad_elements(self._h, C.c_void_p(d_lambda), C.c_void_p(d_x),
                                             C.c_void_p(d_grad), C.c_void_p(stream)))

    def input_matrix(self):
        """(n, rows1, cols1, vals, rhs) the handle holds, in entry order."""
        n, nnz = C.c_int(), C.c_int()
        self._check(self._L.dg_get_input(self._h, C.byref(n), C.byref(nnz), None, None, None, None))
        r = np.zeros(nnz.value, np.int32)
        c = np.zeros(nnz.value, np.int32)
        v = np.zeros(nnz.value, np.float64)
        b = np.zeros(n.value, np.float64)
        self._check(self._L.dg_get_input(self._h, None, None, _ip(r), _ip(c), _dp(v), _dp(b)))
        return n.value, r, c, v, b

    def set_rhs(self, b) -> None:
        b = np.ascontiguousarray(b, dtype=np.float64)
        self._check(self._L.dg_set_rhs(self._h, _dp(b)))

    def set_partition(self, part) -> None:
        p = np.ascontiguousarray(part, dtype=np.int32)
        self._check(self._L.dg_set_partition(self._h, _ip(p), int(p.max())))

    # --- setup / solve ----------------------------------------------------
    def setup(self) -> None:
        self._check(self._L.dg_setup(self._h))

    def set_systems(self, systems, rhs=None) -> None:
        """Batched independent systems: ``systems`` is a sequence of
        (n, rows1, cols1, vals) with 1-based indices per system; ``rhs`` an
        optional sequence of right-hand sides (default b = 1).  dg_solve then
        takes and returns the concatenated vectors; system_stats() gives the
        per-system iterations, status, residuals and times."""
        ns = np.array([int(t[0]) for t in systems], np.int32)
        nz = np.array([len(t[3]) for t in systems], np.int64)
        r = np.ascontiguousarray(np.concatenate([np.asarray(t[1], np.int32) for t in systems]))
        c = np.ascontiguousarray(np.concatenate([np.asarray(t[2], np.int32) for t in systems]))
        v = np.ascontiguousarray(np.concatenate([np.asarray(t[3], np.float64) for t in systems]))
        b = None
        if rhs is not None:
            b = np.ascontiguousarray(np.concatenate([np.asarray(x, np.float64) for x in rhs]))
            if b.shape[0] != int(ns.sum()):
                raise ValueError("right-hand sides do not match the systems' sizes")
        self._check(self._L.dg_set_systems(self._h, len(systems), _ip(ns), nz.ctypes.data_as(C.POINTER(C.c_longlong)),
                                           _ip(r), _ip(c), _dp(v), _dp(b) if b is not None else None))
        self._sys_n = ns

    def solve_multi(self, B, allow_not_converged: bool = False):
        """Solves A X = B for the columns of B (n x nrhs) together; returns
        (X, stats).  Per right-hand side: system_stats()."""
        B = np.asarray(B, dtype=np.float64)
        n, k = B.shape
        Bt = np.ascontiguousarray(B.T)            # right-hand sides one after the other
        Xt = np.zeros_like(Bt)
        st = _Stats()
        rc = self._L.dg_solve_multi(self._h, k, _dp(Bt), _dp(Xt), C.byref(st))
        self._check(rc, allow=(DG_NOT_CONVERGED,) if allow_not_converged else ())
        self._sys_n = np.full(k, n, np.int32)
        return Xt.T.copy(), self._stats(rc, st)

    def solve_multi_device(self, nrhs: int, b_ptr: int, x_ptr: int, stream: int = 0, allow_not_converged=False):
        """solve_multi with device pointers: nrhs vectors of n doubles one after the other."""
        st = _Stats()
        rc = self._L.dg_solve_multi_device(self._h, int(nrhs), C.c_void_p(b_ptr), C.c_void_p(x_ptr), C.byref(st),
                                           C.c_void_p(stream))
        self._check(rc, allow=(DG_NOT_CONVERGED,) if allow_not_converged else ())
        self._sys_n = np.full(int(nrhs), self.sizes()["n"], np.int32)
        return self._stats(rc, st)

    def system_stats(self) -> dict:
        """Per-system results of the last batched solve, or per right-hand
        side of the last solve_multi (numpy arrays)."""
        k = len(self._sys_n)
        it = np.zeros(k, np.int32)
        stt = np.zeros(k, np.int32)
        rel = np.zeros(k)
        sec = np.zeros(k)
        self._check(self._L.dg_get_system_stats(self._h, _ip(it), _ip(stt), _dp(rel), _dp(sec)))
        return {"iterations": it, "status": stt, "rel_residual": rel, "seconds": sec}

    def split(self, x):
        """Splits a concatenated batched vector into the systems' vectors."""
        return np.split(np.asarray(x), np.cumsum(self._sys_n)[:-1])

    def autotune(self) -> tuple[dict, float]:
        """Time full solves of the stored right-hand side over a grid of the
        batch parameters (nd_leaf, panel_rows, fwd_task_kb, lean_task_kb),
        keep the fastest and leave the solver set up with it.  Returns the
        chosen words and the fastest factor + iterate time in seconds."""
        t = C.c_double(0.0)
        ch = (C.c_int * 4)()
        self._check(self._L.dg_autotune(self._h, C.byref(t), ch))
        keys = ("nd_leaf", "panel_rows", "fwd_task_kb", "lean_task_kb")
        return {k: int(ch[i]) for i, k in enumerate(keys)}, t.value

    def setup_host_only(self) -> int:
        """Run the host setup; a missing GPU is reported, not raised.  The
        parity export (aggregates, subdomains, R, AC) is available after it."""
        return self._check(self._L.dg_setup(self._h), allow=(DG_NO_DEVICE, DG_CUDA_ERROR))

    def solve(self, b=None, allow_not_converged: bool = False):
        n = self.sizes()["n"]
        x = np.zeros(n, dtype=np.float64)
        st = _Stats()
        bb = None if b is None else np.ascontiguousarray(b, dtype=np.float64)
        rc = self._L.dg_solve(self._h, _dp(bb) if bb is not None else None, _dp(x), C.byref(st))
        self._check(rc, allow=(DG_NOT_CONVERGED,) if allow_not_converged else ())
        return x, self._stats(rc, st)

    def solve_device(self, b_ptr: int, x_ptr: int, stream: int = 0, allow_not_converged=False):
        """Solve with device pointers (e.g. ``tensor.data_ptr()``) on a CUDA stream."""
        st = _Stats()
        rc = self._L.dg_solve_device(self._h, C.c_void_p(b_ptr), C.c_void_p(x_ptr), C.byref(st),
                                     C.c_void_p(stream))
        self._check(rc, allow=(DG_NOT_CONVERGED,) if allow_not_converged else ())
        return self._stats(rc, st)

    def write_solution(self, x) -> None:
        x = np.ascontiguousarray(x, dtype=np.float64)
        self._check(self._L.dg_write_solution(self._h, _dp(x)))

    @staticmethod
    def _stats(rc, st):
        return SolveStats(rc, st.iterations, st.init_norm, st.final_norm, st.true_rel_residual,
                          st.cond_num, st.t_setup_s, st.t_factor_s, st.t_iterate_s, st.t_total_s,
                          st.n, st.nsubdomains, st.ncoarse, st.gpu_launches, st.factor_nnz,
                          st.factor_gflop, st.t_subsolve_s, st.subsolve_bytes, st.t_coarse_s,
                          st.coarse_bytes, st.t_spmv_s, st.spmv_bytes)

    # --- parity export ----------------------------------------------------
    def setup_phases(self) -> dict:
        """Seconds of the last setup: host part up to the fine aggregates,
        restriction + Galerkin product (device time when on the GPU), total."""
        a, c, t = C.c_double(), C.c_double(), C.c_double()
        d = C.c_int()
        self._check(self._L.dg_get_setup_phases(self._h, C.byref(a), C.byref(c), C.byref(d), C.byref(t)))
        return {"aggregation_s": a.value, "coarse_s": c.value, "coarse_on_device": bool(d.value),
                "total_s": t.value}

    def sizes(self) -> dict:
        v = [C.c_int() for _ in range(4)]
        tot = C.c_longlong()
        rn, an = C.c_int(), C.c_int()
        self._check(self._L.dg_get_sizes(self._h, C.byref(v[0]), C.byref(v[1]), C.byref(v[2]),
                                         C.byref(v[3]), C.byref(tot), C.byref(rn), C.byref(an)))
        return {"n": v[0].value, "nagr_fine": v[1].value, "nagr_coarse": v[2].value,
                "nsubdomains": v[3].value, "subdomain_total": tot.value, "R_nnz": rn.value,
                "AC_nnz": an.value}

    def aggregates(self):
        s = self.sizes()
        f = np.zeros(s["n"], dtype=np.int32)
        c = np.zeros(max(s["nagr_fine"], 1), dtype=np.int32)
        self._check(self._L.dg_get_aggregates(self._h, _ip(f), _ip(c)))
        return f, c[: s["nagr_fine"]]

    def subdomains(self):
        s = self.sizes()
        st = np.zeros(s["nsubdomains"] + 1, dtype=np.int64)
        nd = np.zeros(max(s["subdomain_total"], 1), dtype=np.int32)
        self._check(self._L.dg_get_subdomains(self._h, st.ctypes.data_as(C.POINTER(C.c_longlong)),
                                              _ip(nd)))
        return [nd[st[i]:st[i + 1]].copy() for i in range(s["nsubdomains"])]

    def restriction(self):
        s = self.sizes()
        k = s["R_nnz"]
        i, j, v = np.zeros(k, np.int32), np.zeros(k, np.int32), np.zeros(k, np.float64)
        self._check(self._L.dg_get_restriction(self._h, _ip(i), _ip(j), _dp(v)))
        return i, j, v

    def coarse_matrix(self):
        s = self.sizes()
        k = s["AC_nnz"]
        i, j, v = np.zeros(k, np.int32), np.zeros(k, np.int32), np.zeros(k, np.float64)
        self._check(self._L.dg_get_coarse_matrix(self._h, _ip(i), _ip(j), _dp(v)))
        return i, j, v
