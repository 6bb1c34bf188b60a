"""ctypes front end of the C oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module, and only as the checker.  It builds
``oracle/_build/libdougoracle.so`` from ``oracle/doug_oracle.c`` on first use
(gcc, no GPU needed).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libdougoracle.so")
_lock = threading.Lock()
_lib = None


class _Result(C.Structure):
    _fields_ = [
        ("status", C.c_int), ("errmsg", C.c_char * 512), ("n", C.c_int),
        ("x", C.POINTER(C.c_double)), ("b", C.POINTER(C.c_double)),
        ("iterations", C.c_int), ("cond_num", C.c_double), ("init_norm", C.c_double),
        ("res_hist", C.POINTER(C.c_double)),
        ("nagr_fine", C.c_int), ("aggr_fine", C.POINTER(C.c_int)),
        ("nagr_fine_full", C.c_int), ("aggr_fine_full", C.POINTER(C.c_int)),
        ("nagr_coarse", C.c_int), ("aggr_coarse", C.POINTER(C.c_int)),
        ("nagr_coarse_full", C.c_int), ("aggr_coarse_full", C.POINTER(C.c_int)),
        ("nsubd", C.c_int), ("subd_starts", C.POINTER(C.c_int)), ("subd_nodes", C.POINTER(C.c_int)),
        ("R_nrows", C.c_int), ("R_ncols", C.c_int), ("R_nnz", C.c_int),
        ("R_i", C.POINTER(C.c_int)), ("R_j", C.POINTER(C.c_int)), ("R_v", C.POINTER(C.c_double)),
        ("AC_n", C.c_int), ("AC_nnz", C.c_int),
        ("AC_i", C.POINTER(C.c_int)), ("AC_j", C.POINTER(C.c_int)), ("AC_v", C.POINTER(C.c_double)),
        ("overlap", C.c_int), ("smoothers", C.c_int), ("levels", C.c_int), ("method", C.c_int),
        ("strong1", C.c_double), ("strong2", C.c_double),
        ("radius1", C.c_int), ("radius2", C.c_int), ("minasize1", C.c_int), ("maxasize1", C.c_int),
        ("minasize2", C.c_int), ("maxasize2", C.c_int),
        ("tol", C.c_double), ("maxit", C.c_int),
        ("t_setup", C.c_double), ("t_factor", C.c_double), ("t_solve", C.c_double),
        ("cnsd", C.c_int), ("cxyz", C.POINTER(C.c_double)),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc)."""
    srcs = [os.path.join(_HERE, f) for f in ("doug_oracle.c", "doug_oracle.h", "spchol.c", "spchol.h",
                                               "Makefile")]
    if force or not os.path.exists(_SO) or os.path.getmtime(_SO) < max(os.path.getmtime(f) for f in srcs):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _SO


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_SO)
            P = C.POINTER
            L.orc_run_coo.argtypes = [C.c_int, C.c_int, P(C.c_int), P(C.c_int), P(C.c_double),
                                      P(C.c_double), C.c_char_p, P(C.c_int), C.c_int,
                                      P(P(_Result))]
            L.orc_setup_coo.argtypes = [C.c_int, C.c_int, P(C.c_int), P(C.c_int), P(C.c_double),
                                        C.c_char_p, P(C.c_int), C.c_int, P(P(_Result))]
            L.orc_run_ctl.argtypes = [C.c_char_p, C.c_char_p, P(P(_Result))]
            L.orc_run_ctl_part.argtypes = [C.c_char_p, C.c_char_p, P(C.c_int), C.c_int, P(P(_Result))]
            L.orc_free.argtypes = [P(_Result)]
            L.orc_read_assembled.argtypes = [C.c_char_p, C.c_int, P(C.c_int), P(C.c_int),
                                             P(P(C.c_int)), P(P(C.c_int)), P(P(C.c_double))]
            L.orc_read_vector.argtypes = [C.c_char_p, C.c_int, C.c_int, P(C.c_double)]
            L.orc_read_elemental.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, P(C.c_int),
                                             P(C.c_int), P(P(C.c_int)), P(P(C.c_int)),
                                             P(P(C.c_double)), P(P(C.c_double))]
            L.orc_free_buffers.argtypes = [C.c_void_p] * 4
            L.orc_write_solution.argtypes = [C.c_char_p, C.c_int, C.c_int, P(C.c_double)]
            L.orc_spd_solve.argtypes = [C.c_int, C.c_int, P(C.c_int), P(C.c_int), P(C.c_double),
                                        P(C.c_double), P(C.c_double)]
            L.orc_spd_factor.argtypes = [C.c_int, C.c_int, P(C.c_int), P(C.c_int), P(C.c_double)]
            L.orc_spd_factor.restype = C.c_void_p
            L.orc_spd_solve_factored.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
            L.orc_spd_free.argtypes = [C.c_void_p]
            L.orc_session_new.argtypes = [C.c_int, C.c_int, P(C.c_int), P(C.c_int), P(C.c_double),
                                          C.c_char_p, P(C.c_int), C.c_int, P(C.c_void_p),
                                          P(P(_Result))]
            L.orc_session_solve.argtypes = [C.c_void_p, P(C.c_double), P(P(_Result))]
            L.orc_session_free.argtypes = [C.c_void_p]
            L.orc_set_threads.argtypes = [C.c_int]
            L.orc_set_geometry.argtypes = [C.c_int, C.c_int, P(C.c_double), C.c_int, P(C.c_int)]
            for nm in ("orc_parse_i10", "orc_parse_l1"):
                getattr(L, nm).argtypes = [C.c_char_p, P(C.c_int)]
            L.orc_parse_f10_5.argtypes = [C.c_char_p, P(C.c_double)]
            _lib = L
    return _lib


def _arr(ptr, n, dtype):
    if n <= 0 or not ptr:
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


class OracleResult(dict):
    """Plain dict of numpy arrays and scalars copied out of the C result."""


def _convert(res_p) -> OracleResult:
    r = res_p.contents
    out = OracleResult()
    out["status"] = r.status
    out["errmsg"] = r.errmsg.decode(errors="replace")
    if r.status != 0:
        return out
    n = r.n
    out["n"] = n
    out["x"] = _arr(r.x, n, np.float64) if r.x else None
    out["b"] = _arr(r.b, n, np.float64)
    out["iterations"] = r.iterations
    out["cond_num"] = r.cond_num
    out["init_norm"] = r.init_norm
    out["res_hist"] = _arr(r.res_hist, r.iterations, np.float64) if r.res_hist else None
    out["nagr_fine"] = r.nagr_fine
    out["aggr_fine"] = _arr(r.aggr_fine, n, np.int32)
    out["nagr_fine_full"] = r.nagr_fine_full
    out["aggr_fine_full"] = _arr(r.aggr_fine_full, n, np.int32)
    out["nagr_coarse"] = r.nagr_coarse
    out["aggr_coarse"] = _arr(r.aggr_coarse, r.nagr_fine, np.int32)
    out["nagr_coarse_full"] = r.nagr_coarse_full
    out["aggr_coarse_full"] = _arr(r.aggr_coarse_full, r.nagr_fine, np.int32)
    ns = r.nsubd
    starts = _arr(r.subd_starts, ns + 1, np.int64)
    nodes = _arr(r.subd_nodes, int(starts[-1]) if ns > 0 else 0, np.int32)
    out["subdomains"] = [nodes[starts[i]:starts[i + 1]] for i in range(ns)]
    out["R"] = (r.R_nrows, r.R_ncols, _arr(r.R_i, r.R_nnz, np.int32),
                _arr(r.R_j, r.R_nnz, np.int32), _arr(r.R_v, r.R_nnz, np.float64))
    out["AC"] = (r.AC_n, _arr(r.AC_i, r.AC_nnz, np.int32), _arr(r.AC_j, r.AC_nnz, np.int32),
                 _arr(r.AC_v, r.AC_nnz, np.float64))
    out["coarse_xyz"] = (_arr(r.cxyz, r.cnsd * r.AC_n, np.float64).reshape(r.AC_n, r.cnsd)
                         if r.cnsd > 0 else None)
    for k in ("overlap", "smoothers", "levels", "method", "strong1", "strong2", "radius1",
              "radius2", "minasize1", "maxasize1", "minasize2", "maxasize2", "tol", "maxit",
              "t_setup", "t_factor", "t_solve"):
        out[k] = getattr(r, k)
    return out


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def run_coo(n, rows1, cols1, vals, rhs=None, ctl="", part=None, setup_only=False):
    """Run the oracle on 1-based COO triplets (assembled-file semantics)."""
    L = lib()
    ii = np.ascontiguousarray(rows1, dtype=np.int32)
    jj = np.ascontiguousarray(cols1, dtype=np.int32)
    vv = np.ascontiguousarray(vals, dtype=np.float64)
    res = C.POINTER(_Result)()
    pp = None
    npart = 0
    if part is not None:
        pp = np.ascontiguousarray(part, dtype=np.int32)
        npart = int(pp.max())
    if setup_only:
        L.orc_setup_coo(n, len(vv), _ip(ii), _ip(jj), _dp(vv), ctl.encode(),
                        _ip(pp) if pp is not None else None, npart, C.byref(res))
    else:
        bb = None if rhs is None else np.ascontiguousarray(rhs, dtype=np.float64)
        L.orc_run_coo(n, len(vv), _ip(ii), _ip(jj), _dp(vv), _dp(bb) if bb is not None else None,
                      ctl.encode(), _ip(pp) if pp is not None else None, npart, C.byref(res))
    out = _convert(res)
    L.orc_free(res)
    return out


def run_ctl(path, overrides="", part=None):
    """Run the oracle on a control file; part: optional 1-based partition of
    the unknowns replacing the default subdomains."""
    L = lib()
    res = C.POINTER(_Result)()
    if part is None:
        L.orc_run_ctl(path.encode(), overrides.encode(), C.byref(res))
    else:
        pp = np.ascontiguousarray(part, dtype=np.int32)
        L.orc_run_ctl_part(path.encode(), overrides.encode(), _ip(pp), int(pp.max()), C.byref(res))
    out = _convert(res)
    L.orc_free(res)
    return out


def read_assembled(path, fmt=0):
    L = lib()
    n = C.c_int()
    nnz = C.c_int()
    ii = C.POINTER(C.c_int)()
    jj = C.POINTER(C.c_int)()
    vv = C.POINTER(C.c_double)()
    rc = L.orc_read_assembled(path.encode(), fmt, C.byref(n), C.byref(nnz), C.byref(ii),
                              C.byref(jj), C.byref(vv))
    if rc:
        raise IOError(f"oracle could not read {path}: {rc}")
    m = max(n.value, nnz.value)
    return (n.value, nnz.value, _arr(ii, m, np.int32), _arr(jj, m, np.int32), _arr(vv, m, np.float64))


def read_elemental(info, freelists, elemmat, number_of_blocks=1):
    """Elemental input files assembled as one DOUG process assembles them:
    (n, rows1, cols1, vals, rhs), the COO in the reference's entry order."""
    L = lib()
    n, nnz = C.c_int(), C.c_int()
    ii, jj = C.POINTER(C.c_int)(), C.POINTER(C.c_int)()
    vv, bb = C.POINTER(C.c_double)(), C.POINTER(C.c_double)()
    rc = L.orc_read_elemental(info.encode(), freelists.encode(), elemmat.encode(), int(number_of_blocks),
                              C.byref(n), C.byref(nnz), C.byref(ii), C.byref(jj), C.byref(vv), C.byref(bb))
    if rc:
        raise RuntimeError(f"orc_read_elemental failed ({rc})")
    out = (n.value, np.ctypeslib.as_array(ii, (nnz.value,)).copy(),
           np.ctypeslib.as_array(jj, (nnz.value,)).copy(), np.ctypeslib.as_array(vv, (nnz.value,)).copy(),
           np.ctypeslib.as_array(bb, (n.value,)).copy())
    L.orc_free_buffers(C.cast(ii, C.c_void_p), C.cast(jj, C.c_void_p), C.cast(vv, C.c_void_p),
                       C.cast(bb, C.c_void_p))
    return out


def read_vector(path, fmt, n):
    L = lib()
    x = np.zeros(n, dtype=np.float64)
    rc = L.orc_read_vector(path.encode(), fmt, n, _dp(x))
    if rc:
        raise IOError(f"oracle could not read vector {path}: {rc}")
    return x


def write_solution(path, fmt, x):
    L = lib()
    x = np.ascontiguousarray(x, dtype=np.float64)
    rc = L.orc_write_solution(path.encode(), fmt, len(x), _dp(x))
    if rc:
        raise IOError(f"oracle could not write {path}: {rc}")


def spd_solve(n, rows0, cols0, vals, b):
    L = lib()
    ii = np.ascontiguousarray(rows0, dtype=np.int32)
    jj = np.ascontiguousarray(cols0, dtype=np.int32)
    vv = np.ascontiguousarray(vals, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(n, dtype=np.float64)
    rc = L.orc_spd_solve(n, len(vv), _ip(ii), _ip(jj), _dp(vv), _dp(bb), _dp(x))
    if rc:
        raise RuntimeError("oracle SPD solve failed")
    return x


def parse_value(kind, text):
    L = lib()
    if kind == "i10":
        v = C.c_int()
        rc = L.orc_parse_i10(text.encode(), C.byref(v))
    elif kind == "f10.5":
        v = C.c_double()
        rc = L.orc_parse_f10_5(text.encode(), C.byref(v))
    else:
        v = C.c_int()
        rc = L.orc_parse_l1(text.encode(), C.byref(v))
    if rc:
        raise ValueError(text)
    return v.value


class SpdFactor:
    """Exact SPD factorisation of the oracle (nested dissection + multifrontal Cholesky)."""

    def __init__(self, n, rows0, cols0, vals):
        L = lib()
        ii = np.ascontiguousarray(rows0, dtype=np.int32)
        jj = np.ascontiguousarray(cols0, dtype=np.int32)
        vv = np.ascontiguousarray(vals, dtype=np.float64)
        self.n = n
        self._L = L
        self._f = L.orc_spd_factor(n, len(vv), _ip(ii), _ip(jj), _dp(vv))
        if not self._f:
            raise RuntimeError("oracle factorisation failed")

    def solve(self, b):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.n, dtype=np.float64)
        self._L.orc_spd_solve_factored(self._f, _dp(b), _dp(x))
        return x

    def __del__(self):
        try:
            if self._f:
                self._L.orc_spd_free(self._f)
                self._f = None
        except Exception:
            pass


def set_geometry(coords=None, unode=None):
    """Node geometry for coarse_method 3 (used by the following runs):
    coords (nnode x nsd) and the 1-based node of every unknown.  No
    arguments: clear it."""
    L = lib()
    if coords is None:
        L.orc_set_geometry(0, 0, None, 0, None)
        return
    xyz = np.ascontiguousarray(coords, dtype=np.float64)
    un = np.ascontiguousarray(unode, dtype=np.int32)
    L.orc_set_geometry(xyz.shape[1], xyz.shape[0], _dp(xyz), len(un), _ip(un))


def set_threads(n):
    """Host threads of the oracle's factorisations, subdomain solves and
    vector loops (results do not depend on the count)."""
    lib().orc_set_threads(int(n))


class Session:
    """The oracle's setup kept for repeated solves: ``setup`` holds the setup
    result (aggregates, subdomains, R, AC, t_setup); ``solve(b)`` runs the
    numeric factorisations and the PCG and returns the solve result."""

    def __init__(self, n, rows1, cols1, vals, ctl="", part=None):
        L = lib()
        self._L = L
        ii = np.ascontiguousarray(rows1, dtype=np.int32)
        jj = np.ascontiguousarray(cols1, dtype=np.int32)
        vv = np.ascontiguousarray(vals, dtype=np.float64)
        pp, npart = None, 0
        if part is not None:
            pp = np.ascontiguousarray(part, dtype=np.int32)
            npart = int(pp.max())
        res = C.POINTER(_Result)()
        self._s = C.c_void_p()
        L.orc_session_new(n, len(vv), _ip(ii), _ip(jj), _dp(vv), ctl.encode(),
                          _ip(pp) if pp is not None else None, npart, C.byref(self._s), C.byref(res))
        self.setup = _convert(res)
        L.orc_free(res)
        if self.setup["status"] != 0:
            raise RuntimeError("oracle setup failed: " + self.setup["errmsg"])
        self.n = n

    def solve(self, b=None):
        res = C.POINTER(_Result)()
        bb = None if b is None else np.ascontiguousarray(b, dtype=np.float64)
        self._L.orc_session_solve(self._s, _dp(bb) if bb is not None else None, C.byref(res))
        r = res.contents
        out = {"status": r.status, "errmsg": r.errmsg.decode(errors="replace")}
        if r.status == 0:
            out.update(x=_arr(r.x, self.n, np.float64), iterations=r.iterations, cond_num=r.cond_num,
                       init_norm=r.init_norm, res_hist=_arr(r.res_hist, r.iterations, np.float64),
                       t_factor=r.t_factor, t_solve=r.t_solve)
        self._L.orc_free(res)
        return out

    def close(self):
        if self._s:
            self._L.orc_session_free(self._s)
            self._s = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
