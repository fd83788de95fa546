"""ctypes bindings for the CPU oracle (oracle/oracle.c) and the reference harness.

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by
the CPU-baseline leg of ``bench.py``.  The GPU library never imports this package.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

_i64p = ctypes.POINTER(ctypes.c_int64)
_f32p = ctypes.POINTER(ctypes.c_float)
_lib = None


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and, with ref=True, RNNG's drivers + harness)."""
    targets = ["all"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_l2seq.restype = ctypes.c_float
        L.orc_l2seq.argtypes = [_f32p, _f32p, ctypes.c_int64]
        L.orc_edit.restype = ctypes.c_float
        L.orc_edit.argtypes = [ctypes.c_char_p, ctypes.c_int64, ctypes.c_char_p, ctypes.c_int64]
        L.orc_eps_graph_l2.restype = ctypes.c_int64
        L.orc_eps_graph_l2.argtypes = [_f32p, ctypes.c_int64, ctypes.c_int64, ctypes.c_float, ctypes.c_int64,
                                       ctypes.c_int64, ctypes.POINTER(_i64p), ctypes.POINTER(_i64p),
                                       ctypes.POINTER(_f32p)]
        L.orc_cross_l2.restype = ctypes.c_int64
        L.orc_cross_l2.argtypes = [_f32p, ctypes.c_int64, _f32p, ctypes.c_int64, ctypes.c_int64, ctypes.c_float,
                                   ctypes.POINTER(_i64p), ctypes.POINTER(_i64p), ctypes.POINTER(_f32p)]
        L.orc_eps_graph_edit.restype = ctypes.c_int64
        L.orc_eps_graph_edit.argtypes = [ctypes.c_void_p, _i64p, ctypes.c_int64, ctypes.c_float, ctypes.c_int64,
                                         ctypes.c_int64, ctypes.POINTER(_i64p), ctypes.POINTER(_i64p),
                                         ctypes.POINTER(_f32p)]
        L.orc_binom.restype = ctypes.c_int64
        L.orc_binom.argtypes = [ctypes.c_int64, ctypes.c_int64]
        L.orc_simplex_id.restype = ctypes.c_int64
        L.orc_simplex_id.argtypes = [_i64p, ctypes.c_int64]
        L.orc_rips.restype = ctypes.c_int64
        L.orc_rips.argtypes = [ctypes.c_int64, _i64p, _i64p, _f32p, ctypes.c_int64, ctypes.c_int,
                               ctypes.POINTER(_i64p), ctypes.POINTER(_f32p)]
        L.orc_voronoi.argtypes = [_f32p, ctypes.c_int64, _f32p, ctypes.c_int64, ctypes.c_int64, _i64p, _f32p]
        L.orc_free.argtypes = [ctypes.c_void_p]
        L.orc_num_threads.restype = ctypes.c_int
        L.orc_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def num_threads() -> int:
    return int(lib().orc_num_threads())


def set_threads(t: int) -> None:
    lib().orc_set_threads(int(t))


def _take(ptr, n, dtype):
    if n == 0:
        out = np.zeros(0, dtype=dtype)
    else:
        out = np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)
    lib().orc_free(ctypes.cast(ptr, ctypes.c_void_p))
    return out


def _edges(n, pu, pv, pw, sort=True):
    u = _take(pu, n, np.int64)
    v = _take(pv, n, np.int64)
    w = _take(pw, n, np.float32)
    if sort:
        order = np.lexsort((v, u))
        u, v, w = u[order], v[order], w[order]
    return u, v, w


def l2seq(p: np.ndarray, q: np.ndarray) -> np.float32:
    p = np.ascontiguousarray(p, np.float32)
    q = np.ascontiguousarray(q, np.float32)
    return np.float32(lib().orc_l2seq(p.ctypes.data_as(_f32p), q.ctypes.data_as(_f32p), p.size))


def edit(s: bytes, t: bytes) -> np.float32:
    return np.float32(lib().orc_edit(s, len(s), t, len(t)))


def eps_graph_l2(X: np.ndarray, eps, rows: tuple[int, int] | None = None):
    """All unordered pairs i<j (i in rows) with the reference L2 <= eps, sorted by (u, v)."""
    X = np.ascontiguousarray(X, np.float32)
    n, d = X.shape
    r0, r1 = rows if rows is not None else (0, n)
    pu, pv, pw = _i64p(), _i64p(), _f32p()
    cnt = lib().orc_eps_graph_l2(X.ctypes.data_as(_f32p), n, d, ctypes.c_float(eps), r0, r1,
                                 ctypes.byref(pu), ctypes.byref(pv), ctypes.byref(pw))
    return _edges(cnt, pu, pv, pw)


def cross_l2(X: np.ndarray, Q: np.ndarray, eps):
    """All (query row, point row) pairs with the reference L2 <= eps, sorted."""
    X = np.ascontiguousarray(X, np.float32)
    Q = np.ascontiguousarray(Q, np.float32)
    pu, pv, pw = _i64p(), _i64p(), _f32p()
    cnt = lib().orc_cross_l2(X.ctypes.data_as(_f32p), X.shape[0], Q.ctypes.data_as(_f32p), Q.shape[0],
                             X.shape[1], ctypes.c_float(eps), ctypes.byref(pu), ctypes.byref(pv), ctypes.byref(pw))
    return _edges(cnt, pu, pv, pw)


def eps_graph_edit(atoms: np.ndarray, offsets: np.ndarray, eps, rows: tuple[int, int] | None = None):
    atoms = np.ascontiguousarray(atoms, np.uint8)
    offsets = np.ascontiguousarray(offsets, np.int64)
    n = offsets.size - 1
    r0, r1 = rows if rows is not None else (0, n)
    pu, pv, pw = _i64p(), _i64p(), _f32p()
    cnt = lib().orc_eps_graph_edit(atoms.ctypes.data_as(ctypes.c_void_p), offsets.ctypes.data_as(_i64p), n,
                                   ctypes.c_float(eps), r0, r1, ctypes.byref(pu), ctypes.byref(pv),
                                   ctypes.byref(pw))
    return _edges(cnt, pu, pv, pw)


def voronoi(X: np.ndarray, C: np.ndarray):
    X = np.ascontiguousarray(X, np.float32)
    C = np.ascontiguousarray(C, np.float32)
    cell = np.zeros(X.shape[0], np.int64)
    dist = np.zeros(X.shape[0], np.float32)
    lib().orc_voronoi(X.ctypes.data_as(_f32p), X.shape[0], C.ctypes.data_as(_f32p), C.shape[0], X.shape[1],
                      cell.ctypes.data_as(_i64p), dist.ctypes.data_as(_f32p))
    return cell, dist


def binom(n: int, k: int) -> int:
    return int(lib().orc_binom(n, k))


def simplex_id(verts) -> int:
    v = np.ascontiguousarray(sorted(verts), np.int64)
    return int(lib().orc_simplex_id(v.ctypes.data_as(_i64p), v.size))


def rips(n: int, u: np.ndarray, v: np.ndarray, w: np.ndarray, maxdim: int = 2):
    """Filtration (ids, values) sorted by (value, id) from an epsilon graph with u < v."""
    u = np.ascontiguousarray(u, np.int64)
    v = np.ascontiguousarray(v, np.int64)
    w = np.ascontiguousarray(w, np.float32)
    pid, pval = _i64p(), _f32p()
    cnt = lib().orc_rips(n, u.ctypes.data_as(_i64p), v.ctypes.data_as(_i64p), w.ctypes.data_as(_f32p), u.size,
                         maxdim, ctypes.byref(pid), ctypes.byref(pval))
    return _take(pid, cnt, np.int64), _take(pval, cnt, np.float32)


# ----------------------------------------------------------------------------- reference harness

def have_ref() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "ref_harness"))


def read_edge_dump(path: str):
    with open(path, "rb") as f:
        n = int(np.frombuffer(f.read(8), np.int64)[0])
        u = np.frombuffer(f.read(8 * n), np.int64)
        v = np.frombuffer(f.read(8 * n), np.int64)
        w = np.frombuffer(f.read(4 * n), np.float32)
    return u, v, w


def read_simplex_dump(path: str):
    with open(path, "rb") as f:
        n = int(np.frombuffer(f.read(8), np.int64)[0])
        ids = np.frombuffer(f.read(8 * n), np.int64)
        vals = np.frombuffer(f.read(4 * n), np.float32)
    return ids, vals


def reference_graph_semantics(u, v, w):
    """Graph::redistribute_edges at one rank (include/graph.hpp:79-111): both
    orientations of every recorded (u, v, w), sorted by (u, v, w bits), duplicates
    removed.  Returns the unordered edge set u < v (self-loops dropped) with weights."""
    uu = np.concatenate([u, v])
    vv = np.concatenate([v, u])
    ww = np.concatenate([w, w]).view(np.uint32)
    order = np.lexsort((ww, vv, uu))
    uu, vv, ww = uu[order], vv[order], ww[order]
    keep = np.ones(uu.size, bool)
    keep[1:] = (uu[1:] != uu[:-1]) | (vv[1:] != vv[:-1]) | (ww[1:] != ww[:-1])
    uu, vv, ww = uu[keep], vv[keep], ww[keep]
    full_count = uu.size
    sel = uu < vv
    return uu[sel], vv[sel], ww[sel].view(np.float32), full_count


def merge_filtration(ids, vals):
    """merge_and_write_filtration at one rank (include/simplex.hpp:130-196): sort by
    (value, id) and keep the first of each run of equal ids."""
    ids = np.asarray(ids, np.int64)
    vals = np.asarray(vals, np.float32)
    order = np.lexsort((ids, vals))
    ids, vals = ids[order], vals[order]
    keep = np.ones(ids.size, bool)
    keep[1:] = ids[1:] != ids[:-1]
    return ids[keep], vals[keep]
