"""rnng_gb300: GB300-native epsilon-graph / Vietoris-Rips hot path of RNNG.

The compute lives in ``librnng_gpu.so`` (CUDA for sm_103a, C ABI in include/rnng_gpu.h).
This module is a thin ctypes binding over that ABI for tests, the benchmark and
Python users.  There is no CPU fallback: if the library is missing or no GPU is
present, calls raise.

Public API (mirrors the C ABI; point ids default to 0..n-1):

    ctx = Context(device=0)
    u, v, w = ctx.eps_graph_l2(X, radius, mode="bf16")      # unordered edges u < v
    u, v, w = ctx.eps_graph_edit(seqs, radius)
    ids, values = ctx.rips_l2(X, radius, maxdim=2)
    u, v, w = ctx.radius_query_l2(X, Q, radius)              # (query, point) pairs
    cell, dist = ctx.voronoi_l2(X, centers)
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB

RNNG_OK = 0
ERRORS = {1: "INVALID", 2: "CUDA", 3: "NOMEM", 4: "OVERFLOW", 5: "DEVICE", 6: "UNSUPPORTED"}
INPUT_DEVICE = 1
OUTPUT_DEVICE = 2
SORT_OUTPUT = 4
MODES = {"fp32": 0, "bf16": 1}

# every entry point include/rnng_gpu.h declares
EXPORTS = [
    "rnng_ctx_create", "rnng_ctx_destroy", "rnng_last_error", "rnng_get_stats", "rnng_ctx_stream", "rnng_ctx_trim",
    "rnng_ctx_set_gram_tuning", "rnng_gram_probe_bf16", "rnng_ctx_fault_drill",
    "rnng_eps_graph_l2", "rnng_radius_query_l2", "rnng_voronoi_l2", "rnng_eps_graph_edit", "rnng_rips_l2",
    "rnng_graph_finalize", "rnng_edges_free", "rnng_simplices_free", "rnng_eps_graph_l2_static",
    "rnng_voronoi_edit", "rnng_rips_edges",
]


class RnngError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"rnng error {ERRORS.get(code, code)}: {msg}")
        self.code = code


class Edges(ctypes.Structure):
    _fields_ = [("count", ctypes.c_int64), ("u", ctypes.c_void_p), ("v", ctypes.c_void_p), ("w", ctypes.c_void_p),
                ("on_device", ctypes.c_int), ("staged", ctypes.c_int)]


class Simplices(ctypes.Structure):
    _fields_ = [("count", ctypes.c_int64), ("id", ctypes.c_void_p), ("value", ctypes.c_void_p),
                ("on_device", ctypes.c_int), ("staged", ctypes.c_int), ("flag", ctypes.c_void_p)]


class Stats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("ms_total", "ms_h2d", "ms_partition", "ms_sort", "ms_bounds",
                                                 "ms_prune", "ms_tiles", "ms_recheck", "ms_finalize", "ms_d2h")] + \
               [(k, ctypes.c_int64) for k in ("num_cells", "super_pairs", "tile_pairs", "tile_pairs_all", "pairs_evaluated",
                                              "candidates", "edges", "retries", "simplices", "kernel_launches")] + \
               [("ms_gram", ctypes.c_double), ("prune_widen", ctypes.c_double), ("prune_tensor", ctypes.c_int64),
                ("gram_nt", ctypes.c_int64), ("gram_chunk", ctypes.c_int64), ("gram_slots", ctypes.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Loads librnng_gpu.so (building it first when allowed)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError(f"{LIB_PATH} is missing; run rnng_gb300.build.build()")
        _build.build()
    L = ctypes.CDLL(LIB_PATH)
    vp, i64, f32, u32, ip = ctypes.c_void_p, ctypes.c_int64, ctypes.c_float, ctypes.c_uint, ctypes.c_int
    L.rnng_ctx_create.argtypes = [ip, ctypes.POINTER(vp)]
    L.rnng_ctx_destroy.argtypes = [vp]
    L.rnng_last_error.restype = ctypes.c_char_p
    L.rnng_last_error.argtypes = [vp]
    L.rnng_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    L.rnng_ctx_stream.argtypes = [vp, ctypes.POINTER(vp)]
    L.rnng_ctx_trim.argtypes = [vp]
    L.rnng_ctx_set_gram_tuning.argtypes = [vp, ip, ip, ip]
    L.rnng_gram_probe_bf16.argtypes = [vp, vp, i64, vp, vp, vp]
    L.rnng_ctx_fault_drill.argtypes = [vp, ip]
    L.rnng_eps_graph_l2.argtypes = [vp, vp, vp, i64, i64, f32, ip, u32, ctypes.POINTER(Edges)]
    L.rnng_radius_query_l2.argtypes = [vp, vp, vp, i64, vp, vp, i64, i64, f32, u32, ctypes.POINTER(Edges)]
    L.rnng_voronoi_l2.argtypes = [vp, vp, i64, vp, i64, i64, u32, vp, vp]
    L.rnng_eps_graph_edit.argtypes = [vp, vp, vp, vp, i64, f32, u32, ctypes.POINTER(Edges)]
    L.rnng_rips_l2.argtypes = [vp, vp, vp, i64, i64, f32, ip, ip, u32, ctypes.POINTER(Simplices)]
    L.rnng_graph_finalize.argtypes = [vp, ctypes.POINTER(Edges), i64, u32, ctypes.POINTER(Edges)]
    L.rnng_edges_free.argtypes = [ctypes.POINTER(Edges)]
    L.rnng_simplices_free.argtypes = [ctypes.POINTER(Simplices)]
    L.rnng_voronoi_edit.argtypes = [vp, vp, vp, i64, vp, vp, i64, u32, vp, vp]
    L.rnng_rips_edges.argtypes = [vp, i64, vp, vp, vp, vp, vp, i64, ip, u32, ctypes.POINTER(Simplices)]
    L.rnng_eps_graph_l2_static.argtypes = [vp, vp, i64, i64, f32, vp, vp, vp, i64, ctypes.POINTER(i64), vp]
    _lib = L
    return L


def _ptr(a) -> int | None:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return int(a.data_ptr())  # torch tensor (device or pinned host)


def _csr(seqs):
    """(atoms uint8, offsets int64) from a list of bytes or an (atoms, offsets) pair."""
    if isinstance(seqs, tuple):
        atoms, offsets = seqs
    else:
        lens = np.fromiter((len(s) for s in seqs), dtype=np.int64, count=len(seqs))
        offsets = np.zeros(len(seqs) + 1, np.int64)
        np.cumsum(lens, out=offsets[1:])
        atoms = np.frombuffer(b"".join(seqs), np.uint8) if seqs else np.zeros(0, np.uint8)
    atoms = np.ascontiguousarray(atoms, np.uint8)
    if atoms.size == 0:
        atoms = np.zeros(1, np.uint8)
    return atoms, np.ascontiguousarray(offsets, np.int64)


def _host_copy(ptr: int, n: int, dtype) -> np.ndarray:
    if n == 0:
        return np.zeros(0, dtype=dtype)
    nbytes = n * np.dtype(dtype).itemsize
    buf = (ctypes.c_char * nbytes).from_address(ptr)
    return np.frombuffer(buf, dtype=dtype, count=n).copy()


class Context:
    """One GPU, one stream, reusable scratch (rnng_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        self._check(self.lib.rnng_ctx_create(device, ctypes.byref(h)), None)
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.rnng_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int, h) -> None:
        if rc != RNNG_OK:
            msg = self.lib.rnng_last_error(h).decode() if h else "context creation failed"
            raise RnngError(rc, msg)

    def stats(self) -> dict:
        s = Stats()
        self._check(self.lib.rnng_get_stats(self.h, ctypes.byref(s)), self.h)
        return s.as_dict()

    def set_gram_tuning(self, nt: int = 0, chunk: int = 0, slots: int = 0) -> None:
        """Forces the Gram kernel's column tiles per item, queue chunk and B slots (0: the
        tuning table's value or the default)."""
        self._check(self.lib.rnng_ctx_set_gram_tuning(self.h, nt, chunk, slots), self.h)

    def fault_drill(self, on: bool) -> None:
        """rnng_ctx_fault_drill: the Gram kernel's bounded wait runs out on purpose."""
        self._check(self.lib.rnng_ctx_fault_drill(self.h, 1 if on else 0), self.h)

    def gram_probe_bf16(self, X):
        """One tile pair through the Gram kernel (rnng_gram_probe_bf16): X is 256 x d; returns
        (G 128 x 128 raw accumulators, Xb 256 x d BF16 operand rows, rowinfo 256 x 4)."""
        X = np.ascontiguousarray(X, np.float32)
        n, d = X.shape
        G = np.zeros((128, 128), np.float32)
        Xb = np.zeros((n, d), np.float32)
        info = np.zeros((n, 4), np.float32)
        self._check(self.lib.rnng_gram_probe_bf16(self.h, _ptr(X), d, _ptr(G), _ptr(Xb), _ptr(info)), self.h)
        return G, Xb, info

    def stream(self) -> int:
        p = ctypes.c_void_p()
        self._check(self.lib.rnng_ctx_stream(self.h, ctypes.byref(p)), self.h)
        return p.value or 0

    def _edges_out(self, e: Edges):
        if e.on_device:
            return e  # caller frees with free_edges
        u = _host_copy(e.u, e.count, np.int64)
        v = _host_copy(e.v, e.count, np.int64)
        w = _host_copy(e.w, e.count, np.float32)
        return u, v, w

    def free_edges(self, e: Edges) -> None:
        self.lib.rnng_edges_free(ctypes.byref(e))

    # ------------------------------------------------------------------ L2
    def eps_graph_l2(self, X, radius, mode: str = "bf16", ids=None, sort: bool = True, device_io: bool = False):
        """Unordered edges u < v with the reference L2 <= radius.

        X: (n, d) float32 numpy array (host) or, with device_io=True, a CUDA tensor;
        with device_io the result stays on the device (an Edges struct)."""
        if isinstance(X, np.ndarray):
            X = np.ascontiguousarray(X, dtype=np.float32)
            if ids is not None:
                ids = np.ascontiguousarray(ids, dtype=np.int64)
        n, d = X.shape
        flags = (SORT_OUTPUT if sort else 0) | ((INPUT_DEVICE | OUTPUT_DEVICE) if device_io else 0)
        e = Edges()
        rc = self.lib.rnng_eps_graph_l2(self.h, _ptr(X), _ptr(ids), n, d, ctypes.c_float(radius), MODES[mode], flags,
                                        ctypes.byref(e))
        self._check(rc, self.h)
        return self._edges_out(e)

    def eps_graph_l2_raw(self, x_ptr: int, ids_ptr, n: int, d: int, radius, mode: int, flags: int) -> Edges:
        """Direct C-ABI call with raw pointers (benchmark use)."""
        e = Edges()
        rc = self.lib.rnng_eps_graph_l2(self.h, x_ptr, ids_ptr, n, d, ctypes.c_float(radius), mode, flags,
                                        ctypes.byref(e))
        self._check(rc, self.h)
        return e

    def eps_graph_edit_raw(self, atoms_ptr: int, offsets_ptr: int, n: int, radius, flags: int) -> Edges:
        """Direct C-ABI call with raw pointers (benchmark use)."""
        e = Edges()
        rc = self.lib.rnng_eps_graph_edit(self.h, atoms_ptr, offsets_ptr, None, n, ctypes.c_float(radius), flags,
                                          ctypes.byref(e))
        self._check(rc, self.h)
        return e

    def rips_l2_raw(self, x_ptr: int, n: int, d: int, radius, maxdim: int, mode: int, flags: int) -> Simplices:
        """Direct C-ABI call with raw pointers (benchmark use)."""
        s = Simplices()
        rc = self.lib.rnng_rips_l2(self.h, x_ptr, None, n, d, ctypes.c_float(radius), maxdim, mode, flags,
                                   ctypes.byref(s))
        self._check(rc, self.h)
        return s

    def radius_query_l2(self, X, Q, radius, ids=None, qids=None, sort: bool = True):
        X = np.ascontiguousarray(X, dtype=np.float32)
        Q = np.ascontiguousarray(Q, dtype=np.float32)
        ids = None if ids is None else np.ascontiguousarray(ids, np.int64)
        qids = None if qids is None else np.ascontiguousarray(qids, np.int64)
        e = Edges()
        rc = self.lib.rnng_radius_query_l2(self.h, _ptr(X), _ptr(ids), X.shape[0], _ptr(Q), _ptr(qids), Q.shape[0],
                                           X.shape[1], ctypes.c_float(radius), SORT_OUTPUT if sort else 0,
                                           ctypes.byref(e))
        self._check(rc, self.h)
        return self._edges_out(e)

    def voronoi_l2(self, X, C):
        X = np.ascontiguousarray(X, dtype=np.float32)
        C = np.ascontiguousarray(C, dtype=np.float32)
        cell = np.zeros(X.shape[0], np.int64)
        dist = np.zeros(X.shape[0], np.float32)
        rc = self.lib.rnng_voronoi_l2(self.h, _ptr(X), X.shape[0], _ptr(C), C.shape[0], X.shape[1], 0, _ptr(cell),
                                      _ptr(dist))
        self._check(rc, self.h)
        return cell, dist

    # ------------------------------------------------------------------ edit distance
    def eps_graph_edit(self, seqs, radius, ids=None, sort: bool = True):
        """seqs: list of bytes, or (atoms uint8, offsets int64) in CSR form."""
        atoms, offsets = _csr(seqs)
        ids = None if ids is None else np.ascontiguousarray(ids, np.int64)
        e = Edges()
        rc = self.lib.rnng_eps_graph_edit(self.h, _ptr(atoms), _ptr(offsets), _ptr(ids), offsets.size - 1,
                                          ctypes.c_float(radius), SORT_OUTPUT if sort else 0, ctypes.byref(e))
        self._check(rc, self.h)
        return self._edges_out(e)

    def voronoi_edit(self, seqs, centres):
        """Nearest centre per string (edit distance, last of equal wins): (cell, dist)."""
        atoms, offsets = _csr(seqs)
        catoms, coffsets = _csr(centres)
        n = offsets.size - 1
        cell = np.zeros(max(n, 1), np.int64)
        dist = np.zeros(max(n, 1), np.float32)
        rc = self.lib.rnng_voronoi_edit(self.h, _ptr(atoms), _ptr(offsets), n, _ptr(catoms), _ptr(coffsets),
                                        coffsets.size - 1, 0, _ptr(cell), _ptr(dist))
        self._check(rc, self.h)
        return cell[:n], dist[:n]

    # ------------------------------------------------------------------ Rips
    def rips_l2(self, X, radius, maxdim: int = 2, mode: str = "bf16", ids=None):
        X = np.ascontiguousarray(X, dtype=np.float32)
        ids = None if ids is None else np.ascontiguousarray(ids, np.int64)
        s = Simplices()
        rc = self.lib.rnng_rips_l2(self.h, _ptr(X), _ptr(ids), X.shape[0], X.shape[1], ctypes.c_float(radius), maxdim,
                                   MODES[mode], SORT_OUTPUT, ctypes.byref(s))
        self._check(rc, self.h)
        return _host_copy(s.id, s.count, np.int64), _host_copy(s.value, s.count, np.float32)

    def rips_edges(self, n: int, u, v, w, maxdim: int = 2, ids=None, vertex_flags=None):
        """Filtration of a given graph over rows 0..n-1 (edges u, v with values w):
        (ids, values), plus per-simplex flags when vertex_flags is given."""
        u = np.ascontiguousarray(u, np.int64)
        v = np.ascontiguousarray(v, np.int64)
        w = np.ascontiguousarray(w, np.float32)
        ids = None if ids is None else np.ascontiguousarray(ids, np.int64)
        vf = None if vertex_flags is None else np.ascontiguousarray(vertex_flags, np.uint8)
        s = Simplices()
        rc = self.lib.rnng_rips_edges(self.h, n, _ptr(ids), _ptr(vf), _ptr(u) if u.size else None,
                                      _ptr(v) if v.size else None, _ptr(w) if w.size else None, u.size, maxdim, 0,
                                      ctypes.byref(s))
        self._check(rc, self.h)
        out = (_host_copy(s.id, s.count, np.int64), _host_copy(s.value, s.count, np.float32))
        if vf is not None:
            out += (_host_copy(s.flag, s.count, np.uint8),)
        return out

    def graph_finalize(self, u, v, w, num_vertices: int):
        """Both orientations plus self-loops, sorted by (u, v) (Graph::redistribute_edges)."""
        u = np.ascontiguousarray(u, np.int64)
        v = np.ascontiguousarray(v, np.int64)
        w = np.ascontiguousarray(w, np.float32)
        ein = Edges(u.size, u.ctypes.data, v.ctypes.data, w.ctypes.data, 0, 0)
        e = Edges()
        rc = self.lib.rnng_graph_finalize(self.h, ctypes.byref(ein), num_vertices, 0, ctypes.byref(e))
        self._check(rc, self.h)
        return self._edges_out(e)
