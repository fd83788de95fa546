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


def ref_source_dir() -> str | None:
    """The RNNG source tree the recipe builds from ($RNNG_SRC, see oracle/Makefile), if present."""
    r = subprocess.run(["make", "-s", "-C", HERE, "ref-src"], capture_output=True, text=True)
    out = r.stdout.strip()
    return out if r.returncode == 0 and out else None


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
        L.orc_voronoi_edit.argtypes = [ctypes.c_void_p, _i64p, ctypes.c_int64, ctypes.c_void_p, _i64p,
                                       ctypes.c_int64, _i64p, _f32p]
        L.orc_dist_matrix_l2.argtypes = [_f32p, ctypes.c_int64, _f32p, ctypes.c_int64, ctypes.c_int64, _f32p]
        L.orc_dist_matrix_edit.argtypes = [ctypes.c_void_p, _i64p, ctypes.c_int64, ctypes.c_void_p, _i64p,
                                           ctypes.c_int64, _f32p]
        L.orc_landmark_l2.restype = ctypes.c_int64
        L.orc_landmark_l2.argtypes = [_f32p, ctypes.c_int64, ctypes.c_int64, ctypes.c_float, ctypes.c_int64,
                                      ctypes.c_float, ctypes.c_int64, ctypes.c_uint64, ctypes.POINTER(_i64p),
                                      ctypes.POINTER(_i64p), ctypes.POINTER(_f32p),
                                      ctypes.POINTER(ctypes.c_double), _i64p]
        L.orc_landmark_edit.restype = ctypes.c_int64
        L.orc_landmark_edit.argtypes = [ctypes.c_void_p, _i64p, ctypes.c_int64, ctypes.c_float, ctypes.c_int64,
                                        ctypes.c_float, ctypes.c_int64, ctypes.c_uint64, ctypes.POINTER(_i64p),
                                        ctypes.POINTER(_i64p), ctypes.POINTER(_f32p),
                                        ctypes.POINTER(ctypes.c_double), _i64p]
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


LANDMARK_PHASES = ("voronoi", "cells", "ghosts", "neighbours", "graph")


def landmark_l2(X: np.ndarray, eps, num_centers: int, cover: float = 1.5, leaf_size: int = 10, seed: int = 7):
    """RNNG's landmark pipeline (Voronoi cells, cover trees, ghosts, batched radius
    queries; oracle/landmark.c) on the host threads: (u, v, w) sorted, and a dict of
    phase seconds and counts."""
    X = np.ascontiguousarray(X, np.float32)
    n, d = X.shape
    pu, pv, pw = _i64p(), _i64p(), _f32p()
    ph = (ctypes.c_double * 5)()
    st = (ctypes.c_int64 * 4)()
    cnt = lib().orc_landmark_l2(X.ctypes.data_as(_f32p), n, d, ctypes.c_float(eps), num_centers,
                                ctypes.c_float(cover), leaf_size, seed, ctypes.byref(pu), ctypes.byref(pv),
                                ctypes.byref(pw), ph, st)
    info = {k: ph[i] for i, k in enumerate(LANDMARK_PHASES)}
    info.update({"seconds": sum(ph), "num_cells": int(st[0]), "num_ghosts": int(st[1]), "threads": int(st[2]),
                 "empty_cells": int(st[3])})
    return _edges(cnt, pu, pv, pw, sort=False), info


def landmark_edit(atoms: np.ndarray, offsets: np.ndarray, eps, num_centers: int, cover: float = 1.5,
                  leaf_size: int = 10, seed: int = 7):
    """The same pipeline over strings under RNNG's edit distance (its driver's `-D edit`
    path): (u, v, w) and the phase dict, as landmark_l2."""
    atoms = np.ascontiguousarray(atoms, np.uint8)
    offsets = np.ascontiguousarray(offsets, np.int64)
    n = offsets.size - 1
    pu, pv, pw = _i64p(), _i64p(), _f32p()
    ph = (ctypes.c_double * 5)()
    st = (ctypes.c_int64 * 4)()
    cnt = lib().orc_landmark_edit(atoms.ctypes.data_as(ctypes.c_void_p), offsets.ctypes.data_as(_i64p), n,
                                  ctypes.c_float(eps), num_centers, ctypes.c_float(cover), leaf_size, seed,
                                  ctypes.byref(pu), ctypes.byref(pv), ctypes.byref(pw), ph, st)
    info = {k: ph[i] for i, k in enumerate(LANDMARK_PHASES)}
    info.update({"seconds": sum(ph), "num_cells": int(st[0]), "num_ghosts": int(st[1]), "threads": int(st[2]),
                 "empty_cells": int(st[3])})
    return _edges(cnt, pu, pv, pw, sort=False), info


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


def voronoi_edit(atoms: np.ndarray, offsets: np.ndarray, catoms: np.ndarray, coffsets: np.ndarray):
    """Nearest centre per string under the reference edit distance (last of equal wins)."""
    atoms = np.ascontiguousarray(atoms, np.uint8)
    offsets = np.ascontiguousarray(offsets, np.int64)
    catoms = np.ascontiguousarray(catoms, np.uint8)
    coffsets = np.ascontiguousarray(coffsets, np.int64)
    n, m = offsets.size - 1, coffsets.size - 1
    cell = np.zeros(n, np.int64)
    dist = np.zeros(n, np.float32)
    lib().orc_voronoi_edit(atoms.ctypes.data_as(ctypes.c_void_p), offsets.ctypes.data_as(_i64p), n,
                           catoms.ctypes.data_as(ctypes.c_void_p), coffsets.ctypes.data_as(_i64p), m,
                           cell.ctypes.data_as(_i64p), dist.ctypes.data_as(_f32p))
    return cell, dist


class _Points:
    """Dense float rows (L2) or CSR strings (edit distance), the oracle's view of a
    PointContainer."""

    def __init__(self, metric, data):
        self.metric = metric
        if metric == "l2":
            self.x = np.ascontiguousarray(data, np.float32)
            self.n = self.x.shape[0]
        else:
            atoms, offsets = data
            self.atoms = np.ascontiguousarray(atoms, np.uint8)
            self.offsets = np.ascontiguousarray(offsets, np.int64)
            self.n = self.offsets.size - 1

    def rows(self, idx):
        idx = np.asarray(idx, np.int64)
        if self.metric == "l2":
            return _Points("l2", self.x[idx])
        parts = [self.atoms[self.offsets[i]:self.offsets[i + 1]] for i in idx]
        offs = np.zeros(idx.size + 1, np.int64)
        offs[1:] = np.cumsum([p.size for p in parts]) if parts else []
        atoms = np.concatenate(parts) if parts else np.zeros(0, np.uint8)
        return _Points("edit", (atoms, offs))

    def dist_matrix(self, centres: "_Points") -> np.ndarray:
        """out[i, c] = distance(centre c, point i), the reference's float arithmetic."""
        out = np.zeros((self.n, centres.n), np.float32)
        if self.n == 0 or centres.n == 0:
            return out
        if self.metric == "l2":
            lib().orc_dist_matrix_l2(self.x.ctypes.data_as(_f32p), self.n, centres.x.ctypes.data_as(_f32p), centres.n,
                                     self.x.shape[1], out.ctypes.data_as(_f32p))
        else:
            lib().orc_dist_matrix_edit(self.atoms.ctypes.data_as(ctypes.c_void_p), self.offsets.ctypes.data_as(_i64p),
                                       self.n, centres.atoms.ctypes.data_as(ctypes.c_void_p),
                                       centres.offsets.ctypes.data_as(_i64p), centres.n, out.ctypes.data_as(_f32p))
        return out

    def eps_graph(self, radius):
        if self.metric == "l2":
            return eps_graph_l2(self.x, radius)
        return eps_graph_edit(self.atoms, self.offsets, radius)


def landmark_cells(metric: str, data, landmarks, radius, rips: bool) -> dict:
    """The Voronoi cells of RNNG's landmark and rips drivers at one rank, restated:

    VoronoiDiagram (include/point.hpp:537-559): nearest landmark, last of equal wins.
    coalesce_cells (include/point.hpp:562-758): cells in landmark order, points in row
    order (id = row), the landmark's own point swapped into slot 0; a cell that got no
    point keeps id 0 (its id is only set from received points).
    add_ghost_points_systolic[_rips] (include/point.hpp:762-1124): every point q of cell A
    (in cell order) with its distance dq to A's landmark is tested against the k-th
    non-empty cell's slot-0 point s_k: when distance(s_k, q) <= dq + 2r, the cell at index
    k (cells[k], which is the k-th non-empty cell only when no cell is empty) gets q as
    a ghost if it is not empty, does not hold q, and has a point within r of q.  The
    rips version marks a point interior when it became nobody's ghost.

    Returns the flattened cell arrays of the harness's `cells` dump."""
    pts = _Points(metric, data)
    radius = np.float32(radius)
    landmarks = np.asarray(landmarks, np.int64)
    cents = pts.rows(landmarks)
    m = landmarks.size
    dmat = pts.dist_matrix(cents)  # (n, m)
    cell = np.zeros(pts.n, np.int64)
    dist = np.full(pts.n, np.float32(np.finfo(np.float32).max), np.float32)
    for c in range(m):  # `dist <= best`, centres in order
        upd = dmat[:, c] <= dist
        dist[upd] = dmat[upd, c]
        cell[upd] = c
    cells = []
    for c in range(m):
        rows = list(np.nonzero(cell == c)[0])
        dd = [dist[r] for r in rows]
        if rows:
            slot = next((k for k, r in enumerate(rows) if r == landmarks[c]), 0)
            rows[0], rows[slot] = rows[slot], rows[0]
            dd[0], dd[slot] = dd[slot], dd[0]
        cells.append({"id": c if rows else 0, "rows": rows, "dist": dd, "ghosts": [], "interior": [False] * len(rows)})
    # ghosts
    nonempty = [k for k, cl in enumerate(cells) if cl["rows"]]
    slot0 = pts.rows([cells[k]["rows"][0] for k in nonempty])
    qrows = [r for cl in cells for r in cl["rows"]]
    qdist = np.array([d for cl in cells for d in cl["dist"]], np.float32)
    to_slot0 = pts.rows(qrows).dist_matrix(slot0) if qrows else np.zeros((0, 0), np.float32)
    u, v, _ = pts.eps_graph(radius)
    nbrs = [set() for _ in range(pts.n)]
    for a, b in zip(u.tolist(), v.tolist()):
        nbrs[a].add(b)
        nbrs[b].add(a)
    own = [set(cl["rows"]) for cl in cells]       # the points each cell's cover tree holds
    members = [set(cl["rows"]) for cl in cells]   # treeids_set: own points and tested ids
    shared = np.zeros(len(qrows), np.int64)
    two_r = np.float32(2) * radius
    for qi, q in enumerate(qrows):
        bound = np.float32(qdist[qi] + two_r)
        for k in range(len(nonempty)):
            if not (to_slot0[qi, k] <= bound):
                continue
            target = cells[k]
            if not target["rows"] or q in members[k]:
                continue
            if nbrs[q] & own[k]:
                target["ghosts"].append(q)
                shared[qi] += 1
            members[k].add(q)  # the tested id joins the cell's id set (treeids_set)
    if rips:
        qi = 0
        for cl in cells:
            for j in range(len(cl["rows"])):
                cl["interior"][j] = shared[qi] == 0
                qi += 1
    res = {
        "cell_id": np.array([cl["id"] for cl in cells], np.int64),
        "npts": np.array([len(cl["rows"]) for cl in cells], np.int64),
        "ids": np.array([r for cl in cells for r in cl["rows"]], np.int64),
        "dist": np.array([d for cl in cells for d in cl["dist"]], np.float32),
        "interior": np.array([b for cl in cells for b in cl["interior"]], np.uint8),
        "nghost": np.array([len(cl["ghosts"]) for cl in cells], np.int64),
        "ghosts": np.array([g for cl in cells for g in cl["ghosts"]], np.int64),
    }
    return res


def binom(n: int, k: int) -> int:
    return int(lib().orc_binom(n, k))


def simplex_id(verts) -> int:
    v = np.ascontiguousarray(sorted(verts), np.int64)
    return int(lib().orc_simplex_id(v.ctypes.data_as(_i64p), v.size))


def rips(n: int, u: np.ndarray, v: np.ndarray, w: np.ndarray, maxdim: int = 2):
    """Filtration (ids, values) sorted by (value, id) from an epsilon graph with u < v
    over vertices 0..n-1, cliques up to maxdim + 1 vertices."""
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


def read_cells_dump(path: str) -> dict:
    """Cells written by the harness's `cells` mode, flattened: landmarks, cell_id, npts,
    ids, dist, interior, nghost, ghosts (per-cell runs concatenated in cell order)."""
    with open(path, "rb") as f:
        buf = f.read()
    pos = 0

    def take(dtype, count):
        nonlocal pos
        a = np.frombuffer(buf, dtype, count, pos)
        pos += a.nbytes
        return a

    nland = int(take(np.int64, 1)[0])
    landmarks = take(np.int64, nland).copy()
    ncell = int(take(np.int64, 1)[0])
    out = {k: [] for k in ("cell_id", "npts", "ids", "dist", "interior", "nghost", "ghosts")}
    for _ in range(ncell):
        out["cell_id"].append(int(take(np.int64, 1)[0]))
        npts = int(take(np.int64, 1)[0])
        out["npts"].append(npts)
        out["ids"].append(take(np.int64, npts))
        out["dist"].append(take(np.float32, npts))
        out["interior"].append(take(np.uint8, npts))
        ng = int(take(np.int64, 1)[0])
        out["nghost"].append(ng)
        out["ghosts"].append(take(np.int64, ng))
    assert pos == len(buf)
    res = {"landmarks": landmarks, "cell_id": np.array(out["cell_id"], np.int64),
           "npts": np.array(out["npts"], np.int64), "nghost": np.array(out["nghost"], np.int64)}
    for k, dt in (("ids", np.int64), ("dist", np.float32), ("interior", np.uint8), ("ghosts", np.int64)):
        res[k] = np.concatenate(out[k]).astype(dt) if out[k] else np.zeros(0, dt)
    return res


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
