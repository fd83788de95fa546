"""Seeded synthetic workloads with the shapes and value distributions of the five
epsilon-graph / Rips configurations, plus the fvecs / seqs file formats that RNNG's
readers consume.

RNNG ships no datasets.  Its readers take ``.fvecs`` (a little-endian int32 ``d``
followed by ``d`` float32 values, per record; include/point.hpp:113-168) and a text
file with one sequence per line (include/point.hpp:170-205).  The generators here
stand in for those files; every one is a pure function of its seed (numpy PCG64).

Workloads (n is scalable so tests can run the same distribution at small sizes):

* ``l2_mixture``     - K1: isotropic Gaussian mixture, centres U[-10,10]^d, sigma 1.
* ``descriptor``     - K2: integer-valued 0..255 vectors, 1,000 Gamma centres with
                       Poisson jitter (vector-descriptor-like).
* ``dna_families``   - K3: random ACGT seeds of length 80..120, mutants at a 3%
                       per-position rate over {substitution, insertion, deletion}.
* ``torus16``        - K4: noisy torus (R=3, r=1, sigma 0.02) embedded in R^16.
* ``zipf_mixture``   - K5: 4,096 Gaussians with Zipf(1.2) weights in R^32.
"""
from __future__ import annotations

import struct

import numpy as np

# Epsilon values are frozen as float32 bit patterns so that every run (and every
# machine) uses the identical radius; they were chosen by bisection on exact
# brute-force subsamples for the mean degrees named in each docstring.
EPS_K1 = np.float32(1.5)
EPS_K3 = np.float32(8.0)


def _f32(hexbits: int) -> np.float32:
    return np.frombuffer(struct.pack("<I", hexbits), dtype=np.float32)[0]


EPS_K2 = _f32(0x4263791B)   # 56.868267, mean degree ~20 on descriptor(1_000_000)
EPS_K4 = _f32(0x3D5A71CC)   # 0.05333118, mean degree ~30 on torus16(500_000)
EPS_K5 = _f32(0x408EF2DD)   # 4.4671464, mean degree ~20 on zipf_mixture(5_000_000)


def l2_mixture(n: int = 20_000, d: int = 8, k: int = 16, sigma: float = 1.0, seed: int = 1) -> np.ndarray:
    """K1: n points in R^d from k equal-weight Gaussians, centres U[-10,10]^d."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-10.0, 10.0, size=(k, d))
    comp = rng.integers(0, k, size=n)
    x = centres[comp] + rng.normal(0.0, sigma, size=(n, d))
    return x.astype(np.float32)


def descriptor(n: int = 1_000_000, d: int = 128, k: int = 1000, seed: int = 2, chunk: int = 1 << 17) -> np.ndarray:
    """K2: integers 0..255 stored as float32.

    Centre coordinates are clamp(round(Gamma(shape 0.8, scale 25)), 0, 255); a point
    is min(255, Poisson(centre coordinate)) around a uniformly chosen centre.
    """
    rng = np.random.default_rng(seed)
    centres = np.clip(np.rint(rng.gamma(0.8, 25.0, size=(k, d))), 0, 255)
    comp = rng.integers(0, k, size=n)
    out = np.empty((n, d), dtype=np.float32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        lam = centres[comp[s:e]]
        out[s:e] = np.minimum(rng.poisson(lam), 255).astype(np.float32)
    return out


def dna_families(n_seeds: int = 5000, mutants: int = 40, rate: float = 0.03, seed: int = 3,
                 min_len: int = 80, max_len: int = 120) -> list[bytes]:
    """K3: n_seeds * mutants DNA strings (the seeds themselves are not emitted)."""
    rng = np.random.default_rng(seed)
    alphabet = np.frombuffer(b"ACGT", dtype=np.uint8)
    out: list[bytes] = []
    for _ in range(n_seeds):
        length = int(rng.integers(min_len, max_len + 1))
        base = alphabet[rng.integers(0, 4, size=length)]
        for _ in range(mutants):
            hit = rng.random(length) < rate
            kinds = rng.integers(0, 3, size=length)       # 0 sub, 1 ins, 2 del
            letters = alphabet[rng.integers(0, 4, size=length)]
            # position i emits its (possibly substituted) base unless deleted, and an
            # inserted letter after it when the mutation is an insertion
            first = np.where(hit & (kinds == 0), letters, base)
            inter = np.empty(2 * length, dtype=np.uint8)
            inter[0::2] = first
            inter[1::2] = letters
            keep = np.empty(2 * length, dtype=bool)
            keep[0::2] = ~(hit & (kinds == 2))
            keep[1::2] = hit & (kinds == 1)
            out.append(inter[keep].tobytes())
    return out


def torus16(n: int = 500_000, R: float = 3.0, r: float = 1.0, noise: float = 0.02, seed: int = 4) -> np.ndarray:
    """K4: torus in R^3 with uniform angles, Gaussian noise, mapped to R^16 by a
    16x3 matrix with orthonormal columns (QR of a seeded Gaussian matrix)."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(0.0, 2.0 * np.pi, size=n)
    v = rng.uniform(0.0, 2.0 * np.pi, size=n)
    p = np.stack([(R + r * np.cos(v)) * np.cos(u), (R + r * np.cos(v)) * np.sin(u), r * np.sin(v)], axis=1)
    p = p + rng.normal(0.0, noise, size=p.shape)
    q, _ = np.linalg.qr(rng.normal(size=(16, 3)))
    return (p @ q.T).astype(np.float32)


def zipf_mixture(n: int = 5_000_000, d: int = 32, k: int = 4096, a: float = 1.2, seed: int = 5,
                 chunk: int = 1 << 20) -> np.ndarray:
    """K5: Gaussian mixture with Zipf(a) component weights (w_j proportional to j^-a)."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-10.0, 10.0, size=(k, d))
    w = np.arange(1, k + 1, dtype=np.float64) ** (-a)
    w /= w.sum()
    comp = rng.choice(k, size=n, p=w)
    out = np.empty((n, d), dtype=np.float32)
    for s in range(0, n, chunk):
        e = min(n, s + chunk)
        out[s:e] = (centres[comp[s:e]] + rng.normal(size=(e - s, d))).astype(np.float32)
    return out


# ----------------------------------------------------------------------------- file formats

def write_fvecs(path: str, x: np.ndarray) -> None:
    """fvecs: per record an int32 dimension followed by d float32 values."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    n, d = x.shape
    rec = np.empty((n, d + 1), dtype=np.float32)
    rec[:, 0] = np.frombuffer(np.int32(d).tobytes(), dtype=np.float32)[0]
    rec[:, 1:] = x
    rec.tofile(path)


def read_fvecs(path: str) -> np.ndarray:
    raw = np.fromfile(path, dtype=np.float32)
    if raw.size == 0:
        return np.zeros((0, 0), dtype=np.float32)
    d = int(raw[:1].view(np.int32)[0])
    rec = raw.reshape(-1, d + 1)
    if not np.all(rec[:, 0].view(np.int32) == d):
        raise ValueError(f"{path}: inconsistent record dimensions")
    return np.ascontiguousarray(rec[:, 1:])


def write_seqs(path: str, seqs: list[bytes]) -> None:
    with open(path, "wb") as f:
        for s in seqs:
            f.write(s)
            f.write(b"\n")


def read_seqs(path: str) -> list[bytes]:
    out = []
    with open(path, "rb") as f:
        for line in f.read().split(b"\n"):
            if line.endswith(b"\r"):
                line = line[:-1]
            if line:
                out.append(line)
    return out


def pack_seqs(seqs: list[bytes]) -> tuple[np.ndarray, np.ndarray]:
    """CSR layout (atoms, offsets[n+1]) as in RNNG's PointContainer (include/point.h:77-79)."""
    lens = np.fromiter((len(s) for s in seqs), dtype=np.int64, count=len(seqs))
    offsets = np.zeros(len(seqs) + 1, dtype=np.int64)
    np.cumsum(lens, out=offsets[1:])
    atoms = np.frombuffer(b"".join(seqs), dtype=np.uint8).copy() if seqs else np.zeros(0, np.uint8)
    return atoms, offsets


def choose_eps(x: np.ndarray, mean_degree: float, sample: int = 30_000, seed: int = 11,
               block: int = 4096) -> np.float32:
    """Radius for a target mean degree, from the exact pairwise distances of a uniform
    subsample: the full set's expected degree is the subsample's times (n-1)/(s-1), so
    the radius is the k-th smallest subsample distance with k = s*(s-1)/(n-1)*deg/2."""
    n = x.shape[0]
    s = min(sample, n)
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(n, size=s, replace=False))
    y = x[idx].astype(np.float64)
    k = max(1, int(round(s * (s - 1) / max(1, n - 1) * mean_degree / 2)))
    sq = (y * y).sum(1)
    best = np.empty(0)
    for i in range(0, s, block):
        g = sq[i:i + block, None] + sq[None, :] - 2.0 * (y[i:i + block] @ y.T)
        rows = np.arange(i, min(s, i + block))
        mask = np.arange(s)[None, :] > rows[:, None]
        cand = np.sqrt(np.maximum(g[mask], 0.0))
        best = np.partition(np.concatenate([best, cand]), min(k, best.size + cand.size - 1))[:k + 1] \
            if best.size + cand.size > k else np.concatenate([best, cand])
    best.sort()
    return np.float32(best[min(k, best.size) - 1])
