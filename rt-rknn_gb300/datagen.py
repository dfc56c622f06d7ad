"""Seeded synthetic facility/user sets and the reference's text format.

The reference reads one text file per run (rknn-inf/inf.cpp:129-161,
rknn-naive/rknn.cpp:299-328):

    nf
    id x y        (nf lines, facilities)
    nu
    id x y        (nu lines, users)

and answers one query, given as an index into the facility list (`-q`,
inf.cpp:207 `fac[q]`).  The reference parses coordinates as `double`
(rknn-inf) or `int` (rknn-naive).  This engine stores float32 coordinates, so
every generated coordinate is a float32 value written with 17 significant
digits: `strtod` then yields exactly that float32 value as a double, and the
double-precision reference and the float32 engine see the same point.

Workloads (sizes as the reference's benchmark configurations name them):

* ``uniform``      facilities and users i.i.d. uniform in [0,1000]^2
* ``gaussmix``     64-component isotropic Gaussian mixture (centres uniform in
                   [0,1000]^2, sigma uniform in [2,20], clipped to the box), with
                   1% of users placed exactly on a q-f perpendicular bisector and
                   0.1% of users duplicating another user's coordinates
* ``street``       users on a jittered 400x400 street grid with 30% of the edges
                   dropped, N(0,0.5) jitter; facilities sampled from the same
                   points

Facilities get ids 0..nf-1 and users nf..nf+nu-1, so a facility's id equals its
index in the file.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

BOX = 1000.0


@dataclass
class Dataset:
    fxy: np.ndarray            # (nf, 2) float32
    uxy: np.ndarray            # (nu, 2) float32
    fid: np.ndarray            # (nf,) int32
    uid: np.ndarray            # (nu,) int32
    queries: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    ks: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    name: str = ""
    ties: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int64))  # (user, q, f)

    @property
    def nf(self) -> int:
        return int(self.fxy.shape[0])

    @property
    def nu(self) -> int:
        return int(self.uxy.shape[0])


def _ids(nf: int, nu: int):
    return (np.arange(nf, dtype=np.int32),
            np.arange(nf, nf + nu, dtype=np.int32))


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def uniform(nf: int, nu: int, seed: int = 1, nq: int = 10, k: int = 5,
            integer: bool = False) -> Dataset:
    """Uniform [0,1000]^2.  ``integer=True`` rounds every coordinate to an
    integer (the form rknn-naive can read, rknn-naive/rknn.cpp:39)."""
    rng = np.random.default_rng(seed)
    fxy = rng.uniform(0.0, BOX, size=(nf, 2))
    uxy = rng.uniform(0.0, BOX, size=(nu, 2))
    if integer:
        fxy = np.rint(fxy)
        uxy = np.rint(uxy)
    fid, uid = _ids(nf, nu)
    q = rng.choice(nf, size=min(nq, nf), replace=False).astype(np.int64)
    ks = np.full(q.shape[0], k, np.int32)
    return Dataset(_f32(fxy), _f32(uxy), fid, uid, q, ks,
                   f"uniform_f{nf}_u{nu}{'_int' if integer else ''}")


def _exact_d2_diff(ux, uy, fx, fy, qx, qy, scale):
    """d2(u,f) - d2(u,q) in exact integer arithmetic for coordinates on a
    dyadic grid of step 1/scale."""
    U = (int(ux * scale), int(uy * scale))
    F = (int(fx * scale), int(fy * scale))
    Q = (int(qx * scale), int(qy * scale))
    df = (U[0] - F[0]) ** 2 + (U[1] - F[1]) ** 2
    dq = (U[0] - Q[0]) ** 2 + (U[1] - Q[1]) ** 2
    return df - dq


def gaussmix(nf: int, nu: int, seed: int = 3, nq: int = 2000, k: int = 10,
             ncomp: int = 64, tie_frac: float = 0.01,
             dup_frac: float = 0.001) -> Dataset:
    """Skewed precision workload with forced ties (exact bisector users and
    duplicated coordinates)."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.0, BOX, size=(ncomp, 2))
    sigmas = rng.uniform(2.0, 20.0, size=ncomp)

    def draw(n):
        c = rng.integers(0, ncomp, size=n)
        p = centres[c] + rng.normal(size=(n, 2)) * sigmas[c, None]
        return np.clip(p, 0.0, BOX)

    # facilities on a 2^-6 grid so that exact bisector points exist in float32
    fxy = np.round(draw(nf) * 64.0) / 64.0
    uxy = draw(nu)
    q = rng.choice(nf, size=min(nq, nf), replace=False).astype(np.int64)

    n_tie = int(round(tie_frac * nu))
    n_dup = int(round(dup_frac * nu))
    ties = []
    if n_tie > 0 and nf > 1:
        # neighbours of each query facility among facilities (brute force on a
        # coarse grid is enough for a generator)
        from scipy.spatial import cKDTree  # scipy is available in this image
        tree = cKDTree(fxy)
        nn = min(12, nf)
        _, nbr = tree.query(fxy[q], k=nn)
        slots = rng.choice(nu, size=n_tie, replace=False)
        qi = rng.integers(0, q.shape[0], size=n_tie)
        placed = 0
        for s, j in zip(slots, qi):
            qq = q[j]
            cand = nbr[j][1:] if nn > 1 else nbr[j:j + 1]
            f = int(cand[rng.integers(0, len(cand))])
            if f == qq:
                continue
            qx, qy = fxy[qq]
            fx, fy = fxy[f]
            if qx == fx and qy == fy:
                continue
            mx, my = (qx + fx) / 2.0, (qy + fy) / 2.0
            t = rng.integers(-64, 65) / 64.0
            ux = mx - t * (fy - qy)
            uy = my + t * (fx - qx)
            if not (0.0 <= ux <= BOX and 0.0 <= uy <= BOX):
                continue
            # on the 2^-13 grid, < 2^10: exactly representable in float32
            if (np.float32(ux) != ux) or (np.float32(uy) != uy):
                continue
            if _exact_d2_diff(ux, uy, fx, fy, qx, qy, 8192) != 0:
                continue
            uxy[s] = (ux, uy)
            ties.append((int(s), int(qq), f))
            placed += 1
    if n_dup > 0:
        tie_users = {t[0] for t in ties}
        dst = np.array([d for d in rng.choice(nu, size=n_dup + len(tie_users), replace=False)
                        if d not in tie_users][:n_dup], dtype=np.int64)
        src = rng.integers(0, nu, size=dst.shape[0])
        uxy[dst] = uxy[src]
    fid, uid = _ids(nf, nu)
    ks = np.full(q.shape[0], k, np.int32)
    return Dataset(_f32(fxy), _f32(uxy), fid, uid, q, ks,
                   f"gaussmix_f{nf}_u{nu}", np.array(ties, np.int64).reshape(-1, 3))


def street(nu: int = 2_000_000, nf: int = 20_000, seed: int = 4,
           nq: int = 16384, side: int = 400, drop: float = 0.30,
           jitter: float = 0.5, kmax: int = 100) -> Dataset:
    """Road-network-like layout: points on the edges of a jittered street
    grid; facilities are a random sample of the same points."""
    rng = np.random.default_rng(seed)
    step = BOX / side
    gx, gy = np.meshgrid(np.arange(side), np.arange(side), indexing="ij")
    nodes = np.stack([gx.ravel(), gy.ravel()], 1).astype(np.float64) * step
    nodes += rng.uniform(-0.3, 0.3, size=nodes.shape) * step
    idx = np.arange(side * side).reshape(side, side)
    eh = np.stack([idx[:-1, :].ravel(), idx[1:, :].ravel()], 1)
    ev = np.stack([idx[:, :-1].ravel(), idx[:, 1:].ravel()], 1)
    edges = np.concatenate([eh, ev], 0)
    keep = rng.uniform(size=edges.shape[0]) >= drop
    edges = edges[keep]
    n = nu + nf
    e = edges[rng.integers(0, edges.shape[0], size=n)]
    t = rng.uniform(size=(n, 1))
    p = nodes[e[:, 0]] + t * (nodes[e[:, 1]] - nodes[e[:, 0]])
    p += rng.normal(scale=jitter, size=p.shape)
    p = np.clip(p, 0.0, BOX)
    perm = rng.permutation(n)
    fxy = p[perm[:nf]]
    uxy = p[perm[nf:]]
    q = rng.choice(nf, size=min(nq, nf), replace=(nq > nf)).astype(np.int64)
    ks = np.floor(np.exp(rng.uniform(0.0, math.log(kmax + 1), size=q.shape[0])))
    ks = np.clip(ks, 1, kmax).astype(np.int32)
    fid, uid = _ids(nf, nu)
    return Dataset(_f32(fxy), _f32(uxy), fid, uid, q, ks, f"street_f{nf}_u{nu}")


def config(n: int, seed: int | None = None, scale: float = 1.0) -> Dataset:
    """The five benchmark workloads by number (1-based).  ``scale`` < 1 shrinks
    the point counts (for tests), keeping densities' ratio."""
    def s(x):
        return max(1, int(round(x * scale)))
    if n == 1:
        return uniform(s(1000), s(10000), seed=seed or 1, nq=10, k=5)
    if n == 2:
        return uniform(s(100_000), s(1_000_000), seed=seed or 2, nq=1000, k=10)
    if n == 3:
        return gaussmix(s(200_000), s(4_000_000), seed=seed or 3, nq=2000, k=10)
    if n == 4:
        return street(nu=s(2_000_000), nf=s(20_000), seed=seed or 4, nq=16384)
    if n == 5:
        return uniform(s(1_000_000), s(10_000_000), seed=seed or 5, nq=1000, k=10)
    raise ValueError(f"no workload {n}")


# ---------------------------------------------------------------- text format

def write_text(path: str | os.PathLike, ds: Dataset, integer: bool = False) -> None:
    """Write the reference's text format.  Float coordinates get 17
    significant digits (exact round trip of the float32 value through
    strtod); ``integer=True`` writes integers for rknn-naive."""
    fmt = "%d %d %d" if integer else "%d %.17g %.17g"
    with open(path, "w") as fh:
        fh.write(f"{ds.nf}\n")
        for i0 in range(0, ds.nf, 1 << 18):
            blk = slice(i0, min(ds.nf, i0 + (1 << 18)))
            arr = np.column_stack([ds.fid[blk].astype(np.float64),
                                   ds.fxy[blk].astype(np.float64)])
            np.savetxt(fh, arr, fmt=fmt)
        fh.write(f"{ds.nu}\n")
        for i0 in range(0, ds.nu, 1 << 18):
            blk = slice(i0, min(ds.nu, i0 + (1 << 18)))
            arr = np.column_stack([ds.uid[blk].astype(np.float64),
                                   ds.uxy[blk].astype(np.float64)])
            np.savetxt(fh, arr, fmt=fmt)


def read_text(path: str | os.PathLike) -> Dataset:
    """Parse the reference's text format (whitespace separated, as the
    reference's `ifstream >>` loop accepts it)."""
    with open(path) as fh:
        tok = fh.read().split()
    nf = int(tok[0])
    f = np.array(tok[1:1 + 3 * nf], dtype=np.float64).reshape(nf, 3)
    nu = int(tok[1 + 3 * nf])
    base = 2 + 3 * nf
    u = np.array(tok[base:base + 3 * nu], dtype=np.float64).reshape(nu, 3)
    return Dataset(_f32(f[:, 1:]), _f32(u[:, 1:]), f[:, 0].astype(np.int32),
                   u[:, 0].astype(np.int32))
