"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is involved: meshes, optodes and parameter fields are
generated here from a seed.

* disc(rings)      2D disc of radius 25 mm built from concentric node rings
                   (ring k holds 6k nodes); 32 rings -> 3169 nodes (~3.3k),
                   64 rings -> 12481 nodes (~13k).
* cylinder()       3D cylinder R = 25 mm, H = 50 mm: a jittered 2D ring
                   triangulation extruded through z layers; every prism is
                   split into three tetrahedra with a split that conforms
                   across shared faces.  Default: 30 layers of 1027 nodes
                   = 30810 nodes, ~170k tetrahedra.
* box()            3D box 80 x 80 x 60 mm on a 64 x 64 x 61 node grid, 6-tet
                   (Kuhn) split, interior nodes jittered by +-0.2 h.

Node numbering: after generation the nodes are renumbered by a seeded random
permutation, the way a mesher's output order looks.  The reference's own
fixtures have shallow incomplete-Cholesky dependency graphs (circle25_32.msh:
25 levels, cyl2.msh: 59), and so do these meshes (15-30 levels); a ring or
layer ordering would give thousands.  The reference and the GPU path both solve
in this ("natural") order.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
from scipy.spatial import Delaunay

from .meshio import QMSpec


def _scramble(coords, elems, rng, *fields):
    perm = rng.permutation(len(coords)).astype(np.int32)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(len(perm), dtype=np.int32)
    return (coords[perm], inv[elems].astype(np.int32)) + tuple(f[perm] for f in fields)


@dataclass
class Problem:
    """One forward-path problem: mesh, optodes, optical parameters, modulation."""

    name: str
    coords: np.ndarray      # n x dim
    elems: np.ndarray       # ne x nn (0-based, positively oriented)
    qm: QMSpec
    mua: np.ndarray
    mus: np.ndarray
    nref: np.ndarray
    freq_mhz: float
    qwidth: float = 2.0
    mwidth: float = 2.0

    @property
    def n(self) -> int:
        return int(self.coords.shape[0])

    @property
    def dim(self) -> int:
        return int(self.coords.shape[1])

    @property
    def complex(self) -> bool:
        return self.freq_mhz != 0.0


def _orient(coords: np.ndarray, elems: np.ndarray) -> np.ndarray:
    """Reorder element nodes so every element has positive size (the reference
    uses the signed size, src/libfe/tri3.cc:184-189, src/libfe/tet4.cc:1010)."""
    elems = elems.copy()
    p = coords[elems]
    if elems.shape[1] == 3:
        v = (p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1]) - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1])
    else:
        v = np.einsum("ij,ij->i", np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), p[:, 3] - p[:, 0])
    neg = v < 0
    elems[neg, 0], elems[neg, 1] = elems[neg, 1].copy(), elems[neg, 0].copy()
    return elems


def _ring_points(rings: int, radius: float, rng: np.random.Generator | None = None, jitter: float = 0.0):
    pts = [np.zeros(2)]
    for k in range(1, rings + 1):
        r = radius * k / rings
        m = 6 * k
        th = 2 * np.pi * (np.arange(m) + (0.5 * (k % 2))) / m
        rr = np.full(m, r)
        if rng is not None and jitter > 0 and k < rings:
            h = radius / rings
            rr = rr + rng.uniform(-jitter, jitter, m) * h
            th = th + rng.uniform(-jitter, jitter, m) * (2 * np.pi / m)
        pts.append(np.stack([rr * np.cos(th), rr * np.sin(th)], 1))
    return np.vstack(pts)


def _blob_field(points: np.ndarray, centres: np.ndarray, sigma: float) -> np.ndarray:
    d2 = ((points[:, None, :] - centres[None, :, :]) ** 2).sum(-1)
    return np.exp(-d2 / (2 * sigma * sigma)).sum(1)


def disc(rings: int = 32, seed: int = 0, freq_mhz: float = 0.0, nopt: int = 16, radius: float = 25.0) -> Problem:
    rng = np.random.default_rng(seed)
    coords = _ring_points(rings, radius)
    tri = Delaunay(coords)
    elems = _orient(coords, tri.simplices.astype(np.int32))
    # two Gaussian blobs (sigma 3 mm), centres uniform in r < 18 mm
    u = rng.uniform(size=(2, 2))
    cen = np.stack([18 * np.sqrt(u[:, 0]) * np.cos(2 * np.pi * u[:, 1]),
                    18 * np.sqrt(u[:, 0]) * np.sin(2 * np.pi * u[:, 1])], 1)
    B = _blob_field(coords, cen, 3.0)
    mua = 0.025 * (1 + 0.5 * B)
    mus = 2.0 * (1 + 0.5 * B)
    nref = np.full(len(coords), 1.4)
    ang_q = 2 * np.pi * np.arange(nopt) / nopt
    ang_m = 2 * np.pi * (np.arange(nopt) + 0.5) / nopt
    Q = np.stack([radius * np.cos(ang_q), radius * np.sin(ang_q)], 1)
    M = np.stack([radius * np.cos(ang_m), radius * np.sin(ang_m)], 1)
    coords, elems, mua, mus, nref = _scramble(coords, elems, rng, mua, mus, nref)
    return Problem(f"disc{rings}", coords, elems, QMSpec.all_to_all(Q, M), mua, mus, nref, freq_mhz)


def _extrude(coords2: np.ndarray, tris: np.ndarray, z: np.ndarray):
    n2 = len(coords2)
    L = len(z)
    coords = np.concatenate([np.column_stack([coords2, np.full(n2, zz)]) for zz in z])
    t = np.sort(tris, axis=1)  # v0 < v1 < v2 -> conforming prism split
    els = []
    for l in range(L - 1):
        v = t + l * n2
        w = t + (l + 1) * n2
        els.append(np.stack([v[:, 0], v[:, 1], v[:, 2], w[:, 2]], 1))
        els.append(np.stack([v[:, 0], v[:, 1], w[:, 1], w[:, 2]], 1))
        els.append(np.stack([v[:, 0], w[:, 0], w[:, 1], w[:, 2]], 1))
    return coords, np.concatenate(els).astype(np.int32)


def cylinder(rings: int = 18, layers: int = 30, seed: int = 0, freq_mhz: float = 100.0,
             radius: float = 25.0, height: float = 50.0, jitter: float = 0.2) -> Problem:
    rng = np.random.default_rng(seed)
    c2 = _ring_points(rings, radius, rng, jitter)
    tri = Delaunay(c2)
    z = np.linspace(-height / 2, height / 2, layers)
    coords, elems = _extrude(c2, tri.simplices.astype(np.int32), z)
    # jitter interior nodes in z (boundary layers and the outer ring stay put)
    h = height / (layers - 1)
    n2 = len(c2)
    r2 = np.hypot(c2[:, 0], c2[:, 1])
    for l in range(1, layers - 1):
        sl = slice(l * n2, (l + 1) * n2)
        coords[sl, 2] += rng.uniform(-jitter, jitter, n2) * h * (r2 < radius * (1 - 0.5 / rings))
    elems = _orient(coords, elems)
    # three Gaussian inclusions (sigma 4 mm), contrast c in U[1.5, 3]
    base_mua, base_mus = 0.01, 1.0
    mua = np.full(len(coords), base_mua)
    mus = np.full(len(coords), base_mus)
    for _ in range(3):
        rr = 15 * np.sqrt(rng.uniform())
        th = 2 * np.pi * rng.uniform()
        cen = np.array([[rr * np.cos(th), rr * np.sin(th), rng.uniform(-15, 15)]])
        c = rng.uniform(1.5, 3.0)
        g = _blob_field(coords, cen, 4.0)
        mua *= 1 + (c - 1) * g
        mus *= 1 + (c - 1) * g
    nref = np.full(len(coords), 1.4)
    Q, M = [], []
    for zr in (-20.0, -10.0, 0.0, 10.0, 20.0):
        for i in range(16):
            aq = 2 * np.pi * i / 16
            am = aq + np.deg2rad(11.25)
            Q.append([radius * np.cos(aq), radius * np.sin(aq), zr])
            M.append([radius * np.cos(am), radius * np.sin(am), zr])
    coords, elems, mua, mus, nref = _scramble(coords, elems, rng, mua, mus, nref)
    return Problem(f"cyl{len(coords)}", coords, elems, QMSpec.all_to_all(np.array(Q), np.array(M)),
                   mua, mus, nref, freq_mhz)


def box(nx: int = 64, ny: int = 64, nz: int = 61, size=(80.0, 80.0, 60.0), seed: int = 0,
        freq_mhz: float = 100.0, nq: int = 128) -> Problem:
    rng = np.random.default_rng(seed)
    xs = np.linspace(0, size[0], nx)
    ys = np.linspace(0, size[1], ny)
    zs = np.linspace(0, size[2], nz)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    coords = np.stack([X.ravel(), Y.ravel(), Z.ravel()], 1)
    h = np.array([xs[1] - xs[0], ys[1] - ys[0], zs[1] - zs[0]])
    ii = np.arange(len(coords))
    ix, iy, iz = ii % nx, (ii // nx) % ny, ii // (nx * ny)
    interior = (ix > 0) & (ix < nx - 1) & (iy > 0) & (iy < ny - 1) & (iz > 0) & (iz < nz - 1)
    coords[interior] += rng.uniform(-0.2, 0.2, (interior.sum(), 3)) * h
    # Kuhn split of each cube into 6 tetrahedra along the main diagonal
    def nid(i, j, k):
        return (k * ny + j) * nx + i
    I, J, K = np.meshgrid(np.arange(nx - 1), np.arange(ny - 1), np.arange(nz - 1), indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    v = [nid(I + a, J + b, K + c) for c in (0, 1) for b in (0, 1) for a in (0, 1)]  # v[a + 2b + 4c]
    paths = [(1, 2, 4), (1, 4, 2), (2, 1, 4), (2, 4, 1), (4, 1, 2), (4, 2, 1)]
    els = []
    for p in paths:
        a = 0
        b = a + p[0]
        c = b + p[1]
        els.append(np.stack([v[0], v[b], v[c], v[7]], 1))
    elems = _orient(coords, np.concatenate(els).astype(np.int32))
    # smooth log-normal field: sum of 20 Gaussians, rescaled to +-30 %
    cen = rng.uniform([0, 0, 0], size, (20, 3))
    f = _blob_field(coords, cen, 10.0) * rng.choice([-1, 1])
    f = (f - f.mean()) / (np.abs(f - f.mean()).max() + 1e-30)
    fac = np.exp(np.log(1.3) * f)
    mua = 0.01 * fac
    mus = 1.0 * fac
    nref = np.full(len(coords), 1.4)
    gx = np.linspace(10, size[0] - 10, 16)
    gy = np.linspace(10, size[1] - 10, nq // 16)
    GX, GY = np.meshgrid(gx, gy, indexing="ij")
    Q = np.stack([GX.ravel(), GY.ravel(), np.zeros(GX.size)], 1)
    M = np.stack([GX.ravel(), GY.ravel(), np.full(GX.size, size[2])], 1)
    coords, elems, mua, mus, nref = _scramble(coords, elems, rng, mua, mus, nref)
    return Problem(f"box{len(coords)}", coords, elems, QMSpec.all_to_all(Q, M), mua, mus, nref, freq_mhz)


CONFIGS = {
    "c0_disc3k_cw": lambda seed=0: disc(32, seed, 0.0, 16),
    "c1_disc13k_fd": lambda seed=0: disc(64, seed, 100.0, 32),
    "c2_cyl30k_fd": lambda seed=0: cylinder(seed=seed),
    "c3_box250k_fd": lambda seed=0: box(seed=seed),
    # the 30k cylinder's optode layout on a 7.5k-node cylinder: the small case
    # of the profiling captures (a few GB on the device)
    "c2s_cyl7k_fd": lambda seed=1: cylinder(rings=12, layers=16, seed=seed),
    # a 106k-node box (inputs past L2, a few GB): profiling captures of the
    # SpMM and IC(0) kernels at the 250k box's column count
    "c3s_box106k_fd": lambda seed=0: box(nx=48, ny=48, nz=46, seed=seed),
}
