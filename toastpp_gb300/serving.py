"""The mixed-mesh request stream of the serving configuration, driven through
the request server (tg_server, capi.Server).

Requests arrive as a seeded Poisson process.  Each draws a mesh from the
2D 3.3k disc, 2D 13k disc, 3D 30k cylinder and 3D 250k box (weights 0.4, 0.3,
0.2, 0.1), a source count, CW or 100 MHz with equal probability, and a
fresh seeded parameter field (Gaussian blobs on the mesh's base parameters).
Sources and detectors sit at seeded boundary nodes.  Every request is a
whole forward path with projections and the nodal Jacobian.
"""
from __future__ import annotations

import threading
import time
from dataclasses import dataclass

import numpy as np

from . import capi, workloads

MESHES = [("c0_disc3k", lambda: workloads.disc(32, 0, 0.0, 16)),
          ("c1_disc13k", lambda: workloads.disc(64, 0, 100.0, 32)),
          ("c2_cyl30k", lambda: workloads.cylinder(seed=0)),
          ("c3_box250k", lambda: workloads.box(seed=0))]
WEIGHTS = [0.4, 0.3, 0.2, 0.1]


@dataclass
class StreamSpec:
    requests: int = 24
    rate_hz: float = 20.0          # mean arrival rate
    src_min: int = 8
    src_max: int = 128
    src_max_large: int = 64        # cap for the 250k mesh: its FP32 Jacobian is 2 nQM x 2n, 16 GB at 64
                                   # sources and 65 GB at 128, against 199 GB of host memory on the GPU machine
    seed: int = 0
    precision: str = "mixed"
    tol: float = 1e-10


class MeshSet:
    """The four meshes, built once, with their boundary nodes."""

    def __init__(self, which=(0, 1, 2, 3)):
        self.items = {}
        for i in which:
            name, make = MESHES[i]
            P = make()
            gm = capi.Mesh(P.coords, P.elems)
            bnd = np.nonzero(gm.boundary())[0]
            self.items[i] = (name, P, gm, bnd)


def fresh_params(P, rng):
    """Base parameters of the mesh times 1 + (c-1) g for 2-3 seeded blobs."""
    lo, hi = P.coords.min(0), P.coords.max(0)
    mua, mus = P.mua.copy(), P.mus.copy()
    for _ in range(int(rng.integers(2, 4))):
        cen = (lo + (hi - lo) * rng.uniform(0.2, 0.8, P.dim))[None, :]
        c = rng.uniform(1.5, 3.0)
        g = np.exp(-((P.coords - cen) ** 2).sum(1) / (2 * 4.0 ** 2))
        mua *= 1 + (c - 1) * g
        mus *= 1 + (c - 1) * g
    return mua, mus, P.nref


def make_requests(ms: MeshSet, spec: StreamSpec):
    rng = np.random.default_rng(spec.seed)
    keys = sorted(ms.items)
    w = np.array([WEIGHTS[k] for k in keys])
    w = w / w.sum()
    out = []
    t = 0.0
    for r in range(spec.requests):
        t += rng.exponential(1.0 / spec.rate_hz)
        k = int(rng.choice(keys, p=w))
        name, P, gm, bnd = ms.items[k]
        smax = spec.src_max_large if name.startswith("c3") else spec.src_max
        # sources and detectors at distinct boundary nodes (a small mesh caps the count)
        ns = min(int(rng.integers(spec.src_min, smax + 1)), len(bnd) // 2)
        freq = 100.0 if rng.uniform() < 0.5 else 0.0
        mua, mus, nref = fresh_params(P, rng)
        cm, ck, ca = capi.optical_coefficients(mua, mus, nref)
        pick = rng.choice(bnd, size=2 * ns, replace=False)
        Q, M = P.coords[pick[:ns]], P.coords[pick[ns:]]
        qvec = gm.qvec_gaussian(Q, 2.0)
        mvec = gm.qvec_gaussian(M, 2.0) * ca[None, :]
        links = capi.Links.all_to_all(ns, ns)
        req = capi.Request(gm, cm, ck, ca, capi.omega_of(freq), qvec, mvec, links, tol=spec.tol,
                           precision=spec.precision, want_jac=True, j_fp32=True)
        out.append((t, name, ns, freq, req))
    return out


def run_stream(requests, slots=4, hbm_budget_gb=120.0):
    """Submit each request at its arrival time while a collector thread waits
    for the results in submission order; returns per-request records, the
    server's statistics and the wall time."""
    import queue
    srv = capi.Server(slots=slots, hbm_budget_gb=hbm_budget_gb)
    q = queue.Queue()
    done = []

    def collect():
        while True:
            item = q.get()
            if item is None:
                return
            tk, rec = item
            req = srv.wait(tk)
            done.append((rec, req.latency_ms, req))

    th = threading.Thread(target=collect, daemon=True)
    srv.reset_stats()
    t0 = time.perf_counter()
    th.start()
    for arr, name, ns, freq, req in requests:
        now = time.perf_counter() - t0
        if arr > now:
            time.sleep(arr - now)
        q.put((srv.submit(req), (name, ns, freq)))
    q.put(None)
    th.join()
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    return done, st, wall


def summarize(done, st, wall):
    lat = np.array([d[1] for d in done])
    solves = sum(2 * d[0][1] for d in done)
    per = {}
    for (name, ns, freq), l, _ in done:
        per.setdefault(name, []).append(l)
    return {"requests": len(done), "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "solves_per_s": solves / wall, "wall_s": wall, "server": st,
            "per_mesh_p50_ms": {k: float(np.percentile(v, 50)) for k, v in sorted(per.items())},
            "per_mesh_count": {k: len(v) for k, v in sorted(per.items())}}
