"""Source sharding over ranks (multi-GPU row of the path: shard the sources,
all-gather the adjoint fields, Jacobian rows per rank), run as two gloo
ranks on the host.  The solves inside each rank come from the oracle, so the
test checks the partition, the exchange and the row assembly against a
single-process run."""
import os
import socket

import numpy as np
import pytest

from toastpp_gb300 import shard


def test_source_range_partitions_like_calcfields_engine():
    for nq in [0, 1, 7, 80, 81]:
        for w in [1, 2, 3, 8]:
            r = [shard.source_range(nq, i, w) for i in range(w)]
            assert r[0][0] == 0 and r[-1][1] == nq
            assert all(a[1] == b[0] for a, b in zip(r, r[1:]))
            assert max(b - a for a, b in r) - min(b - a for a, b in r) <= 1
    with pytest.raises(ValueError):
        shard.source_range(4, 2, 2)


def test_local_links():
    ofs = np.array([0, 3, 5, 9], np.int32)
    m = np.arange(9, dtype=np.int32)
    lo, lm, l0 = shard.local_links(ofs, m, 1, 3)
    assert l0 == 3 and list(lo) == [0, 2, 6] and list(lm) == list(range(3, 9))


class OracleEngine:
    """The solver methods forward_path_sharded uses, computed by the oracle."""

    def __init__(self, oracle, P):
        self.O = oracle
        self.mesh = oracle.Mesh(P.coords, P.elems)
        self.cplx = P.complex
        cm, ck, ca = oracle.optical_coefficients(P.mua, P.mus, P.nref)
        self.val = self.mesh.assemble(cm, ck, ca, P.freq_mhz * 2 * np.pi * 1e-6, self.cplx)
        self.method = "BICGSTAB" if self.cplx else "CG"

    def calc_fields(self, B):
        X, its, errs = self.O.solve(self.mesh.rowptr, self.mesh.colidx, self.val, B, self.method, "ICH", 1e-12)
        return X, list(zip(its, errs))

    def project_all(self, mvec, phi, links, scale):
        return self.O.project(phi, mvec, links.ofs, links.m, logscale=(scale == 2))

    def jacobian(self, dphi, aphi, proj, links, scale):
        return self.O.jacobian(self.mesh, dphi, aphi, proj, links.ofs, links.m, logscale=(scale == 2))


def problem(freq):
    from toastpp_gb300 import workloads
    return workloads.disc(8, 3, freq, 5)


def inputs(oracle, P):
    m = oracle.Mesh(P.coords, P.elems)
    _, _, ca = oracle.optical_coefficients(P.mua, P.mus, P.nref)
    dt = np.complex128 if P.complex else np.float64
    q = np.stack([m.qvec_gaussian(x, P.qwidth) for x in P.qm.Q]).astype(dt)
    mv = np.stack([m.qvec_gaussian(x, P.mwidth) * ca for x in P.qm.M]).astype(dt)
    return q, mv


def _worker(rank, world, port, freq, queue):
    import torch.distributed as dist
    from oracle import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        oracle.build()
        P = problem(freq)
        q, mv = inputs(oracle, P)
        res = shard.forward_path_sharded(OracleEngine(oracle, P), q, mv, P.qm.link_ofs, P.qm.link_m, rank, world)
        queue.put((rank, res))
    finally:
        dist.destroy_process_group()


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


@pytest.mark.parametrize("freq", [0.0, 100.0])
def test_two_gloo_ranks_match_single_process(oracle_mod, freq):
    import torch.multiprocessing as mp
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, freq, q)) for r in range(world)]
    for p in procs:
        p.start()
    parts = dict(q.get(timeout=300) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    P = problem(freq)
    ref = oracle_mod.forward_path(oracle_mod.Mesh(P.coords, P.elems), P.qm.Q, P.qm.M, P.qm.link_ofs, P.qm.link_m,
                                  P.mua, P.mus, P.nref, P.freq_mhz, P.qwidth, P.mwidth, None, "ICH", 1e-12)
    order = [parts[r] for r in range(world)]
    proj = np.concatenate([p.proj for p in order])
    lproj = np.concatenate([p.logproj for p in order])
    J = shard.assemble_jacobian(order, P.qm.nQM)
    # identical arithmetic per source (the oracle solves each right-hand side alone)
    assert np.array_equal(proj, ref.proj)
    assert np.array_equal(lproj, ref.logproj)
    assert np.array_equal(J, ref.J)
