"""One forward-path request sharded over ranks (one GPU per rank).

Sources are independent right-hand sides of the same system.  Rank r of W
solves the contiguous source range that CalcFields_engine gives task r of W
(q0 = r nQ / W, q1 = (r+1) nQ / W; src/libstoast/fwdsolver.cc:618-643) and
the detector range split the same way.  The one exchange step is an
all-gather of the adjoint fields, the counterpart of CalcFields'
MPI_Allgatherv of the fields (fwdsolver.cc:760-780), after which every rank
projects and builds the Jacobian rows of its own sources' links.  Ranks hold
the mesh, the system matrix and the preconditioner each (replicated), as the
MPI build of the reference does.

The engine is any object with the solver methods used here
(calc_fields / project_all / jacobian of toastpp_gb300.capi.FwdSolver, with
the system already reset); the communication goes through torch.distributed
on whatever process group is passed (NCCL on GPUs, gloo on host ranks).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


def source_range(count: int, rank: int, world: int) -> tuple[int, int]:
    """[q0, q1) of rank `rank`: the split of CalcFields_engine (fwdsolver.cc:624-625)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("invalid rank / world size")
    return (rank * count) // world, ((rank + 1) * count) // world


def local_links(link_ofs, link_m, q0: int, q1: int):
    """The link list of sources [q0, q1) and the global index of its first link."""
    link_ofs = np.asarray(link_ofs, np.int32)
    l0, l1 = int(link_ofs[q0]), int(link_ofs[q1])
    return (link_ofs[q0:q1 + 1] - l0).astype(np.int32), np.asarray(link_m[l0:l1], np.int32), l0


def allgather_rows(local: np.ndarray, count: int, world: int, group=None) -> np.ndarray:
    """Concatenate the row blocks of all ranks in rank order (Allgatherv of
    contiguous [q0, q1) blocks), through torch.distributed."""
    import torch
    import torch.distributed as dist

    cplx = np.iscomplexobj(local)
    width = local.shape[1] if local.ndim > 1 else 1
    rows = [source_range(count, r, world) for r in range(world)]
    maxr = max(b - a for a, b in rows)
    buf = np.zeros((maxr, width), np.complex128 if cplx else local.dtype)
    buf[:local.shape[0]] = local.reshape(local.shape[0], width)
    t = torch.from_numpy(buf.view(np.float64) if cplx else buf)
    outs = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(outs, t, group=group)
    parts = []
    for (a, b), o in zip(rows, outs):
        o = o.numpy()
        if cplx:
            o = o.view(np.complex128)
        parts.append(o[:b - a])
    out = np.concatenate(parts, axis=0)
    return out if local.ndim > 1 else out.reshape(-1)


@dataclass
class ShardResult:
    q0: int
    q1: int
    l0: int                 # global index of this rank's first link
    proj: np.ndarray        # linear projections of this rank's links
    logproj: np.ndarray
    J: np.ndarray | None    # Jacobian rows of this rank's links ([Re; Im] blocks as tg_jacobian)
    iters: list


def forward_path_sharded(engine, qvec, mvec, link_ofs, link_m, rank: int, world: int, group=None,
                         want_jac: bool = True, scale_log: bool = True) -> ShardResult:
    """This rank's share of one request: forward solves of its sources, adjoint
    solves of its detectors, all-gather of the adjoint fields, projections and
    Jacobian rows of its links."""
    from .capi import DATA_LIN, DATA_LOG, Links

    nq, nm = qvec.shape[0], mvec.shape[0]
    q0, q1 = source_range(nq, rank, world)
    m0, m1 = source_range(nm, rank, world)
    dphi, rq = engine.calc_fields(qvec[q0:q1])
    aphi_loc, rm = engine.calc_fields(mvec[m0:m1])
    aphi = allgather_rows(aphi_loc, nm, world, group)
    lofs, lm, l0 = local_links(link_ofs, link_m, q0, q1)
    links = Links(lofs, lm)
    proj = engine.project_all(mvec, dphi, links, DATA_LIN)
    lproj = engine.project_all(mvec, dphi, links, DATA_LOG)
    J = None
    if want_jac:
        J = engine.jacobian(dphi, aphi, proj if scale_log else None, links, DATA_LOG if scale_log else DATA_LIN)
    return ShardResult(q0, q1, l0, proj, lproj, J, list(rq) + list(rm))


def assemble_jacobian(parts: list[ShardResult], nqm: int) -> np.ndarray:
    """Global J from the rank blocks: rank r's rows [0, nl) are links l0..l0+nl
    of the first (Re / mua) block and rows [nl, 2 nl) the same links of the
    second block (Im, or kappa for CW)."""
    width = parts[0].J.shape[1]
    J = np.zeros((2 * nqm, width), parts[0].J.dtype)
    for p in parts:
        nl = p.J.shape[0] // 2
        J[p.l0:p.l0 + nl] = p.J[:nl]
        J[nqm + p.l0:nqm + p.l0 + nl] = p.J[nl:]
    return J
