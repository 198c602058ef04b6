"""Generates the golden fixtures of this directory by running the reference
itself (oracle/_ref/ref_driver, compiled from the reference sources by
oracle/Makefile.ref) on small seeded problems.

Each fixture <name>.npz holds the problem (mesh, optodes, nodal parameters,
solver settings) and the reference's outputs: linear and log projections
(ProjectAll, DATA_LIN / DATA_LOG), the per-call iteration counts and, where
asked, the nodal Jacobian of GenerateJacobian (toastmodule.cc CalcJacobian /
CalcJacobianCW call sequence, LOG data).  The GPU parity tests and the oracle
tests compare against these files, so they need neither the reference tree
nor the compiled reference at run time.

The *_grid fixtures add the grid-basis Jacobian of Raster_Pixel with the
basis equal to the grid (what toast.Raster(mesh, grd) builds,
src/python/toastmodule.cc:696), the raster's element reference per grid
point and the reference's own fields, so the oracle's raster and grid
Jacobian are checked on exactly the reference's inputs.

The *_igrid fixtures (and *_igrad, the data gradient) use a Raster_Pixel
with an intermediate grid finer than its basis (toast.Raster(mesh, grd,
intgrd)): the grid Jacobian is mapped from the fine grid to the basis, and
the fixtures add the solution points' basis indices and the maps through
the basis.

The *_cgrid fixtures (and *_cgrad) use the cubic pixel basis
(Raster_CubicPixel, raster_cp.cc) on its basis grid or on an intermediate
grid, with the same contents.

The *blob* fixtures use the blob bases (Raster_GaussBlob, Raster_HanningBlob,
Raster_RampBlob, Raster_SplineBlob: raster_bl.cc and its subclasses), which
pad the basis grid by the support radius; rgdim / rbdim hold the padded
sizes.

The *_el fixtures reset the solver in the element basis (one mua, mus',
nref per element, seeded) and hold the reference's system matrix, fields,
projections and element-basis Jacobian.

The qm_* fixtures hold a QM file written here (seeded positions off the
boundary, sparse link lists, normals on some lines), its mesh, and what the
reference's QMMesh::LoadQM made of them: source positions, detector
positions after InitM's placement (pulled to the boundary, or fixed and
nudged into an element; "external" lists as LoadQM leaves them) and the
link list.

Usage:  make -f oracle/Makefile.ref REF=<reference tree> -j8
        python tests/golden/make_golden.py [fixture names]
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from toastpp_gb300 import meshio, workloads  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")


def small_cylinder(freq, nopt=4):
    P = workloads.cylinder(rings=4, layers=6, seed=5, freq_mhz=freq)
    idx = np.arange(0, 80, 80 // nopt)[:nopt]
    P.qm = type(P.qm).all_to_all(P.qm.Q[idx] * 1.0, P.qm.M[idx] * 1.0)
    return P


# name -> (problem factory, solver, precon, tol, Jacobian)
FIXTURES = {
    "disc_cw_cg_ich": (lambda: workloads.disc(8, 3, 0.0, 6), "CG", "ICH", 1e-15, True),
    "disc_cw_cg_diag": (lambda: workloads.disc(8, 3, 0.0, 6), "CG", "DIAG", 1e-15, False),
    "disc_cw_cg_none": (lambda: workloads.disc(8, 3, 0.0, 6), "CG", "NONE", 1e-15, False),
    "disc_fd_bicgstab_ich": (lambda: workloads.disc(8, 3, 100.0, 6), "BICGSTAB", "ICH", 1e-15, True),
    "disc_fd_bicgstab_diag": (lambda: workloads.disc(8, 3, 100.0, 6), "BICGSTAB", "DIAG", 1e-15, False),
    "disc_fd_bicgstab_none": (lambda: workloads.disc(8, 3, 100.0, 6), "BICGSTAB", "NONE", 1e-15, False),
    "disc_fd_gmres_ich": (lambda: workloads.disc(8, 3, 100.0, 6), "GMRES", "ICH", 1e-15, False),
    "disc_fd_gmres_diag": (lambda: workloads.disc(8, 3, 100.0, 6), "GMRES", "DIAG", 1e-15, False),
    "disc_fd_gmres_none": (lambda: workloads.disc(8, 3, 100.0, 6), "GMRES", "NONE", 1e-15, False),
    "cyl_cw_cg_ich": (lambda: small_cylinder(0.0), "CG", "ICH", 1e-15, True),
    "cyl_fd_bicgstab_ich": (lambda: small_cylinder(100.0), "BICGSTAB", "ICH", 1e-15, True),
    "cyl_fd_gmres_ich": (lambda: small_cylinder(100.0), "GMRES", "ICH", 1e-15, False),
    # LSOLVER_DIRECT: Cholesky (real) and SuperLU (complex), exact FP64 solves
    # up to round-off: the accuracy reference of the mixed path
    "disc_cw_direct": (lambda: workloads.disc(8, 3, 0.0, 6), "DIRECT", "NONE", 1e-15, True),
    "disc_fd_direct": (lambda: workloads.disc(8, 3, 100.0, 6), "DIRECT", "NONE", 1e-15, True),
    "cyl_cw_direct": (lambda: small_cylinder(0.0), "DIRECT", "NONE", 1e-15, True),
    "cyl_fd_direct": (lambda: small_cylinder(100.0), "DIRECT", "NONE", 1e-15, True),
    # grid-basis Jacobians (Raster_Pixel, basis = grid)
    "disc_cw_grid": (lambda: workloads.disc(8, 3, 0.0, 6), "CG", "ICH", 1e-15, False, (24, 24)),
    "disc_fd_grid": (lambda: workloads.disc(8, 3, 100.0, 6), "BICGSTAB", "ICH", 1e-15, False, (24, 20)),
    "cyl_cw_grid": (lambda: small_cylinder(0.0), "CG", "ICH", 1e-15, False, (9, 10, 12)),
    "cyl_fd_grid": (lambda: small_cylinder(100.0), "BICGSTAB", "ICH", 1e-15, False, (10, 9, 11)),
    # element basis (Reset(sol, omega, true), GenerateJacobian(RASTER_ELBASIS, ...))
    "disc_cw_el": (lambda: workloads.disc(8, 3, 0.0, 6), "CG", "ICH", 1e-15, False, None, True),
    "disc_fd_el": (lambda: workloads.disc(8, 3, 100.0, 6), "BICGSTAB", "ICH", 1e-15, False, None, True),
    "cyl_cw_el": (lambda: small_cylinder(0.0), "CG", "ICH", 1e-15, False, None, True),
    "cyl_fd_el": (lambda: small_cylinder(100.0), "BICGSTAB", "ICH", 1e-15, False, None, True),
    # data gradient on a raster (toast Gradient: GetGradient / AddDataGradient)
    "disc_fd_grad": (lambda: workloads.disc(8, 3, 100.0, 6), "BICGSTAB", "ICH", 1e-15, False, (20, 20), False,
                     True),
    "cyl_fd_grad": (lambda: small_cylinder(100.0), "BICGSTAB", "ICH", 1e-15, False, (9, 9, 10), False, True),
    # Raster_Pixel with an intermediate grid (toast.Raster(mesh, grd, intgrd)):
    # basis grd, fine grid intgrd
    "disc_cw_igrid": (lambda: workloads.disc(8, 3, 0.0, 6), "CG", "ICH", 1e-15, False, (12, 12), False, False,
                      (24, 24)),
    "disc_fd_igrid": (lambda: workloads.disc(8, 3, 100.0, 6), "BICGSTAB", "ICH", 1e-15, False, (11, 9), False,
                      False, (31, 25)),
    "cyl_cw_igrid": (lambda: small_cylinder(0.0), "CG", "ICH", 1e-15, False, (5, 6, 7), False, False, (11, 12, 13)),
    "cyl_fd_igrid": (lambda: small_cylinder(100.0), "BICGSTAB", "ICH", 1e-15, False, (6, 5, 6), False, False,
                     (14, 12, 11)),
    "disc_fd_igrad": (lambda: workloads.disc(8, 3, 100.0, 6), "BICGSTAB", "ICH", 1e-15, False, (10, 10), False,
                      True, (28, 28)),
    # Raster_CubicPixel (cubic B-spline basis), on its basis grid or an
    # intermediate grid
    "disc_cw_cgrid": (lambda: workloads.disc(8, 3, 0.0, 6), "CG", "ICH", 1e-15, False, (14, 14), False, False,
                      (14, 14), "cubic"),
    "disc_fd_cgrid": (lambda: workloads.disc(8, 3, 100.0, 6), "BICGSTAB", "ICH", 1e-15, False, (10, 9), False,
                      False, (27, 25), "cubic"),
    "cyl_cw_cgrid": (lambda: small_cylinder(0.0), "CG", "ICH", 1e-15, False, (5, 6, 6), False, False, (11, 12, 13),
                     "cubic"),
    "cyl_fd_cgrid": (lambda: small_cylinder(100.0), "BICGSTAB", "ICH", 1e-15, False, (6, 6, 5), False, False,
                     (6, 6, 5), "cubic"),
    "disc_fd_cgrad": (lambda: workloads.disc(8, 3, 100.0, 6), "BICGSTAB", "ICH", 1e-15, False, (9, 9), False,
                      True, (25, 25), "cubic"),
    # blob bases (Raster_Blob): Gaussian, Hanning, ramp and spline blobs on a
    # padded grid of the basis size
    "disc_fd_gblob": (lambda: workloads.disc(8, 3, 100.0, 6), "BICGSTAB", "ICH", 1e-15, False, (12, 11), False,
                      False, (12, 11), "gauss:1.0:2.5"),
    "disc_cw_hblob": (lambda: workloads.disc(8, 3, 0.0, 6), "CG", "ICH", 1e-15, False, (10, 10), False, False,
                      (10, 10), "hanning::2.0"),
    "cyl_fd_rblob": (lambda: small_cylinder(100.0), "BICGSTAB", "ICH", 1e-15, False, (5, 5, 6), False, False,
                     (5, 5, 6), "ramp::1.5"),
    "cyl_cw_sblob": (lambda: small_cylinder(0.0), "CG", "ICH", 1e-15, False, (5, 6, 5), False, False, (5, 6, 5),
                     "spline::2.0"),
    "disc_fd_sblob_grad": (lambda: workloads.disc(8, 3, 100.0, 6), "BICGSTAB", "ICH", 1e-15, False, (11, 11),
                           False, True, (11, 11), "spline::2.0"),
}


def element_params(P, seed=11):
    """Seeded per-element parameters: the element mean of the nodal mua and
    mus' times 1 + 0.3 u (u uniform in [-1, 1]); the nodal refractive index's
    element mean."""
    rng = np.random.default_rng(seed)
    ne = len(P.elems)
    mua = P.mua[P.elems].mean(1) * (1 + 0.3 * rng.uniform(-1, 1, ne))
    mus = P.mus[P.elems].mean(1) * (1 + 0.3 * rng.uniform(-1, 1, ne))
    nref = P.nref[P.elems].mean(1)
    return mua, mus, nref


def rd(path, dtype):
    return np.fromfile(path, dtype=dtype)


def synthetic_data(logproj, seed=17):
    """Measured data for the gradient fixtures: the model's log amplitude and
    phase perturbed by seeded noise, and their standard deviations."""
    rng = np.random.default_rng(seed)
    mod, arg = logproj.real, logproj.imag
    data = np.concatenate([mod + 0.02 * rng.standard_normal(mod.size), arg + 0.01 * rng.standard_normal(arg.size)])
    sd = np.concatenate([0.05 * np.abs(mod) + 0.01, 0.05 * np.abs(arg) + 0.01])
    return data, sd


def run(name, factory, solver, precon, tol, jac, grid=None, elbasis=False, gradient=False, gdim=None,
        raster="pixel"):
    P = factory()
    cplx = P.complex
    with tempfile.TemporaryDirectory() as td:
        msh = os.path.join(td, "m.msh")
        meshio.write_mesh(msh, P.coords, P.elems)
        opt = os.path.join(td, "opt.bin")
        with open(opt, "wb") as f:
            np.array([P.dim, len(P.qm.Q), len(P.qm.M)], np.int32).tofile(f)
            np.ascontiguousarray(P.qm.Q, np.float64).tofile(f)
            np.ascontiguousarray(P.qm.M, np.float64).tofile(f)
        par = os.path.join(td, "par.bin")
        np.stack([P.mua, P.mus, P.nref], axis=1).astype(np.float64).tofile(par)
        out = os.path.join(td, "r")
        args = [DRIVER, f"mesh={msh}", f"optodes={opt}", f"out={out}", f"params={par}",
                f"dtype={'complex' if cplx else 'real'}", f"solver={solver}", f"precon={precon}", f"tol={tol}",
                "maxit=0", f"freq={P.freq_mhz}", f"qwidth={P.qwidth}", f"mwidth={P.mwidth}", f"jac={int(jac)}"]
        if grid:
            args += ["grid=" + ",".join(str(g) for g in grid), "fields=1"]
        if gdim:
            args += ["gdim=" + ",".join(str(g) for g in gdim)]
        if raster != "pixel":
            kind, sigma, sup = (raster.split(":") + ["", ""])[:3]
            args += [f"raster={kind}"] + ([f"sigma={sigma}"] if sigma else []) + ([f"sup={sup}"] if sup else [])
        if elbasis:
            emua, emus, eref = element_params(P)
            epar = os.path.join(td, "elpar.bin")
            np.stack([emua, emus, eref], axis=1).astype(np.float64).tofile(epar)
            args += [f"elparams={epar}", "fields=1", "sysmat=1"]
        if gradient:
            # the model data first, then the run with the perturbed data
            subprocess.run(args, check=True)
            lp = rd(out + "_logproj.bin", np.complex128)
            gdata, gsd = synthetic_data(lp)
            dfile, sfile = os.path.join(td, "data.bin"), os.path.join(td, "sd.bin")
            gdata.tofile(dfile)
            gsd.tofile(sfile)
            args += [f"data={dfile}", f"sd={sfile}"]
        subprocess.run(args, check=True)
        info = dict(l.split() for l in open(out + "_info.txt") if l.strip())
        ct = np.complex128 if cplx else np.float64
        res = dict(proj=rd(out + "_proj.bin", ct), logproj=rd(out + "_logproj.bin", ct),
                   it_fwd=int(info["it_fwd"]), it_adj=int(info["it_adj"]))
        if jac:
            nqm = len(res["proj"])
            J = rd(out + "_J.bin", np.float64)
            res["J"] = J.reshape((2 * nqm, 2 * P.n) if cplx else (2 * nqm, P.n))
        if elbasis:
            nqm = len(res["proj"])
            ne = len(P.elems)
            Je = rd(out + "_Jel.bin", np.float64)
            res["Jel"] = Je.reshape((2 * nqm, 2 * ne) if cplx else (2 * nqm, ne))
            res["elmua"], res["elmus"], res["elnref"] = element_params(P)
            res["sysval"] = rd(out + "_sysval.bin", ct)
            res["dphi"] = rd(out + "_dphi.bin", ct).reshape(len(P.qm.Q), P.n)
            res["aphi"] = rd(out + "_aphi.bin", ct).reshape(len(P.qm.M), P.n)
        if gradient:
            res["data"], res["sd"] = gdata, gsd
            res["grad"] = rd(out + "_grad.bin", np.float64)
        if grid:
            nqm = len(res["proj"])
            slen = int(info["slen"])
            Jg = rd(out + "_Jgrid.bin", np.float64)
            res["Jgrid"] = Jg.reshape((2 * nqm, 2 * slen) if cplx else (2 * nqm, slen))
            for key in ("m2g", "m2s", "s2m", "g2m"):
                res["map_" + key] = rd(out + f"_{key}.bin", np.float64)
            res["elref"] = rd(out + "_elref.bin", np.int32)
            res["bdim"] = np.array(grid, np.int32)
            if raster != "pixel":
                kind, sigma, sup = (raster.split(":") + ["", ""])[:3]
                res["raster"] = kind
                if sigma:
                    res["sigma"] = float(sigma)
                if sup:
                    res["sup"] = float(sup)
                dims = rd(out + "_rgdim.bin", np.int32)
                res["rgdim"], res["rbdim"] = dims[:P.dim], dims[P.dim:]
            if gdim:
                res["gdim"] = np.array(gdim, np.int32)
                res["sol2basis"] = rd(out + "_sol2basis.bin", np.int32)
                for key in ("m2b", "b2m", "g2b", "b2g", "g2s", "s2g"):
                    res["map_" + key] = rd(out + f"_{key}.bin", np.float64)
                for key in ("cm2s", "cs2m"):
                    res["map_" + key] = rd(out + f"_{key}.bin", np.complex128)
            res["dphi"] = rd(out + "_dphi.bin", ct).reshape(len(P.qm.Q), P.n)
            res["aphi"] = rd(out + "_aphi.bin", ct).reshape(len(P.qm.M), P.n)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), coords=P.coords, elems=P.elems, Q=P.qm.Q, M=P.qm.M,
                        link_ofs=P.qm.link_ofs, link_m=P.qm.link_m, mua=P.mua, mus=P.mus, nref=P.nref,
                        freq_mhz=P.freq_mhz, qwidth=P.qwidth, mwidth=P.mwidth, solver=solver, precon=precon,
                        tol=tol, **res)
    print(name, "n", P.n, "links", len(res["proj"]), "its", res["it_fwd"], res["it_adj"])


def qm_text(P, Q, M, links, mflag, seed, qflag="", QN=None, MN=None):
    """A QM file as QMMesh::LoadQM reads it (qmmesh.cc:319-460): every other
    position line also carries a normal, which the reader parses and drops
    for non-external lists; QN / MN, where given, are the normals of every
    line of that list."""
    rng = np.random.default_rng(seed)
    dim = P.dim
    out = [f"QM file {dim}D", f"Dimension {dim}", "", f"SourceList {len(Q)}" + (" " + qflag if qflag else "")]
    for i, p in enumerate(Q):
        nrm = list(QN[i]) if QN is not None else (list(rng.standard_normal(dim)) if i % 2 else [])
        out.append(" ".join(repr(float(v)) for v in list(p) + nrm))
    out += ["", f"MeasurementList {len(M)}" + (" " + mflag if mflag else "")]
    for i, p in enumerate(M):
        nrm = list(MN[i]) if MN is not None else (list(rng.standard_normal(dim)) if i % 2 == 0 else [])
        out.append(" ".join(repr(float(v)) for v in list(p) + nrm))
    out += ["", "LinkList"]
    for ms in links:
        out.append(f"{len(ms)}: " + " ".join(str(m) for m in ms))
    return "\n".join(out) + "\n"


def _radial(P, pts, dr):
    """Points moved by dr along their radius in the cross-section."""
    pts = np.array(pts, float)
    r = np.linalg.norm(pts[:, :2], axis=1, keepdims=True)
    pts[:, :2] *= (r + dr[:, None]) / r
    return pts


def _tilted_inward(rng, Q, deg):
    """Unit normals along -q turned by up to deg degrees in the x-y plane,
    scaled by a random length (the reader normalises them)."""
    out = []
    for q in Q:
        n = -np.asarray(q, float) / np.linalg.norm(q)
        t = np.radians(rng.uniform(-deg, deg))
        c, s = np.cos(t), np.sin(t)
        n[:2] = c * n[0] - s * n[1], s * n[0] + c * n[1]
        out.append(n * rng.uniform(0.5, 2.0))
    return np.array(out)


def qm_case(kind):
    """Problem and QM text of a QM fixture: detectors pulled to the boundary
    (2D and 3D) or at fixed positions just inside (or, one of them, 5e-5
    outside) the boundary; sparse link lists with a source without links.
    The *_external cases put the sources outside the mesh in an "external"
    list: 2D with the "default" normals (towards the origin), 3D with
    normals read from the file, tilted from the inward radius; their
    detectors are an "external" list too, kept where they were read."""
    seeds = {"qm_disc_pull": 31, "qm_cyl_pull": 32, "qm_disc_fixed": 33, "qm_disc_external": 34,
             "qm_cyl_external": 35}
    rng = np.random.default_rng(seeds[kind])
    P = workloads.disc(8, 3, 0.0, 6) if kind.startswith("qm_disc") else small_cylinder(0.0, nopt=6)
    nq, nm = len(P.qm.Q), len(P.qm.M)
    qflag, QN, MN = "", None, None
    if kind.endswith("_external"):
        Q = _radial(P, P.qm.Q, rng.uniform(0.05, 0.5, nq))
    else:
        Q = _radial(P, P.qm.Q, rng.uniform(-0.3, 0.3, nq))
    if kind == "qm_disc_fixed":
        # midpoints of boundary edges (edges of one triangle only), moved
        # inward 1e-3 (the last 5e-5 outward)
        cnt = {}
        for t in P.elems:
            for a, b in ((t[0], t[1]), (t[1], t[2]), (t[2], t[0])):
                k = (min(a, b), max(a, b))
                cnt[k] = cnt.get(k, 0) + 1
        edges = [k for k, c in cnt.items() if c == 1]
        mids = np.array([0.5 * (P.coords[a] + P.coords[b]) for a, b in edges])
        order = np.argsort(np.arctan2(mids[:, 1], mids[:, 0]))
        M = mids[order[np.linspace(0, len(order) - 1, nm, endpoint=False).astype(int)]]
        M = _radial(P, np.array(M), np.array([-1e-3] * (nm - 1) + [5e-5]))
        flag = "fixed"
    elif kind == "qm_disc_external":
        M = _radial(P, P.qm.M, rng.uniform(-0.4, 0.4, nm))
        qflag, flag = "external default", "external"
        MN = rng.standard_normal((nm, P.dim))
    elif kind == "qm_cyl_external":
        M = _radial(P, P.qm.M, rng.uniform(-0.4, 0.4, nm))
        qflag, flag = "external", "external default"
        QN = _tilted_inward(rng, Q, 25.0)
    else:
        M = _radial(P, P.qm.M, rng.uniform(-0.4, 0.4, nm))
        flag = ""
    links = []
    for q in range(nq):
        if q == 1:
            links.append([])
        else:
            ms = [m for m in range(nm) if q == 0 or rng.uniform() < 0.7]
            links.append(ms)
    return P, qm_text(P, Q, M, links, flag, rng.integers(1 << 30), qflag, QN, MN)


def run_qm(name):
    P, text = qm_case(name)
    with tempfile.TemporaryDirectory() as td:
        msh = os.path.join(td, "m.msh")
        meshio.write_mesh(msh, P.coords, P.elems)
        qmf = os.path.join(td, "f.qm")
        with open(qmf, "w") as f:
            f.write(text)
        out = os.path.join(td, "r")
        subprocess.run([DRIVER, f"mesh={msh}", f"qm={qmf}", f"out={out}", "qmdump=1"], check=True)
        qpos = rd(out + "_qpos.bin", np.float64).reshape(-1, P.dim)
        mpos = rd(out + "_mpos.bin", np.float64).reshape(-1, P.dim)
        nref = rd(out + "_nqmref.bin", np.int32)
        qmref = rd(out + "_qmref.bin", np.int32)
    ofs = np.concatenate([[0], np.cumsum(nref)]).astype(np.int32)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), coords=P.coords, elems=P.elems, qm_text=text,
                        qpos=qpos, mpos=mpos, link_ofs=ofs, link_m=qmref)
    print(name, "nQ", len(qpos), "nM", len(mpos), "nQM", len(qmref))


QM_FIXTURES = ("qm_disc_pull", "qm_cyl_pull", "qm_disc_fixed", "qm_disc_external", "qm_cyl_external")


def main():
    if not os.path.exists(DRIVER):
        sys.exit("build the reference driver first: make -f oracle/Makefile.ref REF=<reference tree>")
    names = sys.argv[1:] or list(FIXTURES) + list(QM_FIXTURES)
    for name in names:
        if name in QM_FIXTURES:
            run_qm(name)
        else:
            run(name, *FIXTURES[name])


if __name__ == "__main__":
    main()
