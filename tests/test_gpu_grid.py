"""Grid-basis Jacobian (pixel raster: basis = grid, or a basis on an
intermediate grid) on the GPU against the reference's own outputs
(tests/golden/*_grid.npz, *_igrid.npz, made by the compiled reference) and
the oracle."""
import numpy as np
import pytest

from tests.golden_util import load, names, sparse_links
from tests.gpu_util import rel2
from toastpp_gb300 import capi

pytestmark = pytest.mark.gpu

GRID = [n for n in names() if n.endswith("_grid")]
# Raster_Pixel with an intermediate grid finer than the basis
IGRID = [n for n in names() if n.endswith("_igrid")]
# Raster_CubicPixel, on its basis grid or an intermediate grid
CGRID = [n for n in names() if n.endswith("_cgrid")]
# the blob bases (Gaussian, Hanning, ramp, spline)
BLOB_KINDS = ("gauss", "hanning", "ramp", "spline")
BLOB = [n for n in names() if str(load(n).get("raster", "pixel")) in BLOB_KINDS]


def kind(g):
    return str(g.get("raster", "pixel"))


def make_raster(gm, g):
    return capi.Raster(gm, g["bdim"], g.get("gdim"), kind=kind(g), sup=float(g.get("sup", 2.0)),
                       sigma=float(g.get("sigma", 1.0)))


def oracle_jacobian(oracle_mod, g, om, proj, ofs, lm, logscale=True):
    """The oracle's grid-basis Jacobian of the fixture's raster."""
    if kind(g) in BLOB_KINDS:
        B = oracle_mod.BlobRaster(om, kind(g), g["bdim"], float(g["sup"]), float(g.get("sigma", 1.0)))
        return B.jacobian(g["dphi"], g["aphi"], proj, ofs, lm, logscale=logscale)
    return oracle_mod.jacobian_grid(om, g["bdim"], g["dphi"], g["aphi"], proj, ofs, lm, logscale=logscale,
                                    gdim=g.get("gdim"), kind=kind(g))


def setup(name):
    g = load(name)
    gm = capi.Mesh(g["coords"], g["elems"])
    r = make_raster(gm, g)
    cplx = np.iscomplexobj(g["proj"])
    s = capi.FwdSolver(gm, g["solver"], 1e-15, g["precon"], cplx, precision="fp64")
    return g, gm, r, s, capi.Links(g["link_ofs"], g["link_m"])


@pytest.mark.parametrize("name", GRID + IGRID + CGRID)
def test_raster_matches_reference(name):
    g, gm, r, s, L = setup(name)
    assert r.glen == int(np.prod(g.get("gdim", g["bdim"])))
    assert r.blen == int(np.prod(g["bdim"]))
    assert np.array_equal(r.elref(), g["elref"])
    if "gdim" in g:
        assert np.array_equal(r.sol2basis(), g["sol2basis"])
    else:
        assert r.slen == int((g["elref"] >= 0).sum())
        assert np.array_equal(r.sol2basis(), np.nonzero(g["elref"] >= 0)[0])


@pytest.mark.parametrize("name", GRID + IGRID + CGRID + BLOB)
def test_grid_jacobian_on_reference_fields(name):
    """Same fields as the reference: FP64 agrees to round-off, FP32 to FP32
    accuracy."""
    g, gm, r, s, L = setup(name)
    J = s.jacobian_grid(r, g["dphi"], g["aphi"], g["proj"], L)
    ref = g["Jgrid"]
    assert J.shape == ref.shape
    assert rel2(J, ref) < 1e-13
    assert np.abs(J - ref).max() <= 1e-12 * np.abs(ref).max()
    J32 = s.jacobian_grid(r, g["dphi"], g["aphi"], g["proj"], L, fp32=True)
    assert J32.dtype == np.float32
    assert rel2(J32.astype(np.float64), ref) < 1e-5


@pytest.mark.parametrize("name", GRID + IGRID + CGRID + BLOB)
def test_grid_jacobian_linear_data_against_oracle(name, oracle_mod):
    g, gm, r, s, L = setup(name)
    J = s.jacobian_grid(r, g["dphi"], g["aphi"], None, L, scale=capi.DATA_LIN)
    om = oracle_mod.Mesh(g["coords"], g["elems"])
    ref = oracle_jacobian(oracle_mod, g, om, g["proj"], g["link_ofs"], g["link_m"], logscale=False)
    assert rel2(J, ref) < 1e-13


@pytest.mark.parametrize("name", IGRID + CGRID)
def test_grid_jacobian_chunks(name, monkeypatch):
    """With an intermediate grid the rows are formed on the grid a chunk of
    sources at a time and then mapped to the basis; one-source chunks give
    the same J as one chunk."""
    g, gm, r, s, L = setup(name)
    J1 = s.jacobian_grid(r, g["dphi"], g["aphi"], g["proj"], L)
    monkeypatch.setenv("TOASTGPU_GRID_CHUNK_BYTES", "1")
    J2 = s.jacobian_grid(r, g["dphi"], g["aphi"], g["proj"], L)
    assert np.array_equal(J1, J2)


@pytest.mark.parametrize("name", GRID + IGRID + CGRID + BLOB)
def test_grid_jacobian_end_to_end(name):
    """GPU fields (FP64 path) -> projections -> grid Jacobian, against the
    reference's Jacobian from its own fields."""
    g, gm, r, s, L = setup(name)
    cm, ck, ca = capi.optical_coefficients(g["mua"], g["mus"], g["nref"])
    s.reset(cm, ck, ca, capi.omega_of(g["freq_mhz"]))
    q = gm.qvec_gaussian(g["Q"], g["qwidth"])
    m = gm.qvec_gaussian(g["M"], g["mwidth"]) * ca[None, :]
    dphi, _ = s.calc_fields(q)
    aphi, _ = s.calc_fields(m)
    proj = s.project_all(m, dphi, L, capi.DATA_LIN)
    J = s.jacobian_grid(r, dphi, aphi, proj, L)
    assert rel2(J, g["Jgrid"]) < 1e-9


@pytest.mark.parametrize("name", GRID + IGRID + CGRID + BLOB)
def test_grid_jacobian_sparse_links_against_oracle(name, oracle_mod):
    """Links missing for some (source, detector) pairs and a source without
    any, with a source count that leaves a partial group of sources."""
    g, gm, r, s, L = setup(name)
    ofs, lm, keep = sparse_links(g)
    J = s.jacobian_grid(r, g["dphi"], g["aphi"], g["proj"][keep], capi.Links(ofs, lm))
    om = oracle_mod.Mesh(g["coords"], g["elems"])
    ref = oracle_jacobian(oracle_mod, g, om, g["proj"][keep], ofs, lm)
    assert J.shape == ref.shape == (2 * len(keep), g["Jgrid"].shape[1])
    assert rel2(J, ref) < 1e-13


def test_raster_of_another_mesh_is_rejected():
    g, gm, r, s, L = setup(GRID[0])
    g2 = load(GRID[-1])
    other = capi.Mesh(g2["coords"], g2["elems"])
    r2 = capi.Raster(other, g2["bdim"])
    with pytest.raises(capi.ToastGPUError):
        s.jacobian_grid(r2, g["dphi"], g["aphi"], g["proj"], L)


GRAD = [n for n in names() if n.endswith(("_grad", "_igrad", "_cgrad"))]


@pytest.mark.parametrize("name", GRAD)
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 1e-6)])
def test_data_gradient_against_reference(name, precision, tol):
    """toast's Gradient on the GPU (forward solves, projections, weighted
    adjoint solves, grid products) against the compiled reference's.  The
    adjoint sources weight each detector by 1/|y|^2, so the far detectors'
    fields (|y| ~ e^-20 of the near ones) set the accuracy: the mixed path,
    stopped at the same 1e-15 relative residual, agrees to 4e-7 on the disc."""
    g = load(name)
    gm = capi.Mesh(g["coords"], g["elems"])
    r = make_raster(gm, g)
    s = capi.FwdSolver(gm, g["solver"], 1e-15, g["precon"], True, precision=precision)
    cm, ck, ca = capi.optical_coefficients(g["mua"], g["mus"], g["nref"])
    s.reset(cm, ck, ca, capi.omega_of(g["freq_mhz"]))
    q = gm.qvec_gaussian(g["Q"], g["qwidth"])
    m = gm.qvec_gaussian(g["M"], g["mwidth"]) * ca[None, :]
    grad, res = s.gradient(r, q, m, capi.Links(g["link_ofs"], g["link_m"]), g["data"], g["sd"])
    assert all(x[1] == 0 for x in res), res
    if precision == "mixed" and name in BLOB:
        # measured on the spline blob fixture: 2.0e-6 for the mixed path,
        # below 1e-9 for the FP64 path on the same basis (the blob mapping is
        # exact; the adjoint weights 1/|y|^2 amplify the solves' error by a
        # basis-dependent amount)
        tol = 5e-6
    assert rel2(grad, g["grad"]) < tol
    # grad is accumulated into: a second call from the first result doubles the sum
    grad2, _ = s.gradient(r, q, m, capi.Links(g["link_ofs"], g["link_m"]), g["data"], g["sd"], grad=grad)
    assert rel2(grad2, 2 * grad) < 1e-12


@pytest.mark.parametrize("name", GRID)
def test_raster_maps_match_reference(name):
    """tg_raster_map: mesh -> grid, mesh -> solution, solution -> mesh and
    grid -> mesh equal the reference's maps bit for bit; complex vectors map
    component by component; stacks map row by row."""
    g, gm, r, s, L = setup(name)
    sin = np.arange(1, r.slen + 1, dtype=float)
    m2g = r.map("M->G", g["mua"])
    assert np.array_equal(m2g, g["map_m2g"])
    assert np.array_equal(r.map("M->S", g["mua"]), g["map_m2s"])
    assert np.array_equal(r.map("S->M", sin), g["map_s2m"])
    assert np.array_equal(r.map("G->M", m2g), g["map_g2m"])
    assert np.array_equal(r.map("G->S", m2g), g["map_m2s"])
    assert np.array_equal(r.map("S->G", r.map("G->S", m2g))[g["elref"] >= 0], m2g[g["elref"] >= 0])
    z = r.map("M->S", g["mua"] + 2j * g["mua"])
    assert np.array_equal(z.real, g["map_m2s"]) and np.array_equal(z.imag, 2 * g["map_m2s"])
    st = r.map("S->M", np.stack([sin, 3 * sin]))
    assert np.array_equal(st[0], g["map_s2m"]) and np.array_equal(st[1], r.map("S->M", 3 * sin))


@pytest.mark.parametrize("name", IGRID + CGRID)
def test_basis_maps_match_reference(name):
    """With an intermediate grid or the cubic basis: every map through the
    basis (G, GI, the pixel raster's products G B and BI GI, the support)
    equals the reference's bit for bit, real and complex; the grid maps
    too."""
    g, gm, r, s, L = setup(name)
    b = np.arange(1, r.blen + 1, dtype=float)
    sv = np.arange(1, r.slen + 1, dtype=float)
    m2g = r.map("M->G", g["mua"])
    assert np.array_equal(m2g, g["map_m2g"])
    assert np.array_equal(r.map("G->M", m2g), g["map_g2m"])
    assert np.array_equal(r.map("M->B", g["mua"]), g["map_m2b"])
    assert np.array_equal(r.map("B->M", b), g["map_b2m"])
    assert np.array_equal(r.map("G->B", m2g), g["map_g2b"])
    assert np.array_equal(r.map("B->G", b), g["map_b2g"])
    assert np.array_equal(r.map("G->S", m2g), g["map_g2s"])
    assert np.array_equal(r.map("S->G", sv), g["map_s2g"])
    assert np.array_equal(r.map("M->S", g["mua"]), g["map_m2s"])
    assert np.array_equal(r.map("S->M", sv), g["map_s2m"])
    assert np.array_equal(r.map("B->S", b), b[r.sol2basis()])
    sb = r.map("S->B", sv)
    assert np.array_equal(sb[r.sol2basis()], sv) and np.count_nonzero(sb) == r.slen
    assert np.array_equal(r.map("M->S", g["mua"] + 1j * g["mus"]), g["map_cm2s"])
    cs = np.arange(1, r.slen + 1) - 0.5j * np.arange(r.slen)
    assert np.array_equal(r.map("S->M", cs), g["map_cs2m"])


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("name", BLOB)
def test_blob_raster_matches_reference(name):
    """A blob basis: the padded grid, the element per grid point and the
    solution points equal the reference's; every map agrees to round-off
    (the Gaussian and Hanning blob values come from the host's exp and cos;
    the ramp and spline ones are exact arithmetic)."""
    g, gm, r, s, L = setup(name)
    assert r.glen == r.blen == int(np.prod(g["rbdim"]))
    assert np.array_equal(r.elref(), g["elref"])
    assert np.array_equal(r.sol2basis(), g["sol2basis"])
    tol = 1e-14 if kind(g) in ("gauss", "hanning") else 0.0
    b = np.arange(1, r.blen + 1, dtype=float)
    sv = np.arange(1, r.slen + 1, dtype=float)
    m2g = r.map("M->G", g["mua"])
    checks = [(m2g, "m2g"), (r.map("M->S", g["mua"]), "m2s"), (r.map("S->M", sv), "s2m"),
              (r.map("G->M", m2g), "g2m"), (r.map("M->B", g["mua"]), "m2b"), (r.map("B->M", b), "b2m"),
              (r.map("G->B", m2g), "g2b"), (r.map("B->G", b), "b2g"), (r.map("G->S", m2g), "g2s"),
              (r.map("S->G", sv), "s2g"), (r.map("M->S", g["mua"] + 1j * g["mus"]), "cm2s")]
    cs = np.arange(1, r.slen + 1) - 0.5j * np.arange(r.slen)
    checks.append((r.map("S->M", cs), "cs2m"))
    for got, key in checks:
        assert _rel(got, g["map_" + key]) <= tol, key
