"""The oracle against the committed golden fixtures (outputs of the compiled
reference on small seeded problems, tests/golden/make_golden.py): projections
and, where stored, the nodal Jacobian -- the Jacobian has no golden vectors in
the reference's own test data, so these fixtures are what pin it."""
import numpy as np
import pytest

from tests.golden_util import load, load_qm, names, qm_names
from tests.gpu_util import rel2, relmax


@pytest.mark.parametrize("name", names(nodal_only=True))
def test_oracle_matches_reference_fixture(oracle_mod, name):
    g = load(name)
    mesh = oracle_mod.Mesh(g["coords"], g["elems"])
    res = oracle_mod.forward_path(mesh, g["Q"], g["M"], g["link_ofs"], g["link_m"], g["mua"], g["mus"], g["nref"],
                                  freq_mhz=g["freq_mhz"], qwidth=g["qwidth"], mwidth=g["mwidth"], method=g["solver"],
                                  precon=g["precon"], tol=g["tol"], jac="J" in g)
    # both solve to |r|/|b| <= 1e-12 with the same algorithm; the elementwise
    # bound is the reference's own cmpvec tolerance for these outputs
    assert relmax(res.proj, g["proj"]) < 1e-8
    assert rel2(res.proj, g["proj"]) < 1e-10
    assert relmax(res.logproj.real, g["logproj"].real) < 1e-8
    if np.iscomplexobj(g["logproj"]):
        assert relmax(res.logproj.imag, g["logproj"].imag) < 1e-7
    if "J" in g:
        J = res.J.reshape(g["J"].shape)
        assert rel2(J, g["J"]) < 1e-9


GRID = [n for n in names() if n.endswith("_grid")]
# Raster_Pixel with an intermediate grid finer than the basis, and
# Raster_CubicPixel
IGRID = [n for n in names() if "gdim" in load(n) and str(load(n).get("raster", "pixel")) in ("pixel", "cubic")]
# the blob bases
BLOB = [n for n in names() if str(load(n).get("raster", "pixel")) in ("gauss", "hanning", "ramp", "spline")]


def blob_raster(oracle_mod, g, mesh):
    return oracle_mod.BlobRaster(mesh, str(g["raster"]), g["bdim"], g["sup"], g.get("sigma", 1.0))


@pytest.mark.parametrize("name", BLOB)
def test_oracle_blob_raster_matches_reference(oracle_mod, name):
    """The blob bases (Gaussian, Hanning, ramp, spline): the padded basis
    grid, the element per grid point, the solution points, the grid-basis
    Jacobian on the reference's fields and every basis map equal the
    reference's bit for bit."""
    g = load(name)
    mesh = oracle_mod.Mesh(g["coords"], g["elems"])
    B = blob_raster(oracle_mod, g, mesh)
    assert np.array_equal(B.pdim, g["rbdim"]) and np.array_equal(B.pdim, g["rgdim"])
    assert np.array_equal(B.elref, g["elref"])
    assert np.array_equal(B.sol2basis, g["sol2basis"])
    J = B.jacobian(g["dphi"], g["aphi"], g["proj"], g["link_ofs"], g["link_m"])
    assert np.array_equal(J, g["Jgrid"])
    for key, val in B.maps(g["mua"], g["mus"]).items():
        assert np.array_equal(val, g["map_" + key]), key


@pytest.mark.parametrize("name", GRID + IGRID)
def test_oracle_grid_jacobian_matches_reference(oracle_mod, name):
    """Raster_Pixel (basis = grid, or an intermediate grid), Raster_CubicPixel,
    and the grid-basis Jacobian on the reference's own fields: the element
    reference per grid point, the solution points and every Jacobian entry
    equal the reference's bit for bit."""
    g = load(name)
    mesh = oracle_mod.Mesh(g["coords"], g["elems"])
    gdim, kind = g.get("gdim"), str(g.get("raster", "pixel"))
    r = oracle_mod.raster_pixel(mesh, g["bdim"] if gdim is None else gdim)
    assert np.array_equal(r.elref, g["elref"])
    if gdim is not None:
        assert np.array_equal(oracle_mod.raster_support(mesh, g["bdim"], gdim, kind), g["sol2basis"])
    J = oracle_mod.jacobian_grid(mesh, g["bdim"], g["dphi"], g["aphi"], g["proj"], g["link_ofs"], g["link_m"],
                                 gdim=gdim, kind=kind)
    assert J.shape == g["Jgrid"].shape
    assert np.array_equal(J, g["Jgrid"])


@pytest.mark.parametrize("name", IGRID)
def test_oracle_basis_maps_match_reference(oracle_mod, name):
    """With an intermediate grid (or the cubic basis) the maps through the
    basis (Grid2LinPix G, LinPix2Grid GI, the products C = G B and CI = BI GI
    in the reference's entry order, the support D; the cubic raster's G and
    GI) equal the reference's bit for bit, the complex M->S / S->M (run
    through the grid) included."""
    g = load(name)
    mesh = oracle_mod.Mesh(g["coords"], g["elems"])
    maps = oracle_mod.raster_basis_maps(mesh, g["bdim"], g["gdim"], g["mua"], g["mus"],
                                        str(g.get("raster", "pixel")))
    for key in ("m2b", "b2m", "g2b", "b2g", "g2s", "s2g", "m2s", "s2m", "cm2s", "cs2m"):
        assert np.array_equal(maps[key], g["map_" + key]), key


ELEM = [n for n in names() if n.endswith("_el")]


@pytest.mark.parametrize("name", ELEM)
def test_oracle_element_basis_matches_reference(oracle_mod, name):
    """Element-basis assembly (one coefficient per element) and the
    element-basis Jacobian on the reference's own fields: both equal the
    reference's bit for bit."""
    g = load(name)
    mesh = oracle_mod.Mesh(g["coords"], g["elems"])
    cm, ck, ca = oracle_mod.optical_coefficients(g["elmua"], g["elmus"], g["elnref"])
    cplx = np.iscomplexobj(g["proj"])
    val = oracle_mod.assemble_el(mesh, cm, ck, ca, g["freq_mhz"] * 2 * np.pi * 1e-6, cplx)
    assert np.array_equal(val, g["sysval"])
    J = oracle_mod.jacobian_el(mesh, g["dphi"], g["aphi"], g["proj"], g["link_ofs"], g["link_m"])
    assert np.array_equal(J, g["Jel"])


GRAD = [n for n in names() if n.endswith(("_grad", "_igrad", "_cgrad"))]


@pytest.mark.parametrize("name", GRAD)
def test_oracle_data_gradient_matches_reference(oracle_mod, name):
    """toast's Gradient (weights from the data residuals, one adjoint solve per
    source, grid products) on the reference's fields: equal to the
    reference's bit for bit, adjoint solves included."""
    g = load(name)
    m = oracle_mod.Mesh(g["coords"], g["elems"])
    cm, ck, ca = oracle_mod.optical_coefficients(g["mua"], g["mus"], g["nref"])
    val = m.assemble(cm, ck, ca, g["freq_mhz"] * 2 * np.pi * 1e-6, True)
    mvec = np.stack([m.qvec_gaussian(x, g["mwidth"]) * ca for x in g["M"]]).astype(np.complex128)
    kind = str(g.get("raster", "pixel"))
    if name in BLOB:
        kind = blob_raster(oracle_mod, g, m)
    grad = oracle_mod.data_gradient(m, g["bdim"], val, g["dphi"], mvec, g["proj"], g["logproj"], g["link_ofs"],
                                    g["link_m"], g["data"], g["sd"], g["solver"], g["precon"], g["tol"],
                                    gdim=g.get("gdim"), kind=kind)
    assert np.array_equal(grad, g["grad"])


@pytest.mark.parametrize("name", GRID + IGRID)
def test_oracle_raster_maps_match_reference(oracle_mod, name):
    """The pixel raster's basis maps (mesh -> grid, mesh -> solution,
    solution -> mesh through NodeMapMatrix, grid -> mesh) equal the
    reference's bit for bit (with an intermediate grid: mesh -> grid and
    grid -> mesh; the rest run through the basis)."""
    g = load(name)
    mesh = oracle_mod.Mesh(g["coords"], g["elems"])
    grid = g.get("gdim", g["bdim"])
    slen = int((g["elref"] >= 0).sum())
    maps = oracle_mod.raster_maps(mesh, grid, g["mua"], np.arange(1, slen + 1, dtype=float))
    keys = ("m2g", "m2s", "s2m", "g2m") if "gdim" not in g else ("m2g", None, None, "g2m")
    for a, key in zip(maps, keys):
        if key:
            assert np.array_equal(a, g["map_" + key]), key


@pytest.mark.parametrize("name", qm_names())
def test_oracle_qm_placement_matches_reference(oracle_mod, name, tmp_path):
    """The QM file parsed (meshio.read_qm) and the detectors placed as InitM
    places them (pulled to the boundary, or fixed and nudged into an
    element) equal what the compiled reference's LoadQM made, bit for bit.
    qm_disc_pull has two detectors whose projection no boundary side takes:
    the reference keeps them where they were read.  The *_external files
    move their sources to the boundary along the normals (2D: the segment
    from near the origin; 3D: the whole line, where the reference takes the
    crossing on the far side) and keep their detectors as read."""
    from toastpp_gb300 import meshio
    g, path = load_qm(name, tmp_path)
    qm = meshio.read_qm(path)
    mesh = oracle_mod.Mesh(g["coords"], g["elems"])
    if qm.q_external:
        Q = mesh.external_sources(qm.Q, None if qm.q_default_normals else qm.QN)
        assert not np.array_equal(Q, qm.Q)
    else:
        Q = qm.Q
    assert np.array_equal(Q, g["qpos"])
    M = qm.M if qm.m_external else mesh.place_detectors(qm.M, qm.m_fixed)
    assert np.array_equal(M, g["mpos"])
    assert np.array_equal(qm.link_ofs, g["link_ofs"]) and np.array_equal(qm.link_m, g["link_m"])
