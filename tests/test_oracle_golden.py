"""The oracle against the reference's own test fixtures (CPU only)."""
import numpy as np
import pytest

from helpers import golden, golden_problem, rel_err, to_zorder
from oracle import pyoracle as po


@pytest.mark.parametrize("method", ["bicgstab", "gmres", "si"])
def test_golden_flux(method):
    """tests/RadiativeTransfer_test.cc:84-152: 64 scalar-flux dofs within 1e-3."""
    import ouranos_gb300 as og
    prob, g = golden_problem(og)
    # the oracle builds its own quadrature from the reference's GLC table
    spec = prob.arrays()
    q = po.quadrature(po.QUAD_GLC, 4, 0, False, 1.0, 2)
    spec.update(omega=q["omega"], m2d=q["m2d"], d2m=q["d2m"], moment_l=q["moment_l"],
                most_normal=q["most_normal"])
    P = po.OracleProblem(spec)
    x, it, hist = P.solve(method, tol=1e-10, max_it=500)
    got = to_zorder(x, 4, 4)
    assert np.max(np.abs(got - np.array(g["solution"]))) < g["tolerance"]


def _fe_oracle(case):
    m = case["mesh"]
    n = m["subdivisions"]
    q = po.quadrature(po.QUAD_LS, 2, 0, False, 1.0, 2)
    spec = dict(dim=2, fe_order=m["fe_order"], n_cells=[n, n], lower=[m["lo"]] * 2,
                upper=[m["hi"]] * 2, n_groups=1, omega=q["omega"], m2d=q["m2d"], d2m=q["d2m"],
                moment_l=q["moment_l"], weight_sum=1.0, sigma_t=np.ones((1, 1)),
                sigma_s=np.zeros(1), l_max=0, material_id=np.zeros(n * n, np.int32))
    P = po.OracleProblem(spec)
    # deal.II cell index of the test -> lexicographic (subdivided_hyper_cube numbers
    # coarse cells lexicographically)
    return P.fecell(m["cell"])


@pytest.mark.parametrize("name", ["one cell", "two cells"])
def test_fecell_facts(name):
    """tests/FECell_test.cc: every pinned FE matrix entry and normal."""
    case = golden("fecell_facts.json")[name]
    fe = _fe_oracle(case)
    mats = {"mass": fe["mass"][None], "grad": fe["grad"], "downwind": fe["downwind"],
            "upwind": fe["upwind"]}
    assert case["facts"]
    for f in case["facts"]:
        if f["matrix"] in ("material_id", "source_id"):
            continue
        if f["matrix"] == "normal":
            v = fe["normals"][f["arg"], f["i"]]
        else:
            arg = 0 if f["arg"] is None else f["arg"]
            v = mats[f["matrix"]][arg, f["i"], f["j"]]
        if f["exact"]:
            assert v == f["value"], f
        else:
            assert abs(v - f["value"]) < f["tol"], f


def test_quadrature_facts_oracle():
    """tests/RTQuadrature_test.cc: LS S4 Galerkin and GLC S4 facts."""
    facts = golden("quadrature_facts.json")
    ls = facts["LS"]
    q = po.quadrature(po.QUAD_LS, ls["sn"], ls["L_max"], ls["galerkin"], 4 * np.pi, 2,
                      po.HARM_REFERENCE)
    assert q["n_dir"] == ls["n_dir"] and q["n_mom"] == ls["n_mom"]
    assert list(q["moment_l"]) == ls["l"]
    assert list(q["omega"][0]) == ls["omega0"]
    assert (q["most_normal"].astype(bool) == np.array(ls["most_normal"])).all()
    assert np.abs(q["d2m"] @ q["m2d"] - np.eye(ls["n_dir"])).max() < 1e-12
    glc = facts["GLC"]
    q = po.quadrature(po.QUAD_GLC, glc["sn"], glc["L_max"], glc["galerkin"], 4 * np.pi, 2)
    assert q["n_dir"] == glc["n_dir"] and q["n_mom"] == glc["n_mom"]
    assert list(q["moment_l"]) == glc["l"]
    assert np.abs(q["omega"][0] - np.array(glc["omega0"])).max() < 1e-12


def test_material_layout():
    """tests/RTMaterialProperties_test.cc: sigma_s[mom + gp(L+1) + g G(L+1) + mat G^2(L+1)]."""
    import ouranos_gb300.inp as inp
    m = golden("inputs.json")
    mat = inp.read_materials(m["files"]["rtmaterial_properties.inp"], m["materials"]["n_materials"],
                             m["materials"]["n_groups"])
    for (a, g), v in m["materials"]["sigma_t"]:
        assert mat.sigma_t[a, g] == v
    for (a, g, gp, l), v in m["materials"]["sigma_s"]:
        assert mat.sigma_s[a, g, gp, l] == v


@pytest.mark.parametrize("which", ["geometry_2D", "geometry_3D"])
def test_geometry_layout(which):
    """tests/Geometry_test.cc: material / source ids laid out i + j nx + k nx ny."""
    import ouranos_gb300.inp as inp
    m = golden("inputs.json")
    geo = inp.read_geometry(m["files"][which + ".inp"], 2 if which.endswith("2D") else 3)
    exp = m[which]
    assert list(geo.n_subdivisions) == exp["subdivisions"]
    assert geo.n_materials == exp["n_materials"]
    for ijk, v in exp["material_ids"]:
        assert geo.coarse_material(*ijk) == v
    for ijk, v in exp["source_ids"]:
        assert geo.coarse_source(*ijk) == v


def test_oracle_schedulers_agree():
    """The reference's all-task scan and the linear ready counters run the same order."""
    import ouranos_gb300 as og
    p = og.config_small(n=6, sn=4)
    P = po.OracleProblem(p.arrays())
    x = np.random.default_rng(1).standard_normal(P.length)
    P.scattering_source(x)
    a = P.sweep(scheduler=0)
    o0 = P.last_order().copy()
    b = P.sweep(scheduler=1)
    o1 = P.last_order().copy()
    assert (o0 == o1).all()
    assert rel_err(a, b) == 0.0


def test_oracle_threads_agree():
    import ouranos_gb300 as og
    p = og.heterogeneous_2d(seed=3, n=12, fe_order=2, sn=8, l_max=3, blocks=3)
    P = po.OracleProblem(p.arrays())
    x = np.random.default_rng(2).standard_normal(P.length)
    assert rel_err(P.apply(x, threads=4), P.apply(x, threads=1)) < 1e-14


def test_oracle_infinite_medium():
    """Analytic check: with reflective-like symmetry absent, a thick homogeneous slab
    centre approaches q / sigma_a (phi_0 = sqrt(ws) * scalar flux / ws...)."""
    import ouranos_gb300 as og
    # very large domain relative to the mean free path: centre flux -> q / (sigma_t - sigma_s)
    q = og.build_quadrature("LS", 4, 0, dim=2)
    p = og.uniform_problem(2, 1, (24, 24), (0, 0), (240, 240), q, 1.0, 0.5, 1.0)
    P = po.OracleProblem(p.arrays())
    x, it, _ = P.solve("gmres", tol=1e-11, max_it=300)
    n = 4
    c = 12 + 24 * 12
    scalar = x[c * n:(c + 1) * n] * np.sqrt(4 * np.pi)  # phi_0 * Y00^-1
    assert np.allclose(scalar, 1.0 / 0.5, rtol=1e-3)
