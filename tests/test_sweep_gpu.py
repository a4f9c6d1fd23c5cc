"""GPU parity: the sm_103a sweep through the C-ABI against the oracle."""
import numpy as np
import pytest

from helpers import golden, golden_problem, rel_err, to_zorder
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

# FP64 parity bar: the GPU sweep matches the reference's CPU sweep to 1e-12
# relative (norm-wise over the whole flux-moment vector).
TOL64 = 1e-12


def _problems():
    import ouranos_gb300 as og
    P = {}
    P["2d-q1-ls4"] = lambda: og.config_small(n=8, sn=4)
    P["2d-q1-ls8-32"] = lambda: og.config_small(n=32, sn=8)
    P["2d-q2-ls8-p3"] = lambda: og.heterogeneous_2d(seed=11, n=16, fe_order=2, sn=8, l_max=3, blocks=4)
    P["2d-q1-ls16-ragged"] = lambda: og.heterogeneous_2d(seed=12, n=21, fe_order=1, sn=16, l_max=1, blocks=3)
    P["2d-q3-glc6"] = lambda: og.uniform_problem(2, 3, (9, 7), (0, 0), (3.0, 2.0),
                                                 og.build_quadrature("GLC", 6, 2, dim=2), 2.0, 1.5, 1.0)
    P["2d-q4-ls4"] = lambda: og.uniform_problem(2, 4, (6, 5), (0, 0), (1.0, 1.0),
                                                og.build_quadrature("LS", 4, 0, dim=2), 5.0, 1.0, 1.0)
    P["3d-q1-glc4"] = lambda: og.thick_3d(seed=2001, n=6, sn=4, block=2, width=2.0)
    P["3d-q1-ls4-box"] = lambda: og.uniform_problem(3, 1, (5, 6, 7), (0, 0, 0), (1.0, 2.0, 3.0),
                                                    og.build_quadrature("LS", 4, 1, dim=3), 1.0, 0.7, 1.0)
    P["3d-q2-ls4"] = lambda: og.uniform_problem(3, 2, (4, 5, 3), (0, 0, 0), (1.0, 1.0, 1.0),
                                                og.build_quadrature("LS", 4, 0, dim=3), 3.0, 2.0, 1.0)
    P["3d-q1-glc6-aniso"] = lambda: _aniso3d(og)
    return P


def _aniso3d(og):
    q = og.build_quadrature("GLC", 6, 2, dim=3)
    p = og.uniform_problem(3, 1, (6, 5, 6), (0, 0, 0), (2.0, 2.0, 2.0), q, 2.0, 1.5, 1.0)
    ss = np.zeros((1, 1, 1, 3))
    ss[0, 0, 0] = [1.5, 0.6, 0.2]
    p.sigma_s = ss
    return p


PROBLEMS = _problems()


@pytest.mark.parametrize("name", sorted(PROBLEMS))
def test_apply_matches_oracle(name):
    import ouranos_gb300 as og
    prob = PROBLEMS[name]()
    x = np.random.default_rng(hash(name) % 2 ** 32).standard_normal(prob.vector_length)
    ref = po.OracleProblem(prob.arrays()).apply(x)
    with og.RadiativeTransfer(prob) as rt:
        y = rt.apply(x)
    assert rel_err(y, ref) < TOL64


@pytest.mark.parametrize("tiling", [(32, 1, 1), (16, 1, 2), (8, 1, 4), (4, 1, 8), (2, 1, 16)])
def test_tilings_2d(tiling):
    import ouranos_gb300 as og
    prob = og.heterogeneous_2d(seed=5, n=40, fe_order=2, sn=8, l_max=1, blocks=5)
    x = np.random.default_rng(3).standard_normal(prob.vector_length)
    ref = po.OracleProblem(prob.arrays()).apply(x)
    with og.RadiativeTransfer(prob) as rt:
        rt.set_tiling(*tiling)
        assert rt.tiling() == tiling
        y = rt.apply(x)
    assert rel_err(y, ref) < TOL64


@pytest.mark.parametrize("tiling", [(16, 1, 1), (8, 1, 2), (4, 1, 4), (2, 1, 8), (1, 1, 16)])
@pytest.mark.parametrize("order", [2, 3, 4])
def test_two_lanes_per_cell_2d(tiling, order):
    """Cells of 9 or more dofs may be solved by two lanes each (16 cells per
    warp): every 16-lane tiling matches the oracle, in FP64 and FP32."""
    import ouranos_gb300 as og
    prob = og.heterogeneous_2d(seed=6, n=21, fe_order=order, sn=6, l_max=1, blocks=3)
    x = np.random.default_rng(5).standard_normal(prob.vector_length)
    ref = po.OracleProblem(prob.arrays()).apply(x)
    with og.RadiativeTransfer(prob) as rt:
        rt.set_tiling(*tiling)
        assert rt.tiling() == tiling
        assert rel_err(rt.apply(x), ref) < TOL64
        rt.set_precision("fp32")
        assert rel_err(rt.apply(x), ref) < 2e-6


@pytest.mark.parametrize("tiling", [(4, 4, 1), (4, 2, 2), (2, 2, 4), (16, 1, 1)])
def test_two_lanes_per_cell_3d(tiling):
    import ouranos_gb300 as og
    prob = og.thick_3d(seed=2003, n=9, fe_order=2, sn=4, block=3, width=3.0)
    x = np.random.default_rng(6).standard_normal(prob.vector_length)
    ref = po.OracleProblem(prob.arrays()).apply(x)
    with og.RadiativeTransfer(prob) as rt:
        rt.set_tiling(*tiling)
        assert rel_err(rt.apply(x), ref) < TOL64


def test_default_tiling_and_lane_rules():
    """Q2+ cells default to two lanes per cell (16 cells per warp); Q1 cells
    keep one lane per cell and reject 16-lane tilings."""
    import ouranos_gb300 as og
    from ouranos_gb300 import _capi
    with og.RadiativeTransfer(og.heterogeneous_2d(seed=7, n=16, fe_order=2, sn=4, l_max=0, blocks=2)) as rt:
        assert rt.tiling() == (16, 1, 1)
    with og.RadiativeTransfer(og.thick_3d(seed=2004, n=8, fe_order=2, sn=4, block=4, width=2.0)) as rt:
        assert rt.tiling() == (4, 4, 1)
    with og.RadiativeTransfer(og.thick_3d(seed=2004, n=8, sn=4, block=4, width=2.0)) as rt:
        assert rt.tiling() == (4, 8, 1)
    with og.RadiativeTransfer(og.config_small(n=16, sn=4)) as rt:
        assert rt.tiling() == (32, 1, 1)
        with pytest.raises(_capi.OuranosError) as e:
            rt.set_tiling(16, 1, 1)
        assert e.value.code == _capi.ERR_BAD_INPUT


@pytest.mark.parametrize("tiling", [(4, 4, 2), (8, 4, 1), (4, 8, 1), (4, 2, 4), (2, 2, 8), (2, 4, 4)])
def test_tilings_3d(tiling):
    import ouranos_gb300 as og
    prob = og.thick_3d(seed=2002, n=9, sn=4, block=3, width=3.0)
    x = np.random.default_rng(4).standard_normal(prob.vector_length)
    ref = po.OracleProblem(prob.arrays()).apply(x)
    with og.RadiativeTransfer(prob) as rt:
        rt.set_tiling(*tiling)
        y = rt.apply(x)
    assert rel_err(y, ref) < TOL64


def _sourced_problem(og, dim=2):
    """Multigroup problem with sources, isotropic and most-normal inflow."""
    if dim == 2:
        q = og.build_quadrature("LS", 6, 1, dim=2)
        n, lo, hi = (7, 9), (0, 0), (1.5, 2.0)
        bc = (1, 2, 0, 1, 0, 0)
    else:
        q = og.build_quadrature("LS", 4, 1, dim=3)
        n, lo, hi = (5, 4, 6), (0, 0, 0), (1.0, 1.0, 1.5)
        bc = (1, 0, 2, 0, 1, 2)
    G = 3
    nc = int(np.prod(n))
    rng = np.random.default_rng(7)
    st = rng.uniform(0.5, 3.0, (2, G))
    ss = rng.uniform(0.0, 0.3, (2, G, G, 2))
    mat = rng.integers(0, 2, nc).astype(np.int32)
    sid = rng.integers(0, 2, nc).astype(np.int32)
    src = rng.uniform(0.0, 2.0, (2, G))
    inc = rng.uniform(0.5, 1.5, (2 * dim, G))
    return og.Problem(dim, 1, n, lo, hi, q, st, ss, mat, sid, src, bc, inc)


@pytest.mark.parametrize("dim", [2, 3])
def test_rhs_sweep_sources_boundaries_groups(dim):
    """The driver's RHS sweep (src/ouranos.cc:152-158): fixed sources, other-group
    scattering and ISOTROPIC / MOST_NORMAL inflow, every group."""
    import ouranos_gb300 as og
    prob = _sourced_problem(og, dim)
    O = po.OracleProblem(prob.arrays())
    gf = np.random.default_rng(9).standard_normal(prob.n_groups * prob.vector_length)
    with og.RadiativeTransfer(prob) as rt:
        for g in range(prob.n_groups):
            rt.set_group(g)
            O.set_group(g)
            O.clear_scattering_source()
            ref = O.sweep(group_flux=gf)
            got = rt.rhs(group_flux=gf)
            assert rel_err(got, ref) < TOL64
            # sweep() with a stored scattering source accumulates into its argument
            x = np.random.default_rng(g).standard_normal(prob.vector_length)
            O.scattering_source(x)
            base = np.random.default_rng(100 + g).standard_normal(prob.vector_length)
            ref2 = O.sweep(flux=base.copy(), group_flux=gf)
            rt.compute_scattering_source(x)
            got2 = rt.sweep(base.copy(), gf)
            assert rel_err(got2, ref2) < TOL64


def test_levels_match_oracle_dag():
    import ouranos_gb300 as og
    prob = og.thick_3d(seed=2003, n=5, sn=4, block=5, width=1.0)
    with og.RadiativeTransfer(prob) as rt:
        lv = rt.task_levels()
    assert (lv == po.OracleProblem(prob.arrays()).task_levels()).all()


@pytest.mark.parametrize("method", ["gmres", "bicgstab", "si"])
def test_golden_flux_through_product(method):
    """tests/RadiativeTransfer_test.cc:84-152 replayed on the GPU operator, with the
    reference's z-order dof numbering passed through cell_order."""
    import ouranos_gb300 as og
    prob, g = golden_problem(og)
    prob.cell_order = og.zorder_cells(4, 4)
    with og.RadiativeTransfer(prob) as rt:
        x, info, hist = rt.solve(method, tol=1e-10, max_it=400)
    assert info["converged"]
    assert np.max(np.abs(x - np.array(g["solution"]))) < g["tolerance"]


def test_cell_order_permutation():
    import ouranos_gb300 as og
    prob = og.heterogeneous_2d(seed=21, n=8, fe_order=2, sn=4, l_max=1, blocks=2)
    x = np.random.default_rng(5).standard_normal(prob.vector_length)
    with og.RadiativeTransfer(prob) as rt:
        y_lex = rt.apply(x)
    order = np.random.default_rng(6).permutation(64).astype(np.int64)
    prob.cell_order = order
    n = prob.dofs_per_cell
    xp = np.zeros_like(x)
    for m in range(prob.quad.n_mom):
        for c in range(64):
            xp[m * prob.n_dofs + order[c] * n:m * prob.n_dofs + (order[c] + 1) * n] = \
                x[m * prob.n_dofs + c * n:m * prob.n_dofs + (c + 1) * n]
    with og.RadiativeTransfer(prob) as rt:
        yp = rt.apply(xp)
    back = np.zeros_like(yp)
    for m in range(prob.quad.n_mom):
        for c in range(64):
            back[m * prob.n_dofs + c * n:m * prob.n_dofs + (c + 1) * n] = \
                yp[m * prob.n_dofs + order[c] * n:m * prob.n_dofs + (order[c] + 1) * n]
    assert rel_err(back, y_lex) < 1e-14


def test_solvers_match_oracle():
    import ouranos_gb300 as og
    prob = og.heterogeneous_2d(seed=31, n=12, fe_order=2, sn=8, l_max=3, blocks=3)
    O = po.OracleProblem(prob.arrays())
    xo, it_o, _ = O.solve("gmres", tol=1e-11, max_it=400, restart=30)
    with og.RadiativeTransfer(prob) as rt:
        for method in ("gmres", "bicgstab", "si"):
            x, info, hist = rt.solve(method, tol=1e-11, max_it=2000)
            assert info["converged"], (method, info)
            assert rel_err(x, xo) < 1e-9, method
        x, info, hist = rt.solve("fgmres_mixed", tol=1e-10, max_it=400)
        assert info["converged"] and info["residual"] < 1e-10
        assert rel_err(x, xo) < 1e-8


def test_fp32_sweep_accuracy():
    import ouranos_gb300 as og
    prob = og.heterogeneous_2d(seed=41, n=24, fe_order=2, sn=8, l_max=3, blocks=4)
    x = np.random.default_rng(8).standard_normal(prob.vector_length)
    ref = po.OracleProblem(prob.arrays()).apply(x)
    with og.RadiativeTransfer(prob, precision="fp32") as rt:
        y = rt.apply(x)
    assert rel_err(y, ref) < 2e-6


def test_device_pointers():
    torch = pytest.importorskip("torch")
    import ouranos_gb300 as og
    prob = og.config_small(n=16, sn=4)
    x = np.random.default_rng(1).standard_normal(prob.vector_length)
    ref = po.OracleProblem(prob.arrays()).apply(x)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    with og.RadiativeTransfer(prob) as rt:
        rt.Apply(xd, yd)
        torch.cuda.synchronize()
    assert rel_err(yd.cpu().numpy(), ref) < TOL64


def test_device_input_written_just_before_the_call():
    """A device vector whose last write is still queued on the default stream
    (behind a long kernel) when Apply is called is read complete: the handle's
    stream is ordered after the caller's earlier default-stream work."""
    torch = pytest.importorskip("torch")
    import ouranos_gb300 as og
    prob = og.config_small(n=16, sn=4)
    x = np.random.default_rng(3).standard_normal(prob.vector_length)
    ref = po.OracleProblem(prob.arrays()).apply(x)
    src = torch.from_numpy(x).cuda()
    big = torch.randn(4096, 4096, device="cuda")
    torch.cuda.synchronize()
    with og.RadiativeTransfer(prob) as rt:
        for _ in range(3):
            xd = torch.zeros_like(src)
            yd = torch.empty_like(src)
            for _ in range(8):
                big = big @ big
                big = big / big.norm()
            xd.copy_(src)  # queued behind the matmuls
            rt.Apply(xd, yd)
            assert rel_err(yd.cpu().numpy(), ref) < TOL64


def test_wait_timeout_reports_error_and_recovers():
    """A dependency wait that cannot be satisfied (target biased past the end)
    runs out after the wait limit: the call returns OURANOS_ERR_TIMEOUT, no
    fault, and the next call on the same handle is correct."""
    import ouranos_gb300 as og
    from ouranos_gb300 import _capi
    prob = og.config_small(n=40, sn=4)  # several tiles -> inter-tile waits
    x = np.random.default_rng(2).standard_normal(prob.vector_length)
    ref = po.OracleProblem(prob.arrays()).apply(x)
    with og.RadiativeTransfer(prob) as rt:
        rt.set_tiling(8, 1, 4)
        rt.set_wait_limit(2e7)  # 20 ms
        rt.debug_wait_bias(1 << 20)
        with pytest.raises(_capi.OuranosError) as e:
            rt.apply(x)
        assert e.value.code == _capi.ERR_TIMEOUT
        rt.debug_wait_bias(0)
        rt.set_wait_limit(2e9)
        y = rt.apply(x)
    assert rel_err(y, ref) < TOL64


@pytest.mark.parametrize("mode", ["native", "df64", "df64_sweep", "df64_sweep_tc"])
def test_fp64_contraction_modes_match_oracle(mode):
    """Every FP64 arithmetic (native FP64; double-float contractions; double-float
    contractions and cell solves; the latter with the contractions on the tensor
    cores) keeps the 1e-12 parity bar, on P3 (expanded
    source), P0 (fused moments), 2-D Q1-Q4 and 3-D Q1-Q2, Apply and RHS sweeps."""
    import ouranos_gb300 as og
    probs = [og.heterogeneous_2d(seed=61, n=20, fe_order=2, sn=8, l_max=3, blocks=4),
             og.heterogeneous_2d(seed=62, n=12, fe_order=4, sn=4, l_max=1, blocks=4),
             og.heterogeneous_2d(seed=63, n=16, fe_order=1, sn=4, l_max=0, blocks=4),
             og.thick_3d(seed=2061, n=6, sn=4, block=2, width=2.0),
             og.uniform_problem(3, 2, (4, 5, 3), (0, 0, 0), (1.0, 1.0, 1.0),
                                og.build_quadrature("LS", 4, 0, dim=3), 2.0, 1.5, 1.0)]
    for prob in probs:
        x = np.random.default_rng(61).standard_normal(prob.vector_length)
        O = po.OracleProblem(prob.arrays())
        ref = O.apply(x)
        ref_rhs = O.rhs()
        with og.RadiativeTransfer(prob) as rt:
            rt.set_fp64_contractions(mode)
            y = rt.apply(x)
            r = rt.rhs()
        assert rel_err(y, ref) < TOL64, prob.name
        assert rel_err(r, ref_rhs) < TOL64, prob.name


def _three_group_problem(og, dim):
    """Three groups with down- and up-scatter (P1), sources, inflow and
    reflective sides."""
    if dim == 2:
        q = og.build_quadrature("LS", 4, 1, dim=2)
        n, lo, hi, bc = (6, 7), (0, 0), (1.2, 1.4), (1, 3, 0, 2, 0, 0)
    else:
        q = og.build_quadrature("LS", 4, 1, dim=3)
        n, lo, hi, bc = (4, 3, 5), (0, 0, 0), (1.0, 0.8, 1.2), (1, 0, 3, 0, 2, 0)
    G = 3
    nc = int(np.prod(n))
    rng = np.random.default_rng(29)
    st = rng.uniform(1.0, 5.0, (2, G))
    ss = np.zeros((2, G, G, 2))
    for m in range(2):
        for gf in range(G):
            for gt in range(G):
                ss[m, gf, gt, 0] = rng.uniform(0.05, 0.25) * st[m, gt]
            ss[m, gf, gf, 0] = rng.uniform(0.3, 0.6) * st[m, gf]
            ss[m, gf, gf, 1] = 0.3 * ss[m, gf, gf, 0]
    mat = rng.integers(0, 2, nc).astype(np.int32)
    sid = rng.integers(0, 2, nc).astype(np.int32)
    src = rng.uniform(0.0, 2.0, (2, G))
    inc = rng.uniform(0.5, 1.5, (2 * dim, G))
    return og.Problem(dim, 1, n, lo, hi, q, st, ss, mat, sid, src, bc, inc)


@pytest.mark.parametrize("dim,method,dsa", [(2, "gmres", False), (2, "si", False), (3, "bicgstab", False),
                                            (2, "fgmres_mixed", True), (3, "gmres", True)])
def test_multigroup_outer_iteration_matches_oracle(dim, method, dsa):
    """Gauss-Seidel over the groups (src/ouranos.cc:62-207) against the same
    outer loop driven through the oracle's single-group solves."""
    import ouranos_gb300 as og
    prob = _three_group_problem(og, dim)
    O = po.OracleProblem(prob.arrays())
    G, L = prob.n_groups, O.length
    ref = np.zeros(G * L)
    for _ in range(200):
        old = ref.copy()
        for g in range(G):
            O.set_group(g)
            ref[g * L:(g + 1) * L] = O.solve("gmres", tol=1e-13, max_it=800, group_flux=ref)[0]
        if np.linalg.norm(ref - old) < 1e-12 * np.linalg.norm(ref):
            break
    with og.RadiativeTransfer(prob) as rt:
        if dsa:
            rt.set_dsa(10)
        gf, info = rt.solve_multigroup(method, inner_tol=1e-12, outer_tol=1e-11, max_outer_it=200, dsa=dsa)
    assert info["converged"] and info["outer_iterations"] > 1
    tol = 1e-6 if method == "fgmres_mixed" else 1e-8
    assert rel_err(gf, ref) < tol


@pytest.mark.parametrize("case", ["2d-q2-p3-df64", "2d-q2-p3-native", "2d-q2-p3-tc", "2d-q2-p3-fp32", "3d-q1-fused",
                                  "ragged"])
def test_pinned_host_apply_overlaps_and_matches_the_device_apply(case):
    """Apply on page-locked host vectors moves x and y in cell ranges on a copy
    stream, overlapped with the per-cell kernels on either side of the sweep;
    the kernels and their per-dof arithmetic are the device Apply's, so y is
    bit-identical (also in place, and for cell counts that do not split
    evenly)."""
    torch = pytest.importorskip("torch")
    import ouranos_gb300 as og
    if case.startswith("2d"):
        prob = og.heterogeneous_2d(seed=11, n=32, fe_order=2, sn=8, l_max=3, blocks=4)
    elif case == "3d-q1-fused":
        prob = og.thick_3d(seed=2003, n=12, sn=4, block=3, width=3.0)
    else:
        prob = og.heterogeneous_2d(seed=12, n=23, fe_order=1, sn=4, l_max=1, blocks=1)
    prec = "fp32" if case.endswith("fp32") else "fp64"
    with og.RadiativeTransfer(prob, precision=prec) as rt:
        if case.endswith("native"):
            rt.set_fp64_contractions("native")
        if case.endswith("tc"):
            rt.set_fp64_contractions("df64_sweep_tc")
        x = torch.from_numpy(np.random.default_rng(8).standard_normal(prob.vector_length)).cuda()
        yd = torch.empty_like(x)
        rt.Apply(x, yd)
        xh = x.cpu().pin_memory()
        yh = torch.empty_like(xh).pin_memory()
        for _ in range(2):
            rt.Apply(xh, yh)
            assert torch.equal(yh, yd.cpu())
        rt.Apply(xh, xh)  # in place
        assert torch.equal(xh, yd.cpu())


@pytest.mark.parametrize("k", [-60, 60])
def test_double_float_apply_is_exactly_scale_invariant(k):
    """The double-float sweep and contractions hold the FP32 exponent range
    (about 1e-38 .. 3e38 per part).  Every operation of the Apply is linear
    and rounds the same way after an exact power-of-two scaling, so
    Apply(2^k x) = 2^k Apply(x) bit for bit while no part leaves that range."""
    import ouranos_gb300 as og
    prob = og.heterogeneous_2d(seed=81, n=24, fe_order=2, sn=8, l_max=3, blocks=3)
    x = np.random.default_rng(81).standard_normal(prob.vector_length)
    with og.RadiativeTransfer(prob) as rt:
        y = rt.apply(x)
        ys = rt.apply(np.ldexp(x, k))
    assert np.array_equal(ys, np.ldexp(y, k))


@pytest.mark.parametrize("scale", [1e-25, 1e25])
@pytest.mark.parametrize("mode", ["df64_sweep", "df64_sweep_tc"])
def test_double_float_apply_far_from_unit_scale_matches_oracle(scale, mode):
    """Flux moments of magnitude 1e+-25 (sigma_t from 0.1 to 100, cells of
    width 0.4): the double-float Apply stays within the 1e-12 parity bar."""
    import ouranos_gb300 as og
    prob = og.heterogeneous_2d(seed=82, n=24, fe_order=2, sn=8, l_max=3, blocks=3)
    x = scale * np.random.default_rng(82).standard_normal(prob.vector_length)
    ref = po.OracleProblem(prob.arrays()).apply(x)
    with og.RadiativeTransfer(prob) as rt:
        rt.set_fp64_contractions(mode)
        y = rt.apply(x)
    assert rel_err(y, ref) < TOL64
