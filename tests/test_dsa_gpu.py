"""Diffusion synthetic acceleration on the GPU: the correction against the
oracle's restatement (FP32 CG against FP64 CG with the same number of steps),
and its use in the solvers."""
import dataclasses

import numpy as np
import pytest

from helpers import rel_err
from oracle import dsa_oracle as do
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
TOL_CG = 1e-4  # FP32 vectors against the FP64 restatement, relative L2 of the correction


def _thick(n=8, seed=7000):
    import ouranos_gb300 as og
    return og.thick_3d(seed=seed, n=n, sn=4, width=10.0 * n / 64)


def _check_apply(prob, k, inv_vdt=0.0):
    import ouranos_gb300 as og
    d = do.Diffusion(prob, inv_vdt=inv_vdt)
    rng = np.random.default_rng(11)
    with og.RadiativeTransfer(prob) as rt:
        if inv_vdt:
            rt.set_time_step(inv_vdt)
        rt.set_dsa(k)
        v = rng.standard_normal(rt.length)
        z = rt.dsa_apply(v)
        ref = d.apply(v, k=k)
        n0 = d.vid.shape[0] * d.nodes
        assert rel_err(z[:n0] - v[:n0], ref[:n0] - v[:n0]) < TOL_CG
        assert np.array_equal(z[n0:], v[n0:])  # higher moments pass unchanged


@pytest.mark.parametrize("k", [1, 3, 20])
def test_3d_correction_matches_oracle(k):
    _check_apply(_thick(), k)


def test_3d_correction_with_time_step_matches_oracle():
    _check_apply(_thick(seed=7001), 10, inv_vdt=0.5)


@pytest.mark.parametrize("k", [1, 10])
def test_2d_anisotropic_reflective_correction_matches_oracle(k):
    """2-D Q1, P1 scattering (D uses sigma_s1), reflective on the low x and y
    sides (no Marshak term there)."""
    import ouranos_gb300 as og
    p = og.heterogeneous_2d(seed=1201, n=12, fe_order=1, sn=4, l_max=1, g_aniso=0.5, blocks=4)
    p = dataclasses.replace(p, bc_type=(3, 0, 3, 0, 0, 0))
    _check_apply(p, k)


def test_in_place_and_device_vectors():
    import torch

    import ouranos_gb300 as og
    prob = _thick(seed=7002)
    with og.RadiativeTransfer(prob) as rt:
        rt.set_dsa(5)
        v = np.random.default_rng(5).standard_normal(rt.length)
        ref = rt.dsa_apply(v)
        t = torch.tensor(v, device="cuda")
        rt.dsa_apply(t, out=t)
        assert np.array_equal(t.cpu().numpy(), ref)


@pytest.mark.parametrize("order,k", [(2, 1), (2, 10), (3, 6), (4, 6)])
def test_2d_higher_order_correction_matches_oracle(order, k):
    """DG Q_p cells: the Q_p residual enters through the mixed mass matrix of
    the vertex hat functions, the correction is the vertex field at the
    nodes."""
    import ouranos_gb300 as og
    p = og.heterogeneous_2d(seed=1203, n=10, fe_order=order, sn=4, l_max=1, g_aniso=0.4, blocks=5)
    _check_apply(p, k)


@pytest.mark.parametrize("k", [1, 10])
def test_3d_q2_correction_matches_oracle(k):
    import ouranos_gb300 as og
    _check_apply(og.thick_3d(seed=7004, n=6, fe_order=2, sn=4, block=3, width=1.0), k)


def test_q2_fgmres_with_dsa_converges_in_fewer_iterations():
    """3-D Q2 on the thick, scattering map: FGMRES(30) with FP32 sweeps and the
    diffusion correction takes a fraction of the plain iterations, to the FP64
    GMRES solution."""
    import ouranos_gb300 as og
    prob = og.thick_3d(seed=7005, n=12, fe_order=2, sn=4, block=3, width=10.0 * 12 / 64)
    with og.RadiativeTransfer(prob) as rt:
        x64, i64, _ = rt.solve("gmres", tol=1e-8, max_it=3000)
        rt.set_dsa(20)
        xm, im, _ = rt.solve("fgmres_mixed", tol=1e-8, max_it=3000, dsa=True)
    assert i64["converged"] and im["converged"]
    assert im["iterations"] * 3 < i64["iterations"]
    n0 = prob.total_cells * prob.dofs_per_cell
    assert rel_err(xm[:n0], x64[:n0]) < 1e-6


def test_missing_setup():
    import ouranos_gb300 as og
    from ouranos_gb300 import _capi
    with og.RadiativeTransfer(_thick()) as rt:
        with pytest.raises(_capi.OuranosError) as e:
            rt.solve("fgmres_mixed", dsa=True)
        assert e.value.code == _capi.ERR_BAD_INPUT


def test_fgmres_with_dsa_converges_in_fewer_iterations():
    """16^3 thick diffusive map: FGMRES(30) with FP32 sweeps and the diffusion
    correction reaches 1e-8 in a fraction of the plain iterations, at the FP64
    GMRES solution (scalar flux within 1e-6)."""
    import ouranos_gb300 as og
    prob = _thick(n=16)
    with og.RadiativeTransfer(prob) as rt:
        x64, i64, _ = rt.solve("gmres", tol=1e-8, max_it=2000)
        rt.set_dsa(20)
        xm, im, _ = rt.solve("fgmres_mixed", tol=1e-8, max_it=2000, dsa=True)
        xd, idd, _ = rt.solve("gmres", tol=1e-8, max_it=2000, dsa=True)
    assert i64["converged"] and im["converged"] and idd["converged"]
    assert im["iterations"] * 4 < i64["iterations"]
    assert idd["iterations"] * 4 < i64["iterations"]
    n0 = prob.total_cells * 8
    assert rel_err(xm[:n0], x64[:n0]) < 1e-6
    assert rel_err(xd[:n0], x64[:n0]) < 1e-6


def test_source_iteration_with_dsa():
    """Accelerated source iteration converges in far fewer sweeps than plain
    source iteration, to the GMRES solution."""
    import ouranos_gb300 as og
    prob = _thick(n=8, seed=7003)
    with og.RadiativeTransfer(prob) as rt:
        xg, _, _ = rt.solve("gmres", tol=1e-10, max_it=2000)
        xs, isi, _ = rt.solve("si", tol=1e-9, max_it=20000)
        rt.set_dsa(30)
        xa, ia, _ = rt.solve("si", tol=1e-9, max_it=20000, dsa=True)
    assert ia["converged"]
    assert ia["iterations"] * 5 < isi["iterations"]
    n0 = prob.total_cells * 8
    assert rel_err(xa[:n0], xg[:n0]) < 1e-6


def test_time_step_with_dsa_matches_plain():
    import ouranos_gb300 as og
    prob = og.time_dependent_3d(seed=4110, n=8, sn=4, block=4, width=2.5, inv_vdt=0.5)
    out = []
    for dsa in (False, True):
        with og.RadiativeTransfer(prob, precision="fp32") as rt:
            rt.set_time_step(0.5)
            if dsa:
                rt.set_dsa(10)
            phi = np.zeros(rt.length)
            its = 0
            for step in range(3):
                rt.set_source([[0.0], [og.pulse_strength(step, peak=10.0, center=1, width=1.0)]])
                info = rt.time_advance(phi, method="fgmres_mixed", tol=1e-10, dsa=dsa)
                assert info["converged"]
                its += info["iterations"]
            out.append((phi.copy(), its))
    # psi^n is stored in FP32 after every step: the two runs differ at its rounding
    assert rel_err(out[1][0], out[0][0]) < 1e-6
    assert out[1][1] < out[0][1]


@pytest.mark.parametrize("dim", [2, 3])
def test_multigroup_inflow_boundaries_uneven_cells(dim):
    """Three groups with P1 scattering, inflow (Marshak) and reflective sides,
    cells of different widths per axis: every group's correction matches the
    oracle after ouranos_rt_set_group (the tables follow the group)."""
    import ouranos_gb300 as og
    if dim == 2:
        q = og.build_quadrature("LS", 4, 1, dim=2)
        n, lo, hi, bc = (7, 9), (0, 0), (1.5, 2.0), (1, 3, 0, 2, 0, 0)
    else:
        q = og.build_quadrature("LS", 4, 1, dim=3)
        n, lo, hi, bc = (5, 4, 6), (0, 0, 0), (1.0, 1.3, 1.5), (1, 0, 3, 0, 2, 3)
    G = 3
    nc = int(np.prod(n))
    rng = np.random.default_rng(17)
    st = rng.uniform(0.5, 30.0, (2, G))
    ss = np.zeros((2, G, G, 2))
    for m in range(2):
        for g in range(G):
            ss[m, g, :, 0] = rng.uniform(0.0, 0.3, G) * st[m, g]
            ss[m, g, g, 0] = rng.uniform(0.5, 0.99) * st[m, g]
            ss[m, g, g, 1] = 0.4 * ss[m, g, g, 0]
    mat = rng.integers(0, 2, nc).astype(np.int32)
    prob = og.Problem(dim, 1, n, lo, hi, q, st, ss, mat, np.zeros(nc, dtype=np.int32),
                      np.ones((1, G)), bc, rng.uniform(0.5, 1.5, (2 * dim, G)))
    v = rng.standard_normal(prob.vector_length)
    with og.RadiativeTransfer(prob) as rt:
        rt.set_dsa(12)
        for g in (2, 0, 1):
            rt.set_group(g)
            z = rt.dsa_apply(v)
            d = do.Diffusion(prob, group=g)
            ref = d.apply(v, k=12)
            n0 = d.vid.shape[0] * d.nodes
            assert rel_err(z[:n0] - v[:n0], ref[:n0] - v[:n0]) < TOL_CG
            assert np.array_equal(z[n0:], v[n0:])


def test_grid_barrier_timeout_reports_error_and_recovers():
    """A grid barrier of the diffusion CG that cannot complete (the epoch it
    waits for is biased past what any block publishes) runs out after the
    wait limit: OURANOS_ERR_TIMEOUT with the diffusion message, no fault, and
    the next call on the same handle gives the same correction as before."""
    import ouranos_gb300 as og
    from ouranos_gb300 import _capi
    prob = _thick()
    with og.RadiativeTransfer(prob) as rt:
        v = np.random.default_rng(5).standard_normal(rt.length)
        rt.set_dsa(5)
        ref = rt.dsa_apply(v)
        rt.set_wait_limit(2e7)  # 20 ms
        rt.debug_wait_bias(1)
        with pytest.raises(_capi.OuranosError) as e:
            rt.dsa_apply(v)
        assert e.value.code == _capi.ERR_TIMEOUT
        assert "barrier" in str(e.value)
        rt.debug_wait_bias(0)
        rt.set_wait_limit(2e9)
        assert np.array_equal(rt.dsa_apply(v), ref)
