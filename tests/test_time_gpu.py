"""Implicit Euler on the GPU against the oracle: the shifted operator, the
psi^n source of source sweeps, whole steps with a pulse source, checkpoint
round trips and warm starts."""
import numpy as np
import pytest

from helpers import rel_err
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu
TOL64 = 1e-12


def _prob(seed=4100):
    import ouranos_gb300 as og
    return og.time_dependent_3d(seed=seed, n=8, sn=4, block=4, width=2.5, inv_vdt=0.5)


def test_shifted_apply_matches_oracle():
    import ouranos_gb300 as og
    prob = _prob()
    x = np.random.default_rng(1).standard_normal(prob.vector_length)
    O = po.OracleProblem(prob.arrays())
    O.set_time_step(0.5)
    with og.RadiativeTransfer(prob) as rt:
        rt.set_time_step(0.5)
        assert rel_err(rt.apply(x), O.apply(x)) < TOL64


def test_source_sweep_with_psi_n_matches_oracle():
    """rhs = D L^-1 (q + inflow + inv_vdt M psi^n) for a given psi^n (values
    exact in FP32, the storage precision of psi^n)."""
    import ouranos_gb300 as og
    prob = _prob(4101)
    O = po.OracleProblem(prob.arrays())
    O.set_time_step(0.5)
    psi = np.random.default_rng(2).uniform(0.0, 2.0, O.n_dir * O.n_dofs).astype(np.float32).astype(np.float64)
    O.set_angular_flux(psi)
    O.set_source([[0.0], [7.5]])
    with og.RadiativeTransfer(prob) as rt:
        rt.set_time_step(0.5)
        rt.set_angular_flux(psi)
        rt.set_source([[0.0], [7.5]])
        assert np.array_equal(rt.angular_flux(), psi)
        assert rel_err(rt.rhs(), O.rhs()) < TOL64


def test_time_steps_with_a_pulse_match_oracle():
    import ouranos_gb300 as og
    prob = _prob(4102)
    O = po.OracleProblem(prob.arrays())
    O.set_time_step(0.5)
    with og.RadiativeTransfer(prob) as rt:
        rt.set_time_step(0.5)
        phi = np.zeros(rt.length)
        for step in range(4):
            q = og.pulse_strength(step, peak=10.0, center=2, width=1.0)
            O.set_source([[0.0], [q]])
            rt.set_source([[0.0], [q]])
            ref = O.solve("gmres", tol=1e-13, max_it=500)[0]
            O.advance_angular(ref)
            info = rt.time_advance(phi, method="fgmres_mixed", tol=1e-11, max_it=500)
            assert info["converged"]
            # psi^n is stored in FP32 on the GPU, in FP64 by the oracle
            assert rel_err(phi, ref) < 1e-6, step
        assert rel_err(rt.angular_flux(), O.angular_flux()) < 1e-6


def test_checkpoint_round_trip_continues_identically():
    import ouranos_gb300 as og
    prob = _prob(4103)
    with og.RadiativeTransfer(prob) as a, og.RadiativeTransfer(prob) as b:
        a.set_time_step(0.5)
        a.set_source([[0.0], [5.0]])
        phi = np.zeros(a.length)
        for _ in range(2):
            a.time_advance(phi, method="gmres", tol=1e-11)
        saved_phi, saved_psi = phi.copy(), a.angular_flux()
        a.time_advance(phi, method="gmres", tol=1e-11)
        b.set_time_step(0.5)
        b.set_source([[0.0], [5.0]])
        b.set_angular_flux(saved_psi)
        phi_b = saved_phi.copy()
        b.time_advance(phi_b, method="gmres", tol=1e-11)
        assert np.array_equal(phi_b, phi)
        assert np.array_equal(b.angular_flux(), a.angular_flux())


def test_warm_start_from_the_solution_needs_no_iterations():
    import ouranos_gb300 as og
    prob = og.config_small(n=16, sn=4)
    with og.RadiativeTransfer(prob) as rt:
        x, info, _ = rt.solve("gmres", tol=1e-10, max_it=500)
        x2 = x.copy()
        _, info2, _ = rt.solve("gmres", tol=1e-9, max_it=500, x=x2, warm=True)
        assert info2["iterations"] == 0 and info2["converged"]
        _, info3, _ = rt.solve("fgmres_mixed", tol=1e-9, max_it=500, x=x.copy(), warm=True)
        assert info3["iterations"] <= 1 and info3["converged"]
