"""Implicit Euler in the oracle: the time-step fixed point is the steady state."""
import numpy as np

from helpers import rel_err
from oracle import pyoracle as po


def test_implicit_euler_steps_approach_the_steady_solution():
    import ouranos_gb300 as og
    quad = og.build_quadrature("LS", 4, 0, dim=2)
    prob = og.uniform_problem(2, 1, (6, 6), (0, 0), (3.0, 3.0), quad, 1.0, 0.5, 1.0)
    steady = po.OracleProblem(prob.arrays()).solve("gmres", tol=1e-13, max_it=400)[0]
    O = po.OracleProblem(prob.arrays())
    O.set_time_step(2.0)
    phi = np.zeros(O.length)
    prev = None
    for _ in range(60):
        phi = O.solve("gmres", tol=1e-13, max_it=400)[0]
        O.advance_angular(phi)
        if prev is not None:
            assert rel_err(phi, steady) <= rel_err(prev, steady) * (1 + 1e-9)  # monotone approach
        prev = phi
    assert rel_err(phi, steady) < 1e-9
    # the stored psi^n reproduces phi through the quadrature: phi_m = sum_d D2M psi_d
    psi = O.angular_flux().reshape(O.n_dir, O.n_dofs)
    d2m = np.asarray(prob.quad.d2m).reshape(prob.quad.n_mom, prob.quad.n_dir)
    assert rel_err(d2m @ psi, phi.reshape(prob.quad.n_mom, O.n_dofs)) < 1e-12


def test_first_step_from_rest_is_a_shifted_steady_solve():
    """From psi^0 = 0 one step solves the steady problem with sigma_t + 1/(v dt)."""
    import ouranos_gb300 as og
    quad = og.build_quadrature("LS", 4, 0, dim=2)
    prob = og.uniform_problem(2, 1, (5, 5), (0, 0), (2.0, 2.0), quad, 1.0, 0.5, 1.0)
    O = po.OracleProblem(prob.arrays())
    O.set_time_step(0.75)
    phi = O.solve("gmres", tol=1e-13, max_it=400)[0]
    shifted = og.uniform_problem(2, 1, (5, 5), (0, 0), (2.0, 2.0), quad, 1.75, 0.5, 1.0)
    ref = po.OracleProblem(shifted.arrays()).solve("gmres", tol=1e-13, max_it=400)[0]
    assert rel_err(phi, ref) < 1e-11
