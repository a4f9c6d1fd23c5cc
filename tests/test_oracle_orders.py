"""The oracle's task orders and its own workload generator (CPU only).

The ready-list order restates the reference scheduler
(src/RadiativeTransfer.cc:605-692); the cartesian order runs the same tasks
without the task graph, for the meshes whose graph would not fit in memory.
Both must give the same flux moments up to the order of the additions.
"""
import numpy as np
import pytest

from helpers import rel_err
from oracle import pyoracle as po
from oracle import workloads


def _cases(og):
    return [og.heterogeneous_2d(seed=11, n=16, fe_order=2, sn=8, l_max=3, blocks=4),
            og.heterogeneous_2d(seed=12, n=13, fe_order=1, sn=4, l_max=1, blocks=3),
            og.thick_3d(seed=2001, n=6, sn=4, block=2, width=2.0),
            og.uniform_problem(3, 2, (4, 5, 3), (0, 0, 0), (1.0, 1.0, 1.0),
                               og.build_quadrature("LS", 4, 1, dim=3), 3.0, 2.0, 1.0)]


@pytest.mark.parametrize("k", range(4))
@pytest.mark.parametrize("threads", [1, 3])
def test_cartesian_order_matches_ready_list(k, threads):
    import ouranos_gb300 as og
    prob = _cases(og)[k]
    x = np.random.default_rng(k).standard_normal(prob.vector_length)
    fifo = po.OracleProblem(prob.arrays())
    cart = po.OracleProblem(prob.arrays(), order="cartesian")
    assert rel_err(cart.apply(x, threads=threads), fifo.apply(x, threads=threads)) < 1e-14
    assert rel_err(cart.rhs(threads=threads), fifo.rhs(threads=threads)) < 1e-14


def test_cartesian_order_with_sources_inflow_and_time_step():
    """Right-hand side with fixed sources and ISOTROPIC / MOST_NORMAL inflow,
    and an implicit-Euler angular-flux advance, in both orders."""
    import ouranos_gb300 as og
    q = og.build_quadrature("LS", 4, 1, dim=3)
    rng = np.random.default_rng(3)
    n = (4, 3, 5)
    nc = int(np.prod(n))
    prob = og.Problem(3, 1, n, (0, 0, 0), (1.0, 0.8, 1.2), q, rng.uniform(1, 3, (2, 1)),
                      rng.uniform(0, 0.5, (2, 1, 1, 2)), rng.integers(0, 2, nc).astype(np.int32),
                      rng.integers(0, 2, nc).astype(np.int32), rng.uniform(0, 2, (2, 1)),
                      (1, 0, 2, 0, 1, 2), rng.uniform(0.5, 1.5, (6, 1)))
    fifo = po.OracleProblem(prob.arrays())
    cart = po.OracleProblem(prob.arrays(), order="cartesian")
    assert rel_err(cart.rhs(), fifo.rhs()) < 1e-14
    for o in (fifo, cart):
        o.set_time_step(0.5)
    phi = rng.standard_normal(prob.vector_length)
    fifo.advance_angular(phi)
    cart.advance_angular(phi, threads=2)
    assert rel_err(cart.angular_flux(), fifo.angular_flux()) < 1e-14
    assert rel_err(cart.rhs(), fifo.rhs()) < 1e-14


def test_task_graph_built_on_demand():
    """Levels and task ids still come from the reference's task graph when the
    problem sweeps in the cartesian order."""
    import ouranos_gb300 as og
    prob = og.thick_3d(seed=2003, n=4, sn=4, block=4, width=1.0)
    cart = po.OracleProblem(prob.arrays(), order="cartesian")
    lv = cart.task_levels()
    assert lv.shape == (prob.quad.n_dir, prob.total_cells)
    assert (lv == po.OracleProblem(prob.arrays()).task_levels()).all()


@pytest.mark.parametrize("args", [dict(seed=1001, n=32), dict(seed=5, n=21, fe_order=1, sn=8, l_max=1, blocks=4)])
def test_oracle_workload_equals_product_problem(args):
    """The oracle's own generator (used by the CPU baseline arm) draws the
    same material map, source region and quadrature as the product's."""
    import ouranos_gb300 as og
    spec = workloads.heterogeneous_2d(**args)
    prob = og.heterogeneous_2d(**args).arrays()
    for key in ("material_id", "source_id", "sigma_t", "sigma_s", "moment_l", "most_normal", "source"):
        assert np.array_equal(np.asarray(spec[key]).reshape(-1), np.asarray(prob[key]).reshape(-1)), key
    for key in ("omega", "m2d", "d2m"):
        assert np.allclose(spec[key], prob[key], rtol=0, atol=1e-13), key
    assert spec["n_cells"] == prob["n_cells"] and spec["upper"] == list(prob["upper"])
    assert workloads.vector_length(spec) == og.heterogeneous_2d(**args).vector_length
