"""The double-float sweep's direction-axis contractions on the tensor cores
(exact BF16 digit products, OURANOS_FP64_DF64_SWEEP_TC) against the oracle and
against the same contractions on the CUDA cores.

Both forms carry about 48 significant bits (double-float inputs and
outputs), so they agree far below the 1e-12 parity bar; the bound below
(1e-14 norm-wise) is what the digit scheme promises: seven digits per value
(56 bits below the row's largest), exact level sums, and a last accumulator
whose FP32 rounding sits near 2^-48 of the scale.
"""
import numpy as np
import pytest

from helpers import rel_err
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL_FORMS = 1e-14


def _cases(og):
    return {
        "2d-q2-ls16-p3": og.heterogeneous_2d(seed=71, n=40, fe_order=2, sn=16, l_max=3, blocks=5),
        "2d-q1-ls6-p1-ragged": og.heterogeneous_2d(seed=72, n=37, fe_order=1, sn=6, l_max=1, blocks=3),
        "2d-q3-glc8-p2": og.uniform_problem(2, 3, (13, 9), (0, 0), (2.0, 1.5),
                                            og.build_quadrature("GLC", 8, 2, dim=2), 3.0, 2.0, 1.0),
        "3d-q1-glc12-p1": og.thick_3d(seed=2071, n=10, sn=12, block=2, width=2.0),
        "3d-q2-ls8-p3": og.uniform_problem(3, 2, (5, 4, 6), (0, 0, 0), (1.0, 1.2, 0.8),
                                           og.build_quadrature("LS", 8, 3, dim=3), 2.0, 1.0, 1.0),
    }


@pytest.mark.parametrize("name", ["2d-q2-ls16-p3", "2d-q1-ls6-p1-ragged", "2d-q3-glc8-p2", "3d-q1-glc12-p1",
                                  "3d-q2-ls8-p3"])
def test_tensor_core_contractions_match_oracle_and_cuda_cores(name):
    """Apply and RHS (sources, expanded q with the isotropic part) with the
    contractions on the tensor cores: within 1e-12 of the oracle and 1e-14 of
    the CUDA-core double-float contractions (directions in one to four chunks
    of 48, 3 to 16 moments)."""
    import ouranos_gb300 as og
    prob = _cases(og)[name]
    x = np.random.default_rng(71).standard_normal(prob.vector_length)
    O = po.OracleProblem(prob.arrays())
    ref, ref_rhs = O.apply(x), O.rhs()
    with og.RadiativeTransfer(prob) as rt:
        y_cc, r_cc = rt.apply(x), rt.rhs()
        rt.set_fp64_contractions("df64_sweep_tc")
        y_tc, r_tc = rt.apply(x), rt.rhs()
        y_tc2 = rt.apply(x)
    print(name, rel_err(y_tc, ref), rel_err(y_tc, y_cc), rel_err(r_tc, r_cc))
    assert np.array_equal(y_tc, y_tc2)  # deterministic
    assert rel_err(y_tc, ref) < TOL64
    assert rel_err(r_tc, ref_rhs) < TOL64
    assert rel_err(y_tc, y_cc) < TOL_FORMS
    assert rel_err(r_tc, r_cc) < TOL_FORMS


def test_tensor_core_contractions_wide_dynamic_range():
    """Flux moments spanning 1e-20 .. 1e20 across the cells: each dof row is
    scaled by its own power of two, so small and large rows keep their digits."""
    import ouranos_gb300 as og
    prob = og.heterogeneous_2d(seed=73, n=24, fe_order=2, sn=8, l_max=3, blocks=3)
    rng = np.random.default_rng(73)
    n0 = prob.n_dofs
    x = rng.standard_normal(prob.vector_length)
    scale = 10.0 ** rng.uniform(-20, 20, n0)
    x = (x.reshape(-1, n0) * scale).reshape(-1)
    ref = po.OracleProblem(prob.arrays()).apply(x)
    with og.RadiativeTransfer(prob) as rt:
        rt.set_fp64_contractions("df64_sweep_tc")
        y = rt.apply(x)
    assert rel_err(y, ref) < TOL64


def test_tensor_core_gmres_solve_matches_oracle():
    import ouranos_gb300 as og
    prob = og.heterogeneous_2d(seed=74, n=24, fe_order=2, sn=8, l_max=3, blocks=3)
    xo, _, _ = po.OracleProblem(prob.arrays()).solve("gmres", tol=1e-10, max_it=300)
    with og.RadiativeTransfer(prob) as rt:
        rt.set_fp64_contractions("df64_sweep_tc")
        x, info, _ = rt.solve("gmres", tol=1e-10, max_it=300)
    assert info["converged"]
    n0 = prob.n_dofs
    assert rel_err(x[:n0], xo[:n0]) < 1e-8


def test_tensor_core_contractions_refused_beyond_192_directions():
    """3-D LS S16 has 288 directions: more chunks of 48 than the reduction's
    tensor memory holds; the mode is refused and the handle keeps its own."""
    import ouranos_gb300 as og
    from ouranos_gb300 import _capi
    prob = og.uniform_problem(3, 1, (3, 3, 3), (0, 0, 0), (1.0, 1.0, 1.0),
                              og.build_quadrature("LS", 16, 0, dim=3), 1.0, 0.5, 1.0)
    assert prob.quad.n_dir == 288
    x = np.random.default_rng(0).standard_normal(prob.vector_length)
    with og.RadiativeTransfer(prob) as rt:
        y0 = rt.apply(x)
        with pytest.raises(_capi.OuranosError) as e:
            rt.set_fp64_contractions("df64_sweep_tc")
        assert e.value.code == _capi.ERR_UNSUPPORTED
        assert np.array_equal(rt.apply(x), y0)
