"""The FP32 path's direction-axis contractions on the tensor cores
(tcgen05, three-part BF16 splits with FP32 accumulation) through the C-ABI:
against the oracle at the FP32 sweep's tolerance and against the same Apply
with the contractions on the CUDA cores."""
import numpy as np
import pytest

from helpers import rel_err
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

TOL32 = 2e-6   # the FP32 sweep against the FP64 oracle (small cases)


def _cases():
    import ouranos_gb300 as og

    def aniso3d(l_max):
        q = og.build_quadrature("GLC", 6, l_max, dim=3)
        p = og.uniform_problem(3, 1, (6, 5, 7), (0, 0, 0), (2.0, 2.0, 2.0), q, 2.0, 1.5, 1.0)
        ss = np.zeros((1, 1, 1, l_max + 1))
        ss[0, 0, 0] = [1.5 * 0.5 ** l for l in range(l_max + 1)]
        p.sigma_s = ss
        return p
    return {
        "2d-q2-ls16-p3": lambda: og.heterogeneous_2d(seed=71, n=24, fe_order=2, sn=16, l_max=3, blocks=4),
        "2d-q1-ls8-p3-ragged": lambda: og.heterogeneous_2d(seed=72, n=23, fe_order=1, sn=8, l_max=3, blocks=3),
        "2d-q3-ls4-p1": lambda: og.heterogeneous_2d(seed=73, n=9, fe_order=3, sn=4, l_max=1, blocks=3),
        "3d-q1-glc12-p0": lambda: og.thick_3d(seed=2071, n=8, sn=12, block=2, width=2.0),
        "3d-q1-glc6-p1": lambda: aniso3d(1),
        "3d-q1-glc6-p3": lambda: aniso3d(3),
    }


CASES = _cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_tensor_contractions_apply(name):
    import ouranos_gb300 as og
    prob = CASES[name]()
    x = np.random.default_rng(7).standard_normal(prob.vector_length)
    O = po.OracleProblem(prob.arrays())
    ref = O.apply(x)
    ref_rhs = O.rhs()
    with og.RadiativeTransfer(prob, precision="fp32") as rt:
        y_cc = rt.apply(x)
        rt.set_fp32_contractions("tensor")
        y_tc = rt.apply(x)
        r_tc = rt.rhs()
    assert rel_err(y_tc, ref) < TOL32, rel_err(y_tc, ref)
    assert rel_err(r_tc, ref_rhs) < TOL32
    # the two FP32 forms differ by FP32 rounding only
    assert rel_err(y_tc, y_cc) < 1e-6


def test_tensor_contractions_host_vectors_in_ranges():
    """The host-vector Apply runs the contractions on cell ranges (offset
    pointers, rows n_dofs apart): identical to the device-vector Apply."""
    torch = pytest.importorskip("torch")
    import ouranos_gb300 as og
    prob = og.heterogeneous_2d(seed=74, n=37, fe_order=2, sn=8, l_max=3, blocks=4)
    with og.RadiativeTransfer(prob, precision="fp32") as rt:
        rt.set_fp32_contractions("tensor")
        x = torch.from_numpy(np.random.default_rng(8).standard_normal(prob.vector_length)).cuda()
        yd = torch.empty_like(x)
        rt.Apply(x, yd)
        xh = x.cpu().pin_memory()
        yh = torch.empty_like(xh).pin_memory()
        rt.Apply(xh, yh)
        assert torch.equal(yh, yd.cpu())


def test_tensor_contractions_full_size_workload():
    """The benchmark workload (256^2 Q2, LS S16, P3) in FP32 with the
    contractions on the tensor cores against the FP64 oracle."""
    import os
    import ouranos_gb300 as og
    prob = og.heterogeneous_2d(seed=1001, n=256, fe_order=2, sn=16, l_max=3, blocks=8)
    x = np.random.default_rng(1001).standard_normal(prob.vector_length)
    ref = po.OracleProblem(prob.arrays(), order="cartesian").apply(x, threads=os.cpu_count() or 1)
    with og.RadiativeTransfer(prob, precision="fp32") as rt:
        rt.set_fp32_contractions("tensor")
        y = rt.apply(x)
    assert rel_err(y, ref) < 1e-5


def test_tensor_contractions_limits():
    import ouranos_gb300 as og
    from ouranos_gb300 import _capi
    q = og.build_quadrature("GLC", 16, 0, dim=3)  # 288 directions
    prob = og.uniform_problem(3, 1, (2, 2, 2), (0, 0, 0), (1.0, 1.0, 1.0), q, 1.0, 0.5, 1.0)
    with og.RadiativeTransfer(prob, precision="fp32") as rt:
        with pytest.raises(_capi.OuranosError) as e:
            rt.set_fp32_contractions("tensor")
        assert e.value.code == _capi.ERR_UNSUPPORTED
