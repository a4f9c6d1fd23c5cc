"""GPU parity at the full sizes of the benchmark workloads, through the C-ABI,
against the oracle on the host's cores.

The small cases of test_sweep_gpu.py cover every code path; these run the
regimes the benchmark times: hundreds of cell diagonals, more warp tasks than
resident warps (several waves of tickets), S16 with Q2 and P3, GLC S12 in
3-D, the shifted operator of a 128^3 time step, and both classes of the
batched uneven workload.  The oracle sweeps in its cartesian order here
(identical task values, no task graph: at 10^8 tasks the graph alone would
need tens of GB of host memory).
"""
import os

import numpy as np
import pytest

from helpers import rel_err
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

# the parity bar of the FP64 sweep (norm-wise relative, whole flux-moment vector)
TOL64 = 1e-12
# the FP32 sweep against the FP64 oracle at these sizes: single-precision
# rounding along up to 511 dependent cell diagonals
TOL32 = 1e-5
THREADS = os.cpu_count() or 1


def _oracle_apply(prob, x, shift=0.0):
    spec = prob.arrays()
    if shift:
        # the implicit-Euler operator: sigma_t + 1/(v dt), scattering unchanged
        spec = dict(spec, sigma_t=prob.sigma_t + shift)
    return po.OracleProblem(spec, order="cartesian").apply(x, threads=THREADS)


def test_small_homogeneous_source_iteration():
    """32 x 32 DG Q1, LS S8, sigma_t = 1, sigma_s = 0.5, q = 1, vacuum: source
    iteration to a 1e-10 relative change (src/ouranos.cc:72-95 written as
    intended) on the GPU and in the oracle -- the same iterates, so the same
    count and the same flux."""
    import ouranos_gb300 as og
    prob = og.config_small(n=32, sn=8)
    O = po.OracleProblem(prob.arrays())
    xo, it_o, _ = O.solve("si", tol=1e-10, max_it=500, threads=THREADS)
    with og.RadiativeTransfer(prob) as rt:
        x, info, _ = rt.solve("si", tol=1e-10, max_it=500)
    assert info["converged"]
    assert abs(info["iterations"] - it_o) <= 1
    n0 = prob.n_dofs
    assert rel_err(x[:n0], xo[:n0]) < 1e-10


def test_2d_heterogeneous_q2_s16_p3_apply_every_arithmetic():
    """256 x 256 DG Q2, LS S16 (144 directions), P3 (10 moments), 8 x 8
    seeded blocks: the benchmark's Apply in the default double-float sweep,
    the same with the contractions on the tensor cores (exact digit
    products), the double-float contractions with an FP64 sweep, native FP64,
    and FP32."""
    import ouranos_gb300 as og
    prob = og.heterogeneous_2d(seed=1001, n=256, fe_order=2, sn=16, l_max=3, blocks=8)
    x = np.random.default_rng(1001).standard_normal(prob.vector_length)
    ref = _oracle_apply(prob, x)
    with og.RadiativeTransfer(prob) as rt:
        assert rt.tiling() == (16, 1, 1)
        errs = {}
        for mode in ("df64_sweep", "df64_sweep_tc", "df64", "native"):
            rt.set_fp64_contractions(mode)
            errs[mode] = rel_err(rt.apply(x), ref)
        rt.set_precision("fp32")
        errs["fp32"] = rel_err(rt.apply(x), ref)
    print(errs)
    for mode in ("df64_sweep", "df64_sweep_tc", "df64", "native"):
        assert errs[mode] < TOL64, (mode, errs)
    assert errs["fp32"] < TOL32, errs


def test_3d_thick_glc12_apply():
    """64^3 DG Q1, GLC S12 (168 directions, 8 octants), the thick map of the
    time-to-solution runs (seed 7000): default FP64 arithmetic, the
    tensor-core contractions (four chunks of directions), and FP32."""
    import ouranos_gb300 as og
    prob = og.thick_3d(seed=7000, n=64, sn=12)
    x = np.random.default_rng(7000).standard_normal(prob.vector_length)
    ref = _oracle_apply(prob, x)
    with og.RadiativeTransfer(prob) as rt:
        e64 = rel_err(rt.apply(x), ref)
        rt.set_fp64_contractions("df64_sweep_tc")
        etc = rel_err(rt.apply(x), ref)
        rt.set_precision("fp32")
        e32 = rel_err(rt.apply(x), ref)
    print(e64, etc, e32)
    assert e64 < TOL64
    assert etc < TOL64
    assert e32 < TOL32


def test_3d_time_step_operator_128cubed():
    """128^3 DG Q1, LS S8 (80 directions), two-material map: the Apply of an
    implicit-Euler step, sigma_t shifted by 1/(v dt) = 0.5 (16.8 M dofs,
    168 M cell-direction solves)."""
    import ouranos_gb300 as og
    prob = og.time_dependent_3d(seed=4000, n=128)
    x = np.random.default_rng(4000).standard_normal(prob.vector_length)
    ref = _oracle_apply(prob, x, shift=prob.meta["inv_vdt"])
    with og.RadiativeTransfer(prob) as rt:
        rt.set_time_step(prob.meta["inv_vdt"])
        y = rt.apply(x)
    assert rel_err(y, ref) < TOL64


def test_batched_uneven_workload_one_member_per_class():
    """The 64 uneven 2-D problems in one batch (sides 32..512, Q1 or Q2, LS
    S4..S16, P1): one batched Apply in FP64 and one in FP32; the largest
    member of each sweep class (Q1 with moments fused into the sweep, Q2 with
    the expanded source) against the oracle."""
    import ouranos_gb300 as og
    probs = og.batch_2d(seed=3000, count=64)
    picks = {}
    for i, p in enumerate(probs):
        k = p.fe_order
        if k not in picks or p.total_cells * p.quad.n_dir > probs[picks[k]].total_cells * probs[picks[k]].quad.n_dir:
            picks[k] = i
    assert sorted(picks) == [1, 2]
    with og.Batch(probs) as b:
        x = np.random.default_rng(3000).standard_normal(b.length)
        y64 = b.apply(x, "fp64")
        y32 = b.apply(x, "fp32")
        xs, s64, s32 = b.slices(x), b.slices(y64), b.slices(y32)
    for k, i in sorted(picks.items()):
        ref = _oracle_apply(probs[i], xs[i])
        assert rel_err(s64[i], ref) < TOL64, probs[i].name
        assert rel_err(s32[i], ref) < TOL32, probs[i].name
