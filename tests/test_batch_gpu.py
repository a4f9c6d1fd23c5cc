"""Many problems in one persistent launch: the batched Apply against the
single-problem operator (same task code: bit-identical) and the oracle, graph
replays, the batched solve, the autotuner."""
import numpy as np
import pytest

from helpers import rel_err
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def _problems(count=6, seed=31):
    import ouranos_gb300 as og
    # small uneven mix: sides, DG orders, quadratures and P1 scattering vary
    return og.batch_2d(seed=seed, count=count, sides=(8, 16, 24, 40), orders=(1, 2), sns=(4, 8))


def _singles(problems, x_slices, precision="fp64"):
    """Single-problem Applies with the batch's arithmetic: its FP64 sweep is the
    FP64 kernel with double-float contractions (mode 'df64')."""
    import ouranos_gb300 as og
    out = []
    for p, x in zip(problems, x_slices):
        with og.RadiativeTransfer(p, precision=precision) as rt:
            rt.set_fp64_contractions("df64")
            out.append(rt.apply(np.ascontiguousarray(x)))
    return out


def test_batched_apply_is_bit_identical_to_single_problems():
    import ouranos_gb300 as og
    probs = _problems()
    with og.Batch(probs) as b:
        x = np.random.default_rng(1).standard_normal(b.length)
        y = b.apply(x)
        for ys, yb in zip(_singles(probs, b.slices(x)), b.slices(y)):
            assert np.array_equal(ys, yb)
        y32 = b.apply(x, precision="fp32")
        for ys, yb in zip(_singles(probs, b.slices(x), "fp32"), b.slices(y32)):
            assert np.array_equal(ys, yb)


def test_batched_apply_matches_the_oracle():
    import ouranos_gb300 as og
    probs = _problems(count=4, seed=33)
    with og.Batch(probs) as b:
        x = np.random.default_rng(2).standard_normal(b.length)
        y = b.apply(x)
        for p, xs, ys in zip(probs, b.slices(x), b.slices(y)):
            ref = po.OracleProblem(p.arrays()).apply(np.ascontiguousarray(xs))
            assert rel_err(ys, ref) < 1e-12


def test_graph_replays_equal_eager_and_no_graph_runs():
    import ouranos_gb300 as og
    probs = _problems(count=5, seed=35)
    with og.Batch(probs) as b:
        x = np.random.default_rng(3).standard_normal(b.length)
        runs = [b.apply(x) for _ in range(4)]  # eager, capture, replay, replay
        _, launches = b.stats()
        assert launches >= 3
        for r in runs[1:]:
            assert np.array_equal(r, runs[0])
        b.set_graphs(False)
        assert np.array_equal(b.apply(x), runs[0])


def test_batched_rhs_matches_single_problems():
    import ouranos_gb300 as og
    probs = _problems(count=4, seed=37)
    with og.Batch(probs) as b:
        r = b.rhs()
        for p, rb in zip(probs, b.slices(r)):
            with og.RadiativeTransfer(p) as rt:
                rt.set_fp64_contractions("df64")
                assert np.array_equal(rt.rhs(), rb)


def test_batched_solve_matches_single_problem_gmres():
    import ouranos_gb300 as og
    probs = _problems(count=5, seed=39)
    with og.Batch(probs) as b:
        x, infos = b.solve(inner="fp32", tol=1e-8, max_it=1500)
        x64, infos64 = b.solve(inner="fp64", tol=1e-8, max_it=1500)
        for p, xs, info in zip(probs, b.slices(x), infos):
            assert info["converged"] and info["residual"] < 1e-8
            with og.RadiativeTransfer(p) as rt:
                xr, ir, _ = rt.solve("gmres", tol=1e-10, max_it=3000)
            assert rel_err(xs, xr) < 1e-6
        for xs, xd in zip(b.slices(x), b.slices(x64)):
            assert rel_err(xs, xd) < 1e-6
        assert all(i["converged"] for i in infos64)


def test_batched_solve_with_dsa():
    """FGMRES with every problem's diffusion correction (Q1 and Q2 problems,
    P1 scattering): the same solutions as single-problem FP64 GMRES, in no
    more iterations than the plain batched solve for any problem and far
    fewer in total."""
    import ouranos_gb300 as og
    probs = _problems(count=5, seed=39)
    with og.Batch(probs) as b:
        x0, i0 = b.solve(inner="fp32", tol=1e-8, max_it=1500)
        b.set_dsa(15)
        x, infos = b.solve(inner="fp32", tol=1e-8, max_it=1500, dsa=True)
        for p, xs, info in zip(probs, b.slices(x), infos):
            assert info["converged"] and info["residual"] < 1e-8
            with og.RadiativeTransfer(p) as rt:
                xr, _, _ = rt.solve("gmres", tol=1e-10, max_it=3000)
            assert rel_err(xs, xr) < 1e-6
        assert sum(i["iterations"] for i in infos) < sum(i["iterations"] for i in i0)


@pytest.mark.parametrize("steps", [1, 15])
def test_batched_dsa_matches_each_problems_own(steps):
    """All members' diffusion corrections in one cooperative launch (blocks
    split over the problems by vertex count) against each problem's own
    single-problem launch: the same CG in FP32 with FP64 scalars, only the
    order of the partial sums differs."""
    import ouranos_gb300 as og
    probs = _problems(count=5, seed=47)
    with og.Batch(probs) as b:
        b.set_dsa(steps)
        x = np.random.default_rng(6).standard_normal(b.length)
        z = b.dsa_apply(x)
        for p, xs, zs in zip(probs, b.slices(x), b.slices(z)):
            with og.RadiativeTransfer(p) as rt:
                rt.set_dsa(steps)
                zr = rt.dsa_apply(np.ascontiguousarray(xs))
            # the correction itself (z - x), relative to its own size
            assert rel_err(zs - xs, zr - xs) < 1e-4
            n0 = p.total_cells * p.dofs_per_cell
            assert np.array_equal(zs[n0:], xs[n0:])  # higher moments pass unchanged


def test_autotune_keeps_results_and_reports_tilings():
    import ouranos_gb300 as og
    probs = _problems(count=4, seed=41)
    with og.Batch(probs) as b:
        x = np.random.default_rng(4).standard_normal(b.length)
        before = b.apply(x)
        t = b.autotune(reps=2)
        assert t.shape == (4, 3)
        for p, (cx, cy, kd) in zip(probs, t):
            # 32 lanes: one per cell, or two per cell (16 cells) for cells of 9+ dofs
            assert cx * cy * kd == 32 or (cx * cy * kd == 16 and p.dofs_per_cell >= 9)
        after = b.apply(x)
        for p, xs, ys in zip(probs, b.slices(x), b.slices(after)):
            ref = po.OracleProblem(p.arrays()).apply(np.ascontiguousarray(xs))
            assert rel_err(ys, ref) < 1e-12
        assert rel_err(after, before) < 1e-13


def test_device_vectors_through_the_batch():
    torch = pytest.importorskip("torch")
    import ouranos_gb300 as og
    probs = _problems(count=3, seed=43)
    with og.Batch(probs) as b:
        xh = np.random.default_rng(5).standard_normal(b.length)
        yh = b.apply(xh)
        xd = torch.from_numpy(xh).cuda()
        yd = b.apply(xd)
        assert np.array_equal(yd.cpu().numpy(), yh)
