"""Learned preconditioner: GPU network kernels against the CPU oracle, and the
preconditioner inside FGMRES."""
import numpy as np
import pytest

from oracle import cnn_oracle

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-30))


# (24, 20, 12): 180 voxel chunks of the weight gradient on the finest level
# (23 CTAs, each reusing both staging buffers), ragged chunk counts on the
# coarser ones
@pytest.mark.parametrize("grid", [(8, 8, 8), (12, 8, 4), (24, 20, 12)])
def test_network_forward_and_gradients_match_oracle(grid):
    torch = pytest.importorskip("torch")
    from ouranos_gb300.learned import Network
    nx, ny, nz = grid
    V = nx * ny * nz
    net = Network(nx, ny, nz, seed=11)
    rng = np.random.default_rng(5)
    p = net.params()
    assert p.size == cnn_oracle.n_params()
    ng = sum(3 * c for _, c, _ in cnn_oracle.LAYERS)
    p[-ng:] += rng.uniform(-0.3, 0.3, ng)  # gates away from their (1, 0, 0) start
    net.set_params(p)
    feat = rng.standard_normal((V, cnn_oracle.FEATURES)).astype(np.float32)
    feat[:, 8:] = rng.uniform(0, 1, (V, 2))  # material channels
    target = rng.standard_normal((V, cnn_oracle.OUTPUTS)).astype(np.float32)
    fd = torch.from_numpy(feat.reshape(-1)).cuda()
    td = torch.from_numpy(target.reshape(-1)).cuda()
    out = torch.empty(V * cnn_oracle.OUTPUTS, dtype=torch.float32, device="cuda")
    net.forward(fd, out)
    loss, grads = net.gradients(fd, td)
    loss_o, grads_o, out_o = cnn_oracle.gradients(p.astype(np.float64), feat.astype(np.float64),
                                                  target.astype(np.float64), grid)
    # BF16 activations/gradients: only FP32 vs FP64 accumulation order differs
    e_out = _rel(out.cpu().numpy(), out_o.reshape(-1))
    e_loss = abs(loss - loss_o) / loss_o
    off, e_w = 0, []
    for li, (cin, cout, _) in enumerate(cnn_oracle.LAYERS):
        n = 27 * cin * cout
        e_w.append(_rel(grads[off:off + n], grads_o[off:off + n]))
        off += n
    e_g = _rel(grads[off:], grads_o[off:])
    print("network vs oracle: output %.2e loss %.2e weight grads max %.2e gate grads %.2e"
          % (e_out, e_loss, max(e_w), e_g))
    # measured on GB300: output 2.5e-3, loss 1.3e-6, weight gradients 7.5e-3,
    # gate gradients 2.7e-3 (FP32 against FP64 sums, and the rare value that
    # lands on the other side of a BF16 rounding boundary)
    assert e_out < 1e-2
    assert e_loss < 1e-4
    for li, e in enumerate(e_w):
        assert e < 2e-2, ("weights", li, e)
    assert e_g < 1e-2


def test_training_reduces_loss():
    torch = pytest.importorskip("torch")
    from ouranos_gb300.learned import Network
    net = Network(8, 8, 8, seed=3)
    rng = np.random.default_rng(9)
    feat = torch.from_numpy(rng.standard_normal(8 ** 3 * cnn_oracle.FEATURES).astype(np.float32)).cuda()
    # a continuous target: the network's output is continuous by construction
    t = cnn_oracle.project(np.tanh(rng.standard_normal((8, 8, 8, cnn_oracle.OUTPUTS))))
    target = torch.from_numpy(t.reshape(-1).astype(np.float32)).cuda()
    first = net.train_step(feat, target, 1e-3)
    for _ in range(200):
        last = net.train_step(feat, target, 1e-3)
    assert last < 0.5 * first


def test_preconditioner_features_and_target():
    """Features/targets of a known pair: e and v constant in space."""
    torch = pytest.importorskip("torch")
    import ctypes as C
    import ouranos_gb300 as og
    from ouranos_gb300 import learned
    prob = og.thick_3d(seed=2100, n=8, sn=4, block=4, width=2.0)
    L = learned._lib()
    nf, no = cnn_oracle.FEATURES, cnn_oracle.OUTPUTS
    with og.RadiativeTransfer(prob) as rt:
        e = torch.full((prob.vector_length,), 2.0, dtype=torch.float64, device="cuda")
        v = torch.full_like(e, 0.5)
        feat = torch.empty(prob.total_cells * nf, dtype=torch.float32, device="cuda")
        tgt = torch.empty(prob.total_cells * no, dtype=torch.float32, device="cuda")
        scale = C.c_double()
        assert L.ouranos_rt_pc_features(rt._h, v.data_ptr(), feat.data_ptr(), C.byref(scale)) == 0
        assert L.ouranos_rt_pc_target(rt._h, v.data_ptr(), e.data_ptr(), tgt.data_ptr()) == 0
        f = feat.cpu().numpy().reshape(-1, nf)
        assert abs(scale.value - 0.5) < 1e-12
        assert np.allclose(f[:, :8], 1.0, rtol=1e-6)
        st = prob.sigma_t[prob.material_id, 0]
        ss = prob.sigma_s[prob.material_id, 0, 0, 0]
        assert np.allclose(f[:, 8], np.log(st) / np.log(100.0), rtol=1e-6)
        assert np.allclose(f[:, 9], ss / st, rtol=1e-6)
        # K = 64; the projection leaves a constant field unchanged
        assert np.allclose(tgt.cpu().numpy(), (2.0 - 0.5) / 0.5 / 64.0, rtol=1e-6)


def test_preconditioner_nodal_features_follow_the_dofs():
    """Each cell's eight feature channels are its eight scalar-moment dofs over
    the RMS of the vector; the correction lands on the same dofs."""
    torch = pytest.importorskip("torch")
    import ctypes as C
    import ouranos_gb300 as og
    from ouranos_gb300 import learned
    prob = og.thick_3d(seed=2102, n=8, sn=4, block=4, width=2.0)
    L = learned._lib()
    nf = cnn_oracle.FEATURES
    rng = np.random.default_rng(4)
    vh = rng.standard_normal(prob.vector_length)
    with og.RadiativeTransfer(prob) as rt:
        v = torch.from_numpy(vh).cuda()
        feat = torch.empty(prob.total_cells * nf, dtype=torch.float32, device="cuda")
        scale = C.c_double()
        assert L.ouranos_rt_pc_features(rt._h, v.data_ptr(), feat.data_ptr(), C.byref(scale)) == 0
        s = np.sqrt(np.mean(vh[:prob.total_cells * 8] ** 2))
        assert abs(scale.value - s) < 1e-12 * s
        f = feat.cpu().numpy().reshape(-1, nf)
        assert np.allclose(f[:, :8], (vh[:prob.total_cells * 8] / s).reshape(-1, 8), rtol=1e-6, atol=1e-6)
        # the target is the continuity projection of (e - v) / (s K)
        eh = rng.standard_normal(prob.vector_length)
        e = torch.from_numpy(eh).cuda()
        tgt = torch.empty(prob.total_cells * 8, dtype=torch.float32, device="cuda")
        assert L.ouranos_rt_pc_target(rt._h, v.data_ptr(), e.data_ptr(), tgt.data_ptr()) == 0
        d = ((eh - vh)[:prob.total_cells * 8] / (s * 64.0)).reshape(8, 8, 8, 8)
        want = cnn_oracle.project(d).reshape(-1)
        assert _rel(tgt.cpu().numpy(), want) < 1e-6
        # a zero network output leaves the vector unchanged
        net = learned.Network(8, 8, 8, seed=9)
        net.set_params(np.zeros(net.n_params, dtype=np.float32))
        learned.install(rt, net)
        z = torch.empty_like(v)
        assert L.ouranos_rt_pc_apply(rt._h, v.data_ptr(), z.data_ptr()) == 0
        assert torch.equal(z, v)


def test_preconditioner_rejects_unsupported_meshes():
    pytest.importorskip("torch")
    import ouranos_gb300 as og
    from ouranos_gb300 import _capi, learned
    net = learned.Network(8, 8, 8, seed=2)
    with og.RadiativeTransfer(og.heterogeneous_2d(seed=5, n=16, fe_order=1, sn=4, l_max=0)) as rt:
        with pytest.raises(_capi.OuranosError) as ei:
            learned.install(rt, net)
        assert ei.value.code == _capi.ERR_UNSUPPORTED
    with og.RadiativeTransfer(og.thick_3d(seed=2103, n=12, sn=4, block=4, width=2.0)) as rt:
        with pytest.raises(_capi.OuranosError) as ei:
            learned.install(rt, net)
        assert ei.value.code == _capi.ERR_BAD_INPUT


def test_learned_fgmres_converges_and_falls_back():
    """FGMRES with an (untrained) network still converges to 1e-8: a stagnating
    preconditioned cycle hands over to the plain method."""
    pytest.importorskip("torch")
    import ouranos_gb300 as og
    from ouranos_gb300.learned import Network, install
    prob = og.thick_3d(seed=2101, n=8, sn=4, block=2, width=2.0)
    with og.RadiativeTransfer(prob) as rt:
        xg, ig, _ = rt.solve("gmres", tol=1e-8, max_it=800)
        net = Network(8, 8, 8, seed=1)
        install(rt, net)
        xl, il, _ = rt.solve("fgmres_learned", tol=1e-8, max_it=800)
    assert il["converged"] and il["residual"] < 1e-8
    assert _rel(xl, xg) < 1e-6


def test_solver_pairs_are_exact_and_the_trainer_runs():
    """The Arnoldi pairs of fgmres_pairs satisfy w = A z to the operator's
    accuracy (z is the exact error of the residual w), its FGMRES converges
    like the device solver's, and the trainer on solver-generated pairs runs
    end to end (both collection passes) on a small grid with a finite loss."""
    torch = pytest.importorskip("torch")
    import ouranos_gb300 as og
    from ouranos_gb300 import learned
    prob = og.thick_3d(seed=2102, n=8, sn=4, block=2, width=2.0)
    with og.RadiativeTransfer(prob) as rt:
        b = torch.zeros(rt.length, dtype=torch.float64, device="cuda")
        rt.rhs(out=b)
        seen = []
        x, it = learned.fgmres_pairs(rt, b, lambda v: v, lambda w, z: seen.append((w.clone(), z.clone())),
                                     max_it=400)
        assert len(seen) == it > 5
        for w, z in seen[:5]:
            assert _rel(w.cpu().numpy(), rt.apply(z).cpu().numpy()) < 1e-13
        xg, info, _ = rt.solve("gmres", tol=1e-8, max_it=800)
        assert float((b - rt.apply(x)).norm() / b.norm()) < 1e-7
        assert _rel(x.cpu().numpy(), xg) < 1e-6
    net, hist = learned.train_on_solver_pairs(n=8, maps=2, steps_per_map=6, passes=2, epochs=3, lr=1e-3,
                                              sn=4, dsa=40, log=lambda s: None)
    assert len(hist) == 6 and all(np.isfinite(hist))


def test_network_guess_of_the_diffusion_solve_converges_to_the_same_correction():
    """The network's output starts the diffusion CG: with enough CG steps the
    correction is the one a zero start reaches (the CG converges to the same
    f from any start), and FGMRES with the learned guess converges."""
    torch = pytest.importorskip("torch")
    import ouranos_gb300 as og
    from ouranos_gb300 import learned
    prob = og.thick_3d(seed=2103, n=12, sn=4, block=2, width=12 * 10.0 / 64)
    with og.RadiativeTransfer(prob) as rt:
        net = learned.Network(12, 12, 12, seed=3)
        learned.install(rt, net)
        v = torch.randn(rt.length, dtype=torch.float64, device="cuda",
                        generator=torch.Generator(device="cuda").manual_seed(4))
        rt.set_dsa(600)
        plain = rt.dsa_apply(v).cpu().numpy()
        guessed = learned.guess_precondition(rt)(v).cpu().numpy()
        assert _rel(guessed, plain) < 1e-4
        rt.set_dsa(3)
        xg, ig, _ = rt.solve("gmres", tol=1e-8, max_it=800)
        xl, il, _ = rt.solve("fgmres_learned", tol=1e-8, max_it=800, dsa=True)
    assert il["converged"] and _rel(xl, xg) < 1e-6


def test_learned_application_as_a_graph_repeats_the_first_call():
    """ouranos_rt_pc_dsa_apply runs the network's forward in the order of the
    operator's stream: eagerly on the first call with the handle's buffers,
    recorded into a CUDA graph on the second, replayed after that.  Nothing on
    this path uses atomics, so every call on the same vector gives the same
    bits; the graph reads each call's input; another handle (other feature
    buffers) records its own graph, and going back records the first anew."""
    torch = pytest.importorskip("torch")
    import ouranos_gb300 as og
    from ouranos_gb300 import learned
    prob = og.thick_3d(seed=2103, n=12, sn=4, block=2, width=12 * 10.0 / 64)
    gen = torch.Generator(device="cuda").manual_seed(8)
    net = learned.Network(12, 12, 12, seed=3)
    with og.RadiativeTransfer(prob) as rt:
        learned.install(rt, net)
        rt.set_dsa(3)
        pc = learned.guess_precondition(rt)
        v = torch.randn(rt.length, dtype=torch.float64, device="cuda", generator=gen)
        w = torch.randn(rt.length, dtype=torch.float64, device="cuda", generator=gen)
        first = pc(v).cpu().numpy()
        for _ in range(3):  # recorded, then replayed
            assert np.array_equal(pc(v).cpu().numpy(), first)
        other = pc(w).cpu().numpy()
        assert _rel(other, first) > 1e-3
        assert np.array_equal(learned.guess_precondition(rt)(w).cpu().numpy(), other)
        with og.RadiativeTransfer(prob) as rt2:
            learned.install(rt2, net)
            rt2.set_dsa(3)
            pc2 = learned.guess_precondition(rt2)
            for _ in range(3):
                assert np.array_equal(pc2(v).cpu().numpy(), first)
            learned.install(rt2, None)
        for _ in range(3):
            assert np.array_equal(pc(v).cpu().numpy(), first)
        learned.install(rt, None)
    net.close()


def test_trainer_for_the_diffusion_guess_runs():
    pytest.importorskip("torch")
    from ouranos_gb300 import learned
    net, hist = learned.train_dsa_guess(n=8, maps=2, steps_per_map=4, passes=2, epochs=2, lr=1e-3, sn=4,
                                        target_cg=40, inner_cg=2, log=lambda s: None)
    assert len(hist) == 4 and all(np.isfinite(hist))
    net.close()


def test_trained_network_gains_over_the_same_cg_budget():
    """What the trained network gains: the committed weights (trained on the
    seeded thick maps 2000-2511) start the diffusion CG of FGMRES with FP32
    sweeps on the evaluation map (seed 7000, 32^3 cells of the 64^3
    workload's width).  With the same 3 CG steps per preconditioner
    application, the learned start needs markedly fewer FGMRES iterations than
    the zero start, and both reach the same solution."""
    import os
    import ouranos_gb300 as og
    from ouranos_gb300.learned import Network, install
    weights = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "ouranos_gb300",
                           "weights", "dsa_guess_thick3d.npz")
    prob = og.thick_3d(seed=7000, n=32, sn=12, width=5.0)
    with og.RadiativeTransfer(prob) as rt:
        rt.set_dsa(3)
        x0, i0, _ = rt.solve("fgmres_mixed", tol=1e-8, max_it=1000, dsa=True)
        net = Network.load(weights, (32, 32, 32))
        install(rt, net)
        x1, i1, _ = rt.solve("fgmres_learned", tol=1e-8, max_it=1000, dsa=True)
        install(rt, None)
        net.close()
    print("iterations without / with the network:", i0["iterations"], i1["iterations"])
    assert i0["converged"] and i1["converged"]
    assert i1["iterations"] <= 0.85 * i0["iterations"]
    assert _rel(x1, x0) < 1e-6
