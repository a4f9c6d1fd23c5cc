"""The network oracle's analytic gradients against central finite differences
(exact arithmetic: BF16 rounding switched off for the check)."""
import numpy as np
import pytest

from oracle import cnn_oracle


def test_oracle_gradients_match_finite_differences(monkeypatch):
    monkeypatch.setattr(cnn_oracle, "bf16", lambda x: np.asarray(x, dtype=np.float64))
    grid = (4, 4, 4)
    V = 64
    rng = np.random.default_rng(0)
    n_params = cnn_oracle.n_params()
    p = rng.standard_normal(n_params) * 0.2
    feat = rng.standard_normal((V, cnn_oracle.FEATURES))
    tgt = rng.standard_normal((V, cnn_oracle.OUTPUTS))
    loss, g, out = cnn_oracle.gradients(p, feat, tgt, grid)
    assert out.shape == (V, cnn_oracle.OUTPUTS)
    assert loss == pytest.approx(np.mean((out - tgt) ** 2))
    # every layer's weights and some gate coefficients are sampled
    offs = np.cumsum([0] + [27 * a * b for a, b, _ in cnn_oracle.LAYERS])
    idx = [int(rng.integers(offs[i], offs[i + 1])) for i in range(len(cnn_oracle.LAYERS))]
    idx += list(rng.choice(np.arange(offs[-1], n_params), 4, replace=False))
    h = 1e-6
    for i in idx:
        pp = p.copy()
        pp[i] += h
        lp = cnn_oracle.gradients(pp, feat, tgt, grid)[0]
        pp[i] -= 2 * h
        lm = cnn_oracle.gradients(pp, feat, tgt, grid)[0]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * max(abs(fd), 1e-3), (i, fd, g[i])


def test_continuity_projection_is_a_symmetric_projection():
    rng = np.random.default_rng(1)
    a = rng.standard_normal((3, 4, 5, 8))
    b = rng.standard_normal((3, 4, 5, 8))
    sa = cnn_oracle.project(a)
    assert np.allclose(cnn_oracle.project(sa), sa)
    assert np.isclose(np.sum(sa * b), np.sum(a * cnn_oracle.project(b)))
    # a continuous field (nodal values of one vertex field) is left unchanged
    vert = rng.standard_normal((4, 5, 6))
    c = np.empty_like(a)
    for k in range(8):
        x, y, z = k & 1, (k >> 1) & 1, k >> 2
        c[..., k] = vert[z:z + 3, y:y + 4, x:x + 5]
    assert np.allclose(cnn_oracle.project(c), c)


def test_network_is_linear_in_the_residual(monkeypatch):
    """For fixed materials the network output is linear in the residual
    channels (no bias, no ReLU; gates depend on the materials only)."""
    monkeypatch.setattr(cnn_oracle, "bf16", lambda x: np.asarray(x, dtype=np.float64))
    grid = (4, 4, 4)
    rng = np.random.default_rng(2)
    p = rng.standard_normal(cnn_oracle.n_params()) * 0.3
    mats = rng.uniform(0, 1, (64, 2))
    # dyadic inputs: exact in FP32, so the only inexactness is the check's own
    f1 = np.concatenate([rng.integers(-64, 64, (64, 8)) / 16.0, mats], axis=1)
    f2 = np.concatenate([rng.integers(-64, 64, (64, 8)) / 16.0, mats], axis=1)
    f3 = np.concatenate([2.0 * f1[:, :8] - 3.0 * f2[:, :8], mats], axis=1)
    y1 = cnn_oracle.forward(p, f1, grid)[0]
    y2 = cnn_oracle.forward(p, f2, grid)[0]
    y3 = cnn_oracle.forward(p, f3, grid)[0]
    assert np.allclose(y3, 2.0 * y1 - 3.0 * y2, rtol=1e-10, atol=1e-12 * np.abs(y3).max())
