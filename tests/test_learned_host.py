"""Host logic of the learned preconditioner's training-pair driver, on the CPU:
FGMRES with a fake operator (a dense nonsymmetric matrix) hands out exact
pairs and converges to the direct solution."""
import numpy as np
import pytest


class _DenseOperator:
    """A stand-in for the transport operator: apply(x) = A x."""

    def __init__(self, A, torch):
        self.A = torch.from_numpy(A)

    def apply(self, x):
        return self.A @ x


@pytest.mark.parametrize("restart", [30, 7])
def test_fgmres_pairs_are_exact_and_converge(restart):
    torch = pytest.importorskip("torch")
    from ouranos_gb300.learned import fgmres_pairs
    rng = np.random.default_rng(3)
    n = 120
    A = np.eye(n) + 0.3 * rng.standard_normal((n, n)) / np.sqrt(n)
    b = rng.standard_normal(n)
    op = _DenseOperator(A, torch)
    seen = []
    x, it = fgmres_pairs(op, torch.from_numpy(b), lambda v: v, lambda w, z: seen.append((w.clone(), z.clone())),
                         m=restart, max_it=500, tol=1e-10)
    assert len(seen) == it > 0
    for w, z in seen:  # w = A z exactly: z is the true error of the residual w
        assert np.allclose(w.numpy(), A @ z.numpy(), rtol=0, atol=1e-13)
    xs = np.linalg.solve(A, b)
    assert np.linalg.norm(x.numpy() - xs) / np.linalg.norm(xs) < 1e-8


def test_fgmres_pairs_with_a_preconditioner_needs_fewer_steps():
    """A right preconditioner close to A^-1 (the direct inverse of A's
    diagonal-dominant part) cuts the steps; the recorded z are P(v)."""
    torch = pytest.importorskip("torch")
    from ouranos_gb300.learned import fgmres_pairs
    rng = np.random.default_rng(5)
    n = 100
    D = np.diag(np.linspace(1.0, 1e3, n))
    A = D + 0.05 * rng.standard_normal((n, n))
    b = rng.standard_normal(n)
    op = _DenseOperator(A, torch)
    Dinv = torch.from_numpy(np.diag(1.0 / np.diag(D)))
    _, it0 = fgmres_pairs(op, torch.from_numpy(b), lambda v: v, lambda w, z: None, m=30, max_it=400, tol=1e-10)
    zs = []
    x, it1 = fgmres_pairs(op, torch.from_numpy(b), lambda v: Dinv @ v, lambda w, z: zs.append(z), m=30,
                          max_it=400, tol=1e-10)
    assert it1 < it0 / 2
    xs = np.linalg.solve(A, b)
    assert np.linalg.norm(x.numpy() - xs) / np.linalg.norm(xs) < 1e-8
