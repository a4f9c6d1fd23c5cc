"""Diffusion synthetic acceleration, CPU side: the restated diffusion system's
analytic properties, and its effect on the oracle's Krylov solve."""
import numpy as np
import pytest

import ouranos_gb300 as og
from oracle import dsa_oracle as do
from oracle import pyoracle as po


def homogeneous(dim, n, sigma_t, sigma_s, bc, sn=4, l_max=0, width=2.0, fe_order=1):
    quad = og.build_quadrature("GLC" if dim == 3 else "LS", sn, l_max, dim=dim)
    p = og.uniform_problem(dim, fe_order, (n,) * dim, (0.0,) * dim, (width,) * dim, quad, sigma_t, sigma_s,
                           1.0, bc=bc)
    return p


@pytest.mark.parametrize("p,dim", [(1, 2), (2, 2), (3, 2), (1, 3), (2, 3)])
def test_cell_tables(p, dim):
    """The mixed mass matrix and the nodal interpolation of the vertex hat
    functions: Q1 gives the Q1 mass matrix and the identity; the hat
    functions sum to one at every node and each integrates to vol / 2^dim."""
    vol = 0.37
    mix, ipl = do.q1_qp_tables(p, dim, vol)
    nc, n = 2 ** dim, (p + 1) ** dim
    assert mix.shape == (nc, n) and ipl.shape == (n, nc)
    assert np.allclose(ipl.sum(axis=1), 1.0, atol=1e-14)
    assert np.allclose(mix.sum(axis=1), vol / nc, rtol=1e-13)
    if p == 1:
        m1 = np.array([[1 / 3, 1 / 6], [1 / 6, 1 / 3]])
        ref = m1 if dim == 1 else np.kron(m1, m1) if dim == 2 else np.kron(np.kron(m1, m1), m1)
        assert np.allclose(mix, vol * ref, atol=1e-15)
        assert np.allclose(ipl, np.eye(nc))


@pytest.mark.parametrize("dim,order", [(2, 1), (3, 1), (2, 2), (3, 2), (2, 4)])
def test_flat_residual_in_an_infinite_medium(dim, order):
    """Reflective on every side, homogeneous: a flat scalar-moment residual v has
    the flat correction sigma_s/sigma_a v, so P v = v / (1 - c) -- the exact
    inverse of source iteration's error operator for that mode -- for every
    DG order (the hat functions sum to one).  The time-step term adds 1/(v dt)
    to sigma_t (so to sigma_a)."""
    n = 5
    for inv_vdt in (0.0, 0.5):
        p = homogeneous(dim, n, 1.0, 0.9, (3,) * 6, fe_order=order)
        d = do.Diffusion(p, inv_vdt=inv_vdt)
        nodes = (order + 1) ** dim
        v = np.zeros(p.quad.n_mom * n ** dim * nodes)
        v[: n ** dim * nodes] = 1.0
        expect = 1.0 + 0.9 / (0.1 + inv_vdt)
        z = d.apply(v)
        assert np.allclose(z[: n ** dim * nodes], expect, rtol=1e-12)
        z = d.apply(v, k=200)
        assert np.allclose(z[: n ** dim * nodes], expect, rtol=1e-8)


@pytest.mark.parametrize("dim", [2, 3])
def test_system_is_spd_and_balanced(dim):
    """C is symmetric positive definite; summed over all entries it is the
    absorption sigma_a |domain| plus the Marshak term |vacuum boundary| / 2
    (the stiffness part annihilates constants)."""
    n, width = 4, 2.0
    bc = (0, 3, 0, 3, 0, 3)
    p = homogeneous(dim, n, 2.0, 1.5, bc, width=width)
    d = do.Diffusion(p)
    C = d.C.toarray()
    assert np.allclose(C, C.T, atol=1e-14)
    assert np.linalg.eigvalsh(C).min() > 0
    vac_area = dim * width ** (dim - 1)  # one vacuum side per axis
    assert C.sum() == pytest.approx(0.5 * width ** dim + 0.5 * vac_area, rel=1e-12)


def test_cg_converges_to_the_direct_solve():
    p = og.thick_3d(seed=7000, n=8, sn=4, width=1.25)
    d = do.Diffusion(p)
    rng = np.random.default_rng(3)
    v = rng.standard_normal(p.quad.n_mom * 8 ** 3 * 8)
    exact = d.apply(v)
    assert np.linalg.norm(d.apply(v, k=300) - exact) / np.linalg.norm(exact) < 1e-8


def fgmres(A, b, M, tol=1e-8, m=30, max_it=600):
    """Right-preconditioned restarted FGMRES (modified Gram-Schmidt, dense
    least squares); returns (x, iterations)."""
    x = np.zeros_like(b)
    nb = np.linalg.norm(b)
    it = 0
    while it < max_it:
        r = b - A(x)
        beta = np.linalg.norm(r)
        if beta / nb < tol:
            break
        V, Z, H = [r / beta], [], np.zeros((m + 1, m))
        for j in range(m):
            z = M(V[j])
            Z.append(z)
            w = A(z)
            it += 1
            for i in range(j + 1):
                H[i, j] = w @ V[i]
                w = w - H[i, j] * V[i]
            H[j + 1, j] = np.linalg.norm(w)
            V.append(w / H[j + 1, j])
            e1 = np.zeros(j + 2)
            e1[0] = beta
            y = np.linalg.lstsq(H[: j + 2, : j + 1], e1, rcond=None)[0]
            res = np.linalg.norm(H[: j + 2, : j + 1] @ y - e1)
            if res / nb < tol:
                break
        x = x + np.array(Z).T @ y
        if res / nb < tol:
            break
    return x, it


def test_dsa_cuts_krylov_iterations_on_thick_diffusive_cells():
    """8^3 cells of the thick diffusive map (GLC S4, cells 0.16 wide): the
    unpreconditioned FGMRES(30) of the oracle operator needs ~165 iterations
    to 1e-8; with the diffusion correction (5 CG steps) it needs under 35, and
    both reach the same solution."""
    p = og.thick_3d(seed=7000, n=8, sn=4, width=1.25)
    P = po.OracleProblem(p.arrays())
    d = do.Diffusion(p)
    A = lambda x: P.apply(x, threads=4)
    b = P.rhs(threads=4)
    x0, it0 = fgmres(A, b, lambda v: v)
    x1, it1 = fgmres(A, b, lambda v: d.apply(v, k=5))
    assert it0 > 120
    assert it1 < 35
    assert np.linalg.norm(x1 - x0) / np.linalg.norm(x0) < 1e-6
