"""CPU restatement of the diffusion synthetic acceleration (test infrastructure).

The preconditioner has no counterpart in the reference (its Krylov solves run
unpreconditioned and its source iteration plain: src/ouranos.cc:72-95,
160-171), so this restates the definition the GPU implements and is pinned by
analytic properties in the tests, not by reference outputs:

    P v = v + f,   (-div D grad + sigma_a) f = sigma_s0 v_0

with f continuous Q1 on the mesh vertices (Galerkin, exact element
integrals), the Marshak term (1/2) integral f w on the faces of vacuum and
inflow boundaries and none on reflective ones, D = 1/(3 (sigma_t' -
sigma_s1)), sigma_a = sigma_t' - sigma_s0, sigma_t' = sigma_t + 1/(v dt), and
f (interpolated at the cell's DG Q_p nodes) added to the scalar moment's
nodal values; for Q_p cells the right-hand side takes the residual through
the mixed mass matrix of the vertex hat functions and the Q_p basis.  `apply`
solves the diffusion
system by k steps of Jacobi-preconditioned conjugate gradients (k = None: a
direct solve), in FP64.

Layout conventions: cells lexicographic (x fastest), DG Q_p nodes of a cell
on the equidistant points j/p, x fastest; corner index a + 2 b (+ 4 c) for
the corner offsets (a, b, c);
vertices lexicographic on the (nx+1) x (ny+1) (x (nz+1)) grid.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl

BC_REFLECTIVE = 3


def cell_coefficients(problem, group=0, inv_vdt=0.0):
    """Per-cell (D, sigma_a, sigma_s0)."""
    mat = np.asarray(problem.material_id)
    st = problem.sigma_t[mat, group] + inv_vdt
    L = problem.sigma_s.shape[-1] - 1
    s0 = problem.sigma_s[mat, group, group, 0]
    s1 = problem.sigma_s[mat, group, group, 1] if L >= 1 else np.zeros_like(s0)
    tr = st - s1
    tr = np.where(tr > 1e-8, tr, np.where(st > 1e-8, st, 1e-8))
    sa = np.maximum(st - s0, 0.0)
    return 1.0 / (3.0 * tr), sa, s0


def q1_qp_tables(p, dim, vol):
    """Mixed mass matrix [corner][node] (vertex hat functions against the DG
    Q_p basis on the equidistant nodes j/p, cell measure vol) and the hat
    functions' values at the nodes [node][corner]; tensor products of 1-D
    factors, x fastest."""
    gx, gw = np.polynomial.legendre.leggauss(p + 2)
    gx, gw = 0.5 * (gx + 1.0), 0.5 * gw
    nodes1 = np.arange(p + 1) / p

    def lag(k, x):
        v = np.ones_like(x)
        for j in range(p + 1):
            if j != k:
                v = v * (x - nodes1[j]) / (nodes1[k] - nodes1[j])
        return v

    hat = [lambda x: 1.0 - x, lambda x: x]
    m1 = np.array([[np.sum(gw * hat[a](gx) * lag(k, gx)) for k in range(p + 1)] for a in range(2)])
    i1 = np.array([[hat[a](nodes1[k]) for a in range(2)] for k in range(p + 1)])
    nc, p1 = 2 ** dim, p + 1
    n = p1 ** dim
    mix = np.zeros((nc, n))
    ipl = np.zeros((n, nc))
    for cr in range(nc):
        for j in range(n):
            mm, ip = vol, 1.0
            for ax in range(dim):
                bit = (cr >> ax) & 1
                comp = (j // p1 ** ax) % p1
                mm *= m1[bit, comp]
                ip *= i1[comp, bit]
            mix[cr, j] = mm
            ipl[j, cr] = ip
    return mix, ipl


class Diffusion:
    """The assembled vertex system of one problem."""

    def __init__(self, problem, group=0, inv_vdt=0.0):
        dim = problem.dim
        n = list(problem.n_cells)
        h = [(problem.upper[a] - problem.lower[a]) / n[a] for a in range(dim)]
        self.dim, self.n = dim, n
        nv = [k + 1 for k in n]
        self.nv = nv
        nodes = 2 ** dim  # corners of a cell
        self.corners = nodes
        self.nodes = (problem.fe_order + 1) ** dim  # DG nodes of a cell
        D, sa, s0 = cell_coefficients(problem, group, inv_vdt)
        self.s0 = s0
        vol = float(np.prod(h))
        m1 = np.array([[1 / 3, 1 / 6], [1 / 6, 1 / 3]])
        k1 = np.array([[1.0, -1.0], [-1.0, 1.0]])

        def kron(factors):  # factors[a] for axis a; axis 0 (x) is the fastest index
            out = np.ones((1, 1))
            for f in reversed(factors):
                out = np.kron(out, f)
            return out

        self.Mref = vol * kron([m1] * dim)
        self.mix, self.ipl = q1_qp_tables(problem.fe_order, dim, vol)
        Kref = np.zeros((nodes, nodes))
        for a in range(dim):
            fac = [m1] * dim
            fac[a] = k1
            Kref += (vol / h[a] ** 2) * kron(fac)
        # vertex ids of every cell's corners
        idx = np.indices(n[::-1]).reshape(dim, -1)[::-1]  # idx[a] = cell coordinate on axis a
        vid = np.zeros((idx.shape[1], nodes), dtype=np.int64)
        for k in range(nodes):
            off = [(k >> a) & 1 for a in range(dim)]
            v = np.zeros(idx.shape[1], dtype=np.int64)
            mul = 1
            for a in range(dim):
                v += (idx[a] + off[a]) * mul
                mul *= nv[a]
            vid[:, k] = v
        self.vid = vid
        NV = int(np.prod(nv))
        self.NV = NV
        vals = D[:, None, None] * Kref[None] + sa[:, None, None] * self.Mref[None]
        rows = np.repeat(vid, nodes, axis=1).ravel()
        cols = np.tile(vid, (1, nodes)).ravel()
        C = sp.coo_matrix((vals.ravel(), (rows, cols)), shape=(NV, NV)).tocsr()
        # Marshak boundary terms on non-reflective sides
        bc = list(problem.bc_type) + [0] * 6
        grid = np.arange(NV).reshape(nv[::-1])  # [z][y][x] or [y][x]
        fb = []
        for a in range(dim):
            others = [b for b in range(dim) if b != a]
            fmass = 0.5 * (vol / h[a]) * kron([m1] * (dim - 1))
            for side in (0, 1):
                if bc[2 * a + side] == BC_REFLECTIVE:
                    continue
                sl = [slice(None)] * dim
                sl[dim - 1 - a] = 0 if side == 0 else nv[a] - 1
                F = grid[tuple(sl)]  # vertices of the plane, axes in [..][other fastest] order
                F = F.reshape([nv[b] for b in others][::-1])
                # faces: cells of the plane, corners in the local order of the other axes
                fidx = np.indices([n[b] for b in others][::-1]).reshape(dim - 1, -1)[::-1]
                corners = []
                for k in range(2 ** (dim - 1)):
                    off = [(k >> j) & 1 for j in range(dim - 1)]
                    pos = tuple((fidx[j] + off[j]) for j in range(dim - 1))[::-1]
                    corners.append(F[pos])
                corners = np.stack(corners, 1)
                r = np.repeat(corners, corners.shape[1], axis=1).ravel()
                c = np.tile(corners, (1, corners.shape[1])).ravel()
                fb.append(sp.coo_matrix((np.tile(fmass.ravel(), corners.shape[0]), (r, c)), shape=(NV, NV)))
        for m in fb:
            C = C + m.tocsr()
        self.C = C.tocsr()
        self.diag = self.C.diagonal()

    def rhs(self, v0):
        """Assembled sigma_s0 M v0 (v0: the DG scalar-moment values, [cell][node]),
        through the mixed mass matrix of the vertex hat functions."""
        ve = np.asarray(v0, dtype=np.float64).reshape(-1, self.nodes)
        r = self.s0[:, None] * (ve @ self.mix.T)
        return np.bincount(self.vid.ravel(), weights=r.ravel(), minlength=self.NV)

    def solve(self, b, k=None):
        """k Jacobi-preconditioned CG steps from zero (None: direct solve)."""
        if k is None:
            return spl.spsolve(self.C.tocsc(), b)
        x = np.zeros_like(b)
        r = b.copy()
        z = r / self.diag
        p = z.copy()
        rz = r @ z
        for _ in range(k):
            q = self.C @ p
            pq = p @ q
            a = rz / pq if pq > 0 else 0.0
            x += a * p
            r -= a * q
            z = r / self.diag
            rzn = r @ z
            beta = rzn / rz if rz > 0 else 0.0
            rz = rzn
            p = z + beta * p
        return x

    def apply(self, v, k=None):
        """P v for a [mom][dof] vector v."""
        v = np.asarray(v, dtype=np.float64)
        n0 = self.vid.shape[0] * self.nodes
        f = self.solve(self.rhs(v[:n0]), k)
        out = v.copy()
        out[:n0] += (f[self.vid] @ self.ipl.T).ravel()  # the vertex field at each cell's nodes
        return out
