"""Problem descriptions: quadrature, mesh, materials, sources and boundaries.

The reference reads these from deal.II ParameterHandler files
(src/Parameters.cc, src/Geometry.cc, src/RTMaterialProperties.cc); here a
``Problem`` holds them as arrays, built either from those files
(``ouranos_gb300.inp``) or by the seeded generators below, which produce the
synthetic workloads the benchmark and the tests use.  Every generator draws
from one SplitMix64 stream (Steele, Lea & Flood 2014) seeded explicitly.
"""
import ctypes as C
import math
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _capi


# ----------------------------------------------------------------- random
class SplitMix64:
    """SplitMix64 generator: 64-bit state, golden-ratio increment."""

    MASK = (1 << 64) - 1

    def __init__(self, seed):
        self.state = seed & self.MASK

    def next_u64(self):
        self.state = (self.state + 0x9E3779B97F4A7C15) & self.MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & self.MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & self.MASK
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0):
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / (1 << 53)))

    def integer(self, n):
        return self.next_u64() % n

    def choice(self, seq):
        return seq[self.integer(len(seq))]


# ------------------------------------------------------------- quadrature
@dataclass
class Quadrature:
    kind: int
    sn: int
    l_max: int
    galerkin: bool
    weight_sum: float
    dim: int
    harmonics: int
    omega: np.ndarray
    weight: np.ndarray
    m2d: np.ndarray
    d2m: np.ndarray
    moment_l: np.ndarray
    most_normal: np.ndarray

    @property
    def n_dir(self):
        return self.omega.shape[0]

    @property
    def n_mom(self):
        return self.m2d.shape[1]


def build_quadrature(kind, sn, l_max, galerkin=False, weight_sum=4 * math.pi, dim=2,
                     harmonics=_capi.HARM_ORTHONORMAL):
    """RTQuadrature::build_quadrature (src/RTQuadrature.cc:27-56) through the C-ABI."""
    if isinstance(kind, str):
        kind = {"LS": _capi.QUAD_LS, "GLC": _capi.QUAD_GLC}[kind.upper()]
    L = _capi.lib()
    nd, nm = C.c_int(), C.c_int()
    _capi.check(L.ouranos_quadrature_sizes(sn, l_max, int(galerkin), dim, C.byref(nd), C.byref(nm)))
    nd, nm = nd.value, nm.value
    om, w = np.zeros((nd, 3)), np.zeros(nd)
    m2d, d2m = np.zeros((nd, nm)), np.zeros((nm, nd))
    ml = np.zeros(nm, dtype=np.int32)
    mn = np.zeros((2 * dim, nd), dtype=np.int32)
    _capi.check(L.ouranos_quadrature_build(kind, sn, l_max, int(galerkin), float(weight_sum), dim,
                                           harmonics, om.ctypes.data, w.ctypes.data,
                                           m2d.ctypes.data, d2m.ctypes.data, ml.ctypes.data,
                                           mn.ctypes.data))
    return Quadrature(kind, sn, l_max, bool(galerkin), float(weight_sum), dim, harmonics,
                      om, w, m2d, d2m, ml, mn)


# ---------------------------------------------------------------- problem
@dataclass
class Problem:
    dim: int
    fe_order: int
    n_cells: tuple
    lower: tuple
    upper: tuple
    quad: Quadrature
    sigma_t: np.ndarray                  # [mat][g]
    sigma_s: np.ndarray                  # [mat][g_from][g_to][l]
    material_id: np.ndarray              # [cell]
    source_id: Optional[np.ndarray] = None
    source: Optional[np.ndarray] = None  # [src][g]
    bc_type: tuple = (0, 0, 0, 0, 0, 0)
    inc_flux: Optional[np.ndarray] = None  # [face][g]
    cell_order: Optional[np.ndarray] = None
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def n_groups(self):
        return self.sigma_t.shape[1]

    @property
    def l_max(self):
        return self.sigma_s.shape[3] - 1

    @property
    def total_cells(self):
        return int(np.prod(self.n_cells))

    @property
    def dofs_per_cell(self):
        return (self.fe_order + 1) ** self.dim

    @property
    def n_dofs(self):
        return self.total_cells * self.dofs_per_cell

    @property
    def vector_length(self):
        return self.quad.n_mom * self.n_dofs

    def arrays(self):
        """Plain-array view (the oracle's input format)."""
        return dict(
            dim=self.dim, fe_order=self.fe_order, n_cells=list(self.n_cells),
            lower=list(self.lower), upper=list(self.upper), n_groups=self.n_groups,
            omega=self.quad.omega, m2d=self.quad.m2d, d2m=self.quad.d2m,
            moment_l=self.quad.moment_l, most_normal=self.quad.most_normal,
            weight_sum=self.quad.weight_sum, sigma_t=self.sigma_t,
            sigma_s=self.sigma_s.reshape(-1), l_max=self.l_max, material_id=self.material_id,
            source_id=self.source_id, source=self.source, bc_type=list(self.bc_type),
            inc_flux=self.inc_flux,
        )

    def desc(self):
        """A ProblemDesc for ouranos_rt_create plus the arrays it points into."""
        keep = []

        def ptr(a, dtype):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=dtype)
            keep.append(a)
            return a.ctypes.data

        d = _capi.ProblemDesc()
        d.dim = self.dim
        d.fe_order = self.fe_order
        nc = list(self.n_cells) + [1] * (3 - len(self.n_cells))
        d.n_cells = (C.c_int * 3)(*nc)
        d.lower = (C.c_double * 3)(*(list(self.lower) + [0.0] * (3 - len(self.lower))))
        d.upper = (C.c_double * 3)(*(list(self.upper) + [1.0] * (3 - len(self.upper))))
        d.n_groups = self.n_groups
        d.n_dir = self.quad.n_dir
        d.n_mom = self.quad.n_mom
        d.omega = ptr(self.quad.omega, np.float64)
        d.m2d = ptr(self.quad.m2d, np.float64)
        d.d2m = ptr(self.quad.d2m, np.float64)
        d.moment_l = ptr(self.quad.moment_l, np.int32)
        d.most_normal = ptr(self.quad.most_normal, np.int32)
        d.weight_sum = self.quad.weight_sum
        d.n_materials = self.sigma_t.shape[0]
        d.l_max = self.l_max
        d.sigma_t = ptr(self.sigma_t, np.float64)
        d.sigma_s = ptr(self.sigma_s, np.float64)
        d.material_id = ptr(self.material_id, np.int32)
        d.source_id = ptr(self.source_id, np.int32)
        d.n_sources = 0 if self.source is None else self.source.shape[0]
        d.source = ptr(self.source, np.float64)
        d.bc_type = (C.c_int * 6)(*(list(self.bc_type) + [0] * 6)[:6])
        d.inc_flux = ptr(self.inc_flux, np.float64)
        d.cell_order = ptr(self.cell_order, np.int64)
        return d, keep


def _block_index(n_cells, block):
    """Block id of every cell (lexicographic cells, lexicographic blocks)."""
    dim = len(n_cells)
    grids = np.meshgrid(*[np.arange(n) // b for n, b in zip(n_cells, block)], indexing="ij")
    nb = [(n + b - 1) // b for n, b in zip(n_cells, block)]
    idx = np.zeros(grids[0].shape, dtype=np.int64)
    mul = 1
    for a in range(dim):
        idx += grids[a] * mul
        mul *= nb[a]
    # meshgrid 'ij' is [x][y][z]; cells are x fastest -> transpose to [z][y][x]
    return idx.transpose(tuple(range(dim))[::-1]).reshape(-1), int(np.prod(nb))


def uniform_problem(dim, fe_order, n_cells, lower, upper, quad, sigma_t, sigma_s, q,
                    bc=(0,) * 6, name=""):
    nc = int(np.prod(n_cells))
    L = quad.l_max if not quad.galerkin else 0
    ss = np.zeros((1, 1, 1, L + 1))
    ss[0, 0, 0, 0] = sigma_s
    return Problem(dim, fe_order, tuple(n_cells), tuple(lower), tuple(upper), quad,
                   np.array([[sigma_t]], dtype=np.float64), ss,
                   np.zeros(nc, dtype=np.int32), np.zeros(nc, dtype=np.int32),
                   np.array([[q]], dtype=np.float64), tuple(bc), None, None, name)


# ----------------------------------------------------------- workloads
def config_small(n=32, sn=8):
    """2-D homogeneous case: [0,10]^2, n x n Q1, LS S8, sigma_t=1, sigma_s=0.5,
    isotropic scattering, q=1, vacuum boundaries (the CPU-runnable case)."""
    quad = build_quadrature("LS", sn, 0, dim=2)
    return uniform_problem(2, 1, (n, n), (0.0, 0.0), (10.0, 10.0), quad, 1.0, 0.5, 1.0,
                           name="2d-q1-ls%d-%dx%d" % (sn, n, n))


def heterogeneous_2d(seed=1001, n=256, fe_order=2, sn=16, l_max=3, g_aniso=0.7,
                     blocks=8, source_frac=0.25, width=10.0, g_sample=None, name=None):
    """2-D heterogeneous anisotropic case: n x n cells of DG Q_p on [0,width]^2,
    LS S_sn, blocks x blocks material blocks with sigma_t ~ LogUniform[0.1,100]
    and scattering ratio c ~ U[0.5,0.9999]; Henyey-Greenstein Legendre moments
    sigma_s,l = c sigma_t g^l up to l_max; q = 1 on the central square of side
    source_frac*width, 0 elsewhere; vacuum boundaries."""
    rng = SplitMix64(seed)
    quad = build_quadrature("LS", sn, l_max, dim=2)
    nb = blocks * blocks
    g = g_aniso if g_sample is None else g_sample
    st = np.zeros((nb, 1))
    ss = np.zeros((nb, 1, 1, l_max + 1))
    for b in range(nb):
        sig = math.exp(rng.uniform(math.log(0.1), math.log(100.0)))
        c = rng.uniform(0.5, 0.9999)
        st[b, 0] = sig
        for l in range(l_max + 1):
            ss[b, 0, 0, l] = c * sig * g ** l
    bs = max(1, n // blocks)
    mat, _ = _block_index((n, n), (bs, bs))
    mat = np.minimum(mat, nb - 1).astype(np.int32)
    ij = np.arange(n)
    lo = int(round(n * (0.5 - source_frac / 2)))
    hi = int(round(n * (0.5 + source_frac / 2)))
    inside = (ij >= lo) & (ij < hi)
    sid = (inside[None, :] & inside[:, None]).astype(np.int32).reshape(-1)  # [y][x]
    src = np.array([[0.0], [1.0]])
    return Problem(2, fe_order, (n, n), (0.0, 0.0), (width, width), quad, st, ss, mat, sid, src,
                   (0,) * 6, None, None,
                   name or "2d-q%d-ls%d-p%d-%dx%d-seed%d" % (fe_order, sn, l_max, n, n, seed),
                   {"seed": seed})


def thick_3d(seed=2000, n=64, fe_order=1, sn=12, block=4, width=10.0):
    """3-D thick diffusive case: [0,width]^3, n^3 hexes DG Q_p, GLC S_sn
    (8 octants); material blocks of block^3 cells, each (sigma_t, c) = (100,
    0.999) with probability 1/2 else (1, 0.9); isotropic scattering; q = 1
    everywhere; vacuum boundaries."""
    rng = SplitMix64(seed)
    quad = build_quadrature("GLC", sn, 0, dim=3)
    blk, nb = _block_index((n, n, n), (block, block, block))
    kind = np.array([1 if rng.uniform() < 0.5 else 0 for _ in range(nb)], dtype=np.int32)
    mat = kind[blk].astype(np.int32)
    st = np.array([[1.0], [100.0]])
    ss = np.array([[[[0.9 * 1.0]]], [[[0.999 * 100.0]]]])
    nc = n ** 3
    return Problem(3, fe_order, (n, n, n), (0.0,) * 3, (width,) * 3, quad, st, ss, mat,
                   np.zeros(nc, dtype=np.int32), np.array([[1.0]]), (0,) * 6, None, None,
                   "3d-q%d-glc%d-%d^3-seed%d" % (fe_order, sn, n, seed), {"seed": seed})


def batch_2d(seed=3000, count=64, sides=(32, 64, 128, 256, 512), orders=(1, 2),
             sns=(4, 8, 12, 16)):
    """Batched uneven workload: `count` independent 2-D problems, each with its
    own seed; side, DG order and LS order drawn uniformly; heterogeneous
    materials with P1 Henyey-Greenstein scattering, g ~ U[0,0.8]."""
    rng = SplitMix64(seed)
    out = []
    for i in range(count):
        side = rng.choice(sides)
        p = rng.choice(orders)
        sn = rng.choice(sns)
        g = rng.uniform(0.0, 0.8)
        out.append(heterogeneous_2d(seed=seed * 1000 + i, n=side, fe_order=p, sn=sn, l_max=1,
                                    g_sample=g,
                                    name="batch%d-%d: %dx%d q%d ls%d" % (seed, i, side, side, p, sn)))
    return out


def time_dependent_3d(seed=4000, n=128, fe_order=1, sn=8, block=8, width=20.0, inv_vdt=0.5):
    """3-D time-dependent case: [0,width]^3, n^3 hexes, LS S_sn (8 octants);
    two-material map on block^3 blocks, (physical) sigma_t in {0.5, 50}, c in
    {0.7, 0.99}; source id 1 marks the pulse region, a seeded block^3-cell box
    of unit strength (scaled per step with set_source).  1/(v dt) is in
    meta["inv_vdt"], for RadiativeTransfer.set_time_step."""
    rng = SplitMix64(seed)
    quad = build_quadrature("LS", sn, 0, dim=3)
    blk, nb = _block_index((n, n, n), (block, block, block))
    kind = np.array([1 if rng.uniform() < 0.5 else 0 for _ in range(nb)], dtype=np.int32)
    mat = kind[blk].astype(np.int32)
    st = np.array([[0.5], [50.0]])
    ss = np.array([[[[0.7 * 0.5]]], [[[0.99 * 50.0]]]])
    pulse_block = rng.integer(nb)
    sid = (blk == pulse_block).astype(np.int32)
    return Problem(3, fe_order, (n, n, n), (0.0,) * 3, (width,) * 3, quad, st, ss, mat, sid,
                   np.array([[0.0], [1.0]]), (0,) * 6, None, None,
                   "3d-td-q%d-ls%d-%d^3-seed%d" % (fe_order, sn, n, seed),
                   {"seed": seed, "inv_vdt": inv_vdt})


def pulse_strength(step, peak=10.0, center=20, width=5.0):
    """Gaussian-in-time pulse: q = peak exp(-(step - center)^2 / (2 width^2))."""
    return peak * math.exp(-0.5 * ((step - center) / width) ** 2)


def zorder_cells(nx, ny):
    """deal.II's hierarchical cell order of a globally refined single coarse
    square (z-order): index of each lexicographic cell."""
    out = np.zeros(nx * ny, dtype=np.int64)
    bits = max(nx, ny).bit_length()
    for j in range(ny):
        for i in range(nx):
            z = 0
            for b in range(bits):
                z |= ((i >> b) & 1) << (2 * b)
                z |= ((j >> b) & 1) << (2 * b + 1)
            out[i + nx * j] = z
    return out
