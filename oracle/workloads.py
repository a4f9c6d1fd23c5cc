"""ORACLE -- test infrastructure only.

The seeded synthetic workloads restated for the oracle's own use, so that the
CPU baseline arm of bench.py builds its inputs without loading the product
library: a SplitMix64 stream (Steele, Lea & Flood 2014) drawn in the same
order as the product's generators, and the quadrature from the reference's
own LS tables through oracle/pyoracle.quadrature.  The result is a spec dict
in the format OracleProblem takes.  tests/test_oracle_orders.py checks that
these specs equal the product's problems of the same seed.
"""
import math

import numpy as np

from . import pyoracle

MASK = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed):
        self.state = seed & MASK

    def next_u64(self):
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0):
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / (1 << 53)))


def heterogeneous_2d(seed=1001, n=256, fe_order=2, sn=16, l_max=3, g_aniso=0.7, blocks=8,
                     source_frac=0.25, width=10.0):
    """[0,width]^2 with n x n DG Q_p cells, LS S_sn, blocks x blocks material
    blocks: sigma_t = exp(U[ln 0.1, ln 100]), c ~ U[0.5, 0.9999], Henyey-
    Greenstein moments sigma_s,l = c sigma_t g^l for l <= l_max; q = 1 on the
    central square of side source_frac * width; vacuum boundaries."""
    rng = SplitMix64(seed)
    quad = pyoracle.quadrature(pyoracle.QUAD_LS, sn, l_max, False, 4 * math.pi, 2)
    nb = blocks * blocks
    st = np.zeros((nb, 1))
    ss = np.zeros((nb, 1, 1, l_max + 1))
    for b in range(nb):
        sig = math.exp(rng.uniform(math.log(0.1), math.log(100.0)))
        c = rng.uniform(0.5, 0.9999)
        st[b, 0] = sig
        for l in range(l_max + 1):
            ss[b, 0, 0, l] = c * sig * g_aniso ** l
    bs = max(1, n // blocks)
    i = np.arange(n) // bs
    per_row = (n + bs - 1) // bs
    mat = np.minimum(i[None, :] + per_row * i[:, None], nb - 1).astype(np.int32).reshape(-1)  # [y][x]
    lo = int(round(n * (0.5 - source_frac / 2)))
    hi = int(round(n * (0.5 + source_frac / 2)))
    inside = (np.arange(n) >= lo) & (np.arange(n) < hi)
    sid = (inside[None, :] & inside[:, None]).astype(np.int32).reshape(-1)
    return dict(dim=2, fe_order=fe_order, n_cells=[n, n], lower=[0.0, 0.0], upper=[width, width],
                n_groups=1, omega=quad["omega"], m2d=quad["m2d"], d2m=quad["d2m"],
                moment_l=quad["moment_l"], most_normal=quad["most_normal"], weight_sum=4 * math.pi,
                sigma_t=st, sigma_s=ss.reshape(-1), l_max=l_max, material_id=mat, source_id=sid,
                source=np.array([[0.0], [1.0]]), bc_type=[0] * 6, inc_flux=None)


def solves_per_sweep(spec):
    return int(np.prod(spec["n_cells"])) * spec["omega"].shape[0]


def vector_length(spec):
    n = (spec["fe_order"] + 1) ** spec["dim"]
    return int(np.prod(spec["n_cells"])) * n * spec["m2d"].shape[1]
