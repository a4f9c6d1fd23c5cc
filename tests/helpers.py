"""Shared helpers for the test-suite."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def rel_err(a, b):
    b = np.asarray(b)
    nb = np.linalg.norm(b)
    return np.linalg.norm(np.asarray(a) - b) / (nb if nb > 0 else 1.0)


def golden_problem(og):
    """The problem of tests/RadiativeTransfer_test.cc (tests/rt_*.inp): [0,2]^2 refined
    twice (4x4 cells), DG Q1, GLC S4, weight sum 1, sigma_t = 1, sigma_s = 0.5,
    q = 1, vacuum boundaries."""
    g = golden("rt_golden.json")
    prm, geo, xs = g["parameters"], g["geometry"], g["xs"]
    lo = [float(v) for v in geo["Bottom left point"].split(",")]
    hi = [float(v) for v in geo["Upper right point"].split(",")]
    n = 2 ** int(geo["Number of global refinements"])
    sn = int(prm["Sn order"])
    ws = float(prm["Sum weight"])
    q = og.build_quadrature(prm["Quadrature type"], sn, int(xs["L_max"]), False, ws, 2)
    p = og.uniform_problem(2, int(prm["FE order"]), (n, n), lo, hi, q, float(xs["Sigma_t"]),
                           float(xs["Sigma_s"]), float(prm["Source intensity"]))
    return p, g


def to_zorder(x, n_cells_side, n_local):
    """Reorder a lexicographic-cell vector into deal.II's z-order cell numbering."""
    import ouranos_gb300 as og
    z = og.zorder_cells(n_cells_side, n_cells_side)
    out = np.zeros_like(x)
    for c, zc in enumerate(z):
        out[zc * n_local:(zc + 1) * n_local] = x[c * n_local:(c + 1) * n_local]
    return out
