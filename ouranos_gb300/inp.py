"""Reader for the reference's input files (deal.II ParameterHandler syntax,
``set Name = value`` lines and ``subsection ... end`` blocks).

Mirrors the fields of Parameters (src/Parameters.cc:28-302), Geometry
(src/Geometry.cc:85-128) and RTMaterialProperties (src/RTMaterialProperties.cc:34-54)
that the transport path needs, so a reference input deck can be replayed on
the GB300 operator.  Coarse-cell ids are looked up by cell centre relative to
the box's lower corner; the reference divides the absolute centre coordinate
by the coarse cell size (src/Geometry.cc:67-70), which agrees whenever the
lower corner is at the origin.
"""
import math
import os
from dataclasses import dataclass, field

import numpy as np

BC = {"vacuum": 0, "isotropic": 1, "most normal": 2, "reflective": 3}
SOLVERS = ("SI", "GMRES", "BICGSTAB")


def parse_prm(text):
    """Nested dict of the `set` entries; subsections become sub-dicts."""
    root = {}
    stack = [root]
    for raw in text.splitlines():
        line = raw.split("#", 1)[0].strip()
        if not line:
            continue
        low = line.lower()
        if low.startswith("subsection "):
            sub = {}
            stack[-1][line[len("subsection "):].strip()] = sub
            stack.append(sub)
        elif low == "end":
            if len(stack) == 1:
                raise ValueError("unbalanced 'end'")
            stack.pop()
        elif low.startswith("set "):
            name, _, value = line[4:].partition("=")
            stack[-1][name.strip()] = value.strip()
        else:
            raise ValueError("cannot parse line: %r" % raw)
    if len(stack) != 1:
        raise ValueError("missing 'end'")
    return root


def _list(s, n=None, conv=float):
    vals = [conv(v) for v in s.replace(",", " ").split()]
    if n is not None:
        vals = (vals + [conv(0)] * n)[:n]
    return vals


@dataclass
class Parameters:
    dimension: int = 2
    fe_order: int = 1
    geometry_filename: str = "geometry.inp"
    n_refinements: int = 0
    refinement_factor: float = 0.0
    coarsening_factor: float = 0.0
    output_filename: str = "output"
    xs_filename: str = "xs.inp"
    solver_type: str = "SI"
    max_outer_it: int = 1
    max_inner_it: int = 1
    outer_tolerance: float = 1e-4
    inner_tolerance: float = 1e-6
    sn_order: int = 2
    quad_type: str = "GLC"
    weight_sum: float = 4 * math.pi
    galerkin: bool = False
    bc_type: list = field(default_factory=lambda: [0] * 6)
    inc_flux: list = field(default_factory=lambda: [[] for _ in range(6)])
    n_src: int = 0
    n_groups: int = 1
    src: list = field(default_factory=list)   # [source][group]

    def get_inc_flux(self, face, g):
        return self.inc_flux[face][g]

    def get_src(self, s, g):
        return self.src[s][g]


def read_parameters(text):
    """Parameters::parse_parameters (src/Parameters.cc:105-302)."""
    d = parse_prm(text)
    rt = d.get("Radiative Transfer parameters", {})
    p = Parameters()
    p.dimension = int(d.get("Dimension", 2))
    p.fe_order = int(d.get("FE order", 1))
    p.geometry_filename = d.get("Geometry file", p.geometry_filename)
    p.n_refinements = int(d.get("Number of refinements", 0))
    p.refinement_factor = float(d.get("Refinement factor", 0.0))
    p.coarsening_factor = float(d.get("Coarsening factor", 0.0))
    p.output_filename = d.get("Output file", p.output_filename)
    p.xs_filename = rt.get("Cross sections file", p.xs_filename)
    st = rt.get("Solver type", "SI")
    if st not in SOLVERS:
        raise ValueError("Solver type must be SI, GMRES or BICGSTAB")
    p.solver_type = st
    p.max_outer_it = int(rt.get("Max outer iterations", 1))
    p.max_inner_it = int(rt.get("Max inner iterations", 1))
    p.outer_tolerance = float(rt.get("Tolerance outer solver", 1e-4))
    p.inner_tolerance = float(rt.get("Tolerance inner solver", 1e-6))
    p.sn_order = int(rt.get("Sn order", 2))
    p.quad_type = rt.get("Quadrature type", "GLC")
    ws = rt.get("Sum weight", "4PI")
    p.weight_sum = {"1": 1.0, "2PI": 2 * math.pi, "4PI": 4 * math.pi}[ws]
    p.galerkin = rt.get("Galerkin", "false").strip().lower() == "true"
    p.n_groups = int(rt.get("Number of groups", 1))
    names = ["Xmin", "Xmax", "Ymin", "Ymax", "Zmin", "Zmax"]
    for f, nm in enumerate(names):
        if f >= 2 * p.dimension:
            break
        p.bc_type[f] = BC[rt.get(nm + " BC", "vacuum")]
        if p.bc_type[f] in (BC["isotropic"], BC["most normal"]):
            p.inc_flux[f] = _list(rt.get(nm + " BC values", "0"), p.n_groups)
        else:
            p.inc_flux[f] = [0.0] * p.n_groups
    p.n_src = int(rt.get("Number of sources", 0))
    vals = _list(rt.get("Source intensity", "1."), p.n_src * p.n_groups)
    p.src = [vals[s * p.n_groups:(s + 1) * p.n_groups] for s in range(p.n_src)]
    return p


@dataclass
class Geometry:
    dim: int
    bottom_left: list
    upper_right: list
    n_subdivisions: list
    n_global_refinements: int
    material_ids: list
    source_ids: list

    @property
    def n_materials(self):
        return max(self.material_ids) + 1

    def _coarse(self, ids, i, j, k=0):
        n = self.n_subdivisions
        return ids[i + j * n[0] + (k * n[0] * n[1] if self.dim == 3 else 0)]

    def coarse_material(self, i, j, k=0):
        return self._coarse(self.material_ids, i, j, k)

    def coarse_source(self, i, j, k=0):
        return self._coarse(self.source_ids, i, j, k)

    def n_cells(self):
        r = 2 ** self.n_global_refinements
        return [s * r for s in self.n_subdivisions]

    def cell_ids(self):
        """Material and source id of every fine cell (lexicographic)."""
        r = 2 ** self.n_global_refinements
        nc = self.n_cells()
        idx = [np.arange(n) // r for n in nc]
        if self.dim == 2:
            J, I = np.meshgrid(idx[1], idx[0], indexing="ij")
            coarse = I + J * self.n_subdivisions[0]
        else:
            K, J, I = np.meshgrid(idx[2], idx[1], idx[0], indexing="ij")
            coarse = I + J * self.n_subdivisions[0] + K * self.n_subdivisions[0] * self.n_subdivisions[1]
        coarse = coarse.reshape(-1)
        return (np.asarray(self.material_ids, dtype=np.int32)[coarse],
                np.asarray(self.source_ids, dtype=np.int32)[coarse])


def read_geometry(text, dim):
    """Geometry::parse_parameters (src/Geometry.cc:102-128)."""
    d = parse_prm(text)
    nsub = _list(d.get("Number of subdivisions", "1,1"), dim, int)
    ncoarse = int(np.prod(nsub))
    return Geometry(dim, _list(d.get("Bottom left point", "0,0"), dim),
                    _list(d.get("Upper right point", "0,0"), dim), nsub,
                    int(d.get("Number of global refinements", 0)),
                    _list(d.get("Material IDs", "0"), ncoarse, int),
                    _list(d.get("Source IDs", "0"), ncoarse, int))


@dataclass
class Materials:
    l_max: int
    sigma_t: np.ndarray   # [mat][g]
    sigma_s: np.ndarray   # [mat][g][gp][l]


def read_materials(text, n_materials, n_groups):
    """RTMaterialProperties::parse_parameters (src/RTMaterialProperties.cc:43-54)."""
    d = parse_prm(text)
    L = int(d.get("L_max", 0))
    st = np.array(_list(d.get("Sigma_t", "1."), n_materials * n_groups)).reshape(n_materials, n_groups)
    ss = np.array(_list(d.get("Sigma_s", "0."), n_materials * n_groups * n_groups * (L + 1)))
    return Materials(L, st, ss.reshape(n_materials, n_groups, n_groups, L + 1))


def problem_from_files(parameters_path, base_dir=None, harmonics=0):
    """Build an ouranos_gb300 Problem from a reference input deck.

    File names inside the deck are resolved against ``base_dir`` (default:
    the current directory, as the reference does)."""
    from .problem import Problem, build_quadrature
    base = base_dir or os.getcwd()

    def rd(path):
        with open(path if os.path.isabs(path) else os.path.join(base, path)) as f:
            return f.read()

    prm = read_parameters(rd(parameters_path))
    geo = read_geometry(rd(prm.geometry_filename), prm.dimension)
    mat = read_materials(rd(prm.xs_filename), geo.n_materials, prm.n_groups)
    quad = build_quadrature(prm.quad_type, prm.sn_order, mat.l_max, prm.galerkin, prm.weight_sum,
                            prm.dimension, harmonics)
    mid, sid = geo.cell_ids()
    src = np.array(prm.src, dtype=np.float64) if prm.n_src else None
    inc = np.array([(prm.inc_flux[f] or [0.0] * prm.n_groups) for f in range(2 * prm.dimension)])
    return Problem(prm.dimension, prm.fe_order, tuple(geo.n_cells()), tuple(geo.bottom_left),
                   tuple(geo.upper_right), quad, mat.sigma_t, mat.sigma_s, mid, sid, src,
                   tuple(prm.bc_type), inc, None, os.path.basename(parameters_path),
                   {"parameters": prm, "geometry": geo})
