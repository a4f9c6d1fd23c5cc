"""ORACLE -- test infrastructure only.

ctypes wrapper around oracle/_build/liboracle.so (the FP64 CPU restatement of
the reference sweep, oracle/oracle.cpp).  Used by tests/, by
__graft_entry__.smoke() and by bench.py's CPU-baseline arm, only as the
checker or the CPU baseline -- never as the product path.

Quadrature tables come from the reference's own LS/GLC source tables,
extracted into tests/golden/ls_tables.json and tests/golden/glc_gauss.json.
"""
import ctypes as C
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(os.path.dirname(HERE), "tests", "golden")

_lib = None

HARM_ORTHONORMAL = 0
HARM_REFERENCE = 1
QUAD_LS = 0
QUAD_GLC = 1


class OrcDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("fe_order", C.c_int), ("n_cells", C.c_int * 3),
        ("lower", C.c_double * 3), ("upper", C.c_double * 3),
        ("n_groups", C.c_int), ("group", C.c_int),
        ("n_dir", C.c_int), ("n_mom", C.c_int),
        ("omega", C.c_void_p), ("m2d", C.c_void_p), ("d2m", C.c_void_p),
        ("moment_l", C.c_void_p), ("most_normal", C.c_void_p),
        ("weight_sum", C.c_double),
        ("n_materials", C.c_int), ("l_max", C.c_int),
        ("sigma_t", C.c_void_p), ("sigma_s", C.c_void_p),
        ("material_id", C.c_void_p), ("source_id", C.c_void_p),
        ("n_sources", C.c_int), ("source", C.c_void_p),
        ("bc_type", C.c_int * 6), ("inc_flux", C.c_void_p),
    ]


def lib():
    global _lib
    if _lib is None:
        import importlib.util
        spec = importlib.util.spec_from_file_location("_oracle_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        path = mod.build()
        L = C.CDLL(path)
        vp, i, d, l = C.c_void_p, C.c_int, C.c_double, C.c_long
        L.orc_create.restype = vp
        L.orc_create.argtypes = [C.POINTER(OrcDesc)]
        L.orc_destroy.argtypes = [vp]
        L.orc_set_group.argtypes = [vp, i]
        L.orc_set_scheduler.argtypes = [vp, i]
        L.orc_set_time_step.argtypes = [vp, C.c_double]
        L.orc_set_source.argtypes = [vp, vp]
        L.orc_advance_angular.argtypes = [vp, vp, i]
        L.orc_get_angular.argtypes = [vp, vp]
        L.orc_set_angular.argtypes = [vp, vp]
        L.orc_n_dofs.restype = l
        L.orc_n_dofs.argtypes = [vp]
        L.orc_n_tasks.restype = l
        L.orc_n_tasks.argtypes = [vp]
        L.orc_scattering_source.argtypes = [vp, vp]
        L.orc_clear_scattering_source.argtypes = [vp]
        L.orc_sweep.argtypes = [vp, vp, vp, i, i]
        L.orc_apply.argtypes = [vp, vp, vp, i]
        L.orc_last_order.argtypes = [vp, vp]
        L.orc_task_levels.argtypes = [vp, vp]
        L.orc_task_ids.argtypes = [vp, vp]
        L.orc_fecell.argtypes = [vp, l, vp, vp, vp, vp, vp]
        L.orc_solve.restype = i
        L.orc_solve.argtypes = [vp, i, i, i, d, vp, vp, vp, i]
        L.orc_quadrature_sizes.restype = i
        L.orc_quadrature_sizes.argtypes = [i, i, i, i, C.POINTER(i), C.POINTER(i)]
        L.orc_quadrature_build.restype = i
        L.orc_quadrature_build.argtypes = [i, i, i, i, d, i, i, vp, vp, vp, vp, vp, vp, vp, vp]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def _tables(kind, sn):
    if kind == QUAD_LS:
        with open(os.path.join(GOLDEN, "ls_tables.json")) as f:
            t = json.load(f)[str(sn)]
        return np.array(t["direction"], dtype=np.float64), np.array(t["weight"], dtype=np.float64)
    with open(os.path.join(GOLDEN, "glc_gauss.json")) as f:
        t = json.load(f)[str(sn)]
    return np.array(t["nodes"], dtype=np.float64), np.array(t["weights"], dtype=np.float64)


def quadrature(kind, sn, l_max, galerkin, weight_sum, dim, harmonics=HARM_ORTHONORMAL):
    """RTQuadrature::build_quadrature restated; tables from the reference text."""
    L = lib()
    nd, nm = C.c_int(), C.c_int()
    if L.orc_quadrature_sizes(sn, l_max, int(galerkin), dim, C.byref(nd), C.byref(nm)):
        raise ValueError("bad quadrature order")
    nd, nm = nd.value, nm.value
    ta, tb = _tables(kind, sn)
    out = {
        "omega": np.zeros((nd, 3)), "weight": np.zeros(nd),
        "m2d": np.zeros((nd, nm)), "d2m": np.zeros((nm, nd)),
        "moment_l": np.zeros(nm, dtype=np.int32),
        "most_normal": np.zeros((2 * dim, nd), dtype=np.int32),
    }
    rc = L.orc_quadrature_build(kind, sn, l_max, int(galerkin), float(weight_sum), dim, harmonics,
                                _ptr(ta), _ptr(tb), _ptr(out["omega"]), _ptr(out["weight"]),
                                _ptr(out["m2d"]), _ptr(out["d2m"]), _ptr(out["moment_l"]),
                                _ptr(out["most_normal"]))
    if rc:
        raise ValueError("quadrature build failed (%d)" % rc)
    out["n_dir"], out["n_mom"] = nd, nm
    return out


class OracleProblem:
    """The reference operator restated on the CPU for one problem.

    ``spec`` is a dict with the keys of ``ouranos_gb300.problem.Problem.arrays()``
    (dim, fe_order, n_cells, lower, upper, n_groups, omega, m2d, d2m, moment_l,
    most_normal, weight_sum, sigma_t, sigma_s, l_max, material_id, source_id,
    source, bc_type, inc_flux).

    ``order`` picks the task order of apply/solve: "fifo" is the reference's
    ready list with linear dependency counters (src/RadiativeTransfer.cc:
    605-692); "cartesian" runs each direction's cells in upwind-first
    lexicographic order without building the task graph (identical task
    values, for meshes whose graph would not fit in memory).
    """

    ORDERS = {"fifo": 0, "cartesian": 2}

    def __init__(self, spec, order="fifo"):
        L = lib()
        self._keep = {}

        def arr(key, dtype):
            v = spec.get(key)
            if v is None:
                return None
            a = np.ascontiguousarray(v, dtype=dtype)
            self._keep[key] = a
            return a

        d = OrcDesc()
        d.dim = spec["dim"]
        d.fe_order = spec["fe_order"]
        nc = list(spec["n_cells"]) + [1] * (3 - len(spec["n_cells"]))
        d.n_cells = (C.c_int * 3)(*nc)
        lo = list(spec["lower"]) + [0.0] * (3 - len(spec["lower"]))
        hi = list(spec["upper"]) + [1.0] * (3 - len(spec["upper"]))
        d.lower = (C.c_double * 3)(*lo)
        d.upper = (C.c_double * 3)(*hi)
        d.n_groups = spec.get("n_groups", 1)
        d.group = spec.get("group", 0)
        om = arr("omega", np.float64)
        d.n_dir = om.shape[0]
        m2d = arr("m2d", np.float64)
        d.n_mom = m2d.shape[1]
        d.omega, d.m2d = _ptr(om), _ptr(m2d)
        d.d2m = _ptr(arr("d2m", np.float64))
        d.moment_l = _ptr(arr("moment_l", np.int32))
        d.most_normal = _ptr(arr("most_normal", np.int32))
        d.weight_sum = spec["weight_sum"]
        st = arr("sigma_t", np.float64)
        d.n_materials = st.shape[0] if st.ndim > 1 else st.size // d.n_groups
        d.l_max = spec.get("l_max", 0)
        d.sigma_t = _ptr(st)
        d.sigma_s = _ptr(arr("sigma_s", np.float64))
        d.material_id = _ptr(arr("material_id", np.int32))
        d.source_id = _ptr(arr("source_id", np.int32))
        src = arr("source", np.float64)
        d.n_sources = 0 if src is None else (src.shape[0] if src.ndim > 1 else src.size // d.n_groups)
        d.source = _ptr(src)
        bc = list(spec.get("bc_type", [0] * 6)) + [0] * 6
        d.bc_type = (C.c_int * 6)(*bc[:6])
        d.inc_flux = _ptr(arr("inc_flux", np.float64))
        self._desc = d
        self.h = L.orc_create(C.byref(d))
        if not self.h:
            raise ValueError("oracle rejected the problem")
        L.orc_set_scheduler(self.h, self.ORDERS[order])
        self.n_dofs = L.orc_n_dofs(self.h)
        self.n_mom = d.n_mom
        self.n_dir = d.n_dir
        self.n_cells = int(np.prod(nc))
        self.n_groups = d.n_groups
        self.length = self.n_mom * self.n_dofs

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def set_group(self, g):
        lib().orc_set_group(self.h, g)

    # implicit Euler in time (an extension: the reference operator is steady)
    def set_time_step(self, inv_vdt):
        lib().orc_set_time_step(self.h, float(inv_vdt))

    def set_source(self, source):
        src = np.ascontiguousarray(source, dtype=np.float64)
        lib().orc_set_source(self.h, _ptr(src))

    def advance_angular(self, phi, threads=1):
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        lib().orc_advance_angular(self.h, _ptr(phi), threads)

    def angular_flux(self):
        out = np.zeros(self.n_dir * self.n_dofs)
        lib().orc_get_angular(self.h, _ptr(out))
        return out

    def set_angular_flux(self, psi):
        psi = np.ascontiguousarray(psi, dtype=np.float64)
        assert psi.size == self.n_dir * self.n_dofs
        lib().orc_set_angular(self.h, _ptr(psi))

    def scattering_source(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        lib().orc_scattering_source(self.h, _ptr(x))

    def clear_scattering_source(self):
        lib().orc_clear_scattering_source(self.h)

    def sweep(self, flux=None, group_flux=None, scheduler=0, threads=1):
        """scheduler: 0 ready list, 1 the reference's all-task scan, 2 cartesian."""
        flux = np.zeros(self.length) if flux is None else np.ascontiguousarray(flux, dtype=np.float64)
        gf = None if group_flux is None else np.ascontiguousarray(group_flux, dtype=np.float64)
        lib().orc_sweep(self.h, _ptr(flux), _ptr(gf), scheduler, threads)
        return flux

    def apply(self, x, threads=1):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(x)
        lib().orc_apply(self.h, _ptr(x), _ptr(y), threads)
        return y

    def rhs(self, group_flux=None, threads=1):
        """The right-hand side sweep of the Krylov form (src/ouranos.cc:149-158)."""
        if group_flux is None:
            group_flux = np.zeros(self.n_groups * self.length)
        self.clear_scattering_source()
        return self.sweep(group_flux=group_flux, threads=threads)

    def last_order(self):
        o = np.zeros(self.n_dir * self.n_cells, dtype=np.int64)
        lib().orc_last_order(self.h, _ptr(o))
        return o

    def task_levels(self):
        o = np.zeros(self.n_dir * self.n_cells, dtype=np.int32)
        lib().orc_task_levels(self.h, _ptr(o))
        return o.reshape(self.n_dir, self.n_cells)

    def task_ids(self):
        o = np.zeros(self.n_dir * self.n_cells, dtype=np.int64)
        lib().orc_task_ids(self.h, _ptr(o))
        return o.reshape(self.n_dir, self.n_cells)

    def fecell(self, cell=0):
        dim = self._desc.dim
        n = self.n_dofs // self.n_cells
        out = dict(mass=np.zeros((n, n)), grad=np.zeros((dim, n, n)),
                   downwind=np.zeros((2 * dim, n, n)), upwind=np.zeros((2 * dim, n, n)),
                   normals=np.zeros((2 * dim, 3)))
        lib().orc_fecell(self.h, cell, _ptr(out["mass"]), _ptr(out["grad"]), _ptr(out["downwind"]),
                         _ptr(out["upwind"]), _ptr(out["normals"]))
        return out

    def solve(self, kind="gmres", tol=1e-10, max_it=1000, restart=30, group_flux=None, threads=1):
        k = {"si": 0, "gmres": 1, "bicgstab": 2}[kind]
        x = np.zeros(self.length)
        hist = np.zeros(max_it + 2)
        gf = None if group_flux is None else np.ascontiguousarray(group_flux, dtype=np.float64)
        it = lib().orc_solve(self.h, k, restart, max_it, tol, _ptr(gf), _ptr(x), _ptr(hist), threads)
        return x, it, hist[: it + 1]
