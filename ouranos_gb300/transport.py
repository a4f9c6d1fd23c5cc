"""Python mirror of the reference operator ``RadiativeTransfer<dim,tensor_dim>``
(src/RadiativeTransfer.hh:46-263) over the C-ABI.

Method names and argument meanings follow the reference so that a driver
written against it (src/ouranos.cc:43-209) reads the same:

    rt = RadiativeTransfer(problem)       # constructor + setup()
    rt.set_group(0)
    rhs = np.zeros(rt.length)
    rt.sweep(rhs, group_flux)             # RHS sweep (src/ouranos.cc:152-158)
    rt.Apply(x, y)                        # Epetra_Operator::Apply, returns 0

Vectors are numpy arrays (host) or CUDA tensors (anything with
``data_ptr()``, i.e. device memory), in the [mom][dof] layout.
"""
import ctypes as C

import numpy as np

from . import _capi
from .problem import Problem


def _ptr(v):
    if v is None:
        return None
    if hasattr(v, "data_ptr"):
        if not v.is_contiguous() or str(v.dtype) != "torch.float64":
            raise ValueError("device vectors must be contiguous float64 tensors")
        return v.data_ptr()
    if not (isinstance(v, np.ndarray) and v.dtype == np.float64 and v.flags["C_CONTIGUOUS"]):
        raise ValueError("host vectors must be C-contiguous float64 numpy arrays")
    return v.ctypes.data


class RadiativeTransfer:
    """The transport operator y = x - D L^-1 M2D S x on one GPU."""

    def __init__(self, problem: Problem, device: int = -1, precision: str = "fp64"):
        self.problem = problem
        L = _capi.lib()
        desc, keep = problem.desc()
        h = C.c_void_p()
        rc = L.ouranos_rt_create(C.byref(desc), device, C.byref(h))
        self._h = h.value
        if rc != _capi.OK:
            msg = _capi.last_error(self._h)
            if self._h:
                L.ouranos_rt_destroy(self._h)
                self._h = None
            raise _capi.OuranosError(rc, msg)
        del keep
        n = C.c_long()
        _capi.check(L.ouranos_rt_vector_length(self._h, C.byref(n)), self._h)
        self.length = n.value
        _capi.check(L.ouranos_rt_n_tasks(self._h, C.byref(n)), self._h)
        self.n_tasks = n.value
        self.set_precision(precision)

    # ---- lifetime
    def close(self):
        if getattr(self, "_h", None):
            _capi.lib().ouranos_rt_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        return _capi.check(rc, self._h)

    # ---- reference surface
    def setup(self):
        """RadiativeTransfer::setup -- done by the constructor; kept for drivers."""

    def set_group(self, g):
        self._check(_capi.lib().ouranos_rt_set_group(self._h, g))

    def set_precision(self, precision):
        p = {"fp64": _capi.FP64, "fp32": _capi.FP32}[precision]
        self._check(_capi.lib().ouranos_rt_set_precision(self._h, p))
        self.precision = precision

    def set_fp64_contractions(self, mode):
        """FP64 path arithmetic: 'native' FP64; 'df64' (moment contractions in
        double-float on the FP32 pipes, sweep in FP64); 'df64_sweep' (the sweep's
        cell solves too; the default); 'df64_sweep_tc' (the double-float sweep
        with its contractions on the tensor cores as exact BF16 digit
        products)."""
        m = {"native": _capi.FP64_NATIVE, "df64": _capi.FP64_DF64,
             "df64_sweep": _capi.FP64_DF64_SWEEP, "df64_sweep_tc": _capi.FP64_DF64_SWEEP_TC}[mode]
        self._check(_capi.lib().ouranos_rt_set_fp64_contractions(self._h, m))

    def set_fp32_contractions(self, mode):
        """FP32 path contractions: 'cuda_cores' (FP32 multiply-adds) or
        'tensor' (tcgen05 MMAs on three-part BF16 splits)."""
        m = {"cuda_cores": _capi.FP32_CONTRACT_CUDA_CORES, "tensor": _capi.FP32_CONTRACT_TENSOR}[mode]
        self._check(_capi.lib().ouranos_rt_set_fp32_contractions(self._h, m))

    def get_n_tasks_to_execute(self):
        return self.n_tasks

    def compute_scattering_source(self, x):
        self._check(_capi.lib().ouranos_rt_scattering_source(self._h, _ptr(x)))

    def sweep(self, flux_moments, group_flux=None):
        """flux_moments += D L^-1 (M2D S [+ q + other groups + inflow])."""
        self._check(_capi.lib().ouranos_rt_sweep(self._h, _ptr(flux_moments), _ptr(group_flux)))
        return flux_moments

    def Apply(self, x, y):
        """Epetra_Operator::Apply: y = x - D L^-1 M2D S x; returns 0."""
        self._check(_capi.lib().ouranos_rt_apply(self._h, _ptr(x), _ptr(y)))
        return 0

    def apply(self, x):
        y = np.empty_like(x) if isinstance(x, np.ndarray) else x.new_empty(x.shape)
        self.Apply(x, y)
        return y

    def rhs(self, group_flux=None, out=None):
        """Right-hand side of the Krylov form, in-group scattering taken as zero."""
        if out is None:
            out = np.zeros(self.length)
        self._check(_capi.lib().ouranos_rt_sweep_rhs(self._h, _ptr(group_flux), _ptr(out)))
        return out

    # Epetra_Operator trivia (src/RadiativeTransfer.hh:97-118)
    def UseTranspose(self):
        return False

    def SetUseTranspose(self, flag):
        return 0

    def ApplyInverse(self, x, y):
        return 0

    def NormInf(self):
        return 0.0

    def HasNormInf(self):
        return False

    def Label(self):
        return "radiative_transfer"

    # ---- extensions
    def task_levels(self):
        out = np.zeros(self.n_tasks, dtype=np.int32)
        self._check(_capi.lib().ouranos_rt_task_levels(self._h, out.ctypes.data))
        return out.reshape(self.problem.quad.n_dir, self.problem.total_cells)

    def last_sweep_ms(self):
        ms, k = C.c_double(), C.c_int()
        self._check(_capi.lib().ouranos_rt_last_sweep_ms(self._h, C.byref(ms), C.byref(k)))
        return ms.value, k.value

    def set_tiling(self, cells_x=0, cells_y=0, dirs=0):
        self._check(_capi.lib().ouranos_rt_set_tiling(self._h, cells_x, cells_y, dirs))

    def tiling(self):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        self._check(_capi.lib().ouranos_rt_get_tiling(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def set_stream(self, stream):
        """Run on a caller's cudaStream_t (an int handle, e.g. torch's
        ``torch.cuda.current_stream().cuda_stream``); None = own stream."""
        self._check(_capi.lib().ouranos_rt_set_stream(self._h, stream or None))

    def set_wait_limit(self, ns):
        self._check(_capi.lib().ouranos_rt_set_wait_limit(self._h, float(ns)))

    def debug_wait_bias(self, extra):
        self._check(_capi.lib().ouranos_rt_debug_wait_bias(self._h, int(extra)))

    # ---- implicit Euler in time (an extension: the reference operator is steady)
    def set_time_step(self, inv_vdt):
        """1/(v dt) > 0 turns on implicit Euler (sigma_t + 1/(v dt), psi^n source,
        psi^n = 0); 0 turns it off."""
        self._check(_capi.lib().ouranos_rt_set_time_step(self._h, float(inv_vdt)))

    def set_source(self, source):
        """New fixed-source strengths, [n_sources][n_groups]."""
        src = np.ascontiguousarray(source, dtype=np.float64)
        self._check(_capi.lib().ouranos_rt_set_source(self._h, src.ctypes.data))

    def time_advance(self, phi, method="fgmres_mixed", tol=1e-8, max_it=1000, restart=30, dsa=False):
        """One implicit Euler step: phi (in: guess, e.g. phi^n; out: phi^{n+1})."""
        kind = {"si": _capi.SOLVER_SI, "gmres": _capi.SOLVER_GMRES,
                "fgmres_mixed": _capi.SOLVER_FGMRES_MIXED,
                "fgmres_learned": _capi.SOLVER_FGMRES_LEARNED}[method]
        if dsa:
            kind |= _capi.SOLVER_DSA
        info = _capi.SolveInfo()
        self._check(_capi.lib().ouranos_rt_time_advance(self._h, kind, restart, max_it, tol, _ptr(phi),
                                                        C.byref(info)))
        return dict(iterations=info.iterations, restarts=info.restarts, residual=info.residual,
                    seconds=info.seconds, converged=bool(info.converged))

    def angular_flux(self):
        """psi^n ([dir][dof], lexicographic cells) -- checkpoint state."""
        out = np.zeros(self.problem.quad.n_dir * self.problem.total_cells * self.problem.dofs_per_cell)
        self._check(_capi.lib().ouranos_rt_get_angular_flux(self._h, out.ctypes.data))
        return out

    def set_angular_flux(self, psi):
        psi = np.ascontiguousarray(psi, dtype=np.float64)
        self._check(_capi.lib().ouranos_rt_set_angular_flux(self._h, psi.ctypes.data))

    def set_dsa(self, cg_iterations):
        """Diffusion synthetic acceleration of the scalar flux (DG Q_p meshes):
        the diffusion correction is solved by `cg_iterations` Jacobi-CG steps;
        0 switches it off.  Solves use it with solve(..., dsa=True)."""
        self._check(_capi.lib().ouranos_rt_set_dsa(self._h, int(cg_iterations)))

    def dsa_apply(self, v, out=None):
        """out = v + f, f the diffusion correction of v's scalar moment."""
        if out is None:
            out = np.empty_like(v) if isinstance(v, np.ndarray) else v.new_empty(v.shape)
        self._check(_capi.lib().ouranos_rt_dsa_apply(self._h, _ptr(v), _ptr(out)))
        return out

    def solve_multigroup(self, method="gmres", inner_tol=1e-8, max_inner_it=1000, outer_tol=1e-8,
                         max_outer_it=100, restart=30, group_flux=None, dsa=False):
        """Gauss-Seidel outer iteration over the groups (src/ouranos.cc:62-207):
        returns (group_flux [n_groups * length], info dict); group_flux (host
        or device, [group][mom][dof]) is the initial guess and is updated in
        place."""
        kind = {"si": _capi.SOLVER_SI, "gmres": _capi.SOLVER_GMRES,
                "bicgstab": _capi.SOLVER_BICGSTAB, "fgmres_mixed": _capi.SOLVER_FGMRES_MIXED,
                "fgmres_learned": _capi.SOLVER_FGMRES_LEARNED}[method]
        if dsa:
            kind |= _capi.SOLVER_DSA
        if group_flux is None:
            group_flux = np.zeros(self.problem.n_groups * self.length)
        info = _capi.MultigroupInfo()
        rc = _capi.lib().ouranos_solve_multigroup(self._h, kind, restart, max_inner_it, inner_tol, max_outer_it,
                                                  outer_tol, _ptr(group_flux), C.byref(info))
        if rc not in (_capi.OK, _capi.ERR_NOT_CONVERGED):
            self._check(rc)
        return group_flux, dict(outer_iterations=info.outer_iterations, inner_iterations=info.inner_iterations,
                                change=info.change, seconds=info.seconds, converged=bool(info.converged))

    def solve(self, method="gmres", tol=1e-8, max_it=1000, restart=30, group_flux=None, x=None,
              warm=False, dsa=False):
        """Drivers of src/ouranos.cc:43-209. Returns (x, info dict, residual history);
        warm=True starts from the given x; dsa=True preconditions with the
        diffusion synthetic acceleration (set_dsa)."""
        kind = {"si": _capi.SOLVER_SI, "gmres": _capi.SOLVER_GMRES,
                "bicgstab": _capi.SOLVER_BICGSTAB, "fgmres_mixed": _capi.SOLVER_FGMRES_MIXED,
                "fgmres_learned": _capi.SOLVER_FGMRES_LEARNED}[method]
        if x is None:
            x = np.zeros(self.length)
        if warm:
            kind |= _capi.SOLVER_WARM_START
        if dsa:
            kind |= _capi.SOLVER_DSA
        hist = np.zeros(max_it + 2)
        info = _capi.SolveInfo()
        rc = _capi.lib().ouranos_solve(self._h, kind, restart, max_it, tol, _ptr(group_flux),
                                       _ptr(x), hist.ctypes.data, C.byref(info))
        if rc not in (_capi.OK, _capi.ERR_NOT_CONVERGED):
            self._check(rc)
        n = info.iterations + 1
        return x, dict(iterations=info.iterations, restarts=info.restarts,
                       residual=info.residual, seconds=info.seconds,
                       converged=bool(info.converged)), hist[:n]
