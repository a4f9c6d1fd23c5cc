"""Many independent problems behind one handle (the C-ABI's ouranos_batch_*).

    batch = Batch(problems)              # one persistent sweep launch per class
    y = batch.apply(x)                   # x, y: concatenated [mom][dof] vectors
    x, infos = batch.solve(tol=1e-8)     # FP32 Arnoldi sweeps, FP64 restarts
    batch.slices(y)                      # per-problem views

Vectors are numpy arrays (host) or contiguous float64 CUDA tensors.
"""
import ctypes as C

import numpy as np

from . import _capi
from .transport import _ptr


class Batch:
    def __init__(self, problems, device=-1, autotune=False):
        L = _capi.lib()
        self.problems = list(problems)
        descs = (_capi.ProblemDesc * len(self.problems))()
        keep = []
        for i, p in enumerate(self.problems):
            d, k = p.desc()
            descs[i] = d
            keep.append(k)
        h = C.c_void_p()
        rc = L.ouranos_batch_create(descs, len(self.problems), device, C.byref(h))
        self._h = h.value
        if rc != _capi.OK:
            msg = self._error()
            if self._h:
                L.ouranos_batch_destroy(self._h)
                self._h = None
            raise _capi.OuranosError(rc, msg)
        del keep
        n, total = C.c_int(), C.c_long()
        offs = np.zeros(len(self.problems) + 1, dtype=np.int64)
        self._check(L.ouranos_batch_layout(self._h, C.byref(n), C.byref(total), offs.ctypes.data))
        self.count = n.value
        self.length = total.value
        self.offsets = offs
        self.tiling = None
        if autotune:
            self.autotune()

    def _error(self):
        buf = C.create_string_buffer(512)
        if self._h:
            _capi.lib().ouranos_batch_last_error(self._h, buf, 512)
        return buf.value.decode(errors="replace")

    def _check(self, rc, allow=()):
        if rc != _capi.OK and rc not in allow:
            raise _capi.OuranosError(rc, self._error())
        return rc

    def close(self):
        if getattr(self, "_h", None):
            _capi.lib().ouranos_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _out(self, like):
        if like is not None and hasattr(like, "data_ptr"):
            return like.new_empty((self.length,))
        return np.empty(self.length)

    def slices(self, v):
        return [v[self.offsets[i]:self.offsets[i + 1]] for i in range(self.count)]

    def apply(self, x, precision="fp64", out=None):
        prec = {"fp64": _capi.FP64, "fp32": _capi.FP32}[precision]
        y = self._out(x) if out is None else out
        self._check(_capi.lib().ouranos_batch_apply(self._h, prec, _ptr(x), _ptr(y)))
        return y

    def rhs(self, out=None):
        y = np.empty(self.length) if out is None else out
        self._check(_capi.lib().ouranos_batch_rhs(self._h, _ptr(y)))
        return y

    def set_dsa(self, cg_iterations):
        """Diffusion synthetic acceleration on every problem (0 switches it off)."""
        self._check(_capi.lib().ouranos_batch_set_dsa(self._h, int(cg_iterations)))

    def dsa_apply(self, x, out=None):
        """z = P x for every problem (its diffusion correction), all problems'
        CG solves in one launch."""
        z = self._out(x) if out is None else out
        self._check(_capi.lib().ouranos_batch_dsa_apply(self._h, _ptr(x), _ptr(z)))
        return z

    def solve(self, inner="fp32", tol=1e-8, max_it=2000, restart=30, out=None, dsa=False):
        """Restarted GMRES on all problems at once; dsa=True: FGMRES with each
        problem's diffusion correction (set_dsa) as right preconditioner."""
        prec = {"fp64": _capi.FP64, "fp32": _capi.FP32}[inner]
        if dsa:
            prec |= _capi.SOLVER_DSA
        x = np.empty(self.length) if out is None else out
        infos = (_capi.SolveInfo * self.count)()
        self._check(_capi.lib().ouranos_batch_solve(self._h, prec, restart, max_it, tol, _ptr(x), infos),
                    allow=(_capi.ERR_NOT_CONVERGED,))
        res = [dict(iterations=i.iterations, restarts=i.restarts, residual=i.residual,
                    seconds=i.seconds, converged=bool(i.converged)) for i in infos]
        return x, res

    def autotune(self, precision="fp32", reps=3):
        prec = {"fp64": _capi.FP64, "fp32": _capi.FP32}[precision]
        t = np.zeros(3 * self.count, dtype=np.int32)
        self._check(_capi.lib().ouranos_batch_autotune(self._h, prec, reps, t.ctypes.data))
        self.tiling = t.reshape(self.count, 3)
        return self.tiling

    def set_graphs(self, enable):
        self._check(_capi.lib().ouranos_batch_set_graphs(self._h, int(bool(enable))))

    def stats(self):
        ms, n = C.c_double(), C.c_int()
        self._check(_capi.lib().ouranos_batch_stats(self._h, C.byref(ms), C.byref(n)))
        return ms.value, n.value
