"""Learned preconditioner: the convolutional network of csrc/cnn.cu, trained on
the GPU by the project's own forward/backward kernels, used as the right
preconditioner of FGMRES (OURANOS_SOLVER_FGMRES_LEARNED).

Training pairs come from the solver's own operator: for a seeded material map
and an error field e, the residual is v = A e (one Apply), the network input is
the per-cell feature set of v (its eight Q1 nodal scalar-flux values over the
RMS s of v, log sigma_t, scattering ratio) and the target the nodal values of
(e - v)/s -- so z = v + s*correction approximates A^-1 v.  The errors mix
smooth random fields, power iterates T^j e0 of the transport iteration (what
FGMRES's Krylov vectors are made of) and rough noise.
"""
import ctypes as C
import math
import os

import numpy as np

from . import _capi
from .problem import thick_3d

HERE = os.path.dirname(os.path.abspath(__file__))
WEIGHTS = os.path.join(HERE, "weights")
FEATURES = 10  # OURANOS_CNN_FEATURES
OUTPUTS = 8    # OURANOS_CNN_OUTPUTS


def _lib():
    L = _capi.lib()
    if not getattr(L, "_cnn_bound", False):
        vp, i, l, f = C.c_void_p, C.c_int, C.c_long, C.c_float
        sig = {
            "ouranos_cnn_create": [i, i, i, C.c_ulonglong, C.POINTER(vp)],
            "ouranos_cnn_destroy": [vp],
            "ouranos_cnn_n_params": [vp, C.POINTER(l)],
            "ouranos_cnn_get_params": [vp, vp],
            "ouranos_cnn_set_params": [vp, vp],
            "ouranos_cnn_forward": [vp, vp, vp],
            "ouranos_cnn_gradients": [vp, vp, vp, vp, C.POINTER(f)],
            "ouranos_cnn_train_step": [vp, vp, vp, f, C.POINTER(f)],
            "ouranos_cnn_last_error": [vp, C.c_char_p, C.c_size_t],
            "ouranos_rt_set_preconditioner": [vp, vp],
            "ouranos_rt_pc_features": [vp, vp, vp, C.POINTER(C.c_double)],
            "ouranos_rt_pc_target": [vp, vp, vp, vp],
            "ouranos_rt_pc_apply": [vp, vp, vp],
        }
        for name, args in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = i
        L._cnn_bound = True
    return L


class Network:
    """The preconditioner network on an nx x ny x nz cell grid (sides % 4 == 0)."""

    def __init__(self, nx, ny, nz, seed=1234):
        h = C.c_void_p()
        rc = _lib().ouranos_cnn_create(nx, ny, nz, seed, C.byref(h))
        self._h = h.value
        if rc != _capi.OK:
            if self._h:
                _lib().ouranos_cnn_destroy(self._h)
            raise _capi.OuranosError(rc, "network creation failed (grid sides must be multiples of 4)")
        n = C.c_long()
        _lib().ouranos_cnn_n_params(self._h, C.byref(n))
        self.n_params = n.value
        self.grid = (nx, ny, nz)

    def close(self):
        if getattr(self, "_h", None):
            _lib().ouranos_cnn_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def _check(self, rc):
        if rc != _capi.OK:
            buf = C.create_string_buffer(512)
            _lib().ouranos_cnn_last_error(self._h, buf, 512)
            raise _capi.OuranosError(rc, buf.value.decode())

    def params(self):
        out = np.zeros(self.n_params, dtype=np.float32)
        self._check(_lib().ouranos_cnn_get_params(self._h, out.ctypes.data))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n_params
        self._check(_lib().ouranos_cnn_set_params(self._h, p.ctypes.data))

    def forward(self, feat, out):
        """feat: CUDA float32 tensor [cells*FEATURES]; out: CUDA float32 tensor [cells*OUTPUTS]."""
        self._check(_lib().ouranos_cnn_forward(self._h, feat.data_ptr(), out.data_ptr()))
        return out

    def gradients(self, feat, target):
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = C.c_float()
        self._check(_lib().ouranos_cnn_gradients(self._h, feat.data_ptr(), target.data_ptr(),
                                                 g.ctypes.data, C.byref(loss)))
        return loss.value, g

    def train_step(self, feat, target, lr):
        loss = C.c_float()
        self._check(_lib().ouranos_cnn_train_step(self._h, feat.data_ptr(), target.data_ptr(),
                                                  float(lr), C.byref(loss)))
        return loss.value

    def save(self, path, meta=None):
        np.savez_compressed(path, params=self.params(), grid=np.array(self.grid),
                            **{k: np.array(v) for k, v in (meta or {}).items()})

    @classmethod
    def load(cls, path, grid):
        d = np.load(path)
        net = cls(*grid)
        net.set_params(d["params"])
        return net


def smooth_field(shape, rng, corr_cells):
    """Zero-mean Gaussian random field with correlation length ~corr_cells cells."""
    noise = rng.standard_normal(shape)
    k = [np.fft.fftfreq(n) for n in shape]
    kk = np.meshgrid(*k, indexing="ij")
    k2 = sum(x * x for x in kk)
    filt = np.exp(-0.5 * k2 * (2 * math.pi * corr_cells) ** 2)
    f = np.real(np.fft.ifftn(np.fft.fftn(noise) * filt))
    return f / (np.std(f) + 1e-30)


def nodal_error_field(problem, rng):
    """A smooth random scalar-flux error in the DG space (nodal values of a field
    on the vertex grid); higher moments zero."""
    nx, ny, nz = problem.n_cells
    p = problem.fe_order
    corr = math.exp(rng.uniform(0.0, math.log(16.0)))  # 1 to 16 cells, log-uniform
    f = smooth_field((nz * p + 1, ny * p + 1, nx * p + 1), rng, corr * p)
    f += rng.uniform(-1.0, 1.0) * 0.5  # some mean component
    n = problem.dofs_per_cell
    e = np.zeros(problem.vector_length)
    iz, iy, ix = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    cell = (ix + nx * (iy + ny * iz)).reshape(-1)
    ixr, iyr, izr = ix.reshape(-1), iy.reshape(-1), iz.reshape(-1)
    for k in range(n):
        a, b, c = k % (p + 1), (k // (p + 1)) % (p + 1), k // ((p + 1) ** 2)
        e[cell * n + k] = f[izr * p + c, iyr * p + b, ixr * p + a]
    return e


def _start_field(rt, problem, rng, torch, kind):
    if kind == "smooth":
        return torch.from_numpy(nodal_error_field(problem, rng)).cuda()
    if kind == "rough":
        return torch.from_numpy(rng.standard_normal(problem.vector_length)).cuda()
    # the map's own right-hand side: the start of every Krylov space on it
    b = torch.zeros(problem.vector_length, dtype=torch.float64, device="cuda")
    rt.rhs(out=b)
    return b


def power_iterate(rt, e, steps, torch):
    """e <- T^steps e with T = I - A (source iteration on the error, no
    source), renormalised each step; T^j e is what the j-th Krylov vector is
    made of, so pairs built on it look like FGMRES's own inputs."""
    v = torch.empty_like(e)
    for _ in range(steps):
        rt.Apply(e, v)
        e = e - v
        e = e / (e.norm() / math.sqrt(e.numel()) + 1e-300)
    return e


def make_pairs(rt, problem, count, rng, torch, feat_out, target_out, offset, mix=(0.25, 0.5, 0.25)):
    """Fill feat_out[offset:offset+count] / target_out[...] (CUDA tensors) with
    (features(A e), target(A e, e)) pairs.  A fraction mix[0] of the errors e
    are smooth random fields, mix[1] power iterates T^j e0 (j log-uniform in
    [1, 64], e0 smooth, rough or the map's right-hand side) and mix[2] rough
    per-dof noise, so that the network sees the slow modes, the Krylov-like
    differences A T^j e0 and inputs it must leave nearly alone."""
    L = _lib()
    n_cells = problem.total_cells
    for k in range(count):
        u = rng.uniform()
        if u < mix[0]:
            e = _start_field(rt, problem, rng, torch, "smooth")
        elif u < mix[0] + mix[1]:
            start = ("smooth", "rough", "rhs")[int(rng.integers(0, 3))]
            steps = int(round(math.exp(rng.uniform(0.0, math.log(64.0)))))
            e = power_iterate(rt, _start_field(rt, problem, rng, torch, start), steps, torch)
        else:
            e = _start_field(rt, problem, rng, torch, "rough")
        e = e.contiguous()
        v = torch.empty_like(e)
        rt.Apply(e, v)
        f = feat_out[offset + k]
        t = target_out[offset + k]
        _capi.check(L.ouranos_rt_pc_features(rt._h, v.data_ptr(), f.data_ptr(), None), rt._h)
        _capi.check(L.ouranos_rt_pc_target(rt._h, v.data_ptr(), e.data_ptr(), t.data_ptr()), rt._h)
        assert f.numel() == FEATURES * n_cells and t.numel() == OUTPUTS * n_cells


def train(n=64, maps=128, fields_per_map=4, epochs=8, lr=3e-4, seed=7, map_seed0=2000,
          sn=12, log=print):
    """Train the network on seeded 3-D thick-diffusive maps; returns (net, history)."""
    import torch
    from .transport import RadiativeTransfer
    rng = np.random.default_rng(seed)
    n_pairs = maps * fields_per_map
    feats = torch.empty((n_pairs, n ** 3 * FEATURES), dtype=torch.float32, device="cuda")
    targets = torch.empty((n_pairs, n ** 3 * OUTPUTS), dtype=torch.float32, device="cuda")
    for m in range(maps):
        prob = thick_3d(seed=map_seed0 + m, n=n, sn=sn)
        with RadiativeTransfer(prob, precision="fp32") as rt:
            make_pairs(rt, prob, fields_per_map, rng, torch, feats, targets, m * fields_per_map)
    net = Network(n, n, n, seed=seed)
    hist = []
    order = np.arange(n_pairs)
    for ep in range(epochs):
        rng.shuffle(order)
        tot = 0.0
        rate = lr * 0.5 * (1 + math.cos(math.pi * ep / max(1, epochs)))
        for i in order:
            tot += net.train_step(feats[i], targets[i], rate)
        hist.append(tot / n_pairs)
        log("epoch %d loss %.4e" % (ep, hist[-1]))
    return net, hist


def install(rt, net):
    """Use `net` as the right preconditioner of rt's FGMRES_LEARNED solves."""
    _capi.check(_lib().ouranos_rt_set_preconditioner(rt._h, net._h if net else None), rt._h)
    rt._pc_net = net  # keep it alive
