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

`train_on_solver_pairs` trains instead on the vectors FGMRES itself meets:
the inputs of its right preconditioner in a diffusion-accelerated solve (and
then in the learned-preconditioned one), each with its diffusion correction
as the target; `fgmres_pairs` exposes every Arnoldi step's exact pair
(w = A z, z).
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
            "ouranos_rt_pc_dsa_apply": [vp, vp, vp],
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


def fgmres_pairs(rt, b, precondition, record, m=30, max_it=60, tol=1e-8):
    """Restarted FGMRES(m) on A = rt's operator (CUDA float64 vectors), that
    hands every Arnoldi step's exact pair to record(w, z): z = P(v_j) is the
    preconditioned basis vector and w = A z the operator's image of it, taken
    before the orthogonalisation.  So z is the true error of the residual w,
    and the pairs are the ones the solver itself meets, with the distribution
    of its own Krylov vectors.  Classical Gram-Schmidt with one
    re-orthogonalisation, like csrc/solvers.cu.  Returns (x, iterations)."""
    import torch
    x = torch.zeros_like(b)
    nb = float(b.norm())
    it, res = 0, float("inf")
    while it < max_it:
        r = b - rt.apply(x) if it else b.clone()
        beta = float(r.norm())
        if beta <= tol * nb:
            break
        V = [r / beta]
        Z = []
        H = torch.zeros((m + 1, m), dtype=torch.float64)
        y = None
        for j in range(m):
            z = precondition(V[j])
            w = rt.apply(z)
            record(w, z)
            Z.append(z)
            it += 1
            Vs = torch.stack(V)
            for _ in range(2):
                h = Vs @ w
                w = w - Vs.T @ h
                H[: j + 1, j] += h.cpu()
            H[j + 1, j] = float(w.norm())
            V.append(w / max(float(H[j + 1, j]), 1e-300))
            e1 = torch.zeros(j + 2, dtype=torch.float64)
            e1[0] = beta
            y = torch.linalg.lstsq(H[: j + 2, : j + 1], e1[:, None]).solution[:, 0]
            res = float((H[: j + 2, : j + 1] @ y - e1).norm())
            if res <= tol * nb or it >= max_it:
                break
        x = x + torch.stack(Z).T @ y.to(x.device)
        if res <= tol * nb:
            break
    return x, it


def solver_pairs(rt, count, feat_out, target_out, offset, precondition=None, base=None, m=30):
    """Fill feat_out/target_out[offset:offset+count] with the pairs of the first
    `count` Arnoldi steps of FGMRES(m) on rt's own right-hand side: features of
    w = A z and the target (z - base(w)) / (s K) -- the part of the true error z
    that the network has to add to base(w) (base=None: w itself, the plain
    network; the diffusion correction when the network refines it).
    precondition=None is the identity, else a function v -> z.  Returns how
    many pairs were written (fewer if the solve converged first)."""
    import torch
    L = _lib()
    b = torch.zeros(rt.length, dtype=torch.float64, device="cuda")
    rt.rhs(out=b)
    done = [0]

    def record(w, z):
        if done[0] >= count:
            return
        k = offset + done[0]
        w = w.contiguous()
        e = z if base is None else z - base(w) + w
        e = e.contiguous()
        _capi.check(L.ouranos_rt_pc_features(rt._h, w.data_ptr(), feat_out[k].data_ptr(), None), rt._h)
        _capi.check(L.ouranos_rt_pc_target(rt._h, w.data_ptr(), e.data_ptr(), target_out[k].data_ptr()),
                    rt._h)
        done[0] += 1

    fgmres_pairs(rt, b, precondition or (lambda v: v), record, m=m, max_it=count)
    return done[0]


def learned_precondition(rt, dsa=False):
    """v -> P v through the network installed on rt (ouranos_rt_pc_apply);
    dsa=True: the network's correction added to the diffusion correction,
    P v = DSA(v) + (network part)."""
    L = _lib()

    def pc(v):
        v = v.contiguous()
        z = v.new_empty(v.shape)
        _capi.check(L.ouranos_rt_pc_apply(rt._h, v.data_ptr(), z.data_ptr()), rt._h)
        if dsa:
            z = z - v + rt.dsa_apply(v)
        return z
    return pc


def train_on_solver_pairs(n=32, maps=32, steps_per_map=60, passes=2, epochs=6, lr=3e-4, seed=7,
                          map_seed0=2000, sn=12, dsa=100, log=print):
    """Train the network to predict the diffusion correction of the residuals
    FGMRES meets on seeded thick maps.

    The pairs are (v, DSA(v)) for the solver's own Krylov vectors v -- the
    inputs of its right preconditioner -- with the diffusion correction
    solved to convergence (`dsa` CG steps): the correction is a linear,
    material-dependent, local-scale map of the scalar flux (its range is the
    diffusion length: ~12 cells in the scattering cells, ~1 in the thick
    ones), which the gated-linear network can represent.  The first
    collection pass takes the vectors of FGMRES(30) preconditioned by that
    correction; every later pass installs the network trained so far and takes
    the vectors of the learned-preconditioned FGMRES, which are the ones the
    network meets in use, and trains on all pairs so far.  Returns (net, loss history per
    epoch)."""
    import torch
    from .transport import RadiativeTransfer
    rng = np.random.default_rng(seed)
    L = _lib()
    cap = maps * steps_per_map * passes
    cells = n ** 3
    feats = torch.empty((cap, cells * FEATURES), dtype=torch.float32, device="cuda")
    targets = torch.empty((cap, cells * OUTPUTS), dtype=torch.float32, device="cuda")
    net = Network(n, n, n, seed=seed)
    rts = [RadiativeTransfer(thick_3d(seed=map_seed0 + k, n=n, sn=sn, width=10.0 * n / 64), precision="fp32")
           for k in range(maps)]
    hist = []
    filled = 0
    try:
        for rt in rts:
            rt.set_dsa(dsa)
        for rnd in range(passes):
            for rt in rts:
                if rnd:
                    install(rt, net)
                inner = learned_precondition(rt) if rnd else rt.dsa_apply
                b = torch.zeros(rt.length, dtype=torch.float64, device="cuda")
                rt.rhs(out=b)
                start = filled

                def pc(v, rt=rt, inner=inner, start=start):
                    nonlocal filled
                    if filled - start < steps_per_map:
                        v = v.contiguous()
                        e = rt.dsa_apply(v)
                        _capi.check(L.ouranos_rt_pc_features(rt._h, v.data_ptr(), feats[filled].data_ptr(),
                                                             None), rt._h)
                        _capi.check(L.ouranos_rt_pc_target(rt._h, v.data_ptr(), e.data_ptr(),
                                                           targets[filled].data_ptr()), rt._h)
                        filled += 1
                    return inner(v)

                fgmres_pairs(rt, b, pc, lambda w, z: None, max_it=steps_per_map)
                if rnd:
                    install(rt, None)
            for ep in range(epochs):
                order = rng.permutation(filled)
                rate = lr * (0.5 * (1 + math.cos(math.pi * ep / epochs))) / (1 + rnd)
                tot = 0.0
                for i in order:
                    tot += net.train_step(feats[i], targets[i], rate)
                hist.append(tot / filled)
                log("pass %d epoch %d pairs %d loss %.4e" % (rnd, ep, filled, hist[-1]))
    finally:
        for rt in rts:
            rt.close()
    return net, hist


def guess_precondition(rt):
    """v -> P v: the diffusion acceleration of rt (its set_dsa CG steps)
    started from the installed network's prediction (ouranos_rt_pc_dsa_apply)."""
    L = _lib()

    def pc(v):
        v = v.contiguous()
        z = v.new_empty(v.shape)
        _capi.check(L.ouranos_rt_pc_dsa_apply(rt._h, v.data_ptr(), z.data_ptr()), rt._h)
        return z
    return pc


def train_dsa_guess(n=32, maps=512, steps_per_map=8, passes=2, epochs=6, lr=3e-4, seed=7, map_seed0=2000,
                    sn=12, target_cg=100, inner_cg=3, log=print):
    """Train the network to predict the diffusion correction f of the
    residuals FGMRES hands its right preconditioner, for use as the initial
    guess of the diffusion CG (ouranos_rt_pc_dsa_apply).

    Maps: the seeded thick diffusive maps, seeds map_seed0 .. map_seed0 +
    maps - 1, n^3 cells of the 64^3 workload's cell width (side 10 n / 64).
    Pairs: (v, DSA(v) with target_cg CG steps) for the first steps_per_map
    Krylov vectors v of FGMRES(30) on each map's right-hand side, the
    preconditioner being the diffusion correction with inner_cg CG steps from
    a zero guess in the first pass and from the network trained so far in
    later passes (the vectors the learned solve meets).  Each pass is followed
    by `epochs` epochs of Adam over every pair collected so far.  Maps are
    visited one at a time, so memory holds one handle and the pairs.  Returns
    (net, loss history per epoch)."""
    import torch
    from .transport import RadiativeTransfer
    rng = np.random.default_rng(seed)
    L = _lib()
    cap = maps * steps_per_map * passes
    cells = n ** 3
    feats = torch.empty((cap, cells * FEATURES), dtype=torch.float32, device="cuda")
    targets = torch.empty((cap, cells * OUTPUTS), dtype=torch.float32, device="cuda")
    net = Network(n, n, n, seed=seed)
    hist = []
    filled = 0
    for rnd in range(passes):
        for k in range(maps):
            with RadiativeTransfer(thick_3d(seed=map_seed0 + k, n=n, sn=sn, width=10.0 * n / 64),
                                   precision="fp32") as rt:
                if rnd:
                    install(rt, net)
                b = torch.zeros(rt.length, dtype=torch.float64, device="cuda")
                rt.rhs(out=b)
                start = filled
                inner = guess_precondition(rt) if rnd else rt.dsa_apply

                def pc(v, rt=rt, inner=inner, start=start):
                    nonlocal filled
                    v = v.contiguous()
                    if filled - start < steps_per_map:
                        rt.set_dsa(target_cg)
                        e = rt.dsa_apply(v)
                        _capi.check(L.ouranos_rt_pc_features(rt._h, v.data_ptr(), feats[filled].data_ptr(),
                                                             None), rt._h)
                        _capi.check(L.ouranos_rt_pc_target(rt._h, v.data_ptr(), e.data_ptr(),
                                                           targets[filled].data_ptr()), rt._h)
                        filled += 1
                    rt.set_dsa(inner_cg)
                    return inner(v)

                rt.set_dsa(inner_cg)
                fgmres_pairs(rt, b, pc, lambda w, z: None, max_it=steps_per_map)
                if rnd:
                    install(rt, None)
        for ep in range(epochs):
            order = rng.permutation(filled)
            rate = lr * (0.5 * (1 + math.cos(math.pi * ep / epochs))) / (1 + rnd)
            tot = 0.0
            for i in order:
                tot += net.train_step(feats[i], targets[i], rate)
            hist.append(tot / filled)
            log("pass %d epoch %d pairs %d loss %.4e" % (rnd, ep, filled, hist[-1]))
    return net, hist


def compare_dsa_guess(net_path, n=64, seed=7000, sn=12, cgs=(2, 3, 5, 10, 20), tol=1e-8, max_it=1000):
    """FGMRES(30) with FP32 sweeps on the thick map (seed, n^3) to `tol`,
    preconditioned by the diffusion acceleration with k CG steps from a zero
    guess and from the network's prediction, for each k in cgs.  Returns
    {k: {"dsa": info, "learned": info}} (iterations, seconds, residual)."""
    from .transport import RadiativeTransfer
    out = {}
    with RadiativeTransfer(thick_3d(seed=seed, n=n, sn=sn)) as rt:
        net = Network.load(net_path, (n, n, n))
        for k in cgs:
            rt.set_dsa(k)
            row = {}
            for name in ("dsa", "learned"):
                install(rt, net if name == "learned" else None)
                method = "fgmres_learned" if name == "learned" else "fgmres_mixed"
                _, info, _ = rt.solve(method, tol=tol, max_it=max_it, restart=30, dsa=True)
                row[name] = {key: info[key] for key in ("iterations", "seconds", "residual", "converged")}
            install(rt, None)
            out[k] = row
        net.close()
    return out


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


def time_forward(n=64, reps=20, seed=1):
    """Device time (ms, CUDA events) of one network forward on an n^3 grid
    (random weights and features; the cost does not depend on the values)."""
    import torch
    net = Network(n, n, n, seed=seed)
    feat = torch.randn(n ** 3 * FEATURES, device="cuda", dtype=torch.float32,
                       generator=torch.Generator(device="cuda").manual_seed(seed))
    out = torch.empty(n ** 3 * OUTPUTS, device="cuda", dtype=torch.float32)
    for _ in range(3):
        net.forward(feat, out)
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        net.forward(feat, out)
    e.record()
    e.synchronize()
    net.close()
    return s.elapsed_time(e) / reps


if __name__ == "__main__":
    import argparse
    import json
    ap = argparse.ArgumentParser(description="time the network forward on an n^3 grid")
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--reps", type=int, default=20)
    a = ap.parse_args()
    print(json.dumps({"forward_ms": time_forward(a.n, a.reps), "grid": a.n}))
