"""ORACLE -- test infrastructure only.

CPU restatement (numpy) of the learned preconditioner's network
(ouranos_gb300/csrc/cnn.cu): the same three-level 3-D U-Net, forward pass,
MSE loss and backward pass.  Accumulation is FP64; values are rounded to
BF16 wherever the GPU stores a BF16 tensor (activations, weights as the
tensor cores read them, gradients between layers), so the GPU's FP32
accumulation is the only remaining difference.  Used by tests/ to check the
GPU forward output and every parameter gradient.
"""
import numpy as np

LAYERS = [  # (cin, cout, relu, level) in parameter order: a0 b0 a1 b1 a2 b2 c1 d1 c0 out
    (16, 16, True, 0), (16, 16, True, 0), (16, 32, True, 1), (32, 32, True, 1),
    (32, 32, True, 2), (32, 32, True, 2), (32, 32, True, 1), (32, 16, True, 1),
    (16, 16, True, 0), (16, 16, False, 0),
]


def bf16(x):
    """Round to bfloat16 (round to nearest even) and return float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    ws, bs, off = [], [], 0
    for cin, cout, _, _ in LAYERS:
        n = 27 * cin * cout
        ws.append(params[off:off + n].reshape(27, cin, cout).astype(np.float64))
        off += n
    for cin, cout, _, _ in LAYERS:
        bs.append(params[off:off + cout].astype(np.float64))
        off += cout
    return ws, bs


def _taps():
    return [(t % 3 - 1, (t // 3) % 3 - 1, t // 9 - 1) for t in range(27)]


def conv(x, w, b, relu):
    """x [nz,ny,nx,cin] -> [nz,ny,nx,cout]; w [27][cin][cout] (BF16-rounded)."""
    nz, ny, nx, _ = x.shape
    xp = np.zeros((nz + 2, ny + 2, nx + 2, x.shape[3]))
    xp[1:-1, 1:-1, 1:-1] = x
    out = np.zeros((nz, ny, nx, w.shape[2]))
    for t, (dx, dy, dz) in enumerate(_taps()):
        sl = xp[1 + dz:1 + dz + nz, 1 + dy:1 + dy + ny, 1 + dx:1 + dx + nx]
        out += sl @ w[t]
    if b is not None:
        out += b
    return np.maximum(out, 0.0) if relu else out


def conv_dgrad(g, w):
    """adjoint of conv (no bias): g [.., cout] -> [.., cin]"""
    nz, ny, nx, _ = g.shape
    gp = np.zeros((nz + 2, ny + 2, nx + 2, g.shape[3]))
    gp[1:-1, 1:-1, 1:-1] = g
    out = np.zeros((nz, ny, nx, w.shape[1]))
    for t, (dx, dy, dz) in enumerate(_taps()):
        sl = gp[1 - dz:1 - dz + nz, 1 - dy:1 - dy + ny, 1 - dx:1 - dx + nx]
        out += sl @ w[t].T
    return out


def conv_wgrad(x, g):
    nz, ny, nx, cin = x.shape
    xp = np.zeros((nz + 2, ny + 2, nx + 2, cin))
    xp[1:-1, 1:-1, 1:-1] = x
    dw = np.zeros((27, cin, g.shape[3]))
    for t, (dx, dy, dz) in enumerate(_taps()):
        sl = xp[1 + dz:1 + dz + nz, 1 + dy:1 + dy + ny, 1 + dx:1 + dx + nx]
        dw[t] = sl.reshape(-1, cin).T @ g.reshape(-1, g.shape[3])
    return dw, g.reshape(-1, g.shape[3]).sum(axis=0)


def pool(x):
    nz, ny, nx, c = x.shape
    return x.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, c).mean(axis=(1, 3, 5))


def pool_bwd(g):
    return np.repeat(np.repeat(np.repeat(g, 2, 0), 2, 1), 2, 2) * 0.125


def up(x):
    return np.repeat(np.repeat(np.repeat(x, 2, 0), 2, 1), 2, 2)


def up_bwd(g):
    nz, ny, nx, c = g.shape
    return g.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, c).sum(axis=(1, 3, 5))


def forward(params, feat, grid):
    """feat [cells][3] (x fastest) -> (output [cells], cache)."""
    nx, ny, nz = grid
    ws, bs = unpack(params)
    wq = [bf16(w) for w in ws]
    x0 = np.zeros((nz, ny, nx, 16))
    x0[..., :3] = bf16(feat.reshape(nz, ny, nx, 3))
    A = {}
    A["x0"] = x0
    A["ha0"] = bf16(conv(x0, wq[0], bs[0], True))
    A["s0"] = bf16(conv(A["ha0"], wq[1], bs[1], True))
    A["p0"] = bf16(pool(A["s0"]))
    A["ha1"] = bf16(conv(A["p0"], wq[2], bs[2], True))
    A["s1"] = bf16(conv(A["ha1"], wq[3], bs[3], True))
    A["p1"] = bf16(pool(A["s1"]))
    A["ha2"] = bf16(conv(A["p1"], wq[4], bs[4], True))
    A["hb2"] = bf16(conv(A["ha2"], wq[5], bs[5], True))
    A["u1"] = bf16(up(A["hb2"]) + A["s1"])
    A["hc1"] = bf16(conv(A["u1"], wq[6], bs[6], True))
    A["hd1"] = bf16(conv(A["hc1"], wq[7], bs[7], True))
    A["u0"] = bf16(up(A["hd1"]) + A["s0"])
    A["hc0"] = bf16(conv(A["u0"], wq[8], bs[8], True))
    A["out"] = conv(A["hc0"], wq[9], bs[9], False)
    return A["out"][..., 0].reshape(-1), (A, wq)


def gradients(params, feat, target, grid):
    """(loss, flat gradient vector in the GPU parameter order)."""
    out, (A, wq) = forward(params, feat, grid)
    V = out.size
    d = out - target
    loss = float(np.mean(d * d))
    g = np.zeros(A["out"].shape)
    g[..., 0] = (2.0 * d / V).reshape(g.shape[:3])
    g = bf16(g)
    dws, dbs = [None] * 10, [None] * 10

    def back(l, x, gout, need_in=True):
        dws[l], dbs[l] = conv_wgrad(x, gout)
        return bf16(conv_dgrad(gout, wq[l])) if need_in else None

    def mask(a, g):
        return np.where(a > 0, g, 0.0)

    ga = back(9, A["hc0"], g)
    ga = mask(A["hc0"], ga)
    gu0 = back(8, A["u0"], ga)
    gskip0 = gu0
    ga = mask(A["hd1"], bf16(up_bwd(gu0)))
    ga = mask(A["hc1"], back(7, A["hc1"], ga))
    gu1 = back(6, A["u1"], ga)
    gskip1 = gu1
    ga = mask(A["hb2"], bf16(up_bwd(gu1)))
    ga = mask(A["ha2"], back(5, A["ha2"], ga))
    gp1 = back(4, A["p1"], ga)
    gs1 = bf16(bf16(pool_bwd(gp1)) + gskip1)
    gs1 = mask(A["s1"], gs1)
    ga = mask(A["ha1"], back(3, A["ha1"], gs1))
    gp0 = back(2, A["p0"], ga)
    gs0 = bf16(bf16(pool_bwd(gp0)) + gskip0)
    gs0 = mask(A["s0"], gs0)
    ga = mask(A["ha0"], back(1, A["ha0"], gs0))
    back(0, A["x0"], ga, need_in=False)
    flat = np.concatenate([w.reshape(-1) for w in dws] + [b for b in dbs])
    return loss, flat, out
