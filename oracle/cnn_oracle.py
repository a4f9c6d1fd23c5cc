"""ORACLE -- test infrastructure only.

CPU restatement (numpy) of the learned preconditioner's network
(ouranos_gb300/csrc/cnn.cu): the same three-level 3-D U-Net of gated-linear
layers (3x3x3 convolution without bias, then a per-channel gate affine in the
pooled material features), the continuity projection of its output, the MSE
loss and the backward pass.  Accumulation is FP64; values are rounded to BF16
wherever the GPU stores a BF16 tensor (activations, weights as the tensor
cores read them, gradients between layers), so the GPU's FP32 accumulation is
the only remaining difference.  Used by tests/ to check the GPU forward
output and every parameter gradient.
"""
import numpy as np

FEATURES = 10  # input channels per cell: 8 nodal residual values, log sigma_t, ratio
OUTPUTS = 8    # output channels per cell: the nodal correction

LAYERS = [  # (cin, cout, level) in parameter order: a0 b0 a1 b1 a2 b2 c1 d1 c0 out
    (16, 16, 0), (16, 16, 0), (16, 32, 1), (32, 32, 1), (32, 32, 2),
    (32, 32, 2), (32, 32, 1), (32, 16, 1), (16, 16, 0), (16, 16, 0),
]


def n_params():
    return sum(27 * a * b + 3 * b for a, b, _ in LAYERS)


def bf16(x):
    """Round to bfloat16 (round to nearest even) and return float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    """(weights [27][cin][cout] per layer, gates [cout][3] per layer)."""
    ws, gs, off = [], [], 0
    for cin, cout, _ in LAYERS:
        n = 27 * cin * cout
        ws.append(params[off:off + n].reshape(27, cin, cout).astype(np.float64))
        off += n
    for cin, cout, _ in LAYERS:
        gs.append(params[off:off + 3 * cout].reshape(cout, 3).astype(np.float64))
        off += 3 * cout
    return ws, gs


def gamma(a, m):
    """Gate values [.., cout] of gate coefficients a [cout][3] on materials m [.., 2]."""
    return a[:, 0] + a[:, 1] * m[..., 0:1] + a[:, 2] * m[..., 1:2]


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


def project(y):
    """Continuity projection S of nodal fields y [nz][ny][nx][8] (value k at
    corner (k&1, (k>>1)&1, k>>2)): average the values sharing a mesh vertex and
    copy the average back (csrc/cnn_kernels.cuh, vertex_average/scatter)."""
    nz, ny, nx, _ = y.shape
    vs = np.zeros((nz + 1, ny + 1, nx + 1))
    cnt = np.zeros_like(vs)
    for k in range(8):
        a, b, c = k & 1, (k >> 1) & 1, k >> 2
        vs[c:c + nz, b:b + ny, a:a + nx] += y[..., k]
        cnt[c:c + nz, b:b + ny, a:a + nx] += 1
    avg = vs / cnt
    out = np.empty_like(y)
    for k in range(8):
        a, b, c = k & 1, (k >> 1) & 1, k >> 2
        out[..., k] = avg[c:c + nz, b:b + ny, a:a + nx]
    return out


def forward(params, feat, grid):
    """feat [cells][FEATURES] (x fastest) -> (output [cells][OUTPUTS], cache)."""
    nx, ny, nz = grid
    ws, gs = unpack(params)
    wq = [bf16(w) for w in ws]
    f = np.asarray(feat, dtype=np.float64).reshape(nz, ny, nx, FEATURES)
    x0 = np.zeros((nz, ny, nx, 16))
    fin = f[..., :8].astype(np.float32).astype(np.float64)
    x0[..., :8] = bf16(fin)
    x0[..., 8:] = bf16(fin - x0[..., :8])  # what the BF16 rounding lost
    m0 = f[..., 8:10].astype(np.float32).astype(np.float64)
    M = [m0, pool(m0), pool(pool(m0))]
    A = {"x0": x0}

    def layer(l, x):
        o = bf16(conv(x, wq[l], None, False))
        A["o%d" % l] = o
        return bf16(o * gamma(gs[l], M[LAYERS[l][2]]))

    A["ha0"] = layer(0, x0)
    A["s0"] = layer(1, A["ha0"])
    A["p0"] = bf16(pool(A["s0"]))
    A["ha1"] = layer(2, A["p0"])
    A["s1"] = layer(3, A["ha1"])
    A["p1"] = bf16(pool(A["s1"]))
    A["ha2"] = layer(4, A["p1"])
    A["hb2"] = layer(5, A["ha2"])
    A["u1"] = bf16(up(A["hb2"]) + A["s1"])
    A["hc1"] = layer(6, A["u1"])
    A["hd1"] = layer(7, A["hc1"])
    A["u0"] = bf16(up(A["hd1"]) + A["s0"])
    A["hc0"] = layer(8, A["u0"])
    A["out"] = conv(A["hc0"], wq[9], None, False)
    A["outg"] = A["out"] * gamma(gs[9], M[0])
    A["M"] = M
    return project(A["outg"][..., :OUTPUTS]).reshape(-1, OUTPUTS), (A, wq, gs)


def gradients(params, feat, target, grid):
    """(loss, flat gradient vector in the GPU parameter order, output)."""
    out, (A, wq, gs) = forward(params, feat, grid)
    M = A["M"]
    d = out - target.reshape(out.shape)
    loss = float(np.mean(d * d))
    g = np.zeros(A["out"].shape)
    g[..., :OUTPUTS] = project((2.0 * d / d.size).reshape(g.shape[:3] + (OUTPUTS,)))
    g = bf16(g)
    dws, dgs = [None] * 10, [None] * 10

    def gate_back(l, gx, o):
        m = M[LAYERS[l][2]]
        go = (gx * o).reshape(-1, gx.shape[3])
        mm = m.reshape(-1, 2)
        dgs[l] = np.stack([go.sum(0), (go * mm[:, 0:1]).sum(0), (go * mm[:, 1:2]).sum(0)], axis=1)
        return bf16(gx * gamma(gs[l], m))

    def back(l, x, g_o, need_in=True):
        dws[l], _ = conv_wgrad(x, g_o)
        return bf16(conv_dgrad(g_o, wq[l])) if need_in else None

    g = gate_back(9, g, A["out"])
    ga = back(9, A["hc0"], g)
    ga = gate_back(8, ga, A["o8"])
    gu0 = back(8, A["u0"], ga)
    gskip0 = gu0
    ga = gate_back(7, bf16(up_bwd(gu0)), A["o7"])
    ga = gate_back(6, back(7, A["hc1"], ga), A["o6"])
    gu1 = back(6, A["u1"], ga)
    gskip1 = gu1
    ga = gate_back(5, bf16(up_bwd(gu1)), A["o5"])
    ga = gate_back(4, back(5, A["ha2"], ga), A["o4"])
    gp1 = back(4, A["p1"], ga)
    gs1 = bf16(bf16(pool_bwd(gp1)) + gskip1)
    gs1 = gate_back(3, gs1, A["o3"])
    ga = gate_back(2, back(3, A["ha1"], gs1), A["o2"])
    gp0 = back(2, A["p0"], ga)
    gs0 = bf16(bf16(pool_bwd(gp0)) + gskip0)
    gs0 = gate_back(1, gs0, A["o1"])
    ga = gate_back(0, back(1, A["ha0"], gs0), A["o0"])
    back(0, A["x0"], ga, need_in=False)
    flat = np.concatenate([w.reshape(-1) for w in dws] + [a.reshape(-1) for a in dgs])
    return loss, flat, out
