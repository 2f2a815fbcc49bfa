"""CPU oracle of the learned initial guess network (test infrastructure only).

A NumPy restatement of the U-Net in baorec.jl_gb300/csrc/guess_net.cu and
guess_kernels.cu: the same layer table, parameter layout and tap order, the
forward pass and a hand-derived backward pass.  With ``bf16=True`` it rounds
weights, inputs and every stored activation / activation gradient to BF16
(round to nearest even) the way the device kernels store them, and
accumulates in FP64; with ``bf16=False`` it is an exact FP64 network whose
backward pass the CPU tests check against finite differences.

Arrays are channels-last, indexed [z, y, x, c] (x fastest in memory).
Convolution geometries (tap t):
  C3: 3x3x3, stride 1, zero padding 1, t = dx + 3 dy + 9 dz, source v + d - 1
  DN: 2x2x2, stride 2, t = dx + 2 dy + 4 dz, source 2 v + d
  UP: 2x2x2 transposed, stride 2, output 2 v + p reads v through tap p
There is no counterpart in the reference package; the network is an
addition of this implementation.
"""
import numpy as np

C3, DN, UP = 0, 1, 2
TAPS = {C3: 27, DN: 8, UP: 8}
# tensor id -> (level, channels)
TENSORS = {"X": (0, 8), "A0": (0, 16), "CAT0": (0, 32), "B0": (0, 16), "C0": (0, 16), "A1": (1, 32),
           "B1": (1, 32), "CAT1": (1, 64), "D1": (1, 32), "E1": (1, 32), "A2": (2, 64), "B2": (2, 64),
           "C2": (2, 64)}
# kind, cin, cout, (in tensor, channel offset), (out tensor, channel offset)
LAYERS = [
    (C3, 8, 16, ("X", 0), ("A0", 0)), (C3, 16, 16, ("A0", 0), ("CAT0", 16)),
    (DN, 16, 32, ("CAT0", 16), ("A1", 0)), (C3, 32, 32, ("A1", 0), ("B1", 0)),
    (C3, 32, 32, ("B1", 0), ("CAT1", 32)), (DN, 32, 64, ("CAT1", 32), ("A2", 0)),
    (C3, 64, 64, ("A2", 0), ("B2", 0)), (C3, 64, 64, ("B2", 0), ("C2", 0)),
    (UP, 64, 32, ("C2", 0), ("CAT1", 0)), (C3, 64, 32, ("CAT1", 0), ("D1", 0)),
    (C3, 32, 32, ("D1", 0), ("E1", 0)), (UP, 32, 16, ("E1", 0), ("CAT0", 0)),
    (C3, 32, 16, ("CAT0", 0), ("B0", 0)), (C3, 16, 16, ("B0", 0), ("C0", 0)),
]
HEAD_IN = 16


def layout():
    """[(w offset, w shape, b offset, b size)] per layer + the head, and the total."""
    out, o = [], 0
    for kind, cin, cout, _, _ in LAYERS:
        shape = (TAPS[kind], cin, cout)
        out.append((o, shape, o + int(np.prod(shape)), cout))
        o += int(np.prod(shape)) + cout
    out.append((o, (HEAD_IN,), o + HEAD_IN, 1))
    o += HEAD_IN + 1
    return out, o


def num_params():
    return layout()[1]


def bf16_round(a):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    r = np.where(np.isnan(f), u, r)
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params, bf16):
    lay, _ = layout()
    ws, bs = [], []
    for i, (wo, shape, bo, nb) in enumerate(lay):
        w = np.asarray(params[wo:wo + int(np.prod(shape))], np.float64).reshape(shape)
        # the convolutions read BF16 weight copies; the head keeps FP32
        ws.append(bf16_round(w) if bf16 and i < len(LAYERS) else w)
        bs.append(np.asarray(params[bo:bo + nb], np.float64))
    return ws, bs


def _conv(kind, x, w, nout):
    """Gather convolution without bias: x (m,m,m,cin) -> (nout,nout,nout,cout)."""
    cout = w.shape[2]
    y = np.zeros((nout, nout, nout, cout))
    if kind == C3:
        xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
        for t in range(27):
            dx, dy, dz = t % 3, (t // 3) % 3, t // 9
            y += xp[dz:dz + nout, dy:dy + nout, dx:dx + nout, :] @ w[t]
    elif kind == DN:
        for t in range(8):
            dx, dy, dz = t & 1, (t >> 1) & 1, t >> 2
            y += x[dz::2, dy::2, dx::2, :] @ w[t]
    else:
        for t in range(8):
            px, py, pz = t & 1, (t >> 1) & 1, t >> 2
            y[pz::2, py::2, px::2, :] = x @ w[t]
    return y


def _conv_back(kind, x, w, dy):
    """(dx, dw) of the gather convolution for the output gradient dy."""
    dw = np.zeros_like(w)
    dx = np.zeros_like(x)
    if kind == C3:
        n = x.shape[0]
        xp = np.pad(x, ((1, 1), (1, 1), (1, 1), (0, 0)))
        dxp = np.zeros_like(xp)
        for t in range(27):
            dx_, dy_, dz_ = t % 3, (t // 3) % 3, t // 9
            xs = xp[dz_:dz_ + n, dy_:dy_ + n, dx_:dx_ + n, :]
            dw[t] = np.einsum("zyxi,zyxo->io", xs, dy)
            dxp[dz_:dz_ + n, dy_:dy_ + n, dx_:dx_ + n, :] += dy @ w[t].T
        dx = dxp[1:-1, 1:-1, 1:-1, :]
    elif kind == DN:
        for t in range(8):
            a, b, c = t & 1, (t >> 1) & 1, t >> 2
            dw[t] = np.einsum("zyxi,zyxo->io", x[c::2, b::2, a::2, :], dy)
            dx[c::2, b::2, a::2, :] = dy @ w[t].T
    else:
        for t in range(8):
            a, b, c = t & 1, (t >> 1) & 1, t >> 2
            g = dy[c::2, b::2, a::2, :]
            dw[t] = np.einsum("zyxi,zyxo->io", x, g)
            dx += g @ w[t].T
    return dx, dw


def forward(params, feats, n, bf16=True):
    """feats (n,n,n,8) -> (out (n,n,n), activations dict)."""
    ws, bs = unpack(params, bf16)
    rnd = bf16_round if bf16 else (lambda a: np.asarray(a, np.float64))
    act = {k: np.zeros((n >> lv,) * 3 + (ch,)) for k, (lv, ch) in TENSORS.items()}
    act["X"] = rnd(feats)
    for l, (kind, cin, cout, (ti, oi), (to, oo)) in enumerate(LAYERS):
        x = act[ti][..., oi:oi + cin]
        y = _conv(kind, x, ws[l], n >> TENSORS[to][0]) + bs[l]
        act[to][..., oo:oo + cout] = rnd(np.maximum(y, 0.0))
    out = act["C0"] @ ws[-1] + bs[-1][0]
    return out, act


def laplacian(a):
    """7-point Laplacian on the periodic mesh (cell units)."""
    return sum(np.roll(a, s, axis=ax) for ax in range(3) for s in (1, -1)) - 6.0 * a


def loss_and_grads(params, feats, target, n, bf16=True, loss="mse"):
    """Loss (MSE of the error, or of its Laplacian), head output and the flat
    parameter gradient."""
    ws, bs = unpack(params, bf16)
    rnd = bf16_round if bf16 else (lambda a: np.asarray(a, np.float64))
    out, act = forward(params, feats, n, bf16)
    N = out.size
    d = out - target
    if loss == "laplacian":
        q = laplacian(d)
        loss = float(np.mean(q * q))
        dout = 2.0 * laplacian(q) / N
    else:
        loss = float(np.mean(d * d))
        dout = 2.0 * d / N
    lay, total = layout()
    grad = np.zeros(total)
    gr = {k: np.zeros_like(v) for k, v in act.items()}
    # head
    wo, _, bo, _ = lay[-1]
    grad[wo:wo + HEAD_IN] = np.einsum("zyxc,zyx->c", act["C0"], dout)
    grad[bo] = dout.sum()
    gr["C0"] = rnd(dout[..., None] * ws[-1][None, None, None, :])
    for l in range(len(LAYERS) - 1, -1, -1):
        kind, cin, cout, (ti, oi), (to, oo) = LAYERS[l]
        y = act[to][..., oo:oo + cout]
        dy = np.where(y > 0.0, gr[to][..., oo:oo + cout], 0.0)
        x = act[ti][..., oi:oi + cin]
        dx, dw = _conv_back(kind, x, ws[l], dy)
        wo, shape, bo, nb = lay[l]
        grad[wo:wo + int(np.prod(shape))] = dw.ravel()
        grad[bo:bo + nb] = dy.sum(axis=(0, 1, 2))
        if l == 0:
            break
        accumulate = (ti, oi) in (("CAT0", 16), ("CAT1", 32))
        if accumulate:
            gr[ti][..., oi:oi + cin] = rnd(gr[ti][..., oi:oi + cin] + dx)
        else:
            gr[ti][..., oi:oi + cin] = rnd(dx)
    return loss, out, grad


def init_params(seed, head_scale=1e-3):
    """He-initialised weights (independent of the device initialiser's stream)."""
    rng = np.random.default_rng(seed)
    lay, total = layout()
    p = np.zeros(total)
    for l, (kind, cin, cout, _, _) in enumerate(LAYERS):
        wo, shape, _, _ = lay[l]
        p[wo:wo + int(np.prod(shape))] = rng.normal(0.0, np.sqrt(2.0 / (TAPS[kind] * cin)), int(np.prod(shape)))
    wo = lay[-1][0]
    p[wo:wo + HEAD_IN] = rng.normal(0.0, head_scale, HEAD_IN)
    return p
