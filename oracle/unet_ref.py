"""FP64 numpy restatement of the learned preconditioner's U-Net, forward and
backward, for checking the GPU network (test infrastructure; the product
never imports it).

The network has no counterpart in the reference; its definition is the one
carpio_gb300/csrc/nn.cu implements: input layer 1 -> 32, encoder levels of
two 3x3 convolutions (32, 64, 128 channels) with 2x2 average pooling, a
256-channel bottleneck, decoder levels that concatenate the nearest-upsampled
coarser level with the encoder's skip and apply two 3x3 convolutions, a 1x1
output layer; ReLU after every 3x3 layer and the input layer; no biases.
Loss: sum (z - t)^2 / sum t^2.

With emulate_bf16 the activations and gradients are rounded to BF16 where
the GPU stores them, and the 3x3 weights are rounded as the GPU rounds them,
so the comparison isolates arithmetic order from storage precision.
"""
import numpy as np

C = (32, 64, 128, 256)
# (cin0, cin1, cout) of the 13 3x3 layers in parameter order
LAYERS = [(C[0], 0, C[0]), (C[0], 0, C[1]), (C[1], 0, C[1]), (C[1], 0, C[2]),
          (C[2], 0, C[2]), (C[2], 0, C[3]), (C[3], 0, C[3]), (C[3], C[2], C[2]),
          (C[2], 0, C[2]), (C[2], C[1], C[1]), (C[1], 0, C[1]), (C[1], C[0], C[0]),
          (C[0], 0, C[0])]


def offsets():
    off = [9 * C[0]]
    for ci0, ci1, co in LAYERS:
        off.append(off[-1] + 9 * co * (ci0 + ci1))
    return off


def num_params():
    return offsets()[-1] + C[0]


def bf16_round(a):
    """round to the nearest BF16 (ties to even), returned as float64"""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = ((u + 0x7FFF + lsb) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p, emulate_bf16=False):
    p = np.asarray(p, dtype=np.float64)
    off = offsets()
    w_in = p[:off[0]].reshape(9, C[0])
    ws = []
    for k, (ci0, ci1, co) in enumerate(LAYERS):
        w = p[off[k]:off[k + 1]].reshape(9, co, ci0 + ci1)
        ws.append(bf16_round(w) if emulate_bf16 else w)
    w_out = p[off[-1]:off[-1] + C[0]]
    return w_in, ws, w_out


def conv3x3(x, w):
    n, h, wd, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((n, h, wd, w.shape[1]))
    for t in range(9):
        dy, dx = divmod(t, 3)
        out += np.einsum("nhwc,oc->nhwo", xp[:, dy:dy + h, dx:dx + wd], w[t], optimize=True)
    return out


def conv3x3_bwd(x, w, g):
    """input and weight gradients of conv3x3(x, w) given the output gradient g"""
    n, h, wd, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    gxp = np.zeros_like(xp)
    gw = np.zeros_like(w)
    for t in range(9):
        dy, dx = divmod(t, 3)
        gxp[:, dy:dy + h, dx:dx + wd] += np.einsum("nhwo,oc->nhwc", g, w[t], optimize=True)
        gw[t] = np.einsum("nhwo,nhwc->oc", g, xp[:, dy:dy + h, dx:dx + wd], optimize=True)
    return gxp[:, 1:-1, 1:-1], gw


def pool(x):
    n, h, w, c = x.shape
    return x.reshape(n, h // 2, 2, w // 2, 2, c).mean(axis=(2, 4))


def pool_bwd(g):
    return np.repeat(np.repeat(g, 2, axis=1), 2, axis=2) * 0.25


def up(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up_bwd(g):
    n, h, w, c = g.shape
    return g.reshape(n, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4))


def forward(p, x, emulate_bf16=False):
    """x [n, h, w] -> (z [n, h, w], activations)"""
    q = bf16_round if emulate_bf16 else (lambda a: a)
    w_in, ws, w_out = unpack(p, emulate_bf16)
    A = {}
    A["x"] = np.asarray(x, dtype=np.float64)
    A["a0"] = q(np.maximum(conv3x3(A["x"][..., None], w_in[:, :, None]), 0))
    relu_conv = lambda t, k: q(np.maximum(conv3x3(t, ws[k]), 0))
    A["s0"] = relu_conv(A["a0"], 0)
    A["p0"] = q(pool(A["s0"]))
    A["a1"] = relu_conv(A["p0"], 1)
    A["s1"] = relu_conv(A["a1"], 2)
    A["p1"] = q(pool(A["s1"]))
    A["a2"] = relu_conv(A["p1"], 3)
    A["s2"] = relu_conv(A["a2"], 4)
    A["p2"] = q(pool(A["s2"]))
    A["a3"] = relu_conv(A["p2"], 5)
    A["b3"] = relu_conv(A["a3"], 6)
    A["u2"] = up(A["b3"])
    A["c2"] = relu_conv(np.concatenate([A["u2"], A["s2"]], axis=3), 7)
    A["d2"] = relu_conv(A["c2"], 8)
    A["u1"] = up(A["d2"])
    A["c1"] = relu_conv(np.concatenate([A["u1"], A["s1"]], axis=3), 9)
    A["d1"] = relu_conv(A["c1"], 10)
    A["u0"] = up(A["d1"])
    A["c0"] = relu_conv(np.concatenate([A["u0"], A["s0"]], axis=3), 11)
    A["d0"] = relu_conv(A["c0"], 12)
    z = A["d0"] @ w_out
    return z, A


def neumann_apply(f):
    """the all-Neumann 5-point operator with unit face coefficients, per
    image of f [n, h, w]"""
    a = np.zeros_like(f)
    d = f[:, 1:, :] - f[:, :-1, :]
    a[:, 1:, :] += d
    a[:, :-1, :] -= d
    d = f[:, :, 1:] - f[:, :, :-1]
    a[:, :, 1:] += d
    a[:, :, :-1] -= d
    return a


def loss_and_grad(p, x, t, emulate_bf16=False, loss="mse"):
    """(loss, gradient in the flat parameter layout); loss "mse":
    sum (z - t)^2 / sum t^2, "energy": (e, A e) / (t, A t) with e = z - t"""
    q = bf16_round if emulate_bf16 else (lambda a: a)
    w_in, ws, w_out = unpack(p, emulate_bf16)
    z, A = forward(p, x, emulate_bf16)
    t = np.asarray(t, dtype=np.float64)
    if loss == "energy":
        e = z - t
        if emulate_bf16:
            e = e.astype(np.float32).astype(np.float64)
        qq = np.sum(t * neumann_apply(t)) or 1.0
        value = np.sum(e * neumann_apply(e)) / qq
        dz = 2.0 * neumann_apply(e) / qq
    else:
        qq = np.sum(t * t) or 1.0
        value = np.sum((z - t) ** 2) / qq
        dz = 2.0 * (z - t) / qq
    if emulate_bf16:
        dz = dz.astype(np.float32).astype(np.float64)
    loss = value
    G = [None] * 13
    g_out = np.einsum("nhwc,nhw->c", A["d0"], dz)
    gpre = q(np.where(A["d0"] > 0, dz[..., None] * w_out, 0))       # d0

    def back(k, inp, gpre_k, mask=None, split=None):
        gx, G[k] = conv3x3_bwd(inp, ws[k], gpre_k)
        if split is not None:
            return q(gx[..., :split]), q(gx[..., split:])
        if mask is not None:
            gx = np.where(mask > 0, gx, 0)
        return q(gx)

    skip = {}
    for lvl, (kd, kc) in enumerate([(12, 11), (10, 9), (8, 7)]):
        gc = back(kd, A[f"c{lvl}"], gpre, mask=A[f"c{lvl}"])
        cat = np.concatenate([A[f"u{lvl}"], A[f"s{lvl}"]], axis=3)
        gu, skip[lvl] = back(kc, cat, gc, split=LAYERS[kc][0])
        low = A["b3"] if lvl == 2 else A[f"d{lvl + 1}"]
        gpre = q(np.where(low > 0, up_bwd(gu), 0))
    # bottleneck
    ga3 = back(6, A["a3"], gpre, mask=A["a3"])
    gp = back(5, A["p2"], ga3)
    for lvl in (2, 1, 0):
        gs = q(np.where(A[f"s{lvl}"] > 0, pool_bwd(gp) + skip[lvl], 0))
        ks = 2 * lvl
        ga = back(ks, A[f"a{lvl}"], gs, mask=A[f"a{lvl}"])
        if lvl > 0:
            gp = back(2 * lvl - 1, A[f"p{lvl - 1}"], ga)
    # input layer: a0 = relu(conv(x)), ga is already masked by a0 > 0
    _, g_in = conv3x3_bwd(A["x"][..., None], w_in[:, :, None], ga)
    grad = np.concatenate([g_in[:, :, 0].reshape(-1)] + [g.reshape(-1) for g in G] + [g_out])
    return loss, grad
