"""CPU reference of the denoiser U-Net (TEST INFRASTRUCTURE ONLY).

A float64 numpy restatement of yapt_gb300/denoise.py's network, with BF16 rounding at the
same points as the device (weights, stored activations and activation gradients), used by the
tests to check the CUDA forward and backward passes (gradient check against the CPU oracle).
Tensors are NHWC arrays (n, h, w, c).
"""
import numpy as np

from yapt_gb300.denoise import EPS, HEAD, LAYERS, parameter_layout


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    u = np.ascontiguousarray(np.asarray(x, np.float32)).view(np.uint32).copy()
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.view(np.float32).astype(np.float64)


def conv3x3(x, w, b=None):
    """x (n,h,w,cin), w (cout,3,3,cin) -> (n,h,w,cout), zero padding."""
    n, h, wd, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    y = np.zeros((n, h, wd, w.shape[0]))
    for dy in range(3):
        for dx in range(3):
            y += np.einsum("nhwc,oc->nhwo", xp[:, dy:dy + h, dx:dx + wd, :], w[:, dy, dx, :])
    if b is not None:
        y += b
    return y


def conv3x3_wgrad(x, dy):
    """dW (cout,3,3,cin) = sum over pixels of dy x shifted x."""
    n, h, wd, cin = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    dw = np.zeros((dy.shape[3], 3, 3, cin))
    for a in range(3):
        for c in range(3):
            dw[:, a, c, :] = np.einsum("nhwo,nhwc->oc", dy, xp[:, a:a + h, c:c + wd, :])
    return dw, dy.sum(axis=(0, 1, 2))


def conv3x3_dgrad(dy, w):
    """dX = conv of dy with the spatially flipped, transposed weights."""
    wt = np.transpose(w[:, ::-1, ::-1, :], (3, 1, 2, 0))
    return conv3x3(dy, wt)


def pool(x):
    n, h, w, c = x.shape
    return x.reshape(n, h // 2, 2, w // 2, 2, c).mean(axis=(2, 4))


def pool_bwd(d):
    return np.repeat(np.repeat(d, 2, axis=1), 2, axis=2) * 0.25


def up(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up_bwd(d):
    n, h, w, c = d.shape
    return d.reshape(n, h // 2, 2, w // 2, 2, c).sum(axis=(2, 4))


def unpack(params):
    lay, _ = parameter_layout()
    P = {}
    for name, cin, cout in LAYERS:
        w0, nw, b0, nb = lay[name]
        P[name] = (bf16(params[w0:w0 + nw]).reshape(cout, 3, 3, cin), np.asarray(params[b0:b0 + nb], np.float64))
    h0 = lay["head"][0]
    P["head"] = (np.asarray(params[h0:h0 + 96], np.float64).reshape(3, 32), np.asarray(params[h0 + 96:h0 + 99], np.float64))
    return P


def forward(params, x):
    """x: (n,h,w,16) network input (BF16 values). Returns output and the stored activations."""
    P = unpack(params)
    A = {}

    def cv(name, inp):
        w, b = P[name]
        return bf16(np.maximum(conv3x3(inp, w, b), 0.0))

    A["x0"] = bf16(x)
    A["e0a"] = cv("e0a", A["x0"])
    A["e0b"] = cv("e0b", A["e0a"])
    A["p0"] = bf16(pool(A["e0b"]))
    A["e1a"] = cv("e1a", A["p0"])
    A["e1b"] = cv("e1b", A["e1a"])
    A["p1"] = bf16(pool(A["e1b"]))
    A["e2a"] = cv("e2a", A["p1"])
    A["e2b"] = cv("e2b", A["e2a"])
    A["p2"] = bf16(pool(A["e2b"]))
    A["ba"] = cv("ba", A["p2"])
    A["bb"] = cv("bb", A["ba"])
    A["cat2"] = np.concatenate([up(A["bb"]), A["e2b"]], axis=3)
    A["d2a"] = cv("d2a", A["cat2"])
    A["d2b"] = cv("d2b", A["d2a"])
    A["cat1"] = np.concatenate([up(A["d2b"]), A["e1b"]], axis=3)
    A["d1a"] = cv("d1a", A["cat1"])
    A["d1b"] = cv("d1b", A["d1a"])
    A["cat0"] = np.concatenate([up(A["d1b"]), A["e0b"]], axis=3)
    A["d0a"] = cv("d0a", A["cat0"])
    A["d0b"] = cv("d0b", A["d0a"])
    hw, hb = P["head"]
    z = np.einsum("nhwc,oc->nhwo", A["d0b"], hw) + hb + A["x0"][..., :3]
    A["z"] = z
    return np.expm1(np.minimum(z, 20.0)), A


def loss_and_gradients(params, x, target):
    """relMSE loss and its gradient wrt the flat parameter vector."""
    lay, nparams = parameter_layout()
    P = unpack(params)
    y, A = forward(params, x)
    t = target
    cnt = y.size
    loss = float(np.sum((y - t) ** 2 / (t * t + EPS)) / cnt)
    G = np.zeros(nparams)
    dz = 2.0 * (y - t) / (t * t + EPS) * np.exp(np.minimum(A["z"], 20.0)) * (A["z"] < 20.0) / cnt
    hw, hb = P["head"]
    h0 = lay["head"][0]
    G[h0:h0 + 96] = np.einsum("nhwo,nhwc->oc", dz, A["d0b"]).reshape(-1)
    G[h0 + 96:h0 + 99] = dz.sum(axis=(0, 1, 2))
    g = bf16(np.einsum("nhwo,oc->nhwc", dz, hw) * (A["d0b"] > 0))

    def back(name, inp, dy, mask=None):
        w, _ = P[name]
        dw, db = conv3x3_wgrad(inp, dy)
        w0, nw, b0, nb = lay[name]
        G[w0:w0 + nw] = dw.reshape(-1)
        G[b0:b0 + nb] = db
        dx = conv3x3_dgrad(dy, w)
        if mask is not None:
            dx = dx * (mask > 0)
        return bf16(dx)

    g = back("d0b", A["d0a"], g, A["d0a"])
    gc0 = back("d0a", A["cat0"], g)
    g = bf16(up_bwd(gc0[..., :64]) * (A["d1b"] > 0))
    g = back("d1b", A["d1a"], g, A["d1a"])
    gc1 = back("d1a", A["cat1"], g)
    g = bf16(up_bwd(gc1[..., :128]) * (A["d2b"] > 0))
    g = back("d2b", A["d2a"], g, A["d2a"])
    gc2 = back("d2a", A["cat2"], g)
    g = bf16(up_bwd(gc2[..., :256]) * (A["bb"] > 0))
    g = back("bb", A["ba"], g, A["ba"])
    g = back("ba", A["p2"], g)
    g = bf16((pool_bwd(g) + gc2[..., 256:]) * (A["e2b"] > 0))
    g = back("e2b", A["e2a"], g, A["e2a"])
    g = back("e2a", A["p1"], g)
    g = bf16((pool_bwd(g) + gc1[..., 128:]) * (A["e1b"] > 0))
    g = back("e1b", A["e1a"], g, A["e1a"])
    g = back("e1a", A["p0"], g)
    g = bf16((pool_bwd(g) + gc0[..., 64:]) * (A["e0b"] > 0))
    g = back("e0b", A["e0a"], g, A["e0a"])
    w, _ = P["e0a"]
    dw, db = conv3x3_wgrad(A["x0"], g)
    w0, nw, b0, nb = lay["e0a"]
    G[w0:w0 + nw] = dw.reshape(-1)
    G[b0:b0 + nb] = db
    return loss, G
