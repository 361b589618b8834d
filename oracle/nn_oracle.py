"""FP64 numpy restatement of the learned right preconditioner's network.

TEST INFRASTRUCTURE ONLY: the CUDA network (picpp_gb300/csrc/nn*.cu) is
checked against this module (forward output, loss, every parameter
gradient); nothing in the product imports it.  The network has no
counterpart in the reference (PIC++ solves the implicit Maxwell system
with plain GMRES, PIC++/specialmath.cpp:367-671); this module is the
definition the GPU kernels follow.

Architecture: a 3-level encoder-decoder of 3x3x3 convolutions (zero
padding 1), 16/32/64 channels, 2x2x2 average pooling down, nearest
upsampling with skip concatenation up, no activation (every layer linear:
the preconditioner z = r + s net(r / s, mu) is then a fixed linear operator
for a fixed mu).  The code below keeps a per-layer ReLU flag (all False).
Activations are NDHWC; input channels 0-2 carry the scaled residual, 3-5
the mu diagonal (xx, yy, zz), 6-15 are zero; output channels 0-2 are the
scaled correction, 3-15 are zero padding.

Parameters are one flat FP32 vector, per layer in LAYERS order: the weights
W[27][cout][cin] (tap = (kd*3+kh)*3+kw) followed by the bias b[cout]; the
last entry is the preconditioner's identity gate g (z = g r + s net(r / s,
mu)), which acts outside the network (its gradient here is 0).
"""
import numpy as np

LAYERS = [  # name, cin, cout, relu
    ("e0a", 16, 16, False), ("e0b", 16, 16, False),
    ("e1a", 16, 32, False), ("e1b", 32, 32, False),
    ("e2a", 32, 64, False), ("e2b", 64, 64, False),
    ("d1a", 96, 32, False), ("d1b", 32, 32, False),
    ("d0a", 48, 16, False), ("d0b", 16, 16, False),
    ("head", 16, 16, False),
]
IN_CH, OUT_CH = 6, 3


def layer_offsets():
    """Per layer (name, cin, cout, weight offset, bias offset) and the
    parameter count (the layers plus the gate slot at the end)."""
    off, out = 0, []
    for name, ci, co, _ in LAYERS:
        out.append((name, ci, co, off, off + 27 * co * ci))
        off += 27 * co * ci + co
    return out, off + 1


def n_params():
    return layer_offsets()[1]


def unpack(p):
    offs, _ = layer_offsets()
    return {name: (p[w0:b0].reshape(27, co, ci).astype(np.float64), p[b0:b0 + co].astype(np.float64))
            for name, ci, co, w0, b0 in offs}


def bf16_round(a):
    """Nearest BF16 value (ties to even) of every element, as FP64."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _ident(a):
    return a


def flops_per_voxel():
    """Multiply-adds x 2 per full-resolution voxel (padded channel counts)."""
    lvl = {"e0a": 0, "e0b": 0, "e1a": 1, "e1b": 1, "e2a": 2, "e2b": 2, "d1a": 1, "d1b": 1, "d0a": 0, "d0b": 0,
           "head": 0}
    return sum(2 * 27 * ci * co / 8 ** lvl[n] for n, ci, co, _ in LAYERS)


def _pad(x):
    return np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))


def _taps():
    for kd in range(3):
        for kh in range(3):
            for kw in range(3):
                yield (kd * 3 + kh) * 3 + kw, kd, kh, kw


def conv(x, W, b):
    N, D, H, Wd, _ = x.shape
    xp = _pad(x)
    y = np.broadcast_to(b, (N, D, H, Wd, W.shape[1])).copy()
    for t, kd, kh, kw in _taps():
        y += xp[:, kd:kd + D, kh:kh + H, kw:kw + Wd, :] @ W[t].T
    return y


def conv_bwd(x, W, gy):
    """Gradients of conv(x, W, b) given dL/dy: (dx, dW, db)."""
    N, D, H, Wd, _ = x.shape
    xp = _pad(x)
    dxp = np.zeros_like(xp)
    dW = np.zeros_like(W)
    for t, kd, kh, kw in _taps():
        xs = xp[:, kd:kd + D, kh:kh + H, kw:kw + Wd, :]
        dW[t] = np.einsum("ndhwo,ndhwi->oi", gy, xs)
        dxp[:, kd:kd + D, kh:kh + H, kw:kw + Wd, :] += gy @ W[t]
    return dxp[:, 1:-1, 1:-1, 1:-1, :], dW, gy.sum(axis=(0, 1, 2, 3))


def pool(x):
    N, D, H, W, C = x.shape
    return x.reshape(N, D // 2, 2, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4, 6))


def pool_bwd(g):
    return up(g) / 8.0


def up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2).repeat(2, axis=3)


def up_bwd(g):
    N, D, H, W, C = g.shape
    return g.reshape(N, D // 2, 2, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4, 6))


def forward(p, x0, keep=False, bf16=False):
    """bf16=True rounds like the device: weights, every stored activation
    (not the FP32 head output) and, in loss_and_grad, every back-propagated
    pre-activation gradient to BF16."""
    R = bf16_round if bf16 else _ident
    P = unpack(p)
    acts = {"x0": x0}

    def cv(name, x):
        W, b = P[name]
        y = conv(x, R(W), b)
        relu = dict((n, r) for n, _, _, r in LAYERS)[name]
        if relu:
            y = np.maximum(y, 0.0)
        if name != "head":
            y = R(y)
        acts[name] = y
        return y

    e0 = cv("e0b", cv("e0a", x0))
    acts["p1"] = R(pool(e0))
    e1 = cv("e1b", cv("e1a", acts["p1"]))
    acts["p2"] = R(pool(e1))
    e2 = cv("e2b", cv("e2a", acts["p2"]))
    acts["c1"] = np.concatenate([up(e2), e1], axis=-1)
    d1 = cv("d1b", cv("d1a", acts["c1"]))
    acts["c0"] = np.concatenate([up(d1), e0], axis=-1)
    d0 = cv("d0b", cv("d0a", acts["c0"]))
    out = cv("head", d0)
    return (out, acts) if keep else out


def loss_and_grad(p, x0, target, bf16=False):
    """L = mean over voxels and the 3 output channels of (out - target)^2;
    returns (L, dL/dp as a flat FP64 vector in the parameter layout)."""
    R = bf16_round if bf16 else _ident
    out, a = forward(p, x0, keep=True, bf16=bf16)
    nvox = out.shape[0] * out.shape[1] * out.shape[2] * out.shape[3]
    diff = out[..., :OUT_CH] - target
    L = float((diff ** 2).sum() / (nvox * OUT_CH))
    g = np.zeros_like(out)
    g[..., :OUT_CH] = 2.0 * diff / (nvox * OUT_CH)
    P = unpack(p)
    grads = {}

    def back(name, x, gy):
        relu = dict((n, r) for n, _, _, r in LAYERS)[name]
        if relu:
            gy = gy * (a[name] > 0)
        dx, dW, db = conv_bwd(x, R(P[name][0]), R(gy))
        grads[name] = (dW, db)
        return dx

    g_d0 = back("head", a["d0b"], g)
    g_c0 = back("d0a", a["c0"], back("d0b", a["d0a"], g_d0))
    c_lo = a["d1b"].shape[-1]
    g_d1, g_e0 = up_bwd(g_c0[..., :c_lo]), g_c0[..., c_lo:]
    g_c1 = back("d1a", a["c1"], back("d1b", a["d1a"], g_d1))
    c_lo = a["e2b"].shape[-1]
    g_e2, g_e1 = up_bwd(g_c1[..., :c_lo]), g_c1[..., c_lo:]
    g_p2 = back("e2a", a["p2"], back("e2b", a["e2a"], g_e2))
    g_e1 = g_e1 + pool_bwd(g_p2)
    g_p1 = back("e1a", a["p1"], back("e1b", a["e1a"], g_e1))
    g_e0 = g_e0 + pool_bwd(g_p1)
    back("e0a", a["x0"], back("e0b", a["e0a"], g_e0))
    offs, n = layer_offsets()
    flat = np.zeros(n)
    for name, ci, co, w0, b0 in offs:
        flat[w0:b0] = grads[name][0].reshape(-1)
        flat[b0:b0 + co] = grads[name][1]
    return L, flat


def init_params(seed):
    """He-normal weights on the real input channels, zero biases; the
    padded input channels of e0a and the padded outputs of the head stay 0."""
    rng = np.random.default_rng(seed)
    offs, n = layer_offsets()
    p = np.zeros(n, dtype=np.float32)
    for name, ci, co, w0, b0 in offs:
        cin_real = IN_CH if name == "e0a" else ci
        cout_real = OUT_CH if name == "head" else co
        W = np.zeros((27, co, ci))
        W[:, :cout_real, :cin_real] = rng.standard_normal((27, cout_real, cin_real)) * np.sqrt(2.0 / (27 * cin_real))
        p[w0:b0] = W.reshape(-1)
    return p
