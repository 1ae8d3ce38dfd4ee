"""Oracle (test infrastructure only): float64 restatement of the three-level U-Net of the learned initial guess
of the 3-D pressure solve -- its forward pass and the gradients of its loss -- with the BF16 rounding of the
tensor-core operands at the same points as the CUDA path (snac_gb300/csrc/k_unet.cu), so that the GPU
network and its gradients can be compared with it.  With rnd=False every rounding is skipped, which is the
form the finite-difference check of this module uses.

The network is this project's own (the reference solves its pressure with HYPRE and has no learned part):
  E0 conv3 16->16 ReLU, pool, E1 conv3 16->32 ReLU, pool, B conv3 32->64 ReLU,
  D1 conv3 [up(B) | E1] 96->32 ReLU, D0 conv3 [up(D1) | E0] 48->16 ReLU, head 1x1 16->1.
Parameters, layer by layer: W[co][ci][tap] (tap = 9 (dz+1) + 3 (dy+1) + (dx+1)) then the biases; then the
head's 16 weights and its bias.  Arrays are (volume, channel, z, y, x).
"""
import numpy as np

CIN = (16, 16, 32, 96, 48)
COUT = (16, 32, 64, 32, 16)
TAPS = 27


def woff(l):
    return sum(CIN[j] * COUT[j] * TAPS + COUT[j] for j in range(l))


HEAD = woff(5)
NPAR = HEAD + 17


def bf16(a, on=True):
    """Round to the nearest BF16 (ties to even), returned as float64; identity when on is False."""
    if not on:
        return np.asarray(a, dtype=np.float64)
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    layers = []
    for l in range(5):
        o = woff(l)
        w = p[o:o + CIN[l] * COUT[l] * TAPS].reshape(COUT[l], CIN[l], TAPS)
        b = p[o + CIN[l] * COUT[l] * TAPS:o + CIN[l] * COUT[l] * TAPS + COUT[l]]
        layers.append((w, b))
    return layers, p[HEAD:HEAD + 16], p[HEAD + 16]


def _shifts(shape):
    n2, n1, n0 = shape
    for q in range(TAPS):
        dz, dy, dx = q // 9, (q // 3) % 3, q % 3
        yield q, (slice(dz, dz + n2), slice(dy, dy + n1), slice(dx, dx + n0))


def conv(x, w):
    """y[b, o] = sum_{c, tap} w[o, c, tap] x[b, c](cell + offset(tap)), zero outside the grid."""
    nb, c, n2, n1, n0 = x.shape
    xp = np.zeros((nb, c, n2 + 2, n1 + 2, n0 + 2))
    xp[:, :, 1:-1, 1:-1, 1:-1] = x
    y = np.zeros((nb, w.shape[0], n2, n1, n0))
    for q, (sz, sy, sx) in _shifts((n2, n1, n0)):
        y += np.einsum("oc,bczyx->bozyx", w[:, :, q], xp[:, :, sz, sy, sx], optimize=True)
    return y


def conv_input_grad(dz, w):
    """Gradient of conv(x, w) with respect to x: the convolution with the transposed, tap-mirrored weights."""
    return conv(dz, np.ascontiguousarray(w.transpose(1, 0, 2)[:, :, ::-1]))


def weight_grad(dz, x):
    """dW[o, c, tap] = sum over cells of dz[b, o](cell) x[b, c](cell + offset(tap))."""
    nb, c, n2, n1, n0 = x.shape
    xp = np.zeros((nb, c, n2 + 2, n1 + 2, n0 + 2))
    xp[:, :, 1:-1, 1:-1, 1:-1] = x
    g = np.zeros((dz.shape[1], c, TAPS))
    for q, (sz, sy, sx) in _shifts((n2, n1, n0)):
        g[:, :, q] = np.einsum("bozyx,bczyx->oc", dz, xp[:, :, sz, sy, sx], optimize=True)
    return g


def coarse_shape(shape):
    return tuple((n + 1) // 2 for n in shape)


def pool(a):
    """Mean of the 2x2x2 children, zero outside the grid (odd extents: the last window is partial)."""
    nb, c, n2, n1, n0 = a.shape
    m2, m1, m0 = coarse_shape((n2, n1, n0))
    ap = np.zeros((nb, c, 2 * m2, 2 * m1, 2 * m0))
    ap[:, :, :n2, :n1, :n0] = a
    return ap.reshape(nb, c, m2, 2, m1, 2, m0, 2).sum(axis=(3, 5, 7)) * 0.125


def unpool(g, shape):
    """Transpose of pool: each fine cell receives 1/8 of its parent's value."""
    return upsample(g, shape) * 0.125


def upsample(a, shape):
    """Nearest neighbour: the fine cell (z, y, x) takes the coarse cell (z//2, y//2, x//2)."""
    n2, n1, n0 = shape
    return a[:, :, np.arange(n2) // 2][:, :, :, np.arange(n1) // 2][:, :, :, :, np.arange(n0) // 2]


def sum_children(g, cshape):
    """Transpose of upsample: the sum over each coarse cell's children inside the fine grid."""
    nb, c, n2, n1, n0 = g.shape
    m2, m1, m0 = cshape
    gp = np.zeros((nb, c, 2 * m2, 2 * m1, 2 * m0))
    gp[:, :, :n2, :n1, :n0] = g
    return gp.reshape(nb, c, m2, 2, m1, 2, m0, 2).sum(axis=(3, 5, 7))


def network_input(x2, rnd=True):
    """x2 (nb, 2, z, y, x): residual and live mask -> the 16-channel input (channels 2..15 zero)."""
    r, live = x2[:, 0], x2[:, 1] != 0
    nb = x2.shape[0]
    inp = np.zeros((nb, 16) + x2.shape[2:])
    inp[:, 0] = np.where(live, bf16(r, rnd), 0.0)
    inp[:, 1] = live
    return inp


def forward(x2, params, rnd=True):
    """Head output c (nb, z, y, x) and the activations the gradients need."""
    layers, hw, hb = unpack(params)
    wb = [bf16(w, rnd) for w, _ in layers]
    relu = lambda v: np.maximum(v, 0.0)
    s0 = x2.shape[2:]
    s1 = coarse_shape(s0)
    inp = network_input(x2, rnd)
    a0 = bf16(relu(conv(inp, wb[0]) + layers[0][1][None, :, None, None, None]), rnd)
    p0 = bf16(pool(a0), rnd)
    a1 = bf16(relu(conv(p0, wb[1]) + layers[1][1][None, :, None, None, None]), rnd)
    p1 = bf16(pool(a1), rnd)
    a2 = bf16(relu(conv(p1, wb[2]) + layers[2][1][None, :, None, None, None]), rnd)
    x3 = np.concatenate([upsample(a2, s1), a1], axis=1)
    a3 = bf16(relu(conv(x3, wb[3]) + layers[3][1][None, :, None, None, None]), rnd)
    x4 = np.concatenate([upsample(a3, s0), a0], axis=1)
    a4 = bf16(relu(conv(x4, wb[4]) + layers[4][1][None, :, None, None, None]), rnd)
    c = hb + np.einsum("j,bjzyx->bzyx", hw, a4)
    cache = dict(inp=inp, a0=a0, p0=p0, a1=a1, p1=p1, a2=a2, x3=x3, a3=a3, x4=x4, a4=a4, wb=wb, hw=hw)
    return c, cache


def loss_and_grad(x2, target, params, rnd=True):
    """L = (1/nb) sum_b sum_live (c - t)^2 / sum_live t^2 and dL/dparams (NPAR)."""
    c, k = forward(x2, params, rnd)
    live = x2[:, 1] != 0
    nb = x2.shape[0]
    s0 = x2.shape[2:]
    s1, s2 = coarse_shape(s0), coarse_shape(coarse_shape(s0))
    tn = np.array([np.sum(np.where(live[b], target[b], 0.0) ** 2) for b in range(nb)])
    e = np.where(live, c - target, 0.0)
    L = sum(np.sum(e[b] ** 2) / tn[b] for b in range(nb) if tn[b] > 0) / nb
    sc = np.where(tn > 0, 2.0 / (nb * np.where(tn > 0, tn, 1.0)), 0.0)
    dc = e * sc[:, None, None, None]
    g = np.zeros(NPAR)
    g[HEAD:HEAD + 16] = np.einsum("bzyx,bjzyx->j", dc, k["a4"])
    g[HEAD + 16] = dc.sum()
    wb, hw = k["wb"], k["hw"]

    def put(l, dz, x):
        o = woff(l)
        n = CIN[l] * COUT[l] * TAPS
        g[o:o + n] = weight_grad(dz, x).ravel()
        g[o + n:o + n + COUT[l]] = dz.sum(axis=(0, 2, 3, 4))

    dz4 = hw[None, :, None, None, None] * dc[:, None] * (k["a4"] > 0)
    put(4, dz4, k["x4"])
    gx4 = conv_input_grad(bf16(dz4, rnd), wb[4])
    dz3 = sum_children(gx4[:, :32], s1) * (k["a3"] > 0)
    put(3, dz3, k["x3"])
    gx3 = conv_input_grad(bf16(dz3, rnd), wb[3])
    dz2 = sum_children(gx3[:, :64], s2) * (k["a2"] > 0)
    put(2, dz2, k["p1"])
    gx2 = conv_input_grad(bf16(dz2, rnd), wb[2])
    dz1 = (gx3[:, 64:] + unpool(gx2, s1)) * (k["a1"] > 0)
    put(1, dz1, k["p0"])
    gx1 = conv_input_grad(bf16(dz1, rnd), wb[1])
    dz0 = (gx4[:, 32:] + unpool(gx1, s0)) * (k["a0"] > 0)
    put(0, dz0, k["inp"])
    return L, g


def init_params(seed=1):
    """He-initialised weights (fan-in 27 cin; 27 x 2 for the first layer), zero biases, a small head."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPAR)
    for l in range(5):
        fan = 27.0 * (2 if l == 0 else CIN[l])
        n = CIN[l] * COUT[l] * TAPS
        p[woff(l):woff(l) + n] = np.sqrt(2.0 / fan) * rng.standard_normal(n)
    p[HEAD:HEAD + 16] = 0.05 * rng.standard_normal(16)
    return p
