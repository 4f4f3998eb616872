"""CPU restatement of the warm-start U-Net (include/thesis_unet.h,
thesis_gb300/csrc/unet.cu): forward pass, weighted MSE loss and the
backward pass, in FP64, optionally rounding to BF16 where the GPU stores BF16
(weights, activations, pooled tensors, the output gradient and the
activation gradients), so the GPU's parameter gradients can be checked
against it.  Without rounding it is plain FP64 backpropagation, which the
tests pin with finite differences.

TEST INFRASTRUCTURE ONLY: imported by tests/ and never by the product.
"""
import numpy as np

# (cin, cout, relu) of the 15 convolutions, in parameter order
SPEC = [(16, 16, 1), (16, 16, 1), (16, 32, 1), (32, 32, 1), (32, 64, 1), (64, 64, 1), (64, 64, 1),
        (64, 64, 1), (128, 64, 1), (64, 32, 1), (64, 32, 1), (32, 16, 1), (32, 16, 1), (16, 16, 1),
        (16, 16, 0)]


def param_count():
    return sum(9 * ci * co + co for ci, co, _ in SPEC)


def bf16(x, on=True):
    """Round to BF16 (round to nearest even) and back, in float64."""
    if not on:
        return np.asarray(x, np.float64)
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    out, off = [], 0
    for ci, co, _ in SPEC:
        w = np.asarray(params[off:off + 9 * ci * co], np.float64).reshape(9, co, ci)
        off += 9 * ci * co
        b = np.asarray(params[off:off + co], np.float64)
        off += co
        out.append((w, b))
    return out


def conv(x, w, b=None):
    """3x3 convolution, zero padding: x [B,H,W,ci], w [9, co, ci]."""
    B, H, W, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((B, H, W, w.shape[1]))
    for tap in range(9):
        ky, kx = divmod(tap, 3)
        out += np.einsum("bhwc,oc->bhwo", xp[:, ky:ky + H, kx:kx + W, :], w[tap], optimize=True)
    if b is not None:
        out += b
    return out


def conv_data_grad(d, w):
    """Gradient of conv's input: d [B,H,W,co] -> [B,H,W,ci]."""
    wt = np.transpose(w[::-1], (0, 2, 1))  # tap' -> 8 - tap, [ci, co]
    return conv(d, wt)


def conv_weight_grad(d, x):
    """dW [9, co, ci] = sum_p d[p, co] x[p + tap offset, ci]."""
    B, H, W, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    g = np.zeros((9, d.shape[-1], x.shape[-1]))
    for tap in range(9):
        ky, kx = divmod(tap, 3)
        g[tap] = np.einsum("bhwo,bhwc->oc", d, xp[:, ky:ky + H, kx:kx + W, :], optimize=True)
    return g


def pool(x):
    B, H, W, C = x.shape
    return 0.25 * x.reshape(B, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


def up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2)


def up_grad(g):
    B, H, W, C = g.shape
    return g.reshape(B, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


def forward(params, x_in, rnd=True):
    """x_in [B,H,W,in_ch] -> (output [B,H,W,16], cache)."""
    P = unpack(params)
    Wr = [bf16(w, rnd) for w, _ in P]
    R = lambda a: bf16(a, rnd)
    B, H, W, ic = x_in.shape
    x0 = np.zeros((B, H, W, 16))
    x0[..., :ic] = x_in
    x0 = R(x0)
    c = {"x0": x0}

    def cv(k, x):
        y = conv(x, Wr[k], P[k][1])
        return R(np.maximum(y, 0.0)) if SPEC[k][2] else y

    c["e0a"] = cv(0, x0)
    c["e0b"] = cv(1, c["e0a"])
    c["p0"] = R(pool(c["e0b"]))
    c["e1a"] = cv(2, c["p0"])
    c["e1b"] = cv(3, c["e1a"])
    c["p1"] = R(pool(c["e1b"]))
    c["e2a"] = cv(4, c["p1"])
    c["e2b"] = cv(5, c["e2a"])
    c["p2"] = R(pool(c["e2b"]))
    c["ba"] = cv(6, c["p2"])
    c["bb"] = cv(7, c["ba"])
    c["cat2"] = np.concatenate([up(c["bb"]), c["e2b"]], -1)
    c["d2a"] = cv(8, c["cat2"])
    c["d2b"] = cv(9, c["d2a"])
    c["cat1"] = np.concatenate([up(c["d2b"]), c["e1b"]], -1)
    c["d1a"] = cv(10, c["cat1"])
    c["d1b"] = cv(11, c["d1a"])
    c["cat0"] = np.concatenate([up(c["d1b"]), c["e0b"]], -1)
    c["d0a"] = cv(12, c["cat0"])
    c["d0b"] = cv(13, c["d0a"])
    c["out"] = cv(14, c["d0b"])
    c["Wr"] = Wr
    return c["out"], c


def loss_and_grad(out, target, weight, oc, rnd=True):
    """Weighted MSE over the first oc channels and its output gradient."""
    d = out[..., :oc] - target
    sw = weight.sum()
    loss = float((weight[..., None] * d * d).sum() / (oc * sw))
    g = np.zeros_like(out)
    g[..., :oc] = 2.0 * weight[..., None] * d / (oc * sw)
    return loss, bf16(g, rnd)


def backward(params, cache, dout, rnd=True):
    """Parameter gradients in parameter order (FP64)."""
    c = cache
    Wr = c["Wr"]
    R = lambda a: bf16(a, rnd)
    grads = [None] * 15

    def layer(k, dpre, x):
        grads[k] = (conv_weight_grad(dpre, x), dpre.sum(axis=(0, 1, 2)))
        return R(conv_data_grad(dpre, Wr[k]))

    relu = lambda g, a: g * (a > 0)
    g = layer(14, dout, c["d0b"])
    g = layer(13, relu(g, c["d0b"]), c["d0a"])
    g_cat0 = layer(12, relu(g, c["d0a"]), c["cat0"])
    g = layer(11, R(up_grad(g_cat0[..., :16])) * (c["d1b"] > 0), c["d1a"])
    g_cat1 = layer(10, relu(g, c["d1a"]), c["cat1"])
    g = layer(9, R(up_grad(g_cat1[..., :32])) * (c["d2b"] > 0), c["d2a"])
    g_cat2 = layer(8, relu(g, c["d2a"]), c["cat2"])
    g = layer(7, R(up_grad(g_cat2[..., :64])) * (c["bb"] > 0), c["ba"])
    g_p2 = layer(6, relu(g, c["ba"]), c["p2"])
    g = layer(5, R(0.25 * up(g_p2) + g_cat2[..., 64:]) * (c["e2b"] > 0), c["e2a"])
    g_p1 = layer(4, relu(g, c["e2a"]), c["p1"])
    g = layer(3, R(0.25 * up(g_p1) + g_cat1[..., 32:]) * (c["e1b"] > 0), c["e1a"])
    g_p0 = layer(2, relu(g, c["e1a"]), c["p0"])
    g = layer(1, R(0.25 * up(g_p0) + g_cat0[..., 16:]) * (c["e0b"] > 0), c["e0a"])
    d0 = relu(g, c["e0a"])
    grads[0] = (conv_weight_grad(d0, c["x0"]), d0.sum(axis=(0, 1, 2)))
    return np.concatenate([np.concatenate([w.reshape(-1), b]) for w, b in grads])


def loss_and_gradients(params, x_in, target, weight, oc, rnd=True):
    out, cache = forward(params, x_in, rnd)
    loss, dout = loss_and_grad(out, target, weight, oc, rnd)
    return loss, backward(params, cache, dout, rnd)


def init_params(in_channels, out_channels, seed):
    """He-normal weights over the real fan-in (any generator: the tests set
    the GPU's parameters from this)."""
    rng = np.random.default_rng(seed)
    out = []
    for k, (ci, co, _) in enumerate(SPEC):
        cin_real = in_channels if k == 0 else ci
        cout_real = out_channels if k == 14 else co
        w = rng.standard_normal((9, co, ci)) * np.sqrt(2.0 / (9 * cin_real))
        w[:, cout_real:, :] = 0.0
        w[:, :, cin_real:] = 0.0
        out.append(w.reshape(-1))
        out.append(rng.standard_normal(co) * 0.05)
    return np.concatenate(out).astype(np.float32)
