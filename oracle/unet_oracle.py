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

def ch(l, base=16):
    """Width of level l: min(base * 2^l, 64)."""
    return min(base << l, 64)


def spec(levels=3, base=16):
    """(cin, cout, relu) of the 4L + 3 convolutions, in parameter order:
    two per encoder level, two at the bottleneck, two per decoder level from
    the deepest up, and the output convolution."""
    c = lambda l: ch(l, base)  # noqa: E731
    out = []
    for l in range(levels):
        out += [(16 if l == 0 else c(l - 1), c(l), 1), (c(l), c(l), 1)]
    out += [(c(levels - 1), c(levels), 1), (c(levels), c(levels), 1)]
    for l in range(levels - 1, -1, -1):
        up = c(levels) if l == levels - 1 else c(l)
        out += [(up + c(l), c(l), 1), (c(l), c(l - 1) if l > 0 else c(0), 1)]
    out.append((c(0), 16, 0))
    return out


SPEC = spec(3)


def param_count(levels=3, base=16):
    return sum(9 * ci * co + co for ci, co, _ in spec(levels, base))


def bf16(x, on=True):
    """Round to BF16 (round to nearest even) and back, in float64."""
    if not on:
        return np.asarray(x, np.float64)
    a = np.ascontiguousarray(x, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params, levels=3, base=16):
    out, off = [], 0
    for ci, co, _ in spec(levels, base):
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


def forward(params, x_in, rnd=True, levels=3, base=16):
    """x_in [B,H,W,in_ch] -> (output [B,H,W,16], cache)."""
    S = spec(levels, base)
    P = unpack(params, levels, base)
    Wr = [bf16(w, rnd) for w, _ in P]
    R = lambda a: bf16(a, rnd)
    B, H, W, ic = x_in.shape
    x0 = np.zeros((B, H, W, 16))
    x0[..., :ic] = x_in
    x0 = R(x0)
    c = {"x0": x0, "Wr": Wr, "levels": levels}

    def cv(k, x):
        y = conv(x, Wr[k], P[k][1])
        return R(np.maximum(y, 0.0)) if S[k][2] else y

    x = x0
    for l in range(levels):
        c["ea%d" % l] = cv(2 * l, x)
        c["eb%d" % l] = cv(2 * l + 1, c["ea%d" % l])
        x = c["p%d" % l] = R(pool(c["eb%d" % l]))
    c["ba"] = cv(2 * levels, x)
    prev = c["bb"] = cv(2 * levels + 1, c["ba"])
    for l in range(levels - 1, -1, -1):
        k = 2 * levels + 2 + 2 * (levels - 1 - l)
        c["cat%d" % l] = np.concatenate([up(prev), c["eb%d" % l]], -1)
        c["da%d" % l] = cv(k, c["cat%d" % l])
        prev = c["db%d" % l] = cv(k + 1, c["da%d" % l])
    c["out"] = cv(4 * levels + 2, prev)
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
    Wr, levels = c["Wr"], c["levels"]
    R = lambda a: bf16(a, rnd)
    grads = [None] * (4 * levels + 3)

    def layer(k, dpre, x, data_grad=True):
        grads[k] = (conv_weight_grad(dpre, x), dpre.sum(axis=(0, 1, 2)))
        return R(conv_data_grad(dpre, Wr[k])) if data_grad else None

    relu = lambda g, a: g * (a > 0)
    g = layer(4 * levels + 2, dout, c["db0"])
    g_cat = {}
    for l in range(levels):
        k = 2 * levels + 2 + 2 * (levels - 1 - l)
        if l == 0:
            dpre = relu(g, c["db0"])
        else:
            cu = c["db%d" % l].shape[-1]
            dpre = R(up_grad(g_cat[l - 1][..., :cu])) * (c["db%d" % l] > 0)
        g = layer(k + 1, dpre, c["da%d" % l])
        g_cat[l] = layer(k, relu(g, c["da%d" % l]), c["cat%d" % l])
    cb = c["bb"].shape[-1]
    g = layer(2 * levels + 1, R(up_grad(g_cat[levels - 1][..., :cb])) * (c["bb"] > 0), c["ba"])
    g_p = layer(2 * levels, relu(g, c["ba"]), c["p%d" % (levels - 1)])
    for l in range(levels - 1, -1, -1):
        cu = g_cat[l].shape[-1] - c["eb%d" % l].shape[-1]
        dpre = R(0.25 * up(g_p) + g_cat[l][..., cu:]) * (c["eb%d" % l] > 0)
        g = layer(2 * l + 1, dpre, c["ea%d" % l])
        x = c["x0"] if l == 0 else c["p%d" % (l - 1)]
        g_p = layer(2 * l, relu(g, c["ea%d" % l]), x, data_grad=l > 0)
    return np.concatenate([np.concatenate([w.reshape(-1), b]) for w, b in grads])


def loss_and_gradients(params, x_in, target, weight, oc, rnd=True, levels=3, base=16):
    out, cache = forward(params, x_in, rnd, levels, base)
    loss, dout = loss_and_grad(out, target, weight, oc, rnd)
    return loss, backward(params, cache, dout, rnd)


def init_params(in_channels, out_channels, seed, levels=3, base=16):
    """He-normal weights over the real fan-in (any generator: the tests set
    the GPU's parameters from this)."""
    rng = np.random.default_rng(seed)
    out = []
    S = spec(levels, base)
    for k, (ci, co, _) in enumerate(S):
        cin_real = in_channels if k == 0 else ci
        cout_real = out_channels if k == len(S) - 1 else co
        w = rng.standard_normal((9, co, ci)) * np.sqrt(2.0 / (9 * cin_real))
        w[:, cout_real:, :] = 0.0
        w[:, :, cin_real:] = 0.0
        out.append(w.reshape(-1))
        out.append(rng.standard_normal(co) * 0.05)
    return np.concatenate(out).astype(np.float32)
