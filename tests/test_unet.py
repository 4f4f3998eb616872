"""Warm-start U-Net (include/thesis_unet.h): the CPU oracle's backward pass
against finite differences, the GPU's BF16 tensor-core gradients and
predictions against the oracle, and training.

Tolerances: the oracle in FP64 without rounding agrees with central
differences to 1e-6 relative.  The GPU rounds weights, activations and
activation gradients to BF16 (8-bit mantissa) and accumulates in FP32; the
oracle rounds at the same places, so per-layer parameter gradients agree to
3e-2 relative (L2) and the loss to 1e-3; a BF16 rounding that falls the other
way on one side is the remaining difference.
"""
import numpy as np
import pytest

from oracle import unet_oracle as uo


def _problem(B, H, W, ic, oc, seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((B, H, W, ic)).astype(np.float32)
    t = rng.standard_normal((B, H, W, oc)).astype(np.float32)
    w = (rng.uniform(size=(B, H, W)) > 0.2).astype(np.float32)
    return x, t, w


@pytest.mark.parametrize("levels", [3, 4])
def test_oracle_matches_finite_differences(levels):
    x, t, w = _problem(1, 16, 32, 4, 3, 0)
    p = uo.init_params(4, 3, 1, levels).astype(np.float64)
    loss, g = uo.loss_and_gradients(p, x, t, w, 3, rnd=False, levels=levels)
    assert p.size == uo.param_count(levels) == g.size
    rng = np.random.default_rng(2)
    live = np.nonzero(np.abs(g) > 1e-6 * np.abs(g).max())[0]
    for i in rng.choice(live, 24, replace=False):
        e = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += e
        pm[i] -= e
        fd = (uo.loss_and_gradients(pp, x, t, w, 3, rnd=False, levels=levels)[0] -
              uo.loss_and_gradients(pm, x, t, w, 3, rnd=False, levels=levels)[0]) / (2 * e)
        assert abs(fd - g[i]) <= 1e-6 * max(abs(g[i]), 1e-3 * np.abs(g).max()), (i, fd, g[i])


def _layer_slices(levels, base=16):
    off = 0
    for ci, co, _ in uo.spec(levels, base):
        n = 9 * ci * co + co
        yield slice(off, off + n)
        off += n


@pytest.mark.gpu
@pytest.mark.parametrize("levels", [3, 4])
def test_gpu_gradients_match_oracle(levels):
    from thesis_gb300.warmstart import UNet
    B, H, W, ic, oc = 2, 16, 32, 4, 3
    x, t, w = _problem(B, H, W, ic, oc, 5)
    p = uo.init_params(ic, oc, 7, levels)
    with UNet(H, W, max_batch=B, in_channels=ic, out_channels=oc, levels=levels) as net:
        assert net.num_params == p.size
        net.set_params(p)
        np.testing.assert_array_equal(net.params(), p)
        net.set_dataset(x, t, w)
        g, loss = net.gradients([0, 1])
        pred = net.predict(x)
    ref_loss, ref_g = uo.loss_and_gradients(p, x, t, w, oc, rnd=True, levels=levels)
    assert abs(loss - ref_loss) <= 1e-3 * ref_loss
    for k, s in enumerate(_layer_slices(levels)):
        a, b = g[s].astype(np.float64), ref_g[s]
        nb = np.linalg.norm(b)
        if nb == 0:
            assert np.linalg.norm(a) == 0
            continue
        assert np.linalg.norm(a - b) <= 3e-2 * nb, (k, np.linalg.norm(a - b) / nb)
    out, _ = uo.forward(p, x, rnd=True, levels=levels)
    err = np.abs(pred - out[..., :oc]).max() / np.abs(out[..., :oc]).max()
    assert err < 2e-2, err


@pytest.mark.gpu
def test_gpu_training_reduces_loss_and_fits_a_field():
    """Regression of a smooth field from amplitude and position features: the
    loss falls by two orders of magnitude in 300 Adam steps."""
    from thesis_gb300.warmstart import UNet
    rng = np.random.default_rng(3)
    B, H, W = 8, 16, 64
    x = np.zeros((B, H, W, 2), np.float32)
    yy, xx = np.mgrid[0:H, 0:W]
    t = np.zeros((B, H, W, 1), np.float32)
    for b in range(B):
        a = rng.uniform(0.5, 2.0)
        x[b, ..., 0] = a
        x[b, ..., 1] = xx / W
        t[b, ..., 0] = a * np.sin(np.pi * yy / (H - 1)) * (xx / W)
    w = np.ones((B, H, W), np.float32)
    with UNet(H, W, max_batch=B, in_channels=2, out_channels=1, seed=4) as net:
        net.set_dataset(x, t, w)
        hist = net.train(epochs=300, batch=B, lr=3e-3, lr_final=3e-4)
        pred = net.predict(x)
    assert hist[-1] < 1e-2 * hist[0], (hist[0], hist[-1])
    assert np.abs(pred - t).max() < 0.15 * np.abs(t).max()


@pytest.mark.gpu
@pytest.mark.parametrize("levels,base", [(3, 16), (4, 32)])
def test_gpu_tcgen05_convolutions_match_mma_sync(monkeypatch, levels, base):
    """The tcgen05 convolutions (16 to 128 output channels: accumulator in
    tensor memory) against the mma.sync ones (THESIS_UNET_TC=0) on the same
    parameters and inputs: predictions and parameter gradients agree to the
    FP32 accumulation order, far inside the oracle tolerances; and the
    tcgen05 network's gradients match the FP64 oracle like the mma.sync
    network's do."""
    from thesis_gb300.warmstart import UNet
    B, H, W, ic, oc = 2, 32, 256, 4, 3
    x, t, w = _problem(B, H, W, ic, oc, 11)
    p = uo.init_params(ic, oc, 13, levels, base)
    res = {}
    for tc in ("1", "0"):
        monkeypatch.setenv("THESIS_UNET_TC", tc)
        with UNet(H, W, max_batch=B, in_channels=ic, out_channels=oc, levels=levels, base_channels=base) as net:
            assert net.num_params == p.size
            net.set_params(p)
            net.set_dataset(x, t, w)
            g, loss = net.gradients([0, 1])
            res[tc] = (net.predict(x), g, loss)
    (p1, g1, l1), (p0, g0, l0) = res["1"], res["0"]
    perr = np.abs(p1 - p0).max() / np.abs(p0).max()
    gerr = np.linalg.norm(g1 - g0) / np.linalg.norm(g0)
    print("tcgen05 vs mma.sync: prediction %.2e, gradient %.2e, loss %.3e / %.3e" % (perr, gerr, l1, l0))
    assert perr < 2e-2 and gerr < 3e-2 and abs(l1 - l0) <= 1e-3 * l0
    ref_loss, ref_g = uo.loss_and_gradients(p, x, t, w, oc, rnd=True, levels=levels, base=base)
    assert abs(l1 - ref_loss) <= 1e-3 * ref_loss
    for k, s in enumerate(_layer_slices(levels, base)):
        a, b = g1[s].astype(np.float64), ref_g[s]
        nb = np.linalg.norm(b)
        if nb > 0:
            assert np.linalg.norm(a - b) <= 3e-2 * nb, (k, np.linalg.norm(a - b) / nb)


@pytest.mark.gpu
def test_gpu_tcgen05_persistent_tiles_match_mma_sync(monkeypatch):
    """At 4 x 64 x 1024 every level-0 convolution has 2,048 row tiles of 128
    pixels, so each persistent tcgen05 CTA walks many tiles through both
    input stages and both tensor-memory accumulators, and the 128-channel
    decoder inputs take several chunks per tile.  Predictions and every
    layer's parameter gradient agree with the mma.sync kernels."""
    from thesis_gb300.warmstart import UNet
    B, H, W, ic, oc, levels, base = 4, 64, 1024, 4, 3, 4, 32
    x, t, w = _problem(B, H, W, ic, oc, 17)
    p = uo.init_params(ic, oc, 19, levels, base)
    res = {}
    for tc in ("1", "0"):
        monkeypatch.setenv("THESIS_UNET_TC", tc)
        with UNet(H, W, max_batch=B, in_channels=ic, out_channels=oc, levels=levels, base_channels=base) as net:
            net.set_params(p)
            net.set_dataset(x, t, w)
            g, loss = net.gradients(list(range(B)))
            res[tc] = (net.predict(x), g, loss)
    (p1, g1, l1), (p0, g0, l0) = res["1"], res["0"]
    perr = np.abs(p1 - p0).max() / np.abs(p0).max()
    print("persistent tcgen05 vs mma.sync: prediction %.2e, loss %.4e / %.4e" % (perr, l1, l0))
    assert perr < 2e-2 and abs(l1 - l0) <= 1e-3 * l0
    for k, s in enumerate(_layer_slices(levels, base)):
        a, b = g1[s].astype(np.float64), g0[s].astype(np.float64)
        nb = np.linalg.norm(b)
        assert nb > 0 and np.linalg.norm(a - b) <= 3e-2 * nb, (k, np.linalg.norm(a - b) / nb)


@pytest.mark.gpu
def test_gpu_tcgen05_ragged_rows_match_mma_sync(monkeypatch):
    """Widths that are not multiples of the 128-pixel tile: at 3 x 16 x 384
    the level-1 rows are 192 pixels (a full and a half tile) and level 2 and 3
    rows are shorter than one tile, so the tensor copies read past the image
    edge (zero fill) and the epilogues store only the pixels inside it."""
    from thesis_gb300.warmstart import UNet
    B, H, W, ic, oc, levels, base = 3, 16, 384, 4, 3, 3, 32
    x, t, w = _problem(B, H, W, ic, oc, 23)
    p = uo.init_params(ic, oc, 29, levels, base)
    res = {}
    for tc in ("1", "0"):
        monkeypatch.setenv("THESIS_UNET_TC", tc)
        with UNet(H, W, max_batch=B, in_channels=ic, out_channels=oc, levels=levels, base_channels=base) as net:
            net.set_params(p)
            net.set_dataset(x, t, w)
            g, loss = net.gradients(list(range(B)))
            res[tc] = (net.predict(x), g, loss)
    (p1, g1, l1), (p0, g0, l0) = res["1"], res["0"]
    assert np.abs(p1 - p0).max() < 2e-2 * np.abs(p0).max() and abs(l1 - l0) <= 1e-3 * l0
    for k, s in enumerate(_layer_slices(levels, base)):
        a, b = g1[s].astype(np.float64), g0[s].astype(np.float64)
        nb = np.linalg.norm(b)
        assert nb > 0 and np.linalg.norm(a - b) <= 3e-2 * nb, (k, np.linalg.norm(a - b) / nb)
