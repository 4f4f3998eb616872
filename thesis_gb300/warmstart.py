"""Learned warm start of steady 2D channel flows (include/thesis_unet.h).

A U-Net trained on steady fields that the batched solver produces predicts
u, v and rho of a new channel geometry from its node-flag mask, Reynolds
number and inlet profile; the prediction seeds equilibrium populations and
the plain LBM iterates them to the same residual tolerance as a cold start.
The network's kernels (BF16 tensor cores) and the solver run in the CUDA
library; this module builds features and targets and drives the two.

Workload: n x m = 1024 x 256 channels (any size with the same proportions
through size_scale), D2Q9 TRT, walls at y = 0 and y = m-1 (half-way
bounce-back), 1-6 circles and rectangles, parabolic velocity inlet at x = 0
with centre-line velocity 0.05, pressure outlet rho = 1 at x = n-1,
Re = 0.05 m / nu uniform in [20, 200], FP32 storage with the collision in
storage units (deviations from the rest state keep their digits, so a
steady run reaches a 1e-6 residual).  Residual: sqrt(sum |u - u_prev|^2) /
sqrt(sum |u|^2) over fluid nodes every 100 steps (lbm_batch_residuals),
tolerance 1e-6; a run that has not met it after max_steps keeps its last
residual (the warm-start bench lists such runs' Reynolds numbers).
"""
import ctypes as C
import time

import numpy as np

from . import lattice
from . import native as N
from .batch import Batch
from .solver import Arguments

UMAX = 0.05
SCALE_U = 0.05        # u, v targets in units of the inlet centre-line velocity
SCALE_RHO = 0.01      # rho - 1 target scale
IN_CHANNELS = 4       # fluid mask, Re / 200, inlet profile, x / n
OUT_CHANNELS = 3      # u, v, rho - 1 (scaled)
RE_RANGE = (20.0, 200.0)
TOL = 1e-6


def geometry(seed, n=1024, m=256):
    return lattice.channel2d(n, m, seed=seed, size_scale=m / 256.0)


def reynolds(seed, re_range=RE_RANGE):
    """Re uniform in re_range, from SplitMix64(1,000,003 + seed)."""
    g = lattice.SplitMix64(1_000_003 + seed)
    return float(g.uniform(*re_range))


def channel_args(re, m, storage=N.STORE_F32):
    """Physics-mode channel: nu = u_max m / Re, TRT, pressure outlet."""
    return Arguments(u=UMAX, viscosity=UMAX * m / re, collision_model=N.TRT, mode=N.MODE_PHYSICS,
                     init_equilibrium=1, outlet_profile=N.OUTLET_PRESSURE, rho_out=1.0, storage=storage)


def inlet_profile(m):
    """Parabolic profile between the half-way walls at y = -1/2 and m - 1/2."""
    y = np.arange(m) + 0.5
    return 4.0 * UMAX * y * (m - y) / (m * m)


def inlet_velocity(lat):
    """Per-node u for lbm_set_inlet_velocity: the profile on every row."""
    u = np.broadcast_to(inlet_profile(lat.m)[:, None], (lat.m, lat.n))
    return np.ascontiguousarray(u, np.float32).reshape(-1)


def features(lat, re):
    """[m, n, 4]: fluid mask, Re / 200, inlet profile / u_max, x / (n - 1)."""
    m, n = lat.m, lat.n
    f = np.zeros((m, n, IN_CHANNELS), np.float32)
    f[..., 0] = (lat.node_type.reshape(m, n) == 1)
    f[..., 1] = re / 200.0
    f[..., 2] = (inlet_profile(m) / UMAX)[:, None]
    f[..., 3] = np.linspace(0.0, 1.0, n)[None, :]
    return f


def targets(lat, rho, u, v):
    """[m, n, 3] scaled fields and [m, n] loss weights (fluid nodes)."""
    m, n = lat.m, lat.n
    fl = (lat.node_type.reshape(m, n) == 1).astype(np.float32)
    t = np.zeros((m, n, OUT_CHANNELS), np.float32)
    t[..., 0] = u.reshape(m, n) / SCALE_U * fl
    t[..., 1] = v.reshape(m, n) / SCALE_U * fl
    t[..., 2] = (rho.reshape(m, n) - 1.0) / SCALE_RHO * fl
    return t, fl


def fields(lat, pred):
    """Predicted [m, n, 3] -> rho, u, v node arrays (solid nodes at rest)."""
    fl = (lat.node_type == 1)
    p = pred.reshape(-1, OUT_CHANNELS)
    u = np.where(fl, p[:, 0] * SCALE_U, 0.0).astype(np.float32)
    v = np.where(fl, p[:, 1] * SCALE_U, 0.0).astype(np.float32)
    rho = np.where(fl, 1.0 + p[:, 2] * SCALE_RHO, 1.0).astype(np.float32)
    return rho, u, v


class UNet:
    """Handle of the BF16 tensor-core U-Net (lbm_unet_*)."""

    def __init__(self, height, width, max_batch=32, seed=0, in_channels=IN_CHANNELS, out_channels=OUT_CHANNELS,
                 levels=3, base_channels=16):
        self._lib = N.lib()
        cfg = N.UnetConfig(height, width, in_channels, out_channels, max_batch, seed, levels, base_channels, 64)
        h = C.c_void_p()
        N.check_unet(self._lib.lbm_unet_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self.height, self.width, self.max_batch = height, width, max_batch
        self.in_channels, self.out_channels, self.levels = in_channels, out_channels, levels
        self.dataset_size = 0

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lbm_unet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def num_params(self):
        return int(self._lib.lbm_unet_param_count(self._h))

    def params(self):
        p = np.empty(self.num_params, np.float32)
        N.check_unet(self._lib.lbm_unet_get_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.num_params
        N.check_unet(self._lib.lbm_unet_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float))))

    def set_dataset(self, x, y, w):
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        w = np.ascontiguousarray(w, np.float32)
        fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        N.check_unet(self._lib.lbm_unet_set_dataset(self._h, int(x.shape[0]), fp(x), fp(y), fp(w)))
        self.dataset_size = int(x.shape[0])

    def train_step(self, idx, lr):
        idx = np.ascontiguousarray(idx, np.int32)
        loss = C.c_double()
        N.check_unet(self._lib.lbm_unet_train_step(self._h, int(idx.size), idx.ctypes.data_as(C.POINTER(C.c_int)),
                                                   float(lr), C.byref(loss)))
        return loss.value

    def gradients(self, idx):
        idx = np.ascontiguousarray(idx, np.int32)
        g = np.empty(self.num_params, np.float32)
        loss = C.c_double()
        N.check_unet(self._lib.lbm_unet_gradients(self._h, int(idx.size), idx.ctypes.data_as(C.POINTER(C.c_int)),
                                                  g.ctypes.data_as(C.POINTER(C.c_float)), C.byref(loss)))
        return g, loss.value

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32)
        out = np.empty(x.shape[:-1] + (self.out_channels,), np.float32)
        for s0 in range(0, x.shape[0], self.max_batch):
            k = min(self.max_batch, x.shape[0] - s0)
            N.check_unet(self._lib.lbm_unet_predict(
                self._h, k, x[s0:s0 + k].ctypes.data_as(C.POINTER(C.c_float)),
                out[s0:s0 + k].ctypes.data_as(C.POINTER(C.c_float))))
        return out

    @property
    def last_ms(self):
        return float(self._lib.lbm_unet_last_ms(self._h))

    def train(self, epochs, batch, lr=2e-3, lr_final=1e-4, seed=0, log_every=0):
        """Adam over the resident dataset, shuffled each epoch, learning rate
        decayed geometrically from lr to lr_final.  Returns the loss history."""
        rng = np.random.default_rng(seed)
        n = self.dataset_size
        batch = min(batch, n, self.max_batch)
        steps_per_epoch = max(1, n // batch)
        total = epochs * steps_per_epoch
        hist = []
        self.step_ms = []
        k = 0
        for ep in range(epochs):
            perm = rng.permutation(n)
            for s in range(steps_per_epoch):
                rate = lr * (lr_final / lr) ** (k / max(total - 1, 1))
                hist.append(self.train_step(perm[s * batch:(s + 1) * batch], rate))
                self.step_ms.append(self.last_ms)
                k += 1
            if log_every and (ep + 1) % log_every == 0:
                print("epoch %d loss %.4e" % (ep + 1, float(np.mean(hist[-steps_per_epoch:]))), flush=True)
        return np.array(hist)


def solve_batch(lats, res, init=None, tol=TOL, check_every=100, max_steps=400_000, storage=N.STORE_F32):
    """Run every channel to the residual tolerance in one batch.  init: None
    (fluid at rest, rho = 1) or a list of (rho, u, v) per domain.  Returns
    (steps, residuals, status, seconds, fields, total seconds): seconds of the
    iteration, fields[d] = (rho, u, v), and the time from batch creation to
    the fields' read-back."""
    t_all = time.perf_counter()
    args = [channel_args(r, lat.m, storage) for lat, r in zip(lats, res)]
    with Batch(lats, args) as b:
        b.init()
        for d, lat in enumerate(lats):
            b.set_inlet_velocity(d, u=inlet_velocity(lat))
            nn = lat.num_nodes
            if init is None:
                b.init_fields(d, np.ones(nn, np.float32), np.zeros(nn, np.float32), np.zeros(nn, np.float32))
            else:
                rho, u, v = init[d]
                b.init_fields(d, rho, u, v)
        t0 = time.perf_counter()
        steps, resid, rc = b.run_to_tolerance(tol, check_every, max_steps)
        secs = time.perf_counter() - t0
        out = []
        for d in range(len(lats)):
            rho, u, v, _ = b.macro(d)
            out.append((rho, u, v))
    return steps, resid, rc, secs, out, time.perf_counter() - t_all


def dataset(seeds, n=1024, m=256, chunk=512, re_range=RE_RANGE, **kw):
    """Steady fields of the channels `seeds` from the batched solver, solved
    `chunk` channels per batch: inputs [k, m, n, 4], targets [k, m, n, 3],
    weights [k, m, n] and the solves' steps and residuals; domains that did
    not reach the tolerance get weight 0."""
    seeds = list(seeds)
    tol = kw.get("tol", TOL)
    X = np.zeros((len(seeds), m, n, IN_CHANNELS), np.float32)
    Y = np.zeros((len(seeds), m, n, OUT_CHANNELS), np.float32)
    Wt = np.zeros((len(seeds), m, n), np.float32)
    steps_all, resid_all, secs = [], [], 0.0
    for c0 in range(0, len(seeds), chunk):
        part = seeds[c0:c0 + chunk]
        lats = [geometry(s, n, m) for s in part]
        res = [reynolds(s, re_range) for s in part]
        steps, resid, rc, sec, out, _ = solve_batch(lats, res, **kw)
        secs += sec
        for k, (lat, r) in enumerate(zip(lats, res)):
            d = c0 + k
            X[d] = features(lat, r)
            if resid[k] <= tol and np.all(np.isfinite(out[k][1])):
                Y[d], Wt[d] = targets(lat, *out[k])
        steps_all.append(np.asarray(steps))
        resid_all.append(np.asarray(resid))
    return X, Y, Wt, np.concatenate(steps_all), np.concatenate(resid_all), secs


def compare(unet, seeds, n=1024, m=256, tol=TOL, check_every=100, max_steps=400_000, warm_max_steps=None,
            re_range=RE_RANGE):
    """Cold start (fluid at rest) against the U-Net warm start on the same
    channels, each batch run to the tolerance.  A warm run gets at most
    warm_max_steps (default max_steps) before its channel falls back to the
    cold start.  Returns a dict with per-domain steps, wall times, the
    prediction time and the converged fields' difference
    (max |u_warm - u_cold| / u_max)."""
    seeds = list(seeds)
    lats = [geometry(s, n, m) for s in seeds]
    res = [reynolds(s, re_range) for s in seeds]
    X = np.stack([features(l, r) for l, r in zip(lats, res)])
    t0 = time.perf_counter()
    pred = unet.predict(X)
    t_pred = time.perf_counter() - t0
    init = [fields(l, p) for l, p in zip(lats, pred)]
    cold = solve_batch(lats, res, None, tol, check_every, max_steps)
    warm = solve_batch(lats, res, init, tol, check_every, warm_max_steps or max_steps)
    # channels whose warm run missed the tolerance fall back to the cold start
    miss = [d for d in range(len(lats)) if not warm[1][d] <= tol]
    t_fallback = 0.0
    if miss:
        fb = solve_batch([lats[d] for d in miss], [res[d] for d in miss], None, tol, check_every, max_steps)
        t_fallback = fb[5]
    du = []
    for d, lat in enumerate(lats):
        fl = lat.node_type == 1
        du.append(float(np.abs(warm[4][d][1] - cold[4][d][1])[fl].max() / UMAX))
    return dict(seeds=seeds, re=res, lats=lats, cold_steps=cold[0], warm_steps=warm[0], cold_res=cold[1],
                warm_res=warm[1], cold_seconds=cold[3], warm_seconds=warm[3], predict_seconds=t_pred,
                cold_total_seconds=cold[5], warm_total_seconds=warm[5] + t_pred + t_fallback,
                fallbacks=len(miss),
                converged_du=np.array(du), pred=pred, init=init, cold_fields=cold[4], warm_fields=warm[4])


def solve_with_warm_start(unet, lats, res, tol=TOL, check_every=100, max_steps=400_000, warm_max_steps=None):
    """Steady solve of every channel from the network's prediction; a domain
    whose warm run diverges or misses the tolerance within warm_max_steps
    (default max_steps) is solved again from rest, so the plain cold start is
    the fallback and the converged LBM field, not the prediction, is the
    result.  Returns (steps, residuals, fields, cold) with cold[d] True where
    the fallback ran (steps then count both runs)."""
    X = np.stack([features(l, r) for l, r in zip(lats, res)])
    pred = unet.predict(X)
    init = [fields(l, p) for l, p in zip(lats, pred)]
    steps, resid, rc, _, out, _ = solve_batch(lats, res, init, tol, check_every, warm_max_steps or max_steps)
    redo = [d for d in range(len(lats))
            if not (resid[d] <= tol and np.all(np.isfinite(out[d][1])))]
    cold = np.zeros(len(lats), bool)
    if redo:
        s2, r2, _, _, o2, _ = solve_batch([lats[d] for d in redo], [res[d] for d in redo], None, tol, check_every,
                                          max_steps)
        for k, d in enumerate(redo):
            steps[d], resid[d], out[d], cold[d] = steps[d] + s2[k], r2[k], o2[k], True
    return steps, resid, out, cold


def forward_flops(height, width, levels=3, base_channels=16):
    """Multiply-add FLOPs (2 per MAC) of one forward pass of the network."""
    ch = lambda l: min(base_channels << l, 64)
    layers = []
    for l in range(levels):
        layers += [(16 if l == 0 else ch(l - 1), ch(l), l), (ch(l), ch(l), l)]
    layers += [(ch(levels - 1), ch(levels), levels), (ch(levels), ch(levels), levels)]
    for l in range(levels - 1, -1, -1):
        up = ch(levels) if l == levels - 1 else ch(l)
        layers += [(up + ch(l), ch(l), l), (ch(l), ch(l - 1) if l > 0 else ch(0), l)]
    layers.append((ch(0), 16, 0))
    return sum(2 * 9 * ci * co * (height >> l) * (width >> l) for ci, co, l in layers)
