"""Colour-gradient two-phase D3Q19: the oracle pinned against the reference's
3D collision kernels (gpuCollBgkwGC3D / gpuCollEnhancedBgkwGC3D run on the
host, oracle/_ref), oracle invariants, and the CUDA path (lbm_cg_create3d)
against the oracle.

The reference computes the 3D colour gradient one-sided on the faces, zero
on edges and corners and, with the 104-point stencil, zero on the layer next
to the faces (its direction maps, GpuInit.cu:262-321); this path wraps
periodically, so the pin compares nodes at least one (two for the 104-point
stencil) away from every face, where the reference's map selects the full
stencil."""
import numpy as np
import pytest

from oracle import pyoracle as po
from thesis_gb300 import multiphase as mp

COMBOS = [(ho, enh) for ho in (0, 1) for enh in (0, 1)]


def _collide_inputs(n, m, h, seed):
    rng = np.random.default_rng(seed)
    nn = n * m * h
    idx = np.arange(nn)
    i, j, k = idx % n, (idx // n) % m, idx // (n * m)
    phi = np.tanh((np.sqrt((i - n / 2) ** 2 + (j - m / 2) ** 2 + (k - h / 2) ** 2) - n / 4) / 2.0)
    r_rho = 0.5 * (1 - phi) + 0.01 * rng.random(nn)
    b_rho = 0.5 * (1 + phi) + 0.01 * rng.random(nn)
    rho = r_rho + b_rho
    u, v, w = (0.02 * rng.standard_normal(nn) for _ in range(3))
    f = rng.random((19, nn)) * rho[None, :] / 9.5
    return rho, r_rho, b_rho, u, v, w, f


@pytest.mark.parametrize("ho,enh", COMBOS)
@pytest.mark.parametrize("fp64", [True, False])
def test_cg3d_collision_pinned_to_reference(ho, enh, fp64):
    if po.ref_lib(fp64) is None:
        pytest.skip("reference kernels not built (oracle/_ref)")
    n, m, h = 14, 12, 11
    p = po.cg_params(high_order=ho, enhanced=enh, r_viscosity=0.5, b_viscosity=0.2, beta=0.99, A=0.01,
                     r_alpha=0.5, b_alpha=4 / 9)
    orc, ref = po.cg3_collide_pair(n, m, h, p, *_collide_inputs(n, m, h, 3 + ho + 2 * enh), fp64=fp64)
    idx = np.arange(n * m * h)
    i, j, k = idx % n, (idx // n) % m, idx // (n * m)
    e = 2 if ho else 1
    interior = (i >= e) & (i < n - e) & (j >= e) & (j < m - e) & (k >= e) & (k < h - e)
    assert np.all(ref[2][interior] == 0)  # the reference's full-stencil nodes
    for a, b in ((orc[0], ref[0]), (orc[1], ref[1])):
        d = np.abs(a[:, interior] - b[:, interior]).max()
        if fp64:
            # the 18-neighbour sums run in the reference's order (bit-exact);
            # the 104-point sums run in another order
            assert d <= (0.0 if not ho else 2e-16), d
        else:
            # FP32: the reference promotes a few products to FP64 (2.0 * u)
            assert d <= 2.4e-7, d


def test_cg3d_oracle_conserves_colour_mass():
    a = mp.CgArguments(bubble_radius=0.3, A=0.005, beta=0.99)
    n, m, h = 14, 12, 10
    r0, b0 = mp.create_bubble3d(n, m, h, a)
    p = po.cg_params(A=a.A, beta=a.beta, high_order=1, enhanced=1)
    r = po.run_oracle_cg3(n, m, h, p, r0, b0, 30, fp64=True, extra_collide=True)
    assert r.rc == 0
    # the extra collision conserves each colour's mass too
    assert abs(r.rfc.sum() - r0.sum()) < 1e-10 * r0.sum()
    assert abs(r.bfc.sum() - b0.sum()) < 1e-10 * b0.sum()
    assert np.all(r.rr + r.br > 0)


def test_create_bubble3d():
    a = mp.CgArguments(bubble_radius=0.25, r_density=1.0, b_density=0.5)
    n = 12
    r, b = mp.create_bubble3d(n, n, n, a)
    assert r.shape == (19, n ** 3)
    centre = 6 + n * (6 + n * 6)
    np.testing.assert_allclose(r[:, centre].sum(), 1.0)
    assert r[0, centre] == 0 and np.all(b[:, centre] == 0)
    np.testing.assert_allclose(b[:, 0].sum(), 0.5)
    np.testing.assert_allclose(mp.rest_weights3d(0.3).sum(), 1.0)
    lap = np.array([10.0, 10.0, 9.0, 10.0, 0.0])
    dp = mp.laplace_pressure_jump3d(lap, mp.CgArguments(r_alpha=0.2, b_alpha=0.4))
    assert abs(dp - (0.5 * 0.8 * 1.0 - 0.5 * 0.6 * 0.9)) < 1e-15


def _gpu_case(n, m, h, ho, enh, seed=3):
    a = mp.CgArguments(bubble_radius=0.3, A=0.01, beta=0.99, r_viscosity=0.3, b_viscosity=0.1,
                       r_alpha=0.5, b_alpha=4 / 9, high_order=bool(ho), enhanced_distrib=bool(enh),
                       control_param=0.9)
    r0, b0 = mp.create_bubble3d(n, m, h, a)
    rng = np.random.default_rng(seed)
    r0 = r0 * (1 + 0.01 * rng.random(r0.shape))
    b0 = b0 * (1 + 0.01 * rng.random(b0.shape))
    p = po.cg_params(r_density=a.r_density, b_density=a.b_density, r_alpha=a.r_alpha, b_alpha=a.b_alpha,
                     r_viscosity=a.r_viscosity, b_viscosity=a.b_viscosity, beta=a.beta, A=a.A,
                     g_limit=a.g_limit, control_param=a.control_param, high_order=ho, enhanced=enh)
    return a, p, r0.astype(np.float32).astype(np.float64), b0.astype(np.float32).astype(np.float64)


@pytest.mark.gpu
@pytest.mark.parametrize("ho,enh", COMBOS)
def test_cg3d_gpu_matches_oracle(ho, enh):
    n, m, h, steps = 24, 20, 18, 30
    a, p, r0, b0 = _gpu_case(n, m, h, ho, enh)
    orc = po.run_oracle_cg3(n, m, h, p, r0, b0, steps, fp64=False, extra_collide=True)
    assert orc.rc == 0
    with mp.CgSolver(n, m, a, h=h) as s:
        s.init(r0, b0)
        s.step(steps, write_macro=True)
        rf, bf = s.populations()
        rr, br, u, v, w = s.macro()
        lap, rc = s.laplace()
    assert rc == 0
    # FP32, another operation order and FMA contraction on the GPU
    tol = 2e-5
    for got, want in ((rf, orc.rfc), (bf, orc.bfc), (rr, orc.rr), (br, orc.br), (u, orc.u), (v, orc.v),
                      (w, orc.w)):
        assert np.abs(got - want).max() < tol
    assert abs(lap[1] - orc.laplace[1]) <= 2 and abs(lap[3] - orc.laplace[3]) <= 2
    np.testing.assert_allclose(lap[4], orc.laplace[4], rtol=1e-3, atol=1e-6)


@pytest.mark.gpu
def test_cg3d_gpu_mass_conservation_and_refusals():
    from thesis_gb300 import native as N
    n, m, h, steps = 64, 48, 40, 300
    a = mp.CgArguments(bubble_radius=0.25, A=0.005, beta=0.99, high_order=True)
    r0, b0 = mp.create_bubble3d(n, m, h, a)
    with mp.CgSolver(n, m, a, h=h) as s:
        assert s._lib.lbm_cg_q(s._h) == 19
        s.init(r0, b0)
        s.step(steps, write_macro=True)
        rf, bf = s.populations()
        lap, rc = s.laplace()
    assert rc == 0
    assert abs(rf.astype(np.float64).sum() - r0.sum()) < 1e-4 * r0.sum()
    assert abs(bf.astype(np.float64).sum() - b0.sum()) < 1e-4 * b0.sum()
    assert lap[4] < 0.05
    with pytest.raises(N.LbmError):
        mp.CgSolver(16, 16, a, h=4)


@pytest.mark.gpu
def test_cg3d_gpu_laplace_law():
    """A static 3D drop obeys Laplace's law Delta p = 2 sigma / R: the total
    pressure (1 - alpha)/2 rho between the drop's core and the far field,
    times R/2, is the same for R = 8 and 12 (within 10 %) and within 15 % of
    the prediction 4A/(9 omega) (Iterate3D.cu:230; the FP64 oracle gives
    +8.5 % at R = 5 and 7), and vanishes without the perturbation.  (The
    reference's own 3D check, calculateSurfaceTension3D, takes R Delta p
    from one colour's density per phase.)"""
    n, steps = 48, 2000
    idx = np.arange(n ** 3)
    x, y, z = idx % n, (idx // n) % n, idx // (n * n)
    dist = np.sqrt((x - (n - 1) / 2) ** 2 + (y - (n - 1) / 2) ** 2 + (z - (n - 1) / 2) ** 2)
    sigma = {}
    for A in (0.005, 0.0):
        for R in (8, 12):
            a = mp.CgArguments(A=A, beta=0.7, control_param=0.9)
            r0, b0 = mp.create_bubble3d(n, n, n, a, radius_nodes=R)
            with mp.CgSolver(n, n, a, h=n) as s:
                s.init(r0, b0)
                s.step(steps, write_macro=True)
                rr, br, _, _, _ = s.macro()
            rho = rr.astype(np.float64) + br
            dp = 0.5 * (1 - a.r_alpha) * (rho[dist < R / 2].mean() - rho[dist > R + 6].mean())
            sigma[(A, R)] = dp * R / 2
    assert abs(sigma[(0.0, 8)]) < 1e-5 and abs(sigma[(0.0, 12)]) < 1e-5, sigma
    s8, s12 = sigma[(0.005, 8)], sigma[(0.005, 12)]
    pred = mp.predicted_surface_tension(mp.CgArguments(A=0.005))
    assert abs(s8 - s12) < 0.1 * pred, (s8, s12)
    assert abs(s8 - pred) < 0.15 * pred and abs(s12 - pred) < 0.15 * pred, (s8, s12, pred)
    print("3D Laplace: sigma = R dp / 2 = %.4e (R 8), %.4e (R 12); predicted %.4e" % (s8, s12, pred))
