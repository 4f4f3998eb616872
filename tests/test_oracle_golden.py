"""The oracle restatement against golden outputs of the reference's own
kernels (tests/golden/reference_runs.npz, made by tests/golden/make_golden.py).
Runs on every machine; no GPU."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_runs.npz")


@pytest.fixture(scope="module")
def golden():
    return np.load(GOLDEN)


@pytest.mark.parametrize("case", make_golden.cases(), ids=lambda c: c[0])
def test_oracle_matches_reference_golden(oracle, golden, case):
    name, spec, kw, steps = case
    lat = make_golden.make_lattice(spec)
    assert bytes(golden[name + "/lattice_sha256"]).decode() == make_golden.bc_hash(lat), \
        "lattice builder changed since the fixture was made"
    r = oracle.run_oracle(lat, steps, fp64=False, **kw, **make_golden.link_q_kwargs(lat, kw, True))
    assert r.rc == 0
    np.testing.assert_array_equal(r.mask, golden[name + "/mask"])
    np.testing.assert_array_equal(r.stream, golden[name + "/stream"])
    # FP32 restatement in the reference's expression order, no FMA contraction:
    # bit-identical on x86-64; 1e-6 allows another host's libm-free rounding.
    for k in ("f", "fc"):
        g = golden[name + "/" + k].astype(np.float64)
        assert np.abs(getattr(r, k) - g).max() <= 1e-6 * max(1.0, np.abs(g).max()), k
    for k in ("rho", "u", "v", "w"):
        g = golden[name + "/" + k].astype(np.float64)
        assert np.abs(getattr(r, k) - g).max() <= 1e-6 * max(1.0, np.abs(g).max()), k
    np.testing.assert_allclose(r.resid[:steps], golden[name + "/resid"], rtol=1e-5)
