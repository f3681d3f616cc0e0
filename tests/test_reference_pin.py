"""Pins the oracle to the reference: the reference's own stage functions, compiled
unmodified from its sources against the AMReX / Maestro stand-ins in oracle/refshim/
(oracle/_ref/libmaestro_ref.so), against the oracle's restatement of the same functions on
the same seeded inputs, bit for bit.

Runs where the reference sources are present; elsewhere tests/test_golden.py checks the
oracle against fixtures this library wrote (tests/golden/make_golden.py).
"""
import itertools

import numpy as np
import pytest

import pyoracle
import pyref
from maestroex_gb300 import configs
from maestroex_gb300.params import make_params

pytestmark = pytest.mark.skipif(not pyref.available(), reason="reference sources not present on this host")

# AMReX BCType values: reflect_odd -1, int_dir 0, reflect_even 1, foextrap 2, ext_dir 3, hoextrap 4
BCTYPES = (-1, 0, 1, 2, 3, 4)


def field(rng, lo, n, scale=1e7, ties=0.05):
    """Smooth stratified data with noise, plateaus (exact ties in every limiter) and a few
    sign changes, on the index box [lo, lo + n)."""
    z, y, x = np.meshgrid(*[np.arange(lo[d], lo[d] + n[d]) for d in (2, 1, 0)], indexing="ij")
    f = scale * np.exp(-z / 9.0) * (1 + 0.3 * np.sin(0.7 * x) * np.cos(0.45 * y))
    f = f + rng.normal(0, 3e-3 * scale, f.shape)
    f[rng.random(f.shape) < ties] = 0.5 * scale
    f[rng.random(f.shape) < 0.02] *= -1.0
    return f


def ppm_inputs(seed, ppm_type, is_umac, dom_n, bx):
    rng = np.random.default_rng(seed)
    cfg = configs.planar_config(n=dom_n, nspec=1, ppm_type=ppm_type, max_grid=max(dom_n), seed=seed)
    p = make_params(cfg)
    g = 3 if ppm_type == 2 else 2
    lo = [bx[d] - g for d in range(3)]
    n = [bx[3 + d] - bx[d] + 1 + 2 * g for d in range(3)]
    s = np.stack([field(rng, lo, n, 1.0), field(rng, lo, n)])
    vel = []
    for d in range(3):
        m = [bx[3 + e] - bx[e] + 1 + (1 if (is_umac and e == d) else 0) for e in range(3)]
        v = rng.normal(0, 3e5, (1, m[2], m[1], m[0]))
        v[rng.random(v.shape) < 0.1] = 0.0
        v[rng.random(v.shape) < 0.05] = p.rel_eps
        v[rng.random(v.shape) < 0.05] = -p.rel_eps
        vel.append(v)
    return p, s, lo, vel, [bx[:3]] * 3


PPM_CASES = [(ppm_type, is_umac, k) for ppm_type in (1, 2) for is_umac in (0, 1) for k in range(10)]


@pytest.mark.parametrize("ppm_type,is_umac,k", PPM_CASES)
def test_ppm_matches_reference_source(ppm_type, is_umac, k):
    rng = np.random.default_rng(1000 + k)
    bc = [int(v) for v in rng.choice(BCTYPES, size=6)]
    dom_n = (12, 10, 8)
    # the box the stage passes to PPM: the valid box grown by one cell, here touching both
    # domain ends so that every boundary stencil runs (or shifted inside for some cases)
    if k % 3 == 2:
        bx = (2, 1, 1, 8, 7, 5)
    else:
        bx = (-1, -1, -1, dom_n[0], dom_n[1], dom_n[2])
    p, s, s_lo, vel, vel_lo = ppm_inputs(77 + k, ppm_type, is_umac, dom_n, bx)
    a = pyoracle.ppm(p, bx, s, s_lo, 1, vel, vel_lo, is_umac, bc)
    b = pyref.ppm(p, bx, s, s_lo, 1, vel, vel_lo, is_umac, bc)
    assert not np.isnan(b[0]).any() and not np.isnan(b[1]).any()
    assert np.array_equal(a[0], b[0]), f"Ip differs, bc {bc}"
    assert np.array_equal(a[1], b[1]), f"Im differs, bc {bc}"


@pytest.mark.parametrize("slope_order,d", list(itertools.product((0, 2, 4), (0, 1, 2))))
def test_slopes_match_reference_source(slope_order, d):
    rng = np.random.default_rng(2000 + 3 * slope_order + d)
    dom = (0, 0, 0, 11, 9, 7)
    bx = (-1, -1, -1, 12, 10, 8)
    lo = [bx[e] - 2 for e in range(3)]
    n = [bx[3 + e] - bx[e] + 1 + 4 for e in range(3)]
    ncomp = 4
    s = np.stack([field(rng, lo, n, 10.0 ** (c + 1)) for c in range(ncomp)])
    for trial in range(4):
        bcs = [tuple(int(v) for v in rng.choice(BCTYPES, size=6)) for _ in range(ncomp)]
        a = pyoracle.slopes(slope_order, d, dom, bx, s, lo, bcs)
        b = pyref.slopes(slope_order, d, dom, bx, s, lo, bcs)
        assert not np.isnan(b).any()
        assert np.array_equal(a, b), f"slopes differ, bcs {bcs}"
