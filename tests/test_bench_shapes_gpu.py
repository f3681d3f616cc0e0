"""GPU parity at the benchmark workloads' shapes: the box sizes, species counts, PPM types
and hierarchies the bench legs time, at sizes the oracle finishes in seconds.

* single level, 64^3 boxes (the headline layout), NumSpec 13 and 21, ppm_type 1, w0 != 0,
  x/y periodic, z slip wall / outflow;
* the same with negative species planted in the old state, so that UpdateScal's
  negative-species redistribution (Source/MaestroAdvection.cpp:186-250, a loop over the
  species in component order) runs with 13 and 21 species;
* two levels with uneven level-0 boxes (edges 16-64) and level-1 boxes of 16-32 fine cells
  around three bubbles (about 14% of the domain), NumSpec 13 and 21, ppm_type 2, reflux_type 1 and 2;
* the spherical full star on two levels, NumSpec 21, ppm_type 2, w0 of amplitude 1e5.

Bar: every component within 1e-12 of its max-norm (the benchmark's error definition);
the tests also require bitwise equality, which is what the library is built for.
"""
import numpy as np
import pytest

import pyoracle
from maestroex_gb300 import capi, configs
from maestroex_gb300.params import FIRSTSPEC, RHO
from test_amr_gpu import compare_levels
from test_parity_gpu import compare

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from maestroex_gb300 import build
    build.build_library()


def headline_shape(nspec, n=(128, 128, 128), seed=20261203 + 1):
    return configs.planar_config(n=n, nspec=nspec, ppm_type=1, max_grid=64, seed=seed, w0_amp=1.0e4, cfl=0.7)


@pytest.mark.parametrize("nspec", [13, 21])
def test_headline_layout_matches_oracle(nspec):
    from maestroex_gb300.stage import run_stage_gpu
    cfg = headline_shape(nspec)
    assert len(cfg["boxes"]) == 8
    ref = pyoracle.run_stage(cfg)
    gpu = run_stage_gpu(cfg, mode=capi.MODE_GRAPH)
    worst, bitwise = compare(cfg, gpu, ref, f"64^3 boxes, NumSpec {nspec}")
    assert bitwise, worst


def plant_negative_species(cfg, frac=2e-3, seed=7):
    """Set one species of a seeded fraction of the cells to a small negative partial density
    (up to 1e-3 of the density); the stage then leaves those species negative in the
    updated state and UpdateScal's redistribution has to clear them."""
    rng = np.random.default_rng(seed)
    s = cfg["sold"]
    shape = s.shape[1:]
    cells = rng.random(shape) < frac
    comp = rng.integers(0, cfg["nspec"], size=shape)
    for c in range(cfg["nspec"]):
        m = cells & (comp == c)
        s[FIRSTSPEC + c][m] = -1e-3 * rng.random(int(m.sum())) * s[RHO][m]
    return int(cells.sum())


@pytest.mark.parametrize("nspec", [13, 21])
def test_negative_species_redistribution_matches_oracle(nspec):
    from maestroex_gb300.stage import run_stage_gpu
    cfg = headline_shape(nspec, n=(128, 64, 64), seed=20261203 + 21)
    planted = plant_negative_species(cfg)
    assert planted > 100
    ref = pyoracle.run_stage(cfg)
    gpu = run_stage_gpu(cfg)
    spec = ref["snew"][FIRSTSPEC:FIRSTSPEC + nspec]
    # the redistribution sets a negative species to exactly zero and leaves none negative
    assert (spec == 0.0).sum() > 50 and (spec >= 0.0).all()
    worst, bitwise = compare(cfg, gpu, ref, f"negative species, NumSpec {nspec}")
    assert bitwise, worst


@pytest.mark.parametrize("nspec,reflux_type", [(13, 1), (21, 1), (13, 2)])
def test_two_level_uneven_boxes_matches_oracle(nspec, reflux_type):
    from maestroex_gb300.stage import run_amr_stage_gpu
    cfg = configs.two_level_sample(nspec)
    cfg["reflux_type"] = reflux_type
    l0, l1 = cfg["levels"][0]["boxes"], cfg["levels"][1]["boxes"]
    edges = {b[3 + d] - b[d] + 1 for b in l0 for d in range(3)}
    assert len(edges) > 1 and len(l1) > 3
    cover = sum((b[3] - b[0] + 1) * (b[4] - b[1] + 1) * (b[5] - b[2] + 1) for b in l1) / 8 / 64 ** 3
    assert 0.08 < cover < 0.25
    ref = pyoracle.run_stage_levels(cfg)
    gpu = run_amr_stage_gpu(cfg, mode=capi.MODE_GRAPH)
    assert compare_levels(cfg, gpu, ref, f"two levels NumSpec {nspec} reflux {reflux_type}")


def test_spherical_two_levels_numspec21_matches_oracle():
    from maestroex_gb300.stage import run_amr_stage_gpu
    cfg = configs.spherical_two_level_sample()
    assert len(cfg["levels"][0]["boxes"]) > 1 and len(cfg["levels"][1]["boxes"]) > 3
    ref = pyoracle.run_stage_levels(cfg)
    gpu = run_amr_stage_gpu(cfg, mode=capi.MODE_GRAPH)
    assert compare_levels(cfg, gpu, ref, "spherical two levels NumSpec 21")
