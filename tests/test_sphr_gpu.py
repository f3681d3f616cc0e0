"""GPU parity of the spherical stage (full star, exact base state) against the oracle's
restatement of the reference's spherical branches: every output within 1e-12 of its
max-norm, in practice bitwise."""
import numpy as np
import pytest

import pyoracle
from maestroex_gb300 import capi, configs
from maestroex_gb300.configs import uneven_boxes
from test_parity_gpu import compare

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from maestroex_gb300 import build
    build.build_library()


def run_both(cfg, mode=capi.MODE_BATCHED):
    from maestroex_gb300.stage import run_stage_gpu
    return run_stage_gpu(cfg, mode=mode), pyoracle.run_stage(cfg, checked=False)


@pytest.mark.parametrize("ppm_type", [1, 2, 0])
def test_spherical_stage(ppm_type):
    cfg = configs.spherical_config(n=32, max_grid=16, ppm_type=ppm_type)
    gpu, ref = run_both(cfg)
    worst, bitwise = compare(cfg, gpu, ref, f"spherical ppm{ppm_type}")
    assert bitwise, worst


def test_spherical_uneven_boxes_and_graph():
    rng = np.random.default_rng(11)
    boxes = uneven_boxes((48, 48, 48), (8, 16, 24), rng)
    cfg = configs.spherical_config(n=48, boxes=boxes, ppm_type=2, nspec=5)
    gpu, ref = run_both(cfg, mode=capi.MODE_GRAPH)
    worst, bitwise = compare(cfg, gpu, ref, "spherical uneven")
    assert bitwise, worst


@pytest.mark.parametrize("ppm_type", [2, 1])
def test_spherical_two_levels(ppm_type):
    """Two levels on one radial grid (the fine level's): every level maps its cells to the
    fine radial bins; coarse-fine coupling as in the plane-parallel hierarchy."""
    from maestroex_gb300.stage import run_amr_stage_gpu
    from test_amr_gpu import compare_levels
    fine = configs.bubble_boxes((32, 32, 32), nbubbles=3, cover=0.12, block_edges=(4, 8), max_edge=8,
                                rng=np.random.default_rng(5))
    cfg = configs.spherical_amr_config(n0=32, max_grid=16, ppm_type=ppm_type, fine_boxes=fine)
    assert len(fine) > 1
    gpu = run_amr_stage_gpu(cfg, mode=capi.MODE_GRAPH)
    ref = pyoracle.run_stage_levels(cfg)
    assert compare_levels(cfg, gpu, ref, f"spherical 2 levels ppm{ppm_type}")


# uniform radial bins (use_exact_base_state = 0, the reference's default): every interpolation
# type of Put1dArrayOnCart, MakeW0mac and MakeS0mac, drdxfac, and (rho h) predicted
UNIFORM_CASES = {
    "defaults": {},
    "rhoh predicted": {"enthalpy_pred_type": 0},
    "w0 constant, s0 linear": {"w0_interp_type": 1, "s0_interp_type": 2},
    "w0 quadratic, s0 constant": {"w0_interp_type": 3, "s0_interp_type": 1},
    "w0mac linear, s0mac linear": {"w0mac_interp_type": 2, "s0mac_interp_type": 2},
    "w0mac quadratic, s0mac quadratic": {"w0mac_interp_type": 3, "s0mac_interp_type": 3},
    "w0mac nodal, drdxfac 5": {"w0mac_interp_type": 4, "drdxfac": 5},
    "h predicted": {"enthalpy_pred_type": 2},
    "h predicted, rhoX": {"enthalpy_pred_type": 2, "species_pred_type": 2},
}


@pytest.mark.parametrize("ppm_type", [1, 2])
@pytest.mark.parametrize("name", list(UNIFORM_CASES))
def test_spherical_uniform_bins(name, ppm_type):
    kw = dict(UNIFORM_CASES[name])
    ept = kw.pop("enthalpy_pred_type", 1)
    spt = kw.pop("species_pred_type", 1)
    cfg = configs.spherical_config(n=32, max_grid=16, ppm_type=ppm_type, exact=False, **kw)
    cfg["enthalpy_pred_type"], cfg["species_pred_type"] = ept, spt
    gpu, ref = run_both(cfg, mode=capi.MODE_GRAPH)
    worst, bitwise = compare(cfg, gpu, ref, f"spherical uniform bins, {name}, ppm{ppm_type}")
    assert bitwise, worst


@pytest.mark.parametrize("kw", [{"w0_interp_type": 3}, {"w0mac_interp_type": 4}, {"w0mac_interp_type": 2}])
def test_spherical_exact_grid_interpolation_types(kw):
    """The exact grid with the uniform-bin w0mac types (they index w0 by r / dr_fine, as the
    reference does whatever the grid) and the quadratic w0."""
    cfg = configs.spherical_config(n=16, max_grid=8, ppm_type=1, **kw)
    gpu, ref = run_both(cfg)
    worst, bitwise = compare(cfg, gpu, ref, f"spherical exact grid {kw}")
    assert bitwise, worst


@pytest.mark.parametrize("corner", [False, True])
def test_spherical_uniform_bins_two_levels(corner):
    """corner: one more level-1 box in the domain's top corner, whose rows (fine z up to 63)
    lie past the 56 radial bins -- the one radial level is read whole on every level, not in
    the plane-parallel chunks the fine rows would give."""
    from maestroex_gb300.stage import run_amr_stage_gpu
    from test_amr_gpu import compare_levels
    fine = configs.bubble_boxes((32, 32, 32), nbubbles=3, cover=0.12, block_edges=(4, 8), max_edge=8,
                                rng=np.random.default_rng(5))
    if corner:
        fine = fine + [(56, 56, 56, 63, 63, 63)]
    cfg = configs.spherical_amr_config(n0=32, max_grid=16, ppm_type=2, fine_boxes=fine, exact=False,
                                       w0mac_interp_type=4)
    assert cfg["nr"] < 64
    gpu = run_amr_stage_gpu(cfg, mode=capi.MODE_GRAPH)
    ref = pyoracle.run_stage_levels(cfg)
    assert compare_levels(cfg, gpu, ref, "spherical uniform bins, 2 levels")


def test_spherical_uniform_bins_rejections():
    from maestroex_gb300.params import make_params
    from maestroex_gb300.stage import ScalarAdvectionStage
    for exact, kw in ((True, {"s0mac_interp_type": 2}), (True, {"enthalpy_pred_type": 2}),
                      (False, {"w0mac_interp_type": 5})):
        cfg = configs.spherical_config(n=16, max_grid=16, exact=exact)
        cfg.update(kw)
        with pytest.raises(capi.MadvError):
            ScalarAdvectionStage(make_params(cfg))
