"""GPU parity on two-level hierarchies (refinement ratio 2): the CUDA stage with its
coarse-fine coupling (two-level FillPatch with cell_cons_interp, AverageDown,
AverageDownFaces, FillPatchUedge, per-level radial chunks) against the CPU oracle's
multi-level restatement, level by level, within 1e-12 of each component's max-norm
(in practice bitwise).
"""
import numpy as np
import pytest

import pyoracle
from maestroex_gb300 import capi, configs
from maestroex_gb300.params import FIRSTSPEC, INTERIOR, OUTFLOW, RHO, RHOH, SLIPWALL, SYMMETRY

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _built():
    from maestroex_gb300 import build
    build.build_library()


def nan_rel_err(gpu, ref):
    """rel_err over the cells / faces a level covers (NaN elsewhere in both)."""
    gpu, ref = np.asarray(gpu), np.asarray(ref)
    m = np.isfinite(ref)
    assert m.any()
    assert np.array_equal(m, np.isfinite(gpu)), "coverage differs"
    scale = np.abs(ref[m]).max()
    d = np.abs(gpu[m] - ref[m]).max()
    return float(d / scale) if scale > 0 else float(d)


def compare_levels(cfg, gpu, ref, label=""):
    nspec = cfg["nspec"]
    comps = [RHO, RHOH] + list(range(FIRSTSPEC, FIRSTSPEC + nspec))
    bitwise = True
    for lev, (g, r) in enumerate(zip(gpu, ref)):
        for d in range(3):
            e = nan_rel_err(g["umac_end"][d], r["umac_end"][d])
            assert e <= TOL, f"{label} level {lev} umac[{d}] {e}"
            bitwise &= np.array_equal(g["umac_end"][d], r["umac_end"][d], equal_nan=True)
            for key in ("sedge", "sflux"):
                for c in comps:
                    e = nan_rel_err(g[key][d][c], r[key][d][c])
                    assert e <= TOL, f"{label} level {lev} {key}[{d}] comp {c} {e}"
                    bitwise &= np.array_equal(g[key][d][c], r[key][d][c], equal_nan=True)
        for key in ("snew", "sold_end"):
            for c in comps:
                e = nan_rel_err(g[key][c], r[key][c])
                assert e <= TOL, f"{label} level {lev} {key} comp {c} {e}"
                bitwise &= np.array_equal(g[key][c], r[key][c], equal_nan=True)
        e = nan_rel_err(g["etarhoflux"], r["etarhoflux"])
        assert e <= TOL, f"{label} level {lev} etarhoflux {e}"
    return bitwise


def small_amr(ppm_type=2, nspec=2, seed=20261203 + 2, **kw):
    rng = np.random.default_rng(seed + 7)
    fine = configs.bubble_boxes((32, 32, 32), nbubbles=2, cover=0.08, block_edges=(4, 8), max_edge=8, rng=rng)
    return configs.planar_amr_config(n0=(32, 32, 32), nspec=nspec, ppm_type=ppm_type, max_grid=16,
                                     fine_boxes=fine, seed=seed, **kw)


@pytest.mark.parametrize("ppm_type", [2, 1])
def test_two_level_stage_matches_oracle(ppm_type):
    from maestroex_gb300.stage import run_amr_stage_gpu
    cfg = small_amr(ppm_type=ppm_type)
    assert 0 < len(cfg["levels"][1]["boxes"])
    ref = pyoracle.run_stage_levels(cfg)
    gpu = run_amr_stage_gpu(cfg, mode=capi.MODE_BATCHED)
    assert compare_levels(cfg, gpu, ref, f"ppm{ppm_type}")


def test_two_level_walls_and_prediction_types():
    """Fine boxes touching non-periodic walls on every side, species_pred_type 2 and
    enthalpy_pred_type 0."""
    from maestroex_gb300.stage import run_amr_stage_gpu
    fine = [(0, 0, 0, 15, 15, 15), (16, 0, 0, 31, 15, 15), (48, 48, 48, 63, 63, 63), (40, 0, 32, 63, 15, 47)]
    cfg = configs.planar_amr_config(n0=(32, 32, 32), nspec=2, ppm_type=2, max_grid=16, fine_boxes=fine,
                                    bc_lo=(SLIPWALL, OUTFLOW, SLIPWALL), bc_hi=(OUTFLOW, SYMMETRY, OUTFLOW),
                                    species_pred_type=2, enthalpy_pred_type=0)
    ref = pyoracle.run_stage_levels(cfg)
    gpu = run_amr_stage_gpu(cfg)
    assert compare_levels(cfg, gpu, ref, "walls")


def test_two_level_launch_modes_agree():
    from maestroex_gb300.stage import run_amr_stage_gpu
    cfg = small_amr(ppm_type=2, seed=20261203 + 9)
    a = run_amr_stage_gpu(cfg, mode=capi.MODE_BATCHED)
    for mode in (capi.MODE_PER_BOX, capi.MODE_GRAPH):
        b = run_amr_stage_gpu(cfg, mode=mode)
        for la, lb in zip(a, b):
            for key in ("snew", "sold_end"):
                assert np.array_equal(la[key], lb[key], equal_nan=True), (mode, key)
            for key in ("umac_end", "sedge", "sflux"):
                for d in range(3):
                    assert np.array_equal(la[key][d], lb[key][d], equal_nan=True), (mode, key, d)


def test_fine_level_covering_domain_equals_single_level():
    """A level 1 that covers the whole domain never interpolates from level 0, so it must
    reproduce the single-level stage at the fine resolution bit for bit."""
    from maestroex_gb300.stage import run_amr_stage_gpu, run_stage_gpu
    fb = configs.tile_boxes((32, 32, 32), 16)
    cfg = configs.planar_amr_config(n0=(16, 16, 16), nspec=2, ppm_type=1, max_grid=8, fine_boxes=fb)
    two = run_amr_stage_gpu(cfg)
    one_cfg = dict(cfg)
    one_cfg.update(cfg["levels"][1])
    one_cfg.pop("levels")
    one = run_stage_gpu(one_cfg)
    for key in ("snew", "sold_end"):
        assert np.array_equal(two[1][key], one[key])
    for key in ("umac_end", "sedge", "sflux"):
        for d in range(3):
            assert np.array_equal(two[1][key][d], one[key][d])


def test_rejects_misaligned_fine_box():
    from maestroex_gb300.params import make_params
    from maestroex_gb300.stage import ScalarAdvectionStage
    cfg = small_amr()
    st = ScalarAdvectionStage(make_params(cfg))
    with pytest.raises(capi.MadvError) as e:
        st.set_layout_levels([cfg["levels"][0]["boxes"], [(1, 0, 0, 16, 15, 15)]])
    assert e.value.code == -2
    st.close()


@pytest.mark.parametrize("walls", [False, True])
def test_two_level_flux_register_matches_oracle(walls):
    """reflux_type 2: the coarse level is updated with its own fluxes and then takes back the
    coarse-fine flux mismatch from the flux registers (CrseInit / FineAdd / Reflux); the GPU
    registers against the oracle's, all launch modes."""
    from maestroex_gb300.stage import run_amr_stage_gpu
    if walls:
        fine = [(0, 0, 0, 15, 15, 15), (16, 0, 0, 31, 15, 15), (48, 48, 48, 63, 63, 63), (40, 0, 32, 63, 15, 47)]
        cfg = configs.planar_amr_config(n0=(32, 32, 32), nspec=2, ppm_type=2, max_grid=16, fine_boxes=fine,
                                        bc_lo=(SLIPWALL, OUTFLOW, SLIPWALL), bc_hi=(OUTFLOW, SYMMETRY, OUTFLOW))
    else:
        cfg = small_amr(ppm_type=2, seed=20261203 + 11)
    cfg["reflux_type"] = 2
    ref = pyoracle.run_stage_levels(cfg)
    gpu = run_amr_stage_gpu(cfg, mode=capi.MODE_BATCHED)
    assert compare_levels(cfg, gpu, ref, "reflux 2")
    g2 = run_amr_stage_gpu(cfg, mode=capi.MODE_GRAPH)
    for la, lb in zip(gpu, g2):
        assert np.array_equal(la["snew"], lb["snew"], equal_nan=True)
