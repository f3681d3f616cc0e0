"""Species streaming: a stage call that asks for no edge states and no fluxes (sedge = sflux =
NULL, 3-D) runs each species' edge state, flux and update through three-component slots
instead of nscal-component edge-state and flux fields.  Its results must be the full stage's
bit for bit -- the state, the MAC velocities, etarhoflux -- on one and two levels, both
reflux types, every prediction type, plane-parallel and spherical, in every launch mode;
and the oracle's.
"""
import numpy as np
import pytest

import pyoracle
from maestroex_gb300 import capi, configs
from maestroex_gb300.params import FIRSTSPEC, OUTFLOW, RHO, RHOH, SLIPWALL, SYMMETRY

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from maestroex_gb300 import build
    build.build_library()


def same(a, b, label):
    for key in ("snew", "sold_end", "etarhoflux"):
        assert np.array_equal(a[key], b[key], equal_nan=True), f"{label}: {key}"
    for d in range(3):
        assert np.array_equal(a["umac_end"][d], b["umac_end"][d], equal_nan=True), f"{label}: umac[{d}]"


def vs_oracle(cfg, got, ref, label):
    comps = [RHO, RHOH] + list(range(FIRSTSPEC, FIRSTSPEC + cfg["nspec"]))
    for c in comps:
        assert np.array_equal(got["snew"][c], ref["snew"][c]), f"{label}: snew comp {c}"
        assert np.array_equal(got["sold_end"][c], ref["sold_end"][c]), f"{label}: sold comp {c}"
    assert np.array_equal(got["etarhoflux"], ref["etarhoflux"]), f"{label}: etarhoflux"


SINGLE = {
    "rho', X": dict(species_pred_type=1, enthalpy_pred_type=1),
    "rho X": dict(species_pred_type=2, enthalpy_pred_type=1),
    "rho, X": dict(species_pred_type=3, enthalpy_pred_type=0),
    "h predicted": dict(species_pred_type=1, enthalpy_pred_type=2),
    "h predicted, rho X": dict(species_pred_type=2, enthalpy_pred_type=2),
}


@pytest.mark.parametrize("ppm_type", [1, 2, 0])
@pytest.mark.parametrize("name", list(SINGLE))
def test_single_level_streamed_equals_full_and_oracle(name, ppm_type):
    from maestroex_gb300.stage import run_stage_gpu
    cfg = configs.planar_config(n=(16, 24, 32), nspec=5, ppm_type=ppm_type, max_grid=(16, 8, 16),
                                seed=1700 + ppm_type, **SINGLE[name])
    full = run_stage_gpu(cfg, mode=capi.MODE_BATCHED)
    for mode in (capi.MODE_BATCHED, capi.MODE_GRAPH, capi.MODE_PER_BOX):
        got = run_stage_gpu(cfg, mode=mode, edges=False)
        same(full, got, f"{name} ppm{ppm_type} mode {mode}")
    vs_oracle(cfg, got, pyoracle.run_stage(cfg, checked=False), f"{name} ppm{ppm_type}")


def test_traced_forces_and_thirteen_species():
    """ppm_trace_forces (the density's force traced) and NumSpec 13 with negative species to
    redistribute: the closing pass sees every species' new value."""
    from maestroex_gb300.stage import run_stage_gpu
    for kw in (dict(nspec=3, ppm_type=2, ppm_trace_forces=1), dict(nspec=13, ppm_type=1)):
        extra = {k: kw.pop(k) for k in ("ppm_trace_forces",) if k in kw}
        cfg = configs.planar_config(n=(32, 16, 16), max_grid=16, seed=1750, **kw)
        cfg.update(extra)
        full = run_stage_gpu(cfg)
        got = run_stage_gpu(cfg, edges=False)
        same(full, got, str(kw))


@pytest.mark.parametrize("reflux_type", [1, 2])
@pytest.mark.parametrize("walls", [False, True])
def test_two_levels_streamed_equals_full(reflux_type, walls):
    from maestroex_gb300.stage import run_amr_stage_gpu
    if walls:
        fine = [(0, 0, 0, 15, 15, 15), (16, 0, 0, 31, 15, 15), (48, 48, 48, 63, 63, 63), (40, 0, 32, 63, 15, 47)]
        cfg = configs.planar_amr_config(n0=(32, 32, 32), nspec=3, ppm_type=2, max_grid=16, fine_boxes=fine,
                                        bc_lo=(SLIPWALL, OUTFLOW, SLIPWALL), bc_hi=(OUTFLOW, SYMMETRY, OUTFLOW),
                                        species_pred_type=2, enthalpy_pred_type=0)
    else:
        rng = np.random.default_rng(1777)
        fine = configs.bubble_boxes((32, 32, 32), nbubbles=2, cover=0.08, block_edges=(4, 8), max_edge=8, rng=rng)
        cfg = configs.planar_amr_config(n0=(32, 32, 32), nspec=4, ppm_type=1, max_grid=16, fine_boxes=fine,
                                        seed=1778)
    cfg["reflux_type"] = reflux_type
    full = run_amr_stage_gpu(cfg)
    for mode in (capi.MODE_BATCHED, capi.MODE_GRAPH):
        got = run_amr_stage_gpu(cfg, mode=mode, edges=False)
        for lev, (a, b) in enumerate(zip(full, got)):
            same(a, b, f"reflux {reflux_type} walls {walls} mode {mode} level {lev}")
    ref = pyoracle.run_stage_levels(cfg)
    for lev, (g, r) in enumerate(zip(got, ref)):
        for key in ("snew", "sold_end"):
            assert np.array_equal(g[key], r[key], equal_nan=True), f"level {lev} {key}"


@pytest.mark.parametrize("exact", [True, False])
def test_spherical_two_levels_streamed_equals_full(exact):
    from maestroex_gb300.stage import run_amr_stage_gpu
    fine = configs.bubble_boxes((32, 32, 32), nbubbles=3, cover=0.12, block_edges=(4, 8), max_edge=8,
                                rng=np.random.default_rng(5))
    if not exact:
        fine = fine + [(56, 56, 56, 63, 63, 63)]
    cfg = configs.spherical_amr_config(n0=32, nspec=4, max_grid=16, ppm_type=2, fine_boxes=fine, exact=exact)
    full = run_amr_stage_gpu(cfg, mode=capi.MODE_GRAPH)
    got = run_amr_stage_gpu(cfg, mode=capi.MODE_GRAPH, edges=False)
    for lev, (a, b) in enumerate(zip(full, got)):
        same(a, b, f"spherical exact={exact} level {lev}")


def test_streamed_then_full_in_one_context():
    """One context serves a streamed call and then a full one (and back): the slots and the
    full edge-state fields are separate storage, and the graph is keyed on the call."""
    import torch
    from maestroex_gb300.stage import StageBuffers, make_stage
    cfg = configs.planar_config(n=(16, 16, 32), nspec=3, ppm_type=1, max_grid=16, seed=1790)
    st = make_stage(cfg)
    outs = []
    for edges in (False, True, False):
        buf = StageBuffers(cfg, edges=edges).load(cfg)
        st.stage_forward(buf.uold, buf.sold, buf.gpi, buf.snew, buf.umac, buf.sedge, buf.sflux, buf.eta,
                         thermal=buf.thermal, mode=capi.MODE_GRAPH)
        torch.cuda.synchronize()
        outs.append(buf.snew.to_domain(cfg["n"]).cpu().numpy())
    st.close()
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[1], outs[2])
