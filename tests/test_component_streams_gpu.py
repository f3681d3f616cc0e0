"""Component streams (option "component_streams"): the components of a MakeEdgeScal call
alternate between the level's stream and a second one, the second working in copies of
the per-component scratch.  Every output must be the one-stream stage's bit for bit, in
the batched and graph modes, on one and two levels, for every PPM form and the
conservative species form."""
import numpy as np
import pytest
import torch

from maestroex_gb300 import capi, configs
from maestroex_gb300.stage import StageBuffers, amr_buffers, make_amr_stage, make_stage

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from maestroex_gb300 import build
    build.build_library()


def outputs(buf, n):
    r = [buf.snew.to_domain(n), buf.sold.to_domain(n), buf.eta.to_domain(n)]
    r += [buf.umac[d].to_domain(n) for d in range(3)]
    if buf.sedge is not None:
        r += [buf.sedge[d].to_domain(n) for d in range(3)] + [buf.sflux[d].to_domain(n) for d in range(3)]
    return [t.cpu().numpy() for t in r]


def run_single(cfg, streams, mode, edges=True):
    st = make_stage(cfg)
    st.set_option("component_streams", streams)
    buf = StageBuffers(cfg, edges=edges).load(cfg)
    st.stage_forward(buf.uold, buf.sold, buf.gpi, buf.snew, buf.umac, buf.sedge, buf.sflux, buf.eta,
                     thermal=buf.thermal, mode=mode)
    torch.cuda.synchronize()
    out = outputs(buf, cfg["n"])
    st.close()
    return out


@pytest.mark.parametrize("ppm_type,spt", [(1, 1), (2, 2), (0, 3), (1, 2)])
def test_single_level_two_streams_equal_one(ppm_type, spt):
    cfg = configs.planar_config(n=(32, 16, 24), nspec=5, ppm_type=ppm_type, max_grid=(16, 16, 8),
                                seed=1800 + ppm_type, species_pred_type=spt)
    one = run_single(cfg, 0, capi.MODE_BATCHED)
    for mode in (capi.MODE_BATCHED, capi.MODE_GRAPH):
        two = run_single(cfg, 1, mode)
        for k, (a, b) in enumerate(zip(one, two)):
            assert np.array_equal(a, b, equal_nan=True), (ppm_type, spt, mode, k)


def test_traced_forces_and_repeated_graph_replays():
    """ppm_trace_forces (the force scratch is per component too), and a graph replayed
    several times on the same buffers."""
    cfg = configs.planar_config(n=(16, 32, 16), nspec=4, ppm_type=2, max_grid=16, seed=1850)
    cfg["ppm_trace_forces"] = 1
    one = run_single(cfg, 0, capi.MODE_BATCHED)
    st = make_stage(cfg)
    st.set_option("component_streams", 1)
    for _ in range(3):
        buf = StageBuffers(cfg).load(cfg)
        st.stage_forward(buf.uold, buf.sold, buf.gpi, buf.snew, buf.umac, buf.sedge, buf.sflux, buf.eta,
                         thermal=buf.thermal, mode=capi.MODE_GRAPH)
        torch.cuda.synchronize()
        for k, (a, b) in enumerate(zip(one, outputs(buf, cfg["n"]))):
            assert np.array_equal(a, b, equal_nan=True), k
    st.close()


def test_two_levels_two_streams_equal_one():
    rng = np.random.default_rng(1860)
    fine = configs.bubble_boxes((32, 32, 32), nbubbles=2, cover=0.08, block_edges=(4, 8), max_edge=8, rng=rng)
    cfg = configs.planar_amr_config(n0=(32, 32, 32), nspec=4, ppm_type=2, max_grid=16, fine_boxes=fine, seed=1861)
    res = []
    for streams in (0, 1):
        st = make_amr_stage(cfg)
        st.set_option("component_streams", streams)
        bufs = amr_buffers(cfg)
        st.stage_forward_levels(bufs, mode=capi.MODE_GRAPH)
        torch.cuda.synchronize()
        res.append([outputs(b, L["n"]) for b, L in zip(bufs, cfg["levels"])])
        st.close()
    for lev, (a, b) in enumerate(zip(*res)):
        for k, (x, y) in enumerate(zip(a, b)):
            assert np.array_equal(x, y, equal_nan=True), (lev, k)
