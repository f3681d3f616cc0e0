"""The oracle against golden fixtures written by the reference's own PPM and slope
functions (tests/golden/make_golden.py): bit for bit.  Runs on every host; the fixtures
carry the reference's results where its sources are absent."""
import os

import numpy as np
import pytest

import pyoracle
from maestroex_gb300 import configs
from maestroex_gb300.params import make_params

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ppm_slopes.npz")


def golden():
    return np.load(GOLDEN)


def ppm_fixture(g, c):
    pre = f"ppm{c}_"
    m = [int(v) for v in g[pre + "meta"]]
    ppm_type, is_umac, bc, bx, s_lo, dom_n = m[0], m[1], m[2:8], tuple(m[8:14]), m[14:17], tuple(m[17:20])
    cfg = configs.planar_config(n=dom_n, nspec=1, ppm_type=ppm_type, max_grid=max(dom_n))
    p = make_params(cfg)
    p.dt, p.rel_eps = float(g[pre + "real"][0]), float(g[pre + "real"][1])
    for d in range(3):
        p.dx[d] = float(g[pre + "real"][2 + d])
    vel = [g[pre + f"vel{d}"] for d in range(3)]
    return p, ppm_type, is_umac, bc, bx, g[pre + "s"], s_lo, vel, g[pre + "Ip"], g[pre + "Im"]


def n_fixtures(g, kind):
    return sum(1 for k in g.files if k.startswith(kind) and k.endswith("_meta"))


@pytest.mark.parametrize("c", range(6))
def test_oracle_ppm_matches_golden(c):
    g = golden()
    assert n_fixtures(g, "ppm") == 6
    p, ppm_type, is_umac, bc, bx, s, s_lo, vel, Ip, Im = ppm_fixture(g, c)
    a, b = pyoracle.ppm(p, bx, s, s_lo, 1, vel, [bx[:3]] * 3, is_umac, bc)
    assert np.array_equal(a, Ip) and np.array_equal(b, Im)


@pytest.mark.parametrize("c", range(6))
def test_oracle_slopes_match_golden(c):
    g = golden()
    assert n_fixtures(g, "slope") == 6
    m = [int(v) for v in g[f"slope{c}_meta"]]
    so, d, dom, bx, lo = m[0], m[1], tuple(m[2:8]), tuple(m[8:14]), m[14:17]
    bcs = [tuple(int(v) for v in b) for b in g[f"slope{c}_bcs"]]
    out = pyoracle.slopes(so, d, dom, bx, g[f"slope{c}_s"], lo, bcs)
    assert np.array_equal(out, g[f"slope{c}_slope"])


STAGE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "stage.npz")
STAGE_NAMES = ("planar_ppm1_w0", "planar_ppm2_walls", "spherical_ppm2", "planar_2d_ppm1")


def stage_fixture(name):
    """The configuration of a whole-stage fixture with the fixture's stored inputs, and the
    reference's outputs: snew (Rho, RhoH, species), umac at the end of the stage, the
    density flux per direction."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(GOLDEN)))
    from make_golden import STAGE_FIXTURES, STAGE_INPUTS
    g = np.load(STAGE)
    cfg = STAGE_FIXTURES[name]()
    for k in STAGE_INPUTS:
        cfg[k] = g[f"{name}_in_{k}"]
    nd = 2 if cfg.get("dim") == 2 else 3
    ref = {"snew": g[f"{name}_snew"], "umac_end": [g[f"{name}_umac_end{d}"] for d in range(nd)],
           "sflux_rho": [g[f"{name}_sflux{d}_rho"] for d in range(nd)]}
    return cfg, ref


def check_stage(cfg, res, ref, label):
    from maestroex_gb300.params import FIRSTSPEC, RHO, RHOH
    comps = [RHO, RHOH] + list(range(FIRSTSPEC, FIRSTSPEC + cfg["nspec"]))
    assert np.array_equal(res["snew"][comps], ref["snew"]), f"{label}: snew"
    for d in range(len(ref["umac_end"])):
        assert np.array_equal(res["umac_end"][d], ref["umac_end"][d]), f"{label}: umac[{d}]"
        assert np.array_equal(res["sflux"][d][RHO], ref["sflux_rho"][d]), f"{label}: density flux [{d}]"


@pytest.mark.parametrize("name", STAGE_NAMES)
def test_oracle_stage_matches_golden(name):
    cfg, ref = stage_fixture(name)
    run = pyoracle.run_stage_2d if cfg.get("dim") == 2 else pyoracle.run_stage
    check_stage(cfg, run(cfg, checked=True), ref, name)
