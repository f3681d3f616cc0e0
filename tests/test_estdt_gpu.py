"""GPU parity of madv_est_dt (Maestro::EstDt: advective and force constraints, rel_eps)
against the oracle's box-by-box restatement: dt and umax bit for bit, single level
(plane-parallel with w0, spherical) and two levels; and the max_dt / fixed_dt /
small_dt limits."""
import numpy as np
import pytest

import pyoracle
from maestroex_gb300 import configs
from maestroex_gb300.capi import MadvError
from maestroex_gb300.stage import StageBuffers, amr_buffers, make_amr_stage, make_stage

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from maestroex_gb300 import build
    build.build_library()


CASES = {
    "planar": lambda: configs.planar_config(n=(32, 32, 32), max_grid=16, ppm_type=1, rho_pert=1e-3, gpi_amp=1e-3),
    "spherical": lambda: configs.spherical_config(n=32, max_grid=16, ppm_type=2),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("cfl,drdxfac", [(0.5, 1), (0.9, 5)])
def test_est_dt_matches_oracle(name, cfl, drdxfac):
    cfg = CASES[name]()
    st = make_stage(cfg)
    buf = StageBuffers(cfg).load(cfg)
    dt, dt_est, umax, rel_eps = st.est_dt(buf.uold, buf.sold, buf.gpi, cfl=cfl, drdxfac=drdxfac)
    rdt, rumax = pyoracle.est_dt(cfg, cfl=cfl, drdxfac=drdxfac)
    assert dt == dt_est == rdt, (dt, rdt)
    assert umax == rumax and rel_eps == umax * 1e-8
    assert 0.0 < dt < 1e20


def test_est_dt_two_levels_and_limits():
    fine = configs.bubble_boxes((32, 32, 32), nbubbles=2, cover=0.12, block_edges=(4, 8), max_edge=8,
                                rng=np.random.default_rng(3))
    cfg = configs.planar_amr_config(n0=(32, 32, 32), max_grid=16, ppm_type=2, fine_boxes=fine)
    st = make_amr_stage(cfg)
    bufs = amr_buffers(cfg)
    dt, dt_est, umax, _ = st.est_dt([b.uold for b in bufs], [b.sold for b in bufs], [b.gpi for b in bufs])
    rdt, rumax = pyoracle.est_dt(cfg)
    assert dt == rdt and umax == rumax
    lv = ([b.uold for b in bufs], [b.sold for b in bufs], [b.gpi for b in bufs])
    assert st.est_dt(*lv, max_dt=0.5 * dt)[0] == 0.5 * dt
    assert st.est_dt(*lv, fixed_dt=123.0)[0] == 123.0
    with pytest.raises(MadvError):
        st.est_dt(*lv, small_dt=2.0 * dt)


@pytest.mark.parametrize("kw", [{}, {"w0mac_interp_type": 4, "drdxfac": 2}])
def test_est_dt_spherical_uniform_bins(kw):
    """Uniform radial bins with an evolving base state: the velocity limit adds w0mac
    (MakeW0mac) averaged to the cells; the radial spacing is the bins' dr."""
    cfg = configs.spherical_config(n=32, max_grid=16, ppm_type=1, exact=False, **kw)
    st = make_stage(cfg)
    buf = StageBuffers(cfg).load(cfg)
    f = kw.get("drdxfac", 1)
    dt, dt_est, umax, rel_eps = st.est_dt(buf.uold, buf.sold, buf.gpi, cfl=0.7, drdxfac=f)
    rdt, rumax = pyoracle.est_dt(cfg, cfl=0.7, drdxfac=f)
    assert dt == rdt and umax == rumax
    with pytest.raises(MadvError):  # the radial grid's drdxfac only
        st.est_dt(buf.uold, buf.sold, buf.gpi, cfl=0.7, drdxfac=f + 1)
