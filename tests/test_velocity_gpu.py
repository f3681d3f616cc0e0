"""GPU parity of madv_velocity_advance (Maestro::VelocityAdvance + UpdateVel) against the
oracle's restatement (pyoracle.run_velocity_advance): the MAC velocity from
madv_advance_premac (bitwise the oracle's VelPred output), then the velocity edge states
(MakeEdgeScal with is_vel: the outflow clamps of the normal component) and the update,
with and without a sponge, plane-parallel and spherical."""
import numpy as np
import pytest
import torch

import pyoracle
from maestroex_gb300 import configs
from maestroex_gb300.params import OUTFLOW, RHO, SLIPWALL
from maestroex_gb300.stage import MultiFab, StageBuffers, make_stage

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from maestroex_gb300 import build
    build.build_library()


def run_gpu(cfg, rhohalf, sponge=None):
    st = make_stage(cfg)
    buf = StageBuffers(cfg).load(cfg)
    boxes = cfg["boxes"]
    umac = [MultiFab(boxes, 1, 1, nodal=d) for d in range(3)]
    st.advance_premac(buf.uold, buf.sold, buf.gpi, umac)
    rh = MultiFab(boxes, 1, 0).from_domain(rhohalf[None])
    sp = MultiFab(boxes, 1, 0).from_domain(sponge[None]) if sponge is not None else None
    unew = MultiFab(boxes, 3, buf.sold.ng)
    uedge = [MultiFab(boxes, 3, 0, nodal=d) for d in range(3)]
    st.velocity_advance(buf.uold, buf.sold, rh, buf.gpi, umac, unew, uedge, sponge=sp)
    torch.cuda.synchronize()
    n = cfg["n"]
    return dict(unew=unew.to_domain(n).cpu().numpy(), uedge=[u.to_domain(n).cpu().numpy() for u in uedge],
                umac=[u.to_domain(n)[0].cpu().numpy() for u in umac])


def compare(gpu, ref, label):
    ok = True
    for d in range(3):
        assert np.array_equal(gpu["umac"][d], ref["umac"][d]), f"{label}: MAC velocity {d}"
        for n in range(3):
            g, r = gpu["uedge"][d][n], ref["uedge"][d][n]
            err = np.abs(g - r).max() / max(np.abs(r).max(), 1e-300)
            assert err <= 1e-12, f"{label}: uedge[{d}] comp {n} {err}"
            ok &= np.array_equal(g, r)
        g, r = gpu["unew"][d], ref["unew"][d]
        err = np.abs(g - r).max() / max(np.abs(r).max(), 1e-300)
        assert err <= 1e-12, f"{label}: unew comp {d} {err}"
        ok &= np.array_equal(g, r)
    return ok


CASES = {
    "planar ppm1": lambda: configs.planar_config(n=(32, 32, 32), max_grid=16, ppm_type=1),
    "planar ppm2 outflow": lambda: configs.planar_config(n=(32, 32, 32), max_grid=16, ppm_type=2,
                                                         bc_lo=(OUTFLOW, SLIPWALL, SLIPWALL),
                                                         bc_hi=(OUTFLOW, OUTFLOW, OUTFLOW)),
    "planar ppm0": lambda: configs.planar_config(n=(32, 32, 32), max_grid=16, ppm_type=0),
    "spherical ppm2": lambda: configs.spherical_config(n=32, max_grid=16, ppm_type=2),
    "spherical uniform bins ppm2": lambda: configs.spherical_config(n=32, max_grid=16, ppm_type=2, exact=False),
    "spherical uniform bins, w0mac nodal, s0 linear": lambda: configs.spherical_config(
        n=32, max_grid=16, ppm_type=1, exact=False, w0mac_interp_type=4, s0_interp_type=2),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("with_sponge", [False, True])
def test_velocity_advance_matches_oracle(name, with_sponge):
    cfg = CASES[name]()
    rng = np.random.default_rng(17)
    rhohalf = cfg["sold"][RHO] * (1.0 + 1e-4 * rng.standard_normal(cfg["sold"][RHO].shape))
    sponge = rng.uniform(0.5, 1.0, size=rhohalf.shape) if with_sponge else None
    gpu = run_gpu(cfg, rhohalf, sponge)
    ref = pyoracle.run_velocity_advance(cfg, rhohalf, sponge)
    assert compare(gpu, ref, name), f"{name}: within 1e-12 but not bitwise"


def test_velocity_advance_with_traced_forces_matches_oracle():
    cfg = configs.planar_config(n=(32, 32, 32), max_grid=16, ppm_type=2, gpi_amp=1e-3)
    cfg["ppm_trace_forces"] = 1
    rng = np.random.default_rng(19)
    rhohalf = cfg["sold"][RHO] * (1.0 + 1e-4 * rng.standard_normal(cfg["sold"][RHO].shape))
    gpu = run_gpu(cfg, rhohalf)
    ref = pyoracle.run_velocity_advance(cfg, rhohalf)
    assert compare(gpu, ref, "traced forces"), "within 1e-12 but not bitwise"
