"""GPU parity of the per-member-function entry points (madv_make_utrans, madv_vel_pred,
madv_make_edge_scal, madv_make_rhox_flux, madv_make_rhoh_flux, madv_update_scal) against the
oracle's restatement of the same Maestro member functions (pyoracle.member), on caller
FABs whose ghost cells hold arbitrary (seeded) values: both sides read the ghost cells as
given, so the comparison covers every boundary branch the functions take."""
import numpy as np
import pytest
import torch

import pyoracle
from maestroex_gb300 import configs
from maestroex_gb300.stage import MultiFab, make_stage
from members import FIRSTSPEC, RHO, RHOH, MemberInputs, zeros_like

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from maestroex_gb300 import build
    build.build_library()


def planar(ppm_type):
    cfg = configs.planar_config(n=(32, 32, 32), max_grid=16, ppm_type=ppm_type)
    cfg["rho0_new"] = cfg["rho0_old"] * (1.0 + 1e-3)
    cfg["rhoh0_new"] = cfg["rhoh0_old"] * (1.0 - 1e-3)
    return cfg


CASES = {
    "planar ppm1": lambda: planar(1),
    "planar ppm2": lambda: planar(2),
    "planar ppm0": lambda: planar(0),
    "spherical ppm2": lambda: configs.spherical_config(n=32, max_grid=16, ppm_type=2),
}


def to_mf(fabs, boxes, g, nodal=-1):
    mf = MultiFab(boxes, fabs[0][0].shape[0], g, nodal=nodal)
    for b, (t, (a, lo)) in enumerate(zip(mf.fabs, fabs)):
        assert list(mf.los[b]) == list(lo) and tuple(t.shape) == a.shape
        t.copy_(torch.from_numpy(a))
    return mf


def compare(mf, ref_fabs, comps, what):
    """Max over boxes of |gpu - ref| / max |ref| per component, over the whole FABs."""
    torch.cuda.synchronize()
    worst, bitwise = 0.0, True
    for c in comps:
        g = [t[c].cpu().numpy() for t in mf.fabs]
        r = [a[c] for a, _ in ref_fabs]
        scale = max(float(np.abs(x).max()) for x in r)
        diff = max(float(np.abs(x - y).max()) for x, y in zip(g, r))
        assert all(np.isfinite(x).all() for x in g), (what, c)
        bitwise &= all(np.array_equal(x, y) for x, y in zip(g, r))
        worst = max(worst, diff / scale if scale > 0 else diff)
    print(f"{what}: worst rel err {worst:.3e}, bitwise {bitwise}")
    return worst, bitwise


@pytest.fixture(scope="module", params=list(CASES))
def case(request):
    cfg = CASES[request.param]()
    return request.param, cfg, make_stage(cfg), MemberInputs(cfg)


def test_make_utrans(case):
    name, cfg, st, inp = case
    b, g = inp.boxes, inp.ng
    ut, uf = inp.fabs("utilde", g), inp.fabs("ufull", g)
    out = [MultiFab(b, 1, 1, nodal=d) for d in range(3)]
    st.make_utrans(to_mf(ut, b, g), to_mf(uf, b, g), out)
    ref = [zeros_like(f) for f in inp.fabs("uface", 1)]
    pyoracle.member(cfg, "make_utrans", {"utilde": ut, "ufull": uf, "utrans": ref})
    for d in range(3):
        worst, bitwise = compare(out[d], ref[d], [0], f"{name} utrans {d}")
        assert bitwise, worst


def test_vel_pred(case):
    name, cfg, st, inp = case
    b, g = inp.boxes, inp.ng
    ut, uf = inp.fabs("utilde", g), inp.fabs("ufull", g)
    utr, force = inp.fabs("uface", 1), inp.fabs("vel_force", 1)
    out = [MultiFab(b, 1, 0, nodal=d) for d in range(3)]
    st.vel_pred(to_mf(ut, b, g), to_mf(uf, b, g), [to_mf(utr[d], b, 1, d) for d in range(3)], out,
                to_mf(force, b, 1))
    ref = [zeros_like(f) for f in inp.fabs("uface", 0)]
    pyoracle.member(cfg, "vel_pred", {"utilde": ut, "ufull": uf, "utrans": utr, "force": force, "umac": ref})
    for d in range(3):
        worst, bitwise = compare(out[d], ref[d], [0], f"{name} umac {d}")
        assert bitwise, worst


@pytest.mark.parametrize("which", ["species", "rhoh", "rho conservative"])
def test_make_edge_scal(case, which):
    name, cfg, st, inp = case
    b, g = inp.boxes, inp.ng
    start, num, cons = {"species": (FIRSTSPEC, inp.nspec, 0), "rhoh": (RHOH, 1, 0),
                        "rho conservative": (RHO, 1, 1)}[which]
    state, umac, force = inp.fabs("state", g), inp.fabs("uface", 1), inp.fabs("scal_force", 1)
    out = [MultiFab(b, inp.nscal, 0, nodal=d) for d in range(3)]
    st.make_edge_scal(to_mf(state, b, g), out, [to_mf(umac[d], b, 1, d) for d in range(3)], to_mf(force, b, 1),
                      0, start, start, num, cons)
    ref = [zeros_like(f) for f in inp.fabs("sedge", 0)]
    pyoracle.member(cfg, "make_edge_scal", {"state": state, "umac": umac, "force": force, "sedge": ref},
                    start_comp=start, num_comp=num, is_conservative=cons)
    for d in range(3):
        worst, bitwise = compare(out[d], ref[d], range(start, start + num), f"{name} sedge {which} {d}")
        assert bitwise, worst


@pytest.mark.parametrize("which_step", [1, 2])
def test_fluxes(case, which_step):
    name, cfg, st, inp = case
    b = inp.boxes
    sedge, umac, eta = inp.fabs("sedge", 0), inp.fabs("uface", 0), inp.fabs("eta", 0)
    eta_gpu = to_mf(eta, b, 0, 2)
    out = [MultiFab(b, inp.nscal, 0, nodal=d) for d in range(3)]
    se = [to_mf(sedge[d], b, 0, d) for d in range(3)]
    um = [to_mf(umac[d], b, 0, d) for d in range(3)]
    st.make_rhox_flux(which_step, out, eta_gpu, se, um, FIRSTSPEC, inp.nspec)
    st.make_rhoh_flux(which_step, out, se, um)
    ref = [zeros_like(f) for f in inp.fabs("sflux", 0)]
    pyoracle.member(cfg, "make_rhox_flux", {"sedge": sedge, "umac": umac, "sflux": ref, "eta": eta},
                    which_step=which_step, start_comp=FIRSTSPEC, num_comp=inp.nspec)
    pyoracle.member(cfg, "make_rhoh_flux", {"sedge": sedge, "umac": umac, "sflux": ref}, which_step=which_step)
    comps = [RHO, RHOH] + list(range(FIRSTSPEC, inp.nscal))
    for d in range(3):
        worst, bitwise = compare(out[d], ref[d], comps, f"{name} sflux step {which_step} {d}")
        assert bitwise, worst
    worst, bitwise = compare(eta_gpu, eta, [0], f"{name} etarhoflux")
    assert bitwise, worst


def test_update_scal(case):
    name, cfg, st, inp = case
    b, g = inp.boxes, inp.ng
    sold, force, sflux = inp.fabs("state", 0), inp.fabs("scal_force", 0), inp.fabs("sflux", 0)
    snew = zeros_like(inp.fabs("state", g))
    snew_gpu = to_mf(snew, b, g)
    args = (to_mf(sold, b, 0), snew_gpu, [to_mf(sflux[d], b, 0, d) for d in range(3)], to_mf(force, b, 0))
    st.update_scal(*args, FIRSTSPEC, inp.nspec)
    pyoracle.member(cfg, "update_scal", {"state": sold, "snew": snew, "sflux": sflux, "force": force},
                    start_comp=FIRSTSPEC, num_comp=inp.nspec)
    worst, bitwise = compare(snew_gpu, snew, [RHO] + list(range(FIRSTSPEC, inp.nscal)), f"{name} snew species")
    assert bitwise, worst
    st.update_scal(*args, RHOH, 1)
    pyoracle.member(cfg, "update_scal", {"state": sold, "snew": snew, "sflux": sflux, "force": force},
                    start_comp=RHOH, num_comp=1)
    worst, bitwise = compare(snew_gpu, snew, [RHOH], f"{name} snew rhoh")
    assert bitwise, worst


def test_member_entries_reject_what_they_do_not_cover():
    from maestroex_gb300.capi import MadvError
    cfg = planar(1)
    st, inp = make_stage(cfg), MemberInputs(cfg)
    b, g = inp.boxes, inp.ng
    state = to_mf(inp.fabs("state", g), b, g)
    umac = [to_mf(inp.fabs("uface", 1)[d], b, 1, d) for d in range(3)]
    force = to_mf(inp.fabs("scal_force", 1), b, 1)
    out = [MultiFab(b, inp.nscal, 0, nodal=d) for d in range(3)]
    with pytest.raises(MadvError) as e:  # velocity edge states are not built
        st.make_edge_scal(state, out, umac, force, 1, 0, 0, 3, 0)
    assert e.value.code == -3
    with pytest.raises(MadvError):  # too few ghost cells in the state
        st.make_edge_scal(to_mf(inp.fabs("state", 1), b, 1), out, umac, force, 0, RHOH, RHOH, 1, 0)
