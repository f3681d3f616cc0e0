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


# ---------------------------------------------------------------------------- whole stage
# The stage as the reference's AdvanceTimeStep predictor runs it (AdvancePremac, Addw0,
# DensityAdvance, EnthalpyAdvance; MAC projection skipped), every Maestro function on the
# path compiled from the reference sources (MakeUtrans, VelPred, MakeVelForce,
# MakeEdgeScal, PPM, Slopes, MakeRhoXFlux, MakeRhoHFlux, UpdateScal, ModifyScalForce,
# MakeRhoHForce, PutInPertForm, ConvertRhoXToX, Put1dArrayOnCart, Addw0, MakeW0mac,
# MakeS0mac, CelltoEdge, FillPatch, FillUmacGhost, ScalarFill / VelFill / FillExtBC,
# BaseStateGeometry), only AMReX's containers and its generic fills restated in
# oracle/refshim/AMReX_shim.H.

def stage_cases():
    from maestroex_gb300.params import INTERIOR, NOSLIPWALL, OUTFLOW, SLIPWALL, SYMMETRY
    C = {}
    for ppm in (1, 2, 0):
        C[f"planar ppm{ppm}"] = lambda ppm=ppm: configs.planar_config(n=(32, 32, 32), nspec=3, ppm_type=ppm,
                                                                     max_grid=16, seed=101 + ppm)
    bcs = [((SYMMETRY, SLIPWALL, SLIPWALL), (OUTFLOW, NOSLIPWALL, OUTFLOW)),
           ((OUTFLOW, INTERIOR, NOSLIPWALL), (SYMMETRY, INTERIOR, SLIPWALL)),
           ((SLIPWALL, OUTFLOW, SYMMETRY), (SLIPWALL, SYMMETRY, SYMMETRY))]
    for i, (lo, hi) in enumerate(bcs):
        for ppm in (1, 2):
            C[f"walls{i} ppm{ppm}"] = lambda lo=lo, hi=hi, i=i, ppm=ppm: configs.planar_config(
                n=(24, 16, 24), nspec=2, ppm_type=ppm, max_grid=(8, 16, 12), bc_lo=lo, bc_hi=hi, seed=200 + i, cfl=0.5)
    for so in (2, 4, 0):
        C[f"ppm0 slope_order {so}"] = lambda so=so: configs.planar_config(
            n=(16, 16, 24), nspec=2, ppm_type=0, slope_order=so, max_grid=8, bc_lo=(SLIPWALL, INTERIOR, SLIPWALL),
            bc_hi=(OUTFLOW, INTERIOR, OUTFLOW), seed=300 + so)
    for spt, ept in [(2, 1), (3, 1), (1, 0), (2, 0), (1, 2), (2, 2), (3, 2)]:
        C[f"species_pred_type {spt} enthalpy_pred_type {ept}"] = lambda spt=spt, ept=ept: configs.planar_config(
            n=(16, 24, 16), nspec=3, ppm_type=1, max_grid=8, species_pred_type=spt, enthalpy_pred_type=ept,
            seed=400 + 10 * spt + ept)
    C["uneven boxes ppm2"] = lambda: configs.planar_config(
        n=(48, 32, 40), nspec=2, ppm_type=2, boxes=configs.uneven_boxes((48, 32, 40), [8, 16, 24],
                                                                       np.random.default_rng(5)), seed=501)
    for ppm in (1, 2, 0):
        C[f"spherical ppm{ppm}"] = lambda ppm=ppm: configs.spherical_config(n=32, max_grid=16, ppm_type=ppm)
    C["NumSpec 13, 32^3 boxes, w0"] = lambda: configs.planar_config(n=(64, 64, 64), nspec=13, ppm_type=1,
                                                                    max_grid=32, seed=7, w0_amp=1e4)

    def traced(cfg):
        cfg["ppm_trace_forces"] = 1
        return cfg

    for ppm in (1, 2):
        C[f"traced forces ppm{ppm}"] = lambda ppm=ppm: traced(configs.planar_config(
            n=(32, 32, 32), nspec=3, ppm_type=ppm, max_grid=16, seed=101 + ppm, gpi_amp=1e-3, rho_pert=1e-3))
    C["traced forces, walls"] = lambda: traced(configs.planar_config(
        n=(24, 16, 24), nspec=2, ppm_type=2, max_grid=(8, 16, 12), bc_lo=(SYMMETRY, SLIPWALL, SLIPWALL),
        bc_hi=(OUTFLOW, NOSLIPWALL, OUTFLOW), seed=200, cfl=0.5, gpi_amp=1e-3))
    C["traced forces, spherical"] = lambda: traced(configs.spherical_config(n=32, max_grid=16, ppm_type=2))
    # spherical with uniform radial bins (use_exact_base_state = 0, the reference's default):
    # every interpolation type of Put1dArrayOnCart, MakeW0mac and MakeS0mac, drdxfac, rhoh
    inexact = {"uniform bins": {}, "uniform bins, rhoh predicted": {"enthalpy_pred_type": 0},
               "uniform bins, w0 constant, s0 linear": {"w0_interp_type": 1, "s0_interp_type": 2},
               "uniform bins, w0 quadratic, s0 constant": {"w0_interp_type": 3, "s0_interp_type": 1},
               "uniform bins, w0mac linear, s0mac linear": {"w0mac_interp_type": 2, "s0mac_interp_type": 2},
               "uniform bins, w0mac quadratic, s0mac quadratic": {"w0mac_interp_type": 3, "s0mac_interp_type": 3},
               "uniform bins, w0mac nodal, drdxfac 5": {"w0mac_interp_type": 4, "drdxfac": 5},
               "uniform bins, h predicted": {"enthalpy_pred_type": 2},
               "uniform bins, h predicted, rhoX": {"enthalpy_pred_type": 2, "species_pred_type": 2}}
    for name, kw in inexact.items():
        ept = kw.pop("enthalpy_pred_type", 1)
        spt = kw.pop("species_pred_type", 1)
        for ppm in (1, 2):
            C[f"spherical {name} ppm{ppm}"] = lambda kw=kw, ept=ept, spt=spt, ppm=ppm: dict(
                configs.spherical_config(n=16, max_grid=8, ppm_type=ppm, exact=False, **kw), enthalpy_pred_type=ept,
                species_pred_type=spt)
    for name, kw in {"w0 constant": {"w0_interp_type": 1}, "w0 quadratic": {"w0_interp_type": 3},
                     "w0mac nodal": {"w0mac_interp_type": 4}, "w0mac quadratic": {"w0mac_interp_type": 3}}.items():
        C[f"spherical exact grid, {name}"] = lambda kw=kw: configs.spherical_config(n=16, max_grid=8, ppm_type=1, **kw)

    def negative_species():
        from test_bench_shapes_gpu import headline_shape, plant_negative_species
        cfg = headline_shape(13, n=(64, 64, 64), seed=20261203 + 21)
        plant_negative_species(cfg)
        return cfg

    C["NumSpec 13, negative species planted"] = negative_species
    return C


STAGE_CASES = stage_cases()


def assert_stage_bitwise(cfg, a, b, label):
    from maestroex_gb300.params import FIRSTSPEC, RHO, RHOH
    comps = [RHO, RHOH] + list(range(FIRSTSPEC, FIRSTSPEC + cfg["nspec"]))
    for key in ("umac_vp", "umac_end"):
        for d in range(3):
            assert np.array_equal(a[key][d], b[key][d]), f"{label}: {key}[{d}]"
    for key in ("sedge", "sflux"):
        for d in range(3):
            for c in comps:
                assert np.array_equal(a[key][d][c], b[key][d][c]), f"{label}: {key}[{d}] comp {c}"
    for key in ("snew", "sold_end"):
        for c in comps:
            assert np.array_equal(a[key][c], b[key][c]), f"{label}: {key} comp {c}"
    assert np.array_equal(a["etarhoflux"], b["etarhoflux"]), f"{label}: etarhoflux"


@pytest.mark.parametrize("case", list(STAGE_CASES))
def test_stage_matches_reference_source(case):
    cfg = STAGE_CASES[case]()
    ours = pyoracle.run_stage(cfg, checked=True)
    ref = pyref.run_stage(cfg)
    assert_stage_bitwise(cfg, ours, ref, case)


@pytest.mark.parametrize("ppm_type,is_cons", [(1, 0), (1, 1), (2, 0), (0, 1)])
def test_make_edge_scal_member_matches_reference_source(ppm_type, is_cons):
    """Maestro::MakeEdgeScal on caller FABs whose ghost cells hold arbitrary values (every
    boundary branch reads them as given)."""
    from members import MemberInputs, zeros_like
    cfg = configs.planar_config(n=(32, 32, 32), max_grid=16, ppm_type=ppm_type, seed=33 + ppm_type)
    mi = MemberInputs(cfg)
    outs = []
    for L in (pyoracle, pyref):
        sedge = [zeros_like(f) for f in mi.fabs("sedge")]
        args = dict(state=mi.fabs("state", mi.ng), force=mi.fabs("scal_force", 1), umac=mi.fabs("uface", 1),
                    sedge=sedge)
        L.member(cfg, "make_edge_scal", args, start_comp=0, num_comp=mi.nscal, is_conservative=is_cons)
        outs.append(sedge)
    for d in range(3):
        for b in range(len(cfg["boxes"])):
            assert np.array_equal(outs[0][d][b][0], outs[1][d][b][0]), (d, b)


# ------------------------------------------------------------------- VelocityAdvance
def velocity_cases():
    from maestroex_gb300.params import OUTFLOW, SLIPWALL
    return {
        "planar ppm1": lambda: configs.planar_config(n=(32, 32, 32), max_grid=16, ppm_type=1),
        "planar ppm2 outflow": lambda: configs.planar_config(n=(32, 32, 32), max_grid=16, ppm_type=2,
                                                             bc_lo=(OUTFLOW, SLIPWALL, SLIPWALL),
                                                             bc_hi=(OUTFLOW, OUTFLOW, OUTFLOW)),
        "planar ppm0": lambda: configs.planar_config(n=(32, 32, 32), max_grid=16, ppm_type=0),
        "spherical ppm2": lambda: configs.spherical_config(n=32, max_grid=16, ppm_type=2),
        "spherical uniform bins ppm2": lambda: configs.spherical_config(n=16, max_grid=8, ppm_type=2, exact=False),
        "spherical uniform bins, w0mac nodal, s0 linear": lambda: configs.spherical_config(
            n=16, max_grid=8, ppm_type=1, exact=False, w0mac_interp_type=4, s0_interp_type=2),
        "planar ppm2 traced forces": lambda: dict(configs.planar_config(n=(32, 32, 32), max_grid=16, ppm_type=2,
                                                                        gpi_amp=1e-3), ppm_trace_forces=1),
    }


VELOCITY_CASES = velocity_cases()


@pytest.mark.parametrize("name", list(VELOCITY_CASES))
@pytest.mark.parametrize("with_sponge", [False, True])
def test_velocity_advance_matches_reference_source(name, with_sponge):
    """AdvancePremac, then Maestro::VelocityAdvance with UpdateVel (and the sponge)."""
    from maestroex_gb300.params import RHO
    cfg = VELOCITY_CASES[name]()
    rng = np.random.default_rng(17)
    rhohalf = cfg["sold"][RHO] * (1.0 + 1e-4 * rng.standard_normal(cfg["sold"][RHO].shape))
    sponge = rng.uniform(0.5, 1.0, size=rhohalf.shape) if with_sponge else None
    ours = pyoracle.run_velocity_advance(cfg, rhohalf, sponge, checked=True)
    ref = pyref.run_velocity_advance(cfg, rhohalf, sponge)
    for d in range(3):
        assert np.array_equal(ours["umac"][d], ref["umac"][d]), f"{name}: umac[{d}]"
        assert np.array_equal(ours["unew"][d], ref["unew"][d]), f"{name}: unew comp {d}"


# --------------------------------------------------------------------------- 2-D stage
# the reference built with AMREX_SPACEDIM = 2 (its 2-D branches: y radial, two velocity
# components), the same predictor sequence
def stage_cases_2d():
    from maestroex_gb300.params import NOSLIPWALL, OUTFLOW, SLIPWALL, SYMMETRY
    C = {}
    for ppm in (1, 2, 0):
        C[f"2-D ppm{ppm}"] = lambda ppm=ppm: configs.planar_config_2d(n=(48, 64), nspec=3, ppm_type=ppm, max_grid=16,
                                                                     rho_pert=1e-3, w0_amp=1e4)
    C["2-D walls ppm2"] = lambda: configs.planar_config_2d(n=(40, 48), nspec=2, ppm_type=2, max_grid=16,
                                                           bc_lo=(SLIPWALL, NOSLIPWALL), bc_hi=(OUTFLOW, SYMMETRY))
    for spt in (1, 2):
        C[f"2-D enthalpy_pred_type 2, species_pred_type {spt}"] = lambda spt=spt: configs.planar_config_2d(
            n=(32, 48), nspec=3, ppm_type=1, max_grid=16, rho_pert=1e-3, w0_amp=1e4, species_pred_type=spt,
            enthalpy_pred_type=2)
    C["2-D 256^2 one box (the 2-D workload)"] = lambda: configs.workload_2d(n=256)
    return C


STAGE_CASES_2D = stage_cases_2d()


@pytest.mark.parametrize("case", list(STAGE_CASES_2D))
def test_2d_stage_matches_reference_source(case):
    from maestroex_gb300.params import FIRSTSPEC, RHO, RHOH
    cfg = STAGE_CASES_2D[case]()
    a = pyoracle.run_stage_2d(cfg, checked=True)
    b = pyref.run_stage_2d(cfg)
    comps = [RHO, RHOH] + list(range(FIRSTSPEC, FIRSTSPEC + cfg["nspec"]))
    for key in ("umac_vp", "umac_end"):
        for d in range(2):
            assert np.array_equal(a[key][d], b[key][d]), f"{case}: {key}[{d}]"
    for key in ("sedge", "sflux"):
        for d in range(2):
            for c in comps:
                assert np.array_equal(a[key][d][c], b[key][d][c]), f"{case}: {key}[{d}] comp {c}"
    for key in ("snew", "sold_end"):
        for c in comps:
            assert np.array_equal(a[key][c], b[key][c]), f"{case}: {key} comp {c}"
    assert np.array_equal(a["etarhoflux"], b["etarhoflux"]), f"{case}: etarhoflux"
