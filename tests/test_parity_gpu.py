"""GPU parity: the CUDA stage against the CPU oracle on the same seeded inputs.

Bar: every output component within 1e-12 of the oracle, relative to the component's
max-norm (the error definition of the benchmark).  The library evaluates the reference
expressions in the same order without FMA contraction, so in practice the results are
bitwise equal; the tests record that too.
"""
import numpy as np
import pytest

import pyoracle
from maestroex_gb300 import capi, configs
from maestroex_gb300.params import (FIRSTSPEC, INTERIOR, NOSLIPWALL, OUTFLOW, RHO, RHOH, SLIPWALL,
                                    SYMMETRY)
from helpers import per_comp_rel_err, rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _built():
    from maestroex_gb300 import build
    build.build_library()


def compare(cfg, res_gpu, res_ref, label=""):
    nspec = cfg["nspec"]
    comps = [RHO, RHOH] + list(range(FIRSTSPEC, FIRSTSPEC + nspec))
    worst = 0.0
    bitwise = True
    for d in range(3):
        e = rel_err(res_gpu["umac_end"][d], res_ref["umac_end"][d])
        assert e <= TOL, f"{label} umac[{d}] rel err {e}"
        worst = max(worst, e)
        bitwise &= np.array_equal(res_gpu["umac_end"][d], res_ref["umac_end"][d])
        for key in ("sedge", "sflux"):
            for c in comps:
                e = rel_err(res_gpu[key][d][c], res_ref[key][d][c])
                assert e <= TOL, f"{label} {key}[{d}] comp {c} rel err {e}"
                worst = max(worst, e)
                bitwise &= np.array_equal(res_gpu[key][d][c], res_ref[key][d][c])
    for key in ("snew", "sold_end"):
        for c in comps:
            e = rel_err(res_gpu[key][c], res_ref[key][c])
            assert e <= TOL, f"{label} {key} comp {c} rel err {e}"
            worst = max(worst, e)
            bitwise &= np.array_equal(res_gpu[key][c], res_ref[key][c])
    e = rel_err(res_gpu["etarhoflux"], res_ref["etarhoflux"])
    assert e <= TOL, f"{label} etarhoflux rel err {e}"
    return worst, bitwise


def run_both(cfg, mode=capi.MODE_BATCHED):
    from maestroex_gb300.stage import run_stage_gpu
    ref = pyoracle.run_stage(cfg, checked=False)
    gpu = run_stage_gpu(cfg, mode=mode)
    return gpu, ref


@pytest.mark.parametrize("ppm_type", [1, 2, 0])
def test_stage_planar_default_bcs(ppm_type):
    cfg = configs.planar_config(n=(32, 32, 32), nspec=3, ppm_type=ppm_type, max_grid=16, seed=101 + ppm_type)
    gpu, ref = run_both(cfg)
    worst, bitwise = compare(cfg, gpu, ref, f"ppm{ppm_type}")
    assert bitwise, f"not bitwise (worst rel err {worst})"


BC_CASES = [
    ((SYMMETRY, SLIPWALL, SLIPWALL), (OUTFLOW, NOSLIPWALL, OUTFLOW)),
    ((OUTFLOW, INTERIOR, NOSLIPWALL), (SYMMETRY, INTERIOR, SLIPWALL)),
    ((SLIPWALL, OUTFLOW, SYMMETRY), (SLIPWALL, SYMMETRY, SYMMETRY)),
]


@pytest.mark.parametrize("ppm_type", [1, 2])
@pytest.mark.parametrize("case", range(len(BC_CASES)))
def test_stage_boundary_conditions(ppm_type, case):
    lo, hi = BC_CASES[case]
    cfg = configs.planar_config(n=(24, 16, 24), nspec=2, ppm_type=ppm_type, max_grid=(8, 16, 12), bc_lo=lo,
                                bc_hi=hi, seed=200 + case, cfl=0.5)
    gpu, ref = run_both(cfg)
    compare(cfg, gpu, ref, f"bc{case} ppm{ppm_type}")


@pytest.mark.parametrize("slope_order", [2, 4, 0])
def test_stage_slopes(slope_order):
    cfg = configs.planar_config(n=(16, 16, 24), nspec=2, ppm_type=0, slope_order=slope_order, max_grid=8,
                                bc_lo=(SLIPWALL, INTERIOR, SLIPWALL), bc_hi=(OUTFLOW, INTERIOR, OUTFLOW),
                                seed=300 + slope_order)
    gpu, ref = run_both(cfg)
    compare(cfg, gpu, ref, f"slope{slope_order}")


@pytest.mark.parametrize("spt,ept", [(2, 1), (3, 1), (1, 0), (2, 0), (1, 2), (2, 2), (3, 2)])
def test_stage_prediction_types(spt, ept):
    cfg = configs.planar_config(n=(16, 24, 16), nspec=3, ppm_type=1, max_grid=8, species_pred_type=spt,
                                enthalpy_pred_type=ept, seed=400 + 10 * spt + ept)
    gpu, ref = run_both(cfg)
    compare(cfg, gpu, ref, f"spt{spt} ept{ept}")


def test_uneven_boxes():
    rng = np.random.default_rng(5)
    boxes = configs.uneven_boxes((48, 32, 40), [8, 16, 24], rng)
    cfg = configs.planar_config(n=(48, 32, 40), nspec=2, ppm_type=2, boxes=boxes, seed=501)
    gpu, ref = run_both(cfg)
    compare(cfg, gpu, ref, "uneven")


@pytest.mark.parametrize("mode", [capi.MODE_PER_BOX, capi.MODE_GRAPH])
def test_launch_modes_identical(mode):
    from maestroex_gb300.stage import run_stage_gpu
    cfg = configs.planar_config(n=(32, 16, 16), nspec=2, ppm_type=1, max_grid=8, seed=601)
    a = run_stage_gpu(cfg, mode=capi.MODE_BATCHED)
    b = run_stage_gpu(cfg, mode=mode)
    for key in ("snew", "sold_end"):
        assert np.array_equal(a[key], b[key])
    for d in range(3):
        assert np.array_equal(a["sedge"][d], b["sedge"][d])
        assert np.array_equal(a["umac_end"][d], b["umac_end"][d])
    assert b["launches"] > 0


def test_decomposition_independent():
    from maestroex_gb300.stage import run_stage_gpu
    one = configs.planar_config(n=(32, 32, 16), nspec=2, ppm_type=2, boxes=[(0, 0, 0, 31, 31, 15)], seed=701)
    many = dict(one)
    many["boxes"] = configs.tile_boxes((32, 32, 16), (8, 16, 8))
    a = run_stage_gpu(one)
    b = run_stage_gpu(many)
    assert np.array_equal(a["snew"], b["snew"])
    for d in range(3):
        assert np.array_equal(a["sflux"][d], b["sflux"][d])


def test_maestro_entry_points_match_stage():
    """AdvancePremac -> Addw0 -> DensityAdvance -> Addw0 x2 -> EnthalpyAdvance -> Addw0 through
    the individual entry points equals the whole-stage call."""
    import torch
    from maestroex_gb300.stage import StageBuffers, make_stage, run_stage_gpu
    cfg = configs.planar_config(n=(16, 16, 32), nspec=3, ppm_type=1, max_grid=16, seed=801)
    whole = run_stage_gpu(cfg)
    st = make_stage(cfg)
    b = StageBuffers(cfg).load(cfg)
    st.advance_premac(b.uold, b.sold, b.gpi, b.umac)
    st.addw0(b.umac, 1.0)
    st.density_advance(b.sold, b.snew, b.sedge, b.sflux, b.eta, b.umac)
    st.addw0(b.umac, -1.0)
    st.addw0(b.umac, 1.0)
    st.enthalpy_advance(b.sold, b.snew, b.sedge, b.sflux, b.umac, thermal=b.thermal)
    st.addw0(b.umac, -1.0)
    torch.cuda.synchronize()
    n = cfg["n"]
    assert np.array_equal(b.snew.to_domain(n).cpu().numpy()[[0, 1, 4, 5, 6]], whole["snew"][[0, 1, 4, 5, 6]])
    for d in range(3):
        assert np.array_equal(b.sflux[d].to_domain(n).cpu().numpy(), whole["sflux"][d])
        assert np.array_equal(b.umac[d].to_domain(n)[0].cpu().numpy(), whole["umac_end"][d])
    st.close()


def test_corrector_which_step_2_matches_oracle():
    """DensityAdvance / EnthalpyAdvance with which_step 2 (old/new base-state averages in
    the fluxes and in the final MakeRhoHForce) through the entry points, against the oracle."""
    import torch
    from maestroex_gb300.stage import StageBuffers, make_stage
    cfg = configs.planar_config(n=(16, 16, 32), nspec=2, ppm_type=1, max_grid=16, seed=802)
    z = np.linspace(0.0, 1.0, cfg["n"][2])
    cfg["rho0_new"] = cfg["rho0_old"] * (1.0 + 1e-3 * np.sin(3.0 * z))
    cfg["rhoh0_new"] = cfg["rhoh0_old"] * (1.0 - 2e-3 * np.cos(2.0 * z))
    cfg["p0_new"] = cfg["p0_old"] * (1.0 + 5e-4 * z)
    c = dict(cfg)
    c["levels"] = [{k: cfg[k] for k in configs.LEVEL_KEYS}]
    ref = pyoracle.run_stage_levels(c, which_step=2)[0]
    st = make_stage(cfg)
    b = StageBuffers(cfg).load(cfg)
    st.advance_premac(b.uold, b.sold, b.gpi, b.umac)
    st.addw0(b.umac, 1.0)
    st.density_advance(b.sold, b.snew, b.sedge, b.sflux, b.eta, b.umac, which_step=2)
    st.addw0(b.umac, -1.0)
    st.addw0(b.umac, 1.0)
    st.enthalpy_advance(b.sold, b.snew, b.sedge, b.sflux, b.umac, thermal=b.thermal, which_step=2)
    st.addw0(b.umac, -1.0)
    torch.cuda.synchronize()
    n = cfg["n"]
    comps = [RHO, RHOH, FIRSTSPEC, FIRSTSPEC + 1]
    snew = b.snew.to_domain(n).cpu().numpy()
    for cc in comps:
        assert rel_err(snew[cc], ref["snew"][cc]) <= TOL
        for d in range(3):
            assert rel_err(b.sflux[d].to_domain(n).cpu().numpy()[cc], ref["sflux"][d][cc]) <= TOL
    assert rel_err(b.eta.to_domain(n)[0].cpu().numpy(), ref["etarhoflux"]) <= TOL
    st.close()


def test_rejects_bad_layout_and_params():
    from maestroex_gb300.params import make_params
    from maestroex_gb300.stage import ScalarAdvectionStage
    cfg = configs.planar_config(n=(16, 16, 16), nspec=2, max_grid=8)
    st = ScalarAdvectionStage(make_params(cfg))
    with pytest.raises(capi.MadvError) as e:
        st.set_layout([(0, 0, 0, 7, 7, 7)])  # does not cover the domain
    assert e.value.code == -2
    # traced forces need PPM (with ppm_type 0 the reference reads traces it never formed)
    for ppm_type, ptf in ((0, 1), (1, 2)):
        p = make_params(cfg)
        p.ppm_type, p.ppm_trace_forces = ppm_type, ptf
        with pytest.raises(capi.MadvError) as e:
            ScalarAdvectionStage(p)
        assert e.value.code == -3


@pytest.mark.parametrize("y,thr", [(6.0, 0.0), (3.0, 1e-3), (390625.0, 6.45e-3), (1e8 / 256 * 2, 12.5),
                                   (0.1, 1e-300), (7.77e-9, 3.3e5)])
def test_exact_helpers_match_ieee(y, thr):
    import ctypes as C
    nfail = C.c_longlong(-1)
    capi.check(capi.lib().madv_selftest_exact(y, thr, 1 << 24, C.byref(nfail), None))
    assert nfail.value == 0


def test_autotuner_keeps_results_and_round_trips():
    """Block sizes and the PPM form change nothing but speed: the stage after autotuning
    (graph mode) and a second context given the saved table reproduce the untuned result
    bit for bit."""
    from maestroex_gb300.stage import StageBuffers, make_stage
    cfg = configs.planar_config(n=(32, 32, 32), max_grid=16, seed=20261203 + 9)

    def run(st, mode):
        buf = StageBuffers(cfg).load(cfg)
        st.stage_forward(buf.uold, buf.sold, buf.gpi, buf.snew, buf.umac, buf.sedge, buf.sflux, buf.eta,
                         thermal=buf.thermal, mode=mode)
        return buf.snew.to_domain(cfg["n"]).cpu().numpy()

    st = make_stage(cfg)
    ref = run(st, capi.MODE_BATCHED)
    table = st.autotune(lambda: run(st, capi.MODE_BATCHED), candidates=(64, 512, 128))
    assert table and all(v in (64, 128, 512) for k, v in table.items() if not k.endswith("ppm_form"))
    assert table["L0 ppm_form"] in range(5)  # the PPM form chosen for the level
    assert np.array_equal(run(st, capi.MODE_GRAPH), ref, equal_nan=True)
    st2 = make_stage(cfg)
    st2.autotune_apply(table)
    assert np.array_equal(run(st2, capi.MODE_BATCHED), ref, equal_nan=True)


@pytest.mark.parametrize("mode", [capi.MODE_BATCHED, capi.MODE_GRAPH])
def test_caller_layouts_work_in_place_or_through_copies(mode):
    """Caller FABs laid out exactly as the stage's fields (sold / snew with ng_s ghost cells,
    umac with one, edge states and fluxes with none) are worked in directly; FABs with more
    ghost cells go through copies.  Both give the same valid-region results, bit for bit,
    and the in-place path leaves Temp and Pi of the edge states and fluxes zero, as the
    reference's setVal(0) does."""
    import torch
    from maestroex_gb300.params import PI, TEMP
    from maestroex_gb300.stage import MultiFab, StageBuffers, make_stage
    cfg = configs.planar_config(n=(32, 32, 32), max_grid=16, ppm_type=1)
    st = make_stage(cfg)
    a = StageBuffers(cfg).load(cfg)
    b = StageBuffers(cfg)
    boxes, nscal, g = cfg["boxes"], 4 + cfg["nspec"], a.sold.ng
    b.sold = MultiFab(boxes, nscal, g + 1)
    b.snew = MultiFab(boxes, nscal, g + 1)
    b.umac = [MultiFab(boxes, 1, 2, nodal=d) for d in range(3)]
    b.sedge = [MultiFab(boxes, nscal, 1, nodal=d, fill=7.0) for d in range(3)]
    b.sflux = [MultiFab(boxes, nscal, 1, nodal=d, fill=7.0) for d in range(3)]
    b.load(cfg)
    for buf in (a, b, a):  # the second run of `a` replays or rebuilds the in-place path
        if buf is a:
            buf.load(cfg)
        st.stage_forward(buf.uold, buf.sold, buf.gpi, buf.snew, buf.umac, buf.sedge, buf.sflux, buf.eta,
                         thermal=buf.thermal, mode=mode)
    torch.cuda.synchronize()
    n = cfg["n"]
    for name in ("snew", "sold"):
        assert torch.equal(getattr(a, name).to_domain(n), getattr(b, name).to_domain(n)), name
    for d in range(3):
        assert torch.equal(a.umac[d].to_domain(n), b.umac[d].to_domain(n))
        for name in ("sedge", "sflux"):
            x, y = getattr(a, name)[d].to_domain(n), getattr(b, name)[d].to_domain(n)
            assert torch.equal(x, y), (name, d)
            assert torch.all(x[TEMP:PI + 1] == 0.0)


def test_working_copies_allocated_at_first_use():
    """A context whose stage calls work in the caller's FABs never allocates its own copies
    of sold, snew, umac, sedge and sflux; the first entry point that needs them (EstDt here)
    allocates them, and the stage's results stay the same bit for bit."""
    import torch
    from maestroex_gb300.stage import StageBuffers, make_stage
    cfg = configs.planar_config(n=(32, 32, 32), max_grid=16, ppm_type=1, seed=20261203 + 12)
    st = make_stage(cfg)
    a = StageBuffers(cfg).load(cfg)

    def run():
        a.load(cfg)
        st.stage_forward(a.uold, a.sold, a.gpi, a.snew, a.umac, a.sedge, a.sflux, a.eta, thermal=a.thermal,
                         mode=capi.MODE_GRAPH)
        torch.cuda.synchronize()
        return [t.clone() for t in a.snew.fabs] + [t.clone() for m in a.sflux for t in m.fabs]

    first = run()
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    a.load(cfg)
    st.est_dt(a.uold, a.sold, a.gpi)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    nscal, g = 4 + cfg["nspec"], a.sold.ng
    cells = sum((b[3] - b[0] + 1 + 2 * g) * (b[4] - b[1] + 1 + 2 * g) * (b[5] - b[2] + 1 + 2 * g)
                for b in cfg["boxes"])
    faces = sum((b[3] - b[0] + 2) * (b[4] - b[1] + 1) * (b[5] - b[2] + 1) for b in cfg["boxes"])
    deferred = 8 * (2 * nscal * cells + 3 * 2 * nscal * faces)
    assert free0 - free1 >= 0.9 * deferred, (free0 - free1, deferred)
    second = run()
    assert all(torch.equal(x, y) for x, y in zip(first, second))


STAGED_CASES = {
    "planar ppm1": lambda: configs.planar_config(n=(32, 32, 32), nspec=2, ppm_type=1, max_grid=16, seed=701),
    "planar ppm2 walls": lambda: configs.planar_config(n=(24, 16, 24), nspec=2, ppm_type=2, max_grid=(8, 16, 12),
                                                       bc_lo=(SYMMETRY, SLIPWALL, SLIPWALL),
                                                       bc_hi=(OUTFLOW, NOSLIPWALL, OUTFLOW), seed=702, cfl=0.5),
    # odd box extents: rows that miss the bulk copy's 16-byte rules take ordinary loads
    "odd boxes ppm1": lambda: configs.planar_config(n=(21, 18, 20), nspec=2, ppm_type=1,
                                                    boxes=[(0, 0, 0, 10, 8, 9), (11, 0, 0, 20, 8, 9),
                                                           (0, 9, 0, 20, 17, 19), (0, 0, 10, 20, 8, 19)],
                                                    seed=703),
    "odd boxes ppm2": lambda: configs.planar_config(n=(21, 18, 20), nspec=2, ppm_type=2,
                                                    boxes=[(0, 0, 0, 10, 8, 9), (11, 0, 0, 20, 8, 9),
                                                           (0, 9, 0, 20, 17, 19), (0, 0, 10, 20, 8, 19)],
                                                    seed=704),
    "spherical ppm2": lambda: configs.spherical_config(n=32, max_grid=16, ppm_type=2),
}


@pytest.mark.parametrize("name", list(STAGED_CASES))
def test_staged_ppm_sweeps_match_three_launch_form(name):
    """The PPM sweeps staged in shared memory (one kernel per direction) against the
    three-launch form through global memory, bit for bit, in the batched, per-box and graph
    modes, and against the oracle."""
    from maestroex_gb300.stage import StageBuffers, make_stage
    import torch
    cfg = STAGED_CASES[name]()
    outs = {}
    for staged in (0, 1):
        for mode in (capi.MODE_BATCHED, capi.MODE_PER_BOX, capi.MODE_GRAPH):
            st = make_stage(cfg)
            st.set_option("staged_ppm", staged)
            buf = StageBuffers(cfg).load(cfg)
            st.stage_forward(buf.uold, buf.sold, buf.gpi, buf.snew, buf.umac, buf.sedge, buf.sflux, buf.eta,
                             thermal=buf.thermal, mode=mode)
            torch.cuda.synchronize()
            n = cfg["n"]
            outs[(staged, mode)] = (buf.snew.to_domain(n).cpu().numpy(),
                                    [buf.sedge[d].to_domain(n).cpu().numpy() for d in range(3)],
                                    [buf.umac[d].to_domain(n).cpu().numpy() for d in range(3)])
            st.close()
    ref = outs[(0, capi.MODE_BATCHED)]
    for key, o in outs.items():
        assert np.array_equal(o[0], ref[0]), (name, key, "snew")
        for d in range(3):
            assert np.array_equal(o[1][d], ref[1][d]), (name, key, "sedge", d)
            assert np.array_equal(o[2][d], ref[2][d]), (name, key, "umac", d)
    oracle = pyoracle.run_stage(cfg, checked=False, want=("snew",))["snew"]
    comps = [RHO, RHOH] + list(range(FIRSTSPEC, FIRSTSPEC + cfg["nspec"]))
    assert np.array_equal(ref[0][comps], oracle[comps])


def test_set_option_rejects_unknown_keys():
    st = make_stage_small()
    with pytest.raises(capi.MadvError):
        st.set_option("no_such_option", 1)
    with pytest.raises(capi.MadvError):
        st.set_option("sweep_tile_1a", 0)
    st.set_option("sweep_tile_1a", 16)
    st.close()


def make_stage_small():
    from maestroex_gb300.stage import make_stage
    return make_stage(configs.planar_config(n=(16, 16, 16), nspec=2, ppm_type=1, max_grid=16, seed=705))


def traced(cfg):
    cfg["ppm_trace_forces"] = 1
    return cfg


TRACED_CASES = {
    "planar ppm1": lambda: traced(configs.planar_config(n=(32, 32, 32), nspec=3, ppm_type=1, max_grid=16, seed=801,
                                                        gpi_amp=1e-3, rho_pert=1e-3)),
    "planar ppm2 walls": lambda: traced(configs.planar_config(n=(24, 16, 24), nspec=2, ppm_type=2,
                                                              max_grid=(8, 16, 12), bc_lo=(SYMMETRY, SLIPWALL, SLIPWALL),
                                                              bc_hi=(OUTFLOW, NOSLIPWALL, OUTFLOW), seed=802, cfl=0.5,
                                                              gpi_amp=1e-3)),
    "spherical ppm2": lambda: traced(configs.spherical_config(n=32, max_grid=16, ppm_type=2)),
    "species 2, h predicted": lambda: traced(configs.planar_config(n=(16, 24, 16), nspec=3, ppm_type=1, max_grid=8,
                                                                   species_pred_type=2, enthalpy_pred_type=2,
                                                                   seed=803)),
}


@pytest.mark.parametrize("name", list(TRACED_CASES))
def test_traced_forces_match_oracle(name):
    """ppm_trace_forces = 1: the velocity and scalar forces traced by PPM (Ipf / Imf) in
    VelPred and MakeEdgeScal, with ng_s ghost cells on the forces."""
    cfg = TRACED_CASES[name]()
    gpu, ref = run_both(cfg, mode=capi.MODE_GRAPH)
    worst, bitwise = compare(cfg, gpu, ref, f"traced forces, {name}")
    assert bitwise, worst
