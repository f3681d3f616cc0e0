"""GPU parity of the 2-D stage (the reference's AMREX_SPACEDIM == 2 code, y radial)
against the CPU oracle's 2-D restatement: every output component within 1e-12 of its
max-norm (in practice bitwise)."""
import numpy as np
import pytest

import pyoracle
from maestroex_gb300 import capi, configs
from maestroex_gb300.params import FIRSTSPEC, INTERIOR, NOSLIPWALL, OUTFLOW, RHO, RHOH, SLIPWALL, SYMMETRY
from helpers import rel_err

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _built():
    from maestroex_gb300 import build
    build.build_library()


def compare_2d(cfg, gpu, ref, label):
    comps = [RHO, RHOH] + list(range(FIRSTSPEC, FIRSTSPEC + cfg["nspec"]))
    bitwise = True
    for d in range(2):
        e = rel_err(gpu["umac_end"][d], ref["umac_end"][d])
        assert e <= TOL, f"{label} umac[{d}] {e}"
        bitwise &= np.array_equal(gpu["umac_end"][d], ref["umac_end"][d])
        for key in ("sedge", "sflux"):
            for c in comps:
                e = rel_err(gpu[key][d][c], ref[key][d][c])
                assert e <= TOL, f"{label} {key}[{d}] comp {c} {e}"
                bitwise &= np.array_equal(gpu[key][d][c], ref[key][d][c])
    for key in ("snew", "sold_end"):
        for c in comps:
            e = rel_err(gpu[key][c], ref[key][c])
            assert e <= TOL, f"{label} {key} comp {c} {e}"
            bitwise &= np.array_equal(gpu[key][c], ref[key][c])
    e = rel_err(gpu["etarhoflux"], ref["etarhoflux"])
    assert e <= TOL, f"{label} etarhoflux {e}"
    return bitwise


def run_both(cfg, mode=capi.MODE_BATCHED):
    from maestroex_gb300.stage import run_stage_gpu
    return run_stage_gpu(cfg, mode=mode), pyoracle.run_stage_2d(cfg)


@pytest.mark.parametrize("ppm_type", [1, 2, 0])
def test_2d_stage(ppm_type):
    cfg = configs.planar_config_2d(n=(48, 64), nspec=3, ppm_type=ppm_type, max_grid=16, rho_pert=1e-3, w0_amp=1e4,
                                   gpi_amp=1e-5, seed=901 + ppm_type)
    gpu, ref = run_both(cfg)
    assert compare_2d(cfg, gpu, ref, f"2d ppm{ppm_type}")


@pytest.mark.parametrize("case", ["walls", "symmetry", "noslip"])
def test_2d_boundaries(case):
    bc = {"walls": ((SLIPWALL, OUTFLOW), (OUTFLOW, SLIPWALL)),
          "symmetry": ((SYMMETRY, SLIPWALL), (SYMMETRY, OUTFLOW)),
          "noslip": ((NOSLIPWALL, NOSLIPWALL), (OUTFLOW, NOSLIPWALL))}[case]
    cfg = configs.planar_config_2d(n=(40, 48), nspec=2, ppm_type=2, max_grid=16, bc_lo=bc[0], bc_hi=bc[1],
                                   rho_pert=1e-3, w0_amp=1e4, gpi_amp=1e-5, seed=911)
    gpu, ref = run_both(cfg)
    assert compare_2d(cfg, gpu, ref, case)


def test_2d_prediction_types_and_modes():
    cfg = configs.planar_config_2d(n=(32, 32), nspec=2, ppm_type=1, max_grid=16, rho_pert=1e-3, w0_amp=1e4,
                                   species_pred_type=2, enthalpy_pred_type=0, seed=921)
    gpu, ref = run_both(cfg, mode=capi.MODE_PER_BOX)
    assert compare_2d(cfg, gpu, ref, "spt2")
    from maestroex_gb300.stage import run_stage_gpu
    g = run_stage_gpu(cfg, mode=capi.MODE_GRAPH)
    assert np.array_equal(g["snew"], gpu["snew"])


def test_one_256_box():
    """2-D, one 256 x 256 box, NumSpec 3, ppm_type 1, w0 = 0."""
    cfg = configs.workload_2d(n=256)
    gpu, ref = run_both(cfg)
    assert compare_2d(cfg, gpu, ref, "256 x 256")


@pytest.mark.parametrize("spt", [1, 2])
def test_2d_enthalpy_prediction_of_h(spt):
    """enthalpy_pred_type 2: h = (rho h) / rho predicted, the flux rho h u."""
    cfg = configs.planar_config_2d(n=(32, 48), nspec=3, ppm_type=1, max_grid=16, rho_pert=1e-3, w0_amp=1e4,
                                   species_pred_type=spt, enthalpy_pred_type=2, seed=931 + spt)
    gpu, ref = run_both(cfg)
    assert compare_2d(cfg, gpu, ref, f"ept2 spt{spt}")
