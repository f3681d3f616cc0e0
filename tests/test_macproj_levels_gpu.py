"""GPU MAC projection on two plane-parallel levels (madv_mac_project_levels): the composite
solve against the oracle's direct solve of the same composite system
(oracle/mo_macproj_levels.py), level by level.  The GPU conjugate gradients stop at
max|residual| <= tol_rel max|rhs| (1e-12 here), so the projected velocities agree with the
exact discrete solution to 1e-8 of max|u|, not bitwise.  Also: a level 1 covering the whole
domain gives the one-level projection at the fine resolution, and the rejections."""
import numpy as np
import pytest
import torch

import mo_macproj
import mo_macproj_levels
from maestroex_gb300 import capi, configs
from maestroex_gb300.params import INTERIOR, OUTFLOW, RHO, SLIPWALL, SYMMETRY
from maestroex_gb300.stage import MultiFab, make_amr_stage

pytestmark = pytest.mark.gpu

CASES = {
    "periodic_xy_outflow_z": ((INTERIOR, INTERIOR, SYMMETRY), (INTERIOR, INTERIOR, OUTFLOW)),
    "all_periodic": ((INTERIOR,) * 3, (INTERIOR,) * 3),
    "outflow_x_walls_z": ((OUTFLOW, INTERIOR, SLIPWALL), (OUTFLOW, INTERIOR, SLIPWALL)),
}
FINE = [(4, 4, 4, 11, 13, 9), (12, 4, 6, 19, 9, 13), (20, 16, 16, 27, 27, 27)]


def face_field(rng, n, bc, scale):
    nx, ny, nz = n
    u = [scale * rng.standard_normal(s) for s in ((nz, ny, nx + 1), (nz, ny + 1, nx), (nz + 1, ny, nx))]
    for d in range(3):  # periodic copies agree, walls carry no flux
        v = np.moveaxis(u[d], 2 - d, -1)
        if bc[0][d] == INTERIOR:
            v[..., -1] = v[..., 0]
        else:
            if bc[0][d] != OUTFLOW:
                v[..., 0] = 0.0
            if bc[1][d] != OUTFLOW:
                v[..., -1] = 0.0
    return u


def inputs(bc, fine=FINE, n0=(16, 16, 16), seed=20261203 + 80):
    cfg = configs.planar_amr_config(n0=n0, nspec=2, ppm_type=1, max_grid=8, fine_boxes=fine, bc_lo=bc[0],
                                    bc_hi=bc[1], seed=seed, rho_pert=1e-2, w0_amp=0.0)
    rng = np.random.default_rng(seed)
    lev = []
    for L in cfg["levels"]:
        nx, ny, nz = L["n"]
        umax = float(np.nanmax(np.abs(L["uold"])))
        beta0 = np.asarray(L["rho0_old"]) * (1.0 + 0.1 * np.linspace(0.0, 1.0, nz))
        if bc[0][2] == INTERIOR:
            beta0 = np.full(nz, float(beta0.mean()))
        lev.append(dict(umac=face_field(rng, L["n"], bc, umax), rho=np.nan_to_num(L["sold"][RHO], nan=1.0),
                        beta0=beta0,
                        macrhs=1e-3 * umax / L["dx"][0] * beta0[:, None, None] * rng.standard_normal((nz, ny, nx))))
    # one radial profile seen at both resolutions: level 1's rows are level 0's, halved
    lev[1]["beta0"] = np.repeat(lev[0]["beta0"], 2)
    return cfg, lev


def run_gpu(cfg, lev, tol=1e-12):
    st = make_amr_stage(cfg)
    um, rh, ro, ph = [], [], [], []
    for L, a in zip(cfg["levels"], lev):
        b = L["boxes"]
        faces = [MultiFab(b, 1, 1, nodal=d) for d in range(3)]
        for d in range(3):
            faces[d].from_domain(torch.from_numpy(np.ascontiguousarray(a["umac"][d][None])).cuda())
        um.append(faces)
        rh.append(MultiFab(b, 1, 0).from_domain(torch.from_numpy(a["macrhs"][None]).cuda()))
        ro.append(MultiFab(b, 1, 0).from_domain(torch.from_numpy(a["rho"][None]).cuda()))
        ph.append(MultiFab(b, 1, 0))
    it, ratio = st.mac_project_levels(um, rh, ro, [a["beta0"] for a in lev], macphi=ph, tol_rel=tol, max_iter=400)
    torch.cuda.synchronize()
    out = [dict(u=[um[l][d].to_domain(L["n"])[0].cpu().numpy() for d in range(3)],
                phi=ph[l].to_domain(L["n"])[0].cpu().numpy()) for l, L in enumerate(cfg["levels"])]
    st.close()
    return out, it, ratio


def oracle(cfg, lev, bc):
    L0, L1 = cfg["levels"]
    return mo_macproj_levels.mac_project_levels(lev[0]["umac"], lev[1]["umac"], lev[0]["macrhs"], lev[1]["macrhs"],
                                                lev[0]["rho"], lev[1]["rho"], lev[0]["beta0"], lev[1]["beta0"],
                                                L1["boxes"], L0["dx"], bc[0], bc[1])


@pytest.mark.parametrize("case", sorted(CASES))
def test_two_level_mac_projection_matches_oracle(case):
    bc = CASES[case]
    cfg, lev = inputs(bc)
    gpu, it, ratio = run_gpu(cfg, lev)
    u0, u1, p0, p1 = oracle(cfg, lev, bc)
    assert ratio <= 1e-12 and it > 0
    for l, (ou, op) in enumerate(((u0, p0), (u1, p1))):
        g = gpu[l]
        scale = max(float(np.nanmax(np.abs(ou[d]))) for d in range(3))
        for d in range(3):
            m = np.isfinite(g["u"][d])
            assert np.array_equal(m, np.isfinite(ou[d])) and m.any()
            err = float(np.abs(g["u"][d][m] - ou[d][m]).max()) / scale
            print(f"{case} level {l} u[{d}]: {err:.2e} ({it} iterations)")
            assert err <= 1e-8, (l, d, err)
        mp = np.isfinite(g["phi"])
        perr = float(np.abs(g["phi"][mp] - op[mp]).max()) / float(np.abs(op[mp]).max())
        assert perr <= 1e-8, (l, perr)


def test_fine_level_covering_the_domain_is_the_fine_one_level_projection():
    """With level 1 covering the domain there is no coarse unknown: level 1 is the one-level
    projection at the fine resolution, and level 0's faces the averages of level 1's."""
    bc = CASES["periodic_xy_outflow_z"]
    full = [(0, 0, 0, 15, 15, 15), (16, 0, 0, 31, 31, 15), (0, 16, 0, 15, 31, 15), (0, 0, 16, 31, 31, 31)]
    cfg, lev = inputs(bc, fine=full)
    gpu, it, ratio = run_gpu(cfg, lev)
    L1 = cfg["levels"][1]
    u1, p1 = mo_macproj.mac_project(lev[1]["umac"], lev[1]["macrhs"], lev[1]["rho"], lev[1]["beta0"], L1["dx"],
                                    bc[0], bc[1])
    scale = max(float(np.abs(u1[d]).max()) for d in range(3))
    for d in range(3):
        assert float(np.abs(gpu[1]["u"][d] - u1[d]).max()) / scale <= 1e-8
        # the level-0 faces: means of the four level-1 faces under them
        f = u1[d]
        t = [a for a in range(3) if a != d]
        acc = 0.0
        for q in range(4):
            s = [slice(0, None, 2)] * 3
            s[2 - t[0]] = slice(q & 1, None, 2)
            s[2 - t[1]] = slice(q >> 1, None, 2)
            acc = acc + f[tuple(s)]
        assert float(np.abs(gpu[0]["u"][d] - 0.25 * acc).max()) / scale <= 1e-8


def test_two_level_mac_projection_rejections():
    cfg, lev = inputs(CASES["all_periodic"])
    st = make_amr_stage(cfg)
    with pytest.raises(capi.MadvError) as e:  # one entry per level
        st.mac_project_levels([[MultiFab(cfg["levels"][0]["boxes"], 1, 1, nodal=d) for d in range(3)]],
                              [MultiFab(cfg["levels"][0]["boxes"], 1, 0)], [MultiFab(cfg["levels"][0]["boxes"], 1, 0)],
                              [lev[0]["beta0"]])
    assert e.value.code == -1  # MADV_ERR_PARAM
    st.close()
