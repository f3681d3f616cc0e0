"""GPU MAC projection (madv_mac_project, Maestro::MacProj on one level, plane-parallel or
spherical)
against the oracle's direct solve of the same discrete system (oracle/mo_macproj.py).  The
GPU multigrid stops at max|residual| <= tol_rel max|rhs| (tol_rel 1e-12 here), so the
projected velocities agree with the exact discrete solution to a tolerance, not bitwise:
1e-8 of max|u| here.  Also checked: div(beta0 u) = macrhs after the projection, the number
of V-cycles, and the rejection of configurations the entry does not cover."""
import numpy as np
import pytest
import torch

import mo_macproj
from maestroex_gb300 import capi, configs
from maestroex_gb300.params import INTERIOR, OUTFLOW, RHO, SLIPWALL, SYMMETRY
from maestroex_gb300.stage import MultiFab, make_stage

pytestmark = pytest.mark.gpu

CASES = {
    "periodic_xy_outflow_z": ((INTERIOR, INTERIOR, SLIPWALL), (INTERIOR, INTERIOR, OUTFLOW)),
    "all_periodic": ((INTERIOR,) * 3, (INTERIOR,) * 3),
    "walls_z": ((INTERIOR, INTERIOR, SLIPWALL), (INTERIOR, INTERIOR, SLIPWALL)),
    "outflow_x_symmetry_y": ((OUTFLOW, SYMMETRY, SLIPWALL), (OUTFLOW, SLIPWALL, OUTFLOW)),
}


def inputs(bc, n=(32, 32, 48), max_grid=16, seed=20261203 + 70):
    cfg = configs.planar_config(n=n, nspec=2, ppm_type=1, max_grid=max_grid, bc_lo=bc[0], bc_hi=bc[1],
                                rho_pert=1e-2, w0_amp=0.0, seed=seed)
    rng = np.random.default_rng(seed)
    nx, ny, nz = cfg["n"]
    shapes = [(nz, ny, nx + 1), (nz, ny + 1, nx), (nz + 1, ny, nx)]
    umax = float(np.abs(cfg["uold"]).max())
    umac = [umax * rng.standard_normal(s) for s in shapes]
    # a consistent face field: the two copies of a periodic face agree, walls carry no flux
    for d in range(3):
        ax = 2 - d
        u = np.moveaxis(umac[d], ax, -1)
        if bc[0][d] == INTERIOR:
            u[..., -1] = u[..., 0]
        else:
            if bc[0][d] != OUTFLOW:
                u[..., 0] = 0.0
            if bc[1][d] != OUTFLOW:
                u[..., -1] = 0.0
    rho = cfg["sold"][RHO]
    beta0 = cfg["rho0_old"] * (1.0 + 0.1 * np.linspace(0.0, 1.0, nz))
    if bc[0][2] == INTERIOR:  # periodic z: the two copies of a z face see the same beta0
        beta0 = np.full(nz, float(beta0.mean()))
    macrhs = 1e-3 * umax / cfg["dx"][0] * beta0[:, None, None] * rng.standard_normal((nz, ny, nx))
    return cfg, umac, rho, beta0, macrhs


def run_gpu(cfg, umac, rho, beta0, macrhs, tol=1e-12, options=None):
    st = make_stage(cfg)
    for k, v in (options or {}).items():
        st.set_option(k, v)
    boxes = cfg["boxes"]
    um = [MultiFab(boxes, 1, 1, nodal=d) for d in range(3)]
    for d in range(3):
        um[d].from_domain(torch.from_numpy(umac[d][None]).cuda())
    rh = MultiFab(boxes, 1, 0).from_domain(torch.from_numpy(macrhs[None]).cuda())
    ro = MultiFab(boxes, 1, 0).from_domain(torch.from_numpy(rho[None]).cuda())
    phi = MultiFab(boxes, 1, 0)
    it, ratio = st.mac_project(um, rh, ro, beta0, macphi=phi, tol_rel=tol)
    torch.cuda.synchronize()
    n = cfg["n"]
    out = [um[d].to_domain(n)[0].cpu().numpy() for d in range(3)]
    st.close()
    return out, phi.to_domain(n)[0].cpu().numpy(), it, ratio


@pytest.mark.parametrize("case", sorted(CASES))
def test_mac_projection_matches_direct_solve(case):
    bc = CASES[case]
    cfg, umac, rho, beta0, macrhs = inputs(bc)
    gpu, gphi, it, ratio = run_gpu(cfg, umac, rho, beta0, macrhs)
    ref, rphi = mo_macproj.mac_project(umac, macrhs, rho, beta0, cfg["dx"], bc[0], bc[1])
    umax = max(float(np.abs(r).max()) for r in ref)
    err = max(float(np.abs(g - r).max()) for g, r in zip(gpu, ref)) / umax
    print(f"{case}: {it} V-cycles, residual ratio {ratio:.2e}, max |u_gpu - u_direct| / max|u| {err:.2e}")
    assert ratio <= 1e-12 and 1 <= it <= 60
    assert err <= 1e-8
    # the projected field: div(beta0 u) = macrhs (mean-free rhs when every face is Neumann or periodic)
    b0e = mo_macproj.cell_to_edge(beta0)
    bz = [beta0[:, None, None], beta0[:, None, None], b0e[:, None, None]]
    dx = cfg["dx"]

    def div_b0(u):
        bu = [g * b for g, b in zip(u, bz)]
        return ((bu[0][:, :, 1:] - bu[0][:, :, :-1]) / dx[0] + (bu[1][:, 1:] - bu[1][:, :-1]) / dx[1] +
                (bu[2][1:] - bu[2][:-1]) / dx[2])

    div = div_b0(gpu)
    # singular (no Dirichlet face): the solver's rhs is made mean-free, so the projection
    # meets macrhs up to that mean
    singular = case in ("all_periodic", "walls_z")
    target = macrhs - (macrhs - div_b0(umac)).mean() if singular else macrhs
    # to the solve's tolerance, on the scale of the solver's rhs macrhs - div(beta0 u*)
    assert float(np.abs(div - target).max()) <= 1e-10 * float(np.abs(macrhs - div_b0(umac)).max())
    if case in ("all_periodic", "walls_z"):
        assert abs(float(gphi.mean())) <= 1e-12 * float(np.abs(gphi).max())


def test_mac_projection_rejects_two_levels_and_odd_domains():
    from maestroex_gb300.stage import make_amr_stage
    fine = configs.bubble_boxes((16, 16, 16), nbubbles=1, cover=0.2, block_edges=(4,), max_edge=4,
                                rng=np.random.default_rng(3))
    cfg = configs.planar_amr_config(n0=(16, 16, 16), max_grid=8, fine_boxes=fine)
    st = make_amr_stage(cfg)
    boxes = cfg["levels"][0]["boxes"]
    um = [MultiFab(boxes, 1, 1, nodal=d) for d in range(3)]
    cell = MultiFab(boxes, 1, 0, fill=1.0)
    with pytest.raises(capi.MadvError) as e:  # the composite two-level solve is not built
        st.mac_project(um, cell, cell, np.ones(16))
    assert e.value.code == -3
    st.close()
    bc = CASES["periodic_xy_outflow_z"]
    cfg2, *_ = inputs(bc, n=(32, 32, 31), max_grid=32)
    st = make_stage(cfg2)
    um = [MultiFab(cfg2["boxes"], 1, 1, nodal=d) for d in range(3)]
    cell = MultiFab(cfg2["boxes"], 1, 0, fill=1.0)
    with pytest.raises(capi.MadvError) as e:
        st.mac_project(um, cell, cell, np.ones(31))
    assert e.value.code == -3


@pytest.mark.parametrize("case", ["walls_z", "periodic_xy_outflow_z"])
def test_mac_projection_on_extents_that_are_not_powers_of_two(case):
    """40 x 40 x 60 cells: the multigrid coarsens to 10 x 10 x 15 (x and the periodic y stay
    even, z goes odd) and still converges in a few V-cycles."""
    bc = CASES[case]
    cfg, umac, rho, beta0, macrhs = inputs(bc, n=(40, 40, 60), max_grid=20)
    gpu, gphi, it, ratio = run_gpu(cfg, umac, rho, beta0, macrhs)
    ref, rphi = mo_macproj.mac_project(umac, macrhs, rho, beta0, cfg["dx"], bc[0], bc[1])
    umax = max(float(np.abs(r).max()) for r in ref)
    err = max(float(np.abs(g - r).max()) for g, r in zip(gpu, ref)) / umax
    assert ratio <= 1e-12 and 1 <= it <= 40, (it, ratio)
    assert err <= 1e-8


@pytest.mark.parametrize("case,n", [(c, (64, 64, 48)) for c in sorted(CASES)] +
                         [("walls_z", (40, 40, 60)), ("periodic_xy_outflow_z", (128, 128, 128))])
def test_mac_block_cycle_is_bitwise_the_launch_per_step_cycle(case, n):
    """The V-cycle's coarse grids (<= 4096 cells) in one thread block (option mg_block_cycle,
    the default) give the same bits as one launch per sweep, residual, restriction and
    prolongation: the same per-cell arithmetic in the same order."""
    bc = CASES[case]
    cfg, umac, rho, beta0, macrhs = inputs(bc, n=n, max_grid=32 if n[0] % 32 == 0 else 20)
    a = run_gpu(cfg, umac, rho, beta0, macrhs, options={"mg_block_cycle": 1})
    b = run_gpu(cfg, umac, rho, beta0, macrhs, options={"mg_block_cycle": 0})
    assert a[2] == b[2] and a[3] == b[3]
    for x, y in zip(a[0], b[0]):
        assert np.array_equal(x, y)
    assert np.array_equal(a[1], b[1])


def test_mac_projection_removes_an_analytic_gradient():
    """A closed form, independent of the oracle's restatement: with constant rho and beta0 on
    a periodic box, u* = grad psi (face differences of psi = cos(2 pi x / Lx) + sin(4 pi y /
    Ly) cos(2 pi z / Lz)) is removed entirely, and phi = (rho / beta0) psi up to a constant."""
    bc = CASES["all_periodic"]
    cfg, umac, rho, beta0, macrhs = inputs(bc, n=(32, 24, 16), max_grid=16)
    nx, ny, nz = cfg["n"]
    dx = cfg["dx"]
    x = (np.arange(nx) + 0.5) / nx
    y = (np.arange(ny) + 0.5) / ny
    z = (np.arange(nz) + 0.5) / nz
    psi = (np.cos(2 * np.pi * x)[None, None, :] + np.sin(4 * np.pi * y)[None, :, None] *
           np.cos(2 * np.pi * z)[:, None, None])
    psi = psi * float(np.abs(cfg["uold"]).max()) * dx[0]

    def grad(p, d):  # face differences, periodic: face 0 and face n carry the same value
        ax = 2 - d
        g = (p - np.roll(p, 1, axis=ax)) / dx[d]
        return np.concatenate([g, np.take(g, [0], axis=ax)], axis=ax)

    ustar = [grad(psi, d) for d in range(3)]
    rho_c, beta_c = 2.5e7, 3.0e7
    rho = np.full((nz, ny, nx), rho_c)
    beta0 = np.full(nz, beta_c)
    gpu, gphi, it, ratio = run_gpu(cfg, ustar, rho, beta0, np.zeros((nz, ny, nx)))
    umax = max(float(np.abs(u).max()) for u in ustar)
    assert max(float(np.abs(u).max()) for u in gpu) <= 1e-8 * umax
    want = rho_c / beta_c * psi
    assert float(np.abs((gphi - gphi.mean()) - (want - want.mean())).max()) <= 1e-8 * float(np.abs(want).max())


def oracle_beta_faces(cfg, beta0):
    """beta0 on the faces of a spherical configuration: the oracle's MakeS0mac (mo_member),
    gathered from the boxes into domain face arrays."""
    import pyoracle
    c = dict(cfg)
    c["rho0_old"] = np.asarray(beta0, dtype=np.float64)
    nx, ny, nz = cfg["n"]
    fabs = []
    for d in range(3):
        per_box = []
        for b in cfg["boxes"]:
            lo = [b[e] - 1 for e in range(3)]
            ext = [b[3 + e] - b[e] + 3 + (1 if e == d else 0) for e in range(3)]
            per_box.append((np.zeros((1, ext[2], ext[1], ext[0])), lo))
        fabs.append(per_box)
    pyoracle.member(c, "make_s0mac", {"umac": fabs})
    out = []
    for d in range(3):
        shape = [nz, ny, nx]
        shape[2 - d] += 1
        a = np.full(shape, np.nan)
        for b, (f, lo) in zip(cfg["boxes"], fabs[d]):
            hi = [b[3 + e] + (1 if e == d else 0) for e in range(3)]
            a[b[2]:hi[2] + 1, b[1]:hi[1] + 1, b[0]:hi[0] + 1] = \
                f[0, b[2] - lo[2]:hi[2] - lo[2] + 1, b[1] - lo[1]:hi[1] - lo[1] + 1, b[0] - lo[0]:hi[0] - lo[0] + 1]
        assert not np.isnan(a).any()
        out.append(a)
    return out


@pytest.mark.parametrize("exact", [True, False])
def test_mac_projection_spherical(exact):
    """Spherical geometry (outflow on every face): beta0 on the faces from MakeS0mac of the
    radial beta0, against the direct solve of the same system with the oracle's faces."""
    cfg = configs.spherical_config(n=32, max_grid=16, ppm_type=1, exact=exact)
    rng = np.random.default_rng(20261203 + 71)
    nx, ny, nz = cfg["n"]
    umax = float(np.abs(cfg["uold"]).max())
    umac = [umax * rng.standard_normal(s) for s in [(nz, ny, nx + 1), (nz, ny + 1, nx), (nz + 1, ny, nx)]]
    rho = cfg["sold"][RHO]
    beta0 = cfg["rho0_old"] * (1.0 + 0.1 * np.linspace(0.0, 1.0, cfg["nr"]))
    bf = oracle_beta_faces(cfg, beta0)
    macrhs = 1e-3 * umax / cfg["dx"][0] * float(np.abs(beta0).max()) * rng.standard_normal((nz, ny, nx))
    gpu, gphi, it, ratio = run_gpu(cfg, umac, rho, beta0, macrhs)
    ref, rphi = mo_macproj.mac_project(umac, macrhs, rho, None, cfg["dx"], cfg["bc_lo"], cfg["bc_hi"], beta_faces=bf)
    umax_ref = max(float(np.abs(r).max()) for r in ref)
    err = max(float(np.abs(g - r).max()) for g, r in zip(gpu, ref)) / umax_ref
    print(f"spherical exact={exact}: {it} V-cycles, residual ratio {ratio:.2e}, rel err {err:.2e}")
    assert ratio <= 1e-12 and 1 <= it <= 60
    assert err <= 1e-8
    # div(beta0mac u) = macrhs after the projection
    div = sum(np.diff(g * b, axis=2 - d) / cfg["dx"][d] for d, (g, b) in enumerate(zip(gpu, bf)))
    start = macrhs - sum(np.diff(u * b, axis=2 - d) / cfg["dx"][d] for d, (u, b) in enumerate(zip(umac, bf)))
    assert float(np.abs(div - macrhs).max()) <= 1e-10 * float(np.abs(start).max())
