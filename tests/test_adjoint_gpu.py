"""Adjoint of the multi-step scalar path (madv_stage_adjoint): the gradient of
J = <weight, s_nsteps> with respect to the initial state against central finite
differences of the same GPU forward, with the states differenced before the weights are
applied (J itself is ~1e25 at these magnitudes)."""
import numpy as np
import pytest
import torch

from maestroex_gb300 import configs
from maestroex_gb300.capi import MadvError
from maestroex_gb300.params import (FIRSTSPEC, INTERIOR, NOSLIPWALL, OUTFLOW, PI, RHO, RHOH, SLIPWALL, SYMMETRY,
                                    TEMP)
from maestroex_gb300.stage import MultiFab, make_stage

pytestmark = pytest.mark.gpu


class Case:
    def __init__(self, n=(32, 32, 32), max_grid=16, nspec=3, nsteps=4, ckpt=2, seed=20261203 + 4, bc=None, cfg=None):
        kw = {} if bc is None else dict(bc_lo=bc[0], bc_hi=bc[1])
        if cfg is None:
            cfg = configs.adjoint_config(n=n, max_grid=max_grid, nspec=nspec, seed=seed, **kw)
        self.cfg = cfg
        n, nspec = cfg["n"], cfg["nspec"]
        self.n, self.boxes, self.nscal = cfg["n"], cfg["boxes"], 4 + nspec
        self.nsteps, self.ckpt = nsteps, ckpt
        self.st = make_stage(cfg)
        self.uold = MultiFab(self.boxes, 3, 0).from_domain(cfg["uold"])
        self.sold = MultiFab(self.boxes, self.nscal, 0).from_domain(cfg["sold"])
        rng = np.random.default_rng(seed + 1)
        shape = (n[2], n[1], n[0])
        w = np.zeros((self.nscal,) + shape)
        w[RHOH] = rng.normal(size=shape)
        w[FIRSTSPEC:] = rng.normal(size=(nspec,) + shape)
        self.w = w
        self.weight = MultiFab(self.boxes, self.nscal, 0).from_domain(w)

    def adjoint(self, want_u=False):
        grad = MultiFab(self.boxes, self.nscal, 0, fill=float("nan"))
        gu = MultiFab(self.boxes, 3, 0, fill=float("nan")) if want_u else None
        sfin = MultiFab(self.boxes, self.nscal, 0)
        J, nbytes = self.st.stage_adjoint(self.uold, self.sold, self.weight, self.nsteps, self.ckpt, grad_s=grad,
                                          sfinal=sfin, grad_u=gu)
        torch.cuda.synchronize()
        if want_u:
            return J, grad, sfin, nbytes, gu
        return J, grad, sfin, nbytes

    def final(self, s0, u=None):
        sfin = MultiFab(self.boxes, self.nscal, 0)
        self.st.stage_adjoint(self.uold if u is None else u, s0, self.weight, self.nsteps, self.ckpt, sfinal=sfin)
        return sfin

    def locate(self, i, j, k):
        for b, bx in enumerate(self.boxes):
            if bx[0] <= i <= bx[3] and bx[1] <= j <= bx[4] and bx[2] <= k <= bx[5]:
                return b, (k - bx[2], j - bx[1], i - bx[0])
        raise AssertionError("cell outside the layout")

    def perturbed(self, comp, cell, h, src=None):
        src = self.sold if src is None else src
        s = MultiFab(self.boxes, src.ncomp, 0)
        for a, b in zip(s.fabs, src.fabs):
            a.copy_(b)
        bi, loc = self.locate(*cell)
        s.fabs[bi][(comp,) + loc] += h
        return s

    def dJ(self, a, b):
        return sum(float((w * (x - y)).sum()) for w, x, y in zip(self.weight.fabs, a.fabs, b.fabs))


def test_adjoint_matches_central_differences():
    """Central differences with h = 1e-6 |x| (and h/2 to detect a limiter switch inside
    [x - h, x + h]) at random cells of every differentiated component: density, enthalpy
    and the species, 4 steps with a stored state every 2.  |x| is floored at a tenth of
    the component's RMS, so that h stays above the rounding of the differenced states."""
    case = Case()
    J, grad, _, _ = case.adjoint()
    G = grad.to_domain(case.n).cpu().numpy()
    S = case.cfg["sold"]
    rng = np.random.default_rng(99)
    comps = [RHO, RHOH] + list(range(FIRSTSPEC, case.nscal))
    rms = np.sqrt((S ** 2).mean(axis=(1, 2, 3)))
    worst, checked, kinks = 0.0, 0, 0
    for t in range(60):
        comp = comps[t % len(comps)]
        cell = tuple(int(v) for v in rng.integers(0, case.n[0], size=3))
        i, j, k = cell
        x = max(abs(S[comp, k, j, i]), 0.1 * rms[comp])
        fd = []
        for rel in (1e-6, 0.5e-6):
            h = rel * x
            sp, sm = case.perturbed(comp, cell, h), case.perturbed(comp, cell, -h)
            fd.append(case.dJ(case.final(sp), case.final(sm)) / (2.0 * h))
        scale = max(abs(fd[0]), abs(fd[1]))
        if abs(fd[0] - fd[1]) > 1e-7 * scale:
            kinks += 1
            continue
        g = G[comp, k, j, i]
        err = abs(g - fd[0]) / max(scale, abs(g), 1e-300)
        worst = max(worst, err)
        checked += 1
    assert np.isfinite(J)
    assert checked >= 40, (checked, kinks)
    assert worst <= 1e-6, worst


def test_velocity_adjoint_matches_central_differences():
    """dJ/duold (the velocity held fixed over the steps, so the MAC-velocity adjoints of
    every step go through one transposed VelPred + MakeUtrans) against central
    differences, h = 1e-6 max(|u|, 0.1 rms(u)), with the h/2 check for limiter switches;
    the state gradient of the same call is unchanged by asking for the velocity one."""
    case = Case()
    J, grad, _, _, gu = case.adjoint(want_u=True)
    J0, grad0, _, _ = case.adjoint()
    assert J == J0
    assert np.array_equal(grad.to_domain(case.n).cpu().numpy(), grad0.to_domain(case.n).cpu().numpy()) or \
        np.abs(grad.to_domain(case.n).cpu().numpy() - grad0.to_domain(case.n).cpu().numpy()).max() <= \
        1e-12 * np.abs(grad0.to_domain(case.n).cpu().numpy()).max()
    GU = gu.to_domain(case.n).cpu().numpy()
    U = case.cfg["uold"]
    rms = np.sqrt((U ** 2).mean(axis=(1, 2, 3)))
    rng = np.random.default_rng(123)
    worst, checked, kinks = 0.0, 0, 0
    for t in range(45):
        d = t % 3
        cell = tuple(int(v) for v in rng.integers(0, case.n[0], size=3))
        i, j, k = cell
        x = max(abs(U[d, k, j, i]), 0.1 * rms[d])
        fd = []
        for rel in (1e-6, 0.5e-6):
            h = rel * x
            up = case.perturbed(d, cell, h, src=case.uold)
            um = case.perturbed(d, cell, -h, src=case.uold)
            fd.append(case.dJ(case.final(case.sold, up), case.final(case.sold, um)) / (2.0 * h))
        scale = max(abs(fd[0]), abs(fd[1]))
        if abs(fd[0] - fd[1]) > 1e-7 * scale:
            kinks += 1
            continue
        g = GU[d, k, j, i]
        err = abs(g - fd[0]) / max(scale, abs(g), 1e-300)
        worst = max(worst, err)
        checked += 1
    assert np.all(np.isfinite(GU))
    assert checked >= 30, (checked, kinks)
    assert worst <= 1e-6, worst


class StageSteps(torch.autograd.Function):
    """The multi-step stage as a torch function of (sold0, uold), domain-sized tensors; its
    backward is madv_stage_adjoint with the incoming gradient as the weight.  Used only in
    this gradient-check harness."""

    @staticmethod
    def forward(ctx, s0, u, case):
        ctx.case = case
        sm = MultiFab(case.boxes, case.nscal, 0).from_domain(s0)
        um = MultiFab(case.boxes, 3, 0).from_domain(u)
        ctx.mf = (sm, um)
        out = MultiFab(case.boxes, case.nscal, 0)
        case.st.stage_adjoint(um, sm, case.weight, case.nsteps, case.ckpt, sfinal=out)
        return out.to_domain(case.n)

    @staticmethod
    def backward(ctx, g):
        case = ctx.case
        sm, um = ctx.mf
        w = MultiFab(case.boxes, case.nscal, 0).from_domain(g.contiguous())
        gs = MultiFab(case.boxes, case.nscal, 0)
        gu = MultiFab(case.boxes, 3, 0)
        case.st.stage_adjoint(um, sm, w, case.nsteps, case.ckpt, grad_s=gs, grad_u=gu)
        return gs.to_domain(case.n), gu.to_domain(case.n), None


def test_autograd_wrapper_matches_the_c_abi_adjoint():
    """torch.autograd through StageSteps gives the gradients of the direct call."""
    case = Case(nsteps=2, ckpt=1)
    s0 = torch.from_numpy(case.cfg["sold"]).cuda().requires_grad_(True)
    u = torch.from_numpy(case.cfg["uold"]).cuda().requires_grad_(True)
    w = torch.from_numpy(case.w).cuda()
    J = (w * StageSteps.apply(s0, u, case)).sum()
    gs, gu = torch.autograd.grad(J, (s0, u))
    _, grad, _, _, gud = case.adjoint(want_u=True)
    G, GU = grad.to_domain(case.n), gud.to_domain(case.n)
    for a, b in ((gs, G), (gu, GU)):
        scale = b.abs().amax(dim=(1, 2, 3), keepdim=True).clamp_min(1e-300)
        assert float(((a - b).abs() / scale).max()) <= 1e-12


def test_adjoint_carried_components_and_determinism():
    """Temperature and pi are carried unchanged, so their gradient is the weight; two runs
    give the same J bit for bit and gradients equal to atomic-summation rounding."""
    case = Case(n=(32, 32, 32), max_grid=16, nsteps=3, ckpt=2)
    case.w[TEMP] = 1.0
    case.w[PI] = -2.0
    case.weight.from_domain(case.w)
    J1, g1, s1, nbytes = case.adjoint()
    J2, g2, s2, _ = case.adjoint()
    G1 = g1.to_domain(case.n).cpu().numpy()
    G2 = g2.to_domain(case.n).cpu().numpy()
    assert J1 == J2
    assert np.array_equal(s1.to_domain(case.n).cpu().numpy(), s2.to_domain(case.n).cpu().numpy())
    assert np.all(G1[TEMP] == 1.0) and np.all(G1[PI] == -2.0)
    assert np.all(np.isfinite(G1))
    scale = np.abs(G1).max(axis=(1, 2, 3), keepdims=True)
    assert np.abs(G1 - G2).max() <= 1e-12 * scale.max()
    assert nbytes > 0


def test_adjoint_forward_matches_stage_forward_steps():
    """The adjoint's forward is the stage: one step of it equals madv_stage_forward's snew
    (density, enthalpy, species) bit for bit."""
    from maestroex_gb300.stage import run_stage_gpu
    case = Case(nsteps=1, ckpt=1)
    sf = case.final(case.sold).to_domain(case.n).cpu().numpy()
    cfg = dict(case.cfg)
    cfg["gpi"] = np.zeros_like(cfg["gpi"])
    ref = run_stage_gpu(cfg)["snew"]
    for comp in [RHO, RHOH] + list(range(FIRSTSPEC, case.nscal)):
        assert np.array_equal(sf[comp], ref[comp]), comp


def test_adjoint_rejects_unsupported_configurations():
    cfg = configs.planar_config(n=(16, 16, 16), max_grid=16, w0_amp=0.0)
    st = make_stage(cfg)
    boxes, nscal = cfg["boxes"], 4 + cfg["nspec"]
    u = MultiFab(boxes, 3, 0)
    s = MultiFab(boxes, nscal, 0).from_domain(cfg["sold"])
    g = MultiFab(boxes, nscal, 0)
    with pytest.raises(MadvError) as e:
        st.stage_adjoint(u, s, s, 2, 1, grad_s=g)
    assert e.value.code == -3
    # the velocity gradient off a periodic domain (inflow is rejected when the context is made)
    for bc, want_u in ((((OUTFLOW, INTERIOR, INTERIOR), (OUTFLOW, INTERIOR, INTERIOR)), True),):
        case = Case(n=(16, 16, 16), bc=bc, nsteps=2, ckpt=1)
        with pytest.raises(MadvError) as e:
            case.adjoint(want_u=want_u)
        assert e.value.code == -3


@pytest.mark.parametrize("part", ["state", "velocity"])
def test_adjoint_matches_cpu_tangent_linear_model(part):
    """Dot-product check of every gradient entry at once: <grad, v> from the GPU adjoint
    against <w, dS_final> from the oracle's tangent-linear build (pyoracle.steps_tl, the same
    4 steps on the CPU, branches decided by the forward values) along a seeded random
    direction v over every cell of the state (density, enthalpy, species, temperature, pi)
    or of the velocity.  Agreement to 1e-10 of the sum of |terms|."""
    import pyoracle
    case = Case()
    J, grad, _, _, gu = case.adjoint(want_u=True)
    G = grad.to_domain(case.n).cpu().numpy()
    GU = gu.to_domain(case.n).cpu().numpy()
    S, U = case.cfg["sold"], case.cfg["uold"]
    rng = np.random.default_rng(2026)
    rms_s = np.sqrt((S ** 2).mean(axis=(1, 2, 3), keepdims=True))
    rms_u = np.sqrt((U ** 2).mean(axis=(1, 2, 3), keepdims=True))
    vs = rng.standard_normal(S.shape) * rms_s if part == "state" else np.zeros_like(S)
    vu = rng.standard_normal(U.shape) * rms_u if part == "velocity" else np.zeros_like(U)
    _, ds = pyoracle.steps_tl(case.cfg, S, vs, U, vu, case.nsteps)
    tl = float((case.w * ds).sum())
    adj = float((G * vs).sum() + (GU * vu).sum())
    scale = float(np.abs(G * vs).sum() + np.abs(GU * vu).sum())
    print(f"{part}: tangent-linear {tl:.15e}, adjoint {adj:.15e}, diff / sum|terms| {abs(tl - adj) / scale:.2e}")
    assert abs(tl - adj) <= 1e-10 * scale


NON_PERIODIC = {
    "outflow": ((OUTFLOW,) * 3, (OUTFLOW,) * 3),
    "mixed": ((SYMMETRY, INTERIOR, OUTFLOW), (OUTFLOW, INTERIOR, SYMMETRY)),
    "walls": ((SLIPWALL, INTERIOR, NOSLIPWALL), (NOSLIPWALL, INTERIOR, SLIPWALL)),
}


def spherical_adjoint_config(n=32, nspec=3, max_grid=16, w0_amp=0.0, ppm_type=1):
    """Full-star spherical configuration (exact base state, outflow on every face) with a
    state-independent MAC velocity: no gravity, w0 of amplitude w0_amp."""
    cfg = configs.spherical_config(n=n, nspec=nspec, ppm_type=ppm_type, max_grid=max_grid, w0_amp=w0_amp)
    cfg["grav_cell"] = np.zeros_like(cfg["grav_cell"])
    return cfg


def tl_dot(case, G, vs):
    import pyoracle
    S, U = case.cfg["sold"], case.cfg["uold"]
    _, ds = pyoracle.steps_tl(case.cfg, S, vs, U, np.zeros_like(U), case.nsteps)
    return float((case.w * ds).sum()), float((G * vs).sum()), float(np.abs(G * vs).sum())


@pytest.mark.parametrize("w0_amp", [0.0, 1.0e5])
def test_spherical_adjoint_matches_cpu_tangent_linear_model(w0_amp):
    """Spherical geometry (32^3 full star in 8 boxes, outflow faces): the density fluxes'
    face base state of MakeS0mac in the flux transpose; the rest of the transposes are the
    plane-parallel ones; with w0 != 0 the force transpose takes the MAC velocity without
    w0mac, as ModifyScalForce does.  Dot-product check against the oracle's tangent-linear
    build over every cell, and over the cells of the star's ambient/surface shell alone."""
    case = Case(cfg=spherical_adjoint_config(w0_amp=w0_amp))
    J, grad, _, _ = case.adjoint()
    G = grad.to_domain(case.n).cpu().numpy()
    S = case.cfg["sold"]
    rng = np.random.default_rng(2028)
    vs = rng.standard_normal(S.shape) * np.sqrt((S ** 2).mean(axis=(1, 2, 3), keepdims=True))
    tl, adj, scale = tl_dot(case, G, vs)
    print(f"spherical: tangent-linear {tl:.15e}, adjoint {adj:.15e}, diff / sum|terms| {abs(tl - adj) / scale:.2e}")
    assert abs(tl - adj) <= 1e-10 * scale
    shell = (S[RHO] < 1e-3 * S[RHO].max())[None]
    tl, adj, scale = tl_dot(case, G, vs * shell)
    assert abs(tl - adj) <= 1e-10 * scale


@pytest.mark.parametrize("bc", sorted(NON_PERIODIC))
def test_non_periodic_adjoint_matches_cpu_tangent_linear_model(bc):
    """Outflow, symmetry and wall boundaries: FillPatch's physical-boundary fill, the edge
    states' boundary overrides and (walls: hoextrap scalar BCs) PPM's boundary stencils
    transposed.  The dot-product check of the state gradient
    against the oracle's tangent-linear build, as on the periodic domain, over every cell,
    boundary cells included (boxes of 16^3 and 8^3 edges touch every face)."""
    import pyoracle
    case = Case(n=(32, 24, 40), max_grid=16, bc=NON_PERIODIC[bc], seed=20261203 + 14)
    J, grad, _, _ = case.adjoint()
    G = grad.to_domain(case.n).cpu().numpy()
    S, U = case.cfg["sold"], case.cfg["uold"]
    rng = np.random.default_rng(2027)
    vs = rng.standard_normal(S.shape) * np.sqrt((S ** 2).mean(axis=(1, 2, 3), keepdims=True))
    _, ds = pyoracle.steps_tl(case.cfg, S, vs, U, np.zeros_like(U), case.nsteps)
    tl = float((case.w * ds).sum())
    adj = float((G * vs).sum())
    scale = float(np.abs(G * vs).sum())
    print(f"{bc}: tangent-linear {tl:.15e}, adjoint {adj:.15e}, diff / sum|terms| {abs(tl - adj) / scale:.2e}")
    assert abs(tl - adj) <= 1e-10 * scale
    # the boundary layers on their own (a wrong boundary transpose would show here even if
    # the interior dominated the sum above)
    edge = np.zeros(S.shape[1:], dtype=bool)
    edge[:2], edge[-2:], edge[:, :2], edge[:, -2:], edge[:, :, :2], edge[:, :, -2:] = (True,) * 6
    vb = vs * edge
    _, dsb = pyoracle.steps_tl(case.cfg, S, vb, U, np.zeros_like(U), case.nsteps)
    tlb, adjb = float((case.w * dsb).sum()), float((G * vb).sum())
    assert abs(tlb - adjb) <= 1e-10 * float(np.abs(G * vb).sum())


def test_planar_adjoint_with_w0_matches_cpu_tangent_linear_model():
    """Plane-parallel, w0 != 0 (amplitude 1e4 cm/s): the MAC velocity carries w0 on the z
    faces in the edge states and fluxes and not in ModifyScalForce.  Dot-product check of the
    state gradient against the oracle's tangent-linear build; the velocity gradient is
    rejected with w0 != 0."""
    cfg = configs.adjoint_config(n=(32, 32, 32), max_grid=16, nspec=3, w0_amp=1.0e4,
                                 bc_lo=(INTERIOR, INTERIOR, OUTFLOW), bc_hi=(INTERIOR, INTERIOR, OUTFLOW))
    assert np.abs(cfg["w0"]).max() > 0.0
    case = Case(cfg=cfg)
    J, grad, _, _ = case.adjoint()
    G = grad.to_domain(case.n).cpu().numpy()
    S = case.cfg["sold"]
    rng = np.random.default_rng(2029)
    vs = rng.standard_normal(S.shape) * np.sqrt((S ** 2).mean(axis=(1, 2, 3), keepdims=True))
    tl, adj, scale = tl_dot(case, G, vs)
    print(f"planar w0: tangent-linear {tl:.15e}, adjoint {adj:.15e}, diff / sum|terms| {abs(tl - adj) / scale:.2e}")
    assert abs(tl - adj) <= 1e-10 * scale
    with pytest.raises(MadvError) as e:
        case.adjoint(want_u=True)
    assert e.value.code == -3


@pytest.mark.parametrize("case", ["periodic", "outflow_symmetry", "spherical"])
def test_ppm2_adjoint_matches_cpu_tangent_linear_model(case):
    """ppm_type 2 (fourth-order interfaces, Colella-Sekora limiter): the limiter and the
    limited interfaces differentiated on the forward's branch.  Dot-product check of the
    state gradient against the oracle's tangent-linear build: plane-parallel periodic,
    plane-parallel with outflow and symmetry faces and w0 != 0, and the spherical full star
    with w0 of amplitude 1e5 (the spherical workload's settings)."""
    if case == "spherical":
        cfg = spherical_adjoint_config(w0_amp=1.0e5, ppm_type=2)
    else:
        kw = {} if case == "periodic" else dict(bc_lo=(SYMMETRY, INTERIOR, OUTFLOW),
                                                bc_hi=(OUTFLOW, INTERIOR, SYMMETRY), w0_amp=1.0e4)
        cfg = configs.adjoint_config(n=(32, 24, 40), max_grid=16, nspec=3, ppm_type=2, seed=20261203 + 15, **kw)
    case_ = Case(cfg=cfg)
    J, grad, _, _ = case_.adjoint()
    G = grad.to_domain(case_.n).cpu().numpy()
    S = case_.cfg["sold"]
    rng = np.random.default_rng(2030)
    vs = rng.standard_normal(S.shape) * np.sqrt((S ** 2).mean(axis=(1, 2, 3), keepdims=True))
    tl, adj, scale = tl_dot(case_, G, vs)
    print(f"ppm2 {case}: tangent-linear {tl:.15e}, adjoint {adj:.15e}, diff / sum|terms| {abs(tl - adj) / scale:.2e}")
    assert abs(tl - adj) <= 1e-10 * scale


def test_ppm2_adjoint_rejects_walls_and_velocity_gradient():
    for bc, want_u in ((((SLIPWALL, INTERIOR, INTERIOR), (SLIPWALL, INTERIOR, INTERIOR)), False),
                       (((INTERIOR,) * 3, (INTERIOR,) * 3), True)):
        cfg = configs.adjoint_config(n=(16, 16, 16), max_grid=16, nspec=3, ppm_type=2, bc_lo=bc[0], bc_hi=bc[1])
        case = Case(cfg=cfg, nsteps=2, ckpt=1)
        with pytest.raises(MadvError) as e:
            case.adjoint(want_u=want_u)
        assert e.value.code == -3


@pytest.mark.parametrize("kw", [{}, {"w0mac_interp_type": 4, "s0_interp_type": 2}])
def test_spherical_uniform_bins_adjoint_matches_cpu_tangent_linear_model(kw):
    """Spherical geometry on uniform radial bins (the reference's default): ModifyScalForce's
    div w0 of the shells enters the force transpose; the interpolated base state is a
    constant of the derivative.  Dot-product check against the oracle's tangent-linear build."""
    cfg = configs.spherical_config(n=32, nspec=3, ppm_type=1, max_grid=16, w0_amp=1.0e5, exact=False, **kw)
    cfg["grav_cell"] = np.zeros_like(cfg["grav_cell"])
    case = Case(cfg=cfg)
    J, grad, _, _ = case.adjoint()
    G = grad.to_domain(case.n).cpu().numpy()
    S = case.cfg["sold"]
    rng = np.random.default_rng(2029)
    vs = rng.standard_normal(S.shape) * np.sqrt((S ** 2).mean(axis=(1, 2, 3), keepdims=True))
    tl, adj, scale = tl_dot(case, G, vs)
    print(f"spherical uniform bins: tangent-linear {tl:.15e}, adjoint {adj:.15e}, "
          f"diff / sum|terms| {abs(tl - adj) / scale:.2e}")
    assert abs(tl - adj) <= 1e-10 * scale


# buoyancy: with gravity the MAC velocity depends on the density through MakeVelForce and
# VelPred's final states, so each reverse step carries its MAC-velocity adjoint (the flux,
# tracing, transverse and force transposes, the transverse coefficients, the ghost faces)
# back to the density through the force.  The stage has no MAC projection and these steps
# no force-limited dt, so at full strength the buoyant kicks drain cells within the four
# steps: the gravity is scaled down (1e-3 plane-parallel, 1e-5 for the star).  The path
# still dominates the density's sensitivity (by ~1e17 over the same configuration without
# gravity), so the density-only dot product checks it.
BUOYANCY = {
    "periodic": dict(n=(32, 32, 32)),
    "outflow": dict(n=(32, 24, 32), seed=20261203 + 40, bc_lo=NON_PERIODIC["outflow"][0],
                    bc_hi=NON_PERIODIC["outflow"][1]),
    "mixed": dict(n=(32, 24, 32), seed=20261203 + 40, bc_lo=NON_PERIODIC["mixed"][0], bc_hi=NON_PERIODIC["mixed"][1]),
}


def density_and_state_dots(case, label):
    J, grad, _, _ = case.adjoint()
    G = grad.to_domain(case.n).cpu().numpy()
    S = case.cfg["sold"]
    rng = np.random.default_rng(2030)
    vs = rng.standard_normal(S.shape) * np.sqrt((S ** 2).mean(axis=(1, 2, 3), keepdims=True))
    for part, v in (("state", vs), ("density", vs * (np.arange(S.shape[0]) == RHO)[:, None, None, None])):
        tl, adj, scale = tl_dot(case, G, v)
        print(f"{label} {part}: tangent-linear {tl:.15e}, adjoint {adj:.15e}, "
              f"diff / sum|terms| {abs(tl - adj) / scale:.2e}")
        assert abs(tl - adj) <= 1e-10 * scale, part


@pytest.mark.parametrize("ppm_type,bc", [(1, "periodic"), (1, "outflow"), (1, "mixed"), (2, "periodic"),
                                         (2, "outflow")])
def test_buoyancy_adjoint_matches_cpu_tangent_linear_model(ppm_type, bc):
    """Plane-parallel with gravity: dot-product check of the state gradient against the
    oracle's tangent-linear build (whose forward recomputes the MAC velocity from the state in
    every step), over every cell and over the density alone."""
    cfg = configs.adjoint_config(max_grid=16, nspec=3, ppm_type=ppm_type, gravity=True, **BUOYANCY[bc])
    cfg["grav_cell"] = cfg["grav_cell"] * 1.0e-3
    density_and_state_dots(Case(cfg=cfg), f"buoyancy ppm{ppm_type} {bc}")


@pytest.mark.parametrize("ppm_type,w0_amp,exact", [(1, 0.0, True), (2, 1.0e5, True), (1, 1.0e5, False)])
def test_spherical_buoyancy_adjoint_matches_cpu_tangent_linear_model(ppm_type, w0_amp, exact):
    """The full star with gravity (outflow faces, the force along the radius, w0mac in
    VelPred's decisions): dot-product check against the oracle's tangent-linear build over
    every cell and over the density alone."""
    cfg = configs.spherical_config(n=32, nspec=3, ppm_type=ppm_type, max_grid=16, w0_amp=w0_amp, exact=exact)
    cfg["grav_cell"] = cfg["grav_cell"] * 1.0e-5
    density_and_state_dots(Case(cfg=cfg), f"spherical buoyancy ppm{ppm_type} w0 {w0_amp} exact {exact}")


def test_buoyancy_adjoint_rejects_walls_and_velocity_gradient():
    cfg = configs.adjoint_config(n=(16, 16, 16), max_grid=16, gravity=True)
    case = Case(cfg=cfg, nsteps=2, ckpt=1)
    with pytest.raises(MadvError) as e:
        case.adjoint(want_u=True)
    assert e.value.code == -3
    walls = NON_PERIODIC["walls"]
    cfg = configs.adjoint_config(n=(16, 16, 16), max_grid=16, gravity=True, bc_lo=walls[0], bc_hi=walls[1])
    case = Case(cfg=cfg, nsteps=2, ckpt=1)
    with pytest.raises(MadvError) as e:
        case.adjoint()
    assert e.value.code == -3
