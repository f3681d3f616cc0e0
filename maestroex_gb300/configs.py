"""Seeded synthetic inputs for the scalar-advection stage.

The reference publishes no dataset for this path; these generators build the plane-parallel
atmospheres the benchmark configurations describe: an isothermal base state
rho0(z) = 1e7 exp(-z/H) with H = L/4 in hydrostatic equilibrium under constant gravity,
seeded smooth mass fractions (sums of Gaussian bumps, clipped and renormalised), a smooth
enthalpy field rho*(1e17 + 1e16 G), a divergence-free velocity from a seeded vector
potential scaled to Mach 0.01, and a seeded base-state velocity w0(z).

Arrays are numpy float64, shaped [ncomp, nz, ny, nx] (x fastest), i.e. the Fortran-order
component blocks the C ABI and the oracle use.
"""
import math

import numpy as np

from .params import INTERIOR, OUTFLOW, SLIPWALL, RHO, RHOH, TEMP, PI, FIRSTSPEC

L_DOMAIN = 1.0e8
GRAV = -1.0e8


def tile_boxes(n, max_grid):
    """Chop the domain [0, n) into boxes of edge max_grid (AMReX max_grid_size tiling)."""
    mg = max_grid if isinstance(max_grid, (tuple, list)) else (max_grid,) * 3
    boxes = []
    for k0 in range(0, n[2], mg[2]):
        for j0 in range(0, n[1], mg[1]):
            for i0 in range(0, n[0], mg[0]):
                boxes.append((i0, j0, k0, min(i0 + mg[0], n[0]) - 1, min(j0 + mg[1], n[1]) - 1,
                              min(k0 + mg[2], n[2]) - 1))
    return boxes


def uneven_boxes(n, edges, rng, p_stop=0.35):
    """Seeded guillotine split of the domain into boxes whose edges come from `edges`;
    a piece whose extents are all in `edges` stops splitting with probability p_stop."""
    out = []

    def split(lo, hi):
        ext = [hi[d] - lo[d] for d in range(3)]
        if all(e in edges for e in ext) and rng.random() < p_stop:
            out.append((lo[0], lo[1], lo[2], hi[0] - 1, hi[1] - 1, hi[2] - 1))
            return
        cands = []
        for d in range(3):
            for e in edges:
                if e < ext[d] and (ext[d] - e) in edges or (e < ext[d] and ext[d] - e >= min(edges)):
                    cands.append((d, e))
        cands = [(d, e) for d, e in cands if (ext[d] - e) >= min(edges)]
        if not cands:
            out.append((lo[0], lo[1], lo[2], hi[0] - 1, hi[1] - 1, hi[2] - 1))
            return
        d, e = cands[rng.integers(len(cands))]
        mid = list(hi)
        mid[d] = lo[d] + e
        split(lo, tuple(mid))
        lo2 = list(lo)
        lo2[d] = lo[d] + e
        split(tuple(lo2), hi)

    split((0, 0, 0), tuple(n))
    return out


def _coords(n, dx):
    return [(np.arange(n[d]) + 0.5) * dx[d] for d in range(3)]


def _smooth_field(rng, n, dx, periodic, nmodes=8):
    """Unit-RMS sum of seeded separable Fourier modes."""
    x, y, z = _coords(n, dx)
    f = np.zeros((n[2], n[1], n[0]))
    for _ in range(nmodes):
        kx, ky, kz = rng.integers(1, 5, size=3)
        px, py, pz = rng.uniform(0, 2 * math.pi, size=3)
        a = rng.normal()
        fx = np.cos(2 * math.pi * kx * x / L_DOMAIN + px)
        fy = np.cos(2 * math.pi * ky * y / L_DOMAIN + py)
        fz = np.cos(2 * math.pi * kz * z / L_DOMAIN + pz)
        f += a * fz[:, None, None] * fy[None, :, None] * fx[None, None, :]
    rms = math.sqrt(float(np.mean(f * f)))
    return f / rms


def _gauss1d(c, w, L, periodic, dx, n):
    x = (np.arange(n) + 0.5) * dx
    dd = x - c
    if periodic:
        dd = dd - L * np.round(dd / L)
    return np.exp(-(dd * dd) / (w * w))


def planar_config(n=(32, 32, 32), nspec=3, ppm_type=1, bc_lo=(INTERIOR, INTERIOR, SLIPWALL),
                  bc_hi=(INTERIOR, INTERIOR, OUTFLOW), max_grid=16, boxes=None, seed=20261203,
                  w0_amp=1.0e4, cfl=0.7, rho_pert=1.0e-5, gpi_amp=1.0e-5, species_pred_type=1,
                  enthalpy_pred_type=1, slope_order=4, evolve_base_state=1):
    """Build one plane-parallel 3-D stage configuration (parameters + input arrays)."""
    rng = np.random.default_rng(seed)
    n = tuple(int(v) for v in n)
    dx = tuple(L_DOMAIN / n[d] for d in range(3))
    periodic = [bc_lo[d] == INTERIOR for d in range(3)]
    x, y, z = _coords(n, dx)
    H = 0.25 * L_DOMAIN
    nr = n[2]
    r_cc = (np.arange(nr) + 0.5) * dx[2]
    rho0 = 1.0e7 * np.exp(-r_cc / H)
    p0 = rho0 * abs(GRAV) * H

    shape = (n[2], n[1], n[0])
    # species: sums of 6 Gaussian bumps, clipped and renormalised
    X = np.zeros((nspec,) + shape)
    for s in range(nspec):
        for _ in range(6):
            w = rng.uniform(0.05, 0.2) * L_DOMAIN
            c = rng.uniform(0, L_DOMAIN, size=3)
            A = rng.uniform(0.2, 1.0)
            gx = _gauss1d(c[0], w, L_DOMAIN, periodic[0], dx[0], n[0])
            gy = _gauss1d(c[1], w, L_DOMAIN, periodic[1], dx[1], n[1])
            gz = _gauss1d(c[2], w, L_DOMAIN, periodic[2], dx[2], n[2])
            X[s] += A * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
    X = np.maximum(X, 1.0e-10)
    X /= X.sum(axis=0, keepdims=True)

    rho = rho0[:, None, None] * (1.0 + rho_pert * _smooth_field(rng, n, dx, periodic))
    h = 1.0e17 + 1.0e16 * _smooth_field(rng, n, dx, periodic)
    rhoh = rho * h
    rhoh0 = rhoh.mean(axis=(1, 2))

    nscal = 4 + nspec
    sold = np.zeros((nscal,) + shape)
    sold[RHO] = rho
    sold[RHOH] = rhoh
    sold[TEMP] = 1.0e8
    sold[PI] = 0.0
    sold[FIRSTSPEC:] = rho[None] * X

    # divergence-free velocity u = curl A, A_x, A_y ~ sin(pi kz z / L) so w = 0 at z walls
    u = np.zeros((3,) + shape)
    for _ in range(8):
        kx, ky, kz = rng.integers(1, 5, size=3)
        px, py, pz = rng.uniform(0, 2 * math.pi, size=3)
        ax, ay, az = rng.normal(size=3)
        cx = 2 * math.pi * kx / L_DOMAIN
        cy = 2 * math.pi * ky / L_DOMAIN
        cz = math.pi * kz / L_DOMAIN
        Cx, Sx = np.cos(cx * x + px), np.sin(cx * x + px)
        Cy, Sy = np.cos(cy * y + py), np.sin(cy * y + py)
        Sz, Cz = np.sin(cz * z), np.cos(cz * z)
        Czp, Szp = np.cos(cz * z + pz), np.sin(cz * z + pz)

        def o(fz, fy, fx):
            return fz[:, None, None] * fy[None, :, None] * fx[None, None, :]

        # A_x = ax Sz Cx Cy ; A_y = ay Sz Cx Cy ; A_z = az Czp Cx Cy
        # u = dAz/dy - dAy/dz ; v = dAx/dz - dAz/dx ; w = dAy/dx - dAx/dy
        u[0] += az * o(Czp, -cy * Sy, Cx) - ay * o(cz * Cz, Cy, Cx)
        u[1] += ax * o(cz * Cz, Cy, Cx) - az * o(Czp, Cy, -cx * Sx)
        u[2] += ay * o(Sz, Cy, -cx * Sx) - ax * o(Sz, -cy * Sy, Cx)
    cs = math.sqrt(5.0 / 3.0 * abs(GRAV) * H)
    u *= 0.01 * cs / np.abs(u).max()

    # base-state velocity at radial edges, w0(0) = 0
    r_edge = np.arange(nr + 1) * dx[2]
    w0 = np.zeros(nr + 1)
    if w0_amp != 0.0:
        for m in range(1, 5):
            w0 += rng.normal() * np.sin(m * math.pi * r_edge / L_DOMAIN)
        w0 *= w0_amp / np.abs(w0).max()
        w0[0] = 0.0

    gpi = np.zeros((3,) + shape)
    for d in range(3):
        gpi[d] = gpi_amp * abs(GRAV) * rho0[:, None, None] * _smooth_field(rng, n, dx, periodic)

    umax_d = [float(np.abs(u[d]).max()) for d in range(3)]
    umax_d[2] = max(umax_d[2], float(np.abs(u[2]).max() + np.abs(w0).max()))
    umax = max(umax_d)
    dt = cfl * min(dx[d] / umax_d[d] for d in range(3))

    if boxes is None:
        boxes = tile_boxes(n, max_grid)

    # 1-D arrays
    from .basestate import cell_to_edge
    cfg = dict(
        n=n, dx=dx, nspec=nspec, ppm_type=ppm_type, slope_order=slope_order, bc_lo=tuple(bc_lo),
        bc_hi=tuple(bc_hi), species_pred_type=species_pred_type,
        enthalpy_pred_type=enthalpy_pred_type, evolve_base_state=evolve_base_state,
        dt=dt, rel_eps=1.0e-8 * umax, base_cutoff_density=1.0e3, buoyancy_cutoff_factor=5.0,
        boxes=boxes, seed=seed,
        uold=np.ascontiguousarray(u), sold=np.ascontiguousarray(sold), gpi=gpi,
        thermal=np.zeros((1,) + shape),
        rho0_old=rho0.copy(), rho0_new=rho0.copy(), rhoh0_old=rhoh0.copy(), rhoh0_new=rhoh0.copy(),
        p0_old=p0.copy(), p0_new=p0.copy(), psi=np.zeros(nr), grav_cell=np.full(nr, GRAV),
        w0_force=np.zeros(nr), w0=w0, rho0_predicted_edge=cell_to_edge(rho0),
    )
    return cfg


def workload_planar(n=256, box=64, nspec=13, seed=20261203 + 1):
    """3-D single level, 256^3 in 64 boxes of 64^3, NumSpec 13, ppm_type 1, w0 != 0 (the bench workload)."""
    return planar_config(n=(n, n, n), nspec=nspec, ppm_type=1, max_grid=box, seed=seed,
                         w0_amp=1.0e4, cfl=0.7)


def adjoint_config(n=(128, 128, 128), max_grid=64, nspec=3, seed=20261203 + 4, cfl=0.5, bc_lo=(INTERIOR,) * 3,
                   bc_hi=(INTERIOR,) * 3, w0_amp=0.0, ppm_type=1, gravity=False):
    """3-D single-level configuration of the multi-step adjoint (periodic unless bc_lo /
    bc_hi say otherwise): the cell velocity is held fixed (gpi = 0; w0 of amplitude w0_amp,
    default 0), ppm_type 1 (or 2), species_pred_type 1, enthalpy_pred_type 1; dt from CFL
    0.5.  gravity=False: grav_cell = 0, so the MAC velocity does not depend on the state;
    True: the constant gravity of planar_config, the MAC velocity taking the buoyancy of the
    density through MakeVelForce.  The density perturbation rho - rho0 is 1% of rho0, so
    that a perturbation of 1e-6 rho is small against it."""
    cfg = planar_config(n=n, nspec=nspec, ppm_type=ppm_type, bc_lo=bc_lo, bc_hi=bc_hi,
                        max_grid=max_grid, seed=seed, w0_amp=w0_amp, cfl=cfl, gpi_amp=0.0, evolve_base_state=0,
                        rho_pert=1.0e-2)
    if not gravity:
        cfg["grav_cell"] = np.zeros_like(cfg["grav_cell"])
    return cfg


def lane_emden(n_poly=1.5, h=1.0e-4):
    """theta(xi) of the Lane-Emden equation theta'' + 2 theta'/xi + theta^n = 0 (RK4 from the
    series start), integrated to the first zero xi_1; returns (xi, theta) arrays."""
    xi = [h]
    th = [1.0 - h * h / 6.0]
    dth = -h / 3.0

    def f(x, t, dt):
        return dt, -2.0 * dt / x - max(t, 0.0) ** n_poly

    x, t = h, th[0]
    while t > 0.0:
        k1 = f(x, t, dth)
        k2 = f(x + h / 2, t + h / 2 * k1[0], dth + h / 2 * k1[1])
        k3 = f(x + h / 2, t + h / 2 * k2[0], dth + h / 2 * k2[1])
        k4 = f(x + h, t + h * k3[0], dth + h * k3[1])
        t += h / 6 * (k1[0] + 2 * k2[0] + 2 * k3[0] + k4[0])
        dth += h / 6 * (k1[1] + 2 * k2[1] + 2 * k3[1] + k4[1])
        x += h
        xi.append(x)
        th.append(t)
    return np.array(xi), np.maximum(np.array(th), 0.0)


def _sph_bins_to_cells(s0, radius, drf, t):
    """Cell values of a bin-centred radial array on uniform bins of drf, as the reference's
    Put1dArrayOnCart forms them (s0_interp_type t: 1 constant, 2 linear, 3 quadratic clipped
    to its three points' range); used to lay the initial state on the base state."""
    nr = len(s0)
    rcc = (np.arange(nr) + 0.5) * drf
    index = (radius / drf).astype(np.int64)
    if t == 1:
        return s0[np.minimum(index, nr - 1)]
    if t == 2:
        return np.interp(radius, rcc, s0)
    i = np.clip(index, 1, nr - 2)
    x0, x1, x2 = rcc[i - 1], rcc[i], rcc[i + 1]
    y0, y1, y2 = s0[i - 1], s0[i], s0[i + 1]
    y = (y0 + (y1 - y0) / (x1 - x0) * (radius - x0) +
         ((y2 - y1) / (x2 - x1) - (y1 - y0) / (x1 - x0)) / (x2 - x0) * (radius - x0) * (radius - x1))
    return np.clip(y, np.minimum(y0, np.minimum(y1, y2)), np.maximum(y0, np.maximum(y1, y2)))


def spherical_config(n=64, nspec=3, ppm_type=1, max_grid=32, boxes=None, seed=20261203 + 5, cfl=0.5,
                     rho_c=2.0e9, w0_amp=1.0e5, u_amp=1.0e6, L=5.0e8, pert=1.0e-9, n_base=None, exact=True,
                     drdxfac=1, **interp):
    """Full-star spherical configuration with the exact base state: an n^3 Cartesian domain
    [0, L]^3 with the star at its centre, outflow on every face; an n = 1.5 polytrope of
    central density rho_c and radius 0.9 L/2 (Lane-Emden, integrated here) on the irregular
    radial grid r_cc(i) = sqrt(0.75 + 2i) dx, with a constant ambient density 1e-5 rho_c
    outside; w0 on the radial edges a seeded smooth profile of amplitude w0_amp, zero at
    the centre and beyond 0.8 of the radius; a seeded smooth velocity of amplitude u_amp tapered to
    zero at 0.8 of the radius; density and enthalpy perturbed by `pert` (relative);
    base_cutoff_density half the ambient density, so the buoyancy cutoff (5x) covers the
    ambient.  n_base: extent of the finest level of a hierarchy, whose cell size sets the
    radial grid (default n).  exact=False: the uniform radial bins of the reference's default
    (use_exact_base_state = 0), dr = dx_fine / drdxfac, nr = int(max_dist / dr) + 1 with
    max_dist the centre-to-corner distance; interp: w0_interp_type, w0mac_interp_type,
    s0_interp_type, s0mac_interp_type (the reference's defaults when absent)."""
    rng = np.random.default_rng(seed)
    n3 = (n, n, n)
    dx = L / n
    nb = n if n_base is None else n_base
    dxb = L / nb
    if exact:
        nr_irreg = int((3.0 * (nb / 2 - 0.5) * (nb / 2 - 0.5) - 0.75) / 2.0)
        nr = nr_irreg + 1
        r_cc = np.sqrt(0.75 + 2.0 * np.arange(nr)) * dxb
        r_edge = np.concatenate([[0.0], np.sqrt(0.75 + 2.0 * (np.arange(nr) + 0.5)) * dxb])
    else:
        drf = dxb / drdxfac
        half = 0.5 * L
        nr = int(math.sqrt(3.0 * half * half) / drf) + 1
        r_cc = (np.arange(nr) + 0.5) * drf
        r_edge = np.arange(nr + 1) * drf
    npoly, gamma = 1.5, 5.0 / 3.0
    xi, theta = lane_emden(npoly)
    R = 0.9 * 0.5 * L
    a = R / xi[-1]
    G = 6.674e-8
    K = 4.0 * math.pi * G * a * a * rho_c ** (1.0 - 1.0 / npoly) / (npoly + 1.0)
    th_r = np.interp(r_cc / a, xi, theta, right=0.0)
    rho_floor = 1.0e-5 * rho_c
    rho0 = np.maximum(rho_c * th_r ** npoly, rho_floor)
    p0 = K * rho0 ** (1.0 + 1.0 / npoly)
    rhoh0 = gamma / (gamma - 1.0) * p0
    # gravity from the enclosed mass of the shells between the radial edges
    shell = 4.0 / 3.0 * math.pi * (r_edge[1:] ** 3 - r_edge[:-1] ** 3)
    menc = np.cumsum(rho0 * shell) - 0.5 * rho0 * shell
    grav = -G * menc / r_cc ** 2
    w0 = np.zeros(nr + 1)
    inside = r_edge < 0.8 * R
    for m in range(1, 4):
        w0[inside] += rng.normal() * np.sin(m * math.pi * r_edge[inside] / (0.8 * R))
    w0 *= w0_amp / max(np.abs(w0).max(), 1e-300)
    w0[0] = 0.0

    # cell -> radial index, as Maestro::InitBaseStateMapSphr (round half away from zero), or
    # the uniform bin of the cell centre
    c = (np.arange(n) + 0.5) * dx - 0.5 * L
    X3, Y3, Z3 = c[None, None, :], c[None, :, None], c[:, None, None]
    r2 = X3 * X3 + Y3 * Y3 + Z3 * Z3
    if exact:
        idx = np.floor(r2 / (2.0 * dxb * dxb) - 0.375 + 0.5).astype(np.int64)

        def on_cells(a):
            return a[idx]
    else:
        # the cells hold the base state as Put1dArrayOnCart interpolates it there, so that
        # the buoyancy starts at the seeded perturbation
        t = interp.get("s0_interp_type", 3)

        def on_cells(a):
            return _sph_bins_to_cells(a, np.sqrt(r2), dxb / drdxfac, t)
    shape = (n, n, n)
    periodic = [False, False, False]
    rho = on_cells(rho0) * (1.0 + pert * _smooth_field(rng, n3, (L / n,) * 3, periodic))
    X = np.zeros((nspec,) + shape)
    for sp in range(nspec):
        X[sp] = 1.0 + 0.5 * _smooth_field(rng, n3, (L / n,) * 3, periodic)
    X = np.maximum(X, 0.05)
    X /= X.sum(axis=0, keepdims=True)
    h = on_cells(rhoh0) / on_cells(rho0) * (1.0 + pert * _smooth_field(rng, n3, (L / n,) * 3, periodic))
    nscal = 4 + nspec
    sold = np.zeros((nscal,) + shape)
    sold[RHO] = rho
    sold[RHOH] = rho * h
    sold[TEMP] = 1.0e8
    sold[FIRSTSPEC:] = rho[None] * X
    # the velocity lives inside the star: a smooth seeded field tapered to zero at 0.8 R
    taper = np.maximum(0.0, 1.0 - r2 / (0.8 * R) ** 2) ** 2
    u = np.zeros((3,) + shape)
    for d in range(3):
        u[d] = u_amp * taper * _smooth_field(rng, n3, (L / n,) * 3, periodic)
    umax = max(float(np.abs(u).max()), 1.0) + w0_amp
    # Maestro::EstDt: the advective limit and the force limit sqrt(2 dx / |f|) with the
    # buoyancy (rho - rho0) g / rho of the seeded perturbation (Source/MaestroDt.cpp:150-225)
    fmax = float(np.abs(grav).max()) * float(np.abs(rho / on_cells(rho0) - 1.0).max())
    dt = cfl * min(dx / umax, math.sqrt(2.0 * dx / max(fmax, 1e-300)))
    if boxes is None:
        boxes = tile_boxes(n3, max_grid)
    from .basestate import cell_to_edge
    extra = dict(drdxfac=drdxfac, **interp)
    return dict(
        n=n3, dx=(dx, dx, dx), nspec=nspec, ppm_type=ppm_type, slope_order=4, bc_lo=(OUTFLOW,) * 3,
        bc_hi=(OUTFLOW,) * 3, species_pred_type=1, enthalpy_pred_type=1, evolve_base_state=1,
        use_exact_base_state=1 if exact else 0, spherical=1, prob_lo=(0.0, 0.0, 0.0), prob_hi=(L, L, L), nr=nr,
        **extra,
        dt=dt, rel_eps=1.0e-8 * umax, base_cutoff_density=0.5 * rho_floor, buoyancy_cutoff_factor=5.0,
        boxes=boxes, seed=seed, uold=np.ascontiguousarray(u), sold=np.ascontiguousarray(sold),
        gpi=np.zeros((3,) + shape), thermal=np.zeros((1,) + shape),
        rho0_old=rho0.copy(), rho0_new=rho0.copy(), rhoh0_old=rhoh0.copy(), rhoh0_new=rhoh0.copy(),
        p0_old=p0.copy(), p0_new=p0.copy(), psi=np.zeros(nr), grav_cell=grav, w0_force=np.zeros(nr), w0=w0,
        rho0_predicted_edge=cell_to_edge(rho0),
    )


def spherical_amr_config(n0=32, nspec=3, ppm_type=2, max_grid=16, fine_boxes=None, seed=20261203 + 6,
                         cover=0.12, inject=False, level0_boxes=None, **kw):
    """Two-level spherical configuration (refinement ratio 2) on one radial grid set by the
    fine level.  Level 1: seeded boxes (bubble_boxes) covering about `cover` of the
    domain.  inject=False: both levels are the same star evaluated at their resolution,
    level-0 cells under level 1 holding the average of their children; inject=True:
    level-1 cells take their parent's values (filled on the device by stage.amr_buffers),
    for sizes whose fine level cannot be evaluated on the whole domain.  dt is the
    fine level's."""
    n1 = 2 * n0
    rng = np.random.default_rng(seed + 100)
    if fine_boxes is None:
        fine_boxes = bubble_boxes((n0, n0, n0), nbubbles=3, cover=cover, block_edges=(8, 16, 24, 32), max_edge=32,
                                  rng=rng)
    c0 = spherical_config(n=n0, nspec=nspec, ppm_type=ppm_type, max_grid=max_grid, boxes=level0_boxes, seed=seed,
                          n_base=n1, **kw)
    if inject:
        lev1 = dict(n=(n1,) * 3, dx=tuple(v / 2 for v in c0["dx"]), boxes=list(fine_boxes), inject=True)
        for k in LEVEL_KEYS:
            if k not in lev1 and k not in ("uold", "sold", "gpi", "thermal"):
                lev1[k] = c0[k]
        c0["dt"] *= 0.5
    else:
        c1 = spherical_config(n=n1, nspec=nspec, ppm_type=ppm_type, boxes=list(fine_boxes), seed=seed, **kw)
        for key in ("sold", "uold", "gpi"):
            _average_down(c1[key], c0[key], fine_boxes)
        c0["dt"] = min(c0["dt"], c1["dt"])
        c0["rel_eps"] = max(c0["rel_eps"], c1["rel_eps"])
        lev1 = {k: c1[k] for k in LEVEL_KEYS}
    c0["levels"] = [{k: c0[k] for k in LEVEL_KEYS}, lev1]
    return c0


def bubble_boxes(n0, nbubbles=3, cover=0.12, block_edges=(8, 16, 32), rng=None, max_edge=32):
    """Level-1 boxes (refinement ratio 2, fine index space) around seeded bubble centres.

    The coarse domain is cut along each axis into segments whose lengths come from
    `block_edges` (coarse cells, clipped to max_edge); every block that contains a cell within
    radius R of a bubble centre becomes one fine box.  R is chosen so the tagged volume is
    about `cover` of the domain.  Boxes are coarse-aligned (even lo, odd hi in fine cells).
    """
    rng = np.random.default_rng(20261203 + 3) if rng is None else rng
    n0 = tuple(int(v) for v in n0)
    centres = [rng.uniform(0.2, 0.8, size=3) * np.array(n0) for _ in range(nbubbles)]
    R = (cover * n0[0] * n0[1] * n0[2] / nbubbles * 3.0 / (4.0 * math.pi)) ** (1.0 / 3.0)
    cuts = []
    for d in range(3):
        pts, p = [0], 0
        while p < n0[d]:
            e = int(min(rng.choice(block_edges), max_edge, n0[d] - p))
            p += e
            pts.append(p)
        cuts.append(pts)
    z, y, x = np.meshgrid(*[np.arange(n0[d]) + 0.5 for d in (2, 1, 0)], indexing="ij")
    tag = np.zeros((n0[2], n0[1], n0[0]), bool)
    for c in centres:
        tag |= (x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 <= R * R
    boxes = []
    for k in range(len(cuts[2]) - 1):
        for j in range(len(cuts[1]) - 1):
            for i in range(len(cuts[0]) - 1):
                lo = (cuts[0][i], cuts[1][j], cuts[2][k])
                hi = (cuts[0][i + 1], cuts[1][j + 1], cuts[2][k + 1])
                if tag[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]].any():
                    boxes.append((2 * lo[0], 2 * lo[1], 2 * lo[2], 2 * hi[0] - 1, 2 * hi[1] - 1, 2 * hi[2] - 1))
    return boxes


def _average_down(fine, coarse, fine_boxes):
    """Coarse cells under fine boxes become the mean of their 8 children (in place)."""
    for b in fine_boxes:
        i0, j0, k0, i1, j1, k1 = b
        f = fine[..., k0:k1 + 1, j0:j1 + 1, i0:i1 + 1]
        c = f.reshape(f.shape[:-3] + (f.shape[-3] // 2, 2, f.shape[-2] // 2, 2, f.shape[-1] // 2, 2))
        c = c.sum(axis=(-1, -3, -5)) * 0.125
        coarse[..., k0 // 2:(k1 + 1) // 2, j0 // 2:(j1 + 1) // 2, i0 // 2:(i1 + 1) // 2] = c


LEVEL_KEYS = ("n", "dx", "boxes", "uold", "sold", "gpi", "thermal", "rho0_old", "rho0_new", "rhoh0_old",
              "rhoh0_new", "p0_old", "p0_new", "psi", "grav_cell", "w0_force", "w0", "rho0_predicted_edge")


def planar_amr_config(n0=(32, 32, 32), nspec=3, ppm_type=2, max_grid=16, fine_boxes=None, level0_boxes=None,
                      seed=20261203 + 2, nbubbles=3, cover=0.12, **kw):
    """Two-level plane-parallel configuration (refinement ratio 2).

    Both levels are the same seeded atmosphere evaluated at their own resolution; level-0
    cells under level 1 hold the average of their children (the state a previous step's
    AverageDown leaves); dt is the CFL step of the finer level.  Returns the level-0 dict
    (parameters as for planar_config) with "levels": [level-0 arrays, level-1 arrays].
    """
    n0 = tuple(int(v) for v in n0)
    c0 = planar_config(n=n0, nspec=nspec, ppm_type=ppm_type, max_grid=max_grid, boxes=level0_boxes, seed=seed, **kw)
    n1 = tuple(2 * v for v in n0)
    if fine_boxes is None:
        fine_boxes = bubble_boxes(n0, nbubbles=nbubbles, cover=cover, rng=np.random.default_rng(seed + 100))
    c1 = planar_config(n=n1, nspec=nspec, ppm_type=ppm_type, max_grid=max_grid, boxes=list(fine_boxes),
                       seed=seed, **kw)
    for key in ("sold", "uold", "gpi"):
        _average_down(c1[key], c0[key], fine_boxes)
    c0["dt"] = min(c0["dt"], c1["dt"])
    c0["rel_eps"] = max(c0["rel_eps"], c1["rel_eps"])
    c0["levels"] = [{k: c0[k] for k in LEVEL_KEYS}, {k: c1[k] for k in LEVEL_KEYS}]
    return c0


def workload_amr(n0=256, nspec=13, seed=20261203 + 3, cover=0.06, p_stop=0.8):
    """Two-level AMR, level 0 = n0^3 in uneven boxes (edges from
    {16, 32, 48, 64, 96, 128}), level 1 (ratio 2) = boxes of 16-64 fine cells of random
    aspect around 3 seeded bubbles covering about `cover` of the domain; NumSpec 13,
    ppm_type 2.  Level-1 state is injected from level 0 (each fine cell takes its parent's
    value: "inject" levels are filled on the device by stage.amr_buffers); the level-1
    base state is the same atmosphere on the fine radial grid.  dt is halved for the
    fine level's CFL condition.
    """
    from .basestate import cell_to_edge
    rng = np.random.default_rng(seed)
    n = (n0, n0, n0)
    l0 = uneven_boxes(n, [16, 32, 48, 64, 96, 128], rng, p_stop=p_stop)
    fine = bubble_boxes(n, nbubbles=3, cover=cover, block_edges=(8, 16, 24, 32), max_edge=32,
                        rng=np.random.default_rng(seed + 100))
    cfg = planar_config(n=n, nspec=nspec, ppm_type=2, boxes=l0, seed=seed, w0_amp=1.0e4, cfl=0.7)
    cfg["dt"] *= 0.5
    n1 = tuple(2 * v for v in n)
    dx1 = tuple(L_DOMAIN / v for v in n1)
    nr1 = n1[2]
    H = 0.25 * L_DOMAIN
    r_cc = (np.arange(nr1) + 0.5) * dx1[2]
    rho0 = 1.0e7 * np.exp(-r_cc / H)
    w0c = cfg["w0"]
    w0 = np.zeros(nr1 + 1)
    w0[0::2] = w0c
    w0[1::2] = 0.5 * (w0c[:-1] + w0c[1:])
    lev1 = dict(n=n1, dx=dx1, boxes=fine, inject=True,
                rho0_old=rho0.copy(), rho0_new=rho0.copy(),
                rhoh0_old=np.repeat(cfg["rhoh0_old"], 2), rhoh0_new=np.repeat(cfg["rhoh0_new"], 2),
                p0_old=rho0 * abs(GRAV) * H, p0_new=rho0 * abs(GRAV) * H, psi=np.zeros(nr1),
                grav_cell=np.full(nr1, GRAV), w0_force=np.zeros(nr1), w0=w0,
                rho0_predicted_edge=cell_to_edge(rho0))
    cfg["levels"] = [{k: cfg[k] for k in LEVEL_KEYS}, lev1]
    return cfg


def two_level_sample(nspec=13, n0=64, seed=20261203 + 3, **kw):
    """The two-level AMR workload's shape at a size the oracle checks in seconds: level 0
    n0^3 in uneven boxes (edges 16-64), level 1 (ratio 2) in boxes of 16-32 fine cells around
    3 seeded bubbles (about 14% of the domain at n0 = 64), ppm_type 2, w0 != 0; both levels
    evaluated at their own resolution (no injection)."""
    rng = np.random.default_rng(seed)
    l0 = uneven_boxes((n0,) * 3, [16, 32, 48, 64], rng, p_stop=0.35)
    fine = bubble_boxes((n0,) * 3, nbubbles=3, cover=0.01, block_edges=(8, 16), max_edge=16,
                        rng=np.random.default_rng(seed + 100))
    return planar_amr_config(n0=(n0,) * 3, nspec=nspec, ppm_type=2, fine_boxes=fine, level0_boxes=l0, seed=seed,
                             w0_amp=1.0e4, cfl=0.7, **kw)


def spherical_two_level_sample(nspec=21, n0=48, seed=20261203 + 50):
    """The spherical workload's shape at a size the oracle checks in seconds: the full star
    on level 0 n0^3 in uneven boxes (edges 16-48) and a level 1 of 16-32-cell boxes around 3
    bubbles (about 16% of the domain at n0 = 48), NumSpec 21, ppm_type 2, w0 amplitude 1e5."""
    l0 = uneven_boxes((n0,) * 3, [16, 32, 48], np.random.default_rng(seed), p_stop=0.35)
    fine = bubble_boxes((n0,) * 3, nbubbles=3, cover=0.01, block_edges=(8, 16), max_edge=16,
                        rng=np.random.default_rng(seed + 1))
    return spherical_amr_config(n0=n0, nspec=nspec, ppm_type=2, fine_boxes=fine, level0_boxes=l0, w0_amp=1.0e5)


def planar_config_2d(n=(64, 64), nspec=3, ppm_type=1, bc_lo=(INTERIOR, SLIPWALL), bc_hi=(INTERIOR, OUTFLOW),
                     max_grid=None, boxes=None, seed=20261203, rho_pert=0.0, w0_amp=0.0, cfl=0.7, gpi_amp=0.0,
                     species_pred_type=1, enthalpy_pred_type=1, slope_order=4, evolve_base_state=1):
    """2-D plane-parallel configuration (y radial): rho0(y) = 1e7 exp(-y/H), H = L/4,
    p0 = rho0 |g| H; NumSpec mass fractions from 6 seeded Gaussian bumps each;
    rho h = rho (1e17 + 1e16 G) with G a unit-RMS sum of 8 Fourier modes; rhoh0 = the
    horizontal mean of rho h; divergence-free velocity from a seeded streamfunction of 8
    modes (evaluated at nodes, differenced to faces, averaged to cells) scaled to Mach 0.01;
    w0 = 0 unless w0_amp is given.  Arrays are [ncomp, 1, ny, nx]; boxes carry k = 0.
    """
    rng = np.random.default_rng(seed)
    nx, ny = int(n[0]), int(n[1])
    dx = (L_DOMAIN / nx, L_DOMAIN / ny, 1.0)
    periodic = [bc_lo[d] == INTERIOR for d in range(2)]
    H = 0.25 * L_DOMAIN
    x = (np.arange(nx) + 0.5) * dx[0]
    y = (np.arange(ny) + 0.5) * dx[1]
    rho0 = 1.0e7 * np.exp(-y / H)
    p0 = rho0 * abs(GRAV) * H
    X = np.zeros((nspec, ny, nx))
    for s in range(nspec):
        for _ in range(6):
            w = rng.uniform(0.05, 0.2) * L_DOMAIN
            c = rng.uniform(0, L_DOMAIN, size=2)
            A = rng.uniform(0.2, 1.0)
            gx = _gauss1d(c[0], w, L_DOMAIN, periodic[0], dx[0], nx)
            gy = _gauss1d(c[1], w, L_DOMAIN, periodic[1], dx[1], ny)
            X[s] += A * gy[:, None] * gx[None, :]
    X = np.maximum(X, 1.0e-10)
    X /= X.sum(axis=0, keepdims=True)

    def smooth():
        f = np.zeros((ny, nx))
        for _ in range(8):
            kx, ky = rng.integers(1, 5, size=2)
            px, py = rng.uniform(0, 2 * math.pi, size=2)
            f += rng.normal() * np.cos(2 * math.pi * ky * y / L_DOMAIN + py)[:, None] * \
                np.cos(2 * math.pi * kx * x / L_DOMAIN + px)[None, :]
        return f / math.sqrt(float(np.mean(f * f)))

    rho = rho0[:, None] * (1.0 + rho_pert * smooth()) if rho_pert else np.repeat(rho0[:, None], nx, axis=1)
    h = 1.0e17 + 1.0e16 * smooth()
    rhoh = rho * h
    rhoh0 = rhoh.mean(axis=1)
    nscal = 4 + nspec
    sold = np.zeros((nscal, 1, ny, nx))
    sold[RHO, 0] = rho
    sold[RHOH, 0] = rhoh
    sold[TEMP, 0] = 1.0e8
    sold[FIRSTSPEC:, 0] = rho[None] * X
    # streamfunction at nodes; u = dpsi/dy on x faces, v = -dpsi/dx on y faces
    xn = np.arange(nx + 1) * dx[0]
    yn = np.arange(ny + 1) * dx[1]
    psi = np.zeros((ny + 1, nx + 1))
    for _ in range(8):
        km, lm = rng.integers(1, 5, size=2)
        phi = rng.uniform(0, 2 * math.pi)
        a = rng.normal()
        psi += a * np.sin(math.pi * km * yn / L_DOMAIN)[:, None] * np.cos(2 * math.pi * lm * xn / L_DOMAIN + phi)[None, :]
    uf = (psi[1:, :] - psi[:-1, :]) / dx[1]          # x faces (ny, nx+1)
    vf = -(psi[:, 1:] - psi[:, :-1]) / dx[0]         # y faces (ny+1, nx)
    u = np.zeros((3, 1, ny, nx))
    u[0, 0] = 0.5 * (uf[:, 1:] + uf[:, :-1])
    u[1, 0] = 0.5 * (vf[1:, :] + vf[:-1, :])
    cs = math.sqrt(5.0 / 3.0 * abs(GRAV) * H)
    u *= 0.01 * cs / np.abs(u).max()
    u = u[:2]
    r_edge = np.arange(ny + 1) * dx[1]
    w0 = np.zeros(ny + 1)
    if w0_amp:
        for m in range(1, 5):
            w0 += rng.normal() * np.sin(m * math.pi * r_edge / L_DOMAIN)
        w0 *= w0_amp / np.abs(w0).max()
        w0[0] = 0.0
    gpi = np.zeros((2, 1, ny, nx))
    if gpi_amp:
        for d in range(2):
            gpi[d, 0] = gpi_amp * abs(GRAV) * rho0[:, None] * smooth()
    umax_d = [float(np.abs(u[0]).max()), max(float(np.abs(u[1]).max()), float(np.abs(u[1]).max() + np.abs(w0).max()))]
    umax = max(umax_d)
    dt = cfl * min(dx[d] / umax_d[d] for d in range(2))
    if boxes is None:
        mg = max_grid or max(nx, ny)
        boxes = [(b[0], b[1], 0, b[3], b[4], 0) for b in tile_boxes((nx, ny, 1), (mg, mg, 1))]
    from .basestate import cell_to_edge
    return dict(
        dim=2, n=(nx, ny, 1), dx=dx, nspec=nspec, ppm_type=ppm_type, slope_order=slope_order,
        bc_lo=(bc_lo[0], bc_lo[1], INTERIOR), bc_hi=(bc_hi[0], bc_hi[1], INTERIOR),
        species_pred_type=species_pred_type, enthalpy_pred_type=enthalpy_pred_type,
        evolve_base_state=evolve_base_state, dt=dt, rel_eps=1.0e-8 * umax, base_cutoff_density=1.0e3,
        buoyancy_cutoff_factor=5.0, boxes=boxes, seed=seed,
        uold=np.ascontiguousarray(u), sold=np.ascontiguousarray(sold), gpi=gpi, thermal=np.zeros((1, 1, ny, nx)),
        rho0_old=rho0.copy(), rho0_new=rho0.copy(), rhoh0_old=rhoh0.copy(), rhoh0_new=rhoh0.copy(),
        p0_old=p0.copy(), p0_new=p0.copy(), psi=np.zeros(ny), grav_cell=np.full(ny, GRAV),
        w0_force=np.zeros(ny), w0=w0, rho0_predicted_edge=cell_to_edge(rho0),
    )


def workload_2d(n=256, nspec=3, seed=20261203):
    """2-D single level, one n x n box, NumSpec 3, ppm_type 1, w0 = 0, x periodic,
    y slipwall (lo) / outflow (hi)."""
    return planar_config_2d(n=(n, n), nspec=nspec, ppm_type=1, seed=seed)
