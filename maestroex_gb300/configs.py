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


def uneven_boxes(n, edges, rng):
    """Seeded guillotine split of the domain into boxes whose edges come from `edges`."""
    out = []

    def split(lo, hi):
        ext = [hi[d] - lo[d] for d in range(3)]
        if all(e in edges for e in ext) and rng.random() < 0.35:
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


def config_c2(n=256, box=64, nspec=13, seed=20261203 + 1):
    """Config 2: 3-D single level, 256^3 in 64 boxes of 64^3, NumSpec 13, ppm_type 1, w0 != 0."""
    return planar_config(n=(n, n, n), nspec=nspec, ppm_type=1, max_grid=box, seed=seed,
                         w0_amp=1.0e4, cfl=0.7)
