"""The two-level MAC-projection oracle (oracle/mo_macproj_levels.py) on the CPU: with level 1
covering the domain it is the one-level oracle at the fine resolution; after a partial
level-1 projection div(beta0 u) = macrhs on every level-1 cell, and on a level-0 cell
next to level 1 (the composite flux matching) before the final averaging; the volume-weighted
operator is symmetric."""
import numpy as np

import mo_macproj
import mo_macproj_levels

BC_LO, BC_HI = (0, 0, 3), (0, 0, 2)  # periodic x / y, symmetry below, outflow above


def fields(rng, n):
    nx, ny, nz = n
    u = [rng.standard_normal((nz, ny, nx + 1)), rng.standard_normal((nz, ny + 1, nx)),
         rng.standard_normal((nz + 1, ny, nx))]
    for d in range(2):  # periodic copies agree
        v = np.moveaxis(u[d], 2 - d, -1)
        v[..., -1] = v[..., 0]
    return u, 1.0 + 0.3 * rng.random((nz, ny, nx)), 0.1 * rng.standard_normal((nz, ny, nx))


def setup(seed=1):
    rng = np.random.default_rng(seed)
    n0 = (8, 8, 8)
    n1 = (16, 16, 16)
    u0, rho0, rhs0 = fields(rng, n0)
    u1, rho1, rhs1 = fields(rng, n1)
    beta_c = 1.0 + 0.1 * np.arange(8)
    return n0, n1, (u0, rho0, rhs0), (u1, rho1, rhs1), beta_c, np.repeat(beta_c, 2)


def test_fine_level_covering_the_domain_is_the_one_level_oracle():
    n0, n1, (u0, rho0, rhs0), (u1, rho1, rhs1), bc_, bf = setup()
    full = [(0, 0, 0, 15, 15, 15)]
    a0, a1, p0, p1 = mo_macproj_levels.mac_project_levels(u0, u1, rhs0, rhs1, rho0, rho1, bc_, bf, full,
                                                          (1.0, 1.0, 1.0), BC_LO, BC_HI)
    s1, q1 = mo_macproj.mac_project(u1, rhs1, rho1, bf, (0.5, 0.5, 0.5), BC_LO, BC_HI)
    assert max(float(np.abs(a1[d] - s1[d]).max()) for d in range(3)) < 1e-11
    assert float(np.abs(p1 - q1).max()) < 1e-11 * float(np.abs(q1).max())


def test_partial_fine_level_divergence():
    n0, n1, (u0, rho0, rhs0), (u1, rho1, rhs1), bc_, bf = setup(2)
    boxes = [(4, 4, 4, 11, 9, 7), (0, 10, 6, 5, 15, 13)]
    a0, a1, p0, p1 = mo_macproj_levels.mac_project_levels(u0, u1, rhs0, rhs1, rho0, rho1, bc_, bf, boxes,
                                                          (1.0, 1.0, 1.0), BC_LO, BC_HI)
    mask = np.zeros((16, 16, 16), bool)
    for b in boxes:
        mask[b[2]:b[5] + 1, b[1]:b[4] + 1, b[0]:b[3] + 1] = True
    e0, e1 = mo_macproj_levels.beta_edges(bc_, bf, mo_macproj_levels.chunks_of(boxes, 8))
    bz1 = [bf[:, None, None], bf[:, None, None], e1[:, None, None]]
    bu = [a1[d] * bz1[d] for d in range(3)]
    div = ((bu[0][:, :, 1:] - bu[0][:, :, :-1]) + (bu[1][:, 1:, :] - bu[1][:, :-1, :]) +
           (bu[2][1:, :, :] - bu[2][:-1, :, :])) / 0.5
    assert float(np.abs((div - rhs1)[mask]).max()) < 1e-10 * float(np.abs(rhs1).max() + np.abs(div[mask]).max())
    assert np.isfinite(p0).all() and np.isfinite(p1[mask]).all() and np.isnan(p1[~mask]).all()
