"""Test infrastructure only: the CPU oracle of Maestro::MacProj, 3-D, one level,
plane-parallel or spherical (Source/MaestroMacProj.cpp:11-236, MultFacesByBeta0 :238-329, ComputeMACSolverRHS
:331-372, SetMacSolverBCs :424-453).  Nothing in the product library uses this file; the
tests compare the GPU projection with it.

The discrete problem is restated and solved to 1e-14 of its rhs (diagonally preconditioned
conjugate gradients; for a singular operator on the mean-free rhs), so the comparison is
against the solution of the same discrete system; the GPU multigrid meets the reference's stopping test
(max|residual| <= tol_rel max|rhs|), so the two agree to the tolerance, not bitwise.

Parity status: unpinned (the reference's MLMG cannot be built here); the oracle follows the
reference's discretisation: B = beta0^2 / (0.5 (rho_l + rho_r)) (average_cellcenter_to_face,
invert, MultFacesByBeta0 twice with use_alt_energy_fix), the 7-point operator
-div(B grad phi), outflow faces Dirichlet phi = 0 through the ghost 2 phi_b - phi_0 (MLMG,
maxorder 2), other physical faces Neumann, and fluxes -B grad phi added to beta0 umac.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

INTERIOR, OUTFLOW = 0, 2


def cell_to_edge(cc):
    """Maestro::CelltoEdge on one chunk (Source/MaestroCelltoEdge.cpp:17-54): 4th-order
    interior edges clamped between the neighbours, 2nd order next to the ends."""
    nr = len(cc)
    e = np.zeros(nr + 1)
    for r in range(nr + 1):
        if r == 0:
            e[r] = cc[0]
        elif r == 1:
            e[r] = 0.5 * (cc[0] + cc[1])
        elif r == nr:
            e[r] = cc[nr - 1]
        elif r == nr - 1:
            e[r] = 0.5 * (cc[r] + cc[r - 1])
        else:
            t = 7.0 / 12.0 * (cc[r] + cc[r - 1]) - 1.0 / 12.0 * (cc[r + 1] + cc[r - 2])
            e[r] = min(max(t, min(cc[r - 1], cc[r])), max(cc[r - 1], cc[r]))
    return e


def mac_project(umac, macrhs, rho, beta0, dx, bc_lo, bc_hi, beta_faces=None):
    """umac: [x faces (nz, ny, nx+1), y faces (nz, ny+1, nx), z faces (nz+1, ny, nx)];
    macrhs, rho: (nz, ny, nx); beta0: (nz,).  bc_lo / bc_hi: PhysBCType per direction
    (x, y, z).  beta_faces: spherical geometry, beta0 on the faces (MakeS0mac of beta0,
    Source/MaestroMacProj.cpp:41-44), three arrays shaped like umac, used in place of beta0
    and its CelltoEdge.  Returns (projected umac, phi)."""
    nz, ny, nx = rho.shape
    n = (nx, ny, nz)
    per = [bc_lo[d] == INTERIOR for d in range(3)]
    kind = []  # per direction: (lo, hi) in {"per", "dir", "neu"}
    for d in range(3):
        if per[d]:
            kind.append(("per", "per"))
        else:
            kind.append(tuple("dir" if b == OUTFLOW else "neu" for b in (bc_lo[d], bc_hi[d])))
    # beta0 on the faces: plane-parallel, x and y faces beta0(k), z faces beta0_edge(k);
    # spherical, the given face arrays
    if beta_faces is None:
        b0 = np.asarray(beta0, dtype=np.float64)
        b0e = cell_to_edge(b0)
        bz = [b0[:, None, None], b0[:, None, None], b0e[:, None, None]]
    else:
        bz = [np.asarray(b, dtype=np.float64) for b in beta_faces]
    bu = [umac[d] * bz[d] for d in range(3)]
    rhs = macrhs - ((bu[0][:, :, 1:] - bu[0][:, :, :-1]) / dx[0] + (bu[1][:, 1:, :] - bu[1][:, :-1, :]) / dx[1] +
                    (bu[2][1:, :, :] - bu[2][:-1, :, :]) / dx[2])
    # face coefficients (axis order of the arrays is z, y, x: direction d is axis 2 - d)
    B = []
    for d in range(3):
        ax = 2 - d
        r = np.moveaxis(rho, ax, -1)
        if per[d]:
            left = np.concatenate([r[..., -1:], r], axis=-1)
            right = np.concatenate([r, r[..., :1]], axis=-1)
        else:
            left = np.concatenate([r[..., :1], r], axis=-1)
            right = np.concatenate([r, r[..., -1:]], axis=-1)
        face = 0.5 * (left + right)
        Bd = np.moveaxis(1.0 / face, -1, ax)
        Bd = Bd * bz[d]
        Bd = Bd * bz[d]
        B.append(Bd)
    # the operator -div(B grad phi)
    N = nx * ny * nz
    idx = np.arange(N).reshape(nz, ny, nx)
    rows, cols, vals = [], [], []
    diag = np.zeros((nz, ny, nx))
    for d in range(3):
        ax = 2 - d
        ih2 = 1.0 / (dx[d] * dx[d])
        Bd = np.moveaxis(B[d], ax, -1)
        I = np.moveaxis(idx, ax, -1)
        w = Bd * ih2  # (.., n+1)
        m = n[d]
        # interior faces 1..m-1 couple cells f-1 and f
        wi = w[..., 1:m]
        a, b = I[..., :m - 1], I[..., 1:m]
        rows += [a.ravel(), b.ravel()]
        cols += [b.ravel(), a.ravel()]
        vals += [-wi.ravel(), -wi.ravel()]
        dg = np.zeros(I.shape)
        dg[..., :m - 1] += wi
        dg[..., 1:m] += wi
        lo, hi = kind[d]
        if lo == "per":
            wp = w[..., 0]
            rows += [I[..., 0].ravel(), I[..., m - 1].ravel()]
            cols += [I[..., m - 1].ravel(), I[..., 0].ravel()]
            vals += [-wp.ravel(), -wp.ravel()]
            dg[..., 0] += wp
            dg[..., m - 1] += wp
        else:
            if lo == "dir":
                dg[..., 0] += 2.0 * w[..., 0]
            if hi == "dir":
                dg[..., m - 1] += 2.0 * w[..., m]
        diag += np.moveaxis(dg, -1, ax)
    rows.append(idx.ravel())
    cols.append(idx.ravel())
    vals.append(diag.ravel())
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))
    singular = not any("dir" in kind[d] for d in range(3))
    f = rhs.ravel().copy()
    if singular:
        f -= f.mean()
    # conjugate gradients with the diagonal as preconditioner, to 1e-14 of the rhs
    M = sp.diags(1.0 / A.diagonal())
    phi, info = spla.cg(A, f, rtol=1e-14, atol=0.0, maxiter=50000, M=M)
    assert info == 0, "oracle CG did not converge"
    if singular:
        phi -= phi.mean()
    phi = phi.reshape(nz, ny, nx)
    # fluxes -B grad phi on every face, added to beta0 umac, then divided by beta0
    out = []
    for d in range(3):
        ax = 2 - d
        P = np.moveaxis(phi, ax, -1)
        m = n[d]
        grad = np.zeros(P.shape[:-1] + (m + 1,))
        grad[..., 1:m] = (P[..., 1:] - P[..., :-1]) / dx[d]
        lo, hi = kind[d]
        if lo == "per":
            grad[..., 0] = grad[..., m] = (P[..., 0] - P[..., m - 1]) / dx[d]
        else:
            grad[..., 0] = (P[..., 0] - (-P[..., 0])) / dx[d] if lo == "dir" else 0.0
            grad[..., m] = ((-P[..., m - 1]) - P[..., m - 1]) / dx[d] if hi == "dir" else 0.0
        flux = -np.moveaxis(B[d], ax, -1) * grad
        u = np.moveaxis(bu[d], ax, -1) + flux
        out.append(np.moveaxis(u, -1, ax) / bz[d])
    return out, phi
