"""Test infrastructure only: the CPU oracle of the two-level MAC projection (Maestro::MacProj
on an AMR hierarchy, Source/MaestroMacProj.cpp:11-236, plane-parallel, refinement ratio 2).
Nothing in the product library uses this file; the tests compare the GPU projection with it.

Parity status: unpinned.  The reference solves the composite problem with AMReX's MLMG,
whose coarse-fine boundary interpolation is not in the reference tree; this oracle states
the composite discretisation the library implements and solves it directly:

* unknowns: phi on the level-0 cells no level-1 box covers, and on the level-1 cells;
* a level-1 cell uses the 7-point operator -div(B grad phi) with spacing h1; across a
  coarse-fine face its neighbour is the ghost value (1/3) phi_fine + (2/3) phi_parent (the
  linear interpolant along the face normal between the fine cell's centre, h1/2 inside, and
  the coarse cell's, h1 outside), so the face flux is B (2/3) (phi_c - phi_parent) / h1^2;
* a level-0 cell uses the 7-point operator with spacing h0, except that across a face
  shared with a covered cell (a coarse-fine face) its flux is the mean of the four fine
  fluxes through it (flux matching, as reflux does);
* with volume weights this operator is symmetric; it is solved directly;
* covered level-0 cells take the mean of their eight children's phi;
* B = beta0^2 / (0.5 (rho_l + rho_r)) per level (a level-1 face on the coarse-fine boundary
  takes the parent coarse cell's rho outside); beta0 per level, CelltoEdge over the level's
  radial chunks and the fine edges restricted onto the coarse ones (RestrictBase);
* umac is averaged down (level-1 faces onto the level-0 faces under them) as the reference
  does (AverageDownFaces): beta0 umac before the rhs is formed, umac after the correction.
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from mo_macproj import INTERIOR, OUTFLOW


def chunks_of(fine_boxes, nr0):
    """Radial chunks of level 1 (BaseStateGeometry::InitMultiLevel, planar): runs of level-0
    rows under a level-1 box, as [2 r0, 2 r1 + 1]."""
    tag = np.zeros(nr0, dtype=bool)
    for b in fine_boxes:
        tag[b[2] // 2:b[5] // 2 + 1] = True
    out, r = [], 0
    while r < nr0:
        if tag[r]:
            s = r
            while r < nr0 and tag[r]:
                r += 1
            out.append((2 * s, 2 * r - 1))
        else:
            r += 1
    return out


def cell_to_edge_chunk(cc, e, lo, hi):
    """Maestro::CelltoEdge on the edges lo .. hi of one chunk of a level's rows
    (Source/MaestroCelltoEdge.cpp:17-54): the chunk's end edges average the cells on either
    side (the cells outside the chunk belong to the level's rows too), the domain's end edges
    take the end cell, the others the clamped 4th-order interpolant."""
    nr = len(cc)
    for r in range(lo, hi + 1):
        if r == 0:
            e[r] = cc[r]
        elif r == 1 or r == lo:
            e[r] = 0.5 * (cc[r - 1] + cc[r])
        elif r == nr:
            e[r] = cc[r - 1]
        elif r == nr - 1 or r == hi:
            e[r] = 0.5 * (cc[r] + cc[r - 1])
        else:
            t = 7.0 / 12.0 * (cc[r] + cc[r - 1]) - 1.0 / 12.0 * (cc[r + 1] + cc[r - 2])
            e[r] = min(max(t, min(cc[r - 1], cc[r])), max(cc[r - 1], cc[r]))


def beta_edges(beta_c, beta_f, chunks):
    """Edge values of beta0 on both levels: CelltoEdge per chunk (level 0: one chunk of all
    its rows), then the fine edges of each chunk restricted onto the coarse edges (every
    second one, RestrictBase)."""
    bc, bf = np.asarray(beta_c, dtype=np.float64), np.asarray(beta_f, dtype=np.float64)
    e0, e1 = np.zeros(len(bc) + 1), np.zeros(len(bf) + 1)
    cell_to_edge_chunk(bc, e0, 0, len(bc))
    for a, b in chunks:
        cell_to_edge_chunk(bf, e1, a, b + 1)
    for a, b in chunks:
        for j in range(a, b + 2, 2):
            e0[j // 2] = e1[j]
    return e0, e1


def mac_project_levels(u0, u1, rhs0, rhs1, rho0, rho1, beta_c, beta_f, fine_boxes, dx0, bc_lo, bc_hi):
    """u0 / u1: level-0 / level-1 face velocities as domain arrays [x (nz, ny, nx+1), y, z];
    rhs*, rho*: (nz, ny, nx) domain arrays of each level (level 1: the fine domain, read on
    its boxes only); beta_c / beta_f: beta0 per level (nr0, nr1 = 2 nr0 rows).  Returns
    (u0', u1', phi0, phi1): projected velocities (level-0 faces under level 1 averaged down)
    and phi (level 1: NaN off the boxes)."""
    nz0, ny0, nx0 = rho0.shape
    n0 = np.array([nx0, ny0, nz0])
    n1 = 2 * n0
    h0 = np.asarray(dx0, dtype=np.float64)
    h1 = h0 / 2
    per = [bc_lo[d] == INTERIOR for d in range(3)]
    kind = [("per", "per") if per[d] else tuple("dir" if b == OUTFLOW else "neu" for b in (bc_lo[d], bc_hi[d]))
            for d in range(3)]
    mask = np.zeros((n1[2], n1[1], n1[0]), dtype=bool)
    for b in fine_boxes:
        mask[b[2]:b[5] + 1, b[1]:b[4] + 1, b[0]:b[3] + 1] = True
    cov = mask.reshape(nz0, 2, ny0, 2, nx0, 2).all(axis=(1, 3, 5))
    e0, e1 = beta_edges(beta_c, beta_f, chunks_of(fine_boxes, nz0))
    bz0 = [np.asarray(beta_c)[:, None, None], np.asarray(beta_c)[:, None, None], e0[:, None, None]]
    bz1 = [np.asarray(beta_f)[:, None, None], np.asarray(beta_f)[:, None, None], e1[:, None, None]]

    def face_ok1(d):  # level-1 faces that belong to a level-1 box (either side in the mask)
        m = np.moveaxis(mask, 2 - d, -1)
        ok = np.zeros(m.shape[:-1] + (m.shape[-1] + 1,), dtype=bool)
        ok[..., :-1] |= m
        ok[..., 1:] |= m
        if per[d]:
            ok[..., 0] |= m[..., -1]
            ok[..., -1] |= m[..., 0]
        return np.moveaxis(ok, -1, 2 - d)

    ok1 = [face_ok1(d) for d in range(3)]
    bu1 = [np.where(ok1[d], np.nan_to_num(u1[d]) * bz1[d], np.nan) for d in range(3)]
    bu0 = [u0[d] * bz0[d] for d in range(3)]

    def avg_down(fine, d, coarse):  # coarse faces under level 1 = mean of the 4 fine faces
        t = [0, 1, 2]
        t.remove(d)
        out = coarse.copy()
        nf = list(n1)
        nf[d] += 1
        for k in range(n0[2] + (d == 2)):
            for j in range(n0[1] + (d == 1)):
                for i in range(n0[0] + (d == 0)):
                    a = [i, j, k]
                    s, ok = 0.0, True
                    for q in range(4):
                        b = [2 * a[0], 2 * a[1], 2 * a[2]]
                        b[t[0]] += q & 1
                        b[t[1]] += q >> 1
                        v = fine[b[2], b[1], b[0]]
                        if not np.isfinite(v):
                            ok = False
                            break
                        s += v
                    if ok:
                        out[k, j, i] = 0.25 * s
        return out

    bu0 = [avg_down(bu1[d], d, bu0[d]) for d in range(3)]

    def div(bu, h):
        return ((bu[0][:, :, 1:] - bu[0][:, :, :-1]) / h[0] + (bu[1][:, 1:, :] - bu[1][:, :-1, :]) / h[1] +
                (bu[2][1:, :, :] - bu[2][:-1, :, :]) / h[2])

    f0 = rhs0 - div(bu0, h0)
    f1 = np.where(mask, np.nan_to_num(rhs1) - np.nan_to_num(div(bu1, h1)), 0.0)
    # unknown numbering: uncovered coarse cells, then fine cells
    id0 = -np.ones(cov.shape, dtype=np.int64)
    id0[~cov] = np.arange((~cov).sum())
    id1 = -np.ones(mask.shape, dtype=np.int64)
    id1[mask] = (~cov).sum() + np.arange(mask.sum())
    N = int((~cov).sum() + mask.sum())
    vol = np.concatenate([np.ones((~cov).sum()), np.full(mask.sum(), 0.125)])
    # rho on the fine faces' outside: the parent coarse cell
    rho1f = np.where(mask, np.nan_to_num(rho1), np.repeat(np.repeat(np.repeat(rho0, 2, 0), 2, 1), 2, 2))

    def Bfaces(rho, bz, n):
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
            Bd = np.moveaxis(1.0 / (0.5 * (left + right)), -1, ax)
            B.append(Bd * bz[d] * bz[d])
        return B

    B0, B1 = Bfaces(rho0, bz0, n0), Bfaces(rho1f, bz1, n1)
    A = sp.lil_matrix((N, N))
    b = np.zeros(N)

    def nbr(n, idx, d, s):  # neighbour index along d (s = -1 / +1), or None at a non-periodic edge
        j = list(idx)
        j[d] += s
        if j[d] < 0 or j[d] >= n[d]:
            if not per[d]:
                return None
            j[d] %= n[d]
        return j

    for k in range(n1[2]):
        for j in range(n1[1]):
            for i in range(n1[0]):
                if not mask[k, j, i]:
                    continue
                r_ = id1[k, j, i]
                b[r_] = f1[k, j, i]
                for d in range(3):
                    for s in (-1, 1):
                        fidx = [i, j, k]
                        if s == 1:
                            fidx[d] += 1
                        w = B1[d][fidx[2], fidx[1], fidx[0]] / (h1[d] * h1[d])
                        q = nbr(n1, (i, j, k), d, s)
                        if q is None:
                            t = kind[d][0 if s < 0 else 1]
                            if t == "dir":
                                A[r_, r_] += 2.0 * w
                            continue
                        if mask[q[2], q[1], q[0]]:
                            A[r_, r_] += w
                            A[r_, id1[q[2], q[1], q[0]]] -= w
                        else:  # coarse-fine face: ghost (1/3) phi_c + (2/3) phi_parent
                            pc = id0[q[2] // 2, q[1] // 2, q[0] // 2]
                            A[r_, r_] += (2.0 / 3.0) * w
                            A[r_, pc] -= (2.0 / 3.0) * w
    for k in range(n0[2]):
        for j in range(n0[1]):
            for i in range(n0[0]):
                if cov[k, j, i]:
                    continue
                r_ = id0[k, j, i]
                b[r_] = f0[k, j, i]
                for d in range(3):
                    for s in (-1, 1):
                        fidx = [i, j, k]
                        if s == 1:
                            fidx[d] += 1
                        q = nbr(n0, (i, j, k), d, s)
                        if q is None:
                            if kind[d][0 if s < 0 else 1] == "dir":
                                A[r_, r_] += 2.0 * B0[d][fidx[2], fidx[1], fidx[0]] / (h0[d] * h0[d])
                            continue
                        if not cov[q[2], q[1], q[0]]:
                            w = B0[d][fidx[2], fidx[1], fidx[0]] / (h0[d] * h0[d])
                            A[r_, r_] += w
                            A[r_, id0[q[2], q[1], q[0]]] -= w
                            continue
                        # coarse-fine face: the mean of the 4 fine fluxes, each B (2/3) (phi_C - phi_c) / h1
                        t = [0, 1, 2]
                        t.remove(d)
                        for m in range(4):
                            c = [2 * q[0], 2 * q[1], 2 * q[2]]
                            if s == 1:
                                c[d] = 2 * q[d]
                            else:
                                c[d] = 2 * q[d] + 1
                            c[t[0]] += m & 1
                            c[t[1]] += m >> 1
                            ff = list(c)
                            if s == -1:
                                ff[d] = c[d] + 1
                            wf = 0.25 * (2.0 / 3.0) * B1[d][ff[2], ff[1], ff[0]] / (h0[d] * h1[d])
                            A[r_, r_] += wf
                            A[r_, id1[c[2], c[1], c[0]]] -= wf
    A = A.tocsr()
    singular = not any("dir" in kind[d] for d in range(3))
    if singular:
        b -= (vol * b).sum() / vol.sum()
        # pin the null space: solve with one extra row fixing the volume-weighted mean
        Aa = sp.vstack([sp.hstack([A, sp.csr_matrix(vol[:, None])]),
                        sp.hstack([sp.csr_matrix(vol[None, :]), sp.csr_matrix((1, 1))])]).tocsc()
        x = spla.spsolve(Aa, np.concatenate([b, [0.0]]))[:N]
    else:
        x = spla.spsolve(A.tocsc(), b)
    phi0 = np.zeros(cov.shape)
    phi0[~cov] = x[id0[~cov]]
    phi1 = np.full(mask.shape, np.nan)
    phi1[mask] = x[id1[mask]]
    fill = np.where(mask, phi1, 0.0).reshape(nz0, 2, ny0, 2, nx0, 2).mean(axis=(1, 3, 5))
    phi0 = np.where(cov, fill, phi0)

    def corrected(bu, B, phi, n, h, is_fine):
        out = []
        for d in range(3):
            ax = 2 - d
            P = np.moveaxis(phi, ax, -1)
            m = n[d]
            g = np.full(P.shape[:-1] + (m + 1,), np.nan)
            g[..., 1:m] = (P[..., 1:] - P[..., :-1]) / h[d]
            lo, hi = kind[d]
            if lo == "per":
                g[..., 0] = g[..., m] = (P[..., 0] - P[..., m - 1]) / h[d]
            else:
                g[..., 0] = 2.0 * P[..., 0] / h[d] if lo == "dir" else 0.0
                g[..., m] = -2.0 * P[..., m - 1] / h[d] if hi == "dir" else 0.0
            out.append(np.moveaxis(np.moveaxis(bu[d], ax, -1) - np.moveaxis(B[d], ax, -1) * g, -1, ax))
        return out

    # level-1 faces: a coarse-fine face sees the ghost value (1/3) phi_c + (2/3) phi_parent
    par = np.repeat(np.repeat(np.repeat(phi0, 2, 0), 2, 1), 2, 2)
    ghosted = np.where(mask, phi1, np.nan)
    bun1 = []
    for d in range(3):
        ax = 2 - d
        Pm = np.moveaxis(ghosted, ax, -1)
        Pp = np.moveaxis(par, ax, -1)
        M = np.moveaxis(mask, ax, -1)
        m = n1[d]
        g = np.full(Pm.shape[:-1] + (m + 1,), np.nan)
        for f in range(m + 1):
            li, ri = f - 1, f
            if f == 0 or f == m:
                if per[d]:
                    li, ri = m - 1, 0
                else:
                    side = 0 if f == 0 else 1
                    cell = 0 if f == 0 else m - 1
                    pv = Pm[..., cell]
                    if kind[d][side] == "dir":
                        g[..., f] = np.where(M[..., cell], (2.0 * pv if f == 0 else -2.0 * pv) / h1[d], np.nan)
                    else:
                        g[..., f] = np.where(M[..., cell], 0.0, np.nan)
                    continue
            lm, rm = M[..., li], M[..., ri]
            lv = np.where(lm, Pm[..., li], (1.0 / 3.0) * np.nan_to_num(Pm[..., ri]) + (2.0 / 3.0) * Pp[..., li])
            rv = np.where(rm, Pm[..., ri], (1.0 / 3.0) * np.nan_to_num(Pm[..., li]) + (2.0 / 3.0) * Pp[..., ri])
            g[..., f] = np.where(lm | rm, (rv - lv) / h1[d], np.nan)
        bun1.append(np.moveaxis(np.moveaxis(bu1[d], ax, -1) - np.moveaxis(B1[d], ax, -1) * g, -1, ax))
    bun0 = corrected(bu0, B0, phi0, n0, h0, False)
    u1n = [bun1[d] / bz1[d] for d in range(3)]
    # the level-0 faces under level 1 take the mean of the fine velocities (AverageDownFaces of
    # umac after the division by beta0)
    u0n = [avg_down(u1n[d], d, bun0[d] / bz0[d]) for d in range(3)]
    return u0n, u1n, phi0, phi1
