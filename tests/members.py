"""Inputs of the per-member-function parity tests: per-box FABs (ghost cells included) cut
from padded domain arrays, so that the GPU entry points and the oracle read the same
values, ghost cells included, whatever the boundary conditions."""
import numpy as np

from maestroex_gb300.params import FIRSTSPEC, RHO, RHOH

PAD = 5


def pad(a):
    """Domain array [nc, nz, ny, nx] (faces: +1 in their direction) padded by PAD cells."""
    return np.pad(a, ((0, 0), (PAD, PAD), (PAD, PAD), (PAD, PAD)), mode="reflect")


def cut(padded, boxes, g, nodal=-1):
    """Per-box FABs [(array, lo)] of the boxes grown by g (faces: nodal in direction `nodal`)."""
    out = []
    for bx in boxes:
        lo = [bx[d] - g for d in range(3)]
        hi = [bx[3 + d] + g for d in range(3)]
        if nodal >= 0:
            hi[nodal] += 1
        sl = tuple(slice(lo[d] + PAD, hi[d] + PAD + 1) for d in (2, 1, 0))
        out.append((np.ascontiguousarray(padded[(slice(None),) + sl]), lo))
    return out


def zeros_like(fabs):
    return [(np.zeros_like(a), lo) for a, lo in fabs]


def faces_of(cells, d):
    """Face values of a padded cell array in direction d (arithmetic mean of the two cells),
    with the same PAD convention (one more entry along d)."""
    a = np.moveaxis(cells, 3 - d, -1)
    f = np.empty(a.shape[:-1] + (a.shape[-1] + 1,))
    f[..., 1:-1] = 0.5 * (a[..., :-1] + a[..., 1:])
    f[..., 0] = a[..., 0]
    f[..., -1] = a[..., -1]
    return np.ascontiguousarray(np.moveaxis(f, -1, 3 - d))


class MemberInputs:
    """Seeded inputs of every member function for one configuration."""

    def __init__(self, cfg, seed=7):
        rng = np.random.default_rng(seed)
        self.cfg = cfg
        self.boxes = cfg["boxes"]
        self.nscal = 4 + cfg["nspec"]
        self.nspec = cfg["nspec"]
        self.ng = 4 if cfg["ppm_type"] == 2 else 3
        u = cfg["uold"]
        s = cfg["sold"]
        umax = float(np.abs(u).max())
        dt = cfg["dt"]
        shape = u.shape[1:]
        U = pad(u)
        self.utilde = U
        self.ufull = U + pad(0.01 * umax * rng.standard_normal((3,) + shape))
        self.vel_force = pad(0.05 * umax / dt * rng.standard_normal((3,) + shape))
        # transverse / MAC velocities: face means of the cell velocity, padded
        self.uface = [faces_of(U[d:d + 1], d) for d in range(3)]
        S = pad(s)
        self.state = S
        self.scal_force = pad(1e-3 * np.abs(s) / dt * rng.standard_normal(s.shape))
        self.sedge = [faces_of(S, d) for d in range(3)]
        self.sflux = [faces_of(S * U[d:d + 1], d) * (1.0 + 1e-3 * rng.standard_normal(self.sedge[d].shape))
                      for d in range(3)]
        self.eta = faces_of(S[RHO:RHO + 1] * 1e-3, 2)

    def fabs(self, name, g=0):
        b = self.boxes
        if name in ("utilde", "ufull", "vel_force", "state", "scal_force"):
            return cut(getattr(self, name), b, g)
        if name in ("uface", "sedge", "sflux"):
            return [cut(getattr(self, name)[d], b, g, d) for d in range(3)]
        if name == "eta":
            return cut(self.eta, b, g, 2)
        raise KeyError(name)


__all__ = ["MemberInputs", "cut", "zeros_like", "pad", "faces_of", "RHO", "RHOH", "FIRSTSPEC"]
