"""Writes the golden fixtures of tests/golden/ from the reference's own stage functions
(oracle/_ref/libmaestro_ref.so: the reference sources compiled unmodified against the
stand-ins in oracle/refshim/).  Run where the reference sources are present:

    python tests/golden/make_golden.py

Each fixture holds the seeded inputs and the reference's outputs; tests/test_golden.py
checks the oracle against them and tests/test_golden_gpu.py the GPU library, on hosts
without the reference.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]

import pyref  # noqa: E402
from maestroex_gb300 import configs  # noqa: E402
from maestroex_gb300.params import FIRSTSPEC, INTERIOR, NOSLIPWALL, OUTFLOW, RHO, RHOH, SLIPWALL, SYMMETRY  # noqa: E402
from test_reference_pin import field, ppm_inputs  # noqa: E402

# whole-stage fixtures: small single-level configurations (the inputs are stored with the
# outputs, so that hosts whose random streams differ still read the same values)
STAGE_FIXTURES = {
    "planar_ppm1_w0": lambda: configs.planar_config(n=(16, 12, 12), nspec=2, ppm_type=1, max_grid=(8, 12, 12),
                                                    seed=901, w0_amp=1.0e4),
    "planar_ppm2_walls": lambda: configs.planar_config(n=(12, 12, 16), nspec=2, ppm_type=2, max_grid=(12, 6, 8),
                                                       bc_lo=(SYMMETRY, SLIPWALL, NOSLIPWALL),
                                                       bc_hi=(OUTFLOW, SLIPWALL, OUTFLOW), seed=902, cfl=0.5),
    "spherical_ppm2": lambda: configs.spherical_config(n=12, nspec=2, ppm_type=2, max_grid=6),
    "planar_2d_ppm1": lambda: configs.planar_config_2d(n=(32, 32), nspec=2, ppm_type=1, max_grid=16, rho_pert=1e-3,
                                                       w0_amp=1e4),
}
STAGE_INPUTS = ("uold", "sold", "gpi", "rho0_old", "rho0_new", "rhoh0_old", "rhoh0_new", "p0_old", "p0_new", "psi",
                "grav_cell", "w0_force", "w0", "rho0_predicted_edge")

# (ppm_type, is_umac, bc lo[3] hi[3]): every BCType on some face, both tracing velocities
PPM_FIXTURES = [
    (1, 1, (4, 0, 3, 2, 0, 4)), (1, 0, (3, 1, -1, 4, 2, 2)),
    (2, 1, (4, 0, 3, 2, 0, 4)), (2, 0, (3, 1, -1, 4, 2, 2)),
    (2, 1, (3, 4, 2, 0, 3, 1)), (1, 1, (2, 2, 4, 3, 4, 3)),
]
SLOPE_FIXTURES = [(so, d) for so in (2, 4) for d in range(3)]


def main():
    dom_n = (10, 8, 8)
    out = {}
    for c, (ppm_type, is_umac, bc) in enumerate(PPM_FIXTURES):
        bx = (-1, -1, -1, dom_n[0], dom_n[1], dom_n[2])
        p, s, s_lo, vel, vel_lo = ppm_inputs(500 + c, ppm_type, is_umac, dom_n, bx)
        Ip, Im = pyref.ppm(p, bx, s, s_lo, 1, vel, vel_lo, is_umac, bc)
        pre = f"ppm{c}_"
        out[pre + "meta"] = np.array([ppm_type, is_umac, *bc, *bx, *s_lo, *dom_n], dtype=np.int64)
        out[pre + "real"] = np.array([p.dt, p.rel_eps, *p.dx])
        out[pre + "s"] = s
        for d in range(3):
            out[pre + f"vel{d}"] = vel[d]
        out[pre + "Ip"] = Ip
        out[pre + "Im"] = Im
    rng = np.random.default_rng(3000)
    for c, (so, d) in enumerate(SLOPE_FIXTURES):
        dom = (0, 0, 0, dom_n[0] - 1, dom_n[1] - 1, dom_n[2] - 1)
        bx = (-1, -1, -1, dom_n[0], dom_n[1], dom_n[2])
        lo = [bx[e] - 2 for e in range(3)]
        n = [bx[3 + e] - bx[e] + 5 for e in range(3)]
        s = np.stack([field(rng, lo, n, 10.0 ** (k + 1)) for k in range(3)])
        bcs = [tuple(int(v) for v in rng.choice((-1, 0, 1, 2, 3, 4), size=6)) for _ in range(3)]
        pre = f"slope{c}_"
        out[pre + "meta"] = np.array([so, d, *dom, *bx, *lo], dtype=np.int64)
        out[pre + "bcs"] = np.array(bcs, dtype=np.int64)
        out[pre + "s"] = s
        out[pre + "slope"] = pyref.slopes(so, d, dom, bx, s, lo, bcs)
    np.savez_compressed(os.path.join(HERE, "ppm_slopes.npz"), **out)
    print(f"wrote {len(PPM_FIXTURES)} PPM and {len(SLOPE_FIXTURES)} slope fixtures")

    out = {}
    for name, make in STAGE_FIXTURES.items():
        cfg = make()
        nd = 2 if cfg.get("dim") == 2 else 3
        ref = pyref.run_stage_2d(cfg) if nd == 2 else pyref.run_stage(cfg)
        comps = [RHO, RHOH] + list(range(FIRSTSPEC, FIRSTSPEC + cfg["nspec"]))
        for k in STAGE_INPUTS:
            out[f"{name}_in_{k}"] = cfg[k]
        out[f"{name}_snew"] = ref["snew"][comps]
        for d in range(nd):
            out[f"{name}_umac_end{d}"] = ref["umac_end"][d]
            out[f"{name}_sflux{d}_rho"] = ref["sflux"][d][RHO]
    np.savez_compressed(os.path.join(HERE, "stage.npz"), **out)
    print(f"wrote {len(STAGE_FIXTURES)} stage fixtures")


if __name__ == "__main__":
    main()
