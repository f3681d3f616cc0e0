"""GPU parity of the single-box PPM entry point (madv_ppm, the drop-in for Maestro::PPM)
against the oracle's restatement of Source/MaestroPPM.cpp, bit for bit."""
import numpy as np
import pytest

import pyoracle
from maestroex_gb300 import configs
from maestroex_gb300.params import make_params

pytestmark = pytest.mark.gpu

# BCType values: int_dir 0, reflect_even 1, foextrap 2, ext_dir 3, hoextrap 4
BCS = [(4, 0, 2, 2, 0, 3), (3, 1, 4, 4, 1, 2), (2, 0, 3, 3, 0, 4)]


def ppm_case(ppm_type, is_umac, bc, seed, bx=(-1, 3, 11, 12, 16, 24), ndom=24, comp=1):
    rng = np.random.default_rng(seed)
    cfg = configs.planar_config(n=(ndom, ndom, ndom), nspec=1, ppm_type=ppm_type, max_grid=ndom, seed=seed)
    p = make_params(cfg)
    g = 3 if ppm_type == 2 else 2
    lo = [bx[d] - g for d in range(3)]
    n = [bx[3 + d] - bx[d] + 1 + 2 * g for d in range(3)]
    z, y, x = np.meshgrid(*[np.arange(lo[d], lo[d] + n[d]) for d in (2, 1, 0)], indexing="ij")
    s = np.empty((2, n[2], n[1], n[0]))
    s[0] = 1.0
    s[1] = 1e7 * np.exp(-z / 9.0) * (1 + 0.3 * np.sin(0.7 * x) * np.cos(0.45 * y)) + rng.normal(0, 3e4, z.shape)
    s[1][rng.random(z.shape) < 0.05] = 5e6  # plateaus: exact ties in the limiters
    vel, vel_lo = [], []
    for d in range(3):
        m = [bx[3 + e] - bx[e] + 1 + (1 if (is_umac and e == d) else 0) for e in range(3)]
        v = rng.normal(0, 3e5, (1, m[2], m[1], m[0]))
        v[rng.random(v.shape) < 0.1] = 0.0
        v[rng.random(v.shape) < 0.05] = p.rel_eps
        vel.append(v)
        vel_lo.append(bx[:3])
    return p, s, lo, vel, vel_lo


@pytest.mark.parametrize("ppm_type", [1, 2])
@pytest.mark.parametrize("is_umac", [1, 0])
@pytest.mark.parametrize("bci", range(len(BCS)))
def test_madv_ppm_matches_oracle(ppm_type, is_umac, bci):
    import torch
    from maestroex_gb300.stage import ScalarAdvectionStage
    bx = (-1, 3, 11, 12, 16, 24)
    p, s, s_lo, vel, vel_lo = ppm_case(ppm_type, is_umac, BCS[bci], 900 + 10 * bci + ppm_type)
    Ip_ref, Im_ref = pyoracle.ppm(p, bx, s, s_lo, 1, vel, vel_lo, is_umac, BCS[bci])
    st = ScalarAdvectionStage(p)
    dev = torch.device("cuda")
    ts = torch.from_numpy(s).to(dev)
    tv = [torch.from_numpy(np.ascontiguousarray(v)).to(dev) for v in vel]
    n = [bx[3 + d] - bx[d] + 1 for d in range(3)]
    Ip = torch.full((3, n[2], n[1], n[0]), float("nan"), dtype=torch.float64, device=dev)
    Im = torch.full_like(Ip, float("nan"))
    st.ppm(bx, ts, s_lo, 1, tv, vel_lo, is_umac, BCS[bci], Ip, Im)
    torch.cuda.synchronize()
    assert np.array_equal(Ip.cpu().numpy(), Ip_ref)
    assert np.array_equal(Im.cpu().numpy(), Im_ref)
    st.close()
