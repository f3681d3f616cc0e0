"""madv_ppm_noalloc -- PPM on one box without any device allocation -- against madv_ppm.

Some callers cannot call cudaMalloc where they run PPM: an AMReX application whose arena
already holds most of the GPU's memory, or code that must not pay the implicit device
synchronisation of cudaMalloc/cudaFree.  For them madv_ppm_noalloc keeps its scratch in a
static device array.  This test calls it twice in a row through the C ABI, with different
inputs, parameters and box sizes, and checks each result against madv_ppm (which grows
its scratch with cudaMalloc) within the suite's tolerance: 1e-12 of the component's
max-norm.  It also checks that a box too large for the static array is refused.

The file name sorts last so that a run stopping at the first failure has run every other
test first; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _built():
    from maestroex_gb300 import build
    build.build_library()


def make_inputs(ppm_type, is_umac, bx, seed, dev):
    import torch
    rng = np.random.default_rng(seed)
    g = 3 if ppm_type == 2 else 2
    lo = [bx[d] - g for d in range(3)]
    n = [bx[3 + d] - bx[d] + 1 + 2 * g for d in range(3)]
    z, y, x = np.meshgrid(*[np.arange(lo[d], lo[d] + n[d]) for d in (2, 1, 0)], indexing="ij")
    s = np.empty((3, n[2], n[1], n[0]))
    s[0] = 1.0
    s[1] = 2.0
    s[2] = 1e7 * np.exp(-z / 11.0) * (1 + 0.2 * np.sin(0.6 * x) * np.cos(0.35 * y)) + rng.normal(0, 2e4, z.shape)
    vel = []
    for d in range(3):
        m = [bx[3 + e] - bx[e] + 1 + (1 if (is_umac and e == d) else 0) for e in range(3)]
        v = rng.normal(0, 3e5, (1, m[2], m[1], m[0]))
        v[rng.random(v.shape) < 0.1] = 0.0
        vel.append(torch.from_numpy(v).to(dev))
    return torch.from_numpy(s).to(dev), lo, vel


def params_for(ppm_type, ndom=64):
    from maestroex_gb300 import configs
    from maestroex_gb300.params import make_params
    cfg = configs.planar_config(n=(ndom, ndom, ndom), nspec=1, ppm_type=ppm_type, max_grid=ndom, seed=77)
    return make_params(cfg)


def call_noalloc(p, bx, s, s_lo, comp, vel, is_umac, bc, Ip, Im):
    import torch
    from maestroex_gb300 import capi
    from maestroex_gb300.stage import fab_of_tensor
    fabs = [fab_of_tensor(s, s_lo)] + [fab_of_tensor(vel[d], bx[:3]) for d in range(3)] + \
           [fab_of_tensor(Ip, bx[:3]), fab_of_tensor(Im, bx[:3])]
    box = capi.MadvBox()
    for d in range(3):
        box.lo[d], box.hi[d] = bx[d], bx[3 + d]
    return capi.lib().madv_ppm_noalloc(C.byref(p), C.byref(box), C.byref(fabs[0]), comp, C.byref(fabs[1]),
                                       C.byref(fabs[2]), C.byref(fabs[3]), is_umac, (C.c_int * 6)(*bc),
                                       C.byref(fabs[4]), C.byref(fabs[5]),
                                       C.c_void_p(torch.cuda.current_stream().cuda_stream))


def rel(a, b):
    a = a.cpu().numpy()
    b = b.cpu().numpy()
    return max(float(np.abs(a[c] - b[c]).max() / max(np.abs(b[c]).max(), 1e-300)) for c in range(3))


def test_noalloc_ppm_matches_madv_ppm_twice_in_a_row():
    import torch
    from maestroex_gb300 import capi
    from maestroex_gb300.stage import ScalarAdvectionStage
    dev = torch.device("cuda")
    # call 1: ppm_type 1, face velocity, a 64^3 box grown by one cell next to hoextrap / ext_dir walls
    # call 2: ppm_type 2, cell velocity, a smaller uneven box next to the opposite walls
    calls = [
        (1, 1, (-1, -1, -1, 64, 64, 64), (4, 0, 3, 2, 0, 4), 2, 11),
        (2, 0, (20, 30, 10, 47, 48, 35), (2, 4, 0, 3, 4, 0), 2, 12),
    ]
    outs = []
    for ppm_type, is_umac, bx, bc, comp, seed in calls:
        p = params_for(ppm_type)
        s, s_lo, vel = make_inputs(ppm_type, is_umac, bx, seed, dev)
        n = [bx[3 + d] - bx[d] + 1 for d in range(3)]
        Ip = torch.full((3, n[2], n[1], n[0]), float("nan"), dtype=torch.float64, device=dev)
        Im = torch.full_like(Ip, float("nan"))
        rc = call_noalloc(p, bx, s, s_lo, comp, vel, is_umac, bc, Ip, Im)
        assert rc == 0, capi.lib().madv_last_error().decode()
        outs.append((p, bx, s, s_lo, comp, vel, is_umac, bc, Ip, Im))
    torch.cuda.synchronize()
    for p, bx, s, s_lo, comp, vel, is_umac, bc, Ip, Im in outs:
        st = ScalarAdvectionStage(p)
        Ip_ref = torch.full_like(Ip, float("nan"))
        Im_ref = torch.full_like(Im, float("nan"))
        st.ppm(bx, s, s_lo, comp, vel, [bx[:3]] * 3, is_umac, bc, Ip_ref, Im_ref)
        torch.cuda.synchronize()
        assert torch.isfinite(Ip_ref).all() and torch.isfinite(Im_ref).all()
        assert rel(Ip, Ip_ref) <= TOL
        assert rel(Im, Im_ref) <= TOL
        st.close()


def test_noalloc_refuses_boxes_beyond_its_scratch():
    import torch
    from maestroex_gb300 import capi
    from maestroex_gb300.stage import fab_of_tensor
    p = params_for(1, ndom=128)
    bx = (0, 0, 0, 79, 79, 79)
    dummy = torch.zeros((1, 1, 1, 1), dtype=torch.float64, device="cuda")
    f = fab_of_tensor(dummy, (0, 0, 0))
    box = capi.MadvBox()
    for d in range(3):
        box.lo[d], box.hi[d] = bx[d], bx[3 + d]
    rc = capi.lib().madv_ppm_noalloc(C.byref(p), C.byref(box), C.byref(f), 0, C.byref(f), C.byref(f), C.byref(f),
                                     1, (C.c_int * 6)(0, 0, 0, 0, 0, 0), C.byref(f), C.byref(f), None)
    assert rc == -2
    assert b"static" in capi.lib().madv_last_error()
