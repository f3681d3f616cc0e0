"""The GPU library's PPM (madv_ppm, the drop-in for Maestro::PPM) against golden fixtures
written by the reference's own PPM (tests/golden/make_golden.py): bit for bit."""
import numpy as np
import pytest

from test_golden import golden, ppm_fixture

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from maestroex_gb300 import build
    build.build_library()


@pytest.mark.parametrize("c", range(6))
def test_madv_ppm_matches_golden(c):
    import torch
    from maestroex_gb300.stage import ScalarAdvectionStage
    p, ppm_type, is_umac, bc, bx, s, s_lo, vel, Ip_ref, Im_ref = ppm_fixture(golden(), c)
    st = ScalarAdvectionStage(p)
    dev = torch.device("cuda")
    ts = torch.from_numpy(np.ascontiguousarray(s)).to(dev)
    tv = [torch.from_numpy(np.ascontiguousarray(v)).to(dev) for v in vel]
    n = [bx[3 + d] - bx[d] + 1 for d in range(3)]
    Ip = torch.full((3, n[2], n[1], n[0]), float("nan"), dtype=torch.float64, device=dev)
    Im = torch.full_like(Ip, float("nan"))
    st.ppm(bx, ts, s_lo, 1, tv, [bx[:3]] * 3, is_umac, bc, Ip, Im)
    torch.cuda.synchronize()
    assert np.array_equal(Ip.cpu().numpy(), Ip_ref)
    assert np.array_equal(Im.cpu().numpy(), Im_ref)
    st.close()


@pytest.mark.parametrize("name", ("planar_ppm1_w0", "planar_ppm2_walls", "spherical_ppm2", "planar_2d_ppm1"))
def test_gpu_stage_matches_golden(name):
    """The whole stage on the GPU (graph-replayed batched kernels) against the reference's
    own stage on the same inputs, bit for bit."""
    from maestroex_gb300 import capi
    from maestroex_gb300.stage import run_stage_gpu
    from test_golden import check_stage, stage_fixture
    cfg, ref = stage_fixture(name)
    check_stage(cfg, run_stage_gpu(cfg, mode=capi.MODE_GRAPH), ref, name)
