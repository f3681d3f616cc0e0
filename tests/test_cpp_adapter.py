"""The Maestro-shaped C++ layer (include/maestro_adv.hpp) over the C ABI.

tests/cpp/maestro_adapter_main.cpp runs the scalar-advection calls of
Maestro::AdvanceTimeStep (AdvancePremac, Addw0, DensityAdvance, EnthalpyAdvance) with the
reference's member signatures over a MultiFab of device FABs.  The CPU test compiles and
links it against libmaestro_adv.so; the GPU test runs it and compares every output with
the oracle's stage (bitwise, like the Python path).
"""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from maestroex_gb300 import build, configs
from maestroex_gb300.params import FIRSTSPEC, RHO, RHOH, make_params

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "maestro_adapter_main.cpp")
BASE_KEYS = ("rho0_old", "rho0_new", "rhoh0_old", "rhoh0_new", "p0_old", "p0_new", "psi", "grav_cell",
             "w0_force", "w0", "rho0_predicted_edge")
HAVE_NVCC = shutil.which("nvcc") is not None or os.path.exists("/usr/local/cuda/bin/nvcc")


def compile_adapter(out_dir):
    lib = build.build_library()
    exe = os.path.join(out_dir, "maestro_adapter_main")
    cmd = [build.nvcc(), "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", os.path.dirname(lib), "-lmaestro_adv", "-Xlinker", "-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    assert r.returncode == 0, r.stdout.decode()
    return exe


def write_input(cfg, path):
    raw = bytes(make_params(cfg))
    with open(path, "wb") as f:
        f.write(struct.pack("<i", len(raw)))
        f.write(raw)
        f.write(struct.pack("<i", len(cfg["boxes"])))
        for b in cfg["boxes"]:
            f.write(struct.pack("<6i", *[int(v) for v in b]))
        nr = cfg["n"][2]
        f.write(struct.pack("<i", nr))
        for k in BASE_KEYS:
            a = np.ascontiguousarray(cfg[k], dtype="<f8")
            assert a.size == (nr + 1 if k in ("w0", "rho0_predicted_edge") else nr), k
            f.write(a.tobytes())
        for k in ("uold", "sold", "gpi", "thermal"):
            f.write(np.ascontiguousarray(cfg[k], dtype="<f8").tobytes())


def read_output(cfg, path):
    nx, ny, nz = cfg["n"]
    nscal = 4 + cfg["nspec"]
    raw = np.fromfile(path, dtype="<f8")
    pos = 0

    def take(nc, nodal=-1):
        nonlocal pos
        n = [nx, ny, nz]
        if nodal >= 0:
            n[nodal] += 1
        size = nc * n[0] * n[1] * n[2]
        a = raw[pos:pos + size].reshape(nc, n[2], n[1], n[0])
        pos += size
        return a

    res = dict(snew=take(nscal), sold_end=take(nscal))
    res["umac_end"] = [take(1, d)[0] for d in range(3)]
    res["sedge"] = [take(nscal, d) for d in range(3)]
    res["sflux"] = [take(nscal, d) for d in range(3)]
    res["etarhoflux"] = take(1, 2)[0]
    assert pos == raw.size
    return res


def test_input_file_layout(tmp_path):
    cfg = configs.planar_config(n=(16, 8, 8), nspec=2, ppm_type=1, max_grid=8, seed=3)
    path = str(tmp_path / "in.bin")
    write_input(cfg, path)
    ncell = 16 * 8 * 8
    nr = 8
    want = 4 + len(bytes(make_params(cfg))) + 4 + 24 * len(cfg["boxes"]) + 4 + 8 * (9 * nr + 2 * (nr + 1)) + \
        8 * ncell * (3 + 6 + 3 + 1)
    assert os.path.getsize(path) == want


@pytest.mark.skipif(not HAVE_NVCC, reason="needs nvcc")
def test_adapter_compiles_and_links(tmp_path):
    exe = compile_adapter(str(tmp_path))
    assert os.path.exists(exe)


@pytest.mark.gpu
@pytest.mark.parametrize("ppm_type,nspec", [(1, 3), (2, 2), (0, 2)])
def test_adapter_stage_matches_oracle(tmp_path, ppm_type, nspec):
    import pyoracle
    cfg = configs.planar_config(n=(16, 24, 32), nspec=nspec, ppm_type=ppm_type, max_grid=(16, 8, 16),
                                seed=900 + ppm_type)
    exe = compile_adapter(str(tmp_path))
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    write_input(cfg, fin)
    r = subprocess.run([exe, fin, fout], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, timeout=300)
    assert r.returncode == 0, r.stdout.decode()
    got = read_output(cfg, fout)
    ref = pyoracle.run_stage(cfg, checked=False)
    comps = [RHO, RHOH] + list(range(FIRSTSPEC, FIRSTSPEC + nspec))
    for c in comps:
        assert np.array_equal(got["snew"][c], ref["snew"][c]), f"snew comp {c}"
        assert np.array_equal(got["sold_end"][c], ref["sold_end"][c]), f"sold comp {c}"
    for d in range(3):
        assert np.array_equal(got["umac_end"][d], ref["umac_end"][d]), f"umac[{d}]"
        for c in comps:
            assert np.array_equal(got["sedge"][d][c], ref["sedge"][d][c]), f"sedge[{d}] comp {c}"
            assert np.array_equal(got["sflux"][d][c], ref["sflux"][d][c]), f"sflux[{d}] comp {c}"
    assert np.array_equal(got["etarhoflux"], ref["etarhoflux"])
