"""Test infrastructure only: ctypes binding of the reference's own stage functions,
compiled unmodified from the reference sources against the stand-ins in oracle/refshim/
(oracle/Makefile, target `ref`, output oracle/_ref/libmaestro_ref.so).

Available only where the reference tree is present (the development host); tests that use
it skip elsewhere.  The fixtures it generates (tests/golden/) carry its results to hosts
without the reference.
"""
import ctypes as C
import os
import subprocess

import numpy as np

import pyoracle

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("MAESTRO_REFERENCE", "/root/reference")
_LIB = []


def available():
    return os.path.isdir(os.path.join(REF, "Source"))


NUMSPECS = (2, 3, 5, 13)  # the reference's NumSpec is a compile-time constant: one build each
NUMSPECS_2D = (2, 3)


def lib(nspec=3, dim=3):
    """The reference build for NumSpec = nspec in dim dimensions
    (oracle/_ref/ns<nspec>[_2d]/libmaestro_ref.so)."""
    if not _LIB:
        if not available():
            raise RuntimeError(f"reference sources not found under {REF}")
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF}"], check=True)
        _LIB.append({})
    if nspec not in (NUMSPECS if dim == 3 else NUMSPECS_2D):
        raise ValueError(f"no {dim}-D reference build for NumSpec {nspec}")
    libs = _LIB[0]
    key = (nspec, dim)
    if key not in libs:
        L = C.CDLL(os.path.join(HERE, "_ref", f"ns{nspec}" + ("_2d" if dim == 2 else ""), "libmaestro_ref.so"))
        L.ref_last_error.restype = C.c_char_p
        libs[key] = L
    return libs[key]


def _check(rc, nspec=3):
    if rc != 0:
        raise RuntimeError("reference: " + lib(nspec).ref_last_error().decode())


def ppm(params, bx, s, s_lo, comp, vel, vel_lo, is_umac, bc):
    """Maestro::PPM of the reference on box bx, same arguments and results as pyoracle.ppm."""
    n = [bx[3 + d] - bx[d] + 1 for d in range(3)]
    Ip = np.full((3, n[2], n[1], n[0]), np.nan)
    Im = np.full((3, n[2], n[1], n[0]), np.nan)
    keep = []
    fs, a = pyoracle.fab_of(s, s_lo); keep.append(a)
    fv = []
    for d in range(3):
        f, a = pyoracle.fab_of(vel[d], vel_lo[d]); keep.append(a); fv.append(f)
    fip, _ = pyoracle.fab_of(Ip, bx[:3])
    fim, _ = pyoracle.fab_of(Im, bx[:3])
    dom = (C.c_int * 6)(*params.dom_lo, *params.dom_hi)
    dx = (C.c_double * 3)(*params.dx)
    _check(lib().ref_ppm(int(params.ppm_type), C.c_double(params.dt), C.c_double(params.rel_eps), dx, dom,
                         (C.c_int * 6)(*bx), C.byref(fs), int(comp), C.byref(fv[0]), C.byref(fv[1]), C.byref(fv[2]),
                         int(is_umac), (C.c_int * 6)(*bc), C.byref(fip), C.byref(fim)))
    return Ip, Im


def slopes(slope_order, d, dom, bx, s, s_lo, bcs):
    """Maestro::Slopex/y/z of the reference, same arguments and result as pyoracle.slopes."""
    n = [bx[3 + e] - bx[e] + 1 for e in range(3)]
    out = np.full((s.shape[0], n[2], n[1], n[0]), np.nan)
    keep = []
    fs, a = pyoracle.fab_of(s, s_lo); keep.append(a)
    fo, _ = pyoracle.fab_of(out, bx[:3])
    _check(lib().ref_slopes(int(slope_order), int(d), (C.c_int * 6)(*dom), (C.c_int * 6)(*bx), C.byref(fs),
                            s.shape[0], (C.c_int * (6 * len(bcs)))(*[v for b in bcs for v in b]), C.byref(fo)))
    return out


def member(cfg, fn, args, which_step=1, start_comp=0, num_comp=0, is_conservative=0):
    """The reference's own member function on caller FABs, same arguments as
    pyoracle.member (outputs written into the argument arrays, valid cells / faces only)."""
    L = lib(cfg["nspec"])
    pyoracle.member_call(L, L.ref_member, L.ref_last_error, cfg, fn, args, which_step, start_comp, num_comp,
                         is_conservative)


def run_stage(cfg, want=("umac_vp", "umac_end", "sedge", "sflux", "snew", "sold_end", "etarhoflux")):
    """The stage of pyoracle.run_stage run by the reference's own AdvancePremac,
    DensityAdvance and EnthalpyAdvance (utrans and vel_force stay inside AdvancePremac)."""
    L = lib(cfg["nspec"])
    return pyoracle.run_stage(cfg, want=want, _entry=(L.ref_run_stage, L.ref_last_error))


def run_velocity_advance(cfg, rhohalf, sponge=None):
    """pyoracle.run_velocity_advance run by the reference's own AdvancePremac and
    VelocityAdvance (unew and umac; uedge stays inside VelocityAdvance)."""
    L = lib(cfg["nspec"])
    return pyoracle.run_velocity_advance(cfg, rhohalf, sponge, _entry=(L.ref_run_velocity_advance, L.ref_last_error))


def run_stage_2d(cfg):
    """pyoracle.run_stage_2d run by the reference's own 2-D stage (AMREX_SPACEDIM 2 build)."""
    L = lib(cfg["nspec"], dim=2)
    return pyoracle.run_stage_2d(cfg, _entry=(L.ref_run_stage, L.ref_last_error))
