"""Test infrastructure only: ctypes binding of the CPU oracle (the checker).

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs.  The
product library never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS = {}


class MoInputs(C.Structure):
    _fields_ = [(name, C.POINTER(C.c_double)) for name in (
        "uold", "sold", "gpi", "thermal", "rho0_old", "rho0_new", "rhoh0_old", "rhoh0_new",
        "p0_old", "p0_new", "psi", "grav_cell", "w0_force", "w0", "rho0_predicted_edge")]


class MoOutputs(C.Structure):
    _fields_ = [
        ("utrans", C.POINTER(C.c_double) * 3),
        ("umac_vp", C.POINTER(C.c_double) * 3),
        ("umac_end", C.POINTER(C.c_double) * 3),
        ("vel_force", C.POINTER(C.c_double)),
        ("sedge", C.POINTER(C.c_double) * 3),
        ("sflux", C.POINTER(C.c_double) * 3),
        ("snew", C.POINTER(C.c_double)),
        ("sold_end", C.POINTER(C.c_double)),
        ("etarhoflux", C.POINTER(C.c_double)),
    ]


def build():
    """Compile the oracle shared libraries with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib(checked=False):
    name = "libmaestro_oracle_chk.so" if checked else "libmaestro_oracle.so"
    if name not in _LIBS:
        path = os.path.join(HERE, name)
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.mo_run_stage.restype = C.c_int
        L.mo_run_stage_levels.restype = C.c_int
        L.mo_run_stage_2d.restype = C.c_int
        L.mo_last_error.restype = C.c_char_p
        _LIBS[name] = L
    return _LIBS[name]


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def run_stage(cfg, checked=False, nthreads=0, want=("utrans", "umac_vp", "umac_end", "vel_force",
                                                      "sedge", "sflux", "snew", "sold_end",
                                                      "etarhoflux"), _entry=None):
    """Run AdvancePremac + DensityAdvance + EnthalpyAdvance on the CPU; returns numpy arrays.
    _entry: (call, last_error) of another C entry with mo_run_stage's arguments but the
    thread count (the reference build's, pyref.run_stage)."""
    from maestroex_gb300.params import make_params
    p = make_params(cfg)
    n = cfg["n"]
    nscal = 4 + cfg["nspec"]
    keep = []

    def arr(x):
        a = np.ascontiguousarray(x, dtype=np.float64)
        keep.append(a)
        return _p(a)

    inp = MoInputs()
    for name in ("uold", "sold", "gpi", "thermal", "rho0_old", "rho0_new", "rhoh0_old", "rhoh0_new",
                 "p0_old", "p0_new", "psi", "grav_cell", "w0_force", "w0", "rho0_predicted_edge"):
        setattr(inp, name, arr(cfg[name]))
    out = MoOutputs()
    res = {}
    fshape = [(n[2], n[1], n[0] + 1), (n[2], n[1] + 1, n[0]), (n[2] + 1, n[1], n[0])]
    for key in ("utrans", "umac_vp", "umac_end"):
        if key in want:
            res[key] = [np.full(fshape[d], np.nan) for d in range(3)]
            for d in range(3):
                getattr(out, key)[d] = _p(res[key][d])
    for key in ("sedge", "sflux"):
        if key in want:
            res[key] = [np.full((nscal,) + fshape[d], np.nan) for d in range(3)]
            for d in range(3):
                getattr(out, key)[d] = _p(res[key][d])
    cshape = (n[2], n[1], n[0])
    if "vel_force" in want:
        res["vel_force"] = np.full((3,) + cshape, np.nan)
        out.vel_force = _p(res["vel_force"])
    for key in ("snew", "sold_end"):
        if key in want:
            res[key] = np.full((nscal,) + cshape, np.nan)
            setattr(out, key, _p(res[key]))
    if "etarhoflux" in want:
        res["etarhoflux"] = np.full(fshape[2], np.nan)
        out.etarhoflux = _p(res["etarhoflux"])
    boxes = np.ascontiguousarray(np.array(cfg["boxes"], dtype=np.int32).reshape(-1))
    if _entry is not None:
        call, last_error = _entry
        rc = call(C.byref(p), len(cfg["boxes"]), boxes.ctypes.data_as(C.POINTER(C.c_int)), C.byref(inp),
                  C.byref(out))
        if rc != 0:
            raise RuntimeError(last_error().decode())
        return res
    rc = lib(checked).mo_run_stage(C.byref(p), len(cfg["boxes"]), boxes.ctypes.data_as(C.POINTER(C.c_int)),
                                   C.byref(inp), C.byref(out), nthreads)
    if rc != 0:
        raise RuntimeError("oracle: " + lib(checked).mo_last_error().decode())
    return res


def run_stage_levels(cfg, checked=False, nthreads=0, want=("utrans", "umac_vp", "umac_end", "vel_force",
                                                             "sedge", "sflux", "snew", "sold_end",
                                                             "etarhoflux"), which_step=1):
    """The stage on the hierarchy cfg["levels"]; returns one dict of arrays per level
    (domain-sized at the level's resolution, NaN where the level has no box)."""
    from maestroex_gb300.params import make_params
    p = make_params(cfg)
    levels = cfg["levels"]
    nlev = len(levels)
    nscal = 4 + cfg["nspec"]
    keep = []

    def arr(x):
        a = np.ascontiguousarray(x, dtype=np.float64)
        keep.append(a)
        return _p(a)

    ins = (MoInputs * nlev)()
    outs = (MoOutputs * nlev)()
    res = []
    for lev, L in enumerate(levels):
        inp = ins[lev]
        for name in ("uold", "sold", "gpi", "thermal", "rho0_old", "rho0_new", "rhoh0_old", "rhoh0_new",
                     "p0_old", "p0_new", "psi", "grav_cell", "w0_force", "w0", "rho0_predicted_edge"):
            setattr(inp, name, arr(L[name]))
        n = L["n"]
        out = outs[lev]
        r = {}
        fshape = [(n[2], n[1], n[0] + 1), (n[2], n[1] + 1, n[0]), (n[2] + 1, n[1], n[0])]
        for key in ("utrans", "umac_vp", "umac_end"):
            if key in want:
                r[key] = [np.full(fshape[d], np.nan) for d in range(3)]
                for d in range(3):
                    getattr(out, key)[d] = _p(r[key][d])
        for key in ("sedge", "sflux"):
            if key in want:
                r[key] = [np.full((nscal,) + fshape[d], np.nan) for d in range(3)]
                for d in range(3):
                    getattr(out, key)[d] = _p(r[key][d])
        cshape = (n[2], n[1], n[0])
        if "vel_force" in want:
            r["vel_force"] = np.full((3,) + cshape, np.nan)
            out.vel_force = _p(r["vel_force"])
        for key in ("snew", "sold_end"):
            if key in want:
                r[key] = np.full((nscal,) + cshape, np.nan)
                setattr(out, key, _p(r[key]))
        if "etarhoflux" in want:
            r["etarhoflux"] = np.full(fshape[2], np.nan)
            out.etarhoflux = _p(r["etarhoflux"])
        res.append(r)
    nboxes = (C.c_int * nlev)(*[len(L["boxes"]) for L in levels])
    boxes = np.ascontiguousarray(np.array([b for L in levels for b in L["boxes"]], dtype=np.int32).reshape(-1))
    rc = lib(checked).mo_run_stage_levels(C.byref(p), nlev, nboxes, boxes.ctypes.data_as(C.POINTER(C.c_int)),
                                          ins, outs, which_step, nthreads)
    if rc != 0:
        raise RuntimeError("oracle: " + lib(checked).mo_last_error().decode())
    return res


def run_stage_2d(cfg, checked=False, nthreads=0, which_step=1, _entry=None):
    """The 2-D stage (configs.planar_config_2d) on the CPU; arrays shaped like the inputs:
    cells [nc, 1, ny, nx], x faces [.., 1, ny, nx+1], y faces [.., 1, ny+1, nx]."""
    from maestroex_gb300.params import make_params
    p = make_params(cfg)
    nx, ny = cfg["n"][0], cfg["n"][1]
    nscal = 4 + cfg["nspec"]
    keep = []

    def arr(x):
        a = np.ascontiguousarray(x, dtype=np.float64)
        keep.append(a)
        return _p(a)

    inp = MoInputs()
    for name in ("uold", "sold", "gpi", "thermal", "rho0_old", "rho0_new", "rhoh0_old", "rhoh0_new",
                 "p0_old", "p0_new", "psi", "grav_cell", "w0_force", "w0", "rho0_predicted_edge"):
        setattr(inp, name, arr(cfg[name]))
    out = MoOutputs()
    fshape = [(1, ny, nx + 1), (1, ny + 1, nx)]
    res = {}
    for key in ("utrans", "umac_vp", "umac_end"):
        res[key] = [np.full(fshape[d], np.nan) for d in range(2)]
        for d in range(2):
            getattr(out, key)[d] = _p(res[key][d])
    for key in ("sedge", "sflux"):
        res[key] = [np.full((nscal,) + fshape[d], np.nan) for d in range(2)]
        for d in range(2):
            getattr(out, key)[d] = _p(res[key][d])
    res["vel_force"] = np.full((2, 1, ny, nx), np.nan)
    out.vel_force = _p(res["vel_force"])
    for key in ("snew", "sold_end"):
        res[key] = np.full((nscal, 1, ny, nx), np.nan)
        setattr(out, key, _p(res[key]))
    res["etarhoflux"] = np.full(fshape[1], np.nan)
    out.etarhoflux = _p(res["etarhoflux"])
    boxes = np.ascontiguousarray(np.array(cfg["boxes"], dtype=np.int32).reshape(-1))
    if _entry is not None:  # (call, last_error) of the reference's 2-D build (predictor only)
        call, last_error = _entry
        call.restype = C.c_int
        if call(C.byref(p), len(cfg["boxes"]), boxes.ctypes.data_as(C.POINTER(C.c_int)), C.byref(inp),
                C.byref(out)) != 0:
            raise RuntimeError(last_error().decode())
        return res
    rc = lib(checked).mo_run_stage_2d(C.byref(p), len(cfg["boxes"]), boxes.ctypes.data_as(C.POINTER(C.c_int)),
                                      C.byref(inp), C.byref(out), which_step, nthreads)
    if rc != 0:
        raise RuntimeError("oracle: " + lib(checked).mo_last_error().decode())
    return res


class MoFab(C.Structure):
    _fields_ = [("p", C.POINTER(C.c_double)), ("lo", C.c_int * 3), ("hi", C.c_int * 3), ("nc", C.c_int)]


def fab_of(arr, lo):
    """mo_fab over a numpy array shaped [nc, nz, ny, nx] whose first cell is `lo`."""
    a = np.ascontiguousarray(arr)
    f = MoFab()
    f.p = a.ctypes.data_as(C.POINTER(C.c_double))
    for d in range(3):
        f.lo[d] = lo[d]
        f.hi[d] = lo[d] + a.shape[3 - d] - 1
    f.nc = a.shape[0]
    return f, a


def ppm(params, bx, s, s_lo, comp, vel, vel_lo, is_umac, bc, checked=True):
    """Oracle Maestro::PPM on box bx (lo0,lo1,lo2,hi0,hi1,hi2); returns (Ip, Im) [3, nz, ny, nx]."""
    n = [bx[3 + d] - bx[d] + 1 for d in range(3)]
    Ip = np.full((3, n[2], n[1], n[0]), np.nan)
    Im = np.full((3, n[2], n[1], n[0]), np.nan)
    keep = []
    fs, a = fab_of(s, s_lo); keep.append(a)
    fv = []
    for d in range(3):
        f, a = fab_of(vel[d], vel_lo[d]); keep.append(a); fv.append(f)
    fip, _ = fab_of(Ip, bx[:3])
    fim, _ = fab_of(Im, bx[:3])
    bcs = (C.c_int * 6)(*bc)
    bxa = (C.c_int * 6)(*bx)
    L = lib(checked)
    rc = L.mo_ppm(C.byref(params), bxa, C.byref(fs), comp, C.byref(fv[0]), C.byref(fv[1]), C.byref(fv[2]),
                  int(is_umac), bcs, C.byref(fip), C.byref(fim))
    if rc != 0:
        raise RuntimeError("oracle: " + L.mo_last_error().decode())
    return Ip, Im


def slopes(slope_order, d, dom, bx, s, s_lo, bcs, checked=True):
    """Oracle Maestro::Slopex/y/z in direction d over bx for every component of s
    ([nc, nz, ny, nx] at s_lo); bcs: one (lo0, lo1, lo2, hi0, hi1, hi2) per component.
    Returns the slopes [nc, nz, ny, nx] on bx (NaN where not written)."""
    n = [bx[3 + e] - bx[e] + 1 for e in range(3)]
    out = np.full((s.shape[0], n[2], n[1], n[0]), np.nan)
    keep = []
    fs, a = fab_of(s, s_lo); keep.append(a)
    fo, _ = fab_of(out, bx[:3])
    L = lib(checked)
    rc = L.mo_slopes(int(slope_order), int(d), (C.c_int * 6)(*dom), (C.c_int * 6)(*bx), C.byref(fs), s.shape[0],
                     (C.c_int * (6 * len(bcs)))(*[v for b in bcs for v in b]), C.byref(fo))
    if rc != 0:
        raise RuntimeError("oracle: " + L.mo_last_error().decode())
    return out


MO_SLOT = dict(utilde=0, ufull=1, utrans=2, umac=5, force=8, state=9, snew=10, sedge=11, sflux=14, eta=17)
MO_FACE_SLOTS = ("utrans", "umac", "sedge", "sflux")
MO_NSLOT = 18
MO_FN = dict(make_utrans=0, vel_pred=1, make_edge_scal=2, make_rhox_flux=3, make_rhoh_flux=4, update_scal=5,
             make_s0mac=6)


def member(cfg, fn, args, which_step=1, start_comp=0, num_comp=0, is_conservative=0, checked=True):
    """Oracle mo_member: one Maestro member function on caller FABs.  args maps a slot name
    to the per-box FABs [(array [nc, nz, ny, nx], lo), ...] (three such lists, one per
    direction, for utrans / umac / sedge / sflux).  Outputs are written into the arrays."""
    L = lib(checked)
    member_call(L, L.mo_member, L.mo_last_error, cfg, fn, args, which_step, start_comp, num_comp, is_conservative)


def member_call(L, entry, last_error, cfg, fn, args, which_step, start_comp, num_comp, is_conservative):
    """Calls a C entry with mo_member's arguments (the oracle's, or the reference build's)."""
    from maestroex_gb300.params import make_params
    p = make_params(cfg)
    nb = len(cfg["boxes"])
    tab = (MoFab * (MO_NSLOT * nb))()
    keep = []
    for name, v in args.items():
        lists = v if name in MO_FACE_SLOTS else [v]
        for d, fabs in enumerate(lists):
            assert len(fabs) == nb
            for b, (a, lo) in enumerate(fabs):
                assert a.dtype == np.float64 and a.flags.c_contiguous
                f, _ = fab_of(a, lo)
                tab[(MO_SLOT[name] + d) * nb + b] = f
                keep.append(a)

    def arr(x):
        a = np.ascontiguousarray(x, dtype=np.float64)
        keep.append(a)
        return _p(a)

    inp = MoInputs()
    for name in ("uold", "sold", "gpi", "thermal", "rho0_old", "rho0_new", "rhoh0_old", "rhoh0_new",
                 "p0_old", "p0_new", "psi", "grav_cell", "w0_force", "w0", "rho0_predicted_edge"):
        setattr(inp, name, arr(cfg[name]))
    boxes = np.ascontiguousarray(np.array(cfg["boxes"], dtype=np.int32).reshape(-1))
    entry.restype = C.c_int
    rc = entry(C.byref(p), nb, boxes.ctypes.data_as(C.POINTER(C.c_int)), C.byref(inp), MO_FN[fn],
               which_step, start_comp, num_comp, is_conservative, tab)
    if rc != 0:
        raise RuntimeError(last_error().decode())


def lib_tl():
    """The tangent-linear build of the oracle (libmaestro_oracle_tl.so)."""
    name = "libmaestro_oracle_tl.so"
    if name not in _LIBS:
        path = os.path.join(HERE, name)
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.mo_run_stage_tl.restype = C.c_int
        L.mo_last_error.restype = C.c_char_p
        _LIBS[name] = L
    return _LIBS[name]


def run_stage_tl(cfg, duold, dsold, nthreads=0):
    """The stage and its tangent-linear model on one level: returns (snew, dsnew), dsnew the
    derivative of snew along (duold, dsold) (domain arrays shaped like uold / sold)."""
    from maestroex_gb300.params import make_params
    p = make_params(cfg)
    n = cfg["n"]
    nscal = 4 + cfg["nspec"]
    keep = []

    def arr(x):
        a = np.ascontiguousarray(x, dtype=np.float64)
        keep.append(a)
        return _p(a)

    inp = MoInputs()
    for name in ("uold", "sold", "gpi", "thermal", "rho0_old", "rho0_new", "rhoh0_old", "rhoh0_new",
                 "p0_old", "p0_new", "psi", "grav_cell", "w0_force", "w0", "rho0_predicted_edge"):
        setattr(inp, name, arr(cfg[name]))
    out = MoOutputs()
    snew = np.full((nscal, n[2], n[1], n[0]), np.nan)
    dsnew = np.full_like(snew, np.nan)
    out.snew = _p(snew)
    boxes = np.ascontiguousarray(np.array(cfg["boxes"], dtype=np.int32).reshape(-1))
    L = lib_tl()
    rc = L.mo_run_stage_tl(C.byref(p), len(cfg["boxes"]), boxes.ctypes.data_as(C.POINTER(C.c_int)), C.byref(inp),
                           arr(duold), arr(dsold), C.byref(out), _p(dsnew), nthreads)
    if rc != 0:
        raise RuntimeError("oracle: " + L.mo_last_error().decode())
    return snew, dsnew


def steps_tl(cfg, s0, ds0, u, du, nsteps, nthreads=0):
    """nsteps of the stage on a fixed velocity u (dt and rel_eps of cfg), the state carried
    as the multi-step adjoint carries it (Rho, RhoH and the species from snew; Temp and Pi
    unchanged), with its tangent along (du, ds0): returns (s_final, ds_final)."""
    from maestroex_gb300.params import FIRSTSPEC, RHO, RHOH
    comps = [RHO, RHOH] + list(range(FIRSTSPEC, s0.shape[0]))
    s, ds = s0.copy(), ds0.copy()
    c = dict(cfg)
    c["uold"] = u
    for _ in range(nsteps):
        c["sold"] = s
        snew, dsnew = run_stage_tl(c, du, ds, nthreads)
        s, ds = s.copy(), ds.copy()
        s[comps] = snew[comps]
        ds[comps] = dsnew[comps]
    return s, ds


def run_velocity_advance(cfg, rhohalf, sponge=None, nthreads=0, checked=False, _entry=None):
    """AdvancePremac (MAC projection skipped) then VelocityAdvance + UpdateVel on the CPU:
    returns dict(unew [3, nz, ny, nx], uedge [3 arrays 3 x faces], umac [3 face arrays])."""
    from maestroex_gb300.params import make_params
    p = make_params(cfg)
    n = cfg["n"]
    keep = []

    def arr(x):
        a = np.ascontiguousarray(x, dtype=np.float64)
        keep.append(a)
        return _p(a)

    inp = MoInputs()
    for name in ("uold", "sold", "gpi", "thermal", "rho0_old", "rho0_new", "rhoh0_old", "rhoh0_new",
                 "p0_old", "p0_new", "psi", "grav_cell", "w0_force", "w0", "rho0_predicted_edge"):
        setattr(inp, name, arr(cfg[name]))
    fshape = [(n[2], n[1], n[0] + 1), (n[2], n[1] + 1, n[0]), (n[2] + 1, n[1], n[0])]
    unew = np.full((3, n[2], n[1], n[0]), np.nan)
    uedge = [np.full((3,) + fshape[d], np.nan) for d in range(3)]
    umac = [np.full(fshape[d], np.nan) for d in range(3)]
    ue = (C.POINTER(C.c_double) * 3)(*[_p(a) for a in uedge])
    um = (C.POINTER(C.c_double) * 3)(*[_p(a) for a in umac])
    boxes = np.ascontiguousarray(np.array(cfg["boxes"], dtype=np.int32).reshape(-1))
    args = (C.byref(p), len(cfg["boxes"]), boxes.ctypes.data_as(C.POINTER(C.c_int)), C.byref(inp), arr(rhohalf),
            arr(sponge) if sponge is not None else None, _p(unew), ue, um)
    if _entry is not None:  # (call, last_error) of the reference build: no thread count
        call, last_error = _entry
        call.restype = C.c_int
        if call(*args) != 0:
            raise RuntimeError(last_error().decode())
        return dict(unew=unew, uedge=uedge, umac=umac)
    L = lib(checked)
    L.mo_run_velocity_advance.restype = C.c_int
    rc = L.mo_run_velocity_advance(*args, nthreads)
    if rc != 0:
        raise RuntimeError("oracle: " + L.mo_last_error().decode())
    return dict(unew=unew, uedge=uedge, umac=umac)


def est_dt(cfg, cfl=0.5, drdxfac=1):
    """Oracle EstDt (advective + force constraints) on cfg's single level or cfg["levels"]:
    returns (dt before the max_dt / fixed_dt limits, umax)."""
    from maestroex_gb300.params import make_params
    p = make_params(cfg)
    levels = cfg["levels"] if "levels" in cfg else [cfg]
    nlev = len(levels)
    keep = []

    def arr(x):
        a = np.ascontiguousarray(x, dtype=np.float64)
        keep.append(a)
        return _p(a)

    ins = (MoInputs * nlev)()
    for lev, Lv in enumerate(levels):
        for name in ("uold", "sold", "gpi", "thermal", "rho0_old", "rho0_new", "rhoh0_old", "rhoh0_new",
                     "p0_old", "p0_new", "psi", "grav_cell", "w0_force", "w0", "rho0_predicted_edge"):
            setattr(ins[lev], name, arr(Lv[name] if name in Lv else cfg[name]))
    nboxes = (C.c_int * nlev)(*[len(Lv["boxes"]) for Lv in levels])
    boxes = np.ascontiguousarray(np.array([b for Lv in levels for b in Lv["boxes"]], dtype=np.int32).reshape(-1))
    dt, umax = C.c_double(0.0), C.c_double(0.0)
    L = lib()
    L.mo_est_dt.restype = C.c_int
    rc = L.mo_est_dt(C.byref(p), nlev, nboxes, boxes.ctypes.data_as(C.POINTER(C.c_int)), ins, C.c_double(cfl),
                     int(drdxfac), C.byref(dt), C.byref(umax))
    if rc != 0:
        raise RuntimeError("oracle: " + L.mo_last_error().decode())
    return dt.value, umax.value
