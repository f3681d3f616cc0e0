"""Host-side mirror of the Maestro member functions of the scalar-advection stage.

``ScalarAdvectionStage`` plays the role the ``Maestro`` object plays for these functions
in the reference (Source/Maestro.H): it owns the stage state (parameters, box layout,
1-D base state) and exposes AdvancePremac, Addw0, DensityAdvance, EnthalpyAdvance and the
whole stage with the reference's argument meaning, over ``MultiFab`` objects whose FABs
live in device memory.  All compute goes through the C ABI of libmaestro_adv.so.
"""
import ctypes as C

import numpy as np
import torch

from . import capi
from .capi import MadvBaseState, MadvBox, MadvFab, MadvMultiFab, check, lib


class MultiFab:
    """Per-box FABs (torch float64, Fortran order, ghost cells included) on one device.

    ``nodal`` = -1 for cell data, d for faces normal to direction d.
    """

    ALIGN = 32  # doubles: every FAB starts on a 256-byte boundary

    def __init__(self, boxes, ncomp, ngrow, nodal=-1, device="cuda", fill=0.0):
        self.boxes = [tuple(int(v) for v in b) for b in boxes]
        self.ncomp, self.ng, self.nodal = ncomp, ngrow, nodal
        self.fabs, self.los, self.his = [], [], []
        shapes, offs, tot = [], [], 0
        for b in self.boxes:
            lo = [b[0] - ngrow, b[1] - ngrow, b[2] - ngrow]
            hi = [b[3] + ngrow, b[4] + ngrow, b[5] + ngrow]
            if nodal >= 0:
                hi[nodal] += 1
            shape = (ncomp, hi[2] - lo[2] + 1, hi[1] - lo[1] + 1, hi[0] - lo[0] + 1)
            shapes.append(shape)
            offs.append(tot)
            tot += -(-int(np.prod(shape)) // self.ALIGN) * self.ALIGN
            self.los.append(lo)
            self.his.append(hi)
        # one allocation for the whole MultiFab (thousands of per-box allocations would each
        # round up in the caching allocator), FABs as views into it
        self.data = torch.full((max(tot, 1),), fill, dtype=torch.float64, device=device)
        for shape, o in zip(shapes, offs):
            self.fabs.append(self.data[o:o + int(np.prod(shape))].view(shape))
        self._desc = None

    def desc(self):
        if self._desc is None:
            arr = (MadvFab * len(self.fabs))()
            for b, t in enumerate(self.fabs):
                arr[b].p = t.data_ptr()
                for d in range(3):
                    arr[b].lo[d] = self.los[b][d]
                    arr[b].hi[d] = self.his[b][d]
                arr[b].ncomp = self.ncomp
            mf = MadvMultiFab(len(self.fabs), arr)
            self._desc = (mf, arr)
        return self._desc[0]

    def _slices(self, b, grow=0):
        bx = self.boxes[b]
        lo, hi = list(bx[:3]), list(bx[3:])
        if self.nodal >= 0:
            hi[self.nodal] += 1
        fs, ds = [], []
        for d in (2, 1, 0):
            a, z = lo[d] - grow, hi[d] + grow
            fs.append(slice(a - self.los[b][d], z - self.los[b][d] + 1))
            ds.append(slice(a, z + 1))
        return tuple(fs), tuple(ds)

    def from_domain(self, arr, c0=0):
        """Copy a domain-sized array [nc, nz(+1), ny(+1), nx(+1)] into the valid regions."""
        t = arr if torch.is_tensor(arr) else torch.from_numpy(np.ascontiguousarray(arr))
        nc = t.shape[0]
        for b, f in enumerate(self.fabs):  # box by box: no domain-sized copy on the device
            fs, ds = self._slices(b)
            f[(slice(c0, c0 + nc),) + fs] = t[(slice(None),) + ds].to(f.device)
        return self

    def to_domain(self, domain_n, comps=None):
        """Gather the valid regions into a domain-sized tensor."""
        comps = list(range(self.ncomp)) if comps is None else list(comps)
        n = list(domain_n)
        if self.nodal >= 0:
            n[self.nodal] += 1
        out = torch.full((len(comps), n[2], n[1], n[0]), float("nan"), dtype=torch.float64,
                         device=self.fabs[0].device)
        for b, f in enumerate(self.fabs):
            fs, ds = self._slices(b)
            out[(slice(None),) + ds] = f[(comps,) + fs]
        return out


def fab_of_tensor(t, lo):
    """madv_fab over a contiguous float64 device tensor [nc, nz, ny, nx] starting at cell lo."""
    assert t.is_contiguous() and t.dtype == torch.float64
    f = MadvFab()
    f.p = t.data_ptr()
    for d in range(3):
        f.lo[d] = int(lo[d])
        f.hi[d] = int(lo[d]) + t.shape[3 - d] - 1
    f.ncomp = t.shape[0]
    return f


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ref(mf):
    return C.byref(mf.desc()) if mf is not None else None


def _ref3(mfs):
    """Three face MultiFabs as a contiguous madv_multifab[3]."""
    if mfs is None:
        return None
    arr = (MadvMultiFab * 3)(*[m.desc() for m in mfs][:3])
    _ref3.keep.append(arr)
    if len(_ref3.keep) > 64:
        del _ref3.keep[:32]
    return C.cast(arr, C.POINTER(MadvMultiFab))


_ref3.keep = []


class ScalarAdvectionStage:
    def __init__(self, params):
        self.params = params
        self.ctx = C.c_void_p()
        check(lib().madv_ctx_create(C.byref(params), C.byref(self.ctx)))
        self.nscal = 4 + params.nspec

    def close(self):
        if self.ctx:
            lib().madv_ctx_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_layout(self, boxes):
        arr = (MadvBox * len(boxes))()
        for b, bx in enumerate(boxes):
            for d in range(3):
                arr[b].lo[d] = int(bx[d])
                arr[b].hi[d] = int(bx[3 + d])
        self.boxes = [tuple(b) for b in boxes]
        check(lib().madv_set_layout(self.ctx, len(boxes), arr))

    def set_base_state(self, rho0_old, rho0_new, rhoh0_old, rhoh0_new, p0_old, p0_new, psi, grav_cell,
                       w0_force, w0, rho0_predicted_edge):
        keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (
            rho0_old, rho0_new, rhoh0_old, rhoh0_new, p0_old, p0_new, psi, grav_cell, w0_force, w0,
            rho0_predicted_edge)]
        bs = MadvBaseState(*[_dptr(a) for a in keep])
        check(lib().madv_set_base_state(self.ctx, C.byref(bs)))

    def set_layout_levels(self, level_boxes):
        """grids[lev] of an AMR hierarchy (level-l index space, refinement ratio 2)."""
        allb = [b for boxes in level_boxes for b in boxes]
        arr = (MadvBox * len(allb))()
        for b, bx in enumerate(allb):
            for d in range(3):
                arr[b].lo[d] = int(bx[d])
                arr[b].hi[d] = int(bx[3 + d])
        nb = (C.c_int * len(level_boxes))(*[len(b) for b in level_boxes])
        self.level_boxes = [[tuple(b) for b in boxes] for boxes in level_boxes]
        check(lib().madv_set_layout_levels(self.ctx, len(level_boxes), nb, arr))

    def set_base_state_levels(self, levels):
        """levels[l]: dict with level l's 1-D arrays (rho0_old ... rho0_predicted_edge)."""
        names = ("rho0_old", "rho0_new", "rhoh0_old", "rhoh0_new", "p0_old", "p0_new", "psi", "grav_cell",
                 "w0_force", "w0", "rho0_predicted_edge")
        self._bs_keep = [[np.ascontiguousarray(L[n], dtype=np.float64) for n in names] for L in levels]
        arr = (MadvBaseState * len(levels))()
        for l, keep in enumerate(self._bs_keep):
            arr[l] = MadvBaseState(*[_dptr(a) for a in keep])
        check(lib().madv_set_base_state_levels(self.ctx, len(levels), arr))

    def stage_forward_levels(self, bufs, mode=capi.MODE_BATCHED, stream=None):
        """The stage on all levels; bufs[l] holds level l's MultiFabs (StageBuffers).  Buffers
        without edge states and fluxes (StageBuffers(edges=False)) ask for neither: the library
        then streams the species through slots of its own."""
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        nl = len(bufs)

        def cells(name):
            return (MadvMultiFab * nl)(*[getattr(b, name).desc() for b in bufs])

        def faces(name):
            if getattr(bufs[0], name) is None:
                return None
            return (MadvMultiFab * (3 * nl))(*[getattr(b, name)[d].desc() for b in bufs for d in range(3)])

        args = [cells("uold"), cells("sold"), cells("gpi"), cells("thermal"), cells("snew"), faces("umac"),
                faces("sedge"), faces("sflux"), cells("eta")]
        self._fwd_keep = args
        P = C.POINTER(MadvMultiFab)
        check(lib().madv_stage_forward_levels(self.ctx, mode, nl, *[C.cast(a, P) for a in args], C.c_void_p(s)))

    def set_dt(self, dt, rel_eps):
        check(lib().madv_set_dt(self.ctx, dt, rel_eps))

    def stage_forward(self, uold, sold, gpi, snew, umac, sedge=None, sflux=None, etarhoflux=None,
                      thermal=None, mode=capi.MODE_BATCHED, stream=None):
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(lib().madv_stage_forward(self.ctx, mode, _ref(uold), _ref(sold), _ref(gpi), _ref(thermal),
                                       _ref(snew), _ref3(umac), _ref3(sedge), _ref3(sflux),
                                       _ref(etarhoflux), C.c_void_p(s)))

    def advance_premac(self, uold, sold, gpi, umac, utrans=None, stream=None):
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(lib().madv_advance_premac(self.ctx, _ref(uold), _ref(sold), _ref(gpi), _ref3(umac),
                                        _ref3(utrans), C.c_void_p(s)))

    def addw0(self, umac, mult, stream=None):
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(lib().madv_addw0(self.ctx, _ref3(umac), float(mult), C.c_void_p(s)))

    def density_advance(self, sold, snew, sedge, sflux, etarhoflux, umac, which_step=1, stream=None):
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(lib().madv_density_advance(self.ctx, which_step, _ref(sold), _ref(snew), _ref3(sedge),
                                         _ref3(sflux), _ref(etarhoflux), _ref3(umac), C.c_void_p(s)))

    def enthalpy_advance(self, sold, snew, sedge, sflux, umac, thermal=None, which_step=1, stream=None):
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(lib().madv_enthalpy_advance(self.ctx, which_step, _ref(sold), _ref(snew), _ref3(sedge),
                                          _ref3(sflux), _ref3(umac), _ref(thermal), C.c_void_p(s)))

    # the member functions inside AdvancePremac / DensityAdvance / EnthalpyAdvance (3-D, one level)
    def make_utrans(self, utilde, ufull, utrans, stream=None):
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(lib().madv_make_utrans(self.ctx, _ref(utilde), _ref(ufull), _ref3(utrans), C.c_void_p(s)))

    def vel_pred(self, utilde, ufull, utrans, umac, force, stream=None):
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(lib().madv_vel_pred(self.ctx, _ref(utilde), _ref(ufull), _ref3(utrans), _ref3(umac), _ref(force),
                                  C.c_void_p(s)))

    def make_edge_scal(self, state, sedge, umac, force, is_vel, start_scomp, start_bccomp, num_comp,
                       is_conservative, stream=None):
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(lib().madv_make_edge_scal(self.ctx, _ref(state), _ref3(sedge), _ref3(umac), _ref(force), int(is_vel),
                                        start_scomp, start_bccomp, num_comp, int(is_conservative), C.c_void_p(s)))

    def make_rhox_flux(self, which_step, sflux, etarhoflux, sedge, umac, start_comp, num_comp, stream=None):
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(lib().madv_make_rhox_flux(self.ctx, which_step, _ref3(sflux), _ref(etarhoflux), _ref3(sedge),
                                        _ref3(umac), start_comp, num_comp, C.c_void_p(s)))

    def make_rhoh_flux(self, which_step, sflux, sedge, umac, stream=None):
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(lib().madv_make_rhoh_flux(self.ctx, which_step, _ref3(sflux), _ref3(sedge), _ref3(umac),
                                        C.c_void_p(s)))

    def update_scal(self, stateold, statenew, sflux, force, start_comp, num_comp, stream=None):
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(lib().madv_update_scal(self.ctx, _ref(stateold), _ref(statenew), _ref3(sflux), _ref(force),
                                     start_comp, num_comp, C.c_void_p(s)))

    def mac_project(self, umac, macrhs, rho, beta0, macphi=None, tol_rel=1.0e-10, max_iter=100, stream=None):
        """Maestro::MacProj (one level, plane-parallel or spherical): umac (3 face MultiFabs,
        >= 1 ghost) projected in place so that div(beta0 umac) = macrhs; returns (V-cycles,
        final max|residual| / max|rhs|).  rho, macrhs: cell MultiFabs; beta0: 1-D cell array
        (spherical: on the radial bins)."""
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        b0 = np.ascontiguousarray(beta0, dtype=np.float64)
        res = capi.MadvMacResult()
        check(lib().madv_mac_project(self.ctx, _ref3(umac), _ref(macphi), _ref(macrhs), _ref(rho), _dptr(b0),
                                     float(tol_rel), int(max_iter), C.byref(res), C.c_void_p(s)))
        return res.iterations, res.resid_ratio

    def mac_project_levels(self, umac, macrhs, rho, beta0, macphi=None, tol_rel=1.0e-10, max_iter=200, stream=None):
        """Maestro::MacProj on the layout's levels (two plane-parallel levels: the composite
        solve): umac[l] (3 face MultiFabs per level, >= 1 ghost) projected in place; macrhs[l],
        rho[l], macphi[l] per level; beta0[l] the level's radial rows.  Returns (iterations,
        final max|residual| / max|rhs|)."""
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        nl = len(macrhs)
        b0 = np.ascontiguousarray(np.concatenate([np.asarray(b, dtype=np.float64) for b in beta0]))
        faces = (capi.MadvMultiFab * (3 * nl))(*[umac[l][d].desc() for l in range(nl) for d in range(3)])
        cells = [(capi.MadvMultiFab * nl)(*[m[l].desc() for l in range(nl)]) for m in (macrhs, rho)]
        phi = None if macphi is None else (capi.MadvMultiFab * nl)(*[macphi[l].desc() for l in range(nl)])
        res = capi.MadvMacResult()
        P = C.POINTER(capi.MadvMultiFab)
        check(lib().madv_mac_project_levels(self.ctx, nl, C.cast(faces, P), None if phi is None else C.cast(phi, P),
                                            C.cast(cells[0], P), C.cast(cells[1], P), _dptr(b0), float(tol_rel),
                                            int(max_iter), C.byref(res), C.c_void_p(s)))
        return res.iterations, res.resid_ratio

    def est_dt(self, uold, sold, gpi, cfl=0.5, drdxfac=1, max_dt=1.0e33, fixed_dt=-1.0, small_dt=1.0e-10,
               stream=None):
        """Maestro::EstDt (advective and force constraints): returns (dt, dt_estimate, umax,
        rel_eps).  uold / sold / gpi: one MultiFab, or a list with one per level."""
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        lv = [uold, sold, gpi]
        if not isinstance(uold, (list, tuple)):
            lv = [[uold], [sold], [gpi]]
        nl = len(lv[0])
        arrs = [(capi.MadvMultiFab * nl)(*[m.desc() for m in mfs]) for mfs in lv]
        prm = capi.MadvDtParams(cfl, drdxfac, max_dt, fixed_dt, small_dt)
        res = capi.MadvDtResult()
        check(lib().madv_est_dt(self.ctx, nl, arrs[0], arrs[1], arrs[2], C.byref(prm), C.byref(res), C.c_void_p(s)))
        return res.dt, res.dt_estimate, res.umax, res.rel_eps

    def velocity_advance(self, uold, sold, rhohalf, gpi, umac, unew, uedge=None, sponge=None, stream=None):
        """Maestro::VelocityAdvance + UpdateVel (3-D, one level): unew (and the velocity edge
        states uedge) from uold, the projected MAC velocity umac (without w0) and rhohalf."""
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(lib().madv_velocity_advance(self.ctx, _ref(uold), _ref(sold), _ref(rhohalf), _ref(gpi), _ref3(umac),
                                          _ref(sponge), _ref(unew), _ref3(uedge), C.c_void_p(s)))

    def launch_count(self):
        return lib().madv_last_launch_count(self.ctx)

    def set_option(self, key, value):
        """madv_set_option: an implementation option (staged PPM sweeps, their tile shape)."""
        check(lib().madv_set_option(self.ctx, key.encode(), int(value)))

    def autotune(self, run_batched, candidates=(32, 64, 128, 256, 512), ppm_forms=range(5)):
        """Launch-shape autotuner (madv_autotune_*): run_batched() runs the caller's stage once
        in MODE_BATCHED; it is timed per kernel for every candidate block size, and the fastest
        per (level, kernel) is applied; then per level the fastest PPM form (three launches or
        the staged sweep with one of its tile shapes) among ppm_forms.  Returns the chosen
        table (dict)."""
        import json
        for t in candidates:
            check(lib().madv_autotune_trial(self.ctx, int(t)))
            run_batched()
        for f in ppm_forms:
            check(lib().madv_autotune_ppm_trial(self.ctx, int(f)))
            run_batched()
        buf = C.create_string_buffer(1 << 20)
        check(lib().madv_autotune_finish(self.ctx, buf, len(buf)))
        return json.loads(buf.value.decode())

    def autotune_apply(self, table):
        import json
        check(lib().madv_autotune_apply(self.ctx, json.dumps(table).encode()))

    def stage_adjoint(self, uold, sold0, weight, nsteps, ckpt_interval, grad_s=None, sfinal=None, grad_u=None,
                      stream=None):
        """madv_stage_adjoint: nsteps fixed-velocity steps from sold0, J = <weight, s_nsteps>,
        dJ/dsold0 into grad_s, dJ/duold into grad_u (both None: forward only) and s_nsteps
        into sfinal.  Returns (J, device bytes the call allocated)."""
        P = C.POINTER(capi.MadvMultiFab)
        seed = capi.MadvAdjSeed(int(nsteps), int(ckpt_interval), C.pointer(uold.desc()), C.pointer(sold0.desc()),
                                C.pointer(weight.desc()))
        res = capi.MadvAdjResult()
        res.sfinal = C.pointer(sfinal.desc()) if sfinal is not None else P()
        res.grad_s = C.pointer(grad_s.desc()) if grad_s is not None else P()
        res.grad_u = C.pointer(grad_u.desc()) if grad_u is not None else P()
        s = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(lib().madv_stage_adjoint(self.ctx, C.byref(seed), C.byref(res), C.c_void_p(s)))
        return res.J, res.device_bytes

    def ppm(self, bx, s, s_lo, comp, vel, vel_lo, is_umac, bc, Ip, Im, stream=None):
        """Maestro::PPM on one box through madv_ppm.  s, vel[d], Ip, Im: torch tensors
        [nc, nz, ny, nx] on the device whose first cell is s_lo / vel_lo[d] / bx lo."""
        fabs = [fab_of_tensor(s, s_lo)] + [fab_of_tensor(vel[d], vel_lo[d]) for d in range(3)] + \
               [fab_of_tensor(Ip, bx[:3]), fab_of_tensor(Im, bx[:3])]
        box = MadvBox()
        for d in range(3):
            box.lo[d], box.hi[d] = int(bx[d]), int(bx[3 + d])
        bcs = (C.c_int * 6)(*bc)
        st = stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream
        check(lib().madv_ppm(self.ctx, C.byref(box), C.byref(fabs[0]), comp, C.byref(fabs[1]), C.byref(fabs[2]),
                             C.byref(fabs[3]), int(is_umac), bcs, C.byref(fabs[4]), C.byref(fabs[5]),
                             C.c_void_p(st)))


class StageBuffers:
    """The caller-side MultiFabs of one stage configuration (as AdvanceTimeStep owns them).
    edges=False: no edge-state and flux MultiFabs (a caller that needs neither after the stage)."""

    def __init__(self, cfg, device="cuda", edges=True):
        boxes = cfg["boxes"]
        nscal = 4 + cfg["nspec"]
        ng = 4 if cfg["ppm_type"] == 2 else 3
        nd = cfg.get("dim", 3)
        self.n = cfg["n"]
        self.nd = nd
        self.uold = MultiFab(boxes, nd, ng, device=device)
        self.sold = MultiFab(boxes, nscal, ng, device=device)
        self.gpi = MultiFab(boxes, nd, 0, device=device)
        self.thermal = MultiFab(boxes, 1, 1, device=device)
        self.snew = MultiFab(boxes, nscal, ng, device=device)
        self.umac = [MultiFab(boxes, 1, 1, nodal=d, device=device) for d in range(nd)]
        self.sedge = [MultiFab(boxes, nscal, 0, nodal=d, device=device) for d in range(nd)] if edges else None
        self.sflux = [MultiFab(boxes, nscal, 0, nodal=d, device=device) for d in range(nd)] if edges else None
        self.eta = MultiFab(boxes, 1, 0, nodal=nd - 1, device=device)

    def load(self, cfg):
        self.uold.from_domain(cfg["uold"])
        self.sold.from_domain(cfg["sold"])
        self.gpi.from_domain(cfg["gpi"])
        self.thermal.from_domain(cfg["thermal"])
        return self


def make_stage(cfg):
    from .params import make_params
    st = ScalarAdvectionStage(make_params(cfg))
    st.set_layout(cfg["boxes"])
    st.set_base_state(cfg["rho0_old"], cfg["rho0_new"], cfg["rhoh0_old"], cfg["rhoh0_new"],
                      cfg["p0_old"], cfg["p0_new"], cfg["psi"], cfg["grav_cell"], cfg["w0_force"],
                      cfg["w0"], cfg["rho0_predicted_edge"])
    return st


def run_stage_gpu(cfg, mode=capi.MODE_BATCHED, device="cuda", edges=True):
    """Run the whole stage on the GPU for a config dict; returns domain arrays (numpy).
    edges=False: no edge states or fluxes asked for (3-D: the species are streamed)."""
    st = make_stage(cfg)
    buf = StageBuffers(cfg, device, edges).load(cfg)
    st.stage_forward(buf.uold, buf.sold, buf.gpi, buf.snew, buf.umac, buf.sedge, buf.sflux, buf.eta,
                     thermal=buf.thermal, mode=mode)
    torch.cuda.synchronize()
    n = cfg["n"]
    nd = buf.nd
    res = dict(
        umac_end=[buf.umac[d].to_domain(n)[0].cpu().numpy() for d in range(nd)],
        snew=buf.snew.to_domain(n).cpu().numpy(),
        sold_end=buf.sold.to_domain(n).cpu().numpy(),
        etarhoflux=buf.eta.to_domain(n)[0].cpu().numpy(),
        launches=st.launch_count(),
    )
    if edges:
        res["sedge"] = [buf.sedge[d].to_domain(n).cpu().numpy() for d in range(nd)]
        res["sflux"] = [buf.sflux[d].to_domain(n).cpu().numpy() for d in range(nd)]
    st.close()
    return res


def make_amr_stage(cfg):
    """Context for a two-level configuration (configs.planar_amr_config)."""
    from .params import make_params
    st = ScalarAdvectionStage(make_params(cfg))
    st.set_layout_levels([L["boxes"] for L in cfg["levels"]])
    st.set_base_state_levels(cfg["levels"])
    return st


def amr_buffers(cfg, device="cuda", edges=True):
    """One StageBuffers per level, loaded with the level's input arrays.  A level marked
    "inject" has no arrays of its own: each of its cells takes the value of its parent cell
    on the level below (filled on the device box by box).  edges=False: no edge-state and
    flux MultiFabs."""
    out = []
    for lev, L in enumerate(cfg["levels"]):
        c = dict(cfg)
        c.update(L)
        if not L.get("inject"):
            out.append(StageBuffers(c, device, edges).load(c))
            continue
        buf = StageBuffers(c, device, edges)
        P = cfg["levels"][lev - 1]
        for name in ("uold", "sold", "gpi", "thermal"):
            src = torch.from_numpy(np.ascontiguousarray(P[name]))  # host: only parent blocks travel
            mf = getattr(buf, name)
            for b, bx in enumerate(mf.boxes):
                i0, j0, k0, i1, j1, k1 = bx
                blk = src[:, k0 // 2:(k1 + 1) // 2, j0 // 2:(j1 + 1) // 2, i0 // 2:(i1 + 1) // 2].to(device)
                blk = blk.repeat_interleave(2, dim=1).repeat_interleave(2, dim=2).repeat_interleave(2, dim=3)
                if name == "sold" and cfg.get("spherical"):
                    blk = _sph_rebin(blk, bx, c, P)
                fs, _ = mf._slices(b)
                mf.fabs[b][(slice(None),) + fs] = blk
            del src
        out.append(buf)
    return out


def _sph_rebin(blk, bx, fine, coarse):
    """Spherical injection: the injected density, species and enthalpy are rescaled by the
    ratio of the base state at the fine cell's centre to that at its parent's centre (the
    perturbation relative to the base state is what is injected).  The base state at a cell
    is its radial bin's value on the exact grid, and on uniform bins the Put1dArrayOnCart
    interpolation of s0_interp_type the state was laid on."""
    dev = blk.device
    L = fine["prob_hi"][0] - fine["prob_lo"][0]
    dxf = fine["dx"][0]
    exact = fine.get("use_exact_base_state", 1)
    drf = dxf / fine.get("drdxfac", 1)
    t = fine.get("s0_interp_type", 3)

    def radius2(lo, hi, dx, refine):
        ax = [(torch.arange(lo[d], hi[d] + 1, device=dev, dtype=torch.float64) // refine + 0.5) * dx -
              0.5 * L for d in range(3)]
        return ax[2][:, None, None] ** 2 + ax[1][None, :, None] ** 2 + ax[0][None, None, :] ** 2

    def on_cells(s0, r2):
        if exact:  # the exact grid's bin of the cell centre
            return s0[torch.floor(r2 / (2.0 * dxf * dxf) - 0.375 + 0.5).long()]
        nr = s0.numel()
        r = torch.sqrt(r2)
        index = (r / drf).long()
        if t == 1:
            return s0[torch.clamp(index, max=nr - 1)]
        rcc = (torch.arange(nr, device=dev, dtype=torch.float64) + 0.5) * drf
        if t == 2:  # linear between the two nearest bin centres, constant past the ends
            i = torch.clamp(torch.searchsorted(rcc, r) - 1, 0, nr - 2)
            x0, x1 = rcc[i], rcc[i + 1]
            w = torch.clamp((r - x0) / (x1 - x0), 0.0, 1.0)
            return s0[i] + w * (s0[i + 1] - s0[i])
        i = torch.clamp(index, 1, nr - 2)  # quadratic through three bins, clipped to their range
        x0, x1, x2 = rcc[i - 1], rcc[i], rcc[i + 1]
        y0, y1, y2 = s0[i - 1], s0[i], s0[i + 1]
        y = (y0 + (y1 - y0) / (x1 - x0) * (r - x0) +
             ((y2 - y1) / (x2 - x1) - (y1 - y0) / (x1 - x0)) / (x2 - x0) * (r - x0) * (r - x1))
        return torch.minimum(torch.maximum(y, torch.minimum(y0, torch.minimum(y1, y2))),
                             torch.maximum(y0, torch.maximum(y1, y2)))

    lo, hi = bx[:3], bx[3:]
    rf2 = radius2(lo, hi, dxf, 1)
    rc2 = radius2(lo, hi, 2.0 * dxf, 2)
    r0 = torch.from_numpy(np.ascontiguousarray(fine["rho0_old"])).to(dev)
    h0 = torch.from_numpy(np.ascontiguousarray(fine["rhoh0_old"])).to(dev)
    out = blk.clone()
    fr = on_cells(r0, rf2) / on_cells(r0, rc2)
    out[0] *= fr
    out[4:] *= fr[None]
    out[1] *= on_cells(h0, rf2) / on_cells(h0, rc2)
    return out


def run_amr_stage_gpu(cfg, mode=capi.MODE_BATCHED, device="cuda", edges=True):
    """The stage on every level of cfg["levels"]; returns one dict of domain arrays per level
    (edges=False: species streamed, no edge states or fluxes returned)."""
    st = make_amr_stage(cfg)
    bufs = amr_buffers(cfg, device, edges)
    st.stage_forward_levels(bufs, mode=mode)
    torch.cuda.synchronize()
    res = []
    for L, buf in zip(cfg["levels"], bufs):
        n = L["n"]
        r = dict(
            umac_end=[buf.umac[d].to_domain(n)[0].cpu().numpy() for d in range(3)],
            snew=buf.snew.to_domain(n).cpu().numpy(),
            sold_end=buf.sold.to_domain(n).cpu().numpy(),
            etarhoflux=buf.eta.to_domain(n)[0].cpu().numpy(),
        )
        if edges:
            r["sedge"] = [buf.sedge[d].to_domain(n).cpu().numpy() for d in range(3)]
            r["sflux"] = [buf.sflux[d].to_domain(n).cpu().numpy() for d in range(3)]
        res.append(r)
    res[0]["launches"] = st.launch_count()
    st.close()
    return res
