"""Stage parameters shared by the C ABI (``madv_params`` in include/maestro_adv.h).

The fields are the Maestro runtime parameters the scalar-advection stage reads
(Source/param/_cpp_parameters: ppm_type :396, slope_order :388, species_pred_type :376,
enthalpy_pred_type :368, ppm_trace_forces :405, base_cutoff_density :309,
buoyancy_cutoff_factor :328, do_eos_h_above_cutoff :359) plus the geometry and the
time-step state (``dt``, ``rel_eps`` from Source/MaestroDt.cpp:481-483) that the
reference keeps as ``Maestro`` members.
"""
import ctypes as C

# AMReX PhysBCType values, as used in Maestro inputs files (lo_bc / hi_bc).
INTERIOR, INFLOW, OUTFLOW, SYMMETRY, SLIPWALL, NOSLIPWALL = 0, 1, 2, 3, 4, 5

# Reference state component indices (Source/param/_variables:9-15).
RHO, RHOH, TEMP, PI, FIRSTSPEC = 0, 1, 2, 3, 4


class MadvParams(C.Structure):
    _fields_ = [
        ("nspec", C.c_int),
        ("ppm_type", C.c_int),
        ("slope_order", C.c_int),
        ("species_pred_type", C.c_int),
        ("enthalpy_pred_type", C.c_int),
        ("ppm_trace_forces", C.c_int),
        ("evolve_base_state", C.c_int),
        ("use_exact_base_state", C.c_int),
        ("phys_bc_lo", C.c_int * 3),
        ("phys_bc_hi", C.c_int * 3),
        ("dom_lo", C.c_int * 3),
        ("dom_hi", C.c_int * 3),
        ("dx", C.c_double * 3),
        ("dt", C.c_double),
        ("rel_eps", C.c_double),
        ("base_cutoff_density", C.c_double),
        ("buoyancy_cutoff_factor", C.c_double),
        ("do_eos_h_above_cutoff", C.c_int),
        ("base_cutoff_density_coord", C.c_int),
        ("dim", C.c_int),
        ("spherical", C.c_int),
        ("prob_lo", C.c_double * 3),
        ("prob_hi", C.c_double * 3),
        ("reflux_type", C.c_int),
        ("drdxfac", C.c_int),
        ("w0_interp_type", C.c_int),
        ("w0mac_interp_type", C.c_int),
        ("s0_interp_type", C.c_int),
        ("s0mac_interp_type", C.c_int),
    ]


def make_params(cfg):
    """Build a MadvParams from a config dict (see configs.py)."""
    p = MadvParams()
    p.nspec = cfg["nspec"]
    p.ppm_type = cfg["ppm_type"]
    p.slope_order = cfg.get("slope_order", 4)
    p.species_pred_type = cfg.get("species_pred_type", 1)
    p.enthalpy_pred_type = cfg.get("enthalpy_pred_type", 1)
    p.ppm_trace_forces = cfg.get("ppm_trace_forces", 0)
    p.evolve_base_state = cfg.get("evolve_base_state", 1)
    p.use_exact_base_state = cfg.get("use_exact_base_state", 0)
    for d in range(3):
        p.phys_bc_lo[d] = cfg["bc_lo"][d]
        p.phys_bc_hi[d] = cfg["bc_hi"][d]
        p.dom_lo[d] = 0
        p.dom_hi[d] = cfg["n"][d] - 1
        p.dx[d] = cfg["dx"][d]
    p.dt = cfg["dt"]
    p.rel_eps = cfg["rel_eps"]
    p.base_cutoff_density = cfg["base_cutoff_density"]
    p.buoyancy_cutoff_factor = cfg.get("buoyancy_cutoff_factor", 5.0)
    p.do_eos_h_above_cutoff = cfg.get("do_eos_h_above_cutoff", 1)
    p.dim = cfg.get("dim", 3)
    p.base_cutoff_density_coord = cfg["n"][p.dim - 1]
    p.spherical = cfg.get("spherical", 0)
    lo = cfg.get("prob_lo", (0.0, 0.0, 0.0))
    for d in range(3):
        p.prob_lo[d] = lo[d]
        p.prob_hi[d] = cfg.get("prob_hi", tuple(lo[e] + cfg["n"][e] * cfg["dx"][e] for e in range(3)))[d]
    if p.spherical:
        p.base_cutoff_density_coord = cfg["nr"]
    p.reflux_type = cfg.get("reflux_type", 1)
    # spherical radial interpolation (Source/param/_cpp_parameters: drdxfac :116,
    # s0_interp_type :527, w0_interp_type :533, s0mac_interp_type :539, w0mac_interp_type :546)
    p.drdxfac = cfg.get("drdxfac", 1)
    p.w0_interp_type = cfg.get("w0_interp_type", 2)
    p.w0mac_interp_type = cfg.get("w0mac_interp_type", 1)
    p.s0_interp_type = cfg.get("s0_interp_type", 3)
    p.s0mac_interp_type = cfg.get("s0mac_interp_type", 1)
    return p
