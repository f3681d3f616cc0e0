// Test infrastructure only: stand-in for the reference's generated maestro_params.H (made
// from Source/param/_cpp_parameters by its build), declaring the runtime parameters that
// the compiled stage sources read.  Defaults are the reference's; ref_entry.cpp defines
// them and sets them from the caller's parameters before each call.
#ifndef REFSHIM_MAESTRO_PARAMS_H
#define REFSHIM_MAESTRO_PARAMS_H

#include "AMReX_shim.H"

namespace maestro {
extern int reflux_type;
extern int maestro_verbose;
extern amrex::Real cfl;
extern amrex::Real init_shrink;
extern amrex::Real small_dt;
extern amrex::Real max_dt;
extern amrex::Real fixed_dt;
extern bool use_soundspeed_firstdt;
extern bool use_divu_firstdt;
extern bool spherical;
extern bool octant;
extern bool do_sponge;
extern amrex::Real anelastic_cutoff_density;
extern amrex::Real base_cutoff_density;
extern amrex::Real burning_cutoff_density_lo;
extern amrex::Real burning_cutoff_density_hi;
extern amrex::Real buoyancy_cutoff_factor;
extern bool evolve_base_state;
extern bool use_exact_base_state;
extern bool average_base_state;
extern bool do_eos_h_above_cutoff;
extern int enthalpy_pred_type;
extern int species_pred_type;
extern int slope_order;
extern int ppm_type;
extern int ppm_trace_forces;
extern bool use_centrifugal;
extern bool use_alt_energy_fix;
extern int s0_interp_type;
extern int w0_interp_type;
extern int s0mac_interp_type;
extern int w0mac_interp_type;
extern int drdxfac;
extern amrex::Real grav_const;
extern amrex::Real planar_invsq_mass;
extern bool do_planar_invsq_grav;
extern bool do_2d_planar_octant;
}  // namespace maestro

#endif
