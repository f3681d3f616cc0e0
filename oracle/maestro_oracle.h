/* Test infrastructure only: C entry points of the CPU oracle for the MAESTROeX
 * scalar-advection stage.  Loaded by tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py as the checker; the product library
 * never links or calls it.
 *
 * Parity status: pinned.  The oracle is a line-by-line restatement of the reference
 * functions, each citing its file:line, and is checked bit for bit against the reference's
 * own stage sources compiled against AMReX stand-ins (refshim/, ref_entry.cpp; entry points
 * ref_run_stage, ref_run_velocity_advance, ref_ppm, ref_slopes, ref_member with the
 * arguments of the mo_ functions below).
 *
 * All field arrays are single-level, domain-sized, Fortran ordered (i fastest), one
 * contiguous block per component.  Face arrays in direction d have extent n_d + 1 in d.
 */
#ifndef MAESTRO_ORACLE_H
#define MAESTRO_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Same field layout as madv_params in include/maestro_adv.h. */
typedef struct {
    int nspec;
    int ppm_type;           /* 0, 1, 2 */
    int slope_order;        /* 0, 2, 4 (ppm_type 0 only) */
    int species_pred_type;  /* 1 rho' & X, 2 rhoX, 3 rho & X */
    int enthalpy_pred_type; /* 0 rhoh, 1 rhoh' */
    int ppm_trace_forces;   /* must be 0 */
    int evolve_base_state;
    int use_exact_base_state;
    int phys_bc_lo[3];
    int phys_bc_hi[3];
    int dom_lo[3];
    int dom_hi[3];
    double dx[3];
    double dt;
    double rel_eps;
    double base_cutoff_density;
    double buoyancy_cutoff_factor;
    int do_eos_h_above_cutoff;
    int base_cutoff_density_coord;
    int dim; /* 3 (or 0) / 2 */
    int spherical;      /* spherical geometry with the exact (irregular) base state */
    double prob_lo[3];
    double prob_hi[3];
    int reflux_type; /* 1 (or 0): AverageDownFaces of the fluxes; 2: FluxRegister reflux */
    int drdxfac;           /* spherical, inexact base state (0 means 1) */
    int w0_interp_type;    /* 1, 2 (0 means 2), 3 */
    int w0mac_interp_type; /* 1 (0 means 1), 2, 3, 4 */
    int s0_interp_type;    /* 1, 2, 3 (0 means 3) */
    int s0mac_interp_type; /* 1 (0 means 1), 2, 3 */
} mo_params;

typedef struct {
    const double* uold;      /* [3][ncell] */
    const double* sold;      /* [nscal][ncell], nscal = 4 + nspec */
    const double* gpi;       /* [3][ncell] */
    const double* thermal;   /* [ncell] (may be NULL => 0) */
    const double* rho0_old;  /* [nr] */
    const double* rho0_new;
    const double* rhoh0_old;
    const double* rhoh0_new;
    const double* p0_old;
    const double* p0_new;
    const double* psi;
    const double* grav_cell;
    const double* w0_force;            /* [nr] */
    const double* w0;                  /* [nr+1] */
    const double* rho0_predicted_edge; /* [nr+1] */
} mo_inputs;

typedef struct {
    double* utrans[3];   /* after MakeUtrans (before w0 is added), valid faces */
    double* umac_vp[3];  /* VelPred output, valid faces */
    double* umac_end[3]; /* umac at the end of the stage (after the Addw0 sequence) */
    double* vel_force;   /* [3][ncell] */
    double* sedge[3];    /* [nscal][faces_d] */
    double* sflux[3];    /* [nscal][faces_d] */
    double* snew;        /* [nscal][ncell] */
    double* sold_end;    /* [nscal][ncell]: sold after the in-place conversions */
    double* etarhoflux;  /* [z faces] */
} mo_outputs;

/* Runs AdvancePremac -> Addw0 -> DensityAdvance(1) -> EnthalpyAdvance(1) as
 * AdvanceTimeStep does (MAC projection skipped).  boxes: nboxes*6 ints
 * (lo0 lo1 lo2 hi0 hi1 hi2).  Returns 0, or a negative code with mo_last_error() set. */
int mo_run_stage(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* in,
                 mo_outputs* out, int nthreads);

/* The stage on an AMR hierarchy of nlev levels (refinement ratio 2).  Level l has the
 * domain and cell size of level 0 refined 2^l times; nboxes[l] boxes of level l follow
 * those of level l-1 in `boxes` (level-l index space).  in[l] / out[l] hold level l's
 * domain-sized field arrays (only cells and faces of the level's boxes are read or
 * written) and its base state (nr_l = nr_0 * 2^l cells).  which_step 1 runs
 * DensityAdvance / EnthalpyAdvance as the predictor, 2 as the corrector.  nlev = 1,
 * which_step 1 is mo_run_stage. */
int mo_run_stage_levels(const mo_params* p, int nlev, const int* nboxes, const int* boxes,
                        const mo_inputs* in, mo_outputs* out, int which_step, int nthreads);

/* The 2-D stage (the reference's AMREX_SPACEDIM == 2 code, y radial) on one level:
 * domain arrays are [nc][ny][nx] with 2 velocity components, boxes give lo/hi in x and y
 * (z entries ignored), face arrays utrans/umac/sedge/sflux use indices 0 and 1 and
 * etarhoflux lives on y faces. */
int mo_run_stage_2d(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* in,
                    mo_outputs* out, int which_step, int nthreads);

/* A FAB: data covering the index box [lo, hi] (i fastest), nc components. */
typedef struct {
    double* p;
    int lo[3];
    int hi[3];
    int nc;
} mo_fab;

/* Maestro::PPM (Source/MaestroPPM.cpp:5-2262) over the cell box bx[6] (lo, hi) for
 * component comp of s, tracing velocity u/v/w (face FABs if is_umac, else cell FABs);
 * bc = {lo[3], hi[3]}; writes Ip/Im comps 0..2. */
int mo_ppm(const mo_params* p, const int* bx, const mo_fab* s, int comp, const mo_fab* u, const mo_fab* v,
           const mo_fab* w, int is_umac, const int* bc, const mo_fab* Ip, const mo_fab* Im);

/* Maestro::Slopex/y/z (Source/MaestroSlopes.cpp:6-600) in direction d over the cell box
 * bx[6] for components 0..ncomp-1 of s into slope, domain dom[6]; bcs[6 n + (0..5)] are
 * component n's BCTypes (lo[3], hi[3]). */
int mo_slopes(int slope_order, int d, const int* dom, const int* bx, const mo_fab* s, int ncomp, const int* bcs,
              const mo_fab* slope);

/* One Maestro member function of the stage on one 3-D level, on caller FABs that hold
 * ghost cells as the caller filled them: args[slot * nboxes + b] is box b's FAB of argument
 * `slot` (p = NULL for arguments the function does not take).  base gives the base state
 * (only the 1-D arrays are read); which_step 1 passes the old base state as "new" to the
 * fluxes, 2 the new one.  Outputs are written on the valid region grown by the ghost cells
 * the reference fills (utrans 1, statenew ng_s), where the caller's FAB has them. */
enum {
    MO_UTILDE, MO_UFULL, MO_UTRANS0, MO_UTRANS1, MO_UTRANS2, MO_UMAC0, MO_UMAC1, MO_UMAC2, MO_FORCE, MO_STATE,
    MO_SNEW, MO_SEDGE0, MO_SEDGE1, MO_SEDGE2, MO_SFLUX0, MO_SFLUX1, MO_SFLUX2, MO_ETA, MO_NSLOT
};
enum { MO_MAKE_UTRANS, MO_VEL_PRED, MO_MAKE_EDGE_SCAL, MO_MAKE_RHOX_FLUX, MO_MAKE_RHOH_FLUX, MO_UPDATE_SCAL,
       MO_MAKE_S0MAC };
/*   MO_MAKE_UTRANS    MakeUtrans(utilde, ufull, utrans)
 *   MO_VEL_PRED       VelPred(utilde, ufull, utrans, umac, force)
 *   MO_MAKE_EDGE_SCAL MakeEdgeScal(state, sedge, umac, force, bcs_s, start, start, num, is_conservative)
 *   MO_MAKE_RHOX_FLUX MakeRhoXFlux(sflux, etarhoflux (may be absent), sedge, umac, start, num)
 *   MO_MAKE_RHOH_FLUX MakeRhoHFlux(sflux, sedge, umac)
 *   MO_UPDATE_SCAL    UpdateScal(state, snew, sflux, force, start, num)
 *   MO_MAKE_S0MAC     MakeS0mac(rho0_old, umac): spherical, the base state's rho0_old on the
 *                     faces (one ghost face) */
int mo_member(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* base, int fn, int which_step,
              int start_comp, int num_comp, int is_conservative, const mo_fab* args);

/* Tangent build only (libmaestro_oracle_tl.so, compiled with MO_TANGENT): mo_run_stage with
 * the directional derivatives duold [3][ncell] and dsold [nscal][ncell] of its inputs;
 * dsnew [nscal][ncell] receives the derivative of snew along them (the tangent-linear model
 * of the stage, branches decided by the forward values; out receives the values, bitwise
 * those of mo_run_stage).  mo_ppm and mo_member are not in the tangent build. */
int mo_run_stage_tl(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* in, const double* duold,
                    const double* dsold, mo_outputs* out, double* dsnew, int nthreads);

/* AdvancePremac for the MAC velocity (MAC projection skipped; its ghost faces filled by
 * FillBoundary + FillUmacGhost as MacProj leaves them), then Maestro::VelocityAdvance
 * (Source/MaestroVelocityAdvance.cpp:5-82) with UpdateVel (Source/MaestroAdvection.cpp:
 * 299-526) on one 3-D level: uold gets its ghost cells by FillPatch with bcs_u.  rhohalf
 * [ncell] is the half-time density of the second MakeVelForce (with rho0_nph = (rho0_old +
 * rho0_new) / 2 and grav_cell); sponge [ncell] may be NULL (do_sponge = 0).  Writes unew
 * [3][ncell], uedge[d] [3][faces_d] (may be NULL) and the MAC velocity VelocityAdvance was
 * given, umac[d] (may be NULL). */
int mo_run_velocity_advance(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* in,
                            const double* rhohalf, const double* sponge, double* unew, double* const* uedge,
                            double* const* umac, int nthreads);

/* Maestro::EstDt (Source/MaestroDt.cpp:11-225, spherical :301-384) on an nlev hierarchy
 * laid out as for mo_run_stage_levels: the advective (|u|, with the cell-centred w0 on the
 * radial direction, and |w0|) and force (MakeVelForce with zero MAC velocity and w0_force)
 * constraints, cfl and drdxfac (spherical dr = finest dx / drdxfac) as the runtime
 * parameters.  dt: before max_dt / fixed_dt / small_dt; umax: rel_eps = 1e-8 umax.  The
 * divU and dS/dt constraints are not included. */
int mo_est_dt(const mo_params* p, int nlev, const int* nboxes, const int* boxes, const mo_inputs* in, double cfl,
              int drdxfac, double* dt, double* umax);

/* 1-D CelltoEdge (Source/MaestroCelltoEdge.cpp:5-55), single level. */
int mo_cell_to_edge(const double* s0_cell, int nr, double* s0_edge);

const char* mo_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
