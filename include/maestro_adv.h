/* maestro_adv.h -- C ABI of the GB300 scalar-advection stage for MAESTROeX.
 *
 * Drop-in boundary for the Maestro member functions of the scalar-advection stage
 * (declarations in Source/Maestro.H of the reference):
 *   AdvancePremac   Source/Maestro.H:189   (MakeUtrans :1172, MakeVelForce, Addw0, VelPred :1711)
 *   DensityAdvance  Source/Maestro.H:499   (MakeEdgeScal :913, MakeRhoXFlux :230, UpdateScal :306)
 *   EnthalpyAdvance Source/Maestro.H:566   (MakeEdgeScal, MakeRhoHFlux :270, UpdateScal)
 *   Addw0           Source/MaestroFill3dData.cpp:357
 *
 * A MultiFab is passed as a list of FABs (one per box, in BoxArray order), each a device
 * pointer to Fortran-ordered storage (i fastest, then j, k, component) covering the
 * FAB's index box, ghost cells included -- the layout of amrex::FArrayBox::dataPtr()
 * with box() and nComp().  The caller owns every buffer; the library never frees them.
 * Scratch memory is owned by the context.
 *
 * Every entry point returns MADV_OK (0) or a negative error code; none aborts.  All work
 * is ordered on the stream passed in (cudaStream_t as void*; NULL = legacy default
 * stream).  A context is single-stream and not thread-safe; separate contexts are
 * independent.
 */
#ifndef MAESTRO_ADV_H
#define MAESTRO_ADV_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
    MADV_OK = 0,
    MADV_ERR_PARAM = -1,       /* invalid or inconsistent parameter */
    MADV_ERR_LAYOUT = -2,      /* bad box list / FAB descriptor */
    MADV_ERR_UNSUPPORTED = -3, /* option the library does not implement */
    MADV_ERR_CUDA = -4,        /* CUDA runtime error (see madv_last_error) */
    MADV_ERR_STATE = -5,       /* call order (layout / base state not set) */
    MADV_ERR_EOS = -6,         /* a cell fell to base_cutoff_density: needs the EOS */
    MADV_ERR_NOCONV = -7       /* an iterative solve did not reach its tolerance */
};

/* AMReX PhysBCType values (Maestro inputs lo_bc / hi_bc). */
enum { MADV_INTERIOR = 0, MADV_INFLOW = 1, MADV_OUTFLOW = 2, MADV_SYMMETRY = 3,
       MADV_SLIPWALL = 4, MADV_NOSLIPWALL = 5 };

/* Stage parameters: the Maestro runtime parameters and member state the stage reads. */
typedef struct {
    int nspec;                  /* NumSpec; state has 4 + nspec components */
    int ppm_type;               /* 0 (slopes), 1, 2 */
    int slope_order;            /* 0, 2, 4 (ppm_type 0) */
    int species_pred_type;      /* 1 rho'&X, 2 rhoX, 3 rho&X */
    int enthalpy_pred_type;     /* 0 rhoh, 1 rhoh', 2 h (spherical with the exact base state: 1) */
    int ppm_trace_forces;       /* 0, or 1 (ppm_type 1/2, 3-D): forces traced by PPM */
    int evolve_base_state;
    int use_exact_base_state;   /* planar: 0; spherical: 1 the exact (irregular) radial grid,
                                   0 uniform radial bins of dx_fine / drdxfac */
    int phys_bc_lo[3];
    int phys_bc_hi[3];
    int dom_lo[3];              /* level-0 domain box */
    int dom_hi[3];
    double dx[3];
    double dt;
    double rel_eps;
    double base_cutoff_density;
    double buoyancy_cutoff_factor;
    int do_eos_h_above_cutoff;
    int base_cutoff_density_coord;
    int dim;                    /* 3 (0 means 3) or 2: the AMREX_SPACEDIM == 2 form, y radial,
                                   boxes and domain with z = [0, 0], 2 velocity components */
    int spherical;              /* 1: full-star spherical geometry (3-D, one or two levels):
                                   use_exact_base_state = 1: the irregular radial grid
                                   r_cc(i) = sqrt(0.75 + 2i) dx, nr = nr_irreg + 1; 0: r_cc(i) =
                                   (i + 1/2) dr, dr = dx / drdxfac, nr = int(max_dist / dr) + 1
                                   with max_dist the centre-to-corner distance; dx the finest */
    double prob_lo[3];          /* physical domain (the star's centre is its midpoint) */
    double prob_hi[3];
    int reflux_type;            /* coarse-fine flux synchronisation: 1 (or 0) AverageDownFaces
                                   of the fluxes, 2 FluxRegister reflux of the coarse state */
    int drdxfac;                /* spherical, inexact base state: radial bins per cell width
                                   (0 means 1) */
    int w0_interp_type;         /* spherical Put1dArrayOnCart of edge-centred w0: 1 constant,
                                   2 linear (default, 0 means 2), 3 quadratic */
    int w0mac_interp_type;      /* spherical MakeW0mac: 1 (default, 0 means 1) face average of
                                   w0_cart, 2 linear, 3 quadratic at the faces, 4 nodes then faces */
    int s0_interp_type;         /* spherical, inexact base state, Put1dArrayOnCart of cell-centred
                                   arrays: 1 constant, 2 linear, 3 quadratic (default, 0 means 3) */
    int s0mac_interp_type;      /* spherical MakeS0mac: 1 (default, 0 means 1) cell values averaged
                                   to faces; inexact base state also 2 linear, 3 quadratic */
} madv_params;

typedef struct {
    int lo[3];
    int hi[3];
} madv_box;

typedef struct {
    double* p;   /* device pointer to element (lo) of component 0 */
    int lo[3];   /* index box covered by the storage (ghosts / nodal extent included) */
    int hi[3];
    int ncomp;
} madv_fab;

typedef struct {
    int nfab;            /* must equal the number of boxes of the layout */
    const madv_fab* fab; /* host array of nfab descriptors */
} madv_multifab;

/* 1-D radial base state of one level (host arrays, nr = dom_hi[2]-dom_lo[2]+1), the
 * BaseState<Real> members the stage reads.  Copied into the context. */
typedef struct {
    const double* rho0_old;            /* [nr] */
    const double* rho0_new;            /* [nr] */
    const double* rhoh0_old;           /* [nr] */
    const double* rhoh0_new;           /* [nr] */
    const double* p0_old;              /* [nr] */
    const double* p0_new;              /* [nr] */
    const double* psi;                 /* [nr] */
    const double* grav_cell;           /* [nr] */
    const double* w0_force;            /* [nr] */
    const double* w0;                  /* [nr+1] edge centred */
    const double* rho0_predicted_edge; /* [nr+1] */
} madv_base_state;

typedef struct madv_ctx madv_ctx;

/* Context: parameters are copied; replaces the Maestro member state of the stage. */
int madv_ctx_create(const madv_params* params, madv_ctx** ctx);
void madv_ctx_destroy(madv_ctx* ctx);
/* New dt / rel_eps for the next step (Maestro::EstDt, Source/MaestroDt.cpp:481-483). */
int madv_set_dt(madv_ctx* ctx, double dt, double rel_eps);

/* One level: boxes in BoxArray order.  Allocates the context's scratch. */
int madv_set_layout(madv_ctx* ctx, int nboxes, const madv_box* boxes);
int madv_set_base_state(madv_ctx* ctx, const madv_base_state* bs);

/* An AMR hierarchy of nlev levels (1 or 2, refinement ratio 2), the grids[lev] BoxArrays
 * of the reference (Source/Maestro.H:1855-2025): nboxes[l] boxes of level l follow those
 * of level l-1 in `boxes`, in level-l index space.  Level 0 covers the domain; level-1
 * boxes are coarse-aligned (even lo, odd hi).  Replaces madv_set_layout. */
int madv_set_layout_levels(madv_ctx* ctx, int nlev, const int* nboxes, const madv_box* boxes);

/* Base state of every level, bs[l] holding level l's arrays (nr_l = nr_0 * 2^l cells),
 * i.e. the (lev, r) rows of the reference's BaseState arrays (Source/BaseState.H:14-130).
 * Edge states come from Maestro::CelltoEdge over each level's radial chunks followed by
 * RestrictBase (Source/MaestroCelltoEdge.cpp:5-58); with two levels the per-level
 * base_cutoff_density_coord follows BaseStateGeometry::ComputeCutoffCoords
 * (Source/BaseStateGeometry.cpp:112-210) applied to rho0_old.  Call after the layout. */
int madv_set_base_state_levels(madv_ctx* ctx, int nlev, const madv_base_state* bs);

/* Maestro::AdvancePremac (Source/MaestroAdvection.cpp:7-84), one level.
 * uold: 3 comps, sold: 4+nspec comps (only Rho is read), gpi: 3 comps (valid region read).
 * umac[3]: face MultiFabs with >= 1 ghost, written on the valid faces (VelPred output).
 * utrans[3] (may be NULL): receives the transverse velocities (with w0 added). */
int madv_advance_premac(madv_ctx* ctx, const madv_multifab* uold, const madv_multifab* sold,
                        const madv_multifab* gpi, const madv_multifab* umac,
                        const madv_multifab* utrans, void* stream);

/* Maestro::Addw0, planar (Source/MaestroFill3dData.cpp:357-462): wmac += mult*w0 and
 * refill of the face ghosts. */
int madv_addw0(madv_ctx* ctx, const madv_multifab* umac, double mult, void* stream);

/* Maestro::DensityAdvance (Source/MaestroDensityAdvance.cpp:6-243), which_step 1
 * (predictor) or 2 (corrector: old/new base-state averages in the fluxes).
 * sold is converted and restored in place exactly as the reference does; snew receives
 * rho and rhoX.  umac must hold the full velocity (w0 added), ghosts filled.
 * sedge/sflux (may be NULL) receive the edge states / fluxes; etarhoflux may be NULL. */
int madv_density_advance(madv_ctx* ctx, int which_step, const madv_multifab* sold,
                         const madv_multifab* snew, const madv_multifab* sedge,
                         const madv_multifab* sflux, const madv_multifab* etarhoflux,
                         const madv_multifab* umac, void* stream);

/* Maestro::EnthalpyAdvance (Source/MaestroEnthalpyAdvance.cpp:6-352), which_step 1 or 2
 * (2 averages the old and new base state in the fluxes and the final MakeRhoHForce).
 * thermal may be NULL (zero). */
int madv_enthalpy_advance(madv_ctx* ctx, int which_step, const madv_multifab* sold,
                          const madv_multifab* snew, const madv_multifab* sedge,
                          const madv_multifab* sflux, const madv_multifab* umac,
                          const madv_multifab* thermal, void* stream);

/* ---- The member functions inside AdvancePremac / DensityAdvance / EnthalpyAdvance, one
 * level, 3-D.  Inputs carry the ghost cells the reference's callers fill before the call
 * (ng_adv = ng_s = 3, or 4 for ppm_type 2); the implicit inputs (dt, rel_eps, BCs, w0 and the
 * base state) come from the context, as the reference reads them from Maestro members. */

/* Maestro::MakeUtrans (Source/Maestro.H:1172, Source/MaestroMakeUtrans.cpp:6-648).
 * utilde, ufull: 3 comps, ng_adv ghosts.  utrans[3]: written on the valid faces and, where
 * the FAB holds it, the ghost face layer the reference fills (FillBoundary + FillUmacGhost).
 * w0mac (spherical) is built from the context's w0. */
int madv_make_utrans(madv_ctx* ctx, const madv_multifab* utilde, const madv_multifab* ufull,
                     const madv_multifab* utrans, void* stream);

/* Maestro::VelPred (Source/Maestro.H:1711, Source/MaestroVelPred.cpp:5-292).
 * utilde, ufull: ng_adv ghosts; utrans[3]: 1 ghost (w0 already added, as AdvancePremac
 * passes it); force: 3 comps, 1 ghost.  umac[3] receives the valid faces. */
int madv_vel_pred(madv_ctx* ctx, const madv_multifab* utilde, const madv_multifab* ufull,
                  const madv_multifab* utrans, const madv_multifab* umac, const madv_multifab* force,
                  void* stream);

/* Maestro::MakeEdgeScal (Source/Maestro.H:913, Source/MaestroMakeEdgeScalars.cpp:6-302) for
 * scalars with bcs_s: is_vel must be 0 and start_bccomp == start_scomp (every scalar call of
 * the reference).  state: ng_s ghosts; umac[3]: full velocity, 1 ghost; force: 1 ghost.
 * sedge[3] receives components start_scomp .. start_scomp+num_comp-1 on the valid faces. */
int madv_make_edge_scal(madv_ctx* ctx, const madv_multifab* state, const madv_multifab* sedge,
                        const madv_multifab* umac, const madv_multifab* force, int is_vel,
                        int start_scomp, int start_bccomp, int num_comp, int is_conservative,
                        void* stream);

/* Maestro::MakeRhoXFlux (Source/Maestro.H:230, Source/MaestroMakeFlux.cpp:18-465) for the
 * species (start_comp = FirstSpec, num_comp = NumSpec, the reference's only call): sflux[3]
 * receives Rho and the species; etarhoflux (may be NULL) is accumulated into.  which_step 1
 * passes rho0_old as the new base state (DensityAdvance's predictor), 2 rho0_new. */
int madv_make_rhox_flux(madv_ctx* ctx, int which_step, const madv_multifab* sflux,
                        const madv_multifab* etarhoflux, const madv_multifab* sedge,
                        const madv_multifab* umac, int start_comp, int num_comp, void* stream);

/* Maestro::MakeRhoHFlux (Source/Maestro.H:270, Source/MaestroMakeFlux.cpp:467-1067): sflux[3]
 * receives RhoH; which_step as for madv_make_rhox_flux (rhoh0). */
int madv_make_rhoh_flux(madv_ctx* ctx, int which_step, const madv_multifab* sflux,
                        const madv_multifab* sedge, const madv_multifab* umac, void* stream);

/* Maestro::VelocityAdvance (Source/Maestro.H:1689, Source/MaestroVelocityAdvance.cpp:5-82) with
 * UpdateVel (Source/MaestroAdvection.cpp:299-526), one level, 3-D: the velocity edge states
 * (MakeEdgeScal with is_vel, bcs_u) from the MAC velocity plus w0, and unew = uold - dt
 * (Utilde.grad)Utilde + dt force - dt (w0.grad)Utilde, times the sponge.
 * uold: 3 comps, valid region read (its ghost cells are filled with bcs_u, as the previous
 * UpdateVel's FillPatch leaves them); sold: Rho of the first MakeVelForce (rho0_old);
 * rhohalf: 1 comp, the density of the second (rho0_nph = (rho0_old + rho0_new) / 2); the
 * gravity of both is the context's grav_cell.  gpi: 3 comps.  umac[3]: the projected MAC
 * velocity without w0, valid faces read (ghost faces filled as MacProj leaves them).
 * sponge: 1 comp or NULL (do_sponge = 0).  unew: 3 comps, written on the valid region and
 * the ghost cells of the closing FillPatch it holds; uedge[3] (may be NULL): the velocity
 * edge states, 3 comps on the valid faces. */
int madv_velocity_advance(madv_ctx* ctx, const madv_multifab* uold, const madv_multifab* sold,
                          const madv_multifab* rhohalf, const madv_multifab* gpi,
                          const madv_multifab* umac, const madv_multifab* sponge,
                          const madv_multifab* unew, const madv_multifab* uedge, void* stream);

/* Runtime parameters of EstDt (Source/param/_cpp_parameters: cfl, drdxfac, max_dt,
 * fixed_dt, small_dt). */
typedef struct {
    double cfl;      /* 0.5 by default */
    int drdxfac;     /* spherical radial spacing = finest dx / drdxfac (1 by default) */
    double max_dt;   /* 1e33 */
    double fixed_dt; /* -1: not fixed */
    double small_dt; /* 1e-10: a smaller estimate is an error, as the reference aborts */
} madv_dt_params;

typedef struct {
    double dt;          /* after the max_dt / fixed_dt limits */
    double dt_estimate; /* before them */
    double umax;        /* the largest speed; rel_eps = 1e-8 umax */
    double rel_eps;
} madv_dt_result;

/* Maestro::EstDt (Source/Maestro.H:530, Source/MaestroDt.cpp:11-225 planar, :301-384 spherical,
 * :440-483), 3-D, over nlev levels: dt = cfl min(dx / max|u_d|, dr / max|w0|) (the radial speed
 * with the cell-centred w0), limited by sqrt(2 dx / max|f_d|) with vel_force from
 * MakeVelForce at zero MAC velocity and w0_force; rel_eps = 1e-8 umax.  uold, gpi: ndim comps,
 * sold: Rho, valid regions read.  Bit for bit the reference's values.  The divU and dS/dt
 * constraints of EstDt (:226-300) need S_cc, dSdt and gamma1bar from the reactions / EOS
 * part of the step and are left to the caller (min with this dt). */
int madv_est_dt(madv_ctx* ctx, int nlev, const madv_multifab* uold, const madv_multifab* sold,
                const madv_multifab* gpi, const madv_dt_params* params, madv_dt_result* result,
                void* stream);

/* Maestro::UpdateScal (Source/Maestro.H:306, Source/MaestroAdvection.cpp:86-297) for RhoH
 * (start_comp 1, num_comp 1) or the species (FirstSpec, NumSpec; Rho follows).  stateold,
 * force: valid region; statenew: the updated components on the valid region and, where
 * the FAB holds them, the ng_s ghost cells of the closing FillPatch. */
int madv_update_scal(madv_ctx* ctx, const madv_multifab* stateold, const madv_multifab* statenew,
                     const madv_multifab* sflux, const madv_multifab* force, int start_comp,
                     int num_comp, void* stream);

/* The whole stage as Maestro::AdvanceTimeStep runs it with the MAC projection
 * skipped (Source/MaestroAdvance.cpp:359, 448-455, 541-548): AdvancePremac, Addw0(+1),
 * DensityAdvance, Addw0(-1), Addw0(+1), EnthalpyAdvance, Addw0(-1).
 * mode: MADV_MODE_BATCHED runs every kernel once over all boxes;
 *       MADV_MODE_PER_BOX launches every kernel once per box (the AMReX MFIter form);
 *       MADV_MODE_GRAPH replays a CUDA graph of the batched form (captured on first use
 *       for the given buffers).
 * sedge and sflux both NULL (3-D): the caller wants neither the edge states nor the fluxes
 * (the reference's AdvanceTimeStep reads neither after the stage: etarhoflux and the flux
 * registers carry what it needs).  The species are then streamed: each species' edge
 * states, fluxes and update pass through slots of three components (Rho, RhoH, the species
 * in flight), so the context holds 6 face-centred doubles per cell instead of 2 nscal.
 * The new state, the MAC velocities and etarhoflux are the full stage's bit for bit. */
enum { MADV_MODE_BATCHED = 0, MADV_MODE_PER_BOX = 1, MADV_MODE_GRAPH = 2 };
int madv_stage_forward(madv_ctx* ctx, int mode, const madv_multifab* uold,
                       const madv_multifab* sold, const madv_multifab* gpi,
                       const madv_multifab* thermal, const madv_multifab* snew,
                       const madv_multifab* umac, const madv_multifab* sedge,
                       const madv_multifab* sflux, const madv_multifab* etarhoflux,
                       void* stream);

/* madv_stage_forward on an AMR hierarchy: the reference's Vector<MultiFab> arguments,
 * uold[l], sold[l], gpi[l], thermal[l], snew[l], etarhoflux[l] for level l and
 * umac[3*l + d], sedge[3*l + d], sflux[3*l + d] for its faces (thermal, snew, umac, sedge,
 * sflux and etarhoflux may be NULL).  Between the per-level computations the levels are
 * coupled as the reference couples them: AverageDown + FillPatch (cell_cons_interp) after
 * each cell-centred update (Source/MaestroFillData.cpp:7-154), AverageDownFaces +
 * FillPatchUedge for the face velocities (:156-174, :455-835), AverageDownFaces of the
 * fluxes (reflux_type 1, Source/MaestroMakeFlux.cpp:460-462).  In MADV_MODE_BATCHED /
 * MADV_MODE_GRAPH each kernel covers all boxes of one level per launch. */
int madv_stage_forward_levels(madv_ctx* ctx, int mode, int nlev, const madv_multifab* uold,
                              const madv_multifab* sold, const madv_multifab* gpi,
                              const madv_multifab* thermal, const madv_multifab* snew,
                              const madv_multifab* umac, const madv_multifab* sedge,
                              const madv_multifab* sflux, const madv_multifab* etarhoflux,
                              void* stream);

/* Maestro::PPM (Source/Maestro.H:1396, Source/MaestroPPM.cpp:5-2262) on one box: for
 * component comp of s, the traced edge states Ip(.,d) and Im(.,d), d = 0..2, over the cell
 * box bx (the reference passes the box grown by one cell).  u, v, w: the tracing
 * velocity, face-centred (is_umac = 1: FABs covering the x-, y-, z-faces of bx) or
 * cell-centred (is_umac = 0).  bc = {lo[0..2], hi[0..2]}: the BCRec bcs[bccomp].
 * ppm_type (1 or 2), dt, rel_eps, dx and the domain box come from the context.  s must
 * cover bx grown by 2 (ppm_type 1) or 3 (ppm_type 2) cells; Ip and Im are 3-component
 * FABs covering bx.  Scratch comes from the context and is grown with cudaMalloc when a
 * larger box arrives. */
int madv_ppm(madv_ctx* ctx, const madv_box* bx, const madv_fab* s, int comp, const madv_fab* u,
             const madv_fab* v, const madv_fab* w, int is_umac, const int* bc, const madv_fab* Ip,
             const madv_fab* Im, void* stream);

/* madv_ppm without any device allocation, for callers that cannot call cudaMalloc where
 * they run PPM -- e.g. an AMReX application whose arena already holds most of the GPU's
 * memory, or code that must avoid the implicit device synchronisation of cudaMalloc and
 * cudaFree.  No counterpart in the reference.  Same arguments and results as madv_ppm,
 * with the parameters taken from `params` instead of a context.  Scratch is one static
 * device array of MADV_PPM_NOALLOC_MAX_DOUBLES doubles (9.04 MiB) that every GPU loading
 * the library holds until exit; a box needing more (larger than 66 x 66 x 66 cells) is
 * rejected with MADV_ERR_LAYOUT.  The first call on each device looks up the array's
 * device address (cudaGetSymbolAddress) and must come before any stream capture; the
 * address is cached for the process, so do not call this entry point on a device after
 * cudaDeviceReset.  All calls share the array: calls that overlap on the GPU race, so keep
 * them on one stream. */
#define MADV_PPM_NOALLOC_MAX_DOUBLES 1184832
int madv_ppm_noalloc(const madv_params* params, const madv_box* bx, const madv_fab* s, int comp,
                     const madv_fab* u, const madv_fab* v, const madv_fab* w, int is_umac,
                     const int* bc, const madv_fab* Ip, const madv_fab* Im, void* stream);

/* Adjoint of the scalar path over several advection steps with the velocity held fixed
 * (the multi-step form of Exec/unit_tests/test_advect/MaestroEvolve.cpp:140-190, which
 * re-runs AdvancePremac + DensityAdvance + EnthalpyAdvance on a fixed velocity):
 *     s_0 = sold0,  s_{n+1} = Stage(uold, s_n)  (n < nsteps),  J = sum weight * s_nsteps
 * over valid cells and all nscal components.  Stage is madv_stage_forward's computation
 * (snew's density, enthalpy and species; temperature and pi are carried), with gpi = 0
 * and thermal = 0.  The velocity is held fixed, so dJ/duold sums the MAC-velocity
 * adjoints of all steps through one transposed AdvancePremac (VelPred, MakeUtrans).
 * The reverse sweep transposes each phase with the forward's limiter
 * and upwind decisions frozen; states are stored every ckpt_interval steps and each
 * block is recomputed from its stored state, so memory grows with nsteps/ckpt_interval
 * + ckpt_interval states.  No counterpart in the reference.
 * Scope: one level, 3-D, plane-parallel or spherical, ppm_type 1 (or 2: state gradient, no
 * walls), species_pred_type 1, enthalpy_pred_type 1.  The state gradient (grad_s) also
 * allows outflow, symmetry and wall boundaries and w0 != 0, and gravity (grav_cell != 0:
 * the MAC velocity then depends on the density through MakeVelForce and VelPred, and each
 * reverse step carries its MAC-velocity adjoint back to the density) on periodic, outflow
 * and symmetry boundaries.  The velocity gradient (grad_u) needs a periodic domain,
 * w0 = 0 and grav_cell = 0.  Anything else returns MADV_ERR_UNSUPPORTED.  The UpdateScal
 * floor and negative-species branches are taken as not active. */
typedef struct {
    int nsteps;                  /* advection steps (>= 1) */
    int ckpt_interval;           /* steps between stored states (>= 1) */
    const madv_multifab* uold;   /* cell velocity, 3 components, held fixed */
    const madv_multifab* sold0;  /* initial state, nscal components */
    const madv_multifab* weight; /* J = sum(weight * s_nsteps), nscal components */
} madv_adj_seed;

typedef struct {
    const madv_multifab* sfinal; /* out (may be NULL): s_nsteps, nscal components */
    const madv_multifab* grad_s; /* out (may be NULL): dJ/dsold0, nscal components */
    const madv_multifab* grad_u; /* out (may be NULL): dJ/duold, 3 components; both NULL:
                                    forward only */
    double J;                    /* out */
    long long device_bytes;      /* out: device memory the call allocated (freed on return) */
} madv_adj_result;

int madv_stage_adjoint(madv_ctx* ctx, const madv_adj_seed* seed, madv_adj_result* res, void* stream);

/* Number of kernel launches issued by the last madv_* call (for launch accounting). */
long madv_last_launch_count(const madv_ctx* ctx);

/* Per-kernel timing, the counterpart of the reference's BL_PROFILE_VAR regions
 * (TinyProfiler): when enabled, CUDA events bracket every batched-mode launch.
 * madv_profile_report synchronises the device and writes a JSON object
 * {"kernel name": [launches, total_ms], ...} into buf. */
int madv_profile(madv_ctx* ctx, int enable);
int madv_profile_report(madv_ctx* ctx, char* buf, int len);

/* Launch-shape autotuner: the threads per block of every stage kernel, chosen per level (the
 * levels hold a hierarchy's box-size classes) from timed trials of the caller's own stage:
 *     for each candidate t:  madv_autotune_trial(ctx, t);  run the stage in MADV_MODE_BATCHED;
 *     madv_autotune_finish(ctx, json, len);
 * finish picks the fastest candidate per (level, kernel), applies it to later launches and
 * graphs, and writes the table {"L<level> <kernel symbol>": threads, ...} (a cache for
 * madv_autotune_apply in a later run).  Kernels are clamped to the block size they can take.
 * No counterpart in the reference. */
int madv_autotune_trial(madv_ctx* ctx, int threads);
/* The PPM form, tuned the same way per level: for each form f in [0, MADV_AUTOTUNE_PPM_FORMS):
 * madv_autotune_ppm_trial(ctx, f); run the stage.  Form 0 is the three-launch PPM (slopes,
 * interfaces, cell limiter); forms 1-4 the staged sweep kernel with tile shapes (across x;
 * across y and z) 4x2; 32x2, 8x2; 32x1, 2x2; 16x2 and 4x4; 16x4.  finish keeps the form
 * whose PPM kernels took the least time on each level ("L<level> ppm_form" in the table).
 * Results do not depend on the form. */
#define MADV_AUTOTUNE_PPM_FORMS 5
int madv_autotune_ppm_trial(madv_ctx* ctx, int form);
int madv_autotune_finish(madv_ctx* ctx, char* json, int len);
int madv_autotune_apply(madv_ctx* ctx, const char* json);

/* Implementation options of a context (no counterpart in the reference; results never
 * depend on them):
 *   "staged_ppm"      1: each PPM direction runs as one kernel over tiles of whole pencils
 *                     staged in shared memory by bulk copies; 0 (default): three launches
 *                     (slopes, interface values, cell limiter) through global memory, which
 *                     measure faster on GB300 (the stage is FP64-issue bound, and the fused
 *                     kernel's registers and shared memory cut its occupancy).
 *   "sweep_tile_Da", "sweep_tile_Db" (D = 0, 1, 2): cells of a staged tile across
 *                     direction D, in the first / second transverse direction (x before y
 *                     before z); defaults 4 x 2 for D = 0 and 32 x 2 for D = 1, 2.
 *   "component_streams" 1: in a stage call (3-D, not per box, not while madv_profile
 *                     times launches) the components of each MakeEdgeScal alternate between
 *                     the caller's stream and a second one, which works in its own copy of
 *                     the per-component scratch (allocated at first use: about 46 doubles per
 *                     cell); 0 (default): one stream -- the stage is FP64-issue bound and
 *                     the overlap measures 0.5% on GB300.
 *   "es_inline"       1 (default): with ppm_type 1 / 2, MakeEdgeScal's transverse and edge
 *                     kernels take the predictor's left / right states straight from the
 *                     traced Ip / Im, and only the upwind state is stored per face; 0: the
 *                     predictor stores all three (as the reference's slx / srx / simhx).
 *   "mg_block_cycle"  1 (default): the MAC projection's multigrid V-cycle, from its first
 *                     grid of at most 4096 cells down to the coarsest, runs in one thread
 *                     block with the same per-cell arithmetic (bitwise the same result);
 *                     0: one launch per smoothing sweep, residual, restriction and
 *                     prolongation on those grids too.
 * Returns MADV_ERR_PARAM for an unknown key or a value outside 1..256. */
int madv_set_option(madv_ctx* ctx, const char* key, int value);

/* FP64 FMA issue-rate probe of the current device (TFLOP/s, 2 flops per FMA): the
 * ceiling of the FP64-bound stage kernels.  No counterpart in the reference. */
int madv_probe_fp64_peak(double* tflops, void* stream);

/* Device self-test of the library's exact arithmetic helpers: n seeded operands a over
 * the whole double range (zeros, subnormals, [2^-1000, 2^1000], both signs) are divided by
 * y with the library's division-by-constant sequence and compared bit for bit with IEEE
 * a / y, and the integer sign/threshold tests are compared with the IEEE comparisons
 * against `threshold`.  *failures = number of mismatches (0 expected).  No counterpart
 * in the reference. */
int madv_selftest_exact(double y, double threshold, long long n, long long* failures, void* stream);

const char* madv_last_error(void);
const char* madv_version(void);

/* Maestro::MacProj (Source/MaestroMacProj.cpp:11-236, declared at Source/Maestro.H:835),
 * 3-D, one level, plane-parallel or spherical (beta0 on the faces from MakeS0mac, :41-44).
 * umac[3] (>= 1 ghost face) enters with Utilde^* and leaves
 * with Utilde = Utilde^* - (B / beta0) grad phi, B = beta0^2 / rho_face (use_alt_energy_fix),
 * where phi solves -div(B grad phi) = macrhs - div(beta0 Utilde^*) to
 * max|residual| <= tol_rel * max|rhs| (the reference's mac_tol_rel: min(eps_mac *
 * mac_level_factor^finest_level, eps_mac_max) = 1e-10 on one level).  Boundaries: periodic,
 * outflow Dirichlet phi = 0, other physical faces Neumann (SetMacSolverBCs).  The ghost
 * faces of umac are refilled (FillBoundary + FillUmacGhost).  rho: the density the
 * reference fills from sold (predictor) or the sold / snew average (corrector), valid
 * cells read.  macrhs: beta0 (S - Sbar), valid cells.  beta0: host array [nr] (spherical:
 * the radial bins of the base state).  macphi
 * (may be NULL) receives phi on the valid cells (mean-free when no face is Dirichlet).
 * The solve is a cell-centred geometric multigrid on the level's domain (even extents).
 * Returns MADV_ERR_NOCONV if max_iter V-cycles do not reach the tolerance. */
typedef struct {
    int iterations;       /* V-cycles taken */
    double resid_ratio;   /* final max|residual| / max|rhs| */
} madv_mac_result;
int madv_mac_project(madv_ctx* ctx, const madv_multifab* umac, const madv_multifab* macphi,
                     const madv_multifab* macrhs, const madv_multifab* rho, const double* beta0, double tol_rel,
                     int max_iter, madv_mac_result* result, void* stream);

/* Maestro::MacProj on an AMR hierarchy (the layout's nlev levels; one level: madv_mac_project),
 * two plane-parallel 3-D levels: umac[3*nlev] (faces of level l at [3l + d]), macphi[nlev]
 * (may be NULL), macrhs[nlev], rho[nlev], beta0: host array of every level's rows, level 0's
 * nr0 then level 1's nr1 = 2 nr0 (the (lev, r) rows of the reference's BaseState); its edges
 * come from CelltoEdge over each level's radial chunks, level 1's restricted onto level 0.
 * The composite problem: phi on the level-0 cells no level-1 box covers and on the level-1
 * cells; a level-1 cell sees across a coarse-fine face the ghost (1/3) phi_fine +
 * (2/3) phi_parent, and a level-0 cell's flux through that face is the mean of the four fine
 * fluxes.  (The reference's MLMG interpolates its coarse-fine ghosts in AMReX's own way,
 * which is not restated here: the two agree to the discretisation error at the coarse-fine
 * boundary, not to the tolerance.)  Solved to max|residual| <= tol_rel max|rhs| by
 * conjugate gradients preconditioned with a level-0 V-cycle and level-1 smoothing; then
 * AverageDownFaces and FillPatchUedge of umac, as the reference ends.  result.iterations
 * counts conjugate-gradient iterations.  A level-1 face on the coarse-fine boundary takes
 * the parent coarse cell's rho outside. */
int madv_mac_project_levels(madv_ctx* ctx, int nlev, const madv_multifab* umac, const madv_multifab* macphi,
                            const madv_multifab* macrhs, const madv_multifab* rho, const double* beta0,
                            double tol_rel, int max_iter, madv_mac_result* result, void* stream);

#ifdef __cplusplus
}
#endif
#endif
