// Host-side context of the scalar-advection stage library: one Ctx per AMR level.
#pragma once
#include <cuda_runtime.h>

#include <array>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "../../include/maestro_adv.h"
#include "madv_core.cuh"

namespace madv {

// thrown by table builders when a device allocation fails
struct Fail {
    int code;
};

// Full-star spherical geometry: cell (i,j,k) of a level sits at prob_lo + (i + 1/2) dx - centre
// (Source/MaestroFill3dData.cpp:103-110); with the exact base state, cells of every level map
// to the radial bin round(r^2 / (2 dxf^2) - 3/8), dxf the finest cell size
// (Source/MaestroBaseStateGeometry.cpp:24-35); with uniform bins (use_exact_base_state = 0)
// to int(r / drf), drf = dxf / drdxfac, and the radial arrays are interpolated
// (Source/MaestroFill3dData.cpp:193-336).
struct SphGeo {
    double plo[3], dx[3], ctr[3];
    double dxf;  // cell size of the finest level, which sets the radial grid
    double drf;  // base_geom.dr_fine
    int exact;   // use_exact_base_state
    int nr;      // nr_fine
    int w0i, w0maci, s0i, s0maci;  // w0_interp_type, w0mac_interp_type, s0_interp_type, s0mac_interp_type
};

struct HBox {
    int lo[3];
    int hi[3];
};

// Internal fields of a level.  The working copies of the caller's state (sold, snew,
// umac, ...) live here too: the entry points copy the caller's FABs in and out, so the
// kernels see one fixed layout.
enum FieldId {
    F_SOLD, F_SNEW, F_GPI, F_THERMAL, F_W0CART, F_W0FCART, F_UTILDE, F_UFULL,
    F_UTRANS0, F_UTRANS1, F_UTRANS2, F_UMAC0, F_UMAC1, F_UMAC2,
    F_VELFORCE, F_SCALFORCE,
    F_SEDGE0, F_SEDGE1, F_SEDGE2, F_SFLUX0, F_SFLUX1, F_SFLUX2, F_ETA,
    F_RHO0CART, F_RHOH0CART, F_S0ECART, F_P0CART, F_PSICART, F_GRAVCART,
    F_FACE0, F_FACE1, F_FACE2,     // PPM interface values, per direction
    F_IPC0, F_IPC1, F_IPC2,        // Ip of traced component c (3 directional comps)
    F_IMC0, F_IMC1, F_IMC2,
    F_SL0, F_SL1, F_SL2,           // left/right predictor states and upwind state per
    F_SR0, F_SR1, F_SR2,           // face direction (3 comps for velocity, 1 for scalars)
    F_SIMH0, F_SIMH1, F_SIMH2,
    F_Q01, F_Q02, F_Q10, F_Q12, F_Q20, F_Q21,  // transverse states [d][t] / [c][d]
    F_DIVU, F_SLOPE,
    F_DSVL,                        // van Leer slope per cell (ppm_type 1), one direction
    F_TRA0, F_TRA1, F_TRA2,        // tracing coefficients (A, B) per D-face of umac
    F_TRC,                         // tracing coefficients per cell of ufull (A_d, B_d)
    F_TCOEF,                       // transverse coefficients per cell (dt6: 0-2, dt4: 3-5)
    F_W0MAC0, F_W0MAC1, F_W0MAC2,  // spherical: w0 on faces (MakeW0mac)
    F_S0CART2,                     // spherical: a base-state array on cells, two ghosts (MakeS0mac)
    F_S0MAC0, F_S0MAC1, F_S0MAC2,  // spherical: base state on faces (MakeS0mac), old
    F_S0MACB0, F_S0MACB1, F_S0MACB2,  //   and new
    F_S0MACC0, F_S0MACC1, F_S0MACC2,  // spherical, uniform bins: rho0 on faces, old
    F_S0MACD0, F_S0MACD1, F_S0MACD2,  //   and new (h0 on faces goes into F_S0MAC*, F_S0MACB*)
    F_W0NODAL,                     // spherical, w0mac_interp_type 4: w0 at the nodes (3 comps)
    F_GRADW0,                      // spherical, uniform bins: dw0/dr on cells (MakeVelForce)
    F_DIVW0,                       // spherical, uniform bins: div w0 on cells (ModifyScalForce)
    F_IPF, F_IMF,                  // ppm_trace_forces: the traced force, 3 directional comps
    F_SEDGES0, F_SEDGES1, F_SEDGES2,  // species streaming: edge-state slots (Rho, RhoH, one species)
    F_SFLUXS0, F_SFLUXS1, F_SFLUXS2,  //   and flux slots, standing in for F_SEDGE* / F_SFLUX*
    F_USER,                        // first slot of per-call views of caller FABs
    NF_INTERNAL = F_USER
};
constexpr int N_USER_SLOTS = 72;
constexpr int NF_TOTAL = F_USER + N_USER_SLOTS;

// transverse-state field for the ordered pair (a, b), a != b
#define Q_FIELD(a, b) (F_Q01 + 2 * (a) + ((b) > (a) ? (b)-1 : (b)))

struct FieldSpec {
    int ncomp = 0, ng = 0, nodal = -1;
};

struct Field {
    FieldSpec spec;
    double* base = nullptr;
    size_t bytes = 0;
    bool deferred = false;  // storage not allocated yet: its views are empty
};

struct RegionTable {
    RegionBox* d = nullptr;
    std::vector<RegionBox> h;  // region pieces (one per box, two for boundary slabs)
    long total = 0;
};

struct CopyDesc {
    int dst_b, src_b;
    int lo[3];
    int n[3];
    int shift[3];
    int pad;
    long start;
};
static_assert(sizeof(CopyDesc) == 56, "CopyDesc layout");

struct CopyTable {
    CopyDesc* d = nullptr;
    std::vector<CopyDesc> h;
    long total = 0;
};

struct Ctx {
    madv_params P{};  // dx, domain and base_cutoff_density_coord are this level's
    int lev = 0;
    int ndim = 3;     // 2: the 2-D form (y radial, k = 0 only, regions never grow in z)
    bool sph = false; // spherical geometry, exact base state (one level)
    SphGeo geo{};
    int nspec = 0, nscal = 0, ng_s = 3, ng_adv = 3, nr = 0;
    bool per[3] = {false, false, false};
    std::vector<HBox> ba;
    int nb = 0;
    bool have_layout = false, have_base = false;
    BCRecD bcs_s[MAX_SCAL], bcs_u[3], bcs_f[MAX_SCAL];
    BCRecD* d_bcs = nullptr;  // [0,nscal): bcs_s, [nscal, nscal+3): bcs_u, then bcs_f
    // 1-D base state on the device
    std::map<std::string, double*> d1;
    std::map<std::string, std::vector<double>> h1;
    Field F[NF_INTERNAL];
    std::vector<FabView> hviews;  // NF_TOTAL * nb
    FabView* dviews = nullptr;
    FabView* hviews_pinned = nullptr;
    // the table of a stage call that works in caller FABs laid out as its fields
    // (built from hviews_pinned with those fields' views replaced; allocated on first use)
    FabView* dviews_alias = nullptr;
    FabView* hviews_alias = nullptr;
    std::map<std::array<int, 8>, RegionTable> regions;
    std::map<std::array<int, 3>, CopyTable> copies;
    cudaStream_t stream = nullptr;
    int per_box = 0;      // launch mode: 0 batched, 1 one launch per box
    bool dry = false;     // build region / copy tables only, launch nothing
    // per-kernel timing (madv_profile): events around every launch
    bool profiling = false;
    struct ProfRec {
        const void* fn;
        cudaEvent_t e0, e1;
    };
    std::vector<ProfRec> prof;
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_next = 0;
    cudaEvent_t next_event();
    long launches = 0;
    // launch shape: threads per block of each kernel (autotuned per level; 256 by default),
    // a trial value that overrides them all while the autotuner times a candidate, and the
    // largest block each kernel can take
    std::map<const void*, int> tpb_choice;
    std::map<std::string, int> tpb_by_name;  // a loaded table, resolved at first launch
    std::map<const void*, int> tpb_max;
    std::map<const void*, std::map<int, double>> tune_ms;
    int tpb_trial = 0;
    // PPM form trials of the autotuner (madv_autotune_ppm_trial): the candidate being timed
    // (-1: none), the PPM kernels' device time per candidate, and the per-kernel cache of
    // "is a PPM kernel" (k_dsvl, k_ppm_face, k_ppm_cell, k_ppm_sweep)
    int ppm_trial = -1;
    std::map<int, double> ppm_tune_ms;
    std::map<const void*, bool> is_ppm_fn;
    int ppm_form = -1;  // the candidate chosen or loaded (-1: the context's own options)
    int tpb_of(const void* fn);
    int* d_flag = nullptr;  // device error flag (EOS cutoff)
    unsigned long long* d_red = nullptr;  // EstDt maxima (allocated on first use)
    double* d_reg = nullptr;  // flux register of this (fine) level with the level below (reflux_type 2)
    struct MacMG* mac = nullptr;  // MAC-projection multigrid grids of this level (madv_macproj.cu)
    // graph mode
    cudaGraphExec_t graph_exec = nullptr;
    std::vector<const void*> graph_key;
    long graph_launches = 0;
    // called before / after each component of MakeEdgeScal (3-D): the adjoint points the
    // component's PPM and transverse scratch (F_FACE*, F_Q*, F_SIMH*) at its own storage
    // there, to keep them for the reverse sweep
    std::function<void(int)> edge_tape_begin, edge_tape;
    // PPM sweeps: the staged (fused) form (madv_sweep.cu) when turned on; tile shape
    // across each direction D (cells in the two transverse directions), default when absent
    bool staged_ppm = false;
    std::map<int, std::array<int, 2>> sweep_shape;
    // component streams (option "component_streams"): the components of a MakeEdgeScal call
    // alternate between the level's stream and `side`, the side's components working in
    // copies of the per-component scratch fields (views in dviews_side, a copy of the table
    // side_mirror with those fields moved); built per stage call, used while dviews ==
    // side_mirror
    bool comp_streams = false;
    // option "es_inline": MakeEdgeScal's edge kernels form the predictor's l / r from Ip / Im
    // and only the upwind state is stored (ppm_type 1 / 2, outside the adjoint's tape)
    bool es_inline = true;
    // option "mg_block_cycle": the MAC multigrid's V-cycle from the first grid of at most 4096
    // cells down runs in one thread block (one launch per cycle instead of ~170)
    bool mg_block_cycle = true;
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::map<int, double*> side_scratch;
    FabView* dviews_side = nullptr;
    FabView* hviews_side = nullptr;
    const FabView* side_mirror = nullptr;
    // scratch of the single-box entry points (madv_ppm), grown on demand
    double* box_scratch = nullptr;
    long box_scratch_n = 0;

    // coarse-fine data (hierarchies of more than one level)
    std::vector<int> h_owner;  // box owning each cell of the level's domain, -1 = none
    int* d_owner = nullptr;
    std::vector<std::array<int, 2>> chunks;  // radial cell ranges of the level's base state
    std::map<std::array<int, 4>, RegionTable> amr_tables;

    double* b1(const char* name) { return d1.at(name); }
    const FabView* V() const { return dviews; }
};

// The levels of one hierarchy (level 0 first); every level shares the stream and flags.
struct Hier {
    std::vector<Ctx*> L;
    int n() const { return (int)L.size(); }
    Ctx& operator[](int l) const { return *L[l]; }
};

// Region of each box: the valid cell box grown by glo (low side) / ghi (high side), with
// `nodal` marking a face-centred index space (hi[nodal] + 1 before growing).
// `slab` >= 0 selects, for the physical-boundary fill, only cells outside the domain in
// direction slab (both sides).
const RegionTable& region(Ctx& c, int glo0, int glo1, int glo2, int ghi0, int ghi1, int ghi2,
                          int nodal = -1, int slab = -1);
const CopyTable& copy_table(Ctx& c, int ng, int nodal);

void set_error(const std::string& s);
bool cuda_ok(cudaError_t e, const char* what);

// ---- staged PPM sweep (madv_sweep.cu) ----
bool ppm_sweep(Ctx& c, int D, int fs, int sc, int fu, int uc, int umac, int fip, int fim, int lo_ext, int hi_ext);
void sweep_free(Ctx& c);

// ---- kernel launch wrappers (madv_kernels.cu) ----
void fill_boundary(Ctx& c, int fid, int c0, int nc);
void phys_fill(Ctx& c, int fid, int c0, int nc, const BCRecD* bcs_dev, int bc_c0, int is_vel,
               int state_c0);
void fill_patch(Ctx& c, int fid, int c0, int nc, int which_bcs, int bc_c0, int is_vel, int state_c0);
void fill_face_ghosts(Ctx& c, int f0);  // FillBoundary + FillUmacGhost of 3 face fields f0..f0+2
void mac_free(Ctx& c);
int mac_project_level(Ctx& c, int srhs, int srho, int sphi, const double* beta0, const double* beta0_edge,
                      double tol_rel, int max_iter, int* iters_out, double* ratio_out);
// MacProj on two plane-parallel levels (madv_macproj.cu): level 0 in c, level 1 in f
int mac_project_two_levels(Ctx& c, Ctx& f, int srhs, int srho, int sphi, const double* b0c, const double* b0ce,
                           const double* b1, const double* b1e, double tol_rel, int max_iter, int* iters_out,
                           double* ratio_out);
void addw0(Ctx& c, int f0, double mult);
void set_val(Ctx& c, int fid, double v, int c0, int nc, int ngrow);
void copy_fab(Ctx& c, int dst, int dc0, int src, int sc0, int nc, int ngrow);
void add_fab(Ctx& c, int dst, int src, int nc, int ngrow);
void put1d(Ctx& c, int fid, const double* d_s0, int outcomp, int edge, int vec = 0);
void make_utrans(Ctx& c);
// valid cells; face velocity fe .. fe+2; F_GRAVCART / F_RHO0CART filled by the caller
void make_vel_force(Ctx& c, int fe = F_UTRANS0);
void vel_pred(Ctx& c);
void vel_pred_prep(Ctx& c);  // the MakeUtrans work VelPred reuses, for a VelPred call on its own
// slot >= 0: the edge state of every component goes to component `slot` of F_SEDGE* (species
// streaming); setup = false: the velocity-only coefficients are already in place
void make_edge_scal(Ctx& c, int start_comp, int num_comp, int which_bcs, int is_conservative,
                    int force_zero, int is_vel = 0, int slot = -1, bool setup = true);
void edge_scal_setup(Ctx& c, int is_conservative);
void modify_scal_force(Ctx& c, int comp, int s0cart_fid, int fullform);
void make_rhoh_force(Ctx& c, int is_prediction, int add_thermal);
void put_in_pert_form(Ctx& c, const double* d_s0, int comp, int flag);
void convert_rhox_to_x(Ctx& c, int flag, int c0 = FIRSTSPEC, int nc = -1);  // nc -1: every species
// species c0 .. c0+nc-1 (nc -1: every species); slot >= 0: their edge state and flux in component
// `slot` of F_SEDGE* / F_SFLUX* (one species per call), the Rho flux and etarhoflux accumulated
void make_rhox_flux(Ctx& c, const double* r0_old, const double* r0e_old, const double* r0_new,
                    const double* r0e_new, int c0 = FIRSTSPEC, int nc = -1, int slot = -1);
void sum_species_edge_step(Ctx& c, int slot, int first);  // species_pred_type 2, streamed
void make_rhoh_flux(Ctx& c, const double* rh0_old, const double* rh0e_old, const double* rh0_new,
                    const double* rh0e_new, const double* r0_old, const double* r0e_old, const double* r0_new,
                    const double* r0e_new);
void convert_rhoh_to_h(Ctx& c, int flag);  // valid region
void h_force(Ctx& c);                      // scal_force(RhoH) /= sold(Rho), valid + 1 ghost
void sum_species_edges(Ctx& c);
long ppm_box_scratch_doubles(const int n[3]);
int ppm_box_run(const madv_params& P, const madv_box* bx, const madv_fab* s, int comp, const madv_fab* u,
                const madv_fab* v, const madv_fab* w, int is_umac, const int* bc, const madv_fab* Ip,
                const madv_fab* Im, double* scratch, cudaStream_t st, long& launches);
void update_scal(Ctx& c, int start_comp);
// UpdateScal of the species split for streaming: one species from its flux in F_SFLUX* comp
// `slot`, then the density, floor and negative-species pass over all of them
void update_species(Ctx& c, int comp, int slot);
void update_rhox_fix(Ctx& c);
void update_vel(Ctx& c, int fu, int fsponge);  // UpdateVel into F_SNEW comps 0-2; fsponge -1: no sponge
// EstDt maxima of a level into c.d_red[0..6] (spdx, spdy, spdz, spdr, fx, fy, fz as bit patterns)
void dt_maxima(Ctx& c);

// ---- spherical forms (madv_sphr.cu), reached through the wrappers above when c.sph
void put1d_sph(Ctx& c, int fid, const double* d_s0, int outcomp, int edge, int vec);
void make_w0mac(Ctx& c);
void make_s0mac_faces(Ctx& c, int dst0);  // faces of F_S0CART2 into dst0 .. dst0 + 2
void make_s0mac_interp(Ctx& c, const double* d_s0, int dst0);  // s0mac_interp_type 2, 3 (uniform bins)
void addw0_sph(Ctx& c, int f0, double mult);
void make_vel_force_sph(Ctx& c, int fe);
void modify_scal_force_sph(Ctx& c, int comp, int s0cart_fid, int fullform);
void make_rhoh_force_sph(Ctx& c, int is_prediction, int add_thermal);
void put_in_pert_form_sph(Ctx& c, const double* d_s0, int comp, int flag);
void make_rhox_flux_sph(Ctx& c, int c0, int nc, int slot);
void make_rhoh_flux_sph(Ctx& c);

// ---- 2-D forms (madv_kernels.cu), reached through the wrappers above when c.ndim == 2
void put1d_2d(Ctx& c, int fid, const double* d_s0, int outcomp, int edge);
void addw0_2d(Ctx& c, int f0, double mult);
void make_utrans_2d_entry(Ctx& c);
void make_vel_force_2d(Ctx& c);
void vel_pred_2d_entry(Ctx& c);
void make_edge_scal_2d_entry(Ctx& c, int start_comp, int num_comp, int which_bcs, int is_cons);
void modify_scal_force_2d(Ctx& c, int comp, int s0cart_fid, int fullform);
void make_rhoh_force_2d(Ctx& c, int is_prediction, int add_thermal);
void put_in_pert_form_2d(Ctx& c, const double* d_s0, int comp, int flag);
void make_rhox_flux_2d(Ctx& c, const double* r0_old, const double* r0e_old, const double* r0_new,
                       const double* r0e_new);
void make_rhoh_flux_2d(Ctx& c, const double* rh0_old, const double* rh0e_old, const double* rh0_new,
                       const double* rh0e_new, const double* r0_old, const double* r0e_old, const double* r0_new,
                       const double* r0e_new);
void sum_species_edges_2d(Ctx& c);
void update_scal_2d(Ctx& c, int start_comp);

// ---- coarse-fine operations between level cf and its parent cc (madv_amr.cu)
int build_owner(Ctx& c);  // owner map of the level's domain (host + device)
void interp_fill(Ctx& cc, Ctx& cf, int fid, int c0, int nc, int which_bcs, int bc_c0, int is_vel, int state_c0);
void average_down(Ctx& cf, Ctx& cc, int fid, int comp, int ncomp);
void average_down_faces(Ctx& cf, Ctx& cc, int f0, int c0, int ncomp);
void uedge_interface(Ctx& cc, Ctx& cf, int f0);
// slot >= 0: the flux of component c0 (nc 1) is read from F_SFLUX* component `slot`
void flux_reg_crse_init(Ctx& cf, Ctx& cc, int c0, int nc, double dt, int slot = -1);
void flux_reg_fine_add(Ctx& cf, int c0, int nc, double dt, int slot = -1);
void flux_reg_reflux(Ctx& cf, Ctx& cc, int c0, int nc);

// ---- reverse sweep (madv_adjoint.cu).  User slots bound by the adjoint driver: working
// state (A_WSOLD / A_WSNEW), state adjoints (A_ASOLD / A_ASNEW), edge-state adjoints, the
// per-component scratch of the MakeEdgeScal transpose, and the caller's FABs.
enum {
    A_WSOLD = 28, A_WSNEW, A_ASOLD, A_ASNEW, A_AS, A_AFORCE,
    A_AEDGE0, A_AEDGE1, A_AEDGE2,
    A_ASL0, A_ASL1, A_ASL2, A_ASR0, A_ASR1, A_ASR2, A_ASIMH0, A_ASIMH1, A_ASIMH2,
    A_AQ01, A_AQ02, A_AQ10, A_AQ12, A_AQ20, A_AQ21,
    A_ASM, A_ASP, A_ADSVL,
    A_WEIGHT, A_SOLD0, A_GRADS, A_SFIN,
    A_AUMAC0, A_AUMAC1, A_AUMAC2, A_ATCOEF, A_AUTRANS0, A_AUTRANS1, A_AUTRANS2, A_AUT, A_GRADU,
    A_AVELF,  // buoyancy: adjoint of MakeVelForce's force (3 components, one ghost cell)
    A_END
};
static_assert(A_END <= N_USER_SLOTS, "user slots");
void ppm_faces(Ctx& c, int d, int fs, int sc, int faces);  // van Leer slopes (+ interface values)
void edge_scal_coeffs(Ctx& c);                  // tracing / transverse coefficients of F_UMAC0..2
void adj_update(Ctx& c);
void adj_flux(Ctx& c, int want_u);
void adj_edge_scal(Ctx& c, int fs, int comp, int force_zero, double* dir, size_t dir_bytes, int want_u);
void adj_fill_boundary(Ctx& c, int slot, int nc, int ng, int nodal);
void adj_phys_fill(Ctx& c, int slot, int n, int ng, const BCRecD& bc);
void adj_convert_x(Ctx& c, int comp);
void adj_pert_force(Ctx& c, int comp, int want_u);
void adj_tcoef(Ctx& c, int ts);
void adj_vel_pred(Ctx& c, double* dir, size_t dir_bytes);
// buoyancy (a MAC velocity that depends on the density through MakeVelForce): the MAC
// velocity adjoint's ghost faces (FillUmacGhost^T, then FillBoundary^T), VelPred's final
// states transposed with respect to the force, the force's FillPatch^T, and MakeVelForce^T
// into the density adjoint (A_ASOLD)
void adj_umac_ghosts(Ctx& c);
void adj_vel_force(Ctx& c);
// face-velocity terms of the spherical (rho h) flux (F_S0MAC* set as rhoh_flux sets them) and
// ModifyScalForce (Cartesian base state in field s0c), and of MakeRhoHForce (force adjoint
// scale * component comp of slot src; F_P0CART and, spherical, p0 faces in F_S0MAC* current)
void adj_flux_rhoh_u_sph(Ctx& c);
void adj_pert_u_sph(Ctx& c, int comp, int s0c);
void adj_rhoh_force_u(Ctx& c, int src, int comp, double scale);
long adj_dot_parts(Ctx& c);
void adj_dot(Ctx& c, int slot_a, int slot_b, int nc, double* part, double* d_out);

enum { BCS_S = 0, BCS_U = 1, BCS_F = 2 };
inline const BCRecD* bcs_dev(const Ctx& c, int which) {
    return which == BCS_S ? c.d_bcs : (which == BCS_U ? c.d_bcs + c.nscal : c.d_bcs + c.nscal + 3);
}
inline const BCRecD* bcs_host(const Ctx& c, int which) {
    return which == BCS_S ? c.bcs_s : (which == BCS_U ? c.bcs_u : c.bcs_f);
}

}  // namespace madv
