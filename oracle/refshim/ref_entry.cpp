// Test infrastructure only: C entry points into the reference's own stage functions,
// compiled unmodified from the reference sources against AMReX_shim.H / Maestro.H (see
// oracle/Makefile, target `ref`; the library goes to oracle/_ref/).  Used by tests/ to pin
// the oracle's restatement (and, through tests/golden/, the GPU library) to the reference.
#include <cstring>
#include <string>

#include "Maestro.H"
#include "maestro_oracle.h"

namespace maestro {
int reflux_type = 1;
int maestro_verbose = 0;
amrex::Real cfl = 0.5;
amrex::Real init_shrink = 1.0;
amrex::Real small_dt = 1.e-10;
amrex::Real max_dt = 1.e33;
amrex::Real fixed_dt = -1.0;
bool use_soundspeed_firstdt = false;
bool use_divu_firstdt = false;
bool spherical = false;
bool octant = false;
bool do_sponge = false;
amrex::Real anelastic_cutoff_density = -1.0;
amrex::Real base_cutoff_density = -1.0;
amrex::Real burning_cutoff_density_lo = -1.0;
amrex::Real burning_cutoff_density_hi = 1.e100;
amrex::Real buoyancy_cutoff_factor = 5.0;
bool evolve_base_state = true;
bool use_exact_base_state = false;
bool average_base_state = false;
bool do_eos_h_above_cutoff = true;
int enthalpy_pred_type = 1;
int species_pred_type = 1;
int slope_order = 4;
int ppm_type = 1;
int ppm_trace_forces = 0;
bool use_centrifugal = true;
bool use_alt_energy_fix = true;
int s0_interp_type = 3;
int w0_interp_type = 2;
int s0mac_interp_type = 1;
int w0mac_interp_type = 1;
int drdxfac = 5;
amrex::Real grav_const = -1.5e10;
amrex::Real planar_invsq_mass = 0.0;
bool do_planar_invsq_grav = false;
bool do_2d_planar_octant = false;
}  // namespace maestro

int Maestro::ng_s = 3;
// needs the equation of state (temperature predictions): not in this build
void Maestro::HfromRhoTedge(FaceMFs&, const BaseState<Real>&, const BaseState<Real>&, const BaseState<Real>&,
                            const BaseState<Real>&) {
    amrex::Abort("HfromRhoTedge needs the equation of state");
}

amrex::IntVect Maestro::nodal_flag(1, 1, 1);
amrex::IntVect Maestro::nodal_flag_x(1, 0, 0);
amrex::IntVect Maestro::nodal_flag_y(0, 1, 0);
amrex::IntVect Maestro::nodal_flag_z(0, 0, 1);

amrex::Interpolater amrex::cell_cons_interp;

using namespace amrex;

namespace {
std::string g_err;

struct RefFab {  // same layout as the oracle's mo_fab
    double* p;
    int lo[3];
    int hi[3];
    int nc;
};

template <class T>
Array4<T> arr(const RefFab* f) {
    return Array4<T>(f->p, Dim3{f->lo[0], f->lo[1], f->lo[2]}, Dim3{f->hi[0] + 1, f->hi[1] + 1, f->hi[2] + 1},
                     f->nc);
}

Box box_of(const int* b) {
    Box bx;
    for (int d = 0; d < 3; ++d) {
        bx.lo[d] = b[d];
        bx.hi[d] = b[3 + d];
    }
    return bx;
}
void set_params(const mo_params* p) {
    maestro::ppm_type = p->ppm_type;
    maestro::slope_order = p->slope_order;
    maestro::ppm_trace_forces = p->ppm_trace_forces;
    maestro::spherical = p->spherical;
    maestro::use_exact_base_state = p->use_exact_base_state;
    maestro::evolve_base_state = p->evolve_base_state;
    maestro::species_pred_type = p->species_pred_type;
    maestro::enthalpy_pred_type = p->enthalpy_pred_type;
    maestro::reflux_type = p->reflux_type;
    maestro::base_cutoff_density = p->base_cutoff_density;
    maestro::buoyancy_cutoff_factor = p->buoyancy_cutoff_factor;
    maestro::do_eos_h_above_cutoff = p->do_eos_h_above_cutoff;
    maestro::drdxfac = p->drdxfac > 0 ? p->drdxfac : 1;
    maestro::w0_interp_type = p->w0_interp_type ? p->w0_interp_type : 2;
    maestro::w0mac_interp_type = p->w0mac_interp_type ? p->w0mac_interp_type : 1;
    maestro::s0_interp_type = p->s0_interp_type ? p->s0_interp_type : 3;
    maestro::s0mac_interp_type = p->s0mac_interp_type ? p->s0mac_interp_type : 1;
}

// phys_bc -> BCType of the velocity, scalar and "first-order extrapolation" components,
// the table of Maestro::BCSetup (Source/MaestroSetup.cpp:329-500)
void bc_setup(Maestro& m) {
    using namespace amrex::BCType;
    m.bcs_s.assign(Nscal, BCRec());
    m.bcs_u.assign(AMREX_SPACEDIM, BCRec());
    m.bcs_f.assign(Nscal, BCRec());
    for (int side = 0; side < 2; ++side)
        for (int dir = 0; dir < AMREX_SPACEDIM; ++dir) {
            const int pb = side == 0 ? m.phys_bc.lo(dir) : m.phys_bc.hi(dir);
            int u, s, t, pi, f;
            int udir = -999;
            switch (pb) {
                case 0: u = s = t = pi = f = int_dir; break;                                  // interior
                case 1: u = s = t = ext_dir; pi = f = foextrap; break;                         // inflow
                case 2: u = s = t = foextrap; pi = ext_dir; f = foextrap; break;               // outflow
                case 3: u = s = t = pi = f = reflect_even; udir = reflect_odd; break;          // symmetry
                case 4: u = s = t = hoextrap; udir = ext_dir; pi = f = foextrap; break;        // slipwall
                case 5: u = ext_dir; s = t = hoextrap; pi = f = foextrap; break;               // noslipwall
                default: amrex::Abort("Invalid phys_bc");
            }
            auto set = [&](BCRec& r, int v) { side == 0 ? r.setLo(dir, v) : r.setHi(dir, v); };
            for (int c = 0; c < AMREX_SPACEDIM; ++c) set(m.bcs_u[c], (c == dir && udir != -999) ? udir : u);
            set(m.bcs_s[Rho], s);
            set(m.bcs_s[RhoH], s);
            for (int c = FirstSpec; c < FirstSpec + NumSpec; ++c) set(m.bcs_s[c], s);
            set(m.bcs_s[Temp], t);
            set(m.bcs_s[Pi], pi);
            for (int c = 0; c < Nscal; ++c) set(m.bcs_f[c], f);
        }
}

void setup_base_state(Maestro& m, const mo_params* p, const mo_inputs* in);

void setup(Maestro& m, const mo_params* p, int nboxes, const int* boxes, const mo_inputs* in) {
    if ((p->dim == 2 ? 2 : 3) != AMREX_SPACEDIM)
        amrex::Abort("this reference build is " + std::to_string(AMREX_SPACEDIM) + "-D");
    if (p->nspec != NumSpec) amrex::Abort("the reference build has NumSpec " + std::to_string(NumSpec));
    set_params(p);
    m.dt = p->dt;
    m.rel_eps = p->rel_eps;
    m.finest_level = 0;
    Geometry g;
    for (int d = 0; d < 3; ++d) {
        g.domain.lo[d] = p->dom_lo[d];
        g.domain.hi[d] = p->dom_hi[d];
        g.dx_[d] = p->dx[d];
        g.rb.lo_[d] = p->prob_lo[d];
        g.rb.hi_[d] = p->prob_hi[d];
        g.per[d] = p->phys_bc_lo[d] == 0;
        m.phys_bc.setLo(d, p->phys_bc_lo[d]);
        m.phys_bc.setHi(d, p->phys_bc_hi[d]);
    }
    m.geom.assign(1, g);
    std::vector<Box> bl;
    for (int b = 0; b < nboxes; ++b) bl.push_back(box_of(boxes + 6 * b));
    m.grids.assign(1, BoxArray(bl));
    m.dmap.assign(1, DistributionMapping());
    MultiFab::domain_for_fills() = g.domain;
    bc_setup(m);
    Maestro::ng_s = maestro::ppm_type == 2 ? 4 : 3;
    m.ng_adv = Maestro::ng_s;
    m.t_old = 0.0;
    m.t_new = p->dt;
    setup_base_state(m, p, in);
}

// The radial base state as Maestro::Setup (Source/MaestroSetup.cpp:57-118) sizes it and
// BaseStateGeometry::Init / InitMultiLevel / ComputeCutoffCoords lay it out, holding the
// caller's 1-D arrays; spherical geometry also gets the cell normals and the cell-to-bin
// map (Source/MaestroInit.cpp:71-72, 120-121).
void setup_base_state(Maestro& m, const mo_params* p, const mo_inputs* in) {
    int nr_fine, nr_irreg = 0;
    Real dr_fine;
    if (maestro::spherical) {
        const Real domhi = p->dom_hi[0] + 1;
        nr_irreg = int((3.0 * (domhi / 2 - 0.5) * (domhi / 2 - 0.5) - 0.75) / 2.0);
        dr_fine = p->dx[0] / maestro::drdxfac;
        if (maestro::use_exact_base_state) {
            nr_fine = nr_irreg + 1;
        } else {
            const double lenx = 0.5 * (p->prob_hi[0] - p->prob_lo[0]);
            const double leny = 0.5 * (p->prob_hi[1] - p->prob_lo[1]);
            const double lenz = 0.5 * (p->prob_hi[2] - p->prob_lo[2]);
            const double max_dist = std::sqrt(lenx * lenx + leny * leny + lenz * lenz);
            nr_fine = int(max_dist / dr_fine) + 1;
        }
    } else {
        nr_fine = p->dom_hi[AMREX_SPACEDIM - 1] + 1;
        dr_fine = p->dx[AMREX_SPACEDIM - 1];
    }
    // plane-parallel gravity is the constant grav_const (MakeGravCell,
    // Source/MaestroMakeGrav.cpp); the caller's grav_cell holds it
    if (!maestro::spherical) maestro::grav_const = in->grav_cell[0];
    m.base_geom.max_radial_level = 0;
    m.base_geom.Init(0, nr_fine, dr_fine, nr_irreg, m.geom, 0, m.center);
    BaseState<int> tags(1, nr_fine);
    tags.setVal(0);
    m.base_geom.InitMultiLevel(0, tags.array());
    auto fill = [&](BaseState<Real>& b, const double* src, int len) {
        b.resize(1, len);
        auto a = b.array();
        for (int r = 0; r < len; ++r) a(0, r) = src ? src[r] : 0.0;
    };
    fill(m.rho0_old, in->rho0_old, nr_fine);
    fill(m.rho0_new, in->rho0_new, nr_fine);
    fill(m.rhoh0_old, in->rhoh0_old, nr_fine);
    fill(m.rhoh0_new, in->rhoh0_new, nr_fine);
    fill(m.p0_old, in->p0_old, nr_fine);
    fill(m.p0_new, in->p0_new, nr_fine);
    fill(m.psi, in->psi, nr_fine);
    fill(m.grav_cell_old, in->grav_cell, nr_fine);
    fill(m.grav_cell_new, in->grav_cell, nr_fine);
    fill(m.w0_force, in->w0_force, nr_fine);
    fill(m.w0, in->w0, nr_fine + 1);
    fill(m.tempbar, nullptr, nr_fine);
    fill(m.etarho_cc, nullptr, nr_fine);
    fill(m.etarho_ec, nullptr, nr_fine + 1);
    m.base_geom.ComputeCutoffCoords(m.rho0_old.array());
    if (m.base_geom.base_cutoff_density_coord(0) != p->base_cutoff_density_coord)
        amrex::Abort("base cutoff coordinate " + std::to_string(m.base_geom.base_cutoff_density_coord(0)) +
                     " differs from the caller's " + std::to_string(p->base_cutoff_density_coord));
    const BoxArray& ba = m.grids[0];
    m.w0_cart.resize(1);
    m.w0_cart[0].define(ba, DistributionMapping(), AMREX_SPACEDIM, 2);
    m.w0_cart[0].setVal(0.0);
#if (AMREX_SPACEDIM == 3)
    if (maestro::spherical) {
        m.normal.resize(1);
        m.normal[0].define(ba, DistributionMapping(), 3, 1);
        m.cell_cc_to_r.resize(1);
        m.cell_cc_to_r[0].define(ba, DistributionMapping(), 1, 0);
        m.MakeNormal();
        m.MakeCCtoRadii();
    }
#endif
    m.Put1dArrayOnCart(m.w0, m.w0_cart, true, true, m.bcs_u, 0, 1);
}

// domain arrays (i fastest, one block per component) <-> valid regions of a MultiFab
void scatter(const Box& dom, const double* src, MultiFab& mf, int c0, int nc) {
    const long nx = dom.length(0), ny = dom.length(1), nz = dom.length(2);
    for (int b = 0; b < mf.size(); ++b) {
        const auto a = mf.array(b);
        ParallelFor(mf.boxArray()[b], nc, [&](int i, int j, int k, int n) {
            a(i, j, k, c0 + n) = src[(((long)n * nz + (k - dom.lo[2])) * ny + (j - dom.lo[1])) * nx + (i - dom.lo[0])];
        });
    }
}
void gather(const Box& dom, const MultiFab& mf, int c0, int nc, double* dst) {
    if (!dst) return;
    Box d = dom;
    for (int e = 0; e < 3; ++e)
        if (mf.boxArray()[0].typ[e]) d.surroundingNodes(e);
    const long nx = d.length(0), ny = d.length(1), nz = d.length(2);
    for (int b = 0; b < mf.size(); ++b) {
        const auto a = mf.array(b);
        ParallelFor(mf.boxArray()[b], nc, [&](int i, int j, int k, int n) {
            dst[(((long)n * nz + (k - d.lo[2])) * ny + (j - d.lo[1])) * nx + (i - d.lo[0])] = a(i, j, k, c0 + n);
        });
    }
}

BoxArray faces(const BoxArray& ba, int d) { return convert(ba, IntVect(d == 0, d == 1, d == 2)); }

#if (AMREX_SPACEDIM == 3)
int run_velocity_advance(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* in,
                         const double* rhohalf, const double* sponge, double* unew_out, double* const* umac_out) {
    Maestro m;
    setup(m, p, nboxes, boxes, in);
    maestro::do_sponge = sponge != nullptr;
    const BoxArray& ba = m.grids[0];
    const DistributionMapping dm;
    const Box dom = m.geom[0].Domain();
    const int ng = Maestro::ng_s;
    m.uold.resize(1);
    m.uold[0].define(ba, dm, AMREX_SPACEDIM, ng);
    m.uold[0].setVal(0.0);
    scatter(dom, in->uold, m.uold[0], 0, 3);
    m.unew.resize(1);
    m.unew[0].define(ba, dm, AMREX_SPACEDIM, ng);
    m.unew[0].setVal(0.0);
    m.sold.resize(1);
    m.sold[0].define(ba, dm, Nscal, ng);
    m.sold[0].setVal(0.0);
    scatter(dom, in->sold, m.sold[0], 0, Nscal);
    m.gpi.resize(1);
    m.gpi[0].define(ba, dm, AMREX_SPACEDIM, 0);
    scatter(dom, in->gpi, m.gpi[0], 0, 3);
    Vector<MultiFab> w0_force_cart(1), rh(1), sp(1);
    w0_force_cart[0].define(ba, dm, AMREX_SPACEDIM, 1);
    w0_force_cart[0].setVal(0.0);
    rh[0].define(ba, dm, 1, 1);
    rh[0].setVal(0.0);
    scatter(dom, rhohalf, rh[0], 0, 1);
    // the reference always holds a sponge field (read only with do_sponge)
    sp[0].define(ba, dm, 1, 0);
    sp[0].setVal(1.0);
    if (sponge) scatter(dom, sponge, sp[0], 0, 1);
    Vector<std::array<MultiFab, AMREX_SPACEDIM>> umac(1), w0mac(1);
    for (int d = 0; d < 3; ++d) {
        umac[0][d].define(faces(ba, d), dm, 1, 1);
        w0mac[0][d].define(faces(ba, d), dm, 1, 1);
        umac[0][d].setVal(0.0);
        w0mac[0][d].setVal(0.0);
    }
    if (maestro::spherical) m.MakeW0mac(w0mac);
    if (maestro::evolve_base_state) m.Put1dArrayOnCart(m.w0_force, w0_force_cart, false, true, m.bcs_f, 0);
    m.FillPatch(m.t_old, m.sold, m.sold, m.sold, 0, 0, Nscal, 0, m.bcs_s);
    m.AdvancePremac(umac, w0mac, w0_force_cart);
    m.FillPatchUedge(umac);
    for (int d = 0; d < 3; ++d) gather(dom, umac[0][d], 0, 1, umac_out ? umac_out[d] : nullptr);
    m.FillPatch(m.t_old, m.uold, m.uold, m.uold, 0, 0, AMREX_SPACEDIM, 0, m.bcs_u, 1);
    // rho0_nph = (rho0_old + rho0_new) / 2 and the cell gravity, as the caller passes them
    BaseState<Real> rho0_nph(1, m.base_geom.nr_fine);
    {
        auto a = rho0_nph.array();
        const auto o = m.rho0_old.array(), n = m.rho0_new.array();
        for (int r = 0; r < m.base_geom.nr_fine; ++r) a(0, r) = 0.5 * (o(0, r) + n(0, r));
    }
    m.VelocityAdvance(rh, umac, w0mac, w0_force_cart, rho0_nph, m.grav_cell_old, sp);
    gather(dom, m.unew[0], 0, 3, unew_out);
    return 0;
}

// AdvancePremac -> Addw0 -> DensityAdvance(1) -> Addw0 -> EnthalpyAdvance(1) as the
// predictor of Maestro::AdvanceTimeStep calls them (Source/MaestroAdvance.cpp:160-210,
// 290-360, 436-548), the MAC projection skipped
#endif

int run_stage(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* in, mo_outputs* out) {
    Maestro m;
    setup(m, p, nboxes, boxes, in);
    const BoxArray& ba = m.grids[0];
    const DistributionMapping dm;
    const Box dom = m.geom[0].Domain();
    const int ng = Maestro::ng_s;
    m.uold.resize(1);
    m.uold[0].define(ba, dm, AMREX_SPACEDIM, ng);
    m.uold[0].setVal(0.0);
    scatter(dom, in->uold, m.uold[0], 0, AMREX_SPACEDIM);
    m.sold.resize(1);
    m.sold[0].define(ba, dm, Nscal, ng);
    m.sold[0].setVal(0.0);
    scatter(dom, in->sold, m.sold[0], 0, Nscal);
    m.snew.resize(1);
    m.snew[0].define(ba, dm, Nscal, ng);
    m.snew[0].setVal(0.0);
    MultiFab::Copy(m.snew[0], m.sold[0], Temp, Temp, 1, ng);
    m.gpi.resize(1);
    m.gpi[0].define(ba, dm, AMREX_SPACEDIM, 0);
    scatter(dom, in->gpi, m.gpi[0], 0, AMREX_SPACEDIM);
    Vector<MultiFab> thermal(1), scal_force(1), etarhoflux(1), w0_force_cart(1);
    thermal[0].define(ba, dm, 1, 1);
    thermal[0].setVal(0.0);
    if (in->thermal) scatter(dom, in->thermal, thermal[0], 0, 1);
    // the forces carry ng_s ghost cells when they are traced (Source/MaestroAdvance.cpp:150-155)
    scal_force[0].define(ba, dm, Nscal, maestro::ppm_trace_forces ? ng : 1);
    scal_force[0].setVal(0.0);
    etarhoflux[0].define(faces(ba, AMREX_SPACEDIM - 1), dm, 1, 1);
    etarhoflux[0].setVal(0.0);
    w0_force_cart[0].define(ba, dm, AMREX_SPACEDIM, 1);
    w0_force_cart[0].setVal(0.0);
    Vector<std::array<MultiFab, AMREX_SPACEDIM>> umac(1), sedge(1), sflux(1), w0mac(1);
    for (int d = 0; d < AMREX_SPACEDIM; ++d) {
        umac[0][d].define(faces(ba, d), dm, 1, 1);
        sedge[0][d].define(faces(ba, d), dm, Nscal, 0);
        sflux[0][d].define(faces(ba, d), dm, Nscal, 0);
        w0mac[0][d].define(faces(ba, d), dm, 1, 1);
        umac[0][d].setVal(0.0);
        sedge[0][d].setVal(0.0);
        sflux[0][d].setVal(0.0);
        w0mac[0][d].setVal(0.0);
    }
#if (AMREX_SPACEDIM == 3)
    if (maestro::spherical) m.MakeW0mac(w0mac);
#endif
    if (maestro::evolve_base_state) m.Put1dArrayOnCart(m.w0_force, w0_force_cart, false, true, m.bcs_f, 0);
    BaseState<Real> rho0_predicted_edge(1, m.base_geom.nr_fine + 1);
    {
        auto a = rho0_predicted_edge.array();
        for (int r = 0; r <= m.base_geom.nr_fine; ++r) a(0, r) = in->rho0_predicted_edge[r];
    }
    // the old state's ghost cells as the previous step's UpdateScal leaves them
    m.FillPatch(m.t_old, m.sold, m.sold, m.sold, 0, 0, Nscal, 0, m.bcs_s);

    m.AdvancePremac(umac, w0mac, w0_force_cart);
    for (int d = 0; d < AMREX_SPACEDIM; ++d) gather(dom, umac[0][d], 0, 1, out->umac_vp[d]);
    m.Addw0(umac, w0mac, 1.);
    m.DensityAdvance(1, m.sold, m.snew, sedge, sflux, scal_force, etarhoflux, umac, w0mac, rho0_predicted_edge);
    m.Addw0(umac, w0mac, -1.);
    m.Addw0(umac, w0mac, 1.);
    m.EnthalpyAdvance(1, m.sold, m.snew, sedge, sflux, scal_force, umac, w0mac, thermal);
    m.Addw0(umac, w0mac, -1.);

    for (int d = 0; d < AMREX_SPACEDIM; ++d) {
        gather(dom, umac[0][d], 0, 1, out->umac_end[d]);
        gather(dom, sedge[0][d], 0, Nscal, out->sedge[d]);
        gather(dom, sflux[0][d], 0, Nscal, out->sflux[d]);
    }
    gather(dom, m.snew[0], 0, Nscal, out->snew);
    gather(dom, m.sold[0], 0, Nscal, out->sold_end);
    gather(dom, etarhoflux[0], 0, 1, out->etarhoflux);
    return 0;
}

// A MultiFab on ba (typed nodal in direction `nodal` if >= 0) with ng ghosts and nc
// components holding the caller's FABs where they overlap (NaN elsewhere).
void mf_from(MultiFab& mf, const BoxArray& ba, const mo_fab* f, int nc, int ng, int nodal) {
    BoxArray b2 = nodal >= 0 ? convert(ba, IntVect(nodal == 0, nodal == 1, nodal == 2)) : ba;
    mf.define(b2, DistributionMapping(), nc, ng);
    for (int i = 0; i < mf.size(); ++i) {
        const auto dst = mf.array(i);
        const auto src = arr<Real>(reinterpret_cast<const RefFab*>(&f[i]));
        const int ncopy = std::min(nc, f[i].nc);
        ParallelFor(mf.fabs_[i].box, ncopy, [&](int x, int y, int z, int n) {
            if (src.contains(x, y, z)) dst(x, y, z, n) = src(x, y, z, n);
        });
    }
}

// copies components [c0, c0 + nc) of the valid region of mf into the caller's FABs
void mf_to(const MultiFab& mf, const mo_fab* f, int c0, int nc) {
    for (int i = 0; i < mf.size(); ++i) {
        const auto src = mf.array(i);
        const auto dst = arr<Real>(reinterpret_cast<const RefFab*>(&f[i]));
        const Box vb = mf.boxArray()[i];
        ParallelFor(vb, nc, [&](int x, int y, int z, int n) {
            if (dst.contains(x, y, z)) dst(x, y, z, c0 + n) = src(x, y, z, c0 + n);
        });
    }
}

#if (AMREX_SPACEDIM == 3)
int member(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* base, int fn, int which_step,
           int start_comp, int num_comp, int is_cons, const mo_fab* args) {
    Maestro m;
    setup(m, p, nboxes, boxes, base);
    const BoxArray& ba = m.grids[0];
    const int ng_s = Maestro::ng_s;
    auto A = [&](int slot) { return args + (long)slot * nboxes; };
    Vector<MultiFab> m1(1), m2(1), m3(1);
    Vector<std::array<MultiFab, AMREX_SPACEDIM>> f1(1), f2(1);
    switch (fn) {
        case MO_MAKE_EDGE_SCAL: {
            mf_from(m1[0], ba, A(MO_STATE), Nscal, ng_s, -1);
            mf_from(m2[0], ba, A(MO_FORCE), Nscal, 1, -1);
            for (int d = 0; d < 3; ++d) {
                mf_from(f1[0][d], ba, A(MO_UMAC0 + d), 1, 1, d);
                f2[0][d].define(convert(ba, IntVect(d == 0, d == 1, d == 2)), DistributionMapping(), Nscal, 0);
                f2[0][d].setVal(0.0);
            }
            m.MakeEdgeScal(m1, f2, f1, m2, false, m.bcs_s, Nscal, start_comp, start_comp, num_comp, is_cons != 0);
            for (int d = 0; d < 3; ++d) mf_to(f2[0][d], A(MO_SEDGE0 + d), start_comp, num_comp);
            return 0;
        }
        default:
            amrex::Abort("member function not in this reference build");
    }
}
#endif

}  // namespace

extern "C" {

/* Maestro::PPM (Source/MaestroPPM.cpp) for component comp of s over the cell box bx[6],
 * domain dom[6], bc = {lo[3], hi[3]} (BCType of component comp), tracing velocity u/v/w. */
int ref_ppm(int ppm_type_, double dt, double rel_eps, const double* dx, const int* dom, const int* bx,
            const RefFab* s, int comp, const RefFab* u, const RefFab* v, const RefFab* w, int is_umac, const int* bc,
            const RefFab* Ip, const RefFab* Im) {
    try {
        maestro::ppm_type = ppm_type_;
        Maestro m;
        m.dt = dt;
        m.rel_eps = rel_eps;
        Vector<BCRec> bcs(comp + 1);
        for (int d = 0; d < 3; ++d) {
            bcs[comp].setLo(d, bc[d]);
            bcs[comp].setHi(d, bc[3 + d]);
        }
        GpuArray<Real, AMREX_SPACEDIM> dxa;
        for (int d = 0; d < AMREX_SPACEDIM; ++d) dxa[d] = dx[d];
        m.PPM(box_of(bx), arr<const Real>(s), arr<const Real>(u), arr<const Real>(v),
#if (AMREX_SPACEDIM == 3)
              arr<const Real>(w),
#endif
              arr<Real>(Ip), arr<Real>(Im), box_of(dom), bcs, dxa, is_umac != 0, comp, comp);
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

/* Maestro::Slopex/y/z (Source/MaestroSlopes.cpp) in direction d over bx for ncomp
 * components of s; bcs[6 * n + (0..5)] = lo[3], hi[3] of component n. */
int ref_slopes(int slope_order_, int d, const int* dom, const int* bx, const RefFab* s, int ncomp, const int* bcs_,
               const RefFab* slope) {
    try {
        maestro::slope_order = slope_order_;
        Vector<BCRec> bcs(ncomp);
        for (int n = 0; n < ncomp; ++n)
            for (int e = 0; e < 3; ++e) {
                bcs[n].setLo(e, bcs_[6 * n + e]);
                bcs[n].setHi(e, bcs_[6 * n + 3 + e]);
            }
        auto sa = arr<Real>(s);
        auto sl = arr<Real>(slope);
        if (d == 0) Maestro::Slopex(box_of(bx), sa, sl, box_of(dom), bcs, ncomp, 0);
        if (d == 1) Maestro::Slopey(box_of(bx), sa, sl, box_of(dom), bcs, ncomp, 0);
#if (AMREX_SPACEDIM == 3)
        if (d == 2) Maestro::Slopez(box_of(bx), sa, sl, box_of(dom), bcs, ncomp, 0);
#endif
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

#if (AMREX_SPACEDIM == 3)
/* mo_run_velocity_advance (oracle/maestro_oracle.h) run by the reference's own
 * AdvancePremac, FillPatchUedge (the MAC projection's closing face fill) and
 * VelocityAdvance with UpdateVel; writes unew and umac (uedge stays inside
 * VelocityAdvance). */
int ref_run_velocity_advance(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* in,
                             const double* rhohalf, const double* sponge, double* unew_out, double* const* uedge_out,
                             double* const* umac_out) {
    (void)uedge_out;
    try {
        return run_velocity_advance(p, nboxes, boxes, in, rhohalf, sponge, unew_out, umac_out);
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}
#endif

/* The stage of mo_run_stage (oracle/maestro_oracle.h) run by the reference's own
 * AdvancePremac, DensityAdvance and EnthalpyAdvance on one 3-D level; every output but
 * utrans and vel_force (local to AdvancePremac). */
int ref_run_stage(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* in, mo_outputs* out) {
    try {
        return run_stage(p, nboxes, boxes, in, out);
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

#if (AMREX_SPACEDIM == 3)
/* One Maestro member function on one 3-D level, the arguments of mo_member
 * (oracle/maestro_oracle.h): the same slots, per-box FABs and outputs, run by the
 * reference's own member function on MultiFabs holding copies of the caller's FABs;
 * outputs are copied back on the valid cells / faces. */
int ref_member(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* base, int fn, int which_step,
               int start_comp, int num_comp, int is_cons, const mo_fab* args) {
    try {
        return member(p, nboxes, boxes, base, fn, which_step, start_comp, num_comp, is_cons, args);
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}
#endif

const char* ref_last_error(void) { return g_err.c_str(); }
}
