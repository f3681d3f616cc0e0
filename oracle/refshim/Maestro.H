// Test infrastructure only: a stand-in for the reference's Source/Maestro.H, declaring the
// part of class Maestro (member functions, members and runtime parameters) that the
// reference's stage sources compiled by oracle/Makefile (target `ref`) define or use, so
// that those sources compile unmodified against AMReX_shim.H.  The member function
// declarations have the reference's signatures (Source/Maestro.H:1396 PPM, :1576-1593
// Slopex/y/z), which a definition must match.
#ifndef REFSHIM_MAESTRO_H
#define REFSHIM_MAESTRO_H

#include "AMReX_shim.H"
#include <BaseState.H>
#include <BaseStateGeometry.H>


#include "maestro_params.H"
using namespace maestro;

// state component indices (the reference generates them from Source/param/_variables)
#ifndef REFSHIM_NUMSPEC
#define REFSHIM_NUMSPEC 3
#endif
constexpr int NumSpec = REFSHIM_NUMSPEC;
constexpr int NumAux = 0;
constexpr int Rho = 0, RhoH = 1, Temp = 2, Pi = 3, FirstSpec = 4, FirstAux = 4 + NumSpec;
constexpr int Nscal = 4 + NumSpec;

// the algorithm options of Source/Maestro.H:50-60
enum species_pred { predict_rhoprime_and_X = 1, predict_rhoX, predict_rho_and_X };
enum enthalpy_pred {
    predict_rhoh = 0,
    predict_rhohprime,
    predict_h,
    predict_T_then_rhohprime,
    predict_T_then_h,
    predict_hprime,
    predict_Tprime_then_h
};

// the equation of state (Microphysics, absent): the stage calls it only below the base
// cutoff density and for temperature predictions, which the comparisons never reach
enum eos_input_t { eos_input_rt = 1, eos_input_rh, eos_input_tp, eos_input_rp, eos_input_re, eos_input_ps, eos_input_ph, eos_input_th };
struct eos_t {
    amrex::Real rho = 0, T = 0, p = 0, e = 0, h = 0, s = 0, cs = 0, gam1 = 0, cp = 0, cv = 0, dpdr = 0, dedr = 0,
                dpdT = 0, dedT = 0, dhdr = 0, dhdT = 0;
    amrex::Real xn[NumSpec > 0 ? NumSpec : 1] = {};
    amrex::Real aux[1] = {};
};
using eos_rh_t = eos_t;
using eos_rep_t = eos_t;
using eos_re_t = eos_t;
using eos_rp_t = eos_t;
template <class S>
inline void eos(eos_input_t, S&) {
    amrex::Abort("equation of state not available in the reference build");
}

// Source/MaestroFill3dData.cpp:339 (declared in the reference's Maestro.H)
amrex::Real QuadInterp(const amrex::Real x, const amrex::Real x0, const amrex::Real x1, const amrex::Real x2,
                       const amrex::Real y0, const amrex::Real y1, const amrex::Real y2, const bool limit = true);

class Maestro {
  public:
    using A4 = amrex::Array4<amrex::Real>;
    using MF = amrex::MultiFab;
    using Box = amrex::Box;
    using Real = amrex::Real;
    using BCs = amrex::Vector<amrex::BCRec>;
    using DX = amrex::GpuArray<amrex::Real, AMREX_SPACEDIM>;
    using FaceMFs = amrex::Vector<std::array<amrex::MultiFab, AMREX_SPACEDIM>>;

  public:
    Real dt = 0.0;
    Real rel_eps = 0.0;
    int finest_level = 0;
    amrex::Vector<amrex::Geometry> geom;
    amrex::Vector<amrex::BoxArray> grids;
    amrex::Vector<amrex::DistributionMapping> dmap;

    // boundary conditions (Source/MaestroSetup.cpp:276-500 maps phys_bc onto them)
    amrex::BCRec phys_bc;
    BCs bcs_s, bcs_u, bcs_f;

    // Source/MaestroBCFill.cpp
    static void ScalarFill(const A4& scal, const Box& bx, const Box& domainBox, const Real* dx,
                           const amrex::BCRec bcs, const Real* gridlo, const int comp);
    static void VelFill(const A4& vel, const Box& bx, const Box& domainBox, const Real* dx, const amrex::BCRec bcs,
                        const Real* gridlo, const int comp = 0);
    static void FillExtBC(const A4& q, const Box& bx, const Box& domainBox, const Real* dx, const amrex::BCRec bcs,
                          const int comp, const bool is_vel = false);

    // Source/MaestroFillData.cpp
    void FillCoarsePatch(int lev, Real time, MF& mf, amrex::Vector<MF>& mf_old, amrex::Vector<MF>& mf_new,
                         int srccomp, int destcomp, int ncomp, const BCs& bcs, int variable_type = 0);
    void GetData(int lev, Real time, amrex::Vector<MF*>& mf, amrex::Vector<Real>& mftime, amrex::Vector<MF>& mf_old,
                 amrex::Vector<MF>& mf_new) const;
    void FillPatch(Real time, amrex::Vector<MF>& mf, amrex::Vector<MF>& mf_old, amrex::Vector<MF>& mf_new,
                   int srccomp, int destcomp, int ncomp, int startbccomp, const BCs& bcs_in, int variable_type = 0);
    void FillPatch(int lev, Real time, MF& mf, amrex::Vector<MF>& mf_old, amrex::Vector<MF>& mf_new, int srccomp,
                   int destcomp, int ncomp, int startbccomp, const BCs& bcs_in, int variable_type = 0);
    void AverageDown(amrex::Vector<MF>& mf, int comp, int ncomp);
    void AverageDownFaces(FaceMFs& edge);
    void FillUmacGhost(FaceMFs& umac_in, int level = -1);
    void FillPatchUedge(FaceMFs& uedge);

    using C4 = amrex::Array4<const amrex::Real>;
    amrex::Vector<MF> w0_cart;
    amrex::Vector<MF> normal;
    amrex::Vector<amrex::iMultiFab> cell_cc_to_r;
    BaseStateGeometry base_geom;
    BaseState<Real> w0;
    amrex::GpuArray<Real, 3> center;
    int max_level = 0;
    int max_radial_level = 0;
    Real t_old = 0.0, t_new = 0.0;
    amrex::Vector<MF> sold, snew, uold, unew;
    static amrex::IntVect nodal_flag, nodal_flag_x, nodal_flag_y, nodal_flag_z;
    static int ng_s;
    static constexpr Real Gconst = 6.67428e-8;  // Source/Maestro.H:1864
    int ng_adv = 3;
    BaseState<Real> rho0_old, rho0_new, rhoh0_old, rhoh0_new, p0_old, p0_new, tempbar, psi, grav_cell_old,
        grav_cell_new, w0_force, etarho_cc, etarho_ec;
    amrex::Vector<MF> gpi;
    amrex::Vector<std::unique_ptr<amrex::FluxRegister>> flux_reg_s;
    amrex::IntVect refRatio(int) const { return amrex::IntVect(2, 2, 2); }

    // Source/MaestroMakeGrav.cpp, Source/MaestroRhoHT.cpp
    void MakeGravCell(BaseState<Real>& grav_cell, const BaseState<Real>& rho0_s) const;
    void MakeGravEdge(BaseState<Real>& grav_edge_state, const BaseState<Real>& rho0_state) const;
    void HfromRhoTedge(FaceMFs& sedge, const BaseState<Real>& rho0_edge_old, const BaseState<Real>& rhoh0_edge_old,
                       const BaseState<Real>& rho0_edge_new, const BaseState<Real>& rhoh0_edge_new);

    // Source/MaestroFill3dData.cpp
    void Put1dArrayOnCart(const BaseState<Real>& s0, amrex::Vector<MF>& s0_cart, const bool is_input_edge_centered,
                          const bool is_output_a_vector, const BCs& bcs = BCs(), const int sbccomp = 0,
                          const int variable_type = 0);
    void Put1dArrayOnCart(const int level, const BaseState<Real>& s0, MF& s0_cart,
                          const bool is_input_edge_centered, const bool is_output_a_vector, const BCs& bcs = BCs(),
                          const int sbccomp = 0);
    void Put1dArrayOnCart(const int level, const BaseState<Real>& s0, amrex::Vector<MF>& s0_cart,
                          const bool is_input_edge_centered, const bool is_output_a_vector, const BCs& bcs = BCs(),
                          const int sbccomp = 0);
    void Addw0(FaceMFs& u_edge, const FaceMFs& w0mac, const Real& mult);
#if (AMREX_SPACEDIM == 3)
    void MakeW0mac(FaceMFs& w0mac);
    void MakeS0mac(const BaseState<Real>& s0, FaceMFs& s0mac);
#endif
    void MakeNormal();
    void PutDataOnFaces(const amrex::Vector<MF>& s_cc, FaceMFs& face, const bool harmonic_avg);
#if (AMREX_SPACEDIM == 3)
    void MakeCCtoRadii();
#endif

    // Source/MaestroBaseStateGeometry.cpp
#if (AMREX_SPACEDIM == 3)
    void InitBaseStateMapSphr(const int lev, const amrex::MFIter& mfi, const DX dx_fine, const DX dx_lev);
#endif
    void ComputeCutoffCoords(const BaseState<Real>& rho0_state) const;
    void RestrictBase(BaseState<Real>& s0, const bool is_cell_centered) const;
    void RestrictBase(const BaseStateArray<Real>& s0, const bool is_cell_centered) const;
    void FillGhostBase(BaseState<Real>& s0, const bool is_cell_centered) const;
    void FillGhostBase(const BaseStateArray<Real>& s0, const bool is_cell_centered) const;

    using VMF = amrex::Vector<MF>;
    using BS = BaseState<Real>;

    // Source/MaestroAdvection.cpp
    void AdvancePremac(FaceMFs& umac, const FaceMFs& w0mac, const VMF& w0_force_cart);
    void UpdateScal(const VMF& stateold, VMF& statenew, const FaceMFs& sflux, const VMF& force, int start_comp,
                    int num_comp, const VMF& p0_cart);
    void UpdateVel(const FaceMFs& umac, const FaceMFs& uedge, const VMF& force, const VMF& sponge,
                   const FaceMFs& w0mac);

    // Source/MaestroDensityAdvance.cpp, Source/MaestroEnthalpyAdvance.cpp, Source/MaestroVelocityAdvance.cpp
    void DensityAdvance(int which_step, VMF& scalold, VMF& scalnew, FaceMFs& sedge, FaceMFs& sflux, VMF& scal_force,
                        VMF& etarhoflux, FaceMFs& umac, const FaceMFs& w0mac, const BS& rho0_predicted_edge);
    void EnthalpyAdvance(int which_step, VMF& scalold, VMF& scalnew, FaceMFs& sedge, FaceMFs& sflux,
                         VMF& scal_force, FaceMFs& umac, const FaceMFs& w0mac, const VMF& thermal);
    void VelocityAdvance(const VMF& rhohalf, FaceMFs& umac, const FaceMFs& w0mac, const VMF& w0_force_cart,
                         const BS& rho0_nph, const BS& grav_cell_nph, const VMF& sponge);

    // Source/MaestroMakeFlux.cpp
    void MakeRhoXFlux(const VMF& state, FaceMFs& sflux, VMF& etarhoflux, FaceMFs& sedge, const FaceMFs& umac,
                      const BS& rho0_old_in, const BS& rho0_edge_old, const FaceMFs& r0mac_old, const BS& rho0_new_in,
                      const BS& rho0_edge_new, const FaceMFs& r0mac_new, const BS& rho0_predicted_edge,
                      int start_comp, int num_comp);
    void MakeRhoHFlux(const VMF& state, FaceMFs& sflux, FaceMFs& sedge, const FaceMFs& umac, const FaceMFs& w0mac,
                      const BS& rho0_old_in, const BS& rho0_edge_old, const FaceMFs& r0mac_old, const BS& rho0_new_in,
                      const BS& rho0_edge_new, const FaceMFs& r0mac_new, const BS& rhoh0_old_in,
                      const BS& rhoh0_edge_old, const FaceMFs& rh0mac_old, const BS& rhoh0_new_in,
                      const BS& rhoh0_edge_new, const FaceMFs& rh0mac_new, const FaceMFs& h0mac_old,
                      const FaceMFs& h0mac_new);

    // Source/MaestroForce.cpp
    void MakeVelForce(VMF& vel_force_cart, const FaceMFs& uedge_in, const VMF& rho, const BS& rho0,
                      const BS& grav_cell, const VMF& w0_force_cart, int do_add_utilde_force);
    void ModifyScalForce(VMF& scal_force, const VMF& state, const FaceMFs& umac_in, const BS& s0_edge,
                         const VMF& s0_cart, int comp, const BCs& bcs, int fullform);
    void MakeRhoHForce(VMF& scal_force, int is_prediction, const VMF& thermal, const FaceMFs& umac_cart,
                       int add_thermal, const int& which_step);
    void MakeTempForce(VMF& temp_force, const VMF& scal, const VMF& thermal, const FaceMFs& umac_in);

    // Source/MaestroConvert.cpp, Source/MaestroCelltoEdge.cpp
    void PutInPertForm(VMF& scal, const BS& s0, int comp, int bccomp, const BCs& bcs, bool flag);
    void PutInPertForm(int level, VMF& scal, const BS& s0, int comp, int bccomp, const BCs& bcs, bool flag);
    void ConvertRhoXToX(VMF& scal, bool flag);
    void ConvertRhoHToH(VMF& scal, bool flag);
    void CelltoEdge(const BS& s0_cell_in, BS& s0_edge_in) const;

    // Source/MaestroMakeUtrans.cpp
    void MakeUtrans(const amrex::Vector<MF>& utilde, const amrex::Vector<MF>& ufull, FaceMFs& utrans,
                    const FaceMFs& w0mac);

    // Source/MaestroVelPred.cpp
    void VelPred(amrex::Vector<MF>& utilde, const amrex::Vector<MF>& ufull, const FaceMFs& utrans, FaceMFs& umac,
                 const FaceMFs& w0mac, const amrex::Vector<MF>& force);
#if (AMREX_SPACEDIM == 2)
    void VelPredInterface(const amrex::MFIter& mfi, C4 utilde, C4 ufull, C4 utrans, C4 vtrans, C4 Imu, C4 Ipu,
                          C4 Imv, C4 Ipv, A4 ulx, A4 urx, A4 uimhx, A4 uly, A4 ury, A4 uimhy, const Box& domainBox,
                          const DX& dx) const;
    void VelPredVelocities(const amrex::MFIter& mfi, C4 utilde, C4 utrans, C4 vtrans, A4 umac, A4 vmac, C4 Imfx,
                           C4 Ipfx, C4 Imfy, C4 Ipfy, C4 ulx, C4 urx, C4 uimhx, C4 uly, C4 ury, C4 uimhy, C4 force,
                           C4 w0_cart_in, const Box& domainBox, const DX& dx) const;

#else
    void VelPredInterface(const amrex::MFIter& mfi, C4 utilde, C4 ufull, C4 utrans, C4 vtrans, C4 wtrans, C4 Imu,
                          C4 Ipu, C4 Imv, C4 Ipv, C4 Imw, C4 Ipw, A4 ulx, A4 urx, A4 uimhx, A4 uly, A4 ury,
                          A4 uimhy, A4 ulz, A4 urz, A4 uimhz, const Box& domainBox, const DX& dx) const;
    void VelPredTransverse(const amrex::MFIter& mfi, C4 utilde, C4 utrans, C4 vtrans, C4 wtrans, C4 ulx, C4 urx,
                           C4 uimhx, C4 uly, C4 ury, C4 uimhy, C4 ulz, C4 urz, C4 uimhz, A4 uimhyz, A4 uimhzy,
                           A4 vimhxz, A4 vimhzx, A4 wimhxy, A4 wimhyx, const Box& domainBox, const DX& dx) const;
    void VelPredVelocities(const amrex::MFIter& mfi, C4 utilde, C4 utrans, C4 vtrans, C4 wtrans, A4 umac, A4 vmac,
                           A4 wmac, C4 w0macx, C4 w0macy, C4 w0macz, C4 Imfx, C4 Ipfx, C4 Imfy, C4 Ipfy, C4 Imfz,
                           C4 Ipfz, C4 ulx, C4 urx, C4 uly, C4 ury, C4 ulz, C4 urz, C4 uimhyz, C4 uimhzy,
                           C4 vimhxz, C4 vimhzx, C4 wimhxy, C4 wimhyx, C4 force, C4 w0_cart_in,
                           const Box& domainBox, const DX& dx) const;
#endif

    // Source/MaestroMakeEdgeScalars.cpp
    void MakeEdgeScal(amrex::Vector<MF>& state, FaceMFs& sedge, FaceMFs& umac, amrex::Vector<MF>& force,
                      const bool is_vel, const BCs& bcs, int nbccomp, int start_scomp, int start_bccomp,
                      int num_comp, const bool is_conservative);
#if (AMREX_SPACEDIM == 2)
    void MakeEdgeScalPredictor(const amrex::MFIter& mfi, A4 slx, A4 srx, A4 sly, A4 sry, A4 scal, A4 Ip, A4 Im,
                               A4 umac, A4 vmac, A4 simhx, A4 simhy, const Box& domainBox, const BCs& bcs,
                               const DX dx, int comp, int bccomp, bool is_vel) const;
    void MakeEdgeScalEdges(const amrex::MFIter& mfi, A4 slx, A4 srx, A4 sly, A4 sry, A4 scal, A4 sedgex, A4 sedgey,
                           A4 force, A4 umac, A4 vmac, A4 Ipf, A4 Imf, A4 simhx, A4 simhy, const Box& domainBox,
                           const BCs& bcs, const DX dx, int comp, int bccomp, const bool is_vel,
                           const bool is_conservative) const;
#else
    static void MakeDivU(const Box& bx, A4 divu, A4 umac, A4 vmac, A4 wmac, const DX dx);
    void MakeEdgeScalPredictor(const amrex::MFIter& mfi, A4 slx, A4 srx, A4 sly, A4 sry, A4 slz, A4 srz, A4 scal,
                               A4 Ip, A4 Im, A4 slopez, A4 umac, A4 vmac, A4 wmac, A4 simhx, A4 simhy, A4 simhz,
                               const Box& domainBox, const BCs& bcs, const DX dx, int comp, int bccomp,
                               const bool is_vel) const;
    void MakeEdgeScalTransverse(const amrex::MFIter& mfi, A4 slx, A4 srx, A4 sly, A4 sry, A4 slz, A4 srz, A4 scal,
                                A4 divu, A4 umac, A4 vmac, A4 wmac, A4 simhx, A4 simhy, A4 simhz, A4 simhxy,
                                A4 simhxz, A4 simhyx, A4 simhyz, A4 simhzx, A4 simhzy, const Box& domainBox,
                                const BCs& bcs, const DX dx, int comp, int bccomp, const bool is_vel,
                                const bool is_conservative) const;
    void MakeEdgeScalEdges(const amrex::MFIter& mfi, A4 slx, A4 srx, A4 sly, A4 sry, A4 slz, A4 srz, A4 scal,
                           A4 sedgex, A4 sedgey, A4 sedgez, A4 force, A4 umac, A4 vmac, A4 wmac, A4 Ipf, A4 Imf,
                           A4 simhxy, A4 simhxz, A4 simhyx, A4 simhyz, A4 simhzx, A4 simhzy, const Box& domainBox,
                           const BCs& bcs, const DX dx, int comp, int bccomp, const bool is_vel,
                           const bool is_conservative) const;

#endif

    void PPM(const amrex::Box& bx, amrex::Array4<const amrex::Real> const s,
             amrex::Array4<const amrex::Real> const u, amrex::Array4<const amrex::Real> const v,
#if (AMREX_SPACEDIM == 3)
             amrex::Array4<const amrex::Real> const w,
#endif
             amrex::Array4<amrex::Real> const Ip, amrex::Array4<amrex::Real> const Im,
             const amrex::Box& domainBox, const amrex::Vector<amrex::BCRec>& bcs,
             const amrex::GpuArray<amrex::Real, AMREX_SPACEDIM> dx, const bool is_umac, const int comp,
             const int bccomp) const;

    static void Slopex(const amrex::Box& bx, amrex::Array4<amrex::Real> const s,
                       amrex::Array4<amrex::Real> const slx, const amrex::Box& domainBox,
                       const amrex::Vector<amrex::BCRec>& bcs, int ncomp, int bc_start_comp);
    static void Slopey(const amrex::Box& bx, amrex::Array4<amrex::Real> const s,
                       amrex::Array4<amrex::Real> const sly, const amrex::Box& domainBox,
                       const amrex::Vector<amrex::BCRec>& bcs, int ncomp, int bc_start_comp);
#if (AMREX_SPACEDIM == 3)
    static void Slopez(const amrex::Box& bx, amrex::Array4<amrex::Real> const s,
                       amrex::Array4<amrex::Real> const slz, const amrex::Box& domainBox,
                       const amrex::Vector<amrex::BCRec>& bcs, int ncomp, int bc_start_comp);
#endif
};

#endif
