// Test infrastructure only: a stand-in for the reference's Source/Maestro.H, declaring the
// part of class Maestro (member functions, members and runtime parameters) that the
// reference's stage sources compiled by oracle/Makefile (target `ref`) define or use, so
// that those sources compile unmodified against AMReX_shim.H.  The member function
// declarations have the reference's signatures (Source/Maestro.H:1396 PPM, :1576-1593
// Slopex/y/z), which a definition must match.
#ifndef REFSHIM_MAESTRO_H
#define REFSHIM_MAESTRO_H

#include "AMReX_shim.H"

// runtime parameters (the reference generates these from Source/param/_cpp_parameters into
// namespace maestro); the entry points of ref_entry.cpp set them before each call
namespace maestro {
extern int ppm_type;
extern int slope_order;
}  // namespace maestro
using namespace maestro;

class Maestro {
  public:
    amrex::Real dt = 0.0;
    amrex::Real rel_eps = 0.0;

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
