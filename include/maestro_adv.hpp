// maestro_adv.hpp -- a Maestro-shaped C++ layer over the C ABI of maestro_adv.h.
//
// A code that keeps the reference's call chain (Maestro::AdvanceTimeStep calling
// AdvancePremac, Addw0, DensityAdvance, EnthalpyAdvance, and inside them MakeEdgeScal and
// UpdateScal) calls the member functions below with the reference's argument lists
// (Source/Maestro.H:189, 499, 566, 913, 306 and Source/MaestroFill3dData.cpp:357).  The
// MultiFab here stands in for amrex::MultiFab: one device FAB per box in BoxArray order,
// Fortran ordered (i fastest), one block per component, over the box grown by the ghost
// width (nodal in one direction for face data), i.e. what amrex::FArrayBox::dataPtr() /
// box() / nComp() describe; an AMReX build maps its own MultiFab the same way and needs no
// copy.
//
// Implicit inputs are the context's, as the reference reads them from Maestro members: dt,
// rel_eps, the boundary conditions, the base state (with w0 and the face quantities built
// from it: w0mac, w0_force_cart, rho0_predicted_edge, p0_cart), the state members uold,
// sold, gpi.  Arguments the reference passes for those are accepted and not read.
// Errors raise std::runtime_error with madv_last_error() (the reference aborts).
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "maestro_adv.h"

namespace madvx {

template <class T>
using Vector = std::vector<T>;
// BaseState<Real>: the 1-D radial arrays; the stage reads the context's copy
template <class T>
using BaseState = std::vector<T>;

struct Box {
    int lo[3];
    int hi[3];
};
using BoxArray = std::vector<Box>;

inline void check(int rc) {
    if (rc != MADV_OK) throw std::runtime_error(std::string("maestro_adv: ") + madv_last_error());
}
inline void check_cuda(cudaError_t e) {
    if (e != cudaSuccess) throw std::runtime_error(std::string("CUDA: ") + cudaGetErrorString(e));
}

// One level's MultiFab: device FABs over the boxes grown by ngrow (nodal in direction
// `nodal` when >= 0), ncomp components each, in one allocation.
class MultiFab {
  public:
    MultiFab() = default;
    MultiFab(const BoxArray& ba, int ncomp, int ngrow, int nodal = -1) { define(ba, ncomp, ngrow, nodal); }
    MultiFab(const MultiFab&) = delete;
    MultiFab& operator=(const MultiFab&) = delete;
    MultiFab(MultiFab&& o) noexcept { *this = std::move(o); }
    MultiFab& operator=(MultiFab&& o) noexcept {
        std::swap(base_, o.base_);
        std::swap(fabs_, o.fabs_);
        std::swap(ncomp_, o.ncomp_);
        std::swap(ngrow_, o.ngrow_);
        std::swap(nodal_, o.nodal_);
        std::swap(ba_, o.ba_);
        return *this;
    }
    ~MultiFab() {
        if (base_) cudaFree(base_);
    }

    void define(const BoxArray& ba, int ncomp, int ngrow, int nodal = -1) {
        ba_ = ba;
        ncomp_ = ncomp;
        ngrow_ = ngrow;
        nodal_ = nodal;
        fabs_.assign(ba.size(), madv_fab{});
        size_t total = 0;
        std::vector<size_t> off(ba.size());
        for (size_t b = 0; b < ba.size(); ++b) {
            madv_fab& f = fabs_[b];
            for (int d = 0; d < 3; ++d) {
                f.lo[d] = ba[b].lo[d] - ngrow;
                f.hi[d] = ba[b].hi[d] + ngrow + (d == nodal ? 1 : 0);
            }
            f.ncomp = ncomp;
            off[b] = total;
            total += npts(f) * (size_t)ncomp;
        }
        if (base_) cudaFree(base_);
        base_ = nullptr;
        check_cuda(cudaMalloc(&base_, total * sizeof(double) + 16));
        for (size_t b = 0; b < ba.size(); ++b) fabs_[b].p = base_ + off[b];
    }
    // every value (ghost cells included) set to zero
    void setVal0(cudaStream_t st = nullptr) {
        size_t n = 0;
        for (auto& f : fabs_) n += npts(f) * (size_t)ncomp_;
        check_cuda(cudaMemsetAsync(base_, 0, n * sizeof(double), st));
    }
    madv_multifab view() const { return madv_multifab{(int)fabs_.size(), fabs_.data()}; }
    int nComp() const { return ncomp_; }
    int nGrow() const { return ngrow_; }
    const std::vector<madv_fab>& fabs() const { return fabs_; }

    // host <-> device through a domain-sized array [ncomp][nz][ny][nx] (valid region only;
    // one more point in the nodal direction)
    void from_domain(const double* h, const int dom_n[3], cudaStream_t st = nullptr) {
        domain_copy(const_cast<double*>(h), dom_n, true, st);
    }
    void to_domain(double* h, const int dom_n[3], cudaStream_t st = nullptr) const {
        const_cast<MultiFab*>(this)->domain_copy(h, dom_n, false, st);
    }

  private:
    static size_t npts(const madv_fab& f) {
        return (size_t)(f.hi[0] - f.lo[0] + 1) * (f.hi[1] - f.lo[1] + 1) * (f.hi[2] - f.lo[2] + 1);
    }
    void domain_copy(double* h, const int dom_n[3], bool in, cudaStream_t st) {
        int dn[3] = {dom_n[0], dom_n[1], dom_n[2]};
        if (nodal_ >= 0) dn[nodal_] += 1;
        for (size_t b = 0; b < fabs_.size(); ++b) {
            const madv_fab& f = fabs_[b];
            const long fx = f.hi[0] - f.lo[0] + 1, fy = f.hi[1] - f.lo[1] + 1, fz = f.hi[2] - f.lo[2] + 1;
            int vlo[3], vhi[3];
            for (int d = 0; d < 3; ++d) {
                vlo[d] = ba_[b].lo[d];
                vhi[d] = ba_[b].hi[d] + (d == nodal_ ? 1 : 0);
            }
            const size_t w = (size_t)(vhi[0] - vlo[0] + 1) * sizeof(double);
            for (int n = 0; n < ncomp_; ++n)
                for (int k = vlo[2]; k <= vhi[2]; ++k)
                    for (int j = vlo[1]; j <= vhi[1]; ++j) {
                        double* dev =
                            f.p + (((long)n * fz + (k - f.lo[2])) * fy + (j - f.lo[1])) * fx + (vlo[0] - f.lo[0]);
                        double* host = h + (((long)n * dn[2] + k) * dn[1] + j) * dn[0] + vlo[0];
                        check_cuda(in ? cudaMemcpyAsync(dev, host, w, cudaMemcpyHostToDevice, st)
                                      : cudaMemcpyAsync(host, dev, w, cudaMemcpyDeviceToHost, st));
                    }
        }
        check_cuda(cudaStreamSynchronize(st));
    }

    double* base_ = nullptr;
    std::vector<madv_fab> fabs_;
    int ncomp_ = 0, ngrow_ = 0, nodal_ = -1;
    BoxArray ba_;
};

using FaceMultiFabs = std::array<MultiFab, 3>;

inline std::array<madv_multifab, 3> views(const FaceMultiFabs& f) { return {f[0].view(), f[1].view(), f[2].view()}; }

// The stage's part of class Maestro: one level, 3-D.  Owns the context.
class Maestro {
  public:
    Maestro(const madv_params& p, const BoxArray& grids, const madv_base_state& bs, cudaStream_t st = nullptr)
        : params(p), stream(st), grids_(grids) {
        check(madv_ctx_create(&params, &ctx_));
        std::vector<madv_box> b(grids.size());
        for (size_t i = 0; i < grids.size(); ++i)
            for (int d = 0; d < 3; ++d) {
                b[i].lo[d] = grids[i].lo[d];
                b[i].hi[d] = grids[i].hi[d];
            }
        check(madv_set_layout(ctx_, (int)b.size(), b.data()));
        check(madv_set_base_state(ctx_, &bs));
    }
    ~Maestro() { madv_ctx_destroy(ctx_); }
    Maestro(const Maestro&) = delete;
    Maestro& operator=(const Maestro&) = delete;

    madv_params params;
    cudaStream_t stream;
    // the state members the stage reads (Source/Maestro.H:1855-2025)
    Vector<MultiFab> uold, sold, gpi;

    // Maestro::AdvancePremac (Source/MaestroAdvection.cpp:7-84)
    void AdvancePremac(Vector<FaceMultiFabs>& umac, const Vector<FaceMultiFabs>& w0mac,
                       const Vector<MultiFab>& w0_force_cart) {
        (void)w0mac;
        (void)w0_force_cart;
        const madv_multifab uo = uold[0].view(), so = sold[0].view(), gp = gpi[0].view();
        auto um = views(umac[0]);
        check(madv_advance_premac(ctx_, &uo, &so, &gp, um.data(), nullptr, stream));
    }
    // Maestro::Addw0 (Source/MaestroFill3dData.cpp:357-462)
    void Addw0(Vector<FaceMultiFabs>& u_edge, const Vector<FaceMultiFabs>& w0mac, const double& mult) {
        (void)w0mac;
        auto ue = views(u_edge[0]);
        check(madv_addw0(ctx_, ue.data(), mult, stream));
    }
    // Maestro::DensityAdvance (Source/MaestroDensityAdvance.cpp:6-243); scal_force is the
    // stage's own work array
    void DensityAdvance(int which_step, Vector<MultiFab>& scalold, Vector<MultiFab>& scalnew,
                        Vector<FaceMultiFabs>& sedge, Vector<FaceMultiFabs>& sflux, Vector<MultiFab>& scal_force,
                        Vector<MultiFab>& etarhoflux, Vector<FaceMultiFabs>& umac, const Vector<FaceMultiFabs>& w0mac,
                        const BaseState<double>& rho0_predicted_edge) {
        (void)scal_force;
        (void)w0mac;
        (void)rho0_predicted_edge;
        const madv_multifab so = scalold[0].view(), sn = scalnew[0].view(), eta = etarhoflux[0].view();
        auto se = views(sedge[0]), sf = views(sflux[0]), um = views(umac[0]);
        check(madv_density_advance(ctx_, which_step, &so, &sn, se.data(), sf.data(), &eta, um.data(), stream));
    }
    // Maestro::EnthalpyAdvance (Source/MaestroEnthalpyAdvance.cpp:6-352)
    void EnthalpyAdvance(int which_step, Vector<MultiFab>& scalold, Vector<MultiFab>& scalnew,
                         Vector<FaceMultiFabs>& sedge, Vector<FaceMultiFabs>& sflux, Vector<MultiFab>& scal_force,
                         Vector<FaceMultiFabs>& umac, const Vector<FaceMultiFabs>& w0mac,
                         const Vector<MultiFab>& thermal) {
        (void)scal_force;
        (void)w0mac;
        const madv_multifab so = scalold[0].view(), sn = scalnew[0].view(), th = thermal[0].view();
        auto se = views(sedge[0]), sf = views(sflux[0]), um = views(umac[0]);
        check(madv_enthalpy_advance(ctx_, which_step, &so, &sn, se.data(), sf.data(), um.data(), &th, stream));
    }
    // Maestro::MakeEdgeScal (Source/MaestroMakeEdgeScalars.cpp:6-302), scalars
    void MakeEdgeScal(Vector<MultiFab>& state, Vector<FaceMultiFabs>& sedge, Vector<FaceMultiFabs>& umac,
                      Vector<MultiFab>& force, const bool is_vel, int nbccomp, int start_scomp, int start_bccomp,
                      int num_comp, const bool is_conservative) {
        (void)nbccomp;
        const madv_multifab s = state[0].view(), f = force[0].view();
        auto se = views(sedge[0]), um = views(umac[0]);
        check(madv_make_edge_scal(ctx_, &s, se.data(), um.data(), &f, is_vel, start_scomp, start_bccomp, num_comp,
                                  is_conservative, stream));
    }
    // Maestro::UpdateScal (Source/MaestroAdvection.cpp:86-297); p0_cart is the context's p0
    void UpdateScal(const Vector<MultiFab>& stateold, Vector<MultiFab>& statenew, const Vector<FaceMultiFabs>& sflux,
                    const Vector<MultiFab>& force, int start_comp, int num_comp, const Vector<MultiFab>& p0_cart) {
        (void)p0_cart;
        const madv_multifab so = stateold[0].view(), sn = statenew[0].view(), f = force[0].view();
        auto sf = views(sflux[0]);
        check(madv_update_scal(ctx_, &so, &sn, sf.data(), &f, start_comp, num_comp, stream));
    }

    madv_ctx* ctx() const { return ctx_; }
    const BoxArray& grids() const { return grids_; }

  private:
    madv_ctx* ctx_ = nullptr;
    BoxArray grids_;
};

}  // namespace madvx
