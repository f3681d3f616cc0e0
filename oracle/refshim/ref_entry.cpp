// Test infrastructure only: C entry points into the reference's own stage functions,
// compiled unmodified from the reference sources against AMReX_shim.H / Maestro.H (see
// oracle/Makefile, target `ref`; the library goes to oracle/_ref/).  Used by tests/ to pin
// the oracle's restatement (and, through tests/golden/, the GPU library) to the reference.
#include <cstring>
#include <string>

#include "Maestro.H"

namespace maestro {
int ppm_type = 1;
int slope_order = 4;
}  // namespace maestro

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
        m.PPM(box_of(bx), arr<const Real>(s), arr<const Real>(u), arr<const Real>(v), arr<const Real>(w),
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
        if (d == 2) Maestro::Slopez(box_of(bx), sa, sl, box_of(dom), bcs, ncomp, 0);
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

const char* ref_last_error(void) { return g_err.c_str(); }
}
