// Test infrastructure only: types for the CPU oracle of the MAESTROeX scalar-advection
// stage.  Nothing in the product library includes this file; tests, smoke() and the
// cpu_baseline leg of bench.py load the oracle as the checker.
//
// Parity status: unpinned.  The reference stage cannot be compiled (its AMReX and
// Microphysics dependencies are empty submodules), and the reference ships no stage-level
// golden outputs.  The oracle restates the reference functions line by line instead; each
// function cites the reference file:line it follows.
//
// Box / Array4 / MultiFab semantics restated from the AMReX conventions the reference
// relies on (Fortran-order storage, i fastest, one contiguous block per component, face
// data stored on the box made nodal in the face direction, ghost cells by growing the box).
#pragma once
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef MO_TANGENT
#include "mo_dual.hpp"
#endif

namespace mo {

// The oracle's arithmetic type: double, or (tangent build) a value with its directional
// derivative.  Geometry, indices and parameters are plain numbers in either build.
#ifdef MO_TANGENT
using real = Dual;
#else
using real = double;
inline double value_of(double a) { return a; }
inline double tangent_of(double) { return 0.0; }
#endif
inline double fabs_r(double a) { return std::fabs(a); }
inline double copysign_r(double a, double b) { return std::copysign(a, b); }
inline double sqrt_r(double a) { return std::sqrt(a); }

// Reference state indices (Source/param/_variables:9-15, NumAux = 0).
enum { Rho = 0, RhoH = 1, Temp = 2, Pi = 3, FirstSpec = 4 };
// AMReX BCType values used by the reference (Source/MaestroSetup.cpp:276-500).
enum { reflect_odd = -1, int_dir = 0, reflect_even = 1, foextrap = 2, ext_dir = 3, hoextrap = 4 };
// AMReX PhysBCType values (inputs-file lo_bc/hi_bc integers).
enum { interior = 0, inflow = 1, outflow = 2, symmetry = 3, slipwall = 4, noslipwall = 5 };

// amrex::min / amrex::max (std::min / std::max semantics: first argument wins ties).
inline real mn(real a, real b) { return (b < a) ? b : a; }
inline real mx(real a, real b) { return (a < b) ? b : a; }
inline real cps(real a, real b) { return copysign_r(a, b); }
inline real fab(real a) { return fabs_r(a); }

struct Box {
    int lo[3];
    int hi[3];
};
inline Box grow(Box b, int n) {
    for (int d = 0; d < 3; ++d) { b.lo[d] -= n; b.hi[d] += n; }
    return b;
}
inline Box grow(Box b, int d, int n) { b.lo[d] -= n; b.hi[d] += n; return b; }
inline Box growLo(Box b, int d, int n) { b.lo[d] -= n; return b; }
inline Box growHi(Box b, int d, int n) { b.hi[d] += n; return b; }
inline Box nodal(Box b, int d) { b.hi[d] += 1; return b; }
inline bool contains(const Box& b, int i, int j, int k) {
    return i >= b.lo[0] && i <= b.hi[0] && j >= b.lo[1] && j <= b.hi[1] && k >= b.lo[2] &&
           k <= b.hi[2];
}

[[noreturn]] inline void bounds_fail(int i, int j, int k, int n, const int* lo, const int* hi, int nc) {
    char buf[256];
    std::snprintf(buf, sizeof(buf), "oracle index (%d,%d,%d,%d) outside [%d:%d,%d:%d,%d:%d] x %d", i, j,
                  k, n, lo[0], hi[0], lo[1], hi[1], lo[2], hi[2], nc);
    throw std::runtime_error(buf);
}

// Array4-like view: (i,j,k,n) with i fastest.
struct Arr {
    real* p = nullptr;
    int lo[3] = {0, 0, 0};
    int hi[3] = {-1, -1, -1};
    long sj = 0, sk = 0, sn = 0;
    int nc = 0;
    inline real& operator()(int i, int j, int k, int n = 0) const {
#ifdef MO_BOUNDS
        if (i < lo[0] || i > hi[0] || j < lo[1] || j > hi[1] || k < lo[2] || k > hi[2] || n < 0 ||
            n >= nc)
            bounds_fail(i, j, k, n, lo, hi, nc);
#endif
        return p[(long)(i - lo[0]) + (long)(j - lo[1]) * sj + (long)(k - lo[2]) * sk + (long)n * sn];
    }
    // array(mfi, comp): the same view starting at component c
    Arr comp(int c) const {
        Arr a = *this;
        a.p += (long)c * sn;
        a.nc -= c;
        return a;
    }
};

// MultiFab-like container: one Fortran-ordered FAB per box, ghost width ng, face
// direction ix (-1 = cell centred).
struct MF {
    std::vector<Box> ba;
    int nc = 0, ng = 0, ix = -1;
    std::vector<std::vector<real>> store;
    std::vector<Arr> a;
    void define(const std::vector<Box>& ba_, int nc_, int ng_, int ix_ = -1,
                real init = std::nan("")) {
        ba = ba_;
        nc = nc_;
        ng = ng_;
        ix = ix_;
        store.assign(ba.size(), {});
        a.assign(ba.size(), Arr{});
        for (size_t b = 0; b < ba.size(); ++b) {
            Box f = fabbox((int)b);
            long nx = f.hi[0] - f.lo[0] + 1, ny = f.hi[1] - f.lo[1] + 1, nz = f.hi[2] - f.lo[2] + 1;
            store[b].assign((size_t)(nx * ny * nz * nc), init);
            Arr& r = a[b];
            r.p = store[b].data();
            for (int d = 0; d < 3; ++d) { r.lo[d] = f.lo[d]; r.hi[d] = f.hi[d]; }
            r.sj = nx;
            r.sk = nx * ny;
            r.sn = nx * ny * nz;
            r.nc = nc;
        }
    }
    Box validbox(int b) const { return ix >= 0 ? nodal(ba[b], ix) : ba[b]; }
    Box fabbox(int b) const { return grow(validbox(b), ng); }
    int size() const { return (int)ba.size(); }
    const Arr& operator[](int b) const { return a[b]; }
    void setVal(real v) {
        for (auto& s : store) std::fill(s.begin(), s.end(), v);
    }
    void setVal(real v, int c0, int ncomp, int ngr) {
        for (int b = 0; b < size(); ++b) {
            Box bx = grow(validbox(b), ngr);
            const Arr& f = a[b];
            for (int n = c0; n < c0 + ncomp; ++n)
                for (int k = bx.lo[2]; k <= bx.hi[2]; ++k)
                    for (int j = bx.lo[1]; j <= bx.hi[1]; ++j)
                        for (int i = bx.lo[0]; i <= bx.hi[0]; ++i) f(i, j, k, n) = v;
        }
    }
};

struct BCRec {
    int lo[3];
    int hi[3];
};

#define MO_FOR3(bx)                                          \
    for (int k = (bx).lo[2]; k <= (bx).hi[2]; ++k)           \
        for (int j = (bx).lo[1]; j <= (bx).hi[1]; ++j)       \
            for (int i = (bx).lo[0]; i <= (bx).hi[0]; ++i)

}  // namespace mo
