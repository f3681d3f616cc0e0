// Test infrastructure only (the checker's checker): the few AMReX containers and helpers
// that the reference's own stage sources use, written here so that those sources compile
// unmodified on the CPU (AMReX itself is an empty submodule of the reference).  Nothing
// in the product library includes this file.
//
// Semantics restated from AMReX's public documentation: a Box is an index range
// [lo, hi] with a cell / node type per direction; Array4 indexes a Fortran-ordered FAB,
// component blocks contiguous; ParallelFor on the CPU runs k, j, i loops (i fastest);
// amrex::min / max are std::min / max; BCRec holds the BCType of the lo and hi face in
// each direction.
#ifndef REFSHIM_AMREX_H
#define REFSHIM_AMREX_H

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#ifndef AMREX_SPACEDIM
#define AMREX_SPACEDIM 3
#endif
#define AMREX_GPU_DEVICE
#define AMREX_GPU_HOST
#define AMREX_GPU_HOST_DEVICE
#define AMREX_FORCE_INLINE inline
#define AMREX_INLINE inline
#define AMREX_RESTRICT __restrict__
#define AMREX_GPU_MANAGED
#define BL_PROFILE_VAR(a, b)
#define BL_PROFILE_VAR_STOP(a)
#define BL_PROFILE(a)
#define AMREX_ASSERT(x) ((void)0)
#define AMREX_ALWAYS_ASSERT(x)                                                       \
    do {                                                                             \
        if (!(x)) throw std::runtime_error("assertion failed: " #x);                 \
    } while (0)
#define AMREX_PARALLEL_FOR_1D(n, i, block)   \
    for (long i = 0; i < (long)(n); ++i) block
#if AMREX_SPACEDIM == 2
#define AMREX_D_TERM(a, b, c) a b
#define AMREX_D_DECL(a, b, c) a, b
#else
#define AMREX_D_TERM(a, b, c) a b c
#define AMREX_D_DECL(a, b, c) a, b, c
#endif

namespace amrex {

using Real = double;
// amrex::Vector: a std::vector with dataPtr()
template <class T>
class Vector : public std::vector<T> {
  public:
    using std::vector<T>::vector;
    T* dataPtr() { return this->data(); }
    const T* dataPtr() const { return this->data(); }
};

// std::cout-like sink for amrex::Print (the stand-in prints nothing)
struct Print {
    template <class T>
    Print& operator<<(const T&) {
        return *this;
    }
    Print& operator<<(std::ostream& (*)(std::ostream&)) { return *this; }
};

[[noreturn]] inline void Abort(const std::string& msg = "") { throw std::runtime_error("amrex::Abort: " + msg); }
[[noreturn]] inline void Error(const std::string& msg = "") { throw std::runtime_error("amrex::Error: " + msg); }
template <class... T>
inline void ignore_unused(const T&...) {}

template <class T, int N>
struct GpuArray {
    T arr[N];
    T& operator[](int i) { return arr[i]; }
    const T& operator[](int i) const { return arr[i]; }
    T* data() { return arr; }
    const T* data() const { return arr; }
};

struct Dim3 {
    int x, y, z;
};

class IntVect {
  public:
    int v[3] = {0, 0, 0};
    IntVect() = default;
    IntVect(int a, int b, int c) : v{a, b, c} {}
    int& operator[](int d) { return v[d]; }
    const int& operator[](int d) const { return v[d]; }
    const int* getVect() const { return v; }
};

namespace IndexType_ {
}

class Box {
  public:
    int lo[3] = {0, 0, 0};
    int hi[3] = {-1, -1, -1};
    int typ[3] = {0, 0, 0};  // 0 cell-centred, 1 nodal
    Box() = default;
    Box(const IntVect& l, const IntVect& h) {
        for (int d = 0; d < 3; ++d) {
            lo[d] = l[d];
            hi[d] = h[d];
        }
    }
    const int* loVect() const { return lo; }
    const int* hiVect() const { return hi; }
    GpuArray<int, 3> loVect3d() const { return {{lo[0], lo[1], lo[2]}}; }
    GpuArray<int, 3> hiVect3d() const { return {{hi[0], hi[1], hi[2]}}; }
    IntVect smallEnd() const { return IntVect(lo[0], lo[1], lo[2]); }
    IntVect bigEnd() const { return IntVect(hi[0], hi[1], hi[2]); }
    int smallEnd(int d) const { return lo[d]; }
    int bigEnd(int d) const { return hi[d]; }
    int length(int d) const { return hi[d] - lo[d] + 1; }
    bool ok() const { return hi[0] >= lo[0] && hi[1] >= lo[1] && hi[2] >= lo[2]; }
    bool contains(int i, int j, int k) const {
        return i >= lo[0] && i <= hi[0] && j >= lo[1] && j <= hi[1] && k >= lo[2] && k <= hi[2];
    }
    long numPts() const { return ok() ? (long)length(0) * length(1) * length(2) : 0; }
    Box& grow(int n) {
        for (int d = 0; d < AMREX_SPACEDIM; ++d) {
            lo[d] -= n;
            hi[d] += n;
        }
        return *this;
    }
    Box& grow(int d, int n) {
        lo[d] -= n;
        hi[d] += n;
        return *this;
    }
    Box& growLo(int d, int n) {
        lo[d] -= n;
        return *this;
    }
    Box& growHi(int d, int n) {
        hi[d] += n;
        return *this;
    }
    Box& surroundingNodes(int d) {
        if (!typ[d]) {
            typ[d] = 1;
            hi[d] += 1;
        }
        return *this;
    }
    Box& surroundingNodes() {
        for (int d = 0; d < AMREX_SPACEDIM; ++d) surroundingNodes(d);
        return *this;
    }
    Box& enclosedCells(int d) {
        if (typ[d]) {
            typ[d] = 0;
            hi[d] -= 1;
        }
        return *this;
    }
    Box& enclosedCells() {
        for (int d = 0; d < AMREX_SPACEDIM; ++d) enclosedCells(d);
        return *this;
    }
    Box& setSmall(int d, int v) {
        lo[d] = v;
        return *this;
    }
    Box& setBig(int d, int v) {
        hi[d] = v;
        return *this;
    }
    bool operator==(const Box& o) const {
        for (int d = 0; d < 3; ++d)
            if (lo[d] != o.lo[d] || hi[d] != o.hi[d] || typ[d] != o.typ[d]) return false;
        return true;
    }
};

inline Box grow(Box b, int n) { return b.grow(n); }
inline Box grow(Box b, const IntVect& v) {
    for (int d = 0; d < AMREX_SPACEDIM; ++d) b.grow(d, v[d]);
    return b;
}
inline Box grow(Box b, int d, int n) { return b.grow(d, n); }
inline Box growLo(Box b, int d, int n) { return b.growLo(d, n); }
inline Box growHi(Box b, int d, int n) { return b.growHi(d, n); }
inline Box surroundingNodes(Box b, int d) { return b.surroundingNodes(d); }
inline Box surroundingNodes(Box b) { return b.surroundingNodes(); }
inline Box enclosedCells(Box b) { return b.enclosedCells(); }
inline Dim3 lbound(const Box& b) { return {b.lo[0], b.lo[1], b.lo[2]}; }
inline Dim3 ubound(const Box& b) { return {b.hi[0], b.hi[1], b.hi[2]}; }

namespace BCType {
enum mathematicalBndryTypes : int {
    bogus = -666,
    reflect_odd = -1,
    int_dir = 0,
    reflect_even = 1,
    foextrap = 2,
    ext_dir = 3,
    hoextrap = 4,
    hoextrapcc = 5,
    user_1 = 1001,
    user_2 = 1002,
    user_3 = 1003
};
}

namespace PhysBCType {
enum physicalBndryTypes : int { interior = 0, inflow, outflow, symmetry, slipwall, noslipwall };
}

class BCRec {
  public:
    int bc[6] = {0, 0, 0, 0, 0, 0};
    BCRec() = default;
    const int* lo() const { return bc; }
    const int* hi() const { return bc + 3; }
    int lo(int d) const { return bc[d]; }
    int hi(int d) const { return bc[3 + d]; }
    void setLo(int d, int v) { bc[d] = v; }
    void setHi(int d, int v) { bc[3 + d] = v; }
};

namespace Math {
template <class T>
inline T abs(T x) {
    return std::abs(x);
}
inline double copysign(double a, double b) { return std::copysign(a, b); }
inline double round(double x) { return std::round(x); }
inline double sqrt(double x) { return std::sqrt(x); }
inline double powi2(double x) { return x * x; }
}  // namespace Math

template <class T>
inline const T& min(const T& a, const T& b) {
    return std::min(a, b);
}
template <class T>
inline const T& max(const T& a, const T& b) {
    return std::max(a, b);
}
template <class T, class... Ts>
inline T min(const T& a, const T& b, const Ts&... rest) {
    return min(min(a, b), rest...);
}
template <class T, class... Ts>
inline T max(const T& a, const T& b, const Ts&... rest) {
    return max(max(a, b), rest...);
}

template <class T>
struct Array4 {
    T* p = nullptr;
    long jstride = 0, kstride = 0, nstride = 0;
    Dim3 begin{0, 0, 0}, end{0, 0, 0};  // end exclusive
    int ncomp = 0;
    Array4() = default;
    Array4(T* ptr, Dim3 lo, Dim3 hi_excl, int nc) : p(ptr), begin(lo), end(hi_excl), ncomp(nc) {
        jstride = end.x - begin.x;
        kstride = jstride * (end.y - begin.y);
        nstride = kstride * (end.z - begin.z);
    }
    template <class U, class = typename std::enable_if<std::is_same<const U, T>::value>::type>
    Array4(const Array4<U>& o)
        : p(o.p), jstride(o.jstride), kstride(o.kstride), nstride(o.nstride), begin(o.begin), end(o.end),
          ncomp(o.ncomp) {}
    T& operator()(int i, int j, int k) const { return at(i, j, k, 0); }
    T& operator()(int i, int j, int k, int n) const { return at(i, j, k, n); }
    T& at(int i, int j, int k, int n) const {
#ifdef REFSHIM_BOUNDS
        if (i < begin.x || i >= end.x || j < begin.y || j >= end.y || k < begin.z || k >= end.z || n < 0 ||
            n >= ncomp) {
            char b[200];
            std::snprintf(b, sizeof b, "Array4 index (%d,%d,%d,%d) outside [%d,%d)x[%d,%d)x[%d,%d) nc %d", i, j, k,
                          n, begin.x, end.x, begin.y, end.y, begin.z, end.z, ncomp);
            throw std::out_of_range(b);
        }
#endif
        return p[(i - begin.x) + (j - begin.y) * jstride + (k - begin.z) * kstride + n * nstride];
    }
    bool contains(int i, int j, int k) const {
        return i >= begin.x && i < end.x && j >= begin.y && j < end.y && k >= begin.z && k < end.z;
    }
    int nComp() const { return ncomp; }
};

template <class T>
class AsyncArray {
    std::vector<T> v_;

  public:
    AsyncArray(const T* p, std::size_t n) : v_(p, p + n) {}
    T* data() { return v_.data(); }
};

template <class F>
inline void ParallelFor(const Box& bx, F&& f) {
    for (int k = bx.lo[2]; k <= bx.hi[2]; ++k)
        for (int j = bx.lo[1]; j <= bx.hi[1]; ++j)
            for (int i = bx.lo[0]; i <= bx.hi[0]; ++i) f(i, j, k);
}

template <class F>
inline void ParallelFor(const Box& bx, int ncomp, F&& f) {
    for (int n = 0; n < ncomp; ++n)
        for (int k = bx.lo[2]; k <= bx.hi[2]; ++k)
            for (int j = bx.lo[1]; j <= bx.hi[1]; ++j)
                for (int i = bx.lo[0]; i <= bx.hi[0]; ++i) f(i, j, k, n);
}

class BoxArray {
    std::vector<Box> b_;

  public:
    BoxArray() = default;
    explicit BoxArray(std::vector<Box> b) : b_(std::move(b)) {}
    int size() const { return (int)b_.size(); }
    const Box& operator[](int i) const { return b_[i]; }
    Box get(int i) const { return b_[i]; }
    bool empty() const { return b_.empty(); }
    void push_back(const Box& b) { b_.push_back(b); }
};

// index type flags (1 = nodal in that direction)
inline BoxArray convert(const BoxArray& ba, const IntVect& typ) {
    std::vector<Box> out;
    for (int i = 0; i < ba.size(); ++i) {
        Box b = ba[i];
        for (int d = 0; d < 3; ++d) {
            if (typ[d] && !b.typ[d]) b.surroundingNodes(d);
            if (!typ[d] && b.typ[d]) b.enclosedCells(d);
        }
        out.push_back(b);
    }
    return BoxArray(out);
}

class DistributionMapping {
  public:
    DistributionMapping() = default;
    explicit DistributionMapping(const BoxArray&) {}
};

class Periodicity {
  public:
    bool per[3] = {false, false, false};
};

class RealBox {
  public:
    Real lo_[3] = {0, 0, 0}, hi_[3] = {0, 0, 0};
    const Real* lo() const { return lo_; }
    const Real* hi() const { return hi_; }
    Real lo(int d) const { return lo_[d]; }
    Real hi(int d) const { return hi_[d]; }
};

class Geometry {
  public:
    Box domain;
    Real dx_[3] = {1, 1, 1};
    RealBox rb;
    bool per[3] = {false, false, false};
    const Box& Domain() const { return domain; }
    const Real* CellSize() const { return dx_; }
    Real CellSize(int d) const { return dx_[d]; }
    GpuArray<Real, AMREX_SPACEDIM> CellSizeArray() const {
        GpuArray<Real, AMREX_SPACEDIM> a;
        for (int d = 0; d < AMREX_SPACEDIM; ++d) a[d] = dx_[d];
        return a;
    }
    GpuArray<Real, AMREX_SPACEDIM> InvCellSizeArray() const {
        GpuArray<Real, AMREX_SPACEDIM> a;
        for (int d = 0; d < AMREX_SPACEDIM; ++d) a[d] = 1.0 / dx_[d];
        return a;
    }
    const Real* ProbLo() const { return rb.lo_; }
    const Real* ProbHi() const { return rb.hi_; }
    Real ProbLo(int d) const { return rb.lo_[d]; }
    Real ProbHi(int d) const { return rb.hi_[d]; }
    GpuArray<Real, AMREX_SPACEDIM> ProbLoArray() const {
        GpuArray<Real, AMREX_SPACEDIM> a;
        for (int d = 0; d < AMREX_SPACEDIM; ++d) a[d] = rb.lo_[d];
        return a;
    }
    GpuArray<Real, AMREX_SPACEDIM> ProbHiArray() const {
        GpuArray<Real, AMREX_SPACEDIM> a;
        for (int d = 0; d < AMREX_SPACEDIM; ++d) a[d] = rb.hi_[d];
        return a;
    }
    const RealBox& ProbDomain() const { return rb; }
    bool isPeriodic(int d) const { return per[d]; }
    bool isAnyPeriodic() const { return per[0] || per[1] || per[2]; }
    Periodicity periodicity() const {
        Periodicity p;
        for (int d = 0; d < 3; ++d) p.per[d] = per[d];
        return p;
    }
};

class MFIter;

// One FAB per box: the box grown by the ghost width (typed like the BoxArray), ncomp
// components, Fortran order, one contiguous block per component.  Either owned storage
// (define) or a caller's buffer (alias).
template <class T>
class FabArrayOf {
  public:
    using MultiFab = FabArrayOf<T>;
    using Real = T;
    struct Fab {
        Box box;
        T* p = nullptr;
        std::vector<T> own;
    };
    BoxArray ba_;
    int nc_ = 0, ng_ = 0;
    std::vector<Fab> fabs_;

    FabArrayOf() = default;
    FabArrayOf(const BoxArray& ba, const DistributionMapping& dm, int nc, int ng) { define(ba, dm, nc, ng); }
    FabArrayOf(const FabArrayOf&) = delete;
    FabArrayOf& operator=(const FabArrayOf&) = delete;
    FabArrayOf(FabArrayOf&&) = default;
    FabArrayOf& operator=(FabArrayOf&&) = default;

    void define(const BoxArray& ba, const DistributionMapping&, int nc, int ng) {
        ba_ = ba;
        nc_ = nc;
        ng_ = ng;
        fabs_.clear();
        fabs_.resize(ba.size());
        for (int i = 0; i < ba.size(); ++i) {
            Fab& f = fabs_[i];
            f.box = grow(ba[i], ng);
            f.own.assign((std::size_t)f.box.numPts() * nc, std::is_floating_point<T>::value ? T(NAN) : T(-99999));
            f.p = f.own.data();
        }
    }
    // wraps caller buffers (one per box, each covering ba[i] grown by ng)
    void alias(const BoxArray& ba, int nc, int ng, const std::vector<T*>& ptrs) {
        ba_ = ba;
        nc_ = nc;
        ng_ = ng;
        fabs_.clear();
        fabs_.resize(ba.size());
        for (int i = 0; i < ba.size(); ++i) {
            fabs_[i].box = grow(ba[i], ng);
            fabs_[i].p = ptrs[i];
        }
    }
    bool ok() const { return !fabs_.empty(); }
    int nGrow() const { return ng_; }
    IntVect nGrowVect() const { return IntVect(ng_, ng_, ng_); }
    int nComp() const { return nc_; }
    int size() const { return (int)fabs_.size(); }
    const BoxArray& boxArray() const { return ba_; }
    DistributionMapping DistributionMap() const { return DistributionMapping(); }
    Array4<T> array(int i) const {
        const Box& b = fabs_[i].box;
        return Array4<T>(fabs_[i].p, Dim3{b.lo[0], b.lo[1], b.lo[2]}, Dim3{b.hi[0] + 1, b.hi[1] + 1, b.hi[2] + 1},
                         nc_);
    }
    Array4<const T> const_array(int i) const { return Array4<const T>(array(i)); }
    inline Array4<T> array(const MFIter& mfi) const;
    inline Array4<const T> const_array(const MFIter& mfi) const;

    void setVal(Real v) { setVal(v, 0, nc_, ng_); }
    void setVal(Real v, int ng) { setVal(v, 0, nc_, ng); }
    void setVal(Real v, int comp, int ncomp, int ng = 0) {
        for (int i = 0; i < size(); ++i) {
            Box b = grow(ba_[i], ng);
            auto a = array(i);
            ParallelFor(b, ncomp, [&](int x, int y, int z, int n) { a(x, y, z, comp + n) = v; });
        }
    }
    void setVal(Real v, int comp, int ncomp, const IntVect& ng) { setVal(v, comp, ncomp, ng[0]); }
    // ghost exchange between boxes and physical fills belong to AMReX and are left to the
    // caller: the stand-in keeps the data as it is (comparisons cover valid regions)
    void FillBoundary(const Periodicity&) {}
    void FillBoundary(int, int, const Periodicity&) {}
    void FillBoundary() {}

    template <class F>
    static void each(MultiFab& dst, int ng, int ncomp, F&& f) {
        for (int i = 0; i < dst.size(); ++i) {
            Box b = grow(dst.ba_[i], ng);
            ParallelFor(b, ncomp, [&](int x, int y, int z, int n) { f(i, x, y, z, n); });
        }
    }
    static void Copy(MultiFab& dst, const MultiFab& src, int scomp, int dcomp, int ncomp, int ng) {
        each(dst, ng, ncomp, [&](int i, int x, int y, int z, int n) {
            dst.array(i)(x, y, z, dcomp + n) = src.array(i)(x, y, z, scomp + n);
        });
    }
    static void Copy(MultiFab& dst, const MultiFab& src, int scomp, int dcomp, int ncomp, const IntVect& ng) {
        Copy(dst, src, scomp, dcomp, ncomp, ng[0]);
    }
    static void LinComb(MultiFab& dst, Real a, const MultiFab& x, int xcomp, Real b, const MultiFab& y, int ycomp,
                        int dcomp, int ncomp, int ng) {
        each(dst, ng, ncomp, [&](int i, int p, int q, int r, int n) {
            dst.array(i)(p, q, r, dcomp + n) = a * x.array(i)(p, q, r, xcomp + n) + b * y.array(i)(p, q, r, ycomp + n);
        });
    }
    static void Add(MultiFab& dst, const MultiFab& src, int scomp, int dcomp, int ncomp, int ng) {
        each(dst, ng, ncomp, [&](int i, int x, int y, int z, int n) {
            dst.array(i)(x, y, z, dcomp + n) += src.array(i)(x, y, z, scomp + n);
        });
    }
    static void Subtract(MultiFab& dst, const MultiFab& src, int scomp, int dcomp, int ncomp, int ng) {
        each(dst, ng, ncomp, [&](int i, int x, int y, int z, int n) {
            dst.array(i)(x, y, z, dcomp + n) -= src.array(i)(x, y, z, scomp + n);
        });
    }
    static void Multiply(MultiFab& dst, const MultiFab& src, int scomp, int dcomp, int ncomp, int ng) {
        each(dst, ng, ncomp, [&](int i, int x, int y, int z, int n) {
            dst.array(i)(x, y, z, dcomp + n) *= src.array(i)(x, y, z, scomp + n);
        });
    }
    static void Divide(MultiFab& dst, const MultiFab& src, int scomp, int dcomp, int ncomp, int ng) {
        each(dst, ng, ncomp, [&](int i, int x, int y, int z, int n) {
            dst.array(i)(x, y, z, dcomp + n) /= src.array(i)(x, y, z, scomp + n);
        });
    }
    void plus(Real v, int comp, int ncomp, int ng = 0) {
        each(*this, ng, ncomp, [&](int i, int x, int y, int z, int n) { array(i)(x, y, z, comp + n) += v; });
    }
    void mult(Real v, int comp, int ncomp, int ng = 0) {
        each(*this, ng, ncomp, [&](int i, int x, int y, int z, int n) { array(i)(x, y, z, comp + n) *= v; });
    }
};

class MFIter {
    const BoxArray* ba_;
    int ng_;
    int i_ = 0;

  public:
    template <class T>
    MFIter(const FabArrayOf<T>& mf, bool = false) : ba_(&mf.boxArray()), ng_(mf.nGrow()) {}
    bool isValid() const { return i_ < ba_->size(); }
    MFIter& operator++() {
        ++i_;
        return *this;
    }
    int index() const { return i_; }
    int LocalIndex() const { return i_; }
    Box validbox() const { return (*ba_)[i_]; }
    Box tilebox() const { return validbox(); }
    Box tilebox(const IntVect& nodal) const { return convert(BoxArray({validbox()}), nodal)[0]; }
    Box growntilebox(int ng) const { return grow(validbox(), ng); }
    Box growntilebox() const { return grow(validbox(), ng_); }
    Box fabbox() const { return grow(validbox(), ng_); }
    Box nodaltilebox(int d) const {
        Box b = validbox();
        return b.surroundingNodes(d);
    }
    Box grownnodaltilebox(int d, int ng) const {
        Box b = validbox();
        if (d >= 0) b.surroundingNodes(d);
        return b.grow(ng);
    }
};

template <class T>
inline Array4<T> FabArrayOf<T>::array(const MFIter& mfi) const {
    return array(mfi.index());
}
template <class T>
inline Array4<const T> FabArrayOf<T>::const_array(const MFIter& mfi) const {
    return const_array(mfi.index());
}
using MultiFab = FabArrayOf<Real>;
using iMultiFab = FabArrayOf<int>;
inline bool TilingIfNotGPU() { return false; }

namespace Gpu {
template <class T>
class ManagedVector : public std::vector<T> {
  public:
    using std::vector<T>::vector;
    T* dataPtr() { return this->data(); }
    const T* dataPtr() const { return this->data(); }
};
template <class T>
using DeviceVector = ManagedVector<T>;
template <class T>
using HostVector = ManagedVector<T>;
inline void synchronize() {}
inline void streamSynchronize() {}
inline bool notInLaunchRegion() { return true; }
inline bool inLaunchRegion() { return false; }
inline void setLaunchRegion(bool) {}
}  // namespace Gpu

}  // namespace amrex

#endif
