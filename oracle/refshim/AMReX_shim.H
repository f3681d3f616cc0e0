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
#include <memory>
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
#define BL_ASSERT(x) ((void)0)
#define BL_SPACEDIM AMREX_SPACEDIM
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
    IntVect(int a, int b) : v{a, b, 0} {}
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
    int bc[2 * AMREX_SPACEDIM] = {};  // lo[dim], hi[dim]; directions beyond dim read int_dir
    BCRec() = default;
    const int* lo() const { return bc; }
    const int* hi() const { return bc + AMREX_SPACEDIM; }
    int lo(int d) const { return d < AMREX_SPACEDIM ? bc[d] : 0; }
    int hi(int d) const { return d < AMREX_SPACEDIM ? bc[AMREX_SPACEDIM + d] : 0; }
    void setLo(int d, int v) {
        if (d < AMREX_SPACEDIM) bc[d] = v;
    }
    void setHi(int d, int v) {
        if (d < AMREX_SPACEDIM) bc[AMREX_SPACEDIM + d] = v;
    }
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
    explicit BoxArray(class BoxList&&);
    int size() const { return (int)b_.size(); }
    const Box& operator[](int i) const { return b_[i]; }
    Box get(int i) const { return b_[i]; }
    bool empty() const { return b_.empty(); }
    void push_back(const Box& b) { b_.push_back(b); }
    // used by the multi-level branches only (never reached with one level)
    BoxArray& maxSize(int) { return *this; }
    BoxArray& coarsen(const IntVect&) { Abort("stand-in BoxArray::coarsen: one level only"); }
    BoxArray& refine(const IntVect&) { Abort("stand-in BoxArray::refine: one level only"); }
    BoxArray& surroundingNodes(int d) {
        for (auto& b : b_) b.surroundingNodes(d);
        return *this;
    }
};

class BoxList {
  public:
    std::vector<Box> boxes;
};
inline BoxList GetBndryCells(const BoxArray&, int) { Abort("stand-in GetBndryCells: one level only"); }
inline BoxArray::BoxArray(BoxList&& bl) : b_(std::move(bl.boxes)) {}

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
    void KnapSackProcessorMap(const std::vector<long>&, int) {}
};

namespace ParallelDescriptor {
inline int NProcs() { return 1; }
inline int MyProc() { return 0; }
inline int IOProcessorNumber() { return 0; }
inline bool IOProcessor() { return true; }
}  // namespace ParallelDescriptor

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
    // the FAB's view from component c on (AMReX's array(mfi, start_comp))
    Array4<T> array(int i, int c) const {
        Array4<T> a = array(i);
        a.p += (long)c * a.nstride;
        a.ncomp -= c;
        return a;
    }
    inline Array4<T> array(const MFIter& mfi, int c) const;
    inline Array4<const T> const_array(const MFIter& mfi, int c) const;
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
    // Copies into the cells of dst box b grown by dst_ng (skipping b's own valid region when
    // ghosts_only) the values of every box c's region grown by src_ng of src, also through
    // the periodic images of src; boxes and shifts are visited in order (box, z, y, x shift)
    // and a later source overwrites an earlier one.
    static void copy_regions(FabArrayOf& dst, const FabArrayOf& src, int scomp, int dcomp, int ncomp, int src_ng,
                             int dst_ng, const Periodicity& per, const Box& dom, bool ghosts_only) {
        int len[3];
        for (int d = 0; d < 3; ++d) len[d] = dom.hi[d] - dom.lo[d] + 1;
        for (int b = 0; b < dst.size(); ++b) {
            const Box vb = dst.ba_[b];
            const Box gb = grow(vb, dst_ng);
            const auto D = dst.array(b);
            for (int c = 0; c < src.size(); ++c) {
                const Box sb = grow(src.ba_[c], src_ng);
                const auto S = src.array(c);
                for (int sz = -1; sz <= 1; ++sz)
                    for (int sy = -1; sy <= 1; ++sy)
                        for (int sx = -1; sx <= 1; ++sx) {
                            const int sh[3] = {sx, sy, sz};
                            bool ok = true;
                            for (int d = 0; d < 3; ++d)
                                if (sh[d] != 0 && !per.per[d]) ok = false;
                            if (!ok) continue;
                            if (ghosts_only && c == b && sx == 0 && sy == 0 && sz == 0) continue;
                            Box r;
                            bool empty = false;
                            for (int d = 0; d < 3; ++d) {
                                r.lo[d] = std::max(gb.lo[d], sb.lo[d] + sh[d] * len[d]);
                                r.hi[d] = std::min(gb.hi[d], sb.hi[d] + sh[d] * len[d]);
                                if (r.lo[d] > r.hi[d]) empty = true;
                            }
                            if (empty) continue;
                            ParallelFor(r, ncomp, [&](int i, int j, int k, int n) {
                                if (ghosts_only && vb.contains(i, j, k)) return;
                                D(i, j, k, dcomp + n) =
                                    S(i - sx * len[0], j - sy * len[1], k - sz * len[2], scomp + n);
                            });
                        }
            }
        }
    }
    // the level's domain (cell-centred) for the periodic images: set by the caller
    static Box& domain_for_fills() {
        static Box dom;
        return dom;
    }
    void FillBoundary(int scomp, int ncomp, int ng, const Periodicity& per) {
        copy_regions(*this, *this, scomp, scomp, ncomp, 0, ng, per, domain_for_fills(), true);
    }
    void FillBoundary(int scomp, int ncomp, const IntVect& ng, const Periodicity& per) {
        FillBoundary(scomp, ncomp, ng[0], per);
    }
    void FillBoundary(int scomp, int ncomp, const Periodicity& per) { FillBoundary(scomp, ncomp, ng_, per); }
    void FillBoundary(const Periodicity& per) { FillBoundary(0, nc_, ng_, per); }
    void ParallelCopy(const FabArrayOf& src, int scomp, int dcomp, int ncomp, int src_ng, int dst_ng,
                      const Periodicity& per = Periodicity()) {
        copy_regions(*this, src, scomp, dcomp, ncomp, src_ng, dst_ng, per, domain_for_fills(), false);
    }
    void ParallelCopy(const FabArrayOf& src, int scomp, int dcomp, int ncomp, const IntVect& src_ng,
                      const IntVect& dst_ng, const Periodicity& per = Periodicity()) {
        ParallelCopy(src, scomp, dcomp, ncomp, src_ng[0], dst_ng[0], per);
    }
    void ParallelCopy(const FabArrayOf& src) { ParallelCopy(src, 0, 0, nc_, 0, 0); }
    inline class FArrayBox operator[](const MFIter& mfi) const;
    void clear() {
        fabs_.clear();
        ba_ = BoxArray();
    }

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
template <class T>
inline Array4<T> FabArrayOf<T>::array(const MFIter& mfi, int c) const {
    return array(mfi.index(), c);
}
template <class T>
inline Array4<const T> FabArrayOf<T>::const_array(const MFIter& mfi, int c) const {
    return Array4<const T>(array(mfi.index(), c));
}
using MultiFab = FabArrayOf<Real>;
using iMultiFab = FabArrayOf<int>;

// one FAB of a MultiFab (a view: box incl. ghosts, components, data)
class FArrayBox {
  public:
    Box box_;
    int nc_ = 0;
    Real* p_ = nullptr;
    const Box& box() const { return box_; }
    const int* loVect() const { return box_.lo; }
    const int* hiVect() const { return box_.hi; }
    int nComp() const { return nc_; }
    Array4<Real> array(int c = 0) const {
        Array4<Real> a(p_, Dim3{box_.lo[0], box_.lo[1], box_.lo[2]},
                       Dim3{box_.hi[0] + 1, box_.hi[1] + 1, box_.hi[2] + 1}, nc_);
        a.p += (long)c * a.nstride;
        a.ncomp -= c;
        return a;
    }
};
template <class T>
inline FArrayBox FabArrayOf<T>::operator[](const MFIter& mfi) const {
    FArrayBox f;
    f.box_ = fabs_[mfi.index()].box;
    f.nc_ = nc_;
    f.p_ = fabs_[mfi.index()].p;
    return f;
}

// AMReX's generic physical-boundary fill of cell-centred data (fab_filcc) for the cells of
// bx outside the domain, direction by direction (x, then y, then z, each over the whole of
// bx in the other directions):
//   foextrap      the nearest interior value;
//   hoextrap      the first ghost cell takes the value at the face of the quadratic through
//                 the first three interior cells, (15 q0 - 10 q1 + 3 q2)/8 (linear,
//                 (3 q0 - q1)/2, with fewer than three), deeper ghost cells the nearest
//                 interior value;
//   reflect_even  the mirror image; reflect_odd the mirror image with its sign changed;
//   int_dir, ext_dir  left as they are (periodic images; Dirichlet data is the caller's).
inline void fab_filcc(const Box& bx, const Array4<Real>& q, int ncomp, const Box& dom, const Real*, const Real*,
                      const BCRec* bcr) {
    for (int n = 0; n < ncomp; ++n) {
        const BCRec& bc = bcr[n];
        for (int d = 0; d < AMREX_SPACEDIM; ++d) {
            const int dlo = dom.lo[d], dhi = dom.hi[d];
            for (int side = 0; side < 2; ++side) {
                const int t = side == 0 ? bc.lo(d) : bc.hi(d);
                if (t != BCType::foextrap && t != BCType::hoextrap && t != BCType::reflect_even &&
                    t != BCType::reflect_odd)
                    continue;
                Box r = bx;
                if (side == 0) r.hi[d] = std::min(bx.hi[d], dlo - 1);
                else r.lo[d] = std::max(bx.lo[d], dhi + 1);
                if (r.lo[d] > r.hi[d]) continue;
                ParallelFor(r, [&](int i, int j, int k) {
                    int idx[3] = {i, j, k};
                    const int m = idx[d];
                    auto at = [&](int pnt) {
                        int id2[3] = {i, j, k};
                        id2[d] = pnt;
                        return q(id2[0], id2[1], id2[2], n);
                    };
                    Real v;
                    if (t == BCType::foextrap) {
                        v = at(side == 0 ? dlo : dhi);
                    } else if (t == BCType::hoextrap) {
                        if (side == 0) {
                            if (m < dlo - 1) v = at(dlo);
                            else if (dlo + 2 <= std::min(bx.hi[d], dhi))
                                v = 0.125 * (15. * at(dlo) - 10. * at(dlo + 1) + 3. * at(dlo + 2));
                            else v = 0.5 * (3. * at(dlo) - at(dlo + 1));
                        } else {
                            if (m > dhi + 1) v = at(dhi);
                            else if (dhi - 2 >= std::max(bx.lo[d], dlo))
                                v = 0.125 * (15. * at(dhi) - 10. * at(dhi - 1) + 3. * at(dhi - 2));
                            else v = 0.5 * (3. * at(dhi) - at(dhi - 1));
                        }
                    } else if (t == BCType::reflect_even) {
                        v = at(side == 0 ? 2 * dlo - 1 - m : 2 * dhi + 1 - m);
                    } else {
                        v = -at(side == 0 ? 2 * dlo - 1 - m : 2 * dhi + 1 - m);
                    }
                    q(i, j, k, n) = v;
                });
            }
        }
    }
}

class BndryFuncArray {};

// physical-boundary fill of a MultiFab: the functor runs on every FAB whose box grown by
// nghost reaches outside the domain (grown in the periodic directions)
template <class F>
class PhysBCFunct {
    Geometry geom_;
    Vector<BCRec> bcr_;
    F f_;

  public:
    PhysBCFunct() = default;
    void define(const Geometry& g, const Vector<BCRec>& bcr, F f) {
        geom_ = g;
        bcr_ = bcr;
        f_ = f;
    }
    void operator()(MultiFab& mf, int dcomp, int ncomp, const IntVect& nghost, Real time, int bccomp) {
        Box gdom = geom_.Domain();
        for (int d = 0; d < AMREX_SPACEDIM; ++d)
            if (geom_.isPeriodic(d)) gdom.grow(d, nghost[d]);
        for (MFIter mfi(mf); mfi.isValid(); ++mfi) {
            Box gbx = grow(mfi.validbox(), nghost);
            Box gd = gdom;
            for (int d = 0; d < 3; ++d)
                if (gbx.typ[d]) gd.surroundingNodes(d);
            bool inside = true;
            for (int d = 0; d < 3; ++d)
                if (gbx.lo[d] < gd.lo[d] || gbx.hi[d] > gd.hi[d]) inside = false;
            if (inside) continue;
            FArrayBox dest = mf[mfi];
            f_(gbx, dest, dcomp, ncomp, geom_, time, bcr_, bccomp, dcomp);
        }
    }
};

class Interpolater {};
extern Interpolater cell_cons_interp;

// FillPatchSingleLevel on one time level: the components come from the valid regions of
// the source (through the periodic images) into mf's valid and ghost cells, then the
// physical boundary fill
template <class BC>
inline void FillPatchSingleLevel(MultiFab& mf, Real time, const Vector<MultiFab*>& smf, const Vector<Real>&,
                                 int scomp, int dcomp, int ncomp, const Geometry& geom, BC& physbc, int bccomp) {
    if (smf.size() != 1) Abort("stand-in FillPatchSingleLevel: one time level");
    const IntVect ng = mf.nGrowVect();
    if (smf[0] == &mf && scomp == dcomp) mf.FillBoundary(dcomp, ncomp, ng, geom.periodicity());
    else mf.ParallelCopy(*smf[0], scomp, dcomp, ncomp, IntVect(0, 0, 0), ng, geom.periodicity());
    physbc(mf, dcomp, ncomp, ng, time, bccomp);
}
template <class... A>
inline void FillPatchTwoLevels(A&&...) {
    Abort("stand-in FillPatchTwoLevels: one level only");
}
template <class... A>
inline void InterpFromCoarseLevel(A&&...) {
    Abort("stand-in InterpFromCoarseLevel: one level only");
}
template <class... A>
inline void average_down_faces(A&&...) {
    Abort("stand-in average_down_faces: one level only");
}
inline bool TilingIfNotGPU() { return false; }

template <class F>
inline void ParallelFor(long n, F&& f) {
    for (long i = 0; i < n; ++i) f((int)i);
}
template <class F1, class F2>
inline void ParallelFor(const Box& b1, const Box& b2, F1&& f1, F2&& f2) {
    ParallelFor(b1, f1);
    ParallelFor(b2, f2);
}
template <class F1, class F2, class F3>
inline void ParallelFor(const Box& b1, const Box& b2, const Box& b3, F1&& f1, F2&& f2, F3&& f3) {
    ParallelFor(b1, f1);
    ParallelFor(b2, f2);
    ParallelFor(b3, f3);
}

// coarse-fine flux registers: one level only here, so any use is an error
class FluxRegister {
  public:
    template <class... A>
    void CrseInit(A&&...) {
        Abort("stand-in FluxRegister: one level only");
    }
    template <class... A>
    void FineAdd(A&&...) {
        Abort("stand-in FluxRegister: one level only");
    }
    template <class... A>
    void Reflux(A&&...) {
        Abort("stand-in FluxRegister: one level only");
    }
    void setVal(Real) {}
};

template <class... A>
inline void average_down(A&&...) {
    Abort("stand-in average_down: one level only");
}

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
