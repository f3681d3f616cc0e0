// Device-side building blocks of the scalar-advection stage.
//
// Data layout in HBM: every field of a level is one allocation holding one FAB per box
// (the box grown by the field's ghost width, nodal in the face direction for face data),
// Fortran order (i fastest) and one contiguous block per component, i.e. the
// amrex::FArrayBox layout the reference's Array4 views index.  A kernel sees a field
// through a FabView per box.
//
// Work decomposition: a launch covers one index region per box (e.g. the box grown by one
// cell, or its nodal x-faces).  The regions of all boxes are laid end to end; thread gid
// finds its box by binary search over the prefix of region sizes, so one launch covers
// boxes of any (uneven) sizes.  The per-box form of a launch restricts [g0, g1) to one box.
#pragma once
#include <cstdint>

namespace madv {

// AMReX BCType / PhysBCType values used by the reference.
enum { BC_REFLECT_ODD = -1, BC_INT_DIR = 0, BC_REFLECT_EVEN = 1, BC_FOEXTRAP = 2,
       BC_EXT_DIR = 3, BC_HOEXTRAP = 4 };
enum { PB_INTERIOR = 0, PB_INFLOW = 1, PB_OUTFLOW = 2, PB_SYMMETRY = 3, PB_SLIPWALL = 4,
       PB_NOSLIPWALL = 5 };
enum { RHO = 0, RHOH = 1, TEMP = 2, PI = 3, FIRSTSPEC = 4 };

constexpr int MAX_SCAL = 64;

struct FabView {
    double* p;  // element (lo) of component 0
    int lo0, lo1, lo2;
    int sj;
    long sk, sn;
};

__host__ __device__ __forceinline__ double& at(const FabView& f, int i, int j, int k, int n = 0) {
    return f.p[(long)(i - f.lo0) + (long)(j - f.lo1) * f.sj + (long)(k - f.lo2) * f.sk + (long)n * f.sn];
}

struct RegionBox {
    int lo[3];
    int n[3];
    int b;  // box owning this piece of the region
    int pad;
    long start;
};

struct BCRecD {
    int lo[3];
    int hi[3];
};

// Binary search of the region piece owning element gid (largest e with start <= gid).
__device__ __forceinline__ int find_box(const RegionBox* __restrict__ R, int nb, long gid) {
    int lo = 0, hi = nb - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (R[mid].start <= gid) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ void region_ijk(const RegionBox& r, long l, int& i, int& j, int& k) {
    const long nx = r.n[0], ny = r.n[1];
    const long q = l / nx;
    i = r.lo[0] + (int)(l - q * nx);
    const long q2 = q / ny;
    j = r.lo[1] + (int)(q - q2 * ny);
    k = r.lo[2] + (int)q2;
}

// Common launch prologue: returns false for threads past the range.
#define MADV_ELEMENT(R, ne, g0, g1, b, i, j, k)                            \
    const long gid_ = (g0) + (long)blockIdx.x * blockDim.x + threadIdx.x; \
    if (gid_ >= (g1)) return;                                             \
    const int e_ = find_box((R), (ne), gid_);                             \
    const int b = (R)[e_].b;                                              \
    int i, j, k;                                                          \
    region_ijk((R)[e_], gid_ - (R)[e_].start, i, j, k)

// amrex::min / amrex::max (std::min / std::max semantics).  (An integer-key form measured
// slower: the FP64 min/max instruction is not the costly part of the FP64 pipe.)
__device__ __forceinline__ double mn(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double mx(double a, double b) { return (a < b) ? b : a; }

}  // namespace madv
