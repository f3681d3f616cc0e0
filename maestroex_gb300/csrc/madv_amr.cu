// Coarse-fine operations of a two-level hierarchy (refinement ratio 2): the parts of the
// reference's multi-level stage that couple the levels.
//
//   interp_fill         FillPatchTwoLevels with cell_cons_interp (Source/MaestroFillData.cpp:46-73):
//                       fine ghost cells inside the domain that no fine box covers
//   average_down        average_down (Source/MaestroFillData.cpp:145-154)
//   average_down_faces  average_down_faces (Source/MaestroFillData.cpp:156-174)
//   uedge_interface     the coarse-fine part of Maestro::FillPatchUedge
//                       (Source/MaestroFillData.cpp:466-825)
//   flux register       FluxRegister CrseInit / FineAdd / Reflux of reflux_type 2
//                       (Source/MaestroMakeFlux.cpp:412-456, Source/MaestroAdvection.cpp:258-276)
//
// The AMReX routines are restated from their published algorithms (the reference's AMReX
// submodule is empty and unpinned):
//   * coarse values outside the domain are the coarse level's boundary fill of a FAB that
//     spans the domain (directions swept x, y, z, the last direction applied wins);
//   * cell_cons_interp: per coarse cell and direction the central slope 0.5 (u+ - u-), or
//     (u+ + 3 u0 - 4 u-) / 3 and (4 u+ - 3 u0 - u-) / 3 on an ext_dir / hoextrap domain
//     face, limited against 2 (u+ - u0) and 2 (u0 - u-) (monotonized central); the fine
//     value is u0 + xoff sx + yoff sy + zoff sz with offsets of -1/4 and +1/4;
//   * average_down: the sum of the 8 children (k outer, i inner) times 1/8; faces: the sum
//     of the 4 fine faces (outer = the higher transverse direction) times 1/4.
//   * FluxRegister: one register face per coarse face of each coarsened fine box's six
//     sides (orientations x-lo, y-lo, z-lo, x-hi, y-hi, z-hi).  CrseInit sets it to
//     mult * (coarse flux of the face, read from the box owning the coarse cell inside the
//     fine box); FineAdd adds mult * each of its 4 fine faces in turn (outer = the higher
//     transverse direction); Reflux adds -reg / vol (lo side) or +reg / vol (hi side) to the
//     coarse cell outside the face (periodic images wrapped, cells outside the domain
//     skipped), the orientations one after the other.  With CrseInit's mult = -dt * (coarse
//     face area) and FineAdd's dt * (fine face area), reg = dt A_c (<F_fine> - F_coarse),
//     the flux mismatch the outside coarse cell's update takes back.
// FillPatchUedge on a ghost face: a face on a coarse face takes the fine valid value if a
// fine box has it (the box owning the cell above it, else below), else the coarse face
// (owner of the cell above, else below, else of the nearest domain cell, from its ghost
// faces); a face between coarse faces takes the linear interpolation between its two
// neighbours in the face direction at the first fine index of its coarse face in the
// other two directions.  Ghost faces that are valid in another fine box are overwritten by
// the FillBoundary that follows, as in the reference.
//
// Level lookups use an owner map per level (the box owning each cell of the level's
// domain, int32): 67 MB for a 256^3 level, 537 MB for a 512^3 level.
#include "madv_exact.cuh"
#include "madv_launch.cuh"

namespace madv {

struct LevelGeo {
    int dlo[3], dhi[3], per[3];
    long nx, ny;
    const int* owner;
};

static LevelGeo geo_of(const Ctx& c) {
    LevelGeo g{};
    for (int d = 0; d < 3; ++d) {
        g.dlo[d] = c.P.dom_lo[d];
        g.dhi[d] = c.P.dom_hi[d];
        g.per[d] = c.per[d] ? 1 : 0;
    }
    g.nx = c.P.dom_hi[0] - c.P.dom_lo[0] + 1;
    g.ny = c.P.dom_hi[1] - c.P.dom_lo[1] + 1;
    g.owner = c.d_owner;
    return g;
}

int build_owner(Ctx& c) {
    const long nx = c.P.dom_hi[0] - c.P.dom_lo[0] + 1, ny = c.P.dom_hi[1] - c.P.dom_lo[1] + 1,
               nz = c.P.dom_hi[2] - c.P.dom_lo[2] + 1;
    c.h_owner.assign((size_t)(nx * ny * nz), -1);
    for (int b = 0; b < c.nb; ++b) {
        const HBox& x = c.ba[b];
        for (int k = x.lo[2]; k <= x.hi[2]; ++k)
            for (int j = x.lo[1]; j <= x.hi[1]; ++j)
                for (int i = x.lo[0]; i <= x.hi[0]; ++i)
                    c.h_owner[(size_t)((i - c.P.dom_lo[0]) + nx * ((j - c.P.dom_lo[1]) + ny * (long)(k - c.P.dom_lo[2])))] =
                        b;
    }
    if (c.d_owner) cudaFree(c.d_owner);
    c.d_owner = nullptr;
    if (!cuda_ok(cudaMalloc(&c.d_owner, sizeof(int) * c.h_owner.size()), "cudaMalloc(owner)") ||
        !cuda_ok(cudaMemcpy(c.d_owner, c.h_owner.data(), sizeof(int) * c.h_owner.size(), cudaMemcpyHostToDevice),
                 "cudaMemcpy(owner)"))
        return MADV_ERR_CUDA;
    return MADV_OK;
}

__device__ __forceinline__ int owner_in(const LevelGeo& g, int i, int j, int k) {
    if (i < g.dlo[0] || i > g.dhi[0] || j < g.dlo[1] || j > g.dhi[1] || k < g.dlo[2] || k > g.dhi[2]) return -1;
    return g.owner[(i - g.dlo[0]) + g.nx * ((j - g.dlo[1]) + g.ny * (long)(k - g.dlo[2]))];
}

__device__ __forceinline__ int wrap(const LevelGeo& g, int d, int m) {
    if (!g.per[d]) return m;
    const int len = g.dhi[d] - g.dlo[d] + 1;
    while (m < g.dlo[d]) m += len;
    while (m > g.dhi[d]) m -= len;
    return m;
}

// Coarse value at a (periodically wrapped) index: valid data, or the boundary fill along
// the highest direction in which the index lies outside the domain (directions below D may
// still be outside and are resolved recursively).
template <int D>
__device__ double cval(const LevelGeo& g, const FabView* __restrict__ Vc, int nbc, int fid, int n, const BCRecD& bc,
                       bool velish, int p0, int p1, int p2, int* err) {
    if constexpr (D < 0) {
        const int b = owner_in(g, p0, p1, p2);
        if (b < 0) {
            atomicOr(err, 2);
            return 0.0;
        }
        return at(Vc[fid * nbc + b], p0, p1, p2, n);
    } else {
        const int p[3] = {p0, p1, p2};
        const int m = p[D], dlo = g.dlo[D], dhi = g.dhi[D];
        if (m >= dlo && m <= dhi) return cval<D - 1>(g, Vc, nbc, fid, n, bc, velish, p0, p1, p2, err);
        const bool lo = m < dlo;
        const int t = lo ? bc.lo[D] : bc.hi[D];
        auto at_m = [&](int q) {
            int r[3] = {p0, p1, p2};
            r[D] = q;
            return cval<D - 1>(g, Vc, nbc, fid, n, bc, velish, r[0], r[1], r[2], err);
        };
        switch (t) {
            case BC_FOEXTRAP: return at_m(lo ? dlo : dhi);
            case BC_HOEXTRAP:
                if (lo)
                    return m < dlo - 1 ? at_m(dlo) : 0.125 * (15. * at_m(dlo) - 10. * at_m(dlo + 1) + 3. * at_m(dlo + 2));
                return m > dhi + 1 ? at_m(dhi) : 0.125 * (15. * at_m(dhi) - 10. * at_m(dhi - 1) + 3. * at_m(dhi - 2));
            case BC_REFLECT_EVEN: return at_m(lo ? 2 * dlo - 1 - m : 2 * dhi + 1 - m);
            case BC_REFLECT_ODD: return -at_m(lo ? 2 * dlo - 1 - m : 2 * dhi + 1 - m);
            case BC_EXT_DIR:
                if (!velish) atomicOr(err, 2);
                return 0.0;
            default: atomicOr(err, 2); return 0.0;
        }
    }
}

__device__ __forceinline__ double cv(const LevelGeo& g, const FabView* __restrict__ Vc, int nbc, int fid, int n,
                                     const BCRecD& bc, bool velish, int a, int b, int c, int* err) {
    const int p0 = wrap(g, 0, a), p1 = wrap(g, 1, b), p2 = wrap(g, 2, c);
    // a cell of the domain: its owner's value (what cval reaches through its recursion)
    if (p0 >= g.dlo[0] && p0 <= g.dhi[0] && p1 >= g.dlo[1] && p1 <= g.dhi[1] && p2 >= g.dlo[2] && p2 <= g.dhi[2]) {
        const int ob = g.owner[(p0 - g.dlo[0]) + g.nx * ((p1 - g.dlo[1]) + g.ny * (long)(p2 - g.dlo[2]))];
        if (ob >= 0) return at(Vc[fid * nbc + ob], p0, p1, p2, n);
        atomicOr(err, 2);
        return 0.0;
    }
    return cval<2>(g, Vc, nbc, fid, n, bc, velish, p0, p1, p2, err);
}

static const RegionTable& shell_table(Ctx& c, int ng, int nodal) {
    std::array<int, 4> key{0, ng, nodal, 0};
    auto it = c.amr_tables.find(key);
    if (it != c.amr_tables.end()) return it->second;
    RegionTable& t = c.amr_tables[key];
    long start = 0;
    auto push = [&](int b, const int lo[3], const int hi[3]) {
        RegionBox r{};
        for (int d = 0; d < 3; ++d) {
            r.lo[d] = lo[d];
            r.n[d] = hi[d] - lo[d] + 1;
            if (r.n[d] <= 0) return;
        }
        r.b = b;
        r.start = start;
        start += (long)r.n[0] * r.n[1] * r.n[2];
        t.h.push_back(r);
    };
    for (int b = 0; b < c.nb; ++b) {
        int vlo[3], vhi[3], glo[3], ghi[3];
        for (int d = 0; d < 3; ++d) {
            vlo[d] = c.ba[b].lo[d];
            vhi[d] = c.ba[b].hi[d] + (d == nodal ? 1 : 0);
            glo[d] = vlo[d] - ng;
            ghi[d] = vhi[d] + ng;
        }
        // z slabs (full x, y), y slabs (full x, valid z), x slabs (valid y, z)
        for (int side = 0; side < 2; ++side) {
            int lo[3] = {glo[0], glo[1], side ? vhi[2] + 1 : glo[2]};
            int hi[3] = {ghi[0], ghi[1], side ? ghi[2] : vlo[2] - 1};
            push(b, lo, hi);
        }
        for (int side = 0; side < 2; ++side) {
            int lo[3] = {glo[0], side ? vhi[1] + 1 : glo[1], vlo[2]};
            int hi[3] = {ghi[0], side ? ghi[1] : vlo[1] - 1, vhi[2]};
            push(b, lo, hi);
        }
        for (int side = 0; side < 2; ++side) {
            int lo[3] = {side ? vhi[0] + 1 : glo[0], vlo[1], vlo[2]};
            int hi[3] = {side ? ghi[0] : vlo[0] - 1, vhi[1], vhi[2]};
            push(b, lo, hi);
        }
    }
    t.total = start;
    if (!t.h.empty()) {
        if (cudaMalloc(&t.d, sizeof(RegionBox) * t.h.size()) != cudaSuccess ||
            cudaMemcpy(t.d, t.h.data(), sizeof(RegionBox) * t.h.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            throw Fail{MADV_ERR_CUDA};
    }
    return t;
}

// Coarse cells (nodal = -1) or coarse d-faces under each fine box, split by the coarse box
// holding them (a face on a coarse box boundary appears once per coarse box).  Stored in
// the fine level; RegionBox.b = coarse box, RegionBox.pad = fine box.
static const RegionTable& down_table(Ctx& cf, const Ctx& cc, int nodal) {
    std::array<int, 4> key{1, nodal, 0, 0};
    auto it = cf.amr_tables.find(key);
    if (it != cf.amr_tables.end()) return it->second;
    RegionTable& t = cf.amr_tables[key];
    long start = 0;
    for (int fb = 0; fb < cf.nb; ++fb) {
        int clo[3], chi[3];
        for (int d = 0; d < 3; ++d) {
            clo[d] = cf.ba[fb].lo[d] >> 1;
            chi[d] = (cf.ba[fb].hi[d] >> 1) + (d == nodal ? 1 : 0);
        }
        for (int cb = 0; cb < cc.nb; ++cb) {
            RegionBox r{};
            bool empty = false;
            for (int d = 0; d < 3; ++d) {
                const int lo = std::max(clo[d], cc.ba[cb].lo[d]);
                const int hi = std::min(chi[d], cc.ba[cb].hi[d] + (d == nodal ? 1 : 0));
                if (lo > hi) empty = true;
                r.lo[d] = lo;
                r.n[d] = hi - lo + 1;
            }
            if (empty) continue;
            r.b = cb;
            r.pad = fb;
            r.start = start;
            start += (long)r.n[0] * r.n[1] * r.n[2];
            t.h.push_back(r);
        }
    }
    t.total = start;
    if (!t.h.empty()) {
        if (cudaMalloc(&t.d, sizeof(RegionBox) * t.h.size()) != cudaSuccess ||
            cudaMemcpy(t.d, t.h.data(), sizeof(RegionBox) * t.h.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            throw Fail{MADV_ERR_CUDA};
    }
    return t;
}

// ------------------------------------------------------------------ kernels
// cell_cons_interp value of fine cell (i, j, k), component n.  The exact bit-pattern forms
// of 2x, x/2, |x|, the product sign and copysign(1, dc) * m of madv_exact.cuh replace the FP
// instructions of the literal expressions.  (Resolving the 7 coarse neighbours once for all
// components was tried: it costs registers, and the kernel ran slower.)
__device__ double cons_interp(const LevelGeo& gc, const FabView* __restrict__ Vc, int nbc, int fid, int n,
                              const BCRecD& bc, bool velish, int i, int j, int k, int* err) {
    const int I[3] = {i >> 1, j >> 1, k >> 1};
    const int f[3] = {i, j, k};
    const double u0 = cv(gc, Vc, nbc, fid, n, bc, velish, I[0], I[1], I[2], err);
    double s[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        int pp[3] = {I[0], I[1], I[2]}, pm[3] = {I[0], I[1], I[2]};
        pp[d] += 1;
        pm[d] -= 1;
        const double up = cv(gc, Vc, nbc, fid, n, bc, velish, pp[0], pp[1], pp[2], err);
        const double dn = cv(gc, Vc, nbc, fid, n, bc, velish, pm[0], pm[1], pm[2], err);
        double dc = half(up - dn);
        if (!gc.per[d]) {
            if (I[d] == gc.dlo[d] && (bc.lo[d] == BC_EXT_DIR || bc.lo[d] == BC_HOEXTRAP))
                dc = (up + 3.0 * u0 - 4.0 * dn) / 3.0;
            if (I[d] == gc.dhi[d] && (bc.hi[d] == BC_EXT_DIR || bc.hi[d] == BC_HOEXTRAP))
                dc = (4.0 * up - 3.0 * u0 - dn) / 3.0;
        }
        const double df = twice(up - u0);
        const double db = twice(u0 - dn);
        // sl = (df * db >= 0) ? min(|df|, |db|) : 0;  s = copysign(1, dc) * min(sl, |dc|)
        long long sl = 0;
        if (!prod_gt0(df, -db)) sl = min(dbits(df) & ABS_MASK, dbits(db) & ABS_MASK);
        const long long m = min(sl, dbits(dc) & ABS_MASK);
        s[d] = __longlong_as_double(m | (dbits(dc) & SIGN_BIT));
    }
    double off[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) off[d] = (f[d] - 2 * I[d]) == 0 ? -0.25 : 0.25;
    return u0 + off[0] * s[0] + off[1] * s[1] + off[2] * s[2];
}

__global__ void k_interp_fill(KARGS, const FabView* __restrict__ Vc, int nbc, LevelGeo gc, LevelGeo gf, int fid,
                              int c0, int nc, const BCRecD* __restrict__ bcs, int bc_c0, int is_vel, int state_c0,
                              int* err) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const int p[3] = {i, j, k};
#pragma unroll
    for (int d = 0; d < 3; ++d)
        if (!gf.per[d] && (p[d] < gf.dlo[d] || p[d] > gf.dhi[d])) return;
    if (owner_in(gf, wrap(gf, 0, i), wrap(gf, 1, j), wrap(gf, 2, k)) >= 0) return;
    const FabView f = VW(fid);
    for (int n = c0; n < c0 + nc; ++n) {
        const BCRecD bc = bcs[bc_c0 + n - c0];
        const bool velish = is_vel || (state_c0 >= 0 && state_c0 + (n - c0) == PI);
        at(f, i, j, k, n) = cons_interp(gc, Vc, nbc, fid, n, bc, velish, i, j, k, err);
    }
}

void interp_fill(Ctx& cc, Ctx& cf, int fid, int c0, int nc, int which_bcs, int bc_c0, int is_vel, int state_c0) {
    const RegionTable& rt = shell_table(cf, cf.F[fid].spec.ng, -1);
    launch(cf, rt, 1, k_interp_fill, cf.V(), cc.V(), cc.nb, geo_of(cc), geo_of(cf), fid, c0, nc,
           bcs_dev(cf, which_bcs), bc_c0, is_vel, state_c0, cf.d_flag);
}

__global__ void k_avgdown(KARGS, const FabView* __restrict__ Vf, int nbf, int fid, int comp, int ncomp) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView f = Vf[fid * nbf + R[e_].pad], c = VW(fid);
    for (int n = comp; n < comp + ncomp; ++n) {
        double s = 0.0;
        for (int kr = 0; kr < 2; ++kr)
            for (int jr = 0; jr < 2; ++jr)
                for (int ir = 0; ir < 2; ++ir) s += at(f, 2 * i + ir, 2 * j + jr, 2 * k + kr, n);
        at(c, i, j, k, n) = 0.125 * s;
    }
}

void average_down(Ctx& cf, Ctx& cc, int fid, int comp, int ncomp) {
    const RegionTable& rt = down_table(cf, cc, -1);
    launch(cc, rt, 1, k_avgdown, cc.V(), cf.V(), cf.nb, fid, comp, ncomp);
}

template <int D>
__global__ void k_avgdown_faces(KARGS, const FabView* __restrict__ Vf, int nbf, int fid, int c0, int ncomp) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int t1 = D == 0 ? 1 : 0, t2 = D == 2 ? 1 : 2;
    const FabView f = Vf[fid * nbf + R[e_].pad], c = VW(fid);
    for (int n = c0; n < c0 + ncomp; ++n) {
        double s = 0.0;
        for (int o = 0; o < 2; ++o)
            for (int in = 0; in < 2; ++in) {
                int q[3] = {2 * i, 2 * j, 2 * k};
                q[t1] += in;
                q[t2] += o;
                s += at(f, q[0], q[1], q[2], n);
            }
        at(c, i, j, k, n) = s * 0.25;
    }
}

void average_down_faces(Ctx& cf, Ctx& cc, int f0, int c0, int ncomp) {
    for (int d = 0; d < 3; ++d) {
        const RegionTable& rt = down_table(cf, cc, d);
        if (d == 0) launch(cc, rt, 1, k_avgdown_faces<0>, cc.V(), cf.V(), cf.nb, f0, c0, ncomp);
        else if (d == 1) launch(cc, rt, 1, k_avgdown_faces<1>, cc.V(), cf.V(), cf.nb, f0 + 1, c0, ncomp);
        else launch(cc, rt, 1, k_avgdown_faces<2>, cc.V(), cf.V(), cf.nb, f0 + 2, c0, ncomp);
    }
}

// ---- flux register (reflux_type 2)
// register faces of orientation o of every fine box: coarse face planes, box index in .b
static const RegionTable& reg_table(Ctx& cf, int o) {
    std::array<int, 4> key{2, o, 0, 0};
    auto it = cf.amr_tables.find(key);
    if (it != cf.amr_tables.end()) return it->second;
    RegionTable& t = cf.amr_tables[key];
    const int D = o % 3, side = o / 3;
    long start = 0;
    for (int fb = 0; fb < cf.nb; ++fb) {
        RegionBox r{};
        for (int d = 0; d < 3; ++d) {
            const int lo = cf.ba[fb].lo[d] >> 1, hi = cf.ba[fb].hi[d] >> 1;
            r.lo[d] = lo;
            r.n[d] = hi - lo + 1;
        }
        if (side == 1) r.lo[D] += r.n[D];  // the hi face: coarsened hi + 1
        r.n[D] = 1;
        r.b = fb;
        r.pad = o;
        r.start = start;
        start += (long)r.n[0] * r.n[1] * r.n[2];
        t.h.push_back(r);
    }
    t.total = start;
    if (!cuda_ok(cudaMalloc(&t.d, sizeof(RegionBox) * t.h.size()), "cudaMalloc(register table)") ||
        !cuda_ok(cudaMemcpy(t.d, t.h.data(), sizeof(RegionBox) * t.h.size(), cudaMemcpyHostToDevice),
                 "cudaMemcpy(register table)"))
        throw Fail{MADV_ERR_CUDA};
    return t;
}

// register storage of a fine level: [orientation][face][component], allocated on first use
static double* reg_storage(Ctx& cf, long off[7]) {
    off[0] = 0;
    for (int o = 0; o < 6; ++o) off[o + 1] = off[o] + reg_table(cf, o).total;
    if (!cf.d_reg) {
        if (!cuda_ok(cudaMalloc(&cf.d_reg, sizeof(double) * (size_t)off[6] * cf.nscal), "cudaMalloc(register)"))
            throw Fail{MADV_ERR_CUDA};
        cudaMemset(cf.d_reg, 0, sizeof(double) * (size_t)off[6] * cf.nscal);
    }
    return cf.d_reg;
}

// CrseInit: reg = mult * coarse flux on the face (the coarse box owning the inside cell)
template <int D, int SIDE>
__global__ void k_fr_crse_init(KARGS, const FabView* __restrict__ Vc, int nbc, LevelGeo gc, int ff, double* reg,
                               long off, int nscal, int c0, int nc, double mult, int slot, int* err) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    int q[3] = {i, j, k};
    if (SIDE == 1) q[D] -= 1;  // the inside cell of a hi face
    const int cb = owner_in(gc, q[0], q[1], q[2]);
    if (cb < 0) {
        atomicOr(err, 4);
        return;
    }
    const FabView fl = Vc[(ff + D) * nbc + cb];
    double* r = reg + (off + gid_) * nscal;
    for (int n = c0; n < c0 + nc; ++n) r[n] = mult * at(fl, i, j, k, slot >= 0 ? slot : n);
}

// FineAdd: reg += mult * each fine face of the coarse face, in turn
template <int D>
__global__ void k_fr_fine_add(KARGS, int ff, double* reg, long off, int nscal, int c0, int nc, double mult,
                              int slot) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int t1 = D == 0 ? 1 : 0, t2 = D == 2 ? 1 : 2;
    const FabView fl = VW(ff + D);
    double* r = reg + (off + gid_) * nscal;
    for (int n = c0; n < c0 + nc; ++n) {
        double v = r[n];
        for (int o = 0; o < 2; ++o)
            for (int in = 0; in < 2; ++in) {
                int q[3] = {2 * i, 2 * j, 2 * k};
                q[t1] += in;
                q[t2] += o;
                v = v + mult * at(fl, q[0], q[1], q[2], slot >= 0 ? slot : n);
            }
        r[n] = v;
    }
}

// Reflux: the coarse cell outside the face takes -reg/vol (lo side) or +reg/vol (hi side)
template <int D, int SIDE>
__global__ void k_fr_reflux(KARGS, const FabView* __restrict__ Vc, int nbc, LevelGeo gc, int fs, const double* reg,
                            long off, int nscal, int c0, int nc, double vol) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    int q[3] = {i, j, k};
    if (SIDE == 0) q[D] -= 1;
    q[D] = wrap(gc, D, q[D]);
    const int cb = owner_in(gc, q[0], q[1], q[2]);
    if (cb < 0) return;  // outside the domain, or no coarse box there
    const FabView sn = Vc[fs * nbc + cb];
    const double* r = reg + (off + gid_) * nscal;
    for (int n = c0; n < c0 + nc; ++n) {
        if (SIDE == 0) at(sn, q[0], q[1], q[2], n) = at(sn, q[0], q[1], q[2], n) - r[n] / vol;
        else at(sn, q[0], q[1], q[2], n) = at(sn, q[0], q[1], q[2], n) + r[n] / vol;
    }
}

template <int D, int SIDE>
static void fr_crse_init_o(Ctx& cf, Ctx& cc, double* reg, long off, int c0, int nc, double mult, int slot) {
    launch(cf, reg_table(cf, D + 3 * SIDE), 1, k_fr_crse_init<D, SIDE>, cf.V(), cc.V(), cc.nb, geo_of(cc), F_SFLUX0,
           reg, off, cf.nscal, c0, nc, mult, slot, cf.d_flag);
}
template <int D>
static void fr_fine_add_o(Ctx& cf, int o, double* reg, long off, int c0, int nc, double mult, int slot) {
    launch(cf, reg_table(cf, o), 1, k_fr_fine_add<D>, cf.V(), F_SFLUX0, reg, off, cf.nscal, c0, nc, mult, slot);
}
template <int D, int SIDE>
static void fr_reflux_o(Ctx& cf, Ctx& cc, const double* reg, long off, int c0, int nc, double vol) {
    launch(cf, reg_table(cf, D + 3 * SIDE), 1, k_fr_reflux<D, SIDE>, cf.V(), cc.V(), cc.nb, geo_of(cc), F_SNEW,
           reg, off, cf.nscal, c0, nc, vol);
}

// FluxRegister::CrseInit of the coarse level's fluxes, components c0 .. c0+nc-1, mult =
// -dt * coarse face area (Source/MaestroMakeFlux.cpp:430-439)
void flux_reg_crse_init(Ctx& cf, Ctx& cc, int c0, int nc, double dt, int slot) {
    long off[7];
    double* reg = reg_storage(cf, off);
    const double area[3] = {cc.P.dx[1] * cc.P.dx[2], cc.P.dx[0] * cc.P.dx[2], cc.P.dx[0] * cc.P.dx[1]};
    fr_crse_init_o<0, 0>(cf, cc, reg, off[0], c0, nc, -1.0 * dt * area[0], slot);
    fr_crse_init_o<0, 1>(cf, cc, reg, off[3], c0, nc, -1.0 * dt * area[0], slot);
    fr_crse_init_o<1, 0>(cf, cc, reg, off[1], c0, nc, -1.0 * dt * area[1], slot);
    fr_crse_init_o<1, 1>(cf, cc, reg, off[4], c0, nc, -1.0 * dt * area[1], slot);
    fr_crse_init_o<2, 0>(cf, cc, reg, off[2], c0, nc, -1.0 * dt * area[2], slot);
    fr_crse_init_o<2, 1>(cf, cc, reg, off[5], c0, nc, -1.0 * dt * area[2], slot);
}

// FluxRegister::FineAdd of the fine level's fluxes, mult = dt * fine face area (:441-450)
void flux_reg_fine_add(Ctx& cf, int c0, int nc, double dt, int slot) {
    long off[7];
    double* reg = reg_storage(cf, off);
    const double area[3] = {cf.P.dx[1] * cf.P.dx[2], cf.P.dx[0] * cf.P.dx[2], cf.P.dx[0] * cf.P.dx[1]};
    for (int side = 0; side < 2; ++side) {
        fr_fine_add_o<0>(cf, 0 + 3 * side, reg, off[0 + 3 * side], c0, nc, 1.0 * dt * area[0], slot);
        fr_fine_add_o<1>(cf, 1 + 3 * side, reg, off[1 + 3 * side], c0, nc, 1.0 * dt * area[1], slot);
        fr_fine_add_o<2>(cf, 2 + 3 * side, reg, off[2 + 3 * side], c0, nc, 1.0 * dt * area[2], slot);
    }
}

// FluxRegister::Reflux into the coarse level's new state (Source/MaestroAdvection.cpp:259-276),
// the orientations in turn
void flux_reg_reflux(Ctx& cf, Ctx& cc, int c0, int nc) {
    long off[7];
    const double* reg = reg_storage(cf, off);
    const double vol = cc.P.dx[0] * cc.P.dx[1] * cc.P.dx[2];
    fr_reflux_o<0, 0>(cf, cc, reg, off[0], c0, nc, vol);
    fr_reflux_o<1, 0>(cf, cc, reg, off[1], c0, nc, vol);
    fr_reflux_o<2, 0>(cf, cc, reg, off[2], c0, nc, vol);
    fr_reflux_o<0, 1>(cf, cc, reg, off[3], c0, nc, vol);
    fr_reflux_o<1, 1>(cf, cc, reg, off[4], c0, nc, vol);
    fr_reflux_o<2, 1>(cf, cc, reg, off[5], c0, nc, vol);
}

template <int D>
__device__ double uedge_even(const FabView* __restrict__ V, int nb, const FabView* __restrict__ Vc, int nbc,
                             const LevelGeo& gc, const LevelGeo& gf, int fid, int i, int j, int k, int* err) {
    int q[3] = {i, j, k};
    int b = owner_in(gf, i, j, k);
    if (b < 0) {
        q[D] -= 1;
        b = owner_in(gf, q[0], q[1], q[2]);
    }
    if (b >= 0) return at(VW(fid), i, j, k);
    const int P[3] = {i >> 1, j >> 1, k >> 1};
    int c[3] = {P[0], P[1], P[2]};
    int cb = owner_in(gc, c[0], c[1], c[2]);
    if (cb < 0) {
        c[D] -= 1;
        cb = owner_in(gc, c[0], c[1], c[2]);
    }
    if (cb < 0) {
#pragma unroll
        for (int e = 0; e < 3; ++e) c[e] = min(max(P[e], gc.dlo[e]), gc.dhi[e]);
        cb = owner_in(gc, c[0], c[1], c[2]);
    }
    if (cb < 0) {
        atomicOr(err, 4);
        return 0.0;
    }
    const FabView v = Vc[fid * nbc + cb];
    const long nx = v.sj, ny = v.sk / v.sj, nz = v.sn / v.sk;
    if (P[0] < v.lo0 || P[0] >= v.lo0 + nx || P[1] < v.lo1 || P[1] >= v.lo1 + ny || P[2] < v.lo2 ||
        P[2] >= v.lo2 + nz) {
        atomicOr(err, 4);
        return 0.0;
    }
    return at(v, P[0], P[1], P[2]);
}

template <int D>
__global__ void k_uedge_iface(KARGS, const FabView* __restrict__ Vc, int nbc, LevelGeo gc, LevelGeo gf, int fid,
                              int* err) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    int q[3] = {i, j, k};
    double v;
    if ((q[D] & 1) == 0) {
        v = uedge_even<D>(V, nb, Vc, nbc, gc, gf, fid, i, j, k, err);
    } else {
#pragma unroll
        for (int e = 0; e < 3; ++e)
            if (e != D) q[e] -= (q[e] & 1);
        int a[3] = {q[0], q[1], q[2]}, c[3] = {q[0], q[1], q[2]};
        a[D] -= 1;
        c[D] += 1;
        const double fa = uedge_even<D>(V, nb, Vc, nbc, gc, gf, fid, a[0], a[1], a[2], err);
        const double fc = uedge_even<D>(V, nb, Vc, nbc, gc, gf, fid, c[0], c[1], c[2], err);
        const double df = fc - fa;
        v = fa + df * 1.0 / 2.0;
    }
    at(VW(fid), i, j, k) = v;
}

void uedge_interface(Ctx& cc, Ctx& cf, int f0) {
    const LevelGeo gc = geo_of(cc), gf = geo_of(cf);
    for (int d = 0; d < 3; ++d) {
        const RegionTable& rt = shell_table(cf, 1, d);
        if (d == 0) launch(cf, rt, 1, k_uedge_iface<0>, cf.V(), cc.V(), cc.nb, gc, gf, f0, cf.d_flag);
        else if (d == 1) launch(cf, rt, 1, k_uedge_iface<1>, cf.V(), cc.V(), cc.nb, gc, gf, f0 + 1, cf.d_flag);
        else launch(cf, rt, 1, k_uedge_iface<2>, cf.V(), cc.V(), cc.nb, gc, gf, f0 + 2, cf.d_flag);
    }
}

}  // namespace madv
