// Test infrastructure only (oracle): coarse-fine operations of a two-level hierarchy
// (refinement ratio 2), restated from the AMReX routines the reference calls.
//
// The reference's AMReX dependency is an empty, unpinned submodule, so these follow the
// published AMReX algorithms as the reference uses them:
//   FillPatchTwoLevels with cell_cons_interp  (Source/MaestroFillData.cpp:46-73)
//   average_down / average_down_faces         (Source/MaestroFillData.cpp:145-174)
// and the reference's own FillPatchUedge (Source/MaestroFillData.cpp:455-835).
//
// Coarse data for the interpolation is the coarse level's valid data, extended outside the
// domain by the coarse level's boundary conditions exactly as the physical fill of a FAB
// spanning the whole domain would extend it (directions swept x, y, z; a cell outside the
// domain in several directions takes the value of the last direction applied).
//
// cell_cons_interp: per coarse cell and direction the central slope 0.5 (u+ - u-) (one-sided
// (u+ + 3 u0 - 4 u-) / 3 resp. (4 u+ - 3 u0 - u-) / 3 on a domain face with ext_dir or
// hoextrap), limited by monotonized-central limiting against 2 (u+ - u0) and 2 (u0 - u-);
// the fine value is u0 + xoff sx + yoff sy + zoff sz with offsets -1/4, +1/4.
#pragma once
#include <algorithm>
#include <array>

#include "mo_fill.hpp"

namespace mo {

// Ownership map of a level: box index of each cell of the level's domain (-1 = uncovered).
struct Owner {
    Box dom;
    std::vector<int> id;
    long nx = 0, ny = 0;
    void build(const Level& L) {
        dom = L.dom;
        nx = dom.hi[0] - dom.lo[0] + 1;
        ny = dom.hi[1] - dom.lo[1] + 1;
        long nz = dom.hi[2] - dom.lo[2] + 1;
        id.assign((size_t)(nx * ny * nz), -1);
        for (int b = 0; b < (int)L.ba.size(); ++b) MO_FOR3(L.ba[b]) id[idx(i, j, k)] = b;
    }
    long idx(int i, int j, int k) const {
        return (i - dom.lo[0]) + nx * ((j - dom.lo[1]) + ny * (long)(k - dom.lo[2]));
    }
    // box owning cell (i,j,k) after the periodic wrap, -1 if uncovered or outside the domain
    int at(const Level& L, int i, int j, int k) const {
        int p[3] = {i, j, k};
        for (int d = 0; d < 3; ++d) {
            const int len = dom.hi[d] - dom.lo[d] + 1;
            if (L.per[d]) {
                while (p[d] < dom.lo[d]) p[d] += len;
                while (p[d] > dom.hi[d]) p[d] -= len;
            }
            if (p[d] < dom.lo[d] || p[d] > dom.hi[d]) return -1;
        }
        return id[idx(p[0], p[1], p[2])];
    }
};

inline int floordiv2(int a) { return a >= 0 ? a / 2 : -((-a + 1) / 2); }

// Coarse value of component n at (I,J,K), extended by the BC fill of a domain-wide FAB.
inline real coarse_value(const Level& Lc, const Owner& oc, const MF& cmf, int n, const BCRec& bc, bool velish,
                           int I, int J, int K) {
    int p[3] = {I, J, K};
    for (int d = 0; d < 3; ++d)
        if (Lc.per[d]) {
            const int len = Lc.dom.hi[d] - Lc.dom.lo[d] + 1;
            while (p[d] < Lc.dom.lo[d]) p[d] += len;
            while (p[d] > Lc.dom.hi[d]) p[d] -= len;
        }
    int dmax = -1;
    for (int d = 0; d < 3; ++d)
        if (p[d] < Lc.dom.lo[d] || p[d] > Lc.dom.hi[d]) dmax = d;
    if (dmax < 0) {
        const int b = oc.id[oc.idx(p[0], p[1], p[2])];
        if (b < 0) throw std::runtime_error("two-level fill: coarse cell not covered (nesting)");
        return cmf[b](p[0], p[1], p[2], n);
    }
    const int d = dmax;
    const int dlo = Lc.dom.lo[d], dhi = Lc.dom.hi[d];
    const bool lo = p[d] < dlo;
    const int t = lo ? bc.lo[d] : bc.hi[d];
    auto at = [&](int m) {
        int q[3] = {p[0], p[1], p[2]};
        q[d] = m;
        return coarse_value(Lc, oc, cmf, n, bc, velish, q[0], q[1], q[2]);
    };
    const int m = p[d];
    switch (t) {
        case foextrap: return at(lo ? dlo : dhi);
        case hoextrap:
            if (lo) return m < dlo - 1 ? at(dlo) : 0.125 * (15. * at(dlo) - 10. * at(dlo + 1) + 3. * at(dlo + 2));
            return m > dhi + 1 ? at(dhi) : 0.125 * (15. * at(dhi) - 10. * at(dhi - 1) + 3. * at(dhi - 2));
        case reflect_even: return at(lo ? 2 * dlo - 1 - m : 2 * dhi + 1 - m);
        case reflect_odd: return -at(lo ? 2 * dlo - 1 - m : 2 * dhi + 1 - m);
        case ext_dir:
            if (!velish) throw std::runtime_error("scalar Dirichlet (inflow) boundary needs problem-specific data");
            return 0.0;
        default: throw std::runtime_error("two-level fill: bad BC");
    }
}

// cell_cons_interp value of fine cell (i,j,k) (restated as described at the top).
inline real cons_interp(const Level& Lc, const Owner& oc, const MF& cmf, int n, const BCRec& bc, bool velish, int i,
                          int j, int k) {
    const int I[3] = {floordiv2(i), floordiv2(j), floordiv2(k)};
    const int f[3] = {i, j, k};
    auto cv = [&](int a, int b, int c) { return coarse_value(Lc, oc, cmf, n, bc, velish, a, b, c); };
    const real u0 = cv(I[0], I[1], I[2]);
    real s[3];
    for (int d = 0; d < 3; ++d) {
        int pp[3] = {I[0], I[1], I[2]}, pm[3] = {I[0], I[1], I[2]};
        pp[d] += 1;
        pm[d] -= 1;
        const real up = cv(pp[0], pp[1], pp[2]);
        const real dn = cv(pm[0], pm[1], pm[2]);
        real dc = 0.5 * (up - dn);
        if (!Lc.per[d]) {
            if (I[d] == Lc.dom.lo[d] && (bc.lo[d] == ext_dir || bc.lo[d] == hoextrap))
                dc = (up + 3.0 * u0 - 4.0 * dn) / 3.0;
            if (I[d] == Lc.dom.hi[d] && (bc.hi[d] == ext_dir || bc.hi[d] == hoextrap))
                dc = (4.0 * up - 3.0 * u0 - dn) / 3.0;
        }
        const real df = 2.0 * (up - u0);
        const real db = 2.0 * (u0 - dn);
        real sl = (df * db >= 0.0) ? mn(fab(df), fab(db)) : 0.0;
        s[d] = cps(1.0, dc) * mn(sl, fab(dc));
    }
    real off[3];
    for (int d = 0; d < 3; ++d) off[d] = (f[d] - 2 * I[d]) == 0 ? -0.25 : 0.25;
    return u0 + off[0] * s[0] + off[1] * s[1] + off[2] * s[2];
}

// FillPatchTwoLevels for level Lf from level Lc: ghost cells inside the fine domain that no
// fine box covers (after the periodic wrap) are interpolated from the coarse level, then
// the fine level's FillBoundary and physical fill run.
inline void FillPatchTwoLevels(const Level& Lc, const MF& cmf, const Level& Lf, MF& fmf, int c0, int nc, int bccomp,
                               const std::vector<BCRec>& bcs, bool is_vel, int state_comp0) {
    Owner oc, of;
    oc.build(Lc);
    of.build(Lf);
    const int ng = fmf.ng;
#pragma omp parallel for schedule(dynamic)
    for (int b = 0; b < fmf.size(); ++b) {
        const Box vb = fmf.validbox(b);
        const Box gb = grow(vb, ng);
        const Arr& q = fmf[b];
        MO_FOR3(gb) {
            if (contains(vb, i, j, k)) continue;
            bool inside = true;
            const int p[3] = {i, j, k};
            for (int d = 0; d < 3; ++d)
                if (!Lf.per[d] && (p[d] < Lf.dom.lo[d] || p[d] > Lf.dom.hi[d])) inside = false;
            if (!inside) continue;
            if (of.at(Lf, i, j, k) >= 0) continue;
            for (int n = c0; n < c0 + nc; ++n) {
                const BCRec& bc = bcs[bccomp + n - c0];
                const bool velish = is_vel || (state_comp0 >= 0 && state_comp0 + (n - c0) == Pi);
                q(i, j, k, n) = cons_interp(Lc, oc, cmf, n, bc, velish, i, j, k);
            }
        }
    }
    FillBoundary(Lf, fmf, c0, nc, ng);
    PhysFill(Lf, fmf, c0, nc, ng, bcs, bccomp, is_vel, state_comp0);
}

// average_down: every coarse cell under a fine box becomes the mean of its 8 children
// (summed k-outer, i-inner, times 1/8).
inline void AverageDown(const Level& Lf, const MF& fmf, const Level& Lc, MF& cmf, int comp, int ncomp) {
    Owner oc;
    oc.build(Lc);
    const real volfrac = 1.0 / 8.0;
    for (int b = 0; b < fmf.size(); ++b) {
        const Box& fb = Lf.ba[b];
        Box cb;
        for (int d = 0; d < 3; ++d) {
            cb.lo[d] = floordiv2(fb.lo[d]);
            cb.hi[d] = floordiv2(fb.hi[d]);
        }
        const Arr& f = fmf[b];
        for (int n = comp; n < comp + ncomp; ++n) MO_FOR3(cb) {
                real c = 0.0;
                for (int kr = 0; kr < 2; ++kr)
                    for (int jr = 0; jr < 2; ++jr)
                        for (int ir = 0; ir < 2; ++ir) c += f(2 * i + ir, 2 * j + jr, 2 * k + kr, n);
                const int cbx = oc.id[oc.idx(i, j, k)];
                if (cbx < 0) throw std::runtime_error("average_down: fine box not nested");
                cmf[cbx](i, j, k, n) = volfrac * c;
            }
    }
    (void)Lc;
}

// average_down_faces: every coarse face of a coarsened fine box becomes the mean of the 4
// fine faces on it (summed over the two transverse offsets, outer = higher direction),
// written to every coarse box whose faces include it.
inline void AverageDownFaces(const Level& Lf, const std::array<MF, 3>& ff, const Level& Lc, std::array<MF, 3>& cf) {
    const real facInv = 1.0 / 4.0;
    for (int d = 0; d < 3; ++d) {
        const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;  // inner, outer transverse
        for (int b = 0; b < ff[d].size(); ++b) {
            const Box& fb = Lf.ba[b];
            Box cb;
            for (int e = 0; e < 3; ++e) {
                cb.lo[e] = floordiv2(fb.lo[e]);
                cb.hi[e] = floordiv2(fb.hi[e]);
            }
            cb = nodal(cb, d);
            const Arr& f = ff[d][b];
            for (int n = 0; n < ff[d].nc; ++n) MO_FOR3(cb) {
                    real c = 0.0;
                    for (int o = 0; o < 2; ++o)
                        for (int in = 0; in < 2; ++in) {
                            int q[3] = {2 * i, 2 * j, 2 * k};
                            q[t1] += in;
                            q[t2] += o;
                            c += f(q[0], q[1], q[2], n);
                        }
                    const real v = c * facInv;
                    for (int cbx = 0; cbx < cf[d].size(); ++cbx)
                        if (contains(nodal(Lc.ba[cbx], d), i, j, k)) cf[d][cbx](i, j, k, n) = v;
                }
        }
    }
}

// The interface part of Maestro::FillPatchUedge (Source/MaestroFillData.cpp:466-825) for
// one fine level and face direction d.  The reference builds source faces around the
// fine boxes' boundary cells (every fine cell whose coarse parent has a child next to the
// fine boxes but not in them): faces on coarse faces take the coarse face value (or the
// fine valid value where the face is a valid fine face), faces in between take the linear
// interpolation in d of the two neighbouring coarse-aligned faces at the first transverse
// fine index of their coarse face; ghost faces of the fine FABs then receive these values.
// Every ghost face of a fine FAB is either such a source face or a valid face of another
// fine box (one of its two cells lies next to the box: if no fine box covers that cell it
// is a boundary cell, else the face is valid in the box covering it), and the latter are
// overwritten by the FillBoundary that follows.  So the rule is applied to every ghost
// face.  Lookups: a fine face is valid in the box owning the cell above it, else the cell
// below; a coarse face is read from the coarse box owning the cell above it, else below,
// else (outside the domain) the box owning the nearest domain cell, from its ghost faces.
struct UedgeInterface {
    const Level& Lc;
    const Level& Lf;
    const MF& cu;  // coarse faces (valid + 1 ghost, already filled)
    const MF& fu;  // fine faces
    int d;
    Owner oc, of;
    UedgeInterface(const Level& Lc_, const Level& Lf_, const MF& cu_, const MF& fu_, int d_)
        : Lc(Lc_), Lf(Lf_), cu(cu_), fu(fu_), d(d_) {
        oc.build(Lc);
        of.build(Lf);
    }
    static int owner_in(const Owner& o, int i, int j, int k) {
        if (i < o.dom.lo[0] || i > o.dom.hi[0] || j < o.dom.lo[1] || j > o.dom.hi[1] || k < o.dom.lo[2] ||
            k > o.dom.hi[2])
            return -1;
        return o.id[o.idx(i, j, k)];
    }
    real coarse_face(int I, int J, int K) const {
        int q[3] = {I, J, K};
        int b = owner_in(oc, I, J, K);
        if (b < 0) {
            q[d] -= 1;
            b = owner_in(oc, q[0], q[1], q[2]);
        }
        if (b < 0) {
            int c[3] = {I, J, K};
            for (int e = 0; e < 3; ++e) c[e] = std::min(std::max(c[e], Lc.dom.lo[e]), Lc.dom.hi[e]);
            b = owner_in(oc, c[0], c[1], c[2]);
        }
        if (b < 0 || !contains(grow(nodal(Lc.ba[b], d), 1), I, J, K))
            throw std::runtime_error("FillPatchUedge: coarse face not available");
        return cu[b](I, J, K);
    }
    // value of a coarse-aligned face
    real even_value(int i, int j, int k) const {
        int q[3] = {i, j, k};
        int b = owner_in(of, i, j, k);
        if (b < 0) {
            q[d] -= 1;
            b = owner_in(of, q[0], q[1], q[2]);
        }
        if (b >= 0) return fu[b](i, j, k);
        return coarse_face(floordiv2(i), floordiv2(j), floordiv2(k));
    }
    real value(int i, int j, int k) const {
        int q[3] = {i, j, k};
        if ((q[d] & 1) == 0) return even_value(i, j, k);
        for (int e = 0; e < 3; ++e)
            if (e != d) q[e] -= (q[e] & 1);
        int a[3] = {q[0], q[1], q[2]}, c[3] = {q[0], q[1], q[2]};
        a[d] -= 1;
        c[d] += 1;
        const real fa = even_value(a[0], a[1], a[2]);
        const real fc = even_value(c[0], c[1], c[2]);
        const real df = fc - fa;
        return fa + df * 1.0 / 2.0;
    }
    void apply(MF& fout) const {
#pragma omp parallel for schedule(dynamic)
        for (int b = 0; b < fout.size(); ++b) {
            const Box vb = nodal(Lf.ba[b], d);
            const Box gb = grow(vb, 1);
            const Arr& q = fout[b];
            MO_FOR3(gb) {
                if (contains(vb, i, j, k)) continue;
                q(i, j, k) = value(i, j, k);
            }
        }
    }
};

}  // namespace mo
