// Test infrastructure only (oracle): single-level ghost fills.
//
// FillBoundary: ghost cells/faces that lie in another box's valid region (after the
// periodic wrap) are copied from it; valid data is never overwritten.
// Physical-boundary fill (the oracle's restatement of AMReX fab_filcc as the reference
// uses it through ScalarFill/VelFill, Source/MaestroBCFill.cpp:8-171): directions are swept
// x, then y, then z over the whole FAB in the other directions, so an edge/corner ghost
// takes the value of the last direction applied.
//   foextrap      ghost = nearest valid value
//   hoextrap      first ghost = face value of the quadratic through the first three
//                 valid cells, (15 q0 - 10 q1 + 3 q2)/8; deeper ghosts = nearest valid
//   reflect_even  mirror;  reflect_odd  mirror with sign change
//   ext_dir       0 for velocity and Pi (FillExtBC, Source/MaestroBCFill.cpp:30-171);
//                 any other scalar is an error, as in the reference.
#pragma once
#include "mo_types.hpp"

namespace mo {

struct Level {
    Box dom;
    bool per[3];
    double dx[3];
    std::vector<Box> ba;
};

inline void FillBoundary(const Level& L, MF& mf, int c0, int nc, int ngf) {
    const int nb = mf.size();
    int len[3];
    for (int d = 0; d < 3; ++d) len[d] = L.dom.hi[d] - L.dom.lo[d] + 1;
#pragma omp parallel for schedule(dynamic)
    for (int b = 0; b < nb; ++b) {
        Box vb = mf.validbox(b);
        Box gb = grow(vb, ngf);
        const Arr& dst = mf[b];
        for (int c = 0; c < nb; ++c) {
            Box sv = mf.validbox(c);
            for (int sz = -1; sz <= 1; ++sz)
                for (int sy = -1; sy <= 1; ++sy)
                    for (int sx = -1; sx <= 1; ++sx) {
                        int s[3] = {sx, sy, sz};
                        bool ok = true;
                        for (int d = 0; d < 3; ++d)
                            if (s[d] != 0 && !L.per[d]) ok = false;
                        if (!ok) continue;
                        if (c == b && sx == 0 && sy == 0 && sz == 0) continue;
                        Box r;
                        bool empty = false;
                        for (int d = 0; d < 3; ++d) {
                            int sl = sv.lo[d] + s[d] * len[d], sh = sv.hi[d] + s[d] * len[d];
                            r.lo[d] = std::max(gb.lo[d], sl);
                            r.hi[d] = std::min(gb.hi[d], sh);
                            if (r.lo[d] > r.hi[d]) empty = true;
                        }
                        if (empty) continue;
                        const Arr& src = mf[c];
                        for (int n = c0; n < c0 + nc; ++n)
                            MO_FOR3(r) {
                                if (contains(vb, i, j, k)) continue;
                                dst(i, j, k, n) =
                                    src(i - sx * len[0], j - sy * len[1], k - sz * len[2], n);
                            }
                    }
        }
    }
}

// Physical-boundary fill of a cell-centred MF; bcs[bccomp + n - c0] gives the BC of
// component n.  is_vel selects the VelFill path (ext_dir -> 0); pi_comp is the state
// component index of Pi if the filled components are state components, else -1.
inline void PhysFill(const Level& L, MF& mf, int c0, int nc, int ngf, const std::vector<BCRec>& bcs,
                     int bccomp, bool is_vel, int state_comp0 = -1) {
    const int nb = mf.size();
    for (int b = 0; b < nb; ++b) {
        const Arr& q = mf[b];
        Box fb = grow(mf.validbox(b), ngf);
        for (int n = c0; n < c0 + nc; ++n) {
            const BCRec& bc = bcs[bccomp + n - c0];
            bool velish = is_vel || (state_comp0 >= 0 && state_comp0 + (n - c0) == Pi);
            for (int d = 0; d < 3; ++d) {
                if (L.per[d]) continue;
                int dlo = L.dom.lo[d], dhi = L.dom.hi[d];
                for (int side = 0; side < 2; ++side) {
                    int t = side == 0 ? bc.lo[d] : bc.hi[d];
                    Box r = fb;
                    if (side == 0) {
                        r.hi[d] = std::min(fb.hi[d], dlo - 1);
                    } else {
                        r.lo[d] = std::max(fb.lo[d], dhi + 1);
                    }
                    if (r.lo[d] > r.hi[d]) continue;
                    if (t == int_dir) continue;
                    if (t == ext_dir && !velish)
                        throw std::runtime_error(
                            "scalar Dirichlet (inflow) boundary needs problem-specific data");
                    MO_FOR3(r) {
                        int idx[3] = {i, j, k};
                        int m = idx[d];
                        auto at = [&](int p) -> real {
                            int id2[3] = {i, j, k};
                            id2[d] = p;
                            return q(id2[0], id2[1], id2[2], n);
                        };
                        real v;
                        if (t == foextrap) {
                            v = at(side == 0 ? dlo : dhi);
                        } else if (t == hoextrap) {
                            if (side == 0) {
                                if (m < dlo - 1) {
                                    v = at(dlo);
                                } else if (dlo + 2 <= std::min(fb.hi[d], dhi)) {
                                    v = 0.125 * (15. * at(dlo) - 10. * at(dlo + 1) + 3. * at(dlo + 2));
                                } else {
                                    v = 0.5 * (3. * at(dlo) - at(dlo + 1));
                                }
                            } else {
                                if (m > dhi + 1) {
                                    v = at(dhi);
                                } else if (dhi - 2 >= std::max(fb.lo[d], dlo)) {
                                    v = 0.125 * (15. * at(dhi) - 10. * at(dhi - 1) + 3. * at(dhi - 2));
                                } else {
                                    v = 0.5 * (3. * at(dhi) - at(dhi - 1));
                                }
                            }
                        } else if (t == reflect_even) {
                            v = at(side == 0 ? 2 * dlo - 1 - m : 2 * dhi + 1 - m);
                        } else if (t == reflect_odd) {
                            v = -at(side == 0 ? 2 * dlo - 1 - m : 2 * dhi + 1 - m);
                        } else if (t == ext_dir) {
                            v = 0.0;
                        } else {
                            throw std::runtime_error("unknown BC type");
                        }
                        q(i, j, k, n) = v;
                    }
                }
            }
        }
    }
}

// FillPatch at one level (no coarser level): FillBoundary then the physical fill.
inline void FillPatch(const Level& L, MF& mf, int c0, int nc, int bccomp, const std::vector<BCRec>& bcs,
                      bool is_vel, int state_comp0 = -1) {
    FillBoundary(L, mf, c0, nc, mf.ng);
    PhysFill(L, mf, c0, nc, mf.ng, bcs, bccomp, is_vel, state_comp0);
}

}  // namespace mo
