// Test infrastructure only: CPU oracle of the MAESTROeX scalar-advection stage (3-D,
// planar geometry, one AMR level).  It restates, function by function, the reference's
// AdvancePremac -> DensityAdvance -> EnthalpyAdvance call chain so that the GPU library
// can be checked against it; it is never linked into or called by the product.
//
// Parity status: pinned (see maestro_oracle.h).
//
// Build: -O3 -ffp-contract=off (no FMA contraction), no fast-math, so every expression is
// evaluated in the reference's operation order with IEEE binary64 rounding.
#include "maestro_oracle.h"

#include <algorithm>
#include <cstring>
#include <string>

#include "mo_amr.hpp"
#include "mo_ppm.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace mo {

static thread_local std::string g_err;

// One AMR level of the stage: the per-level bodies of the reference functions.  The
// coarse-fine synchronisation the reference runs between them (AverageDown, FillPatch,
// AverageDownFaces, FillPatchUedge) lives in Stage below.
struct Lev {
    mo_params P;
    Level L;
    int lev = 0, cutoff = 0;  // level index, base_cutoff_density_coord(lev)
    int nspec = 0, nscal = 0, nb = 0, nr = 0;
    int ng_s = 3, ng_adv = 3;
    std::vector<BCRec> bcs_s, bcs_u, bcs_f;
    std::vector<real> rho0_old, rho0_new, rhoh0_old, rhoh0_new, p0_old, p0_new, psi, grav_cell,
        w0_force, w0, rho0_predicted_edge;
    MF w0_cart;  // 3 comps, 2 ghosts
    MF gpi, thermal;
    PPMCtx pc;
    double dt = 0, rel_eps = 0;

    // ------------------------------------------------------------------ spherical
    // Full-star geometry: centre, the radii of the radial grid (Source/BaseStateGeometry.cpp:
    // 86-104) -- the exact (irregular) grid, or uniform bins of drf = dxf / drdxfac -- and w0 on
    // faces (MakeW0mac).
    double center[3] = {0.0, 0.0, 0.0};
    double dxf = 0.0;  // finest cell size: it sets the radial grid of every level
    double drf = 0.0;  // base_geom.dr_fine = dxf / drdxfac (Source/MaestroSetup.cpp:68)
    std::vector<double> r_cc_loc, r_edge_loc;
    MF w0mac[3];

    void InitSphr() {
        for (int d = 0; d < 3; ++d) center[d] = 0.5 * (P.prob_lo[d] + P.prob_hi[d]);
        drf = dxf / (P.drdxfac > 0 ? P.drdxfac : 1);
        // one radius past the last cell: Put1dArrayOnCart reads r_cc_loc(nr_fine) for the
        // outermost cells (Source/MaestroFill3dData.cpp:115-118, past its array); the
        // same formula continued
        r_cc_loc.assign(nr + 1, 0.0);
        r_edge_loc.assign(nr + 1, 0.0);
        if (P.use_exact_base_state) {
            for (int i = 0; i <= nr; ++i) r_cc_loc[i] = std::sqrt(0.75 + 2.0 * double(i)) * dxf;
            for (int i = 0; i < nr; ++i) r_edge_loc[i + 1] = std::sqrt(0.75 + 2.0 * (double(i) + 0.5)) * dxf;
        } else {
            for (int i = 0; i <= nr; ++i) r_cc_loc[i] = (double(i) + 0.5) * drf;
            for (int i = 0; i <= nr; ++i) r_edge_loc[i] = double(i) * drf;
        }
    }
    // Put1dArrayOnCart's value of a cell-centred array at cell (i, j, k)
    real sph_cell_at(const std::vector<real>& s0, int i, int j, int k) const {
        if (P.use_exact_base_state) return s0[cc_to_r(i, j, k)];
        double x, y, z;
        sph_xyz(i, j, k, x, y, z);
        return sph_cell_value(s0, std::sqrt(x * x + y * y + z * z), s0_interp());
    }
    int w0_interp() const { return P.w0_interp_type ? P.w0_interp_type : 2; }
    int w0mac_interp() const { return P.w0mac_interp_type ? P.w0mac_interp_type : 1; }
    int s0_interp() const { return P.s0_interp_type ? P.s0_interp_type : 3; }
    // QuadInterp with its limiter on, the default of its declaration (Source/Maestro.H:65-68,
    // Source/MaestroFill3dData.cpp:338-355): the quadratic through three points, clipped to
    // the range of their values
    static real QuadInterp(real x, real x0, real x1, real x2, real y0, real y1, real y2) {
        real y = y0 + (y1 - y0) / (x1 - x0) * (x - x0) +
                 ((y2 - y1) / (x2 - x1) - (y1 - y0) / (x1 - x0)) / (x2 - x0) * (x - x0) * (x - x1);
        const real m12 = y1 > y2 ? y1 : y2, mx = y0 > m12 ? y0 : m12;
        const real n12 = y1 < y2 ? y1 : y2, mn = y0 < n12 ? y0 : n12;
        if (y > mx) y = mx;
        if (y < mn) y = mn;
        return y;
    }
    // Put1dArrayOnCart's value of an edge-centred array at radius `radius`: index is the
    // cell's bin (cc_to_r with the exact grid, int(radius / drf) with uniform bins) and rfac
    // its fraction (Source/MaestroFill3dData.cpp:111-159, 207-256)
    real sph_edge_value(const std::vector<real>& s0, double radius, int index) const {
        double rfac;
        if (P.use_exact_base_state) {
            if (index < nr) rfac = (radius - r_edge_loc[index + 1]) / (r_cc_loc[index + 1] - r_cc_loc[index]);
            else rfac = (radius - r_edge_loc[index + 1]) / (r_cc_loc[index] - r_cc_loc[index - 1]);
        } else {
            rfac = (radius - double(index) * drf) / drf;
        }
        const int t = w0_interp();
        if (t == 1) return rfac > 0.5 ? s0[index + 1] : s0[index];
        if (t == 2) return index < nr ? rfac * s0[index + 1] + (1.0 - rfac) * s0[index] : s0[nr];
        if (index <= 0) index = 0;
        else if (index >= nr - 1) index = nr - 2;
        else if (radius - r_edge_loc[index] < r_edge_loc[index + 1]) index--;
        return QuadInterp(radius, r_edge_loc[index], r_edge_loc[index + 1], r_edge_loc[index + 2], s0[index],
                          s0[index + 1], s0[index + 2]);
    }
    // Put1dArrayOnCart's value of a cell-centred array, uniform bins, s0_interp_type
    // (Source/MaestroFill3dData.cpp:259-320); an index past the last bin takes the last value
    // whichever way the reference's comparison (which reads past its radii there) goes
    real sph_cell_value(const std::vector<real>& s0, double radius, int t) const {
        int index = int(radius / drf);
        if (t == 1) return s0[index];
        if (t == 2) {
            if (index > nr - 1) return s0[nr - 1];
            if (radius >= r_cc_loc[index]) {
                if (index >= nr - 1) return s0[nr - 1];
                return s0[index + 1] * (radius - r_cc_loc[index]) / drf + s0[index] * (r_cc_loc[index + 1] - radius) / drf;
            }
            if (index == 0) return s0[index];
            return s0[index] * (radius - r_cc_loc[index - 1]) / drf + s0[index - 1] * (r_cc_loc[index] - radius) / drf;
        }
        if (index == 0) index = 1;
        else if (index >= nr - 1) index = nr - 2;
        return QuadInterp(radius, r_cc_loc[index - 1], r_cc_loc[index], r_cc_loc[index + 1], s0[index - 1], s0[index],
                          s0[index + 1]);
    }
    // cell centre relative to the star's centre (Source/MaestroFill3dData.cpp:103-110)
    void sph_xyz(int i, int j, int k, double& x, double& y, double& z) const {
        x = P.prob_lo[0] + (double(i) + 0.5) * L.dx[0] - center[0];
        y = P.prob_lo[1] + (double(j) + 0.5) * L.dx[1] - center[1];
        z = P.prob_lo[2] + (double(k) + 0.5) * L.dx[2] - center[2];
    }
    // Maestro::InitBaseStateMapSphr (Source/MaestroBaseStateGeometry.cpp:17-35)
    int cc_to_r(int i, int j, int k) const {
        double x, y, z;
        sph_xyz(i, j, k, x, y, z);
        const double index = (x * x + y * y + z * z) / (2.0 * dxf * dxf) - 0.375;
        return (int)std::round(index);
    }
    // Put1dArrayOnCart, spherical (Source/MaestroFill3dData.cpp:94-336): an edge-centred
    // input with w0_interp_type, a cell-centred one injected (exact grid) or interpolated
    // with s0_interp_type (uniform bins); vector output = value times the radial unit vector
    void Put1dSphr(const std::vector<real>& s0, MF& s0_cart, bool edge, bool vec) {
        for (int b = 0; b < nb; ++b) {
            const Arr& a = s0_cart[b];
            MO_FOR3(L.ba[b]) {
                double x, y, z;
                sph_xyz(i, j, k, x, y, z);
                const double radius = std::sqrt(x * x + y * y + z * z);
                const int index = P.use_exact_base_state ? cc_to_r(i, j, k) : int(radius / drf);
                real v;
                if (edge) v = sph_edge_value(s0, radius, index);
                else v = P.use_exact_base_state ? s0[index] : sph_cell_value(s0, radius, s0_interp());
                if (vec) {
                    a(i, j, k, 0) = v * x / radius;
                    a(i, j, k, 1) = v * y / radius;
                    a(i, j, k, 2) = v * z / radius;
                } else {
                    a(i, j, k, 0) = v;
                }
            }
        }
    }
    // w0 interpolated linearly in uniform bins of drf at radius `radius` (MakeW0mac types 2, 4)
    real w0_linear(double radius) const {
        const int index = int(radius / drf);
        const double rfac = (radius - double(index) * drf) / drf;
        return index < nr ? rfac * w0[index + 1] + (1.0 - rfac) * w0[index] : w0[nr];
    }
    // Maestro::MakeW0mac (Source/MaestroFill3dData.cpp:464-710) over the nodal boxes grown by
    // one: w0mac_interp_type 1 averages w0_cart to the faces; 2 / 3 interpolate w0 at the
    // face centres (linear in uniform bins / quadratic in r_edge_loc); 4 interpolates it at
    // the nodes (grown by one) and averages their four values on each face
    void MakeW0mac() {
        const int t = w0mac_interp();
        MF w0_nodal;
        if (t == 4) {
            // node (i,j,k) kept at cell (i,j,k): two ghost cells hold the nodes of the box grown by one
            w0_nodal.define(L.ba, 3, 2, -1, 0.0);
            for (int b = 0; b < nb; ++b) {
                Box nb1 = grow(L.ba[b], 1);
                for (int d = 0; d < 3; ++d) nb1.hi[d] += 1;
                const Arr& o = w0_nodal[b];
                MO_FOR3(nb1) {
                    const double x = P.prob_lo[0] + double(i) * L.dx[0] - center[0];
                    const double y = P.prob_lo[1] + double(j) * L.dx[1] - center[1];
                    const double z = P.prob_lo[2] + double(k) * L.dx[2] - center[2];
                    const double radius = std::sqrt(x * x + y * y + z * z);
                    const real v = w0_linear(radius);
                    if (radius == 0.0) {
                        for (int n = 0; n < 3; ++n) o(i, j, k, n) = v;
                    } else {
                        o(i, j, k, 0) = v * x / radius;
                        o(i, j, k, 1) = v * y / radius;
                        o(i, j, k, 2) = v * z / radius;
                    }
                }
            }
        }
        for (int d = 0; d < 3; ++d) {
            w0mac[d].define(L.ba, 1, 1, d, 0.0);
            const int di = d == 0, dj = d == 1, dk = d == 2;
            for (int b = 0; b < nb; ++b) {
                const Arr& wc = w0_cart[b];
                const Arr& o = w0mac[d][b];
                MO_FOR3(grow(nodal(L.ba[b], d), 1)) {
                    if (t == 1) {
                        o(i, j, k) = 0.5 * (wc(i - di, j - dj, k - dk, d) + wc(i, j, k, d));
                    } else if (t == 2 || t == 3) {
                        const double x = P.prob_lo[0] + (double(i) + (di ? 0.0 : 0.5)) * L.dx[0] - center[0];
                        const double y = P.prob_lo[1] + (double(j) + (dj ? 0.0 : 0.5)) * L.dx[1] - center[1];
                        const double z = P.prob_lo[2] + (double(k) + (dk ? 0.0 : 0.5)) * L.dx[2] - center[2];
                        const double radius = std::sqrt(x * x + y * y + z * z);
                        real v;
                        if (t == 2) {
                            v = w0_linear(radius);
                        } else {
                            int index = int(radius / drf);
                            if (index <= 0) index = 0;
                            else if (index >= nr - 1) index = nr - 2;
                            else if (radius - r_edge_loc[index] < r_edge_loc[index + 1]) index--;
                            v = QuadInterp(radius, r_edge_loc[index], r_edge_loc[index + 1], r_edge_loc[index + 2],
                                           w0[index], w0[index + 1], w0[index + 2]);
                        }
                        o(i, j, k) = v * (d == 0 ? x : d == 1 ? y : z) / radius;
                    } else {
                        const Arr& wn = w0_nodal[b];
                        // the four nodes of the face: the two transverse directions, low / high
                        const int T1 = d == 0 ? 1 : 0, T2 = d == 2 ? 1 : 2;
                        int a1[3] = {0, 0, 0}, a2[3] = {0, 0, 0};
                        a1[T1] = 1;
                        a2[T2] = 1;
                        o(i, j, k) = 0.25 * (wn(i, j, k, d) + wn(i + a1[0], j + a1[1], k + a1[2], d) +
                                             wn(i + a2[0], j + a2[1], k + a2[2], d) +
                                             wn(i + a1[0] + a2[0], j + a1[1] + a2[1], k + a1[2] + a2[2], d));
                    }
                }
            }
        }
    }

    // ------------------------------------------------------------------ setup
    // Maestro::BCSetup (Source/MaestroSetup.cpp:276-500)
    void BCSetup() {
        bcs_s.assign(nscal, BCRec{});
        bcs_u.assign(3, BCRec{});
        bcs_f.assign(nscal, BCRec{});
        for (int dir = 0; dir < 3; ++dir) {
            for (int side = 0; side < 2; ++side) {
                int pb = side == 0 ? P.phys_bc_lo[dir] : P.phys_bc_hi[dir];
                auto set = [&](BCRec& r, int v) { (side == 0 ? r.lo : r.hi)[dir] = v; };
                int u = 0, un = 0, s = 0, spi = 0, f = 0;
                switch (pb) {
                    case interior: u = un = s = spi = f = int_dir; break;
                    case inflow: u = un = ext_dir; s = ext_dir; spi = foextrap; f = foextrap; break;
                    case outflow: u = un = foextrap; s = foextrap; spi = ext_dir; f = foextrap; break;
                    case symmetry: u = reflect_even; un = reflect_odd; s = spi = reflect_even; f = reflect_even; break;
                    case slipwall: u = hoextrap; un = ext_dir; s = hoextrap; spi = foextrap; f = foextrap; break;
                    case noslipwall: u = un = ext_dir; s = hoextrap; spi = foextrap; f = foextrap; break;
                    default: throw std::runtime_error("invalid phys_bc");
                }
                for (int c = 0; c < 3; ++c) set(bcs_u[c], c == dir ? un : u);
                for (int c = 0; c < nscal; ++c) set(bcs_s[c], c == Pi ? spi : s);
                for (int c = 0; c < nscal; ++c) set(bcs_f[c], f);
            }
        }
    }

    // Maestro::Put1dArrayOnCart, planar branch, one level (Source/MaestroFill3dData.cpp:42-93):
    // valid cells from the level's 1-D array.
    void Put1d(const std::vector<real>& s0, MF& s0_cart, bool edge, bool vec) {
        const int outcomp = vec ? 2 : 0;
        for (int b = 0; b < nb; ++b) {
            const Arr& a = s0_cart[b];
            MO_FOR3(L.ba[b]) {
                const int r = k;
                a(i, j, k, outcomp) = edge ? 0.5 * (s0[r] + s0[r + 1]) : s0[r];
            }
        }
    }

    // Maestro::CelltoEdge (Source/MaestroCelltoEdge.cpp:17-54) on one chunk [lo, hi] of
    // edges of a level with nr_lev cells; edges outside the chunk are left alone.
    static void CelltoEdgeChunk(const std::vector<real>& c, std::vector<real>& e, int lo, int hi) {
        const int nr_lev = (int)c.size();
        for (int r = lo; r <= hi; ++r) {
            if (r == 0) {
                e[r] = c[r];
            } else if (r == 1 || r == lo) {
                e[r] = 0.5 * (c[r - 1] + c[r]);
            } else if (r == nr_lev) {
                e[r] = c[r - 1];
            } else if (r == nr_lev - 1 || r == hi) {
                e[r] = 0.5 * (c[r] + c[r - 1]);
            } else {
                real tmp = 7.0 / 12.0 * (c[r] + c[r - 1]) - 1.0 / 12.0 * (c[r + 1] + c[r - 2]);
                real s0min = mn(c[r], c[r - 1]);
                real s0max = mx(c[r], c[r - 1]);
                e[r] = mn(mx(tmp, s0min), s0max);
            }
        }
    }
    // one level, one chunk spanning the level
    static void CelltoEdge(const std::vector<real>& c, std::vector<real>& e) {
        e.assign(c.size() + 1, 0.0);
        CelltoEdgeChunk(c, e, 0, (int)c.size());
    }

    // ------------------------------------------------------------------ face ghosts
    // Maestro::FillUmacGhost (Source/MaestroFillData.cpp:176-453), one level; nd = 2 for
    // the 2-D form (no w faces).
    void FillUmacGhost(MF* um, int nd = 3) {
        const int* dlo = L.dom.lo;
        const int* dhi = L.dom.hi;
        for (int b = 0; b < nb; ++b) {
            const Arr& umac = um[0][b];
            const Arr& vmac = um[1][b];
            const Arr& wmac = nd == 3 ? um[2][b] : um[1][b];
            for (int dd = 0; dd < nd; ++dd) {
                Box gb = grow(nodal(L.ba[b], dd), 1);
                const int bclo = P.phys_bc_lo[dd], bchi = P.phys_bc_hi[dd];
                MO_FOR3(gb) {
                    const int I = dd == 0 ? i : (dd == 1 ? j : k);
                    const int di = dd == 0, dj = dd == 1, dk = dd == 2;
                    // q_n is the face velocity normal to dd, q_t the two tangential ones
                    const Arr* comp[3] = {&umac, &vmac, &wmac};
                    const Arr& qn = *comp[dd];
                    if (I == dlo[dd] - 1) {
                        switch (bclo) {
                            case inflow:
                                for (int c = 0; c < nd; ++c)
                                    (*comp[c])(i, j, k) = c == dd ? qn(i + di, j + dj, k + dk) : 0.0;
                                break;
                            case slipwall:
                            case noslipwall:
                                for (int c = 0; c < nd; ++c) (*comp[c])(i, j, k) = 0.0;
                                break;
                            case outflow:
                                for (int c = 0; c < nd; ++c)
                                    (*comp[c])(i, j, k) = (*comp[c])(i + di, j + dj, k + dk);
                                break;
                            case symmetry:
                                for (int c = 0; c < nd; ++c)
                                    (*comp[c])(i, j, k) = c == dd ? -qn(i + 2 * di, j + 2 * dj, k + 2 * dk)
                                                                  : (*comp[c])(i + di, j + dj, k + dk);
                                break;
                            default: break;
                        }
                    }
                    if (I == dhi[dd] + 2) {
                        switch (bchi) {
                            case inflow:
                                for (int c = 0; c < nd; ++c) {
                                    if (c == dd) qn(i, j, k) = qn(i - di, j - dj, k - dk);
                                    else (*comp[c])(i - di, j - dj, k - dk) = 0.0;
                                }
                                break;
                            case slipwall:
                            case noslipwall:
                                for (int c = 0; c < nd; ++c) {
                                    if (c == dd) qn(i, j, k) = 0.0;
                                    else (*comp[c])(i - di, j - dj, k - dk) = 0.0;
                                }
                                break;
                            case outflow:
                                for (int c = 0; c < nd; ++c) {
                                    if (c == dd) qn(i, j, k) = qn(i - di, j - dj, k - dk);
                                    else (*comp[c])(i - di, j - dj, k - dk) = (*comp[c])(i - 2 * di, j - 2 * dj, k - 2 * dk);
                                }
                                break;
                            case symmetry:
                                for (int c = 0; c < nd; ++c) {
                                    if (c == dd) qn(i, j, k) = -qn(i - 2 * di, j - 2 * dj, k - 2 * dk);
                                    else (*comp[c])(i - di, j - dj, k - dk) = (*comp[c])(i - 2 * di, j - 2 * dj, k - 2 * dk);
                                }
                                break;
                            default: break;
                        }
                    }
                }
            }
        }
    }

    // Maestro::Addw0, planar, one level (Source/MaestroFill3dData.cpp:365-423)
    void Addw0(MF* uedge, real mult) {
        if (P.spherical) {  // Source/MaestroFill3dData.cpp:395-419: valid faces += mult w0mac
            for (int b = 0; b < nb; ++b)
                for (int d = 0; d < 3; ++d) {
                    const Arr& e = uedge[d][b];
                    const Arr& w = w0mac[d][b];
                    MO_FOR3(nodal(L.ba[b], d)) { e(i, j, k) += mult * w(i, j, k); }
                }
            return;
        }
        for (int b = 0; b < nb; ++b) {
            const Arr& wedge = uedge[2][b];
            Box zbx = grow(grow(nodal(L.ba[b], 2), 0, 1), 1, 1);
            MO_FOR3(zbx) { wedge(i, j, k) += mult * w0[k]; }
        }
    }

    // ------------------------------------------------------------------ MakeUtrans
    // Maestro::MakeUtrans, 3-D, one level (Source/MaestroMakeUtrans.cpp:6-56, 270-628)
    void MakeUtrans(MF& utilde, MF& ufull, MF* utrans) {
        const real dt2 = 0.5 * dt;
        const int* domlo = L.dom.lo;
        const int* domhi = L.dom.hi;
        MF Ip, Im;
        Ip.define(L.ba, 3, 2);
        Im.define(L.ba, 3, 2);
        MF& velsrc = (P.ppm_type == 0) ? utilde : ufull;  // u_mf / v_mf / w_mf copies
        for (int d = 0; d < 3; ++d) {
#pragma omp parallel for schedule(dynamic)
            for (int b = 0; b < nb; ++b) {
                const Box obx = grow(L.ba[b], 1);
                const Box xbx = nodal(L.ba[b], d);
                const Arr& ut = utilde[b];
                const Arr& uf = ufull[b];
                const Arr& Ipa = Ip[b];
                const Arr& Ima = Im[b];
                const Arr& tr = utrans[d][b];
                const Arr& w0a = w0_cart[b];
                if (P.ppm_type == 0) {
                    Slope_dir(P.slope_order, L.dom, obx, velsrc[b].comp(d), Ipa, 1, bcs_u, d, d);
                } else {
                    PPM(pc, obx, ut, velsrc[b].comp(0), velsrc[b].comp(1), velsrc[b].comp(2), Ipa, Ima,
                        bcs_u[d], false, d);
                }
                const int bclo = P.phys_bc_lo[d], bchi = P.phys_bc_hi[d];
                const int di = d == 0, dj = d == 1, dk = d == 2;
                MO_FOR3(xbx) {
                    const int I = d == 0 ? i : (d == 1 ? j : k);
                    real l = 0.0, r = 0.0;
                    if (P.ppm_type == 0) {
                        l = ut(i - di, j - dj, k - dk, d) +
                            (0.5 - (dt2 / L.dx[d]) * mx(0.0, uf(i - di, j - dj, k - dk, d))) *
                                Ipa(i - di, j - dj, k - dk, 0);
                        r = ut(i, j, k, d) - (0.5 + (dt2 / L.dx[d]) * mn(0.0, uf(i, j, k, d))) * Ipa(i, j, k, 0);
                    } else {
                        l = Ipa(i - di, j - dj, k - dk, d);
                        r = Ima(i, j, k, d);
                    }
                    if (I == domlo[d]) {
                        switch (bclo) {
                            case inflow: l = ut(i - di, j - dj, k - dk, d); r = ut(i - di, j - dj, k - dk, d); break;
                            case slipwall: case noslipwall: case symmetry: l = 0.0; r = 0.0; break;
                            case outflow: l = mn(r, 0.0); r = l; break;
                            default: break;
                        }
                    } else if (I == domhi[d] + 1) {
                        switch (bchi) {
                            case inflow: l = ut(i + di, j + dj, k + dk, d); r = ut(i + di, j + dj, k + dk, d); break;
                            case slipwall: case noslipwall: case symmetry: l = 0.0; r = 0.0; break;
                            case outflow: l = mx(l, 0.0); r = l; break;
                            default: break;
                        }
                    }
                    if (P.spherical) {  // Source/MaestroMakeUtrans.cpp:368-377: with w0mac
                        const real w0c = w0mac[d][b](i, j, k);
                        bool test = (l + w0c <= 0.0 && r + w0c >= 0.0) || (fab(l + r + 2.0 * w0c) < rel_eps);
                        real v = 0.5 * (l + r) + w0c > 0.0 ? l : r;
                        tr(i, j, k) = test ? 0.0 : v;
                    } else if (d < 2) {
                        bool test = (l <= 0.0 && r >= 0.0) || (fab(l + r) < rel_eps);
                        real v = 0.5 * (l + r) > 0.0 ? l : r;
                        tr(i, j, k) = test ? 0.0 : v;
                    } else {
                        const real w0c = w0a(i, j, k, 2);
                        bool test = (l + w0c <= 0.0 && r + w0c >= 0.0) || (fab(l + r + 2.0 * w0c) < rel_eps);
                        real v = 0.5 * (l + r) + w0c > 0.0 ? l : r;
                        tr(i, j, k) = test ? 0.0 : v;
                    }
                }
            }
        }
    }

    // ------------------------------------------------------------------ MakeVelForce
    // Maestro::MakeVelForce, planar, one level (Source/MaestroForce.cpp:58-126)
    void MakeVelForce(MF& vel_force, MF* uedge, MF& sold, MF& w0_force_cart, MF& grav_cart, MF& rho0_cart,
                      const MF* gradw0_cart = nullptr) {
        vel_force.setVal(0.0);
        if (P.spherical) {
            // Source/MaestroForce.cpp:151-252; gradw0_cart holds dw0/dr of the uniform bins; the
            // exact base state has gradw0 = 0 (:30-41), so the utilde term subtracts Ut.e_r * 0 * e_r
            for (int b = 0; b < nb; ++b) {
                const Arr& gpi_arr = gpi[b];
                const Arr& rho_arr = sold[b];
                const Arr& ue = uedge[0][b];
                const Arr& ve = uedge[1][b];
                const Arr& we = uedge[2][b];
                const Arr& w0f = w0_force_cart[b];
                const Arr& grav = grav_cart[b];
                const Arr& r0 = rho0_cart[b];
                const Arr& vf = vel_force[b];
                MO_FOR3(L.ba[b]) {
                    double x, y, z;
                    sph_xyz(i, j, k, x, y, z);
                    const double inv_radius = 1.0 / std::sqrt(x * x + y * y + z * z);  // MakeNormal
                    const double nrm[3] = {x * inv_radius, y * inv_radius, z * inv_radius};
                    real rhopert = rho_arr(i, j, k) - r0(i, j, k);
                    if (rho_arr(i, j, k) < (P.buoyancy_cutoff_factor * P.base_cutoff_density)) rhopert = 0.0;
                    for (int dim = 0; dim < 3; ++dim)
                        vf(i, j, k, dim) =
                            (rhopert * grav(i, j, k, dim) - gpi_arr(i, j, k, dim)) / rho_arr(i, j, k) - w0f(i, j, k, dim);
                    const real ut_dot_er = 0.5 * (ue(i, j, k) + ue(i + 1, j, k)) * nrm[0] +
                                             0.5 * (ve(i, j, k) + ve(i, j + 1, k)) * nrm[1] +
                                             0.5 * (we(i, j, k) + we(i, j, k + 1)) * nrm[2];
                    const real gradw0 = gradw0_cart ? (*gradw0_cart)[b](i, j, k) : real(0.0);
                    for (int dim = 0; dim < 3; ++dim) vf(i, j, k, dim) -= ut_dot_er * gradw0 * nrm[dim];
                }
            }
            return;
        }
        const int domhi = L.dom.hi[2];
        for (int b = 0; b < nb; ++b) {
            const Arr& gpi_arr = gpi[b];
            const Arr& rho_arr = sold[b];
            const Arr& wedge = uedge[2][b];
            const Arr& w0_arr = w0_cart[b];
            const Arr& w0f = w0_force_cart[b];
            const Arr& grav = grav_cart[b];
            const Arr& r0 = rho0_cart[b];
            const Arr& vf = vel_force[b];
            MO_FOR3(L.ba[b]) {
                real rhopert = rho_arr(i, j, k) - r0(i, j, k);
                if (rho_arr(i, j, k) < (P.buoyancy_cutoff_factor * P.base_cutoff_density)) rhopert = 0.0;
                for (int dim = 0; dim < 2; ++dim) vf(i, j, k, dim) = -gpi_arr(i, j, k, dim) / rho_arr(i, j, k);
                vf(i, j, k, 2) = (rhopert * grav(i, j, k, 2) - gpi_arr(i, j, k, 2)) / rho_arr(i, j, k) - w0f(i, j, k, 2);
                if (k <= -1 || k >= domhi) {
                } else {
                    vf(i, j, k, 2) -= (wedge(i, j, k + 1) + wedge(i, j, k)) *
                                      (w0_arr(i, j, k + 1, 2) - w0_arr(i, j, k, 2)) / (2.0 * L.dx[2]);
                }
            }
        }
    }

    // ------------------------------------------------------------------ VelPred
    // Maestro::VelPred, 3-D, one level (Source/MaestroVelPred.cpp:5-288, 735-1915)
    void VelPred(MF& utilde, MF& ufull, MF* utrans, MF* umac, MF& force) {
        const real dt2 = 0.5 * dt, dt4 = 0.25 * dt, dt6 = dt / 6.0;
        const int* domlo = L.dom.lo;
        const int* domhi = L.dom.hi;
        const real h[3] = {L.dx[0], L.dx[1], L.dx[2]};
        // Ipu..Imw: per velocity component c, 3 directional comps, 1 ghost
        MF Ipc[3], Imc[3];
        for (int c = 0; c < 3; ++c) {
            Ipc[c].define(L.ba, 3, 1);
            Imc[c].define(L.ba, 3, 1);
        }
        MF ul[3], ur[3], uimh[3];  // ulx/urx/uimhx ... 3 comps, 1 ghost
        for (int d = 0; d < 3; ++d) {
            ul[d].define(L.ba, 3, 1);
            ur[d].define(L.ba, 3, 1);
            uimh[d].define(L.ba, 3, 1);
        }
        // transverse states q_{d|t} of component c = the third direction: index [c][d]
        MF qimh[3][3];
        for (int c = 0; c < 3; ++c)
            for (int d = 0; d < 3; ++d)
                if (c != d) qimh[c][d].define(L.ba, 1, 1);
        MF& velsrc = (P.ppm_type == 0) ? utilde : ufull;
        // ppm_trace_forces: the force of each component traced like the component (Ipfx..Imfz)
        const bool ptf = P.ppm_trace_forces == 1;
        MF Ipf[3], Imf[3];
        if (ptf)
            for (int c = 0; c < 3; ++c) {
                Ipf[c].define(L.ba, 3, 1);
                Imf[c].define(L.ba, 3, 1);
            }
#pragma omp parallel for schedule(dynamic)
        for (int b = 0; b < nb; ++b) {
            const Box obx = grow(L.ba[b], 1);
            const Arr& ut = utilde[b];
            const Arr& uf = ufull[b];
            // PPM / slopes (:205-255)
            if (P.ppm_type == 0) {
                Slope_dir(P.slope_order, L.dom, obx, ut, Ipc[0][b], 3, bcs_u, 0, 0);  // slopex -> Ipu
                Slope_dir(P.slope_order, L.dom, obx, ut, Imc[1][b], 3, bcs_u, 0, 1);  // slopey -> Imv
                Slope_dir(P.slope_order, L.dom, obx, ut, Imc[2][b], 3, bcs_u, 0, 2);  // slopez -> Imw
            } else {
                for (int c = 0; c < 3; ++c) {
                    PPM(pc, obx, ut, velsrc[b].comp(0), velsrc[b].comp(1), velsrc[b].comp(2), Ipc[c][b], Imc[c][b],
                        bcs_u[c], false, c);
                    if (ptf)  // (:117-137, 203-247)
                        PPM(pc, obx, force[b], velsrc[b].comp(0), velsrc[b].comp(1), velsrc[b].comp(2), Ipf[c][b],
                            Imf[c][b], bcs_u[c], false, c);
                }
            }
            // VelPredInterface (:735-1128)
            for (int d = 0; d < 3; ++d) {
                const Box mbx = growLo(obx, d, -1);
                const int di = d == 0, dj = d == 1, dk = d == 2;
                const int bclo = P.phys_bc_lo[d], bchi = P.phys_bc_hi[d];
                const Arr& l = ul[d][b];
                const Arr& r = ur[d][b];
                const Arr& im = uimh[d][b];
                const Arr& tr = utrans[d][b];
                const Arr& slope = (d == 0) ? Ipc[0][b] : (d == 1 ? Imc[1][b] : Imc[2][b]);
                MO_FOR3(mbx) {
                    const int I = d == 0 ? i : (d == 1 ? j : k);
                    if (P.ppm_type == 0) {
                        real maxu = 0.5 - dt2 * mx(0.0, uf(i - di, j - dj, k - dk, d)) / h[d];
                        real minu = 0.5 + dt2 * mn(0.0, uf(i, j, k, d)) / h[d];
                        for (int n = 0; n < 3; ++n) {
                            l(i, j, k, n) = ut(i - di, j - dj, k - dk, n) + maxu * slope(i - di, j - dj, k - dk, n);
                            r(i, j, k, n) = ut(i, j, k, n) - minu * slope(i, j, k, n);
                        }
                    } else {
                        for (int n = 0; n < 3; ++n) {
                            l(i, j, k, n) = Ipc[n][b](i - di, j - dj, k - dk, d);
                            r(i, j, k, n) = Imc[n][b](i, j, k, d);
                        }
                    }
                    if (I == domlo[d]) {
                        switch (bclo) {
                            case inflow:
                                for (int n = 0; n < 3; ++n) {
                                    l(i, j, k, n) = ut(i - di, j - dj, k - dk, n);
                                    r(i, j, k, n) = ut(i - di, j - dj, k - dk, n);
                                }
                                break;
                            case slipwall:
                            case symmetry:
                                for (int n = 0; n < 3; ++n) {
                                    if (n == d) { l(i, j, k, n) = 0.0; r(i, j, k, n) = 0.0; }
                                    else l(i, j, k, n) = r(i, j, k, n);
                                }
                                break;
                            case noslipwall:
                                for (int n = 0; n < 3; ++n) { l(i, j, k, n) = 0.0; r(i, j, k, n) = 0.0; }
                                break;
                            case outflow:
                                r(i, j, k, d) = mn(r(i, j, k, d), 0.0);
                                for (int n = 0; n < 3; ++n) l(i, j, k, n) = r(i, j, k, n);
                                break;
                            default: break;
                        }
                    } else if (I == domhi[d] + 1) {
                        switch (bchi) {
                            case inflow:
                                for (int n = 0; n < 3; ++n) {
                                    l(i, j, k, n) = ut(i, j, k, n);
                                    r(i, j, k, n) = ut(i, j, k, n);
                                }
                                break;
                            case slipwall:
                            case symmetry:
                                for (int n = 0; n < 3; ++n) {
                                    if (n == d) { l(i, j, k, n) = 0.0; r(i, j, k, n) = 0.0; }
                                    else r(i, j, k, n) = l(i, j, k, n);
                                }
                                break;
                            case noslipwall:
                                for (int n = 0; n < 3; ++n) { l(i, j, k, n) = 0.0; r(i, j, k, n) = 0.0; }
                                break;
                            case outflow:
                                l(i, j, k, d) = mx(l(i, j, k, d), 0.0);
                                for (int n = 0; n < 3; ++n) r(i, j, k, n) = l(i, j, k, n);
                                break;
                            default: break;
                        }
                    }
                    for (int n = 0; n < 3; ++n) {
                        if (n == d) continue;
                        real v = tr(i, j, k) > 0.0 ? l(i, j, k, n) : r(i, j, k, n);
                        im(i, j, k, n) = fab(tr(i, j, k)) < rel_eps ? 0.5 * (l(i, j, k, n) + r(i, j, k, n)) : v;
                    }
                }
            }
            // VelPredTransverse (:1130-1595): component c on faces d, transverse t
            for (int c = 0; c < 3; ++c)
                for (int d = 0; d < 3; ++d) {
                    if (c == d) continue;
                    const int t = 3 - c - d;
                    Box imhbox = growHi(grow(L.ba[b], c, 1), d, 1);
                    const int di = d == 0, dj = d == 1, dk = d == 2;
                    const int ti = t == 0, tj = t == 1, tk = t == 2;
                    const int bclo = P.phys_bc_lo[d], bchi = P.phys_bc_hi[d];
                    const Arr& l = ul[d][b];
                    const Arr& r = ur[d][b];
                    const Arr& trt = utrans[t][b];
                    const Arr& imt = uimh[t][b];
                    const Arr& trd = utrans[d][b];
                    const Arr& out = qimh[c][d][b];
                    MO_FOR3(imhbox) {
                        const int I = d == 0 ? i : (d == 1 ? j : k);
                        const int il = i - di, jl = j - dj, kl = k - dk;
                        real lq = l(i, j, k, c) - (dt6 / h[t]) * (trt(il + ti, jl + tj, kl + tk) + trt(il, jl, kl)) *
                                                        (imt(il + ti, jl + tj, kl + tk, c) - imt(il, jl, kl, c));
                        real rq = r(i, j, k, c) - (dt6 / h[t]) * (trt(i + ti, j + tj, k + tk) + trt(i, j, k)) *
                                                        (imt(i + ti, j + tj, k + tk, c) - imt(i, j, k, c));
                        if (I == domlo[d]) {
                            switch (bclo) {
                                case inflow: lq = ut(il, jl, kl, c); rq = ut(il, jl, kl, c); break;
                                case slipwall: case symmetry: case outflow: lq = rq; break;
                                case noslipwall: lq = 0.0; rq = 0.0; break;
                                default: break;
                            }
                        } else if (I == domhi[d] + 1) {
                            switch (bchi) {
                                case inflow: lq = ut(i, j, k, c); rq = ut(i, j, k, c); break;
                                case slipwall: case symmetry: case outflow: rq = lq; break;
                                case noslipwall: lq = 0.0; rq = 0.0; break;
                                default: break;
                            }
                        }
                        real v = trd(i, j, k) > 0.0 ? lq : rq;
                        out(i, j, k) = fab(trd(i, j, k)) < rel_eps ? 0.5 * (lq + rq) : v;
                    }
                }
            // VelPredVelocities (:1597-1915)
            for (int d = 0; d < 3; ++d) {
                const Box xbx = nodal(L.ba[b], d);
                const int di = d == 0, dj = d == 1, dk = d == 2;
                const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
                const int a1i = t1 == 0, a1j = t1 == 1, a1k = t1 == 2;
                const int a2i = t2 == 0, a2j = t2 == 1, a2k = t2 == 2;
                const Arr& l = ul[d][b];
                const Arr& r = ur[d][b];
                const Arr& tr1 = utrans[t1][b];
                const Arr& tr2 = utrans[t2][b];
                const Arr& q1 = qimh[d][t1][b];  // e.g. uimhyz for d = x
                const Arr& q2 = qimh[d][t2][b];  // e.g. uimhzy
                const Arr& f = force[b];
                const Arr& out = umac[d][b];
                const Arr& w0a = w0_cart[b];
                const int bclo = P.phys_bc_lo[d], bchi = P.phys_bc_hi[d];
                MO_FOR3(xbx) {
                    const int I = d == 0 ? i : (d == 1 ? j : k);
                    const int il = i - di, jl = j - dj, kl = k - dk;
                    // the traced force if ppm_trace_forces = 1 (:581-584, 656-659, 1644-1647)
                    real fl = ptf ? Ipf[d][b](il, jl, kl, d) : f(il, jl, kl, d);
                    real fr = ptf ? Imf[d][b](i, j, k, d) : f(i, j, k, d);
                    real ml = l(i, j, k, d) -
                                (dt4 / h[t1]) * (tr1(il + a1i, jl + a1j, kl + a1k) + tr1(il, jl, kl)) *
                                    (q1(il + a1i, jl + a1j, kl + a1k) - q1(il, jl, kl)) -
                                (dt4 / h[t2]) * (tr2(il + a2i, jl + a2j, kl + a2k) + tr2(il, jl, kl)) *
                                    (q2(il + a2i, jl + a2j, kl + a2k) - q2(il, jl, kl)) +
                                dt2 * fl;
                    real mr = r(i, j, k, d) -
                                (dt4 / h[t1]) * (tr1(i + a1i, j + a1j, k + a1k) + tr1(i, j, k)) *
                                    (q1(i + a1i, j + a1j, k + a1k) - q1(i, j, k)) -
                                (dt4 / h[t2]) * (tr2(i + a2i, j + a2j, k + a2k) + tr2(i, j, k)) *
                                    (q2(i + a2i, j + a2j, k + a2k) - q2(i, j, k)) +
                                dt2 * fr;
                    if (P.spherical) {  // Source/MaestroVelPred.cpp:1664-1673: with w0mac
                        const real w0c = w0mac[d][b](i, j, k);
                        bool test = (ml + w0c <= 0.0 && mr + w0c >= 0.0) || (fab(ml + mr + 2.0 * w0c) < rel_eps);
                        real v = 0.5 * (ml + mr) + w0c > 0.0 ? ml : mr;
                        out(i, j, k) = test ? 0.0 : v;
                    } else if (d < 2) {
                        bool test = (ml <= 0.0 && mr >= 0.0) || (fab(ml + mr) < rel_eps);
                        real v = 0.5 * (ml + mr) > 0.0 ? ml : mr;
                        out(i, j, k) = test ? 0.0 : v;
                    } else {
                        const real w0c = w0a(i, j, k, 2);
                        bool test = (ml + w0c <= 0.0 && mr + w0c >= 0.0) || (fab(ml + mr + 2.0 * w0c) < rel_eps);
                        real v = 0.5 * (ml + mr) + w0c > 0.0 ? ml : mr;
                        out(i, j, k) = test ? 0.0 : v;
                    }
                    if (I == domlo[d]) {
                        switch (bclo) {
                            case inflow: out(i, j, k) = ut(il, jl, kl, d); break;
                            case slipwall: case symmetry: case noslipwall: out(i, j, k) = 0.0; break;
                            case outflow: out(i, j, k) = mn(mr, 0.0); break;
                            default: break;
                        }
                    } else if (I == domhi[d] + 1) {
                        switch (bchi) {
                            case inflow: out(i, j, k) = ut(i, j, k, d); break;
                            case slipwall: case symmetry: case noslipwall: out(i, j, k) = 0.0; break;
                            case outflow: out(i, j, k) = mx(ml, 0.0); break;
                            default: break;
                        }
                    }
                }
            }
        }
    }

    // ------------------------------------------------------------------ MakeEdgeScal
    // Maestro::MakeDivU (Source/MaestroMakeEdgeScalars.cpp:648-660)
    void MakeDivU(const Box& bx, const Arr& divu, const Arr& u, const Arr& v, const Arr& w) {
        MO_FOR3(bx) {
            divu(i, j, k) = u(i + 1, j, k) - u(i, j, k) + v(i, j + 1, k) - v(i, j, k) + w(i, j, k + 1) - w(i, j, k);
            divu(i, j, k) /= L.dx[0];
        }
    }

    // Maestro::MakeEdgeScal, 3-D, is_vel = false (Source/MaestroMakeEdgeScalars.cpp:6-302,
    // 662-1667).  BC overrides of the is_vel branches are kept for completeness.
    void MakeEdgeScal(MF& state, MF* sedge, MF* umac, MF& force, const std::vector<BCRec>& bcs, int start_scomp,
                      int start_bccomp, int num_comp, bool is_conservative, bool is_vel = false) {
        const int* domlo = L.dom.lo;
        const int* domhi = L.dom.hi;
        const real h[3] = {L.dx[0], L.dx[1], L.dx[2]};
        MF Ip, Im, Ipf, Imf;
        Ip.define(L.ba, 3, 1);
        Im.define(L.ba, 3, 1);
        const bool ptf = P.ppm_trace_forces == 1;
        if (ptf) {
            Ipf.define(L.ba, 3, 1);
            Imf.define(L.ba, 3, 1);
        }
        MF sl[3], sr[3], simh[3];
        for (int d = 0; d < 3; ++d) {
            sl[d].define(L.ba, 1, 1, -1, 0.0);
            sr[d].define(L.ba, 1, 1, -1, 0.0);
            simh[d].define(L.ba, 1, 1, -1, 0.0);
        }
        MF slopez, divu;
        slopez.define(L.ba, 1, 1);
        divu.define(L.ba, 1, 1);
        MF simh2[3][3];  // simh2[d][t]: d-faces corrected by t (simhxy = [0][1])
        for (int d = 0; d < 3; ++d)
            for (int t = 0; t < 3; ++t)
                if (d != t) simh2[d][t].define(L.ba, 1, 1, -1, 0.0);
        const real dt2 = 0.5 * dt, dt4 = 0.25 * dt, dt3 = dt / 3.0, dt6 = dt / 6.0;

        for (int scomp = start_scomp; scomp < start_scomp + num_comp; ++scomp) {
            const int bccomp = start_bccomp + scomp - start_scomp;
            const int comp = scomp;
#pragma omp parallel for schedule(dynamic)
            for (int b = 0; b < nb; ++b) {
                const Box obx = grow(L.ba[b], 1);
                if (is_conservative) MakeDivU(obx, divu[b], umac[0][b], umac[1][b], umac[2][b]);
                if (P.ppm_type == 0) {
                    Arr sc = state[b].comp(comp);
                    sc.nc = 1;
                    std::vector<BCRec> one(1, bcs[bccomp]);
                    Slope_dir(P.slope_order, L.dom, obx, sc, Ip[b], 1, one, 0, 0);
                    Slope_dir(P.slope_order, L.dom, obx, sc, Im[b], 1, one, 0, 1);
                    Slope_dir(P.slope_order, L.dom, obx, sc, slopez[b], 1, one, 0, 2);
                } else {
                    PPM(pc, obx, state[b], umac[0][b], umac[1][b], umac[2][b], Ip[b], Im[b], bcs[bccomp], true, comp);
                    if (ptf)  // the force traced like the component (:137-141, 223-227)
                        PPM(pc, obx, force[b], umac[0][b], umac[1][b], umac[2][b], Ipf[b], Imf[b], bcs[bccomp], true,
                            comp);
                }
            }
            const int bc_lo[3] = {bcs[bccomp].lo[0], bcs[bccomp].lo[1], bcs[bccomp].lo[2]};
            const int bc_hi[3] = {bcs[bccomp].hi[0], bcs[bccomp].hi[1], bcs[bccomp].hi[2]};
#pragma omp parallel for schedule(dynamic)
            for (int b = 0; b < nb; ++b) {
                const Box obx = grow(L.ba[b], 1);
                const Arr& scal = state[b];
                const Arr* uu[3] = {&umac[0][b], &umac[1][b], &umac[2][b]};
                // MakeEdgeScalPredictor (:662-863)
                for (int d = 0; d < 3; ++d) {
                    const Box mbx = growLo(obx, d, -1);
                    const int di = d == 0, dj = d == 1, dk = d == 2;
                    const Arr& l = sl[d][b];
                    const Arr& r = sr[d][b];
                    const Arr& sm = simh[d][b];
                    const Arr& ud = *uu[d];
                    const Arr& slope = d == 0 ? Ip[b] : (d == 1 ? Im[b] : slopez[b]);
                    MO_FOR3(mbx) {
                        const int I = d == 0 ? i : (d == 1 ? j : k);
                        const int il = i - di, jl = j - dj, kl = k - dk;
                        if (P.ppm_type == 0) {
                            l(i, j, k) = scal(il, jl, kl, comp) + 0.5 * (1.0 - dt * ud(i, j, k) / h[d]) * slope(il, jl, kl, 0);
                            r(i, j, k) = scal(i, j, k, comp) - 0.5 * (1.0 + dt * ud(i, j, k) / h[d]) * slope(i, j, k, 0);
                        } else {
                            l(i, j, k) = Ip[b](il, jl, kl, d);
                            r(i, j, k) = Im[b](i, j, k, d);
                        }
                        if (I == domlo[d]) {
                            int bclo = bc_lo[d];
                            if (bclo == ext_dir) {
                                l(i, j, k) = scal(il, jl, kl, comp);
                                r(i, j, k) = scal(il, jl, kl, comp);
                            } else if (bclo == foextrap || bclo == hoextrap) {
                                if (is_vel && comp == d) r(i, j, k) = mn(r(i, j, k), 0.0);
                                l(i, j, k) = r(i, j, k);
                            } else if (bclo == reflect_even) {
                                l(i, j, k) = r(i, j, k);
                            } else if (bclo == reflect_odd) {
                                l(i, j, k) = 0.0;
                                r(i, j, k) = 0.0;
                            }
                        } else if (I == domhi[d] + 1) {
                            int bchi = bc_hi[d];
                            if (bchi == ext_dir) {
                                l(i, j, k) = scal(i, j, k, comp);
                                r(i, j, k) = scal(i, j, k, comp);
                            } else if (bchi == foextrap || bchi == hoextrap) {
                                if (is_vel && comp == d) l(i, j, k) = mx(l(i, j, k), 0.0);
                                r(i, j, k) = l(i, j, k);
                            } else if (bchi == reflect_even) {
                                r(i, j, k) = l(i, j, k);
                            } else if (bchi == reflect_odd) {
                                l(i, j, k) = 0.0;
                                r(i, j, k) = 0.0;
                            }
                        }
                        sm(i, j, k) = (ud(i, j, k) > 0.0) ? l(i, j, k) : r(i, j, k);
                        sm(i, j, k) = (fab(ud(i, j, k)) > 0.0) ? sm(i, j, k) : 0.5 * (l(i, j, k) + r(i, j, k));
                    }
                }
                // MakeEdgeScalTransverse (:865-1359): d-faces corrected by direction t
                for (int d = 0; d < 3; ++d)
                    for (int t = 0; t < 3; ++t) {
                        if (d == t) continue;
                        const int o = 3 - d - t;
                        Box imhbox = growHi(grow(L.ba[b], o, 1), d, 1);
                        const int di = d == 0, dj = d == 1, dk = d == 2;
                        const int ti = t == 0, tj = t == 1, tk = t == 2;
                        const Arr& l = sl[d][b];
                        const Arr& r = sr[d][b];
                        const Arr& st = simh[t][b];
                        const Arr& ut = *uu[t];
                        const Arr& ud = *uu[d];
                        const Arr& dv = divu[b];
                        const Arr& out = simh2[d][t][b];
                        MO_FOR3(imhbox) {
                            const int I = d == 0 ? i : (d == 1 ? j : k);
                            const int il = i - di, jl = j - dj, kl = k - dk;
                            real lq, rq;
                            if (is_conservative) {
                                lq = l(i, j, k) -
                                     (dt3 / h[t]) * (st(il + ti, jl + tj, kl + tk) * ut(il + ti, jl + tj, kl + tk) -
                                                     st(il, jl, kl) * ut(il, jl, kl)) -
                                     dt3 * scal(il, jl, kl, comp) * dv(il, jl, kl) +
                                     (dt3 / h[t]) * scal(il, jl, kl, comp) *
                                         (ut(il + ti, jl + tj, kl + tk) - ut(il, jl, kl));
                                rq = r(i, j, k) -
                                     (dt3 / h[t]) * (st(i + ti, j + tj, k + tk) * ut(i + ti, j + tj, k + tk) -
                                                     st(i, j, k) * ut(i, j, k)) -
                                     dt3 * scal(i, j, k, comp) * dv(i, j, k) +
                                     (dt3 / h[t]) * scal(i, j, k, comp) * (ut(i + ti, j + tj, k + tk) - ut(i, j, k));
                            } else {
                                lq = l(i, j, k) - (dt6 / h[t]) * (ut(il + ti, jl + tj, kl + tk) + ut(il, jl, kl)) *
                                                      (st(il + ti, jl + tj, kl + tk) - st(il, jl, kl));
                                rq = r(i, j, k) - (dt6 / h[t]) * (ut(i + ti, j + tj, k + tk) + ut(i, j, k)) *
                                                      (st(i + ti, j + tj, k + tk) - st(i, j, k));
                            }
                            if (I == domlo[d]) {
                                int bclo = bc_lo[d];
                                if (bclo == ext_dir) {
                                    lq = scal(il, jl, kl, comp);
                                    rq = scal(il, jl, kl, comp);
                                } else if (bclo == foextrap || bclo == hoextrap) {
                                    if (is_vel && comp == d) rq = mn(rq, 0.0);
                                    lq = rq;
                                } else if (bclo == reflect_even) {
                                    lq = rq;
                                } else if (bclo == reflect_odd) {
                                    lq = 0.0;
                                    rq = 0.0;
                                }
                            } else if (I == domhi[d] + 1) {
                                int bchi = bc_hi[d];
                                if (bchi == ext_dir) {
                                    lq = scal(i, j, k, comp);
                                    rq = scal(i, j, k, comp);
                                } else if (bchi == foextrap || bchi == hoextrap) {
                                    if (is_vel && comp == d) lq = mx(lq, 0.0);
                                    rq = lq;
                                } else if (bchi == reflect_even) {
                                    rq = lq;
                                } else if (bchi == reflect_odd) {
                                    lq = 0.0;
                                    rq = 0.0;
                                }
                            }
                            out(i, j, k) = (ud(i, j, k) > 0.0) ? lq : rq;
                            out(i, j, k) = (fab(ud(i, j, k)) > rel_eps) ? out(i, j, k) : 0.5 * (lq + rq);
                        }
                    }
                // MakeEdgeScalEdges (:1361-1667)
                for (int d = 0; d < 3; ++d) {
                    const Box xbx = nodal(L.ba[b], d);
                    const int di = d == 0, dj = d == 1, dk = d == 2;
                    const int t1 = d == 0 ? 1 : 0, t2 = d == 2 ? 1 : 2;
                    const int a1i = t1 == 0, a1j = t1 == 1, a1k = t1 == 2;
                    const int a2i = t2 == 0, a2j = t2 == 1, a2k = t2 == 2;
                    const Arr& l = sl[d][b];
                    const Arr& r = sr[d][b];
                    const Arr& q1 = simh2[t1][t2][b];  // simhyz for d = x
                    const Arr& q2 = simh2[t2][t1][b];  // simhzy for d = x
                    const Arr& u1 = *uu[t1];
                    const Arr& u2 = *uu[t2];
                    const Arr& ud = *uu[d];
                    const Arr& f = force[b];
                    const Arr& se = sedge[d][b];
                    MO_FOR3(xbx) {
                        const int I = d == 0 ? i : (d == 1 ? j : k);
                        const int il = i - di, jl = j - dj, kl = k - dk;
                        // the traced force if ppm_trace_forces = 1 (:1405-1408, 1495-1498, 1585-1588)
                        real fl = ptf ? Ipf[b](il, jl, kl, d) : f(il, jl, kl, comp);
                        real fr = ptf ? Imf[b](i, j, k, d) : f(i, j, k, comp);
                        real lq, rq;
                        if (is_conservative) {
                            lq = l(i, j, k) -
                                 (dt2 / h[t1]) * (q1(il + a1i, jl + a1j, kl + a1k) * u1(il + a1i, jl + a1j, kl + a1k) -
                                                  q1(il, jl, kl) * u1(il, jl, kl)) -
                                 (dt2 / h[t2]) * (q2(il + a2i, jl + a2j, kl + a2k) * u2(il + a2i, jl + a2j, kl + a2k) -
                                                  q2(il, jl, kl) * u2(il, jl, kl)) -
                                 (dt2 / h[d]) * scal(il, jl, kl, comp) * (ud(i, j, k) - ud(il, jl, kl)) + dt2 * fl;
                            rq = r(i, j, k) -
                                 (dt2 / h[t1]) * (q1(i + a1i, j + a1j, k + a1k) * u1(i + a1i, j + a1j, k + a1k) -
                                                  q1(i, j, k) * u1(i, j, k)) -
                                 (dt2 / h[t2]) * (q2(i + a2i, j + a2j, k + a2k) * u2(i + a2i, j + a2j, k + a2k) -
                                                  q2(i, j, k) * u2(i, j, k)) -
                                 (dt2 / h[d]) * scal(i, j, k, comp) * (ud(i + di, j + dj, k + dk) - ud(i, j, k)) +
                                 dt2 * fr;
                        } else {
                            lq = l(i, j, k) -
                                 (dt4 / h[t1]) * (u1(il + a1i, jl + a1j, kl + a1k) + u1(il, jl, kl)) *
                                     (q1(il + a1i, jl + a1j, kl + a1k) - q1(il, jl, kl)) -
                                 (dt4 / h[t2]) * (u2(il + a2i, jl + a2j, kl + a2k) + u2(il, jl, kl)) *
                                     (q2(il + a2i, jl + a2j, kl + a2k) - q2(il, jl, kl)) +
                                 dt2 * fl;
                            rq = r(i, j, k) -
                                 (dt4 / h[t1]) * (u1(i + a1i, j + a1j, k + a1k) + u1(i, j, k)) *
                                     (q1(i + a1i, j + a1j, k + a1k) - q1(i, j, k)) -
                                 (dt4 / h[t2]) * (u2(i + a2i, j + a2j, k + a2k) + u2(i, j, k)) *
                                     (q2(i + a2i, j + a2j, k + a2k) - q2(i, j, k)) +
                                 dt2 * fr;
                        }
                        real v = (ud(i, j, k) > 0.0) ? lq : rq;
                        v = (fab(ud(i, j, k)) > rel_eps) ? v : 0.5 * (lq + rq);
                        if (I == domlo[d]) {
                            int bclo = bc_lo[d];
                            if (bclo == ext_dir) v = scal(il, jl, kl, comp);
                            else if (bclo == foextrap || bclo == hoextrap) v = (is_vel && comp == d) ? mn(rq, 0.0) : rq;
                            else if (bclo == reflect_even) v = rq;
                            else if (bclo == reflect_odd) v = 0.0;
                        } else if (I == domhi[d] + 1) {
                            int bchi = bc_hi[d];
                            if (bchi == ext_dir) v = scal(i, j, k, comp);
                            else if (bchi == foextrap || bchi == hoextrap) v = (is_vel && comp == d) ? mx(lq, 0.0) : lq;
                            else if (bchi == reflect_even) v = lq;
                            else if (bchi == reflect_odd) v = 0.0;
                        }
                        se(i, j, k, comp) = v;
                    }
                }
            }
        }
    }

    // ------------------------------------------------------------------ forces
    // Maestro::ModifyScalForce, planar 3-D, one level (Source/MaestroForce.cpp:261-453)
    void ModifyScalForce(MF& scal_force, MF& state, MF* umac, MF& s0_edge_cart, MF& s0_cart, int comp,
                         int fullform, const MF* divu_cart = nullptr) {
        const double* dx = L.dx;
        if (P.spherical) {
            // Source/MaestroForce.cpp:335-412; divu_cart = Put1dArrayOnCart(divw0), which is 0
            // with the exact base state (:283-302)
            const int* domlo = L.dom.lo;
            const int* domhi = L.dom.hi;
            for (int b = 0; b < nb; ++b) {
                const Arr scal = state[b].comp(comp);
                const Arr& um = umac[0][b];
                const Arr& vm = umac[1][b];
                const Arr& wm = umac[2][b];
                const Arr& s0a = s0_cart[b];
                const Arr force = scal_force[b].comp(comp);
                MO_FOR3(L.ba[b]) {
                    const real divu_c = divu_cart ? (*divu_cart)[b](i, j, k) : real(0.0);
                    real divumac = (um(i + 1, j, k) - um(i, j, k)) / dx[0] + (vm(i, j + 1, k) - vm(i, j, k)) / dx[1] +
                                     (wm(i, j, k + 1) - wm(i, j, k)) / dx[2];
                    if (fullform == 1) {
                        force(i, j, k) -= scal(i, j, k) * (divumac + divu_c);
                    } else {
                        const real s0x_hi = i < domhi[0] ? 0.5 * (s0a(i, j, k) + s0a(i + 1, j, k)) : s0a(i, j, k);
                        const real s0x_lo = i > domlo[0] ? 0.5 * (s0a(i, j, k) + s0a(i - 1, j, k)) : s0a(i, j, k);
                        const real s0y_hi = j < domhi[1] ? 0.5 * (s0a(i, j, k) + s0a(i, j + 1, k)) : s0a(i, j, k);
                        const real s0y_lo = j > domlo[1] ? 0.5 * (s0a(i, j, k) + s0a(i, j - 1, k)) : s0a(i, j, k);
                        const real s0z_hi = k < domhi[2] ? 0.5 * (s0a(i, j, k) + s0a(i, j, k + 1)) : s0a(i, j, k);
                        const real s0z_lo = k > domlo[2] ? 0.5 * (s0a(i, j, k) + s0a(i, j, k - 1)) : s0a(i, j, k);
                        real divs0u = (um(i + 1, j, k) * s0x_hi - um(i, j, k) * s0x_lo) / dx[0] +
                                        (vm(i, j + 1, k) * s0y_hi - vm(i, j, k) * s0y_lo) / dx[1] +
                                        (wm(i, j, k + 1) * s0z_hi - wm(i, j, k) * s0z_lo) / dx[2];
                        force(i, j, k) += -divs0u - (scal(i, j, k) - s0a(i, j, k)) * (divumac + divu_c);
                    }
                }
            }
            return;
        }
        for (int b = 0; b < nb; ++b) {
            const Arr scal = state[b].comp(comp);
            const Arr& um = umac[0][b];
            const Arr& vm = umac[1][b];
            const Arr& wm = umac[2][b];
            const Arr& s0a = s0_cart[b];
            const Arr& s0e = s0_edge_cart[b];
            const Arr& w0a = w0_cart[b];
            const Arr force = scal_force[b].comp(comp);
            MO_FOR3(L.ba[b]) {
                real divu = (um(i + 1, j, k) - um(i, j, k)) / dx[0] + (vm(i, j + 1, k) - vm(i, j, k)) / dx[1] +
                              (wm(i, j, k + 1) - wm(i, j, k)) / dx[2];
                divu += (w0a(i, j, k + 1, 2) - w0a(i, j, k, 2)) / dx[2];
                if (fullform == 1) {
                    force(i, j, k) -= scal(i, j, k) * divu;
                } else {
                    real divs0u = s0a(i, j, k) * ((um(i + 1, j, k) - um(i, j, k)) / dx[0] +
                                                    (vm(i, j + 1, k) - vm(i, j, k)) / dx[1]) +
                                    (wm(i, j, k + 1) * s0e(i, j, k + 1) - wm(i, j, k) * s0e(i, j, k)) / dx[2];
                    force(i, j, k) += -(scal(i, j, k) - s0a(i, j, k)) * divu - divs0u;
                }
            }
        }
    }

    // Maestro::MakeRhoHForce, planar 3-D, one level (Source/MaestroForce.cpp:541-674)
    void MakeRhoHForce(MF& scal_force, int is_prediction, MF* umac, int add_thermal, MF& p0_cart, MF& psi_cart,
                       MF& grav_cart, MF& rho0_cart, MF* p0mac = nullptr) {
        const int domhi = L.dom.hi[2];
        const bool psi_in = (is_prediction == 1 && P.enthalpy_pred_type == 2) ||
                            (is_prediction == 1 && P.enthalpy_pred_type == 0) || (is_prediction == 0);
        if (P.spherical) {  // Source/MaestroForce.cpp:637-670: u grad p0 = div(u p0) - p0 div u
            const double* dx = L.dx;
            for (int b = 0; b < nb; ++b) {
                const Arr& um = umac[0][b];
                const Arr& vm = umac[1][b];
                const Arr& wm = umac[2][b];
                const Arr& px = p0mac[0][b];
                const Arr& py = p0mac[1][b];
                const Arr& pz = p0mac[2][b];
                const Arr& p0c = p0_cart[b];
                const Arr& th = thermal[b];
                const Arr& ps = psi_cart[b];
                const Arr rf = scal_force[b].comp(RhoH);
                MO_FOR3(L.ba[b]) {
                    real divup = (um(i + 1, j, k) * px(i + 1, j, k) - um(i, j, k) * px(i, j, k)) / dx[0] +
                                   (vm(i, j + 1, k) * py(i, j + 1, k) - vm(i, j, k) * py(i, j, k)) / dx[1] +
                                   (wm(i, j, k + 1) * pz(i, j, k + 1) - wm(i, j, k) * pz(i, j, k)) / dx[2];
                    real p0divu = ((um(i + 1, j, k) - um(i, j, k)) / dx[0] + (vm(i, j + 1, k) - vm(i, j, k)) / dx[1] +
                                     (wm(i, j, k + 1) - wm(i, j, k)) / dx[2]) *
                                    p0c(i, j, k);
                    rf(i, j, k) = divup - p0divu;
                    if (psi_in) rf(i, j, k) += ps(i, j, k);
                    if (add_thermal == 1) rf(i, j, k) += th(i, j, k);
                }
            }
            return;
        }
        for (int b = 0; b < nb; ++b) {
            const Arr& wm = umac[2][b];
            const Arr& p0c = p0_cart[b];
            const Arr& th = thermal[b];
            const Arr& ps = psi_cart[b];
            const Arr& gc = grav_cart[b];
            const Arr& rc = rho0_cart[b];
            const Arr rf = scal_force[b].comp(RhoH);
            MO_FOR3(L.ba[b]) {
                real gradp0 = 0.0;
                if (k < cutoff) {
                    gradp0 = rc(i, j, k) * gc(i, j, k);
                } else if (k == domhi) {
                    gradp0 = (p0c(i, j, k) - p0c(i, j - 1, k)) / L.dx[2];
                } else {
                    gradp0 = (p0c(i, j + 1, k) - p0c(i, j, k)) / L.dx[2];
                }
                real veladv = 0.5 * (wm(i, j, k) + wm(i, j, k + 1));
                rf(i, j, k) = veladv * gradp0;
                if (psi_in) rf(i, j, k) += ps(i, j, k);
                if (add_thermal == 1) rf(i, j, k) += th(i, j, k);
            }
        }
    }

    // ------------------------------------------------------------------ conversions
    // Maestro::PutInPertForm, one level (Source/MaestroConvert.cpp:6-30)
    void PutInPertForm(MF& scal, const std::vector<real>& s0, int comp, bool flag) {
        for (int b = 0; b < nb; ++b) {
            const Arr& a = scal[b];
            MO_FOR3(L.ba[b]) {
                const real s0c = P.spherical ? sph_cell_at(s0, i, j, k) : s0[k];
                if (flag) a(i, j, k, comp) = a(i, j, k, comp) - s0c;
                else a(i, j, k, comp) = a(i, j, k, comp) + s0c;
            }
        }
    }

    // Maestro::ConvertRhoXToX, one level (Source/MaestroConvert.cpp:64-81)
    void ConvertRhoXToX(MF& scal, bool flag) {
        for (int b = 0; b < nb; ++b) {
            const Arr& a = scal[b];
            for (int comp = FirstSpec; comp < FirstSpec + nspec; ++comp)
                MO_FOR3(L.ba[b]) {
                    if (flag) a(i, j, k, comp) = a(i, j, k, comp) / a(i, j, k, Rho);
                    else a(i, j, k, comp) = a(i, j, k, comp) * a(i, j, k, Rho);
                }
        }
    }

    // Maestro::ConvertRhoHToH, the valid region (Source/MaestroConvert.cpp:93-105):
    // flag: (rho h) -> h = (rho h) / rho; else h -> rho h
    void ConvertRhoHToH(MF& scal, bool flag) {
        for (int b = 0; b < nb; ++b) {
            const Arr& a = scal[b];
            MO_FOR3(L.ba[b]) {
                if (flag) a(i, j, k, RhoH) = a(i, j, k, RhoH) / a(i, j, k, Rho);
                else a(i, j, k, RhoH) = a(i, j, k, RhoH) * a(i, j, k, Rho);
            }
        }
    }

    // ------------------------------------------------------------------ fluxes
    // Maestro::MakeRhoXFlux, planar 3-D (Source/MaestroMakeFlux.cpp:18-465)
    void MakeRhoXFlux(MF* sflux, MF& etarhoflux, MF* sedge, MF* umac, const std::vector<real>& r0_old,
                      const std::vector<real>& r0e_old, const std::vector<real>& r0_new,
                      const std::vector<real>& r0e_new, int start_comp, int num_comp, MF* r0mac_old = nullptr,
                      MF* r0mac_new = nullptr) {
        const int spt = P.species_pred_type;
        for (int d = 0; d < 3; ++d) sflux[d].setVal(0.0, Rho, 1, 0);
        if (P.spherical) {  // Source/MaestroMakeFlux.cpp:56-71, 306-408
            for (int b = 0; b < nb; ++b)
                for (int d = 0; d < 3; ++d) {
                    const Arr& f = sflux[d][b];
                    const Arr& e = sedge[d][b];
                    const Arr& u = umac[d][b];
                    const Arr& ro = r0mac_old[d][b];
                    const Arr& rn = r0mac_new[d][b];
                    MO_FOR3(nodal(L.ba[b], d)) {
                        const real rho0_edge = 0.5 * ro(i, j, k) + 0.5 * rn(i, j, k);  // MultiFab::LinComb
                        for (int comp = start_comp; comp < num_comp + start_comp; ++comp) {
                            if (spt == 1) f(i, j, k, comp) = u(i, j, k) * (rho0_edge + e(i, j, k, Rho)) * e(i, j, k, comp);
                            else if (spt == 2) f(i, j, k, comp) = u(i, j, k) * e(i, j, k, comp);
                            else if (spt == 3) f(i, j, k, comp) = u(i, j, k) * e(i, j, k, Rho) * e(i, j, k, comp);
                            f(i, j, k, Rho) += f(i, j, k, comp);
                        }
                    }
                }
            return;
        }
        for (int b = 0; b < nb; ++b) {
            for (int d = 0; d < 3; ++d) {
                const Arr& f = sflux[d][b];
                const Arr& e = sedge[d][b];
                const Arr& u = umac[d][b];
                const Arr& eta = etarhoflux[b];
                MO_FOR3(nodal(L.ba[b], d)) {
                    for (int comp = start_comp; comp < num_comp + start_comp; ++comp) {
                        real rho0_edge = d < 2 ? 0.5 * (r0_old[k] + r0_new[k]) : 0.5 * (r0e_old[k] + r0e_new[k]);
                        if (spt == 1) {
                            f(i, j, k, comp) = u(i, j, k) * (rho0_edge + e(i, j, k, Rho)) * e(i, j, k, comp);
                        } else if (spt == 2) {
                            f(i, j, k, comp) = u(i, j, k) * e(i, j, k, comp);
                        } else if (spt == 3) {
                            f(i, j, k, comp) = u(i, j, k) * e(i, j, k, Rho) * e(i, j, k, comp);
                        }
                        if (d == 2 && P.evolve_base_state && !P.use_exact_base_state) {
                            if (comp >= FirstSpec && comp <= FirstSpec + nspec - 1) eta(i, j, k) += f(i, j, k, comp);
                            if (comp == FirstSpec + nspec - 1) eta(i, j, k) -= w0[k] * rho0_predicted_edge[k];
                        }
                        f(i, j, k, Rho) += f(i, j, k, comp);
                    }
                }
            }
        }
    }

    // Maestro::MakeRhoHFlux, planar 3-D (Source/MaestroMakeFlux.cpp:467-1067)
    void MakeRhoHFlux(MF* sflux, MF* sedge, MF* umac, const std::vector<real>& rh0_old,
                      const std::vector<real>& rh0e_old, const std::vector<real>& rh0_new,
                      const std::vector<real>& rh0e_new, MF* rh0mac_old = nullptr, MF* rh0mac_new = nullptr,
                      const std::vector<real>* r0_old = nullptr, const std::vector<real>* r0e_old = nullptr,
                      const std::vector<real>* r0_new = nullptr, const std::vector<real>* r0e_new = nullptr,
                      MF* r0mac_old = nullptr, MF* r0mac_new = nullptr) {
        const int ept = P.enthalpy_pred_type;
        const int spt = P.species_pred_type;
        if (P.spherical && P.use_exact_base_state) {
            // exact base state, (rho h)' predicted (Source/MaestroMakeFlux.cpp:540-548, 788-840)
            for (int b = 0; b < nb; ++b)
                for (int d = 0; d < 3; ++d) {
                    const Arr& f = sflux[d][b];
                    const Arr& e = sedge[d][b];
                    const Arr& u = umac[d][b];
                    const Arr& ho = rh0mac_old[d][b];
                    const Arr& hn = rh0mac_new[d][b];
                    MO_FOR3(nodal(L.ba[b], d)) {
                        const real rhoh0_edge = 0.5 * ho(i, j, k) + 0.5 * hn(i, j, k);
                        f(i, j, k, RhoH) = u(i, j, k) * (rhoh0_edge + e(i, j, k, RhoH));
                    }
                }
            return;
        }
        if (P.spherical) {
            // uniform bins (Source/MaestroMakeFlux.cpp:549-575, 846-1000): rhoh predicted; h
            // predicted, times (rho0mac + rho') or rho; or (rho h)' with (rho h)_0 on the faces as
            // rho0mac * h0mac; rh0mac_old / _new carry h0mac here, r0mac_old / _new rho0mac
            for (int b = 0; b < nb; ++b)
                for (int d = 0; d < 3; ++d) {
                    const Arr& f = sflux[d][b];
                    const Arr& e = sedge[d][b];
                    const Arr& u = umac[d][b];
                    MO_FOR3(nodal(L.ba[b], d)) {
                        if (ept == 0) {
                            f(i, j, k, RhoH) = u(i, j, k) * e(i, j, k, RhoH);
                        } else if (ept == 2) {
                            const real rho0_edge = 0.5 * r0mac_old[d][b](i, j, k) + 0.5 * r0mac_new[d][b](i, j, k);
                            if (spt == 1) f(i, j, k, RhoH) = u(i, j, k) * (rho0_edge + e(i, j, k, Rho)) * e(i, j, k, RhoH);
                            else f(i, j, k, RhoH) = u(i, j, k) * e(i, j, k, Rho) * e(i, j, k, RhoH);
                        } else {
                            const real rho0_edge = 0.5 * r0mac_old[d][b](i, j, k) + 0.5 * r0mac_new[d][b](i, j, k);
                            const real h0_edge = 0.5 * rh0mac_old[d][b](i, j, k) + 0.5 * rh0mac_new[d][b](i, j, k);
                            f(i, j, k, RhoH) = u(i, j, k) * (rho0_edge * h0_edge + e(i, j, k, RhoH));
                        }
                    }
                }
            return;
        }
        for (int b = 0; b < nb; ++b)
            for (int d = 0; d < 3; ++d) {
                const Arr& f = sflux[d][b];
                const Arr& e = sedge[d][b];
                const Arr& u = umac[d][b];
                MO_FOR3(nodal(L.ba[b], d)) {
                    if (ept == 0) {
                        f(i, j, k, RhoH) = u(i, j, k) * e(i, j, k, RhoH);
                    } else if (ept == 1) {
                        if (d < 2) {
                            real rhoh0_edge = 0.5 * (rh0_old[k] + rh0_new[k]);
                            f(i, j, k, RhoH) = u(i, j, k) * (rhoh0_edge + e(i, j, k, RhoH));
                        } else {
                            real rhoh0_edge = 0.5 * (rh0e_old[k] + rh0e_new[k]);
                            f(i, j, k, RhoH) = u(i, j, k) * (e(i, j, k, RhoH) + rhoh0_edge);
                        }
                    } else if (ept == 2) {  // the edge state is h (:673-786, have_h)
                        if (spt == 1) {  // density edge state rho': x / y faces cell rho0, z faces edge rho0
                            const real rho0_edge = d < 2 ? 0.5 * ((*r0_old)[k] + (*r0_new)[k])
                                                         : 0.5 * ((*r0e_old)[k] + (*r0e_new)[k]);
                            f(i, j, k, RhoH) = u(i, j, k) * (rho0_edge + e(i, j, k, Rho)) * e(i, j, k, RhoH);
                        } else {  // density edge state rho
                            f(i, j, k, RhoH) = u(i, j, k) * e(i, j, k, Rho) * e(i, j, k, RhoH);
                        }
                    }
                }
            }
    }

    // ------------------------------------------------------------------ UpdateScal
    // Maestro::UpdateScal, one level (Source/MaestroAdvection.cpp:86-256)
    // Maestro::UpdateVel (Source/MaestroAdvection.cpp:299-526): unew = uold - dt (U.grad)U
    // + dt force, minus the w0 advection term, times the sponge where one is given
    void UpdateVel(MF& uold, MF& unew, MF* umac, MF* uedge, MF& force, MF* sponge) {
        const double* dx = L.dx;
        const real dt_loc = dt;
        for (int b = 0; b < nb; ++b) {
            const Arr &uo = uold[b], &un = unew[b], &um = umac[0][b], &vm = umac[1][b], &wm = umac[2][b];
            const Arr &ex = uedge[0][b], &ey = uedge[1][b], &ez = uedge[2][b], &f = force[b];
            MO_FOR3(L.ba[b]) {
                const real ubar = 0.5 * (um(i, j, k) + um(i + 1, j, k));
                const real vbar = 0.5 * (vm(i, j, k) + vm(i, j + 1, k));
                const real wbar = 0.5 * (wm(i, j, k) + wm(i, j, k + 1));
                real ugrad[3];
                for (int n = 0; n < 3; ++n)
                    ugrad[n] = ubar * (ex(i + 1, j, k, n) - ex(i, j, k, n)) / dx[0] +
                               vbar * (ey(i, j + 1, k, n) - ey(i, j, k, n)) / dx[1] +
                               wbar * (ez(i, j, k + 1, n) - ez(i, j, k, n)) / dx[2];
                for (int n = 0; n < 3; ++n) un(i, j, k, n) = uo(i, j, k, n) - dt_loc * ugrad[n] + dt_loc * f(i, j, k, n);
                if (!P.spherical) {
                    const Arr& w0c = w0_cart[b];
                    const real w0bar = 0.5 * (w0c(i, j, k, 2) + w0c(i, j, k + 1, 2));
                    for (int n = 0; n < 3; ++n) {
                        un(i, j, k, n) -= dt_loc * w0bar * (ez(i, j, k + 1, n) - ez(i, j, k, n)) / dx[2];
                        if (sponge) un(i, j, k, n) *= (*sponge)[b](i, j, k);
                    }
                } else {
                    const Arr &w0x = w0mac[0][b], &w0y = w0mac[1][b], &w0z = w0mac[2][b];
                    real w0r[3];
                    for (int n = 0; n < 3; ++n) {
                        const real gx = (ex(i + 1, j, k, n) - ex(i, j, k, n)) / dx[0];
                        const real gy = (ey(i, j + 1, k, n) - ey(i, j, k, n)) / dx[1];
                        const real gz = (ez(i, j, k + 1, n) - ez(i, j, k, n)) / dx[2];
                        w0r[n] = gx * 0.5 * (w0x(i, j, k) + w0x(i + 1, j, k)) +
                                 gy * 0.5 * (w0y(i, j, k) + w0y(i, j + 1, k)) +
                                 gz * 0.5 * (w0z(i, j, k) + w0z(i, j, k + 1));
                    }
                    for (int n = 0; n < 3; ++n) un(i, j, k, n) -= dt_loc * w0r[n];
                    if (sponge)
                        for (int n = 0; n < 3; ++n) un(i, j, k, n) *= (*sponge)[b](i, j, k);
                }
            }
        }
    }

    void UpdateScal(MF& sold, MF& snew, MF* sflux, MF& force, int start_comp, int num_comp) {
        const double* dx = L.dx;
        const real dt_loc = dt;
        for (int b = 0; b < nb; ++b) {
            const Arr& so = sold[b];
            const Arr& sn = snew[b];
            const Arr& fx = sflux[0][b];
            const Arr& fy = sflux[1][b];
            const Arr& fz = sflux[2][b];
            const Arr& fo = force[b];
            if (start_comp == RhoH) {
                MO_FOR3(L.ba[b]) {
                    real divterm = ((fx(i + 1, j, k, RhoH) - fx(i, j, k, RhoH)) / dx[0] +
                                      (fy(i, j + 1, k, RhoH) - fy(i, j, k, RhoH)) / dx[1] +
                                      (fz(i, j, k + 1, RhoH) - fz(i, j, k, RhoH)) / dx[2]);
                    sn(i, j, k, RhoH) = so(i, j, k, RhoH) + dt_loc * (-divterm + fo(i, j, k, RhoH));
                    if (P.do_eos_h_above_cutoff && sn(i, j, k, Rho) <= P.base_cutoff_density)
                        throw std::runtime_error("UpdateScal: cell at or below base_cutoff_density needs the EOS");
                }
            } else {
                for (int n = 0; n < nspec; ++n) {
                    const int comp = FirstSpec + n;
                    MO_FOR3(L.ba[b]) {
                        real divterm = (fx(i + 1, j, k, comp) - fx(i, j, k, comp)) / dx[0];
                        divterm += (fy(i, j + 1, k, comp) - fy(i, j, k, comp)) / dx[1];
                        divterm += (fz(i, j, k + 1, comp) - fz(i, j, k, comp)) / dx[2];
                        sn(i, j, k, comp) = so(i, j, k, comp) + dt_loc * (-divterm + fo(i, j, k, comp));
                    }
                }
                MO_FOR3(L.ba[b]) {
                    sn(i, j, k, Rho) = so(i, j, k, Rho);
                    bool has_negative_species = false;
                    for (int comp = start_comp; comp < start_comp + nspec; ++comp) {
                        sn(i, j, k, Rho) += sn(i, j, k, comp) - so(i, j, k, comp);
                        if (sn(i, j, k, comp) < 0.0) has_negative_species = true;
                    }
                    if (sn(i, j, k, Rho) < 0.5 * P.base_cutoff_density) {
                        for (int comp = start_comp; comp < start_comp + nspec; ++comp)
                            sn(i, j, k, comp) *= 0.5 * P.base_cutoff_density / sn(i, j, k, Rho);
                        sn(i, j, k, Rho) = 0.5 * P.base_cutoff_density;
                    }
                    if (has_negative_species) {
                        for (int comp = start_comp; comp < start_comp + nspec; ++comp) {
                            if (sn(i, j, k, comp) < 0.0) {
                                real delta = -sn(i, j, k, comp);
                                real sumX = 0.0;
                                for (int comp2 = start_comp; comp2 < start_comp + nspec; ++comp2)
                                    if (comp2 != comp && sn(i, j, k, comp2) >= 0.0) sumX += sn(i, j, k, comp2);
                                for (int comp2 = start_comp; comp2 < start_comp + nspec; ++comp2)
                                    if (comp2 != comp && sn(i, j, k, comp2) >= 0.0) {
                                        real frac = sn(i, j, k, comp2) / sumX;
                                        sn(i, j, k, comp2) -= frac * delta;
                                    }
                                sn(i, j, k, comp) = 0.0;
                            }
                        }
                    }
                }
            }
        }
        (void)num_comp;
    }

};

using VMF = std::vector<MF>;                // one MultiFab per level
using VF = std::vector<std::array<MF, 3>>;  // face MultiFabs per level
using BS = std::vector<std::vector<real>>;  // a base-state array per level

// The stage over all levels, with the coarse-fine synchronisation of the reference:
// AverageDown + FillPatch after every cell-centred update, AverageDownFaces + FillPatchUedge
// for face velocities, AverageDownFaces for fluxes (reflux_type 1, the default).
struct Stage {
    mo_params P;
    int nlev = 1, nspec = 0, nscal = 0, ng_s = 3, ng_adv = 3;
    std::vector<Lev> S;
    std::vector<std::vector<std::array<int, 2>>> chunks;  // per level: radial cell ranges

    const std::vector<BCRec>& bcs_s() const { return S[0].bcs_s; }
    const std::vector<BCRec>& bcs_u() const { return S[0].bcs_u; }
    const std::vector<BCRec>& bcs_f() const { return S[0].bcs_f; }
    BS bs(std::vector<real> Lev::*m) const {
        BS r(nlev);
        for (int l = 0; l < nlev; ++l) r[l] = S[l].*m;
        return r;
    }

    // ------------------------------------------------------------------ level sync
    // Maestro::FillPatch over all levels (Source/MaestroFillData.cpp:7-74)
    void FillPatch(VMF& mf, int c0, int nc, int bccomp, const std::vector<BCRec>& bcs, bool is_vel, int sc0 = -1) {
        for (int lev = 0; lev < nlev; ++lev) {
            if (lev == 0) mo::FillPatch(S[0].L, mf[0], c0, nc, bccomp, bcs, is_vel, sc0);
            else FillPatchTwoLevels(S[lev - 1].L, mf[lev - 1], S[lev].L, mf[lev], c0, nc, bccomp, bcs, is_vel, sc0);
        }
    }
    // Maestro::AverageDown (Source/MaestroFillData.cpp:145-154)
    void AverageDown(VMF& mf, int comp, int ncomp) {
        for (int lev = nlev - 2; lev >= 0; --lev)
            mo::AverageDown(S[lev + 1].L, mf[lev + 1], S[lev].L, mf[lev], comp, ncomp);
    }
    // Maestro::AverageDownFaces (Source/MaestroFillData.cpp:156-174)
    void AverageDownFaces(VF& f) {
        for (int lev = nlev - 2; lev >= 0; --lev) mo::AverageDownFaces(S[lev + 1].L, f[lev + 1], S[lev].L, f[lev]);
    }
    // Maestro::FillPatchUedge (Source/MaestroFillData.cpp:455-835)
    void FillPatchUedge(VF& u) {
        for (int lev = 0; lev < nlev; ++lev) {
            if (lev > 0)
                for (int d = 0; d < 3; ++d) {
                    UedgeInterface ui(S[lev - 1].L, S[lev].L, u[lev - 1][d], u[lev][d], d);
                    ui.apply(u[lev][d]);
                }
            for (int d = 0; d < 3; ++d) FillBoundary(S[lev].L, u[lev][d], 0, 1, u[lev][d].ng);
            S[lev].FillUmacGhost(u[lev].data());
        }
    }
    // the face-velocity ghost fill that closes MakeUtrans and Addw0
    // (Source/MaestroMakeUtrans.cpp:631-647, Source/MaestroFill3dData.cpp:425-461)
    void SyncFaces(VF& u) {
        if (nlev == 1) {
            for (int d = 0; d < 3; ++d) FillBoundary(S[0].L, u[0][d], 0, 1, u[0][d].ng);
            S[0].FillUmacGhost(u[0].data());
        } else {
            AverageDownFaces(u);
            FillPatchUedge(u);
        }
    }

    // ------------------------------------------------------------------ base state
    // Maestro::Put1dArrayOnCart, planar (Source/MaestroFill3dData.cpp:9-36)
    void Put1dArrayOnCart(const BS& s0, VMF& s0_cart, bool edge, bool vec, const std::vector<BCRec>* bcs, int bccomp,
                          bool is_vel) {
        for (int lev = 0; lev < nlev; ++lev) {
            if (P.spherical) S[lev].Put1dSphr(s0[lev], s0_cart[lev], edge, vec);
            else S[lev].Put1d(s0[lev], s0_cart[lev], edge, vec);
        }
        const int nc = vec ? 3 : 1;
        AverageDown(s0_cart, 0, nc);
        if (s0_cart[0].ng > 0) FillPatch(s0_cart, 0, nc, bccomp, *bcs, is_vel);
    }
    // Maestro::MakeS0mac (Source/MaestroFill3dData.cpp:712-1188) over the nodal boxes grown by
    // one: s0mac_interp_type 1 puts s0 on the cells (two ghost cells, FillPatch with bcs_f) and
    // averages them to the faces; with uniform bins, 2 / 3 interpolate s0 at the face centres
    // (linear / quadratic in r_cc_loc, as Put1dArrayOnCart does at the cell centres)
    void MakeS0mac(const BS& s0, VF& s0mac) {
        const int t = P.s0mac_interp_type ? P.s0mac_interp_type : 1;
        VMF s0_cart(nlev);
        for (int lev = 0; lev < nlev; ++lev) s0_cart[lev].define(S[lev].L.ba, 1, 2, -1, 0.0);
        if (t == 1) Put1dArrayOnCart(s0, s0_cart, false, false, &bcs_f(), 0, false);
        for (int lev = 0; lev < nlev; ++lev) {
            const Lev& V = S[lev];
            const Level& L = V.L;
            for (int d = 0; d < 3; ++d) {
                s0mac[lev][d].define(L.ba, 1, 1, d, 0.0);
                const int di = d == 0, dj = d == 1, dk = d == 2;
                for (int b = 0; b < (int)L.ba.size(); ++b) {
                    const Arr& c = s0_cart[lev][b];
                    const Arr& o = s0mac[lev][d][b];
                    MO_FOR3(grow(nodal(L.ba[b], d), 1)) {
                        if (t == 1) {
                            o(i, j, k) = 0.5 * (c(i - di, j - dj, k - dk) + c(i, j, k));
                        } else {
                            const double x = P.prob_lo[0] + (double(i) + (di ? 0.0 : 0.5)) * L.dx[0] - V.center[0];
                            const double y = P.prob_lo[1] + (double(j) + (dj ? 0.0 : 0.5)) * L.dx[1] - V.center[1];
                            const double z = P.prob_lo[2] + (double(k) + (dk ? 0.0 : 0.5)) * L.dx[2] - V.center[2];
                            o(i, j, k) = V.sph_cell_value(s0[lev], std::sqrt(x * x + y * y + z * z), t);
                        }
                    }
                }
            }
        }
    }
    // Maestro::CelltoEdge over the chunks of every level, then RestrictBase of the edges
    // (Source/MaestroCelltoEdge.cpp:17-58, Source/MaestroBaseStateGeometry.cpp:240-262)
    void CelltoEdge(const BS& c, BS& e) const {
        e.assign(nlev, {});
        for (int n = 0; n < nlev; ++n) {
            e[n].assign(c[n].size() + 1, 0.0);
            for (auto& ch : chunks[n]) Lev::CelltoEdgeChunk(c[n], e[n], ch[0], ch[1] + 1);
        }
        for (int n = nlev - 1; n >= 1; --n)
            for (auto& ch : chunks[n])
                for (int j = ch[0]; j <= ch[1] + 1; j += 2) e[n - 1][j / 2] = e[n][j];
    }
    // BaseStateGeometry::InitMultiLevel, planar (Source/BaseStateGeometry.cpp:355-382), with the
    // radial rows of level n - 1 tagged wherever a level-n box lies above them.  Spherical: one
    // radial level (max_radial_level 0, Source/MaestroSetup.cpp:65), read whole by every level.
    void InitChunks() {
        chunks.assign(nlev, {});
        chunks[0].push_back({0, S[0].nr - 1});
        for (int n = 1; n < nlev; ++n) {
            if (P.spherical) {
                chunks[n].push_back({0, S[n].nr - 1});
                continue;
            }
            const int nrc = S[n - 1].nr;
            std::vector<int> tag(nrc, 0);
            for (const Box& b : S[n].L.ba)
                for (int r = b.lo[2]; r <= b.hi[2]; ++r) tag[r / 2] = 1;
            bool in = false;
            for (int r = 0; r < nrc; ++r) {
                if (tag[r] && !in) {
                    in = true;
                    chunks[n].push_back({2 * r, 0});
                } else if (!tag[r] && in) {
                    chunks[n].back()[1] = 2 * r - 1;
                    in = false;
                }
                if (in && r == nrc - 1) chunks[n].back()[1] = 2 * r + 1;
            }
        }
    }
    // BaseStateGeometry::ComputeCutoffCoords, base cutoff only (Source/BaseStateGeometry.cpp:164-210)
    void ComputeCutoffCoords() {
        bool found = false;
        int which = 0;
        std::vector<int> coord(nlev, 0);
        for (int n = nlev - 1; n >= 0; --n)
            for (auto& ch : chunks[n]) {
                if (found) break;
                for (int r = ch[0]; r <= ch[1]; ++r)
                    if (S[n].rho0_old[r] <= P.base_cutoff_density) {
                        coord[n] = r;
                        which = n;
                        found = true;
                        break;
                    }
            }
        if (!found) {
            which = nlev - 1;
            coord[which] = S[which].nr;
        }
        for (int n = which + 1; n < nlev; ++n) coord[n] = 2 * coord[n - 1] + 1;
        for (int n = which - 1; n >= 0; --n) coord[n] = coord[n + 1] % 2 == 0 ? coord[n + 1] / 2 : coord[n + 1] / 2 + 1;
        for (int n = 0; n < nlev; ++n) S[n].cutoff = coord[n];
    }

    // ------------------------------------------------------------------ FluxRegister
    // reflux_type 2 (Source/MaestroMakeFlux.cpp:412-456, Source/MaestroAdvection.cpp:258-276),
    // AMReX FluxRegister restated: level l >= 1 holds, per fine box and orientation (x-lo,
    // y-lo, z-lo, x-hi, y-hi, z-hi), one register value per coarse face of the coarsened
    // box's side and component.  CrseInit sets mult * coarse flux (read from the coarse box
    // owning the inside cell), FineAdd adds mult * each of the 4 fine faces in turn (outer =
    // the higher transverse direction), Reflux adds -reg/vol (lo) or +reg/vol (hi) to the
    // coarse cell outside the face, orientation by orientation.
    std::vector<std::vector<std::array<std::vector<real>, 6>>> freg;  // [lev][box][orientation]
    Box RegFaces(int lev, int b, int o) const {
        const int D = o % 3;
        Box f;
        for (int d = 0; d < 3; ++d) {
            f.lo[d] = S[lev].L.ba[b].lo[d] >> 1;
            f.hi[d] = S[lev].L.ba[b].hi[d] >> 1;
        }
        if (o >= 3) f.lo[D] = f.hi[D] + 1;
        f.hi[D] = f.lo[D];
        return f;
    }
    std::vector<real>& Reg(int lev, int b, int o) {
        if (freg.size() != (size_t)nlev) freg.assign(nlev, {});
        if (freg[lev].size() != S[lev].L.ba.size()) freg[lev].assign(S[lev].L.ba.size(), {});
        std::vector<real>& r = freg[lev][b][o];
        const Box f = RegFaces(lev, b, o);
        const size_t n = (size_t)(f.hi[0] - f.lo[0] + 1) * (f.hi[1] - f.lo[1] + 1) * (f.hi[2] - f.lo[2] + 1) * nscal;
        if (r.size() != n) r.assign(n, 0.0);
        return r;
    }
    static long FaceIdx(const Box& f, int i, int j, int k) {
        const long nx = f.hi[0] - f.lo[0] + 1, ny = f.hi[1] - f.lo[1] + 1;
        return (i - f.lo[0]) + nx * ((j - f.lo[1]) + ny * (long)(k - f.lo[2]));
    }
    void CrseInit(int levf, VF& sflux, int c0, int nc) {
        const int levc = levf - 1;
        const double* dx = S[levc].L.dx;
        const double area[3] = {dx[1] * dx[2], dx[0] * dx[2], dx[0] * dx[1]};
        Owner oc;
        oc.build(S[levc].L);
        for (int b = 0; b < (int)S[levf].L.ba.size(); ++b)
            for (int o = 0; o < 6; ++o) {
                const int D = o % 3;
                const double mult = -1.0 * dt_ * area[D];
                std::vector<real>& r = Reg(levf, b, o);
                const Box f = RegFaces(levf, b, o);
                MO_FOR3(f) {
                    int q[3] = {i, j, k};
                    if (o >= 3) q[D] -= 1;
                    const int cb = oc.at(S[levc].L, q[0], q[1], q[2]);
                    if (cb < 0) throw std::runtime_error("CrseInit: a coarse cell under the fine level has no box");
                    for (int n = c0; n < c0 + nc; ++n)
                        r[FaceIdx(f, i, j, k) * nscal + n] = mult * sflux[levc][D][cb](i, j, k, n);
                }
            }
    }
    void FineAdd(int levf, VF& sflux, int c0, int nc) {
        const double* dx = S[levf].L.dx;
        const double area[3] = {dx[1] * dx[2], dx[0] * dx[2], dx[0] * dx[1]};
        for (int b = 0; b < (int)S[levf].L.ba.size(); ++b)
            for (int o = 0; o < 6; ++o) {
                const int D = o % 3, t1 = D == 0 ? 1 : 0, t2 = D == 2 ? 1 : 2;
                const double mult = 1.0 * dt_ * area[D];
                std::vector<real>& r = Reg(levf, b, o);
                const Box f = RegFaces(levf, b, o);
                const Arr& fl = sflux[levf][D][b];
                MO_FOR3(f) {
                    for (int n = c0; n < c0 + nc; ++n) {
                        real v = r[FaceIdx(f, i, j, k) * nscal + n];
                        for (int oo = 0; oo < 2; ++oo)
                            for (int in = 0; in < 2; ++in) {
                                int q[3] = {2 * i, 2 * j, 2 * k};
                                q[t1] += in;
                                q[t2] += oo;
                                v = v + mult * fl(q[0], q[1], q[2], n);
                            }
                        r[FaceIdx(f, i, j, k) * nscal + n] = v;
                    }
                }
            }
    }
    void Reflux(int levf, VMF& snew, int c0, int nc) {
        const int levc = levf - 1;
        const Level& Lc = S[levc].L;
        const double vol = Lc.dx[0] * Lc.dx[1] * Lc.dx[2];
        Owner oc;
        oc.build(Lc);
        for (int o = 0; o < 6; ++o)
            for (int b = 0; b < (int)S[levf].L.ba.size(); ++b) {
                const int D = o % 3;
                std::vector<real>& r = Reg(levf, b, o);
                const Box f = RegFaces(levf, b, o);
                MO_FOR3(f) {
                    int q[3] = {i, j, k};
                    if (o < 3) q[D] -= 1;
                    const int len = Lc.dom.hi[D] - Lc.dom.lo[D] + 1;
                    if (Lc.per[D]) {
                        if (q[D] < Lc.dom.lo[D]) q[D] += len;
                        if (q[D] > Lc.dom.hi[D]) q[D] -= len;
                    }
                    const int cb = oc.at(Lc, q[0], q[1], q[2]);
                    if (cb < 0) continue;
                    const Arr& sn = snew[levc][cb];
                    for (int n = c0; n < c0 + nc; ++n) {
                        const real g = r[FaceIdx(f, i, j, k) * nscal + n];
                        if (o < 3) sn(q[0], q[1], q[2], n) = sn(q[0], q[1], q[2], n) - g / vol;
                        else sn(q[0], q[1], q[2], n) = sn(q[0], q[1], q[2], n) + g / vol;
                    }
                }
            }
    }
    double dt_ = 0.0;
    // the fluxes across levels: reflux_type 1 AverageDownFaces (Source/MaestroMakeFlux.cpp:460-462),
    // 2 the registers of the updated components (and Rho with the species)
    void FluxSync(VF& sflux, int c0, int nc) {
        if (P.reflux_type != 2) {
            AverageDownFaces(sflux);
            return;
        }
        dt_ = P.dt;
        for (int lev = 0; lev < nlev; ++lev) {
            if (lev + 1 < nlev) {
                CrseInit(lev + 1, sflux, c0, nc);
                if (c0 == FirstSpec) CrseInit(lev + 1, sflux, Rho, 1);
            }
            if (lev > 0) {
                FineAdd(lev, sflux, c0, nc);
                if (c0 == FirstSpec) FineAdd(lev, sflux, Rho, 1);
            }
        }
    }

    // ------------------------------------------------------------------ AdvancePremac
    void MakeUtrans(VMF& utilde, VMF& ufull, VF& utrans) {
        for (int lev = 0; lev < nlev; ++lev) S[lev].MakeUtrans(utilde[lev], ufull[lev], utrans[lev].data());
        SyncFaces(utrans);
    }
    void Addw0(VF& u, real mult) {
        for (int lev = 0; lev < nlev; ++lev) S[lev].Addw0(u[lev].data(), mult);
        SyncFaces(u);
    }
    // Maestro::MakeVelForce, planar (Source/MaestroForce.cpp:6-259)
    void MakeVelForce(VMF& vel_force, VF& uedge, VMF& sold, VMF& w0_force_cart, const BS* rho0 = nullptr) {
        VMF grav_cart(nlev), rho0_cart(nlev), gradw0_cart(nlev);
        for (int lev = 0; lev < nlev; ++lev) {
            grav_cart[lev].define(S[lev].L.ba, 3, 1, -1, 0.0);
            rho0_cart[lev].define(S[lev].L.ba, 1, 1, -1, 0.0);
        }
        // gradw0 = (w0(r+1) - w0(r)) / dr of the uniform bins, on the cells (Source/MaestroForce.cpp:36-50)
        const bool grad = P.spherical && !P.use_exact_base_state;
        if (grad) {
            BS gradw0(nlev);
            for (int lev = 0; lev < nlev; ++lev) {
                const Lev& L = S[lev];
                gradw0[lev].assign(L.nr, 0.0);
                for (int r = 0; r < L.nr; ++r) gradw0[lev][r] = (L.w0[r + 1] - L.w0[r]) / L.drf;
                gradw0_cart[lev].define(L.L.ba, 1, 1, -1, 0.0);
            }
            Put1dArrayOnCart(gradw0, gradw0_cart, false, false, &bcs_u(), 0, true);
        }
        Put1dArrayOnCart(rho0 ? *rho0 : bs(&Lev::rho0_old), rho0_cart, false, false, &bcs_s(), Rho, false);
        Put1dArrayOnCart(bs(&Lev::grav_cell), grav_cart, false, true, &bcs_f(), 0, false);
        for (int lev = 0; lev < nlev; ++lev)
            S[lev].MakeVelForce(vel_force[lev], uedge[lev].data(), sold[lev], w0_force_cart[lev], grav_cart[lev],
                                rho0_cart[lev], grad ? &gradw0_cart[lev] : nullptr);
        AverageDown(vel_force, 0, 3);
        FillPatch(vel_force, 0, 3, 0, bcs_u(), true);
    }
    void VelPred(VMF& utilde, VMF& ufull, VF& utrans, VF& umac, VMF& force) {
        for (int lev = 0; lev < nlev; ++lev)
            S[lev].VelPred(utilde[lev], ufull[lev], utrans[lev].data(), umac[lev].data(), force[lev]);
        AverageDownFaces(umac);
    }
    // Maestro::AdvancePremac (Source/MaestroAdvection.cpp:7-84)
    void AdvancePremac(VMF& uold, VMF& sold, VF& umac, VMF& w0_force_cart, VF& utrans, VMF& vel_force) {
        VMF utilde(nlev), ufull(nlev);
        for (int lev = 0; lev < nlev; ++lev) {
            const Level& L = S[lev].L;
            utilde[lev].define(L.ba, 3, ng_adv, -1, 0.0);
            for (int b = 0; b < (int)L.ba.size(); ++b)
                MO_FOR3(L.ba[b]) for (int n = 0; n < 3; ++n) utilde[lev][b](i, j, k, n) = uold[lev][b](i, j, k, n);
        }
        FillPatch(utilde, 0, 3, 0, bcs_u(), true);
        for (int lev = 0; lev < nlev; ++lev) {
            const Level& L = S[lev].L;
            ufull[lev].define(L.ba, 3, ng_adv, -1, 0.0);
            for (int b = 0; b < (int)L.ba.size(); ++b)
                MO_FOR3(L.ba[b]) for (int n = 0; n < 3; ++n) ufull[lev][b](i, j, k, n) = S[lev].w0_cart[b](i, j, k, n);
        }
        FillPatch(ufull, 0, 3, 0, bcs_u(), true);
        for (int lev = 0; lev < nlev; ++lev) {
            const Level& L = S[lev].L;
            for (int b = 0; b < (int)L.ba.size(); ++b)
                MO_FOR3(grow(L.ba[b], ng_adv)) for (int n = 0; n < 3; ++n) ufull[lev][b](i, j, k, n) +=
                    utilde[lev][b](i, j, k, n);
            for (int d = 0; d < 3; ++d) utrans[lev][d].define(L.ba, 1, 1, d, 0.0);
        }
        MakeUtrans(utilde, ufull, utrans);
        // the forces carry ng_s ghost cells when they are traced (Source/MaestroAdvection.cpp:62-67)
        const int ngf = P.ppm_trace_forces ? ng_s : 1;
        for (int lev = 0; lev < nlev; ++lev) vel_force[lev].define(S[lev].L.ba, 3, ngf, -1, 0.0);
        MakeVelForce(vel_force, utrans, sold, w0_force_cart);
        Addw0(utrans, 1.0);
        VelPred(utilde, ufull, utrans, umac, vel_force);
    }

    // ------------------------------------------------------------------ scalars
    void MakeEdgeScal(VMF& state, VF& sedge, VF& umac, VMF& force, const std::vector<BCRec>& bcs, int start_scomp,
                      int start_bccomp, int num_comp, bool is_conservative, bool is_vel = false) {
        for (int lev = 0; lev < nlev; ++lev)
            S[lev].MakeEdgeScal(state[lev], sedge[lev].data(), umac[lev].data(), force[lev], bcs, start_scomp,
                                start_bccomp, num_comp, is_conservative, is_vel);
        // edge restriction of velocity edge states (Source/MaestroMakeEdgeScalars.cpp:294-301)
        if (is_vel && nlev > 1) AverageDownFaces(sedge);
    }
    // Maestro::ModifyScalForce (Source/MaestroForce.cpp:261-467)
    void ModifyScalForce(VMF& scal_force, VMF& state, VF& umac, const BS& s0_edge, VMF& s0_cart, int comp,
                         int fullform) {
        VMF s0_edge_cart(nlev);
        for (int lev = 0; lev < nlev; ++lev) s0_edge_cart[lev].define(S[lev].L.ba, 1, 1);
        if (!P.spherical) Put1dArrayOnCart(s0_edge, s0_edge_cart, false, false, &bcs_f(), 0, false);
        // uniform bins: div(w0) of the shells on the cells (Source/MaestroForce.cpp:283-305)
        const bool divw = P.spherical && !P.use_exact_base_state;
        VMF divu_cart(nlev);
        if (divw) {
            BS divw0(nlev);
            for (int lev = 0; lev < nlev; ++lev) {
                const Lev& L = S[lev];
                divw0[lev].assign(L.nr, 0.0);
                const auto& re = L.r_edge_loc;
                const auto& rc = L.r_cc_loc;
                for (int r = 0; r < L.nr - 1; ++r) {
                    const double dr_loc = re[r + 1] - re[r];
                    divw0[lev][r] = (re[r + 1] * re[r + 1] * L.w0[r + 1] - re[r] * re[r] * L.w0[r]) / (dr_loc * rc[r] * rc[r]);
                }
                divu_cart[lev].define(L.L.ba, 1, 0, -1, 0.0);
            }
            Put1dArrayOnCart(divw0, divu_cart, false, false, &bcs_u(), 0, false);
        }
        for (int lev = 0; lev < nlev; ++lev)
            S[lev].ModifyScalForce(scal_force[lev], state[lev], umac[lev].data(), s0_edge_cart[lev], s0_cart[lev], comp,
                                   fullform, divw ? &divu_cart[lev] : nullptr);
        AverageDown(scal_force, comp, 1);
        FillPatch(scal_force, comp, 1, 0, bcs_f(), false);
    }
    // Maestro::MakeRhoHForce (Source/MaestroForce.cpp:469-679)
    void MakeRhoHForce(VMF& scal_force, int is_prediction, VF& umac, int add_thermal, int which_step) {
        BS r0(nlev), pp0(nlev);
        for (int lev = 0; lev < nlev; ++lev) {
            const Lev& L = S[lev];
            r0[lev].resize(L.nr);
            pp0[lev].resize(L.nr);
            for (int r = 0; r < L.nr; ++r) {
                r0[lev][r] = which_step == 1 ? L.rho0_old[r] : 0.5 * (L.rho0_old[r] + L.rho0_new[r]);
                pp0[lev][r] = which_step == 1 ? L.p0_old[r] : 0.5 * (L.p0_old[r] + L.p0_new[r]);
            }
        }
        VMF p0_cart(nlev), psi_cart(nlev), grav_cart(nlev), rho0_cart(nlev);
        for (int lev = 0; lev < nlev; ++lev) {
            p0_cart[lev].define(S[lev].L.ba, 1, 1, -1, 0.0);
            psi_cart[lev].define(S[lev].L.ba, 1, 1, -1, 0.0);
            grav_cart[lev].define(S[lev].L.ba, 1, 1, -1, 0.0);
            rho0_cart[lev].define(S[lev].L.ba, 1, 1, -1, 0.0);
        }
        Put1dArrayOnCart(pp0, p0_cart, false, false, &bcs_f(), 0, false);
        VF p0mac(nlev);
        if (P.spherical) MakeS0mac(pp0, p0mac);
        Put1dArrayOnCart(bs(&Lev::psi), psi_cart, false, false, &bcs_f(), 0, false);
        Put1dArrayOnCart(r0, rho0_cart, false, false, &bcs_s(), Rho, false);
        // MakeGravCell: planar, the constant gravity of grav_cell; the spherical force does
        // not read it
        if (!P.spherical) Put1dArrayOnCart(bs(&Lev::grav_cell), grav_cart, false, false, &bcs_f(), 0, false);
        for (int lev = 0; lev < nlev; ++lev)
            S[lev].MakeRhoHForce(scal_force[lev], is_prediction, umac[lev].data(), add_thermal, p0_cart[lev],
                                 psi_cart[lev], grav_cart[lev], rho0_cart[lev], p0mac[lev].data());
        AverageDown(scal_force, RhoH, 1);
        FillPatch(scal_force, RhoH, 1, 0, bcs_f(), false);
    }
    // Maestro::PutInPertForm (Source/MaestroConvert.cpp:6-34)
    void PutInPertForm(VMF& scal, const BS& s0, int comp, int bccomp, const std::vector<BCRec>& bcs, bool flag) {
        for (int lev = 0; lev < nlev; ++lev) S[lev].PutInPertForm(scal[lev], s0[lev], comp, flag);
        AverageDown(scal, comp, 1);
        FillPatch(scal, comp, 1, bccomp, bcs, false, comp);
    }
    // Maestro::ConvertRhoXToX (Source/MaestroConvert.cpp:64-91)
    void ConvertRhoXToX(VMF& scal, bool flag) {
        for (int lev = 0; lev < nlev; ++lev) S[lev].ConvertRhoXToX(scal[lev], flag);
        AverageDown(scal, FirstSpec, nspec);
        if (flag) FillPatch(scal, FirstSpec, nspec, 0, bcs_f(), false, FirstSpec);
        else FillPatch(scal, FirstSpec, nspec, FirstSpec, bcs_s(), false, FirstSpec);
    }
    // Maestro::MakeRhoXFlux (Source/MaestroMakeFlux.cpp:18-465)
    void MakeRhoXFlux(VF& sflux, VMF& eta, VF& sedge, VF& umac, const BS& r0_old, const BS& r0e_old, const BS& r0_new,
                      const BS& r0e_new, int start_comp, int num_comp) {
        VF r0mac_old(nlev), r0mac_new(nlev);
        if (P.spherical) {  // Source/MaestroDensityAdvance.cpp:167-179, 193-213
            MakeS0mac(r0_old, r0mac_old);
            MakeS0mac(r0_new, r0mac_new);
        }
        for (int lev = 0; lev < nlev; ++lev)
            S[lev].MakeRhoXFlux(sflux[lev].data(), eta[lev], sedge[lev].data(), umac[lev].data(), r0_old[lev],
                                r0e_old[lev], r0_new[lev], r0e_new[lev], start_comp, num_comp, r0mac_old[lev].data(),
                                r0mac_new[lev].data());
        FluxSync(sflux, start_comp, num_comp);
    }
    // Maestro::MakeRhoHFlux (Source/MaestroMakeFlux.cpp:467-1067)
    void MakeRhoHFlux(VF& sflux, VF& sedge, VF& umac, const BS& rh0_old, const BS& rh0e_old, const BS& rh0_new,
                      const BS& rh0e_new, const BS* r0_old = nullptr, const BS* r0e_old = nullptr,
                      const BS* r0_new = nullptr, const BS* r0e_new = nullptr) {
        VF h0mac_old(nlev), h0mac_new(nlev), r0mac_old(nlev), r0mac_new(nlev);
        if (P.spherical && P.use_exact_base_state) {  // rhoh0 on faces (Source/MaestroEnthalpyAdvance.cpp:187-220)
            MakeS0mac(rh0_old, h0mac_old);
            MakeS0mac(rh0_new, h0mac_new);
        } else if (P.spherical) {  // rho0 and h0 = rhoh0 / rho0 on faces (:194-220, 251-300)
            BS h0o(nlev), h0n(nlev);
            for (int lev = 0; lev < nlev; ++lev) {
                h0o[lev].resize(rh0_old[lev].size());
                h0n[lev].resize(rh0_new[lev].size());
                for (size_t r = 0; r < h0o[lev].size(); ++r) {
                    h0o[lev][r] = rh0_old[lev][r] / (*r0_old)[lev][r];
                    h0n[lev][r] = rh0_new[lev][r] / (*r0_new)[lev][r];
                }
            }
            MakeS0mac(*r0_old, r0mac_old);
            MakeS0mac(*r0_new, r0mac_new);
            MakeS0mac(h0o, h0mac_old);
            MakeS0mac(h0n, h0mac_new);
        }
        for (int lev = 0; lev < nlev; ++lev)
            S[lev].MakeRhoHFlux(sflux[lev].data(), sedge[lev].data(), umac[lev].data(), rh0_old[lev], rh0e_old[lev],
                                rh0_new[lev], rh0e_new[lev], h0mac_old[lev].data(), h0mac_new[lev].data(),
                                r0_old ? &(*r0_old)[lev] : nullptr, r0e_old ? &(*r0e_old)[lev] : nullptr,
                                r0_new ? &(*r0_new)[lev] : nullptr, r0e_new ? &(*r0e_new)[lev] : nullptr,
                                r0mac_old[lev].data(), r0mac_new[lev].data());
        FluxSync(sflux, RhoH, 1);
    }
    // Maestro::ConvertRhoHToH with its AverageDown and FillPatch (Source/MaestroConvert.cpp:93-114)
    void ConvertRhoHToH(VMF& scal, bool flag) {
        for (int lev = 0; lev < nlev; ++lev) S[lev].ConvertRhoHToH(scal[lev], flag);
        AverageDown(scal, RhoH, 1);
        if (flag) FillPatch(scal, RhoH, 1, 0, bcs_f(), false, RhoH);
        else FillPatch(scal, RhoH, 1, RhoH, bcs_s(), false, RhoH);
    }
    // Maestro::UpdateScal (Source/MaestroAdvection.cpp:86-297)
    void UpdateScal(VMF& sold, VMF& snew, VF& sflux, VMF& force, int start_comp, int num_comp) {
        for (int lev = 0; lev < nlev; ++lev)
            S[lev].UpdateScal(sold[lev], snew[lev], sflux[lev].data(), force[lev], start_comp, num_comp);
        if (P.reflux_type == 2)
            for (int lev = nlev - 2; lev >= 0; --lev) {
                Reflux(lev + 1, snew, start_comp, num_comp);
                if (start_comp == FirstSpec) Reflux(lev + 1, snew, Rho, 1);
            }
        AverageDown(snew, start_comp, num_comp);
        FillPatch(snew, start_comp, num_comp, start_comp, bcs_s(), false, start_comp);
        if (start_comp == FirstSpec) {
            AverageDown(snew, Rho, 1);
            FillPatch(snew, Rho, 1, Rho, bcs_s(), false, Rho);
        }
    }

    // ------------------------------------------------------------------ drivers
    // Maestro::DensityAdvance (Source/MaestroDensityAdvance.cpp:6-243); which_step 2 passes the
    // new base state to the flux for the old/new averages (:186-219)
    void DensityAdvance(VMF& scalold, VMF& scalnew, VF& sedge, VF& sflux, VMF& scal_force, VMF& etarhoflux, VF& umac,
                        int which_step) {
        const int spt = P.species_pred_type;
        const BS rho0_old = bs(&Lev::rho0_old), rho0_new = bs(&Lev::rho0_new);
        BS rho0_edge_old(nlev), rho0_edge_new(nlev);
        if (!P.spherical) {  // spherical: no planar edge state (Source/MaestroDensityAdvance.cpp:22-25)
            CelltoEdge(rho0_old, rho0_edge_old);
            CelltoEdge(rho0_new, rho0_edge_new);
        }
        for (auto& f : scal_force) f.setVal(0.0);
        VMF rho0_old_cart(nlev);
        for (int lev = 0; lev < nlev; ++lev) rho0_old_cart[lev].define(S[lev].L.ba, 1, 1, -1, 0.0);
        Put1dArrayOnCart(rho0_old, rho0_old_cart, false, false, &bcs_s(), Rho, false);
        Addw0(umac, -1.0);
        if (spt == 1) ModifyScalForce(scal_force, scalold, umac, rho0_edge_old, rho0_old_cart, Rho, 0);
        else if (spt == 3) ModifyScalForce(scal_force, scalold, umac, rho0_edge_old, rho0_old_cart, Rho, 1);
        Addw0(umac, 1.0);
        if (spt == 1 || spt == 3) ConvertRhoXToX(scalold, true);
        if (spt == 1) PutInPertForm(scalold, rho0_old, Rho, 0, bcs_f(), true);
        MakeEdgeScal(scalold, sedge, umac, scal_force, bcs_s(), FirstSpec, FirstSpec, nspec, spt == 2);
        if (spt == 1 || spt == 3) {
            MakeEdgeScal(scalold, sedge, umac, scal_force, bcs_s(), Rho, Rho, 1, false);
        } else {
            for (int lev = 0; lev < nlev; ++lev)
                for (int d = 0; d < 3; ++d)
                    for (int b = 0; b < (int)S[lev].L.ba.size(); ++b) {
                        const Arr& e = sedge[lev][d][b];
                        MO_FOR3(nodal(S[lev].L.ba[b], d)) {
                            e(i, j, k, Rho) = e(i, j, k, FirstSpec);
                            for (int ispec = 1; ispec < nspec; ++ispec) e(i, j, k, Rho) += e(i, j, k, FirstSpec + ispec);
                        }
                    }
        }
        if (spt == 1) PutInPertForm(scalold, rho0_old, Rho, Rho, bcs_s(), false);
        if (spt == 1 || spt == 3) ConvertRhoXToX(scalold, false);
        if (which_step == 1)
            MakeRhoXFlux(sflux, etarhoflux, sedge, umac, rho0_old, rho0_edge_old, rho0_old, rho0_edge_old, FirstSpec,
                         nspec);
        else
            MakeRhoXFlux(sflux, etarhoflux, sedge, umac, rho0_old, rho0_edge_old, rho0_new, rho0_edge_new, FirstSpec,
                         nspec);
        for (auto& f : scal_force) f.setVal(0.0);
        UpdateScal(scalold, scalnew, sflux, scal_force, FirstSpec, nspec);
    }

    // Maestro::EnthalpyAdvance (Source/MaestroEnthalpyAdvance.cpp:6-352); which_step 2 averages
    // the old and new base state in the flux (:234-317) and in the final MakeRhoHForce (:336)
    void EnthalpyAdvance(VMF& scalold, VMF& scalnew, VF& sedge, VF& sflux, VMF& scal_force, VF& umac, int which_step) {
        const int ept = P.enthalpy_pred_type;
        const BS rhoh0_old = bs(&Lev::rhoh0_old), rhoh0_new = bs(&Lev::rhoh0_new);
        BS rhoh0_edge_old(nlev), rhoh0_edge_new(nlev);
        if (!P.spherical) {
            CelltoEdge(rhoh0_old, rhoh0_edge_old);
            CelltoEdge(rhoh0_new, rhoh0_edge_new);
        }
        // predict_h: (rho h) -> h (Source/MaestroEnthalpyAdvance.cpp:40-43)
        if (ept == 2) ConvertRhoHToH(scalold, true);
        for (auto& f : scal_force) f.setVal(0.0);
        VMF rhoh0_old_cart(nlev);
        for (int lev = 0; lev < nlev; ++lev) rhoh0_old_cart[lev].define(S[lev].L.ba, 1, 1, -1, 0.0);
        Addw0(umac, -1.0);
        MakeRhoHForce(scal_force, 1, umac, 1, 1);
        if (ept == 1) {
            Put1dArrayOnCart(rhoh0_old, rhoh0_old_cart, false, false, &bcs_s(), RhoH, false);
            ModifyScalForce(scal_force, scalold, umac, rhoh0_edge_old, rhoh0_old_cart, RhoH, 0);
        }
        if (ept == 2)  // the force of h: that of (rho h) over rho, one ghost cell (:80-88)
            for (int lev = 0; lev < nlev; ++lev)
                for (int b = 0; b < S[lev].nb; ++b) {
                    const Arr& f = scal_force[lev][b];
                    const Arr& so = scalold[lev][b];
                    MO_FOR3(grow(S[lev].L.ba[b], 1)) f(i, j, k, RhoH) = f(i, j, k, RhoH) / so(i, j, k, Rho);
                }
        Addw0(umac, 1.0);
        if (ept == 1) PutInPertForm(scalold, rhoh0_old, RhoH, 0, bcs_f(), true);
        MakeEdgeScal(scalold, sedge, umac, scal_force, bcs_s(), RhoH, RhoH, 1, ept == 0);
        if (ept == 1) PutInPertForm(scalold, rhoh0_old, RhoH, RhoH, bcs_s(), false);
        if (ept == 2) ConvertRhoHToH(scalold, false);  // h -> (rho h) (:164-167)
        const BS rho0_old = bs(&Lev::rho0_old), rho0_new = bs(&Lev::rho0_new);
        BS rho0_edge_old(nlev), rho0_edge_new(nlev);
        if (!P.spherical) {
            CelltoEdge(rho0_old, rho0_edge_old);
            CelltoEdge(rho0_new, rho0_edge_new);
        }
        if (which_step == 1)
            MakeRhoHFlux(sflux, sedge, umac, rhoh0_old, rhoh0_edge_old, rhoh0_old, rhoh0_edge_old, &rho0_old,
                         &rho0_edge_old, &rho0_old, &rho0_edge_old);
        else
            MakeRhoHFlux(sflux, sedge, umac, rhoh0_old, rhoh0_edge_old, rhoh0_new, rhoh0_edge_new, &rho0_old,
                         &rho0_edge_old, &rho0_new, &rho0_edge_new);
        for (auto& f : scal_force) f.setVal(0.0, RhoH, 1, 1);
        Addw0(umac, -1.0);
        MakeRhoHForce(scal_force, 0, umac, 0, which_step);
        Addw0(umac, 1.0);
        UpdateScal(scalold, scalnew, sflux, scal_force, RhoH, 1);
    }

    // Maestro::VelocityAdvance (Source/MaestroVelocityAdvance.cpp:5-82) and UpdateVel
    // (Source/MaestroAdvection.cpp:299-526, with its AverageDown + FillPatch): umac holds the
    // projected MAC velocity without w0, its ghost faces filled; uold its ghost cells
    void VelocityAdvance(VMF& uold, VMF& sold, VMF& rhohalf, VF& umac, VMF& w0_force_cart, VMF& unew, VF& uedge,
                         VMF* sponge) {
        VMF vel_force(nlev);
        for (int lev = 0; lev < nlev; ++lev) {
            vel_force[lev].define(S[lev].L.ba, 3, P.ppm_trace_forces ? ng_s : 1, -1, 0.0);
            for (int d = 0; d < 3; ++d) uedge[lev][d].define(S[lev].L.ba, 3, 0, d, 0.0);
        }
        MakeVelForce(vel_force, umac, sold, w0_force_cart);
        Addw0(umac, 1.0);
        MakeEdgeScal(uold, uedge, umac, vel_force, bcs_u(), 0, 0, 3, false, true);
        Addw0(umac, -1.0);
        BS rho0_nph(nlev);
        for (int lev = 0; lev < nlev; ++lev) {
            const Lev& L = S[lev];
            rho0_nph[lev].resize(L.nr);
            for (int r = 0; r < L.nr; ++r) rho0_nph[lev][r] = 0.5 * (L.rho0_old[r] + L.rho0_new[r]);
        }
        MakeVelForce(vel_force, umac, rhohalf, w0_force_cart, &rho0_nph);
        for (int lev = 0; lev < nlev; ++lev)
            S[lev].UpdateVel(uold[lev], unew[lev], umac[lev].data(), uedge[lev].data(), vel_force[lev],
                             sponge ? &(*sponge)[lev] : nullptr);
        AverageDown(unew, 0, 3);
        FillPatch(unew, 0, 3, 0, bcs_u(), true);
    }

    // Maestro::EstDt (Source/MaestroDt.cpp:11-225 planar, :301-384 spherical; the divU and
    // dS/dt constraints :226-300, :385-438 are not restated: they need S_cc, dSdt and
    // gamma1bar from the reactions / EOS part of the step), evaluated box by box as the
    // reference does.  vel_force: MakeVelForce with a zero MAC velocity and w0_force
    // (:14-81); the spherical w0mac is zero with the exact base state (:44-64).  Returns dt
    // before the max_dt / fixed_dt / small_dt clamps; umax before the 1e-8 of rel_eps.
    void EstDt(VMF& uold, VMF& sold, double cfl, int drdxfac, double& dt, double& umax) {
        VMF vel_force(nlev), w0f(nlev);
        VF umac0(nlev);
        for (int lev = 0; lev < nlev; ++lev) {
            vel_force[lev].define(S[lev].L.ba, 3, P.ppm_trace_forces ? ng_s : 1, -1, 0.0);
            w0f[lev].define(S[lev].L.ba, 3, 1, -1, 0.0);
            for (int d = 0; d < 3; ++d) umac0[lev][d].define(S[lev].L.ba, 1, 1, d, 0.0);
        }
        MakeVelForce(vel_force, umac0, sold, w0f);
        dt = 1.e20;
        umax = 0.0;
        const int nd = P.dim == 2 ? 2 : 3;
        for (int lev = 0; lev < nlev; ++lev) {
            const Lev& L = S[lev];
            const double* dx = L.L.dx;
            double dt_lev = 1.e50, umax_lev = 0.0;
            for (int b = 0; b < L.nb; ++b) {
                const Arr &u = uold[lev][b], &w0c = L.w0_cart[b], &f = vel_force[lev][b];
                double spd[3] = {0.0, 0.0, 0.0}, spdr = 0.0, fm[3] = {0.0, 0.0, 0.0};
                // spherical: w0mac from MakeW0mac with uniform bins and an evolving base
                // state, else 0 (Source/MaestroDt.cpp:42-64, 313-334)
                const bool w0m = P.spherical && !P.use_exact_base_state && P.evolve_base_state;
                MO_FOR3(L.L.ba[b]) {
                    for (int d = 0; d < nd; ++d) {
                        real v = u(i, j, k, d);
                        if (!P.spherical && d == nd - 1)
                            v = u(i, j, k, d) + 0.5 * (w0c(i, j, k, d) + w0c(i, j + (d == 1), k + (d == 2), d));
                        if (P.spherical && w0m)
                            v = u(i, j, k, d) + 0.5 * (L.w0mac[d][b](i, j, k) +
                                                       L.w0mac[d][b](i + (d == 0), j + (d == 1), k + (d == 2)));
                        else if (P.spherical)
                            v = u(i, j, k, d) + 0.5 * (0.0 + 0.0);
                        spd[d] = std::max(spd[d], std::fabs(value_of(v)));
                        fm[d] = std::max(fm[d], std::fabs(value_of(f(i, j, k, d))));
                    }
                    spdr = std::max(spdr, std::fabs(value_of(w0c(i, j, k, P.spherical ? 0 : nd - 1))));
                }
                const double eps = 1.e-8;
                double dt_temp = 1.e99;
                const double umax_grid = std::max(spd[0], std::max(spd[1], std::max(spd[2], spdr)));
                for (int d = 0; d < nd; ++d)
                    if (spd[d] > eps) dt_temp = std::min(dt_temp, dx[d] / spd[d]);
                const double dr = P.spherical ? (L.dxf / drdxfac) : dx[nd - 1];
                if (spdr > eps) dt_temp = std::min(dt_temp, dr / spdr);
                dt_temp *= cfl;
                for (int d = 0; d < nd; ++d)
                    if (fm[d] > eps) dt_temp = std::min(dt_temp, std::sqrt(2.0 * dx[d] / fm[d]));
                dt_lev = std::min(dt_lev, dt_temp);
                umax_lev = std::max(umax_lev, umax_grid);
            }
            umax = std::max(umax, umax_lev);
            dt = std::min(dt, dt_lev);
        }
    }
};

}  // namespace mo
#include "mo_stage2d.hpp"
namespace mo {

// ---------------------------------------------------------------------- flat I/O
static long ncell_of(const Box& d) {
    return (long)(d.hi[0] - d.lo[0] + 1) * (d.hi[1] - d.lo[1] + 1) * (d.hi[2] - d.lo[2] + 1);
}
static void face_ext(const Box& dom, int d, long ext[3]) {
    for (int e = 0; e < 3; ++e) ext[e] = dom.hi[e] - dom.lo[e] + 1 + (e == d ? 1 : 0);
}
// scatter domain-flat cell data [nc][ncell] into the valid region of an MF
static void scatter_cells(const Box& dom, const double* src, MF& mf, int c0, int nc) {
    long nx = dom.hi[0] - dom.lo[0] + 1, ny = dom.hi[1] - dom.lo[1] + 1, N = ncell_of(dom);
    for (int b = 0; b < mf.size(); ++b)
        for (int n = 0; n < nc; ++n) MO_FOR3(mf.ba[b]) {
                long idx = (i - dom.lo[0]) + nx * ((j - dom.lo[1]) + ny * (long)(k - dom.lo[2]));
                mf[b](i, j, k, c0 + n) = src[(long)n * N + idx];
            }
}
#ifdef MO_TANGENT
// the directional derivative of scattered cell data (its values already in place)
static void seed_cells(const Box& dom, const double* dsrc, MF& mf, int c0, int nc) {
    long nx = dom.hi[0] - dom.lo[0] + 1, ny = dom.hi[1] - dom.lo[1] + 1, N = ncell_of(dom);
    for (int b = 0; b < mf.size(); ++b)
        for (int n = 0; n < nc; ++n) MO_FOR3(mf.ba[b]) {
                long idx = (i - dom.lo[0]) + nx * ((j - dom.lo[1]) + ny * (long)(k - dom.lo[2]));
                mf[b](i, j, k, c0 + n).d = dsrc[(long)n * N + idx];
            }
}
#endif
static void gather_cells(const Box& dom, const MF& mf, int c0, int nc, double* dst, bool tangent = false) {
    long nx = dom.hi[0] - dom.lo[0] + 1, ny = dom.hi[1] - dom.lo[1] + 1, N = ncell_of(dom);
    for (int b = 0; b < mf.size(); ++b)
        for (int n = 0; n < nc; ++n) MO_FOR3(mf.ba[b]) {
                long idx = (i - dom.lo[0]) + nx * ((j - dom.lo[1]) + ny * (long)(k - dom.lo[2]));
                const real& x = mf[b](i, j, k, c0 + n);
                dst[(long)n * N + idx] = tangent ? tangent_of(x) : value_of(x);
            }
}
static void gather_faces(const Box& dom, const MF& mf, int d, int c0, int nc, double* dst) {
    long ext[3];
    face_ext(dom, d, ext);
    long N = ext[0] * ext[1] * ext[2];
    for (int b = 0; b < mf.size(); ++b) {
        Box vb = nodal(mf.ba[b], d);
        for (int n = 0; n < nc; ++n) MO_FOR3(vb) {
                long idx = (i - dom.lo[0]) + ext[0] * ((j - dom.lo[1]) + ext[1] * (long)(k - dom.lo[2]));
                dst[(long)n * N + idx] = value_of(mf[b](i, j, k, c0 + n));
            }
    }
}

// nr_fine of spherical geometry with uniform radial bins (Source/MaestroSetup.cpp:83-95)
static int mo_sph_nr_fine(const mo_params* p, int nlev) {
    const double dxf = p->dx[0] / (1 << (nlev - 1));
    const double drf = dxf / (p->drdxfac > 0 ? p->drdxfac : 1);
    const double lenx = 0.5 * (p->prob_hi[0] - p->prob_lo[0]);
    const double leny = 0.5 * (p->prob_hi[1] - p->prob_lo[1]);
    const double lenz = 0.5 * (p->prob_hi[2] - p->prob_lo[2]);
    const double max_dist = std::sqrt(lenx * lenx + leny * leny + lenz * lenz);
    return int(max_dist / drf) + 1;
}

// The levels, boundary conditions, base state, w0_cart and (spherical) w0mac of a stage call.
static void setup_stage(Stage& H, const mo_params* p, int nlev, const int* nboxes, const int* boxes,
                        const mo_inputs* in) {
    if (nlev < 1 || nlev > 4) throw std::runtime_error("1 to 4 levels");
    if (p->ppm_trace_forces != 0 && (p->ppm_type == 0 || p->ppm_trace_forces != 1))
        throw std::runtime_error("ppm_trace_forces = 1 needs ppm_type 1 or 2 (the reference reads untraced forces "
                                 "with ppm_type 0)");
    if (p->use_exact_base_state && !p->spherical) throw std::runtime_error("use_exact_base_state is spherical-only");
    if (p->spherical) {
        if (p->use_exact_base_state && p->enthalpy_pred_type != 1)
            throw std::runtime_error("spherical with the exact base state: enthalpy_pred_type 1");
        if (!p->use_exact_base_state && p->enthalpy_pred_type > 2)
            throw std::runtime_error("spherical with uniform radial bins: enthalpy_pred_type 0, 1 or 2");
        if (p->use_exact_base_state && p->s0mac_interp_type > 1)
            throw std::runtime_error("exact base state: s0mac_interp_type 1 (types 2 and 3 index the irregular grid "
                                     "past its end, Source/MaestroFill3dData.cpp:786-790)");
        if (p->w0_interp_type < 0 || p->w0_interp_type > 3 || p->w0mac_interp_type < 0 || p->w0mac_interp_type > 4 ||
            p->s0_interp_type < 0 || p->s0_interp_type > 3 || p->s0mac_interp_type < 0 || p->s0mac_interp_type > 3 ||
            p->drdxfac < 0)
            throw std::runtime_error("interpolation type out of range");
    }
    if (!(p->enthalpy_pred_type >= 0 && p->enthalpy_pred_type <= 2))
        throw std::runtime_error("enthalpy_pred_type must be 0, 1 or 2");
    if (!(p->species_pred_type >= 1 && p->species_pred_type <= 3))
        throw std::runtime_error("species_pred_type must be 1, 2 or 3");
    H.P = *p;
    H.nlev = nlev;
    H.nspec = p->nspec;
    H.nscal = 4 + p->nspec;
    H.ng_s = H.ng_adv = p->ppm_type == 2 ? 4 : 3;
    H.S.resize(nlev);
    int off = 0;
    for (int lev = 0; lev < nlev; ++lev) {
        Lev& S = H.S[lev];
        S.P = *p;
        S.lev = lev;
        S.nspec = H.nspec;
        S.nscal = H.nscal;
        const int r = 1 << lev;
        for (int d = 0; d < 3; ++d) {
            S.L.dom.lo[d] = p->dom_lo[d] * r;
            S.L.dom.hi[d] = (p->dom_hi[d] + 1) * r - 1;
            S.L.per[d] = (p->phys_bc_lo[d] == interior);
            if ((p->phys_bc_lo[d] == interior) != (p->phys_bc_hi[d] == interior))
                throw std::runtime_error("periodic direction needs interior on both sides");
            S.L.dx[d] = p->dx[d] / r;
        }
        for (int b = 0; b < nboxes[lev]; ++b) {
            Box bx;
            for (int d = 0; d < 3; ++d) {
                bx.lo[d] = boxes[6 * (off + b) + d];
                bx.hi[d] = boxes[6 * (off + b) + 3 + d];
            }
            S.L.ba.push_back(bx);
        }
        off += nboxes[lev];
        S.nb = nboxes[lev];
        S.nr = S.L.dom.hi[2] - S.L.dom.lo[2] + 1;
        if (p->spherical) {
            // nr_fine from the finest level (Source/MaestroSetup.cpp:60-96): nr_irreg + 1 for the
            // exact base state, else int(max_dist / dr_fine) + 1 with dr_fine = dx_fine / drdxfac
            const int rf = 1 << (nlev - 1);
            S.dxf = p->dx[0] / rf;
            if (p->use_exact_base_state) {
                const double domhi = (p->dom_hi[0] + 1) * rf;
                S.nr = int((3.0 * (domhi / 2 - 0.5) * (domhi / 2 - 0.5) - 0.75) / 2.0) + 1;
            } else {
                S.nr = mo_sph_nr_fine(p, nlev);
            }
        }
        S.ng_s = S.ng_adv = H.ng_s;
        S.dt = p->dt;
        S.rel_eps = p->rel_eps;
        S.pc = PPMCtx{p->ppm_type, p->dt, p->rel_eps, {S.L.dx[0], S.L.dx[1], S.L.dx[2]}, S.L.dom};
        S.BCSetup();
        const int nr = S.nr;
        auto vec = [](const double* a, int n) { return std::vector<real>(a, a + n); };
        const mo_inputs& I = p->spherical ? in[0] : in[lev];  // spherical: one radial base state
        S.rho0_old = vec(I.rho0_old, nr);
        S.rho0_new = vec(I.rho0_new, nr);
        S.rhoh0_old = vec(I.rhoh0_old, nr);
        S.rhoh0_new = vec(I.rhoh0_new, nr);
        S.p0_old = vec(I.p0_old, nr);
        S.p0_new = vec(I.p0_new, nr);
        S.psi = vec(I.psi, nr);
        S.grav_cell = vec(I.grav_cell, nr);
        S.w0_force = vec(I.w0_force, nr);
        S.w0 = vec(I.w0, nr + 1);
        S.rho0_predicted_edge = vec(I.rho0_predicted_edge, nr + 1);
        S.cutoff = p->base_cutoff_density_coord;
        if (p->spherical) S.InitSphr();
    }
    H.InitChunks();
    if (nlev > 1 && !p->spherical) H.ComputeCutoffCoords();  // spherical: no kernel reads it

    // w0_cart: Put1dArrayOnCart(w0, w0_cart, true, true, bcs_u, 0, 1) (Source/MaestroAdvance.cpp:326)
    VMF w0c(nlev);
    for (int lev = 0; lev < nlev; ++lev) w0c[lev].define(H.S[lev].L.ba, 3, 2, -1, 0.0);
    H.Put1dArrayOnCart(H.bs(&Lev::w0), w0c, true, true, &H.bcs_u(), 0, true);
    for (int lev = 0; lev < nlev; ++lev) H.S[lev].w0_cart = std::move(w0c[lev]);
    if (p->spherical)  // MakeW0mac (Source/MaestroAdvance.cpp:335-338)
        for (int lev = 0; lev < nlev; ++lev) H.S[lev].MakeW0mac();
}

// Tangent seeds of one level (tangent build): derivatives of uold and sold, and where the
// derivative of snew goes; all [nc][ncell] like the values.
struct TangentIO {
    const double* duold;
    const double* dsold;
    double* dsnew;
};

static int run_stage(const mo_params* p, int nlev, const int* nboxes, const int* boxes, const mo_inputs* in,
                     mo_outputs* out, int which_step, const TangentIO* tl = nullptr) {
    if (which_step != 1 && which_step != 2) throw std::runtime_error("which_step must be 1 or 2");
    Stage H;
    setup_stage(H, p, nlev, nboxes, boxes, in);
    const int nscal = H.nscal;
    VMF w0_force_cart(nlev);
    for (int lev = 0; lev < nlev; ++lev) w0_force_cart[lev].define(H.S[lev].L.ba, 3, 1, -1, 0.0);
    if (p->evolve_base_state)
        H.Put1dArrayOnCart(H.bs(&Lev::w0_force), w0_force_cart, false, true, &H.bcs_f(), 0, false);

    VMF uold(nlev), sold(nlev), snew(nlev), etarhoflux(nlev), scal_force(nlev), vel_force(nlev);
    VF umac(nlev), utrans(nlev), sedge(nlev), sflux(nlev);
    for (int lev = 0; lev < nlev; ++lev) {
        Lev& S = H.S[lev];
        const Box& dom = S.L.dom;
        uold[lev].define(S.L.ba, 3, H.ng_s, -1, 0.0);
        sold[lev].define(S.L.ba, nscal, H.ng_s, -1, 0.0);
        snew[lev].define(S.L.ba, nscal, H.ng_s, -1, 0.0);
        S.gpi.define(S.L.ba, 3, 0, -1, 0.0);
        S.thermal.define(S.L.ba, 1, 1, -1, 0.0);
        scatter_cells(dom, in[lev].uold, uold[lev], 0, 3);
        scatter_cells(dom, in[lev].sold, sold[lev], 0, nscal);
#ifdef MO_TANGENT
        if (tl) {
            seed_cells(dom, tl[lev].duold, uold[lev], 0, 3);
            seed_cells(dom, tl[lev].dsold, sold[lev], 0, nscal);
        }
#else
        if (tl) throw std::runtime_error("tangent seeds need the tangent build");
#endif
        scatter_cells(dom, in[lev].gpi, S.gpi, 0, 3);
        if (in[lev].thermal) scatter_cells(dom, in[lev].thermal, S.thermal, 0, 1);
        for (int d = 0; d < 3; ++d) {
            umac[lev][d].define(S.L.ba, 1, 1, d, 0.0);
            sedge[lev][d].define(S.L.ba, nscal, 0, d, 0.0);
            sflux[lev][d].define(S.L.ba, nscal, 0, d, 0.0);
        }
        etarhoflux[lev].define(S.L.ba, 1, 0, 2, 0.0);
        scal_force[lev].define(S.L.ba, nscal, p->ppm_trace_forces ? H.ng_s : 1, -1, 0.0);
    }

    // sold ghost cells as the previous step's UpdateScal leaves them
    H.FillPatch(sold, 0, nscal, 0, H.bcs_s(), false, 0);

    // STEP 3: AdvancePremac (MacProj skipped)
    H.AdvancePremac(uold, sold, umac, w0_force_cart, utrans, vel_force);
    for (int lev = 0; lev < nlev; ++lev) {
        const Box& dom = H.S[lev].L.dom;
        if (out[lev].utrans[0])
            for (int d = 0; d < 3; ++d) gather_faces(dom, utrans[lev][d], d, 0, 1, out[lev].utrans[d]);
        if (out[lev].umac_vp[0])
            for (int d = 0; d < 3; ++d) gather_faces(dom, umac[lev][d], d, 0, 1, out[lev].umac_vp[d]);
        if (out[lev].vel_force) gather_cells(dom, vel_force[lev], 0, 3, out[lev].vel_force);
    }
    // STEP 4 (Source/MaestroAdvance.cpp:436-548)
    H.Addw0(umac, 1.0);
    H.DensityAdvance(sold, snew, sedge, sflux, scal_force, etarhoflux, umac, which_step);
    H.Addw0(umac, -1.0);
    H.Addw0(umac, 1.0);
    H.EnthalpyAdvance(sold, snew, sedge, sflux, scal_force, umac, which_step);
    H.Addw0(umac, -1.0);

    for (int lev = 0; lev < nlev; ++lev) {
        const Box& dom = H.S[lev].L.dom;
        mo_outputs& o = out[lev];
        if (o.umac_end[0])
            for (int d = 0; d < 3; ++d) gather_faces(dom, umac[lev][d], d, 0, 1, o.umac_end[d]);
        for (int d = 0; d < 3; ++d) {
            if (o.sedge[d]) gather_faces(dom, sedge[lev][d], d, 0, nscal, o.sedge[d]);
            if (o.sflux[d]) gather_faces(dom, sflux[lev][d], d, 0, nscal, o.sflux[d]);
        }
        if (o.snew) gather_cells(dom, snew[lev], 0, nscal, o.snew);
        if (tl) gather_cells(dom, snew[lev], 0, nscal, tl[lev].dsnew, true);
        if (o.sold_end) gather_cells(dom, sold[lev], 0, nscal, o.sold_end);
        if (o.etarhoflux) gather_faces(dom, etarhoflux[lev], 2, 0, 1, o.etarhoflux);
    }
    return 0;
}

// AdvancePremac for the MAC velocity (the projection skipped; its ghost faces filled as
// MacProj leaves them), then VelocityAdvance on the state's velocity.
static int run_velocity_advance(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* in,
                                const double* rhohalf, const double* sponge, double* unew_out, double* const* uedge_out,
                                double* const* umac_out) {
    if (p->dim == 2) throw std::runtime_error("VelocityAdvance: 3-D");
    Stage H;
    setup_stage(H, p, 1, &nboxes, boxes, in);
    Lev& S = H.S[0];
    const Box& dom = S.L.dom;
    const int nscal = H.nscal;
    VMF w0_force_cart(1), uold(1), sold(1), vel_force(1), rh(1), unew(1), sp(1);
    VF umac(1), utrans(1), uedge(1);
    w0_force_cart[0].define(S.L.ba, 3, 1, -1, 0.0);
    if (p->evolve_base_state)
        H.Put1dArrayOnCart(H.bs(&Lev::w0_force), w0_force_cart, false, true, &H.bcs_f(), 0, false);
    uold[0].define(S.L.ba, 3, H.ng_s, -1, 0.0);
    sold[0].define(S.L.ba, nscal, H.ng_s, -1, 0.0);
    S.gpi.define(S.L.ba, 3, 0, -1, 0.0);
    S.thermal.define(S.L.ba, 1, 1, -1, 0.0);
    scatter_cells(dom, in->uold, uold[0], 0, 3);
    scatter_cells(dom, in->sold, sold[0], 0, nscal);
    scatter_cells(dom, in->gpi, S.gpi, 0, 3);
    for (int d = 0; d < 3; ++d) umac[0][d].define(S.L.ba, 1, 1, d, 0.0);
    H.FillPatch(sold, 0, nscal, 0, H.bcs_s(), false, 0);
    H.AdvancePremac(uold, sold, umac, w0_force_cart, utrans, vel_force);
    H.SyncFaces(umac);
    for (int d = 0; d < 3; ++d)
        if (umac_out && umac_out[d]) gather_faces(dom, umac[0][d], d, 0, 1, umac_out[d]);
    H.FillPatch(uold, 0, 3, 0, H.bcs_u(), true);
    rh[0].define(S.L.ba, 1, 1, -1, 0.0);
    scatter_cells(dom, rhohalf, rh[0], 0, 1);
    if (sponge) {
        sp[0].define(S.L.ba, 1, 0, -1, 0.0);
        scatter_cells(dom, sponge, sp[0], 0, 1);
    }
    unew[0].define(S.L.ba, 3, H.ng_s, -1, 0.0);
    H.VelocityAdvance(uold, sold, rh, umac, w0_force_cart, unew, uedge, sponge ? &sp : nullptr);
    gather_cells(dom, unew[0], 0, 3, unew_out);
    for (int d = 0; d < 3; ++d)
        if (uedge_out && uedge_out[d]) gather_faces(dom, uedge[0][d], d, 0, 3, uedge_out[d]);
    return 0;
}

static int est_dt(const mo_params* p, int nlev, const int* nboxes, const int* boxes, const mo_inputs* in, double cfl,
                  int drdxfac, double* dt, double* umax) {
    if (p->dim == 2) throw std::runtime_error("EstDt: 3-D");
    Stage H;
    setup_stage(H, p, nlev, nboxes, boxes, in);
    VMF uold(nlev), sold(nlev);
    for (int lev = 0; lev < nlev; ++lev) {
        Lev& S = H.S[lev];
        const Box& dom = S.L.dom;
        uold[lev].define(S.L.ba, 3, 0, -1, 0.0);
        sold[lev].define(S.L.ba, H.nscal, 1, -1, 0.0);
        S.gpi.define(S.L.ba, 3, 0, -1, 0.0);
        scatter_cells(dom, in[lev].uold, uold[lev], 0, p->dim == 2 ? 2 : 3);
        scatter_cells(dom, in[lev].sold, sold[lev], 0, H.nscal);
        scatter_cells(dom, in[lev].gpi, S.gpi, 0, p->dim == 2 ? 2 : 3);
    }
    H.EstDt(uold, sold, cfl, drdxfac, *dt, *umax);
    return 0;
}

// The 2-D stage (AdvancePremac, DensityAdvance, EnthalpyAdvance with the Addw0 calls of
// AdvanceTimeStep) on one level; domain arrays are [nc][ny][nx].
static int run_stage_2d(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* in, mo_outputs* out,
                        int which_step) {
    if (p->ppm_trace_forces != 0) throw std::runtime_error("ppm_trace_forces = 1 is not supported");
    if (!(p->enthalpy_pred_type >= 0 && p->enthalpy_pred_type <= 2))
        throw std::runtime_error("enthalpy_pred_type must be 0, 1 or 2");
    Stage2D T;
    Lev& S = T.S;
    S.P = *p;
    S.P.phys_bc_lo[2] = S.P.phys_bc_hi[2] = interior;
    S.nspec = T.nspec = p->nspec;
    S.nscal = T.nscal = 4 + p->nspec;
    for (int d = 0; d < 2; ++d) {
        S.L.dom.lo[d] = p->dom_lo[d];
        S.L.dom.hi[d] = p->dom_hi[d];
        S.L.per[d] = (p->phys_bc_lo[d] == interior);
        if ((p->phys_bc_lo[d] == interior) != (p->phys_bc_hi[d] == interior))
            throw std::runtime_error("periodic direction needs interior on both sides");
        S.L.dx[d] = p->dx[d];
    }
    S.L.dom.lo[2] = S.L.dom.hi[2] = 0;
    S.L.per[2] = true;
    S.L.dx[2] = 1.0;
    for (int b = 0; b < nboxes; ++b) {
        Box bx;
        for (int d = 0; d < 3; ++d) {
            bx.lo[d] = d < 2 ? boxes[6 * b + d] : 0;
            bx.hi[d] = d < 2 ? boxes[6 * b + 3 + d] : 0;
        }
        S.L.ba.push_back(bx);
    }
    S.nb = T.nb = nboxes;
    S.nr = p->dom_hi[1] - p->dom_lo[1] + 1;
    S.ng_s = S.ng_adv = T.ng_s = T.ng_adv = p->ppm_type == 2 ? 4 : 3;
    S.dt = T.dt = p->dt;
    S.rel_eps = T.rel_eps = p->rel_eps;
    S.pc = PPMCtx{p->ppm_type, p->dt, p->rel_eps, {p->dx[0], p->dx[1], 1.0}, S.L.dom};
    S.BCSetup();
    S.cutoff = p->base_cutoff_density_coord;
    const int nr = S.nr;
    auto vec = [](const double* a, int n) { return std::vector<real>(a, a + n); };
    S.rho0_old = vec(in->rho0_old, nr);
    S.rho0_new = vec(in->rho0_new, nr);
    S.rhoh0_old = vec(in->rhoh0_old, nr);
    S.rhoh0_new = vec(in->rhoh0_new, nr);
    S.p0_old = vec(in->p0_old, nr);
    S.p0_new = vec(in->p0_new, nr);
    S.psi = vec(in->psi, nr);
    S.grav_cell = vec(in->grav_cell, nr);
    S.w0_force = vec(in->w0_force, nr);
    S.w0 = vec(in->w0, nr + 1);
    S.rho0_predicted_edge = vec(in->rho0_predicted_edge, nr + 1);
    const Box& dom = S.L.dom;
    const int nscal = T.nscal;

    S.w0_cart.define(S.L.ba, 2, 2, -1, 0.0);
    T.Put1dArrayOnCart(S.w0, S.w0_cart, true, true, &S.bcs_u, 0, true);
    MF w0_force_cart;
    w0_force_cart.define(S.L.ba, 2, 1, -1, 0.0);
    if (p->evolve_base_state) T.Put1dArrayOnCart(S.w0_force, w0_force_cart, false, true, &S.bcs_f, 0, false);

    MF uold, sold, snew;
    uold.define(S.L.ba, 2, T.ng_s, -1, 0.0);
    sold.define(S.L.ba, nscal, T.ng_s, -1, 0.0);
    snew.define(S.L.ba, nscal, T.ng_s, -1, 0.0);
    S.gpi.define(S.L.ba, 2, 0, -1, 0.0);
    S.thermal.define(S.L.ba, 1, 1, -1, 0.0);
    scatter_cells(dom, in->uold, uold, 0, 2);
    scatter_cells(dom, in->sold, sold, 0, nscal);
    scatter_cells(dom, in->gpi, S.gpi, 0, 2);
    if (in->thermal) scatter_cells(dom, in->thermal, S.thermal, 0, 1);
    MF umac[2], utrans[2], sedge[2], sflux[2], etarhoflux, scal_force, vel_force;
    for (int d = 0; d < 2; ++d) {
        umac[d].define(S.L.ba, 1, 1, d, 0.0);
        sedge[d].define(S.L.ba, nscal, 0, d, 0.0);
        sflux[d].define(S.L.ba, nscal, 0, d, 0.0);
    }
    etarhoflux.define(S.L.ba, 1, 0, 1, 0.0);
    scal_force.define(S.L.ba, nscal, 1, -1, 0.0);

    FillPatch(S.L, sold, 0, nscal, 0, S.bcs_s, false, 0);
    T.AdvancePremac(uold, sold, umac, w0_force_cart, utrans, vel_force);
    if (out->utrans[0])
        for (int d = 0; d < 2; ++d) gather_faces(dom, utrans[d], d, 0, 1, out->utrans[d]);
    if (out->umac_vp[0])
        for (int d = 0; d < 2; ++d) gather_faces(dom, umac[d], d, 0, 1, out->umac_vp[d]);
    if (out->vel_force) gather_cells(dom, vel_force, 0, 2, out->vel_force);
    T.Addw0(umac, 1.0);
    T.DensityAdvance(sold, snew, sedge, sflux, scal_force, etarhoflux, umac, which_step);
    T.Addw0(umac, -1.0);
    T.Addw0(umac, 1.0);
    T.EnthalpyAdvance(sold, snew, sedge, sflux, scal_force, umac, which_step);
    T.Addw0(umac, -1.0);
    if (out->umac_end[0])
        for (int d = 0; d < 2; ++d) gather_faces(dom, umac[d], d, 0, 1, out->umac_end[d]);
    for (int d = 0; d < 2; ++d) {
        if (out->sedge[d]) gather_faces(dom, sedge[d], d, 0, nscal, out->sedge[d]);
        if (out->sflux[d]) gather_faces(dom, sflux[d], d, 0, nscal, out->sflux[d]);
    }
    if (out->snew) gather_cells(dom, snew, 0, nscal, out->snew);
    if (out->sold_end) gather_cells(dom, sold, 0, nscal, out->sold_end);
    if (out->etarhoflux) gather_faces(dom, etarhoflux, 1, 0, 1, out->etarhoflux);
    return 0;
}

}  // namespace mo

#ifndef MO_TANGENT  // the FAB-based entries read and write plain doubles
static mo::Arr arr_of(const mo_fab* f) {
    mo::Arr a;
    a.p = f->p;
    for (int d = 0; d < 3; ++d) {
        a.lo[d] = f->lo[d];
        a.hi[d] = f->hi[d];
    }
    const long nx = f->hi[0] - f->lo[0] + 1, ny = f->hi[1] - f->lo[1] + 1, nz = f->hi[2] - f->lo[2] + 1;
    a.sj = nx;
    a.sk = nx * ny;
    a.sn = nx * ny * nz;
    a.nc = f->nc;
    return a;
}

// ---------------------------------------------------------------------- one member function
namespace mo {
// Argument FABs: args[slot * nboxes + b] is box b's FAB of argument `slot` (p == NULL when
// the function does not take that argument).
static Box fab_box(const mo_fab& f) {
    Box b;
    for (int d = 0; d < 3; ++d) {
        b.lo[d] = f.lo[d];
        b.hi[d] = f.hi[d];
    }
    return b;
}
static Box intersect(const Box& a, const Box& b) {
    Box r;
    for (int d = 0; d < 3; ++d) {
        r.lo[d] = std::max(a.lo[d], b.lo[d]);
        r.hi[d] = std::min(a.hi[d], b.hi[d]);
    }
    return r;
}
// an input MF from the caller's FABs: every FAB must cover the box grown by ng (in_out: the
// caller's data is copied where it exists, zero elsewhere)
static void mf_in(MF& mf, const std::vector<Box>& ba, const mo_fab* f, int nc, int ng, int ix, bool in_out = false) {
    mf.define(ba, nc, ng, ix, 0.0);
    for (int b = 0; b < mf.size(); ++b) {
        if (!f[b].p || f[b].nc < nc) throw std::runtime_error("missing argument FAB or too few components");
        const Box need = mf.fabbox(b), have = fab_box(f[b]);
        Box r = intersect(need, have);
        if (!in_out)
            for (int d = 0; d < 3; ++d)
                if (have.lo[d] > need.lo[d] || have.hi[d] < need.hi[d])
                    throw std::runtime_error("argument FAB does not cover its box and ghost cells");
        const Arr src = arr_of(&f[b]);
        for (int n = 0; n < nc; ++n) MO_FOR3(r) mf[b](i, j, k, n) = src(i, j, k, n);
    }
}
// components c0 .. c0+nc of an MF back into the caller's FABs, on the valid box grown by ng
static void mf_out(const MF& mf, const mo_fab* f, int c0, int nc, int ng) {
    for (int b = 0; b < mf.size(); ++b) {
        const Box r = intersect(grow(mf.validbox(b), std::min(ng, mf.ng)), fab_box(f[b]));
        const Arr dst = arr_of(&f[b]);
        for (int n = c0; n < c0 + nc; ++n) MO_FOR3(r) dst(i, j, k, n) = mf[b](i, j, k, n);
    }
}

static int member(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* base, int fn, int which_step,
                  int start_comp, int num_comp, int is_cons, const mo_fab* args) {
    if (which_step != 1 && which_step != 2) throw std::runtime_error("which_step must be 1 or 2");
    if (p->dim == 2) throw std::runtime_error("mo_member is 3-D");
    Stage H;
    setup_stage(H, p, 1, &nboxes, boxes, base);
    Lev& S = H.S[0];
    const std::vector<Box>& ba = S.L.ba;
    const int nscal = H.nscal, ng_s = H.ng_s, nga = H.ng_adv;
    auto A = [&](int slot) { return args + (long)slot * nboxes; };
    VMF m1(1), m2(1), m3(1), m4(1);
    VF f1(1), f2(1), f3(1);
    switch (fn) {
        case MO_MAKE_UTRANS: {  // Maestro::MakeUtrans (Source/MaestroMakeUtrans.cpp:6-648)
            mf_in(m1[0], ba, A(MO_UTILDE), 3, nga, -1);
            mf_in(m2[0], ba, A(MO_UFULL), 3, nga, -1);
            for (int d = 0; d < 3; ++d) f1[0][d].define(ba, 1, 1, d, 0.0);
            H.MakeUtrans(m1, m2, f1);
            for (int d = 0; d < 3; ++d) mf_out(f1[0][d], A(MO_UTRANS0 + d), 0, 1, 1);
            break;
        }
        case MO_VEL_PRED: {  // Maestro::VelPred (Source/MaestroVelPred.cpp:5-292)
            mf_in(m1[0], ba, A(MO_UTILDE), 3, nga, -1);
            mf_in(m2[0], ba, A(MO_UFULL), 3, nga, -1);
            mf_in(m3[0], ba, A(MO_FORCE), 3, p->ppm_trace_forces ? ng_s : 1, -1);
            for (int d = 0; d < 3; ++d) {
                mf_in(f1[0][d], ba, A(MO_UTRANS0 + d), 1, 1, d);
                f2[0][d].define(ba, 1, 1, d, 0.0);
            }
            H.VelPred(m1, m2, f1, f2, m3);
            for (int d = 0; d < 3; ++d) mf_out(f2[0][d], A(MO_UMAC0 + d), 0, 1, 0);
            break;
        }
        case MO_MAKE_EDGE_SCAL: {  // Maestro::MakeEdgeScal (Source/MaestroMakeEdgeScalars.cpp:6-302)
            if (start_comp < 0 || num_comp < 1 || start_comp + num_comp > nscal)
                throw std::runtime_error("component range outside the state");
            mf_in(m1[0], ba, A(MO_STATE), nscal, ng_s, -1);
            mf_in(m2[0], ba, A(MO_FORCE), nscal, p->ppm_trace_forces ? ng_s : 1, -1);
            for (int d = 0; d < 3; ++d) {
                mf_in(f1[0][d], ba, A(MO_UMAC0 + d), 1, 1, d);
                f2[0][d].define(ba, nscal, 0, d, 0.0);
            }
            H.MakeEdgeScal(m1, f2, f1, m2, H.bcs_s(), start_comp, start_comp, num_comp, is_cons != 0);
            for (int d = 0; d < 3; ++d) mf_out(f2[0][d], A(MO_SEDGE0 + d), start_comp, num_comp, 0);
            break;
        }
        case MO_MAKE_S0MAC: {  // Maestro::MakeS0mac of rho0_old (Source/MaestroFill3dData.cpp:712-1188)
            if (!p->spherical) throw std::runtime_error("MakeS0mac is spherical-only");
            H.MakeS0mac(H.bs(&Lev::rho0_old), f1);
            for (int d = 0; d < 3; ++d) mf_out(f1[0][d], A(MO_UMAC0 + d), 0, 1, 1);
            break;
        }
        case MO_MAKE_RHOX_FLUX:    // Maestro::MakeRhoXFlux (Source/MaestroMakeFlux.cpp:18-465)
        case MO_MAKE_RHOH_FLUX: {  // Maestro::MakeRhoHFlux (Source/MaestroMakeFlux.cpp:467-1067)
            const bool x = fn == MO_MAKE_RHOX_FLUX;
            for (int d = 0; d < 3; ++d) {
                mf_in(f1[0][d], ba, A(MO_SEDGE0 + d), nscal, 0, d);
                mf_in(f2[0][d], ba, A(MO_UMAC0 + d), 1, 0, d);
                f3[0][d].define(ba, nscal, 0, d, 0.0);
            }
            const BS s0o = H.bs(x ? &Lev::rho0_old : &Lev::rhoh0_old);
            const BS s0n = which_step == 1 ? s0o : H.bs(x ? &Lev::rho0_new : &Lev::rhoh0_new);
            BS s0eo(1), s0en(1);
            if (!p->spherical) {
                H.CelltoEdge(s0o, s0eo);
                H.CelltoEdge(s0n, s0en);
            }
            if (x) {
                if (start_comp != FirstSpec || num_comp != H.nspec)
                    throw std::runtime_error("MakeRhoXFlux: the species FirstSpec .. FirstSpec+NumSpec-1");
                if (A(MO_ETA)[0].p) mf_in(m1[0], ba, A(MO_ETA), 1, 0, 2);
                else m1[0].define(ba, 1, 0, 2, 0.0);
                H.MakeRhoXFlux(f3, m1, f1, f2, s0o, s0eo, s0n, s0en, start_comp, num_comp);
                for (int d = 0; d < 3; ++d) {
                    mf_out(f3[0][d], A(MO_SFLUX0 + d), Rho, 1, 0);
                    mf_out(f3[0][d], A(MO_SFLUX0 + d), FirstSpec, H.nspec, 0);
                }
                if (A(MO_ETA)[0].p) mf_out(m1[0], A(MO_ETA), 0, 1, 0);
            } else {
                H.MakeRhoHFlux(f3, f1, f2, s0o, s0eo, s0n, s0en);
                for (int d = 0; d < 3; ++d) mf_out(f3[0][d], A(MO_SFLUX0 + d), RhoH, 1, 0);
            }
            break;
        }
        case MO_UPDATE_SCAL: {  // Maestro::UpdateScal (Source/MaestroAdvection.cpp:86-297)
            if (!((start_comp == RhoH && num_comp == 1) || (start_comp == FirstSpec && num_comp == H.nspec)))
                throw std::runtime_error("UpdateScal: RhoH, or the species");
            mf_in(m1[0], ba, A(MO_STATE), nscal, 0, -1);
            mf_in(m2[0], ba, A(MO_SNEW), nscal, ng_s, -1, true);
            mf_in(m3[0], ba, A(MO_FORCE), nscal, 0, -1);
            for (int d = 0; d < 3; ++d) mf_in(f1[0][d], ba, A(MO_SFLUX0 + d), nscal, 0, d);
            H.UpdateScal(m1, m2, f1, m3, start_comp, num_comp);
            mf_out(m2[0], A(MO_SNEW), start_comp, num_comp, ng_s);
            if (start_comp == FirstSpec) mf_out(m2[0], A(MO_SNEW), Rho, 1, ng_s);
            break;
        }
        default:
            throw std::runtime_error("unknown member function");
    }
    return 0;
}

}  // namespace mo
#endif

extern "C" {

int mo_run_stage_levels(const mo_params* p, int nlev, const int* nboxes, const int* boxes, const mo_inputs* in,
                        mo_outputs* out, int which_step, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    try {
        return mo::run_stage(p, nlev, nboxes, boxes, in, out, which_step);
    } catch (const std::exception& e) {
        mo::g_err = e.what();
        return -1;
    }
}

int mo_run_stage_2d(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* in, mo_outputs* out,
                    int which_step, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    try {
        return mo::run_stage_2d(p, nboxes, boxes, in, out, which_step);
    } catch (const std::exception& e) {
        mo::g_err = e.what();
        return -1;
    }
}

int mo_run_stage(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* in, mo_outputs* out,
                 int nthreads) {
    return mo_run_stage_levels(p, 1, &nboxes, boxes, in, out, 1, nthreads);
}

int mo_run_velocity_advance(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* in,
                            const double* rhohalf, const double* sponge, double* unew, double* const* uedge,
                            double* const* umac, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    try {
        return mo::run_velocity_advance(p, nboxes, boxes, in, rhohalf, sponge, unew, uedge, umac);
    } catch (const std::exception& e) {
        mo::g_err = e.what();
        return -1;
    }
}

int mo_est_dt(const mo_params* p, int nlev, const int* nboxes, const int* boxes, const mo_inputs* in, double cfl,
              int drdxfac, double* dt, double* umax) {
    try {
        return mo::est_dt(p, nlev, nboxes, boxes, in, cfl, drdxfac, dt, umax);
    } catch (const std::exception& e) {
        mo::g_err = e.what();
        return -1;
    }
}

int mo_cell_to_edge(const double* s0_cell, int nr, double* s0_edge) {
    std::vector<mo::real> c(s0_cell, s0_cell + nr), e;
    mo::Lev::CelltoEdge(c, e);
    for (int r = 0; r <= nr; ++r) s0_edge[r] = mo::value_of(e[r]);
    return 0;
}


#ifndef MO_TANGENT
int mo_ppm(const mo_params* p, const int* bx, const mo_fab* s, int comp, const mo_fab* u, const mo_fab* v,
           const mo_fab* w, int is_umac, const int* bc, const mo_fab* Ip, const mo_fab* Im) {
    try {
        mo::Box dom, b;
        for (int d = 0; d < 3; ++d) {
            dom.lo[d] = p->dom_lo[d];
            dom.hi[d] = p->dom_hi[d];
            b.lo[d] = bx[d];
            b.hi[d] = bx[3 + d];
        }
        mo::PPMCtx pc{p->ppm_type, p->dt, p->rel_eps, {p->dx[0], p->dx[1], p->dx[2]}, dom};
        mo::BCRec r;
        for (int d = 0; d < 3; ++d) {
            r.lo[d] = bc[d];
            r.hi[d] = bc[3 + d];
        }
        mo::PPM(pc, b, arr_of(s), arr_of(u), arr_of(v), arr_of(w), arr_of(Ip), arr_of(Im), r, is_umac != 0, comp);
        return 0;
    } catch (const std::exception& e) {
        mo::g_err = e.what();
        return -1;
    }
}

int mo_slopes(int slope_order, int d, const int* dom, const int* bx, const mo_fab* s, int ncomp, const int* bcs,
              const mo_fab* slope) {
    try {
        mo::Box D, b;
        for (int e = 0; e < 3; ++e) {
            D.lo[e] = dom[e];
            D.hi[e] = dom[3 + e];
            b.lo[e] = bx[e];
            b.hi[e] = bx[3 + e];
        }
        std::vector<mo::BCRec> r(ncomp);
        for (int n = 0; n < ncomp; ++n)
            for (int e = 0; e < 3; ++e) {
                r[n].lo[e] = bcs[6 * n + e];
                r[n].hi[e] = bcs[6 * n + 3 + e];
            }
        mo::Slope_dir(slope_order, D, b, arr_of(s), arr_of(slope), ncomp, r, 0, d);
        return 0;
    } catch (const std::exception& e) {
        mo::g_err = e.what();
        return -1;
    }
}

int mo_member(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* base, int fn, int which_step,
              int start_comp, int num_comp, int is_conservative, const mo_fab* args) {
    try {
        return mo::member(p, nboxes, boxes, base, fn, which_step, start_comp, num_comp, is_conservative, args);
    } catch (const std::exception& e) {
        mo::g_err = e.what();
        return -1;
    }
}

#else
int mo_run_stage_tl(const mo_params* p, int nboxes, const int* boxes, const mo_inputs* in, const double* duold,
                    const double* dsold, mo_outputs* out, double* dsnew, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    try {
        const mo::TangentIO t{duold, dsold, dsnew};
        return mo::run_stage(p, 1, &nboxes, boxes, in, out, 1, &t);
    } catch (const std::exception& e) {
        mo::g_err = e.what();
        return -1;
    }
}
#endif

const char* mo_last_error(void) { return mo::g_err.c_str(); }
}
