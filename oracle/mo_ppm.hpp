// Test infrastructure only (oracle): PPM and limited slopes, restated from
// Source/MaestroPPM.cpp and Source/MaestroSlopes.cpp.
//
// The reference writes the x, y and z sweeps out three times.  A token-level diff of the
// three copies shows they are the same algorithm with these differences, which the
// restatement keeps as direction flags:
//   * ppm_type 2, lo-side re-limit of cells domlo+1/domlo+2, bigm branch: x tests
//     `>= 1.e10` (Source/MaestroPPM.cpp:566), y and z test `>= 1.e-10`.
//   * ppm_type 2, y only: at j == domlo also sets sedge = s(j-1) (:1192; no effect on
//     the outputs because that cell skips the re-limit).
//   * ppm_type 2, y and z: in the domhi-1 branch also set sedgerr = s(+2)
//     (:1343, :2087); x keeps the interpolated value.
//   * slope_order 4 at ext_dir/hoextrap boundaries: x uses the centred `dlim`
//     where y and z use the one-sided `slim` (Source/MaestroSlopes.cpp:142,156,178,192).
#pragma once
#include "mo_types.hpp"

namespace mo {

struct PPMCtx {
    int ppm_type;
    double dt, rel_eps;
    double dx[3];
    Box dom;
};

// One direction d of Maestro::PPM (Source/MaestroPPM.cpp:33-252 ppm1 x, 254-771 ppm2 x;
// y 779-1513; z 1522-2260).  s(.., n) is the traced field, u the velocity used for the
// characteristic tracing in direction d (face velocity if is_umac, else cell velocity).
inline void PPM_dir(const PPMCtx& c, const Box& bx, const Arr& s, int n, const Arr& u, const Arr& Ip,
                    const Arr& Im, int d, int bclo, int bchi, bool is_umac) {
    const int di = d == 0, dj = d == 1, dk = d == 2;
    const int domlo = c.dom.lo[d], domhi = c.dom.hi[d];
    const real dt_local = c.dt, rel_eps_local = c.rel_eps, dxd = c.dx[d];
    const real C = 1.25;
    const bool lo_bigm_quirk = (d == 0);       // 1.e10 in the x lo re-limit
    const bool hi_sedgerr_reset = (d != 0);    // y/z reset sedgerr at domhi-1
    const bool lo_sedge_reset = (d == 1);      // y resets sedge at domlo
    const bool lo_ext = (bclo == ext_dir || bclo == hoextrap);
    const bool hi_ext = (bchi == ext_dir || bchi == hoextrap);

    MO_FOR3(bx) {
        const int I = d == 0 ? i : (d == 1 ? j : k);
        auto S = [&](int m) -> real { return s(i + m * di, j + m * dj, k + m * dk, n); };
        real sm, sp;
        if (c.ppm_type == 1) {
            // van Leer slopes (:37-73)
            real dsvl_l = 0.0, dsvl_r = 0.0;
            real dsc = 0.5 * (S(0) - S(-2));
            real dsl = 2.0 * (S(-1) - S(-2));
            real dsr = 2.0 * (S(0) - S(-1));
            if (dsl * dsr > 0.0) dsvl_l = cps(1.0, dsc) * mn(fab(dsc), mn(fab(dsl), fab(dsr)));
            dsc = 0.5 * (S(1) - S(-1));
            dsl = 2.0 * (S(0) - S(-1));
            dsr = 2.0 * (S(1) - S(0));
            if (dsl * dsr > 0.0) dsvl_r = cps(1.0, dsc) * mn(fab(dsc), mn(fab(dsl), fab(dsr)));
            sm = 0.5 * (S(0) + S(-1)) - (dsvl_r - dsvl_l) / 6.0;
            sm = mx(sm, mn(S(0), S(-1)));
            sm = mn(sm, mx(S(0), S(-1)));
            // sp (:80-111)
            dsvl_l = 0.0;
            dsvl_r = 0.0;
            dsc = 0.5 * (S(1) - S(-1));
            dsl = 2.0 * (S(0) - S(-1));
            dsr = 2.0 * (S(1) - S(0));
            if (dsl * dsr > 0.0) dsvl_l = cps(1.0, dsc) * mn(fab(dsc), mn(fab(dsl), fab(dsr)));
            dsc = 0.5 * (S(2) - S(0));
            dsl = 2.0 * (S(1) - S(0));
            dsr = 2.0 * (S(2) - S(1));
            if (dsl * dsr > 0.0) dsvl_r = cps(1.0, dsc) * mn(fab(dsc), mn(fab(dsl), fab(dsr)));
            sp = 0.5 * (S(1) + S(0)) - (dsvl_r - dsvl_l) / 6.0;
            sp = mx(sp, mn(S(1), S(0)));
            sp = mn(sp, mx(S(1), S(0)));
            const real sedgel = sp, sedger = sm;
            auto quadlim = [&]() {  // (:117-128)
                if ((sp - S(0)) * (S(0) - sm) <= 0.0) {
                    sp = S(0);
                    sm = S(0);
                } else if (fab(sp - S(0)) >= 2.0 * fab(sm - S(0))) {
                    sp = 3.0 * S(0) - 2.0 * sm;
                } else if (fab(sm - S(0)) >= 2.0 * fab(sp - S(0))) {
                    sm = 3.0 * S(0) - 2.0 * sp;
                }
            };
            quadlim();
            // boundary stencils (:131-205)
            if (I == domlo) {
                if (lo_ext) {
                    sm = S(-1);
                    sp = -0.2 * S(-1) + 0.75 * S(0) + 0.5 * S(1) - 0.05 * S(2);
                    sp = mx(sp, mn(S(1), S(0)));
                    sp = mn(sp, mx(S(1), S(0)));
                }
            } else if (I == domlo + 1) {
                if (lo_ext) {
                    sm = -0.2 * S(-2) + 0.75 * S(-1) + 0.5 * S(0) - 0.05 * S(1);
                    sm = mx(sm, mn(S(0), S(-1)));
                    sm = mn(sm, mx(S(0), S(-1)));
                    sp = sedgel;
                    quadlim();
                }
            } else if (I == domhi) {
                if (hi_ext) {
                    sp = S(1);
                    sm = -0.2 * S(1) + 0.75 * S(0) + 0.5 * S(-1) - 0.05 * S(-2);
                    sm = mx(sm, mn(S(-1), S(0)));
                    sm = mn(sm, mx(S(-1), S(0)));
                }
            } else if (I == domhi - 1) {
                if (hi_ext) {
                    sp = -0.2 * S(2) + 0.75 * S(1) + 0.5 * S(0) - 0.05 * S(-1);
                    sp = mx(sp, mn(S(0), S(1)));
                    sp = mn(sp, mx(S(0), S(1)));
                    sm = sedger;
                    quadlim();
                }
            }
        } else {
            // ppm_type 2 (:255-640): limited 4th-order face values around the cell
            auto face = [&](int m) -> real {  // face between cells m-1 and m
                real se = (7.0 / 12.0) * (S(m - 1) + S(m)) - (1.0 / 12.0) * (S(m - 2) + S(m + 1));
                if ((se - S(m - 1)) * (S(m) - se) < 0.0) {
                    real D2 = 3.0 * (S(m - 1) - 2.0 * se + S(m));
                    real D2L = S(m - 2) - 2.0 * S(m - 1) + S(m);
                    real D2R = S(m - 1) - 2.0 * S(m) + S(m + 1);
                    real sgn = cps(1.0, D2);
                    real D2LIM = sgn * mx(mn(C * sgn * D2L, mn(C * sgn * D2R, sgn * D2)), 0.0);
                    se = 0.5 * (S(m - 1) + S(m)) - D2LIM / 6.0;
                }
                return se;
            };
            real sedgel = face(-1);
            real sedge = face(0);
            real sedger = face(1);
            real sedgerr = face(2);
            real alphap, alpham;
            bool bigp, bigm, extremum;
            // Colella 2008 limiter (:337-434); bigm_tol differs only in the x lo re-limit
            auto limiter = [&](real bigm_tol) {
                alphap = sedger - S(0);
                alpham = sedge - S(0);
                bigp = fab(alphap) > 2.0 * fab(alpham);
                bigm = fab(alpham) > 2.0 * fab(alphap);
                extremum = false;
                if (alpham * alphap >= 0.0) {
                    extremum = true;
                } else if (bigp || bigm) {
                    real dafacem = sedge - sedgel;
                    real dafacep = sedgerr - sedger;
                    real dabarm = S(0) - S(-1);
                    real dabarp = S(1) - S(0);
                    real dafacemin = mn(fab(dafacem), fab(dafacep));
                    real dabarmin = mn(fab(dabarm), fab(dabarp));
                    real dachkm = 0.0, dachkp = 0.0;
                    if (dafacemin >= dabarmin) {
                        dachkm = dafacem;
                        dachkp = dafacep;
                    } else {
                        dachkm = dabarm;
                        dachkp = dabarp;
                    }
                    extremum = (dachkm * dachkp <= 0.0);
                }
                if (extremum) {
                    real D2 = 6.0 * (alpham + alphap);
                    real D2L = S(-2) - 2.0 * S(-1) + S(0);
                    real D2R = S(0) - 2.0 * S(1) + S(2);
                    real D2C = S(-1) - 2.0 * S(0) + S(1);
                    real sgn = cps(1.0, D2);
                    real D2LIM = mx(mn(sgn * D2, mn(C * sgn * D2L, mn(C * sgn * D2R, C * sgn * D2C))), 0.0);
                    real D2ABS = mx(fab(D2), 1.e-10);
                    alpham = alpham * D2LIM / D2ABS;
                    alphap = alphap * D2LIM / D2ABS;
                } else {
                    if (bigp) {
                        real sgn = cps(1.0, alpham);
                        real amax = -alphap * alphap / (4.0 * (alpham + alphap));
                        real delam = S(-1) - S(0);
                        if (sgn * amax >= sgn * delam) {
                            if (sgn * (delam - alpham) >= 1.e-10) {
                                alphap = -2.0 * delam - 2.0 * sgn * sqrt_r(delam * delam - delam * alpham);
                            } else {
                                alphap = -2.0 * alpham;
                            }
                        }
                    }
                    if (bigm) {
                        real sgn = cps(1.0, alphap);
                        real amax = -alpham * alpham / (4.0 * (alpham + alphap));
                        real delap = S(1) - S(0);
                        if (sgn * amax >= sgn * delap) {
                            if (sgn * (delap - alphap) >= bigm_tol) {
                                alpham = (-2.0 * delap - 2.0 * sgn * sqrt_r(delap * delap - delap * alphap));
                            } else {
                                alpham = -2.0 * alphap;
                            }
                        }
                    }
                }
                sm = S(0) + alpham;
                sp = S(0) + alphap;
            };
            limiter(1.e-10);
            if (lo_ext) {  // (:443-570)
                if (I == domlo) {
                    sm = S(-1);
                    if (lo_sedge_reset) sedge = S(-1);
                    sp = -0.2 * S(-1) + 0.75 * S(0) + 0.5 * S(1) - 0.05 * S(2);
                    sp = mx(sp, mn(S(1), S(0)));
                    sp = mn(sp, mx(S(1), S(0)));
                } else if (I == domlo + 1) {
                    sedgel = S(-2);
                    sedge = -0.2 * S(-2) + 0.75 * S(-1) + 0.5 * S(0) - 0.05 * S(1);
                    sedge = mx(sedge, mn(S(0), S(-1)));
                    sedge = mn(sedge, mx(S(0), S(-1)));
                } else if (I == domlo + 2) {
                    sedgel = -0.2 * S(-3) + 0.75 * S(-2) + 0.5 * S(-1) - 0.05 * S(0);
                    sedgel = mx(sedgel, mn(S(-1), S(-2)));
                    sedgel = mn(sedgel, mx(S(-1), S(-2)));
                }
                if (I == domlo + 1 || I == domlo + 2) limiter(lo_bigm_quirk ? 1.e10 : 1.e-10);
            }
            if (hi_ext) {  // (:572-700)
                if (I == domhi) {
                    sp = S(1);
                    sm = -0.2 * S(1) + 0.75 * S(0) + 0.5 * S(-1) - 0.05 * S(-2);
                    sm = mx(sm, mn(S(-1), S(0)));
                    sm = mn(sm, mx(S(-1), S(0)));
                } else if (I == domhi - 1) {
                    if (hi_sedgerr_reset) sedgerr = S(2);
                    sedger = -0.2 * S(2) + 0.75 * S(1) + 0.5 * S(0) - 0.05 * S(-1);
                    sedger = mx(sedger, mn(S(0), S(1)));
                    sedger = mn(sedger, mx(S(0), S(1)));
                } else if (I == domhi - 2) {
                    sedgerr = -0.2 * S(3) + 0.75 * S(2) + 0.5 * S(1) - 0.05 * S(0);
                    sedgerr = mx(sedgerr, mn(S(1), S(2)));
                    sedgerr = mn(sedgerr, mx(S(1), S(2)));
                }
                if (I == domhi - 1 || I == domhi - 2) limiter(1.e-10);
            }
        }
        // characteristic tracing (:209-251, :706-770)
        real s6 = 6.0 * S(0) - 3.0 * (sm + sp);
        const int ii = i + di, jj = j + dj, kk = k + dk;
        real up = is_umac ? u(ii, jj, kk) : u(i, j, k);
        real sigma = fab(up) * dt_local / dxd;
        if (up > rel_eps_local) {
            Ip(i, j, k, d) = sp - 0.5 * sigma * (sp - sm - (1.0 - 2.0 / 3.0 * sigma) * s6);
        } else {
            Ip(i, j, k, d) = S(0);
        }
        real um = u(i, j, k);
        sigma = fab(um) * dt_local / dxd;
        if (um < -rel_eps_local) {
            Im(i, j, k, d) = sm + 0.5 * sigma * (sp - sm + (1.0 - 2.0 / 3.0 * sigma) * s6);
        } else {
            Im(i, j, k, d) = S(0);
        }
    }
}

// Maestro::PPM (Source/MaestroPPM.cpp:5-2262): all three directions for component n.
inline void PPM(const PPMCtx& c, const Box& bx, const Arr& s, const Arr& u, const Arr& v, const Arr& w,
                const Arr& Ip, const Arr& Im, const BCRec& bc, bool is_umac, int n) {
    PPM_dir(c, bx, s, n, u, Ip, Im, 0, bc.lo[0], bc.hi[0], is_umac);
    PPM_dir(c, bx, s, n, v, Ip, Im, 1, bc.lo[1], bc.hi[1], is_umac);
    PPM_dir(c, bx, s, n, w, Ip, Im, 2, bc.lo[2], bc.hi[2], is_umac);
}

// Maestro::Slopex/y/z (Source/MaestroSlopes.cpp:6-600) for direction d, components
// 0..ncomp-1 of s into slope comps 0..ncomp-1; bcs[bc_start + n].
inline void Slope_dir(int slope_order, const Box& dom, const Box& bx, const Arr& s, const Arr& slope,
                      int ncomp, const std::vector<BCRec>& bcs, int bc_start, int d) {
    const int di = d == 0, dj = d == 1, dk = d == 2;
    const int ilo = dom.lo[d], ihi = dom.hi[d];
    const bool x_dlim_quirk = (d == 0);
    for (int n = 0; n < ncomp; ++n) {
        const int bclo = bcs[bc_start + n].lo[d], bchi = bcs[bc_start + n].hi[d];
        const bool lo_ext = (bclo == ext_dir || bclo == hoextrap);
        const bool hi_ext = (bchi == ext_dir || bchi == hoextrap);
        MO_FOR3(bx) {
            const int I = d == 0 ? i : (d == 1 ? j : k);
            auto S = [&](int m) -> real { return s(i + m * di, j + m * dj, k + m * dk, n); };
            real& out = slope(i, j, k, n);
            if (slope_order == 0) {
                out = 0.0;
            } else if (slope_order == 2) {
                real del = 0.5 * (S(1) - S(-1));
                real dpls = 2.0 * (S(1) - S(0));
                real dmin = 2.0 * (S(0) - S(-1));
                real slim = mn(fab(dpls), fab(dmin));
                slim = dpls * dmin > 0.0 ? slim : 0.0;
                real sflag = cps(1.0, del);
                out = sflag * mn(slim, fab(del));
                if (lo_ext) {
                    if (I == ilo - 1) {
                        out = 0.0;
                    } else if (I == ilo) {
                        del = (S(1) + 3.0 * S(0) - 4.0 * S(-1)) / 3.0;
                        dpls = 2.0 * (S(1) - S(0));
                        dmin = 2.0 * (S(0) - S(-1));
                        slim = mn(fab(dpls), fab(dmin));
                        slim = dpls * dmin > 0.0 ? slim : 0.0;
                        sflag = cps(1.0, del);
                        out = sflag * mn(slim, fab(del));
                    }
                }
                if (hi_ext) {
                    if (I == ihi + 1) {
                        out = 0.0;
                    } else if (I == ihi) {
                        del = -(S(-1) + 3.0 * S(0) - 4.0 * S(1)) / 3.0;
                        dpls = 2.0 * (S(0) - S(-1));
                        dmin = 2.0 * (S(1) - S(0));
                        slim = mn(fab(dpls), fab(dmin));
                        slim = dpls * dmin > 0.0 ? slim : 0.0;
                        sflag = cps(1.0, del);
                        out = sflag * mn(slim, fab(del));
                    }
                }
            } else if (slope_order == 4) {
                real dcen = 0.5 * (S(0) - S(-2));
                real dmin = 2.0 * (S(-1) - S(-2));
                real dpls = 2.0 * (S(0) - S(-1));
                real dlim = mn(fab(dmin), fab(dpls));
                dlim = dpls * dmin > 0.0 ? dlim : 0.0;
                real dflag = cps(1.0, dcen);
                real dxl = dflag * mn(dlim, fab(dcen));
                dcen = 0.5 * (S(2) - S(0));
                dmin = 2.0 * (S(1) - S(0));
                dpls = 2.0 * (S(2) - S(1));
                dlim = mn(fab(dmin), fab(dpls));
                dlim = dpls * dmin > 0.0 ? dlim : 0.0;
                dflag = cps(1.0, dcen);
                real dxr = dflag * mn(dlim, fab(dcen));
                dcen = 0.5 * (S(1) - S(-1));
                dmin = 2.0 * (S(0) - S(-1));
                dpls = 2.0 * (S(1) - S(0));
                dlim = mn(fab(dmin), fab(dpls));
                dlim = dpls * dmin > 0.0 ? dlim : 0.0;
                dflag = cps(1.0, dcen);
                real ds = 4.0 / 3.0 * dcen - (dxr + dxl) / 6.0;
                out = dflag * mn(fab(ds), dlim);
                if (lo_ext) {
                    if (I == ilo - 1) {
                        out = 0.0;
                    } else if (I == ilo) {
                        real del = -16.0 / 15.0 * S(-1) + 0.5 * S(0) + 2.0 / 3.0 * S(1) - 0.1 * S(2);
                        dmin = 2.0 * (S(0) - S(-1));
                        dpls = 2.0 * (S(1) - S(0));
                        real slim = mn(fab(dpls), fab(dmin));
                        slim = dpls * dmin > 0.0 ? (x_dlim_quirk ? dlim : slim) : 0.0;
                        real sflag = cps(1.0, del);
                        out = sflag * mn(slim, fab(del));
                    } else if (I == ilo + 1) {
                        real del = -16.0 / 15.0 * S(-2) + 0.5 * S(-1) + 2.0 / 3.0 * S(0) - 0.1 * S(1);
                        dmin = 2.0 * (S(-1) - S(-2));
                        dpls = 2.0 * (S(0) - S(-1));
                        real slim = mn(fab(dpls), fab(dmin));
                        slim = dpls * dmin > 0.0 ? (x_dlim_quirk ? dlim : slim) : 0.0;
                        real sflag = cps(1.0, del);
                        dxl = sflag * mn(slim, fab(del));
                        ds = 4.0 / 3.0 * dcen - (dxr + dxl) / 6.0;
                        out = dflag * mn(fab(ds), dlim);
                    }
                }
                if (hi_ext) {
                    if (I == ihi + 1) {
                        out = 0.0;
                    } else if (I == ihi) {
                        real del = -(-16.0 / 15.0 * S(1) + 0.5 * S(0) + 2.0 / 3.0 * S(-1) - 0.1 * S(-2));
                        dmin = 2.0 * (S(0) - S(-1));
                        dpls = 2.0 * (S(1) - S(0));
                        real slim = mn(fab(dpls), fab(dmin));
                        slim = dpls * dmin > 0.0 ? (x_dlim_quirk ? dlim : slim) : 0.0;
                        real sflag = cps(1.0, del);
                        out = sflag * mn(slim, fab(del));
                    } else if (I == ihi - 1) {
                        real del = -(-16.0 / 15.0 * S(2) + 0.5 * S(1) + 2.0 / 3.0 * S(0) - 0.1 * S(-1));
                        dmin = 2.0 * (S(1) - S(0));
                        dpls = 2.0 * (S(2) - S(1));
                        real slim = mn(fab(dpls), fab(dmin));
                        slim = dpls * dmin > 0.0 ? (x_dlim_quirk ? dlim : slim) : 0.0;
                        real sflag = cps(1.0, del);
                        dxr = sflag * mn(slim, fab(del));
                        ds = 4.0 / 3.0 * dcen - (dxl + dxr) / 6.0;
                        out = dflag * mn(fab(ds), dlim);
                    }
                }
            }
        }
    }
}

}  // namespace mo
