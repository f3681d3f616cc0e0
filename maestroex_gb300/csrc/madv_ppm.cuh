// Per-element PPM arithmetic shared by the level kernels (madv_kernels.cu) and the
// single-box entry points (madv_box.cu).  Source: Maestro::PPM,
// Source/MaestroPPM.cpp (ppm_type 1 x-sweep :33-252, ppm_type 2 x-sweep :254-771; the y and
// z sweeps :779-2260 are the same algorithm with the differences kept as flags below).
#pragma once
#include "madv_core.cuh"
#include "madv_exact.cuh"

namespace madv {

// S(m): the field at cell (index + m) along direction D.
#define SHIFT_S(s, sc) [&](int m) -> double { return at(s, i + m * di, j + m * dj, k + m * dk, sc); }

// Van Leer slope of cell (i,j,k) along D (Source/MaestroPPM.cpp:37-73).
template <int D>
__device__ __forceinline__ double ppm_dsvl(const FabView& s, int sc, int i, int j, int k) {
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    auto S = SHIFT_S(s, sc);
    const double dsc = half(S(1) - S(-1));
    const double dsl = twice(S(0) - S(-1));
    const double dsr = twice(S(1) - S(0));
    // reference: if (dsl*dsr > 0) dsvl = copysign(1,dsc) * min(|dsc|, min(|dsl|, |dsr|)).
    // The minimum of non-negative (finite) doubles is the minimum of their bit patterns, and
    // copysign(1, dsc) * m with m >= 0 is m with the sign of dsc.
    if (!prod_gt0(dsl, dsr)) return 0.0;
    long long m = dbits(dsc) & ABS_MASK;
    m = min(m, dbits(dsl) & ABS_MASK);
    m = min(m, dbits(dsr) & ABS_MASK);
    return __longlong_as_double(m | (dbits(dsc) & SIGN_BIT));
}

// Interior fourth-order limited face value (ppm_type 2), face between cells c+m-1 and c+m.
template <int D>
__device__ __forceinline__ double ppm2_face_regular(const FabView& s, int sc, int i, int j, int k, int m,
                                                    const RecipC& r6) {
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    auto S = SHIFT_S(s, sc);
    const double C = 1.25;
    double se = (7.0 / 12.0) * (S(m - 1) + S(m)) - (1.0 / 12.0) * (S(m - 2) + S(m + 1));
    // reference: (se - s(m-1)) * (s(m) - se) < 0, i.e. the product of (se - s(m-1)) and
    // -(s(m) - se) = se - s(m) (exact) is positive
    if (prod_gt0(se - S(m - 1), se - S(m))) {
        double D2 = 3.0 * (S(m - 1) - 2.0 * se + S(m));
        double D2L = S(m - 2) - 2.0 * S(m - 1) + S(m);
        double D2R = S(m - 1) - 2.0 * S(m) + S(m + 1);
        double sgn = copysign(1.0, D2);
        double D2LIM = sgn * mx(mn(C * sgn * D2L, mn(C * sgn * D2R, sgn * D2)), 0.0);
        se = half(S(m - 1) + S(m)) - div_c(D2LIM, r6);
    }
    return se;
}

// Limited interface value of the face (i,j,k) between cells f-1 and f along D
// (ppm_type 1 :37-111, ppm_type 2 :257-335; the boundary stencils of :131-205 / :443-700
// are the values the reference assigns to the faces next to an ext_dir/hoextrap
// boundary).  dv: van Leer slopes per cell (ppm_type 1).
template <int D, int PPMT>
__device__ __forceinline__ double ppm_face_value(const FabView& s, int sc, const FabView& dv, int i, int j, int k,
                                                 int lo_ext, int hi_ext, int domlo, int domhi, const RecipC& r6) {
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    auto S = SHIFT_S(s, sc);
    const int I = D == 0 ? i : (D == 1 ? j : k);
    double v;
    if (lo_ext && I == domlo) {
        v = S(-1);
    } else if (hi_ext && I == domhi + 1) {
        v = S(0);
    } else if (lo_ext && I == domlo + 1) {
        v = -0.2 * S(-2) + 0.75 * S(-1) + 0.5 * S(0) - 0.05 * S(1);
        v = mx(v, mn(S(0), S(-1)));
        v = mn(v, mx(S(0), S(-1)));
    } else if (hi_ext && I == domhi) {
        v = -0.2 * S(1) + 0.75 * S(0) + 0.5 * S(-1) - 0.05 * S(-2);
        v = mx(v, mn(S(-1), S(0)));
        v = mn(v, mx(S(-1), S(0)));
    } else if (PPMT == 1) {
        const double dvl = at(dv, i - di, j - dj, k - dk);
        const double dvr = at(dv, i, j, k);
        v = half(S(0) + S(-1)) - div_c(dvr - dvl, r6);
        v = mx(v, mn(S(0), S(-1)));
        v = mn(v, mx(S(0), S(-1)));
    } else {
        v = ppm2_face_regular<D>(s, sc, i, j, k, 0, r6);
    }
    return v;
}

// Characteristic-tracing coefficients (Source/MaestroPPM.cpp:209-251):
// sigma = |u| dt / dx, A = 0.5 sigma, B = 1 - 2/3 sigma.
__device__ __forceinline__ void trace_coeffs(double u, double dt, double dxd, double& A, double& B) {
    const double sigma = fabs(u) * dt / dxd;
    A = 0.5 * sigma;
    B = 1.0 - 2.0 / 3.0 * sigma;
}

// Edge values sm, sp of cell (i,j,k) along D from the face values F (quadratic limiter
// :117-128 for ppm_type 1, Colella-2008 limiter :337-434 for ppm_type 2, with the
// boundary re-limiting of :131-205 / :443-700).
//
// F holds, on the two faces next to an ext_dir/hoextrap boundary, the values the reference
// assigns for the first interior cells.  Cells outside the domain (ghost cells of a grown
// box) are not re-limited by the reference and see the regular interpolants on those faces,
// which are recomputed here (dv: van Leer slopes, ppm_type 1).
template <int D, int PPMT>
__device__ __forceinline__ void ppm_cell_edges(const FabView& s, int sc, const FabView& F, const FabView& dv, int i,
                                               int j, int k, int lo_ext, int hi_ext, int domlo, int domhi,
                                               const RecipC& r6, double& sm, double& sp) {
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    auto S = SHIFT_S(s, sc);
    const int I = D == 0 ? i : (D == 1 ? j : k);
    const bool outside = (lo_ext && I < domlo) || (hi_ext && I > domhi);
    auto Fc = [&](int m) -> double {
        const int f = I + m;
        if (outside && ((lo_ext && (f == domlo || f == domlo + 1)) || (hi_ext && (f == domhi || f == domhi + 1)))) {
            if (PPMT == 2) return ppm2_face_regular<D>(s, sc, i, j, k, m, r6);
            const double dvl = at(dv, i + (m - 1) * di, j + (m - 1) * dj, k + (m - 1) * dk);
            const double dvr = at(dv, i + m * di, j + m * dj, k + m * dk);
            double v = half(S(m) + S(m - 1)) - div_c(dvr - dvl, r6);
            v = mx(v, mn(S(m), S(m - 1)));
            return mn(v, mx(S(m), S(m - 1)));
        }
        return at(F, i + m * di, j + m * dj, k + m * dk);
    };
    const double s0 = S(0);
    if (PPMT == 1) {
        sm = Fc(0);
        sp = Fc(1);
        const bool special = (lo_ext && I == domlo) || (hi_ext && I == domhi);
        if (!special) {
            // reference: (sp-s0)*(s0-sm) <= 0;  |sp-s0| >= 2|sm-s0|;  |sm-s0| >= 2|sp-s0|.
            // sm-s0 = -(s0-sm) exactly; non-negative doubles compare like their bit patterns.
            const double a = sp - s0, q = s0 - sm;
            if (!prod_gt0(a, q)) {
                sp = s0;
                sm = s0;
            } else if ((dbits(a) & ABS_MASK) >= (dbits(twice(q)) & ABS_MASK)) {
                sp = 3.0 * s0 - twice(sm);
            } else if ((dbits(q) & ABS_MASK) >= (dbits(twice(a)) & ABS_MASK)) {
                sm = 3.0 * s0 - twice(sp);
            }
        }
    } else {
        const double C = 1.25;
        double sedgel = Fc(-1), sedge = Fc(0), sedger = Fc(1), sedgerr = Fc(2);
        if (D == 0 && hi_ext && I == domhi - 1) sedgerr = ppm2_face_regular<D>(s, sc, i, j, k, 2, r6);
        if (lo_ext && I == domlo) {
            sm = sedge;
            sp = sedger;
        } else if (hi_ext && I == domhi) {
            sp = sedger;
            sm = sedge;
        } else {
            const double bigm_tol = (D == 0 && lo_ext && (I == domlo + 1 || I == domlo + 2)) ? 1.e10 : 1.e-10;
            double alphap = sedger - s0;
            double alpham = sedge - s0;
            // |alphap| > 2|alpham| and |alpham| > 2|alphap| on magnitudes' bit patterns;
            // alpham * alphap >= 0 is "not (alpham * -alphap > 0)"
            const bool bigp = (dbits(alphap) & ABS_MASK) > (dbits(twice(alpham)) & ABS_MASK);
            const bool bigm = (dbits(alpham) & ABS_MASK) > (dbits(twice(alphap)) & ABS_MASK);
            bool extremum = false;
            if (!prod_gt0(alpham, -alphap)) {
                extremum = true;
            } else if (bigp || bigm) {
                double dafacem = sedge - sedgel;
                double dafacep = sedgerr - sedger;
                double dabarm = s0 - S(-1);
                double dabarp = S(1) - s0;
                double dafacemin = mn(fabs(dafacem), fabs(dafacep));
                double dabarmin = mn(fabs(dabarm), fabs(dabarp));
                double dachkm, dachkp;
                if (dafacemin >= dabarmin) {
                    dachkm = dafacem;
                    dachkp = dafacep;
                } else {
                    dachkm = dabarm;
                    dachkp = dabarp;
                }
                extremum = !prod_gt0(dachkm, dachkp);
            }
            if (extremum) {
                double D2 = 6.0 * (alpham + alphap);
                double D2L = S(-2) - 2.0 * S(-1) + s0;
                double D2R = s0 - 2.0 * S(1) + S(2);
                double D2C = S(-1) - 2.0 * s0 + S(1);
                double sgn = copysign(1.0, D2);
                double D2LIM = mx(mn(sgn * D2, mn(C * sgn * D2L, mn(C * sgn * D2R, C * sgn * D2C))), 0.0);
                double D2ABS = mx(fabs(D2), 1.e-10);
                alpham = alpham * D2LIM / D2ABS;
                alphap = alphap * D2LIM / D2ABS;
            } else {
                if (bigp) {
                    double sgn = copysign(1.0, alpham);
                    double amax = -alphap * alphap / (4.0 * (alpham + alphap));
                    double delam = S(-1) - s0;
                    if (sgn * amax >= sgn * delam) {
                        if (sgn * (delam - alpham) >= 1.e-10) {
                            alphap = -2.0 * delam - 2.0 * sgn * sqrt(delam * delam - delam * alpham);
                        } else {
                            alphap = -2.0 * alpham;
                        }
                    }
                }
                if (bigm) {
                    double sgn = copysign(1.0, alphap);
                    double amax = -alpham * alpham / (4.0 * (alpham + alphap));
                    double delap = S(1) - s0;
                    if (sgn * amax >= sgn * delap) {
                        if (sgn * (delap - alphap) >= bigm_tol) {
                            alpham = (-2.0 * delap - 2.0 * sgn * sqrt(delap * delap - delap * alphap));
                        } else {
                            alpham = -2.0 * alphap;
                        }
                    }
                }
            }
            sm = s0 + alpham;
            sp = s0 + alphap;
        }
    }
}

// Characteristic tracing of one cell: Ip from the velocity at the high face (coefficients
// Ap, Bp), Im from the low face (Am, Bm); tb = bits(rel_eps).
__device__ __forceinline__ void ppm_trace(double s0, double sm, double sp, double up, double um, double Ap, double Bp,
                                          double Am, double Bm, long long tb, double& ip, double& im) {
    const double s6 = 6.0 * s0 - 3.0 * (sm + sp);
    ip = s0;
    im = s0;
    if (gt_t(up, tb)) ip = sp - Ap * (sp - sm - Bp * s6);
    if (lt_negt(um, tb)) im = sm + Am * (sp - sm + Bm * s6);
}

}  // namespace madv
