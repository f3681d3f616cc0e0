// Reverse (adjoint) sweep of the advection stage on a fixed velocity: the transposes of
// UpdateScal, MakeRhoXFlux / MakeRhoHFlux (species_pred_type 1, enthalpy_pred_type 1),
// MakeEdgeScal with PPM ppm_type 1 (van Leer slopes, interface values, cell-edge limiter,
// characteristic tracing, predictor, transverse and edge corrections) and ppm_type 2 (the
// fourth-order interfaces and the Colella-Sekora limiter, on their branch), the pointwise
// conversions and forces of DensityAdvance / EnthalpyAdvance, FillBoundary and the
// physical-boundary fill; and, for the gradient with respect to the cell velocity, of
// VelPred and MakeUtrans.
//
// Every limiter, clamp and upwind decision is recomputed from the forward inputs with the
// forward's own expressions (the same compile flags, so the same bits), i.e. the
// decisions are frozen at the forward pass; the adjoint is the transpose of the
// forward's derivative on that branch.  Scatter transposes use atomicAdd into the
// adjoint FABs, which have the forward FABs' index spaces (and zero-filled margins
// wherever a transpose reads one cell past the forward region).
//
// Scope: 3-D, one level, plane-parallel or spherical (either radial grid), MAC velocities independent of the
// state (grav_cell = 0, no pressure gradient), so the velocity force has no state term.
// The state gradient allows w0 != 0 and outflow, symmetry and wall boundaries (scalar BCs
// foextrap, reflect_even, hoextrap: PPM's boundary stencils transposed; ppm_type 2 without
// walls); the gradient with respect to the velocity needs a periodic domain and w0 = 0.  With
// grav_cell = 0 the gradp0 of MakeRhoHForce is zero (below the cutoff it is rho0 g; above
// it the reference differences the planar p0 across j, Source/MaestroForce.cpp:606-614),
// so the rhoh forces' veladv term has no derivative.  The forward kernels mirrored here
// are in madv_kernels.cu.
#include "madv_launch.cuh"
#include "madv_ppm.cuh"

namespace madv {

#define AW(s) VW(F_USER + (s))
#define AQ_SLOT(a, b) (A_AQ01 + 2 * (a) + ((b) > (a) ? (b)-1 : (b)))

// Weights of the scalar upwinding  v = (u > 0) ? l : r  for |u| > t, (l + r)/2 otherwise.
__device__ __forceinline__ void upwind_w(double u, long long tb, double& wl, double& wr) {
    const long long ub = dbits(u);
    if ((ub & ABS_MASK) > tb) {
        wl = ub > 0 ? 1.0 : 0.0;
        wr = 1.0 - wl;
    } else {
        wl = 0.5;
        wr = 0.5;
    }
}

// Weights of VelPred's upwinding by the transverse velocity: (l + r)/2 for |tr| < rel_eps.
__device__ __forceinline__ void upwind_w_vp(double tr, long long tb, double& wl, double& wr) {
    if ((dbits(tr) & ABS_MASK) >= tb) {
        wl = gt0(tr) ? 1.0 : 0.0;
        wr = 1.0 - wl;
    } else {
        wl = 0.5;
        wr = 0.5;
    }
}

// The edge and transverse states of a scalar on a domain face with a physical boundary:
// foextrap and reflect_even take the inside state (r on the low face, l on the high face),
// reflect_odd gives zero (3-D blocks of Source/MaestroMakeEdgeScalars.cpp: predictor
// :711-860, transverse :934-1340, edges :1456-1660).  ext_dir and hoextrap scalars are
// rejected on the host.
__device__ __forceinline__ void boundary_w(int I, int bclo, int bchi, int domlo, int domhi, double& wl, double& wr) {
    if (I == domlo && bclo != BC_INT_DIR) {
        wl = 0.0;
        wr = bclo == BC_REFLECT_ODD ? 0.0 : 1.0;
    } else if (I == domhi + 1 && bchi != BC_INT_DIR) {
        wr = 0.0;
        wl = bchi == BC_REFLECT_ODD ? 0.0 : 1.0;
    }
}

// The Riemann selection of MakeUtrans / VelPredVelocities (w0c = w0_cart on z-faces):
// 0 (the value 0), 1 (l) or 2 (r).
__device__ __forceinline__ int riemann_pick(double l, double r, double w0c, bool zdir, double rel_eps) {
    bool test;
    double v;
    if (!zdir) {
        test = (l <= 0.0 && r >= 0.0) || (fabs(l + r) < rel_eps);
        v = 0.5 * (l + r);
    } else {
        test = (l + w0c <= 0.0 && r + w0c >= 0.0) || (fabs(l + r + 2.0 * w0c) < rel_eps);
        v = 0.5 * (l + r) + w0c;
    }
    if (test) return 0;
    return v > 0.0 ? 1 : 2;
}

// ------------------------------------------------------------------ UpdateScal^T
// Forward (valid cells): rhoX_new = rhoX_old - dt div F_X, rho_new = rho_old +
// sum(rhoX_new - rhoX_old), rhoh_new = rhoh_old + dt(-div F_h + f); temperature and pi
// are carried.  In: A_ASNEW.  Out: A_ASOLD += the direct terms, and A_ASNEW's species
// components become the total adjoints of rhoX_new (which the flux transpose reads).
// The floor (rho < base_cutoff_density / 2) and negative-species branches are taken as
// not active.
__global__ void k_adj_update(KARGS, int nspec) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView an = AW(A_ASNEW), ao = AW(A_ASOLD);
    const double arho = at(an, i, j, k, RHO);
    at(ao, i, j, k, RHO) += arho;
    at(ao, i, j, k, RHOH) += at(an, i, j, k, RHOH);
    at(ao, i, j, k, TEMP) += at(an, i, j, k, TEMP);
    at(ao, i, j, k, PI) += at(an, i, j, k, PI);
    for (int comp = FIRSTSPEC; comp < FIRSTSPEC + nspec; ++comp) {
        const double a = at(an, i, j, k, comp);
        at(ao, i, j, k, comp) += a;
        at(an, i, j, k, comp) = a + arho;
    }
}

// Flux transposes on the valid D-faces of each box.  The update of a box reads only its
// own face fluxes, so the flux adjoint of face f is dt/h (a(f) - a(f-1)) over the cells
// f, f-1 that lie in the box.  With F_X = u (rho0_edge + rho'_e) X_e and
// F_h = u (rhoh0_edge + rhoh'_e): edge-state adjoints to A_AEDGE0+D, and (want_u) the
// face-velocity adjoint to A_AUMAC0+D.
template <int D>
__global__ void k_adj_flux(KARGS, int nspec, double dtdx, const double* __restrict__ r0a,
                           const double* __restrict__ r0b, const double* __restrict__ h0a,
                           const double* __restrict__ h0b, int want_u, int sph) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const RegionBox& rr = R[e_];
    const int I = D == 0 ? i : (D == 1 ? j : k);
    const bool cell_hi = I < rr.lo[D] + rr.n[D] - 1;  // cell I lies in the box
    const bool cell_lo = I > rr.lo[D];                // cell I-1 lies in the box
    const FabView an = AW(A_ASNEW), ae = AW(A_AEDGE0 + D), e = VW(F_SEDGE0 + D);
    const double u = at(VW(F_UMAC0 + D), i, j, k);
    auto fbar = [&](int comp) {
        double a = 0.0;
        if (cell_hi) a += at(an, i, j, k, comp);
        if (cell_lo) a -= at(an, i - di, j - dj, k - dk, comp);
        return dtdx * a;
    };
    // rho0_edge: planar, the old and new edge base state of row k; spherical, MakeS0mac's
    // face values of the two (F_S0MAC*, F_S0MACB*), combined as k_rhox_flux_sph does
    const double r0f = sph ? 0.5 * at(VW(F_S0MAC0 + D), i, j, k) + 0.5 * at(VW(F_S0MACB0 + D), i, j, k)
                           : 0.5 * (r0a[k] + r0b[k]);
    const double erho = r0f + at(e, i, j, k, RHO);
    const double cx = u * erho;
    double arho = 0.0, gu = 0.0;
    for (int comp = FIRSTSPEC; comp < FIRSTSPEC + nspec; ++comp) {
        const double fb = fbar(comp);
        const double ex = at(e, i, j, k, comp);
        at(ae, i, j, k, comp) = cx * fb;
        arho += u * ex * fb;
        gu += erho * ex * fb;
    }
    at(ae, i, j, k, RHO) = arho;
    const double fh = fbar(RHOH);
    at(ae, i, j, k, RHOH) = u * fh;
    if (want_u) {
        // spherical: the (rho h) term reads MakeS0mac's faces (k_adj_flux_rhoh_u_sph)
        if (!sph) gu += (0.5 * (h0a[k] + h0b[k]) + at(e, i, j, k, RHOH)) * fh;
        at(AW(A_AUMAC0 + D), i, j, k) += gu;
    }
}

// The (rho h) flux's face-velocity adjoint, spherical (k_rhoh_flux_sph, enthalpy_pred_type 1):
// F_h = u (rhoh0_face + rhoh'_e) with rhoh0_face the LinComb of F_S0MAC* and F_S0MACB*
// (exact base state), or rho0_face h0_face (uniform bins: rho0 in F_S0MACC* / F_S0MACD*).
template <int D>
__global__ void k_adj_flux_rhoh_u_sph(KARGS, double dtdx, int exact) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const RegionBox& rr = R[e_];
    const int I = D == 0 ? i : (D == 1 ? j : k);
    const FabView an = AW(A_ASNEW);
    double a = 0.0;
    if (I < rr.lo[D] + rr.n[D] - 1) a += at(an, i, j, k, RHOH);
    if (I > rr.lo[D]) a -= at(an, i - di, j - dj, k - dk, RHOH);
    if (a == 0.0) return;
    const double h0f = 0.5 * at(VW(F_S0MAC0 + D), i, j, k) + 0.5 * at(VW(F_S0MACB0 + D), i, j, k);
    const double base =
        exact ? h0f : (0.5 * at(VW(F_S0MACC0 + D), i, j, k) + 0.5 * at(VW(F_S0MACD0 + D), i, j, k)) * h0f;
    at(AW(A_AUMAC0 + D), i, j, k) += (base + at(VW(F_SEDGE0 + D), i, j, k, RHOH)) * (dtdx * a);
}

// ------------------------------------------------------------------ MakeEdgeScal^T
// k_es_edges (advective form) transposed: valid D-faces.  want_u: the adjoint of the
// transverse coefficients (F_TCOEF comps 3+t) into A_ATCOEF, from the forward transverse
// states of this component (F_Q fields).
template <int D>
__global__ void k_adj_es_edges(KARGS, int comp, int force_zero, double dt2, long long epsb, int want_u, int bclo,
                               int bchi, int domlo, int domhi) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    constexpr int T1 = D == 0 ? 1 : 0, T2 = D == 2 ? 1 : 2;
    constexpr int a1i = T1 == 0, a1j = T1 == 1, a1k = T1 == 2;
    constexpr int a2i = T2 == 0, a2j = T2 == 1, a2k = T2 == 2;
    const int il = i - di, jl = j - dj, kl = k - dk;
    const double ab = at(AW(A_AEDGE0 + D), i, j, k, comp);
    double wl, wr;
    upwind_w(at(VW(F_UMAC0 + D), i, j, k), epsb, wl, wr);
    boundary_w(D == 0 ? i : (D == 1 ? j : k), bclo, bchi, domlo, domhi, wl, wr);
    const double la = wl * ab, ra = wr * ab;
    at(AW(A_ASL0 + D), i, j, k) += la;
    at(AW(A_ASR0 + D), i, j, k) += ra;
    const FabView tc = VW(F_TCOEF);
    const FabView q1 = AW(AQ_SLOT(T1, T2)), q2 = AW(AQ_SLOT(T2, T1));
    double c1 = at(tc, il, jl, kl, 3 + T1) * la, c2 = at(tc, il, jl, kl, 3 + T2) * la;
    atomicAdd(&at(q1, il + a1i, jl + a1j, kl + a1k), -c1);
    atomicAdd(&at(q1, il, jl, kl), c1);
    atomicAdd(&at(q2, il + a2i, jl + a2j, kl + a2k), -c2);
    atomicAdd(&at(q2, il, jl, kl), c2);
    c1 = at(tc, i, j, k, 3 + T1) * ra;
    c2 = at(tc, i, j, k, 3 + T2) * ra;
    atomicAdd(&at(q1, i + a1i, j + a1j, k + a1k), -c1);
    atomicAdd(&at(q1, i, j, k), c1);
    atomicAdd(&at(q2, i + a2i, j + a2j, k + a2k), -c2);
    atomicAdd(&at(q2, i, j, k), c2);
    if (!force_zero) {
        const FabView af = AW(A_AFORCE);
        atomicAdd(&at(af, il, jl, kl), dt2 * la);
        atomicAdd(&at(af, i, j, k), dt2 * ra);
    }
    if (want_u) {
        const FabView atc = AW(A_ATCOEF), f1 = VW(Q_FIELD(T1, T2)), f2 = VW(Q_FIELD(T2, T1));
        atomicAdd(&at(atc, il, jl, kl, 3 + T1), -la * (at(f1, il + a1i, jl + a1j, kl + a1k) - at(f1, il, jl, kl)));
        atomicAdd(&at(atc, il, jl, kl, 3 + T2), -la * (at(f2, il + a2i, jl + a2j, kl + a2k) - at(f2, il, jl, kl)));
        atomicAdd(&at(atc, i, j, k, 3 + T1), -ra * (at(f1, i + a1i, j + a1j, k + a1k) - at(f1, i, j, k)));
        atomicAdd(&at(atc, i, j, k, 3 + T2), -ra * (at(f2, i + a2i, j + a2j, k + a2k) - at(f2, i, j, k)));
    }
}

// k_es_transverse (advective form) transposed: D-faces corrected in direction T.
template <int D, int T>
__global__ void k_adj_es_transverse(KARGS, long long epsb, int want_u, int bclo, int bchi, int domlo, int domhi) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    constexpr int ti = T == 0, tj = T == 1, tk = T == 2;
    const int il = i - di, jl = j - dj, kl = k - dk;
    const double qb = at(AW(AQ_SLOT(D, T)), i, j, k);
    double wl, wr;
    upwind_w(at(VW(F_UMAC0 + D), i, j, k), epsb, wl, wr);
    boundary_w(D == 0 ? i : (D == 1 ? j : k), bclo, bchi, domlo, domhi, wl, wr);
    const double la = wl * qb, ra = wr * qb;
    at(AW(A_ASL0 + D), i, j, k) += la;
    at(AW(A_ASR0 + D), i, j, k) += ra;
    const FabView tc = VW(F_TCOEF), sh = AW(A_ASIMH0 + T);
    const double cl = at(tc, il, jl, kl, T) * la, cr = at(tc, i, j, k, T) * ra;
    atomicAdd(&at(sh, il + ti, jl + tj, kl + tk), -cl);
    atomicAdd(&at(sh, il, jl, kl), cl);
    atomicAdd(&at(sh, i + ti, j + tj, k + tk), -cr);
    atomicAdd(&at(sh, i, j, k), cr);
    if (want_u) {
        const FabView atc = AW(A_ATCOEF), s = VW(F_SIMH0 + T);
        atomicAdd(&at(atc, il, jl, kl, T), -la * (at(s, il + ti, jl + tj, kl + tk) - at(s, il, jl, kl)));
        atomicAdd(&at(atc, i, j, k, T), -ra * (at(s, i + ti, j + tj, k + tk) - at(s, i, j, k)));
    }
}

// k_es_predictor (ppm_type 1) transposed: simh = upwind(u, l, r, 0).  On a domain face
// with a physical boundary the forward set l, r and simh all to the inside state (r on the
// low face, l on the high face; zero for reflect_odd), so that state takes all three
// adjoints and the outside one none.
template <int D>
__global__ void k_adj_es_predictor(KARGS, int bclo, int bchi, int domlo, int domhi) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const double sb = at(AW(A_ASIMH0 + D), i, j, k);
    const int I = D == 0 ? i : (D == 1 ? j : k);
    double& la = at(AW(A_ASL0 + D), i, j, k);
    double& ra = at(AW(A_ASR0 + D), i, j, k);
    if (I == domlo && bclo != BC_INT_DIR) {
        ra = bclo == BC_REFLECT_ODD ? 0.0 : ra + la + sb;
        la = 0.0;
        return;
    }
    if (I == domhi + 1 && bchi != BC_INT_DIR) {
        la = bchi == BC_REFLECT_ODD ? 0.0 : la + ra + sb;
        ra = 0.0;
        return;
    }
    double wl, wr;
    upwind_w(at(VW(F_UMAC0 + D), i, j, k), 0, wl, wr);
    la += wl * sb;
    ra += wr * sb;
}

// ------------------------------------------------------------------ ppm_type 2 transposed
// A value with one directional derivative.  The value is formed by exactly the forward's
// double operations (so every decision taken on it is the forward's); the derivative is
// that of the branch taken.
struct Dv {
    double v, d;
};
__device__ __forceinline__ Dv operator+(Dv a, Dv b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dv operator-(Dv a, Dv b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dv operator-(Dv a) { return {-a.v, -a.d}; }
__device__ __forceinline__ Dv operator*(Dv a, Dv b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__device__ __forceinline__ Dv operator*(double a, Dv b) { return {a * b.v, a * b.d}; }
__device__ __forceinline__ Dv operator/(Dv a, Dv b) { return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
__device__ __forceinline__ Dv dv_mn(Dv a, Dv b) { return (b.v < a.v) ? b : a; }
__device__ __forceinline__ Dv dv_mx(Dv a, Dv b) { return (a.v < b.v) ? b : a; }

// The ppm_type 2 edge values of one cell away from ext_dir / hoextrap boundaries
// (ppm_cell_edges, Colella-Sekora limiter, Source/MaestroPPM.cpp:337-434) and their
// transpose: S[0..4] = s(-2..2), F[0..3] = faces -1..2 of the cell.  The forward part
// repeats the forward's double operations, so every decision is the forward's; the reverse
// part takes the edge adjoints bsm, bsp of the branch taken and adds the input adjoints to
// gS, gF.  Returns the edges in sm, sp.
__device__ __forceinline__ void ppm2_edges_adj(const double* S, const double* F, double bsm, double bsp, double* gS,
                                               double* gF, double& sm, double& sp) {
    const double C = 1.25;
    const double s0 = S[2];
    const double am0 = F[1] - s0, ap0 = F[2] - s0;
    double alpham = am0, alphap = ap0;
    const bool bigp = (dbits(alphap) & ABS_MASK) > (dbits(twice(alpham)) & ABS_MASK);
    const bool bigm = (dbits(alpham) & ABS_MASK) > (dbits(twice(alphap)) & ABS_MASK);
    bool extremum = false;
    if (!prod_gt0(alpham, -alphap)) {
        extremum = true;
    } else if (bigp || bigm) {
        const double dafacem = F[1] - F[0], dafacep = F[3] - F[2];
        const double dabarm = s0 - S[1], dabarp = S[3] - s0;
        const double dafacemin = mn(fabs(dafacem), fabs(dafacep));
        const double dabarmin = mn(fabs(dabarm), fabs(dabarp));
        const bool face = dafacemin >= dabarmin;
        extremum = !prod_gt0(face ? dafacem : dabarm, face ? dafacep : dabarp);
    }
    double gam = 0.0, gap = 0.0;  // adjoints of am0, ap0
    gS[2] += bsm + bsp;           // sm = s0 + alpham, sp = s0 + alphap
    if (extremum) {
        const double D2 = 6.0 * (alpham + alphap);
        const double D2L = S[0] - 2.0 * S[1] + s0;
        const double D2R = s0 - 2.0 * S[3] + S[4];
        const double D2C = S[1] - 2.0 * s0 + S[3];
        const double sgn = copysign(1.0, D2);
        // D2LIM = mx(mn(sgn D2, mn(C sgn D2L, mn(C sgn D2R, C sgn D2C))), 0): which term it is
        const double cD = sgn * D2, cL = C * sgn * D2L, cR = C * sgn * D2R, cC = C * sgn * D2C;
        int pick = (cC < cR) ? 3 : 2;  // 0: D2, 1: D2L, 2: D2R, 3: D2C, 4: the constant 0
        double v = pick == 3 ? cC : cR;
        if (v < cL) {
        } else {
            pick = 1;
            v = cL;
        }
        if (v < cD) {
        } else {
            pick = 0;
            v = cD;
        }
        if (v < 0.0) {
            pick = 4;
            v = 0.0;
        }
        const double D2LIM = v;
        const bool abs_pick = !(fabs(D2) < 1.e-10);
        const double D2ABS = abs_pick ? fabs(D2) : 1.e-10;
        alpham = alpham * D2LIM / D2ABS;
        alphap = alphap * D2LIM / D2ABS;
        const double q = bsm * am0 + bsp * ap0;
        gam += bsm * D2LIM / D2ABS;
        gap += bsp * D2LIM / D2ABS;
        const double gL = q / D2ABS;                     // d/dD2LIM
        double gD2 = 0.0;
        if (abs_pick) gD2 -= (signbit(D2) ? -1.0 : 1.0) * q * D2LIM / (D2ABS * D2ABS);
        if (pick == 0) gD2 += gL * sgn;
        const double gc = gL * C * sgn;                  // d/d(D2L, D2R or D2C)
        if (pick == 1) {
            gS[0] += gc;
            gS[1] -= 2.0 * gc;
            gS[2] += gc;
        } else if (pick == 2) {
            gS[2] += gc;
            gS[3] -= 2.0 * gc;
            gS[4] += gc;
        } else if (pick == 3) {
            gS[1] += gc;
            gS[2] -= 2.0 * gc;
            gS[3] += gc;
        }
        gam += 6.0 * gD2;
        gap += 6.0 * gD2;
    } else {
        // bigp rewrites alphap from (alpham, delam); bigm then alpham from (alphap, delap)
        int p_case = 0, m_case = 0;  // 0: unchanged, 1: the square-root form, 2: -2 x the other
        double p_sq = 0.0, p_sg = 0.0, delam = 0.0, m_sq = 0.0, m_sg = 0.0, delap = 0.0, ap_in = 0.0;
        if (bigp) {
            const double sgn = copysign(1.0, alpham);
            const double amax = -alphap * alphap / (4.0 * (alpham + alphap));
            delam = S[1] - s0;
            if (sgn * amax >= sgn * delam) {
                if (sgn * (delam - alpham) >= 1.e-10) {
                    p_sq = sqrt(delam * delam - delam * alpham);
                    alphap = -2.0 * delam - 2.0 * sgn * p_sq;
                    p_case = 1;
                } else {
                    alphap = -2.0 * alpham;
                    p_case = 2;
                }
                p_sg = sgn;
            }
        }
        ap_in = alphap;
        if (bigm) {
            const double sgn = copysign(1.0, alphap);
            const double amax = -alpham * alpham / (4.0 * (alpham + alphap));
            delap = S[3] - s0;
            if (sgn * amax >= sgn * delap) {
                if (sgn * (delap - alphap) >= 1.e-10) {
                    m_sq = sqrt(delap * delap - delap * alphap);
                    alpham = -2.0 * delap - 2.0 * sgn * m_sq;
                    m_case = 1;
                } else {
                    alpham = -2.0 * alphap;
                    m_case = 2;
                }
                m_sg = sgn;
            }
        }
        double g_am = bsm, g_ap = bsp;  // adjoints of the final alpham, alphap
        if (m_case == 1) {              // alpham = -2 delap - 2 sg sqrt(delap^2 - delap ap_in)
            const double gdp = g_am * (-2.0 - m_sg * (2.0 * delap - ap_in) / m_sq);
            g_ap += g_am * (m_sg * delap / m_sq);
            gS[3] += gdp;
            gS[2] -= gdp;
            g_am = 0.0;
        } else if (m_case == 2) {
            g_ap += -2.0 * g_am;
            g_am = 0.0;
        }
        if (p_case == 1) {  // alphap = -2 delam - 2 sg sqrt(delam^2 - delam am0)
            const double gdm = g_ap * (-2.0 - p_sg * (2.0 * delam - am0) / p_sq);
            g_am += g_ap * (p_sg * delam / p_sq);
            gS[1] += gdm;
            gS[2] -= gdm;
            g_ap = 0.0;
        } else if (p_case == 2) {
            g_am += -2.0 * g_ap;
            g_ap = 0.0;
        }
        gam += g_am;
        gap += g_ap;
    }
    // am0 = F(0) - s0, ap0 = F(1) - s0
    gF[1] += gam;
    gF[2] += gap;
    gS[2] -= gam + gap;
    sm = s0 + alpham;
    sp = s0 + alphap;
}

// ppm2_face_regular on values with a derivative, face between cells m-1 and m:
// S[0..3] = s(m-2 .. m+1).
__device__ __forceinline__ Dv ppm2_face_dv(const Dv* S, const RecipC& r6) {
    const double C = 1.25;
    Dv se = (7.0 / 12.0) * (S[1] + S[2]) - (1.0 / 12.0) * (S[0] + S[3]);
    if (prod_gt0(se.v - S[1].v, se.v - S[2].v)) {
        const Dv D2 = 3.0 * (S[1] - 2.0 * se + S[2]);
        const Dv D2L = S[0] - 2.0 * S[1] + S[2];
        const Dv D2R = S[1] - 2.0 * S[2] + S[3];
        const double sgn = copysign(1.0, D2.v);
        const Dv D2LIM = sgn * dv_mx(dv_mn(C * sgn * D2L, dv_mn(C * sgn * D2R, sgn * D2)), Dv{0.0, 0.0});
        // div_c(x, 6) is the correctly rounded x / 6: its derivative is d / 6
        se = 0.5 * (S[1] + S[2]) - Dv{div_c(D2LIM.v, r6), D2LIM.d / 6.0};
    }
    return se;
}

// k_ppm_cell<D, 2, 1> transposed away from ext_dir / hoextrap boundaries (cells of the box
// grown by one): the tracing as for ppm_type 1, then the limiter's transpose on the
// forward's branch (ppm2_edges_adj).  Face adjoints: faces -1, 0 into A_ASM of cells
// -1, 0 and faces 1, 2 into A_ASP of cells 0, 1 (k_adj_ppm2_face gathers A_ASM(f) +
// A_ASP(f-1)); cell adjoints to slot ts, component tcomp.
// want_u: the tracing coefficients' velocity adjoint into A_AUMAC0+D, as for ppm_type 1
// (the tracing is the same function of the limited edges sm, sp and s6).
template <int D>
__global__ void k_adj_ppm2_cell(KARGS, int fs, int sc, int lc, int ts, int tcomp, long long epsb, double dtdx,
                                int want_u) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const double ipb = at(AW(A_ASL0 + D), i + di, j + dj, k + dk, lc);
    const double imb = at(AW(A_ASR0 + D), i, j, k, lc);
    if (ipb == 0.0 && imb == 0.0) return;
    const FabView s = VW(fs), F = VW(F_FACE0 + D);
    double Sv[5], Fv[4];
    for (int m = 0; m < 5; ++m) Sv[m] = at(s, i + (m - 2) * di, j + (m - 2) * dj, k + (m - 2) * dk, sc);
    for (int m = 0; m < 4; ++m) Fv[m] = at(F, i + (m - 1) * di, j + (m - 1) * dj, k + (m - 1) * dk);
    // the edges first (the tracing's transpose needs only the branch, not the values: its
    // weights are the tracing coefficients), then the tracing adjoints into the limiter's
    const FabView T = VW(F_TRA0 + D), u = VW(F_UMAC0 + D);
    const double up = at(u, i + di, j + dj, k + dk), um = at(u, i, j, k);
    const double Ap = at(T, i + di, j + dj, k + dk, 0), Bp = at(T, i + di, j + dj, k + dk, 1);
    const double Am = at(T, i, j, k, 0), Bm = at(T, i, j, k, 1);
    double bs0 = 0.0, bsm = 0.0, bsp = 0.0;
    if (gt_t(up, epsb)) {
        const double t = Ap * ipb, w = 3.0 * (Bp * t);
        bsp += (ipb - t) - w;
        bsm += t - w;
        bs0 += twice(w);
    } else {
        bs0 += ipb;
    }
    if (lt_negt(um, epsb)) {
        const double t = Am * imb, w = 3.0 * (Bm * t);
        bsm += (imb - t) - w;
        bsp += t - w;
        bs0 += twice(w);
    } else {
        bs0 += imb;
    }
    double gS[5] = {0.0, 0.0, bs0, 0.0, 0.0}, gF[4] = {0.0, 0.0, 0.0, 0.0};
    double sm, sp;
    ppm2_edges_adj(Sv, Fv, bsm, bsp, gS, gF, sm, sp);
    if (want_u) {  // d ip/dA = -(sp - sm - B s6), d ip/dB = A s6; d im/dA = sp - sm + B s6, d im/dB = A s6
        const double s6 = 6.0 * Sv[2] - 3.0 * (sm + sp), dpm = sp - sm;
        const FabView au = AW(A_AUMAC0 + D);
        if (gt_t(up, epsb))
            atomicAdd(&at(au, i + di, j + dj, k + dk),
                      copysign(dtdx, up) * ipb * (half(Bp * s6 - dpm) - (2.0 / 3.0) * Ap * s6));
        if (lt_negt(um, epsb))
            atomicAdd(&at(au, i, j, k), copysign(dtdx, um) * imb * (half(dpm + Bm * s6) - (2.0 / 3.0) * Am * s6));
    }
    const FabView as = AW(ts);
    for (int m = 0; m < 5; ++m)
        if (gS[m] != 0.0) atomicAdd(&at(as, i + (m - 2) * di, j + (m - 2) * dj, k + (m - 2) * dk, tcomp), gS[m]);
    const FabView am = AW(A_ASM), ap = AW(A_ASP);
    if (gF[0] != 0.0) atomicAdd(&at(am, i - di, j - dj, k - dk), gF[0]);
    if (gF[1] != 0.0) atomicAdd(&at(am, i, j, k), gF[1]);
    if (gF[2] != 0.0) atomicAdd(&at(ap, i, j, k), gF[2]);
    if (gF[3] != 0.0) atomicAdd(&at(ap, i + di, j + dj, k + dk), gF[3]);
}

// k_ppm_face<D, 2> transposed away from ext_dir / hoextrap boundaries, faces lo-2 .. hi+3 of
// the box along D (the forward's face region): the fourth-order interpolant, or on a limited
// face its limited form differentiated along each of its four cells.
template <int D>
__global__ void k_adj_ppm2_face(KARGS, int fs, int sc, int ts, int tcomp, RecipC r6) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const RegionBox& rr = R[e_];
    const int I = D == 0 ? i : (D == 1 ? j : k);
    // A_ASM / A_ASP cover cells lo-2 .. hi+2: the last face has no A_ASM entry and the first
    // no A_ASP entry, and the cell kernel writes none there
    double fb = 0.0;
    if (I != rr.lo[D] + rr.n[D] - 1) fb += at(AW(A_ASM), i, j, k);
    if (I != rr.lo[D]) fb += at(AW(A_ASP), i - di, j - dj, k - dk);
    if (fb == 0.0) return;
    const FabView s = VW(fs), as = AW(ts);
    Dv Sv[4];
    for (int m = 0; m < 4; ++m) Sv[m] = Dv{at(s, i + (m - 2) * di, j + (m - 2) * dj, k + (m - 2) * dk, sc), 0.0};
    const double se = (7.0 / 12.0) * (Sv[1].v + Sv[2].v) - (1.0 / 12.0) * (Sv[0].v + Sv[3].v);
    double g[4];
    if (!prod_gt0(se - Sv[1].v, se - Sv[2].v)) {
        g[0] = g[3] = -(1.0 / 12.0) * fb;
        g[1] = g[2] = (7.0 / 12.0) * fb;
    } else {
        for (int q = 0; q < 4; ++q) {
            Sv[q].d = 1.0;
            g[q] = fb * ppm2_face_dv(Sv, r6).d;
            Sv[q].d = 0.0;
        }
    }
    for (int m = 0; m < 4; ++m)
        if (g[m] != 0.0) atomicAdd(&at(as, i + (m - 2) * di, j + (m - 2) * dj, k + (m - 2) * dk, tcomp), g[m]);
}

// The interior face value of ppm_type 1 transposed, face f between cells f-1 and f
// (face = the cell (i,j,k) of index f along D): v = clamp(v0) between the two cells,
// v0 = (s(f) + s(f-1))/2 - (dv(f) - dv(f-1))/6, the clamp decided as the forward decides it
// (mn(a, b) = (b < a) ? b : a, mx(a, b) = (a < b) ? b : a).  v0 is formed with the forward's
// expression: half() for the stored faces, 0.5 * () for the ones a ghost cell recomputes.
// Adjoint fb to the two cells (slot as, component tc) and the slopes (A_ADSVL).
template <int D>
__device__ __forceinline__ void adj_face_regular(const FabView* __restrict__ V, int nb, int b, const FabView& s, int sc,
                                                 const FabView& dv, const FabView& as, int tc, int i, int j, int k,
                                                 double fb, const RecipC& r6, bool halved) {
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const double sl = at(s, i - di, j - dj, k - dk, sc), s0 = at(s, i, j, k, sc);
    const double sum = s0 + sl;
    const double v0 = (halved ? half(sum) : 0.5 * sum) - div_c(at(dv, i, j, k) - at(dv, i - di, j - dj, k - dk), r6);
    const double lo = mn(s0, sl), hi = mx(s0, sl);
    int src = 0;  // 0: v0, 1: s0, 2: s-1
    double v = v0;
    if (v < lo) {
        v = lo;
        src = (sl < s0) ? 2 : 1;
    }
    if (hi < v) src = (s0 < sl) ? 2 : 1;
    if (src == 0) {
        atomicAdd(&at(as, i, j, k, tc), 0.5 * fb);
        atomicAdd(&at(as, i - di, j - dj, k - dk, tc), 0.5 * fb);
        const FabView ad = AW(A_ADSVL);
        const double f6 = div_c(fb, r6);
        atomicAdd(&at(ad, i, j, k), -f6);
        atomicAdd(&at(ad, i - di, j - dj, k - dk), f6);
    } else if (src == 1) {
        atomicAdd(&at(as, i, j, k, tc), fb);
    } else {
        atomicAdd(&at(as, i - di, j - dj, k - dk, tc), fb);
    }
}

// k_ppm_cell<D, 1, UMAC> transposed (cells of the box grown by one).  The predictors read
// l(face f) = Ip(cell f-1) and r(face f) = Im(cell f), so Ip / Im of a cell take the
// adjoints of its high / low face, component lc of A_ASL0+D / A_ASR0+D.  Tracing is
// linear in (s0, sm, sp) for the frozen upwind tests; the quadratic limiter
// (Source/MaestroPPM.cpp:117-128) is piecewise linear in (s0, interface values).
// Interface adjoints go to A_ASM (low face) and A_ASP (high face) per cell, gathered per
// face by k_adj_ppm_face; the cell adjoint to slot ts, component tcomp.
// want_u: the tracing coefficients A = |u| dt/(2h), B = 1 - (2/3)|u| dt/h depend on the
// tracing velocity: UMAC = 1, the D-faces of F_UMAC0+D (adjoint atomically into
// A_AUMAC0+D); UMAC = 0, component D of the cell velocity F_UFULL = F_UTILDE + w0_cart
// (adjoint into ts, component D).
template <int D, int UMAC>
__global__ void k_adj_ppm_cell(KARGS, int fs, int sc, int lc, int ts, int tcomp, long long epsb, double dtdx,
                               int want_u, int lo_ext, int hi_ext, int domlo, int domhi, RecipC r6) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const double ipb = at(AW(A_ASL0 + D), i + di, j + dj, k + dk, lc);
    const double imb = at(AW(A_ASR0 + D), i, j, k, lc);
    if (ipb == 0.0 && imb == 0.0) return;  // A_ASM / A_ASP were cleared
    const FabView s = VW(fs), F = VW(F_FACE0 + D);
    const double s0 = at(s, i, j, k, sc);
    // Next to an ext_dir / hoextrap boundary (ppm_cell_edges): the first interior cell is
    // not limited, and a ghost cell beyond the boundary reads the interior interpolants of
    // the two boundary faces, recomputed, instead of the boundary values stored there.
    const int I = D == 0 ? i : (D == 1 ? j : k);
    const bool outside = (lo_ext && I < domlo) || (hi_ext && I > domhi);
    auto recomputed = [&](int f) {
        return outside && ((lo_ext && (f == domlo || f == domlo + 1)) || (hi_ext && (f == domhi || f == domhi + 1)));
    };
    auto regular = [&](int ii, int jj, int kk) {
        const FabView dv = VW(F_DSVL);
        const double sl = at(s, ii - di, jj - dj, kk - dk, sc), sr = at(s, ii, jj, kk, sc);
        double v = 0.5 * (sr + sl) - div_c(at(dv, ii, jj, kk) - at(dv, ii - di, jj - dj, kk - dk), r6);
        v = mx(v, mn(sr, sl));
        return mn(v, mx(sr, sl));
    };
    const bool rm = recomputed(I), rp = recomputed(I + 1);
    double sm = rm ? regular(i, j, k) : at(F, i, j, k);
    double sp = rp ? regular(i + di, j + dj, k + dk) : at(F, i + di, j + dj, k + dk);
    const bool special = (lo_ext && I == domlo) || (hi_ext && I == domhi);
    int cs = 3;  // the forward limiter's case, decided as k_ppm_cell decides it
    const double a = sp - s0, q = s0 - sm;
    if (special) {
    } else if (!prod_gt0(a, q)) {
        sp = s0;
        sm = s0;
        cs = 0;
    } else if ((dbits(a) & ABS_MASK) >= (dbits(twice(q)) & ABS_MASK)) {
        sp = 3.0 * s0 - twice(sm);
        cs = 1;
    } else if ((dbits(q) & ABS_MASK) >= (dbits(twice(a)) & ABS_MASK)) {
        sm = 3.0 * s0 - twice(sp);
        cs = 2;
    }
    double up, um, Ap, Bp, Am, Bm;
    if (UMAC) {
        const FabView T = VW(F_TRA0 + D), u = VW(F_UMAC0 + D);
        up = at(u, i + di, j + dj, k + dk);
        um = at(u, i, j, k);
        Ap = at(T, i + di, j + dj, k + dk, 0);
        Bp = at(T, i + di, j + dj, k + dk, 1);
        Am = at(T, i, j, k, 0);
        Bm = at(T, i, j, k, 1);
    } else {
        const FabView T = VW(F_TRC);
        up = um = at(VW(F_UFULL), i, j, k, D);
        Ap = Am = at(T, i, j, k, 2 * D);
        Bp = Bm = at(T, i, j, k, 2 * D + 1);
    }
    const double s6 = 6.0 * s0 - 3.0 * (sm + sp);
    const double dpm = sp - sm;
    double bs0 = 0.0, bsm = 0.0, bsp = 0.0, gup = 0.0, gum = 0.0;
    // ip = sp - A (sp - sm - B s6): d/dsp = 1 - A - 3AB, d/dsm = A - 3AB, d/ds0 = 6AB, with
    // t = A ipb and w = 3AB ipb (the adjoint is not held to the forward's rounding)
    if (gt_t(up, epsb)) {
        const double t = Ap * ipb, w = 3.0 * (Bp * t);
        bsp += (ipb - t) - w;
        bsm += t - w;
        bs0 += twice(w);
        // d ip/dA = -(sp - sm - B s6), d ip/dB = A s6; dA/du = sign(u) dt/dx / 2, dB/du = -(2/3) sign(u) dt/dx
        if (want_u) gup = copysign(dtdx, up) * ipb * (half(Bp * s6 - dpm) - (2.0 / 3.0) * Ap * s6);
    } else {
        bs0 += ipb;
    }
    // im = sm + A (sp - sm + B s6): d/dsm = 1 - A - 3AB, d/dsp = A - 3AB, d/ds0 = 6AB
    if (lt_negt(um, epsb)) {
        const double t = Am * imb, w = 3.0 * (Bm * t);
        bsm += (imb - t) - w;
        bsp += t - w;
        bs0 += twice(w);
        // d im/dA = sp - sm + B s6, d im/dB = A s6
        if (want_u) gum = copysign(dtdx, um) * imb * (half(dpm + Bm * s6) - (2.0 / 3.0) * Am * s6);
    } else {
        bs0 += imb;
    }
    double fm = 0.0, fp = 0.0;
    if (cs == 0) {
        bs0 += bsm + bsp;
    } else if (cs == 1) {  // sp = 3 s0 - 2 sm
        bs0 += 3.0 * bsp;
        fm = bsm - 2.0 * bsp;
    } else if (cs == 2) {  // sm = 3 s0 - 2 sp
        bs0 += 3.0 * bsm;
        fp = bsp - 2.0 * bsm;
    } else {
        fm = bsm;
        fp = bsp;
    }
    const FabView t = AW(ts);
    // a recomputed face's adjoint goes straight through its interior interpolant; the
    // stored boundary value's transpose (k_adj_ppm_face) sees none of it
    if (rm) adj_face_regular<D>(V, nb, b, s, sc, VW(F_DSVL), t, tcomp, i, j, k, fm, r6, false);
    if (rp) adj_face_regular<D>(V, nb, b, s, sc, VW(F_DSVL), t, tcomp, i + di, j + dj, k + dk, fp, r6, false);
    at(AW(A_ASM), i, j, k) = rm ? 0.0 : fm;
    at(AW(A_ASP), i, j, k) = rp ? 0.0 : fp;
    at(t, i, j, k, tcomp) += bs0;
    if (want_u) {
        if (UMAC) {
            const FabView au = AW(A_AUMAC0 + D);
            if (gup != 0.0) atomicAdd(&at(au, i + di, j + dj, k + dk), gup);
            if (gum != 0.0) atomicAdd(&at(au, i, j, k), gum);
        } else {
            at(t, i, j, k, D) += gup + gum;
        }
    }
}

// k_ppm_face<D, 1> transposed (Source/MaestroPPM.cpp:37-111 interior form):
// v = min(max(v0, min(s0, s-1)), max(s0, s-1)), v0 = (s0 + s-1)/2 - (dv(f) - dv(f-1))/6.
// Cell adjoints to slot ts, component tcomp.
// Faces next to an ext_dir / hoextrap boundary (ppm_face_value): the boundary face takes
// the ghost cell's value, the next one the one-sided cubic
// -s(-2)/5 + 3 s(-1)/4 + s(0)/2 - s(1)/20 (mirrored on the high side), clamped like the
// interior interpolant.
template <int D>
__global__ void k_adj_ppm_face(KARGS, int fs, int sc, int ts, int tcomp, RecipC r6, int lo_ext, int hi_ext, int domlo,
                               int domhi) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const double fb = at(AW(A_ASM), i, j, k) + at(AW(A_ASP), i - di, j - dj, k - dk);
    if (fb == 0.0) return;
    const FabView s = VW(fs), as = AW(ts);
    const int I = D == 0 ? i : (D == 1 ? j : k);
    auto add = [&](int m, double v) { atomicAdd(&at(as, i + m * di, j + m * dj, k + m * dk, tcomp), v); };
    if (lo_ext && I == domlo) {
        add(-1, fb);
        return;
    }
    if (hi_ext && I == domhi + 1) {
        add(0, fb);
        return;
    }
    const bool cub_lo = lo_ext && I == domlo + 1, cub_hi = hi_ext && I == domhi;
    if (cub_lo || cub_hi) {
        auto S = SHIFT_S(s, sc);
        const double v0 = cub_lo ? -0.2 * S(-2) + 0.75 * S(-1) + 0.5 * S(0) - 0.05 * S(1)
                                 : -0.2 * S(1) + 0.75 * S(0) + 0.5 * S(-1) - 0.05 * S(-2);
        const double sl = S(-1), s0 = S(0);
        const double lo = mn(s0, sl), hi = mx(s0, sl);
        int src = 0;
        double v = v0;
        if (v < lo) {
            v = lo;
            src = (sl < s0) ? 2 : 1;
        }
        if (hi < v) src = (s0 < sl) ? 2 : 1;
        if (src == 1) {
            add(0, fb);
        } else if (src == 2) {
            add(-1, fb);
        } else if (cub_lo) {
            add(-2, -0.2 * fb);
            add(-1, 0.75 * fb);
            add(0, 0.5 * fb);
            add(1, -0.05 * fb);
        } else {
            add(1, -0.2 * fb);
            add(0, 0.75 * fb);
            add(-1, 0.5 * fb);
            add(-2, -0.05 * fb);
        }
        return;
    }
    adj_face_regular<D>(V, nb, b, s, sc, VW(F_DSVL), as, tcomp, i, j, k, fb, r6, true);
}

// k_dsvl<D> transposed (Source/MaestroPPM.cpp:37-73):
// dv = sign(dsc) min(|dsc|, |dsl|, |dsr|) where dsl dsr > 0, else 0.
template <int D>
__global__ void k_adj_dsvl(KARGS, int fs, int sc, int ts, int tcomp) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const double g = at(AW(A_ADSVL), i, j, k);
    if (g == 0.0) return;
    const FabView s = VW(fs), as = AW(ts);
    auto S = SHIFT_S(s, sc);
    // the forward's decisions, taken as k_dsvl takes them (bit-pattern scaling, product sign,
    // minimum of the magnitudes' bit patterns)
    const double dsc = half(S(1) - S(-1));
    const double dsl = twice(S(0) - S(-1));
    const double dsr = twice(S(1) - S(0));
    if (!prod_gt0(dsl, dsr)) return;
    const long long ac = dbits(dsc) & ABS_MASK, al = dbits(dsl) & ABS_MASK, ar = dbits(dsr) & ABS_MASK;
    const bool inner_r = ar < al;  // mn(|dsl|, |dsr|)
    const long long inner = inner_r ? ar : al;
    auto add = [&](int m, double v) { atomicAdd(&at(as, i + m * di, j + m * dj, k + m * dk, tcomp), v); };
    if (inner < ac) {  // dv = sign(dsc) |dsl| or sign(dsc) |dsr|: weight +-2 g
        const long long sg = (dbits(dsc) ^ dbits(inner_r ? dsr : dsl)) & SIGN_BIT;
        const double w = __longlong_as_double(dbits(twice(g)) ^ sg);
        if (inner_r) {
            add(1, w);
            add(0, -w);
        } else {
            add(0, w);
            add(-1, -w);
        }
    } else {  // dv = dsc
        add(1, half(g));
        add(-1, -half(g));
    }
}

// FillBoundary transposed: every ghost cell (or face) was copied from one valid one, so
// its adjoint is added there and cleared.
__global__ void k_adj_fill_boundary(const CopyDesc* __restrict__ D, int nd, long total, const FabView* __restrict__ V,
                                    int nb, int f, int nc) {
    const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= total) return;
    int lo = 0, hi = nd - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (D[mid].start <= gid) lo = mid;
        else hi = mid - 1;
    }
    const CopyDesc& cd = D[lo];
    long l = gid - cd.start;
    const long nx = cd.n[0], ny = cd.n[1];
    const long q = l / nx;
    const int i = cd.lo[0] + (int)(l - q * nx);
    const long q2 = q / ny;
    const int j = cd.lo[1] + (int)(q - q2 * ny);
    const int k = cd.lo[2] + (int)q2;
    const FabView dst = V[f * nb + cd.dst_b], src = V[f * nb + cd.src_b];
    for (int n = 0; n < nc; ++n) {
        double& g = at(dst, i, j, k, n);
        const double v = g;
        if (v != 0.0) atomicAdd(&at(src, i - cd.shift[0], j - cd.shift[1], k - cd.shift[2], n), v);
        g = 0.0;
    }
}

// FillPatch's physical-boundary fill of direction d (k_phys_fill) transposed, component n
// of adjoint slot s: each ghost cell outside the domain in d hands its adjoint to the cell
// it was copied from (foextrap: the boundary cell; reflect_even / odd: the mirror cell,
// negated for odd) and is cleared, since the fill overwrote it.  The cells written are
// inside the domain in d and the cells read outside, so one pass has no read-write
// overlap; several ghost cells feeding one cell add atomically.  Run d = 2, 1, 0 (the
// reverse of the forward's order: a corner filled by a later direction from a ghost cell of
// an earlier one passes its adjoint on through that ghost cell), then FillBoundary^T.
__global__ void k_adj_phys_fill(KARGS, int s, int n, BCRecD bc, int d, int domlo, int domhi) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView q = AW(s);
    const int m = d == 0 ? i : (d == 1 ? j : k);
    const int side = m < domlo ? 0 : 1;
    const int t = side == 0 ? bc.lo[d] : bc.hi[d];
    if (t == BC_INT_DIR) return;
    double& g = at(q, i, j, k, n);
    const double a = g;
    g = 0.0;
    int p;
    double w = 1.0;
    if (t == BC_FOEXTRAP) {
        p = side == 0 ? domlo : domhi;
    } else if (t == BC_REFLECT_EVEN || t == BC_REFLECT_ODD) {
        p = side == 0 ? 2 * domlo - 1 - m : 2 * domhi + 1 - m;
        if (t == BC_REFLECT_ODD) w = -1.0;
    } else {  // ext_dir: the ghost value does not depend on the state
        return;
    }
    const int i2 = d == 0 ? p : i, j2 = d == 1 ? p : j, k2 = d == 2 ? p : k;
    atomicAdd(&at(q, i2, j2, k2, n), w * a);
}

// ConvertRhoXToX transposed (valid cells): X = rhoX / rho.
__global__ void k_adj_x(KARGS, int comp) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const double a = at(AW(A_AS), i, j, k);
    const FabView ao = AW(A_ASOLD);
    const double rho = at(AW(A_WSOLD), i, j, k, RHO);
    const double x = at(VW(F_SOLD), i, j, k, comp);
    const double ar = a / rho;  // d(rhoX / rho): one division for both partials
    at(ao, i, j, k, comp) += ar;
    at(ao, i, j, k, RHO) -= ar * x;
}

// PutInPertForm transposed (s' = s - s0) together with the traced force of
// ModifyScalForce, fullform 0 (Source/MaestroForce.cpp:413-441, valid cells):
// f = ... - (s - s0) divu - [s0 (du + dv) + (w(k+1) s0e(k+1) - w(k) s0e(k))/dz].
// want_u: the force's face-velocity adjoint, d f/du(i+1) = -s/dx, d f/dw(k+1) =
// -(s - s0 + s0e(k+1))/dz, ...  (atomically into A_AUMAC0..2).  s0e(k) is the edge value
// the forward read from its Cartesian copy: above the top cell that is the ghost cell
// FillPatch filled (BCS_F): in a periodic domain the image of the bottom edge, else (first-
// order extrapolation, or the even reflection of symmetry) the top cell's own.
__global__ void k_adj_pert(KARGS, int comp, const double* __restrict__ s0a, const double* __restrict__ s0e,
                           RecipC r0, RecipC r1, RecipC r2, int domlo, int domhi, int want_u,
                           const double* __restrict__ w0, int sph, int zper) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView um = VW(F_UMAC0), vm = VW(F_UMAC1), wm = VW(F_UMAC2);
    // ModifyScalForce runs between Addw0(-1) and Addw0(+1): its umac is the MAC velocity
    // without w0 (planar: w0 on the z faces; spherical: w0mac on every face)
    auto U = [&](const FabView& f, int d, int a, int bb, int cc) {
        const double v = at(f, a, bb, cc);
        if (sph) return v + -1.0 * at(VW(F_W0MAC0 + d), a, bb, cc);
        return d == 2 ? v + -1.0 * w0[cc] : v;
    };
    const double du = div_c(U(um, 0, i + 1, j, k) - U(um, 0, i, j, k), r0);
    const double dv = div_c(U(vm, 1, i, j + 1, k) - U(vm, 1, i, j, k), r1);
    double divu = du + dv + div_c(U(wm, 2, i, j, k + 1) - U(wm, 2, i, j, k), r2);
    // planar: ModifyScalForce adds the divergence of w0_cart (Source/MaestroForce.cpp:413-441);
    // spherical on uniform bins, div w0 of the shells on the cells (:283-305; sph == 2)
    if (!sph) divu += div_c(at(VW(F_W0CART), i, j, k + 1, 2) - at(VW(F_W0CART), i, j, k, 2), r2);
    if (sph == 2) divu = divu + at(VW(F_DIVW0), i, j, k);
    const double fb = at(AW(A_AFORCE), i, j, k);
    at(AW(A_ASOLD), i, j, k, comp) += at(AW(A_AS), i, j, k) - divu * fb;
    if (want_u && fb != 0.0 && !sph) {  // spherical: k_adj_pert_u_sph
        const double s = at(AW(A_WSOLD), i, j, k, comp), s0 = s0a[k];
        const double gx = s * fb / r0.y, gy = s * fb / r1.y;
        atomicAdd(&at(AW(A_AUMAC0), i + 1, j, k), -gx);
        atomicAdd(&at(AW(A_AUMAC0), i, j, k), gx);
        atomicAdd(&at(AW(A_AUMAC1), i, j + 1, k), -gy);
        atomicAdd(&at(AW(A_AUMAC1), i, j, k), gy);
        const int kp = k + 1 > domhi ? (zper ? domlo : domhi) : k + 1;
        atomicAdd(&at(AW(A_AUMAC2), i, j, k + 1), -(s - s0 + s0e[kp]) * fb / r2.y);
        atomicAdd(&at(AW(A_AUMAC2), i, j, k), (s - s0 + s0e[k]) * fb / r2.y);
    }
}

// Transverse coefficients transposed (k_transverse_coeffs: per cell c and direction t,
// dt6/h_t (u_t(c+e_t) + u_t(c)) and dt4/h_t (...)), gathered per t-face from the two
// cells that read it: the adjoints of F_TCOEF are in A_ATCOEF, the face-velocity adjoint
// is added to slot ts + T.
template <int T>
__global__ void k_adj_tcoef(KARGS, int ts, double dt6h, double dt4h) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int ti = T == 0, tj = T == 1, tk = T == 2;
    const FabView a = AW(A_ATCOEF);
    const double g = dt6h * (at(a, i, j, k, T) + at(a, i - ti, j - tj, k - tk, T)) +
                     dt4h * (at(a, i, j, k, 3 + T) + at(a, i - ti, j - tj, k - tk, 3 + T));
    at(AW(ts + T), i, j, k) += g;
}

// ------------------------------------------------------------------ VelPred^T, MakeUtrans^T
// k_vp_velocities transposed (valid D-faces): umac = Riemann(ml, mr) with
// ml = SL_D(D) - tc(3+T1) dq1 - tc(3+T2) dq2 + dt/2 f (the force is state- and
// velocity-independent here).
template <int D>
__global__ void k_adj_vp_velocities(KARGS, double dt2, double rel_eps) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    constexpr int T1 = D == 0 ? 1 : 0, T2 = D == 2 ? 1 : 2;
    constexpr int a1i = T1 == 0, a1j = T1 == 1, a1k = T1 == 2;
    constexpr int a2i = T2 == 0, a2j = T2 == 1, a2k = T2 == 2;
    const int il = i - di, jl = j - dj, kl = k - dk;
    const double vb = at(AW(A_AUMAC0 + D), i, j, k);
    if (vb == 0.0) return;
    const FabView tc = VW(F_TCOEF);
    const FabView q1 = VW(Q_FIELD(D, T1)), q2 = VW(Q_FIELD(D, T2));
    const FabView f = VW(F_VELFORCE);
    const double dq1l = at(q1, il + a1i, jl + a1j, kl + a1k) - at(q1, il, jl, kl);
    const double dq2l = at(q2, il + a2i, jl + a2j, kl + a2k) - at(q2, il, jl, kl);
    const double dq1r = at(q1, i + a1i, j + a1j, k + a1k) - at(q1, i, j, k);
    const double dq2r = at(q2, i + a2i, j + a2j, k + a2k) - at(q2, i, j, k);
    const double ml = at(VW(F_SL0 + D), i, j, k, D) - at(tc, il, jl, kl, 3 + T1) * dq1l -
                      at(tc, il, jl, kl, 3 + T2) * dq2l + dt2 * at(f, il, jl, kl, D);
    const double mr = at(VW(F_SR0 + D), i, j, k, D) - at(tc, i, j, k, 3 + T1) * dq1r -
                      at(tc, i, j, k, 3 + T2) * dq2r + dt2 * at(f, i, j, k, D);
    const double w0c = D == 2 ? at(VW(F_W0CART), i, j, k, 2) : 0.0;
    const int pick = riemann_pick(ml, mr, w0c, D == 2, rel_eps);
    if (pick == 0) return;
    const FabView qa1 = AW(AQ_SLOT(D, T1)), qa2 = AW(AQ_SLOT(D, T2)), atc = AW(A_ATCOEF);
    if (pick == 1) {
        at(AW(A_ASL0 + D), i, j, k, D) += vb;
        double c1 = at(tc, il, jl, kl, 3 + T1) * vb, c2 = at(tc, il, jl, kl, 3 + T2) * vb;
        atomicAdd(&at(qa1, il + a1i, jl + a1j, kl + a1k), -c1);
        atomicAdd(&at(qa1, il, jl, kl), c1);
        atomicAdd(&at(qa2, il + a2i, jl + a2j, kl + a2k), -c2);
        atomicAdd(&at(qa2, il, jl, kl), c2);
        atomicAdd(&at(atc, il, jl, kl, 3 + T1), -vb * dq1l);
        atomicAdd(&at(atc, il, jl, kl, 3 + T2), -vb * dq2l);
    } else {
        at(AW(A_ASR0 + D), i, j, k, D) += vb;
        double c1 = at(tc, i, j, k, 3 + T1) * vb, c2 = at(tc, i, j, k, 3 + T2) * vb;
        atomicAdd(&at(qa1, i + a1i, j + a1j, k + a1k), -c1);
        atomicAdd(&at(qa1, i, j, k), c1);
        atomicAdd(&at(qa2, i + a2i, j + a2j, k + a2k), -c2);
        atomicAdd(&at(qa2, i, j, k), c2);
        atomicAdd(&at(atc, i, j, k, 3 + T1), -vb * dq1r);
        atomicAdd(&at(atc, i, j, k, 3 + T2), -vb * dq2r);
    }
}

// k_vp_transverse<C, D> transposed: component C on D-faces corrected in T = 3 - C - D,
// upwinded by utrans_D.
template <int C, int D>
__global__ void k_adj_vp_transverse(KARGS, long long epsb) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int T = 3 - C - D;
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    constexpr int ti = T == 0, tj = T == 1, tk = T == 2;
    const int il = i - di, jl = j - dj, kl = k - dk;
    const double qb = at(AW(AQ_SLOT(C, D)), i, j, k);
    if (qb == 0.0) return;
    double wl, wr;
    upwind_w_vp(at(VW(F_UTRANS0 + D), i, j, k), epsb, wl, wr);
    const double la = wl * qb, ra = wr * qb;
    at(AW(A_ASL0 + D), i, j, k, C) += la;
    at(AW(A_ASR0 + D), i, j, k, C) += ra;
    const FabView tc = VW(F_TCOEF), s = VW(F_SIMH0 + T), sh = AW(A_ASIMH0 + T), atc = AW(A_ATCOEF);
    const double cl = at(tc, il, jl, kl, T) * la, cr = at(tc, i, j, k, T) * ra;
    atomicAdd(&at(sh, il + ti, jl + tj, kl + tk, C), -cl);
    atomicAdd(&at(sh, il, jl, kl, C), cl);
    atomicAdd(&at(sh, i + ti, j + tj, k + tk, C), -cr);
    atomicAdd(&at(sh, i, j, k, C), cr);
    atomicAdd(&at(atc, il, jl, kl, T), -la * (at(s, il + ti, jl + tj, kl + tk, C) - at(s, il, jl, kl, C)));
    atomicAdd(&at(atc, i, j, k, T), -ra * (at(s, i + ti, j + tj, k + tk, C) - at(s, i, j, k, C)));
}

// k_utrans<D> transposed (valid D-faces, ppm_type 1): utrans = Riemann(Ip(il), Im(i)) of
// the D component traced along D; its adjoint joins VelPred's at SL_D / SR_D comp D.
template <int D>
__global__ void k_adj_utrans(KARGS, double rel_eps) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const double vb = at(AW(A_AUTRANS0 + D), i, j, k);
    if (vb == 0.0) return;
    const double l = at(VW(F_IPC0 + D), i - di, j - dj, k - dk, D);
    const double r = at(VW(F_IMC0 + D), i, j, k, D);
    const double w0c = D == 2 ? at(VW(F_W0CART), i, j, k, 2) : 0.0;
    const int pick = riemann_pick(l, r, w0c, D == 2, rel_eps);
    if (pick == 1) at(AW(A_ASL0 + D), i, j, k, D) += vb;
    else if (pick == 2) at(AW(A_ASR0 + D), i, j, k, D) += vb;
}

// k_vp_interface<D> transposed (ppm_type 1): simh_D(n) = upwind by utrans_D of
// (Ip_n(il), Im_n(i)) for n != D.
template <int D>
__global__ void k_adj_vp_interface(KARGS, long long epsb) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    double wl, wr;
    upwind_w_vp(at(VW(F_UTRANS0 + D), i, j, k), epsb, wl, wr);
    const FabView sh = AW(A_ASIMH0 + D), L = AW(A_ASL0 + D), Rr = AW(A_ASR0 + D);
    for (int n = 0; n < 3; ++n) {
        if (n == D) continue;
        const double sb = at(sh, i, j, k, n);
        at(L, i, j, k, n) += wl * sb;
        at(Rr, i, j, k, n) += wr * sb;
    }
}

// sum over the region of sum_n A(n) B(n): one partial sum per block, then a fixed-order
// reduction of the partials (the same bits on every run)
__global__ void k_adj_dot(const RegionBox* __restrict__ R, int ne, long total, const FabView* __restrict__ V, int nb,
                          int fa, int fb, int nc, double* __restrict__ part) {
    __shared__ double sh[TPB];
    const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (gid < total) {
        const int e = find_box(R, ne, gid);
        const int b = R[e].b;
        int i, j, k;
        region_ijk(R[e], gid - R[e].start, i, j, k);
        const FabView A = V[fa * nb + b], B = V[fb * nb + b];
        for (int n = 0; n < nc; ++n) v += at(A, i, j, k, n) * at(B, i, j, k, n);
    }
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = TPB / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_sum_parts(const double* __restrict__ part, long n, double* __restrict__ out) {
    __shared__ double sh[TPB];
    double v = 0.0;
    for (long t = threadIdx.x; t < n; t += TPB) v += part[t];
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = TPB / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

// ------------------------------------------------------------------ host wrappers
void adj_update(Ctx& c) { launch(c, rg_grow(c, 0), 1, k_adj_update, c.V(), c.nspec); }

void adj_flux(Ctx& c, int want_u) {
    const double *r0 = c.b1("rho0_old"), *r0e = c.b1("rho0_edge_old");
    const double *h0 = c.b1("rhoh0_old"), *h0e = c.b1("rhoh0_edge_old");
    const int ns = c.nspec;
    const int sph = c.sph ? 1 : 0;
    launch(c, rg_grow(c, 0, 0), 1, k_adj_flux<0>, c.V(), ns, c.P.dt / c.P.dx[0], r0, r0, h0, h0, want_u, sph);
    launch(c, rg_grow(c, 0, 1), 1, k_adj_flux<1>, c.V(), ns, c.P.dt / c.P.dx[1], r0, r0, h0, h0, want_u, sph);
    launch(c, rg_grow(c, 0, 2), 1, k_adj_flux<2>, c.V(), ns, c.P.dt / c.P.dx[2], r0e, r0e, h0e, h0e, want_u, sph);
}

template <int D, int T>
static void adj_transverse_launch(Ctx& c, long long eb, int want_u, const BCRecD& bc) {
    constexpr int O = 3 - D - T;
    int glo[3] = {0, 0, 0}, ghi[3] = {0, 0, 0};
    glo[O] = 1;
    ghi[O] = 1;
    ghi[D] = 1;
    launch(c, region(c, glo[0], glo[1], glo[2], ghi[0], ghi[1], ghi[2], -1), 1, k_adj_es_transverse<D, T>, c.V(), eb,
           want_u, bc.lo[D], bc.hi[D], c.P.dom_lo[D], c.P.dom_hi[D]);
}

template <int D>
static void adj_predictor_launch(Ctx& c, const BCRecD& bc) {
    int glo[3] = {1, 1, 1};
    glo[D] = 0;
    launch(c, region(c, glo[0], glo[1], glo[2], 1, 1, 1, -1), 1, k_adj_es_predictor<D>, c.V(), bc.lo[D], bc.hi[D],
           c.P.dom_lo[D], c.P.dom_hi[D]);
}

// PPM^T of component sc of field fs along D (ppm_type 1, interior form): adjoints of
// Ip / Im from component lc of A_ASL0+D / A_ASR0+D, cell adjoints into slot ts comp tc.
// faces: recompute the interface values F_FACE0+D (0: they hold the forward's already).
template <int D, int UMAC>
static void adj_ppm_launch(Ctx& c, int fs, int sc, int lc, int ts, int tc, double* dir, size_t dir_bytes,
                          int want_u, int faces, const BCRecD& bc) {
    if (c.P.ppm_type == 2) {  // scalars (UMAC = 1), no ext_dir / hoextrap side
        if (!c.dry) cudaMemsetAsync(dir, 0, dir_bytes, c.stream);
        int g[3] = {1, 1, 1};
        g[D] = 2;
        launch(c, rg_grow(c, 1), 1, k_adj_ppm2_cell<D>, c.V(), fs, sc, lc, ts, tc, dbits_host(c.P.rel_eps),
               c.P.dt / c.P.dx[D], want_u);
        launch(c, region(c, g[0], g[1], g[2], g[0], g[1], g[2], D), 1, k_adj_ppm2_face<D>, c.V(), fs, sc, ts, tc,
               make_recip(6.0));
        return;
    }
    ppm_faces(c, D, fs, sc, faces);
    if (!c.dry) cudaMemsetAsync(dir, 0, dir_bytes, c.stream);
    const long long eb = dbits_host(c.P.rel_eps);
    const RecipC r6 = make_recip(6.0);
    // the forward's boundary stencils (ppm_any): ext_dir / hoextrap sides
    auto ext = [](int t) { return (t == BC_EXT_DIR || t == BC_HOEXTRAP) ? 1 : 0; };
    const int le = ext(bc.lo[D]), he = ext(bc.hi[D]), dl = c.P.dom_lo[D], dh = c.P.dom_hi[D];
    launch(c, rg_grow(c, 1), 1, k_adj_ppm_cell<D, UMAC>, c.V(), fs, sc, lc, ts, tc, eb, c.P.dt / c.P.dx[D], want_u,
           le, he, dl, dh, r6);
    launch(c, region(c, 1, 1, 1, 1, 1, 1, D), 1, k_adj_ppm_face<D>, c.V(), fs, sc, ts, tc, r6, le, he, dl, dh);
    int glo[3] = {1, 1, 1};
    glo[D] = 2;
    launch(c, region(c, glo[0], glo[1], glo[2], glo[0], glo[1], glo[2], -1), 1, k_adj_dsvl<D>, c.V(), fs, sc, ts, tc);
}

// MakeEdgeScal^T of component comp of field fs (advective form, ppm_type 1): from the
// edge-state adjoints A_AEDGE0..2 (comp) into A_AS (and A_AFORCE unless force_zero).
// dir: the storage of A_ASM / A_ASP / A_ADSVL, cleared before each direction.  want_u
// also accumulates the face-velocity adjoints (A_AUMAC0..2, A_ATCOEF); it needs the
// forward F_Q / F_SIMH fields of this component.  F_FACE0..2 must hold this component's
// forward interface values.
void adj_edge_scal(Ctx& c, int fs, int comp, int force_zero, double* dir, size_t dir_bytes, int want_u) {
    const long long eb = dbits_host(c.P.rel_eps);
    const double dt2 = 0.5 * c.P.dt;
    const BCRecD& bc = bcs_host(c, BCS_S)[comp];  // the forward's edge-state BCs of comp
    const int *lo = c.P.dom_lo, *hi = c.P.dom_hi;
    launch(c, rg_grow(c, 0, 0), 1, k_adj_es_edges<0>, c.V(), comp, force_zero, dt2, eb, want_u, bc.lo[0], bc.hi[0],
           lo[0], hi[0]);
    launch(c, rg_grow(c, 0, 1), 1, k_adj_es_edges<1>, c.V(), comp, force_zero, dt2, eb, want_u, bc.lo[1], bc.hi[1],
           lo[1], hi[1]);
    launch(c, rg_grow(c, 0, 2), 1, k_adj_es_edges<2>, c.V(), comp, force_zero, dt2, eb, want_u, bc.lo[2], bc.hi[2],
           lo[2], hi[2]);
    adj_transverse_launch<0, 1>(c, eb, want_u, bc);
    adj_transverse_launch<0, 2>(c, eb, want_u, bc);
    adj_transverse_launch<1, 0>(c, eb, want_u, bc);
    adj_transverse_launch<1, 2>(c, eb, want_u, bc);
    adj_transverse_launch<2, 0>(c, eb, want_u, bc);
    adj_transverse_launch<2, 1>(c, eb, want_u, bc);
    adj_predictor_launch<0>(c, bc);
    adj_predictor_launch<1>(c, bc);
    adj_predictor_launch<2>(c, bc);
    adj_ppm_launch<0, 1>(c, fs, comp, 0, A_AS, 0, dir, dir_bytes, want_u, 0, bc);
    adj_ppm_launch<1, 1>(c, fs, comp, 0, A_AS, 0, dir, dir_bytes, want_u, 0, bc);
    adj_ppm_launch<2, 1>(c, fs, comp, 0, A_AS, 0, dir, dir_bytes, want_u, 0, bc);
}

void adj_fill_boundary(Ctx& c, int slot, int nc, int ng, int nodal) {
    const CopyTable& ct = copy_table(c, ng, nodal);
    if (ct.total == 0 || c.dry) return;
    unsigned grid = (unsigned)((ct.total + TPB - 1) / TPB);
    k_adj_fill_boundary<<<grid, TPB, 0, c.stream>>>(ct.d, (int)ct.h.size(), ct.total, c.V(), c.nb, F_USER + slot, nc);
    c.launches++;
}

// PhysBC^T of component n of adjoint slot `slot` (cell-centred, ng ghost cells) under the
// BCs bc, the transpose of phys_fill: every non-periodic direction, last one first
void adj_phys_fill(Ctx& c, int slot, int n, int ng, const BCRecD& bc) {
    for (int d = 2; d >= 0; --d) {
        if (c.per[d] || d >= c.ndim) continue;
        launch(c, region(c, ng, ng, ng, ng, ng, ng, -1, d), 1, k_adj_phys_fill, c.V(), slot, n, bc, d,
               c.P.dom_lo[d], c.P.dom_hi[d]);
    }
}

void adj_convert_x(Ctx& c, int comp) { launch(c, rg_grow(c, 0), 1, k_adj_x, c.V(), comp); }

void adj_pert_force(Ctx& c, int comp, int want_u) {
    const double* s0 = c.b1(comp == RHO ? "rho0_old" : "rhoh0_old");
    const double* s0e = c.b1(comp == RHO ? "rho0_edge_old" : "rhoh0_edge_old");
    launch(c, rg_grow(c, 0), 1, k_adj_pert, c.V(), comp, s0, s0e, make_recip(c.P.dx[0]), make_recip(c.P.dx[1]),
           make_recip(c.P.dx[2]), c.P.dom_lo[2], c.P.dom_hi[2], want_u, c.b1("w0"),
           c.sph ? (c.geo.exact ? 1 : 2) : 0, c.per[2] ? 1 : 0);
}

// F_TCOEF^T into face slots ts .. ts+2 (A_AUMAC0 or A_AUTRANS0)
void adj_tcoef(Ctx& c, int ts) {
    const double dt6 = c.P.dt / 6.0, dt4 = 0.25 * c.P.dt;
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 0), 1, k_adj_tcoef<0>, c.V(), ts, dt6 / c.P.dx[0], dt4 / c.P.dx[0]);
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 1), 1, k_adj_tcoef<1>, c.V(), ts, dt6 / c.P.dx[1], dt4 / c.P.dx[1]);
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 2), 1, k_adj_tcoef<2>, c.V(), ts, dt6 / c.P.dx[2], dt4 / c.P.dx[2]);
}

template <int C, int D>
static void adj_vp_transverse_launch(Ctx& c, long long eb) {
    int glo[3] = {0, 0, 0}, ghi[3] = {0, 0, 0};
    glo[C] = 1;
    ghi[C] = 1;
    ghi[D] = 1;
    launch(c, region(c, glo[0], glo[1], glo[2], ghi[0], ghi[1], ghi[2], -1), 1, k_adj_vp_transverse<C, D>, c.V(), eb);
}

template <int D>
static void adj_vp_interface_launch(Ctx& c, long long eb) {
    int glo[3] = {1, 1, 1};
    glo[D] = 0;
    launch(c, region(c, glo[0], glo[1], glo[2], 1, 1, 1, -1), 1, k_adj_vp_interface<D>, c.V(), eb);
}

// VelPred^T then MakeUtrans^T (ppm_type 1): from the MAC-velocity adjoints A_AUMAC0..2
// (valid faces) into the cell-velocity adjoint A_AUT (3 components, with ghost cells).
// The forward fields of AdvancePremac (F_UTILDE, F_UFULL, F_TRC, F_IPC / F_IMC, F_UTRANS,
// F_TCOEF of utrans, F_SL / F_SR / F_SIMH, F_Q) must be current.  A_ATCOEF, A_AUTRANS,
// A_AUT and the per-direction scratch must be zero.
void adj_vel_pred(Ctx& c, double* dir, size_t dir_bytes) {
    const long long eb = dbits_host(c.P.rel_eps);
    const double dt2 = 0.5 * c.P.dt, re = c.P.rel_eps;
    launch(c, rg_grow(c, 0, 0), 1, k_adj_vp_velocities<0>, c.V(), dt2, re);
    launch(c, rg_grow(c, 0, 1), 1, k_adj_vp_velocities<1>, c.V(), dt2, re);
    launch(c, rg_grow(c, 0, 2), 1, k_adj_vp_velocities<2>, c.V(), dt2, re);
    adj_vp_transverse_launch<0, 1>(c, eb);
    adj_vp_transverse_launch<0, 2>(c, eb);
    adj_vp_transverse_launch<1, 0>(c, eb);
    adj_vp_transverse_launch<1, 2>(c, eb);
    adj_vp_transverse_launch<2, 0>(c, eb);
    adj_vp_transverse_launch<2, 1>(c, eb);
    adj_tcoef(c, A_AUTRANS0);
    for (int d = 0; d < 3; ++d) adj_fill_boundary(c, A_AUTRANS0 + d, 1, 1, d);
    launch(c, rg_grow(c, 0, 0), 1, k_adj_utrans<0>, c.V(), re);
    launch(c, rg_grow(c, 0, 1), 1, k_adj_utrans<1>, c.V(), re);
    launch(c, rg_grow(c, 0, 2), 1, k_adj_utrans<2>, c.V(), re);
    adj_vp_interface_launch<0>(c, eb);
    adj_vp_interface_launch<1>(c, eb);
    adj_vp_interface_launch<2>(c, eb);
    for (int cc = 0; cc < 3; ++cc) {
        adj_ppm_launch<0, 0>(c, F_UTILDE, cc, cc, A_AUT, cc, dir, dir_bytes, 1, 1, c.bcs_u[cc]);
        adj_ppm_launch<1, 0>(c, F_UTILDE, cc, cc, A_AUT, cc, dir, dir_bytes, 1, 1, c.bcs_u[cc]);
        adj_ppm_launch<2, 0>(c, F_UTILDE, cc, cc, A_AUT, cc, dir, dir_bytes, 1, 1, c.bcs_u[cc]);
    }
}

// ModifyScalForce's face-velocity adjoint, spherical, fullform 0 (k_modify_scal_force_sph,
// valid cells): f += -div(s0_face u) - (s - s0) div u, s0_face the average of the two
// cells' s0 (the cell's own at the domain edge), s0 the Cartesian base state in field s0c.
__global__ void k_adj_pert_u_sph(KARGS, int comp, int s0c, double dx0, double dx1, double dx2, int lo0, int lo1,
                                 int lo2, int hi0, int hi1, int hi2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const double fb = at(AW(A_AFORCE), i, j, k);
    if (fb == 0.0) return;
    const FabView s0a = VW(s0c);
    const double s = at(s0a, i, j, k);
    const double c = at(AW(A_WSOLD), i, j, k, comp) - s;
    const double sxh = i < hi0 ? 0.5 * (s + at(s0a, i + 1, j, k)) : s;
    const double sxl = i > lo0 ? 0.5 * (s + at(s0a, i - 1, j, k)) : s;
    const double syh = j < hi1 ? 0.5 * (s + at(s0a, i, j + 1, k)) : s;
    const double syl = j > lo1 ? 0.5 * (s + at(s0a, i, j - 1, k)) : s;
    const double szh = k < hi2 ? 0.5 * (s + at(s0a, i, j, k + 1)) : s;
    const double szl = k > lo2 ? 0.5 * (s + at(s0a, i, j, k - 1)) : s;
    atomicAdd(&at(AW(A_AUMAC0), i + 1, j, k), -(sxh + c) * fb / dx0);
    atomicAdd(&at(AW(A_AUMAC0), i, j, k), (sxl + c) * fb / dx0);
    atomicAdd(&at(AW(A_AUMAC1), i, j + 1, k), -(syh + c) * fb / dx1);
    atomicAdd(&at(AW(A_AUMAC1), i, j, k), (syl + c) * fb / dx1);
    atomicAdd(&at(AW(A_AUMAC2), i, j, k + 1), -(szh + c) * fb / dx2);
    atomicAdd(&at(AW(A_AUMAC2), i, j, k), (szl + c) * fb / dx2);
}

// MakeRhoHForce's face-velocity adjoint (valid cells), the force's adjoint being scale times
// component comp of slot src.  Plane-parallel (k_rhoh_force): f = (w(k) + w(k+1))/2 gradp0,
// gradp0 as the forward forms it; spherical (k_rhoh_force_sph): f = div(u p0_face) - p0 div u,
// p0_face in F_S0MAC*.  F_P0CART (and plane-parallel F_RHO0CART, F_GRAVCART) current.
__global__ void k_adj_rhoh_force_u(KARGS, int src, int comp, double scale, int sph, int cutoff, int domhi, RecipC rdz,
                                   double dx0, double dx1, double dx2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const double fb = scale * at(AW(src), i, j, k, comp);
    if (fb == 0.0) return;
    const FabView p0c = VW(F_P0CART);
    if (!sph) {
        double gradp0;
        if (k < cutoff) gradp0 = at(VW(F_RHO0CART), i, j, k) * at(VW(F_GRAVCART), i, j, k, 2);
        else if (k == domhi) gradp0 = div_c(at(p0c, i, j, k) - at(p0c, i, j - 1, k), rdz);
        else gradp0 = div_c(at(p0c, i, j + 1, k) - at(p0c, i, j, k), rdz);
        const double g = 0.5 * gradp0 * fb;
        atomicAdd(&at(AW(A_AUMAC2), i, j, k), g);
        atomicAdd(&at(AW(A_AUMAC2), i, j, k + 1), g);
        return;
    }
    const double p0 = at(p0c, i, j, k);
    const FabView px = VW(F_S0MAC0), py = VW(F_S0MAC1), pz = VW(F_S0MAC2);
    atomicAdd(&at(AW(A_AUMAC0), i + 1, j, k), (at(px, i + 1, j, k) - p0) * fb / dx0);
    atomicAdd(&at(AW(A_AUMAC0), i, j, k), -(at(px, i, j, k) - p0) * fb / dx0);
    atomicAdd(&at(AW(A_AUMAC1), i, j + 1, k), (at(py, i, j + 1, k) - p0) * fb / dx1);
    atomicAdd(&at(AW(A_AUMAC1), i, j, k), -(at(py, i, j, k) - p0) * fb / dx1);
    atomicAdd(&at(AW(A_AUMAC2), i, j, k + 1), (at(pz, i, j, k + 1) - p0) * fb / dx2);
    atomicAdd(&at(AW(A_AUMAC2), i, j, k), -(at(pz, i, j, k) - p0) * fb / dx2);
}

void adj_flux_rhoh_u_sph(Ctx& c) {
    const int ex = c.geo.exact ? 1 : 0;
    launch(c, rg_grow(c, 0, 0), 1, k_adj_flux_rhoh_u_sph<0>, c.V(), c.P.dt / c.P.dx[0], ex);
    launch(c, rg_grow(c, 0, 1), 1, k_adj_flux_rhoh_u_sph<1>, c.V(), c.P.dt / c.P.dx[1], ex);
    launch(c, rg_grow(c, 0, 2), 1, k_adj_flux_rhoh_u_sph<2>, c.V(), c.P.dt / c.P.dx[2], ex);
}

void adj_pert_u_sph(Ctx& c, int comp, int s0c) {
    launch(c, rg_grow(c, 0), 1, k_adj_pert_u_sph, c.V(), comp, s0c, c.P.dx[0], c.P.dx[1], c.P.dx[2], c.P.dom_lo[0],
           c.P.dom_lo[1], c.P.dom_lo[2], c.P.dom_hi[0], c.P.dom_hi[1], c.P.dom_hi[2]);
}

void adj_rhoh_force_u(Ctx& c, int src, int comp, double scale) {
    launch(c, rg_grow(c, 0), 1, k_adj_rhoh_force_u, c.V(), src, comp, scale, c.sph ? 1 : 0,
           c.P.base_cutoff_density_coord, c.P.dom_hi[2], make_recip(c.P.dx[2]), c.P.dx[0], c.P.dx[1], c.P.dx[2]);
}

// ------------------------------------------------------------------ buoyancy
// k_umac_ghost transposed (one face direction dd): a ghost face the forward set to w times
// a source face passes w times its adjoint to the source and keeps none; one set to zero
// keeps none.  Every ghost and every source belongs to one thread of the launch.
__global__ void k_adj_umac_ghost(KARGS, int dd, int bclo, int bchi, int dlo, int dhi) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const int I = dd == 0 ? i : (dd == 1 ? j : k);
    if (I != dlo - 1 && I != dhi + 2) return;
    const int di = dd == 0, dj = dd == 1, dk = dd == 2;
    const FabView q[3] = {AW(A_AUMAC0), AW(A_AUMAC1), AW(A_AUMAC2)};
    auto move = [&](const FabView& f, int s, int t, double w) {  // ghost at offset s, source at t (in dd)
        double& g = at(f, i + s * di, j + s * dj, k + s * dk);
        const double a = g;
        g = 0.0;
        if (w != 0.0) at(f, i + t * di, j + t * dj, k + t * dk) += w * a;
    };
    if (I == dlo - 1) {
        for (int cc = 0; cc < 3; ++cc) switch (bclo) {
                case PB_INFLOW: move(q[cc], 0, 1, cc == dd ? 1.0 : 0.0); break;
                case PB_SLIPWALL:
                case PB_NOSLIPWALL: move(q[cc], 0, 0, 0.0); break;
                case PB_OUTFLOW: move(q[cc], 0, 1, 1.0); break;
                case PB_SYMMETRY: cc == dd ? move(q[dd], 0, 2, -1.0) : move(q[cc], 0, 1, 1.0); break;
                default: break;
            }
    } else {
        for (int cc = 0; cc < 3; ++cc) switch (bchi) {
                case PB_INFLOW: cc == dd ? move(q[dd], 0, -1, 1.0) : move(q[cc], -1, -1, 0.0); break;
                case PB_SLIPWALL:
                case PB_NOSLIPWALL: cc == dd ? move(q[dd], 0, 0, 0.0) : move(q[cc], -1, -1, 0.0); break;
                case PB_OUTFLOW: cc == dd ? move(q[dd], 0, -1, 1.0) : move(q[cc], -1, -2, 1.0); break;
                case PB_SYMMETRY: cc == dd ? move(q[dd], 0, -2, -1.0) : move(q[cc], -1, -2, 1.0); break;
                default: break;
            }
    }
}

// k_vp_velocities<D> (untraced forces) transposed with respect to the force: the face value
// is the left state ml (which carries + dt/2 f of cell il), the right state mr (+ dt/2 f of
// cell i) or zero, decided as the forward decides it, boundary faces included (outflow:
// min(mr, 0) on the low side, max(ml, 0) on the high side); valid faces.
template <int D>
__global__ void k_adj_vp_force(KARGS, double dt2, int bclo, int bchi, int domlo, int domhi, double rel_eps, int sph) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const double vb = at(AW(A_AUMAC0 + D), i, j, k);
    if (vb == 0.0) return;
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    constexpr int T1 = D == 0 ? 1 : 0, T2 = D == 2 ? 1 : 2;
    constexpr int a1i = T1 == 0, a1j = T1 == 1, a1k = T1 == 2;
    constexpr int a2i = T2 == 0, a2j = T2 == 1, a2k = T2 == 2;
    const int I = D == 0 ? i : (D == 1 ? j : k);
    const int il = i - di, jl = j - dj, kl = k - dk;
    const FabView tc = VW(F_TCOEF), f = VW(F_VELFORCE);
    const FabView q1 = VW(Q_FIELD(D, T1)), q2 = VW(Q_FIELD(D, T2));
    const double ml = at(VW(F_SL0 + D), i, j, k, D) -
                      at(tc, il, jl, kl, 3 + T1) * (at(q1, il + a1i, jl + a1j, kl + a1k) - at(q1, il, jl, kl)) -
                      at(tc, il, jl, kl, 3 + T2) * (at(q2, il + a2i, jl + a2j, kl + a2k) - at(q2, il, jl, kl)) +
                      dt2 * at(f, il, jl, kl, D);
    const double mr = at(VW(F_SR0 + D), i, j, k, D) -
                      at(tc, i, j, k, 3 + T1) * (at(q1, i + a1i, j + a1j, k + a1k) - at(q1, i, j, k)) -
                      at(tc, i, j, k, 3 + T2) * (at(q2, i + a2i, j + a2j, k + a2k) - at(q2, i, j, k)) +
                      dt2 * at(f, i, j, k, D);
    int side;  // 0: zero, 1: ml, 2: mr
    if (D < 2 && !sph) {
        const bool test = (ml <= 0.0 && mr >= 0.0) || (fabs(ml + mr) < rel_eps);
        side = test ? 0 : (0.5 * (ml + mr) > 0.0 ? 1 : 2);
    } else {
        const double w0c = sph ? at(VW(F_W0MAC0 + D), i, j, k) : at(VW(F_W0CART), i, j, k, 2);
        const bool test = (ml + w0c <= 0.0 && mr + w0c >= 0.0) || (fabs(ml + mr + 2.0 * w0c) < rel_eps);
        side = test ? 0 : (0.5 * (ml + mr) + w0c > 0.0 ? 1 : 2);
    }
    if (I == domlo) {
        if (bclo == PB_OUTFLOW) side = mr < 0.0 ? 2 : 0;
        else if (bclo != PB_INTERIOR) side = 0;
    } else if (I == domhi + 1) {
        if (bchi == PB_OUTFLOW) side = ml > 0.0 ? 1 : 0;
        else if (bchi != PB_INTERIOR) side = 0;
    }
    const FabView af = AW(A_AVELF);
    if (side == 1) atomicAdd(&at(af, il, jl, kl, D), dt2 * vb);
    else if (side == 2) atomicAdd(&at(af, i, j, k, D), dt2 * vb);
}

// MakeVelForce transposed with respect to the density (valid cells): f_d = (rho' g_d -
// gpi_d) / rho + terms free of rho, with rho' = rho - rho0 (0 below the buoyancy cutoff),
// so df_d/drho = ((rho >= cutoff ? rho0 : 0) g_d + gpi_d) / rho^2.  The plane-parallel
// gravity has its z component only (F_GRAVCART comps 0, 1 are zero).
__global__ void k_adj_vel_force(KARGS, double cutoff_rho) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView a = AW(A_AVELF), g = VW(F_GRAVCART), gp = VW(F_GPI);
    const double r = at(VW(F_SOLD), i, j, k, RHO);
    const double r0 = r < cutoff_rho ? 0.0 : at(VW(F_RHO0CART), i, j, k);
    double acc = 0.0;
    for (int d = 0; d < 3; ++d) acc += at(a, i, j, k, d) * (r0 * at(g, i, j, k, d) + at(gp, i, j, k, d));
    if (acc != 0.0) at(AW(A_ASOLD), i, j, k, RHO) += acc / (r * r);
}

// The MAC-velocity adjoint's ghost faces back onto the valid faces: FillUmacGhost^T per
// non-periodic direction (z, y, x: the reverse of the forward's order), then FillBoundary^T
void adj_umac_ghosts(Ctx& c) {
    for (int dd = 2; dd >= 0; --dd) {
        if (c.per[dd]) continue;
        launch(c, region(c, 1, 1, 1, 1, 1, 1, dd), 1, k_adj_umac_ghost, c.V(), dd, c.P.phys_bc_lo[dd],
               c.P.phys_bc_hi[dd], c.P.dom_lo[dd], c.P.dom_hi[dd]);
    }
    for (int d = 0; d < 3; ++d) adj_fill_boundary(c, A_AUMAC0 + d, 1, 1, d);
}

// From the valid-face MAC-velocity adjoints into the density adjoint: VelPred's final states
// with respect to the force, the force's FillPatch (BCS_U) transposed, MakeVelForce^T.
// AdvancePremac's forward fields of the step (F_SL*, F_SR*, F_Q*, F_TCOEF of utrans,
// F_VELFORCE, F_RHO0CART, F_GRAVCART, F_SOLD) must be current; A_AVELF must be zero.
void adj_vel_force(Ctx& c) {
    const double dt2 = 0.5 * c.P.dt, re = c.P.rel_eps;
    const int sph = c.sph ? 1 : 0;
    const int *lo = c.P.phys_bc_lo, *hi = c.P.phys_bc_hi, *dl = c.P.dom_lo, *dh = c.P.dom_hi;
    launch(c, rg_grow(c, 0, 0), 1, k_adj_vp_force<0>, c.V(), dt2, lo[0], hi[0], dl[0], dh[0], re, sph);
    launch(c, rg_grow(c, 0, 1), 1, k_adj_vp_force<1>, c.V(), dt2, lo[1], hi[1], dl[1], dh[1], re, sph);
    launch(c, rg_grow(c, 0, 2), 1, k_adj_vp_force<2>, c.V(), dt2, lo[2], hi[2], dl[2], dh[2], re, sph);
    for (int n = 0; n < 3; ++n) adj_phys_fill(c, A_AVELF, n, 1, c.bcs_u[n]);
    adj_fill_boundary(c, A_AVELF, 3, 1, -1);
    launch(c, rg_grow(c, 0), 1, k_adj_vel_force, c.V(), c.P.buoyancy_cutoff_factor * c.P.base_cutoff_density);
}

long adj_dot_parts(Ctx& c) { return (rg_grow(c, 0).total + TPB - 1) / TPB; }

// part: adj_dot_parts(c) doubles of scratch
void adj_dot(Ctx& c, int slot_a, int slot_b, int nc, double* part, double* d_out) {
    const RegionTable& rt = rg_grow(c, 0);
    if (rt.total == 0 || c.dry) return;
    const unsigned grid = (unsigned)((rt.total + TPB - 1) / TPB);
    k_adj_dot<<<grid, TPB, 0, c.stream>>>(rt.d, (int)rt.h.size(), rt.total, c.V(), c.nb, F_USER + slot_a,
                                          F_USER + slot_b, nc, part);
    k_sum_parts<<<1, TPB, 0, c.stream>>>(part, (long)grid, d_out);
    c.launches += 2;
}

}  // namespace madv
