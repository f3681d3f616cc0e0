// Kernels of the GB300 scalar-advection stage (3-D, plane-parallel base state), per level.
//
// Each reference ParallelFor of the stage becomes one launch over all boxes of the level
// (or one launch per box in the per-box mode).  The arithmetic of every element follows
// the reference expression for expression (same operands, same order, IEEE binary64,
// no FMA contraction: the library is built with --fmad=false), so results match the
// reference algorithm bit for bit.  What changes is the amount of FP64 work: GB300 issues
// FP64 at a small fraction of its FP32 rate, so every intermediate of the stage is
// computed once and stored, where the reference recomputes it:
//   * PPM: the limited interface value of each face is computed once per face (the
//     reference evaluates four van Leer slopes and two interface values per cell and
//     direction, and in MakeUtrans sweeps all three directions where one is used);
//   * constant quotients such as (dt/6)/dy are formed once on the host, where the
//     reference forms them per element (same IEEE operations, same values).
#include <cstdio>
#include <type_traits>

#include "madv_ctx.hpp"
#include "madv_exact.cuh"
#include "madv_launch.cuh"
#include "madv_ppm.cuh"

namespace madv {

// ============================================================ elementwise utilities
__global__ void k_set_val(KARGS, int f, double v, int c0, int nc) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView a = VW(f);
    for (int n = c0; n < c0 + nc; ++n) at(a, i, j, k, n) = v;
}

void set_val(Ctx& c, int fid, double v, int c0, int nc, int ngrow) {
    launch(c, rg_grow(c, ngrow, c.F[fid].spec.nodal), 1, k_set_val, c.V(), fid, v, c0, nc);
}

__global__ void k_copy(KARGS, int fd, int dc0, int fs, int sc0, int nc, int add) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView d = VW(fd), s = VW(fs);
    for (int n = 0; n < nc; ++n) {
        if (add) at(d, i, j, k, dc0 + n) += at(s, i, j, k, sc0 + n);
        else at(d, i, j, k, dc0 + n) = at(s, i, j, k, sc0 + n);
    }
}

static int nodal_of(const Ctx& c, int fid) { return fid < NF_INTERNAL ? c.F[fid].spec.nodal : -1; }

void copy_fab(Ctx& c, int dst, int dc0, int src, int sc0, int nc, int ngrow) {
    int nd = dst < NF_INTERNAL ? nodal_of(c, dst) : nodal_of(c, src);
    launch(c, rg_grow(c, ngrow, nd), 1, k_copy, c.V(), dst, dc0, src, sc0, nc, 0);
}

void add_fab(Ctx& c, int dst, int src, int nc, int ngrow) {
    launch(c, rg_grow(c, ngrow, nodal_of(c, dst)), 1, k_copy, c.V(), dst, 0, src, 0, nc, 1);
}

// Put1dArrayOnCart, planar (Source/MaestroFill3dData.cpp:79-93): valid cells only.
__global__ void k_put1d(KARGS, int f, const double* __restrict__ s0, int outcomp, int edge) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const int r = k;
    at(VW(f), i, j, k, outcomp) = edge ? half(s0[r] + s0[r + 1]) : s0[r];
}

void put1d(Ctx& c, int fid, const double* d_s0, int outcomp, int edge, int vec) {
    if (c.ndim == 2) return put1d_2d(c, fid, d_s0, outcomp, edge);
    if (c.sph) return put1d_sph(c, fid, d_s0, outcomp, edge, vec);
    launch(c, rg_grow(c, 0), 1, k_put1d, c.V(), fid, d_s0, outcomp, edge);
}

// ============================================================ ghost fills
__global__ void k_fill_boundary(const CopyDesc* __restrict__ D, int nd, long total, const FabView* __restrict__ V,
                                int nb, int f, int c0, int nc) {
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
    const FabView dst = V[f * nb + cd.dst_b];
    const FabView src = V[f * nb + cd.src_b];
    for (int n = c0; n < c0 + nc; ++n)
        at(dst, i, j, k, n) = at(src, i - cd.shift[0], j - cd.shift[1], k - cd.shift[2], n);
}

void fill_boundary(Ctx& c, int fid, int c0, int nc) {
    const FieldSpec& s = c.F[fid].spec;
    const CopyTable& ct = copy_table(c, s.ng, s.nodal);
    if (ct.total == 0 || c.dry) return;
    unsigned grid = (unsigned)((ct.total + TPB - 1) / TPB);
    k_fill_boundary<<<grid, TPB, 0, c.stream>>>(ct.d, (int)ct.h.size(), ct.total, c.V(), c.nb, fid, c0, nc);
    c.launches++;
}

// Physical-boundary fill of direction d (both sides) for a cell-centred field.  The
// definitions of the BC types match the oracle's restatement of fab_filcc (foextrap,
// hoextrap = quadratic face extrapolation in the first ghost, reflect_even/odd,
// ext_dir = 0 for velocities).
__global__ void k_phys_fill(KARGS, int f, int c0, int nc, const BCRecD* __restrict__ bcs, int bc_c0, int is_vel,
                            int state_c0, int d, int domlo, int domhi) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView q = VW(f);
    const int idx[3] = {i, j, k};
    const int m = idx[d];
    const int side = m < domlo ? 0 : 1;
    auto A = [&](int p, int n) -> double {
        int i2 = i, j2 = j, k2 = k;
        if (d == 0) i2 = p;
        else if (d == 1) j2 = p;
        else k2 = p;
        return at(q, i2, j2, k2, n);
    };
    for (int n = c0; n < c0 + nc; ++n) {
        const BCRecD bc = bcs[bc_c0 + n - c0];
        const int t = side == 0 ? bc.lo[d] : bc.hi[d];
        double v;
        if (t == BC_INT_DIR) continue;
        if (t == BC_FOEXTRAP) {
            v = A(side == 0 ? domlo : domhi, n);
        } else if (t == BC_HOEXTRAP) {
            if (side == 0) {
                if (m < domlo - 1) v = A(domlo, n);
                else if (domlo + 2 <= domhi) v = 0.125 * (15. * A(domlo, n) - 10. * A(domlo + 1, n) + 3. * A(domlo + 2, n));
                else v = half(3. * A(domlo, n) - A(domlo + 1, n));
            } else {
                if (m > domhi + 1) v = A(domhi, n);
                else if (domhi - 2 >= domlo) v = 0.125 * (15. * A(domhi, n) - 10. * A(domhi - 1, n) + 3. * A(domhi - 2, n));
                else v = half(3. * A(domhi, n) - A(domhi - 1, n));
            }
        } else if (t == BC_REFLECT_EVEN) {
            v = A(side == 0 ? 2 * domlo - 1 - m : 2 * domhi + 1 - m, n);
        } else if (t == BC_REFLECT_ODD) {
            v = -A(side == 0 ? 2 * domlo - 1 - m : 2 * domhi + 1 - m, n);
        } else {  // ext_dir: zero for velocities and Pi; scalars are rejected on the host
            v = 0.0;
        }
        (void)is_vel;
        (void)state_c0;
        at(q, i, j, k, n) = v;
    }
}

void phys_fill(Ctx& c, int fid, int c0, int nc, const BCRecD* bcs_d, int bc_c0, int is_vel, int state_c0) {
    const FieldSpec& s = c.F[fid].spec;
    for (int d = 0; d < 3; ++d) {
        if (c.per[d]) continue;
        const RegionTable& rt = region(c, s.ng, s.ng, s.ng, s.ng, s.ng, s.ng, s.nodal, d);
        launch(c, rt, 1, k_phys_fill, c.V(), fid, c0, nc, bcs_d, bc_c0, is_vel, state_c0, d, c.P.dom_lo[d],
               c.P.dom_hi[d]);
    }
}

void fill_patch(Ctx& c, int fid, int c0, int nc, int which_bcs, int bc_c0, int is_vel, int state_c0) {
    fill_boundary(c, fid, c0, nc);
    phys_fill(c, fid, c0, nc, bcs_dev(c, which_bcs), bc_c0, is_vel, state_c0);
}

// FillUmacGhost (Source/MaestroFillData.cpp:176-453): ghost faces behind physical
// boundaries, one face direction dd per launch (x, then y, then z, as the reference).
__global__ void k_umac_ghost(KARGS, int f0, int dd, int bclo, int bchi, int dlo, int dhi) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const int I = dd == 0 ? i : (dd == 1 ? j : k);
    if (I != dlo - 1 && I != dhi + 2) return;
    const int di = dd == 0, dj = dd == 1, dk = dd == 2;
    const FabView q[3] = {VW(f0), VW(f0 + 1), VW(f0 + 2)};
    if (I == dlo - 1) {
        switch (bclo) {
            case PB_INFLOW:
                for (int cc = 0; cc < 3; ++cc) at(q[cc], i, j, k) = cc == dd ? at(q[dd], i + di, j + dj, k + dk) : 0.0;
                break;
            case PB_SLIPWALL:
            case PB_NOSLIPWALL:
                for (int cc = 0; cc < 3; ++cc) at(q[cc], i, j, k) = 0.0;
                break;
            case PB_OUTFLOW:
                for (int cc = 0; cc < 3; ++cc) at(q[cc], i, j, k) = at(q[cc], i + di, j + dj, k + dk);
                break;
            case PB_SYMMETRY:
                for (int cc = 0; cc < 3; ++cc)
                    at(q[cc], i, j, k) = cc == dd ? -at(q[dd], i + 2 * di, j + 2 * dj, k + 2 * dk)
                                                  : at(q[cc], i + di, j + dj, k + dk);
                break;
            default: break;
        }
    } else {
        switch (bchi) {
            case PB_INFLOW:
                for (int cc = 0; cc < 3; ++cc) {
                    if (cc == dd) at(q[dd], i, j, k) = at(q[dd], i - di, j - dj, k - dk);
                    else at(q[cc], i - di, j - dj, k - dk) = 0.0;
                }
                break;
            case PB_SLIPWALL:
            case PB_NOSLIPWALL:
                for (int cc = 0; cc < 3; ++cc) {
                    if (cc == dd) at(q[dd], i, j, k) = 0.0;
                    else at(q[cc], i - di, j - dj, k - dk) = 0.0;
                }
                break;
            case PB_OUTFLOW:
                for (int cc = 0; cc < 3; ++cc) {
                    if (cc == dd) at(q[dd], i, j, k) = at(q[dd], i - di, j - dj, k - dk);
                    else at(q[cc], i - di, j - dj, k - dk) = at(q[cc], i - 2 * di, j - 2 * dj, k - 2 * dk);
                }
                break;
            case PB_SYMMETRY:
                for (int cc = 0; cc < 3; ++cc) {
                    if (cc == dd) at(q[dd], i, j, k) = -at(q[dd], i - 2 * di, j - 2 * dj, k - 2 * dk);
                    else at(q[cc], i - di, j - dj, k - dk) = at(q[cc], i - 2 * di, j - 2 * dj, k - 2 * dk);
                }
                break;
            default: break;
        }
    }
}

void fill_face_ghosts(Ctx& c, int f0) {
    for (int d = 0; d < 3; ++d) fill_boundary(c, f0 + d, 0, 1);
    for (int dd = 0; dd < 3; ++dd) {
        if (c.per[dd]) continue;
        const RegionTable& rt = region(c, 1, 1, 1, 1, 1, 1, dd);
        launch(c, rt, 1, k_umac_ghost, c.V(), f0, dd, c.P.phys_bc_lo[dd], c.P.phys_bc_hi[dd], c.P.dom_lo[dd],
               c.P.dom_hi[dd]);
    }
}

// Addw0, planar (Source/MaestroFill3dData.cpp:381-393)
__global__ void k_addw0(KARGS, int f, const double* __restrict__ w0, double mult) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    at(VW(f), i, j, k) += mult * w0[k];
}

void addw0(Ctx& c, int f0, double mult) {
    if (c.sph) return addw0_sph(c, f0, mult);
    if (c.ndim == 2) return addw0_2d(c, f0, mult);
    launch(c, region(c, 1, 1, 0, 1, 1, 0, 2), 1, k_addw0, c.V(), f0 + 2, (const double*)c.b1("w0"), mult);
}

// ============================================================ PPM
// Van Leer slope of each cell along D (Source/MaestroPPM.cpp:37-73).  The reference
// evaluates it four times per cell and direction; here once.
template <int D>
__global__ void k_dsvl(KARGS, int fs, int sc) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    at(VW(F_DSVL), i, j, k) = ppm_dsvl<D>(VW(fs), sc, i, j, k);
}

// Limited interface value of each face, once per face (the reference computes each face
// twice, as sp of one cell and sm of the next).
template <int D, int PPMT>
__global__ void k_ppm_face(KARGS, int fs, int sc, int ff, int lo_ext, int hi_ext, int domlo, int domhi, RecipC r6) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    at(VW(ff), i, j, k) = ppm_face_value<D, PPMT>(VW(fs), sc, VW(F_DSVL), i, j, k, lo_ext, hi_ext, domlo, domhi, r6);
}

// Characteristic-tracing coefficients.  They depend on the velocity only, so they are
// formed once per velocity field and direction and shared by every traced component
// (the reference forms them per component, cell and direction).
// Face-centred velocity (the is_umac case): one (A, B) per D-face.
template <int D>
__global__ void k_trace_face(KARGS, int fu, int fout, double dt, double dxd) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    double A, B;
    trace_coeffs(at(VW(fu), i, j, k), dt, dxd, A, B);
    const FabView o = VW(fout);
    at(o, i, j, k, 0) = A;
    at(o, i, j, k, 1) = B;
}

// Cell-centred velocity (the velocity predictions): (A, B) per cell for each direction d,
// from component d of the tracing velocity.
__global__ void k_trace_cell(KARGS, int fu, double dt, double dx0, double dx1, double dx2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView u = VW(fu), o = VW(F_TRC);
    const double dx[3] = {dx0, dx1, dx2};
    for (int d = 0; d < 3; ++d) {
        double A, B;
        trace_coeffs(at(u, i, j, k, d), dt, dx[d], A, B);
        at(o, i, j, k, 2 * d) = A;
        at(o, i, j, k, 2 * d + 1) = B;
    }
}

// Per-cell limiting and characteristic tracing (Source/MaestroPPM.cpp).
template <int D, int PPMT, int UMAC>
__global__ void k_ppm_cell(KARGS, int fs, int sc, int ff, int fu, int uc, int fip, int fim, int lo_ext, int hi_ext,
                           int domlo, int domhi, long long epsb, RecipC r6) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const FabView s = VW(fs);
    double sm, sp;
    ppm_cell_edges<D, PPMT>(s, sc, VW(ff), VW(F_DSVL), i, j, k, lo_ext, hi_ext, domlo, domhi, r6, sm, sp);
    const FabView u = VW(fu);
    double up, um, Ap, Bp, Am, Bm;
    if (UMAC) {
        const FabView T = VW(F_TRA0 + D);
        up = at(u, i + di, j + dj, k + dk);
        um = at(u, i, j, k);
        Ap = at(T, i + di, j + dj, k + dk, 0);
        Bp = at(T, i + di, j + dj, k + dk, 1);
        Am = at(T, i, j, k, 0);
        Bm = at(T, i, j, k, 1);
    } else {
        const FabView T = VW(F_TRC);
        up = um = at(u, i, j, k, uc);
        Ap = Am = at(T, i, j, k, 2 * D);
        Bp = Bm = at(T, i, j, k, 2 * D + 1);
    }
    double ip, im;
    ppm_trace(at(s, i, j, k, sc), sm, sp, up, um, Ap, Bp, Am, Bm, epsb, ip, im);
    at(VW(fip), i, j, k, D) = ip;
    at(VW(fim), i, j, k, D) = im;
}

// Limited slopes for ppm_type 0 (Maestro::Slopex/y/z, Source/MaestroSlopes.cpp:6-600).
template <int D>
__global__ void k_slope(KARGS, int fs, int sc, int fout, int oc, int ncomp, const BCRecD* __restrict__ bcs, int bc_c0,
                        int slope_order, int ilo, int ihi) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const FabView s = VW(fs);
    const FabView o = VW(fout);
    const int I = D == 0 ? i : (D == 1 ? j : k);
    for (int n = 0; n < ncomp; ++n) {
        auto S = SHIFT_S(s, sc + n);
        const int bclo = bcs[bc_c0 + n].lo[D], bchi = bcs[bc_c0 + n].hi[D];
        const bool lo_ext = (bclo == BC_EXT_DIR || bclo == BC_HOEXTRAP);
        const bool hi_ext = (bchi == BC_EXT_DIR || bchi == BC_HOEXTRAP);
        double out = 0.0;
        if (slope_order == 2) {
            double del = half(S(1) - S(-1));
            double dpls = 2.0 * (S(1) - S(0));
            double dmin = 2.0 * (S(0) - S(-1));
            double slim = mn(fabs(dpls), fabs(dmin));
            slim = dpls * dmin > 0.0 ? slim : 0.0;
            double sflag = copysign(1.0, del);
            out = sflag * mn(slim, fabs(del));
            if (lo_ext) {
                if (I == ilo - 1) {
                    out = 0.0;
                } else if (I == ilo) {
                    del = (S(1) + 3.0 * S(0) - 4.0 * S(-1)) / 3.0;
                    dpls = 2.0 * (S(1) - S(0));
                    dmin = 2.0 * (S(0) - S(-1));
                    slim = mn(fabs(dpls), fabs(dmin));
                    slim = dpls * dmin > 0.0 ? slim : 0.0;
                    sflag = copysign(1.0, del);
                    out = sflag * mn(slim, fabs(del));
                }
            }
            if (hi_ext) {
                if (I == ihi + 1) {
                    out = 0.0;
                } else if (I == ihi) {
                    del = -(S(-1) + 3.0 * S(0) - 4.0 * S(1)) / 3.0;
                    dpls = 2.0 * (S(0) - S(-1));
                    dmin = 2.0 * (S(1) - S(0));
                    slim = mn(fabs(dpls), fabs(dmin));
                    slim = dpls * dmin > 0.0 ? slim : 0.0;
                    sflag = copysign(1.0, del);
                    out = sflag * mn(slim, fabs(del));
                }
            }
        } else if (slope_order == 4) {
            double dcen = half(S(0) - S(-2));
            double dmin = 2.0 * (S(-1) - S(-2));
            double dpls = 2.0 * (S(0) - S(-1));
            double dlim = mn(fabs(dmin), fabs(dpls));
            dlim = dpls * dmin > 0.0 ? dlim : 0.0;
            double dflag = copysign(1.0, dcen);
            double dxl = dflag * mn(dlim, fabs(dcen));
            dcen = half(S(2) - S(0));
            dmin = 2.0 * (S(1) - S(0));
            dpls = 2.0 * (S(2) - S(1));
            dlim = mn(fabs(dmin), fabs(dpls));
            dlim = dpls * dmin > 0.0 ? dlim : 0.0;
            dflag = copysign(1.0, dcen);
            double dxr = dflag * mn(dlim, fabs(dcen));
            dcen = half(S(1) - S(-1));
            dmin = 2.0 * (S(0) - S(-1));
            dpls = 2.0 * (S(1) - S(0));
            dlim = mn(fabs(dmin), fabs(dpls));
            dlim = dpls * dmin > 0.0 ? dlim : 0.0;
            dflag = copysign(1.0, dcen);
            double ds = 4.0 / 3.0 * dcen - (dxr + dxl) / 6.0;
            out = dflag * mn(fabs(ds), dlim);
            // the x sweep tests the centred dlim where y and z test the one-sided slim
            if (lo_ext) {
                if (I == ilo - 1) {
                    out = 0.0;
                } else if (I == ilo) {
                    double del = -16.0 / 15.0 * S(-1) + 0.5 * S(0) + 2.0 / 3.0 * S(1) - 0.1 * S(2);
                    dmin = 2.0 * (S(0) - S(-1));
                    dpls = 2.0 * (S(1) - S(0));
                    double slim = mn(fabs(dpls), fabs(dmin));
                    slim = dpls * dmin > 0.0 ? (D == 0 ? dlim : slim) : 0.0;
                    double sflag = copysign(1.0, del);
                    out = sflag * mn(slim, fabs(del));
                } else if (I == ilo + 1) {
                    double del = -16.0 / 15.0 * S(-2) + 0.5 * S(-1) + 2.0 / 3.0 * S(0) - 0.1 * S(1);
                    dmin = 2.0 * (S(-1) - S(-2));
                    dpls = 2.0 * (S(0) - S(-1));
                    double slim = mn(fabs(dpls), fabs(dmin));
                    slim = dpls * dmin > 0.0 ? (D == 0 ? dlim : slim) : 0.0;
                    double sflag = copysign(1.0, del);
                    dxl = sflag * mn(slim, fabs(del));
                    ds = 4.0 / 3.0 * dcen - (dxr + dxl) / 6.0;
                    out = dflag * mn(fabs(ds), dlim);
                }
            }
            if (hi_ext) {
                if (I == ihi + 1) {
                    out = 0.0;
                } else if (I == ihi) {
                    double del = -(-16.0 / 15.0 * S(1) + 0.5 * S(0) + 2.0 / 3.0 * S(-1) - 0.1 * S(-2));
                    dmin = 2.0 * (S(0) - S(-1));
                    dpls = 2.0 * (S(1) - S(0));
                    double slim = mn(fabs(dpls), fabs(dmin));
                    slim = dpls * dmin > 0.0 ? (D == 0 ? dlim : slim) : 0.0;
                    double sflag = copysign(1.0, del);
                    out = sflag * mn(slim, fabs(del));
                } else if (I == ihi - 1) {
                    double del = -(-16.0 / 15.0 * S(2) + 0.5 * S(1) + 2.0 / 3.0 * S(0) - 0.1 * S(-1));
                    dmin = 2.0 * (S(1) - S(0));
                    dpls = 2.0 * (S(2) - S(1));
                    double slim = mn(fabs(dpls), fabs(dmin));
                    slim = dpls * dmin > 0.0 ? (D == 0 ? dlim : slim) : 0.0;
                    double sflag = copysign(1.0, del);
                    dxr = sflag * mn(slim, fabs(del));
                    ds = 4.0 / 3.0 * dcen - (dxl + dxr) / 6.0;
                    out = dflag * mn(fabs(ds), dlim);
                }
            }
        }
        at(o, i, j, k, oc + n) = out;
    }
}


static bool ext_like(int t) { return t == BC_EXT_DIR || t == BC_HOEXTRAP; }

// PPM of component sc of field fs in direction D into fip/fim comp D over the box grown
// by one cell.  umac: trace with the D-face velocity fu (coefficients F_TRA0+D), else
// with component uc of the cell velocity fu (coefficients F_TRC).
template <int D>
static void ppm_dir(Ctx& c, int fs, int sc, const BCRecD& bc, int fu, int uc, int umac, int fip, int fim) {
    const int lo_ext = ext_like(bc.lo[D]), hi_ext = ext_like(bc.hi[D]);
    if (ppm_sweep(c, D, fs, sc, fu, uc, umac, fip, fim, lo_ext, hi_ext)) return;
    const int dlo = c.P.dom_lo[D], dhi = c.P.dom_hi[D];
    const RecipC r6 = make_recip(6.0);
    const int gf = c.P.ppm_type == 2 ? 2 : 1;
    int glo[3] = {1, 1, 1}, ghi[3] = {1, 1, 1};
    if (c.P.ppm_type == 1) {
        glo[D] = 2;
        ghi[D] = 2;
        launch(c, region(c, glo[0], glo[1], glo[2], ghi[0], ghi[1], ghi[2], -1), 1, k_dsvl<D>, c.V(), fs, sc);
    }
    glo[D] = gf;
    ghi[D] = gf;
    const RegionTable& rf = region(c, glo[0], glo[1], glo[2], ghi[0], ghi[1], ghi[2], D);
    const int ff = F_FACE0 + D;
    if (c.P.ppm_type == 1)
        launch(c, rf, 1, k_ppm_face<D, 1>, c.V(), fs, sc, ff, lo_ext, hi_ext, dlo, dhi, r6);
    else
        launch(c, rf, 1, k_ppm_face<D, 2>, c.V(), fs, sc, ff, lo_ext, hi_ext, dlo, dhi, r6);
    const RegionTable& rc = rg_grow(c, 1);
    const long long eb = dbits_host(c.P.rel_eps);
    if (c.P.ppm_type == 1) {
        if (umac) launch(c, rc, 1, k_ppm_cell<D, 1, 1>, c.V(), fs, sc, ff, fu, uc, fip, fim, lo_ext, hi_ext, dlo, dhi, eb, r6);
        else launch(c, rc, 1, k_ppm_cell<D, 1, 0>, c.V(), fs, sc, ff, fu, uc, fip, fim, lo_ext, hi_ext, dlo, dhi, eb, r6);
    } else {
        if (umac) launch(c, rc, 1, k_ppm_cell<D, 2, 1>, c.V(), fs, sc, ff, fu, uc, fip, fim, lo_ext, hi_ext, dlo, dhi, eb, r6);
        else launch(c, rc, 1, k_ppm_cell<D, 2, 0>, c.V(), fs, sc, ff, fu, uc, fip, fim, lo_ext, hi_ext, dlo, dhi, eb, r6);
    }
}

static void ppm_any(Ctx& c, int d, int fs, int sc, const BCRecD& bc, int fu, int uc, int umac, int fip, int fim) {
    if (d == 0) ppm_dir<0>(c, fs, sc, bc, fu, uc, umac, fip, fim);
    else if (d == 1) ppm_dir<1>(c, fs, sc, bc, fu, uc, umac, fip, fim);
    else ppm_dir<2>(c, fs, sc, bc, fu, uc, umac, fip, fim);
}

// The first two launches of the ppm_type 1 sweep of ppm_dir (van Leer slopes into F_DSVL,
// and with `faces` the interface values into F_FACE0+d) for component sc of field fs,
// interior form: the reverse sweep reads them to recover the forward's limiter decisions.
void ppm_faces(Ctx& c, int d, int fs, int sc, int faces) {
    const RecipC r6 = make_recip(6.0);
    auto one = [&](auto dir) {
        constexpr int D = decltype(dir)::value;
        int glo[3] = {1, 1, 1};
        glo[D] = 2;
        launch(c, region(c, glo[0], glo[1], glo[2], glo[0], glo[1], glo[2], -1), 1, k_dsvl<D>, c.V(), fs, sc);
        if (faces)
            launch(c, region(c, 1, 1, 1, 1, 1, 1, D), 1, k_ppm_face<D, 1>, c.V(), fs, sc, F_FACE0 + D, 0, 0,
                   c.P.dom_lo[D], c.P.dom_hi[D], r6);
    };
    if (d == 0) one(std::integral_constant<int, 0>{});
    else if (d == 1) one(std::integral_constant<int, 1>{});
    else one(std::integral_constant<int, 2>{});
}

// tracing coefficients of the face velocity fields umac0..2 (or utrans0..2)
static void trace_coeffs_faces(Ctx& c, int fu0) {
    // faces lo-1 .. hi+2 along d, cells lo-1 .. hi+1 across
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 0), 1, k_trace_face<0>, c.V(), fu0, F_TRA0, c.P.dt, c.P.dx[0]);
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 1), 1, k_trace_face<1>, c.V(), fu0 + 1, F_TRA1, c.P.dt, c.P.dx[1]);
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 2), 1, k_trace_face<2>, c.V(), fu0 + 2, F_TRA2, c.P.dt, c.P.dx[2]);
}

static void slope_any(Ctx& c, int d, int fs, int sc, int fout, int oc, int ncomp, const BCRecD* bcs_d, int bc_c0) {
    const RegionTable& rc = rg_grow(c, 1);
    const int lo = c.P.dom_lo[d], hi = c.P.dom_hi[d], so = c.P.slope_order;
    if (d == 0) launch(c, rc, 1, k_slope<0>, c.V(), fs, sc, fout, oc, ncomp, bcs_d, bc_c0, so, lo, hi);
    else if (d == 1) launch(c, rc, 1, k_slope<1>, c.V(), fs, sc, fout, oc, ncomp, bcs_d, bc_c0, so, lo, hi);
    else launch(c, rc, 1, k_slope<2>, c.V(), fs, sc, fout, oc, ncomp, bcs_d, bc_c0, so, lo, hi);
}

// Transverse-correction coefficients of a face velocity field (u0..u2 = three D-face
// fields): per cell and direction t, (dt/6)/h_t * (u_t(c+e_t) + u_t(c)) and the same with
// dt/4.  These are the leading products of the reference's transverse expressions, e.g.
// (dt6/hy)*(vmac(i,j+1,k)+vmac(i,j,k)) (Source/MaestroMakeEdgeScalars.cpp:920-927,
// Source/MaestroVelPred.cpp:1166-1172), so forming them once keeps every result bitwise.
__global__ void k_transverse_coeffs(KARGS, int fu0, double dt6h0, double dt6h1, double dt6h2, double dt4h0,
                                    double dt4h1, double dt4h2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView o = VW(F_TCOEF);
    const FabView u0 = VW(fu0), u1 = VW(fu0 + 1), u2 = VW(fu0 + 2);
    const double s0 = at(u0, i + 1, j, k) + at(u0, i, j, k);
    const double s1 = at(u1, i, j + 1, k) + at(u1, i, j, k);
    const double s2 = at(u2, i, j, k + 1) + at(u2, i, j, k);
    at(o, i, j, k, 0) = dt6h0 * s0;
    at(o, i, j, k, 1) = dt6h1 * s1;
    at(o, i, j, k, 2) = dt6h2 * s2;
    at(o, i, j, k, 3) = dt4h0 * s0;
    at(o, i, j, k, 4) = dt4h1 * s1;
    at(o, i, j, k, 5) = dt4h2 * s2;
}

static void transverse_coeffs(Ctx& c, int fu0) {
    const double dt6 = c.P.dt / 6.0, dt4 = 0.25 * c.P.dt;
    launch(c, rg_grow(c, 1), 1, k_transverse_coeffs, c.V(), fu0, dt6 / c.P.dx[0], dt6 / c.P.dx[1], dt6 / c.P.dx[2],
           dt4 / c.P.dx[0], dt4 / c.P.dx[1], dt4 / c.P.dx[2]);
}

void edge_scal_coeffs(Ctx& c) {
    trace_coeffs_faces(c, F_UMAC0);
    transverse_coeffs(c, F_UMAC0);
}

// ============================================================ MakeUtrans
// Face kernel of Maestro::MakeUtrans, 3-D (Source/MaestroMakeUtrans.cpp:304-387, 419-502,
// 535-627).  Planar: the z solve tests the full velocity w + w0_cart.  The PPM of
// utilde component D along D (ufull tracing) is the same sweep VelPred needs, so it is
// stored where VelPred reads it (F_IPC0+D / F_IMC0+D, comp D) and not repeated there.
template <int D>
__global__ void k_utrans(KARGS, int ppm_type, double dt2dx, int bclo, int bchi, int domlo, int domhi, double rel_eps,
                         int sph) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const int I = D == 0 ? i : (D == 1 ? j : k);
    const FabView ut = VW(F_UTILDE);
    double l, r;
    if (ppm_type == 0) {
        const FabView uf = VW(F_UFULL);
        const FabView sl = VW(F_SLOPE);
        l = at(ut, i - di, j - dj, k - dk, D) + (0.5 - dt2dx * mx(0.0, at(uf, i - di, j - dj, k - dk, D))) * at(sl, i - di, j - dj, k - dk, 0);
        r = at(ut, i, j, k, D) - (0.5 + dt2dx * mn(0.0, at(uf, i, j, k, D))) * at(sl, i, j, k, 0);
    } else {
        l = at(VW(F_IPC0 + D), i - di, j - dj, k - dk, D);
        r = at(VW(F_IMC0 + D), i, j, k, D);
    }
    if (I == domlo) {
        switch (bclo) {
            case PB_INFLOW: l = at(ut, i - di, j - dj, k - dk, D); r = l; break;
            case PB_SLIPWALL: case PB_NOSLIPWALL: case PB_SYMMETRY: l = 0.0; r = 0.0; break;
            case PB_OUTFLOW: l = mn(r, 0.0); r = l; break;
            default: break;
        }
    } else if (I == domhi + 1) {
        switch (bchi) {
            case PB_INFLOW: l = at(ut, i + di, j + dj, k + dk, D); r = l; break;
            case PB_SLIPWALL: case PB_NOSLIPWALL: case PB_SYMMETRY: l = 0.0; r = 0.0; break;
            case PB_OUTFLOW: l = mx(l, 0.0); r = l; break;
            default: break;
        }
    }
    double v;
    if (D < 2 && !sph) {
        const bool test = (l <= 0.0 && r >= 0.0) || (fabs(l + r) < rel_eps);
        v = half(l + r) > 0.0 ? l : r;
        v = test ? 0.0 : v;
    } else {
        // planar z: the full velocity w + w0_cart; spherical (:368-377): + w0mac in every direction
        const double w0c = sph ? at(VW(F_W0MAC0 + D), i, j, k) : at(VW(F_W0CART), i, j, k, 2);
        const bool test = (l + w0c <= 0.0 && r + w0c >= 0.0) || (fabs(l + r + 2.0 * w0c) < rel_eps);
        v = half(l + r) + w0c > 0.0 ? l : r;
        v = test ? 0.0 : v;
    }
    at(VW(F_UTRANS0 + D), i, j, k) = v;
}

void make_utrans(Ctx& c) {
    if (c.ndim == 2) return make_utrans_2d_entry(c);
    const double dt2 = 0.5 * c.P.dt;
    if (c.P.ppm_type != 0)
        launch(c, rg_grow(c, 1), 1, k_trace_cell, c.V(), F_UFULL, c.P.dt, c.P.dx[0], c.P.dx[1], c.P.dx[2]);
    for (int d = 0; d < 3; ++d) {
        if (c.P.ppm_type == 0) {
            slope_any(c, d, F_UTILDE, d, F_SLOPE, 0, 1, bcs_dev(c, BCS_U), d);
        } else {
            ppm_any(c, d, F_UTILDE, d, c.bcs_u[d], F_UFULL, d, 0, F_IPC0 + d, F_IMC0 + d);
        }
        const RegionTable& rt = rg_grow(c, 0, d);
        const double dt2dx = dt2 / c.P.dx[d];
        const int bl = c.P.phys_bc_lo[d], bh = c.P.phys_bc_hi[d], dl = c.P.dom_lo[d], dh = c.P.dom_hi[d];
        const int sph = c.sph;
        if (d == 0) launch(c, rt, 1, k_utrans<0>, c.V(), c.P.ppm_type, dt2dx, bl, bh, dl, dh, c.P.rel_eps, sph);
        else if (d == 1) launch(c, rt, 1, k_utrans<1>, c.V(), c.P.ppm_type, dt2dx, bl, bh, dl, dh, c.P.rel_eps, sph);
        else launch(c, rt, 1, k_utrans<2>, c.V(), c.P.ppm_type, dt2dx, bl, bh, dl, dh, c.P.rel_eps, sph);
    }
}

// ============================================================ MakeVelForce
// Maestro::MakeVelForce, planar (Source/MaestroForce.cpp:100-126)
__global__ void k_vel_force(KARGS, double cutoff_rho, int domhi, RecipC r2dz, int fe) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView gpi = VW(F_GPI), rho = VW(F_SOLD), vf = VW(F_VELFORCE);
    const double r = at(rho, i, j, k, RHO);
    double rhopert = r - at(VW(F_RHO0CART), i, j, k);
    if (r < cutoff_rho) rhopert = 0.0;
    for (int dim = 0; dim < 2; ++dim) at(vf, i, j, k, dim) = -at(gpi, i, j, k, dim) / r;
    double f2 = (rhopert * at(VW(F_GRAVCART), i, j, k, 2) - at(gpi, i, j, k, 2)) / r - at(VW(F_W0FCART), i, j, k, 2);
    if (k <= -1 || k >= domhi) {
    } else {
        const FabView we = VW(fe + 2), w0 = VW(F_W0CART);
        f2 -= div_c((at(we, i, j, k + 1) + at(we, i, j, k)) * (at(w0, i, j, k + 1, 2) - at(w0, i, j, k, 2)), r2dz);
    }
    at(vf, i, j, k, 2) = f2;
}

// valid cells of one level; F_GRAVCART and F_RHO0CART are filled by the caller
void make_vel_force(Ctx& c, int fe) {
    if (c.sph) return make_vel_force_sph(c, fe);
    if (c.ndim == 2) return make_vel_force_2d(c);
    set_val(c, F_VELFORCE, 0.0, 0, 3, c.F[F_VELFORCE].spec.ng);
    launch(c, rg_grow(c, 0), 1, k_vel_force, c.V(), c.P.buoyancy_cutoff_factor * c.P.base_cutoff_density,
           c.P.dom_hi[2], make_recip(2.0 * c.P.dx[2]), fe);
}

// ============================================================ VelPred
// VelPredInterface, 3-D (Source/MaestroVelPred.cpp:735-1128): predictor states of all
// three velocity components on D-faces, and their upwind values.
template <int D>
__global__ void k_vp_interface(KARGS, int ppm_type, double dt2, double hd, int bclo, int bchi, int domlo, int domhi,
                               long long epsb) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const int I = D == 0 ? i : (D == 1 ? j : k);
    const int il = i - di, jl = j - dj, kl = k - dk;
    const FabView ut = VW(F_UTILDE);
    double l[3], r[3];
    if (ppm_type == 0) {
        const FabView uf = VW(F_UFULL);
        const FabView sl = D == 0 ? VW(F_IPC0) : (D == 1 ? VW(F_IMC1) : VW(F_IMC2));
        const double maxu = 0.5 - dt2 * mx(0.0, at(uf, il, jl, kl, D)) / hd;
        const double minu = 0.5 + dt2 * mn(0.0, at(uf, i, j, k, D)) / hd;
        for (int n = 0; n < 3; ++n) {
            l[n] = at(ut, il, jl, kl, n) + maxu * at(sl, il, jl, kl, n);
            r[n] = at(ut, i, j, k, n) - minu * at(sl, i, j, k, n);
        }
    } else {
        const FabView ip[3] = {VW(F_IPC0), VW(F_IPC1), VW(F_IPC2)};
        const FabView im[3] = {VW(F_IMC0), VW(F_IMC1), VW(F_IMC2)};
        for (int n = 0; n < 3; ++n) {
            l[n] = at(ip[n], il, jl, kl, D);
            r[n] = at(im[n], i, j, k, D);
        }
    }
    if (I == domlo) {
        switch (bclo) {
            case PB_INFLOW:
                for (int n = 0; n < 3; ++n) { l[n] = at(ut, il, jl, kl, n); r[n] = l[n]; }
                break;
            case PB_SLIPWALL: case PB_SYMMETRY:
                for (int n = 0; n < 3; ++n) {
                    if (n == D) { l[n] = 0.0; r[n] = 0.0; }
                    else l[n] = r[n];
                }
                break;
            case PB_NOSLIPWALL:
                for (int n = 0; n < 3; ++n) { l[n] = 0.0; r[n] = 0.0; }
                break;
            case PB_OUTFLOW:
                r[D] = mn(r[D], 0.0);
                for (int n = 0; n < 3; ++n) l[n] = r[n];
                break;
            default: break;
        }
    } else if (I == domhi + 1) {
        switch (bchi) {
            case PB_INFLOW:
                for (int n = 0; n < 3; ++n) { l[n] = at(ut, i, j, k, n); r[n] = l[n]; }
                break;
            case PB_SLIPWALL: case PB_SYMMETRY:
                for (int n = 0; n < 3; ++n) {
                    if (n == D) { l[n] = 0.0; r[n] = 0.0; }
                    else r[n] = l[n];
                }
                break;
            case PB_NOSLIPWALL:
                for (int n = 0; n < 3; ++n) { l[n] = 0.0; r[n] = 0.0; }
                break;
            case PB_OUTFLOW:
                l[D] = mx(l[D], 0.0);
                for (int n = 0; n < 3; ++n) r[n] = l[n];
                break;
            default: break;
        }
    }
    const FabView L = VW(F_SL0 + D), Rr = VW(F_SR0 + D), M = VW(F_SIMH0 + D);
    const double tr = at(VW(F_UTRANS0 + D), i, j, k);
    // reference: v = tr > 0 ? l : r;  v = |tr| < rel_eps ? (l+r)/2 : v
    const bool avg = !((dbits(tr) & ABS_MASK) >= epsb);
    const bool left = gt0(tr);
    for (int n = 0; n < 3; ++n) {
        at(L, i, j, k, n) = l[n];
        at(Rr, i, j, k, n) = r[n];
        if (n == D) continue;
        at(M, i, j, k, n) = avg ? half(l[n] + r[n]) : (left ? l[n] : r[n]);
    }
}

// VelPredTransverse (Source/MaestroVelPred.cpp:1130-1595): component C on D-faces
// corrected in the third direction T.  F_TCOEF comp T holds (dt6/h_T)*(trans_T sum).
template <int C, int D>
__global__ void k_vp_transverse(KARGS, int bclo, int bchi, int domlo, int domhi, long long epsb) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int T = 3 - C - D;
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    constexpr int ti = T == 0, tj = T == 1, tk = T == 2;
    const int I = D == 0 ? i : (D == 1 ? j : k);
    const int il = i - di, jl = j - dj, kl = k - dk;
    const FabView L = VW(F_SL0 + D), Rr = VW(F_SR0 + D), imt = VW(F_SIMH0 + T), tc = VW(F_TCOEF);
    double lq = at(L, i, j, k, C) - at(tc, il, jl, kl, T) * (at(imt, il + ti, jl + tj, kl + tk, C) - at(imt, il, jl, kl, C));
    double rq = at(Rr, i, j, k, C) - at(tc, i, j, k, T) * (at(imt, i + ti, j + tj, k + tk, C) - at(imt, i, j, k, C));
    const FabView ut = VW(F_UTILDE);
    if (I == domlo) {
        switch (bclo) {
            case PB_INFLOW: lq = at(ut, il, jl, kl, C); rq = lq; break;
            case PB_SLIPWALL: case PB_SYMMETRY: case PB_OUTFLOW: lq = rq; break;
            case PB_NOSLIPWALL: lq = 0.0; rq = 0.0; break;
            default: break;
        }
    } else if (I == domhi + 1) {
        switch (bchi) {
            case PB_INFLOW: lq = at(ut, i, j, k, C); rq = lq; break;
            case PB_SLIPWALL: case PB_SYMMETRY: case PB_OUTFLOW: rq = lq; break;
            case PB_NOSLIPWALL: lq = 0.0; rq = 0.0; break;
            default: break;
        }
    }
    const double trd = at(VW(F_UTRANS0 + D), i, j, k);
    const bool avg = !((dbits(trd) & ABS_MASK) >= epsb);
    at(VW(Q_FIELD(C, D)), i, j, k) = avg ? half(lq + rq) : (gt0(trd) ? lq : rq);
}

// VelPredVelocities (Source/MaestroVelPred.cpp:1597-1915).  F_TCOEF comps 3..5 hold
// (dt4/h_t)*(trans_t sum).
template <int D>
__global__ void k_vp_velocities(KARGS, double dt2, int bclo, int bchi, int domlo, int domhi, double rel_eps, int sph,
                                int ptf) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    constexpr int T1 = D == 0 ? 1 : 0, T2 = D == 2 ? 1 : 2;
    constexpr int a1i = T1 == 0, a1j = T1 == 1, a1k = T1 == 2;
    constexpr int a2i = T2 == 0, a2j = T2 == 1, a2k = T2 == 2;
    const int I = D == 0 ? i : (D == 1 ? j : k);
    const int il = i - di, jl = j - dj, kl = k - dk;
    const FabView tc = VW(F_TCOEF);
    const FabView q1 = VW(Q_FIELD(D, T1)), q2 = VW(Q_FIELD(D, T2));
    // the traced force if ppm_trace_forces = 1 (Source/MaestroVelPred.cpp:1644-1647)
    const FabView f = VW(F_VELFORCE);
    const double fl = ptf ? at(VW(F_IPF), il, jl, kl, D) : at(f, il, jl, kl, D);
    const double fr = ptf ? at(VW(F_IMF), i, j, k, D) : at(f, i, j, k, D);
    const double ml = at(VW(F_SL0 + D), i, j, k, D) -
                      at(tc, il, jl, kl, 3 + T1) * (at(q1, il + a1i, jl + a1j, kl + a1k) - at(q1, il, jl, kl)) -
                      at(tc, il, jl, kl, 3 + T2) * (at(q2, il + a2i, jl + a2j, kl + a2k) - at(q2, il, jl, kl)) +
                      dt2 * fl;
    const double mr = at(VW(F_SR0 + D), i, j, k, D) -
                      at(tc, i, j, k, 3 + T1) * (at(q1, i + a1i, j + a1j, k + a1k) - at(q1, i, j, k)) -
                      at(tc, i, j, k, 3 + T2) * (at(q2, i + a2i, j + a2j, k + a2k) - at(q2, i, j, k)) +
                      dt2 * fr;
    double v;
    if (D < 2 && !sph) {
        const bool test = (ml <= 0.0 && mr >= 0.0) || (fabs(ml + mr) < rel_eps);
        v = half(ml + mr) > 0.0 ? ml : mr;
        v = test ? 0.0 : v;
    } else {
        // spherical (Source/MaestroVelPred.cpp:1664-1673): + w0mac in every direction
        const double w0c = sph ? at(VW(F_W0MAC0 + D), i, j, k) : at(VW(F_W0CART), i, j, k, 2);
        const bool test = (ml + w0c <= 0.0 && mr + w0c >= 0.0) || (fabs(ml + mr + 2.0 * w0c) < rel_eps);
        v = half(ml + mr) + w0c > 0.0 ? ml : mr;
        v = test ? 0.0 : v;
    }
    const FabView ut = VW(F_UTILDE);
    if (I == domlo) {
        switch (bclo) {
            case PB_INFLOW: v = at(ut, il, jl, kl, D); break;
            case PB_SLIPWALL: case PB_SYMMETRY: case PB_NOSLIPWALL: v = 0.0; break;
            case PB_OUTFLOW: v = mn(mr, 0.0); break;
            default: break;
        }
    } else if (I == domhi + 1) {
        switch (bchi) {
            case PB_INFLOW: v = at(ut, i, j, k, D); break;
            case PB_SLIPWALL: case PB_SYMMETRY: case PB_NOSLIPWALL: v = 0.0; break;
            case PB_OUTFLOW: v = mx(ml, 0.0); break;
            default: break;
        }
    }
    at(VW(F_UMAC0 + D), i, j, k) = v;
}

template <int C, int D>
static void vp_transverse_launch(Ctx& c) {
    int glo[3] = {0, 0, 0}, ghi[3] = {0, 0, 0};
    glo[C] = 1;
    ghi[C] = 1;
    ghi[D] = 1;
    const RegionTable& rt = region(c, glo[0], glo[1], glo[2], ghi[0], ghi[1], ghi[2], -1);
    launch(c, rt, 1, k_vp_transverse<C, D>, c.V(), c.P.phys_bc_lo[D], c.P.phys_bc_hi[D], c.P.dom_lo[D],
           c.P.dom_hi[D], dbits_host(c.P.rel_eps));
}

template <int D>
static void vp_interface_launch(Ctx& c) {
    int glo[3] = {1, 1, 1};
    glo[D] = 0;
    const RegionTable& rt = region(c, glo[0], glo[1], glo[2], 1, 1, 1, -1);
    launch(c, rt, 1, k_vp_interface<D>, c.V(), c.P.ppm_type, 0.5 * c.P.dt, c.P.dx[D], c.P.phys_bc_lo[D],
           c.P.phys_bc_hi[D], c.P.dom_lo[D], c.P.dom_hi[D], dbits_host(c.P.rel_eps));
}

template <int D>
static void vp_velocities_launch(Ctx& c) {
    launch(c, rg_grow(c, 0, D), 1, k_vp_velocities<D>, c.V(), 0.5 * c.P.dt, c.P.phys_bc_lo[D], c.P.phys_bc_hi[D],
           c.P.dom_lo[D], c.P.dom_hi[D], c.P.rel_eps, (int)c.sph, c.P.ppm_trace_forces);
}

void vel_pred(Ctx& c) {
    if (c.ndim == 2) return vel_pred_2d_entry(c);
    if (c.P.ppm_type == 0) {
        slope_any(c, 0, F_UTILDE, 0, F_IPC0, 0, 3, bcs_dev(c, BCS_U), 0);  // slopex -> Ipu
        slope_any(c, 1, F_UTILDE, 0, F_IMC1, 0, 3, bcs_dev(c, BCS_U), 0);  // slopey -> Imv
        slope_any(c, 2, F_UTILDE, 0, F_IMC2, 0, 3, bcs_dev(c, BCS_U), 0);  // slopez -> Imw
    } else {
        // the sweeps of component d along d were done by make_utrans (same inputs)
        for (int cc = 0; cc < 3; ++cc)
            for (int d = 0; d < 3; ++d)
                if (cc != d) ppm_any(c, d, F_UTILDE, cc, c.bcs_u[cc], F_UFULL, d, 0, F_IPC0 + cc, F_IMC0 + cc);
        // ppm_trace_forces: force component d traced along d, the direction VelPredVelocities
        // reads (Source/MaestroVelPred.cpp:117-137, 203-247)
        if (c.P.ppm_trace_forces)
            for (int d = 0; d < 3; ++d) ppm_any(c, d, F_VELFORCE, d, c.bcs_u[d], F_UFULL, d, 0, F_IPF, F_IMF);
    }
    vp_interface_launch<0>(c);
    vp_interface_launch<1>(c);
    vp_interface_launch<2>(c);
    transverse_coeffs(c, F_UTRANS0);
    vp_transverse_launch<0, 1>(c);
    vp_transverse_launch<0, 2>(c);
    vp_transverse_launch<1, 0>(c);
    vp_transverse_launch<1, 2>(c);
    vp_transverse_launch<2, 0>(c);
    vp_transverse_launch<2, 1>(c);
    vp_velocities_launch<0>(c);
    vp_velocities_launch<1>(c);
    vp_velocities_launch<2>(c);
}

// ============================================================ MakeEdgeScal
// MakeDivU (Source/MaestroMakeEdgeScalars.cpp:648-660)
__global__ void k_divu(KARGS, RecipC rdx0) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView u = VW(F_UMAC0), v = VW(F_UMAC1), w = VW(F_UMAC2);
    double d = at(u, i + 1, j, k) - at(u, i, j, k) + at(v, i, j + 1, k) - at(v, i, j, k) + at(w, i, j, k + 1) -
               at(w, i, j, k);
    at(VW(F_DIVU), i, j, k) = div_c(d, rdx0);
}

// MakeEdgeScalPredictor's boundary rules (Source/MaestroMakeEdgeScalars.cpp:662-863) on the
// D-face whose index along D is I: l and r replaced on the domain's low and high faces.
// sc_l / sc_r: the state of the cell below / above the face (ext_dir takes the ghost value).
__device__ __forceinline__ void es_pred_bc(int I, int bclo, int bchi, int domlo, int domhi, int vclamp, double sc_l,
                                           double sc_r, double& l, double& r) {
    if (I == domlo) {
        if (bclo == BC_EXT_DIR) {
            l = sc_l;
            r = l;
        } else if (bclo == BC_FOEXTRAP || bclo == BC_HOEXTRAP || bclo == BC_REFLECT_EVEN) {
            if (vclamp && bclo != BC_REFLECT_EVEN) r = mn(r, 0.0);  // is_vel, comp == D
            l = r;
        } else if (bclo == BC_REFLECT_ODD) {
            l = 0.0;
            r = 0.0;
        }
    } else if (I == domhi + 1) {
        if (bchi == BC_EXT_DIR) {
            l = sc_r;
            r = l;
        } else if (bchi == BC_FOEXTRAP || bchi == BC_HOEXTRAP || bchi == BC_REFLECT_EVEN) {
            if (vclamp && bchi != BC_REFLECT_EVEN) l = mx(l, 0.0);
            r = l;
        } else if (bchi == BC_REFLECT_ODD) {
            l = 0.0;
            r = 0.0;
        }
    }
}

// The predictor's states of the D-face (i,j,k) with ppm_type 1 / 2 as its consumers use them:
// Ip of the cell below, Im of the cell above (F_IPC0 / F_IMC0 component D).  On a domain face
// the consumers' own boundary rules (k_es_transverse, k_es_edges) overwrite both states for
// ext_dir and reflect_odd, and the outside one (l below, r above) for foextrap, hoextrap and
// reflect_even, so of the predictor's rules only the velocity clamp of the inside state is
// left to apply here.  k_es_simh stores the upwind state with every rule.
template <int D>
__device__ __forceinline__ void es_pred_lr(const FabView& ip, const FabView& im, int bclo, int bchi, int domlo,
                                           int domhi, int vclamp, int i, int j, int k, double& l, double& r) {
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const int I = D == 0 ? i : (D == 1 ? j : k);
    l = at(ip, i - di, j - dj, k - dk, D);
    r = at(im, i, j, k, D);
    if (vclamp) {
        if (I == domlo && (bclo == BC_FOEXTRAP || bclo == BC_HOEXTRAP)) r = mn(r, 0.0);
        else if (I == domhi + 1 && (bchi == BC_FOEXTRAP || bchi == BC_HOEXTRAP)) l = mx(l, 0.0);
    }
}

// MakeEdgeScalPredictor, 3-D (Source/MaestroMakeEdgeScalars.cpp:662-863)
template <int D>
__global__ void k_es_predictor(KARGS, int comp, int ppm_type, double dt, double hd, int bclo, int bchi, int domlo,
                               int domhi, int vclamp) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const int I = D == 0 ? i : (D == 1 ? j : k);
    const int il = i - di, jl = j - dj, kl = k - dk;
    const FabView sc = VW(F_SOLD);
    const double ud = at(VW(F_UMAC0 + D), i, j, k);
    double l, r;
    if (ppm_type == 0) {
        const FabView sl = VW(F_SLOPE);
        l = at(sc, il, jl, kl, comp) + half(1.0 - dt * ud / hd) * at(sl, il, jl, kl, D);
        r = at(sc, i, j, k, comp) - half(1.0 + dt * ud / hd) * at(sl, i, j, k, D);
    } else {
        l = at(VW(F_IPC0), il, jl, kl, D);
        r = at(VW(F_IMC0), i, j, k, D);
    }
    if (I == domlo || I == domhi + 1)
        es_pred_bc(I, bclo, bchi, domlo, domhi, vclamp, at(sc, il, jl, kl, comp), at(sc, i, j, k, comp), l, r);
    at(VW(F_SL0 + D), i, j, k) = l;
    at(VW(F_SR0 + D), i, j, k) = r;
    at(VW(F_SIMH0 + D), i, j, k) = upwind(ud, l, r, 0);  // tie test |u| > 0
}

// The predictor's upwind state alone (ppm_type 1 / 2): the transverse kernels read it at
// neighbouring faces, while the edge states' l and r are formed where they are used.
template <int D>
__global__ void k_es_simh(KARGS, int comp, int bclo, int bchi, int domlo, int domhi, int vclamp) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const int I = D == 0 ? i : (D == 1 ? j : k);
    double l = at(VW(F_IPC0), i - di, j - dj, k - dk, D), r = at(VW(F_IMC0), i, j, k, D);
    if (I == domlo || I == domhi + 1) {
        const FabView sc = VW(F_SOLD);
        es_pred_bc(I, bclo, bchi, domlo, domhi, vclamp, at(sc, i - di, j - dj, k - dk, comp), at(sc, i, j, k, comp), l, r);
    }
    at(VW(F_SIMH0 + D), i, j, k) = upwind(at(VW(F_UMAC0 + D), i, j, k), l, r, 0);  // tie test |u| > 0
}

// MakeEdgeScalTransverse, 3-D (Source/MaestroMakeEdgeScalars.cpp:865-1359): D-faces
// corrected in direction T.  Advective form: F_TCOEF comp T = (dt6/h_T)*(u_T sum).
// INL (ppm_type 1 / 2): the D-face's predictor states l and r are formed here from F_IPC0 /
// F_IMC0 instead of read from F_SL0 / F_SR0 (the same values: Ip, Im and the boundary rules).
template <int D, int T, bool CONS, bool INL>
__global__ void __launch_bounds__(TPB, CONS ? 4 : 6) k_es_transverse(KARGS, int comp, double dt3, double dt3h, int bclo, int bchi, int domlo, int domhi,
                                long long epsb, int vclamp) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    constexpr int ti = T == 0, tj = T == 1, tk = T == 2;
    const int I = D == 0 ? i : (D == 1 ? j : k);
    const int il = i - di, jl = j - dj, kl = k - dk;
    const FabView st = VW(F_SIMH0 + T), sc = VW(F_SOLD), ut = VW(F_UMAC0 + T);
    auto simh = [&](int a, int bb, int cc) -> double { return at(st, a, bb, cc); };
    double sl, sr;
    if (INL) {
        es_pred_lr<D>(VW(F_IPC0), VW(F_IMC0), bclo, bchi, domlo, domhi, vclamp, i, j, k, sl, sr);
    } else {
        sl = at(VW(F_SL0 + D), i, j, k);
        sr = at(VW(F_SR0 + D), i, j, k);
    }
    double lq, rq;
    if (CONS) {
        const FabView dv = VW(F_DIVU);
        lq = sl -
             dt3h * (simh(il + ti, jl + tj, kl + tk) * at(ut, il + ti, jl + tj, kl + tk) - simh(il, jl, kl) * at(ut, il, jl, kl)) -
             dt3 * at(sc, il, jl, kl, comp) * at(dv, il, jl, kl) +
             dt3h * at(sc, il, jl, kl, comp) * (at(ut, il + ti, jl + tj, kl + tk) - at(ut, il, jl, kl));
        rq = sr -
             dt3h * (simh(i + ti, j + tj, k + tk) * at(ut, i + ti, j + tj, k + tk) - simh(i, j, k) * at(ut, i, j, k)) -
             dt3 * at(sc, i, j, k, comp) * at(dv, i, j, k) +
             dt3h * at(sc, i, j, k, comp) * (at(ut, i + ti, j + tj, k + tk) - at(ut, i, j, k));
    } else {
        const FabView tc = VW(F_TCOEF);
        lq = sl - at(tc, il, jl, kl, T) * (simh(il + ti, jl + tj, kl + tk) - simh(il, jl, kl));
        rq = sr - at(tc, i, j, k, T) * (simh(i + ti, j + tj, k + tk) - simh(i, j, k));
    }
    if (I == domlo) {
        if (bclo == BC_EXT_DIR) {
            lq = at(sc, il, jl, kl, comp);
            rq = lq;
        } else if (bclo == BC_FOEXTRAP || bclo == BC_HOEXTRAP || bclo == BC_REFLECT_EVEN) {
            if (vclamp && bclo != BC_REFLECT_EVEN) rq = mn(rq, 0.0);
            lq = rq;
        } else if (bclo == BC_REFLECT_ODD) {
            lq = 0.0;
            rq = 0.0;
        }
    } else if (I == domhi + 1) {
        if (bchi == BC_EXT_DIR) {
            lq = at(sc, i, j, k, comp);
            rq = lq;
        } else if (bchi == BC_FOEXTRAP || bchi == BC_HOEXTRAP || bchi == BC_REFLECT_EVEN) {
            if (vclamp && bchi != BC_REFLECT_EVEN) lq = mx(lq, 0.0);
            rq = lq;
        } else if (bchi == BC_REFLECT_ODD) {
            lq = 0.0;
            rq = 0.0;
        }
    }
    at(VW(Q_FIELD(D, T)), i, j, k) = upwind(at(VW(F_UMAC0 + D), i, j, k), lq, rq, epsb);
}

// MakeEdgeScalEdges, 3-D (Source/MaestroMakeEdgeScalars.cpp:1361-1667).  Advective form:
// F_TCOEF comp 3+t = (dt4/h_t)*(u_t sum).  force_zero: the component's force is
// identically zero (species), so the + dt/2*force term is skipped.
// INL: the D-face's predictor states formed from F_IPC0 / F_IMC0 (as in k_es_transverse).
template <int D, bool CONS, bool INL>
__global__ void k_es_edges(KARGS, int comp, int force_zero, double dt2, double dt2h1, double dt2h2, double dt2hd,
                           int bclo, int bchi, int domlo, int domhi, long long epsb, int vclamp, int ptf, int oc) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    constexpr int T1 = D == 0 ? 1 : 0, T2 = D == 2 ? 1 : 2;
    constexpr int a1i = T1 == 0, a1j = T1 == 1, a1k = T1 == 2;
    constexpr int a2i = T2 == 0, a2j = T2 == 1, a2k = T2 == 2;
    const int I = D == 0 ? i : (D == 1 ? j : k);
    const int il = i - di, jl = j - dj, kl = k - dk;
    const FabView q1 = VW(Q_FIELD(T1, T2)), q2 = VW(Q_FIELD(T2, T1));
    const FabView udf = VW(F_UMAC0 + D);
    const FabView sc = VW(F_SOLD);
    double sl, sr;
    if (INL) {
        es_pred_lr<D>(VW(F_IPC0), VW(F_IMC0), bclo, bchi, domlo, domhi, vclamp, i, j, k, sl, sr);
    } else {
        sl = at(VW(F_SL0 + D), i, j, k);
        sr = at(VW(F_SR0 + D), i, j, k);
    }
    double lq, rq;
    if (CONS) {
        // the traced force if ppm_trace_forces = 1 (Source/MaestroMakeEdgeScalars.cpp:1405-1408)
        const FabView u1 = VW(F_UMAC0 + T1), u2 = VW(F_UMAC0 + T2), f = VW(F_SCALFORCE);
        // force_zero: the force is zero (and so is its trace, which is not formed)
        const double fl = force_zero ? 0.0 : ptf ? at(VW(F_IPF), il, jl, kl, D) : at(f, il, jl, kl, comp);
        const double fr = force_zero ? 0.0 : ptf ? at(VW(F_IMF), i, j, k, D) : at(f, i, j, k, comp);
        lq = sl -
             dt2h1 * (at(q1, il + a1i, jl + a1j, kl + a1k) * at(u1, il + a1i, jl + a1j, kl + a1k) - at(q1, il, jl, kl) * at(u1, il, jl, kl)) -
             dt2h2 * (at(q2, il + a2i, jl + a2j, kl + a2k) * at(u2, il + a2i, jl + a2j, kl + a2k) - at(q2, il, jl, kl) * at(u2, il, jl, kl)) -
             dt2hd * at(sc, il, jl, kl, comp) * (at(udf, i, j, k) - at(udf, il, jl, kl)) + dt2 * fl;
        rq = sr -
             dt2h1 * (at(q1, i + a1i, j + a1j, k + a1k) * at(u1, i + a1i, j + a1j, k + a1k) - at(q1, i, j, k) * at(u1, i, j, k)) -
             dt2h2 * (at(q2, i + a2i, j + a2j, k + a2k) * at(u2, i + a2i, j + a2j, k + a2k) - at(q2, i, j, k) * at(u2, i, j, k)) -
             dt2hd * at(sc, i, j, k, comp) * (at(udf, i + di, j + dj, k + dk) - at(udf, i, j, k)) + dt2 * fr;
    } else {
        const FabView tc = VW(F_TCOEF);
        lq = sl -
             at(tc, il, jl, kl, 3 + T1) * (at(q1, il + a1i, jl + a1j, kl + a1k) - at(q1, il, jl, kl)) -
             at(tc, il, jl, kl, 3 + T2) * (at(q2, il + a2i, jl + a2j, kl + a2k) - at(q2, il, jl, kl));
        rq = sr -
             at(tc, i, j, k, 3 + T1) * (at(q1, i + a1i, j + a1j, k + a1k) - at(q1, i, j, k)) -
             at(tc, i, j, k, 3 + T2) * (at(q2, i + a2i, j + a2j, k + a2k) - at(q2, i, j, k));
        if (!force_zero) {
            const FabView f = VW(F_SCALFORCE);
            lq = lq + dt2 * (ptf ? at(VW(F_IPF), il, jl, kl, D) : at(f, il, jl, kl, comp));
            rq = rq + dt2 * (ptf ? at(VW(F_IMF), i, j, k, D) : at(f, i, j, k, comp));
        }
    }
    double v = upwind(at(udf, i, j, k), lq, rq, epsb);
    if (I == domlo) {
        if (bclo == BC_EXT_DIR) v = at(sc, il, jl, kl, comp);
        else if (bclo == BC_FOEXTRAP || bclo == BC_HOEXTRAP) v = vclamp ? mn(rq, 0.0) : rq;
        else if (bclo == BC_REFLECT_EVEN) v = rq;
        else if (bclo == BC_REFLECT_ODD) v = 0.0;
    } else if (I == domhi + 1) {
        if (bchi == BC_EXT_DIR) v = at(sc, i, j, k, comp);
        else if (bchi == BC_FOEXTRAP || bchi == BC_HOEXTRAP) v = vclamp ? mx(lq, 0.0) : lq;
        else if (bchi == BC_REFLECT_EVEN) v = lq;
        else if (bchi == BC_REFLECT_ODD) v = 0.0;
    }
    at(VW(F_SEDGE0 + D), i, j, k, oc) = v;
}

// vclamp: velocity edge states (is_vel) of the component normal to the faces, whose
// outflow-boundary values are clamped to outflow (Source/MaestroMakeEdgeScalars.cpp:715, 732)
template <int D>
static void es_predictor_launch(Ctx& c, int comp, const BCRecD& bc, int vclamp) {
    int glo[3] = {1, 1, 1};
    glo[D] = 0;
    const RegionTable& rt = region(c, glo[0], glo[1], glo[2], 1, 1, 1, -1);
    launch(c, rt, 1, k_es_predictor<D>, c.V(), comp, c.P.ppm_type, c.P.dt, c.P.dx[D], bc.lo[D], bc.hi[D],
           c.P.dom_lo[D], c.P.dom_hi[D], vclamp);
}

template <int D>
static void es_simh_launch(Ctx& c, int comp, const BCRecD& bc, int vclamp) {
    int glo[3] = {1, 1, 1};
    glo[D] = 0;
    const RegionTable& rt = region(c, glo[0], glo[1], glo[2], 1, 1, 1, -1);
    launch(c, rt, 1, k_es_simh<D>, c.V(), comp, bc.lo[D], bc.hi[D], c.P.dom_lo[D], c.P.dom_hi[D], vclamp);
}

template <int D, int T, bool INL>
static void es_transverse_launch_t(Ctx& c, const RegionTable& rt, int comp, const BCRecD& bc, int is_cons,
                                   int vclamp) {
    const double dt3 = c.P.dt / 3.0;
    if (is_cons)
        launch(c, rt, 1, k_es_transverse<D, T, true, INL>, c.V(), comp, dt3, dt3 / c.P.dx[T], bc.lo[D], bc.hi[D],
               c.P.dom_lo[D], c.P.dom_hi[D], dbits_host(c.P.rel_eps), vclamp);
    else
        launch(c, rt, 1, k_es_transverse<D, T, false, INL>, c.V(), comp, dt3, dt3 / c.P.dx[T], bc.lo[D], bc.hi[D],
               c.P.dom_lo[D], c.P.dom_hi[D], dbits_host(c.P.rel_eps), vclamp);
}

// inl: the D-face's predictor states formed in the kernel
template <int D, int T>
static void es_transverse_launch(Ctx& c, int comp, const BCRecD& bc, int is_cons, int vclamp, bool inl) {
    constexpr int O = 3 - D - T;
    int glo[3] = {0, 0, 0}, ghi[3] = {0, 0, 0};
    glo[O] = 1;
    ghi[O] = 1;
    ghi[D] = 1;
    const RegionTable& rt = region(c, glo[0], glo[1], glo[2], ghi[0], ghi[1], ghi[2], -1);
    if (inl) es_transverse_launch_t<D, T, true>(c, rt, comp, bc, is_cons, vclamp);
    else es_transverse_launch_t<D, T, false>(c, rt, comp, bc, is_cons, vclamp);
}

template <int D, bool INL>
static void es_edges_launch_t(Ctx& c, int comp, const BCRecD& bc, int is_cons, int force_zero, int vclamp, int oc) {
    constexpr int T1 = D == 0 ? 1 : 0, T2 = D == 2 ? 1 : 2;
    const double dt2 = 0.5 * c.P.dt;
    const int ptf = c.P.ppm_trace_forces;
    if (is_cons)
        launch(c, rg_grow(c, 0, D), 1, k_es_edges<D, true, INL>, c.V(), comp, force_zero, dt2, dt2 / c.P.dx[T1],
               dt2 / c.P.dx[T2], dt2 / c.P.dx[D], bc.lo[D], bc.hi[D], c.P.dom_lo[D], c.P.dom_hi[D],
               dbits_host(c.P.rel_eps), vclamp, ptf, oc);
    else
        launch(c, rg_grow(c, 0, D), 1, k_es_edges<D, false, INL>, c.V(), comp, force_zero, dt2, dt2 / c.P.dx[T1],
               dt2 / c.P.dx[T2], dt2 / c.P.dx[D], bc.lo[D], bc.hi[D], c.P.dom_lo[D], c.P.dom_hi[D],
               dbits_host(c.P.rel_eps), vclamp, ptf, oc);
}

template <int D>
static void es_edges_launch(Ctx& c, int comp, const BCRecD& bc, int is_cons, int force_zero, int vclamp, int oc,
                            bool inl) {
    if (inl) es_edges_launch_t<D, true>(c, comp, bc, is_cons, force_zero, vclamp, oc);
    else es_edges_launch_t<D, false>(c, comp, bc, is_cons, force_zero, vclamp, oc);
}

// velocity-only quantities shared by every component of a MakeEdgeScal call
void edge_scal_setup(Ctx& c, int is_cons) {
    if (is_cons) launch(c, rg_grow(c, 1), 1, k_divu, c.V(), make_recip(c.P.dx[0]));
    if (c.P.ppm_type != 0) trace_coeffs_faces(c, F_UMAC0);
    if (!is_cons) transverse_coeffs(c, F_UMAC0);
}

// force_zero: the components' force is identically zero (DensityAdvance species)
void make_edge_scal(Ctx& c, int start_comp, int num_comp, int which_bcs, int is_cons, int force_zero, int is_vel,
                    int slot, bool setup) {
    if (c.ndim == 2) return make_edge_scal_2d_entry(c, start_comp, num_comp, which_bcs, is_cons);
    const BCRecD* bh = bcs_host(c, which_bcs);
    if (setup) edge_scal_setup(c, is_cons);
    // component streams: every other component on the side stream, in its own scratch
    // (components are independent: each reads the state, the velocities and the shared
    // coefficients formed above, and writes only its scratch and its edge state)
    // (not while per-launch timing runs: the autotuner's trials time each kernel alone)
    const bool two = c.comp_streams && c.side_mirror && c.side_mirror == c.dviews && !c.per_box &&
                     !c.edge_tape_begin && !c.staged_ppm && !c.profiling && num_comp > 1;
    cudaStream_t main_stream = c.stream;
    FabView* main_views = c.dviews;
    if (two && !c.dry) {
        cudaEventRecord(c.ev_fork, main_stream);
        cudaStreamWaitEvent(c.side, c.ev_fork, 0);
    }
    for (int comp = start_comp; comp < start_comp + num_comp; ++comp) {
        const bool alt = two && ((comp - start_comp) & 1);
        c.stream = alt ? c.side : main_stream;
        c.dviews = alt ? c.dviews_side : main_views;
        if (c.edge_tape_begin) c.edge_tape_begin(comp);
        const BCRecD& bc = bh[comp];  // start_bccomp == start_scomp at every call site
        if (c.P.ppm_type == 0) {
            for (int d = 0; d < 3; ++d) slope_any(c, d, F_SOLD, comp, F_SLOPE, d, 1, bcs_dev(c, which_bcs), comp);
        } else {
            for (int d = 0; d < 3; ++d) ppm_any(c, d, F_SOLD, comp, bc, F_UMAC0 + d, 0, 1, F_IPC0, F_IMC0);
            // ppm_trace_forces: the component's force traced like it (Source/MaestroMakeEdgeScalars.cpp:
            // 137-141, 223-227); a force known to be zero traces to zero and is not read
            if (c.P.ppm_trace_forces && !force_zero)
                for (int d = 0; d < 3; ++d) ppm_any(c, d, F_SCALFORCE, comp, bc, F_UMAC0 + d, 0, 1, F_IPF, F_IMF);
        }
        const int v0 = is_vel && comp == 0, v1 = is_vel && comp == 1, v2 = is_vel && comp == 2;
        // with PPM the predictor's l and r are Ip / Im passed on: the transverse and edge
        // kernels form them themselves and only the upwind state is stored (the full
        // predictor runs where the adjoint's tape keeps its fields)
        const bool inl = c.es_inline && c.P.ppm_type != 0 && !c.edge_tape_begin;
        if (inl) {
            es_simh_launch<0>(c, comp, bc, v0);
            es_simh_launch<1>(c, comp, bc, v1);
            es_simh_launch<2>(c, comp, bc, v2);
        } else {
            es_predictor_launch<0>(c, comp, bc, v0);
            es_predictor_launch<1>(c, comp, bc, v1);
            es_predictor_launch<2>(c, comp, bc, v2);
        }
        es_transverse_launch<0, 1>(c, comp, bc, is_cons, v0, inl);
        es_transverse_launch<0, 2>(c, comp, bc, is_cons, v0, inl);
        es_transverse_launch<1, 0>(c, comp, bc, is_cons, v1, inl);
        es_transverse_launch<1, 2>(c, comp, bc, is_cons, v1, inl);
        es_transverse_launch<2, 0>(c, comp, bc, is_cons, v2, inl);
        es_transverse_launch<2, 1>(c, comp, bc, is_cons, v2, inl);
        const int oc = slot >= 0 ? slot : comp;
        es_edges_launch<0>(c, comp, bc, is_cons, force_zero, v0, oc, inl);
        es_edges_launch<1>(c, comp, bc, is_cons, force_zero, v1, oc, inl);
        es_edges_launch<2>(c, comp, bc, is_cons, force_zero, v2, oc, inl);
        if (c.edge_tape) c.edge_tape(comp);
    }
    c.stream = main_stream;
    c.dviews = main_views;
    if (two && !c.dry) {
        cudaEventRecord(c.ev_join, c.side);
        cudaStreamWaitEvent(main_stream, c.ev_join, 0);
    }
}

// ============================================================ forces
// ModifyScalForce, planar 3-D (Source/MaestroForce.cpp:413-441)
__global__ void k_modify_scal_force(KARGS, int comp, int s0cart, int fullform, RecipC r0, RecipC r1, RecipC r2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView um = VW(F_UMAC0), vm = VW(F_UMAC1), wm = VW(F_UMAC2);
    const FabView s0a = VW(s0cart), s0e = VW(F_S0ECART), w0a = VW(F_W0CART);
    const double scal = at(VW(F_SOLD), i, j, k, comp);
    const double du = div_c(at(um, i + 1, j, k) - at(um, i, j, k), r0);
    const double dv = div_c(at(vm, i, j + 1, k) - at(vm, i, j, k), r1);
    double divu = du + dv + div_c(at(wm, i, j, k + 1) - at(wm, i, j, k), r2);
    divu += div_c(at(w0a, i, j, k + 1, 2) - at(w0a, i, j, k, 2), r2);
    double& force = at(VW(F_SCALFORCE), i, j, k, comp);
    if (fullform == 1) {
        force -= scal * divu;
    } else {
        const double s0 = at(s0a, i, j, k);
        const double divs0u =
            s0 * (du + dv) + div_c(at(wm, i, j, k + 1) * at(s0e, i, j, k + 1) - at(wm, i, j, k) * at(s0e, i, j, k), r2);
        force += -(scal - s0) * divu - divs0u;
    }
}

// valid cells of one level; F_S0ECART and the s0 cart field are filled by the caller
void modify_scal_force(Ctx& c, int comp, int s0cart_fid, int fullform) {
    if (c.sph) return modify_scal_force_sph(c, comp, s0cart_fid, fullform);
    if (c.ndim == 2) return modify_scal_force_2d(c, comp, s0cart_fid, fullform);
    launch(c, rg_grow(c, 0), 1, k_modify_scal_force, c.V(), comp, s0cart_fid, fullform, make_recip(c.P.dx[0]),
           make_recip(c.P.dx[1]), make_recip(c.P.dx[2]));
}

// MakeRhoHForce, planar 3-D (Source/MaestroForce.cpp:602-627)
__global__ void k_rhoh_force(KARGS, int cutoff, int domhi, RecipC rdz, int psi_in, int add_thermal) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView p0c = VW(F_P0CART);
    double gradp0 = 0.0;
    if (k < cutoff) {
        gradp0 = at(VW(F_RHO0CART), i, j, k) * at(VW(F_GRAVCART), i, j, k, 2);
    } else if (k == domhi) {
        gradp0 = div_c(at(p0c, i, j, k) - at(p0c, i, j - 1, k), rdz);
    } else {
        gradp0 = div_c(at(p0c, i, j + 1, k) - at(p0c, i, j, k), rdz);
    }
    const FabView wm = VW(F_UMAC2);
    const double veladv = half(at(wm, i, j, k) + at(wm, i, j, k + 1));
    double f = veladv * gradp0;
    if (psi_in) f += at(VW(F_PSICART), i, j, k);
    if (add_thermal == 1) f += at(VW(F_THERMAL), i, j, k);
    at(VW(F_SCALFORCE), i, j, k, RHOH) = f;
}

// valid cells of one level; F_P0CART, F_PSICART, F_RHO0CART and F_GRAVCART are filled by
// the caller (which_step 1: rho0_old and p0_old)
void make_rhoh_force(Ctx& c, int is_prediction, int add_thermal) {
    if (c.sph) return make_rhoh_force_sph(c, is_prediction, add_thermal);
    if (c.ndim == 2) return make_rhoh_force_2d(c, is_prediction, add_thermal);
    const int ept = c.P.enthalpy_pred_type;
    const int psi_in = (is_prediction == 1 && ept == 2) || (is_prediction == 1 && ept == 0) || (is_prediction == 0);
    launch(c, rg_grow(c, 0), 1, k_rhoh_force, c.V(), c.P.base_cutoff_density_coord, c.P.dom_hi[2],
           make_recip(c.P.dx[2]), psi_in, add_thermal);
}

// ============================================================ conversions
// PutInPertForm (Source/MaestroConvert.cpp:6-34), valid region
__global__ void k_pert(KARGS, int comp, const double* __restrict__ s0, int flag) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    double& a = at(VW(F_SOLD), i, j, k, comp);
    a = flag ? a - s0[k] : a + s0[k];
}

void put_in_pert_form(Ctx& c, const double* d_s0, int comp, int flag) {
    if (c.sph) return put_in_pert_form_sph(c, d_s0, comp, flag);
    if (c.ndim == 2) return put_in_pert_form_2d(c, d_s0, comp, flag);
    launch(c, rg_grow(c, 0), 1, k_pert, c.V(), comp, d_s0, flag);
}

// ConvertRhoXToX (Source/MaestroConvert.cpp:64-91), valid region
__global__ void k_rhox_to_x(KARGS, int c0, int nc, int flag) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView s = VW(F_SOLD);
    for (int comp = c0; comp < c0 + nc; ++comp) {
        if (flag) at(s, i, j, k, comp) = at(s, i, j, k, comp) / at(s, i, j, k, RHO);
        else at(s, i, j, k, comp) = at(s, i, j, k, comp) * at(s, i, j, k, RHO);
    }
}

void convert_rhox_to_x(Ctx& c, int flag, int c0, int nc) {
    launch(c, rg_grow(c, 0), 1, k_rhox_to_x, c.V(), c0, nc < 0 ? c.nspec : nc, flag);
}

// ============================================================ fluxes
// MakeRhoXFlux, planar 3-D (Source/MaestroMakeFlux.cpp:189-306)
// Species c0 .. c0+nc-1 of nspec; slot >= 0: the one species' edge state and flux are in
// component `slot`.  The Rho flux (the species fluxes summed in order from 0) and etarhoflux
// carry over between calls, so species streamed one call at a time sum in the same order.
template <int D>
__global__ void k_rhox_flux(KARGS, int c0, int nc, int nspec, int slot, int spt, int do_eta,
                            const double* __restrict__ r0o, const double* __restrict__ r0n,
                            const double* __restrict__ w0, const double* __restrict__ r0pe) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView fl = VW(F_SFLUX0 + D), e = VW(F_SEDGE0 + D);
    const double u = at(VW(F_UMAC0 + D), i, j, k);
    double frho = c0 == FIRSTSPEC ? 0.0 : at(fl, i, j, k, RHO);
    // etarhoflux is accumulated into species by species, as the reference does (:170-178)
    double eta = D == 2 && do_eta ? at(VW(F_ETA), i, j, k) : 0.0;
    for (int comp = c0; comp < c0 + nc; ++comp) {
        const int ec = slot >= 0 ? slot : comp;
        const double rho0_edge = half(r0o[k] + r0n[k]);
        double f = 0.0;
        if (spt == 1) f = u * (rho0_edge + at(e, i, j, k, RHO)) * at(e, i, j, k, ec);
        else if (spt == 2) f = u * at(e, i, j, k, ec);
        else f = u * at(e, i, j, k, RHO) * at(e, i, j, k, ec);
        at(fl, i, j, k, ec) = f;
        if (D == 2 && do_eta) {
            eta += f;
            if (comp == FIRSTSPEC + nspec - 1) eta -= w0[k] * r0pe[k];
        }
        frho += f;
    }
    at(fl, i, j, k, RHO) = frho;
    if (D == 2 && do_eta) at(VW(F_ETA), i, j, k) = eta;
}

void make_rhox_flux(Ctx& c, const double* r0_old, const double* r0e_old, const double* r0_new, const double* r0e_new,
                    int c0, int nc, int slot) {
    if (nc < 0) nc = c.nspec;
    if (c.sph) return make_rhox_flux_sph(c, c0, nc, slot);  // face base state from MakeS0mac (F_S0MAC*, F_S0MACB*)
    if (c.ndim == 2) return make_rhox_flux_2d(c, r0_old, r0e_old, r0_new, r0e_new);
    const int do_eta = c.P.evolve_base_state && !c.P.use_exact_base_state;
    const double* w0 = c.b1("w0");
    const double* rpe = c.b1("rho0_predicted_edge");
    const int ns = c.nspec, spt = c.P.species_pred_type;
    launch(c, rg_grow(c, 0, 0), 1, k_rhox_flux<0>, c.V(), c0, nc, ns, slot, spt, 0, r0_old, r0_new, w0, rpe);
    launch(c, rg_grow(c, 0, 1), 1, k_rhox_flux<1>, c.V(), c0, nc, ns, slot, spt, 0, r0_old, r0_new, w0, rpe);
    launch(c, rg_grow(c, 0, 2), 1, k_rhox_flux<2>, c.V(), c0, nc, ns, slot, spt, do_eta, r0e_old, r0e_new, w0, rpe);
}

// MakeRhoHFlux, planar 3-D (Source/MaestroMakeFlux.cpp:673-786)
// enthalpy_pred_type 2 (the edge state is h, :673-786 have_h): (rho0 edge + rho') h with
// species_pred_type 1 (ra, rb: rho0 on the faces' radial positions), rho h otherwise
template <int D>
__global__ void k_rhoh_flux(KARGS, int ept, const double* __restrict__ a, const double* __restrict__ bb, int spt,
                            const double* __restrict__ ra, const double* __restrict__ rb) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView e = VW(F_SEDGE0 + D);
    const double u = at(VW(F_UMAC0 + D), i, j, k);
    double f;
    if (ept == 0) {
        f = u * at(e, i, j, k, RHOH);
    } else if (ept == 2) {
        if (spt == 1) {
            const double rho0_edge = half(ra[k] + rb[k]);
            f = u * (rho0_edge + at(e, i, j, k, RHO)) * at(e, i, j, k, RHOH);
        } else {
            f = u * at(e, i, j, k, RHO) * at(e, i, j, k, RHOH);
        }
    } else {
        const double rhoh0_edge = half(a[k] + bb[k]);
        f = D < 2 ? u * (rhoh0_edge + at(e, i, j, k, RHOH)) : u * (at(e, i, j, k, RHOH) + rhoh0_edge);
    }
    at(VW(F_SFLUX0 + D), i, j, k, RHOH) = f;
}

void make_rhoh_flux(Ctx& c, const double* rh0_old, const double* rh0e_old, const double* rh0_new,
                    const double* rh0e_new, const double* r0_old, const double* r0e_old, const double* r0_new,
                    const double* r0e_new) {
    if (c.sph) return make_rhoh_flux_sph(c);
    if (c.ndim == 2) return make_rhoh_flux_2d(c, rh0_old, rh0e_old, rh0_new, rh0e_new, r0_old, r0e_old, r0_new, r0e_new);
    const int ept = c.P.enthalpy_pred_type, spt = c.P.species_pred_type;
    launch(c, rg_grow(c, 0, 0), 1, k_rhoh_flux<0>, c.V(), ept, rh0_old, rh0_new, spt, r0_old, r0_new);
    launch(c, rg_grow(c, 0, 1), 1, k_rhoh_flux<1>, c.V(), ept, rh0_old, rh0_new, spt, r0_old, r0_new);
    launch(c, rg_grow(c, 0, 2), 1, k_rhoh_flux<2>, c.V(), ept, rh0e_old, rh0e_new, spt, r0e_old, r0e_new);
}

// Maestro::ConvertRhoHToH on the valid region (Source/MaestroConvert.cpp:93-105): flag,
// (rho h) -> h = (rho h) / rho; else h -> h rho
__global__ void k_rhoh_to_h(KARGS, int flag) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView s = VW(F_SOLD);
    double& a = at(s, i, j, k, RHOH);
    a = flag ? a / at(s, i, j, k, RHO) : a * at(s, i, j, k, RHO);
}
void convert_rhoh_to_h(Ctx& c, int flag) { launch(c, rg_grow(c, 0), 1, k_rhoh_to_h, c.V(), flag); }

// the prediction force of h: the (rho h) force over rho, valid cells and one ghost cell
// (MultiFab::Divide, Source/MaestroEnthalpyAdvance.cpp:83-88)
__global__ void k_h_force(KARGS) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    double& f = at(VW(F_SCALFORCE), i, j, k, RHOH);
    f = f / at(VW(F_SOLD), i, j, k, RHO);
}
void h_force(Ctx& c) {
    const int gz = c.ndim == 2 ? 0 : 1;
    launch(c, region(c, 1, 1, gz, 1, 1, gz, -1), 1, k_h_force, c.V());
}

// species_pred_type 2: rho edge state = sum of the (rho X) edge states
template <int D>
__global__ void k_sum_species(KARGS, int nspec) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView e = VW(F_SEDGE0 + D);
    double s = at(e, i, j, k, FIRSTSPEC);
    for (int n = 1; n < nspec; ++n) s += at(e, i, j, k, FIRSTSPEC + n);
    at(e, i, j, k, RHO) = s;
}

// the same sum, one species at a time from edge-state component `slot`
template <int D>
__global__ void k_sum_species_step(KARGS, int slot, int first) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView e = VW(F_SEDGE0 + D);
    at(e, i, j, k, RHO) = first ? at(e, i, j, k, slot) : at(e, i, j, k, RHO) + at(e, i, j, k, slot);
}

void sum_species_edge_step(Ctx& c, int slot, int first) {
    launch(c, rg_grow(c, 0, 0), 1, k_sum_species_step<0>, c.V(), slot, first);
    launch(c, rg_grow(c, 0, 1), 1, k_sum_species_step<1>, c.V(), slot, first);
    launch(c, rg_grow(c, 0, 2), 1, k_sum_species_step<2>, c.V(), slot, first);
}

void sum_species_edges(Ctx& c) {
    if (c.ndim == 2) return sum_species_edges_2d(c);
    launch(c, rg_grow(c, 0, 0), 1, k_sum_species<0>, c.V(), c.nspec);
    launch(c, rg_grow(c, 0, 1), 1, k_sum_species<1>, c.V(), c.nspec);
    launch(c, rg_grow(c, 0, 2), 1, k_sum_species<2>, c.V(), c.nspec);
}

// ============================================================ UpdateScal
// Source/MaestroAdvection.cpp:117-251.  The species update and the density / floor /
// negative-species pass of the reference are two ParallelFors over the same cells; they
// are one kernel here with the same per-cell order of operations.
// the new (rho X) of one species from its flux in component fc of F_SFLUX*
__device__ __forceinline__ void update_species_cell(const FabView* __restrict__ V, int nb, int b, int comp, int fc,
                                                    double dt, const RecipC& r0, const RecipC& r1, const RecipC& r2,
                                                    int i, int j, int k) {
    const FabView so = VW(F_SOLD), sn = VW(F_SNEW), fx = VW(F_SFLUX0), fy = VW(F_SFLUX1), fz = VW(F_SFLUX2),
                  fo = VW(F_SCALFORCE);
    double divterm = div_c(at(fx, i + 1, j, k, fc) - at(fx, i, j, k, fc), r0);
    divterm += div_c(at(fy, i, j + 1, k, fc) - at(fy, i, j, k, fc), r1);
    divterm += div_c(at(fz, i, j, k + 1, fc) - at(fz, i, j, k, fc), r2);
    at(sn, i, j, k, comp) = at(so, i, j, k, comp) + dt * (-divterm + at(fo, i, j, k, comp));
}

// rho from the species' changes, the density floor and the negative-species fix
__device__ __forceinline__ void rhox_fix_cell(const FabView* __restrict__ V, int nb, int b, int nspec,
                                              double half_cutoff, int i, int j, int k) {
    const FabView so = VW(F_SOLD), sn = VW(F_SNEW);
    double rho = at(so, i, j, k, RHO);
    bool neg = false;
    for (int comp = FIRSTSPEC; comp < FIRSTSPEC + nspec; ++comp) {
        rho += at(sn, i, j, k, comp) - at(so, i, j, k, comp);
        if (lt0(at(sn, i, j, k, comp))) neg = true;
    }
    if (rho < half_cutoff) {
        for (int comp = FIRSTSPEC; comp < FIRSTSPEC + nspec; ++comp) at(sn, i, j, k, comp) *= half_cutoff / rho;
        rho = half_cutoff;
    }
    at(sn, i, j, k, RHO) = rho;
    if (neg) {
        for (int comp = FIRSTSPEC; comp < FIRSTSPEC + nspec; ++comp) {
            if (at(sn, i, j, k, comp) < 0.0) {
                const double delta = -at(sn, i, j, k, comp);
                double sumX = 0.0;
                for (int c2 = FIRSTSPEC; c2 < FIRSTSPEC + nspec; ++c2)
                    if (c2 != comp && at(sn, i, j, k, c2) >= 0.0) sumX += at(sn, i, j, k, c2);
                for (int c2 = FIRSTSPEC; c2 < FIRSTSPEC + nspec; ++c2)
                    if (c2 != comp && at(sn, i, j, k, c2) >= 0.0) {
                        const double frac = at(sn, i, j, k, c2) / sumX;
                        at(sn, i, j, k, c2) -= frac * delta;
                    }
                at(sn, i, j, k, comp) = 0.0;
            }
        }
    }
}

__global__ void k_update_rhox(KARGS, int nspec, double dt, RecipC r0, RecipC r1, RecipC r2, double half_cutoff) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    for (int n = 0; n < nspec; ++n) update_species_cell(V, nb, b, FIRSTSPEC + n, FIRSTSPEC + n, dt, r0, r1, r2, i, j, k);
    rhox_fix_cell(V, nb, b, nspec, half_cutoff, i, j, k);
}

__global__ void k_update_species(KARGS, int comp, int fc, double dt, RecipC r0, RecipC r1, RecipC r2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    update_species_cell(V, nb, b, comp, fc, dt, r0, r1, r2, i, j, k);
}

__global__ void k_update_rhox_fix(KARGS, int nspec, double half_cutoff) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    rhox_fix_cell(V, nb, b, nspec, half_cutoff, i, j, k);
}

__global__ void k_update_rhoh(KARGS, double dt, RecipC r0, RecipC r1, RecipC r2, int eos_check, double cutoff,
                              int* flag) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView so = VW(F_SOLD), sn = VW(F_SNEW), fx = VW(F_SFLUX0), fy = VW(F_SFLUX1), fz = VW(F_SFLUX2),
                  fo = VW(F_SCALFORCE);
    const double divterm = (div_c(at(fx, i + 1, j, k, RHOH) - at(fx, i, j, k, RHOH), r0) +
                            div_c(at(fy, i, j + 1, k, RHOH) - at(fy, i, j, k, RHOH), r1) +
                            div_c(at(fz, i, j, k + 1, RHOH) - at(fz, i, j, k, RHOH), r2));
    at(sn, i, j, k, RHOH) = at(so, i, j, k, RHOH) + dt * (-divterm + at(fo, i, j, k, RHOH));
    if (eos_check && at(sn, i, j, k, RHO) <= cutoff) atomicOr(flag, 1);
}

// Maestro::UpdateVel, 3-D (Source/MaestroAdvection.cpp:299-526): unew = uold - dt (Utilde.grad)
// Utilde + dt force, minus dt (w0.grad) Utilde (planar: w0bar from w0_cart of cells k and k+1;
// spherical: w0mac averaged to the cell, every direction), times the sponge where given.
// uold: field fu; MAC velocity without w0: F_UMAC*; edge states: F_SEDGE* comps 0-2; force:
// F_VELFORCE; output F_SNEW comps 0-2.
__global__ void k_update_vel(KARGS, int fu, int fsp, int sph, double dt, RecipC r0, RecipC r1, RecipC r2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView uo = VW(fu), un = VW(F_SNEW), um = VW(F_UMAC0), vm = VW(F_UMAC1), wm = VW(F_UMAC2);
    const FabView ex = VW(F_SEDGE0), ey = VW(F_SEDGE1), ez = VW(F_SEDGE2), f = VW(F_VELFORCE);
    const double ubar = half(at(um, i, j, k) + at(um, i + 1, j, k));
    const double vbar = half(at(vm, i, j, k) + at(vm, i, j + 1, k));
    const double wbar = half(at(wm, i, j, k) + at(wm, i, j, k + 1));
    double v[3];
    for (int n = 0; n < 3; ++n) {
        const double ugrad = div_c(ubar * (at(ex, i + 1, j, k, n) - at(ex, i, j, k, n)), r0) +
                             div_c(vbar * (at(ey, i, j + 1, k, n) - at(ey, i, j, k, n)), r1) +
                             div_c(wbar * (at(ez, i, j, k + 1, n) - at(ez, i, j, k, n)), r2);
        v[n] = at(uo, i, j, k, n) - dt * ugrad + dt * at(f, i, j, k, n);
    }
    if (!sph) {
        const FabView w0c = VW(F_W0CART);
        const double w0bar = half(at(w0c, i, j, k, 2) + at(w0c, i, j, k + 1, 2));
        for (int n = 0; n < 3; ++n) {
            v[n] -= div_c(dt * w0bar * (at(ez, i, j, k + 1, n) - at(ez, i, j, k, n)), r2);
            if (fsp >= 0) v[n] *= at(VW(fsp), i, j, k);
        }
    } else {
        const FabView wx = VW(F_W0MAC0), wy = VW(F_W0MAC1), wz = VW(F_W0MAC2);
        double w0r[3];
        for (int n = 0; n < 3; ++n) {
            const double gx = div_c(at(ex, i + 1, j, k, n) - at(ex, i, j, k, n), r0);
            const double gy = div_c(at(ey, i, j + 1, k, n) - at(ey, i, j, k, n), r1);
            const double gz = div_c(at(ez, i, j, k + 1, n) - at(ez, i, j, k, n), r2);
            w0r[n] = gx * 0.5 * (at(wx, i, j, k) + at(wx, i + 1, j, k)) +
                     gy * 0.5 * (at(wy, i, j, k) + at(wy, i, j + 1, k)) +
                     gz * 0.5 * (at(wz, i, j, k) + at(wz, i, j, k + 1));
        }
        for (int n = 0; n < 3; ++n) v[n] -= dt * w0r[n];
        if (fsp >= 0)
            for (int n = 0; n < 3; ++n) v[n] *= at(VW(fsp), i, j, k);
    }
    for (int n = 0; n < 3; ++n) at(un, i, j, k, n) = v[n];
}

void update_vel(Ctx& c, int fu, int fsponge) {
    launch(c, rg_grow(c, 0), 1, k_update_vel, c.V(), fu, fsponge, (int)c.sph, c.P.dt, make_recip(c.P.dx[0]),
           make_recip(c.P.dx[1]), make_recip(c.P.dx[2]));
}

// EstDt (Source/MaestroDt.cpp:128-225 planar, :301-384 spherical): maxima over a level's
// valid cells of |u| per direction (the radial one with the cell-centred w0 added; the
// spherical w0mac of EstDt is zero with the exact base state), of |w0_cart| (radial
// component; component 0 in spherical geometry, as the reference reads it) and of
// |vel_force| per direction.  The magnitudes' bit patterns order like their values, so the
// maxima are exact: warp maxima by shuffles, then one atomicMax per warp and quantity.
// w0m: spherical with uniform bins and an evolving base state, the face w0mac averaged to the
// cell (Source/MaestroDt.cpp:313-334); other spherical cases add 0.5 (0 + 0)
__global__ void k_dt_maxima(KARGS, int sph, int nd, int w0m, unsigned long long* out) {
    const long gid = g0 + (long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long m[7] = {0ULL, 0ULL, 0ULL, 0ULL, 0ULL, 0ULL, 0ULL};
    if (gid < g1) {
        const int e = find_box(R, ne, gid);
        const int b = R[e].b;
        int i, j, k;
        region_ijk(R[e], gid - R[e].start, i, j, k);
        const FabView u = VW(F_UTILDE), w0c = VW(F_W0CART), f = VW(F_VELFORCE);
        for (int d = 0; d < nd; ++d) {
            double v = at(u, i, j, k, d);
            if (!sph && d == nd - 1) v = v + half(at(w0c, i, j, k, d) + at(w0c, i, j + (d == 1), k + (d == 2), d));
            if (sph && w0m) {
                const FabView wm = VW(F_W0MAC0 + d);
                v = v + half(at(wm, i, j, k) + at(wm, i + (d == 0), j + (d == 1), k + (d == 2)));
            } else if (sph) {
                v = v + 0.5 * (0.0 + 0.0);
            }
            m[d] = (unsigned long long)(dbits(v) & ABS_MASK);
            m[4 + d] = (unsigned long long)(dbits(at(f, i, j, k, d)) & ABS_MASK);
        }
        m[3] = (unsigned long long)(dbits(at(w0c, i, j, k, sph ? 0 : nd - 1)) & ABS_MASK);
    }
    for (int q = 0; q < 7; ++q) {
        unsigned long long v = m[q];
        for (int off = 16; off > 0; off >>= 1) {
            const unsigned long long o = __shfl_xor_sync(0xffffffffu, v, off);
            v = o > v ? o : v;
        }
        m[q] = v;
    }
    if ((threadIdx.x & 31) == 0)
        for (int q = 0; q < 7; ++q)
            if (m[q]) atomicMax(out + q, m[q]);
}

void dt_maxima(Ctx& c) {
    const int w0m = c.sph && !c.geo.exact && c.P.evolve_base_state;
    launch(c, rg_grow(c, 0), 1, k_dt_maxima, c.V(), (int)c.sph, c.ndim, w0m, c.d_red);
}

void update_scal(Ctx& c, int start_comp) {
    if (c.ndim == 2) return update_scal_2d(c, start_comp);
    const RegionTable& rt = rg_grow(c, 0);
    if (start_comp == RHOH) {
        launch(c, rt, 1, k_update_rhoh, c.V(), c.P.dt, make_recip(c.P.dx[0]), make_recip(c.P.dx[1]),
               make_recip(c.P.dx[2]), c.P.do_eos_h_above_cutoff, c.P.base_cutoff_density, c.d_flag);
    } else {
        launch(c, rt, 1, k_update_rhox, c.V(), c.nspec, c.P.dt, make_recip(c.P.dx[0]), make_recip(c.P.dx[1]),
               make_recip(c.P.dx[2]), 0.5 * c.P.base_cutoff_density);
    }
}

void update_species(Ctx& c, int comp, int slot) {
    launch(c, rg_grow(c, 0), 1, k_update_species, c.V(), comp, slot, c.P.dt, make_recip(c.P.dx[0]),
           make_recip(c.P.dx[1]), make_recip(c.P.dx[2]));
}

void update_rhox_fix(Ctx& c) {
    launch(c, rg_grow(c, 0), 1, k_update_rhox_fix, c.V(), c.nspec, 0.5 * c.P.base_cutoff_density);
}

}  // namespace madv

// ============================================================ 2-D (AMREX_SPACEDIM == 2)
// The 2-D form of the stage: y is radial (base-state index r = j), boxes and the domain
// have k = 0 only, two velocity components.  Regions of a 2-D context never grow in z.
// PPM, the limited slopes, the fills and the x-face transverse velocity are the 3-D
// kernels run in x and y; the kernels below restate the 2-D branches of the reference
// (their expressions and quirks differ from 3-D), with plain IEEE division.
namespace madv {

static const RegionTable& rg2(Ctx& c, int g, int nodal = -1) { return region(c, g, g, 0, g, g, 0, nodal); }

// Put1dArrayOnCart, planar 2-D (Source/MaestroFill3dData.cpp:79-93): r = j
__global__ void k_put1d_2d(KARGS, int f, const double* __restrict__ s0, int outcomp, int edge) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    at(VW(f), i, j, k, outcomp) = edge ? half(s0[j] + s0[j + 1]) : s0[j];
}

// Addw0, planar 2-D (Source/MaestroFill3dData.cpp:380-386): vedge += mult * w0(j)
__global__ void k_addw0_2d(KARGS, int f, const double* __restrict__ w0, double mult) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    at(VW(f), i, j, k) += mult * w0[j];
}

// MakeUtrans, 2-D y faces (Source/MaestroMakeUtrans.cpp:161-266): the lo-side wall case
// sets vry = 0 twice and leaves vly; the solve tests v + w0_cart.
__global__ void k_utrans_2dy(KARGS, int ppm_type, double dt2dy, int bclo, int bchi, int domlo, int domhi,
                             double rel_eps) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView ut = VW(F_UTILDE);
    double l, r;
    if (ppm_type == 0) {
        const FabView uf = VW(F_UFULL), sl = VW(F_SLOPE);
        l = at(ut, i, j - 1, k, 1) + (0.5 - dt2dy * mx(0.0, at(uf, i, j - 1, k, 1))) * at(sl, i, j - 1, k, 0);
        r = at(ut, i, j, k, 1) - (0.5 + dt2dy * mn(0.0, at(uf, i, j, k, 1))) * at(sl, i, j, k, 0);
    } else {
        l = at(VW(F_IPC0 + 1), i, j - 1, k, 1);
        r = at(VW(F_IMC0 + 1), i, j, k, 1);
    }
    if (j == domlo) {
        switch (bclo) {
            case PB_INFLOW: l = at(ut, i, j - 1, k, 1); r = l; break;
            case PB_SLIPWALL: case PB_NOSLIPWALL: case PB_SYMMETRY: r = 0.0; break;
            case PB_OUTFLOW: l = mn(r, 0.0); r = l; break;
            default: break;
        }
    } else if (j == domhi + 1) {
        switch (bchi) {
            case PB_INFLOW: l = at(ut, i, j, k, 1); r = l; break;
            case PB_SLIPWALL: case PB_NOSLIPWALL: case PB_SYMMETRY: l = 0.0; r = 0.0; break;
            case PB_OUTFLOW: l = mx(l, 0.0); r = l; break;
            default: break;
        }
    }
    const double w0c = at(VW(F_W0CART), i, j, k, 1);
    const bool test = (l + w0c <= 0.0 && r + w0c >= 0.0) || (fabs(l + r + 2.0 * w0c) < rel_eps);
    double v = half(l + r) + w0c > 0.0 ? l : r;
    at(VW(F_UTRANS1), i, j, k) = test ? 0.0 : v;
}

static void make_utrans_2d(Ctx& c) {
    const double dt2 = 0.5 * c.P.dt;
    if (c.P.ppm_type != 0)
        launch(c, rg2(c, 1), 1, k_trace_cell, c.V(), F_UFULL, c.P.dt, c.P.dx[0], c.P.dx[1], c.P.dx[2]);
    for (int d = 0; d < 2; ++d) {
        if (c.P.ppm_type == 0) slope_any(c, d, F_UTILDE, d, F_SLOPE, 0, 1, bcs_dev(c, BCS_U), d);
        else ppm_any(c, d, F_UTILDE, d, c.bcs_u[d], F_UFULL, d, 0, F_IPC0 + d, F_IMC0 + d);
        const RegionTable& rt = rg2(c, 0, d);
        const double dt2dx = dt2 / c.P.dx[d];
        const int bl = c.P.phys_bc_lo[d], bh = c.P.phys_bc_hi[d], dl = c.P.dom_lo[d], dh = c.P.dom_hi[d];
        if (d == 0) launch(c, rt, 1, k_utrans<0>, c.V(), c.P.ppm_type, dt2dx, bl, bh, dl, dh, c.P.rel_eps, 0);
        else launch(c, rt, 1, k_utrans_2dy, c.V(), c.P.ppm_type, dt2dx, bl, bh, dl, dh, c.P.rel_eps);
    }
}

// MakeVelForce, planar 2-D (Source/MaestroForce.cpp:100-137)
__global__ void k_vel_force_2d(KARGS, double cutoff_rho, int domhi, double dy) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView gpi = VW(F_GPI), rho = VW(F_SOLD), vf = VW(F_VELFORCE);
    const double r = at(rho, i, j, k, RHO);
    double rhopert = r - at(VW(F_RHO0CART), i, j, k);
    if (r < cutoff_rho) rhopert = 0.0;
    at(vf, i, j, k, 0) = -at(gpi, i, j, k, 0) / r;
    double f1 = (rhopert * at(VW(F_GRAVCART), i, j, k, 1) - at(gpi, i, j, k, 1)) / r - at(VW(F_W0FCART), i, j, k, 1);
    if (j <= -1 || j >= domhi) {
    } else {
        const FabView ve = VW(F_UTRANS1), w0 = VW(F_W0CART);
        f1 -= (at(ve, i, j + 1, k) + at(ve, i, j, k)) * (at(w0, i, j + 1, k, 1) - at(w0, i, j, k, 1)) / (2.0 * dy);
    }
    at(vf, i, j, k, 1) = f1;
}

// VelPredInterface, 2-D (Source/MaestroVelPred.cpp:296-537).  D = 0: ulx/urx/uimhx into
// F_SL0/F_SR0/F_SIMH0; D = 1: uly/ury/uimhy into F_SL1/F_SR1/F_SIMH1.
template <int D>
__global__ void k_vp_interface_2d(KARGS, int ppm_type, double dt2h, int bclo, int bchi, int domlo, int domhi,
                                  double rel_eps) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1;
    constexpr int T = 1 - D;  // the transverse component upwinded into uimh
    const int I = D == 0 ? i : j;
    const FabView ut = VW(F_UTILDE), uf = VW(F_UFULL);
    const FabView l = VW(F_SL0 + D), r = VW(F_SR0 + D);
    double L[2], Rr[2];
    if (ppm_type == 0) {
        const double maxu = mx(0.0, at(uf, i - di, j - dj, k, D));
        const double minu = mn(0.0, at(uf, i, j, k, D));
        const FabView sl = D == 0 ? VW(F_IPC0) : VW(F_IMC1);
        for (int n = 0; n < 2; ++n) {
            L[n] = at(ut, i - di, j - dj, k, n) + (0.5 - dt2h * maxu) * at(sl, i - di, j - dj, k, n);
            Rr[n] = at(ut, i, j, k, n) - (0.5 + dt2h * minu) * at(sl, i, j, k, n);
        }
    } else {
        for (int n = 0; n < 2; ++n) {
            L[n] = at(VW(F_IPC0 + n), i - di, j - dj, k, D);
            Rr[n] = at(VW(F_IMC0 + n), i, j, k, D);
        }
    }
    if (I == domlo) {
        switch (bclo) {
            case PB_INFLOW:
                for (int n = 0; n < 2; ++n) L[n] = Rr[n] = at(ut, i - di, j - dj, k, n);
                break;
            case PB_SLIPWALL: case PB_SYMMETRY:
                if (D == 0) {
                    L[0] = 0.0;
                    Rr[0] = 0.0;
                    L[1] = Rr[1];
                } else {
                    L[0] = Rr[0];
                    L[1] = 0.0;
                    Rr[1] = 0.0;
                }
                break;
            case PB_NOSLIPWALL:
                for (int n = 0; n < 2; ++n) L[n] = Rr[n] = 0.0;
                break;
            case PB_OUTFLOW:
                if (D == 0) {
                    Rr[0] = mn(Rr[0], 0.0);
                    for (int n = 0; n < 2; ++n) Rr[n] = L[n];
                } else {
                    Rr[1] = mn(Rr[1], 0.0);
                    for (int n = 0; n < 2; ++n) L[n] = Rr[n];
                }
                break;
            default: break;
        }
    } else if (I == domhi + 1) {
        switch (bchi) {
            case PB_INFLOW:
                for (int n = 0; n < 2; ++n) L[n] = Rr[n] = at(ut, i, j, k, n);
                break;
            case PB_SLIPWALL: case PB_SYMMETRY:
                if (D == 0) {
                    L[0] = 0.0;
                    Rr[0] = 0.0;
                    Rr[1] = L[1];
                } else {
                    Rr[0] = L[0];
                    L[1] = 0.0;
                    Rr[1] = 0.0;
                }
                break;
            case PB_NOSLIPWALL:
                for (int n = 0; n < 2; ++n) L[n] = Rr[n] = 0.0;
                break;
            case PB_OUTFLOW:
                L[D] = mx(L[D], 0.0);
                for (int n = 0; n < 2; ++n) Rr[n] = L[n];
                break;
            default: break;
        }
    }
    for (int n = 0; n < 2; ++n) {
        at(l, i, j, k, n) = L[n];
        at(r, i, j, k, n) = Rr[n];
    }
    const double tr = at(VW(F_UTRANS0 + D), i, j, k);
    const double v = tr > 0.0 ? L[T] : Rr[T];
    at(VW(F_SIMH0 + D), i, j, k, T) = fabs(tr) < rel_eps ? half(L[T] + Rr[T]) : v;
}

// VelPredVelocities, 2-D (Source/MaestroVelPred.cpp:539-727)
template <int D>
__global__ void k_vp_velocities_2d(KARGS, double dt2, double dt4h, int bclo, int bchi, int domlo, int domhi,
                                   double rel_eps) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1;
    constexpr int T = 1 - D;
    constexpr int ti = T == 0, tj = T == 1;
    const int I = D == 0 ? i : j;
    const int il = i - di, jl = j - dj;
    const FabView f = VW(F_VELFORCE), ttr = VW(F_UTRANS0 + T), q = VW(F_SIMH0 + T);
    const double fl = at(f, il, jl, k, D), fr = at(f, i, j, k, D);
    const double ml = at(VW(F_SL0 + D), i, j, k, D) -
                      dt4h * (at(ttr, il + ti, jl + tj, k) + at(ttr, il, jl, k)) *
                          (at(q, il + ti, jl + tj, k, D) - at(q, il, jl, k, D)) +
                      dt2 * fl;
    const double mr = at(VW(F_SR0 + D), i, j, k, D) -
                      dt4h * (at(ttr, i + ti, j + tj, k) + at(ttr, i, j, k)) *
                          (at(q, i + ti, j + tj, k, D) - at(q, i, j, k, D)) +
                      dt2 * fr;
    double v;
    if (D == 0) {
        v = half(ml + mr) > 0.0 ? ml : mr;
        v = (ml <= 0.0 && mr >= 0.0) || (fabs(ml + mr) < rel_eps) ? 0.0 : v;
    } else {
        const double w0c = at(VW(F_W0CART), i, j, k, 1);
        const bool test = (ml + w0c <= 0.0 && mr + w0c >= 0.0) || (fabs(ml + mr + 2.0 * w0c) < rel_eps);
        v = half(ml + mr) + w0c > 0.0 ? ml : mr;
        v = test ? 0.0 : v;
    }
    const FabView ut = VW(F_UTILDE);
    if (I == domlo) {
        switch (bclo) {
            case PB_INFLOW: v = at(ut, il, jl, k, D); break;
            case PB_SLIPWALL: case PB_NOSLIPWALL: case PB_SYMMETRY: v = 0.0; break;
            case PB_OUTFLOW: v = mn(mr, 0.0); break;
            default: break;
        }
    } else if (I == domhi + 1) {
        switch (bchi) {
            case PB_INFLOW: v = at(ut, i, j, k, D); break;
            case PB_SLIPWALL: case PB_NOSLIPWALL: case PB_SYMMETRY: v = 0.0; break;
            case PB_OUTFLOW: v = mx(ml, 0.0); break;
            default: break;
        }
    }
    at(VW(F_UMAC0 + D), i, j, k) = v;
}

static void vel_pred_2d(Ctx& c) {
    if (c.P.ppm_type == 0) {
        slope_any(c, 0, F_UTILDE, 0, F_IPC0, 0, 2, bcs_dev(c, BCS_U), 0);  // slopex -> Ipu
        slope_any(c, 1, F_UTILDE, 0, F_IMC1, 0, 2, bcs_dev(c, BCS_U), 0);  // slopey -> Imv
    } else {
        // component d along d was traced by make_utrans (same inputs)
        ppm_any(c, 1, F_UTILDE, 0, c.bcs_u[0], F_UFULL, 1, 0, F_IPC0, F_IMC0);
        ppm_any(c, 0, F_UTILDE, 1, c.bcs_u[1], F_UFULL, 0, 0, F_IPC0 + 1, F_IMC0 + 1);
    }
    const double dt2 = 0.5 * c.P.dt, dt4 = 0.25 * c.P.dt;
    for (int d = 0; d < 2; ++d) {
        const RegionTable& rm = region(c, d == 0 ? 0 : 1, d == 1 ? 0 : 1, 0, 1, 1, 0, -1);  // growLo(obx, d, -1)
        const int bl = c.P.phys_bc_lo[d], bh = c.P.phys_bc_hi[d], dl = c.P.dom_lo[d], dh = c.P.dom_hi[d];
        if (d == 0)
            launch(c, rm, 1, k_vp_interface_2d<0>, c.V(), c.P.ppm_type, dt2 / c.P.dx[0], bl, bh, dl, dh, c.P.rel_eps);
        else
            launch(c, rm, 1, k_vp_interface_2d<1>, c.V(), c.P.ppm_type, dt2 / c.P.dx[1], bl, bh, dl, dh, c.P.rel_eps);
    }
    for (int d = 0; d < 2; ++d) {
        const int bl = c.P.phys_bc_lo[d], bh = c.P.phys_bc_hi[d], dl = c.P.dom_lo[d], dh = c.P.dom_hi[d];
        const double dt4h = dt4 / c.P.dx[1 - d];
        if (d == 0) launch(c, rg2(c, 0, 0), 1, k_vp_velocities_2d<0>, c.V(), dt2, dt4h, bl, bh, dl, dh, c.P.rel_eps);
        else launch(c, rg2(c, 0, 1), 1, k_vp_velocities_2d<1>, c.V(), dt2, dt4h, bl, bh, dl, dh, c.P.rel_eps);
    }
}

// MakeEdgeScalPredictor, 2-D (Source/MaestroMakeEdgeScalars.cpp:306-452)
template <int D>
__global__ void k_es_predictor_2d(KARGS, int comp, int ppm_type, double dt2, double hd, int bclo, int bchi, int domlo,
                                  int domhi, double rel_eps) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1;
    const int I = D == 0 ? i : j;
    const FabView s = VW(F_SOLD), ud = VW(F_UMAC0 + D);
    const double u = at(ud, i, j, k);
    double l, r;
    if (ppm_type == 0) {
        const FabView sl = VW(F_SLOPE);
        l = at(s, i - di, j - dj, k, comp) + (0.5 - dt2 * u / hd) * at(sl, i - di, j - dj, k, D);
        r = at(s, i, j, k, comp) - (0.5 + dt2 * u / hd) * at(sl, i, j, k, D);
    } else {
        l = at(VW(F_IPC0), i - di, j - dj, k, D);
        r = at(VW(F_IMC0), i, j, k, D);
    }
    if (I == domlo) {
        if (bclo == BC_EXT_DIR) {
            l = r = at(s, i - di, j - dj, k, comp);
        } else if (bclo == BC_FOEXTRAP || bclo == BC_HOEXTRAP || bclo == BC_REFLECT_EVEN) {
            l = r;
        } else if (bclo == BC_REFLECT_ODD) {
            l = r = 0.0;
        }
    } else if (I == domhi + 1) {
        if (bchi == BC_EXT_DIR) {
            l = r = at(s, i, j, k, comp);
        } else if (bchi == BC_FOEXTRAP || bchi == BC_HOEXTRAP || bchi == BC_REFLECT_EVEN) {
            r = l;
        } else if (bchi == BC_REFLECT_ODD) {
            l = r = 0.0;
        }
    }
    at(VW(F_SL0 + D), i, j, k) = l;
    at(VW(F_SR0 + D), i, j, k) = r;
    double sm = (u > 0.0) ? l : r;
    at(VW(F_SIMH0 + D), i, j, k) = (fabs(u) > rel_eps) ? sm : half(l + r);
}

// MakeEdgeScalEdges, 2-D (Source/MaestroMakeEdgeScalars.cpp:454-644)
template <int D>
__global__ void k_es_edges_2d(KARGS, int comp, int is_cons, double dt2, double dt4, double hd, double ht, int bclo,
                              int bchi, int domlo, int domhi, double rel_eps) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1;
    constexpr int T = 1 - D;
    constexpr int ti = T == 0, tj = T == 1;
    const int I = D == 0 ? i : j;
    const int il = i - di, jl = j - dj;
    const FabView s = VW(F_SOLD), ud = VW(F_UMAC0 + D), ut = VW(F_UMAC0 + T), st = VW(F_SIMH0 + T);
    const FabView f = VW(F_SCALFORCE);
    const double fl = at(f, il, jl, k, comp), fr = at(f, i, j, k, comp);
    const double l = at(VW(F_SL0 + D), i, j, k), r = at(VW(F_SR0 + D), i, j, k);
    double lq, rq;
    if (is_cons) {
        lq = l - (dt2 / ht) * (at(st, il + ti, jl + tj, k) * at(ut, il + ti, jl + tj, k) - at(st, il, jl, k) * at(ut, il, jl, k)) -
             (dt2 / hd) * at(s, il, jl, k, comp) * (at(ud, i, j, k) - at(ud, il, jl, k)) + dt2 * fl;
        rq = r - (dt2 / ht) * (at(st, i + ti, j + tj, k) * at(ut, i + ti, j + tj, k) - at(st, i, j, k) * at(ut, i, j, k)) -
             (dt2 / hd) * at(s, i, j, k, comp) * (at(ud, i + di, j + dj, k) - at(ud, i, j, k)) + dt2 * fr;
    } else {
        lq = l - (dt4 / ht) * (at(ut, il + ti, jl + tj, k) + at(ut, il, jl, k)) *
                     (at(st, il + ti, jl + tj, k) - at(st, il, jl, k)) +
             dt2 * fl;
        rq = r - (dt4 / ht) * (at(ut, i + ti, j + tj, k) + at(ut, i, j, k)) * (at(st, i + ti, j + tj, k) - at(st, i, j, k)) +
             dt2 * fr;
    }
    const double u = at(ud, i, j, k);
    double v = (u > 0.0) ? lq : rq;
    v = (fabs(u) > rel_eps) ? v : half(lq + rq);
    if (I == domlo) {
        if (bclo == BC_EXT_DIR) v = at(s, il, jl, k, comp);
        else if (bclo == BC_FOEXTRAP || bclo == BC_HOEXTRAP || bclo == BC_REFLECT_EVEN) v = rq;
        else if (bclo == BC_REFLECT_ODD) v = 0.0;
    } else if (I == domhi + 1) {
        if (bchi == BC_EXT_DIR) v = at(s, i, j, k, comp);
        else if (bchi == BC_FOEXTRAP || bchi == BC_HOEXTRAP || bchi == BC_REFLECT_EVEN) v = lq;
        else if (bchi == BC_REFLECT_ODD) v = 0.0;
    }
    at(VW(F_SEDGE0 + D), i, j, k, comp) = v;
}

static void make_edge_scal_2d(Ctx& c, int start_comp, int num_comp, int which_bcs, int is_cons) {
    const BCRecD* bh = bcs_host(c, which_bcs);
    const double dt2 = 0.5 * c.P.dt, dt4 = 0.25 * c.P.dt;
    if (c.P.ppm_type != 0) {
        launch(c, region(c, 1, 1, 0, 1, 1, 0, 0), 1, k_trace_face<0>, c.V(), F_UMAC0, F_TRA0, c.P.dt, c.P.dx[0]);
        launch(c, region(c, 1, 1, 0, 1, 1, 0, 1), 1, k_trace_face<1>, c.V(), F_UMAC1, F_TRA1, c.P.dt, c.P.dx[1]);
    }
    for (int comp = start_comp; comp < start_comp + num_comp; ++comp) {
        const BCRecD& bc = bh[comp];
        if (c.P.ppm_type == 0) {
            for (int d = 0; d < 2; ++d) slope_any(c, d, F_SOLD, comp, F_SLOPE, d, 1, bcs_dev(c, which_bcs), comp);
        } else {
            for (int d = 0; d < 2; ++d) ppm_any(c, d, F_SOLD, comp, bc, F_UMAC0 + d, 0, 1, F_IPC0, F_IMC0);
        }
        for (int d = 0; d < 2; ++d) {
            const RegionTable& rm = region(c, d == 0 ? 0 : 1, d == 1 ? 0 : 1, 0, 1, 1, 0, -1);
            const int dl = c.P.dom_lo[d], dh = c.P.dom_hi[d];
            if (d == 0)
                launch(c, rm, 1, k_es_predictor_2d<0>, c.V(), comp, c.P.ppm_type, dt2, c.P.dx[0], bc.lo[0], bc.hi[0], dl,
                       dh, c.P.rel_eps);
            else
                launch(c, rm, 1, k_es_predictor_2d<1>, c.V(), comp, c.P.ppm_type, dt2, c.P.dx[1], bc.lo[1], bc.hi[1], dl,
                       dh, c.P.rel_eps);
        }
        for (int d = 0; d < 2; ++d) {
            const int dl = c.P.dom_lo[d], dh = c.P.dom_hi[d];
            if (d == 0)
                launch(c, rg2(c, 0, 0), 1, k_es_edges_2d<0>, c.V(), comp, is_cons, dt2, dt4, c.P.dx[0], c.P.dx[1],
                       bc.lo[0], bc.hi[0], dl, dh, c.P.rel_eps);
            else
                launch(c, rg2(c, 0, 1), 1, k_es_edges_2d<1>, c.V(), comp, is_cons, dt2, dt4, c.P.dx[1], c.P.dx[0],
                       bc.lo[1], bc.hi[1], dl, dh, c.P.rel_eps);
        }
    }
}

// ModifyScalForce, planar 2-D (Source/MaestroForce.cpp:419-447)
__global__ void k_modify_scal_force_2d(KARGS, int comp, int s0cart, int fullform, double dx0, double dx1) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView um = VW(F_UMAC0), vm = VW(F_UMAC1), s0a = VW(s0cart), s0e = VW(F_S0ECART), w0a = VW(F_W0CART);
    const double scal = at(VW(F_SOLD), i, j, k, comp);
    double divu = (at(um, i + 1, j, k) - at(um, i, j, k)) / dx0 + (at(vm, i, j + 1, k) - at(vm, i, j, k)) / dx1;
    divu += (at(w0a, i, j + 1, k, 1) - at(w0a, i, j, k, 1)) / dx1;
    double& force = at(VW(F_SCALFORCE), i, j, k, comp);
    if (fullform == 1) {
        force -= scal * divu;
    } else {
        const double s0 = at(s0a, i, j, k);
        const double divs0u = s0 * (at(um, i + 1, j, k) - at(um, i, j, k)) / dx0 +
                              (at(vm, i, j + 1, k) * at(s0e, i, j + 1, k) - at(vm, i, j, k) * at(s0e, i, j, k)) / dx1;
        force += -(scal - s0) * divu - divs0u;
    }
}

// MakeRhoHForce, planar 2-D (Source/MaestroForce.cpp:586-603)
__global__ void k_rhoh_force_2d(KARGS, int cutoff, int domhi, double dy, int psi_in, int add_thermal) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView p0c = VW(F_P0CART);
    double gradp0;
    if (j < cutoff) gradp0 = at(VW(F_RHO0CART), i, j, k) * at(VW(F_GRAVCART), i, j, k, 1);
    else if (j == domhi) gradp0 = (at(p0c, i, j, k) - at(p0c, i, j - 1, k)) / dy;
    else gradp0 = (at(p0c, i, j + 1, k) - at(p0c, i, j, k)) / dy;
    const FabView vm = VW(F_UMAC1);
    const double veladv = half(at(vm, i, j, k) + at(vm, i, j + 1, k));
    double f = veladv * gradp0;
    if (psi_in) f += at(VW(F_PSICART), i, j, k);
    if (add_thermal == 1) f += at(VW(F_THERMAL), i, j, k);
    at(VW(F_SCALFORCE), i, j, k, RHOH) = f;
}

// PutInPertForm, 2-D (r = j)
__global__ void k_pert_2d(KARGS, int comp, const double* __restrict__ s0, int flag) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    double& a = at(VW(F_SOLD), i, j, k, comp);
    a = flag ? a - s0[j] : a + s0[j];
}

// MakeRhoXFlux, 2-D (Source/MaestroMakeFlux.cpp:101-182)
template <int D>
__global__ void k_rhox_flux_2d(KARGS, int nspec, int spt, int do_eta, const double* __restrict__ r0o,
                               const double* __restrict__ r0n, const double* __restrict__ w0,
                               const double* __restrict__ r0pe) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView fl = VW(F_SFLUX0 + D), e = VW(F_SEDGE0 + D);
    const double u = at(VW(F_UMAC0 + D), i, j, k);
    double frho = 0.0, eta = D == 1 && do_eta ? at(VW(F_ETA), i, j, k) : 0.0;
    for (int comp = FIRSTSPEC; comp < FIRSTSPEC + nspec; ++comp) {
        const double rho0_edge = half(r0o[j] + r0n[j]);
        double f;
        if (spt == 1) f = u * (rho0_edge + at(e, i, j, k, RHO)) * at(e, i, j, k, comp);
        else if (spt == 2) f = u * at(e, i, j, k, comp);
        else f = u * at(e, i, j, k, RHO) * at(e, i, j, k, comp);
        at(fl, i, j, k, comp) = f;
        if (D == 1 && do_eta) {
            eta += f;
            if (comp == FIRSTSPEC + nspec - 1) eta -= w0[j] * r0pe[j];
        }
        frho += f;
    }
    at(fl, i, j, k, RHO) = frho;
    if (D == 1 && do_eta) at(VW(F_ETA), i, j, k) = eta;
}

// MakeRhoHFlux, 2-D (Source/MaestroMakeFlux.cpp:597-662)
template <int D>
__global__ void k_rhoh_flux_2d(KARGS, int ept, const double* __restrict__ a, const double* __restrict__ bb, int spt,
                               const double* __restrict__ ra, const double* __restrict__ rb) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView e = VW(F_SEDGE0 + D);
    const double u = at(VW(F_UMAC0 + D), i, j, k);
    double f;
    if (ept == 0) {
        f = u * at(e, i, j, k, RHOH);
    } else if (ept == 2) {  // the edge state is h (Source/MaestroMakeFlux.cpp:597-662, have_h)
        if (spt == 1) {
            const double rho0_edge = half(ra[j] + rb[j]);
            f = u * (rho0_edge + at(e, i, j, k, RHO)) * at(e, i, j, k, RHOH);
        } else {
            f = u * at(e, i, j, k, RHO) * at(e, i, j, k, RHOH);
        }
    } else {
        const double rhoh0_edge = half(a[j] + bb[j]);
        f = D == 0 ? u * (rhoh0_edge + at(e, i, j, k, RHOH)) : u * (at(e, i, j, k, RHOH) + rhoh0_edge);
    }
    at(VW(F_SFLUX0 + D), i, j, k, RHOH) = f;
}

// UpdateScal, 2-D (Source/MaestroAdvection.cpp:117-251)
__global__ void k_update_rhox_2d(KARGS, int nspec, double dt, double dx0, double dx1, double half_cutoff) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView so = VW(F_SOLD), sn = VW(F_SNEW), fx = VW(F_SFLUX0), fy = VW(F_SFLUX1), fo = VW(F_SCALFORCE);
    for (int n = 0; n < nspec; ++n) {
        const int comp = FIRSTSPEC + n;
        double divterm = (at(fx, i + 1, j, k, comp) - at(fx, i, j, k, comp)) / dx0;
        divterm += (at(fy, i, j + 1, k, comp) - at(fy, i, j, k, comp)) / dx1;
        at(sn, i, j, k, comp) = at(so, i, j, k, comp) + dt * (-divterm + at(fo, i, j, k, comp));
    }
    double rho = at(so, i, j, k, RHO);
    bool neg = false;
    for (int comp = FIRSTSPEC; comp < FIRSTSPEC + nspec; ++comp) {
        rho += at(sn, i, j, k, comp) - at(so, i, j, k, comp);
        if (at(sn, i, j, k, comp) < 0.0) neg = true;
    }
    if (rho < half_cutoff) {
        for (int comp = FIRSTSPEC; comp < FIRSTSPEC + nspec; ++comp) at(sn, i, j, k, comp) *= half_cutoff / rho;
        rho = half_cutoff;
    }
    at(sn, i, j, k, RHO) = rho;
    if (neg) {
        for (int comp = FIRSTSPEC; comp < FIRSTSPEC + nspec; ++comp) {
            if (at(sn, i, j, k, comp) < 0.0) {
                const double delta = -at(sn, i, j, k, comp);
                double sumX = 0.0;
                for (int c2 = FIRSTSPEC; c2 < FIRSTSPEC + nspec; ++c2)
                    if (c2 != comp && at(sn, i, j, k, c2) >= 0.0) sumX += at(sn, i, j, k, c2);
                for (int c2 = FIRSTSPEC; c2 < FIRSTSPEC + nspec; ++c2)
                    if (c2 != comp && at(sn, i, j, k, c2) >= 0.0) {
                        const double frac = at(sn, i, j, k, c2) / sumX;
                        at(sn, i, j, k, c2) -= frac * delta;
                    }
                at(sn, i, j, k, comp) = 0.0;
            }
        }
    }
}

__global__ void k_update_rhoh_2d(KARGS, double dt, double dx0, double dx1, int eos_check, double cutoff, int* flag) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView so = VW(F_SOLD), sn = VW(F_SNEW), fx = VW(F_SFLUX0), fy = VW(F_SFLUX1), fo = VW(F_SCALFORCE);
    const double divterm = ((at(fx, i + 1, j, k, RHOH) - at(fx, i, j, k, RHOH)) / dx0 +
                            (at(fy, i, j + 1, k, RHOH) - at(fy, i, j, k, RHOH)) / dx1);
    at(sn, i, j, k, RHOH) = at(so, i, j, k, RHOH) + dt * (-divterm + at(fo, i, j, k, RHOH));
    if (eos_check && at(sn, i, j, k, RHO) <= cutoff) atomicOr(flag, 1);
}

// ---- wrappers (dispatched to by the 3-D entry points when c.ndim == 2)
void put1d_2d(Ctx& c, int fid, const double* d_s0, int outcomp, int edge) {
    launch(c, rg2(c, 0), 1, k_put1d_2d, c.V(), fid, d_s0, outcomp, edge);
}
void addw0_2d(Ctx& c, int f0, double mult) {
    launch(c, region(c, 1, 0, 0, 1, 0, 0, 1), 1, k_addw0_2d, c.V(), f0 + 1, (const double*)c.b1("w0"), mult);
}
void make_vel_force_2d(Ctx& c) {
    set_val(c, F_VELFORCE, 0.0, 0, 2, 1);
    launch(c, rg2(c, 0), 1, k_vel_force_2d, c.V(), c.P.buoyancy_cutoff_factor * c.P.base_cutoff_density,
           c.P.dom_hi[1], c.P.dx[1]);
}
void modify_scal_force_2d(Ctx& c, int comp, int s0cart_fid, int fullform) {
    launch(c, rg2(c, 0), 1, k_modify_scal_force_2d, c.V(), comp, s0cart_fid, fullform, c.P.dx[0], c.P.dx[1]);
}
void make_rhoh_force_2d(Ctx& c, int is_prediction, int add_thermal) {
    const int ept = c.P.enthalpy_pred_type;
    const int psi_in = (is_prediction == 1 && ept == 2) || (is_prediction == 1 && ept == 0) || (is_prediction == 0);
    launch(c, rg2(c, 0), 1, k_rhoh_force_2d, c.V(), c.P.base_cutoff_density_coord, c.P.dom_hi[1], c.P.dx[1], psi_in,
           add_thermal);
}
void put_in_pert_form_2d(Ctx& c, const double* d_s0, int comp, int flag) {
    launch(c, rg2(c, 0), 1, k_pert_2d, c.V(), comp, d_s0, flag);
}
void make_rhox_flux_2d(Ctx& c, const double* r0_old, const double* r0e_old, const double* r0_new,
                       const double* r0e_new) {
    const int do_eta = c.P.evolve_base_state && !c.P.use_exact_base_state;
    const double* w0 = c.b1("w0");
    const double* rpe = c.b1("rho0_predicted_edge");
    launch(c, rg2(c, 0, 0), 1, k_rhox_flux_2d<0>, c.V(), c.nspec, c.P.species_pred_type, 0, r0_old, r0_new, w0, rpe);
    launch(c, rg2(c, 0, 1), 1, k_rhox_flux_2d<1>, c.V(), c.nspec, c.P.species_pred_type, do_eta, r0e_old, r0e_new,
           w0, rpe);
}
void make_rhoh_flux_2d(Ctx& c, const double* rh0_old, const double* rh0e_old, const double* rh0_new,
                       const double* rh0e_new, const double* r0_old, const double* r0e_old, const double* r0_new,
                       const double* r0e_new) {
    const int ept = c.P.enthalpy_pred_type, spt = c.P.species_pred_type;
    launch(c, rg2(c, 0, 0), 1, k_rhoh_flux_2d<0>, c.V(), ept, rh0_old, rh0_new, spt, r0_old, r0_new);
    launch(c, rg2(c, 0, 1), 1, k_rhoh_flux_2d<1>, c.V(), ept, rh0e_old, rh0e_new, spt, r0e_old, r0e_new);
}
void sum_species_edges_2d(Ctx& c) {
    launch(c, rg2(c, 0, 0), 1, k_sum_species<0>, c.V(), c.nspec);
    launch(c, rg2(c, 0, 1), 1, k_sum_species<1>, c.V(), c.nspec);
}
void update_scal_2d(Ctx& c, int start_comp) {
    const RegionTable& rt = rg2(c, 0);
    if (start_comp == RHOH)
        launch(c, rt, 1, k_update_rhoh_2d, c.V(), c.P.dt, c.P.dx[0], c.P.dx[1], c.P.do_eos_h_above_cutoff,
               c.P.base_cutoff_density, c.d_flag);
    else
        launch(c, rt, 1, k_update_rhox_2d, c.V(), c.nspec, c.P.dt, c.P.dx[0], c.P.dx[1], 0.5 * c.P.base_cutoff_density);
}
void make_utrans_2d_entry(Ctx& c) { make_utrans_2d(c); }

// What VelPred takes over from MakeUtrans when the two run back to back (ppm_type 1/2): the
// tracing coefficients of ufull per cell and the PPM sweep of each velocity component along
// its own direction.  A VelPred call on its own recomputes them from the same inputs.
void vel_pred_prep(Ctx& c) {
    if (c.P.ppm_type == 0) return;
    const RegionTable& rt = c.ndim == 2 ? rg2(c, 1) : rg_grow(c, 1);
    launch(c, rt, 1, k_trace_cell, c.V(), F_UFULL, c.P.dt, c.P.dx[0], c.P.dx[1], c.P.dx[2]);
    for (int d = 0; d < c.ndim; ++d) ppm_any(c, d, F_UTILDE, d, c.bcs_u[d], F_UFULL, d, 0, F_IPC0 + d, F_IMC0 + d);
}
void vel_pred_2d_entry(Ctx& c) { vel_pred_2d(c); }
void make_edge_scal_2d_entry(Ctx& c, int start_comp, int num_comp, int which_bcs, int is_cons) {
    make_edge_scal_2d(c, start_comp, num_comp, which_bcs, is_cons);
}

}  // namespace madv
