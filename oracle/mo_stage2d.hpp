// Test infrastructure only (oracle): the 2-D plane-parallel stage, i.e. the
// AMREX_SPACEDIM == 2 branches of the reference functions, one level.  y is the radial
// direction (base-state index r = j); boxes are stored with k = 0 only (their ghost layers
// in z are periodic copies and never read).  Each function cites the 2-D lines it follows;
// the 2-D code has its own quirks, kept here:
//   * MakeUtrans, y lo slipwall/noslipwall/symmetry sets vry = 0 twice and leaves vly
//     (Source/MaestroMakeUtrans.cpp:216-221);
//   * VelPredInterface, x lo outflow: urx(0) = min(urx(0), 0) is overwritten by urx = ulx
//     (Source/MaestroVelPred.cpp:376-381);
//   * 2-D predictor states use (0.5 - dt2*u/h) * slope and the rel_eps upwind threshold
//     (Source/MaestroMakeEdgeScalars.cpp:339-390), not the 3-D forms;
//   * ModifyScalForce divs0u = s0*du/dx + d(v s0_edge)/dy (Source/MaestroForce.cpp:439-446).
#pragma once
#include "mo_amr.hpp"
#include "mo_ppm.hpp"

namespace mo {

inline Box g2(const Box& b, int n) {
    Box r = b;
    for (int d = 0; d < 2; ++d) {
        r.lo[d] -= n;
        r.hi[d] += n;
    }
    return r;
}

struct Stage2D {
    Lev S;  // parameters, level, BCs, base state (index j), PPM context
    int nspec = 0, nscal = 0, nb = 0, ng_s = 3, ng_adv = 3;
    double dt = 0, rel_eps = 0;

    const Level& L() const { return S.L; }

    // Put1dArrayOnCart, planar 2-D (Source/MaestroFill3dData.cpp:79-93, r = j)
    void Put1dArrayOnCart(const std::vector<real>& s0, MF& s0_cart, bool edge, bool vec,
                          const std::vector<BCRec>* bcs, int bccomp, bool is_vel) {
        const int outcomp = vec ? 1 : 0;
        for (int b = 0; b < nb; ++b) {
            const Arr& a = s0_cart[b];
            MO_FOR3(L().ba[b]) {
                const int r = j;
                a(i, j, k, outcomp) = edge ? 0.5 * (s0[r] + s0[r + 1]) : s0[r];
            }
        }
        if (s0_cart.ng > 0) FillPatch(S.L, s0_cart, 0, vec ? 2 : 1, bccomp, *bcs, is_vel);
    }

    void SyncFaces(MF* u) {
        for (int d = 0; d < 2; ++d) FillBoundary(S.L, u[d], 0, 1, u[d].ng);
        S.FillUmacGhost(u, 2);
    }

    // Addw0, planar 2-D (Source/MaestroFill3dData.cpp:380-386)
    void Addw0(MF* uedge, real mult) {
        for (int b = 0; b < nb; ++b) {
            const Arr& vedge = uedge[1][b];
            Box ybx = grow(nodal(L().ba[b], 1), 0, 1);
            MO_FOR3(ybx) { vedge(i, j, k) += mult * S.w0[j]; }
        }
        SyncFaces(uedge);
    }

    // MakeUtrans, 2-D (Source/MaestroMakeUtrans.cpp:57-268)
    void MakeUtrans(MF& utilde, MF& ufull, MF* utrans) {
        const real dt2 = 0.5 * dt;
        const int* domlo = L().dom.lo;
        const int* domhi = L().dom.hi;
        MF Ip, Im;
        Ip.define(L().ba, 2, 2);
        Im.define(L().ba, 2, 2);
        MF& velsrc = (S.P.ppm_type == 0) ? utilde : ufull;
        for (int d = 0; d < 2; ++d) {
            for (int b = 0; b < nb; ++b) {
                const Box obx = g2(L().ba[b], 1);
                const Box xbx = nodal(L().ba[b], d);
                const Arr& ut = utilde[b];
                const Arr& uf = ufull[b];
                const Arr& Ipa = Ip[b];
                const Arr& Ima = Im[b];
                const Arr& tr = utrans[d][b];
                const Arr& w0a = S.w0_cart[b];
                if (S.P.ppm_type == 0) {
                    Slope_dir(S.P.slope_order, L().dom, obx, velsrc[b].comp(d), Ipa, 1, S.bcs_u, d, d);
                } else {
                    PPM_dir(S.pc, obx, ut, d, velsrc[b].comp(0), Ipa, Ima, 0, S.bcs_u[d].lo[0], S.bcs_u[d].hi[0], false);
                    PPM_dir(S.pc, obx, ut, d, velsrc[b].comp(1), Ipa, Ima, 1, S.bcs_u[d].lo[1], S.bcs_u[d].hi[1], false);
                }
                const int bclo = S.P.phys_bc_lo[d], bchi = S.P.phys_bc_hi[d];
                const int di = d == 0, dj = d == 1;
                MO_FOR3(xbx) {
                    const int I = d == 0 ? i : j;
                    real l = 0.0, r = 0.0;
                    if (S.P.ppm_type == 0) {
                        l = ut(i - di, j - dj, k, d) +
                            (0.5 - (dt2 / L().dx[d]) * mx(0.0, uf(i - di, j - dj, k, d))) * Ipa(i - di, j - dj, k, 0);
                        r = ut(i, j, k, d) - (0.5 + (dt2 / L().dx[d]) * mn(0.0, uf(i, j, k, d))) * Ipa(i, j, k, 0);
                    } else {
                        l = Ipa(i - di, j - dj, k, d);
                        r = Ima(i, j, k, d);
                    }
                    if (I == domlo[d]) {
                        switch (bclo) {
                            case inflow: l = ut(i - di, j - dj, k, d); r = ut(i - di, j - dj, k, d); break;
                            case slipwall: case noslipwall: case symmetry:
                                if (d == 0) l = 0.0;
                                r = 0.0;
                                break;
                            case outflow: l = mn(r, 0.0); r = l; break;
                            default: break;
                        }
                    } else if (I == domhi[d] + 1) {
                        switch (bchi) {
                            case inflow: l = ut(i, j, k, d); r = ut(i, j, k, d); break;
                            case slipwall: case noslipwall: case symmetry: l = 0.0; r = 0.0; break;
                            case outflow: l = mx(l, 0.0); r = l; break;
                            default: break;
                        }
                    }
                    if (d == 0) {
                        bool test = (l <= 0.0 && r >= 0.0) || (fab(l + r) < rel_eps);
                        real v = 0.5 * (l + r) > 0.0 ? l : r;
                        tr(i, j, k) = test ? 0.0 : v;
                    } else {
                        const real w0c = w0a(i, j, k, 1);
                        bool test = (l + w0c <= 0.0 && r + w0c >= 0.0) || (fab(l + r + 2.0 * w0c) < rel_eps);
                        real v = 0.5 * (l + r) + w0c > 0.0 ? l : r;
                        tr(i, j, k) = test ? 0.0 : v;
                    }
                }
            }
        }
        SyncFaces(utrans);
    }

    // MakeVelForce, planar 2-D (Source/MaestroForce.cpp:100-137, 253-259)
    void MakeVelForce(MF& vel_force, MF* uedge, MF& sold, MF& w0_force_cart) {
        MF grav_cart, rho0_cart;
        grav_cart.define(L().ba, 2, 1, -1, 0.0);
        rho0_cart.define(L().ba, 1, 1, -1, 0.0);
        Put1dArrayOnCart(S.rho0_old, rho0_cart, false, false, &S.bcs_s, Rho, false);
        Put1dArrayOnCart(S.grav_cell, grav_cart, false, true, &S.bcs_f, 0, false);
        vel_force.setVal(0.0);
        const int domhi = L().dom.hi[1];
        for (int b = 0; b < nb; ++b) {
            const Arr& gpi_arr = S.gpi[b];
            const Arr& rho_arr = sold[b];
            const Arr& vedge = uedge[1][b];
            const Arr& w0_arr = S.w0_cart[b];
            const Arr& w0f = w0_force_cart[b];
            const Arr& grav = grav_cart[b];
            const Arr& r0 = rho0_cart[b];
            const Arr& vf = vel_force[b];
            MO_FOR3(L().ba[b]) {
                real rhopert = rho_arr(i, j, k) - r0(i, j, k);
                if (rho_arr(i, j, k) < (S.P.buoyancy_cutoff_factor * S.P.base_cutoff_density)) rhopert = 0.0;
                vf(i, j, k, 0) = -gpi_arr(i, j, k, 0) / rho_arr(i, j, k);
                vf(i, j, k, 1) = (rhopert * grav(i, j, k, 1) - gpi_arr(i, j, k, 1)) / rho_arr(i, j, k) - w0f(i, j, k, 1);
                if (j <= -1 || j >= domhi) {
                } else {
                    vf(i, j, k, 1) -= (vedge(i, j + 1, k) + vedge(i, j, k)) *
                                      (w0_arr(i, j + 1, k, 1) - w0_arr(i, j, k, 1)) / (2.0 * L().dx[1]);
                }
            }
        }
        FillPatch(S.L, vel_force, 0, 2, 0, S.bcs_u, true);
    }

    // VelPred, 2-D (Source/MaestroVelPred.cpp:80-160, 294-727)
    void VelPred(MF& utilde, MF& ufull, MF* utrans, MF* umac, MF& force) {
        const real dt2 = 0.5 * dt, dt4 = 0.25 * dt;
        const int* domlo = L().dom.lo;
        const int* domhi = L().dom.hi;
        const real hx = L().dx[0], hy = L().dx[1];
        MF Ipu, Imu, Ipv, Imv;
        Ipu.define(L().ba, 2, 1);
        Imu.define(L().ba, 2, 1);
        Ipv.define(L().ba, 2, 1);
        Imv.define(L().ba, 2, 1);
        MF ulx, urx, uimhx, uly, ury, uimhy;
        for (MF* m : {&ulx, &urx, &uimhx, &uly, &ury, &uimhy}) m->define(L().ba, 2, 1);
        MF& velsrc = (S.P.ppm_type == 0) ? utilde : ufull;
        for (int b = 0; b < nb; ++b) {
            const Box obx = g2(L().ba[b], 1);
            const Arr& ut = utilde[b];
            const Arr& uf = ufull[b];
            if (S.P.ppm_type == 0) {
                Slope_dir(S.P.slope_order, L().dom, obx, ut, Ipu[b], 2, S.bcs_u, 0, 0);
                Slope_dir(S.P.slope_order, L().dom, obx, ut, Imv[b], 2, S.bcs_u, 0, 1);
            } else {
                for (int c = 0; c < 2; ++c) {
                    const Arr& Ip = c == 0 ? Ipu[b] : Ipv[b];
                    const Arr& Im = c == 0 ? Imu[b] : Imv[b];
                    PPM_dir(S.pc, obx, ut, c, velsrc[b].comp(0), Ip, Im, 0, S.bcs_u[c].lo[0], S.bcs_u[c].hi[0], false);
                    PPM_dir(S.pc, obx, ut, c, velsrc[b].comp(1), Ip, Im, 1, S.bcs_u[c].lo[1], S.bcs_u[c].hi[1], false);
                }
            }
            // VelPredInterface, x faces (:327-402)
            {
                const Box mxbx = growLo(obx, 0, -1);
                const Arr &l = ulx[b], &r = urx[b], &im = uimhx[b], &tr = utrans[0][b];
                const int bclo = S.P.phys_bc_lo[0], bchi = S.P.phys_bc_hi[0];
                MO_FOR3(mxbx) {
                    if (S.P.ppm_type == 0) {
                        const real maxu = mx(0.0, uf(i - 1, j, k, 0));
                        const real minu = mn(0.0, uf(i, j, k, 0));
                        for (int n = 0; n < 2; ++n) {
                            l(i, j, k, n) = ut(i - 1, j, k, n) + (0.5 - (dt2 / hx) * maxu) * Ipu[b](i - 1, j, k, n);
                            r(i, j, k, n) = ut(i, j, k, n) - (0.5 + (dt2 / hx) * minu) * Ipu[b](i, j, k, n);
                        }
                    } else {
                        l(i, j, k, 0) = Ipu[b](i - 1, j, k, 0);
                        l(i, j, k, 1) = Ipv[b](i - 1, j, k, 0);
                        r(i, j, k, 0) = Imu[b](i, j, k, 0);
                        r(i, j, k, 1) = Imv[b](i, j, k, 0);
                    }
                    if (i == domlo[0]) {
                        switch (bclo) {
                            case inflow:
                                for (int n = 0; n < 2; ++n) l(i, j, k, n) = r(i, j, k, n) = ut(i - 1, j, k, n);
                                break;
                            case slipwall: case symmetry:
                                l(i, j, k, 0) = 0.0;
                                r(i, j, k, 0) = 0.0;
                                l(i, j, k, 1) = r(i, j, k, 1);
                                break;
                            case noslipwall:
                                for (int n = 0; n < 2; ++n) l(i, j, k, n) = r(i, j, k, n) = 0.0;
                                break;
                            case outflow:
                                r(i, j, k, 0) = mn(r(i, j, k, 0), 0.0);
                                for (int n = 0; n < 2; ++n) r(i, j, k, n) = l(i, j, k, n);
                                break;
                            default: break;
                        }
                    } else if (i == domhi[0] + 1) {
                        switch (bchi) {
                            case inflow:
                                for (int n = 0; n < 2; ++n) l(i, j, k, n) = r(i, j, k, n) = ut(i, j, k, n);
                                break;
                            case slipwall: case symmetry:
                                l(i, j, k, 0) = 0.0;
                                r(i, j, k, 0) = 0.0;
                                r(i, j, k, 1) = l(i, j, k, 1);
                                break;
                            case noslipwall:
                                for (int n = 0; n < 2; ++n) l(i, j, k, n) = r(i, j, k, n) = 0.0;
                                break;
                            case outflow:
                                l(i, j, k, 0) = mx(l(i, j, k, 0), 0.0);
                                for (int n = 0; n < 2; ++n) r(i, j, k, n) = l(i, j, k, n);
                                break;
                            default: break;
                        }
                    }
                    real v = tr(i, j, k) > 0.0 ? l(i, j, k, 1) : r(i, j, k, 1);
                    im(i, j, k, 1) = fab(tr(i, j, k)) < rel_eps ? 0.5 * (l(i, j, k, 1) + r(i, j, k, 1)) : v;
                }
            }
            // VelPredInterface, y faces (:440-537)
            {
                const Box mybx = growLo(obx, 1, -1);
                const Arr &l = uly[b], &r = ury[b], &im = uimhy[b], &tr = utrans[1][b];
                const int bclo = S.P.phys_bc_lo[1], bchi = S.P.phys_bc_hi[1];
                MO_FOR3(mybx) {
                    if (S.P.ppm_type == 0) {
                        const real maxu = mx(0.0, uf(i, j - 1, k, 1));
                        const real minu = mn(0.0, uf(i, j, k, 1));
                        for (int n = 0; n < 2; ++n) {
                            l(i, j, k, n) = ut(i, j - 1, k, n) + (0.5 - (dt2 / hy) * maxu) * Imv[b](i, j - 1, k, n);
                            r(i, j, k, n) = ut(i, j, k, n) - (0.5 + (dt2 / hy) * minu) * Imv[b](i, j, k, n);
                        }
                    } else {
                        l(i, j, k, 0) = Ipu[b](i, j - 1, k, 1);
                        l(i, j, k, 1) = Ipv[b](i, j - 1, k, 1);
                        r(i, j, k, 0) = Imu[b](i, j, k, 1);
                        r(i, j, k, 1) = Imv[b](i, j, k, 1);
                    }
                    if (j == domlo[1]) {
                        switch (bclo) {
                            case inflow:
                                for (int n = 0; n < 2; ++n) l(i, j, k, n) = r(i, j, k, n) = ut(i, j - 1, k, n);
                                break;
                            case slipwall: case symmetry:
                                l(i, j, k, 0) = r(i, j, k, 0);
                                l(i, j, k, 1) = 0.0;
                                r(i, j, k, 1) = 0.0;
                                break;
                            case noslipwall:
                                for (int n = 0; n < 2; ++n) l(i, j, k, n) = r(i, j, k, n) = 0.0;
                                break;
                            case outflow:
                                r(i, j, k, 1) = mn(r(i, j, k, 1), 0.0);
                                for (int n = 0; n < 2; ++n) l(i, j, k, n) = r(i, j, k, n);
                                break;
                            default: break;
                        }
                    } else if (j == domhi[1] + 1) {
                        switch (bchi) {
                            case inflow:
                                for (int n = 0; n < 2; ++n) l(i, j, k, n) = r(i, j, k, n) = ut(i, j, k, n);
                                break;
                            case slipwall: case symmetry:
                                r(i, j, k, 0) = l(i, j, k, 0);
                                l(i, j, k, 1) = 0.0;
                                r(i, j, k, 1) = 0.0;
                                break;
                            case noslipwall:
                                for (int n = 0; n < 2; ++n) l(i, j, k, n) = r(i, j, k, n) = 0.0;
                                break;
                            case outflow:
                                l(i, j, k, 1) = mx(l(i, j, k, 1), 0.0);
                                for (int n = 0; n < 2; ++n) r(i, j, k, n) = l(i, j, k, n);
                                break;
                            default: break;
                        }
                    }
                    real v = tr(i, j, k) > 0.0 ? l(i, j, k, 0) : r(i, j, k, 0);
                    im(i, j, k, 0) = fab(tr(i, j, k)) < rel_eps ? 0.5 * (l(i, j, k, 0) + r(i, j, k, 0)) : v;
                }
            }
            // VelPredVelocities (:582-725)
            {
                const Box xbx = nodal(L().ba[b], 0);
                const Arr &l = ulx[b], &r = urx[b], &vtr = utrans[1][b], &qy = uimhy[b], &f = force[b];
                const Arr& out = umac[0][b];
                const int bclo = S.P.phys_bc_lo[0], bchi = S.P.phys_bc_hi[0];
                MO_FOR3(xbx) {
                    const real fl = f(i - 1, j, k, 0), fr = f(i, j, k, 0);
                    const real ml = l(i, j, k, 0) -
                                      (dt4 / hy) * (vtr(i - 1, j + 1, k) + vtr(i - 1, j, k)) *
                                          (qy(i - 1, j + 1, k, 0) - qy(i - 1, j, k, 0)) +
                                      dt2 * fl;
                    const real mr = r(i, j, k, 0) -
                                      (dt4 / hy) * (vtr(i, j + 1, k) + vtr(i, j, k)) *
                                          (qy(i, j + 1, k, 0) - qy(i, j, k, 0)) +
                                      dt2 * fr;
                    real v = 0.5 * (ml + mr) > 0.0 ? ml : mr;
                    v = (ml <= 0.0 && mr >= 0.0) || (fab(ml + mr) < rel_eps) ? 0.0 : v;
                    if (i == domlo[0]) {
                        switch (bclo) {
                            case inflow: v = ut(i - 1, j, k, 0); break;
                            case slipwall: case noslipwall: case symmetry: v = 0.0; break;
                            case outflow: v = mn(mr, 0.0); break;
                            default: break;
                        }
                    } else if (i == domhi[0] + 1) {
                        switch (bchi) {
                            case inflow: v = ut(i, j, k, 0); break;
                            case slipwall: case noslipwall: case symmetry: v = 0.0; break;
                            case outflow: v = mx(ml, 0.0); break;
                            default: break;
                        }
                    }
                    out(i, j, k) = v;
                }
            }
            {
                const Box ybx = nodal(L().ba[b], 1);
                const Arr &l = uly[b], &r = ury[b], &utr = utrans[0][b], &qx = uimhx[b], &f = force[b];
                const Arr& out = umac[1][b];
                const Arr& w0a = S.w0_cart[b];
                const int bclo = S.P.phys_bc_lo[1], bchi = S.P.phys_bc_hi[1];
                MO_FOR3(ybx) {
                    const real fl = f(i, j - 1, k, 1), fr = f(i, j, k, 1);
                    const real ml = l(i, j, k, 1) -
                                      (dt4 / hx) * (utr(i + 1, j - 1, k) + utr(i, j - 1, k)) *
                                          (qx(i + 1, j - 1, k, 1) - qx(i, j - 1, k, 1)) +
                                      dt2 * fl;
                    const real mr = r(i, j, k, 1) -
                                      (dt4 / hx) * (utr(i + 1, j, k) + utr(i, j, k)) *
                                          (qx(i + 1, j, k, 1) - qx(i, j, k, 1)) +
                                      dt2 * fr;
                    const real w0c = w0a(i, j, k, 1);
                    const bool test = (ml + w0c <= 0.0 && mr + w0c >= 0.0) || (fab(ml + mr + 2.0 * w0c) < rel_eps);
                    real v = 0.5 * (ml + mr) + w0c > 0.0 ? ml : mr;
                    v = test ? 0.0 : v;
                    if (j == domlo[1]) {
                        switch (bclo) {
                            case inflow: v = ut(i, j - 1, k, 1); break;
                            case slipwall: case noslipwall: case symmetry: v = 0.0; break;
                            case outflow: v = mn(mr, 0.0); break;
                            default: break;
                        }
                    } else if (j == domhi[1] + 1) {
                        switch (bchi) {
                            case inflow: v = ut(i, j, k, 1); break;
                            case slipwall: case noslipwall: case symmetry: v = 0.0; break;
                            case outflow: v = mx(ml, 0.0); break;
                            default: break;
                        }
                    }
                    out(i, j, k) = v;
                }
            }
        }
    }

    // AdvancePremac (Source/MaestroAdvection.cpp:7-84), 2-D
    void AdvancePremac(MF& uold, MF& sold, MF* umac, MF& w0_force_cart, MF* utrans, MF& vel_force) {
        MF utilde, ufull;
        utilde.define(L().ba, 2, ng_adv, -1, 0.0);
        for (int b = 0; b < nb; ++b)
            MO_FOR3(L().ba[b]) for (int n = 0; n < 2; ++n) utilde[b](i, j, k, n) = uold[b](i, j, k, n);
        FillPatch(S.L, utilde, 0, 2, 0, S.bcs_u, true);
        ufull.define(L().ba, 2, ng_adv, -1, 0.0);
        for (int b = 0; b < nb; ++b)
            MO_FOR3(L().ba[b]) for (int n = 0; n < 2; ++n) ufull[b](i, j, k, n) = S.w0_cart[b](i, j, k, n);
        FillPatch(S.L, ufull, 0, 2, 0, S.bcs_u, true);
        for (int b = 0; b < nb; ++b)
            MO_FOR3(grow(L().ba[b], ng_adv)) for (int n = 0; n < 2; ++n) ufull[b](i, j, k, n) += utilde[b](i, j, k, n);
        for (int d = 0; d < 2; ++d) utrans[d].define(L().ba, 1, 1, d, 0.0);
        MakeUtrans(utilde, ufull, utrans);
        vel_force.define(L().ba, 2, 1, -1, 0.0);
        MakeVelForce(vel_force, utrans, sold, w0_force_cart);
        Addw0(utrans, 1.0);
        VelPred(utilde, ufull, utrans, umac, vel_force);
    }

    // MakeEdgeScal, 2-D, is_vel = false (Source/MaestroMakeEdgeScalars.cpp:85-168, 306-644)
    void MakeEdgeScal(MF& state, MF* sedge, MF* umac, MF& force, const std::vector<BCRec>& bcs, int start_scomp,
                      int start_bccomp, int num_comp, bool is_conservative) {
        const int* domlo = L().dom.lo;
        const int* domhi = L().dom.hi;
        const real hx = L().dx[0], hy = L().dx[1];
        const real dt2 = 0.5 * dt, dt4 = 0.25 * dt;
        MF Ip, Im, slx, srx, sly, sry, simhx, simhy;
        Ip.define(L().ba, 2, 1);
        Im.define(L().ba, 2, 1);
        for (MF* m : {&slx, &srx, &sly, &sry, &simhx, &simhy}) m->define(L().ba, 1, 1, -1, 0.0);
        for (int scomp = start_scomp; scomp < start_scomp + num_comp; ++scomp) {
            const int bccomp = start_bccomp + scomp - start_scomp;
            const int comp = scomp;
            const int bc_lo[2] = {bcs[bccomp].lo[0], bcs[bccomp].lo[1]};
            const int bc_hi[2] = {bcs[bccomp].hi[0], bcs[bccomp].hi[1]};
            for (int b = 0; b < nb; ++b) {
                const Box obx = g2(L().ba[b], 1);
                const Arr& s = state[b];
                const Arr& um = umac[0][b];
                const Arr& vm = umac[1][b];
                if (S.P.ppm_type == 0) {
                    Arr sc = s.comp(comp);
                    sc.nc = 1;
                    std::vector<BCRec> one(1, bcs[bccomp]);
                    Slope_dir(S.P.slope_order, L().dom, obx, sc, Ip[b], 1, one, 0, 0);
                    Slope_dir(S.P.slope_order, L().dom, obx, sc, Im[b], 1, one, 0, 1);
                } else {
                    PPM_dir(S.pc, obx, s, comp, um, Ip[b], Im[b], 0, bc_lo[0], bc_hi[0], true);
                    PPM_dir(S.pc, obx, s, comp, vm, Ip[b], Im[b], 1, bc_lo[1], bc_hi[1], true);
                }
                // MakeEdgeScalPredictor (:306-452)
                for (int d = 0; d < 2; ++d) {
                    const Box mbx = growLo(obx, d, -1);
                    const int di = d == 0, dj = d == 1;
                    const Arr& l = d == 0 ? slx[b] : sly[b];
                    const Arr& r = d == 0 ? srx[b] : sry[b];
                    const Arr& sm = d == 0 ? simhx[b] : simhy[b];
                    const Arr& ud = d == 0 ? um : vm;
                    const Arr& slope = d == 0 ? Ip[b] : Im[b];
                    const real h = d == 0 ? hx : hy;
                    MO_FOR3(mbx) {
                        const int I = d == 0 ? i : j;
                        if (S.P.ppm_type == 0) {
                            l(i, j, k) = s(i - di, j - dj, k, comp) + (0.5 - dt2 * ud(i, j, k) / h) * slope(i - di, j - dj, k, 0);
                            r(i, j, k) = s(i, j, k, comp) - (0.5 + dt2 * ud(i, j, k) / h) * slope(i, j, k, 0);
                        } else {
                            l(i, j, k) = Ip[b](i - di, j - dj, k, d);
                            r(i, j, k) = Im[b](i, j, k, d);
                        }
                        if (I == domlo[d]) {
                            const int t = bc_lo[d];
                            if (t == ext_dir) {
                                l(i, j, k) = s(i - di, j - dj, k, comp);
                                r(i, j, k) = s(i - di, j - dj, k, comp);
                            } else if (t == foextrap || t == hoextrap || t == reflect_even) {
                                l(i, j, k) = r(i, j, k);
                            } else if (t == reflect_odd) {
                                l(i, j, k) = 0.0;
                                r(i, j, k) = 0.0;
                            }
                        } else if (I == domhi[d] + 1) {
                            const int t = bc_hi[d];
                            if (t == ext_dir) {
                                l(i, j, k) = s(i, j, k, comp);
                                r(i, j, k) = s(i, j, k, comp);
                            } else if (t == foextrap || t == hoextrap || t == reflect_even) {
                                r(i, j, k) = l(i, j, k);
                            } else if (t == reflect_odd) {
                                l(i, j, k) = 0.0;
                                r(i, j, k) = 0.0;
                            }
                        }
                        sm(i, j, k) = (ud(i, j, k) > 0.0) ? l(i, j, k) : r(i, j, k);
                        sm(i, j, k) = (fab(ud(i, j, k)) > rel_eps) ? sm(i, j, k) : 0.5 * (l(i, j, k) + r(i, j, k));
                    }
                }
                // MakeEdgeScalEdges (:454-644)
                for (int d = 0; d < 2; ++d) {
                    const Box xbx = nodal(L().ba[b], d);
                    const int di = d == 0, dj = d == 1;
                    const int ti = d == 1, tj = d == 0;  // transverse direction offsets
                    const Arr& l = d == 0 ? slx[b] : sly[b];
                    const Arr& r = d == 0 ? srx[b] : sry[b];
                    const Arr& st = d == 0 ? simhy[b] : simhx[b];
                    const Arr& ut = d == 0 ? vm : um;
                    const Arr& ud = d == 0 ? um : vm;
                    const real ht = d == 0 ? hy : hx, hd = d == 0 ? hx : hy;
                    const Arr& f = force[b];
                    const Arr& se = sedge[d][b];
                    MO_FOR3(xbx) {
                        const int I = d == 0 ? i : j;
                        const int il = i - di, jl = j - dj;
                        const real fl = f(il, jl, k, comp), fr = f(i, j, k, comp);
                        real lq, rq;
                        if (is_conservative) {
                            lq = l(i, j, k) -
                                 (dt2 / ht) * (st(il + ti, jl + tj, k) * ut(il + ti, jl + tj, k) -
                                               st(il, jl, k) * ut(il, jl, k)) -
                                 (dt2 / hd) * s(il, jl, k, comp) * (ud(i, j, k) - ud(il, jl, k)) + dt2 * fl;
                            rq = r(i, j, k) -
                                 (dt2 / ht) * (st(i + ti, j + tj, k) * ut(i + ti, j + tj, k) - st(i, j, k) * ut(i, j, k)) -
                                 (dt2 / hd) * s(i, j, k, comp) * (ud(i + di, j + dj, k) - ud(i, j, k)) + dt2 * fr;
                        } else {
                            lq = l(i, j, k) -
                                 (dt4 / ht) * (ut(il + ti, jl + tj, k) + ut(il, jl, k)) *
                                     (st(il + ti, jl + tj, k) - st(il, jl, k)) +
                                 dt2 * fl;
                            rq = r(i, j, k) -
                                 (dt4 / ht) * (ut(i + ti, j + tj, k) + ut(i, j, k)) * (st(i + ti, j + tj, k) - st(i, j, k)) +
                                 dt2 * fr;
                        }
                        real v = (ud(i, j, k) > 0.0) ? lq : rq;
                        v = (fab(ud(i, j, k)) > rel_eps) ? v : 0.5 * (lq + rq);
                        if (I == domlo[d]) {
                            const int t = bc_lo[d];
                            if (t == ext_dir) v = s(il, jl, k, comp);
                            else if (t == foextrap || t == hoextrap || t == reflect_even) v = rq;
                            else if (t == reflect_odd) v = 0.0;
                        } else if (I == domhi[d] + 1) {
                            const int t = bc_hi[d];
                            if (t == ext_dir) v = s(i, j, k, comp);
                            else if (t == foextrap || t == hoextrap || t == reflect_even) v = lq;
                            else if (t == reflect_odd) v = 0.0;
                        }
                        se(i, j, k, comp) = v;
                    }
                }
            }
        }
    }

    // ModifyScalForce, planar 2-D (Source/MaestroForce.cpp:261-467)
    void ModifyScalForce(MF& scal_force, MF& state, MF* umac, const std::vector<real>& s0_edge, MF& s0_cart,
                         int comp, int fullform) {
        MF s0_edge_cart;
        s0_edge_cart.define(L().ba, 1, 1);
        Put1dArrayOnCart(s0_edge, s0_edge_cart, false, false, &S.bcs_f, 0, false);
        const double* dx = L().dx;
        for (int b = 0; b < nb; ++b) {
            const Arr scal = state[b].comp(comp);
            const Arr& um = umac[0][b];
            const Arr& vm = umac[1][b];
            const Arr& s0a = s0_cart[b];
            const Arr& s0e = s0_edge_cart[b];
            const Arr& w0a = S.w0_cart[b];
            const Arr force = scal_force[b].comp(comp);
            MO_FOR3(L().ba[b]) {
                real divu = (um(i + 1, j, k) - um(i, j, k)) / dx[0] + (vm(i, j + 1, k) - vm(i, j, k)) / dx[1];
                divu += (w0a(i, j + 1, k, 1) - w0a(i, j, k, 1)) / dx[1];
                if (fullform == 1) {
                    force(i, j, k) -= scal(i, j, k) * divu;
                } else {
                    real divs0u = s0a(i, j, k) * (um(i + 1, j, k) - um(i, j, k)) / dx[0] +
                                    (vm(i, j + 1, k) * s0e(i, j + 1, k) - vm(i, j, k) * s0e(i, j, k)) / dx[1];
                    force(i, j, k) += -(scal(i, j, k) - s0a(i, j, k)) * divu - divs0u;
                }
            }
        }
        FillPatch(S.L, scal_force, comp, 1, 0, S.bcs_f, false);
    }

    // MakeRhoHForce, planar 2-D (Source/MaestroForce.cpp:469-679)
    void MakeRhoHForce(MF& scal_force, int is_prediction, MF* umac, int add_thermal, int which_step) {
        const int nr = S.nr;
        std::vector<real> r0(nr), pp0(nr);
        for (int r = 0; r < nr; ++r) {
            r0[r] = which_step == 1 ? S.rho0_old[r] : 0.5 * (S.rho0_old[r] + S.rho0_new[r]);
            pp0[r] = which_step == 1 ? S.p0_old[r] : 0.5 * (S.p0_old[r] + S.p0_new[r]);
        }
        MF p0_cart, psi_cart, grav_cart, rho0_cart;
        for (MF* m : {&p0_cart, &psi_cart, &grav_cart, &rho0_cart}) m->define(L().ba, 1, 1, -1, 0.0);
        Put1dArrayOnCart(pp0, p0_cart, false, false, &S.bcs_f, 0, false);
        Put1dArrayOnCart(S.psi, psi_cart, false, false, &S.bcs_f, 0, false);
        Put1dArrayOnCart(r0, rho0_cart, false, false, &S.bcs_s, Rho, false);
        Put1dArrayOnCart(S.grav_cell, grav_cart, false, false, &S.bcs_f, 0, false);
        const int domhi = L().dom.hi[1];
        const int cutoff = S.cutoff;
        const bool psi_in = (is_prediction == 1 && S.P.enthalpy_pred_type == 2) ||
                            (is_prediction == 1 && S.P.enthalpy_pred_type == 0) || (is_prediction == 0);
        for (int b = 0; b < nb; ++b) {
            const Arr& vm = umac[1][b];
            const Arr& p0c = p0_cart[b];
            const Arr& th = S.thermal[b];
            const Arr& ps = psi_cart[b];
            const Arr& gc = grav_cart[b];
            const Arr& rc = rho0_cart[b];
            const Arr rf = scal_force[b].comp(RhoH);
            MO_FOR3(L().ba[b]) {
                real gradp0 = 0.0;
                if (j < cutoff) gradp0 = rc(i, j, k) * gc(i, j, k);
                else if (j == domhi) gradp0 = (p0c(i, j, k) - p0c(i, j - 1, k)) / L().dx[1];
                else gradp0 = (p0c(i, j + 1, k) - p0c(i, j, k)) / L().dx[1];
                real veladv = 0.5 * (vm(i, j, k) + vm(i, j + 1, k));
                rf(i, j, k) = veladv * gradp0;
                if (psi_in) rf(i, j, k) += ps(i, j, k);
                if (add_thermal == 1) rf(i, j, k) += th(i, j, k);
            }
        }
        FillPatch(S.L, scal_force, RhoH, 1, 0, S.bcs_f, false);
    }

    // PutInPertForm, 2-D (r = j)
    void PutInPertForm(MF& scal, const std::vector<real>& s0, int comp, int bccomp, const std::vector<BCRec>& bcs,
                       bool flag) {
        for (int b = 0; b < nb; ++b) {
            const Arr& a = scal[b];
            MO_FOR3(L().ba[b]) {
                const real s0c = s0[j];
                if (flag) a(i, j, k, comp) = a(i, j, k, comp) - s0c;
                else a(i, j, k, comp) = a(i, j, k, comp) + s0c;
            }
        }
        FillPatch(S.L, scal, comp, 1, bccomp, bcs, false, comp);
    }

    // ConvertRhoHToH (Source/MaestroConvert.cpp:93-114), one level
    void ConvertRhoHToH(MF& scal, bool flag) {
        S.ConvertRhoHToH(scal, flag);
        if (flag) FillPatch(S.L, scal, RhoH, 1, 0, S.bcs_f, false, RhoH);
        else FillPatch(S.L, scal, RhoH, 1, RhoH, S.bcs_s, false, RhoH);
    }

    void ConvertRhoXToX(MF& scal, bool flag) {
        S.ConvertRhoXToX(scal, flag);
        if (flag) FillPatch(S.L, scal, FirstSpec, nspec, 0, S.bcs_f, false, FirstSpec);
        else FillPatch(S.L, scal, FirstSpec, nspec, FirstSpec, S.bcs_s, false, FirstSpec);
    }

    // MakeRhoXFlux, 2-D (Source/MaestroMakeFlux.cpp:101-182)
    void MakeRhoXFlux(MF* sflux, MF& etarhoflux, MF* sedge, MF* umac, const std::vector<real>& r0_old,
                      const std::vector<real>& r0e_old, const std::vector<real>& r0_new,
                      const std::vector<real>& r0e_new, int start_comp, int num_comp) {
        const int spt = S.P.species_pred_type;
        for (int d = 0; d < 2; ++d) sflux[d].setVal(0.0, Rho, 1, 0);
        for (int b = 0; b < nb; ++b)
            for (int d = 0; d < 2; ++d) {
                const Arr& f = sflux[d][b];
                const Arr& e = sedge[d][b];
                const Arr& u = umac[d][b];
                const Arr& eta = etarhoflux[b];
                MO_FOR3(nodal(L().ba[b], d)) {
                    for (int comp = start_comp; comp < num_comp + start_comp; ++comp) {
                        real rho0_edge = d == 0 ? 0.5 * (r0_old[j] + r0_new[j]) : 0.5 * (r0e_old[j] + r0e_new[j]);
                        if (spt == 1) f(i, j, k, comp) = u(i, j, k) * (rho0_edge + e(i, j, k, Rho)) * e(i, j, k, comp);
                        else if (spt == 2) f(i, j, k, comp) = u(i, j, k) * e(i, j, k, comp);
                        else f(i, j, k, comp) = u(i, j, k) * e(i, j, k, Rho) * e(i, j, k, comp);
                        if (d == 1 && S.P.evolve_base_state && !S.P.use_exact_base_state) {
                            if (comp >= FirstSpec && comp <= FirstSpec + nspec - 1) eta(i, j, k) += f(i, j, k, comp);
                            if (comp == FirstSpec + nspec - 1) eta(i, j, k) -= S.w0[j] * S.rho0_predicted_edge[j];
                        }
                        f(i, j, k, Rho) += f(i, j, k, comp);
                    }
                }
            }
    }

    // MakeRhoHFlux, 2-D (Source/MaestroMakeFlux.cpp:597-662)
    void MakeRhoHFlux(MF* sflux, MF* sedge, MF* umac, const std::vector<real>& rh0_old,
                      const std::vector<real>& rh0e_old, const std::vector<real>& rh0_new,
                      const std::vector<real>& rh0e_new, const std::vector<real>& r0_old,
                      const std::vector<real>& r0e_old, const std::vector<real>& r0_new,
                      const std::vector<real>& r0e_new) {
        const int ept = S.P.enthalpy_pred_type;
        const int spt = S.P.species_pred_type;
        for (int b = 0; b < nb; ++b)
            for (int d = 0; d < 2; ++d) {
                const Arr& f = sflux[d][b];
                const Arr& e = sedge[d][b];
                const Arr& u = umac[d][b];
                MO_FOR3(nodal(L().ba[b], d)) {
                    if (ept == 0) {
                        f(i, j, k, RhoH) = u(i, j, k) * e(i, j, k, RhoH);
                    } else if (ept == 2) {  // the edge state is h (Source/MaestroMakeFlux.cpp:597-662, have_h)
                        if (spt == 1) {
                            const real rho0_edge = d == 0 ? 0.5 * (r0_old[j] + r0_new[j]) : 0.5 * (r0e_old[j] + r0e_new[j]);
                            f(i, j, k, RhoH) = u(i, j, k) * (rho0_edge + e(i, j, k, Rho)) * e(i, j, k, RhoH);
                        } else {
                            f(i, j, k, RhoH) = u(i, j, k) * e(i, j, k, Rho) * e(i, j, k, RhoH);
                        }
                    } else if (d == 0) {
                        real rhoh0_edge = 0.5 * (rh0_old[j] + rh0_new[j]);
                        f(i, j, k, RhoH) = u(i, j, k) * (rhoh0_edge + e(i, j, k, RhoH));
                    } else {
                        real rhoh0_edge = 0.5 * (rh0e_old[j] + rh0e_new[j]);
                        f(i, j, k, RhoH) = u(i, j, k) * (e(i, j, k, RhoH) + rhoh0_edge);
                    }
                }
            }
    }

    // UpdateScal, 2-D (Source/MaestroAdvection.cpp:86-256)
    void UpdateScal(MF& sold, MF& snew, MF* sflux, MF& force, int start_comp, int num_comp) {
        const double* dx = L().dx;
        for (int b = 0; b < nb; ++b) {
            const Arr& so = sold[b];
            const Arr& sn = snew[b];
            const Arr& fx = sflux[0][b];
            const Arr& fy = sflux[1][b];
            const Arr& fo = force[b];
            if (start_comp == RhoH) {
                MO_FOR3(L().ba[b]) {
                    real divterm = ((fx(i + 1, j, k, RhoH) - fx(i, j, k, RhoH)) / dx[0] +
                                      (fy(i, j + 1, k, RhoH) - fy(i, j, k, RhoH)) / dx[1]);
                    sn(i, j, k, RhoH) = so(i, j, k, RhoH) + dt * (-divterm + fo(i, j, k, RhoH));
                    if (S.P.do_eos_h_above_cutoff && sn(i, j, k, Rho) <= S.P.base_cutoff_density)
                        throw std::runtime_error("UpdateScal: cell at or below base_cutoff_density needs the EOS");
                }
            } else {
                for (int n = 0; n < nspec; ++n) {
                    const int comp = FirstSpec + n;
                    MO_FOR3(L().ba[b]) {
                        real divterm = (fx(i + 1, j, k, comp) - fx(i, j, k, comp)) / dx[0];
                        divterm += (fy(i, j + 1, k, comp) - fy(i, j, k, comp)) / dx[1];
                        sn(i, j, k, comp) = so(i, j, k, comp) + dt * (-divterm + fo(i, j, k, comp));
                    }
                }
                MO_FOR3(L().ba[b]) {
                    sn(i, j, k, Rho) = so(i, j, k, Rho);
                    bool has_negative_species = false;
                    for (int comp = start_comp; comp < start_comp + nspec; ++comp) {
                        sn(i, j, k, Rho) += sn(i, j, k, comp) - so(i, j, k, comp);
                        if (sn(i, j, k, comp) < 0.0) has_negative_species = true;
                    }
                    if (sn(i, j, k, Rho) < 0.5 * S.P.base_cutoff_density) {
                        for (int comp = start_comp; comp < start_comp + nspec; ++comp)
                            sn(i, j, k, comp) *= 0.5 * S.P.base_cutoff_density / sn(i, j, k, Rho);
                        sn(i, j, k, Rho) = 0.5 * S.P.base_cutoff_density;
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
        FillPatch(S.L, snew, start_comp, num_comp, start_comp, S.bcs_s, false, start_comp);
        if (start_comp == FirstSpec) FillPatch(S.L, snew, Rho, 1, Rho, S.bcs_s, false, Rho);
    }

    // DensityAdvance, 2-D (Source/MaestroDensityAdvance.cpp:6-243)
    void DensityAdvance(MF& scalold, MF& scalnew, MF* sedge, MF* sflux, MF& scal_force, MF& etarhoflux, MF* umac,
                        int which_step) {
        const int spt = S.P.species_pred_type;
        std::vector<real> rho0_edge_old, rho0_edge_new;
        Lev::CelltoEdge(S.rho0_old, rho0_edge_old);
        Lev::CelltoEdge(S.rho0_new, rho0_edge_new);
        scal_force.setVal(0.0);
        MF rho0_old_cart;
        rho0_old_cart.define(L().ba, 1, 1, -1, 0.0);
        Put1dArrayOnCart(S.rho0_old, rho0_old_cart, false, false, &S.bcs_s, Rho, false);
        Addw0(umac, -1.0);
        if (spt == 1) ModifyScalForce(scal_force, scalold, umac, rho0_edge_old, rho0_old_cart, Rho, 0);
        else if (spt == 3) ModifyScalForce(scal_force, scalold, umac, rho0_edge_old, rho0_old_cart, Rho, 1);
        Addw0(umac, 1.0);
        if (spt == 1 || spt == 3) ConvertRhoXToX(scalold, true);
        if (spt == 1) PutInPertForm(scalold, S.rho0_old, Rho, 0, S.bcs_f, true);
        MakeEdgeScal(scalold, sedge, umac, scal_force, S.bcs_s, FirstSpec, FirstSpec, nspec, spt == 2);
        if (spt == 1 || spt == 3) {
            MakeEdgeScal(scalold, sedge, umac, scal_force, S.bcs_s, Rho, Rho, 1, false);
        } else {
            for (int d = 0; d < 2; ++d)
                for (int b = 0; b < nb; ++b) {
                    const Arr& e = sedge[d][b];
                    MO_FOR3(nodal(L().ba[b], d)) {
                        e(i, j, k, Rho) = e(i, j, k, FirstSpec);
                        for (int ispec = 1; ispec < nspec; ++ispec) e(i, j, k, Rho) += e(i, j, k, FirstSpec + ispec);
                    }
                }
        }
        if (spt == 1) PutInPertForm(scalold, S.rho0_old, Rho, Rho, S.bcs_s, false);
        if (spt == 1 || spt == 3) ConvertRhoXToX(scalold, false);
        if (which_step == 1)
            MakeRhoXFlux(sflux, etarhoflux, sedge, umac, S.rho0_old, rho0_edge_old, S.rho0_old, rho0_edge_old, FirstSpec,
                         nspec);
        else
            MakeRhoXFlux(sflux, etarhoflux, sedge, umac, S.rho0_old, rho0_edge_old, S.rho0_new, rho0_edge_new, FirstSpec,
                         nspec);
        scal_force.setVal(0.0);
        UpdateScal(scalold, scalnew, sflux, scal_force, FirstSpec, nspec);
    }

    // EnthalpyAdvance, 2-D (Source/MaestroEnthalpyAdvance.cpp:6-352)
    void EnthalpyAdvance(MF& scalold, MF& scalnew, MF* sedge, MF* sflux, MF& scal_force, MF* umac, int which_step) {
        const int ept = S.P.enthalpy_pred_type;
        std::vector<real> rhoh0_edge_old, rhoh0_edge_new;
        Lev::CelltoEdge(S.rhoh0_old, rhoh0_edge_old);
        Lev::CelltoEdge(S.rhoh0_new, rhoh0_edge_new);
        if (ept == 2) ConvertRhoHToH(scalold, true);  // predict_h (Source/MaestroEnthalpyAdvance.cpp:40-43)
        scal_force.setVal(0.0);
        MF rhoh0_old_cart;
        rhoh0_old_cart.define(L().ba, 1, 1, -1, 0.0);
        Addw0(umac, -1.0);
        MakeRhoHForce(scal_force, 1, umac, 1, 1);
        if (ept == 1) {
            Put1dArrayOnCart(S.rhoh0_old, rhoh0_old_cart, false, false, &S.bcs_s, RhoH, false);
            ModifyScalForce(scal_force, scalold, umac, rhoh0_edge_old, rhoh0_old_cart, RhoH, 0);
        }
        if (ept == 2)  // the force of h (:80-88)
            for (int b = 0; b < nb; ++b) {
                const Arr& f = scal_force[b];
                const Arr& so = scalold[b];
                MO_FOR3(g2(L().ba[b], 1)) f(i, j, k, RhoH) = f(i, j, k, RhoH) / so(i, j, k, Rho);
            }
        Addw0(umac, 1.0);
        if (ept == 1) PutInPertForm(scalold, S.rhoh0_old, RhoH, 0, S.bcs_f, true);
        MakeEdgeScal(scalold, sedge, umac, scal_force, S.bcs_s, RhoH, RhoH, 1, ept == 0);
        if (ept == 1) PutInPertForm(scalold, S.rhoh0_old, RhoH, RhoH, S.bcs_s, false);
        if (ept == 2) ConvertRhoHToH(scalold, false);
        std::vector<real> rho0_edge_old, rho0_edge_new;
        Lev::CelltoEdge(S.rho0_old, rho0_edge_old);
        Lev::CelltoEdge(S.rho0_new, rho0_edge_new);
        if (which_step == 1)
            MakeRhoHFlux(sflux, sedge, umac, S.rhoh0_old, rhoh0_edge_old, S.rhoh0_old, rhoh0_edge_old, S.rho0_old,
                         rho0_edge_old, S.rho0_old, rho0_edge_old);
        else
            MakeRhoHFlux(sflux, sedge, umac, S.rhoh0_old, rhoh0_edge_old, S.rhoh0_new, rhoh0_edge_new, S.rho0_old,
                         rho0_edge_old, S.rho0_new, rho0_edge_new);
        scal_force.setVal(0.0, RhoH, 1, 1);
        Addw0(umac, -1.0);
        MakeRhoHForce(scal_force, 0, umac, 0, which_step);
        Addw0(umac, 1.0);
        UpdateScal(scalold, scalnew, sflux, scal_force, RhoH, 1);
    }
};

}  // namespace mo
