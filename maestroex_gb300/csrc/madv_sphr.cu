// Full-star spherical geometry of the stage with the exact base state (3-D, one or two
// levels sharing one radial grid): r_cc(i) = sqrt(0.75 + 2i) dxf, r_edge(i+1) = sqrt(0.75 +
// 2(i + 1/2)) dxf with dxf the finest cell size (Source/BaseStateGeometry.cpp:86-96), the
// cell-to-bin map, and the
// spherical branches of Put1dArrayOnCart, MakeW0mac, MakeS0mac, Addw0, MakeVelForce,
// ModifyScalForce, MakeRhoHForce, PutInPertForm, MakeRhoXFlux and MakeRhoHFlux.  The
// MakeUtrans / VelPred Riemann solves with w0mac are flags of their kernels in
// madv_kernels.cu.  Divisions by dx and radii are IEEE divisions, as the reference writes
// them; `sqrt` is the correctly rounded square root.
#include "madv_launch.cuh"

namespace madv {

__device__ __forceinline__ void sph_xyz(const SphGeo& g, int i, int j, int k, double& x, double& y, double& z) {
    x = g.plo[0] + (double(i) + 0.5) * g.dx[0] - g.ctr[0];
    y = g.plo[1] + (double(j) + 0.5) * g.dx[1] - g.ctr[1];
    z = g.plo[2] + (double(k) + 0.5) * g.dx[2] - g.ctr[2];
}

// Maestro::InitBaseStateMapSphr (Source/MaestroBaseStateGeometry.cpp:17-35)
__device__ __forceinline__ int sph_bin(const SphGeo& g, int i, int j, int k) {
    double x, y, z;
    sph_xyz(g, i, j, k, x, y, z);
    const double index = (x * x + y * y + z * z) / (2.0 * g.dxf * g.dxf) - 0.375;
    return (int)round(index);
}

// Put1dArrayOnCart, spherical, exact base state (Source/MaestroFill3dData.cpp:94-192): an
// edge-centred array (w0) with w0_interp_type 2 (linear in radius), a cell-centred one
// injected; vector output = value times the radial unit vector.  rcc holds nr + 1 radii:
// the reference reads r_cc_loc(nr_fine) for the outermost bin, one past its array; the
// context continues the formula there.
__global__ void k_put1d_sph(KARGS, int f, const double* __restrict__ s0, int outcomp, int edge, int vec,
                            const double* __restrict__ rcc, const double* __restrict__ redge, int nr, SphGeo g) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    double x, y, z;
    sph_xyz(g, i, j, k, x, y, z);
    const double radius = sqrt(x * x + y * y + z * z);
    const int index = sph_bin(g, i, j, k);
    double v;
    if (edge) {
        double rfac;
        if (index < nr) rfac = (radius - redge[index + 1]) / (rcc[index + 1] - rcc[index]);
        else rfac = (radius - redge[index + 1]) / (rcc[index] - rcc[index - 1]);
        if (index < nr) v = rfac * s0[index + 1] + (1.0 - rfac) * s0[index];
        else v = s0[nr];
    } else {
        v = s0[index];
    }
    const FabView o = VW(f);
    if (vec) {
        at(o, i, j, k, 0) = v * x / radius;
        at(o, i, j, k, 1) = v * y / radius;
        at(o, i, j, k, 2) = v * z / radius;
    } else {
        at(o, i, j, k, outcomp) = v;
    }
}

void put1d_sph(Ctx& c, int fid, const double* d_s0, int outcomp, int edge, int vec) {
    launch(c, rg_grow(c, 0), 1, k_put1d_sph, c.V(), fid, d_s0, outcomp, edge, vec, c.b1("r_cc_loc"),
           c.b1("r_edge_loc"), c.nr, c.geo);
}

// face average of a cell field over the nodal boxes grown by one: MakeW0mac with
// w0mac_interp_type 1 (Source/MaestroFill3dData.cpp:552-569, component D of w0_cart) and
// MakeS0mac with s0mac_interp_type 1 (:768-783, component 0 of s0_cart)
template <int D>
__global__ void k_face_avg(KARGS, int src, int sc, int dst) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const FabView s = VW(src);
    at(VW(dst), i, j, k) = 0.5 * (at(s, i - di, j - dj, k - dk, sc) + at(s, i, j, k, sc));
}

static void face_avg(Ctx& c, int src, int comp_is_dir, int dst0) {
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 0), 1, k_face_avg<0>, c.V(), src, comp_is_dir ? 0 : 0, dst0);
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 1), 1, k_face_avg<1>, c.V(), src, comp_is_dir ? 1 : 0, dst0 + 1);
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 2), 1, k_face_avg<2>, c.V(), src, comp_is_dir ? 2 : 0, dst0 + 2);
}

void make_w0mac(Ctx& c) { face_avg(c, F_W0CART, 1, F_W0MAC0); }
void make_s0mac_faces(Ctx& c, int dst0) { face_avg(c, F_S0CART2, 0, dst0); }

// Addw0, spherical (Source/MaestroFill3dData.cpp:395-419): valid faces += mult w0mac
template <int D>
__global__ void k_addw0_sph(KARGS, int f, double mult) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    at(VW(f), i, j, k) += mult * at(VW(F_W0MAC0 + D), i, j, k);
}

void addw0_sph(Ctx& c, int f0, double mult) {
    launch(c, rg_grow(c, 0, 0), 1, k_addw0_sph<0>, c.V(), f0, mult);
    launch(c, rg_grow(c, 0, 1), 1, k_addw0_sph<1>, c.V(), f0 + 1, mult);
    launch(c, rg_grow(c, 0, 2), 1, k_addw0_sph<2>, c.V(), f0 + 2, mult);
}

// MakeVelForce, spherical (Source/MaestroForce.cpp:151-252; MakeNormal :1190-1227).  The
// exact base state has gradw0 = 0 (:30-41): the utilde term subtracts Ut.e_r * 0 * e_r.
__global__ void k_vel_force_sph(KARGS, double cutoff_rho, SphGeo g, int fe) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const double gradw0 = 0.0;
    double x, y, z;
    sph_xyz(g, i, j, k, x, y, z);
    const double inv_radius = 1.0 / sqrt(x * x + y * y + z * z);
    const double nrm[3] = {x * inv_radius, y * inv_radius, z * inv_radius};
    const FabView gpi = VW(F_GPI), vf = VW(F_VELFORCE), grav = VW(F_GRAVCART), w0f = VW(F_W0FCART);
    const double r = at(VW(F_SOLD), i, j, k, RHO);
    double rhopert = r - at(VW(F_RHO0CART), i, j, k);
    if (r < cutoff_rho) rhopert = 0.0;
    for (int dim = 0; dim < 3; ++dim)
        at(vf, i, j, k, dim) = (rhopert * at(grav, i, j, k, dim) - at(gpi, i, j, k, dim)) / r - at(w0f, i, j, k, dim);
    const FabView ue = VW(fe), ve = VW(fe + 1), we = VW(fe + 2);
    const double ut_dot_er = 0.5 * (at(ue, i, j, k) + at(ue, i + 1, j, k)) * nrm[0] +
                             0.5 * (at(ve, i, j, k) + at(ve, i, j + 1, k)) * nrm[1] +
                             0.5 * (at(we, i, j, k) + at(we, i, j, k + 1)) * nrm[2];
    for (int dim = 0; dim < 3; ++dim) at(vf, i, j, k, dim) -= ut_dot_er * gradw0 * nrm[dim];
}

void make_vel_force_sph(Ctx& c, int fe) {
    set_val(c, F_VELFORCE, 0.0, 0, 3, c.F[F_VELFORCE].spec.ng);
    launch(c, rg_grow(c, 0), 1, k_vel_force_sph, c.V(), c.P.buoyancy_cutoff_factor * c.P.base_cutoff_density, c.geo,
           fe);
}

// ModifyScalForce, spherical (Source/MaestroForce.cpp:335-412); divu_cart is
// Put1dArrayOnCart of divw0 = 0 with the exact base state (:283-302)
__global__ void k_modify_scal_force_sph(KARGS, int comp, int s0cart, int fullform, double dx0, double dx1, double dx2,
                                        int lo0, int lo1, int lo2, int hi0, int hi1, int hi2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView um = VW(F_UMAC0), vm = VW(F_UMAC1), wm = VW(F_UMAC2), s0a = VW(s0cart);
    const double divu_c = 0.0;
    const double scal = at(VW(F_SOLD), i, j, k, comp);
    double& force = at(VW(F_SCALFORCE), i, j, k, comp);
    const double divumac = (at(um, i + 1, j, k) - at(um, i, j, k)) / dx0 + (at(vm, i, j + 1, k) - at(vm, i, j, k)) / dx1 +
                           (at(wm, i, j, k + 1) - at(wm, i, j, k)) / dx2;
    if (fullform == 1) {
        force -= scal * (divumac + divu_c);
    } else {
        const double s = at(s0a, i, j, k);
        const double sxh = i < hi0 ? 0.5 * (s + at(s0a, i + 1, j, k)) : s;
        const double sxl = i > lo0 ? 0.5 * (s + at(s0a, i - 1, j, k)) : s;
        const double syh = j < hi1 ? 0.5 * (s + at(s0a, i, j + 1, k)) : s;
        const double syl = j > lo1 ? 0.5 * (s + at(s0a, i, j - 1, k)) : s;
        const double szh = k < hi2 ? 0.5 * (s + at(s0a, i, j, k + 1)) : s;
        const double szl = k > lo2 ? 0.5 * (s + at(s0a, i, j, k - 1)) : s;
        const double divs0u = (at(um, i + 1, j, k) * sxh - at(um, i, j, k) * sxl) / dx0 +
                              (at(vm, i, j + 1, k) * syh - at(vm, i, j, k) * syl) / dx1 +
                              (at(wm, i, j, k + 1) * szh - at(wm, i, j, k) * szl) / dx2;
        force += -divs0u - (scal - s) * (divumac + divu_c);
    }
}

void modify_scal_force_sph(Ctx& c, int comp, int s0cart_fid, int fullform) {
    launch(c, rg_grow(c, 0), 1, k_modify_scal_force_sph, c.V(), comp, s0cart_fid, fullform, c.P.dx[0], c.P.dx[1],
           c.P.dx[2], c.P.dom_lo[0], c.P.dom_lo[1], c.P.dom_lo[2], c.P.dom_hi[0], c.P.dom_hi[1], c.P.dom_hi[2]);
}

// MakeRhoHForce, spherical (Source/MaestroForce.cpp:637-670): u.grad p0 = div(u p0) - p0 div u,
// p0 on faces in F_S0MAC0..2 (MakeS0mac of p0)
__global__ void k_rhoh_force_sph(KARGS, int psi_in, int add_thermal, double dx0, double dx1, double dx2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView um = VW(F_UMAC0), vm = VW(F_UMAC1), wm = VW(F_UMAC2);
    const FabView px = VW(F_S0MAC0), py = VW(F_S0MAC1), pz = VW(F_S0MAC2);
    const double divup = (at(um, i + 1, j, k) * at(px, i + 1, j, k) - at(um, i, j, k) * at(px, i, j, k)) / dx0 +
                         (at(vm, i, j + 1, k) * at(py, i, j + 1, k) - at(vm, i, j, k) * at(py, i, j, k)) / dx1 +
                         (at(wm, i, j, k + 1) * at(pz, i, j, k + 1) - at(wm, i, j, k) * at(pz, i, j, k)) / dx2;
    const double p0divu = ((at(um, i + 1, j, k) - at(um, i, j, k)) / dx0 + (at(vm, i, j + 1, k) - at(vm, i, j, k)) / dx1 +
                           (at(wm, i, j, k + 1) - at(wm, i, j, k)) / dx2) *
                          at(VW(F_P0CART), i, j, k);
    double f = divup - p0divu;
    if (psi_in) f += at(VW(F_PSICART), i, j, k);
    if (add_thermal == 1) f += at(VW(F_THERMAL), i, j, k);
    at(VW(F_SCALFORCE), i, j, k, RHOH) = f;
}

void make_rhoh_force_sph(Ctx& c, int is_prediction, int add_thermal) {
    const int ept = c.P.enthalpy_pred_type;
    const int psi_in = (is_prediction == 1 && ept == 2) || (is_prediction == 1 && ept == 0) || (is_prediction == 0);
    launch(c, rg_grow(c, 0), 1, k_rhoh_force_sph, c.V(), psi_in, add_thermal, c.P.dx[0], c.P.dx[1], c.P.dx[2]);
}

// PutInPertForm with the spherical Put1dArrayOnCart (cell-centred s0 injected by bin)
__global__ void k_pert_sph(KARGS, int comp, const double* __restrict__ s0, int flag, SphGeo g) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    double& a = at(VW(F_SOLD), i, j, k, comp);
    const double s = s0[sph_bin(g, i, j, k)];
    a = flag ? a - s : a + s;
}

void put_in_pert_form_sph(Ctx& c, const double* d_s0, int comp, int flag) {
    launch(c, rg_grow(c, 0), 1, k_pert_sph, c.V(), comp, d_s0, flag, c.geo);
}

// MakeRhoXFlux, spherical (Source/MaestroMakeFlux.cpp:56-71, 306-408): the face base state is
// the LinComb 0.5 old + 0.5 new of MakeS0mac (F_S0MAC*, F_S0MACB*)
template <int D>
__global__ void k_rhox_flux_sph(KARGS, int nspec, int spt) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView fl = VW(F_SEDGE0 + D), sf = VW(F_SFLUX0 + D);
    const double u = at(VW(F_UMAC0 + D), i, j, k);
    const double rho0_edge = 0.5 * at(VW(F_S0MAC0 + D), i, j, k) + 0.5 * at(VW(F_S0MACB0 + D), i, j, k);
    double frho = 0.0;
    for (int comp = FIRSTSPEC; comp < FIRSTSPEC + nspec; ++comp) {
        double f = 0.0;
        if (spt == 1) f = u * (rho0_edge + at(fl, i, j, k, RHO)) * at(fl, i, j, k, comp);
        else if (spt == 2) f = u * at(fl, i, j, k, comp);
        else f = u * at(fl, i, j, k, RHO) * at(fl, i, j, k, comp);
        at(sf, i, j, k, comp) = f;
        frho += f;
    }
    at(sf, i, j, k, RHO) = frho;
}

void make_rhox_flux_sph(Ctx& c) {
    const int ns = c.nspec, spt = c.P.species_pred_type;
    launch(c, rg_grow(c, 0, 0), 1, k_rhox_flux_sph<0>, c.V(), ns, spt);
    launch(c, rg_grow(c, 0, 1), 1, k_rhox_flux_sph<1>, c.V(), ns, spt);
    launch(c, rg_grow(c, 0, 2), 1, k_rhox_flux_sph<2>, c.V(), ns, spt);
}

// MakeRhoHFlux, spherical, exact base state, (rho h)' predicted (Source/MaestroMakeFlux.cpp:540-548,
// 788-840)
template <int D>
__global__ void k_rhoh_flux_sph(KARGS) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const double rhoh0_edge = 0.5 * at(VW(F_S0MAC0 + D), i, j, k) + 0.5 * at(VW(F_S0MACB0 + D), i, j, k);
    at(VW(F_SFLUX0 + D), i, j, k, RHOH) =
        at(VW(F_UMAC0 + D), i, j, k) * (rhoh0_edge + at(VW(F_SEDGE0 + D), i, j, k, RHOH));
}

void make_rhoh_flux_sph(Ctx& c) {
    launch(c, rg_grow(c, 0, 0), 1, k_rhoh_flux_sph<0>, c.V());
    launch(c, rg_grow(c, 0, 1), 1, k_rhoh_flux_sph<1>, c.V());
    launch(c, rg_grow(c, 0, 2), 1, k_rhoh_flux_sph<2>, c.V());
}

}  // namespace madv
