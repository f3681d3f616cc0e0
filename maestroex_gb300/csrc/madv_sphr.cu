// Full-star spherical geometry of the stage (3-D, one or two levels sharing one radial grid):
// the exact base state, r_cc(i) = sqrt(0.75 + 2i) dxf, r_edge(i+1) = sqrt(0.75 + 2(i + 1/2)) dxf
// with dxf the finest cell size, and its cell-to-bin map, or uniform bins r_cc(i) = (i + 1/2)
// drf, r_edge(i) = i drf, drf = dxf / drdxfac (Source/BaseStateGeometry.cpp:86-104), and the
// spherical branches of Put1dArrayOnCart, MakeW0mac, MakeS0mac, Addw0, MakeVelForce,
// ModifyScalForce, MakeRhoHForce, PutInPertForm, MakeRhoXFlux and MakeRhoHFlux.  The
// MakeUtrans / VelPred Riemann solves with w0mac are flags of their kernels in
// madv_kernels.cu.  Divisions by dx and radii are IEEE divisions, as the reference writes
// them; `sqrt` is the correctly rounded square root.
#include "madv_exact.cuh"
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

// QuadInterp with its limiter on, the default of its declaration (Source/Maestro.H:65-68,
// Source/MaestroFill3dData.cpp:338-355): the quadratic through three points, clipped to the
// range of their values
__device__ __forceinline__ double quad_interp(double x, double x0, double x1, double x2, double y0, double y1,
                                              double y2) {
    double y = y0 + (y1 - y0) / (x1 - x0) * (x - x0) +
               ((y2 - y1) / (x2 - x1) - (y1 - y0) / (x1 - x0)) / (x2 - x0) * (x - x0) * (x - x1);
    const double m12 = y1 > y2 ? y1 : y2, mx = y0 > m12 ? y0 : m12;
    const double n12 = y1 < y2 ? y1 : y2, mn = y0 < n12 ? y0 : n12;
    if (y > mx) y = mx;
    if (y < mn) y = mn;
    return y;
}

// Put1dArrayOnCart's value of an edge-centred array (w0) at `radius` in bin `index`, with
// w0_interp_type t (Source/MaestroFill3dData.cpp:111-159 exact grid, 207-256 uniform bins);
// rcc holds nr + 1 radii (the reference reads r_cc_loc(nr_fine) for the outermost exact bin)
__device__ __forceinline__ double sph_edge_value(const SphGeo& g, const double* __restrict__ s0,
                                                 const double* __restrict__ rcc, const double* __restrict__ redge,
                                                 double radius, int index, int t) {
    const int nr = g.nr;
    double rfac;
    if (g.exact) {
        if (index < nr) rfac = (radius - redge[index + 1]) / (rcc[index + 1] - rcc[index]);
        else rfac = (radius - redge[index + 1]) / (rcc[index] - rcc[index - 1]);
    } else {
        rfac = (radius - double(index) * g.drf) / g.drf;
    }
    if (t == 1) return rfac > 0.5 ? s0[index + 1] : s0[index];
    if (t == 2) return index < nr ? rfac * s0[index + 1] + (1.0 - rfac) * s0[index] : s0[nr];
    if (index <= 0) index = 0;
    else if (index >= nr - 1) index = nr - 2;
    else if (radius - redge[index] < redge[index + 1]) index--;
    return quad_interp(radius, redge[index], redge[index + 1], redge[index + 2], s0[index], s0[index + 1],
                       s0[index + 2]);
}

// The value of a bin-centred array at `radius` on uniform bins, s0_interp_type t
// (Source/MaestroFill3dData.cpp:259-320, and MakeS0mac's types 2, 3 at face centres,
// :991-1188).  Past the last bin the reference's comparison reads beyond its radii, but
// either branch gives the last value: it is returned without the read.
__device__ __forceinline__ double sph_cell_value(const SphGeo& g, const double* __restrict__ s0,
                                                 const double* __restrict__ rcc, double radius, int t) {
    const int nr = g.nr;
    const double drf = g.drf;
    int index = int(radius / drf);
    if (t == 1) return s0[index];
    if (t == 2) {
        if (index > nr - 1) return s0[nr - 1];
        if (radius >= rcc[index]) {
            if (index >= nr - 1) return s0[nr - 1];
            return s0[index + 1] * (radius - rcc[index]) / drf + s0[index] * (rcc[index + 1] - radius) / drf;
        }
        if (index == 0) return s0[index];
        return s0[index] * (radius - rcc[index - 1]) / drf + s0[index - 1] * (rcc[index] - radius) / drf;
    }
    if (index == 0) index = 1;
    else if (index >= nr - 1) index = nr - 2;
    return quad_interp(radius, rcc[index - 1], rcc[index], rcc[index + 1], s0[index - 1], s0[index], s0[index + 1]);
}

// the value of a bin-centred array at cell (i, j, k): injected from the cell's bin (exact
// grid) or interpolated with s0_interp_type (uniform bins)
__device__ __forceinline__ double sph_cell_at(const SphGeo& g, const double* __restrict__ s0,
                                              const double* __restrict__ rcc, int i, int j, int k) {
    if (g.exact) return s0[sph_bin(g, i, j, k)];
    double x, y, z;
    sph_xyz(g, i, j, k, x, y, z);
    return sph_cell_value(g, s0, rcc, sqrt(x * x + y * y + z * z), g.s0i);
}

// Put1dArrayOnCart, spherical (Source/MaestroFill3dData.cpp:94-336): an edge-centred array
// (w0) with w0_interp_type, a cell-centred one injected (exact grid) or interpolated with
// s0_interp_type (uniform bins); vector output = value times the radial unit vector.
__global__ void k_put1d_sph(KARGS, int f, const double* __restrict__ s0, int outcomp, int edge, int vec,
                            const double* __restrict__ rcc, const double* __restrict__ redge, SphGeo g) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    double x, y, z;
    sph_xyz(g, i, j, k, x, y, z);
    const double radius = sqrt(x * x + y * y + z * z);
    double v;
    if (edge) {
        const int index = g.exact ? sph_bin(g, i, j, k) : int(radius / g.drf);
        v = sph_edge_value(g, s0, rcc, redge, radius, index, g.w0i);
    } else {
        v = g.exact ? s0[sph_bin(g, i, j, k)] : sph_cell_value(g, s0, rcc, radius, g.s0i);
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
           c.b1("r_edge_loc"), c.geo);
}

// face average of a cell field over the nodal boxes grown by one: MakeW0mac with
// w0mac_interp_type 1 (Source/MaestroFill3dData.cpp:552-569, component D of w0_cart) and
// MakeS0mac with s0mac_interp_type 1 (:768-783, component 0 of s0_cart)
template <int D>
__global__ void k_face_avg(KARGS, int src, int sc, int dst) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const FabView s = VW(src);
    at(VW(dst), i, j, k) = half(at(s, i - di, j - dj, k - dk, sc) + at(s, i, j, k, sc));
}

static void face_avg(Ctx& c, int src, int comp_is_dir, int dst0) {
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 0), 1, k_face_avg<0>, c.V(), src, comp_is_dir ? 0 : 0, dst0);
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 1), 1, k_face_avg<1>, c.V(), src, comp_is_dir ? 1 : 0, dst0 + 1);
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 2), 1, k_face_avg<2>, c.V(), src, comp_is_dir ? 2 : 0, dst0 + 2);
}

// centre of the D-face (i, j, k) relative to the star's centre
template <int D>
__device__ __forceinline__ void sph_face_xyz(const SphGeo& g, int i, int j, int k, double& x, double& y, double& z) {
    x = g.plo[0] + (double(i) + (D == 0 ? 0.0 : 0.5)) * g.dx[0] - g.ctr[0];
    y = g.plo[1] + (double(j) + (D == 1 ? 0.0 : 0.5)) * g.dx[1] - g.ctr[1];
    z = g.plo[2] + (double(k) + (D == 2 ? 0.0 : 0.5)) * g.dx[2] - g.ctr[2];
}

// w0 interpolated linearly in uniform bins of drf (MakeW0mac types 2 and 4)
__device__ __forceinline__ double w0_linear(const SphGeo& g, const double* __restrict__ w0, double radius) {
    const int index = int(radius / g.drf);
    const double rfac = (radius - double(index) * g.drf) / g.drf;
    return index < g.nr ? rfac * w0[index + 1] + (1.0 - rfac) * w0[index] : w0[g.nr];
}

// MakeW0mac, w0mac_interp_type 2 / 3 (Source/MaestroFill3dData.cpp:571-680): w0 interpolated
// at the face centre (linear in uniform bins / quadratic in r_edge_loc), times the face's
// component of the radial unit vector
template <int D>
__global__ void k_w0mac_interp(KARGS, const double* __restrict__ w0, const double* __restrict__ redge, SphGeo g) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    double x, y, z;
    sph_face_xyz<D>(g, i, j, k, x, y, z);
    const double radius = sqrt(x * x + y * y + z * z);
    double v;
    if (g.w0maci == 2) {
        v = w0_linear(g, w0, radius);
    } else {
        int index = int(radius / g.drf);
        if (index <= 0) index = 0;
        else if (index >= g.nr - 1) index = g.nr - 2;
        else if (radius - redge[index] < redge[index + 1]) index--;
        v = quad_interp(radius, redge[index], redge[index + 1], redge[index + 2], w0[index], w0[index + 1],
                        w0[index + 2]);
    }
    at(VW(F_W0MAC0 + D), i, j, k) = v * (D == 0 ? x : D == 1 ? y : z) / radius;
}

// MakeW0mac, w0mac_interp_type 4, the nodes (Source/MaestroFill3dData.cpp:497-540): w0 at the
// nodes of the box grown by one (node (i,j,k) kept at cell (i,j,k) of F_W0NODAL), radial
// components; at the centre itself every component takes the value
__global__ void k_w0_nodal(KARGS, const double* __restrict__ w0, SphGeo g) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const double x = g.plo[0] + double(i) * g.dx[0] - g.ctr[0];
    const double y = g.plo[1] + double(j) * g.dx[1] - g.ctr[1];
    const double z = g.plo[2] + double(k) * g.dx[2] - g.ctr[2];
    const double radius = sqrt(x * x + y * y + z * z);
    const double v = w0_linear(g, w0, radius);
    const FabView o = VW(F_W0NODAL);
    if (radius == 0.0) {
        for (int n = 0; n < 3; ++n) at(o, i, j, k, n) = v;
    } else {
        at(o, i, j, k, 0) = v * x / radius;
        at(o, i, j, k, 1) = v * y / radius;
        at(o, i, j, k, 2) = v * z / radius;
    }
}

// MakeW0mac, w0mac_interp_type 4, the faces (:682-706): the mean of the face's four nodes
template <int D>
__global__ void k_w0mac_nodal(KARGS) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int T1 = D == 0 ? 1 : 0, T2 = D == 2 ? 1 : 2;
    constexpr int ai = T1 == 0, aj = T1 == 1, ak = T1 == 2, bi = T2 == 0, bj = T2 == 1, bk = T2 == 2;
    const FabView n = VW(F_W0NODAL);
    at(VW(F_W0MAC0 + D), i, j, k) = 0.25 * (at(n, i, j, k, D) + at(n, i + ai, j + aj, k + ak, D) +
                                            at(n, i + bi, j + bj, k + bk, D) +
                                            at(n, i + ai + bi, j + aj + bj, k + ak + bk, D));
}

// Maestro::MakeW0mac (Source/MaestroFill3dData.cpp:464-710) over the nodal boxes grown by one
void make_w0mac(Ctx& c) {
    const int t = c.geo.w0maci;
    if (t == 1) return face_avg(c, F_W0CART, 1, F_W0MAC0);
    const double* w0 = c.b1("w0");
    if (t == 2 || t == 3) {
        const double* re = c.b1("r_edge_loc");
        launch(c, region(c, 1, 1, 1, 1, 1, 1, 0), 1, k_w0mac_interp<0>, c.V(), w0, re, c.geo);
        launch(c, region(c, 1, 1, 1, 1, 1, 1, 1), 1, k_w0mac_interp<1>, c.V(), w0, re, c.geo);
        launch(c, region(c, 1, 1, 1, 1, 1, 1, 2), 1, k_w0mac_interp<2>, c.V(), w0, re, c.geo);
        return;
    }
    // nodes lo - 1 .. hi + 2 of every box: the cells grown by one, plus one on the high side
    launch(c, region(c, 1, 1, 1, 2, 2, 2, -1), 1, k_w0_nodal, c.V(), w0, c.geo);
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 0), 1, k_w0mac_nodal<0>, c.V());
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 1), 1, k_w0mac_nodal<1>, c.V());
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 2), 1, k_w0mac_nodal<2>, c.V());
}

void make_s0mac_faces(Ctx& c, int dst0) { face_avg(c, F_S0CART2, 0, dst0); }

// MakeS0mac, uniform bins, s0mac_interp_type 2 / 3 (Source/MaestroFill3dData.cpp:991-1188): s0
// interpolated at the face centres as Put1dArrayOnCart does at the cell centres
template <int D>
__global__ void k_s0mac_interp(KARGS, const double* __restrict__ s0, const double* __restrict__ rcc, int dst,
                               SphGeo g) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    double x, y, z;
    sph_face_xyz<D>(g, i, j, k, x, y, z);
    at(VW(dst), i, j, k) = sph_cell_value(g, s0, rcc, sqrt(x * x + y * y + z * z), g.s0maci);
}

void make_s0mac_interp(Ctx& c, const double* d_s0, int dst0) {
    const double* rc = c.b1("r_cc_loc");
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 0), 1, k_s0mac_interp<0>, c.V(), d_s0, rc, dst0, c.geo);
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 1), 1, k_s0mac_interp<1>, c.V(), d_s0, rc, dst0 + 1, c.geo);
    launch(c, region(c, 1, 1, 1, 1, 1, 1, 2), 1, k_s0mac_interp<2>, c.V(), d_s0, rc, dst0 + 2, c.geo);
}

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

// MakeVelForce, spherical (Source/MaestroForce.cpp:151-252; MakeNormal :1190-1227).  gradw0:
// dw0/dr of the uniform bins on the cells (F_GRADW0); the exact base state has gradw0 = 0
// (:30-41), so the utilde term subtracts Ut.e_r * 0 * e_r.
__global__ void k_vel_force_sph(KARGS, double cutoff_rho, SphGeo g, int fe) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const double gradw0 = g.exact ? 0.0 : at(VW(F_GRADW0), i, j, k);
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
    const double ut_dot_er = half(at(ue, i, j, k) + at(ue, i + 1, j, k)) * nrm[0] +
                             half(at(ve, i, j, k) + at(ve, i, j + 1, k)) * nrm[1] +
                             half(at(we, i, j, k) + at(we, i, j, k + 1)) * nrm[2];
    for (int dim = 0; dim < 3; ++dim) at(vf, i, j, k, dim) -= ut_dot_er * gradw0 * nrm[dim];
}

void make_vel_force_sph(Ctx& c, int fe) {
    set_val(c, F_VELFORCE, 0.0, 0, 3, c.F[F_VELFORCE].spec.ng);
    launch(c, rg_grow(c, 0), 1, k_vel_force_sph, c.V(), c.P.buoyancy_cutoff_factor * c.P.base_cutoff_density, c.geo,
           fe);
}

// ModifyScalForce, spherical (Source/MaestroForce.cpp:335-412); divu_cart is Put1dArrayOnCart
// of divw0 (F_DIVW0, uniform bins), 0 with the exact base state (:283-302)
__global__ void k_modify_scal_force_sph(KARGS, int comp, int s0cart, int fullform, double dx0, double dx1, double dx2,
                                        int lo0, int lo1, int lo2, int hi0, int hi1, int hi2, int exact) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView um = VW(F_UMAC0), vm = VW(F_UMAC1), wm = VW(F_UMAC2), s0a = VW(s0cart);
    const double divu_c = exact ? 0.0 : at(VW(F_DIVW0), i, j, k);
    const double scal = at(VW(F_SOLD), i, j, k, comp);
    double& force = at(VW(F_SCALFORCE), i, j, k, comp);
    const double divumac = (at(um, i + 1, j, k) - at(um, i, j, k)) / dx0 + (at(vm, i, j + 1, k) - at(vm, i, j, k)) / dx1 +
                           (at(wm, i, j, k + 1) - at(wm, i, j, k)) / dx2;
    if (fullform == 1) {
        force -= scal * (divumac + divu_c);
    } else {
        const double s = at(s0a, i, j, k);
        const double sxh = i < hi0 ? half(s + at(s0a, i + 1, j, k)) : s;
        const double sxl = i > lo0 ? half(s + at(s0a, i - 1, j, k)) : s;
        const double syh = j < hi1 ? half(s + at(s0a, i, j + 1, k)) : s;
        const double syl = j > lo1 ? half(s + at(s0a, i, j - 1, k)) : s;
        const double szh = k < hi2 ? half(s + at(s0a, i, j, k + 1)) : s;
        const double szl = k > lo2 ? half(s + at(s0a, i, j, k - 1)) : s;
        const double divs0u = (at(um, i + 1, j, k) * sxh - at(um, i, j, k) * sxl) / dx0 +
                              (at(vm, i, j + 1, k) * syh - at(vm, i, j, k) * syl) / dx1 +
                              (at(wm, i, j, k + 1) * szh - at(wm, i, j, k) * szl) / dx2;
        force += -divs0u - (scal - s) * (divumac + divu_c);
    }
}

void modify_scal_force_sph(Ctx& c, int comp, int s0cart_fid, int fullform) {
    launch(c, rg_grow(c, 0), 1, k_modify_scal_force_sph, c.V(), comp, s0cart_fid, fullform, c.P.dx[0], c.P.dx[1],
           c.P.dx[2], c.P.dom_lo[0], c.P.dom_lo[1], c.P.dom_lo[2], c.P.dom_hi[0], c.P.dom_hi[1], c.P.dom_hi[2],
           c.geo.exact);
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

// PutInPertForm with the spherical Put1dArrayOnCart (cell-centred s0 injected by bin, or
// interpolated in uniform bins)
__global__ void k_pert_sph(KARGS, int comp, const double* __restrict__ s0, const double* __restrict__ rcc, int flag,
                           SphGeo g) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    double& a = at(VW(F_SOLD), i, j, k, comp);
    const double s = sph_cell_at(g, s0, rcc, i, j, k);
    a = flag ? a - s : a + s;
}

void put_in_pert_form_sph(Ctx& c, const double* d_s0, int comp, int flag) {
    launch(c, rg_grow(c, 0), 1, k_pert_sph, c.V(), comp, d_s0, c.b1("r_cc_loc"), flag, c.geo);
}

// MakeRhoXFlux, spherical (Source/MaestroMakeFlux.cpp:56-71, 306-408): the face base state is
// the LinComb 0.5 old + 0.5 new of MakeS0mac (F_S0MAC*, F_S0MACB*)
// species c0 .. c0+nc-1; slot >= 0: the one species' edge state and flux in component `slot`,
// the Rho flux carried over between calls (as in the plane-parallel kernel)
template <int D>
__global__ void k_rhox_flux_sph(KARGS, int c0, int nc, int slot, int spt) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView fl = VW(F_SEDGE0 + D), sf = VW(F_SFLUX0 + D);
    const double u = at(VW(F_UMAC0 + D), i, j, k);
    const double rho0_edge = 0.5 * at(VW(F_S0MAC0 + D), i, j, k) + 0.5 * at(VW(F_S0MACB0 + D), i, j, k);
    double frho = c0 == FIRSTSPEC ? 0.0 : at(sf, i, j, k, RHO);
    for (int comp = c0; comp < c0 + nc; ++comp) {
        const int ec = slot >= 0 ? slot : comp;
        double f = 0.0;
        if (spt == 1) f = u * (rho0_edge + at(fl, i, j, k, RHO)) * at(fl, i, j, k, ec);
        else if (spt == 2) f = u * at(fl, i, j, k, ec);
        else f = u * at(fl, i, j, k, RHO) * at(fl, i, j, k, ec);
        at(sf, i, j, k, ec) = f;
        frho += f;
    }
    at(sf, i, j, k, RHO) = frho;
}

void make_rhox_flux_sph(Ctx& c, int c0, int nc, int slot) {
    const int spt = c.P.species_pred_type;
    launch(c, rg_grow(c, 0, 0), 1, k_rhox_flux_sph<0>, c.V(), c0, nc, slot, spt);
    launch(c, rg_grow(c, 0, 1), 1, k_rhox_flux_sph<1>, c.V(), c0, nc, slot, spt);
    launch(c, rg_grow(c, 0, 2), 1, k_rhox_flux_sph<2>, c.V(), c0, nc, slot, spt);
}

// MakeRhoHFlux, spherical (Source/MaestroMakeFlux.cpp:540-575, 788-1000).  Exact base state,
// (rho h)' predicted: rhoh0 on the faces in F_S0MAC* (old) and F_S0MACB* (new).  Uniform bins:
// (rho h) predicted (ept 0); h predicted (ept 2), times rho0mac + rho' (species_pred_type 1) or
// rho; or (rho h)' with (rho h)_0 on the faces as rho0mac * h0mac, rho0 in F_S0MACC* /
// F_S0MACD*, h0 in F_S0MAC* / F_S0MACB*; each the LinComb 0.5 old + 0.5 new.
template <int D>
__global__ void k_rhoh_flux_sph(KARGS, int exact, int ept, int spt) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const double u = at(VW(F_UMAC0 + D), i, j, k), e = at(VW(F_SEDGE0 + D), i, j, k, RHOH);
    double f;
    if (exact) {
        const double rhoh0_edge = 0.5 * at(VW(F_S0MAC0 + D), i, j, k) + 0.5 * at(VW(F_S0MACB0 + D), i, j, k);
        f = u * (rhoh0_edge + e);
    } else if (ept == 0) {
        f = u * e;
    } else if (ept == 2) {
        const double rho0_edge = 0.5 * at(VW(F_S0MACC0 + D), i, j, k) + 0.5 * at(VW(F_S0MACD0 + D), i, j, k);
        const double r = at(VW(F_SEDGE0 + D), i, j, k, RHO);
        f = spt == 1 ? u * (rho0_edge + r) * e : u * r * e;
    } else {
        const double rho0_edge = 0.5 * at(VW(F_S0MACC0 + D), i, j, k) + 0.5 * at(VW(F_S0MACD0 + D), i, j, k);
        const double h0_edge = 0.5 * at(VW(F_S0MAC0 + D), i, j, k) + 0.5 * at(VW(F_S0MACB0 + D), i, j, k);
        f = u * (rho0_edge * h0_edge + e);
    }
    at(VW(F_SFLUX0 + D), i, j, k, RHOH) = f;
}

void make_rhoh_flux_sph(Ctx& c) {
    const int ex = c.geo.exact, ept = c.P.enthalpy_pred_type, spt = c.P.species_pred_type;
    launch(c, rg_grow(c, 0, 0), 1, k_rhoh_flux_sph<0>, c.V(), ex, ept, spt);
    launch(c, rg_grow(c, 0, 1), 1, k_rhoh_flux_sph<1>, c.V(), ex, ept, spt);
    launch(c, rg_grow(c, 0, 2), 1, k_rhoh_flux_sph<2>, c.V(), ex, ept, spt);
}

}  // namespace madv
