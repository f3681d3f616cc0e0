// Reverse (adjoint) sweep of the scalar path of the advection stage: the transposes of
// UpdateScal, MakeRhoXFlux / MakeRhoHFlux (species_pred_type 1, enthalpy_pred_type 1),
// MakeEdgeScal with PPM ppm_type 1 (van Leer slopes, interface values, cell-edge limiter,
// characteristic tracing, predictor, transverse and edge corrections), the pointwise
// conversions of DensityAdvance / EnthalpyAdvance and FillBoundary.
//
// Every limiter, clamp and upwind decision is recomputed from the forward inputs with the
// forward's own expressions (the same compile flags, so the same bits), i.e. the
// decisions are frozen at the forward pass; the adjoint is the transpose of the
// forward's derivative on that branch.  Scatter transposes use atomicAdd into the
// adjoint FABs, which have the forward FABs' index spaces (and zero-filled margins
// wherever a transpose reads one cell past the forward region).
//
// Scope: 3-D, one level, periodic domain, MAC velocities independent of the state
// (no buoyancy or pressure-gradient force, w0 = 0).  The forward kernels this mirrors
// are in madv_kernels.cu (k_update_rhox / k_update_rhoh, k_rhox_flux / k_rhoh_flux,
// k_es_edges, k_es_transverse, k_es_predictor, k_ppm_cell, k_ppm_face, k_dsvl,
// k_rhox_to_x, k_pert, k_modify_scal_force, k_fill_boundary).
#include "madv_launch.cuh"
#include "madv_ppm.cuh"

namespace madv {

#define AW(s) VW(F_USER + (s))

// Weights of the reference's upwinding  v = (u > 0) ? l : r  for |u| > t, (l + r)/2 otherwise.
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
// f, f-1 that lie in the box.  Then, with F_X = u (rho0_edge + rho'_e) X_e and
// F_h = u (rhoh0_edge + rhoh'_e): the edge-state adjoints go to A_AEDGE0+D.
template <int D>
__global__ void k_adj_flux(KARGS, int nspec, double dtdx, const double* __restrict__ r0a,
                           const double* __restrict__ r0b) {
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
    const double r0e = 0.5 * (r0a[k] + r0b[k]);
    const double cx = u * (r0e + at(e, i, j, k, RHO));
    double arho = 0.0;
    for (int comp = FIRSTSPEC; comp < FIRSTSPEC + nspec; ++comp) {
        const double fb = fbar(comp);
        at(ae, i, j, k, comp) = cx * fb;
        arho += u * at(e, i, j, k, comp) * fb;
    }
    at(ae, i, j, k, RHO) = arho;
    at(ae, i, j, k, RHOH) = u * fbar(RHOH);
}

// ------------------------------------------------------------------ MakeEdgeScal^T
#define AQ_SLOT(a, b) (A_AQ01 + 2 * (a) + ((b) > (a) ? (b)-1 : (b)))

// k_es_edges (advective form) transposed: valid D-faces.
template <int D>
__global__ void k_adj_es_edges(KARGS, int comp, int force_zero, double dt2, long long epsb) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    constexpr int T1 = D == 0 ? 1 : 0, T2 = D == 2 ? 1 : 2;
    constexpr int a1i = T1 == 0, a1j = T1 == 1, a1k = T1 == 2;
    constexpr int a2i = T2 == 0, a2j = T2 == 1, a2k = T2 == 2;
    const int il = i - di, jl = j - dj, kl = k - dk;
    const double ab = at(AW(A_AEDGE0 + D), i, j, k, comp);
    double wl, wr;
    upwind_w(at(VW(F_UMAC0 + D), i, j, k), epsb, wl, wr);
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
}

// k_es_transverse (advective form) transposed: D-faces corrected in direction T.
template <int D, int T>
__global__ void k_adj_es_transverse(KARGS, long long epsb) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    constexpr int ti = T == 0, tj = T == 1, tk = T == 2;
    const int il = i - di, jl = j - dj, kl = k - dk;
    const double qb = at(AW(AQ_SLOT(D, T)), i, j, k);
    double wl, wr;
    upwind_w(at(VW(F_UMAC0 + D), i, j, k), epsb, wl, wr);
    const double la = wl * qb, ra = wr * qb;
    at(AW(A_ASL0 + D), i, j, k) += la;
    at(AW(A_ASR0 + D), i, j, k) += ra;
    const FabView tc = VW(F_TCOEF), sh = AW(A_ASIMH0 + T);
    const double cl = at(tc, il, jl, kl, T) * la, cr = at(tc, i, j, k, T) * ra;
    atomicAdd(&at(sh, il + ti, jl + tj, kl + tk), -cl);
    atomicAdd(&at(sh, il, jl, kl), cl);
    atomicAdd(&at(sh, i + ti, j + tj, k + tk), -cr);
    atomicAdd(&at(sh, i, j, k), cr);
}

// k_es_predictor (ppm_type 1) transposed: simh = upwind(u, l, r, 0).
template <int D>
__global__ void k_adj_es_predictor(KARGS) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const double sb = at(AW(A_ASIMH0 + D), i, j, k);
    double wl, wr;
    upwind_w(at(VW(F_UMAC0 + D), i, j, k), 0, wl, wr);
    at(AW(A_ASL0 + D), i, j, k) += wl * sb;
    at(AW(A_ASR0 + D), i, j, k) += wr * sb;
}

// k_ppm_cell<D, 1, 1> transposed (cells of the box grown by one): the predictor reads
// l(face f) = Ip(cell f-1) and r(face f) = Im(cell f), so Ip / Im of a cell take the
// adjoints of its high / low face.  Tracing is linear in (s0, sm, sp) for the frozen
// upwind tests; the quadratic limiter (Source/MaestroPPM.cpp:117-128) is piecewise
// linear in (s0, interface values).  Interface adjoints go to A_ASM (low face) and A_ASP
// (high face) per cell, gathered per face by k_adj_ppm_face.
template <int D>
__global__ void k_adj_ppm_cell(KARGS, int fs, int sc, long long epsb) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const double ipb = at(AW(A_ASL0 + D), i + di, j + dj, k + dk);
    const double imb = at(AW(A_ASR0 + D), i, j, k);
    const FabView s = VW(fs), F = VW(F_FACE0 + D), T = VW(F_TRA0 + D), u = VW(F_UMAC0 + D);
    const double s0 = at(s, i, j, k, sc);
    double sm = at(F, i, j, k), sp = at(F, i + di, j + dj, k + dk);
    int cs = 3;
    if ((sp - s0) * (s0 - sm) <= 0.0) {
        cs = 0;
    } else if (fabs(sp - s0) >= 2.0 * fabs(sm - s0)) {
        cs = 1;
    } else if (fabs(sm - s0) >= 2.0 * fabs(sp - s0)) {
        cs = 2;
    }
    double bs0 = 0.0, bsm = 0.0, bsp = 0.0;
    if (gt_t(at(u, i + di, j + dj, k + dk), epsb)) {
        const double A = at(T, i + di, j + dj, k + dk, 0), B = at(T, i + di, j + dj, k + dk, 1);
        bsp += (1.0 - A - 3.0 * A * B) * ipb;
        bsm += (A - 3.0 * A * B) * ipb;
        bs0 += 6.0 * A * B * ipb;
    } else {
        bs0 += ipb;
    }
    if (lt_negt(at(u, i, j, k), epsb)) {
        const double A = at(T, i, j, k, 0), B = at(T, i, j, k, 1);
        bsm += (1.0 - A - 3.0 * A * B) * imb;
        bsp += (A - 3.0 * A * B) * imb;
        bs0 += 6.0 * A * B * imb;
    } else {
        bs0 += imb;
    }
    double fm = 0.0, fp = 0.0;
    if (cs == 0) {  // sm = sp = s0
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
    at(AW(A_ASM), i, j, k) = fm;
    at(AW(A_ASP), i, j, k) = fp;
    at(AW(A_AS), i, j, k) += bs0;
}

// k_ppm_face<D, 1> transposed (Source/MaestroPPM.cpp:37-111 interior form):
// v = min(max(v0, min(s0, s-1)), max(s0, s-1)), v0 = (s0 + s-1)/2 - (dv(f) - dv(f-1))/6.
template <int D>
__global__ void k_adj_ppm_face(KARGS, int fs, int sc, RecipC r6) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const double fb = at(AW(A_ASM), i, j, k) + at(AW(A_ASP), i - di, j - dj, k - dk);
    if (fb == 0.0) return;
    const FabView s = VW(fs), dv = VW(F_DSVL), as = AW(A_AS);
    const double sl = at(s, i - di, j - dj, k - dk, sc), s0 = at(s, i, j, k, sc);
    const double v0 = 0.5 * (s0 + sl) - div_c(at(dv, i, j, k) - at(dv, i - di, j - dj, k - dk), r6);
    // mn(a, b) = (b < a) ? b : a and mx(a, b) = (a < b) ? b : a, as in the forward
    const double lo = mn(s0, sl), hi = mx(s0, sl);
    int src = 0;  // 0: v0, 1: s0, 2: s-1
    double v = v0;
    if (v < lo) {
        v = lo;
        src = (sl < s0) ? 2 : 1;
    }
    if (hi < v) src = (s0 < sl) ? 2 : 1;
    if (src == 0) {
        atomicAdd(&at(as, i, j, k), 0.5 * fb);
        atomicAdd(&at(as, i - di, j - dj, k - dk), 0.5 * fb);
        const FabView ad = AW(A_ADSVL);
        atomicAdd(&at(ad, i, j, k), -fb / 6.0);
        atomicAdd(&at(ad, i - di, j - dj, k - dk), fb / 6.0);
    } else if (src == 1) {
        atomicAdd(&at(as, i, j, k), fb);
    } else {
        atomicAdd(&at(as, i - di, j - dj, k - dk), fb);
    }
}

// k_dsvl<D> transposed (Source/MaestroPPM.cpp:37-73):
// dv = sign(dsc) min(|dsc|, |dsl|, |dsr|) where dsl dsr > 0, else 0.
template <int D>
__global__ void k_adj_dsvl(KARGS, int fs, int sc) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    const double g = at(AW(A_ADSVL), i, j, k);
    if (g == 0.0) return;
    const FabView s = VW(fs), as = AW(A_AS);
    auto S = SHIFT_S(s, sc);
    const double dsc = 0.5 * (S(1) - S(-1));
    const double dsl = 2.0 * (S(0) - S(-1));
    const double dsr = 2.0 * (S(1) - S(0));
    if (!(dsl * dsr > 0.0)) return;
    const double ac = fabs(dsc), al = fabs(dsl), ar = fabs(dsr);
    const bool inner_r = ar < al;  // mn(|dsl|, |dsr|)
    const double inner = inner_r ? ar : al;
    auto add = [&](int m, double v) { atomicAdd(&at(as, i + m * di, j + m * dj, k + m * dk), v); };
    if (inner < ac) {  // dv = sign(dsc) |dsl| or sign(dsc) |dsr|
        const double sg = copysign(1.0, dsc);
        if (inner_r) {
            const double w = 2.0 * sg * copysign(1.0, dsr) * g;
            add(1, w);
            add(0, -w);
        } else {
            const double w = 2.0 * sg * copysign(1.0, dsl) * g;
            add(0, w);
            add(-1, -w);
        }
    } else {  // dv = dsc
        add(1, 0.5 * g);
        add(-1, -0.5 * g);
    }
}

// FillBoundary transposed: every ghost cell was copied from one valid cell, so its
// adjoint is added to that cell and cleared.
__global__ void k_adj_fill_boundary(const CopyDesc* __restrict__ D, int nd, long total, const FabView* __restrict__ V,
                                    int nb, int f) {
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
    double& g = at(V[f * nb + cd.dst_b], i, j, k);
    const double v = g;
    if (v != 0.0) atomicAdd(&at(V[f * nb + cd.src_b], i - cd.shift[0], j - cd.shift[1], k - cd.shift[2]), v);
    g = 0.0;
}

// ConvertRhoXToX transposed (valid cells): X = rhoX / rho.
__global__ void k_adj_x(KARGS, int comp) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const double a = at(AW(A_AS), i, j, k);
    const FabView ao = AW(A_ASOLD);
    const double rho = at(AW(A_WSOLD), i, j, k, RHO);
    const double x = at(VW(F_SOLD), i, j, k, comp);
    at(ao, i, j, k, comp) += a / rho;
    at(ao, i, j, k, RHO) -= a * x / rho;
}

// PutInPertForm transposed (s' = s - s0) together with the state term of the traced
// force, ModifyScalForce fullform 0: f = ... - (s - s0) divu - div(s0 u) (valid cells).
__global__ void k_adj_pert(KARGS, int comp, RecipC r0, RecipC r1, RecipC r2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView um = VW(F_UMAC0), vm = VW(F_UMAC1), wm = VW(F_UMAC2);
    const double du = div_c(at(um, i + 1, j, k) - at(um, i, j, k), r0);
    const double dv = div_c(at(vm, i, j + 1, k) - at(vm, i, j, k), r1);
    const double divu = du + dv + div_c(at(wm, i, j, k + 1) - at(wm, i, j, k), r2);
    at(AW(A_ASOLD), i, j, k, comp) += at(AW(A_AS), i, j, k) - divu * at(AW(A_AFORCE), i, j, k);
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

void adj_flux(Ctx& c, const double* r0, const double* r0e) {
    launch(c, rg_grow(c, 0, 0), 1, k_adj_flux<0>, c.V(), c.nspec, c.P.dt / c.P.dx[0], r0, r0);
    launch(c, rg_grow(c, 0, 1), 1, k_adj_flux<1>, c.V(), c.nspec, c.P.dt / c.P.dx[1], r0, r0);
    launch(c, rg_grow(c, 0, 2), 1, k_adj_flux<2>, c.V(), c.nspec, c.P.dt / c.P.dx[2], r0e, r0e);
}

template <int D, int T>
static void adj_transverse_launch(Ctx& c, long long eb) {
    constexpr int O = 3 - D - T;
    int glo[3] = {0, 0, 0}, ghi[3] = {0, 0, 0};
    glo[O] = 1;
    ghi[O] = 1;
    ghi[D] = 1;
    launch(c, region(c, glo[0], glo[1], glo[2], ghi[0], ghi[1], ghi[2], -1), 1, k_adj_es_transverse<D, T>, c.V(), eb);
}

template <int D>
static void adj_predictor_launch(Ctx& c) {
    int glo[3] = {1, 1, 1};
    glo[D] = 0;
    launch(c, region(c, glo[0], glo[1], glo[2], 1, 1, 1, -1), 1, k_adj_es_predictor<D>, c.V());
}

template <int D>
static void adj_ppm_launch(Ctx& c, int fs, int comp, long long eb, double* dir, size_t dir_bytes) {
    ppm_faces(c, D, fs, comp);
    if (!c.dry) cudaMemsetAsync(dir, 0, dir_bytes, c.stream);
    const RecipC r6 = make_recip(6.0);
    launch(c, rg_grow(c, 1), 1, k_adj_ppm_cell<D>, c.V(), fs, comp, eb);
    int glo[3] = {1, 1, 1};
    glo[D] = 1;
    launch(c, region(c, glo[0], glo[1], glo[2], glo[0], glo[1], glo[2], D), 1, k_adj_ppm_face<D>, c.V(), fs, comp, r6);
    glo[D] = 2;
    launch(c, region(c, glo[0], glo[1], glo[2], glo[0], glo[1], glo[2], -1), 1, k_adj_dsvl<D>, c.V(), fs, comp);
}

// MakeEdgeScal^T of component comp of field fs (advective form, ppm_type 1): from the
// edge-state adjoints A_AEDGE0..2 (comp) into A_AS (and A_AFORCE unless force_zero).
// dir: the storage of A_ASM / A_ASP / A_ADSVL, cleared before each direction.
void adj_edge_scal(Ctx& c, int fs, int comp, int force_zero, double* dir, size_t dir_bytes) {
    const long long eb = dbits_host(c.P.rel_eps);
    const double dt2 = 0.5 * c.P.dt;
    launch(c, rg_grow(c, 0, 0), 1, k_adj_es_edges<0>, c.V(), comp, force_zero, dt2, eb);
    launch(c, rg_grow(c, 0, 1), 1, k_adj_es_edges<1>, c.V(), comp, force_zero, dt2, eb);
    launch(c, rg_grow(c, 0, 2), 1, k_adj_es_edges<2>, c.V(), comp, force_zero, dt2, eb);
    adj_transverse_launch<0, 1>(c, eb);
    adj_transverse_launch<0, 2>(c, eb);
    adj_transverse_launch<1, 0>(c, eb);
    adj_transverse_launch<1, 2>(c, eb);
    adj_transverse_launch<2, 0>(c, eb);
    adj_transverse_launch<2, 1>(c, eb);
    adj_predictor_launch<0>(c);
    adj_predictor_launch<1>(c);
    adj_predictor_launch<2>(c);
    adj_ppm_launch<0>(c, fs, comp, eb, dir, dir_bytes);
    adj_ppm_launch<1>(c, fs, comp, eb, dir, dir_bytes);
    adj_ppm_launch<2>(c, fs, comp, eb, dir, dir_bytes);
}

void adj_fill_boundary(Ctx& c, int slot, int ng) {
    const CopyTable& ct = copy_table(c, ng, -1);
    if (ct.total == 0 || c.dry) return;
    unsigned grid = (unsigned)((ct.total + TPB - 1) / TPB);
    k_adj_fill_boundary<<<grid, TPB, 0, c.stream>>>(ct.d, (int)ct.h.size(), ct.total, c.V(), c.nb, F_USER + slot);
    c.launches++;
}

void adj_convert_x(Ctx& c, int comp) { launch(c, rg_grow(c, 0), 1, k_adj_x, c.V(), comp); }

void adj_pert_force(Ctx& c, int comp) {
    launch(c, rg_grow(c, 0), 1, k_adj_pert, c.V(), comp, make_recip(c.P.dx[0]), make_recip(c.P.dx[1]),
           make_recip(c.P.dx[2]));
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
