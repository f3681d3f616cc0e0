// Single-box entry points: Maestro::PPM on one box (Source/Maestro.H:1396,
// Source/MaestroPPM.cpp:5-2262), the routine the reference calls once per box and per
// traced component.  Scratch (interface values, van Leer slopes, tracing coefficients)
// is owned by the context and grown on demand.
#include <cstring>

#include "madv_ctx.hpp"
#include "madv_exact.cuh"
#include "madv_ppm.cuh"

namespace madv {

struct PPMBoxArgs {
    RegionBox r;  // lo, n; b and start unused
    FabView s, u, T, F, DV, Ip, Im;
    int sc, uc, lo_ext, hi_ext, domlo, domhi;
    long long epsb;
    double dt, dxd;
    RecipC r6;
};

__device__ __forceinline__ bool box_ijk(const RegionBox& r, int& i, int& j, int& k) {
    const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (long)r.n[0] * r.n[1] * r.n[2]) return false;
    region_ijk(r, gid, i, j, k);
    return true;
}

template <int D>
__global__ void k_box_dsvl(PPMBoxArgs a) {
    int i, j, k;
    if (!box_ijk(a.r, i, j, k)) return;
    at(a.DV, i, j, k) = ppm_dsvl<D>(a.s, a.sc, i, j, k);
}

template <int D, int PPMT>
__global__ void k_box_face(PPMBoxArgs a) {
    int i, j, k;
    if (!box_ijk(a.r, i, j, k)) return;
    at(a.F, i, j, k) = ppm_face_value<D, PPMT>(a.s, a.sc, a.DV, i, j, k, a.lo_ext, a.hi_ext, a.domlo, a.domhi, a.r6);
}

// tracing coefficients: per face of the face velocity (umac) or per cell of component
// uc of the cell velocity
__global__ void k_box_trace(PPMBoxArgs a) {
    int i, j, k;
    if (!box_ijk(a.r, i, j, k)) return;
    double A, B;
    trace_coeffs(at(a.u, i, j, k, a.uc), a.dt, a.dxd, A, B);
    at(a.T, i, j, k, 0) = A;
    at(a.T, i, j, k, 1) = B;
}

template <int D, int PPMT, int UMAC>
__global__ void k_box_cell(PPMBoxArgs a) {
    int i, j, k;
    if (!box_ijk(a.r, i, j, k)) return;
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    double sm, sp;
    ppm_cell_edges<D, PPMT>(a.s, a.sc, a.F, a.DV, i, j, k, a.lo_ext, a.hi_ext, a.domlo, a.domhi, a.r6, sm, sp);
    double up, um, Ap, Bp, Am, Bm;
    if (UMAC) {
        up = at(a.u, i + di, j + dj, k + dk);
        um = at(a.u, i, j, k);
        Ap = at(a.T, i + di, j + dj, k + dk, 0);
        Bp = at(a.T, i + di, j + dj, k + dk, 1);
        Am = at(a.T, i, j, k, 0);
        Bm = at(a.T, i, j, k, 1);
    } else {
        up = um = at(a.u, i, j, k, a.uc);
        Ap = Am = at(a.T, i, j, k, 0);
        Bp = Bm = at(a.T, i, j, k, 1);
    }
    double ip, im;
    ppm_trace(at(a.s, i, j, k, a.sc), sm, sp, up, um, Ap, Bp, Am, Bm, a.epsb, ip, im);
    at(a.Ip, i, j, k, D) = ip;
    at(a.Im, i, j, k, D) = im;
}

static FabView view_of(const madv_fab& f) {
    FabView v{};
    v.p = f.p;
    v.lo0 = f.lo[0];
    v.lo1 = f.lo[1];
    v.lo2 = f.lo[2];
    const long nx = f.hi[0] - f.lo[0] + 1, ny = f.hi[1] - f.lo[1] + 1, nz = f.hi[2] - f.lo[2] + 1;
    v.sj = (int)nx;
    v.sk = nx * ny;
    v.sn = nx * ny * nz;
    return v;
}

static FabView scratch_view(double* p, const int lo[3], const int hi[3]) {
    madv_fab f{};
    f.p = p;
    for (int d = 0; d < 3; ++d) {
        f.lo[d] = lo[d];
        f.hi[d] = hi[d];
    }
    f.ncomp = 1;
    return view_of(f);
}

static bool covers(const madv_fab* f, const int lo[3], const int hi[3], int ncomp) {
    if (!f || !f->p || f->ncomp < ncomp) return false;
    for (int d = 0; d < 3; ++d)
        if (f->lo[d] > lo[d] || f->hi[d] < hi[d]) return false;
    return true;
}

static void launch_box(const RegionBox& r, cudaStream_t st, void (*kern)(PPMBoxArgs), PPMBoxArgs a, long& count) {
    a.r = r;
    const long n = (long)r.n[0] * r.n[1] * r.n[2];
    if (n <= 0) return;
    kern<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a);
    ++count;
}

static RegionBox rbox(const int lo[3], const int hi[3]) {
    RegionBox r{};
    for (int d = 0; d < 3; ++d) {
        r.lo[d] = lo[d];
        r.n[d] = hi[d] - lo[d] + 1;
    }
    return r;
}

// Scratch (doubles) that one PPM call on box extents n needs: per direction (reused)
// an interface-value array (n_d + 4 faces), a van Leer slope array (n_d + 2 cells) and
// two tracing-coefficient arrays (n_d + 1 faces), the transverse extents being n_t.
long ppm_box_scratch_doubles(const int n[3]) {
    long worst = 0;
    for (int d = 0; d < 3; ++d) {
        long t = 1;
        for (int e = 0; e < 3; ++e)
            if (e != d) t *= n[e];
        const long need = t * ((n[d] + 4) + (n[d] + 2) + 2 * (n[d] + 1));
        worst = need > worst ? need : worst;
    }
    return worst;
}

// Validates the arguments and runs the PPM of one box with the scratch at `scratch`
// (at least ppm_box_scratch_doubles(n) doubles).  Returns a madv error code.
int ppm_box_run(const madv_params& P, const madv_box* bx, const madv_fab* s, int comp, const madv_fab* u,
                const madv_fab* v, const madv_fab* w, int is_umac, const int* bc, const madv_fab* Ip,
                const madv_fab* Im, double* scratch, cudaStream_t st, long& launches) {
    if (!bx || !s || !u || !v || !w || !bc || !Ip || !Im || !scratch) return MADV_ERR_PARAM;
    if (P.ppm_type != 1 && P.ppm_type != 2) {
        set_error("madv_ppm: ppm_type must be 1 or 2 (ppm_type 0 uses the slopes)");
        return MADV_ERR_UNSUPPORTED;
    }
    int n[3];
    for (int d = 0; d < 3; ++d) {
        n[d] = bx->hi[d] - bx->lo[d] + 1;
        if (n[d] <= 0) return MADV_ERR_LAYOUT;
    }
    const int g = P.ppm_type == 2 ? 3 : 2;
    int slo[3], shi[3];
    for (int d = 0; d < 3; ++d) {
        slo[d] = bx->lo[d] - g;
        shi[d] = bx->hi[d] + g;
    }
    if (!covers(s, slo, shi, comp + 1)) {
        set_error("madv_ppm: s must cover the box grown by 2 (ppm_type 1) or 3 (ppm_type 2) ghost cells");
        return MADV_ERR_LAYOUT;
    }
    const madv_fab* vel[3] = {u, v, w};
    for (int d = 0; d < 3; ++d) {
        int hi[3] = {bx->hi[0], bx->hi[1], bx->hi[2]};
        if (is_umac) hi[d] += 1;
        if (!covers(vel[d], bx->lo, hi, 1)) {
            set_error("madv_ppm: tracing velocity FAB does not cover the box (faces if is_umac)");
            return MADV_ERR_LAYOUT;
        }
    }
    if (!covers(Ip, bx->lo, bx->hi, 3) || !covers(Im, bx->lo, bx->hi, 3)) {
        set_error("madv_ppm: Ip/Im must be 3-component FABs covering the box");
        return MADV_ERR_LAYOUT;
    }
    PPMBoxArgs a{};
    a.s = view_of(*s);
    a.sc = comp;
    a.Ip = view_of(*Ip);
    a.Im = view_of(*Im);
    a.epsb = dbits_host(P.rel_eps);
    a.dt = P.dt;
    a.r6 = make_recip(6.0);
    for (int d = 0; d < 3; ++d) {
        const int lo_ext = (bc[d] == BC_EXT_DIR || bc[d] == BC_HOEXTRAP);
        const int hi_ext = (bc[3 + d] == BC_EXT_DIR || bc[3 + d] == BC_HOEXTRAP);
        a.lo_ext = lo_ext;
        a.hi_ext = hi_ext;
        a.domlo = P.dom_lo[d];
        a.domhi = P.dom_hi[d];
        a.dxd = P.dx[d];
        a.u = view_of(*vel[d]);
        a.uc = 0;
        long t = 1;
        for (int e = 0; e < 3; ++e)
            if (e != d) t *= n[e];
        double* pF = scratch;
        double* pDV = pF + t * (n[d] + 4);
        double* pT = pDV + t * (n[d] + 2);
        // van Leer slopes: cells lo-1 .. hi+1 along d
        int lo[3] = {bx->lo[0], bx->lo[1], bx->lo[2]}, hi[3] = {bx->hi[0], bx->hi[1], bx->hi[2]};
        lo[d] -= 1;
        hi[d] += 1;
        a.DV = scratch_view(pDV, lo, hi);
        // interface values: faces lo .. hi+1 (ppm_type 1) or lo-1 .. hi+2 (ppm_type 2)
        int flo[3] = {bx->lo[0], bx->lo[1], bx->lo[2]}, fhi[3] = {bx->hi[0], bx->hi[1], bx->hi[2]};
        flo[d] -= 2;
        fhi[d] += 2;
        a.F = scratch_view(pF, flo, fhi);
        // tracing coefficients: faces lo .. hi+1 (umac) or cells lo .. hi; 2 comps
        int tlo[3] = {bx->lo[0], bx->lo[1], bx->lo[2]}, thi[3] = {bx->hi[0], bx->hi[1], bx->hi[2]};
        if (is_umac) thi[d] += 1;
        {
            madv_fab tf{};
            tf.p = pT;
            for (int e = 0; e < 3; ++e) {
                tf.lo[e] = tlo[e];
                tf.hi[e] = thi[e];
            }
            tf.ncomp = 2;
            a.T = view_of(tf);
        }
        launch_box(rbox(tlo, thi), st, k_box_trace, a, launches);
        int clo[3] = {bx->lo[0], bx->lo[1], bx->lo[2]}, chi[3] = {bx->hi[0], bx->hi[1], bx->hi[2]};
        if (P.ppm_type == 1) {
            launch_box(rbox(lo, hi), st, d == 0 ? k_box_dsvl<0> : (d == 1 ? k_box_dsvl<1> : k_box_dsvl<2>), a,
                       launches);
            int f1lo[3] = {bx->lo[0], bx->lo[1], bx->lo[2]}, f1hi[3] = {bx->hi[0], bx->hi[1], bx->hi[2]};
            f1hi[d] += 1;
            launch_box(rbox(f1lo, f1hi), st,
                       d == 0 ? k_box_face<0, 1> : (d == 1 ? k_box_face<1, 1> : k_box_face<2, 1>), a, launches);
            void (*kc)(PPMBoxArgs) = is_umac ? (d == 0 ? k_box_cell<0, 1, 1> : (d == 1 ? k_box_cell<1, 1, 1> : k_box_cell<2, 1, 1>))
                                             : (d == 0 ? k_box_cell<0, 1, 0> : (d == 1 ? k_box_cell<1, 1, 0> : k_box_cell<2, 1, 0>));
            launch_box(rbox(clo, chi), st, kc, a, launches);
        } else {
            int f2lo[3] = {bx->lo[0], bx->lo[1], bx->lo[2]}, f2hi[3] = {bx->hi[0], bx->hi[1], bx->hi[2]};
            f2lo[d] -= 1;
            f2hi[d] += 2;
            launch_box(rbox(f2lo, f2hi), st,
                       d == 0 ? k_box_face<0, 2> : (d == 1 ? k_box_face<1, 2> : k_box_face<2, 2>), a, launches);
            void (*kc)(PPMBoxArgs) = is_umac ? (d == 0 ? k_box_cell<0, 2, 1> : (d == 1 ? k_box_cell<1, 2, 1> : k_box_cell<2, 2, 1>))
                                             : (d == 0 ? k_box_cell<0, 2, 0> : (d == 1 ? k_box_cell<1, 2, 0> : k_box_cell<2, 2, 0>));
            launch_box(rbox(clo, chi), st, kc, a, launches);
        }
    }
    return cuda_ok(cudaGetLastError(), "madv_ppm launch") ? MADV_OK : MADV_ERR_CUDA;
}

}  // namespace madv
