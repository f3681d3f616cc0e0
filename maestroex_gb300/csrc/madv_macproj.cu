// Maestro::MacProj (Source/MaestroMacProj.cpp:11-246): one level, plane-parallel or spherical,
// and two plane-parallel levels (the composite solve at the end of this file).
//
// umac enters holding Utilde^* and leaves with Utilde:
//   B = beta0^2 / rho_face on the faces (average_cellcenter_to_face of rho, inverted, times
//       beta0 twice: use_alt_energy_fix, the reference's default; beta0 on x/y faces,
//       CelltoEdge(beta0) on z faces),
//   solve  -div(B grad phi) = macrhs - div(beta0 Utilde^*)  (MLABecLaplacian, alpha = 0,
//       beta = 1; outflow faces Dirichlet phi = 0, other physical faces Neumann,
//       Source/MaestroMacProj.cpp:424-453),
//   beta0 Utilde = beta0 Utilde^* - B grad phi, then the face ghosts refilled.
//
// The solve is a cell-centred geometric multigrid on the level's domain (the layout covers
// it), gathered into one array per grid: V-cycles of red-black Gauss-Seidel, residual
// restriction by the mean of the 8 children, face coefficients restricted by the mean of
// the 4 fine faces under a coarse face, piecewise-constant prolongation; the coarsest grid
// is smoothed to convergence.  The stopping test is the reference's: max |residual| <=
// tol_rel * max |rhs| (MLMG's max norm).  Without a Dirichlet face the operator is
// singular: the rhs is made mean-free, as MLMG does, and phi is returned mean-free.
#include <cstring>

#include "madv_launch.cuh"

namespace madv {

#define MP_CK(x)                                                   \
    do {                                                           \
        if ((x) != cudaSuccess) {                                  \
            set_error(std::string(#x) + ": " + cudaGetErrorString(cudaGetLastError())); \
            return MADV_ERR_CUDA;                                  \
        }                                                          \
    } while (0)

enum { MG_PER = 0, MG_NEU = 1, MG_DIR = 2 };

struct MGGrid {
    int n[3];
    double ih2[3];  // 1 / h_d^2
    double *phi, *rhs, *res, *B[3];
    // the operator's weights, formed once per solve (k_mg_prep): W_d = B_d / h_d^2 on every
    // face, and per cell the diagonal and its reciprocal (0 where the diagonal is 0)
    double *W[3], *diag, *idiag;
};
struct MGBC {
    int lo[3], hi[3];
};

__device__ __forceinline__ long mg_cell(const MGGrid& g, int i, int j, int k) {
    return i + (long)g.n[0] * (j + (long)g.n[1] * k);
}
// face f along d (0 .. n[d]) of the row through (i, j, k)
template <int D>
__device__ __forceinline__ long mg_face(const MGGrid& g, int i, int j, int k) {
    const long nx = g.n[0] + (D == 0), ny = g.n[1] + (D == 1);
    return i + nx * (j + ny * (long)k);
}
__device__ __forceinline__ void mg_ijk(const MGGrid& g, long c, int& i, int& j, int& k) {
    i = (int)(c % g.n[0]);
    const long q = c / g.n[0];
    j = (int)(q % g.n[1]);
    k = (int)(q / g.n[1]);
}

// The six face terms of cell (i,j,k): coefficient w_f (B / h^2, doubled on a Dirichlet face)
// and the neighbour's index (-1: none, Dirichlet value 0 or Neumann)
template <int D>
__device__ __forceinline__ void mg_side(const MGGrid& g, const MGBC& bc, int i, int j, int k, int hi, double& w,
                                        long& nb) {
    const int idx[3] = {i, j, k};
    const int m = idx[D], n = g.n[D];
    const int fi = hi ? m + 1 : m;  // face index along D
    int a[3] = {i, j, k};
    a[D] = fi;
    const double B = g.B[D][mg_face<D>(g, a[0], a[1], a[2])];
    const bool edge = hi ? (m == n - 1) : (m == 0);
    if (!edge) {
        int b[3] = {i, j, k};
        b[D] = hi ? m + 1 : m - 1;
        w = B * g.ih2[D];
        nb = mg_cell(g, b[0], b[1], b[2]);
        return;
    }
    const int t = hi ? bc.hi[D] : bc.lo[D];
    if (t == MG_PER) {
        int b[3] = {i, j, k};
        b[D] = hi ? 0 : n - 1;
        w = B * g.ih2[D];
        nb = mg_cell(g, b[0], b[1], b[2]);
    } else if (t == MG_DIR) {
        w = 2.0 * B * g.ih2[D];
        nb = -1;
    } else {
        w = 0.0;
        nb = -1;
    }
}

// (A phi)_c = sum_f w_f (phi_c - phi_nb), and the diagonal sum_f w_f
__device__ __forceinline__ void mg_apply(const MGGrid& g, const MGBC& bc, int i, int j, int k, double& off,
                                         double& diag) {
    off = 0.0;
    diag = 0.0;
    double w;
    long nb;
#define MG_TERM(D, HI)                                  \
    mg_side<D>(g, bc, i, j, k, HI, w, nb);              \
    diag += w;                                          \
    if (nb >= 0) off += w * g.phi[nb];
    MG_TERM(0, 0) MG_TERM(0, 1) MG_TERM(1, 0) MG_TERM(1, 1) MG_TERM(2, 0) MG_TERM(2, 1)
#undef MG_TERM
}

// sum_f W_f phi_nb over the faces of cell (i,j,k) with a neighbour (interior and periodic
// faces), in mg_apply's order, from the stored weights
__device__ __forceinline__ double mg_off(const MGGrid& g, const MGBC& bc, const double* __restrict__ phi, int i,
                                         int j, int k) {
    double off = 0.0;
    const int idx[3] = {i, j, k};
#pragma unroll
    for (int D = 0; D < 3; ++D)
#pragma unroll
        for (int hi = 0; hi < 2; ++hi) {
            const int m = idx[D], n = g.n[D];
            const bool edge = hi ? (m == n - 1) : (m == 0);
            int b[3] = {i, j, k};
            if (!edge) {
                b[D] = hi ? m + 1 : m - 1;
            } else if ((hi ? bc.hi[D] : bc.lo[D]) == MG_PER) {
                b[D] = hi ? 0 : n - 1;
            } else {
                continue;
            }
            int a[3] = {i, j, k};
            a[D] = hi ? m + 1 : m;
            const long f = D == 0 ? mg_face<0>(g, a[0], a[1], a[2])
                                  : (D == 1 ? mg_face<1>(g, a[0], a[1], a[2]) : mg_face<2>(g, a[0], a[1], a[2]));
            off += g.W[D][f] * phi[mg_cell(g, b[0], b[1], b[2])];
        }
    return off;
}

// W_d = B_d / h_d^2 on the faces of direction D
template <int D>
__global__ void k_mg_prep_w(MGGrid g) {
    long nf = (long)g.n[0] * g.n[1] * g.n[2] / g.n[D] * (g.n[D] + 1);
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c < nf) g.W[D][c] = g.B[D][c] * g.ih2[D];
}

// the diagonal of every cell (mg_apply's sum, Dirichlet faces doubled) and its reciprocal
__global__ void k_mg_prep_diag(MGGrid g, MGBC bc) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)g.n[0] * g.n[1] * g.n[2]) return;
    int i, j, k;
    mg_ijk(g, c, i, j, k);
    double off, diag;
    mg_apply(g, bc, i, j, k, off, diag);
    g.diag[c] = diag;
    g.idiag[c] = diag > 0.0 ? 1.0 / diag : 0.0;
}

// Gauss-Seidel update of cell (i,j,k), from the stored weights
__device__ __forceinline__ void mg_smooth_cell(const MGGrid& g, const MGBC& bc, int i, int j, int k) {
    const long c = mg_cell(g, i, j, k);
    const double id = g.idiag[c];
    if (id > 0.0) g.phi[c] = (g.rhs[c] + mg_off(g, bc, g.phi, i, j, k)) * id;
}
__device__ __forceinline__ void mg_resid_cell(const MGGrid& g, const MGBC& bc, int i, int j, int k) {
    const long c = mg_cell(g, i, j, k);
    g.res[c] = g.rhs[c] - (g.diag[c] * g.phi[c] - mg_off(g, bc, g.phi, i, j, k));
}
__device__ __forceinline__ void mg_restrict_cell(const MGGrid& f, const MGGrid& cg, int I, int J, int K) {
    double s = 0.0;
    for (int q = 0; q < 8; ++q) s += f.res[mg_cell(f, 2 * I + (q & 1), 2 * J + ((q >> 1) & 1), 2 * K + (q >> 2))];
    const long c = mg_cell(cg, I, J, K);
    cg.rhs[c] = 0.125 * s;
    cg.phi[c] = 0.0;
}

// Gauss-Seidel on the cells of one colour ((i + j + k) % 2 == color)
__global__ void k_mg_smooth(MGGrid g, MGBC bc, int color) {
    const long half = (long)g.n[0] * g.n[1] * g.n[2] / 2;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= half) return;
    // the t-th cell of the colour: rows of n[0] cells hold n[0]/2 of each colour
    const long row = t / (g.n[0] / 2);
    const int jj = (int)(row % g.n[1]), kk = (int)(row / g.n[1]);
    mg_smooth_cell(g, bc, 2 * (int)(t % (g.n[0] / 2)) + ((jj + kk + color) & 1), jj, kk);
}

// res = rhs - A phi
__global__ void k_mg_resid(MGGrid g, MGBC bc) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)g.n[0] * g.n[1] * g.n[2]) return;
    int i, j, k;
    mg_ijk(g, c, i, j, k);
    mg_resid_cell(g, bc, i, j, k);
}

// coarse rhs = mean of the 8 fine residuals; coarse phi = 0
__global__ void k_mg_restrict(MGGrid f, MGGrid cg) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)cg.n[0] * cg.n[1] * cg.n[2]) return;
    int I, J, K;
    mg_ijk(cg, c, I, J, K);
    mg_restrict_cell(f, cg, I, J, K);
}

// coarse face coefficient = mean of the 4 fine faces it covers
template <int D>
__global__ void k_mg_coarsen_b(MGGrid f, MGGrid cg) {
    constexpr int T1 = D == 0 ? 1 : 0, T2 = D == 2 ? 1 : 2;
    int nc[3] = {cg.n[0], cg.n[1], cg.n[2]};
    nc[D] += 1;
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)nc[0] * nc[1] * nc[2]) return;
    int a[3];
    a[0] = (int)(c % nc[0]);
    a[1] = (int)((c / nc[0]) % nc[1]);
    a[2] = (int)(c / ((long)nc[0] * nc[1]));
    double s = 0.0;
    for (int q = 0; q < 4; ++q) {
        int b[3] = {2 * a[0], 2 * a[1], 2 * a[2]};
        b[T1] += q & 1;
        b[T2] += q >> 1;
        s += f.B[D][mg_face<D>(f, b[0], b[1], b[2])];
    }
    cg.B[D][c] = 0.25 * s;
}

// fine phi += coarse phi (piecewise constant)
__device__ __forceinline__ void mg_prolong_cell(const MGGrid& cg, const MGGrid& f, int i, int j, int k) {
    f.phi[mg_cell(f, i, j, k)] += cg.phi[mg_cell(cg, i / 2, j / 2, k / 2)];
}
__global__ void k_mg_prolong(MGGrid cg, MGGrid f) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)f.n[0] * f.n[1] * f.n[2]) return;
    int i, j, k;
    mg_ijk(f, c, i, j, k);
    mg_prolong_cell(cg, f, i, j, k);
}

// The V-cycle from a grid of at most MG_BLOCK_CELLS cells down, in one thread block: the
// same per-cell smoothing, residual, restriction and prolongation as the launches of
// mg_vcycle, in the same order (a colour's update reads only the other colour, so the order
// within a sweep does not matter), with the block synchronised between steps.  The result
// is bitwise that of one launch per step; the coarse levels' ~170 launches of a few cells
// each become one.
constexpr long MG_BLOCK_CELLS = 4096;
constexpr int MG_BLOCK_LEVELS = 12;
constexpr int MG_BLOCK_THREADS = 1024;
struct MGStack {
    MGGrid g[MG_BLOCK_LEVELS];
    int n;
};

__device__ void mgb_smooth(const MGGrid& g, const MGBC& bc, int color) {
    const int nh = g.n[0] / 2, tot = nh * g.n[1] * g.n[2];
    for (int t = threadIdx.x; t < tot; t += blockDim.x) {
        const int row = t / nh, jj = row % g.n[1], kk = row / g.n[1];
        mg_smooth_cell(g, bc, 2 * (t % nh) + ((jj + kk + color) & 1), jj, kk);
    }
    __syncthreads();
}

__global__ void __launch_bounds__(MG_BLOCK_THREADS) k_mg_block_cycle(MGStack S, MGBC bc, int nu, int bottom) {
    const int last = S.n - 1;
    for (int l = 0; l < last; ++l) {
        const MGGrid& g = S.g[l];
        const MGGrid& cg = S.g[l + 1];
        for (int s = 0; s < nu; ++s) {
            mgb_smooth(g, bc, 0);
            mgb_smooth(g, bc, 1);
        }
        const int n = g.n[0] * g.n[1] * g.n[2];
        for (int c = threadIdx.x; c < n; c += blockDim.x)
            mg_resid_cell(g, bc, c % g.n[0], (c / g.n[0]) % g.n[1], c / (g.n[0] * g.n[1]));
        __syncthreads();
        const int nc = cg.n[0] * cg.n[1] * cg.n[2];
        for (int c = threadIdx.x; c < nc; c += blockDim.x)
            mg_restrict_cell(g, cg, c % cg.n[0], (c / cg.n[0]) % cg.n[1], c / (cg.n[0] * cg.n[1]));
        __syncthreads();
    }
    for (int s = 0; s < bottom; ++s) {
        mgb_smooth(S.g[last], bc, 0);
        mgb_smooth(S.g[last], bc, 1);
    }
    for (int l = last - 1; l >= 0; --l) {
        const MGGrid& g = S.g[l];
        const int n = g.n[0] * g.n[1] * g.n[2];
        for (int c = threadIdx.x; c < n; c += blockDim.x)
            mg_prolong_cell(S.g[l + 1], g, c % g.n[0], (c / g.n[0]) % g.n[1], c / (g.n[0] * g.n[1]));
        __syncthreads();
        for (int s = 0; s < nu; ++s) {
            mgb_smooth(g, bc, 1);
            mgb_smooth(g, bc, 0);
        }
    }
}

// out_max = max |x| (bit pattern of a non-negative double); part[block] = the block's sum of
// x.  Every partial sum is formed in a fixed order (grid-stride per thread, a shuffle tree
// per warp, warps in order per block), so the sum does not depend on scheduling.
__global__ void k_mg_norms(const double* __restrict__ x, long n, unsigned long long* out_max, double* part) {
    __shared__ double ws[32];
    double m = 0.0, s = 0.0;
    for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x) {
        m = fmax(m, fabs(x[c]));
        s += x[c];
    }
    for (int o = 16; o > 0; o >>= 1) {
        m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
        s += __shfl_down_sync(0xffffffffu, s, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out_max, (unsigned long long)__double_as_longlong(m));
        ws[threadIdx.x >> 5] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += ws[w];
        part[blockIdx.x] = b;
    }
}

// sum of the block partials, in block order (one thread)
__global__ void k_mg_sum_parts(const double* __restrict__ part, int nb, double* out_sum) {
    double s = 0.0;
    for (int q = 0; q < nb; ++q) s += part[q];
    out_sum[0] = s;
}

__global__ void k_mg_shift(double* __restrict__ x, long n, const double* __restrict__ sum, double inv_n) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n) x[c] -= sum[0] * inv_n;
}

// beta0 on the faces: plane-parallel, beta0(k) on x / y faces and beta0_edge(k) on z faces;
// spherical, one value per face of the domain (MakeS0mac of beta0, gathered from the boxes)
struct MPBeta {
    const double* b0;
    const double* b0e;
    const double* f[3];
    int sph;
};
template <int D>
__device__ __forceinline__ double mp_beta(const MPBeta& be, const MGGrid& g, int a0, int a1, int a2) {
    if (be.sph) return be.f[D][mg_face<D>(g, a0, a1, a2)];
    return D == 2 ? be.b0e[a2] : be.b0[a2];
}

// spherical: the beta0 faces of the boxes (F_S0MAC*) into the domain's face arrays; a face
// two boxes share holds the same value in both
template <int D>
__global__ void k_mp_beta_faces(KARGS, MGGrid g, double* __restrict__ out, int l0, int l1, int l2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    out[mg_face<D>(g, i - l0, j - l1, k - l2)] = at(VW(F_S0MAC0 + D), i, j, k);
}

// ---- the level's FABs <-> the multigrid's arrays (domain cell (i,j,k) at i - lo0, ...)
// Valid cells: rho into g.res (read by the coefficient kernels), the solver rhs
// macrhs - div(beta0 umac) (ComputeMACSolverRHS after MultFacesByBeta0 or, spherical, the
// product with beta0mac), phi = 0.
__global__ void k_mp_gather(KARGS, MGGrid g, int srhs, int srho, MPBeta be, double dx0, double dx1, double dx2, int l0,
                            int l1, int l2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const FabView u = VW(F_UMAC0), v = VW(F_UMAC1), w = VW(F_UMAC2);
    const int a0 = i - l0, a1 = j - l1, kr = k - l2;
    const long c = mg_cell(g, a0, a1, kr);
    g.res[c] = at(VW(F_USER + srho), i, j, k);
    g.rhs[c] = at(VW(F_USER + srhs), i, j, k) -
               ((at(u, i + 1, j, k) * mp_beta<0>(be, g, a0 + 1, a1, kr) - at(u, i, j, k) * mp_beta<0>(be, g, a0, a1, kr)) / dx0 +
                (at(v, i, j + 1, k) * mp_beta<1>(be, g, a0, a1 + 1, kr) - at(v, i, j, k) * mp_beta<1>(be, g, a0, a1, kr)) / dx1 +
                (at(w, i, j, k + 1) * mp_beta<2>(be, g, a0, a1, kr + 1) - at(w, i, j, k) * mp_beta<2>(be, g, a0, a1, kr)) / dx2);
    g.phi[c] = 0.0;
}

// Face coefficients B = beta^2 / (0.5 (rho_l + rho_r)) on every face of the domain, rho in
// g.res; across a physical face the ghost cell is the inside cell (foextrap / reflect_even;
// only outflow's Dirichlet faces read it)
template <int D>
__global__ void k_mp_bcoef(MGGrid g, MGBC bc, MPBeta be) {
    int nf[3] = {g.n[0], g.n[1], g.n[2]};
    nf[D] += 1;
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)nf[0] * nf[1] * nf[2]) return;
    int a[3];
    a[0] = (int)(c % nf[0]);
    a[1] = (int)((c / nf[0]) % nf[1]);
    a[2] = (int)(c / ((long)nf[0] * nf[1]));
    const int m = a[D], n = g.n[D];
    int l[3] = {a[0], a[1], a[2]}, r[3] = {a[0], a[1], a[2]};
    l[D] = m - 1;
    if (m == 0) l[D] = bc.lo[D] == MG_PER ? n - 1 : 0;
    if (m == n) r[D] = bc.hi[D] == MG_PER ? 0 : n - 1;
    const double face = 0.5 * (g.res[mg_cell(g, l[0], l[1], l[2])] + g.res[mg_cell(g, r[0], r[1], r[2])]);
    double Bv = 1.0 / face;
    const double beta = mp_beta<D>(be, g, a[0], a[1], a[2]);
    Bv *= beta;
    Bv *= beta;
    g.B[D][c] = Bv;
}

// Valid D-faces of every box: beta0 umac += -B grad phi, then umac /= beta0 (getFluxes with
// maxorder 2: a Dirichlet face sees the ghost 2 phi_b - phi_0, phi_b = 0)
template <int D>
__global__ void k_mp_correct(KARGS, MGGrid g, MGBC bc, MPBeta be, double inv_h, int l0, int l1, int l2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    int a[3] = {i - l0, j - l1, k - l2};
    const int m = a[D], n = g.n[D];
    const double B = g.B[D][mg_face<D>(g, a[0], a[1], a[2])];
    auto P = [&](int q) {
        int s[3] = {a[0], a[1], a[2]};
        s[D] = q;
        return g.phi[mg_cell(g, s[0], s[1], s[2])];
    };
    double grad;
    if (m > 0 && m < n) {
        grad = (P(m) - P(m - 1)) * inv_h;
    } else {
        const int t = m == 0 ? bc.lo[D] : bc.hi[D];
        if (t == MG_PER) grad = (P(0) - P(n - 1)) * inv_h;
        else if (t == MG_DIR) grad = m == 0 ? (P(0) - (-P(0))) * inv_h : ((-P(n - 1)) - P(n - 1)) * inv_h;
        else grad = 0.0;
    }
    const double flux = -B * grad;
    const double beta = mp_beta<D>(be, g, a[0], a[1], a[2]);
    double& u = at(VW(F_UMAC0 + D), i, j, k);
    u = (u * beta + flux) / beta;
}

__global__ void k_mp_phi_out(KARGS, MGGrid g, int sphi, int l0, int l1, int l2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    at(VW(F_USER + sphi), i, j, k) = g.phi[mg_cell(g, i - l0, j - l1, k - l2)];
}

// ---- conjugate gradients preconditioned by one V-cycle (used where the coefficients jump by
// orders of magnitude: spherical geometry, B ~ rho0 from the core to the ambient)
// q = A p (p read through a copy of the grid whose phi is p)
__global__ void k_pcg_apply(MGGrid g, MGBC bc, const double* __restrict__ p, double* __restrict__ q) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)g.n[0] * g.n[1] * g.n[2]) return;
    int i, j, k;
    mg_ijk(g, c, i, j, k);
    q[c] = g.diag[c] * p[c] - mg_off(g, bc, p, i, j, k);
}

// part[block] = the block's sum of x * y, in a fixed order (as k_mg_norms)
__global__ void k_pcg_dot(const double* __restrict__ x, const double* __restrict__ y, long n, double* part) {
    __shared__ double ws[32];
    double s = 0.0;
    for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x)
        s += x[c] * y[c];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += ws[w];
        part[blockIdx.x] = b;
    }
}

// x += a p, r -= a q
__global__ void k_pcg_step(double* __restrict__ x, double* __restrict__ r, const double* __restrict__ p,
                           const double* __restrict__ q, double a, long n) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    x[c] += a * p[c];
    r[c] -= a * q[c];
}

// p = z + b p
__global__ void k_pcg_dir(double* __restrict__ p, const double* __restrict__ z, double b, long n) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    p[c] = z[c] + b * p[c];
}

// ---- the hierarchy and the solve
struct MacMG {
    std::vector<MGGrid> lev;
    std::vector<double*> mem;
    int n0[3] = {0, 0, 0};
    unsigned long long* d_max = nullptr;
    double* d_sum = nullptr;
    double* d_part = nullptr;  // per-block partial sums of k_mg_norms
    double* d_beta = nullptr;  // beta0 [nr], beta0_edge [nr + 1]
    double* d_bface[3] = {nullptr, nullptr, nullptr};  // spherical: beta0 on the domain's faces
    double* pcg = nullptr;  // spherical: x, r, p, q, z of the PCG, one block of ncell each
    struct MLFine* ml = nullptr;  // two levels: the level-1 grid and the composite solve's arrays
};

// Two levels (refinement ratio 2): the level-1 domain as one dense grid (its cells off the
// level-1 boxes unused), the masks, the composite diagonals and the PCG vectors of both levels
struct MLFine {
    MGGrid g{};
    int n1[3] = {0, 0, 0};
    std::vector<double*> mem;
    double *mask = nullptr, *cov = nullptr;      // level-1 cells of a box; covered level-0 cells
    double *cdiag0 = nullptr, *cdiag1 = nullptr;  // the composite operator's diagonals
    double *v0 = nullptr, *v1 = nullptr;          // x r p q z per level, five blocks each
    double* beta1 = nullptr;                      // level 1: beta0 [nr1], beta0_edge [nr1 + 1]
};

static void ml_free(MLFine*& m) {
    if (!m) return;
    for (double* p : m->mem) cudaFree(p);
    delete m;
    m = nullptr;
}

void mac_free(Ctx& c) {
    if (!c.mac) return;
    ml_free(c.mac->ml);
    for (double* p : c.mac->mem) cudaFree(p);
    if (c.mac->d_max) cudaFree(c.mac->d_max);
    if (c.mac->d_sum) cudaFree(c.mac->d_sum);
    if (c.mac->d_part) cudaFree(c.mac->d_part);
    if (c.mac->d_beta) cudaFree(c.mac->d_beta);
    for (double* p : c.mac->d_bface)
        if (p) cudaFree(p);
    if (c.mac->pcg) cudaFree(c.mac->pcg);
    delete c.mac;
    c.mac = nullptr;
}

// blocks of the norm / sum kernel: a fixed grid for every array size, so the order of the
// partial sums is fixed too
constexpr long NORM_BLOCKS = 152L * 8;

static dim3 blocks_of(long n) { return dim3((unsigned)((n + TPB - 1) / TPB)); }

static long ncell(const MGGrid& g) { return (long)g.n[0] * g.n[1] * g.n[2]; }

// Builds (once per domain) grids coarsened by 2 in every direction (rule below).
static int mac_hierarchy(Ctx& c, const int n0[3], int nr) {
    if (c.mac && c.mac->n0[0] == n0[0] && c.mac->n0[1] == n0[1] && c.mac->n0[2] == n0[2]) return MADV_OK;
    mac_free(c);
    c.mac = new MacMG();
    MacMG& M = *c.mac;
    for (int d = 0; d < 3; ++d) M.n0[d] = n0[d];
    int n[3] = {n0[0], n0[1], n0[2]};
    double h2[3] = {c.P.dx[0] * c.P.dx[0], c.P.dx[1] * c.P.dx[1], c.P.dx[2] * c.P.dx[2]};
    auto alloc = [&](long cnt) -> double* {
        double* p = nullptr;
        if (cudaMalloc(&p, sizeof(double) * cnt) != cudaSuccess) return nullptr;
        M.mem.push_back(p);
        return p;
    };
    while (true) {
        MGGrid g{};
        for (int d = 0; d < 3; ++d) {
            g.n[d] = n[d];
            g.ih2[d] = 1.0 / h2[d];
        }
        const long nc = (long)n[0] * n[1] * n[2];
        g.phi = alloc(nc);
        g.rhs = alloc(nc);
        g.res = alloc(nc);
        g.diag = alloc(nc);
        g.idiag = alloc(nc);
        for (int d = 0; d < 3; ++d) {
            g.B[d] = alloc(nc / n[d] * (n[d] + 1));
            g.W[d] = alloc(nc / n[d] * (n[d] + 1));
        }
        if (!g.phi || !g.rhs || !g.res || !g.diag || !g.idiag || !g.B[0] || !g.B[1] || !g.B[2] || !g.W[0] || !g.W[1] ||
            !g.W[2]) {
            set_error("cudaMalloc(MAC multigrid)");
            mac_free(c);
            return MADV_ERR_CUDA;
        }
        M.lev.push_back(g);
        // coarsen while every extent halves to >= 2 cells.  A periodic extent must halve to an
        // even one, so that the red-black colouring stays consistent across the wrap, and so
        // must x, whose rows the smoother splits into two colours of n[0] / 2 cells
        bool more = true;
        for (int d = 0; d < 3; ++d) {
            const bool even_needed = d == 0 || c.P.phys_bc_lo[d] == MADV_INTERIOR;
            more = more && n[d] % 2 == 0 && n[d] / 2 >= 2 && (!even_needed || (n[d] / 2) % 2 == 0);
        }
        if (!more) break;
        for (int d = 0; d < 3; ++d) {
            n[d] /= 2;
            h2[d] *= 4.0;
        }
    }
    if (cudaMalloc(&M.d_max, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&M.d_sum, sizeof(double)) != cudaSuccess ||
        cudaMalloc(&M.d_part, sizeof(double) * NORM_BLOCKS) != cudaSuccess ||
        cudaMalloc(&M.d_beta, sizeof(double) * (2 * nr + 1)) != cudaSuccess ||
        (c.sph && (cudaMalloc(&M.d_bface[0], sizeof(double) * (n0[0] + 1) * n0[1] * n0[2]) != cudaSuccess ||
                   cudaMalloc(&M.d_bface[1], sizeof(double) * n0[0] * (n0[1] + 1) * n0[2]) != cudaSuccess ||
                   cudaMalloc(&M.d_bface[2], sizeof(double) * n0[0] * n0[1] * (n0[2] + 1)) != cudaSuccess ||
                   cudaMalloc(&M.pcg, sizeof(double) * 5 * (size_t)n0[0] * n0[1] * n0[2]) != cudaSuccess))) {
        set_error("cudaMalloc(MAC multigrid)");
        mac_free(c);
        return MADV_ERR_CUDA;
    }
    return MADV_OK;
}

static void mg_smooth(Ctx& c, const MGGrid& g, const MGBC& bc, int color) {
    k_mg_smooth<<<blocks_of(ncell(g) / 2), TPB, 0, c.stream>>>(g, bc, color);
    c.launches++;
}

static void mg_resid(Ctx& c, const MGGrid& g, const MGBC& bc) {
    k_mg_resid<<<blocks_of(ncell(g)), TPB, 0, c.stream>>>(g, bc);
    c.launches++;
}

static int mg_bottom_sweeps(const MGGrid& g) {  // the coarsest grid: to convergence
    const int nmax = std::max(g.n[0], std::max(g.n[1], g.n[2]));
    return std::min(2000, std::max(64, 2 * nmax * nmax));
}

static void mg_vcycle(Ctx& c, const MGBC& bc, int l) {
    MacMG& M = *c.mac;
    const MGGrid& g = M.lev[l];
    const int nu = 2, bottom = mg_bottom_sweeps(g);
    const int nrest = (int)M.lev.size() - l;
    if (c.mg_block_cycle && ncell(g) <= MG_BLOCK_CELLS && nrest <= MG_BLOCK_LEVELS) {
        MGStack S{};
        S.n = nrest;
        for (int q = 0; q < nrest; ++q) S.g[q] = M.lev[l + q];
        k_mg_block_cycle<<<1, MG_BLOCK_THREADS, 0, c.stream>>>(S, bc, nu, mg_bottom_sweeps(M.lev.back()));
        c.launches++;
        return;
    }
    if (l + 1 == (int)M.lev.size()) {
        for (int s = 0; s < bottom; ++s) {
            mg_smooth(c, g, bc, 0);
            mg_smooth(c, g, bc, 1);
        }
        return;
    }
    for (int s = 0; s < nu; ++s) {
        mg_smooth(c, g, bc, 0);
        mg_smooth(c, g, bc, 1);
    }
    const MGGrid& cg = M.lev[l + 1];
    mg_resid(c, g, bc);
    k_mg_restrict<<<blocks_of(ncell(cg)), TPB, 0, c.stream>>>(g, cg);
    c.launches++;
    mg_vcycle(c, bc, l + 1);
    k_mg_prolong<<<blocks_of(ncell(g)), TPB, 0, c.stream>>>(cg, g);
    c.launches++;
    for (int s = 0; s < nu; ++s) {  // the reverse colour order keeps the cycle symmetric
        mg_smooth(c, g, bc, 1);
        mg_smooth(c, g, bc, 0);
    }
}

// max |x| and sum x of an array, read back (the stream is synchronised)
static int mg_norms(Ctx& c, const double* x, long n, double& amax, double* sum_out, bool device_sum_only = false) {
    MacMG& M = *c.mac;
    MP_CK(cudaMemsetAsync(M.d_max, 0, sizeof(unsigned long long), c.stream));
    const unsigned nb = (unsigned)std::min<long>((n + TPB - 1) / TPB, NORM_BLOCKS);
    k_mg_norms<<<nb, TPB, 0, c.stream>>>(x, n, M.d_max, M.d_part);
    k_mg_sum_parts<<<1, 1, 0, c.stream>>>(M.d_part, (int)nb, M.d_sum);
    c.launches += 2;
    if (device_sum_only) return MADV_OK;
    unsigned long long bits = 0;
    double s = 0.0;
    MP_CK(cudaMemcpyAsync(&bits, M.d_max, sizeof(bits), cudaMemcpyDeviceToHost, c.stream));
    MP_CK(cudaMemcpyAsync(&s, M.d_sum, sizeof(s), cudaMemcpyDeviceToHost, c.stream));
    MP_CK(cudaStreamSynchronize(c.stream));
    std::memcpy(&amax, &bits, sizeof(double));
    if (sum_out) *sum_out = s;
    return MADV_OK;
}

// MacProj on one plane-parallel level.  The caller has bound macrhs (slot srhs), rho
// (slot srho) and macphi (slot sphi, may be < 0) and copied umac (valid faces and one
// ghost) into F_UMAC0..2; umac is corrected there and its ghost faces refilled.
// sum over the blocks of k_pcg_dot, read back (the stream is synchronised)
static int pcg_dot(Ctx& c, const double* x, const double* y, long n, double& out) {
    MacMG& M = *c.mac;
    const unsigned nb = (unsigned)std::min<long>((n + TPB - 1) / TPB, NORM_BLOCKS);
    k_pcg_dot<<<nb, TPB, 0, c.stream>>>(x, y, n, M.d_part);
    k_mg_sum_parts<<<1, 1, 0, c.stream>>>(M.d_part, (int)nb, M.d_sum);
    c.launches += 2;
    MP_CK(cudaMemcpyAsync(&out, M.d_sum, sizeof(out), cudaMemcpyDeviceToHost, c.stream));
    MP_CK(cudaStreamSynchronize(c.stream));
    return MADV_OK;
}

// Conjugate gradients on A phi = rhs of the finest grid, preconditioned by one V-cycle
// (symmetric: the post-smoothing runs the colours in reverse), from phi = 0, until
// max|r| <= target; the flexible (Polak-Ribiere) update tolerates the fixed-sweep coarsest
// solve.  phi ends in g.phi.  Every dot product is summed in a fixed order.
static int mac_pcg(Ctx& c, const MGBC& bc, double target, int max_iter, int& it, double& res_max) {
    MacMG& M = *c.mac;
    MGGrid& g = M.lev[0];
    const long n = ncell(g);
    double *x = M.pcg, *r = x + n, *p = r + n, *q = p + n, *z = q + n;
    int rc;
    MP_CK(cudaMemsetAsync(x, 0, sizeof(double) * n, c.stream));
    MP_CK(cudaMemcpyAsync(r, g.rhs, sizeof(double) * n, cudaMemcpyDeviceToDevice, c.stream));
    auto precondition = [&]() -> int {  // z = V-cycle(r) from zero
        MP_CK(cudaMemcpyAsync(g.rhs, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, c.stream));
        MP_CK(cudaMemsetAsync(g.phi, 0, sizeof(double) * n, c.stream));
        mg_vcycle(c, bc, 0);
        MP_CK(cudaMemcpyAsync(z, g.phi, sizeof(double) * n, cudaMemcpyDeviceToDevice, c.stream));
        return MADV_OK;
    };
    it = 0;
    if ((rc = mg_norms(c, r, n, res_max, nullptr))) return rc;
    if (res_max <= target) {
        MP_CK(cudaMemsetAsync(g.phi, 0, sizeof(double) * n, c.stream));
        return MADV_OK;
    }
    if ((rc = precondition())) return rc;
    MP_CK(cudaMemcpyAsync(p, z, sizeof(double) * n, cudaMemcpyDeviceToDevice, c.stream));
    double rz = 0.0;
    if ((rc = pcg_dot(c, r, z, n, rz))) return rc;
    while (it < max_iter) {
        k_pcg_apply<<<blocks_of(n), TPB, 0, c.stream>>>(g, bc, p, q);
        c.launches++;
        double pq = 0.0;
        if ((rc = pcg_dot(c, p, q, n, pq))) return rc;
        if (!(pq > 0.0)) break;  // exact solution reached, or not positive definite
        const double a = rz / pq;
        k_pcg_step<<<blocks_of(n), TPB, 0, c.stream>>>(x, r, p, q, a, n);
        c.launches++;
        ++it;
        if ((rc = mg_norms(c, r, n, res_max, nullptr))) return rc;
        if (res_max <= target) break;
        // z_old into q (free until the next apply), then z = M^-1 r; beta = r.(z - z_old) / rz
        MP_CK(cudaMemcpyAsync(q, z, sizeof(double) * n, cudaMemcpyDeviceToDevice, c.stream));
        if ((rc = precondition())) return rc;
        double rz_new = 0.0, rzo = 0.0;
        if ((rc = pcg_dot(c, r, z, n, rz_new)) || (rc = pcg_dot(c, r, q, n, rzo))) return rc;
        const double b = (rz_new - rzo) / rz;
        rz = rz_new;
        k_pcg_dir<<<blocks_of(n), TPB, 0, c.stream>>>(p, z, b, n);
        c.launches++;
    }
    MP_CK(cudaMemcpyAsync(g.phi, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, c.stream));
    return MADV_OK;
}

int mac_project_level(Ctx& c, int srhs, int srho, int sphi, const double* beta0, const double* beta0_edge,
                      double tol_rel, int max_iter, int* iters_out, double* ratio_out) {
    int n0[3], l[3];
    MGBC bc{};
    bool dirichlet = false;
    for (int d = 0; d < 3; ++d) {
        l[d] = c.P.dom_lo[d];
        n0[d] = c.P.dom_hi[d] - c.P.dom_lo[d] + 1;
        if (n0[d] % 2 != 0) {
            set_error("the MAC projection needs even domain extents");
            return MADV_ERR_UNSUPPORTED;
        }
        auto t = [&](int pb) {
            if (c.per[d]) return (int)MG_PER;
            if (pb == PB_OUTFLOW) return (int)MG_DIR;
            return (int)MG_NEU;
        };
        bc.lo[d] = t(c.P.phys_bc_lo[d]);
        bc.hi[d] = t(c.P.phys_bc_hi[d]);
        dirichlet = dirichlet || bc.lo[d] == MG_DIR || bc.hi[d] == MG_DIR;
    }
    const int nr = n0[2];
    int rc = mac_hierarchy(c, n0, nr);
    if (rc) return rc;
    MacMG& M = *c.mac;
    const MGGrid& g = M.lev[0];
    MPBeta be{M.d_beta, M.d_beta + nr, {M.d_bface[0], M.d_bface[1], M.d_bface[2]}, c.sph ? 1 : 0};
    if (c.sph) {  // beta0mac (F_S0MAC*, made by the caller) onto the domain's faces
        launch(c, rg_grow(c, 0, 0), 1, k_mp_beta_faces<0>, c.V(), g, M.d_bface[0], l[0], l[1], l[2]);
        launch(c, rg_grow(c, 0, 1), 1, k_mp_beta_faces<1>, c.V(), g, M.d_bface[1], l[0], l[1], l[2]);
        launch(c, rg_grow(c, 0, 2), 1, k_mp_beta_faces<2>, c.V(), g, M.d_bface[2], l[0], l[1], l[2]);
    } else {
        MP_CK(cudaMemcpyAsync(M.d_beta, beta0, sizeof(double) * nr, cudaMemcpyHostToDevice, c.stream));
        MP_CK(cudaMemcpyAsync(M.d_beta + nr, beta0_edge, sizeof(double) * (nr + 1), cudaMemcpyHostToDevice, c.stream));
    }
    launch(c, rg_grow(c, 0), 1, k_mp_gather, c.V(), g, srhs, srho, be, c.P.dx[0], c.P.dx[1], c.P.dx[2], l[0], l[1],
           l[2]);
    auto faces = [&](long n, int d) { return n / g.n[d] * (g.n[d] + 1); };
    k_mp_bcoef<0><<<blocks_of(faces(ncell(g), 0)), TPB, 0, c.stream>>>(g, bc, be);
    k_mp_bcoef<1><<<blocks_of(faces(ncell(g), 1)), TPB, 0, c.stream>>>(g, bc, be);
    k_mp_bcoef<2><<<blocks_of(faces(ncell(g), 2)), TPB, 0, c.stream>>>(g, bc, be);
    c.launches += 3;
    for (size_t q = 1; q < M.lev.size(); ++q) {
        const MGGrid &f = M.lev[q - 1], &cg = M.lev[q];
        const long nc = ncell(cg);
        k_mg_coarsen_b<0><<<blocks_of(nc / cg.n[0] * (cg.n[0] + 1)), TPB, 0, c.stream>>>(f, cg);
        k_mg_coarsen_b<1><<<blocks_of(nc / cg.n[1] * (cg.n[1] + 1)), TPB, 0, c.stream>>>(f, cg);
        k_mg_coarsen_b<2><<<blocks_of(nc / cg.n[2] * (cg.n[2] + 1)), TPB, 0, c.stream>>>(f, cg);
        c.launches += 3;
    }
    for (const MGGrid& q : M.lev) {  // the weights and diagonals every sweep reads
        const long nc = ncell(q);
        k_mg_prep_w<0><<<blocks_of(nc / q.n[0] * (q.n[0] + 1)), TPB, 0, c.stream>>>(q);
        k_mg_prep_w<1><<<blocks_of(nc / q.n[1] * (q.n[1] + 1)), TPB, 0, c.stream>>>(q);
        k_mg_prep_w<2><<<blocks_of(nc / q.n[2] * (q.n[2] + 1)), TPB, 0, c.stream>>>(q);
        k_mg_prep_diag<<<blocks_of(nc), TPB, 0, c.stream>>>(q, bc);
        c.launches += 4;
    }
    const long n = ncell(g);
    if (!dirichlet) {  // singular: the rhs made mean-free
        double dummy;
        if ((rc = mg_norms(c, g.rhs, n, dummy, nullptr, true))) return rc;
        k_mg_shift<<<blocks_of(n), TPB, 0, c.stream>>>(g.rhs, n, M.d_sum, 1.0 / (double)n);
        c.launches++;
    }
    double rhs_max = 0.0;
    if ((rc = mg_norms(c, g.rhs, n, rhs_max, nullptr))) return rc;
    const double target = tol_rel * rhs_max;
    int it = 0;
    double res_max = 0.0;
    if (!c.sph) {  // V-cycles on the residual equation until the reference's stopping test holds
        while (true) {
            mg_resid(c, g, bc);
            if ((rc = mg_norms(c, g.res, n, res_max, nullptr))) return rc;
            if (res_max <= target || it >= max_iter) break;
            mg_vcycle(c, bc, 0);
            ++it;
        }
    } else if ((rc = mac_pcg(c, bc, target, max_iter, it, res_max))) {
        return rc;
    }
    if (iters_out) *iters_out = it;
    if (ratio_out) *ratio_out = rhs_max > 0.0 ? res_max / rhs_max : 0.0;
    if (res_max > target) {
        set_error("MAC projection: multigrid did not reach the tolerance in " + std::to_string(max_iter) +
                  " V-cycles");
        return MADV_ERR_NOCONV;
    }
    if (!dirichlet) {  // phi made mean-free
        double dummy;
        if ((rc = mg_norms(c, g.phi, n, dummy, nullptr, true))) return rc;
        k_mg_shift<<<blocks_of(n), TPB, 0, c.stream>>>(g.phi, n, M.d_sum, 1.0 / (double)n);
        c.launches++;
    }
    launch(c, rg_grow(c, 0, 0), 1, k_mp_correct<0>, c.V(), g, bc, be, 1.0 / c.P.dx[0], l[0], l[1], l[2]);
    launch(c, rg_grow(c, 0, 1), 1, k_mp_correct<1>, c.V(), g, bc, be, 1.0 / c.P.dx[1], l[0], l[1], l[2]);
    launch(c, rg_grow(c, 0, 2), 1, k_mp_correct<2>, c.V(), g, bc, be, 1.0 / c.P.dx[2], l[0], l[1], l[2]);
    if (sphi >= 0) launch(c, rg_grow(c, 0), 1, k_mp_phi_out, c.V(), g, sphi, l[0], l[1], l[2]);
    fill_face_ghosts(c, F_UMAC0);
    return MADV_OK;
}


// ======================================================================= two levels
// The composite system (plane-parallel, refinement ratio 2).  Unknowns: phi on the level-0
// cells no level-1 box covers and on the level-1 cells.  A level-1 cell sees across a
// coarse-fine face the ghost (1/3) phi_c + (2/3) phi_parent (linear along the normal between
// its own centre, h1/2 inside, and the coarse centre, h1 outside): face weight (2/3) W1.  A
// level-0 cell takes across a face shared with a covered cell the mean of the four fine
// fluxes: weight (1/4)(2/3) B1 / (h0 h1) per fine cell.  With volume weights the operator is
// symmetric.  MLMG's coarse-fine interpolation is AMReX's and not restated here.

// the neighbour of grid cell a along D on side s (-1 / +1): false outside a non-periodic
// face (t receives the face's boundary type), else b holds it (wrapped)
__device__ __forceinline__ bool ml_nb(const MGGrid& g, const MGBC& bc, const int a[3], int D, int s, int b[3], int& t) {
    b[0] = a[0];
    b[1] = a[1];
    b[2] = a[2];
    b[D] += s;
    if (b[D] >= 0 && b[D] < g.n[D]) return true;
    t = s < 0 ? bc.lo[D] : bc.hi[D];
    if (t != MG_PER) return false;
    b[D] = s < 0 ? g.n[D] - 1 : 0;
    return true;
}
// face index along D of the s-side face of cell a
__device__ __forceinline__ long ml_face(const MGGrid& g, const int a[3], int D, int s) {
    int f[3] = {a[0], a[1], a[2]};
    if (s > 0) f[D] += 1;
    return D == 0 ? mg_face<0>(g, f[0], f[1], f[2]) : (D == 1 ? mg_face<1>(g, f[0], f[1], f[2]) : mg_face<2>(g, f[0], f[1], f[2]));
}

// level-1 cells of the boxes (valid cells of the fine level) into the mask
__global__ void k_ml_mask(KARGS, MGGrid F, double* mask, int l0, int l1, int l2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    mask[mg_cell(F, i - l0, j - l1, k - l2)] = 1.0;
}
// covered level-0 cells: all eight children in the mask
__global__ void k_ml_cov(MGGrid C, MGGrid F, const double* __restrict__ mask, double* cov) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)C.n[0] * C.n[1] * C.n[2]) return;
    int I, J, K;
    mg_ijk(C, c, I, J, K);
    double m = 1.0;
    for (int q = 0; q < 8; ++q) m *= mask[mg_cell(F, 2 * I + (q & 1), 2 * J + ((q >> 1) & 1), 2 * K + (q >> 2))];
    cov[c] = m;
}

// valid cells of a level: rho into g.res, macrhs into g.rhs, phi = 0
__global__ void k_ml_gather_cells(KARGS, MGGrid g, int srhs, int srho, int l0, int l1, int l2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const long c = mg_cell(g, i - l0, j - l1, k - l2);
    g.res[c] = at(VW(F_USER + srho), i, j, k);
    g.rhs[c] = at(VW(F_USER + srhs), i, j, k);
    g.phi[c] = 0.0;
}
// valid D-faces of a level: beta0 umac into g.W[D] (scratch until the weights are formed)
template <int D>
__global__ void k_ml_gather_faces(KARGS, MGGrid g, MPBeta be, int l0, int l1, int l2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const int a0 = i - l0, a1 = j - l1, a2 = k - l2;
    g.W[D][mg_face<D>(g, a0, a1, a2)] = at(VW(F_UMAC0 + D), i, j, k) * mp_beta<D>(be, g, a0, a1, a2);
}
// a level-1 face belongs to a box when a cell on either side is in the mask (across a
// periodic face, the wrapped cell)
template <int D>
__device__ __forceinline__ bool ml_box_face(const MGGrid& F, const MGBC& bc, const double* __restrict__ mask, int f0,
                                            int f1, int f2) {
    const int a[3] = {f0, f1, f2};
    int l[3] = {f0, f1, f2}, r[3] = {f0, f1, f2};
    l[D] -= 1;
    bool in = false;
    if (a[D] < F.n[D]) in = in || mask[mg_cell(F, r[0], r[1], r[2])] != 0.0;
    else if (bc.hi[D] == MG_PER) {
        r[D] = 0;
        in = in || mask[mg_cell(F, r[0], r[1], r[2])] != 0.0;
    }
    if (a[D] > 0) in = in || mask[mg_cell(F, l[0], l[1], l[2])] != 0.0;
    else if (bc.lo[D] == MG_PER) {
        l[D] = F.n[D] - 1;
        in = in || mask[mg_cell(F, l[0], l[1], l[2])] != 0.0;
    }
    return in;
}
// AverageDownFaces of beta0 umac: a level-0 face whose four level-1 faces belong to boxes
// takes their mean
template <int D>
__global__ void k_ml_avgdown_bu(MGGrid C, MGGrid F, MGBC bc, const double* __restrict__ mask) {
    constexpr int T1 = D == 0 ? 1 : 0, T2 = D == 2 ? 1 : 2;
    int nc[3] = {C.n[0], C.n[1], C.n[2]};
    nc[D] += 1;
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)nc[0] * nc[1] * nc[2]) return;
    int a[3];
    a[0] = (int)(c % nc[0]);
    a[1] = (int)((c / nc[0]) % nc[1]);
    a[2] = (int)(c / ((long)nc[0] * nc[1]));
    double s = 0.0;
    for (int q = 0; q < 4; ++q) {
        int b[3] = {2 * a[0], 2 * a[1], 2 * a[2]};
        b[T1] += q & 1;
        b[T2] += q >> 1;
        if (!ml_box_face<D>(F, bc, mask, b[0], b[1], b[2])) return;
        s += F.W[D][mg_face<D>(F, b[0], b[1], b[2])];
    }
    C.W[D][c] = 0.25 * s;
}
// rhs -= div(beta0 umac) (faces in g.W), on the cells of weight != 0 (every cell: wt null)
__global__ void k_ml_rhs(MGGrid g, const double* __restrict__ wt) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)g.n[0] * g.n[1] * g.n[2]) return;
    if (wt && wt[c] == 0.0) {
        g.rhs[c] = 0.0;
        return;
    }
    int i, j, k;
    mg_ijk(g, c, i, j, k);
    const double h0 = sqrt(1.0 / g.ih2[0]), h1 = sqrt(1.0 / g.ih2[1]), h2 = sqrt(1.0 / g.ih2[2]);
    g.rhs[c] -= (g.W[0][mg_face<0>(g, i + 1, j, k)] - g.W[0][mg_face<0>(g, i, j, k)]) / h0 +
                (g.W[1][mg_face<1>(g, i, j + 1, k)] - g.W[1][mg_face<1>(g, i, j, k)]) / h1 +
                (g.W[2][mg_face<2>(g, i, j, k + 1)] - g.W[2][mg_face<2>(g, i, j, k)]) / h2;
}
// level-1 cells off the boxes take their parent's rho (the outside of a coarse-fine face)
__global__ void k_ml_rho_out(MGGrid F, MGGrid C, const double* __restrict__ mask) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)F.n[0] * F.n[1] * F.n[2]) return;
    if (mask[c] != 0.0) return;
    int i, j, k;
    mg_ijk(F, c, i, j, k);
    F.res[c] = C.res[mg_cell(C, i / 2, j / 2, k / 2)];
}

// the weight of the s-side face of level-1 cell a toward a coarse-fine ghost or a fine
// neighbour; fc receives the neighbour (or the parent, coarse) and its kind
struct MLTerm {
    double w;
    long nb;   // fine neighbour, or parent coarse cell, or -1 (boundary)
    int coarse;
};
__device__ __forceinline__ MLTerm ml_fine_term(const MGGrid& F, const MGGrid& C, const MGBC& bc,
                                               const double* __restrict__ mask, const int a[3], int D, int s) {
    const double W = F.W[D][ml_face(F, a, D, s)];
    int b[3], t = MG_PER;
    if (!ml_nb(F, bc, a, D, s, b, t)) return MLTerm{t == MG_DIR ? 2.0 * W : 0.0, -1, 0};
    const long nb = mg_cell(F, b[0], b[1], b[2]);
    if (mask[nb] != 0.0) return MLTerm{W, nb, 0};
    return MLTerm{(2.0 / 3.0) * W, mg_cell(C, b[0] / 2, b[1] / 2, b[2] / 2), 1};
}

// composite diagonal of the level-1 cells
__global__ void k_ml_cdiag1(MGGrid F, MGGrid C, MGBC bc, const double* __restrict__ mask, double* cd) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)F.n[0] * F.n[1] * F.n[2]) return;
    if (mask[c] == 0.0) {
        cd[c] = 0.0;
        return;
    }
    int a[3];
    mg_ijk(F, c, a[0], a[1], a[2]);
    double d = 0.0;
    for (int D = 0; D < 3; ++D)
        for (int s = -1; s <= 1; s += 2) d += ml_fine_term(F, C, bc, mask, a, D, s).w;
    cd[c] = d;
}

// the level-0 side of a coarse-fine face: the four level-1 cells behind it and the weight of
// each, (1/4)(2/3) B1 / (h0 h1) = W1 / 12 (W1 = B1 / h1^2, h0 = 2 h1)
__device__ __forceinline__ void ml_cf_cells(const MGGrid& F, const int q[3], int D, int s, long cells[4], double w[4]) {
    const int T1 = D == 0 ? 1 : 0, T2 = D == 2 ? 1 : 2;
    for (int m = 0; m < 4; ++m) {
        int cc[3] = {2 * q[0], 2 * q[1], 2 * q[2]};
        cc[D] = s > 0 ? 2 * q[D] : 2 * q[D] + 1;
        cc[T1] += m & 1;
        cc[T2] += m >> 1;
        cells[m] = mg_cell(F, cc[0], cc[1], cc[2]);
        w[m] = F.W[D][ml_face(F, cc, D, -s)] / 12.0;
    }
}

// composite diagonal of the uncovered level-0 cells (0 on covered ones)
__global__ void k_ml_cdiag0(MGGrid C, MGGrid F, MGBC bc, const double* __restrict__ cov, double* cd) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)C.n[0] * C.n[1] * C.n[2]) return;
    if (cov[c] != 0.0) {
        cd[c] = 0.0;
        return;
    }
    int a[3];
    mg_ijk(C, c, a[0], a[1], a[2]);
    double d = 0.0;
    for (int D = 0; D < 3; ++D)
        for (int s = -1; s <= 1; s += 2) {
            const double W = C.W[D][ml_face(C, a, D, s)];
            int q[3], t = MG_PER;
            if (!ml_nb(C, bc, a, D, s, q, t)) {
                if (t == MG_DIR) d += 2.0 * W;
                continue;
            }
            if (cov[mg_cell(C, q[0], q[1], q[2])] == 0.0) {
                d += W;
                continue;
            }
            long cells[4];
            double w[4];
            ml_cf_cells(F, q, D, s, cells, w);
            d += w[0] + w[1] + w[2] + w[3];
        }
    cd[c] = d;
}

// q = A p on both levels (cells outside the unknowns get 0)
__global__ void k_ml_apply0(MGGrid C, MGGrid F, MGBC bc, const double* __restrict__ cov,
                            const double* __restrict__ cd, const double* __restrict__ p0,
                            const double* __restrict__ p1, double* __restrict__ q0) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)C.n[0] * C.n[1] * C.n[2]) return;
    if (cov[c] != 0.0) {
        q0[c] = 0.0;
        return;
    }
    int a[3];
    mg_ijk(C, c, a[0], a[1], a[2]);
    double off = 0.0;
    for (int D = 0; D < 3; ++D)
        for (int s = -1; s <= 1; s += 2) {
            int q[3], t = MG_PER;
            if (!ml_nb(C, bc, a, D, s, q, t)) continue;
            const long nb = mg_cell(C, q[0], q[1], q[2]);
            if (cov[nb] == 0.0) {
                off += C.W[D][ml_face(C, a, D, s)] * p0[nb];
                continue;
            }
            long cells[4];
            double w[4];
            ml_cf_cells(F, q, D, s, cells, w);
            for (int m = 0; m < 4; ++m) off += w[m] * p1[cells[m]];
        }
    q0[c] = cd[c] * p0[c] - off;
}
__global__ void k_ml_apply1(MGGrid F, MGGrid C, MGBC bc, const double* __restrict__ mask,
                            const double* __restrict__ cd, const double* __restrict__ p1,
                            const double* __restrict__ p0, double* __restrict__ q1) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)F.n[0] * F.n[1] * F.n[2]) return;
    if (mask[c] == 0.0) {
        q1[c] = 0.0;
        return;
    }
    int a[3];
    mg_ijk(F, c, a[0], a[1], a[2]);
    double off = 0.0;
    for (int D = 0; D < 3; ++D)
        for (int s = -1; s <= 1; s += 2) {
            const MLTerm t = ml_fine_term(F, C, bc, mask, a, D, s);
            if (t.nb >= 0) off += t.w * (t.coarse ? p0[t.nb] : p1[t.nb]);
        }
    q1[c] = cd[c] * p1[c] - off;
}

// part[block] = the block's sum over both levels of wt * x * y (weights: 1 on uncovered
// level-0 cells, 1/8 on level-1 cells of the boxes, 0 elsewhere), in a fixed order;
// out_max (when given) = max |x| over the unknowns
__global__ void k_ml_dot(const double* __restrict__ x0, const double* __restrict__ y0, const double* __restrict__ cov,
                         long n0, const double* __restrict__ x1, const double* __restrict__ y1,
                         const double* __restrict__ mask, long n1, double* part, unsigned long long* out_max) {
    __shared__ double ws[32];
    double s = 0.0, m = 0.0;
    for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < n0 + n1; c += (long)gridDim.x * blockDim.x) {
        double w, x, y;
        if (c < n0) {
            w = 1.0 - cov[c];
            x = x0[c];
            y = y0 ? y0[c] : 1.0;
        } else {
            w = 0.125 * mask[c - n0];
            x = x1[c - n0];
            y = y1 ? y1[c - n0] : 1.0;
        }
        if (w != 0.0) {
            s += w * x * y;
            m = fmax(m, fabs(x));
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, o);
        m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    }
    if ((threadIdx.x & 31) == 0) {
        ws[threadIdx.x >> 5] = s;
        if (out_max) atomicMax(out_max, (unsigned long long)__double_as_longlong(m));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += ws[w];
        part[blockIdx.x] = b;
    }
}
// x -= sum / vol on the unknowns (a mean-free projection of a singular system)
__global__ void k_ml_shift(double* __restrict__ x0, const double* __restrict__ cov, long n0, double* __restrict__ x1,
                           const double* __restrict__ mask, long n1, const double* __restrict__ sum, double inv_vol) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c < n0) {
        if (cov[c] == 0.0) x0[c] -= sum[0] * inv_vol;
    } else if (c < n0 + n1) {
        if (mask[c - n0] != 0.0) x1[c - n0] -= sum[0] * inv_vol;
    }
}

// preconditioner: the coarse rhs (uncovered cells: r0; covered: the mean of the children's
// r1), a level-0 V-cycle, the result prolonged to level 1 and smoothed there
__global__ void k_ml_restrict(MGGrid C, MGGrid F, const double* __restrict__ cov, const double* __restrict__ r0,
                              const double* __restrict__ r1) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)C.n[0] * C.n[1] * C.n[2]) return;
    double v = r0[c];
    if (cov[c] != 0.0) {
        int I, J, K;
        mg_ijk(C, c, I, J, K);
        double s = 0.0;
        for (int q = 0; q < 8; ++q) s += r1[mg_cell(F, 2 * I + (q & 1), 2 * J + ((q >> 1) & 1), 2 * K + (q >> 2))];
        v = 0.125 * s;
    }
    C.rhs[c] = v;
    C.phi[c] = 0.0;
}
__global__ void k_ml_prolong(MGGrid F, MGGrid C, const double* __restrict__ mask, const double* __restrict__ cov,
                             double* __restrict__ z0, double* __restrict__ z1) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long n0 = (long)C.n[0] * C.n[1] * C.n[2];
    if (c < n0) z0[c] = cov[c] != 0.0 ? 0.0 : C.phi[c];
    if (c >= (long)F.n[0] * F.n[1] * F.n[2]) return;
    int i, j, k;
    mg_ijk(F, c, i, j, k);
    z1[c] = mask[c] != 0.0 ? C.phi[mg_cell(C, i / 2, j / 2, k / 2)] : 0.0;
}
// Gauss-Seidel on the level-1 cells of one colour for A z = r, the coarse-fine ghosts from z0
__global__ void k_ml_smooth1(MGGrid F, MGGrid C, MGBC bc, const double* __restrict__ mask,
                             const double* __restrict__ cd, const double* __restrict__ r1,
                             const double* __restrict__ z0, double* __restrict__ z1, int color) {
    const long half = (long)F.n[0] * F.n[1] * F.n[2] / 2;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= half) return;
    const long row = t / (F.n[0] / 2);
    const int jj = (int)(row % F.n[1]), kk = (int)(row / F.n[1]);
    const int ii = 2 * (int)(t % (F.n[0] / 2)) + ((jj + kk + color) & 1);
    const long c = mg_cell(F, ii, jj, kk);
    if (mask[c] == 0.0 || cd[c] <= 0.0) return;
    const int a[3] = {ii, jj, kk};
    double off = 0.0;
    for (int D = 0; D < 3; ++D)
        for (int s = -1; s <= 1; s += 2) {
            const MLTerm q = ml_fine_term(F, C, bc, mask, a, D, s);
            if (q.nb >= 0) off += q.w * (q.coarse ? z0[q.nb] : z1[q.nb]);
        }
    z1[c] = (r1[c] + off) / cd[c];
}
// x += a p, r -= a q on a level
__global__ void k_ml_step(double* __restrict__ x, double* __restrict__ r, const double* __restrict__ p,
                          const double* __restrict__ q, double a, long n) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    x[c] += a * p[c];
    r[c] -= a * q[c];
}

// phi of both levels from the solution: level 1 on its cells; level 0 on the uncovered
// cells, and on the covered ones the mean of the children
__global__ void k_ml_phi(MGGrid C, MGGrid F, const double* __restrict__ cov, const double* __restrict__ mask,
                         const double* __restrict__ x0, const double* __restrict__ x1) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long n0 = (long)C.n[0] * C.n[1] * C.n[2], n1 = (long)F.n[0] * F.n[1] * F.n[2];
    if (c < n1) F.phi[c] = mask[c] != 0.0 ? x1[c] : 0.0;
    if (c >= n0) return;
    if (cov[c] == 0.0) {
        C.phi[c] = x0[c];
        return;
    }
    int I, J, K;
    mg_ijk(C, c, I, J, K);
    double s = 0.0;
    for (int q = 0; q < 8; ++q) s += x1[mg_cell(F, 2 * I + (q & 1), 2 * J + ((q >> 1) & 1), 2 * K + (q >> 2))];
    C.phi[c] = 0.125 * s;
}

// valid D-faces of the level-1 boxes: beta0 umac += -B grad phi, umac /= beta0; a cell off
// the boxes is the ghost (1/3) phi of the cell across + (2/3) phi of its parent
template <int D>
__global__ void k_ml_correct1(KARGS, MGGrid F, MGGrid C, MGBC bc, MPBeta be, const double* __restrict__ mask,
                              double inv_h, int l0, int l1, int l2) {
    MADV_ELEMENT(R, ne, g0, g1, b, i, j, k);
    const int a[3] = {i - l0, j - l1, k - l2};
    const double B = F.B[D][mg_face<D>(F, a[0], a[1], a[2])];
    int r[3] = {a[0], a[1], a[2]};  // the cell on the high side (wrapped)
    if (r[D] >= F.n[D]) r[D] = 0;
    auto value = [&](const int q[3], const int other[3]) {
        const long cq = mg_cell(F, q[0], q[1], q[2]);
        if (mask[cq] != 0.0) return F.phi[cq];
        return (1.0 / 3.0) * F.phi[mg_cell(F, other[0], other[1], other[2])] +
               (2.0 / 3.0) * C.phi[mg_cell(C, q[0] / 2, q[1] / 2, q[2] / 2)];
    };
    double grad;
    if (a[D] == 0 && bc.lo[D] != MG_PER) {
        grad = bc.lo[D] == MG_DIR ? (F.phi[mg_cell(F, r[0], r[1], r[2])] - (-F.phi[mg_cell(F, r[0], r[1], r[2])])) * inv_h
                                  : 0.0;
    } else if (a[D] == F.n[D] && bc.hi[D] != MG_PER) {
        int q[3] = {a[0], a[1], a[2]};
        q[D] = F.n[D] - 1;
        const double v = F.phi[mg_cell(F, q[0], q[1], q[2])];
        grad = bc.hi[D] == MG_DIR ? ((-v) - v) * inv_h : 0.0;
    } else {
        int q[3] = {a[0], a[1], a[2]};  // the low-side cell (wrapped)
        q[D] = a[D] == 0 ? F.n[D] - 1 : a[D] - 1;
        grad = (value(r, q) - value(q, r)) * inv_h;
    }
    const double beta = mp_beta<D>(be, F, a[0], a[1], a[2]);
    double& u = at(VW(F_UMAC0 + D), i, j, k);
    u = (u * beta + -B * grad) / beta;
}


// sum over the unknowns of both levels of wt x y (y null: wt x) and max |x|, read back
static int ml_dot(Ctx& c, const double* x0, const double* y0, long n0, const double* x1, const double* y1, long n1,
                  double& sum, double* amax) {
    MacMG& M = *c.mac;
    MLFine& L = *M.ml;
    if (amax) MP_CK(cudaMemsetAsync(M.d_max, 0, sizeof(unsigned long long), c.stream));
    const unsigned nb = (unsigned)std::min<long>((n0 + n1 + TPB - 1) / TPB, NORM_BLOCKS);
    k_ml_dot<<<nb, TPB, 0, c.stream>>>(x0, y0, L.cov, n0, x1, y1, L.mask, n1, M.d_part, amax ? M.d_max : nullptr);
    k_mg_sum_parts<<<1, 1, 0, c.stream>>>(M.d_part, (int)nb, M.d_sum);
    c.launches += 2;
    unsigned long long bits = 0;
    MP_CK(cudaMemcpyAsync(&sum, M.d_sum, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    if (amax) MP_CK(cudaMemcpyAsync(&bits, M.d_max, sizeof(bits), cudaMemcpyDeviceToHost, c.stream));
    MP_CK(cudaStreamSynchronize(c.stream));
    if (amax) std::memcpy(amax, &bits, sizeof(double));
    return MADV_OK;
}

// MacProj on two plane-parallel levels (the composite system above).  The caller has bound
// macrhs (slot srhs), rho (srho), macphi (sphi, may be < 0) on both levels and copied umac
// into F_UMAC0..2 of both; umac is corrected there (level-0 faces under level 1 are left for
// the caller's AverageDownFaces).  b0c / b0ce: beta0 and its edges of level 0 (nr0, nr0 + 1);
// b1 / b1e of level 1 (nr1 = 2 nr0).  The solve: conjugate gradients in the volume-weighted
// inner product, preconditioned by a level-0 V-cycle on the restricted residual, prolonged
// and smoothed on level 1 (two red-black sweeps), flexible update; every sum in a fixed order.
int mac_project_two_levels(Ctx& c, Ctx& f, int srhs, int srho, int sphi, const double* b0c, const double* b0ce,
                           const double* b1, const double* b1e, double tol_rel, int max_iter, int* iters_out,
                           double* ratio_out) {
    int n0[3], lo0[3], lo1[3], n1[3];
    MGBC bc{};
    bool dirichlet = false;
    for (int d = 0; d < 3; ++d) {
        lo0[d] = c.P.dom_lo[d];
        lo1[d] = f.P.dom_lo[d];
        n0[d] = c.P.dom_hi[d] - c.P.dom_lo[d] + 1;
        n1[d] = 2 * n0[d];
        if (n0[d] % 2 != 0) {
            set_error("the MAC projection needs even domain extents");
            return MADV_ERR_UNSUPPORTED;
        }
        auto t = [&](int pb) {
            if (c.per[d]) return (int)MG_PER;
            if (pb == PB_OUTFLOW) return (int)MG_DIR;
            return (int)MG_NEU;
        };
        bc.lo[d] = t(c.P.phys_bc_lo[d]);
        bc.hi[d] = t(c.P.phys_bc_hi[d]);
        dirichlet = dirichlet || bc.lo[d] == MG_DIR || bc.hi[d] == MG_DIR;
    }
    const int nr0 = n0[2], nr1 = n1[2];
    int rc = mac_hierarchy(c, n0, nr0);
    if (rc) return rc;
    MacMG& M = *c.mac;
    if (!M.ml || M.ml->n1[0] != n1[0] || M.ml->n1[1] != n1[1] || M.ml->n1[2] != n1[2]) {
        ml_free(M.ml);
        M.ml = new MLFine();
        MLFine& L = *M.ml;
        for (int d = 0; d < 3; ++d) L.n1[d] = n1[d];
        const long c1 = (long)n1[0] * n1[1] * n1[2], c0 = (long)n0[0] * n0[1] * n0[2];
        auto alloc = [&](long cnt) -> double* {
            double* p = nullptr;
            if (cudaMalloc(&p, sizeof(double) * cnt) != cudaSuccess) return nullptr;
            L.mem.push_back(p);
            return p;
        };
        MGGrid& F = L.g;
        for (int d = 0; d < 3; ++d) F.n[d] = n1[d];
        F.phi = alloc(c1);
        F.rhs = alloc(c1);
        F.res = alloc(c1);
        bool ok = F.phi && F.rhs && F.res;
        for (int d = 0; d < 3; ++d) {
            F.B[d] = alloc(c1 / n1[d] * (n1[d] + 1));
            F.W[d] = alloc(c1 / n1[d] * (n1[d] + 1));
            ok = ok && F.B[d] && F.W[d];
        }
        L.mask = alloc(c1);
        L.cov = alloc(c0);
        L.cdiag0 = alloc(c0);
        L.cdiag1 = alloc(c1);
        L.v0 = alloc(5 * c0);
        L.v1 = alloc(5 * c1);
        L.beta1 = alloc(2 * nr1 + 1);
        ok = ok && L.mask && L.cov && L.cdiag0 && L.cdiag1 && L.v0 && L.v1 && L.beta1;
        if (!ok) {
            ml_free(M.ml);
            set_error("cudaMalloc(two-level MAC projection)");
            return MADV_ERR_CUDA;
        }
    }
    MLFine& L = *M.ml;
    MGGrid& C = M.lev[0];
    MGGrid& F = L.g;
    for (int d = 0; d < 3; ++d) F.ih2[d] = 1.0 / (f.P.dx[d] * f.P.dx[d]);
    const long N0 = ncell(C), N1 = ncell(F);
    MP_CK(cudaMemcpyAsync(M.d_beta, b0c, sizeof(double) * nr0, cudaMemcpyHostToDevice, c.stream));
    MP_CK(cudaMemcpyAsync(M.d_beta + nr0, b0ce, sizeof(double) * (nr0 + 1), cudaMemcpyHostToDevice, c.stream));
    MP_CK(cudaMemcpyAsync(L.beta1, b1, sizeof(double) * nr1, cudaMemcpyHostToDevice, c.stream));
    MP_CK(cudaMemcpyAsync(L.beta1 + nr1, b1e, sizeof(double) * (nr1 + 1), cudaMemcpyHostToDevice, c.stream));
    const MPBeta be0{M.d_beta, M.d_beta + nr0, {nullptr, nullptr, nullptr}, 0};
    const MPBeta be1{L.beta1, L.beta1 + nr1, {nullptr, nullptr, nullptr}, 0};
    // the level-1 cells and the covered level-0 cells
    MP_CK(cudaMemsetAsync(L.mask, 0, sizeof(double) * N1, c.stream));
    launch(f, rg_grow(f, 0), 1, k_ml_mask, f.V(), F, L.mask, lo1[0], lo1[1], lo1[2]);
    k_ml_cov<<<blocks_of(N0), TPB, 0, c.stream>>>(C, F, L.mask, L.cov);
    // rho, macrhs and beta0 umac of both levels; beta0 umac averaged down; the rhs
    MP_CK(cudaMemsetAsync(F.res, 0, sizeof(double) * N1, c.stream));
    MP_CK(cudaMemsetAsync(F.rhs, 0, sizeof(double) * N1, c.stream));
    MP_CK(cudaMemsetAsync(F.phi, 0, sizeof(double) * N1, c.stream));
    auto faces = [&](const MGGrid& g, int d) { return ncell(g) / g.n[d] * (g.n[d] + 1); };
    for (int d = 0; d < 3; ++d) MP_CK(cudaMemsetAsync(F.W[d], 0, sizeof(double) * faces(F, d), c.stream));
    launch(c, rg_grow(c, 0), 1, k_ml_gather_cells, c.V(), C, srhs, srho, lo0[0], lo0[1], lo0[2]);
    launch(f, rg_grow(f, 0), 1, k_ml_gather_cells, f.V(), F, srhs, srho, lo1[0], lo1[1], lo1[2]);
    launch(c, rg_grow(c, 0, 0), 1, k_ml_gather_faces<0>, c.V(), C, be0, lo0[0], lo0[1], lo0[2]);
    launch(c, rg_grow(c, 0, 1), 1, k_ml_gather_faces<1>, c.V(), C, be0, lo0[0], lo0[1], lo0[2]);
    launch(c, rg_grow(c, 0, 2), 1, k_ml_gather_faces<2>, c.V(), C, be0, lo0[0], lo0[1], lo0[2]);
    launch(f, rg_grow(f, 0, 0), 1, k_ml_gather_faces<0>, f.V(), F, be1, lo1[0], lo1[1], lo1[2]);
    launch(f, rg_grow(f, 0, 1), 1, k_ml_gather_faces<1>, f.V(), F, be1, lo1[0], lo1[1], lo1[2]);
    launch(f, rg_grow(f, 0, 2), 1, k_ml_gather_faces<2>, f.V(), F, be1, lo1[0], lo1[1], lo1[2]);
    k_ml_avgdown_bu<0><<<blocks_of(faces(C, 0)), TPB, 0, c.stream>>>(C, F, bc, L.mask);
    k_ml_avgdown_bu<1><<<blocks_of(faces(C, 1)), TPB, 0, c.stream>>>(C, F, bc, L.mask);
    k_ml_avgdown_bu<2><<<blocks_of(faces(C, 2)), TPB, 0, c.stream>>>(C, F, bc, L.mask);
    k_ml_rhs<<<blocks_of(N0), TPB, 0, c.stream>>>(C, nullptr);
    k_ml_rhs<<<blocks_of(N1), TPB, 0, c.stream>>>(F, L.mask);
    k_ml_rho_out<<<blocks_of(N1), TPB, 0, c.stream>>>(F, C, L.mask);
    c.launches += 7;
    // face coefficients of both levels, the level-0 multigrid (the preconditioner's), weights
    k_mp_bcoef<0><<<blocks_of(faces(C, 0)), TPB, 0, c.stream>>>(C, bc, be0);
    k_mp_bcoef<1><<<blocks_of(faces(C, 1)), TPB, 0, c.stream>>>(C, bc, be0);
    k_mp_bcoef<2><<<blocks_of(faces(C, 2)), TPB, 0, c.stream>>>(C, bc, be0);
    k_mp_bcoef<0><<<blocks_of(faces(F, 0)), TPB, 0, c.stream>>>(F, bc, be1);
    k_mp_bcoef<1><<<blocks_of(faces(F, 1)), TPB, 0, c.stream>>>(F, bc, be1);
    k_mp_bcoef<2><<<blocks_of(faces(F, 2)), TPB, 0, c.stream>>>(F, bc, be1);
    c.launches += 6;
    for (size_t q = 1; q < M.lev.size(); ++q) {
        const MGGrid &fg = M.lev[q - 1], &cg = M.lev[q];
        k_mg_coarsen_b<0><<<blocks_of(faces(cg, 0)), TPB, 0, c.stream>>>(fg, cg);
        k_mg_coarsen_b<1><<<blocks_of(faces(cg, 1)), TPB, 0, c.stream>>>(fg, cg);
        k_mg_coarsen_b<2><<<blocks_of(faces(cg, 2)), TPB, 0, c.stream>>>(fg, cg);
        c.launches += 3;
    }
    for (const MGGrid& q : M.lev) {
        k_mg_prep_w<0><<<blocks_of(faces(q, 0)), TPB, 0, c.stream>>>(q);
        k_mg_prep_w<1><<<blocks_of(faces(q, 1)), TPB, 0, c.stream>>>(q);
        k_mg_prep_w<2><<<blocks_of(faces(q, 2)), TPB, 0, c.stream>>>(q);
        k_mg_prep_diag<<<blocks_of(ncell(q)), TPB, 0, c.stream>>>(q, bc);
        c.launches += 4;
    }
    k_mg_prep_w<0><<<blocks_of(faces(F, 0)), TPB, 0, c.stream>>>(F);
    k_mg_prep_w<1><<<blocks_of(faces(F, 1)), TPB, 0, c.stream>>>(F);
    k_mg_prep_w<2><<<blocks_of(faces(F, 2)), TPB, 0, c.stream>>>(F);
    k_ml_cdiag0<<<blocks_of(N0), TPB, 0, c.stream>>>(C, F, bc, L.cov, L.cdiag0);
    k_ml_cdiag1<<<blocks_of(N1), TPB, 0, c.stream>>>(F, C, bc, L.mask, L.cdiag1);
    c.launches += 5;
    // conjugate gradients on the composite system
    double *x0 = L.v0, *r0 = x0 + N0, *p0 = r0 + N0, *q0 = p0 + N0, *z0 = q0 + N0;
    double *x1 = L.v1, *r1 = x1 + N1, *p1 = r1 + N1, *q1 = p1 + N1, *z1 = q1 + N1;
    MP_CK(cudaMemsetAsync(x0, 0, sizeof(double) * N0, c.stream));
    MP_CK(cudaMemsetAsync(x1, 0, sizeof(double) * N1, c.stream));
    MP_CK(cudaMemcpyAsync(r0, C.rhs, sizeof(double) * N0, cudaMemcpyDeviceToDevice, c.stream));
    MP_CK(cudaMemcpyAsync(r1, F.rhs, sizeof(double) * N1, cudaMemcpyDeviceToDevice, c.stream));
    const double inv_vol = 1.0 / (double)N0;  // the composite volume in level-0 cells
    double sum = 0.0, rhs_max = 0.0;
    if (!dirichlet) {  // singular: the rhs made mean-free in the volume-weighted sense
        if ((rc = ml_dot(c, r0, nullptr, N0, r1, nullptr, N1, sum, nullptr))) return rc;
        k_ml_shift<<<blocks_of(N0 + N1), TPB, 0, c.stream>>>(r0, L.cov, N0, r1, L.mask, N1, M.d_sum, inv_vol);
        c.launches++;
    }
    if ((rc = ml_dot(c, r0, nullptr, N0, r1, nullptr, N1, sum, &rhs_max))) return rc;
    const double target = tol_rel * rhs_max;
    auto precondition = [&]() {
        k_ml_restrict<<<blocks_of(N0), TPB, 0, c.stream>>>(C, F, L.cov, r0, r1);
        c.launches++;
        mg_vcycle(c, bc, 0);
        k_ml_prolong<<<blocks_of(std::max(N0, N1)), TPB, 0, c.stream>>>(F, C, L.mask, L.cov, z0, z1);
        c.launches++;
        for (int s = 0; s < 2; ++s) {
            k_ml_smooth1<<<blocks_of(N1 / 2), TPB, 0, c.stream>>>(F, C, bc, L.mask, L.cdiag1, r1, z0, z1, s);
            c.launches++;
        }
        for (int s = 1; s >= 0; --s) {
            k_ml_smooth1<<<blocks_of(N1 / 2), TPB, 0, c.stream>>>(F, C, bc, L.mask, L.cdiag1, r1, z0, z1, s);
            c.launches++;
        }
    };
    auto apply = [&](const double* a0, const double* a1, double* b0, double* b1v) {
        k_ml_apply0<<<blocks_of(N0), TPB, 0, c.stream>>>(C, F, bc, L.cov, L.cdiag0, a0, a1, b0);
        k_ml_apply1<<<blocks_of(N1), TPB, 0, c.stream>>>(F, C, bc, L.mask, L.cdiag1, a1, a0, b1v);
        c.launches += 2;
    };
    int it = 0;
    double res_max = rhs_max;
    if (res_max > target) {
        precondition();
        MP_CK(cudaMemcpyAsync(p0, z0, sizeof(double) * N0, cudaMemcpyDeviceToDevice, c.stream));
        MP_CK(cudaMemcpyAsync(p1, z1, sizeof(double) * N1, cudaMemcpyDeviceToDevice, c.stream));
        double rz = 0.0;
        if ((rc = ml_dot(c, r0, z0, N0, r1, z1, N1, rz, nullptr))) return rc;
        while (it < max_iter) {
            apply(p0, p1, q0, q1);
            double pq = 0.0;
            if ((rc = ml_dot(c, p0, q0, N0, p1, q1, N1, pq, nullptr))) return rc;
            if (!(pq > 0.0)) break;
            const double a = rz / pq;
            k_ml_step<<<blocks_of(N0), TPB, 0, c.stream>>>(x0, r0, p0, q0, a, N0);
            k_ml_step<<<blocks_of(N1), TPB, 0, c.stream>>>(x1, r1, p1, q1, a, N1);
            c.launches += 2;
            ++it;
            if ((rc = ml_dot(c, r0, nullptr, N0, r1, nullptr, N1, sum, &res_max))) return rc;
            if (res_max <= target) break;
            // z_old into q, z = M^-1 r; flexible (Polak-Ribiere) beta = r.(z - z_old) / rz
            MP_CK(cudaMemcpyAsync(q0, z0, sizeof(double) * N0, cudaMemcpyDeviceToDevice, c.stream));
            MP_CK(cudaMemcpyAsync(q1, z1, sizeof(double) * N1, cudaMemcpyDeviceToDevice, c.stream));
            precondition();
            double rz_new = 0.0, rzo = 0.0;
            if ((rc = ml_dot(c, r0, z0, N0, r1, z1, N1, rz_new, nullptr)) ||
                (rc = ml_dot(c, r0, q0, N0, r1, q1, N1, rzo, nullptr)))
                return rc;
            const double bb = (rz_new - rzo) / rz;
            rz = rz_new;
            k_pcg_dir<<<blocks_of(N0), TPB, 0, c.stream>>>(p0, z0, bb, N0);
            k_pcg_dir<<<blocks_of(N1), TPB, 0, c.stream>>>(p1, z1, bb, N1);
            c.launches += 2;
        }
    }
    if (iters_out) *iters_out = it;
    if (ratio_out) *ratio_out = rhs_max > 0.0 ? res_max / rhs_max : 0.0;
    if (res_max > target) {
        set_error("MAC projection: the composite solve did not reach the tolerance in " + std::to_string(max_iter) +
                  " iterations");
        return MADV_ERR_NOCONV;
    }
    if (!dirichlet) {  // phi made mean-free (volume-weighted)
        if ((rc = ml_dot(c, x0, nullptr, N0, x1, nullptr, N1, sum, nullptr))) return rc;
        k_ml_shift<<<blocks_of(N0 + N1), TPB, 0, c.stream>>>(x0, L.cov, N0, x1, L.mask, N1, M.d_sum, inv_vol);
        c.launches++;
    }
    k_ml_phi<<<blocks_of(std::max(N0, N1)), TPB, 0, c.stream>>>(C, F, L.cov, L.mask, x0, x1);
    c.launches++;
    launch(c, rg_grow(c, 0, 0), 1, k_mp_correct<0>, c.V(), C, bc, be0, 1.0 / c.P.dx[0], lo0[0], lo0[1], lo0[2]);
    launch(c, rg_grow(c, 0, 1), 1, k_mp_correct<1>, c.V(), C, bc, be0, 1.0 / c.P.dx[1], lo0[0], lo0[1], lo0[2]);
    launch(c, rg_grow(c, 0, 2), 1, k_mp_correct<2>, c.V(), C, bc, be0, 1.0 / c.P.dx[2], lo0[0], lo0[1], lo0[2]);
    launch(f, rg_grow(f, 0, 0), 1, k_ml_correct1<0>, f.V(), F, C, bc, be1, (const double*)L.mask, 1.0 / f.P.dx[0],
           lo1[0], lo1[1], lo1[2]);
    launch(f, rg_grow(f, 0, 1), 1, k_ml_correct1<1>, f.V(), F, C, bc, be1, (const double*)L.mask, 1.0 / f.P.dx[1],
           lo1[0], lo1[1], lo1[2]);
    launch(f, rg_grow(f, 0, 2), 1, k_ml_correct1<2>, f.V(), F, C, bc, be1, (const double*)L.mask, 1.0 / f.P.dx[2],
           lo1[0], lo1[1], lo1[2]);
    if (sphi >= 0) {
        launch(c, rg_grow(c, 0), 1, k_mp_phi_out, c.V(), C, sphi, lo0[0], lo0[1], lo0[2]);
        launch(f, rg_grow(f, 0), 1, k_mp_phi_out, f.V(), F, sphi, lo1[0], lo1[1], lo1[2]);
    }
    return MADV_OK;
}

}  // namespace madv
