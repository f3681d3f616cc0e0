// Maestro::MacProj, plane-parallel, one level (Source/MaestroMacProj.cpp:11-236).
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

// Gauss-Seidel on the cells of one colour ((i + j + k) % 2 == color), from the stored weights
__global__ void k_mg_smooth(MGGrid g, MGBC bc, int color) {
    const long half = (long)g.n[0] * g.n[1] * g.n[2] / 2;
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= half) return;
    // the t-th cell of the colour: rows of n[0] cells hold n[0]/2 of each colour
    const long row = t / (g.n[0] / 2);
    const int jj = (int)(row % g.n[1]), kk = (int)(row / g.n[1]);
    const int ii = 2 * (int)(t % (g.n[0] / 2)) + ((jj + kk + color) & 1);
    const long c = mg_cell(g, ii, jj, kk);
    const double id = g.idiag[c];
    if (id > 0.0) g.phi[c] = (g.rhs[c] + mg_off(g, bc, g.phi, ii, jj, kk)) * id;
}

// res = rhs - A phi
__global__ void k_mg_resid(MGGrid g, MGBC bc) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)g.n[0] * g.n[1] * g.n[2]) return;
    int i, j, k;
    mg_ijk(g, c, i, j, k);
    g.res[c] = g.rhs[c] - (g.diag[c] * g.phi[c] - mg_off(g, bc, g.phi, i, j, k));
}

// coarse rhs = mean of the 8 fine residuals; coarse phi = 0
__global__ void k_mg_restrict(MGGrid f, MGGrid cg) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)cg.n[0] * cg.n[1] * cg.n[2]) return;
    int I, J, K;
    mg_ijk(cg, c, I, J, K);
    double s = 0.0;
    for (int q = 0; q < 8; ++q) s += f.res[mg_cell(f, 2 * I + (q & 1), 2 * J + ((q >> 1) & 1), 2 * K + (q >> 2))];
    cg.rhs[c] = 0.125 * s;
    cg.phi[c] = 0.0;
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
__global__ void k_mg_prolong(MGGrid cg, MGGrid f) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)f.n[0] * f.n[1] * f.n[2]) return;
    int i, j, k;
    mg_ijk(f, c, i, j, k);
    f.phi[c] += cg.phi[mg_cell(cg, i / 2, j / 2, k / 2)];
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
};

void mac_free(Ctx& c) {
    if (!c.mac) return;
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

static void mg_vcycle(Ctx& c, const MGBC& bc, int l) {
    MacMG& M = *c.mac;
    const MGGrid& g = M.lev[l];
    const int nmax = std::max(g.n[0], std::max(g.n[1], g.n[2]));
    const int nu = 2, bottom = std::min(2000, std::max(64, 2 * nmax * nmax));  // the coarsest grid: to convergence
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
    k_mg_resid<<<blocks_of(ncell(g)), TPB, 0, c.stream>>>(g, bc);
    k_mg_restrict<<<blocks_of(ncell(cg)), TPB, 0, c.stream>>>(g, cg);
    c.launches += 2;
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
            k_mg_resid<<<blocks_of(n), TPB, 0, c.stream>>>(g, bc);
            c.launches++;
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

}  // namespace madv
