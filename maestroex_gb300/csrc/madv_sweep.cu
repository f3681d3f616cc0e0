// Staged PPM sweep: the three steps of one PPM direction D (van Leer slopes, limited
// interface values, cell limiter + characteristic tracing; Source/MaestroPPM.cpp) fused in
// one kernel over tiles that are whole pencils along D.
//
// A tile is a rectangle of pencils: the full extent of the box grown by one along D and a
// small rectangle across it.  Its cells' data along D, with the PPM halo (3 cells for
// ppm_type 1, 4 for ppm_type 2), is staged in shared memory by the TMA engine: one bulk
// copy (cp.async.bulk, global -> shared, completion counted on an mbarrier) per row of
// contiguous x-values.  Staging along D needs no halo across D, so no FP64 work is
// repeated between tiles.  The slopes and interface values then live in shared memory
// only; the kernel writes just Ip / Im.  The arithmetic is the element functions of
// madv_ppm.cuh, applied to shared-memory views, so results are bitwise those of the
// three-launch form (k_dsvl, k_ppm_face, k_ppm_cell).
//
// Rows whose addresses or lengths do not meet the bulk copy's 16-byte rules (odd FAB
// extents) are staged with ordinary loads instead.  The mbarrier wait is bounded: after
// its limit the tile records MADV_FLAG_STAGE in the device flag and returns.
#include <cuda.h>

#include "madv_launch.cuh"
#include "madv_ppm.cuh"

namespace madv {

constexpr int SWEEP_TPB = 256;
constexpr int MADV_FLAG_STAGE = 8;

struct SweepTile {
    int b;
    int lo[3];  // first cell of the tile (the box grown by one)
    int n[3];   // cells of the tile per direction; n[D] is the whole pencil
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// bounded wait for phase `parity` of the mbarrier at `addr`
__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity) {
    for (int it = 0; it < (1 << 22); ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

template <int D, int PPMT, int UMAC>
__global__ void __launch_bounds__(SWEEP_TPB)
    k_ppm_sweep(const SweepTile* __restrict__ tiles, int tile0, const FabView* __restrict__ V, int nb, int fs,
                int sc, int fu, int uc, int fip, int fim, int lo_ext, int hi_ext, int domlo, int domhi, long long epsb,
                RecipC r6, int* flag) {
    extern __shared__ __align__(128) double sm[];
    __shared__ __align__(8) unsigned long long mbar;
    constexpr int di = D == 0, dj = D == 1, dk = D == 2;
    constexpr int GS = PPMT == 2 ? 4 : 3;  // stencil reach along D from the tile's cells
    const SweepTile t = tiles[tile0 + blockIdx.x];
    const int b = t.b;
    const FabView gs = V[fs * nb + b];

    // the staged box of s: the tile widened by GS - 1 along D; x from an even offset in the
    // FAB, x-length even (16-byte rows)
    int slo[3], se[3];
    for (int d = 0; d < 3; ++d) {
        slo[d] = t.lo[d] - (d == D ? GS - 1 : 0);
        se[d] = t.n[d] + (d == D ? 2 * (GS - 1) : 0);
    }
    const int shift = (slo[0] - gs.lo0) & 1;
    slo[0] -= shift;
    se[0] += shift;
    se[0] += se[0] & 1;
    const int px = se[0];
    const long ns = (long)px * se[1] * se[2];
    double* s_sm = sm;
    double* dv_sm = sm + ns;                             // ppm_type 1: slopes, same box as s
    double* f_sm = sm + (PPMT == 1 ? 2 * ns : ns);       // faces along D: one more along D
    const int fpx = px + di;
    const FabView sv{s_sm, slo[0], slo[1], slo[2], px, (long)px * se[1], 0};
    const FabView dvv{dv_sm, slo[0], slo[1], slo[2], px, (long)px * se[1], 0};
    const FabView fv{f_sm, slo[0], slo[1], slo[2], fpx, (long)fpx * (se[1] + dj), 0};

    // ---- stage s: one row per (y, z) of the staged box
    const int rows = se[1] * se[2];
    const double* g0 = &at(gs, slo[0], slo[1], slo[2], sc);
    const bool bulk = ((reinterpret_cast<uintptr_t>(g0) & 15) == 0) && ((gs.sj & 1) == 0) && ((gs.sk & 1) == 0) &&
                      slo[0] + px - 1 <= gs.lo0 + gs.sj - 1;
    const uint32_t mb = smem_u32(&mbar);
    if (bulk) {
        if (threadIdx.x == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            const uint32_t bytes = (uint32_t)(rows * px * 8);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
        }
        __syncthreads();
        for (int r = threadIdx.x; r < rows; r += blockDim.x) {
            const int y = slo[1] + r % se[1], z = slo[2] + r / se[1];
            const double* src = &at(gs, slo[0], y, z, sc);
            double* dst = s_sm + (long)r * px;
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    smem_u32(dst)),
                "l"(src), "r"(px * 8), "r"(mb)
                : "memory");
        }
        if (!mbar_wait(mb, 0)) {
            if (threadIdx.x == 0) atomicOr(flag, MADV_FLAG_STAGE);
            mbar_wait(mb, 0);  // the copies this tile issued, before its shared memory goes
            return;
        }
    } else {
        for (long e = threadIdx.x; e < (long)rows * px; e += blockDim.x) {
            const int r = (int)(e / px), x = (int)(e - (long)r * px);
            const int y = slo[1] + r % se[1], z = slo[2] + r / se[1];
            // the even-length row may end one past the FAB's x range: that value is never read
            s_sm[e] = slo[0] + x <= gs.lo0 + gs.sj - 1 ? at(gs, slo[0] + x, y, z, sc) : 0.0;
        }
        __syncthreads();
    }

    // ---- van Leer slopes (ppm_type 1): cells lo-2 .. hi+2 along D
    if (PPMT == 1) {
        int lo[3] = {t.lo[0], t.lo[1], t.lo[2]}, n[3] = {t.n[0], t.n[1], t.n[2]};
        lo[D] -= 1;
        n[D] += 2;
        const long cnt = (long)n[0] * n[1] * n[2];
        for (long e = threadIdx.x; e < cnt; e += blockDim.x) {
            const int i = lo[0] + (int)(e % n[0]);
            const long q = e / n[0];
            const int j = lo[1] + (int)(q % n[1]);
            const int k = lo[2] + (int)(q / n[1]);
            at(dvv, i, j, k) = ppm_dsvl<D>(sv, 0, i, j, k);
        }
        __syncthreads();
    }
    // ---- limited interface values: faces lo-1 .. hi+2 (ppm_type 2: lo-2 .. hi+3) along D
    {
        int lo[3] = {t.lo[0], t.lo[1], t.lo[2]}, n[3] = {t.n[0], t.n[1], t.n[2]};
        lo[D] -= PPMT == 2 ? 1 : 0;
        n[D] += PPMT == 2 ? 3 : 1;
        const long cnt = (long)n[0] * n[1] * n[2];
        for (long e = threadIdx.x; e < cnt; e += blockDim.x) {
            const int i = lo[0] + (int)(e % n[0]);
            const long q = e / n[0];
            const int j = lo[1] + (int)(q % n[1]);
            const int k = lo[2] + (int)(q / n[1]);
            at(fv, i, j, k) = ppm_face_value<D, PPMT>(sv, 0, dvv, i, j, k, lo_ext, hi_ext, domlo, domhi, r6);
        }
        __syncthreads();
    }
    // ---- cell limiter and tracing: the tile's cells
    const FabView u = V[fu * nb + b];
    const FabView ipv = V[fip * nb + b], imv = V[fim * nb + b];
    const FabView T = V[(UMAC ? F_TRA0 + D : F_TRC) * nb + b];
    const long cnt = (long)t.n[0] * t.n[1] * t.n[2];
    for (long e = threadIdx.x; e < cnt; e += blockDim.x) {
        const int i = t.lo[0] + (int)(e % t.n[0]);
        const long q = e / t.n[0];
        const int j = t.lo[1] + (int)(q % t.n[1]);
        const int k = t.lo[2] + (int)(q / t.n[1]);
        double smv, spv;
        ppm_cell_edges<D, PPMT>(sv, 0, fv, dvv, i, j, k, lo_ext, hi_ext, domlo, domhi, r6, smv, spv);
        double up, um, Ap, Bp, Am, Bm;
        if (UMAC) {
            up = at(u, i + di, j + dj, k + dk);
            um = at(u, i, j, k);
            Ap = at(T, i + di, j + dj, k + dk, 0);
            Bp = at(T, i + di, j + dj, k + dk, 1);
            Am = at(T, i, j, k, 0);
            Bm = at(T, i, j, k, 1);
        } else {
            up = um = at(u, i, j, k, uc);
            Ap = Am = at(T, i, j, k, 2 * D);
            Bp = Bm = at(T, i, j, k, 2 * D + 1);
        }
        double ip, im;
        ppm_trace(at(sv, i, j, k), smv, spv, up, um, Ap, Bp, Am, Bm, epsb, ip, im);
        at(ipv, i, j, k, D) = ip;
        at(imv, i, j, k, D) = im;
    }
}

// ---------------------------------------------------------------- host side
struct SweepPlan {
    SweepTile* d = nullptr;
    std::vector<SweepTile> h;
    std::vector<int> box_first;  // first tile of each box (and the total at the end)
    size_t smem = 0;
};

// tile shape across D: (tA, tB) cells in the two transverse directions (increasing index)
static void default_shape(int D, int& tA, int& tB) {
    if (D == 0) {
        tA = 4;  // y
        tB = 2;  // z
    } else {
        tA = 32;  // x
        tB = 2;
    }
}

static size_t smem_bytes(int D, int ppmt, const int n[3]) {
    const int GS = ppmt == 2 ? 4 : 3;
    int e[3] = {n[0], n[1], n[2]};
    e[D] += 2 * (GS - 1);
    e[0] += 2;  // even start and even length
    const long ns = (long)e[0] * e[1] * e[2];
    long nf = (long)(e[0] + (D == 0)) * (e[1] + (D == 1)) * (e[2] + (D == 2));
    return (size_t)((ppmt == 1 ? 2 * ns : ns) + nf) * sizeof(double);
}

static std::map<std::array<int, 4>, SweepPlan>& plans_of(Ctx& c) {
    static std::map<const Ctx*, std::map<std::array<int, 4>, SweepPlan>> all;
    return all[&c];
}

void sweep_free(Ctx& c) {
    auto& P = plans_of(c);
    for (auto& kv : P)
        if (kv.second.d) cudaFree(kv.second.d);
    P.clear();
}

static const SweepPlan* sweep_plan(Ctx& c, int D, int ppmt) {
    int tA, tB;
    default_shape(D, tA, tB);
    auto it = c.sweep_shape.find(D);
    if (it != c.sweep_shape.end()) {
        tA = it->second[0];
        tB = it->second[1];
    }
    const std::array<int, 4> key{D, ppmt, tA, tB};
    auto& P = plans_of(c);
    auto f = P.find(key);
    if (f != P.end()) return &f->second;
    SweepPlan pl;
    const int A = D == 0 ? 1 : 0, B = D == 2 ? 1 : 2;
    for (int b = 0; b < c.nb; ++b) {
        pl.box_first.push_back((int)pl.h.size());
        int lo[3], hi[3];
        for (int d = 0; d < 3; ++d) {
            lo[d] = c.ba[b].lo[d] - 1;
            hi[d] = c.ba[b].hi[d] + 1;
        }
        for (int a0 = lo[A]; a0 <= hi[A]; a0 += tA)
            for (int b0 = lo[B]; b0 <= hi[B]; b0 += tB) {
                SweepTile t{};
                t.b = b;
                t.lo[D] = lo[D];
                t.n[D] = hi[D] - lo[D] + 1;
                t.lo[A] = a0;
                t.n[A] = std::min(tA, hi[A] - a0 + 1);
                t.lo[B] = b0;
                t.n[B] = std::min(tB, hi[B] - b0 + 1);
                pl.smem = std::max(pl.smem, smem_bytes(D, ppmt, t.n));
                pl.h.push_back(t);
            }
    }
    pl.box_first.push_back((int)pl.h.size());
    if (!cuda_ok(cudaMalloc(&pl.d, pl.h.size() * sizeof(SweepTile)), "cudaMalloc") ||
        !cuda_ok(cudaMemcpy(pl.d, pl.h.data(), pl.h.size() * sizeof(SweepTile), cudaMemcpyHostToDevice),
                 "cudaMemcpy"))
        throw Fail{MADV_ERR_CUDA};
    return &(P[key] = std::move(pl));
}

template <int D, int PPMT, int UMAC>
static void sweep_launch(Ctx& c, const SweepPlan& pl, int fs, int sc, int fu, int uc, int fip, int fim, int lo_ext,
                         int hi_ext) {
    auto kern = k_ppm_sweep<D, PPMT, UMAC>;
    static std::map<const void*, size_t> attr_set;
    size_t& have = attr_set[(const void*)kern];
    if (pl.smem > have) {  // set outside any capture: the dry pass reaches here first
        if (!cuda_ok(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)pl.smem),
                     "cudaFuncSetAttribute"))
            throw Fail{MADV_ERR_CUDA};
        have = pl.smem;
    }
    if (c.dry) return;
    const long long eb = dbits_host(c.P.rel_eps);
    const RecipC r6 = make_recip(6.0);
    const int dlo = c.P.dom_lo[D], dhi = c.P.dom_hi[D];
    auto one = [&](int t0, int t1) {
        if (t1 <= t0) return;
        kern<<<t1 - t0, SWEEP_TPB, pl.smem, c.stream>>>(pl.d, t0, c.V(), c.nb, fs, sc, fu, uc, fip, fim, lo_ext,
                                                        hi_ext, dlo, dhi, eb, r6, c.d_flag);
        c.launches++;
    };
    if (!c.per_box) {
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (c.profiling) {
            e0 = c.next_event();
            e1 = c.next_event();
            cudaEventRecord(e0, c.stream);
        }
        one(0, (int)pl.h.size());
        if (c.profiling) {
            cudaEventRecord(e1, c.stream);
            c.prof.push_back({(const void*)kern, e0, e1});
        }
    } else {
        for (int b = 0; b < c.nb; ++b) one(pl.box_first[b], pl.box_first[b + 1]);
    }
}

// The fused sweep of direction D for component sc of field fs (Ip / Im into comps D of
// fip / fim); false when the caller should use the three-launch form (2-D, or the adjoint
// keeping the interface values on its tape).
bool ppm_sweep(Ctx& c, int D, int fs, int sc, int fu, int uc, int umac, int fip, int fim, int lo_ext, int hi_ext) {
    if (!c.staged_ppm || c.ndim != 3 || c.edge_tape_begin || c.P.ppm_type == 0) return false;
    const int ppmt = c.P.ppm_type;
    const SweepPlan& pl = *sweep_plan(c, D, ppmt);
    static int smem_max = -1;
    if (smem_max < 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
            smem_max = 0;
    }
    if (pl.smem > (size_t)smem_max) return false;  // pencils too long for shared memory
#define MADV_SW(DD, PP, UU) sweep_launch<DD, PP, UU>(c, pl, fs, sc, fu, uc, fip, fim, lo_ext, hi_ext)
#define MADV_SW_D(DD)                     \
    if (ppmt == 1 && umac) MADV_SW(DD, 1, 1); \
    else if (ppmt == 1) MADV_SW(DD, 1, 0);    \
    else if (umac) MADV_SW(DD, 2, 1);         \
    else MADV_SW(DD, 2, 0)
    if (D == 0) {
        MADV_SW_D(0);
    } else if (D == 1) {
        MADV_SW_D(1);
    } else {
        MADV_SW_D(2);
    }
#undef MADV_SW_D
#undef MADV_SW
    return true;
}

}  // namespace madv
