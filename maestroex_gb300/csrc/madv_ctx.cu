// Context, layout, base state and the C ABI of the scalar-advection stage library.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>

#include "madv_ctx.hpp"

namespace madv {

static thread_local std::string g_err;
void set_error(const std::string& s) { g_err = s; }
bool cuda_ok(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return true;
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return false;
}

#define CK(x)                              \
    do {                                   \
        if (!cuda_ok((x), #x)) return MADV_ERR_CUDA; \
    } while (0)


// ------------------------------------------------------------------ region tables
static HBox valid_box(const Ctx& c, int b, int nodal) {
    HBox r = c.ba[b];
    if (nodal >= 0) r.hi[nodal] += 1;
    return r;
}

const RegionTable& region(Ctx& c, int glo0, int glo1, int glo2, int ghi0, int ghi1, int ghi2, int nodal, int slab) {
    if (c.ndim == 2) glo2 = ghi2 = 0;
    std::array<int, 8> key{glo0, glo1, glo2, ghi0, ghi1, ghi2, nodal, slab};
    auto it = c.regions.find(key);
    if (it != c.regions.end()) return it->second;
    RegionTable& t = c.regions[key];
    const int glo[3] = {glo0, glo1, glo2}, ghi[3] = {ghi0, ghi1, ghi2};
    long start = 0;
    auto push = [&](int b, const int lo[3], const int hi[3]) {
        RegionBox r{};
        for (int d = 0; d < 3; ++d) {
            r.lo[d] = lo[d];
            r.n[d] = hi[d] - lo[d] + 1;
        }
        if (r.n[0] <= 0 || r.n[1] <= 0 || r.n[2] <= 0) return;
        r.b = b;
        r.start = start;
        start += (long)r.n[0] * r.n[1] * r.n[2];
        t.h.push_back(r);
    };
    for (int b = 0; b < c.nb; ++b) {
        HBox v = valid_box(c, b, nodal);
        int lo[3], hi[3];
        for (int d = 0; d < 3; ++d) {
            lo[d] = v.lo[d] - glo[d];
            hi[d] = v.hi[d] + ghi[d];
        }
        if (slab < 0) {
            push(b, lo, hi);
        } else {
            const int d = slab;
            if (lo[d] < c.P.dom_lo[d]) {
                int l2[3] = {lo[0], lo[1], lo[2]}, h2[3] = {hi[0], hi[1], hi[2]};
                h2[d] = c.P.dom_lo[d] - 1;
                push(b, l2, h2);
            }
            if (hi[d] > c.P.dom_hi[d]) {
                int l2[3] = {lo[0], lo[1], lo[2]}, h2[3] = {hi[0], hi[1], hi[2]};
                l2[d] = c.P.dom_hi[d] + 1;
                push(b, l2, h2);
            }
        }
    }
    t.total = start;
    if (!t.h.empty()) {
        if (cudaMalloc(&t.d, sizeof(RegionBox) * t.h.size()) != cudaSuccess ||
            cudaMemcpy(t.d, t.h.data(), sizeof(RegionBox) * t.h.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            throw Fail{MADV_ERR_CUDA};
    }
    return t;
}

// a minus b as up to six disjoint boxes appended to out
static void box_minus(const HBox& a, const HBox& b, std::vector<HBox>& out) {
    for (int d = 0; d < 3; ++d)
        if (b.hi[d] < a.lo[d] || b.lo[d] > a.hi[d]) {
            out.push_back(a);
            return;
        }
    HBox rem = a;
    for (int d = 0; d < 3; ++d) {
        if (rem.lo[d] < b.lo[d]) {
            HBox p = rem;
            p.hi[d] = b.lo[d] - 1;
            out.push_back(p);
            rem.lo[d] = b.lo[d];
        }
        if (rem.hi[d] > b.hi[d]) {
            HBox p = rem;
            p.lo[d] = b.hi[d] + 1;
            out.push_back(p);
            rem.hi[d] = b.hi[d];
        }
    }
}

// FillBoundary copy list: every piece of a box's ghost region that lies in another box's
// valid region (after the periodic shift), minus the box's own valid region.  Face data
// can have one ghost face covered by two sources (a face shared by two boxes, or the two
// periodic images of a face); the sources are ordered by (source box, z, y, x shift) and
// the last one wins, as a sequential FillBoundary over that order leaves it.  Destination
// pieces are made disjoint, so the batched copy has no write conflicts.
const CopyTable& copy_table(Ctx& c, int ng, int nodal) {
    std::array<int, 3> key{ng, nodal, 0};
    auto it = c.copies.find(key);
    if (it != c.copies.end()) return it->second;
    CopyTable& t = c.copies[key];
    int len[3];
    for (int d = 0; d < 3; ++d) len[d] = c.P.dom_hi[d] - c.P.dom_lo[d] + 1;
    long start = 0;
    for (int b = 0; b < c.nb; ++b) {
        HBox vb = valid_box(c, b, nodal);
        HBox gb = vb;
        for (int d = 0; d < c.ndim; ++d) {
            gb.lo[d] -= ng;
            gb.hi[d] += ng;
        }
        struct Cand {
            int src;
            int shift[3];
            HBox r;
        };
        std::vector<Cand> cands;
        for (int cbx = 0; cbx < c.nb; ++cbx) {
            HBox sv = valid_box(c, cbx, nodal);
            const int zs = c.ndim == 2 ? 0 : 1;
            for (int sz = -zs; sz <= zs; ++sz)
                for (int sy = -1; sy <= 1; ++sy)
                    for (int sx = -1; sx <= 1; ++sx) {
                        int s[3] = {sx, sy, sz};
                        bool ok = true;
                        for (int d = 0; d < 3; ++d)
                            if (s[d] != 0 && !c.per[d]) ok = false;
                        if (!ok || (cbx == b && sx == 0 && sy == 0 && sz == 0)) continue;
                        HBox r;
                        bool empty = false;
                        for (int d = 0; d < 3; ++d) {
                            r.lo[d] = std::max(gb.lo[d], sv.lo[d] + s[d] * len[d]);
                            r.hi[d] = std::min(gb.hi[d], sv.hi[d] + s[d] * len[d]);
                            if (r.lo[d] > r.hi[d]) empty = true;
                        }
                        if (empty) continue;
                        // without the destination's valid box
                        std::vector<HBox> parts;
                        box_minus(r, vb, parts);
                        for (auto& p : parts) cands.push_back({cbx, {s[0] * len[0], s[1] * len[1], s[2] * len[2]}, p});
                    }
        }
        // last candidate wins: walk backwards, keep what no later candidate claimed
        std::vector<HBox> claimed;
        for (int q = (int)cands.size() - 1; q >= 0; --q) {
            std::vector<HBox> pieces{cands[q].r};
            for (const HBox& cl : claimed) {
                std::vector<HBox> next;
                for (const HBox& p : pieces) box_minus(p, cl, next);
                pieces.swap(next);
                if (pieces.empty()) break;
            }
            for (const HBox& p : pieces) {
                CopyDesc cd{};
                cd.dst_b = b;
                cd.src_b = cands[q].src;
                for (int d = 0; d < 3; ++d) {
                    cd.lo[d] = p.lo[d];
                    cd.n[d] = p.hi[d] - p.lo[d] + 1;
                    cd.shift[d] = cands[q].shift[d];
                }
                cd.start = start;
                start += (long)cd.n[0] * cd.n[1] * cd.n[2];
                t.h.push_back(cd);
            }
            claimed.push_back(cands[q].r);
        }
    }
    t.total = start;
    if (!t.h.empty()) {
        if (cudaMalloc(&t.d, sizeof(CopyDesc) * t.h.size()) != cudaSuccess ||
            cudaMemcpy(t.d, t.h.data(), sizeof(CopyDesc) * t.h.size(), cudaMemcpyHostToDevice) != cudaSuccess)
            throw Fail{MADV_ERR_CUDA};
    }
    return t;
}

// ------------------------------------------------------------------ setup helpers
// Maestro::BCSetup (Source/MaestroSetup.cpp:276-500)
static int bc_setup(Ctx& c) {
    for (int dir = 0; dir < 3; ++dir)
        for (int side = 0; side < 2; ++side) {
            const int pb = side == 0 ? c.P.phys_bc_lo[dir] : c.P.phys_bc_hi[dir];
            int u, un, s, spi, f;
            switch (pb) {
                case PB_INTERIOR: u = un = s = spi = f = BC_INT_DIR; break;
                case PB_INFLOW: u = un = BC_EXT_DIR; s = BC_EXT_DIR; spi = BC_FOEXTRAP; f = BC_FOEXTRAP; break;
                case PB_OUTFLOW: u = un = BC_FOEXTRAP; s = BC_FOEXTRAP; spi = BC_EXT_DIR; f = BC_FOEXTRAP; break;
                case PB_SYMMETRY: u = BC_REFLECT_EVEN; un = BC_REFLECT_ODD; s = spi = f = BC_REFLECT_EVEN; break;
                case PB_SLIPWALL: u = BC_HOEXTRAP; un = BC_EXT_DIR; s = BC_HOEXTRAP; spi = BC_FOEXTRAP; f = BC_FOEXTRAP; break;
                case PB_NOSLIPWALL: u = un = BC_EXT_DIR; s = BC_HOEXTRAP; spi = BC_FOEXTRAP; f = BC_FOEXTRAP; break;
                default: return MADV_ERR_PARAM;
            }
            auto set = [&](BCRecD& r, int v) { (side == 0 ? r.lo : r.hi)[dir] = v; };
            for (int k = 0; k < 3; ++k) set(c.bcs_u[k], k == dir ? un : u);
            for (int k = 0; k < c.nscal; ++k) set(c.bcs_s[k], k == PI ? spi : s);
            for (int k = 0; k < c.nscal; ++k) set(c.bcs_f[k], f);
        }
    return MADV_OK;
}

static FabView make_view(double* p, const int lo[3], const int hi[3]) {
    FabView v{};
    v.p = p;
    v.lo0 = lo[0];
    v.lo1 = lo[1];
    v.lo2 = lo[2];
    const long nx = hi[0] - lo[0] + 1, ny = hi[1] - lo[1] + 1, nz = hi[2] - lo[2] + 1;
    v.sj = (int)nx;
    v.sk = nx * ny;
    v.sn = nx * ny * nz;
    return v;
}

static void field_specs(Ctx& c) {
    auto S = [&](int f, int nc, int ng, int nodal = -1) { c.F[f].spec = FieldSpec{nc, ng, nodal}; };
    S(F_SOLD, c.nscal, c.ng_s);
    S(F_SNEW, c.nscal, c.ng_s);
    S(F_GPI, 3, 0);
    S(F_THERMAL, 1, 1);
    S(F_W0CART, 3, 2);
    S(F_W0FCART, 3, 1);
    S(F_UTILDE, 3, c.ng_adv);
    S(F_UFULL, 3, c.ng_adv);
    for (int d = 0; d < 3; ++d) {
        S(F_UTRANS0 + d, 1, 1, d);
        S(F_UMAC0 + d, 1, 1, d);
        S(F_SEDGE0 + d, c.nscal, 0, d);
        S(F_SFLUX0 + d, c.nscal, 0, d);
        S(F_FACE0 + d, 1, 2, d);
        S(F_IPC0 + d, 3, 1);
        S(F_IMC0 + d, 3, 1);
        S(F_SL0 + d, 3, 1);
        S(F_SR0 + d, 3, 1);
        S(F_SIMH0 + d, 3, 1);
    }
    // the forces carry ng_s ghost cells when they are traced (Source/MaestroAdvance.cpp:150-155,
    // Source/MaestroAdvection.cpp:62-67)
    const int ngf = c.P.ppm_trace_forces ? c.ng_s : 1;
    S(F_VELFORCE, 3, ngf);
    S(F_SCALFORCE, c.nscal, ngf);
    S(F_IPF, c.P.ppm_trace_forces ? 3 : 0, 1);
    S(F_IMF, c.P.ppm_trace_forces ? 3 : 0, 1);
    S(F_ETA, 1, 0, c.ndim - 1);
    S(F_RHO0CART, 1, 1);
    S(F_RHOH0CART, 1, 1);
    S(F_S0ECART, 1, 1);
    S(F_P0CART, 1, 1);
    S(F_PSICART, 1, 1);
    S(F_GRAVCART, 3, 1);
    for (int q = F_Q01; q <= F_Q21; ++q) S(q, 1, 1);
    S(F_DIVU, 1, 1);
    S(F_SLOPE, 3, 1);
    S(F_DSVL, 1, 2);
    for (int d = 0; d < 3; ++d) S(F_TRA0 + d, 2, 1, d);
    S(F_TRC, 6, 1);
    S(F_TCOEF, 6, 1);
    // spherical only (one component each; a planar context allocates them empty)
    const int ns = c.sph ? 1 : 0;
    for (int d = 0; d < 3; ++d) {
        S(F_W0MAC0 + d, ns, 1, d);
        S(F_S0MAC0 + d, ns, 1, d);
        S(F_S0MACB0 + d, ns, 1, d);
    }
    S(F_S0CART2, ns, 2);
    const int nu = c.sph && !c.P.use_exact_base_state ? 1 : 0;  // uniform radial bins only
    for (int d = 0; d < 3; ++d) {
        S(F_S0MACC0 + d, nu, 1, d);
        S(F_S0MACD0 + d, nu, 1, d);
    }
    S(F_GRADW0, nu, 1);
    S(F_DIVW0, nu, 0);
    // nodes of the box grown by one, node (i,j,k) at cell (i,j,k): two ghost cells
    S(F_W0NODAL, c.sph && c.geo.w0maci == 4 ? 3 : 0, 2);
    // species streaming (a stage call that returns no edge states or fluxes): Rho, RhoH and
    // the species in flight, in place of the nscal components of F_SEDGE* / F_SFLUX*
    for (int d = 0; d < 3; ++d) {
        S(F_SEDGES0 + d, c.ndim == 3 ? 3 : 0, 0, d);
        S(F_SFLUXS0 + d, c.ndim == 3 ? 3 : 0, 0, d);
    }
}

static void free_layout(Ctx& c) {
    for (auto& f : c.F)
        if (f.base) {
            cudaFree(f.base);
            f.base = nullptr;
        }
    for (auto& kv : c.regions)
        if (kv.second.d) cudaFree(kv.second.d);
    c.regions.clear();
    for (auto& kv : c.copies)
        if (kv.second.d) cudaFree(kv.second.d);
    c.copies.clear();
    if (c.dviews) cudaFree(c.dviews);
    c.dviews = nullptr;
    if (c.hviews_pinned) cudaFreeHost(c.hviews_pinned);
    c.hviews_pinned = nullptr;
    if (c.dviews_alias) cudaFree(c.dviews_alias);
    c.dviews_alias = nullptr;
    if (c.hviews_alias) cudaFreeHost(c.hviews_alias);
    c.hviews_alias = nullptr;
    if (c.graph_exec) cudaGraphExecDestroy(c.graph_exec);
    c.graph_exec = nullptr;
    c.graph_key.clear();
    for (auto& kv : c.amr_tables)
        if (kv.second.d) cudaFree(kv.second.d);
    c.amr_tables.clear();
    sweep_free(c);
    for (auto& kv : c.side_scratch) cudaFree(kv.second);
    c.side_scratch.clear();
    if (c.dviews_side) cudaFree(c.dviews_side);
    c.dviews_side = nullptr;
    if (c.hviews_side) cudaFreeHost(c.hviews_side);
    c.hviews_side = nullptr;
    c.side_mirror = nullptr;
    if (c.d_owner) cudaFree(c.d_owner);
    c.d_owner = nullptr;
    c.h_owner.clear();
}

// Maestro::CelltoEdge (Source/MaestroCelltoEdge.cpp:17-54) on the edges [lo, hi] of one
// chunk of a level with nr cells.
static void cell_to_edge_chunk(const std::vector<double>& cc, std::vector<double>& e, int lo, int hi) {
    const int nr = (int)cc.size();
    for (int r = lo; r <= hi; ++r) {
        if (r == 0) e[r] = cc[r];
        else if (r == 1 || r == lo) e[r] = 0.5 * (cc[r - 1] + cc[r]);
        else if (r == nr) e[r] = cc[r - 1];
        else if (r == nr - 1 || r == hi) e[r] = 0.5 * (cc[r] + cc[r - 1]);
        else {
            double tmp = 7.0 / 12.0 * (cc[r] + cc[r - 1]) - 1.0 / 12.0 * (cc[r + 1] + cc[r - 2]);
            double lo_ = (cc[r - 1] < cc[r]) ? cc[r - 1] : cc[r];  // min(cc[r], cc[r-1])
            double hi_ = (cc[r] < cc[r - 1]) ? cc[r - 1] : cc[r];  // max(cc[r], cc[r-1])
            double t = (tmp < lo_) ? lo_ : tmp;
            e[r] = (hi_ < t) ? hi_ : t;
        }
    }
}

// ------------------------------------------------------------------ user FAB binding
struct Binding {
    int slot;
    const madv_multifab* mf;
    int ncomp;
    int nodal;
    int ng;  // ghost cells the library reads or writes in the caller's FAB
};

static int bind(Ctx& c, int slot, const madv_multifab* mf, int ncomp, int nodal, int ng) {
    if (!mf) return MADV_OK;
    if (mf->nfab != c.nb || !mf->fab) {
        set_error("MultiFab has " + std::to_string(mf->nfab) + " FABs, layout has " + std::to_string(c.nb));
        return MADV_ERR_LAYOUT;
    }
    for (int b = 0; b < c.nb; ++b) {
        const madv_fab& f = mf->fab[b];
        HBox v = valid_box(c, b, nodal);
        if (!f.p || f.ncomp < ncomp) {
            set_error("FAB " + std::to_string(b) + ": null pointer or too few components");
            return MADV_ERR_LAYOUT;
        }
        for (int d = 0; d < 3; ++d)
            if (f.lo[d] > v.lo[d] - ng || f.hi[d] < v.hi[d] + ng) {
                set_error("FAB " + std::to_string(b) + " does not cover its box grown by " + std::to_string(ng));
                return MADV_ERR_LAYOUT;
            }
        if (((uintptr_t)f.p) % 8 != 0) {
            set_error("FAB pointer not 8-byte aligned");
            return MADV_ERR_LAYOUT;
        }
        c.hviews_pinned[(F_USER + slot) * c.nb + b] = make_view(f.p, f.lo, f.hi);
    }
    return MADV_OK;
}

static int upload_user_views(Ctx& c) {
    const size_t off = (size_t)F_USER * c.nb;
    CK(cudaMemcpyAsync(c.dviews + off, c.hviews_pinned + off, sizeof(FabView) * N_USER_SLOTS * c.nb,
                       cudaMemcpyHostToDevice, c.stream));
    return MADV_OK;
}

enum {
    U_UOLD = 0, U_SOLD, U_GPI, U_THERMAL, U_SNEW, U_UMAC0, U_UMAC1, U_UMAC2, U_SEDGE0, U_SEDGE1, U_SEDGE2,
    U_SFLUX0, U_SFLUX1, U_SFLUX2, U_ETA, U_UTRANS0, U_UTRANS1, U_UTRANS2, U_UFULL, U_FORCE,
    U_RHOHALF, U_SPONGE, U_UEDGE0, U_UEDGE1, U_UEDGE2
};
static_assert(U_UEDGE2 < A_WSOLD, "user slots of the entry points and of the adjoint");

// Ghost width (at most maxg) that every FAB of mf holds around its box
static int held_ghosts(const Ctx& c, const madv_multifab* mf, int nodal, int maxg) {
    int g = maxg;
    for (int b = 0; b < c.nb; ++b) {
        const madv_fab& f = mf->fab[b];
        HBox v = valid_box(c, b, nodal);
        for (int d = 0; d < 3; ++d) g = std::min(g, std::min(v.lo[d] - f.lo[d], f.hi[d] - v.hi[d]));
    }
    return std::max(g, 0);
}

// ------------------------------------------------------------------ level coupling
// Maestro::FillPatch over all levels (Source/MaestroFillData.cpp:7-74): level 0 is filled
// from itself; level l > 0 interpolates its uncovered ghost cells from level l-1 first.
static void fill_patch_h(Hier& H, int fid, int c0, int nc, int which_bcs, int bc_c0, int is_vel, int state_c0) {
    for (int l = 0; l < H.n(); ++l) {
        if (l > 0) interp_fill(H[l - 1], H[l], fid, c0, nc, which_bcs, bc_c0, is_vel, state_c0);
        fill_patch(H[l], fid, c0, nc, which_bcs, bc_c0, is_vel, state_c0);
    }
}
// Maestro::AverageDown (Source/MaestroFillData.cpp:145-154)
static void average_down_h(Hier& H, int fid, int comp, int ncomp) {
    for (int l = H.n() - 2; l >= 0; --l) average_down(H[l + 1], H[l], fid, comp, ncomp);
}
// Maestro::AverageDownFaces (Source/MaestroFillData.cpp:156-174)
static void average_down_faces_h(Hier& H, int f0, int c0, int ncomp) {
    for (int l = H.n() - 2; l >= 0; --l) average_down_faces(H[l + 1], H[l], f0, c0, ncomp);
}
// The face-velocity ghost fill closing MakeUtrans and Addw0 (Source/MaestroMakeUtrans.cpp:631-647,
// Source/MaestroFill3dData.cpp:425-461): one level: FillBoundary + FillUmacGhost;
// several: AverageDownFaces, then FillPatchUedge (Source/MaestroFillData.cpp:455-835).
static void sync_faces_h(Hier& H, int f0) {
    if (H.n() == 1) {
        fill_face_ghosts(H[0], f0);
        return;
    }
    average_down_faces_h(H, f0, 0, 1);
    for (int l = 0; l < H.n(); ++l) {
        if (l > 0) uedge_interface(H[l - 1], H[l], f0);
        fill_face_ghosts(H[l], f0);
    }
}
// Maestro::Put1dArrayOnCart, planar (Source/MaestroFill3dData.cpp:9-36)
static void put1d_h(Hier& H, int fid, const char* s0, int outcomp, int nc, int edge, int which_bcs, int bc_c0,
                    int is_vel, int state_c0) {
    for (auto* c : H.L) {
        set_val(*c, fid, 0.0, 0, nc, c->F[fid].spec.ng);
        put1d(*c, fid, c->b1(s0), outcomp, edge, nc == 3);
    }
    average_down_h(H, fid, 0, nc);
    fill_patch_h(H, fid, 0, nc, which_bcs, bc_c0, is_vel, state_c0);
}
// Maestro::Addw0 (Source/MaestroFill3dData.cpp:357-462)
static void addw0_h(Hier& H, int f0, double mult) {
    for (auto* c : H.L) addw0(*c, f0, mult);
    sync_faces_h(H, f0);
}

// Maestro::MakeS0mac (Source/MaestroFill3dData.cpp:712-1188) into dst0 .. dst0 + 2 over the
// nodal boxes grown by one: s0mac_interp_type 1 puts the array on the cells (two ghosts,
// FillPatch with bcs_f) and averages it to the faces; 2 / 3 (uniform bins) interpolate it at the
// face centres
static void make_s0mac_h(Hier& H, const char* s0, int dst0) {
    if (H[0].geo.s0maci != 1) {
        for (auto* c : H.L) make_s0mac_interp(*c, c->b1(s0), dst0);
        return;
    }
    put1d_h(H, F_S0CART2, s0, 0, 1, 0, BCS_F, 0, 0, -1);
    for (auto* c : H.L) make_s0mac_faces(*c, dst0);
}

// ------------------------------------------------------------------ stage pieces
static void w0_carts(Hier& H) {
    const int nd = H[0].ndim;
    // Put1dArrayOnCart(w0, w0_cart, true, true, bcs_u, 0, 1)  (Source/MaestroAdvance.cpp:326)
    put1d_h(H, F_W0CART, "w0", nd - 1, nd, 1, BCS_U, 0, 1, -1);
    // MakeW0mac (Source/MaestroAdvance.cpp:335-338)
    if (H[0].sph)
        for (auto* c : H.L) make_w0mac(*c);
    // Put1dArrayOnCart(w0_force, w0_force_cart, false, true, bcs_f, 0) (:341), evolve_base_state only
    for (auto* c : H.L) set_val(*c, F_W0FCART, 0.0, 0, 3, 1);
    if (H[0].P.evolve_base_state) put1d_h(H, F_W0FCART, "w0_force", nd - 1, nd, 0, BCS_F, 0, 0, -1);
}

// Maestro::MakeVelForce, planar (Source/MaestroForce.cpp:6-259)
// fe: the face velocity of the utilde force term (utrans in AdvancePremac, umac in
// VelocityAdvance); rho0: the base-state density of the buoyancy
static void make_vel_force_h(Hier& H, int fe = F_UTRANS0, const char* rho0 = "rho0_old") {
    const int nd = H[0].ndim;
    // spherical, uniform bins: dw0/dr on the cells (Source/MaestroForce.cpp:36-52)
    if (H[0].sph && !H[0].geo.exact) put1d_h(H, F_GRADW0, "gradw0", 0, 1, 0, BCS_U, 0, 1, -1);
    put1d_h(H, F_GRAVCART, "grav_cell", nd - 1, nd, 0, BCS_F, 0, 0, -1);
    put1d_h(H, F_RHO0CART, rho0, 0, 1, 0, BCS_S, RHO, 0, RHO);
    for (auto* c : H.L) make_vel_force(*c, fe);
    average_down_h(H, F_VELFORCE, 0, nd);
    fill_patch_h(H, F_VELFORCE, 0, nd, BCS_U, 0, 1, -1);
}

// Maestro::AdvancePremac (Source/MaestroAdvection.cpp:7-84) on the internal fields.
static void advance_premac(Hier& H) {
    const int nga = H[0].ng_adv, nd = H[0].ndim;
    fill_patch_h(H, F_UTILDE, 0, nd, BCS_U, 0, 1, -1);
    for (auto* c : H.L) {
        set_val(*c, F_UFULL, 0.0, 0, 3, nga);
        copy_fab(*c, F_UFULL, 0, F_W0CART, 0, nd, 0);
    }
    fill_patch_h(H, F_UFULL, 0, nd, BCS_U, 0, 1, -1);
    for (auto* c : H.L) {
        add_fab(*c, F_UFULL, F_UTILDE, nd, nga);
        for (int d = 0; d < 3; ++d) set_val(*c, F_UTRANS0 + d, 0.0, 0, 1, 1);
    }
    for (auto* c : H.L) make_utrans(*c);
    sync_faces_h(H, F_UTRANS0);
    make_vel_force_h(H);
    addw0_h(H, F_UTRANS0, 1.0);
    for (auto* c : H.L) vel_pred(*c);
    average_down_faces_h(H, F_UMAC0, 0, 1);
}

// Maestro::ModifyScalForce (Source/MaestroForce.cpp:261-467)
static void modify_scal_force_h(Hier& H, int comp, const char* s0_edge, int s0cart_fid, int fullform) {
    if (!H[0].sph) put1d_h(H, F_S0ECART, s0_edge, 0, 1, 0, BCS_F, 0, 0, -1);  // planar only (:275-277)
    // spherical, uniform bins: div w0 on the cells (:283-305)
    if (H[0].sph && !H[0].geo.exact) put1d_h(H, F_DIVW0, "divw0", 0, 1, 0, BCS_U, 0, 0, -1);
    for (auto* c : H.L) modify_scal_force(*c, comp, s0cart_fid, fullform);
    average_down_h(H, F_SCALFORCE, comp, 1);
    fill_patch_h(H, F_SCALFORCE, comp, 1, BCS_F, 0, 0, comp);
}

// Maestro::MakeRhoHForce (Source/MaestroForce.cpp:469-679): which_step 1 uses rho0_old and
// p0_old, which_step 2 their old/new averages (:493-499)
static void make_rhoh_force_h(Hier& H, int is_prediction, int add_thermal, int which_step) {
    const char* p0n = which_step == 1 ? "p0_old" : "p0_avg";
    put1d_h(H, F_P0CART, p0n, 0, 1, 0, BCS_F, 0, 0, -1);
    if (H[0].sph) make_s0mac_h(H, p0n, F_S0MAC0);  // p0mac (Source/MaestroForce.cpp:526-530)
    put1d_h(H, F_PSICART, "psi", 0, 1, 0, BCS_F, 0, 0, -1);
    put1d_h(H, F_RHO0CART, which_step == 1 ? "rho0_old" : "rho0_avg", 0, 1, 0, BCS_S, RHO, 0, RHO);
    // the planar force's gravity (MakeGravCell); the spherical force does not read it
    if (!H[0].sph) put1d_h(H, F_GRAVCART, "grav_cell", H[0].ndim - 1, H[0].ndim, 0, BCS_F, 0, 0, -1);
    for (auto* c : H.L) make_rhoh_force(*c, is_prediction, add_thermal);
    average_down_h(H, F_SCALFORCE, RHOH, 1);
    fill_patch_h(H, F_SCALFORCE, RHOH, 1, BCS_F, 0, 0, RHOH);
}

// Maestro::PutInPertForm (Source/MaestroConvert.cpp:6-34)
static void put_in_pert_form_h(Hier& H, const char* s0, int comp, int bccomp, int which_bcs, int flag) {
    for (auto* c : H.L) put_in_pert_form(*c, c->b1(s0), comp, flag);
    average_down_h(H, F_SOLD, comp, 1);
    fill_patch_h(H, F_SOLD, comp, 1, which_bcs, bccomp, 0, comp);
}

// Maestro::ConvertRhoXToX (Source/MaestroConvert.cpp:64-91)
static void convert_rhox_to_x_h(Hier& H, int flag) {
    const int ns = H[0].nspec;
    for (auto* c : H.L) convert_rhox_to_x(*c, flag);
    average_down_h(H, F_SOLD, FIRSTSPEC, ns);
    if (flag) fill_patch_h(H, F_SOLD, FIRSTSPEC, ns, BCS_F, 0, 0, FIRSTSPEC);
    else fill_patch_h(H, F_SOLD, FIRSTSPEC, ns, BCS_S, FIRSTSPEC, 0, FIRSTSPEC);
}

// Maestro::UpdateScal (Source/MaestroAdvection.cpp:86-297): the update on every level, then
// the levels' synchronisation
static void update_scal_sync_h(Hier& H, int start_comp);
static void update_scal_h(Hier& H, int start_comp) {
    for (auto* c : H.L) update_scal(*c, start_comp);
    update_scal_sync_h(H, start_comp);
}
static void update_scal_sync_h(Hier& H, int start_comp) {
    // reflux_type 2: the coarse cells next to each finer level take back the flux mismatch,
    // the finest pair first (Source/MaestroAdvection.cpp:258-276)
    if (H[0].P.reflux_type == 2)
        for (int l = H.n() - 2; l >= 0; --l) {
            if (start_comp == RHOH) {
                flux_reg_reflux(H[l + 1], H[l], RHOH, 1);
            } else {
                flux_reg_reflux(H[l + 1], H[l], FIRSTSPEC, H[0].nspec);
                flux_reg_reflux(H[l + 1], H[l], RHO, 1);
            }
        }
    if (start_comp == RHOH) {
        average_down_h(H, F_SNEW, RHOH, 1);
        fill_patch_h(H, F_SNEW, RHOH, 1, BCS_S, RHOH, 0, RHOH);
    } else {
        const int ns = H[0].nspec;
        average_down_h(H, F_SNEW, FIRSTSPEC, ns);
        fill_patch_h(H, F_SNEW, FIRSTSPEC, ns, BCS_S, FIRSTSPEC, 0, FIRSTSPEC);
        average_down_h(H, F_SNEW, RHO, 1);
        fill_patch_h(H, F_SNEW, RHO, 1, BCS_S, RHO, 0, RHO);
    }
}

// the fluxes across levels: reflux_type 1 averages the fine fluxes down onto the coarse faces
// (Source/MaestroMakeFlux.cpp:460-462); reflux_type 2 records the flux mismatch of the
// updated components (and Rho with the species) in the flux registers (:420-456)
// (stream: species streaming, whose flux slots hold Rho and RhoH at their own components)
static void flux_sync_h(Hier& H, int c0, int nc, bool stream = false) {
    if (H[0].P.reflux_type != 2) {
        if (stream) average_down_faces_h(H, F_SFLUX0, c0, nc);
        else average_down_faces_h(H, F_SFLUX0, 0, H[0].nscal);
        return;
    }
    const double dt = H[0].P.dt;
    for (int l = 0; l < H.n(); ++l) {
        if (l + 1 < H.n()) {
            flux_reg_crse_init(H[l + 1], H[l], c0, nc, dt);
            if (c0 == FIRSTSPEC) flux_reg_crse_init(H[l + 1], H[l], RHO, 1, dt);
        }
        if (l > 0) {
            flux_reg_fine_add(H[l], c0, nc, dt);
            if (c0 == FIRSTSPEC) flux_reg_fine_add(H[l], RHO, 1, dt);
        }
    }
}

// one component's flux across the levels, read from F_SFLUX* component `slot` (-1: comp)
static void flux_sync_one_h(Hier& H, int comp, int slot) {
    if (H[0].P.reflux_type != 2) {
        average_down_faces_h(H, F_SFLUX0, slot >= 0 ? slot : comp, 1);
        return;
    }
    const double dt = H[0].P.dt;
    for (int l = 0; l < H.n(); ++l) {
        if (l + 1 < H.n()) flux_reg_crse_init(H[l + 1], H[l], comp, 1, dt, slot);
        if (l > 0) flux_reg_fine_add(H[l], comp, 1, dt, slot);
    }
}

// DensityAdvance with the species streamed: a stage call that returns no edge states and no
// fluxes holds one species' edge states and fluxes at a time (component SLOT of the slot
// fields) instead of all of them.  Each species' values and every sum are those of
// density_advance below, in the same order:
// * the species are independent of each other up to UpdateScal's density sum and
//   negative-species fix, so each runs edge state -> back to rho X -> flux -> coarse-fine
//   flux sync -> update before the next; the Rho flux and etarhoflux, sums over the species
//   in component order, carry over from species to species;
// * the edge state of rho (species_pred_type 1, 3) reads only the density and its force, so
//   it is formed first, while the density is in perturbational form, and the density goes
//   back before the species do (converting X back to rho X reads the full density);
// * the closing pass (density from the species' changes, floor, negative-species fix) and
//   the reflux follow the last species, as in UpdateScal.
static void density_advance_streamed(Hier& H, int which_step) {
    constexpr int SLOT = 2;
    const int spt = H[0].P.species_pred_type;
    const int ns = H[0].nspec, nscal = H[0].nscal;
    for (auto* c : H.L) set_val(*c, F_SCALFORCE, 0.0, 0, nscal, c->F[F_SCALFORCE].spec.ng);
    put1d_h(H, F_RHO0CART, "rho0_old", 0, 1, 0, BCS_S, RHO, 0, RHO);
    addw0_h(H, F_UMAC0, -1.0);
    if (spt == 1) modify_scal_force_h(H, RHO, "rho0_edge_old", F_RHO0CART, 0);
    else if (spt == 3) modify_scal_force_h(H, RHO, "rho0_edge_old", F_RHO0CART, 1);
    addw0_h(H, F_UMAC0, 1.0);
    if (spt == 1 || spt == 3) convert_rhox_to_x_h(H, 1);
    if (spt == 1) put_in_pert_form_h(H, "rho0_old", RHO, 0, BCS_F, 1);
    const int cons = spt == 2;  // the species' form; rho's edge state is advective
    for (auto* c : H.L) edge_scal_setup(*c, cons);
    if (spt == 1 || spt == 3)
        for (auto* c : H.L) make_edge_scal(*c, RHO, 1, BCS_S, 0, 0, 0, -1, false);
    if (spt == 1) put_in_pert_form_h(H, "rho0_old", RHO, RHO, BCS_S, 0);
    const char* r0n = which_step == 1 ? "rho0_old" : "rho0_new";
    const char* r0en = which_step == 1 ? "rho0_edge_old" : "rho0_edge_new";
    if (H[0].sph) {  // rho0 on faces (Source/MaestroDensityAdvance.cpp:167-213)
        make_s0mac_h(H, "rho0_old", F_S0MAC0);
        make_s0mac_h(H, r0n, F_S0MACB0);
    }
    for (int n = 0; n < ns; ++n) {
        const int comp = FIRSTSPEC + n;
        for (auto* c : H.L) make_edge_scal(*c, comp, 1, BCS_S, cons, 1, 0, SLOT, false);  // no force for X / rho X
        if (spt == 2)
            for (auto* c : H.L) sum_species_edge_step(*c, SLOT, n == 0);
        if (spt == 1 || spt == 3) {  // X -> rho X (Maestro::ConvertRhoXToX, flag false)
            for (auto* c : H.L) convert_rhox_to_x(*c, 0, comp, 1);
            average_down_h(H, F_SOLD, comp, 1);
            fill_patch_h(H, F_SOLD, comp, 1, BCS_S, comp, 0, comp);
        }
        for (auto* c : H.L)
            make_rhox_flux(*c, c->b1("rho0_old"), c->b1("rho0_edge_old"), c->b1(r0n), c->b1(r0en), comp, 1, SLOT);
        flux_sync_one_h(H, comp, SLOT);
        for (auto* c : H.L) update_species(*c, comp, SLOT);
    }
    flux_sync_one_h(H, RHO, -1);
    for (auto* c : H.L) set_val(*c, F_SCALFORCE, 0.0, RHO, 1, c->F[F_SCALFORCE].spec.ng);
    for (auto* c : H.L) update_rhox_fix(*c);
    update_scal_sync_h(H, FIRSTSPEC);
}

// Maestro::DensityAdvance (Source/MaestroDensityAdvance.cpp:6-243); which_step 2 passes the
// new base state to the fluxes (:186-219)
static void density_advance(Hier& H, int which_step, bool stream = false) {
    if (stream) return density_advance_streamed(H, which_step);
    const int spt = H[0].P.species_pred_type;
    const int ns = H[0].nspec, nscal = H[0].nscal;
    for (auto* c : H.L) set_val(*c, F_SCALFORCE, 0.0, 0, nscal, c->F[F_SCALFORCE].spec.ng);
    put1d_h(H, F_RHO0CART, "rho0_old", 0, 1, 0, BCS_S, RHO, 0, RHO);
    addw0_h(H, F_UMAC0, -1.0);
    if (spt == 1) modify_scal_force_h(H, RHO, "rho0_edge_old", F_RHO0CART, 0);
    else if (spt == 3) modify_scal_force_h(H, RHO, "rho0_edge_old", F_RHO0CART, 1);
    addw0_h(H, F_UMAC0, 1.0);
    if (spt == 1 || spt == 3) convert_rhox_to_x_h(H, 1);
    if (spt == 1) put_in_pert_form_h(H, "rho0_old", RHO, 0, BCS_F, 1);
    for (auto* c : H.L) make_edge_scal(*c, FIRSTSPEC, ns, BCS_S, spt == 2, 1);  // no force for X / rho X
    if (spt == 1 || spt == 3)
        for (auto* c : H.L) make_edge_scal(*c, RHO, 1, BCS_S, 0, 0);
    else
        for (auto* c : H.L) sum_species_edges(*c);
    if (spt == 1) put_in_pert_form_h(H, "rho0_old", RHO, RHO, BCS_S, 0);
    if (spt == 1 || spt == 3) convert_rhox_to_x_h(H, 0);
    const char* r0n = which_step == 1 ? "rho0_old" : "rho0_new";
    const char* r0en = which_step == 1 ? "rho0_edge_old" : "rho0_edge_new";
    if (H[0].sph) {  // rho0 on faces (Source/MaestroDensityAdvance.cpp:167-213)
        make_s0mac_h(H, "rho0_old", F_S0MAC0);
        make_s0mac_h(H, r0n, F_S0MACB0);
    }
    for (auto* c : H.L) make_rhox_flux(*c, c->b1("rho0_old"), c->b1("rho0_edge_old"), c->b1(r0n), c->b1(r0en));
    flux_sync_h(H, FIRSTSPEC, ns);
    // scal_force.setVal(0) before UpdateScal (Source/MaestroDensityAdvance.cpp:229-231): of
    // the components read from here on, only Rho has been written since the zeroing above
    for (auto* c : H.L) set_val(*c, F_SCALFORCE, 0.0, RHO, 1, c->F[F_SCALFORCE].spec.ng);
    update_scal_h(H, FIRSTSPEC);
}

// Maestro::EnthalpyAdvance (Source/MaestroEnthalpyAdvance.cpp:6-352); which_step 2 averages
// the old and new base state in the fluxes (:234-317) and the final MakeRhoHForce (:336)
// Maestro::ConvertRhoHToH (Source/MaestroConvert.cpp:93-114)
static void convert_rhoh_to_h_h(Hier& H, int flag) {
    for (auto* c : H.L) convert_rhoh_to_h(*c, flag);
    average_down_h(H, F_SOLD, RHOH, 1);
    if (flag) fill_patch_h(H, F_SOLD, RHOH, 1, BCS_F, 0, 0, RHOH);
    else fill_patch_h(H, F_SOLD, RHOH, 1, BCS_S, RHOH, 0, RHOH);
}

// spherical: the face base state of the (rho h) fluxes (Source/MaestroEnthalpyAdvance.cpp:
// 187-220, 251-300): rhoh0 (exact base state), or rho0 and h0 = rhoh0 / rho0 (uniform bins)
static void rhoh_face_base_h(Hier& H, int which_step) {
    const char* rh0n = which_step == 1 ? "rhoh0_old" : "rhoh0_new";
    const char* r0n = which_step == 1 ? "rho0_old" : "rho0_new";
    if (H[0].sph && H[0].geo.exact) {
        make_s0mac_h(H, "rhoh0_old", F_S0MAC0);
        make_s0mac_h(H, rh0n, F_S0MACB0);
    } else if (H[0].sph) {
        make_s0mac_h(H, "rho0_old", F_S0MACC0);
        make_s0mac_h(H, r0n, F_S0MACD0);
        make_s0mac_h(H, "h0_old", F_S0MAC0);
        make_s0mac_h(H, which_step == 1 ? "h0_old" : "h0_new", F_S0MACB0);
    }
}

// the fluxes of (rho h): the base state of the enthalpy (and, for the h prediction, of the
// density) at the old time, with the new one for which_step 2
static void rhoh_flux_h(Hier& H, int which_step) {
    const char* rh0n = which_step == 1 ? "rhoh0_old" : "rhoh0_new";
    const char* rh0en = which_step == 1 ? "rhoh0_edge_old" : "rhoh0_edge_new";
    const char* r0n = which_step == 1 ? "rho0_old" : "rho0_new";
    const char* r0en = which_step == 1 ? "rho0_edge_old" : "rho0_edge_new";
    rhoh_face_base_h(H, which_step);
    for (auto* c : H.L)
        make_rhoh_flux(*c, c->b1("rhoh0_old"), c->b1("rhoh0_edge_old"), c->b1(rh0n), c->b1(rh0en), c->b1("rho0_old"),
                       c->b1("rho0_edge_old"), c->b1(r0n), c->b1(r0en));
}

static void enthalpy_advance(Hier& H, int which_step, bool stream = false) {
    const int ept = H[0].P.enthalpy_pred_type;
    const int nscal = H[0].nscal;
    // predict_h: (rho h) -> h (Source/MaestroEnthalpyAdvance.cpp:40-43)
    if (ept == 2) convert_rhoh_to_h_h(H, 1);
    // scal_force.setVal(0) (Source/MaestroEnthalpyAdvance.cpp:51); the enthalpy half reads RhoH only
    for (auto* c : H.L) set_val(*c, F_SCALFORCE, 0.0, RHOH, 1, c->F[F_SCALFORCE].spec.ng);
    addw0_h(H, F_UMAC0, -1.0);
    make_rhoh_force_h(H, 1, 1, 1);
    if (ept == 1) {
        put1d_h(H, F_RHOH0CART, "rhoh0_old", 0, 1, 0, BCS_S, RHOH, 0, RHOH);
        modify_scal_force_h(H, RHOH, "rhoh0_edge_old", F_RHOH0CART, 0);
    }
    if (ept == 2)  // the force of h: the (rho h) force over rho (:80-88)
        for (auto* c : H.L) h_force(*c);
    addw0_h(H, F_UMAC0, 1.0);
    if (ept == 1) put_in_pert_form_h(H, "rhoh0_old", RHOH, 0, BCS_F, 1);
    for (auto* c : H.L) make_edge_scal(*c, RHOH, 1, BCS_S, ept == 0, 0);
    if (ept == 1) put_in_pert_form_h(H, "rhoh0_old", RHOH, RHOH, BCS_S, 0);
    if (ept == 2) convert_rhoh_to_h_h(H, 0);  // h -> (rho h) (:164-167)
    rhoh_flux_h(H, which_step);
    flux_sync_h(H, RHOH, 1, stream);
    for (auto* c : H.L) set_val(*c, F_SCALFORCE, 0.0, RHOH, 1, c->F[F_SCALFORCE].spec.ng);
    addw0_h(H, F_UMAC0, -1.0);
    make_rhoh_force_h(H, 0, 0, which_step);
    addw0_h(H, F_UMAC0, 1.0);
    update_scal_h(H, RHOH);
}

// The stage's working copies of the caller's sold, snew, umac, sedge and sflux: a call that
// hands over FABs laid out as these fields works in them directly, so their storage is
// allocated at the first call that does not (at 256^3 with NumSpec 13 they are 60% of a
// level's fields).
static bool stream_slot(int f) { return f >= F_SEDGES0 && f <= F_SFLUXS2; }
static bool deferrable(int f) {
    return f == F_SOLD || f == F_SNEW || (f >= F_UMAC0 && f <= F_UMAC2) || (f >= F_SEDGE0 && f <= F_SEDGE2) ||
           (f >= F_SFLUX0 && f <= F_SFLUX2) || stream_slot(f);
}

// host views of field f: one FAB per box (valid box grown by the field's ghost width), laid
// end to end from the field's base
static void field_views(Ctx& c, int f) {
    const FieldSpec& s = c.F[f].spec;
    size_t off = 0;
    for (int b = 0; b < c.nb; ++b) {
        HBox v = valid_box(c, b, s.nodal);
        int lo[3], hi[3];
        size_t n = 1;
        for (int d = 0; d < 3; ++d) {
            lo[d] = v.lo[d] - s.ng;
            hi[d] = v.hi[d] + s.ng;
            n *= (size_t)(hi[d] - lo[d] + 1);
        }
        c.hviews_pinned[f * c.nb + b] = make_view(c.F[f].base + off, lo, hi);
        off += n * s.ncomp;
    }
}

// allocates, zeroes and enters in the base view table a deferred field; on failure the
// field stays deferred with empty views
static void materialize(Ctx& c, int f) {
    Field& F = c.F[f];
    if (!F.deferred) return;
    if (!cuda_ok(cudaMalloc(&F.base, F.bytes), "cudaMalloc(field)")) {
        F.base = nullptr;
        throw Fail{MADV_ERR_CUDA};
    }
    field_views(c, f);
    const size_t v0 = (size_t)f * c.nb;
    if (!cuda_ok(cudaMemset(F.base, 0, F.bytes), "cudaMemset") ||
        !cuda_ok(cudaMemcpy(c.dviews + v0, c.hviews_pinned + v0, sizeof(FabView) * c.nb, cudaMemcpyHostToDevice),
                 "cudaMemcpy(views)") ||
        !cuda_ok(cudaDeviceSynchronize(), "cudaDeviceSynchronize")) {
        cudaFree(F.base);
        F.base = nullptr;
        std::memset(c.hviews_pinned + v0, 0, sizeof(FabView) * c.nb);
        throw Fail{MADV_ERR_CUDA};
    }
    F.deferred = false;
}

// every_field: allocate the deferred fields too (every entry point but the stage, which
// allocates those its caller does not hand over); the streaming slots only the stage uses
static int check_ready_h(const Hier& H, bool every_field = true) {
    for (auto* c : H.L)
        if (!c->have_layout || !c->have_base) {
            set_error("the layout and the base state must be set first");
            return MADV_ERR_STATE;
        }
    if (every_field) try {
            for (auto* c : H.L)
                for (int f = 0; f < NF_INTERNAL; ++f)
                    if (!stream_slot(f)) materialize(*c, f);
        } catch (const Fail& f) {
            return f.code;
        }
    return MADV_OK;
}

struct StageIO {
    const madv_multifab *uold, *sold, *gpi, *thermal, *snew, *umac, *sedge, *sflux, *eta;
    int sold_out = 1;  // copy the converted-and-restored sold back to the caller
    int alias = 0;     // AL_* fields worked in the caller's FABs directly (no copies)
    int stream = 0;    // species streaming: the species' edge states and fluxes pass through slots
};
enum { AL_SOLD = 1, AL_SNEW = 2, AL_UMAC = 4, AL_SEDGE = 8, AL_SFLUX = 16, AL_STREAM = 32 };

// A caller FAB can stand in for field fid when it has the field's index box (valid box grown
// by the field's ghost width) and at least its components: views of both then address the
// same elements.
static bool can_alias(const Ctx& c, int fid, const madv_multifab* mf) {
    if (!mf || mf->nfab != c.nb || !mf->fab) return false;
    const FieldSpec& s = c.F[fid].spec;
    for (int b = 0; b < c.nb; ++b) {
        const madv_fab& f = mf->fab[b];
        if (!f.p || f.ncomp < s.ncomp) return false;
        const HBox v = valid_box(c, b, s.nodal);
        for (int d = 0; d < 3; ++d)
            if (f.lo[d] != v.lo[d] - s.ng || f.hi[d] != v.hi[d] + s.ng) return false;
    }
    return true;
}

// Decide which stage fields work in the caller's FABs (sold and snew, the MAC velocities,
// edge states and fluxes: the largest copies of the stage) and point c.dviews at a table
// with those views replaced.  The caller's FABs must be distinct from each other.
// Returns the table to restore afterwards.
static FabView* alias_fields(Ctx& c, StageIO& io) {
    FabView* base = c.dviews;
    io.alias = 0;
    std::vector<const double*> ptrs;
    auto add = [&](const madv_multifab* m, int n) {
        for (int k = 0; m && k < n; ++k)
            for (int b = 0; b < m[k].nfab; ++b) ptrs.push_back(m[k].fab[b].p);
    };
    add(io.uold, 1), add(io.sold, 1), add(io.gpi, 1), add(io.thermal, 1), add(io.snew, 1), add(io.eta, 1);
    add(io.umac, c.ndim), add(io.sedge, c.ndim), add(io.sflux, c.ndim);
    std::vector<const double*> sorted = ptrs;
    std::sort(sorted.begin(), sorted.end());
    const bool distinct = std::adjacent_find(sorted.begin(), sorted.end()) == sorted.end();
    auto all = [&](int f0, const madv_multifab* m) {
        if (!m) return false;
        for (int d = 0; d < c.ndim; ++d)
            if (!can_alias(c, f0 + d, &m[d])) return false;
        return true;
    };
    if (distinct) {
        if (io.sold_out && can_alias(c, F_SOLD, io.sold)) io.alias |= AL_SOLD;
        if (can_alias(c, F_SNEW, io.snew)) io.alias |= AL_SNEW;
        if (all(F_UMAC0, io.umac)) io.alias |= AL_UMAC;
        if (all(F_SEDGE0, io.sedge)) io.alias |= AL_SEDGE;
        if (all(F_SFLUX0, io.sflux)) io.alias |= AL_SFLUX;
    }
    if (io.stream) io.alias |= AL_STREAM;
    // the fields this call does not work in the caller's FABs need their own storage
    if (!(io.alias & AL_SOLD)) materialize(c, F_SOLD);
    if (!(io.alias & AL_SNEW)) materialize(c, F_SNEW);
    for (int d = 0; d < 3; ++d) {
        const bool in_call = d < c.ndim;
        if (!(in_call && (io.alias & AL_UMAC))) materialize(c, F_UMAC0 + d);
        if (io.alias & AL_STREAM) {
            materialize(c, F_SEDGES0 + d);
            materialize(c, F_SFLUXS0 + d);
            continue;
        }
        if (!(in_call && (io.alias & AL_SEDGE))) materialize(c, F_SEDGE0 + d);
        if (!(in_call && (io.alias & AL_SFLUX))) materialize(c, F_SFLUX0 + d);
    }
    if (!io.alias) return base;
    const size_t nv = (size_t)NF_TOTAL * c.nb;
    if (!c.dviews_alias) {
        if (!cuda_ok(cudaMalloc(&c.dviews_alias, sizeof(FabView) * nv), "cudaMalloc(views)") ||
            !cuda_ok(cudaMallocHost(&c.hviews_alias, sizeof(FabView) * nv), "cudaMallocHost(views)"))
            throw Fail{MADV_ERR_CUDA};
    }
    std::memcpy(c.hviews_alias, c.hviews_pinned, sizeof(FabView) * nv);
    auto swap = [&](int fid, int slot) {
        for (int b = 0; b < c.nb; ++b) c.hviews_alias[fid * c.nb + b] = c.hviews_pinned[(F_USER + slot) * c.nb + b];
    };
    if (io.alias & AL_SOLD) swap(F_SOLD, U_SOLD);
    if (io.alias & AL_SNEW) swap(F_SNEW, U_SNEW);
    for (int d = 0; d < c.ndim; ++d) {
        if (io.alias & AL_UMAC) swap(F_UMAC0 + d, U_UMAC0 + d);
        if (io.alias & AL_SEDGE) swap(F_SEDGE0 + d, U_SEDGE0 + d);
        if (io.alias & AL_SFLUX) swap(F_SFLUX0 + d, U_SFLUX0 + d);
        if (io.alias & AL_STREAM)  // the slots stand in for the edge states and fluxes
            for (int b = 0; b < c.nb; ++b) {
                c.hviews_alias[(F_SEDGE0 + d) * c.nb + b] = c.hviews_pinned[(F_SEDGES0 + d) * c.nb + b];
                c.hviews_alias[(F_SFLUX0 + d) * c.nb + b] = c.hviews_pinned[(F_SFLUXS0 + d) * c.nb + b];
            }
    }
    if (!cuda_ok(cudaMemcpyAsync(c.dviews_alias, c.hviews_alias, sizeof(FabView) * nv, cudaMemcpyHostToDevice, c.stream),
                 "cudaMemcpyAsync(views)"))
        throw Fail{MADV_ERR_CUDA};
    c.dviews = c.dviews_alias;
    return base;
}

// The per-component scratch of MakeEdgeScal (3-D): what one component's chain writes
// before its edge state (PPM, slopes, predictor, transverse states, traced force)
static const int SIDE_SCRATCH[] = {F_DSVL, F_FACE0, F_FACE1, F_FACE2, F_IPC0, F_IMC0, F_SLOPE, F_SL0, F_SL1,
                                   F_SL2,  F_SR0,   F_SR1,   F_SR2,   F_SIMH0, F_SIMH1, F_SIMH2, F_Q01, F_Q02,
                                   F_Q10,  F_Q12,   F_Q20,   F_Q21,   F_IPF,  F_IMF};

// component streams: the side stream's view table, a copy of the current one (c.dviews,
// whose host image is `host`) with the per-component scratch moved to the side's copies
// (allocated and zeroed at first use); uploaded on the level's stream
static void side_views(Ctx& c, const FabView* host) {
    c.side_mirror = nullptr;
    if (!c.comp_streams || c.ndim != 3) return;
    if (!c.side) {
        if (!cuda_ok(cudaStreamCreateWithFlags(&c.side, cudaStreamNonBlocking), "cudaStreamCreate") ||
            !cuda_ok(cudaEventCreateWithFlags(&c.ev_fork, cudaEventDisableTiming), "cudaEventCreate") ||
            !cuda_ok(cudaEventCreateWithFlags(&c.ev_join, cudaEventDisableTiming), "cudaEventCreate"))
            throw Fail{MADV_ERR_CUDA};
    }
    const size_t nv = (size_t)NF_TOTAL * c.nb;
    if (!c.dviews_side) {
        if (!cuda_ok(cudaMalloc(&c.dviews_side, sizeof(FabView) * nv), "cudaMalloc(views)") ||
            !cuda_ok(cudaMallocHost(&c.hviews_side, sizeof(FabView) * nv), "cudaMallocHost(views)"))
            throw Fail{MADV_ERR_CUDA};
    }
    std::memcpy(c.hviews_side, host, sizeof(FabView) * nv);
    for (int f : SIDE_SCRATCH) {
        const Field& F = c.F[f];
        if (!F.base || F.bytes == 0) continue;
        double*& dup = c.side_scratch[f];
        if (!dup) {
            if (!cuda_ok(cudaMalloc(&dup, F.bytes), "cudaMalloc(side scratch)") ||
                !cuda_ok(cudaMemset(dup, 0, F.bytes), "cudaMemset"))
                throw Fail{MADV_ERR_CUDA};
        }
        for (int b = 0; b < c.nb; ++b) {
            FabView& v = c.hviews_side[(size_t)f * c.nb + b];
            v.p = dup + (v.p - F.base);
        }
    }
    if (!cuda_ok(cudaMemcpyAsync(c.dviews_side, c.hviews_side, sizeof(FabView) * nv, cudaMemcpyHostToDevice, c.stream),
                 "cudaMemcpyAsync(views)"))
        throw Fail{MADV_ERR_CUDA};
    c.side_mirror = c.dviews;
}

static int bind_stage(Ctx& c, const StageIO& io) {
    int rc;
    if ((rc = bind(c, U_UOLD, io.uold, c.ndim, -1, 0))) return rc;
    if ((rc = bind(c, U_SOLD, io.sold, c.nscal, -1, 0))) return rc;
    if ((rc = bind(c, U_GPI, io.gpi, c.ndim, -1, 0))) return rc;
    if ((rc = bind(c, U_THERMAL, io.thermal, 1, -1, 0))) return rc;
    if ((rc = bind(c, U_SNEW, io.snew, c.nscal, -1, 0))) return rc;
    for (int d = 0; d < c.ndim; ++d) {
        if (io.umac && (rc = bind(c, U_UMAC0 + d, &io.umac[d], 1, d, 0))) return rc;
        if (io.sedge && (rc = bind(c, U_SEDGE0 + d, &io.sedge[d], c.nscal, d, 0))) return rc;
        if (io.sflux && (rc = bind(c, U_SFLUX0 + d, &io.sflux[d], c.nscal, d, 0))) return rc;
    }
    if ((rc = bind(c, U_ETA, io.eta, 1, c.ndim - 1, 0))) return rc;
    return upload_user_views(c);
}

// The whole stage on the internal fields of every level, inputs already bound to the user
// slots (io[l] for level l).
static void stage_body(Hier& H, const std::vector<StageIO>& io) {
    for (int l = 0; l < H.n(); ++l) {
        Ctx& c = H[l];
        if (!c.dry) cudaMemsetAsync(c.d_flag, 0, sizeof(int), c.stream);
        set_val(c, F_UTILDE, 0.0, 0, 3, c.ng_adv);
        copy_fab(c, F_UTILDE, 0, F_USER + U_UOLD, 0, c.ndim, 0);
        if (!(io[l].alias & AL_SOLD)) copy_fab(c, F_SOLD, 0, F_USER + U_SOLD, 0, c.nscal, 0);
    }
    fill_patch_h(H, F_SOLD, 0, H[0].nscal, BCS_S, 0, 0, 0);
    for (int l = 0; l < H.n(); ++l) {
        Ctx& c = H[l];
        if (io[l].gpi) copy_fab(c, F_GPI, 0, F_USER + U_GPI, 0, c.ndim, 0);
        else set_val(c, F_GPI, 0.0, 0, 3, 0);
        set_val(c, F_THERMAL, 0.0, 0, 1, 1);
        if (io[l].thermal) copy_fab(c, F_THERMAL, 0, F_USER + U_THERMAL, 0, 1, 0);
        const int al = io[l].alias;
        if (!(al & AL_SNEW)) set_val(c, F_SNEW, 0.0, 0, c.nscal, c.ng_s);
        for (int d = 0; d < 3; ++d) {
            set_val(c, F_UMAC0 + d, 0.0, 0, 1, 1);
            if (al & AL_STREAM) {  // the three slots
                set_val(c, F_SEDGE0 + d, 0.0, 0, 3, 0);
                set_val(c, F_SFLUX0 + d, 0.0, 0, 3, 0);
                continue;
            }
            // (Source/MaestroAdvance.cpp:190-191); in a caller's FAB only Temp and Pi are not
            // overwritten by the stage
            if (al & AL_SEDGE) set_val(c, F_SEDGE0 + d, 0.0, TEMP, 2, 0);
            else set_val(c, F_SEDGE0 + d, 0.0, 0, c.nscal, 0);
            if (al & AL_SFLUX) set_val(c, F_SFLUX0 + d, 0.0, TEMP, 2, 0);
            else set_val(c, F_SFLUX0 + d, 0.0, 0, c.nscal, 0);
        }
        set_val(c, F_ETA, 0.0, 0, 1, 0);
    }
    w0_carts(H);
    // STEP 3 and STEP 4 of Maestro::AdvanceTimeStep (Source/MaestroAdvance.cpp:359-548)
    const bool stream = io[0].stream;
    advance_premac(H);
    addw0_h(H, F_UMAC0, 1.0);
    density_advance(H, 1, stream);
    addw0_h(H, F_UMAC0, -1.0);
    addw0_h(H, F_UMAC0, 1.0);
    enthalpy_advance(H, 1, stream);
    addw0_h(H, F_UMAC0, -1.0);
    // outputs (valid region)
    for (int l = 0; l < H.n(); ++l) {
        Ctx& c = H[l];
        const int al = io[l].alias;
        if (io[l].snew && !(al & AL_SNEW)) {
            copy_fab(c, F_USER + U_SNEW, RHO, F_SNEW, RHO, 2, 0);
            copy_fab(c, F_USER + U_SNEW, FIRSTSPEC, F_SNEW, FIRSTSPEC, c.nspec, 0);
        }
        if (io[l].sold_out && !(al & AL_SOLD)) copy_fab(c, F_USER + U_SOLD, 0, F_SOLD, 0, c.nscal, 0);
        for (int d = 0; d < c.ndim; ++d) {
            if (io[l].umac && !(al & AL_UMAC)) copy_fab(c, F_USER + U_UMAC0 + d, 0, F_UMAC0 + d, 0, 1, 0);
            if (io[l].sedge && !(al & AL_SEDGE)) copy_fab(c, F_USER + U_SEDGE0 + d, 0, F_SEDGE0 + d, 0, c.nscal, 0);
            if (io[l].sflux && !(al & AL_SFLUX)) copy_fab(c, F_USER + U_SFLUX0 + d, 0, F_SFLUX0 + d, 0, c.nscal, 0);
        }
        if (io[l].eta) copy_fab(c, F_USER + U_ETA, 0, F_ETA, 0, 1, 0);
    }
}

static int finish(Hier& H) {
    std::vector<int> flags(H.n(), 0);
    for (int l = 0; l < H.n(); ++l)
        CK(cudaMemcpyAsync(&flags[l], H[l].d_flag, sizeof(int), cudaMemcpyDeviceToHost, H[0].stream));
    CK(cudaStreamSynchronize(H[0].stream));
    CK(cudaGetLastError());
    for (int f : flags) {
        if (f & 1) {
            set_error("UpdateScal: a cell reached base_cutoff_density; the EOS reset is not implemented");
            return MADV_ERR_EOS;
        }
        if (f & 6) {
            set_error("coarse-fine fill: a coarse cell or face was not available (levels not properly nested)");
            return MADV_ERR_LAYOUT;
        }
        if (f & 8) {
            set_error("staged PPM sweep: a shared-memory staging copy did not complete in time");
            return MADV_ERR_CUDA;
        }
    }
    return MADV_OK;
}

static void set_mode(Hier& H, cudaStream_t st, int per_box, bool dry) {
    for (auto* c : H.L) {
        c->stream = st;
        c->per_box = per_box;
        c->dry = dry;
    }
}
static long total_launches(const Hier& H) {
    long n = 0;
    for (auto* c : H.L) n += c->launches;
    return n;
}
static void reset_launches(Hier& H) {
    for (auto* c : H.L) c->launches = 0;
}

}  // namespace madv

using namespace madv;

// Threads per block for kernel fn on this level: the autotuner's trial value while it times
// a candidate, else the chosen value (a loaded table is matched by name at the kernel's first
// launch), else 256; never more than the kernel can take.
int Ctx::tpb_of(const void* fn) {
    auto mx = tpb_max.find(fn);
    int maxt;
    if (mx == tpb_max.end()) {
        cudaFuncAttributes a{};
        maxt = (cudaFuncGetAttributes(&a, fn) == cudaSuccess && a.maxThreadsPerBlock > 0) ? a.maxThreadsPerBlock : 256;
        maxt = maxt / 32 * 32;
        tpb_max[fn] = maxt;
        if (!tpb_by_name.empty()) {
            const char* nm = nullptr;
            if (cudaFuncGetName(&nm, fn) == cudaSuccess && nm) {
                auto it = tpb_by_name.find("L" + std::to_string(lev) + " " + nm);
                if (it != tpb_by_name.end()) tpb_choice[fn] = it->second;
            }
        }
    } else {
        maxt = mx->second;
    }
    int t = tpb_trial;
    if (!t) {
        auto it = tpb_choice.find(fn);
        t = it == tpb_choice.end() ? 256 : it->second;
    }
    return t > maxt ? maxt : t;
}

cudaEvent_t Ctx::next_event() {
    if (ev_next == ev_pool.size()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        ev_pool.push_back(e);
    }
    return ev_pool[ev_next++];
}

struct madv_ctx {
    Ctx c;                                   // level 0
    std::vector<std::unique_ptr<Ctx>> fine;  // levels 1, 2, ...
    Hier H() {
        Hier h;
        h.L.push_back(&c);
        for (auto& f : fine) h.L.push_back(f.get());
        return h;
    }
};

// The spherical radial grid from the finest level (Source/MaestroSetup.cpp:60-96): its cell
// size dxf and x extent nfine cells; dr_fine = dxf / drdxfac; nr_fine = nr_irreg + 1 for the
// exact base state, else int(max_dist / dr_fine) + 1 with max_dist the centre-to-corner distance
static void sph_radial_grid(Ctx& c, double dxf, int nfine) {
    c.geo.dxf = dxf;
    c.geo.drf = dxf / (c.P.drdxfac > 0 ? c.P.drdxfac : 1);
    if (c.geo.exact) {
        const double domhi = nfine;
        c.nr = int((3.0 * (domhi / 2 - 0.5) * (domhi / 2 - 0.5) - 0.75) / 2.0) + 1;
    } else {
        const double lenx = 0.5 * (c.P.prob_hi[0] - c.P.prob_lo[0]);
        const double leny = 0.5 * (c.P.prob_hi[1] - c.P.prob_lo[1]);
        const double lenz = 0.5 * (c.P.prob_hi[2] - c.P.prob_lo[2]);
        const double max_dist = std::sqrt(lenx * lenx + leny * leny + lenz * lenz);
        c.nr = int(max_dist / c.geo.drf) + 1;
    }
    c.geo.nr = c.nr;
}

static int init_level(Ctx& c, const madv_params& p, int lev) {
    c.P = p;
    c.lev = lev;
    const int r = 1 << lev;
    for (int d = 0; d < 3; ++d) {
        c.P.dx[d] = p.dx[d] / r;
        c.P.dom_lo[d] = p.dom_lo[d] * r;
        c.P.dom_hi[d] = (p.dom_hi[d] + 1) * r - 1;
    }
    c.ndim = p.dim == 2 ? 2 : 3;
    if (c.ndim == 2) {
        c.P.dom_lo[2] = c.P.dom_hi[2] = 0;
        c.P.phys_bc_lo[2] = c.P.phys_bc_hi[2] = PB_INTERIOR;
    }
    c.nspec = p.nspec;
    c.nscal = 4 + p.nspec;
    c.ng_s = c.ng_adv = p.ppm_type == 2 ? 4 : 3;
    c.nr = c.P.dom_hi[c.ndim - 1] - c.P.dom_lo[c.ndim - 1] + 1;
    c.sph = p.spherical != 0;
    if (c.sph) {
        for (int d = 0; d < 3; ++d) {
            c.geo.plo[d] = p.prob_lo[d];
            c.geo.dx[d] = c.P.dx[d];
            c.geo.ctr[d] = 0.5 * (p.prob_lo[d] + p.prob_hi[d]);
        }
        c.geo.exact = p.use_exact_base_state != 0;
        c.geo.w0i = p.w0_interp_type ? p.w0_interp_type : 2;
        c.geo.w0maci = p.w0mac_interp_type ? p.w0mac_interp_type : 1;
        c.geo.s0i = p.s0_interp_type ? p.s0_interp_type : 3;
        c.geo.s0maci = p.s0mac_interp_type ? p.s0mac_interp_type : 1;
        sph_radial_grid(c, c.P.dx[0], c.P.dom_hi[0] - c.P.dom_lo[0] + 1);  // set again with the layout's levels
    }
    for (int d = 0; d < 3; ++d) c.per[d] = c.P.phys_bc_lo[d] == PB_INTERIOR;
    int rc = bc_setup(c);
    if (rc) return rc;
    BCRecD all[2 * MAX_SCAL + 3];
    for (int k = 0; k < c.nscal; ++k) all[k] = c.bcs_s[k];
    for (int k = 0; k < 3; ++k) all[c.nscal + k] = c.bcs_u[k];
    for (int k = 0; k < c.nscal; ++k) all[c.nscal + 3 + k] = c.bcs_f[k];
    if (!cuda_ok(cudaMalloc(&c.d_bcs, sizeof(BCRecD) * (2 * c.nscal + 3)), "cudaMalloc") ||
        !cuda_ok(cudaMemcpy(c.d_bcs, all, sizeof(BCRecD) * (2 * c.nscal + 3), cudaMemcpyHostToDevice), "cudaMemcpy") ||
        !cuda_ok(cudaMalloc(&c.d_flag, sizeof(int)), "cudaMalloc"))
        return MADV_ERR_CUDA;
    field_specs(c);
    return MADV_OK;
}

static void destroy_level(Ctx& c) {
    free_layout(c);
    for (auto& kv : c.d1) cudaFree(kv.second);
    c.d1.clear();
    for (auto e : c.ev_pool) cudaEventDestroy(e);
    c.ev_pool.clear();
    if (c.side) cudaStreamDestroy(c.side);
    if (c.ev_fork) cudaEventDestroy(c.ev_fork);
    if (c.ev_join) cudaEventDestroy(c.ev_join);
    c.side = nullptr;
    c.ev_fork = c.ev_join = nullptr;
    if (c.box_scratch) cudaFree(c.box_scratch);
    c.box_scratch = nullptr;
    if (c.d_bcs) cudaFree(c.d_bcs);
    c.d_bcs = nullptr;
    if (c.d_flag) cudaFree(c.d_flag);
    if (c.d_red) cudaFree(c.d_red);
    c.d_red = nullptr;
    if (c.d_reg) cudaFree(c.d_reg);
    mac_free(c);
    c.d_reg = nullptr;
    c.d_flag = nullptr;
}

// Layout of one level: field allocations and views.  Level 0 must cover the domain; finer
// levels must be coarse-aligned (even lo, odd hi) and lie inside their domain.
static int layout_level(Ctx& c, int nboxes, const madv_box* boxes, bool cover) {
    free_layout(c);
    c.have_layout = false;
    c.ba.assign(nboxes, HBox{});
    long vol = 0;
    for (int b = 0; b < nboxes; ++b) {
        for (int d = 0; d < 3; ++d) {
            c.ba[b].lo[d] = boxes[b].lo[d];
            c.ba[b].hi[d] = boxes[b].hi[d];
            if (boxes[b].lo[d] > boxes[b].hi[d] || boxes[b].lo[d] < c.P.dom_lo[d] || boxes[b].hi[d] > c.P.dom_hi[d]) {
                set_error("level " + std::to_string(c.lev) + " box " + std::to_string(b) +
                          " is empty or outside the domain");
                return MADV_ERR_LAYOUT;
            }
            if (c.lev > 0 && (((boxes[b].lo[d] & 1) != 0) || ((boxes[b].hi[d] & 1) != 1))) {
                set_error("level " + std::to_string(c.lev) + " box " + std::to_string(b) +
                          " is not aligned with the coarser level (even lo, odd hi)");
                return MADV_ERR_LAYOUT;
            }
        }
        vol += (long)(boxes[b].hi[0] - boxes[b].lo[0] + 1) * (boxes[b].hi[1] - boxes[b].lo[1] + 1) *
               (boxes[b].hi[2] - boxes[b].lo[2] + 1);
    }
    for (int a = 0; a < nboxes; ++a)
        for (int b = a + 1; b < nboxes; ++b) {
            bool ov = true;
            for (int d = 0; d < 3; ++d)
                if (c.ba[a].hi[d] < c.ba[b].lo[d] || c.ba[b].hi[d] < c.ba[a].lo[d]) ov = false;
            if (ov) {
                set_error("boxes " + std::to_string(a) + " and " + std::to_string(b) + " overlap");
                return MADV_ERR_LAYOUT;
            }
        }
    long dvol = 1;
    for (int d = 0; d < 3; ++d) dvol *= (c.P.dom_hi[d] - c.P.dom_lo[d] + 1);
    if (cover && vol != dvol) {
        set_error("level 0 must cover the domain");
        return MADV_ERR_LAYOUT;
    }
    c.nb = nboxes;
    try {
        for (int f = 0; f < NF_INTERNAL; ++f) {
            const FieldSpec& s = c.F[f].spec;
            size_t tot = 0;
            for (int b = 0; b < c.nb; ++b) {
                HBox v = valid_box(c, b, s.nodal);
                size_t n = 1;
                for (int d = 0; d < 3; ++d) n *= (size_t)(v.hi[d] - v.lo[d] + 1 + 2 * s.ng);
                tot += n * s.ncomp;
            }
            c.F[f].bytes = tot * sizeof(double);
            c.F[f].deferred = false;
            if (tot == 0) continue;  // a field this context does not use
            if (deferrable(f)) {
                c.F[f].deferred = true;
                continue;
            }
            if (!cuda_ok(cudaMalloc(&c.F[f].base, c.F[f].bytes), "cudaMalloc(field)")) throw Fail{MADV_ERR_CUDA};
            if (!cuda_ok(cudaMemset(c.F[f].base, 0, c.F[f].bytes), "cudaMemset")) throw Fail{MADV_ERR_CUDA};
        }
        if (!cuda_ok(cudaMallocHost(&c.hviews_pinned, sizeof(FabView) * NF_TOTAL * c.nb), "cudaMallocHost"))
            throw Fail{MADV_ERR_CUDA};
        std::memset(c.hviews_pinned, 0, sizeof(FabView) * NF_TOTAL * c.nb);
        for (int f = 0; f < NF_INTERNAL; ++f)
            if (!c.F[f].deferred) field_views(c, f);
        if (!cuda_ok(cudaMalloc(&c.dviews, sizeof(FabView) * NF_TOTAL * c.nb), "cudaMalloc(views)") ||
            !cuda_ok(cudaMemcpy(c.dviews, c.hviews_pinned, sizeof(FabView) * NF_TOTAL * c.nb, cudaMemcpyHostToDevice),
                     "cudaMemcpy(views)"))
            throw Fail{MADV_ERR_CUDA};
    } catch (const Fail& f) {
        free_layout(c);
        return f.code;
    }
    c.have_layout = true;
    return MADV_OK;
}

static void drop_graph(madv_ctx* h) {
    if (h->c.graph_exec) cudaGraphExecDestroy(h->c.graph_exec);
    h->c.graph_exec = nullptr;
    h->c.graph_key.clear();
}

// ------------------------------------------------------------------ adjoint driver
// Device storage of the reverse sweep, freed when the call returns.
struct AdjWork {
    std::vector<double*> owned;
    size_t bytes = 0;
    ~AdjWork() {
        for (auto p : owned) cudaFree(p);
    }
    double* alloc(size_t b) {
        double* p = nullptr;
        if (!cuda_ok(cudaMalloc(&p, b), "cudaMalloc(adjoint)")) throw Fail{MADV_ERR_CUDA};
        if (!cuda_ok(cudaMemset(p, 0, b), "cudaMemset(adjoint)")) throw Fail{MADV_ERR_CUDA};
        owned.push_back(p);
        bytes += b;
        return p;
    }
};

// doubles of one FAB per box (nc components, ng ghost cells, nodal direction or -1)
static size_t fab_doubles(const Ctx& c, int nc, int ng, int nodal) {
    size_t tot = 0;
    for (int b = 0; b < c.nb; ++b) {
        HBox v = valid_box(c, b, nodal);
        size_t n = 1;
        for (int d = 0; d < 3; ++d) n *= (size_t)(v.hi[d] - v.lo[d] + 1 + 2 * ng);
        tot += n * nc;
    }
    return tot;
}

// user slot `slot` over FABs laid end to end at p; fabs (optional) receives the
// madv_fab descriptors of the same storage
static void bind_raw(Ctx& c, int slot, double* p, int nc, int ng, int nodal, std::vector<madv_fab>* fabs = nullptr) {
    size_t off = 0;
    if (fabs) fabs->resize(c.nb);
    for (int b = 0; b < c.nb; ++b) {
        HBox v = valid_box(c, b, nodal);
        int lo[3], hi[3];
        size_t n = 1;
        for (int d = 0; d < 3; ++d) {
            lo[d] = v.lo[d] - ng;
            hi[d] = v.hi[d] + ng;
            n *= (size_t)(hi[d] - lo[d] + 1);
        }
        c.hviews_pinned[(F_USER + slot) * c.nb + b] = make_view(p + off, lo, hi);
        if (fabs) {
            madv_fab& f = (*fabs)[b];
            f.p = p + off;
            for (int d = 0; d < 3; ++d) {
                f.lo[d] = lo[d];
                f.hi[d] = hi[d];
            }
            f.ncomp = nc;
        }
        off += n * nc;
    }
}

extern "C" {

const char* madv_last_error(void) { return g_err.c_str(); }
const char* madv_version(void) { return "maestro_adv 0.2 (sm_103a, FP64, 1-2 AMR levels)"; }

int madv_ctx_create(const madv_params* p, madv_ctx** out) {
    if (!p || !out) return MADV_ERR_PARAM;
    *out = nullptr;
    if (p->nspec < 1 || p->nspec + 4 > MAX_SCAL) {
        set_error("nspec out of range");
        return MADV_ERR_PARAM;
    }
    if (p->ppm_type < 0 || p->ppm_type > 2 || !(p->slope_order == 0 || p->slope_order == 2 || p->slope_order == 4)) {
        set_error("ppm_type must be 0..2 and slope_order 0, 2 or 4");
        return MADV_ERR_PARAM;
    }
    if (p->species_pred_type < 1 || p->species_pred_type > 3 || p->enthalpy_pred_type < 0 ||
        p->enthalpy_pred_type > 2) {
        set_error("species_pred_type must be 1..3, enthalpy_pred_type 0, 1 or 2 (3-6 predict the temperature "
                  "and need the equation of state)");
        return MADV_ERR_UNSUPPORTED;
    }
    if (p->spherical && (p->w0_interp_type < 0 || p->w0_interp_type > 3 || p->w0mac_interp_type < 0 ||
                         p->w0mac_interp_type > 4 || p->s0_interp_type < 0 || p->s0_interp_type > 3 ||
                         p->s0mac_interp_type < 0 || p->s0mac_interp_type > 3 || p->drdxfac < 0)) {
        set_error("spherical: w0_interp_type 1-3, w0mac_interp_type 1-4, s0_interp_type 1-3, s0mac_interp_type 1-3, "
                  "drdxfac >= 1 (0: the default)");
        return MADV_ERR_PARAM;
    }
    if (p->spherical && p->use_exact_base_state && p->s0mac_interp_type > 1) {
        set_error("spherical with the exact base state: s0mac_interp_type 1 (the reference's types 2 and 3 index the "
                  "irregular radial grid with the uniform-grid formula and read past its end)");
        return MADV_ERR_UNSUPPORTED;
    }
    if (p->spherical && (p->dim == 2 || (p->use_exact_base_state && p->enthalpy_pred_type != 1))) {
        set_error("spherical geometry needs 3-D, and enthalpy_pred_type 1 with the exact base state (the reference "
                  "supports neither (rho h) nor h there, Source/MaestroMakeFlux.cpp:791-796)");
        return MADV_ERR_UNSUPPORTED;
    }
    if ((p->ppm_trace_forces != 0 && (p->ppm_trace_forces != 1 || p->ppm_type == 0 || p->dim == 2)) ||
        (p->use_exact_base_state != 0 && !p->spherical)) {
        set_error("ppm_trace_forces = 1 needs ppm_type 1 or 2 in 3-D (with ppm_type 0 the reference reads forces it "
                  "never traced; its 2-D VelPred reads force traces it never writes); use_exact_base_state needs "
                  "spherical geometry");
        return MADV_ERR_UNSUPPORTED;
    }
    if (p->reflux_type < 0 || p->reflux_type > 2 || (p->reflux_type == 2 && p->dim == 2)) {
        set_error("reflux_type must be 1 (or 0) or 2; 2 is built for 3-D");
        return MADV_ERR_UNSUPPORTED;
    }
    if (!(p->dt > 0.0) || !(p->rel_eps >= 0.0)) {
        set_error("dt must be > 0 and rel_eps >= 0");
        return MADV_ERR_PARAM;
    }
    const int nd = p->dim == 2 ? 2 : 3;
    if (p->dim != 0 && p->dim != 2 && p->dim != 3) {
        set_error("dim must be 2 or 3");
        return MADV_ERR_PARAM;
    }
    if (nd == 2 && (p->dom_lo[2] != 0 || p->dom_hi[2] != 0)) {
        set_error("a 2-D domain has z = [0, 0]");
        return MADV_ERR_PARAM;
    }
    for (int d = 0; d < nd; ++d) {
        const int lo = p->phys_bc_lo[d], hi = p->phys_bc_hi[d];
        if (lo < 0 || lo > 5 || hi < 0 || hi > 5) {
            set_error("invalid phys_bc");
            return MADV_ERR_PARAM;
        }
        if ((lo == PB_INTERIOR) != (hi == PB_INTERIOR)) {
            set_error("a periodic direction needs interior on both sides");
            return MADV_ERR_PARAM;
        }
        if (lo == PB_INFLOW || hi == PB_INFLOW) {
            set_error("inflow needs problem-specific Dirichlet data for the scalars");
            return MADV_ERR_UNSUPPORTED;
        }
        if (!(p->dx[d] > 0.0)) {
            set_error("dx must be > 0");
            return MADV_ERR_PARAM;
        }
        const int n = p->dom_hi[d] - p->dom_lo[d] + 1;
        if (n < 8) {
            set_error("each domain extent must be at least 8 cells");
            return MADV_ERR_PARAM;
        }
    }
    if (p->dom_lo[nd - 1] != 0) {
        set_error("the radial domain (z, or y in 2-D) must start at 0");
        return MADV_ERR_PARAM;
    }
    madv_ctx* h = new madv_ctx();
    int rc = init_level(h->c, *p, 0);
    if (rc) {
        destroy_level(h->c);
        delete h;
        return rc;
    }
    *out = h;
    return MADV_OK;
}

void madv_ctx_destroy(madv_ctx* h) {
    if (!h) return;
    for (auto& f : h->fine) destroy_level(*f);
    destroy_level(h->c);
    delete h;
}

int madv_set_dt(madv_ctx* h, double dt, double rel_eps) {
    if (!h || !(dt > 0.0) || !(rel_eps >= 0.0)) return MADV_ERR_PARAM;
    Hier H = h->H();
    for (auto* c : H.L) {
        c->P.dt = dt;
        c->P.rel_eps = rel_eps;
    }
    drop_graph(h);
    return MADV_OK;
}

int madv_set_layout_levels(madv_ctx* h, int nlev, const int* nboxes, const madv_box* boxes) {
    if (!h || nlev < 1 || !nboxes || !boxes) return MADV_ERR_PARAM;
    if (nlev > 2 || (nlev > 1 && h->c.ndim == 2)) {
        set_error("at most two levels (refinement ratio 2), one in 2-D");
        return MADV_ERR_UNSUPPORTED;
    }
    for (auto& f : h->fine) destroy_level(*f);
    h->fine.clear();
    drop_graph(h);
    for (int l = 1; l < nlev; ++l) {
        h->fine.emplace_back(new Ctx());
        int rc = init_level(*h->fine.back(), h->c.P, l);
        if (rc) return rc;
    }
    Hier H = h->H();
    if (h->c.sph) {
        // one radial grid for every level, set by the finest level's cell size
        // (Source/MaestroSetup.cpp:60-96, Source/BaseStateGeometry.cpp:86-104)
        const Ctx& fl = H[nlev - 1];
        for (auto* c : H.L) {
            sph_radial_grid(*c, fl.P.dx[0], fl.P.dom_hi[0] - fl.P.dom_lo[0] + 1);
            c->have_base = false;
        }
    }
    int off = 0;
    for (int l = 0; l < nlev; ++l) {
        if (nboxes[l] <= 0) {
            set_error("every level needs at least one box");
            return MADV_ERR_LAYOUT;
        }
        int rc = layout_level(H[l], nboxes[l], boxes + off, l == 0);
        if (rc) return rc;
        off += nboxes[l];
        if (nlev > 1 && (rc = build_owner(H[l]))) return rc;
        if (nlev > 1) H[l].have_base = false;  // radial chunks depend on the layout
    }
    return MADV_OK;
}

int madv_set_layout(madv_ctx* h, int nboxes, const madv_box* boxes) {
    if (!h || nboxes <= 0 || !boxes) return MADV_ERR_PARAM;
    return madv_set_layout_levels(h, 1, &nboxes, boxes);
}

int madv_set_base_state_levels(madv_ctx* h, int nlev, const madv_base_state* bsl) {
    if (!h || !bsl) return MADV_ERR_PARAM;
    Hier H = h->H();
    if (nlev != H.n()) {
        set_error("the base state needs one entry per level of the layout");
        return MADV_ERR_PARAM;
    }
    for (int l = 0; l < nlev; ++l)
        if (!H[l].have_layout && nlev > 1) {
            set_error("madv_set_layout_levels must come first");
            return MADV_ERR_STATE;
        }
    // radial chunks per level (BaseStateGeometry::InitMultiLevel, planar, Source/BaseStateGeometry.cpp:355-382):
    // rows of level l-1 lying under a level-l box are tagged; each run of tagged rows r0..r1
    // is the level-l chunk [2 r0, 2 r1 + 1].  Spherical: one radial level (max_radial_level 0,
    // Source/MaestroSetup.cpp:65) that every level reads whole, so one chunk of all nr bins
    const bool sph = H[0].sph;
    H[0].chunks.assign(1, {0, H[0].nr - 1});
    for (int l = 1; l < nlev; ++l) {
        if (sph) {
            H[l].chunks.assign(1, {0, H[l].nr - 1});
            continue;
        }
        const int nrc = H[l - 1].nr;
        std::vector<int> tag(nrc, 0);
        for (auto& b : H[l].ba)
            for (int r = b.lo[2]; r <= b.hi[2]; ++r) tag[r / 2] = 1;
        auto& ch = H[l].chunks;
        ch.clear();
        bool in = false;
        for (int r = 0; r < nrc; ++r) {
            if (tag[r] && !in) {
                in = true;
                ch.push_back({2 * r, 0});
            } else if (!tag[r] && in) {
                ch.back()[1] = 2 * r - 1;
                in = false;
            }
            if (in && r == nrc - 1) ch.back()[1] = 2 * r + 1;
        }
    }
    for (int l = 0; l < nlev; ++l) {
        Ctx& c = H[l];
        // spherical: one radial base state (max_radial_level = 0) that every level reads
        const madv_base_state* bs = c.sph ? &bsl[0] : &bsl[l];
        const int nr = c.nr;
        struct Arr1 {
            const char* name;
            const double* p;
            int n;
        } arrs[] = {{"rho0_old", bs->rho0_old, nr},   {"rho0_new", bs->rho0_new, nr}, {"rhoh0_old", bs->rhoh0_old, nr},
                    {"rhoh0_new", bs->rhoh0_new, nr}, {"p0_old", bs->p0_old, nr},     {"p0_new", bs->p0_new, nr},
                    {"psi", bs->psi, nr},             {"grav_cell", bs->grav_cell, nr}, {"w0_force", bs->w0_force, nr},
                    {"w0", bs->w0, nr + 1},           {"rho0_predicted_edge", bs->rho0_predicted_edge, nr + 1}};
        for (auto& a : arrs) {
            if (!a.p) {
                set_error(std::string("base state array ") + a.name + " is NULL");
                return MADV_ERR_PARAM;
            }
            c.h1[a.name] = std::vector<double>(a.p, a.p + a.n);
        }
    }
    // spherical: radii of the radial grid (Source/BaseStateGeometry.cpp:86-104), the exact one
    // or uniform bins of drf; r_cc_loc continued one bin past the last (Put1dArrayOnCart reads
    // r_cc_loc(nr_fine) with the exact grid)
    for (int l = 0; l < nlev; ++l) {
        Ctx& c = H[l];
        if (!c.sph) continue;
        std::vector<double> rc(c.nr + 1), re(c.nr + 1, 0.0);
        const double dxf = c.geo.dxf, drf = c.geo.drf;
        if (c.geo.exact) {
            for (int i = 0; i <= c.nr; ++i) rc[i] = std::sqrt(0.75 + 2.0 * double(i)) * dxf;
            for (int i = 0; i < c.nr; ++i) re[i + 1] = std::sqrt(0.75 + 2.0 * (double(i) + 0.5)) * dxf;
        } else {
            for (int i = 0; i <= c.nr; ++i) rc[i] = (double(i) + 0.5) * drf;
            for (int i = 0; i <= c.nr; ++i) re[i] = double(i) * drf;
        }
        c.h1["r_cc_loc"] = rc;
        c.h1["r_edge_loc"] = re;
        if (!c.geo.exact) {
            // dw0/dr on the bins (Source/MaestroForce.cpp:36-50), div w0 of the shells
            // (:283-297, the last bin 0) and h0 = rhoh0 / rho0 (Source/MaestroEnthalpyAdvance.cpp:194)
            const auto& w0 = c.h1["w0"];
            std::vector<double> g(c.nr), dv(c.nr, 0.0), ho(c.nr), hn(c.nr);
            for (int r = 0; r < c.nr; ++r) g[r] = (w0[r + 1] - w0[r]) / drf;
            for (int r = 0; r < c.nr - 1; ++r) {
                const double dr_loc = re[r + 1] - re[r];
                dv[r] = (re[r + 1] * re[r + 1] * w0[r + 1] - re[r] * re[r] * w0[r]) / (dr_loc * rc[r] * rc[r]);
            }
            for (int r = 0; r < c.nr; ++r) {
                ho[r] = c.h1["rhoh0_old"][r] / c.h1["rho0_old"][r];
                hn[r] = c.h1["rhoh0_new"][r] / c.h1["rho0_new"][r];
            }
            c.h1["gradw0"] = g;
            c.h1["divw0"] = dv;
            c.h1["h0_old"] = ho;
            c.h1["h0_new"] = hn;
        }
    }
    // which_step 2 averages of MakeRhoHForce: 0.5 * (old + new) (Source/MaestroForce.cpp:496-497)
    for (int l = 0; l < nlev; ++l) {
        Ctx& c = H[l];
        std::vector<double> ra(c.nr), pa(c.nr);
        for (int r = 0; r < c.nr; ++r) {
            ra[r] = 0.5 * (c.h1["rho0_old"][r] + c.h1["rho0_new"][r]);
            pa[r] = 0.5 * (c.h1["p0_old"][r] + c.h1["p0_new"][r]);
        }
        c.h1["rho0_avg"] = ra;
        c.h1["p0_avg"] = pa;
    }
    // Maestro::CelltoEdge over the chunks of every level, then RestrictBase of the edges
    // (Source/MaestroCelltoEdge.cpp:17-58, Source/MaestroBaseStateGeometry.cpp:240-262)
    for (const char* name : {"rho0_old", "rho0_new", "rhoh0_old", "rhoh0_new"}) {
        const std::string en = std::string(name).replace(std::string(name).find("0_"), 2, "0_edge_");
        for (int l = 0; l < nlev; ++l) {
            std::vector<double> e(H[l].nr + 1, 0.0);
            for (auto& ch : H[l].chunks) cell_to_edge_chunk(H[l].h1[name], e, ch[0], ch[1] + 1);
            H[l].h1[en] = e;
        }
        for (int l = nlev - 1; l >= 1 && !sph; --l)
            for (auto& ch : H[l].chunks)
                for (int j = ch[0]; j <= ch[1] + 1; j += 2) H[l - 1].h1[en][j / 2] = H[l].h1[en][j];
    }
    // BaseStateGeometry::ComputeCutoffCoords, base cutoff (Source/BaseStateGeometry.cpp:164-210);
    // one level, and spherical geometry (one radial level; no spherical kernel reads the
    // coordinate), keep the caller's base_cutoff_density_coord
    if (nlev > 1 && !sph) {
        bool found = false;
        int which = 0;
        std::vector<int> coord(nlev, 0);
        for (int n = nlev - 1; n >= 0 && !found; --n)
            for (auto& ch : H[n].chunks) {
                if (found) break;
                for (int r = ch[0]; r <= ch[1]; ++r)
                    if (H[n].h1["rho0_old"][r] <= H[0].P.base_cutoff_density) {
                        coord[n] = r;
                        which = n;
                        found = true;
                        break;
                    }
            }
        if (!found) {
            which = nlev - 1;
            coord[which] = H[which].nr;
        }
        for (int n = which + 1; n < nlev; ++n) coord[n] = 2 * coord[n - 1] + 1;
        for (int n = which - 1; n >= 0; --n) coord[n] = coord[n + 1] % 2 == 0 ? coord[n + 1] / 2 : coord[n + 1] / 2 + 1;
        for (int n = 0; n < nlev; ++n) H[n].P.base_cutoff_density_coord = coord[n];
    }
    for (int l = 0; l < nlev; ++l) {
        Ctx& c = H[l];
        for (auto& kv : c.h1) {
            double*& d = c.d1[kv.first];
            if (!d && !cuda_ok(cudaMalloc(&d, sizeof(double) * (c.nr + 1)), "cudaMalloc(base)")) return MADV_ERR_CUDA;
            if (!cuda_ok(cudaMemcpy(d, kv.second.data(), sizeof(double) * kv.second.size(), cudaMemcpyHostToDevice),
                         "cudaMemcpy(base)"))
                return MADV_ERR_CUDA;
        }
        c.have_base = true;
    }
    drop_graph(h);
    return MADV_OK;
}

int madv_set_base_state(madv_ctx* h, const madv_base_state* bs) {
    if (!h || !bs) return MADV_ERR_PARAM;
    if (!h->fine.empty()) {
        set_error("the layout has several levels: use madv_set_base_state_levels");
        return MADV_ERR_STATE;
    }
    return madv_set_base_state_levels(h, 1, bs);
}

static int stage_forward_h(madv_ctx* h, int mode, int nlev, const madv_multifab* uold, const madv_multifab* sold,
                           const madv_multifab* gpi, const madv_multifab* thermal, const madv_multifab* snew,
                           const madv_multifab* umac, const madv_multifab* sedge, const madv_multifab* sflux,
                           const madv_multifab* etarhoflux, void* stream) {
    Hier H = h->H();
    if (nlev != H.n()) {
        set_error("the call passes " + std::to_string(nlev) + " levels, the layout has " + std::to_string(H.n()));
        return MADV_ERR_PARAM;
    }
    int rc = check_ready_h(H, false);
    if (rc) return rc;
    if (!uold || !sold || !gpi) {
        set_error("uold, sold and gpi are required");
        return MADV_ERR_PARAM;
    }
    if (mode < MADV_MODE_BATCHED || mode > MADV_MODE_GRAPH) return MADV_ERR_PARAM;
    std::vector<StageIO> io(nlev);
    for (int l = 0; l < nlev; ++l) {
        io[l] = StageIO{&uold[l], &sold[l], &gpi[l], thermal ? &thermal[l] : nullptr, snew ? &snew[l] : nullptr,
                        umac ? &umac[3 * l] : nullptr, sedge ? &sedge[3 * l] : nullptr,
                        sflux ? &sflux[3 * l] : nullptr, etarhoflux ? &etarhoflux[l] : nullptr};
        // no edge states and no fluxes returned (3-D): the species are streamed
        io[l].stream = !sedge && !sflux && H[l].ndim == 3;
    }
    Ctx& c = h->c;
    set_mode(H, (cudaStream_t)stream, 0, false);
    reset_launches(H);
    // restores every level's view table on every way out
    std::vector<FabView*> base_views(nlev, nullptr);
    struct Restore {
        Hier& H;
        std::vector<FabView*>& v;
        ~Restore() {
            for (int l = 0; l < (int)v.size(); ++l) {
                if (v[l]) H[l].dviews = v[l];
                H[l].side_mirror = nullptr;
            }
        }
    } restore{H, base_views};
    try {
        for (int l = 0; l < nlev; ++l)
            if ((rc = bind_stage(H[l], io[l]))) return rc;
        // caller FABs laid out as the stage's fields are worked in directly (no copies)
        for (int l = 0; l < nlev; ++l) base_views[l] = alias_fields(H[l], io[l]);
        for (int l = 0; l < nlev; ++l)
            side_views(H[l], H[l].dviews == H[l].dviews_alias ? H[l].hviews_alias : H[l].hviews_pinned);
        if (mode == MADV_MODE_GRAPH) {
            std::vector<const void*> key;
            for (int l = 0; l < nlev; ++l) {
                key.push_back((const void*)(intptr_t)io[l].alias);
                const madv_multifab* all[] = {io[l].uold, io[l].sold, io[l].gpi, io[l].thermal, io[l].snew, io[l].eta};
                for (auto m : all) {
                    key.push_back(m);
                    if (m)
                        for (int b = 0; b < m->nfab; ++b) key.push_back(m->fab[b].p);
                }
                for (auto m3 : {io[l].umac, io[l].sedge, io[l].sflux}) {
                    key.push_back(m3);
                    if (m3)
                        for (int d = 0; d < H[l].ndim; ++d)
                            for (int b = 0; b < m3[d].nfab; ++b) key.push_back(m3[d].fab[b].p);
                }
            }
            if (!c.graph_exec || key != c.graph_key) {
                drop_graph(h);
                // a dry pass builds every region / copy table (no allocation may happen
                // while capturing), then the stage is captured
                set_mode(H, (cudaStream_t)stream, 0, true);
                stage_body(H, io);
                cudaStream_t cs;
                CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
                set_mode(H, cs, 0, false);
                reset_launches(H);
                cudaGraph_t g;
                CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
                for (auto* lc : H.L) upload_user_views(*lc);
                stage_body(H, io);
                CK(cudaStreamEndCapture(cs, &g));
                CK(cudaGraphInstantiate(&c.graph_exec, g, 0));
                cudaGraphDestroy(g);
                cudaStreamDestroy(cs);
                set_mode(H, (cudaStream_t)stream, 0, false);
                c.graph_key = key;
                c.graph_launches = total_launches(H);
            }
            CK(cudaGraphLaunch(c.graph_exec, c.stream));
            reset_launches(H);
            c.launches = c.graph_launches;
            return finish(H);
        }
        set_mode(H, (cudaStream_t)stream, mode == MADV_MODE_PER_BOX, false);
        stage_body(H, io);
        set_mode(H, (cudaStream_t)stream, 0, false);
        return finish(H);
    } catch (const Fail& f) {
        set_mode(H, (cudaStream_t)stream, 0, false);
        return f.code;
    }
}

int madv_stage_forward(madv_ctx* h, int mode, const madv_multifab* uold, const madv_multifab* sold,
                       const madv_multifab* gpi, const madv_multifab* thermal, const madv_multifab* snew,
                       const madv_multifab* umac, const madv_multifab* sedge, const madv_multifab* sflux,
                       const madv_multifab* etarhoflux, void* stream) {
    if (!h) return MADV_ERR_PARAM;
    return stage_forward_h(h, mode, 1, uold, sold, gpi, thermal, snew, umac, sedge, sflux, etarhoflux, stream);
}

int madv_stage_forward_levels(madv_ctx* h, int mode, int nlev, const madv_multifab* uold, const madv_multifab* sold,
                              const madv_multifab* gpi, const madv_multifab* thermal, const madv_multifab* snew,
                              const madv_multifab* umac, const madv_multifab* sedge, const madv_multifab* sflux,
                              const madv_multifab* etarhoflux, void* stream) {
    if (!h) return MADV_ERR_PARAM;
    return stage_forward_h(h, mode, nlev, uold, sold, gpi, thermal, snew, umac, sedge, sflux, etarhoflux, stream);
}

// ---- Maestro-shaped entry points (one level): the same pieces, with the caller's FABs
// copied in and out around each call.
// levels: the entry takes every level of the layout (else it takes one level only)
static int begin_call(madv_ctx* h, void* stream, Hier& H, bool levels = false) {
    if (!h) return MADV_ERR_PARAM;
    if (!h->fine.empty() && !levels) {
        set_error("the per-function entry points take one level; use madv_stage_forward_levels");
        return MADV_ERR_UNSUPPORTED;
    }
    H = h->H();
    int rc = check_ready_h(H);
    if (rc) return rc;
    set_mode(H, (cudaStream_t)stream, 0, false);
    reset_launches(H);
    cudaMemsetAsync(h->c.d_flag, 0, sizeof(int), h->c.stream);
    return MADV_OK;
}

int madv_advance_premac(madv_ctx* h, const madv_multifab* uold, const madv_multifab* sold, const madv_multifab* gpi,
                        const madv_multifab* umac, const madv_multifab* utrans, void* stream) {
    Hier H;
    int rc = begin_call(h, stream, H);
    if (rc) return rc;
    Ctx& c = h->c;
    if (!uold || !sold || !gpi || !umac) return MADV_ERR_PARAM;
    try {
        if ((rc = bind(c, U_UOLD, uold, c.ndim, -1, 0)) || (rc = bind(c, U_SOLD, sold, 1, -1, 0)) ||
            (rc = bind(c, U_GPI, gpi, c.ndim, -1, 0)))
            return rc;
        for (int d = 0; d < c.ndim; ++d) {
            if ((rc = bind(c, U_UMAC0 + d, &umac[d], 1, d, 0))) return rc;
            if (utrans && (rc = bind(c, U_UTRANS0 + d, &utrans[d], 1, d, 0))) return rc;
        }
        if ((rc = upload_user_views(c))) return rc;
        set_val(c, F_UTILDE, 0.0, 0, 3, c.ng_adv);
        copy_fab(c, F_UTILDE, 0, F_USER + U_UOLD, 0, c.ndim, 0);
        copy_fab(c, F_SOLD, RHO, F_USER + U_SOLD, RHO, 1, 0);
        copy_fab(c, F_GPI, 0, F_USER + U_GPI, 0, c.ndim, 0);
        for (int d = 0; d < c.ndim; ++d) set_val(c, F_UMAC0 + d, 0.0, 0, 1, 1);
        w0_carts(H);
        advance_premac(H);
        for (int d = 0; d < c.ndim; ++d) {
            copy_fab(c, F_USER + U_UMAC0 + d, 0, F_UMAC0 + d, 0, 1, 0);
            if (utrans) copy_fab(c, F_USER + U_UTRANS0 + d, 0, F_UTRANS0 + d, 0, 1, 0);
        }
        return finish(H);
    } catch (const Fail& f) {
        return f.code;
    }
}

int madv_addw0(madv_ctx* h, const madv_multifab* umac, double mult, void* stream) {
    Hier H;
    int rc = begin_call(h, stream, H);
    if (rc) return rc;
    Ctx& c = h->c;
    if (!umac) return MADV_ERR_PARAM;
    try {
        for (int d = 0; d < c.ndim; ++d)
            if ((rc = bind(c, U_UMAC0 + d, &umac[d], 1, d, 1))) return rc;
        if ((rc = upload_user_views(c))) return rc;
        for (int d = 0; d < c.ndim; ++d) copy_fab(c, F_UMAC0 + d, 0, F_USER + U_UMAC0 + d, 0, 1, 1);
        addw0_h(H, F_UMAC0, mult);
        for (int d = 0; d < c.ndim; ++d) copy_fab(c, F_USER + U_UMAC0 + d, 0, F_UMAC0 + d, 0, 1, 1);
        return finish(H);
    } catch (const Fail& f) {
        return f.code;
    }
}

static int scalar_advance(madv_ctx* h, int which, int which_step, const madv_multifab* sold, const madv_multifab* snew,
                          const madv_multifab* sedge, const madv_multifab* sflux, const madv_multifab* eta,
                          const madv_multifab* umac, const madv_multifab* thermal, void* stream) {
    Hier H;
    int rc = begin_call(h, stream, H);
    if (rc) return rc;
    Ctx& c = h->c;
    if (which_step != 1 && which_step != 2) {
        set_error("which_step must be 1 (predictor) or 2 (corrector)");
        return MADV_ERR_PARAM;
    }
    if (!sold || !snew || !umac) return MADV_ERR_PARAM;
    try {
        if ((rc = bind(c, U_SOLD, sold, c.nscal, -1, 0)) || (rc = bind(c, U_SNEW, snew, c.nscal, -1, 0)) ||
            (rc = bind(c, U_ETA, eta, 1, c.ndim - 1, 0)) || (rc = bind(c, U_THERMAL, thermal, 1, -1, 0)))
            return rc;
        for (int d = 0; d < c.ndim; ++d) {
            if ((rc = bind(c, U_UMAC0 + d, &umac[d], 1, d, 1))) return rc;
            if (sedge && (rc = bind(c, U_SEDGE0 + d, &sedge[d], c.nscal, d, 0))) return rc;
            if (sflux && (rc = bind(c, U_SFLUX0 + d, &sflux[d], c.nscal, d, 0))) return rc;
        }
        if ((rc = upload_user_views(c))) return rc;
        copy_fab(c, F_SOLD, 0, F_USER + U_SOLD, 0, c.nscal, 0);
        fill_patch_h(H, F_SOLD, 0, c.nscal, BCS_S, 0, 0, 0);
        copy_fab(c, F_SNEW, 0, F_USER + U_SNEW, 0, c.nscal, 0);
        for (int d = 0; d < c.ndim; ++d) {
            copy_fab(c, F_UMAC0 + d, 0, F_USER + U_UMAC0 + d, 0, 1, 1);
            if (sedge) copy_fab(c, F_SEDGE0 + d, 0, F_USER + U_SEDGE0 + d, 0, c.nscal, 0);
            if (sflux) copy_fab(c, F_SFLUX0 + d, 0, F_USER + U_SFLUX0 + d, 0, c.nscal, 0);
        }
        set_val(c, F_THERMAL, 0.0, 0, 1, 1);
        if (thermal) copy_fab(c, F_THERMAL, 0, F_USER + U_THERMAL, 0, 1, 0);
        w0_carts(H);
        if (which == 0) {
            set_val(c, F_ETA, 0.0, 0, 1, 0);
            if (eta) copy_fab(c, F_ETA, 0, F_USER + U_ETA, 0, 1, 0);
            density_advance(H, which_step);
            copy_fab(c, F_USER + U_SNEW, RHO, F_SNEW, RHO, 1, 0);
            copy_fab(c, F_USER + U_SNEW, FIRSTSPEC, F_SNEW, FIRSTSPEC, c.nspec, 0);
            if (eta) copy_fab(c, F_USER + U_ETA, 0, F_ETA, 0, 1, 0);
        } else {
            enthalpy_advance(H, which_step);
            copy_fab(c, F_USER + U_SNEW, RHOH, F_SNEW, RHOH, 1, 0);
        }
        copy_fab(c, F_USER + U_SOLD, 0, F_SOLD, 0, c.nscal, 0);
        for (int d = 0; d < c.ndim; ++d) {
            copy_fab(c, F_USER + U_UMAC0 + d, 0, F_UMAC0 + d, 0, 1, 1);
            if (sedge) copy_fab(c, F_USER + U_SEDGE0 + d, 0, F_SEDGE0 + d, 0, c.nscal, 0);
            if (sflux) copy_fab(c, F_USER + U_SFLUX0 + d, 0, F_SFLUX0 + d, 0, c.nscal, 0);
        }
        return finish(H);
    } catch (const Fail& f) {
        return f.code;
    }
}

int madv_density_advance(madv_ctx* h, int which_step, const madv_multifab* sold, const madv_multifab* snew,
                         const madv_multifab* sedge, const madv_multifab* sflux, const madv_multifab* etarhoflux,
                         const madv_multifab* umac, void* stream) {
    return scalar_advance(h, 0, which_step, sold, snew, sedge, sflux, etarhoflux, umac, nullptr, stream);
}

int madv_enthalpy_advance(madv_ctx* h, int which_step, const madv_multifab* sold, const madv_multifab* snew,
                          const madv_multifab* sedge, const madv_multifab* sflux, const madv_multifab* umac,
                          const madv_multifab* thermal, void* stream) {
    return scalar_advance(h, 1, which_step, sold, snew, sedge, sflux, nullptr, umac, thermal, stream);
}

// ---- the member functions inside AdvancePremac / DensityAdvance / EnthalpyAdvance, one
// level, 3-D.  Inputs are read with the ghost cells the reference's callers fill before the
// call; each entry recomputes the implicit inputs it needs from the context (w0_cart, w0mac,
// the face base state of the spherical fluxes).
static int begin_member(madv_ctx* h, void* stream, Hier& H) {
    int rc = begin_call(h, stream, H);
    if (rc) return rc;
    if (h->c.ndim != 3) {
        set_error("the per-member-function entry points are 3-D");
        return MADV_ERR_UNSUPPORTED;
    }
    return MADV_OK;
}

int madv_make_utrans(madv_ctx* h, const madv_multifab* utilde, const madv_multifab* ufull,
                     const madv_multifab* utrans, void* stream) {
    Hier H;
    int rc = begin_member(h, stream, H);
    if (rc) return rc;
    Ctx& c = h->c;
    if (!utilde || !ufull || !utrans) return MADV_ERR_PARAM;
    try {
        const int nga = c.ng_adv;
        if ((rc = bind(c, U_UOLD, utilde, 3, -1, nga)) || (rc = bind(c, U_UFULL, ufull, 3, -1, nga))) return rc;
        for (int d = 0; d < 3; ++d)
            if ((rc = bind(c, U_UTRANS0 + d, &utrans[d], 1, d, 0))) return rc;
        if ((rc = upload_user_views(c))) return rc;
        copy_fab(c, F_UTILDE, 0, F_USER + U_UOLD, 0, 3, nga);
        copy_fab(c, F_UFULL, 0, F_USER + U_UFULL, 0, 3, nga);
        w0_carts(H);
        for (int d = 0; d < 3; ++d) set_val(c, F_UTRANS0 + d, 0.0, 0, 1, 1);
        make_utrans(c);
        sync_faces_h(H, F_UTRANS0);  // FillBoundary + FillUmacGhost (Source/MaestroMakeUtrans.cpp:630-639)
        for (int d = 0; d < 3; ++d)
            copy_fab(c, F_USER + U_UTRANS0 + d, 0, F_UTRANS0 + d, 0, 1, held_ghosts(c, &utrans[d], d, 1));
        return finish(H);
    } catch (const Fail& f) {
        return f.code;
    }
}

int madv_vel_pred(madv_ctx* h, const madv_multifab* utilde, const madv_multifab* ufull, const madv_multifab* utrans,
                  const madv_multifab* umac, const madv_multifab* force, void* stream) {
    Hier H;
    int rc = begin_member(h, stream, H);
    if (rc) return rc;
    Ctx& c = h->c;
    if (!utilde || !ufull || !utrans || !umac || !force) return MADV_ERR_PARAM;
    try {
        const int nga = c.ng_adv;
        if ((rc = bind(c, U_UOLD, utilde, 3, -1, nga)) || (rc = bind(c, U_UFULL, ufull, 3, -1, nga)) ||
            (rc = bind(c, U_FORCE, force, 3, -1, c.F[F_VELFORCE].spec.ng)))
            return rc;
        for (int d = 0; d < 3; ++d)
            if ((rc = bind(c, U_UTRANS0 + d, &utrans[d], 1, d, 1)) || (rc = bind(c, U_UMAC0 + d, &umac[d], 1, d, 0)))
                return rc;
        if ((rc = upload_user_views(c))) return rc;
        copy_fab(c, F_UTILDE, 0, F_USER + U_UOLD, 0, 3, nga);
        copy_fab(c, F_UFULL, 0, F_USER + U_UFULL, 0, 3, nga);
        copy_fab(c, F_VELFORCE, 0, F_USER + U_FORCE, 0, 3, c.F[F_VELFORCE].spec.ng);
        for (int d = 0; d < 3; ++d) {
            copy_fab(c, F_UTRANS0 + d, 0, F_USER + U_UTRANS0 + d, 0, 1, 1);
            set_val(c, F_UMAC0 + d, 0.0, 0, 1, 1);
        }
        w0_carts(H);
        vel_pred_prep(c);
        vel_pred(c);
        for (int d = 0; d < 3; ++d) copy_fab(c, F_USER + U_UMAC0 + d, 0, F_UMAC0 + d, 0, 1, 0);
        return finish(H);
    } catch (const Fail& f) {
        return f.code;
    }
}

int madv_make_edge_scal(madv_ctx* h, const madv_multifab* state, const madv_multifab* sedge,
                        const madv_multifab* umac, const madv_multifab* force, int is_vel, int start_scomp,
                        int start_bccomp, int num_comp, int is_conservative, void* stream) {
    Hier H;
    int rc = begin_member(h, stream, H);
    if (rc) return rc;
    Ctx& c = h->c;
    if (!state || !sedge || !umac || !force) return MADV_ERR_PARAM;
    if (is_vel || start_bccomp != start_scomp) {
        set_error("MakeEdgeScal: scalars with start_bccomp == start_scomp (velocity edges are not built)");
        return MADV_ERR_UNSUPPORTED;
    }
    if (start_scomp < 0 || num_comp < 1 || start_scomp + num_comp > c.nscal) {
        set_error("MakeEdgeScal: component range outside the state");
        return MADV_ERR_PARAM;
    }
    try {
        if ((rc = bind(c, U_SOLD, state, start_scomp + num_comp, -1, c.ng_s)) ||
            (rc = bind(c, U_FORCE, force, start_scomp + num_comp, -1, c.F[F_SCALFORCE].spec.ng)))
            return rc;
        for (int d = 0; d < 3; ++d)
            if ((rc = bind(c, U_UMAC0 + d, &umac[d], 1, d, 1)) ||
                (rc = bind(c, U_SEDGE0 + d, &sedge[d], start_scomp + num_comp, d, 0)))
                return rc;
        if ((rc = upload_user_views(c))) return rc;
        copy_fab(c, F_SOLD, start_scomp, F_USER + U_SOLD, start_scomp, num_comp, c.ng_s);
        copy_fab(c, F_SCALFORCE, start_scomp, F_USER + U_FORCE, start_scomp, num_comp, c.F[F_SCALFORCE].spec.ng);
        for (int d = 0; d < 3; ++d) copy_fab(c, F_UMAC0 + d, 0, F_USER + U_UMAC0 + d, 0, 1, 1);
        make_edge_scal(c, start_scomp, num_comp, BCS_S, is_conservative != 0, 0);
        for (int d = 0; d < 3; ++d)
            copy_fab(c, F_USER + U_SEDGE0 + d, start_scomp, F_SEDGE0 + d, start_scomp, num_comp, 0);
        return finish(H);
    } catch (const Fail& f) {
        return f.code;
    }
}

// MakeRhoXFlux / MakeRhoHFlux: which_step 1 passes the old base state as the "new" one, as
// DensityAdvance / EnthalpyAdvance do in the predictor (Source/MaestroDensityAdvance.cpp:186-219)
static int flux_member(madv_ctx* h, int which, int which_step, const madv_multifab* sflux,
                       const madv_multifab* etarhoflux, const madv_multifab* sedge, const madv_multifab* umac,
                       void* stream) {
    Hier H;
    int rc = begin_member(h, stream, H);
    if (rc) return rc;
    Ctx& c = h->c;
    if (!sflux || !sedge || !umac) return MADV_ERR_PARAM;
    if (which_step != 1 && which_step != 2) {
        set_error("which_step must be 1 (predictor) or 2 (corrector)");
        return MADV_ERR_PARAM;
    }
    try {
        if ((rc = bind(c, U_ETA, etarhoflux, 1, 2, 0))) return rc;
        for (int d = 0; d < 3; ++d)
            if ((rc = bind(c, U_SEDGE0 + d, &sedge[d], c.nscal, d, 0)) ||
                (rc = bind(c, U_UMAC0 + d, &umac[d], 1, d, 0)) || (rc = bind(c, U_SFLUX0 + d, &sflux[d], c.nscal, d, 0)))
                return rc;
        if ((rc = upload_user_views(c))) return rc;
        for (int d = 0; d < 3; ++d) {
            copy_fab(c, F_SEDGE0 + d, 0, F_USER + U_SEDGE0 + d, 0, c.nscal, 0);
            set_val(c, F_UMAC0 + d, 0.0, 0, 1, 1);
            copy_fab(c, F_UMAC0 + d, 0, F_USER + U_UMAC0 + d, 0, 1, 0);
        }
        w0_carts(H);
        if (which == 0) {
            set_val(c, F_ETA, 0.0, 0, 1, 0);
            if (etarhoflux) copy_fab(c, F_ETA, 0, F_USER + U_ETA, 0, 1, 0);
            const char* r0n = which_step == 1 ? "rho0_old" : "rho0_new";
            const char* r0en = which_step == 1 ? "rho0_edge_old" : "rho0_edge_new";
            if (c.sph) {
                make_s0mac_h(H, "rho0_old", F_S0MAC0);
                make_s0mac_h(H, r0n, F_S0MACB0);
            }
            make_rhox_flux(c, c.b1("rho0_old"), c.b1("rho0_edge_old"), c.b1(r0n), c.b1(r0en));
            for (int d = 0; d < 3; ++d) {
                copy_fab(c, F_USER + U_SFLUX0 + d, RHO, F_SFLUX0 + d, RHO, 1, 0);
                copy_fab(c, F_USER + U_SFLUX0 + d, FIRSTSPEC, F_SFLUX0 + d, FIRSTSPEC, c.nspec, 0);
            }
            if (etarhoflux) copy_fab(c, F_USER + U_ETA, 0, F_ETA, 0, 1, 0);
        } else {
            rhoh_flux_h(H, which_step);
            for (int d = 0; d < 3; ++d) copy_fab(c, F_USER + U_SFLUX0 + d, RHOH, F_SFLUX0 + d, RHOH, 1, 0);
        }
        return finish(H);
    } catch (const Fail& f) {
        return f.code;
    }
}

int madv_make_rhox_flux(madv_ctx* h, int which_step, const madv_multifab* sflux, const madv_multifab* etarhoflux,
                        const madv_multifab* sedge, const madv_multifab* umac, int start_comp, int num_comp,
                        void* stream) {
    if (h && (start_comp != FIRSTSPEC || num_comp != h->c.nspec)) {
        set_error("MakeRhoXFlux: the species FirstSpec .. FirstSpec+NumSpec-1 (the reference's only call)");
        return MADV_ERR_UNSUPPORTED;
    }
    return flux_member(h, 0, which_step, sflux, etarhoflux, sedge, umac, stream);
}

int madv_make_rhoh_flux(madv_ctx* h, int which_step, const madv_multifab* sflux, const madv_multifab* sedge,
                        const madv_multifab* umac, void* stream) {
    return flux_member(h, 1, which_step, sflux, nullptr, sedge, umac, stream);
}

int madv_update_scal(madv_ctx* h, const madv_multifab* stateold, const madv_multifab* statenew,
                     const madv_multifab* sflux, const madv_multifab* force, int start_comp, int num_comp,
                     void* stream) {
    Hier H;
    int rc = begin_member(h, stream, H);
    if (rc) return rc;
    Ctx& c = h->c;
    if (!stateold || !statenew || !sflux || !force) return MADV_ERR_PARAM;
    if (!((start_comp == RHOH && num_comp == 1) || (start_comp == FIRSTSPEC && num_comp == c.nspec))) {
        set_error("UpdateScal: RhoH, or the species FirstSpec .. FirstSpec+NumSpec-1");
        return MADV_ERR_UNSUPPORTED;
    }
    try {
        if ((rc = bind(c, U_SOLD, stateold, c.nscal, -1, 0)) || (rc = bind(c, U_SNEW, statenew, c.nscal, -1, 0)) ||
            (rc = bind(c, U_FORCE, force, c.nscal, -1, 0)))
            return rc;
        for (int d = 0; d < 3; ++d)
            if ((rc = bind(c, U_SFLUX0 + d, &sflux[d], c.nscal, d, 0))) return rc;
        if ((rc = upload_user_views(c))) return rc;
        copy_fab(c, F_SOLD, 0, F_USER + U_SOLD, 0, c.nscal, 0);
        copy_fab(c, F_SNEW, 0, F_USER + U_SNEW, 0, c.nscal, 0);
        copy_fab(c, F_SCALFORCE, 0, F_USER + U_FORCE, 0, c.nscal, 0);
        for (int d = 0; d < 3; ++d) copy_fab(c, F_SFLUX0 + d, 0, F_USER + U_SFLUX0 + d, 0, c.nscal, 0);
        update_scal_h(H, start_comp);  // with AverageDown + FillPatch of the updated components
        const int g = held_ghosts(c, statenew, -1, c.ng_s);
        copy_fab(c, F_USER + U_SNEW, start_comp, F_SNEW, start_comp, num_comp, g);
        if (start_comp == FIRSTSPEC) copy_fab(c, F_USER + U_SNEW, RHO, F_SNEW, RHO, 1, g);
        return finish(H);
    } catch (const Fail& f) {
        return f.code;
    }
}

// Maestro::VelocityAdvance (Source/MaestroVelocityAdvance.cpp:5-82) with UpdateVel
// (Source/MaestroAdvection.cpp:299-526), one level, 3-D.  The velocity edge states are
// MakeEdgeScal with is_vel on the internal state field (components 0-2 hold uold) and the
// updated velocity goes through F_SNEW components 0-2, both scratch of this call.
int madv_velocity_advance(madv_ctx* h, const madv_multifab* uold, const madv_multifab* sold,
                          const madv_multifab* rhohalf, const madv_multifab* gpi, const madv_multifab* umac,
                          const madv_multifab* sponge, const madv_multifab* unew, const madv_multifab* uedge,
                          void* stream) {
    Hier H;
    int rc = begin_member(h, stream, H);
    if (rc) return rc;
    Ctx& c = h->c;
    if (!uold || !sold || !rhohalf || !gpi || !umac || !unew) return MADV_ERR_PARAM;
    try {
        if ((rc = bind(c, U_UOLD, uold, 3, -1, 0)) || (rc = bind(c, U_SOLD, sold, 1, -1, 0)) ||
            (rc = bind(c, U_RHOHALF, rhohalf, 1, -1, 0)) || (rc = bind(c, U_GPI, gpi, 3, -1, 0)) ||
            (rc = bind(c, U_SPONGE, sponge, 1, -1, 0)) || (rc = bind(c, U_SNEW, unew, 3, -1, 0)))
            return rc;
        for (int d = 0; d < 3; ++d) {
            if ((rc = bind(c, U_UMAC0 + d, &umac[d], 1, d, 0))) return rc;
            if (uedge && (rc = bind(c, U_UEDGE0 + d, &uedge[d], 3, d, 0))) return rc;
        }
        if ((rc = upload_user_views(c))) return rc;
        copy_fab(c, F_GPI, 0, F_USER + U_GPI, 0, 3, 0);
        for (int d = 0; d < 3; ++d) {
            set_val(c, F_UMAC0 + d, 0.0, 0, 1, 1);
            copy_fab(c, F_UMAC0 + d, 0, F_USER + U_UMAC0 + d, 0, 1, 0);
        }
        sync_faces_h(H, F_UMAC0);  // the ghost faces as MacProj leaves them (FillUmacGhost)
        w0_carts(H);
        // MakeVelForce(vel_force, umac, sold, rho0_old, grav_cell_old, w0_force_cart, 1)
        copy_fab(c, F_SOLD, RHO, F_USER + U_SOLD, RHO, 1, 0);
        make_vel_force_h(H, F_UMAC0, "rho0_old");
        addw0_h(H, F_UMAC0, 1.0);
        // MakeEdgeScal(uold, uedge, umac, vel_force, true, bcs_u, AMREX_SPACEDIM, 0, 0, AMREX_SPACEDIM, false)
        copy_fab(c, F_SOLD, 0, F_USER + U_UOLD, 0, 3, 0);
        fill_patch_h(H, F_SOLD, 0, 3, BCS_U, 0, 1, -1);
        copy_fab(c, F_SCALFORCE, 0, F_VELFORCE, 0, 3, c.F[F_VELFORCE].spec.ng);
        for (int d = 0; d < 3; ++d) set_val(c, F_SEDGE0 + d, 0.0, 0, 3, 0);
        make_edge_scal(c, 0, 3, BCS_U, 0, 0, 1);
        addw0_h(H, F_UMAC0, -1.0);
        // MakeVelForce(vel_force, umac, rhohalf, rho0_nph, grav_cell_nph, w0_force_cart, 1)
        copy_fab(c, F_SOLD, RHO, F_USER + U_RHOHALF, 0, 1, 0);
        make_vel_force_h(H, F_UMAC0, "rho0_avg");
        update_vel(c, F_USER + U_UOLD, sponge ? F_USER + U_SPONGE : -1);
        average_down_h(H, F_SNEW, 0, 3);
        fill_patch_h(H, F_SNEW, 0, 3, BCS_U, 0, 1, -1);
        copy_fab(c, F_USER + U_SNEW, 0, F_SNEW, 0, 3, held_ghosts(c, unew, -1, c.ng_s));
        if (uedge)
            for (int d = 0; d < 3; ++d) copy_fab(c, F_USER + U_UEDGE0 + d, 0, F_SEDGE0 + d, 0, 3, 0);
        return finish(H);
    } catch (const Fail& f) {
        return f.code;
    }
}

// Maestro::MacProj, plane-parallel, one level (Source/MaestroMacProj.cpp:11-236): the
// caller's umac is copied in with its ghost faces, projected, refilled and copied back
int madv_mac_project(madv_ctx* h, const madv_multifab* umac, const madv_multifab* macphi, const madv_multifab* macrhs,
                     const madv_multifab* rho, const double* beta0, double tol_rel, int max_iter,
                     madv_mac_result* result, void* stream) {
    Hier H;
    int rc = begin_call(h, stream, H);
    if (rc) return rc;
    Ctx& c = h->c;
    if (!umac || !macrhs || !rho || !beta0 || !(tol_rel > 0.0) || max_iter < 1) {
        set_error("madv_mac_project: umac, macrhs, rho, beta0, tol_rel > 0 and max_iter >= 1 are required");
        return MADV_ERR_PARAM;
    }
    if (c.ndim != 3 || H.n() != 1) {
        set_error("madv_mac_project covers one 3-D level, plane-parallel or spherical");
        return MADV_ERR_UNSUPPORTED;
    }
    try {
        for (int d = 0; d < 3; ++d)
            if ((rc = bind(c, U_UMAC0 + d, &umac[d], 1, d, 1))) return rc;
        if ((rc = bind(c, U_FORCE, macrhs, 1, -1, 0)) || (rc = bind(c, U_RHOHALF, rho, 1, -1, 0)) ||
            (rc = bind(c, U_SPONGE, macphi, 1, -1, 0)))
            return rc;
        if ((rc = upload_user_views(c))) return rc;
        for (int d = 0; d < 3; ++d) copy_fab(c, F_UMAC0 + d, 0, F_USER + U_UMAC0 + d, 0, 1, 1);
        if (c.sph) {  // beta0 on the faces: MakeS0mac (Source/MaestroMacProj.cpp:41-44) into F_S0MAC*
            std::vector<double>& b = c.h1["beta0_mac"];
            b.assign(beta0, beta0 + c.nr);
            double*& d = c.d1["beta0_mac"];
            if (!d && !cuda_ok(cudaMalloc(&d, sizeof(double) * (c.nr + 1)), "cudaMalloc(beta0)")) return MADV_ERR_CUDA;
            if (!cuda_ok(cudaMemcpyAsync(d, b.data(), sizeof(double) * c.nr, cudaMemcpyHostToDevice, c.stream),
                         "cudaMemcpyAsync(beta0)"))
                return MADV_ERR_CUDA;
            make_s0mac_h(H, "beta0_mac", F_S0MAC0);
        }
        // plane-parallel: beta0 on the radial edges, CelltoEdge (Source/MaestroCelltoEdge.cpp:17-54)
        const int nr = c.P.dom_hi[2] - c.P.dom_lo[2] + 1;
        std::vector<double> b0(nr, 0.0), b0e(nr + 1, 0.0);  // spherical: unused (beta0 is on the faces)
        if (!c.sph) {
            b0.assign(beta0, beta0 + nr);
            cell_to_edge_chunk(b0, b0e, 0, nr);
        }
        int it = 0;
        double ratio = 0.0;
        rc = mac_project_level(c, U_FORCE, U_RHOHALF, macphi ? U_SPONGE : -1, b0.data(), b0e.data(), tol_rel, max_iter,
                               &it, &ratio);
        if (result) {
            result->iterations = it;
            result->resid_ratio = ratio;
        }
        if (rc) return rc;
        for (int d = 0; d < 3; ++d) copy_fab(c, F_USER + U_UMAC0 + d, 0, F_UMAC0 + d, 0, 1, 1);
        return finish(H);
    } catch (const Fail& f) {
        return f.code;
    }
}

// MacProj on an AMR hierarchy of two plane-parallel levels (Source/MaestroMacProj.cpp:11-236):
// the composite solve of madv_macproj.cu, then AverageDownFaces and FillPatchUedge of umac.
int madv_mac_project_levels(madv_ctx* h, int nlev, const madv_multifab* umac, const madv_multifab* macphi,
                            const madv_multifab* macrhs, const madv_multifab* rho, const double* beta0,
                            double tol_rel, int max_iter, madv_mac_result* result, void* stream) {
    Hier H;
    int rc = begin_call(h, stream, H, true);
    if (rc) return rc;
    if (!umac || !macrhs || !rho || !beta0 || !(tol_rel > 0.0) || max_iter < 1 || nlev != H.n()) {
        set_error("madv_mac_project_levels: one entry per level of the layout; umac, macrhs, rho, beta0, "
                  "tol_rel > 0 and max_iter >= 1 are required");
        return MADV_ERR_PARAM;
    }
    if (nlev == 1) return madv_mac_project(h, umac, macphi, macrhs, rho, beta0, tol_rel, max_iter, result, stream);
    if (nlev != 2 || H[0].sph || H[0].ndim != 3) {
        set_error("madv_mac_project_levels covers one or two 3-D plane-parallel levels");
        return MADV_ERR_UNSUPPORTED;
    }
    try {
        for (int l = 0; l < 2; ++l) {
            Ctx& c = H[l];
            for (int d = 0; d < 3; ++d)
                if ((rc = bind(c, U_UMAC0 + d, &umac[3 * l + d], 1, d, 1))) return rc;
            if ((rc = bind(c, U_FORCE, &macrhs[l], 1, -1, 0)) || (rc = bind(c, U_RHOHALF, &rho[l], 1, -1, 0)) ||
                (rc = bind(c, U_SPONGE, macphi ? &macphi[l] : nullptr, 1, -1, 0)))
                return rc;
            if ((rc = upload_user_views(c))) return rc;
            for (int d = 0; d < 3; ++d) copy_fab(c, F_UMAC0 + d, 0, F_USER + U_UMAC0 + d, 0, 1, 1);
        }
        // beta0 on the radial edges of both levels: CelltoEdge over each level's chunks, the
        // level-1 edges restricted onto level 0 (Source/MaestroCelltoEdge.cpp:17-58,
        // Source/BaseStateGeometry.cpp:240-262)
        const int nr0 = H[0].nr, nr1 = H[1].nr;
        std::vector<double> b0(beta0, beta0 + nr0), b1(beta0 + nr0, beta0 + nr0 + nr1);
        std::vector<double> e0(nr0 + 1, 0.0), e1(nr1 + 1, 0.0);
        cell_to_edge_chunk(b0, e0, 0, nr0);
        for (auto& ch : H[1].chunks) cell_to_edge_chunk(b1, e1, ch[0], ch[1] + 1);
        for (auto& ch : H[1].chunks)
            for (int j = ch[0]; j <= ch[1] + 1; j += 2) e0[j / 2] = e1[j];
        int it = 0;
        double ratio = 0.0;
        rc = mac_project_two_levels(H[0], H[1], U_FORCE, U_RHOHALF, macphi ? U_SPONGE : -1, b0.data(), e0.data(),
                                    b1.data(), e1.data(), tol_rel, max_iter, &it, &ratio);
        if (result) {
            result->iterations = it;
            result->resid_ratio = ratio;
        }
        if (rc) return rc;
        sync_faces_h(H, F_UMAC0);  // AverageDownFaces, FillPatchUedge, the ghost faces
        for (int l = 0; l < 2; ++l)
            for (int d = 0; d < 3; ++d) copy_fab(H[l], F_USER + U_UMAC0 + d, 0, F_UMAC0 + d, 0, 1, 1);
        return finish(H);
    } catch (const Fail& f) {
        return f.code;
    }
}

// Maestro::EstDt (Source/MaestroDt.cpp:11-225 planar, :301-384 spherical, :440-483): the
// advective and force constraints and rel_eps on every level.  The per-level maxima are exact
// (k_dt_maxima), and the reference's per-box minima of monotone functions of per-box maxima
// equal the same functions of the level maxima, so dt and umax match it bit for bit.
int madv_est_dt(madv_ctx* h, int nlev, const madv_multifab* uold, const madv_multifab* sold,
                const madv_multifab* gpi, const madv_dt_params* prm, madv_dt_result* res, void* stream) {
    if (!h || !uold || !sold || !gpi || !prm || !res) return MADV_ERR_PARAM;
    Hier H = h->H();
    if (nlev != H.n()) {
        set_error("the call passes " + std::to_string(nlev) + " levels, the layout has " + std::to_string(H.n()));
        return MADV_ERR_PARAM;
    }
    int rc = check_ready_h(H);
    if (rc) return rc;
    if (!(prm->cfl > 0.0) || prm->drdxfac < 1) {
        set_error("EstDt: cfl > 0 and drdxfac >= 1");
        return MADV_ERR_PARAM;
    }
    if (H[0].ndim != 3) {
        set_error("EstDt: 3-D");
        return MADV_ERR_UNSUPPORTED;
    }
    if (H[0].sph && !H[0].geo.exact && prm->drdxfac != (H[0].P.drdxfac > 0 ? H[0].P.drdxfac : 1)) {
        set_error("EstDt: drdxfac must be the radial grid's (madv_params.drdxfac)");
        return MADV_ERR_PARAM;
    }
    set_mode(H, (cudaStream_t)stream, 0, false);
    reset_launches(H);
    try {
        const int nd = H[0].ndim;
        for (int l = 0; l < nlev; ++l) {
            Ctx& c = H[l];
            if ((rc = bind(c, U_UOLD, &uold[l], nd, -1, 0)) || (rc = bind(c, U_SOLD, &sold[l], 1, -1, 0)) ||
                (rc = bind(c, U_GPI, &gpi[l], nd, -1, 0)) || (rc = upload_user_views(c)))
                return rc;
            if (!c.d_red && !cuda_ok(cudaMalloc(&c.d_red, 7 * sizeof(unsigned long long)), "cudaMalloc(EstDt)"))
                return MADV_ERR_CUDA;
            cudaMemsetAsync(c.d_flag, 0, sizeof(int), c.stream);
            set_val(c, F_UTILDE, 0.0, 0, 3, 0);
            copy_fab(c, F_UTILDE, 0, F_USER + U_UOLD, 0, nd, 0);
            copy_fab(c, F_SOLD, RHO, F_USER + U_SOLD, RHO, 1, 0);
            set_val(c, F_GPI, 0.0, 0, 3, 0);
            copy_fab(c, F_GPI, 0, F_USER + U_GPI, 0, nd, 0);
            for (int d = 0; d < 3; ++d) set_val(c, F_UTRANS0 + d, 0.0, 0, 1, 1);  // umac_dummy (:24-37)
        }
        w0_carts(H);
        // MakeVelForce(vel_force, umac_dummy, sold, rho0_old, grav_cell_old, w0_force_cart_dummy, 0)
        for (auto* c : H.L) set_val(*c, F_W0FCART, 0.0, 0, 3, 1);
        make_vel_force_h(H);
        std::vector<std::array<unsigned long long, 7>> mx(nlev);
        for (int l = 0; l < nlev; ++l) {
            Ctx& c = H[l];
            CK(cudaMemsetAsync(c.d_red, 0, 7 * sizeof(unsigned long long), c.stream));
            dt_maxima(c);
            CK(cudaMemcpyAsync(mx[l].data(), c.d_red, 7 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                               c.stream));
        }
        if ((rc = finish(H))) return rc;
        auto val = [](unsigned long long b) {
            double v;
            std::memcpy(&v, &b, sizeof(v));
            return v;
        };
        const double eps = 1.e-8;
        double dt = 1.e20, umax = 0.0;
        for (int l = 0; l < nlev; ++l) {
            const Ctx& c = H[l];
            const double spd[3] = {val(mx[l][0]), val(mx[l][1]), val(mx[l][2])}, spdr = val(mx[l][3]);
            const double f[3] = {val(mx[l][4]), val(mx[l][5]), val(mx[l][6])};
            double dt_temp = 1.e99;
            umax = std::max(umax, std::max(spd[0], std::max(spd[1], std::max(spd[2], spdr))));
            for (int d = 0; d < nd; ++d)
                if (spd[d] > eps) dt_temp = std::min(dt_temp, c.P.dx[d] / spd[d]);
            // radial spacing: dx of the radial direction, or base_geom.dr(0) = finest dx / drdxfac
            const double dr = c.sph ? c.geo.dxf / prm->drdxfac : c.P.dx[nd - 1];
            if (spdr > eps) dt_temp = std::min(dt_temp, dr / spdr);
            dt_temp *= prm->cfl;
            for (int d = 0; d < nd; ++d)
                if (f[d] > eps) dt_temp = std::min(dt_temp, std::sqrt(2.0 * c.P.dx[d] / f[d]));
            dt = std::min(dt, std::min(1.e50, dt_temp));
        }
        res->dt_estimate = dt;
        if (dt < prm->small_dt) {
            set_error("EstDt: dt < small_dt");
            return MADV_ERR_PARAM;
        }
        if (dt > prm->max_dt) dt = prm->max_dt;
        if (prm->fixed_dt != -1.0) dt = prm->fixed_dt;
        res->dt = dt;
        res->umax = umax;
        res->rel_eps = umax * 1.e-8;
        return MADV_OK;
    } catch (const Fail& f) {
        return f.code;
    }
}

long madv_last_launch_count(const madv_ctx* h) {
    if (!h) return -1;
    long n = h->c.launches;
    for (auto& f : h->fine) n += f->launches;
    return n;
}

int madv_ppm(madv_ctx* h, const madv_box* bx, const madv_fab* s, int comp, const madv_fab* u, const madv_fab* v,
             const madv_fab* w, int is_umac, const int* bc, const madv_fab* Ip, const madv_fab* Im, void* stream) {
    if (!h || !bx) return MADV_ERR_PARAM;
    Ctx& c = h->c;
    int n[3];
    for (int d = 0; d < 3; ++d) {
        n[d] = bx->hi[d] - bx->lo[d] + 1;
        if (n[d] <= 0) return MADV_ERR_LAYOUT;
    }
    const long need = ppm_box_scratch_doubles(n);
    if (need > c.box_scratch_n) {
        if (c.box_scratch) cudaFree(c.box_scratch);
        c.box_scratch = nullptr;
        c.box_scratch_n = 0;
        if (!cuda_ok(cudaMalloc(&c.box_scratch, sizeof(double) * need), "cudaMalloc(madv_ppm scratch)"))
            return MADV_ERR_CUDA;
        c.box_scratch_n = need;
    }
    c.launches = 0;
    return ppm_box_run(c.P, bx, s, comp, u, v, w, is_umac, bc, Ip, Im, c.box_scratch, (cudaStream_t)stream,
                       c.launches);
}

// ------------------------------------------------------------------ launch-shape autotuner
// The PPM forms the autotuner tries per level: three launches (slopes, interfaces, cell
// limiter), or the staged sweep kernel with a tile shape across x (D = 0) and across y / z.
struct PpmForm {
    int staged;
    int x_a, x_b, yz_a, yz_b;
};
static const PpmForm PPM_FORMS[] = {{0, 0, 0, 0, 0}, {1, 4, 2, 32, 2}, {1, 8, 2, 32, 1}, {1, 2, 2, 16, 2}, {1, 4, 4, 16, 4}};
constexpr int N_PPM_FORMS = (int)(sizeof(PPM_FORMS) / sizeof(PPM_FORMS[0]));

static void set_ppm_form(Ctx& c, int k) {
    const PpmForm& f = PPM_FORMS[k];
    c.staged_ppm = f.staged != 0;
    c.sweep_shape.clear();
    if (f.staged) {
        c.sweep_shape[0] = {f.x_a, f.x_b};
        c.sweep_shape[1] = {f.yz_a, f.yz_b};
        c.sweep_shape[2] = {f.yz_a, f.yz_b};
    }
}

static bool is_ppm_kernel(Ctx& c, const void* fn) {
    auto it = c.is_ppm_fn.find(fn);
    if (it != c.is_ppm_fn.end()) return it->second;
    const char* nm = nullptr;
    bool yes = false;
    if (cudaFuncGetName(&nm, fn) == cudaSuccess && nm)
        yes = std::strstr(nm, "k_dsvl") || std::strstr(nm, "k_ppm_face") || std::strstr(nm, "k_ppm_cell") ||
              std::strstr(nm, "k_ppm_sweep");
    return c.is_ppm_fn[fn] = yes;
}

// fold the timed launches of the current trial into the per-kernel totals (block-size
// trials) or the PPM kernels' total (PPM form trials)
static int tune_collect(Hier& H) {
    if (!cuda_ok(cudaDeviceSynchronize(), "cudaDeviceSynchronize")) return MADV_ERR_CUDA;
    for (auto* c : H.L) {
        if (c->tpb_trial || c->ppm_trial >= 0)
            for (auto& r : c->prof) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, r.e0, r.e1);
                if (c->tpb_trial) c->tune_ms[r.fn][c->tpb_trial] += ms;
                else if (is_ppm_kernel(*c, r.fn)) c->ppm_tune_ms[c->ppm_trial] += ms;
            }
        c->prof.clear();
        c->ev_next = 0;
    }
    return MADV_OK;
}

int madv_autotune_trial(madv_ctx* h, int threads) {
    if (!h || threads < 32 || threads > 1024 || threads % 32 != 0) {
        set_error("threads per block: a multiple of 32 in [32, 1024]");
        return MADV_ERR_PARAM;
    }
    Hier H = h->H();
    int rc = tune_collect(H);
    if (rc) return rc;
    for (auto* c : H.L) {
        c->tpb_trial = threads;
        c->ppm_trial = -1;
        c->profiling = true;
    }
    drop_graph(h);
    return MADV_OK;
}

int madv_autotune_ppm_trial(madv_ctx* h, int form) {
    if (!h || form < 0 || form >= N_PPM_FORMS) {
        set_error("madv_autotune_ppm_trial: form must be in [0, MADV_AUTOTUNE_PPM_FORMS)");
        return MADV_ERR_PARAM;
    }
    Hier H = h->H();
    int rc = tune_collect(H);
    if (rc) return rc;
    for (auto* c : H.L) {
        c->tpb_trial = 0;
        c->ppm_trial = form;
        set_ppm_form(*c, form);
        c->profiling = true;
    }
    drop_graph(h);
    return MADV_OK;
}

static void json_out(const std::string& js, char* buf, int len) {
    if (buf && len > 0) std::snprintf(buf, (size_t)len, "%s", js.c_str());
}

int madv_autotune_finish(madv_ctx* h, char* json, int len) {
    if (!h) return MADV_ERR_PARAM;
    Hier H = h->H();
    int rc = tune_collect(H);
    if (rc) return rc;
    std::string js = "{";
    bool first = true;
    for (auto* c : H.L) {
        for (auto& kv : c->tune_ms) {
            int best = 256;
            double bms = 1e300;
            for (auto& tv : kv.second)
                if (tv.second < bms) {
                    bms = tv.second;
                    best = tv.first;
                }
            c->tpb_choice[kv.first] = best;
            const char* nm = nullptr;
            if (cudaFuncGetName(&nm, kv.first) != cudaSuccess || !nm) continue;
            js += (first ? "\"L" : ", \"L") + std::to_string(c->lev) + " " + nm + "\": " + std::to_string(best);
            first = false;
        }
        if (!c->ppm_tune_ms.empty()) {  // the fastest PPM form of this level's box sizes
            int best = 0;
            double bms = 1e300;
            for (auto& kv : c->ppm_tune_ms)
                if (kv.second < bms) {
                    bms = kv.second;
                    best = kv.first;
                }
            c->ppm_form = best;
            set_ppm_form(*c, best);
            js += (first ? "\"L" : ", \"L") + std::to_string(c->lev) + " ppm_form\": " + std::to_string(best);
            first = false;
        } else if (c->ppm_trial >= 0) {
            set_ppm_form(*c, c->ppm_form >= 0 ? c->ppm_form : 0);
        }
        c->tune_ms.clear();
        c->ppm_tune_ms.clear();
        c->tpb_trial = 0;
        c->ppm_trial = -1;
        c->profiling = false;
    }
    js += "}";
    drop_graph(h);
    json_out(js, json, len);
    return (int)js.size() < len ? MADV_OK : MADV_ERR_PARAM;
}

int madv_autotune_apply(madv_ctx* h, const char* json) {
    if (!h || !json) return MADV_ERR_PARAM;
    std::map<std::string, int> tab;
    const char* p = json;
    while ((p = std::strchr(p, '"'))) {
        const char* q = std::strchr(p + 1, '"');
        if (!q) break;
        std::string key(p + 1, q);
        const char* colon = std::strchr(q, ':');
        if (!colon) break;
        tab[key] = std::atoi(colon + 1);
        p = colon + 1;
    }
    Hier H = h->H();
    for (auto* c : H.L) {
        c->tpb_by_name = tab;
        c->tpb_choice.clear();
        c->tpb_max.clear();
        auto it = tab.find("L" + std::to_string(c->lev) + " ppm_form");
        if (it != tab.end() && it->second >= 0 && it->second < N_PPM_FORMS) {
            c->ppm_form = it->second;
            set_ppm_form(*c, it->second);
        }
    }
    drop_graph(h);
    return MADV_OK;
}

int madv_set_option(madv_ctx* h, const char* key, int value) {
    if (!h || !key) return MADV_ERR_PARAM;
    Hier H = h->H();
    const std::string k(key);
    if (k == "staged_ppm") {
        for (auto* c : H.L) c->staged_ppm = value != 0;
    } else if (k == "component_streams") {
        for (auto* c : H.L) c->comp_streams = value != 0;
    } else if (k == "es_inline") {
        for (auto* c : H.L) c->es_inline = value != 0;
    } else if (k == "mg_block_cycle") {
        for (auto* c : H.L) c->mg_block_cycle = value != 0;
    } else if (k.rfind("sweep_tile_", 0) == 0 && k.size() == 13 && k[11] >= '0' && k[11] <= '2' &&
               (k[12] == 'a' || k[12] == 'b')) {
        if (value < 1 || value > 256) return MADV_ERR_PARAM;
        const int D = k[11] - '0';
        for (auto* c : H.L) {
            auto it = c->sweep_shape.find(D);
            std::array<int, 2> sh = it != c->sweep_shape.end() ? it->second
                                                             : (D == 0 ? std::array<int, 2>{4, 2}
                                                                       : std::array<int, 2>{32, 2});
            sh[k[12] == 'a' ? 0 : 1] = value;
            c->sweep_shape[D] = sh;
        }
    } else {
        set_error("madv_set_option: unknown option " + k);
        return MADV_ERR_PARAM;
    }
    drop_graph(h);
    return MADV_OK;
}

int madv_profile(madv_ctx* h, int enable) {
    if (!h) return MADV_ERR_PARAM;
    Hier H = h->H();
    for (auto* c : H.L) {
        c->profiling = enable != 0;
        c->prof.clear();
        c->ev_next = 0;
    }
    return MADV_OK;
}

int madv_profile_report(madv_ctx* h, char* buf, int len) {
    if (!h || !buf || len <= 0) return MADV_ERR_PARAM;
    Hier H = h->H();
    if (!cuda_ok(cudaDeviceSynchronize(), "cudaDeviceSynchronize")) return MADV_ERR_CUDA;
    std::map<std::string, std::pair<long, double>> agg;
    std::vector<Ctx::ProfRec> recs;
    for (auto* c : H.L) recs.insert(recs.end(), c->prof.begin(), c->prof.end());
    for (auto& r : recs) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r.e0, r.e1);
        const char* name = nullptr;
        if (cudaFuncGetName(&name, r.fn) != cudaSuccess || !name) name = "?";
        auto& a = agg[name];
        a.first += 1;
        a.second += ms;
    }
    std::string js = "{";
    bool first = true;
    for (auto& kv : agg) {
        char tmp[512];
        std::snprintf(tmp, sizeof(tmp), "%s\"%s\": [%ld, %.6f]", first ? "" : ", ", kv.first.c_str(), kv.second.first,
                      kv.second.second);
        js += tmp;
        first = false;
    }
    js += "}";
    std::snprintf(buf, (size_t)len, "%s", js.c_str());
    return (int)js.size() < len ? MADV_OK : MADV_ERR_PARAM;
}

// Multi-step forward s_{n+1} = Stage(uold, s_n) with the velocity held fixed, J = <weight,
// s_N>, and the reverse sweep dJ/ds_0.  States are stored every ckpt_interval steps; each
// block of steps is recomputed from its stored state (keeping the block's states and
// edge states), then reversed step by step.  The last block's states are kept by the
// first forward pass.
static int stage_adjoint(madv_ctx* h, const madv_adj_seed* sd, madv_adj_result* res, void* stream) {
    Hier H;
    int rc = begin_call(h, stream, H);
    if (rc) return rc;
    Ctx& c = h->c;
    if (!sd || !res || !sd->uold || !sd->sold0 || !sd->weight || sd->nsteps < 1 || sd->ckpt_interval < 1) {
        set_error("madv_stage_adjoint: uold, sold0, weight, nsteps >= 1 and ckpt_interval >= 1 are required");
        return MADV_ERR_PARAM;
    }
    if (c.ndim != 3 || (c.P.ppm_type != 1 && c.P.ppm_type != 2) || c.P.species_pred_type != 1 ||
        c.P.enthalpy_pred_type != 1 || c.P.ppm_trace_forces) {
        set_error("the adjoint covers 3-D domains with ppm_type 1 or 2, species_pred_type 1, enthalpy_pred_type 1 "
                  "and untraced forces");
        return MADV_ERR_UNSUPPORTED;
    }
    // ppm_type 2: the state gradient away from walls (their boundary stencils are not transposed)
    if (c.P.ppm_type == 2) {
        bool wall = false;
        for (int d = 0; d < 3; ++d)
            for (int pb : {c.P.phys_bc_lo[d], c.P.phys_bc_hi[d]}) wall |= pb == PB_SLIPWALL || pb == PB_NOSLIPWALL;
        if (wall || res->grad_u) {
            set_error("the ppm_type 2 adjoint covers the state gradient on periodic, outflow and symmetry boundaries");
            return MADV_ERR_UNSUPPORTED;
        }
    }
    // physical boundaries: outflow, symmetry and walls (the traced fields' ghost cells are
    // copies, BCS_F; walls' hoextrap scalar BCs select PPM's boundary stencils); inflow's
    // ext_dir scalars are not covered; the velocity gradient needs a periodic domain
    for (int d = 0; d < 3; ++d)
        for (int pb : {c.P.phys_bc_lo[d], c.P.phys_bc_hi[d]}) {
            if (pb == PB_INTERIOR) continue;
            if (pb == PB_INFLOW || res->grad_u) {
                set_error("the adjoint covers periodic, outflow, symmetry and wall boundaries (the velocity "
                          "gradient periodic ones only)");
                return MADV_ERR_UNSUPPORTED;
            }
        }
    // buoyancy: with gravity the MAC velocity depends on the density through MakeVelForce, so
    // every reverse step carries the MAC-velocity adjoint back to the density (state
    // gradient; the force's ghost fill is transposed for periodic, outflow and symmetry faces)
    bool buoy = false;
    for (double v : c.h1.at("grav_cell")) buoy |= v != 0.0;
    if (buoy) {
        bool wall = false;
        for (int d = 0; d < 3; ++d)
            for (int pb : {c.P.phys_bc_lo[d], c.P.phys_bc_hi[d]}) wall |= pb == PB_SLIPWALL || pb == PB_NOSLIPWALL;
        if (wall || res->grad_u) {
            set_error("with gravity the adjoint covers the state gradient on periodic, outflow and symmetry "
                      "boundaries");
            return MADV_ERR_UNSUPPORTED;
        }
    }
    if (res->grad_u)
        for (double v : c.h1.at("w0"))
            if (v != 0.0) {
                set_error("the adjoint's velocity gradient needs w0 = 0");
                return MADV_ERR_UNSUPPORTED;
            }
    const int ns = c.nscal, K = sd->ckpt_interval, N = sd->nsteps;
    const int nck = (N + K - 1) / K;
    const int last0 = (nck - 1) * K;  // first step of the last block
    const bool want_u = res->grad_u != nullptr;
    const bool rev = res->grad_s != nullptr || want_u;
    const bool need_u = want_u || (buoy && rev);  // the scalar transposes accumulate the MAC-velocity adjoint
    const cudaMemcpyKind DD = cudaMemcpyDeviceToDevice;
    AdjWork W;
    const size_t st_b = fab_doubles(c, ns, 0, -1) * sizeof(double);
    double* wsold = W.alloc(st_b);
    double* wsnew = W.alloc(st_b);
    std::vector<madv_fab> fo, fn;
    bind_raw(c, A_WSOLD, wsold, ns, 0, -1, &fo);
    bind_raw(c, A_WSNEW, wsnew, ns, 0, -1, &fn);
    const madv_multifab mso{c.nb, fo.data()}, msn{c.nb, fn.data()};
    StageIO io{sd->uold, &mso, nullptr, nullptr, &msn, nullptr, nullptr, nullptr, nullptr};
    io.sold_out = 0;
    std::vector<StageIO> ios{io};
    if ((rc = bind_stage(c, io))) return rc;
    if ((rc = bind(c, A_SOLD0, sd->sold0, ns, -1, 0)) || (rc = bind(c, A_WEIGHT, sd->weight, ns, -1, 0)) ||
        (rc = bind(c, A_SFIN, res->sfinal, ns, -1, 0)) || (rc = bind(c, A_GRADS, res->grad_s, ns, -1, 0)) ||
        (rc = bind(c, A_GRADU, res->grad_u, 3, -1, 0)))
        return rc;
    std::vector<double*> ck, bst;
    std::vector<std::array<double*, 3>> bed;
    double *asold = nullptr, *scr = nullptr, *dir = nullptr, *atc = nullptr, *avelf = nullptr;
    std::array<double*, 3> aumac{};
    std::array<size_t, 3> aumac_b{};
    size_t scr_b = 0, dir_b = 0, atc_b = 0, avelf_b = 0, n_2 = 0;
    if (rev) {
        for (int j = 0; j < nck; ++j) ck.push_back(W.alloc(st_b));
        for (int j = 0; j < std::min(K, N); ++j) {
            bst.push_back(W.alloc(st_b));
            std::array<double*, 3> e;
            for (int d = 0; d < 3; ++d) e[d] = W.alloc(c.F[F_SEDGE0 + d].bytes);
            bed.push_back(e);
        }
        asold = W.alloc(st_b);
        bind_raw(c, A_ASOLD, asold, ns, 0, -1);
        bind_raw(c, A_ASNEW, W.alloc(st_b), ns, 0, -1);
        for (int d = 0; d < 3; ++d) bind_raw(c, A_AEDGE0 + d, W.alloc(fab_doubles(c, ns, 0, d) * 8), ns, 0, d);
        // per-component scratch in one block, cleared per component: A_AS, A_AFORCE,
        // A_ASL0 .. A_ASIMH2, A_AQ01 .. A_AQ21 (one component each; the velocity transpose
        // rebinds A_ASL0 .. A_ASIMH2 to three-component storage)
        const size_t n_as = fab_doubles(c, 1, c.ng_s, -1), n_f = fab_doubles(c, 1, 1, -1);
        n_2 = fab_doubles(c, 1, 2, -1);
        scr_b = (n_as + n_f + 15 * n_2) * sizeof(double);
        scr = W.alloc(scr_b);
        bind_raw(c, A_AS, scr, 1, c.ng_s, -1);
        bind_raw(c, A_AFORCE, scr + n_as, 1, 1, -1);
        double* p = scr + n_as + n_f;
        for (int s = A_ASL0; s <= A_AQ21; ++s, p += n_2) bind_raw(c, s, p, 1, 2, -1);
        dir_b = 3 * n_2 * sizeof(double);
        dir = W.alloc(dir_b);
        for (int s = A_ASM; s <= A_ADSVL; ++s) bind_raw(c, s, dir + (size_t)(s - A_ASM) * n_2, 1, 2, -1);
        if (need_u) {
            for (int d = 0; d < 3; ++d) {
                aumac_b[d] = fab_doubles(c, 1, 1, d) * 8;
                aumac[d] = W.alloc(aumac_b[d]);
                bind_raw(c, A_AUMAC0 + d, aumac[d], 1, 1, d);
            }
            atc_b = fab_doubles(c, 6, 2, -1) * 8;
            atc = W.alloc(atc_b);
            bind_raw(c, A_ATCOEF, atc, 6, 2, -1);
        }
        if (want_u) {
            for (int d = 0; d < 3; ++d) bind_raw(c, A_AUTRANS0 + d, W.alloc(fab_doubles(c, 1, 1, d) * 8), 1, 1, d);
            bind_raw(c, A_AUT, W.alloc(fab_doubles(c, 3, c.ng_adv, -1) * 8), 3, c.ng_adv, -1);
        }
        if (buoy) {
            avelf_b = fab_doubles(c, 3, 1, -1) * 8;
            avelf = W.alloc(avelf_b);
            bind_raw(c, A_AVELF, avelf, 3, 1, -1);
        }
    }
    // the forward's PPM interface values of every traced component of the block's steps
    // (F_FACE0..2) and, with the velocity gradient, its transverse states (F_Q01..F_Q21,
    // F_SIMH0..2), kept as the forward forms them
    static const int TAPE_F[12] = {F_FACE0, F_FACE1, F_FACE2, F_Q01, F_Q02, F_Q10,
                                   F_Q12,   F_Q20,   F_Q21,   F_SIMH0, F_SIMH1, F_SIMH2};
    const int ntape = need_u ? 12 : 3;
    std::vector<std::vector<std::array<double*, 12>>> tape;
    if (rev) {
        tape.resize(std::min(K, N));
        for (auto& t : tape) {
            t.resize(ns);
            for (int comp = 0; comp < ns; ++comp) {
                if (comp == TEMP || comp == PI) continue;
                for (int f = 0; f < ntape; ++f) t[comp][f] = W.alloc(c.F[TAPE_F[f]].bytes);
            }
        }
    }
    // Device view tables, one per (block step, component): the level's table with the taped
    // fields pointing at that step's and component's storage (same layout as the field).
    // Kernels take the table at launch, so the forward writes the taped fields straight
    // into the tape and the reverse reads them from there: nothing is copied.
    FabView* const base_views = c.dviews;
    struct ViewsGuard {
        Ctx& c;
        FabView* v;
        ~ViewsGuard() {
            c.dviews = v;
            c.edge_tape_begin = nullptr;
            c.edge_tape = nullptr;
        }
    } views_guard{c, base_views};
    std::vector<std::vector<FabView*>> vt(tape.size(), std::vector<FabView*>(ns, nullptr));
    // With w0 != 0 the stage ends with umac - w0 in F_UMAC, while the edge states and fluxes
    // saw umac + w0 (the density and the enthalpy halves each form it once).  Without gravity
    // the velocity is the same in every step: the first taped forward step keeps both, and
    // the reverse steps put them back, so every upwind and tracing decision is the
    // forward's.  With gravity the MAC velocity is the step's own: every taped step keeps
    // its pair.
    bool has_w0 = false;
    for (double v : c.h1.at("w0")) has_w0 |= v != 0.0;
    const bool keep_per_step = buoy;
    const bool keeps = has_w0 || keep_per_step;
    std::vector<std::array<std::array<double*, 3>, 2>> umac_keep(keep_per_step ? std::min(K, N) : 1);
    if (rev && keeps)
        for (auto& pair : umac_keep)
            for (auto& a : pair)
                for (int d = 0; d < 3; ++d) a[d] = W.alloc(c.F[F_UMAC0 + d].bytes);
    auto keep_umac = [&](int slot, int which) {
        auto& a = umac_keep[keep_per_step ? slot : 0][which];
        for (int d = 0; d < 3; ++d)
            cudaMemcpyAsync(a[d], c.F[F_UMAC0 + d].base, c.F[F_UMAC0 + d].bytes, DD, c.stream);
    };
    auto put_umac = [&](int slot, int which) {
        if (!keeps) return;
        auto& a = umac_keep[keep_per_step ? slot : 0][which];
        for (int d = 0; d < 3; ++d)
            cudaMemcpyAsync(c.F[F_UMAC0 + d].base, a[d], c.F[F_UMAC0 + d].bytes, DD, c.stream);
        edge_scal_coeffs(c);
    };
    bool umac_kept = false;
    auto tape_on = [&](int slot) {
        if (!rev) return;
        c.edge_tape_begin = [&, slot](int comp) {
            if (keeps && (keep_per_step || !umac_kept) && (comp == FIRSTSPEC || comp == RHOH)) {
                keep_umac(slot, comp == RHOH ? 1 : 0);
                umac_kept = comp == RHOH;
            }
            c.dviews = vt[slot][comp];
        };
        c.edge_tape = [&](int) { c.dviews = base_views; };
    };
    auto tape_off = [&]() {
        c.edge_tape_begin = nullptr;
        c.edge_tape = nullptr;
    };
    double* dJ = W.alloc(sizeof(double));
    double* dpart = W.alloc(sizeof(double) * (size_t)adj_dot_parts(c));
    if ((rc = upload_user_views(c))) return rc;
    if (rev) {
        const size_t nv = (size_t)NF_TOTAL * c.nb;
        std::vector<FabView> h(nv);
        for (size_t sl = 0; sl < tape.size(); ++sl)
            for (int comp = 0; comp < ns; ++comp) {
                if (comp == TEMP || comp == PI) continue;
                std::memcpy(h.data(), c.hviews_pinned, nv * sizeof(FabView));
                for (int f = 0; f < ntape; ++f) {
                    const int fid = TAPE_F[f];
                    for (int b = 0; b < c.nb; ++b) {
                        FabView& v = h[(size_t)fid * c.nb + b];
                        v.p = tape[sl][comp][f] + (v.p - c.F[fid].base);
                    }
                }
                FabView* d = reinterpret_cast<FabView*>(W.alloc(nv * sizeof(FabView)));
                CK(cudaMemcpy(d, h.data(), nv * sizeof(FabView), cudaMemcpyHostToDevice));
                vt[sl][comp] = d;
            }
    }

    auto fwd_step = [&]() {
        stage_body(H, ios);
        copy_fab(c, F_USER + A_WSOLD, RHO, F_USER + A_WSNEW, RHO, 2, 0);
        copy_fab(c, F_USER + A_WSOLD, FIRSTSPEC, F_USER + A_WSNEW, FIRSTSPEC, c.nspec, 0);
    };
    auto keep_step = [&](int slot) {  // state and edge states of the step about to run / just run
        cudaMemcpyAsync(bst[slot], wsold, st_b, DD, c.stream);
    };
    auto keep_edges = [&](int slot) {
        for (int d = 0; d < 3; ++d)
            cudaMemcpyAsync(bed[slot][d], c.F[F_SEDGE0 + d].base, c.F[F_SEDGE0 + d].bytes, DD, c.stream);
    };
    auto rev_step = [&](int slot) {
        // the step's traced fields (X, rho', rhoh') as the forward formed them
        copy_fab(c, F_SOLD, 0, F_USER + A_WSOLD, 0, ns, 0);
        fill_patch_h(H, F_SOLD, 0, ns, BCS_S, 0, 0, 0);
        convert_rhox_to_x_h(H, 1);
        put_in_pert_form_h(H, "rho0_old", RHO, 0, BCS_F, 1);
        put_in_pert_form_h(H, "rhoh0_old", RHOH, 0, BCS_F, 1);
        edge_scal_coeffs(c);
        put_umac(slot, 0);  // the density half's MAC velocity (w0 != 0, or gravity)
        if (buoy) {  // this step's MAC-velocity adjoint only
            for (int d = 0; d < 3; ++d) cudaMemsetAsync(aumac[d], 0, aumac_b[d], c.stream);
            cudaMemsetAsync(atc, 0, atc_b, c.stream);
        }
        // spherical: the face base state of the density fluxes (which_step 1: rho0_old for
        // both of MakeRhoXFlux's old and new)
        if (c.sph) {
            make_s0mac_h(H, "rho0_old", F_S0MAC0);
            make_s0mac_h(H, "rho0_old", F_S0MACB0);
        }
        adj_update(c);
        adj_flux(c, need_u);
        if (need_u) {
            // the spherical (rho h) flux's face-velocity term, on the faces it was formed with
            if (c.sph) {
                rhoh_face_base_h(H, 1);
                adj_flux_rhoh_u_sph(c);
            }
            // MakeRhoHForce's and ModifyScalForce's fields (which_step 1: p0_old, rho0_old,
            // rhoh0_old), then the final (rho h) force's face-velocity term (rhoh_new = ... + dt f)
            put1d_h(H, F_P0CART, "p0_old", 0, 1, 0, BCS_F, 0, 0, -1);
            put1d_h(H, F_RHO0CART, "rho0_old", 0, 1, 0, BCS_S, RHO, 0, RHO);
            if (c.sph) {
                make_s0mac_h(H, "p0_old", F_S0MAC0);
                put1d_h(H, F_RHOH0CART, "rhoh0_old", 0, 1, 0, BCS_S, RHOH, 0, RHOH);
            } else {
                put1d_h(H, F_GRAVCART, "grav_cell", c.ndim - 1, c.ndim, 0, BCS_F, 0, 0, -1);
            }
            adj_rhoh_force_u(c, A_ASNEW, RHOH, c.P.dt);
        }
        for (int comp = 0; comp < ns; ++comp) {
            if (comp == TEMP || comp == PI) continue;
            cudaMemsetAsync(scr, 0, scr_b, c.stream);
            if (comp == RHOH) put_umac(slot, 1);  // the enthalpy half's (w0 != 0, or gravity)
            // this component's interface values (and for the velocity adjoint its
            // transverse states) as the forward formed them, read from the tape
            c.dviews = vt[slot][comp];
            adj_edge_scal(c, F_SOLD, comp, comp >= FIRSTSPEC, dir, dir_b, need_u);
            c.dviews = base_views;
            // the traced field's and the force's FillPatch (BCS_F, the BC entries the
            // forward's fills read), transposed
            const BCRecD* bf = bcs_host(c, BCS_F);
            adj_phys_fill(c, A_AS, 0, c.ng_s, bf[comp >= FIRSTSPEC ? comp - FIRSTSPEC : 0]);
            adj_fill_boundary(c, A_AS, 1, c.ng_s, -1);
            if (comp >= FIRSTSPEC) {
                adj_convert_x(c, comp);
            } else {
                adj_phys_fill(c, A_AFORCE, 0, 1, bf[0]);
                adj_fill_boundary(c, A_AFORCE, 1, 1, -1);
                adj_pert_force(c, comp, need_u);
                if (need_u && c.sph) adj_pert_u_sph(c, comp, comp == RHO ? F_RHO0CART : F_RHOH0CART);
                if (need_u && comp == RHOH) adj_rhoh_force_u(c, A_AFORCE, 0, 1.0);  // the traced force's
            }
            if (comp == RHOH) put_umac(slot, 0);
        }
        if (buoy) {
            // the step's MAC-velocity adjoint onto its valid faces (transverse coefficients,
            // then the ghost faces), then through the force into the density: AdvancePremac's
            // fields of this step recomputed from its state
            adj_tcoef(c, A_AUMAC0);
            adj_umac_ghosts(c);
            copy_fab(c, F_SOLD, 0, F_USER + A_WSOLD, 0, ns, 0);
            fill_patch_h(H, F_SOLD, 0, ns, BCS_S, 0, 0, 0);
            set_val(c, F_UTILDE, 0.0, 0, 3, c.ng_adv);
            copy_fab(c, F_UTILDE, 0, F_USER + U_UOLD, 0, 3, 0);
            advance_premac(H);
            cudaMemsetAsync(avelf, 0, avelf_b, c.stream);
            adj_vel_force(c);
        }
        copy_fab(c, F_USER + A_ASNEW, 0, F_USER + A_ASOLD, 0, ns, 0);
        cudaMemsetAsync(asold, 0, st_b, c.stream);
    };

    copy_fab(c, F_USER + A_WSOLD, 0, F_USER + A_SOLD0, 0, ns, 0);
    for (int n = 0; n < N; ++n) {
        if (rev && n % K == 0) CK(cudaMemcpyAsync(ck[n / K], wsold, st_b, DD, c.stream));
        if (rev && n >= last0) {
            keep_step(n - last0);
            tape_on(n - last0);
        }
        fwd_step();
        tape_off();
        if (rev && n >= last0) keep_edges(n - last0);
    }
    adj_dot(c, A_WEIGHT, A_WSOLD, ns, dpart, dJ);
    if (res->sfinal) copy_fab(c, F_USER + A_SFIN, 0, F_USER + A_WSOLD, 0, ns, 0);
    if (rev) {
        copy_fab(c, F_USER + A_ASNEW, 0, F_USER + A_WEIGHT, 0, ns, 0);
        for (int bk = nck - 1; bk >= 0; --bk) {
            const int n0 = bk * K, n1 = std::min(N, n0 + K);
            if (bk != nck - 1) {
                CK(cudaMemcpyAsync(wsold, ck[bk], st_b, DD, c.stream));
                for (int n = n0; n < n1; ++n) {
                    keep_step(n - n0);
                    tape_on(n - n0);
                    fwd_step();
                    tape_off();
                    keep_edges(n - n0);
                }
            }
            for (int n = n1 - 1; n >= n0; --n) {
                CK(cudaMemcpyAsync(wsold, bst[n - n0], st_b, DD, c.stream));
                for (int d = 0; d < 3; ++d)
                    CK(cudaMemcpyAsync(c.F[F_SEDGE0 + d].base, bed[n - n0][d], c.F[F_SEDGE0 + d].bytes, DD, c.stream));
                rev_step(n - n0);
            }
        }
        if (res->grad_s) copy_fab(c, F_USER + A_GRADS, 0, F_USER + A_ASNEW, 0, ns, 0);
        if (want_u) {
            // MAC-velocity adjoint of every step: the transverse coefficients, then the
            // ghost faces back to the valid faces they were copied from
            adj_tcoef(c, A_AUMAC0);
            for (int d = 0; d < 3; ++d) adj_fill_boundary(c, A_AUMAC0 + d, 1, 1, d);
            // AdvancePremac's fields (identical in every step), then its transpose
            copy_fab(c, F_SOLD, 0, F_USER + A_WSOLD, 0, ns, 0);
            fill_patch_h(H, F_SOLD, 0, ns, BCS_S, 0, 0, 0);
            set_val(c, F_UTILDE, 0.0, 0, 3, c.ng_adv);
            copy_fab(c, F_UTILDE, 0, F_USER + U_UOLD, 0, 3, 0);
            advance_premac(H);
            CK(cudaMemsetAsync(atc, 0, atc_b, c.stream));
            CK(cudaMemsetAsync(scr, 0, scr_b, c.stream));
            // three-component predictor / transverse adjoints of the velocity
            double* vs = W.alloc(27 * n_2 * sizeof(double));
            CK(cudaStreamSynchronize(c.stream));  // no launch in flight reads the views
            for (int s = A_ASL0; s <= A_ASIMH2; ++s) bind_raw(c, s, vs + (size_t)(s - A_ASL0) * 3 * n_2, 3, 2, -1);
            if ((rc = upload_user_views(c))) return rc;
            adj_vel_pred(c, dir, dir_b);
            adj_fill_boundary(c, A_AUT, 3, c.ng_adv, -1);
            copy_fab(c, F_USER + A_GRADU, 0, F_USER + A_AUT, 0, 3, 0);
        }
    }
    double Jh = 0.0;
    CK(cudaMemcpyAsync(&Jh, dJ, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    rc = finish(H);
    res->J = Jh;
    res->device_bytes = (long long)W.bytes;
    return rc;
}

int madv_stage_adjoint(madv_ctx* h, const madv_adj_seed* seed, madv_adj_result* res, void* stream) {
    try {
        return stage_adjoint(h, seed, res, stream);
    } catch (const Fail& f) {
        return f.code;
    }
}

}  // extern "C"
