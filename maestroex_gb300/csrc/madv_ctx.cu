// Context, layout, base state and the C ABI of the scalar-advection stage library.
#include <cstdio>
#include <cstring>
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

struct Fail {
    int code;
};

// ------------------------------------------------------------------ region tables
static HBox valid_box(const Ctx& c, int b, int nodal) {
    HBox r = c.ba[b];
    if (nodal >= 0) r.hi[nodal] += 1;
    return r;
}

const RegionTable& region(Ctx& c, int glo0, int glo1, int glo2, int ghi0, int ghi1, int ghi2, int nodal, int slab) {
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

// FillBoundary copy list: every piece of a box's ghost region that lies in another box's
// valid region (after the periodic shift), minus the box's own valid region.
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
        for (int d = 0; d < 3; ++d) {
            gb.lo[d] -= ng;
            gb.hi[d] += ng;
        }
        for (int cbx = 0; cbx < c.nb; ++cbx) {
            HBox sv = valid_box(c, cbx, nodal);
            for (int sz = -1; sz <= 1; ++sz)
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
                        // subtract the destination's valid box: up to six disjoint pieces
                        HBox rem = r;
                        auto emit = [&](const HBox& p) {
                            CopyDesc cd{};
                            cd.dst_b = b;
                            cd.src_b = cbx;
                            for (int d = 0; d < 3; ++d) {
                                cd.lo[d] = p.lo[d];
                                cd.n[d] = p.hi[d] - p.lo[d] + 1;
                                cd.shift[d] = s[d] * len[d];
                            }
                            cd.start = start;
                            start += (long)cd.n[0] * cd.n[1] * cd.n[2];
                            t.h.push_back(cd);
                        };
                        for (int d = 0; d < 3; ++d) {
                            if (rem.lo[d] < vb.lo[d]) {
                                HBox p = rem;
                                p.hi[d] = std::min(rem.hi[d], vb.lo[d] - 1);
                                emit(p);
                                rem.lo[d] = vb.lo[d];
                            }
                            if (rem.hi[d] > vb.hi[d]) {
                                HBox p = rem;
                                p.lo[d] = std::max(rem.lo[d], vb.hi[d] + 1);
                                emit(p);
                                rem.hi[d] = vb.hi[d];
                            }
                            if (rem.lo[d] > rem.hi[d]) break;
                        }
                    }
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
    S(F_VELFORCE, 3, 1);
    S(F_SCALFORCE, c.nscal, 1);
    S(F_ETA, 1, 0, 2);
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
    if (c.graph_exec) cudaGraphExecDestroy(c.graph_exec);
    c.graph_exec = nullptr;
    c.graph_key.clear();
}

static std::vector<double> cell_to_edge(const std::vector<double>& cc) {
    // Maestro::CelltoEdge (Source/MaestroCelltoEdge.cpp:5-55), one level, one chunk
    const int nr = (int)cc.size();
    std::vector<double> e(nr + 1);
    for (int r = 0; r <= nr; ++r) {
        if (r == 0) e[r] = cc[r];
        else if (r == 1) e[r] = 0.5 * (cc[r - 1] + cc[r]);
        else if (r == nr) e[r] = cc[r - 1];
        else if (r == nr - 1) e[r] = 0.5 * (cc[r] + cc[r - 1]);
        else {
            double tmp = 7.0 / 12.0 * (cc[r] + cc[r - 1]) - 1.0 / 12.0 * (cc[r + 1] + cc[r - 2]);
            double lo = (cc[r - 1] < cc[r]) ? cc[r - 1] : cc[r];  // min(cc[r], cc[r-1])
            double hi = (cc[r] < cc[r - 1]) ? cc[r - 1] : cc[r];  // max(cc[r], cc[r-1])
            double t = (tmp < lo) ? lo : tmp;
            e[r] = (hi < t) ? hi : t;
        }
    }
    return e;
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
    U_SFLUX0, U_SFLUX1, U_SFLUX2, U_ETA, U_UTRANS0, U_UTRANS1, U_UTRANS2
};

// ------------------------------------------------------------------ stage pieces
static void w0_carts(Ctx& c) {
    // Put1dArrayOnCart(w0, w0_cart, true, true, bcs_u, 0, 1)  (Source/MaestroAdvance.cpp:326)
    set_val(c, F_W0CART, 0.0, 0, 3, 2);
    put1d(c, F_W0CART, c.b1("w0"), 2, 1);
    fill_patch(c, F_W0CART, 0, 3, BCS_U, 0, 1, -1);
    // Put1dArrayOnCart(w0_force, w0_force_cart, false, true, bcs_f, 0) (:341), evolve_base_state only
    set_val(c, F_W0FCART, 0.0, 0, 3, 1);
    if (c.P.evolve_base_state) {
        put1d(c, F_W0FCART, c.b1("w0_force"), 2, 0);
        fill_patch(c, F_W0FCART, 0, 3, BCS_F, 0, 0, -1);
    }
}

// Maestro::AdvancePremac (Source/MaestroAdvection.cpp:7-84) on the internal fields.
static void advance_premac(Ctx& c) {
    fill_patch(c, F_UTILDE, 0, 3, BCS_U, 0, 1, -1);
    set_val(c, F_UFULL, 0.0, 0, 3, c.ng_adv);
    copy_fab(c, F_UFULL, 0, F_W0CART, 0, 3, 0);
    fill_patch(c, F_UFULL, 0, 3, BCS_U, 0, 1, -1);
    add_fab(c, F_UFULL, F_UTILDE, 3, c.ng_adv);
    for (int d = 0; d < 3; ++d) set_val(c, F_UTRANS0 + d, 0.0, 0, 1, 1);
    make_utrans(c);
    make_vel_force(c);
    addw0(c, F_UTRANS0, 1.0);
    vel_pred(c);
}

// Maestro::DensityAdvance, which_step 1 (Source/MaestroDensityAdvance.cpp:6-243)
static void density_advance(Ctx& c) {
    const int spt = c.P.species_pred_type;
    set_val(c, F_SCALFORCE, 0.0, 0, c.nscal, 1);
    set_val(c, F_RHO0CART, 0.0, 0, 1, 1);
    put1d(c, F_RHO0CART, c.b1("rho0_old"), 0, 0);
    fill_patch(c, F_RHO0CART, 0, 1, BCS_S, RHO, 0, RHO);
    addw0(c, F_UMAC0, -1.0);
    if (spt == 1) modify_scal_force(c, RHO, c.b1("rho0_edge_old"), F_RHO0CART, 0);
    else if (spt == 3) modify_scal_force(c, RHO, c.b1("rho0_edge_old"), F_RHO0CART, 1);
    addw0(c, F_UMAC0, 1.0);
    if (spt == 1 || spt == 3) convert_rhox_to_x(c, 1);
    if (spt == 1) put_in_pert_form(c, c.b1("rho0_old"), RHO, 0, BCS_F, 1);
    make_edge_scal(c, FIRSTSPEC, c.nspec, BCS_S, spt == 2, 1);  // no force for X / rho X
    if (spt == 1 || spt == 3) make_edge_scal(c, RHO, 1, BCS_S, 0, 0);
    else sum_species_edges(c);
    if (spt == 1) put_in_pert_form(c, c.b1("rho0_old"), RHO, RHO, BCS_S, 0);
    if (spt == 1 || spt == 3) convert_rhox_to_x(c, 0);
    make_rhox_flux(c, c.b1("rho0_old"), c.b1("rho0_edge_old"), c.b1("rho0_old"), c.b1("rho0_edge_old"));
    set_val(c, F_SCALFORCE, 0.0, 0, c.nscal, 1);
    update_scal(c, FIRSTSPEC);
}

// Maestro::EnthalpyAdvance, which_step 1 (Source/MaestroEnthalpyAdvance.cpp:6-352)
static void enthalpy_advance(Ctx& c) {
    const int ept = c.P.enthalpy_pred_type;
    set_val(c, F_SCALFORCE, 0.0, 0, c.nscal, 1);
    addw0(c, F_UMAC0, -1.0);
    make_rhoh_force(c, 1, 1, 1);
    if (ept == 1) {
        set_val(c, F_RHOH0CART, 0.0, 0, 1, 1);
        put1d(c, F_RHOH0CART, c.b1("rhoh0_old"), 0, 0);
        fill_patch(c, F_RHOH0CART, 0, 1, BCS_S, RHOH, 0, RHOH);
        modify_scal_force(c, RHOH, c.b1("rhoh0_edge_old"), F_RHOH0CART, 0);
    }
    addw0(c, F_UMAC0, 1.0);
    if (ept == 1) put_in_pert_form(c, c.b1("rhoh0_old"), RHOH, 0, BCS_F, 1);
    make_edge_scal(c, RHOH, 1, BCS_S, ept == 0, 0);
    if (ept == 1) put_in_pert_form(c, c.b1("rhoh0_old"), RHOH, RHOH, BCS_S, 0);
    make_rhoh_flux(c, c.b1("rhoh0_old"), c.b1("rhoh0_edge_old"), c.b1("rhoh0_old"), c.b1("rhoh0_edge_old"));
    set_val(c, F_SCALFORCE, 0.0, RHOH, 1, 1);
    addw0(c, F_UMAC0, -1.0);
    make_rhoh_force(c, 0, 0, 1);
    addw0(c, F_UMAC0, 1.0);
    update_scal(c, RHOH);
}

static int check_ready_c(Ctx* c) {
    if (!c) return MADV_ERR_PARAM;
    if (!c->have_layout || !c->have_base) {
        set_error("madv_set_layout and madv_set_base_state must be called first");
        return MADV_ERR_STATE;
    }
    return MADV_OK;
}

struct StageIO {
    const madv_multifab *uold, *sold, *gpi, *thermal, *snew, *umac, *sedge, *sflux, *eta;
};

static int bind_stage(Ctx& c, const StageIO& io) {
    int rc;
    const int ngs = c.ng_s;
    if ((rc = bind(c, U_UOLD, io.uold, 3, -1, 0))) return rc;
    if ((rc = bind(c, U_SOLD, io.sold, c.nscal, -1, 0))) return rc;
    if ((rc = bind(c, U_GPI, io.gpi, 3, -1, 0))) return rc;
    if ((rc = bind(c, U_THERMAL, io.thermal, 1, -1, 0))) return rc;
    if ((rc = bind(c, U_SNEW, io.snew, c.nscal, -1, 0))) return rc;
    for (int d = 0; d < 3; ++d) {
        if (io.umac && (rc = bind(c, U_UMAC0 + d, &io.umac[d], 1, d, 0))) return rc;
        if (io.sedge && (rc = bind(c, U_SEDGE0 + d, &io.sedge[d], c.nscal, d, 0))) return rc;
        if (io.sflux && (rc = bind(c, U_SFLUX0 + d, &io.sflux[d], c.nscal, d, 0))) return rc;
    }
    if ((rc = bind(c, U_ETA, io.eta, 1, 2, 0))) return rc;
    (void)ngs;
    return upload_user_views(c);
}

// The whole stage on the internal fields, inputs already bound to user slots.
static void stage_body(Ctx& c, const StageIO& io) {
    if (!c.dry) cudaMemsetAsync(c.d_flag, 0, sizeof(int), c.stream);
    // inputs
    set_val(c, F_UTILDE, 0.0, 0, 3, c.ng_adv);
    copy_fab(c, F_UTILDE, 0, F_USER + U_UOLD, 0, 3, 0);
    copy_fab(c, F_SOLD, 0, F_USER + U_SOLD, 0, c.nscal, 0);
    fill_patch(c, F_SOLD, 0, c.nscal, BCS_S, 0, 0, 0);
    copy_fab(c, F_GPI, 0, F_USER + U_GPI, 0, 3, 0);
    set_val(c, F_THERMAL, 0.0, 0, 1, 1);
    if (io.thermal) copy_fab(c, F_THERMAL, 0, F_USER + U_THERMAL, 0, 1, 0);
    set_val(c, F_SNEW, 0.0, 0, c.nscal, c.ng_s);
    for (int d = 0; d < 3; ++d) {
        set_val(c, F_UMAC0 + d, 0.0, 0, 1, 1);
        set_val(c, F_SEDGE0 + d, 0.0, 0, c.nscal, 0);
        set_val(c, F_SFLUX0 + d, 0.0, 0, c.nscal, 0);
    }
    set_val(c, F_ETA, 0.0, 0, 1, 0);
    w0_carts(c);
    // STEP 3 and STEP 4 of Maestro::AdvanceTimeStep (Source/MaestroAdvance.cpp:359-548)
    advance_premac(c);
    addw0(c, F_UMAC0, 1.0);
    density_advance(c);
    addw0(c, F_UMAC0, -1.0);
    addw0(c, F_UMAC0, 1.0);
    enthalpy_advance(c);
    addw0(c, F_UMAC0, -1.0);
    // outputs (valid region)
    if (io.snew) {
        copy_fab(c, F_USER + U_SNEW, RHO, F_SNEW, RHO, 2, 0);
        copy_fab(c, F_USER + U_SNEW, FIRSTSPEC, F_SNEW, FIRSTSPEC, c.nspec, 0);
    }
    copy_fab(c, F_USER + U_SOLD, 0, F_SOLD, 0, c.nscal, 0);
    for (int d = 0; d < 3; ++d) {
        if (io.umac) copy_fab(c, F_USER + U_UMAC0 + d, 0, F_UMAC0 + d, 0, 1, 0);
        if (io.sedge) copy_fab(c, F_USER + U_SEDGE0 + d, 0, F_SEDGE0 + d, 0, c.nscal, 0);
        if (io.sflux) copy_fab(c, F_USER + U_SFLUX0 + d, 0, F_SFLUX0 + d, 0, c.nscal, 0);
    }
    if (io.eta) copy_fab(c, F_USER + U_ETA, 0, F_ETA, 0, 1, 0);
}

static int finish(Ctx& c) {
    int flag = 0;
    CK(cudaMemcpyAsync(&flag, c.d_flag, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    CK(cudaStreamSynchronize(c.stream));
    CK(cudaGetLastError());
    if (flag) {
        set_error("UpdateScal: a cell reached base_cutoff_density; the EOS reset is not implemented");
        return MADV_ERR_EOS;
    }
    return MADV_OK;
}

}  // namespace madv

using namespace madv;

cudaEvent_t Ctx::next_event() {
    if (ev_next == ev_pool.size()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        ev_pool.push_back(e);
    }
    return ev_pool[ev_next++];
}

struct madv_ctx {
    Ctx c;
};

static int check_ready(madv_ctx* h) { return h ? check_ready_c(&h->c) : MADV_ERR_PARAM; }

extern "C" {

const char* madv_last_error(void) { return g_err.c_str(); }
const char* madv_version(void) { return "maestro_adv 0.1 (sm_103a, FP64)"; }

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
        p->enthalpy_pred_type > 1) {
        set_error("species_pred_type must be 1..3, enthalpy_pred_type 0 or 1");
        return MADV_ERR_UNSUPPORTED;
    }
    if (p->ppm_trace_forces != 0 || p->use_exact_base_state != 0) {
        set_error("ppm_trace_forces and use_exact_base_state must be 0");
        return MADV_ERR_UNSUPPORTED;
    }
    if (!(p->dt > 0.0) || !(p->rel_eps >= 0.0)) {
        set_error("dt must be > 0 and rel_eps >= 0");
        return MADV_ERR_PARAM;
    }
    for (int d = 0; d < 3; ++d) {
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
    if (p->dom_lo[2] != 0) {
        set_error("the radial (z) domain must start at 0");
        return MADV_ERR_PARAM;
    }
    madv_ctx* h = new madv_ctx();
    Ctx& c = h->c;
    c.P = *p;
    c.nspec = p->nspec;
    c.nscal = 4 + p->nspec;
    c.ng_s = c.ng_adv = p->ppm_type == 2 ? 4 : 3;
    c.nr = p->dom_hi[2] - p->dom_lo[2] + 1;
    for (int d = 0; d < 3; ++d) c.per[d] = p->phys_bc_lo[d] == PB_INTERIOR;
    int rc = bc_setup(c);
    if (rc) {
        delete h;
        return rc;
    }
    BCRecD all[2 * MAX_SCAL + 3];
    for (int k = 0; k < c.nscal; ++k) all[k] = c.bcs_s[k];
    for (int k = 0; k < 3; ++k) all[c.nscal + k] = c.bcs_u[k];
    for (int k = 0; k < c.nscal; ++k) all[c.nscal + 3 + k] = c.bcs_f[k];
    if (!cuda_ok(cudaMalloc(&c.d_bcs, sizeof(BCRecD) * (2 * c.nscal + 3)), "cudaMalloc") ||
        !cuda_ok(cudaMemcpy(c.d_bcs, all, sizeof(BCRecD) * (2 * c.nscal + 3), cudaMemcpyHostToDevice), "cudaMemcpy") ||
        !cuda_ok(cudaMalloc(&c.d_flag, sizeof(int)), "cudaMalloc")) {
        delete h;
        return MADV_ERR_CUDA;
    }
    field_specs(c);
    *out = h;
    return MADV_OK;
}

void madv_ctx_destroy(madv_ctx* h) {
    if (!h) return;
    Ctx& c = h->c;
    free_layout(c);
    for (auto& kv : c.d1) cudaFree(kv.second);
    for (auto e : c.ev_pool) cudaEventDestroy(e);
    if (c.box_scratch) cudaFree(c.box_scratch);
    if (c.d_bcs) cudaFree(c.d_bcs);
    if (c.d_flag) cudaFree(c.d_flag);
    delete h;
}

int madv_set_dt(madv_ctx* h, double dt, double rel_eps) {
    if (!h || !(dt > 0.0) || !(rel_eps >= 0.0)) return MADV_ERR_PARAM;
    h->c.P.dt = dt;
    h->c.P.rel_eps = rel_eps;
    if (h->c.graph_exec) cudaGraphExecDestroy(h->c.graph_exec);
    h->c.graph_exec = nullptr;
    h->c.graph_key.clear();
    return MADV_OK;
}

int madv_set_layout(madv_ctx* h, int nboxes, const madv_box* boxes) {
    if (!h || nboxes <= 0 || !boxes) return MADV_ERR_PARAM;
    Ctx& c = h->c;
    free_layout(c);
    c.have_layout = false;
    c.ba.assign(nboxes, HBox{});
    long vol = 0;
    for (int b = 0; b < nboxes; ++b) {
        for (int d = 0; d < 3; ++d) {
            c.ba[b].lo[d] = boxes[b].lo[d];
            c.ba[b].hi[d] = boxes[b].hi[d];
            if (boxes[b].lo[d] > boxes[b].hi[d] || boxes[b].lo[d] < c.P.dom_lo[d] || boxes[b].hi[d] > c.P.dom_hi[d]) {
                set_error("box " + std::to_string(b) + " is empty or outside the domain");
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
    if (vol != dvol) {
        set_error("a single-level layout must cover the domain");
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
            if (!cuda_ok(cudaMalloc(&c.F[f].base, c.F[f].bytes), "cudaMalloc(field)")) throw Fail{MADV_ERR_CUDA};
            if (!cuda_ok(cudaMemset(c.F[f].base, 0, c.F[f].bytes), "cudaMemset")) throw Fail{MADV_ERR_CUDA};
        }
        if (!cuda_ok(cudaMallocHost(&c.hviews_pinned, sizeof(FabView) * NF_TOTAL * c.nb), "cudaMallocHost"))
            throw Fail{MADV_ERR_CUDA};
        std::memset(c.hviews_pinned, 0, sizeof(FabView) * NF_TOTAL * c.nb);
        for (int f = 0; f < NF_INTERNAL; ++f) {
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

int madv_set_base_state(madv_ctx* h, const madv_base_state* bs) {
    if (!h || !bs) return MADV_ERR_PARAM;
    Ctx& c = h->c;
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
    c.h1["rho0_edge_old"] = cell_to_edge(c.h1["rho0_old"]);
    c.h1["rho0_edge_new"] = cell_to_edge(c.h1["rho0_new"]);
    c.h1["rhoh0_edge_old"] = cell_to_edge(c.h1["rhoh0_old"]);
    c.h1["rhoh0_edge_new"] = cell_to_edge(c.h1["rhoh0_new"]);
    for (auto& kv : c.h1) {
        double*& d = c.d1[kv.first];
        if (!d && !cuda_ok(cudaMalloc(&d, sizeof(double) * (nr + 1)), "cudaMalloc(base)")) return MADV_ERR_CUDA;
        if (!cuda_ok(cudaMemcpy(d, kv.second.data(), sizeof(double) * kv.second.size(), cudaMemcpyHostToDevice),
                     "cudaMemcpy(base)"))
            return MADV_ERR_CUDA;
    }
    c.have_base = true;
    return MADV_OK;
}

int madv_stage_forward(madv_ctx* h, int mode, const madv_multifab* uold, const madv_multifab* sold,
                       const madv_multifab* gpi, const madv_multifab* thermal, const madv_multifab* snew,
                       const madv_multifab* umac, const madv_multifab* sedge, const madv_multifab* sflux,
                       const madv_multifab* etarhoflux, void* stream) {
    int rc = check_ready(h);
    if (rc) return rc;
    Ctx& c = h->c;
    if (!uold || !sold || !gpi) {
        set_error("uold, sold and gpi are required");
        return MADV_ERR_PARAM;
    }
    if (mode < MADV_MODE_BATCHED || mode > MADV_MODE_GRAPH) return MADV_ERR_PARAM;
    c.stream = (cudaStream_t)stream;
    c.launches = 0;
    StageIO io{uold, sold, gpi, thermal, snew, umac, sedge, sflux, etarhoflux};
    try {
        if ((rc = bind_stage(c, io))) return rc;
        if (mode == MADV_MODE_GRAPH) {
            std::vector<const void*> key;
            const madv_multifab* all[] = {uold, sold, gpi, thermal, snew, etarhoflux};
            for (auto m : all) {
                key.push_back(m);
                if (m)
                    for (int b = 0; b < m->nfab; ++b) key.push_back(m->fab[b].p);
            }
            for (auto m3 : {umac, sedge, sflux}) {
                key.push_back(m3);
                if (m3)
                    for (int d = 0; d < 3; ++d)
                        for (int b = 0; b < m3[d].nfab; ++b) key.push_back(m3[d].fab[b].p);
            }
            if (!c.graph_exec || key != c.graph_key) {
                if (c.graph_exec) cudaGraphExecDestroy(c.graph_exec);
                c.graph_exec = nullptr;
                // a dry pass builds every region / copy table (no allocation may happen
                // while capturing), then the stage is captured
                c.per_box = 0;
                c.dry = true;
                stage_body(c, io);
                c.dry = false;
                cudaStream_t cs;
                CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
                cudaStream_t user = c.stream;
                c.stream = cs;
                c.launches = 0;
                cudaGraph_t g;
                CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
                upload_user_views(c);
                stage_body(c, io);
                CK(cudaStreamEndCapture(cs, &g));
                CK(cudaGraphInstantiate(&c.graph_exec, g, 0));
                cudaGraphDestroy(g);
                cudaStreamDestroy(cs);
                c.stream = user;
                c.graph_key = key;
                c.graph_launches = c.launches;
            }
            CK(cudaGraphLaunch(c.graph_exec, c.stream));
            c.launches = c.graph_launches;
            return finish(c);
        }
        c.per_box = mode == MADV_MODE_PER_BOX;
        stage_body(c, io);
        c.per_box = 0;
        return finish(c);
    } catch (const Fail& f) {
        return f.code;
    }
}

// ---- Maestro-shaped entry points: the same pieces, with the caller's FABs copied in and
// out around each call.
static int begin_call(madv_ctx* h, void* stream) {
    int rc = check_ready(h);
    if (rc) return rc;
    h->c.stream = (cudaStream_t)stream;
    h->c.launches = 0;
    h->c.per_box = 0;
    cudaMemsetAsync(h->c.d_flag, 0, sizeof(int), h->c.stream);
    return MADV_OK;
}

int madv_advance_premac(madv_ctx* h, const madv_multifab* uold, const madv_multifab* sold, const madv_multifab* gpi,
                        const madv_multifab* umac, const madv_multifab* utrans, void* stream) {
    int rc = begin_call(h, stream);
    if (rc) return rc;
    Ctx& c = h->c;
    if (!uold || !sold || !gpi || !umac) return MADV_ERR_PARAM;
    try {
        if ((rc = bind(c, U_UOLD, uold, 3, -1, 0)) || (rc = bind(c, U_SOLD, sold, 1, -1, 0)) ||
            (rc = bind(c, U_GPI, gpi, 3, -1, 0)))
            return rc;
        for (int d = 0; d < 3; ++d) {
            if ((rc = bind(c, U_UMAC0 + d, &umac[d], 1, d, 0))) return rc;
            if (utrans && (rc = bind(c, U_UTRANS0 + d, &utrans[d], 1, d, 0))) return rc;
        }
        if ((rc = upload_user_views(c))) return rc;
        set_val(c, F_UTILDE, 0.0, 0, 3, c.ng_adv);
        copy_fab(c, F_UTILDE, 0, F_USER + U_UOLD, 0, 3, 0);
        copy_fab(c, F_SOLD, RHO, F_USER + U_SOLD, RHO, 1, 0);
        copy_fab(c, F_GPI, 0, F_USER + U_GPI, 0, 3, 0);
        for (int d = 0; d < 3; ++d) set_val(c, F_UMAC0 + d, 0.0, 0, 1, 1);
        w0_carts(c);
        advance_premac(c);
        for (int d = 0; d < 3; ++d) {
            copy_fab(c, F_USER + U_UMAC0 + d, 0, F_UMAC0 + d, 0, 1, 0);
            if (utrans) copy_fab(c, F_USER + U_UTRANS0 + d, 0, F_UTRANS0 + d, 0, 1, 0);
        }
        return finish(c);
    } catch (const Fail& f) {
        return f.code;
    }
}

int madv_addw0(madv_ctx* h, const madv_multifab* umac, double mult, void* stream) {
    int rc = begin_call(h, stream);
    if (rc) return rc;
    Ctx& c = h->c;
    if (!umac) return MADV_ERR_PARAM;
    try {
        for (int d = 0; d < 3; ++d)
            if ((rc = bind(c, U_UMAC0 + d, &umac[d], 1, d, 1))) return rc;
        if ((rc = upload_user_views(c))) return rc;
        for (int d = 0; d < 3; ++d) copy_fab(c, F_UMAC0 + d, 0, F_USER + U_UMAC0 + d, 0, 1, 1);
        addw0(c, F_UMAC0, mult);
        for (int d = 0; d < 3; ++d) copy_fab(c, F_USER + U_UMAC0 + d, 0, F_UMAC0 + d, 0, 1, 1);
        return finish(c);
    } catch (const Fail& f) {
        return f.code;
    }
}

static int scalar_advance(madv_ctx* h, int which, int which_step, const madv_multifab* sold, const madv_multifab* snew,
                          const madv_multifab* sedge, const madv_multifab* sflux, const madv_multifab* eta,
                          const madv_multifab* umac, const madv_multifab* thermal, void* stream) {
    int rc = begin_call(h, stream);
    if (rc) return rc;
    Ctx& c = h->c;
    if (which_step != 1) {
        set_error("only which_step 1 (the predictor) is implemented");
        return MADV_ERR_UNSUPPORTED;
    }
    if (!sold || !snew || !umac) return MADV_ERR_PARAM;
    try {
        if ((rc = bind(c, U_SOLD, sold, c.nscal, -1, 0)) || (rc = bind(c, U_SNEW, snew, c.nscal, -1, 0)) ||
            (rc = bind(c, U_ETA, eta, 1, 2, 0)) || (rc = bind(c, U_THERMAL, thermal, 1, -1, 0)))
            return rc;
        for (int d = 0; d < 3; ++d) {
            if ((rc = bind(c, U_UMAC0 + d, &umac[d], 1, d, 1))) return rc;
            if (sedge && (rc = bind(c, U_SEDGE0 + d, &sedge[d], c.nscal, d, 0))) return rc;
            if (sflux && (rc = bind(c, U_SFLUX0 + d, &sflux[d], c.nscal, d, 0))) return rc;
        }
        if ((rc = upload_user_views(c))) return rc;
        copy_fab(c, F_SOLD, 0, F_USER + U_SOLD, 0, c.nscal, 0);
        fill_patch(c, F_SOLD, 0, c.nscal, BCS_S, 0, 0, 0);
        copy_fab(c, F_SNEW, 0, F_USER + U_SNEW, 0, c.nscal, 0);
        for (int d = 0; d < 3; ++d) {
            copy_fab(c, F_UMAC0 + d, 0, F_USER + U_UMAC0 + d, 0, 1, 1);
            if (sedge) copy_fab(c, F_SEDGE0 + d, 0, F_USER + U_SEDGE0 + d, 0, c.nscal, 0);
            if (sflux) copy_fab(c, F_SFLUX0 + d, 0, F_USER + U_SFLUX0 + d, 0, c.nscal, 0);
        }
        set_val(c, F_THERMAL, 0.0, 0, 1, 1);
        if (thermal) copy_fab(c, F_THERMAL, 0, F_USER + U_THERMAL, 0, 1, 0);
        w0_carts(c);
        if (which == 0) {
            set_val(c, F_ETA, 0.0, 0, 1, 0);
            if (eta) copy_fab(c, F_ETA, 0, F_USER + U_ETA, 0, 1, 0);
            density_advance(c);
            copy_fab(c, F_USER + U_SNEW, RHO, F_SNEW, RHO, 1, 0);
            copy_fab(c, F_USER + U_SNEW, FIRSTSPEC, F_SNEW, FIRSTSPEC, c.nspec, 0);
            if (eta) copy_fab(c, F_USER + U_ETA, 0, F_ETA, 0, 1, 0);
        } else {
            enthalpy_advance(c);
            copy_fab(c, F_USER + U_SNEW, RHOH, F_SNEW, RHOH, 1, 0);
        }
        copy_fab(c, F_USER + U_SOLD, 0, F_SOLD, 0, c.nscal, 0);
        for (int d = 0; d < 3; ++d) {
            copy_fab(c, F_USER + U_UMAC0 + d, 0, F_UMAC0 + d, 0, 1, 1);
            if (sedge) copy_fab(c, F_USER + U_SEDGE0 + d, 0, F_SEDGE0 + d, 0, c.nscal, 0);
            if (sflux) copy_fab(c, F_USER + U_SFLUX0 + d, 0, F_SFLUX0 + d, 0, c.nscal, 0);
        }
        return finish(c);
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

long madv_last_launch_count(const madv_ctx* h) { return h ? h->c.launches : -1; }

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

int madv_profile(madv_ctx* h, int enable) {
    if (!h) return MADV_ERR_PARAM;
    h->c.profiling = enable != 0;
    h->c.prof.clear();
    h->c.ev_next = 0;
    return MADV_OK;
}

int madv_profile_report(madv_ctx* h, char* buf, int len) {
    if (!h || !buf || len <= 0) return MADV_ERR_PARAM;
    Ctx& c = h->c;
    if (!cuda_ok(cudaDeviceSynchronize(), "cudaDeviceSynchronize")) return MADV_ERR_CUDA;
    std::map<std::string, std::pair<long, double>> agg;
    for (auto& r : c.prof) {
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

}  // extern "C"
