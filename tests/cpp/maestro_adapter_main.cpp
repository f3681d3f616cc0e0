// The scalar-advection part of Maestro::AdvanceTimeStep (Source/MaestroAdvance.cpp:359,
// 448-455, 541-548, MAC projection left out) written against the Maestro-shaped C++ layer of
// include/maestro_adv.hpp, i.e. the calls a reference-side caller keeps:
//
//   AdvancePremac(umac, w0mac, w0_force_cart);
//   Addw0(umac, w0mac, 1.0);
//   DensityAdvance(1, sold, snew, sedge, sflux, scal_force, etarhoflux, umac, w0mac, rho0_predicted_edge);
//   Addw0(umac, w0mac, -1.0);
//   Addw0(umac, w0mac, 1.0);
//   EnthalpyAdvance(1, sold, snew, sedge, sflux, scal_force, umac, w0mac, thermal);
//   Addw0(umac, w0mac, -1.0);
//
// Usage: maestro_adapter_main <input> <output>.  The input (little endian) holds
//   int32 sizeof(madv_params), the madv_params bytes,
//   int32 nboxes, nboxes x (lo[3], hi[3]) int32,
//   int32 nr, then rho0_old rho0_new rhoh0_old rhoh0_new p0_old p0_new psi grav_cell w0_force
//   (nr doubles each), w0 rho0_predicted_edge (nr+1 each),
//   then domain arrays [ncomp][nz][ny][nx] of doubles: uold (3), sold (4+nspec), gpi (3),
//   thermal (1).
// The output holds, as domain arrays: snew, sold (after the stage), umac[0..2] (faces, 1
// comp), sedge[0..2], sflux[0..2] (faces, 4+nspec comps), etarhoflux (z faces, 1 comp).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "maestro_adv.hpp"

using madvx::BoxArray;
using madvx::FaceMultiFabs;
using madvx::MultiFab;
using madvx::Vector;

namespace {

struct Reader {
    FILE* f;
    template <class T>
    T one() {
        T v;
        if (std::fread(&v, sizeof(T), 1, f) != 1) throw std::runtime_error("short input");
        return v;
    }
    template <class T>
    std::vector<T> many(size_t n) {
        std::vector<T> v(n);
        if (n && std::fread(v.data(), sizeof(T), n, f) != n) throw std::runtime_error("short input");
        return v;
    }
};

void put(FILE* f, const std::vector<double>& v) {
    if (std::fwrite(v.data(), sizeof(double), v.size(), f) != v.size()) throw std::runtime_error("short write");
}

std::vector<double> gather(const MultiFab& mf, const int n[3], int nodal) {
    size_t pts = 1;
    for (int d = 0; d < 3; ++d) pts *= (size_t)(n[d] + (d == nodal ? 1 : 0));
    std::vector<double> h(pts * mf.nComp(), 0.0);
    mf.to_domain(h.data(), n);
    return h;
}

int run(const char* in_path, const char* out_path) {
    FILE* fi = std::fopen(in_path, "rb");
    if (!fi) throw std::runtime_error("cannot open input");
    Reader r{fi};
    if (r.one<int>() != (int)sizeof(madv_params)) throw std::runtime_error("madv_params size mismatch");
    madv_params p = r.one<madv_params>();
    const int nboxes = r.one<int>();
    BoxArray grids(nboxes);
    for (auto& b : grids) {
        for (int d = 0; d < 3; ++d) b.lo[d] = r.one<int>();
        for (int d = 0; d < 3; ++d) b.hi[d] = r.one<int>();
    }
    const int nr = r.one<int>();
    std::vector<std::vector<double>> bsa;
    for (int a = 0; a < 9; ++a) bsa.push_back(r.many<double>(nr));
    for (int a = 0; a < 2; ++a) bsa.push_back(r.many<double>(nr + 1));
    const madv_base_state bs{bsa[0].data(), bsa[1].data(), bsa[2].data(), bsa[3].data(), bsa[4].data(), bsa[5].data(),
                             bsa[6].data(), bsa[7].data(), bsa[8].data(), bsa[9].data(), bsa[10].data()};
    const int n[3] = {p.dom_hi[0] - p.dom_lo[0] + 1, p.dom_hi[1] - p.dom_lo[1] + 1, p.dom_hi[2] - p.dom_lo[2] + 1};
    const size_t ncell = (size_t)n[0] * n[1] * n[2];
    const int nscal = 4 + p.nspec;
    const int ng = p.ppm_type == 2 ? 4 : 3;  // ng_s
    auto uold_h = r.many<double>(3 * ncell);
    auto sold_h = r.many<double>(nscal * ncell);
    auto gpi_h = r.many<double>(3 * ncell);
    auto thermal_h = r.many<double>(ncell);
    std::fclose(fi);

    madvx::Maestro m(p, grids, bs);
    m.uold.emplace_back(grids, 3, ng);
    m.sold.emplace_back(grids, nscal, ng);
    m.gpi.emplace_back(grids, 3, 0);
    m.uold[0].setVal0();
    m.sold[0].setVal0();
    m.uold[0].from_domain(uold_h.data(), n);
    m.sold[0].from_domain(sold_h.data(), n);
    m.gpi[0].from_domain(gpi_h.data(), n);

    Vector<MultiFab> snew, thermal, etarhoflux, scal_force(1), w0_force_cart(1);
    snew.emplace_back(grids, nscal, ng);
    thermal.emplace_back(grids, 1, 1);
    etarhoflux.emplace_back(grids, 1, 0, 2);
    snew[0].setVal0();
    thermal[0].setVal0();
    etarhoflux[0].setVal0();
    thermal[0].from_domain(thermal_h.data(), n);
    Vector<FaceMultiFabs> umac(1), sedge(1), sflux(1), w0mac(1);
    for (int d = 0; d < 3; ++d) {
        umac[0][d].define(grids, 1, 1, d);
        sedge[0][d].define(grids, nscal, 0, d);
        sflux[0][d].define(grids, nscal, 0, d);
        umac[0][d].setVal0();
        sedge[0][d].setVal0();
        sflux[0][d].setVal0();
    }
    const madvx::BaseState<double> rho0_predicted_edge(bsa[10]);

    m.AdvancePremac(umac, w0mac, w0_force_cart);
    m.Addw0(umac, w0mac, 1.0);
    m.DensityAdvance(1, m.sold, snew, sedge, sflux, scal_force, etarhoflux, umac, w0mac, rho0_predicted_edge);
    m.Addw0(umac, w0mac, -1.0);
    m.Addw0(umac, w0mac, 1.0);
    m.EnthalpyAdvance(1, m.sold, snew, sedge, sflux, scal_force, umac, w0mac, thermal);
    m.Addw0(umac, w0mac, -1.0);
    madvx::check_cuda(cudaDeviceSynchronize());

    FILE* fo = std::fopen(out_path, "wb");
    if (!fo) throw std::runtime_error("cannot open output");
    put(fo, gather(snew[0], n, -1));
    put(fo, gather(m.sold[0], n, -1));
    for (int d = 0; d < 3; ++d) put(fo, gather(umac[0][d], n, d));
    for (int d = 0; d < 3; ++d) put(fo, gather(sedge[0][d], n, d));
    for (int d = 0; d < 3; ++d) put(fo, gather(sflux[0][d], n, d));
    put(fo, gather(etarhoflux[0], n, 2));
    std::fclose(fo);
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s <input> <output>\n", argv[0]);
        return 2;
    }
    try {
        return run(argv[1], argv[2]);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
}
