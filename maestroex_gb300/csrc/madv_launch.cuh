// Launch helper shared by the kernel files: one launch over the region pieces of every box
// (batched), or one launch per piece (the per-box form of the reference's MFIter loop).
#pragma once
#include "madv_ctx.hpp"

namespace madv {

#define KARGS const RegionBox *__restrict__ R, int ne, long g0, long g1, const FabView *__restrict__ V, int nb
#define VW(f) V[(f) * nb + b]

static constexpr int TPB = 256;

// One launch over every box (batched), or one launch per region piece (per-box mode, the
// MFIter + ParallelFor form of the reference).  Kernel arguments after the region are
// (V, nb, ...).  Threads per block: the kernel's autotuned value on this level.
template <typename Kern, typename... Args>
static inline void launch(Ctx& c, const RegionTable& rt, int gy, Kern kern, const FabView* V, Args... args) {
    const int tpb = c.tpb_of((const void*)kern);  // before a dry return: no attribute query while capturing
    if (rt.total == 0 || c.dry) return;
    const int ne = (int)rt.h.size();
    if (!c.per_box) {
        dim3 grid((unsigned)((rt.total + tpb - 1) / tpb), gy);
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (c.profiling) {
            e0 = c.next_event();
            e1 = c.next_event();
            cudaEventRecord(e0, c.stream);
        }
        kern<<<grid, tpb, 0, c.stream>>>(rt.d, ne, 0L, rt.total, V, c.nb, args...);
        if (c.profiling) {
            cudaEventRecord(e1, c.stream);
            c.prof.push_back({(const void*)kern, e0, e1});
        }
        c.launches++;
    } else {
        for (int e = 0; e < ne; ++e) {
            long s0 = rt.h[e].start;
            long s1 = (e + 1 < ne) ? rt.h[e + 1].start : rt.total;
            if (s1 <= s0) continue;
            dim3 grid((unsigned)((s1 - s0 + tpb - 1) / tpb), gy);
            kern<<<grid, tpb, 0, c.stream>>>(rt.d, ne, s0, s1, V, c.nb, args...);
            c.launches++;
        }
    }
}

// Region helpers: the valid box grown by g, and face boxes.
static inline const RegionTable& rg_grow(Ctx& c, int g, int nodal = -1) { return region(c, g, g, g, g, g, g, nodal); }

}  // namespace madv
