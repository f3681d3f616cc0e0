// madv_ppm_noalloc: Maestro::PPM on one box without allocating any device memory.
//
// Who needs it.  Some callers cannot call cudaMalloc at the point where they run PPM:
// an AMReX application usually reserves most of the GPU's memory for its own arena at
// start-up, so a third-party cudaMalloc there fails or eats into what is left; and code
// that must stay asynchronous cannot afford the implicit device synchronisation that
// cudaMalloc / cudaFree perform.  madv_ppm grows its scratch with cudaMalloc; this entry
// point uses a static device array instead and allocates nothing.
//
// The scratch.  One file-scope static __device__ array of MADV_PPM_NOALLOC_MAX_DOUBLES
// doubles (9.04 MiB).  Every GPU that loads this library holds it until the process
// exits.  A box whose scratch need exceeds it is rejected with MADV_ERR_LAYOUT before
// anything runs; every box up to 66 x 66 x 66 cells fits (a 64^3 box grown by one cell,
// the box the reference passes to PPM).
//
// Host code cannot use the array's name as a device address.  The first call on each
// device, with that device current, looks the address up with cudaGetSymbolAddress and
// caches it; make that first call on a device before any stream capture.  The cached
// address belongs to the device's primary context: a process that resets a device
// (cudaDeviceReset) or otherwise destroys its primary context must not call this entry
// point on that device afterwards, because the cache would still hold the old address.
//
// Nothing in the array has to start at zero: every element a call reads was written
// earlier in the same call.  All calls share the array and it keeps the last call's
// contents, so calls that overlap on the GPU (on different streams, or from different
// host threads without ordering) race on it: order them on one stream.
#include <mutex>

#include "madv_ctx.hpp"

namespace madv {

static __device__ __align__(256) double g_ppm_noalloc_scratch[MADV_PPM_NOALLOC_MAX_DOUBLES];

constexpr int NOALLOC_MAX_DEVICES = 64;
static std::mutex g_noalloc_mu;
static double* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Device address of the static scratch on the current device (looked up once per device).
static int noalloc_scratch(double** out) {
    int dev = -1;
    if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return MADV_ERR_CUDA;
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        set_error("madv_ppm_noalloc: device index out of range");
        return MADV_ERR_PARAM;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        if (!cuda_ok(cudaGetSymbolAddress(&p, g_ppm_noalloc_scratch), "cudaGetSymbolAddress(madv_ppm_noalloc)"))
            return MADV_ERR_CUDA;
        g_noalloc_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return MADV_OK;
}

}  // namespace madv

using namespace madv;

extern "C" int madv_ppm_noalloc(const madv_params* params, const madv_box* bx, const madv_fab* s, int comp,
                                const madv_fab* u, const madv_fab* v, const madv_fab* w, int is_umac, const int* bc,
                                const madv_fab* Ip, const madv_fab* Im, void* stream) {
    if (!params || !bx) return MADV_ERR_PARAM;
    if (!(params->dt > 0.0) || !(params->rel_eps >= 0.0) || !(params->dx[0] > 0.0) || !(params->dx[1] > 0.0) ||
        !(params->dx[2] > 0.0)) {
        set_error("madv_ppm_noalloc: dt and dx must be > 0, rel_eps >= 0");
        return MADV_ERR_PARAM;
    }
    int n[3];
    for (int d = 0; d < 3; ++d) {
        n[d] = bx->hi[d] - bx->lo[d] + 1;
        if (n[d] <= 0) {
            set_error("madv_ppm_noalloc: empty box");
            return MADV_ERR_LAYOUT;
        }
    }
    const long need = ppm_box_scratch_doubles(n);
    if (need > (long)MADV_PPM_NOALLOC_MAX_DOUBLES) {
        set_error("madv_ppm_noalloc: the box needs " + std::to_string(need) + " doubles of scratch but the static " +
                  "array holds " + std::to_string((long)MADV_PPM_NOALLOC_MAX_DOUBLES) +
                  " (boxes up to 66 x 66 x 66 cells fit); use madv_ppm for larger boxes");
        return MADV_ERR_LAYOUT;
    }
    double* scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc != MADV_OK) return rc;
    long launches = 0;
    return ppm_box_run(*params, bx, s, comp, u, v, w, is_umac, bc, Ip, Im, scratch, (cudaStream_t)stream, launches);
}
