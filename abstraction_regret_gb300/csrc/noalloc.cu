// gbfsm_nfa_run_static: the plain NFA batch launch (nfa_warp_kernel / nfa_bitmap_kernel)
// with its scratch taken from a fixed array in device memory instead of a caller-supplied
// workspace, so that a call performs no device allocation at all.
//
// The scratch is the file-scope array below, reserved when this module is loaded. At the
// first call on a device (with that device current) its address is looked up once with
// cudaGetSymbolAddress and cached; every call then hands that address to the kernel as
// its workspace. That first call is the set-up step: it loads the module and should come
// before any stream capture on the device. The cached address belongs to the device's
// context: after a cudaDeviceReset of that device it is stale, so the entry point must
// not be called again in that process.
//
// Nothing in the scratch has to start at zero: both kernels clear each warp's (or
// thread's) slice of it before use, so no memset is issued.
//
// There is one scratch array per device, shared by every call: two calls whose kernels
// overlap on the GPU (different streams, or different host threads without ordering)
// race on it and may return wrong verdicts. Calls must be ordered, e.g. on one stream.
#include <mutex>

#include "common.cuh"
#include "engine.hpp"

namespace gbfsm {
namespace {

constexpr int kStaticDevices = 64;
static __device__ __align__(256) uint8_t g_static_scratch[GBFSM_STATIC_SCRATCH_BYTES];

std::mutex g_static_mu;
void *g_static_ptr[kStaticDevices] = {nullptr};

// Device address of the scratch array on the current device (looked up once per device).
gbfsm_status static_scratch(void **out) {
    int dev = 0;
    GBFSM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kStaticDevices)
        return fail(GBFSM_UNSUPPORTED, "device ordinal %d above %d", dev, kStaticDevices - 1);
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (g_static_ptr[dev] == nullptr) {
        void *ptr = nullptr;
        const cudaError_t rc = cudaGetSymbolAddress(&ptr, g_static_scratch);
        if (rc != cudaSuccess || ptr == nullptr)
            return cuda_fail(rc == cudaSuccess ? cudaErrorInvalidSymbol : rc,
                             "cudaGetSymbolAddress(static scratch)");
        g_static_ptr[dev] = ptr;
    }
    *out = g_static_ptr[dev];
    return GBFSM_OK;
}

}  // namespace
}  // namespace gbfsm

extern "C" gbfsm_status gbfsm_nfa_run_static(const gbfsm_nfa_dev *nfa, const uint8_t *data,
                                             const int64_t *offsets, int32_t n_inputs,
                                             const gbfsm_plan *plan, int32_t *flags,
                                             int32_t *lens, int32_t *examined, void *stream) {
    using namespace gbfsm;
    if (!nfa) return fail(GBFSM_INVALID_ARG, "gbfsm_nfa_run_static: nfa descriptor is NULL");
    const size_t need = n_inputs > 0 ? gbfsm_nfa_workspace_bytes(nfa, n_inputs, plan) : 0;
    if (need > (size_t)GBFSM_STATIC_SCRATCH_BYTES)
        return fail(GBFSM_INVALID_ARG,
                    "gbfsm_nfa_run_static: this batch needs %zu bytes of scratch, above the "
                    "%zu-byte static scratch; use gbfsm_nfa_run with a workspace, or fewer "
                    "inputs per call",
                    need, (size_t)GBFSM_STATIC_SCRATCH_BYTES);
    void *scratch = nullptr;
    const gbfsm_status st = static_scratch(&scratch);
    if (st != GBFSM_OK) return st;
    return gbfsm_nfa_run(nfa, data, offsets, n_inputs, plan, flags, lens, examined, scratch,
                         (size_t)GBFSM_STATIC_SCRATCH_BYTES, stream);
}
