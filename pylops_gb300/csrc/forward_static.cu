// Forward application that allocates nothing: kgb_kirchhoff_forward_static.
//
// The regular forward (kgb_kirchhoff_forward) keeps its scratch -- the model
// scaled by 2/v and the statistics of its magnitude (maximum, exponent
// histogram) that set the forward's fixed-point scale -- in buffers the
// operator allocated.  This entry point
// keeps the same scratch in the file-scope device array below instead, so the
// call itself never allocates device memory.  It is meant for callers that
// must not call cudaMalloc while they run: code working inside a fixed
// device-memory budget reserved at start-up, code whose device memory is owned
// by a caching allocator or memory pool that raw allocations would fragment,
// and latency-critical loops that cannot afford the device-wide
// synchronisation a cudaMalloc may imply.  Inputs (the operator's tables, the
// model) and the output (the data) are still the caller's.
//
// Limits and sharing:
//  * at most kStaticMaxImagePoints image points (4,194,304: 16 MiB of
//    float32); larger operators are rejected with KGB_ERR_VALUE;
//  * the array lives on every GPU on which the library's device code is
//    loaded and stays allocated until the process exits;
//  * every call on a GPU uses the same array: calls whose kernels overlap on
//    that GPU (for example on two streams) race and must be serialised by the
//    caller.  The scale block is cleared at the start of every call; the
//    scaled model is rewritten in full by every call;
//  * the array's device address is looked up (cudaGetSymbolAddress, with
//    the operator's device current) when an operator is created
//    (kgb_kirchhoff_create calls static_scratch_prepare), which is also when
//    a lazily loaded module places the array in device memory; the call
//    itself only reads the cached address.  Create the operator before any
//    stream capture.  A device reset (cudaDeviceReset, or the primary
//    context released and created again) invalidates the cached address
//    together with every operator of that device; operators created after
//    it look the address up again.
#include <cuda_runtime.h>

#include <mutex>

#include "kgb_internal.h"

namespace {

constexpr int64_t kStaticMaxImagePoints = (int64_t)1 << 22;
// scaled model (kStaticMaxImagePoints floats) followed by the forward's
// scale block (kgb::kScaleWords words), which therefore starts on a 256-byte
// boundary too
__device__ __align__(256) float g_forward_scratch[kStaticMaxImagePoints + 512];
static_assert(kgb::kScaleWords <= 512, "scale block does not fit the static scratch");

constexpr int kMaxDevices = 64;
float* g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

}  // namespace

namespace kgb {

// Look up the device address of g_forward_scratch on the current device and
// cache it for that device (host code may not use the symbol itself as a
// device pointer).  Called by kgb_kirchhoff_create with the operator's
// device current; every creation looks it up again, so a cache left stale by
// a device reset is replaced by the next operator created on that device.
int static_scratch_prepare() {
    int dev = 0;
    KGB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return KGB_OK;  // forward_static then refuses this device
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_forward_scratch);
    if (e != cudaSuccess) return cuda_error(e, "forward_static scratch: cudaGetSymbolAddress");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    g_scratch_ptr[dev] = static_cast<float*>(p);
    return KGB_OK;
}

}  // namespace kgb

namespace {

// The cached address for device `dev` (set when an operator was created there).
int scratch_for_device(int dev, float** out) {
    if (dev < 0 || dev >= kMaxDevices)
        return kgb::set_error(KGB_ERR_VALUE, "forward_static: device %d beyond the supported %d", dev, kMaxDevices);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    *out = g_scratch_ptr[dev];
    if (!*out) return kgb::set_error(KGB_ERR_STATE, "forward_static: no operator was created on device %d", dev);
    return KGB_OK;
}

}  // namespace

extern "C" int kgb_kirchhoff_forward_static(kgb_kirchhoff* op, const float* m_dev, float* d_dev, void* stream) {
    using kgb::set_error;
    if (!op) return set_error(KGB_ERR_STATE, "forward_static: null operator");
    if (!op->trav_ready) return set_error(KGB_ERR_STATE, "forward_static: traveltime tables not set");
    if (op->dynamic && !op->dyn_ready) return set_error(KGB_ERR_STATE, "forward_static: dynamic tables not set");
    if (!m_dev || !d_dev) return set_error(KGB_ERR_VALUE, "forward_static: null pointer");
    if (op->ni > kStaticMaxImagePoints)
        return set_error(KGB_ERR_VALUE,
                         "forward_static: %lld image points exceed the static scratch maximum of %lld; "
                         "use kgb_kirchhoff_forward",
                         (long long)op->ni, (long long)kStaticMaxImagePoints);
    int dev = 0;
    KGB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev != op->device)
        return set_error(KGB_ERR_STATE, "forward_static: current device %d is not the operator's device %d", dev,
                         op->device);
    float* scratch = nullptr;
    int rc = scratch_for_device(dev, &scratch);
    if (rc) return rc;
    kgb::KirchDev K = op->view();
    K.mv = scratch;
    K.absmax = reinterpret_cast<unsigned*>(scratch + kStaticMaxImagePoints);
    // the split accumulation keeps wide contributions in operator memory;
    // this entry point uses the carry accumulation, whose traces are the
    // same bit for bit, and no scratch beyond the static array
    K.split_ok = 0;
    K.wacc = nullptr;
    return kgb::launch_spread(K, op->dynamic, op->has_gate, m_dev, d_dev, op->h_dev, op->L, true,
                              (cudaStream_t)stream);
}
