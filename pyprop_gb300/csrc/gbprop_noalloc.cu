// Allocation-free variant of the Arnoldi block inner product.
//
// Some callers cannot allocate device memory at the point where they need
// the block inner product: custom allocators or memory pools that call back
// into this library (allocating there would re-enter the allocator), and
// embedded or real-time hosts that hand the library only fixed buffers and
// allow no allocation after start-up.  gbprop_block_inner_product asks its caller
// for a workspace; this entry point instead uses the fixed scratch array
// below, so it calls no cudaMalloc, cudaFree or allocating library routine.
//
// The scratch holds the per-block partial sums of the two-level reduction
// and the block-completion counter.  Its size does not depend on the vector
// length: the launch shape keeps the partials at 2 * values * chunks <= 608
// doubles for any length and at most 45 vectors (+1 for the norm).
#include "gbprop_internal.h"
#include "../../include/gbprop.h"

#include <mutex>
#include <string>

namespace {

// 1024 doubles of partial sums + one 256-byte slot for the counter word.
constexpr size_t kNoallocDoubles = 1024;
constexpr size_t kNoallocBytes = kNoallocDoubles * sizeof(double) + 256;

// Every GPU that loads the library holds this array until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mutex;

gbprop_status noalloc_fail(gbprop_status st, const std::string& msg) {
    gbprop::set_last_error(msg.c_str());     // reported by gbprop_last_error()
    return st;
}

// Device address of the scratch array on the current device.  In host code the
// array's name is only a host-side stand-in; the real address comes from
// cudaGetSymbolAddress, called once per device with that device current.
cudaError_t scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" {

gbprop_status gbprop_block_inner_product_noalloc(int precision, const void* V, long n, int nv, const void* w,
                                                 int want_norm, double* out, void* stream) {
    if (precision != GBPROP_FP64 && precision != GBPROP_FP32_MIXED)
        return noalloc_fail(GBPROP_EINVAL, "unknown precision");
    if (n <= 0 || nv < 1 || nv > gbprop::kMaxBasis)
        return noalloc_fail(GBPROP_EINVAL, "need n > 0 and 1 <= nv <= 45");
    if (!V || !w || !out) return noalloc_fail(GBPROP_EINVAL, "null buffer");
    const int nvals = nv + (want_norm ? 1 : 0);
    const size_t need = gbprop::block_inner_scratch_doubles(n, nvals);
    if (need > kNoallocDoubles)
        return noalloc_fail(GBPROP_EINVAL, "reduction scratch of " + std::to_string(need) +
                                               " doubles exceeds the fixed " + std::to_string(kNoallocDoubles));
    void* base = nullptr;
    cudaError_t e = scratch_address(&base);
    if (e != cudaSuccess) return noalloc_fail(GBPROP_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    double* partials = (double*)base;
    unsigned* counter = (unsigned*)((char*)base + kNoallocDoubles * sizeof(double));
    cudaStream_t s = (cudaStream_t)stream;
    // the array keeps the previous call's contents: the counter must start at zero
    e = cudaMemsetAsync(counter, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return noalloc_fail(GBPROP_ECUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    e = gbprop::launch_block_inner(precision == GBPROP_FP64 ? 0 : 1, V, n, nv, w, want_norm ? 1 : 0, out, partials,
                                   counter, s);
    if (e != cudaSuccess) return noalloc_fail(GBPROP_ECUDA, std::string("launch: ") + cudaGetErrorString(e));
    return GBPROP_OK;
}

}  // extern "C"
