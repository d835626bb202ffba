// Device helpers shared by the kernel translation units (complex make/convert, warp sum).
#pragma once
#include "gbprop_internal.h"

#include <mutex>
#include <unordered_set>

namespace gbprop {

// ---------------------------------------------------------------------------
// small complex helpers
// ---------------------------------------------------------------------------
template <typename T> __device__ __forceinline__ cx<T> mk(T re, T im);
template <> __device__ __forceinline__ double2 mk<double>(double re, double im) { return make_double2(re, im); }
template <> __device__ __forceinline__ float2 mk<float>(float re, float im) { return make_float2(re, im); }

template <typename C> struct elem_of;
template <> struct elem_of<double2> { using type = double; };
template <> struct elem_of<float2> { using type = float; };

template <typename CO, typename CI> __device__ __forceinline__ CO conv(CI v) {
    using E = typename elem_of<CO>::type;
    CO o;
    o.x = (E)v.x;
    o.y = (E)v.y;
    return o;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Error-free transformations in FP32 (no contraction: explicit round-to-nearest ops).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// acc (hi, lo) += (uh + ul) * x, with uh*x split exactly into product and rounding error.
__device__ __forceinline__ void acc_prod(float& hi, float& lo, float uh, float ul, float x) {
    const float p = __fmul_rn(uh, x);
    const float pe = __fmaf_rn(uh, x, -p);
    float t;
    two_sum(hi, p, hi, t);
    lo = __fadd_rn(lo, __fadd_rn(t, __fmaf_rn(ul, x, pe)));
}

// (hi, lo) += (ch + cl) * (sh + sl), first order in the low parts.
__device__ __forceinline__ void acc_scaled(float& hi, float& lo, float ch, float cl, float sh, float sl) {
    const float p = __fmul_rn(ch, sh);
    const float pe = __fmaf_rn(ch, sh, -p);
    float t;
    two_sum(hi, p, hi, t);
    lo = __fadd_rn(lo, __fadd_rn(t, __fadd_rn(pe, __fmaf_rn(ch, sl, __fmul_rn(cl, sh)))));
}

// (hi, lo) += (bh + bl)
__device__ __forceinline__ void acc_pair(float& hi, float& lo, float bh, float bl) {
    float t;
    two_sum(hi, bh, hi, t);
    lo = __fadd_rn(lo, __fadd_rn(bl, t));
}

// x * (h + l) rounded once to FP32 (exact product x*h, the low part to first order)
__device__ __forceinline__ float mul_pair(float x, float h, float l) {
    const float p = __fmul_rn(x, h);
    const float e = __fmaf_rn(x, h, -p);
    return __fadd_rn(p, __fmaf_rn(x, l, e));
}

// 1 / beta for the next basis vector: FP64, and as an FP32 pair for the complex64 solve
__device__ __forceinline__ void set_inv_beta(Ctrl* c, double beta) {
    const double ib = 1.0 / beta;
    c->inv_beta = ib;
    const float h = (float)ib;
    c->inv_beta_f[0] = h;
    c->inv_beta_f[1] = (float)(ib - (double)h);
}

// ---------------------------------------------------------------------------
// bulk asynchronous copies global -> shared, completed on an mbarrier
// ---------------------------------------------------------------------------
constexpr long kInvWaitLimit = 1L << 24;      // try_wait polls before a staging wait gives up

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

// Bounded wait for phase 0 of the mbarrier; false when the poll limit was reached.
__device__ __forceinline__ bool mbar_wait0(unsigned long long* bar) {
    const unsigned a = smem_u32(bar);
    for (long it = 0; it < kInvWaitLimit; ++it) {
        unsigned done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n"
                     " selp.u32 %0, 1, 0, p;\n}" : "=r"(done) : "r"(a) : "memory");
        if (done) return true;
    }
    return false;
}

// Programmatic dependent launch: a kernel launched with launch_pdl is scheduled as its
// predecessor's CTAs retire (no explicit early trigger: CTAs of the next kernel waiting on
// SMs slowed the solve measurably), hiding the launch gap between stream-launched kernels;
// inside a captured graph the gap is already small.  The kernel must execute pdl_wait()
// before it reads anything the predecessor wrote and before any early return (so that
// completion stays transitive along a chain of such kernels).  Without the launch
// attribute pdl_wait is a no-op.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

bool pdl_enabled();                         // GBPROP_PDL=0 disables the attribute

template <typename K, typename... Args>
inline cudaError_t launch_pdl(K kern, dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl_enabled() ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}

// Raise a kernel's dynamic shared-memory limit to the device's opt-in maximum, once per
// kernel.  The limit then does not depend on which launch set it last, so graph nodes of
// one kernel with different shared-memory sizes all stay valid, also when a tool replays
// them one by one.
template <typename K> inline cudaError_t allow_max_smem(K kern) {
    static std::mutex mu;
    static std::unordered_set<const void*> done;
    std::lock_guard<std::mutex> lock(mu);
    const void* key = reinterpret_cast<const void*>(kern);
    if (done.count(key)) return cudaSuccess;
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kern);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
    if (e == cudaSuccess) done.insert(key);
    return e;
}

}  // namespace gbprop
