// Device helpers shared by the kernel translation units (complex make/convert, warp sum).
#pragma once
#include "gbprop_internal.h"

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

}  // namespace gbprop
