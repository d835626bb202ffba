// Device helpers shared by the kernel translation units (complex make/convert, warp sum).
#pragma once
#include "gbprop_internal.h"

#include <cfloat>
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

// (h, l) += (ah + al)(bh + bl): exact ah*bh, cross terms to first order, error-free sum
__device__ __forceinline__ void df_mac(float& h, float& l, float ah, float al, float bh, float bl) {
    const float p = __fmul_rn(ah, bh);
    const float e = __fmaf_rn(ah, bh, -p);
    const float lo = __fmaf_rn(ah, bl, __fmaf_rn(al, bh, e));
    float t;
    two_sum(h, p, h, t);
    l = __fadd_rn(l, __fadd_rn(t, lo));
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
// float <-> double conversions by integer operations.  On this GPU a conversion instruction
// between FP32 and FP64 issues on the FP64 pipe at the rate of an FP64 FMA (measured: 628 vs
// 528 G/s over all SMs, against 14 T/s for integer ops), so the FP64-accurate solve, which
// converts every element several times, forms them from the bit patterns instead.
// Precision probe of FP64 handles (Ctrl::round_matvec): a complex128 value rounded to
// complex64, as the FP32-mixed path stores it.  Bit 0: band matvec outputs; bit 1: the
// outputs of the Arnoldi loop's solves and of the Gram-Schmidt update.
__device__ __forceinline__ double2 round_c64(double2 v) {
    return make_double2((double)(float)v.x, (double)(float)v.y);
}

//   d2f_fast: round to nearest even, as (float)d for results in FP32's normal range; results
//             below it are flushed to signed zero; overflow gives +-inf and NaN stays NaN.
//   f2d_fast: exact, as (double)f, except that subnormal floats become signed zero.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float d2f_fast(double d) {
    const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
    const unsigned sign = hi & 0x80000000u;
    const unsigned e = (hi >> 20) & 0x7ffu;
    const unsigned fm = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1fffffffu;
    const unsigned up = (rem > 0x10000000u) | ((rem == 0x10000000u) & fm & 1u);
    unsigned bits;
    if (e <= 896u) bits = sign;
    else if (e >= 1151u) bits = sign | ((e == 2047u && ((hi & 0xfffffu) | lo)) ? 0x7fc00000u : 0x7f800000u);
    else bits = sign | (((e - 896u) << 23) + fm + up);
    return __uint_as_float(bits);
}

__device__ __forceinline__ double f2d_fast(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu, sign = u & 0x80000000u;
    const unsigned de = e == 255u ? 2047u : e + 896u;
    const unsigned hi = e == 0 ? sign : (sign | (de << 20) | ((u & 0x7fffffu) >> 3));
    const unsigned lo = e == 0 ? 0u : (u & 0x7u) << 29;
    return __hiloint2double((int)hi, (int)lo);
}

// ---------------------------------------------------------------------------
// bulk asynchronous copies global -> shared, completed on an mbarrier
// ---------------------------------------------------------------------------
constexpr long kInvWaitLimit = 1L << 24;      // try_wait polls before a staging wait gives up

// Poll budget of the first bounded wait of a launch (the staging wait, the grid barrier):
// the handle's Ctrl::wait_limit when set (> 0), none when negative (a test makes the wait
// give up at once), else `dflt`.  Waits that only drain copies in flight before an early
// exit keep the fixed default, so a CTA never leaves with bulk copies still landing.
__device__ __forceinline__ long wait_budget(const Ctrl* ctrl, long dflt) {
    const long long v = ctrl ? ctrl->wait_limit : 0;
    return v == 0 ? dflt : (v < 0 ? 0L : (long)v);
}

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

// dst, src 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar)) : "memory");
}

// Bounded wait for phase 0 of the mbarrier; false when the poll limit was reached.
__device__ __forceinline__ bool mbar_wait0(unsigned long long* bar, long limit = kInvWaitLimit) {
    const unsigned a = smem_u32(bar);
    for (long it = 0; it < limit; ++it) {
        unsigned done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n"
                     " selp.u32 %0, 1, 0, p;\n}" : "=r"(done) : "r"(a) : "memory");
        if (done) return true;
    }
    return false;
}

// FP32 Gauss-Jordan inverse of the m x m complex matrix D = dval(r, c) (float2) with partial
// pivoting on |re|+|im| (first maximum) on [D | I], rows of 2m float2.  The row swap and the
// pivot-row scaling are folded into the update, out(r) = row'(r) - mult'(r) * newrow with row' the
// swapped rows, so a pivot step reads one buffer and writes the other and costs two block
// barriers; finished left columns (<= k) are not written.  Fa is read first; the result ends in Fa
// when m is even, in Fb when m is odd, as the right half (row stride 2m).  Returns 0, or the
// 1-based column of the first zero pivot (then the buffers hold no inverse).  Whole block.
template <typename DV>
__device__ int gj_inverse_f32(int m, DV dval, float2* Fa, float2* Fb) {
    __shared__ int s_piv;
    __shared__ float2 s_inv;
    const int tid = threadIdx.x, w2 = 2 * m;
    for (int k = tid; k < m * w2; k += blockDim.x) {
        const int r = k / w2, c = k - r * w2;
        const float2 v = c < m ? dval(r, c) : make_float2(c - m == r ? 1.f : 0.f, 0.f);
        Fa[k] = v;
        Fb[k] = v;
    }
    __syncthreads();
    float2* Fr = Fa;
    float2* Fw = Fb;
    int info = 0;
    for (int k = 0; k < m; ++k) {
        if (tid < 32) {
            float best = -1.f;
            int bi = k;
            for (int r = k + tid; r < m; r += 32) {
                const float v = fabsf(Fr[r * w2 + k].x) + fabsf(Fr[r * w2 + k].y);
                if (v > best) { best = v; bi = r; }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const float ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (tid == 0) {
                s_piv = (best == 0.f) ? -1 : bi;
                if (best != 0.f) {
                    const float2 d = Fr[bi * w2 + k];
                    const float den = d.x * d.x + d.y * d.y;
                    s_inv = make_float2(d.x / den, -d.y / den);
                }
            }
        }
        __syncthreads();
        const int p = s_piv;
        if (p < 0) { info = k + 1; break; }           // singular (uniform: s_piv is shared)
        const float2 inv = s_inv;
        const int nleft = m - k - 1, ncols = nleft + m;
        const float2 fkk = Fr[k * w2 + k];             // multiplier of the row that moves to p
        for (int j = tid & 63; j < ncols; j += 64) {
            const int c = j < nleft ? k + 1 + j : m + (j - nleft);
            const float2 pr = Fr[p * w2 + c], rk = Fr[k * w2 + c];
            const float2 nw = make_float2(pr.x * inv.x - pr.y * inv.y, pr.x * inv.y + pr.y * inv.x);
            for (int r = tid >> 6; r < m; r += (int)(blockDim.x >> 6)) {
                float2 out = nw;
                if (r != k) {
                    const float2 src = r == p ? rk : Fr[r * w2 + c];
                    const float2 f = r == p ? fkk : Fr[r * w2 + k];
                    out = make_float2(src.x - (f.x * nw.x - f.y * nw.y), src.y - (f.x * nw.y + f.y * nw.x));
                }
                Fw[r * w2 + c] = out;
            }
        }
        __syncthreads();
        float2* t = Fr;
        Fr = Fw;
        Fw = t;
    }
    return info;
}

// compensated butterfly over the warp: every lane ends with the same (hi, lo)
__device__ __forceinline__ void warp_pair_sum(float& h, float& l) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, h, o), ol = __shfl_xor_sync(0xffffffffu, l, o);
        acc_pair(h, l, oh, ol);
    }
}

// beta = ||w|| of the next basis vector from the cooperative Gram-Schmidt kernel's per-CTA
// ||w||^2 partials, summed by one warp in a fixed order (the same beta in every CTA that
// calls it).  PAIRS: FP32-pair partials (float4 hi, lo, -, -) of the complex64 form, else one
// double per CTA.  Whole warp; returns beta in every lane.
template <bool PAIRS>
__device__ __forceinline__ double gs_beta(const void* part, int G) {
    const int lane = threadIdx.x & 31;
    if constexpr (PAIRS) {
        const float4* p = reinterpret_cast<const float4*>(part);
        float a = 0.f, c = 0.f;
        for (int g0 = lane; g0 < G; g0 += 8 * 32) {
            float4 t[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int g = g0 + 32 * u;
                t[u] = g < G ? __ldcg(p + g) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) acc_pair(a, c, t[u].x, t[u].y);
        }
        warp_pair_sum(a, c);
        return sqrt((double)a + (double)c);
    } else {
        const double* p = reinterpret_cast<const double*>(part);
        double t = 0.0;
        for (int g = lane; g < G; g += 32) t += __ldcg(p + g);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        return sqrt(t);
    }
}

// Records beta of the next basis vector (pamp.h:330-345; happy breakdown below sqrt(eps),
// pamp.h:79) in the control block when `writer`; returns true on breakdown.
__device__ __forceinline__ bool gs_record_beta(Ctrl* ctrl, double beta, bool writer) {
    const bool brk = fabs(beta) < sqrt(DBL_EPSILON);
    if (writer) {
        ctrl->resid_norm = beta;
        if (!isfinite(beta)) ctrl->nonfinite = 1;
        if (brk) {
            ctrl->broken = 1;
            ctrl->breakdown_count++;
        } else {
            ctrl->beta = beta;
            set_inv_beta(ctrl, beta);
        }
    }
    return brk;
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
