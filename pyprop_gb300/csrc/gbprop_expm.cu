// Hessenberg exponential of the FP32-mixed path in double-float arithmetic.
//
// The same scaling-and-squaring Pade (order 6) as the FP64 cluster kernel (pamp.h:430-564: scaling
// order s = max(0, ceil(log2 max|a_ij|)), Horner in A^2, X = (Q - P)^-1 P, E = I + 2X, s
// squarings, first column), with every matrix entry an unevaluated sum of two FP32 numbers and
// every product an exact FP32 product plus first-order cross terms, accumulated with error-free
// sums.  Entries carry ~48 bits; s squarings amplify the rounding by up to 2^s, so at s = 17 the
// exponential is good to ~1e-9 relative -- far below the complex64 basis it multiplies (6e-8 per
// element), and it leaves the FP64 pipe, which retires about one warp instruction per 120 cycles
// per sub-partition in this few-warp kernel (a 30 x 30 complex FP64 product costs ~9k cycles on
// each of 16 SMs; the double-float one is FP32 issue).  The scaling order, the Hessenberg
// written back and the statistics are those of the FP64 kernel.
//
// Layout as the FP64 cluster kernel: each of the CL CTAs of a thread-block cluster holds full
// copies of the matrices in shared memory (float4 per entry: re_hi, re_lo, im_hi, im_lo); a
// product's rows are computed by their owner CTA (row % CL) and stored into every CTA's copy
// through distributed shared memory, followed by a cluster barrier.
#include "gbprop_internal.h"
#include "gbprop_device.cuh"

#include <cooperative_groups.h>

#include <cfloat>
#include <cmath>

namespace gbprop {

namespace cg = cooperative_groups;

namespace {

__device__ __forceinline__ float4 df_of(double re, double im) {
    const float a = (float)re, b = (float)im;
    return make_float4(a, (float)(re - (double)a), b, (float)(im - (double)b));
}

__device__ __forceinline__ float4 df_normal(float rh, float rl, float ih, float il) {
    float a, b, c, d;
    two_sum(rh, rl, a, b);
    two_sum(ih, il, c, d);
    return make_float4(a, b, c, d);
}

// real double-float scalar (ch + cl) times a complex double-float entry
__device__ __forceinline__ float4 df_scale(float ch, float cl, float4 a) {
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
    df_mac(rh, rl, ch, cl, a.x, a.y);
    df_mac(ih, il, ch, cl, a.z, a.w);
    return df_normal(rh, rl, ih, il);
}

// a + (ch + cl) on the real part
__device__ __forceinline__ float4 df_add_real(float4 a, float ch, float cl) {
    float h = a.x, l = a.y;
    acc_pair(h, l, ch, cl);
    float s, e;
    two_sum(h, l, s, e);
    return make_float4(s, e, a.z, a.w);
}

// C = A B for the rows this CTA owns, stored into every CTA's copy; four threads per entry
// split the k sum, combined by compensated shuffles within aligned lane quads.
template <int CL>
__device__ void cl_matmul_df(cg::cluster_group& cl, int rank, int m, const float4* A, const float4* B, float4* Cdst) {
    constexpr int KS = 4;
    const int mine = (m - rank + CL - 1) / CL;            // rows r = rank, rank + CL, ...
    const int total = mine * m * KS;
    for (int base = 0; base < total; base += blockDim.x) {
        const int idx = base + threadIdx.x;
        const bool act = idx < total;
        const int o = idx / KS, ks = idx % KS;
        const int r = rank + (o / m) * CL, c = o % m;
        float r1h = 0.f, r1l = 0.f, r2h = 0.f, r2l = 0.f, i1h = 0.f, i1l = 0.f, i2h = 0.f, i2l = 0.f;
        if (act)
            for (int k = ks; k < m; k += KS) {
                const float4 a = A[r * m + k], b = B[k * m + c];
                df_mac(r1h, r1l, a.x, a.y, b.x, b.y);      //  ar br
                df_mac(r2h, r2l, -a.z, -a.w, b.z, b.w);    // -ai bi
                df_mac(i1h, i1l, a.x, a.y, b.z, b.w);      //  ar bi
                df_mac(i2h, i2l, a.z, a.w, b.x, b.y);      //  ai br
            }
        acc_pair(r1h, r1l, r2h, r2l);
        acc_pair(i1h, i1l, i2h, i2l);
#pragma unroll
        for (int w = 1; w < KS; w <<= 1) {
            const float a = __shfl_xor_sync(0xffffffffu, r1h, w), b = __shfl_xor_sync(0xffffffffu, r1l, w);
            const float c2 = __shfl_xor_sync(0xffffffffu, i1h, w), d = __shfl_xor_sync(0xffffffffu, i1l, w);
            acc_pair(r1h, r1l, a, b);
            acc_pair(i1h, i1l, c2, d);
        }
        if (act && ks == 0) {
            const float4 v = df_normal(r1h, r1l, i1h, i1l);
#pragma unroll
            for (int q = 0; q < CL; ++q) {
                float4* dst = cl.map_shared_rank(Cdst, q);
                dst[r * m + c] = v;
            }
        }
    }
    cl.sync();
}

}  // namespace

template <int CL>
__global__ void __launch_bounds__(256) k_expm_cluster_df(Ctrl* ctrl, double* Hg, int m, const SchedEntry* sched) {
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int mm = m * m;
    float4* buf[7];
    for (int k = 0; k < 7; ++k) buf[k] = reinterpret_cast<float4*>(smem_raw) + (size_t)k * mm;
    float4* A = buf[0];
    float4* A2 = buf[1];
    float4* P = buf[2];
    float4* Q = buf[3];
    float4* T = buf[4];
    float4* LU = buf[5];
    float4* X = buf[6];
    __shared__ double s_mx[CL];                          // every CTA's max |a|^2 (written by all)
    __shared__ double red[8];
    __shared__ int s_sord;
    __shared__ float2 s_c[8];                            // Pade coefficients as FP32 pairs
    const int tid = threadIdx.x;
    const SchedEntry se = sched[ctrl->step];
    const double2 f = make_double2(se.dt_im, -se.dt_re);   // -i * dt (pamp.h:634)
    cl.sync();                                           // every CTA running before remote writes
    // A = f H for the rows this CTA owns (FP64 product, split), broadcast to every CTA; the
    // same values written back to the global Hessenberg (the reference scales it in place)
    double mx = 0.0;
    for (int k = tid; k < mm; k += blockDim.x) {
        const int r = k / m;
        if (r % CL != rank) continue;
        const double hr = Hg[2 * k], hi = Hg[2 * k + 1];
        const double ar = hr * f.x - hi * f.y, ai = hr * f.y + hi * f.x;
        Hg[2 * k] = ar;
        Hg[2 * k + 1] = ai;
        mx = fmax(mx, fma(ar, ar, ai * ai));
        const float4 v = df_of(ar, ai);
#pragma unroll
        for (int q = 0; q < CL; ++q) cl.map_shared_rank(A, q)[k] = v;
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0) red[tid >> 5] = mx;
    __syncthreads();
    if (tid == 0) {
        double v2 = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v2 = fmax(v2, red[w]);
#pragma unroll
        for (int q = 0; q < CL; ++q) cl.map_shared_rank(s_mx, q)[rank] = v2;
    }
    cl.sync();
    if (tid == 0) {
        double v2 = 0.0;
        for (int q = 0; q < CL; ++q) v2 = fmax(v2, s_mx[q]);
        // s = max(0, ceil(log2 max|a|)) from the exponent of max|a| (as the FP64 kernel)
        int sord = 0;
        if (!(v2 <= DBL_MAX)) {
            if (rank == 0) ctrl->nonfinite = 1;
        } else if (v2 > 0.0) {
            int e;
            const double fr = frexp(sqrt(v2), &e);
            sord = (fr == 0.5) ? e - 1 : e;
        }
        if (sord < 0) sord = 0;
        s_sord = sord;
        const int order = 6;
        double c = 1.0;
        for (int i = 0; i <= order; ++i) {
            const float h = (float)c;
            s_c[i] = make_float2(h, (float)(c - (double)h));
            c = c * (double)(order - i) / (double)((i + 1) * (2 * order - i));
        }
    }
    __syncthreads();
    const int sorder = s_sord;
    const float isc = ldexpf(1.f, -min(sorder, 126));     // exact power of two (s <= 126 here)
    for (int k = tid; k < mm; k += blockDim.x) {
        const float4 a = A[k];
        A[k] = make_float4(a.x * isc, a.y * isc, a.z * isc, a.w * isc);
    }
    __syncthreads();
    cl_matmul_df<CL>(cl, rank, m, A, A, A2);
    // Horner in A^2 (pamp.h:497-539); first factors are scalar multiples of I
    for (int k = tid; k < mm; k += blockDim.x) {
        Q[k] = df_scale(s_c[6].x, s_c[6].y, A2[k]);
        P[k] = df_scale(s_c[5].x, s_c[5].y, A2[k]);
    }
    __syncthreads();
    for (int r = tid; r < m; r += blockDim.x) {
        Q[r * m + r] = df_add_real(Q[r * m + r], s_c[4].x, s_c[4].y);
        P[r * m + r] = df_add_real(P[r * m + r], s_c[3].x, s_c[3].y);
    }
    __syncthreads();
    cl_matmul_df<CL>(cl, rank, m, Q, A2, T);               // i = 2
    { float4* t = Q; Q = T; T = t; }
    for (int r = tid; r < m; r += blockDim.x) Q[r * m + r] = df_add_real(Q[r * m + r], s_c[2].x, s_c[2].y);
    __syncthreads();
    cl_matmul_df<CL>(cl, rank, m, P, A2, T);               // i = 1
    { float4* t = P; P = T; T = t; }
    for (int r = tid; r < m; r += blockDim.x) P[r * m + r] = df_add_real(P[r * m + r], s_c[1].x, s_c[1].y);
    __syncthreads();
    cl_matmul_df<CL>(cl, rank, m, Q, A2, T);               // i = 0
    { float4* t = Q; Q = T; T = t; }
    for (int r = tid; r < m; r += blockDim.x) Q[r * m + r] = df_add_real(Q[r * m + r], s_c[0].x, s_c[0].y);
    __syncthreads();
    cl_matmul_df<CL>(cl, rank, m, P, A, T);                // P = P A
    { float4* t = P; P = T; T = t; }
    // X = (Q - P)^-1 P: D = Q - P, an FP32 Gauss-Jordan inverse Z of its leading parts, then
    // X refined with double-float residuals R = P - D X split over the cluster by column
    for (int k = tid; k < mm; k += blockDim.x) {
        const float4 q = Q[k], p = P[k];
        float rh = q.x, rl = q.y, ih = q.z, il = q.w;
        acc_pair(rh, rl, -p.x, -p.y);
        acc_pair(ih, il, -p.z, -p.w);
        LU[k] = df_normal(rh, rl, ih, il);
    }
    __syncthreads();
    const int w2 = 2 * m;
    const int gi = gj_inverse_f32(
        m, [&](int r, int c) { return make_float2(LU[r * m + c].x, LU[r * m + c].z); },
        reinterpret_cast<float2*>((m & 1) ? T : X), reinterpret_cast<float2*>((m & 1) ? X : T));
    const float2* Z = reinterpret_cast<const float2*>(X) + m;   // Z(r, k) = Z[r * w2 + k]
    const int info = gi ? gi : (ctrl->inject_lu ? m : 0);       // inject_lu: host-set test hook
    if (info) {
        if (rank == 0 && tid == 0 && !ctrl->nonfinite) ctrl->lu_info = info;   // non-finite matrix: that is the cause
    } else {
        const int ncol = (m - rank + CL - 1) / CL;           // this CTA's columns c = rank + j*CL
        float4* Xc = T;
        float4* R = Q;
        float2* R32 = reinterpret_cast<float2*>(A);           // A is free and never written remotely
        for (int it = 0; it < 3; ++it) {
            for (int base = 0; base < ncol * m * 4; base += blockDim.x) {
                const int idx = base + tid, ks = idx & 3, o = idx >> 2;
                const bool act = o < ncol * m;
                const int c = act ? rank + (o / m) * CL : 0, r = act ? o % m : 0;
                float r1h = 0.f, r1l = 0.f, r2h = 0.f, r2l = 0.f, i1h = 0.f, i1l = 0.f, i2h = 0.f, i2l = 0.f;
                if (act && it > 0)
                    for (int k = ks; k < m; k += 4) {
                        const float4 d = LU[r * m + k], x = Xc[k * m + c];
                        df_mac(r1h, r1l, -d.x, -d.y, x.x, x.y);
                        df_mac(r2h, r2l, d.z, d.w, x.z, x.w);
                        df_mac(i1h, i1l, -d.x, -d.y, x.z, x.w);
                        df_mac(i2h, i2l, -d.z, -d.w, x.x, x.y);
                    }
                acc_pair(r1h, r1l, r2h, r2l);
                acc_pair(i1h, i1l, i2h, i2l);
#pragma unroll
                for (int w = 1; w < 4; w <<= 1) {
                    const float a = __shfl_xor_sync(0xffffffffu, r1h, w), b = __shfl_xor_sync(0xffffffffu, r1l, w);
                    const float c2 = __shfl_xor_sync(0xffffffffu, i1h, w), d = __shfl_xor_sync(0xffffffffu, i1l, w);
                    acc_pair(r1h, r1l, a, b);
                    acc_pair(i1h, i1l, c2, d);
                }
                if (act && ks == 0) {
                    const float4 p = P[r * m + c];
                    acc_pair(r1h, r1l, p.x, p.y);
                    acc_pair(i1h, i1l, p.z, p.w);
                    const float4 v = df_normal(r1h, r1l, i1h, i1l);
                    R[r * m + c] = v;
                    R32[r * m + c] = make_float2(v.x, v.z);
                }
            }
            __syncthreads();
            // X += Z R (FP32 products on the leading parts of the residual)
            for (int idx = tid; idx < ncol * m; idx += blockDim.x) {
                const int c = rank + (idx / m) * CL, r = idx % m;
                float ar = 0.f, ai = 0.f;
                for (int k = 0; k < m; ++k) {
                    const float2 zz = Z[r * w2 + k];
                    const float xr = R32[k * m + c].x, xi = R32[k * m + c].y;
                    ar = fmaf(zz.x, xr, ar);
                    ar = fmaf(-zz.y, xi, ar);
                    ai = fmaf(zz.x, xi, ai);
                    ai = fmaf(zz.y, xr, ai);
                }
                if (it == 0) {
                    Xc[r * m + c] = make_float4(ar, 0.f, ai, 0.f);
                } else {
                    const float4 x = Xc[r * m + c];
                    float h1 = x.x, l1 = x.y, h2 = x.z, l2 = x.w;
                    acc_pair(h1, l1, ar, 0.f);
                    acc_pair(h2, l2, ai, 0.f);
                    Xc[r * m + c] = df_normal(h1, l1, h2, l2);
                }
            }
            __syncthreads();
        }
        // E = I + 2 X for this CTA's columns, broadcast into every CTA's A2 buffer
        for (int idx = tid; idx < ncol * m; idx += blockDim.x) {
            const int c = rank + (idx / m) * CL, r = idx % m;
            const float4 x = Xc[r * m + c];
            float4 v = make_float4(2.f * x.x, 2.f * x.y, 2.f * x.z, 2.f * x.w);
            if (r == c) v = df_add_real(v, 1.f, 0.f);
#pragma unroll
            for (int q = 0; q < CL; ++q) cl.map_shared_rank(A2, q)[r * m + c] = v;
        }
    }
    cl.sync();
    { float4* t = A; A = A2; A2 = t; }
    if (!info) {
        for (int i = 0; i < sorder; ++i) {
            cl_matmul_df<CL>(cl, rank, m, A, A, T);
            float4* t = A; A = T; T = t;
        }
        if (rank == 0) {
            for (int k = tid; k < m; k += blockDim.x) {
                const float4 a = A[k * m];
                ctrl->y[2 * k] = (double)a.x + (double)a.y;
                ctrl->y[2 * k + 1] = (double)a.z + (double)a.w;
            }
            if (tid == 0) {
                const float4 a = A[(m - 1) * m];
                const double yr = (double)a.x + (double)a.y, yi = (double)a.z + (double)a.w;
                ctrl->err_est = yr * yr + yi * yi;
                ctrl->scaling_order = sorder;
            }
        }
    }
    // no CTA may exit while others can still address its shared memory
    cl.sync();
}

template <int CL>
static cudaError_t launch_df(Ctrl* ctrl, double* H, int m, const SchedEntry* sched, cudaStream_t s) {
    const size_t smem = (size_t)7 * m * m * sizeof(float4);
    auto kern = k_expm_cluster_df<CL>;
    cudaError_t e = allow_max_smem(kern);
    if (e != cudaSuccess) return e;
    if (CL > 8) {
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(CL);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, ctrl, H, m, sched);
}

cudaError_t launch_expm_df(Ctrl* ctrl, double* H, int m, const SchedEntry* sched, int cluster, cudaStream_t s) {
    if (cluster == 16) return launch_df<16>(ctrl, H, m, sched, s);
    if (cluster == 8) return launch_df<8>(ctrl, H, m, sched, s);
    if (cluster == 1) return launch_df<1>(ctrl, H, m, sched, s);   // one CTA (batches)
    return cudaErrorInvalidValue;
}

bool expm_df_single_fits(int m) {
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, k_expm_cluster_df<1>) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return (size_t)7 * m * m * sizeof(float4) + fa.sharedSizeBytes + 1024 <= (size_t)optin;
}

}  // namespace gbprop
