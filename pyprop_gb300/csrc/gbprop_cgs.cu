// One Arnoldi step's classical Gram-Schmidt in a single cooperative kernel
// (pamp.h:317-345 without re-orthogonalisation; BLASIntegrationFunctor block
// InnerProduct + zgemv + norm, functors.h:182-241):
//     h = V_{0..J}^H w,   w <- w - V h,   beta = ||w||,   Hessenberg column J, breakdown test.
// The grid has one CTA per SM (co-resident by the cooperative launch).  CTA b owns the
// element chunk [b*C, (b+1)*C) of every basis vector: it reads its chunk of V once into
// shared memory (when it fits), forms its partial inner products, and after a grid
// barrier every CTA sums all CTAs' partials in the same fixed order (deterministic, the
// same h everywhere), updates its chunk of w from the cached V and contributes ||w||^2;
// after a second barrier CTA 0 writes the Hessenberg column and the control block.
// Versus separate dot / update / finalize kernels this reads V once instead of twice and
// removes two launches and two last-block reductions per Arnoldi step.
#include "gbprop_internal.h"
#include "gbprop_device.cuh"

#include <cfloat>

namespace gbprop {

constexpr int kFuseThreads = 512;
constexpr long kBarrierSpinLimit = 1L << 24;   // polls (each an L2 round trip) before a barrier gives up

// Sense-reversing grid barrier for a co-resident grid: bar[0] = arrivals, bar[1] = generation.
// Bounded: after kBarrierSpinLimit polls it records ctrl->wait_timeout and returns false.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned nblocks, Ctrl* ctrl) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        volatile unsigned* gen = bar + 1;
        const unsigned g = *gen;
        __threadfence();
        const unsigned arrived = atomicAdd(bar, 1u);
        if (arrived == nblocks - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long it = 0;
            while (*gen == g) {
                if (++it > kBarrierSpinLimit) {
                    ctrl->wait_timeout = 1;
                    ok = 0;
                    break;
                }
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// complex conj(v) * x accumulated in FP64
__device__ __forceinline__ void acc_dot64(double& ar, double& ai, double vr, double vi, double xr, double xi) {
    ar = fma(vr, xr, ar);
    ar = fma(vi, xi, ar);
    ai = fma(vr, xi, ai);
    ai = fma(-vi, xr, ai);
}

template <typename T, bool CACHE>
__global__ void __launch_bounds__(kFuseThreads) k_arnoldi_cgs(const cx<T>* __restrict__ V,
                                                              const double2* __restrict__ v0, long n, int J, int m,
                                                              cx<T>* __restrict__ w, double* __restrict__ part,
                                                              unsigned* bar, Ctrl* ctrl, double* H, int update,
                                                              int chunk) {
    using C = cx<T>;
    constexpr bool kF32 = sizeof(T) < sizeof(double);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double hs[2 * (kMaxBasis + 1)];
    __shared__ double red[kFuseThreads / 32];
    if (ctrl->broken) return;                        // uniform: written only between launches
    const int nv = J + 1, G = gridDim.x, b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long i0 = (long)b * chunk;
    const int cl = (int)max(0L, min((long)chunk, n - i0));
    // shared memory: w chunk | first vector (FP64, complex64 basis with v0) | cached rows
    C* ws = reinterpret_cast<C*>(smem_raw);
    double2* c0 = reinterpret_cast<double2*>(smem_raw + (((size_t)chunk * sizeof(C) + 15) & ~(size_t)15));
    C* cache = reinterpret_cast<C*>(reinterpret_cast<unsigned char*>(c0) + (v0 ? (size_t)chunk * 16 : 0));
    for (int i = tid; i < cl; i += kFuseThreads) ws[i] = w[i0 + i];
    __syncthreads();

    // ---- phase A: partial inner products, one warp per basis vector ------------------------
    for (int k = warp; k < nv; k += kFuseThreads / 32) {
        double ar = 0.0, ai = 0.0, br = 0.0, bi = 0.0;
        if (v0 && k == 0) {
            for (int i = lane; i < cl; i += 32) {
                const double2 v = v0[i0 + i];
                if (CACHE) c0[i] = v;
                const C x = ws[i];
                acc_dot64(ar, ai, v.x, v.y, (double)x.x, (double)x.y);
            }
        } else if (kF32) {
            // complex64 operands: error-free FP32 products, compensated FP32 sums; four
            // loads in flight per lane, two independent compensated chains
            float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f, sh = 0.f, sl = 0.f, th = 0.f, tl = 0.f;
            const C* vk = V + (size_t)k * n + i0;
            int i = lane;
            for (; i + 96 < cl; i += 128) {
                C v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) v[u] = vk[i + 32 * u];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (CACHE) cache[(size_t)k * chunk + i + 32 * u] = v[u];
                    const C x = ws[i + 32 * u];
                    if (u & 1) {
                        acc_prod(sh, sl, (float)v[u].x, 0.f, (float)x.x);
                        acc_prod(sh, sl, (float)v[u].y, 0.f, (float)x.y);
                        acc_prod(th, tl, (float)v[u].x, 0.f, (float)x.y);
                        acc_prod(th, tl, -(float)v[u].y, 0.f, (float)x.x);
                    } else {
                        acc_prod(rh, rl, (float)v[u].x, 0.f, (float)x.x);
                        acc_prod(rh, rl, (float)v[u].y, 0.f, (float)x.y);
                        acc_prod(ih, il, (float)v[u].x, 0.f, (float)x.y);
                        acc_prod(ih, il, -(float)v[u].y, 0.f, (float)x.x);
                    }
                }
            }
            for (; i < cl; i += 32) {
                const C v = vk[i];
                if (CACHE) cache[(size_t)k * chunk + i] = v;
                const C x = ws[i];
                acc_prod(rh, rl, (float)v.x, 0.f, (float)x.x);
                acc_prod(rh, rl, (float)v.y, 0.f, (float)x.y);
                acc_prod(ih, il, (float)v.x, 0.f, (float)x.y);
                acc_prod(ih, il, -(float)v.y, 0.f, (float)x.x);
            }
            ar = ((double)rh + (double)rl) + ((double)sh + (double)sl);
            ai = ((double)ih + (double)il) + ((double)th + (double)tl);
        } else {
            const C* vk = V + (size_t)k * n + i0;
            int i = lane;
            for (; i + 96 < cl; i += 128) {
                C v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) v[u] = vk[i + 32 * u];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (CACHE) cache[(size_t)k * chunk + i + 32 * u] = v[u];
                    const C x = ws[i + 32 * u];
                    if (u & 1) acc_dot64(br, bi, (double)v[u].x, (double)v[u].y, (double)x.x, (double)x.y);
                    else acc_dot64(ar, ai, (double)v[u].x, (double)v[u].y, (double)x.x, (double)x.y);
                }
            }
            for (; i + 32 < cl; i += 64) {
                const C v = vk[i], u = vk[i + 32];
                if (CACHE) {
                    cache[(size_t)k * chunk + i] = v;
                    cache[(size_t)k * chunk + i + 32] = u;
                }
                const C x = ws[i], y = ws[i + 32];
                acc_dot64(ar, ai, (double)v.x, (double)v.y, (double)x.x, (double)x.y);
                acc_dot64(br, bi, (double)u.x, (double)u.y, (double)y.x, (double)y.y);
            }
            if (i < cl) {
                const C v = vk[i];
                if (CACHE) cache[(size_t)k * chunk + i] = v;
                const C x = ws[i];
                acc_dot64(ar, ai, (double)v.x, (double)v.y, (double)x.x, (double)x.y);
            }
        }
        ar += br;
        ai += bi;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            ar += __shfl_xor_sync(0xffffffffu, ar, o);
            ai += __shfl_xor_sync(0xffffffffu, ai, o);
        }
        if (lane == 0) {
            part[((size_t)k * G + b) * 2] = ar;
            part[((size_t)k * G + b) * 2 + 1] = ai;
        }
    }
    if (!grid_barrier(bar, G, ctrl)) return;

    // ---- phase B: h = sum of the partials (fixed order; tpv threads per value, a power of
    // two <= 32 so that each value's threads are consecutive lanes of one warp) --------------
    __shared__ float2 hf[kMaxBasis + 1], hl[kMaxBasis + 1];
    {
        const int vals = 2 * nv;
        int tpv = 32;
        while (tpv > 1 && tpv * vals > kFuseThreads) tpv >>= 1;
        const int v = tid / tpv, q = tid % tpv;
        double s0 = 0.0, s1 = 0.0;
        if (v < vals) {
            const int k = v >> 1, c = v & 1;
            const double* p = part + (size_t)k * G * 2 + c;
            int g = q;
            for (; g + tpv < G; g += 2 * tpv) {
                s0 += __ldcg(p + (size_t)g * 2);
                s1 += __ldcg(p + (size_t)(g + tpv) * 2);
            }
            if (g < G) s0 += __ldcg(p + (size_t)g * 2);
        }
        double s = s0 + s1;
        for (int o = 1; o < tpv; o <<= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (v < vals && q == 0) hs[v] = s;
    }
    __syncthreads();
    if (kF32 && tid < nv) {
        // FP32 hi / lo parts of h, formed once for the complex64 update
        const float hr = (float)hs[2 * tid], hi = (float)hs[2 * tid + 1];
        hf[tid] = make_float2(hr, hi);
        hl[tid] = make_float2((float)(hs[2 * tid] - (double)hr), (float)(hs[2 * tid + 1] - (double)hi));
    }
    __syncthreads();

    double nrm = 0.0;
    if (update) {
        // w -= V h on this chunk; ||w||^2 partial
        for (int i = tid; i < cl; i += kFuseThreads) {
            C r = ws[i];
            if (kF32) {
                float sr = 0.f, si = 0.f, cr = 0.f, ci = 0.f;
                int k = 0;
                if (v0) {
                    const double2 a = CACHE ? c0[i] : v0[i0 + i];
                    const double hr = hs[0], hi = hs[1];
                    // FP64 first vector: its product in FP64, folded into the remainder sum
                    const double pr = a.x * hr - a.y * hi, pi = a.x * hi + a.y * hr;
                    sr = (float)pr;
                    si = (float)pi;
                    cr = (float)(pr - (double)sr);
                    ci = (float)(pi - (double)si);
                    k = 1;
                }
                for (; k < nv; ++k) {
                    const C vk = CACHE ? cache[(size_t)k * chunk + i] : V[(size_t)k * n + i0 + i];
                    const float hr = hf[k].x, hi = hf[k].y, lr = hl[k].x, li = hl[k].y;
                    sr = fmaf((float)vk.x, hr, sr);
                    sr = fmaf(-(float)vk.y, hi, sr);
                    si = fmaf((float)vk.x, hi, si);
                    si = fmaf((float)vk.y, hr, si);
                    cr = fmaf((float)vk.x, lr, cr);
                    cr = fmaf(-(float)vk.y, li, cr);
                    ci = fmaf((float)vk.x, li, ci);
                    ci = fmaf((float)vk.y, lr, ci);
                }
                r.x = (T)((float)r.x - (sr + cr));
                r.y = (T)((float)r.y - (si + ci));
            } else {
                double sr0 = 0.0, si0 = 0.0, sr1 = 0.0, si1 = 0.0;
                int k = 0;
                for (; k + 1 < nv; k += 2) {
                    const C a = CACHE ? cache[(size_t)k * chunk + i] : V[(size_t)k * n + i0 + i];
                    const C c = CACHE ? cache[(size_t)(k + 1) * chunk + i] : V[(size_t)(k + 1) * n + i0 + i];
                    const double ar_ = (double)a.x, ai_ = (double)a.y, cr_ = (double)c.x, ci_ = (double)c.y;
                    sr0 = fma(ar_, hs[2 * k], sr0);
                    sr0 = fma(-ai_, hs[2 * k + 1], sr0);
                    si0 = fma(ar_, hs[2 * k + 1], si0);
                    si0 = fma(ai_, hs[2 * k], si0);
                    sr1 = fma(cr_, hs[2 * k + 2], sr1);
                    sr1 = fma(-ci_, hs[2 * k + 3], sr1);
                    si1 = fma(cr_, hs[2 * k + 3], si1);
                    si1 = fma(ci_, hs[2 * k + 2], si1);
                }
                if (k < nv) {
                    const C a = CACHE ? cache[(size_t)k * chunk + i] : V[(size_t)k * n + i0 + i];
                    sr0 = fma((double)a.x, hs[2 * k], sr0);
                    sr0 = fma(-(double)a.y, hs[2 * k + 1], sr0);
                    si0 = fma((double)a.x, hs[2 * k + 1], si0);
                    si0 = fma((double)a.y, hs[2 * k], si0);
                }
                r.x -= (sr0 + sr1);
                r.y -= (si0 + si1);
            }
            w[i0 + i] = r;
            nrm = fma((double)r.x, (double)r.x, nrm);
            nrm = fma((double)r.y, (double)r.y, nrm);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
        if (lane == 0) red[warp] = nrm;
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            for (int q = 0; q < kFuseThreads / 32; ++q) t += red[q];
            part[(size_t)nv * G * 2 + b] = t;
        }
        if (!grid_barrier(bar, G, ctrl)) return;
    }

    // ---- phase C: Hessenberg column, beta and the breakdown test (CTA 0) --------------------
    if (b != 0) return;
    __shared__ double s_beta;
    if (update && warp == 0) {
        double t = 0.0;
        for (int g = lane; g < G; g += 32) t += __ldcg(part + (size_t)nv * G * 2 + g);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) s_beta = sqrt(t);
    }
    __syncthreads();
    for (int k = tid; k < nv; k += kFuseThreads) {
        H[2 * ((size_t)k * m + J)] = hs[2 * k];
        H[2 * ((size_t)k * m + J) + 1] = hs[2 * k + 1];
        ctrl->h[2 * k] = hs[2 * k];
        ctrl->h[2 * k + 1] = hs[2 * k + 1];
    }
    if (tid == 0) {
        ctrl->nbasis = nv;
        ctrl->operator_count++;
        if (J == 0) ctrl->inner_product_count++;
        if (J + 1 < m) {
            const double beta = s_beta;
            ctrl->resid_norm = beta;
            const double tol = sqrt(DBL_EPSILON);   // pamp.h:79
            if (!isfinite(beta)) ctrl->nonfinite = 1;
            if (fabs(beta) < tol) {
                ctrl->broken = 1;
                ctrl->breakdown_count++;
            } else {
                H[2 * ((size_t)(J + 1) * m + J)] = beta;
                H[2 * ((size_t)(J + 1) * m + J) + 1] = 0.0;
                ctrl->beta = beta;
                ctrl->inv_beta = 1.0 / beta;
            }
        }
    }
}

size_t arnoldi_cgs_smem(int prec, long n, int nv, int grid, int with_v0, int cache) {
    const size_t es = prec == 0 ? sizeof(double2) : sizeof(float2);
    const long chunk = ((n + grid - 1) / grid + 7) / 8 * 8;
    size_t b = (((size_t)chunk * es + 15) & ~(size_t)15);
    if (with_v0) b += (size_t)chunk * 16;
    if (cache) b += (size_t)nv * chunk * es;
    return b;
}

template <typename T, bool CACHE>
static cudaError_t arnoldi_cgs_launch(const void* V, const double2* v0, long n, int J, int m, void* w, double* part,
                                      unsigned* bar, Ctrl* ctrl, double* H, int update, int grid, cudaStream_t s) {
    const int chunk = (int)(((n + grid - 1) / grid + 7) / 8 * 8);
    const size_t smem = arnoldi_cgs_smem(sizeof(T) == 8 ? 0 : 1, n, J + 1, grid, v0 != nullptr, CACHE);
    auto kern = k_arnoldi_cgs<T, CACHE>;
    cudaError_t e = allow_max_smem(kern);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kFuseThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, (const cx<T>*)V, v0, n, J, m, (cx<T>*)w, part, bar, ctrl, H, update, chunk);
}

cudaError_t launch_arnoldi_cgs(int prec, const void* V, const double2* v0, long n, int J, int m, void* w,
                               double* part, unsigned* bar, Ctrl* ctrl, double* H, int update, int grid, int cache,
                               cudaStream_t s) {
    count_launch();
    if (prec == 0)
        return cache ? arnoldi_cgs_launch<double, true>(V, nullptr, n, J, m, w, part, bar, ctrl, H, update, grid, s)
                     : arnoldi_cgs_launch<double, false>(V, nullptr, n, J, m, w, part, bar, ctrl, H, update, grid, s);
    return cache ? arnoldi_cgs_launch<float, true>(V, v0, n, J, m, w, part, bar, ctrl, H, update, grid, s)
                 : arnoldi_cgs_launch<float, false>(V, v0, n, J, m, w, part, bar, ctrl, H, update, grid, s);
}

// Largest grid of co-resident CTAs for this configuration (0 when the cooperative form
// cannot run: no cooperative launch support or shared memory too large).
int arnoldi_cgs_grid(int prec, long n, int m, int with_v0, int cache) {
    int dev = 0, sms = 0, coop = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (!coop || sms <= 0) return 0;
    const size_t smem = arnoldi_cgs_smem(prec, n, m, sms, with_v0, cache);
    if (smem + 4096 > (size_t)optin) return 0;
    int per_sm = 0;
    cudaError_t e;
    if (prec == 0) {
        auto kern = cache ? k_arnoldi_cgs<double, true> : k_arnoldi_cgs<double, false>;
        allow_max_smem(kern);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFuseThreads, smem);
    } else {
        auto kern = cache ? k_arnoldi_cgs<float, true> : k_arnoldi_cgs<float, false>;
        allow_max_smem(kern);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFuseThreads, smem);
    }
    cudaGetLastError();
    if (e != cudaSuccess || per_sm < 1) return 0;
    return sms;
}

}  // namespace gbprop
