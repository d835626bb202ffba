// One Arnoldi step's classical Gram-Schmidt in a single cooperative kernel
// (pamp.h:317-345 without re-orthogonalisation; BLASIntegrationFunctor block
// InnerProduct + zgemv + norm, functors.h:182-241):
//     h = V_{0..J}^H w,   w <- w - V h,   beta = ||w||,   Hessenberg column J, breakdown test.
// The grid has one CTA per SM (co-resident by the cooperative launch).  CTA b owns the
// element chunk [b*C, (b+1)*C) of every basis vector: it reads its chunk of V once into
// shared memory (when it fits), forms its partial inner products, and after a grid
// barrier every CTA sums all CTAs' partials in the same fixed order (deterministic, the
// same h everywhere), updates its chunk of w from the cached V and writes its share of
// ||w||^2; CTA 0 writes the Hessenberg column and the counters.  beta = ||w|| is formed from
// those shares by the next solve, the first kernel that needs it (see launch_solve_inv).
// Versus separate dot / update / finalize kernels this reads V once instead of twice and
// removes two launches and two last-block reductions per Arnoldi step.
#include "gbprop_internal.h"
#include "gbprop_device.cuh"

#include <algorithm>
#include <cfloat>

namespace gbprop {

constexpr int kFuseThreads = 512;
constexpr long kBarrierSpinLimit = 1L << 24;   // polls (each an L2 round trip) before a barrier gives up

// Grid barrier for a co-resident grid on a counter that only grows within an Arnoldi step
// (zeroed before the step's first launch): barrier number t of the step completes when the
// counter reaches (t + 1) * nblocks.  One acquire-release atomic per CTA and acquire polls
// (1.2 us per barrier over 152 CTAs, against 2.3 us with full fences around a volatile
// sense flag).  Bounded: after kBarrierSpinLimit polls (or the handle's Ctrl::wait_limit, see
// wait_budget) it records ctrl->wait_timeout and returns false.
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned nblocks, unsigned t, Ctrl* ctrl) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        unsigned old;
        asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;" : "=r"(old) : "l"(bar) : "memory");
        const unsigned target = (t + 1) * nblocks;
        const long lim = wait_budget(ctrl, kBarrierSpinLimit);
        long it = 0;
        while ((int)(ld_acquire_gpu(bar) - target) < 0) {
            if (++it > lim) {
                ctrl->wait_timeout = 1;
                ok = 0;
                break;
            }
        }
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

// Phase C (CTA 0): the Hessenberg column J and the counters (pamp.h:305-345).  beta of the next
// vector, its breakdown test and 1/beta are formed from the ||w||^2 partials by the next solve
// (the first kernel that needs them), which saves a grid barrier here; H(J, J-1) = beta_J,
// recorded by the solve of this Arnoldi step, is written now.
__device__ __forceinline__ void cgs_finish(Ctrl* ctrl, double* H, const double* hs, int m, int J, int b) {
    if (b != 0) return;
    const int nv = J + 1;
    for (int k = threadIdx.x; k < nv; k += blockDim.x) {
        H[2 * ((size_t)k * m + J)] = hs[2 * k];
        H[2 * ((size_t)k * m + J) + 1] = hs[2 * k + 1];
        ctrl->h[2 * k] = hs[2 * k];
        ctrl->h[2 * k + 1] = hs[2 * k + 1];
    }
    if (threadIdx.x == 0) {
        ctrl->nbasis = nv;
        ctrl->operator_count++;
        if (J == 0) ctrl->inner_product_count++;
        if (J > 0) {
            H[2 * ((size_t)J * m + J - 1)] = ctrl->beta;
            H[2 * ((size_t)J * m + J - 1) + 1] = 0.0;
        }
    }
}

template <bool CACHE>
__global__ void __launch_bounds__(kFuseThreads) k_arnoldi_cgs(const double2* __restrict__ V, long n, int J, int m,
                                                              double2* __restrict__ w, double* __restrict__ part,
                                                              unsigned* bar, Ctrl* ctrl, double* H, int update,
                                                              int chunk) {
    using C = double2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double hs[2 * (kMaxBasis + 1)];
    __shared__ double red[kFuseThreads / 32];
    __shared__ __align__(8) unsigned long long s_bar;
    const int nv = J + 1, G = gridDim.x, b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long i0 = (long)b * chunk;
    const int cl = (int)max(0L, min((long)chunk, n - i0));
    // shared memory: w chunk | cached rows of V
    C* ws = reinterpret_cast<C*>(smem_raw);
    C* cache = reinterpret_cast<C*>(smem_raw + (((size_t)chunk * sizeof(C) + 15) & ~(size_t)15));
    // With the cache, the CTA's basis rows (written by kernels before the predecessor) are
    // copied in by bulk asynchronous copies issued before the dependency wait; w, the
    // predecessor's output, follows it and carries the barrier's one arrival (rows start on
    // 16-byte boundaries: 16-byte elements)
    const bool tma = CACHE && cl > 0;
    const unsigned row = (unsigned)cl * 16;
    if (tma) {
        if (tid == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&s_bar)) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();
        if (tid == 0) {
            asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;"
                         :: "r"(smem_u32(&s_bar)), "r"(row * (unsigned)nv) : "memory");
            for (int k = 0; k < nv; ++k) bulk_g2s(cache + (size_t)k * chunk, V + (size_t)k * n + i0, row, &s_bar);
        }
    }
    pdl_wait();
    if (ctrl->broken) {                              // uniform: written only between launches
        if (tma) {
            if (tid == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(smem_u32(&s_bar)) : "memory");
            mbar_wait0(&s_bar);                      // copies in flight land before exit
        }
        return;
    }
    const bool rnd = ctrl->round_matvec & 2;        // precision probe (FP64 handles)
    if (tma) {
        if (tid == 0) {
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                         :: "r"(smem_u32(&s_bar)), "r"(row) : "memory");
            bulk_g2s(ws, w + i0, row, &s_bar);
        }
        if (!__syncthreads_and(mbar_wait0(&s_bar, wait_budget(ctrl, kInvWaitLimit)))) {
            if (tid == 0) ctrl->wait_timeout = 1;
            mbar_wait0(&s_bar);                      // copies in flight land before exit
            return;
        }
    } else {
        for (int i = tid; i < cl; i += kFuseThreads) ws[i] = w[i0 + i];
        __syncthreads();
    }

    // ---- phase A: partial inner products, one warp per basis vector.  The FP64 pipe retires
    // one warp instruction per 16 SM cycles and its dependent latency is about as long, so two
    // accumulator pairs per warp keep it busy; every extra add is pipe time. ----------------
    for (int k = warp; k < nv; k += kFuseThreads / 32) {
        double ar = 0.0, ai = 0.0, br = 0.0, bi = 0.0;
        const C* vk = V + (size_t)k * n + i0;
        int i = lane;
        const C* ck = cache + (size_t)k * chunk;     // (staged rows when CACHE)
        for (; i + 96 < cl; i += 128) {
            C v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) v[u] = CACHE ? ck[i + 32 * u] : vk[i + 32 * u];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const C x = ws[i + 32 * u];
                if (u & 1) acc_dot64(br, bi, v[u].x, v[u].y, x.x, x.y);
                else acc_dot64(ar, ai, v[u].x, v[u].y, x.x, x.y);
            }
        }
        for (; i + 32 < cl; i += 64) {
            const C v = CACHE ? ck[i] : vk[i], u = CACHE ? ck[i + 32] : vk[i + 32];
            const C x = ws[i], y = ws[i + 32];
            acc_dot64(ar, ai, v.x, v.y, x.x, x.y);
            acc_dot64(br, bi, u.x, u.y, y.x, y.y);
        }
        if (i < cl) {
            const C v = CACHE ? ck[i] : vk[i];
            const C x = ws[i];
            acc_dot64(ar, ai, v.x, v.y, x.x, x.y);
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
    if (!grid_barrier(bar, G, J, ctrl)) return;   // the launch's only barrier: number J of the step

    // ---- phase B: h = sum of the partials (fixed order; tpv threads per value, a power of
    // two <= 32 so that each value's threads are consecutive lanes of one warp) --------------
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

    double nrm = 0.0;
    if (update) {
        // w -= V h on this chunk; ||w||^2 partial
        for (int i = tid; i < cl; i += kFuseThreads) {
            C r = ws[i];
            double sr0 = 0.0, si0 = 0.0, sr1 = 0.0, si1 = 0.0;
            int k = 0;
            for (; k + 1 < nv; k += 2) {
                const C a = CACHE ? cache[(size_t)k * chunk + i] : V[(size_t)k * n + i0 + i];
                const C c = CACHE ? cache[(size_t)(k + 1) * chunk + i] : V[(size_t)(k + 1) * n + i0 + i];
                sr0 = fma(a.x, hs[2 * k], sr0);
                sr0 = fma(-a.y, hs[2 * k + 1], sr0);
                si0 = fma(a.x, hs[2 * k + 1], si0);
                si0 = fma(a.y, hs[2 * k], si0);
                sr1 = fma(c.x, hs[2 * k + 2], sr1);
                sr1 = fma(-c.y, hs[2 * k + 3], sr1);
                si1 = fma(c.x, hs[2 * k + 3], si1);
                si1 = fma(c.y, hs[2 * k + 2], si1);
            }
            if (k < nv) {
                const C a = CACHE ? cache[(size_t)k * chunk + i] : V[(size_t)k * n + i0 + i];
                sr0 = fma(a.x, hs[2 * k], sr0);
                sr0 = fma(-a.y, hs[2 * k + 1], sr0);
                si0 = fma(a.x, hs[2 * k + 1], si0);
                si0 = fma(a.y, hs[2 * k], si0);
            }
            r.x -= (sr0 + sr1);
            r.y -= (si0 + si1);
            if (rnd) r = round_c64(r);
            w[i0 + i] = r;
            nrm = fma(r.x, r.x, nrm);
            nrm = fma(r.y, r.y, nrm);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
        if (lane == 0) red[warp] = nrm;
        __syncthreads();
        if (tid == 0) {
            double t = 0.0;
            for (int q = 0; q < kFuseThreads / 32; ++q) t += red[q];
            part[(size_t)nv * G * 2 + b] = t;     // beta is formed from these by the next solve
        }
    }
    cgs_finish(ctrl, H, hs, m, J, b);
}

// ---------------------------------------------------------------------------
// Complex64 basis (FP32-mixed path).  The same phases, with every inner product, partial
// sum and norm share formed by error-free FP32 transformations (hi + lo pairs): on this
// GPU the FP64 pipe retires two thread operations per clock per SM, so FP64 adds in
// reductions (every lane of every warp) cost as much as the products themselves.  The
// first vector comes split into FP32 pairs (v0s, float4 re_hi, im_hi, re_lo, im_lo);
// partials are float4 (re_hi, re_lo, im_hi, im_lo) per (vector, CTA).  Only single
// threads touch FP64 (the Hessenberg entries).
constexpr int kCgsWarps = kFuseThreads / 32;
constexpr int kCgsItems = 64;

template <bool CACHE>
__global__ void __launch_bounds__(kFuseThreads) k_arnoldi_cgs32(const float2* __restrict__ V,
                                                                const float4* __restrict__ v0s, long n, int J,
                                                                int m, float2* __restrict__ w,
                                                                float4* __restrict__ part, unsigned* bar,
                                                                Ctrl* ctrl, double* H, int update, int chunk) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ float4 psum[kCgsItems];
    __shared__ float2 hf[kMaxBasis + 1], hl[kMaxBasis + 1];
    __shared__ double hs[2 * (kMaxBasis + 1)];
    __shared__ float2 red[kCgsWarps];
    __shared__ __align__(8) unsigned long long s_bar;
    const int nv = J + 1, G = gridDim.x, b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const long i0 = (long)b * chunk;
    const int cl = (int)max(0L, min((long)chunk, n - i0));
    float2* ws = reinterpret_cast<float2*>(smem_raw);
    float4* c0 = reinterpret_cast<float4*>(smem_raw + (((size_t)chunk * sizeof(float2) + 15) & ~(size_t)15));
    float2* cache = reinterpret_cast<float2*>(reinterpret_cast<unsigned char*>(c0) + (v0s ? (size_t)chunk * 16 : 0));
    // With the cache, the CTA's whole share (w, the first vector, every basis row) arrives by
    // bulk asynchronous copies issued at once, so phase A waits one memory latency instead
    // of one per unrolled load round.  Row starts are 16-byte aligned when n is even (chunk
    // is a multiple of 8).
    const bool tma = CACHE && (n & 1) == 0 && cl > 0;
    const int k_first = v0s ? 1 : 0;                 // rows of V read (row 0 replaced by v0s)
    // The basis rows and the split first vector were written by kernels before the
    // predecessor, so their copies are issued before the dependency wait (overlapping the
    // predecessor's tail); w, the predecessor's output, and the control block after it.  The
    // barrier's single arrival comes with w's bytes, so the phase cannot complete early.
    const unsigned row = (unsigned)cl * 8;
    if (tma) {
        if (tid == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&s_bar)) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();
        if (tid == 0) {
            const unsigned bytes = row * (unsigned)((v0s ? 2 : 0) + (nv - k_first));
            if (bytes)
                asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;"
                             :: "r"(smem_u32(&s_bar)), "r"(bytes) : "memory");
            if (v0s) bulk_g2s(c0, v0s + i0, 2 * row, &s_bar);
            for (int k = k_first; k < nv; ++k) bulk_g2s(cache + (size_t)k * chunk, V + (size_t)k * n + i0, row, &s_bar);
        }
    }
    pdl_wait();
    if (ctrl->broken) {                              // uniform: written only between launches
        if (tma) {
            if (tid == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(smem_u32(&s_bar)) : "memory");
            mbar_wait0(&s_bar);                      // copies in flight land before exit
        }
        return;
    }
    if (tma) {
        if (tid == 0) {
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                         :: "r"(smem_u32(&s_bar)), "r"(row) : "memory");
            bulk_g2s(ws, w + i0, row, &s_bar);
        }
        if (!__syncthreads_and(mbar_wait0(&s_bar, wait_budget(ctrl, kInvWaitLimit)))) {
            if (tid == 0) ctrl->wait_timeout = 1;
            mbar_wait0(&s_bar);                      // copies in flight land before exit
            return;
        }
    } else {
        for (int i = tid; i < cl; i += kFuseThreads) ws[i] = w[i0 + i];
        __syncthreads();
    }

    // ---- phase A: partials of conj(v_k) . w; with fewer vectors than warps each vector's
    // chunk is cut into S slices (one warp each), summed in slice order afterwards
    const int S = nv >= kCgsWarps ? 1 : max(1, min(kCgsWarps / nv, cl / 32));
    const int sl = ((cl + S - 1) / S + 31) & ~31;
    for (int it = warp; it < nv * S; it += kCgsWarps) {
        const int k = it / S;
        const int e0 = min(cl, (it % S) * sl), e1 = min(cl, e0 + sl);
        float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f, sh = 0.f, sl2 = 0.f, th = 0.f, tl = 0.f;
        if (v0s && k == 0) {
            for (int i = e0 + lane; i < e1; i += 32) {
                const float4 a = tma ? c0[i] : v0s[i0 + i];
                if (CACHE && !tma) c0[i] = a;
                const float2 x = ws[i];
                // conj(a) x with a = hi + lo: re = ar xr + ai xi, im = ar xi - ai xr
                acc_prod(rh, rl, a.x, a.z, x.x);
                acc_prod(sh, sl2, a.y, a.w, x.y);
                acc_prod(ih, il, a.x, a.z, x.y);
                acc_prod(th, tl, -a.y, -a.w, x.x);
            }
        } else {
            const float2* vk = tma ? cache + (size_t)k * chunk : V + (size_t)k * n + i0;
            const bool fill = CACHE && !tma;
            int i = e0 + lane;
            for (; i + 96 < e1; i += 128) {
                float2 v[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) v[u] = vk[i + 32 * u];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    if (fill) cache[(size_t)k * chunk + i + 32 * u] = v[u];
                    const float2 x = ws[i + 32 * u];
                    if (u & 1) {
                        acc_prod(sh, sl2, v[u].x, 0.f, x.x);
                        acc_prod(sh, sl2, v[u].y, 0.f, x.y);
                        acc_prod(th, tl, v[u].x, 0.f, x.y);
                        acc_prod(th, tl, -v[u].y, 0.f, x.x);
                    } else {
                        acc_prod(rh, rl, v[u].x, 0.f, x.x);
                        acc_prod(rh, rl, v[u].y, 0.f, x.y);
                        acc_prod(ih, il, v[u].x, 0.f, x.y);
                        acc_prod(ih, il, -v[u].y, 0.f, x.x);
                    }
                }
            }
            for (; i < e1; i += 32) {
                const float2 v = vk[i];
                if (fill) cache[(size_t)k * chunk + i] = v;
                const float2 x = ws[i];
                acc_prod(rh, rl, v.x, 0.f, x.x);
                acc_prod(rh, rl, v.y, 0.f, x.y);
                acc_prod(ih, il, v.x, 0.f, x.y);
                acc_prod(ih, il, -v.y, 0.f, x.x);
            }
        }
        acc_pair(rh, rl, sh, sl2);
        acc_pair(ih, il, th, tl);
        warp_pair_sum(rh, rl);
        warp_pair_sum(ih, il);
        if (lane == 0) {
            const float4 r = make_float4(rh, rl, ih, il);
            if (S == 1) part[(size_t)k * G + b] = r;
            else psum[it] = r;
        }
    }
    if (S > 1) {
        __syncthreads();
        if (tid < nv) {
            float4 a = psum[tid * S];
            for (int q = 1; q < S; ++q) {
                const float4 c = psum[tid * S + q];
                acc_pair(a.x, a.y, c.x, c.y);
                acc_pair(a.z, a.w, c.z, c.w);
            }
            part[(size_t)tid * G + b] = a;
        }
    }
    if (!grid_barrier(bar, G, J, ctrl)) return;   // the launch's only barrier: number J of the step

    // ---- phase B: h_k = sum over the CTAs' partials, every CTA in the same fixed order:
    // tpv consecutive lanes per vector, lane q taking partials q, q + tpv, ... (four loads in
    // flight), then a compensated shuffle tree inside the group
    {
        int tpv = 32;
        while (tpv > 1 && tpv * nv > kFuseThreads) tpv >>= 1;
        const int k = tid / tpv, q = tid % tpv;
        float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
        if (k < nv) {
            // all of a lane's partials in flight at once (12 per round covers G <= 12 tpv);
            // zero padding leaves a compensated sum unchanged
            constexpr int kRound = 12;
            const float4* p = part + (size_t)k * G;
            for (int g0 = q; g0 < G; g0 += kRound * tpv) {
                float4 c[kRound];
#pragma unroll
                for (int u = 0; u < kRound; ++u) {
                    const int g = g0 + u * tpv;
                    c[u] = g < G ? __ldcg(p + g) : make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int u = 0; u < kRound; ++u) {
                    acc_pair(rh, rl, c[u].x, c[u].y);
                    acc_pair(ih, il, c[u].z, c[u].w);
                }
            }
        }
        for (int o = 1; o < tpv; o <<= 1) {
            const float a = __shfl_xor_sync(0xffffffffu, rh, o), c = __shfl_xor_sync(0xffffffffu, rl, o);
            const float d = __shfl_xor_sync(0xffffffffu, ih, o), e = __shfl_xor_sync(0xffffffffu, il, o);
            acc_pair(rh, rl, a, c);
            acc_pair(ih, il, d, e);
        }
        if (k < nv && q == 0) {
            float h1, l1, h2, l2;
            two_sum(rh, rl, h1, l1);                 // normalised pairs
            two_sum(ih, il, h2, l2);
            hf[k] = make_float2(h1, h2);
            hl[k] = make_float2(l1, l2);
            hs[2 * k] = (double)h1 + (double)l1;
            hs[2 * k + 1] = (double)h2 + (double)l2;
        }
    }
    __syncthreads();

    if (update) {
        // w -= V h on this chunk (the first vector's product to first order in the low
        // parts); ||w||^2 partial as an exact-square compensated sum
        float nh = 0.f, nl = 0.f;
        for (int i = tid; i < cl; i += kFuseThreads) {
            float2 r = ws[i];
            float sr = 0.f, si = 0.f, cr = 0.f, ci = 0.f;
            int k = 0;
            if (v0s) {
                const float4 a = CACHE ? c0[i] : v0s[i0 + i];
                const float2 H0 = hf[0], L0 = hl[0];
                acc_prod(sr, cr, H0.x, L0.x, a.x);
                acc_prod(sr, cr, -H0.y, -L0.y, a.y);
                acc_prod(si, ci, H0.y, L0.y, a.x);
                acc_prod(si, ci, H0.x, L0.x, a.y);
                cr = __fmaf_rn(a.z, H0.x, __fmaf_rn(-a.w, H0.y, cr));
                ci = __fmaf_rn(a.z, H0.y, __fmaf_rn(a.w, H0.x, ci));
                k = 1;
            }
            for (; k < nv; ++k) {
                const float2 vk = CACHE ? cache[(size_t)k * chunk + i] : V[(size_t)k * n + i0 + i];
                const float2 Hk = hf[k], Lk = hl[k];
                sr = fmaf(vk.x, Hk.x, sr);
                sr = fmaf(-vk.y, Hk.y, sr);
                si = fmaf(vk.x, Hk.y, si);
                si = fmaf(vk.y, Hk.x, si);
                cr = fmaf(vk.x, Lk.x, cr);
                cr = fmaf(-vk.y, Lk.y, cr);
                ci = fmaf(vk.x, Lk.y, ci);
                ci = fmaf(vk.y, Lk.x, ci);
            }
            r.x = r.x - (sr + cr);
            r.y = r.y - (si + ci);
            w[i0 + i] = r;
            acc_prod(nh, nl, r.x, 0.f, r.x);
            acc_prod(nh, nl, r.y, 0.f, r.y);
        }
        warp_pair_sum(nh, nl);
        if (lane == 0) red[warp] = make_float2(nh, nl);
        __syncthreads();
        if (tid == 0) {
            float a = 0.f, c = 0.f;
            for (int q = 0; q < kCgsWarps; ++q) acc_pair(a, c, red[q].x, red[q].y);
            part[(size_t)nv * G + b] = make_float4(a, c, 0.f, 0.f);   // for the next solve's beta
        }
    }
    cgs_finish(ctrl, H, hs, m, J, b);
}

size_t arnoldi_cgs_smem(int prec, long n, int nv, int grid, int with_v0, int cache) {
    const size_t es = prec == 0 ? sizeof(double2) : sizeof(float2);
    const long chunk = ((n + grid - 1) / grid + 7) / 8 * 8;
    size_t b = (((size_t)chunk * es + 15) & ~(size_t)15);
    if (with_v0) b += (size_t)chunk * 16;
    if (cache) b += (size_t)nv * chunk * es;
    return b;
}

template <typename Kern, typename... Args>
static cudaError_t cgs_coop_launch(Kern kern, int grid, size_t smem, cudaStream_t s, Args... args) {
    cudaError_t e = allow_max_smem(kern);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kFuseThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;   // the kernels call pdl_wait
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl_enabled() ? 2 : 1;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}

cudaError_t launch_arnoldi_cgs(int prec, const void* V, const void* v0, long n, int J, int m, void* w,
                               double* part, unsigned* bar, Ctrl* ctrl, double* H, int update, int grid, int cache,
                               cudaStream_t s) {
    count_launch();
    const int chunk = (int)(((n + grid - 1) / grid + 7) / 8 * 8);
    const size_t smem = arnoldi_cgs_smem(prec, n, J + 1, grid, v0 != nullptr, cache);
    if (prec == 0) {
        auto kern = cache ? k_arnoldi_cgs<true> : k_arnoldi_cgs<false>;
        return cgs_coop_launch(kern, grid, smem, s, (const double2*)V, n, J, m, (double2*)w, part, bar, ctrl, H, update,
                               chunk);
    }
    auto kern = cache ? k_arnoldi_cgs32<true> : k_arnoldi_cgs32<false>;
    return cgs_coop_launch(kern, grid, smem, s, (const float2*)V, (const float4*)v0, n, J, m, (float2*)w,
                           (float4*)part, bar, ctrl, H, update, chunk);
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
        auto kern = cache ? k_arnoldi_cgs<true> : k_arnoldi_cgs<false>;
        allow_max_smem(kern);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFuseThreads, smem);
    } else {
        auto kern = cache ? k_arnoldi_cgs32<true> : k_arnoldi_cgs32<false>;
        allow_max_smem(kern);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFuseThreads, smem);
    }
    cudaGetLastError();
    if (e != cudaSuccess || per_sm < 1) return 0;
    return sms;
}

// Grid of the cooperative form for a problem inside a batch, where other problems fill the
// GPU: the fewest CTAs whose chunk of V fits in shared memory (V read once per Arnoldi step),
// else one CTA per ~2048 elements without the cache; 0 when neither is co-resident.
int arnoldi_cgs_grid_batch(int prec, long n, int m, int with_v0, int* cache) {
    int dev = 0, sms = 0, coop = 0, optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (!coop || sms <= 0) return 0;
    for (int c = 1; c >= 0; --c) {
        int grid = c ? 1 : (int)std::min<long>(sms, std::max<long>(1, (n + 2047) / 2048));
        if (c)
            while (grid <= sms && arnoldi_cgs_smem(prec, n, m, grid, with_v0, 1) + 4096 > (size_t)optin) ++grid;
        if (grid > sms) continue;
        const size_t smem = arnoldi_cgs_smem(prec, n, m, grid, with_v0, c);
        if (smem + 4096 > (size_t)optin) continue;
        int per_sm = 0;
        cudaError_t e;
        if (prec == 0) {
            auto kern = c ? k_arnoldi_cgs<true> : k_arnoldi_cgs<false>;
            allow_max_smem(kern);
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFuseThreads, smem);
        } else {
            auto kern = c ? k_arnoldi_cgs32<true> : k_arnoldi_cgs32<false>;
            allow_max_smem(kern);
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFuseThreads, smem);
        }
        cudaGetLastError();
        if (e != cudaSuccess || per_sm < 1 || grid > per_sm * sms) continue;
        *cache = c;
        return grid;
    }
    return 0;
}

}  // namespace gbprop
