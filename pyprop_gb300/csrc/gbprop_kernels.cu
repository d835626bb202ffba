// CUDA kernels of the pAMP x TensorPotential propagation step, written for
// sm_103a (GB300).  On this part FP64 issue rate is ~1/58 of FP32 and a
// dependent FP64 FMA costs ~64 cycles, so the kernels are shaped to keep FP64
// work minimal and never put a long FP64 dependency chain on the critical path:
//   * the banded triangular solves along r (ztbsv in the reference) live in
//     gbprop_solve.cu;
//   * the tensor-potential matvec applies real band slots to complex vectors
//     (2 FMA per band entry instead of 4) with the source halo tile in smem;
//   * Gram-Schmidt runs as one cooperative kernel per Arnoldi step
//     (gbprop_cgs.cu); the dot / update / finalize kernels here serve
//     re-orthogonalisation and batches, with two-level reductions (block
//     partials + last-block finalize in fixed order: deterministic, no atomics
//     on values);
//   * the FP32-mixed path's exponential is in double-float (gbprop_expm.cu).
#include "gbprop_internal.h"
#include "gbprop_device.cuh"

#include <cooperative_groups.h>

#include <algorithm>
#include <cstdlib>
#include <cfloat>
#include <cmath>

namespace gbprop {

// Last-block detection for a two-level reduction: every block writes its
// partials, fences, and bumps `counter`; the block that sees gridDim-1 does
// the final sum (and resets the counter for the next launch).
__device__ __forceinline__ bool is_last_block(unsigned* counter) {
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned v = atomicAdd(counter, 1u);
        s_last = (v == gridDim.x - 1);
    }
    __syncthreads();
    if (s_last) __threadfence();
    return s_last != 0;
}

// Sum `nvals` values over all blocks' partials (stride `pstride` doubles per
// block) in fixed order; result into out[0..nvals).  Called by the last block.
// Threads are split into segments per value, each summing a strided subset with
// four independent accumulators (FP64 add latency is ~64 cycles on this part),
// then the segments are combined in shared memory.
__device__ void final_sum(const double* partials, int nblocks, int pstride, int nvals, double* out) {
    __shared__ double seg_sum[8][2 * kMaxBasis + 4];
    const int S = max(1, min(8, (int)blockDim.x / max(nvals, 1)));
    const int t = threadIdx.x;
    if (t < S * nvals) {
        const int v = t % nvals, sg = t / nvals;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
        int b = sg;
        for (; b + 3 * S < nblocks; b += 4 * S) {
            a0 += __ldcg(partials + (size_t)b * pstride + v);
            a1 += __ldcg(partials + (size_t)(b + S) * pstride + v);
            a2 += __ldcg(partials + (size_t)(b + 2 * S) * pstride + v);
            a3 += __ldcg(partials + (size_t)(b + 3 * S) * pstride + v);
        }
        for (; b < nblocks; b += S) a0 += __ldcg(partials + (size_t)b * pstride + v);
        seg_sum[sg][v] = (a0 + a1) + (a2 + a3);
    }
    __syncthreads();
    if (t < nvals) {
        double a = 0.0;
        for (int sg = 0; sg < S; ++sg) a += seg_sum[sg][t];
        out[t] = a;
    }
    __syncthreads();
}

// Reduce-scatter of 16 per-lane values across a warp: after 4 butterfly levels
// every lane holds the warp total of one value (16 adds per lane instead of 80
// for sixteen full shuffle reductions -- the lane-wide FP64 adds are issue-bound).
// Returns the total of value index `vidx` (valid on every lane; lanes 2k, 2k+1 agree).
__device__ __forceinline__ double warp_reduce_scatter16(const double (&acc)[16], int lane, int& vidx) {
    double a8[8];
    const bool u16 = lane & 16;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const double send = u16 ? acc[j] : acc[j + 8];
        const double keep = u16 ? acc[j + 8] : acc[j];
        a8[j] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
    double a4[4];
    const bool u8 = lane & 8;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const double send = u8 ? a8[j] : a8[j + 4];
        const double keep = u8 ? a8[j + 4] : a8[j];
        a4[j] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    double a2[2];
    const bool u4 = lane & 4;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const double send = u4 ? a4[j] : a4[j + 2];
        const double keep = u4 ? a4[j + 2] : a4[j];
        a2[j] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    const bool u2 = lane & 2;
    const double send = u2 ? a2[0] : a2[1];
    const double keep = u2 ? a2[1] : a2[0];
    double a1 = keep + __shfl_xor_sync(0xffffffffu, send, 2);
    a1 += __shfl_xor_sync(0xffffffffu, a1, 1);
    vidx = (u16 ? 8 : 0) + (u8 ? 4 : 0) + (u4 ? 2 : 0) + (u2 ? 1 : 0);
    return a1;
}

// Block-level sum of NV per-thread values into partials[blockIdx.x*pstride + off + k].
template <int NV>
__device__ void block_partials(double (&acc)[NV], int nvalid, double* partials, int pstride, int off) {
    __shared__ double red[32][NV];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double v = warp_sum(acc[k]);
        if (lane == 0) red[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < NV && threadIdx.x < nvalid) {
        double s = 0.0;
        for (int w = 0; w < nw; ++w) s += red[w][threadIdx.x];
        partials[(size_t)blockIdx.x * pstride + off + threadIdx.x] = s;
    }
    __syncthreads();
}

template <>
__device__ void block_partials<16>(double (&acc)[16], int nvalid, double* partials, int pstride, int off) {
    __shared__ double red16[32][16];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    int vidx;
    const double v = warp_reduce_scatter16(acc, lane, vidx);
    if ((lane & 1) == 0) red16[warp][vidx] = v;
    __syncthreads();
    if (threadIdx.x < 16 && threadIdx.x < nvalid) {
        double s0 = 0.0, s1 = 0.0;
        int w = 0;
        for (; w + 1 < nw; w += 2) { s0 += red16[w][threadIdx.x]; s1 += red16[w + 1][threadIdx.x]; }
        if (w < nw) s0 += red16[w][threadIdx.x];
        partials[(size_t)blockIdx.x * pstride + off + threadIdx.x] = s0 + s1;
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// tensor-potential matvec over the term list (TensorPotentialMultiply_*_BandNH)
// ---------------------------------------------------------------------------
// Tile shapes of the band kernel the autotuner chooses between:
// (threads per block, radial elements per thread).
// Variants 4 and 5 stage nothing: one thread per element reads its stencil through L1.
// Variants 6, 7, 8 (even nr): two elements per thread with vector loads (k_band_apply_x2 / _x2d;
// 128, 64, 32 threads).
constexpr int kBandVariants = 9;
__host__ __device__ constexpr int band_threads(int v) {
    return v == 0 ? 64 : v == 1 ? 128 : v == 2 ? 128 : v == 3 ? 256 : v == 4 ? 128 : 256;
}
__host__ __device__ constexpr int band_per(int v) { return v == 0 ? 2 : v == 1 ? 2 : v == 2 ? 4 : 1; }

// Output element of the band matvec; the precision probe (Ctrl::round_matvec, FP64 handles)
// rounds it to complex64 to measure what complex64 matvec outputs alone cost a propagation.
template <typename T>
__device__ __forceinline__ cx<T> band_out(T re, T im, const Ctrl* ctrl) {
    if constexpr (sizeof(T) == sizeof(double)) {
        if (ctrl && (ctrl->round_matvec & 1)) return mk<T>((double)(float)re, (double)(float)im);
    }
    return mk<T>(re, im);
}

// Term factor coef_t * (s if time-dependent) of term t, formed by one thread per CTA and
// shared: FP64 (cr, ci) for the FP64 band, the FP32 pairs (Cr, Crl, Ci, Cil) for the
// complex64 band.  Per thread this was ~10 FP64 instructions per term, a large share of
// the complex64 kernel on a GPU whose FP64 pipe retires two thread operations per clock.
template <typename T>
__device__ __forceinline__ void band_term_coef(const BandOp<T>& op, int t, const double* scal, double2* cd,
                                               float4* cf) {
    double cr = op.t_coef[2 * t], ci = op.t_coef[2 * t + 1];
    const int td = op.t_timedep[t];
    if (td) {
        const double sv = scal[td - 1];
        cr *= sv;
        ci *= sv;
    }
    if constexpr (sizeof(T) == sizeof(double)) {
        *cd = make_double2(cr, ci);
    } else {
        const float a = (float)cr, b = (float)ci;
        *cf = make_float4(a, (float)(cr - (double)a), b, (float)(ci - (double)b));
    }
}

// One block: destination row l = blockIdx.y, radial tile blockIdx.x.  For every term
// of row l the source row's tile (with a kb halo) is staged in shared memory; each
// thread accumulates PER elements with the band sum split into even/odd diagonals
// (four independent FMA chains per element to cover the FP64 latency).
template <typename T, int KB, int THREADS, int PER>
__global__ void __launch_bounds__(THREADS) k_band_apply(BandOp<T> op, const cx<T>* __restrict__ x,
                                                        cx<T>* __restrict__ y, const SchedEntry* __restrict__ sched,
                                                        const Ctrl* __restrict__ ctrl, Scalings scal_val,
                                                        int check_broken) {
    using C = cx<T>;
    constexpr int W = 2 * KB + 1;
    constexpr int TILE = THREADS * PER;
    __shared__ C sx[TILE + 2 * KB];
    __shared__ double2 s_cd;
    __shared__ float4 s_cf;
    pdl_wait();
    if (check_broken && ctrl->broken) return;
    const int l = blockIdx.y, i0 = blockIdx.x * TILE, tid = threadIdx.x;
    const int nr = op.nr;
    const bool kSplit = sizeof(T) < sizeof(double) && op.slots_lo != nullptr;
    T yr[PER], yi[PER], zr[PER], zi[PER];
#pragma unroll
    for (int e = 0; e < PER; ++e) { yr[e] = 0; yi[e] = 0; zr[e] = 0; zi[e] = 0; }
    const int t0 = op.row_ptr[l], t1 = op.row_ptr[l + 1];
    for (int t = t0; t < t1; ++t) {
        const size_t sbase = (size_t)op.t_src[t] * nr;
        __syncthreads();
        for (int j = tid; j < TILE + 2 * KB; j += THREADS) {
            const int g = i0 - KB + j;
            sx[j] = (g >= 0 && g < nr) ? x[sbase + g] : mk<T>(0, 0);
        }
        if (tid == 0) band_term_coef(op, t, sched ? sched[ctrl->step].scaling.s : scal_val.s, &s_cd, &s_cf);
        __syncthreads();
        const T* A = op.slots + (size_t)op.t_slot[t] * W * nr;
        T Cr, Ci;
        if constexpr (sizeof(T) == sizeof(double)) { Cr = s_cd.x; Ci = s_cd.y; }
        else { Cr = s_cf.x; Ci = s_cf.z; }
        if constexpr (sizeof(T) < sizeof(double)) {
            if (kSplit) {
                // complex64 path: error-free products and compensated sums of the band
                // (coefficient = hi + lo) and of the term factor, so the result is the FP64
                // operator applied to the complex64 source, rounded once.  The kinetic band's
                // large alternating entries make plain FP32 sums lose ~eps32 * sum|a s|.
                const float* Alo = op.slots_lo + (size_t)op.t_slot[t] * W * nr;
                const float Crl = s_cf.y, Cil = s_cf.w;
#pragma unroll
                for (int e = 0; e < PER; ++e) {
                    const int li = tid + e * THREADS;
                    const int i = i0 + li;
                    if (i < nr) {
                        // even and odd diagonals in separate compensated chains, merged exactly
                        float srh = 0.f, srl = 0.f, sih = 0.f, sil = 0.f;
                        float orh = 0.f, orl = 0.f, oih = 0.f, oil = 0.f;
#pragma unroll
                        for (int d = 0; d < W; ++d) {
                            const C v = sx[li + d];
                            const float a = __ldg(A + (size_t)d * nr + i), al = __ldg(Alo + (size_t)d * nr + i);
                            if (d & 1) {
                                acc_prod(orh, orl, a, al, v.x);
                                acc_prod(oih, oil, a, al, v.y);
                            } else {
                                acc_prod(srh, srl, a, al, v.x);
                                acc_prod(sih, sil, a, al, v.y);
                            }
                        }
                        float t;
                        two_sum(srh, orh, srh, t);
                        srl = __fadd_rn(__fadd_rn(srl, orl), t);
                        two_sum(sih, oih, sih, t);
                        sil = __fadd_rn(__fadd_rn(sil, oil), t);
                        if (Cr != 0.f || Crl != 0.f) {
                            acc_scaled(yr[e], zr[e], Cr, Crl, srh, srl);
                            acc_scaled(yi[e], zi[e], Cr, Crl, sih, sil);
                        }
                        if (Ci != 0.f || Cil != 0.f) {
                            acc_scaled(yr[e], zr[e], -Ci, -Cil, sih, sil);
                            acc_scaled(yi[e], zi[e], Ci, Cil, srh, srl);
                        }
                    }
                }
                continue;
            }
        }
#pragma unroll
        for (int e = 0; e < PER; ++e) {
            const int li = tid + e * THREADS;
            const int i = i0 + li;
            if (i < nr) {
                T a[W];
#pragma unroll
                for (int d = 0; d < W; ++d) a[d] = __ldg(A + (size_t)d * nr + i);
                T ar0 = 0, ai0 = 0, ar1 = 0, ai1 = 0;
#pragma unroll
                for (int d = 0; d < W; d += 2) {
                    const C v = sx[li + d];
                    ar0 = fma(a[d], v.x, ar0);
                    ai0 = fma(a[d], v.y, ai0);
                }
#pragma unroll
                for (int d = 1; d < W; d += 2) {
                    const C v = sx[li + d];
                    ar1 = fma(a[d], v.x, ar1);
                    ai1 = fma(a[d], v.y, ai1);
                }
                const T ar = ar0 + ar1, ai = ai0 + ai1;
                // a term's factor is real or imaginary (one part of a potential): skip the other
                if (Ci == T(0)) { yr[e] = fma(Cr, ar, yr[e]); yi[e] = fma(Cr, ai, yi[e]); }
                else if (Cr == T(0)) { yr[e] = fma(-Ci, ai, yr[e]); yi[e] = fma(Ci, ar, yi[e]); }
                else { yr[e] += Cr * ar - Ci * ai; yi[e] += Cr * ai + Ci * ar; }
            }
        }
    }
#pragma unroll
    for (int e = 0; e < PER; ++e) {
        const int i = i0 + tid + e * THREADS;
        if (i < nr) y[(size_t)l * nr + i] = band_out<T>(yr[e] + zr[e], yi[e] + zi[e], ctrl);
    }
}

// Unstaged form: thread = (row l, element i); every term's 2kb+1 source values come
// through the read-only/L1 path (a source element is shared by 2kb+1 neighbouring threads),
// so no block barrier ever waits on a global load.
template <typename T, int KB, int THREADS>
__global__ void __launch_bounds__(THREADS) k_band_apply_l1(BandOp<T> op, const cx<T>* __restrict__ x,
                                                           cx<T>* __restrict__ y, const SchedEntry* __restrict__ sched,
                                                           const Ctrl* __restrict__ ctrl, Scalings scal_val,
                                                           int check_broken) {
    using C = cx<T>;
    constexpr int W = 2 * KB + 1;
    constexpr int kTerms = 32;                      // term factors staged per round
    __shared__ double2 s_cd[kTerms];
    __shared__ float4 s_cf[kTerms];
    pdl_wait();
    if (check_broken && ctrl->broken) return;
    const int l = blockIdx.y, nr = op.nr;
    const int i = blockIdx.x * THREADS + threadIdx.x;
    const bool active = i < nr;
    const bool split = sizeof(T) < sizeof(double) && op.slots_lo != nullptr;
    T yr = 0, yi = 0, zr = 0, zi = 0;
    const int t0 = op.row_ptr[l], t1 = op.row_ptr[l + 1];
    for (int tg = t0; tg < t1; tg += kTerms) {
        const int tn = min(kTerms, t1 - tg);
        if (tg > t0) __syncthreads();
        if ((int)threadIdx.x < tn)
            band_term_coef(op, tg + threadIdx.x, sched ? sched[ctrl->step].scaling.s : scal_val.s, &s_cd[threadIdx.x],
                           &s_cf[threadIdx.x]);
        __syncthreads();
        if (!active) continue;
        for (int t = tg; t < tg + tn; ++t) {
            const C* xs = x + (size_t)op.t_src[t] * nr;
            const T* A = op.slots + (size_t)op.t_slot[t] * W * nr;
            T Cr, Ci;
            if constexpr (sizeof(T) == sizeof(double)) { Cr = s_cd[t - tg].x; Ci = s_cd[t - tg].y; }
            else { Cr = s_cf[t - tg].x; Ci = s_cf[t - tg].z; }
            C v[W];
#pragma unroll
            for (int d = 0; d < W; ++d) {
                const int g = i + d - KB;
                v[d] = (g >= 0 && g < nr) ? __ldg(xs + g) : mk<T>(0, 0);
            }
            if constexpr (sizeof(T) < sizeof(double)) {
                if (split) {
                    const float* Alo = op.slots_lo + (size_t)op.t_slot[t] * W * nr;
                    const float Crl = s_cf[t - tg].y, Cil = s_cf[t - tg].w;
                    float srh = 0.f, srl = 0.f, sih = 0.f, sil = 0.f, orh = 0.f, orl = 0.f, oih = 0.f, oil = 0.f;
#pragma unroll
                    for (int d = 0; d < W; ++d) {
                        const float a = __ldg(A + (size_t)d * nr + i), al = __ldg(Alo + (size_t)d * nr + i);
                        if (d & 1) {
                            acc_prod(orh, orl, a, al, v[d].x);
                            acc_prod(oih, oil, a, al, v[d].y);
                        } else {
                            acc_prod(srh, srl, a, al, v[d].x);
                            acc_prod(sih, sil, a, al, v[d].y);
                        }
                    }
                    float tt;
                    two_sum(srh, orh, srh, tt);
                    srl = __fadd_rn(__fadd_rn(srl, orl), tt);
                    two_sum(sih, oih, sih, tt);
                    sil = __fadd_rn(__fadd_rn(sil, oil), tt);
                    if (Cr != 0.f || Crl != 0.f) {
                        acc_scaled(yr, zr, Cr, Crl, srh, srl);
                        acc_scaled(yi, zi, Cr, Crl, sih, sil);
                    }
                    if (Ci != 0.f || Cil != 0.f) {
                        acc_scaled(yr, zr, -Ci, -Cil, sih, sil);
                        acc_scaled(yi, zi, Ci, Cil, srh, srl);
                    }
                    continue;
                }
            }
            T ar0 = 0, ai0 = 0, ar1 = 0, ai1 = 0;
#pragma unroll
            for (int d = 0; d < W; ++d) {
                const T a = __ldg(A + (size_t)d * nr + i);
                if (d & 1) { ar1 = fma(a, v[d].x, ar1); ai1 = fma(a, v[d].y, ai1); }
                else { ar0 = fma(a, v[d].x, ar0); ai0 = fma(a, v[d].y, ai0); }
            }
            const T ar = ar0 + ar1, ai = ai0 + ai1;
            if (Ci == T(0)) { yr = fma(Cr, ar, yr); yi = fma(Cr, ai, yi); }
            else if (Cr == T(0)) { yr = fma(-Ci, ai, yr); yi = fma(Ci, ar, yi); }
            else { yr += Cr * ar - Ci * ai; yi += Cr * ai + Ci * ar; }
        }
    }
    if (active) y[(size_t)l * nr + i] = band_out<T>(yr + zr, yi + zi, ctrl);
}

// Complex64 form with two neighbouring elements per thread (even nr): the hi and lo coefficients of
// both come in one 8-byte load per diagonal and the source window in 16-byte loads, so a warp issues
// about 2.4 times fewer load instructions per element than the one-element form (9% less time on the
// hydrogen operator; four elements per thread with 16-byte coefficient loads measured as slow as one,
// with 147 registers); the sums are the same compensated chains.
template <int KB, int THREADS>
__global__ void __launch_bounds__(THREADS) k_band_apply_x2(BandOp<float> op, const float2* __restrict__ x,
                                                            float2* __restrict__ y, const SchedEntry* __restrict__ sched,
                                                            const Ctrl* __restrict__ ctrl, Scalings scal_val,
                                                            int check_broken) {
    constexpr int EPT = 2;
    constexpr int W = 2 * KB + 1;
    constexpr int XS = KB + (KB & 1);               // the window starts at i - XS (even)
    constexpr int NX = XS + EPT / 2;                // 16-byte loads: 2 XS + EPT complex values
    constexpr int kTerms = 32;
    __shared__ float4 s_cf[kTerms];
    __shared__ double2 s_cd[kTerms];
    pdl_wait();
    if (check_broken && ctrl->broken) return;
    const int l = blockIdx.y, nr = op.nr;
    const int i = EPT * (blockIdx.x * THREADS + threadIdx.x);
    const bool active = i < nr;                     // nr even: i + 1 < nr too
    float yr[EPT], yi[EPT], zr[EPT], zi[EPT];
#pragma unroll
    for (int e = 0; e < EPT; ++e) { yr[e] = 0.f; yi[e] = 0.f; zr[e] = 0.f; zi[e] = 0.f; }
    const int t0 = op.row_ptr[l], t1 = op.row_ptr[l + 1];
    for (int tg = t0; tg < t1; tg += kTerms) {
        const int tn = min(kTerms, t1 - tg);
        if (tg > t0) __syncthreads();
        if ((int)threadIdx.x < tn)
            band_term_coef(op, tg + threadIdx.x, sched ? sched[ctrl->step].scaling.s : scal_val.s, &s_cd[threadIdx.x],
                           &s_cf[threadIdx.x]);
        __syncthreads();
        if (!active) continue;
        for (int t = tg; t < tg + tn; ++t) {
            const float2* xs = x + (size_t)op.t_src[t] * nr;
            const size_t so = (size_t)op.t_slot[t] * W * nr + i;
            float4 xw[NX];
#pragma unroll
            for (int k = 0; k < NX; ++k) {
                const int g = i - XS + 2 * k;
                xw[k] = (g >= 0 && g < nr) ? __ldg(reinterpret_cast<const float4*>(xs + g))
                                           : make_float4(0.f, 0.f, 0.f, 0.f);
            }
            float ah[W][EPT], al[W][EPT];
#pragma unroll
            for (int d = 0; d < W; ++d) {
                const float2 h2 = __ldg(reinterpret_cast<const float2*>(op.slots + so + (size_t)d * nr));
                const float2 l2 = __ldg(reinterpret_cast<const float2*>(op.slots_lo + so + (size_t)d * nr));
                ah[d][0] = h2.x;
                ah[d][1] = h2.y;
                al[d][0] = l2.x;
                al[d][1] = l2.y;
            }
            const float4 c = s_cf[t - tg];
#pragma unroll
            for (int e = 0; e < EPT; ++e) {
                float srh = 0.f, srl = 0.f, sih = 0.f, sil = 0.f, orh = 0.f, orl = 0.f, oih = 0.f, oil = 0.f;
#pragma unroll
                for (int d = 0; d < W; ++d) {
                    const int j = d - KB + XS + e;          // window offset of x[i + e + d - KB]
                    const float4 q = xw[j >> 1];
                    const float vx = (j & 1) ? q.z : q.x, vy = (j & 1) ? q.w : q.y;
                    if (d & 1) {
                        acc_prod(orh, orl, ah[d][e], al[d][e], vx);
                        acc_prod(oih, oil, ah[d][e], al[d][e], vy);
                    } else {
                        acc_prod(srh, srl, ah[d][e], al[d][e], vx);
                        acc_prod(sih, sil, ah[d][e], al[d][e], vy);
                    }
                }
                float tt;
                two_sum(srh, orh, srh, tt);
                srl = __fadd_rn(__fadd_rn(srl, orl), tt);
                two_sum(sih, oih, sih, tt);
                sil = __fadd_rn(__fadd_rn(sil, oil), tt);
                if (c.x != 0.f || c.y != 0.f) {
                    acc_scaled(yr[e], zr[e], c.x, c.y, srh, srl);
                    acc_scaled(yi[e], zi[e], c.x, c.y, sih, sil);
                }
                if (c.z != 0.f || c.w != 0.f) {
                    acc_scaled(yr[e], zr[e], -c.z, -c.w, sih, sil);
                    acc_scaled(yi[e], zi[e], c.z, c.w, srh, srl);
                }
            }
        }
    }
    if (active)
        *reinterpret_cast<float4*>(y + (size_t)l * nr + i) =
            make_float4(yr[0] + zr[0], yi[0] + zi[0], yr[1] + zr[1], yi[1] + zi[1]);
}

// The FP64 form with two neighbouring elements per thread (even nr): both elements' coefficients in
// one 16-byte load per diagonal, the source window shared between them.
template <int KB, int THREADS>
__global__ void __launch_bounds__(THREADS) k_band_apply_x2d(BandOp<double> op, const double2* __restrict__ x,
                                                            double2* __restrict__ y, const SchedEntry* __restrict__ sched,
                                                            const Ctrl* __restrict__ ctrl, Scalings scal_val,
                                                            int check_broken) {
    constexpr int W = 2 * KB + 1;
    constexpr int kTerms = 32;
    __shared__ float4 s_cf[kTerms];
    __shared__ double2 s_cd[kTerms];
    pdl_wait();
    if (check_broken && ctrl->broken) return;
    const int l = blockIdx.y, nr = op.nr;
    const int i = 2 * (blockIdx.x * THREADS + threadIdx.x);
    const bool active = i < nr;                     // nr even: i + 1 < nr too
    double yr0 = 0, yi0 = 0, yr1 = 0, yi1 = 0;
    const int t0 = op.row_ptr[l], t1 = op.row_ptr[l + 1];
    for (int tg = t0; tg < t1; tg += kTerms) {
        const int tn = min(kTerms, t1 - tg);
        if (tg > t0) __syncthreads();
        if ((int)threadIdx.x < tn)
            band_term_coef(op, tg + threadIdx.x, sched ? sched[ctrl->step].scaling.s : scal_val.s, &s_cd[threadIdx.x],
                           &s_cf[threadIdx.x]);
        __syncthreads();
        if (!active) continue;
        for (int t = tg; t < tg + tn; ++t) {
            const double2* xs = x + (size_t)op.t_src[t] * nr;
            const size_t so = (size_t)op.t_slot[t] * W * nr + i;
            double2 a[W];
#pragma unroll
            for (int d = 0; d < W; ++d) a[d] = __ldg(reinterpret_cast<const double2*>(op.slots + so + (size_t)d * nr));
            double2 v[W + 1];
#pragma unroll
            for (int k = 0; k <= W; ++k) {
                const int g = i + k - KB;
                v[k] = (g >= 0 && g < nr) ? __ldg(xs + g) : make_double2(0.0, 0.0);
            }
            double ar0 = 0, ai0 = 0, br0 = 0, bi0 = 0, ar1 = 0, ai1 = 0, br1 = 0, bi1 = 0;
#pragma unroll
            for (int d = 0; d < W; ++d) {
                if (d & 1) {
                    br0 = fma(a[d].x, v[d].x, br0);
                    bi0 = fma(a[d].x, v[d].y, bi0);
                    br1 = fma(a[d].y, v[d + 1].x, br1);
                    bi1 = fma(a[d].y, v[d + 1].y, bi1);
                } else {
                    ar0 = fma(a[d].x, v[d].x, ar0);
                    ai0 = fma(a[d].x, v[d].y, ai0);
                    ar1 = fma(a[d].y, v[d + 1].x, ar1);
                    ai1 = fma(a[d].y, v[d + 1].y, ai1);
                }
            }
            const double2 c = s_cd[t - tg];
            const double sr0 = ar0 + br0, si0 = ai0 + bi0, sr1 = ar1 + br1, si1 = ai1 + bi1;
            if (c.y == 0.0) {
                yr0 = fma(c.x, sr0, yr0); yi0 = fma(c.x, si0, yi0);
                yr1 = fma(c.x, sr1, yr1); yi1 = fma(c.x, si1, yi1);
            } else if (c.x == 0.0) {
                yr0 = fma(-c.y, si0, yr0); yi0 = fma(c.y, sr0, yi0);
                yr1 = fma(-c.y, si1, yr1); yi1 = fma(c.y, sr1, yi1);
            } else {
                yr0 += c.x * sr0 - c.y * si0; yi0 += c.x * si0 + c.y * sr0;
                yr1 += c.x * sr1 - c.y * si1; yi1 += c.x * si1 + c.y * sr1;
            }
        }
    }
    if (active) {
        y[(size_t)l * nr + i] = band_out<double>(yr0, yi0, ctrl);
        y[(size_t)l * nr + i + 1] = band_out<double>(yr1, yi1, ctrl);
    }
}

bool band_variant_vec_ok(int v, int nr) { return v < 6 || nr % 2 == 0; }

template <typename T, int KB, int V>
static void band_apply_v(const BandOp<T>& op, const void* x, void* y, const SchedEntry* sched, const Ctrl* ctrl,
                         const Scalings& scaling, int check_broken, cudaStream_t s) {
    if constexpr (V >= 6) {
        // (selected by the host only for complex64 operators with split coefficients and even nr;
        // vectors not on a 16-byte boundary take the one-element form)
        if constexpr (sizeof(T) < sizeof(double)) {
            constexpr int TH = V == 6 ? 128 : V == 7 ? 64 : 32;
            if (op.slots_lo != nullptr && op.nr % 2 == 0 && ((uintptr_t)x & 15) == 0 && ((uintptr_t)y & 15) == 0) {
                dim3 grid((op.nr / 2 + TH - 1) / TH, op.nl);
                launch_pdl(k_band_apply_x2<KB, TH>, grid, dim3(TH), 0, s, op, (const float2*)x, (float2*)y, sched,
                           ctrl, scaling, check_broken);
                return;
            }
        }
        if constexpr (sizeof(T) == sizeof(double)) {
            constexpr int TH = V == 6 ? 128 : V == 7 ? 64 : 32;
            if (op.nr % 2 == 0) {
                dim3 grid((op.nr / 2 + TH - 1) / TH, op.nl);
                launch_pdl(k_band_apply_x2d<KB, TH>, grid, dim3(TH), 0, s, op, (const double2*)x, (double2*)y,
                           sched, ctrl, scaling, check_broken);
                return;
            }
        }
        band_apply_v<T, KB, 4>(op, x, y, sched, ctrl, scaling, check_broken, s);
        return;
    }
    if constexpr (V >= 4) {
        constexpr int TH = band_threads(V);
        dim3 grid((op.nr + TH - 1) / TH, op.nl);
        launch_pdl(k_band_apply_l1<T, KB, TH>, grid, dim3(TH), 0, s, op, (const cx<T>*)x, (cx<T>*)y, sched, ctrl,
                   scaling, check_broken);
        return;
    }
    constexpr int TH = band_threads(V), PE = band_per(V);
    dim3 grid((op.nr + TH * PE - 1) / (TH * PE), op.nl);
    launch_pdl(k_band_apply<T, KB, TH, PE>, grid, dim3(TH), 0, s, op, (const cx<T>*)x, (cx<T>*)y, sched, ctrl, scaling,
               check_broken);
}

template <typename T, int KB>
static void band_apply_kb(const BandOp<T>& op, const void* x, void* y, const SchedEntry* sched, const Ctrl* ctrl,
                          const Scalings& scaling, int check_broken, cudaStream_t s) {
    switch (op.variant) {
        case 0: band_apply_v<T, KB, 0>(op, x, y, sched, ctrl, scaling, check_broken, s); break;
        case 2: band_apply_v<T, KB, 2>(op, x, y, sched, ctrl, scaling, check_broken, s); break;
        case 3: band_apply_v<T, KB, 3>(op, x, y, sched, ctrl, scaling, check_broken, s); break;
        case 4: band_apply_v<T, KB, 4>(op, x, y, sched, ctrl, scaling, check_broken, s); break;
        case 5: band_apply_v<T, KB, 5>(op, x, y, sched, ctrl, scaling, check_broken, s); break;
        case 6: band_apply_v<T, KB, 6>(op, x, y, sched, ctrl, scaling, check_broken, s); break;
        case 7: band_apply_v<T, KB, 7>(op, x, y, sched, ctrl, scaling, check_broken, s); break;
        case 8: band_apply_v<T, KB, 8>(op, x, y, sched, ctrl, scaling, check_broken, s); break;
        default: band_apply_v<T, KB, 1>(op, x, y, sched, ctrl, scaling, check_broken, s); break;
    }
}

template <typename T>
static cudaError_t band_apply_dispatch(const BandOp<T>& op, const void* x, void* y, const SchedEntry* sched,
                                       const Ctrl* ctrl, const Scalings& scaling, int check_broken, cudaStream_t s) {
    switch (op.kb) {
#define GB_KB(K) case K: band_apply_kb<T, K>(op, x, y, sched, ctrl, scaling, check_broken, s); break;
        GB_KB(1) GB_KB(2) GB_KB(3) GB_KB(4) GB_KB(5) GB_KB(6) GB_KB(7) GB_KB(8)
#undef GB_KB
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

int band_variant_count() { return kBandVariants; }

cudaError_t launch_band_apply(int arith, const void* opv, const void* x, void* y, const SchedEntry* sched,
                              const Ctrl* ctrl, const Scalings& scaling, int check_broken, cudaStream_t s) {
    count_launch();
    if (arith == 0) return band_apply_dispatch(*(const BandOp<double>*)opv, x, y, sched, ctrl, scaling, check_broken, s);
    return band_apply_dispatch(*(const BandOp<float>*)opv, x, y, sched, ctrl, scaling, check_broken, s);
}

// ---------------------------------------------------------------------------
// x <- U x  (ztbmv 'U','N'), elementwise parallel; U diagonal-major ud[d*nr + i] = U(i, i+d)
// ---------------------------------------------------------------------------
template <typename T, typename TI, typename TO>
__global__ void k_tbmv(int kd, const T* __restrict__ ud, int nl, int nr, const TI* __restrict__ in,
                       TO* __restrict__ out) {
    const size_t N = (size_t)nl * nr;
    for (size_t g = blockIdx.x * (size_t)blockDim.x + threadIdx.x; g < N; g += (size_t)gridDim.x * blockDim.x) {
        const int l = (int)(g / nr), i = (int)(g - (size_t)l * nr);
        const size_t base = (size_t)l * nr;
        T sr = 0, si = 0;
        for (int d = 0; d <= kd && i + d < nr; ++d) {
            const T u = ud[(size_t)d * nr + i];
            const TI v = in[base + i + d];
            sr = fma(u, (T)v.x, sr);
            si = fma(u, (T)v.y, si);
        }
        TO o;
        o.x = (typename elem_of<TO>::type)sr;
        o.y = (typename elem_of<TO>::type)si;
        out[g] = o;
    }
}

cudaError_t launch_tbmv(int arith, int kd, const void* ud, int nl, int nr, const void* in, int in_prec, void* out,
                        int out_prec, cudaStream_t s) {
    count_launch();
    const size_t N = (size_t)nl * nr;
    int blocks = (int)((N + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (arith != 0) return cudaErrorInvalidValue;
    if (in_prec == 0 && out_prec == 0)
        k_tbmv<double, double2, double2><<<blocks, 256, 0, s>>>(kd, (const double*)ud, nl, nr, (const double2*)in, (double2*)out);
    else if (in_prec == 1 && out_prec == 0)
        k_tbmv<double, float2, double2><<<blocks, 256, 0, s>>>(kd, (const double*)ud, nl, nr, (const float2*)in, (double2*)out);
    else if (in_prec == 1 && out_prec == 1)
        k_tbmv<double, float2, float2><<<blocks, 256, 0, s>>>(kd, (const double*)ud, nl, nr, (const float2*)in, (float2*)out);
    else
        k_tbmv<double, double2, float2><<<blocks, 256, 0, s>>>(kd, (const double*)ud, nl, nr, (const double2*)in, (float2*)out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// reductions: ||x||, Gram-Schmidt projections and updates
// ---------------------------------------------------------------------------
constexpr int kRedThreads = 512;
constexpr int kPStride = 2 * kMaxBasis + 4;   // doubles of partials per block

int grid_reduce_blocks() { return 152; }

bool pdl_enabled() {
    static const bool on = [] {
        const char* e = std::getenv("GBPROP_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}

// doubles of reduction scratch every launcher may use (update: up to 4*152 blocks of
// kPStride; dot: 2 values per (value, chunk) with at most ~304 + values chunks)
size_t partials_capacity() {
    const size_t upd = (size_t)4 * 152 * kPStride;
    const size_t dot = (size_t)2 * (kMaxBasis + 1) * (304 + kMaxBasis + 1);
    return upd > dot ? upd : dot;
}

template <typename CI>
__global__ void __launch_bounds__(kRedThreads) k_norm(const CI* __restrict__ x, long n, double* partials,
                                                      unsigned* counter, Ctrl* ctrl) {
    double acc[1] = {0.0};
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const CI v = x[i];
        const double re = (double)v.x, im = (double)v.y;
        acc[0] = fma(re, re, acc[0]);
        acc[0] = fma(im, im, acc[0]);
    }
    block_partials<1>(acc, 1, partials, kPStride, 0);
    if (is_last_block(counter)) {
        __shared__ double tot[1];
        final_sum(partials, gridDim.x, kPStride, 1, tot);
        if (threadIdx.x == 0) {
            const double b = sqrt(tot[0]);
            ctrl->beta0 = b;
            ctrl->beta = b;
            set_inv_beta(ctrl, b);
            if (!isfinite(b) || b == 0.0) ctrl->nonfinite = 1;
            *counter = 0;
        }
    }
}

// x <- x / ctrl->beta0 (Problem.AdvanceStep's psi.Normalize(), Problem.py:167-168, on the state in
// balanced coordinates, where the overlap-metric norm is the Euclidean one); beta0 = ||x|| from
// the k_norm launched just before.
__global__ void k_renormalize(double2* __restrict__ x, long n, const Ctrl* __restrict__ ctrl) {
    const double b = ctrl->beta0;
    if (!(b > 0.0) || !isfinite(b)) return;          // k_norm has flagged it
    const double ib = 1.0 / b;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double2 v = x[i];
        v.x *= ib;
        v.y *= ib;
        x[i] = v;
    }
}

cudaError_t launch_renormalize(double2* x, long n, double* partials, unsigned* counter, Ctrl* ctrl,
                               cudaStream_t s) {
    cudaError_t e = launch_norm(0, x, n, partials, counter, ctrl, s);
    if (e != cudaSuccess) return e;
    count_launch();
    k_renormalize<<<grid_reduce_blocks(), 256, 0, s>>>(x, n, ctrl);
    return cudaGetLastError();
}

cudaError_t launch_norm(int prec, const void* x, long n, double* partials, unsigned* counter, Ctrl* ctrl,
                        cudaStream_t s) {
    count_launch();
    const int blocks = grid_reduce_blocks();
    if (prec == 0) k_norm<double2><<<blocks, kRedThreads, 0, s>>>((const double2*)x, n, partials, counter, ctrl);
    else k_norm<float2><<<blocks, kRedThreads, 0, s>>>((const float2*)x, n, partials, counter, ctrl);
    return cudaGetLastError();
}

// h_k = <v_k, w> for k < nv (BLASIntegrationFunctor block InnerProduct, functors.h:236-240),
// and ||w||^2 as value nv when want_norm.
// Grid: (element chunks, values).  A block reduces ONE value over a contiguous chunk of
// 256*epl elements, with four interleaved accumulators per component, so the lane-wide
// FP64 reduction (the FP64 pipe is ~1/64 of FP32 on this part) is amortised over many
// products.  Block partials [value][chunk] are summed by the last block in fixed order.
// Destination: ctrl->h (mode 0; ||w|| into ctrl->orig_norm) or ctrl->h3 (mode 1, only
// while a re-orthogonalisation pass is requested), or hout[0..2nv] (+ hout[2nv] = ||w||^2)
// when ctrl is null.
constexpr int kDotThreads = 256;

// conj(vh + vl) * x accumulated as FP32 pairs (error-free products, low parts to first order)
__device__ __forceinline__ void dot_acc_pair(float& rh, float& rl, float& ih, float& il, float2 vh, float2 vl,
                                             float2 x) {
    acc_prod(rh, rl, vh.x, vl.x, x.x);
    acc_prod(rh, rl, vh.y, vl.y, x.y);
    acc_prod(ih, il, vh.x, vl.x, x.y);
    acc_prod(ih, il, -vh.y, -vl.y, x.x);
}

template <typename T>
__global__ void __launch_bounds__(kDotThreads) k_cgs_dot(const cx<T>* __restrict__ V,
                                                         const double2* __restrict__ v0,
                                                         const float4* __restrict__ v0s, long n, int nv,
                                                         const cx<T>* __restrict__ w, double* partials,
                                                         unsigned* counter, Ctrl* ctrl, int mode, int want_norm,
                                                         double* hout, int epl) {
    using C = cx<T>;
    __shared__ double red[kDotThreads / 32][2];
    if (ctrl) {
        if (ctrl->broken) return;
        if (mode == 1 && !ctrl->ro_go) return;
    }
    const int k = blockIdx.y, nchunks = gridDim.x, chunk = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const C* vk = k < nv ? V + (size_t)k * n : w;
    const bool row64 = v0 != nullptr && k == 0;     // complex64 basis with its first vector in FP64
    const long e0 = (long)chunk * kDotThreads * epl + tid;
    double ar[4] = {0.0, 0.0, 0.0, 0.0}, ai[4] = {0.0, 0.0, 0.0, 0.0};
    int t = 0;
    if constexpr (sizeof(T) < sizeof(double)) {
        if (!row64 || v0s) {
            // complex64 operands: error-free FP32 products and compensated FP32 sums (the
            // result equals the FP64 dot to ~2^-48); FP64 only for the block reduction.  The
            // FP64 first vector enters as its FP32-pair split (hi, lo), no FP64 instruction
            float rh0 = 0.f, rl0 = 0.f, ih0 = 0.f, il0 = 0.f, rh1 = 0.f, rl1 = 0.f, ih1 = 0.f, il1 = 0.f;
            auto vload = [&](long e, float2& vh, float2& vl) {
                if (row64) {
                    const float4 a = v0s[e];
                    vh = make_float2(a.x, a.y);
                    vl = make_float2(a.z, a.w);
                } else {
                    const C v = vk[e];
                    vh = make_float2(v.x, v.y);
                    vl = make_float2(0.f, 0.f);
                }
            };
            for (; t + 1 < epl; t += 2) {
                const long ea = e0 + (long)t * kDotThreads, eb = ea + kDotThreads;
                if (ea < n) {
                    float2 vh, vl;
                    vload(ea, vh, vl);
                    const C x = w[ea];
                    dot_acc_pair(rh0, rl0, ih0, il0, vh, vl, make_float2(x.x, x.y));
                }
                if (eb < n) {
                    float2 vh, vl;
                    vload(eb, vh, vl);
                    const C x = w[eb];
                    dot_acc_pair(rh1, rl1, ih1, il1, vh, vl, make_float2(x.x, x.y));
                }
            }
            for (; t < epl; ++t) {
                const long ea = e0 + (long)t * kDotThreads;
                if (ea < n) {
                    float2 vh, vl;
                    vload(ea, vh, vl);
                    const C x = w[ea];
                    dot_acc_pair(rh0, rl0, ih0, il0, vh, vl, make_float2(x.x, x.y));
                }
            }
            ar[0] = ((double)rh0 + (double)rl0) + ((double)rh1 + (double)rl1);
            ai[0] = ((double)ih0 + (double)il0) + ((double)ih1 + (double)il1);
            t = epl;
        }
    }
    for (; t + 3 < epl; t += 4) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const long e = e0 + (long)(t + q) * kDotThreads;
            if (e < n) {
                const C x = w[e];
                double vr, vi;
                if (row64) { const double2 v = v0[e]; vr = v.x; vi = v.y; }
                else { const C v = vk[e]; vr = (double)v.x; vi = (double)v.y; }
                const double xr = (double)x.x, xi = (double)x.y;
                ar[q] = fma(vr, xr, ar[q]);
                ar[q] = fma(vi, xi, ar[q]);
                ai[q] = fma(vr, xi, ai[q]);
                ai[q] = fma(-vi, xr, ai[q]);
            }
        }
    }
    for (; t < epl; ++t) {
        const long e = e0 + (long)t * kDotThreads;
        if (e < n) {
            const C x = w[e];
            double vr, vi;
            if (row64) { const double2 v = v0[e]; vr = v.x; vi = v.y; }
            else { const C v = vk[e]; vr = (double)v.x; vi = (double)v.y; }
            const double xr = (double)x.x, xi = (double)x.y;
            ar[0] = fma(vr, xr, ar[0]);
            ar[0] = fma(vi, xi, ar[0]);
            ai[0] = fma(vr, xi, ai[0]);
            ai[0] = fma(-vi, xr, ai[0]);
        }
    }
    double sr = (ar[0] + ar[1]) + (ar[2] + ar[3]);
    double si = (ai[0] + ai[1]) + (ai[2] + ai[3]);
    sr = warp_sum(sr);
    si = warp_sum(si);
    if (lane == 0) { red[warp][0] = sr; red[warp][1] = si; }
    __syncthreads();
    if (tid < 2) {
        double a = 0.0;
        for (int q = 0; q < kDotThreads / 32; ++q) a += red[q][tid];
        partials[((size_t)k * nchunks + chunk) * 2 + tid] = a;
    }
    // last block of the whole grid sums the chunks of every value in fixed order
    __shared__ int s_last;
    __threadfence();
    __syncthreads();
    if (tid == 0) {
        const unsigned v = atomicAdd(counter, 1u);
        s_last = (v == gridDim.x * gridDim.y - 1);
    }
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    const int nvals = gridDim.y;
    __shared__ double tot[2 * (kMaxBasis + 1)];
    for (int vv = warp; vv < 2 * nvals; vv += kDotThreads / 32) {
        const int kk = vv >> 1, c = vv & 1;
        double a = 0.0;
        for (int ch = lane; ch < nchunks; ch += 32) a += __ldcg(partials + ((size_t)kk * nchunks + ch) * 2 + c);
        a = warp_sum(a);
        if (lane == 0) tot[vv] = a;
    }
    __syncthreads();
    if (ctrl) {
        double* dst = mode ? ctrl->h3 : ctrl->h;
        for (int q = tid; q < 2 * nv; q += kDotThreads) dst[q] = tot[q];
        if (tid == 0 && want_norm && mode == 0) {
            ctrl->orig_norm = sqrt(tot[2 * nv]);
            ctrl->pre_norm = ctrl->orig_norm;
        }
    } else {
        for (int q = tid; q < 2 * nv; q += kDotThreads) hout[q] = tot[q];
        if (tid == 0 && want_norm) hout[2 * nv] = tot[2 * nv];
    }
    if (tid == 0) *counter = 0;
}

static void dot_shape(long n, int nvals, int* epl, int* nchunks) {
    const int target = max(1, 304 / max(nvals, 1));
    long e = (n + (long)kDotThreads * target - 1) / ((long)kDotThreads * target);
    if (e < 1) e = 1;
    *epl = (int)e;
    *nchunks = (int)((n + (long)kDotThreads * e - 1) / ((long)kDotThreads * e));
}

cudaError_t launch_cgs_dot(int prec, const void* V, const double2* v0, const float4* v0s, long n, int nv,
                           const void* w, double* partials, unsigned* counter, Ctrl* ctrl, int mode, int want_norm,
                           cudaStream_t s) {
    count_launch();
    const int nvals = nv + ((want_norm && mode == 0) ? 1 : 0);
    int epl, nch;
    dot_shape(n, nvals, &epl, &nch);
    dim3 grid(nch, nvals);
    if (prec == 0)
        k_cgs_dot<double><<<grid, kDotThreads, 0, s>>>((const double2*)V, nullptr, nullptr, n, nv, (const double2*)w,
                                                       partials, counter, ctrl, mode, want_norm, nullptr, epl);
    else
        k_cgs_dot<float><<<grid, kDotThreads, 0, s>>>((const float2*)V, v0, v0s, n, nv, (const float2*)w, partials,
                                                      counter, ctrl, mode, want_norm, nullptr, epl);
    return cudaGetLastError();
}

size_t block_inner_scratch_doubles(long n, int nvals) {
    int epl, nch;
    dot_shape(n, nvals, &epl, &nch);
    return (size_t)2 * nvals * nch;
}

cudaError_t launch_block_inner(int prec, const void* V, long n, int nv, const void* w, int want_norm, double* out,
                               double* partials, unsigned* counter, cudaStream_t s) {
    count_launch();
    const int nvals = nv + (want_norm ? 1 : 0);
    int epl, nch;
    dot_shape(n, nvals, &epl, &nch);
    dim3 grid(nch, nvals);
    if (prec == 0)
        k_cgs_dot<double><<<grid, kDotThreads, 0, s>>>((const double2*)V, nullptr, nullptr, n, nv, (const double2*)w,
                                                       partials, counter, nullptr, 0, want_norm, out, epl);
    else
        k_cgs_dot<float><<<grid, kDotThreads, 0, s>>>((const float2*)V, nullptr, nullptr, n, nv, (const float2*)w,
                                                      partials, counter, nullptr, 0, want_norm, out, epl);
    return cudaGetLastError();
}

// w <- w - V h  (zgemv 'N' + zaxpy, pamp.h:330-332) and ||w||.
// mode 0: primary pass (h), sets resid_norm and the re-orthogonalisation request
//         (pamp.h:369: resid < 0.717 * orig) when mode bit 1 (double orth) is set;
// mode 1: re-orthogonalisation pass (h3), h += h3, orig <- resid, resid <- ||w||.
// The basis loads of four vectors are issued together per step of the k loop.
constexpr int kUpdThreads = 256;

__device__ void arnoldi_finalize_block(Ctrl* ctrl, double* H, int m, int J, int double_orth, double brk_tol);

// mode bit 2 (primary pass without re-orthogonalisation): the last block also writes the
// Hessenberg column J, the next beta and the breakdown decision (k_arnoldi_finalize), one
// launch fewer per Arnoldi step.
template <typename T>
__global__ void __launch_bounds__(kUpdThreads) k_cgs_update(const cx<T>* __restrict__ V,
                                                            const double2* __restrict__ v0,
                                                            const float4* __restrict__ v0s, long n, int nv,
                                                            cx<T>* __restrict__ w, double* partials,
                                                            unsigned* counter, Ctrl* ctrl, int mode, double* H,
                                                            int m, double brk_tol) {
    using C = cx<T>;
    __shared__ C hs[kMaxBasis];
    __shared__ C hl[kMaxBasis];
    if (ctrl->broken) return;
    const int pass = mode & 1;
    const int dorth = (mode >> 1) & 1;
    if (pass == 1 && !ctrl->ro_go) return;
    const double* h = pass ? ctrl->h3 : ctrl->h;
    // complex64 basis: the coefficients keep their FP32 rounding remainders (hl), so the
    // vector subtracted is V h with the FP64 h of the Hessenberg matrix
    constexpr bool kSplit = sizeof(T) < sizeof(double);
    for (int k = threadIdx.x; k < nv; k += blockDim.x) {
        const T a = (T)h[2 * k], b = (T)h[2 * k + 1];
        hs[k] = mk<T>(a, b);
        hl[k] = mk<T>((T)(h[2 * k] - (double)a), (T)(h[2 * k + 1] - (double)b));
    }
    __syncthreads();
    double acc[1] = {0.0};
    float nh = 0.f, nl = 0.f;                      // ||w||^2 as an FP32 pair (complex64 basis)
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        T sr[4] = {0, 0, 0, 0}, si[4] = {0, 0, 0, 0};
        T cr = 0, ci = 0;                          // remainder sums (complex64 basis only)
        int k = 0;
        if (v0) {                                    // first vector kept in FP64: hi + lo parts
            const C hk = hs[0], hlk = hl[0];
            T ax, ay, bx, by;
            if (v0s) {                               // its FP32-pair split (no FP64 instruction)
                const float4 a = v0s[i];
                ax = (T)a.x; ay = (T)a.y; bx = (T)a.z; by = (T)a.w;
            } else {
                const double2 a = v0[i];
                ax = (T)a.x; ay = (T)a.y;
                bx = (T)(a.x - (double)ax); by = (T)(a.y - (double)ay);
            }
            sr[0] = fma(ax, hk.x, sr[0]);
            sr[0] = fma(-ay, hk.y, sr[0]);
            si[0] = fma(ax, hk.y, si[0]);
            si[0] = fma(ay, hk.x, si[0]);
            cr = fma(bx, hk.x, cr); cr = fma(-by, hk.y, cr); cr = fma(ax, hlk.x, cr); cr = fma(-ay, hlk.y, cr);
            ci = fma(bx, hk.y, ci); ci = fma(by, hk.x, ci); ci = fma(ax, hlk.y, ci); ci = fma(ay, hlk.x, ci);
            k = 1;
        }
        for (; k + 3 < nv; k += 4) {
            C v[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] = V[(size_t)(k + q) * n + i];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const C hk = hs[k + q];
                sr[q] = fma(v[q].x, hk.x, sr[q]);
                sr[q] = fma(-v[q].y, hk.y, sr[q]);
                si[q] = fma(v[q].x, hk.y, si[q]);
                si[q] = fma(v[q].y, hk.x, si[q]);
                if (kSplit) {
                    const C hlk = hl[k + q];
                    cr = fma(v[q].x, hlk.x, cr);
                    cr = fma(-v[q].y, hlk.y, cr);
                    ci = fma(v[q].x, hlk.y, ci);
                    ci = fma(v[q].y, hlk.x, ci);
                }
            }
        }
        for (; k < nv; ++k) {
            const C vk = V[(size_t)k * n + i];
            const C hk = hs[k];
            sr[0] = fma(vk.x, hk.x, sr[0]);
            sr[0] = fma(-vk.y, hk.y, sr[0]);
            si[0] = fma(vk.x, hk.y, si[0]);
            si[0] = fma(vk.y, hk.x, si[0]);
            if (kSplit) {
                const C hlk = hl[k];
                cr = fma(vk.x, hlk.x, cr);
                cr = fma(-vk.y, hlk.y, cr);
                ci = fma(vk.x, hlk.y, ci);
                ci = fma(vk.y, hlk.x, ci);
            }
        }
        C r = w[i];
        r.x -= ((sr[0] + sr[1]) + (sr[2] + sr[3])) + cr;
        r.y -= ((si[0] + si[1]) + (si[2] + si[3])) + ci;
        if constexpr (!kSplit) {
            if (ctrl->round_matvec & 2) r = round_c64(r);
        }
        w[i] = r;
        if constexpr (kSplit) {
            acc_prod(nh, nl, r.x, 0.f, r.x);
            acc_prod(nh, nl, r.y, 0.f, r.y);
        } else {
            acc[0] = fma((double)r.x, (double)r.x, acc[0]);
            acc[0] = fma((double)r.y, (double)r.y, acc[0]);
        }
    }
    if constexpr (kSplit) acc[0] = (double)nh + (double)nl;
    block_partials<1>(acc, 1, partials, kPStride, 0);
    if (is_last_block(counter)) {
        __shared__ double tot[1];
        final_sum(partials, gridDim.x, kPStride, 1, tot);
        if (threadIdx.x == 0) {
            const double resid = sqrt(tot[0]);
            if (!isfinite(resid)) ctrl->nonfinite = 1;
            if (pass == 0) {
                ctrl->resid_norm = resid;
                ctrl->ro_count = 0;
                ctrl->ro_go = dorth && (fabs(resid) < 0.717 * fabs(ctrl->orig_norm));
            } else {
                ctrl->orthogonalization_count++;
                ctrl->ro_count++;
                ctrl->orig_norm = ctrl->resid_norm;
                ctrl->resid_norm = resid;
                // the reference loop runs at most MaxOrthogonalizationCount = 3 passes (pamp.h:75,375)
                ctrl->ro_go = (fabs(resid) < 0.717 * fabs(ctrl->orig_norm)) ? 1 : 0;
            }
            *counter = 0;
        }
        if (pass == 1) {
            __syncthreads();
            for (int k = threadIdx.x; k < 2 * nv; k += blockDim.x) ctrl->h[k] += ctrl->h3[k];
        }
        if (mode & 4) {
            __syncthreads();
            arnoldi_finalize_block(ctrl, H, m, nv - 1, 0, brk_tol);
        }
    }
}

cudaError_t launch_cgs_update(int prec, const void* V, const double2* v0, const float4* v0s, long n, int nv, void* w,
                              double* partials, unsigned* counter, Ctrl* ctrl, int mode, cudaStream_t s, double* H,
                              int m, double brk_tol) {
    count_launch();
    int blocks = (int)((n + kUpdThreads - 1) / kUpdThreads);
    if (blocks > grid_reduce_blocks() * 4) blocks = grid_reduce_blocks() * 4;
    if (prec == 0)
        k_cgs_update<double><<<blocks, kUpdThreads, 0, s>>>((const double2*)V, nullptr, nullptr, n, nv, (double2*)w,
                                                            partials, counter, ctrl, mode, H, m, brk_tol);
    else
        k_cgs_update<float><<<blocks, kUpdThreads, 0, s>>>((const float2*)V, v0, v0s, n, nv, (float2*)w, partials,
                                                           counter, ctrl, mode, H, m, brk_tol);
    return cudaGetLastError();
}

// Writes Hessenberg column J, the next beta and the happy-breakdown decision
// (pamp.h:305-315, 345).  One block (its threads share the column).
__device__ void arnoldi_finalize_block(Ctrl* ctrl, double* H, int m, int J, int double_orth, double brk_tol) {
    const int nv = J + 1;
    for (int k = threadIdx.x; k < nv; k += blockDim.x) {
        H[2 * ((size_t)k * m + J)] = ctrl->h[2 * k];
        H[2 * ((size_t)k * m + J) + 1] = ctrl->h[2 * k + 1];
    }
    if (threadIdx.x == 0) {
        ctrl->nbasis = nv;
        ctrl->operator_count++;
        if (J == 0) ctrl->inner_product_count++;
        // after the third pass the reference counts once more and stops (pamp.h:372-381)
        if (double_orth && ctrl->ro_go && ctrl->ro_count >= 3) ctrl->orthogonalization_count++;
        if (J + 1 < m) {
            const double beta = ctrl->resid_norm;
            if (!isfinite(beta)) ctrl->nonfinite = 1;
            if (fabs(beta) < brk_tol) {
                ctrl->broken = 1;
                ctrl->breakdown_count++;
            } else {
                H[2 * ((size_t)(J + 1) * m + J)] = beta;
                H[2 * ((size_t)(J + 1) * m + J) + 1] = 0.0;
                ctrl->beta = beta;
                set_inv_beta(ctrl, beta);
            }
        }
    }
}

__global__ void k_arnoldi_finalize(Ctrl* ctrl, double* H, int m, int J, int double_orth, double brk_tol) {
    if (ctrl->broken) return;
    arnoldi_finalize_block(ctrl, H, m, J, double_orth, brk_tol);
}

cudaError_t launch_arnoldi_finalize(Ctrl* ctrl, double* H, int m, int J, int double_orth, double brk_tol,
                                    cudaStream_t s) {
    count_launch();
    k_arnoldi_finalize<<<1, 64, 0, s>>>(ctrl, H, m, J, double_orth, brk_tol);
    return cudaGetLastError();
}

__global__ void k_step_begin(Ctrl* ctrl, double* H, int m) {
    for (int k = threadIdx.x; k < 2 * m * m; k += blockDim.x) H[k] = 0.0;
    if (threadIdx.x == 0) {
        ctrl->broken = 0;
        ctrl->nbasis = 0;
        ctrl->ro_go = 0;
        ctrl->ro_count = 0;
    }
}

cudaError_t launch_step_begin(Ctrl* ctrl, double* H, int m, cudaStream_t s) {
    count_launch();
    k_step_begin<<<1, 256, 0, s>>>(ctrl, H, m);
    return cudaGetLastError();
}

__global__ void k_step_end(Ctrl* ctrl) {
    ctrl->step++;
    ctrl->step_count++;
}

cudaError_t launch_step_end(Ctrl* ctrl, cudaStream_t s) {
    count_launch();
    k_step_end<<<1, 1, 0, s>>>(ctrl);
    return cudaGetLastError();
}

__global__ void k_gather_flags(Ctrl* const* ctrls, int count, int* out) {
    __shared__ int s_f[4];
    if (threadIdx.x < 4) s_f[threadIdx.x] = threadIdx.x == 3 ? 0x7fffffff : 0;
    __syncthreads();
    for (int p = threadIdx.x; p < count; p += blockDim.x) {
        const Ctrl* c = ctrls[p];
        const int lu = c->lu_info, nf = c->nonfinite, to = c->wait_timeout;
        if (lu) atomicMax(&s_f[0], lu);
        if (nf) atomicMax(&s_f[1], nf);
        if (to) atomicMax(&s_f[2], to);
        if (lu || nf || to) atomicMin(&s_f[3], p);
    }
    __syncthreads();
    if (threadIdx.x < 3) out[threadIdx.x] = s_f[threadIdx.x];
    if (threadIdx.x == 3) out[3] = s_f[3] == 0x7fffffff ? 0 : s_f[3] + 1;
}

cudaError_t launch_gather_flags(Ctrl* const* ctrls, int count, int* out, cudaStream_t s) {
    count_launch();
    k_gather_flags<<<1, 256, 0, s>>>(ctrls, count, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Hessenberg exponential: pAMP::ScalingPadeExponential + PadeExponential
// (pamp.h:430-564), FP64, one CTA.  Matrices are row-major m*m complex in smem.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 cmulz(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ void smem_matmul(int m, const double2* A, const double2* B, double2* Cm) {
    for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
        const int r = idx / m, c = idx - r * m;
        double sr = 0.0, si = 0.0;
        for (int k = 0; k < m; ++k) {
            const double2 a = A[r * m + k], b = B[k * m + c];
            sr = fma(a.x, b.x, sr);
            sr = fma(-a.y, b.y, sr);
            si = fma(a.x, b.y, si);
            si = fma(a.y, b.x, si);
        }
        Cm[idx] = make_double2(sr, si);
    }
    __syncthreads();
}

__device__ __forceinline__ double cabs1d(double2 a) { return fabs(a.x) + fabs(a.y); }
__device__ __forceinline__ double2 cadd2(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 conjz(double2 a) { return make_double2(a.x, -a.y); }

__device__ double2 cdivz(double2 a, double2 b) {
    // Smith's algorithm
    if (fabs(b.x) >= fabs(b.y)) {
        const double q = b.y / b.x, d = b.x + b.y * q;
        return make_double2((a.x + a.y * q) / d, (a.y - a.x * q) / d);
    }
    const double q = b.x / b.y, d = b.y + b.x * q;
    return make_double2((a.x * q + a.y) / d, (a.y * q - a.x) / d);
}

__global__ void __launch_bounds__(256) k_expm(Ctrl* ctrl, double* Hg, int m, const SchedEntry* sched) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int mm = m * m;
    double2* A = reinterpret_cast<double2*>(smem_raw);
    double2* A2 = A + mm;
    double2* P = A2 + mm;
    double2* Q = P + mm;
    double2* T = Q + mm;
    __shared__ double red[8];
    __shared__ int piv[kMaxBasis];
    __shared__ int s_p;
    __shared__ double s_c[8];
    const int tid = threadIdx.x;
    const SchedEntry se = sched[ctrl->step];
    // HessenbergMatrix *= -dt * i   (pamp.h:634), kept in global for GetHessenbergMatrix
    const double2 f = make_double2(se.dt_im, -se.dt_re);
    double mx = 0.0;
    for (int k = tid; k < mm; k += blockDim.x) {
        const double2 h = make_double2(Hg[2 * k], Hg[2 * k + 1]);
        const double2 a = cmulz(h, f);
        Hg[2 * k] = a.x;
        Hg[2 * k + 1] = a.y;
        A[k] = a;
        mx = fmax(mx, hypot(a.x, a.y));
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0) red[tid >> 5] = mx;
    __syncthreads();
    if (tid == 0) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v = fmax(v, red[w]);
        int s = v > 0.0 ? (int)ceil(log2(v)) : 0;
        if (s < 0) s = 0;
        s_p = s;
        // Pade coefficients, order 6 (pamp.h:491-495)
        const int order = 6;
        s_c[0] = 1.0;
        for (int i = 0; i < order; ++i) s_c[i + 1] = s_c[i] * (double)(order - i) / (double)((i + 1) * (2 * order - i));
    }
    __syncthreads();
    const int sorder = s_p;
    const double sc = pow(2.0, (double)sorder);
    for (int k = tid; k < mm; k += blockDim.x) { A[k].x /= sc; A[k].y /= sc; }
    __syncthreads();
    smem_matmul(m, A, A, A2);
    // Horner in A^2 (pamp.h:497-539).  The first product of each polynomial is
    // with a scalar multiple of I and is formed directly (exactly equal).
    const int order = 6;
    for (int k = tid; k < mm; k += blockDim.x) {
        Q[k] = make_double2(s_c[order] * A2[k].x, s_c[order] * A2[k].y);       // i = 4 (odd step)
        P[k] = make_double2(s_c[order - 1] * A2[k].x, s_c[order - 1] * A2[k].y); // i = 3
    }
    __syncthreads();
    for (int r = tid; r < m; r += blockDim.x) { Q[r * m + r].x += s_c[4]; P[r * m + r].x += s_c[3]; }
    __syncthreads();
    // i = 2: Q = Q A2 + c2 I ; i = 1: P = P A2 + c1 I ; i = 0: Q = Q A2 + c0 I
    smem_matmul(m, Q, A2, T);
    for (int k = tid; k < mm; k += blockDim.x) Q[k] = T[k];
    __syncthreads();
    for (int r = tid; r < m; r += blockDim.x) Q[r * m + r].x += s_c[2];
    __syncthreads();
    smem_matmul(m, P, A2, T);
    for (int k = tid; k < mm; k += blockDim.x) P[k] = T[k];
    __syncthreads();
    for (int r = tid; r < m; r += blockDim.x) P[r * m + r].x += s_c[1];
    __syncthreads();
    smem_matmul(m, Q, A2, T);
    for (int k = tid; k < mm; k += blockDim.x) Q[k] = T[k];
    __syncthreads();
    for (int r = tid; r < m; r += blockDim.x) Q[r * m + r].x += s_c[0];
    __syncthreads();
    // odd == false at loop end for order 6: P = P A (pamp.h:530-539)
    smem_matmul(m, P, A, T);
    for (int k = tid; k < mm; k += blockDim.x) {
        P[k] = T[k];
        Q[k] = make_double2(Q[k].x - T[k].x, Q[k].y - T[k].y);   // Q = Q - P
    }
    __syncthreads();
    // zgetrf: LU with partial pivoting on |re|+|im| (first maximum), rows swapped whole
    int info = 0;
    for (int k = 0; k < m; ++k) {
        if (tid < 32) {
            double best = -1.0;
            int bi = k;
            for (int r = k + tid; r < m; r += 32) {
                const double v = cabs1d(Q[r * m + k]);
                if (v > best) { best = v; bi = r; }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (tid == 0) { piv[k] = bi; s_p = (best == 0.0) ? -1 : bi; }
        }
        __syncthreads();
        const int p = s_p;
        if (p < 0) { if (!info) info = k + 1; __syncthreads(); continue; }
        if (p != k)
            for (int c = tid; c < m; c += blockDim.x) {
                const double2 t = Q[k * m + c];
                Q[k * m + c] = Q[p * m + c];
                Q[p * m + c] = t;
            }
        __syncthreads();
        const double2 inv = cdivz(make_double2(1.0, 0.0), Q[k * m + k]);
        for (int r = k + 1 + tid; r < m; r += blockDim.x) Q[r * m + k] = cmulz(Q[r * m + k], inv);
        __syncthreads();
        const int rem = m - k - 1;
        for (int idx = tid; idx < rem * rem; idx += blockDim.x) {
            const int r = k + 1 + idx / rem, c = k + 1 + idx % rem;
            const double2 fr = Q[r * m + k], u = Q[k * m + c];
            double2 q = Q[r * m + c];
            q.x -= fr.x * u.x - fr.y * u.y;
            q.y -= fr.x * u.y + fr.y * u.x;
            Q[r * m + c] = q;
        }
        __syncthreads();
    }
    if (!info && ctrl->inject_lu) info = m;       // host-set test hook: report a zero last pivot
    if (info) {
        if (tid == 0 && !ctrl->nonfinite) ctrl->lu_info = info;   // a non-finite matrix is the cause
    } else {
        // zgetrs 'N': apply the row interchanges to P, then L y = b, U x = y (column-parallel axpy form)
        for (int k = 0; k < m; ++k) {
            const int p = piv[k];
            if (p != k)
                for (int c = tid; c < m; c += blockDim.x) {
                    const double2 t = P[k * m + c];
                    P[k * m + c] = P[p * m + c];
                    P[p * m + c] = t;
                }
            __syncthreads();
        }
        for (int r = 0; r < m; ++r) {
            for (int idx = tid; idx < (m - r - 1) * m; idx += blockDim.x) {
                const int rr = r + 1 + idx / m, c = idx % m;
                const double2 lf = Q[rr * m + r], x = P[r * m + c];
                double2 b = P[rr * m + c];
                b.x -= lf.x * x.x - lf.y * x.y;
                b.y -= lf.x * x.y + lf.y * x.x;
                P[rr * m + c] = b;
            }
            __syncthreads();
        }
        for (int r = m - 1; r >= 0; --r) {
            for (int c = tid; c < m; c += blockDim.x) P[r * m + c] = cdivz(P[r * m + c], Q[r * m + r]);
            __syncthreads();
            for (int idx = tid; idx < r * m; idx += blockDim.x) {
                const int rr = idx / m, c = idx % m;
                const double2 uf = Q[rr * m + r], x = P[r * m + c];
                double2 b = P[rr * m + c];
                b.x -= uf.x * x.x - uf.y * x.y;
                b.y -= uf.x * x.y + uf.y * x.x;
                P[rr * m + c] = b;
            }
            __syncthreads();
        }
    }
    // output = I + 2 P  (not negated: odd == false for order 6)
    for (int k = tid; k < mm; k += blockDim.x) A[k] = make_double2(2.0 * P[k].x, 2.0 * P[k].y);
    __syncthreads();
    for (int r = tid; r < m; r += blockDim.x) A[r * m + r].x += 1.0;
    __syncthreads();
    for (int i = 0; i < sorder; ++i) {
        smem_matmul(m, A, A, T);
        for (int k = tid; k < mm; k += blockDim.x) A[k] = T[k];
        __syncthreads();
    }
    for (int k = tid; k < m; k += blockDim.x) {
        ctrl->y[2 * k] = A[k * m].x;
        ctrl->y[2 * k + 1] = A[k * m].y;
    }
    if (tid == 0) {
        const double2 yl = A[(m - 1) * m];
        ctrl->err_est = yl.x * yl.x + yl.y * yl.y;
        ctrl->scaling_order = sorder;
    }
}


// ---------------------------------------------------------------------------
// Cluster version of the Hessenberg exponential: the same scaling-and-squaring
// Pade (order 6) as k_expm, with every m x m product split by rows over the CL
// CTAs of a thread-block cluster.  Each CTA keeps full copies of the matrices in
// its shared memory; a product's rows are computed by their owner CTA (row % CL)
// and stored into every CTA's copy through distributed shared memory, followed by
// a cluster barrier.  The FP32 inversion of Q-P runs redundantly in every CTA
// (identical arithmetic, so identical results); the m right-hand sides of the
// refined solve are split over the CTAs by column.  FP64 throughput is ~2 FMA/clk/SM on
// GB300, so spreading the products over CL SMs is what makes this step cheap.
// ---------------------------------------------------------------------------
namespace cg = cooperative_groups;

template <int CL>
__device__ void cl_matmul(cg::cluster_group& cl, int rank, int m, const double2* A, const double2* B, double2* Cdst) {
    constexpr int KS = 4;                                // threads per output entry (split over k)
    const int mine = (m - rank + CL - 1) / CL;           // rows r = rank, rank + CL, ...
    const int total = mine * m * KS;
    for (int base = 0; base < total; base += blockDim.x) {
        const int idx = base + threadIdx.x;
        const bool act = idx < total;
        const int o = idx / KS, ks = idx % KS;
        const int r = rank + (o / m) * CL, c = o % m;
        double arA = 0.0, arB = 0.0, aiA = 0.0, aiB = 0.0;
        if (act)
            for (int k = ks; k < m; k += KS) {
                const double2 a = A[r * m + k], b = B[k * m + c];
                arA = fma(a.x, b.x, arA);
                arB = fma(a.y, b.y, arB);
                aiA = fma(a.x, b.y, aiA);
                aiB = fma(a.y, b.x, aiB);
            }
        double sr = arA - arB, si = aiA + aiB;
        sr += __shfl_xor_sync(0xffffffffu, sr, 1);
        si += __shfl_xor_sync(0xffffffffu, si, 1);
        sr += __shfl_xor_sync(0xffffffffu, sr, 2);
        si += __shfl_xor_sync(0xffffffffu, si, 2);
        if (act && ks == 0) {
            const double2 v = make_double2(sr, si);
#pragma unroll
            for (int q = 0; q < CL; ++q) {
                double2* dst = cl.map_shared_rank(Cdst, q);
                dst[r * m + c] = v;
            }
        }
    }
    cl.sync();
}

template <int CL>
__global__ void __launch_bounds__(256) k_expm_cluster(Ctrl* ctrl, double* Hg, int m, const SchedEntry* sched) {
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int mm = m * m;
    double2* buf[7];
    for (int k = 0; k < 7; ++k) buf[k] = reinterpret_cast<double2*>(smem_raw) + (size_t)k * mm;
    double2* A = buf[0];
    double2* A2 = buf[1];
    double2* P = buf[2];
    double2* Q = buf[3];
    double2* T = buf[4];
    double2* LU = buf[5];
    double2* X = buf[6];
    __shared__ double red[8];
    __shared__ int s_p;
    __shared__ int s_info;
    __shared__ double s_c[8];
    const int tid = threadIdx.x;
    const SchedEntry se = sched[ctrl->step];
    const double2 f = make_double2(se.dt_im, -se.dt_re);   // -i * dt (pamp.h:634)
    // max |a|^2 (no FP64 square roots or divisions on the wide path: they are long
    // instruction sequences on this part's FP64 unit)
    double mx = 0.0;
    for (int k = tid; k < mm; k += blockDim.x) {
        const double2 a = cmulz(make_double2(Hg[2 * k], Hg[2 * k + 1]), f);
        A[k] = a;
        mx = fmax(mx, fma(a.x, a.x, a.y * a.y));
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((tid & 31) == 0) red[tid >> 5] = mx;
    __syncthreads();
    if (tid == 0) {
        double v2 = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v2 = fmax(v2, red[w]);
        // s = max(0, ceil(log2 max|a|)) (pamp.h:441-447): from the exponent of max|a|,
        // exact except when max|a| is a power of two, which frexp resolves
        int sord = 0;
        if (!(v2 <= DBL_MAX)) {
            ctrl->nonfinite = 1;                        // Inf/NaN Hessenberg: no scaling, flag it
        } else if (v2 > 0.0) {
            int e;
            const double fr = frexp(sqrt(v2), &e);      // max|a| = fr * 2^e, fr in [0.5, 1)
            sord = (fr == 0.5) ? e - 1 : e;
        }
        if (sord < 0) sord = 0;
        s_p = sord;
        s_info = 0;
        const int order = 6;
        s_c[0] = 1.0;
        for (int i = 0; i < order; ++i) s_c[i + 1] = s_c[i] * (double)(order - i) / (double)((i + 1) * (2 * order - i));
    }
    __syncthreads();
    const int sorder = s_p;
    const double isc = ldexp(1.0, -sorder);            // exact power of two
    for (int k = tid; k < mm; k += blockDim.x) { A[k].x *= isc; A[k].y *= isc; }
    // every CTA scaled its own copy of A: barrier before anyone writes remotely
    cl.sync();
    if (rank == 0)
        for (int k = tid; k < mm; k += blockDim.x) {
            const double2 a = cmulz(make_double2(Hg[2 * k], Hg[2 * k + 1]), f);
            Hg[2 * k] = a.x;
            Hg[2 * k + 1] = a.y;
        }
    cl_matmul<CL>(cl, rank, m, A, A, A2);
    // Horner in A^2 (pamp.h:497-539); first factors are scalar multiples of I
    for (int k = tid; k < mm; k += blockDim.x) {
        Q[k] = make_double2(s_c[6] * A2[k].x, s_c[6] * A2[k].y);
        P[k] = make_double2(s_c[5] * A2[k].x, s_c[5] * A2[k].y);
    }
    __syncthreads();
    for (int r = tid; r < m; r += blockDim.x) { Q[r * m + r].x += s_c[4]; P[r * m + r].x += s_c[3]; }
    __syncthreads();
    cl_matmul<CL>(cl, rank, m, Q, A2, T);                  // i = 2
    { double2* t = Q; Q = T; T = t; }
    for (int r = tid; r < m; r += blockDim.x) Q[r * m + r].x += s_c[2];
    __syncthreads();
    cl_matmul<CL>(cl, rank, m, P, A2, T);                  // i = 1
    { double2* t = P; P = T; T = t; }
    for (int r = tid; r < m; r += blockDim.x) P[r * m + r].x += s_c[1];
    __syncthreads();
    cl_matmul<CL>(cl, rank, m, Q, A2, T);                  // i = 0
    { double2* t = Q; Q = T; T = t; }
    for (int r = tid; r < m; r += blockDim.x) Q[r * m + r].x += s_c[0];
    __syncthreads();
    cl_matmul<CL>(cl, rank, m, P, A, T);                   // P = P A
    { double2* t = P; P = T; T = t; }
    // X = (Q - P)^-1 P (pamp.h:541-556).  D = Q - P is the Pade denominator, well
    // conditioned after scaling; it is inverted approximately in FP32 (Gauss-Jordan
    // with partial pivoting), and X is refined twice
    // with FP64 residuals R = P - D X.  Each refinement squares the FP32 error
    // (~1e-6), so X is FP64-accurate; only the FP64 residual products are
    // throughput-heavy and they are split over the cluster by column.
    for (int k = tid; k < mm; k += blockDim.x) LU[k] = make_double2(Q[k].x - P[k].x, Q[k].y - P[k].y);   // D (FP64)
    __syncthreads();                                      // D is read below with another mapping
    // Z = D^-1 in FP32 (Gauss-Jordan, see gj_inverse_f32); X and T are free here, the start
    // buffer is chosen so that the result lands in X
    const int w2 = 2 * m;
    {
        const int gi = gj_inverse_f32(
            m, [&](int r, int c) { return make_float2((float)LU[r * m + c].x, (float)LU[r * m + c].y); },
            reinterpret_cast<float2*>((m & 1) ? T : X), reinterpret_cast<float2*>((m & 1) ? X : T));
        if (tid == 0 && gi && !s_info) s_info = gi;
    }
    __syncthreads();
    const float2* Z = reinterpret_cast<const float2*>(X) + m;   // the inverse: Z(r, k) = Z[r * w2 + k]
    const int info = s_info ? s_info : (ctrl->inject_lu ? m : 0);   // inject_lu: host-set test hook
    if (info) {
        if (rank == 0 && tid == 0 && !ctrl->nonfinite) ctrl->lu_info = info;   // non-finite matrix: that is the cause
    } else {
        // this CTA's columns c = rank + j*CL of X (FP64, kept in T), residual R in Q's buffer
        const int ncol = (m - rank + CL - 1) / CL;
        double2* Xc = T;
        double2* R = Q;
        // FP32 copy of the residual: A is free after P = P A and, unlike A2 (the target of
        // the E broadcast) and T (matmul target), never written by another CTA
        float2* R32 = reinterpret_cast<float2*>(A);
        for (int it = 0; it < 3; ++it) {
            // R = P - D X  (it == 0: R = P, X = 0); four threads per entry split the k sum
            // (independent FP64 chains), combined by shuffles within aligned lane quads
            for (int base = 0; base < ncol * m * 4; base += blockDim.x) {
                const int idx = base + tid, ks = idx & 3, o = idx >> 2;
                const bool act = o < ncol * m;
                const int c = act ? rank + (o / m) * CL : 0, r = act ? o % m : 0;
                double ra = 0.0, rb = 0.0, ia = 0.0, ib = 0.0;
                if (act && it > 0)
                    for (int k = ks; k < m; k += 4) {
                        const double2 d = LU[r * m + k], x = Xc[k * m + c];
                        ra = fma(-d.x, x.x, ra);
                        rb = fma(d.y, x.y, rb);
                        ia = fma(-d.x, x.y, ia);
                        ib = fma(-d.y, x.x, ib);
                    }
                double rr = ra + rb, ri = ia + ib;
                rr += __shfl_xor_sync(0xffffffffu, rr, 1);
                ri += __shfl_xor_sync(0xffffffffu, ri, 1);
                rr += __shfl_xor_sync(0xffffffffu, rr, 2);
                ri += __shfl_xor_sync(0xffffffffu, ri, 2);
                if (act && ks == 0) {
                    const double2 v = make_double2(P[r * m + c].x + rr, P[r * m + c].y + ri);
                    R[r * m + c] = v;
                    R32[r * m + c] = make_float2((float)v.x, (float)v.y);
                }
            }
            __syncthreads();
            // X += Z R  (FP32 products on the FP32-rounded residual; FP64 update)
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
                if (it == 0) Xc[r * m + c] = make_double2((double)ar, (double)ai);
                else { Xc[r * m + c].x += (double)ar; Xc[r * m + c].y += (double)ai; }
            }
            __syncthreads();
        }
        // E = I + 2 X for this CTA's columns, broadcast into every CTA's A2 buffer
        for (int idx = tid; idx < ncol * m; idx += blockDim.x) {
            const int c = rank + (idx / m) * CL, r = idx % m;
            double2 v = make_double2(2.0 * Xc[r * m + c].x, 2.0 * Xc[r * m + c].y);
            if (r == c) v.x += 1.0;
#pragma unroll
            for (int q = 0; q < CL; ++q) {
                double2* dst = cl.map_shared_rank(A2, q);
                dst[r * m + c] = v;
            }
        }
    }
    cl.sync();
    { double2* t = A; A = A2; A2 = t; }
    if (!info) {
        for (int i = 0; i < sorder; ++i) {
            cl_matmul<CL>(cl, rank, m, A, A, T);
            double2* t = A; A = T; T = t;
        }
        if (rank == 0) {
            for (int k = tid; k < m; k += blockDim.x) {
                ctrl->y[2 * k] = A[k * m].x;
                ctrl->y[2 * k + 1] = A[k * m].y;
            }
            if (tid == 0) {
                const double2 yl = A[(m - 1) * m];
                ctrl->err_est = yl.x * yl.x + yl.y * yl.y;
                ctrl->scaling_order = sorder;
            }
        }
    }
    // no CTA may exit while others can still address its shared memory
    cl.sync();
}

static int g_expm_cluster[kMaxBasis + 1];   // per basis size: 0 unknown, 1 single CTA, else cluster size

template <int CL>
static cudaError_t launch_expm_cl(Ctrl* ctrl, double* H, int m, const SchedEntry* sched, cudaStream_t s) {
    const size_t smem = (size_t)7 * m * m * sizeof(double2);
    auto kern = k_expm_cluster<CL>;
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

template <int CL>
static bool cluster_fits(int m) {
    const size_t smem = (size_t)7 * m * m * sizeof(double2);
    auto kern = k_expm_cluster<CL>;
    if (allow_max_smem(kern) != cudaSuccess) return false;
    if (CL > 8 && cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
        return false;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(CL);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    cudaError_t e = cudaOccupancyMaxActiveClusters(&n, kern, &cfg);
    cudaGetLastError();
    return e == cudaSuccess && n > 0;
}

int expm_cluster_size(int m) {
    if (m < 1 || m > kMaxBasis) return 0;
    if (g_expm_cluster[m] == 0) {
        if (cluster_fits<16>(m)) g_expm_cluster[m] = 16;
        else if (cluster_fits<8>(m)) g_expm_cluster[m] = 8;
        else g_expm_cluster[m] = 1;
    }
    return g_expm_cluster[m] == 1 ? 0 : g_expm_cluster[m];
}

// ---------------------------------------------------------------------------
// pAMP::EigenvectorExponential (pamp.h:567-607; krylov_exponentiation_method = 1,
// pampwrapper.cpp:56-61): y = exp(A) e1 for A = -i dt H_m from the eigen-decomposition of A.
// The reference takes zgeev's unit right eigenvectors W and forms W diag(e^lambda) W^H, which is
// exp(A) for a normal A; for Arnoldi on the Hermitian balanced operator H_m is Hermitian (to
// rounding) and A normal, so the same y is formed from the eigen-decomposition of the Hermitian
// part of H_m, H_m = Q diag(mu) Q^H, lambda = -i dt mu:  y = Q (e^{-i dt mu} .* conj(Q(0, :))).
// The decomposition is a parallel cyclic Jacobi iteration on one CTA (round-robin pairing of
// the m (padded to even) indices, m/2 disjoint complex rotations per round, applied to the
// columns and then to the rows), FP64, until the off-diagonal part is below 1e-15 of the matrix
// (Frobenius) or after 20 sweeps.  Writes -i dt H_m back (GetHessenbergMatrix), y, |y[m-1]|^2.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_expm_eig(Ctrl* ctrl, double* Hg, int m, const SchedEntry* sched) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int mp = m + (m & 1);
    double2* A = reinterpret_cast<double2*>(smem_raw);     // mp x mp
    double2* Q = A + mp * mp;                               // mp x mp
    constexpr int kPairs = (kMaxBasis + 1) / 2;
    __shared__ int s_p[kPairs], s_q[kPairs];
    __shared__ double2 s_g[kPairs][4];                      // (g_pp, g_pq, g_qp, g_qq) of pair k
    __shared__ double s_off[8], s_tot[8];
    __shared__ int s_go;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    const SchedEntry se = sched[ctrl->step];
    const double2 f = make_double2(se.dt_im, -se.dt_re);   // -i dt
    for (int k = tid; k < mp * mp; k += blockDim.x) {
        const int i = k / mp, j = k - i * mp;
        double2 a = make_double2(0.0, 0.0);
        if (i < m && j < m) {
            const double2 hij = make_double2(Hg[2 * (i * m + j)], Hg[2 * (i * m + j) + 1]);
            const double2 hji = make_double2(Hg[2 * (j * m + i)], Hg[2 * (j * m + i) + 1]);
            a = make_double2(0.5 * (hij.x + hji.x), 0.5 * (hij.y - hji.y));   // Hermitian part
        }
        A[k] = a;
        Q[k] = make_double2(i == j ? 1.0 : 0.0, 0.0);
    }
    __syncthreads();
    // -i dt H_m kept in global, as the Pade kernels do (read back by GetHessenbergMatrix)
    for (int k = tid; k < m * m; k += blockDim.x) {
        const double2 h = make_double2(Hg[2 * k], Hg[2 * k + 1]);
        const double2 a = cmulz(h, f);
        Hg[2 * k] = a.x;
        Hg[2 * k + 1] = a.y;
    }
    const int npairs = mp / 2;
    for (int sweep = 0; sweep < 20; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int k = tid; k < mp * mp; k += blockDim.x) {
            const double2 a = A[k];
            const double v = a.x * a.x + a.y * a.y;
            tot += v;
            if (k / mp != k % mp) off += v;
        }
        for (int o = 16; o > 0; o >>= 1) {
            off += __shfl_xor_sync(0xffffffffu, off, o);
            tot += __shfl_xor_sync(0xffffffffu, tot, o);
        }
        if (lane == 0) { s_off[warp] = off; s_tot[warp] = tot; }
        __syncthreads();
        if (tid == 0) {
            double o2 = 0.0, t2 = 0.0;
            for (int w = 0; w < nw; ++w) { o2 += s_off[w]; t2 += s_tot[w]; }
            s_go = o2 > 1e-30 * t2;
        }
        __syncthreads();
        if (!s_go) break;
        for (int r = 0; r < mp - 1; ++r) {
            if (tid < npairs) {
                auto idx = [&](int j) { return j == 0 ? 0 : 1 + (j - 1 + r) % (mp - 1); };
                int p = idx(tid), q = idx(mp - 1 - tid);
                if (p > q) { const int t = p; p = q; q = t; }
                double2 g0 = make_double2(1.0, 0.0), g1 = make_double2(0.0, 0.0), g2 = g1, g3 = g0;
                const double2 c = A[p * mp + q];
                const double rr = hypot(c.x, c.y);
                if (q < m && rr > 0.0) {
                    const double a = A[p * mp + p].x, b = A[q * mp + q].x;
                    const double tau = (b - a) / (2.0 * rr);
                    const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
                    const double cs = 1.0 / sqrt(1.0 + t * t), sn = t * cs;
                    const double er = c.x / rr, ei = -c.y / rr;    // e^{-i phi}
                    g0 = make_double2(cs, 0.0);
                    g1 = make_double2(sn, 0.0);
                    g2 = make_double2(-sn * er, -sn * ei);
                    g3 = make_double2(cs * er, cs * ei);
                }
                s_p[tid] = p;
                s_q[tid] = q;
                s_g[tid][0] = g0; s_g[tid][1] = g1; s_g[tid][2] = g2; s_g[tid][3] = g3;
            }
            __syncthreads();
            // A <- A G and Q <- Q G (columns p, q of every pair)
            for (int k = tid; k < npairs * mp; k += blockDim.x) {
                const int pr = k / mp, i = k - pr * mp;
                const int p = s_p[pr], q = s_q[pr];
                const double2 gpp = s_g[pr][0], gpq = s_g[pr][1], gqp = s_g[pr][2], gqq = s_g[pr][3];
                double2 ap = A[i * mp + p], aq = A[i * mp + q];
                A[i * mp + p] = cadd2(cmulz(ap, gpp), cmulz(aq, gqp));
                A[i * mp + q] = cadd2(cmulz(ap, gpq), cmulz(aq, gqq));
                ap = Q[i * mp + p];
                aq = Q[i * mp + q];
                Q[i * mp + p] = cadd2(cmulz(ap, gpp), cmulz(aq, gqp));
                Q[i * mp + q] = cadd2(cmulz(ap, gpq), cmulz(aq, gqq));
            }
            __syncthreads();
            // A <- G^H A (rows p, q of every pair)
            for (int k = tid; k < npairs * mp; k += blockDim.x) {
                const int pr = k / mp, j = k - pr * mp;
                const int p = s_p[pr], q = s_q[pr];
                const double2 gpp = conjz(s_g[pr][0]), gpq = conjz(s_g[pr][1]), gqp = conjz(s_g[pr][2]),
                              gqq = conjz(s_g[pr][3]);
                const double2 ap = A[p * mp + j], aq = A[q * mp + j];
                A[p * mp + j] = cadd2(cmulz(gpp, ap), cmulz(gqp, aq));
                A[q * mp + j] = cadd2(cmulz(gpq, ap), cmulz(gqq, aq));
            }
            __syncthreads();
        }
    }
    // y_k = sum_j Q(k, j) e^{-i dt mu_j} conj(Q(0, j))
    for (int k = tid; k < m; k += blockDim.x) {
        double yr = 0.0, yi = 0.0;
        for (int j = 0; j < m; ++j) {
            const double mu = A[j * mp + j].x;
            double sn, cs;
            sincos(se.dt_re * mu, &sn, &cs);
            const double amp = exp(se.dt_im * mu);
            const double2 e = make_double2(amp * cs, -amp * sn);
            const double2 w = cmulz(Q[k * mp + j], conjz(Q[j]));
            const double2 t = cmulz(w, e);
            yr += t.x;
            yi += t.y;
        }
        ctrl->y[2 * k] = yr;
        ctrl->y[2 * k + 1] = yi;
        if (k == m - 1) ctrl->err_est = yr * yr + yi * yi;
    }
    if (tid == 0) ctrl->scaling_order = 0;
}

cudaError_t launch_expm_eig(Ctrl* ctrl, double* H, int m, const SchedEntry* sched, cudaStream_t s) {
    count_launch();
    const int mp = m + (m & 1);
    const size_t smem = (size_t)2 * mp * mp * sizeof(double2);
    if (smem > 48 * 1024) {
        cudaError_t e = allow_max_smem(k_expm_eig);
        if (e != cudaSuccess) return e;
    }
    k_expm_eig<<<1, 256, smem, s>>>(ctrl, H, m, sched);
    return cudaGetLastError();
}

cudaError_t launch_expm(Ctrl* ctrl, double* H, int m, const SchedEntry* sched, int max_cluster, cudaStream_t s,
                        int df32) {
    count_launch();
    const int cl = max_cluster >= 8 ? expm_cluster_size(m) : 0;
    if (df32 && (cl == 16 || cl == 8) && cl <= max_cluster) return launch_expm_df(ctrl, H, m, sched, cl, s);
    if (df32 && cl == 0) {
        static int fits[kMaxBasis + 1];              // 0 unknown, 1 yes, 2 no
        if (m >= 1 && m <= kMaxBasis && fits[m] == 0) fits[m] = expm_df_single_fits(m) ? 1 : 2;
        if (m >= 1 && m <= kMaxBasis && fits[m] == 1) return launch_expm_df(ctrl, H, m, sched, 1, s);
    }
    if (cl == 16 && max_cluster >= 16) return launch_expm_cl<16>(ctrl, H, m, sched, s);
    if (cl == 8) return launch_expm_cl<8>(ctrl, H, m, sched, s);
    const size_t smem = (size_t)5 * m * m * sizeof(double2);
    if (smem > 48 * 1024) {
        cudaError_t e = allow_max_smem(k_expm);
        if (e != cudaSuccess) return e;
    }
    k_expm<<<1, 256, smem, s>>>(ctrl, H, m, sched);
    return cudaGetLastError();
}

// psi = beta0 * V y  (pamp.h:657-662), FP64 accumulation, complex128 output.
template <typename T>
__global__ void k_combine(const cx<T>* __restrict__ V, const double2* __restrict__ v0, long n,
                          const Ctrl* __restrict__ ctrl, double2* __restrict__ out) {
    __shared__ double2 ys[kMaxBasis];
    const int nb = ctrl->nbasis;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) ys[k] = make_double2(ctrl->y[2 * k], ctrl->y[2 * k + 1]);
    __syncthreads();
    const double b0 = ctrl->beta0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double sr = 0.0, si = 0.0;
        for (int k = 0; k < nb; ++k) {
            double vr, vi;
            if (v0 && k == 0) { const double2 a = v0[i]; vr = a.x; vi = a.y; }
            else { const cx<T> v = V[(size_t)k * n + i]; vr = (double)v.x; vi = (double)v.y; }
            sr = fma(vr, ys[k].x, sr);
            sr = fma(-vi, ys[k].y, sr);
            si = fma(vr, ys[k].y, si);
            si = fma(vi, ys[k].x, si);
        }
        out[i] = make_double2(sr * b0, si * b0);
    }
}

// Complex64 basis: x = sum_k (beta0 y_k) v_k with beta0 y_k as FP32 pairs, error-free products
// and compensated sums (the FP64 first vector split into FP32 pairs per element), FP64 output.
// Per element ~14 FP64 instructions instead of ~6 per basis vector.
__global__ void k_combine32(const float2* __restrict__ V, const double2* __restrict__ v0, long n,
                            const Ctrl* __restrict__ ctrl, double2* __restrict__ out) {
    __shared__ float4 ys[kMaxBasis];                 // beta0 y_k: (re_hi, re_lo, im_hi, im_lo)
    const int nb = ctrl->nbasis;
    if ((int)threadIdx.x < nb) {
        const double b0 = ctrl->beta0;
        const double yr = ctrl->y[2 * threadIdx.x] * b0, yi = ctrl->y[2 * threadIdx.x + 1] * b0;
        const float a = (float)yr, b = (float)yi;
        ys[threadIdx.x] = make_float4(a, (float)(yr - (double)a), b, (float)(yi - (double)b));
    }
    __syncthreads();
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
        int k = 0;
        if (v0 && nb > 0) {
            const double2 a = v0[i];
            const float ah = (float)a.x, bh = (float)a.y;
            const float al = (float)(a.x - (double)ah), bl = (float)(a.y - (double)bh);
            const float4 y = ys[0];
            df_mac(rh, rl, y.x, y.y, ah, al);
            df_mac(rh, rl, -y.z, -y.w, bh, bl);
            df_mac(ih, il, y.x, y.y, bh, bl);
            df_mac(ih, il, y.z, y.w, ah, al);
            k = 1;
        }
        for (; k < nb; ++k) {
            const float2 v = V[(size_t)k * n + i];
            const float4 y = ys[k];
            acc_prod(rh, rl, y.x, y.y, v.x);
            acc_prod(rh, rl, -y.z, -y.w, v.y);
            acc_prod(ih, il, y.x, y.y, v.y);
            acc_prod(ih, il, y.z, y.w, v.x);
        }
        out[i] = make_double2((double)rh + (double)rl, (double)ih + (double)il);
    }
}

cudaError_t launch_combine(int prec, const void* V, const double2* v0, long n, const Ctrl* ctrl, void* out,
                           cudaStream_t s) {
    count_launch();
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 8) blocks = 152 * 8;
    if (prec == 0) k_combine<double><<<blocks, 256, 0, s>>>((const double2*)V, nullptr, n, ctrl, (double2*)out);
    else k_combine32<<<blocks, 256, 0, s>>>((const float2*)V, v0, n, ctrl, (double2*)out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// stateless reference-storage kernel: TensorPotentialMultiply_{Diag,Simp}_BandNH
// V complex band in BLAS storage (element (i,j) at j*(2kb+1) + kb + i - j)
// ---------------------------------------------------------------------------
__global__ void k_tensor_multiply_ref(int storage, const double2* __restrict__ V, int npairs,
                                      const int* __restrict__ pairs, int kb, double scaling,
                                      const double2* __restrict__ src, double2* __restrict__ dst, int nl, int nr) {
    const int l = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nr) return;
    const int W = 2 * kb + 1;
    double sr = 0.0, si = 0.0;
    const int j0 = max(0, i - kb), j1 = min(nr - 1, i + kb);
    auto band = [&](const double2* A, const double2* x) {
        for (int j = j0; j <= j1; ++j) {
            const double2 a = A[(size_t)j * W + kb + i - j];
            const double2 v = x[j];
            sr += a.x * v.x - a.y * v.y;
            si += a.x * v.y + a.y * v.x;
        }
    };
    if (storage == 0) {
        band(V + (size_t)l * W * nr, src + (size_t)l * nr);
    } else {
        for (int p = 0; p < npairs; ++p) {
            if (pairs[2 * p] != l) continue;
            band(V + (size_t)p * W * nr, src + (size_t)pairs[2 * p + 1] * nr);
        }
    }
    double2 d = dst[(size_t)l * nr + i];
    d.x += scaling * sr;
    d.y += scaling * si;
    dst[(size_t)l * nr + i] = d;
}

cudaError_t launch_tensor_multiply_ref(int storage, const double2* V, int npairs, const int* pairs, int kb,
                                       double scaling, const double2* src, double2* dst, int nl, int nr,
                                       cudaStream_t s) {
    count_launch();
    dim3 grid((nr + 127) / 128, nl);
    k_tensor_multiply_ref<<<grid, 128, 0, s>>>(storage, V, npairs, pairs, kb, scaling, src, dst, nl, nr);
    return cudaGetLastError();
}

__global__ void k_zero(unsigned char* p, size_t bytes) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < bytes; i += (size_t)gridDim.x * blockDim.x)
        p[i] = 0;
}

cudaError_t launch_zero(void* p, size_t bytes, cudaStream_t s) {
    count_launch();
    k_zero<<<64, 256, 0, s>>>((unsigned char*)p, bytes);
    return cudaGetLastError();
}

}  // namespace gbprop
