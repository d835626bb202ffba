// Banded triangular solves along r (ztbsv 'U','N' / 'U','C' in the reference,
// piram/piram/blitzblas.h:454-487, called from overlapmatrix.cpp:137-229):
//   * k_solve_inv   -- banded approximate inverse of the overlap factor applied in FP32
//                      with FP64-residual refinement (the runtime's default);
//   * k_solve_ir    -- FP32 block back-substitution + FP64 refinement (fallback for
//                      factors whose inverse decays too slowly);
//   * k_solve       -- the block back-substitution in one precision.
#include "gbprop_internal.h"
#include "gbprop_device.cuh"

#include <algorithm>
#include <cmath>

namespace gbprop {

// ---------------------------------------------------------------------------
// parallel banded triangular solve (ztbsv 'U','N' / 'U','C' along r)
// ---------------------------------------------------------------------------
constexpr int kPitch = 33;   // smem pitch of the block-interleaved row buffer

// One warp solves U~ x = b for one row held in smem in block-interleaved e order
// (element e = B*L + i at buf[i*kPitch + B]); lane B owns block B.
//   1) local back-substitution of the block with rows pre-scaled by 1/U(e,e);
//   2) warp-shuffle suffix scan of the kd-vector recurrence t_B = y_B[0:kd] - F_B t_{B+1};
//   3) correction x_B -= G_B t_{B+1}.
template <typename T, int KD>
__device__ __forceinline__ void warp_block_solve(const SolveTab<T>& tab, cx<T>* buf, int lane) {
    using C = cx<T>;
    const int n = tab.n, L = tab.L, P = tab.P;
    const int B = lane;
    C win[KD];
#pragma unroll
    for (int d = 0; d < KD; ++d) win[d] = mk<T>(0, 0);
    for (int i = L - 1; i >= 0; --i) {
        const int e = B * L + i;
        const int idx = i * kPitch + B;
        const T inv = tab.invd[i * 32 + B];
        C x = mk<T>(0, 0);
        if (e < n) {
            const C b = buf[idx];
            T sr = b.x * inv, si = b.y * inv;
#pragma unroll
            for (int d = KD; d >= 1; --d) {
                const T u = tab.ud[((d - 1) * L + i) * 32 + B];
                sr = fma(-u, win[d - 1].x, sr);
                si = fma(-u, win[d - 1].y, si);
            }
            x = mk<T>(sr, si);
            buf[idx] = x;
        }
#pragma unroll
        for (int d = KD - 1; d >= 1; --d) win[d] = win[d - 1];
        win[0] = x;
    }
    C a[KD];
#pragma unroll
    for (int c = 0; c < KD; ++c) a[c] = (B * L + c < n && B < P) ? buf[c * kPitch + B] : mk<T>(0, 0);
    for (int lev = 0; lev < tab.levels; ++lev) {
        const int s = 1 << lev;
        C nb[KD];
#pragma unroll
        for (int c = 0; c < KD; ++c) {
            nb[c].x = __shfl_down_sync(0xffffffffu, a[c].x, s);
            nb[c].y = __shfl_down_sync(0xffffffffu, a[c].y, s);
        }
        if (B + s < P) {
            const T* M = tab.mlev + ((size_t)(lev * 32 + B) * KD) * KD;
#pragma unroll
            for (int r = 0; r < KD; ++r) {
                T ar = a[r].x, ai = a[r].y;
#pragma unroll
                for (int c = 0; c < KD; ++c) {
                    const T mv = M[r * KD + c];
                    ar = fma(mv, nb[c].x, ar);
                    ai = fma(mv, nb[c].y, ai);
                }
                a[r] = mk<T>(ar, ai);
            }
        }
    }
    C t[KD];
#pragma unroll
    for (int c = 0; c < KD; ++c) {
        t[c].x = __shfl_down_sync(0xffffffffu, a[c].x, 1);
        t[c].y = __shfl_down_sync(0xffffffffu, a[c].y, 1);
    }
    if (B + 1 < P) {
        for (int i = 0; i < L; ++i) {
            const int e = B * L + i;
            if (e >= n) break;
            const int idx = i * kPitch + B;
            C x = buf[idx];
#pragma unroll
            for (int c = 0; c < KD; ++c) {
                const T gv = tab.g[(c * L + i) * 32 + B];
                x.x = fma(-gv, t[c].x, x.x);
                x.y = fma(-gv, t[c].y, x.y);
            }
            buf[idx] = x;
        }
    }
    __syncwarp();
}

// Working-precision solve (the complex64 Krylov basis of the mixed path), one warp per row.
template <typename T, int KD, typename TI, typename TO, typename TV>
__global__ void __launch_bounds__(32) k_solve(SolveTab<T> tab, const TI* in, TO* out,
                                              TV* __restrict__ vstore, const Ctrl* __restrict__ ctrl,
                                              int scale_mode, int check_broken) {
    using C = cx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* buf = reinterpret_cast<C*>(smem_raw);
    if (check_broken && ctrl->broken) return;
    const int l = blockIdx.x, lane = threadIdx.x;
    const int n = tab.n, L = tab.L;
    const double sc = scale_mode ? ctrl->inv_beta : 1.0;
    const size_t base = (size_t)l * n;
    for (int p = lane; p < n; p += 32) {
        TI v = in[base + p];
        double re = (double)v.x, im = (double)v.y;
        if (scale_mode) { re *= sc; im *= sc; }
        C c = mk<T>((T)re, (T)im);
        if (vstore) vstore[base + p] = conv<TV>(c);
        const int e = tab.dir ? (n - 1 - p) : p;
        const int B = e / L, i = e - B * L;
        buf[i * kPitch + B] = c;
    }
    __syncwarp();
    warp_block_solve<T, KD>(tab, buf, lane);
    for (int p = lane; p < n; p += 32) {
        const int e = tab.dir ? (n - 1 - p) : p;
        const int Bq = e / L, i = e - Bq * L;
        out[base + p] = conv<TO>(buf[i * kPitch + Bq]);
    }
}

// FP64-accurate solve for the FP64 path: FP32 block solve of the (power-of-two
// scaled) residual, refined three times with FP64 residuals r = b - U~ x
// (mixed-precision iterative refinement: each pass multiplies the error by the
// FP32 solve's relative accuracy, c*eps32*cond(U) ~ 1e-5 for the B-spline overlap
// factors, so three passes reach the FP64 level).  One CTA per row; the FP64 work
// is the residual band products (2*(kd+1) FMA per element per pass).
constexpr int kIrThreads = 256;
constexpr int kIrRefinements = 3;

template <int KD, typename TI, typename TO, typename TV>
__global__ void __launch_bounds__(kIrThreads) k_solve_ir(SolveTab<float> tab, const double* __restrict__ udp,
                                                         const TI* in, TO* out, TV* __restrict__ vstore,
                                                         const Ctrl* __restrict__ ctrl, int scale_mode,
                                                         int check_broken, int stage_tables, int stage_udp) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = tab.n, L = tab.L, dir = tab.dir;
    double2* bd = reinterpret_cast<double2*>(smem_raw);
    double2* xd = bd + n;
    double2* rd = xd + n;
    float2* rf = reinterpret_cast<float2*>(rd + n);
    float* tsm = reinterpret_cast<float*>(rf + (size_t)L * kPitch);  // FP32 solve tables (when staged)
    const int nud = KD * L * 32, ninv = L * 32, ng = KD * L * 32, nm = max(tab.levels, 1) * 32 * KD * KD;
    double* ud_smem = reinterpret_cast<double*>(tsm + (stage_tables ? nud + ninv + ng + nm : 0));
    const double* ud_s = stage_udp ? ud_smem : udp;                    // (KD+1) x n FP64 diagonals
    __shared__ float s_red[kIrThreads / 32];
    if (check_broken && ctrl->broken) return;
    const int l = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // stage the solve tables (shared by every row; L2-resident) in shared memory
    SolveTab<float> st = tab;
    if (stage_tables) {
        float* p_ud = tsm;
        float* p_inv = p_ud + nud;
        float* p_g = p_inv + ninv;
        float* p_m = p_g + ng;
        for (int k = tid; k < nud; k += kIrThreads) p_ud[k] = tab.ud[k];
        for (int k = tid; k < ninv; k += kIrThreads) p_inv[k] = tab.invd[k];
        for (int k = tid; k < ng; k += kIrThreads) p_g[k] = tab.g[k];
        for (int k = tid; k < nm; k += kIrThreads) p_m[k] = tab.mlev[k];
        st.ud = p_ud;
        st.invd = p_inv;
        st.g = p_g;
        st.mlev = p_m;
    }
    if (stage_udp)
        for (int k = tid; k < (KD + 1) * n; k += kIrThreads) ud_smem[k] = udp[k];
    const double sc = scale_mode ? ctrl->inv_beta : 1.0;
    const size_t base = (size_t)l * n;
    for (int p = tid; p < n; p += kIrThreads) {
        const TI v = in[base + p];
        double2 b = make_double2((double)v.x, (double)v.y);
        if (scale_mode) { b.x *= sc; b.y *= sc; }
        if (vstore) vstore[base + p] = conv<TV>(b);
        bd[p] = b;
        rd[p] = b;
        xd[p] = make_double2(0.0, 0.0);
    }
    __syncthreads();
    for (int it = 0; it <= kIrRefinements; ++it) {
        if (it > 0) {
            // r = b - U~ x in FP64 (physical coordinates)
            for (int p = tid; p < n; p += kIrThreads) {
                double rr = bd[p].x, ri = bd[p].y;
                if (dir == 0) {
#pragma unroll
                    for (int d = 0; d <= KD; ++d) {
                        if (p + d < n) {
                            const double u = ud_s[(size_t)d * n + p];
                            rr = fma(-u, xd[p + d].x, rr);
                            ri = fma(-u, xd[p + d].y, ri);
                        }
                    }
                } else {
#pragma unroll
                    for (int d = 0; d <= KD; ++d) {
                        if (p - d >= 0) {
                            const double u = ud_s[(size_t)d * n + p - d];
                            rr = fma(-u, xd[p - d].x, rr);
                            ri = fma(-u, xd[p - d].y, ri);
                        }
                    }
                }
                rd[p] = make_double2(rr, ri);
            }
            __syncthreads();
        }
        // power-of-two scale so that the FP32 right-hand side is O(1)
        float mx = 0.f;
        for (int p = tid; p < n; p += kIrThreads) mx = fmaxf(mx, fmaxf(fabsf((float)rd[p].x), fabsf((float)rd[p].y)));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        if (lane == 0) s_red[warp] = mx;
        __syncthreads();
        mx = 0.f;
#pragma unroll
        for (int w = 0; w < kIrThreads / 32; ++w) mx = fmaxf(mx, s_red[w]);
        if (mx == 0.f) break;                       // exact solution reached (or zero rhs)
        int ex;
        frexpf(mx, &ex);
        const double scale = ldexp(1.0, -ex), unscale = ldexp(1.0, ex);
        for (int p = tid; p < n; p += kIrThreads) {
            const int e = dir ? (n - 1 - p) : p;
            const int B = e / L, i = e - B * L;
            rf[i * kPitch + B] = make_float2((float)(rd[p].x * scale), (float)(rd[p].y * scale));
        }
        __syncthreads();
        if (warp == 0) warp_block_solve<float, KD>(st, rf, lane);
        __syncthreads();
        for (int p = tid; p < n; p += kIrThreads) {
            const int e = dir ? (n - 1 - p) : p;
            const int B = e / L, i = e - B * L;
            const float2 dlt = rf[i * kPitch + B];
            xd[p].x += (double)dlt.x * unscale;
            xd[p].y += (double)dlt.y * unscale;
        }
        __syncthreads();
    }
    for (int p = tid; p < n; p += kIrThreads) out[base + p] = conv<TO>(xd[p]);
}

template <typename T, int KD>
static cudaError_t solve_kd(const SolveTab<T>& tab, int nrows, const void* in, int in_prec, void* out, int out_prec,
                            void* vstore, int v_prec, const Ctrl* ctrl, int scale_mode, int check_broken,
                            cudaStream_t s) {
    const size_t smem = (size_t)tab.L * kPitch * sizeof(cx<T>);
    dim3 grid(nrows), block(32);
    // in/out/vstore precision combinations used by the runtime
#define GB_SOLVE_CASE(TI_, TO_, TV_)                                                                             \
    {                                                                                                            \
        auto kern = k_solve<T, KD, TI_, TO_, TV_>;                                                               \
        if (smem > 48 * 1024) {                                                                                  \
            cudaError_t ea = allow_max_smem(kern);                                                               \
            if (ea != cudaSuccess) return ea;                                                                    \
        }                                                                                                        \
        kern<<<grid, block, smem, s>>>(tab, (const TI_*)in, (TO_*)out, (TV_*)vstore, ctrl, scale_mode,           \
                                       check_broken);                                                            \
        return cudaGetLastError();                                                                               \
    }
    // combinations the runtime uses (the complex64 Krylov basis of the mixed path)
    const int key = in_prec * 4 + out_prec * 2 + v_prec;
    switch (key) {
        case 3: GB_SOLVE_CASE(double2, float2, float2)
        case 7: GB_SOLVE_CASE(float2, float2, float2)
        default: return cudaErrorInvalidValue;
    }
#undef GB_SOLVE_CASE
}

template <typename T>
static cudaError_t solve_dispatch(const SolveTab<T>& tab, int nrows, const void* in, int in_prec, void* out,
                                  int out_prec, void* vstore, int v_prec, const Ctrl* ctrl, int scale_mode,
                                  int check_broken, cudaStream_t s) {
    switch (tab.kd) {
#define GB_KD(K) \
    case K: return solve_kd<T, K>(tab, nrows, in, in_prec, out, out_prec, vstore, v_prec, ctrl, scale_mode, check_broken, s);
        GB_KD(1) GB_KD(2) GB_KD(3) GB_KD(4) GB_KD(5) GB_KD(6) GB_KD(7) GB_KD(8)
#undef GB_KD
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_solve(int arith, const void* tab, int nrows, const void* in, int in_prec, void* out, int out_prec,
                         void* vstore, int v_prec, const Ctrl* ctrl, int scale_mode, int check_broken,
                         cudaStream_t s) {
    count_launch();
    if (arith == 0) return cudaErrorInvalidValue;     // FP64 solves go through the refined kernels
    return solve_dispatch(*(const SolveTab<float>*)tab, nrows, in, in_prec, out, out_prec, vstore, v_prec, ctrl,
                          scale_mode, check_broken, s);
}

template <int KD>
static cudaError_t solve_ir_kd(const SolveTab<float>& tab, const double* udp, int nrows, const void* in, int in_prec,
                               void* out, int out_prec, void* vstore, int v_prec, const Ctrl* ctrl, int scale_mode,
                               int check_broken, cudaStream_t s) {
    // shared memory: b, x, r rows + FP32 work row are required; the solve tables and the FP64
    // diagonals are staged only while they fit (otherwise read through L1/L2)
    const size_t limit = 220 * 1024;
    const size_t base = (size_t)3 * tab.n * sizeof(double2) + (size_t)tab.L * kPitch * sizeof(float2);
    const size_t tabb = ((size_t)KD * tab.L * 32 * 2 + (size_t)tab.L * 32 +
                         (size_t)(tab.levels > 0 ? tab.levels : 1) * 32 * KD * KD) * sizeof(float);
    const size_t udb = (size_t)(KD + 1) * tab.n * sizeof(double);
    const int stage_tables = base + tabb <= limit;
    const int stage_udp = base + (stage_tables ? tabb : 0) + udb <= limit;
    const size_t smem = base + (stage_tables ? tabb : 0) + (stage_udp ? udb : 0);
    if (smem > limit) return cudaErrorInvalidValue;
    dim3 grid(nrows), block(kIrThreads);
#define GB_IR_CASE(TI_, TO_, TV_)                                                                                \
    {                                                                                                            \
        auto kern = k_solve_ir<KD, TI_, TO_, TV_>;                                                               \
        if (smem > 48 * 1024) {                                                                                  \
            cudaError_t ea = allow_max_smem(kern);                                                               \
            if (ea != cudaSuccess) return ea;                                                                    \
        }                                                                                                        \
        kern<<<grid, block, smem, s>>>(tab, udp, (const TI_*)in, (TO_*)out, (TV_*)vstore, ctrl, scale_mode,      \
                                       check_broken, stage_tables, stage_udp);                                   \
        return cudaGetLastError();                                                                               \
    }
    // combinations the runtime uses: refined solves store double2 (or nothing)
    const int key = in_prec * 4 + out_prec * 2 + v_prec;
    switch (key) {
        case 0: GB_IR_CASE(double2, double2, double2)
        case 2: GB_IR_CASE(double2, float2, double2)
        case 4: GB_IR_CASE(float2, double2, double2)
        case 6: GB_IR_CASE(float2, float2, double2)
        default: return cudaErrorInvalidValue;
    }
#undef GB_IR_CASE
}

cudaError_t launch_solve_ir(const void* tabf, const double* udp, int nrows, const void* in, int in_prec, void* out,
                            int out_prec, void* vstore, int v_prec, const Ctrl* ctrl, int scale_mode, int check_broken,
                            cudaStream_t s) {
    count_launch();
    const SolveTab<float>& tab = *(const SolveTab<float>*)tabf;
    switch (tab.kd) {
#define GB_KD(K) \
    case K: return solve_ir_kd<K>(tab, udp, nrows, in, in_prec, out, out_prec, vstore, v_prec, ctrl, scale_mode, check_broken, s);
        GB_KD(1) GB_KD(2) GB_KD(3) GB_KD(4) GB_KD(5) GB_KD(6) GB_KD(7) GB_KD(8)
#undef GB_KD
        default: return cudaErrorInvalidValue;
    }
}

// ---------------------------------------------------------------------------
// solve through the banded approximate inverse (all threads busy, no recursion)
// ---------------------------------------------------------------------------
// CTA (chunk c, row l) produces x on q in [q0, q0 + cl), q0 = c * chunk.  With P
// refinement passes, pass k (0..P) updates x on [q0, q0 + R_k), R_k = cl + (P-k)(w+kd):
//     r = b - U~ x          (FP64; pass 0: r = b, x = 0)
//     x += 2^e * M (2^-e r) (FP32 products and sums; 2^-e only when max|r| leaves the
//                            comfortable FP32 exponent range)
// x on R_k needs r on R_k + w, which needs the previous x on R_k + w + kd = R_{k-1}, so
// the chunk's halo is recomputed instead of exchanged.  Every element of the region is
// independent inside a pass: one thread per element, two barriers per pass.  The chunk's
// slices of M and U~ arrive by bulk asynchronous copies (one mbarrier) while the threads
// load the right-hand side.
constexpr int kInvThreads = 512;
// x (+)= M r32 for the elements q and q + 1 (q even; r32 16-byte aligned and readable up to
// q + w + 1): FP32 products, two independent chains per component.  Every pair of r32
// values is one 16-byte load and every pair of M entries one 8-byte load, each used for
// both outputs -- 3 loads per 8 FMAs instead of 8.  With t = j for element q and t = j + 1
// for element q + 1, r32[q + t] meets M[t][q] and M[t-1][q+1].
template <bool STAGE>
__device__ __forceinline__ float2 inv_m2(const float* mrow, size_t mstride, int t) {
    const float2* p = reinterpret_cast<const float2*>(mrow + (size_t)t * mstride);
    return STAGE ? *p : __ldg(p);
}

template <bool STAGE>
__device__ __forceinline__ float4 inv_apply2(const float* mrow, size_t mstride, const float2* r32, int q, int w) {
    const float4* r4 = reinterpret_cast<const float4*>(r32 + q);
    float a0r = 0.f, a0i = 0.f, b0r = 0.f, b0i = 0.f;   // element q: even / odd t
    float a1r = 0.f, a1i = 0.f, b1r = 0.f, b1i = 0.f;   // element q + 1
    float pm = 0.f;                                     // M[t-1][q+1] (none at t = 0)
    int t = 0;
    for (; t + 1 <= w; t += 2) {
        const float4 rr = r4[t >> 1];                   // r[q+t], r[q+t+1]
        const float2 m0 = inv_m2<STAGE>(mrow, mstride, t), m1 = inv_m2<STAGE>(mrow, mstride, t + 1);
        a0r = fmaf(m0.x, rr.x, a0r); a0i = fmaf(m0.x, rr.y, a0i);
        a1r = fmaf(pm, rr.x, a1r);   a1i = fmaf(pm, rr.y, a1i);
        b0r = fmaf(m1.x, rr.z, b0r); b0i = fmaf(m1.x, rr.w, b0i);
        b1r = fmaf(m0.y, rr.z, b1r); b1i = fmaf(m0.y, rr.w, b1i);
        pm = m1.y;
    }
    if (t <= w) {                                       // w even: t = w
        const float4 rr = r4[t >> 1];
        const float2 m0 = inv_m2<STAGE>(mrow, mstride, t);
        a0r = fmaf(m0.x, rr.x, a0r); a0i = fmaf(m0.x, rr.y, a0i);
        a1r = fmaf(pm, rr.x, a1r);   a1i = fmaf(pm, rr.y, a1i);
        b1r = fmaf(m0.y, rr.z, b1r); b1i = fmaf(m0.y, rr.w, b1i);
    } else {                                            // w odd: t = w + 1
        const float2 rl = r32[q + t];
        a1r = fmaf(pm, rl.x, a1r); a1i = fmaf(pm, rl.y, a1i);
    }
    return make_float4(a0r + b0r, a0i + b0i, a1r + b1r, a1i + b1i);
}

template <int KD, bool R64, bool STAGE, typename TI, typename TO, typename TV>
__global__ void __launch_bounds__(kInvThreads) k_solve_inv(InvTab tab, const TI* __restrict__ in,
                                                           TO* __restrict__ out, TV* __restrict__ vstore,
                                                           Ctrl* __restrict__ ctrl, int dir, int scale_mode,
                                                           int check_broken, const double* __restrict__ bpart,
                                                           int bG) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ unsigned s_red[kInvThreads / 32];
    __shared__ __align__(8) unsigned long long s_bar;
    const int n = tab.n, w = tab.w, P = R64 ? tab.refine : 0;
    const int l = blockIdx.y, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int q0 = blockIdx.x * tab.chunk;
    int cl, R0, RB;
    inv_region(n, q0, tab.chunk, P, w, KD, &cl, &R0, &RB);
    const int R0p = (R0 + 3) & ~3;
    // carve shared memory (see inv_smem_bytes)
    unsigned char* sp = smem_raw;
    double2* bq = reinterpret_cast<double2*>(sp);
    sp += (size_t)RB * 16;
    double2* xq = reinterpret_cast<double2*>(sp);
    double2* rq = xq + R0;
    if (R64) sp += (size_t)R0 * 16 + (size_t)RB * 16;
    float* Ms = reinterpret_cast<float*>(sp);
    if (STAGE) sp += (size_t)(w + 1) * R0p * 4;
    float2* r32 = reinterpret_cast<float2*>(sp);     // 16-byte aligned; 2 slots of padding
    sp += (size_t)(R0 + w + 2) * 8;
    float2* x0f = reinterpret_cast<float2*>(sp);     // FP32 first iterate (exact in FP32)

    const float* Mg = tab.m + q0;
    const double* Ug = tab.u + q0;
    const float* Uhg = tab.uh + q0;
    const float* Ulg = tab.ul + q0;
    if (STAGE) {
        // one thread arms the barrier with the byte count and issues one bulk copy per
        // diagonal (rows of R0p elements: sizes and addresses are multiples of 16 bytes)
        if (tid == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&s_bar)) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();                               // barrier initialised before anyone polls it
        if (tid == 0) {
            const unsigned mrow = (unsigned)R0p * 4;
            const unsigned bytes = (unsigned)(w + 1) * mrow;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                         :: "r"(smem_u32(&s_bar)), "r"(bytes) : "memory");
            for (int j = 0; j <= w; ++j) bulk_g2s(Ms + (size_t)j * R0p, Mg + (size_t)j * tab.npad, mrow, &s_bar);
        }
    }
    // the band of M is constant and is staged before the wait; everything below reads what
    // earlier kernels wrote
    pdl_wait();
    if (check_broken && ctrl->broken) {
        if (STAGE) mbar_wait0(&s_bar);             // copies in flight land before exit
        return;
    }
    const float* mbase = STAGE ? Ms : Mg;
    const size_t mstride = STAGE ? (size_t)R0p : (size_t)tab.npad;
    const double* ubase = Ug;
    const float* uhb = Uhg;
    const float* ulb = Ulg;
    const size_t ustride = (size_t)tab.npad;
    const size_t base = (size_t)l * n;

    {
        // late: 1/beta comes from the Gram-Schmidt kernel's norm partials -- warp 0 forms it
        // while the other warps load the right-hand side, which is scaled afterwards
        const bool late = scale_mode && bpart;
        const double sc = scale_mode && !late ? ctrl->inv_beta : 1.0;
        __shared__ double s_ibeta;
        __shared__ int s_brk;
        if (late && warp == 0) {
            const double beta = gs_beta<false>(bpart, bG);
            if (lane == 0) {
                s_brk = gs_record_beta(ctrl, beta, blockIdx.x == 0 && blockIdx.y == 0);
                s_ibeta = 1.0 / beta;
            }
        }
        const int t0 = late ? tid - 32 : tid, tstep = late ? kInvThreads - 32 : kInvThreads;
        if (t0 >= 0)
            for (int q = t0; q < RB; q += tstep) {
                const int p = dir ? (n - 1 - (q0 + q)) : (q0 + q);
                const TI t = in[base + p];
                double2 b = make_double2((double)t.x, (double)t.y);
                if (scale_mode && !late) { b.x *= sc; b.y *= sc; }
                if (vstore && q < cl && !late) vstore[base + p] = conv<TV>(b);
                bq[q] = b;
                if (q < R0) xq[q] = make_double2(0.0, 0.0);
            }
        if (late) {
            __syncthreads();
            if (s_brk) {                               // uniform: the same beta in every CTA
                if (STAGE) mbar_wait0(&s_bar);
                return;
            }
            const double ib = s_ibeta;
            for (int q = tid; q < RB; q += kInvThreads) {
                double2 b = bq[q];
                b.x *= ib;
                b.y *= ib;
                bq[q] = b;
                if (vstore && q < cl) vstore[base + (dir ? (n - 1 - (q0 + q)) : (q0 + q))] = conv<TV>(b);
            }
        }
        bool ok = true;
        if (STAGE) ok = mbar_wait0(&s_bar, wait_budget(ctrl, kInvWaitLimit));
        if (!__syncthreads_and(ok)) {
            if (tid == 0) ctrl->wait_timeout = 1;
            if (STAGE) mbar_wait0(&s_bar);
            return;
        }
        bool x0_exact = false;                     // x after pass 0 is the FP32 vector x0f
        for (int k = 0; k <= P; ++k) {
            const int Rk = min(n - q0, cl + (P - k) * (w + KD));
            const int Rr = min(n - q0, Rk + w);
            if (k == 1 && P >= 2 && x0_exact) {
                // first refinement: r = b - U~ x0 with x0 exact in FP32, formed with FP32 pairs
                // (U~ = uh + ul, b = bh + bl; error-free products and sums).  Its relative error
                // (~2^-48 |b| / |r|) is far below what this pass needs; the last pass uses an FP64
                // residual.  No scaling: |b| has an FP32-safe exponent (checked at pass 0).
                for (int q = tid; q < Rk + w + 2; q += kInvThreads) {
                    float2 v = make_float2(0.f, 0.f);
                    if (q < Rr) {
                        float hr = 0.f, lr = 0.f, hi_ = 0.f, li = 0.f;
#pragma unroll
                        for (int d = 0; d <= KD; ++d) {
                            if (q + d < n - q0) {
                                const float uh = __ldg(uhb + (size_t)d * ustride + q);
                                const float ul = __ldg(ulb + (size_t)d * ustride + q);
                                const float2 xv = x0f[q + d];
                                acc_prod(hr, lr, uh, ul, xv.x);
                                acc_prod(hi_, li, uh, ul, xv.y);
                            }
                        }
                        const double2 b = bq[q];
                        const float bhx = d2f_fast(b.x), bhy = d2f_fast(b.y);
                        const float blx = d2f_fast(b.x - f2d_fast(bhx)), bly = d2f_fast(b.y - f2d_fast(bhy));
                        float s_, e_;
                        two_sum(bhx, -hr, s_, e_);
                        v.x = __fadd_rn(s_, __fadd_rn(e_, __fsub_rn(blx, lr)));
                        two_sum(bhy, -hi_, s_, e_);
                        v.y = __fadd_rn(s_, __fadd_rn(e_, __fsub_rn(bly, li)));
                    }
                    r32[q] = v;
                }
                __syncthreads();
                for (int q = 2 * tid; q < Rk; q += 2 * kInvThreads) {
                    const float4 f = inv_apply2<STAGE>(mbase + q, mstride, r32, q, w);
                    double2 x = xq[q];
                    x.x += f2d_fast(f.x);
                    x.y += f2d_fast(f.y);
                    xq[q] = x;
                    if (q + 1 < Rk) {
                        x = xq[q + 1];
                        x.x += f2d_fast(f.z);
                        x.y += f2d_fast(f.w);
                        xq[q + 1] = x;
                    }
                }
                __syncthreads();
                continue;
            }
            // residual r = b - U~ x (FP64, two FMA chains per component) and the max of
            // its high words (monotone in |r|)
            unsigned hmax = 0;
            for (int q = tid; q < Rr; q += kInvThreads) {
                double2 r = bq[q];
                if (k > 0) {
                    double ar = 0.0, ai = 0.0;
#pragma unroll
                    for (int d = 0; d <= KD; ++d) {
                        if (q + d < n - q0) {
                            const double u = __ldg(ubase + (size_t)d * ustride + q);
                            const double2 xv = xq[q + d];
                            if (d & 1) { ar = fma(-u, xv.x, ar); ai = fma(-u, xv.y, ai); }
                            else { r.x = fma(-u, xv.x, r.x); r.y = fma(-u, xv.y, r.y); }
                        }
                    }
                    r.x += ar;
                    r.y += ai;
                    rq[q] = r;
                }
                hmax = max(hmax, max((unsigned)__double2hiint(r.x) & 0x7fffffffu,
                                     (unsigned)__double2hiint(r.y) & 0x7fffffffu));
            }
            hmax = __reduce_max_sync(0xffffffffu, hmax);
            if (lane == 0) s_red[warp] = hmax;
            __syncthreads();
            hmax = 0;
#pragma unroll
            for (int i = 0; i < kInvThreads / 32; ++i) hmax = max(hmax, s_red[i]);
            if (hmax == 0) break;                      // zero residual: x is exact (or b = 0)
            const int e = (int)(hmax >> 20) - 1022;
            const bool scaled = e < -100 || e > 100;
            const double sdown = scaled ? ldexp(1.0, -e) : 1.0, sup = scaled ? ldexp(1.0, e) : 1.0;
            const double2* rsrc = k > 0 ? rq : bq;
            for (int q = tid; q < Rk + w + 2; q += kInvThreads) {
                float2 v = make_float2(0.f, 0.f);
                if (q < Rr) {
                    double2 r = rsrc[q];
                    if (scaled) { r.x *= sdown; r.y *= sdown; }
                    v = make_float2(d2f_fast(r.x), d2f_fast(r.y));
                }
                r32[q] = v;
            }
            __syncthreads();
            for (int q = 2 * tid; q < Rk; q += 2 * kInvThreads) {
                const float4 f4 = inv_apply2<STAGE>(mbase + q, mstride, r32, q, w);
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    if (e == 1 && q + 1 >= Rk) break;
                    const float2 f = e ? make_float2(f4.z, f4.w) : make_float2(f4.x, f4.y);
                    double2 x = xq[q + e];
                    if (scaled) { x.x = fma(f2d_fast(f.x), sup, x.x); x.y = fma(f2d_fast(f.y), sup, x.y); }
                    else if (k == 0) x = make_double2(f2d_fast(f.x), f2d_fast(f.y));   // x was 0: no add
                    else { x.x += f2d_fast(f.x); x.y += f2d_fast(f.y); }
                    xq[q + e] = x;
                    if (k == 0) x0f[q + e] = f;          // x0 = f exactly when unscaled
                }
            }
            if (k == 0) x0_exact = !scaled && e > -60 && e < 60;   // the FP32-pair residual stays normal
            __syncthreads();
        }
        const bool rnd = check_broken && (ctrl->round_matvec & 2);   // precision probe, Arnoldi solves
        for (int q = tid; q < cl; q += kInvThreads) {
            const int p = dir ? (n - 1 - (q0 + q)) : (q0 + q);
            out[base + p] = conv<TO>(rnd ? round_c64(xq[q]) : xq[q]);
        }
    }
}

// Complex64 solve of the mixed path's Krylov basis (one CTA per chunk of a row):
//   x0 = M b_hi                       FP32
//   r  = b - U~ x0                    FP32 pairs: U~ = uh + ul, b = bh + bl (bl = 0 for a
//                                     complex64 operand), error-free products and sums
//   x  = x0 + M r                     FP32, rounded once
// The refinement makes the operator seen by the basis U^-1 to ~1e-13 (the FP32 band of
// M alone perturbs it by ~1e-7, which shifts high eigenvalues systematically).  A
// double2 operand (the FP64 first vector) is used as hi + lo, a complex64 operand as
// stored, so the solve acts on exactly the vector kept in the basis.
template <int KD, bool STAGE, typename TI, typename TV>
__global__ void __launch_bounds__(kInvThreads) k_solve_mixed(InvTab tab, const TI* __restrict__ in,
                                                             float2* __restrict__ out, TV* __restrict__ vstore,
                                                             Ctrl* __restrict__ ctrl, int dir, int scale_mode,
                                                             int check_broken, float4* __restrict__ v0s,
                                                             const float4* __restrict__ bpart, int bG) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(8) unsigned long long s_bar;
    const int n = tab.n, w = tab.w;
    const int l = blockIdx.y, tid = threadIdx.x;
    const int q0 = blockIdx.x * tab.chunk;
    int cl, R0, RB;
    inv_region(n, q0, tab.chunk, 1, w, KD, &cl, &R0, &RB);
    const int R0p = (R0 + 3) & ~3;
    unsigned char* sp = smem_raw;                  // bulk-copy destinations first (16-byte aligned)
    float* Ms = reinterpret_cast<float*>(sp);
    float* Uh = Ms + (size_t)(w + 1) * R0p;
    float* Ul = Uh + (size_t)(KD + 1) * R0p;
    if (STAGE) sp += (size_t)(w + 1) * R0p * 4 + (size_t)2 * (KD + 1) * R0p * 4;
    float2* bh = reinterpret_cast<float2*>(sp);
    float2* bl = bh + RB;
    float2* x0 = bl + RB;                          // 16-byte aligned
    float2* r32 = x0 + ((R0 + 1) & ~1);            // 16-byte aligned; 2 slots of padding

    const float* Mg = tab.m + q0;
    const float* Uhg = tab.uh + q0;
    const float* Ulg = tab.ul + q0;
    if (STAGE) {
        if (tid == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&s_bar)) : "memory");
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();
        if (tid == 0) {
            const unsigned row = (unsigned)R0p * 4;
            const unsigned bytes = (unsigned)(w + 1 + 2 * (KD + 1)) * row;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                         :: "r"(smem_u32(&s_bar)), "r"(bytes) : "memory");
            for (int j = 0; j <= w; ++j) bulk_g2s(Ms + (size_t)j * R0p, Mg + (size_t)j * tab.npad, row, &s_bar);
            for (int d = 0; d <= KD; ++d) {
                bulk_g2s(Uh + (size_t)d * R0p, Uhg + (size_t)d * tab.npad, row, &s_bar);
                bulk_g2s(Ul + (size_t)d * R0p, Ulg + (size_t)d * tab.npad, row, &s_bar);
            }
        }
    }
    pdl_wait();
    if (check_broken && ctrl->broken) {
        if (STAGE) mbar_wait0(&s_bar);
        return;
    }
    const float* mbase = STAGE ? Ms : Mg;
    const size_t mstride = STAGE ? (size_t)R0p : (size_t)tab.npad;
    const float* uhb = STAGE ? Uh : Uhg;
    const float* ulb = STAGE ? Ul : Ulg;
    const size_t ustride = STAGE ? (size_t)R0p : (size_t)tab.npad;
    const size_t base = (size_t)l * n;
    constexpr bool kWide = sizeof(TI) == sizeof(double2);
    if constexpr (kWide) {
        // the FP64 first vector (once per step): scaled in FP64, kept as hi + lo
        const double sc = scale_mode ? ctrl->inv_beta : 1.0;
        for (int q = tid; q < R0 + w + 2; q += kInvThreads) {
            float2 hi = make_float2(0.f, 0.f), lo = make_float2(0.f, 0.f);
            if (q < RB) {
                const int p = dir ? (n - 1 - (q0 + q)) : (q0 + q);
                const TI t = in[base + p];
                double2 b = make_double2((double)t.x, (double)t.y);
                if (scale_mode) { b.x *= sc; b.y *= sc; }
                hi = make_float2(d2f_fast(b.x), d2f_fast(b.y));
                lo = make_float2(d2f_fast(b.x - f2d_fast(hi.x)), d2f_fast(b.y - f2d_fast(hi.y)));
                if (q < cl) {
                    if (vstore) vstore[base + p] = conv<TV>(b);
                    if (v0s) v0s[base + p] = make_float4(hi.x, hi.y, lo.x, lo.y);
                }
                bh[q] = hi;
                bl[q] = lo;
            }
            r32[q] = hi;
        }
    } else {
        // a complex64 vector: scaled by 1/beta as an FP32 pair, rounded once (no FP64
        // instruction per element).  late: 1/beta from the Gram-Schmidt kernel's norm
        // partials, formed by warp 0 while the other warps load (see k_solve_inv)
        const bool late = scale_mode && bpart;
        __shared__ float2 s_ibf;
        __shared__ int s_brk;
        if (late && (tid >> 5) == 0) {
            const double beta = gs_beta<true>(bpart, bG);
            if ((tid & 31) == 0) {
                s_brk = gs_record_beta(ctrl, beta, blockIdx.x == 0 && blockIdx.y == 0);
                const double ib = 1.0 / beta;
                const float h = (float)ib;
                s_ibf = make_float2(h, (float)(ib - (double)h));
            }
        }
        float sh = 1.f, sl = 0.f;
        if (scale_mode && !late) { sh = ctrl->inv_beta_f[0]; sl = ctrl->inv_beta_f[1]; }
        const int t0 = late ? tid - 32 : tid, tstep = late ? kInvThreads - 32 : kInvThreads;
        if (t0 >= 0)
            for (int q = t0; q < R0 + w + 2; q += tstep) {
                float2 hi = make_float2(0.f, 0.f);
                if (q < RB) {
                    const int p = dir ? (n - 1 - (q0 + q)) : (q0 + q);
                    const TI t = in[base + p];
                    hi = make_float2((float)t.x, (float)t.y);
                    if (scale_mode && !late) hi = make_float2(mul_pair(hi.x, sh, sl), mul_pair(hi.y, sh, sl));
                    if (vstore && q < cl && !late) vstore[base + p] = conv<TV>(hi);
                    bh[q] = hi;
                    bl[q] = make_float2(0.f, 0.f);
                }
                r32[q] = hi;
            }
        if (late) {
            __syncthreads();
            if (s_brk) {                               // uniform: the same beta in every CTA
                if (STAGE) mbar_wait0(&s_bar);
                return;
            }
            sh = s_ibf.x;
            sl = s_ibf.y;
            for (int q = tid; q < RB; q += kInvThreads) {
                const float2 b = bh[q];
                const float2 hi = make_float2(mul_pair(b.x, sh, sl), mul_pair(b.y, sh, sl));
                bh[q] = hi;
                r32[q] = hi;
                if (vstore && q < cl) vstore[base + (dir ? (n - 1 - (q0 + q)) : (q0 + q))] = conv<TV>(hi);
            }
        }
    }
    bool ok = true;
    if (STAGE) ok = mbar_wait0(&s_bar, wait_budget(ctrl, kInvWaitLimit));
    if (!__syncthreads_and(ok)) {
        if (tid == 0) ctrl->wait_timeout = 1;
        if (STAGE) mbar_wait0(&s_bar);             // let copies in flight land before exit
        return;
    }
    for (int q = 2 * tid; q < R0; q += 2 * kInvThreads) {
        const float4 f = inv_apply2<STAGE>(mbase + q, mstride, r32, q, w);
        if (q + 1 < R0) *reinterpret_cast<float4*>(x0 + q) = f;
        else x0[q] = make_float2(f.x, f.y);
    }
    __syncthreads();
    const int Rr = min(n - q0, cl + w);
    for (int q = tid; q < cl + w; q += kInvThreads) {
        float2 r = make_float2(0.f, 0.f);
        if (q < Rr) {
            float hr = 0.f, lr = 0.f, hi_ = 0.f, li = 0.f;
#pragma unroll
            for (int d = 0; d <= KD; ++d) {
                if (q + d < n - q0) {
                    const float uh = uhb[(size_t)d * ustride + q], ul = ulb[(size_t)d * ustride + q];
                    const float2 xv = x0[q + d];
                    acc_prod(hr, lr, uh, ul, xv.x);
                    acc_prod(hi_, li, uh, ul, xv.y);
                }
            }
            const float2 b_h = bh[q], b_l = bl[q];
            float s, e;
            two_sum(b_h.x, -hr, s, e);
            r.x = __fadd_rn(s, __fadd_rn(e, __fsub_rn(b_l.x, lr)));
            two_sum(b_h.y, -hi_, s, e);
            r.y = __fadd_rn(s, __fadd_rn(e, __fsub_rn(b_l.y, li)));
        }
        r32[q] = r;
    }
    __syncthreads();
    for (int q = 2 * tid; q < cl; q += 2 * kInvThreads) {
        const float4 d = inv_apply2<STAGE>(mbase + q, mstride, r32, q, w);
        float2 x = x0[q];
        out[base + (dir ? (n - 1 - (q0 + q)) : (q0 + q))] = make_float2(__fadd_rn(x.x, d.x), __fadd_rn(x.y, d.y));
        if (q + 1 < cl) {
            x = x0[q + 1];
            out[base + (dir ? (n - 2 - (q0 + q)) : (q0 + q + 1))] = make_float2(__fadd_rn(x.x, d.z), __fadd_rn(x.y, d.w));
        }
    }
}

template <int KD, bool STAGE>
static cudaError_t solve_mixed_launch(const InvTab& tab, int nrows, const void* in, int in_prec, void* out,
                                      int out_prec, void* vstore, int v_prec, Ctrl* ctrl, int dir, int scale_mode,
                                      int check_broken, cudaStream_t s, float4* v0s, const void* bpart, int bG) {
    if (out_prec != 1) return cudaErrorInvalidValue;
    size_t smem = 0;
    for (int c = 0; c < tab.nchunks; ++c)
        smem = std::max(smem, inv_smem_bytes_mixed(tab.n, c * tab.chunk, tab.chunk, tab.w, KD, STAGE));
    dim3 grid(tab.nchunks, nrows), block(kInvThreads);
#define GB_MIX_CASE(TI_, TV_)                                                                                    \
    {                                                                                                            \
        auto kern = k_solve_mixed<KD, STAGE, TI_, TV_>;                                                          \
        if (smem > 48 * 1024) {                                                                                  \
            cudaError_t ea = allow_max_smem(kern);                                                               \
            if (ea != cudaSuccess) return ea;                                                                    \
        }                                                                                                        \
        cudaError_t el = launch_pdl(kern, grid, block, smem, s, tab, (const TI_*)in, (float2*)out, (TV_*)vstore,  \
                                    ctrl, dir, scale_mode, check_broken, v0s, (const float4*)bpart, bG);         \
        return el != cudaSuccess ? el : cudaGetLastError();                                                      \
    }
    // in: the FP64 first vector (with its FP64 copy stored) or a complex64 vector
    if (in_prec == 0 && v_prec == 0) GB_MIX_CASE(double2, double2)
    if (v0s) return cudaErrorInvalidValue;
    if (in_prec == 1) GB_MIX_CASE(float2, float2)
#undef GB_MIX_CASE
    return cudaErrorInvalidValue;
}

template <int KD, bool R64, bool STAGE>
static cudaError_t solve_inv_launch(const InvTab& tab, int nrows, const void* in, int in_prec, void* out,
                                    int out_prec, void* vstore, int v_prec, Ctrl* ctrl, int dir,
                                    int scale_mode, int check_broken, cudaStream_t s, const void* bpart, int bG) {
    const int P = R64 ? tab.refine : 0;
    size_t smem = 0;
    for (int c = 0; c < tab.nchunks; ++c)
        smem = std::max(smem, inv_smem_bytes(tab.n, c * tab.chunk, tab.chunk, P, tab.w, KD, STAGE, R64));
    dim3 grid(tab.nchunks, nrows), block(kInvThreads);
#define GB_INV_CASE(TI_, TO_, TV_)                                                                               \
    {                                                                                                            \
        auto kern = k_solve_inv<KD, R64, STAGE, TI_, TO_, TV_>;                                                  \
        if (smem > 48 * 1024) {                                                                                  \
            cudaError_t ea = allow_max_smem(kern);                                                               \
            if (ea != cudaSuccess) return ea;                                                                    \
        }                                                                                                        \
        cudaError_t el = launch_pdl(kern, grid, block, smem, s, tab, (const TI_*)in, (TO_*)out, (TV_*)vstore,     \
                                    ctrl, dir, scale_mode, check_broken, (const double*)bpart, bG);              \
        return el != cudaSuccess ? el : cudaGetLastError();                                                      \
    }
    // combinations the runtime uses: refined solves store double2 (or nothing)
    const int key = in_prec * 4 + out_prec * 2 + v_prec;
    switch (key) {
        case 0: GB_INV_CASE(double2, double2, double2)
        case 2: GB_INV_CASE(double2, float2, double2)
        case 4: GB_INV_CASE(float2, double2, double2)
        case 6: GB_INV_CASE(float2, float2, double2)
        default: return cudaErrorInvalidValue;
    }
#undef GB_INV_CASE
}

template <int KD>
static cudaError_t solve_inv_kd(const InvTab& tab, int nrows, int refine64, const void* in, int in_prec, void* out,
                                int out_prec, void* vstore, int v_prec, Ctrl* ctrl, int dir, int scale_mode,
                                int check_broken, cudaStream_t s, float4* v0s, const void* bpart, int bG) {
    if (refine64) {
        if (tab.stage)
            return solve_inv_launch<KD, true, true>(tab, nrows, in, in_prec, out, out_prec, vstore, v_prec, ctrl, dir,
                                                    scale_mode, check_broken, s, bpart, bG);
        return solve_inv_launch<KD, true, false>(tab, nrows, in, in_prec, out, out_prec, vstore, v_prec, ctrl, dir,
                                                 scale_mode, check_broken, s, bpart, bG);
    }
    if (tab.stage)
        return solve_mixed_launch<KD, true>(tab, nrows, in, in_prec, out, out_prec, vstore, v_prec, ctrl, dir,
                                            scale_mode, check_broken, s, v0s, bpart, bG);
    return solve_mixed_launch<KD, false>(tab, nrows, in, in_prec, out, out_prec, vstore, v_prec, ctrl, dir,
                                         scale_mode, check_broken, s, v0s, bpart, bG);
}

cudaError_t launch_solve_inv(const InvTab& tab, int nrows, int refine64, const void* in, int in_prec, void* out,
                             int out_prec, void* vstore, int v_prec, Ctrl* ctrl, int dir, int scale_mode,
                             int check_broken, cudaStream_t s, float4* v0s, const void* bpart, int bG) {
    count_launch();
    switch (tab.kd) {
#define GB_KD(K)                                                                                                 \
    case K:                                                                                                      \
        return solve_inv_kd<K>(tab, nrows, refine64, in, in_prec, out, out_prec, vstore, v_prec, ctrl, dir,      \
                               scale_mode, check_broken, s, v0s, bpart, bG);
        GB_KD(1) GB_KD(2) GB_KD(3) GB_KD(4) GB_KD(5) GB_KD(6) GB_KD(7) GB_KD(8)
#undef GB_KD
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace gbprop
