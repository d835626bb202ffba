// Radial TensorPotential set-up on the GPU: the B-spline band matrices <B_i| f |d^n B_j> of a
// B-spline basis by Gauss-Legendre quadrature, and the upper Cholesky factor of the overlap
// (the reference's set-up of this path: RepresentPotentialInBasisBSpline,
// core/tensorpotential/basis_bspline.h:10-48 -> BSpline::BSplineGlobalOverlapIntegral,
// core/transform/bspline/bspline.cpp:373-467, with the tables of bspline.cpp:26-289, and
// OverlapMatrix::Setup -> zpbtrf, core/representation/overlapmatrix.cpp:9-104).
//
// The arithmetic follows the host restatement (pyprop_gb300/basis/bspline.py: local_tables,
// band_diagonals, band_cholesky_upper_diagonals) operation by operation -- the same
// three-point recursions with the `> eps` guards, the same product and summation orders -- and
// this file is compiled without FMA contraction, so the device results equal the host's.
#include "gbprop_internal.h"
#include "../../include/gbprop.h"

#include <cstring>
#include <string>
#include <vector>

namespace gbprop {

constexpr double kEps = 1e-15;     // the recursions' guard (bspline.cpp:26-164)
constexpr int kMaxOrder = 9;

// t[i] of the knot sequence padded with `order` copies of its end knots on both sides
__device__ __forceinline__ double knot(const double* tp, int k, int i) { return tp[i + k]; }

// One thread per quadrature point g: its knot span, grid point, weight, and the values,
// first and second derivatives of the `order` splines that can be non-zero there.
__global__ void k_bspline_tables(int k, int nt, const double* __restrict__ tp, int nb, const double* __restrict__ bp,
                                 int nq, const double* __restrict__ nodes, const double* __restrict__ weights,
                                 double* __restrict__ xg, double* __restrict__ wg, int* __restrict__ first,
                                 double* __restrict__ tab) {
    const int ng = (nb - 1) * nq;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= ng) return;
    const int iv = g / nq, qn = g - iv * nq;
    const double a = bp[iv], b = bp[iv + 1];
    const double x = (nodes[qn] - 1.0) * (b - a) / 2.0 + b;      // scale_and_translate (bspline.h:173-176)
    const double w = (b - a) / 2.0 * weights[qn];
    // mu = index of the last knot <= x
    int lo = 0, hi = nt;                                          // first knot > x
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (knot(tp, k, mid) <= x) lo = mid + 1;
        else hi = mid;
    }
    const int mu = lo - 1;
    double lev[kMaxOrder + 1][kMaxOrder];                          // lev[q][a], q = 1..k
    lev[1][0] = 1.0;
    for (int q = 2; q <= k; ++q)
        for (int aa = 0; aa < q; ++aa) {
            const int i = mu - q + 1 + aa;
            double cur = 0.0;
            if (aa >= 1) {
                const double b0 = lev[q - 1][aa - 1];
                const double d0 = knot(tp, k, i + q - 1) - knot(tp, k, i);
                cur += b0 > kEps ? (x - knot(tp, k, i)) / d0 * b0 : 0.0;
            }
            if (aa <= q - 2) {
                const double b1 = lev[q - 1][aa];
                const double d1 = knot(tp, k, i + q) - knot(tp, k, i + 1);
                cur += b1 > kEps ? (knot(tp, k, i + q) - x) / d1 * b1 : 0.0;
            }
            lev[q][aa] = cur;
        }
    double* Bv = tab + (size_t)g * 3 * k;
    double* D1 = Bv + k;
    double* D2 = D1 + k;
    for (int aa = 0; aa < k; ++aa) {
        const int i = mu - k + 1 + aa;
        double d1 = 0.0, d2 = 0.0;
        if (aa >= 1) {
            const double p1 = lev[k - 1][aa - 1];
            d1 += p1 > kEps ? (k - 1.0) / (knot(tp, k, i + k - 1) - knot(tp, k, i)) * p1 : 0.0;
        }
        if (aa <= k - 2) {
            const double p2 = lev[k - 1][aa];
            d1 -= p2 > kEps ? (k - 1.0) / (knot(tp, k, i + k) - knot(tp, k, i + 1)) * p2 : 0.0;
        }
        if (k > 2) {
            double q1 = (aa - 2 >= 0 && aa - 2 <= k - 3) ? lev[k - 2][aa - 2] : 0.0;
            double q2 = (aa - 1 >= 0 && aa - 1 <= k - 3) ? lev[k - 2][aa - 1] : 0.0;
            double q3 = (aa <= k - 3) ? lev[k - 2][aa] : 0.0;
            q1 = q1 > kEps ? q1 * ((k - 2.0) / (knot(tp, k, i + k - 2) - knot(tp, k, i))) : q1;
            q2 = q2 > kEps ? q2 * ((k - 2.0) / (knot(tp, k, i + k - 1) - knot(tp, k, i + 1))) : q2;
            q3 = q3 > kEps ? q3 * ((k - 2.0) / (knot(tp, k, i + k) - knot(tp, k, i + 2))) : q3;
            const double a_ = (k - 1.0) / (knot(tp, k, i + k - 1) - knot(tp, k, i));
            const double dd = (k - 1.0) / (knot(tp, k, i + k) - knot(tp, k, i + 1));
            d2 += (q1 > kEps || q2 > kEps) ? a_ * (q1 - q2) : 0.0;
            d2 -= (q2 > kEps || q3 > kEps) ? dd * (q2 - q3) : 0.0;
        }
        // np.nan_to_num of the host tables
        const double bv = lev[k][aa];
        Bv[aa] = isnan(bv) ? 0.0 : bv;
        D1[aa] = isnan(d1) ? 0.0 : d1;
        D2[aa] = isnan(d2) ? 0.0 : d2;
    }
    xg[g] = x;
    wg[g] = w;
    first[g] = mu - k + 1;
}

// f(x) of a radial term: 0 -> c, 1 -> c / x, 2 -> c / (2 x x)
__device__ __forceinline__ double radial_fn(int fid, double c, double x) {
    if (fid == 1) return c / x;
    if (fid == 2) return c / (2.0 * x * x);
    return c;
}

// One thread per (matrix, diagonal d >= 0, spline i): D[kb + d][i] = sum over a of (sum over
// the points whose first spline is i - a, ascending) of (w f)(x) B_{i}(x) d^n B_{i+d}(x); the
// lower diagonals follow the swap rule D[kb - d][i + d] = (-1)^n D[kb + d][i] (bspline.cpp:384-392).
__global__ void k_bspline_band(int k, int n, int ng, int nmat, const int* __restrict__ fid,
                               const int* __restrict__ deriv, const double* __restrict__ coef,
                               const double* __restrict__ xg, const double* __restrict__ wg,
                               const int* __restrict__ first, const double* __restrict__ tab,
                               const int* __restrict__ span0, double* __restrict__ out) {
    const int kb = k - 1, W = 2 * kb + 1;
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)nmat * k * n) return;
    const int i = (int)(idx % n);
    const int d = (int)((idx / n) % k);
    const int mtx = (int)(idx / ((long)n * k));
    double* D = out + (size_t)mtx * W * n;
    if (i + d >= n) {
        D[(size_t)(kb + d) * n + i] = 0.0;
        return;
    }
    const int nd = deriv[mtx], f = fid[mtx];
    const double c = coef[mtx];
    double acc = 0.0;
    for (int a = 0; a + d < k; ++a) {
        const int f0 = i - a;
        if (f0 < -kb || f0 >= n) continue;
        // points whose first spline is f0 are contiguous; span0[f0 + kb] .. span0[f0 + kb + 1]
        const int g0 = span0[f0 + kb], g1 = span0[f0 + kb + 1];
        double s = 0.0;
        for (int g = g0; g < g1; ++g) {
            const double* T = tab + (size_t)g * 3 * k;
            const double wf = wg[g] * radial_fn(f, c, xg[g]);
            s += wf * T[a] * T[nd * k + a + d];
        }
        acc += s;
    }
    D[(size_t)(kb + d) * n + i] = acc;
    if (d > 0) D[(size_t)(kb - d) * n + i + d] = (nd & 1 ? -1.0 : 1.0) * acc;
}

// Upper band Cholesky factor of the symmetric band matrix S (diagonals Sd[kd + d][i] =
// S(i, i+d)): Ud[d][j] = U(j, j+d); one thread, the column order of the host restatement.
// info[0] = 0, or 1 + the column where S is not positive definite.
__global__ void k_band_cholesky(int n, int kd, const double* __restrict__ Sd, double* __restrict__ Ud, int* info) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    info[0] = 0;
    for (int j = 0; j < n; ++j) {
        double d0 = Sd[(size_t)kd * n + j];
        for (int t = 1; t <= (kd < j ? kd : j); ++t) {
            const double u = Ud[(size_t)t * n + j - t];
            d0 -= u * u;
        }
        if (!(d0 > 0.0)) {
            info[0] = j + 1;
            return;
        }
        d0 = sqrt(d0);
        Ud[j] = d0;
        for (int dd = 1; dd <= kd; ++dd) {
            const int i = j + dd;
            if (i >= n) break;
            double sv = Sd[(size_t)(kd + dd) * n + j];
            for (int t = 1; t <= kd; ++t) {
                const int r = j - t;
                if (r < 0 || i - r > kd) continue;
                sv -= Ud[(size_t)t * n + r] * Ud[(size_t)(i - r) * n + r];
            }
            Ud[(size_t)dd * n + j] = sv / d0;
        }
    }
}

}  // namespace gbprop

using namespace gbprop;

namespace {
struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { if (p) cudaFree(p); }
};
}  // namespace

extern "C" gbprop_status gbprop_bspline_bands(int order, int nknots, const double* knots, int nbreak,
                                              const double* breakpoints, int nquad, const double* nodes,
                                              const double* weights, int nmat, const int* fid, const int* deriv,
                                              const double* coef, double* bands, double* cholesky, void* stream) {
    const int k = order, kb = order - 1;
    if (k < 2 || k > kMaxOrder) { set_last_error("order must be in [2, 9]"); return GBPROP_EINVAL; }
    if (!knots || !breakpoints || !nodes || !weights || !bands || nknots <= k || nbreak < 2 || nquad < 1 ||
        nmat < 1 || !fid || !deriv || !coef) {
        set_last_error("bad argument");
        return GBPROP_EINVAL;
    }
    for (int m = 0; m < nmat; ++m)
        if (fid[m] < 0 || fid[m] > 2 || deriv[m] < 0 || deriv[m] > 2) {
            set_last_error("radial term: function id in [0, 2], derivative order in [0, 2]");
            return GBPROP_EINVAL;
        }
    const int n = nknots - k, ng = (nbreak - 1) * nquad, W = 2 * kb + 1;
    cudaStream_t s = (cudaStream_t)stream;
    // host side: padded knots and, per first-spline index f0 = -kb..n-1, its run of points
    std::vector<double> tp(nknots + 2 * k);
    for (int i = 0; i < k; ++i) { tp[i] = knots[0]; tp[nknots + k + i] = knots[nknots - 1]; }
    std::memcpy(tp.data() + k, knots, nknots * sizeof(double));
    DevBuf d_tp, d_bp, d_nodes, d_w, d_xg, d_wg, d_first, d_tab, d_span, d_fid, d_der, d_coef, d_out, d_ud, d_info;
    auto alloc = [&](DevBuf& b, size_t bytes) { return cudaMalloc(&b.p, bytes ? bytes : 16); };
    cudaError_t e = cudaSuccess;
    e = e ? e : alloc(d_tp, tp.size() * 8);
    e = e ? e : alloc(d_bp, nbreak * 8);
    e = e ? e : alloc(d_nodes, nquad * 8);
    e = e ? e : alloc(d_w, nquad * 8);
    e = e ? e : alloc(d_xg, ng * 8);
    e = e ? e : alloc(d_wg, ng * 8);
    e = e ? e : alloc(d_first, ng * 4);
    e = e ? e : alloc(d_tab, (size_t)ng * 3 * k * 8);
    e = e ? e : alloc(d_span, (n + kb + 1) * 4);
    e = e ? e : alloc(d_fid, nmat * 4);
    e = e ? e : alloc(d_der, nmat * 4);
    e = e ? e : alloc(d_coef, nmat * 8);
    e = e ? e : alloc(d_out, (size_t)nmat * W * n * 8);
    e = e ? e : alloc(d_ud, (size_t)k * n * 8);
    e = e ? e : alloc(d_info, 4);
    e = e ? e : cudaMemcpyAsync(d_tp.p, tp.data(), tp.size() * 8, cudaMemcpyHostToDevice, s);
    e = e ? e : cudaMemcpyAsync(d_bp.p, breakpoints, nbreak * 8, cudaMemcpyHostToDevice, s);
    e = e ? e : cudaMemcpyAsync(d_nodes.p, nodes, nquad * 8, cudaMemcpyHostToDevice, s);
    e = e ? e : cudaMemcpyAsync(d_w.p, weights, nquad * 8, cudaMemcpyHostToDevice, s);
    e = e ? e : cudaMemcpyAsync(d_fid.p, fid, nmat * 4, cudaMemcpyHostToDevice, s);
    e = e ? e : cudaMemcpyAsync(d_der.p, deriv, nmat * 4, cudaMemcpyHostToDevice, s);
    e = e ? e : cudaMemcpyAsync(d_coef.p, coef, nmat * 8, cudaMemcpyHostToDevice, s);
    if (e) { set_last_error(cudaGetErrorString(e)); return GBPROP_ECUDA; }
    count_launch();
    k_bspline_tables<<<(ng + 127) / 128, 128, 0, s>>>(k, nknots, (const double*)d_tp.p, nbreak, (const double*)d_bp.p,
                                                      nquad, (const double*)d_nodes.p, (const double*)d_w.p,
                                                      (double*)d_xg.p, (double*)d_wg.p, (int*)d_first.p,
                                                      (double*)d_tab.p);
    // runs of points per first-spline index (points are in increasing x, so first[] is
    // non-decreasing): span[f0 + kb] = first point with first >= f0
    std::vector<int> first(ng);
    e = cudaMemcpyAsync(first.data(), d_first.p, ng * 4, cudaMemcpyDeviceToHost, s);
    e = e ? e : cudaStreamSynchronize(s);
    if (e) { set_last_error(cudaGetErrorString(e)); return GBPROP_ECUDA; }
    std::vector<int> span(n + kb + 1);
    int g = 0;
    for (int f0 = -kb; f0 <= n; ++f0) {
        while (g < ng && first[g] < f0) ++g;
        span[f0 + kb] = g;
    }
    e = cudaMemcpyAsync(d_span.p, span.data(), span.size() * 4, cudaMemcpyHostToDevice, s);
    if (e) { set_last_error(cudaGetErrorString(e)); return GBPROP_ECUDA; }
    const long total = (long)nmat * k * n;
    e = cudaMemsetAsync(d_out.p, 0, (size_t)nmat * W * n * 8, s);
    if (e) { set_last_error(cudaGetErrorString(e)); return GBPROP_ECUDA; }
    count_launch();
    k_bspline_band<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(
        k, n, ng, nmat, (const int*)d_fid.p, (const int*)d_der.p, (const double*)d_coef.p, (const double*)d_xg.p,
        (const double*)d_wg.p, (const int*)d_first.p, (const double*)d_tab.p, (const int*)d_span.p, (double*)d_out.p);
    int info = 0;
    if (cholesky) {
        e = cudaMemsetAsync(d_ud.p, 0, (size_t)k * n * 8, s);      // U(i, i+d) = 0 beyond the matrix
        if (e) { set_last_error(cudaGetErrorString(e)); return GBPROP_ECUDA; }
        count_launch();
        k_band_cholesky<<<1, 32, 0, s>>>(n, kb, (const double*)d_out.p, (double*)d_ud.p, (int*)d_info.p);
        e = cudaMemcpyAsync(cholesky, d_ud.p, (size_t)k * n * 8, cudaMemcpyDeviceToHost, s);
        e = e ? e : cudaMemcpyAsync(&info, d_info.p, 4, cudaMemcpyDeviceToHost, s);
        if (e) { set_last_error(cudaGetErrorString(e)); return GBPROP_ECUDA; }
    }
    e = cudaMemcpyAsync(bands, d_out.p, (size_t)nmat * W * n * 8, cudaMemcpyDeviceToHost, s);
    e = e ? e : cudaStreamSynchronize(s);
    e = e ? e : cudaGetLastError();
    if (e) { set_last_error(cudaGetErrorString(e)); return GBPROP_ECUDA; }
    if (info) {
        set_last_error(("the first matrix (overlap) is not positive definite at column " + std::to_string(info - 1)).c_str());
        return GBPROP_EINVAL;
    }
    return GBPROP_OK;
}
