// Field-free bound states on the GPU: the eigenpairs with E < emax of the generalized
// symmetric banded problems H_l c = E S c, one per angular row l (the static, angular-diagonal
// TensorPotentials in the B-spline overlap metric).  The reference's hydrogen analysis solves
// them with a dense generalized eigensolver per l
// (examples/tensor/helium_stabilization_sae/analysis.py:92-160); here the band structure is
// used directly:
//   * inertia: the number of eigenvalues below sigma is the number of negative pivots of the
//     banded LDL^T factorisation of H - sigma S (Sylvester's law of inertia, S positive
//     definite), O(n kd^2) per count with a sliding window of the last kd rows of L in
//     registers;
//   * bisection on that count for every wanted eigenvalue (one thread per (row, index));
//   * inverse iteration at the converged eigenvalue (three banded LDL^T solves, the factor kept
//     in a global scratch array), normalised in the S metric.
// Bands are diagonal-major: A[d * n + i] = A(i, i + d - kd), d = 0..2kd (symmetric; only the
// lower half and the diagonal are read).
#include "gbprop_internal.h"
#include "../../include/gbprop.h"

#include <cfloat>
#include <cmath>
#include <string>
#include <vector>

namespace gbprop {

namespace {

constexpr int kBoundThreads = 128;

// Banded LDL^T of A = H - sigma S, row by row: li[m] = L(i, i-KD+m), d_i the pivot.
// Returns the number of negative pivots; with Lout != null the factor rows are stored
// (Lout[i * (KD+1) + m] = L(i, i-KD+m), Lout[i * (KD+1) + KD] = 1 / d_i).
template <int KD>
__device__ int band_ldlt(const double* __restrict__ Hb, const double* __restrict__ Sb, int n, double sigma,
                         double* __restrict__ Lout) {
    double W[KD][KD];           // L rows of the previous KD rows (row r: W[r][m] = L(i-KD+r, i-2KD+r+m))
    double dp[KD], ip[KD];      // their pivots and inverse pivots
#pragma unroll
    for (int r = 0; r < KD; ++r) {
        dp[r] = 1.0;
        ip[r] = 0.0;            // rows before the start: no contribution
#pragma unroll
        for (int m = 0; m < KD; ++m) W[r][m] = 0.0;
    }
    int neg = 0;
    const double tiny = 1e-280;
    for (int i = 0; i < n; ++i) {
        double li[KD];
#pragma unroll
        for (int m = 0; m < KD; ++m) {
            const int j = i - KD + m;
            double a = 0.0;
            if (j >= 0) a = __ldg(Hb + (size_t)m * n + i) - sigma * __ldg(Sb + (size_t)m * n + i);
#pragma unroll
            for (int p = 0; p < m; ++p) a = fma(-li[p] * dp[p], W[m][p + KD - m], a);
            li[m] = a * ip[m];
        }
        double d = __ldg(Hb + (size_t)KD * n + i) - sigma * __ldg(Sb + (size_t)KD * n + i);
#pragma unroll
        for (int m = 0; m < KD; ++m) d = fma(-li[m] * li[m], dp[m], d);
        if (!(fabs(d) >= tiny)) d = (d < 0.0) ? -tiny : tiny;   // exact zero (or NaN): a tiny pivot
        neg += d < 0.0;
        const double id = 1.0 / d;
        if (Lout) {
#pragma unroll
            for (int m = 0; m < KD; ++m) Lout[(size_t)i * (KD + 1) + m] = li[m];
            Lout[(size_t)i * (KD + 1) + KD] = id;
        }
#pragma unroll
        for (int r = 0; r + 1 < KD; ++r) {
            dp[r] = dp[r + 1];
            ip[r] = ip[r + 1];
#pragma unroll
            for (int m = 0; m < KD; ++m) W[r][m] = W[r + 1][m];
        }
        dp[KD - 1] = d;
        ip[KD - 1] = id;
#pragma unroll
        for (int m = 0; m < KD; ++m) W[KD - 1][m] = li[m];
    }
    return neg;
}

// x <- A^-1 b with the stored factor (L unit lower, D): forward, diagonal, backward sweeps.
template <int KD>
__device__ void band_ldlt_solve(const double* __restrict__ L, int n, double* __restrict__ x) {
    double z[KD];
#pragma unroll
    for (int m = 0; m < KD; ++m) z[m] = 0.0;
    for (int i = 0; i < n; ++i) {                   // z_i = b_i - sum_m L(i, i-KD+m) z_{i-KD+m}
        double v = x[i];
#pragma unroll
        for (int m = 0; m < KD; ++m) v = fma(-L[(size_t)i * (KD + 1) + m], z[m], v);
#pragma unroll
        for (int m = 0; m + 1 < KD; ++m) z[m] = z[m + 1];
        z[KD - 1] = v;
        x[i] = v * L[(size_t)i * (KD + 1) + KD];      // y = D^-1 z
    }
    double w[KD];                                    // w[m] = x_{i+1+m}
#pragma unroll
    for (int m = 0; m < KD; ++m) w[m] = 0.0;
    for (int i = n - 1; i >= 0; --i) {              // x_i = y_i - sum_{j=i+1}^{i+KD} L(j, i) x_j
        double v = x[i];
#pragma unroll
        for (int m = 0; m < KD; ++m) {
            const int j = i + 1 + m;
            if (j < n) v = fma(-L[(size_t)j * (KD + 1) + (i - j + KD)], w[m], v);
        }
        x[i] = v;
#pragma unroll
        for (int m = KD - 1; m > 0; --m) w[m] = w[m - 1];
        w[0] = v;
    }
}

// y = S x (symmetric band)
template <int KD>
__device__ void band_sym_mul(const double* __restrict__ Sb, int n, const double* __restrict__ x,
                             double* __restrict__ y) {
    for (int i = 0; i < n; ++i) {
        double v = 0.0;
#pragma unroll
        for (int d = 0; d <= 2 * KD; ++d) {
            const int j = i + d - KD;
            if (j >= 0 && j < n) {
                // S(i, j) from the lower half and the diagonal: S(i, j) = S(j, i) for j > i
                const double s = d <= KD ? __ldg(Sb + (size_t)d * n + i) : __ldg(Sb + (size_t)(2 * KD - d) * n + j);
                v = fma(s, x[j], v);
            }
        }
        y[i] = v;
    }
}

template <int KD>
__global__ void __launch_bounds__(kBoundThreads) k_bound_count(const double* __restrict__ Hb,
                                                               const double* __restrict__ Sb, int n, int nrows,
                                                               double emax, int* __restrict__ counts) {
    const int l = blockIdx.x * blockDim.x + threadIdx.x;
    if (l >= nrows) return;
    counts[l] = band_ldlt<KD>(Hb + (size_t)l * (2 * KD + 1) * n, Sb, n, emax, nullptr);
}

// One thread per (row, index k): the k-th smallest eigenvalue by bisection on the inertia,
// below emax; lo found by doubling from min(-1, emax - |emax| - 1) until no eigenvalue lies
// below it.
template <int KD>
__global__ void __launch_bounds__(kBoundThreads) k_bound_bisect(const double* __restrict__ Hb,
                                                                const double* __restrict__ Sb, int n,
                                                                const int2* __restrict__ tasks, int ntasks,
                                                                double emax, double* __restrict__ energy) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntasks) return;
    const int l = tasks[t].x, k = tasks[t].y;
    const double* H = Hb + (size_t)l * (2 * KD + 1) * n;
    double lo = fmin(-1.0, emax - fabs(emax) - 1.0);
    for (int it = 0; it < 64 && band_ldlt<KD>(H, Sb, n, lo, nullptr) > 0; ++it) lo *= 2.0;
    double hi = emax;
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (!(mid > lo && mid < hi)) break;          // adjacent doubles: converged
        if (band_ldlt<KD>(H, Sb, n, mid, nullptr) > k) hi = mid;
        else lo = mid;
    }
    energy[t] = 0.5 * (lo + hi);
}

// Inverse iteration at the converged eigenvalue: x <- (H - E S)^-1 S x three times from a fixed
// pseudo-random start, then x / sqrt(x^T S x).  scratch: (KD+1) n doubles for the factor and
// n for S x, per task.
template <int KD>
__global__ void __launch_bounds__(kBoundThreads) k_bound_vector(const double* __restrict__ Hb,
                                                                const double* __restrict__ Sb, int n,
                                                                const int2* __restrict__ tasks, int ntasks,
                                                                const double* __restrict__ energy,
                                                                double* __restrict__ scratch,
                                                                double* __restrict__ vec) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntasks) return;
    const int l = tasks[t].x;
    const double* H = Hb + (size_t)l * (2 * KD + 1) * n;
    double* L = scratch + (size_t)t * (KD + 2) * n;
    double* sx = L + (size_t)(KD + 1) * n;
    double* x = vec + (size_t)t * n;
    band_ldlt<KD>(H, Sb, n, energy[t], L);
    for (int i = 0; i < n; ++i) {                    // start: hashed values in [0.5, 1.5)
        unsigned h = (unsigned)i * 2654435761u + 0x9e3779b9u * (unsigned)(t + 1);
        h ^= h >> 15;
        h *= 0x2c1b3c6du;
        h ^= h >> 12;
        x[i] = 0.5 + (double)(h >> 8) * (1.0 / 16777216.0);
    }
    for (int pass = 0; pass < 3; ++pass) {
        band_sym_mul<KD>(Sb, n, x, sx);
        for (int i = 0; i < n; ++i) x[i] = sx[i];
        band_ldlt_solve<KD>(L, n, x);
        double mx = 0.0;                              // rescale (the solve amplifies by 1/|E - E_k|)
        for (int i = 0; i < n; ++i) mx = fmax(mx, fabs(x[i]));
        const double s = mx > 0.0 ? 1.0 / mx : 0.0;
        for (int i = 0; i < n; ++i) x[i] *= s;
    }
    band_sym_mul<KD>(Sb, n, x, sx);
    double nrm = 0.0;
    for (int i = 0; i < n; ++i) nrm = fma(x[i], sx[i], nrm);
    const double s = nrm > 0.0 ? 1.0 / sqrt(nrm) : 0.0;
    for (int i = 0; i < n; ++i) x[i] *= s;
}

template <int KD>
cudaError_t bound_kd(const double* Hb, const double* Sb, int n, int nrows, double emax, int max_states,
                     int* counts_host, double* energies_host, double* vectors, cudaStream_t s, int* ntasks_out) {
    int* d_counts = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&d_counts, sizeof(int) * nrows, s);
    if (e != cudaSuccess) return e;
    count_launch();
    k_bound_count<KD><<<(nrows + kBoundThreads - 1) / kBoundThreads, kBoundThreads, 0, s>>>(Hb, Sb, n, nrows, emax,
                                                                                          d_counts);
    if ((e = cudaGetLastError()) == cudaSuccess)
        e = cudaMemcpyAsync(counts_host, d_counts, sizeof(int) * nrows, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFreeAsync(d_counts, s);
    if (e != cudaSuccess) return e;
    std::vector<int2> tasks;
    for (int l = 0; l < nrows; ++l) {
        const int c = counts_host[l] < max_states ? counts_host[l] : max_states;
        for (int k = 0; k < c; ++k) tasks.push_back(make_int2(l, k));
    }
    const int nt = (int)tasks.size();
    *ntasks_out = nt;
    for (int i = 0; i < nrows * max_states; ++i) energies_host[i] = 0.0;
    if (nt == 0) return cudaSuccess;
    int2* d_tasks = nullptr;
    double *d_energy = nullptr, *d_scratch = nullptr, *d_vec = nullptr;
    e = cudaMallocAsync((void**)&d_tasks, sizeof(int2) * nt, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_energy, sizeof(double) * nt, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_scratch, sizeof(double) * (size_t)nt * (KD + 2) * n, s);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&d_vec, sizeof(double) * (size_t)nt * n, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_tasks, tasks.data(), sizeof(int2) * nt, cudaMemcpyHostToDevice, s);
    const int blocks = (nt + kBoundThreads - 1) / kBoundThreads;
    if (e == cudaSuccess) {
        count_launch();
        k_bound_bisect<KD><<<blocks, kBoundThreads, 0, s>>>(Hb, Sb, n, d_tasks, nt, emax, d_energy);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        count_launch();
        k_bound_vector<KD><<<blocks, kBoundThreads, 0, s>>>(Hb, Sb, n, d_tasks, nt, d_energy, d_scratch, d_vec);
        e = cudaGetLastError();
    }
    // vectors: (row, index) slots of the caller's (nrows, max_states, n) array
    for (int t = 0; t < nt && e == cudaSuccess; ++t)
        e = cudaMemcpyAsync(vectors + ((size_t)tasks[t].x * max_states + tasks[t].y) * n, d_vec + (size_t)t * n,
                            sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
    std::vector<double> en(nt);
    if (e == cudaSuccess) e = cudaMemcpyAsync(en.data(), d_energy, sizeof(double) * nt, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    for (int t = 0; t < nt && e == cudaSuccess; ++t) energies_host[tasks[t].x * max_states + tasks[t].y] = en[t];
    cudaFreeAsync(d_tasks, s);
    cudaFreeAsync(d_energy, s);
    cudaFreeAsync(d_scratch, s);
    cudaFreeAsync(d_vec, s);
    return e;
}

}  // namespace

cudaError_t launch_bound_states(const double* Hb, const double* Sb, int n, int kd, int nrows, double emax,
                                int max_states, int* counts, double* energies, double* vectors, cudaStream_t s,
                                int* ntasks) {
    switch (kd) {
        case 1: return bound_kd<1>(Hb, Sb, n, nrows, emax, max_states, counts, energies, vectors, s, ntasks);
        case 2: return bound_kd<2>(Hb, Sb, n, nrows, emax, max_states, counts, energies, vectors, s, ntasks);
        case 3: return bound_kd<3>(Hb, Sb, n, nrows, emax, max_states, counts, energies, vectors, s, ntasks);
        case 4: return bound_kd<4>(Hb, Sb, n, nrows, emax, max_states, counts, energies, vectors, s, ntasks);
        case 5: return bound_kd<5>(Hb, Sb, n, nrows, emax, max_states, counts, energies, vectors, s, ntasks);
        case 6: return bound_kd<6>(Hb, Sb, n, nrows, emax, max_states, counts, energies, vectors, s, ntasks);
        case 7: return bound_kd<7>(Hb, Sb, n, nrows, emax, max_states, counts, energies, vectors, s, ntasks);
        case 8: return bound_kd<8>(Hb, Sb, n, nrows, emax, max_states, counts, energies, vectors, s, ntasks);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace gbprop
