// Internal declarations shared by the host runtime (gbprop_api.cpp) and the
// CUDA kernels (gbprop_kernels.cu).  Not part of the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace gbprop {

constexpr int kMaxBasis = 45;       // largest krylov_basis_size a handle accepts (7 m*m complex in smem)
constexpr int kWarp = 32;
constexpr int kSolveLanes = 32;     // radial blocks per l-row in the parallel solve
constexpr int kMaxKd = 8;           // largest band half-width of the overlap factor (order 9)

template <typename T> struct cx_of;
template <> struct cx_of<double> { using type = double2; };
template <> struct cx_of<float> { using type = float2; };
template <typename T> using cx = typename cx_of<T>::type;

// Tables of the parallel upper-band triangular solve U x = b in "e" coordinates
// (e = p for U^-1, e = n-1-p for U^-T), block-interleaved so that lane B of a
// warp reads entry (.., i, B) coalesced.  Built on the host in FP64.
//   n       radial length,  kd  superdiagonals,  L  block length,  P  blocks (<= 32)
//   ud      ((d-1)*L + i)*32 + B : U(e, e+d) / U(e, e), d = 1..kd, zero outside the block
//   invd    i*32 + B             : 1 / U(e, e), zero for e >= n
//   g       (c*L + i)*32 + B     : coupling of x_e to x_{(B+1)L + c} (within-block solve of
//                                  the block's upper-right corner), zero for the last block
//   mlev    ((lev*32 + B)*kd + r)*kd + c : suffix-scan operators of the kd-vector recurrence
//                                  t_B = y_B[0:kd] - F_B t_{B+1}, lev = 0..levels-1
template <typename T> struct SolveTab {
    int n, kd, L, P, levels, dir;
    const T* ud;
    const T* invd;
    const T* g;
    const T* mlev;
};

// Banded approximate inverse of one direction of the overlap-factor solve, in solve
// coordinates q (q = p for U x = b, q = n-1-p for U^T x = b), where both directions
// are upper triangular:  U~(q, q+d), d = 0..kd  and  M(q, q+j) ~ U~^-1(q, q+j), j = 0..w.
// U^-1 of a B-spline overlap factor decays geometrically away from the diagonal, so
// w is chosen (on the host) where the dropped part is below 2^-26 of the kept one.
//   m  (j*npad + q)  FP32, zero where q + j >= n;  npad = n rounded up to 4
//   u  (d*npad + q)  FP64, zero where q + d >= n
// Each CTA owns `chunk` radial elements (a multiple of 4) of one row and recomputes the
// halo its refinement passes need; stage = 1 copies the chunk's slice of m into shared memory
// with bulk asynchronous copies (16-byte aligned: q0, npad multiples of 4).
struct InvTab {
    int n, kd, w, npad;
    int chunk, nchunks;
    int refine;             // FP64-residual refinement passes of the FP64-accurate solve
    int stage;
    const float* m;
    const double* u;
    const float* uh;        // u split into FP32 pairs u = uh + ul (same layout), for the
    const float* ul;        // error-free residual of the complex64 solve
};

// Region of the CTA whose chunk starts at q0, for P refinement passes: cl elements written,
// x kept on [q0, q0 + R0), right-hand side read on [q0, q0 + RB).
__host__ __device__ inline void inv_region(int n, int q0, int chunk, int P, int w, int kd, int* cl, int* R0, int* RB) {
    const int left = n - q0;
    *cl = chunk < left ? chunk : left;
    const int r0 = *cl + P * (w + kd);
    *R0 = r0 < left ? r0 : left;
    const int rb = *R0 + w;
    *RB = rb < left ? rb : left;
}

// Shared-memory bytes of that CTA: b | x, r (FP64, refined solve only) | M slice (staged; read
// three times) | r32 | x0 (FP32 first iterate, refined solve only).  U~ is read once per
// residual pass and comes through L2.
__host__ __device__ inline size_t inv_smem_bytes(int n, int q0, int chunk, int P, int w, int kd, int stage, int r64) {
    int cl, R0, RB;
    inv_region(n, q0, chunk, P, w, kd, &cl, &R0, &RB);
    const int R0p = (R0 + 3) & ~3;
    size_t b = (size_t)RB * 16;
    if (r64) b += (size_t)R0 * 16 + (size_t)RB * 16;
    if (stage) b += (size_t)(w + 1) * R0p * 4;
    b += (size_t)(R0 + w + 2) * 8;                  // r32 with the padding of the paired M product
    if (r64) b += (size_t)R0 * 8;
    return b;
}

// Shared memory of the complex64 (mixed-path) solve with one refinement:
// M slice | uh, ul slices (staged) | b hi, b lo | x0 | r32.
__host__ __device__ inline size_t inv_smem_bytes_mixed(int n, int q0, int chunk, int w, int kd, int stage) {
    int cl, R0, RB;
    inv_region(n, q0, chunk, 1, w, kd, &cl, &R0, &RB);
    const int R0p = (R0 + 3) & ~3;
    size_t b = 0;
    if (stage) b += (size_t)(w + 1) * R0p * 4 + (size_t)2 * (kd + 1) * R0p * 4;
    b += (size_t)RB * 16 + (size_t)((R0 + 1) & ~1) * 8 + (size_t)(R0 + w + 2) * 8;
    return b;
}

// Term list of the tensor-potential matvec, grouped by destination row l:
//   y[l][i] += coef_t * s_t * sum_d slot[t][d][i] * x[src_t][i + d - kb]
// slots are real bands stored diagonal-major: (slot*(2kb+1) + d)*nr + i = A(i, i+d-kb).
template <typename T> struct BandOp {
    int nl, nr, kb, nterms;
    int variant;             // tile shape of the band kernel (chosen by the autotuner)
    const int* row_ptr;      // nl + 1
    const int* t_src;        // nterms
    const int* t_slot;       // nterms
    const int* t_timedep;    // nterms: 0 static, k >= 1 scaled by time function k
    const double* t_coef;    // 2 * nterms (re, im)
    const T* slots;
    const T* slots_lo;       // FP32 only: slot - (float)slot, the coefficients' rounding remainder
};

// Device control block of one handle.  Every field is written by kernels only, except
// inject_lu, wait_limit and round_matvec (set by the host through gbprop_debug_set).
struct Ctrl {
    int step;               // index of the current entry of the schedule array
    int broken;             // happy breakdown seen in the current step
    int nbasis;             // Krylov vectors built in the current step
    int scaling_order;      // s of the last scaling-and-squaring
    // error flags (sticky until the host reports them; kept adjacent: copied and cleared as one)
    int lu_info;            // last non-zero LU info of the Pade solve
    int nonfinite;          // a NaN/Inf norm was seen
    int wait_timeout;       // a bounded device-side wait (bulk-copy staging, grid barrier) gave up
    int inject_lu;          // test hook: the next exponentials report a zero pivot (host-set)
    long long wait_limit;   // polls of a launch's first bounded wait: 0 = default, < 0 = give up at once
    int round_matvec;       // precision probe (host-set): bit 0 band outputs, bit 1 solve and
                            // Gram-Schmidt outputs of FP64 handles rounded to complex64
    int ro_go;              // re-orthogonalisation requested for the current vector
    int ro_count;           // re-orthogonalisation passes done for the current vector
    long long operator_count;
    long long inner_product_count;
    long long orthogonalization_count;
    long long breakdown_count;
    long long step_count;
    double beta0;           // ||U psi|| at the start of the step
    double beta;            // current residual norm
    double inv_beta;        // 1 / beta (the reference scales by the reciprocal)
    float inv_beta_f[2];    // inv_beta as an FP32 pair (hi, lo) for the complex64 solve
    double orig_norm;       // ||w|| before Gram-Schmidt (re-orthogonalisation rule; updated per pass)
    double pre_norm;        // ||w|| of the operator output, before any Gram-Schmidt pass
    double resid_norm;      // ||w|| after Gram-Schmidt
    double err_est;         // |y[m-1]|^2
    double h[2 * kMaxBasis];
    double h3[2 * kMaxBasis];
    double y[2 * kMaxBasis];
};

// Up to this many distinct time functions per handle (the consolidated TensorPotentials of
// one problem, each scaled by its own f(t), TensorPotential.py:98-100).
constexpr int kMaxTimeFuncs = 4;

// Values of the time functions at one instant: s[k] scales the terms of time function k + 1.
struct Scalings {
    double s[kMaxTimeFuncs];
};

// Schedule entry per step: the time functions at the step start and the complex time step.
struct SchedEntry {
    Scalings scaling;
    double dt_re;
    double dt_im;
};

// Message returned by gbprop_last_error() on the calling thread.
void set_last_error(const char* msg);

// Launch counter shared by all launchers (process-wide).
void count_launch(int n = 1);
long long launch_count();

// ---- launchers (gbprop_kernels.cu) -------------------------------------------
// All return the cudaGetLastError() of their launch.
// Parallel banded triangular solve, one warp per l-row.
//   in_prec/out_prec/v_prec: 0 = complex128, 1 = complex64;  arith: 0 = double, 1 = float
//   scale_mode 1 multiplies the input by ctrl->inv_beta; vstore (if not null) receives the
//   scaled input; check_broken skips the launch body after a happy breakdown.
cudaError_t launch_solve(int arith, const void* tab, int nrows, const void* in, int in_prec,
                         void* out, int out_prec, void* vstore, int v_prec, const Ctrl* ctrl,
                         int scale_mode, int check_broken, cudaStream_t s);
// FP64-accurate solve: FP32 block solve + FP64 iterative refinement, one CTA per row.
// tabf: SolveTab<float> of the direction; udp: (kd+1) x nr diagonals U(i, i+d) in FP64.
cudaError_t launch_solve_ir(const void* tabf, const double* udp, int nrows, const void* in, int in_prec, void* out,
                            int out_prec, void* vstore, int v_prec, const Ctrl* ctrl, int scale_mode, int check_broken,
                            cudaStream_t s);
// Solve through the banded approximate inverse of the overlap factor (see InvTab):
// x = M b in FP32, then `refine` passes x += M (b - U~ x) with FP64 residuals when
// refine64 is set (FP64-accurate result).  refine64 = 0 is the complex64 solve of the mixed
// path's Krylov basis: one refinement whose residual is formed with error-free FP32 products
// and sums, complex64 output.  Grid: (tab.nchunks, nrows); arguments as launch_solve.
// v0s (complex64 solve of the FP64 first vector only, may be null) receives the scaled input
// split into FP32 pairs, float4 (re_hi, im_hi, re_lo, im_lo) per element.  bpart (scale_mode
// 1, may be null): the cooperative Gram-Schmidt kernel's bG per-CTA ||w||^2 partials (double,
// or float4 FP32 pairs for refine64 = 0); the solve forms beta from them, records it in ctrl
// (breakdown test, 1/beta) and scales by 1/beta, instead of reading ctrl->inv_beta.
cudaError_t launch_solve_inv(const InvTab& tab, int nrows, int refine64, const void* in, int in_prec, void* out,
                             int out_prec, void* vstore, int v_prec, Ctrl* ctrl, int dir, int scale_mode,
                             int check_broken, cudaStream_t s, float4* v0s = nullptr, const void* bpart = nullptr,
                             int bG = 0);
// sched (device, may be null): the time functions come from sched[ctrl->step]; else `scaling`.
cudaError_t launch_band_apply(int arith, const void* op, const void* x, void* y, const SchedEntry* sched,
                              const Ctrl* ctrl, const Scalings& scaling, int check_broken, cudaStream_t s);
cudaError_t launch_tbmv(int arith, int kd, const void* ud_phys, int nl, int nr, const void* in, int in_prec,
                        void* out, int out_prec, cudaStream_t s);
cudaError_t launch_norm(int prec, const void* x, long n, double* partials, unsigned* counter, Ctrl* ctrl,
                        cudaStream_t s);
// x <- x / ||x|| (FP64 state): a k_norm launch and a scaling launch.
cudaError_t launch_renormalize(double2* x, long n, double* partials, unsigned* counter, Ctrl* ctrl,
                               cudaStream_t s);
// v0 (complex64 basis only, may be null): FP64 copy of the first basis vector, used in
// place of V row 0 by the dot, the update and the combination.
// v0: the FP64 first vector of a complex64 basis; v0s: its FP32-pair split (hi, lo), read
// instead when given (written by the inverse-band solve of that vector)
cudaError_t launch_cgs_dot(int prec, const void* V, const double2* v0, const float4* v0s, long n, int nv,
                           const void* w, double* partials, unsigned* counter, Ctrl* ctrl, int mode, int want_norm,
                           cudaStream_t s);
// Stateless block inner product into a caller buffer (out: 2nv doubles, + ||w||^2 when want_norm).
size_t block_inner_scratch_doubles(long n, int nvals);
cudaError_t launch_block_inner(int prec, const void* V, long n, int nv, const void* w, int want_norm, double* out,
                               double* partials, unsigned* counter, cudaStream_t s);
// mode: bit 0 re-orthogonalisation pass, bit 1 double orthogonalisation requested, bit 2 the
// last block also finalizes Arnoldi step nv - 1 (H column, beta, breakdown; H, m, brk_tol as
// launch_arnoldi_finalize)
cudaError_t launch_cgs_update(int prec, const void* V, const double2* v0, const float4* v0s, long n, int nv, void* w,
                              double* partials, unsigned* counter, Ctrl* ctrl, int mode, cudaStream_t s,
                              double* H = nullptr, int m = 0, double brk_tol = 0.0);
// brk_tol: happy-breakdown threshold on the new basis norm (pAMP: sqrt(eps), pamp.h:79;
// Expokit: 1e-7).
cudaError_t launch_arnoldi_finalize(Ctrl* ctrl, double* H, int m, int J, int double_orth, double brk_tol,
                                    cudaStream_t s);
// One Arnoldi step's Gram-Schmidt (dot, update, norm, Hessenberg column, breakdown) as a
// single cooperative kernel of `grid` co-resident CTAs (gbprop_cgs.cu).  part: at least
// arnoldi_cgs_part_doubles(grid) doubles; bar: two words, zero before the first launch.
// update = 0 forms only the Hessenberg column (last vector).  cache: keep V's chunk in
// shared memory between the two passes.
// The complex64 form takes the first vector as FP32 pairs (v0s, see launch_solve_inv) and
// forms every sum with error-free FP32 transformations.
cudaError_t launch_arnoldi_cgs(int prec, const void* V, const void* v0, long n, int J, int m, void* w,
                               double* part, unsigned* bar, Ctrl* ctrl, double* H, int update, int grid, int cache,
                               cudaStream_t s);
// Grid size for the cooperative Gram-Schmidt (0 if it cannot run co-resident).
int arnoldi_cgs_grid(int prec, long n, int m, int with_v0, int cache);
int arnoldi_cgs_grid_batch(int prec, long n, int m, int with_v0, int* cache);
inline size_t arnoldi_cgs_part_doubles(int grid) { return (size_t)(2 * (kMaxBasis + 1) + 1) * grid; }
cudaError_t launch_step_begin(Ctrl* ctrl, double* H, int m, cudaStream_t s);
// max_cluster: 16 lets one problem's exponential spread over a thread-block cluster; 1 keeps it on
// one CTA (batches, where other problems fill the GPU).
// df32 = 1 (FP32-mixed handles): the cluster form in double-float arithmetic (gbprop_expm.cu).
cudaError_t launch_expm(Ctrl* ctrl, double* H, int m, const SchedEntry* sched, int max_cluster, cudaStream_t s,
                        int df32 = 0);
// krylov_exponentiation_method = 1 (pamp.h:567-607): y from the eigen-decomposition, one CTA.
cudaError_t launch_expm_eig(Ctrl* ctrl, double* H, int m, const SchedEntry* sched, cudaStream_t s);
// cluster: 16 or 8 CTAs, or 1 (one CTA, for batches; when expm_df_single_fits(m))
cudaError_t launch_expm_df(Ctrl* ctrl, double* H, int m, const SchedEntry* sched, int cluster, cudaStream_t s);
bool expm_df_single_fits(int m);
cudaError_t launch_combine(int prec, const void* V, const double2* v0, long n, const Ctrl* ctrl, void* out,
                           cudaStream_t s);
cudaError_t launch_step_end(Ctrl* ctrl, cudaStream_t s);
// out[0..2] = max of the members' (lu_info, nonfinite, wait_timeout); out[3] = 1 + the first
// member with any of them set (0 if none).  One CTA.
cudaError_t launch_gather_flags(Ctrl* const* ctrls, int count, int* out, cudaStream_t s);
cudaError_t launch_tensor_multiply_ref(int storage, const double2* V, int npairs, const int* pairs, int kb,
                                       double scaling, const double2* src, double2* dst, int nl, int nr,
                                       cudaStream_t s);
cudaError_t launch_zero(void* p, size_t bytes, cudaStream_t s);

int grid_reduce_blocks();
int band_variant_count();
bool band_variant_vec_ok(int v, int nr);    // the variant's radial-size condition (even nr for 6, 7, 8)
// Bound states of banded generalized symmetric problems (gbprop_bound.cu; see gbprop_bound_states)
cudaError_t launch_bound_states(const double* Hb, const double* Sb, int n, int kd, int nrows, double emax,
                                int max_states, int* counts, double* energies, double* vectors, cudaStream_t s,
                                int* ntasks);
size_t partials_capacity();

}  // namespace gbprop
