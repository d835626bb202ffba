/*
 * gbprop.h -- C ABI of libgbprop, the GB300 (sm_103a) implementation of
 * pyprop's pAMP x TensorPotential propagation step.
 *
 * Plain C types only: device pointers are `void*`, complex numbers are
 * interleaved (re, im) pairs of double (complex128) or float (complex64),
 * streams are passed as `void*` (a cudaStream_t; NULL = legacy default stream).
 * Every call returns a gbprop_status; gbprop_last_error() gives the message of
 * the most recent failure on the calling thread.
 *
 * Layout conventions (the reference's own):
 *   wavefunction   psi[l][r], C order, radial index fastest, nl*nr complex
 *                  (Wavefunction<2> data, core/wavefunction.h:11-116)
 *   band storage   BLAS general band, element (i,j) at j*(2kb+1) + kb + i - j
 *                  (GeometryInfoCommonBandedNonHermitian, pyprop/tensorpotential/GeometryInfo.py:407-459)
 *   overlap factor upper band, element U(i,j) at j*(kd+1) + kd + i - j
 *                  (OverlapMatrix::OverlapCholeskyUpper, core/representation/overlapmatrix.cpp:22-37)
 *   angular pairs  int32 (row, col) per stored potential slot
 *                  (GeometryInfoReducedSphHarmSelectionRule.GetBasisPairs,
 *                   pyprop/tensorpotential/basis/ReducedSphericalHarmonic.py:22-37)
 */
#ifndef GBPROP_H
#define GBPROP_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GBPROP_OK = 0,
    GBPROP_EINVAL = 1,       /* bad argument (sizes, null pointers, state) */
    GBPROP_ECUDA = 2,        /* a CUDA runtime call failed */
    GBPROP_EBREAKDOWN = 3,   /* informational: happy breakdown happened in the last step */
    GBPROP_ENONFINITE = 4,   /* NaN/Inf seen in the Krylov norms */
    GBPROP_ETIMEOUT = 5,     /* a bounded device-side wait gave up */
    GBPROP_ELU = 6,          /* the Pade denominator was singular (pamp.h:544-550) */
    GBPROP_EUNSUPPORTED = 7  /* storage/precision combination not provided */
} gbprop_status;

typedef enum {
    GBPROP_FP64 = 0,         /* complex128 everywhere (the drop-in) */
    GBPROP_FP32_MIXED = 1    /* complex64 basis + matvec, FP64 reductions/expm/state update */
} gbprop_precision;

typedef enum {
    GBPROP_STORAGE_DIAG = 0, /* angular "Diag": one band per l, row = col = l */
    GBPROP_STORAGE_IDENT = 1,/* angular "Ident": one band for every l */
    GBPROP_STORAGE_SIMP = 2  /* angular "Simp": one band per (row, col) pair */
} gbprop_storage;

typedef struct gbprop_ctx* gbprop_handle;

/* Counters as pAMP keeps them (pamp.h:121-124, PampWrapper::GetOperatorCount ...). */
typedef struct {
    long long operator_count;
    long long inner_product_count;
    long long orthogonalization_count;
    long long breakdown_count;
    long long step_count;
    int last_basis_size;      /* Krylov vectors built in the last step */
    int last_scaling_order;   /* s of the last scaling-and-squaring */
    double error_estimate;    /* |y[m-1]|^2 of the last step (pamp.h:207-210,666) */
} gbprop_stats;

/* Library / device ---------------------------------------------------------- */
const char* gbprop_version(void);
const char* gbprop_last_error(void);
/* Number of kernel launches made by this process since load (all handles). */
long long gbprop_launch_count(void);

/* Propagator handle: replaces core.krylov_PampWrapper_<Rank> (Boost.Python,
 * core/krylov/pamp/pampwrapper.h:15-123) + the TensorPotential list of
 * BasisPropagator (pyprop/tensorpotential/BasisPropagator.py:41-108).
 *   krylov_basis_size       config key krylov_basis_size (pampwrapper.cpp:53)
 *   exponentiation_method   krylov_exponentiation_method (pampwrapper.cpp:56-61): 0 = Pade
 *                           scaling-and-squaring (pamp.h:430-564), 1 = eigenvector exponential
 *                           (pamp.h:567-607)
 *   double_orthogonalization krylov_double_orthogonalization (pampwrapper.cpp:64-69)
 * stream: the CUDA stream every call of this handle is ordered on. */
gbprop_status gbprop_create(gbprop_handle* out, int nl, int nr, int precision,
                            int krylov_basis_size, int exponentiation_method,
                            int double_orthogonalization, void* stream);
gbprop_status gbprop_destroy(gbprop_handle h);

/* Overlap Cholesky factor U (S = U^T U) of the radial rank, HOST pointer,
 * upper band storage (nr, kd+1) of real values (OverlapCholeskyUpper is real
 * for a real B-spline basis). Replaces OverlapMatrix::Setup (overlapmatrix.cpp:9-37). */
gbprop_status gbprop_set_overlap(gbprop_handle h, int kd, const double* U_band);

/* Add one consolidated TensorPotential (TensorPotential.py:33-87) in the
 * reference storage, HOST pointers:
 *   storage        gbprop_storage of the angular rank; the radial rank is BandNH
 *   npairs         number of stored angular slots (nl for Diag, 1 for Ident)
 *   pairs          (npairs, 2) int32 (row, col); NULL for Diag/Ident
 *   kb             band half-width of the radial BandNH storage (order - 1)
 *   data           (npairs, (2kb+1)*nr) complex128 interleaved (PotentialData)
 *   time_dependent 0: static; k = 1..4: scaled by time function number k.  Every
 *                  potential is scaled by its own time function f_k(t)
 *                  (TensorPotential.py:98-100, looped in Propagator.py:61-66); potentials
 *                  sharing one function share its number.  The handle's time-function
 *                  count K is the largest number used (1 if none).
 * dest[row] += f_k(t) * data[pair] * src[col]   (generator.py:352). */
gbprop_status gbprop_add_potential(gbprop_handle h, int storage, int npairs, const int* pairs,
                                   int kb, const double* data, int time_dependent);

/* Build device tables (solve coupling tables, band slots); call once after the
 * overlap and all potentials are set.  Replaces PamPropagator.SetupStep /
 * PampWrapper::Setup (PamPropagator.py:29-45, pampwrapper.cpp:74-81). */
gbprop_status gbprop_finalize(gbprop_handle h);

/* PamPropagator.AdvanceStep (PamPropagator.py:50-57) + PampWrapper::AdvanceStep
 * (pampwrapper.cpp:84-108) for nsteps consecutive steps, on a DEVICE
 * wavefunction psi (complex128 for FP64, complex64 for FP32_MIXED), in place:
 *   psi <- U^-1 pAMP_m(U psi, dt; H(t_n))   for n = 0..nsteps-1
 * scalings (HOST array, nsteps x K, step-major) holds the K time functions at the
 * start of each step: scalings[n*K + k-1] = f_k(t_n) (TensorPotential.py:98-100 with
 * t = PropagatedTime; K = 1 for the reference's single-pulse configurations, where
 * this is one value per step).  dt may be complex (imaginary time).  Asynchronous
 * on the handle's stream.
 *
 * Failures on the device (the reference throws at once, pamp.h:544-550) are
 * returned as GBPROP_ELU (singular Pade denominator), GBPROP_ENONFINITE (NaN/Inf
 * norm or Hessenberg entry) or GBPROP_ETIMEOUT (a bounded device-side wait gave
 * up) by the first call on the handle after the GPU has finished the failing
 * step: a later gbprop_advance (without waiting), or at the latest
 * gbprop_synchronize, gbprop_advance_host or gbprop_get_stats (which wait).  A
 * reported failure is cleared, so the handle stays usable. */
gbprop_status gbprop_advance(gbprop_handle h, void* psi, int nsteps, const double* scalings,
                             double dt_re, double dt_im);

/* Same as gbprop_advance on a HOST wavefunction: copies psi to the device,
 * advances, copies it back and synchronises the stream. */
gbprop_status gbprop_advance_host(gbprop_handle h, void* psi_host, int nsteps, const double* scalings,
                                  double dt_re, double dt_im);

/* BasisPropagator.MultiplyHamiltonianBalancedOverlap (BasisPropagator.py:131-159)
 * when balanced != 0: dst = U^-H H(t) U^-1 src; otherwise
 * MultiplyHamiltonianNoOverlap (:126-129): dst = H(t) src.  DEVICE pointers of
 * the handle's precision; src is not modified.  gbprop_matvec scales every
 * time-dependent potential by `scaling`; gbprop_matvec_scalings takes the K time
 * functions' values (HOST array of K doubles). */
gbprop_status gbprop_matvec(gbprop_handle h, const void* src, void* dst, double scaling, int balanced);
gbprop_status gbprop_matvec_scalings(gbprop_handle h, const void* src, void* dst, const double* scalings,
                                     int balanced);

/* Problem.AdvanceStep's renormalization (Problem.py:167-168: psi.Normalize() after every
 * step when the Propagation key renormalization is true; Wavefunction::Normalize,
 * core/wavefunction.cpp:194-218): on != 0 makes every step of gbprop_advance and
 * gbprop_expokit_advance end with psi <- psi / ||psi||_S, on the device. */
gbprop_status gbprop_set_renormalization(gbprop_handle h, int on);

/* Wavefunction::InnerProduct (core/wavefunction.cpp:207-218 -> CombinedRepresentation::
 * InnerProduct, combinedrepresentation.cpp:423-474): out[0], out[1] = Re, Im of a^H (I x S) b
 * for DEVICE wavefunctions a, b of the handle's precision, with S = U^T U the radial overlap
 * (formed as (U a)^H (U b) in FP64).  Synchronous; the norm is sqrt(out[0]) for b = a. */
gbprop_status gbprop_inner_product(gbprop_handle h, const void* a, const void* b, double* out);

/* CombinedRepresentation::MultiplySqrtOverlap(false) / SolveSqrtOverlap(conj)
 * (combinedrepresentation.cpp:207-238), in place on a DEVICE wavefunction. */
gbprop_status gbprop_multiply_sqrt_overlap(gbprop_handle h, void* psi);
gbprop_status gbprop_solve_sqrt_overlap(gbprop_handle h, int conj, void* psi);

gbprop_status gbprop_get_stats(gbprop_handle h, gbprop_stats* out);
gbprop_status gbprop_reset_stats(gbprop_handle h);
/* Copy the last step's (scaled, -i*dt*H) Hessenberg matrix, m*m complex128
 * row-major, to HOST memory (pAMP::GetHessenbergMatrix, pamp.h:197-200). */
gbprop_status gbprop_get_hessenberg(gbprop_handle h, double* out);
/* Waits for the handle's work; returns a device-side failure of it (see gbprop_advance). */
gbprop_status gbprop_synchronize(gbprop_handle h);

/* Per-phase times of one propagation step: the pAMP timers ("Operator", "InnerProduct",
 * "PadeExponential", pamp.h:149-151, printed by PrintStatistics, :671-687), split by kernel
 * phase.  gbprop_time_step runs one step (psi <- U^-1 pAMP(U psi)) on a DEVICE wavefunction
 * outside the step's CUDA graph, with an event after every launch, waits for it and fills
 * `out`: ms[p] and count[p] are the time and the launches of phase p (the time between the
 * event before a launch and the one after it), total_ms their sum, launches all kernel
 * launches.  Slower than gbprop_advance (no graph); the same arithmetic. */
typedef enum {
    GBPROP_PHASE_SOLVE = 0,         /* overlap-factor solves (U^-1, U^-T; state transform) */
    GBPROP_PHASE_BAND = 1,          /* TensorPotential band matvec */
    GBPROP_PHASE_GRAM_SCHMIDT = 2,  /* inner products, update, norms, Hessenberg column */
    GBPROP_PHASE_EXPONENTIAL = 3,   /* Pade scaling-and-squaring of the Hessenberg matrix */
    GBPROP_PHASE_COMBINE = 4,       /* psi = beta0 V exp(-i dt H) e1 */
    GBPROP_PHASE_OTHER = 5,         /* U psi, step bookkeeping */
    GBPROP_PHASE_COUNT = 6
} gbprop_phase;
typedef struct {
    double ms[GBPROP_PHASE_COUNT];
    int count[GBPROP_PHASE_COUNT];
    double total_ms;
    long long launches;
} gbprop_step_timers;
gbprop_status gbprop_time_step(gbprop_handle h, void* psi, const double* scalings, double dt_re, double dt_im,
                               gbprop_step_timers* out);

/* Test hooks for the failure paths, no counterpart in the reference (its failures are
 * CPU exceptions).  Neither faults nor hangs the GPU; both stay set until changed.
 *   GBPROP_DEBUG_WAIT_LIMIT  value = polls of the first bounded wait of each launch (the
 *                            bulk-copy staging wait, the cooperative grid barrier); 0 restores
 *                            the default, a negative value makes those waits give up at once
 *                            (the launch records the timeout and returns: GBPROP_ETIMEOUT)
 *   GBPROP_DEBUG_INJECT_LU   value != 0: every Pade solve reports a zero pivot, as zgetrf's
 *                            info != 0 in pamp.h:544-550 (GBPROP_ELU); 0 clears it
 *   GBPROP_DEBUG_ROUND_MATVEC precision probe of FP64 handles, bits of value: 1 = the band
 *                            matvec's outputs are rounded to complex64; 2 = the outputs of the
 *                            Arnoldi loop's solves and of the Gram-Schmidt update are too.  1
 *                            measures what complex64 matvec outputs alone cost a propagation, 3
 *                            what complex64 storage of every Arnoldi vector costs (the FP32-mixed
 *                            path's storage, with FP64 arithmetic); 0 clears it
 * Synchronises the handle's stream. */
typedef enum {
    GBPROP_DEBUG_WAIT_LIMIT = 0,
    GBPROP_DEBUG_INJECT_LU = 1,
    GBPROP_DEBUG_ROUND_MATVEC = 2
} gbprop_debug_key;
gbprop_status gbprop_debug_set(gbprop_handle h, int key, long long value);

/* Precision probe of the Hessenberg exponentials, no counterpart in the reference: runs one
 * exponential of the handle on a HOST Hessenberg matrix H (m x m complex128 row-major, unscaled,
 * m = krylov_basis_size) at time step dt and returns y = exp(-i dt H) e1 (HOST, 2m doubles) and the
 * scaling order.  form: 0 = the FP64 Pade kernel, 1 = the double-float Pade kernel of the
 * FP32-mixed path, 2 = the eigenvector exponential.  Synchronous; overwrites the handle's
 * Hessenberg buffer (as a step does). */
gbprop_status gbprop_debug_expm(gbprop_handle h, const double* H, double dt_re, double dt_im, int form, double* y,
                                int* scaling_order);

/* Statistics of one gbprop_expokit_advance call (Expokit's zgexpv diagnostics). */
typedef struct {
    long long substeps;      /* accepted Krylov sub-steps */
    long long rejections;    /* rejected sub-step sizes */
    long long matvecs;       /* operator applications */
    double error;            /* sum of the local error estimates */
    double hump;             /* max ||w|| over the sub-steps / ||w_0|| (conditioning measure) */
    double last_step;        /* last accepted sub-step size */
} gbprop_expokit_stats;

/* ExpokitPropagator.AdvanceStep (pyprop/propagator/KrylovPropagator.py:44-49 ->
 * core/krylov/expokit/expokitpropagator.cpp:36-103 -> Expokit zgexpv): nsteps steps of size
 * |dt|, each psi <- U^-1 exp(-i |dt| A) U psi (imaginary dt: exp(-|dt| A)), A the balanced
 * operator at the time functions of step k (scalings as in gbprop_advance, fixed within the
 * step, as the reference's callback fixes the step's start time), evaluated by Krylov
 * sub-steps with local error control.  The Krylov dimension
 * is the handle's krylov_basis_size - 1 (a handle for Expokit holds m + 1 vectors); tol and
 * anorm are krylov_tolerance and krylov_norm.  stats may be NULL.  Host-driven (the sub-step
 * sizes depend on the error estimates); returns after the work is enqueued and the last
 * sub-step decision is taken. */
gbprop_status gbprop_expokit_advance(gbprop_handle h, void* psi, int nsteps, const double* scalings,
                                     double dt_re, double dt_im, double tol, double anorm,
                                     gbprop_expokit_stats* stats);

/* Band-kernel tile autotuner: times every tile shape of the TensorPotential matvec
 * kernel on this handle's operator and keeps the fastest; *variant (if not NULL)
 * receives its index.  Synchronises the handle's stream.  If *variant >= 0 on entry,
 * that shape is selected without timing (GBPROP_EINVAL if it does not exist, or if it
 * does not apply: shapes 6, 7 and 8 form two radial elements per thread and need an even
 * radial size).  No counterpart in the reference (its generated kernels have one shape). */
gbprop_status gbprop_autotune(gbprop_handle h, int* variant);

/* Field-free bound states: for every angular row l the eigenpairs with E < emax of the
 * generalized symmetric banded problem H_l c = E S c (the static angular-diagonal operator of
 * row l in the B-spline overlap metric) -- the analysis of the reference's hydrogen example
 * (examples/tensor/helium_stabilization_sae/analysis.py:92-160, a dense generalized
 * eigensolver per l there).  Here: inertia counts of banded LDL^T factorisations of
 * H - sigma S, bisection to the double-precision eigenvalue (one GPU thread per state) and
 * inverse iteration for the vector, normalised in the S metric (sign arbitrary).
 *   h_bands  DEVICE, nrows x (2kd+1) x nr doubles: h_bands[(l (2kd+1) + d) nr + i] = H_l(i, i+d-kd)
 *            (symmetric; the lower half and the diagonal are read)
 *   s_band   DEVICE, (2kd+1) x nr doubles, S(i, i+d-kd), positive definite
 *   counts   HOST out, nrows: the number of eigenvalues below emax of each row (states beyond
 *            max_states are not computed)
 *   energies HOST out, nrows x max_states (unused slots 0)
 *   vectors  DEVICE out, nrows x max_states x nr (slot (l, k) for k < min(counts[l], max_states))
 * Synchronises `stream`.  No counterpart in the reference. */
gbprop_status gbprop_bound_states(int nr, int kd, int nrows, const double* h_bands, const double* s_band, double emax,
                                  int max_states, int* counts, double* energies, double* vectors, void* stream);

/* The choices gbprop_autotune made (or that were pinned): the band kernel's tile variant and
 * the radial chunk counts of the two overlap-factor solve directions (U^-1, U^-T; 0 = the
 * block solver).  The environment GBPROP_BAND_VARIANT=v and GBPROP_SOLVE_CHUNKS=n0,n1 make
 * gbprop_autotune use those instead of timing them (a profiler run reproduces a live run's
 * configuration).  No counterpart in the reference. */
gbprop_status gbprop_get_tuning(gbprop_handle h, int* band_variant, int* solve_chunks);

/* Batches of independent problems (each a finalized handle, all of one precision,
 * each with its own operator, sizes, Krylov size, time function and time step),
 * advanced together: one step of the batch is a single CUDA graph launch whose
 * branches are the problems' step sequences.  The handles must outlive the batch.
 * autotune != 0 runs gbprop_autotune on every member first. */
typedef struct gbprop_batch_ctx* gbprop_batch;
gbprop_status gbprop_batch_create(gbprop_batch* out, const gbprop_handle* problems, int count, int autotune,
                                  void* stream);
/* psi[p]: DEVICE wavefunction of problem p; scalings: HOST array of the problems'
 * blocks one after another, problem p's block nsteps x K_p as in gbprop_advance
 * (K_p = 1 for every problem: a count x nsteps array, row p = problem p's time
 * function at the start of each step); dt: count x 2 HOST array (re, im of each
 * problem's time step). */
gbprop_status gbprop_batch_advance(gbprop_batch b, void* const* psi, int nsteps, const double* scalings,
                                   const double* dt);
/* Waits for the batch's work; returns a device-side failure of any member (see
 * gbprop_advance; gbprop_batch_advance also returns one once it is known, without waiting). */
gbprop_status gbprop_batch_synchronize(gbprop_batch b);
gbprop_status gbprop_batch_destroy(gbprop_batch b);

/* Stateless kernel ABI: TensorPotentialMultiply_<S0>_BandNH
 * (generator.py:1373-1426 Fortran entry, :1486-1495 C++ wrapper,
 *  TensorPotential.py:106-112 Python call), complex128 DEVICE buffers:
 *   dst[row, :] += scaling * V[pair] (band) src[col, :]
 * storage: GBPROP_STORAGE_DIAG (V is (nl, (2kb+1)*nr), pairs ignored) or
 * GBPROP_STORAGE_SIMP (V is (npairs, (2kb+1)*nr), pairs (npairs, 2) int32 DEVICE). */
gbprop_status gbprop_tensor_multiply_bandnh(int storage, const void* V, int npairs, const int* pairs,
                                            int kb, double scaling, const void* src, void* dst,
                                            int nl, int nr, void* stream);

/* Stateless block inner product of the Arnoldi step: BLASIntegrationFunctor::InnerProduct
 * (core/krylov/piram/piram/functors.h:236-240, zgemv 'C' over the first nv Krylov vectors):
 *   out[2k], out[2k+1] = Re, Im of sum_i conj(V[k][i]) * w[i],  k < nv
 * and, when want_norm != 0, out[2nv] = sum_i |w[i]|^2.  V is nv rows of n elements
 * (row stride n), all DEVICE pointers of the given precision (GBPROP_FP64: complex128,
 * GBPROP_FP32_MIXED: complex64; sums are accumulated in FP64 either way).  workspace is
 * caller-owned DEVICE scratch of at least gbprop_block_inner_product_workspace(n, nv)
 * bytes -- the role of the reference's `temp` argument.  Deterministic summation order. */
size_t gbprop_block_inner_product_workspace(long n, int nv);
gbprop_status gbprop_block_inner_product(int precision, const void* V, long n, int nv, const void* w, int want_norm,
                                         double* out, void* workspace, size_t workspace_bytes, void* stream);

/* Allocation-free variant of gbprop_block_inner_product, for callers that cannot
 * allocate device memory when they need it: memory pools or custom allocators that
 * call back into this library (allocating there would re-enter the allocator), and
 * hosts that hand over only fixed buffers and allow no allocation after start-up.  No
 * counterpart in the reference (its temp vector is always caller-allocated).
 * Same arguments and results as gbprop_block_inner_product minus the workspace:
 * the reduction scratch is one fixed array of 1024 doubles + a counter word in
 * the library's device memory (on every GPU that loads the library, held until
 * exit).  Calls no cudaMalloc/cudaFree.  Limits: 1 <= nv <= 45, any n > 0; larger
 * requests are rejected with GBPROP_EINVAL.  The first call on each device looks
 * up the array's device address (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture.  Every call shares the one
 * array: calls that overlap on the GPU (different streams, or different host
 * threads on one device) race and must be serialised by the caller. */
gbprop_status gbprop_block_inner_product_noalloc(int precision, const void* V, long n, int nv, const void* w,
                                                 int want_norm, double* out, void* stream);

/* Radial TensorPotential set-up on the GPU (TensorPotentialGenerator's B-spline projection,
 * pyprop/tensorpotential/TensorPotentialGenerator.py:72-256 -> RepresentPotentialInBasisBSpline,
 * core/tensorpotential/basis_bspline.h:10-48 -> BSpline::BSplineGlobalOverlapIntegral,
 * core/transform/bspline/bspline.cpp:373-467; overlap Cholesky, overlapmatrix.cpp:9-104).
 * For a B-spline basis of `order` on `knots` (nknots values; n = nknots - order splines), with the
 * Gauss-Legendre rule (nodes, weights on [-1, 1], nquad points) on every interval of
 * `breakpoints`, forms nmat band matrices M_m(i, j) = <B_i| f_m |d^deriv[m] B_j>, f_m(r) = coef[m]
 * (fid 0), coef[m]/r (fid 1) or coef[m]/(2 r^2) (fid 2), with the reference's swap rule
 * M(j, i) = (-1)^deriv M(i, j).  bands (HOST, nmat x (2 order - 1) x n): diagonal-major,
 * bands[m][order - 1 + d][i] = M_m(i, i + d).  cholesky (HOST, order x n, or NULL): the upper
 * Cholesky factor of matrix 0 (the overlap), cholesky[d][i] = U(i, i + d).  All HOST pointers;
 * synchronous on `stream`; allocates its own device scratch. */
gbprop_status gbprop_bspline_bands(int order, int nknots, const double* knots, int nbreak, const double* breakpoints,
                                   int nquad, const double* nodes, const double* weights, int nmat, const int* fid,
                                   const int* deriv, const double* coef, double* bands, double* cholesky,
                                   void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GBPROP_H */
