/*
 * oracle.c -- CPU restatement of pyprop's pAMP x TensorPotential propagation step.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (pyprop_gb300/, libgbprop)
 * links, loads or calls this file.  It is the oracle the GPU kernels are
 * compared against (tests/, __graft_entry__.smoke) and the timed CPU baseline
 * of bench.py.  Everything is complex128 arithmetic written out in real and
 * imaginary parts, in the reference's own order of operations where that
 * order is visible in the reference source:
 *
 *   pAMP::PropagateVector            core/krylov/pamp/pamp/pamp.h:613-669
 *   pAMP::PerformInitialArnoldiStep  pamp.h:271-290
 *   pAMP::PerformArnoldiStep         pamp.h:293-350   (classical Gram-Schmidt)
 *   pAMP::PerformOrthogonalization   pamp.h:353-400   (0.717 rule, <=3 passes)
 *   pAMP::ScalingPadeExponential     pamp.h:430-467
 *   pAMP::PadeExponential            pamp.h:470-564   (Horner in A^2, I+2 Q^-1 P)
 *   BLASIntegrationFunctor           core/krylov/piram/piram/functors.h:182-241
 *   PamPropagator.AdvanceStep        pyprop/propagator/PamPropagator.py:50-57
 *   MultiplyHamiltonianBalancedOverlap
 *                                    pyprop/tensorpotential/BasisPropagator.py:131-159
 *   OverlapMatrix::{Multiply,Solve}SqrtOverlapVector
 *                                    core/representation/overlapmatrix.cpp:137-150
 *   OverlapMatrix::Setup (zpbtrf)    overlapmatrix.cpp:9-37
 *   TensorPotentialMultiply_Diag_BandNH / _Simp_BandNH
 *                                    core/tensorpotential/tensorpotentialmultiply_generator.py:302-363,403-432,622-735
 *   Problem.AdvanceStep time update  pyprop/Problem.py:158-173
 *
 * The BLAS/LAPACK routines the reference calls (zgbmv, ztbmv, ztbsv, zpbtrf,
 * zdotc, zgemv, zaxpy, zscal, zgemm, zgetrf, zgetrs) are restated from their
 * published definitions (netlib reference BLAS/LAPACK semantics).
 *
 * Parity status: the reference cannot be built or run in this environment
 * (Python 2 + Boost.Python + gfortran + MPI + MKL).  This restatement is pinned
 * by the reference's own known-answer check (PampWrapper::TestPade,
 * core/krylov/pamp/pampwrapper.h:195-217) against scipy.linalg.expm, by the
 * storage-consistency checks the reference's examples print (banded vs dense,
 * examples/tensor/reducedspherical/example.py:301-332,567-620), by dense
 * numpy/scipy propagation of small cases, and by the reference's own Python
 * setup modules (Gauss-Legendre rule, breakpoint and knot sequences) run here
 * to produce golden fixtures.  No stored golden vector of the propagation
 * itself exists in the reference.
 */
#include <math.h>
#include <float.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double re, im; } cplx;

static inline cplx cmul(cplx a, cplx b) { cplx r = { a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re }; return r; }
static inline cplx cconjmul(cplx a, cplx b) { /* conj(a) * b */ cplx r = { a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re }; return r; }
static inline cplx cadd(cplx a, cplx b) { cplx r = { a.re + b.re, a.im + b.im }; return r; }
static inline cplx csub(cplx a, cplx b) { cplx r = { a.re - b.re, a.im - b.im }; return r; }
static inline cplx cdiv(cplx a, cplx b) {
    /* Smith's algorithm, as netlib's zladiv family does it */
    cplx r;
    if (fabs(b.re) >= fabs(b.im)) {
        double q = b.im / b.re, d = b.re + b.im * q;
        r.re = (a.re + a.im * q) / d; r.im = (a.im - a.re * q) / d;
    } else {
        double q = b.re / b.im, d = b.im + b.re * q;
        r.re = (a.re * q + a.im) / d; r.im = (a.im * q - a.re) / d;
    }
    return r;
}
static inline double cabs1(cplx a) { return fabs(a.re) + fabs(a.im); }

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* BLAS level-1 restatements (functors.h:214-240, pamp.h:281-315)            */
/* ------------------------------------------------------------------------ */

/* zdotc: sum conj(x) * y */
static cplx zdotc(long n, const cplx* x, const cplx* y) {
    double sr = 0.0, si = 0.0;
#pragma omp parallel for reduction(+:sr,si) schedule(static) if (n > 16384)
    for (long i = 0; i < n; i++) {
        sr += x[i].re * y[i].re + x[i].im * y[i].im;
        si += x[i].re * y[i].im - x[i].im * y[i].re;
    }
    cplx r = { sr, si };
    return r;
}

/* BLASIntegrationFunctor::Norm = sqrt(Re <v,v>)  (functors.h:214-217) */
static double global_norm(long n, const cplx* x) { return sqrt(zdotc(n, x, x).re); }

static void zscal(long n, cplx a, cplx* x) {
#pragma omp parallel for schedule(static) if (n > 16384)
    for (long i = 0; i < n; i++) x[i] = cmul(a, x[i]);
}

static void zaxpy(long n, cplx a, const cplx* x, cplx* y) {
#pragma omp parallel for schedule(static) if (n > 16384)
    for (long i = 0; i < n; i++) y[i] = cadd(y[i], cmul(a, x[i]));
}

/* zgemv ConjTrans over nv row vectors of V (row-major, stride n):
 * out[k] = sum_i conj(V[k][i]) * r[i]        (functors.h:236-240) */
static void block_inner(long n, int nv, const cplx* V, const cplx* r, cplx* out) {
    for (int k = 0; k < nv; k++) out[k] = zdotc(n, V + (long)k * n, r);
}

/* zgemv NoTrans: tmp[i] = sum_k V[k][i] * h[k]   (pamp.h:330) */
static void block_combine(long n, int nv, const cplx* V, const cplx* h, cplx* tmp) {
#pragma omp parallel for schedule(static) if (n > 4096)
    for (long i = 0; i < n; i++) {
        double sr = 0.0, si = 0.0;
        for (int k = 0; k < nv; k++) {
            cplx v = V[(long)k * n + i];
            sr += v.re * h[k].re - v.im * h[k].im;
            si += v.re * h[k].im + v.im * h[k].re;
        }
        tmp[i].re = sr; tmp[i].im = si;
    }
}

/* ------------------------------------------------------------------------ */
/* Banded kernels                                                           */
/* ------------------------------------------------------------------------ */

/* zgbmv 'N': y += alpha * A x, A n-by-n in BLAS general band storage with
 * kl = ku = kb, lda = 2*kb+1, element (i,j) at j*lda + kb + i - j
 * (GeometryInfo.py:433-454; generator.py:709-723). */
static void zgbmv_acc(int n, int kb, cplx alpha, const cplx* A, const cplx* x, cplx* y) {
    int lda = 2 * kb + 1;
    /* netlib column sweep: for each column j, temp = alpha*x[j]; y[i] += temp*A(i,j) */
    for (int j = 0; j < n; j++) {
        cplx temp = cmul(alpha, x[j]);
        int i0 = j - kb < 0 ? 0 : j - kb;
        int i1 = j + kb > n - 1 ? n - 1 : j + kb;
        const cplx* col = A + (long)j * lda + kb - j;
        for (int i = i0; i <= i1; i++) y[i] = cadd(y[i], cmul(temp, col[i]));
    }
}

/* Upper band triangular storage of the overlap Cholesky factor U
 * (OverlapMatrix::OverlapCholeskyUpper, overlapmatrix.cpp:23-37):
 * blitz shape (n, kd+1), element U(i,j), i<=j<=i+kd, at j*(kd+1) + kd + i - j. */
#define UB(U, kd, i, j) ((U)[(long)(j) * ((kd) + 1) + (kd) + (i) - (j)])

/* zpbtrf 'U': S = U^H U in place (overlapmatrix.cpp:35-37). Returns info. */
int orc_zpbtrf_upper(int n, int kd, cplx* AB) {
    for (int j = 0; j < n; j++) {
        int k0 = j - kd < 0 ? 0 : j - kd;
        double d = UB(AB, kd, j, j).re;
        for (int k = k0; k < j; k++) { cplx u = UB(AB, kd, k, j); d -= u.re * u.re + u.im * u.im; }
        if (!(d > 0.0)) return j + 1;
        d = sqrt(d);
        UB(AB, kd, j, j).re = d; UB(AB, kd, j, j).im = 0.0;
        int i1 = j + kd > n - 1 ? n - 1 : j + kd;
        for (int i = j + 1; i <= i1; i++) {
            cplx s = UB(AB, kd, j, i);
            int kk0 = i - kd < 0 ? 0 : i - kd;
            if (kk0 < k0) kk0 = k0;
            for (int k = kk0; k < j; k++) s = csub(s, cconjmul(UB(AB, kd, k, j), UB(AB, kd, k, i)));
            s.re /= d; s.im /= d;
            UB(AB, kd, j, i) = s;
        }
    }
    return 0;
}

/* ztbmv 'U','N','N': x <- U x (MultiplySqrtOverlapVector(false), overlapmatrix.cpp:137-142) */
static void ztbmv_upper(int n, int kd, const cplx* U, cplx* x) {
    for (int i = 0; i < n; i++) {
        int j1 = i + kd > n - 1 ? n - 1 : i + kd;
        cplx s = { 0.0, 0.0 };
        for (int j = i; j <= j1; j++) s = cadd(s, cmul(UB(U, kd, i, j), x[j]));
        x[i] = s;
    }
}

/* ztbsv 'U','N','N': x <- U^-1 x (SolveSqrtOverlapVector(false), overlapmatrix.cpp:144-149) */
static void ztbsv_upper(int n, int kd, const cplx* U, cplx* x) {
    for (int i = n - 1; i >= 0; i--) {
        int j1 = i + kd > n - 1 ? n - 1 : i + kd;
        cplx s = x[i];
        for (int j = i + 1; j <= j1; j++) s = csub(s, cmul(UB(U, kd, i, j), x[j]));
        x[i] = cdiv(s, UB(U, kd, i, i));
    }
}

/* ztbsv 'U','C','N': x <- U^-H x (SolveSqrtOverlapVector(true)) */
static void ztbsv_upper_conj(int n, int kd, const cplx* U, cplx* x) {
    for (int i = 0; i < n; i++) {
        int j0 = i - kd < 0 ? 0 : i - kd;
        cplx s = x[i];
        for (int j = j0; j < i; j++) s = csub(s, cconjmul(UB(U, kd, j, i), x[j]));
        cplx d = UB(U, kd, i, i); d.im = -d.im;
        x[i] = cdiv(s, d);
    }
}

/* ------------------------------------------------------------------------ */
/* Operator: TensorPotential list in reference storage + balanced overlap   */
/* ------------------------------------------------------------------------ */

enum { ORC_DIAG_BANDNH = 0, ORC_SIMP_BANDNH = 1 };

typedef struct {
    int nl, nr, kb;          /* angular count, radial count, band half-width (k-1) */
    int kd;                  /* superdiagonals of the overlap Cholesky factor (k-1) */
    const cplx* U;           /* overlap Cholesky factor, upper band storage (nr, kd+1) */
    int npot;
    const int* kind;         /* per potential: ORC_DIAG_BANDNH or ORC_SIMP_BANDNH */
    const int* timedep;      /* per potential: 0 static, k >= 1 scaled by time function k */
    const int* npairs;       /* per potential: angular pair count (Simp) or nl (Diag) */
    const int* const* pairs; /* per potential: (npairs, 2) int32 (row, col); NULL for Diag */
    const cplx* const* data; /* per potential: (npairs, (2kb+1)*nr) complex128 */
    int nfuncs;              /* number of distinct time functions (the largest timedep) */
} orc_operator;

/* PropagatorBase.MultiplyPotential -> TensorPotential.MultiplyPotential for every
 * consolidated potential (Propagator.py:61-66, TensorPotential.py:92-112):
 * dst[row] += s * A_pair * src[col].  s = 1 for static potentials, else the value of the
 * potential's own time function, scalings[timedep - 1] (each potential is scaled by its
 * own f(t), TensorPotential.py:98-100). */
void orc_multiply_potentials(const orc_operator* op, const double* scalings, const cplx* src, cplx* dst) {
    long nr = op->nr;
    int lda = 2 * op->kb + 1;
    for (int p = 0; p < op->npot; p++) {
        cplx s = { op->timedep[p] ? scalings[op->timedep[p] - 1] : 1.0, 0.0 };
        const cplx* V = op->data[p];
        if (op->kind[p] == ORC_DIAG_BANDNH) {
#pragma omp parallel for schedule(static)
            for (int l = 0; l < op->nl; l++)
                zgbmv_acc(op->nr, op->kb, s, V + (long)l * lda * nr, src + l * nr, dst + l * nr);
        } else {
            const int* pr = op->pairs[p];
            int np = op->npairs[p];
            /* pairs are processed in their stored order; rows written by more than
             * one pair are accumulated sequentially per row to keep the order */
#pragma omp parallel for schedule(static)
            for (int row = 0; row < op->nl; row++) {
                for (int i = 0; i < np; i++) {
                    if (pr[2 * i] != row) continue;
                    int col = pr[2 * i + 1];
                    zgbmv_acc(op->nr, op->kb, s, V + (long)i * lda * nr, src + (long)col * nr, dst + (long)row * nr);
                }
            }
        }
    }
}

/* BasisPropagator.MultiplyHamiltonianBalancedOverlap (BasisPropagator.py:131-159):
 * dst = U^-H  H(t)  U^-1 src, src left unchanged. `work` holds nl*nr entries. */
void orc_balanced_matvec(const orc_operator* op, const double* scalings, const cplx* src, cplx* dst, cplx* work) {
    long N = (long)op->nl * op->nr;
    memcpy(work, src, N * sizeof(cplx));                       /* StorePsi + in-place solve */
#pragma omp parallel for schedule(static)
    for (int l = 0; l < op->nl; l++) ztbsv_upper(op->nr, op->kd, op->U, work + (long)l * op->nr);
    memset(dst, 0, N * sizeof(cplx));                          /* dest = 0 */
    orc_multiply_potentials(op, scalings, work, dst);
#pragma omp parallel for schedule(static)
    for (int l = 0; l < op->nl; l++) ztbsv_upper_conj(op->nr, op->kd, op->U, dst + (long)l * op->nr);
}

/* CombinedRepresentation::MultiplySqrtOverlap(false) / SolveSqrtOverlap(false) */
void orc_multiply_sqrt_overlap(const orc_operator* op, cplx* psi) {
#pragma omp parallel for schedule(static)
    for (int l = 0; l < op->nl; l++) ztbmv_upper(op->nr, op->kd, op->U, psi + (long)l * op->nr);
}
void orc_solve_sqrt_overlap(const orc_operator* op, int conj, cplx* psi) {
#pragma omp parallel for schedule(static)
    for (int l = 0; l < op->nl; l++) {
        if (conj) ztbsv_upper_conj(op->nr, op->kd, op->U, psi + (long)l * op->nr);
        else ztbsv_upper(op->nr, op->kd, op->U, psi + (long)l * op->nr);
    }
}

/* ------------------------------------------------------------------------ */
/* Small dense matrices (row-major math layout M[r*m + c])                   */
/* ------------------------------------------------------------------------ */

static void mat_mul(int m, const cplx* A, const cplx* B, cplx* C) {
    for (int r = 0; r < m; r++)
        for (int c = 0; c < m; c++) {
            double sr = 0.0, si = 0.0;
            for (int k = 0; k < m; k++) {
                cplx a = A[r * m + k], b = B[k * m + c];
                sr += a.re * b.re - a.im * b.im;
                si += a.re * b.im + a.im * b.re;
            }
            C[r * m + c].re = sr; C[r * m + c].im = si;
        }
}

/* zgetrf (partial pivoting on |re|+|im|, as izamax) + zgetrs 'N' with m right-hand
 * sides: B <- A^-1 B. Returns info (0 ok, >0 singular pivot). A is overwritten. */
static int lu_solve(int m, cplx* A, cplx* B) {
    int* piv = (int*)malloc(sizeof(int) * m);
    int info = 0;
    for (int k = 0; k < m; k++) {
        int p = k; double best = cabs1(A[k * m + k]);
        for (int r = k + 1; r < m; r++) { double v = cabs1(A[r * m + k]); if (v > best) { best = v; p = r; } }
        piv[k] = p;
        if (best == 0.0) { if (!info) info = k + 1; continue; }
        if (p != k) for (int c = 0; c < m; c++) { cplx t = A[k * m + c]; A[k * m + c] = A[p * m + c]; A[p * m + c] = t; }
        cplx inv = cdiv((cplx){1.0, 0.0}, A[k * m + k]);
        for (int r = k + 1; r < m; r++) {
            cplx f = cmul(A[r * m + k], inv);
            A[r * m + k] = f;
            for (int c = k + 1; c < m; c++) A[r * m + c] = csub(A[r * m + c], cmul(f, A[k * m + c]));
        }
    }
    if (!info) {
        for (int k = 0; k < m; k++) if (piv[k] != k)
            for (int c = 0; c < m; c++) { cplx t = B[k * m + c]; B[k * m + c] = B[piv[k] * m + c]; B[piv[k] * m + c] = t; }
        for (int c = 0; c < m; c++) {
            for (int r = 0; r < m; r++) {            /* L y = b, unit lower */
                cplx s = B[r * m + c];
                for (int k = 0; k < r; k++) s = csub(s, cmul(A[r * m + k], B[k * m + c]));
                B[r * m + c] = s;
            }
            for (int r = m - 1; r >= 0; r--) {       /* U x = y */
                cplx s = B[r * m + c];
                for (int k = r + 1; k < m; k++) s = csub(s, cmul(A[r * m + k], B[k * m + c]));
                B[r * m + c] = cdiv(s, A[r * m + r]);
            }
        }
    }
    free(piv);
    return info;
}

/* pAMP::PadeExponential (pamp.h:470-564): diagonal Pade approximant of the
 * given order, P odd part and Q even part evaluated by Horner in A^2,
 * exp(A) ~ I + 2 (Q-P)^-1 P, negated when `odd` ends true. */
int orc_pade_exponential(int m, const cplx* A, int order, cplx* out) {
    long mm = (long)m * m;
    cplx* Asqr = (cplx*)calloc(mm, sizeof(cplx));
    cplx* P = (cplx*)calloc(mm, sizeof(cplx));
    cplx* Q = (cplx*)calloc(mm, sizeof(cplx));
    cplx* T = (cplx*)calloc(mm, sizeof(cplx));
    double coeff[64];
    mat_mul(m, A, A, Asqr);
    coeff[0] = 1.0;
    for (int i = 0; i < order; i++)
        coeff[i + 1] = coeff[i] * (double)(order - i) / (double)((i + 1) * (2 * order - i));
    for (int i = 0; i < m; i++) { Q[i * m + i].re = coeff[order]; P[i * m + i].re = coeff[order - 1]; }
    int odd = 1;
    for (int i = order - 2; i >= 0; i--) {
        cplx* X = odd ? Q : P;
        mat_mul(m, X, Asqr, T);
        memcpy(X, T, mm * sizeof(cplx));
        for (int r = 0; r < m; r++) X[r * m + r].re += coeff[i];
        odd = !odd;
    }
    cplx* X = odd ? Q : P;
    mat_mul(m, X, A, T);
    memcpy(X, T, mm * sizeof(cplx));
    for (long i = 0; i < mm; i++) Q[i] = csub(Q[i], P[i]);
    int info = lu_solve(m, Q, P);
    for (long i = 0; i < mm; i++) { out[i].re = 2.0 * P[i].re; out[i].im = 2.0 * P[i].im; }
    for (int i = 0; i < m; i++) out[i * m + i].re += 1.0;
    if (odd) for (long i = 0; i < mm; i++) { out[i].re = -out[i].re; out[i].im = -out[i].im; }
    free(Asqr); free(P); free(Q); free(T);
    return info;
}

/* pAMP::ScalingPadeExponential (pamp.h:430-467) with ScalingOrder = -1:
 * s = max(0, ceil(log2(max |A_ij|))), A /= 2^s, Pade, then s squarings.
 * Returns the LU info; *scaling_out receives s. */
int orc_scaling_pade_exponential(int m, const cplx* Ain, int order, cplx* out, int* scaling_out) {
    if (scaling_out) *scaling_out = 0;
    if (m <= 0) return 0;
    long mm = (long)m * m;
    cplx* A = (cplx*)malloc(mm * sizeof(cplx));
    cplx* T = (cplx*)malloc(mm * sizeof(cplx));
    double maxv = 0.0;
    for (long i = 0; i < mm; i++) { double a = hypot(Ain[i].re, Ain[i].im); if (a > maxv) maxv = a; }
    int s = maxv > 0.0 ? (int)ceil(log2(maxv)) : 0;
    if (s < 0) s = 0;
    double sc = pow(2.0, s);
    for (long i = 0; i < mm; i++) { A[i].re = Ain[i].re / sc; A[i].im = Ain[i].im / sc; }
    int info = orc_pade_exponential(m, A, order, out);
    for (int i = 0; i < s; i++) { mat_mul(m, out, out, T); memcpy(out, T, mm * sizeof(cplx)); }
    if (scaling_out) *scaling_out = s;
    free(A); free(T);
    return info;
}

/* ------------------------------------------------------------------------ */
/* pAMP                                                                     */
/* ------------------------------------------------------------------------ */

typedef struct {
    long operator_count;
    long inner_product_count;
    long orthogonalization_count;
    long breakdown_count;
    long pade_info;          /* last non-zero LU info, 0 if none */
    double error_estimate;   /* |y[m-1]|^2 of the last step (GetPropagationErrorEstimate) */
    int last_scaling;        /* scaling order of the last exponential */
    int last_basis;          /* Krylov vectors built in the last step */
} orc_stats;

/* The Arnoldi part of pAMP::PropagateVector on x (balanced coordinates): beta0 = ||x||
 * (returned), the m basis vectors V (m*N) and the Hessenberg matrix H (m*m, H(i, j) =
 * <v_i, A v_j> at H[i*m + j]).  ov, ov3: m + 1 each; r, tmp, work: N each. */
static double pamp_arnoldi(const orc_operator* op, const double* scalings, int m, int double_orth, const cplx* x,
                           cplx* V, cplx* H, cplx* r, cplx* tmp, cplx* work, cplx* ov, cplx* ov3, orc_stats* st) {
    long N = (long)op->nl * op->nr;
    const double tol = sqrt(DBL_EPSILON);          /* pamp.h:79 */

    memcpy(r, x, N * sizeof(cplx));                               /* Residual = input */
    double norm = global_norm(N, r);                               /* pamp.h:619-620 */
    zscal(N, (cplx){1.0 / norm, 0.0}, r);

    /* PerformInitialArnoldiStep, pamp.h:271-290 */
    memset(V, 0, sizeof(cplx) * m * N);
    memset(H, 0, sizeof(cplx) * m * m);
    memcpy(V, r, N * sizeof(cplx));
    orc_balanced_matvec(op, scalings, V, r, work); st->operator_count++;
    cplx alpha = zdotc(N, V, r); st->inner_product_count++;
    zaxpy(N, (cplx){-alpha.re, -alpha.im}, V, r);
    H[0] = alpha;

    int nbasis = 1;
    int breakdown = 0;
    /* RecreateArnoldiFactorization, pamp.h:419-426 -> PerformArnoldiStep, pamp.h:293-350 */
    for (int j = 0; j < m - 1; j++) {
        double beta = global_norm(N, r);
        if (fabs(beta) < tol) { breakdown = 1; st->breakdown_count++; break; }
        zscal(N, (cplx){1.0 / beta, 0.0}, r);
        cplx* vj1 = V + (long)(j + 1) * N;
        memcpy(vj1, r, N * sizeof(cplx));
        H[(j + 1) * m + j].re = beta;                              /* H(j+1, j) = beta */
        orc_balanced_matvec(op, scalings, vj1, r, work); st->operator_count++;
        nbasis = j + 2;
        double orig = global_norm(N, r);
        block_inner(N, j + 2, V, r, ov);
        block_combine(N, j + 2, V, ov, tmp);
        zaxpy(N, (cplx){-1.0, 0.0}, tmp, r);
        double resid = global_norm(N, r);
        if (double_orth) {                                         /* pamp.h:353-400 */
            int count = 0;
            while (fabs(resid) < 0.717 * fabs(orig)) {
                st->orthogonalization_count++;
                count++;
                if (count > 3) break;
                block_inner(N, j + 2, V, r, ov3);
                block_combine(N, j + 2, V, ov3, tmp);
                zaxpy(N, (cplx){-1.0, 0.0}, tmp, r);
                for (int k = 0; k < j + 2; k++) ov[k] = cadd(ov[k], ov3[k]);
                orig = resid;
                resid = global_norm(N, r);
            }
        }
        for (int k = 0; k < j + 2; k++) H[k * m + (j + 1)] = ov[k];  /* column j+1 */
    }
    (void)breakdown;
    st->last_basis = nbasis;
    return norm;
}

/* pAMP::PropagateVector on x (balanced coordinates), one call. V: m*N, H: m*m,
 * r, tmp, work: N each. */
static int pamp_propagate(const orc_operator* op, const double* scalings, int m, cplx dt, int double_orth,
                          cplx* x, cplx* V, cplx* H, cplx* r, cplx* tmp, cplx* work, orc_stats* st) {
    long N = (long)op->nl * op->nr;
    cplx* ov = (cplx*)malloc(sizeof(cplx) * (m + 1));
    cplx* ov3 = (cplx*)malloc(sizeof(cplx) * (m + 1));
    cplx* E = (cplx*)malloc(sizeof(cplx) * m * m);
    const double norm = pamp_arnoldi(op, scalings, m, double_orth, x, V, H, r, tmp, work, ov, ov3, st);

    /* HessenbergMatrix *= -dt * i  (pamp.h:634) */
    cplx f = { dt.im, -dt.re };                                    /* -i*dt */
    for (int i = 0; i < m * m; i++) H[i] = cmul(H[i], f);
    int s = 0;
    int info = orc_scaling_pade_exponential(m, H, 6, E, &s);
    if (info) st->pade_info = info;
    st->last_scaling = s;

    /* y = first column of exp(H); x = norm * V^T y  (pamp.h:657-662) */
    for (int k = 0; k < m; k++) ov[k] = E[k * m + 0];
    block_combine(N, m, V, ov, x);
    zscal(N, (cplx){norm, 0.0}, x);
    st->error_estimate = ov[m - 1].re * ov[m - 1].re + ov[m - 1].im * ov[m - 1].im;
    free(ov); free(ov3); free(E);
    return info;
}

/* Advance `nsteps` PamPropagator steps (PamPropagator.py:50-57, Problem.py:158-173)
 * on psi (nl*nr complex128, C order psi[l][r]).  scalings[n * nfuncs + k] is time function
 * k + 1 evaluated at the start of step n (TensorPotential.py:98-100 with t=PropagatedTime).
 * Returns 0, or the LU info of a failed Pade solve. */
int orc_advance(const orc_operator* op, cplx* psi, int m, double dt_re, double dt_im,
                int nsteps, const double* scalings, int double_orth, orc_stats* st) {
    long N = (long)op->nl * op->nr;
    cplx* V = (cplx*)malloc(sizeof(cplx) * (long)m * N);
    cplx* H = (cplx*)malloc(sizeof(cplx) * m * m);
    cplx* r = (cplx*)malloc(sizeof(cplx) * N);
    cplx* tmp = (cplx*)malloc(sizeof(cplx) * N);
    cplx* work = (cplx*)malloc(sizeof(cplx) * N);
    cplx dt = { dt_re, dt_im };
    const int nf = op->nfuncs > 0 ? op->nfuncs : 1;
    int rc = 0;
    for (int n = 0; n < nsteps && !rc; n++) {
        orc_multiply_sqrt_overlap(op, psi);
        rc = pamp_propagate(op, scalings + (long)n * nf, m, dt, double_orth, psi, V, H, r, tmp, work, st);
        orc_solve_sqrt_overlap(op, 0, psi);
    }
    free(V); free(H); free(r); free(tmp); free(work);
    return rc;
}

/* The Arnoldi part of one pAMP call on x (balanced coordinates, unchanged): V (m*N), the
 * unscaled Hessenberg matrix H (m*m), and beta0 = ||x|| in *norm_out.  Used to restate the
 * eigenvector exponential (pamp.h:567-607), whose zgeev the caller runs. */
int orc_arnoldi(const orc_operator* op, const cplx* x, int m, const double* scalings, int double_orth,
                cplx* V_out, cplx* H_out, double* norm_out, orc_stats* st) {
    long N = (long)op->nl * op->nr;
    cplx* r = (cplx*)malloc(sizeof(cplx) * N);
    cplx* tmp = (cplx*)malloc(sizeof(cplx) * N);
    cplx* work = (cplx*)malloc(sizeof(cplx) * N);
    cplx* ov = (cplx*)malloc(sizeof(cplx) * (m + 1));
    cplx* ov3 = (cplx*)malloc(sizeof(cplx) * (m + 1));
    *norm_out = pamp_arnoldi(op, scalings, m, double_orth, x, V_out, H_out, r, tmp, work, ov, ov3, st);
    free(r); free(tmp); free(work); free(ov); free(ov3);
    return 0;
}

/* One pAMP call on a vector already in balanced coordinates; exposes H and
 * exp(H) for the small-matrix parity tests. */
int orc_pamp_once(const orc_operator* op, cplx* x, int m, double dt_re, double dt_im, const double* scalings,
                  int double_orth, cplx* H_out, orc_stats* st) {
    long N = (long)op->nl * op->nr;
    cplx* V = (cplx*)malloc(sizeof(cplx) * (long)m * N);
    cplx* r = (cplx*)malloc(sizeof(cplx) * N);
    cplx* tmp = (cplx*)malloc(sizeof(cplx) * N);
    cplx* work = (cplx*)malloc(sizeof(cplx) * N);
    int rc = pamp_propagate(op, scalings, m, (cplx){dt_re, dt_im}, double_orth, x, V, H_out, r, tmp, work, st);
    free(V); free(r); free(tmp); free(work);
    return rc;
}


/* ------------------------------------------------------------------------ */
/* ExpokitPropagator (pyprop/propagator/KrylovPropagator.py:44-49,           */
/* core/krylov/expokit/expokitpropagator.cpp:36-103): Expokit zgexpv with the */
/* balanced matvec times -i (real time) or -1 (imaginary time),              */
/* core/krylov/krylovcommon.h:61-70.  Restated from the published algorithm  */
/* (Sidje, ACM TOMS 24, 1998) as the reference calls it: modified Gram-      */
/* Schmidt Arnoldi on the operator itself, augmented (m+2) Hessenberg,       */
/* zgpadm Pade (6,6) scaled by the infinity norm, two-term error estimate,   */
/* step sizes rounded to two significant digits.                            */
/* ------------------------------------------------------------------------ */

/* zgpadm: exp(t H), H n x n row-major, into E; returns LU info. */
static int expokit_pade(int n, const cplx* H, double t, cplx* E) {
    const int p = 6;
    long nn = (long)n * n;
    double hn = 0.0;
    for (int i = 0; i < n; i++) {
        double r = 0.0;
        for (int j = 0; j < n; j++) { cplx v = H[i * n + j]; r += sqrt(v.re * v.re + v.im * v.im); }
        if (r > hn) hn = r;
    }
    hn = fabs(t * hn);
    if (hn == 0.0) {
        memset(E, 0, nn * sizeof(cplx));
        for (int i = 0; i < n; i++) E[i * n + i].re = 1.0;
        return 0;
    }
    int ns = (int)(log(hn) / log(2.0)) + 2;
    if (ns < 0) ns = 0;
    double sc = t / ldexp(1.0, ns), sc2 = sc * sc;
    double c[8];
    c[0] = 1.0;
    for (int k = 1; k <= p; k++) c[k] = c[k - 1] * (double)(p + 1 - k) / (double)(k * (2 * p + 1 - k));
    cplx* H2 = (cplx*)calloc(nn, sizeof(cplx));
    cplx* P = (cplx*)calloc(nn, sizeof(cplx));
    cplx* Q = (cplx*)calloc(nn, sizeof(cplx));
    cplx* T = (cplx*)calloc(nn, sizeof(cplx));
    mat_mul(n, H, H, H2);
    for (long i = 0; i < nn; i++) { H2[i].re *= sc2; H2[i].im *= sc2; }
    for (int i = 0; i < n; i++) { P[i * n + i].re = c[p - 1]; Q[i * n + i].re = c[p]; }
    int odd = 1;
    for (int k = p - 1; k > 0; k--) {
        cplx* X = odd ? Q : P;
        mat_mul(n, X, H2, T);
        memcpy(X, T, nn * sizeof(cplx));
        for (int i = 0; i < n; i++) X[i * n + i].re += c[k - 1];
        odd = 1 - odd;
    }
    cplx* X = odd ? Q : P;
    mat_mul(n, X, H, T);
    for (long i = 0; i < nn; i++) { X[i].re = sc * T[i].re; X[i].im = sc * T[i].im; }
    for (long i = 0; i < nn; i++) Q[i] = csub(Q[i], P[i]);
    int info = lu_solve(n, Q, P);
    for (long i = 0; i < nn; i++) { E[i].re = 2.0 * P[i].re; E[i].im = 2.0 * P[i].im; }
    for (int i = 0; i < n; i++) E[i * n + i].re += 1.0;
    if (ns == 0 && odd) {
        for (long i = 0; i < nn; i++) { E[i].re = -E[i].re; E[i].im = -E[i].im; }
    } else {
        for (int k = 0; k < ns; k++) { mat_mul(n, E, E, T); memcpy(E, T, nn * sizeof(cplx)); }
    }
    free(H2); free(P); free(Q); free(T);
    return info;
}

static double expokit_round(double x) {
    int e = (int)lround(log10(x) - sqrt(0.1)) - 1;
    double p = pow(10.0, (double)e);
    return trunc(x / p + 0.55) * p;
}

typedef struct {
    long substeps, rejections, matvecs;
    double error, hump, last_step;
} orc_expokit_stats;

/* zgexpv on w (balanced coordinates, in place): w <- exp(t_out * fac * A) w. */
static int zgexpv(const orc_operator* op, const double* scalings, int m, double t_out, cplx fac, double tol, double anorm,
                  cplx* w, cplx* V, cplx* work, orc_expokit_stats* st) {
    long N = (long)op->nl * op->nr;
    int mh = m + 2;
    cplx* H = (cplx*)calloc((long)mh * mh, sizeof(cplx));
    cplx* F = (cplx*)calloc((long)mh * mh, sizeof(cplx));
    cplx* Hs = (cplx*)calloc((long)mh * mh, sizeof(cplx));
    double eps = DBL_EPSILON;
    if (tol <= eps) tol = sqrt(eps);
    double rndoff = eps * anorm, btol = 1e-7;
    double beta = global_norm(N, w), vnorm = beta;
    double xm = 1.0 / m;
    double p2 = tol * pow((m + 1) / 2.72, m + 1) * sqrt((m + 1) * 6.28);
    double t_new = expokit_round(1.0 / anorm * pow(p2 / (4.0 * beta * anorm), xm));
    double t_now = 0.0;
    int rc = 0;
    while (t_now < t_out) {
        double t_step = t_out - t_now < t_new ? t_out - t_now : t_new;
        for (long i = 0; i < N; i++) { V[i].re = w[i].re / beta; V[i].im = w[i].im / beta; }
        memset(H, 0, (long)mh * mh * sizeof(cplx));
        int k1 = 2, mb = m;
        double avnorm = 0.0;
        for (int j = 0; j < m; j++) {
            cplx* p = V + (long)(j + 1) * N;
            orc_balanced_matvec(op, scalings, V + (long)j * N, p, work);
            for (long i = 0; i < N; i++) p[i] = cmul(fac, p[i]);
            st->matvecs++;
            for (int i = 0; i <= j; i++) {                   /* modified Gram-Schmidt */
                cplx hij = zdotc(N, V + (long)i * N, p);
                zaxpy(N, (cplx){-hij.re, -hij.im}, V + (long)i * N, p);
                H[i * mh + j] = hij;
            }
            double hj1j = global_norm(N, p);
            if (hj1j <= btol) { k1 = 0; mb = j + 1; t_step = t_out - t_now; break; }
            H[(j + 1) * mh + j].re = hj1j;
            zscal(N, (cplx){1.0 / hj1j, 0.0}, p);
        }
        if (k1 != 0) {
            orc_balanced_matvec(op, scalings, V + (long)m * N, work + N, work);
            for (long i = 0; i < N; i++) work[N + i] = cmul(fac, work[N + i]);
            st->matvecs++;
            avnorm = global_norm(N, work + N);
            H[(m + 1) * mh + m].re = 1.0;
        }
        int ireject = 0, mx;
        double err_loc = 0.0;
        for (;;) {
            mx = mb + k1;
            for (int i = 0; i < mx; i++) for (int j = 0; j < mx; j++) Hs[i * mx + j] = H[i * mh + j];
            if (expokit_pade(mx, Hs, t_step, F)) { rc = 1; goto done; }
            if (k1 == 0) { err_loc = tol; break; }
            double q1 = sqrt(F[m * mx].re * F[m * mx].re + F[m * mx].im * F[m * mx].im) * beta;
            double q2 = sqrt(F[(m + 1) * mx].re * F[(m + 1) * mx].re + F[(m + 1) * mx].im * F[(m + 1) * mx].im) * beta * avnorm;
            if (q1 > 10.0 * q2) { err_loc = q2; xm = 1.0 / m; }
            else if (q1 > q2) { err_loc = q1 * q2 / (q1 - q2); xm = 1.0 / m; }
            else { err_loc = q1; xm = 1.0 / (m - 1); }
            if (err_loc <= 1.2 * t_step * tol) break;
            t_step = expokit_round(0.9 * t_step * pow(t_step * tol / err_loc, xm));
            st->rejections++;
            if (++ireject > 100) { rc = 2; goto done; }
        }
        mx = mb + (k1 - 1 > 0 ? k1 - 1 : 0);
        {
            int ld = mb + k1;
            memset(w, 0, N * sizeof(cplx));
            for (int k = 0; k < mx; k++) {
                cplx f = { beta * F[k * ld].re, beta * F[k * ld].im };
                zaxpy(N, f, V + (long)k * N, w);
            }
        }
        beta = global_norm(N, w);
        if (beta / vnorm > st->hump) st->hump = beta / vnorm;
        t_now += t_step;
        t_new = expokit_round(0.9 * t_step * pow(t_step * tol / err_loc, xm));
        st->error += err_loc > rndoff ? err_loc : rndoff;
        st->last_step = t_step;
        st->substeps++;
    }
done:
    free(H); free(F); free(Hs);
    return rc;
}

int orc_expokit_advance(const orc_operator* op, cplx* psi, int m, double dt_re, double dt_im, int nsteps,
                        const double* scalings, double tol, double anorm, orc_expokit_stats* st) {
    long N = (long)op->nl * op->nr;
    cplx* V = (cplx*)malloc(sizeof(cplx) * (long)(m + 1) * N);
    cplx* work = (cplx*)malloc(sizeof(cplx) * 2 * N);
    double t_out = sqrt(dt_re * dt_re + dt_im * dt_im);
    cplx fac = fabs(dt_im) > 1e-10 ? (cplx){-1.0, 0.0} : (cplx){0.0, -1.0};
    int rc = 0;
    st->substeps = st->rejections = st->matvecs = 0;
    st->error = 0.0; st->hump = 1.0; st->last_step = 0.0;
    const int nf = op->nfuncs > 0 ? op->nfuncs : 1;
    for (int n = 0; n < nsteps && !rc; n++) {
        orc_multiply_sqrt_overlap(op, psi);
        rc = zgexpv(op, scalings + (long)n * nf, m, t_out, fac, tol, anorm, psi, V, work, st);
        orc_solve_sqrt_overlap(op, 0, psi);
    }
    free(V); free(work);
    return rc;
}
