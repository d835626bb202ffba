// Host runtime of libgbprop: the C ABI declared in include/gbprop.h.
//
// One handle = one propagation problem (the reference's PamPropagator +
// krylov_PampWrapper_<2> + the consolidated TensorPotential list of its
// BasisPropagator).  The handle owns the operator tables and the Krylov
// workspace on the device; the wavefunction stays caller-owned, as in the
// reference (pampwrapper.cpp:28-33 wraps the caller's buffers).  A propagation
// step is enqueued as a fixed kernel sequence on the handle's stream and is
// captured once into a CUDA graph, replayed per step; per-step values (time
// function, time step) are read by the kernels from a device schedule array.
#include "gbprop_internal.h"
#include "../../include/gbprop.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace gbprop {
static std::atomic<long long> g_launches{0};
void count_launch(int n) { g_launches += n; }
long long launch_count() { return g_launches.load(); }
}  // namespace gbprop

using namespace gbprop;

namespace {

thread_local std::string t_err;

gbprop_status fail(gbprop_status st, const std::string& msg) {
    t_err = msg;
    return st;
}

}  // namespace

namespace gbprop {
void set_last_error(const char* msg) { t_err = msg ? msg : ""; }
}  // namespace gbprop

namespace {

#define GB_CUDA(call)                                                                                  \
    do {                                                                                               \
        cudaError_t _e = (call);                                                                       \
        if (_e != cudaSuccess)                                                                         \
            return fail(GBPROP_ECUDA, std::string(#call) + ": " + cudaGetErrorString(_e));             \
    } while (0)

struct HostPot {
    int storage;
    int npairs;
    std::vector<int> pairs;
    int kb;
    std::vector<double> data;   // complex interleaved, (npairs, (2kb+1)*nr)
    int timedep;
};

// Device copies of one precision's tables.
template <typename T> struct DevTables {
    SolveTab<T> tab[2];        // [0]: U^-1,  [1]: U^-T
    BandOp<T> op;
};

}  // namespace

struct gbprop_ctx {
    int nl = 0, nr = 0, prec = 0, m = 0, expm_method = 0, double_orth = 0;
    int nfuncs = 1;                   // distinct time functions (values per schedule step)
    int renormalize = 0;              // psi.Normalize() after every step (renormalization = True)
    double2* d_ip = nullptr;          // 2 N complex128: U a, U b of gbprop_inner_product
    long N = 0;
    cudaStream_t stream = nullptr;    // owned capture/work stream (non-blocking)
    cudaStream_t ustream = nullptr;   // caller's stream; ordered against `stream` by events
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    void* d_host_stage = nullptr;     // device copy used by gbprop_advance_host
    int kd = -1;
    std::vector<double> U;            // upper band storage (nr, kd+1)
    std::vector<HostPot> pots;
    int kb = -1;
    bool finalized = false;

    DevTables<double> t64;
    DevTables<float> t32;
    double* d_ud_phys = nullptr;      // (kd+1) x nr : U(i, i+d)
    Ctrl* d_ctrl = nullptr;
    double* d_H = nullptr;
    SchedEntry* d_sched = nullptr;
    int sched_cap = 0;
    double* d_partials = nullptr;
    unsigned* d_counter = nullptr;
    void* d_V = nullptr;              // m x N, Krylov precision
    void* d_r = nullptr;              // N, Krylov precision (residual / w)
    void* d_s = nullptr;              // N, Krylov precision (U^-1 v)
    void* d_y = nullptr;              // N, Krylov precision (H U^-1 v)
    double2* d_x = nullptr;           // N, complex128 (U psi, V y)
    double2* d_v0 = nullptr;          // N, complex128 first basis vector of a complex64 basis
    float4* d_v0s = nullptr;          // N, the same split into FP32 pairs (re_hi, im_hi, re_lo, im_lo)
    int cgs_grid = 0;                 // > 0: Gram-Schmidt as one cooperative kernel of this many CTAs
    int cgs_cache = 0;                // its V chunk cached in shared memory
    int cgs_part_grid = 0;            // the grid d_cgs_part is sized for
    double* d_cgs_part = nullptr;     // its partial sums
    unsigned* d_gridbar = nullptr;    // its grid-barrier words
    std::vector<void*> allocs;

    // per-phase timing of one un-captured step (gbprop_time_step): when `timing` is set, every
    // launch of the step sequence is followed by an event, tagged with its phase
    std::vector<std::pair<int, cudaEvent_t>>* timing = nullptr;
    std::vector<cudaEvent_t> tick_pool;
    // device error flags (Ctrl::lu_info, nonfinite, wait_timeout) copied to pinned host memory
    // after every advance; read once the copy's event has completed (see device_errors)
    int* h_flags = nullptr;
    cudaEvent_t ev_flags = nullptr;
    bool flags_armed = false;

    cudaGraphExec_t graph = nullptr;      // one step on x (independent of the caller's buffers)
    cudaGraphExec_t graph_arnoldi = nullptr;   // Expokit: the Arnoldi part alone (m+1 vectors)
    long long arnoldi_launches = 0;
    long long graph_launches = 0;
    int band_variant = 1;             // tile shape of the band kernel (autotuner)
    int expm_max_cluster = 16;        // 1 when the handle is advanced inside a batch
    bool inv_ok = false;              // solves run through the banded approximate inverse
    InvTab inv[2] = {};               // [0]: U^-1, [1]: U^-T

    ~gbprop_ctx() {
        if (graph) cudaGraphExecDestroy(graph);
        if (graph_arnoldi) cudaGraphExecDestroy(graph_arnoldi);
        for (void* p : allocs) cudaFree(p);
        if (ev_in) cudaEventDestroy(ev_in);
        if (ev_out) cudaEventDestroy(ev_out);
        if (ev_flags) cudaEventDestroy(ev_flags);
        if (h_flags) cudaFreeHost(h_flags);
        for (cudaEvent_t e : tick_pool) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
    // order the handle's work after / before the caller's stream
    cudaError_t begin() {
        cudaError_t e = cudaEventRecord(ev_in, ustream);
        if (e != cudaSuccess) return e;
        return cudaStreamWaitEvent(stream, ev_in, 0);
    }
    cudaError_t end() {
        cudaError_t e = cudaEventRecord(ev_out, stream);
        if (e != cudaSuccess) return e;
        return cudaStreamWaitEvent(ustream, ev_out, 0);
    }

    int kprec() const { return prec == GBPROP_FP64 ? 0 : 1; }     // 0 = complex128, 1 = complex64
    size_t kelem() const { return prec == GBPROP_FP64 ? sizeof(double2) : sizeof(float2); }

    template <typename P> gbprop_status dalloc(P** out, size_t bytes) {
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
        if (e != cudaSuccess) return fail(GBPROP_ECUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        allocs.push_back(p);
        *out = (P*)p;
        return GBPROP_OK;
    }
    template <typename V> gbprop_status upload(V** out, const std::vector<V>& host) {
        gbprop_status st = dalloc(out, host.size() * sizeof(V));
        if (st) return st;
        cudaError_t e = cudaMemcpyAsync(*out, host.data(), host.size() * sizeof(V), cudaMemcpyHostToDevice, stream);
        if (e != cudaSuccess) return fail(GBPROP_ECUDA, std::string("cudaMemcpyAsync: ") + cudaGetErrorString(e));
        return GBPROP_OK;
    }
};

namespace {

// ---- tables of the parallel triangular solve -------------------------------
struct HostSolveTab {
    int n, kd, L, P, levels, dir;
    std::vector<double> ud, invd, g, mlev;
};

// U(i, j) from upper band storage, 0 outside the band.
double uval(const std::vector<double>& U, int n, int kd, int i, int j) {
    if (i < 0 || j < 0 || i >= n || j >= n || j < i || j > i + kd) return 0.0;
    return U[(size_t)j * (kd + 1) + kd + i - j];
}

// Build the tables for U x = b (dir 0) or U^T x = b (dir 1), the latter written
// as an upper solve in reversed coordinates e = n-1-p.
HostSolveTab build_solve_tab(const std::vector<double>& U, int n, int kd, int dir) {
    HostSolveTab t;
    t.n = n;
    t.kd = kd;
    t.dir = dir;
    int L = (n + kSolveLanes - 1) / kSolveLanes;
    if (L < kd) L = kd;
    if (L < 1) L = 1;
    t.L = L;
    t.P = (n + L - 1) / L;
    int lev = 0;
    while ((1 << lev) < t.P) ++lev;
    t.levels = lev;
    auto ut = [&](int e, int f) -> double {       // upper matrix in e coordinates
        if (dir == 0) return uval(U, n, kd, e, f);
        return uval(U, n, kd, n - 1 - f, n - 1 - e);
    };
    t.ud.assign((size_t)std::max(kd, 1) * L * 32, 0.0);
    t.invd.assign((size_t)L * 32, 0.0);
    t.g.assign((size_t)std::max(kd, 1) * L * 32, 0.0);
    t.mlev.assign((size_t)std::max(lev, 1) * 32 * kd * kd, 0.0);
    std::vector<std::vector<double>> F(t.P, std::vector<double>((size_t)kd * kd, 0.0));
    for (int B = 0; B < t.P; ++B) {
        const int e0 = B * L, e1 = std::min(n, e0 + L), Lb = e1 - e0;
        for (int i = 0; i < Lb; ++i) {
            const int e = e0 + i;
            const double dg = ut(e, e);
            t.invd[(size_t)i * 32 + B] = 1.0 / dg;
            for (int d = 1; d <= kd; ++d)
                if (i + d < Lb) t.ud[((size_t)(d - 1) * L + i) * 32 + B] = ut(e, e + d) / dg;
        }
        if (B + 1 >= t.P) continue;
        // G_B = U_BB^-1 C_B, C_B[i][c] = U~(e0+i, e1+c); back substitution per column c
        std::vector<double> G((size_t)Lb * kd, 0.0);
        for (int c = 0; c < kd; ++c) {
            if (e1 + c >= n) continue;
            for (int i = Lb - 1; i >= 0; --i) {
                const int e = e0 + i;
                double s = ut(e, e1 + c);
                for (int d = 1; d <= kd && i + d < Lb; ++d) s -= ut(e, e + d) * G[(size_t)(i + d) * kd + c];
                G[(size_t)i * kd + c] = s / ut(e, e);
            }
        }
        for (int i = 0; i < Lb; ++i)
            for (int c = 0; c < kd; ++c) t.g[((size_t)c * L + i) * 32 + B] = G[(size_t)i * kd + c];
        for (int r = 0; r < kd && r < Lb; ++r)
            for (int c = 0; c < kd; ++c) F[B][(size_t)r * kd + c] = -G[(size_t)r * kd + c];
    }
    // suffix-scan operators: M^0_B = -F_B, M^{l+1}_B = M^l_B M^l_{B+s}
    std::vector<std::vector<double>> M = F;
    for (int lv = 0; lv < lev; ++lv) {
        const int s = 1 << lv;
        for (int B = 0; B < t.P; ++B)
            for (int k = 0; k < kd * kd; ++k) t.mlev[((size_t)(lv * 32 + B)) * kd * kd + k] = M[B][k];
        std::vector<std::vector<double>> Mn(t.P, std::vector<double>((size_t)kd * kd, 0.0));
        for (int B = 0; B + s < t.P; ++B)
            for (int r = 0; r < kd; ++r)
                for (int c = 0; c < kd; ++c) {
                    double acc = 0.0;
                    for (int k = 0; k < kd; ++k) acc += M[B][(size_t)r * kd + k] * M[B + s][(size_t)k * kd + c];
                    Mn[B][(size_t)r * kd + c] = acc;
                }
        M.swap(Mn);
    }
    return t;
}

// ---- banded approximate inverse of the overlap factor ------------------------
constexpr int kMaxInvBand = 160;      // widest inverse band considered
constexpr int kMaxRefine = 4;

struct HostInvTab {
    bool ok = false;
    int n = 0, kd = 0, w = 0, npad = 0, refine = 0;
    double contraction = 0.0;          // simulated error ratio of one refinement pass
    std::vector<float> m;              // (w+1) x npad
    std::vector<double> u;             // (kd+1) x npad
};

// U~ = U (dir 0) or U^T in reversed coordinates q = n-1-p (dir 1): upper triangular in q.
// Column c of U~^-1 by back substitution down to row c - Wmax; entries beyond the band whose
// tail (relative to the row's total) falls below 2^-26 are dropped.  The number of FP64
// refinement passes is the smallest that brings a simulated solve (FP32 products of the
// device kernel, FP64 residuals) of a fixed pseudo-random right-hand side to the FP64 level.
HostInvTab build_inv_tab(const std::vector<double>& U, int n, int kd, int dir) {
    HostInvTab t;
    t.n = n;
    t.kd = kd;
    t.npad = (n + 3) & ~3;
    auto ut = [&](int e, int f) -> double {
        if (dir == 0) return uval(U, n, kd, e, f);
        return uval(U, n, kd, n - 1 - f, n - 1 - e);
    };
    const int W = std::min(n - 1, kMaxInvBand);
    std::vector<double> inv((size_t)(W + 1) * n, 0.0);        // inv[j*n + q] = U~^-1(q, q+j)
    std::vector<double> y(n, 0.0);
    for (int c = 0; c < n; ++c) {
        const int lo = std::max(0, c - W);
        for (int i = c; i >= lo; --i) {
            double s = (i == c) ? 1.0 : 0.0;
            for (int d = 1; d <= kd && i + d <= c; ++d) s -= ut(i, i + d) * y[i + d];
            y[i] = s / ut(i, i);
            inv[(size_t)(c - i) * n + i] = y[i];
        }
    }
    // band width: largest relative tail over rows
    std::vector<double> tot(n, 0.0), tail(n, 0.0);
    for (int j = 0; j <= W; ++j)
        for (int q = 0; q < n; ++q) tot[q] += std::fabs(inv[(size_t)j * n + q]);
    int w = W;
    {
        std::vector<double> acc(n, 0.0);
        for (int j = W; j >= 1; --j) {
            double worst = 0.0;
            for (int q = 0; q < n; ++q) {
                acc[q] += std::fabs(inv[(size_t)j * n + q]);
                if (tot[q] > 0) worst = std::max(worst, acc[q] / tot[q]);
            }
            if (worst > std::ldexp(1.0, -26)) break;
            w = j - 1;
        }
    }
    t.w = w;
    t.m.assign((size_t)(w + 1) * t.npad, 0.0f);
    for (int j = 0; j <= w; ++j)
        for (int q = 0; q + j < n; ++q) t.m[(size_t)j * t.npad + q] = (float)inv[(size_t)j * n + q];
    t.u.assign((size_t)(kd + 1) * t.npad, 0.0);
    for (int d = 0; d <= kd; ++d)
        for (int q = 0; q + d < n; ++q) t.u[(size_t)d * t.npad + q] = ut(q, q + d);
    // simulate the refined solve on a pseudo-random complex right-hand side
    std::vector<double> br(n), bi(n), xr(n, 0.0), xi(n, 0.0), er(n), ei(n);
    uint64_t st = 0x9e3779b97f4a7c15ull;
    auto rnd = [&]() {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        return (double)(int64_t)(st >> 11) / (double)(1ull << 52) - 1.0;
    };
    for (int q = 0; q < n; ++q) { br[q] = rnd(); bi[q] = rnd(); }
    for (int q = n - 1; q >= 0; --q) {                       // exact (FP64) back substitution
        double sr = br[q], si = bi[q];
        for (int d = 1; d <= kd && q + d < n; ++d) { sr -= ut(q, q + d) * er[q + d]; si -= ut(q, q + d) * ei[q + d]; }
        er[q] = sr / ut(q, q);
        ei[q] = si / ut(q, q);
    }
    double xn = 0.0;
    for (int q = 0; q < n; ++q) xn += er[q] * er[q] + ei[q] * ei[q];
    xn = std::sqrt(xn);
    std::vector<float> rr(n + w + 1, 0.f), ri(n + w + 1, 0.f);
    double prev = 1.0;
    t.refine = -1;
    for (int k = 0; k <= kMaxRefine; ++k) {
        for (int q = 0; q < n; ++q) {
            double sr = br[q], si = bi[q];
            for (int d = 0; d <= kd && q + d < n; ++d) { sr -= ut(q, q + d) * xr[q + d]; si -= ut(q, q + d) * xi[q + d]; }
            rr[q] = (float)sr;
            ri[q] = (float)si;
        }
        for (int q = 0; q < n; ++q) {
            float a[4] = {0, 0, 0, 0}, b[4] = {0, 0, 0, 0};
            for (int j = 0; j <= w; ++j) {
                const float mv = t.m[(size_t)j * t.npad + q];
                a[j & 3] = std::fma(mv, rr[q + j], a[j & 3]);
                b[j & 3] = std::fma(mv, ri[q + j], b[j & 3]);
            }
            xr[q] += (double)((a[0] + a[1]) + (a[2] + a[3]));
            xi[q] += (double)((b[0] + b[1]) + (b[2] + b[3]));
        }
        double e = 0.0;
        for (int q = 0; q < n; ++q) e += (xr[q] - er[q]) * (xr[q] - er[q]) + (xi[q] - ei[q]) * (xi[q] - ei[q]);
        e = std::sqrt(e) / xn;
        if (k == 1) t.contraction = e / prev;
        if (k >= 1 && e <= 1e-15) {                // FP64 level reached
            t.refine = k;
            t.ok = true;
            break;
        }
        if (k >= 1 && e >= 0.5 * prev) {           // stagnated: the previous pass was the last useful one
            t.refine = std::max(1, k - 1);
            t.ok = prev <= 1e-14;
            break;
        }
        prev = e;
    }
    return t;
}

template <typename T>
gbprop_status upload_solve_tab(gbprop_ctx* h, const HostSolveTab& ht, SolveTab<T>* out) {
    auto cvt = [](const std::vector<double>& v) { return std::vector<T>(v.begin(), v.end()); };
    T *ud, *invd, *g, *ml;
    gbprop_status st;
    if ((st = h->upload(&ud, cvt(ht.ud)))) return st;
    if ((st = h->upload(&invd, cvt(ht.invd)))) return st;
    if ((st = h->upload(&g, cvt(ht.g)))) return st;
    if ((st = h->upload(&ml, cvt(ht.mlev)))) return st;
    out->n = ht.n;
    out->kd = ht.kd;
    out->L = ht.L;
    out->P = ht.P;
    out->levels = ht.levels;
    out->dir = ht.dir;
    out->ud = ud;
    out->invd = invd;
    out->g = g;
    out->mlev = ml;
    return GBPROP_OK;
}

// ---- term list of the tensor-potential matvec -------------------------------
struct HostBandOp {
    int kb;
    std::vector<int> row_ptr, src, slot, timedep;
    std::vector<double> coef;
    std::vector<double> slots;   // nslots x (2kb+1) x nr
};

HostBandOp build_band_op(const gbprop_ctx* h) {
    HostBandOp op;
    op.kb = h->kb;
    const int nr = h->nr, kb = h->kb, W = 2 * kb + 1;
    struct Term { int dst, src, slot, td; double cr, ci; };
    std::vector<Term> terms;
    int nslots = 0;
    for (const HostPot& p : h->pots) {
        // split complex band data into a real part (coefficient 1) and an
        // imaginary part (coefficient i); a part that is identically zero is dropped
        for (int part = 0; part < 2; ++part) {
            bool any = false;
            for (size_t k = part; k < p.data.size(); k += 2)
                if (p.data[k] != 0.0) { any = true; break; }
            if (!any) continue;
            const double cr = part == 0 ? 1.0 : 0.0, ci = part == 0 ? 0.0 : 1.0;
            for (int q = 0; q < p.npairs; ++q) {
                const int slot = nslots++;
                op.slots.resize((size_t)nslots * W * nr, 0.0);
                double* S = op.slots.data() + (size_t)slot * W * nr;
                const double* D = p.data.data() + (size_t)q * W * nr * 2;
                for (int i = 0; i < nr; ++i)
                    for (int d = 0; d < W; ++d) {
                        const int j = i + d - kb;
                        if (j < 0 || j >= nr) continue;
                        S[(size_t)d * nr + i] = D[2 * ((size_t)j * W + kb + i - j) + part];
                    }
                if (p.storage == GBPROP_STORAGE_DIAG) {
                    terms.push_back({q, q, slot, p.timedep, cr, ci});
                } else if (p.storage == GBPROP_STORAGE_IDENT) {
                    for (int l = 0; l < h->nl; ++l) terms.push_back({l, l, slot, p.timedep, cr, ci});
                } else {
                    terms.push_back({p.pairs[2 * q], p.pairs[2 * q + 1], slot, p.timedep, cr, ci});
                }
            }
        }
    }
    std::stable_sort(terms.begin(), terms.end(), [](const Term& a, const Term& b) { return a.dst < b.dst; });
    op.row_ptr.assign(h->nl + 1, 0);
    for (const Term& t : terms) {
        op.row_ptr[t.dst + 1]++;
        op.src.push_back(t.src);
        op.slot.push_back(t.slot);
        op.timedep.push_back(t.td);
        op.coef.push_back(t.cr);
        op.coef.push_back(t.ci);
    }
    for (int l = 0; l < h->nl; ++l) op.row_ptr[l + 1] += op.row_ptr[l];
    return op;
}

template <typename T>
gbprop_status upload_band_op(gbprop_ctx* h, const HostBandOp& ho, BandOp<T>* out) {
    int *rp, *src, *slot, *td;
    double* coef;
    T* slots;
    gbprop_status st;
    std::vector<int> srcv = ho.src.empty() ? std::vector<int>{0} : ho.src;
    std::vector<int> slotv = ho.slot.empty() ? std::vector<int>{0} : ho.slot;
    std::vector<int> tdv = ho.timedep.empty() ? std::vector<int>{0} : ho.timedep;
    std::vector<double> coefv = ho.coef.empty() ? std::vector<double>{0, 0} : ho.coef;
    std::vector<T> sl(ho.slots.begin(), ho.slots.end());
    if (sl.empty()) sl.push_back(0);
    if ((st = h->upload(&rp, ho.row_ptr))) return st;
    if ((st = h->upload(&src, srcv))) return st;
    if ((st = h->upload(&slot, slotv))) return st;
    if ((st = h->upload(&td, tdv))) return st;
    if ((st = h->upload(&coef, coefv))) return st;
    if ((st = h->upload(&slots, sl))) return st;
    out->nl = h->nl;
    out->nr = h->nr;
    out->kb = ho.kb;
    out->nterms = (int)ho.src.size();
    out->variant = h->band_variant;
    out->row_ptr = rp;
    out->t_src = src;
    out->t_slot = slot;
    out->t_timedep = td;
    out->t_coef = coef;
    out->slots = slots;
    out->slots_lo = nullptr;
    if (sizeof(T) < sizeof(double)) {
        // complex64 path: the rounding remainder of every coefficient, so the operator
        // applied is the FP64 one (to ~2^-48) and only the FP32 sums round
        std::vector<T> lo(sl.size());
        for (size_t k = 0; k < sl.size(); ++k) lo[k] = (T)(k < ho.slots.size() ? ho.slots[k] - (double)sl[k] : 0.0);
        T* dlo;
        if ((st = h->upload(&dlo, lo))) return st;
        out->slots_lo = dlo;
    }
    return GBPROP_OK;
}

gbprop_status check_handle(gbprop_handle h, bool need_final) {
    if (!h) return fail(GBPROP_EINVAL, "null handle");
    if (need_final && !h->finalized) return fail(GBPROP_EINVAL, "handle not finalized (call gbprop_finalize)");
    return GBPROP_OK;
}

#define GB_LAUNCH(call)                                                                            \
    do {                                                                                           \
        cudaError_t _e = (call);                                                                   \
        if (_e != cudaSuccess) return fail(GBPROP_ECUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

// Phase tag of a launch for gbprop_time_step (the pAMP timers "Operator", "InnerProduct",
// "PadeExponential" of pamp.h:149-151, split finer).
void tick(gbprop_ctx* h, int phase) {
    if (!h->timing) return;
    const size_t k = h->timing->size();
    if (k + 1 >= h->tick_pool.size()) return;          // the last event marks the start
    cudaEventRecord(h->tick_pool[k], h->stream);
    h->timing->push_back({phase, h->tick_pool[k]});
}

// Every time function at the same value (static operators, the autotuner's timing launches).
Scalings uniform_scalings(double v) {
    Scalings sc;
    for (int k = 0; k < kMaxTimeFuncs; ++k) sc.s[k] = v;
    return sc;
}

// Schedule entry of one step from `nf` time-function values.
SchedEntry sched_entry(const double* vals, int nf, double dt_re, double dt_im) {
    SchedEntry e;
    for (int k = 0; k < kMaxTimeFuncs; ++k) e.scaling.s[k] = k < nf ? vals[k] : 0.0;
    e.dt_re = dt_re;
    e.dt_im = dt_im;
    return e;
}

// Chunking of the inverse solve.  `wide` spreads one problem's rows over the GPU: the
// chunk count minimises (waves of CTAs) x (FP64 residual elements of one CTA, halo
// included), the refinement being FP64-issue-bound; otherwise (batches, where other
// problems fill the GPU) the fewest chunks are used.  The chunk's slices of M and U~ are
// staged in shared memory when one CTA's share stays within 220 KB, else read through L2.
void set_inv_chunks(gbprop_ctx* h, bool wide) {
    const int n = h->nr, kd = h->kd, sms = grid_reduce_blocks();
    for (int dir = 0; dir < 2; ++dir) {
        InvTab& t = h->inv[dir];
        const int P = t.refine, w = t.w;
        auto chunk_of = [&](int nch) { return std::max(4, ((n + nch - 1) / nch + 3) & ~3); };
        // the table serves the FP64-accurate solve and, on mixed handles, the complex64 basis
        // solve (which also stages the FP32 pairs of U~): both must fit
        const bool mixed = h->prec != GBPROP_FP64;
        auto smem_of = [&](int chunk, int stage) {
            size_t mx = 0;
            for (int q0 = 0; q0 < n; q0 += chunk) {
                mx = std::max(mx, inv_smem_bytes(n, q0, chunk, P, w, kd, stage, 1));
                if (mixed) mx = std::max(mx, inv_smem_bytes_mixed(n, q0, chunk, w, kd, stage));
            }
            return mx;
        };
        // cost ~ (waves of resident CTAs) x (elements one CTA processes over all passes); CTAs
        // that fit two per SM count as half a wave each (their latency-bound phases overlap)
        auto cost = [&](int chunk, int stage) {
            const int nch = (n + chunk - 1) / chunk;
            long work = 0;
            for (int k = 0; k <= P; ++k) work += std::min(n, chunk + (P - k) * (w + kd) + w);
            const size_t sm = smem_of(chunk, stage) + 1024;
            const int per_sm = std::max(1, std::min(2, (int)((size_t)228 * 1024 / sm)));
            const long waves = ((long)h->nl * nch + (long)sms * per_sm - 1) / ((long)sms * per_sm);
            return waves * work * 2 / per_sm;
        };
        int best = -1, best_stage = 0;
        long best_cost = 0;
        for (int stage = 1; stage >= 0 && best < 0; --stage) {
            for (int nch = 1; nch <= 16; ++nch) {
                const int chunk = chunk_of(nch);
                if (nch > 1 && chunk < 32) break;
                if (smem_of(chunk, stage) > (size_t)220 * 1024) continue;
                const long c = cost(chunk, stage);
                if (best < 0 || (wide ? c < best_cost : false)) {
                    best = chunk;
                    best_cost = c;
                    best_stage = stage;
                }
                if (!wide && best >= 0) break;
            }
        }
        if (best < 0) { best = chunk_of(1); best_stage = 0; }
        t.chunk = best;
        t.nchunks = (n + best - 1) / best;
        t.stage = best_stage;
    }
}

// Use `nch` radial chunks for the solves of direction `dir`, staging the slices when they fit;
// false if one CTA's share exceeds the shared-memory budget either way.
bool set_inv_chunk_count(gbprop_ctx* h, int dir, int nch) {
    InvTab& t = h->inv[dir];
    const int n = h->nr, kd = h->kd, P = t.refine, w = t.w;
    const bool mixed = h->prec != GBPROP_FP64;
    const int chunk = std::max(4, ((n + nch - 1) / nch + 3) & ~3);
    for (int stage = 1; stage >= 0; --stage) {
        size_t mx = 0;
        for (int q0 = 0; q0 < n; q0 += chunk) {
            mx = std::max(mx, inv_smem_bytes(n, q0, chunk, P, w, kd, stage, 1));
            if (mixed) mx = std::max(mx, inv_smem_bytes_mixed(n, q0, chunk, w, kd, stage));
        }
        if (mx <= (size_t)220 * 1024) {
            t.chunk = chunk;
            t.nchunks = (n + chunk - 1) / chunk;
            t.stage = stage;
            return true;
        }
    }
    return false;
}

// Triangular solve of the Krylov precision: FP64-accurate (FP32 solve + FP64 refinement)
// for the FP64 path, plain complex64 for the mixed path's basis.
cudaError_t ksolve(gbprop_ctx* h, int dir, const void* in, int in_prec, void* out, int out_prec, void* vstore,
                   int v_prec, int scale_mode, int check_broken, float4* v0s = nullptr, const void* bpart = nullptr) {
    if (h->inv_ok)
        return launch_solve_inv(h->inv[dir], h->nl, h->prec == GBPROP_FP64 ? 1 : 0, in, in_prec, out, out_prec,
                                vstore, v_prec, h->d_ctrl, dir, scale_mode, check_broken, h->stream, v0s, bpart,
                                h->cgs_grid);
    if (h->prec == GBPROP_FP64)
        return launch_solve_ir(&h->t32.tab[dir], h->d_ud_phys, h->nl, in, in_prec, out, out_prec, vstore, v_prec,
                               h->d_ctrl, scale_mode, check_broken, h->stream);
    return launch_solve(1, &h->t32.tab[dir], h->nl, in, in_prec, out, out_prec, vstore, v_prec, h->d_ctrl,
                        scale_mode, check_broken, h->stream);
}

// FP64-accurate solve of the state transforms (both precisions).
cudaError_t ssolve(gbprop_ctx* h, int dir, const void* in, int in_prec, void* out, int out_prec) {
    if (h->inv_ok)
        return launch_solve_inv(h->inv[dir], h->nl, 1, in, in_prec, out, out_prec, nullptr, 0, h->d_ctrl, dir, 0, 0,
                                h->stream);
    return launch_solve_ir(&h->t32.tab[dir], h->d_ud_phys, h->nl, in, in_prec, out, out_prec, nullptr, 0, h->d_ctrl, 0,
                           0, h->stream);
}

const void* kop(gbprop_ctx* h) {
    return h->prec == GBPROP_FP64 ? (const void*)&h->t64.op : (const void*)&h->t32.op;
}

// The state lives in FP64 balanced coordinates x = U psi (MultiplySqrtOverlap,
// PamPropagator.py:50-52) for the whole of one advance call: enter() forms it, every
// step maps x to x (pamp.h:613-669), leave() returns psi = U^-1 x (SolveSqrtOverlap,
// PamPropagator.py:55-57).  Per step the reference's R^-1 R round trip is exact
// algebra; keeping x removes its rounding and, for complex64 wavefunctions, the
// per-step rounding of the state.
gbprop_status enqueue_enter(gbprop_ctx* h, void* psi, cudaStream_t s) {
    GB_LAUNCH(launch_tbmv(0, h->kd, h->d_ud_phys, h->nl, h->nr, psi, h->kprec(), h->d_x, 0, s));
    tick(h, GBPROP_PHASE_OTHER);
    return GBPROP_OK;
}

gbprop_status enqueue_leave(gbprop_ctx* h, void* psi, cudaStream_t s) {
    cudaStream_t keep = h->stream;
    h->stream = s;
    cudaError_t e = ssolve(h, 0, h->d_x, 0, psi, h->kprec());
    h->stream = keep;
    if (e != cudaSuccess) return fail(GBPROP_ECUDA, std::string("ssolve: ") + cudaGetErrorString(e));
    tick(h, GBPROP_PHASE_SOLVE);
    return GBPROP_OK;
}

// The Arnoldi part of a step on x (pamp.h:271-400): beta0 = ||x||, m basis vectors, the
// Hessenberg matrix.  dorth: re-orthogonalisation passes (pamp.h:353-400); brk_tol: the
// happy-breakdown threshold.
gbprop_status enqueue_arnoldi(gbprop_ctx* h, int dorth, double brk_tol) {
    cudaStream_t s = h->stream;
    const int kp = h->kprec();
    const int m = h->m;
    const long N = h->N;
    char* V = (char*)h->d_V;
    const size_t vbytes = (size_t)N * h->kelem();
    GB_LAUNCH(launch_step_begin(h->d_ctrl, h->d_H, m, s));
    tick(h, GBPROP_PHASE_OTHER);
    // the fused form hands beta to the next solve and (complex64) reads the split first vector:
    // both only the inverse-band solve provides
    const bool fused = h->cgs_grid > 0 && !dorth && h->inv_ok;
    // the FP32-pair split of a complex64 basis's FP64 first vector, written by the inverse-band
    // solve of that vector: read by both Gram-Schmidt forms instead of the FP64 copy
    float4* v0s = (h->d_v0s && h->inv_ok) ? (float4*)h->d_v0s : nullptr;
    if (fused) GB_CUDA(cudaMemsetAsync(h->d_gridbar, 0, 2 * sizeof(unsigned), s));
    // beta0 = ||x||
    GB_LAUNCH(launch_norm(0, h->d_x, N, h->d_partials, h->d_counter, h->d_ctrl, s));
    tick(h, GBPROP_PHASE_GRAM_SCHMIDT);
    for (int J = 0; J < m; ++J) {
        const void* in = J == 0 ? (const void*)h->d_x : (const void*)h->d_r;
        const int in_prec = J == 0 ? 0 : kp;
        // v_J = r / beta_J stored in V[J] (v_0 of a complex64 basis in FP64); s = U^-1 v_J
        // fused: beta_J comes from the previous Gram-Schmidt launch's ||w||^2 partials (see
        // launch_solve_inv); they follow that launch's J inner-product partials, 16 bytes per
        // (vector, CTA) in both forms (two doubles, or one float4 of FP32 pairs)
        const void* bpart = nullptr;
        if (fused && J > 0) bpart = (const char*)h->d_cgs_part + (size_t)J * h->cgs_grid * 16;
        if (J == 0 && h->d_v0)
            GB_LAUNCH(ksolve(h, 0, in, in_prec, h->d_s, kp, h->d_v0, 0, 1, 1, v0s));
        else
            GB_LAUNCH(ksolve(h, 0, in, in_prec, h->d_s, kp, V + J * vbytes, kp, 1, 1, nullptr, bpart));
        tick(h, GBPROP_PHASE_SOLVE);
        // y = sum_t c_t s_t A_t s
        GB_LAUNCH(launch_band_apply(kp, kop(h), h->d_s, h->d_y, h->d_sched, h->d_ctrl, uniform_scalings(0.0), 1, s));
        tick(h, GBPROP_PHASE_BAND);
        // w = U^-T y
        GB_LAUNCH(ksolve(h, 1, h->d_y, kp, h->d_r, kp, nullptr, kp, 0, 1));
        tick(h, GBPROP_PHASE_SOLVE);
        // classical Gram-Schmidt against v_0..v_J
        if (fused) {
            GB_LAUNCH(launch_arnoldi_cgs(kp, V, h->d_v0s, N, J, m, h->d_r, h->d_cgs_part, h->d_gridbar, h->d_ctrl,
                                         h->d_H, J < m - 1, h->cgs_grid, h->cgs_cache, s));
            tick(h, GBPROP_PHASE_GRAM_SCHMIDT);
            continue;
        }
        GB_LAUNCH(launch_cgs_dot(kp, V, h->d_v0, v0s, N, J + 1, h->d_r, h->d_partials, h->d_counter, h->d_ctrl, 0,
                                 dorth, s));
        // without re-orthogonalisation the update's last block also finalizes the step
        const bool fin = !dorth && J < m - 1;
        if (J < m - 1 || dorth)
            GB_LAUNCH(launch_cgs_update(kp, V, h->d_v0, v0s, N, J + 1, h->d_r, h->d_partials, h->d_counter, h->d_ctrl,
                                        dorth ? 2 : (fin ? 4 : 0), s, h->d_H, m, brk_tol));
        if (dorth) {
            for (int pass = 0; pass < 3; ++pass) {
                GB_LAUNCH(launch_cgs_dot(kp, V, h->d_v0, v0s, N, J + 1, h->d_r, h->d_partials, h->d_counter, h->d_ctrl, 1, 0,
                                         s));
                GB_LAUNCH(launch_cgs_update(kp, V, h->d_v0, v0s, N, J + 1, h->d_r, h->d_partials, h->d_counter, h->d_ctrl, 1,
                                            s));
            }
        }
        if (!fin) GB_LAUNCH(launch_arnoldi_finalize(h->d_ctrl, h->d_H, m, J, dorth, brk_tol, s));
        tick(h, GBPROP_PHASE_GRAM_SCHMIDT);
    }
    return GBPROP_OK;
}

// Enqueue one AdvanceStep on x (PamPropagator.py:50-57 around pamp.h:613-669).
gbprop_status enqueue_step(gbprop_ctx* h) {
    cudaStream_t s = h->stream;
    const int kp = h->kprec();
    const int m = h->m;
    const long N = h->N;
    char* V = (char*)h->d_V;
    if (gbprop_status st = enqueue_arnoldi(h, h->double_orth, std::sqrt(DBL_EPSILON))) return st;   // pamp.h:79
    if (h->expm_method == 1)                               // EigenvectorExponential (pamp.h:567-607)
        GB_LAUNCH(launch_expm_eig(h->d_ctrl, h->d_H, m, h->d_sched, s));
    else                                                   // ScalingPadeExponential (pamp.h:430-564)
        GB_LAUNCH(launch_expm(h->d_ctrl, h->d_H, m, h->d_sched, h->expm_max_cluster, s, h->prec != GBPROP_FP64));
    tick(h, GBPROP_PHASE_EXPONENTIAL);
    // x <- beta0 V exp(-i dt H) e1
    GB_LAUNCH(launch_combine(kp, V, h->d_v0, N, h->d_ctrl, h->d_x, s));
    tick(h, GBPROP_PHASE_COMBINE);
    if (h->renormalize) {
        // Problem.AdvanceStep: psi.Normalize() when renormalization is on (Problem.py:167-168)
        GB_LAUNCH(launch_renormalize(h->d_x, N, h->d_partials, h->d_counter, h->d_ctrl, s));
        tick(h, GBPROP_PHASE_OTHER);
    }
    GB_LAUNCH(launch_step_end(h->d_ctrl, s));
    tick(h, GBPROP_PHASE_OTHER);
    return GBPROP_OK;
}

void drop_graph(gbprop_ctx* h) {
    if (h->graph) {
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    if (h->graph_arnoldi) {
        cudaGraphExecDestroy(h->graph_arnoldi);
        h->graph_arnoldi = nullptr;
    }
}

void set_band_variant(gbprop_ctx* h, int v) {
    h->band_variant = v;
    h->t64.op.variant = v;
    h->t32.op.variant = v;
    drop_graph(h);
}

gbprop_status ensure_graph(gbprop_ctx* h) {
    if (h->graph) return GBPROP_OK;
    cudaGraph_t g = nullptr;
    GB_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const long long before = launch_count();
    gbprop_status st = enqueue_step(h);
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (st) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return fail(GBPROP_ECUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
    h->graph_launches = launch_count() - before;
    // the captured launches did not run; take them off the process counter
    count_launch((int)-h->graph_launches);
    e = cudaGraphInstantiate(&h->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(GBPROP_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    return GBPROP_OK;
}

// Device-side failures (pamp.h:544-550 throws on a singular Pade denominator; here the kernels
// record the failure in the handle's Ctrl flags and carry on without hanging).  After each
// advance the three flags are copied to pinned host memory behind an event; device_errors
// reads them once that event has completed -- without waiting (block = false: a failure is
// reported by the first call after the GPU has finished the failing step) or after waiting
// for it (block = true: synchronize, advance_host, get_stats).  A reported failure is cleared
// on the device so that the handle can be used again.
gbprop_status arm_flags(gbprop_ctx* h) {
    GB_CUDA(cudaMemcpyAsync(h->h_flags, &h->d_ctrl->lu_info, 3 * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    GB_CUDA(cudaEventRecord(h->ev_flags, h->stream));
    h->flags_armed = true;
    return GBPROP_OK;
}

gbprop_status report_flags(gbprop_ctx* h, int lu, int nonfinite, int timeout) {
    if (!lu && !nonfinite && !timeout) return GBPROP_OK;
    GB_CUDA(cudaMemsetAsync(&h->d_ctrl->lu_info, 0, 3 * sizeof(int), h->stream));
    // the first cause: a wait that gave up leaves stale data behind it; a failed Pade solve
    // leaves the step's exponential undefined, so later norms turn non-finite (the kernels
    // record no LU failure for a Hessenberg matrix that was non-finite already)
    if (timeout) return fail(GBPROP_ETIMEOUT, "a bounded device-side wait gave up (bulk-copy staging or grid barrier)");
    if (lu) return fail(GBPROP_ELU, "Pade denominator singular (LU info " + std::to_string(lu) + ")");
    return fail(GBPROP_ENONFINITE, "non-finite Krylov norm or Hessenberg matrix");
}

gbprop_status device_errors(gbprop_ctx* h, bool block) {
    if (!h->flags_armed) return GBPROP_OK;
    cudaError_t e = block ? cudaEventSynchronize(h->ev_flags) : cudaEventQuery(h->ev_flags);
    if (e == cudaErrorNotReady) return GBPROP_OK;
    if (e != cudaSuccess) return fail(GBPROP_ECUDA, std::string("flag event: ") + cudaGetErrorString(e));
    h->flags_armed = false;
    return report_flags(h, h->h_flags[0], h->h_flags[1], h->h_flags[2]);
}

gbprop_status ensure_sched(gbprop_ctx* h, int n) {
    if (n <= h->sched_cap) return GBPROP_OK;
    // the schedule pointer is baked into the graph: grow by re-allocation and re-capture
    int cap = std::max(n, std::max(1024, 2 * h->sched_cap));
    SchedEntry* p = nullptr;
    GB_CUDA(cudaStreamSynchronize(h->stream));
    gbprop_status st = h->dalloc(&p, (size_t)cap * sizeof(SchedEntry));
    if (st) return st;
    h->d_sched = p;
    h->sched_cap = cap;
    drop_graph(h);
    return GBPROP_OK;
}

}  // namespace

extern "C" {

const char* gbprop_version(void) { return "gbprop 0.1 (sm_103a)"; }
const char* gbprop_last_error(void) { return t_err.c_str(); }
long long gbprop_launch_count(void) { return launch_count(); }

gbprop_status gbprop_create(gbprop_handle* out, int nl, int nr, int precision, int krylov_basis_size,
                            int exponentiation_method, int double_orthogonalization, void* stream) {
    if (!out) return fail(GBPROP_EINVAL, "null output pointer");
    *out = nullptr;
    if (nl <= 0 || nr <= 0) return fail(GBPROP_EINVAL, "nl and nr must be positive");
    if (nr > 4096) return fail(GBPROP_EUNSUPPORTED, "radial size above 4096 (one angular row must fit a CTA's shared memory)");
    if (precision != GBPROP_FP64 && precision != GBPROP_FP32_MIXED) return fail(GBPROP_EINVAL, "unknown precision");
    if (krylov_basis_size < 1 || krylov_basis_size > kMaxBasis)
        return fail(GBPROP_EINVAL, "krylov_basis_size must be in [1, 45]");
    if (exponentiation_method != 0 && exponentiation_method != 1)
        return fail(GBPROP_EINVAL, "krylov_exponentiation_method must be 0 (Pade) or 1 (eigenvector)");
    gbprop_ctx* h = new gbprop_ctx();
    h->nl = nl;
    h->nr = nr;
    h->N = (long)nl * nr;
    h->prec = precision;
    h->m = krylov_basis_size;
    h->expm_method = exponentiation_method;
    h->double_orth = double_orthogonalization ? 1 : 0;
    h->ustream = (cudaStream_t)stream;
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_in, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_out, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_flags, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&h->h_flags, 3 * sizeof(int));
    if (e != cudaSuccess) {
        delete h;
        return fail(GBPROP_ECUDA, std::string("stream/event creation: ") + cudaGetErrorString(e));
    }
    *out = h;
    return GBPROP_OK;
}

gbprop_status gbprop_destroy(gbprop_handle h) {
    if (!h) return GBPROP_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    delete h;
    return GBPROP_OK;
}

gbprop_status gbprop_set_overlap(gbprop_handle h, int kd, const double* U_band) {
    if (gbprop_status st = check_handle(h, false)) return st;
    if (h->finalized) return fail(GBPROP_EINVAL, "handle already finalized");
    if (kd < 1 || kd > kMaxKd) return fail(GBPROP_EUNSUPPORTED, "overlap band half-width must be in [1, 8]");
    if (!U_band) return fail(GBPROP_EINVAL, "null overlap factor");
    if (h->nr < kd + 1) return fail(GBPROP_EINVAL, "radial size smaller than the overlap band");
    h->kd = kd;
    h->U.assign(U_band, U_band + (size_t)h->nr * (kd + 1));
    for (int i = 0; i < h->nr; ++i)
        if (!(uval(h->U, h->nr, kd, i, i) != 0.0)) return fail(GBPROP_EINVAL, "zero on the overlap factor diagonal");
    return GBPROP_OK;
}

gbprop_status gbprop_add_potential(gbprop_handle h, int storage, int npairs, const int* pairs, int kb,
                                   const double* data, int time_dependent) {
    if (gbprop_status st = check_handle(h, false)) return st;
    if (h->finalized) return fail(GBPROP_EINVAL, "handle already finalized");
    if (storage != GBPROP_STORAGE_DIAG && storage != GBPROP_STORAGE_IDENT && storage != GBPROP_STORAGE_SIMP)
        return fail(GBPROP_EUNSUPPORTED, "angular storage must be Diag, Ident or Simp");
    if (kb < 1 || kb > kMaxKd) return fail(GBPROP_EUNSUPPORTED, "radial band half-width must be in [1, 8]");
    if (h->kb >= 0 && kb != h->kb) return fail(GBPROP_EUNSUPPORTED, "all potentials must share one radial band width");
    if (!data) return fail(GBPROP_EINVAL, "null potential data");
    if (time_dependent < 0 || time_dependent > kMaxTimeFuncs)
        return fail(GBPROP_EUNSUPPORTED, "time_dependent must be 0 (static) or a time function number 1.." +
                                         std::to_string(kMaxTimeFuncs));
    if (storage == GBPROP_STORAGE_DIAG && npairs != h->nl) return fail(GBPROP_EINVAL, "Diag storage needs npairs == nl");
    if (storage == GBPROP_STORAGE_IDENT && npairs != 1) return fail(GBPROP_EINVAL, "Ident storage needs npairs == 1");
    if (storage == GBPROP_STORAGE_SIMP) {
        if (!pairs || npairs < 0) return fail(GBPROP_EINVAL, "Simp storage needs a pair table");
        for (int q = 0; q < npairs; ++q)
            if (pairs[2 * q] < 0 || pairs[2 * q] >= h->nl || pairs[2 * q + 1] < 0 || pairs[2 * q + 1] >= h->nl)
                return fail(GBPROP_EINVAL, "angular pair index out of range");
    }
    HostPot p;
    p.storage = storage;
    p.npairs = npairs;
    if (storage == GBPROP_STORAGE_SIMP) p.pairs.assign(pairs, pairs + 2 * (size_t)npairs);
    p.kb = kb;
    p.data.assign(data, data + (size_t)npairs * (2 * kb + 1) * h->nr * 2);
    p.timedep = time_dependent;
    h->nfuncs = std::max(h->nfuncs, time_dependent);
    h->kb = kb;
    h->pots.push_back(std::move(p));
    return GBPROP_OK;
}

gbprop_status gbprop_finalize(gbprop_handle h) {
    if (gbprop_status st = check_handle(h, false)) return st;
    if (h->finalized) return GBPROP_OK;
    if (h->kd < 0) return fail(GBPROP_EINVAL, "overlap factor not set");
    if (h->kb < 0) h->kb = h->kd;
    gbprop_status st;
    // solve tables: FP64 always (state transforms), FP32 for the mixed Krylov basis
    for (int dir = 0; dir < 2; ++dir) {
        HostSolveTab ht = build_solve_tab(h->U, h->nr, h->kd, dir);
        if ((st = upload_solve_tab<float>(h, ht, &h->t32.tab[dir]))) return st;
    }
    // banded approximate inverse (both directions); the block solve remains for factors
    // whose inverse decays too slowly.  GBPROP_SOLVER=block selects the block solve.
    {
        const char* env = std::getenv("GBPROP_SOLVER");
        bool use_inv = !(env && std::strcmp(env, "block") == 0);
        HostInvTab hi[2];
        for (int dir = 0; dir < 2 && use_inv; ++dir) {
            hi[dir] = build_inv_tab(h->U, h->nr, h->kd, dir);
            if (!hi[dir].ok) use_inv = false;
        }
        if (use_inv) {
            for (int dir = 0; dir < 2; ++dir) {
                InvTab& t = h->inv[dir];
                t.n = h->nr;
                t.kd = h->kd;
                t.w = hi[dir].w;
                t.npad = hi[dir].npad;
                t.refine = std::max(hi[0].refine, hi[1].refine);
                float *dm, *duh, *dul;
                double* du;
                std::vector<float> uh(hi[dir].u.size()), ul(hi[dir].u.size());
                for (size_t k = 0; k < uh.size(); ++k) {
                    uh[k] = (float)hi[dir].u[k];
                    ul[k] = (float)(hi[dir].u[k] - (double)uh[k]);
                }
                if ((st = h->upload(&dm, hi[dir].m))) return st;
                if ((st = h->upload(&du, hi[dir].u))) return st;
                if ((st = h->upload(&duh, uh))) return st;
                if ((st = h->upload(&dul, ul))) return st;
                t.m = dm;
                t.u = du;
                t.uh = duh;
                t.ul = dul;
            }
            set_inv_chunks(h, true);
            h->inv_ok = true;
        }
    }
    HostBandOp ho = build_band_op(h);
    if (h->prec == GBPROP_FP64) {
        if ((st = upload_band_op<double>(h, ho, &h->t64.op))) return st;
    } else {
        if ((st = upload_band_op<float>(h, ho, &h->t32.op))) return st;
    }
    std::vector<double> udp((size_t)(h->kd + 1) * h->nr, 0.0);
    for (int d = 0; d <= h->kd; ++d)
        for (int i = 0; i + d < h->nr; ++i) udp[(size_t)d * h->nr + i] = uval(h->U, h->nr, h->kd, i, i + d);
    if ((st = h->upload(&h->d_ud_phys, udp))) return st;
    if ((st = h->dalloc(&h->d_ctrl, sizeof(Ctrl)))) return st;
    GB_CUDA(cudaMemsetAsync(h->d_ctrl, 0, sizeof(Ctrl), h->stream));
    if ((st = h->dalloc(&h->d_H, (size_t)2 * h->m * h->m * sizeof(double)))) return st;
    GB_CUDA(cudaMemsetAsync(h->d_H, 0, (size_t)2 * h->m * h->m * sizeof(double), h->stream));
    if ((st = h->dalloc(&h->d_partials, partials_capacity() * sizeof(double)))) return st;
    if ((st = h->dalloc(&h->d_counter, 64))) return st;
    GB_CUDA(cudaMemsetAsync(h->d_counter, 0, 64, h->stream));
    const size_t ke = h->kelem();
    if ((st = h->dalloc(&h->d_V, (size_t)h->m * h->N * ke))) return st;
    GB_CUDA(cudaMemsetAsync(h->d_V, 0, (size_t)h->m * h->N * ke, h->stream));
    if ((st = h->dalloc(&h->d_r, (size_t)h->N * ke))) return st;
    if ((st = h->dalloc(&h->d_s, (size_t)h->N * ke))) return st;
    if ((st = h->dalloc(&h->d_y, (size_t)h->N * ke))) return st;
    if ((st = h->dalloc(&h->d_x, (size_t)h->N * sizeof(double2)))) return st;
    if (h->prec != GBPROP_FP64 && (st = h->dalloc(&h->d_v0, (size_t)h->N * sizeof(double2)))) return st;
    if (h->prec != GBPROP_FP64 && (st = h->dalloc(&h->d_v0s, (size_t)h->N * sizeof(float4)))) return st;
    // cooperative Gram-Schmidt (single handles; GBPROP_CGS=separate keeps the three-kernel form)
    {
        const char* env = std::getenv("GBPROP_CGS");
        const bool allow = !(env && std::strcmp(env, "separate") == 0) && !h->double_orth;
        const int kpv = h->kprec(), with_v0 = h->d_v0 != nullptr;
        int grid = allow ? arnoldi_cgs_grid(kpv, h->N, h->m, with_v0, 1) : 0;
        int cache = 1;
        if (allow && grid == 0) {
            grid = arnoldi_cgs_grid(kpv, h->N, h->m, with_v0, 0);
            cache = 0;
        }
        cudaGetLastError();
        if (grid > 0) {
            if ((st = h->dalloc(&h->d_cgs_part, arnoldi_cgs_part_doubles(grid) * sizeof(double)))) return st;
            h->cgs_part_grid = grid;
            if ((st = h->dalloc(&h->d_gridbar, 64))) return st;
            GB_CUDA(cudaMemsetAsync(h->d_gridbar, 0, 64, h->stream));
            h->cgs_grid = grid;
            h->cgs_cache = cache;
        }
    }
    if ((st = ensure_sched(h, 1024))) return st;
    GB_CUDA(cudaStreamSynchronize(h->stream));
    h->finalized = true;
    return GBPROP_OK;
}

gbprop_status gbprop_advance(gbprop_handle h, void* psi, int nsteps, const double* scalings, double dt_re,
                             double dt_im) {
    if (gbprop_status st = check_handle(h, true)) return st;
    if (!psi) return fail(GBPROP_EINVAL, "null wavefunction");
    if (nsteps < 0) return fail(GBPROP_EINVAL, "negative step count");
    if (nsteps == 0) return GBPROP_OK;
    if (!scalings) return fail(GBPROP_EINVAL, "null scaling schedule");
    gbprop_status st;
    if ((st = device_errors(h, false))) return st;      // a failure of an earlier call, if known by now
    GB_CUDA(h->begin());
    if ((st = enqueue_enter(h, psi, h->stream))) return st;
    // steps are issued in chunks of the schedule capacity
    int done = 0;
    while (done < nsteps) {
        const int chunk = std::min(nsteps - done, std::max(h->sched_cap, 1024));
        if ((st = ensure_sched(h, chunk))) return st;
        std::vector<SchedEntry> sched(chunk);
        for (int k = 0; k < chunk; ++k) sched[k] = sched_entry(scalings + (size_t)(done + k) * h->nfuncs, h->nfuncs, dt_re, dt_im);
        // pageable source: staged before the call returns, so `sched` may go out of scope
        GB_CUDA(cudaMemcpyAsync(h->d_sched, sched.data(), chunk * sizeof(SchedEntry), cudaMemcpyHostToDevice, h->stream));
        GB_CUDA(cudaMemsetAsync(&h->d_ctrl->step, 0, sizeof(int), h->stream));
        if ((st = ensure_graph(h))) return st;
        for (int k = 0; k < chunk; ++k) {
            GB_CUDA(cudaGraphLaunch(h->graph, h->stream));
            count_launch((int)h->graph_launches);
        }
        done += chunk;
    }
    if ((st = enqueue_leave(h, psi, h->stream))) return st;
    if ((st = arm_flags(h))) return st;
    GB_CUDA(h->end());
    return GBPROP_OK;
}

gbprop_status gbprop_advance_host(gbprop_handle h, void* psi_host, int nsteps, const double* scalings, double dt_re,
                                  double dt_im) {
    if (gbprop_status st = check_handle(h, true)) return st;
    if (!psi_host) return fail(GBPROP_EINVAL, "null wavefunction");
    const size_t bytes = (size_t)h->N * (h->prec == GBPROP_FP64 ? sizeof(double2) : sizeof(float2));
    if (!h->d_host_stage) {
        gbprop_status st = h->dalloc(&h->d_host_stage, bytes);
        if (st) return st;
    }
    void* d = h->d_host_stage;
    GB_CUDA(cudaMemcpyAsync(d, psi_host, bytes, cudaMemcpyHostToDevice, h->ustream));
    gbprop_status st = gbprop_advance(h, d, nsteps, scalings, dt_re, dt_im);
    if (st) return st;
    GB_CUDA(cudaMemcpyAsync(psi_host, d, bytes, cudaMemcpyDeviceToHost, h->ustream));
    GB_CUDA(cudaStreamSynchronize(h->ustream));
    return device_errors(h, true);
}

gbprop_status gbprop_matvec(gbprop_handle h, const void* src, void* dst, double scaling, int balanced) {
    if (gbprop_status st = check_handle(h, true)) return st;
    std::vector<double> v(h->nfuncs, scaling);
    return gbprop_matvec_scalings(h, src, dst, v.data(), balanced);
}

gbprop_status gbprop_matvec_scalings(gbprop_handle h, const void* src, void* dst, const double* scalings,
                                     int balanced) {
    if (gbprop_status st = check_handle(h, true)) return st;
    if (!src || !dst || !scalings) return fail(GBPROP_EINVAL, "null argument");
    Scalings scaling = uniform_scalings(0.0);
    for (int k = 0; k < h->nfuncs; ++k) scaling.s[k] = scalings[k];
    if (src == dst) return fail(GBPROP_EINVAL, "src and dst must differ");
    const int kp = h->kprec();
    cudaStream_t s = h->stream;
    GB_CUDA(h->begin());
    if (balanced) {
        GB_LAUNCH(ksolve(h, 0, src, kp, h->d_s, kp, nullptr, kp, 0, 0));
        GB_LAUNCH(launch_band_apply(kp, kop(h), h->d_s, h->d_y, nullptr, h->d_ctrl, scaling, 0, s));
        GB_LAUNCH(ksolve(h, 1, h->d_y, kp, dst, kp, nullptr, kp, 0, 0));
    } else {
        GB_LAUNCH(launch_band_apply(kp, kop(h), src, dst, nullptr, h->d_ctrl, scaling, 0, s));
    }
    GB_CUDA(h->end());
    return GBPROP_OK;
}

gbprop_status gbprop_set_renormalization(gbprop_handle h, int on) {
    if (gbprop_status st = check_handle(h, false)) return st;
    if ((on != 0) != (h->renormalize != 0)) {
        h->renormalize = on ? 1 : 0;
        drop_graph(h);
    }
    return GBPROP_OK;
}

gbprop_status gbprop_inner_product(gbprop_handle h, const void* a, const void* b, double* out) {
    if (gbprop_status st = check_handle(h, true)) return st;
    if (!a || !b || !out) return fail(GBPROP_EINVAL, "null argument");
    if (gbprop_status st = device_errors(h, false)) return st;
    const long N = h->N;
    if (!h->d_ip)
        if (gbprop_status st = h->dalloc(&h->d_ip, (size_t)2 * N * sizeof(double2) + 4 * sizeof(double))) return st;
    const int kp = h->kprec();
    double* d_out = reinterpret_cast<double*>(h->d_ip + 2 * N);
    GB_CUDA(h->begin());
    GB_LAUNCH(launch_tbmv(0, h->kd, h->d_ud_phys, h->nl, h->nr, a, kp, h->d_ip, 0, h->stream));
    GB_LAUNCH(launch_tbmv(0, h->kd, h->d_ud_phys, h->nl, h->nr, b, kp, h->d_ip + N, 0, h->stream));
    GB_LAUNCH(launch_block_inner(0, h->d_ip, N, 1, h->d_ip + N, 0, d_out, h->d_partials, h->d_counter, h->stream));
    GB_CUDA(cudaMemcpyAsync(out, d_out, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    GB_CUDA(cudaStreamSynchronize(h->stream));
    GB_CUDA(h->end());
    return GBPROP_OK;
}

gbprop_status gbprop_multiply_sqrt_overlap(gbprop_handle h, void* psi) {
    if (gbprop_status st = check_handle(h, true)) return st;
    if (!psi) return fail(GBPROP_EINVAL, "null wavefunction");
    const int kp = h->kprec();
    GB_CUDA(h->begin());
    GB_LAUNCH(launch_tbmv(0, h->kd, h->d_ud_phys, h->nl, h->nr, psi, kp, h->d_r, kp, h->stream));
    GB_CUDA(cudaMemcpyAsync(psi, h->d_r, (size_t)h->N * h->kelem(), cudaMemcpyDeviceToDevice, h->stream));
    GB_CUDA(h->end());
    return GBPROP_OK;
}

gbprop_status gbprop_solve_sqrt_overlap(gbprop_handle h, int conj, void* psi) {
    if (gbprop_status st = check_handle(h, true)) return st;
    if (!psi) return fail(GBPROP_EINVAL, "null wavefunction");
    const int kp = h->kprec();
    GB_CUDA(h->begin());
    GB_LAUNCH(ssolve(h, conj ? 1 : 0, psi, kp, psi, kp));
    GB_CUDA(h->end());
    return GBPROP_OK;
}

gbprop_status gbprop_get_stats(gbprop_handle h, gbprop_stats* out) {
    if (gbprop_status st = check_handle(h, true)) return st;
    if (!out) return fail(GBPROP_EINVAL, "null output");
    Ctrl c;
    GB_CUDA(cudaMemcpyAsync(&c, h->d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->stream));
    GB_CUDA(cudaStreamSynchronize(h->stream));
    out->operator_count = c.operator_count;
    out->inner_product_count = c.inner_product_count;
    out->orthogonalization_count = c.orthogonalization_count;
    out->breakdown_count = c.breakdown_count;
    out->step_count = c.step_count;
    out->last_basis_size = c.nbasis;
    out->last_scaling_order = c.scaling_order;
    out->error_estimate = c.err_est;
    h->flags_armed = false;                             // the copy above is newer than any armed one
    return report_flags(h, c.lu_info, c.nonfinite, c.wait_timeout);
}

gbprop_status gbprop_reset_stats(gbprop_handle h) {
    if (gbprop_status st = check_handle(h, true)) return st;
    // counters and error flags only: the host-set fields (wait_limit, inject_lu) stay
    GB_CUDA(cudaMemsetAsync(h->d_ctrl, 0, offsetof(Ctrl, inject_lu), h->stream));
    GB_CUDA(cudaMemsetAsync(&h->d_ctrl->ro_go, 0, sizeof(Ctrl) - offsetof(Ctrl, ro_go), h->stream));
    GB_CUDA(cudaStreamSynchronize(h->stream));
    h->flags_armed = false;
    return GBPROP_OK;
}

gbprop_status gbprop_get_hessenberg(gbprop_handle h, double* out) {
    if (gbprop_status st = check_handle(h, true)) return st;
    if (!out) return fail(GBPROP_EINVAL, "null output");
    GB_CUDA(cudaMemcpyAsync(out, h->d_H, (size_t)2 * h->m * h->m * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    GB_CUDA(cudaStreamSynchronize(h->stream));
    return GBPROP_OK;
}

gbprop_status gbprop_synchronize(gbprop_handle h) {
    if (gbprop_status st = check_handle(h, false)) return st;
    GB_CUDA(cudaStreamSynchronize(h->stream));
    GB_CUDA(cudaStreamSynchronize(h->ustream));
    return device_errors(h, true);
}

gbprop_status gbprop_time_step(gbprop_handle h, void* psi, const double* scalings, double dt_re, double dt_im,
                               gbprop_step_timers* out) {
    if (gbprop_status st = check_handle(h, true)) return st;
    if (!psi || !out || !scalings) return fail(GBPROP_EINVAL, "null argument");
    if (gbprop_status st = device_errors(h, false)) return st;
    if (h->tick_pool.empty()) {
        h->tick_pool.resize(4 * kMaxBasis * 8 + 64, nullptr);
        for (cudaEvent_t& e : h->tick_pool) GB_CUDA(cudaEventCreate(&e));
    }
    gbprop_status st;
    if ((st = ensure_sched(h, 1))) return st;
    SchedEntry se = sched_entry(scalings, h->nfuncs, dt_re, dt_im);
    GB_CUDA(h->begin());
    GB_CUDA(cudaMemcpyAsync(h->d_sched, &se, sizeof(se), cudaMemcpyHostToDevice, h->stream));
    GB_CUDA(cudaMemsetAsync(&h->d_ctrl->step, 0, sizeof(int), h->stream));
    std::vector<std::pair<int, cudaEvent_t>> ticks;
    cudaEvent_t start = h->tick_pool.back();
    GB_CUDA(cudaEventRecord(start, h->stream));
    h->timing = &ticks;
    const long long before = launch_count();
    st = enqueue_enter(h, psi, h->stream);
    if (!st) st = enqueue_step(h);
    if (!st) st = enqueue_leave(h, psi, h->stream);
    h->timing = nullptr;
    if (st) return st;
    if ((st = arm_flags(h))) return st;
    GB_CUDA(h->end());
    GB_CUDA(cudaStreamSynchronize(h->stream));
    std::memset(out, 0, sizeof(*out));
    out->launches = launch_count() - before;
    cudaEvent_t prev = start;
    for (const auto& t : ticks) {
        float ms = 0.f;
        GB_CUDA(cudaEventElapsedTime(&ms, prev, t.second));
        out->ms[t.first] += ms;
        out->count[t.first] += 1;
        out->total_ms += ms;
        prev = t.second;
    }
    return device_errors(h, true);
}

gbprop_status gbprop_debug_expm(gbprop_handle h, const double* H, double dt_re, double dt_im, int form, double* y,
                                int* scaling_order) {
    if (gbprop_status st = check_handle(h, true)) return st;
    if (!H || !y) return fail(GBPROP_EINVAL, "null argument");
    if (form < 0 || form > 2) return fail(GBPROP_EINVAL, "form: 0 FP64 Pade, 1 double-float Pade, 2 eigenvector");
    const int m = h->m;
    gbprop_status st;
    if ((st = ensure_sched(h, 1))) return st;
    const double zero[kMaxTimeFuncs] = {0.0, 0.0, 0.0, 0.0};
    SchedEntry se = sched_entry(zero, h->nfuncs, dt_re, dt_im);
    cudaStream_t s = h->stream;
    GB_CUDA(cudaMemcpyAsync(h->d_sched, &se, sizeof(se), cudaMemcpyHostToDevice, s));
    GB_CUDA(cudaMemsetAsync(&h->d_ctrl->step, 0, sizeof(int), s));
    GB_CUDA(cudaMemcpyAsync(h->d_H, H, (size_t)2 * m * m * sizeof(double), cudaMemcpyHostToDevice, s));
    if (form == 2) GB_LAUNCH(launch_expm_eig(h->d_ctrl, h->d_H, m, h->d_sched, s));
    else GB_LAUNCH(launch_expm(h->d_ctrl, h->d_H, m, h->d_sched, h->expm_max_cluster, s, form));
    int so = 0;
    GB_CUDA(cudaMemcpyAsync(y, h->d_ctrl->y, (size_t)2 * m * sizeof(double), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaMemcpyAsync(&so, &h->d_ctrl->scaling_order, sizeof(int), cudaMemcpyDeviceToHost, s));
    GB_CUDA(cudaStreamSynchronize(s));
    if (scaling_order) *scaling_order = so;
    return device_errors(h, true);
}

gbprop_status gbprop_debug_set(gbprop_handle h, int key, long long value) {
    if (gbprop_status st = check_handle(h, true)) return st;
    if (key == GBPROP_DEBUG_WAIT_LIMIT) {
        GB_CUDA(cudaMemcpyAsync(&h->d_ctrl->wait_limit, &value, sizeof(long long), cudaMemcpyHostToDevice, h->stream));
    } else if (key == GBPROP_DEBUG_INJECT_LU) {
        const int v = value ? 1 : 0;
        GB_CUDA(cudaMemcpyAsync(&h->d_ctrl->inject_lu, &v, sizeof(int), cudaMemcpyHostToDevice, h->stream));
    } else if (key == GBPROP_DEBUG_ROUND_MATVEC) {
        const int v = (int)(value & 3);
        GB_CUDA(cudaMemcpyAsync(&h->d_ctrl->round_matvec, &v, sizeof(int), cudaMemcpyHostToDevice, h->stream));
    } else {
        return fail(GBPROP_EINVAL, "unknown debug key");
    }
    GB_CUDA(cudaStreamSynchronize(h->stream));
    return GBPROP_OK;
}

gbprop_status gbprop_tensor_multiply_bandnh(int storage, const void* V, int npairs, const int* pairs, int kb,
                                            double scaling, const void* src, void* dst, int nl, int nr, void* stream) {
    if (storage != GBPROP_STORAGE_DIAG && storage != GBPROP_STORAGE_SIMP)
        return fail(GBPROP_EUNSUPPORTED, "stateless multiply supports Diag and Simp angular storage");
    if (!V || !src || !dst) return fail(GBPROP_EINVAL, "null buffer");
    if (storage == GBPROP_STORAGE_SIMP && (!pairs || npairs < 0)) return fail(GBPROP_EINVAL, "Simp needs pairs");
    if (nl <= 0 || nr <= 0 || kb < 0) return fail(GBPROP_EINVAL, "bad sizes");
    GB_LAUNCH(launch_tensor_multiply_ref(storage == GBPROP_STORAGE_DIAG ? 0 : 1, (const double2*)V, npairs, pairs, kb,
                                         scaling, (const double2*)src, (double2*)dst, nl, nr, (cudaStream_t)stream));
    return GBPROP_OK;
}

// Variants 6, 7 and 8 (two elements per thread, vector loads) need an even radial size.
bool band_variant_available(const gbprop_ctx* h, int v) {
    if (v < 0 || v >= band_variant_count()) return false;
    if (v < 6) return true;
    if (!band_variant_vec_ok(v, h->nr)) return false;
    return h->kprec() == 0 || h->t32.op.slots_lo != nullptr;
}

gbprop_status gbprop_autotune(gbprop_handle h, int* variant) {
    if (gbprop_status st = check_handle(h, true)) return st;
    if (variant && *variant >= 0) {                  // explicit choice, no timing
        if (!band_variant_available(h, *variant)) return fail(GBPROP_EINVAL, "no such band-kernel variant");
        set_band_variant(h, *variant);
        return GBPROP_OK;
    }
    const int kp = h->kprec();
    cudaStream_t s = h->stream;
    cudaEvent_t e0, e1;
    GB_CUDA(cudaEventCreate(&e0));
    GB_CUDA(cudaEventCreate(&e1));
    GB_CUDA(cudaMemsetAsync(h->d_s, 0, (size_t)h->N * h->kelem(), s));
    int best = h->band_variant;
    float best_ms = 1e30f;
    // GBPROP_BAND_VARIANT=v and GBPROP_SOLVE_CHUNKS=n0,n1 pin the choices instead of timing them
    // (a profiler's serialised launches time differently from a live run)
    const char* env_v = std::getenv("GBPROP_BAND_VARIANT");
    const int pin_v = env_v ? std::atoi(env_v) : -1;
    int pin_c[2] = {0, 0};
    if (const char* env_c = std::getenv("GBPROP_SOLVE_CHUNKS")) std::sscanf(env_c, "%d,%d", &pin_c[0], &pin_c[1]);
    const bool pinned = band_variant_available(h, pin_v);
    if (pinned) best = pin_v;
    for (int v = 0; v < band_variant_count() && !pinned; ++v) {
        if (!band_variant_available(h, v)) continue;
        h->t64.op.variant = v;
        h->t32.op.variant = v;
        for (int k = 0; k < 3; ++k)
            GB_LAUNCH(launch_band_apply(kp, kop(h), h->d_s, h->d_y, nullptr, h->d_ctrl, uniform_scalings(1.0), 0, s));
        GB_CUDA(cudaEventRecord(e0, s));
        for (int k = 0; k < 10; ++k)
            GB_LAUNCH(launch_band_apply(kp, kop(h), h->d_s, h->d_y, nullptr, h->d_ctrl, uniform_scalings(1.0), 0, s));
        GB_CUDA(cudaEventRecord(e1, s));
        GB_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        GB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) { best_ms = ms; best = v; }
    }
    // radial chunking of the overlap-factor solves (one problem spread over the GPU): time the
    // Krylov-precision solve of each direction for 1..8 chunks and keep the fastest (batches keep
    // the fewest chunks, other problems fill the GPU)
    if (h->inv_ok && h->expm_max_cluster > 1) {
        // finite non-zero input (0x3f bytes): a zero right-hand side ends the refinement early
        GB_CUDA(cudaMemsetAsync(h->d_s, 0x3f, (size_t)h->N * h->kelem(), s));
        for (int dir = 0; dir < 2; ++dir) {
            const InvTab keep = h->inv[dir];
            if (pin_c[dir] > 0) {
                if (!set_inv_chunk_count(h, dir, pin_c[dir])) h->inv[dir] = keep;
                continue;
            }
            InvTab best_t = keep;
            float best_s = 1e30f;
            for (int nch = 1; nch <= 8; ++nch) {
                if (nch > 1 && (h->nr + nch - 1) / nch < 32) break;
                if (!set_inv_chunk_count(h, dir, nch)) continue;
                for (int k = 0; k < 3; ++k) GB_LAUNCH(ksolve(h, dir, h->d_s, kp, h->d_y, kp, nullptr, kp, 0, 0));
                GB_CUDA(cudaEventRecord(e0, s));
                for (int k = 0; k < 10; ++k) GB_LAUNCH(ksolve(h, dir, h->d_s, kp, h->d_y, kp, nullptr, kp, 0, 0));
                GB_CUDA(cudaEventRecord(e1, s));
                GB_CUDA(cudaEventSynchronize(e1));
                float ms = 0.f;
                GB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                if (ms < best_s) { best_s = ms; best_t = h->inv[dir]; }
            }
            h->inv[dir] = best_t;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    set_band_variant(h, best);
    if (variant) *variant = best;
    return GBPROP_OK;
}

gbprop_status gbprop_bound_states(int nr, int kd, int nrows, const double* h_bands, const double* s_band, double emax,
                                  int max_states, int* counts, double* energies, double* vectors, void* stream) {
    if (nr < 1 || kd < 1 || kd > 8 || nrows < 1 || max_states < 1)
        return fail(GBPROP_EINVAL, "bound states: sizes (nr >= 1, 1 <= kd <= 8, nrows >= 1, max_states >= 1)");
    if (!h_bands || !s_band || !counts || !energies || !vectors) return fail(GBPROP_EINVAL, "null argument");
    if (!(emax == emax)) return fail(GBPROP_EINVAL, "emax is NaN");
    int nt = 0;
    cudaError_t e = launch_bound_states(h_bands, s_band, nr, kd, nrows, emax, max_states, counts, energies, vectors,
                                        (cudaStream_t)stream, &nt);
    if (e != cudaSuccess) return fail(GBPROP_ECUDA, std::string("bound states: ") + cudaGetErrorString(e));
    return GBPROP_OK;
}

gbprop_status gbprop_get_tuning(gbprop_handle h, int* band_variant, int* solve_chunks) {
    if (gbprop_status st = check_handle(h, true)) return st;
    if (band_variant) *band_variant = h->band_variant;
    if (solve_chunks) {
        solve_chunks[0] = h->inv_ok ? h->inv[0].nchunks : 0;
        solve_chunks[1] = h->inv_ok ? h->inv[1].nchunks : 0;
    }
    return GBPROP_OK;
}

size_t gbprop_block_inner_product_workspace(long n, int nv) {
    if (n <= 0 || nv < 1 || nv > kMaxBasis) return 0;
    // partial sums (the launch shape depends on whether ||w||^2 is requested: size for
    // the larger of the two), then one 256-byte aligned counter word
    const size_t a = block_inner_scratch_doubles(n, nv), b = block_inner_scratch_doubles(n, nv + 1);
    const size_t sums = (a > b ? a : b) * sizeof(double);
    return ((sums + 255) / 256) * 256 + 256;
}

gbprop_status gbprop_block_inner_product(int precision, const void* V, long n, int nv, const void* w, int want_norm,
                                         double* out, void* workspace, size_t workspace_bytes, void* stream) {
    if (precision != GBPROP_FP64 && precision != GBPROP_FP32_MIXED) return fail(GBPROP_EINVAL, "unknown precision");
    if (n <= 0 || nv < 1 || nv > kMaxBasis) return fail(GBPROP_EINVAL, "need n > 0 and 1 <= nv <= 45");
    if (!V || !w || !out || !workspace) return fail(GBPROP_EINVAL, "null buffer");
    const size_t need = gbprop_block_inner_product_workspace(n, nv);
    if (workspace_bytes < need)
        return fail(GBPROP_EINVAL, "workspace too small: need " + std::to_string(need) + " bytes");
    const size_t sums = need - 256;
    double* partials = (double*)workspace;
    unsigned* counter = (unsigned*)((char*)workspace + sums);
    cudaStream_t s = (cudaStream_t)stream;
    GB_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned), s));
    GB_LAUNCH(launch_block_inner(precision == GBPROP_FP64 ? 0 : 1, V, n, nv, w, want_norm ? 1 : 0, out, partials,
                                 counter, s));
    return GBPROP_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Expokit driver (ExpokitPropagator: adaptive Krylov sub-steps with local error control)
// ---------------------------------------------------------------------------
namespace {

using cplx = std::complex<double>;

// exp(t H) of an n x n complex matrix (row-major) by the diagonal Pade (6,6) approximant with
// scaling and squaring, in the form of Expokit's zgpadm (Sidje 1998): s = max(0,
// floor(log2 ||tH||_inf) + 2), Horner in (tH/2^s)^2 alternating the two polynomials, the odd
// one times tH/2^s, E = I + 2 (Q - P)^-1 P (negated when s = 0 and the parity is odd), then
// s squarings.  Returns false when the denominator is singular.
bool expokit_pade(const std::vector<cplx>& H, int n, double t, std::vector<cplx>& E) {
    const int p = 6;
    double hn = 0.0;
    for (int i = 0; i < n; ++i) {
        double r = 0.0;
        for (int j = 0; j < n; ++j) r += std::abs(H[(size_t)i * n + j]);
        hn = std::max(hn, r);
    }
    hn = std::fabs(t * hn);
    if (hn == 0.0) {
        E.assign((size_t)n * n, cplx(0.0));
        for (int i = 0; i < n; ++i) E[(size_t)i * n + i] = 1.0;
        return true;
    }
    const int ns = std::max(0, (int)(std::log(hn) / std::log(2.0)) + 2);
    const double sc = t / std::ldexp(1.0, ns), sc2 = sc * sc;
    double c[p + 1];
    c[0] = 1.0;
    for (int k = 1; k <= p; ++k) c[k] = c[k - 1] * (double)(p + 1 - k) / (double)(k * (2 * p + 1 - k));
    auto mul = [n](const std::vector<cplx>& A, const std::vector<cplx>& B, std::vector<cplx>& C_, cplx alpha) {
        C_.assign((size_t)n * n, cplx(0.0));
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < n; ++k) {
                const cplx a = alpha * A[(size_t)i * n + k];
                if (a == cplx(0.0)) continue;
                for (int j = 0; j < n; ++j) C_[(size_t)i * n + j] += a * B[(size_t)k * n + j];
            }
    };
    std::vector<cplx> H2, P((size_t)n * n, 0.0), Q((size_t)n * n, 0.0), T;
    mul(H, H, H2, cplx(sc2));
    for (int i = 0; i < n; ++i) {
        P[(size_t)i * n + i] = c[p - 1];
        Q[(size_t)i * n + i] = c[p];
    }
    int odd = 1;
    for (int k = p - 1; k > 0; --k) {
        mul(odd ? Q : P, H2, T, cplx(1.0));
        for (int i = 0; i < n; ++i) T[(size_t)i * n + i] += c[k - 1];
        (odd ? Q : P).swap(T);
        odd = 1 - odd;
    }
    mul(odd ? Q : P, H, T, cplx(sc));
    (odd ? Q : P).swap(T);
    for (size_t k = 0; k < Q.size(); ++k) Q[k] -= P[k];
    // Q X = P by LU with partial pivoting (largest |re| + |im|)
    std::vector<int> piv(n);
    for (int k = 0; k < n; ++k) {
        int best = k;
        double bv = -1.0;
        for (int r = k; r < n; ++r) {
            const cplx v = Q[(size_t)r * n + k];
            const double a = std::fabs(v.real()) + std::fabs(v.imag());
            if (a > bv) { bv = a; best = r; }
        }
        if (bv == 0.0) return false;
        piv[k] = best;
        if (best != k) {
            for (int j = 0; j < n; ++j) std::swap(Q[(size_t)k * n + j], Q[(size_t)best * n + j]);
            for (int j = 0; j < n; ++j) std::swap(P[(size_t)k * n + j], P[(size_t)best * n + j]);
        }
        const cplx inv = 1.0 / Q[(size_t)k * n + k];
        for (int r = k + 1; r < n; ++r) {
            const cplx f = Q[(size_t)r * n + k] * inv;
            if (f == cplx(0.0)) continue;
            for (int j = k; j < n; ++j) Q[(size_t)r * n + j] -= f * Q[(size_t)k * n + j];
            for (int j = 0; j < n; ++j) P[(size_t)r * n + j] -= f * P[(size_t)k * n + j];
        }
    }
    for (int r = n - 1; r >= 0; --r)
        for (int j = 0; j < n; ++j) {
            cplx a = P[(size_t)r * n + j];
            for (int k = r + 1; k < n; ++k) a -= Q[(size_t)r * n + k] * P[(size_t)k * n + j];
            P[(size_t)r * n + j] = a / Q[(size_t)r * n + r];
        }
    E.assign((size_t)n * n, cplx(0.0));
    for (size_t k = 0; k < P.size(); ++k) E[k] = 2.0 * P[k];
    for (int i = 0; i < n; ++i) E[(size_t)i * n + i] += 1.0;
    if (ns == 0 && odd) {
        for (cplx& v : E) v = -v;
        return true;
    }
    for (int k = 0; k < ns; ++k) {
        mul(E, E, T, cplx(1.0));
        E.swap(T);
    }
    return true;
}

// Expokit's step-size rounding: two significant digits, rounded up (zgexpv).
double expokit_round(double x) {
    const int e = (int)std::lround(std::log10(x) - std::sqrt(0.1)) - 1;
    const double p = std::pow(10.0, (double)e);
    return std::trunc(x / p + 0.55) * p;
}

gbprop_status ensure_arnoldi_graph(gbprop_ctx* h) {
    if (h->graph_arnoldi) return GBPROP_OK;
    cudaGraph_t g = nullptr;
    GB_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    const long long before = launch_count();
    gbprop_status st = enqueue_arnoldi(h, 1, 1e-7);      // re-orthogonalised; zgexpv break_tol
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (st) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return fail(GBPROP_ECUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
    h->arnoldi_launches = launch_count() - before;
    count_launch((int)-h->arnoldi_launches);
    e = cudaGraphInstantiate(&h->graph_arnoldi, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(GBPROP_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    return GBPROP_OK;
}

}  // namespace

extern "C" gbprop_status gbprop_expokit_advance(gbprop_handle h, void* psi, int nsteps, const double* scalings,
                                                double dt_re, double dt_im, double tol, double anorm,
                                                gbprop_expokit_stats* stats) {
    if (gbprop_status st = check_handle(h, true)) return st;
    if (!psi) return fail(GBPROP_EINVAL, "null wavefunction");
    if (nsteps < 0) return fail(GBPROP_EINVAL, "negative step count");
    if (!scalings && nsteps > 0) return fail(GBPROP_EINVAL, "null scaling schedule");
    const int m = h->m - 1;
    if (m < 2) return fail(GBPROP_EINVAL, "Expokit needs a handle with krylov_basis_size >= 3 (m + 1 vectors)");
    if (!(anorm > 0.0)) return fail(GBPROP_EINVAL, "krylov_norm must be positive");
    gbprop_expokit_stats acc = {0, 0, 0, 0.0, 1.0, 0.0};
    if (nsteps == 0) {
        if (stats) *stats = acc;
        return GBPROP_OK;
    }
    const double eps = DBL_EPSILON;
    if (tol <= eps) tol = std::sqrt(eps);
    const double rndoff = eps * anorm;
    const double t_out = std::sqrt(dt_re * dt_re + dt_im * dt_im);
    const bool imag_time = std::fabs(dt_im) > 1e-10;     // expokitpropagator.cpp:61-66
    // the callback applies -i A (real time) or -A (imaginary time) (krylovcommon.h:61-70)
    const cplx fac = imag_time ? cplx(-1.0, 0.0) : cplx(0.0, -1.0);
    const int mh = m + 2, mv = m + 1;                    // augmented size; device Hessenberg is mv x mv
    gbprop_status st;
    GB_CUDA(h->begin());
    if ((st = enqueue_enter(h, psi, h->stream))) return st;
    if ((st = ensure_sched(h, 1))) return st;
    if ((st = ensure_arnoldi_graph(h))) return st;
    std::vector<double> Hd((size_t)2 * mv * mv);
    std::vector<cplx> Ha, F, Hs;
    Ctrl c;
    double vnorm = -1.0;
    for (int n = 0; n < nsteps; ++n) {
        SchedEntry se = sched_entry(scalings + (size_t)n * h->nfuncs, h->nfuncs, dt_re, dt_im);
        GB_CUDA(cudaMemcpyAsync(h->d_sched, &se, sizeof(se), cudaMemcpyHostToDevice, h->stream));
        double t_now = 0.0, t_new = 0.0, xm = 1.0 / m;
        bool first = true;
        while (t_now < t_out) {
            // Arnoldi from the current state (beta = ||w||, m + 1 vectors, Hessenberg)
            GB_CUDA(cudaMemsetAsync(&h->d_ctrl->step, 0, sizeof(int), h->stream));
            GB_CUDA(cudaGraphLaunch(h->graph_arnoldi, h->stream));
            count_launch((int)h->arnoldi_launches);
            GB_CUDA(cudaMemcpyAsync(&c, h->d_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->stream));
            GB_CUDA(cudaMemcpyAsync(Hd.data(), h->d_H, Hd.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
            GB_CUDA(cudaStreamSynchronize(h->stream));
            if (c.nonfinite || c.wait_timeout) return report_flags(h, 0, c.nonfinite, c.wait_timeout);
            const double beta = c.beta0;
            if (vnorm < 0.0) vnorm = beta;
            acc.hump = std::max(acc.hump, beta / vnorm);
            if (first) {
                // initial step size (zgexpv)
                const double p2 = tol * std::pow((m + 1) / 2.72, m + 1) * std::sqrt((m + 1) * 6.28);
                t_new = expokit_round(1.0 / anorm * std::pow(p2 / (4.0 * beta * anorm), xm));
                first = false;
            }
            double t_step = std::min(t_out - t_now, t_new);
            int k1 = 2, mb = m;
            double avnorm = 0.0;
            if (c.broken) {
                k1 = 0;
                mb = c.nbasis;
                t_step = t_out - t_now;
            } else {
                avnorm = c.pre_norm;                     // ||A v_{m+1}|| before orthogonalisation
            }
            acc.matvecs += c.broken ? c.nbasis : mv;
            // augmented (m+2) x (m+2) matrix for the operator fac*A on the basis built for A:
            // fac * H_A (its Krylov approximation beta V exp(t fac H_A) e1 and the magnitudes of
            // the error-estimate entries equal those of the Hessenberg zgexpv builds for fac*A,
            // whose basis differs from V only by the phases fac^j); H(m+1, m) = 1
            Ha.assign((size_t)mh * mh, cplx(0.0));
            for (int J = 0; J < mb; ++J)
                for (int k = 0; k <= std::min(J + 1, mb); ++k) {
                    if (k >= mv) continue;
                    const cplx v(Hd[2 * ((size_t)k * mv + J)], Hd[2 * ((size_t)k * mv + J) + 1]);
                    Ha[(size_t)k * mh + J] = fac * v;
                }
            if (k1 != 0) Ha[(size_t)(m + 1) * mh + m] = 1.0;
            int ireject = 0;
            double err_loc = 0.0;
            int mx = mb + k1;
            for (;;) {
                mx = mb + k1;
                Hs.assign((size_t)mx * mx, cplx(0.0));
                for (int i = 0; i < mx; ++i)
                    for (int j = 0; j < mx; ++j) Hs[(size_t)i * mx + j] = Ha[(size_t)i * mh + j];
                if (!expokit_pade(Hs, mx, t_step, F)) return fail(GBPROP_ELU, "singular Pade denominator (Expokit)");
                if (k1 == 0) {
                    err_loc = tol;
                    break;
                }
                const double p1 = std::abs(F[(size_t)m * mx]) * beta;
                const double p2 = std::abs(F[(size_t)(m + 1) * mx]) * beta * avnorm;
                if (p1 > 10.0 * p2) {
                    err_loc = p2;
                    xm = 1.0 / m;
                } else if (p1 > p2) {
                    err_loc = p1 * p2 / (p1 - p2);
                    xm = 1.0 / m;
                } else {
                    err_loc = p1;
                    xm = 1.0 / (m - 1);
                }
                if (err_loc <= 1.2 * t_step * tol) break;
                t_step = expokit_round(0.9 * t_step * std::pow(t_step * tol / err_loc, xm));
                ++acc.rejections;
                if (++ireject > 100) return fail(GBPROP_EBREAKDOWN, "Expokit: the requested tolerance is too high");
            }
            // w = beta V exp(t_step H) e1 over mx = mb + max(0, k1 - 1) vectors
            mx = mb + std::max(0, k1 - 1);
            const int ld = mb + k1;
            std::vector<double> y((size_t)2 * mx);
            for (int k = 0; k < mx; ++k) {
                y[2 * k] = F[(size_t)k * ld].real();
                y[2 * k + 1] = F[(size_t)k * ld].imag();
            }
            GB_CUDA(cudaMemcpyAsync(h->d_ctrl->y, y.data(), y.size() * sizeof(double), cudaMemcpyHostToDevice,
                                    h->stream));
            GB_CUDA(cudaMemcpyAsync(&h->d_ctrl->nbasis, &mx, sizeof(int), cudaMemcpyHostToDevice, h->stream));
            GB_CUDA(cudaMemsetAsync(&h->d_ctrl->broken, 0, sizeof(int), h->stream));
            GB_LAUNCH(launch_combine(h->kprec(), h->d_V, h->d_v0, h->N, h->d_ctrl, h->d_x, h->stream));
            t_now += t_step;
            t_new = expokit_round(0.9 * t_step * std::pow(t_step * tol / err_loc, xm));
            acc.error += std::max(err_loc, rndoff);
            acc.last_step = t_step;
            ++acc.substeps;
        }
        if (h->renormalize)                              // Problem.py:167-168, after every step
            GB_LAUNCH(launch_renormalize(h->d_x, h->N, h->d_partials, h->d_counter, h->d_ctrl, h->stream));
    }
    if ((st = enqueue_leave(h, psi, h->stream))) return st;
    if ((st = arm_flags(h))) return st;
    GB_CUDA(h->end());
    if (stats) *stats = acc;
    return GBPROP_OK;
}

// ---------------------------------------------------------------------------
// Batches: many independent problems advanced together.  The step sequences
// of all member handles are captured into one CUDA graph (one branch per
// problem, forked from and joined into the batch stream), so a whole-batch
// step is a single graph launch and the GPU overlaps the problems' kernels.
// ---------------------------------------------------------------------------
struct gbprop_batch_ctx {
    std::vector<gbprop_handle> hs;
    cudaStream_t stream = nullptr, ustream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_in = nullptr, ev_out = nullptr;
    std::vector<cudaEvent_t> ev_join;
    // one batch step per graph launch; each problem is one branch whose kernels are, per
    // shape: [0] enter + step + leave (one-step calls), [1] enter + step (first step),
    // [2] step (middle steps), [3] step + leave (last step)
    cudaGraphExec_t g[4] = {nullptr, nullptr, nullptr, nullptr};
    long long g_launches[4] = {0, 0, 0, 0};
    std::vector<void*> graph_psi;
    // members' error flags gathered after each advance (see launch_gather_flags)
    Ctrl** d_ctrls = nullptr;
    int* d_flags = nullptr;
    int* h_flags = nullptr;
    cudaEvent_t ev_flags = nullptr;
    bool flags_armed = false;
    ~gbprop_batch_ctx() {
        for (cudaGraphExec_t x : g)
            if (x) cudaGraphExecDestroy(x);
        for (cudaEvent_t e : ev_join) cudaEventDestroy(e);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_in) cudaEventDestroy(ev_in);
        if (ev_out) cudaEventDestroy(ev_out);
        if (ev_flags) cudaEventDestroy(ev_flags);
        if (h_flags) cudaFreeHost(h_flags);
        if (d_ctrls) cudaFree(d_ctrls);
        if (d_flags) cudaFree(d_flags);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

// Capture one parallel branch per problem (forked from and joined into the batch stream).
// what: bit 0 = enter (x = U psi), bit 1 = one step, bit 2 = leave (psi = U^-1 x).
gbprop_status batch_capture(gbprop_batch b, void* const* psi, int what, cudaGraphExec_t* out, long long* launches) {
    if (*out) {
        cudaGraphExecDestroy(*out);
        *out = nullptr;
    }
    cudaGraph_t g = nullptr;
    GB_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    const long long before = launch_count();
    gbprop_status st = GBPROP_OK;
    cudaError_t e = cudaEventRecord(b->ev_fork, b->stream);
    for (size_t p = 0; p < b->hs.size() && st == GBPROP_OK && e == cudaSuccess; ++p) {
        gbprop_ctx* h = b->hs[p];
        e = cudaStreamWaitEvent(h->stream, b->ev_fork, 0);
        if (e != cudaSuccess) break;
        if (what & 1) st = enqueue_enter(h, psi[p], h->stream);
        if (!st && (what & 2)) st = enqueue_step(h);
        if (!st && (what & 4)) st = enqueue_leave(h, psi[p], h->stream);
        if (st) break;
        e = cudaEventRecord(b->ev_join[p], h->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, b->ev_join[p], 0);
    }
    cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
    if (st) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess || e2 != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return fail(GBPROP_ECUDA, std::string("batch capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
    }
    *launches = launch_count() - before;
    count_launch((int)-*launches);
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(GBPROP_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    return GBPROP_OK;
}

// The members' error flags (see device_errors), gathered into one pinned copy per advance.
gbprop_status batch_errors(gbprop_batch b, bool block) {
    if (!b->flags_armed) return GBPROP_OK;
    cudaError_t e = block ? cudaEventSynchronize(b->ev_flags) : cudaEventQuery(b->ev_flags);
    if (e == cudaErrorNotReady) return GBPROP_OK;
    if (e != cudaSuccess) return fail(GBPROP_ECUDA, std::string("flag event: ") + cudaGetErrorString(e));
    b->flags_armed = false;
    const int p = b->h_flags[3] - 1;
    if (p < 0 || p >= (int)b->hs.size()) return GBPROP_OK;
    gbprop_ctx* h = b->hs[p];
    // clear every member's flags (only members with a failure have any set)
    for (gbprop_ctx* x : b->hs) GB_CUDA(cudaMemsetAsync(&x->d_ctrl->lu_info, 0, 3 * sizeof(int), b->stream));
    cudaStream_t keep = h->stream;
    h->stream = b->stream;
    gbprop_status st = report_flags(h, b->h_flags[0], b->h_flags[1], b->h_flags[2]);
    h->stream = keep;
    set_last_error((std::string(gbprop_last_error()) + " (problem " + std::to_string(p) + " of the batch)").c_str());
    return st;
}

}  // namespace

extern "C" {

gbprop_status gbprop_batch_create(gbprop_batch* out, const gbprop_handle* problems, int count, int autotune,
                                  void* stream) {
    if (!out) return fail(GBPROP_EINVAL, "null output pointer");
    *out = nullptr;
    if (!problems || count < 1) return fail(GBPROP_EINVAL, "a batch needs at least one problem");
    for (int p = 0; p < count; ++p) {
        if (gbprop_status st = check_handle(problems[p], true)) return st;
        if (problems[p]->prec != problems[0]->prec) return fail(GBPROP_EINVAL, "all problems of a batch share one precision");
        for (int q = 0; q < p; ++q)
            if (problems[q] == problems[p]) return fail(GBPROP_EINVAL, "a problem appears twice in the batch");
    }
    gbprop_batch b = new gbprop_batch_ctx();
    b->hs.assign(problems, problems + count);
    b->ustream = (cudaStream_t)stream;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_out, cudaEventDisableTiming);
    b->ev_join.assign(count, nullptr);
    for (int p = 0; p < count && e == cudaSuccess; ++p) e = cudaEventCreateWithFlags(&b->ev_join[p], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_flags, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&b->h_flags, 4 * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_flags, 4 * sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_ctrls, count * sizeof(Ctrl*));
    if (e == cudaSuccess) {
        std::vector<Ctrl*> cs(count);
        for (int p = 0; p < count; ++p) cs[p] = problems[p]->d_ctrl;
        e = cudaMemcpy(b->d_ctrls, cs.data(), count * sizeof(Ctrl*), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        delete b;
        return fail(GBPROP_ECUDA, std::string("batch stream/event creation: ") + cudaGetErrorString(e));
    }
    for (gbprop_handle h : b->hs) {
        h->expm_max_cluster = 1;        // other problems fill the GPU: one CTA per exponential
        if (h->inv_ok) set_inv_chunks(h, false);
        // Gram-Schmidt of a complex64 basis: the cooperative form on a grid sized to the problem
        // (measured: mixed batch 76.0 -> 72.5 ms per step; FP64 batches keep the three-kernel form,
        // 161 against 195 ms with it; GBPROP_CGS=separate keeps it for both)
        {
            const char* env = std::getenv("GBPROP_CGS");
            int cache = 0;
            const int grid = (env && std::strcmp(env, "separate") == 0) || h->double_orth || h->prec == GBPROP_FP64
                                 ? 0
                                 : arnoldi_cgs_grid_batch(h->kprec(), h->N, h->m, h->d_v0 != nullptr, &cache);
            cudaGetLastError();
            if (grid > 0 && !h->d_gridbar) {
                if (gbprop_status st = h->dalloc(&h->d_gridbar, 64)) {
                    delete b;
                    return st;
                }
                cudaMemsetAsync(h->d_gridbar, 0, 64, h->stream);
            }
            if (grid > 0 && (!h->d_cgs_part || grid > h->cgs_part_grid)) {
                if (gbprop_status st = h->dalloc(&h->d_cgs_part, arnoldi_cgs_part_doubles(grid) * sizeof(double))) {
                    delete b;
                    return st;
                }
                h->cgs_part_grid = grid;
            }
            h->cgs_grid = grid;
            h->cgs_cache = cache;
        }
        drop_graph(h);
        if (autotune) {
            gbprop_status st = gbprop_autotune(h, nullptr);
            if (st) {
                delete b;
                return st;
            }
        }
    }
    *out = b;
    return GBPROP_OK;
}

gbprop_status gbprop_batch_advance(gbprop_batch b, void* const* psi, int nsteps, const double* scalings,
                                   const double* dt) {
    if (!b) return fail(GBPROP_EINVAL, "null batch");
    if (!psi || !scalings || !dt) return fail(GBPROP_EINVAL, "null argument");
    if (nsteps < 0) return fail(GBPROP_EINVAL, "negative step count");
    if (nsteps == 0) return GBPROP_OK;
    const size_t P = b->hs.size();
    for (size_t p = 0; p < P; ++p)
        if (!psi[p]) return fail(GBPROP_EINVAL, "null wavefunction in batch");
    if (gbprop_status st = batch_errors(b, false)) return st;
    // problem p's nsteps x nfuncs block of the packed scalings
    std::vector<size_t> off(P + 1, 0);
    for (size_t p = 0; p < P; ++p) off[p + 1] = off[p] + (size_t)nsteps * b->hs[p]->nfuncs;
    GB_CUDA(cudaEventRecord(b->ev_in, b->ustream));
    GB_CUDA(cudaStreamWaitEvent(b->stream, b->ev_in, 0));
    static const int kShape[4] = {1 | 2 | 4, 1 | 2, 2, 2 | 4};
    bool new_psi = b->graph_psi.size() != P;
    for (size_t p = 0; p < P && !new_psi; ++p)
        if (b->graph_psi[p] != psi[p]) new_psi = true;
    if (new_psi) {
        for (int k : {0, 1, 3})
            if (b->g[k]) {
                cudaGraphExecDestroy(b->g[k]);
                b->g[k] = nullptr;
            }
        b->graph_psi.assign(psi, psi + P);
    }
    int done = 0;
    while (done < nsteps) {
        int cap = 1 << 30;
        for (gbprop_handle h : b->hs) cap = std::min(cap, std::max(h->sched_cap, 1024));
        const int chunk = std::min(nsteps - done, cap);
        bool recapture = false;
        for (size_t p = 0; p < P; ++p) {
            gbprop_ctx* h = b->hs[p];
            const int old_cap = h->sched_cap;
            if (gbprop_status st = ensure_sched(h, chunk)) return st;
            if (h->sched_cap != old_cap) recapture = true;
            std::vector<SchedEntry> sched(chunk);
            const double* sp = scalings + off[p] + (size_t)done * h->nfuncs;
            for (int k = 0; k < chunk; ++k)
                sched[k] = sched_entry(sp + (size_t)k * h->nfuncs, h->nfuncs, dt[2 * p], dt[2 * p + 1]);
            GB_CUDA(cudaMemcpyAsync(h->d_sched, sched.data(), chunk * sizeof(SchedEntry), cudaMemcpyHostToDevice,
                                    b->stream));
            GB_CUDA(cudaMemsetAsync(&h->d_ctrl->step, 0, sizeof(int), b->stream));
        }
        if (recapture)
            for (int k = 0; k < 4; ++k)
                if (b->g[k]) {
                    cudaGraphExecDestroy(b->g[k]);
                    b->g[k] = nullptr;
                }
        for (int k = 0; k < chunk; ++k) {
            const int step = done + k;
            const bool first = step == 0, last = step == nsteps - 1;
            const int shape = first && last ? 0 : first ? 1 : last ? 3 : 2;
            if (!b->g[shape])
                if (gbprop_status st = batch_capture(b, psi, kShape[shape], &b->g[shape], &b->g_launches[shape]))
                    return st;
            GB_CUDA(cudaGraphLaunch(b->g[shape], b->stream));
            count_launch((int)b->g_launches[shape]);
        }
        done += chunk;
    }
    GB_LAUNCH(launch_gather_flags(b->d_ctrls, (int)P, b->d_flags, b->stream));
    GB_CUDA(cudaMemcpyAsync(b->h_flags, b->d_flags, 4 * sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    GB_CUDA(cudaEventRecord(b->ev_flags, b->stream));
    b->flags_armed = true;
    GB_CUDA(cudaEventRecord(b->ev_out, b->stream));
    GB_CUDA(cudaStreamWaitEvent(b->ustream, b->ev_out, 0));
    return GBPROP_OK;
}

gbprop_status gbprop_batch_synchronize(gbprop_batch b) {
    if (!b) return fail(GBPROP_EINVAL, "null batch");
    GB_CUDA(cudaStreamSynchronize(b->stream));
    GB_CUDA(cudaStreamSynchronize(b->ustream));
    return batch_errors(b, true);
}

gbprop_status gbprop_batch_destroy(gbprop_batch b) {
    if (!b) return GBPROP_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (gbprop_handle h : b->hs) {
        h->expm_max_cluster = 16;
        if (h->inv_ok) set_inv_chunks(h, true);
    }
    delete b;
    return GBPROP_OK;
}

}  // extern "C"
