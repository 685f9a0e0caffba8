// Host side of the C ABI declared in include/radis_gb300.h.
//
// Object model (reference: radis/gpu/gpu.py gpuApp):
//   rg_ctx    one device + one non-blocking stream  (GPUApplication)
//   rg_lines  device-resident line list, structure of arrays, sorted by v0,
//             plus host-side envelopes of widths and intensities
//             (gpuApp.__init__ upload gpu.py:190-203; init_*_params params.py)
//   rg_plan   spectral grid, FFT factorisation + twiddle tables, line index per
//             grid column and the grow-only LDM / FFT workspace
//             (gpu.py:133-141, 205-239; the x1.5 grow rule of
//             vulkan_compute_lib.py:1308-1323 becomes x1.25 here)
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdarg>
#include <cstring>
#include <limits>
#include <memory>
#include <new>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <thread>

#include <nvtx3/nvToolsExt.h>

#include "rg_internal.h"

using namespace rg;

// ---------------------------------------------------------------------------
// error reporting
// ---------------------------------------------------------------------------
static thread_local std::string g_err;

// NVTX range over a host stage (upload, envelopes, plan, spectrum, served
// request, HITRAN parse): a profiler attached through NVTX (ncu --nvtx) sees
// the stage names; without one a push/pop is a no-op call.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Makes a device current for the life of one C entry point and restores the
// caller's current device when the entry point returns (a caller working on
// another device, e.g. a framework's current device, finds it unchanged).
struct DeviceGuard {
    int prev = -1;
    bool changed = false;
    cudaError_t use(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev == dev) return cudaSuccess;
        const cudaError_t e = cudaSetDevice(dev);
        changed = e == cudaSuccess && prev >= 0;
        return e;
    }
    ~DeviceGuard() {
        if (changed) cudaSetDevice(prev);
    }
    DeviceGuard() = default;
    DeviceGuard(const DeviceGuard&) = delete;
    DeviceGuard& operator=(const DeviceGuard&) = delete;
};

static int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CU(call)                                                                            \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(e_ == cudaErrorMemoryAllocation ? RG_ERR_OOM : RG_ERR_CUDA,         \
                        "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                          \
    } while (0)

#define RG(call)                                                   \
    do {                                                           \
        int r_ = (call);                                           \
        if (r_ != RG_OK) {                                         \
            if (g_err.empty())                                     \
                fail(r_, "%s failed%s%s", #call,                   \
                     r_ == RG_ERR_CUDA && last_launch_error() ? ": " : "", \
                     r_ == RG_ERR_CUDA && last_launch_error() ? last_launch_error() : ""); \
            return r_;                                             \
        }                                                          \
    } while (0)

// ---------------------------------------------------------------------------
// objects
// ---------------------------------------------------------------------------
struct rg_ctx {
    int device = 0;
    int sms = 1;              // streaming multiprocessors of the device
    cudaStream_t stream = nullptr;
    int lines = 0;            // live line lists on this context
    uint32_t magic = 0x52474358;
};

// Host-side summary of a line list: everything the per-spectrum grid and
// scale computation needs (the reference keeps the same data as module
// globals in radis/gpu/params.py:66-86).
struct Envelope {
    int64_t n = 0;
    int n_iso = 1;
    double t_ref = 296.0;
    double log_c2Mm[kMaxIso] = {0};            // log(FWHM_G / (v0 sqrt(T)))
    double lv_min[kMaxIso], lv_max[kMaxIso];   // per-iso min/max log v0
    double max_abs_delta = 0.0;
    Hull wl_lo, wl_hi;   // (n_air, log min/max(g_self, g_air))
    Hull s_hi;           // (E_low, ln S')  S' = S_ref / (1 - exp(-c2 v0 / Tref))
};

struct rg_lines {
    rg_ctx* ctx = nullptr;
    int64_t n = 0;
    float2* v0 = nullptr;
    float* ls2 = nullptr;
    float* el = nullptr;
    float* ga = nullptr;
    float* gs = nullptr;
    float* na = nullptr;
    float* dl = nullptr;
    uint8_t* iso = nullptr;
    int n_iso = 1;
    double t_ref = 296.0;
    Envelope env;
    std::vector<QTable> qtab;       // optional tabulated Q(T) per isotopologue
    std::atomic<int> plans{0};      // plans and server requests referencing the list
    uint32_t magic = 0x52474C4E;
};

// Geometry and device buffers of one spectrum in flight: a plan owns one, a
// server slot owns one per request it runs (tables may be shared).
struct Work {
    rg_plan_desc desc{};
    // FFT factorisation n = n1 n2 and its tables
    int64_t n = 0;
    int n1 = 0, n2 = 0, B = 0;
    FftLen f1, f2;
    const float2* tw_hi = nullptr;
    const float2* tw_lo = nullptr;
    // line index per grid column and the fixed-point bound
    int64_t* col_start = nullptr;
    int col_off = 0, col_count = 0, E = 0;
    double p_atm_max = 0.0;
    int* cmax_dev = nullptr;
    int64_t cmax_host = -1;           // known on the host (plans), -1 otherwise
    // grow-only buffers
    int nodes_cap = 0;                // node rows the LDM / FFT workspace holds at this geometry
    size_t ldm_bytes = 0, y_bytes = 0;   // allocated sizes of ldm and y
    // merged layout (Gaussian stage in real space): its rows, grow-only
    bool allow_merge = true;
    float* mrow = nullptr;
    size_t mrow_bytes = 0;
    int last_fft_rows = 0, last_merged_rows = 0, last_ext = 0;   // layout of the last spectrum
    int last_layout = 0;              // 1 node rows, 2 merged rows, 3 skeleton rows
    double last_layout_err = 0.0;     // skeleton layout: the decomposition's sampled error
    // skeleton layout: projection coefficients [n_nodes][rows_pad] (device,
    // grow-only) and their host staging (copied from pageable memory: the
    // copy has left this buffer when cudaMemcpyAsync returns)
    bool allow_skeleton = true;
    bool proj_fixed = false;          // proj_coef is a fixed piece of scratch (never reallocated)
    float* proj_coef = nullptr;
    size_t proj_bytes = 0;
    std::vector<float> proj_host;
    // the last decomposition, reused while the node grid is the same (a pure
    // function of the axes, spacing, folding threshold and tolerance); the
    // device copy of its coefficients is current while skel_dev is set
    double skel_key[10] = {0};
    // the per-node folded-Voigt parameters of the last grid (fill_voigt_args),
    // reused while the axes, spacing and folding threshold repeat
    double va_key[8] = {0};
    bool va_valid = false;
    std::vector<float> va_norm, va_lnorm, va_alpha, va_beta;
    std::vector<unsigned char> va_nfold;
    int va_any_fold = 0;
    bool skel_valid = false, skel_dev = false;
    int skel_R = 0;
    double skel_err = 0.0;
    std::vector<int> skel_nodes;
    int skel_flush_ks = 0;   // the scatter flush's tensor-core section: node steps (0: none)
    int last_accum = 0;               // accumulator bits of the last scatter (0: chosen on the device)
    int64_t row_stride = 0;
    float* ldm = nullptr;             // LDM [node][row_stride] (the scatter's float values)
    float2* y = nullptr;
    float2* g = nullptr;
    unsigned long long* counter = nullptr;
    unsigned* err = nullptr;          // device flag set by a bounded wait that gave up
    unsigned* err_host = nullptr;     // pinned copy of err, refreshed after every spectrum
    unsigned* err_pub = nullptr;      // device view of err_host when it is mapped (the last kernel writes it)
    bool count_lines = false;         // count the lines in the window (timing = 1 reports it)
    // post-processing rows written by the last kernel (rg_synthesize_quantities):
    // 4 rows of n_v floats, or null; path length (cm) and gas temperature (K)
    float* quant_out = nullptr;
    double quant_path = 0.0, quant_T = 0.0;
    // bound of the scatter's handshake waits (cycles) and the test hook that
    // withholds its line copies (rg_plan_test_scatter_stall)
    long long scat_wait = kScatWaitCycles;
    int scat_withhold = 0;
};

struct rg_plan {
    rg_lines* lines = nullptr;
    std::mutex mu;
    Work w;
    float2* tw_hi_own = nullptr;
    float2* tw_lo_own = nullptr;
    float* out_d = nullptr;
    float* quant_d = nullptr;           // 5 rows of n_v (rg_synthesize_quantities_host), on first use
    double* grad_d = nullptr;           // 3 sums of the adjoint gather, allocated on first use
    // stage events: start, after scatter, fft-col, fft-row, ifft-row, ifft-col,
    // and [6] after the Gaussian stage inside fft-col (at [1] without it)
    static constexpr int kEv = 7;
    cudaEvent_t ev[kEv] = {nullptr};
    // ring of per-stage events recorded without synchronisation (timing == 2)
    static constexpr int kRing = 256;
    std::vector<cudaEvent_t> ring;      // kRing * kEv events, created lazily
    double last_gauss_sum = 0.0;        // Gaussian-stage part of the last ring read
    int ring_used = 0;
    bool ring_ldm_only[kRing] = {false};
    cudaStream_t ring_stream = nullptr;
    // device work of the plan is serialised across streams: work enqueued on a
    // stream other than the last one waits for `done` (recorded after each call)
    cudaEvent_t done = nullptr;
    cudaStream_t last_stream = nullptr;
    bool any = false;
    uint32_t magic = 0x52475041;
};

namespace {

// smallest 5-smooth m >= x
int64_t next_smooth(int64_t x) {
    for (int64_t m = std::max<int64_t>(x, 1);; ++m) {
        int64_t r = m;
        for (int p : {2, 3, 5})
            while (r % p == 0) r /= p;
        if (r == 1) return m;
    }
}

// Radix plan of a length L = 2^a 3^b 5^c: the leftover 2 or 4, the 3s and 5s
// (merged into composite radices: up to 12 first, 6 later), then radix 8
// -- the last pass is radix 8 whenever 8 divides L, which the row kernel
// relies on (n2 is a multiple of 32).
// Partition-function ratio Q(Tref)/Q(T) of isotopologue i: the caller's,
// else the list's tables when every isotopologue has one, else 1.
bool have_qtables(const rg_lines* L) {
    if ((int)L->qtab.size() != L->n_iso) return false;
    for (const QTable& t : L->qtab)
        if (t.T.size() < 2) return false;
    return true;
}
int q_ratio_of(const rg_lines* L, const rg_conditions* c, int i, double* q) {
    if (c->q_ratio) {
        *q = c->q_ratio[i];
        return RG_OK;
    }
    *q = 1.0;
    if (!have_qtables(L)) return RG_OK;
    double q_ref, q_t;
    std::string e;
    int rc = qtable_eval(L->qtab[i], L->t_ref, &q_ref, nullptr, &e);
    if (!rc) rc = qtable_eval(L->qtab[i], c->T, &q_t, nullptr, &e);
    if (rc) return fail(rc, "isotopologue %d: %s", i, e.c_str());
    *q = q_ref / q_t;
    return RG_OK;
}
// d ln(Q(Tref)/Q(T))/dT of isotopologue i: the caller's, else -Q'(T)/Q(T)
// from the tables, else 0.
int dlnq_of(const rg_lines* L, const double* dlnq_dT, double T, int i, double* out) {
    *out = dlnq_dT ? dlnq_dT[i] : 0.0;
    if (dlnq_dT || !have_qtables(L)) return RG_OK;
    double q, dq;
    std::string e;
    const int rc = qtable_eval(L->qtab[i], T, &q, &dq, &e);
    if (rc) return fail(rc, "isotopologue %d: %s", i, e.c_str());
    *out = -dq / q;
    return RG_OK;
}

bool radices(int L, int* rad, int* np) {
    int r = L, k = 0;
    int a = 0, b = 0, c = 0;
    while (r % 2 == 0) {
        r /= 2;
        ++a;
    }
    while (r % 3 == 0) {
        r /= 3;
        ++b;
    }
    while (r % 5 == 0) {
        r /= 5;
        ++c;
    }
    // the small factors (the leftover 2 or 4, the 3s and 5s), merged in order
    // into composite radices (6, 9, 10, 12) within the bounds the row kernels
    // transform in registers without spilling
    int small[64], ns = 0;
    if (a % 3 == 2) small[ns++] = 4;
    if (a % 3 == 1) small[ns++] = 2;
    for (int i = 0; i < b && ns < 64; ++i) small[ns++] = 3;
    for (int i = 0; i < c && ns < 64; ++i) small[ns++] = 5;
    int cur = 1;
    for (int i = 0; i < ns; ++i) {
        const int cap = k == 0 ? kFirstRadixMax : kMidRadixMax;
        if (cur * small[i] <= cap) {
            cur *= small[i];
        } else {
            if (k >= kMaxPasses) return false;
            rad[k++] = cur;
            cur = small[i];
        }
    }
    if (cur > 1) {
        if (k >= kMaxPasses) return false;
        rad[k++] = cur;
    }
    for (int i = 0; i < a / 3; ++i) {
        if (k >= kMaxPasses) return false;
        rad[k++] = 8;
    }
    *np = k;
    return r == 1;
}

constexpr int kN2Max = 256 * 32;   // row FFT limit (threads x register accumulators)

// choose n = n1 * n2 >= n_min, n1 a power of two <= 512, n2 = 32 * (5-smooth).
// The row kernel runs n1 x (pair groups) CTAs, so n1 = 8 (a handful of long
// rows) is taken only when its length is at least a quarter shorter than the
// best with n1 = 512 or 64, or when neither fits.
bool choose_fft(int64_t n_min, int64_t forced, int* n1o, int* n2o) {
    int64_t best = std::numeric_limits<int64_t>::max();
    int b1 = 0, b2 = 0;
    for (int n1 : {512, 64, 8}) {   // radix-8 register column FFTs
        int64_t n2;
        if (forced) {
            if (forced % n1) continue;
            n2 = forced / n1;
            if (n2 % 32) continue;
            int64_t m = n2 / 32, r = m;
            for (int p : {2, 3, 5})
                while (r % p == 0) r /= p;
            if (r != 1) continue;
        } else {
            int64_t need = (n_min + n1 - 1) / n1;
            n2 = 32 * next_smooth((need + 31) / 32);
        }
        if (n2 > kN2Max) continue;
        int64_t n = (int64_t)n1 * n2;
        if (n < n_min) continue;
        // prefer the shorter transform, then the larger n1 (fewer row FFT launches)
        if (n1 == 8 && !forced && b1 && 4 * n > 3 * best) continue;
        if (n < best) {
            best = n;
            b1 = n1;
            b2 = (int)n2;
        }
    }
    if (!b1) return false;
    *n1o = b1;
    *n2o = b2;
    return true;
}

int upload_twiddles(int L, float2** out) {
    std::vector<float2> h(L);
    for (int t = 0; t < L; ++t) {
        double ang = -2.0 * kPi * (double)t / (double)L;
        h[t].x = (float)std::cos(ang);
        h[t].y = (float)std::sin(ang);
    }
    CU(cudaMalloc(out, sizeof(float2) * L));
    CU(cudaMemcpy(*out, h.data(), sizeof(float2) * L, cudaMemcpyHostToDevice));
    return RG_OK;
}

int make_fftlen(int L, FftLen* f) {
    f->L = L;
    if (!radices(L, f->radix, &f->npass)) return fail(RG_ERR_RANGE, "FFT length %d not factorable", L);
    int ns = 1;
    for (int p = 0; p < f->npass; ++p) {
        f->ns[p] = ns;
        f->mag[p] = ns == 1 ? 0u : (unsigned)(((1ull << 32) + ns - 1) / (unsigned long long)ns);
        ns *= f->radix[p];
    }
    return upload_twiddles(L, &f->tw);
}

void split(double v, float* hi, float* lo) {
    *hi = (float)v;
    *lo = (float)(v - (double)*hi);
}

template <typename T>
void dfree(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

// Per-spectrum host parameters (the reference's set_pTQ / set_G_params /
// set_L_params, radis/gpu/params.py:89-155).
// The plan options that select how, not what, is computed.
int check_desc_options(const rg_plan_desc& d) {
    if (d.accumulator != 0 && d.accumulator != 32 && d.accumulator != 64)
        return fail(RG_ERR_ARG, "accumulator must be 0, 32 or 64 (got %d)", (int)d.accumulator);
    if (d.axes_window != 0 && d.axes_window != 1)
        return fail(RG_ERR_ARG, "axes_window must be 0 or 1 (got %d)", (int)d.axes_window);
    if (d.layout < 0 || d.layout > 3) return fail(RG_ERR_ARG, "layout must be 0..3 (got %d)", (int)d.layout);
    if (!(d.layout_tol < 1e-2)) return fail(RG_ERR_ARG, "layout_tol must be < 1e-2 (got %g)", d.layout_tol);
    return RG_OK;
}

struct SpecHost {
    rg_grid grid;
    double p_atm, log_scale_int, log_scale_out;
    int n_nodes;       // padded to even
};

// `lines` (may be NULL: host-only estimate) supplies tabulated Q(T).
int compute_grid_env(const Envelope& E, const rg_lines* lines, const rg_plan_desc& d, int64_t n_ft, int n1, int n2,
                     const rg_conditions* c, SpecHost* s) {
    const Envelope* L = &E;
    if (!(c->T > 0) || !(c->p_bar > 0) || !(c->x >= 0 && c->x <= 1))
        return fail(RG_ERR_ARG, "conditions out of range: T=%g p=%g x=%g", c->T, c->p_bar, c->x);
    const double eps = 1e-4;   // params.py:89,107
    const double T = c->T;
    s->p_atm = c->p_bar / kAtm;
    // Gaussian axis: min/max of log v0 + log_c2Mm + 0.5 log T  (params.py:70-81,107-117),
    // over the list, or (axes_window) over the lines whose shifted centre can
    // fall inside the window: v0 in [vmin - s, vmax + s], s = max |shift| + dv
    double lg_lo = std::numeric_limits<double>::infinity(), lg_hi = -lg_lo;
    for (int pass = d.axes_window ? 0 : 1; pass < 2 && !(lg_lo <= lg_hi); ++pass) {
        double wlo = -std::numeric_limits<double>::infinity(), whi = -wlo;
        if (pass == 0) {   // the window's reach; an empty reach falls back to the list
            const double sh = L->max_abs_delta * s->p_atm + d.dv;
            const double vlo = d.vmin - sh, vhi = d.vmin + (double)(d.n_v - 1) * d.dv + sh;
            if (vlo > 0) wlo = std::log(vlo);
            whi = vhi > 0 ? std::log(vhi) : -std::numeric_limits<double>::infinity();
        }
        for (int i = 0; i < L->n_iso; ++i) {
            const double lo = std::max(L->lv_min[i], wlo), hi = std::min(L->lv_max[i], whi);
            if (!(lo <= hi)) continue;
            lg_lo = std::min(lg_lo, lo + L->log_c2Mm[i]);
            lg_hi = std::max(lg_hi, hi + L->log_c2Mm[i]);
        }
    }
    lg_lo += 0.5 * std::log(T);
    lg_hi += 0.5 * std::log(T) + eps;
    // Lorentzian axis: envelopes over log(T_ref/T)  (params.py:8-67,89-104)
    const double t = std::log(L->t_ref / T);
    const double l2p = std::log(2.0 * s->p_atm);
    double ll_lo = L->wl_lo.min_at(t) + l2p;
    double ll_hi = L->wl_hi.max_at(t) + l2p + eps;
    if (!std::isfinite(lg_lo) || !std::isfinite(lg_hi) || !std::isfinite(ll_lo) || !std::isfinite(ll_hi))
        return fail(RG_ERR_ARG, "line widths are not finite (zero or negative broadening?)");
    rg_grid& g = s->grid;
    g.log_wG_min = lg_lo;
    g.log_wL_min = ll_lo;
    if (d.n_G > 1) {
        g.n_G = d.n_G;
        g.dxG = (lg_hi - lg_lo) / (d.n_G - 1);
    } else {
        g.dxG = d.dxG;
        g.n_G = (int)std::ceil((lg_hi - lg_lo) / d.dxG) + 1;
    }
    if (d.n_L > 1) {
        g.n_L = d.n_L;
        g.dxL = (ll_hi - ll_lo) / (d.n_L - 1);
    } else {
        g.dxL = d.dxL;
        g.n_L = (int)std::ceil((ll_hi - ll_lo) / d.dxL) + 1;
    }
    // a degenerate span (all widths equal) still needs a positive spacing
    if (!(g.dxG > 0)) g.dxG = 1e-3;
    if (!(g.dxL > 0)) g.dxL = 1e-3;
    g.n_G = std::max(g.n_G, 2);
    g.n_L = std::max(g.n_L, 2);
    if (g.n_G > kMaxAxis || g.n_L > kMaxAxis || g.n_G * g.n_L > kMaxNodes - 1)
        return fail(RG_ERR_RANGE, "LDM grid %d x %d exceeds the kernel limits (%d per axis, %d nodes)",
                    g.n_G, g.n_L, kMaxAxis, kMaxNodes - 1);
    g.n_ft = n_ft;
    g.n1 = n1;
    g.n2 = n2;
    s->n_nodes = (g.n_G * g.n_L + 1) & ~1;
    // intensity scale: the largest line intensity is at most exp(log_scale_int)
    const double aT = -kC2 * (1.0 / T - 1.0 / L->t_ref);
    const double dens = (c->p_bar * 1e5) / (kKb * T) * 1e-6 * c->x;   // factory.py:908-912
    double lq = -std::numeric_limits<double>::infinity();
    for (int i = 0; i < L->n_iso; ++i) {
        double q = c->q_ratio ? c->q_ratio[i] : 1.0;
        if (lines) RG(q_ratio_of(lines, c, i, &q));
        if (q > 0) lq = std::max(lq, std::log(q));
    }
    double smax = L->s_hi.max_at(aT);
    double ls = (std::isfinite(smax) && dens > 0 && std::isfinite(lq)) ? smax + std::log(dens) + lq : 0.0;
    s->log_scale_int = ls;
    const double head = ls + std::log((double)std::max<int64_t>(L->n, 1) / d.dv);
    s->log_scale_out = (head < 85.0 && ls > -60.0) ? 0.0 : ls;
    return RG_OK;
}

int compute_grid(const rg_lines* L, const Work& W, const rg_conditions* c, SpecHost* s) {
    return compute_grid_env(L->env, L, W.desc, W.n, W.n1, W.n2, c, s);
}

// Envelope of a host line list (per-iso v0 range, width and intensity hulls).
int build_envelope(const rg_line_arrays* in, const rg_isotopes* iso, Envelope* E) {
    NvtxRange nvtx_("rg/envelopes");
    if (!in || !iso) return fail(RG_ERR_ARG, "NULL argument");
    if (in->n <= 0) return fail(RG_ERR_ARG, "empty line list");
    if (!in->v0 || !in->s_ref || !in->e_low || !in->g_air || !in->g_self || !in->n_air)
        return fail(RG_ERR_ARG, "a required line column is NULL");
    if (iso->n_iso < 1 || iso->n_iso > kMaxIso) return fail(RG_ERR_ARG, "n_iso %d not in [1,16]", iso->n_iso);
    if (!(iso->t_ref > 0)) return fail(RG_ERR_ARG, "t_ref must be positive");
    const int64_t n = in->n;
    E->n = n;
    E->n_iso = iso->n_iso;
    E->t_ref = iso->t_ref;
    for (int i = 0; i < E->n_iso; ++i) {
        if (!(iso->molar_mass[i] > 0)) return fail(RG_ERR_ARG, "molar_mass[%d] must be positive", i);
        // log FWHM_G - log v0 - 0.5 log T = log(2 sqrt(2 NA k ln2 / M) / c)  (broadening.py:170-172)
        E->log_c2Mm[i] = std::log(2.0 / kCcgs * std::sqrt(2.0 * kNA * kKbCgs * kLn2 / iso->molar_mass[i]));
        E->lv_min[i] = std::numeric_limits<double>::infinity();
        E->lv_max[i] = -std::numeric_limits<double>::infinity();
    }
    E->max_abs_delta = 0.0;
    {   // per-isotope log v0 range and the largest |shift|, over host threads;
        // the first bad line (lowest index) is reported
        struct Part {
            double lmin[kMaxIso], lmax[kMaxIso], dmax = 0.0;
            int64_t bad = -1;
        };
        const int T = host_chunk_count(n, kHostMinPerThread);
        std::vector<Part> part(T);
        run_host_chunks(T, n, [&](int t, int64_t i0, int64_t i1) {
            Part& p = part[t];
            for (int k = 0; k < kMaxIso; ++k) {
                p.lmin[k] = std::numeric_limits<double>::infinity();
                p.lmax[k] = -std::numeric_limits<double>::infinity();
            }
            for (int64_t i = i0; i < i1; ++i) {
                const int k = in->iso ? in->iso[i] : 0;
                if (k >= E->n_iso || !(in->v0[i] > 0)) {
                    p.bad = i;
                    return;
                }
                const double lv = std::log(in->v0[i]);
                p.lmin[k] = std::min(p.lmin[k], lv);
                p.lmax[k] = std::max(p.lmax[k], lv);
                if (in->delta) p.dmax = std::max(p.dmax, (double)std::fabs(in->delta[i]));
            }
        });
        for (const Part& p : part) {
            if (p.bad >= 0) {
                const int64_t i = p.bad;
                const int k = in->iso ? in->iso[i] : 0;
                if (k >= E->n_iso) return fail(RG_ERR_ARG, "iso[%lld] = %d >= n_iso", (long long)i, k);
                return fail(RG_ERR_ARG, "v0[%lld] must be positive", (long long)i);
            }
            for (int k = 0; k < E->n_iso; ++k) {
                E->lv_min[k] = std::min(E->lv_min[k], p.lmin[k]);
                E->lv_max[k] = std::max(E->lv_max[k], p.lmax[k]);
            }
            E->max_abs_delta = std::max(E->max_abs_delta, p.dmax);
        }
    }
    struct WidthSrc : PointSource {
        const rg_line_arrays* in;
        bool lo;
        int64_t size() const override { return in->n; }
        void get(int64_t i, double* a, double* b) const override {
            *a = in->n_air[i];
            float g = lo ? std::min(in->g_self[i], in->g_air[i]) : std::max(in->g_self[i], in->g_air[i]);
            *b = g > 0 ? std::log((double)g) : -std::numeric_limits<double>::infinity();
        }
        bool valid_a(int64_t i, double* a) const override {   // log g finite <=> 0 < g < inf
            *a = in->n_air[i];
            const float g = lo ? std::min(in->g_self[i], in->g_air[i]) : std::max(in->g_self[i], in->g_air[i]);
            return std::isfinite(*a) && g > 0 && std::isfinite(g);
        }
    };
    WidthSrc wlo, whi;
    wlo.in = whi.in = in;
    wlo.lo = true;
    whi.lo = false;
    E->wl_lo = lower_hull_src(wlo);
    E->wl_hi = upper_hull_src(whi);
    if (E->wl_lo.a.empty() || E->wl_hi.a.empty())
        return fail(RG_ERR_ARG, "no line has a positive broadening coefficient");
    struct SSrc : PointSource {
        const rg_line_arrays* in;
        double c2_tref;
        int64_t size() const override { return in->n; }
        void get(int64_t i, double* a, double* b) const override {
            *a = in->e_low[i];
            double s = in->s_ref[i];
            *b = s > 0 ? std::log(s) - std::log(-std::expm1(-c2_tref * in->v0[i]))
                       : -std::numeric_limits<double>::infinity();
        }
        // b finite <=> 0 < s < inf and -expm1(-x) > 0, x = c2 v0 / Tref (v0 > 0
        // is checked before the hulls; expm1(-x) is nonzero for every x > 0)
        bool valid_a(int64_t i, double* a) const override {
            *a = in->e_low[i];
            const double s = in->s_ref[i];
            return std::isfinite(*a) && s > 0 && std::isfinite(s) && c2_tref * in->v0[i] > 0;
        }
    };
    SSrc ss;
    ss.in = in;
    ss.c2_tref = kC2 / E->t_ref;
    E->s_hi = upper_hull_src(ss);
    return RG_OK;
}

// LDM / FFT workspace for n_nodes rows at the current geometry (row_stride,
// n), stream ordered.  The buffers grow by bytes (x1.25 margin) and are
// reused across geometries, so a server slot that runs requests of many sizes
// reallocates only when a request is larger than any before it.
int ensure_workspace(Work& W, int n_nodes, cudaStream_t st) {
    const size_t per_l = sizeof(float) * (size_t)W.row_stride, per_y = sizeof(float2) * (size_t)W.n;
    auto fits = [&](int nodes) { return nodes * per_l <= W.ldm_bytes && (size_t)(nodes / 2) * per_y <= W.y_bytes; };
    if (!fits(n_nodes)) {
        const size_t want_l = std::max<size_t>((size_t)n_nodes * per_l, (size_t)(W.ldm_bytes * 1.25));
        const size_t want_y = std::max<size_t>((size_t)(n_nodes / 2) * per_y, (size_t)(W.y_bytes * 1.25));
        if (W.ldm) CU(cudaFreeAsync(W.ldm, st));
        if (W.y) CU(cudaFreeAsync(W.y, st));
        W.ldm = nullptr;
        W.y = nullptr;
        W.ldm_bytes = W.y_bytes = 0;
        W.nodes_cap = 0;
        CU(cudaMallocAsync((void**)&W.ldm, want_l, st));
        W.ldm_bytes = want_l;
        CU(cudaMallocAsync((void**)&W.y, want_y, st));
        W.y_bytes = want_y;
    }
    W.nodes_cap = (int)std::min<size_t>(W.ldm_bytes / per_l, 2 * (W.y_bytes / per_y)) & ~1;
    return RG_OK;
}

// Entries of the scatter's per-tile line-range table: at least the tiles of
// any CTA, whatever tile width the shape takes (>= 32 columns), so at most
// ceil(ceil(n_v / 32) / sms) while the grid is one CTA per SM, and never more
// than kScatMaxTilesPerCta (more CTAs are launched past that); even.
int scatter_rng_cap(int64_t n_v, int sms) {
    const int64_t per = ((n_v + 31) / 32 + std::max(sms, 1) - 1) / std::max(sms, 1);
    const int cap = (int)std::min<int64_t>(kScatMaxTilesPerCta, std::max<int64_t>(per, 1));
    return (cap + 1) & ~1;
}

// Shape of the persistent scatter (one 1024-thread CTA per SM): TMA ring
// stages, chunk (lines) and tile width (columns, a multiple of 32 for the bank
// swizzle), the widest tile that fits beside the ring, the line-range table
// (rng_cap entries) and coef_bytes of skeleton projection data (0 without).
int scatter_shape(int n_nodes, bool wide, size_t coef_bytes, int rng_cap, int* chunk, int* TK, int* stages,
                  size_t* smem) {
    size_t avail = 0;
    RG(scatter_smem_optin(&avail, wide));
    const size_t word = wide ? 8 : 4;   // bytes per tile cell
    auto tile_cols = [&](int S, int ch) {   // widest tile next to the ring (rows of tk + 1 words)
        const size_t fixed = scatter_fixed_smem(ch, S, rng_cap) + coef_bytes + 16;
        if (fixed >= avail) return 0;
        return std::min(1024, ((int)((avail - fixed) / (word * (size_t)n_nodes)) - 1) / 32 * 32);
    };
    auto take = [&](int S, int ch, int tk) {
        *chunk = ch;
        *TK = tk;
        *stages = S;
        *smem = scatter_fixed_smem(ch, S, rng_cap) + scatter_coef_offset((size_t)n_nodes * (tk + 1), word) +
                coef_bytes;
        return RG_OK;
    };
    // GB300 sweeps (CO2 5M / 128 nodes, H2O 100M / 288 nodes): one line per
    // consumer thread per chunk (992 = 31 warps) in three stages while the tile
    // keeps >= 192 columns (CO2 5M: 256 columns, or 224 beside the skeleton
    // projection's 17 KB of tensor-core fragments, where three stages beat two
    // 1536-line ones by 2%); else two 1536-line stages (wider tiles than 2048)
    if (tile_cols(3, 992) >= 192) return take(3, 992, tile_cols(3, 992));
    if (tile_cols(2, 1536) >= 64) return take(2, 1536, tile_cols(2, 1536));
    for (int min_tk : {64, 32})
        for (int ch : {1024, 512, 256})
            if (tile_cols(2, ch) >= min_tk) return take(2, ch, tile_cols(2, ch));
    return fail(RG_ERR_RANGE, "LDM grid of %d nodes does not fit a shared-memory tile", n_nodes);
}

// Shared-memory bytes of the skeleton projection beside the scatter's tile:
// the tensor-core flush's section (32-bit tiles, where the grid has one) or
// the FP32 coefficients.
size_t fuse_smem_bytes(const ProjArgs* fuse, bool wide) {
    if (!fuse) return 0;
    if (!wide && fuse->flush) return flush_tc_bytes(fuse->flush_ks, fuse->flush_nr);
    return sizeof(float) * (size_t)fuse->n_nodes * fuse->rows_pad;
}

// fuse: the skeleton projection done by the scatter's flush (nullable).
int build_scatter_args(const rg_lines* L, const Work& W, const rg_conditions* c, const SpecHost& s, bool wide,
                       const ProjArgs* fuse, ScatterArgs* a) {
    const rg_grid& g = s.grid;
    std::memset(a, 0, sizeof *a);
    a->v0 = L->v0;
    a->ls2 = L->ls2;
    a->el = L->el;
    a->ga = L->ga;
    a->gs = L->gs;
    a->na = L->na;
    a->dl = L->dl;
    a->iso = L->n_iso > 1 ? L->iso : nullptr;
    a->col_start = W.col_start;
    a->col_off = W.col_off;
    a->col_count = W.col_count;
    a->n_v = (int)W.desc.n_v;
    a->n_nodes = s.n_nodes;
    a->NG = g.n_G;
    a->NL = g.n_L;
    a->row_stride = W.row_stride;
    a->ldm = W.ldm;
    const size_t coef_bytes = fuse_smem_bytes(fuse, wide);
    if (fuse) {
        a->proj_coef = fuse->coef;
        a->proj_rows = fuse->rows;
        a->proj_rp = fuse->rows_pad;
        a->n_real = fuse->n_nodes;
        if (!wide && fuse->flush) {
            a->proj_frag = fuse->flush;
            a->proj_ks = fuse->flush_ks;
            a->proj_nr = fuse->flush_nr;
        }
    }
    size_t smem_unused;
    a->rng_cap = scatter_rng_cap(W.desc.n_v, L->ctx->sms);
    RG(scatter_shape(s.n_nodes, wide, coef_bytes, a->rng_cap, &a->chunk, &a->TK, &a->stages, &smem_unused));
    a->n_tiles = (int)((W.desc.n_v + a->TK - 1) / a->TK);
    a->cmax = W.cmax_dev;
    a->err = W.err;
    if (s.p_atm > W.p_atm_max)
        return fail(RG_ERR_RANGE, "pressure %g atm above the shift-index limit %g atm", s.p_atm, W.p_atm_max);
    a->margin_cols = (int)std::ceil(L->env.max_abs_delta * s.p_atm / W.desc.dv) + 1;
    split(W.desc.vmin, &a->vmin_hi, &a->vmin_lo);
    split(1.0 / W.desc.dv, &a->inv_dv_hi, &a->inv_dv_lo);
    a->p_atm = (float)s.p_atm;
    a->x_self = (float)c->x;
    const double T = c->T;
    a->lgG_scale = (float)(kLn2 / g.dxG);
    double lv_lo = std::numeric_limits<double>::infinity(), lv_hi = -lv_lo;
    for (int i = 0; i < L->n_iso; ++i)
        if (L->env.lv_min[i] <= L->env.lv_max[i]) {
            lv_lo = std::min(lv_lo, L->env.lv_min[i]);
            lv_hi = std::max(lv_hi, L->env.lv_max[i]);
        }
    const double lv_ref = 0.5 * (lv_lo + lv_hi);
    a->inv_vref = (float)std::exp(-lv_ref);
    for (int i = 0; i < L->n_iso; ++i)
        a->cG[i] = (float)((lv_ref + L->env.log_c2Mm[i] + 0.5 * std::log(T) - g.log_wG_min) / g.dxG);
    a->lgL_scale = (float)(kLn2 / g.dxL);
    a->tL = (float)(std::log(L->t_ref / T) / g.dxL);
    a->cL = (float)((std::log(2.0 * s.p_atm) - g.log_wL_min) / g.dxL);
    split(-kC2 * (1.0 / T - 1.0 / L->t_ref) * kLog2e, &a->aT_hi, &a->aT_lo);
    const double dens = (c->p_bar * 1e5) / (kKb * T) * 1e-6 * c->x;
    for (int i = 0; i < L->n_iso; ++i) {
        double q;
        RG(q_ratio_of(L, c, i, &q));
        double b = (q > 0 && dens > 0) ? (std::log(q * dens) - s.log_scale_int) * kLog2e : -1e30;
        if (b < -1e30) b = -1e30;
        split(b, &a->bI_hi[i], &a->bI_lo[i]);
    }
    a->stim_c = (float)(kC2 / T * kLog2e);
    a->in_window = W.count_lines ? W.counter : nullptr;
    a->wait_limit = W.scat_wait;
    a->withhold = W.scat_withhold;
    return RG_OK;
}

// folded Voigt FT of one node (broadening.py:1900-1926), FP64 on the host
void node_fold(double dv, double wG, double wL, double thresh, int* nfold, double* norm) {
    auto V = [&](double f) {
        double g = std::exp(-std::pow(kPi * f * wG, 2) / (4.0 * kLn2));
        return g * std::exp(-kPi * f * wL);
    };
    const double h = 1.0 / (2.0 * dv);
    int n = 1;
    double v0 = V(0.0);
    while (V(n * h) >= thresh && n < 255) {
        // bin 0: w_fold[0][0] = 0, w_fold[1][0] = 1/(2 dv)
        v0 += V(n * h + ((n & 1) ? h : 0.0));
        ++n;
    }
    *nfold = n - 1;
    *norm = 1.0 / v0;
}

// Row-kernel arguments of one spectrum: FFT geometry and the folded,
// normalised Voigt FT parameters of every node of the grid.
void fill_voigt_args(Work& W, const SpecHost& s, VoigtArgs* va) {
    const rg_grid& g = s.grid;
    va->f2 = W.f2;
    va->threads = row_threads(W.f2);
    const RowLayout rl = row_layout(W.n2);
    va->pairs_per_pass = rl.pairs;
    va->row_twiddle_table = rl.twr;
    va->n1 = W.n1;
    va->n2 = W.n2;
    va->n = W.n;
    va->n_pairs = s.n_nodes / 2;
    va->n_nodes = s.n_nodes;
    va->NL = g.n_L;
    va->y = W.y;
    va->g = W.g;
    va->tw_hi = W.tw_hi;
    va->tw_lo = W.tw_lo;
    va->inv_ndv = (float)(1.0 / ((double)W.n * W.desc.dv));
    va->half_fs = (float)(0.5 / W.desc.dv);
    const double thresh = W.desc.folding_thresh > 0 ? W.desc.folding_thresh : 1e-6;
    const double key[8] = {g.log_wG_min, g.dxG, (double)g.n_G, g.log_wL_min, g.dxL, (double)g.n_L, W.desc.dv, thresh};
    if (W.va_valid && std::equal(key, key + 8, W.va_key) && (int)W.va_norm.size() == s.n_nodes) {
        std::copy(W.va_alpha.begin(), W.va_alpha.end(), va->alpha);
        std::copy(W.va_beta.begin(), W.va_beta.end(), va->beta);
        std::copy(W.va_norm.begin(), W.va_norm.end(), va->norm);
        std::copy(W.va_lnorm.begin(), W.va_lnorm.end(), va->lnorm);
        std::copy(W.va_nfold.begin(), W.va_nfold.end(), va->nfold);
        va->any_fold = W.va_any_fold;
        return;
    }
    for (int l = 0; l < g.n_G; ++l) {
        double wG = std::exp(g.log_wG_min + l * g.dxG);
        va->alpha[l] = (float)(std::pow(kPi * wG, 2) / (4.0 * kLn2) * kLog2e);
    }
    for (int m = 0; m < g.n_L; ++m) {
        double wL = std::exp(g.log_wL_min + m * g.dxL);
        va->beta[m] = (float)(kPi * wL * kLog2e);
    }
    va->any_fold = 0;
    for (int node = 0; node < s.n_nodes; ++node) {
        if (node >= g.n_G * g.n_L) {
            va->norm[node] = 0.f;
            va->lnorm[node] = -std::numeric_limits<float>::infinity();
            va->nfold[node] = 0;
            continue;
        }
        int l = node / g.n_L, m = node % g.n_L;
        int nf;
        double nrm;
        node_fold(W.desc.dv, std::exp(g.log_wG_min + l * g.dxG), std::exp(g.log_wL_min + m * g.dxL), thresh, &nf,
                  &nrm);
        va->norm[node] = (float)nrm;
        va->lnorm[node] = (float)std::log2(nrm);
        va->nfold[node] = (unsigned char)nf;
        if (nf) va->any_fold = 1;
    }
    std::copy(key, key + 8, W.va_key);
    W.va_alpha.assign(va->alpha, va->alpha + g.n_G);
    W.va_beta.assign(va->beta, va->beta + g.n_L);
    W.va_norm.assign(va->norm, va->norm + s.n_nodes);
    W.va_lnorm.assign(va->lnorm, va->lnorm + s.n_nodes);
    W.va_nfold.assign(va->nfold, va->nfold + s.n_nodes);
    W.va_any_fold = va->any_fold;
    W.va_valid = true;
}

// Merged layout of one spectrum.  Without folding, the Voigt FT of node
// (l, m) factors into the Gaussian FT of l times the Lorentzian FT of m.
// Where the Gaussian FT of node l is below 2^-30 at the Nyquist frequency,
// multiplying by it equals a real-space convolution with the sampled Gaussian
// profile (its inverse DFT, Poisson summation; truncated where the profile
// falls below 1e-8 of its peak).  The node rows of those "wide" l are
// convolved and summed into one row per wL node before the FFT, so only
// n_L x (1 + narrow l) rows are transformed instead of n_G x n_L; the other
// rows keep the full (folded, normalised) Voigt FT.  Wide nodes have no folded
// copies (their FT is below 2^-30 beyond the Nyquist frequency).  Used when
// at least two l are wide.
bool plan_merge(const Work& W, const SpecHost& s, const VoigtArgs& va, GaussArgs* ga, VoigtArgs* vm,
                int* out_rows) {
    if (!W.allow_merge) return false;
    const rg_grid& g = s.grid;
    const double dv = W.desc.dv;
    std::memset(ga, 0, sizeof *ga);
    int K_max = 0;
    for (int l = 0; l < g.n_G; ++l) {
        const double wG = std::exp(g.log_wG_min + l * g.dxG);
        const double nyq = std::pow(kPi * wG / (2.0 * dv), 2) / (4.0 * kLn2) * kLog2e;   // -log2 G(f_nyq)
        const int K = (int)std::ceil(2.5770 * wG / dv);   // exp(-4 ln2 (K dv / wG)^2) <= 1e-8
        bool unfolded = true;   // folded copies are below 2^-30 here unless the threshold is lower still
        for (int m = 0; m < g.n_L; ++m) unfolded &= va.nfold[l * g.n_L + m] == 0;
        if (nyq >= 30.0 && K <= kGaussMaxK && unfolded) {
            const int w = ga->n_wide++;
            ga->wide_l[w] = l;
            ga->K[w] = K;
            ga->c[w] = (float)(dv * 2.0 * std::sqrt(kLn2 / kPi) / wG);
            ga->a2[w] = (float)(4.0 * kLn2 * (dv / wG) * (dv / wG) * kLog2e);
            K_max = std::max(K_max, K);
        } else {
            ga->narrow_l[ga->n_narrow++] = l;
        }
    }
    if (ga->n_wide < 2) return false;
    // Base Gaussian in Fourier space: g_l = d_l conv g_b with sigma_b^2 =
    // sigma_min^2 - 1.2^2, so every residual sigma_d >= 1.2 steps.  The merged
    // rows carry sum_l d_l conv LDM_{l,m} (real space, this stage) and the row
    // kernel multiplies their FT by the base's 2^(-alpha_b f^2) together with
    // the Lorentzian FT.  A sampled residual times the base FT differs from the
    // node's Gaussian FT by the residual's first alias, at most
    // exp(-2 pi^2 d b / (d + b)) for variances d, b in steps^2: ~1e-11 for the
    // CO2 5M grid, <= ~8e-9 for the narrowest wide node (variance 4.2).
    double alpha_b = 0.0;
    {
        // residual taps out to 1e-6 of the kernel's peak (+-5.26 sigma): the mass
        // beyond, erfc(5.26 / sqrt 2) = 1.4e-7 of the kernel, is below the FP32
        // error of the synthesis (~1e-6 of the peak)
        const double kSigMin = 1.2, kTail = std::sqrt(2.0 * std::log(1e6));
        auto sig = [&](int w) { return std::exp(g.log_wG_min + ga->wide_l[w] * g.dxG) / dv / (2.0 * std::sqrt(2.0 * kLn2)); };
        double smin = 1e300;
        for (int w = 0; w < ga->n_wide; ++w) smin = std::min(smin, sig(w));
        const double sb2 = smin * smin - kSigMin * kSigMin;
        if (sb2 > 0) {   // always: a wide node has sigma >= 2 steps
            int ext2 = 0;
            for (int w = 0; w < ga->n_wide; ++w) {
                const double sd2 = sig(w) * sig(w) - sb2;
                ga->K[w] = (int)std::ceil(kTail * std::sqrt(sd2));
                ga->c[w] = (float)(1.0 / std::sqrt(2.0 * kPi * sd2));
                ga->a2[w] = (float)(kLog2e / (2.0 * sd2));
                ext2 = std::max(ext2, ga->K[w]);
            }
            K_max = ext2;
            alpha_b = 2.0 * kPi * kPi * sb2 * dv * dv * kLog2e;   // (pi wG_b)^2 / (4 ln 2) log2 e
        }
    }
    // rows come in blocks of NLv = n_L rounded up to even (a zero row pads odd
    // n_L) so that no pair straddles the merged and a narrow block
    const int NL = g.n_L, NLv = NL + (NL & 1);
    ga->NL = NL;
    ga->NLv = NLv;
    ga->rows = NLv * (1 + ga->n_narrow);
    if (ga->rows >= s.n_nodes) return false;   // no fewer rows (and the FFT workspace holds n_nodes)
    *out_rows = ga->rows;
    ga->n_v = (int)W.desc.n_v;
    ga->ext = K_max;
    ga->out_stride = (ga->n_v + 2 * K_max + 31) / 32 * 32;
    ga->ldm = W.ldm;
    ga->row_stride = W.row_stride;
    ga->cmax = W.cmax_dev;
    *vm = va;
    vm->n_nodes = *out_rows;
    vm->n_pairs = *out_rows / 2;
    vm->NL = NLv;
    vm->alpha[0] = (float)alpha_b;   // merged rows: the base Gaussian's FT (residuals applied already)
    for (int i = 0; i < ga->n_narrow; ++i) vm->alpha[1 + i] = va.alpha[ga->narrow_l[i]];
    vm->alpha[1 + ga->n_narrow] = 0.f;
    for (int r = 0; r < *out_rows; ++r) {
        const int lp = r / NLv, m = r % NLv;
        if (m < NL && lp == 0) {   // merged rows: unfolded, 1 / V(0) = 1
            vm->norm[r] = 1.f;
            vm->lnorm[r] = 0.f;
            vm->nfold[r] = 0;
        } else if (m < NL) {   // narrow node rows keep their folded, normalised Voigt FT
            const int node = ga->narrow_l[lp - 1] * NL + m;
            vm->norm[r] = va.norm[node];
            vm->lnorm[r] = va.lnorm[node];
            vm->nfold[r] = va.nfold[node];
        } else {
            vm->norm[r] = 0.f;
            vm->lnorm[r] = -std::numeric_limits<float>::infinity();
            vm->nfold[r] = 0;
        }
    }
    return true;
}

// rows of the merged-row buffer (one per wL node, plus a zero row for odd
// n_L; the narrow rows are read from the LDM by the column FFT directly)
int NL_merged(const GaussArgs& ga) { return ga.NLv; }

// Skeleton layout of one spectrum (interp_decomp, rg_skeleton.cpp): the
// folded, normalised Voigt transform of every node, sampled at S frequencies
// f_j = (j / (S - 1))^2 / (2 dv) (dense where the wide nodes' transforms
// live; the largest error over the whole DFT grid stays within a few percent
// of the sampled one on the grids tried), is decomposed on the host in FP64.
// Succeeds when at most r_max skeleton rows (rounded up to even) reproduce
// every node's transform within tol; fills the row kernel's arguments (row r
// = skeleton node sk[r], with its own transform) and the projection
// coefficients [n_nodes][rows_pad] in W.proj_host.
// Skeleton projection in the scatter's flush (no LDM round trip through HBM)
// for grids of at most this many nodes; larger grids project in a separate
// pass, with the decomposition computed on the host while the scatter runs.
// Measured on the 288-node H2O 100M grid, also with a tensor-core flush of
// three row blocks: its fragments leave 64-column tiles (4 flush tasks for 31
// warps) and the fused scatter took 1.91 ms against 1.13 + 0.41 ms for the
// scatter and the pass.
constexpr int kFuseMaxNodes = 160;

constexpr int kSkelSamples = 32;
constexpr double kSkelTol = 1e-8;

// The decomposition itself (host only): skeleton nodes sk[0, R) and
// coefficients C[r * n + node] for the n = n_G n_L nodes of grid g.
int skeleton_decomp(const rg_grid& g, double dv, double thresh, double tol, int r_max, std::vector<int>* sk,
                    std::vector<double>* C, int* R, double* err) {
    const int n = g.n_G * g.n_L;
    const double h = 0.5 / dv;
    constexpr int S = kSkelSamples;
    double f[S];
    for (int j = 0; j < S; ++j) f[j] = h * std::pow((double)j / (S - 1), 2);
    std::vector<int> nf(n, 0);
    std::vector<double> nrm(n, 1.0);
    int qmax = 0;
    // folded copies only where the transform at the Nyquist frequency reaches
    // the threshold (node_fold's first test, here from the separable factors)
    std::vector<double> gh(g.n_G), lh(g.n_L);
    for (int l = 0; l < g.n_G; ++l) gh[l] = std::exp(-std::pow(kPi * h * std::exp(g.log_wG_min + l * g.dxG), 2) / (4.0 * kLn2));
    for (int m = 0; m < g.n_L; ++m) lh[m] = std::exp(-kPi * h * std::exp(g.log_wL_min + m * g.dxL));
    for (int node = 0; node < n; ++node) {
        const int l = node / g.n_L, m = node % g.n_L;
        if (!(gh[l] * lh[m] >= thresh)) continue;   // no folded copy: norm 1 / V(0) = 1
        node_fold(dv, std::exp(g.log_wG_min + l * g.dxG), std::exp(g.log_wL_min + m * g.dxL), thresh, &nf[node],
                  &nrm[node]);
        qmax = std::max(qmax, nf[node]);
    }
    // separable factors per folded copy q, at the copy's frequency
    // q h + (q odd ? h - f : f) (broadening.py:1914-1926)
    std::vector<double> Gt((size_t)(qmax + 1) * g.n_G * S), Lt((size_t)(qmax + 1) * g.n_L * S);
    for (int q = 0; q <= qmax; ++q)
        for (int j = 0; j < S; ++j) {
            const double fq = q == 0 ? f[j] : q * h + ((q & 1) ? h - f[j] : f[j]);
            for (int l = 0; l < g.n_G; ++l) {
                const double wG = std::exp(g.log_wG_min + l * g.dxG);
                Gt[((size_t)q * g.n_G + l) * S + j] = std::exp(-std::pow(kPi * fq * wG, 2) / (4.0 * kLn2));
            }
            for (int m = 0; m < g.n_L; ++m) {
                const double wL = std::exp(g.log_wL_min + m * g.dxL);
                Lt[((size_t)q * g.n_L + m) * S + j] = std::exp(-kPi * fq * wL);
            }
        }
    // samples below 1e-30 (far below any tolerance) are flushed to zero:
    // their products would otherwise reach the subnormal range
    std::vector<double> A((size_t)n * S);
    for (int node = 0; node < n; ++node) {
        const int l = node / g.n_L, m = node % g.n_L;
        double* a = &A[(size_t)node * S];
        for (int j = 0; j < S; ++j) {
            double v = 0.0;
            for (int q = 0; q <= nf[node]; ++q)
                v += Gt[((size_t)q * g.n_G + l) * S + j] * Lt[((size_t)q * g.n_L + m) * S + j];
            v *= nrm[node];
            a[j] = v < 1e-30 ? 0.0 : v;
        }
    }
    sk->assign(r_max, 0);
    C->assign((size_t)r_max * n, 0.0);
    return interp_decomp(A.data(), S, n, tol, r_max, sk->data(), C->data(), R, err);
}

// Node order of the scatter flush's tensor-core form (steps of 8 nodes, see
// flush_tc): tile rows have a pitch of 1 (mod 32) words, so node m sits in the
// bank class m mod 32 = 8 ((m / 8) mod 4) + m mod 8, and the four nodes that
// one A-fragment load reads (t = 0..3) must come from the classes v, v + 8,
// v + 16, v + 24.  Nodes are grouped by (m mod 8, (m / 8) mod 4) into such
// quadruples; a class short of nodes repeats one of its nodes (real = 0: a
// zero coefficient), two quadruples make a step.  Below 32 nodes some classes
// are empty and no order is conflict-free: the natural one, padded.
void flush_node_order(int n, std::vector<int>* nodes, std::vector<char>* real) {
    nodes->clear();
    real->clear();
    if (n < 32) {
        for (int j = 0; j < (n + 7) / 8 * 8; ++j) {
            nodes->push_back(j < n ? j : 0);
            real->push_back(j < n ? 1 : 0);
        }
        return;
    }
    std::vector<int> quad_nodes;
    std::vector<char> quad_real;
    for (int v = 0; v < 8 && v < n; ++v) {
        std::vector<int> cls[4];
        for (int m = v; m < n; m += 8) cls[(m / 8) % 4].push_back(m);
        size_t cnt = 0;
        int any = -1;
        for (auto& c : cls) {
            cnt = std::max(cnt, c.size());
            if (any < 0 && !c.empty()) any = c[0];
        }
        for (size_t i = 0; i < cnt; ++i)
            for (int w = 0; w < 4; ++w) {
                const bool have = i < cls[w].size();
                quad_nodes.push_back(have ? cls[w][i] : !cls[w].empty() ? cls[w][0] : any);
                quad_real.push_back(have ? 1 : 0);
            }
    }
    if (quad_nodes.size() % 8) {   // odd number of quadruples: a zero one
        for (int j = 0; j < 4; ++j) {
            quad_nodes.push_back(quad_nodes[quad_nodes.size() - 4]);
            quad_real.push_back(0);
        }
    }
    *nodes = std::move(quad_nodes);
    *real = std::move(quad_real);
}

bool plan_skeleton(Work& W, const SpecHost& s, const VoigtArgs& va, int r_max, VoigtArgs* vk, ProjArgs* pa,
                   double* err_out) {
    const rg_grid& g = s.grid;
    const int n = g.n_G * g.n_L;
    r_max = std::min(r_max, kProjMaxRows);
    if (!W.allow_skeleton || n < 4 || r_max < 2) return false;
    const double thresh = W.desc.folding_thresh > 0 ? W.desc.folding_thresh : 1e-6;
    const double tol = W.desc.layout_tol > 0 ? W.desc.layout_tol : kSkelTol;
    const double key[10] = {g.log_wG_min, g.dxG, (double)g.n_G, g.log_wL_min, g.dxL, (double)g.n_L,
                            W.desc.dv, thresh, tol, (double)r_max};
    const bool hit = W.skel_valid && std::equal(key, key + 10, W.skel_key);
    if (!hit) {
        W.skel_dev = false;
        std::copy(key, key + 10, W.skel_key);
        W.skel_valid = true;
        W.skel_R = 0;   // no skeleton layout for this grid (cached as well)
        W.skel_flush_ks = 0;
        std::vector<int> sk;
        std::vector<double> C;
        int R = 0;
        double err = 0.0;
        if (skeleton_decomp(g, W.desc.dv, thresh, tol, r_max, &sk, &C, &R, &err) != RG_OK) return false;
        const int rows = R + (R & 1);
        if (R < 1 || rows > r_max) return false;
        const int rp = proj_rows_pad(rows);
        // coefficients in shared memory: beside the scatter's tile (grids of up
        // to kFuseMaxNodes nodes) or as the projection pass's fragments
        if ((size_t)n * rp * sizeof(float) > 96 * 1024) return false;
        if (n > kFuseMaxNodes && proj_tc_smem((rows + 7) / 8, 2 * ((n + 15) / 16)) > kProjTcSmemMax) return false;
        // [n][rp] coefficients (the FP32 forms), then the tensor-core pass's B
        // fragments: TF32 hi / lo parts, [nr][ks][part][lane][2] with
        // b0, b1 = C[8 nr + g][8 ks + t], C[8 nr + g][8 ks + t + 4], g = lane / 4,
        // t = lane % 4
        const int NR = (rows + 7) / 8, KSP = 2 * ((n + 15) / 16);
        // the scatter flush's tensor-core section (fused grids of up to two
        // row blocks): B fragments [ks][nr][lane] (b0, b1 hi, b0, b1 lo) in
        // the flush's node order, then that order as a table [ks][t][2]
        std::vector<int> fl_nodes;
        std::vector<char> fl_real;
        if (n <= kFuseMaxNodes && NR <= 2) flush_node_order(n, &fl_nodes, &fl_real);
        const int KSF = (int)fl_nodes.size() / 8;
        W.proj_host.assign((size_t)n * rp + (size_t)NR * KSP * 128 + flush_tc_bytes(KSF, NR) / sizeof(float), 0.f);
        for (int r = 0; r < R; ++r)
            for (int node = 0; node < n; ++node) W.proj_host[(size_t)node * rp + r] = (float)C[(size_t)r * n + node];
        float* fr = W.proj_host.data() + (size_t)n * rp;
        auto cf = [&](int r, int k) { return r < R && k < n ? (float)C[(size_t)r * n + k] : 0.f; };
        for (int nr = 0; nr < NR; ++nr)
            for (int ks = 0; ks < KSP; ++ks)
                for (int lane = 0; lane < 32; ++lane) {
                    const int g = lane >> 2, t = lane & 3;
                    const float v[2] = {cf(8 * nr + g, 8 * ks + t), cf(8 * nr + g, 8 * ks + t + 4)};
                    for (int i = 0; i < 2; ++i) {
                        const float hi = tf32_round_host(v[i]);
                        fr[((size_t)(nr * KSP + ks) * 2 + 0) * 64 + lane * 2 + i] = hi;
                        fr[((size_t)(nr * KSP + ks) * 2 + 1) * 64 + lane * 2 + i] = tf32_round_host(v[i] - hi);
                    }
                }
        float* ff = fr + (size_t)NR * KSP * 128;
        for (int ks = 0; ks < KSF; ++ks)
            for (int nr = 0; nr < NR; ++nr)
                for (int lane = 0; lane < 32; ++lane) {
                    const int g = lane >> 2, t = lane & 3;
                    float* o = ff + ((size_t)(ks * NR + nr) * 32 + lane) * 4;
                    for (int i = 0; i < 2; ++i) {
                        const int j = 8 * ks + t + 4 * i;
                        const float v = fl_real[j] ? cf(8 * nr + g, fl_nodes[j]) : 0.f;
                        o[i] = tf32_round_host(v);
                        o[2 + i] = tf32_round_host(v - o[i]);
                    }
                }
        int32_t* tbl = reinterpret_cast<int32_t*>(ff + (size_t)KSF * NR * 128);
        for (int ks = 0; ks < KSF; ++ks)
            for (int t = 0; t < 4; ++t) {
                tbl[ks * 8 + 2 * t] = fl_nodes[8 * ks + t];
                tbl[ks * 8 + 2 * t + 1] = fl_nodes[8 * ks + t + 4];
            }
        W.skel_flush_ks = KSF;
        W.skel_nodes.assign(sk.begin(), sk.begin() + R);
        W.skel_R = R;
        W.skel_err = err;
    }
    if (W.skel_R == 0) return false;
    if (W.proj_fixed && sizeof(float) * W.proj_host.size() > W.proj_bytes) return false;
    const int R = W.skel_R;
    const int rows = R + (R & 1);
    const int rp = proj_rows_pad(rows);
    const double err = W.skel_err;
    const std::vector<int>& sk = W.skel_nodes;
    *vk = va;
    vk->rowwise = 1;
    vk->n_nodes = rows;
    vk->n_pairs = rows / 2;
    vk->any_fold = 0;
    for (int r = 0; r < rows; ++r) {
        if (r < R) {
            const int node = sk[r];
            vk->alpha[r] = va.alpha[node / g.n_L];
            vk->beta[r] = va.beta[node % g.n_L];
            vk->norm[r] = va.norm[node];
            vk->lnorm[r] = va.lnorm[node];
            vk->nfold[r] = va.nfold[node];
            if (va.nfold[node]) vk->any_fold = 1;
        } else {   // zero pad row
            vk->alpha[r] = vk->beta[r] = 0.f;
            vk->norm[r] = 0.f;
            vk->lnorm[r] = -std::numeric_limits<float>::infinity();
            vk->nfold[r] = 0;
        }
    }
    std::memset(pa, 0, sizeof *pa);
    pa->ldm = W.ldm;
    pa->row_stride = W.row_stride;
    pa->n_v = (int)W.desc.n_v;
    pa->n_nodes = n;   // the pad node row of an odd grid is not read
    pa->rows = rows;
    pa->rows_pad = rp;
    pa->mtiles = (rows + 7) / 8;   // the tensor-core pass's 8-row n-tiles
    pa->ksteps = 2 * ((n + 15) / 16);
    pa->flush_ks = W.skel_flush_ks;
    pa->flush_nr = W.skel_flush_ks ? pa->mtiles : 0;
    *err_out = err;
    return true;
}

// After a synchronisation: report (once) a bounded device wait that gave up.
int take_err(Work& W) {
    if (*W.err_host) {
        *W.err_host = 0;
        return fail(RG_ERR_TIMEOUT, "a bounded device wait in the scatter gave up; the spectrum is invalid");
    }
    return RG_OK;
}

// Enqueue one spectrum on `st` into W's buffers: scatter, the four FFT/Voigt
// stages (unless ldm_only), and the publication of the device error flag.
// ev: 6 events recorded between stages (nullable).
// Shape of the scatter with the 32- or 64-bit accumulator: arguments, grid
// (one persistent CTA per SM, more only past kScatMaxTilesPerCta tiles each)
// and dynamic shared memory.
int scatter_launch_shape(const rg_lines* L, const Work& W, const rg_conditions* c, const SpecHost& s, bool wide,
                         const ProjArgs* fuse, ScatterArgs* sa, int* grid, size_t* smem) {
    RG(build_scatter_args(L, W, c, s, wide, fuse, sa));
    int ch_unused, tk_unused, st_unused;
    RG(scatter_shape(s.n_nodes, wide, fuse_smem_bytes(fuse, wide), sa->rng_cap, &ch_unused, &tk_unused, &st_unused,
                     smem));
    const int sms = L->ctx->sms;
    *grid = std::max(std::min(sa->n_tiles, sms), (sa->n_tiles + kScatMaxTilesPerCta - 1) / kScatMaxTilesPerCta);
    if ((sa->n_tiles + *grid - 1) / *grid > sa->rng_cap)
        return fail(RG_ERR_RANGE, "scatter tiles per CTA above the line-range table");
    return RG_OK;
}

// The FFT-stage layout of one spectrum (rg_plan_desc.layout) and its
// arguments; for the skeleton layout the projection coefficients are
// uploaded (stream ordered) into W.proj_coef.
struct LayoutPlan {
    std::unique_ptr<VoigtArgs> va, vm, vk;
    std::unique_ptr<GaussArgs> ga;
    ProjArgs pa{};
    bool merged = false, skel = false;
    int m_rows = 0;
};

int plan_layout(Work& W, const SpecHost& s, cudaStream_t st, LayoutPlan* lp) {
    lp->va = std::make_unique<VoigtArgs>();
    lp->vm = std::make_unique<VoigtArgs>();
    lp->vk = std::make_unique<VoigtArgs>();
    lp->ga = std::make_unique<GaussArgs>();
    fill_voigt_args(W, s, lp->va.get());
    const int lay = W.desc.layout;
    int& m_rows = lp->m_rows;
    bool merged = lay != 1 && lay != 3 && plan_merge(W, s, *lp->va, lp->ga.get(), lp->vm.get(), &m_rows);
    double sk_err = 0.0;
    const int alt_rows = merged ? m_rows : s.n_nodes;
    // auto: skeleton rows when no more than the merged rows (whose Gaussian
    // stage costs more than the projection), or 3/4 of the node rows
    const bool skel = (lay == 0 || lay == 3) &&
                      plan_skeleton(W, s, *lp->va, lay == 3 ? kProjMaxRows : merged ? alt_rows : 3 * alt_rows / 4,
                                    lp->vk.get(), &lp->pa, &sk_err);
    if (skel) merged = false;
    else if (lay == 3) merged = plan_merge(W, s, *lp->va, lp->ga.get(), lp->vm.get(), &m_rows);
    lp->merged = merged;
    lp->skel = skel;
    W.last_layout = skel ? 3 : merged ? 2 : 1;
    W.last_layout_err = skel ? sk_err : 0.0;
    W.last_fft_rows = skel ? lp->pa.rows : merged ? m_rows : s.n_nodes;
    W.last_merged_rows = merged ? lp->ga->NL : 0;
    W.last_ext = merged ? lp->ga->ext : 0;
    if (skel) {
        const size_t need = sizeof(float) * W.proj_host.size();
        if (need > W.proj_bytes) {
            if (W.proj_coef) CU(cudaFreeAsync(W.proj_coef, st));
            W.proj_coef = nullptr;
            W.proj_bytes = 0;
            W.skel_dev = false;
            const size_t want = std::max<size_t>(need, 64 * 1024);
            CU(cudaMallocAsync((void**)&W.proj_coef, want, st));
            W.proj_bytes = want;
        }
        if (!W.skel_dev) {
            // pageable source: staged before the call returns, so the host
            // vector may be refilled by the next spectrum at once
            CU(cudaMemcpyAsync(W.proj_coef, W.proj_host.data(), need, cudaMemcpyHostToDevice, st));
            W.skel_dev = true;
        }
        lp->pa.coef = W.proj_coef;
        // the tensor-core fragments follow the [n][rp] coefficients, then the
        // scatter flush's section
        lp->pa.frag = W.proj_coef + (size_t)lp->pa.n_nodes * lp->pa.rows_pad;
        lp->pa.flush = lp->pa.flush_ks ? lp->pa.frag + (size_t)lp->pa.mtiles * lp->pa.ksteps * 128 : nullptr;
    }
    return RG_OK;
}


int enqueue_spectrum(const rg_lines* L, Work& W, const rg_conditions* c, const SpecHost& s, float* out,
                     cudaStream_t st, cudaEvent_t* ev, bool ldm_only) {
    RG(ensure_workspace(W, s.n_nodes, st));
    const int n_v = (int)W.desc.n_v;
    const int n_real = s.grid.n_G * s.grid.n_L;
    LayoutPlan lp;
    bool planned = false;
    if (!ldm_only && W.allow_skeleton && (W.desc.layout == 0 || W.desc.layout == 3) && n_real <= kFuseMaxNodes) {
        RG(plan_layout(W, s, st, &lp));
        planned = true;
    }
    lp.pa.sms = L->ctx->sms;
    const ProjArgs* fuse = planned && lp.skel ? &lp.pa : nullptr;
    if (ev) CU(cudaEventRecord(ev[0], st));
    if (W.count_lines) CU(cudaMemsetAsync(W.counter, 0, sizeof(unsigned long long), st));
    // accumulator width: forced, or from the densest column when the host knows
    // it (plans); otherwise both variants are launched and the device decides
    if (W.desc.accumulator || W.cmax_host >= 0) {
        const bool wide = W.desc.accumulator ? W.desc.accumulator == 64 : fx_wide((int)W.cmax_host);
        ScatterArgs sa;
        int grid;
        size_t smem;
        RG(scatter_launch_shape(L, W, c, s, wide, fuse, &sa, &grid, &smem));
        RG(launch_scatter(sa, grid, kScatThreads, smem, wide, st));
        W.last_accum = wide ? 64 : 32;
    } else {
        ScatterArgs a32, a64;
        int g32, g64;
        size_t m32, m64;
        RG(scatter_launch_shape(L, W, c, s, false, fuse, &a32, &g32, &m32));
        RG(scatter_launch_shape(L, W, c, s, true, fuse, &a64, &g64, &m64));
        RG(launch_scatter_auto(a32, a64, std::max(g32, g64), kScatThreads, std::max(m32, m64), st));
        W.last_accum = 0;
    }
    if (fuse) W.last_layout = 4;
    if (ev) CU(cudaEventRecord(ev[1], st));
    if (!ldm_only) {
        ColFftArgs ca;
        std::memset(&ca, 0, sizeof ca);
        ca.f1 = W.f1;
        ca.n1 = W.n1;
        ca.n2 = W.n2;
        ca.B = W.B;
        ca.n_v = n_v;
        ca.n = W.n;
        ca.row_stride = W.row_stride;
        ca.n_pairs = s.n_nodes / 2;
        ca.ldm = W.ldm;
        ca.cmax = W.cmax_dev;
        ca.twiddle = !row_layout(W.n2).twr;
        ca.y = W.y;
        ca.tw_hi = W.tw_hi;
        ca.tw_lo = W.tw_lo;
        if (!planned) {
            RG(plan_layout(W, s, st, &lp));
            lp.pa.sms = L->ctx->sms;
        }
        const bool skel = lp.skel, merged = lp.merged;
        GaussArgs* ga = lp.ga.get();
        ProjArgs& pa = lp.pa;
        if (skel) {
            if (!fuse) RG(launch_node_project(pa, st));
            if (ev) CU(cudaEventRecord(ev[6], st));
            ca.n_pairs = pa.rows / 2;
            RG(launch_col_fft_fwd(ca, st));
        } else if (merged) {
            const size_t need = sizeof(float) * (size_t)NL_merged(*ga) * (size_t)ga->out_stride;
            if (need > W.mrow_bytes) {
                const size_t want = std::max(need, (size_t)(W.mrow_bytes * 1.25));
                if (W.mrow) CU(cudaFreeAsync(W.mrow, st));
                W.mrow = nullptr;
                W.mrow_bytes = 0;
                CU(cudaMallocAsync((void**)&W.mrow, want, st));
                W.mrow_bytes = want;
            }
            ga->out = W.mrow;
            if (ga->NLv > ga->NL)   // zero pad row of odd n_L
                CU(cudaMemsetAsync(W.mrow + (size_t)ga->NL * ga->out_stride, 0, sizeof(float) * ga->out_stride, st));
            RG(launch_gauss_merge(*ga, ga->NL, st));
            if (ev) CU(cudaEventRecord(ev[6], st));
            ColFftArgs cm = ca;   // merged rows (float, extended): pairs [0, NLv / 2)
            cm.src = W.mrow;
            cm.row_stride = ga->out_stride;
            cm.ext = ga->ext;
            cm.n_pairs = ga->NLv / 2;
            RG(launch_col_fft_fwd_f(cm, st));
            if (ga->n_narrow) {   // narrow node rows straight from the LDM: the following pairs
                ColFftArgs cn = ca;
                cn.pair_base = ga->NLv / 2;
                cn.n_pairs = ga->n_narrow * ga->NLv / 2;
                cn.map_n = ga->n_narrow;
                cn.map_NL = ga->NL;
                cn.map_NLv = ga->NLv;
                for (int i = 0; i < ga->n_narrow; ++i) cn.map_l[i] = (unsigned char)ga->narrow_l[i];
                RG(launch_col_fft_fwd(cn, st));
            }
        } else {
            if (ev) CU(cudaEventRecord(ev[6], st));
            RG(launch_col_fft_fwd(ca, st));
        }
        if (ev) CU(cudaEventRecord(ev[2], st));
        VoigtArgs& vr = skel ? *lp.vk : merged ? *lp.vm : *lp.va;
        vr.store_g = vr.n_pairs <= kPairGroup;   // one pair group per row: it stores G itself
        vr.inv_fused = vr.store_g;                // ... after its inverse row DFT
        if (!vr.store_g) CU(cudaMemsetAsync(W.g, 0, sizeof(float2) * (size_t)W.n, st));
        RG(launch_row_fft_voigt(vr, st));
        if (ev) CU(cudaEventRecord(ev[3], st));
        if (!vr.inv_fused) {
            RowIfftArgs ra;
            ra.f2 = W.f2;
            ra.n1 = W.n1;
            ra.n2 = W.n2;
            ra.n = W.n;
            ra.g = W.g;
            ra.tw_hi = W.tw_hi;
            ra.tw_lo = W.tw_lo;
            RG(launch_row_ifft(ra, st));
        }
        if (ev) CU(cudaEventRecord(ev[4], st));
        ca.h = W.g;
        ca.out = out;
        ca.out_scale = (float)(std::exp(s.log_scale_int - s.log_scale_out) / ((double)W.n * W.desc.dv));
        ca.err = W.err;
        ca.err_pub = W.err_pub;   // mapped: the kernel publishes and clears the flag
        if (W.quant_out) {        // fused post-processing of eq_spectrum_gpu
            ca.q_out = W.quant_out;
            ca.q_scale = (float)std::exp(s.log_scale_out);
            ca.q_path = (float)W.quant_path;
            ca.q_c2_T = (float)(kC2 / W.quant_T);
            ca.q_vmin = W.desc.vmin;
            ca.q_dv = W.desc.dv;
        }
        RG(launch_col_ifft(ca, st));
        if (ev) CU(cudaEventRecord(ev[5], st));
        if (W.err_pub) return RG_OK;
    }
    // publish the device error flag to pinned host memory and clear it
    CU(cudaMemcpyAsync(W.err_host, W.err, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    CU(cudaMemsetAsync(W.err, 0, sizeof(unsigned), st));
    return RG_OK;
}

// Derivative coefficients of every line at the conditions (node axes of s
// held fixed); dlnq_dT[iso] = d ln(Q(Tref)/Q(T))/dT (NULL: 0).
int fill_grad_args(const rg_lines* L, const Work& W, const rg_conditions* c, const SpecHost& s,
                   const double* dlnq_dT, GradArgs* g) {
    std::memset(g, 0, sizeof *g);
    RG(build_scatter_args(L, W, c, s, false, nullptr, &g->s));
    if (!(c->x > 0)) return fail(RG_ERR_ARG, "derivatives need a mole fraction x > 0");
    const double T = c->T, p = c->p_bar;
    g->n_lines = L->n;
    g->row_stride = W.row_stride;
    g->c2_T = (float)(kC2 / T);
    g->c2_T2 = (float)(kC2 / (T * T));
    for (int i = 0; i < L->n_iso; ++i) {
        double dl;
        RG(dlnq_of(L, dlnq_dT, T, i, &dl));
        g->cT0[i] = (float)(dl - 1.0 / T);
    }
    g->gT = (float)(0.5 / (T * s.grid.dxG));
    g->lT = (float)(1.0 / (T * s.grid.dxL));
    g->lP = (float)(1.0 / (p * s.grid.dxL));
    g->lX = (float)(1.0 / s.grid.dxL);
    g->kP = (float)(1.0 / (1.01325 * W.desc.dv));
    g->iP = (float)(1.0 / p);
    g->iX = (float)(1.0 / c->x);
    return RG_OK;
}

ColFftArgs col_args(const Work& W, const SpecHost& s) {
    ColFftArgs ca;
    std::memset(&ca, 0, sizeof ca);
    ca.f1 = W.f1;
    ca.n1 = W.n1;
    ca.n2 = W.n2;
    ca.B = W.B;
    ca.n_v = (int)W.desc.n_v;
    ca.n = W.n;
    ca.row_stride = W.row_stride;
    ca.n_pairs = s.n_nodes / 2;
    ca.tw_hi = W.tw_hi;
    ca.tw_lo = W.tw_lo;
    ca.twiddle = !row_layout(W.n2).twr;
    return ca;
}

// Reverse mode: enqueue grad_d[0..2] = sum_k g[k] d(abscoeff_k)/d(T, p_bar, x)
// / exp(log_scale_int), g = n_v floats on the device.  The plan's LDM buffer
// holds the adjoint LDM (float) afterwards.
int enqueue_backward(const rg_lines* L, Work& W, const rg_conditions* c, const SpecHost& s, const double* dlnq_dT,
                     const float* g_dev, double* grad_d, cudaStream_t st) {
    RG(ensure_workspace(W, s.n_nodes, st));
    auto ga = std::make_unique<GradArgs>();
    RG(fill_grad_args(L, W, c, s, dlnq_dT, ga.get()));
    // Ghat = FFT(g): one real row through the column stage and the row stage
    // with unit weights (node 0: V = 1, node 1: V = 0)
    ColFftArgs ca = col_args(W, s);
    ca.src = g_dev;
    ca.single = 1;
    ca.n_pairs = 1;
    ca.y = W.y;
    RG(launch_col_fft_fwd_f(ca, st));
    auto ar = std::make_unique<AdjRowArgs>();
    VoigtArgs& u = ar->v;
    fill_voigt_args(W, s, &u);
    VoigtArgs* unit = new (std::nothrow) VoigtArgs(u);
    if (!unit) return fail(RG_ERR_OOM, "host allocation failed");
    std::unique_ptr<VoigtArgs> uguard(unit);
    unit->n_pairs = 1;
    unit->n_nodes = 2;
    unit->NL = 2;
    unit->alpha[0] = 0.f;
    unit->beta[0] = unit->beta[1] = 0.f;
    unit->norm[0] = 1.f;
    unit->norm[1] = 0.f;
    unit->lnorm[0] = 0.f;
    unit->lnorm[1] = -std::numeric_limits<float>::infinity();
    unit->nfold[0] = unit->nfold[1] = 0;
    unit->any_fold = 0;
    CU(cudaMemsetAsync(W.g, 0, sizeof(float2) * (size_t)W.n, st));
    RG(launch_row_fft_voigt(*unit, st));
    // adjoint LDM rows: Re / Im of IFFT(Ghat (V_a + i V_b)) / (N dv), per pair;
    // with the skeleton layout only the skeleton rows (the gather expands them
    // into node rows with the projection coefficients: C restricted to node n
    // is sum_r C[r][n] times skeleton node s_r's convolution)
    LayoutPlan lp;
    const bool skel = W.desc.layout != 1 && W.desc.layout != 2 && plan_layout(W, s, st, &lp) == RG_OK && lp.skel;
    if (skel) {
        const VoigtArgs ghat = ar->v;   // keeps g = Ghat
        ar->v = *lp.vk;
        ar->v.g = ghat.g;
    }
    ar->y = W.y;
    RG(launch_row_ifft_adj(*ar, st));
    ColFftArgs cb = col_args(W, s);
    if (skel) cb.n_pairs = lp.pa.rows / 2;
    cb.h = W.y;
    cb.out = W.ldm;
    cb.out_scale = (float)(1.0 / ((double)W.n * W.desc.dv));
    RG(launch_col_ifft_adj(cb, st));
    // per-line chain rule gathered at the lines' cells
    if (skel) {
        ga->proj_coef = lp.pa.coef;
        ga->proj_rows = lp.pa.rows;
        ga->proj_rp = lp.pa.rows_pad;
        ga->proj_n = lp.pa.n_nodes;
    }
    ga->adj = W.ldm;
    ga->out = grad_d;
    CU(cudaMemsetAsync(grad_d, 0, 3 * sizeof(double), st));
    RG(launch_gather_grad(*ga, L->ctx->sms * 8, st));
    return RG_OK;
}

// Forward mode: enqueue out + q n_v = d(abscoeff)/d(theta_q) exp(-log_scale_out)
// for theta = (T, p_bar, x), through the float-LDM tangent scatter and the
// ordinary FFT / Voigt / inverse FFT stages.
int enqueue_tangent(const rg_lines* L, Work& W, const rg_conditions* c, const SpecHost& s, const double* dlnq_dT,
                    float* out, cudaStream_t st) {
    RG(ensure_workspace(W, s.n_nodes, st));
    auto ga = std::make_unique<GradArgs>();
    RG(fill_grad_args(L, W, c, s, dlnq_dT, ga.get()));
    auto va = std::make_unique<VoigtArgs>();
    fill_voigt_args(W, s, va.get());
    // skeleton layout: each tangent LDM is projected onto the skeleton rows
    // (in place, tensor cores) before its FFT, as the spectrum's LDM is
    LayoutPlan lp;
    const bool skel = W.desc.layout != 1 && W.desc.layout != 2 && plan_layout(W, s, st, &lp) == RG_OK && lp.skel;
    VoigtArgs& vr = skel ? *lp.vk : *va;
    vr.store_g = vr.n_pairs <= kPairGroup;
    vr.inv_fused = vr.store_g;
    float* tan = W.ldm;
    ga->tan = tan;
    const int n_v = (int)W.desc.n_v;
    for (int q = 0; q < 3; ++q) {
        ga->theta = q;
        CU(cudaMemsetAsync(tan, 0, sizeof(float) * (size_t)s.n_nodes * W.row_stride, st));
        RG(launch_scatter_tangent(*ga, L->ctx->sms * 8, st));
        ColFftArgs ca = col_args(W, s);
        if (skel) {
            ProjArgs pa = lp.pa;
            pa.ldm = tan;
            pa.sms = L->ctx->sms;
            RG(launch_node_project(pa, st));
            ca.n_pairs = pa.rows / 2;
        }
        ca.src = tan;
        ca.y = W.y;
        RG(launch_col_fft_fwd_f(ca, st));
        if (!vr.store_g) CU(cudaMemsetAsync(W.g, 0, sizeof(float2) * (size_t)W.n, st));
        RG(launch_row_fft_voigt(vr, st));
        RowIfftArgs ra;
        ra.f2 = W.f2;
        ra.n1 = W.n1;
        ra.n2 = W.n2;
        ra.n = W.n;
        ra.g = W.g;
        ra.tw_hi = W.tw_hi;
        ra.tw_lo = W.tw_lo;
        if (!vr.inv_fused) RG(launch_row_ifft(ra, st));
        ca.h = W.g;
        ca.out = out + (size_t)q * n_v;
        ca.out_scale = (float)(std::exp(s.log_scale_int - s.log_scale_out) / ((double)W.n * W.desc.dv));
        RG(launch_col_ifft(ca, st));
    }
    return RG_OK;
}

// The plan's workspace is shared by everything enqueued on it: order work on
// a new stream after the plan's previous work (begin) and mark the end (end).
int plan_stream_begin(rg_plan* P, cudaStream_t st) {
    if (!P->done) CU(cudaEventCreateWithFlags(&P->done, cudaEventDisableTiming));
    if (P->any && st != P->last_stream) CU(cudaStreamWaitEvent(st, P->done, 0));
    return RG_OK;
}
int plan_stream_end(rg_plan* P, cudaStream_t st) {
    CU(cudaEventRecord(P->done, st));
    P->last_stream = st;
    P->any = true;
    return RG_OK;
}

int run_spectrum(rg_plan* P, const rg_conditions* c, float* out, cudaStream_t st, int timing, bool ldm_only,
                 rg_spectrum_info* info) {
    NvtxRange nvtx_("rg/spectrum");
    SpecHost s;
    RG(compute_grid(P->lines, P->w, c, &s));
    cudaEvent_t* ev = nullptr;
    if (timing == 2) {
        if (P->ring.empty()) {
            P->ring.assign(rg_plan::kRing * rg_plan::kEv, nullptr);
            for (auto& e : P->ring) CU(cudaEventCreate(&e));
        }
        if (P->ring_used >= rg_plan::kRing) return fail(RG_ERR_RANGE, "stage-timing ring full: read it first");
        ev = &P->ring[rg_plan::kEv * P->ring_used];
        P->ring_ldm_only[P->ring_used] = ldm_only;
        P->ring_used++;
        P->ring_stream = st;
    } else if (timing) {
        for (auto& e : P->ev)
            if (!e) CU(cudaEventCreate(&e));
        ev = P->ev;
    }
    P->w.count_lines = (timing == 1 && info) || ldm_only;
    RG(plan_stream_begin(P, st));
    RG(enqueue_spectrum(P->lines, P->w, c, s, out, st, ev, ldm_only));
    RG(plan_stream_end(P, st));
    if (info) {
        std::memset(info, 0, sizeof *info);
        info->grid = s.grid;
        info->log_scale = ldm_only ? s.log_scale_int : s.log_scale_out;
        info->lines_in_window = -1;
        info->fft_rows = ldm_only ? 0 : P->w.last_fft_rows;
        info->merged_rows = ldm_only ? 0 : P->w.last_merged_rows;
        info->merged_ext = ldm_only ? 0 : P->w.last_ext;
        info->accum_bits = P->w.last_accum;
        info->layout = ldm_only ? 0 : P->w.last_layout;
        info->layout_err = ldm_only ? 0.f : (float)P->w.last_layout_err;
    }
    if (timing == 1 && info) {
        CU(cudaStreamSynchronize(st));
        RG(take_err(P->w));
        int last = ldm_only ? 1 : 5;
        for (int i = 0; i < last; ++i) CU(cudaEventElapsedTime(&info->stage_ms[i], P->ev[i], P->ev[i + 1]));
        CU(cudaEventElapsedTime(&info->stage_ms[5], P->ev[0], P->ev[last]));
        if (!ldm_only) CU(cudaEventElapsedTime(&info->gauss_ms, P->ev[1], P->ev[6]));
        unsigned long long cnt = 0;
        CU(cudaMemcpy(&cnt, P->w.counter, sizeof cnt, cudaMemcpyDeviceToHost));
        info->lines_in_window = (int64_t)cnt;
    }
    return RG_OK;
}

// FFT factorisation, twiddle tables (device, owned by the caller) and line
// index geometry of a spectral grid.
int tw_n_tables(int64_t n, float2** hi_out, float2** lo_out) {
    const int nh = (int)(n / 1024) + 2;
    std::vector<float2> hi(nh), lo(1024);
    for (int t = 0; t < nh; ++t) {
        double ang = -2.0 * kPi * (double)((int64_t)t * 1024 % n) / (double)n;
        hi[t].x = (float)std::cos(ang);
        hi[t].y = (float)std::sin(ang);
    }
    for (int t = 0; t < 1024; ++t) {
        double ang = -2.0 * kPi * (double)t / (double)n;
        lo[t].x = (float)std::cos(ang);
        lo[t].y = (float)std::sin(ang);
    }
    CU(cudaMalloc(hi_out, sizeof(float2) * nh));
    CU(cudaMalloc(lo_out, sizeof(float2) * 1024));
    CU(cudaMemcpy(*hi_out, hi.data(), sizeof(float2) * nh, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(*lo_out, lo.data(), sizeof(float2) * 1024, cudaMemcpyHostToDevice));
    return RG_OK;
}

// Shift-index margin (columns) for pressures up to p_atm_max.
void shift_margin(const rg_lines* L, double dv, int* E, double* p_atm_max) {
    *p_atm_max = 200.0;
    double e = std::ceil(L->env.max_abs_delta * *p_atm_max / dv) + 2;
    if (e > (double)(1 << 22)) {
        *p_atm_max = ((double)(1 << 22) - 2) * dv / L->env.max_abs_delta;
        e = (double)(1 << 22);
    }
    *E = (int)e;
}

bool valid(const rg_ctx* c) { return c && c->magic == 0x52474358; }
bool valid(const rg_lines* l) { return l && l->magic == 0x52474C4E; }
bool valid(const rg_plan* p) { return p && p->magic == 0x52475041; }

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int rg_abi_version(void) { return RG_ABI_VERSION; }

const char* rg_last_error(void) { return g_err.c_str(); }

int rg_ctx_create(int device, rg_ctx** out) {
    g_err.clear();
    if (!out) return fail(RG_ERR_ARG, "out is NULL");
    int n = 0;
    CU(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(RG_ERR_ARG, "device %d not in [0, %d)", device, n);
    DeviceGuard dev_guard_;
    CU(dev_guard_.use(device));
    auto* c = new (std::nothrow) rg_ctx();
    if (!c) return fail(RG_ERR_OOM, "host allocation failed");
    c->device = device;
    if (cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || c->sms < 1)
        c->sms = 1;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return fail(RG_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    // workspaces come from the device's default stream-ordered pool: keep freed
    // blocks cached in this process (no return to the driver at every
    // synchronisation) so plans and server slots of changing sizes reuse them;
    // trimmed when the context is destroyed
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = std::numeric_limits<uint64_t>::max();
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    *out = c;
    return RG_OK;
}

int rg_ctx_destroy(rg_ctx* c) {
    g_err.clear();
    if (!c) return RG_OK;
    if (!valid(c)) return fail(RG_ERR_STATE, "invalid context");
    if (c->lines) return fail(RG_ERR_STATE, "context still has %d line list(s)", c->lines);
    DeviceGuard dev_guard_;
    dev_guard_.use(c->device);
    cudaStreamSynchronize(c->stream);
    cudaStreamDestroy(c->stream);
    cudaMemPool_t pool;   // hand the cached pool memory back
    if (cudaDeviceGetDefaultMemPool(&pool, c->device) == cudaSuccess) {
        cudaDeviceSynchronize();
        cudaMemPoolTrimTo(pool, 0);
    }
    c->magic = 0;
    delete c;
    return RG_OK;
}

int rg_lines_upload(rg_ctx* ctx, const rg_line_arrays* in, const rg_isotopes* iso, rg_lines** out) {
    NvtxRange nvtx_("rg/lines_upload");
    g_err.clear();
    if (!valid(ctx)) return fail(RG_ERR_STATE, "invalid context");
    if (!in || !iso || !out) return fail(RG_ERR_ARG, "NULL argument");
    DeviceGuard dev_guard_;
    CU(dev_guard_.use(ctx->device));
    auto* L = new (std::nothrow) rg_lines();
    if (!L) return fail(RG_ERR_OOM, "host allocation failed");
    std::unique_ptr<rg_lines> guard(L);
    RG(build_envelope(in, iso, &L->env));
    const int64_t n = in->n;
    L->ctx = ctx;
    L->n = n;
    L->n_iso = iso->n_iso;
    L->t_ref = iso->t_ref;

    cudaStream_t st = ctx->stream;
    double* v0_tmp = nullptr;
    double* s_tmp = nullptr;
    int* flag = nullptr;
    auto cleanup_tmp = [&]() {
        if (v0_tmp) cudaFree(v0_tmp);
        if (s_tmp) cudaFree(s_tmp);
        if (flag) cudaFree(flag);
    };
    auto bail = [&](int code) {
        cleanup_tmp();
        dfree(L->v0);
        dfree(L->ls2);
        dfree(L->el);
        dfree(L->ga);
        dfree(L->gs);
        dfree(L->na);
        dfree(L->dl);
        dfree(L->iso);
        return code;
    };
#define CUB(call)                                                                                    \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess)                                                                       \
            return bail(fail(e_ == cudaErrorMemoryAllocation ? RG_ERR_OOM : RG_ERR_CUDA, "%s: %s", #call, \
                             cudaGetErrorString(e_)));                                               \
    } while (0)
    if (n > (int64_t)0x7fff0000) return bail(fail(RG_ERR_RANGE, "more than 2^31 lines"));
    // arrays hold a multiple of 16 lines (zero padding) for the 16-line TMA copies
    const int64_t npad = (n + kLinePad - 1) / kLinePad * kLinePad;
    const size_t f4 = sizeof(float) * (size_t)n, f4p = sizeof(float) * (size_t)npad;
    CUB(cudaMalloc(&v0_tmp, sizeof(double) * n));
    CUB(cudaMalloc(&s_tmp, sizeof(double) * n));
    CUB(cudaMalloc(&flag, sizeof(int)));
    CUB(cudaMalloc(&L->v0, sizeof(float2) * npad));
    CUB(cudaMalloc(&L->ls2, f4p));
    CUB(cudaMalloc(&L->el, f4p));
    CUB(cudaMalloc(&L->ga, f4p));
    CUB(cudaMalloc(&L->gs, f4p));
    CUB(cudaMalloc(&L->na, f4p));
    if (in->delta) CUB(cudaMalloc(&L->dl, f4p));
    if (in->iso && L->n_iso > 1) CUB(cudaMalloc(&L->iso, (size_t)npad));
    if (npad > n) {   // padding lines: v0 = 0 lies outside every window and is dropped
        const int64_t t = npad - n;
        CUB(cudaMemsetAsync(L->v0 + n, 0, sizeof(float2) * t, st));
        for (float* arr : {L->ls2, L->el, L->ga, L->gs, L->na, L->dl})
            if (arr) CUB(cudaMemsetAsync(arr + n, 0, sizeof(float) * t, st));
        if (L->iso) CUB(cudaMemsetAsync(L->iso + n, 0, (size_t)t, st));
    }
    CUB(cudaMemsetAsync(flag, 0, sizeof(int), st));
    CUB(cudaMemcpyAsync(v0_tmp, in->v0, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    CUB(cudaMemcpyAsync(s_tmp, in->s_ref, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    CUB(cudaMemcpyAsync(L->el, in->e_low, f4, cudaMemcpyHostToDevice, st));
    CUB(cudaMemcpyAsync(L->ga, in->g_air, f4, cudaMemcpyHostToDevice, st));
    CUB(cudaMemcpyAsync(L->gs, in->g_self, f4, cudaMemcpyHostToDevice, st));
    CUB(cudaMemcpyAsync(L->na, in->n_air, f4, cudaMemcpyHostToDevice, st));
    if (in->delta) CUB(cudaMemcpyAsync(L->dl, in->delta, f4, cudaMemcpyHostToDevice, st));
    if (L->iso) CUB(cudaMemcpyAsync(L->iso, in->iso, (size_t)n, cudaMemcpyHostToDevice, st));
    if (launch_prepare_lines(v0_tmp, s_tmp, n, kC2 / L->t_ref, L->v0, L->ls2, flag, st) != RG_OK)
        return bail(fail(RG_ERR_CUDA, "prepare_lines launch: %s", cudaGetErrorString(cudaGetLastError())));
    int unsorted = 0;
    CUB(cudaMemcpyAsync(&unsorted, flag, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUB(cudaStreamSynchronize(st));
    cleanup_tmp();
    v0_tmp = nullptr;
    s_tmp = nullptr;
    flag = nullptr;
    if (unsorted) return bail(fail(RG_ERR_UNSORTED, "line positions v0 must be ascending"));
#undef CUB
    ctx->lines++;
    *out = guard.release();
    return RG_OK;
}

int rg_lines_free(rg_lines* L) {
    g_err.clear();
    if (!L) return RG_OK;
    if (!valid(L)) return fail(RG_ERR_STATE, "invalid line list");
    if (L->plans.load()) return fail(RG_ERR_STATE, "line list still has %d plan(s) or queued request(s)", L->plans.load());
    DeviceGuard dev_guard_;
    dev_guard_.use(L->ctx->device);
    cudaStreamSynchronize(L->ctx->stream);
    dfree(L->v0);
    dfree(L->ls2);
    dfree(L->el);
    dfree(L->ga);
    dfree(L->gs);
    dfree(L->na);
    dfree(L->dl);
    dfree(L->iso);
    L->ctx->lines--;
    L->magic = 0;
    delete L;
    return RG_OK;
}

int rg_lines_count(const rg_lines* L, int64_t* n) {
    g_err.clear();
    if (!valid(L) || !n) return fail(RG_ERR_ARG, "invalid argument");
    *n = L->n;
    return RG_OK;
}

int rg_plan_create(rg_lines* L, const rg_plan_desc* d, rg_plan** out) {
    NvtxRange nvtx_("rg/plan_create");
    g_err.clear();
    if (!valid(L)) return fail(RG_ERR_STATE, "invalid line list");
    if (!d || !out) return fail(RG_ERR_ARG, "NULL argument");
    if (!(d->dv > 0) || d->n_v < 2) return fail(RG_ERR_ARG, "dv must be > 0 and n_v >= 2");
    if (d->n_v > (int64_t)1 << 30) return fail(RG_ERR_RANGE, "n_v too large");
    if (!((d->n_G > 1) || d->dxG > 0) || !((d->n_L > 1) || d->dxL > 0))
        return fail(RG_ERR_ARG, "give dxG/dxL > 0 or node counts n_G/n_L > 1");
    RG(check_desc_options(*d));
    DeviceGuard dev_guard_;
    CU(dev_guard_.use(L->ctx->device));
    auto* P = new (std::nothrow) rg_plan();
    if (!P) return fail(RG_ERR_OOM, "host allocation failed");
    std::unique_ptr<rg_plan> guard(P);
    P->lines = L;
    Work& W = P->w;
    W.desc = *d;
    int n1, n2;
    if (!choose_fft(2 * d->n_v, d->n_ft, &n1, &n2))
        return fail(RG_ERR_RANGE, "no supported FFT length >= %lld (n_ft=%lld)", (long long)(2 * d->n_v),
                    (long long)d->n_ft);
    W.n1 = n1;
    W.n2 = n2;
    W.n = (int64_t)n1 * n2;
    W.B = col_block(n1);
    RG(make_fftlen(n1, &W.f1));
    RG(make_fftlen(n2, &W.f2));
    RG(tw_n_tables(W.n, &P->tw_hi_own, &P->tw_lo_own));
    W.tw_hi = P->tw_hi_own;
    W.tw_lo = P->tw_lo_own;
    // line index per grid column, with a margin for pressure shifts up to p_atm_max
    shift_margin(L, d->dv, &W.E, &W.p_atm_max);
    W.col_off = W.E;
    W.col_count = (int)d->n_v + 1 + 2 * W.E;
    cudaStream_t st = L->ctx->stream;
    CU(cudaMalloc(&W.col_start, sizeof(int64_t) * W.col_count));
    RG(launch_col_index(L->v0, L->n, d->vmin, d->dv, -W.E, W.col_count, W.col_start, st));
    CU(cudaMalloc(&W.cmax_dev, sizeof(int)));
    RG(launch_col_cmax(W.col_start, W.col_off, W.col_count, (int)d->n_v, W.E - 1, W.cmax_dev, st));
    W.row_stride = (d->n_v + 31) / 32 * 32;
    CU(cudaMalloc(&W.g, sizeof(float2) * (size_t)W.n));
    CU(cudaMalloc(&P->out_d, sizeof(float) * (size_t)d->n_v));
    CU(cudaMalloc(&W.counter, sizeof(unsigned long long)));
    CU(cudaMalloc(&W.err, sizeof(unsigned)));
    CU(cudaHostAlloc(&W.err_host, sizeof(unsigned), cudaHostAllocMapped));
    *W.err_host = 0;
    CU(cudaHostGetDevicePointer((void**)&W.err_pub, W.err_host, 0));
    CU(cudaMemsetAsync(W.err, 0, sizeof(unsigned), st));
    int cm = 0;
    CU(cudaMemcpyAsync(&cm, W.cmax_dev, sizeof(int), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    W.cmax_host = cm;
    L->plans++;
    *out = guard.release();
    return RG_OK;
}

void free_work(Work& W) {
    dfree(W.col_start);
    dfree(W.cmax_dev);
    dfree(W.ldm);
    dfree(W.y);
    dfree(W.g);
    dfree(W.counter);
    dfree(W.err);
    if (W.err_host) cudaFreeHost(W.err_host);
    W.err_host = nullptr;
    W.nodes_cap = 0;
    W.ldm_bytes = W.y_bytes = 0;
    dfree(W.mrow);
    W.mrow_bytes = 0;
    dfree(W.proj_coef);
    W.proj_bytes = 0;
    W.skel_dev = false;
}

int rg_plan_free(rg_plan* P) {
    g_err.clear();
    if (!P) return RG_OK;
    if (!valid(P)) return fail(RG_ERR_STATE, "invalid plan");
    {
        std::lock_guard<std::mutex> lk(P->mu);
        DeviceGuard dev_guard_;
        dev_guard_.use(P->lines->ctx->device);
        cudaStreamSynchronize(P->lines->ctx->stream);
        cudaDeviceSynchronize();
        dfree(P->w.f1.tw);
        dfree(P->w.f2.tw);
        dfree(P->tw_hi_own);
        dfree(P->tw_lo_own);
        free_work(P->w);
        dfree(P->out_d);
        dfree(P->quant_d);
        dfree(P->grad_d);
        for (auto& e : P->ev)
            if (e) cudaEventDestroy(e);
        for (auto& e : P->ring)
            if (e) cudaEventDestroy(e);
        if (P->done) cudaEventDestroy(P->done);
        P->lines->plans--;
        P->magic = 0;
    }
    delete P;
    return RG_OK;
}

int rg_plan_grid(rg_plan* P, const rg_conditions* c, rg_grid* out) {
    g_err.clear();
    if (!valid(P) || !c || !out) return fail(RG_ERR_ARG, "invalid argument");
    SpecHost s;
    RG(compute_grid(P->lines, P->w, c, &s));
    *out = s.grid;
    return RG_OK;
}

int rg_grid_estimate(const rg_line_arrays* lines, const rg_isotopes* iso, const rg_plan_desc* d,
                     const rg_conditions* c, rg_grid* out) {
    g_err.clear();
    if (!lines || !iso || !d || !c || !out) return fail(RG_ERR_ARG, "NULL argument");
    if (!(d->dv > 0) || d->n_v < 2) return fail(RG_ERR_ARG, "dv must be > 0 and n_v >= 2");
    if (!((d->n_G > 1) || d->dxG > 0) || !((d->n_L > 1) || d->dxL > 0))
        return fail(RG_ERR_ARG, "give dxG/dxL > 0 or node counts n_G/n_L > 1");
    int n1, n2;
    if (!choose_fft(2 * d->n_v, d->n_ft, &n1, &n2))
        return fail(RG_ERR_RANGE, "no supported FFT length >= %lld", (long long)(2 * d->n_v));
    auto env = std::make_unique<Envelope>();
    RG(build_envelope(lines, iso, env.get()));
    SpecHost s;
    RG(compute_grid_env(*env, nullptr, *d, (int64_t)n1 * n2, n1, n2, c, &s));
    *out = s.grid;
    return RG_OK;
}

int rg_grid_skeleton(const rg_grid* grid, double dv, double folding_thresh, double tol, int32_t r_max,
                     int32_t* n_rows, int32_t* nodes, double* coef, double* err) {
    g_err.clear();
    if (!grid || !n_rows || !nodes || !coef || !err) return fail(RG_ERR_ARG, "NULL argument");
    if (!(dv > 0)) return fail(RG_ERR_ARG, "dv must be > 0");
    if (grid->n_G < 1 || grid->n_L < 1 || grid->n_G * grid->n_L > kMaxNodes)
        return fail(RG_ERR_RANGE, "grid %d x %d outside 1..%d nodes", grid->n_G, grid->n_L, kMaxNodes);
    if (r_max < 1 || r_max > grid->n_G * grid->n_L)
        return fail(RG_ERR_ARG, "r_max must be in 1..n_G n_L (got %d)", (int)r_max);
    if (!(tol < 1e-2)) return fail(RG_ERR_ARG, "tol must be < 1e-2 (got %g)", tol);
    const int n = grid->n_G * grid->n_L;
    std::vector<int> sk;
    std::vector<double> C;
    int R = 0;
    double e = 0.0;
    const int rc = skeleton_decomp(*grid, dv, folding_thresh > 0 ? folding_thresh : 1e-6, tol > 0 ? tol : kSkelTol,
                                   r_max, &sk, &C, &R, &e);
    *n_rows = R;
    *err = e;
    if (rc == RG_ERR_RANGE) return fail(RG_ERR_RANGE, "%d skeleton rows leave a sampled error of %g > %g", R, e, tol);
    RG(rc);
    for (int r = 0; r < R; ++r) nodes[r] = sk[r];
    std::copy(C.begin(), C.begin() + (size_t)R * n, coef);
    return RG_OK;
}

int rg_synthesize(rg_plan* P, const rg_conditions* c, float* out_dev, void* stream, int timing,
                  rg_spectrum_info* info) {
    g_err.clear();
    if (!valid(P) || !c || !out_dev) return fail(RG_ERR_ARG, "invalid argument");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard dev_guard_;
    CU(dev_guard_.use(P->lines->ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : P->lines->ctx->stream;
    return run_spectrum(P, c, out_dev, st, timing, false, info);
}

namespace {
// One spectrum with the post-processing rows written by its last kernel into
// out_dev + n_v (4 rows); the epilogue request is cleared on every return.
// Device address of page-locked host memory (cudaHostAlloc'd or registered:
// mapped into the device's address space under unified addressing), or null.
// The spectrum's last kernel then stores into the caller's buffer itself
// (over NVLink-C2C on a Grace host) instead of a copy after it.
float* mapped_host(void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
    return static_cast<float*>(a.devicePointer);
}

int run_quantities(rg_plan* P, const rg_conditions* c, double path_length, float* out_dev, cudaStream_t st,
                   int timing, rg_spectrum_info* info) {
    struct Clear {
        Work& w;
        ~Clear() { w.quant_out = nullptr; }
    } clear_{P->w};
    P->w.quant_out = out_dev + P->w.desc.n_v;
    P->w.quant_path = path_length;
    P->w.quant_T = c->T;
    return run_spectrum(P, c, out_dev, st, timing, false, info);
}
}  // namespace

int rg_synthesize_quantities(rg_plan* P, const rg_conditions* c, double path_length, float* out_dev, void* stream,
                             rg_spectrum_info* info) {
    g_err.clear();
    if (!valid(P) || !c || !out_dev) return fail(RG_ERR_ARG, "invalid argument");
    if (!(path_length > 0)) return fail(RG_ERR_ARG, "path_length must be positive");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard dev_guard_;
    CU(dev_guard_.use(P->lines->ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : P->lines->ctx->stream;
    rg_spectrum_info inf;
    RG(run_quantities(P, c, path_length, out_dev, st, 0, &inf));
    if (info) *info = inf;
    return RG_OK;
}

int rg_synthesize_quantities_host(rg_plan* P, const rg_conditions* c, double path_length, float* out_host,
                                  void* stream, int timing, rg_spectrum_info* info) {
    g_err.clear();
    if (!valid(P) || !c || !out_host) return fail(RG_ERR_ARG, "invalid argument");
    if (!(path_length > 0)) return fail(RG_ERR_ARG, "path_length must be positive");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard dev_guard_;
    CU(dev_guard_.use(P->lines->ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : P->lines->ctx->stream;
    const size_t n5 = 5 * (size_t)P->w.desc.n_v;
    float* direct = mapped_host(out_host);   // page-locked: written by the last kernel
    if (!direct && !P->quant_d) CU(cudaMalloc((void**)&P->quant_d, sizeof(float) * n5));
    RG(run_quantities(P, c, path_length, direct ? direct : P->quant_d, st, (timing && info) ? 1 : 0, info));
    if (!direct) CU(cudaMemcpyAsync(out_host, P->quant_d, sizeof(float) * n5, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return take_err(P->w);
}

int rg_lines_set_partition(rg_lines* L, int32_t iso, int64_t n, const double* T, const double* Q, int32_t interp) {
    g_err.clear();
    if (!valid(L)) return fail(RG_ERR_ARG, "invalid line list");
    if (iso < 0 || iso >= L->n_iso) return fail(RG_ERR_ARG, "isotopologue %d not in [0, %d)", (int)iso, L->n_iso);
    QTable t;
    std::string e;
    const int rc = qtable_build(n, T, Q, interp, &t, &e);
    if (rc) return fail(rc, "%s", e.c_str());
    if ((int)L->qtab.size() != L->n_iso) L->qtab.resize(L->n_iso);
    L->qtab[iso] = std::move(t);
    return RG_OK;
}

int rg_partition_eval(int64_t n, const double* T, const double* Q, int32_t interp, double t, double* q,
                      double* dq_dt) {
    g_err.clear();
    if (!q) return fail(RG_ERR_ARG, "invalid argument");
    QTable tab;
    std::string e;
    int rc = qtable_build(n, T, Q, interp, &tab, &e);
    if (!rc) rc = qtable_eval(tab, t, q, dq_dt, &e);
    if (rc) return fail(rc, "%s", e.c_str());
    return RG_OK;
}

int rg_hitran_count(const char* text, int64_t nbytes, int32_t threads, int64_t* n_records) {
    g_err.clear();
    if (!n_records || nbytes < 0 || (!text && nbytes > 0)) return fail(RG_ERR_ARG, "invalid argument");
    return hitran_count(text, nbytes, threads, n_records);
}

int rg_hitran_parse(const char* text, int64_t nbytes, int32_t threads, const rg_hitran_columns* out) {
    NvtxRange nvtx_("rg/hitran_parse");
    g_err.clear();
    if (!out || nbytes < 0 || (!text && nbytes > 0) || out->n < 0) return fail(RG_ERR_ARG, "invalid argument");
    std::string e;
    const int rc = hitran_parse(text, nbytes, threads, out, &e);
    if (rc) return fail(rc, "%s", e.c_str());
    return RG_OK;
}

int rg_slit_convolve(rg_ctx* ctx, const float* in_dev, int64_t n, const float* slit_dev, int32_t n_slit,
                     double wstep, int32_t mode, float* out_dev, void* stream) {
    g_err.clear();
    if (!valid(ctx) || !in_dev || !slit_dev || !out_dev) return fail(RG_ERR_ARG, "invalid argument");
    if (n < 0 || n_slit <= 0) return fail(RG_ERR_ARG, "n = %lld, n_slit = %d", (long long)n, (int)n_slit);
    if (mode != RG_SLIT_SAME && mode != RG_SLIT_VALID) return fail(RG_ERR_ARG, "unknown slit mode %d", (int)mode);
    if (!(wstep > 0)) return fail(RG_ERR_ARG, "wstep must be positive");
    if (in_dev < out_dev + n && out_dev < in_dev + n) return fail(RG_ERR_ARG, "out_dev overlaps in_dev");
    DeviceGuard dev_guard_;
    CU(dev_guard_.use(ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    SlitArgs a;
    a.in = in_dev;
    a.slit = slit_dev;
    a.out = out_dev;
    a.n = n;
    a.m = n_slit;
    a.scale = (float)wstep;
    a.valid = mode == RG_SLIT_VALID;
    RG(launch_slit_conv(a, st));
    return RG_OK;
}

int rg_plan_test_scatter_stall(rg_plan* P, int32_t withhold, int64_t wait_cycles) {
    g_err.clear();
    if (!valid(P)) return fail(RG_ERR_ARG, "invalid plan");
    if (wait_cycles < 0 || wait_cycles > kScatWaitCycles)
        return fail(RG_ERR_ARG, "wait_cycles must be in [0, %lld]", (long long)kScatWaitCycles);
    std::lock_guard<std::mutex> lk(P->mu);
    P->w.scat_withhold = withhold ? 1 : 0;
    P->w.scat_wait = wait_cycles ? wait_cycles : kScatWaitCycles;
    return RG_OK;
}

int rg_test_flush_order(int32_t n_nodes, int32_t* nodes, uint8_t* real, int32_t capacity, int32_t* count) {
    g_err.clear();
    if (!nodes || !real || !count) return fail(RG_ERR_ARG, "NULL argument");
    if (n_nodes < 1 || n_nodes > kMaxNodes) return fail(RG_ERR_RANGE, "n_nodes %d outside 1..%d", n_nodes, kMaxNodes);
    std::vector<int> nd;
    std::vector<char> re;
    flush_node_order(n_nodes, &nd, &re);
    *count = (int32_t)nd.size();
    if ((int64_t)nd.size() > capacity) return fail(RG_ERR_RANGE, "capacity %d < %d", capacity, (int)nd.size());
    for (size_t i = 0; i < nd.size(); ++i) {
        nodes[i] = nd[i];
        real[i] = re[i] ? 1 : 0;
    }
    return RG_OK;
}

int rg_plan_stage_times(rg_plan* P, double* sum_ms, int64_t* count) {
    g_err.clear();
    if (!valid(P) || !sum_ms || !count) return fail(RG_ERR_ARG, "invalid argument");
    std::lock_guard<std::mutex> lk(P->mu);
    for (int k = 0; k < 6; ++k) sum_ms[k] = 0.0;
    P->last_gauss_sum = 0.0;
    *count = P->ring_used;
    if (!P->ring_used) return RG_OK;
    CU(cudaStreamSynchronize(P->ring_stream));
    for (int r = 0; r < P->ring_used; ++r) {
        cudaEvent_t* ev = &P->ring[rg_plan::kEv * r];
        int last = P->ring_ldm_only[r] ? 1 : 5;
        float ms;
        for (int i = 0; i < last; ++i) {
            CU(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
            sum_ms[i] += ms;
        }
        CU(cudaEventElapsedTime(&ms, ev[0], ev[last]));
        sum_ms[5] += ms;
        if (!P->ring_ldm_only[r]) {
            CU(cudaEventElapsedTime(&ms, ev[1], ev[6]));
            P->last_gauss_sum += ms;
        }
    }
    P->ring_used = 0;
    return take_err(P->w);
}

int rg_plan_stage_times_gauss(rg_plan* P, double* gauss_sum_ms) {
    g_err.clear();
    if (!valid(P) || !gauss_sum_ms) return fail(RG_ERR_ARG, "invalid argument");
    std::lock_guard<std::mutex> lk(P->mu);
    *gauss_sum_ms = P->last_gauss_sum;
    return RG_OK;
}

int rg_synthesize_host(rg_plan* P, const rg_conditions* c, float* out_host, void* stream, int timing,
                       rg_spectrum_info* info) {
    g_err.clear();
    if (!valid(P) || !c || !out_host) return fail(RG_ERR_ARG, "invalid argument");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard dev_guard_;
    CU(dev_guard_.use(P->lines->ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : P->lines->ctx->stream;
    float* direct = mapped_host(out_host);   // page-locked: written by the last kernel
    RG(run_spectrum(P, c, direct ? direct : P->out_d, st, (timing && info) ? 1 : 0, false, info));
    if (!direct)
        CU(cudaMemcpyAsync(out_host, P->out_d, sizeof(float) * (size_t)P->w.desc.n_v, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return take_err(P->w);
}

int rg_debug_ldm(rg_plan* P, const rg_conditions* c, float* ldm_host, int64_t capacity,
                 rg_spectrum_info* info) {
    g_err.clear();
    if (!valid(P) || !c || !ldm_host) return fail(RG_ERR_ARG, "invalid argument");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard dev_guard_;
    CU(dev_guard_.use(P->lines->ctx->device));
    cudaStream_t st = P->lines->ctx->stream;
    rg_spectrum_info tmp;
    rg_spectrum_info* inf = info ? info : &tmp;
    RG(run_spectrum(P, c, nullptr, st, 1, true, inf));
    const int64_t nv = P->w.desc.n_v;
    const int nodes = inf->grid.n_G * inf->grid.n_L;
    if (capacity < (int64_t)nodes * nv)
        return fail(RG_ERR_ARG, "capacity %lld < %lld", (long long)capacity, (long long)nodes * nv);
    CU(cudaMemcpy2DAsync(ldm_host, sizeof(float) * nv, P->w.ldm, sizeof(float) * P->w.row_stride,
                         sizeof(float) * nv, nodes, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    return take_err(P->w);
}

int rg_backward(rg_plan* P, const rg_conditions* c, const double* dlnq_dT, const float* grad_out_dev,
                double grad[3], void* stream, rg_spectrum_info* info) {
    NvtxRange nvtx_("rg/backward");
    g_err.clear();
    if (!valid(P) || !c || !grad_out_dev || !grad) return fail(RG_ERR_ARG, "invalid argument");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard dev_guard_;
    CU(dev_guard_.use(P->lines->ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : P->lines->ctx->stream;
    SpecHost s;
    RG(compute_grid(P->lines, P->w, c, &s));
    if (!P->grad_d) CU(cudaMalloc((void**)&P->grad_d, 3 * sizeof(double)));
    RG(plan_stream_begin(P, st));
    RG(enqueue_backward(P->lines, P->w, c, s, dlnq_dT, grad_out_dev, P->grad_d, st));
    RG(plan_stream_end(P, st));
    double h[3];
    CU(cudaMemcpyAsync(h, P->grad_d, sizeof h, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    const double sc = std::exp(s.log_scale_int);
    for (int q = 0; q < 3; ++q) grad[q] = h[q] * sc;
    if (info) {
        std::memset(info, 0, sizeof *info);
        info->grid = s.grid;
        info->log_scale = 0.0;
        info->lines_in_window = -1;
    }
    return RG_OK;
}

int rg_jvp(rg_plan* P, const rg_conditions* c, const double* dlnq_dT, float* out_dev, void* stream,
           rg_spectrum_info* info) {
    NvtxRange nvtx_("rg/jvp");
    g_err.clear();
    if (!valid(P) || !c || !out_dev) return fail(RG_ERR_ARG, "invalid argument");
    std::lock_guard<std::mutex> lk(P->mu);
    DeviceGuard dev_guard_;
    CU(dev_guard_.use(P->lines->ctx->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : P->lines->ctx->stream;
    SpecHost s;
    RG(compute_grid(P->lines, P->w, c, &s));
    RG(plan_stream_begin(P, st));
    RG(enqueue_tangent(P->lines, P->w, c, s, dlnq_dT, out_dev, st));
    RG(plan_stream_end(P, st));
    if (info) {
        std::memset(info, 0, sizeof *info);
        info->grid = s.grid;
        info->log_scale = s.log_scale_out;
        info->lines_in_window = -1;
    }
    return RG_OK;
}

}  // extern "C"

// ===========================================================================
// Serving engine
// ===========================================================================
namespace {

using Clock = std::chrono::steady_clock;

struct ServerReq {
    int64_t ticket = 0;
    rg_lines* lines = nullptr;
    rg_plan_desc desc{};
    rg_conditions cond{};
    std::vector<double> q;
    float* out_host = nullptr;
    // results
    bool done = false;
    int status = RG_OK;
    std::string msg;
    rg_spectrum_info info{};
    double t_submit = 0, t_start = 0, t_done = 0;
};

struct Slot {
    cudaStream_t st = nullptr;
    Work w;
    float* out_d = nullptr;
    int64_t out_cap = 0, col_cap = 0, g_cap = 0;
    // pinned staging of the spectrum: the device-to-host copy of a request
    // stays asynchronous (a copy into pageable caller memory would block the
    // worker until the request finished); copied to the caller at harvest
    float* pin = nullptr;
    int64_t pin_cap = 0;
    bool direct = false;                  // the request's page-locked buffer is written by the last kernel
    std::shared_ptr<ServerReq> req;       // owned by the worker thread
    std::atomic<bool> notified{false};    // set by the stream's host callback
    size_t bytes() const {
        return (size_t)out_cap * 4 + (size_t)col_cap * 8 + (size_t)g_cap * 8 +
               w.ldm_bytes + w.y_bytes + w.mrow_bytes;
    }
};

}  // namespace

// Locking: `mu` guards the queue, the ticket map, request results and the
// counters; it is never held across a CUDA call.  The worker thread alone
// owns the slots.  Host callbacks on the slot streams touch only atomics and
// `sig_mu` (the worker's doorbell), so they can never wait on a thread that
// is itself inside a CUDA call.
struct rg_server {
    rg_ctx* ctx = nullptr;
    int64_t budget = 0;
    std::vector<Slot> slots;
    std::deque<std::shared_ptr<ServerReq>> pending;
    std::map<int64_t, std::shared_ptr<ServerReq>> reqs;
    std::mutex mu;
    std::condition_variable cv_done;
    std::mutex sig_mu;
    std::condition_variable cv_sig;
    uint64_t sig_count = 0;                // guarded by sig_mu
    std::atomic<int64_t> dev_bytes{0};
    // worker host time (seconds): request sizing, launching, result copies
    std::atomic<double> t_need{0.0}, t_launch{0.0}, t_copy{0.0};
    std::thread worker;
    bool stop = false;
    int64_t next_ticket = 1, completed = 0, failed = 0;
    std::map<int, FftLen> fft;                              // worker only
    std::map<int64_t, std::pair<float2*, float2*>> twn;     // worker only
    Clock::time_point t0 = Clock::now();
    uint32_t magic = 0x52475356;

    void ring() {
        {
            std::lock_guard<std::mutex> lk(sig_mu);
            ++sig_count;
        }
        cv_sig.notify_one();
    }

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
    int64_t used_bytes() const {
        int64_t u = 0;
        for (const Slot& sl : slots) u += (int64_t)sl.bytes();
        return u;
    }
};

namespace {

struct HostNote {
    rg_server* srv;
    int slot;
};

void CUDART_CB slot_done_cb(void* p) {
    // runs on a CUDA driver thread: no CUDA calls and no `mu` here
    auto* hn = static_cast<HostNote*>(p);
    hn->srv->slots[hn->slot].notified.store(true);
    hn->srv->ring();
    delete hn;
}

int server_tables(rg_server* S, Work& W) {
    for (int L : {W.n1, W.n2}) {
        auto it = S->fft.find(L);
        if (it == S->fft.end()) {
            FftLen f;
            RG(make_fftlen(L, &f));
            it = S->fft.emplace(L, f).first;
        }
        (L == W.n1 ? W.f1 : W.f2) = it->second;
    }
    if (W.n1 == W.n2) W.f2 = W.f1;
    auto t = S->twn.find(W.n);
    if (t == S->twn.end()) {
        float2 *hi = nullptr, *lo = nullptr;
        RG(tw_n_tables(W.n, &hi, &lo));
        t = S->twn.emplace(W.n, std::make_pair(hi, lo)).first;
    }
    W.tw_hi = t->second.first;
    W.tw_lo = t->second.second;
    return RG_OK;
}

// Workspace bytes a request needs on a slot (for admission).
int request_need(rg_server* S, const ServerReq& r, SpecHost* sh, int64_t* need, int* n1o, int* n2o) {
    int n1, n2;
    if (!choose_fft(2 * r.desc.n_v, r.desc.n_ft, &n1, &n2))
        return fail(RG_ERR_RANGE, "no supported FFT length >= %lld", (long long)(2 * r.desc.n_v));
    RG(compute_grid_env(r.lines->env, r.lines, r.desc, (int64_t)n1 * n2, n1, n2, &r.cond, sh));
    const int64_t n = (int64_t)n1 * n2, rs = (r.desc.n_v + 31) / 32 * 32;
    int E;
    double pmax;
    shift_margin(r.lines, r.desc.dv, &E, &pmax);
    *need = r.desc.n_v * 4 + (r.desc.n_v + 1 + 2 * (int64_t)E) * 8 + n * 8 +
            (int64_t)sh->n_nodes * (rs * 4 + n * 4) +
            (int64_t)sh->n_nodes * (rs + 2 * kGaussMaxK + 32) * 4;   // merged rows (at most one per node)
    *n1o = n1;
    *n2o = n2;
    (void)S;
    return RG_OK;
}

template <typename T>
int grow(T** p, int64_t* cap, int64_t want, cudaStream_t st) {
    if (want <= *cap) return RG_OK;
    if (*p) CU(cudaFreeAsync(*p, st));
    *p = nullptr;
    *cap = 0;
    CU(cudaMallocAsync((void**)p, sizeof(T) * (size_t)want, st));
    *cap = want;
    return RG_OK;
}

void release_slot_buffers(Slot& sl) {
    if (sl.w.ldm) cudaFreeAsync(sl.w.ldm, sl.st);
    if (sl.w.y) cudaFreeAsync(sl.w.y, sl.st);
    if (sl.w.g) cudaFreeAsync(sl.w.g, sl.st);
    if (sl.w.col_start) cudaFreeAsync(sl.w.col_start, sl.st);
    if (sl.out_d) cudaFreeAsync(sl.out_d, sl.st);
    sl.w.ldm = nullptr;
    sl.w.y = nullptr;
    sl.w.g = nullptr;
    sl.w.col_start = nullptr;
    sl.out_d = nullptr;
    if (sl.w.mrow) cudaFreeAsync(sl.w.mrow, sl.st);
    sl.w.mrow = nullptr;
    sl.w.mrow_bytes = 0;
    if (sl.w.proj_coef) cudaFreeAsync(sl.w.proj_coef, sl.st);
    sl.w.proj_coef = nullptr;
    sl.w.proj_bytes = 0;
    sl.w.skel_dev = false;
    sl.w.nodes_cap = 0;
    sl.w.ldm_bytes = sl.w.y_bytes = 0;
    sl.out_cap = sl.col_cap = sl.g_cap = 0;
}

// Launch request r on slot `si` (called by the worker with the lock held).
int start_on_slot(rg_server* S, int si, const std::shared_ptr<ServerReq>& r, const SpecHost& sh, int n1, int n2) {
    NvtxRange nvtx_("rg/serve_request");
    Slot& sl = S->slots[si];
    Work& W = sl.w;
    const rg_plan_desc& d = r->desc;
    W.desc = d;
    W.n1 = n1;
    W.n2 = n2;
    W.n = (int64_t)n1 * n2;
    W.B = col_block(n1);
    RG(server_tables(S, W));
    shift_margin(r->lines, d.dv, &W.E, &W.p_atm_max);
    W.col_off = W.E;
    W.col_count = (int)d.n_v + 1 + 2 * W.E;
    W.row_stride = (d.n_v + 31) / 32 * 32;
    RG(grow(&W.col_start, &sl.col_cap, W.col_count, sl.st));
    RG(grow(&W.g, &sl.g_cap, W.n, sl.st));
    // a page-locked output buffer is written by the spectrum's last kernel
    // itself: no staging copy, nothing for the worker to copy at harvest
    float* direct = mapped_host(r->out_host);
    sl.direct = direct != nullptr;
    if (!direct) RG(grow(&sl.out_d, &sl.out_cap, d.n_v, sl.st));
    if (!direct && d.n_v > sl.pin_cap) {   // grow-only, at least 2M points (8 MB)
        const int64_t cap = std::max<int64_t>({d.n_v, sl.pin_cap * 3 / 2, (int64_t)1 << 21});
        if (sl.pin) CU(cudaFreeHost(sl.pin));
        sl.pin = nullptr;
        sl.pin_cap = 0;
        CU(cudaHostAlloc((void**)&sl.pin, sizeof(float) * (size_t)cap, cudaHostAllocDefault));
        sl.pin_cap = cap;
    }
    const rg_lines* L = r->lines;
    RG(launch_col_index(L->v0, L->n, d.vmin, d.dv, -W.E, W.col_count, W.col_start, sl.st));
    RG(launch_col_cmax(W.col_start, W.col_off, W.col_count, (int)d.n_v, W.E - 1, W.cmax_dev, sl.st));
    RG(enqueue_spectrum(L, W, &r->cond, sh, direct ? direct : sl.out_d, sl.st, nullptr, false));
    if (!direct)
        CU(cudaMemcpyAsync(sl.pin, sl.out_d, sizeof(float) * (size_t)d.n_v, cudaMemcpyDeviceToHost, sl.st));
    r->info.grid = sh.grid;
    r->info.log_scale = sh.log_scale_out;
    r->info.lines_in_window = -1;
    r->info.fft_rows = W.last_fft_rows;
    r->info.merged_rows = W.last_merged_rows;
    r->info.merged_ext = W.last_ext;
    r->info.accum_bits = W.last_accum;
    r->info.layout = W.last_layout;
    r->info.layout_err = (float)W.last_layout_err;
    sl.notified.store(false);
    auto* hn = new HostNote{S, si};
    CU(cudaLaunchHostFunc(sl.st, slot_done_cb, hn));
    return RG_OK;
}

// With `mu` held.
void finish_request(rg_server* S, const std::shared_ptr<ServerReq>& r, int status, const std::string& msg) {
    r->lines->plans--;
    r->status = status;
    r->msg = msg;
    r->done = true;
    r->t_done = S->now();
    if (status == RG_OK)
        S->completed++;
    else
        S->failed++;
}

void worker_loop(rg_server* S) {
    cudaSetDevice(S->ctx->device);
    uint64_t seen = 0;
    for (;;) {
        // 1. completions (slots are the worker's; the flags come from callbacks)
        std::vector<std::pair<std::shared_ptr<ServerReq>, bool>> finished;
        bool any_busy = false;
        for (Slot& sl : S->slots) {
            if (!sl.req) continue;
            if (sl.notified.load()) {
                const bool bad = *sl.w.err_host != 0;
                *sl.w.err_host = 0;
                if (!bad && !sl.direct) {
                    const double tc = S->now();
                    std::memcpy(sl.req->out_host, sl.pin, sizeof(float) * (size_t)sl.req->desc.n_v);
                    S->t_copy.store(S->t_copy.load() + (S->now() - tc));
                }
                finished.emplace_back(sl.req, bad);
                sl.req.reset();
                sl.notified.store(false);
            } else {
                any_busy = true;
            }
        }
        // 2. take admissible requests off the queue (FIFO: the head waits)
        struct Start {
            int si;
            std::shared_ptr<ServerReq> r;
            SpecHost sh;
            int n1, n2;
        };
        std::vector<Start> starts;
        bool stopping, release_idle = false;
        {
            std::lock_guard<std::mutex> lk(S->mu);
            for (auto& f : finished)
                finish_request(S, f.first, f.second ? RG_ERR_TIMEOUT : RG_OK,
                               f.second ? "a bounded device wait in the scatter gave up" : "");
            int64_t planned = 0;   // bytes the starts below may add
            while (!S->pending.empty()) {
                auto r = S->pending.front();
                Start st;
                int64_t need;
                g_err.clear();
                const double tn = S->now();
                int rc = request_need(S, *r, &st.sh, &need, &st.n1, &st.n2);
                S->t_need.store(S->t_need.load() + (S->now() - tn));
                if (rc != RG_OK || need > S->budget) {
                    S->pending.pop_front();
                    finish_request(S, r, rc != RG_OK ? rc : RG_ERR_OOM,
                                   rc != RG_OK ? g_err : "request needs more device memory than the server budget");
                    continue;
                }
                int si = -1;
                for (size_t i = 0; i < S->slots.size(); ++i) {
                    bool taken = S->slots[i].req != nullptr;
                    for (const Start& o : starts) taken |= o.si == (int)i;
                    if (!taken) {
                        si = (int)i;
                        break;
                    }
                }
                if (si < 0) break;
                const int64_t held = (int64_t)S->slots[si].bytes();   // buffers are reused, grow-only
                const int64_t others = S->used_bytes() - held + planned;
                if (others + std::max(need, held) > S->budget) {
                    // nothing runs: give the idle slots' memory back (outside `mu`), retry
                    if (!any_busy && starts.empty() && S->used_bytes() > 0) release_idle = true;
                    break;
                }
                S->pending.pop_front();
                r->t_start = S->now();
                st.si = si;
                st.r = r;
                planned += need;
                starts.push_back(std::move(st));
            }
            stopping = S->stop && S->pending.empty();
        }
        if (!finished.empty()) S->cv_done.notify_all();
        if (release_idle) {
            for (Slot& sl : S->slots)
                if (!sl.req) release_slot_buffers(sl);
            S->dev_bytes.store(S->used_bytes());
            continue;
        }
        // 3. launch outside `mu`
        for (Start& st : starts) {
            g_err.clear();
            S->slots[st.si].req = st.r;
            const double tl = S->now();
            const int rc = start_on_slot(S, st.si, st.r, st.sh, st.n1, st.n2);
            S->t_launch.store(S->t_launch.load() + (S->now() - tl));
            if (rc != RG_OK) {
                S->slots[st.si].req.reset();
                const std::string msg = g_err;
                {
                    std::lock_guard<std::mutex> lk(S->mu);
                    finish_request(S, st.r, rc, msg);
                }
                S->cv_done.notify_all();
            } else {
                any_busy = true;
            }
        }
        S->dev_bytes.store(S->used_bytes());
        if (stopping && !any_busy) break;
        // 4. sleep until a submission or a completion rings (or 50 ms)
        std::unique_lock<std::mutex> lk(S->sig_mu);
        S->cv_sig.wait_for(lk, std::chrono::milliseconds(50), [&] { return S->sig_count != seen; });
        seen = S->sig_count;
    }
}

bool valid(const rg_server* s) { return s && s->magic == 0x52475356; }

}  // namespace

extern "C" {

int rg_server_create(rg_ctx* ctx, int slots, int64_t mem_budget, rg_server** out) {
    g_err.clear();
    if (!valid(ctx) || !out) return fail(RG_ERR_ARG, "invalid argument");
    if (slots < 1 || slots > 64) return fail(RG_ERR_ARG, "slots must be in [1, 64]");
    if (mem_budget <= 0) return fail(RG_ERR_ARG, "mem_budget must be positive");
    DeviceGuard dev_guard_;
    CU(dev_guard_.use(ctx->device));
    auto* S = new (std::nothrow) rg_server();
    if (!S) return fail(RG_ERR_OOM, "host allocation failed");
    std::unique_ptr<rg_server> guard(S);
    S->ctx = ctx;
    S->budget = mem_budget;
    S->slots = std::vector<Slot>(slots);
    for (Slot& sl : S->slots) {
        CU(cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking));
        CU(cudaMalloc(&sl.w.cmax_dev, sizeof(int)));
        CU(cudaMalloc(&sl.w.counter, sizeof(unsigned long long)));
        CU(cudaMalloc(&sl.w.err, sizeof(unsigned)));
        CU(cudaMemset(sl.w.err, 0, sizeof(unsigned)));
        CU(cudaHostAlloc(&sl.w.err_host, sizeof(unsigned), cudaHostAllocMapped));
        *sl.w.err_host = 0;
        CU(cudaHostGetDevicePointer((void**)&sl.w.err_pub, sl.w.err_host, 0));
    }
    // the FFT tables of every factorisation choose_fft can pick (n1 in {8, 64,
    // 512}, n2 = 32 x 5-smooth <= kN2Max), built before the worker starts: a
    // request never waits for a table upload (an allocation and a blocking
    // copy) on the worker thread
    for (int64_t m = 1; 32 * m <= kN2Max; m = next_smooth(m + 1))
        for (int n1 : {8, 64, 512}) {
            Work t;
            t.n1 = n1;
            t.n2 = (int)(32 * m);
            t.n = (int64_t)t.n1 * t.n2;
            RG(server_tables(S, t));
        }
    ctx->lines++;   // the context stays alive while the server exists
    S->worker = std::thread(worker_loop, S);
    *out = guard.release();
    return RG_OK;
}

int rg_server_submit(rg_server* S, const rg_request* req, int64_t* ticket) {
    g_err.clear();
    if (!valid(S) || !req || !ticket) return fail(RG_ERR_ARG, "invalid argument");
    if (!valid(req->lines) || !req->out_host) return fail(RG_ERR_ARG, "invalid line list or output buffer");
    const rg_plan_desc& d = req->grid;
    if (!(d.dv > 0) || d.n_v < 2 || d.n_v > ((int64_t)1 << 30)) return fail(RG_ERR_ARG, "bad grid");
    if (!((d.n_G > 1) || d.dxG > 0) || !((d.n_L > 1) || d.dxL > 0))
        return fail(RG_ERR_ARG, "give dxG/dxL > 0 or node counts n_G/n_L > 1");
    RG(check_desc_options(d));
    auto r = std::make_shared<ServerReq>();
    r->lines = req->lines;
    r->desc = d;
    r->cond = req->cond;
    if (req->cond.q_ratio) {
        r->q.assign(req->cond.q_ratio, req->cond.q_ratio + req->lines->n_iso);
        r->cond.q_ratio = r->q.data();
    }
    r->out_host = req->out_host;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stop) return fail(RG_ERR_STATE, "server is shutting down");
        r->lines->plans++;   // the list must outlive the request
        r->ticket = S->next_ticket++;
        r->t_submit = S->now();
        S->reqs[r->ticket] = r;
        S->pending.push_back(r);
        *ticket = r->ticket;
    }
    S->ring();
    return RG_OK;
}

int rg_server_wait(rg_server* S, int64_t ticket, double timeout_ms, rg_spectrum_info* info, double* t_submit,
                   double* t_start, double* t_done) {
    g_err.clear();
    if (!valid(S)) return fail(RG_ERR_ARG, "invalid server");
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end()) return fail(RG_ERR_ARG, "unknown ticket %lld", (long long)ticket);
    std::shared_ptr<ServerReq> r = it->second;
    auto ready = [&] { return r->done; };
    if (timeout_ms < 0) {
        S->cv_done.wait(lk, ready);
    } else if (!S->cv_done.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready)) {
        return fail(RG_ERR_TIMEOUT, "ticket %lld not finished within %g ms", (long long)ticket, timeout_ms);
    }
    if (info) *info = r->info;
    if (t_submit) *t_submit = r->t_submit;
    if (t_start) *t_start = r->t_start;
    if (t_done) *t_done = r->t_done;
    S->reqs.erase(ticket);
    if (r->status != RG_OK) return fail(r->status, "%s", r->msg.c_str());
    return RG_OK;
}

int rg_server_stats_get(rg_server* S, rg_server_stats* st) {
    g_err.clear();
    if (!valid(S) || !st) return fail(RG_ERR_ARG, "invalid argument");
    std::lock_guard<std::mutex> lk(S->mu);
    st->completed = S->completed;
    st->failed = S->failed;
    st->queued = (int64_t)S->pending.size();
    st->submitted = S->next_ticket - 1;
    st->in_flight = st->submitted - st->completed - st->failed - st->queued;
    st->device_bytes = S->dev_bytes.load();
    st->host_need_ms = S->t_need.load() * 1e3;
    st->host_launch_ms = S->t_launch.load() * 1e3;
    st->host_copy_ms = S->t_copy.load() * 1e3;
    return RG_OK;
}

int rg_server_destroy(rg_server* S) {
    g_err.clear();
    if (!S) return RG_OK;
    if (!valid(S)) return fail(RG_ERR_STATE, "invalid server");
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->ring();
    if (S->worker.joinable()) S->worker.join();
    DeviceGuard dev_guard_;
    dev_guard_.use(S->ctx->device);
    for (Slot& sl : S->slots) {
        cudaStreamSynchronize(sl.st);
        release_slot_buffers(sl);
        cudaStreamSynchronize(sl.st);
        dfree(sl.w.cmax_dev);
        dfree(sl.w.counter);
        dfree(sl.w.err);
        if (sl.w.err_host) cudaFreeHost(sl.w.err_host);
        if (sl.pin) cudaFreeHost(sl.pin);
        cudaStreamDestroy(sl.st);
    }
    for (auto& kv : S->fft) dfree(kv.second.tw);
    for (auto& kv : S->twn) {
        dfree(kv.second.first);
        dfree(kv.second.second);
    }
    S->ctx->lines--;
    S->magic = 0;
    delete S;
    return RG_OK;
}

}  // extern "C"

// ===========================================================================
// Allocation-free synthesis over a static device scratch array
// ===========================================================================
// For callers that must not allocate device memory at the time they ask for a
// spectrum: code running while a framework's caching allocator owns the
// device memory, inside a memory-accounted service that forbids
// cudaMalloc/cudaFree on the request path, or between setup and teardown of
// a pre-sized job.  Every scratch buffer of one spectrum lives in this array;
// every GPU that loads this library holds it until the process exits.
constexpr size_t kStaticScratchBytes = (size_t)64 << 20;   // 64 MiB
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];
constexpr size_t kStaticProjBytes = 256 * 1024;

namespace {

std::mutex g_static_mu;                      // serialises calls (they share the array)
void* g_static_ptr[64] = {nullptr};          // device address of the array, per device
unsigned g_static_err_host = 0;              // host word the device error flag lands in

// exp(-2 pi i t / L) for t < count (FP64 sincospi, rounded to FP32)
__global__ void k_static_twiddles(float2* tw, int count, long long L, long long stride) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    const long long q = ((long long)t * stride) % L;
    double s, c;
    sincospi(2.0 * (double)q / (double)L, &s, &c);
    tw[t] = make_float2((float)c, (float)-s);
}

int static_twiddles(float2* tw, int count, long long L, long long stride, cudaStream_t st) {
    k_static_twiddles<<<(count + 255) / 256, 256, 0, st>>>(tw, count, L, stride);
    return cudaGetLastError() == cudaSuccess ? RG_OK : RG_ERR_CUDA;
}

// radix plan of one FFT length without any table (the table goes to scratch)
int static_fftlen(int L, FftLen* f) {
    f->L = L;
    if (!radices(L, f->radix, &f->npass)) return fail(RG_ERR_RANGE, "FFT length %d not factorable", L);
    int ns = 1;
    for (int p = 0; p < f->npass; ++p) {
        f->ns[p] = ns;
        f->mag[p] = ns == 1 ? 0u : (unsigned)(((1ull << 32) + ns - 1) / (unsigned long long)ns);
        ns *= f->radix[p];
    }
    return RG_OK;
}

}  // namespace

extern "C" int rg_synthesize_static(rg_lines* L, const rg_plan_desc* d, const rg_conditions* c, float* out_dev,
                                    void* stream, rg_spectrum_info* info) {
    g_err.clear();
    if (!valid(L) || !d || !c || !out_dev) return fail(RG_ERR_ARG, "invalid argument");
    if (!(d->dv > 0) || d->n_v < 2 || d->n_v > ((int64_t)1 << 30)) return fail(RG_ERR_ARG, "bad grid");
    if (!((d->n_G > 1) || d->dxG > 0) || !((d->n_L > 1) || d->dxL > 0))
        return fail(RG_ERR_ARG, "give dxG/dxL > 0 or node counts n_G/n_L > 1");
    RG(check_desc_options(*d));
    const int dev = L->ctx->device;
    if (dev < 0 || dev >= 64) return fail(RG_ERR_ARG, "device ordinal %d not supported", dev);
    std::lock_guard<std::mutex> lk(g_static_mu);
    DeviceGuard dev_guard_;
    CU(dev_guard_.use(dev));
    if (!g_static_ptr[dev]) {
        // once per device, with the device current: host code cannot use the
        // array's name as an address, it needs the device address
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p)
            return fail(RG_ERR_CUDA, "cudaGetSymbolAddress(static scratch): %s", cudaGetErrorString(e));
        g_static_ptr[dev] = p;
    }
    unsigned char* base = static_cast<unsigned char*>(g_static_ptr[dev]);
    cudaStream_t st = stream ? (cudaStream_t)stream : L->ctx->stream;

    Work W;
    W.desc = *d;
    int n1, n2;
    if (!choose_fft(2 * d->n_v, d->n_ft, &n1, &n2))
        return fail(RG_ERR_RANGE, "no supported FFT length >= %lld", (long long)(2 * d->n_v));
    W.n1 = n1;
    W.n2 = n2;
    W.n = (int64_t)n1 * n2;
    W.B = col_block(n1);
    RG(static_fftlen(n1, &W.f1));
    RG(static_fftlen(n2, &W.f2));
    shift_margin(L, d->dv, &W.E, &W.p_atm_max);
    W.col_off = W.E;
    W.col_count = (int)d->n_v + 1 + 2 * W.E;
    W.row_stride = (d->n_v + 31) / 32 * 32;
    SpecHost s;
    RG(compute_grid_env(L->env, L, W.desc, W.n, W.n1, W.n2, c, &s));

    // carve the scratch (256-byte aligned pieces)
    size_t off = 0;
    auto take = [&](size_t bytes) {
        void* q = base + off;
        off += (bytes + 255) / 256 * 256;
        return q;
    };
    const int nh = (int)(W.n / 1024) + 2;
    W.col_start = static_cast<int64_t*>(take(sizeof(int64_t) * (size_t)W.col_count));
    W.cmax_dev = static_cast<int*>(take(sizeof(int)));
    W.counter = static_cast<unsigned long long*>(take(sizeof(unsigned long long)));
    W.err = static_cast<unsigned*>(take(sizeof(unsigned)));
    W.f1.tw = static_cast<float2*>(take(sizeof(float2) * (size_t)n1));
    W.f2.tw = static_cast<float2*>(take(sizeof(float2) * (size_t)n2));
    float2* twh = static_cast<float2*>(take(sizeof(float2) * (size_t)nh));
    float2* twl = static_cast<float2*>(take(sizeof(float2) * 1024));
    W.tw_hi = twh;
    W.tw_lo = twl;
    // sized here: the workspace step finds them large enough and allocates nothing;
    // the merged layout (its own row buffer) is not used on this path; the
    // skeleton layout's coefficients get a fixed piece (the largest a grid can
    // need: [n][rp] <= 96 KB plus tensor-core fragments < 150 KB)
    W.allow_merge = false;
    W.allow_skeleton = true;
    W.proj_fixed = true;
    W.proj_bytes = kStaticProjBytes;
    W.proj_coef = static_cast<float*>(take(kStaticProjBytes));
    W.ldm_bytes = sizeof(float) * (size_t)s.n_nodes * (size_t)W.row_stride;
    W.y_bytes = sizeof(float2) * (size_t)(s.n_nodes / 2) * (size_t)W.n;
    W.ldm = static_cast<float*>(take(W.ldm_bytes));
    W.y = static_cast<float2*>(take(W.y_bytes));
    W.g = static_cast<float2*>(take(sizeof(float2) * (size_t)W.n));
    if (off > kStaticScratchBytes)
        return fail(RG_ERR_RANGE,
                    "spectrum needs %zu bytes of scratch, more than the %zu-byte static array of the "
                    "allocation-free path (use a plan)",
                    off, kStaticScratchBytes);
    W.err_host = &g_static_err_host;

    // From the first enqueue on, every return (an error included) waits for
    // the work already on `st` before the lock is released, so that the next
    // call never reuses the scratch while this call's kernels still run.
    struct DrainOnExit {
        cudaStream_t st;
        bool armed = false;
        ~DrainOnExit() {
            if (armed) cudaStreamSynchronize(st);
        }
    } drain{st};
    drain.armed = true;
    // every piece starts from what the previous call left: clear what must be zero
    CU(cudaMemsetAsync(W.err, 0, sizeof(unsigned), st));
    RG(static_twiddles(W.f1.tw, n1, n1, 1, st));
    RG(static_twiddles(W.f2.tw, n2, n2, 1, st));
    RG(static_twiddles(twh, nh, W.n, 1024, st));
    RG(static_twiddles(twl, 1024, W.n, 1, st));
    RG(launch_col_index(L->v0, L->n, d->vmin, d->dv, -W.E, W.col_count, W.col_start, st));
    RG(launch_col_cmax(W.col_start, W.col_off, W.col_count, (int)d->n_v, W.E - 1, W.cmax_dev, st));
    RG(enqueue_spectrum(L, W, c, s, out_dev, st, nullptr, false));
    drain.armed = false;
    CU(cudaStreamSynchronize(st));
    if (g_static_err_host) {
        g_static_err_host = 0;
        return fail(RG_ERR_TIMEOUT, "a bounded device wait in the scatter gave up; the spectrum is invalid");
    }
    if (info) {
        std::memset(info, 0, sizeof *info);
        info->grid = s.grid;
        info->log_scale = s.log_scale_out;
        info->lines_in_window = -1;
        info->fft_rows = W.last_fft_rows;
        info->accum_bits = W.last_accum;
        info->layout = W.last_layout;
    }
    return RG_OK;
}
