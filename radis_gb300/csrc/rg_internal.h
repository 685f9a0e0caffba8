// Internal types shared by the host side (rg_api.cu, rg_hull.cpp) and the
// kernels (rg_kernels.cu).  Not part of the public ABI.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/radis_gb300.h"

#ifdef __CUDACC__
#include <cuda_runtime.h>
#else
struct float2 { float x, y; };
typedef struct CUstream_st* cudaStream_t;
#endif

namespace rg {

// --- physical constants (radis/phys/constants.py:22,33,38,60,69,75,78) -------
constexpr double kH = 6.62607015e-34;
constexpr double kC = 2.99792458e8;
constexpr double kKb = 1.3806490e-23;
constexpr double kNA = 6.02214076e23;
constexpr double kC2 = kH * kC / kKb * 100.0;      // hc/k, cm K
constexpr double kCcgs = 2.99792458e10;
constexpr double kKbCgs = 1.380648813e-16;         // the CPU Doppler width's k (erg/K)
constexpr double kPi = 3.14159265358979323846;
constexpr double kLn2 = 0.69314718055994530942;
constexpr double kLog2e = 1.44269504088896340736;
constexpr double kAtm = 1.01325;                    // bar per atm (broadening.py:1063)

constexpr int kMaxIso = 16;
constexpr int kMaxAxis = 64;        // max nodes along one LDM axis
constexpr int kMaxNodes = 1024;     // max N_G * N_L (padded to even)
constexpr int kPairGroup = 16;      // node pairs per Voigt-reduce work item
constexpr int kMaxPasses = 16;
// FFT radix plans merge the small factors into composite radices of at most
// kFirstRadixMax in the first pass (no pass twiddles) and kMidRadixMax later:
// the bounds under which the row kernels keep two pairs' butterflies in
// registers without spilling
constexpr int kFirstRadixMax = 12;
constexpr int kMidRadixMax = 6;

// --- host work over line arrays ------------------------------------------------
// [0, n) in T contiguous chunks, chunk t = [n t / T, n (t + 1) / T): one per
// host thread, each of at least min_per items (T = 1 for small n).  Per-chunk
// partial results merged in chunk order reproduce the sequential pass.
inline int host_chunk_count(int64_t n, int64_t min_per) {
    const int64_t hc = std::max(1u, std::thread::hardware_concurrency());
    return (int)std::max<int64_t>(1, std::min<int64_t>(std::min<int64_t>(hc, 64), n / std::max<int64_t>(min_per, 1)));
}
// Runs f(t, begin, end) for the T chunks of [0, n), chunk 0 on the calling thread.
template <typename F>
void run_host_chunks(int T, int64_t n, F&& f) {
    std::vector<std::thread> th;
    th.reserve(T > 1 ? T - 1 : 0);
    for (int t = 1; t < T; ++t) th.emplace_back([&f, t, T, n] { f(t, n * t / T, n * (t + 1) / T); });
    f(0, (int64_t)0, T > 1 ? n / T : n);
    for (auto& x : th) x.join();
}
constexpr int64_t kHostMinPerThread = 1 << 18;

// --- host-side convex envelopes (rg_hull.cpp) ---------------------------------
// Lower convex hull of points (a_i, b_i): min_i (b_i + a_i t) for every t is
// attained at one of its vertices.
struct Hull {
    std::vector<double> a, b;
    double min_at(double t) const;
    double max_at(double t) const;   // for an upper hull stored as-is
};
// exact lower hull / upper hull of n points (non-finite b values are skipped)
Hull lower_hull(const double* a, const double* b, int64_t n);
Hull upper_hull(const double* a, const double* b, int64_t n);
// Same, with the point coordinates produced on the fly by a functor-like
// callback to avoid materialising n-length temporaries.
struct PointSource {
    virtual ~PointSource() {}
    virtual int64_t size() const = 0;
    virtual void get(int64_t i, double* a, double* b) const = 0;
    // a of point i, and whether both coordinates are finite (the points the
    // hull uses); an override must agree with get() exactly and may skip
    // computing b
    virtual bool valid_a(int64_t i, double* a) const {
        double b;
        get(i, a, &b);
        return std::isfinite(*a) && std::isfinite(b);
    }
};
Hull lower_hull_src(const PointSource& s);
Hull upper_hull_src(const PointSource& s);

// --- FFT plan of one sub-length -------------------------------------------------
struct FftLen {
    int L = 0;
    int npass = 0;
    int radix[kMaxPasses] = {0};
    int ns[kMaxPasses] = {0};          // sub-transform length before each pass
    unsigned mag[kMaxPasses] = {0};    // ceil(2^32 / ns): j / ns == umulhi(j, mag) for j, ns < 2^16
    float2* tw = nullptr;       // device: exp(-2 pi i t / L), t < L
};

// --- kernel argument blocks (passed by value) ----------------------------------
struct ScatterArgs {
    const float2* v0;     // (hi, lo) split of the FP64 line centre
    const float* ls2;     // log2 S_ref - log2(1 - exp(-c2 v0 / Tref))
    const float* el;
    const float* ga;
    const float* gs;
    const float* na;
    const float* dl;      // nullable
    const uint8_t* iso;   // nullable
    const int64_t* col_start;   // first line with v0 >= vmin + c dv, c = idx - col_off
    int col_off;
    int col_count;
    int n_v;
    int TK;               // columns per tile (multiple of 8)
    int n_nodes;          // padded to even
    int NG, NL;
    int64_t row_stride;
    float* ldm;           // LDM values: the tile's fixed-point sums / fx_scale, converted at the flush
    int margin_cols;
    float vmin_hi, vmin_lo;
    float inv_dv_hi, inv_dv_lo;
    float p_atm;
    float x_self;
    float lgG_scale;          // ln2 / dxG
    float inv_vref;           // 1 / v_ref (v_ref: geometric middle of the list's v0 range)
    float cG[kMaxIso];        // (log v_ref + log_c2Mm[iso] + 0.5 log T - log_wG_min) / dxG
    float lgL_scale;          // ln2 / dxL
    float tL;                 // log(Tref/T) / dxL
    float cL;                 // (log(2 p_atm) - log_wL_min) / dxL
    float aT_hi, aT_lo;       // -c2 (1/T - 1/Tref) log2e (double-float)
    float bI_hi[kMaxIso], bI_lo[kMaxIso];   // (log(Qr N x) - log_scale) log2e
    float stim_c;             // c2/T log2e
    unsigned long long* in_window;   // nullable counter of lines in the window
    // persistent TMA-fed scatter
    const int* cmax;          // device: most lines that can touch one column (sets the fixed-point scale)
    int n_tiles;
    int chunk;                // lines per staged chunk (multiple of 16)
    int stages;               // chunk buffers in the TMA ring (2..kScatMaxStages)
    unsigned* err;            // set to 1 when a bounded wait gives up
    long long wait_limit;     // SM clock cycles a producer/consumer handshake wait may take
    int withhold;             // test hook: the producer issues no line copies, so the
                              // consumers' waits run out (the error path, exercised safely)
    // skeleton layout fused into the flush (proj_coef non-null): each finished
    // tile is written as proj_rows skeleton rows (ldm rows [0, proj_rows)),
    // row r = sum over the n_real node rows of proj_coef[node * proj_rp + r] x row
    const float* proj_coef;   // [n_real][proj_rp], staged into shared memory after the tile
    int proj_rows;            // even; rows >= the skeleton's are zero rows
    int proj_rp;              // coefficient pitch, a multiple of 4
    int n_real;               // NG x NL (the pad node of an odd grid is not read)
    // tensor-core form of that flush (32-bit tiles; nullable): B fragments
    // [proj_ks][proj_nr][32] x 4 floats (b0, b1 TF32 hi, then lo), then the
    // node table [proj_ks][8] ints (step s: node(s, t), node(s, t + 4) for
    // t = 0..3)
    const float* proj_frag;
    int proj_ks;              // node steps of 8
    int proj_nr;              // row blocks of 8 (1 or 2)
    int rng_cap;              // entries of the per-tile line-range table (>= tiles per CTA, even)
};
constexpr long long kScatWaitCycles = 1LL << 31;   // about one second of SM clocks

// Lines are staged per chunk as [v0 8B][ls2][el][ga][gs][na][dl 4B each][iso 1B]
// x chunk; line arrays are allocated with room for a multiple of 16 lines.
constexpr int kLinePad = 16;
constexpr int kScatThreads = 1024;
constexpr int kScatMaxTilesPerCta = 512;
#ifdef __CUDACC__
#define RG_HD __host__ __device__
#else
#define RG_HD
#endif
constexpr int kScatMaxStages = 4;
RG_HD inline size_t scatter_stage_bytes(int chunk) { return (size_t)33 * chunk; }
// bytes of the tensor-core flush's fragments and node table in shared memory
RG_HD inline size_t flush_tc_bytes(int ks, int nr) { return (size_t)ks * nr * 512 + (size_t)ks * 32; }
// stage ring, its full and empty mbarriers (one 64-byte block) and the
// per-tile line ranges (rng_cap entries of 8 bytes, rng_cap even: the tile
// after them starts on a 16-byte boundary)
RG_HD inline size_t scatter_fixed_smem(int chunk, int stages, int rng_cap) {
    return stages * scatter_stage_bytes(chunk) + 16 * kScatMaxStages + 8 * (size_t)rng_cap;
}
// byte offset of the flush coefficients (skeleton layout) after a tile of
// `words` accumulator words of `word` bytes
RG_HD inline size_t scatter_coef_offset(size_t words, size_t word) { return (words * word + 15) / 16 * 16; }

struct ColFftArgs {       // K2 (forward column FFT) and K4 (inverse column FFT)
    FftLen f1;
    int n1, n2;
    int B;                // columns per CTA
    int n_v;
    int64_t n;            // n_ft
    int64_t row_stride;
    int n_pairs;
    const float* ldm;     // K2 input: the scatter's LDM [node][row_stride]
    const int* cmax;      // device: fixed-point bound of the scatter (scale = fx_scale(*cmax))
    float2* y;            // K2 output [pair][n1][n2]
    const float2* tw_hi;  // exp(-2 pi i 1024 t / N)
    const float2* tw_lo;  // exp(-2 pi i t / N), t < 1024
    const float2* h;      // K4 input [n1][n2]
    float* out;           // K4 output (n_v)
    float out_scale;
    // float-row variants (tangent and adjoint paths)
    const float* src;     // K2 input rows [node][row_stride] (float), or one row when single
    int single;           // K2: one real row (partner row zero), n_pairs = 1
    int twiddle;          // K2: apply the four-step twiddle (row kernel without table)
    int ext;              // K2 float rows: 0, or the rows hold k in [-ext, n_v + ext) at offset k + ext
                          // (circular: k < 0 is FFT index n + k)
    int pair_base;        // K2: first output pair in y
    int map_n;            // K2 fixed point: 0, or virtual row v (blocks of map_NLv rows) reads LDM
    int map_NL, map_NLv;  //   node map_l[v / map_NLv] * map_NL + v % map_NLv, zero when v % map_NLv >= map_NL
    unsigned char map_l[kMaxAxis];
    unsigned* err;        // K4: non-null with err_pub: publish the device error flag
    unsigned* err_pub;    //   into host-mapped memory and clear it (one thread)
    // K4 epilogue (q_out non-null): the post-processing of eq_spectrum_gpu
    // (radis/lbl/factory.py:1284-1297) on each abscoeff value as it is written:
    // q_out rows of n_v floats = absorbance (x exp(-log_scale), like out),
    // emissivity, transmittance, radiance (mW/cm2/sr/nm at Planck(1e7/v nm, T))
    float* q_out;
    float q_scale;        // exp(log_scale): out x q_scale = abscoeff in cm-1 (may be inf)
    float q_path;         // path length (cm)
    float q_c2_T;         // hc / (k T) in cm
    double q_vmin, q_dv;  // v_k = q_vmin + k q_dv (cm-1)
};

struct VoigtArgs {        // K3 (row FFT + Voigt weights + pair reduction)
    FftLen f2;
    int store_g;          // 1: one pair group: store the sums into G (no zeroing, no atomics)
    int threads;          // block size (row_threads), >= n2 / 8
    int pairs_per_pass;   // 2: two pairs as float4 elements; 1: one pair (long rows)
    int row_twiddle_table;// 1: the row kernel applies the four-step twiddle from a
                          // per-row shared table; 0: the column stage applies it
    int n1, n2;
    int64_t n;
    int n_pairs;
    int n_nodes;
    int NL;
    const float2* y;
    float2* g;            // accumulator [n1][n2]
    const float2* tw_hi;  // exp(-2 pi i 1024 t / N)
    const float2* tw_lo;  // exp(-2 pi i t / N), t < 1024
    float inv_ndv;        // 1 / (N dv)
    float half_fs;        // 1 / (2 dv)
    float alpha[kMaxAxis];    // (pi wG_l)^2 / (4 ln 2) * log2e
    float beta[kMaxAxis];     // pi wL_m * log2e
    float norm[kMaxNodes];    // 1 / folded profile at f = 0 (0 for padding node)
    float lnorm[kMaxNodes];   // log2(norm) (-inf for padding node)
    unsigned char nfold[kMaxNodes];
    int any_fold;
    int rowwise;          // 1: row r's transform uses alpha[r], beta[r] (skeleton rows, r < kMaxAxis)
    int inv_fused;        // 1 (with store_g, one pair group): the CTA also applies the inverse
                          // row DFT and inverse twiddle (K3b) to its row of sums before storing it
};

struct RowIfftArgs {      // K3b (inverse row FFT + twiddle, in place)
    FftLen f2;
    int n1, n2;
    int64_t n;
    float2* g;
    const float2* tw_hi;
    const float2* tw_lo;
};

// Gaussian stage of the merged layout: node rows of equal wL whose Gaussian
// FT is negligible at the Nyquist frequency are convolved in real space with
// their Gaussian kernel and summed into one row per wL node (the other,
// narrow-Gaussian node rows stay in the LDM).  Output rows [m][out_stride]
// hold k in [-ext, n_v + ext) at offset k + ext.
// Skeleton layout: the LDM rows projected, in place, onto the rows of a few
// skeleton nodes whose transforms span every node's (interp_decomp):
// row r (r < rows) <- sum_n coef[n * rows_pad + r] x row n, column by column;
// rows [R, rows) of an odd R are the zero pad row.
constexpr int kProjMaxRows = 64;
struct ProjArgs {
    float* ldm;           // LDM [node][row_stride], rows [0, rows) overwritten
    int64_t row_stride;
    int n_v;
    int n_nodes;          // rows read
    int rows;             // rows written (R rounded up to even)
    int rows_pad;         // coefficient row pitch (the kernel's row block)
    const float* coef;    // [n_nodes][rows_pad]
    int sms;              // SMs of the device (persistent grid)
    // tensor-core form: the coefficients as TF32 hi / lo parts in the B
    // fragments of mma.m16n8k8 (rows in blocks of 8, nodes in steps of 8):
    // frag[((nr * ksteps + ks) * 2 + part) * 64 + lane * 2 + i]
    const float* frag;    // null: FP32 pass
    int mtiles;           // row blocks of 8 (<= 8)
    int ksteps;           // node steps of 8 in frag (a multiple of 2)
    // the scatter flush's tensor-core section (ScatterArgs::proj_frag; null
    // where the grid has none)
    const float* flush;
    int flush_ks, flush_nr;
};
// TF32 (10-bit mantissa) rounding to nearest even, as the host prepares the
// tensor-core operands; x - tf32(x) is exact in FP32
inline float tf32_round_host(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u += 0x0FFFu + ((u >> 13) & 1u);
    u &= 0xFFFFE000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

constexpr int kGaussPer = 8;          // outputs per thread
constexpr int kGaussTile = 256 * kGaussPer;   // outputs per CTA (256 threads)
constexpr int kGaussMaxK = 256;       // widest kernel half-width (points)
struct GaussArgs {
    const float* ldm;     // LDM [node][row_stride]
    int64_t row_stride;
    const int* cmax;      // fixed-point bound (scale)
    float* out;
    int64_t out_stride;
    int n_v, ext, NL;
    int NLv;              // NL rounded up to even: rows per block of the merged layout
    int rows;             // rows of the merged layout: NLv (merged) + NLv * n_narrow (LDM rows)
    int n_wide, n_narrow;
    int wide_l[kMaxAxis], K[kMaxAxis];       // wide nodes and kernel half-widths
    float c[kMaxAxis], a2[kMaxAxis];         // taps c ex2(-a2 j^2), |j| <= K
    int narrow_l[kMaxAxis];
    int slot_taps, slot_len;                 // set by the launcher: floats per ring slot (taps, taps + window)
    // The wide Gaussians are split as g_l = d_l conv g_b (sigma_l^2 = sigma_d^2 +
    // sigma_b^2, one base g_b shared by all wide l): c/a2/K above describe the
    // residual d_l, and the base is applied to the merged rows in Fourier space
    // by the row kernel (its alpha of the merged block)
};

// Tabulated partition function of one isotopologue (rg_partition.cpp)
struct QTable {
    int interp = RG_Q_LINEAR;
    std::vector<double> T, Q, M;   // M: spline second derivatives (RG_Q_CUBIC)
};
int qtable_build(int64_t n, const double* T, const double* Q, int interp, QTable* out, std::string* err);
int qtable_eval(const QTable& t, double T, double* q, double* dq_dT, std::string* err);

// HITRAN-160 records -> columns (rg_hitran.cpp)
int hitran_count(const char* text, int64_t nbytes, int threads, int64_t* n_records);
int hitran_parse(const char* text, int64_t nbytes, int threads, const rg_hitran_columns* out, std::string* err);

// Instrument slit convolution ('same' part of the full convolution, x scale)
constexpr int kSlitPass = 512;        // slit taps staged per pass
struct SlitArgs {
    const float* in;      // spectrum [n]
    const float* slit;    // slit sampled on the spectrum step [m]
    float* out;           // [n], not aliasing in
    int64_t n;
    int m;
    float scale;          // wstep (slit.py:737)
    int valid;            // 1: NaN on the boundary points (remove_boundary 'valid')
};

struct AdjRowArgs {       // adjoint row stage: per pair, IFFT_row(Ghat (V_a + i V_b)) x twiddle
    VoigtArgs v;          // v.g holds Ghat [n1][n2] (FFT of the upstream gradient)
    float2* y;            // output [pair][n1][n2]
};

struct GradArgs {         // adjoint gather (reverse mode) and tangent scatter (forward mode)
    ScatterArgs s;        // per-line coefficients at the conditions (fixed point unused)
    int64_t n_lines;
    const float* adj;     // gather input: adjoint LDM rows [node][row_stride]
    float* tan;           // tangent output: LDM rows [node][row_stride], zeroed
    int64_t row_stride;
    int theta;            // tangent direction: 0 = T, 1 = p_bar, 2 = x
    float c2_T, c2_T2;    // c2 / T, c2 / T^2
    float cT0[kMaxIso];   // d ln(Qref/Q)/dT - 1/T (partition ratio and number density)
    float gT;             // d(log-wG node coordinate)/dT = 0.5 / (T dxG)
    float lT, lP, lX;     // 1/(T dxL), 1/(p_bar dxL), 1/dxL
    float kP;             // d(grid position)/d(p_bar) per unit shift = 1 / (1.01325 dv)
    float iP, iX;         // 1/p_bar, 1/x
    double* out;          // gather output: d/dT, d/dp_bar, d/dx sums, zeroed
    // skeleton layout: adj holds the skeleton rows Z_r (r < proj_rows) and a
    // node's adjoint row is sum_r proj_coef[node * proj_rp + r] Z_r (gather);
    // null: adj holds every node row
    const float* proj_coef;
    int proj_rows, proj_rp, proj_n;
};

// Fixed-point scale of the scatter accumulator: 2^e with (cmax + 1) 2^e <= 2^31
// for the 32-bit accumulator (width 31), 2^63 for the 64-bit one (width 63).
// A line adds at most its scaled intensity (<= 1) to a cell and at most cmax
// lines touch a grid column, so no cell sum can overflow.
RG_HD inline float fx_scale_of(int cmax, int width = 31) {
    int bits = 0;
    while (bits < 31 && (1u << bits) <= (unsigned)(cmax + 1)) ++bits;
    const int e = width - bits;
    float s = 1.f;
    for (int i = 0; i < e; ++i) s *= 2.f;
    return s;
}
// The 32-bit accumulator rounds every add to 2^-e of the strongest line, with
// 2^e ~ 2^31 / cmax.  Over the many adds of a dense column the rounding adds up
// like a random walk: a CPU emulation of that rounding on a forest of weak lines
// (2M lines over 200 columns at 0.01 cm-1, cmax 40 470) gives 7.7e-5 of the peak
// absorption, and the error scales as sqrt(cmax).  Up to cmax = 8192 it stays
// below ~3.5e-5; beyond, the scatter accumulates in 64 bits (5e-9 in the same
// emulation), at twice the shared memory per tile cell.
constexpr int kFxNarrowMaxLines = 8192;
RG_HD inline bool fx_wide(int cmax) { return cmax > kFxNarrowMaxLines; }

// --- launchers (rg_kernels.cu) ---------------------------------------------------
int launch_prepare_lines(const double* v0_d, const double* s_d, int64_t n, double c2_tref,
                         float2* v0_out, float* ls2_out, int* unsorted_flag, cudaStream_t st);
int launch_col_index(const float2* v0, int64_t n, double vmin, double dv, int c_min, int count,
                     int64_t* col_start, cudaStream_t st);
// max over grid columns of the lines within E columns (fixed-point bound), into *cmax
int launch_col_cmax(const int64_t* col_start, int col_off, int col_count, int n_v, int E, int* cmax,
                    cudaStream_t st);
// wide: the 64-bit accumulator variant
int launch_scatter(const ScatterArgs& a, int grid, int threads, size_t smem, bool wide, cudaStream_t st);
// one launch, the accumulator chosen on the device from *cmax (a32 / a64: the two shapes)
int launch_scatter_auto(const ScatterArgs& a32, const ScatterArgs& a64, int grid, int threads, size_t smem,
                        cudaStream_t st);
int scatter_smem_optin(size_t* avail, bool wide);
int launch_col_fft_fwd(const ColFftArgs& a, cudaStream_t st);
int launch_row_fft_voigt(const VoigtArgs& a, cudaStream_t st);
int launch_row_ifft(const RowIfftArgs& a, cudaStream_t st);
int launch_col_ifft(const ColFftArgs& a, cudaStream_t st);
// tangent / adjoint path (forward-mode and reverse-mode derivatives)
int launch_col_fft_fwd_f(const ColFftArgs& a, cudaStream_t st);
int launch_row_ifft_adj(const AdjRowArgs& a, cudaStream_t st);
int launch_col_ifft_adj(const ColFftArgs& a, cudaStream_t st);
int launch_gather_grad(const GradArgs& a, int grid, cudaStream_t st);
int launch_gauss_merge(const GaussArgs& a, int out_rows, cudaStream_t st);
const char* last_launch_error();     // the CUDA error of this thread's last failed launch, or null
int proj_rows_pad(int rows);         // pitch of the [node][pitch] projection coefficients for `rows` rows
// shared memory of the tensor-core projection pass (launch_node_project) for
// `row_blocks` blocks of 8 rows and `ksteps` node steps of 8; at most kProjTcSmemMax
size_t proj_tc_smem(int row_blocks, int ksteps);
constexpr size_t kProjTcSmemMax = 200 * 1024;
int launch_node_project(const ProjArgs& a, cudaStream_t st);
// interpolative decomposition of the n columns of A (S samples each, column
// major): skeleton columns sk[0, R) and coefficients C[r * n + j] with
// |A_j - sum_r C[r][j] A_sk[r]| <= tol at every sample; RG_ERR_RANGE when R
// would exceed r_max (rg_skeleton.cpp)
int interp_decomp(const double* A, int S, int n, double tol, int r_max, int* sk, double* C, int* R_out,
                  double* err_out);
int launch_slit_conv(const SlitArgs& a, cudaStream_t st);
int launch_scatter_tangent(const GradArgs& a, int grid, cudaStream_t st);
int col_block(int n1);               // columns per CTA of the column FFTs
int row_threads(const FftLen& f);    // block size of the forward row kernel
struct RowLayout {         // forward row kernel layout for rows of n2 points
    int pairs;            // node pairs per element (2: float4, 1: float2)
    int maxt;             // block size limit
    int twr;              // per-row four-step twiddle table (else the column stage twiddles)
    int stage;            // cp.async staging of the next two rows
};
RowLayout row_layout(int n2);

}  // namespace rg
