/*
 * radis_gb300 — C ABI of the GB300 (sm_103a) equilibrium LDM/DIT spectrum
 * synthesis.  Plain pointers and sizes only; no torch or CUDA-runtime types
 * in the signatures (streams are passed as `void*` = cudaStream_t).
 *
 * The entry points replace the reference's GPU application object
 * (radis 0.17.1, paths relative to the radis project root):
 *
 *   rg_ctx_create / rg_ctx_destroy  <- GPUApplication.__init__ / free
 *        (radis/gpu/vulkan/vulkan_compute_lib.py:26-73, gpu.py:376-380)
 *   rg_lines_upload / rg_lines_free <- gpuApp.__init__ line-database upload
 *        (radis/gpu/gpu.py:127-203; init_G_params/init_L_params params.py:8-81)
 *   rg_plan_create / rg_plan_free   <- gpuApp.__init__ grid, buffers and
 *        pre-recorded command list (gpu.py:133-141, 205-284)
 *   rg_plan_grid                    <- set_pTQ/set_G_params/set_L_params +
 *        get_griddims (params.py:89-155, gpu.py:372-374)
 *   rg_synthesize_quantities <- gpuApp.iterate + the host post-processing of
 *        eq_spectrum_gpu (radis/lbl/factory.py:1284-1297), on the device
 *   rg_slit_convolve <- radis/tools/slit.py:convolve_with_slit (the CPU
 *        instrument slit the reference applies after the GPU path)
 *   rg_lines_set_partition / rg_partition_eval <- the tabulated partition
 *        functions behind eq_spectrum_gpu's Q(T) callables
 *        (radis/levels/partfunc.py:1191-1192, partfunc_cdsd.py:84-117;
 *        gpuApp evaluates them per iterate, radis/gpu/params.py:154-155)
 *   rg_synthesize / rg_synthesize_host <- gpuApp.iterate (gpu.py:302-370):
 *        clear -> FillLDM (cmdFillLDM.comp) -> R2C FFT -> ApplyLineshapes
 *        (cmdApplyLineshapes.comp) -> C2R IFFT -> D2H
 *   rg_grid_estimate                <- the same rules on host arrays, no device
 *   rg_hitran_count / rg_hitran_parse <- the HITRAN-160 column parse of hit2df
 *        (radis/api/hitranapi.py:82-105, 182-380; parse_hitran_file,
 *        radis/api/tools.py:25-78), host only
 *   rg_debug_ldm                    <- no reference entry point: reads back the
 *        LDM tensor so the scatter can be checked on its own
 *   rg_backward / rg_jvp            <- no reference entry point: derivatives of
 *        the spectrum with respect to (T, p, x) (reverse and forward mode)
 *
 * Every function returns an int status (RG_OK = 0); none aborts.  The text of
 * the last error on the calling thread is returned by rg_last_error().
 * A plan is not re-entrant: calls on one plan are serialised by an internal
 * mutex, and its device work is ordered across streams (work enqueued on a
 * stream other than the plan's previous one waits for that work first).
 * Distinct plans may be used concurrently from different threads.  A NULL
 * stream means the context's own stream; pass cudaStreamLegacy ((void*)1)
 * for the legacy default stream.
 */
#ifndef RADIS_GB300_H
#define RADIS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RG_ABI_VERSION 3

enum rg_status {
    RG_OK = 0,
    RG_ERR_ARG = 1,        /* invalid argument / size                         */
    RG_ERR_CUDA = 2,       /* a CUDA runtime call failed                      */
    RG_ERR_OOM = 3,        /* device or host allocation failed                */
    RG_ERR_UNSORTED = 4,   /* line positions v0 are not ascending             */
    RG_ERR_RANGE = 5,      /* grid too large for the kernels' limits          */
    RG_ERR_TIMEOUT = 6,    /* a bounded device wait gave up                   */
    RG_ERR_STATE = 7       /* object used after free / wrong context          */
};

typedef struct rg_ctx rg_ctx;
typedef struct rg_lines rg_lines;
typedef struct rg_plan rg_plan;

/* Line list, host arrays of length n (structure of arrays).
 * Mirrors the columns the reference uploads (gpu.py:190-203): v0 = wav,
 * da = Pshft, na = Tdpair, gamma_arr = (selbrd, airbrd), El, iso; the
 * intensity is given as S_ref = HITRAN line intensity at T_ref (the CPU path's
 * `int` column, base.py:2664) — convert an Einstein-A based S0 with
 * S_ref = S0 exp(-c2 El/Tref) (1 - exp(-c2 v0/Tref)) / Q(Tref). */
typedef struct {
    int64_t n;
    const double* v0;      /* line centre (cm-1), ascending, required        */
    const double* s_ref;   /* intensity at T_ref (cm-1/(molecule cm-2))      */
    const float* e_low;    /* lower-state energy (cm-1)                       */
    const float* g_air;    /* air-broadened HWHM at T_ref (cm-1/atm)          */
    const float* g_self;   /* self-broadened HWHM at T_ref (cm-1/atm)         */
    const float* n_air;    /* temperature exponent of the widths              */
    const float* delta;    /* pressure shift (cm-1/atm); NULL = no shift      */
    const uint8_t* iso;    /* isotope slot in [0, n_iso); NULL = all slot 0   */
} rg_line_arrays;

typedef struct {
    int n_iso;                 /* 1..16                                       */
    double molar_mass[16];     /* g/mol per isotope slot                      */
    double t_ref;              /* reference temperature (K), usually 296      */
} rg_isotopes;

/* Spectral grid v_k = vmin + k dv, k < n_v, and the LDM node policy:
 * dxG/dxL > 0  -> node spacing given, node count from the width envelope
 *                 (the reference's set_G_params/set_L_params, params.py:89-117);
 * n_G/n_L  > 1 -> node count given, spacing = envelope span / (n - 1).     */
typedef struct {
    double vmin;
    double dv;
    int64_t n_v;
    double dxG, dxL;
    int n_G, n_L;
    double folding_thresh;     /* <= 0 -> 1e-6 (factory.py:437)              */
    int64_t n_ft;              /* 0 -> smallest supported length >= 2 n_v     */
    /* fixed-point width of the scatter's accumulator: 0 = chosen from the
     * densest grid column (32 bits up to 8192 lines per column, else 64),
     * 32 or 64 = forced */
    int32_t accumulator;
    /* Gaussian node axis: 0 = from every line of the list (the reference's
     * rule over the lines it was given, radis/gpu/params.py:70-81); 1 = from
     * the lines that can reach the window (v0 within the window widened by the
     * largest pressure shift) -- what the reference computes when its factory
     * loads only the window's lines, and far fewer nodes for a narrow window
     * of a wide list */
    int32_t axes_window;
    /* FFT-stage layout (none changes what is computed, only how): 0 = the
     * one that transforms the fewest rows; 1 = every node row; 2 = merged
     * rows where the grid allows it (wide Gaussian nodes convolved in real
     * space and summed per wL node), else 1; 3 = skeleton rows where the
     * grid allows it (the node rows projected onto the few nodes whose
     * lineshape transforms span all the others within layout_tol), else 0 */
    int32_t layout;
    /* skeleton layout: largest error allowed in any node's normalised
     * lineshape transform (peak 1); <= 0 -> 1e-8 */
    double layout_tol;
} rg_plan_desc;

/* Gas conditions of one spectrum.  Pressure in bar (as the reference API);
 * widths and shift use atm = bar / 1.01325 like the CPU path. */
typedef struct {
    double T;                  /* K                                           */
    double p_bar;              /* bar                                         */
    double x;                  /* mole fraction of the absorber               */
    const double* q_ratio;     /* [n_iso] Q(T_ref)/Q(T); NULL -> all 1        */
} rg_conditions;

/* LDM axes chosen for one condition set (log of FWHM in cm-1). */
typedef struct {
    double log_wG_min, dxG;
    double log_wL_min, dxL;
    int n_G, n_L;
    int64_t n_ft;              /* FFT length                                   */
    int64_t n1, n2;            /* FFT factorisation n_ft = n1 * n2             */
} rg_grid;

typedef struct {
    rg_grid grid;
    double log_scale;          /* abscoeff = out * exp(log_scale)              */
    float stage_ms[6];         /* scatter, fft-col, fft-row+voigt, ifft-row,
                                  ifft-col, total (filled when timing != 0)    */
    int64_t lines_in_window;   /* lines whose k0 >= 0 and k0+1 < n_v          */
    /* layout of the FFT stage: rows transformed (node rows; with the merged
     * layout n_L merged rows + the narrow-Gaussian node rows; with the
     * skeleton layout the skeleton rows), how many of them are merged rows
     * and the half-width (points) of their widest Gaussian */
    int32_t fft_rows, merged_rows, merged_ext;
    float gauss_ms;            /* the real-space stage before the column FFT
                                  (merged layout: the Gaussian stage; skeleton
                                  layout: the projection), part of
                                  stage_ms[1] (timing = 1), else 0             */
    int32_t accum_bits;        /* the scatter's accumulator: 32 or 64 bits, or
                                  0 when it was chosen on the device (served
                                  and allocation-free spectra in auto mode)    */
    int32_t layout;            /* FFT-stage layout used: 1 node rows, 2 merged
                                  rows, 3 skeleton rows (fft_rows of them)
                                  projected in a pass of their own, 4 skeleton
                                  rows projected by the scatter as it writes
                                  each finished tile                           */
    float layout_err;          /* skeleton layout: the largest error of the
                                  decomposition over its frequency samples     */
} rg_spectrum_info;

int rg_abi_version(void);
const char* rg_last_error(void);

int rg_ctx_create(int device, rg_ctx** out);
int rg_ctx_destroy(rg_ctx* ctx);

int rg_lines_upload(rg_ctx* ctx, const rg_line_arrays* lines, const rg_isotopes* iso,
                    rg_lines** out);
int rg_lines_free(rg_lines* lines);
int rg_lines_count(const rg_lines* lines, int64_t* n);

int rg_plan_create(rg_lines* lines, const rg_plan_desc* desc, rg_plan** out);
int rg_plan_free(rg_plan* plan);

/* Host-only: the node axes and FFT factorisation the plan uses at `cond`. */
int rg_plan_grid(rg_plan* plan, const rg_conditions* cond, rg_grid* out);

/* Host-only, no device needed: the grid a plan over these host lines would
 * use at `cond` (the reference's init_*_params + set_*_params + get_griddims,
 * params.py:8-155, gpu.py:372-374).  Lets a scheduler size the LDM of a
 * request before any device memory is touched. */
int rg_grid_estimate(const rg_line_arrays* lines, const rg_isotopes* iso, const rg_plan_desc* desc,
                     const rg_conditions* cond, rg_grid* out);

/* Host-only, no device needed: the skeleton layout (rg_plan_desc.layout 3)
 * of a node grid at spacing dv: the n = n_G n_L nodes' folded, normalised
 * lineshape transforms (folding_thresh <= 0 -> 1e-6) written as combinations
 * of at most r_max of them within tol (<= 0 -> 1e-8) at every frequency
 * sample.  nodes[r], r < *n_rows: node index l n_L + m of skeleton row r;
 * coef[r n + node] (capacity r_max n): its coefficient for every node;
 * *err: the largest sampled error.  RG_ERR_RANGE when r_max rows fall short
 * of tol.  The same decomposition a plan makes for each spectrum. */
int rg_grid_skeleton(const rg_grid* grid, double dv, double folding_thresh, double tol, int32_t r_max,
                     int32_t* n_rows, int32_t* nodes, double* coef, double* err);

/* Host-only, no device needed: HITRAN-2004 160-character records -> columns.
 * `text`: the file's bytes (ASCII).  A record ends at "\n", "\r\n" or "\r";
 * records shorter than 67 characters are skipped; blank numeric fields read as
 * NaN; every value is the correctly rounded double of its decimal field.
 * rg_hitran_count: the number of records.  rg_hitran_parse: fills the non-NULL
 * columns of `out` (out->n must equal the count); RG_ERR_ARG names the line and
 * field of the first field that does not convert.  threads <= 0: one per host
 * core (at most one per MB of text). */
typedef struct {
    int64_t n;
    int32_t* id;      /* molecule number                                   */
    int32_t* iso;     /* isotopologue number: '1'-'9', '0' = 10, 'A' = 11 .. */
    double* v0;       /* wav (cm-1)                                        */
    double* s_ref;    /* int (cm-1/(molecule cm-2)) at 296 K               */
    double* a;        /* A (s-1)                                           */
    double* g_air;    /* airbrd (cm-1/atm)                                 */
    double* g_self;   /* selbrd (cm-1/atm)                                 */
    double* e_low;    /* El (cm-1)                                         */
    double* n_air;    /* Tdpair                                            */
    double* delta;    /* Pshft (cm-1/atm)                                  */
    double* gp;       /* upper-state degeneracy                            */
    double* gpp;      /* lower-state degeneracy                            */
} rg_hitran_columns;
int rg_hitran_count(const char* text, int64_t nbytes, int32_t threads, int64_t* n_records);
int rg_hitran_parse(const char* text, int64_t nbytes, int32_t threads, const rg_hitran_columns* out);

/* Enqueue one spectrum on `stream` (NULL = the context's stream).
 * `out_dev`: device array of n_v floats (abscoeff in cm-1 times
 * exp(-info.log_scale)).  timing = 0: asynchronous; 1: synchronises the stream
 * and fills info->stage_ms; 2: asynchronous, records per-stage CUDA events on
 * `stream` into a ring of 256 spectra read back by rg_plan_stage_times. */
int rg_synthesize(rg_plan* plan, const rg_conditions* cond, float* out_dev, void* stream,
                  int timing, rg_spectrum_info* info);

/* As rg_synthesize, plus the post-processing of eq_spectrum_gpu
 * (radis/lbl/factory.py:1284-1297) fused into the spectrum's last kernel:
 * out_dev holds 5 rows of n_v floats: abscoeff and absorbance
 * (x exp(-info.log_scale), path length in cm), then emissivity = -expm1(-A L),
 * transmittance = 1 - emissivity and radiance (mW/cm2/sr/nm, emissivity x
 * Planck at cond->T) in physical units.  Asynchronous on `stream`. */
int rg_synthesize_quantities(rg_plan* plan, const rg_conditions* cond, double path_length, float* out_dev,
                             void* stream, rg_spectrum_info* info);
/* The same into host memory (5 n_v floats; page-locked memory is written by
 * the last kernel itself, pageable memory gets a copy), blocking: the drop-in
 * form of gpuApp.iterate + the host post-processing of eq_spectrum_gpu
 * (factory.py:1247-1297).  timing = 1 fills info->stage_ms. */
int rg_synthesize_quantities_host(rg_plan* plan, const rg_conditions* cond, double path_length,
                                  float* out_host, void* stream, int timing, rg_spectrum_info* info);

/* Tabulated partition function Q(T) of isotopologue `iso` (0-based, < the
 * list's n_iso), copied from n points (T strictly increasing, Q > 0):
 *   RG_Q_LINEAR  np.interp, clamped outside the table
 *                (radis/levels/partfunc.py:1191-1192, PartFuncExoMol);
 *   RG_Q_CUBIC   interpolating cubic spline as scipy splrep/splev (n >= 4),
 *                refused beyond [0.95 Tmin, 1.05 Tmax] with RG_ERR_RANGE
 *                (radis/levels/partfunc_cdsd.py:84-117, PartFuncCO2_CDSDtab).
 * Once every isotopologue of the list has a table, rg_conditions.q_ratio =
 * NULL means Q(Tref)/Q(T) from the tables (instead of 1), and rg_backward /
 * rg_jvp with dlnq_dT = NULL take d ln(Q(Tref)/Q(T))/dT from them.  Not to be
 * called while spectra of the list are in flight. */
#define RG_Q_LINEAR 0
#define RG_Q_CUBIC 1
int rg_lines_set_partition(rg_lines* lines, int32_t iso, int64_t n, const double* T, const double* Q,
                           int32_t interp);

/* Host-only evaluation of a partition table (no device involved): Q(t) and
 * dQ/dT(t) (dq_dt may be NULL). */
int rg_partition_eval(int64_t n, const double* T, const double* Q, int32_t interp, double t, double* q,
                      double* dq_dt);

/* Instrument slit on the device (replaces the convolution of
 * radis/tools/slit.py:convolve_with_slit, :737, and remove_boundary,
 * :1063-1072; the reference's GPU path leaves it to the CPU, gpu.py:308-310):
 * out[i] = wstep * sum_j slit[j] in[i + (n_slit-1)/2 - j], zero outside
 * [0, n) -- the 'same' part of the full convolution.  RG_SLIT_VALID also sets
 * the first (la-1)/2 and last la/2 outputs to NaN, la = min(n, n_slit).
 * `slit_dev` is the slit sampled on the spectrum's step (n_slit floats);
 * `out_dev` must not overlap `in_dev`.  Asynchronous on `stream` (NULL: the
 * context's stream). */
#define RG_SLIT_SAME 0
#define RG_SLIT_VALID 1
int rg_slit_convolve(rg_ctx* ctx, const float* in_dev, int64_t n, const float* slit_dev, int32_t n_slit,
                     double wstep, int32_t mode, float* out_dev, void* stream);

/* Test hook of the failure path, no counterpart in the reference (whose
 * analogue is the bounded fence wait of
 * radis/gpu/vulkan/vulkan_compute_lib.py:898).  withhold != 0: the scatter's
 * producer issues no line copies in the plan's following spectra, so every
 * consumer's wait for its first chunk runs out; the kernels finish, the
 * spectrum call returns RG_ERR_TIMEOUT and the plan stays usable.
 * wait_cycles: bound of the scatter's producer/consumer handshake waits in SM
 * clock cycles (0 = the default, about one second; at most the default).  The
 * wait for copies already in flight always keeps the default bound. */
int rg_plan_test_scatter_stall(rg_plan* plan, int32_t withhold, int64_t wait_cycles);

/* Test hook, host-only, no counterpart in the reference: the node order in
 * which the scatter's flush projects a tile of n_nodes node rows on the tensor
 * cores (steps of 8 nodes: nodes[8 s + j]; real[8 s + j] = 0 where a node is
 * repeated with a zero coefficient).  *count = 8 x steps; RG_ERR_RANGE when
 * capacity is smaller. */
int rg_test_flush_order(int32_t n_nodes, int32_t* nodes, uint8_t* real, int32_t capacity, int32_t* count);

/* Sums (ms) of the stage times recorded with timing = 2 since the last call:
 * scatter, fft-col, fft-row+voigt, ifft-row, ifft-col, total; *count =
 * spectra recorded.  Synchronises the recording stream and empties the ring.
 * (The reference's per-command Vulkan timestamps, gpu.py:260-280, 360.) */
int rg_plan_stage_times(rg_plan* plan, double* sum_ms, int64_t* count);

/* The Gaussian-stage part (merged layout) of the fft-col sum that the last
 * rg_plan_stage_times call returned, in ms (0 without the merged layout). */
int rg_plan_stage_times_gauss(rg_plan* plan, double* gauss_sum_ms);

/* As rg_synthesize into `out_host` (n_v floats), and waits: the drop-in
 * `iterate()` form.  Page-locked host memory (cudaHostAlloc'd or registered)
 * is written by the spectrum's last kernel itself; pageable memory gets a copy
 * from device memory after it.  timing = 1 fills info->stage_ms (0 or 2 leave
 * it empty). */
int rg_synthesize_host(rg_plan* plan, const rg_conditions* cond, float* out_host,
                       void* stream, int timing, rg_spectrum_info* info);

/* Test hook: runs only the fused scale+scatter and copies the LDM tensor to
 * host as [n_nodes][n_v] floats (node = l*n_L + m), in units of
 * exp(info.log_scale) cm-1 . cm (times dv: no 1/dv yet).  capacity in floats. */
int rg_debug_ldm(rg_plan* plan, const rg_conditions* cond, float* ldm_host, int64_t capacity,
                 rg_spectrum_info* info);

/* Derivatives of the absorption coefficient with respect to the conditions
 * theta = (T [K], p_bar [bar], x), with the LDM node axes held at the values
 * the conditions give (the axes are a discretisation choice, not physics).
 * The reference has no derivatives; these differentiate the same FP32 LDM
 * synthesis that rg_synthesize computes.  dlnq_dT: per isotopologue
 * d ln(Q(Tref)/Q(T)) / dT (NULL = 0, i.e. cond->q_ratio held constant).
 *
 * rg_backward (reverse mode, the adjoint): grad[q] = sum_k g[k] dA_k/dtheta_q
 * for an upstream gradient g of n_v floats on the device (dL/dabscoeff in
 * cm).  Runs the transposed synthesis (FFT of g, per-node Voigt multiply and
 * inverse FFTs, gather at each line's LDM cells) and waits for it; the plan's
 * workspace is reused.  grad is in true units; info (nullable) receives the
 * grid, log_scale 0.
 *
 * rg_jvp (forward mode): out_dev[q n_v + k] = dA_k/dtheta_q x
 * exp(-info.log_scale), three rows of n_v floats on the device (asynchronous
 * on `stream`, like rg_synthesize). */
int rg_backward(rg_plan* plan, const rg_conditions* cond, const double* dlnq_dT,
                const float* grad_out_dev, double grad[3], void* stream, rg_spectrum_info* info);
int rg_jvp(rg_plan* plan, const rg_conditions* cond, const double* dlnq_dT, float* out_dev,
           void* stream, rg_spectrum_info* info);

/* Allocation-free spectrum.  No counterpart in the reference: it exists for
 * callers that may not allocate device memory when they ask for a spectrum
 * (a framework's caching allocator owns the device memory, a service forbids
 * cudaMalloc/cudaFree on its request path, a pre-sized job).  The line list
 * must already be resident (rg_lines_upload at setup) and `out_dev` holds
 * n_v floats (abscoeff x exp(-info.log_scale)).  All scratch of the spectrum
 * (line index, LDM, FFT workspace, twiddle tables, flags) is carved from one
 * static device array of 64 MiB that every GPU loading this library keeps
 * until the process exits; a spectrum that needs more returns RG_ERR_RANGE.
 * Calls no cudaMalloc or cudaFree.  The first call on a device resolves the
 * array's device address, so make it before any stream capture.  The first
 * launch of a kernel variant in a process can make the CUDA driver reserve
 * device memory of its own (lazy module loading; local memory of a kernel
 * that spills): to keep that off a request path too, make one call per
 * spectrum shape at setup.  The array
 * belongs to this process and device (each process that loads the library
 * has its own); all calls in the process share it and a lock serialises
 * them.  Blocking: a call returns only after all the work it enqueued on
 * `stream` has finished, on success and on error alike, so two calls never
 * overlap on the GPU through the library.  The array keeps the last call's
 * contents; a caller who still reads `out_dev` on another stream while the
 * next call writes it must order the two itself. */
int rg_synthesize_static(rg_lines* lines, const rg_plan_desc* grid, const rg_conditions* cond,
                         float* out_dev, void* stream, rg_spectrum_info* info);

/* ---------------------------------------------------------------------------
 * Serving: continuous batching of spectrum requests over resident line lists.
 * No reference counterpart (the reference runs one blocking gpuApp.iterate at a
 * time, radis/gpu/gpu.py:302-370); this is the request-level equivalent of
 * SpectrumFactory.eq_spectrum_gpu + Spectrum.recalc_gpu for many clients.
 * A worker thread admits queued requests (FIFO) into `slots` CUDA streams as
 * slots and device memory (LDM + FFT workspace, within `mem_budget` bytes)
 * free up; admitted requests run concurrently on the device.  A request
 * buffer that is page-locked (cudaHostAlloc / cudaHostRegister, or a pinned
 * torch tensor) is written by the spectrum's last kernel directly; any other
 * host buffer gets the result through its slot's pinned staging buffer (an
 * asynchronous device -> staging copy, then a host copy once the request is
 * complete).
 * ------------------------------------------------------------------------- */
typedef struct rg_server rg_server;

typedef struct {
    rg_lines* lines;           /* resident line list                            */
    rg_plan_desc grid;         /* spectral grid + LDM node policy               */
    rg_conditions cond;        /* q_ratio is copied at submission               */
    float* out_host;           /* n_v floats: abscoeff x exp(-info.log_scale);
                                * page-locked memory is written directly       */
} rg_request;

typedef struct {
    int64_t submitted, completed, failed, in_flight, queued;
    int64_t device_bytes;      /* workspace currently held by the slots         */
    /* worker thread host time so far (ms): sizing requests (grid, memory),
     * launching them, copying results to the callers' buffers */
    double host_need_ms, host_launch_ms, host_copy_ms;
} rg_server_stats;

int rg_server_create(rg_ctx* ctx, int slots, int64_t mem_budget, rg_server** out);
/* Queue a request; returns at once with a ticket (>= 1). */
int rg_server_submit(rg_server* srv, const rg_request* req, int64_t* ticket);
/* Wait for a ticket (timeout_ms < 0: no limit); fills info and the request's
 * timestamps (seconds on the server's clock: submitted, started, finished).
 * Returns the request's own status (RG_ERR_TIMEOUT if the wait expired). */
int rg_server_wait(rg_server* srv, int64_t ticket, double timeout_ms, rg_spectrum_info* info,
                   double* t_submit, double* t_start, double* t_done);
int rg_server_stats_get(rg_server* srv, rg_server_stats* st);
/* Finish the requests in flight and queued, then release everything. */
int rg_server_destroy(rg_server* srv);

#ifdef __cplusplus
}
#endif
#endif /* RADIS_GB300_H */
