/*
 * gwgpu.h -- plain C ABI of the GB300 GWRBasic engine (libgwgpu.so).
 *
 * Two layers, both over plain pointers and sizes:
 *
 *  1. gwgpu_gwr_*  -- the gwm::GWRBasic surface (include/gwmodelpp/GWRBasic.h:29
 *     in libgwmodel) as a C handle: the same setters, fit() and getters.
 *     This is what a non-C++ caller binds (ctypes, cgo, JNI, N-API).
 *  2. gwgpu_engine_* -- the engine primitives behind it: one criterion
 *     evaluation, the final fit, maxDistance, adaptive thresholds.  They
 *     replace bandwidthSizeCriterion{AIC,CV}Cuda (GWRBasic.cpp:709-836),
 *     fitCuda (GWRBasic.cpp:585-663), CRSDistance::maxDistance
 *     (CRSDistance.cpp:133-143) and BandwidthWeight::weight's adaptive
 *     threshold (BandwidthWeight.cpp:40-53).
 *
 * The binary drop-in for libgwmodelcuda (IGWRBasicGpuTask and its three
 * extern "C" factories) is declared in IGWRBasicGpuTask.h.
 *
 * Matrices are column-major doubles (Armadillo layout: (i, j) at i + j*rows).
 * Every function returns GWGPU_OK or an error code; gwgpu_last_error() gives
 * the message of the calling thread's last failure.  No function resets the
 * device.
 */
#ifndef GWGPU_H
#define GWGPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GWGPU_OK 0
#define GWGPU_ERR_INVALID 1     /* bad argument or state */
#define GWGPU_ERR_CUDA 2        /* CUDA runtime error (no device reset is done) */
#define GWGPU_ERR_NOT_SPD 3     /* a local X^T W X is not positive definite */
#define GWGPU_ERR_RUNTIME 4     /* other std::runtime_error (e.g. "Invalid initial values.") */
#define GWGPU_ERR_RANGE 5       /* adaptive bandwidth below one neighbour */

/* BandwidthWeight::KernelFunctionType (BandwidthWeight.h:46-53) */
#define GWGPU_GAUSSIAN 0
#define GWGPU_EXPONENTIAL 1
#define GWGPU_BISQUARE 2
#define GWGPU_TRICUBE 3
#define GWGPU_BOXCAR 4

/* GWRBasic::BandwidthSelectionCriterionType (GWRBasic.h:41-45) */
#define GWGPU_AIC 0
#define GWGPU_CV 1

/* ParallelType (IParallelizable.h:15-20); every value runs on the GPU */
#define GWGPU_SERIAL 1
#define GWGPU_OPENMP 2
#define GWGPU_CUDA 4

/* numeric form */
#define GWGPU_FP64 0
#define GWGPU_MIXED 1

/* Status (Status.h:10-14) */
#define GWGPU_STATUS_SUCCESS 0
#define GWGPU_STATUS_TERMINATED 1

int gwgpu_version(void);
const char* gwgpu_last_error(void);
int gwgpu_device_count(int* count);

/* ---------------------------------------------------------------- telegram */

/* ITelegram (Logger.h:31-83) as C callbacks; any member may be NULL. */
typedef struct gwgpu_telegram {
    void* user;
    void (*print)(void* user, const char* message, int level, const char* fun_name, const char* file_name);
    void (*progress)(void* user, size_t current, size_t total, const char* fun_name, const char* file_name);
    void (*progress_percent)(void* user, double percent, const char* fun_name, const char* file_name);
    int (*stop)(void* user);
} gwgpu_telegram;

/* ------------------------------------------------------- GWRBasic surface */

typedef struct gwgpu_gwr gwgpu_gwr;

int gwgpu_gwr_create(gwgpu_gwr** out);
void gwgpu_gwr_destroy(gwgpu_gwr* g);

int gwgpu_gwr_set_coords(gwgpu_gwr* g, int n, const double* coords /* n x 2 */);
int gwgpu_gwr_set_dependent_variable(gwgpu_gwr* g, int n, const double* y);
int gwgpu_gwr_set_independent_variables(gwgpu_gwr* g, int n, int p, const double* x /* n x p */);
/* SpatialWeight(BandwidthWeight(bandwidth, adaptive, kernel), CRSDistance(geographic)) */
int gwgpu_gwr_set_spatial_weight(gwgpu_gwr* g, double bandwidth, int adaptive, int kernel, int geographic);
int gwgpu_gwr_set_is_autoselect_bandwidth(gwgpu_gwr* g, int on);
int gwgpu_gwr_set_bandwidth_selection_criterion(gwgpu_gwr* g, int criterion);
int gwgpu_gwr_set_golden_upper_bounds(gwgpu_gwr* g, double value);
int gwgpu_gwr_set_golden_lower_bounds(gwgpu_gwr* g, double value);
int gwgpu_gwr_set_has_hat_matrix(gwgpu_gwr* g, int on);
int gwgpu_gwr_set_has_intercept(gwgpu_gwr* g, int on);
int gwgpu_gwr_set_is_autoselect_indep_vars(gwgpu_gwr* g, int on);
int gwgpu_gwr_set_indep_var_selection_threshold(gwgpu_gwr* g, double threshold);
int gwgpu_gwr_set_parallel_type(gwgpu_gwr* g, int type);
int gwgpu_gwr_set_omp_thread_num(gwgpu_gwr* g, int threads);
int gwgpu_gwr_set_gpu_id(gwgpu_gwr* g, int gpu);
int gwgpu_gwr_set_group_size(gwgpu_gwr* g, size_t size);
int gwgpu_gwr_set_precision(gwgpu_gwr* g, int precision);
/* The telegram struct is copied; callbacks must outlive the handle. */
int gwgpu_gwr_set_telegram(gwgpu_gwr* g, const gwgpu_telegram* t);

/* GWRBasic::fit().  GWGPU_OK also when cancelled: check gwgpu_gwr_status. */
int gwgpu_gwr_fit(gwgpu_gwr* g);
/* GWRBasic::predict: coefficients at nr locations (nr x 2 column-major) at the
   spatial weight's bandwidth; betas: nr x p column-major (may be null; the
   getters then return the nr x p matrix). */
int gwgpu_gwr_predict(gwgpu_gwr* g, int nr, const double* locations, double* betas);
int gwgpu_gwr_status(gwgpu_gwr* g);

/* Shapes after fit (p shrinks when variables were selected). */
int gwgpu_gwr_shape(gwgpu_gwr* g, int* n, int* p, int* s_rows);
int gwgpu_gwr_betas(gwgpu_gwr* g, double* out /* n x p */);
int gwgpu_gwr_betas_se(gwgpu_gwr* g, double* out /* n x p */);
int gwgpu_gwr_shat(gwgpu_gwr* g, double* out /* 2: tr(S), tr(S^T S) */);
int gwgpu_gwr_qdiag(gwgpu_gwr* g, double* out /* n */);
int gwgpu_gwr_s(gwgpu_gwr* g, double* out /* s_rows x n */);
/* RSS, AIC, AICc, ENP, EDF, RSquare, RSquareAdjust */
int gwgpu_gwr_diagnostic(gwgpu_gwr* g, double* out /* 7 */);
int gwgpu_gwr_bandwidth(gwgpu_gwr* g, double* bandwidth);
/* bandwidthSelectionCriterionList(): count first (out may be NULL), sorted by bandwidth */
int gwgpu_gwr_bandwidth_criterion_list(gwgpu_gwr* g, int* count, double* bw, double* value);
/* selectedVariables() */
int gwgpu_gwr_selected_vars(gwgpu_gwr* g, int* count, int* vars);
/* indepVarsSelectionCriterionList(): entry i has lens[i] variables starting at vars[offset]. */
int gwgpu_gwr_var_criterion_list(gwgpu_gwr* g, int* count, int* total_vars, int* lens, int* vars, double* value);

/* ------------------------------------------------------------ CSV input */

/* A comma-separated file with a header row of column names (quoted or not) and
   numeric rows, as the reference's callers load with Armadillo's csv_name
   (test/data/londonhp100.cpp:6-26).  Rows are parsed on all host threads;
   blank lines are skipped; an empty or non-numeric cell fails with its line
   number in gwgpu_last_error(). */
typedef struct gwgpu_table gwgpu_table;
int gwgpu_csv_read(const char* path, gwgpu_table** out);
int gwgpu_table_shape(const gwgpu_table* t, int* rows, int* cols);
/* Name of column col (NULL when out of range). */
const char* gwgpu_table_column_name(const gwgpu_table* t, int col);
/* The named columns into out, rows x ncol column-major: the layout of the
   coords / X / y setters. */
int gwgpu_table_columns(const gwgpu_table* t, int ncol, const char* const* names, double* out);
void gwgpu_table_destroy(gwgpu_table* t);

/* -------------------------------------------------- GWRMultiscale surface */

/* gwm::GWRMultiscale (include/gwmodelpp/GWRMultiscale.h:35-1040): multiscale
   GWR by back-fitting.  Per-variable arrays have p entries, p = the columns of
   X given to gwgpu_mgwr_set_independent_variables (set X first). */
typedef struct gwgpu_mgwr gwgpu_mgwr;

/* BandwidthInitilizeType, BandwidthSelectionCriterionType, BackFittingCriterionType */
#define GWGPU_MGWR_INIT_NULL 0
#define GWGPU_MGWR_INIT_INITIAL 1
#define GWGPU_MGWR_INIT_SPECIFIED 2
#define GWGPU_MGWR_CV 0
#define GWGPU_MGWR_AIC 1
#define GWGPU_MGWR_CVR 0
#define GWGPU_MGWR_DCVR 1

int gwgpu_mgwr_create(gwgpu_mgwr** out);
void gwgpu_mgwr_destroy(gwgpu_mgwr* g);
int gwgpu_mgwr_set_coords(gwgpu_mgwr* g, int n, const double* coords /* n x 2 */);
int gwgpu_mgwr_set_dependent_variable(gwgpu_mgwr* g, int n, const double* y);
int gwgpu_mgwr_set_independent_variables(gwgpu_mgwr* g, int n, int p, const double* x /* n x p */);
/* setSpatialWeights: variable k gets BandwidthWeight(bandwidths[k], adaptive[k],
   kernels[k]); every variable shares CRSDistance(geographic). */
int gwgpu_mgwr_set_spatial_weights(gwgpu_mgwr* g, int p, const double* bandwidths, const int* adaptive,
                                   const int* kernels, int geographic);
int gwgpu_mgwr_set_bandwidth_initilize(gwgpu_mgwr* g, int p, const int* types);
int gwgpu_mgwr_set_bandwidth_selection_approach(gwgpu_mgwr* g, int p, const int* approaches);
int gwgpu_mgwr_set_preditor_centered(gwgpu_mgwr* g, int p, const int* centered);
int gwgpu_mgwr_set_bandwidth_select_threshold(gwgpu_mgwr* g, int p, const double* thresholds);
int gwgpu_mgwr_set_bandwidth_select_retry_times(gwgpu_mgwr* g, int times);
int gwgpu_mgwr_set_max_iteration(gwgpu_mgwr* g, int iterations);
int gwgpu_mgwr_set_criterion_type(gwgpu_mgwr* g, int type);
int gwgpu_mgwr_set_criterion_threshold(gwgpu_mgwr* g, double threshold);
int gwgpu_mgwr_set_adaptive_lower(gwgpu_mgwr* g, int lower);
int gwgpu_mgwr_set_golden_upper_bounds(gwgpu_mgwr* g, double value);
int gwgpu_mgwr_set_golden_lower_bounds(gwgpu_mgwr* g, double value);
int gwgpu_mgwr_set_has_hat_matrix(gwgpu_mgwr* g, int on);
int gwgpu_mgwr_set_has_intercept(gwgpu_mgwr* g, int on);
int gwgpu_mgwr_set_parallel_type(gwgpu_mgwr* g, int type);
int gwgpu_mgwr_set_gpu_id(gwgpu_mgwr* g, int gpu);
/* GWGPU_FP64 (default) or GWGPU_MIXED for the bandwidth searches; fits and the hat matrix stay FP64. */
int gwgpu_mgwr_set_precision(gwgpu_mgwr* g, int precision);
int gwgpu_mgwr_set_telegram(gwgpu_mgwr* g, const gwgpu_telegram* t);
/* GWRMultiscale::fit().  GWGPU_OK also when cancelled: check gwgpu_mgwr_status. */
int gwgpu_mgwr_fit(gwgpu_mgwr* g);
int gwgpu_mgwr_status(gwgpu_mgwr* g);
int gwgpu_mgwr_betas(gwgpu_mgwr* g, double* out /* n x p */);
/* diag(C C^T) of the initial fit and betas / betasSE (hat matrix only; zeros otherwise) */
int gwgpu_mgwr_betas_se(gwgpu_mgwr* g, double* out /* n x p */);
int gwgpu_mgwr_betas_tv(gwgpu_mgwr* g, double* out /* n x p */);
/* bandwidths of spatialWeights() after fit */
int gwgpu_mgwr_bandwidths(gwgpu_mgwr* g, double* out /* p */);
/* RSS, AIC (0: the reference leaves it unset), AICc, ENP, EDF, RSquare, RSquareAdjust */
int gwgpu_mgwr_diagnostic(gwgpu_mgwr* g, double* out /* 7 */);
/* the initial all-variable bandwidth and the back-fitting iterations run */
int gwgpu_mgwr_info(gwgpu_mgwr* g, double* initial_bandwidth, int* iterations);
/* Work of the last fit: criterion evaluations, fits, hat updates, this library's kernel
   launches, and host seconds in the searches, the fits and the hat updates (any may be NULL). */
int gwgpu_mgwr_counters(gwgpu_mgwr* g, long long* criterion_evals, long long* fits, long long* hat_updates,
                        long long* kernel_launches, double* seconds /* 3 */);

/* --------------------------------------------------------- engine layer */

typedef struct gwgpu_engine gwgpu_engine;

typedef struct gwgpu_stats {
    int criterion_evals;
    int contract_launches;
    double contract_ms;
    double contract_flops;
    double contract_bytes;
    int select_launches;
    double select_ms;
    long long kernel_launches;  /* every kernel the engine launched */
    long long contract_tiles;   /* 128 x 32 weight tiles the mixed contraction processed */
    /* mixed contraction, clock64 cycles summed over CTAs: producer waits for a
       weight stage, for point records, weight work, accumulator drains; control
       waits for weights, for Z / accumulator, MMA issue; producer tile loop;
       then the largest tile loop of one CTA, prologue, kernel start to end
       (summed), and the largest tile count of one CTA */
    double contract_phase_cycles[12];
    int d2c_fills;              /* distance cache fills (mixed geographic contraction) */
    double d2c_fill_ms;         /* their duration */
} gwgpu_stats;

int gwgpu_engine_create(int device, gwgpu_engine** out);
void gwgpu_engine_destroy(gwgpu_engine* e);
int gwgpu_engine_set_data(gwgpu_engine* e, int n, int p, const double* x, const double* y, const double* coords,
                          int geographic);
int gwgpu_engine_set_precision(gwgpu_engine* e, int precision);
/* Mixed path: 32-point data tiles summed in FP32 on the tensor core before
   each double-float drain (default 64, at least 2). */
int gwgpu_engine_set_flush_tiles(gwgpu_engine* e, int tiles);
/* Mixed path: polls of each pipeline wait of the tensor-core contraction before
   it times out (0 = the default, about two seconds).  A timeout makes the
   kernel wait for its own MMAs and copies, free its tensor memory and report;
   the call then fails with GWGPU_ERR_CUDA and the engine stays usable.  Small
   values are for testing that path (no counterpart in libgwmodel). */
int gwgpu_engine_set_tc_wait_limit(gwgpu_engine* e, unsigned polls);
/* Mixed path: FP64 refinement steps of the final fit (default 1), and
   whether each AICc criterion of the search is refined too (default 0). */
int gwgpu_engine_set_refinement(gwgpu_engine* e, int steps, int refine_search);
/* One bandwidth criterion (DBL_MAX when a local system is not SPD). */
int gwgpu_engine_criterion(gwgpu_engine* e, double bandwidth, int adaptive, int kernel, int criterion,
                           double* value);
/* AICc with every weight one on the given columns (variable selection). */
int gwgpu_engine_global_criterion(gwgpu_engine* e, int ncols, const int* cols, double* value);
/* fitCuda outputs before GWRBasic::fit's sigma scaling of betasSE. */
int gwgpu_engine_fit(gwgpu_engine* e, double bandwidth, int adaptive, int kernel, int store_s, double* betas,
                     double* betas_se, double* shat, double* qdiag, double* s);
int gwgpu_engine_max_distance(gwgpu_engine* e, double* out);
/* BandwidthSelector::optimize (BandwidthSelector.cpp:6-81) on the resident
 * data: writes the chosen bandwidth and up to cap (bandwidth, criterion)
 * pairs sorted by bandwidth; *count receives their number. */
int gwgpu_engine_golden(gwgpu_engine* e, int adaptive, int kernel, int criterion, double lower, double upper,
                        double* bandwidth, int* count, double* list_bw, double* list_value, int cap);
/* Drop the dataset's cached order statistics, distance histograms and
   distance cache contents. */
int gwgpu_engine_clear_cache(gwgpu_engine* e);
/* Distance cache of the mixed geographic contraction (no counterpart in
 * libgwmodel, whose CRSDistance::distance recomputes a focus row's distances
 * at every evaluation, CRSDistance.cpp:122-131): the FP32 squared distance of
 * every pair, filled once per dataset with the arithmetic of the weight
 * producer, so cached and uncached results are bit-identical.  It takes
 * n^2 x 4 bytes (160 GB at n = 200,000); one buffer per device is shared by
 * all engines on it, owned by the engine that used it last and freed with
 * that engine or by _release_.  limit_bytes < 0: automatic (the default; used
 * when max(16 GB, 1/8 of the device) stays free beside it), 0: never, > 0: at
 * most that many bytes. */
int gwgpu_engine_set_distance_cache(gwgpu_engine* e, long long limit_bytes);
int gwgpu_engine_release_distance_cache(gwgpu_engine* e);
/* *active = 1 when the device's distance cache holds this engine's dataset. */
int gwgpu_engine_distance_cache_active(gwgpu_engine* e, int* active);
/* Coefficients at nr prediction locations (nr x 2 column-major) from the
   resident data at the given bandwidth (FP64, exact thresholds); betas nr x p. */
int gwgpu_engine_predict(gwgpu_engine* e, int nr, const double* locations, double bandwidth, int adaptive,
                         int kernel, double* betas);
/* CUDA events on the engine's stream, slots 0..7: device-side timing. */
int gwgpu_engine_event_record(gwgpu_engine* e, int slot);
int gwgpu_engine_event_elapsed(gwgpu_engine* e, int first, int second, float* ms);
int gwgpu_engine_thresholds(gwgpu_engine* e, double bandwidth, int adaptive, double* out /* n */);
/* on: 0 off, 1 event timings and counters, 2 also the mixed contraction's
   clock64 phase counters (contract_phase_cycles; instrumented kernels). */
int gwgpu_engine_enable_stats(gwgpu_engine* e, int on);
int gwgpu_engine_get_stats(gwgpu_engine* e, gwgpu_stats* out);
int gwgpu_engine_reset_stats(gwgpu_engine* e);
/* Tensor-core self-test: D[128 x N] = A[128 x 32] B[N x 32]^T through the same
 * tcgen05 descriptors, swizzled layouts and TMEM reads as the mixed-precision
 * contraction (TF32 inputs, FP32 output; N a multiple of 16 up to 256). */
int gwgpu_engine_tc_selftest(gwgpu_engine* e, int N, const float* A, const float* B, float* D);

/* ------------------------------------------------ no-allocation entry point */

/* Criterion of one bandwidth from normal equations the caller already holds
 * on the device, without allocating any device memory.  No counterpart in
 * libgwmodel.  For callers that cannot let a library call cudaMalloc: code
 * that owns all device memory through its own pool, or must not allocate
 * after start-up (cudaMalloc and cudaFree synchronise the whole device).
 *
 * Inputs (device pointers): G, n x (p(p+1)/2 + p) row-major -- per location
 * the upper triangle of X^T W_i X packed by rows, then X^T W_i y (for CV with
 * w_ii = 0); X, n x p row-major; y, n; thr, per-row bandwidth or NULL for the
 * fixed `bandwidth` (it only gives w_ii through `kernel`).  Outputs (device):
 * beta, n x p row-major; sums[5] = tr(S), RSS (or CV sum), 0, failed local
 * solves, and the criterion (AICc or CV; DBL_MAX on failure).  Runs
 * asynchronously on `stream` (a cudaStream_t, NULL for the default stream).
 *
 * Limits: n in [3, 65536], p in [1, 32].  Scratch is a fixed ~1.2 MB
 * __device__ array shared by all calls on a device: calls that overlap on
 * the GPU race, so serialise them.  The first call on a device resolves the
 * array's address (cudaGetSymbolAddress); make it before any stream capture. */
int gwgpu_criterion_noalloc(int n, int p, int criterion, int kernel, double bandwidth, const double* G,
                            const double* X, const double* y, const double* thr, double* beta, double* sums,
                            void* stream);

/* ------------------------------------------------------- serving loop
 *
 * A request loop on one GPU: fits with a given bandwidth and golden-section
 * bandwidth searches (then the fit) of independent datasets, submitted from
 * any thread as they arrive.  Each of `slots` worker slots keeps one engine
 * (its device buffers grow and are reused, so steady-state serving calls
 * neither cudaMalloc nor cudaFree) and its own stream; requests run as soon
 * as a slot is free and the HBM budget admits them, so their kernels overlap
 * on the device.  Admission is first come, first served: the oldest waiting
 * request is admitted when the memory held by every slot, with the chosen
 * slot grown to the request's estimate, stays within the budget; idle slots
 * give their memory back when that is what blocks it.  A request whose
 * estimate alone exceeds the budget is rejected at submit.
 */
typedef struct gwgpu_server gwgpu_server;

#define GWGPU_REQ_FIT 0    /* fit at the given bandwidth */
#define GWGPU_REQ_SEARCH 1 /* golden-section bandwidth search, then the fit */
#define GWGPU_ERR_TIMEOUT 6 /* gwgpu_server_wait: not finished within the timeout */
#define GWGPU_ERR_REJECTED 7 /* the request does not fit the HBM budget */

typedef struct gwgpu_request {
    int n, p;              /* data points; columns of X (intercept supplied by the caller) */
    const double* coords;  /* n x 2 column-major (u, v) or (lon, lat); copied at submit */
    const double* x;       /* n x p column-major; copied at submit */
    const double* y;       /* n; copied at submit */
    int geographic;        /* 1: great-circle distances */
    int kind;              /* GWGPU_REQ_FIT or GWGPU_REQ_SEARCH */
    int adaptive;          /* bandwidth in neighbours (1) or distance (0) */
    int kernel;            /* GWGPU_GAUSSIAN ... GWGPU_BOXCAR */
    int criterion;         /* search criterion: GWGPU_AIC or GWGPU_CV */
    double bandwidth;      /* GWGPU_REQ_FIT only */
    int precision;         /* GWGPU_FP64 or GWGPU_MIXED */
} gwgpu_request;

typedef struct gwgpu_result {
    int status;            /* GWGPU_OK or the request's error code */
    int slot;              /* worker slot that ran it */
    int evaluations;       /* criterion evaluations of the search (0 for a fit) */
    double bandwidth;      /* given or selected */
    double aicc;           /* GWRBase::AICc of the final fit (GWRBase.h:90-94) */
    double rss;            /* residual sum of squares of the final fit */
    double shat[2];        /* tr(S), tr(S^T S) */
    double submit_ms, start_ms, end_ms;  /* server clock, from its creation */
    char error[160];       /* message when status != GWGPU_OK */
} gwgpu_result;

typedef struct gwgpu_server_stats {
    long long submitted, completed, failed, rejected, running, queued;
    double p50_ms, p99_ms, mean_ms;  /* latency (end - submit) of completed requests */
    double first_start_ms, last_end_ms;
    double local_fits;               /* sum over completed requests of n x (evaluations + 1) */
    double reserved_bytes;           /* memory held by the slots now */
    double peak_reserved_bytes;
    int max_concurrent;              /* most requests running at once */
} gwgpu_server_stats;

int gwgpu_server_create(int device, double hbm_budget_bytes, int slots, gwgpu_server** out);
/* Waits for every admitted request, then stops the workers. */
int gwgpu_server_destroy(gwgpu_server* s);
/* betas_out: n x p column-major output filled when the request finishes (may be null). */
int gwgpu_server_submit(gwgpu_server* s, const gwgpu_request* r, double* betas_out, long long* id);
/* Blocks until the request finished (timeout_ms < 0: no limit); the record is then forgotten. */
int gwgpu_server_wait(gwgpu_server* s, long long id, double timeout_ms, gwgpu_result* out);
int gwgpu_server_poll(gwgpu_server* s, long long id, int* done);
int gwgpu_server_get_stats(gwgpu_server* s, gwgpu_server_stats* out);
/* The estimate this server admits the request with (bytes; host only). */
double gwgpu_server_estimate(gwgpu_server* s, const gwgpu_request* r);
/* Upper bound of one slot's device memory for a request of this shape, with
   the histogram cache counted (host only). */
double gwgpu_estimate_bytes(int n, int p, int geographic, int precision, int adaptive);
/* The admission rule (host only): the slot an idle worker set would give the
   request, or -1 to wait.  reserved: bytes each slot holds; busy: 1 when running. */
int gwgpu_admit_slot(double budget, int slots, const double* reserved, const int* busy, double estimate);

/* ------------------------------------------------------- batched problems
 *
 * Many independent GWR problems (uneven n and p) and many bandwidth
 * candidates per problem, evaluated together: every phase (threshold
 * selects, tensor-core or FP64 contraction, per-location solves, per-pair
 * reductions) is one launch over all (problem, candidate) pairs, and the
 * sequence is captured once into a CUDA graph and replayed.  The schedule
 * (FP32 chunk of the contraction, order of its work table, rows per solve
 * block, select width) is picked by gwgpu_batch_autotune on the batch itself.
 */
typedef struct gwgpu_batch gwgpu_batch;

typedef struct gwgpu_batch_info {
    int problems, segments;     /* segments = (problem, candidate) pairs */
    int flush_tiles, order, solve_rows, select_ctas;  /* schedule in use */
    int tuned;                  /* 1 after gwgpu_batch_autotune */
    double tuned_ms, last_ms;   /* best tuning time; wall time of the last evaluation */
    int graph;                  /* 1 when the evaluation is a captured graph */
    int launches_per_evaluate;  /* kernel launches in one evaluation */
    int contract_ctas;          /* CTAs of the batched contraction */
    double rows_total;          /* sum over segments of n */
} gwgpu_batch_info;

int gwgpu_batch_create(int device, gwgpu_batch** out);
int gwgpu_batch_destroy(gwgpu_batch* b);
/* Copies every problem: x[q] n[q] x p[q] column-major, y[q], coords[q] n[q] x 2 column-major. */
int gwgpu_batch_set_problems(gwgpu_batch* b, int count, const int* n, const int* p, const double* const* x,
                             const double* const* y, const double* const* coords, const int* geographic,
                             int precision);
/* counts[q] candidates bandwidths[q][0..counts[q]) for problem q (adaptive: whole neighbour counts <= n). */
int gwgpu_batch_set_candidates(gwgpu_batch* b, const int* counts, const double* const* bandwidths, int adaptive,
                               int kernel, int criterion);
/* values: the AICc (or CV) of every pair, problem-major (DBL_MAX where a local system is not SPD). */
int gwgpu_batch_evaluate(gwgpu_batch* b, int use_graph, double* values);
int gwgpu_batch_autotune(gwgpu_batch* b, int repeats);
int gwgpu_batch_set_tuning(gwgpu_batch* b, int flush_tiles, int order, int solve_rows, int select_ctas);
int gwgpu_batch_get_info(gwgpu_batch* b, gwgpu_batch_info* out);

#ifdef __cplusplus
}
#endif
#endif /* GWGPU_H */
