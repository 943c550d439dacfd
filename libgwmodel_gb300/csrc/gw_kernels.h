// gw_kernels.h -- host-side launch wrappers of the GWR kernels.
#pragma once

#include <cstddef>
#include <cuda_runtime.h>

#include "gw_common.cuh"

namespace gwgpu {

// Raises (never lowers) the dynamic shared memory limit of kernel fn on the
// current device to `bytes`; safe to call from concurrent host threads.
cudaError_t raise_smem_limit(const void* fn, size_t bytes);

// Solve modes of launch_solve.
enum SolveMode { kSolveAIC = 0, kSolveCV = 1, kSolveFit = 2, kSolveRefine = 3, kSolvePredict = 4 };

// Per-row k-th smallest distance (1-based rank), k_select.cu.
struct SelectArgs {
    int n, ntiles;                 // points, 32-point tiles
    DevPoints P;                   // FP64 coordinates (exact formula)
    const float4* pts;             // FP32 hi/lo proxy data (as the mixed path)
    const float4* tb;              // per tile: planar box (ulo, uhi, vlo, vhi) or cap (cx, cy, cz, rho)
    const float4* stb;             // per super-tile of 32 tiles (1024 points): the same bound, or null
    unsigned* hist_cache;          // n x 4096 proxy histograms of whole rows, or null
    int cache_valid;               // 1: hist_cache holds every row's histogram
    // n x 64: cumulative counts of hist_cache at the end of each 64-bin segment
    // (written by the histogram pass; used with cache_valid), or null
    unsigned* hist_coarse;
    unsigned rank;
    double dlo, dhi;               // expected range of positive distances (first histogram only)
    double eps, delta;             // proxy band: d in [p (1 - eps) - delta, p (1 + eps) + delta]
    double* out;
    int* err;                      // 2: a row's select failed (value left NaN)
    // Focus rows when they are not the data points (prediction): FP64
    // coordinates and FP32 records of F.n focus points.  Null F.u: the data.
    DevPoints F;
    const float4* fpts;
    // Geographic data rows only, or null: the distance cache that histogram pass
    // filled; the selects read their proxy values from it instead of recomputing them.
    const float* d2c;
};
// exact: FP64 order statistics (bit-exact); otherwise the FP32 proxy's.
cudaError_t launch_select(const SelectArgs& a, bool geographic, bool exact, int num_sms, cudaStream_t stream);
size_t select_smem_bytes();
// Fills hist_cache with every row's whole-row proxy histogram (the cache a
// first select pass would store); the selects after it run with cache_valid.
cudaError_t launch_select_hist(const SelectArgs& a, bool geographic, int num_sms, cudaStream_t stream);
// The same histograms of geographic data rows read back from the filled
// distance cache a.d2c instead of recomputing the distances.
cudaError_t launch_select_hist_cached(const SelectArgs& a, int num_sms, cudaStream_t stream);
// Batched forms over many datasets and ranks in one launch each (device
// arrays of per-segment arguments; segment s owns the flattened items
// [start[s], start[s + 1])): whole-row histograms (items are groups of 8
// rows), selects (items are rows) and the FP32 copy of the thresholds.
cudaError_t launch_select_hist_batch(const SelectArgs* segs, const long long* start, int nseg, bool geographic,
                                     int num_sms, cudaStream_t stream);
cudaError_t launch_select_batch(const SelectArgs* segs, const long long* start, int nseg, bool geographic, bool exact,
                                int num_sms, cudaStream_t stream);
cudaError_t launch_to_float_batch(const double* const* in, float* const* out, const long long* start, int nseg,
                                  int num_sms, cudaStream_t stream);
constexpr int kSelHistRows = 8;  // rows per histogram item

// thr = fixbw of BandwidthWeight.cpp:40-53 from order statistics d0 (rank
// floor(bw), or the row maximum when bw >= n) and d1 (rank floor(bw)+1, may
// be null when bw is integral).
cudaError_t launch_threshold_combine(int n, double bw, const double* d0, const double* d1, double* thr,
                                     cudaStream_t stream);
// The same for `rows` focus rows over n data points (dn = bw / n).
cudaError_t launch_threshold_combine_rows(int rows, int n, double bw, const double* d0, const double* d1, double* thr,
                                          cudaStream_t stream);

// out[i] = (float)in[i].
cudaError_t launch_to_float(int n, const double* in, float* out, cudaStream_t stream);

// Z[j, :] = (upper triangle of x_j x_j^T packed by rows, x_j * y_j); X row-major n x p.
cudaError_t launch_build_z(int n, int p, const double* X, const double* y, double* Z, cudaStream_t stream);

// G[i, c] = sum_j w_ij^wpow Z[j, c] for c < mcols, with w_ij = K(d_ij, r_i)
// (r_i = thr[i], or bw when thr is null); exclude_self zeroes w_ii (CV).
// FP64 SIMT, the weight matrix is produced tile by tile and never stored.
// tb16: FP32 bounds of the 16-point tiles (planar box or geographic cap).
cudaError_t launch_contract64(const DevPoints& P, bool geographic, const float4* tb16, const double* Z, int ldz,
                              int mcols, double* G, int ldg, const double* thr, double bw, int kernel,
                              bool exclude_self, int wpow, bool skip_tiles, cudaStream_t stream);
// The same with focus rows F (their 16-point tile bounds ftb16) that are not
// the data points: G[i, :] for every focus row i over the data P (predict).
cudaError_t launch_contract64_focus(const DevPoints& P, const float4* tb16, const DevPoints& F, const float4* ftb16,
                                    bool geographic, const double* Z, int ldz, int mcols, double* G, int ldg,
                                    const double* thr, double bw, int kernel, bool exclude_self, int wpow,
                                    bool skip_tiles, cudaStream_t stream);

// Warp-per-location Cholesky solve of A_i beta_i = b_i and the per-location
// criterion terms; partial sums per block in partials[block*4 + {0..3}] =
// (sum s_ii, sum residual^2, sum ||s_i||^2, failures).  Returns the number
// of partial blocks through nblocks.
struct SolveArgs {
    int n, p, mode, kernel;
    const double* G;   // n x m (A packed upper, then b)
    int ldg;
    const double* G2;  // n x p(p+1)/2 (X^T W^2 X packed upper), fit only
    int ldg2;
    const double* X;   // n x p row-major
    const double* y;
    const double* thr; // per-row threshold or null
    double bw;
    double* beta;      // n x p row-major
    double* sii;       // n
    double* resid;     // n
    double* v;         // n x p: A_i^{-1} x_i (fit)
    double* bse;       // n x p: diag(T A^-1 Q A^-1 T^T) (fit)
    double* partials;
    // Optional linear map T of the coefficients (fit): T = diag(tinv) except
    // row tcol = tvec (the intercept row after centring).  Null: identity.
    const double* tinv;
    const double* tvec;
    int tcol;
    // Refine mode: beta += A^-1 rvec (n x p), then the residuals are recomputed.
    const double* rvec;
    // Fit mode, optional: A_i^-1 (n x p x p, row-major per row).
    double* ainv;
};
// Largest grid launch_solve uses; callers size `partials` (4 doubles per block) for it.
constexpr int kSolveMaxBlocks = 4096;
cudaError_t launch_solve(const SolveArgs& a, int* nblocks, cudaStream_t stream);
// Criterion solves (kSolveAIC / kSolveCV) of many segments in one launch:
// block b solves rows [work[b].y, work[b].z) of segment work[b].x and writes
// partial slot work[b].w of that segment (device arrays; p <= max_p).
cudaError_t launch_solve_batch(const SolveArgs* segs, const int4* work, int nwork, int mode, int max_p,
                               cudaStream_t stream);
// out[4 s .. 4 s + 3] = fixed-order sums of partial blocks [first[s], first[s + 1]).
cudaError_t launch_reduce_batch(const double* partials, const int* first, int nseg, double* out, cudaStream_t stream);

// Sums nblocks x 4 partials into out[4] in a fixed order.
cudaError_t launch_reduce_partials(const double* partials, int nblocks, double* out, cudaStream_t stream);

// qdiag[j] = sum_i (delta_ij - s_ij)^2 with s_ij = w_ij v_i . x_j, w_ij =
// K(d_ij, r_i); also writes S (n x n row-major, sorted order) when S != null
// and row row_target of S into s_row (length n) when s_row != null.
// tile_thr: far-test threshold of each 16-point tile's largest r_i (launch_tile_far_thr).
cudaError_t launch_hat_pass(const DevPoints& P, bool geographic, const float4* tb16, const float* tile_thr,
                            const double* X, int p,
                            const double* v, const double* thr, double bw, int kernel, bool skip_tiles,
                            double* qdiag, double* S, int row_target, double* s_row, cudaStream_t stream);

// Column subset of X for the w == 1 criterion of variable selection.
struct ColumnSet {
    int count;
    int cols[kMaxP];
};

// out[c] = sum_j Z[j, c] (n x m row-major) with nb fixed partial blocks (part: nb x m).
cudaError_t launch_column_sums(int n, int m, const double* Z, double* part, int nb, double* out, cudaStream_t stream);

// Xs = X[:, cols] (n x q row-major) and gsub = the packed X^T X / X^T y of the
// subset taken from the full column sums gall.
cudaError_t launch_gather_subset(int n, int p, const ColumnSet& cs, const double* X, const double* gall, double* Xs,
                                 double* gsub, cudaStream_t stream);

// Mixed-precision W.Z contraction on tcgen05 (k_contract_tc.cu).
struct TcArgs {
    int n, mcols, npad, ntiles;   // ntiles: 32-point tiles
    const float4* pts;            // planar: {u_hi, u_lo, v_hi, v_lo}; geographic: 2 float4 (hi/lo unit vector)
    const float4* tb;             // FP32 bound of each 32-point tile (planar box or geographic cap)
    const unsigned char* zimg;    // per tile: [hi | lo] swizzled images, npad x 128 bytes each
    const float* thr;             // per-row threshold, or null for the fixed bandwidth bw
    float bw;
    int kernel, exclude_self, skip, flush_tiles, wpow;
    float2* acc;                  // double-float sums: ceil(n / 128) x npad x 128 (rows in groups of 128)
    float* stage;                 // FP32 staging of one chunk, same layout (single-accumulator form), or null
    double* G;                    // n x ldg FP64 output (first mcols columns)
    int ldg;
    int* err;                     // set to 1 if a bounded wait timed out
    unsigned long long* tiles;    // if not null: += 128 x 32 weight tiles processed
    unsigned long long* prof;     // if not null: += clock64 cycles per phase (kTcProfSlots slots)
    const float* d2c;             // geographic only, optional: the distance cache of launch_fill_d2_sym
    unsigned wait_limit;          // polls of a pipeline wait before it times out (0: the default)
};
// Phase slots of TcArgs::prof, summed over CTAs (producer: warp 0 lane 0;
// control: the issuing thread).
enum TcProf {
    kTcProfStageWait,   // producer: waiting for a free weight stage
    kTcProfPointsWait,  // producer: waiting for the tile's point records
    kTcProfWeights,     // producer: weights, split and shared-memory stores
    kTcProfFlush,       // drain warp 0: draining accumulators
    kTcProfAWait,       // control: waiting for the weight tile
    kTcProfZWait,       // control: waiting for the Z tile and a free accumulator
    kTcProfIssue,       // control: MMA issue and Z prefetch
    kTcProfLoop,        // producer: whole tile loop
    kTcProfLoopMax,     // producer: largest tile loop of one CTA (maximum, not a sum)
    kTcProfPrologue,    // producer: kernel start to tile loop
    kTcProfEpilogue,    // producer: tile loop end to kernel end
    kTcProfTilesMax,    // largest number of tiles one CTA processed (maximum, not cycles)
    kTcProfSlots
};
size_t contract_tc_smem_bytes(int npad, int ntiles, int nb, bool cached);
cudaError_t launch_contract_tc(const TcArgs& a, bool geographic, cudaStream_t stream);
// Many contractions in one launch: CTA b computes row block work[b].y of
// segment work[b].x (device arrays; every segment's npad <= max_npad and
// ntiles <= max_ntiles; flush_tiles and the weight kernel are shared).
cudaError_t launch_contract_tc_batch(const TcArgs* segs, const int2* work, int nwork, int max_npad, int max_ntiles,
                                     int flush_tiles, bool geographic, int kernel, cudaStream_t stream);
cudaError_t launch_build_zimg(int n, int mcols, int npad, const double* Z, int ldz, unsigned char* img,
                              cudaStream_t stream);
// Distance cache of the mixed geographic contraction: the FP32 squared
// great-circle distance of every (focus row, data point) pair, exactly the
// value the contraction's weight producer computes, for rows padded to whole
// 128-row blocks and points padded to whole 32-point tiles.  Block (rb, tile)
// is 4096 floats at ((rb * ntiles + tile) * 4096), ordered [quarter 4][half 2]
// [row 128][4 points] so the producer thread of (row, quarter) reads its 8
// points as two float4 and a warp's loads are contiguous; padded pairs hold
// FLT_MAX.  pts: the 2 float4 records per point, padded to whole tiles.
size_t d2_cache_bytes(int n);
// The distance cache of geographic mixed data: every pair's FP32 squared
// distance, block (row block rb of 128 rows, 32-point tile t) of 4096 floats at
// (rb * ntiles + t) * 4096, ordered [quarter 4][half 2][row 128][4 points].
// Each pair is computed once (the FP32 distance is symmetric) and written to
// both rows.  scratch: ceil(n / 128) + 2 ints of device memory.
cudaError_t launch_fill_d2_sym(int n, const float4* pts, float* d2c, int* scratch, int num_sms, cudaStream_t stream);
// D[128 x N] = A[128 x 32] B[N x 32]^T through tcgen05 (device pointers).
cudaError_t launch_tc_selftest(const float* A, const float* B, float* D, int N, int* err, cudaStream_t stream);

// Refinement residual of the mixed path: r_i = X~^T W_i (y~ - X~ beta_i) in
// FP64 arithmetic over the FP32 weights of the contraction (n x p output).
struct RefineArgs {
    int n, p, ntiles, kernel, skip;
    const float4* pts;
    const float4* tb;     // FP32 bound of each 32-point tile
    const double* X;      // n x p row-major (X~)
    const double* y;      // y~
    const double* beta;   // n x p
    const float* thr;
    float bw;
    double* r;            // n x p
    const float* d2c;     // geographic only, optional: the distance cache (the contraction's FP32 d^2)
};
cudaError_t launch_refine_residual(const RefineArgs& a, bool geographic, cudaStream_t stream);

// Mixed-precision hat pass: the FP32 weights of the tensor-core contraction.
cudaError_t launch_hat_mixed(int n, bool geographic, const float4* pts, const float4* tb16, const float* tile_thr,
                             const double* X, int p, const double* v, const float* thr32, float bw, int kernel,
                             double* qdiag, double* S, int row_target, double* s_row, cudaStream_t stream);

// tile_thr[t] = far-test threshold of the largest r_i (thr, or bw) over tile t of `tile` points.
cudaError_t launch_tile_far_thr(int n, int tile, bool geographic, const double* thr, double bw, float* tile_thr,
                                cudaStream_t stream);

// Maximum pairwise distance (CRSDistance::maxDistance) as an ordered key: key_out[0]
// for planar data, key_out[1] for geographic data (key_out[0] then holds the
// unit-vector form's maximum).  Both keys start at 0; rowmax (geographic only)
// holds n doubles of scratch.
cudaError_t launch_max_distance(const DevPoints& P, bool geographic, unsigned long long* key_out, double* rowmax,
                                int num_sms, cudaStream_t stream);


// GWRMultiscale hat matrix (k_mgwr.cu).  Matrices are n x n row-major in the
// sorted order; SA holds p of them back to back.
size_t mgwr_hat_all_smem(int p);
// SA_k(i, j) = w_ij x_ik (A_i^-1 x_j)_k and S0(i, j) = sum_k SA_k(i, j) for
// every pair (ainv: n x p x p from the fit's solve).
cudaError_t launch_mgwr_hat_all(const DevPoints& P, bool geographic, const double* X, int p, const double* ainv,
                                const double* thr, double bw, int kernel, double* S0, double* SA, int num_sms,
                                cudaStream_t stream);
// T = SA - S0 over count elements.
cudaError_t launch_mgwr_sub(size_t count, const double* SA, const double* S0, double* T, cudaStream_t stream);
// SA = S (T + I) for the one-variable hat matrix S(i, j) = w_ij v_i x_j of a
// compact kernel (bisquare, tricube, boxcar), over neighbouring data tiles only
// (X: the variable, v: A_i^-1 x_i from the fit, both n sorted).
cudaError_t launch_mgwr_hat_update(const DevPoints& P, bool geographic, const float4* tb16, const double* X,
                                   const double* v, const double* thr, double bw, int kernel, const double* T,
                                   double* SA, cudaStream_t stream);
// SA += S (S may be null: no addition); S0 = SA - T over count elements.
cudaError_t launch_mgwr_post(size_t count, double* SA, const double* S, const double* T, double* S0,
                             cudaStream_t stream);
// partials[4 b + 0] / [4 b + 1]: block b's share of tr(S0) and of sum S0_ij^2;
// *nblocks receives the block count (at most max_blocks).
cudaError_t launch_mgwr_traces(int n, const double* S0, double* partials, int max_blocks, int* nblocks,
                               cudaStream_t stream);

}  // namespace gwgpu
