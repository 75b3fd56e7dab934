/*
 * numbagg_gb300 -- C ABI of the GB300 (sm_103a) scan / reduction library.
 *
 * Every entry point replaces one numba gufunc of numbagg: the decorator's
 * `__call__` (argument checks, axis handling) stays on the host, and what the
 * gufunc computed over the loop dimensions is one call here over a (rows, n)
 * C-contiguous view with the scanned axis last.  Plain pointers and sizes only:
 * device pointers for data, `stream` is a cudaStream_t (NULL = legacy default).
 * Calls are asynchronous on `stream`; every call returns an NBG_* status.
 *
 * Workspaces.  Fills carry state between tiles through a look-back workspace sized by
 * nbg_fill_workspace_bytes().
 * A look-back workspace must be zero-filled once when it is allocated; it then
 * maintains itself across launches.  One workspace per stream: launches that share
 * it must be ordered on one stream.  Moving windows, the exponential moving functions
 * and the grouped reductions take a scratch buffer (nbg_move_workspace_bytes(),
 * nbg_move_exp_workspace_bytes(), nbg_group_workspace_bytes()) that needs no
 * initialisation; do not share a scratch buffer with a look-back workspace.
 */
#ifndef NUMBAGG_GB300_H
#define NUMBAGG_GB300_H

#include <stddef.h>

#if defined(__GNUC__) || defined(__clang__)
#define NBG_API __attribute__((visibility("default")))
#else
#define NBG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------- */
#define NBG_OK 0
#define NBG_INVALID_ARGUMENT 1 /* numbagg raises ValueError/TypeError before compute */
#define NBG_LAUNCH_ERROR 2
#define NBG_WORKSPACE_TOO_SMALL 3
#define NBG_LOOKBACK_TIMEOUT 4 /* recorded on the device; read with nbg_workspace_error */
#define NBG_UNSUPPORTED 5
#define NBG_TOO_LARGE 6 /* beyond the fixed scratch of an allocation-free entry point */

NBG_API int nbg_version(void);
NBG_API const char* nbg_status_string(int status);
NBG_API size_t nbg_workspace_header_bytes(void);
NBG_API int nbg_workspace_error(void* ws, int* code, unsigned* tile, void* stream);
/* Number of kernels this library has launched in the process (all devices). */
NBG_API unsigned long long nbg_launch_count(void);

/* Deterministic mode (no reference counterpart: numbagg is sequential and always
 * reproducible; this mirrors torch.use_deterministic_algorithms).  When on, every
 * call either runs an algorithm whose result bits do not depend on scheduling, or
 * returns NBG_UNSUPPORTED: float group sums / means / variances with more labels than
 * fit the shared-memory bins (several thousand) have only a float64-atomic
 * implementation.  Off by default; process-wide. */
NBG_API void nbg_set_deterministic(int on);
NBG_API int nbg_get_deterministic(void);
/* Test hook for failure detection: one bounded wait on a status nothing publishes. */
NBG_API int nbg_debug_lookback_timeout(void* ws, size_t ws_bytes, int spin_limit, void* stream);

/* ---- moving windows ---------------------------------------------------------------
 * Replaces the gufuncs built by ndmove (numbagg/decorators.py:275-341) from
 *   move_sum  numbagg/moving.py:58-99      move_mean numbagg/moving.py:12-55
 *   move_var  numbagg/moving.py:154-181    move_std  numbagg/moving.py:123-151
 *   move_cov  numbagg/moving.py:184-220    move_corr numbagg/moving.py:223-275
 * signature "(a),(),()->(a)" / "(a),(a),(),()->(a)"; a, b, out: rows x n.
 * min_count is passed unclamped (each kernel applies the reference's max()).
 * ws: a scratch buffer of nbg_move_workspace_bytes(rows, n) bytes, no initialisation
 * needed (reciprocal table and per-row state, rewritten by every call). */
NBG_API size_t nbg_move_workspace_bytes(long long rows, long long n);
#define NBG_DECL_MOVE1(NAME, T, SFX)                                                      \
  NBG_API int nbg_##NAME##_##SFX(const T* a, T* out, long long rows, long long n, long long window, \
                         long long min_count, void* ws, size_t ws_bytes, void* stream);
#define NBG_DECL_MOVE2(NAME, T, SFX)                                                      \
  NBG_API int nbg_##NAME##_##SFX(const T* a, const T* b, T* out, long long rows, long long n,      \
                         long long window, long long min_count, void* ws, size_t ws_bytes, \
                         void* stream);
NBG_DECL_MOVE1(move_sum, double, f64)
NBG_DECL_MOVE1(move_sum, float, f32)
NBG_DECL_MOVE1(move_mean, double, f64)
NBG_DECL_MOVE1(move_mean, float, f32)
NBG_DECL_MOVE1(move_var, double, f64)
NBG_DECL_MOVE1(move_var, float, f32)
NBG_DECL_MOVE1(move_std, double, f64)
NBG_DECL_MOVE1(move_std, float, f32)
NBG_DECL_MOVE2(move_cov, double, f64)
NBG_DECL_MOVE2(move_cov, float, f32)
NBG_DECL_MOVE2(move_corr, double, f64)
NBG_DECL_MOVE2(move_corr, float, f32)
/* FP32-compensated forms of the float64 entry points (no reference counterpart: numbagg
 * computes in float64 only).  A one-pass double-float window scan on the FP32 pipes
 * (values minus the row's first finite value for the variance-like statistics); rows
 * holding an infinity or values beyond its range are recomputed from exact window sums
 * finalised in double-float.  Stated bound: 2e-6 relative to the window's magnitude;
 * ws must then be nbg_move_workspace_bytes(rows, n) bytes (it holds the scan's
 * look-back state). */
NBG_DECL_MOVE1(move_sum, double, f64_fp32c)
NBG_DECL_MOVE1(move_mean, double, f64_fp32c)
NBG_DECL_MOVE1(move_var, double, f64_fp32c)
NBG_DECL_MOVE1(move_std, double, f64_fp32c)
NBG_DECL_MOVE2(move_cov, double, f64_fp32c)
NBG_DECL_MOVE2(move_corr, double, f64_fp32c)
/* Along a non-last axis of a C-contiguous array (the strided core axis numbagg's
 * gufuncs accept, numbagg/decorators.py:340-341): `outer` blocks of n x `inner`
 * values, position p of column i of block o at (o * n + p) * inner + i, scanned along
 * n in place by one thread per column running numbagg's loop (the reference's float64
 * arithmetic, bit for bit).  No workspace. */
#define NBG_DECL_MOVE1_COLS(NAME, T, SFX)                                                        \
  NBG_API int nbg_##NAME##_cols_##SFX(const T* a, T* out, long long outer, long long n, long long inner, \
                                      long long window, long long min_count, void* stream);
#define NBG_DECL_MOVE2_COLS(NAME, T, SFX)                                                        \
  NBG_API int nbg_##NAME##_cols_##SFX(const T* a, const T* b, T* out, long long outer, long long n,    \
                                      long long inner, long long window, long long min_count, void* stream);
#define NBG_DECL_MOVE_COLS_ALL(T, SFX)  \
  NBG_DECL_MOVE1_COLS(move_sum, T, SFX)  \
  NBG_DECL_MOVE1_COLS(move_mean, T, SFX) \
  NBG_DECL_MOVE1_COLS(move_var, T, SFX)  \
  NBG_DECL_MOVE1_COLS(move_std, T, SFX)  \
  NBG_DECL_MOVE2_COLS(move_cov, T, SFX)  \
  NBG_DECL_MOVE2_COLS(move_corr, T, SFX)
NBG_DECL_MOVE_COLS_ALL(double, f64)
NBG_DECL_MOVE_COLS_ALL(float, f32)

/* Ragged batches of moving windows (no reference counterpart: numbagg applies its
 * functions array by array; these run many series of uneven length in one call).
 * values: the series back to back, series s = values[offsets[s] : offsets[s + 1]];
 * offsets: nseries + 1 device int64, offsets[0] = 0, nondecreasing; out: like values.
 * ws: scratch of nbg_move_ragged_workspace_bytes(nseries, total) bytes (total: values
 * in all), with which the _fp32c forms run their double-float tile scan;
 * nbg_move_workspace_bytes(nseries, 0) bytes suffice for the exact kernels alone.
 * chunk_len: positions per work item of the exact kernels (0 = default: eight windows,
 * at least 32768). */
NBG_API size_t nbg_move_ragged_workspace_bytes(long long nseries, long long total);
#define NBG_DECL_MOVE_RAGGED(NAME, SFX)                                                          \
  NBG_API int nbg_##NAME##_ragged_##SFX(const double* values, const long long* offsets, long long nseries, \
                                        double* out, long long window, long long min_count,             \
                                        long long chunk_len, void* ws, size_t ws_bytes, void* stream);
NBG_DECL_MOVE_RAGGED(move_sum, f64)
NBG_DECL_MOVE_RAGGED(move_mean, f64)
NBG_DECL_MOVE_RAGGED(move_var, f64)
NBG_DECL_MOVE_RAGGED(move_std, f64)
NBG_DECL_MOVE_RAGGED(move_sum, f64_fp32c)
NBG_DECL_MOVE_RAGGED(move_mean, f64_fp32c)
NBG_DECL_MOVE_RAGGED(move_var, f64_fp32c)
NBG_DECL_MOVE_RAGGED(move_std, f64_fp32c)

/* ---- exponentially weighted moving functions ---------------------------------------
 * Replaces the gufuncs built by ndmoveexp (numbagg/decorators.py:344-414) from
 *   move_exp_nancount numbagg/moving_exp.py:12-38    move_exp_nanmean numbagg/moving_exp.py:41-71
 *   move_exp_nansum   numbagg/moving_exp.py:74-102   move_exp_nanvar  numbagg/moving_exp.py:105-156
 *   move_exp_nanstd   numbagg/moving_exp.py:158-223  move_exp_nancov  numbagg/moving_exp.py:226-272
 *   move_exp_nancorr  numbagg/moving_exp.py:275-335
 * ws: scratch (no initialisation), nbg_move_exp_workspace_bytes() bytes.
 * alpha_mode 0: scalar alpha_scalar (already rounded to the array dtype);
 * 1: `alpha` holds n values shared by every row; 2: `alpha` holds rows x n values.
 * min_weight is the array-dtype value widened to double. */
NBG_API size_t nbg_move_exp_workspace_bytes(long long rows, long long n);
#define NBG_DECL_EXP1(NAME, T, SFX)                                                         \
  NBG_API int nbg_##NAME##_##SFX(const T* a, const T* alpha, double alpha_scalar, int alpha_mode,    \
                         double min_weight, T* out, long long rows, long long n, void* ws,   \
                         size_t ws_bytes, void* stream);
#define NBG_DECL_EXP2(NAME, T, SFX)                                                         \
  NBG_API int nbg_##NAME##_##SFX(const T* a, const T* b, const T* alpha, double alpha_scalar,        \
                         int alpha_mode, double min_weight, T* out, long long rows,          \
                         long long n, void* ws, size_t ws_bytes, void* stream);
NBG_DECL_EXP1(move_exp_nancount, double, f64)
NBG_DECL_EXP1(move_exp_nancount, float, f32)
NBG_DECL_EXP1(move_exp_nanmean, double, f64)
NBG_DECL_EXP1(move_exp_nanmean, float, f32)
NBG_DECL_EXP1(move_exp_nansum, double, f64)
NBG_DECL_EXP1(move_exp_nansum, float, f32)
NBG_DECL_EXP1(move_exp_nanvar, double, f64)
NBG_DECL_EXP1(move_exp_nanvar, float, f32)
NBG_DECL_EXP1(move_exp_nanstd, double, f64)
NBG_DECL_EXP1(move_exp_nanstd, float, f32)
NBG_DECL_EXP2(move_exp_nancov, double, f64)
NBG_DECL_EXP2(move_exp_nancov, float, f32)
NBG_DECL_EXP2(move_exp_nancorr, double, f64)
NBG_DECL_EXP2(move_exp_nancorr, float, f32)
/* FP32-compensated forms of the float64 entry points (no reference counterpart):
 * the same deterministic scan in double-float on the FP32 pipes, about 2^-46 relative
 * precision per operation; variance, standard deviation, covariance and correlation
 * subtract each row's first finite value first (they are shift invariant). */
NBG_DECL_EXP1(move_exp_nancount, double, f64_fp32c)
NBG_DECL_EXP1(move_exp_nanmean, double, f64_fp32c)
NBG_DECL_EXP1(move_exp_nansum, double, f64_fp32c)
NBG_DECL_EXP1(move_exp_nanvar, double, f64_fp32c)
NBG_DECL_EXP1(move_exp_nanstd, double, f64_fp32c)
NBG_DECL_EXP2(move_exp_nancov, double, f64_fp32c)
NBG_DECL_EXP2(move_exp_nancorr, double, f64_fp32c)

/* The exponentially weighted family along a non-last axis of C-contiguous arrays, as the
 * fills above (numbagg/decorators.py:409-414 hands the gufunc the strided axis): `outer`
 * blocks of n x `inner` values scanned along n, one thread per column running numbagg's
 * loop (the float64 arithmetic repeats the reference's operations in order).
 * alpha_mode 0: scalar; 1: n values along the axis; 2: one per element, laid out like a.
 * No workspace. */
#define NBG_DECL_EXP1_COLS(NAME, T, SFX)                                                              \
  NBG_API int nbg_##NAME##_cols_##SFX(const T* a, const T* alpha, double alpha_scalar, int alpha_mode, \
                                      double min_weight, T* out, long long outer, long long n,         \
                                      long long inner, void* stream);
#define NBG_DECL_EXP2_COLS(NAME, T, SFX)                                                              \
  NBG_API int nbg_##NAME##_cols_##SFX(const T* a, const T* b, const T* alpha, double alpha_scalar,     \
                                      int alpha_mode, double min_weight, T* out, long long outer,      \
                                      long long n, long long inner, void* stream);
#define NBG_DECL_EXP_COLS_ALL(T, SFX)                \
  NBG_DECL_EXP1_COLS(move_exp_nancount, T, SFX)      \
  NBG_DECL_EXP1_COLS(move_exp_nanmean, T, SFX)       \
  NBG_DECL_EXP1_COLS(move_exp_nansum, T, SFX)        \
  NBG_DECL_EXP1_COLS(move_exp_nanvar, T, SFX)        \
  NBG_DECL_EXP1_COLS(move_exp_nanstd, T, SFX)        \
  NBG_DECL_EXP2_COLS(move_exp_nancov, T, SFX)        \
  NBG_DECL_EXP2_COLS(move_exp_nancorr, T, SFX)
NBG_DECL_EXP_COLS_ALL(double, f64)
NBG_DECL_EXP_COLS_ALL(float, f32)
NBG_DECL_EXP_COLS_ALL(double, f64_fp32c)

/* Ragged batches of exponentially weighted functions (no reference counterpart):
 * series as for the moving windows, `total` = offsets[nseries]; alpha_mode 0 (scalar
 * alpha_scalar) or 2 (one alpha per value, laid out like values).  ws:
 * nbg_move_exp_ragged_workspace_bytes(nseries, total) bytes of scratch. */
NBG_API size_t nbg_move_exp_ragged_workspace_bytes(long long nseries, long long total);
#define NBG_DECL_EXP_RAGGED(NAME, SFX)                                                              \
  NBG_API int nbg_##NAME##_ragged_##SFX(const double* values, const long long* offsets, long long nseries, \
                                        long long total, const double* alpha, double alpha_scalar,      \
                                        int alpha_mode, double min_weight, double* out, void* ws,       \
                                        size_t ws_bytes, void* stream);
NBG_DECL_EXP_RAGGED(move_exp_nanmean, f64)
NBG_DECL_EXP_RAGGED(move_exp_nanvar, f64)
NBG_DECL_EXP_RAGGED(move_exp_nanstd, f64)
NBG_DECL_EXP_RAGGED(move_exp_nanmean, f64_fp32c)
NBG_DECL_EXP_RAGGED(move_exp_nanvar, f64_fp32c)
NBG_DECL_EXP_RAGGED(move_exp_nanstd, f64_fp32c)

/* ---- fills --------------------------------------------------------------------------
 * Replaces the gufuncs built by ndfill (numbagg/decorators.py:417-487) from
 *   ffill numbagg/funcs.py:313-326    bfill numbagg/funcs.py:294-311
 * signature "(n),()->(n)"; limit >= 0 (numbagg passes shape[axis] for None).
 * Integer arrays need no workspace. */
NBG_API size_t nbg_fill_workspace_bytes(long long rows, long long n);
#define NBG_DECL_FILL(T, SFX)                                                                \
  NBG_API int nbg_ffill_##SFX(const T* a, T* out, long long rows, long long n, long long limit,       \
                      void* ws, size_t ws_bytes, void* stream);                              \
  NBG_API int nbg_bfill_##SFX(const T* a, T* out, long long rows, long long n, long long limit,       \
                      void* ws, size_t ws_bytes, void* stream);
NBG_DECL_FILL(double, f64)
NBG_DECL_FILL(float, f32)
NBG_DECL_FILL(int, i32)
NBG_DECL_FILL(long long, i64)

/* Fills along a non-last axis of a C-contiguous array, in place of moving the axis last
 * and copying (numbagg's gufuncs take such strided core axes directly,
 * numbagg/decorators.py:340-341, :480-487): `outer` blocks of n x `inner` values, position
 * p of column i of block o at a[(o * n + p) * inner + i]; out laid out like a.  One
 * thread per column, no workspace. */
#define NBG_DECL_FILL_COLS(T, SFX)                                                                   \
  NBG_API int nbg_ffill_cols_##SFX(const T* a, T* out, long long outer, long long n, long long inner, \
                                   long long limit, void* stream);                                   \
  NBG_API int nbg_bfill_cols_##SFX(const T* a, T* out, long long outer, long long n, long long inner, \
                                   long long limit, void* stream);
NBG_DECL_FILL_COLS(double, f64)
NBG_DECL_FILL_COLS(float, f32)
NBG_DECL_FILL_COLS(int, i32)
NBG_DECL_FILL_COLS(long long, i64)

/* Allocation-free forward fill (float64).  No counterpart in numbagg: it exists for
 * callers that may not allocate device memory -- a host application that owns all GPU
 * memory and lends this library only the input and output buffers (a database or
 * stream engine running it as a user-defined function under a fixed budget), or a
 * latency-critical path that must never reach cudaMalloc/cudaFree, which can
 * synchronise the device.  Same results as nbg_ffill_f64; no workspace argument and
 * no allocation of any kind.  The look-back state lives in a 4 MiB array inside the
 * library's device image (every GPU that loads the library keeps it until the
 * process exits), so a call may cover at most that many tiles: rows x ceil(n / 4096)
 * tiles within nbg_ffill_noalloc_max_scratch_bytes(); larger problems return
 * NBG_TOO_LARGE without launching.  The array is zero when the library's device code
 * loads and every launch leaves it in that state.  Each call looks up the array's
 * address on the current device; the first call on a device may load the library's
 * device code, so make it before any stream capture.  All calls on a device share
 * the one array: calls that overlap on the GPU (different streams, or concurrent
 * threads) race and must be serialised by the caller.
 * nbg_ffill_noalloc_error reads and clears the array's error word (a look-back wait
 * that ran out of its bound records NBG_LOOKBACK_TIMEOUT and the tile there, as in a
 * workspace); it synchronises `stream`. */
NBG_API size_t nbg_ffill_noalloc_max_scratch_bytes(void);
NBG_API int nbg_ffill_f64_noalloc(const double* a, double* out, long long rows, long long n,
                                  long long limit, void* stream);
NBG_API int nbg_ffill_noalloc_error(int* code, unsigned* tile, void* stream);

/* ---- grouped reductions ----------------------------------------------------------------
 * Replaces the gufuncs built by groupndreduce (numbagg/decorators.py:490-674) from
 * numbagg/grouped.py:7-270: values rows x m (the broadcast dims flattened, the core
 * dims flattened in C order), labels m (shared by every row), out rows x num_labels.
 * Labels < 0 or >= num_labels are skipped.  ddof is read by nanvar/nanstd only.
 * `func` for the workspace query: 0 sum, 1 count, 2 mean, 3 var, 4 std, 5 sum_of_squares,
 * 6 argmax, 7 argmin, 8 max, 9 min, 10 first, 11 last, 12 prod, 13 any, 14 all. */
NBG_API size_t nbg_group_workspace_bytes(int func, long long rows, long long m, long long num_labels);
#define NBG_DECL_GROUP1(NAME, V, VS, O, L, LS)                                                 \
  NBG_API int nbg_group_##NAME##_##VS##_##LS(const V* values, const L* labels, O* out, long long rows,  \
                                     long long m, long long num_labels, long long ddof,        \
                                     void* ws, size_t ws_bytes, void* stream);
#define NBG_DECL_GROUP_L(NAME, V, VS, O) \
  NBG_DECL_GROUP1(NAME, V, VS, O, int, i32) NBG_DECL_GROUP1(NAME, V, VS, O, long long, i64)
#define NBG_DECL_GROUP_ALL(NAME)                                                   \
  NBG_DECL_GROUP_L(NAME, double, f64, double) NBG_DECL_GROUP_L(NAME, float, f32, float) \
  NBG_DECL_GROUP_L(NAME, int, i32, int) NBG_DECL_GROUP_L(NAME, long long, i64, long long)
#define NBG_DECL_GROUP_FLOAT(NAME) \
  NBG_DECL_GROUP_L(NAME, double, f64, double) NBG_DECL_GROUP_L(NAME, float, f32, float)
NBG_DECL_GROUP_ALL(nansum)            /* numbagg/grouped.py:30-40 */
NBG_DECL_GROUP_ALL(nancount)          /* numbagg/grouped.py:43-51 */
NBG_DECL_GROUP_FLOAT(nanmean)         /* numbagg/grouped.py:7-27 (ints promoted by the caller) */
NBG_DECL_GROUP_FLOAT(nanvar)          /* numbagg/grouped.py:148-176 */
NBG_DECL_GROUP_FLOAT(nanstd)          /* numbagg/grouped.py:179-208 */
NBG_DECL_GROUP_ALL(nansum_of_squares) /* numbagg/grouped.py:135-145 */
NBG_DECL_GROUP_ALL(nanargmax)         /* numbagg/grouped.py:54-75 */
NBG_DECL_GROUP_ALL(nanargmin)         /* numbagg/grouped.py:78-92 */
NBG_DECL_GROUP_ALL(nanmax)            /* numbagg/grouped.py:229-244 */
NBG_DECL_GROUP_ALL(nanmin)            /* numbagg/grouped.py:211-226 */
NBG_DECL_GROUP_ALL(nanfirst)          /* numbagg/grouped.py:95-110 */
NBG_DECL_GROUP_ALL(nanlast)           /* numbagg/grouped.py:113-121 */
NBG_DECL_GROUP_ALL(nanprod)           /* numbagg/grouped.py:124-132 */
NBG_DECL_GROUP_ALL(nanany)            /* numbagg/grouped.py:247-257 */
NBG_DECL_GROUP_ALL(nanall)            /* numbagg/grouped.py:260-270 */

/* Along non-last axes, in place: values whose reduced axes are consecutive and not last,
 * a C-contiguous (outer, m, inner) array with labels over m (the reduced axes flattened,
 * numbagg's np.ndindex order); out[(o * inner + i) * K + k], in the values dtype like the
 * row entry points above.  One thread per column runs numbagg's loop, so the results are
 * the reference's bit for bit.  No workspace; K at most nbg_group_cols_max_labels(func)
 * (func numbered as for nbg_group_workspace_bytes), else NBG_UNSUPPORTED.
 * nanmean/nanvar/nanstd take float values only (numbagg computes integers in float64). */
NBG_API size_t nbg_group_cols_max_labels(int func);
#define NBG_DECL_GROUP_COLS1(NAME, V, VS, L, LS)                                                 \
  NBG_API int nbg_group_##NAME##_cols_##VS##_##LS(const V* values, const L* labels, V* out,      \
                                                  long long outer, long long m, long long inner, \
                                                  long long K, long long ddof, void* stream);
#define NBG_DECL_GROUP_COLS_L(NAME, V, VS) \
  NBG_DECL_GROUP_COLS1(NAME, V, VS, int, i32) NBG_DECL_GROUP_COLS1(NAME, V, VS, long long, i64)
#define NBG_DECL_GROUP_COLS_FLOAT(NAME) NBG_DECL_GROUP_COLS_L(NAME, double, f64) NBG_DECL_GROUP_COLS_L(NAME, float, f32)
#define NBG_DECL_GROUP_COLS_ALL(NAME) \
  NBG_DECL_GROUP_COLS_FLOAT(NAME) NBG_DECL_GROUP_COLS_L(NAME, int, i32) NBG_DECL_GROUP_COLS_L(NAME, long long, i64)
NBG_DECL_GROUP_COLS_ALL(nansum)
NBG_DECL_GROUP_COLS_ALL(nancount)
NBG_DECL_GROUP_COLS_FLOAT(nanmean)
NBG_DECL_GROUP_COLS_FLOAT(nanvar)
NBG_DECL_GROUP_COLS_FLOAT(nanstd)
NBG_DECL_GROUP_COLS_ALL(nansum_of_squares)
NBG_DECL_GROUP_COLS_ALL(nanprod)
NBG_DECL_GROUP_COLS_ALL(nanargmax)
NBG_DECL_GROUP_COLS_ALL(nanargmin)
NBG_DECL_GROUP_COLS_ALL(nanmax)
NBG_DECL_GROUP_COLS_ALL(nanmin)
NBG_DECL_GROUP_COLS_ALL(nanfirst)
NBG_DECL_GROUP_COLS_ALL(nanlast)
NBG_DECL_GROUP_COLS_ALL(nanany)
NBG_DECL_GROUP_COLS_ALL(nanall)

/* Ragged batches of labelled reductions (no reference counterpart): values and labels
 * flat (`total` values), series s = [offsets[s], offsets[s + 1]) with its own labels;
 * out: nseries x num_labels float64 (num_labels <= 8192).  Deterministic: per-chunk
 * partials folded in chunk order.  ws: nbg_group_ragged_workspace_bytes() bytes. */
NBG_API size_t nbg_group_ragged_workspace_bytes(long long nseries, long long total, long long num_labels);
#define NBG_DECL_GROUP_RAGGED(NAME, L, LS)                                                                 \
  NBG_API int nbg_group_##NAME##_ragged_f64_##LS(const double* values, const L* labels, const long long* offsets, \
                                                 long long nseries, long long total, long long num_labels,     \
                                                 double* out, void* ws, size_t ws_bytes, void* stream);
NBG_DECL_GROUP_RAGGED(nansum, int, i32)
NBG_DECL_GROUP_RAGGED(nansum, long long, i64)
NBG_DECL_GROUP_RAGGED(nanmean, int, i32)
NBG_DECL_GROUP_RAGGED(nanmean, long long, i64)
NBG_DECL_GROUP_RAGGED(nancount, int, i32)
NBG_DECL_GROUP_RAGGED(nancount, long long, i64)

/* ---- moving covariance / correlation matrices ----------------------------------------
 * Replaces the gufuncs built by ndmovematrix (numbagg/decorators.py:747-818) from
 *   move_corrmatrix numbagg/moving_matrix.py:16-114
 *   move_covmatrix  numbagg/moving_matrix.py:117-201
 * signature "(m,n),(),()->(m,n,n)": a batch x n_obs x n_vars, out batch x n_obs x n_vars x n_vars. */
#define NBG_DECL_MATRIX(NAME, T, SFX)                                                           \
  NBG_API int nbg_##NAME##_##SFX(const T* a, T* out, long long batch, long long n_obs, long long n_vars, \
                         long long window, long long min_count, void* stream);
NBG_DECL_MATRIX(move_covmatrix, double, f64)
NBG_DECL_MATRIX(move_covmatrix, float, f32)
NBG_DECL_MATRIX(move_corrmatrix, double, f64)
NBG_DECL_MATRIX(move_corrmatrix, float, f32)

/* ---- exponentially weighted covariance / correlation matrices -------------------------
 * Replaces the gufuncs built by ndmoveexpmatrix (numbagg/decorators.py:1031-1100) from
 *   move_exp_nancorrmatrix numbagg/moving_matrix.py:204-320
 *   move_exp_nancovmatrix  numbagg/moving_matrix.py:323-432
 * signature "(m,n),(m),()->(m,n,n)": a batch x n_obs x n_vars, alpha n_obs values per batch
 * entry at alpha + b * alpha_stride (alpha_stride 0: one alpha row shared by the batch),
 * out batch x n_obs x n_vars x n_vars.  min_weight is the array-dtype value widened to
 * double.  ws: nbg_move_exp_matrix_workspace_bytes(corr, f64, batch, n_obs, n_vars) bytes of
 * scratch (per-segment aggregates), no initialisation. */
NBG_API size_t nbg_move_exp_matrix_workspace_bytes(int corr, int f64, long long batch, long long n_obs,
                                                   long long n_vars);
#define NBG_DECL_EXP_MATRIX(NAME, T, SFX)                                                                  \
  NBG_API int nbg_##NAME##_##SFX(const T* a, const T* alpha, long long alpha_stride, double min_weight, T* out, \
                                 long long batch, long long n_obs, long long n_vars, void* ws, size_t ws_bytes, \
                                 void* stream);
NBG_DECL_EXP_MATRIX(move_exp_nancovmatrix, double, f64)
NBG_DECL_EXP_MATRIX(move_exp_nancovmatrix, float, f32)
NBG_DECL_EXP_MATRIX(move_exp_nancorrmatrix, double, f64)
NBG_DECL_EXP_MATRIX(move_exp_nancorrmatrix, float, f32)

/* ---- static pairwise-complete covariance / correlation matrices -----------------------
 * Replaces the gufuncs built by ndmatrix (numbagg/decorators.py:677-744) from
 *   nancorrmatrix numbagg/funcs.py:338-451     nancovmatrix numbagg/funcs.py:454-532
 * signature "(n,m)->(n,n)": a batch x n_vars x n_obs, out batch x n_vars x n_vars (both
 * triangles written).  ws: nbg_pair_matrix_workspace_bytes(corr, f64, batch, n_vars, n_obs)
 * bytes of scratch (per-slice partial sums, folded in slice order), no initialisation. */
NBG_API size_t nbg_pair_matrix_workspace_bytes(int corr, int f64, long long batch, long long n_vars,
                                               long long n_obs);
#define NBG_DECL_PAIR_MATRIX(NAME, T, SFX)                                                                  \
  NBG_API int nbg_##NAME##_##SFX(const T* a, T* out, long long batch, long long n_vars, long long n_obs, void* ws, \
                                 size_t ws_bytes, void* stream);
NBG_DECL_PAIR_MATRIX(nancovmatrix, double, f64)
NBG_DECL_PAIR_MATRIX(nancovmatrix, float, f32)
NBG_DECL_PAIR_MATRIX(nancorrmatrix, double, f64)
NBG_DECL_PAIR_MATRIX(nancorrmatrix, float, f32)

/* ---- static aggregations ------------------------------------------------------------
 * Replace numbagg/funcs.py:23-159 (ndaggregate: allnan, anynan, nancount, nansum,
 * nanmean, nanvar, nanstd) and :162-242 (ndreduce: nanargmax, nanargmin, nanmax,
 * nanmin).  a is a C-contiguous (rows, m) view whose last axis holds the reduced axes
 * (moved last and flattened, numbagg/utils.py:20-32); out has rows elements:
 *   allnan / anynan   -> unsigned char (0 / 1)
 *   nancount          -> long long
 *   nanargmax / min   -> long long, the first extreme column; -1 marks a row whose
 *                        elements are all NaN (numbagg raises "All-NaN slice encountered")
 *   the others        -> the input's type (nanmean / nanvar / nanstd: float64, float32;
 *                        integer nansum wraps like the reference's integer loop)
 * nanvar / nanstd take ddof (NaN unless count > ddof and count > 0).  nanmax / nanmin / nanarg*
 * with m == 0 return NBG_INVALID_ARGUMENT (numbagg raises on an empty reduction).
 * ws: nbg_aggregate_workspace_bytes(rows, m) bytes of scratch, no initialisation.
 * The _cols entry points reduce the middle axis of a C-contiguous (outer, m, inner)
 * array in place (reduced axes that are consecutive and not last, as numbagg's gufuncs
 * read them through strides): out[o * inner + i] reduces a[(o * m + r) * inner + i]
 * over r, and nanarg* return r; ws: nbg_aggregate_cols_workspace_bytes(outer, m, inner). */
NBG_API size_t nbg_aggregate_workspace_bytes(long long rows, long long m);
NBG_API size_t nbg_aggregate_cols_workspace_bytes(long long outer, long long m, long long inner);
#define NBG_DECL_AGG(NAME, T, O, SFX)                                                                      \
  NBG_API int nbg_##NAME##_##SFX(const T* a, O* out, long long rows, long long m, void* ws, size_t ws_bytes, void* stream); \
  NBG_API int nbg_##NAME##_cols_##SFX(const T* a, O* out, long long outer, long long m, long long inner, void* ws,     \
                                      size_t ws_bytes, void* stream);
#define NBG_DECL_AGG_DDOF(NAME, T, SFX)                                                                      \
  NBG_API int nbg_##NAME##_##SFX(const T* a, T* out, long long rows, long long m, long long ddof, void* ws, \
                                 size_t ws_bytes, void* stream);                                            \
  NBG_API int nbg_##NAME##_cols_##SFX(const T* a, T* out, long long outer, long long m, long long inner,    \
                                      long long ddof, void* ws, size_t ws_bytes, void* stream);
#define NBG_DECL_AGG_ALL(NAME, O)          \
  NBG_DECL_AGG(NAME, double, O, f64)       \
  NBG_DECL_AGG(NAME, float, O, f32)        \
  NBG_DECL_AGG(NAME, int, O, i32)          \
  NBG_DECL_AGG(NAME, long long, O, i64)
#define NBG_DECL_AGG_SAME(NAME)                  \
  NBG_DECL_AGG(NAME, double, double, f64)        \
  NBG_DECL_AGG(NAME, float, float, f32)          \
  NBG_DECL_AGG(NAME, int, int, i32)              \
  NBG_DECL_AGG(NAME, long long, long long, i64)
NBG_DECL_AGG_ALL(allnan, unsigned char)
NBG_DECL_AGG_ALL(anynan, unsigned char)
NBG_DECL_AGG_ALL(nancount, long long)
NBG_DECL_AGG_SAME(nansum)
NBG_DECL_AGG(nanmean, double, double, f64)
NBG_DECL_AGG(nanmean, float, float, f32)
NBG_DECL_AGG_DDOF(nanvar, double, f64)
NBG_DECL_AGG_DDOF(nanvar, float, f32)
NBG_DECL_AGG_DDOF(nanstd, double, f64)
NBG_DECL_AGG_DDOF(nanstd, float, f32)
NBG_DECL_AGG_SAME(nanmax)
NBG_DECL_AGG_SAME(nanmin)
NBG_DECL_AGG_ALL(nanargmax, long long)
NBG_DECL_AGG_ALL(nanargmin, long long)

#ifdef __cplusplus
}
#endif

#endif /* NUMBAGG_GB300_H */
