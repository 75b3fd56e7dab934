/*
 * CPU oracle for the numbagg scan / reduction hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, loop for loop, the scalar kernels of numbagg (pure-Python
 * functions compiled by numba.guvectorize) so that the GPU implementation can be
 * checked against them.  Only tests, the smoke check and the CPU-baseline leg of the
 * benchmark may load it; the product path never does.
 *
 * Typing follows numba's rules for the reference sources (no fast-math):
 *   - move_* and move_exp_* kernels: accumulators are float64 locals seeded with
 *     `0.0`, counts are int64, the output is rounded to the array dtype on store
 *     (numbagg/moving.py:16-28, numbagg/moving_exp.py:53-66);
 *   - group_* kernels accumulate in the output dtype, counts in the labels dtype
 *     (numbagg/grouped.py:9-20), selection kernels keep a float64 running extreme
 *     (numbagg/grouped.py:56, :214);
 *   - move_covmatrix / move_corrmatrix accumulate in the input dtype with int64
 *     pair counts (numbagg/moving_matrix.py:48-53, :149-152).
 * Build with -O2 -ffp-contract=off (no FMA contraction, as numba without fastmath).
 *
 * Rows are parallelised with OpenMP `schedule(static)`, which matches numba's
 * `target="parallel"` split of the gufunc loop dimension.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <stdlib.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define EXPORT __attribute__((visibility("default")))

static int orc_threads(int nthreads) {
#ifdef _OPENMP
  return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  (void)nthreads;
  return 1;
#endif
}

/* NaN stored into an integer output: numba lowers it with fptosi, which on x86-64
 * yields the "integer indefinite" value (the minimum of the type). */
#define INT_NAN_i32 INT32_MIN
#define INT_NAN_i64 INT64_MIN

/* ------------------------------------------------------------------------------ */
/* Moving windows and exponentially weighted functions (scan_loops.inc)            */
/* ------------------------------------------------------------------------------ */

#define CAT2(a, b) a##b
#define ACC double
#define ACC_SQRT sqrt
#define ONAME(f, s) CAT2(orc_##f##_, s)
#include "scan_loops.inc"
#undef ACC
#undef ACC_SQRT
#undef ONAME
#define ACC long double
#define ACC_SQRT sqrtl
#define ONAME(f, s) CAT2(orc_##f##_ext_, s)
#include "scan_loops.inc"
#undef ACC
#undef ACC_SQRT
#undef ONAME

/* ------------------------------------------------------------------------------ */
/* Fills: numbagg/funcs.py:294-326.  The carried `current` is float64 in numba     */
/* (unified from `np.nan` and the value), so the store is `(T)(double)val`.        */
/* ------------------------------------------------------------------------------ */

#define IS_NAN_F(v) isnan(v)
#define IS_NAN_I(v) 0

#define DEF_FILL(T, SFX, ISNAN)                                                        \
  EXPORT int orc_ffill_##SFX(const T* a_, T* out_, int64_t rows, int64_t n,            \
                             int64_t limit, int nthreads) {                            \
    _Pragma("omp parallel for schedule(static) num_threads(orc_threads(nthreads))")    \
    for (int64_t r = 0; r < rows; ++r) {                                               \
      const T* a = a_ + r * n; T* out = out_ + r * n;                                  \
      int64_t lives = limit; double current = NAN;                                     \
      for (int64_t i = 0; i < n; ++i) {                                                \
        T val = a[i];                                                                  \
        if (ISNAN(val)) { if (lives <= 0) current = NAN; lives -= 1; }                 \
        else { lives = limit; current = (double)val; }                                 \
        out[i] = (T)current;                                                           \
      }                                                                                \
    }                                                                                  \
    return 0;                                                                          \
  }                                                                                    \
  EXPORT int orc_bfill_##SFX(const T* a_, T* out_, int64_t rows, int64_t n,            \
                             int64_t limit, int nthreads) {                            \
    _Pragma("omp parallel for schedule(static) num_threads(orc_threads(nthreads))")    \
    for (int64_t r = 0; r < rows; ++r) {                                               \
      const T* a = a_ + r * n; T* out = out_ + r * n;                                  \
      int64_t lives = limit; double current = NAN;                                     \
      for (int64_t i = n - 1; i >= 0; --i) {                                           \
        T val = a[i];                                                                  \
        if (ISNAN(val)) { if (lives <= 0) current = NAN; lives -= 1; }                 \
        else { lives = limit; current = (double)val; }                                 \
        out[i] = (T)current;                                                           \
      }                                                                                \
    }                                                                                  \
    return 0;                                                                          \
  }

DEF_FILL(double, f64, IS_NAN_F)
DEF_FILL(float, f32, IS_NAN_F)
DEF_FILL(int32_t, i32, IS_NAN_I)
DEF_FILL(int64_t, i64, IS_NAN_I)

/* ------------------------------------------------------------------------------ */
/* Grouped reductions: numbagg/grouped.py.                                         */
/* values (rows, m) C-contiguous, labels (m,) int64 shared by every row (the        */
/* broadcast of groupndreduce, numbagg/decorators.py:661-673), out (rows, K).      */
/* A label >= K is skipped like a negative one (numba has no bounds check there).  */
/* V = values dtype, O = output dtype.                                             */
/* ------------------------------------------------------------------------------ */

/* Arithmetic in the output dtype.  numba promotes integer operands to int64 and the
 * store truncates, which equals two's-complement wrap-around in the narrow type. */
#define ADD_f64(a, b) ((double)((a) + (b)))
#define ADD_f32(a, b) ((float)((a) + (b)))
#define ADD_i32(a, b) ((int32_t)(uint32_t)((uint64_t)(int64_t)(a) + (uint64_t)(int64_t)(b)))
#define ADD_i64(a, b) ((int64_t)((uint64_t)(int64_t)(a) + (uint64_t)(int64_t)(b)))
#define MUL_f64(a, b) ((double)((a) * (b)))
#define MUL_f32(a, b) ((float)((a) * (b)))
#define MUL_i32(a, b) ((int32_t)(uint32_t)((uint64_t)(int64_t)(a) * (uint64_t)(int64_t)(b)))
#define MUL_i64(a, b) ((int64_t)((uint64_t)(int64_t)(a) * (uint64_t)(int64_t)(b)))

#define V_ISNAN_f64(v) isnan(v)
#define V_ISNAN_f32(v) isnan(v)
#define V_ISNAN_i32(v) 0
#define V_ISNAN_i64(v) 0

#define GROUP_LOOP_BEGIN(V)                                                            \
  _Pragma("omp parallel for schedule(static) num_threads(orc_threads(nthreads))")      \
  for (int64_t r = 0; r < rows; ++r) {                                                 \
    const V* values = values_ + r * m;

#define SKIP_LABEL(label) if ((label) < 0 || (label) >= K) continue;

/* group_nansum, numbagg/grouped.py:30-40 (accumulates in the values dtype) */
#define DEF_G_SUM(V, SFX)                                                              \
  EXPORT int orc_group_nansum_##SFX(const V* values_, const int64_t* labels, V* out_,  \
      int64_t rows, int64_t m, int64_t K, int64_t ddof, int nthreads) {                \
    (void)ddof;                                                                        \
    GROUP_LOOP_BEGIN(V)                                                                \
      V* out = out_ + r * K;                                                           \
      for (int64_t k = 0; k < K; ++k) out[k] = 0;                                      \
      for (int64_t j = 0; j < m; ++j) {                                                \
        int64_t label = labels[j]; SKIP_LABEL(label)                                   \
        V value = values[j];                                                           \
        if (!V_ISNAN_##SFX(value)) out[label] = ADD_##SFX(out[label], value);               \
      }                                                                                \
    }                                                                                  \
    return 0;                                                                          \
  }

/* group_nansum_of_squares, numbagg/grouped.py:135-145 */
#define DEF_G_SUMSQ(V, SFX)                                                            \
  EXPORT int orc_group_nansum_of_squares_##SFX(const V* values_,                        \
      const int64_t* labels, V* out_, int64_t rows, int64_t m, int64_t K,               \
      int64_t ddof, int nthreads) {                                                    \
    (void)ddof;                                                                        \
    GROUP_LOOP_BEGIN(V)                                                                \
      V* out = out_ + r * K;                                                           \
      for (int64_t k = 0; k < K; ++k) out[k] = 0;                                      \
      for (int64_t j = 0; j < m; ++j) {                                                \
        int64_t label = labels[j]; SKIP_LABEL(label)                                   \
        V value = values[j];                                                           \
        if (!V_ISNAN_##SFX(value)) out[label] = ADD_##SFX(out[label], MUL_##SFX(value, value));  \
      }                                                                                \
    }                                                                                  \
    return 0;                                                                          \
  }

/* group_nanprod, numbagg/grouped.py:124-132 */
#define DEF_G_PROD(V, SFX)                                                             \
  EXPORT int orc_group_nanprod_##SFX(const V* values_, const int64_t* labels, V* out_, \
      int64_t rows, int64_t m, int64_t K, int64_t ddof, int nthreads) {                \
    (void)ddof;                                                                        \
    GROUP_LOOP_BEGIN(V)                                                                \
      V* out = out_ + r * K;                                                           \
      for (int64_t k = 0; k < K; ++k) out[k] = 1;                                      \
      for (int64_t j = 0; j < m; ++j) {                                                \
        int64_t label = labels[j]; SKIP_LABEL(label)                                   \
        V value = values[j];                                                           \
        if (!V_ISNAN_##SFX(value)) out[label] = MUL_##SFX(out[label], value);               \
      }                                                                                \
    }                                                                                  \
    return 0;                                                                          \
  }

/* group_nancount, numbagg/grouped.py:43-51 (count stored in the values dtype) */
#define DEF_G_COUNT(V, SFX)                                                            \
  EXPORT int orc_group_nancount_##SFX(const V* values_, const int64_t* labels,         \
      V* out_, int64_t rows, int64_t m, int64_t K, int64_t ddof, int nthreads) {       \
    (void)ddof;                                                                        \
    GROUP_LOOP_BEGIN(V)                                                                \
      V* out = out_ + r * K;                                                           \
      for (int64_t k = 0; k < K; ++k) out[k] = 0;                                      \
      for (int64_t j = 0; j < m; ++j) {                                                \
        int64_t label = labels[j]; SKIP_LABEL(label)                                   \
        (void)values;                                                                  \
        if (!V_ISNAN_##SFX(values[j])) out[label] = ADD_##SFX(out[label], 1);               \
      }                                                                                \
    }                                                                                  \
    return 0;                                                                          \
  }

/* group_nanvar / group_nanstd, numbagg/grouped.py:148-208 */

/* group_nanargmax / group_nanargmin, numbagg/grouped.py:54-92: float64 running     */
/* extreme, strict comparison keeps the first index; the index is flat over the    */
/* core dims and starts at 0 for every row.                                        */

/* group_nanfirst / group_nanlast / group_nanmin / group_nanmax / group_nanany /    */
/* group_nanall: numbagg/grouped.py:95-121, :211-270.                               */

#define DEF_G_ROWHELPERS(V, SFX, OUT_NAN)                                              \
  static void orc_group_mean_row_##SFX(const V* values, const int64_t* labels, V* out, \
                                       int64_t m, int64_t K) {                         \
    int64_t* counts = (int64_t*)calloc((size_t)(K > 0 ? K : 1), sizeof(int64_t));      \
    for (int64_t j = 0; j < m; ++j) {                                                  \
      int64_t label = labels[j]; SKIP_LABEL(label)                                     \
      V value = values[j];                                                             \
      if (!V_ISNAN_##SFX(value)) { counts[label] += 1; out[label] = (V)(out[label] + value); } \
    }                                                                                  \
    for (int64_t k = 0; k < K; ++k) {                                                  \
      if (counts[k] == 0) out[k] = (V)NAN;                                             \
      else out[k] = (V)((double)out[k] / (double)counts[k]);                           \
    }                                                                                  \
    free(counts);                                                                      \
  }

#define DEF_G_VAR(V, SFX, NAME, STD)                                                   \
  EXPORT int orc_group_##NAME##_##SFX(const V* values_, const int64_t* labels, V* out_, \
      int64_t rows, int64_t m, int64_t K, int64_t ddof, int nthreads) {                \
    GROUP_LOOP_BEGIN(V)                                                                \
      V* out = out_ + r * K;                                                           \
      V* sums = (V*)calloc((size_t)(K > 0 ? K : 1), sizeof(V));                        \
      V* sqs = (V*)calloc((size_t)(K > 0 ? K : 1), sizeof(V));                         \
      int64_t* counts = (int64_t*)calloc((size_t)(K > 0 ? K : 1), sizeof(int64_t));    \
      for (int64_t j = 0; j < m; ++j) {                                                \
        int64_t label = labels[j]; SKIP_LABEL(label)                                   \
        V value = values[j];                                                           \
        if (!V_ISNAN_##SFX(value)) {                                                   \
          counts[label] += 1; sums[label] = (V)(sums[label] + value);                  \
          sqs[label] = (V)(sqs[label] + (V)(value * value));                           \
        }                                                                              \
      }                                                                                \
      for (int64_t k = 0; k < K; ++k) {                                                \
        int64_t count = counts[k]; int64_t denom = count - ddof;                       \
        if (denom <= 0) { out[k] = (V)NAN; continue; }                                 \
        V s2 = (V)(sums[k] * sums[k]);                                                 \
        double v = ((double)sqs[k] - (double)s2 / (double)count) / (double)denom;      \
        out[k] = (V)(STD ? sqrt(v) : v);                                               \
      }                                                                                \
      free(sums); free(sqs); free(counts);                                             \
    }                                                                                  \
    return 0;                                                                          \
  }

#define DEF_G_ARG(V, O, SFX, NAME, CMP, ONAN)                                          \
  EXPORT int orc_group_##NAME##_##SFX(const V* values_, const int64_t* labels, O* out_, \
      int64_t rows, int64_t m, int64_t K, int64_t ddof, int nthreads) {                \
    (void)ddof;                                                                        \
    GROUP_LOOP_BEGIN(V)                                                                \
      O* out = out_ + r * K;                                                           \
      double* ext = (double*)malloc((size_t)(K > 0 ? K : 1) * sizeof(double));         \
      for (int64_t k = 0; k < K; ++k) ext[k] = NAN;                                    \
      for (int64_t j = 0; j < m; ++j) {                                                \
        int64_t label = labels[j];                                                     \
        double value = (double)values[j];                                              \
        if (label >= 0 && label < K && !V_ISNAN_##SFX(values[j])) {                    \
          if (isnan(ext[label]) || value CMP ext[label]) {                             \
            ext[label] = value; out[label] = (O)j;                                     \
          }                                                                            \
        }                                                                              \
      }                                                                                \
      for (int64_t k = 0; k < K; ++k) if (isnan(ext[k])) out[k] = ONAN;                \
      free(ext);                                                                       \
    }                                                                                  \
    return 0;                                                                          \
  }

#define DEF_G_MINMAX(V, O, SFX, NAME, CMP, ONAN)                                       \
  EXPORT int orc_group_##NAME##_##SFX(const V* values_, const int64_t* labels, O* out_, \
      int64_t rows, int64_t m, int64_t K, int64_t ddof, int nthreads) {                \
    (void)ddof;                                                                        \
    GROUP_LOOP_BEGIN(V)                                                                \
      O* out = out_ + r * K;                                                           \
      double* ext = (double*)malloc((size_t)(K > 0 ? K : 1) * sizeof(double));         \
      for (int64_t k = 0; k < K; ++k) ext[k] = NAN;                                    \
      for (int64_t j = 0; j < m; ++j) {                                                \
        int64_t label = labels[j]; SKIP_LABEL(label)                                   \
        double value = (double)values[j];                                              \
        if (!V_ISNAN_##SFX(values[j]) && (isnan(ext[label]) || value CMP ext[label]))  \
          ext[label] = value;                                                          \
      }                                                                                \
      for (int64_t k = 0; k < K; ++k) out[k] = isnan(ext[k]) ? ONAN : (O)ext[k];       \
      free(ext);                                                                       \
    }                                                                                  \
    return 0;                                                                          \
  }

#define DEF_G_FIRSTLAST(V, SFX, ONAN, ISFLOAT)                                         \
  EXPORT int orc_group_nanfirst_##SFX(const V* values_, const int64_t* labels, V* out_, \
      int64_t rows, int64_t m, int64_t K, int64_t ddof, int nthreads) {                \
    (void)ddof;                                                                        \
    GROUP_LOOP_BEGIN(V)                                                                \
      V* out = out_ + r * K;                                                           \
      unsigned char* seen = (unsigned char*)calloc((size_t)(K > 0 ? K : 1), 1);        \
      for (int64_t j = 0; j < m; ++j) {                                                \
        int64_t label = labels[j]; SKIP_LABEL(label)                                   \
        if (!seen[label] && !V_ISNAN_##SFX(values[j])) {                               \
          seen[label] = 1; out[label] = values[j];                                     \
        }                                                                              \
      }                                                                                \
      /* float outputs: unseen -> NaN; integer outputs are left as the caller set them \
         (np.empty in the reference: unspecified) */                                   \
      if (ISFLOAT) for (int64_t k = 0; k < K; ++k) if (!seen[k]) out[k] = ONAN;        \
      free(seen);                                                                      \
    }                                                                                  \
    return 0;                                                                          \
  }                                                                                    \
  EXPORT int orc_group_nanlast_##SFX(const V* values_, const int64_t* labels, V* out_, \
      int64_t rows, int64_t m, int64_t K, int64_t ddof, int nthreads) {                \
    (void)ddof;                                                                        \
    GROUP_LOOP_BEGIN(V)                                                                \
      V* out = out_ + r * K;                                                           \
      for (int64_t k = 0; k < K; ++k) out[k] = ONAN;                                   \
      for (int64_t j = 0; j < m; ++j) {                                                \
        int64_t label = labels[j]; SKIP_LABEL(label)                                   \
        if (!V_ISNAN_##SFX(values[j])) out[label] = values[j];                         \
      }                                                                                \
    }                                                                                  \
    return 0;                                                                          \
  }

#define DEF_G_ANYALL(V, SFX)                                                           \
  EXPORT int orc_group_nanany_##SFX(const V* values_, const int64_t* labels, V* out_,  \
      int64_t rows, int64_t m, int64_t K, int64_t ddof, int nthreads) {                \
    (void)ddof;                                                                        \
    GROUP_LOOP_BEGIN(V)                                                                \
      V* out = out_ + r * K;                                                           \
      for (int64_t k = 0; k < K; ++k) out[k] = 0;                                      \
      for (int64_t j = 0; j < m; ++j) {                                                \
        int64_t label = labels[j]; SKIP_LABEL(label)                                   \
        V value = values[j];                                                           \
        if (!V_ISNAN_##SFX(value) && value != 0) out[label] = 1;                       \
      }                                                                                \
    }                                                                                  \
    return 0;                                                                          \
  }                                                                                    \
  EXPORT int orc_group_nanall_##SFX(const V* values_, const int64_t* labels, V* out_,  \
      int64_t rows, int64_t m, int64_t K, int64_t ddof, int nthreads) {                \
    (void)ddof;                                                                        \
    GROUP_LOOP_BEGIN(V)                                                                \
      V* out = out_ + r * K;                                                           \
      for (int64_t k = 0; k < K; ++k) out[k] = 1;                                      \
      for (int64_t j = 0; j < m; ++j) {                                                \
        int64_t label = labels[j]; SKIP_LABEL(label)                                   \
        V value = values[j];                                                           \
        if (!V_ISNAN_##SFX(value) && value == 0) out[label] = 0;                       \
      }                                                                                \
    }                                                                                  \
    return 0;                                                                          \
  }

#define DEF_GROUP_ALL_FLOAT(V, SFX)                                                    \
  DEF_G_SUM(V, SFX) DEF_G_SUMSQ(V, SFX) DEF_G_PROD(V, SFX) DEF_G_COUNT(V, SFX)         \
  DEF_G_ROWHELPERS(V, SFX, NAN)                                                        \
  EXPORT int orc_group_nanmean_##SFX(const V* values_, const int64_t* labels, V* out_, \
      int64_t rows, int64_t m, int64_t K, int64_t ddof, int nthreads) {                \
    (void)ddof;                                                                        \
    GROUP_LOOP_BEGIN(V)                                                                \
      V* out = out_ + r * K;                                                           \
      for (int64_t k = 0; k < K; ++k) out[k] = 0;                                      \
      orc_group_mean_row_##SFX(values, labels, out, m, K);                             \
    }                                                                                  \
    return 0;                                                                          \
  }                                                                                    \
  DEF_G_VAR(V, SFX, nanvar, 0) DEF_G_VAR(V, SFX, nanstd, 1)                            \
  DEF_G_ARG(V, V, SFX, nanargmax, >, (V)NAN) DEF_G_ARG(V, V, SFX, nanargmin, <, (V)NAN) \
  DEF_G_MINMAX(V, V, SFX, nanmax, >, (V)NAN) DEF_G_MINMAX(V, V, SFX, nanmin, <, (V)NAN) \
  DEF_G_FIRSTLAST(V, SFX, (V)NAN, 1) DEF_G_ANYALL(V, SFX)

#define DEF_GROUP_ALL_INT(V, SFX, INAN)                                                \
  DEF_G_SUM(V, SFX) DEF_G_SUMSQ(V, SFX) DEF_G_PROD(V, SFX) DEF_G_COUNT(V, SFX)         \
  DEF_G_ARG(V, V, SFX, nanargmax, >, INAN) DEF_G_ARG(V, V, SFX, nanargmin, <, INAN)    \
  DEF_G_MINMAX(V, V, SFX, nanmax, >, INAN) DEF_G_MINMAX(V, V, SFX, nanmin, <, INAN)    \
  DEF_G_FIRSTLAST(V, SFX, INAN, 0) DEF_G_ANYALL(V, SFX)

DEF_GROUP_ALL_FLOAT(double, f64)
DEF_GROUP_ALL_FLOAT(float, f32)
DEF_GROUP_ALL_INT(int32_t, i32, INT_NAN_i32)
DEF_GROUP_ALL_INT(int64_t, i64, INT_NAN_i64)

/* ------------------------------------------------------------------------------ */
/* Moving matrices: numbagg/moving_matrix.py:16-201.  a (batch, T, V) C-contiguous, */
/* out (batch, T, V, V).  Accumulators in the input dtype, pair counts int64.       */
/* ------------------------------------------------------------------------------ */

#define DEF_MOVE_MATRIX(T, SFX)                                                        \
  EXPORT int orc_move_covmatrix_##SFX(const T* a_, T* out_, int64_t batch,             \
      int64_t n_obs, int64_t n_vars, int64_t window, int64_t min_count, int nthreads) { \
    int64_t VV = n_vars * n_vars;                                                      \
    _Pragma("omp parallel for schedule(static) num_threads(orc_threads(nthreads))")    \
    for (int64_t bi = 0; bi < batch; ++bi) {                                           \
      const T* a = a_ + bi * n_obs * n_vars; T* out = out_ + bi * n_obs * VV;          \
      int64_t mc = min_count > 1 ? min_count : 1;                                      \
      T* sums_i = (T*)calloc((size_t)VV + 1, sizeof(T));                               \
      T* sums_j = (T*)calloc((size_t)VV + 1, sizeof(T));                               \
      T* prods = (T*)calloc((size_t)VV + 1, sizeof(T));                                \
      int64_t* pc = (int64_t*)calloc((size_t)VV + 1, sizeof(int64_t));                 \
      for (int64_t t = 0; t < n_obs; ++t) {                                            \
        if (t >= window) {                                                             \
          const T* o = a + (t - window) * n_vars;                                      \
          for (int64_t i = 0; i < n_vars; ++i) {                                       \
            T vi = o[i]; if (isnan(vi)) continue;                                      \
            for (int64_t j = 0; j < n_vars; ++j) {                                     \
              T vj = o[j]; if (isnan(vj)) continue;                                    \
              int64_t q = i * n_vars + j;                                              \
              sums_i[q] = (T)(sums_i[q] - vi); sums_j[q] = (T)(sums_j[q] - vj);        \
              prods[q] = (T)(prods[q] - (T)(vi * vj)); pc[q] -= 1;                     \
            }                                                                          \
          }                                                                            \
        }                                                                              \
        const T* nw = a + t * n_vars;                                                  \
        for (int64_t i = 0; i < n_vars; ++i) {                                         \
          T vi = nw[i]; if (isnan(vi)) continue;                                       \
          for (int64_t j = 0; j < n_vars; ++j) {                                       \
            T vj = nw[j]; if (isnan(vj)) continue;                                     \
            int64_t q = i * n_vars + j;                                                \
            sums_i[q] = (T)(sums_i[q] + vi); sums_j[q] = (T)(sums_j[q] + vj);          \
            prods[q] = (T)(prods[q] + (T)(vi * vj)); pc[q] += 1;                       \
          }                                                                            \
        }                                                                              \
        T* ot = out + t * VV;                                                          \
        for (int64_t q = 0; q < VV; ++q) {                                             \
          int64_t nn = pc[q];                                                          \
          if (nn >= mc && nn > 1) {                                                    \
            double dn = (double)nn;                                                    \
            double mean_i = (double)sums_i[q] / dn, mean_j = (double)sums_j[q] / dn;   \
            double cov = ((double)prods[q] / dn - mean_i * mean_j) * dn / (double)(nn - 1); \
            ot[q] = (T)cov;                                                            \
          } else {                                                                     \
            ot[q] = (T)NAN;                                                            \
          }                                                                            \
        }                                                                              \
      }                                                                                \
      free(sums_i); free(sums_j); free(prods); free(pc);                               \
    }                                                                                  \
    return 0;                                                                          \
  }                                                                                    \
  EXPORT int orc_move_corrmatrix_##SFX(const T* a_, T* out_, int64_t batch,            \
      int64_t n_obs, int64_t n_vars, int64_t window, int64_t min_count, int nthreads) { \
    int64_t VV = n_vars * n_vars;                                                      \
    _Pragma("omp parallel for schedule(static) num_threads(orc_threads(nthreads))")    \
    for (int64_t bi = 0; bi < batch; ++bi) {                                           \
      const T* a = a_ + bi * n_obs * n_vars; T* out = out_ + bi * n_obs * VV;          \
      int64_t mc = min_count > 1 ? min_count : 1;                                      \
      int64_t mc2 = mc > 2 ? mc : 2;                                                   \
      T* si = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* sj = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* qi = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* qj = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* pr = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      int64_t* pc = (int64_t*)calloc((size_t)VV + 1, sizeof(int64_t));                 \
      for (int64_t t = 0; t < n_obs; ++t) {                                            \
        if (t >= window) {                                                             \
          const T* o = a + (t - window) * n_vars;                                      \
          for (int64_t i = 0; i < n_vars; ++i) {                                       \
            T vi = o[i]; if (isnan(vi)) continue;                                      \
            for (int64_t j = 0; j < n_vars; ++j) {                                     \
              T vj = o[j]; if (isnan(vj)) continue;                                    \
              int64_t q = i * n_vars + j;                                              \
              si[q] = (T)(si[q] - vi); sj[q] = (T)(sj[q] - vj);                        \
              qi[q] = (T)(qi[q] - (T)(vi * vi)); qj[q] = (T)(qj[q] - (T)(vj * vj));    \
              pr[q] = (T)(pr[q] - (T)(vi * vj)); pc[q] -= 1;                           \
            }                                                                          \
          }                                                                            \
        }                                                                              \
        const T* nw = a + t * n_vars;                                                  \
        for (int64_t i = 0; i < n_vars; ++i) {                                         \
          T vi = nw[i]; if (isnan(vi)) continue;                                       \
          for (int64_t j = 0; j < n_vars; ++j) {                                       \
            T vj = nw[j]; if (isnan(vj)) continue;                                     \
            int64_t q = i * n_vars + j;                                                \
            si[q] = (T)(si[q] + vi); sj[q] = (T)(sj[q] + vj);                          \
            qi[q] = (T)(qi[q] + (T)(vi * vi)); qj[q] = (T)(qj[q] + (T)(vj * vj));      \
            pr[q] = (T)(pr[q] + (T)(vi * vj)); pc[q] += 1;                             \
          }                                                                            \
        }                                                                              \
        T* ot = out + t * VV;                                                          \
        for (int64_t q = 0; q < VV; ++q) {                                             \
          int64_t nn = pc[q];                                                          \
          if (nn >= mc2) {                                                             \
            double dn = (double)nn;                                                    \
            double mean_i = (double)si[q] / dn, mean_j = (double)sj[q] / dn;           \
            double var_i = (double)qi[q] / dn - mean_i * mean_i;                       \
            double var_j = (double)qj[q] / dn - mean_j * mean_j;                       \
            double cov = (double)pr[q] / dn - mean_i * mean_j;                         \
            ot[q] = (T)((var_i > 0 && var_j > 0) ? cov / sqrt(var_i * var_j) : NAN);   \
          } else {                                                                     \
            ot[q] = (T)NAN;                                                            \
          }                                                                            \
        }                                                                              \
      }                                                                                \
      free(si); free(sj); free(qi); free(qj); free(pr); free(pc);                      \
    }                                                                                  \
    return 0;                                                                          \
  }

DEF_MOVE_MATRIX(double, f64)
DEF_MOVE_MATRIX(float, f32)
/* extended precision (long double arrays and accumulators) */
DEF_MOVE_MATRIX(long double, ld)

/* ------------------------------------------------------------------------------ */
/* Exponentially weighted moving matrices: numbagg/moving_matrix.py:204-432.        */
/* a (batch, T, V) C-contiguous; alpha: T values per batch entry, batch entry b at   */
/* alpha_ + b * alpha_stride (stride 0: shared); out (batch, T, V, V).  The pair     */
/* states are arrays of the input dtype (:245-263, :371-383).  `decay = 1.0 -        */
/* alpha_t` is float64 in numba even for float32 input (a float64 literal minus a    */
/* float32), so each state is multiplied in D and stored back in T; the additions    */
/* of values and of alpha_t stay in T.  The finalisation follows the same typing:    */
/* `1 - f32` and `f32 / bias` are float64, the means and biased moments are T.      */
/* ------------------------------------------------------------------------------ */
#define DEF_EXP_MATRIX(T, D, SFX, SQRT)                                                \
  EXPORT int orc_move_exp_nancovmatrix_##SFX(const T* a_, const T* alpha_,            \
      int64_t alpha_stride, T min_weight, T* out_, int64_t batch, int64_t n_obs,       \
      int64_t n_vars, int nthreads) {                                                  \
    int64_t VV = n_vars * n_vars;                                                      \
    _Pragma("omp parallel for schedule(static) num_threads(orc_threads(nthreads))")    \
    for (int64_t bi = 0; bi < batch; ++bi) {                                           \
      const T* a = a_ + bi * n_obs * n_vars; const T* al = alpha_ + bi * alpha_stride; \
      T* out = out_ + bi * n_obs * VV;                                                 \
      T* si = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* sj = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* pr = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* pw = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* sw = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* sw2 = (T*)calloc((size_t)VV + 1, sizeof(T));                                  \
      for (int64_t t = 0; t < n_obs; ++t) {                                            \
        T alpha_t = al[t];                                                             \
        D decay = (D)1.0 - (D)alpha_t, decay2 = decay * decay;                         \
        for (int64_t q = 0; q < VV; ++q) {                                             \
          si[q] = (T)((D)si[q] * decay); sj[q] = (T)((D)sj[q] * decay);                \
          pr[q] = (T)((D)pr[q] * decay); pw[q] = (T)((D)pw[q] * decay);                \
          sw[q] = (T)((D)sw[q] * decay); sw2[q] = (T)((D)sw2[q] * decay2);             \
        }                                                                              \
        const T* nw = a + t * n_vars;                                                  \
        for (int64_t i = 0; i < n_vars; ++i) {                                         \
          T vi = nw[i]; if (isnan(vi)) continue;                                       \
          for (int64_t j = 0; j < n_vars; ++j) {                                       \
            T vj = nw[j]; if (isnan(vj)) continue;                                     \
            int64_t q = i * n_vars + j;                                                \
            si[q] = (T)(si[q] + vi); sj[q] = (T)(sj[q] + vj);                          \
            pr[q] = (T)(pr[q] + (T)(vi * vj)); pw[q] = (T)(pw[q] + alpha_t);           \
            sw[q] = (T)((D)sw[q] + (D)1.0); sw2[q] = (T)((D)sw2[q] + (D)1.0);          \
          }                                                                            \
        }                                                                              \
        T* ot = out + t * VV;                                                          \
        for (int64_t q = 0; q < VV; ++q) {                                             \
          T n = sw[q];                                                                 \
          D bias = n > 0 ? (D)1 - (D)(T)(sw2[q] / (T)(n * n)) : (D)0.0;                \
          if (pw[q] >= min_weight && bias > 0) {                                       \
            T mi = (T)(si[q] / n), mj = (T)(sj[q] / n);                                \
            T cb = (T)((T)(pr[q] / n) - (T)(mi * mj));                                 \
            ot[q] = (T)((D)cb / bias);                                                 \
          } else {                                                                     \
            ot[q] = (T)NAN;                                                            \
          }                                                                            \
        }                                                                              \
      }                                                                                \
      free(si); free(sj); free(pr); free(pw); free(sw); free(sw2);                     \
    }                                                                                  \
    return 0;                                                                          \
  }                                                                                    \
  EXPORT int orc_move_exp_nancorrmatrix_##SFX(const T* a_, const T* alpha_,           \
      int64_t alpha_stride, T min_weight, T* out_, int64_t batch, int64_t n_obs,       \
      int64_t n_vars, int nthreads) {                                                  \
    int64_t VV = n_vars * n_vars;                                                      \
    _Pragma("omp parallel for schedule(static) num_threads(orc_threads(nthreads))")    \
    for (int64_t bi = 0; bi < batch; ++bi) {                                           \
      const T* a = a_ + bi * n_obs * n_vars; const T* al = alpha_ + bi * alpha_stride; \
      T* out = out_ + bi * n_obs * VV;                                                 \
      T* si = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* sj = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* qi = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* qj = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* pr = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* pw = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* sw = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* sw2 = (T*)calloc((size_t)VV + 1, sizeof(T));                                  \
      for (int64_t t = 0; t < n_obs; ++t) {                                            \
        T alpha_t = al[t];                                                             \
        D decay = (D)1.0 - (D)alpha_t, decay2 = decay * decay;                         \
        for (int64_t q = 0; q < VV; ++q) {                                             \
          si[q] = (T)((D)si[q] * decay); sj[q] = (T)((D)sj[q] * decay);                \
          qi[q] = (T)((D)qi[q] * decay); qj[q] = (T)((D)qj[q] * decay);                \
          pr[q] = (T)((D)pr[q] * decay); pw[q] = (T)((D)pw[q] * decay);                \
          sw[q] = (T)((D)sw[q] * decay); sw2[q] = (T)((D)sw2[q] * decay2);             \
        }                                                                              \
        const T* nw = a + t * n_vars;                                                  \
        for (int64_t i = 0; i < n_vars; ++i) {                                         \
          T vi = nw[i]; if (isnan(vi)) continue;                                       \
          for (int64_t j = 0; j < n_vars; ++j) {                                       \
            T vj = nw[j]; if (isnan(vj)) continue;                                     \
            int64_t q = i * n_vars + j;                                                \
            si[q] = (T)(si[q] + vi); sj[q] = (T)(sj[q] + vj);                          \
            qi[q] = (T)(qi[q] + (T)(vi * vi)); qj[q] = (T)(qj[q] + (T)(vj * vj));      \
            pr[q] = (T)(pr[q] + (T)(vi * vj)); pw[q] = (T)(pw[q] + alpha_t);           \
            sw[q] = (T)((D)sw[q] + (D)1.0); sw2[q] = (T)((D)sw2[q] + (D)1.0);          \
          }                                                                            \
        }                                                                              \
        T* ot = out + t * VV;                                                          \
        for (int64_t q = 0; q < VV; ++q) {                                             \
          T n = sw[q];                                                                 \
          D bias = n > 0 ? (D)1 - (D)(T)(sw2[q] / (T)(n * n)) : (D)0.0;                \
          if (pw[q] >= min_weight && bias > 0) {                                       \
            T mi = (T)(si[q] / n), mj = (T)(sj[q] / n);                                \
            T vib = (T)((T)(qi[q] / n) - (T)(mi * mi));                                \
            T vjb = (T)((T)(qj[q] / n) - (T)(mj * mj));                                \
            T cb = (T)((T)(pr[q] / n) - (T)(mi * mj));                                 \
            D vi = (D)vib / bias, vj = (D)vjb / bias, cv = (D)cb / bias;               \
            ot[q] = (T)((vi > 0 && vj > 0) ? cv / SQRT(vi * vj) : (D)NAN);             \
          } else {                                                                     \
            ot[q] = (T)NAN;                                                            \
          }                                                                            \
        }                                                                              \
      }                                                                                \
      free(si); free(sj); free(qi); free(qj); free(pr); free(pw); free(sw); free(sw2); \
    }                                                                                  \
    return 0;                                                                          \
  }

DEF_EXP_MATRIX(double, double, f64, sqrt)
DEF_EXP_MATRIX(float, double, f32, sqrt)
DEF_EXP_MATRIX(long double, long double, ld, sqrtl)

/* ------------------------------------------------------------------------------ */
/* Static pairwise-complete matrices: numbagg/funcs.py:338-532.  a (batch, V, n_obs) */
/* C-contiguous, out (batch, V, V).  Sums in the input dtype over the upper          */
/* triangle, observation by observation (:414-430, :508-520), int64 counts; the     */
/* finalisation divides a T sum by an int64 count, which numba types as float64     */
/* (:433-456, :523-532).                                                             */
/* ------------------------------------------------------------------------------ */
#define DEF_STATIC_MATRIX(T, D, SFX, SQRT)                                             \
  EXPORT int orc_nancovmatrix_##SFX(const T* a_, T* out_, int64_t batch,              \
      int64_t n_vars, int64_t n_obs, int nthreads) {                                   \
    int64_t VV = n_vars * n_vars;                                                      \
    _Pragma("omp parallel for schedule(static) num_threads(orc_threads(nthreads))")    \
    for (int64_t bi = 0; bi < batch; ++bi) {                                           \
      const T* a = a_ + bi * n_vars * n_obs; T* out = out_ + bi * VV;                  \
      T* si = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* sj = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* sij = (T*)calloc((size_t)VV + 1, sizeof(T));                                  \
      int64_t* cnt = (int64_t*)calloc((size_t)VV + 1, sizeof(int64_t));                \
      for (int64_t k = 0; k < n_obs; ++k) {                                            \
        for (int64_t i = 0; i < n_vars; ++i) {                                         \
          T vi = a[i * n_obs + k]; if (isnan(vi)) continue;                            \
          for (int64_t j = i; j < n_vars; ++j) {                                       \
            T vj = a[j * n_obs + k]; if (isnan(vj)) continue;                          \
            int64_t q = i * n_vars + j;                                                \
            si[q] = (T)(si[q] + vi); sj[q] = (T)(sj[q] + vj);                          \
            sij[q] = (T)(sij[q] + (T)(vi * vj)); cnt[q] += 1;                          \
          }                                                                            \
        }                                                                              \
      }                                                                                \
      for (int64_t i = 0; i < n_vars; ++i) {                                           \
        for (int64_t j = i; j < n_vars; ++j) {                                         \
          int64_t q = i * n_vars + j, c = cnt[q];                                      \
          T r;                                                                         \
          if (c > 1) {                                                                 \
            D dc = (D)c;                                                               \
            D mi = (D)si[q] / dc, mj = (D)sj[q] / dc;                                  \
            D cov = (D)sij[q] / dc - mi * mj;                                          \
            r = (T)(cov * dc / (D)(c - 1));                                            \
          } else {                                                                     \
            r = (T)NAN;                                                                \
          }                                                                            \
          out[q] = r; out[j * n_vars + i] = r;                                         \
        }                                                                              \
      }                                                                                \
      free(si); free(sj); free(sij); free(cnt);                                        \
    }                                                                                  \
    return 0;                                                                          \
  }                                                                                    \
  EXPORT int orc_nancorrmatrix_##SFX(const T* a_, T* out_, int64_t batch,             \
      int64_t n_vars, int64_t n_obs, int nthreads) {                                   \
    int64_t VV = n_vars * n_vars;                                                      \
    _Pragma("omp parallel for schedule(static) num_threads(orc_threads(nthreads))")    \
    for (int64_t bi = 0; bi < batch; ++bi) {                                           \
      const T* a = a_ + bi * n_vars * n_obs; T* out = out_ + bi * VV;                  \
      T* si = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* sj = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* qi = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* qj = (T*)calloc((size_t)VV + 1, sizeof(T));                                   \
      T* sij = (T*)calloc((size_t)VV + 1, sizeof(T));                                  \
      int64_t* cnt = (int64_t*)calloc((size_t)VV + 1, sizeof(int64_t));                \
      for (int64_t k = 0; k < n_obs; ++k) {                                            \
        for (int64_t i = 0; i < n_vars; ++i) {                                         \
          T vi = a[i * n_obs + k]; if (isnan(vi)) continue;                            \
          for (int64_t j = i; j < n_vars; ++j) {                                       \
            T vj = a[j * n_obs + k]; if (isnan(vj)) continue;                          \
            int64_t q = i * n_vars + j;                                                \
            si[q] = (T)(si[q] + vi); sj[q] = (T)(sj[q] + vj);                          \
            qi[q] = (T)(qi[q] + (T)(vi * vi)); qj[q] = (T)(qj[q] + (T)(vj * vj));      \
            sij[q] = (T)(sij[q] + (T)(vi * vj)); cnt[q] += 1;                          \
          }                                                                            \
        }                                                                              \
      }                                                                                \
      for (int64_t i = 0; i < n_vars; ++i) {                                           \
        for (int64_t j = i; j < n_vars; ++j) {                                         \
          int64_t q = i * n_vars + j, c = cnt[q];                                      \
          T r = (T)NAN;                                                                \
          if (c > 1) {                                                                 \
            D dc = (D)c;                                                               \
            D mi = (D)si[q] / dc, mj = (D)sj[q] / dc;                                  \
            D vi = (D)qi[q] / dc - mi * mi, vj = (D)qj[q] / dc - mj * mj;              \
            D viu = vi * dc / (D)(c - 1), vju = vj * dc / (D)(c - 1);                  \
            D cov = (D)sij[q] / dc - mi * mj;                                          \
            D covu = cov * dc / (D)(c - 1);                                            \
            if (viu > 0 && vju > 0) r = (T)(covu / SQRT(viu * vju));                   \
          }                                                                            \
          out[q] = r; out[j * n_vars + i] = r;                                         \
        }                                                                              \
      }                                                                                \
      free(si); free(sj); free(qi); free(qj); free(sij); free(cnt);                    \
    }                                                                                  \
    return 0;                                                                          \
  }

DEF_STATIC_MATRIX(double, double, f64, sqrt)
DEF_STATIC_MATRIX(float, double, f32, sqrt)
DEF_STATIC_MATRIX(long double, long double, ld, sqrtl)
