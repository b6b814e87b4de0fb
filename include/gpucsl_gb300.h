/*
 * gpucsl_gb300 — C ABI of the GB300 (sm_103a) skeleton-discovery kernels.
 *
 * Plain pointers and sizes only.  Every buffer argument is a DEVICE pointer owned by
 * the caller (the library allocates nothing on the hot path; scratch space is a
 * caller-provided workspace whose size is given by the *_workspace_bytes query).
 * `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 * All calls enqueue work on `stream`; calls that fill a host `gcsl_stats` synchronise
 * that stream before returning.  Return value: GCSL_OK or a GCSL_ERR_* code; the
 * library never aborts and never traps on the device.
 *
 * Each entry point names the reference (hpi-epic/gpucsl) interface it replaces.
 */
#ifndef GPUCSL_GB300_H
#define GPUCSL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GCSL_ABI_VERSION 2

#define GCSL_OK 0
#define GCSL_ERR_INVALID_ARG 1
#define GCSL_ERR_WORKSPACE 2
#define GCSL_ERR_UNSUPPORTED_LEVEL 3
#define GCSL_ERR_TIMEOUT 4
#define GCSL_ERR_DEVICE 5
#define GCSL_ERR_CAPACITY 6
#define GCSL_ERR_UNSUPPORTED 7
#define GCSL_ERR_DEBUG_CHECK 8

#define GCSL_MAX_LEVELS 64
#define GCSL_DTYPE_F64 0
#define GCSL_DTYPE_F32 1
#define GCSL_DTYPE_I32 2
#define GCSL_DTYPE_I64 3
#define GCSL_DTYPE_U8 4

/* Per-level counters returned to the host. */
typedef struct gcsl_stats {
    int32_t levels_run;            /* levels executed, level 0 included */
    int32_t status;                /* device status word (GCSL_OK when clean) */
    int64_t n_records;             /* sepset records written to the record pool */
    int64_t edges[GCSL_MAX_LEVELS];     /* undirected edges alive at level start */
    int64_t tests[GCSL_MAX_LEVELS];     /* canonical executed tests */
    int64_t tests_full[GCSL_MAX_LEVELS];/* full test space sum_dir C(d-1, l) */
    int64_t removed[GCSL_MAX_LEVELS];   /* edges removed at this level */
    int32_t max_degree[GCSL_MAX_LEVELS];/* max compacted degree at level start */
    float level_ms[GCSL_MAX_LEVELS];    /* device time per level (0 when not timed) */
    int32_t debug_site;                 /* debug build: first failed index check (0 = none) */
} gcsl_stats;

/* A sepset record in the int32 record pool: [lo, hi, level, S_0 .. S_{level-1}]. */

int gcsl_version(void);
/* Where and why the last failing CUDA call of the calling thread failed (the call that
 * made an entry point return GCSL_ERR_DEVICE), e.g. "corr_ozaki_kernel launch:
 * cudaErrorLaunchOutOfResources (...)"; "" when none failed. */
const char *gcsl_last_error(void);
const char *gcsl_status_string(int status);
/* Number of kernels this library has launched in this process (instrumentation; no
 * reference counterpart). */
int64_t gcsl_kernel_launches(void);
/* Precision of gcsl_gauss_skeleton's level tests for the calling thread (no reference
 * counterpart): 0 = process default (FP32 first with FP64 where FP32 cannot decide, or
 * FP64 throughout when GCSL_F64_TESTS=1 is set), 1 = FP32 first, 2 = FP64 throughout.
 * Both give the same skeleton, sepsets, test counts and pmax; mode 2 exists to show it. */
int gcsl_set_test_precision(int32_t mode);
/* Debug build only (libgpucsl_gb300_debug.so, the reference's is_debug compile of
 * gpucsl/pc/kernel_management.py:32-33, selected by is_debug in the Python API): every
 * index its kernels derive is checked before use, a failed check returns
 * GCSL_ERR_DEBUG_CHECK with the site in gcsl_stats.debug_site instead of trapping, and
 * this call sets the order in which the calling thread's solves walk the edges of a
 * level, the units of chunked edges and the discrete tests (0 = the release order;
 * another seed reverses and rotates it).  Results must not depend on the order.  The
 * release library returns GCSL_ERR_UNSUPPORTED. */
int gcsl_debug_set_work_order(uint64_t seed);
/* Serving (no reference counterpart): caps the resident blocks per SM of the discrete
 * test kernel (a grid-stride kernel that otherwise fills every SM for the whole level)
 * launched by the calling thread; 0 = as many as fit.  A server that runs discrete
 * solves next to other work sets it so that the other work finds room on every SM.
 * Results do not depend on it. */
int gcsl_set_blocks_per_sm_cap(int32_t cap);

/* ------------------------------------------------------------ correlation (a) */
/* Replaces gpucsl/pc/helpers.py:58-59 (correlation_matrix_of = np.corrcoef(data,
 * rowvar=False)), called at gpucsl/pc/discover_skeleton_gaussian.py:134-135.
 * X: n x p samples, row-major with leading dimension ldx (>= p), FP64 or FP32
 * (dtype GCSL_DTYPE_*); C: p x p FP64 out.  FP64 arithmetic throughout. */
size_t gcsl_corr_workspace_bytes(int64_t n, int32_t p);
int gcsl_corr_f64(const void *X, int32_t dtype, int64_t n, int32_t p, int64_t ldx, double *C, void *workspace,
                  size_t workspace_bytes, void *stream);

/* Same result as gcsl_corr_f64 computed on the tcgen05 tensor cores: the centred,
 * power-of-two-scaled samples are split into seven signed 7-bit integer digits (exact in
 * BF16), digit pairs are accumulated exactly in TMEM and reduced in 64-bit integers, and
 * each covariance is rounded to FP64 once.  Deviation from an FP64 GEMM: at most about
 * 2^-48 of sum_t |x_ti||x_tj|.  A completion-wait timeout poisons C with NaN. */
size_t gcsl_corr_tc_workspace_bytes(int64_t n, int32_t p);
int gcsl_corr_f64_tc(const void *X, int32_t dtype, int64_t n, int32_t p, int64_t ldx, double *C, void *workspace,
                     size_t workspace_bytes, void *stream);
/* The two stages of gcsl_corr_f64_tc on the same workspace: column statistics and the
 * integer digit tiles (FP64 / integer work), then the tensor-core digit products,
 * their exact reduction and the normalisation into C. */
int gcsl_corr_tc_digits(const void *X, int32_t dtype, int64_t n, int32_t p, int64_t ldx, void *workspace,
                        size_t workspace_bytes, void *stream);
int gcsl_corr_tc_product(int64_t n, int32_t p, double *C, void *workspace, size_t workspace_bytes, void *stream);

/* --------------------------------------------------- Gaussian skeleton (b,c,e) */
/* Replaces the level loop of gpucsl/pc/discover_skeleton_gaussian.py:30-113
 * (gaussian_ci_worker) with the kernels of gpucsl/pc/cuda/gaussian_ci.cu:18-120,
 * compaction (gpucsl/pc/cuda/helpers/graph_helpers.cu:35-56) and the zmin->pmax
 * epilogue (gpucsl/pc/helpers.py:62-82).
 *   C            p x p FP64 correlation matrix
 *   thresholds   HOST array of n_thresholds Fisher-z thresholds (helpers.py:42-50)
 *   G            p x p uint16 skeleton out (symmetric, zero diagonal)
 *   sepsets      optional p x p x max_level int32 dense sepsets (pre-filled with -1
 *                by the caller), or NULL
 *   rec_pool     optional int32 record pool of rec_cap ints, or NULL
 *   pmax         p x p FP64 out (upper triangle p-values, -1 on/below the diagonal)
 *   stats        optional host struct; when given the call synchronises `stream`.
 * p > GCSL_GAUSS_MAX_P (pair indices i * p + j must fit in int32) returns
 * GCSL_ERR_UNSUPPORTED. */
#define GCSL_GAUSS_MAX_P 46340
size_t gcsl_gauss_workspace_bytes(int32_t p, int32_t max_level);
int gcsl_gauss_skeleton(const double *C, int32_t p, int64_t n_obs, const double *thresholds, int32_t n_thresholds,
                        int32_t max_level, uint16_t *G, int32_t *sepsets, int32_t *rec_pool, int64_t rec_cap,
                        double *pmax, gcsl_stats *stats, void *workspace, size_t workspace_bytes, void *stream);

/* Allocation-free variant of gcsl_gauss_skeleton (no counterpart in the reference).
 * For callers that cannot call cudaMalloc, e.g. a host runtime whose allocator owns
 * all device memory after start-up.  Same arguments and results as gcsl_gauss_skeleton
 * minus the workspace: the scratch space is a static device array of
 * GCSL_NOALLOC_SCRATCH_BYTES that every GPU loading the library keeps until exit.
 * p < 1 returns GCSL_ERR_INVALID_ARG, p > GCSL_NOALLOC_MAX_P GCSL_ERR_UNSUPPORTED.  The
 * first call on a device looks up the array's address (make it before any stream
 * capture; a cudaDeviceReset after it is not supported).  The call creates nothing, on
 * a thread's first call or later: no device or pinned host allocation, no stream, no
 * event.  All its kernels run in order on `stream`, and it synchronises `stream` to
 * read the level loop's control words into the calling thread's stack, so the call
 * cannot be captured into a CUDA graph.  Calls share
 * the array, so calls whose device work overlaps race and must be serialised. */
#define GCSL_NOALLOC_MAX_P 512
#define GCSL_NOALLOC_SCRATCH_BYTES 17825792
int gcsl_gauss_skeleton_noalloc(const double *C, int32_t p, int64_t n_obs, const double *thresholds,
                                int32_t n_thresholds, int32_t max_level, uint16_t *G, int32_t *sepsets,
                                int32_t *rec_pool, int64_t rec_cap, double *pmax, gcsl_stats *stats, void *stream);

/* Ordinal encoding of discrete samples on the device (replaces the host OrdinalEncoder
 * and dims of gpucsl/pc/discover_skeleton_discrete.py:38-49): per column the observed
 * values, ascending, get codes 0..k-1 and dims[j] = k.
 *   X      device n x p samples, row stride ld elements, dtype GCSL_DTYPE_I32 / I64 / U8,
 *          or F64 holding integers
 *   codes  device out, column j at codes + j * ldc (the layout gcsl_disc_skeleton reads)
 *   dims   device p uint8 out
 *   workspace  device scratch of gcsl_encode_workspace_bytes(p) bytes, 256-byte aligned
 * A column with more than 255 distinct values, a value range of 4096 or more, or a
 * non-integer value returns GCSL_ERR_UNSUPPORTED.  Synchronises `stream`. */
size_t gcsl_encode_workspace_bytes(int32_t p);
int gcsl_ordinal_encode(const void *X, int32_t dtype, int64_t n, int32_t p, int64_t ld, uint8_t *codes, int64_t ldc,
                        uint8_t *dims, void *workspace, size_t workspace_bytes, void *stream);

/* Edge orientation of a skeleton (replaces orient_edges, gpucsl/pc/edge_orientation/
 * edge_orientation.py:25-36: v-structures (v_structures.py:8-35), then Meek's rules
 * R1-R3 to a fixed point (orientation_rules.py:7-89)), with the result of the reference's
 * sequential visiting order.
 *   G        device p x p uint16 skeleton (symmetric, zero diagonal)
 *   sepsets  device p x p x sep_len int32 separating sets, -1 padded (the reference's
 *            dense layout), or NULL with sep_len = 0
 *   dag      device p x p uint8 out: dag[a * p + b] = 1 for the edge a -> b (an undirected
 *            edge has both directions)
 *   passes   optional host out: rule passes run (the last one changed nothing)
 * Synchronises `stream` once per rule pass. */
size_t gcsl_orient_workspace_bytes(int32_t p);
int gcsl_orient_edges(const uint16_t *G, int32_t p, const int32_t *sepsets, int32_t sep_len, uint8_t *dag,
                      int32_t *passes, void *workspace, size_t workspace_bytes, void *stream);

/* ---------------------------------------------------------------- batches
 * Many independent Gaussian skeletons solved together (no counterpart in the reference,
 * whose drivers solve one problem per call: discover_skeleton_gaussian.py:116-172).
 * Every kernel of the level loop runs once for the whole batch; the run enqueues work
 * only (no host reads), so it can be captured into a CUDA graph and replayed.
 *
 *   prepare  builds the device instance table inside `workspace` (synchronous; outside
 *            any capture) and fills the opaque host plan;
 *   run      enqueues the batch on `stream`: level 0, levels 1..max_level (each
 *            instance stops by the reference's rule max degree - 1 < level), pmax;
 *   collect  synchronises and writes status, levels_run, n_records, tests and retests
 *            into the instance array.
 * Precision GCSL_PREC_F64 gives results identical to gcsl_gauss_skeleton per instance.
 * GCSL_PREC_SPLIT tests in FP32 on the instance's FP32 copy C32 and repeats in FP64 the
 * tests whose p-value lies within 10 % of alpha (thresholds band_lo at 1.1 alpha and
 * band_hi at 0.9 alpha) or whose elimination meets a pivot below 1e-3: skeleton and
 * sepsets equal the FP64 ones, pmax carries the FP32 error of z*.
 * With c_err set (device double: a bound on |C - C_exact|, as written by
 * gcsl_corr_tc_batch_run_split), every split decision carries an error bound that
 * includes it; an instance with a test neither FP32 nor FP64 can decide on that C is
 * flagged (exact_rerun).  The full split sequence is
 *   gcsl_corr_tc_batch_run_split -> gcsl_gauss_batch_run ->
 *   gcsl_corr_tc_batch_run_flagged (with gcsl_gauss_batch_flags) -> gcsl_gauss_batch_rerun,
 * after which every instance's skeleton and sepsets equal those of the FP64 path on the
 * exact (seven-digit) correlation.
 * max_level <= GCSL_BATCH_MAX_LEVEL; the instances of a plan must not overlap in time
 * with another run of the same workspace. */
#define GCSL_PREC_F64 0
#define GCSL_PREC_SPLIT 1
#define GCSL_BATCH_MAX_LEVEL 12

typedef struct gcsl_gauss_instance {
    const double *C;          /* device p x p FP64 correlation */
    const float *C32;         /* device p x p FP32 copy (GCSL_PREC_SPLIT), else NULL */
    int32_t p;
    int64_t n_obs;
    const double *thresholds; /* HOST Fisher-z thresholds at alpha (helpers.py:42-50) */
    int32_t n_thresholds;
    const double *band_lo;    /* HOST thresholds at 1.1 alpha (GCSL_PREC_SPLIT), else NULL */
    const double *band_hi;    /* HOST thresholds at 0.9 alpha (GCSL_PREC_SPLIT), else NULL */
    uint16_t *G;              /* device p x p skeleton out */
    double *pmax;             /* device p x p pmax out */
    int32_t *rec_pool;        /* device sepset record pool ([lo, hi, level, S...]), or NULL */
    int64_t rec_cap;
    const double *c_err;      /* device bound on |C - C_exact| (GCSL_PREC_SPLIT on a split correlation), or NULL */
    void *state;              /* device solve state of gcsl_gauss_state_bytes(p) bytes (256-byte aligned) that
                                 persists across plans, or NULL: a slice of the batch workspace */
    int32_t status;           /* out (collect): device status of this instance */
    int32_t levels_run;       /* out (collect) */
    int64_t n_records;        /* out (collect): ints used in rec_pool (may exceed rec_cap) */
    int64_t tests;            /* out (collect): canonical executed tests, level 0 included */
    int64_t retests;          /* out (collect): FP64 re-tests of GCSL_PREC_SPLIT */
    int32_t exact_rerun;      /* out (collect): 1 when the instance needed the exact correlation */
} gcsl_gauss_instance;

typedef struct gcsl_batch_plan {
    int64_t w[48]; /* opaque */
} gcsl_batch_plan;

size_t gcsl_gauss_batch_workspace_bytes(const int32_t *p, int32_t count);
int gcsl_gauss_batch_prepare(const gcsl_gauss_instance *inst, int32_t count, int32_t max_level, int32_t precision,
                             void *workspace, size_t workspace_bytes, gcsl_batch_plan *plan, void *stream);
int gcsl_gauss_batch_run(const gcsl_batch_plan *plan, void *stream);
/* Solves again, with the exact test, the instances flagged by the last run (after their
 * exact correlation); the other instances are left as they are.  Enqueues only. */
int gcsl_gauss_batch_rerun(const gcsl_batch_plan *plan, void *stream);
/* Device array of the plan's per-instance exact_rerun flags (count int32), or NULL. */
const int32_t *gcsl_gauss_batch_flags(const gcsl_batch_plan *plan);
int gcsl_gauss_batch_collect(const gcsl_batch_plan *plan, gcsl_gauss_instance *inst, int32_t count, void *stream);
/* Autotuner hook: lanes per edge (32 or 8; 8 only for levels <= 4) of a level's test
 * kernel.  Results do not depend on it. */
int gcsl_gauss_batch_set_lanes(gcsl_batch_plan *plan, int32_t level, int32_t lanes);

/* Level-by-level stepping for continuous batching (no counterpart in the reference: a
 * server admits new problems between the levels of the ones in flight).  Instances
 * that carry their own `state` (gcsl_gauss_state_bytes(p) bytes) keep their solve state
 * there across plans, so each step's plan may group a different set of instances: those
 * due for the same levels.
 *   table_bytes       workspace of a plan whose instances all carry their state
 *   prepare_staged    as prepare, but builds the plan's tables in the caller's pinned host
 *                     buffer `stage` (table_bytes) and only enqueues their upload: the
 *                     buffer must stay untouched until the stream has passed the copy
 *   step              enqueues levels first_level..last_level of every instance of the plan
 *                     (first_level 0: the state reset and level 0 first), then with finish
 *                     the pmax write-back; instances whose loop ended skip the rest on the
 *                     device.  host_status (pinned, 4 int32 per instance, or NULL) receives
 *                     [done, last level run, status, record ints] once the stream has
 *                     passed the step.
 * Each instance's levels must be stepped in order, one plan at a time. */
size_t gcsl_gauss_state_bytes(int32_t p);
size_t gcsl_gauss_batch_table_bytes(int32_t count);
int gcsl_gauss_batch_prepare_staged(const gcsl_gauss_instance *inst, int32_t count, int32_t max_level,
                                    int32_t precision, void *workspace, size_t workspace_bytes, void *stage,
                                    size_t stage_bytes, gcsl_batch_plan *plan, void *stream);
int gcsl_gauss_batch_step(const gcsl_batch_plan *plan, int32_t first_level, int32_t last_level, int32_t finish,
                          int32_t *host_status, void *stream);

/* Host helper (replaces the dense sepset fill of gpucsl/pc/discover_skeleton_gaussian.py:
 * 166-168): scatters an int32 record pool [lo, hi, level, S...] of n_ints ints into the
 * reference's dense layout out[p][p][max_level] (host memory), -1 where no set; records
 * above max_level are skipped.  Returns GCSL_ERR_INVALID_ARG on a record that leaves
 * the pool or names a variable outside [0, p).  Runs on the calling thread(s), no GPU. */
int gcsl_records_to_dense(const int32_t *rec, int64_t n_ints, int32_t p, int32_t max_level, int32_t *out);

/* Batched tensor-core correlation (the digit-product path of gcsl_corr_f64_tc for many
 * sample matrices in one launch per stage).  X[k] is n[k] x p[k] (row stride ldx[k]),
 * all of type dtype; C[k] receives the FP64 correlation and, when C32 is not NULL and
 * C32[k] is not NULL, its FP32 copy.  prepare is synchronous; run only enqueues. */
size_t gcsl_corr_tc_batch_workspace_bytes(const int64_t *n, const int32_t *p, int32_t count);
int gcsl_corr_tc_batch_prepare(const void *const *X, int32_t dtype, const int64_t *n, const int32_t *p,
                               const int64_t *ldx, double *const *C, float *const *C32, int32_t count,
                               void *workspace, size_t workspace_bytes, gcsl_batch_plan *plan, void *stream);
int gcsl_corr_tc_batch_run(const gcsl_batch_plan *plan, void *stream);
/* Split precision (replaces np.corrcoef, gpucsl/pc/helpers.py:58-59, for the batched
 * split path): the product over the five leading digits only (15 of the 28 digit-pair
 * products); c_err (device, count doubles) receives per instance a bound eps on the
 * distance of each entry of C to the seven-digit result, eps = 2.5 * 2^-35 (1.02 w +
 * sqrt(w)) with w = n / min_i sum_t y_ti^2 (y: centred, power-of-two-scaled samples).
 * Only five digit planes are written; the flagged run writes all seven for its jobs. */
int gcsl_corr_tc_batch_run_split(const gcsl_batch_plan *plan, double *c_err, void *stream);
/* The seven digit planes, their product, diagonal and normalisation for the instances whose device
 * flag (count int32) is non-zero, on the digits of the preceding run of the plan. */
int gcsl_corr_tc_batch_run_flagged(const gcsl_batch_plan *plan, const int32_t *flags, void *stream);

/* ----------------------------------------------------- discrete skeleton (d,e) */
/* Replaces the level loop of gpucsl/pc/discover_skeleton_discrete.py:80-112 with the
 * kernels of gpucsl/pc/cuda/discrete_ci.cu:37-246 (+ helpers/discrete_helpers.cu).
 *   data         p columns of ordinal codes, column-major, column stride ld >= n
 *                (ld a multiple of 16; bytes in [n, ld) are ignored)
 *   dims         p uint8 observed cardinalities (discover_skeleton_discrete.py:49)
 *   max_dim      the largest entry of dims; it sizes each level's shared-memory tables
 *                (a larger cardinality in dims sets GCSL_ERR_UNSUPPORTED)
 *   other arguments as for gcsl_gauss_skeleton; pmax folds every test (the reference
 *   tests every rank, discrete_ci.cu:221-244). */
size_t gcsl_disc_workspace_bytes(int32_t p, int64_t n, int32_t max_level, int32_t max_dim);
int gcsl_disc_skeleton(const uint8_t *data, int64_t ld, int64_t n, int32_t p, const uint8_t *dims,
                       int32_t max_dim, double alpha, int32_t max_level, uint16_t *G, int32_t *sepsets,
                       int32_t *rec_pool, int64_t rec_cap, double *pmax, gcsl_stats *stats, void *workspace,
                       size_t workspace_bytes, void *stream);

/* ------------------------------------------------------------- unit kernels */
/* Single-kernel entry points used by the parity tests, mirroring the reference's
 * PYTHON_TEST kernels (tests/test_cuda_graph_helpers.py, test_cuda_set_helpers.py,
 * test_cuda_discrete_helpers.py). */
/* graph_helpers.cu:35-56: G (p x p uint16) -> adj (p x p int32 [deg, nbrs...]). */
int gcsl_compact(const uint16_t *G, int32_t p, int32_t *adj, void *stream);
/* set_helpers.cu:25-49: out[r * level + c] = 1-based positions of rank r, r < count. */
int gcsl_unrank(int32_t K, int32_t level, int64_t count, int32_t *out, void *stream);
/* math_helpers.cu:128-175: out[k] = pchisq(x[k], df[k]). */
int gcsl_pchisq(const double *x, const int64_t *df, int64_t count, double *out, void *stream);
/* discrete_helpers.cu:40-85 + 120-186: counts (dim_s*d_i*d_j uint32, at most counts_cap
 * are written) and chi^2 + p-value of one test; S is a host array of `level` variable
 * ids.  chi2_pvalue receives -1, -1 when the table does not fit counts_cap or the
 * shared-memory table, or when a code is not below its cardinality. */
int gcsl_disc_table(const uint8_t *data, int64_t ld, int64_t n, const uint8_t *dims, int32_t vi, int32_t vj,
                    const int32_t *S, int32_t level, uint32_t *counts, int64_t counts_cap, double *chi2_pvalue,
                    void *stream);

/* Tensor-core building block (no reference counterpart): D = A B^T with A (M x K) and
 * B (N x K) BF16 row-major, D (M x N) FP32 row-major, through tcgen05 MMAs with TMEM
 * accumulators.  M, N multiples of 128, K a multiple of 64, 16-byte aligned rows.
 * *err (device int, caller-zeroed) is set to 1 if a completion wait timed out. */
int gcsl_tc_gemm_bf16(const uint16_t *A, const uint16_t *B, float *D, int32_t M, int32_t N, int32_t K, int32_t *err,
                      void *stream);

#ifdef __cplusplus
}
#endif
#endif
