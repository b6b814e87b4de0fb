// Shared device helpers of the skeleton-discovery kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <atomic>
#include <cmath>
#include <stdint.h>

#include "../../include/gpucsl_gb300.h"

#define GCSL_WARP 32
#define GCSL_FULL_MASK 0xffffffffu
#define GCSL_KEY_NONE 0xffffffffffffffffull
// Largest conditioning-set size with a register-resident Gaussian test; larger
// levels run the shared-memory kernel.
#define GCSL_GAUSS_REG_LEVELS 12
// Ranks per direction must stay below this bound (keys are rank << 1 | dir).
#define GCSL_RANK_LIMIT (1ll << 56)

namespace gcsl {
namespace host {
// Count of kernels this library has launched (process-wide, for instrumentation).
void note_launch(int kernels);
// Records the first failing CUDA call of the calling thread's current entry point (kept
// for gcsl_last_error) and returns e.
cudaError_t note_error(const char *where, cudaError_t e);
// The calling thread's work-order seed of the debug build (gcsl_debug_set_work_order; 0
// in the release build).
unsigned long long work_order_seed();
// The calling thread's cap on resident blocks per SM of the long grid-stride test kernel
// (gcsl_set_blocks_per_sm_cap; 0 = as many as fit).
int blocks_per_sm_cap();
// Modes of a batched correlation run (corr_tc.cu): every job with seven digits; every job
// with five digits and an error bound; only flagged jobs, seven digits, on the digits of
// a previous run.
enum CorrBatchMode { CORR_BATCH_EXACT = 0, CORR_BATCH_SPLIT = 1, CORR_BATCH_FLAGGED = 2 };
// The Gaussian skeleton solve behind gcsl_gauss_skeleton (capi.cu).  With
// allocation_free set it creates nothing: no side stream, no event, no pinned host
// word; all its work goes on `stream` and the level loop's control words are read
// into the calling thread's stack.
int gauss_skeleton_run(const double *C, int p, long long n_obs, const double *thresholds, int n_thresholds,
                       int max_level, uint16_t *G, int *sepsets, int *rec_pool, long long rec_cap, double *pmax,
                       gcsl_stats *stats, void *workspace, size_t workspace_bytes, void *stream, bool allocation_free);
}  // namespace host

// Level-0 decision bounds on the bit pattern of |r| (non-negative doubles order like
// their bit patterns): |r| < lo removes and hi <= |r| < one keeps without any FP64
// arithmetic; everything else (the knife edge around tanh(tau0), |r| >= 1, NaN) takes
// the reference's logarithm.  lo and hi leave a band of 2e-12 relative in r^2 around
// tanh(tau0)^2, wider than the band inside which r^2 < tanh(tau0)^2 and the logarithm
// can disagree.
struct L0Bounds {
    unsigned long long lo, hi, one;
};

__host__ inline L0Bounds level0_bounds(double t0sq) {
    // first b in [0, bits of 1.0] with fl(x(b)^2) > target (monotone in b)
    auto first_above = [](double target) {
        unsigned long long a = 0, b = 0x3ff0000000000000ull;
        while (a < b) {
            const unsigned long long m = a + (b - a) / 2;
            double x;
            __builtin_memcpy(&x, &m, 8);
            if (x * x > target) b = m;
            else a = m + 1;
        }
        return a;
    };
    L0Bounds B;
    B.lo = t0sq > 0.0 ? first_above(t0sq * (1.0 - 2e-12)) : 0ull;  // t0sq = 0 removes nothing
    B.hi = first_above(t0sq * (1.0 + 2e-12));
    B.one = first_above(std::nextafter(1.0, 0.0));  // fl(x^2) < 1 below it
    return B;
}

// fl32(v) rounded to nearest even, from the bits (results in the normal float range;
// others, and NaN / inf, through the conversion instruction): integer work instead of a
// conversion on the FP64 pipe, which is 1/64 of the FP32 pipe on GB300.
__device__ __forceinline__ float f64_to_f32_rn(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    if (e < -126 || e > 127) return (float)v;
    const unsigned long long m = b & 0xfffffffffffffull;
    unsigned r = (unsigned)(m >> 29);
    const unsigned long long rem = m & ((1ull << 29) - 1ull), half = 1ull << 28;
    r += (rem > half || (rem == half && (r & 1u))) ? 1u : 0u;
    const unsigned fb = ((unsigned)(b >> 63) << 31) | (((unsigned)(e + 127) << 23) + r);  // a carry bumps the exponent
    return __uint_as_float(fb);
}

// Programmatic dependent launch.  A kernel launched by launch_pdl may begin while the
// kernel before it in the stream is still running: it must call pdl_wait() before it
// reads anything that kernel wrote (a no-op when launched normally), and pdl_trigger()
// lets the kernel after it begin early in turn.  The waits are the hardware's grid
// dependency, which ends when the previous grid has completed.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
__host__ inline cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                                       Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// Raises `kernel`'s dynamic shared-memory limit to everything the device allows next to
// its static shared memory, once per device (bit d of `mask`).  The attribute belongs to
// the context, not to a host thread: raising it to one fixed maximum means concurrent
// solves never lower it under each other's launches.
template <typename K>
__host__ inline cudaError_t raise_dyn_smem_limit(K kernel, std::atomic<unsigned long long> &mask) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) return e;
    if ((mask.load() >> dev) & 1ull) return cudaSuccess;
    cudaFuncAttributes fa;
    int optin = 0;
    e = cudaFuncGetAttributes(&fa, kernel);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
    if (e == cudaSuccess) mask.fetch_or(1ull << dev);
    return e;
}

// Device-side state of one skeleton solve.  Per-level slots are written once per
// level, so no counter has to be reset between levels.
struct DevState {
    int32_t status;                          // first error code seen on the device
    int32_t done;                            // level loop finished (sticky)
    int32_t last_level;                      // highest level whose tests ran
    int32_t n_kept;                          // pairs kept at level 0 (Gaussian)
    int32_t debug_site;                      // first failed check of the debug build (GCSL_DCHECK_*), 0 if none
    int32_t reserved_;
    int32_t max_degree[GCSL_MAX_LEVELS];     // max compacted degree at level start
    unsigned long long edges[GCSL_MAX_LEVELS];
    unsigned long long tests[GCSL_MAX_LEVELS];
    unsigned long long tests_full[GCSL_MAX_LEVELS];
    unsigned long long removed[GCSL_MAX_LEVELS];
    unsigned long long n_rec_ints;           // ints used in the record pool
    unsigned long long retests;              // FP64 re-tests of the split-precision path
    unsigned long long cand_ints[GCSL_MAX_LEVELS];  // ints queued for the FP64 z* candidate kernel
    unsigned long long heavy[GCSL_MAX_LEVELS];      // chunked edges registered per level
    unsigned long long units[GCSL_MAX_LEVELS];      // key units reserved per level
};

// Chunked edges of a Gaussian level (the unit kernel walks their keys from key k0 -- 32
// after a first step walked by the level kernel, 0 when the level kernel hands over the
// whole edge -- in parallel units of 32 keys; the last unit of an edge combines them).
struct HeavyEdge {
    int lo, hi;
    long long T;
    long long unit_base;  // units unit_base .. unit_base + n_units - 1 (keys k0 + 32 k ..)
    int n_units;
    int done;             // units finished (atomic)
    long long best;       // smallest removing key found so far (atomic min; T when none)
    double r2_0, ze_0;    // minima of the first step (no remover there; +inf when k0 = 0)
    double floor;         // the pair's exact rho^2 minimum before the level
    int k0;               // first key of the units (0 or one step)
    int degs;             // compacted degrees of lo (low 16 bits) and hi (high 16 bits), p <= 46340
};

struct UnitRes {
    long long first;  // first removing key of the unit (its end when none)
    double r2, ze;    // minima over the unit's keys up to `first`
};

struct ChunkBufs {
    HeavyEdge *heavy;
    long long *chunk_first;  // canonical remover of each chunked edge (T when none)
    long long heavy_cap;
    int *unit_h;             // chunked edge of each unit (-1: unused slot)
    UnitRes *units;
    long long unit_cap;
};

// Arguments of one discrete test-kernel launch.
struct DiscLevelArgs {
    const uint8_t *data;      // column-major codes, column stride ld
    long long ld, n;
    int p;
    const uint8_t *dims;
    double alpha;
    int level;
    const int *adj;
    const long long *prefix;  // per-row weighted prefix of the flattened test list
    uint16_t *G;
    double *pmax;
    unsigned long long *win;  // canonical remover key per (lo, hi)
    int table_cap;            // counters of shared memory for the table and its replicas
    int part_cap;             // strata of the per-stratum statistic buffer (after the table)
    DevState *st;
    unsigned long long order = 0;  // work order of the debug build (0: launch order)
};

__device__ __forceinline__ void set_status(DevState *st, int code) { atomicCAS(&st->status, 0, code); }

// ------------------------------------------------------------ debug build
// The library built with GCSL_DEBUG_CHECKS=1 (selected by the reference's is_debug,
// kernel_management.py:32-33) checks the indices its kernels derive before using them:
// a failed check sets GCSL_ERR_DEBUG_CHECK and the site below in the solve's state and
// the access is redirected to a valid index (never a trap).  It also walks the work of
// the level and test loops in a permuted order (gcsl_debug_set_work_order), which must
// not change any result.
#ifndef GCSL_DEBUG_CHECKS
#define GCSL_DEBUG_CHECKS 0
#endif
enum {
    GCSL_DCHECK_EDGE = 1,      // an edge of the level's list outside [0, p) or not lo < hi
    GCSL_DCHECK_POSITION = 2,  // an unranked position outside [1, K]
    GCSL_DCHECK_SET = 3,       // a conditioning variable outside [0, p), equal to v_i / v_j, or unsorted
    GCSL_DCHECK_DEGREE = 4,    // a compacted degree above p - 1
};
__device__ __forceinline__ bool dcheck(DevState *st, bool ok, int site) {
#if GCSL_DEBUG_CHECKS
    if (!ok && st != nullptr) {
        set_status(st, GCSL_ERR_DEBUG_CHECK);
        atomicCAS(&st->debug_site, 0, site);
    }
    return ok;
#else
    (void)st;
    (void)site;
    return true;
#endif
}
// Work index e of n in the debug build's permuted order (a reflection and a rotation by
// the seed, a bijection on [0, n)); the identity in the release build or for seed 0.
__device__ __forceinline__ long long work_order(long long e, long long n, unsigned long long seed) {
#if GCSL_DEBUG_CHECKS
    if (seed == 0 || n <= 1) return e;
    const long long r = (long long)(seed % (unsigned long long)n);
    const long long x = n - 1 - e + r;
    return x >= n ? x - n : x;
#else
    (void)n;
    (void)seed;
    return e;
#endif
}

// C(n, k) for small k by the exact multiplicative recurrence; k is bounded by KMAX
// so the divisors are compile-time constants after unrolling.
template <int KMAX>
__device__ __forceinline__ long long binom_small(long long n, int k) {
    if (k < 0 || n < k) return 0;
    unsigned long long r = 1;
#pragma unroll
    for (int i = 0; i < KMAX; ++i) {
        if (i < k) r = r * (unsigned long long)(n - i) / (unsigned long long)(i + 1);
    }
    return (long long)r;
}

// C(n, k), general k (runtime loop).
__device__ __forceinline__ long long binom_rt(long long n, int k) {
    if (k < 0 || n < k) return 0;
    if (k > n - k) k = (int)(n - k);
    unsigned long long r = 1;
    for (int i = 0; i < k; ++i) r = r * (unsigned long long)(n - i) / (unsigned long long)(i + 1);
    return (long long)r;
}

// Pascal's triangle C(n, k) for n < GCSL_BT_N, k < GCSL_BT_K (saturated at 2^62; ranks
// at or beyond GCSL_RANK_LIMIT are rejected anyway), built at compile time.  A lookup
// replaces the multiplicative recurrence in the unranking's binary searches, whose
// dependent 64-bit multiply / divide chains set the latency of a test step.
constexpr int GCSL_BT_N = 1024, GCSL_BT_K = 13;
struct BinomTable {
    long long v[GCSL_BT_N][GCSL_BT_K];
};
constexpr BinomTable make_binom_table() {
    BinomTable t{};
    for (int n = 0; n < GCSL_BT_N; ++n) {
        t.v[n][0] = 1;
        for (int k = 1; k < GCSL_BT_K; ++k) {
            const long long a = n > 0 ? t.v[n - 1][k - 1] : 0, b = n > 0 ? t.v[n - 1][k] : 0;
            const long long cap = 1ll << 62;
            t.v[n][k] = (a >= cap - b) ? cap : a + b;
        }
    }
    return t;
}
static __device__ const BinomTable g_binom = make_binom_table();

template <int KMAX>
__device__ __forceinline__ long long binom_fast(long long n, int k) {
    if (k < 0 || n < k) return 0;
    if (n < GCSL_BT_N && k < GCSL_BT_K) return __ldg(&g_binom.v[n][k]);
    return KMAX > 0 ? binom_small<KMAX>(n, k) : binom_rt(n, k);
}

// Rows n < GCSL_SB_N of the table, copied into shared memory by a block that unranks
// (a binary-search probe then costs a shared-memory load instead of an L2 round trip).
constexpr int GCSL_SB_N = 128;
struct BinomRows {
    long long v[GCSL_SB_N][GCSL_BT_K];
};
__device__ __forceinline__ void binom_rows_load(BinomRows &sb) {
    const long long *src = &g_binom.v[0][0];
    long long *dst = &sb.v[0][0];
    for (int k = threadIdx.x; k < GCSL_SB_N * GCSL_BT_K; k += blockDim.x) dst[k] = __ldg(src + k);
}
template <int KMAX>
__device__ __forceinline__ long long binom_rows(const BinomRows *sb, long long n, int k) {
    if (sb != nullptr && n >= 0 && n < GCSL_SB_N && k >= 0 && k < GCSL_BT_K) return n < k ? 0 : sb->v[n][k];
    return binom_fast<KMAX>(n, k);
}

// Lexicographic unranking of `rank` among the L-subsets of {1..K} into 1-based
// positions (the order of set_helpers.cu:25-49).  Each position is found by a binary
// search on the hockey-stick identity sum_{u=1..t} C(N-u, r) = C(N, r+1) - C(N-t, r+1),
// so the cost is O(L^2 log K) instead of the O(L K) walk.
template <int L>
__device__ __forceinline__ void unrank_positions(int K, long long rank, int *pos, const BinomRows *sb = nullptr) {
    int xprev = 0;
#pragma unroll
    for (int c = 0; c < L; ++c) {
        const int r = L - c - 1;  // elements still to place after this one
        const int N = K - xprev;  // numbers still available
        if (r == 0) {
            pos[c] = xprev + (int)rank + 1;
        } else {
            const long long total = binom_rows<L>(sb, N, r + 1);
            const long long target = total - rank;  // want smallest t: C(N-t, r+1) < target
            int lo = 1, hi = N - r;                  // t in [1, N-r]
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (binom_rows<L>(sb, N - mid, r + 1) < target) hi = mid;
                else lo = mid + 1;
            }
            rank -= total - binom_rows<L>(sb, N - lo + 1, r + 1);
            xprev += lo;
            pos[c] = xprev;
        }
    }
}

// Runtime-level variant for the shared-memory kernels (level up to GCSL_MAX_LEVELS).
__device__ __forceinline__ void unrank_positions_rt(int L, int K, long long rank, int *pos) {
    int xprev = 0;
    for (int c = 0; c < L; ++c) {
        const int r = L - c - 1;
        const int N = K - xprev;
        if (r == 0) {
            pos[c] = xprev + (int)rank + 1;
        } else {
            const long long total = binom_fast<0>(N, r + 1);
            const long long target = total - rank;
            int lo = 1, hi = N - r;
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (binom_fast<0>(N - mid, r + 1) < target) hi = mid;
                else lo = mid + 1;
            }
            rank -= total - binom_fast<0>(N - lo + 1, r + 1);
            xprev += lo;
            pos[c] = xprev;
        }
    }
}

// Position q (1-based, over the neighbours of v_i without v_j) -> variable id; the
// ascending neighbour list still contains v_j, which is skipped (set_helpers.cu:51-57).
__device__ __forceinline__ int resolve_position(const int *__restrict__ nbrs, int vj, int q) {
    int idx = q - 1;
    idx += (__ldg(nbrs + idx) >= vj);
    return __ldg(nbrs + idx);
}

__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(GCSL_FULL_MASK, v, o));
    return v;
}

// Ordered atomics on non-negative doubles through their bit patterns.
__device__ __forceinline__ void atomic_max_nonneg(double *addr, double v) {
    atomicMax(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}
__device__ __forceinline__ void atomic_min_nonneg(double *addr, double v) {
    atomicMin(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}

// Largest i in [0, n) with prefix[i] <= x (prefix non-decreasing, prefix[0] = 0).
__device__ __forceinline__ int upper_row(const long long *__restrict__ prefix, int n, long long x) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

}  // namespace gcsl
