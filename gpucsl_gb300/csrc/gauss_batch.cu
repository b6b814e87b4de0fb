// Batches of independent Gaussian skeletons: every kernel of the level loop runs once
// for all instances of a batch, so a batch of hundreds of small problems costs a few
// dozen launches instead of a few dozen per problem, and the whole sequence (no host
// reads between levels) can be captured into one CUDA graph.
//
// Work is mapped to instances through exclusive offset arrays: level-0 tiles, rows and
// p^2 chunks per instance are fixed by the sizes (computed on the host at prepare
// time); the edges of a level are counted on the device and scanned between the
// compaction and the test kernel.  Each instance keeps its own DevState, adjacency,
// zmin / r2min and kept-pair list, exactly as a single solve does, so the results of
// an instance do not depend on the rest of the batch.
//
// Precision GCSL_PREC_F64 runs the FP64 tests of the single-instance path.  Precision
// GCSL_PREC_SPLIT first tests in FP32 on an FP32 copy of C and decides there when the
// FP32 rho^2 is outside the guard band (tanh^2 of the thresholds at 1.1 alpha and
// 0.9 alpha, i.e. the test's p-value is not within 10 % of alpha); otherwise the test is
// repeated in FP64 from C.  The skeleton and sepsets then equal the FP64 ones; z* (and
// pmax) carry the FP32 error.
//
// When an instance's C comes from the split-precision correlation (c_err: a bound eps on
// |C - C_exact|), every decision carries a first-order error bound that includes eps:
// the FP32 test decides outside the band only when its whole interval is, the FP64
// re-test decides when its interval clears the FP64 path's knife edge, and a test that
// neither can decide sets the instance's flag (level 0 likewise when |r| lies within
// eps of tanh(tau_0)).  Flagged instances are solved again (gauss_batch_rerun) after the
// seven-digit correlation, with the exact C; the others keep their results, which then
// equal the exact-C results.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "gauss_dev.cuh"

namespace gcsl {

constexpr int BATCH_MAX_LEVEL = GCSL_GAUSS_REG_LEVELS;
constexpr int BATCH_P2_CHUNK = 4096;  // entries of a p x p array per init / pmax block
constexpr float SPLIT_MIN_PIVOT = 1e-3f;

struct BInst {
    const double *C;
    const float *C32;
    const double *c_err;  // bound on |C - C_exact| (split-precision correlation), or null when C is exact
    int *flag;            // set when a decision needs the exact C
    uint16_t *G;
    double *pmax;
    int *rec;
    long long rec_cap;
    int *adj, *up, *kept;
    long long *prefix;
    double *zmin, *r2min;
    DevState *st;
    long long n_obs;
    int p, n_thr;
    double sqrt_nm3;
    double tau[BATCH_MAX_LEVEL + 1], t2[BATCH_MAX_LEVEL + 1];
    float t2lo[BATCH_MAX_LEVEL + 1], t2hi[BATCH_MAX_LEVEL + 1];
    L0Bounds l0;
};

// ------------------------------------------------------------- FP32 test
// The elimination of gauss_test_reg in FP32 on the FP32 copy of C.  Returns false when a
// pivot (including the trailing H00, H11) is below SPLIT_MIN_PIVOT or the result is not
// finite: the FP32 rho^2 is then not trusted.
template <int L>
__device__ __forceinline__ bool gauss_test_f32(const float *__restrict__ C32, int p, int vi, int vj, const int *S,
                                               float &rho2) {
    if constexpr (L == 1) {
        const float m = __ldg(C32 + (size_t)S[0] * p + S[0]);
        const float a = __ldg(C32 + (size_t)vi * p + S[0]);
        const float b = __ldg(C32 + (size_t)vj * p + S[0]);
        const float r = __ldg(C32 + (size_t)vi * p + vj);
        const float d00 = fmaf(-a, a, m), d11 = fmaf(-b, b, m);
        const float n01 = fmaf(r, m, -(a * b));
        rho2 = (n01 * n01) / (d00 * d11);
        const float lim = SPLIT_MIN_PIVOT * m;
        return m >= SPLIT_MIN_PIVOT && d00 >= lim && d11 >= lim && rho2 < 0.99f;
    }
    constexpr int D = L + 2;
    float A[D * (D + 1) / 2];
#pragma unroll
    for (int r = 0; r < L; ++r) {
        const float *Cr = C32 + (size_t)S[r] * p;
#pragma unroll
        for (int c = 0; c <= r; ++c) A[r * (r + 1) / 2 + c] = __ldg(Cr + S[c]);
        A[L * (L + 1) / 2 + r] = __ldg(C32 + (size_t)vi * p + S[r]);
        A[(L + 1) * (L + 2) / 2 + r] = __ldg(C32 + (size_t)vj * p + S[r]);
    }
    A[L * (L + 1) / 2 + L] = 1.0f;
    A[(L + 1) * (L + 2) / 2 + L] = __ldg(C32 + (size_t)vi * p + vj);
    A[(L + 1) * (L + 2) / 2 + L + 1] = 1.0f;
    float minpiv = 1.0f;
#pragma unroll
    for (int j = 0; j < L; ++j) {
        const float piv = A[j * (j + 1) / 2 + j];
        minpiv = fminf(minpiv, piv);
        const float inv = 1.0f / piv;
#pragma unroll
        for (int i = j + 1; i < D; ++i) {
            const float t = A[i * (i + 1) / 2 + j] * inv;
#pragma unroll
            for (int k = j + 1; k <= i; ++k) A[i * (i + 1) / 2 + k] = fmaf(-t, A[k * (k + 1) / 2 + j], A[i * (i + 1) / 2 + k]);
        }
    }
    const float h00 = A[L * (L + 1) / 2 + L];
    const float h01 = A[(L + 1) * (L + 2) / 2 + L];
    const float h11 = A[(L + 1) * (L + 2) / 2 + L + 1];
    minpiv = fminf(minpiv, fminf(h00, h11));
    rho2 = (h01 * h01) / (h00 * h11);
    return minpiv >= SPLIT_MIN_PIVOT && rho2 < 0.99f;  // NaN fails both
}

// ------------------------------------------------- tests on an approximate C
// The elimination of gauss_test_f32_at (gauss_dev.cuh) in T = float or double, with a
// first-order bound of the distance of every entry to its value for the exact C: the
// inputs start at u|c| + in_err (in_err bounds |C - C_exact| entrywise; the unit
// diagonal of xi and xj is exact in both), and each reciprocal, product and fma adds u
// times its result plus the propagated bounds of its operands.
template <typename T>
struct BoundArith;
template <>
struct BoundArith<float> {
    static constexpr float u = 5.9604645e-08f;  // 2^-24
    static __device__ __forceinline__ float fma_(float a, float b, float c) { return fmaf(a, b, c); }
};
template <>
struct BoundArith<double> {
    static constexpr double u = 1.1102230246251565e-16;  // 2^-53
    static __device__ __forceinline__ double fma_(double a, double b, double c) { return fma(a, b, c); }
};

struct C32Acc {
    const float *__restrict__ C32;
    int p;
    __device__ __forceinline__ float operator()(int a, int b) const { return __ldg(C32 + (size_t)a * p + b); }
};
struct C64Acc {
    const double *__restrict__ C;
    int p;
    __device__ __forceinline__ double operator()(int a, int b) const { return __ldg(C + (size_t)a * p + b); }
};

template <typename T>
__device__ __forceinline__ bool rho2_bound_t(T h00, T e00, T h01, T e01, T h11, T e11, T &rho2, T &err) {
    const T u = BoundArith<T>::u;
    const T lo00 = h00 - e00, lo11 = h11 - e11;
    rho2 = (h01 * h01) / (h00 * h11);
    const T ah = fabs(h01);
    err = T(2) * ((T(2) * ah * e01 + e01 * e01) / (lo00 * lo11) + rho2 * (e00 / lo00 + e11 / lo11) +
                  T(4) * u * rho2);
    return e00 < T(0.25) * h00 && e11 < T(0.25) * h11 && rho2 + err < T(0.98);  // NaN fails
}

template <int L, typename T, class Acc>
__device__ __forceinline__ bool gauss_test_bound(const Acc &at, int xi, int xj, const int *X, T in_err, T &rho2,
                                                 T &err) {
    const T u = BoundArith<T>::u;
    constexpr int D = L + 2;
    T A[D * (D + 1) / 2], E[D * (D + 1) / 2];
#pragma unroll
    for (int r = 0; r < L; ++r) {
#pragma unroll
        for (int c = 0; c <= r; ++c) A[r * (r + 1) / 2 + c] = at(X[r], X[c]);
        A[L * (L + 1) / 2 + r] = at(xi, X[r]);
        A[(L + 1) * (L + 2) / 2 + r] = at(xj, X[r]);
    }
    A[L * (L + 1) / 2 + L] = T(1);
    A[(L + 1) * (L + 2) / 2 + L] = at(xi, xj);
    A[(L + 1) * (L + 2) / 2 + L + 1] = T(1);
#pragma unroll
    for (int k = 0; k < D * (D + 1) / 2; ++k) E[k] = u * fabs(A[k]) + in_err;
    E[L * (L + 1) / 2 + L] = T(0);
    E[(L + 1) * (L + 2) / 2 + L + 1] = T(0);
    bool ok = true;
#pragma unroll
    for (int j = 0; j < L; ++j) {
        const T piv = A[j * (j + 1) / 2 + j], ep = E[j * (j + 1) / 2 + j];
        ok = ok && ep < T(0.25) * piv;
        const T inv = T(1) / piv;
        const T einv = ep * inv * inv * T(1.5) + u * fabs(inv);  // 1/(p - e) <= (1 + 1.5 e/p)/p for e < p/4
#pragma unroll
        for (int i = j + 1; i < D; ++i) {
            const T aij = A[i * (i + 1) / 2 + j];
            const T t = aij * inv;
            const T et = fabs(aij) * einv + fabs(inv) * E[i * (i + 1) / 2 + j] + u * fabs(t);
#pragma unroll
            for (int k = j + 1; k <= i; ++k) {
                const T akj = A[k * (k + 1) / 2 + j];
                const T v = BoundArith<T>::fma_(-t, akj, A[i * (i + 1) / 2 + k]);
                E[i * (i + 1) / 2 + k] += fabs(t) * E[k * (k + 1) / 2 + j] + fabs(akj) * et + u * fabs(v);
                A[i * (i + 1) / 2 + k] = v;
            }
        }
    }
    const int i00 = L * (L + 1) / 2 + L, i01 = (L + 1) * (L + 2) / 2 + L, i11 = (L + 1) * (L + 2) / 2 + L + 1;
    return rho2_bound_t<T>(A[i00], E[i00], A[i01], E[i01], A[i11], E[i11], rho2, err) && ok;
}

// The FP64 re-test of a key whose FP32 interval touches the guard band, on the
// approximate C with its bound: decided when the interval clears the FP64 path's knife
// edge [t2 (1 - 1e-12), t2 (1 + 1e-12)] (then its decision is the exact C's); otherwise
// the instance is flagged for the exact re-solve and the FP64 result stands in.
template <int L>
__device__ __noinline__ TestOut split_retest_call(const double *__restrict__ C, int p, int vi, int vj, const int *S,
                                                  double tau, double t2, double eps, int *flag) {
    double r, e;
    const bool ok = gauss_test_bound<L, double>(C64Acc{C, p}, vi, vj, S, eps * 1.001, r, e);
    const bool decided = ok && (r + e < t2 * (1.0 - 1e-12) || r - e > t2 * (1.0 + 1e-12));
    if (!decided) *(volatile int *)flag = 1;
    TestOut o = gauss_test_reg<L>(C, p, vi, vj, S, tau, t2);
    if (decided) o.remove = r + e < t2 * (1.0 - 1e-12);
    return o;
}

template <int L>
struct SplitTest {
    static constexpr bool kMixed = false;
    const double *__restrict__ C;
    const float *__restrict__ C32;
    int p;
    double tau, t2;
    float t2lo, t2hi;
    unsigned long long *retests;
    double eps;   // bound on |C - C_exact|, or a negative value when C is exact
    float eps32;  // eps * 1.001 rounded up to FP32, formed once per edge rather than per test
    int *flag;
    __device__ __forceinline__ TestOut operator()(int vi, int vj, const int *S) const {
        if (eps32 < 0.f) {
            float r2;
            const bool ok = gauss_test_f32<L>(C32, p, vi, vj, S, r2);
            if (ok && (r2 < t2lo || r2 > t2hi)) {
                TestOut o;
                o.rho2 = f32_nonneg_to_f64(r2);
                o.zexact = __longlong_as_double(0x7ff0000000000000ll);
                o.remove = r2 < t2lo;
                return o;
            }
            ++*retests;
            return gauss_test_reg_call<L>(C, p, vi, vj, S, tau, t2);  // out of line: keeps its registers off this path
        }
        float r, e;
        const bool ok = gauss_test_bound<L, float>(C32Acc{C32, p}, vi, vj, S, eps32, r, e);
        if (ok && (__fadd_ru(r, e) < t2lo || __fsub_rd(r, e) > t2hi)) {
            TestOut o;
            o.rho2 = f32_nonneg_to_f64(r);
            o.zexact = __longlong_as_double(0x7ff0000000000000ll);
            o.remove = __fadd_ru(r, e) < t2lo;
            return o;
        }
        ++*retests;
        return split_retest_call<L>(C, p, vi, vj, S, tau, t2, eps, flag);
    }
};

// ------------------------------------------------------------------ kernels
// Instance of block b under exclusive offsets off[0..count].
__device__ __forceinline__ int inst_of(const long long *__restrict__ off, int count, long long b, long long &lb) {
    const int k = upper_row(off, count, b);
    lb = b - off[k];
    return k;
}

// A kernel of the exact re-solve (rerun) skips every instance whose flag is not set.
__device__ __forceinline__ bool skip_inst(const BInst &I, bool rerun) { return rerun && *(volatile int *)I.flag == 0; }

// Per p^2 chunk: r2min = 1.4e306 (above every stored rho^2); chunk 0 also clears the
// instance's DevState (and, on the first pass, its flag); block 0 builds the erfc
// table of the pmax kernels.
__global__ void batch_init_kernel(const BInst *__restrict__ inst, const long long *__restrict__ off_p2, int count,
                                  double *__restrict__ sftab, bool rerun) {
    if (blockIdx.x == 0 && !rerun) sf_table_build(reinterpret_cast<double (*)[SF_TERMS]>(sftab));  // erfc table for pmax
    long long lb;
    const BInst &I = inst[inst_of(off_p2, count, blockIdx.x, lb)];
    if (skip_inst(I, rerun)) return;
    if (lb == 0 && !rerun && threadIdx.x == 0) *I.flag = 0;
    const long long total = (long long)I.p * I.p;
    const long long k0 = lb * BATCH_P2_CHUNK, k1 = min(total, k0 + BATCH_P2_CHUNK);
    const double big = __longlong_as_double(0x7f7f7f7f7f7f7f7fll);
    for (long long k = k0 + threadIdx.x; k < k1; k += blockDim.x) I.r2min[k] = big;
    if (lb == 0) {
        unsigned *w = reinterpret_cast<unsigned *>(I.st);
        for (int k = threadIdx.x; k < (int)(sizeof(DevState) / sizeof(unsigned)); k += blockDim.x) w[k] = 0u;
    }
}

// Level 0.  On an approximate C (first pass, c_err set) a pair whose |r| lies within the
// bound of tanh(tau_0) cannot be decided: the instance is flagged.
__global__ void batch_level0_kernel(const BInst *__restrict__ inst, const long long *__restrict__ off_tiles,
                                    int count, bool rerun) {
    long long lb;
    const BInst &I = inst[inst_of(off_tiles, count, blockIdx.x, lb)];
    if (skip_inst(I, rerun)) return;
    if (!rerun && I.c_err != nullptr) {
        const double eps = *I.c_err * 1.001 + 1e-15;
        const double t0 = sqrt(I.t2[0]);
        const int nb = (I.p + 31) / 32;
        int rem = (int)lb, bi = 0;
        while (rem >= nb - bi) {
            rem -= nb - bi;
            ++bi;
        }
        const int bj = bi + rem;
        bool unsure = false;
        for (int r = threadIdx.x >> 5; r < 32; r += blockDim.x >> 5) {
            const int i = bi * 32 + r, j = bj * 32 + (threadIdx.x & 31);
            if (i < I.p && j < I.p && i < j) unsure |= !(fabs(fabs(I.C[(size_t)i * I.p + j]) - t0) > eps);
        }
        if (__syncthreads_or(unsure) && threadIdx.x == 0) *(volatile int *)I.flag = 1;
    }
    level0_tile(I.C, I.p, I.tau[0], I.l0, I.G, I.zmin, I.r2min, I.kept, I.st, (int)lb);
}

// Warp per (instance, row); level 1 compacts G, later levels refilter the lists.
__global__ void batch_compact_kernel(const BInst *__restrict__ inst, const long long *__restrict__ off_rows,
                                     int count, int level, bool rerun) {
    const int lane = threadIdx.x & 31;
    const long long rows = off_rows[count];
    const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long g = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; g < rows; g += warps) {
        long long r;
        const BInst &I = inst[inst_of(off_rows, count, g, r)];
        if (skip_inst(I, rerun) || I.st->done) continue;
        const int deg = (level == 1) ? compact_row(I.G, I.p, I.adj, I.up, (int)r, lane)
                                     : recompact_row(I.G, I.p, I.adj, I.up, (int)r, lane, nullptr, nullptr, I.st);
        if (lane == 0) atomicMax(&I.st->max_degree[level], deg);
    }
}

// Block per instance: decide whether the instance runs this level (the reference's stop
// rule max degree - 1 < level, and the level cap), scan its rows into the edge prefix
// and publish its edge count.
__global__ void batch_scan_kernel(const BInst *__restrict__ inst, int count, int level, int max_level,
                                  long long *__restrict__ edges, bool rerun) {
    const BInst &I = inst[blockIdx.x];
    if (skip_inst(I, rerun)) {
        if (threadIdx.x == 0) edges[blockIdx.x] = 0;
        return;
    }
    DevState *st = I.st;
    __shared__ int s_run;
    if (threadIdx.x == 0) {
        int run = !st->done;
        if (run && st->max_degree[level] - 1 < level) run = 0;
        if (run && level >= I.n_thr) {
            set_status(st, GCSL_ERR_UNSUPPORTED_LEVEL);
            run = 0;
        }
        if (run && level > max_level) run = 0;
        if (!run) st->done = 1;
        else st->last_level = level;
        s_run = run;
    }
    __syncthreads();
    if (!s_run) {
        if (threadIdx.x == 0) edges[blockIdx.x] = 0;
        return;
    }
    block_scan_rows(I.up, I.p, I.prefix);
    __syncthreads();
    if (threadIdx.x == 0) {
        edges[blockIdx.x] = I.prefix[I.p];
        st->edges[level] = (unsigned long long)I.prefix[I.p];
    }
}

// One block: exclusive scan of the per-instance edge counts into off[0..count].
__global__ void batch_edge_offsets_kernel(const long long *__restrict__ edges, int count, long long *__restrict__ off) {
    block_scan_rows(edges, count, off);
}

// Levels 1 and 2 (most of a batch's tests) run at three 256-thread blocks per SM: their
// FP32 tests need few registers, and the 24 resident warps hide more of the gathers'
// latency than the 16 that the register count of their rare FP64 re-test path allowed
// (a few spilled values of that path stay in L1).  Higher levels keep their registers.
template <int L, int G, bool SPLIT>
__global__ void __launch_bounds__(256, (L <= 2 ? 3 : 1)) batch_level_kernel(const BInst *__restrict__ inst,
                                                         const long long *__restrict__ edge_off, int count,
                                                         bool rerun) {
    constexpr int GPW = 32 / G;
    const int lane = threadIdx.x & 31, gl = lane & (G - 1), gw = lane / G;
    const unsigned gshift = (unsigned)(gw * G);
    const unsigned gbits = (G == 32) ? 0xffffffffu : ((1u << G) - 1u);
    const long long n_edges = edge_off[count];
    const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    for (long long e0 = (((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * GPW; e0 < n_edges;
         e0 += warps * GPW) {
        const long long e = e0 + gw;
        const bool has = e < n_edges;
        long long le = 0;
        const int k = has ? inst_of(edge_off, count, e, le) : 0;
        const BInst &I = inst[k];
        EdgeJob J;
        J.T = 0;
        if (has && !load_edge<L>(I.adj, I.up, I.prefix, I.p, le, L, J)) {
            if (gl == 0) set_status(I.st, GCSL_ERR_UNSUPPORTED);
            J.T = 0;
        }
        double r2min = inf, zmin_exact = inf;
        bool removed = false;
        unsigned long long n_tests = 0, retests = 0;
        if constexpr (SPLIT) {
            // the rerun has the exact C: no bound
            const double eps = (has && !rerun && I.c_err != nullptr) ? *I.c_err : -1.0;
            // eps widened by 0.1 % in FP32, rounded up (no FP64 instruction per edge)
            const float eps32 = __fmul_ru(f64_nonneg_to_f32_ru(eps), 1.001f);
            walk_edge<L, G>(J, has, I.adj, I.p, gl, gshift, gbits,
                            SplitTest<L>{I.C, I.C32, I.p, I.tau[L], I.t2[L], I.t2lo[L], I.t2hi[L], &retests, eps, eps32,
                                         I.flag},
                            I.G, nullptr, BATCH_MAX_LEVEL, I.rec, I.rec_cap, I.st, r2min, zmin_exact, removed,
                            n_tests);
        } else {
            walk_edge<L, G>(J, has, I.adj, I.p, gl, gshift, gbits, F64Test<L>{I.C, I.p, I.tau[L], I.t2[L]}, I.G,
                            nullptr, BATCH_MAX_LEVEL, I.rec, I.rec_cap, I.st, r2min, zmin_exact, removed, n_tests);
        }
        if (SPLIT && retests) atomicAdd(&I.st->retests, retests);
        if (has && gl == 0 && J.T > 0) {
            const size_t ix = (size_t)J.lo * I.p + J.hi;
            // both non-negative for a pair alive at this level (integer compares, as in walk_edge)
            if (__double_as_longlong(zmin_exact) < __double_as_longlong(inf))
                I.zmin[ix] = min_nonneg(I.zmin[ix], zmin_exact);
            if (__double_as_longlong(r2min) < __double_as_longlong(inf)) I.r2min[ix] = min_nonneg(I.r2min[ix], r2min);
            atomicAdd(&I.st->tests[L], n_tests);
            atomicAdd(&I.st->tests_full[L], (unsigned long long)J.T);
            if (removed) atomicAdd(&I.st->removed[L], 1ull);
        }
    }
}

// pmax of the pairs removed at level 0 and the -1 fill, per p^2 chunk.
__global__ void batch_pmax_removed_kernel(const BInst *__restrict__ inst, const long long *__restrict__ off_p2,
                                          int count, const double *__restrict__ sftab, bool rerun) {
    __shared__ double tab[SF_CENTRES][SF_TERMS];
    long long lb;
    const BInst &I = inst[inst_of(off_p2, count, blockIdx.x, lb)];
    if (skip_inst(I, rerun)) return;  // uniform over the block
    sf_table_load(tab, sftab);
    __syncthreads();
    const unsigned p = (unsigned)I.p;
    const unsigned total = p * p;
    const unsigned k0 = (unsigned)lb * BATCH_P2_CHUNK, k1 = min(total, k0 + (unsigned)BATCH_P2_CHUNK);
    for (unsigned k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
        const unsigned i = k / p, j = k - i * p;
        if (i >= j) I.pmax[k] = -1.0;
        else if (I.zmin[k] < 0.0) I.pmax[k] = two_sf_tab(I.sqrt_nm3 * fisher_z(I.C[k]), tab);
    }
}

// pmax of the pairs kept at level 0, block per instance.
__global__ void batch_pmax_kept_kernel(const BInst *__restrict__ inst, const double *__restrict__ sftab, bool rerun) {
    __shared__ double tab[SF_CENTRES][SF_TERMS];
    const BInst &I = inst[blockIdx.x];
    if (skip_inst(I, rerun)) return;  // uniform over the block
    sf_table_load(tab, sftab);
    __syncthreads();
    const int n = I.st->n_kept;
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
        const int k = I.kept[t];
        double z = I.zmin[k];
        const double r2 = I.r2min[k];
        if (r2 < 1.0) z = fmin(z, fisher_z(sqrt(r2)));
        I.pmax[k] = two_sf_tab(I.sqrt_nm3 * z, tab);
    }
}

// The erfc table of the pmax kernels (a plan whose step finishes without its own init).
__global__ void batch_sftab_kernel(double *__restrict__ sftab) {
    sf_table_build(reinterpret_cast<double (*)[SF_TERMS]>(sftab));
}

// [done, last level run, status, record ints] per instance.
__global__ void batch_status_kernel(const BInst *__restrict__ inst, int count, int *__restrict__ out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const DevState *st = inst[k].st;
    out[4 * k] = *(volatile const int *)&st->done;
    out[4 * k + 1] = *(volatile const int *)&st->last_level;
    out[4 * k + 2] = *(volatile const int *)&st->status;
    out[4 * k + 3] = (int)*(volatile const unsigned long long *)&st->n_rec_ints;
}

// ---------------------------------------------------------------------- host
namespace host {

namespace {

struct BatchLayout {
    size_t table, off_tiles, off_rows, off_p2, edges, edge_off, sftab, flags, status, slices, total;
};

size_t al(size_t x) { return (x + 255) / 256 * 256; }

size_t slice_bytes(int p) {
    const size_t pp = (size_t)p * p;
    return al(sizeof(DevState)) + al(pp * sizeof(int)) + al((size_t)p * sizeof(int)) +
           al(((size_t)p + 1) * sizeof(long long)) + 2 * al(pp * sizeof(double)) +
           al(((size_t)p * (p - 1) / 2 + 1) * sizeof(int));
}

BatchLayout layout(const int *p, int count) {
    BatchLayout L;
    size_t off = 0;
    L.table = off;
    off += al((size_t)count * sizeof(BInst));
    L.off_tiles = off;
    off += al(((size_t)count + 1) * sizeof(long long));
    L.off_rows = off;
    off += al(((size_t)count + 1) * sizeof(long long));
    L.off_p2 = off;
    off += al(((size_t)count + 1) * sizeof(long long));
    L.edges = off;
    off += al((size_t)count * sizeof(long long));
    L.edge_off = off;
    off += al(((size_t)count + 1) * sizeof(long long));
    L.sftab = off;
    off += al((size_t)SF_CENTRES * SF_TERMS * sizeof(double));
    L.flags = off;
    off += al((size_t)count * sizeof(int));
    L.status = off;
    off += al((size_t)count * 4 * sizeof(int));
    L.slices = off;
    if (p)  // p == nullptr: every instance brings its own state slice
        for (int k = 0; k < count; ++k) off += slice_bytes(p[k]);
    L.total = off;
    return L;
}

// plan words
enum {
    PW_MAGIC = 0, PW_WS, PW_COUNT, PW_MAXL, PW_PREC, PW_TILES, PW_ROWS, PW_P2, PW_SMS, PW_FLAGS, PW_STATUS,
    PW_LANES  // PW_LANES + level, up to PW_LANES + BATCH_MAX_LEVEL (< 48 plan words)
};
static_assert(PW_LANES + BATCH_MAX_LEVEL < 48, "plan words");
constexpr long long PLAN_MAGIC = 0x4743534c42415443ll;  // "GCSLBATC"

template <int L, int G, bool SPLIT>
void launch_level_t(const BInst *inst, const long long *eoff, int count, int sms, bool rerun, cudaStream_t s) {
    const int threads = L >= 4 ? 128 : 256;
    const int blocks = sms * (L >= 4 ? 12 : 8);
    batch_level_kernel<L, G, SPLIT><<<blocks, threads, 0, s>>>(inst, eoff, count, rerun);
}

template <bool SPLIT>
cudaError_t launch_level(int L, int lanes, const BInst *inst, const long long *eoff, int count, int sms, bool rerun,
                         cudaStream_t s) {
    const bool g8 = lanes == 8 && L <= 4;
    switch (L) {
#define GCSL_BL(K)                                                                 \
    case K:                                                                        \
        if (g8 && K <= 4) launch_level_t<K, (K <= 4 ? 8 : 32), SPLIT>(inst, eoff, count, sms, rerun, s); \
        else launch_level_t<K, 32, SPLIT>(inst, eoff, count, sms, rerun, s);      \
        break;
        GCSL_BL(1) GCSL_BL(2) GCSL_BL(3) GCSL_BL(4) GCSL_BL(5) GCSL_BL(6)
        GCSL_BL(7) GCSL_BL(8) GCSL_BL(9) GCSL_BL(10) GCSL_BL(11) GCSL_BL(12)
#undef GCSL_BL
    default:
        return cudaErrorInvalidValue;
    }
    note_launch(1);
    return cudaGetLastError();
}

// Builds the instance table and offset arrays in host memory laid out as the device
// header [table | tiles | rows | p^2 chunks] (at `hdr`, Ly.edges bytes).  Instances with
// a state pointer keep their solve state there (it persists across plans and calls);
// the others get a slice of the workspace.  Returns the totals through the plan words.
int build_header(const gcsl_gauss_instance *in, int count, int max_level, int precision, char *base,
                 const BatchLayout &Ly, char *hdr, long long *plan, int sms) {
    BInst *tab = reinterpret_cast<BInst *>(hdr + Ly.table);
    long long *ot = reinterpret_cast<long long *>(hdr + Ly.off_tiles);
    long long *orow = reinterpret_cast<long long *>(hdr + Ly.off_rows);
    long long *op2 = reinterpret_cast<long long *>(hdr + Ly.off_p2);
    ot[0] = orow[0] = op2[0] = 0;
    size_t cur = Ly.slices;
    for (int k = 0; k < count; ++k) {
        const gcsl_gauss_instance &X = in[k];
        BInst &I = tab[k];
        std::memset(&I, 0, sizeof(I));
        const int p = X.p;
        const size_t pp = (size_t)p * p;
        I.C = X.C;
        I.C32 = X.C32;
        I.c_err = precision == GCSL_PREC_SPLIT ? X.c_err : nullptr;
        I.flag = reinterpret_cast<int *>(base + Ly.flags) + k;
        I.G = X.G;
        I.pmax = X.pmax;
        I.rec = X.rec_pool;
        I.rec_cap = X.rec_pool ? X.rec_cap : 0;
        I.n_obs = X.n_obs;
        I.p = p;
        I.n_thr = X.n_thresholds;
        I.sqrt_nm3 = std::sqrt((double)(X.n_obs - 3));
        char *c = X.state != nullptr ? static_cast<char *>(X.state) : base + cur;
        if (X.state == nullptr) cur += slice_bytes(p);
        I.st = reinterpret_cast<DevState *>(c);
        c += al(sizeof(DevState));
        I.adj = reinterpret_cast<int *>(c);
        c += al(pp * sizeof(int));
        I.up = reinterpret_cast<int *>(c);
        c += al((size_t)p * sizeof(int));
        I.prefix = reinterpret_cast<long long *>(c);
        c += al(((size_t)p + 1) * sizeof(long long));
        I.zmin = reinterpret_cast<double *>(c);
        c += al(pp * sizeof(double));
        I.r2min = reinterpret_cast<double *>(c);
        c += al(pp * sizeof(double));
        I.kept = reinterpret_cast<int *>(c);
        for (int l = 0; l <= BATCH_MAX_LEVEL; ++l) {
            const double tau = l < X.n_thresholds ? X.thresholds[l] : 0.0;
            const double t = std::tanh(tau);
            I.tau[l] = tau;
            I.t2[l] = t * t;
            if (l == 0) I.l0 = level0_bounds(t * t);
            if (precision == GCSL_PREC_SPLIT) {
                const double lo = std::tanh(l < X.n_thresholds ? X.band_lo[l] : 0.0);
                const double hi = std::tanh(l < X.n_thresholds ? X.band_hi[l] : 0.0);
                // round outward so the FP32 comparisons never narrow the band
                I.t2lo[l] = std::nextafter((float)(lo * lo), 0.0f);
                I.t2hi[l] = std::nextafter((float)(hi * hi), 2.0f);
            }
        }
        const long long nb = (p + 31) / 32;
        ot[k + 1] = ot[k] + nb * (nb + 1) / 2;
        orow[k + 1] = orow[k] + p;
        op2[k + 1] = op2[k] + ((long long)pp + BATCH_P2_CHUNK - 1) / BATCH_P2_CHUNK;
    }
    if (ot[count] > 0x7fffffffll || op2[count] > 0x7fffffffll) return GCSL_ERR_UNSUPPORTED;
    std::memset(plan, 0, sizeof(long long) * 48);
    plan[PW_MAGIC] = PLAN_MAGIC;
    plan[PW_WS] = (long long)reinterpret_cast<uintptr_t>(base);
    plan[PW_COUNT] = count;
    plan[PW_MAXL] = max_level;
    plan[PW_PREC] = precision;
    plan[PW_TILES] = ot[count];
    plan[PW_ROWS] = orow[count];
    plan[PW_P2] = op2[count];
    plan[PW_SMS] = sms;
    for (int l = 0; l <= BATCH_MAX_LEVEL; ++l) plan[PW_LANES + l] = 32;
    plan[PW_FLAGS] = (long long)reinterpret_cast<uintptr_t>(base + Ly.flags);
    plan[PW_STATUS] = (long long)reinterpret_cast<uintptr_t>(base + Ly.status);
    return GCSL_OK;
}

BatchLayout layout_for(const gcsl_gauss_instance *in, int count) {
    std::vector<int> ps;
    for (int k = 0; k < count; ++k)
        if (in[k].state == nullptr) ps.push_back(in[k].p);
    BatchLayout Ly = layout(nullptr, count);
    for (int p : ps) Ly.total += slice_bytes(p);
    return Ly;
}

}  // namespace

size_t gauss_batch_workspace_bytes(const int *p, int count) { return layout(p, count).total; }

size_t gauss_state_bytes(int p) { return slice_bytes(p); }

size_t gauss_batch_table_bytes(int count) { return layout(nullptr, count).total; }

// Builds the instance table on the host and uploads it with the offset arrays
// (synchronous: outside any stream capture).  thresholds / band arrays are host arrays.
int gauss_batch_prepare(const gcsl_gauss_instance *in, int count, int max_level, int precision, void *ws,
                        size_t ws_bytes, long long *plan, int sms, cudaStream_t s) {
    const BatchLayout Ly = layout_for(in, count);
    if (ws_bytes < Ly.total) return GCSL_ERR_WORKSPACE;
    char *base = static_cast<char *>(ws);
    std::vector<char> hdr(Ly.edges);
    const int rc = build_header(in, count, max_level, precision, base, Ly, hdr.data(), plan, sms);
    if (rc != GCSL_OK) return rc;
    cudaError_t e = cudaMemcpyAsync(base, hdr.data(), hdr.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(base + Ly.flags, 0, (size_t)count * sizeof(int), s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // the host vector dies with this call
    if (e != cudaSuccess) {
        plan[PW_MAGIC] = 0;
        return GCSL_ERR_DEVICE;
    }
    return GCSL_OK;
}

// The same without a synchronisation: the header is built in the caller's host buffer
// `stage` (pinned, gcsl_gauss_batch_table_bytes(count) bytes), which must stay untouched
// until the stream has passed the copy enqueued here.
int gauss_batch_prepare_staged(const gcsl_gauss_instance *in, int count, int max_level, int precision, void *ws,
                               size_t ws_bytes, void *stage, size_t stage_bytes, long long *plan, int sms,
                               cudaStream_t s) {
    const BatchLayout Ly = layout_for(in, count);
    if (ws_bytes < Ly.total || stage_bytes < Ly.edges) return GCSL_ERR_WORKSPACE;
    char *base = static_cast<char *>(ws);
    const int rc = build_header(in, count, max_level, precision, base, Ly, static_cast<char *>(stage), plan, sms);
    if (rc != GCSL_OK) return rc;
    cudaError_t e = cudaMemcpyAsync(base, stage, Ly.edges, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(base + Ly.flags, 0, (size_t)count * sizeof(int), s);
    if (e != cudaSuccess) {
        plan[PW_MAGIC] = 0;
        return GCSL_ERR_DEVICE;
    }
    return GCSL_OK;
}

bool gauss_batch_plan_ok(const long long *plan) { return plan && plan[PW_MAGIC] == PLAN_MAGIC; }

const int *gauss_batch_flags(const long long *plan) {
    return gauss_batch_plan_ok(plan) ? reinterpret_cast<const int *>(static_cast<uintptr_t>(plan[PW_FLAGS])) : nullptr;
}

int gauss_batch_set_lanes(long long *plan, int level, int lanes) {
    if (!gauss_batch_plan_ok(plan) || level < 1 || level > BATCH_MAX_LEVEL || (lanes != 32 && lanes != 8))
        return GCSL_ERR_INVALID_ARG;
    plan[PW_LANES + level] = lanes;
    return GCSL_OK;
}

// Enqueues levels first..last (first == 0: the state reset and level 0 as well) of every
// instance of the plan, then, with finish, the pmax write-back.  Levels run in order per
// instance across calls (its state lives in its slice); an instance whose loop has ended
// skips the rest on the device.  host_status (pinned, 4 ints per instance) receives
// [done, last level run, status, sepset record ints] of every instance after the step.
int gauss_batch_step(const long long *plan, int first, int last, bool finish, bool rerun, int32_t *host_status,
                     cudaStream_t s) {
    if (!gauss_batch_plan_ok(plan)) return GCSL_ERR_INVALID_ARG;
    char *base = reinterpret_cast<char *>(static_cast<uintptr_t>(plan[PW_WS]));
    const int count = (int)plan[PW_COUNT], max_level = (int)plan[PW_MAXL], sms = (int)plan[PW_SMS];
    const bool split = plan[PW_PREC] == GCSL_PREC_SPLIT;
    const BatchLayout Ly = layout(nullptr, count);
    const BInst *inst = reinterpret_cast<const BInst *>(base + Ly.table);
    const long long *ot = reinterpret_cast<const long long *>(base + Ly.off_tiles);
    const long long *orow = reinterpret_cast<const long long *>(base + Ly.off_rows);
    const long long *op2 = reinterpret_cast<const long long *>(base + Ly.off_p2);
    long long *edges = reinterpret_cast<long long *>(base + Ly.edges);
    long long *eoff = reinterpret_cast<long long *>(base + Ly.edge_off);
    double *sftab = reinterpret_cast<double *>(base + Ly.sftab);

    if (first == 0) {
        batch_init_kernel<<<(unsigned)plan[PW_P2], 256, 0, s>>>(inst, op2, count, sftab, rerun);
        batch_level0_kernel<<<(unsigned)plan[PW_TILES], 256, 0, s>>>(inst, ot, count, rerun);
        note_launch(2);
    }
    const long long rows = plan[PW_ROWS];
    const int cblocks = (int)std::min<long long>((rows + 7) / 8, (long long)sms * 16);
    for (int level = std::max(first, 1); level <= std::min(last, max_level); ++level) {
        batch_compact_kernel<<<cblocks, 256, 0, s>>>(inst, orow, count, level, rerun);
        batch_scan_kernel<<<count, 256, 0, s>>>(inst, count, level, max_level, edges, rerun);
        batch_edge_offsets_kernel<<<1, 1024, 0, s>>>(edges, count, eoff);
        note_launch(3);
        const int lanes = (int)plan[PW_LANES + level];
        const cudaError_t e = split ? launch_level<true>(level, lanes, inst, eoff, count, sms, rerun, s)
                                    : launch_level<false>(level, lanes, inst, eoff, count, sms, rerun, s);
        if (e != cudaSuccess) return GCSL_ERR_DEVICE;
    }
    if (finish) {
        if (first != 0) {  // the erfc table of this plan's header is built by its init kernel
            batch_sftab_kernel<<<1, 32, 0, s>>>(sftab);
            note_launch(1);
        }
        batch_pmax_removed_kernel<<<(unsigned)plan[PW_P2], 256, 0, s>>>(inst, op2, count, sftab, rerun);
        batch_pmax_kept_kernel<<<count, 256, 0, s>>>(inst, sftab, rerun);
        note_launch(2);
    }
    if (host_status != nullptr) {
        int *dev_status = reinterpret_cast<int *>(static_cast<uintptr_t>(plan[PW_STATUS]));
        batch_status_kernel<<<(count + 127) / 128, 128, 0, s>>>(inst, count, dev_status);
        note_launch(1);
        if (cudaMemcpyAsync(host_status, dev_status, (size_t)count * 4 * sizeof(int), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess)
            return GCSL_ERR_DEVICE;
    }
    return cudaGetLastError() == cudaSuccess ? GCSL_OK : GCSL_ERR_DEVICE;
}

// Enqueues the whole batch: init, level 0, levels 1..max_level, pmax.  No host reads:
// the sequence can be captured into a CUDA graph.  With rerun set only the flagged
// instances are solved (again), with the test of an exact C.
int gauss_batch_run(const long long *plan, cudaStream_t s, bool rerun) {
    if (!gauss_batch_plan_ok(plan)) return GCSL_ERR_INVALID_ARG;
    return gauss_batch_step(plan, 0, (int)plan[PW_MAXL], true, rerun, nullptr, s);
}

// Synchronises the stream and copies every instance's state back into the outputs.
int gauss_batch_collect(const long long *plan, gcsl_gauss_instance *out, int count, cudaStream_t s) {
    if (!gauss_batch_plan_ok(plan) || count != (int)plan[PW_COUNT]) return GCSL_ERR_INVALID_ARG;
    char *base = reinterpret_cast<char *>(static_cast<uintptr_t>(plan[PW_WS]));
    std::vector<BInst> tab((size_t)count);
    if (cudaMemcpyAsync(tab.data(), base, tab.size() * sizeof(BInst), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GCSL_ERR_DEVICE;
    std::vector<int> flags((size_t)count, 0);
    if (cudaMemcpyAsync(flags.data(), gauss_batch_flags(plan), (size_t)count * sizeof(int), cudaMemcpyDeviceToHost,
                        s) != cudaSuccess)
        return GCSL_ERR_DEVICE;
    std::vector<DevState> st((size_t)count);
    for (int k = 0; k < count; ++k)
        if (cudaMemcpyAsync(&st[(size_t)k], tab[(size_t)k].st, sizeof(DevState), cudaMemcpyDeviceToHost, s) !=
            cudaSuccess)
            return GCSL_ERR_DEVICE;
    if (cudaStreamSynchronize(s) != cudaSuccess) return GCSL_ERR_DEVICE;
    int first = GCSL_OK;
    for (int k = 0; k < count; ++k) {
        const DevState &h = st[(size_t)k];
        gcsl_gauss_instance &o = out[k];
        o.status = h.status;
        o.levels_run = h.last_level + 1;
        o.n_records = (int64_t)h.n_rec_ints;
        long long tests = (long long)o.p * (o.p - 1) / 2;
        for (int l = 1; l <= BATCH_MAX_LEVEL; ++l) tests += (long long)h.tests[l];
        o.tests = tests;
        o.retests = (int64_t)h.retests;
        o.exact_rerun = flags[(size_t)k] != 0 ? 1 : 0;
        if (first == GCSL_OK && h.status != GCSL_OK) first = h.status;
    }
    return first;
}

}  // namespace host
}  // namespace gcsl
