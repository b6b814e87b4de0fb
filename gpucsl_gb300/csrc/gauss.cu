// Gaussian PC-stable skeleton kernels for sm_103a.
//
//   level 0        gauss_level0_kernel     (reference: gpucsl/pc/cuda/gaussian_ci.cu:18-51)
//   compaction     compact_kernel          (reference: gpucsl/pc/cuda/helpers/graph_helpers.cu:35-56)
//   edge prefix    row_scan_kernel
//   level l <= 12  gauss_level_reg_kernel + gauss_level_units_kernel (reference:
//                  gaussian_ci.cu:66-120, helpers/gaussian_helpers.cu:240-262)
//   z* candidates  gauss_cand_kernel (FP64, side stream)
//   level l > 12   gauss_level_smem_kernel
//   zmin -> pmax   pmax_level0_kernel, pmax_kept_kernel (reference: gpucsl/pc/helpers.py:62-82)
//
// Work decomposition of a level (gauss_levels.cuh): one warp owns one undirected edge
// {lo, hi} alive at level start and walks the merged key sequence of both directions,
// key = (rank, dir) with dir 0 for v_i = lo, 32 keys per step (one test per lane); a
// longer walk is cut into units of 32 keys that the unit kernel walks in parallel and
// its last unit combines in key order.  The canonical remover is the smallest removing
// key (its set is the sepset) and z* folds the keys up to it, so the result does not
// depend on scheduling.
#include "gauss_levels.cuh"

namespace gcsl {

// ----------------------------------------------------------------- level 0
__global__ void gauss_level0_kernel(const double *__restrict__ C, int p, double tau0, L0Bounds B,
                                    uint16_t *__restrict__ G, double *__restrict__ zmin, double *__restrict__ r2min,
                                    int *__restrict__ kept, DevState *st, float *C32) {
    level0_tile(C, p, tau0, B, G, zmin, r2min, kept, st, (int)blockIdx.x, C32);
}

// ------------------------------------------------------------- compaction
// Warp per row (level 1: from G; later levels: refiltering the previous list).  Return at
// once when the level loop is already finished.
__global__ void compact_kernel(const uint16_t *__restrict__ G, int p, int *__restrict__ adj, int *__restrict__ up,
                               DevState *st, int level, int2 *elist) {
    pdl_wait();
    pdl_trigger();
    if (st != nullptr && st->done) return;
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    int maxdeg = 0;
    unsigned long long *ecount = (st != nullptr && elist != nullptr) ? &st->edges[level] : nullptr;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < p; r += warps)
        maxdeg = max(maxdeg, compact_row(G, p, adj, up, r, lane, elist, ecount));
    if (lane == 0 && st != nullptr) atomicMax(&st->max_degree[level], maxdeg);
}

// Recompaction by `nblocks` blocks (block index b) for one level.
__device__ __forceinline__ void recompact_blocks(const uint16_t *__restrict__ G, int p, int *__restrict__ adj,
                                                 int *__restrict__ up, DevState *st, int level, int2 *elist, int b,
                                                 int nblocks) {
    if (st->done) return;
    if (st->removed[level - 1] == 0) {  // nothing removed: the lists, degrees and edges stand
        if (b == 0 && threadIdx.x == 0) {
            st->max_degree[level] = st->max_degree[level - 1];
            st->edges[level] = st->edges[level - 1];
        }
        return;
    }
    const int lane = threadIdx.x & 31;
    const int warps = (nblocks * blockDim.x) >> 5;
    int maxdeg = 0;
    for (int r = (b * blockDim.x + threadIdx.x) >> 5; r < p; r += warps)
        maxdeg = max(maxdeg, recompact_row(G, p, adj, up, r, lane, elist, &st->edges[level], st));
    if (lane == 0) atomicMax(&st->max_degree[level], maxdeg);
}

__global__ void recompact_kernel(const uint16_t *__restrict__ G, int p, int *__restrict__ adj, int *__restrict__ up,
                                 DevState *st, int level, int2 *elist) {
    pdl_wait();
    pdl_trigger();
    recompact_blocks(G, p, adj, up, st, level, elist, (int)blockIdx.x, (int)gridDim.x);
}

template <typename T>
__global__ void row_scan_kernel(const T *__restrict__ cnt, int p, long long *__restrict__ prefix, DevState *st) {
    if (st->done) return;
    block_scan_rows(cnt, p, prefix);
}

// Level kernel of level L (1 <= L <= GCSL_GAUSS_REG_LEVELS): the edge phase over one
// resident wave of warps.  The unit kernel follows it when edges are chunked.
//
// Edges only shrink from level to level, so the previous level's edge count bounds this
// one's.  It was written by the (re)compaction of level L - 1, three or more kernels
// before this one: every kernel of the loop waits for its predecessor before it lets its
// successor start, so that compaction has completed when this kernel starts and the
// count can be read before the wait.  Blocks beyond the bound leave before loading the
// binomial rows (the upper levels keep a few hundred edges, and the grid is sized for
// the thousands of level 1); block 0 always stays, it records the end of the loop.
template <int L, bool MIXED>
__global__ void __launch_bounds__(256) gauss_level_reg_kernel(LevelCtx x) {
    __shared__ BinomRows sb;
    if (L >= 2 && blockIdx.x > 0 &&
        (long long)blockIdx.x * (blockDim.x >> 5) >= (long long)__ldcg(&x.st->edges[L - 1]))
        return;
    if (L >= 2) binom_rows_load(sb);  // constant table: before the wait on the previous kernel
    pdl_wait();
    pdl_trigger();
    if (L >= 2) __syncthreads();
    if (!level_active(x.st, L, x.tau_valid)) return;
    const long long n_edges = (long long)x.st->edges[L];  // filled by the (re)compaction
    if ((long long)blockIdx.x * (blockDim.x >> 5) >= n_edges) return;  // no edge for this block
    level_edge_phase<L, MIXED>(x, L >= 2 ? &sb : nullptr, ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                               ((long long)gridDim.x * blockDim.x) >> 5);
}

//
// The units of a level are known only when the level kernel has finished: blocks check
// their share after the wait; the binomial rows are loaded before it by the blocks that
// the level's edge count says will have work, after it by any other block with units.
template <int L, bool MIXED>
__global__ void __launch_bounds__(256) gauss_level_units_kernel(LevelCtx x) {
    __shared__ BinomRows sb;
    // blocks that will likely have units load the binomial rows before the wait, while the
    // level kernel still runs: after a quiet level every edge is handed over as about one
    // unit, so the level's edge count (written by the recompaction, which completed before
    // the level kernel released this one) bounds them
    const bool early = L >= 2 && (long long)blockIdx.x * (blockDim.x >> 5) < (long long)__ldcg(&x.st->edges[L]);
    if (early) binom_rows_load(sb);
    pdl_wait();
    pdl_trigger();
    if (!level_active(x.st, L, x.tau_valid)) return;
    const long long reserved = (long long)x.st->units[L];
    const long long nu = reserved < x.ck.unit_cap ? reserved : x.ck.unit_cap;
    if ((long long)blockIdx.x * (blockDim.x >> 5) >= nu) return;
    if (L >= 2) {
        if (!early) binom_rows_load(sb);
        __syncthreads();
    }
    level_unit_phase<L, MIXED>(x, L >= 2 ? &sb : nullptr, ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5,
                               ((long long)gridDim.x * blockDim.x) >> 5);
}

// FP64 evaluation of the z* candidates queued by the mixed level-L kernel (one thread
// per entry; entries beyond the queue's capacity were evaluated in the level kernel).
// One warp per block: the few thousand entries of a level spread over every SM's FP64
// pipe instead of filling a handful of SMs.
struct CandArgs {
    const double *C;
    int p;
    double tau, t2;
    const int *q;
    long long cap;
    const unsigned long long *count;
    double *zmin, *r2min;
    const long long *chunk_first;  // canonical removers of the level's chunked edges
};

template <int L>
__device__ __forceinline__ void cand_threads(const CandArgs &a, long long t0, long long stride) {
    constexpr int W = CAND_HEADER + L;
    const long long used = (long long)*a.count;
    const long long n = (used < a.cap ? used : a.cap) / W;
    for (long long t = t0; t < n; t += stride)
        eval_candidate<L>(a.C, a.p, a.q + t * W, a.tau, a.t2, a.zmin, a.r2min, a.chunk_first);
}

template <int L>
__global__ void __launch_bounds__(32) gauss_cand_kernel(CandArgs a) {
    cand_threads<L>(a, (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x);
}



// ---------------------------------------------------------- level l, any L
// One warp per edge, one test at a time in key order; the (L+2)-dimensional lower
// triangle lives in shared memory and the lanes split each elimination step.
__global__ void __launch_bounds__(128) gauss_level_smem_kernel(const double *__restrict__ C, int p,
                                                              const int *__restrict__ adj,
                                                              const int *__restrict__ up,
                                                              const long long *__restrict__ prefix, int L,
                                                              double tau, bool tau_valid, uint16_t *G,
                                                              double *zmin, int *sep_dense, int max_level,
                                                              int *rec_pool, long long rec_cap, DevState *st) {
    extern __shared__ double smem[];
    if (!level_active(st, L, tau_valid)) return;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int D = L + 2;
    const int tri = D * (D + 1) / 2;
    double *A = smem + (size_t)wib * (tri + 2);
    int *S = reinterpret_cast<int *>(smem + (size_t)(blockDim.x >> 5) * (tri + 2)) + wib * (GCSL_MAX_LEVELS + 2);
    const long long n_edges = prefix[p];
    const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
    unsigned long long n_tests = 0, n_full = 0, n_removed = 0;
    for (long long e = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < n_edges; e += warps) {
        EdgeJob J;
        if (!load_edge<0>(adj, up, prefix, p, e, L, J)) {
            if (lane == 0) set_status(st, GCSL_ERR_UNSUPPORTED);
            continue;
        }
        n_full += J.T;
        double zl = __longlong_as_double(0x7ff0000000000000ll);
        bool removed = false;
        for (long long m = 0; m < J.T; ++m) {
            long long rank;
            int dir;
            key_of(J, m, rank, dir);
            const int vi = dir ? J.hi : J.lo, vj = dir ? J.lo : J.hi;
            if (lane == 0) {
                unrank_positions_rt(L, (dir ? J.deg_hi : J.deg_lo) - 1, rank, S);
                const int *nbrs = adj + (size_t)vi * p + 1;
                for (int c = 0; c < L; ++c) S[c] = resolve_position(nbrs, vj, S[c]);
                S[L] = vi;
                S[L + 1] = vj;
            }
            __syncwarp();
            // lower triangle of the augmented matrix; index r < L is S_r, L is v_i,
            // L + 1 is v_j; unit diagonal for v_i, v_j and C[v_i, v_j] below it.
            for (int r = 0; r < D; ++r) {
                for (int c = lane; c <= r; c += 32) {
                    double v;
                    if (r == c && r >= L) v = 1.0;
                    else if (r == L + 1 && c == L) v = __ldg(C + (size_t)vi * p + vj);
                    else v = __ldg(C + (size_t)S[r] * p + S[c]);
                    A[r * (r + 1) / 2 + c] = v;
                }
            }
            __syncwarp();
            for (int j = 0; j < L; ++j) {
                const double d = sqrt(A[j * (j + 1) / 2 + j]);
                const double inv = 1.0 / d;
                __syncwarp();
                for (int i = j + 1 + lane; i < D; i += 32) A[i * (i + 1) / 2 + j] *= inv;
                __syncwarp();
                // trailing update of rows/cols > j
                const int nt = D - j - 1;
                const int cnt = nt * (nt + 1) / 2;
                (void)cnt;
                for (int ii = j + 1; ii < D; ++ii) {
                    const double lij = A[ii * (ii + 1) / 2 + j];
                    for (int kk = j + 1 + lane; kk <= ii; kk += 32)
                        A[ii * (ii + 1) / 2 + kk] -= lij * A[kk * (kk + 1) / 2 + j];
                }
                __syncwarp();
            }
            const double h00 = A[L * (L + 1) / 2 + L];
            const double h01 = A[(L + 1) * (L + 2) / 2 + L];
            const double h11 = A[(L + 1) * (L + 2) / 2 + L + 1];
            const double rho = h01 / (sqrt(fabs(h00)) * sqrt(fabs(h11)));
            const double z = fabs(0.5 * (log(fabs(1.0 + rho)) - log(fabs(1.0 - rho))));
            ++n_tests;
            if (!isnan(z)) zl = fmin(zl, z);
            if (z < tau) {
                if (lane == 0) write_removal(J, L, S, p, max_level, G, sep_dense, rec_pool, rec_cap, st);
                removed = true;
            }
            __syncwarp();
            if (removed) break;
        }
        if (lane == 0) {
            double *zp = zmin + (size_t)J.lo * p + J.hi;
            *zp = fmin(*zp, zl);
            n_removed += removed;
        }
    }
    if (lane == 0) {
        atomicAdd(&st->tests[L < GCSL_MAX_LEVELS ? L : GCSL_MAX_LEVELS - 1], n_tests);
        atomicAdd(&st->tests_full[L < GCSL_MAX_LEVELS ? L : GCSL_MAX_LEVELS - 1], n_full);
        atomicAdd(&st->removed[L < GCSL_MAX_LEVELS ? L : GCSL_MAX_LEVELS - 1], n_removed);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) st->edges[L < GCSL_MAX_LEVELS ? L : GCSL_MAX_LEVELS - 1] = n_edges;
}

// ------------------------------------------------------------ zmin -> pmax
// pmax_ij = 2 * sf(sqrt(n - 3) * z*_ij) for i < j (0 when z* = +inf), -1 elsewhere.
// 2 sf(x) = erfc(x / sqrt 2), written as scipy's ndtr does it (erf below 1/sqrt 2).
// Grid: (column blocks of 256, rows); no index division.
// The erfc Taylor table of the pmax kernels, built once per solve by one warp.
__global__ void sf_table_kernel(double *__restrict__ out) {
    __shared__ double tab[SF_CENTRES][SF_TERMS];
    sf_table_build(tab);
    __syncthreads();
    for (int k = threadIdx.x; k < SF_CENTRES * SF_TERMS; k += blockDim.x) out[k] = (&tab[0][0])[k];
}

// Pairs kept at level 0 (the list the level-0 kernel appended): z* = min(zmin, Z of the
// smallest rho^2 any later level stored), pmax = 2 sf(sqrt(n - 3) z*)
// (helpers.py:62-82 with the FP64 z*).
__global__ void pmax_kept_kernel(const int *__restrict__ kept, const DevState *__restrict__ st,
                                 const double *__restrict__ zmin, const double *__restrict__ r2min, double sqrt_nm3,
                                 const double *__restrict__ sftab, double *__restrict__ pmax) {
    __shared__ double tab[SF_CENTRES][SF_TERMS];
    sf_table_load(tab, sftab);
    __syncthreads();
    const int count = st->n_kept;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < count; t += gridDim.x * blockDim.x) {
        const int k = kept[t];
        double z = zmin[k];
        const double r2 = r2min[k];
        if (r2 < 1.0) z = fmin(z, fisher_z(sqrt(r2)));  // Z increasing in rho^2 below 1
        pmax[k] = two_sf_tab(sqrt_nm3 * z, tab);
    }
}

// Every other entry: pairs removed at level 0 (marker zmin = -1) get z* = Z(r) with
// r = C[i*p + j] (gaussian_ci.cu:36-37), the lower triangle and diagonal -1.  Launched on
// a second stream right after level 0; the later levels never touch these entries, so it
// runs concurrently with them.
__global__ void pmax_level0_kernel(const double *__restrict__ C, const double *__restrict__ zmin, int p,
                                   double sqrt_nm3, const double *__restrict__ sftab, double *__restrict__ pmax) {
    __shared__ double tab[SF_CENTRES][SF_TERMS];
    sf_table_load(tab, sftab);
    __syncthreads();
    const unsigned total = (unsigned)p * (unsigned)p;  // p <= 46340: fits in 31 bits
    for (unsigned k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x) {
        const int i = (int)(k / (unsigned)p), j = (int)(k - (unsigned)i * (unsigned)p);
        if (i >= j) {
            pmax[k] = -1.0;
        } else if (zmin[k] < 0.0) {
            pmax[k] = two_sf_tab(sqrt_nm3 * fisher_z(C[k]), tab);
        }
    }
}

// Unit kernel: all positions of ranks [0, count) (one thread per rank).
__global__ void unrank_kernel(int K, int L, long long count, int *out) {
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < count;
         r += (long long)gridDim.x * blockDim.x)
        unrank_positions_rt(L, K, r, out + r * L);
}

// ------------------------------------------------------------- host launchers
namespace host {

cudaError_t launch_level0(const double *C, int p, double tau0, uint16_t *G, double *zmin, double *r2min, int *kept,
                          DevState *st, float *C32, cudaStream_t s) {
    const int nb = (p + 31) / 32;
    const double t0 = tanh(tau0);
    gauss_level0_kernel<<<nb * (nb + 1) / 2, 256, 0, s>>>(C, p, tau0, level0_bounds(t0 * t0), G, zmin, r2min, kept,
                                                         st, C32);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_compact(const uint16_t *G, int p, int *adj, int *up, DevState *st, int level, int2 *elist,
                           cudaStream_t s) {
    const int threads = 256, wpb = threads / 32;
    int blocks = (p + wpb - 1) / wpb;
    const cudaError_t e = launch_pdl(compact_kernel, dim3(blocks), dim3(threads), 0, s, G, p, adj, up, st, level, elist);
    note_launch(1);
    return e;
}

cudaError_t launch_recompact(const uint16_t *G, int p, int *adj, int *up, DevState *st, int level, int2 *elist,
                             cudaStream_t s) {
    const int threads = 256, wpb = threads / 32;
    const cudaError_t e =
        launch_pdl(recompact_kernel, dim3((p + wpb - 1) / wpb), dim3(threads), 0, s, G, p, adj, up, st, level, elist);
    note_launch(1);
    return e;
}

cudaError_t launch_scan_int(const int *cnt, int p, long long *prefix, DevState *st, cudaStream_t s) {
    row_scan_kernel<int><<<1, 1024, 0, s>>>(cnt, p, prefix, st);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_scan_ll(const long long *cnt, int p, long long *prefix, DevState *st, cudaStream_t s) {
    row_scan_kernel<long long><<<1, 1024, 0, s>>>(cnt, p, prefix, st);
    note_launch(1);
    return cudaGetLastError();
}

// The level's context (thresholds, FP32 bounds of the knife edge, queue) for launches.
LevelCtx level_ctx(int L, const double *C, int p, const int *adj, const int2 *elist, double tau, bool tau_valid,
                   uint16_t *G, double *zmin, double *r2min, int *sep_dense, int max_level, int *rec_pool,
                   long long rec_cap, DevState *st, const float *C32, int *qbuf, long long qcap,
                   const ChunkBufs &ck) {
    LevelCtx x;
    x.order = work_order_seed();
    x.C = C;
    x.p = p;
    x.adj = adj;
    x.elist = elist;
    x.tau = tau;
    const double th = tanh(tau);
    x.t2 = th * th;  // Z < tau  <=>  rho^2 < tanh(tau)^2 for |rho| < 1
    x.tau_valid = tau_valid;
    x.G = G;
    x.zmin = zmin;
    x.r2min = r2min;
    x.sep_dense = sep_dense;
    x.max_level = max_level;
    x.rec_pool = rec_pool;
    x.rec_cap = rec_cap;
    x.st = st;
    x.mix.C32 = C32;
    // FP32 bounds of the FP64 knife edge [t2 (1 - 1e-12), t2 (1 + 1e-12)], rounded outward
    x.mix.t2lo = nextafterf((float)(x.t2 * (1.0 - 2e-12)), 0.0f);
    x.mix.t2hi = nextafterf((float)(x.t2 * (1.0 + 2e-12)), 2.0f);
    x.mix.q.buf = qbuf;
    x.mix.q.cap = qcap;
    x.mix.q.count = &st->cand_ints[L < GCSL_MAX_LEVELS ? L : 0];
    x.ck = ck;
    return x;
}

cudaError_t launch_gauss_level(int L, const double *C, int p, const int *adj, const int *up, const int2 *elist,
                               const long long *prefix, double tau, bool tau_valid, uint16_t *G, double *zmin,
                               double *r2min, int *sep_dense, int max_level, int *rec_pool, long long rec_cap,
                               DevState *st, int num_sms, const float *C32, int *qbuf, long long qcap,
                               const ChunkBufs &ck, cudaStream_t s) {
    // register-heavy upper levels run 128-thread blocks
    const int threads = L >= 4 ? 128 : 256;
    const int blocks = num_sms * 8;
    const bool mixed = C32 != nullptr && qbuf != nullptr;
    const LevelCtx x = level_ctx(L, C, p, adj, elist, tau, tau_valid, G, zmin, r2min, sep_dense, max_level, rec_pool,
                                 rec_cap, st, C32, qbuf, qcap, ck);
    // chunked edges: the unit kernel follows the level kernel (it returns at once when no
    // edge was chunked).  Both kernels launch 8 blocks per SM whose warps stride over the
    // edges / units: more than one resident wave at every level's register count, so blocks
    // of later waves pick up the work of the slow ones (measured on p = 1000: 0.771 ms per
    // solve against 0.801 ms with one resident wave and 0.80 / 0.85 ms with 16 / 32 per SM)
    cudaError_t el = cudaSuccess;
#define GCSL_LVL(K)                                                                                      \
    case K:                                                                                              \
        if (mixed) {                                                                                     \
            el = launch_pdl(gauss_level_reg_kernel<K, true>, dim3(blocks), dim3(threads), 0, s, x);      \
            if (el == cudaSuccess && ck.heavy != nullptr)                                                \
                el = launch_pdl(gauss_level_units_kernel<K, true>, dim3(blocks), dim3(threads), 0, s, x); \
        } else {                                                                                         \
            el = launch_pdl(gauss_level_reg_kernel<K, false>, dim3(blocks), dim3(threads), 0, s, x);     \
            if (el == cudaSuccess && ck.heavy != nullptr)                                                \
                el = launch_pdl(gauss_level_units_kernel<K, false>, dim3(blocks), dim3(threads), 0, s, x); \
        }                                                                                                \
        if (ck.heavy != nullptr) note_launch(1);                                                         \
        if (el != cudaSuccess) return note_error("gauss level kernel launch", el);                       \
        break;
    switch (L) {
        GCSL_LVL(1)
        GCSL_LVL(2)
        GCSL_LVL(3)
        GCSL_LVL(4)
        GCSL_LVL(5)
        GCSL_LVL(6)
        GCSL_LVL(7)
        GCSL_LVL(8)
        GCSL_LVL(9)
        GCSL_LVL(10)
        GCSL_LVL(11)
        GCSL_LVL(12)
    default: {
        const int t = 128, wpb = t / 32;
        const int D = L + 2;
        const size_t smem = (size_t)wpb * (D * (D + 1) / 2 + 2) * sizeof(double) +
                            (size_t)wpb * (GCSL_MAX_LEVELS + 2) * sizeof(int);
        static std::atomic<unsigned long long> limit_set{0};
        if (smem > 48 * 1024) {
            const cudaError_t ea = raise_dyn_smem_limit(gauss_level_smem_kernel, limit_set);
            if (ea != cudaSuccess) return note_error("gauss_level_smem_kernel shared memory", ea);
        }
        gauss_level_smem_kernel<<<num_sms * 4, t, smem, s>>>(C, p, adj, up, prefix, L, tau, tau_valid, G, zmin,
                                                               sep_dense, max_level, rec_pool, rec_cap, st);
    }
    }
#undef GCSL_LVL
    note_launch(1);
    return cudaGetLastError();
}

static CandArgs cand_args(int L, const double *C, int p, double tau, double *zmin, double *r2min, const int *qbuf,
                          long long qcap, DevState *st, const long long *chunk_first) {
    const double th = tanh(tau);
    CandArgs a;
    a.C = C;
    a.p = p;
    a.tau = tau;
    a.t2 = th * th;
    a.q = qbuf;
    a.cap = qcap;
    a.count = &st->cand_ints[L];
    a.zmin = zmin;
    a.r2min = r2min;
    a.chunk_first = chunk_first;
    return a;
}

// FP64 z* candidates of mixed level L (1 <= L <= GCSL_GAUSS_REG_LEVELS) on their own.
cudaError_t launch_cand(int L, const double *C, int p, double tau, double *zmin, double *r2min, const int *qbuf,
                        long long qcap, DevState *st, const long long *chunk_first, int num_sms, cudaStream_t s) {
    const CandArgs a = cand_args(L, C, p, tau, zmin, r2min, qbuf, qcap, st, chunk_first);
    switch (L) {
#define GCSL_CAND(K) \
    case K: gauss_cand_kernel<K><<<num_sms * 16, 32, 0, s>>>(a); break;
        GCSL_CAND(1) GCSL_CAND(2) GCSL_CAND(3) GCSL_CAND(4) GCSL_CAND(5) GCSL_CAND(6)
        GCSL_CAND(7) GCSL_CAND(8) GCSL_CAND(9) GCSL_CAND(10) GCSL_CAND(11) GCSL_CAND(12)
#undef GCSL_CAND
    default: return cudaSuccess;
    }
    note_launch(1);
    return cudaGetLastError();
}


cudaError_t launch_unrank(int K, int L, long long count, int *out, cudaStream_t s) {
    const long long blocks = (count + 127) / 128;
    unrank_kernel<<<(int)(blocks > 0 ? (blocks < 65535 ? blocks : 65535) : 1), 128, 0, s>>>(K, L, count, out);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_sf_table(double *out, cudaStream_t s) {
    sf_table_kernel<<<1, 32, 0, s>>>(out);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_pmax_level0(const double *C, const double *zmin, int p, long long n_obs, const double *sftab,
                               double *pmax, int num_sms, cudaStream_t s) {
    const long long total = (long long)p * p;
    const long long want = (total + 255) / 256;
    const int blocks = (int)(want < (long long)num_sms * 4 ? want : (long long)num_sms * 4);
    pmax_level0_kernel<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(C, zmin, p, sqrt((double)(n_obs - 3)), sftab, pmax);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_pmax(const int *kept, const DevState *st, const double *zmin, const double *r2min, int p,
                        long long n_obs, const double *sftab, double *pmax, int num_sms, cudaStream_t s) {
    const long long pairs = (long long)p * (p - 1) / 2;
    const long long want = (pairs + 255) / 256;
    const int blocks = (int)(want < (long long)num_sms * 2 ? want : (long long)num_sms * 2);
    pmax_kept_kernel<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(kept, st, zmin, r2min, sqrt((double)(n_obs - 3)), sftab,
                                                             pmax);
    note_launch(1);
    return cudaGetLastError();
}

}  // namespace host
}  // namespace gcsl
