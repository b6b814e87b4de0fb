// Gaussian PC-stable skeleton kernels for sm_103a.
//
//   level 0        gauss_level0_kernel     (reference: gpucsl/pc/cuda/gaussian_ci.cu:18-51)
//   compaction     compact_kernel          (reference: gpucsl/pc/cuda/helpers/graph_helpers.cu:35-56)
//   edge prefix    row_scan_kernel
//   level l <= 12  gauss_level_reg_kernel  (reference: gaussian_ci.cu:66-120,
//                                           helpers/gaussian_helpers.cu:240-262)
//   level l > 12   gauss_level_smem_kernel
//   zmin -> pmax   pmax_level0_kernel, pmax_kept_kernel (reference: gpucsl/pc/helpers.py:62-82)
//
// Work decomposition of a level: one warp owns one undirected edge {lo, hi} alive at
// level start and walks the merged key sequence of both directions, key = (rank, dir)
// with dir 0 for v_i = lo, 32 keys per step (one test per lane).  The warp stops after
// the first step that contains a removing test; the lowest removing lane is the
// canonical remover (its set is the sepset) and z* folds the keys up to it.  Because
// the warp owns the edge for the whole level, the skeleton, sepset and zmin writes
// need no atomics, and the result does not depend on scheduling.
#include "common.cuh"

namespace gcsl {

// ----------------------------------------------------------------- level 0
// 32 x 32 tiles of the upper triangle (tile row bi <= tile column bj): for i < j,
// Z = |0.5 log|(1+r)/(1-r)||, r = C[i*p + j]; remove iff Z < tau0.  Kept pairs store
// z* = Z (NaN ignored) and append i * p + j to `kept`; removed pairs store the marker
// -1: their z* is final and their pmax is computed from C by pmax_level0_kernel,
// concurrently with the later levels.
// The mirrored skeleton entries are written through a shared-memory transpose so both
// triangles are stored row-contiguously; zero diagonal.
__global__ void gauss_level0_kernel(const double *__restrict__ C, int p, double tau0, double t0sq,
                                    uint16_t *__restrict__ G, double *__restrict__ zmin, int *__restrict__ kept,
                                    DevState *st) {
    __shared__ uint16_t tg[32][33];
    const int nb = (p + 31) / 32;
    int rem = blockIdx.x, bi = 0;
    while (rem >= nb - bi) {
        rem -= nb - bi;
        ++bi;
    }
    const int bj = bi + rem;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 8 rows per pass
    unsigned long long removed = 0;
    for (int r = ty; r < 32; r += 8) {
        const int i = bi * 32 + r, j = bj * 32 + tx;
        uint16_t g = 0;
        if (i < p && j < p && i < j) {
            const double c = __ldg(C + (size_t)i * p + j);
            // Z0 = atanh-like in |r| on [0, 1): Z0 < tau0 <=> r^2 < tanh(tau0)^2; the knife
            // edge, |r| >= 1 and NaN take the reference formula
            const double r2 = c * c;
            bool rem0;
            double z = -1.0;  // marker: z* of a level-0 removal is finished on the side stream
            if (r2 < 1.0 && fabs(r2 - t0sq) > 1e-12 * t0sq) {
                rem0 = r2 < t0sq;
                if (!rem0) z = fabs(0.5 * log(fabs((1.0 + c) / (1.0 - c))));
            } else {
                z = fabs(0.5 * log(fabs((1.0 + c) / (1.0 - c))));
                rem0 = z < tau0;
                if (rem0) z = -1.0;
            }
            g = rem0 ? 0 : 1;
            zmin[(size_t)i * p + j] = isnan(z) ? __longlong_as_double(0x7ff0000000000000ll) : z;
            removed += rem0;
        }
        // kept pairs join the list whose pmax is finished after the last level
        const unsigned km = __ballot_sync(GCSL_FULL_MASK, g != 0 && i < j);
        if (km) {
            int base = 0;
            if (tx == 0) base = atomicAdd(&st->n_kept, __popc(km));
            base = __shfl_sync(GCSL_FULL_MASK, base, 0);
            if (g != 0 && i < j) kept[base + __popc(km & ((1u << tx) - 1u))] = i * p + j;
        }
        if (i < p && j < p && (bi != bj || i <= j)) G[(size_t)i * p + j] = g;  // includes the zero diagonal
        tg[r][tx] = g;
    }
    __syncthreads();
    if (bi != bj) {
        for (int r = ty; r < 32; r += 8) {
            const int j = bj * 32 + r, i = bi * 32 + tx;  // lower triangle (j, i), j > i
            if (i < p && j < p) G[(size_t)j * p + i] = tg[tx][r];
        }
    } else {
        for (int r = ty; r < 32; r += 8) {
            const int j = bj * 32 + r, i = bi * 32 + tx;
            if (i < p && j < p && j > i) G[(size_t)j * p + i] = tg[tx][r];
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) removed += __shfl_xor_sync(GCSL_FULL_MASK, removed, o);
    if ((threadIdx.x & 31) == 0 && removed) atomicAdd(&st->removed[0], removed);
}

// ------------------------------------------------------------- compaction
// Warp per row r: adj[r*p] = degree, adj[r*p + 1 ..] = ascending neighbour ids
// (entries past the degree keep stale values, as in the reference); also writes
// up[r] = #neighbours > r and the level's max degree.  Returns at once when the level
// loop is already finished.
__global__ void compact_kernel(const uint16_t *__restrict__ G, int p, int *__restrict__ adj, int *__restrict__ up,
                               DevState *st, int level) {
    if (st != nullptr && st->done) return;
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    int maxdeg = 0;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < p; r += warps) {
        const uint16_t *Gr = G + (size_t)r * p;
        int *row = adj + (size_t)r * p;
        int cnt = 0, ups = 0;
        for (int c0 = 0; c0 < p; c0 += 32) {
            const int c = c0 + lane;
            const bool e = (c < p) && (c != r) && (Gr[c] != 0);
            const unsigned b = __ballot_sync(GCSL_FULL_MASK, e);
            if (e) row[1 + cnt + __popc(b & ((1u << lane) - 1))] = c;
            cnt += __popc(b);
            ups += __popc(__ballot_sync(GCSL_FULL_MASK, e && c > r));
        }
        if (lane == 0) {
            row[0] = cnt;
            if (up != nullptr) up[r] = ups;
        }
        maxdeg = max(maxdeg, cnt);
    }
    if (lane == 0 && st != nullptr) atomicMax(&st->max_degree[level], maxdeg);
}

// Levels >= 2: each warp refilters one row's previous neighbour list against G (rows
// only shrink, so this touches deg entries instead of p), writing up[r] and the max
// degree; row_scan_kernel then rebuilds the edge prefix.
__global__ void recompact_kernel(const uint16_t *__restrict__ G, int p, int *__restrict__ adj, int *__restrict__ up,
                                 DevState *st, int level) {
    if (st->done) return;
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    int maxdeg = 0;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < p; r += warps) {
        int *row = adj + (size_t)r * p;
        const int deg = row[0];
        int cnt = 0, ups = 0;
        for (int k0 = 0; k0 < deg; k0 += 32) {
            const int k = k0 + lane;
            const int c = k < deg ? row[1 + k] : 0;
            const bool keep = k < deg && G[(size_t)r * p + c] != 0;
            const unsigned b = __ballot_sync(GCSL_FULL_MASK, keep);
            __syncwarp();  // every read of this 32-entry window precedes the writes below
            if (keep) row[1 + cnt + __popc(b & ((1u << lane) - 1))] = c;
            cnt += __popc(b);
            ups += __popc(__ballot_sync(GCSL_FULL_MASK, keep && c > r));
        }
        if (lane == 0) {
            row[0] = cnt;
            up[r] = ups;
        }
        maxdeg = max(maxdeg, cnt);
    }
    if (lane == 0) atomicMax(&st->max_degree[level], maxdeg);
}

// Single-block exclusive scan of a per-row count (int or weighted long long) into
// prefix[0..p]; prefix[p] is the total.
template <typename T>
__global__ void row_scan_kernel(const T *__restrict__ cnt, int p, long long *__restrict__ prefix, DevState *st) {
    if (st->done) return;
    __shared__ long long warp_tot[32];
    const int tid = threadIdx.x, nt = blockDim.x;
    const int per = (p + nt - 1) / nt;
    const int b = tid * per, e = min(p, b + per);
    long long s = 0;
    for (int i = b; i < e; ++i) s += (long long)cnt[i];
    // inclusive scan of s across the block
    long long v = s;
    const int lane = tid & 31, w = tid >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        long long t = __shfl_up_sync(GCSL_FULL_MASK, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) warp_tot[w] = v;
    __syncthreads();
    if (w == 0) {
        long long t = (lane < (nt >> 5)) ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            long long u = __shfl_up_sync(GCSL_FULL_MASK, t, o);
            if (lane >= o) t += u;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    long long base = v - s + (w > 0 ? warp_tot[w - 1] : 0);
    for (int i = b; i < e; ++i) {
        prefix[i] = base;
        base += (long long)cnt[i];
    }
    if (tid == nt - 1) prefix[p] = base;
}

// ---------------------------------------------------------- level l, L <= 12
// One CI test: Gaussian elimination without square roots on the lower triangle of the
// augmented matrix [[C_SS, C_S,vi, C_S,vj], [., 1, C_vi,vj], [., ., 1]].  After the L
// pivots of C_SS the trailing 2x2 block is H = M0 - M1 M2^-1 M1^T of
// gaussian_helpers.cu:78-89, and rho^2 = H01^2 / (|H00| |H11|).
//
// The statistic Z = |0.5 (log|1 + rho| - log|1 - rho|)| increases with |rho| on [0, 1),
// so "Z < tau" is "rho^2 < tanh(tau)^2" there and no logarithm is needed per test.  For
// |rho| >= 1 (Z decreases again), NaN, or rho^2 within 1e-12 of the threshold, Z is
// evaluated with the reference's formula and compared with tau directly.
struct TestOut {
    double rho2;   // rho^2 when the monotone branch decided, +inf otherwise
    double zexact; // Z from the reference formula when evaluated, +inf otherwise (NaN kept)
    bool remove;
};

__device__ __forceinline__ double z_of_rho(double rho) {
    return fabs(0.5 * (log(fabs(1.0 + rho)) - log(fabs(1.0 - rho))));
}

template <int L>
__device__ __forceinline__ TestOut gauss_test_reg(const double *__restrict__ C, int p, int vi, int vj, const int *S,
                                                  double tau, double t2) {
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    if constexpr (L == 1) {
        // closed form: with m = C_ss, a = C_vi,s, b = C_vj,s, r = C_vi,vj the trailing block
        // times m is [[m - a^2, r m - a b], [., m - b^2]]; the decision compares
        // num = (r m - a b)^2 with t^2 den, den = |m - a^2| |m - b^2|, without a division
        const double m = __ldg(C + (size_t)S[0] * p + S[0]);
        const double a = __ldg(C + (size_t)vi * p + S[0]);
        const double b = __ldg(C + (size_t)vj * p + S[0]);
        const double r = __ldg(C + (size_t)vi * p + vj);
        const double d00 = fma(-a, a, m), d11 = fma(-b, b, m);
        const double n01 = fma(r, m, -(a * b));
        const double num = n01 * n01, den = fabs(d00) * fabs(d11);
        TestOut o;
        const double tden = t2 * den;
        if (num < den && fabs(num - tden) > 1e-12 * tden) {
            o.rho2 = num / den;
            o.zexact = inf;
            o.remove = num < tden;
        } else {
            const double z = z_of_rho(n01 / (sqrt(fabs(d00)) * sqrt(fabs(d11))));
            o.rho2 = inf;
            o.zexact = z;
            o.remove = z < tau;
        }
        return o;
    }
    constexpr int D = L + 2;
    double A[D * (D + 1) / 2];  // row-packed lower triangle; rows 0..L-1 = S, L = v_i, L+1 = v_j
#pragma unroll
    for (int r = 0; r < L; ++r) {
        const double *Cr = C + (size_t)S[r] * p;
#pragma unroll
        for (int c = 0; c <= r; ++c) A[r * (r + 1) / 2 + c] = __ldg(Cr + S[c]);
        A[L * (L + 1) / 2 + r] = __ldg(C + (size_t)vi * p + S[r]);
        A[(L + 1) * (L + 2) / 2 + r] = __ldg(C + (size_t)vj * p + S[r]);
    }
    A[L * (L + 1) / 2 + L] = 1.0;
    A[(L + 1) * (L + 2) / 2 + L] = __ldg(C + (size_t)vi * p + vj);
    A[(L + 1) * (L + 2) / 2 + L + 1] = 1.0;
#pragma unroll
    for (int j = 0; j < L; ++j) {
        const double inv = 1.0 / A[j * (j + 1) / 2 + j];
#pragma unroll
        for (int i = j + 1; i < D; ++i) {
            const double t = A[i * (i + 1) / 2 + j] * inv;
#pragma unroll
            for (int k = j + 1; k <= i; ++k) A[i * (i + 1) / 2 + k] -= t * A[k * (k + 1) / 2 + j];
        }
    }
    const double h00 = A[L * (L + 1) / 2 + L];
    const double h01 = A[(L + 1) * (L + 2) / 2 + L];
    const double h11 = A[(L + 1) * (L + 2) / 2 + L + 1];
    const double rho2 = (h01 * h01) / (fabs(h00) * fabs(h11));
    TestOut o;
    if (rho2 < 1.0 && fabs(rho2 - t2) > 1e-12 * t2) {
        o.rho2 = rho2;
        o.zexact = inf;
        o.remove = rho2 < t2;
    } else {
        const double z = z_of_rho(h01 / (sqrt(fabs(h00)) * sqrt(fabs(h11))));
        o.rho2 = inf;
        o.zexact = z;
        o.remove = z < tau;
    }
    return o;
}

struct EdgeJob {
    int lo, hi, deg_lo, deg_hi;
    long long R0, R1, T, Rmin;
    int longer;
};

template <int KMAX>
__device__ __forceinline__ bool load_edge(const int *__restrict__ adj, const int *__restrict__ up,
                                          const long long *__restrict__ prefix, int p, long long e, int L,
                                          EdgeJob &J) {
    const int i = upper_row(prefix, p, e);
    const long long k = e - prefix[i];
    const int *row = adj + (size_t)i * p;
    const int deg = row[0];
    const int j = row[1 + (deg - up[i]) + (int)k];
    J.lo = i;
    J.hi = j;
    J.deg_lo = deg;
    J.deg_hi = adj[(size_t)j * p];
    const int K0 = J.deg_lo - 1, K1 = J.deg_hi - 1;
    J.R0 = (K0 >= L) ? (KMAX > 0 ? binom_small<KMAX>(K0, L) : binom_rt(K0, L)) : 0;
    J.R1 = (K1 >= L) ? (KMAX > 0 ? binom_small<KMAX>(K1, L) : binom_rt(K1, L)) : 0;
    J.T = J.R0 + J.R1;
    J.Rmin = J.R0 < J.R1 ? J.R0 : J.R1;
    J.longer = J.R0 > J.R1 ? 0 : 1;
    return J.R0 < GCSL_RANK_LIMIT && J.R1 < GCSL_RANK_LIMIT;
}

// merged key index m -> (rank, dir)
__device__ __forceinline__ void key_of(const EdgeJob &J, long long m, long long &rank, int &dir) {
    if (m < 2 * J.Rmin) {
        rank = m >> 1;
        dir = (int)(m & 1);
    } else {
        rank = m - J.Rmin;
        dir = J.longer;
    }
}

__device__ __forceinline__ void write_removal(const EdgeJob &J, int L, const int *S, int p, int max_level,
                                              uint16_t *G, int *sep_dense, int *rec_pool, long long rec_cap,
                                              DevState *st) {
    G[(size_t)J.lo * p + J.hi] = 0;
    G[(size_t)J.hi * p + J.lo] = 0;
    if (sep_dense != nullptr && L <= max_level) {
        for (int k = 0; k < L; ++k) {
            sep_dense[((size_t)J.lo * p + J.hi) * max_level + k] = S[k];
            sep_dense[((size_t)J.hi * p + J.lo) * max_level + k] = S[k];
        }
    }
    if (rec_pool != nullptr) {
        const unsigned long long off = atomicAdd(&st->n_rec_ints, (unsigned long long)(3 + L));
        if ((long long)(off + 3 + L) <= rec_cap) {
            rec_pool[off] = J.lo;
            rec_pool[off + 1] = J.hi;
            rec_pool[off + 2] = L;
            for (int k = 0; k < L; ++k) rec_pool[off + 3 + k] = S[k];
        } else {
            set_status(st, GCSL_ERR_CAPACITY);
        }
    }
}

// Common level entry: stop when the loop is finished or the level cannot run.
__device__ __forceinline__ bool level_active(DevState *st, int level, bool tau_valid) {
    if (st->done) return false;
    const int md = st->max_degree[level];
    if (md - 1 < level) {
        if (blockIdx.x == 0 && threadIdx.x == 0) st->done = 1;
        return false;
    }
    if (!tau_valid) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            set_status(st, GCSL_ERR_UNSUPPORTED_LEVEL);
            st->done = 1;
        }
        return false;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) st->last_level = level;
    return true;
}

// Min over the G-lane group (aligned groups of G lanes inside the warp).
template <int G>
__device__ __forceinline__ double group_min(double v) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(GCSL_FULL_MASK, v, o));
    return v;
}

// Level kernel: groups of G lanes each own one edge (32 / G edges per warp) and walk its
// merged key sequence G keys at a time.  Small groups keep the FP64 pipe busy at the
// upper levels, where an edge has only a handful of candidate sets, and stop at most
// G - 1 tests past the first remover.
template <int L, int G>
__global__ void __launch_bounds__(256) gauss_level_reg_kernel(const double *__restrict__ C, int p,
                                                             const int *__restrict__ adj, const int *__restrict__ up,
                                                             const long long *__restrict__ prefix, double tau,
                                                             double t2, bool tau_valid, uint16_t *G_, double *zmin,
                                                             double *r2min_pair, int *sep_dense, int max_level,
                                                             int *rec_pool, long long rec_cap, DevState *st) {
    if (!level_active(st, L, tau_valid)) return;
    constexpr int GPW = 32 / G;  // groups per warp
    const int lane = threadIdx.x & 31, gl = lane & (G - 1), gw = lane / G;
    const unsigned gshift = (unsigned)(gw * G);
    const unsigned gbits = (G == 32) ? 0xffffffffu : ((1u << G) - 1u);
    const long long n_edges = prefix[p];
    const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    unsigned long long n_tests = 0, n_full = 0, n_removed = 0;
    for (long long e0 = (((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * GPW; e0 < n_edges;
         e0 += warps * GPW) {
        const long long e = e0 + gw;
        EdgeJob J;
        J.T = 0;
        bool has = e < n_edges;
        if (has && !load_edge<L>(adj, up, prefix, p, e, L, J)) {
            if (gl == 0) set_status(st, GCSL_ERR_UNSUPPORTED);
            J.T = 0;
        }
        if (has && gl == 0) n_full += J.T;
        double r2min = inf, zmin_exact = inf;
        bool removed = false, done = !has || J.T == 0;
        long long base = 0;
        while (__any_sync(GCSL_FULL_MASK, !done)) {
            const long long m = base + gl;
            const bool valid = !done && m < J.T;
            TestOut o;
            o.rho2 = inf;
            o.zexact = inf;
            o.remove = false;
            int S[L];
            if (valid) {
                long long rank;
                int dir;
                key_of(J, m, rank, dir);
                const int vi = dir ? J.hi : J.lo, vj = dir ? J.lo : J.hi;
                const int K = (dir ? J.deg_hi : J.deg_lo) - 1;
                int pos[L];
                unrank_positions<L>(K, rank, pos);
                const int *nbrs = adj + (size_t)vi * p + 1;
#pragma unroll
                for (int c = 0; c < L; ++c) S[c] = resolve_position(nbrs, vj, pos[c]);
                o = gauss_test_reg<L>(C, p, vi, vj, S, tau, t2);
            }
            const unsigned bal = (__ballot_sync(GCSL_FULL_MASK, o.remove) >> gshift) & gbits;
            const int first = bal ? (__ffs(bal) - 1) : G;
            const bool fold = valid && gl <= first;
            const double r2 = group_min<G>(fold ? o.rho2 : inf);
            const double ze = group_min<G>((fold && !isnan(o.zexact)) ? o.zexact : inf);
            if (!done) {
                r2min = fmin(r2min, r2);
                zmin_exact = fmin(zmin_exact, ze);
                const long long left = J.T - base;
                if (gl == 0) n_tests += (unsigned long long)(bal ? first + 1 : (left < G ? left : G));
                if (bal) {
                    if (gl == first) write_removal(J, L, S, p, max_level, G_, sep_dense, rec_pool, rec_cap, st);
                    removed = true;
                    done = true;
                } else {
                    base += G;
                    if (base >= J.T) done = true;
                }
            }
        }
        if (has && gl == 0 && J.T > 0) {
            // z* candidates: exact Z into zmin, the monotone branch's min rho^2 into r2min
            // (converted to Z once per pair by pmax_kernel)
            const size_t ix = (size_t)J.lo * p + J.hi;
            if (zmin_exact < inf) zmin[ix] = fmin(zmin[ix], zmin_exact);
            if (r2min < inf) r2min_pair[ix] = fmin(r2min_pair[ix], r2min);
            n_removed += removed;
        }
    }
    if (gl == 0) {
        if (n_tests) atomicAdd(&st->tests[L], n_tests);
        if (n_full) atomicAdd(&st->tests_full[L], n_full);
        if (n_removed) atomicAdd(&st->removed[L], n_removed);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) st->edges[L] = (unsigned long long)n_edges;
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
// ------------------------------------------------------------------ p-values
// 2 sf(z) = erfc(z / sqrt 2) from Taylor expansions of erfc about the centres
// c_m = (m + 1/2) / 8, m < 32, which cover [0, 4):  erfc(c + t) = sum_k a_k t^k with
// a_0 = erfc(c) and a_{k+1} = b_k / (k + 1), where b_k are the Taylor coefficients of
// erfc'(c + t) = erfc'(c) exp(-2 c t - t^2):  b_0 = -(2 / sqrt pi) exp(-c^2) and
// (k + 1) b_{k+1} = -2 c b_k - 2 b_{k-1} (from E' = -(2c + 2t) E for E = exp(-2ct - t^2)).
// With |t| <= 1/16, 13 terms leave a truncation error below 1e-18 of the value on the
// whole range; arguments from 4 on (and NaN) go to the library erfc.  One Horner chain
// replaces erf/erfc, which matters on a GPU whose FP64 pipe is 1/64 of its FP32 pipe.
constexpr int SF_CENTRES = 32, SF_TERMS = 13;

// Built by each block into shared memory (one thread per centre).
__device__ void sf_table_build(double (*a)[SF_TERMS]) {
    for (int m = threadIdx.x; m < SF_CENTRES; m += blockDim.x) {
        const double c = (m + 0.5) * 0.125;
        double bprev = 0.0, b = -1.12837916709551257390 * exp(-c * c);  // 2 / sqrt(pi)
        a[m][0] = erfc(c);
        for (int k = 0; k + 1 < SF_TERMS; ++k) {
            a[m][k + 1] = b / (k + 1);
            const double bn = (-2.0 * c * b - 2.0 * bprev) / (k + 1);
            bprev = b;
            b = bn;
        }
    }
}

__device__ __forceinline__ double two_sf_tab(double z, const double (*a)[SF_TERMS]) {
    const double x = fabs(z) * 0.70710678118654752440;
    if (!(x < 4.0)) return erfc(x);
    const int m = (int)(x * 8.0);
    const double t = x - (m + 0.5) * 0.125;
    double v = a[m][SF_TERMS - 1];
#pragma unroll
    for (int k = SF_TERMS - 2; k >= 0; --k) v = fma(v, t, a[m][k]);
    return v;
}

// Z(r) = |atanh r|: for r^2 < 1/100 the series |r| sum_{k<10} r^{2k} / (2k + 1)
// (truncation below 1e-20 of the value), else the reference's form
// |0.5 ln|(1 + r) / (1 - r)|| (gaussian_ci.cu:36-37).
__device__ __forceinline__ double fisher_z(double r) {
    const double u = r * r;
    if (u < 0.01) {
        double s = 1.0 / 19.0;
        s = fma(s, u, 1.0 / 17.0);
        s = fma(s, u, 1.0 / 15.0);
        s = fma(s, u, 1.0 / 13.0);
        s = fma(s, u, 1.0 / 11.0);
        s = fma(s, u, 1.0 / 9.0);
        s = fma(s, u, 1.0 / 7.0);
        s = fma(s, u, 1.0 / 5.0);
        s = fma(s, u, 1.0 / 3.0);
        s = fma(s, u, 1.0);
        return fabs(r) * s;
    }
    return fabs(0.5 * log(fabs((1.0 + r) / (1.0 - r))));
}

// Pairs kept at level 0 (the list the level-0 kernel appended): z* = min(zmin, Z of the
// smallest rho^2 any later level stored), pmax = 2 sf(sqrt(n - 3) z*)
// (helpers.py:62-82 with the FP64 z*).
__global__ void pmax_kept_kernel(const int *__restrict__ kept, const DevState *__restrict__ st,
                                 const double *__restrict__ zmin, const double *__restrict__ r2min, double sqrt_nm3,
                                 double *__restrict__ pmax) {
    __shared__ double tab[SF_CENTRES][SF_TERMS];
    sf_table_build(tab);
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
                                   double sqrt_nm3, double *__restrict__ pmax) {
    __shared__ double tab[SF_CENTRES][SF_TERMS];
    sf_table_build(tab);
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

cudaError_t launch_level0(const double *C, int p, double tau0, uint16_t *G, double *zmin, int *kept, DevState *st,
                          cudaStream_t s) {
    const int nb = (p + 31) / 32;
    const double t0 = tanh(tau0);
    gauss_level0_kernel<<<nb * (nb + 1) / 2, 256, 0, s>>>(C, p, tau0, t0 * t0, G, zmin, kept, st);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_compact(const uint16_t *G, int p, int *adj, int *up, DevState *st, int level, cudaStream_t s) {
    const int threads = 256, wpb = threads / 32;
    int blocks = (p + wpb - 1) / wpb;
    compact_kernel<<<blocks, threads, 0, s>>>(G, p, adj, up, st, level);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_recompact(const uint16_t *G, int p, int *adj, int *up, DevState *st, int level, cudaStream_t s) {
    const int threads = 256, wpb = threads / 32;
    recompact_kernel<<<(p + wpb - 1) / wpb, threads, 0, s>>>(G, p, adj, up, st, level);
    note_launch(1);
    return cudaGetLastError();
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

cudaError_t launch_gauss_level(int L, const double *C, int p, const int *adj, const int *up, const long long *prefix,
                               double tau, bool tau_valid, uint16_t *G, double *zmin, double *r2min, int *sep_dense,
                               int max_level, int *rec_pool, long long rec_cap, DevState *st, int num_sms,
                               cudaStream_t s) {
    // register-heavy upper levels run 128-thread blocks so a full wave of warps is resident
    const int threads = L >= 4 ? 128 : 256;
    const int blocks = num_sms * (L >= 4 ? 12 : 8);
    const double th = tanh(tau);
    const double t2 = th * th;  // Z < tau  <=>  rho^2 < tanh(tau)^2 for |rho| < 1
#define GCSL_LVL(K)                                                                                               \
    case K:                                                                                                       \
        gauss_level_reg_kernel<K, 32><<<blocks, threads, 0, s>>>(C, p, adj, up, prefix, tau, t2, tau_valid, G, zmin, \
                                                                 r2min, sep_dense, max_level, rec_pool, rec_cap, st);\
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
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(gauss_level_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        gauss_level_smem_kernel<<<num_sms * 4, t, smem, s>>>(C, p, adj, up, prefix, L, tau, tau_valid, G, zmin,
                                                               sep_dense, max_level, rec_pool, rec_cap, st);
    }
    }
#undef GCSL_LVL
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_unrank(int K, int L, long long count, int *out, cudaStream_t s) {
    const long long blocks = (count + 127) / 128;
    unrank_kernel<<<(int)(blocks > 0 ? (blocks < 65535 ? blocks : 65535) : 1), 128, 0, s>>>(K, L, count, out);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_pmax_level0(const double *C, const double *zmin, int p, long long n_obs, double *pmax,
                               int num_sms, cudaStream_t s) {
    const long long total = (long long)p * p;
    const long long want = (total + 255) / 256;
    const int blocks = (int)(want < (long long)num_sms * 4 ? want : (long long)num_sms * 4);
    pmax_level0_kernel<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(C, zmin, p, sqrt((double)(n_obs - 3)), pmax);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_pmax(const int *kept, const DevState *st, const double *zmin, const double *r2min, int p,
                        long long n_obs, double *pmax, int num_sms, cudaStream_t s) {
    const long long pairs = (long long)p * (p - 1) / 2;
    const long long want = (pairs + 255) / 256;
    const int blocks = (int)(want < (long long)num_sms * 2 ? want : (long long)num_sms * 2);
    pmax_kept_kernel<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(kept, st, zmin, r2min, sqrt((double)(n_obs - 3)), pmax);
    note_launch(1);
    return cudaGetLastError();
}

}  // namespace host
}  // namespace gcsl
