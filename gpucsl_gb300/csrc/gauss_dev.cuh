// Device helpers of the Gaussian CI tests shared by the single-instance level loop
// (gauss.cu) and the batched one (gauss_batch.cu): the test arithmetic, the edge /
// key bookkeeping of a level, the sepset write-back and the p-value functions.
#pragma once

#include "common.cuh"

namespace gcsl {

// ----------------------------------------------------------------- level 0
// 32 x 32 tiles of the upper triangle (tile row bi <= tile column bj): for i < j,
// Z = |0.5 log|(1+r)/(1-r)||, r = C[i*p + j]; remove iff Z < tau0, decided as
// r^2 < tanh(tau0)^2 away from the knife edge.  Kept pairs store r^2 in r2min (zmin =
// +inf; the exact Z only where the reference formula decided) and append i * p + j to
// `kept`; removed pairs store the marker zmin = -1: their z* is final and their pmax is
// computed from C by pmax_level0_kernel, concurrently with the later levels.
// The mirrored skeleton entries are written through a shared-memory transpose so both
// triangles are stored row-contiguously; zero diagonal.
// One block of 256 threads per tile; `tile` enumerates the upper-triangle tiles row by row.
__device__ __forceinline__ void level0_tile(const double *__restrict__ C, int p, double tau0, L0Bounds B,
                                            uint16_t *__restrict__ G, double *__restrict__ zmin,
                                            double *__restrict__ r2min, int *__restrict__ kept, DevState *st,
                                            int tile, float *__restrict__ C32 = nullptr) {
    __shared__ uint16_t tg[32][33];
    __shared__ float tc[32][33];
    const int nb = (p + 31) / 32;
    int rem = tile, bi = 0;
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
        if (C32 != nullptr && i == j && i < p) C32[(size_t)i * p + i] = f64_to_f32_rn(__ldg(C + (size_t)i * p + i));
        if (i < p && j < p && i < j) {
            const double c = __ldg(C + (size_t)i * p + j);
            if (C32 != nullptr) {  // the FP32 copy of C for the FP32-first levels, both triangles
                const float c32 = f64_to_f32_rn(c);
                C32[(size_t)i * p + j] = c32;
                tc[r][tx] = c32;
            }
            // Z0 = atanh-like in |r| on [0, 1): Z0 < tau0 <=> r^2 < tanh(tau0)^2, decided
            // on the bits of |r| outside the knife edge; the knife edge, |r| >= 1 and NaN
            // take the reference formula
            const unsigned long long a = (unsigned long long)__double_as_longlong(c) & 0x7fffffffffffffffull;
            bool rem0;
            double z = -1.0;  // marker: z* of a level-0 removal is finished on the side stream
            if (a < B.lo) {
                rem0 = true;
            } else if (a >= B.hi && a < B.one) {
                // kept: r^2 joins the pair's rho^2 minimum; the logarithm is taken once,
                // in the pmax kernel, instead of in this (divergent) warp
                rem0 = false;
                z = __longlong_as_double(0x7ff0000000000000ll);
                r2min[(size_t)i * p + j] = c * c;
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
            if (i < p && j < p) {
                G[(size_t)j * p + i] = tg[tx][r];
                if (C32 != nullptr) C32[(size_t)j * p + i] = tc[tx][r];
            }
        }
    } else {
        for (int r = ty; r < 32; r += 8) {
            const int j = bj * 32 + r, i = bi * 32 + tx;
            if (i < p && j < p && j > i) {
                G[(size_t)j * p + i] = tg[tx][r];
                if (C32 != nullptr) C32[(size_t)j * p + i] = tc[tx][r];
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) removed += __shfl_xor_sync(GCSL_FULL_MASK, removed, o);
    if ((threadIdx.x & 31) == 0 && removed) atomicAdd(&st->removed[0], removed);
}

// ------------------------------------------------------------- compaction
// One warp compacts row r: adj[r*p] = degree, adj[r*p + 1 ..] = ascending neighbour ids
// (entries past the degree keep stale values, as in the reference); also writes
// up[r] = #neighbours > r.  Returns the degree.
// The row's edges to larger ids, (r, j) for its last `ups` neighbours, appended to the
// level's edge list at slots reserved with one atomic per row (the list order does not
// matter: a test warp owns its edge).
__device__ __forceinline__ void emit_row_edges(const int *row, int cnt, int ups, int r, int lane,
                                               int2 *__restrict__ elist, unsigned long long *ecount) {
    if (elist == nullptr || ups == 0) return;
    __syncwarp();  // the row's entries are written
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(ecount, (unsigned long long)ups);
    base = __shfl_sync(GCSL_FULL_MASK, base, 0);
    for (int k = lane; k < ups; k += 32) elist[base + k] = make_int2(r, row[1 + cnt - ups + k]);
}

__device__ __forceinline__ int compact_row(const uint16_t *__restrict__ G, int p, int *__restrict__ adj,
                                           int *__restrict__ up, int r, int lane, int2 *elist = nullptr,
                                           unsigned long long *ecount = nullptr) {
    {
        const uint16_t *Gr = G + (size_t)r * p;
        int *row = adj + (size_t)r * p;
        int cnt = 0, ups = 0;
        // 256 columns per pass, 8 consecutive ones per lane (independent loads), positions
        // from a warp prefix sum of the lanes' counts
        for (int c0 = 0; c0 < p; c0 += 256) {
            const int cb = c0 + lane * 8;
            unsigned m = 0;
#pragma unroll
            for (int t = 0; t < 8; ++t) {
                const int c = cb + t;
                if (c < p && c != r && Gr[c] != 0) m |= 1u << t;
            }
            const int nb = __popc(m);
            int x = nb;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(GCSL_FULL_MASK, x, o);
                if (lane >= o) x += y;
            }
            int pos = cnt + x - nb;
#pragma unroll
            for (int t = 0; t < 8; ++t)
                if ((m >> t) & 1u) row[1 + pos++] = cb + t;
            cnt += __shfl_sync(GCSL_FULL_MASK, x, 31);
            // neighbours above r: the bits of columns > r
            const int above = r - cb;  // bits t > above count
            const unsigned mu = above >= 7 ? 0u : (above < 0 ? m : (m & ~((2u << above) - 1u)));
            int u = __popc(mu);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) u += __shfl_xor_sync(GCSL_FULL_MASK, u, o);
            ups += u;
        }
        if (lane == 0) {
            row[0] = cnt;
            if (up != nullptr) up[r] = ups;
        }
        emit_row_edges(row, cnt, ups, r, lane, elist, ecount);
        return cnt;
    }
}

// Levels >= 2: one warp refilters row r's previous neighbour list against G (rows only
// shrink, so this touches deg entries instead of p), writes up[r] and, when given, the
// row's edges.  Returns the degree.
__device__ __forceinline__ int recompact_row(const uint16_t *__restrict__ G, int p, int *__restrict__ adj,
                                             int *__restrict__ up, int r, int lane, int2 *elist = nullptr,
                                             unsigned long long *ecount = nullptr, DevState *st = nullptr) {
    {
        int *row = adj + (size_t)r * p;
        int deg = row[0];
        if (!dcheck(st, deg >= 0 && deg <= p - 1, GCSL_DCHECK_DEGREE)) deg = deg < 0 ? 0 : p - 1;
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
        emit_row_edges(row, cnt, ups, r, lane, elist, ecount);
        return cnt;
    }
}

// Exclusive scan by one whole block of a per-row count (int or weighted long long) into
// prefix[0..p]; prefix[p] is the total.
template <typename T>
__device__ __forceinline__ void block_scan_rows(const T *__restrict__ cnt, int p, long long *__restrict__ prefix) {
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
    bool exact;    // rho2 / zexact hold the FP64 result; else r32 +- e32 encloses FP64 rho^2
    float r32, e32;
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
        o.exact = true;
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
    o.exact = true;
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
    J.R0 = (K0 >= L) ? binom_fast<KMAX>(K0, L) : 0;
    J.R1 = (K1 >= L) ? binom_fast<KMAX>(K1, L) : 0;
    J.T = J.R0 + J.R1;
    J.Rmin = J.R0 < J.R1 ? J.R0 : J.R1;
    J.longer = J.R0 > J.R1 ? 0 : 1;
    return J.R0 < GCSL_RANK_LIMIT && J.R1 < GCSL_RANK_LIMIT;
}

// Edge e of the level from the explicit edge list (lo < hi) written by the edge scan.
template <int KMAX>
__device__ __forceinline__ bool load_edge_list(const int *__restrict__ adj, const int2 *__restrict__ elist, int p,
                                               long long e, int L, EdgeJob &J, DevState *st = nullptr) {
    const int2 ed = elist[e];
    if (!dcheck(st, ed.x >= 0 && ed.x < ed.y && ed.y < p, GCSL_DCHECK_EDGE)) {  // no tests for this edge
        J.lo = 0;
        J.hi = p > 1 ? 1 : 0;
        J.deg_lo = J.deg_hi = 0;
        J.R0 = J.R1 = J.T = J.Rmin = 0;
        J.longer = 0;
        return true;
    }
    J.lo = ed.x;
    J.hi = ed.y;
    J.deg_lo = adj[(size_t)ed.x * p];
    J.deg_hi = adj[(size_t)ed.y * p];
    const int K0 = J.deg_lo - 1, K1 = J.deg_hi - 1;
    J.R0 = (K0 >= L) ? binom_fast<KMAX>(K0, L) : 0;
    J.R1 = (K1 >= L) ? binom_fast<KMAX>(K1, L) : 0;
    J.T = J.R0 + J.R1;
    J.Rmin = J.R0 < J.R1 ? J.R0 : J.R1;
    J.longer = J.R0 > J.R1 ? 0 : 1;
    return J.R0 < GCSL_RANK_LIMIT && J.R1 < GCSL_RANK_LIMIT;
}

// The job of edge (lo, hi) from degrees already known (the unit kernel takes them from the
// chunk record instead of reloading the adjacency rows' counts).
template <int KMAX>
__device__ __forceinline__ void edge_job_from(int lo, int hi, int deg_lo, int deg_hi, int L, EdgeJob &J) {
    J.lo = lo;
    J.hi = hi;
    J.deg_lo = deg_lo;
    J.deg_hi = deg_hi;
    const int K0 = deg_lo - 1, K1 = deg_hi - 1;
    J.R0 = (K0 >= L) ? binom_fast<KMAX>(K0, L) : 0;
    J.R1 = (K1 >= L) ? binom_fast<KMAX>(K1, L) : 0;
    J.T = J.R0 + J.R1;
    J.Rmin = J.R0 < J.R1 ? J.R0 : J.R1;
    J.longer = J.R0 > J.R1 ? 0 : 1;
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

// Minima of the statistics folded into z* (rho^2 and Z: zero or positive, or +inf, never
// NaN here).  For such values the order of the bit patterns as signed 64-bit integers is
// the numeric order, so the comparisons run on the integer pipe: GB300's FP64 pipe runs
// at 1/64 of its FP32 rate, and FP64 minima of every test made it the bound of the
// batched level kernels.
__device__ __forceinline__ double min_nonneg(double a, double b) {
    const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    return __longlong_as_double(x < y ? x : y);
}

// The double of a float that is zero or positive (or +inf), built from its bits on the
// integer pipe (the conversion instruction runs on the FP64 pipe).
__device__ __forceinline__ double f32_nonneg_to_f64(float x) {
    uint32_t u = __float_as_uint(x) & 0x7fffffffu;
    uint32_t e = u >> 23, m = u & 0x7fffffu;
    unsigned long long bits;
    if (e == 255u) {
        bits = 0x7ff0000000000000ull | ((unsigned long long)m << 29);
    } else if (e == 0u) {
        if (m == 0u) {
            bits = 0ull;
        } else {  // subnormal: normalise the significand
            const int lz = __clz((int)m) - 8;  // shifts bit 23 into place
            m = (m << lz) & 0x7fffffu;
            bits = ((unsigned long long)(897 - lz) << 52) | ((unsigned long long)m << 29);
        }
    } else {
        bits = ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
    }
    return __longlong_as_double((long long)bits);
}

// A double that is zero or positive rounded up to FP32 from its bits (negative values
// give -1): the bound eps of a split-precision C, widened rather than rounded.
__device__ __forceinline__ float f64_nonneg_to_f32_ru(double v) {
    const long long b = __double_as_longlong(v);
    if (b < 0) return -1.0f;
    if (b == 0) return 0.0f;
    const int e = (int)(b >> 52);  // biased exponent
    if (e < 1023 - 126) return __int_as_float(0x00800000);  // below FP32's normal range: 2^-126
    if (e > 1023 + 127) return __int_as_float(0x7f800000);
    unsigned fb = ((unsigned)(e - 1023 + 127) << 23) | (unsigned)((b >> 29) & 0x7fffff);
    if (b & ((1ll << 29) - 1)) ++fb;  // round up (a carry moves into the exponent)
    return __uint_as_float(fb);
}

__device__ __forceinline__ bool nan_bits(double v) {
    return (__double_as_longlong(v) & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
}

// Min over the G-lane group (aligned groups of G lanes inside the warp) of values as
// min_nonneg takes them.
template <int G>
__device__ __forceinline__ double group_min(double v) {
    long long b = __double_as_longlong(v);
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        const long long c = __shfl_xor_sync(GCSL_FULL_MASK, b, o);
        b = c < b ? c : b;
    }
    return __longlong_as_double(b);
}

// The FP64 test out of line: the mixed kernels call it rarely (guard band, unusable
// bounds, full queue), and keeping it out of their main path keeps its registers out of
// their register budget.
template <int L>
__device__ __noinline__ TestOut gauss_test_reg_call(const double *__restrict__ C, int p, int vi, int vj,
                                                    const int *S, double tau, double t2) {
    return gauss_test_reg<L>(C, p, vi, vj, S, tau, t2);
}

// ------------------------------------------------------- FP32 test with a bound
// The same elimination in FP32 on the FP32 copy of C, carrying for every entry a
// first-order bound of its distance to the exact value for the FP64 matrix C:
// inputs |fl32(c) - c| <= u|c|; a reciprocal, a product and an fma each add u times
// their result plus the propagated bounds of their operands (u = 2^-24, round to
// nearest).  rho^2 = H01^2 / (H00 H11) gets the first-order bound of the quotient with
// the denominators at their lower ends, doubled for the neglected higher-order terms;
// FP64 rounding of the reference path (~1e-15 relative) is far inside that margin.
// Returns false (bound unusable) when a pivot or H00 / H11 is not clearly positive,
// when a relative bound exceeds 1/4, or when rho^2 + bound reaches 0.98.
constexpr float F32_U = 5.9604645e-08f;  // 2^-24

__device__ __forceinline__ bool f32_rho2_bound(float h00, float e00, float h01, float e01, float h11, float e11,
                                               float &rho2, float &err) {
    const float lo00 = h00 - e00, lo11 = h11 - e11;
    rho2 = (h01 * h01) / (h00 * h11);
    const float ah = fabsf(h01);
    err = 2.f * ((2.f * ah * e01 + e01 * e01) / (lo00 * lo11) + rho2 * (e00 / lo00 + e11 / lo11) +
                 4.f * F32_U * rho2);
    return e00 < 0.25f * h00 && e11 < 0.25f * h11 && rho2 + err < 0.98f;  // NaN fails
}

// Entries of the FP32 correlation copy by variable id (row-major, row stride p).
struct GlobalC32 {
    const float *__restrict__ C32;
    int p;
    __device__ __forceinline__ float operator()(int a, int b) const { return __ldg(C32 + (size_t)a * p + b); }
};

// The FP32 elimination with its running error bound on the entries at(.,.) of the
// (xi, xj, X) submatrix; the diagonal entries of xi and xj are 1 (as in C).
template <int L, class Acc>
__device__ __forceinline__ bool gauss_test_f32_at(const Acc &at, int xi, int xj, const int *X, float &rho2,
                                                  float &err) {
    const float u = F32_U;
    if constexpr (L == 1) {
        const float m = at(X[0], X[0]);
        const float a = at(xi, X[0]);
        const float b = at(xj, X[0]);
        const float r = at(xi, xj);
        const float em = u * fabsf(m), ea = u * fabsf(a), eb = u * fabsf(b), er = u * fabsf(r);
        const float d00 = fmaf(-a, a, m), d11 = fmaf(-b, b, m);
        const float e00 = em + 2.f * fabsf(a) * ea + u * fabsf(d00);
        const float e11 = em + 2.f * fabsf(b) * eb + u * fabsf(d11);
        const float ab = a * b;
        const float eab = fabsf(a) * eb + fabsf(b) * ea + u * fabsf(ab);
        const float n01 = fmaf(r, m, -ab);
        const float e01 = fabsf(m) * er + fabsf(r) * em + eab + u * fabsf(n01);
        return f32_rho2_bound(d00, e00, n01, e01, d11, e11, rho2, err);
    }
    constexpr int D = L + 2;
    float A[D * (D + 1) / 2], E[D * (D + 1) / 2];
#pragma unroll
    for (int r = 0; r < L; ++r) {
#pragma unroll
        for (int c = 0; c <= r; ++c) A[r * (r + 1) / 2 + c] = at(X[r], X[c]);
        A[L * (L + 1) / 2 + r] = at(xi, X[r]);
        A[(L + 1) * (L + 2) / 2 + r] = at(xj, X[r]);
    }
    A[L * (L + 1) / 2 + L] = 1.0f;
    A[(L + 1) * (L + 2) / 2 + L] = at(xi, xj);
    A[(L + 1) * (L + 2) / 2 + L + 1] = 1.0f;
#pragma unroll
    for (int k = 0; k < D * (D + 1) / 2; ++k) E[k] = u * fabsf(A[k]);
    bool ok = true;
#pragma unroll
    for (int j = 0; j < L; ++j) {
        const float piv = A[j * (j + 1) / 2 + j], ep = E[j * (j + 1) / 2 + j];
        ok = ok && ep < 0.25f * piv;
        const float inv = 1.0f / piv;
        const float einv = ep * inv * inv * 1.5f + u * fabsf(inv);  // 1/(p - e) <= (1 + 1.5 e/p)/p for e < p/4
#pragma unroll
        for (int i = j + 1; i < D; ++i) {
            const float aij = A[i * (i + 1) / 2 + j];
            const float t = aij * inv;
            const float et = fabsf(aij) * einv + fabsf(inv) * E[i * (i + 1) / 2 + j] + u * fabsf(t);
#pragma unroll
            for (int k = j + 1; k <= i; ++k) {
                const float akj = A[k * (k + 1) / 2 + j];
                const float v = fmaf(-t, akj, A[i * (i + 1) / 2 + k]);
                E[i * (i + 1) / 2 + k] += fabsf(t) * E[k * (k + 1) / 2 + j] + fabsf(akj) * et + u * fabsf(v);
                A[i * (i + 1) / 2 + k] = v;
            }
        }
    }
    const int i00 = L * (L + 1) / 2 + L, i01 = (L + 1) * (L + 2) / 2 + L, i11 = (L + 1) * (L + 2) / 2 + L + 1;
    return f32_rho2_bound(A[i00], E[i00], A[i01], E[i01], A[i11], E[i11], rho2, err) && ok;
}

template <int L>
__device__ __forceinline__ bool gauss_test_f32b(const float *__restrict__ C32, int p, int vi, int vj, const int *S,
                                                float &rho2, float &err) {
    return gauss_test_f32_at<L>(GlobalC32{C32, p}, vi, vj, S, rho2, err);
}

// FP32 first: the decision is taken there when the bound puts rho^2 clearly on one side
// of the FP64 path's knife edge [t2 (1 - 1e-12), t2 (1 + 1e-12)] (t2lo / t2hi are FP32
// bounds of it, rounded outward); otherwise, or when the bound is unusable, the FP64
// test runs here and its result is exact.
template <int L>
struct MixedTest {
    static constexpr bool kMixed = true;
    const double *__restrict__ C;
    const float *__restrict__ C32;
    int p;
    double tau, t2;
    float t2lo, t2hi;
    __device__ __forceinline__ TestOut operator()(int vi, int vj, const int *S) const {
        float r, e;
        if (gauss_test_f32b<L>(C32, p, vi, vj, S, r, e) && (__fadd_ru(r, e) < t2lo || __fsub_rd(r, e) > t2hi)) {
            TestOut o;
            o.rho2 = __longlong_as_double(0x7ff0000000000000ll);
            o.zexact = o.rho2;
            o.remove = __fadd_ru(r, e) < t2lo;
            o.exact = false;
            o.r32 = r;
            o.e32 = e;
            return o;
        }
        return gauss_test_reg_call<L>(C, p, vi, vj, S, tau, t2);
    }
};

// Deferred FP64 evaluations of level L: entries [pair index lo * p + hi, vi, vj, chunk tag,
// merged key index, S...] appended by the level kernels, evaluated densely by the
// candidate kernel (tag -1: the key always counts).
constexpr int CAND_HEADER = 5;
struct CandQueue {
    int *buf;
    long long cap;                 // ints
    unsigned long long *count;     // ints used (may exceed cap: those entries were evaluated inline)
};

__device__ __forceinline__ void atomic_min_nonneg_f64(double *addr, double v) {
    atomicMin(reinterpret_cast<unsigned long long *>(addr), (unsigned long long)__double_as_longlong(v));
}

template <int G>
__device__ __forceinline__ float group_min_f(float v) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(GCSL_FULL_MASK, v, o));
    return v;
}

// The FP64 test of the plain path as a functor for walk_edge.
template <int L>
struct F64Test {
    static constexpr bool kMixed = false;
    const double *__restrict__ C;
    int p;
    double tau, t2;
    __device__ __forceinline__ TestOut operator()(int vi, int vj, const int *S) const {
        return gauss_test_reg<L>(C, p, vi, vj, S, tau, t2);
    }
};

// One G-lane group walks edge J's merged key sequence G keys at a time: each lane tests
// one key, the lowest removing lane is the canonical remover (its set is written back),
// and the keys up to it fold into the group's minima of rho^2 (r2min) and of the exactly
// evaluated Z (zmin_exact).  Every lane of the warp must call this (warp-wide votes); a
// lane with has == false takes part without testing.
//
// With a mixed (FP32-first) test, keys decided in FP32 carry an interval r32 +- e32
// around their FP64 rho^2: every such key of the fold whose interval reaches below both
// the smallest upper end in its step and the pair's minimum from earlier levels could
// hold the minimum and is queued for the FP64 candidate kernel (or evaluated here when
// the queue is full); exact keys fold directly.
// A slice [m0, m1) of an edge's merged key sequence.  With defer set, the slice is one
// unit of a chunked edge: its first removing key is reported in `first` (m1 when none)
// instead of being written back, and its queued z* candidates carry (tag, key) so the
// candidate kernel can drop the ones behind the edge's canonical remover.
struct WalkRange {
    long long m0, m1;
    bool defer;
    int tag;
    long long first;
};

template <int L, int G, class Test>
__device__ __forceinline__ void walk_edge(const EdgeJob &J, bool has, const int *__restrict__ adj, int p, int gl,
                                          unsigned gshift, unsigned gbits, const Test &test, uint16_t *G_,
                                          int *sep_dense, int max_level, int *rec_pool, long long rec_cap,
                                          DevState *st, double &r2min, double &zmin_exact, bool &removed,
                                          unsigned long long &n_tests, const CandQueue *q = nullptr,
                                          const BinomRows *sb = nullptr, double r2_floor = 0.0,
                                          WalkRange *rg = nullptr) {
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    // r2_floor rounded up to FP32: a key whose FP32 interval starts above it cannot lower
    // z* (the rounding only admits a few more candidates), compared in FP32 per step
    const float floor32 = __double2float_ru(r2_floor);
    long long base = rg ? rg->m0 : 0;
    const long long mend = rg ? rg->m1 : J.T;
    bool done = !has || base >= mend;
    while (__any_sync(GCSL_FULL_MASK, !done)) {
        const long long m = base + gl;
        const bool valid = !done && m < mend;
        TestOut o;
        o.rho2 = inf;
        o.zexact = inf;
        o.remove = false;
        o.exact = true;
        int S[L];
        int vi = 0, vj = 0;
        if (valid) {
            long long rank;
            int dir;
            key_of(J, m, rank, dir);
            vi = dir ? J.hi : J.lo;
            vj = dir ? J.lo : J.hi;
            const int K = (dir ? J.deg_hi : J.deg_lo) - 1;
            int pos[L];
            unrank_positions<L>(K, rank, pos, sb);
            const int *nbrs = adj + (size_t)vi * p + 1;
#pragma unroll
            for (int c = 0; c < L; ++c) {
                const int q = pos[c];
                S[c] = resolve_position(nbrs, vj, dcheck(st, q >= 1 && q <= K, GCSL_DCHECK_POSITION) ? q : 1);
            }
#if GCSL_DEBUG_CHECKS
#pragma unroll
            for (int c = 0; c < L; ++c) {
                const bool ok = S[c] >= 0 && S[c] < p && S[c] != vi && S[c] != vj && (c == 0 || S[c] > S[c - 1]);
                if (!dcheck(st, ok, GCSL_DCHECK_SET)) S[c] = S[c] < 0 || S[c] >= p ? 0 : S[c];
            }
#endif
            o = test(vi, vj, S);
        }
        const unsigned bal = (__ballot_sync(GCSL_FULL_MASK, o.remove) >> gshift) & gbits;
        const int first = bal ? (__ffs(bal) - 1) : G;
        const bool fold = valid && gl <= first;
        if constexpr (Test::kMixed) {
            // interval ends rounded outward; a key whose interval starts above the pair's
            // exact minimum so far (r2_floor, from earlier levels) cannot lower z*
            const float lo32 = __fsub_rd(o.r32, o.e32);
            const float hi = group_min_f<G>((fold && !o.exact) ? __fadd_ru(o.r32, o.e32) : __int_as_float(0x7f800000));
            bool cand = fold && !o.exact && lo32 <= hi && lo32 <= floor32;
            const unsigned cm = __ballot_sync(GCSL_FULL_MASK, cand);
            if (cm) {
                constexpr int W = CAND_HEADER + L;
                unsigned long long b0 = 0;
                const int leader = __ffs(cm) - 1;
                if ((threadIdx.x & 31) == leader) b0 = atomicAdd(q->count, (unsigned long long)(W * __popc(cm)));
                b0 = __shfl_sync(GCSL_FULL_MASK, b0, leader);
                if (cand) {
                    const unsigned long long at = b0 + (unsigned long long)W * __popc(cm & ((1u << (threadIdx.x & 31)) - 1u));
                    if ((long long)(at + W) <= q->cap) {
                        int *e = q->buf + at;
                        e[0] = J.lo * p + J.hi;
                        e[1] = vi;
                        e[2] = vj;
                        e[3] = (rg && rg->defer) ? rg->tag : -1;
                        e[4] = (int)m;
#pragma unroll
                        for (int c = 0; c < L; ++c) e[CAND_HEADER + c] = S[c];
                        cand = false;
                    }
                }
                if (__any_sync(GCSL_FULL_MASK, cand)) {  // queue full: evaluate here
                    if (cand) {
                        o = gauss_test_reg_call<L>(test.C, p, vi, vj, S, test.tau, test.t2);
                        o.remove = false;  // decided already; only the statistic is folded
                    }
                }
            }
            const bool ex = fold && (o.exact || cand);
            if (__any_sync(GCSL_FULL_MASK, ex)) {
                const double r2 = group_min<G>(ex ? o.rho2 : inf);
                const double ze = group_min<G>((ex && !nan_bits(o.zexact)) ? o.zexact : inf);
                if (!done) {
                    r2min = min_nonneg(r2min, r2);
                    zmin_exact = min_nonneg(zmin_exact, ze);
                }
            }
        } else {
            const double r2 = group_min<G>(fold ? o.rho2 : inf);
            const double ze = group_min<G>((fold && !nan_bits(o.zexact)) ? o.zexact : inf);
            if (!done) {
                r2min = min_nonneg(r2min, r2);
                zmin_exact = min_nonneg(zmin_exact, ze);
            }
        }
        if (!done) {
            const long long left = mend - base;
            if (gl == 0) n_tests += (unsigned long long)(bal ? first + 1 : (left < G ? left : G));
            if (bal) {
                if (rg && rg->defer) rg->first = base + first;
                else if (gl == first) write_removal(J, L, S, p, max_level, G_, sep_dense, rec_pool, rec_cap, st);
                removed = true;
                done = true;
            } else {
                base += G;
                if (base >= mend) done = true;
            }
        }
    }
}

// Chunked edges.  An edge whose merged key sequence spans more than one step has its first
// step walked by the level kernel; when that step holds no remover, the rest is cut into
// units of one step each (32 keys), which the unit kernel walks in parallel.  The last unit
// of an edge to finish combines them in key order: the canonical remover is the smallest
// removing key over all units, and z* folds every unit that starts at or before it (up to
// its own first remover), exactly the keys the sequential walk would have folded.
// Registers edge J (first step walked, no remover) for the unit kernel; false when the
// buffers are full, and the caller walks the remaining keys itself.  Whole group calls.
template <int G>
__device__ __forceinline__ bool register_chunked(const EdgeJob &J, int gl, const ChunkBufs &ck, DevState *st, int L,
                                                 double r2_0, double ze_0, double floor, long long k0 = G) {
    const long long nu = (J.T - k0 + G - 1) / G;
    long long h = 0, ub = 0;
    if (gl == 0) {
        h = (long long)atomicAdd(&st->heavy[L], 1ull);
        ub = (long long)atomicAdd(&st->units[L], (unsigned long long)nu);
    }
    h = __shfl_sync(GCSL_FULL_MASK, h, 0, G);
    ub = __shfl_sync(GCSL_FULL_MASK, ub, 0, G);
    const bool ok = h < ck.heavy_cap && ub + nu <= ck.unit_cap && J.T < (1ll << 31);
    if (ok) {
        if (gl == 0) {
            HeavyEdge H;
            H.lo = J.lo;
            H.hi = J.hi;
            H.T = J.T;
            H.unit_base = ub;
            H.n_units = (int)nu;
            H.done = 0;
            H.best = J.T;
            H.r2_0 = r2_0;
            H.ze_0 = ze_0;
            H.floor = floor;
            H.k0 = (int)k0;
            H.degs = J.deg_lo | (J.deg_hi << 16);
            ck.heavy[h] = H;
        }
        for (long long k = gl; k < nu; k += G) ck.unit_h[ub + k] = (int)h;
    } else {
        // reserved unit slots inside the buffer stay marked unused
        for (long long k = ub + gl; k < ub + nu && k < ck.unit_cap; k += G) ck.unit_h[k] = -1;
    }
    return ok;
}

// Candidate kernel body: the FP64 test of queued entry e, folded into the pair's minima.
template <int L>
__device__ __forceinline__ void eval_candidate(const double *__restrict__ C, int p, const int *e, double tau,
                                               double t2, double *zmin, double *r2min,
                                               const long long *__restrict__ chunk_first = nullptr) {
    // a key of a chunked edge behind the edge's canonical remover does not count
    if (e[3] >= 0 && chunk_first != nullptr && (long long)e[4] > chunk_first[e[3]]) return;
    int S[L];
#pragma unroll
    for (int c = 0; c < L; ++c) S[c] = e[CAND_HEADER + c];
    const TestOut o = gauss_test_reg<L>(C, p, e[1], e[2], S, tau, t2);
    const size_t ix = (size_t)e[0];
    if (o.rho2 < __longlong_as_double(0x7ff0000000000000ll)) atomic_min_nonneg_f64(r2min + ix, o.rho2);
    if (o.zexact < __longlong_as_double(0x7ff0000000000000ll)) atomic_min_nonneg_f64(zmin + ix, o.zexact);
}

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
__device__ __forceinline__ void sf_table_build(double (*a)[SF_TERMS]) {
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

// The table built once per solve (sf_table_kernel) copied into a block's shared memory.
__device__ __forceinline__ void sf_table_load(double (*a)[SF_TERMS], const double *__restrict__ g) {
    double *dst = &a[0][0];
    for (int k = threadIdx.x; k < SF_CENTRES * SF_TERMS; k += blockDim.x) dst[k] = __ldg(g + k);
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

}  // namespace gcsl
