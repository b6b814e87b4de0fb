// Discrete (chi-squared) PC-stable skeleton kernels for sm_103a (kernel d + write-back e).
//
//   tests          disc_test_kernel      (reference: gpucsl/pc/cuda/discrete_ci.cu:37-246,
//                                         helpers/discrete_helpers.cu:25-186)
//   p-value        pchisq_dev            (reference: helpers/math_helpers.cu:54-175)
//   write-back     disc_finalize_kernel  (reference: helpers/graph_helpers.cu:81-101)
//
// One CTA evaluates one test at a time (grid-stride over the level's flattened test
// list): the l+2 uint8 columns are streamed with 16-byte loads and counted into a
// shared-memory table N[s][a][b] (several copies when the table is small, so that
// lanes of a warp rarely hit the same counter), the copies are merged, each stratum's
// marginals and (a, b)-ordered chi^2 partial sum are formed by one thread, and thread 0
// adds the strata in ascending order and evaluates the p-value.  Counts are exact
// integers; the chi^2 order is fixed, so results do not depend on scheduling.
//
// As in the reference every rank of every direction is tested (discrete_ci.cu:221-244
// has no effective early exit) and pmax folds all of them.  The removing test with the
// smallest key (rank, dir) is the canonical remover; its set becomes the sepset.
#include "common.cuh"

namespace gcsl {

// ---------------------------------------------------------------- p-value
// Ibbetson (CACM Alg. 209) normal tail as coded by Perlman; the polynomial
// coefficients are those of the published algorithm.
__device__ double poz_dev(double z) {
    double x;
    if (z == 0.0) {
        x = 0.0;
    } else {
        double y = 0.5 * fabs(z);
        if (y >= 3.0) {
            x = 1.0;
        } else if (y < 1.0) {
            const double w = y * y;
            double t = 0.000124818987;
            t = __dadd_rn(__dmul_rn(t, w), -0.001075204047);
            t = __dadd_rn(__dmul_rn(t, w), 0.005198775019);
            t = __dadd_rn(__dmul_rn(t, w), -0.019198292004);
            t = __dadd_rn(__dmul_rn(t, w), 0.059054035642);
            t = __dadd_rn(__dmul_rn(t, w), -0.151968751364);
            t = __dadd_rn(__dmul_rn(t, w), 0.319152932694);
            t = __dadd_rn(__dmul_rn(t, w), -0.531923007300);
            t = __dadd_rn(__dmul_rn(t, w), 0.797884560593);
            x = __dmul_rn(__dmul_rn(t, y), 2.0);
        } else {
            y -= 2.0;
            double t = -0.000045255659;
            t = __dadd_rn(__dmul_rn(t, y), 0.000152529290);
            t = __dadd_rn(__dmul_rn(t, y), -0.000019538132);
            t = __dadd_rn(__dmul_rn(t, y), -0.000676904986);
            t = __dadd_rn(__dmul_rn(t, y), 0.001390604284);
            t = __dadd_rn(__dmul_rn(t, y), -0.000794620820);
            t = __dadd_rn(__dmul_rn(t, y), -0.002034254874);
            t = __dadd_rn(__dmul_rn(t, y), 0.006549791214);
            t = __dadd_rn(__dmul_rn(t, y), -0.010557625006);
            t = __dadd_rn(__dmul_rn(t, y), 0.011630447319);
            t = __dadd_rn(__dmul_rn(t, y), -0.009279453341);
            t = __dadd_rn(__dmul_rn(t, y), 0.005353579108);
            t = __dadd_rn(__dmul_rn(t, y), -0.002141268741);
            t = __dadd_rn(__dmul_rn(t, y), 0.000535310849);
            x = __dadd_rn(__dmul_rn(t, y), 0.999936657524);
        }
    }
    return z > 0.0 ? ((x + 1.0) * 0.5) : ((1.0 - x) * 0.5);
}

__device__ __forceinline__ double ex_dev(double x) { return (x < -20.0) ? 0.0 : exp(x); }

// Upper tail of chi^2 (Hill & Pike, CACM Alg. 299, with the 1985 rounding remark, in
// Perlman's formulation): the finite series of the even / odd df cases.
__device__ double pchisq_dev(double x, long long df) {
    if (x <= 0.0 || df < 1) return 1.0;
    const double a = 0.5 * x;
    const bool even = (df & 1) == 0;
    const double y = (df > 1) ? ex_dev(-a) : 0.0;
    double s = even ? y : 2.0 * poz_dev(-sqrt(x));
    if (df <= 2) return s;
    const double half = 0.5 * ((double)df - 1.0);
    double z = even ? 1.0 : 0.5;
    if (a > 20.0) {
        double e = even ? 0.0 : 0.5723649429247000870717135;
        const double c = log(a);
        while (z <= half) {
            e = __dadd_rn(log(z), e);
            s = __dadd_rn(s, ex_dev(__dsub_rn(__dsub_rn(__dmul_rn(c, z), a), e)));
            z += 1.0;
        }
        return s;
    }
    double e = even ? 1.0 : 0.5641895835477562869480795 / sqrt(a);
    double c = 0.0;
    while (z <= half) {
        e = __dmul_rn(e, a / z);
        c = __dadd_rn(c, e);
        z += 1.0;
    }
    return __dadd_rn(__dmul_rn(c, y), s);
}

// pchisq_dev by the 32 lanes of one warp, with the same result bit for bit: the
// quotients a / z (or logarithms log z) of the series are independent and computed one
// per lane, and the recurrence and the sums run in the same order on every lane.  On a
// GPU whose FP64 pipe is 1/64 of its FP32 pipe this takes the divisions off the serial
// path.  All lanes of the warp must call it; every lane returns the value.
__device__ double pchisq_warp(double x, long long df) {
    const int lane = threadIdx.x & 31;
    if (x <= 0.0 || df < 1) return 1.0;
    const double a = 0.5 * x;
    const bool even = (df & 1) == 0;
    const double y = (df > 1) ? ex_dev(-a) : 0.0;
    double s = even ? y : 2.0 * poz_dev(-sqrt(x));
    if (df <= 2) return s;
    const double half = 0.5 * ((double)df - 1.0);
    const double z0 = even ? 1.0 : 0.5;
    const long long K = (long long)floor(half - z0) + 1;  // iterations z = z0, z0 + 1, .. <= half
    if (a > 20.0) {
        double e = even ? 0.0 : 0.5723649429247000870717135;
        const double c = log(a);
        for (long long k0 = 0; k0 < K; k0 += 32) {
            const long long k = k0 + lane;
            const double z = z0 + (double)k;
            const double lz = k < K ? log(z) : 0.0;
            double ek = 0.0;
            const int m = (int)(K - k0 < 32 ? K - k0 : 32);
            for (int q = 0; q < m; ++q) {
                e = __dadd_rn(__shfl_sync(GCSL_FULL_MASK, lz, q), e);
                if (lane == q) ek = e;
            }
            const double term = k < K ? ex_dev(__dsub_rn(__dsub_rn(__dmul_rn(c, z), a), ek)) : 0.0;
            for (int q = 0; q < m; ++q) s = __dadd_rn(s, __shfl_sync(GCSL_FULL_MASK, term, q));
        }
        return s;
    }
    double e = even ? 1.0 : 0.5641895835477562869480795 / sqrt(a);
    double c = 0.0;
    for (long long k0 = 0; k0 < K; k0 += 32) {
        const long long k = k0 + lane;
        const double q_k = k < K ? a / (z0 + (double)k) : 0.0;
        const int m = (int)(K - k0 < 32 ? K - k0 : 32);
        for (int q = 0; q < m; ++q) {
            e = __dmul_rn(e, __shfl_sync(GCSL_FULL_MASK, q_k, q));
            c = __dadd_rn(c, e);
        }
    }
    return __dadd_rn(__dmul_rn(c, y), s);
}

// ------------------------------------------------------------ test kernel

__device__ __forceinline__ void tri_pair(long long t, int &vi, int &vj) {
    // t -> (vi > vj), t = vi (vi - 1) / 2 + vj
    long long i = (long long)((1.0 + sqrt(1.0 + 8.0 * (double)t)) * 0.5);
    while (i * (i - 1) / 2 > t) --i;
    while ((i + 1) * i / 2 <= t) ++i;
    vi = (int)i;
    vj = (int)(t - i * (i - 1) / 2);
}

// Count the table N[s][a][b] of one test into shared memory (all threads of the CTA).
// S / mult live in shared memory; `copies` replicas of T counters are merged into the
// first one before returning.
//
// `trusted`: every code of every column is below its cardinality (checked once per
// solve by disc_validate_kernel), so no sample needs a range check.  Tables of at most
// 256 cells then take the packed path: with every code in range each byte lane of
// ((sum_k s_k m_k) * di + a) * dj + b stays below T <= 256, so 32-bit multiplies and
// adds on four samples' bytes at once carry nothing between lanes and give the four
// cell indices of the scalar formula.
__device__ void count_table(const uint8_t *__restrict__ data, long long ld, long long n, int vi, int vj,
                            const int *S, const int *mult, int L, int di, int dj, int T, int copies,
                            uint32_t *sm_tab, int *bad, bool trusted) {
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int k = tid; k < T * copies; k += nt) sm_tab[k] = 0;
    __syncthreads();
    uint32_t *tab = sm_tab + (size_t)(tid % copies) * T;
    const uint4 *ci = reinterpret_cast<const uint4 *>(data + (size_t)vi * ld);
    const uint4 *cj = reinterpret_cast<const uint4 *>(data + (size_t)vj * ld);
    const long long nvec = (n + 15) >> 4;
    // the debug build always takes the checked path below (every cell index is checked)
    if (trusted && T <= 256 && !GCSL_DEBUG_CHECKS) {
        const long long nfull = n >> 4;  // vectors of 16 samples, all valid
        for (long long v = tid; v < nfull; v += nt) {
            uint32_t s4[4] = {0u, 0u, 0u, 0u};
            for (int k = 0; k < L; ++k) {
                const uint4 w = __ldg(reinterpret_cast<const uint4 *>(data + (size_t)S[k] * ld) + v);
                const uint32_t mk = (uint32_t)mult[k];
                s4[0] += w.x * mk;
                s4[1] += w.y * mk;
                s4[2] += w.z * mk;
                s4[3] += w.w * mk;
            }
            const uint4 xi = __ldg(ci + v), xj = __ldg(cj + v);
            const uint32_t idx4[4] = {(s4[0] * (uint32_t)di + xi.x) * (uint32_t)dj + xj.x,
                                      (s4[1] * (uint32_t)di + xi.y) * (uint32_t)dj + xj.y,
                                      (s4[2] * (uint32_t)di + xi.z) * (uint32_t)dj + xj.z,
                                      (s4[3] * (uint32_t)di + xi.w) * (uint32_t)dj + xj.w};
#pragma unroll
            for (int q = 0; q < 16; ++q) atomicAdd(&tab[(idx4[q >> 2] >> (8 * (q & 3))) & 0xffu], 1u);
        }
        // the last, partial vector
        if (tid == 0 && (n & 15)) {
            const long long v = nfull;
            const int nvalid = (int)(n & 15);
            for (int q = 0; q < nvalid; ++q) {
                const size_t off = (size_t)(v << 4) + q;
                int sidx = 0;
                for (int k = 0; k < L; ++k) sidx += (int)data[(size_t)S[k] * ld + off] * mult[k];
                const int a = data[(size_t)vi * ld + off], b = data[(size_t)vj * ld + off];
                atomicAdd(&tab[(sidx * di + a) * dj + b], 1u);
            }
        }
    } else
    for (long long v = tid; v < nvec; v += nt) {
        int sidx[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) sidx[q] = 0;
        for (int k = 0; k < L; ++k) {
            const uint4 w = __ldg(reinterpret_cast<const uint4 *>(data + (size_t)S[k] * ld) + v);
            const int mk = mult[k];
            const uint32_t ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
            for (int q = 0; q < 16; ++q) sidx[q] += (int)((ww[q >> 2] >> (8 * (q & 3))) & 0xffu) * mk;
        }
        const uint4 xi = __ldg(ci + v), xj = __ldg(cj + v);
        const uint32_t wi[4] = {xi.x, xi.y, xi.z, xi.w};
        const uint32_t wj[4] = {xj.x, xj.y, xj.z, xj.w};
        const long long rem = n - (v << 4);
        const int nvalid = rem >= 16 ? 16 : (int)rem;
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            if (q < nvalid) {
                const int a = (int)((wi[q >> 2] >> (8 * (q & 3))) & 0xffu);
                const int b = (int)((wj[q >> 2] >> (8 * (q & 3))) & 0xffu);
                const int idx = (sidx[q] * di + a) * dj + b;
                // codes at or above their cardinality are invalid input: never written
                if ((unsigned)idx < (unsigned)T && a < di && b < dj) atomicAdd(&tab[idx], 1u);
                else *bad = 1;
            }
        }
    }
    __syncthreads();
    if (copies > 1) {
        for (int k = tid; k < T; k += nt) {
            uint32_t s = 0;
            for (int c = 0; c < copies; ++c) s += sm_tab[(size_t)c * T + k];
            sm_tab[k] = s;
        }
        __syncthreads();
    }
}

// chi^2 partial sum of one stratum, (a, b) order; E = N_a+ N_+b / N_++, terms with
// N_++ == 0 or E == 0 skipped (discrete_helpers.cu:164-186).
__device__ double stratum_chi2(const uint32_t *Ts, int di, int dj) {
    double part = 0.0;
    if (di <= 16 && dj <= 16) {
        uint32_t ma[16], mb[16];
        uint32_t mt = 0;
#pragma unroll
        for (int a = 0; a < 16; ++a) ma[a] = mb[a] = 0;
        for (int a = 0; a < di; ++a)
            for (int b = 0; b < dj; ++b) {
                const uint32_t o = Ts[a * dj + b];
                ma[a] += o;
                mb[b] += o;
                mt += o;
            }
        if (mt == 0) return 0.0;
        for (int a = 0; a < di; ++a)
            for (int b = 0; b < dj; ++b) {
                const double e = __ddiv_rn(__dmul_rn((double)ma[a], (double)mb[b]), (double)mt);
                if (e == 0.0) continue;
                const double d = __dsub_rn((double)Ts[a * dj + b], e);
                part = __dadd_rn(part, __ddiv_rn(__dmul_rn(d, d), e));
            }
        return part;
    }
    // wide tables: the marginals are recomputed from the table (same integers)
    uint32_t mt = 0;
    for (int k = 0; k < di * dj; ++k) mt += Ts[k];
    if (mt == 0) return 0.0;
    for (int a = 0; a < di; ++a) {
        uint32_t ma = 0;
        for (int b = 0; b < dj; ++b) ma += Ts[a * dj + b];
        for (int b = 0; b < dj; ++b) {
            uint32_t mb = 0;
            for (int a2 = 0; a2 < di; ++a2) mb += Ts[a2 * dj + b];
            const double e = __ddiv_rn(__dmul_rn((double)ma, (double)mb), (double)mt);
            if (e == 0.0) continue;
            const double d = __dsub_rn((double)Ts[a * dj + b], e);
            part = __dadd_rn(part, __ddiv_rn(__dmul_rn(d, d), e));
        }
    }
    return part;
}

// stratum_chi2 by the 32 lanes of one warp (di, dj <= 32), bit for bit: lane a / b holds
// the row / column sums, every lane one cell's term (its two divisions), and the terms
// are added in (a, b) order as in stratum_chi2.  The sum is meaningful in every lane.
__device__ double stratum_chi2_warp(const uint32_t *Ts, int di, int dj) {
    const int lane = threadIdx.x & 31;
    uint32_t ma = 0, mb = 0;
    if (lane < di)
        for (int b = 0; b < dj; ++b) ma += Ts[lane * dj + b];
    if (lane < dj)
        for (int a = 0; a < di; ++a) mb += Ts[a * dj + lane];
    uint32_t mt = lane < di ? ma : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mt += __shfl_xor_sync(GCSL_FULL_MASK, mt, o);
    if (mt == 0) return 0.0;
    double part = 0.0;
    const int cells = di * dj;
    for (int k0 = 0; k0 < cells; k0 += 32) {
        const int k = k0 + lane;
        const int a = k < cells ? k / dj : 0, b = k < cells ? k - (k / dj) * dj : 0;
        const uint32_t mak = __shfl_sync(GCSL_FULL_MASK, ma, a), mbk = __shfl_sync(GCSL_FULL_MASK, mb, b);
        double term = 0.0;
        bool use = false;
        if (k < cells) {
            const double e = __ddiv_rn(__dmul_rn((double)mak, (double)mbk), (double)mt);
            if (e != 0.0) {
                const double d = __dsub_rn((double)Ts[k], e);
                term = __ddiv_rn(__dmul_rn(d, d), e);
                use = true;
            }
        }
        const unsigned um = __ballot_sync(GCSL_FULL_MASK, use);
        const int m = cells - k0 < 32 ? cells - k0 : 32;
        for (int q = 0; q < m; ++q) {
            const double t = __shfl_sync(GCSL_FULL_MASK, term, q);
            if ((um >> q) & 1u) part = __dadd_rn(part, t);
        }
    }
    return part;
}

// Statistic of the counted table: strata in parallel (a warp per stratum), then added in
// ascending s by thread 0 (the return value is meaningful in thread 0 only).
__device__ double table_chi2(const uint32_t *sm_tab, int dim_s, int di, int dj, double *s_part) {
    if (di <= 32 && dj <= 32) {
        const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
        for (int s = warp; s < dim_s; s += nwarps) {
            const double part = stratum_chi2_warp(sm_tab + (size_t)s * di * dj, di, dj);
            if ((threadIdx.x & 31) == 0) s_part[s] = part;
        }
    } else {
        for (int s = threadIdx.x; s < dim_s; s += blockDim.x)
            s_part[s] = stratum_chi2(sm_tab + (size_t)s * di * dj, di, dj);
    }
    __syncthreads();
    double chi = 0.0;
    if (threadIdx.x == 0)
        for (int s = 0; s < dim_s; ++s) chi = __dadd_rn(chi, s_part[s]);
    return chi;
}

// Per-test header prepared by thread 0: table geometry and replica count.
__device__ __forceinline__ bool table_geometry(const uint8_t *dims, const int *S, int *mult, int L, int vi, int vj,
                                               int table_cap, int part_cap, int &dim_s, int &di, int &dj,
                                               int &copies) {
    long long ds = 1;
    for (int k = 0; k < L; ++k) {
        mult[k] = (int)ds;
        ds *= dims[S[k]];
        if (ds > table_cap) return false;
    }
    di = dims[vi];
    dj = dims[vj];
    const long long T = ds * di * dj;
    if (T > table_cap || ds > part_cap) return false;
    dim_s = (int)ds;
    copies = 1;
    if (T <= table_cap / 8) copies = 8;
    else if (T <= table_cap / 4) copies = 4;
    else if (T <= table_cap / 2) copies = 2;
    return true;
}

__global__ void __launch_bounds__(256) disc_test_kernel(DiscLevelArgs A) {
    extern __shared__ uint32_t sm_tab[];
    __shared__ int s_S[GCSL_MAX_LEVELS + 2];
    __shared__ int s_mult[GCSL_MAX_LEVELS + 2];
    __shared__ int s_hdr[7];  // vi, vj, di, dj, dim_s, copies, ok
    __shared__ long long s_rank;
    __shared__ int s_bad;
    // per-stratum statistics follow the counters (8-byte aligned)
    double *s_part = reinterpret_cast<double *>(sm_tab + ((A.table_cap + 1) & ~1));
    __shared__ int s_trusted;
    DevState *st = A.st;
    if (threadIdx.x == 0) {
        s_bad = 0;
        // codes checked in range for this solve: disc_validate_kernel ran before level 0
        // and leaves the status 0 only then (any other error also selects the checked
        // path); read once per CTA, seen by all threads after the first barrier below
        s_trusted = *(volatile const int32_t *)&st->status == 0;
    }
    const int L = A.level;
    if (L > 0) {
        if (st->done) return;
        const int md = st->max_degree[L];
        if (md - 1 < L) {
            if (blockIdx.x == 0 && threadIdx.x == 0) st->done = 1;
            return;
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) st->last_level = L;
    }
    const long long total = (L == 0) ? (long long)A.p * (A.p - 1) / 2 : A.prefix[A.p];
    const int tid = threadIdx.x;

    for (long long t0 = blockIdx.x; t0 < total; t0 += gridDim.x) {
        const long long t = work_order(t0, total, A.order);
        if (tid == 0) {
            int vi, vj;
            long long rank = 0;
            if (L == 0) {
                tri_pair(t, vi, vj);
            } else {
                vi = upper_row(A.prefix, A.p, t);
                const long long off = t - A.prefix[vi];
                const int deg = A.adj[(size_t)vi * A.p];
                const long long R = binom_rt(deg - 1, L);
                const int m = (int)(off / R);
                rank = off - (long long)m * R;
                vj = A.adj[(size_t)vi * A.p + 1 + m];
                unrank_positions_rt(L, deg - 1, rank, s_S);
                const int *nbrs = A.adj + (size_t)vi * A.p + 1;
                for (int c = 0; c < L; ++c) s_S[c] = resolve_position(nbrs, vj, s_S[c]);
            }
            int dim_s = 0, di = 0, dj = 0, copies = 1;
            const bool ok =
                table_geometry(A.dims, s_S, s_mult, L, vi, vj, A.table_cap, A.part_cap, dim_s, di, dj, copies);
            s_hdr[0] = vi;
            s_hdr[1] = vj;
            s_hdr[2] = di;
            s_hdr[3] = dj;
            s_hdr[4] = dim_s;
            s_hdr[5] = copies;
            s_hdr[6] = ok;
            s_rank = rank;
            if (!ok) set_status(st, GCSL_ERR_UNSUPPORTED);
        }
        __syncthreads();
        if (!s_hdr[6]) {
            __syncthreads();
            continue;
        }
        const int vi = s_hdr[0], vj = s_hdr[1], di = s_hdr[2], dj = s_hdr[3], dim_s = s_hdr[4];
        count_table(A.data, A.ld, A.n, vi, vj, s_S, s_mult, L, di, dj, dim_s * di * dj, s_hdr[5], sm_tab,
                    &s_bad, s_trusted != 0);
        const double chi = table_chi2(sm_tab, dim_s, di, dj, s_part);
        if (tid == 0 && s_bad) set_status(st, GCSL_ERR_INVALID_ARG);
        double pv = 1.0;
        if (tid < 32) {  // warp 0: the p-value's series split over the lanes
            const long long df = (long long)(di - 1) * (long long)(dj - 1) * (long long)dim_s;
            pv = pchisq_warp(__shfl_sync(GCSL_FULL_MASK, chi, 0), df);
        }
        if (tid == 0) {
            const int lo = vi < vj ? vi : vj, hi = vi < vj ? vj : vi;
            const size_t ix = (size_t)lo * A.p + hi;
            if (L == 0) {
                A.pmax[ix] = pv;
                const uint16_t keep = (pv >= A.alpha) ? 0 : 1;
                A.G[(size_t)vi * A.p + vj] = keep;
                A.G[(size_t)vj * A.p + vi] = keep;
            } else {
                atomic_max_nonneg(&A.pmax[ix], pv);
                if (pv >= A.alpha) {
                    const unsigned long long key = ((unsigned long long)s_rank << 1) | (vi < vj ? 0ull : 1ull);
                    atomicMin(&A.win[ix], key);
                }
            }
        }
        __syncthreads();
    }
    if (blockIdx.x == 0 && tid == 0) st->tests[L] = (unsigned long long)total;
}

// One test for the unit entry point: counts and (chi^2, p-value) to global memory.
struct UnitSet {
    int S[GCSL_MAX_LEVELS];
};

__global__ void __launch_bounds__(256) disc_table_kernel(const uint8_t *data, long long ld, long long n,
                                                         const uint8_t *dims, int vi, int vj, UnitSet us, int L,
                                                         int table_cap, uint32_t *counts, long long counts_cap,
                                                         double *out2) {
    extern __shared__ uint32_t sm_tab[];
    __shared__ int s_S[GCSL_MAX_LEVELS + 2];
    __shared__ int s_mult[GCSL_MAX_LEVELS + 2];
    __shared__ int s_hdr[4];
    __shared__ double s_part[1024];
    if (threadIdx.x == 0) {
        for (int k = 0; k < L; ++k) s_S[k] = us.S[k];
        int dim_s = 0, di = 0, dj = 0, copies = 1;
        bool ok = table_geometry(dims, s_S, s_mult, L, vi, vj, table_cap, 1024, dim_s, di, dj, copies);
        if (ok && (long long)dim_s * di * dj > counts_cap) ok = false;  // never write past the caller's buffer
        s_hdr[0] = ok ? dim_s : -1;
        s_hdr[1] = di;
        s_hdr[2] = dj;
        s_hdr[3] = copies;
    }
    __syncthreads();
    const int dim_s = s_hdr[0], di = s_hdr[1], dj = s_hdr[2];
    if (dim_s < 0) {
        if (threadIdx.x == 0) out2[0] = out2[1] = -1.0;
        return;
    }
    const int T = dim_s * di * dj;
    __shared__ int s_bad;
    if (threadIdx.x == 0) s_bad = 0;
    count_table(data, ld, n, vi, vj, s_S, s_mult, L, di, dj, T, s_hdr[3], sm_tab, &s_bad, false);
    for (int k = threadIdx.x; k < T; k += blockDim.x) counts[k] = sm_tab[k];
    const double chi = table_chi2(sm_tab, dim_s, di, dj, s_part);
    if (threadIdx.x == 0) {
        if (s_bad) {
            out2[0] = out2[1] = -1.0;
            return;
        }
        out2[0] = chi;
        out2[1] = pchisq_dev(chi, (long long)(di - 1) * (long long)(dj - 1) * (long long)dim_s);
    }
}

// Per-row weights deg_r * C(deg_r - 1, L) of the level's flattened test list.
// Codes in range: every code of columns 0..p-1 (samples 0..n-1) below its cardinality.
// Sets GCSL_ERR_INVALID_ARG otherwise, which makes the test kernels check every sample.
// A byte x of a word is >= d (1 <= d <= 128) iff the high bit of (x + 128 - d) | x is
// set; with all bytes below d nothing carries between bytes, and a byte >= 128 (which
// may carry) has its own high bit set, so the word test is exact.
__global__ void __launch_bounds__(256) disc_validate_kernel(const uint8_t *__restrict__ data, long long ld,
                                                            long long n, int p, const uint8_t *__restrict__ dims,
                                                            DevState *st) {
    const long long nvec = (n + 15) >> 4;
    const long long total = nvec * p;
    bool bad = false;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int col = (int)(i / nvec);
        const long long v = i - (long long)col * nvec;
        const uint32_t d = dims[col];
        const uint4 w = __ldg(reinterpret_cast<const uint4 *>(data + (size_t)col * ld) + v);
        const long long rem = n - (v << 4);
        if (d == 0 || d > 128 || rem < 16) {  // rare: byte by byte
            const uint32_t ww[4] = {w.x, w.y, w.z, w.w};
            const int nvalid = rem >= 16 ? 16 : (int)rem;
            for (int q = 0; q < nvalid; ++q) bad |= ((ww[q >> 2] >> (8 * (q & 3))) & 0xffu) >= d;
        } else {
            const uint32_t add = (0x80u - d) * 0x01010101u;
            const uint32_t hit = (((w.x + add) | w.x) | ((w.y + add) | w.y) | ((w.z + add) | w.z) |
                                  ((w.w + add) | w.w)) & 0x80808080u;
            bad |= hit != 0;
        }
    }
    if (__any_sync(GCSL_FULL_MASK, bad) && (threadIdx.x & 31) == 0) set_status(st, GCSL_ERR_INVALID_ARG);
}

__global__ void disc_weights_kernel(const int *__restrict__ adj, int p, int L, long long *__restrict__ w,
                                    DevState *st) {
    if (st->done) return;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= p) return;
    const int deg = adj[(size_t)r * p];
    const long long R = (deg - 1 >= L) ? binom_rt(deg - 1, L) : 0;
    if (R >= GCSL_RANK_LIMIT) set_status(st, GCSL_ERR_UNSUPPORTED);
    w[r] = (long long)deg * R;
}

// Write-back of a level: canonical remover -> skeleton, sepsets, records.
__global__ void disc_finalize_kernel(const int *__restrict__ adj, int p, int L, uint16_t *G,
                                     unsigned long long *win, int *sep_dense, int max_level, int *rec_pool,
                                     long long rec_cap, DevState *st) {
    if (st->done) return;
    if (st->max_degree[L] - 1 < L) return;
    const long long total = (long long)p * p;
    unsigned long long removed = 0;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const unsigned long long key = win[k];
        if (key == GCSL_KEY_NONE) continue;
        win[k] = GCSL_KEY_NONE;
        const int lo = (int)(k / p), hi = (int)(k - (long long)lo * p);
        const long long rank = (long long)(key >> 1);
        const int vi = (key & 1) ? hi : lo, vj = (key & 1) ? lo : hi;
        const int *row = adj + (size_t)vi * p;
        int S[GCSL_MAX_LEVELS];
        unrank_positions_rt(L, row[0] - 1, rank, S);
        for (int c = 0; c < L; ++c) S[c] = resolve_position(row + 1, vj, S[c]);
        G[(size_t)lo * p + hi] = 0;
        G[(size_t)hi * p + lo] = 0;
        if (sep_dense != nullptr && L <= max_level) {
            for (int c = 0; c < L; ++c) {
                sep_dense[((size_t)lo * p + hi) * max_level + c] = S[c];
                sep_dense[((size_t)hi * p + lo) * max_level + c] = S[c];
            }
        }
        if (rec_pool != nullptr) {
            const unsigned long long off = atomicAdd(&st->n_rec_ints, (unsigned long long)(3 + L));
            if ((long long)(off + 3 + L) <= rec_cap) {
                rec_pool[off] = lo;
                rec_pool[off + 1] = hi;
                rec_pool[off + 2] = L;
                for (int c = 0; c < L; ++c) rec_pool[off + 3 + c] = S[c];
            } else {
                set_status(st, GCSL_ERR_CAPACITY);
            }
        }
        ++removed;
    }
    if (removed) atomicAdd(&st->removed[L], removed);
}

// Edges alive at level start and the level's full test space (for the stats).
__global__ void disc_level_stats_kernel(const long long *__restrict__ prefix, const int *__restrict__ adj, int p,
                                        int L, DevState *st) {
    if (st->done) return;
    if (threadIdx.x == 0 && blockIdx.x == 0) st->tests_full[L] = (unsigned long long)prefix[p];
    unsigned long long e = 0;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < p; r += gridDim.x * blockDim.x)
        e += (unsigned long long)adj[(size_t)r * p];
    if (e) atomicAdd(&st->edges[L], e);  // directed count; halved on the host
}

__global__ void pmax_finish_kernel(double *pmax, int p) {
    const long long total = (long long)p * p;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / p), j = (int)(k - (long long)i * p);
        if (i >= j) pmax[k] = -1.0;
    }
}

// Unit entry point kernels -------------------------------------------------
__global__ void pchisq_kernel(const double *x, const long long *df, long long count, double *out) {
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < count;
         k += (long long)gridDim.x * blockDim.x)
        out[k] = pchisq_dev(x[k], df[k]);
}

namespace host {

int disc_table_cap(int device) {
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    // leave room for the static shared arrays of the kernels and 1024 strata statistics
    const int dyn = optin - 16 * 1024;
    return dyn / (int)sizeof(uint32_t);
}

// Shared memory of one level's tables: the largest table of the level has at most
// max_dim^(L+2) counters; small tables get replicas (fewer atomic collisions) while the
// footprint stays small enough for several CTAs per SM.  Levels whose largest table
// would not fit take the whole budget.
void disc_level_caps(int cap_full, int max_dim, int L, int &table_cap, int &part_cap) {
    long long need = 1, ds = 1;
    for (int k = 0; k < L + 2 && need <= cap_full; ++k) {
        need *= max_dim;
        if (k < L) ds *= max_dim;
    }
    if (need > cap_full || ds > 1024) {
        table_cap = cap_full;
        part_cap = 1024;
        return;
    }
    const long long reps = need <= 512 ? 8 : need <= 2048 ? 4 : need <= 8192 ? 2 : 1;
    table_cap = (int)(need * reps < cap_full ? need * reps : cap_full);
    part_cap = (int)ds;
}

cudaError_t launch_disc_tests(const DiscLevelArgs &A, int num_sms, cudaStream_t s) {
    const size_t smem = (size_t)((A.table_cap + 1) & ~1) * sizeof(uint32_t) + (size_t)A.part_cap * sizeof(double);
    static std::atomic<unsigned long long> limit_set{0};
    const cudaError_t ea = raise_dyn_smem_limit(disc_test_kernel, limit_set);
    if (ea != cudaSuccess) return note_error("disc_test_kernel shared memory", ea);
    int per_sm = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, disc_test_kernel, 256, smem) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    const int cap = blocks_per_sm_cap();  // room left on every SM for concurrent solves
    if (cap > 0 && per_sm > cap) per_sm = cap;
    disc_test_kernel<<<num_sms * per_sm, 256, smem, s>>>(A);
    note_launch(1);
    return note_error("disc_test_kernel launch", cudaGetLastError());
}

cudaError_t launch_disc_validate(const uint8_t *data, long long ld, long long n, int p, const uint8_t *dims,
                                 DevState *st, int num_sms, cudaStream_t s) {
    disc_validate_kernel<<<num_sms * 4, 256, 0, s>>>(data, ld, n, p, dims, st);
    note_launch(1);
    return note_error("disc_validate_kernel launch", cudaGetLastError());
}

cudaError_t launch_disc_weights(const int *adj, int p, int L, long long *w, DevState *st, cudaStream_t s) {
    disc_weights_kernel<<<(p + 255) / 256, 256, 0, s>>>(adj, p, L, w, st);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_disc_finalize(const int *adj, int p, int L, uint16_t *G, unsigned long long *win, int *sep,
                                 int max_level, int *rec, long long rec_cap, DevState *st, int num_sms,
                                 cudaStream_t s) {
    disc_finalize_kernel<<<num_sms * 2, 256, 0, s>>>(adj, p, L, G, win, sep, max_level, rec, rec_cap, st);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_disc_level_stats(const long long *prefix, const int *adj, int p, int L, DevState *st,
                                    cudaStream_t s) {
    disc_level_stats_kernel<<<(p + 255) / 256, 256, 0, s>>>(prefix, adj, p, L, st);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_pmax_finish(double *pmax, int p, int num_sms, cudaStream_t s) {
    pmax_finish_kernel<<<num_sms * 2, 256, 0, s>>>(pmax, p);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_disc_table(const uint8_t *data, long long ld, long long n, const uint8_t *dims, int vi, int vj,
                              const int *S, int L, int table_cap, uint32_t *counts, long long counts_cap, double *out2,
                              cudaStream_t s) {
    UnitSet us;
    for (int k = 0; k < GCSL_MAX_LEVELS; ++k) us.S[k] = k < L ? S[k] : 0;
    const size_t smem = (size_t)table_cap * sizeof(uint32_t);
    cudaFuncSetAttribute(disc_table_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    disc_table_kernel<<<1, 256, smem, s>>>(data, ld, n, dims, vi, vj, us, L, table_cap, counts, counts_cap, out2);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t launch_pchisq(const double *x, const long long *df, long long count, double *out, cudaStream_t s) {
    const int blocks = (int)((count + 255) / 256);
    pchisq_kernel<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(x, df, count, out);
    note_launch(1);
    return cudaGetLastError();
}

}  // namespace host
}  // namespace gcsl
