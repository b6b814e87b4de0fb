/*
 * ORACLE — test infrastructure only. Nothing in the product (gpucsl_gb300/) links,
 * loads or calls this file; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use it, as the checker.
 *
 * Plain-C restatement of the scalar and integer arithmetic of the reference's
 * skeleton-discovery path (hpi-epic/gpucsl), written from the published methods:
 *
 *   binomial coefficient          gpucsl/pc/cuda/helpers/math_helpers.cu:20-33
 *   normal tail (Perlman z.c,     gpucsl/pc/cuda/helpers/math_helpers.cu:54-105
 *     Ibbetson CACM Alg. 209)
 *   chi-squared upper tail        gpucsl/pc/cuda/helpers/math_helpers.cu:128-175
 *     (Hill & Pike CACM Alg. 299, Perlman chisq.c)
 *   lexicographic set unranking   gpucsl/pc/cuda/helpers/set_helpers.cu:25-71
 *   contingency tables, marginals gpucsl/pc/cuda/helpers/discrete_helpers.cu:25-186
 *     and Pearson chi-squared
 *   discrete level loop           gpucsl/pc/discover_skeleton_discrete.py:80-112,
 *                                 gpucsl/pc/cuda/discrete_ci.cu:37-246
 *
 * Canonical rules where the reference is non-deterministic (its sepset is whichever
 * removing test wins a CAS; its level-l chi-squared is a double atomicAdd):
 *   - sepset winner of an edge = the removing test with the smallest key
 *     (rank, direction), direction 0 when v_i = min(i, j);
 *   - level-l chi-squared: each stratum s sums its (a, b) terms a-major, then the
 *     stratum sums are added in ascending s;
 *   - pmax is FP64 (the reference stores FP32).
 * Compiled with -ffp-contract=off so every FP64 operation rounds on its own.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------- binomial */
/* Multiplicative formula in int64; math_helpers.cu:20-33 does the same in int. */
int64_t orc_binomial(int64_t n, int64_t k) {
    if (k < 0 || n < k) return 0;
    if (k > n - k) k = n - k;
    int64_t r = 1;
    for (int64_t i = 0; i < k; ++i) {
        r *= (n - i);
        r /= (i + 1);
    }
    return r;
}

/* ------------------------------------------------------------- unranking */
/* rank -> 1-based positions x_0 < ... < x_{l-1} in {1..K}, lexicographic order
 * (set_helpers.cu:25-49). */
void orc_unrank(int64_t K, int l, int64_t rank, int32_t *pos) {
    int64_t x = 0;
    for (int c = 0; c < l; ++c) {
        x += 1;
        for (;;) {
            int64_t cnt = orc_binomial(K - x, l - c - 1);
            if (rank < cnt) break;
            rank -= cnt;
            x += 1;
        }
        pos[c] = (int32_t)x;
    }
}

/* positions -> variable ids, skipping v_j inside the ascending neighbour list
 * (set_helpers.cu:51-57). */
void orc_resolve(const int32_t *nbrs, int l, int32_t vj, const int32_t *pos, int32_t *S) {
    for (int c = 0; c < l; ++c) {
        int32_t idx = pos[c] - 1;
        if (nbrs[idx] >= vj) idx += 1;
        S[c] = nbrs[idx];
    }
}

/* ------------------------------------------------------- normal / chi^2 */
#define ORC_Z_MAX 6.0
#define ORC_BIGX 20.0
#define ORC_LOG_SQRT_PI 0.5723649429247000870717135
#define ORC_I_SQRT_PI 0.5641895835477562869480795

static double orc_ex(double x) { return (x < -ORC_BIGX) ? 0.0 : exp(x); }

/* Normal CDF approximation of Ibbetson (CACM Alg. 209) as coded by Perlman;
 * the two polynomials are the published ones. */
double orc_poz(double z) {
    double x;
    if (z == 0.0) {
        x = 0.0;
    } else {
        double y = 0.5 * fabs(z);
        if (y >= ORC_Z_MAX * 0.5) {
            x = 1.0;
        } else if (y < 1.0) {
            double w = y * y;
            double t = 0.000124818987;
            t = t * w - 0.001075204047;
            t = t * w + 0.005198775019;
            t = t * w - 0.019198292004;
            t = t * w + 0.059054035642;
            t = t * w - 0.151968751364;
            t = t * w + 0.319152932694;
            t = t * w - 0.531923007300;
            t = t * w + 0.797884560593;
            x = t * y * 2.0;
        } else {
            y -= 2.0;
            double t = -0.000045255659;
            t = t * y + 0.000152529290;
            t = t * y - 0.000019538132;
            t = t * y - 0.000676904986;
            t = t * y + 0.001390604284;
            t = t * y - 0.000794620820;
            t = t * y - 0.002034254874;
            t = t * y + 0.006549791214;
            t = t * y - 0.010557625006;
            t = t * y + 0.011630447319;
            t = t * y - 0.009279453341;
            t = t * y + 0.005353579108;
            t = t * y - 0.002141268741;
            t = t * y + 0.000535310849;
            x = t * y + 0.999936657524;
        }
    }
    return z > 0.0 ? ((x + 1.0) * 0.5) : ((1.0 - x) * 0.5);
}

/* Upper tail of chi^2 with df degrees of freedom, Hill & Pike Alg. 299 with the
 * 1985 rounding remark, in Perlman's formulation (math_helpers.cu:128-175). */
double orc_pchisq(double x, int64_t df) {
    if (x <= 0.0 || df < 1) return 1.0;
    double a = 0.5 * x;
    int even = (df % 2) == 0;
    double y = 0.0;
    if (df > 1) y = orc_ex(-a);
    double s = even ? y : 2.0 * orc_poz(-sqrt(x));
    if (df <= 2) return s;
    double half = 0.5 * ((double)df - 1.0);
    double z = even ? 1.0 : 0.5;
    if (a > ORC_BIGX) {
        double e = even ? 0.0 : ORC_LOG_SQRT_PI;
        double c = log(a);
        while (z <= half) {
            e = log(z) + e;
            s += orc_ex(c * z - a - e);
            z += 1.0;
        }
        return s;
    }
    double e = even ? 1.0 : ORC_I_SQRT_PI / sqrt(a);
    double c = 0.0;
    while (z <= half) {
        e = e * (a / z);
        c = c + e;
        z += 1.0;
    }
    return c * y + s;
}

/* --------------------------------------------------------- discrete test */
/* Counts N[s][a][b] (discrete_helpers.cu:40-85), a = value of v_i, b = value of v_j,
 * stratum s = sum_k x_{S_k} * prod_{k'<k} d_{S_k'}.  data is column-major with
 * column stride ld.  counts must hold dim_s*d_i*d_j entries. */
void orc_contingency(const uint8_t *data, int64_t ld, int64_t n, const uint8_t *dims, int32_t vi,
                     int32_t vj, const int32_t *S, int l, uint32_t *counts) {
    int di = dims[vi], dj = dims[vj];
    int64_t dim_s = 1;
    for (int k = 0; k < l; ++k) dim_s *= dims[S[k]];
    memset(counts, 0, sizeof(uint32_t) * (size_t)(dim_s * di * dj));
    const uint8_t *xi = data + (int64_t)vi * ld;
    const uint8_t *xj = data + (int64_t)vj * ld;
    for (int64_t t = 0; t < n; ++t) {
        int64_t s = 0, m = 1;
        for (int k = 0; k < l; ++k) {
            s += (int64_t)data[(int64_t)S[k] * ld + t] * m;
            m *= dims[S[k]];
        }
        counts[(s * di + xi[t]) * dj + xj[t]] += 1;
    }
}

/* Pearson chi^2 of a level-0 table (discrete_helpers.cu:97-106, 140-155):
 * E = m_i[a] * m_j[b] / n, summed a-major, terms with E == 0 skipped. */
double orc_chi2_level0(const uint32_t *N, int di, int dj, int64_t n) {
    int64_t mi[256], mj[256];
    for (int a = 0; a < di; ++a) mi[a] = 0;
    for (int b = 0; b < dj; ++b) mj[b] = 0;
    for (int a = 0; a < di; ++a)
        for (int b = 0; b < dj; ++b) {
            mi[a] += N[a * dj + b];
            mj[b] += N[a * dj + b];
        }
    double chi = 0.0;
    for (int a = 0; a < di; ++a)
        for (int b = 0; b < dj; ++b) {
            double e = (double)mi[a] * (double)mj[b] / (double)n;
            if (e != 0.0) {
                double o = (double)N[a * dj + b];
                chi += (o - e) * (o - e) / e;
            }
        }
    return chi;
}

/* Pearson chi^2 of a stratified table (discrete_helpers.cu:120-133, 164-186):
 * E = N_{a+s} * N_{+bs} / N_{++s}, terms with N_{++s} == 0 or E == 0 skipped.
 * Canonical order: per stratum a-major partial sum, strata added ascending. */
double orc_chi2_level_n(const uint32_t *N, int64_t dim_s, int di, int dj) {
    double chi = 0.0;
    for (int64_t s = 0; s < dim_s; ++s) {
        const uint32_t *T = N + s * di * dj;
        uint32_t ma[256], mb[256], mt = 0;
        for (int a = 0; a < di; ++a) ma[a] = 0;
        for (int b = 0; b < dj; ++b) mb[b] = 0;
        for (int a = 0; a < di; ++a)
            for (int b = 0; b < dj; ++b) {
                ma[a] += T[a * dj + b];
                mb[b] += T[a * dj + b];
                mt += T[a * dj + b];
            }
        if (mt == 0) continue;
        double part = 0.0;
        for (int a = 0; a < di; ++a)
            for (int b = 0; b < dj; ++b) {
                double e = (double)ma[a] * (double)mb[b] / (double)mt;
                if (e == 0.0) continue;
                double o = (double)T[a * dj + b];
                part += (o - e) * (o - e) / e;
            }
        chi += part;
    }
    return chi;
}

/* One conditional-independence test; returns the p-value and, if out_chi is
 * non-null, the statistic.  work must hold dim_s*d_i*d_j uint32. */
double orc_discrete_test(const uint8_t *data, int64_t ld, int64_t n, const uint8_t *dims, int32_t vi,
                         int32_t vj, const int32_t *S, int l, uint32_t *work, double *out_chi) {
    int di = dims[vi], dj = dims[vj];
    int64_t dim_s = 1;
    for (int k = 0; k < l; ++k) dim_s *= dims[S[k]];
    orc_contingency(data, ld, n, dims, vi, vj, S, l, work);
    double chi = (l == 0) ? orc_chi2_level0(work, di, dj, n) : orc_chi2_level_n(work, dim_s, di, dj);
    if (out_chi) *out_chi = chi;
    int64_t df = (int64_t)(di - 1) * (int64_t)(dj - 1) * dim_s;
    return orc_pchisq(chi, df);
}

/* ------------------------------------------------------ compacted graph */
/* Row r -> [deg_r, sorted neighbour ids...] (graph_helpers.cu:35-56); entries past
 * deg_r are left as they were (the reference does not clear them). */
void orc_compact(const uint16_t *G, int32_t p, int32_t *adj) {
    for (int32_t r = 0; r < p; ++r) {
        int32_t cnt = 0;
        for (int32_t c = 0; c < p; ++c)
            if (c != r && G[(int64_t)r * p + c]) adj[(int64_t)r * p + 1 + cnt++] = c;
        adj[(int64_t)r * p] = cnt;
    }
}

/* ------------------------------------------------ discrete level loop */
typedef struct {
    int32_t levels_run;
    int32_t status;
    int64_t tests[64];
    int64_t removed[64];
} orc_stats;

/* Full discrete skeleton (discover_skeleton_discrete.py:80-112).  Every rank of
 * every direction is tested, as in discrete_ci.cu:221-244; pmax folds all of them.
 * sepsets: p*p*max_level int32 pre-filled with -1 by the caller.  pmax: p*p FP64,
 * upper triangle written (the caller marks the lower triangle -1). */
int orc_discrete_skeleton(const uint8_t *data, int64_t ld, int64_t n, int32_t p, const uint8_t *dims,
                          double alpha, int max_level, uint16_t *G, int32_t *sepsets, double *pmax,
                          int nthreads, orc_stats *st) {
    int max_dim = 0;
    for (int v = 0; v < p; ++v)
        if (dims[v] > max_dim) max_dim = dims[v];
    memset(st, 0, sizeof(*st));
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    /* level 0 */
    for (int64_t k = 0; k < (int64_t)p * p; ++k) pmax[k] = 0.0;
#pragma omp parallel
    {
        uint32_t *work = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)max_dim * max_dim + 4);
#pragma omp for schedule(dynamic, 16)
        for (int32_t vi = 0; vi < p; ++vi) {
            for (int32_t vj = 0; vj < vi; ++vj) {
                double pv = orc_discrete_test(data, ld, n, dims, vi, vj, NULL, 0, work, NULL);
                pmax[(int64_t)vj * p + vi] = pv;
                uint16_t keep = pv >= alpha ? 0 : 1;
                G[(int64_t)vi * p + vj] = keep;
                G[(int64_t)vj * p + vi] = keep;
            }
            G[(int64_t)vi * p + vi] = 0;
        }
        free(work);
    }
    st->tests[0] = (int64_t)p * (p - 1) / 2;
    st->levels_run = 1;

    int32_t *adj = (int32_t *)calloc((size_t)p * p, sizeof(int32_t));
    uint64_t *win = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)p * p);
    int rc = 0;
    for (int level = 1; level <= max_level; ++level) {
        orc_compact(G, p, adj);
        int32_t maxdeg = 0;
        for (int32_t r = 0; r < p; ++r)
            if (adj[(int64_t)r * p] > maxdeg) maxdeg = adj[(int64_t)r * p];
        if (maxdeg - 1 < level) break;
        for (int64_t k = 0; k < (int64_t)p * p; ++k) win[k] = UINT64_MAX;
        int64_t dim_s_max = 1;
        for (int k = 0; k < level; ++k) dim_s_max *= max_dim;
        int64_t tests = 0;
#pragma omp parallel reduction(+ : tests)
        {
            uint32_t *work = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(dim_s_max * max_dim * max_dim) + 4);
            int32_t pos[64], S[64];
#pragma omp for schedule(dynamic, 1)
            for (int32_t vi = 0; vi < p; ++vi) {
                const int32_t *row = adj + (int64_t)vi * p;
                int32_t deg = row[0];
                int64_t K = deg - 1;
                if (K < level) continue;
                int64_t R = orc_binomial(K, level);
                for (int32_t m = 0; m < deg; ++m) {
                    int32_t vj = row[1 + m];
                    int32_t lo = vi < vj ? vi : vj, hi = vi < vj ? vj : vi;
                    uint64_t dir = vi < vj ? 0 : 1;
                    for (int64_t r = 0; r < R; ++r) {
                        orc_unrank(K, level, r, pos);
                        orc_resolve(row + 1, level, vj, pos, S);
                        double pv = orc_discrete_test(data, ld, n, dims, vi, vj, S, level, work, NULL);
                        ++tests;
                        int64_t ix = (int64_t)lo * p + hi;
#pragma omp critical(orc_pmax)
                        {
                            if (pv > pmax[ix]) pmax[ix] = pv;
                            if (pv >= alpha) {
                                uint64_t key = ((uint64_t)r << 1) | dir;
                                if (key < win[ix]) win[ix] = key;
                            }
                        }
                    }
                }
            }
            free(work);
        }
        st->tests[level < 64 ? level : 63] = tests;
        /* write-back: remove edges, canonical sepset (graph_helpers.cu:81-101) */
        int64_t removed = 0;
        int32_t pos[64], S[64];
        for (int32_t lo = 0; lo < p; ++lo)
            for (int32_t hi = lo + 1; hi < p; ++hi) {
                uint64_t key = win[(int64_t)lo * p + hi];
                if (key == UINT64_MAX) continue;
                int64_t r = (int64_t)(key >> 1);
                int32_t vi = (key & 1) ? hi : lo, vj = (key & 1) ? lo : hi;
                const int32_t *row = adj + (int64_t)vi * p;
                orc_unrank(row[0] - 1, level, r, pos);
                orc_resolve(row + 1, level, vj, pos, S);
                G[(int64_t)lo * p + hi] = 0;
                G[(int64_t)hi * p + lo] = 0;
                if (sepsets && level <= max_level) {
                    for (int k = 0; k < level; ++k) {
                        sepsets[((int64_t)lo * p + hi) * max_level + k] = S[k];
                        sepsets[((int64_t)hi * p + lo) * max_level + k] = S[k];
                    }
                }
                ++removed;
            }
        st->removed[level < 64 ? level : 63] = removed;
        st->levels_run = level + 1;
    }
    free(adj);
    free(win);
    return rc;
}
