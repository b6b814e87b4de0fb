// Level phases of the Gaussian skeleton (the level and unit kernels of gauss.cu).
//
// Work decomposition of a level (reference: gpucsl/pc/cuda/gaussian_ci.cu:66-120): one
// warp owns one undirected edge {lo, hi} alive at level start and walks the merged key
// sequence of both directions, key = (rank, dir) with dir 0 for v_i = lo, 32 keys per
// step (one test per lane).  The warp stops after the first step that contains a removing
// test; the lowest removing lane is the canonical remover (its set is the sepset) and z*
// folds the keys up to it.  An edge whose keys span more than one step and whose first
// step holds no remover is chunked: the unit phase walks its remaining steps in parallel,
// one warp per step, and the last unit to finish combines them in key order (HeavyEdge).
#pragma once

#include "gauss_dev.cuh"

namespace gcsl {

// FP32-first tests (MixedTest) read the FP32 copy of C and queue their FP64 z* candidates.
struct MixArgs {
    const float *C32;  // FP32 copy of C
    float t2lo, t2hi;  // FP32 bounds of the knife edge around tanh(tau)^2
    CandQueue q;
};

// Everything one level's phases read or write.
struct LevelCtx {
    const double *C;
    int p;
    const int *adj;
    const int2 *elist;
    double tau, t2;
    bool tau_valid;
    uint16_t *G;
    double *zmin, *r2min;  // per pair: exact Z minimum, rho^2 minimum of the monotone branch
    int *sep_dense;
    int max_level;
    int *rec_pool;
    long long rec_cap;
    DevState *st;
    MixArgs mix;
    ChunkBufs ck;  // ck.heavy == nullptr: every edge is walked whole
    unsigned long long order;  // work order of the debug build (0: list order)
};

// The level's test (FP32-first or FP64) over the keys of range rg of edge J.
template <int L, bool MIXED>
__device__ __forceinline__ void walk_level_keys(const EdgeJob &J, bool has, int lane, const LevelCtx &x,
                                                double &r2min, double &zmin_exact, bool &removed,
                                                unsigned long long &n_tests, const BinomRows *sb, double floor,
                                                WalkRange *rg) {
    if constexpr (MIXED) {
        walk_edge<L, 32>(J, has, x.adj, x.p, lane, 0u, 0xffffffffu,
                         MixedTest<L>{x.C, x.mix.C32, x.p, x.tau, x.t2, x.mix.t2lo, x.mix.t2hi}, x.G, x.sep_dense,
                         x.max_level, x.rec_pool, x.rec_cap, x.st, r2min, zmin_exact, removed, n_tests, &x.mix.q, sb,
                         floor, rg);
    } else {
        walk_edge<L, 32>(J, has, x.adj, x.p, lane, 0u, 0xffffffffu, F64Test<L>{x.C, x.p, x.tau, x.t2}, x.G,
                         x.sep_dense, x.max_level, x.rec_pool, x.rec_cap, x.st, r2min, zmin_exact, removed, n_tests,
                         nullptr, sb, 0.0, rg);
    }
}

// Edges with more keys than one step are chunked: a longer threshold leaves the 2 to 8
// step walks on the level's critical path, which costs more than the unit bookkeeping
// on graphs with long-tailed degrees.
constexpr long long CHUNK_MIN_KEYS = 32;

// Edge phase: warps w0, w0 + nw, ... take the level's edges in list order.  Statistics are
// added to the level's counters before returning.
template <int L, bool MIXED>
__device__ __forceinline__ void level_edge_phase(const LevelCtx &x, const BinomRows *sb, long long w0, long long nw) {
    DevState *st = x.st;
    const int p = x.p;
    const long long n_edges = (long long)__ldcg(&st->edges[L]);  // filled by the (re)compaction
    const int lane = threadIdx.x & 31;
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    unsigned long long n_tests = 0, n_full = 0, n_removed = 0;
    // Upper levels after a level that removed few edges: every edge's keys go to the unit
    // phase from key 0 and nothing is walked here, which takes one step off the level's
    // critical path (the first step's early exit, which the unit phase loses, rarely pays
    // when removals are rare).  The previous level's counts are final: its kernels
    // completed before this kernel's wait returned.
    const bool hand_over = x.ck.heavy != nullptr && L >= 3 &&
                           8ull * __ldcg(&st->removed[L - 1]) < __ldcg(&st->edges[L - 1]);
    for (long long e0 = w0; e0 < n_edges; e0 += nw) {
        const long long e = work_order(e0, n_edges, x.order);
        EdgeJob J;
        if (!load_edge_list<L>(x.adj, x.elist, p, e, L, J, st)) {
            if (lane == 0) set_status(st, GCSL_ERR_UNSUPPORTED);
            J.T = 0;
        }
        if (lane == 0) n_full += J.T;
        if (J.T == 0) continue;
        double r2min = inf, zmin_exact = inf;
        bool removed = false;
        // the pair's exact rho^2 minimum from earlier levels (level 0 stored r^2)
        const double floor = MIXED ? x.r2min[(size_t)J.lo * p + J.hi] : 0.0;
        if (hand_over && register_chunked<32>(J, lane, x.ck, st, L, inf, inf, floor, 0))
            continue;  // tests, minima and the removal come from the unit phase
        // an edge with more than one step of keys walks its first step here; without a
        // remover there, the unit phase walks the rest in parallel
        const bool chunk = x.ck.heavy != nullptr && J.T > CHUNK_MIN_KEYS;
        WalkRange rg{0, chunk ? 32ll : J.T, false, -1, J.T};
        walk_level_keys<L, MIXED>(J, true, lane, x, r2min, zmin_exact, removed, n_tests, sb, floor, &rg);
        bool deferred = false;
        if (chunk && !removed) {
            deferred = register_chunked<32>(J, lane, x.ck, st, L, r2min, zmin_exact, floor);
            if (!deferred) {  // buffers full: the rest of the keys here
                WalkRange rest{32, J.T, false, -1, J.T};
                walk_level_keys<L, MIXED>(J, true, lane, x, r2min, zmin_exact, removed, n_tests, sb, floor, &rest);
            }
        }
        if (lane == 0 && !deferred) {
            // z* candidates: exact Z into zmin, the monotone branch's min rho^2 into r2min
            // (converted to Z once per pair by the pmax kernel); atomic minima because the
            // candidate kernel of an earlier level may update the same pair concurrently
            const size_t ix = (size_t)J.lo * p + J.hi;
            if (zmin_exact < inf) atomic_min_nonneg_f64(x.zmin + ix, zmin_exact);
            if (r2min < inf) atomic_min_nonneg_f64(x.r2min + ix, r2min);
            n_removed += removed;
        }
    }
    if (lane == 0) {
        if (n_tests) atomicAdd(&st->tests[L], n_tests);
        if (n_full) atomicAdd(&st->tests_full[L], n_full);
        if (n_removed) atomicAdd(&st->removed[L], n_removed);
    }
}

// A chunked edge's record, read through L2 (other blocks wrote it in the same launch).
__device__ __forceinline__ HeavyEdge load_heavy(const HeavyEdge *e) {
    HeavyEdge H;
    H.lo = __ldcg(&e->lo);
    H.hi = __ldcg(&e->hi);
    H.T = __ldcg(&e->T);
    H.unit_base = __ldcg(&e->unit_base);
    H.n_units = __ldcg(&e->n_units);
    H.done = 0;
    H.r2_0 = __ldcg(&e->r2_0);
    H.ze_0 = __ldcg(&e->ze_0);
    H.floor = __ldcg(&e->floor);
    H.k0 = __ldcg(&e->k0);
    H.degs = __ldcg(&e->degs);
    return H;
}

// Unit phase: the keys of chunked edges (all of them for an edge handed over whole, else
// those after its first step), one unit (32 keys) per warp; an edge's only unit finishes
// the edge itself; otherwise the last unit of an edge to finish combines its units in
// key order: the smallest removing key is the canonical remover, and z* folds every unit
// that starts at or before it (up to the unit's own first remover) together with the
// first step.
template <int L, bool MIXED>
__device__ __forceinline__ void level_unit_phase(const LevelCtx &x, const BinomRows *sb, long long w0, long long nw) {
    DevState *st = x.st;
    const ChunkBufs &ck = x.ck;
    const int p = x.p;
    const long long reserved = (long long)__ldcg(&st->units[L]);
    const long long nu = reserved < ck.unit_cap ? reserved : ck.unit_cap;
    const int lane = threadIdx.x & 31;
    const double inf = __longlong_as_double(0x7ff0000000000000ll);
    unsigned long long n_extra = 0, n_removed = 0, unit_tests = 0;
    for (long long u0 = w0; u0 < nu; u0 += nw) {
        const long long u = work_order(u0, nu, x.order);
        const int h = __ldcg(ck.unit_h + u);
        if (h < 0) continue;
        const HeavyEdge H = load_heavy(ck.heavy + h);
        EdgeJob J;
        edge_job_from<L>(H.lo, H.hi, H.degs & 0xffff, H.degs >> 16, L, J);
        const long long m0 = H.k0 + (u - H.unit_base) * 32;
        const long long m1 = m0 + 32 < H.T ? m0 + 32 : H.T;
        // the edge's only unit (most edges handed over whole have at most 32 keys) walks
        // like an unchunked edge: its remover, found in key order, is final and is written
        // by the lane that found it, and its tests are the canonical count; nothing is
        // deferred to a combine
        const bool single = H.n_units == 1;
        WalkRange rg{m0, m1, !single, h, H.T};
        double r2 = inf, ze = inf;
        bool rem = false;
        unsigned long long own_tests = 0;
        // a unit that starts behind a remover already found cannot matter: the combine
        // neither folds it nor takes its remover
        if (m0 <= __ldcg(&ck.heavy[h].best))
            walk_level_keys<L, MIXED>(J, true, lane, x, r2, ze, rem, single ? own_tests : unit_tests, sb, H.floor,
                                      &rg);
        if (single) {
            if (lane == 0) {
                const size_t ix = (size_t)J.lo * p + J.hi;
                const double zc = min_nonneg(ze, H.ze_0), rc = min_nonneg(r2, H.r2_0);
                if (__double_as_longlong(zc) < __double_as_longlong(inf)) atomic_min_nonneg_f64(x.zmin + ix, zc);
                if (__double_as_longlong(rc) < __double_as_longlong(inf)) atomic_min_nonneg_f64(x.r2min + ix, rc);
                n_extra += own_tests;
                n_removed += rem;
            }
            continue;
        }
        long long R = H.T;
        double r2c = inf, zec = inf;
        {
            int d = 0;
            if (lane == 0) {
                if (rg.first < H.T) atomicMin(reinterpret_cast<unsigned long long *>(&ck.heavy[h].best),
                                              (unsigned long long)rg.first);
                ck.units[u] = UnitRes{rg.first, r2, ze};
                __threadfence();
                d = atomicAdd(&ck.heavy[h].done, 1);
            }
            d = __shfl_sync(GCSL_FULL_MASK, d, 0);
            if (d != H.n_units - 1) continue;
            // last unit of the edge: combine in key order
            __threadfence();
            for (int k = lane; k < H.n_units; k += 32) {
                const long long f = __ldcg(&ck.units[H.unit_base + k].first);
                R = f < R ? f : R;
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const long long y = __shfl_xor_sync(GCSL_FULL_MASK, R, o);
                R = y < R ? y : R;
            }
            for (int k = lane; k < H.n_units; k += 32) {
                if (H.k0 + (long long)k * 32 <= R) {  // the unit starts at or before the remover
                    r2c = fmin(r2c, __ldcg(&ck.units[H.unit_base + k].r2));
                    zec = fmin(zec, __ldcg(&ck.units[H.unit_base + k].ze));
                }
            }
            r2c = fmin(warp_min(r2c), H.r2_0);
            zec = fmin(warp_min(zec), H.ze_0);
        }
        if (lane == 0) {
            ck.chunk_first[h] = R;
            if (R < H.T) {
                long long rank;
                int dir;
                key_of(J, R, rank, dir);
                const int vi = dir ? J.hi : J.lo, vj = dir ? J.lo : J.hi;
                const int K = (dir ? J.deg_hi : J.deg_lo) - 1;
                int pos[L], S[L];
                unrank_positions<L>(K, rank, pos, sb);
                const int *nbrs = x.adj + (size_t)vi * p + 1;
#pragma unroll
                for (int c = 0; c < L; ++c) S[c] = resolve_position(nbrs, vj, pos[c]);
                write_removal(J, L, S, p, x.max_level, x.G, x.sep_dense, x.rec_pool, x.rec_cap, st);
                ++n_removed;
            }
            const size_t ix = (size_t)J.lo * p + J.hi;
            if (zec < inf) atomic_min_nonneg_f64(x.zmin + ix, zec);
            if (r2c < inf) atomic_min_nonneg_f64(x.r2min + ix, r2c);
            n_extra += (unsigned long long)((R < H.T ? R + 1 : H.T) - H.k0);
        }
    }
    if (lane == 0) {
        if (n_extra) atomicAdd(&st->tests[L], n_extra);
        if (n_removed) atomicAdd(&st->removed[L], n_removed);
    }
}

}  // namespace gcsl
