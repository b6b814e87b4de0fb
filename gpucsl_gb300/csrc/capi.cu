// extern "C" entry points of libgpucsl_gb300.so and the host side of the level loops.
//
// The level loop of the reference (discover_skeleton_gaussian.py:60-108,
// discover_skeleton_discrete.py:80-112) synchronises the host once per level to read
// the maximum degree.  Here every level kernel reads the termination test from the
// device state itself, so levels are enqueued back to back in growing batches and the
// host only checks the sticky `done` flag between batches; levels enqueued past the
// end return at their first instruction.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"

namespace gcsl {
namespace host {
cudaError_t launch_level0(const double *C, int p, double tau0, uint16_t *G, double *zmin, double *r2min, int *kept,
                          DevState *st, float *C32, cudaStream_t s);
cudaError_t launch_sf_table(double *out, cudaStream_t s);
cudaError_t launch_compact(const uint16_t *G, int p, int *adj, int *up, DevState *st, int level, int2 *elist,
                           cudaStream_t s);
cudaError_t launch_scan_int(const int *cnt, int p, long long *prefix, DevState *st, cudaStream_t s);
cudaError_t launch_recompact(const uint16_t *G, int p, int *adj, int *up, DevState *st, int level, int2 *elist,
                             cudaStream_t s);
cudaError_t launch_scan_ll(const long long *cnt, int p, long long *prefix, DevState *st, cudaStream_t s);
cudaError_t launch_gauss_level(int L, const double *C, int p, const int *adj, const int *up, const int2 *elist,
                               const long long *prefix, double tau, bool tau_valid, uint16_t *G, double *zmin,
                               double *r2min, int *sep_dense, int max_level, int *rec_pool, long long rec_cap,
                               DevState *st, int num_sms, const float *C32, int *qbuf, long long qcap,
                               const ChunkBufs &ck, cudaStream_t s);

size_t orient_workspace_bytes(int p);
cudaError_t encode_columns(const void *X, int dtype, long long n, int p, long long ld, uint8_t *codes, long long ldc,
                           uint8_t *dims, void *workspace, cudaStream_t s);
size_t encode_workspace_bytes(int p);
cudaError_t orient_edges(const uint16_t *S, int p, const int *sep, int L, uint8_t *D, void *ws, int num_sms,
                         int *host_word, int *passes, cudaStream_t s);
cudaError_t launch_cand(int L, const double *C, int p, double tau, double *zmin, double *r2min, const int *qbuf,
                        long long qcap, DevState *st, const long long *chunk_first, int num_sms, cudaStream_t s);
cudaError_t launch_pmax(const int *kept, const DevState *st, const double *zmin, const double *r2min, int p,
                        long long n_obs, const double *sftab, double *pmax, int num_sms,
                        cudaStream_t s);
cudaError_t launch_pmax_level0(const double *C, const double *zmin, int p, long long n_obs, const double *sftab,
                               double *pmax,
                               int num_sms, cudaStream_t s);
size_t corr_workspace_bytes(long long n, int p);
cudaError_t corr_f64(const void *X, int dtype, long long n, int p, long long ldx, double *C, void *ws,
                     size_t ws_bytes, int num_sms, cudaStream_t s);
int disc_table_cap(int device);
void disc_level_caps(int cap_full, int max_dim, int L, int &table_cap, int &part_cap);
cudaError_t launch_disc_tests(const DiscLevelArgs &A, int num_sms, cudaStream_t s);
cudaError_t launch_disc_validate(const uint8_t *data, long long ld, long long n, int p, const uint8_t *dims,
                                 DevState *st, int num_sms, cudaStream_t s);
cudaError_t launch_disc_weights(const int *adj, int p, int L, long long *w, DevState *st, cudaStream_t s);
cudaError_t launch_disc_finalize(const int *adj, int p, int L, uint16_t *G, unsigned long long *win, int *sep,
                                 int max_level, int *rec, long long rec_cap, DevState *st, int num_sms,
                                 cudaStream_t s);
cudaError_t launch_disc_level_stats(const long long *prefix, const int *adj, int p, int L, DevState *st,
                                    cudaStream_t s);
cudaError_t launch_pmax_finish(double *pmax, int p, int num_sms, cudaStream_t s);
cudaError_t launch_disc_table(const uint8_t *data, long long ld, long long n, const uint8_t *dims, int vi, int vj,
                              const int *S, int L, int table_cap, uint32_t *counts, long long counts_cap, double *out2,
                              cudaStream_t s);
cudaError_t launch_pchisq(const double *x, const long long *df, long long count, double *out, cudaStream_t s);
cudaError_t launch_unrank(int K, int L, long long count, int *out, cudaStream_t s);
size_t corr_tc_workspace_bytes(long long n, int p, int num_sms);
cudaError_t corr_tc(const void *X, int dtype, long long n, int p, long long ldx, double *C, void *ws, size_t ws_bytes,
                    int num_sms, int *err_out_dev_or_null, cudaStream_t s);
cudaError_t corr_tc_digits(const void *X, int dtype, long long n, int p, long long ldx, void *ws, size_t ws_bytes,
                           int num_sms, cudaStream_t s);
cudaError_t corr_tc_product(long long n, int p, double *C, void *ws, size_t ws_bytes, int num_sms, cudaStream_t s);
size_t corr_tc_batch_workspace_bytes(const long long *n, const int *p, int count);
cudaError_t corr_tc_batch_prepare(const void *const *X, const long long *n, const int *p, const long long *ldx,
                                  double *const *C, float *const *C32, int count, void *ws, size_t ws_bytes,
                                  long long *stage_totals, cudaStream_t s);
cudaError_t corr_tc_batch_run(void *ws, int count, const long long *stage_totals, int dtype, cudaStream_t s);
size_t gauss_batch_workspace_bytes(const int *p, int count);
int gauss_batch_prepare(const gcsl_gauss_instance *in, int count, int max_level, int precision, void *ws,
                        size_t ws_bytes, long long *plan, int sms, cudaStream_t s);
int gauss_batch_set_lanes(long long *plan, int level, int lanes);
int gauss_batch_run(const long long *plan, cudaStream_t s, bool rerun);
int gauss_batch_step(const long long *plan, int first, int last, bool finish, bool rerun, int32_t *host_status,
                     cudaStream_t s);
int gauss_batch_prepare_staged(const gcsl_gauss_instance *in, int count, int max_level, int precision, void *ws,
                               size_t ws_bytes, void *stage, size_t stage_bytes, long long *plan, int sms,
                               cudaStream_t s);
size_t gauss_state_bytes(int p);
size_t gauss_batch_table_bytes(int count);
const int *gauss_batch_flags(const long long *plan);
cudaError_t corr_tc_batch_run_mode(void *ws, int count, const long long *stage_totals, int dtype, int mode,
                                   double *c_err, const int *active, cudaStream_t s);
int gauss_batch_collect(const long long *plan, gcsl_gauss_instance *out, int count, cudaStream_t s);
cudaError_t launch_tc_gemm_bf16(const uint16_t *A, const uint16_t *B, float *D, int M, int N, int K, int *err,
                                cudaStream_t s);
}  // namespace host
}  // namespace gcsl

using namespace gcsl;

#include <atomic>
static std::atomic<long long> g_kernel_launches{0};
void gcsl::host::note_launch(int kernels) { g_kernel_launches.fetch_add(kernels, std::memory_order_relaxed); }

static thread_local char g_last_error[256] = "";
cudaError_t gcsl::host::note_error(const char *where, cudaError_t e) {
    if (e != cudaSuccess)
        std::snprintf(g_last_error, sizeof(g_last_error), "%s: %s (%s)", where, cudaGetErrorName(e),
                      cudaGetErrorString(e));
    return e;
}

namespace {

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

struct Carver {
    char *base;
    size_t off = 0, cap;
    Carver(void *b, size_t c) : base(static_cast<char *>(b)), cap(c) {}
    template <typename T>
    T *take(size_t count) {
        T *p = reinterpret_cast<T *>(base ? base + off : nullptr);
        off = align_up(off + count * sizeof(T));
        return p;
    }
};

int device_sms() {
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

int map_cuda(cudaError_t e) {
    if (e != cudaSuccess && g_last_error[0] == '\0') host::note_error("CUDA call", e);
    return e == cudaSuccess ? GCSL_OK : GCSL_ERR_DEVICE;
}

// A second, lowest-priority stream per device for work that can overlap the level loop
// (its blocks yield SMs to the latency-bound level kernels); created once per device,
// never allocates device memory.
struct SideStream {
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaEvent_t level[GCSL_GAUSS_REG_LEVELS + 1] = {};  // level l's tests done (candidate hand-off)
};

// Per-level device timing (gcsl_stats.level_ms) when GCSL_LEVEL_TIMING=1: one event per
// level boundary on the solve's stream, from a pool created once per device.
struct LevelTimer {
    cudaEvent_t ev[GCSL_MAX_LEVELS + 2] = {};
    bool ok = false;
};

// The timers, the side stream and the pinned control words below exist once per host
// thread and device: solves issued concurrently from several threads (on their own
// streams) never share an event, a stream or a control word.
LevelTimer *level_timer() {
    static const bool enabled = [] {
        const char *e = getenv("GCSL_LEVEL_TIMING");
        return e && e[0] == '1';
    }();
    if (!enabled) return nullptr;
    static thread_local LevelTimer timers[64];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return nullptr;
    LevelTimer &t = timers[dev];
    if (!t.ok) {
        for (auto &e : t.ev)
            if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        t.ok = true;
    }
    return &t;
}

SideStream *side_stream() {
    static thread_local SideStream streams[64];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return nullptr;
    SideStream &s = streams[dev];
    if (!s.stream) {
        int lo = 0, hi = 0;  // numerically larger = lower priority
        if (cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess) lo = 0;
        if (cudaStreamCreateWithPriority(&s.stream, cudaStreamNonBlocking, lo) != cudaSuccess) return nullptr;
        if (cudaEventCreateWithFlags(&s.fork, cudaEventDisableTiming) != cudaSuccess) return nullptr;
        if (cudaEventCreateWithFlags(&s.join, cudaEventDisableTiming) != cudaSuccess) return nullptr;
        for (cudaEvent_t &e : s.level)
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return nullptr;
    }
    return &s;
}

// Level batches replayed from CUDA graphs.  A solve enqueues its levels in batches
// (level 1, then up to 8 levels per host read of the termination state); each batch
// costs about four launches per level, which on the upper levels (little work each) is
// more host time than device time.  When the same batch recurs -- the same workspace,
// matrix, outputs, thresholds and level range, as in repeated solves of one solver --
// it is captured once into a CUDA graph (its side-stream candidate kernels joined back
// at the end of the batch) and replayed by one launch.  A batch seen once, the level
// timers and the allocation-free path launch directly; so does everything unless
// GCSL_LEVEL_GRAPHS=1 (see graphs_off).
struct LevelGraphKey {
    const void *ws;
    const double *C;
    const void *G, *sep, *rec;
    long long rec_cap;
    int p, max_level, a, b, n_thr, mixed, chunked, sms;
    unsigned long long thr_hash;
};

struct LevelGraph {
    LevelGraphKey key;
    cudaGraphExec_t exec = nullptr;
    bool failed = false;  // capture not possible: always launch directly
    long long kernels = 0;
};

struct LevelGraphCache {
    static constexpr int kEntries = 16;
    LevelGraph e[kEntries];
    int used = 0, next = 0;
    cudaStream_t cap = nullptr;   // private stream the batches are captured on
    cudaEvent_t cap_join = nullptr;
};

LevelGraphCache *level_graph_cache() {
    static thread_local LevelGraphCache caches[64];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return nullptr;
    LevelGraphCache &c = caches[dev];
    if (!c.cap) {
        if (cudaStreamCreateWithFlags(&c.cap, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
        if (cudaEventCreateWithFlags(&c.cap_join, cudaEventDisableTiming) != cudaSuccess) return nullptr;
    }
    return &c;
}

// Level-batch graphs are used with GCSL_LEVEL_GRAPHS=1 (measured on the p = 1000,
// n = 10000 solve: the replayed batches were no faster than the programmatic-dependent
// launches, whose prologues overlap the previous kernel).
bool graphs_off() {
    static const bool off = [] {
        const char *e = getenv("GCSL_LEVEL_GRAPHS");
        return !(e && e[0] == '1');
    }();
    return off;
}

// Launches levels key.a..key.b on s: from the cached graph when the batch recurs (captured
// on its second occurrence), else directly.  enqueue_on(level, stream) enqueues a level;
// side is the solve's side stream, joined back into the capture before it ends.
template <typename EnqueueOn>
cudaError_t launch_level_batch(const LevelGraphKey &key, cudaStream_t s, cudaStream_t side, EnqueueOn enqueue_on) {
    auto direct = [&]() -> cudaError_t {
        for (int l = key.a; l <= key.b; ++l) {
            const cudaError_t e = enqueue_on(l, s);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    };
    LevelGraphCache *c = graphs_off() ? nullptr : level_graph_cache();
    if (!c) return direct();
    LevelGraph *g = nullptr;
    for (int i = 0; i < c->used; ++i)
        if (std::memcmp(&c->e[i].key, &key, sizeof(key)) == 0) g = &c->e[i];
    if (!g) {  // first occurrence: remember it, launch directly
        LevelGraph &slot = c->e[c->used < LevelGraphCache::kEntries ? c->used++ : c->next];
        if (c->used == LevelGraphCache::kEntries) c->next = (c->next + 1) % LevelGraphCache::kEntries;
        if (slot.exec) cudaGraphExecDestroy(slot.exec);
        slot = LevelGraph{};
        slot.key = key;
        return direct();
    }
    if (g->failed) return direct();
    if (!g->exec) {
        const long long k0 = g_kernel_launches.load(std::memory_order_relaxed);
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(c->cap, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            for (int l = key.a; l <= key.b && e == cudaSuccess; ++l) e = enqueue_on(l, c->cap);
            if (e == cudaSuccess && side) {
                e = cudaEventRecord(c->cap_join, side);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(c->cap, c->cap_join, 0);
            }
            const cudaError_t ee = cudaStreamEndCapture(c->cap, &graph);
            if (e == cudaSuccess) e = ee;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            cudaGetLastError();  // capture errors are not sticky: clear and launch directly from now on
            g->exec = nullptr;
            g->failed = true;
            g_last_error[0] = '\0';
            return direct();
        }
        g->kernels = g_kernel_launches.load(std::memory_order_relaxed) - k0;
        g_kernel_launches.fetch_sub(g->kernels, std::memory_order_relaxed);  // counted when replayed
    }
    const cudaError_t e = cudaGraphLaunch(g->exec, s);
    if (e == cudaSuccess) host::note_launch((int)g->kernels);
    return host::note_error("level batch graph launch", e);
}

unsigned long long fnv1a(const void *data, size_t bytes) {
    const unsigned char *b = static_cast<const unsigned char *>(data);
    unsigned long long h = 1469598103934665603ull;
    for (size_t i = 0; i < bytes; ++i) h = (h ^ b[i]) * 1099511628211ull;
    return h;
}

// Joins the side stream back into the solve's stream on every return after the fork,
// so no side-stream work of a failed call outlives the call unordered with the stream.
struct SideJoin {
    SideStream *ss;
    cudaStream_t s;
    bool armed = false;
    cudaError_t join() {
        if (!armed) return cudaSuccess;
        armed = false;
        cudaError_t e = cudaEventRecord(ss->join, ss->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ss->join, 0);
        return e;
    }
    ~SideJoin() { join(); }
};

// Copy the device state into the public stats struct.
int finish_stats(const DevState *d_st, gcsl_stats *stats, cudaStream_t s, bool discrete_edges, long long p) {
    DevState h;
    cudaError_t e = cudaMemcpyAsync(&h, d_st, sizeof(DevState), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return GCSL_ERR_DEVICE;
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->levels_run = h.last_level + 1;
        stats->status = h.status;
        stats->debug_site = h.debug_site;
        stats->n_records = (int64_t)h.n_rec_ints;
        for (int l = 0; l < GCSL_MAX_LEVELS; ++l) {
            stats->edges[l] = (int64_t)(discrete_edges ? h.edges[l] / 2 : h.edges[l]);
            stats->tests[l] = (int64_t)h.tests[l];
            stats->tests_full[l] = (int64_t)h.tests_full[l];
            stats->removed[l] = (int64_t)h.removed[l];
            stats->max_degree[l] = h.max_degree[l];
        }
        const long long pairs = p * (p - 1) / 2;
        stats->edges[0] = pairs;
        stats->tests[0] = pairs;
        stats->tests_full[0] = pairs;
    }
    return h.status;
}

// Pinned host words per device for the level loop's control reads (a pageable copy
// costs a staging round trip).
struct HostCtl {
    int32_t *words = nullptr;  // [0] done, [1] max degree of the last level
};

HostCtl *host_ctl() {
    static thread_local HostCtl ctl[64];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return nullptr;
    HostCtl &c = ctl[dev];
    if (!c.words && cudaMallocHost(reinterpret_cast<void **>(&c.words), 2 * sizeof(int32_t)) != cudaSuccess)
        return nullptr;
    return &c;
}

// Run levels 1..max_level with the given per-level enqueue function.  Every level
// kernel reads the termination state on the device, so levels are enqueued in batches:
// level 1 alone, then up to 8 levels per host read of two pinned words (done flag, the
// last level's maximum degree d).  Degrees only shrink, so level l can only run while
// d - 1 >= l: a batch never extends past min(d - 1, ...) of the last read.
// `words` are two host words for the control reads: the calling thread's pinned words,
// or (allocation-free path) words on the caller's stack, read by a synchronous copy.
// enqueue_range(a, b) enqueues levels a..b on `s`.
template <typename EnqueueRange>
int run_levels(int max_level, DevState *d_st, cudaStream_t s, int32_t *words, EnqueueRange enqueue_range) {
    int level = 1;
    int bound = std::min(max_level, GCSL_MAX_LEVELS - 1);  // highest level that may still run
    int batch = 1;
    while (level <= bound) {
        const int last = std::min(bound, level + batch - 1);
        if (enqueue_range(level, last) != cudaSuccess) return GCSL_ERR_DEVICE;
        level = last + 1;
        if (level > bound) break;
        cudaError_t e = cudaMemcpyAsync(&words[0], &d_st->done, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&words[1], &d_st->max_degree[last], sizeof(int32_t), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return GCSL_ERR_DEVICE;
        if (words[0]) break;
        bound = std::min(bound, words[1] - 1);
        // after the first level, up to 8 levels per host read (a level enqueued past the end
        // costs four early-exit launches, about as much as a host read)
        batch = 8;
    }
    if (max_level >= GCSL_MAX_LEVELS && bound >= GCSL_MAX_LEVELS - 1) {
        // levels beyond the state arrays: only an error if the loop had not finished
        if (cudaMemcpyAsync(&words[0], &d_st->done, sizeof(int32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return GCSL_ERR_DEVICE;
        if (!words[0]) return GCSL_ERR_UNSUPPORTED_LEVEL;
    }
    return GCSL_OK;
}

struct GaussWs {
    DevState *st;
    int *adj, *up;
    long long *prefix;
    double *zmin, *r2min;
    int *kept;
    int2 *elist;      // the level's edges (lo, hi)
    float *c32;       // FP32 copy of C for the FP32-first tests
    double *sftab;    // erfc Taylor table of the pmax kernels
    int *cand;        // FP64 z* candidate queue
    long long cand_cap;
    ChunkBufs ck;     // chunked edges of the current level (chunk_first: one region per level)
    size_t bytes;
};

// Ints of the z* candidate queue: entries hold 5 + level ints, about one or two per edge
// and level; a full queue only moves evaluations back into the level kernel.
long long cand_queue_ints(int p) { return std::max<long long>(1ll << 20, 4ll * p * p); }

// The queue holds one region per register level (1 .. GCSL_GAUSS_REG_LEVELS), so a
// level's candidates can still be waiting on the side stream while the next levels append.
long long cand_region_ints(long long cap) { return cap / GCSL_GAUSS_REG_LEVELS; }

// Chunked edges per level and their units of 32 keys; a level that needs more walks the
// excess edges whole in the level kernel.
long long chunk_edges_cap(int p) { return std::max<long long>(1ll << 14, 16ll * p); }
long long chunk_units_cap(int p) { return std::max<long long>(1ll << 16, 64ll * p); }

// FP32-first level tests (default) or FP64 throughout (GCSL_F64_TESTS=1, for comparisons).
// Precision of the plain path's level tests for the calling thread: 0 = the process
// default (FP32 first; GCSL_F64_TESTS=1 makes it FP64 throughout), 1 = FP32 first,
// 2 = FP64 throughout.
static thread_local int g_test_precision = 0;

// Work-order seed of the calling thread's solves (debug build; see gcsl_debug_set_work_order).
static thread_local unsigned long long g_work_order = 0;

// Cap on the resident blocks per SM of the discrete test kernel launched by this thread.
static thread_local int g_blocks_cap = 0;

bool mixed_tests() {
    static const bool mixed = [] {
        const char *e = getenv("GCSL_F64_TESTS");
        return !(e && e[0] == '1');
    }();
    return g_test_precision == 0 ? mixed : g_test_precision == 1;
}

// GCSL_CHUNKED=0 walks every edge whole in the level kernel (for comparisons).
bool chunking_off() {
    static const bool off = [] {
        const char *e = getenv("GCSL_CHUNKED");
        return e && e[0] == '0';
    }();
    return off;
}

GaussWs carve_gauss(void *ws, size_t cap, int p) {
    Carver c(ws, cap);
    GaussWs w;
    w.st = c.take<DevState>(1);
    w.adj = c.take<int>((size_t)p * p);
    w.up = c.take<int>((size_t)p);
    w.prefix = c.take<long long>((size_t)p + 1);
    w.zmin = c.take<double>((size_t)p * p);
    w.r2min = c.take<double>((size_t)p * p);
    w.kept = c.take<int>((size_t)p * (p - 1) / 2 + 1);
    w.elist = c.take<int2>((size_t)p * (p - 1) / 2 + 1);
    w.c32 = c.take<float>((size_t)p * p);
    w.sftab = c.take<double>(32 * 13);
    w.cand_cap = cand_queue_ints(p);
    w.cand = c.take<int>((size_t)w.cand_cap);
    w.ck.heavy_cap = chunk_edges_cap(p);
    w.ck.unit_cap = chunk_units_cap(p);
    w.ck.heavy = c.take<HeavyEdge>((size_t)w.ck.heavy_cap);
    w.ck.chunk_first = c.take<long long>((size_t)w.ck.heavy_cap * GCSL_GAUSS_REG_LEVELS);
    w.ck.unit_h = c.take<int>((size_t)w.ck.unit_cap);
    w.ck.units = c.take<UnitRes>((size_t)w.ck.unit_cap);
    w.bytes = c.off;
    return w;
}

struct DiscWs {
    DevState *st;
    int *adj;
    long long *weights, *prefix;
    unsigned long long *win;
    size_t bytes;
};

DiscWs carve_disc(void *ws, size_t cap, int p) {
    Carver c(ws, cap);
    DiscWs w;
    w.st = c.take<DevState>(1);
    w.adj = c.take<int>((size_t)p * p);
    w.weights = c.take<long long>((size_t)p);
    w.prefix = c.take<long long>((size_t)p + 1);
    w.win = c.take<unsigned long long>((size_t)p * p);
    w.bytes = c.off;
    return w;
}

}  // namespace

unsigned long long gcsl::host::work_order_seed() { return GCSL_DEBUG_CHECKS ? g_work_order : 0ull; }

int gcsl::host::blocks_per_sm_cap() { return g_blocks_cap; }

int gcsl::host::gauss_skeleton_run(const double *C, int p, long long n_obs, const double *thresholds,
                                   int n_thresholds, int max_level, uint16_t *G, int *sepsets, int *rec_pool,
                                   long long rec_cap, double *pmax, gcsl_stats *stats, void *workspace,
                                   size_t workspace_bytes, void *stream, bool allocation_free) {
    if (!C || !G || !pmax || p < 1 || n_obs < 4 || !thresholds || n_thresholds < 1 || max_level < 0)
        return GCSL_ERR_INVALID_ARG;
    if (p > GCSL_GAUSS_MAX_P) return GCSL_ERR_UNSUPPORTED;
    if (rec_pool == nullptr) rec_cap = 0;
    GaussWs w = carve_gauss(workspace, workspace_bytes, p);
    if (!workspace || w.bytes > workspace_bytes) return GCSL_ERR_WORKSPACE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int sms = device_sms();
    if (cudaMemsetAsync(w.st, 0, sizeof(DevState), s) != cudaSuccess) return GCSL_ERR_DEVICE;
    // r2min starts at 0x7f7f... = 1.4e306, above every rho^2 < 1 the levels can store
    if (cudaMemsetAsync(w.r2min, 0x7f, sizeof(double) * (size_t)p * p, s) != cudaSuccess) return GCSL_ERR_DEVICE;
    LevelTimer *lt = stats && !allocation_free ? level_timer() : nullptr;
    int n_timed = 0;  // events recorded: ev[0 .. n_timed]
    if (lt) cudaEventRecord(lt->ev[0], s);
    const bool mixed = mixed_tests() && max_level >= 1;
    if (host::launch_level0(C, p, thresholds[0], G, w.zmin, w.r2min, w.kept, w.st, mixed ? w.c32 : nullptr, s) !=
        cudaSuccess)
        return GCSL_ERR_DEVICE;
    if (lt) {
        cudaEventRecord(lt->ev[1], s);
        n_timed = 1;
    }
    // pmax of the pairs removed at level 0 overlaps the level loop on the side stream (the
    // allocation-free path has none: that work goes on `s` in order)
    SideStream *ss = nullptr;
    int32_t stack_words[2] = {0, 0};
    int32_t *words = stack_words;
    if (!allocation_free) {
        ss = side_stream();
        HostCtl *hc = host_ctl();
        if (!ss || !hc) return GCSL_ERR_DEVICE;
        words = hc->words;
    }
    SideJoin joiner{ss, s};
    if (ss) {
        if (cudaEventRecord(ss->fork, s) != cudaSuccess || cudaStreamWaitEvent(ss->stream, ss->fork, 0) != cudaSuccess)
            return GCSL_ERR_DEVICE;
        joiner.armed = true;  // from here every return joins the side stream back into s
    }
    cudaStream_t aux = ss ? ss->stream : s;
    if (host::launch_sf_table(w.sftab, aux) != cudaSuccess ||
        host::launch_pmax_level0(C, w.zmin, p, n_obs, w.sftab, pmax, sms, aux) != cudaSuccess)
        return GCSL_ERR_DEVICE;
    const long long region = cand_region_ints(w.cand_cap);
    auto enqueue_on = [&](int level, cudaStream_t s) -> cudaError_t {
        // level 1 compacts the full matrix; later levels only shrink the previous lists;
        // (re)compaction writes the level's edge list; the row prefix is only needed by
        // the shared-memory kernel of levels above GCSL_GAUSS_REG_LEVELS
        cudaError_t e = level == 1 ? host::launch_compact(G, p, w.adj, w.up, w.st, level, w.elist, s)
                                   : host::launch_recompact(G, p, w.adj, w.up, w.st, level, w.elist, s);
        if (e == cudaSuccess && level > GCSL_GAUSS_REG_LEVELS) e = host::launch_scan_int(w.up, p, w.prefix, w.st, s);
        const bool tau_valid = level < n_thresholds;
        const double tau = tau_valid ? thresholds[level] : 0.0;
        const bool cand = mixed && level <= GCSL_GAUSS_REG_LEVELS;
        int *qbuf = cand ? w.cand + (size_t)(level - 1) * region : nullptr;
        // level 1 walks its edges whole: its edges are many and short, so the level kernel
        // alone keeps every SM busy
        ChunkBufs ck = w.ck;
        if (level >= 2 && level <= GCSL_GAUSS_REG_LEVELS) ck.chunk_first += (size_t)(level - 1) * ck.heavy_cap;
        else ck.heavy = nullptr;
        if (chunking_off()) ck.heavy = nullptr;
        if (e == cudaSuccess)
            e = host::launch_gauss_level(level, C, p, w.adj, w.up, w.elist, w.prefix, tau, tau_valid, G, w.zmin,
                                         w.r2min, sepsets, max_level, rec_pool, rec_cap, w.st, sms,
                                         mixed ? w.c32 : nullptr, qbuf, region, ck, s);
        // the level's FP64 z* candidates only feed pmax: they run on the low-priority side
        // stream while the next levels proceed
        if (e == cudaSuccess && cand) {
            if (ss) {
                e = cudaEventRecord(ss->level[level], s);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(ss->stream, ss->level[level], 0);
            }
            if (e == cudaSuccess)
                e = host::launch_cand(level, C, p, tau, w.zmin, w.r2min, qbuf, region, w.st,
                                      ck.heavy != nullptr ? ck.chunk_first : nullptr, sms, aux);
        }
        if (lt && level + 1 < GCSL_MAX_LEVELS + 2) {
            cudaEventRecord(lt->ev[level + 1], s);
            n_timed = level + 1;
        }
        return e;
    };
    auto enqueue_range = [&](int a, int b) -> cudaError_t {
        if (lt || allocation_free) {  // timed levels or nothing to create: direct launches
            for (int l = a; l <= b; ++l) {
                const cudaError_t e = enqueue_on(l, s);
                if (e != cudaSuccess) return e;
            }
            return cudaSuccess;
        }
        LevelGraphKey key;
        std::memset(&key, 0, sizeof(key));
        key.ws = workspace;
        key.C = C;
        key.G = G;
        key.sep = sepsets;
        key.rec = rec_pool;
        key.rec_cap = rec_cap;
        key.p = p;
        key.max_level = max_level;
        key.a = a;
        key.b = b;
        key.n_thr = n_thresholds;
        key.mixed = mixed;
        key.chunked = !chunking_off();
        key.sms = sms;
        const int t_end = std::min(b + 1, n_thresholds);
        key.thr_hash = a < t_end ? fnv1a(thresholds + a, sizeof(double) * (size_t)(t_end - a)) : 0ull;
        return launch_level_batch(key, s, ss ? ss->stream : nullptr, enqueue_on);
    };
    const int rc = run_levels(max_level, w.st, s, words, enqueue_range);
    if (joiner.join() != cudaSuccess) return GCSL_ERR_DEVICE;
    if (rc != GCSL_OK) return rc;
    if (host::launch_pmax(w.kept, w.st, w.zmin, w.r2min, p, n_obs, w.sftab, pmax, sms, s) != cudaSuccess)
        return GCSL_ERR_DEVICE;
    const int frc = finish_stats(w.st, stats, s, false, p);
    if (lt) {
        // level l spans events l .. l+1 (level 0 includes the state reset); levels that
        // were enqueued but found the loop finished are reported as well
        for (int l = 0; l < n_timed && l < GCSL_MAX_LEVELS; ++l) {
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, lt->ev[l], lt->ev[l + 1]) == cudaSuccess) stats->level_ms[l] = ms;
        }
        cudaGetLastError();  // a failed timing query must not surface in a later launch check
    }
    return frc;
}

extern "C" {

int gcsl_version(void) { return GCSL_ABI_VERSION; }

int64_t gcsl_kernel_launches(void) { return (int64_t)g_kernel_launches.load(std::memory_order_relaxed); }

const char *gcsl_last_error(void) { return g_last_error; }

int gcsl_debug_set_work_order(uint64_t seed) {
#if GCSL_DEBUG_CHECKS
    g_work_order = (unsigned long long)seed;
    return GCSL_OK;
#else
    (void)seed;
    return GCSL_ERR_UNSUPPORTED;
#endif
}

int gcsl_set_blocks_per_sm_cap(int32_t cap) {
    if (cap < 0) return GCSL_ERR_INVALID_ARG;
    g_blocks_cap = cap;
    return GCSL_OK;
}

int gcsl_set_test_precision(int32_t mode) {
    if (mode < 0 || mode > 2) return GCSL_ERR_INVALID_ARG;
    g_test_precision = mode;
    return GCSL_OK;
}

const char *gcsl_status_string(int status) {
    switch (status) {
    case GCSL_OK: return "ok";
    case GCSL_ERR_INVALID_ARG: return "invalid argument";
    case GCSL_ERR_WORKSPACE: return "workspace too small";
    case GCSL_ERR_UNSUPPORTED_LEVEL: return "level beyond the supported range (no threshold or state slot)";
    case GCSL_ERR_TIMEOUT: return "device wait timed out";
    case GCSL_ERR_DEVICE: return "CUDA error";
    case GCSL_ERR_CAPACITY: return "sepset record pool too small";
    case GCSL_ERR_UNSUPPORTED: return "unsupported problem size";
    case GCSL_ERR_DEBUG_CHECK: return "a bounds check of the debug build failed (gcsl_stats.debug_site)";
    default: return "unknown status";
    }
}

size_t gcsl_corr_workspace_bytes(int64_t n, int32_t p) { return host::corr_workspace_bytes(n, p); }

int gcsl_corr_f64(const void *X, int32_t dtype, int64_t n, int32_t p, int64_t ldx, double *C, void *workspace,
                  size_t workspace_bytes, void *stream) {
    if (!X || !C || n < 2 || p < 1 || ldx < p || (dtype != GCSL_DTYPE_F64 && dtype != GCSL_DTYPE_F32))
        return GCSL_ERR_INVALID_ARG;
    if (!workspace || workspace_bytes < host::corr_workspace_bytes(n, p)) return GCSL_ERR_WORKSPACE;
    return map_cuda(host::corr_f64(X, dtype, n, p, ldx, C, workspace, workspace_bytes, device_sms(),
                                   static_cast<cudaStream_t>(stream)));
}

size_t gcsl_corr_tc_workspace_bytes(int64_t n, int32_t p) {
    if (n < 1 || p < 1) return 0;
    return host::corr_tc_workspace_bytes(n, p, device_sms());
}

int gcsl_corr_f64_tc(const void *X, int32_t dtype, int64_t n, int32_t p, int64_t ldx, double *C, void *workspace,
                     size_t workspace_bytes, void *stream) {
    if (!X || !C || n < 2 || p < 1 || ldx < p || (dtype != GCSL_DTYPE_F64 && dtype != GCSL_DTYPE_F32))
        return GCSL_ERR_INVALID_ARG;
    const int sms = device_sms();
    if (!workspace || workspace_bytes < host::corr_tc_workspace_bytes(n, p, sms)) return GCSL_ERR_WORKSPACE;
    return map_cuda(host::corr_tc(X, dtype, n, p, ldx, C, workspace, workspace_bytes, sms, nullptr,
                                  static_cast<cudaStream_t>(stream)));
}

int gcsl_corr_tc_digits(const void *X, int32_t dtype, int64_t n, int32_t p, int64_t ldx, void *workspace,
                        size_t workspace_bytes, void *stream) {
    if (!X || n < 2 || p < 1 || ldx < p || (dtype != GCSL_DTYPE_F64 && dtype != GCSL_DTYPE_F32))
        return GCSL_ERR_INVALID_ARG;
    const int sms = device_sms();
    if (!workspace || workspace_bytes < host::corr_tc_workspace_bytes(n, p, sms)) return GCSL_ERR_WORKSPACE;
    return map_cuda(host::corr_tc_digits(X, dtype, n, p, ldx, workspace, workspace_bytes, sms,
                                         static_cast<cudaStream_t>(stream)));
}

int gcsl_corr_tc_product(int64_t n, int32_t p, double *C, void *workspace, size_t workspace_bytes, void *stream) {
    if (!C || n < 2 || p < 1) return GCSL_ERR_INVALID_ARG;
    const int sms = device_sms();
    if (!workspace || workspace_bytes < host::corr_tc_workspace_bytes(n, p, sms)) return GCSL_ERR_WORKSPACE;
    return map_cuda(host::corr_tc_product(n, p, C, workspace, workspace_bytes, sms, static_cast<cudaStream_t>(stream)));
}

size_t gcsl_gauss_workspace_bytes(int32_t p, int32_t max_level) {
    (void)max_level;
    return carve_gauss(nullptr, 0, p).bytes;
}

int gcsl_gauss_skeleton(const double *C, int32_t p, int64_t n_obs, const double *thresholds, int32_t n_thresholds,
                        int32_t max_level, uint16_t *G, int32_t *sepsets, int32_t *rec_pool, int64_t rec_cap,
                        double *pmax, gcsl_stats *stats, void *workspace, size_t workspace_bytes, void *stream) {
    return host::gauss_skeleton_run(C, p, n_obs, thresholds, n_thresholds, max_level, G, sepsets, rec_pool, rec_cap,
                                    pmax, stats, workspace, workspace_bytes, stream, false);
}

size_t gcsl_disc_workspace_bytes(int32_t p, int64_t n, int32_t max_level, int32_t max_dim) {
    (void)n;
    (void)max_level;
    (void)max_dim;
    return carve_disc(nullptr, 0, p).bytes;
}

int gcsl_disc_skeleton(const uint8_t *data, int64_t ld, int64_t n, int32_t p, const uint8_t *dims, int32_t max_dim,
                       double alpha, int32_t max_level, uint16_t *G, int32_t *sepsets, int32_t *rec_pool,
                       int64_t rec_cap, double *pmax, gcsl_stats *stats, void *workspace, size_t workspace_bytes,
                       void *stream) {
    if (!data || !dims || !G || !pmax || p < 1 || n < 1 || ld < n || (ld % 16) != 0 || max_level < 0 ||
        max_dim < 1 || max_dim > 255 || reinterpret_cast<uintptr_t>(data) % 16 != 0)
        return GCSL_ERR_INVALID_ARG;
    if (rec_pool == nullptr) rec_cap = 0;
    DiscWs w = carve_disc(workspace, workspace_bytes, p);
    if (!workspace || w.bytes > workspace_bytes) return GCSL_ERR_WORKSPACE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int sms = device_sms();
    int dev = 0;
    cudaGetDevice(&dev);
    const int cap = host::disc_table_cap(dev);
    if ((long long)max_dim * max_dim > cap) return GCSL_ERR_UNSUPPORTED;
    cudaError_t e = cudaMemsetAsync(w.st, 0, sizeof(DevState), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(w.win, 0xff, sizeof(unsigned long long) * (size_t)p * p, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(pmax, 0, sizeof(double) * (size_t)p * p, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(G, 0, sizeof(uint16_t) * (size_t)p * p, s);
    if (e != cudaSuccess) return GCSL_ERR_DEVICE;
    DiscLevelArgs A{data, ld, n, p, dims, alpha, 0, w.adj, w.prefix, G, pmax, w.win, cap, 1024, w.st};
    A.order = host::work_order_seed();
    host::disc_level_caps(cap, max_dim, 0, A.table_cap, A.part_cap);
    // codes in range once per solve; the test kernels skip the per-sample checks then
    if (host::launch_disc_validate(data, ld, n, p, dims, w.st, sms, s) != cudaSuccess) return GCSL_ERR_DEVICE;
    if (host::launch_disc_tests(A, sms, s) != cudaSuccess) return GCSL_ERR_DEVICE;
    HostCtl *hc = host_ctl();
    if (!hc) return GCSL_ERR_DEVICE;
    auto disc_level = [&](int level) -> cudaError_t {
        cudaError_t e2 = host::launch_compact(G, p, w.adj, nullptr, w.st, level, nullptr, s);
        if (e2 == cudaSuccess) e2 = host::launch_disc_weights(w.adj, p, level, w.weights, w.st, s);
        if (e2 == cudaSuccess) e2 = host::launch_scan_ll(w.weights, p, w.prefix, w.st, s);
        if (e2 == cudaSuccess) e2 = host::launch_disc_level_stats(w.prefix, w.adj, p, level, w.st, s);
        DiscLevelArgs B = A;
        B.level = level;
        host::disc_level_caps(cap, max_dim, level, B.table_cap, B.part_cap);
        if (e2 == cudaSuccess) e2 = host::launch_disc_tests(B, sms, s);
        if (e2 == cudaSuccess)
            e2 = host::launch_disc_finalize(w.adj, p, level, G, w.win, sepsets, max_level, rec_pool, rec_cap, w.st,
                                            sms, s);
        return e2;
    };
    int rc = run_levels(max_level, w.st, s, hc->words, [&](int a, int b) -> cudaError_t {
        for (int level = a; level <= b; ++level) {
            const cudaError_t e2 = disc_level(level);
            if (e2 != cudaSuccess) return e2;
        }
        return cudaSuccess;
    });
    if (rc != GCSL_OK) return rc;
    if (host::launch_pmax_finish(pmax, p, sms, s) != cudaSuccess) return GCSL_ERR_DEVICE;
    return finish_stats(w.st, stats, s, true, p);
}

int gcsl_compact(const uint16_t *G, int32_t p, int32_t *adj, void *stream) {
    if (!G || !adj || p < 1) return GCSL_ERR_INVALID_ARG;
    return map_cuda(host::launch_compact(G, p, adj, nullptr, nullptr, 0, nullptr, static_cast<cudaStream_t>(stream)));
}

int gcsl_unrank(int32_t K, int32_t level, int64_t count, int32_t *out, void *stream) {
    if (!out || K < 0 || level < 1 || level >= GCSL_MAX_LEVELS || count < 0) return GCSL_ERR_INVALID_ARG;
    return map_cuda(host::launch_unrank(K, level, count, out, static_cast<cudaStream_t>(stream)));
}

int gcsl_pchisq(const double *x, const int64_t *df, int64_t count, double *out, void *stream) {
    if (!x || !df || !out || count < 0) return GCSL_ERR_INVALID_ARG;
    return map_cuda(host::launch_pchisq(x, reinterpret_cast<const long long *>(df), count, out,
                                        static_cast<cudaStream_t>(stream)));
}

int gcsl_disc_table(const uint8_t *data, int64_t ld, int64_t n, const uint8_t *dims, int32_t vi, int32_t vj,
                    const int32_t *S, int32_t level, uint32_t *counts, int64_t counts_cap, double *chi2_pvalue,
                    void *stream) {
    if (!data || !dims || !counts || !chi2_pvalue || n < 1 || ld < n || (ld % 16) != 0 || level < 0 || counts_cap < 1 ||
        level >= GCSL_MAX_LEVELS || (level > 0 && !S) || reinterpret_cast<uintptr_t>(data) % 16 != 0)
        return GCSL_ERR_INVALID_ARG;
    int dev = 0;
    cudaGetDevice(&dev);
    return map_cuda(host::launch_disc_table(data, ld, n, dims, vi, vj, S, level, host::disc_table_cap(dev), counts,
                                            counts_cap, chi2_pvalue, static_cast<cudaStream_t>(stream)));
}

int gcsl_tc_gemm_bf16(const uint16_t *A, const uint16_t *B, float *D, int32_t M, int32_t N, int32_t K, int32_t *err,
                      void *stream) {
    if (!A || !B || !D || !err || M < 128 || N < 128 || K < 64 || M % 128 || N % 128 || K % 64 ||
        reinterpret_cast<uintptr_t>(A) % 16 || reinterpret_cast<uintptr_t>(B) % 16)
        return GCSL_ERR_INVALID_ARG;
    return map_cuda(host::launch_tc_gemm_bf16(A, B, D, M, N, K, err, static_cast<cudaStream_t>(stream)));
}


// ------------------------------------------------------------------ batches
size_t gcsl_gauss_batch_workspace_bytes(const int32_t *p, int32_t count) {
    if (!p || count < 1) return 0;
    for (int k = 0; k < count; ++k)
        if (p[k] < 1 || p[k] > GCSL_GAUSS_MAX_P) return 0;
    return host::gauss_batch_workspace_bytes(p, count);
}

int gcsl_gauss_batch_prepare(const gcsl_gauss_instance *inst, int32_t count, int32_t max_level, int32_t precision,
                             void *workspace, size_t workspace_bytes, gcsl_batch_plan *plan, void *stream) {
    if (!inst || count < 1 || !plan || !workspace || max_level < 0 || max_level > GCSL_BATCH_MAX_LEVEL ||
        (precision != GCSL_PREC_F64 && precision != GCSL_PREC_SPLIT))
        return GCSL_ERR_INVALID_ARG;
    for (int k = 0; k < count; ++k) {
        const gcsl_gauss_instance &I = inst[k];
        if (!I.C || !I.G || !I.pmax || I.p < 1 || I.n_obs < 4 || !I.thresholds || I.n_thresholds < 1)
            return GCSL_ERR_INVALID_ARG;
        if (I.p > GCSL_GAUSS_MAX_P) return GCSL_ERR_UNSUPPORTED;
        if (precision == GCSL_PREC_SPLIT && (!I.C32 || !I.band_lo || !I.band_hi)) return GCSL_ERR_INVALID_ARG;
    }
    std::vector<int> ps((size_t)count);
    for (int k = 0; k < count; ++k) ps[(size_t)k] = inst[k].p;
    if (workspace_bytes < host::gauss_batch_workspace_bytes(ps.data(), count)) return GCSL_ERR_WORKSPACE;
    return host::gauss_batch_prepare(inst, count, max_level, precision, workspace, workspace_bytes,
                                     reinterpret_cast<long long *>(plan->w), device_sms(),
                                     static_cast<cudaStream_t>(stream));
}

int gcsl_gauss_batch_run(const gcsl_batch_plan *plan, void *stream) {
    if (!plan) return GCSL_ERR_INVALID_ARG;
    return host::gauss_batch_run(reinterpret_cast<const long long *>(plan->w), static_cast<cudaStream_t>(stream),
                                 false);
}

size_t gcsl_gauss_state_bytes(int32_t p) { return (p < 1 || p > GCSL_GAUSS_MAX_P) ? 0 : host::gauss_state_bytes(p); }

size_t gcsl_gauss_batch_table_bytes(int32_t count) { return count < 1 ? 0 : host::gauss_batch_table_bytes(count); }

static int check_instances(const gcsl_gauss_instance *inst, int32_t count, int32_t max_level, int32_t precision) {
    if (!inst || count < 1 || max_level < 0 || max_level > GCSL_BATCH_MAX_LEVEL ||
        (precision != GCSL_PREC_F64 && precision != GCSL_PREC_SPLIT))
        return GCSL_ERR_INVALID_ARG;
    for (int k = 0; k < count; ++k) {
        const gcsl_gauss_instance &I = inst[k];
        if (!I.C || !I.G || !I.pmax || I.p < 1 || I.n_obs < 4 || !I.thresholds || I.n_thresholds < 1)
            return GCSL_ERR_INVALID_ARG;
        if (I.p > GCSL_GAUSS_MAX_P) return GCSL_ERR_UNSUPPORTED;
        if (precision == GCSL_PREC_SPLIT && (!I.C32 || !I.band_lo || !I.band_hi)) return GCSL_ERR_INVALID_ARG;
        if (I.state != nullptr && reinterpret_cast<uintptr_t>(I.state) % 256 != 0) return GCSL_ERR_INVALID_ARG;
    }
    return GCSL_OK;
}

int gcsl_gauss_batch_prepare_staged(const gcsl_gauss_instance *inst, int32_t count, int32_t max_level,
                                    int32_t precision, void *workspace, size_t workspace_bytes, void *stage,
                                    size_t stage_bytes, gcsl_batch_plan *plan, void *stream) {
    if (!plan || !workspace || !stage) return GCSL_ERR_INVALID_ARG;
    const int rc = check_instances(inst, count, max_level, precision);
    if (rc != GCSL_OK) return rc;
    return host::gauss_batch_prepare_staged(inst, count, max_level, precision, workspace, workspace_bytes, stage,
                                            stage_bytes, reinterpret_cast<long long *>(plan->w), device_sms(),
                                            static_cast<cudaStream_t>(stream));
}

int gcsl_gauss_batch_step(const gcsl_batch_plan *plan, int32_t first_level, int32_t last_level, int32_t finish,
                          int32_t *host_status, void *stream) {
    if (!plan || first_level < 0 || last_level > GCSL_BATCH_MAX_LEVEL) return GCSL_ERR_INVALID_ARG;
    return host::gauss_batch_step(reinterpret_cast<const long long *>(plan->w), first_level, last_level, finish != 0,
                                  false, host_status, static_cast<cudaStream_t>(stream));
}

int gcsl_records_to_dense(const int32_t *rec, int64_t n_ints, int32_t p, int32_t max_level, int32_t *out) {
    if (n_ints < 0 || p < 1 || max_level < 0 || (!rec && n_ints > 0) || (!out && max_level > 0))
        return GCSL_ERR_INVALID_ARG;
    const size_t total = (size_t)p * p * (size_t)max_level;
    if (total == 0) return GCSL_OK;
    // the -1 fill is the bulk of the work for large p: split it over a few threads
    const size_t chunk = (size_t)1 << 22;
    const int nt = (int)std::min<size_t>(8, (total + chunk - 1) / chunk);
    if (nt > 1) {
        std::vector<std::thread> th;
        const size_t per = (total + nt - 1) / nt;
        for (int t = 0; t < nt; ++t)
            th.emplace_back([=] {
                const size_t a = (size_t)t * per, b = std::min(total, a + per);
                if (a < b) std::fill(out + a, out + b, -1);
            });
        for (auto &x : th) x.join();
    } else {
        std::fill(out, out + total, -1);
    }
    int64_t k = 0;
    while (k < n_ints) {
        if (k + 3 > n_ints) return GCSL_ERR_INVALID_ARG;
        const int lo = rec[k], hi = rec[k + 1], lev = rec[k + 2];
        if (lev < 0 || k + 3 + lev > n_ints || lo < 0 || lo >= p || hi < 0 || hi >= p) return GCSL_ERR_INVALID_ARG;
        if (lev <= max_level) {
            int32_t *a = out + ((size_t)lo * p + hi) * max_level;
            int32_t *b = out + ((size_t)hi * p + lo) * max_level;
            for (int c = 0; c < lev; ++c) a[c] = b[c] = rec[k + 3 + c];
        }
        k += 3 + lev;
    }
    return GCSL_OK;
}

int gcsl_gauss_batch_rerun(const gcsl_batch_plan *plan, void *stream) {
    if (!plan) return GCSL_ERR_INVALID_ARG;
    return host::gauss_batch_run(reinterpret_cast<const long long *>(plan->w), static_cast<cudaStream_t>(stream),
                                 true);
}

const int32_t *gcsl_gauss_batch_flags(const gcsl_batch_plan *plan) {
    if (!plan) return nullptr;
    return host::gauss_batch_flags(reinterpret_cast<const long long *>(plan->w));
}

int gcsl_gauss_batch_collect(const gcsl_batch_plan *plan, gcsl_gauss_instance *inst, int32_t count, void *stream) {
    if (!plan || !inst) return GCSL_ERR_INVALID_ARG;
    return host::gauss_batch_collect(reinterpret_cast<const long long *>(plan->w), inst, count,
                                     static_cast<cudaStream_t>(stream));
}

int gcsl_gauss_batch_set_lanes(gcsl_batch_plan *plan, int32_t level, int32_t lanes) {
    if (!plan) return GCSL_ERR_INVALID_ARG;
    return host::gauss_batch_set_lanes(reinterpret_cast<long long *>(plan->w), level, lanes);
}

// plan words of a correlation batch: [magic, workspace, count, dtype, stage totals...]
static const long long kCorrPlanMagic = 0x4743534c434f5252ll;  // "GCSLCORR"

size_t gcsl_corr_tc_batch_workspace_bytes(const int64_t *n, const int32_t *p, int32_t count) {
    if (!n || !p || count < 1) return 0;
    std::vector<long long> nn((size_t)count);
    std::vector<int> pp((size_t)count);
    for (int k = 0; k < count; ++k) {
        if (n[k] < 2 || p[k] < 1) return 0;
        nn[(size_t)k] = n[k];
        pp[(size_t)k] = p[k];
    }
    return host::corr_tc_batch_workspace_bytes(nn.data(), pp.data(), count);
}

int gcsl_corr_tc_batch_prepare(const void *const *X, int32_t dtype, const int64_t *n, const int32_t *p,
                               const int64_t *ldx, double *const *C, float *const *C32, int32_t count,
                               void *workspace, size_t workspace_bytes, gcsl_batch_plan *plan, void *stream) {
    if (!X || !n || !p || !ldx || !C || count < 1 || !workspace || !plan ||
        (dtype != GCSL_DTYPE_F64 && dtype != GCSL_DTYPE_F32))
        return GCSL_ERR_INVALID_ARG;
    std::vector<long long> nn((size_t)count), ll((size_t)count);
    std::vector<int> pp((size_t)count);
    for (int k = 0; k < count; ++k) {
        if (!X[k] || !C[k] || n[k] < 2 || p[k] < 1 || ldx[k] < p[k]) return GCSL_ERR_INVALID_ARG;
        nn[(size_t)k] = n[k];
        pp[(size_t)k] = p[k];
        ll[(size_t)k] = ldx[k];
    }
    if (workspace_bytes < host::corr_tc_batch_workspace_bytes(nn.data(), pp.data(), count)) return GCSL_ERR_WORKSPACE;
    long long *w = reinterpret_cast<long long *>(plan->w);
    std::memset(w, 0, sizeof(plan->w));
    const cudaError_t e =
        host::corr_tc_batch_prepare(X, nn.data(), pp.data(), ll.data(), C, C32, count, workspace, workspace_bytes,
                                    w + 4, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return GCSL_ERR_DEVICE;
    w[0] = kCorrPlanMagic;
    w[1] = (long long)reinterpret_cast<uintptr_t>(workspace);
    w[2] = count;
    w[3] = dtype;
    return GCSL_OK;
}

int gcsl_corr_tc_batch_run(const gcsl_batch_plan *plan, void *stream) {
    if (!plan) return GCSL_ERR_INVALID_ARG;
    const long long *w = reinterpret_cast<const long long *>(plan->w);
    if (w[0] != kCorrPlanMagic) return GCSL_ERR_INVALID_ARG;
    return map_cuda(host::corr_tc_batch_run(reinterpret_cast<void *>(static_cast<uintptr_t>(w[1])), (int)w[2], w + 4,
                                            (int)w[3], static_cast<cudaStream_t>(stream)));
}

int gcsl_corr_tc_batch_run_split(const gcsl_batch_plan *plan, double *c_err, void *stream) {
    if (!plan || !c_err) return GCSL_ERR_INVALID_ARG;
    const long long *w = reinterpret_cast<const long long *>(plan->w);
    if (w[0] != kCorrPlanMagic) return GCSL_ERR_INVALID_ARG;
    return map_cuda(host::corr_tc_batch_run_mode(reinterpret_cast<void *>(static_cast<uintptr_t>(w[1])), (int)w[2],
                                                 w + 4, (int)w[3], host::CORR_BATCH_SPLIT, c_err, nullptr,
                                                 static_cast<cudaStream_t>(stream)));
}

int gcsl_corr_tc_batch_run_flagged(const gcsl_batch_plan *plan, const int32_t *flags, void *stream) {
    if (!plan || !flags) return GCSL_ERR_INVALID_ARG;
    const long long *w = reinterpret_cast<const long long *>(plan->w);
    if (w[0] != kCorrPlanMagic) return GCSL_ERR_INVALID_ARG;
    return map_cuda(host::corr_tc_batch_run_mode(reinterpret_cast<void *>(static_cast<uintptr_t>(w[1])), (int)w[2],
                                                 w + 4, (int)w[3], host::CORR_BATCH_FLAGGED, nullptr, flags,
                                                 static_cast<cudaStream_t>(stream)));
}


// ---------------------------------------------------------------- orientation
size_t gcsl_orient_workspace_bytes(int32_t p) {
    if (p < 1 || p > GCSL_GAUSS_MAX_P) return 0;
    return host::orient_workspace_bytes(p);
}

int gcsl_orient_edges(const uint16_t *G, int32_t p, const int32_t *sepsets, int32_t sep_len, uint8_t *dag,
                      int32_t *passes, void *workspace, size_t workspace_bytes, void *stream) {
    if (!G || !dag || p < 1 || sep_len < 0 || (sep_len > 0 && !sepsets)) return GCSL_ERR_INVALID_ARG;
    if (p > GCSL_GAUSS_MAX_P) return GCSL_ERR_UNSUPPORTED;
    if (!workspace || workspace_bytes < host::orient_workspace_bytes(p)) return GCSL_ERR_WORKSPACE;
    HostCtl *hc = host_ctl();
    if (!hc) return GCSL_ERR_DEVICE;
    int n = 0;
    const cudaError_t e = host::orient_edges(G, p, sepsets, sep_len, dag, workspace, device_sms(), &hc->words[0], &n,
                                             static_cast<cudaStream_t>(stream));
    if (passes) *passes = n;
    return map_cuda(e);
}


// ------------------------------------------------------------- ordinal encoding
size_t gcsl_encode_workspace_bytes(int32_t p) { return p < 1 ? 256 : host::encode_workspace_bytes(p); }

int gcsl_ordinal_encode(const void *X, int32_t dtype, int64_t n, int32_t p, int64_t ld, uint8_t *codes, int64_t ldc,
                        uint8_t *dims, void *workspace, size_t workspace_bytes, void *stream) {
    if (!X || !codes || !dims || n < 0 || p < 1 || ld < p || ldc < n ||
        (dtype != GCSL_DTYPE_I32 && dtype != GCSL_DTYPE_I64 && dtype != GCSL_DTYPE_U8 && dtype != GCSL_DTYPE_F64))
        return GCSL_ERR_INVALID_ARG;
    if (!workspace || workspace_bytes < gcsl_encode_workspace_bytes(p) ||
        reinterpret_cast<uintptr_t>(workspace) % 256 != 0)
        return GCSL_ERR_WORKSPACE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int *status = static_cast<int *>(workspace);  // the workspace starts with the status word
    HostCtl *hc = host_ctl();
    if (!hc) return GCSL_ERR_DEVICE;
    cudaError_t e = host::encode_columns(X, dtype, n, p, ld, codes, ldc, dims, workspace, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hc->words[0], status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return map_cuda(e);
    return hc->words[0];
}

}  // extern "C"
