// Allocation-free variant of the Gaussian skeleton entry point.
//
// Some callers cannot call cudaMalloc: a host runtime whose own allocator owns every
// byte of device memory (a JVM/Go/serving process that reserves its pool at start-up
// and forbids later device allocations), or code that must not allocate while other
// work is in flight on the device.  For them gcsl_gauss_skeleton_noalloc takes the
// same inputs and outputs as gcsl_gauss_skeleton, but its scratch space (solve state,
// compacted adjacency, edge prefix, per-pair z*) lives in the file-scope device array
// below instead of a caller-provided workspace.
//
// * The array holds GCSL_NOALLOC_SCRATCH_BYTES; p < 1 is an invalid argument, and
//   problems with p > GCSL_NOALLOC_MAX_P are rejected with GCSL_ERR_UNSUPPORTED before
//   any device work.
// * Every GPU that loads this library holds the array until the process exits.
// * The array's device address is looked up once per device, on the first call made
//   with that device current (cudaGetSymbolAddress); make that first call before any
//   stream capture begins.  The cached address belongs to the device's context as it
//   was at that first call: a cudaDeviceReset after it is not supported.
// * All calls share the one array and it keeps the last call's contents: the solve
//   clears its state block at the start and overwrites every other scratch word before
//   reading it.  Calls whose device work overlaps (different streams, no ordering)
//   race on the array; serialise them.
// * Nothing is allocated or created, on the first call of a thread or any other: no
//   cudaMalloc, cudaFree, cudaMallocHost or allocating library routine, no stream and no
//   event.  Every kernel of the solve goes on the caller's stream in order, and the
//   level loop's control words are read into the calling thread's stack by synchronous
//   copies (the call synchronises the stream, as gcsl_gauss_skeleton does).
#include <mutex>

#include "common.cuh"

static __device__ __align__(256) unsigned char g_gauss_noalloc_scratch[GCSL_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[256] = {nullptr};

// Device address of the scratch array for the current device (looked up once).
int noalloc_scratch(void **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return GCSL_ERR_DEVICE;
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (g_noalloc_ptr[dev] == nullptr) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_gauss_noalloc_scratch) != cudaSuccess || p == nullptr) return GCSL_ERR_DEVICE;
        g_noalloc_ptr[dev] = p;
    }
    *out = g_noalloc_ptr[dev];
    return GCSL_OK;
}

}  // namespace

extern "C" int gcsl_gauss_skeleton_noalloc(const double *C, int32_t p, int64_t n_obs, const double *thresholds,
                                           int32_t n_thresholds, int32_t max_level, uint16_t *G, int32_t *sepsets,
                                           int32_t *rec_pool, int64_t rec_cap, double *pmax, gcsl_stats *stats,
                                           void *stream) {
    if (p < 1) return GCSL_ERR_INVALID_ARG;
    if (p > GCSL_NOALLOC_MAX_P) return GCSL_ERR_UNSUPPORTED;
    if (gcsl_gauss_workspace_bytes(p, max_level) > sizeof(g_gauss_noalloc_scratch)) return GCSL_ERR_UNSUPPORTED;
    void *scratch = nullptr;
    const int rc = noalloc_scratch(&scratch);
    if (rc != GCSL_OK) return rc;
    return gcsl::host::gauss_skeleton_run(C, p, n_obs, thresholds, n_thresholds, max_level, G, sepsets, rec_pool,
                                          rec_cap, pmax, stats, scratch, sizeof(g_gauss_noalloc_scratch), stream,
                                          true);
}
