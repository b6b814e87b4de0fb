// Ordinal encoding of discrete samples on the device (replaces the host OrdinalEncoder
// and the dims computation of gpucsl/pc/discover_skeleton_discrete.py:38-49): per
// column, the observed values in ascending order get codes 0..k-1 and dims = k.
//
// Integer-valued inputs (int32, int64, uint8, or float64 holding integers) whose column
// range is below ENC_RANGE are encoded in four passes, each over a grid of (32-column
// block, row chunk) tiles so that every SM streams its share of X:
//   1. column minimum / maximum and integrality (per-column atomics);
//   2. presence bitmap of v - min per column (shared-memory bitmap per tile, merged into
//      the global one with atomicOr);
//   3. per column, prefix popcounts of the bitmap words (rank of the first value of each
//      word) and dims; one warp per column;
//   4. codes = rank of the word + popcount of the lower bits, transposed through shared
//      memory into the column-major layout of the discrete solver (column j at
//      codes + j * ldc).
// A column with more than 255 distinct values, a wider range, or a non-integer value sets
// GCSL_ERR_UNSUPPORTED in the status word (passes 2 and 4 skip out-of-range values, so
// nothing is written out of bounds).
#include "common.cuh"

namespace gcsl {

constexpr int ENC_RANGE = 4096;  // values per column: min .. min + 4095
constexpr int ENC_WORDS = ENC_RANGE / 32;
constexpr int ENC_ROWS = 256;    // rows per tile (a multiple of 32) unless n needs more

// Per-column scratch of the encoder.
struct EncWs {
    long long *mn, *mx;  // column minimum / maximum
    int *bad;            // column has a non-integer value
    unsigned *bits;      // presence bitmap, ENC_WORDS words per column
    uint8_t *rank;       // rank of the first value of each word, ENC_WORDS per column
    int *status;
};

template <typename T>
__device__ __forceinline__ bool enc_value(T x, long long &v) {
    if constexpr (sizeof(T) == 8 && (T)0.5 != 0) {  // double
        const double d = (double)x;
        v = (long long)d;
        return (double)v == d;  // integral (NaN fails)
    } else {
        v = (long long)x;
        return true;
    }
}

// Pass 1: tile (blockIdx.x: 32 columns, blockIdx.y: ENC_ROWS rows); lane = column.
template <typename T>
__global__ void __launch_bounds__(256) enc_range_kernel(const T *__restrict__ X, long long n, int p, long long ld,
                                                       int rows, EncWs w) {
    __shared__ long long smin[8][32], smax[8][32];
    __shared__ int sbad[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = blockIdx.x * 32 + lane;
    const long long t0 = (long long)blockIdx.y * rows, t1 = min(n, t0 + rows);
    long long mn = 0x7fffffffffffffffll, mx = (long long)0x8000000000000000ull;
    bool ok = true;
    if (threadIdx.x < 32) sbad[threadIdx.x] = 0;
    __syncthreads();
    if (j < p) {
        for (long long t = t0 + warp; t < t1; t += 8) {
            long long v;
            ok = enc_value(X[t * ld + j], v) && ok;
            mn = v < mn ? v : mn;
            mx = v > mx ? v : mx;
        }
    }
    smin[warp][lane] = mn;
    smax[warp][lane] = mx;
    if (!ok) sbad[lane] = 1;
    __syncthreads();
    if (warp == 0 && j < p) {
        for (int q = 1; q < 8; ++q) {
            mn = smin[q][lane] < mn ? smin[q][lane] : mn;
            mx = smax[q][lane] > mx ? smax[q][lane] : mx;
        }
        atomicMin(w.mn + j, mn);
        atomicMax(w.mx + j, mx);
        if (sbad[lane]) atomicOr(w.bad + j, 1);
    }
}

// Pass 2: presence bits of the tile's values, merged into the global bitmap.
template <typename T>
__global__ void __launch_bounds__(256) enc_bits_kernel(const T *__restrict__ X, long long n, int p, long long ld,
                                                      int rows, EncWs w) {
    __shared__ unsigned bits[32][ENC_WORDS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j0 = blockIdx.x * 32, j = j0 + lane;
    for (int k = threadIdx.x; k < 32 * ENC_WORDS; k += blockDim.x) (&bits[0][0])[k] = 0u;
    __syncthreads();
    const long long t0 = (long long)blockIdx.y * rows, t1 = min(n, t0 + rows);
    if (j < p) {
        const long long base = w.mn[j];
        for (long long t = t0 + warp; t < t1; t += 8) {
            long long v;
            enc_value(X[t * ld + j], v);
            const unsigned long long o = (unsigned long long)v - (unsigned long long)base;
            // values repeat: set a bit only when it is not set yet (few atomics)
            if (o < ENC_RANGE) {
                const unsigned bit = 1u << (o & 31);
                if (!(bits[lane][o >> 5] & bit)) atomicOr(&bits[lane][o >> 5], bit);
            }
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 32 * ENC_WORDS; k += blockDim.x) {
        const int c = k / ENC_WORDS, wd = k - c * ENC_WORDS;
        const unsigned b = bits[c][wd];
        if (b != 0u && j0 + c < p) atomicOr(w.bits + (size_t)(j0 + c) * ENC_WORDS + wd, b);
    }
}

// Pass 3: one warp per column: word ranks (exclusive prefix popcounts) and dims.
__global__ void __launch_bounds__(256) enc_rank_kernel(long long n, int p, uint8_t *__restrict__ dims, EncWs w) {
    const int lane = threadIdx.x & 31;
    const int j = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (j >= p) return;
    const unsigned *b = w.bits + (size_t)j * ENC_WORDS;
    int carry = 0;
    for (int w0 = 0; w0 < ENC_WORDS; w0 += 32) {
        const int cnt = __popc(b[w0 + lane]);
        int x = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(GCSL_FULL_MASK, x, o);
            if (lane >= o) x += y;
        }
        const int r = carry + x - cnt;
        w.rank[(size_t)j * ENC_WORDS + w0 + lane] = (uint8_t)(r < 255 ? r : 255);
        carry += __shfl_sync(GCSL_FULL_MASK, x, 31);
    }
    if (lane == 0) {
        // (no values: min > max; otherwise the unsigned difference is the range)
        const bool wide = n > 0 && (unsigned long long)w.mx[j] - (unsigned long long)w.mn[j] >= ENC_RANGE;
        if (carry > 255 || wide || w.bad[j]) atomicCAS(w.status, 0, GCSL_ERR_UNSUPPORTED);
        dims[j] = (uint8_t)(carry > 0 ? (carry > 255 ? 255 : carry) : 1);
    }
}

// Pass 4: codes of the tile, 32 samples x 32 columns at a time, written column-major.
template <typename T>
__global__ void __launch_bounds__(256) enc_codes_kernel(const T *__restrict__ X, long long n, int p, long long ld,
                                                       int rows, uint8_t *__restrict__ codes, long long ldc, EncWs w) {
    __shared__ unsigned bits[32][ENC_WORDS];
    __shared__ uint8_t rank[32][ENC_WORDS];
    __shared__ uint8_t tile[32][33];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j0 = blockIdx.x * 32, j = j0 + lane;
    for (int k = threadIdx.x; k < 32 * ENC_WORDS; k += blockDim.x) {
        const int c = k / ENC_WORDS, wd = k - c * ENC_WORDS;
        const bool col = j0 + c < p;
        bits[c][wd] = col ? w.bits[(size_t)(j0 + c) * ENC_WORDS + wd] : 0u;
        rank[c][wd] = col ? w.rank[(size_t)(j0 + c) * ENC_WORDS + wd] : (uint8_t)0;
    }
    const long long base = j < p ? w.mn[j] : 0;
    __syncthreads();
    const long long t0 = (long long)blockIdx.y * rows, t1 = min(n, t0 + rows);
    for (long long ts = t0; ts < t1; ts += 32) {
        for (int r = warp; r < 32; r += 8) {
            const long long t = ts + r;
            uint8_t code = 0;
            if (j < p && t < t1) {
                long long v;
                enc_value(X[t * ld + j], v);
                const unsigned long long o = (unsigned long long)v - (unsigned long long)base;
                if (o < ENC_RANGE) {
                    const int wd = (int)(o >> 5);
                    code = (uint8_t)(rank[lane][wd] + __popc(bits[lane][wd] & ((1u << (o & 31)) - 1u)));
                }
            }
            tile[r][lane] = code;
        }
        __syncthreads();
        {
            const int c = threadIdx.x >> 3, g = threadIdx.x & 7;  // column, 4-sample group
            const long long t = ts + g * 4;
            if (j0 + c < p && t < t1) {
                uint8_t *dst = codes + (size_t)(j0 + c) * ldc + t;
                if (t + 4 <= t1 && ((reinterpret_cast<uintptr_t>(dst) & 3u) == 0)) {
                    *reinterpret_cast<uint32_t *>(dst) = (uint32_t)tile[g * 4][c] | ((uint32_t)tile[g * 4 + 1][c] << 8) |
                                                         ((uint32_t)tile[g * 4 + 2][c] << 16) |
                                                         ((uint32_t)tile[g * 4 + 3][c] << 24);
                } else {
                    for (int e = 0; e < 4 && t + e < t1; ++e) dst[e] = tile[g * 4 + e][c];
                }
            }
        }
        __syncthreads();
    }
}

namespace host {

size_t encode_workspace_bytes(int p) {
    const size_t per = 2 * sizeof(long long) + sizeof(int) + ENC_WORDS * sizeof(unsigned) + ENC_WORDS;
    return 256 + ((size_t)p * per + 255) / 256 * 256;
}

static EncWs enc_ws(void *ws, int p) {
    uint8_t *c = static_cast<uint8_t *>(ws);
    EncWs w;
    w.status = reinterpret_cast<int *>(c);
    c += 256;
    w.mn = reinterpret_cast<long long *>(c);
    c += (size_t)p * sizeof(long long);
    w.mx = reinterpret_cast<long long *>(c);
    c += (size_t)p * sizeof(long long);
    w.bits = reinterpret_cast<unsigned *>(c);
    c += (size_t)p * ENC_WORDS * sizeof(unsigned);
    w.bad = reinterpret_cast<int *>(c);
    c += (size_t)p * sizeof(int);
    w.rank = c;
    return w;
}

template <typename T>
static cudaError_t encode_typed(const T *X, long long n, int p, long long ld, uint8_t *codes, long long ldc,
                                uint8_t *dims, const EncWs &w, cudaStream_t s) {
    // tiles of ENC_ROWS rows, or more (a multiple of 32) when n needs over 65535 of them
    long long rows = ENC_ROWS;
    if ((n + rows - 1) / rows > 65535) rows = ((n + 65534) / 65535 + 31) / 32 * 32;
    const dim3 grid((unsigned)((p + 31) / 32), (unsigned)((n + rows - 1) / rows));
    if (n > 0) {
        enc_range_kernel<T><<<grid, 256, 0, s>>>(X, n, p, ld, (int)rows, w);
        enc_bits_kernel<T><<<grid, 256, 0, s>>>(X, n, p, ld, (int)rows, w);
    }
    enc_rank_kernel<<<(unsigned)((p + 7) / 8), 256, 0, s>>>(n, p, dims, w);
    if (n > 0) enc_codes_kernel<T><<<grid, 256, 0, s>>>(X, n, p, ld, (int)rows, codes, ldc, w);
    note_launch(n > 0 ? 4 : 1);
    return cudaGetLastError();
}

// status: the first int of the workspace (cleared here); the caller reads it back.
cudaError_t encode_columns(const void *X, int dtype, long long n, int p, long long ld, uint8_t *codes, long long ldc,
                           uint8_t *dims, void *workspace, cudaStream_t s) {
    const EncWs w = enc_ws(workspace, p);
    cudaError_t e = cudaMemsetAsync(w.status, 0, sizeof(int), s);
    // minimum starts at 0x7f7f.. (above every value), maximum at 0x8080.. (below every value)
    if (e == cudaSuccess) e = cudaMemsetAsync(w.mn, 0x7f, (size_t)p * sizeof(long long), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(w.mx, 0x80, (size_t)p * sizeof(long long), s);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(w.bits, 0, (size_t)p * (ENC_WORDS * sizeof(unsigned) + sizeof(int)), s);  // bits, bad
    if (e != cudaSuccess) return e;
    switch (dtype) {
    case GCSL_DTYPE_I32: return encode_typed(static_cast<const int *>(X), n, p, ld, codes, ldc, dims, w, s);
    case GCSL_DTYPE_I64: return encode_typed(static_cast<const long long *>(X), n, p, ld, codes, ldc, dims, w, s);
    case GCSL_DTYPE_U8: return encode_typed(static_cast<const uint8_t *>(X), n, p, ld, codes, ldc, dims, w, s);
    case GCSL_DTYPE_F64: return encode_typed(static_cast<const double *>(X), n, p, ld, codes, ldc, dims, w, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace host
}  // namespace gcsl
