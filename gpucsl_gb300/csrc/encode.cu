// Ordinal encoding of discrete samples on the device (replaces the host OrdinalEncoder
// and the dims computation of gpucsl/pc/discover_skeleton_discrete.py:38-49): per
// column, the observed values in ascending order get codes 0..k-1 and dims = k.
//
// Integer-valued inputs (int32, int64, uint8, or float64 holding integers) whose column
// range is below ENC_RANGE are encoded in one block per 32 columns: a presence bitmap per
// column in shared memory (atomicOr), its prefix popcounts as the rank table, then the
// codes, transposed through shared memory into the column-major layout of the discrete
// solver (column j at codes + j * ldc).  A column with more than 255 distinct values, a
// wider range, or a non-integer value returns GCSL_ERR_UNSUPPORTED (status word).
#include "common.cuh"

namespace gcsl {

constexpr int ENC_RANGE = 4096;  // values per column: min .. min + 4095
constexpr int ENC_WORDS = ENC_RANGE / 32;

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

template <typename T>
__global__ void __launch_bounds__(256) encode_kernel(const T *__restrict__ X, long long n, int p, long long ld,
                                                    uint8_t *__restrict__ codes, long long ldc,
                                                    uint8_t *__restrict__ dims, int *status) {
    __shared__ unsigned bits[32][ENC_WORDS];
    __shared__ int rank0[32][ENC_WORDS];
    __shared__ long long smin[8][32], smax[8][32];
    __shared__ uint8_t tile[32][33];
    __shared__ int bad;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j0 = blockIdx.x * 32, j = j0 + lane;
    const bool col = j < p;
    if (threadIdx.x == 0) bad = 0;
    // pass 0: column min / max (and integrality)
    long long mn = 0x7fffffffffffffffll, mx = (long long)0x8000000000000000ull;
    bool ok = true;
    for (long long t = warp; t < n; t += 8) {
        if (!col) break;
        long long v;
        ok = enc_value(X[t * ld + j], v) && ok;
        mn = v < mn ? v : mn;
        mx = v > mx ? v : mx;
    }
    smin[warp][lane] = mn;
    smax[warp][lane] = mx;
    for (int k = threadIdx.x; k < 32 * ENC_WORDS; k += blockDim.x) (&bits[0][0])[k] = 0u;
    if (!ok) atomicExch(&bad, 1);
    __syncthreads();
    if (warp == 0) {
        for (int q = 1; q < 8; ++q) {
            mn = smin[q][lane] < mn ? smin[q][lane] : mn;
            mx = smax[q][lane] > mx ? smax[q][lane] : mx;
        }
        smin[0][lane] = mn;
        smax[0][lane] = mx;
        if (col && n > 0 && mx - mn >= ENC_RANGE) atomicExch(&bad, 1);
    }
    __syncthreads();
    if (bad) {
        if (threadIdx.x == 0) atomicCAS(status, 0, GCSL_ERR_UNSUPPORTED);
        return;
    }
    const long long base = smin[0][lane];
    // pass 1: presence bits
    for (long long t = warp; t < n; t += 8) {
        if (!col) break;
        long long v;
        enc_value(X[t * ld + j], v);
        const int o = (int)(v - base);
        atomicOr(&bits[lane][o >> 5], 1u << (o & 31));
    }
    __syncthreads();
    // rank table: exclusive prefix popcounts per column (warp w handles columns w, w + 8, ..)
    for (int c = warp; c < 32; c += 8) {
        int carry = 0;
        for (int w0 = 0; w0 < ENC_WORDS; w0 += 32) {
            const int cnt = __popc(bits[c][w0 + lane]);
            int x = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(GCSL_FULL_MASK, x, o);
                if (lane >= o) x += y;
            }
            rank0[c][w0 + lane] = carry + x - cnt;
            carry += __shfl_sync(GCSL_FULL_MASK, x, 31);
        }
        if (lane == 0 && j0 + c < p) {
            if (carry > 255) atomicExch(&bad, 1);
            dims[j0 + c] = (uint8_t)(carry > 0 ? (carry > 255 ? 255 : carry) : 1);
        }
    }
    __syncthreads();
    if (bad) {
        if (threadIdx.x == 0) atomicCAS(status, 0, GCSL_ERR_UNSUPPORTED);
        return;
    }
    // pass 2: codes, 32 samples x 32 columns per tile, written column-major
    for (long long t0 = 0; t0 < n; t0 += 32) {
        for (int r = warp; r < 32; r += 8) {
            const long long t = t0 + r;
            uint8_t code = 0;
            if (col && t < n) {
                long long v;
                enc_value(X[t * ld + j], v);
                const int o = (int)(v - base);
                code = (uint8_t)(rank0[lane][o >> 5] + __popc(bits[lane][o >> 5] & ((1u << (o & 31)) - 1u)));
            }
            tile[r][lane] = code;
        }
        __syncthreads();
        {
            const int c = threadIdx.x >> 3, g = threadIdx.x & 7;  // column, 4-sample group
            if (j0 + c < p) {
                for (int e = 0; e < 4; ++e) {
                    const long long t = t0 + g * 4 + e;
                    if (t < n) codes[(size_t)(j0 + c) * ldc + t] = tile[g * 4 + e][c];
                }
            }
        }
        __syncthreads();
    }
}

namespace host {

cudaError_t encode_columns(const void *X, int dtype, long long n, int p, long long ld, uint8_t *codes, long long ldc,
                           uint8_t *dims, int *status, cudaStream_t s) {
    const unsigned blocks = (unsigned)((p + 31) / 32);
    switch (dtype) {
    case GCSL_DTYPE_I32:
        encode_kernel<int><<<blocks, 256, 0, s>>>(static_cast<const int *>(X), n, p, ld, codes, ldc, dims, status);
        break;
    case GCSL_DTYPE_I64:
        encode_kernel<long long><<<blocks, 256, 0, s>>>(static_cast<const long long *>(X), n, p, ld, codes, ldc, dims,
                                                         status);
        break;
    case GCSL_DTYPE_U8:
        encode_kernel<uint8_t><<<blocks, 256, 0, s>>>(static_cast<const uint8_t *>(X), n, p, ld, codes, ldc, dims,
                                                       status);
        break;
    case GCSL_DTYPE_F64:
        encode_kernel<double><<<blocks, 256, 0, s>>>(static_cast<const double *>(X), n, p, ld, codes, ldc, dims,
                                                      status);
        break;
    default:
        return cudaErrorInvalidValue;
    }
    note_launch(1);
    return cudaGetLastError();
}

}  // namespace host
}  // namespace gcsl
