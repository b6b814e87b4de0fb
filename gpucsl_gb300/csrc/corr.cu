// Correlation matrix build, FP64 (kernel a, plain path).
//
// Replaces gpucsl/pc/helpers.py:58-59 (np.corrcoef(data, rowvar=False)).  Same
// arithmetic as numpy's cov/corrcoef: centre by the column means, cov = X_c^T X_c
// times 1/(n-1), C_ij = (cov_ij / s_i) / s_j with s = sqrt(diag(cov)), clipped to
// [-1, 1].  The GEMM visits upper-triangle tiles only and mirrors them; the column
// means are reduced in a fixed order so the result is run-to-run identical.
//
// On GB300 FP64 runs on the CUDA cores at a small fraction of the FP32 rate, so this
// kernel is FP64-pipe bound; shared-memory staging keeps operand reuse at 4 DFMA per
// shared-memory load.
#include "common.cuh"

namespace gcsl {

constexpr int CORR_ROWS_PER_CHUNK = 256;
constexpr int CT = 64;   // output tile edge
constexpr int CK = 16;   // samples per K step

template <typename T>
__global__ void col_partial_sums_kernel(const T *__restrict__ X, long long n, int p, long long ldx,
                                        double *__restrict__ partial) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    const long long chunk = blockIdx.y;
    if (j >= p) return;
    const long long t0 = chunk * CORR_ROWS_PER_CHUNK;
    const long long t1 = min(n, t0 + CORR_ROWS_PER_CHUNK);
    double s = 0.0;
    for (long long t = t0; t < t1; ++t) s += (double)X[t * ldx + j];
    partial[chunk * p + j] = s;
}

__global__ void col_mean_kernel(const double *__restrict__ partial, long long n, int p, int chunks,
                                double *__restrict__ mean) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= p) return;
    double s = 0.0;
    for (int c = 0; c < chunks; ++c) s += partial[(long long)c * p + j];
    mean[j] = s / (double)n;
}

// cov tile (bi <= bj) of X_c^T X_c scaled by 1/(n-1); 256 threads, 4x4 outputs each.
template <typename T>
__global__ void __launch_bounds__(256) cov_tile_kernel(const T *__restrict__ X, long long n, int p, long long ldx,
                                                       const double *__restrict__ mean, double scale,
                                                       double *__restrict__ C) {
    // map linear block id to an upper-triangle tile (bi <= bj)
    const int nb = (p + CT - 1) / CT;
    int rem = blockIdx.x, bi = 0;
    while (rem >= nb - bi) {
        rem -= nb - bi;
        ++bi;
    }
    const int bj = bi + rem;
    const int i0 = bi * CT, j0 = bj * CT;

    __shared__ double As[CK][CT];
    __shared__ double Bs[CK][CT];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;

    for (long long t0 = 0; t0 < n; t0 += CK) {
#pragma unroll
        for (int q = 0; q < (CK * CT) / 256; ++q) {
            const int idx = threadIdx.x + q * 256;
            const int k = idx / CT, c = idx % CT;
            const long long t = t0 + k;
            const int ci = i0 + c, cj = j0 + c;
            As[k][c] = (t < n && ci < p) ? (double)X[t * ldx + ci] - mean[ci] : 0.0;
            Bs[k][c] = (t < n && cj < p) ? (double)X[t * ldx + cj] - mean[cj] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < CK; ++k) {
            double a[4], b[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                a[q] = As[k][ty + 16 * q];
                b[q] = Bs[k][tx + 16 * q];
            }
#pragma unroll
            for (int x = 0; x < 4; ++x)
#pragma unroll
                for (int y = 0; y < 4; ++y) acc[x][y] = fma(a[x], b[y], acc[x][y]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) {
            const int i = i0 + ty + 16 * x, j = j0 + tx + 16 * y;
            if (i < p && j < p && (bi != bj || i <= j)) {
                const double v = acc[x][y] * scale;
                C[(size_t)i * p + j] = v;
                C[(size_t)j * p + i] = v;
            }
        }
}

__global__ void diag_sqrt_kernel(const double *__restrict__ C, int p, double *__restrict__ sd) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < p) sd[i] = sqrt(C[(size_t)i * p + i]);
}

__global__ void normalize_kernel(double *__restrict__ C, int p, const double *__restrict__ sd) {
    const long long total = (long long)p * p;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / p), j = (int)(k - (long long)i * p);
        double v = C[k] / sd[i];
        v = v / sd[j];
        C[k] = fmin(fmax(v, -1.0), 1.0);
    }
}

namespace host {

size_t corr_workspace_bytes(long long n, int p) {
    const long long chunks = (n + CORR_ROWS_PER_CHUNK - 1) / CORR_ROWS_PER_CHUNK;
    return (size_t)(chunks * p + 2 * (long long)p) * sizeof(double) + 256;
}

template <typename T>
static cudaError_t corr_impl(const T *X, long long n, int p, long long ldx, double *C, void *ws, size_t ws_bytes,
                             int num_sms, cudaStream_t s) {
    const long long chunks = (n + CORR_ROWS_PER_CHUNK - 1) / CORR_ROWS_PER_CHUNK;
    if (ws_bytes < corr_workspace_bytes(n, p)) return cudaErrorInvalidValue;
    double *partial = static_cast<double *>(ws);
    double *mean = partial + chunks * p;
    double *sd = mean + p;
    dim3 g1((p + 127) / 128, (unsigned)chunks);
    col_partial_sums_kernel<T><<<g1, 128, 0, s>>>(X, n, p, ldx, partial);
    note_launch(1);
    col_mean_kernel<<<(p + 127) / 128, 128, 0, s>>>(partial, n, p, (int)chunks, mean);
    note_launch(1);
    const int nb = (p + CT - 1) / CT;
    const int tiles = nb * (nb + 1) / 2;
    const double scale = 1.0 / (double)(n - 1);
    cov_tile_kernel<T><<<tiles, 256, 0, s>>>(X, n, p, ldx, mean, scale, C);
    note_launch(1);
    diag_sqrt_kernel<<<(p + 127) / 128, 128, 0, s>>>(C, p, sd);
    note_launch(1);
    normalize_kernel<<<num_sms * 4, 256, 0, s>>>(C, p, sd);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t corr_partial_means(const void *X, int dtype, long long n, int p, long long ldx, double *partial,
                               double *mean, cudaStream_t s) {
    const long long chunks = (n + CORR_ROWS_PER_CHUNK - 1) / CORR_ROWS_PER_CHUNK;
    dim3 g1((p + 127) / 128, (unsigned)chunks);
    if (dtype == GCSL_DTYPE_F64)
        col_partial_sums_kernel<double><<<g1, 128, 0, s>>>(static_cast<const double *>(X), n, p, ldx, partial);
    else
        col_partial_sums_kernel<float><<<g1, 128, 0, s>>>(static_cast<const float *>(X), n, p, ldx, partial);
    note_launch(1);
    col_mean_kernel<<<(p + 127) / 128, 128, 0, s>>>(partial, n, p, (int)chunks, mean);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t corr_normalize(double *C, int p, double *sd, int num_sms, cudaStream_t s) {
    diag_sqrt_kernel<<<(p + 127) / 128, 128, 0, s>>>(C, p, sd);
    note_launch(1);
    normalize_kernel<<<num_sms * 4, 256, 0, s>>>(C, p, sd);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t corr_f64(const void *X, int dtype, long long n, int p, long long ldx, double *C, void *ws,
                     size_t ws_bytes, int num_sms, cudaStream_t s) {
    if (dtype == GCSL_DTYPE_F64)
        return corr_impl<double>(static_cast<const double *>(X), n, p, ldx, C, ws, ws_bytes, num_sms, s);
    return corr_impl<float>(static_cast<const float *>(X), n, p, ldx, C, ws, ws_bytes, num_sms, s);
}

}  // namespace host
}  // namespace gcsl
