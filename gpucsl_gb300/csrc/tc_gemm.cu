// Tensor-core (tcgen05) GEMM kernels.
//
// tc_gemm_bf16_kernel: D = A B^T with A (M x K) and B (N x K) BF16 row-major (both
// K-major), D FP32 row-major; one CTA of 128 threads per 128 x 128 output tile, the
// accumulator in 128 TMEM columns, K consumed in 64-wide slabs (four 128x128x16 MMAs
// issued by one thread).  It is the unit building block that the correlation kernels
// reuse; the parity test compares it with an exact integer product.
#include "common.cuh"
#include "tc.cuh"

namespace gcsl {

constexpr int TC_TM = 128, TC_TN = 128, TC_TK = 64;
constexpr uint32_t TC_TMEM_COLS = 128;
constexpr unsigned long long TC_WAIT_NS = 2000000000ull;  // 2 s per wait, then error out

__global__ void __launch_bounds__(128) tc_gemm_bf16_kernel(const uint16_t *__restrict__ A,
                                                          const uint16_t *__restrict__ B, float *__restrict__ D,
                                                          int M, int N, int K, int *err) {
    __shared__ __align__(1024) uint8_t sA[TC_TM * TC_TK * 2];
    __shared__ __align__(1024) uint8_t sB[TC_TN * TC_TK * 2];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * TC_TM, n0 = blockIdx.x * TC_TN;
    if (warp == 0) tc::tmem_alloc(&tmem_slot, TC_TMEM_COLS);
    if (tid == 0) tc::mbar_init(&mbar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = tc::idesc_bf16_f32(TC_TM, TC_TN);
    bool ok = true;
    uint32_t phase = 0;
    for (int k0 = 0; k0 < K; k0 += TC_TK) {
        // stage the 128 x 64 slabs of A and B: 16-byte chunks (8 elements along K)
        for (int c = tid; c < TC_TM * (TC_TK / 8); c += 128) {
            const int m = c / (TC_TK / 8), k = (c % (TC_TK / 8)) * 8;
            const uint32_t off = (uint32_t)(k / 16) * 4096u + tc::kmajor_offset(m, k % 16);
            *reinterpret_cast<uint4 *>(sA + off) =
                __ldg(reinterpret_cast<const uint4 *>(A + (size_t)(m0 + m) * K + k0 + k));
            *reinterpret_cast<uint4 *>(sB + off) =
                __ldg(reinterpret_cast<const uint4 *>(B + (size_t)(n0 + m) * K + k0 + k));
        }
        tc::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc::fence_after_sync();
#pragma unroll
            for (int s = 0; s < TC_TK / 16; ++s) {
                const uint64_t ad = tc::sdesc(tc::smem_u32(sA + s * 4096), 128, 256);
                const uint64_t bd = tc::sdesc(tc::smem_u32(sB + s * 4096), 128, 256);
                tc::mma_bf16(tmem, ad, bd, idesc, (k0 > 0 || s > 0) ? 1u : 0u);
            }
            tc::mma_commit(&mbar);
        }
        if (!tc::mbar_wait(&mbar, phase, TC_WAIT_NS)) ok = false;
        phase ^= 1u;
        if (!__syncthreads_and(ok)) {
            ok = false;
            break;
        }
    }
    tc::fence_after_sync();
    if (ok) {
        const int row = warp * 32 + lane;
#pragma unroll 1
        for (int c = 0; c < TC_TN; c += 16) {
            float v[16];
            tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c, v);
            float *dst = D + (size_t)(m0 + row) * N + n0 + c;
#pragma unroll
            for (int i = 0; i < 16; ++i) dst[i] = v[i];
        }
    } else if (tid == 0) {
        atomicExch(err, 1);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TC_TMEM_COLS);
}

namespace host {
cudaError_t launch_tc_gemm_bf16(const uint16_t *A, const uint16_t *B, float *D, int M, int N, int K, int *err,
                                cudaStream_t s) {
    dim3 grid(N / TC_TN, M / TC_TM);
    tc_gemm_bf16_kernel<<<grid, 128, 0, s>>>(A, B, D, M, N, K, err);
    note_launch(1);
    return cudaGetLastError();
}
}  // namespace host
}  // namespace gcsl
