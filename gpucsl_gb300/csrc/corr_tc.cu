// Correlation matrix on the tensor cores with FP64 accuracy (kernel a, plain path).
//
// FP64 runs on GB300's CUDA cores at a small fraction of the BF16 tensor rate, so the
// FP64 product X_c^T X_c is formed from exact integer pieces on the tcgen05 tensor
// cores (the error-free splitting of Ozaki et al., restated for this kernel):
//
//  1. centre each column in FP64 (x - mean, rounded as numpy does) and scale it by a
//     power of two so |y| < 1;  I = round(y * 2^49) is an integer of at most 50 bits;
//  2. split I = sum_k d_k 2^(7 (6 - k)), k = 0..6, into signed 7-bit digits
//     (|d_0| <= 128, |d_k| <= 64): every digit is exact in BF16;
//  3. for each digit pair with k + l = g <= 6 accumulate d_k^T d_l on the tensor core
//     into accumulator g (FP32 in TMEM).  Products are at most 2^14 and a group sums at
//     most (g + 3) 2^12 per sample, so over 448 samples every partial sum stays below
//     2^24: the FP32 accumulators hold exact integers;
//  4. every 448 samples the 7 accumulators are drained into two int64 words per output
//     (groups 0-2 weighted 2^14, 2^7, 1 and groups 3-6 weighted 2^21 .. 1); split-K
//     partial words are summed exactly, and the value 2^28 hi + lo is rounded to FP64
//     once.
//
// Dropped pairs (k + l > 6) weigh at most 2^-48 of sum |x_i||x_j|, the same order as
// the rounding of an FP64 GEMM.  Tile: 128 rows (i) x 64 columns (j), 7 accumulators
// = 448 TMEM columns, K staged 32 samples at a time into two shared-memory buffers
// (84 KB each) while the tensor core consumes the other.
#include "common.cuh"
#include "tc.cuh"

namespace gcsl {

constexpr int OZ_S = 7;                 // digits per value
constexpr int OZ_G = 7;                 // accumulator groups g = k + l <= 6
constexpr int OZ_PAIRS = 28;            // pairs with k + l <= 6
constexpr int OZ_TM = 128, OZ_TN = 64;  // output tile
constexpr int OZ_KS = 32;               // sample padding granule
constexpr int OZ_CHUNK_STEPS = 28;      // 448 samples (28 MMA K steps) between exact drains
constexpr int OZ_NST = 4;               // shared-memory stages (one K step each)
constexpr uint32_t OZ_TMEM_COLS = 512;
constexpr int OZ_A_BYTES = OZ_S * OZ_TM * 16 * 2;  // 28672: 7 digits x 128 rows x 16 samples
constexpr int OZ_B_BYTES = OZ_S * OZ_TN * 16 * 2;  // 14336: 7 digits x 64 rows x 16 samples
constexpr int OZ_STAGE_BYTES = OZ_A_BYTES + OZ_B_BYTES;
constexpr unsigned long long OZ_WAIT_NS = 2000000000ull;

struct OzDims {
    int p, p_pad, n_pad, n_tiles_j, splits, slabs_per_split;  // slabs_per_split counts 16-sample K steps
};

// ------------------------------------------------------------ preparation
// Order-preserving signed key of a double (negative values have their magnitude bits
// flipped), so min / max can be taken with 64-bit integer atomics.
__device__ __forceinline__ long long ordered_key(double x) {
    long long k = __double_as_longlong(x);
    return k < 0 ? (k ^ 0x7fffffffffffffffll) : k;
}
__device__ __forceinline__ double key_value(long long k) {
    return __longlong_as_double(k < 0 ? (k ^ 0x7fffffffffffffffll) : k);
}

constexpr int OZ_STAT_ROWS = 512;  // samples per column-statistics block

__global__ void colstats_init_kernel(int p, long long *__restrict__ kmin, long long *__restrict__ kmax) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < p) {
        kmin[j] = 0x7fffffffffffffffll;
        kmax[j] = (long long)0x8000000000000000ull;
    }
}

// One read of X: per (512-sample chunk, column) FP64 partial sum in a fixed order, and
// column min / max through ordered-key atomics.
template <typename T>
__global__ void colstats_kernel(const T *__restrict__ X, long long n, int p, long long ldx,
                                double *__restrict__ partial, long long *__restrict__ kmin,
                                long long *__restrict__ kmax) {
    __shared__ double ssum[8][32];
    __shared__ long long smin[8][32], smax[8][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int j = blockIdx.x * 32 + lane;
    const long long t0 = (long long)blockIdx.y * OZ_STAT_ROWS, t1 = min(n, t0 + OZ_STAT_ROWS);
    double sum = 0.0;
    long long mn = 0x7fffffffffffffffll, mx = (long long)0x8000000000000000ull;
    if (j < p) {
        for (long long t = t0 + w; t < t1; t += 8) {
            const double x = (double)X[t * ldx + j];
            sum += x;
            const long long k = ordered_key(x);
            mn = k < mn ? k : mn;
            mx = k > mx ? k : mx;
        }
    }
    ssum[w][lane] = sum;
    smin[w][lane] = mn;
    smax[w][lane] = mx;
    __syncthreads();
    if (w == 0 && j < p) {
        for (int q = 1; q < 8; ++q) {
            sum += ssum[q][lane];
            mn = smin[q][lane] < mn ? smin[q][lane] : mn;
            mx = smax[q][lane] > mx ? smax[q][lane] : mx;
        }
        partial[(size_t)blockIdx.y * p + j] = sum;
        atomicMin(&kmin[j], mn);
        atomicMax(&kmax[j], mx);
    }
}

// mean = (chunk sums in order) / n; E = exponent of max |fl(x - mean)| =
// max(fl(max - mean), fl(mean - min)) (rounding is monotone), so |x - mean| < 2^E.
__global__ void col_mean_exp_kernel(const double *__restrict__ partial, long long n, int p, int chunks,
                                    const long long *__restrict__ kmin, const long long *__restrict__ kmax,
                                    double *__restrict__ mean, int *__restrict__ expo) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= p) return;
    double s = 0.0;
    for (int c = 0; c < chunks; ++c) s += partial[(size_t)c * p + j];
    const double mu = s / (double)n;
    mean[j] = mu;
    const double dev = fmax(key_value(kmax[j]) - mu, mu - key_value(kmin[j]));
    int e = 0;
    if (dev > 0.0) frexp(dev, &e);
    expo[j] = e;
}

// Digits of X_c in the tensor-core tile layout: for digit k, 128-row block I and
// 16-sample K step q, a 4 KB block in the canonical no-swizzle K-major layout
// (byte ((k * nI + I) * nq + q) * 4096 + kmajor_offset(row % 128, sample % 16)), zero
// padded to (p_pad, n_pad).  A 64-row operand tile is the first or second 2 KB half of a
// block.  One CTA handles 32 samples x 32 columns.
template <typename T>
__global__ void digit_split_kernel(const T *__restrict__ X, long long n, int p, long long ldx,
                                   const double *__restrict__ mean, const int *__restrict__ expo, int p_pad,
                                   long long n_pad, uint8_t *__restrict__ dig) {
    __shared__ int16_t tile[OZ_S][32][33];  // [digit][sample][column]
    const long long t0 = (long long)blockIdx.x * 32;
    const int j0 = blockIdx.y * 32;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 8 warps
    for (int r = ty; r < 32; r += 8) {
        const long long t = t0 + r;
        const int j = j0 + tx;
        long long I = 0;
        if (t < n && j < p) {
            // y = fl(x - mean) as numpy centres; I = round(|y| 2^(49 - E)) with the sign of y,
            // from the bits of y: |y| = m 2^(ey - 1075), so I = round(m 2^(ey - 1075 + 49 - E)).
            const double y = (double)X[t * ldx + j] - mean[j];
            const long long bits = __double_as_longlong(y);
            const int ey = (int)((bits >> 52) & 0x7ff);
            long long m = bits & 0xfffffffffffffll;
            if (ey != 0) m |= 1ll << 52;
            const int sh = 1075 - (ey != 0 ? ey : 1) - 49 + expo[j];  // right shift, >= 4 since |y| < 2^E
            long long mag = 0;
            if (sh < 63) mag = (m + (1ll << (sh - 1))) >> sh;
            I = bits < 0 ? -mag : mag;
        }
        long long rem = I;
#pragma unroll
        for (int k = 0; k < OZ_S - 1; ++k) {
            const int sh = 7 * (OZ_S - 1 - k);
            const long long d = (rem + (1ll << (sh - 1))) >> sh;  // round half up (arithmetic shift)
            rem -= d * (1ll << sh);
            tile[k][r][tx] = (int16_t)d;
        }
        tile[OZ_S - 1][r][tx] = (int16_t)rem;
    }
    __syncthreads();
    const int nI = p_pad / OZ_TM;
    const long long nq = n_pad / 16;
    // 16-byte chunks: (digit k, column c, 8-sample group g8 in 0..3)
    for (int w = threadIdx.x; w < OZ_S * 32 * 4; w += blockDim.x) {
        const int k = w / 128, c = (w / 4) % 32, g8 = w % 4;
        const int j = j0 + c;
        const long long t = t0 + g8 * 8;
        if (j >= p_pad || t >= n_pad) continue;
        uint32_t word[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float lo = (float)tile[k][g8 * 8 + 2 * e][c], hi = (float)tile[k][g8 * 8 + 2 * e + 1][c];
            word[e] = (__float_as_uint(lo) >> 16) | (__float_as_uint(hi) & 0xffff0000u);  // exact BF16 pair
        }
        const long long q = t / 16;
        const size_t off = (((size_t)k * nI + j / OZ_TM) * nq + q) * 4096 +
                           tc::kmajor_offset((uint32_t)(j % OZ_TM), (uint32_t)(t % 16));
        *reinterpret_cast<uint4 *>(dig + off) = make_uint4(word[0], word[1], word[2], word[3]);
    }
}

// ------------------------------------------------------------- tensor core
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t *r) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void oz_tile_of(int bid, int n_tiles_j, int &I, int &J) {
    // tiles (I: 128 rows, J: 64 columns) with J*64 + 63 >= I*128, i.e. J >= 2I
    int rem = bid, i = 0;
    while (rem >= n_tiles_j - 2 * i) {
        rem -= n_tiles_j - 2 * i;
        ++i;
    }
    I = i;
    J = 2 * i + rem;
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(mbar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *smem_dst, const void *gmem_src, uint32_t bytes, uint64_t *mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     tc::smem_u32(smem_dst)),
                 "l"(gmem_src), "r"(bytes), "r"(tc::smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(tc::smem_u32(mbar)) : "memory");
}

// Bounded wait that reads the timer only every 256 polls.
__device__ __forceinline__ bool mbar_wait_fast(uint64_t *mbar, uint32_t phase) {
    const uint32_t addr = tc::smem_u32(mbar);
    unsigned long long t0 = 0;
    for (uint32_t it = 0;; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(addr), "r"(phase)
            : "memory");
        if (done) return true;
        if ((it & 255u) == 0) {
            const unsigned long long now = tc::globaltimer_ns();
            if (it == 0) t0 = now;
            else if (now - t0 > OZ_WAIT_NS) return false;
        }
    }
}

constexpr int OZ_DRAIN_WARPS = 16;                       // 4 TMEM lane quarters x 4 column quarters
constexpr int OZ_THREADS = (OZ_DRAIN_WARPS + 2) * 32;    // + producer warp + MMA warp

// Warp roles: warps 0..15 drain TMEM into 64-bit integer accumulators at every chunk
// end; warp 16 (lane 0) streams digit blocks into the shared-memory stages with bulk
// copies; warp 17 (lane 0) issues the tensor-core MMAs.  They synchronise only through
// mbarriers: full (copy landed), empty (MMAs done reading a stage), chunk (MMAs of a
// chunk done), drained (TMEM read, accumulators may be overwritten).
__global__ void __launch_bounds__(OZ_THREADS, 1) corr_ozaki_kernel(const uint8_t *__restrict__ dig, OzDims D,
                                                                  long long *__restrict__ part_hi,
                                                                  long long *__restrict__ part_lo, int *err) {
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t full_bar[OZ_NST], empty_bar[OZ_NST], chunk_bar, drained_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    int I, J;
    oz_tile_of(blockIdx.x, D.n_tiles_j, I, J);
    const int split = blockIdx.y;
    const int nI = D.p_pad / OZ_TM;
    const long long nq = D.n_pad / 16;
    const long long q0 = (long long)split * D.slabs_per_split;
    const long long nst = min(q0 + (long long)D.slabs_per_split, nq) - q0;  // K steps of this split
    const int nchunks = (int)((nst + OZ_CHUNK_STEPS - 1) / OZ_CHUNK_STEPS);

    if (warp == 0) tc::tmem_alloc(&tmem_slot, OZ_TMEM_COLS);
    if (tid == 0) {
        for (int b = 0; b < OZ_NST; ++b) {
            tc::mbar_init(&full_bar[b], 1);
            tc::mbar_init(&empty_bar[b], 1);
        }
        tc::mbar_init(&chunk_bar, 1);
        tc::mbar_init(&drained_bar, OZ_DRAIN_WARPS);
        s_fail = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;

    if (warp == OZ_DRAIN_WARPS) {
        // ---------------- producer
        if (lane == 0) {
            for (long long st = 0; st < nst; ++st) {
                const int b = (int)(st % OZ_NST);
                if (st >= OZ_NST && !mbar_wait_fast(&empty_bar[b], (uint32_t)(((st / OZ_NST) - 1) & 1))) {
                    atomicExch(&s_fail, 1);
                    break;
                }
                if (*(volatile int *)&s_fail) break;
                uint8_t *sA = smem + (size_t)b * OZ_STAGE_BYTES;
                uint8_t *sB = sA + OZ_A_BYTES;
                mbar_expect_tx(&full_bar[b], (uint32_t)OZ_STAGE_BYTES);
                const long long q = q0 + st;
                for (int k = 0; k < OZ_S; ++k) {
                    bulk_g2s(sA + k * 4096, dig + (((size_t)k * nI + I) * nq + q) * 4096, 4096u, &full_bar[b]);
                    bulk_g2s(sB + k * 2048,
                             dig + (((size_t)k * nI + (J >> 1)) * nq + q) * 4096 + (size_t)(J & 1) * 2048, 2048u,
                             &full_bar[b]);
                }
            }
        }
    } else if (warp == OZ_DRAIN_WARPS + 1) {
        // ---------------- MMA issuer
        if (lane == 0) {
            for (int c = 0; c < nchunks; ++c) {
                if (c > 0 && !mbar_wait_fast(&drained_bar, (uint32_t)((c - 1) & 1))) {
                    atomicExch(&s_fail, 1);
                    break;
                }
                tc::fence_after_sync();
                const long long c0 = (long long)c * OZ_CHUNK_STEPS, c1 = min(c0 + OZ_CHUNK_STEPS, nst);
                bool bad = false;
                for (long long st = c0; st < c1; ++st) {
                    const int b = (int)(st % OZ_NST);
                    if (!mbar_wait_fast(&full_bar[b], (uint32_t)((st / OZ_NST) & 1))) {
                        bad = true;
                        break;
                    }
                    tc::fence_after_sync();
                    uint8_t *sA = smem + (size_t)b * OZ_STAGE_BYTES;
                    uint8_t *sB = sA + OZ_A_BYTES;
                    // Digit k of A against digits l = 0 .. 6-k of B: the B digits are
                    // consecutive 64-row operands in shared memory and the products land in
                    // consecutive accumulator groups g = k + l (TMEM columns 64 g ..), so up
                    // to four pairs form one MMA with N = 64 x (number of pairs).
#pragma unroll
                    for (int k = 0; k < OZ_S; ++k) {
                        const uint64_t ad = tc::sdesc(tc::smem_u32(sA + k * 4096), 128, 256);
                        const int pairs = OZ_S - k;
                        const uint32_t acc = (st == c0 && k == 0) ? 0u : 1u;  // k = 0 writes every group first
#pragma unroll
                        for (int l0 = 0; l0 < pairs; l0 += 4) {
                            const int cnt = (pairs - l0) < 4 ? (pairs - l0) : 4;
                            const uint64_t bd = tc::sdesc(tc::smem_u32(sB + l0 * 2048), 128, 256);
                            tc::mma_bf16(tmem + (uint32_t)((k + l0) * OZ_TN), ad, bd,
                                         tc::idesc_bf16_f32(OZ_TM, OZ_TN * cnt), acc);
                        }
                    }
                    tc::mma_commit(&empty_bar[b]);
                }
                if (bad) {
                    atomicExch(&s_fail, 1);
                    break;
                }
                tc::mma_commit(&chunk_bar);
            }
        }
    } else {
        // ---------------- drain warps
        const int qd = warp & 3, cq = warp >> 2;  // TMEM lane quarter, column quarter
        long long acc_hi[16], acc_lo[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) acc_hi[c] = acc_lo[c] = 0;
        bool ok = true;
        for (int c = 0; c < nchunks; ++c) {
            if (!mbar_wait_fast(&chunk_bar, (uint32_t)(c & 1))) {
                ok = false;
                break;
            }
            tc::fence_after_sync();
            // groups 0..2 -> hi with weights 2^14, 2^7, 1; groups 3..6 -> lo with 2^21, 2^14, 2^7, 1
#pragma unroll
            for (int g = 0; g < OZ_G; ++g) {
                float v[16];
                tc::tmem_ld16(tmem + ((uint32_t)(qd * 32) << 16) + (uint32_t)(g * OZ_TN + cq * 16), v);
                const long long wgt = 1ll << (7 * ((g < 3 ? 2 : 6) - g));
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    const long long x = (long long)__float2int_rn(v[e]) * wgt;
                    if (g < 3) acc_hi[e] += x;
                    else acc_lo[e] += x;
                }
            }
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) mbar_arrive(&drained_bar);
        }
        if (!ok) atomicExch(&s_fail, 1);
        __syncwarp();
        if (ok) {
            const int row = qd * 32 + lane;
            const size_t base = ((size_t)split * D.p_pad + (size_t)(I * OZ_TM + row)) * D.p_pad + J * OZ_TN + cq * 16;
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                part_hi[base + e] = acc_hi[e];
                part_lo[base + e] = acc_lo[e];
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0 && s_fail) atomicExch(err, 1);
    if (warp == 0) tc::tmem_dealloc(tmem, OZ_TMEM_COLS);
}

__device__ __forceinline__ double pow2(int e) { return __longlong_as_double((long long)(1023 + e) << 52); }

// Covariance of (i, j) from the exact split sums: (2^28 H + L) 2^(E_i + E_j - 56) / (n - 1).
__device__ __forceinline__ double oz_cov(const long long *__restrict__ part_hi, const long long *__restrict__ part_lo,
                                         const OzDims &D, const int *__restrict__ expo, double scale, int i, int j) {
    long long H = 0, Lo = 0;
    for (int s = 0; s < D.splits; ++s) {
        const size_t ix = ((size_t)s * D.p_pad + i) * D.p_pad + j;
        H += part_hi[ix];
        Lo += part_lo[ix];
    }
    const double val = fma((double)H, 268435456.0, (double)Lo);  // exact terms, one rounding
    return (val * pow2(expo[i] + expo[j] - 56)) * scale;
}

__global__ void ozaki_diag_kernel(const long long *__restrict__ part_hi, const long long *__restrict__ part_lo,
                                  OzDims D, const int *__restrict__ expo, double scale, double *__restrict__ inv_sd) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < D.p) inv_sd[i] = 1.0 / sqrt(oz_cov(part_hi, part_lo, D, expo, scale, i, i));
}

// C_ij = clip(cov_ij / s_i / s_j, -1, 1) for i <= j, written to both triangles (the
// normalisation of numpy's corrcoef, with reciprocals of the standard deviations).
__global__ void ozaki_finish_kernel(const long long *__restrict__ part_hi, const long long *__restrict__ part_lo,
                                    OzDims D, const int *__restrict__ expo, double scale,
                                    const double *__restrict__ inv_sd, const int *__restrict__ err,
                                    double *__restrict__ C) {
    const long long total = (long long)D.p * D.p;
    const bool failed = *err != 0;  // a tensor-core wait timed out: poison the output
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(k / D.p), j = (int)(k - (long long)i * D.p);
        if (i > j) continue;
        double v = oz_cov(part_hi, part_lo, D, expo, scale, i, j) * inv_sd[i] * inv_sd[j];
        v = fmin(fmax(v, -1.0), 1.0);
        if (failed) v = __longlong_as_double(0x7ff8000000000000ll);
        C[(size_t)i * D.p + j] = v;
        C[(size_t)j * D.p + i] = v;
    }
}

namespace host {

static OzDims oz_dims(long long n, int p, int num_sms) {
    OzDims D;
    D.p = p;
    D.p_pad = (p + OZ_TM - 1) / OZ_TM * OZ_TM;
    D.n_pad = (int)((n + OZ_KS - 1) / OZ_KS * OZ_KS);
    D.n_tiles_j = D.p_pad / OZ_TN;
    const int n_tiles_i = D.p_pad / OZ_TM;
    int tiles = 0;
    for (int i = 0; i < n_tiles_i; ++i) tiles += D.n_tiles_j - 2 * i;
    const long long steps = D.n_pad / 16;
    int splits = num_sms / tiles;  // one wave: tiles x splits <= SMs (one CTA per SM holds all TMEM)
    if (splits < 1) splits = 1;
    if (splits > steps) splits = (int)steps;
    D.slabs_per_split = (int)((steps + splits - 1) / splits);
    D.splits = (int)((steps + D.slabs_per_split - 1) / D.slabs_per_split);
    return D;
}

static int oz_tiles(const OzDims &D) {
    int tiles = 0;
    for (int i = 0; i < D.p_pad / OZ_TM; ++i) tiles += D.n_tiles_j - 2 * i;
    return tiles;
}

struct OzWs {
    double *partial, *mean, *inv_sd;
    long long *kmin, *kmax;
    int *expo, *err;
    uint8_t *dig;
    long long *phi, *plo;
    size_t bytes;
};

static OzWs oz_carve(void *ws, long long n, int p, const OzDims &D) {
    const long long chunks = (n + OZ_STAT_ROWS - 1) / OZ_STAT_ROWS;
    char *w = static_cast<char *>(ws);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *r = w ? w + off : nullptr;
        off += (bytes + 255) / 256 * 256;
        return r;
    };
    OzWs o;
    o.partial = reinterpret_cast<double *>(take((size_t)(chunks * p) * sizeof(double)));
    o.mean = reinterpret_cast<double *>(take((size_t)p * sizeof(double)));
    o.inv_sd = reinterpret_cast<double *>(take((size_t)p * sizeof(double)));
    o.kmin = reinterpret_cast<long long *>(take((size_t)p * sizeof(long long)));
    o.kmax = reinterpret_cast<long long *>(take((size_t)p * sizeof(long long)));
    o.expo = reinterpret_cast<int *>(take((size_t)p * sizeof(int)));
    o.err = reinterpret_cast<int *>(take(sizeof(int)));
    o.dig = reinterpret_cast<uint8_t *>(take((size_t)OZ_S * D.p_pad * (size_t)D.n_pad * sizeof(uint16_t)));
    o.phi = reinterpret_cast<long long *>(take((size_t)D.splits * D.p_pad * (size_t)D.p_pad * sizeof(long long) * 2));
    o.plo = o.phi ? o.phi + (size_t)D.splits * D.p_pad * (size_t)D.p_pad : nullptr;
    o.bytes = off;
    return o;
}

size_t corr_tc_workspace_bytes(long long n, int p, int num_sms) {
    const OzDims D = oz_dims(n, p, num_sms);
    return oz_carve(nullptr, n, p, D).bytes;
}

// Stage 1: column statistics, exponents and the digit tiles (FP64 / integer work).
cudaError_t corr_tc_digits(const void *X, int dtype, long long n, int p, long long ldx, void *ws, size_t ws_bytes,
                           int num_sms, cudaStream_t s) {
    const OzDims D = oz_dims(n, p, num_sms);
    const OzWs o = oz_carve(ws, n, p, D);
    if (ws_bytes < o.bytes) return cudaErrorInvalidValue;
    const long long chunks = (n + OZ_STAT_ROWS - 1) / OZ_STAT_ROWS;
    cudaError_t e = cudaMemsetAsync(o.err, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    colstats_init_kernel<<<(p + 255) / 256, 256, 0, s>>>(p, o.kmin, o.kmax);
    note_launch(1);
    const dim3 gs((p + 31) / 32, (unsigned)chunks);
    const dim3 gd((unsigned)(D.n_pad / 32), (unsigned)(D.p_pad / 32));
    if (dtype == GCSL_DTYPE_F64)
        colstats_kernel<double><<<gs, 256, 0, s>>>(static_cast<const double *>(X), n, p, ldx, o.partial, o.kmin,
                                                   o.kmax);
    else
        colstats_kernel<float><<<gs, 256, 0, s>>>(static_cast<const float *>(X), n, p, ldx, o.partial, o.kmin,
                                                  o.kmax);
    note_launch(1);
    col_mean_exp_kernel<<<(p + 255) / 256, 256, 0, s>>>(o.partial, n, p, (int)chunks, o.kmin, o.kmax, o.mean,
                                                        o.expo);
    note_launch(1);
    if (dtype == GCSL_DTYPE_F64)
        digit_split_kernel<double><<<gd, 256, 0, s>>>(static_cast<const double *>(X), n, p, ldx, o.mean, o.expo,
                                                       D.p_pad, D.n_pad, o.dig);
    else
        digit_split_kernel<float><<<gd, 256, 0, s>>>(static_cast<const float *>(X), n, p, ldx, o.mean, o.expo,
                                                      D.p_pad, D.n_pad, o.dig);
    note_launch(1);
    return cudaGetLastError();
}

// Stage 2: exact digit products on the tensor cores, reduction, normalisation.
cudaError_t corr_tc_product(long long n, int p, double *C, void *ws, size_t ws_bytes, int num_sms, cudaStream_t s) {
    const OzDims D = oz_dims(n, p, num_sms);
    const OzWs o = oz_carve(ws, n, p, D);
    if (ws_bytes < o.bytes) return cudaErrorInvalidValue;
    const int smem = OZ_NST * OZ_STAGE_BYTES;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(corr_ozaki_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        attr = true;
    }
    dim3 grid(oz_tiles(D), D.splits);
    corr_ozaki_kernel<<<grid, OZ_THREADS, smem, s>>>(o.dig, D, o.phi, o.plo, o.err);
    note_launch(1);
    const double scale = 1.0 / (double)(n - 1);
    ozaki_diag_kernel<<<(p + 255) / 256, 256, 0, s>>>(o.phi, o.plo, D, o.expo, scale, o.inv_sd);
    note_launch(1);
    ozaki_finish_kernel<<<num_sms * 4, 256, 0, s>>>(o.phi, o.plo, D, o.expo, scale, o.inv_sd, o.err, C);
    note_launch(1);
    return cudaGetLastError();
}

cudaError_t corr_tc(const void *X, int dtype, long long n, int p, long long ldx, double *C, void *ws, size_t ws_bytes,
                    int num_sms, int *unused, cudaStream_t s) {
    (void)unused;
    cudaError_t e = corr_tc_digits(X, dtype, n, p, ldx, ws, ws_bytes, num_sms, s);
    if (e != cudaSuccess) return e;
    return corr_tc_product(n, p, C, ws, ws_bytes, num_sms, s);
}

}  // namespace host
}  // namespace gcsl
