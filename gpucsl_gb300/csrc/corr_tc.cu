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
// = 448 TMEM columns, K staged 16 samples at a time into a ring of shared-memory stages
// while the tensor core consumes the others.
//
// Split precision (batches): the same product over the five leading digits only, pairs
// k + l <= 4 (15 of the 28 pair products, 5 accumulators), gives C' with
//   |C' - C| <= eps = 2.5 * 2^-35 * (1.02 w + sqrt(w)),  w = n / min_i sum_t y_ti^2,
// where C is the seven-digit result (derivation at split_eps below); the diagonal
// kernel writes eps per instance.  Instances whose tests cannot be decided exactly with
// C' are flagged by the level loop and get the seven-digit product afterwards (the split
// run writes five digit planes; the flagged jobs' seven are written by that later run).
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

#include <cuda.h>

#include "common.cuh"
#include "tc.cuh"

namespace gcsl {

constexpr int OZ_S = 7;                 // digits per value (all written by the digit split)
constexpr int OZ_S_SPLIT = 5;           // digits of the split-precision product
constexpr int OZ_TM = 128, OZ_TN = 64;  // output tile
constexpr int OZ_KS = 32;               // sample padding granule
constexpr int OZ_CHUNK_STEPS = 28;      // 448 samples (28 MMA K steps) between exact drains
constexpr uint32_t OZ_TMEM_COLS = 512;
// shared-memory bytes of one K step for NS digits: NS x (128 A rows + 64 B rows) x 16
// samples x 2 bytes (NS = 7: 28672 + 14336)
constexpr int oz_a_bytes(int ns) { return ns * OZ_TM * 16 * 2; }
constexpr int oz_stage_bytes(int ns) { return ns * (OZ_TM + OZ_TN) * 16 * 2; }
// Shared-memory stages of the copy ring (one K step each): as many as 210 KB hold, so the
// copies run as far ahead of the MMAs as the SM allows (5 for seven digits, 7 for five).
// Four stages measured the same: the copies' latency is not what idles the tensor pipe.
constexpr int OZ_RING_BYTES = 215040;
constexpr int OZ_NST_MAX = 8;
constexpr int oz_nst(int ns) { return OZ_RING_BYTES / oz_stage_bytes(ns) < OZ_NST_MAX ? OZ_RING_BYTES / oz_stage_bytes(ns)
                                                                                      : OZ_NST_MAX; }
constexpr unsigned long long OZ_WAIT_NS = 2000000000ull;

struct OzDims {
    int p, p_pad, n_pad, n_tiles_j, splits, slabs_per_split;  // slabs_per_split counts 16-sample K steps
};

// One correlation job: input samples, its dimensions and its slice of the workspace.
struct OzJob {
    const void *X;
    long long n, ldx;
    int p, chunks, tiles, pad;
    OzDims D;
    double *partial, *mean, *inv_sd;
    long long *kmin, *kmax;
    int *expo, *err;
    uint8_t *dig;
    long long *phi, *plo;
    double *C;
    float *C32;  // optional FP32 copy of C
    int index;   // position in its batch (0 for a single job)
};

// Kernel stages of a job; each has its own count of blocks per job.
enum OzStage { OZ_INIT = 0, OZ_STATS, OZ_MEAN, OZ_DIGITS, OZ_PRODUCT, OZ_DIAG, OZ_FINISH, OZ_NSTAGES };

// Where a kernel finds its job: one job passed by value (block b of the stage is block b
// of the job), or a device table of jobs with each stage's exclusive block offsets
// (block b belongs to the job k with off[k] <= b < off[k + 1]).
//
// A batch run may also carry, per job index: c_err, where the split-precision diagonal
// kernel writes the bound eps of the job's C (null: exact product, no bound), and
// active, the jobs to compute (null: all; a job whose flag is 0 is skipped by the
// product, diagonal and finish kernels).
struct OneJob {
    OzJob job;
    __device__ __forceinline__ OzJob get(long long b, long long &lb) const {
        lb = b;
        return job;
    }
    // also the first block index past the job's blocks in the stage (unbounded here)
    __device__ __forceinline__ OzJob get(long long b, long long &lb, long long &end) const {
        lb = b;
        end = 0x7fffffffffffffffll;
        return job;
    }
    __device__ __forceinline__ bool skip(int) const { return false; }
    __device__ __forceinline__ double *err_slot(int) const { return nullptr; }
};
struct JobTable {
    const OzJob *jobs;
    const long long *off;
    int count;
    double *c_err = nullptr;
    const int *active = nullptr;
    // per job, in device memory: the tensor maps of its digit planes for the product,
    // [A, B] with all seven planes then [A, B] with the split product's five (or null:
    // the product copies with bulk copies)
    const CUtensorMap *maps = nullptr;
    __device__ __forceinline__ OzJob get(long long b, long long &lb) const {
        const int k = upper_row(off, count, b);
        lb = b - off[k];
        return jobs[k];
    }
    __device__ __forceinline__ OzJob get(long long b, long long &lb, long long &end) const {
        const int k = upper_row(off, count, b);
        lb = b - off[k];
        end = off[k + 1];
        return jobs[k];
    }
    __device__ __forceinline__ bool skip(int index) const { return active != nullptr && active[index] == 0; }
    __device__ __forceinline__ double *err_slot(int index) const {
        return c_err != nullptr ? c_err + index : nullptr;
    }
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

template <class Src>
__global__ void colstats_init_kernel(Src src) {
    pdl_wait();
    pdl_trigger();
    long long lb;
    const OzJob &J = src.get(blockIdx.x, lb);
    const int j = (int)lb * blockDim.x + threadIdx.x;
    if (j < J.p) {
        J.kmin[j] = 0x7fffffffffffffffll;
        J.kmax[j] = (long long)0x8000000000000000ull;
        if (j == 0) {
            *J.err = 0;
            double *slot = src.err_slot(J.index);
            if (slot != nullptr) *slot = 0.0;
        }
    }
}

// Persistent blocks over the `total` blocks of a stage: grid block b takes the contiguous
// range [b per, (b + 1) per) and looks up the job once for each job its range enters
// (thread 0, shared with the block through s_job), so a stage of millions of small
// blocks (a batch's digit tiles) costs one job search per job and grid block rather than
// one per block.  body(job, lb) runs for every block of the range with the whole block
// and must end with a __syncthreads() when it reuses shared memory.
template <class Src, class Body>
__device__ __forceinline__ void stage_blocks(const Src &src, long long total, OzJob &s_job, long long (&s_rng)[2],
                                             Body &&body) {
    const long long per = (total + gridDim.x - 1) / gridDim.x;
    long long b = (long long)blockIdx.x * per;
    const long long b1 = min(total, b + per);
    while (b < b1) {
        if (threadIdx.x == 0) {
            long long lb, end;
            s_job = src.get(b, lb, end);
            s_rng[0] = lb;
            s_rng[1] = end;
        }
        __syncthreads();
        const long long lb0 = s_rng[0], stop = min(b1, s_rng[1]);
        for (long long i = 0; i < stop - b; ++i) body(s_job, lb0 + i);
        b = stop;
        __syncthreads();  // s_job is rewritten for the next job
    }
}

// One read of X: per (512-sample chunk, column) FP64 partial sum in a fixed order, and
// column min / max through ordered-key atomics.
template <typename T>
__device__ __forceinline__ void colstats_block(const OzJob &Jb, long long lb, double (*ssum)[32],
                                               long long (*smin)[32], long long (*smax)[32]) {
    const T *__restrict__ X = static_cast<const T *>(Jb.X);
    const long long n = Jb.n, ldx = Jb.ldx;
    const int p = Jb.p;
    const int nbx = (p + 31) / 32;
    const int bx = (int)(lb % nbx), by = (int)(lb / nbx);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int j = bx * 32 + lane;
    const long long t0 = (long long)by * OZ_STAT_ROWS, t1 = min(n, t0 + OZ_STAT_ROWS);
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
        Jb.partial[(size_t)by * p + j] = sum;
        atomicMin(&Jb.kmin[j], mn);
        atomicMax(&Jb.kmax[j], mx);
    }
    __syncthreads();  // the shared partials are reused by the next block of the range
}

// A single job: one block per stage block, the job from the kernel parameter; a batch:
// persistent blocks over the stage (stage_blocks).
template <typename T, class Src>
__global__ void colstats_kernel(Src src, long long total) {
    __shared__ double ssum[8][32];
    __shared__ long long smin[8][32], smax[8][32];
    pdl_wait();
    pdl_trigger();
    if constexpr (std::is_same<Src, OneJob>::value) {
        (void)total;
        colstats_block<T>(src.job, blockIdx.x, ssum, smin, smax);
    } else {
        __shared__ OzJob s_job;
        __shared__ long long s_rng[2];
        stage_blocks(src, total, s_job, s_rng,
                     [&](const OzJob &J, long long lb) { colstats_block<T>(J, lb, ssum, smin, smax); });
    }
}

// mean = (chunk sums in order) / n; E = exponent of max |fl(x - mean)| =
// max(fl(max - mean), fl(mean - min)) (rounding is monotone), so |x - mean| < 2^E.
template <class Src>
__global__ void col_mean_exp_kernel(Src src) {
    pdl_wait();
    pdl_trigger();
    long long lb;
    const OzJob &J = src.get(blockIdx.x, lb);
    const int p = J.p;
    const int j = (int)lb * blockDim.x + threadIdx.x;
    if (j >= p) return;
    double s = 0.0;
    for (int c = 0; c < J.chunks; ++c) s += J.partial[(size_t)c * p + j];
    const double mu = s / (double)J.n;
    J.mean[j] = mu;
    const double dev = fmax(key_value(J.kmax[j]) - mu, mu - key_value(J.kmin[j]));
    int e = 0;
    if (dev > 0.0) frexp(dev, &e);
    J.expo[j] = e;
}

// Digits of X_c in the tensor-core tile layout: for digit k, 128-row block I and
// 16-sample K step q, a 4 KB block in the canonical no-swizzle K-major layout
// (byte ((k * nI + I) * nq + q) * 4096 + kmajor_offset(row % 128, sample % 16)), zero
// padded to (p_pad, n_pad).  A 64-row operand tile is the first or second 2 KB half of a
// block.  Only the first NW digit planes are written (the split-precision product reads
// five; the exact one seven).
//
// One block covers 32 columns x 64 samples: lane = column, warp = group of 8 consecutive
// samples, so a thread owns one 16-byte row of a core matrix per digit (8 samples of one
// column).  It loads its 8 samples (each load a coalesced row of 32 columns), splits
// them, packs each digit's 8 BF16 values and stores the 16 bytes: no shared memory and
// no barrier.
constexpr int OZ_DIG_SAMPLES = 64;  // samples per digit-split block

// Two floats as one word of two BF16 values, lo in the low half (the lower address).
__device__ __forceinline__ uint32_t bf16x2_rn(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

// digit-split blocks of a job: 64-sample strips x 32-column strips
__host__ __device__ inline long long oz_digit_blocks(const OzDims &D) {
    return (long long)((D.n_pad + OZ_DIG_SAMPLES - 1) / OZ_DIG_SAMPLES) * (D.p_pad / 32);
}

template <typename T, int NW>
__device__ __forceinline__ void digit_split_block(const OzJob &Jb, long long lb) {
    const T *__restrict__ X = static_cast<const T *>(Jb.X);
    const long long n = Jb.n, ldx = Jb.ldx;
    const int p = Jb.p, p_pad = Jb.D.p_pad;
    const long long n_pad = Jb.D.n_pad;
    const long long ntx = (n_pad + OZ_DIG_SAMPLES - 1) / OZ_DIG_SAMPLES;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;  // 8 warps
    const long long tg = (lb % ntx) * OZ_DIG_SAMPLES + 8 * w;  // the thread's first sample
    const int j = (int)(lb / ntx) * 32 + lane;
    if (tg >= n_pad) return;  // the last block of a column strip may cover only 32 samples (uniform per warp)
    const bool col = j < p;
    const double mu = col ? Jb.mean[j] : 0.0;
    const int ej = col ? Jb.expo[j] : 0;
    double x[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        const long long t = tg + e;
        x[e] = (col && t < n) ? (double)X[t * ldx + j] : 0.0;
    }
    uint32_t wds[OZ_S][4];
    float fe[OZ_S];  // the digits of the even sample of the current pair
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        long long I = 0;
        if (col && tg + e < n) {
            // y = fl(x - mean) as numpy centres; I = round(|y| 2^(49 - E)) with the sign of y,
            // from the bits of y: |y| = m 2^(ey - 1075), so I = round(m 2^(ey - 1075 + 49 - E)).
            const double y = x[e] - mu;
            const long long bits = __double_as_longlong(y);
            const int ey = (int)((bits >> 52) & 0x7ff);
            long long m = bits & 0xfffffffffffffll;
            if (ey != 0) m |= 1ll << 52;
            const int sh = 1075 - (ey != 0 ? ey : 1) - 49 + ej;  // right shift, >= 4 since |y| < 2^E
            long long mag = 0;
            if (sh < 63) mag = (m + (1ll << (sh - 1))) >> sh;
            I = bits < 0 ? -mag : mag;
        }
        // digits by rounding half up (arithmetic shifts), in 32-bit arithmetic: with
        // I = H 2^21 + Lo (0 <= Lo < 2^21, |H| <= 2^28) the first three digits (weights
        // 2^42, 2^35, 2^28) round at 2^41, 2^34, 2^27, all above Lo, so they follow from
        // H alone: d = floor((H + 2^(s-1)) / 2^s) for s = 21, 14, 7 with H reduced after
        // each; the remainder H 2^21 + Lo is then below 2^27 in magnitude
        int d[OZ_S];
        int hi = (int)(I >> 21);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const int sh = 7 * (2 - k) + 7;  // 21, 14, 7
            d[k] = (hi + (1 << (sh - 1))) >> sh;
            hi -= d[k] * (1 << sh);
        }
        int rem32 = hi * (1 << 21) + (int)(I & 0x1fffff);
#pragma unroll
        for (int k = 3; k < OZ_S - 1; ++k) {
            const int sh = 7 * (OZ_S - 1 - k);
            d[k] = (rem32 + (1 << (sh - 1))) >> sh;
            rem32 -= d[k] * (1 << sh);
        }
        d[OZ_S - 1] = rem32;
        // small integers to float exactly by the 1.5 * 2^23 offset (an integer add and an
        // FP32 subtraction); a digit (|d| <= 128) has at most 8 significant bits, so it is
        // exact in BF16, and two samples' digits become one packed word by one conversion
#pragma unroll
        for (int k = 0; k < NW; ++k) {
            const float f = __int_as_float(0x4B400000 + d[k]) - 12582912.0f;
            if (e & 1) wds[k][e >> 1] = bf16x2_rn(fe[k], f);
            else fe[k] = f;
        }
    }
    const int nI = p_pad / OZ_TM;
    const long long nq = n_pad / 16;
    uint8_t *__restrict__ dig = Jb.dig;
    const size_t roff = tc::kmajor_offset((uint32_t)(j % OZ_TM), (uint32_t)(tg % 16));
#pragma unroll
    for (int k = 0; k < NW; ++k) {
        const size_t off = (((size_t)k * nI + j / OZ_TM) * nq + tg / 16) * 4096 + roff;
        *reinterpret_cast<uint4 *>(dig + off) = make_uint4(wds[k][0], wds[k][1], wds[k][2], wds[k][3]);
    }
}

template <typename T, class Src, int NW = OZ_S>
__global__ void __launch_bounds__(256) digit_split_kernel(Src src, long long total) {
    pdl_wait();
    pdl_trigger();
    if constexpr (std::is_same<Src, OneJob>::value) {
        (void)total;
        digit_split_block<T, NW>(src.job, blockIdx.x);
    } else {
        __shared__ OzJob s_job;
        __shared__ long long s_rng[2];
        stage_blocks(src, total, s_job, s_rng, [&](const OzJob &J, long long lb) {
            if (src.skip(J.index)) return;  // not selected in this run (uniform over the block)
            digit_split_block<T, NW>(J, lb);
        });
    }
}

// All seven digit planes of the flagged jobs only: a small grid strides over the flagged
// jobs' tiles (the full grid of a batch is millions of blocks, nearly all of which would
// only find their job unflagged).
template <typename T>
__global__ void digit_split_flagged_kernel(const OzJob *__restrict__ jobs, int count, const int *__restrict__ active) {
    for (int k = 0; k < count; ++k) {
        if (active[k] == 0) continue;  // uniform over the block
        const OzJob J = jobs[k];
        const long long nb = oz_digit_blocks(J.D);
        for (long long lb = blockIdx.x; lb < nb; lb += gridDim.x) digit_split_block<T, OZ_S>(J, lb);
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

// One tensor copy of a box of the digit planes (a 5-D tensor map, see
// digit_tensor_maps) into shared memory, completing on the mbarrier.
__device__ __forceinline__ void tma_g2s_5d(void *smem_dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                           int c4, uint64_t *mbar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
        "%6}], [%7];" ::"r"(tc::smem_u32(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(tc::smem_u32(mbar))
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
// end; warp 16 (lane 0) streams digit blocks into the shared-memory stages (two TMA
// tensor copies per K step, or 2 NS bulk copies for a job without tensor maps); warp 17
// (lane 0) issues the tensor-core MMAs.  They synchronise only through
// mbarriers: full (copy landed), empty (MMAs done reading a stage), chunk (MMAs of a
// chunk done), drained (TMEM read, accumulators may be overwritten).
template <class Src, int NS, bool TMAP>
__global__ void __launch_bounds__(OZ_THREADS, 1)
    corr_ozaki_kernel(Src src, const __grid_constant__ CUtensorMap tm_a, const __grid_constant__ CUtensorMap tm_b) {
    extern __shared__ __align__(1024) uint8_t smem[];
    constexpr int NST = oz_nst(NS);
    __shared__ __align__(8) uint64_t full_bar[OZ_NST_MAX], empty_bar[OZ_NST_MAX], chunk_bar, drained_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail;
    // the job lives in shared memory: each role reads its fields where it uses them, so
    // they hold no registers across the drain loop
    __shared__ OzJob s_job;
    __shared__ long long s_lb;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    pdl_wait();
    pdl_trigger();
    if (tid == 0) {
        long long lb0;
        s_job = src.get(blockIdx.x, lb0);
        s_lb = lb0;
    }
    __syncthreads();
    if (src.skip(s_job.index)) return;  // not selected in this run (uniform over the block)
    const long long lb = s_lb;
    const OzDims &D = s_job.D;
    int I, J;
    oz_tile_of((int)(lb % s_job.tiles), D.n_tiles_j, I, J);
    const int split = (int)(lb / s_job.tiles);
    const int nI = D.p_pad / OZ_TM;
    const long long nq = D.n_pad / 16;
    const long long q0 = (long long)split * D.slabs_per_split;
    const long long nst = min(q0 + (long long)D.slabs_per_split, nq) - q0;  // K steps of this split
    const int nchunks = (int)((nst + OZ_CHUNK_STEPS - 1) / OZ_CHUNK_STEPS);

    if (warp == 0) tc::tmem_alloc(&tmem_slot, OZ_TMEM_COLS);
    if (tid == 0) {
        for (int b = 0; b < NST; ++b) {
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
            // a register copy: the copies' memory clobbers would reload a shared-memory field
            const uint8_t *__restrict__ dig = s_job.dig;
            // the tensor maps: kernel parameters of a single job, or the job's maps in device
            // memory (written before the launch; the proxy fence orders their use)
            const CUtensorMap *map_a = &tm_a, *map_b = &tm_b;
            if constexpr (TMAP && !std::is_same<Src, OneJob>::value) {
                map_a = src.maps + 4 * s_job.index + (NS == OZ_S ? 0 : 2);
                map_b = map_a + 1;
                asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(map_a) : "memory");
                asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(map_b) : "memory");
            }
            (void)map_a;
            (void)map_b;
            for (long long st = 0; st < nst; ++st) {
                const int b = (int)(st % NST);
                if (st >= NST && !mbar_wait_fast(&empty_bar[b], (uint32_t)(((st / NST) - 1) & 1))) {
                    atomicExch(&s_fail, 1);
                    break;
                }
                if (*(volatile int *)&s_fail) break;
                uint8_t *sA = smem + (size_t)b * oz_stage_bytes(NS);
                uint8_t *sB = sA + oz_a_bytes(NS);
                mbar_expect_tx(&full_bar[b], (uint32_t)oz_stage_bytes(NS));
                const long long q = q0 + st;
                if constexpr (TMAP) {
                    // two tensor copies per step: the NS A blocks (both halves) and the NS B
                    // halves, each landing digit-major as the loop below lays them out; the
                    // copy engine's cost is per copy, so 2 instead of 2 NS copies measured
                    // as fast as no copies at all
                    tma_g2s_5d(sA, map_a, 0, 0, (int)q, I, 0, &full_bar[b]);
                    tma_g2s_5d(sB, map_b, 0, J & 1, (int)q, J >> 1, 0, &full_bar[b]);
                } else {
                    for (int k = 0; k < NS; ++k) {
                        bulk_g2s(sA + k * 4096, dig + (((size_t)k * nI + I) * nq + q) * 4096, 4096u, &full_bar[b]);
                        bulk_g2s(sB + k * 2048,
                                 dig + (((size_t)k * nI + (J >> 1)) * nq + q) * 4096 + (size_t)(J & 1) * 2048, 2048u,
                                 &full_bar[b]);
                    }
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
                    const int b = (int)(st % NST);
                    if (!mbar_wait_fast(&full_bar[b], (uint32_t)((st / NST) & 1))) {
                        bad = true;
                        break;
                    }
                    tc::fence_after_sync();
                    uint8_t *sA = smem + (size_t)b * oz_stage_bytes(NS);
                    uint8_t *sB = sA + oz_a_bytes(NS);
                    // Digit k of A against digits l = 0 .. NS-1-k of B: the B digits are
                    // consecutive 64-row operands in shared memory and the products land in
                    // consecutive accumulator groups g = k + l (TMEM columns 64 g ..), so up
                    // to four pairs form one MMA with N = 64 x (number of pairs).
#pragma unroll
                    for (int k = 0; k < NS; ++k) {
                        const uint64_t ad = tc::sdesc(tc::smem_u32(sA + k * 4096), 128, 256);
                        const int pairs = NS - k;
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
            // groups 0..2 -> hi with weights 2^14, 2^7, 1; groups 3..NS-1 -> lo with 2^21, 2^14, 2^7, 1
#pragma unroll
            for (int g = 0; g < NS; ++g) {
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
            long long *__restrict__ part_hi = s_job.phi;
            long long *__restrict__ part_lo = s_job.plo;
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                part_hi[base + e] = acc_hi[e];
                part_lo[base + e] = acc_lo[e];
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (tid == 0 && s_fail) atomicExch(s_job.err, 1);
    if (warp == 0) tc::tmem_dealloc(tmem, OZ_TMEM_COLS);
}

__device__ __forceinline__ double pow2(int e) { return __longlong_as_double((long long)(1023 + e) << 52); }

// fl(2^28 H + L) for integers H, L, rounded to nearest even once, from the exact 128-bit
// sum in integer arithmetic (the value fma((double)H, 2^28, (double)L) gives when H and
// L convert exactly) -- GB300's FP64 pipe is 1/64 of its integer and FP32 pipes.
__device__ __forceinline__ double exact_sum_to_f64(long long H, long long L) {
    unsigned long long lo = (unsigned long long)H << 28;
    long long hi = H >> 36;
    const unsigned long long lo2 = lo + (unsigned long long)L;
    hi += (L >> 63) + (lo2 < lo ? 1 : 0);
    lo = lo2;
    const bool neg = hi < 0;
    unsigned long long uh = (unsigned long long)hi;
    if (neg) {
        lo = ~lo + 1ull;
        uh = ~uh + (lo == 0ull ? 1ull : 0ull);
    }
    if (uh == 0ull && lo == 0ull) return 0.0;
    const int nb = uh ? 128 - __clzll((long long)uh) : 64 - __clzll((long long)lo);  // bit length
    unsigned long long m;
    if (nb <= 53) {
        m = lo << (53 - nb);
    } else {
        const int sh = nb - 53;  // 1 .. 75
        m = sh < 64 ? (lo >> sh) | (uh << (64 - sh)) : uh >> (sh - 64);
        const int rb = sh - 1;   // round bit position
        const bool round_bit = rb < 64 ? (lo >> rb) & 1ull : (uh >> (rb - 64)) & 1ull;
        const bool sticky = rb <= 64 ? (rb == 64 ? lo != 0ull : (lo & ((1ull << rb) - 1ull)) != 0ull)
                                     : lo != 0ull || (uh & ((1ull << (rb - 64)) - 1ull)) != 0ull;
        m += (round_bit && (sticky || (m & 1ull))) ? 1ull : 0ull;
    }
    int e = nb - 1;
    if (m >> 53) {  // rounding carried into a new bit
        m >>= 1;
        ++e;
    }
    const unsigned long long bits =
        (neg ? 0x8000000000000000ull : 0ull) | ((unsigned long long)(e + 1023) << 52) | (m & 0xfffffffffffffull);
    return __longlong_as_double((long long)bits);
}

// x 2^e for a normal x whose result stays normal (exact): exponent arithmetic on the bits;
// anything else through the multiplication.
__device__ __forceinline__ double scale_pow2(double x, int e) {
    const long long b = __double_as_longlong(x);
    const int ef = (int)((b >> 52) & 0x7ff);
    if (ef == 0 || ef == 0x7ff || ef + e < 1 || ef + e > 2046) return x * pow2(e);
    return __longlong_as_double(b + ((long long)e << 52));
}

// Covariance of (i, j) from the exact split sums: (2^28 H + L) 2^(E_i + E_j - 56) / (n - 1).
__device__ __forceinline__ double oz_cov(const long long *__restrict__ part_hi, const long long *__restrict__ part_lo,
                                         const OzDims &D, const int *__restrict__ expo, double scale, int i, int j) {
    long long H = 0, Lo = 0;
    for (int s = 0; s < D.splits; ++s) {
        const size_t ix = ((size_t)s * D.p_pad + i) * D.p_pad + j;
        H += part_hi[ix];
        Lo += part_lo[ix];
    }
    const double val = exact_sum_to_f64(H, Lo);  // exact terms, one rounding
    return scale_pow2(val, expo[i] + expo[j] - 56) * scale;
}

// Bound of |C' - C| for the five-digit product C' against the seven-digit C, from the
// column of i (the bound of a job is the maximum over its columns).
//
// With I = round(y 2^49) = sum_{k<5} d_k 2^(42-7k) + r (|r| <= 2^13; |d_0| <= 2^7 and
// |d_k| <= 2^6 after it), the kept pairs k + l <= 4 miss from I_i I_j the pairs
// k + l >= 5 (at most 1.01 * 2^63) and the terms with r (at most 2^13 (|I_i| + |I_j|)
// + 3 * 2^26); the seven-digit product itself misses at most 2^50 (pairs k + l >= 7).
// In units of y (divide by 2^98) a sample contributes at most 1.02 * 2^-35 +
// 2^-36 (|y_ti| + |y_tj|), and by Cauchy-Schwarz sum_t |y_ti| <= sqrt(n S_i) with
// S_i = sum_t y_ti^2.  Relative to sqrt(S_i S_j) the covariance error is then at most
// f(w) = 1.02 * 2^-35 w + 2^-35 sqrt(w) with w = n / min(S_i, S_j), and the
// normalisation by the (equally perturbed) variances at most doubles it to first
// order; the factor 2.5 covers that, the higher-order terms and the roundings.
template <class Src>
__device__ __forceinline__ double split_eps(const OzJob &J, int i) {
    long long H = 0, Lo = 0;
    for (int s = 0; s < J.D.splits; ++s) {
        const size_t ix = ((size_t)s * J.D.p_pad + i) * J.D.p_pad + i;
        H += J.phi[ix];
        Lo += J.plo[ix];
    }
    const double S = scale_pow2(exact_sum_to_f64(H, Lo), -56);  // sum_t y_ti^2
    if (!(S > 0.0)) return __longlong_as_double(0x7ff0000000000000ll);
    const double w = (double)J.n / S;
    return 2.5 * 0x1p-35 * (1.02 * w + sqrt(w));
}

template <class Src>
__global__ void ozaki_diag_kernel(Src src) {
    pdl_wait();
    pdl_trigger();
    long long lb;
    const OzJob &J = src.get(blockIdx.x, lb);
    if (src.skip(J.index)) return;
    const int i = (int)lb * blockDim.x + threadIdx.x;
    const double scale = 1.0 / (double)(J.n - 1);
    if (i < J.p) {
        J.inv_sd[i] = 1.0 / sqrt(oz_cov(J.phi, J.plo, J.D, J.expo, scale, i, i));
        double *slot = src.err_slot(J.index);
        if (slot != nullptr)  // non-negative doubles order like their bit patterns
            atomicMax(reinterpret_cast<unsigned long long *>(slot),
                      (unsigned long long)__double_as_longlong(split_eps<Src>(J, i)));
    }
}

// C_ij = clip(cov_ij / s_i / s_j, -1, 1) (the normalisation of numpy's corrcoef, with
// reciprocals of the standard deviations), for one 32 x 32 tile of the upper triangle
// per block; the mirrored tile is written through shared memory so both triangles are
// stored row-contiguously, and the FP32 copy the same way when the job has one.
template <class Src>
__global__ void ozaki_finish_kernel(Src src) {
    __shared__ double tv[32][33];
    pdl_wait();
    pdl_trigger();
    long long lb;
    const OzJob &J = src.get(blockIdx.x, lb);
    if (src.skip(J.index)) return;
    const int p = J.p;
    const int nb = (p + 31) / 32;
    int rem = (int)lb, bi = 0;
    while (rem >= nb - bi) {
        rem -= nb - bi;
        ++bi;
    }
    const int bj = bi + rem;
    const double scale = 1.0 / (double)(J.n - 1);
    const bool failed = *J.err != 0;  // a tensor-core wait timed out: poison the output
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int r = ty; r < 32; r += 8) {
        const int i = bi * 32 + r, j = bj * 32 + tx;
        double v = 0.0;
        if (i < p && j < p && (bi != bj || i <= j)) {
            v = oz_cov(J.phi, J.plo, J.D, J.expo, scale, i, j) * J.inv_sd[i] * J.inv_sd[j];
            // clip to [-1, 1] on the bits, as fmin(fmax(v, -1), 1) (NaN gives -1)
            const unsigned long long vb = (unsigned long long)__double_as_longlong(v);
            const unsigned long long mag = vb & 0x7fffffffffffffffull;
            if (mag > 0x7ff0000000000000ull) v = -1.0;
            else if (mag > 0x3ff0000000000000ull) v = (vb >> 63) ? -1.0 : 1.0;
            if (failed) v = __longlong_as_double(0x7ff8000000000000ll);
            J.C[(size_t)i * p + j] = v;
            if (J.C32 != nullptr) J.C32[(size_t)i * p + j] = f64_to_f32_rn(v);
        }
        tv[r][tx] = v;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
        const int j = bj * 32 + r, i = bi * 32 + tx;  // lower triangle (j, i)
        if (i < p && j < p && (bi != bj || j > i)) {
            J.C[(size_t)j * p + i] = tv[tx][r];
            if (J.C32 != nullptr) J.C32[(size_t)j * p + i] = f64_to_f32_rn(tv[tx][r]);
        }
    }
}

namespace host {

// splits: K splits of the tile grid; 0 chooses one wave over num_sms SMs
static OzDims oz_dims(long long n, int p, int num_sms, int splits_req = 0) {
    OzDims D;
    D.p = p;
    D.p_pad = (p + OZ_TM - 1) / OZ_TM * OZ_TM;
    D.n_pad = (int)((n + OZ_KS - 1) / OZ_KS * OZ_KS);
    D.n_tiles_j = (p + OZ_TN - 1) / OZ_TN;  // 64-column tiles that hold a column < p
    const int n_tiles_i = D.p_pad / OZ_TM;
    int tiles = 0;
    for (int i = 0; i < n_tiles_i; ++i) tiles += D.n_tiles_j - 2 * i;
    const long long steps = D.n_pad / 16;
    int splits = splits_req > 0 ? splits_req : num_sms / tiles;  // one wave: tiles x splits <= SMs
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

// Carve one job's workspace; with ws == nullptr only the size is computed.
static size_t oz_job(OzJob &J, void *ws, const void *X, long long n, int p, long long ldx, int num_sms,
                     int splits_req) {
    J.X = X;
    J.n = n;
    J.ldx = ldx;
    J.p = p;
    J.chunks = (int)((n + OZ_STAT_ROWS - 1) / OZ_STAT_ROWS);
    J.D = oz_dims(n, p, num_sms, splits_req);
    J.tiles = oz_tiles(J.D);
    J.pad = 0;
    const OzDims &D = J.D;
    char *w = static_cast<char *>(ws);
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *r = w ? w + off : nullptr;
        off += (bytes + 255) / 256 * 256;
        return r;
    };
    J.partial = reinterpret_cast<double *>(take((size_t)J.chunks * p * sizeof(double)));
    J.mean = reinterpret_cast<double *>(take((size_t)p * sizeof(double)));
    J.inv_sd = reinterpret_cast<double *>(take((size_t)p * sizeof(double)));
    J.kmin = reinterpret_cast<long long *>(take((size_t)p * sizeof(long long)));
    J.kmax = reinterpret_cast<long long *>(take((size_t)p * sizeof(long long)));
    J.expo = reinterpret_cast<int *>(take((size_t)p * sizeof(int)));
    J.err = reinterpret_cast<int *>(take(sizeof(int)));
    J.dig = reinterpret_cast<uint8_t *>(take((size_t)OZ_S * D.p_pad * (size_t)D.n_pad * sizeof(uint16_t)));
    J.phi = reinterpret_cast<long long *>(take((size_t)D.splits * D.p_pad * (size_t)D.p_pad * sizeof(long long) * 2));
    J.plo = J.phi ? J.phi + (size_t)D.splits * D.p_pad * (size_t)D.p_pad : nullptr;
    J.C = nullptr;
    J.C32 = nullptr;
    J.index = 0;
    return off;
}

// Blocks of each stage for one job (launch geometry of the kernels above).
static void oz_stage_blocks(const OzJob &J, long long *nb) {
    nb[OZ_INIT] = (J.p + 255) / 256;
    nb[OZ_STATS] = (long long)((J.p + 31) / 32) * J.chunks;
    nb[OZ_MEAN] = (J.p + 255) / 256;
    nb[OZ_DIGITS] = oz_digit_blocks(J.D);
    nb[OZ_PRODUCT] = (long long)J.tiles * J.D.splits;
    nb[OZ_DIAG] = (J.p + 255) / 256;
    const long long tb = (J.p + 31) / 32;
    nb[OZ_FINISH] = tb * (tb + 1) / 2;  // 32 x 32 upper-triangle tiles
}

size_t corr_tc_workspace_bytes(long long n, int p, int num_sms) {
    OzJob J;
    return oz_job(J, nullptr, nullptr, n, p, p, num_sms, 0);
}

template <class Src, int NS>
static cudaError_t set_ozaki_smem() {
    static std::atomic<bool> done{false};  // per instantiation; the value set is the same for every caller
    if (done.load()) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(corr_ozaki_kernel<Src, NS, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, oz_nst(NS) * oz_stage_bytes(NS));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(corr_ozaki_kernel<Src, NS, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 oz_nst(NS) * oz_stage_bytes(NS));
    if (e == cudaSuccess) done.store(true);
    return e;
}


// Stage launches shared by the single-job and batched paths; nb[] = blocks per stage.
// One stage: the single-job path launches with programmatic dependent launch (each
// kernel waits for its predecessor with pdl_wait); the batched path, captured into CUDA
// graphs, launches plainly.
template <class Src, typename K, typename... A>
static cudaError_t launch_stage(K kernel, long long blocks, int threads, size_t smem, const Src &src, cudaStream_t s,
                                const char *what, A... extra) {
    cudaError_t e;
    if constexpr (std::is_same<Src, OneJob>::value) {
        e = launch_pdl(kernel, dim3((unsigned)blocks), dim3(threads), smem, s, src, extra...);
    } else {
        kernel<<<(unsigned)blocks, threads, smem, s>>>(src, extra...);
        e = cudaGetLastError();
    }
    return note_error(what, e);
}

// Grid of a persistent stage kernel (stage_blocks): as many 256-thread blocks as are
// resident at once, at most one per stage block.
template <typename K>
static long long persistent_grid(K kernel, long long total) {
    // resident blocks per SM, once per kernel (kernels of one signature share K)
    static std::mutex mu;
    static std::vector<std::pair<const void *, int>> known;
    int occ = 0;
    {
        std::lock_guard<std::mutex> g(mu);
        for (const auto &kv : known)
            if (kv.first == (const void *)kernel) occ = kv.second;
        if (occ == 0) {
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, 256, 0) != cudaSuccess || occ < 1) occ = 1;
            known.emplace_back((const void *)kernel, occ);
        }
    }
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 1;
    return std::max(1ll, std::min(total, (long long)sms * occ));
}

// Launches a stage kernel written with stage_blocks over `total` stage blocks: a batch
// with as many blocks as are resident (each walks a range of its stage's blocks), a
// single job with one block per stage block (there is no job to look up, and the
// block turnover overlaps the loads of new blocks with the stores of finishing ones).
template <class Src, typename K>
static cudaError_t launch_persistent(K kernel, long long total, const Src &src, cudaStream_t s, const char *what) {
    const long long grid = std::is_same<Src, OneJob>::value ? total : persistent_grid(kernel, total);
    return launch_stage(kernel, grid, 256, 0, src, s, what, total);
}

// Tensor maps of a job's digit planes as a 5-D tensor of 8-byte elements: (256 elements =
// 2 KB half of a 128-row block, 2 halves, nq K steps, nI row blocks, OZ_S planes), and
// the boxes of one K step: A = NS planes x both halves of block I, B = NS planes x half
// J & 1 of block J >> 1.  Encoded through the driver entry point (no link to libcuda).
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_tiled_fn() {
    static EncodeTiledFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

static cudaError_t digit_tensor_maps(const OzJob &J, int ns, CUtensorMap &a, CUtensorMap &b) {
    const EncodeTiledFn enc = encode_tiled_fn();
    if (enc == nullptr) return note_error("cuTensorMapEncodeTiled entry point", cudaErrorNotSupported);
    const cuuint64_t nq = (cuuint64_t)(J.D.n_pad / 16), nI = (cuuint64_t)(J.D.p_pad / OZ_TM);
    const cuuint64_t dims[5] = {256, 2, nq, nI, (cuuint64_t)OZ_S};
    const cuuint64_t strides[4] = {2048, 4096, nq * 4096, nI * nq * 4096};  // bytes, dims 1..4
    const cuuint32_t box_a[5] = {256, 2, 1, 1, (cuuint32_t)ns}, box_b[5] = {256, 1, 1, 1, (cuuint32_t)ns};
    const cuuint32_t unit[5] = {1, 1, 1, 1, 1};
    for (int m = 0; m < 2; ++m) {
        const CUresult r = enc(m == 0 ? &a : &b, CU_TENSOR_MAP_DATA_TYPE_UINT64, 5, J.dig, dims, strides,
                               m == 0 ? box_a : box_b, unit, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return note_error("cuTensorMapEncodeTiled", cudaErrorInvalidValue);
    }
    return cudaSuccess;
}

// The product copies its digits with two tensor copies per K step: a single job's maps
// are kernel parameters, a batch's are in its workspace header (JobTable::maps).
template <class Src, int NS>
static cudaError_t launch_ozaki(const Src &src, long long blocks, cudaStream_t s) {
    const size_t smem = (size_t)oz_nst(NS) * oz_stage_bytes(NS);
    CUtensorMap ta, tb;
    std::memset(&ta, 0, sizeof(ta));
    std::memset(&tb, 0, sizeof(tb));
    if constexpr (std::is_same<Src, OneJob>::value) {
        const cudaError_t e = digit_tensor_maps(src.job, NS, ta, tb);
        if (e != cudaSuccess) return e;
        return launch_stage(corr_ozaki_kernel<Src, NS, true>, blocks, OZ_THREADS, smem, src, s, "corr_ozaki_kernel launch",
                            ta, tb);
    } else {
        if (src.maps != nullptr)
            return launch_stage(corr_ozaki_kernel<Src, NS, true>, blocks, OZ_THREADS, smem, src, s,
                                "corr_ozaki_kernel launch", ta, tb);
        return launch_stage(corr_ozaki_kernel<Src, NS, false>, blocks, OZ_THREADS, smem, src, s,
                            "corr_ozaki_kernel launch", ta, tb);
    }
}

// Stage launches shared by the single-job and batched paths; nb[] = blocks per stage.
template <class Src>
static cudaError_t launch_digits(const Src &src, const long long *nb, int dtype, cudaStream_t s) {
    note_launch(4);
    cudaError_t e = launch_stage(colstats_init_kernel<Src>, nb[OZ_INIT], 256, 0, src, s, "colstats_init_kernel launch");
    if (e != cudaSuccess) return e;
    e = dtype == GCSL_DTYPE_F64
            ? launch_persistent(colstats_kernel<double, Src>, nb[OZ_STATS], src, s, "colstats_kernel launch")
            : launch_persistent(colstats_kernel<float, Src>, nb[OZ_STATS], src, s, "colstats_kernel launch");
    if (e != cudaSuccess) return e;
    e = launch_stage(col_mean_exp_kernel<Src>, nb[OZ_MEAN], 256, 0, src, s, "col_mean_exp_kernel launch");
    if (e != cudaSuccess) return e;
    return dtype == GCSL_DTYPE_F64
               ? launch_persistent(digit_split_kernel<double, Src>, nb[OZ_DIGITS], src, s, "digit_split_kernel launch")
               : launch_persistent(digit_split_kernel<float, Src>, nb[OZ_DIGITS], src, s, "digit_split_kernel launch");
}

template <class Src, int NS = OZ_S>
static cudaError_t launch_product(const Src &src, const long long *nb, cudaStream_t s) {
    note_launch(3);
    cudaError_t e = note_error("corr_ozaki_kernel attribute", set_ozaki_smem<Src, NS>());
    if (e != cudaSuccess) return e;
    e = launch_ozaki<Src, NS>(src, nb[OZ_PRODUCT], s);
    if (e != cudaSuccess) return e;
    e = launch_stage(ozaki_diag_kernel<Src>, nb[OZ_DIAG], 256, 0, src, s, "ozaki_diag_kernel launch");
    if (e != cudaSuccess) return e;
    return launch_stage(ozaki_finish_kernel<Src>, nb[OZ_FINISH], 256, 0, src, s, "ozaki_finish_kernel launch");
}

static bool one_job(OneJob &o, long long *nb, const void *X, long long n, int p, long long ldx, double *C, void *ws,
                    size_t ws_bytes, int num_sms) {
    const size_t need = oz_job(o.job, ws, X, n, p, ldx, num_sms, 0);
    if (ws_bytes < need) return false;
    o.job.C = C;
    oz_stage_blocks(o.job, nb);
    return true;
}

// Stage 1: column statistics, exponents and the digit tiles (FP64 / integer work).
cudaError_t corr_tc_digits(const void *X, int dtype, long long n, int p, long long ldx, void *ws, size_t ws_bytes,
                           int num_sms, cudaStream_t s) {
    OneJob o;
    long long nb[OZ_NSTAGES];
    if (!one_job(o, nb, X, n, p, ldx, nullptr, ws, ws_bytes, num_sms)) return cudaErrorInvalidValue;
    return launch_digits(o, nb, dtype, s);
}

// Stage 2: exact digit products on the tensor cores, reduction, normalisation.
cudaError_t corr_tc_product(long long n, int p, double *C, void *ws, size_t ws_bytes, int num_sms, cudaStream_t s) {
    OneJob o;
    long long nb[OZ_NSTAGES];
    if (!one_job(o, nb, nullptr, n, p, p, C, ws, ws_bytes, num_sms)) return cudaErrorInvalidValue;
    return launch_product(o, nb, s);
}

cudaError_t corr_tc(const void *X, int dtype, long long n, int p, long long ldx, double *C, void *ws, size_t ws_bytes,
                    int num_sms, int *unused, cudaStream_t s) {
    (void)unused;
    cudaError_t e = corr_tc_digits(X, dtype, n, p, ldx, ws, ws_bytes, num_sms, s);
    if (e != cudaSuccess) return e;
    return corr_tc_product(n, p, C, ws, ws_bytes, num_sms, s);
}

// ------------------------------------------------------------------ batches
// Workspace: [job table | stage offsets (OZ_NSTAGES x (count + 1)) | tensor maps | job
// slices].  The
// plan (host) keeps the block totals per stage so the run needs no device reads.
static size_t batch_maps_offset(int count) {
    const size_t a = ((size_t)count * sizeof(OzJob) + 255) / 256 * 256;
    return a + ((size_t)OZ_NSTAGES * (count + 1) * sizeof(long long) + 255) / 256 * 256;
}
// [job table | stage offsets | 4 tensor maps per job]
static size_t batch_header_bytes(int count) {
    return batch_maps_offset(count) + ((size_t)count * 4 * sizeof(CUtensorMap) + 255) / 256 * 256;
}

size_t corr_tc_batch_workspace_bytes(const long long *n, const int *p, int count) {
    size_t total = batch_header_bytes(count);
    for (int k = 0; k < count; ++k) {
        OzJob J;
        total += oz_job(J, nullptr, nullptr, n[k], p[k], p[k], 1, 1);
    }
    return total;
}

cudaError_t corr_tc_batch_prepare(const void *const *X, const long long *n, const int *p, const long long *ldx,
                                  double *const *C, float *const *C32, int count, void *ws, size_t ws_bytes,
                                  long long *stage_totals, cudaStream_t s) {
    if (ws_bytes < corr_tc_batch_workspace_bytes(n, p, count)) return cudaErrorInvalidValue;
    std::vector<OzJob> jobs((size_t)count);
    std::vector<long long> off((size_t)OZ_NSTAGES * (count + 1), 0);
    char *base = static_cast<char *>(ws);
    size_t cur = batch_header_bytes(count);
    for (int k = 0; k < count; ++k) {
        OzJob &J = jobs[(size_t)k];
        cur += oz_job(J, base + cur, X[k], n[k], p[k], ldx[k], 1, 1);
        J.C = C[k];
        J.C32 = C32 ? C32[k] : nullptr;
        J.index = k;
        long long nb[OZ_NSTAGES];
        oz_stage_blocks(J, nb);
        for (int st = 0; st < OZ_NSTAGES; ++st)
            off[(size_t)st * (count + 1) + k + 1] = off[(size_t)st * (count + 1) + k] + nb[st];
    }
    for (int st = 0; st < OZ_NSTAGES; ++st) stage_totals[st] = off[(size_t)st * (count + 1) + count];
    // per job the tensor maps of its digit planes: [A, B] over seven planes, [A, B] over the
    // split product's five
    std::vector<CUtensorMap> maps((size_t)count * 4);
    for (int k = 0; k < count; ++k) {
        cudaError_t e = digit_tensor_maps(jobs[(size_t)k], OZ_S, maps[4 * (size_t)k], maps[4 * (size_t)k + 1]);
        if (e == cudaSuccess)
            e = digit_tensor_maps(jobs[(size_t)k], OZ_S_SPLIT, maps[4 * (size_t)k + 2], maps[4 * (size_t)k + 3]);
        if (e != cudaSuccess) return e;
    }
    const size_t a = ((size_t)count * sizeof(OzJob) + 255) / 256 * 256;
    cudaError_t e = cudaMemcpyAsync(base, jobs.data(), (size_t)count * sizeof(OzJob), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + a, off.data(), off.size() * sizeof(long long), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + batch_maps_offset(count), maps.data(), maps.size() * sizeof(CUtensorMap),
                            cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // the host vectors die with this call
    return e;
}

// Modes of a batch run: every job exactly (seven digits); every job in split precision
// (five digits, bound per job into c_err); or only the jobs whose flag is set, exactly,
// reusing the digits of a previous run (product, diagonal and finish only).
cudaError_t corr_tc_batch_run_mode(void *ws, int count, const long long *stage_totals, int dtype, int mode,
                                   double *c_err, const int *active, cudaStream_t s) {
    char *base = static_cast<char *>(ws);
    const size_t a = ((size_t)count * sizeof(OzJob) + 255) / 256 * 256;
    const OzJob *jobs = reinterpret_cast<const OzJob *>(base);
    const long long *off = reinterpret_cast<const long long *>(base + a);
    long long nb[OZ_NSTAGES];
    for (int st = 0; st < OZ_NSTAGES; ++st) {
        nb[st] = stage_totals[st];
        if (nb[st] <= 0 || nb[st] > 0x7fffffffll) return cudaErrorInvalidValue;
    }
    // one JobTable per stage (the offsets differ); the stage launchers take the table of
    // their first kernel, so launch stage by stage
    JobTable t[OZ_NSTAGES];
    const CUtensorMap *maps = reinterpret_cast<const CUtensorMap *>(base + batch_maps_offset(count));
    for (int st = 0; st < OZ_NSTAGES; ++st) {
        t[st] = JobTable{jobs, off + (size_t)st * (count + 1), count};
        t[st].c_err = mode == CORR_BATCH_SPLIT ? c_err : nullptr;
        t[st].active = mode == CORR_BATCH_FLAGGED ? active : nullptr;
        t[st].maps = maps;
    }
    cudaError_t e;
    if (mode == CORR_BATCH_FLAGGED) {
        // the split run wrote five digit planes: the flagged jobs get all seven (their
        // column statistics are still in their workspace)
        note_launch(1);
        const unsigned fb = 608;  // a few blocks per SM stride over the flagged jobs' tiles
        if (dtype == GCSL_DTYPE_F64) digit_split_flagged_kernel<double><<<fb, 256, 0, s>>>(jobs, count, active);
        else digit_split_flagged_kernel<float><<<fb, 256, 0, s>>>(jobs, count, active);
        if ((e = note_error("digit_split_flagged_kernel launch", cudaGetLastError())) != cudaSuccess) return e;
    } else {
        note_launch(4);
        colstats_init_kernel<JobTable><<<(unsigned)nb[OZ_INIT], 256, 0, s>>>(t[OZ_INIT]);
        if ((e = note_error("colstats_init_kernel launch", cudaGetLastError())) != cudaSuccess) return e;
        e = dtype == GCSL_DTYPE_F64
                ? launch_persistent(colstats_kernel<double, JobTable>, nb[OZ_STATS], t[OZ_STATS], s, "colstats_kernel launch")
                : launch_persistent(colstats_kernel<float, JobTable>, nb[OZ_STATS], t[OZ_STATS], s, "colstats_kernel launch");
        if (e != cudaSuccess) return e;
        col_mean_exp_kernel<JobTable><<<(unsigned)nb[OZ_MEAN], 256, 0, s>>>(t[OZ_MEAN]);
        if ((e = note_error("col_mean_exp_kernel launch", cudaGetLastError())) != cudaSuccess) return e;
        const JobTable &td = t[OZ_DIGITS];
        const char *what = "digit_split_kernel launch";
        if (mode == CORR_BATCH_SPLIT)
            e = dtype == GCSL_DTYPE_F64
                    ? launch_persistent(digit_split_kernel<double, JobTable, OZ_S_SPLIT>, nb[OZ_DIGITS], td, s, what)
                    : launch_persistent(digit_split_kernel<float, JobTable, OZ_S_SPLIT>, nb[OZ_DIGITS], td, s, what);
        else
            e = dtype == GCSL_DTYPE_F64 ? launch_persistent(digit_split_kernel<double, JobTable>, nb[OZ_DIGITS], td, s, what)
                                        : launch_persistent(digit_split_kernel<float, JobTable>, nb[OZ_DIGITS], td, s, what);
        if (e != cudaSuccess) return e;
    }
    note_launch(3);
    if (mode == CORR_BATCH_SPLIT) {
        if ((e = note_error("corr_ozaki_kernel attribute", set_ozaki_smem<JobTable, OZ_S_SPLIT>())) != cudaSuccess)
            return e;
        e = launch_ozaki<JobTable, OZ_S_SPLIT>(t[OZ_PRODUCT], nb[OZ_PRODUCT], s);
    } else {
        if ((e = note_error("corr_ozaki_kernel attribute", set_ozaki_smem<JobTable, OZ_S>())) != cudaSuccess) return e;
        e = launch_ozaki<JobTable, OZ_S>(t[OZ_PRODUCT], nb[OZ_PRODUCT], s);
    }
    if (e != cudaSuccess) return e;
    ozaki_diag_kernel<JobTable><<<(unsigned)nb[OZ_DIAG], 256, 0, s>>>(t[OZ_DIAG]);
    if ((e = note_error("ozaki_diag_kernel launch", cudaGetLastError())) != cudaSuccess) return e;
    ozaki_finish_kernel<JobTable><<<(unsigned)nb[OZ_FINISH], 256, 0, s>>>(t[OZ_FINISH]);
    return note_error("ozaki_finish_kernel launch", cudaGetLastError());
}

cudaError_t corr_tc_batch_run(void *ws, int count, const long long *stage_totals, int dtype, cudaStream_t s) {
    return corr_tc_batch_run_mode(ws, count, stage_totals, dtype, CORR_BATCH_EXACT, nullptr, nullptr, s);
}

}  // namespace host
}  // namespace gcsl
