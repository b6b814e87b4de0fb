// Edge orientation of the skeleton on the GPU: v-structures, then Meek's rules R1-R3 to
// a fixed point, with the result of the reference's sequential CPU code
// (gpucsl/pc/edge_orientation/v_structures.py:8-35, orientation_rules.py:7-89).
//
// The reference visits ordered edges (v1, v2) in column-major order (key v2 * p + v1)
// and inner vertices ascending, writing a live graph.  Its outcome is reproduced in
// parallel from the structure of those writes:
//
// * v-structures read only the skeleton and the sepsets, so every unshielded triple's
//   decision is fixed; a triple with middle b orienting a -> b writes "a -> b present,
//   b -> a absent".  The last writer of a directed pair wins, and the visiting order is
//   by the middle vertex first, so with P[a][b] = "some triple orients a -> b":
//   a -> b is absent at the end iff P[b][a] and (not P[a][b] or a > b).
// * R1 checks the live graph before writing: on each edge the earliest firing (smallest
//   visiting key (v2 p + v1) p + v3) decides the direction (atomicMin per edge).
// * R2 and R3 write without a live check: on each edge the latest firing (largest key
//   v2 p + v1) decides the direction (atomicMax per edge).
// Each rule reads a snapshot (the graph after the previous rule's apply kernel).
//
// D[a * p + b] = 1 means the directed graph has a -> b; an undirected edge has both.
#include "common.cuh"

namespace gcsl {

constexpr unsigned long long OR_NONE = 0xffffffffffffffffull;

__device__ __forceinline__ bool in_sepset(const int *__restrict__ sep, int L, int p, int a, int c, int v) {
    const int *s1 = sep + ((size_t)a * p + c) * L, *s2 = sep + ((size_t)c * p + a) * L;
    for (int k = 0; k < L; ++k)
        if (s1[k] == v || s2[k] == v) return true;
    return false;
}

// P[a][b] for every skeleton edge: some neighbour v != a of b, non-adjacent to a, with b
// in neither sepset(a, v) nor sepset(v, a).  Warp per row a, lanes over N(b).
__global__ void vstruct_flags_kernel(const uint16_t *__restrict__ S, const int *__restrict__ adj, int p,
                                     const int *__restrict__ sep, int L, uint8_t *__restrict__ P) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; a < p; a += warps) {
        const int *ra = adj + (size_t)a * p;
        const int da = ra[0];
        for (int t = 0; t < da; ++t) {
            const int b = ra[1 + t];
            const int *rb = adj + (size_t)b * p;
            const int db = rb[0];
            bool hit = false;
            for (int k = lane; k < db && !hit; k += 32) {
                const int v = rb[1 + k];
                hit = v != a && S[(size_t)a * p + v] == 0 && !in_sepset(sep, L, p, a, v, b);
            }
            const bool any = __any_sync(GCSL_FULL_MASK, hit);
            if (lane == 0) P[(size_t)a * p + b] = any ? 1 : 0;
        }
    }
}

__global__ void vstruct_apply_kernel(const uint16_t *__restrict__ S, int p, const uint8_t *__restrict__ P,
                                     uint8_t *__restrict__ D, unsigned long long *__restrict__ key) {
    const long long total = (long long)p * p;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const int a = (int)(k / p), b = (int)(k - (long long)a * p);
        uint8_t d = 0;
        if (a != b && S[k] != 0) {
            const bool pab = P[k] != 0, pba = P[(size_t)b * p + a] != 0;
            d = (pba && (!pab || a > b)) ? 0 : 1;
        }
        D[k] = d;
        key[k] = OR_NONE;  // rule keys start empty
    }
}

// R1 on snapshot D: v1 -> v2 (directed only), v2 - v3 undirected, v1 and v3
// non-adjacent: orient v2 -> v3.  Earliest key per edge (pair index min * p + max).
__global__ void rule1_kernel(const int *__restrict__ adj, int p, const uint8_t *__restrict__ D,
                             unsigned long long *__restrict__ key) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int v1 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v1 < p; v1 += warps) {
        const int *r1 = adj + (size_t)v1 * p;
        const int d1 = r1[0];
        for (int t = 0; t < d1; ++t) {
            const int v2 = r1[1 + t];
            if (!D[(size_t)v1 * p + v2] || D[(size_t)v2 * p + v1]) continue;
            const int *r2 = adj + (size_t)v2 * p;
            const int d2 = r2[0];
            for (int k = lane; k < d2; k += 32) {
                const int v3 = r2[1 + k];
                if (v3 == v1) continue;
                if (D[(size_t)v2 * p + v3] && D[(size_t)v3 * p + v2] && !D[(size_t)v1 * p + v3] &&
                    !D[(size_t)v3 * p + v1]) {
                    const unsigned long long seq = ((unsigned long long)v2 * p + v1) * p + v3;
                    const int lo = v2 < v3 ? v2 : v3, hi = v2 < v3 ? v3 : v2;
                    atomicMin(&key[(size_t)lo * p + hi], seq * 2 + (v2 < v3 ? 0 : 1));
                }
            }
        }
    }
}

// v1 - v2 undirected in D (the warp's row v1): R2 (mode 2) some v3 with v1 -> v3 -> v2
// directed only; R3 (mode 3) two non-adjacent v3, v4 with v1 - v3 -> v2, v1 - v4 -> v2.
// Orient v1 -> v2, latest key per edge.
__device__ __forceinline__ bool r3_member(const uint8_t *__restrict__ D, int p, int v1, int v2, int v) {
    return D[(size_t)v1 * p + v] && D[(size_t)v * p + v1] && D[(size_t)v * p + v2] && !D[(size_t)v2 * p + v];
}

__global__ void rule23_kernel(const int *__restrict__ adj, int p, const uint8_t *__restrict__ D,
                              unsigned long long *__restrict__ key, int mode) {
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int v1 = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; v1 < p; v1 += warps) {
        const int *r1 = adj + (size_t)v1 * p;
        const int d1 = r1[0];
        for (int t = 0; t < d1; ++t) {
            const int v2 = r1[1 + t];
            if (!D[(size_t)v1 * p + v2] || !D[(size_t)v2 * p + v1]) continue;
            bool fire = false;
            if (mode == 2) {
                for (int k = lane; k < d1 && !fire; k += 32) {
                    const int v3 = r1[1 + k];
                    fire = v3 != v2 && D[(size_t)v1 * p + v3] && !D[(size_t)v3 * p + v1] && D[(size_t)v3 * p + v2] &&
                           !D[(size_t)v2 * p + v3];
                }
            } else {
                const long long npairs = (long long)d1 * (d1 - 1) / 2;
                for (long long q = lane; q < npairs && !fire; q += 32) {
                    // pair index q -> (i, j), i < j, over the neighbour positions of v1
                    int i = (int)((2.0 * d1 - 1.0 - sqrt((2.0 * d1 - 1.0) * (2.0 * d1 - 1.0) - 8.0 * q)) / 2.0);
                    while (i > 0 && (long long)i * (2 * d1 - i - 1) / 2 > q) --i;
                    while ((long long)(i + 1) * (2 * d1 - i - 2) / 2 <= q) ++i;
                    const int j = (int)(q - (long long)i * (2 * d1 - i - 1) / 2) + i + 1;
                    const int v3 = r1[1 + i], v4 = r1[1 + j];
                    fire = v3 != v2 && v4 != v2 && r3_member(D, p, v1, v2, v3) && r3_member(D, p, v1, v2, v4) &&
                           !D[(size_t)v3 * p + v4] && !D[(size_t)v4 * p + v3];
                }
            }
            if (__any_sync(GCSL_FULL_MASK, fire) && lane == 0) {
                const unsigned long long seq = (unsigned long long)v2 * p + v1;
                const int lo = v1 < v2 ? v1 : v2, hi = v1 < v2 ? v2 : v1;
                atomicMax(&key[(size_t)lo * p + hi], seq * 2 + (v1 < v2 ? 0 : 1));
            }
        }
    }
}

// Orient every edge whose key is set (none = `none`), reset the key, flag a change.
__global__ void rule_apply_kernel(int p, uint8_t *__restrict__ D, unsigned long long *__restrict__ key,
                                  unsigned long long none, unsigned long long next_none, int *changed) {
    const long long total = (long long)p * p;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += (long long)gridDim.x * blockDim.x) {
        const unsigned long long v = key[k];
        if (v == none) {
            key[k] = next_none;
            continue;
        }
        const int lo = (int)(k / p), hi = (int)(k - (long long)lo * p);
        if ((v & 1ull) == 0) {  // lo -> hi
            D[(size_t)lo * p + hi] = 1;
            D[(size_t)hi * p + lo] = 0;
        } else {
            D[(size_t)hi * p + lo] = 1;
            D[(size_t)lo * p + hi] = 0;
        }
        key[k] = next_none;
        *changed = 1;
    }
}

namespace host {

size_t orient_workspace_bytes(int p) {
    const size_t pp = (size_t)p * p;
    auto al = [](size_t x) { return (x + 255) / 256 * 256; };
    return al(pp * sizeof(int)) + al(pp) + al(pp * sizeof(unsigned long long)) + al(sizeof(int));
}

cudaError_t launch_compact(const uint16_t *G, int p, int *adj, int *up, DevState *st, int level, int2 *elist,
                           cudaStream_t s);

// Returns the number of rule passes in *passes; `words` is pinned host memory (1 int).
cudaError_t orient_edges(const uint16_t *S, int p, const int *sep, int L, uint8_t *D, void *ws, int num_sms,
                         int *host_word, int *passes, cudaStream_t s) {
    const size_t pp = (size_t)p * p;
    auto al = [](size_t x) { return (x + 255) / 256 * 256; };
    char *w = static_cast<char *>(ws);
    int *adj = reinterpret_cast<int *>(w);
    uint8_t *P = reinterpret_cast<uint8_t *>(w + al(pp * sizeof(int)));
    unsigned long long *key = reinterpret_cast<unsigned long long *>(w + al(pp * sizeof(int)) + al(pp));
    int *changed = reinterpret_cast<int *>(w + al(pp * sizeof(int)) + al(pp) + al(pp * 8));
    const int rows_blocks = (p + 7) / 8, ent_blocks = (int)std::min<long long>(((long long)pp + 255) / 256, num_sms * 8ll);
    cudaError_t e = launch_compact(S, p, adj, nullptr, nullptr, 0, nullptr, s);
    if (e != cudaSuccess) return e;
    vstruct_flags_kernel<<<rows_blocks, 256, 0, s>>>(S, adj, p, sep, L, P);
    vstruct_apply_kernel<<<ent_blocks, 256, 0, s>>>(S, p, P, D, key);
    note_launch(2);
    const long long max_passes = (long long)pp / 2 + 2;  // every pass orients an edge
    int n = 0;
    for (;;) {
        ++n;
        if ((e = cudaMemsetAsync(changed, 0, sizeof(int), s)) != cudaSuccess) return e;
        rule1_kernel<<<rows_blocks, 256, 0, s>>>(adj, p, D, key);
        rule_apply_kernel<<<ent_blocks, 256, 0, s>>>(p, D, key, OR_NONE, 0ull, changed);
        rule23_kernel<<<rows_blocks, 256, 0, s>>>(adj, p, D, key, 2);
        rule_apply_kernel<<<ent_blocks, 256, 0, s>>>(p, D, key, 0ull, 0ull, changed);
        rule23_kernel<<<rows_blocks, 256, 0, s>>>(adj, p, D, key, 3);
        rule_apply_kernel<<<ent_blocks, 256, 0, s>>>(p, D, key, 0ull, OR_NONE, changed);
        note_launch(6);
        if ((e = cudaMemcpyAsync(host_word, changed, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return e;
        if (!*host_word || n >= max_passes) break;
    }
    *passes = n;
    return cudaGetLastError();
}

}  // namespace host
}  // namespace gcsl
