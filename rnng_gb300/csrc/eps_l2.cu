// Epsilon-graph pipeline for dense float32 points under RNNG's L2.
//
// Replaces, on one GPU, the neighbour search that RNNG runs with cover trees over
// MPI ranks (include/search.hpp:6-340, include/point.hpp:537-929): instead of a
// tree walk per query, the points are ordered by a two-level landmark partition
// (the Voronoi idea of include/point.hpp:537-559 applied twice), cut into tiles of
// 128 points, and every pair of tiles that the triangle inequality cannot rule out
// is evaluated in full.  The pruning is exact: a tile pair is skipped only when a
// pivot p gives |d(x,p) - d(y,p)| > radius for all x, y with a rounding slack that
// covers the float error of both the pivot distances and the reference's own
// sequential L2, so no pair with L2seq <= radius is ever skipped.
//
// Stages (all on the context stream):
//   1. level-1 landmarks (strided sample), nearest landmark per point  -> cell1
//   2. sort by cell1; level-2 landmarks inside each cell1, nearest    -> leaf cell
//   3. sort by (leaf, distance to its landmark); gather points in that order
//   4. per tile and per pivot: [min, max] of the pivot distances
//   5. prune super-tile pairs (8x8 tiles), then tile pairs
//   6. evaluate surviving tile pairs (FP32-direct here; BF16 Gram in gram_bf16.cu)
//   7. map sorted indices back to ids, order each edge as u < v
#include <cub/cub.cuh>

#include "common.cuh"
#include "eps_l2.cuh"

namespace rnng {

// ------------------------------------------------------------------------------------------------
// helpers

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Squared L2 (any summation order) of row x against row c, computed by one warp.
__device__ __forceinline__ float warp_dist2(const float* __restrict__ x, const float* __restrict__ c, int d, int lane)
{
    float s = 0.f;
    for (int k = lane; k < d; k += 32) {
        float t = x[k] - c[k];
        s = fmaf(t, t, s);
    }
    return warp_sum(s);
}

__global__ void k_gather_rows(const float* __restrict__ X, int64_t d, const int32_t* __restrict__ idx, int64_t m,
                              float* __restrict__ out)
{
    int64_t total = m * d;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = t / d, k = t - r * d;
        out[t] = X[(int64_t)idx[r] * d + k];
    }
}

__global__ void k_strided_index(int32_t* __restrict__ out, int64_t m, int64_t n)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < m) out[i] = (int32_t)((i * n) / m);
}

// Level 1: nearest of m1 landmarks for each point (warp per point).
// key = (cell << 32) | bits(dist) so that a radix sort groups cells and orders
// points by their distance to the cell landmark.
__global__ void k_assign_level1(const float* __restrict__ X, int64_t n, int d, const float* __restrict__ L, int m1,
                                uint64_t* __restrict__ keys, int32_t* __restrict__ vals)
{
    extern __shared__ float sL[];
    const bool in_smem = (int64_t)m1 * d * 4 <= 48 * 1024;
    if (in_smem)
        for (int t = threadIdx.x; t < m1 * d; t += blockDim.x) sL[t] = L[t];
    __syncthreads();
    const float* LL = in_smem ? sL : L;
    int lane = threadIdx.x & 31;
    int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = warp; i < n; i += nwarps) {
        const float* x = X + i * d;
        float best = INFINITY;
        int bi = 0;
        for (int c = 0; c < m1; ++c) {
            float s = warp_dist2(x, LL + (int64_t)c * d, d, lane);
            if (s < best) { best = s; bi = c; }
        }
        if (lane == 0) {
            float dist = sqrtf(best);
            keys[i] = ((uint64_t)bi << 32) | __float_as_uint(dist);
            vals[i] = (int32_t)i;
        }
    }
}

// Per level-1 cell: start offset in the sorted order and size (cells are contiguous
// after the sort).  One thread per sorted position marks cell boundaries.
__global__ void k_cell_bounds(const uint64_t* __restrict__ sorted_keys, int64_t n, int32_t* __restrict__ start,
                              int32_t* __restrict__ end)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t c = (uint32_t)(sorted_keys[i] >> 32);
    if (i == 0 || (uint32_t)(sorted_keys[i - 1] >> 32) != c) start[c] = (int32_t)i;
    if (i == n - 1 || (uint32_t)(sorted_keys[i + 1] >> 32) != c) end[c] = (int32_t)(i + 1);
}

// Level-2 landmark budget per level-1 cell (single block): m2[c] proportional to the
// cell's size, at least 1 for a non-empty cell, at most kMaxSub; exclusive scan.
__global__ void k_level2_plan(const int32_t* __restrict__ start, const int32_t* __restrict__ end, int m1, int64_t n,
                              int64_t leaves_total, int32_t* __restrict__ m2, int32_t* __restrict__ m2_off)
{
    __shared__ int32_t s[1024];
    int c = threadIdx.x;
    int v = 0;
    if (c < m1) {
        int sz = end[c] - start[c];
        if (sz > 0) {
            int64_t want = (leaves_total * sz + n - 1) / n;
            v = (int)max((int64_t)1, min(want, (int64_t)kMaxSub));
            v = min(v, sz);
        }
        m2[c] = v;
    }
    s[c] = v;
    __syncthreads();
    if (c == 0) {
        int acc = 0;
        for (int j = 0; j < m1; ++j) { int t = s[j]; s[j] = acc; acc += t; }
        m2_off[m1] = acc;
    }
    __syncthreads();
    if (c < m1) m2_off[c] = s[c];
}

// Level-2 landmark rows: sub-landmark k of cell c is the point at position
// start[c] + floor(k * size / m2[c]) of the level-1 order.
__global__ void k_level2_landmarks(const int32_t* __restrict__ start, const int32_t* __restrict__ end,
                                   const int32_t* __restrict__ m2, const int32_t* __restrict__ m2_off, int m1,
                                   const int32_t* __restrict__ order1, int32_t* __restrict__ sub_idx)
{
    int c = blockIdx.x;
    if (c >= m1) return;
    int sz = end[c] - start[c];
    for (int k = threadIdx.x; k < m2[c]; k += blockDim.x)
        sub_idx[m2_off[c] + k] = order1[start[c] + (int)(((int64_t)k * sz) / m2[c])];
}

// Level 2: nearest sub-landmark inside the point's level-1 cell (warp per point,
// points visited in level-1 order so a block's sub-landmarks stay in cache).
__global__ void k_assign_level2(const float* __restrict__ X, int64_t n, int d, const uint64_t* __restrict__ keys1,
                                const int32_t* __restrict__ order1, const float* __restrict__ SL,
                                const int32_t* __restrict__ m2, const int32_t* __restrict__ m2_off,
                                uint64_t* __restrict__ keys2, int32_t* __restrict__ vals2)
{
    int lane = threadIdx.x & 31;
    int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t p = warp; p < n; p += nwarps) {
        int32_t i = order1[p];
        int c = (int)(keys1[p] >> 32);
        const float* x = X + (int64_t)i * d;
        int base = m2_off[c], cnt = m2[c];
        float best = INFINITY;
        int bi = 0;
        for (int k = 0; k < cnt; ++k) {
            float s = warp_dist2(x, SL + (int64_t)(base + k) * d, d, lane);
            if (s < best) { best = s; bi = k; }
        }
        if (lane == 0) {
            keys2[p] = ((uint64_t)(base + bi) << 32) | __float_as_uint(sqrtf(best));
            vals2[p] = i;
        }
    }
}

// Sorted copy of the points, padded with zero rows to a multiple of the tile size.
__global__ void k_gather_sorted(const float* __restrict__ X, int64_t n, int64_t n_pad, int d,
                                const int32_t* __restrict__ perm, float* __restrict__ Xs)
{
    int64_t total = n_pad * d;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t r = t / d, k = t - r * d;
        Xs[t] = (r < n) ? X[(int64_t)perm[r] * d + k] : 0.f;
    }
}

// Per tile (128 sorted rows) and pivot: min and max of the pivot distance over the
// tile's real rows.  Block = 4 warps = one tile; each warp covers 32 rows.
// Output layout is [pivot][tile] so pruning threads read consecutive tiles.
__global__ void k_tile_bounds(const float* __restrict__ Xs, int64_t n, int d, const float* __restrict__ Pv, int P,
                              int64_t T, float* __restrict__ lo, float* __restrict__ hi)
{
    __shared__ float s_lo[4][kMaxPivots], s_hi[4][kMaxPivots];
    int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int64_t t = blockIdx.x;
    for (int p = lane; p < P; p += 32) { s_lo[warp][p] = INFINITY; s_hi[warp][p] = -INFINITY; }
    __syncwarp();
    for (int r = 0; r < 32; ++r) {
        int64_t row = t * kTile + warp * 32 + r;
        if (row >= n) break;
        const float* x = Xs + row * d;
        for (int p = 0; p < P; ++p) {
            float s = sqrtf(warp_dist2(x, Pv + (int64_t)p * d, d, lane));
            if (lane == 0) {
                s_lo[warp][p] = fminf(s_lo[warp][p], s);
                s_hi[warp][p] = fmaxf(s_hi[warp][p], s);
            }
        }
    }
    __syncthreads();
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        float a = fminf(fminf(s_lo[0][p], s_lo[1][p]), fminf(s_lo[2][p], s_lo[3][p]));
        float b = fmaxf(fmaxf(s_hi[0][p], s_hi[1][p]), fmaxf(s_hi[2][p], s_hi[3][p]));
        lo[(int64_t)p * T + t] = a;
        hi[(int64_t)p * T + t] = b;
    }
}

// Super-tile bounds: union of kSuper consecutive tiles' intervals.
__global__ void k_super_bounds(const float* __restrict__ lo, const float* __restrict__ hi, int P, int64_t T, int64_t S,
                               float* __restrict__ slo, float* __restrict__ shi)
{
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= (int64_t)P * S) return;
    int64_t p = t / S, s = t - p * S;
    float a = INFINITY, b = -INFINITY;
    for (int64_t k = s * kSuper; k < min(T, (s + 1) * kSuper); ++k) {
        a = fminf(a, lo[p * T + k]);
        b = fmaxf(b, hi[p * T + k]);
    }
    slo[p * S + s] = a;
    shi[p * S + s] = b;
}

// True when some pivot separates the two intervals by more than the radius plus
// the rounding slack.  relerr bounds the relative error of every computed distance
// (pivot distances here and the reference's sequential L2), so skipping is exact.
__device__ __forceinline__ bool separated(float loA, float hiA, float loB, float hiB, float radius, float relerr)
{
    float g1 = loB - hiA, g2 = loA - hiB;
    float thr1 = radius + relerr * (radius + loB + hiA) + 1e-30f;
    float thr2 = radius + relerr * (radius + loA + hiB) + 1e-30f;
    return (g1 > thr1) || (g2 > thr2);
}

// Level 1 of the pruning: super-tile pairs (I <= J).  blockIdx.y = I.
__global__ void k_prune_super(const float* __restrict__ slo, const float* __restrict__ shi, int P, int64_t S,
                              float radius, float relerr, int2* __restrict__ out, unsigned long long* __restrict__ count,
                              unsigned long long cap)
{
    int64_t I = blockIdx.y;
    int64_t J = I + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    bool keep = false;
    if (J < S) {
        keep = true;
        for (int p = 0; p < P; ++p) {
            if (separated(slo[p * S + I], shi[p * S + I], slo[p * S + J], shi[p * S + J], radius, relerr)) {
                keep = false;
                break;
            }
        }
    }
    unsigned mask = __ballot_sync(0xffffffffu, keep);
    if (!mask) return;
    int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(count, (unsigned long long)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (keep) {
        unsigned long long pos = base + __popc(mask & ((1u << lane) - 1u));
        if (pos < cap) out[pos] = make_int2((int)I, (int)J);
    }
}

// Level 2: the tile pairs (i <= j) inside each surviving super pair.  One warp per
// super pair, kSuper*kSuper = 64 tile pairs, two per lane.
__global__ void k_prune_tiles(const int2* __restrict__ supers, const unsigned long long* __restrict__ nsup_ptr,
                              unsigned long long sup_cap, const float* __restrict__ lo, const float* __restrict__ hi,
                              int P, int64_t T, float radius, float relerr, int2* __restrict__ out,
                              unsigned long long* __restrict__ count, unsigned long long cap)
{
    unsigned long long nsup = min(*nsup_ptr, sup_cap);
    int lane = threadIdx.x & 31;
    int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = warp; w < (int64_t)nsup; w += nwarps) {
        int2 sp = supers[w];
        for (int half = 0; half < 2; ++half) {
            int q = lane + 32 * half;
            int64_t i = (int64_t)sp.x * kSuper + (q / kSuper);
            int64_t j = (int64_t)sp.y * kSuper + (q % kSuper);
            bool keep = (i < T) && (j < T) && (i <= j);
            if (keep) {
                for (int p = 0; p < P; ++p) {
                    if (separated(lo[p * T + i], hi[p * T + i], lo[p * T + j], hi[p * T + j], radius, relerr)) {
                        keep = false;
                        break;
                    }
                }
            }
            unsigned mask = __ballot_sync(0xffffffffu, keep);
            if (!mask) continue;
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(count, (unsigned long long)__popc(mask));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (keep) {
                unsigned long long pos = base + __popc(mask & ((1u << lane) - 1u));
                if (pos < cap) out[pos] = make_int2((int)i, (int)j);
            }
        }
    }
}

// Block-aggregated append: every thread counts its hits, one atomicAdd per block
// reserves space, and each thread writes its hits at its prefix offset.  Returns
// the thread's first output slot.
__device__ __forceinline__ unsigned long long block_reserve(int nhit, unsigned long long* __restrict__ ecount)
{
    __shared__ int s_warp[32];
    __shared__ unsigned long long s_base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    int incl = nhit;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int k = 0; k < nw; ++k) { int t = s_warp[k]; s_warp[k] = acc; acc += t; }
        s_base = acc ? atomicAdd(ecount, (unsigned long long)acc) : 0ull;
    }
    __syncthreads();
    unsigned long long pos = s_base + (unsigned long long)(s_warp[warp] + incl - nhit);
    __syncthreads();  // s_warp / s_base are reused by the next call
    return pos;
}

// FP32-direct tile evaluation.  Block = 256 threads = one 128x128 tile pair at a
// time (persistent over the pair list).  Thread (ty, tx) owns rows ty*8..+8 and
// columns tx*8..+8.  Dimensions are consumed in chunks of kKC in increasing order,
// so every pair's sum is the reference's sequential sum, term by term.
constexpr int kKC = 32;

__global__ void __launch_bounds__(256) k_tiles_fp32(const float* __restrict__ Xs, int64_t n, int d,
                                                    const int2* __restrict__ pairs,
                                                    const unsigned long long* __restrict__ npairs_ptr,
                                                    unsigned long long pair_cap, float radius,
                                                    uint32_t* __restrict__ eu, uint32_t* __restrict__ ev,
                                                    float* __restrict__ ew, unsigned long long* __restrict__ ecount,
                                                    unsigned long long cap)
{
    __shared__ __align__(16) float As[kKC][kTile + 4];
    __shared__ __align__(16) float Bs[kKC][kTile + 4];
    const int tid = threadIdx.x;
    const int ty = tid >> 4, tx = tid & 15;
    const unsigned long long npairs = min(*npairs_ptr, pair_cap);
    for (unsigned long long w = blockIdx.x; w < npairs; w += gridDim.x) {
        const int2 tp = pairs[w];
        const int64_t i0 = (int64_t)tp.x * kTile, j0 = (int64_t)tp.y * kTile;
        float acc[8][8];
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int c = 0; c < 8; ++c) acc[r][c] = 0.f;
        for (int k0 = 0; k0 < d; k0 += kKC) {
            __syncthreads();
            for (int idx = tid; idx < kTile * kKC; idx += 256) {
                int r = idx / kKC, c = idx % kKC;
                int k = k0 + c;
                As[c][r] = (k < d) ? Xs[(i0 + r) * d + k] : 0.f;
                Bs[c][r] = (k < d) ? Xs[(j0 + r) * d + k] : 0.f;
            }
            __syncthreads();
#pragma unroll 4
            for (int k = 0; k < kKC; ++k) {
                float4 a0 = *reinterpret_cast<const float4*>(&As[k][ty * 8]);
                float4 a1 = *reinterpret_cast<const float4*>(&As[k][ty * 8 + 4]);
                float4 b0 = *reinterpret_cast<const float4*>(&Bs[k][tx * 8]);
                float4 b1 = *reinterpret_cast<const float4*>(&Bs[k][tx * 8 + 4]);
                float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
                for (int r = 0; r < 8; ++r)
#pragma unroll
                    for (int c = 0; c < 8; ++c) acc[r][c] = l2seq_acc(acc[r][c], a[r], b[c]);
            }
        }
        // epilogue: count, reserve with one atomic per block, then write
        int nhit = 0;
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                int64_t gi = i0 + ty * 8 + r, gj = j0 + tx * 8 + c;
                acc[r][c] = __fsqrt_rn(acc[r][c]);
                bool ok = gi < n && gj < n && (tp.x != tp.y || gi < gj) && acc[r][c] <= radius;
                nhit += ok;
            }
        unsigned long long pos = block_reserve(nhit, ecount);
#pragma unroll
        for (int r = 0; r < 8; ++r)
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                int64_t gi = i0 + ty * 8 + r, gj = j0 + tx * 8 + c;
                bool ok = gi < n && gj < n && (tp.x != tp.y || gi < gj) && acc[r][c] <= radius;
                if (ok) {
                    if (pos < cap) {
                        eu[pos] = (uint32_t)gi;
                        ev[pos] = (uint32_t)gj;
                        ew[pos] = acc[r][c];
                    }
                    ++pos;
                }
            }
    }
}

// Sorted-index edges -> id edges with u < v.
__global__ void k_finalize_edges(const uint32_t* __restrict__ si, const uint32_t* __restrict__ sj,
                                 const float* __restrict__ sw, int64_t m, const int32_t* __restrict__ perm,
                                 const int64_t* __restrict__ ids, int64_t* __restrict__ u, int64_t* __restrict__ v,
                                 float* __restrict__ w)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        int32_t a = perm[si[e]], b = perm[sj[e]];
        int64_t ia = ids ? ids[a] : (int64_t)a;
        int64_t ib = ids ? ids[b] : (int64_t)b;
        u[e] = ia < ib ? ia : ib;
        v[e] = ia < ib ? ib : ia;
        w[e] = sw[e];
    }
}

// ------------------------------------------------------------------------------------------------
// host side

static int grid_for(rnng_ctx* c, int64_t work, int per_block, int waves = 8)
{
    int64_t g = ceil_div(work, per_block);
    int64_t cap = (int64_t)c->num_sms * waves;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

void sort_pairs_u64(rnng_ctx* c, uint64_t* keys_in, uint64_t* keys_out, int32_t* vals_in, int32_t* vals_out,
                    int64_t n, int end_bit)
{
    size_t tmp = 0;
    RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, keys_in, keys_out, vals_in, vals_out, (int)n, 0, end_bit,
                                              c->stream));
    c->cub_tmp.reserve(tmp);
    RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, keys_in, keys_out, vals_in, vals_out, (int)n, 0,
                                              end_bit, c->stream));
}

static int bits_for(int64_t v)
{
    int b = 1;
    while ((int64_t(1) << b) < v + 1) ++b;
    return b;
}

Layout build_layout(rnng_ctx* c, const float* dX, int64_t n, int d, float radius)
{
    Layout L;
    L.n = n;
    L.d = d;
    L.T = ceil_div(n, kTile);
    L.n_pad = L.T * kTile;
    L.S = ceil_div(L.T, kSuper);
    cudaStream_t s = c->stream;

    // ---- level 1
    int64_t leaves = std::max<int64_t>(1, std::min<int64_t>(n / kLeafTarget, kMaxLeaves));
    int m1 = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)std::ceil(std::sqrt((double)leaves)), kMaxSub));
    if (m1 > n) m1 = (int)n;
    L.m1 = m1;
    c->aux0.reserve(sizeof(int32_t) * (m1 + 1));
    c->aux1.reserve(sizeof(float) * (size_t)m1 * d);
    int32_t* l1_idx = c->aux0.as<int32_t>();
    float* l1_rows = c->aux1.as<float>();
    k_strided_index<<<ceil_div(m1, 256), 256, 0, s>>>(l1_idx, m1, n);
    k_gather_rows<<<grid_for(c, (int64_t)m1 * d, 256), 256, 0, s>>>(dX, d, l1_idx, m1, l1_rows);
    c->keys.reserve(sizeof(uint64_t) * n);
    c->keys_alt.reserve(sizeof(uint64_t) * n);
    c->perm.reserve(sizeof(int32_t) * L.n_pad);
    c->perm_alt.reserve(sizeof(int32_t) * n);
    uint64_t* k1 = c->keys.as<uint64_t>();
    uint64_t* k1s = c->keys_alt.as<uint64_t>();
    int32_t* v1 = c->perm_alt.as<int32_t>();
    int32_t* order1 = c->perm.as<int32_t>();
    size_t smem1 = ((int64_t)m1 * d * 4 <= 48 * 1024) ? (size_t)m1 * d * 4 : 0;
    k_assign_level1<<<grid_for(c, n * 32, 256), 256, smem1, s>>>(dX, n, d, l1_rows, m1, k1, v1);
    sort_pairs_u64(c, k1, k1s, v1, order1, n, 32 + bits_for(m1));

    // ---- level 2
    c->aux2.reserve(sizeof(int32_t) * (4 * (size_t)m1 + 4));
    int32_t* cstart = c->aux2.as<int32_t>();
    int32_t* cend = cstart + m1;
    int32_t* m2 = cend + m1;
    int32_t* m2_off = m2 + m1;
    RNNG_CUDA(cudaMemsetAsync(cstart, 0, sizeof(int32_t) * 2 * m1, s));
    k_cell_bounds<<<ceil_div(n, 256), 256, 0, s>>>(k1s, n, cstart, cend);
    k_level2_plan<<<1, 1024, 0, s>>>(cstart, cend, m1, n, leaves, m2, m2_off);
    int64_t max_sub = (int64_t)m1 * kMaxSub;
    c->aux3.reserve(sizeof(int32_t) * max_sub);
    c->aux4.reserve(sizeof(float) * (size_t)max_sub * d);
    int32_t* sub_idx = c->aux3.as<int32_t>();
    float* sub_rows = c->aux4.as<float>();
    k_level2_landmarks<<<m1, 128, 0, s>>>(cstart, cend, m2, m2_off, m1, order1, sub_idx);
    int32_t total_sub = 0;
    RNNG_CUDA(cudaMemcpyAsync(&total_sub, m2_off + m1, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    RNNG_CUDA(cudaStreamSynchronize(s));
    L.num_cells = total_sub;
    k_gather_rows<<<grid_for(c, (int64_t)total_sub * d, 256), 256, 0, s>>>(dX, d, sub_idx, total_sub, sub_rows);
    uint64_t* k2 = k1;  // reuse
    int32_t* v2 = v1;
    k_assign_level2<<<grid_for(c, n * 32, 256), 256, 0, s>>>(dX, n, d, k1s, order1, sub_rows, m2, m2_off, k2, v2);
    int32_t* perm = order1;  // final order overwrites the level-1 order
    sort_pairs_u64(c, k2, k1s, v2, perm, n, 32 + bits_for(total_sub));
    L.perm = perm;

    // ---- sorted points
    c->x_sorted.reserve(sizeof(float) * (size_t)L.n_pad * d);
    L.Xs = c->x_sorted.as<float>();
    k_gather_sorted<<<grid_for(c, L.n_pad * d, 256), 256, 0, s>>>(dX, n, L.n_pad, d, perm, L.Xs);

    // ---- pivots: a strided subset of the leaf landmarks
    int P = (int)std::min<int64_t>(kMaxPivots, total_sub);
    L.P = P;
    c->pivots.reserve(sizeof(float) * (size_t)P * d);
    c->aux5.reserve(sizeof(int32_t) * P);
    {
        // pivot k = leaf landmark floor(k * total_sub / P): gather through sub_idx
        std::vector<int32_t> hidx(P);
        for (int k = 0; k < P; ++k) hidx[k] = (int32_t)(((int64_t)k * total_sub) / P);
        RNNG_CUDA(cudaMemcpyAsync(c->aux5.ptr, hidx.data(), sizeof(int32_t) * P, cudaMemcpyHostToDevice, s));
        k_gather_rows<<<grid_for(c, (int64_t)P * d, 256), 256, 0, s>>>(sub_rows, d, c->aux5.as<int32_t>(), P,
                                                                       c->pivots.as<float>());
        RNNG_CUDA(cudaStreamSynchronize(s));  // hidx lifetime
    }
    L.relerr = (float)((d + 16) * 1.1920928955078125e-07);  // (d+16) * 2^-23
    L.radius = radius;
    return L;
}

void compute_bounds(rnng_ctx* c, Layout& L)
{
    cudaStream_t s = c->stream;
    c->tile_lo.reserve(sizeof(float) * (size_t)L.P * L.T);
    c->tile_hi.reserve(sizeof(float) * (size_t)L.P * L.T);
    c->super_lo.reserve(sizeof(float) * (size_t)L.P * L.S);
    c->super_hi.reserve(sizeof(float) * (size_t)L.P * L.S);
    k_tile_bounds<<<(unsigned)L.T, 128, 0, s>>>(L.Xs, L.n, L.d, c->pivots.as<float>(), L.P, L.T,
                                                 c->tile_lo.as<float>(), c->tile_hi.as<float>());
    k_super_bounds<<<ceil_div((int64_t)L.P * L.S, 256), 256, 0, s>>>(c->tile_lo.as<float>(), c->tile_hi.as<float>(),
                                                                     L.P, L.T, L.S, c->super_lo.as<float>(),
                                                                     c->super_hi.as<float>());
}

void prune(rnng_ctx* c, Layout& L)
{
    cudaStream_t s = c->stream;
    c->counters.reserve(sizeof(unsigned long long) * 8);
    unsigned long long* cnt = c->counters.as<unsigned long long>();
    RNNG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * 8, s));
    // super pairs: worst case S(S+1)/2, bounded by memory; grown on overflow
    unsigned long long sup_cap = std::max<unsigned long long>(1024, (unsigned long long)L.S * 64);
    sup_cap = std::min<unsigned long long>(sup_cap, (unsigned long long)L.S * (L.S + 1) / 2);
    for (int attempt = 0; attempt < 3; ++attempt) {
        c->super_list.reserve(sizeof(int2) * sup_cap);
        RNNG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s));
        dim3 g1((unsigned)ceil_div(L.S, 256), (unsigned)L.S);
        k_prune_super<<<g1, 256, 0, s>>>(c->super_lo.as<float>(), c->super_hi.as<float>(), L.P, L.S, L.radius,
                                         L.relerr, c->super_list.as<int2>(), cnt, sup_cap);
        unsigned long long got = 0;
        RNNG_CUDA(cudaMemcpyAsync(&got, cnt, sizeof(got), cudaMemcpyDeviceToHost, s));
        RNNG_CUDA(cudaStreamSynchronize(s));
        L.super_pairs = got;
        if (got <= sup_cap) break;
        sup_cap = got;
    }
    unsigned long long tile_cap = std::max<unsigned long long>(1, L.super_pairs * (unsigned long long)(kSuper * kSuper));
    c->pair_list.reserve(sizeof(int2) * tile_cap);
    RNNG_CUDA(cudaMemsetAsync(cnt + 1, 0, sizeof(unsigned long long), s));
    k_prune_tiles<<<grid_for(c, (int64_t)L.super_pairs * 32, 256), 256, 0, s>>>(
        c->super_list.as<int2>(), cnt, L.super_pairs, c->tile_lo.as<float>(), c->tile_hi.as<float>(), L.P, L.T,
        L.radius, L.relerr, c->pair_list.as<int2>(), cnt + 1, tile_cap);
    unsigned long long got = 0;
    RNNG_CUDA(cudaMemcpyAsync(&got, cnt + 1, sizeof(got), cudaMemcpyDeviceToHost, s));
    RNNG_CUDA(cudaStreamSynchronize(s));
    L.tile_pairs = got;
    L.pairs = c->pair_list.as<int2>();
    L.d_tile_pairs = cnt + 1;
}

void run_tiles_fp32(rnng_ctx* c, Layout& L, EdgeOut& E)
{
    int grid = std::max(1, std::min<int>((int)std::min<unsigned long long>(L.tile_pairs, 1ull << 30),
                                         c->num_sms * 4));
    k_tiles_fp32<<<grid, 256, 0, c->stream>>>(L.Xs, L.n, L.d, L.pairs, L.d_tile_pairs, L.tile_pairs, L.radius, E.si,
                                              E.sj, E.w, E.count, E.cap);
    RNNG_CUDA(cudaGetLastError());
}

void finalize_edges(rnng_ctx* c, const Layout& L, const int64_t* d_ids, const EdgeOut& E, int64_t m, int64_t* u,
                    int64_t* v, float* w)
{
    if (m == 0) return;
    k_finalize_edges<<<grid_for(c, m, 256), 256, 0, c->stream>>>(E.si, E.sj, E.w, m, L.perm, d_ids, u, v, w);
}

}  // namespace rnng
