// Tile covers and exact tile-pair pruning by the triangle inequality.
//
// Every tile (128 consecutive points of the partition order) is covered by up to
// kTileBalls balls: greedy k-center groups (the first centre farthest from the tile's
// centroid, each next one the point farthest from the chosen centres, every point in the
// group of its nearest centre), each group stored as (centroid, radius).  A super-tile
// (kSuper consecutive tiles) gets kSuperBalls balls built the same way from its tiles'
// balls.  The greedy gives every separate cluster, and every stray point of another
// cluster, its own ball before it splits a cluster, so a tile that the partition mixed
// from several clusters still gets tight balls (farthest-point bisection into four balls
// left 5.2M of the 30.5M tile pairs of the 1M x 128 descriptors; these covers far fewer).
// A pair of tiles (or super-tiles) is skipped when every pair of their balls is
// separated:  |c1 - c2| (1 - relerr) > eps' + r1 + r2, with radii widened by the
// relative error of their float computation and eps' = eps * (1 + (d+8) 2^-24).
// Then no x in ball 1 and y in ball 2 can have the reference L2 <= eps, so the
// pruning never drops an edge.  This is RNNG's ghost-point reasoning
// (include/point.hpp:904, d(q, c) <= d(q, c_q) + 2r) with balls instead of cells.
//
// Leaf order: the children of every split cell are chained greedily by their
// landmarks (start at the first, always step to the nearest unvisited one), so
// cells that follow each other in the order are close and tiles rarely straddle
// far clusters.
#include <cub/cub.cuh>

#include <vector>

#include "balls.cuh"
#include "common.cuh"
#include "eps_l2.cuh"
#include "partition.cuh"

namespace rnng {

// ------------------------------------------------------------------------------------------------
// leaf chaining

constexpr int kChainMax = kFan;  // children per cell never exceed the partition fan-out

__device__ __forceinline__ int tri_index(int i, int j, int m)
{
    if (i > j) { const int t = i; i = j; j = t; }
    return i * m - i * (i + 1) / 2 + (j - i - 1);
}

// One block per parent cell: pairwise distances of its children's landmarks into
// shared memory (upper triangle; from rows staged in shared memory, a thread per pair,
// or for wide rows a warp per pair with lanes over dimensions), then one warp walks the
// greedy chain.
__global__ void __launch_bounds__(256) k_chain_leaves(const float* __restrict__ L, int d, bool staged,
                                                      const int32_t* __restrict__ m2,
                                                      const int32_t* __restrict__ m2_off, int32_t* __restrict__ rank)
{
    extern __shared__ float Dm[];  // m x m
    const int c = blockIdx.x, m = m2[c], base = m2_off[c];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if (m <= 0) return;
    if (m == 1) {
        if (threadIdx.x == 0) rank[base] = base;
        return;
    }
    if (staged) {
        // the children's landmark rows in shared memory (rows d + 1 floats apart), then one
        // thread per pair
        float* R = Dm + kChainMax * (kChainMax - 1) / 2;
        for (int e = threadIdx.x; e < m * d; e += blockDim.x) R[(e / d) * (d + 1) + e % d] = L[(int64_t)base * d + e];
        __syncthreads();
        for (int p = threadIdx.x; p < m * (m - 1) / 2; p += blockDim.x) {
            // p -> (i, j), i < j, in the order of tri_index
            int i = 0, rest = p;
            while (rest >= m - 1 - i) {
                rest -= m - 1 - i;
                ++i;
            }
            const int j = i + 1 + rest;
            const float* a = R + i * (d + 1);
            const float* b = R + j * (d + 1);
            float s0 = 0.f, s1 = 0.f;
            int k = 0;
            for (; k + 1 < d; k += 2) {
                const float t0 = a[k] - b[k], t1 = a[k + 1] - b[k + 1];
                s0 = fmaf(t0, t0, s0);
                s1 = fmaf(t1, t1, s1);
            }
            if (k < d) {
                const float t0 = a[k] - b[k];
                s0 = fmaf(t0, t0, s0);
            }
            Dm[p] = s0 + s1;
        }
    } else {
        for (int p = warp; p < m * m; p += nw) {
            const int i = p / m, j = p % m;
            if (j <= i) continue;  // warp-uniform
            const float* a = L + (int64_t)(base + i) * d;
            const float* b = L + (int64_t)(base + j) * d;
            float s = 0.f;
            for (int k = lane; k < d; k += 32) {
                const float t = a[k] - b[k];
                s = fmaf(t, t, s);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) Dm[tri_index(i, j, m)] = s;
        }
    }
    __syncthreads();
    if (warp != 0) return;
    // visited flags in registers: lane l owns landmarks l, l+32, ... (m <= kFan)
    uint32_t seen = 0;
    int cur = 0;
    if (lane == 0) {
        seen |= 1u;
        rank[base] = base;
    }
    for (int step = 1; step < m; ++step) {
        float best = INFINITY;
        int bi = m;
        for (int q = 0; q * 32 + lane < m; ++q) {
            const int j = q * 32 + lane;
            if ((seen >> q) & 1u) continue;
            const float v = Dm[tri_index(cur, j, m)];
            if (v < best || (v == best && j < bi)) { best = v; bi = j; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob < best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (bi >= m) break;
        if ((bi & 31) == lane) seen |= 1u << (bi >> 5);
        if (lane == 0) rank[base + bi] = base + step;
        cur = bi;
    }
}

// ------------------------------------------------------------------------------------------------
// covers: farthest-point (k-center) groups, shared by tile balls (over points) and super
// balls (over tile balls)
//
// Items are rows of `src` (points, or ball centres with item radii `irad`); one thread
// per item (at most kCoverItems items).  The first centre is the item farthest from the
// items' centroid; each further centre is the item farthest from all chosen centres
// (Gonzalez' greedy k-center), every item joins its nearest centre, and the greedy stops
// early once every item coincides with a centre.  In clustered data the greedy takes a
// centre in every separate cluster (and every stray point) before it splits a cluster,
// so the groups follow the clusters.  Each group is then stored as (centroid, radius),
// the radius measured from the centroid, so the ball covers its members; radii are
// widened by the relative error of their float computation (`grow`).

constexpr int kCoverItems = kTile > kSuper * kTileBalls ? kTile : kSuper * kTileBalls;
constexpr int kCoverMaxBalls = kTileBalls > kSuperBalls ? kTileBalls : kSuperBalls;
constexpr int kCoverThreads = kCoverItems;

struct CoverState {
    int label[kCoverItems];
    unsigned rad_bits[kCoverMaxBalls];  // group radius (non-negative float bits, atomicMax)
    int count[kCoverMaxBalls];
    float red_v[kCoverThreads / 32];
    int red_i[kCoverThreads / 32];
    int pick;
    float pick_v;
};

// distance of item r (row x, d floats) to row v: fmaf over the dimensions in four interleaved
// partial sums (any order is covered by the radii's widening)
__device__ __forceinline__ float row_dist(const float* __restrict__ x, const float* __restrict__ v, int d)
{
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    int k = 0;
    if ((d & 3) == 0 && ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(v)) & 15) == 0) {
        const float4* x4 = reinterpret_cast<const float4*>(x);
        const float4* v4 = reinterpret_cast<const float4*>(v);
        for (int q = 0; q < (d >> 2); ++q) {
            const float4 a = x4[q], b = v4[q];
            const float t0 = a.x - b.x, t1 = a.y - b.y, t2 = a.z - b.z, t3 = a.w - b.w;
            s0 = fmaf(t0, t0, s0);
            s1 = fmaf(t1, t1, s1);
            s2 = fmaf(t2, t2, s2);
            s3 = fmaf(t3, t3, s3);
        }
        k = d;
    } else {
#pragma unroll 4
        for (; k + 3 < d; k += 4) {
            const float t0 = x[k] - v[k], t1 = x[k + 1] - v[k + 1], t2 = x[k + 2] - v[k + 2], t3 = x[k + 3] - v[k + 3];
            s0 = fmaf(t0, t0, s0);
            s1 = fmaf(t1, t1, s1);
            s2 = fmaf(t2, t2, s2);
            s3 = fmaf(t3, t3, s3);
        }
    }
    for (; k < d; ++k) {
        const float t = x[k] - v[k];
        s0 = fmaf(t, t, s0);
    }
    return sqrtf((s0 + s1) + (s2 + s3));
}

// One item's row for the greedy's distance walks.  NQ = 0: read from memory at every walk
// (row_dist).  NQ > 0 (d = 4 NQ, every row the walks meet on a 16-byte boundary): held in
// registers as NQ float4, so a walk reads only the other row; the arithmetic is
// row_dist's 16-byte form, so the distances are the same floats.
template <int NQ>
struct ItemRow {
    float4 x[NQ];
    __device__ __forceinline__ void load(const float* __restrict__ p)
    {
        const float4* p4 = reinterpret_cast<const float4*>(p);
#pragma unroll
        for (int q = 0; q < NQ; ++q) x[q] = p4[q];
    }
    __device__ __forceinline__ float dist(const float* __restrict__ v, int) const
    {
        const float4* v4 = reinterpret_cast<const float4*>(v);
        float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            const float4 b = v4[q];
            const float t0 = x[q].x - b.x, t1 = x[q].y - b.y, t2 = x[q].z - b.z, t3 = x[q].w - b.w;
            s0 = fmaf(t0, t0, s0);
            s1 = fmaf(t1, t1, s1);
            s2 = fmaf(t2, t2, s2);
            s3 = fmaf(t3, t3, s3);
        }
        return sqrtf((s0 + s1) + (s2 + s3));
    }
};

template <>
struct ItemRow<0> {
    const float* x;
    __device__ __forceinline__ void load(const float* __restrict__ p) { x = p; }
    __device__ __forceinline__ float dist(const float* __restrict__ v, int d) const { return row_dist(x, v, d); }
};

// block-wide (max value, index) with ties to the smaller index; result in st.pick / st.pick_v
__device__ __forceinline__ void cover_argmax(CoverState& st, float v, int i)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float ov = __shfl_xor_sync(0xffffffffu, v, o);
        const int oi = __shfl_xor_sync(0xffffffffu, i, o);
        if (ov > v || (ov == v && oi < i)) {
            v = ov;
            i = oi;
        }
    }
    if (lane == 0) {
        st.red_v[warp] = v;
        st.red_i[warp] = i;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float bv = st.red_v[0];
        int bi = st.red_i[0];
        for (int w = 1; w < kCoverThreads / 32; ++w)
            if (st.red_v[w] > bv || (st.red_v[w] == bv && st.red_i[w] < bi)) {
                bv = st.red_v[w];
                bi = st.red_i[w];
            }
        st.pick = bi;
        st.pick_v = bv;
    }
    __syncthreads();
}

// Up to K groups of the n items; centres into cen[K][d] (global, owned by the block),
// radii into rad[K] (-1: no group).  `cbuf` is d floats of shared memory for the centroid.
// With `sums` (K d floats of shared memory, or null) the group centroids take one pass over
// the items instead of one per group.  NQ > 0 (ItemRow): d = 4 NQ, and src, ld, cbuf and
// cen keep every row on a 16-byte boundary.
template <int NQ>
__device__ __forceinline__ void cover_groups(CoverState& st, const float* __restrict__ src, int ld,
                                             const float* __restrict__ irad, int n, int d, int K, float grow,
                                             float* __restrict__ cbuf, float* __restrict__ sums,
                                             float* __restrict__ cen, float* __restrict__ rad)
{
    // item r is src[r ld .. r ld + d)
    const int t = threadIdx.x;
    const bool mine = t < n;
    ItemRow<NQ> xr;
    xr.load(src + (int64_t)(mine ? t : 0) * ld);
    const float ir = (mine && irad) ? irad[t] : 0.f;
    // centroid of all items
    for (int k = t; k < d; k += blockDim.x) {
        float a = 0.f;
        for (int r = 0; r < n; ++r) a += src[(int64_t)r * ld + k];
        cbuf[k] = n > 0 ? a / (float)n : 0.f;
    }
    if (t < kCoverMaxBalls) {
        st.rad_bits[t] = 0u;
        st.count[t] = 0;
    }
    __syncthreads();
    float dm = mine ? xr.dist(cbuf, d) + ir : -1.f;
    cover_argmax(st, dm, t);
    int ng = 0;
    int lab = 0;
    for (; ng < K && n > 0; ++ng) {
        const int j = st.pick;
        if (ng > 0 && !(st.pick_v > 0.f)) break;  // every item coincides with a centre
        if (mine) {
            const float dj = xr.dist(src + (int64_t)j * ld, d) + ir;
            if (ng == 0 || dj < dm) {
                dm = dj;
                lab = ng;
            }
        }
        if (ng + 1 < K) cover_argmax(st, mine ? dm : -1.f, t);
    }
    if (mine) {
        st.label[t] = lab;
        atomicAdd(&st.count[lab], 1);
    }
    if (sums)
        for (int e = t; e < ng * d; e += blockDim.x) sums[e] = 0.f;
    __syncthreads();
    // group centroids (thread k sums dimension k over the group's items), then radii
    if (sums) {
        for (int k = t; k < d; k += blockDim.x)
            for (int r = 0; r < n; ++r) sums[st.label[r] * d + k] += src[(int64_t)r * ld + k];
        __syncthreads();
        for (int e = t; e < ng * d; e += blockDim.x) {
            const int c = st.count[e / d];
            cen[e] = c ? sums[e] / (float)c : 0.f;
        }
    } else {
        for (int g = 0; g < ng; ++g) {
            const int c = st.count[g];
            for (int k = t; k < d; k += blockDim.x) {
                float a = 0.f;
                for (int r = 0; r < n; ++r)
                    if (st.label[r] == g) a += src[(int64_t)r * ld + k];
                cen[(int64_t)g * d + k] = c ? a / (float)c : 0.f;
            }
        }
    }
    __syncthreads();
    if (mine) {
        const float rr = xr.dist(cen + (int64_t)lab * d, d) + ir;
        atomicMax(&st.rad_bits[lab], __float_as_uint(rr));
    }
    __syncthreads();
    if (t < K) rad[t] = (t < ng && st.count[t] > 0) ? __uint_as_float(st.rad_bits[t]) * grow + 1e-30f : -1.f;
    __syncthreads();
}

// Row stride of a staged tile: d + 4 floats when d is a multiple of 4 (rows on 16-byte
// boundaries, so the distance walks read 16 bytes at a time, and the eight rows of a
// quarter-warp's 16-byte reads four banks apart), else d + 1 (the threads' row walks in
// distinct banks).
__host__ __device__ constexpr int tile_row_stride(int d) { return (d & 3) == 0 ? d + 4 : d + 1; }

// One block per tile.  Output: centres [T][kTileBalls][d], radii [T][kTileBalls] (-1 =
// unused).  With staged = true the tile's rows are first copied to shared memory (rows
// tile_row_stride(d) floats apart), which every pass of the greedy then reads.  Dynamic
// shared memory: d floats (centroid), kTileBalls d floats with use_sums (group sums), and
// kTile tile_row_stride(d) floats when staged.  NQ > 0: d = 4 NQ and staged (cover_groups).
template <int NQ>
__global__ void __launch_bounds__(kCoverThreads) k_tile_balls(const float* __restrict__ Xs, int64_t n, int d,
                                                              float grow, bool staged, bool use_sums,
                                                              float* __restrict__ cen, float* __restrict__ rad)
{
    __shared__ CoverState st;
    extern __shared__ __align__(16) float dsm[];
    float* cbuf = dsm;
    float* sums = dsm + ((d + 3) & ~3);  // kTileBalls d floats when use_sums
    float* tile_rows = sums + (use_sums ? kTileBalls * d : 0);
    const int64_t t = blockIdx.x;
    const int64_t r0 = t * kTile;
    const int nitems = (int)min((int64_t)kTile, n - r0);
    const float* src = Xs + r0 * d;
    int ld = d;
    if (staged) {
        const int total = nitems * d;
        ld = tile_row_stride(d);
        if ((d & 3) == 0) {
            // asynchronous 16-byte copies, all of the tile's in flight at once (a loop that
            // loads and then stores keeps about one load per thread in flight, and the tile
            // then arrives at the pace of the memory latency)
            const int nq = d >> 2;
            const float4* s4 = reinterpret_cast<const float4*>(src);
            for (int i = threadIdx.x; i < total / 4; i += blockDim.x) {
                const int r = i / nq, q = i - r * nq;  // d % 4 == 0: the four stay in row r
                cp_async16(tile_rows + r * ld + 4 * q, s4 + i);
            }
            cp_async_commit();
            cp_async_wait<0>();
        } else {
            for (int i = threadIdx.x; i < total; i += blockDim.x) tile_rows[(i / d) * ld + i % d] = __ldg(src + i);
        }
        __syncthreads();
        src = tile_rows;
    }
    cover_groups<NQ>(st, src, ld, nullptr, nitems, d, kTileBalls, grow, cbuf, use_sums ? sums : nullptr,
                 cen + t * kTileBalls * d, rad + t * kTileBalls);
}

// One block per super-tile: kSuperBalls balls over its tiles' valid balls (items with
// their radii).  Dynamic shared memory: d floats, plus kSuperBalls d with use_sums, plus
// the staged ball centres (64 (d + 4) floats) when d is a multiple of 4 up to 128.
// NQ > 0: d = 4 NQ (staged).
template <int NQ>
__global__ void __launch_bounds__(kCoverThreads) k_super_balls(const float* __restrict__ tcen,
                                                               const float* __restrict__ trad, int64_t T, int d,
                                                               float grow, bool use_sums, float* __restrict__ work,
                                                               float* __restrict__ scen, float* __restrict__ srad)
{
    __shared__ CoverState st;
    __shared__ float irad[kSuper * kTileBalls];
    __shared__ int src_ball[kSuper * kTileBalls];
    __shared__ int wcount[kCoverThreads / 32];
    extern __shared__ __align__(16) float dsm[];
    static_assert(kCoverThreads >= kSuper * kTileBalls, "one thread per tile ball of the super-tile");
    const int64_t s = blockIdx.x;
    const int64_t t0 = s * kSuper, t1 = min(T, t0 + kSuper);
    // the valid tile balls, compacted in ball order (ballot and warp counts)
    const int bi = threadIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool valid = bi < (int)(t1 - t0) * kTileBalls && trad[t0 * kTileBalls + bi] >= 0.f;
    const unsigned bal = __ballot_sync(0xffffffffu, valid);
    if (lane == 0) wcount[warp] = __popc(bal);
    __syncthreads();
    int pos = __popc(bal & ((1u << lane) - 1u)), m = 0;
    for (int w = 0; w < kCoverThreads / 32; ++w) {
        if (w < warp) pos += wcount[w];
        m += wcount[w];
    }
    if (valid) {
        irad[pos] = trad[t0 * kTileBalls + bi];
        src_ball[pos] = bi;
    }
    __syncthreads();
    float* cbuf = dsm;
    float* sums = use_sums ? dsm + ((d + 3) & ~3) : nullptr;
    // their centres: staged in shared memory 16 bytes at a time (rows d + 4 floats apart)
    // when d is a multiple of 4 and at most 128, else compacted in the global workspace
    const bool staged = (d & 3) == 0 && d <= 128;
    float* items;
    int ld;
    if (staged) {
        items = dsm + ((d + 3) & ~3) + (use_sums ? kSuperBalls * d : 0);
        ld = d + 4;
        const int nq = d >> 2;
        const float4* c4 = reinterpret_cast<const float4*>(tcen);
        for (int e = threadIdx.x; e < m * nq; e += blockDim.x) {
            const int i = e / nq, q = e - i * nq;
            cp_async16(items + i * ld + 4 * q, c4 + (t0 * kTileBalls + src_ball[i]) * nq + q);
        }
        cp_async_commit();
        cp_async_wait<0>();
    } else {
        items = work + s * (int64_t)kSuper * kTileBalls * d;
        ld = d;
        for (int i = 0; i < m; ++i)
            for (int j = threadIdx.x; j < d; j += blockDim.x)
                items[(int64_t)i * d + j] = tcen[(t0 * kTileBalls + src_ball[i]) * (int64_t)d + j];
    }
    __syncthreads();
    cover_groups<NQ>(st, items, ld, irad, m, d, kSuperBalls, grow, cbuf, sums, scen + s * kSuperBalls * d,
                 srad + s * kSuperBalls);
}

// ------------------------------------------------------------------------------------------------
// pruning

// Level 1: all super-ball pairs as 128 x 32 distance blocks; a close ball pair marks
// its super-tile pair (I <= J) in an S x S bitmap.
__global__ void __launch_bounds__(256) k_super_close(const float* __restrict__ scen, const float* __restrict__ srad,
                                                     int64_t NB, int d, float eps_p, float shrink,
                                                     uint32_t* __restrict__ bitmap, int64_t S)
{
    __shared__ __align__(16) DistSmem sm;
    const int64_t r0 = (int64_t)blockIdx.x * kDRows, c0 = (int64_t)blockIdx.y * kDCols;
    if (c0 + kDCols <= r0 - kSuperBalls) return;  // strictly below the diagonal of owners
    float acc[4][4];
    dist_block(sm, scen, nullptr, r0, NB, d, scen, c0, NB, acc);
    const int ty = threadIdx.x >> 3, tx = threadIdx.x & 7;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int64_t row = r0 + ty * 4 + r;
        if (row >= NB) continue;
        const float rr = srad[row];
        if (rr < 0.f) continue;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int64_t col = c0 + tx * 4 + c;
            if (col >= NB) continue;
            const int64_t I = row / kSuperBalls, J = col / kSuperBalls;
            if (I > J) continue;
            const float rc = srad[col];
            if (rc < 0.f) continue;
            if (sqrtf(acc[r][c]) * shrink <= eps_p + rr + rc) {
                const int64_t bit = I * S + J;
                atomicOr(&bitmap[bit >> 5], 1u << (bit & 31));
            }
        }
    }
}

__global__ void k_bitmap_pairs(const uint32_t* __restrict__ bitmap, int64_t S, int2* __restrict__ out,
                               unsigned long long* __restrict__ count, unsigned long long cap)
{
    const int64_t words = (S * S + 31) / 32;
    for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < words; w += (int64_t)gridDim.x * blockDim.x) {
        uint32_t m = bitmap[w];
        if (!m) continue;
        const unsigned long long base = atomicAdd(count, (unsigned long long)__popc(m));
        unsigned long long pos = base;
        while (m) {
            const int b = __ffs(m) - 1;
            m &= m - 1;
            const int64_t bit = w * 32 + b;
            if (pos < cap) out[pos] = make_int2((int)(bit / S), (int)(bit % S));
            ++pos;
        }
    }
}

// Shared memory of the tensor-core pruning kernels: two buffers of a column block of 64
// BF16 ball rows (padded by 64 bytes, so that the fragment reads of a quarter-warp, two
// rows of four 16-byte columns, fall in distinct banks) and the balls' float4 terms.
template <int KP>
struct TileCloseSmem {
    static constexpr int rowq = 4 * KP;         // uint4 per BF16 ball row (dp / 8)
    static constexpr int srow = rowq + 4;       // staged row stride in uint4
    static constexpr int buf = 64 * srow + 64;  // uint4 per buffer: 64 rows, then the balls' float4 terms
    static constexpr size_t bytes = 2 * (size_t)buf * sizeof(uint4);
};

// Level 1 on the tensor cores (d <= 256): the same BF16 ball test as k_tile_close_mma
// (below) over all pairs of super balls.  Block pairs (RB <= CB) of four super-tiles
// (64 balls) each, taken as contiguous ranges of the row-major upper triangle per CUDA
// block; warp w takes the 16 balls of row super-tile 4 RB + w against the 64 of the
// column block, keeps the row block's A fragments in registers while RB lasts, and marks
// super-tile pair (I, J), I <= J, in the S x S bitmap when any of its ball pairs passes.
// The next pair's column block is staged in shared memory (cp.async) while the current
// one is multiplied.
template <int KP>
__global__ void __launch_bounds__(128) k_super_close_mma(const uint4* __restrict__ cb, const float4* __restrict__ binfo,
                                                         int64_t S, float eps_p, float kappa,
                                                         uint32_t* __restrict__ bitmap)
{
    using SM = TileCloseSmem<KP>;  // the same staging: a column block of 64 balls, two buffers
    constexpr int rowq = SM::rowq, srow = SM::srow;
    extern __shared__ uint4 ssm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    const int64_t nR = (S + 3) / 4;
    const unsigned long long total = (unsigned long long)nR * (nR + 1) / 2;
    const unsigned long long per = (total + gridDim.x - 1) / gridDim.x;
    const unsigned long long p0 = (unsigned long long)blockIdx.x * per, p1 = min(total, p0 + per);
    if (p0 >= p1) return;
    // (RB, CB) of p0: row RB holds nR - RB block pairs
    int64_t RB = 0;
    unsigned long long first = 0;  // index of (RB, RB)
    {
        const double a = 2.0 * (double)nR + 1.0;
        RB = (int64_t)((a - sqrt(a * a - 8.0 * (double)p0)) * 0.5);
        if (RB < 0) RB = 0;
        if (RB >= nR) RB = nR - 1;
        auto row_first = [&](int64_t r) { return (unsigned long long)(r * nR - r * (r - 1) / 2); };
        while (RB > 0 && row_first(RB) > p0) --RB;
        while (RB + 1 < nR && row_first(RB + 1) <= p0) ++RB;
        first = row_first(RB);
    }
    int64_t CB = RB + (int64_t)(p0 - first);
    // column block cbk into buffer bsel (one commit group)
    auto stage = [&](int64_t cbk, int bsel) {
        const int64_t rbb = cbk * 64;
        const uint4* src = cb + rbb * rowq;
        uint4* dst = ssm + bsel * SM::buf;
        for (int i = threadIdx.x; i < 64 * rowq; i += blockDim.x) {
            const int r = i / rowq, q = i - r * rowq;
            cp_async16(dst + r * srow + q, src + i);
        }
        if (threadIdx.x < 64) cp_async16(dst + 64 * srow + threadIdx.x, binfo + rbb + threadIdx.x);
        cp_async_commit();
    };
    int64_t cur = -1;
    uint4 a0[KP], a1[KP];
    float4 x0 = make_float4(0.f, 0.f, 0.f, -1.f), x1 = x0;
    stage(CB, 0);
    for (unsigned long long p = p0; p < p1; ++p) {
        const int bsel = (int)((p - p0) & 1);
        // the next pair's column block, staged while this pair is multiplied
        const int64_t CBn = CB + 1 < nR ? CB + 1 : RB + 1;
        if (p + 1 < p1) {
            stage(CBn, bsel ^ 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const uint4* bs = ssm + bsel * SM::buf;
        const float4* ys = reinterpret_cast<const float4*>(bs + 64 * srow);
        const int64_t ra = RB * 64 + 16 * warp;
        if (RB != cur) {
            const uint4* pa = cb + (ra + g) * rowq + t;
#pragma unroll
            for (int kp = 0; kp < KP; ++kp) {
                a0[kp] = pa[4 * kp];
                a1[kp] = pa[8 * rowq + 4 * kp];
            }
            x0 = binfo[ra + g];
            x1 = binfo[ra + 8 + g];
            cur = RB;
        }
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[nt][q] = 0.f;
        const uint4* pb = bs + g * srow + t;
#pragma unroll
        for (int kp = 0; kp < KP; ++kp) {
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const uint4 b = pb[(8 * nt) * srow + 4 * kp];
                mma_bf16_16816(acc[nt], a0[kp].x, a1[kp].x, a0[kp].y, a1[kp].y, b.x, b.y);
                mma_bf16_16816(acc[nt], a0[kp].z, a1[kp].z, a0[kp].w, a1[kp].w, b.z, b.w);
            }
        }
        // acc[nt][2h + e]: row ball 8 h + g of super-tile 4 RB + warp, column ball 8 nt + 2 t + e
        // of the column block: super-tile 4 CB + nt / 2
        uint32_t msk = 0;  // bit c: column super-tile 4 CB + c
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const float4 y = ys[8 * nt + 2 * t + e];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float4 x = h ? x1 : x0;
                    const float D = fmaf(-2.f, acc[nt][2 * h + e], x.x + y.x);
                    const float E = eps_p + x.w + y.w + x.y + y.y;
                    const float R = fmaf(E, E, x.z + y.z);
                    const bool keep = x.w >= 0.f && y.w >= 0.f && D <= R + kappa * (x.x + y.x + R);
                    msk |= (keep ? 1u : 0u) << (nt >> 1);
                }
            }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) msk |= __shfl_xor_sync(0xffffffffu, msk, o);
        if (lane < 4 && ((msk >> lane) & 1u)) {
            const int64_t I = 4 * RB + warp, J = 4 * CB + lane;
            if (I < S && J < S && I <= J) {
                const int64_t bit = I * S + J;
                atomicOr(&bitmap[bit >> 5], 1u << (bit & 31));
            }
        }
        if (CB + 1 < nR) {
            ++CB;
        } else {
            ++RB;
            CB = RB;
        }
        __syncthreads();  // every warp is done with buffer bsel before it is staged again
    }
}

// The bitmap's pairs in row-major (I, J) order: popcount per word, an exclusive scan,
// then each word writes its pairs at its offset (so consecutive pairs share I).
__global__ void k_bitmap_count(const uint32_t* __restrict__ bitmap, int64_t words, int32_t* __restrict__ cnt)
{
    for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < words; w += (int64_t)gridDim.x * blockDim.x)
        cnt[w] = __popc(bitmap[w]);
}

__global__ void k_bitmap_emit(const uint32_t* __restrict__ bitmap, int64_t words, int64_t S,
                              const int32_t* __restrict__ off, int2* __restrict__ out, unsigned long long cap)
{
    for (int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; w < words; w += (int64_t)gridDim.x * blockDim.x) {
        uint32_t m = bitmap[w];
        unsigned long long pos = (unsigned long long)off[w];
        while (m) {
            const int b = __ffs(m) - 1;
            m &= m - 1;
            const int64_t bit = w * 32 + b;
            if (pos < cap) out[pos] = make_int2((int)(bit / S), (int)(bit % S));
            ++pos;
        }
    }
}

// Level 2: 64 threads per surviving super pair, kSPB super pairs per block.  Thread
// (ti, tj) owns tile pair (ta0 + ti, tb0 + tj) and its kTileBalls x kTileBalls ball
// pairs; the two super-tiles' ball centres are staged in shared memory kDC dimensions at
// a time, transposed so that one float4 load feeds four balls.  A tile pair survives
// when any of its ball pairs is close; each distance is the sequential fmaf sum over the
// dimensions, as at the super level.
constexpr int kNB = kSuper * kTileBalls;  // balls per super-tile
constexpr int kDC = 32;                   // dimensions per staged chunk
constexpr int kSPB = 2;                   // super pairs per block
static_assert(kTileBalls % 4 == 0, "tile balls are staged four at a time");

__global__ void __launch_bounds__(64 * kSPB) k_tile_close(const int2* __restrict__ supers,
                                                          const unsigned long long* __restrict__ nsup_ptr,
                                                          unsigned long long sup_cap, const float* __restrict__ tcen,
                                                          const float* __restrict__ trad, int64_t T, int d,
                                                          float eps_p, float shrink, int2* __restrict__ out,
                                                          unsigned long long* __restrict__ count,
                                                          unsigned long long cap)
{
    __shared__ __align__(16) float ca[kSPB][kDC][kNB + 4], cb[kSPB][kDC][kNB + 4];
    const unsigned long long nsup = min(*nsup_ptr, sup_cap);
    const int sp = threadIdx.x >> 6;       // super pair of this block's kSPB
    const int t = threadIdx.x & 63;
    const int ti = t >> 3, tj = t & 7;     // tile pair inside the super pair
    for (unsigned long long w0 = (unsigned long long)blockIdx.x * kSPB; w0 < nsup;
         w0 += (unsigned long long)gridDim.x * kSPB) {
        const unsigned long long w = w0 + sp;
        const bool live = w < nsup;
        const int2 spair = live ? supers[w] : make_int2(0, 0);
        const int64_t ta0 = (int64_t)spair.x * kSuper, tb0 = (int64_t)spair.y * kSuper;
        float acc[kTileBalls][kTileBalls];
#pragma unroll
        for (int x = 0; x < kTileBalls; ++x)
#pragma unroll
            for (int y = 0; y < kTileBalls; ++y) acc[x][y] = 0.f;
        for (int k0 = 0; k0 < d; k0 += kDC) {
            __syncthreads();
            // stage: kNB balls x kDC dims per side as float4 along the dimension
            for (int idx = t; idx < kNB * (kDC / 4); idx += 64) {
                const int ball = idx / (kDC / 4), q4 = idx % (kDC / 4), k = k0 + 4 * q4;
                const int64_t t1 = ta0 + ball / kTileBalls, t2 = tb0 + ball / kTileBalls;
                float4 va = make_float4(0.f, 0.f, 0.f, 0.f), vb = va;
                if (live && t1 < T) {
                    const float* src = tcen + (t1 * kTileBalls + ball % kTileBalls) * (int64_t)d;
                    if (k + 3 < d && (d & 3) == 0) va = *reinterpret_cast<const float4*>(src + k);
                    else {
                        va.x = k < d ? src[k] : 0.f;
                        va.y = k + 1 < d ? src[k + 1] : 0.f;
                        va.z = k + 2 < d ? src[k + 2] : 0.f;
                        va.w = k + 3 < d ? src[k + 3] : 0.f;
                    }
                }
                if (live && t2 < T) {
                    const float* src = tcen + (t2 * kTileBalls + ball % kTileBalls) * (int64_t)d;
                    if (k + 3 < d && (d & 3) == 0) vb = *reinterpret_cast<const float4*>(src + k);
                    else {
                        vb.x = k < d ? src[k] : 0.f;
                        vb.y = k + 1 < d ? src[k + 1] : 0.f;
                        vb.z = k + 2 < d ? src[k + 2] : 0.f;
                        vb.w = k + 3 < d ? src[k + 3] : 0.f;
                    }
                }
                ca[sp][4 * q4 + 0][ball] = va.x;
                ca[sp][4 * q4 + 1][ball] = va.y;
                ca[sp][4 * q4 + 2][ball] = va.z;
                ca[sp][4 * q4 + 3][ball] = va.w;
                cb[sp][4 * q4 + 0][ball] = vb.x;
                cb[sp][4 * q4 + 1][ball] = vb.y;
                cb[sp][4 * q4 + 2][ball] = vb.z;
                cb[sp][4 * q4 + 3][ball] = vb.w;
            }
            __syncthreads();
            const int kk_end = min(kDC, d - k0);
#pragma unroll 2
            for (int kk = 0; kk < kk_end; ++kk) {
                float av[kTileBalls], bv[kTileBalls];
#pragma unroll
                for (int q = 0; q < kTileBalls / 4; ++q) {
                    const float4 a4 = *reinterpret_cast<const float4*>(&ca[sp][kk][ti * kTileBalls + 4 * q]);
                    const float4 b4 = *reinterpret_cast<const float4*>(&cb[sp][kk][tj * kTileBalls + 4 * q]);
                    av[4 * q] = a4.x; av[4 * q + 1] = a4.y; av[4 * q + 2] = a4.z; av[4 * q + 3] = a4.w;
                    bv[4 * q] = b4.x; bv[4 * q + 1] = b4.y; bv[4 * q + 2] = b4.z; bv[4 * q + 3] = b4.w;
                }
#pragma unroll
                for (int x = 0; x < kTileBalls; ++x)
#pragma unroll
                    for (int y = 0; y < kTileBalls; ++y) {
                        const float df = av[x] - bv[y];
                        acc[x][y] = fmaf(df, df, acc[x][y]);
                    }
            }
        }
        const int64_t i = ta0 + ti, j = tb0 + tj;
        bool keep = false;
        if (live && i < T && j < T && i <= j) {
#pragma unroll
            for (int x = 0; x < kTileBalls; ++x) {
                const float ra = trad[i * kTileBalls + x];
#pragma unroll
                for (int y = 0; y < kTileBalls; ++y) {
                    const float rb = trad[j * kTileBalls + y];
                    if (ra >= 0.f && rb >= 0.f && sqrtf(acc[x][y]) * shrink <= eps_p + ra + rb) keep = true;
                }
            }
        }
        const unsigned ball = __ballot_sync(0xffffffffu, keep);
        const int lane = threadIdx.x & 31;
        unsigned long long base = 0;
        if (lane == 0 && ball) base = atomicAdd(count, (unsigned long long)__popc(ball));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (keep) {
            const unsigned long long pos = base + __popc(ball & ((1u << lane) - 1u));
            if (pos < cap) out[pos] = make_int2((int)i, (int)j);
        }
    }
}

// Level 2 on the tensor cores (d <= 256): four warps per surviving super pair compute
// the kSB x kSB Gram block of the two super-tiles' BF16 ball centres with mma.sync
// (m16n8k16, FP32 accumulation; warp w takes row balls 16 w .. 16 w + 15) and keep a
// tile pair when one of its kTileBalls x kTileBalls ball pairs passes
//
//     n_a + n_b - 2 g  <=  (eps' + r_a + r_b + a_a + a_b)^2 + q_a + q_b   (+ relative slack)
//
// where n is the norm of the BF16 centre, a >= its distance to the shifted FP32 centre
// and q its share of the tensor-core accumulation error (bf16_row), exactly the BF16
// Gram candidate test with eps' widened by the two radii.  A pair with
// |c_a - c_b| <= eps' + r_a + r_b therefore always passes, so no tile pair holding an
// edge is dropped.  The k order inside each 32-column group is permuted identically
// for both operands (a dot product does not depend on it) so that every lane fetches
// its fragments with 16-byte loads: lane (g, t) reads columns 8t .. 8t + 7, which feed
// k-slots {2t, 2t+1, 2t+8, 2t+9} of two consecutive k-steps.
constexpr int kSB = kSuper * kTileBalls;  // balls per super-tile (64)
static_assert(kTileBalls == 8 && kSB == 64, "the warp layout of k_tile_close_mma: 16 row balls = 2 tiles per warp");

// KP = dp / 32 k-groups.  Block b takes the contiguous range b of the super-pair list
// (row-major, so consecutive pairs share their row super-tile) and keeps the row
// super-tile's A fragments in registers while it lasts.  The column super-tile's 64 ball
// rows and their terms are staged in shared memory by cp.async, the next pair's while
// the current one is multiplied.
template <int KP>
__global__ void __launch_bounds__(128) k_tile_close_mma(const int2* __restrict__ supers,
                                                        const unsigned long long* __restrict__ nsup_ptr,
                                                        unsigned long long sup_cap, const uint4* __restrict__ cb,
                                                        const float4* __restrict__ binfo, int64_t T, float eps_p,
                                                        float kappa, int2* __restrict__ out,
                                                        unsigned long long* __restrict__ count, unsigned long long cap)
{
    using SM = TileCloseSmem<KP>;
    constexpr int rowq = SM::rowq, srow = SM::srow;
    extern __shared__ uint4 tsm[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
    const unsigned long long nsup = min(*nsup_ptr, sup_cap);
    const unsigned long long per = (nsup + gridDim.x - 1) / gridDim.x;
    const unsigned long long w0 = (unsigned long long)blockIdx.x * per, w1 = min(nsup, w0 + per);
    // the column super-tile of pair w into buffer bsel (one commit group)
    auto stage = [&](unsigned long long w, int bsel) {
        const int64_t rb = (int64_t)supers[w].y * kSB;
        const uint4* src = cb + rb * rowq;
        uint4* dst = tsm + bsel * SM::buf;
        for (int i = threadIdx.x; i < kSB * rowq; i += blockDim.x) {
            const int r = i / rowq, q = i - r * rowq;
            cp_async16(dst + r * srow + q, src + i);
        }
        if (threadIdx.x < kSB) cp_async16(dst + kSB * srow + threadIdx.x, binfo + rb + threadIdx.x);
        cp_async_commit();
    };
    int cur = -1;
    uint4 a0[KP], a1[KP];
    float4 x0 = make_float4(0.f, 0.f, 0.f, -1.f), x1 = x0;
    if (w0 < w1) stage(w0, 0);
    for (unsigned long long w = w0; w < w1; ++w) {
        const int bsel = (int)((w - w0) & 1);
        if (w + 1 < w1) {
            stage(w + 1, bsel ^ 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const uint4* bs = tsm + bsel * SM::buf;
        const float4* ys = reinterpret_cast<const float4*>(bs + kSB * srow);
        const int2 sp = supers[w];
        const int64_t ra = (int64_t)sp.x * kSB + 16 * warp;  // first row ball of this warp
        if (sp.x != cur) {
            const uint4* pa = cb + (ra + g) * rowq + t;
#pragma unroll
            for (int kp = 0; kp < KP; ++kp) {
                a0[kp] = pa[4 * kp];
                a1[kp] = pa[8 * rowq + 4 * kp];
            }
            x0 = binfo[ra + g];
            x1 = binfo[ra + 8 + g];
            cur = sp.x;
        }
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[nt][q] = 0.f;
        const uint4* pb = bs + g * srow + t;
#pragma unroll
        for (int kp = 0; kp < KP; ++kp) {
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const uint4 b = pb[(8 * nt) * srow + 4 * kp];
                mma_bf16_16816(acc[nt], a0[kp].x, a1[kp].x, a0[kp].y, a1[kp].y, b.x, b.y);
                mma_bf16_16816(acc[nt], a0[kp].z, a1[kp].z, a0[kp].w, a1[kp].w, b.z, b.w);
            }
        }
        // acc[nt][2h + e] = row ball 16 warp + 8 h + g, column ball 8 nt + 2 t + e: row tile
        // 2 warp + h, column tile nt of the super pair
        uint32_t msk = 0;  // bit 8 h + nt
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const float4 y = ys[8 * nt + 2 * t + e];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float4 x = h ? x1 : x0;
                    const float D = fmaf(-2.f, acc[nt][2 * h + e], x.x + y.x);
                    const float E = eps_p + x.w + y.w + x.y + y.y;
                    const float R = fmaf(E, E, x.z + y.z);
                    const bool keep = x.w >= 0.f && y.w >= 0.f && D <= R + kappa * (x.x + y.x + R);
                    msk |= (keep ? 1u : 0u) << (8 * h + nt);
                }
            }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) msk |= __shfl_xor_sync(0xffffffffu, msk, o);
        // lane b < 16 reports tile pair (row tile 2 warp + b / 8, column tile b % 8)
        const int64_t i = (int64_t)sp.x * kSuper + 2 * warp + (lane >> 3);
        const int64_t j = (int64_t)sp.y * kSuper + (lane & 7);
        const bool mine = lane < 16 && ((msk >> lane) & 1u) && i < T && j < T && i <= j;
        const unsigned bal = __ballot_sync(0xffffffffu, mine);
        if (bal) {
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(count, (unsigned long long)__popc(bal));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (mine) {
                const unsigned long long pos = base + __popc(bal & ((1u << lane) - 1u));
                if (pos < cap) out[pos] = make_int2((int)i, (int)j);
            }
        }
        __syncthreads();  // every warp is done with buffer bsel before it is staged again
    }
}

// Items of the persistent Gram kernel.  The pairs are sorted by (row tile, column
// tile); inside a row they are grouped nt at a time into items {i, j0, j1} (j1 = -1 for
// a row's last odd pair or nt = 1).  The kernel's CTAs take chunks of consecutive items
// from a device-side queue in item order, so all CTAs work on neighbouring rows at any
// moment (their B tiles are shared through L2) and a CTA reloads its resident A tile at
// most once per chunk plus once per row change.
// Sort keys of the tile pairs (i, j): (i, j) for column-tile items (nt = 1, 2); for row
// pairs (nt = 3) (i / 2, j, i % 2), so that the pairs (2 r, j) and (2 r + 1, j) are adjacent.
__global__ void k_schedule_keys(const int2* __restrict__ pairs, int64_t m, int nt, uint64_t* __restrict__ keys)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < m; p += (int64_t)gridDim.x * blockDim.x) {
        const int2 q = pairs[p];
        keys[p] = nt == 3 ? ((uint64_t)(q.x >> 1) << 22) | ((uint64_t)q.y << 1) | (uint64_t)(q.x & 1)
                          : ((uint64_t)q.x << 21) | (uint64_t)q.y;
    }
}

// start[p] = 1 when sorted pair p opens an item: its offset inside its row is a multiple of
// nt (nt = 1, 2), or it is the first pair of its (row pair, column) (nt = 3).
__global__ void k_item_starts(const uint64_t* __restrict__ keys, int64_t m, int nt, int32_t* __restrict__ start)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < m; p += (int64_t)gridDim.x * blockDim.x) {
        if (nt == 3) {
            start[p] = (p == 0 || (keys[p - 1] >> 1) != (keys[p] >> 1)) ? 1 : 0;
            continue;
        }
        const uint64_t row = keys[p] >> 21;
        int64_t lo = 0, hi = p;  // first pair of this row
        while (lo < hi) {
            const int64_t mid = lo + ((hi - lo) >> 1);
            if ((keys[mid] >> 21) < row) lo = mid + 1;
            else hi = mid;
        }
        start[p] = ((p - lo) % nt) == 0 ? 1 : 0;
    }
}

__global__ void k_items(const uint64_t* __restrict__ keys, int64_t m, int nt, int64_t T,
                        const int32_t* __restrict__ start, const int32_t* __restrict__ off, int4* __restrict__ items)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < m; p += (int64_t)gridDim.x * blockDim.x) {
        if (!start[p]) continue;
        const uint64_t k = keys[p];
        if (nt == 3) {
            // {2 r, j, 2 r + 1 (-1 past the last tile), bit h: tile pair (2 r + h, j) present}
            const int r = (int)(k >> 22);
            int mask = 1 << (int)(k & 1);
            if (p + 1 < m && (keys[p + 1] >> 1) == (k >> 1)) mask |= 2;
            items[off[p]] = make_int4(2 * r, (int)((k >> 1) & 0x1fffff), 2 * (int64_t)r + 1 < T ? 2 * r + 1 : -1, mask);
            continue;
        }
        const int row = (int)(k >> 21);
        int j1 = -1;
        if (nt == 2 && p + 1 < m && (int)(keys[p + 1] >> 21) == row) j1 = (int)(keys[p + 1] & 0x1fffff);
        items[off[p]] = make_int4(row, (int)(k & 0x1fffff), j1, 0);
    }
}

// ------------------------------------------------------------------------------------------------
// host

// Bits of the largest tile index (at least 1).
static int bits_for_tiles(int64_t T)
{
    int b = 1;
    while (b < 63 && (int64_t(1) << b) < T) ++b;
    return b;
}

void chain_leaves(rnng_ctx* c, const float* lm_rows, int d, const int32_t* nchild, const int32_t* child_off,
                  int ncells, int32_t* rank)
{
    const bool staged = d <= 128;  // 64 rows of d + 1 floats next to the distances: at most 41 KB
    const size_t smem = sizeof(float) * (kChainMax * (kChainMax - 1) / 2 + (staged ? kChainMax * (d + 1) : 0));
    k_chain_leaves<<<ncells, 256, smem, c->stream>>>(lm_rows, d, staged, nchild, child_off, rank); ++c->launches;
    RNNG_CUDA(cudaGetLastError());
}

// The two cover levels (tile balls, then super balls over them) of one instance.
template <int NQ>
static void launch_covers(rnng_ctx* c, const Layout& L, float grow, bool staged, bool tsums, bool ssums, size_t tsm,
                          size_t ssm)
{
    cudaStream_t s = c->stream;
    RNNG_CUDA(cudaFuncSetAttribute(k_tile_balls<NQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
    RNNG_CUDA(cudaFuncSetAttribute(k_super_balls<NQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssm));
    k_tile_balls<NQ><<<(unsigned)L.T, kCoverThreads, tsm, s>>>(L.Xs, L.n, L.d, grow, staged, tsums,
                                                               c->tile_lo.as<float>(), c->tile_hi.as<float>());
    ++c->launches;
    k_super_balls<NQ><<<(unsigned)L.S, kCoverThreads, ssm, s>>>(c->tile_lo.as<float>(), c->tile_hi.as<float>(), L.T,
                                                                L.d, grow, ssums, c->pivots.as<float>(),
                                                                c->super_lo.as<float>(), c->super_hi.as<float>());
    ++c->launches;
}

void build_covers(rnng_ctx* c, Layout& L)
{
    cudaStream_t s = c->stream;
    const float grow = 1.f + L.relerr;
    c->tile_lo.reserve(sizeof(float) * (size_t)L.T * kTileBalls * L.d);    // tile ball centres
    c->tile_hi.reserve(sizeof(float) * (size_t)L.T * kTileBalls);          // tile ball radii
    c->super_lo.reserve(sizeof(float) * (size_t)L.S * kSuperBalls * L.d);  // super ball centres
    c->super_hi.reserve(sizeof(float) * (size_t)L.S * kSuperBalls);        // super ball radii
    c->pivots.reserve(sizeof(float) * (size_t)L.S * kSuper * kTileBalls * L.d);  // compaction workspace
    // tiles staged in shared memory up to 128 dimensions (64 KB; larger tiles read through L1)
    const bool staged = L.d <= 128;
    const size_t csm = sizeof(float) * (size_t)((L.d + 3) & ~3);
    // group sums in shared memory up to 32 KB
    const bool tsums = (size_t)kTileBalls * L.d * sizeof(float) <= 32768;
    const bool ssums = (size_t)kSuperBalls * L.d * sizeof(float) <= 32768;
    const size_t tsm = csm + (tsums ? sizeof(float) * kTileBalls * (size_t)L.d : 0) +
                       (staged ? sizeof(float) * kTile * (size_t)tile_row_stride(L.d) : 0);
    const size_t ssm = csm + (ssums ? sizeof(float) * kSuperBalls * (size_t)L.d : 0) +
                       ((L.d & 3) == 0 && L.d <= 128 ? sizeof(float) * kSuper * kTileBalls * (size_t)(L.d + 4) : 0);
    // staged rows of 8, 16, 32, 64 or 128 dimensions: each thread's own row in registers
    switch (staged && (L.d & 3) == 0 ? L.d : 0) {
        case 8: launch_covers<2>(c, L, grow, staged, tsums, ssums, tsm, ssm); break;
        case 16: launch_covers<4>(c, L, grow, staged, tsums, ssums, tsm, ssm); break;
        case 32: launch_covers<8>(c, L, grow, staged, tsums, ssums, tsm, ssm); break;
        case 64: launch_covers<16>(c, L, grow, staged, tsums, ssums, tsm, ssm); break;
        case 128: launch_covers<32>(c, L, grow, staged, tsums, ssums, tsm, ssm); break;
        default: launch_covers<0>(c, L, grow, staged, tsums, ssums, tsm, ssm); break;
    }
    RNNG_CUDA(cudaGetLastError());
}

void prune_covers(rnng_ctx* c, Layout& L)
{
    cudaStream_t s = c->stream;
    c->counters.reserve(sizeof(unsigned long long) * kCounterSlots);
    unsigned long long* cnt = c->counters.as<unsigned long long>();
    const float eps_p = widened_radius(L.radius, L.d);
    const float shrink = 1.f - L.relerr;
    // Tensor-core ball Gram blocks (BF16 ball centres with their error terms) unless those
    // terms would widen the ball test by more than kMaxWiden on average: data whose extent
    // is large against eps (then the FP32 kernels prune more).
    constexpr float kMaxWiden = 0.05f;
    const bool b16 = bf16_supported(L.d);
    const int dp = (int)ceil_div(L.d, 64) * 64;
    bool tc = b16, tcs = b16;
    const int64_t nsb_pad = ceil_div(L.S, 4) * 64;  // super balls, padded to blocks of four super-tiles
    if (b16) {
        const int64_t nb = L.T * kTileBalls, nb_pad = L.S * kSB;
        c->ball_b16.reserve(sizeof(__nv_bfloat16) * (size_t)nb_pad * dp);
        c->ball_info.reserve(sizeof(float4) * (size_t)nb_pad);
        const float widen = prepare_ball_bf16(c, L, c->tile_lo.as<float>(), c->tile_hi.as<float>(), nb, nb_pad, eps_p,
                                              c->ball_b16.as<__nv_bfloat16>(), c->ball_info.as<float4>());
        tc = widen <= kMaxWiden;
        c->stats.prune_widen = widen;
        c->sball_b16.reserve(sizeof(__nv_bfloat16) * (size_t)nsb_pad * dp);
        c->sball_info.reserve(sizeof(float4) * (size_t)nsb_pad);
        const float swiden = prepare_ball_bf16(c, L, c->super_lo.as<float>(), c->super_hi.as<float>(),
                                               L.S * kSuperBalls, nsb_pad, eps_p, c->sball_b16.as<__nv_bfloat16>(),
                                               c->sball_info.as<float4>());
        tcs = swiden <= kMaxWiden;
    }
    c->stats.prune_tensor = tc ? 1 : 0;
    // level 1: bitmap of close super-tile pairs
    const int64_t NB = L.S * kSuperBalls;
    const int64_t words = (L.S * L.S + 31) / 32;
    c->aux6.reserve(sizeof(uint32_t) * (size_t)words);
    uint32_t* bitmap = c->aux6.as<uint32_t>();
    RNNG_CUDA(cudaMemsetAsync(bitmap, 0, sizeof(uint32_t) * (size_t)words, s));
    if (tcs) {
        const float kappa = 1.0f / (1 << 20);  // relative slack for the FP32 evaluation of the test
        const int64_t nR = ceil_div(L.S, 4);
        const unsigned sgrid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(nR * (nR + 1) / 2, (int64_t)c->num_sms * 16));
        auto launch = [&](auto kern, size_t smem) {
            RNNG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            kern<<<sgrid, 128, smem, s>>>(c->sball_b16.as<uint4>(), c->sball_info.as<float4>(), L.S, eps_p, kappa,
                                          bitmap);
        };
        switch (dp / 32) {
            case 2: launch(k_super_close_mma<2>, TileCloseSmem<2>::bytes); break;
            case 4: launch(k_super_close_mma<4>, TileCloseSmem<4>::bytes); break;
            case 6: launch(k_super_close_mma<6>, TileCloseSmem<6>::bytes); break;
            default: launch(k_super_close_mma<8>, TileCloseSmem<8>::bytes); break;
        }
        ++c->launches;
    } else {
        dim3 g1((unsigned)ceil_div(NB, kDRows), (unsigned)ceil_div(NB, kDCols));
        k_super_close<<<g1, 256, 0, s>>>(c->super_lo.as<float>(), c->super_hi.as<float>(), NB, L.d, eps_p, shrink,
                                         bitmap, L.S); ++c->launches;
    }
    const unsigned bgrid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(words, 256), (int64_t)c->num_sms * 8));
    if ((unsigned long long)L.S * (L.S + 1) / 2 < (1ull << 31)) {
        // row-major pair list: per-word counts, a scan, then each word's pairs at its offset
        c->sched.reserve(sizeof(int32_t) * 2 * (size_t)(words + 1));
        int32_t* wc = c->sched.as<int32_t>();
        int32_t* wo = wc + words + 1;
        k_bitmap_count<<<bgrid, 256, 0, s>>>(bitmap, words, wc); ++c->launches;
        RNNG_CUDA(cudaMemsetAsync(wc + words, 0, sizeof(int32_t), s));
        exclusive_scan_i32(c, wc, wo, words + 1);
        int32_t total = 0;
        RNNG_CUDA(cudaMemcpyAsync(&total, wo + words, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        RNNG_CUDA(cudaStreamSynchronize(s));
        L.super_pairs = (unsigned long long)total;
        c->super_list.reserve(sizeof(int2) * std::max<unsigned long long>(1, L.super_pairs));
        k_bitmap_emit<<<bgrid, 256, 0, s>>>(bitmap, words, L.S, wo, c->super_list.as<int2>(), L.super_pairs);
        ++c->launches;
        RNNG_CUDA(cudaMemcpyAsync(cnt, &L.super_pairs, sizeof(unsigned long long), cudaMemcpyHostToDevice, s));
    } else {
        unsigned long long sup_cap = std::max<unsigned long long>(4096, (unsigned long long)L.S * 64);
        sup_cap = std::min<unsigned long long>(sup_cap, (unsigned long long)L.S * (L.S + 1) / 2);
        for (int attempt = 0; attempt < 3; ++attempt) {
            c->super_list.reserve(sizeof(int2) * sup_cap);
            RNNG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s));
            k_bitmap_pairs<<<bgrid, 256, 0, s>>>(bitmap, L.S, c->super_list.as<int2>(), cnt, sup_cap); ++c->launches;
            unsigned long long got = 0;
            RNNG_CUDA(cudaMemcpyAsync(&got, cnt, sizeof(got), cudaMemcpyDeviceToHost, s));
            RNNG_CUDA(cudaStreamSynchronize(s));
            L.super_pairs = got;
            if (got <= sup_cap) break;
            sup_cap = got;
        }
    }
    // level 2: tile pairs inside the surviving super pairs
    const unsigned long long tile_cap =
        std::max<unsigned long long>(1, L.super_pairs * (unsigned long long)(kSuper * kSuper));
    c->pair_list.reserve(sizeof(int2) * tile_cap);
    RNNG_CUDA(cudaMemsetAsync(cnt + 1, 0, sizeof(unsigned long long), s));
    const unsigned grid = (unsigned)std::max<unsigned long long>(
        1, std::min<unsigned long long>((L.super_pairs + kSPB - 1) / kSPB, (unsigned long long)c->num_sms * 8));
    if (tc) {
        const float kappa = 1.0f / (1 << 20);  // relative slack for the FP32 evaluation of the test
        const unsigned wgrid = (unsigned)std::max<unsigned long long>(
            1, std::min<unsigned long long>(L.super_pairs, (unsigned long long)c->num_sms * 16));
        auto launch = [&](auto kern, size_t smem) {
            RNNG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            kern<<<wgrid, 128, smem, s>>>(c->super_list.as<int2>(), cnt, L.super_pairs, c->ball_b16.as<uint4>(),
                                          c->ball_info.as<float4>(), L.T, eps_p, kappa, c->pair_list.as<int2>(),
                                          cnt + 1, tile_cap);
        };
        switch (dp / 32) {
            case 2: launch(k_tile_close_mma<2>, TileCloseSmem<2>::bytes); break;
            case 4: launch(k_tile_close_mma<4>, TileCloseSmem<4>::bytes); break;
            case 6: launch(k_tile_close_mma<6>, TileCloseSmem<6>::bytes); break;
            default: launch(k_tile_close_mma<8>, TileCloseSmem<8>::bytes); break;
        }
        ++c->launches;
    } else {
        k_tile_close<<<grid, 64 * kSPB, 0, s>>>(c->super_list.as<int2>(), cnt, L.super_pairs, c->tile_lo.as<float>(),
                                          c->tile_hi.as<float>(), L.T, L.d, eps_p, shrink, c->pair_list.as<int2>(),
                                          cnt + 1, tile_cap); ++c->launches;
    }
    unsigned long long got = 0;
    RNNG_CUDA(cudaMemcpyAsync(&got, cnt + 1, sizeof(got), cudaMemcpyDeviceToHost, s));
    RNNG_CUDA(cudaStreamSynchronize(s));
    L.tile_pairs = got;
    L.pairs = c->pair_list.as<int2>();
    L.d_tile_pairs = cnt + 1;
}

void schedule_items(rnng_ctx* c, Layout& L, int nt)
{
    cudaStream_t s = c->stream;
    const int64_t m = (int64_t)L.tile_pairs;
    L.item_tiles = nt;
    RNNG_REQUIRE(L.T < (1 << 21), RNNG_ERR_INVALID, "too many tiles for the tile-pair schedule");
    RNNG_REQUIRE(m < (int64_t(1) << 31), RNNG_ERR_INVALID, "too many tile pairs for the schedule");
    const int64_t mg = std::max<int64_t>(m, 1);
    // items in (row, column) order
    int64_t ni = 0;
    c->items.reserve(sizeof(int4) * (size_t)mg);
    if (m > 0) {
        c->aux6.reserve(sizeof(uint64_t) * 2 * (size_t)m);
        uint64_t* k0 = c->aux6.as<uint64_t>();
        uint64_t* k1 = k0 + m;
        c->sched_tmp.reserve(sizeof(int32_t) * 2 * ((size_t)m + 1));
        int32_t* start = c->sched_tmp.as<int32_t>();
        int32_t* off = start + m + 1;
        const unsigned grid =
            (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(m, 256), (int64_t)c->num_sms * 8));
        k_schedule_keys<<<grid, 256, 0, s>>>(L.pairs, m, nt, k0); ++c->launches;
        size_t tmp = 0;
        const int bits = (nt == 3 ? 22 : 21) + bits_for_tiles(L.T);
        RNNG_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, tmp, k0, k1, (int)m, 0, bits, s));
        c->cub_tmp.reserve(tmp);
        RNNG_CUDA(cub::DeviceRadixSort::SortKeys(c->cub_tmp.ptr, tmp, k0, k1, (int)m, 0, bits, s)); c->launches += cub_sort_kernels(m, bits);
        k_item_starts<<<grid, 256, 0, s>>>(k1, m, nt, start); ++c->launches;
        RNNG_CUDA(cudaMemsetAsync(start + m, 0, sizeof(int32_t), s));
        exclusive_scan_i32(c, start, off, m + 1);
        int32_t total = 0;
        RNNG_CUDA(cudaMemcpyAsync(&total, off + m, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        k_items<<<grid, 256, 0, s>>>(k1, m, nt, L.T, start, off, c->items.as<int4>()); ++c->launches;
        RNNG_CUDA(cudaStreamSynchronize(s));
        ni = total;
    }
    L.num_items = (unsigned long long)ni;
    L.items = c->items.as<int4>();
}

}  // namespace rnng
