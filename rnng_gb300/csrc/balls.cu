// Tile covers and exact tile-pair pruning by the triangle inequality.
//
// Every tile (128 consecutive points of the partition order) is covered by up to
// kBalls balls: the tile is split by farthest-point bisection (take the group with
// the largest radius, its point a farthest from the centroid, the point b farthest
// from a, and move the points closer to b than to a into a new group) until it has
// kBalls groups; each group is stored as (centroid, radius).  A super-tile (kSuper
// consecutive tiles) gets kBalls balls built the same way from its tiles' balls.
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
// shared memory (upper triangle; a warp per pair, lanes over dimensions), then one
// warp walks the greedy chain.
__global__ void __launch_bounds__(256) k_chain_leaves(const float* __restrict__ L, int d,
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
// farthest-point bisection shared by tile balls (over points) and super balls (over balls)

// Per-block workspace.  Items are rows of `src` (points, or ball centres with
// item radii `irad`).  Dimensions are walked with a stride so d is unbounded.
struct BisectState {
    int label[kSuper * kBalls > kTile ? kSuper * kBalls : kTile];
    float dist[kSuper * kBalls > kTile ? kSuper * kBalls : kTile];
    float rad[kBalls];
    int far_idx[kBalls];
    int count[kBalls];
    int ngroups;
    int a, b;
    float red_v[65];
    int red_i[66];
    float part[256];  // centroid partial sums (blockDim <= 256)
    int pcnt[256];
};

// (max value, index) of a pair (ties -> smaller index), and a count summed alongside
__device__ __forceinline__ void argmax_step(float& v, int& i, int& n, float ov, int oi, int on)
{
    if (ov > v || (ov == v && oi < i)) {
        v = ov;
        i = oi;
    }
    n += on;
}

// block-wide (max value, index) reduction with ties -> smaller index, plus the sum of
// `cnt`: warp shuffles, then one warp over the per-warp results (two block barriers)
__device__ void block_argmax(BisectState& st, float v, int i, float& out_v, int& out_i, int cnt, int* out_cnt)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        argmax_step(v, i, cnt, __shfl_xor_sync(0xffffffffu, v, o), __shfl_xor_sync(0xffffffffu, i, o),
                    __shfl_xor_sync(0xffffffffu, cnt, o));
    if (lane == 0) {
        st.red_v[warp] = v;
        st.red_i[warp] = i;
        st.red_i[32 + warp] = cnt;
    }
    __syncthreads();
    if (warp == 0) {
        float wv = lane < nw ? st.red_v[lane] : -INFINITY;
        int wi = lane < nw ? st.red_i[lane] : -1;
        int wn = lane < nw ? st.red_i[32 + lane] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            argmax_step(wv, wi, wn, __shfl_xor_sync(0xffffffffu, wv, o), __shfl_xor_sync(0xffffffffu, wi, o),
                        __shfl_xor_sync(0xffffffffu, wn, o));
        if (lane == 0) {
            st.red_v[64] = wv;
            st.red_i[64] = wi;
            st.red_i[65] = wn;
        }
    }
    __syncthreads();
    out_v = st.red_v[64];
    out_i = st.red_i[64];
    if (out_cnt) *out_cnt = st.red_i[65];
    __syncthreads();
}

// Euclidean distance of item r to vector v (length d), one warp.
__device__ __forceinline__ float warp_dist(const float* __restrict__ x, const float* __restrict__ v, int d)
{
    const int lane = threadIdx.x & 31;
    float s = 0.f;
    for (int k = lane; k < d; k += 32) {
        const float t = x[k] - v[k];
        s = fmaf(t, t, s);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    return sqrtf(s);
}

// centroid of group g into cen (d floats, global scratch owned by the block): for
// d <= blockDim / 2 the items are split over blockDim / d thread groups (thread t adds
// dimension t % d of items t / d, t / d + H, ...) and the partial sums combined in
// shared memory; any summation order gives a valid centre (radii are measured from it)
__device__ void group_centroid(BisectState& st, const float* __restrict__ src, int nitems, int d, int g,
                               float* __restrict__ cen)
{
    const int H = d <= (int)blockDim.x / 2 ? (int)blockDim.x / d : 1;
    if (H > 1) {
        const int k = threadIdx.x % d, h = threadIdx.x / d;
        float s = 0.f;
        int cnt = 0;
        if (h < H)
            for (int r = h; r < nitems; r += H)
                if (st.label[r] == g) {
                    s += src[(int64_t)r * d + k];
                    ++cnt;
                }
        st.part[threadIdx.x] = s;
        st.pcnt[threadIdx.x] = cnt;
        __syncthreads();
        if ((int)threadIdx.x < d) {
            float t = 0.f;
            int c = 0;
            for (int q = 0; q < H; ++q) {
                t += st.part[q * d + k];
                c += st.pcnt[q * d + k];
            }
            cen[k] = c ? t / (float)c : 0.f;
        }
        __syncthreads();
        return;
    }
    for (int k = threadIdx.x; k < d; k += blockDim.x) {
        float s = 0.f;
        int cnt = 0;
        for (int r = 0; r < nitems; ++r)
            if (st.label[r] == g) {
                s += src[(int64_t)r * d + k];
                ++cnt;
            }
        cen[k] = cnt ? s / (float)cnt : 0.f;
    }
    __syncthreads();
}

// radius of group g around cen: max over items of |x - cen| + irad (irad may be null)
__device__ void group_radius(BisectState& st, const float* __restrict__ src, const float* __restrict__ irad,
                             int nitems, int d, int g, const float* __restrict__ cen)
{
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int r = warp; r < nitems; r += nw) {
        if (st.label[r] != g) continue;  // warp-uniform
        const float dd = warp_dist(src + (int64_t)r * d, cen, d);
        if ((threadIdx.x & 31) == 0) st.dist[r] = dd + (irad ? irad[r] : 0.f);
    }
    __syncthreads();
    float best = -1.f;
    int bi = -1, cnt = 0;
    for (int r = threadIdx.x; r < nitems; r += blockDim.x)
        if (st.label[r] == g) {
            ++cnt;
            if (st.dist[r] > best) { best = st.dist[r]; bi = r; }
        }
    float v;
    int i, total;
    block_argmax(st, best, bi, v, i, cnt, &total);
    if (threadIdx.x == 0) {
        st.rad[g] = v;
        st.far_idx[g] = i;
        st.count[g] = total;
    }
    __syncthreads();
}

// Splits items into up to kBalls groups; centres written to cen[kBalls][d].
__device__ void bisect(BisectState& st, const float* __restrict__ src, const float* __restrict__ irad, int nitems,
                       int d, float* __restrict__ cen)
{
    for (int r = threadIdx.x; r < nitems; r += blockDim.x) st.label[r] = 0;
    if (threadIdx.x == 0) st.ngroups = 1;
    __syncthreads();
    group_centroid(st, src, nitems, d, 0, cen);
    group_radius(st, src, irad, nitems, d, 0, cen);
    const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    while (st.ngroups < kBalls) {
        // group with the largest radius that can still be split
        int g = -1;
        float gr = 0.f;
        for (int k = 0; k < st.ngroups; ++k)
            if (st.count[k] >= 2 && st.rad[k] > gr) { gr = st.rad[k]; g = k; }
        if (g < 0) break;
        const int a = st.far_idx[g];
        // b = farthest (by centre distance) from a within g
        for (int r = warp; r < nitems; r += nw) {
            if (st.label[r] != g) continue;
            const float dd = warp_dist(src + (int64_t)r * d, src + (int64_t)a * d, d);
            if ((threadIdx.x & 31) == 0) st.dist[r] = dd;
        }
        __syncthreads();
        float best = -1.f;
        int bi = -1;
        for (int r = threadIdx.x; r < nitems; r += blockDim.x)
            if (st.label[r] == g && st.dist[r] > best) { best = st.dist[r]; bi = r; }
        float v;
        int b;
        block_argmax(st, best, bi, v, b, 0, nullptr);
        if (b < 0 || b == a || v <= 0.f) {
            // nothing to split: mark the group unsplittable
            if (threadIdx.x == 0) st.count[g] = 1;
            __syncthreads();
            continue;
        }
        const int ng = st.ngroups;
        for (int r = warp; r < nitems; r += nw) {
            if (st.label[r] != g) continue;
            const float db = warp_dist(src + (int64_t)r * d, src + (int64_t)b * d, d);
            if ((threadIdx.x & 31) == 0 && db < st.dist[r]) st.label[r] = ng;
        }
        __syncthreads();
        if (threadIdx.x == 0) st.ngroups = ng + 1;
        __syncthreads();
        group_centroid(st, src, nitems, d, g, cen + (int64_t)g * d);
        group_radius(st, src, irad, nitems, d, g, cen + (int64_t)g * d);
        group_centroid(st, src, nitems, d, ng, cen + (int64_t)ng * d);
        group_radius(st, src, irad, nitems, d, ng, cen + (int64_t)ng * d);
        if (st.count[ng] == 0 || st.count[g] == 0) {
            // degenerate split (all on one side): undo and stop splitting this group
            for (int r = threadIdx.x; r < nitems; r += blockDim.x)
                if (st.label[r] == ng) st.label[r] = g;
            __syncthreads();
            if (threadIdx.x == 0) st.ngroups = ng;
            __syncthreads();
            group_centroid(st, src, nitems, d, g, cen + (int64_t)g * d);
            group_radius(st, src, irad, nitems, d, g, cen + (int64_t)g * d);
            if (threadIdx.x == 0) st.count[g] = 1;
            __syncthreads();
        }
    }
}

// One block per tile.  Output: centres [T][kBalls][d], radii [T][kBalls] (-1 = unused).
// With staged = true the tile's rows are first copied to shared memory (kTile * d
// floats of dynamic shared memory), which every pass of the bisection then reads.
__global__ void __launch_bounds__(256) k_tile_balls(const float* __restrict__ Xs, int64_t n, int d, float grow,
                                                    bool staged, float* __restrict__ cen, float* __restrict__ rad)
{
    __shared__ BisectState st;
    extern __shared__ __align__(16) float tile_rows[];
    const int64_t t = blockIdx.x;
    const int64_t r0 = t * kTile;
    const int nitems = (int)min((int64_t)kTile, n - r0);
    float* mycen = cen + t * kBalls * d;
    const float* src = Xs + r0 * d;
    if (staged) {
        const int total = nitems * d;
        if ((d & 3) == 0) {
            const float4* s4 = reinterpret_cast<const float4*>(src);
            float4* t4 = reinterpret_cast<float4*>(tile_rows);
            for (int i = threadIdx.x; i < total / 4; i += blockDim.x) t4[i] = __ldg(s4 + i);
        } else {
            for (int i = threadIdx.x; i < total; i += blockDim.x) tile_rows[i] = __ldg(src + i);
        }
        __syncthreads();
        src = tile_rows;
    }
    bisect(st, src, nullptr, nitems, d, mycen);
    if (threadIdx.x < kBalls)
        rad[t * kBalls + threadIdx.x] = threadIdx.x < st.ngroups ? st.rad[threadIdx.x] * grow + 1e-30f : -1.f;
}

// One block per super-tile: balls over the (up to kSuper * kBalls) valid tile balls.
__global__ void __launch_bounds__(256) k_super_balls(const float* __restrict__ tcen, const float* __restrict__ trad,
                                                     int64_t T, int d, float grow, float* __restrict__ work,
                                                     float* __restrict__ scen, float* __restrict__ srad)
{
    __shared__ BisectState st;
    __shared__ float irad[kSuper * kBalls];
    __shared__ int nvalid;
    const int64_t s = blockIdx.x;
    const int64_t t0 = s * kSuper, t1 = min(T, t0 + kSuper);
    float* items = work + s * (int64_t)kSuper * kBalls * d;  // compacted valid ball centres
    if (threadIdx.x == 0) {
        int m = 0;
        for (int64_t t = t0; t < t1; ++t)
            for (int k = 0; k < kBalls; ++k)
                if (trad[t * kBalls + k] >= 0.f) irad[m++] = trad[t * kBalls + k];
        nvalid = m;
    }
    __syncthreads();
    // copy valid centres (same order as irad)
    {
        int m = 0;
        for (int64_t t = t0; t < t1; ++t)
            for (int k = 0; k < kBalls; ++k) {
                if (trad[t * kBalls + k] < 0.f) continue;
                for (int j = threadIdx.x; j < d; j += blockDim.x)
                    items[(int64_t)m * d + j] = tcen[(t * kBalls + k) * (int64_t)d + j];
                ++m;
            }
    }
    __syncthreads();
    bisect(st, items, irad, nvalid, d, scen + s * kBalls * d);
    if (threadIdx.x < kBalls)
        srad[s * kBalls + threadIdx.x] = threadIdx.x < st.ngroups ? st.rad[threadIdx.x] * grow + 1e-30f : -1.f;
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
    if (c0 + kDCols <= r0 - kBalls) return;  // strictly below the diagonal of owners
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
            const int64_t I = row / kBalls, J = col / kBalls;
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

// Level 2: 64 threads per surviving super pair, four super pairs per block.  Thread
// (ti, tj) owns tile pair (ta0 + ti, tb0 + tj) and its kBalls x kBalls ball pairs; the
// two super-tiles' ball centres are staged in shared memory kDC dimensions at a time,
// transposed so that one float4 load feeds four balls.  A tile pair survives when any
// of its ball pairs is close; each distance is the sequential fmaf sum over the
// dimensions, as at the super level.
constexpr int kNB = kSuper * kBalls;  // balls per super-tile
constexpr int kDC = 32;               // dimensions per staged chunk
constexpr int kSPB = 4;               // super pairs per block

__global__ void __launch_bounds__(256) k_tile_close(const int2* __restrict__ supers,
                                                    const unsigned long long* __restrict__ nsup_ptr,
                                                    unsigned long long sup_cap, const float* __restrict__ tcen,
                                                    const float* __restrict__ trad, int64_t T, int d, float eps_p,
                                                    float shrink, int2* __restrict__ out,
                                                    unsigned long long* __restrict__ count, unsigned long long cap)
{
    __shared__ __align__(16) float ca[kSPB][kDC][kNB + 4], cb[kSPB][kDC][kNB + 4];
    const unsigned long long nsup = min(*nsup_ptr, sup_cap);
    const int sp = threadIdx.x >> 6;       // super pair of this block's four
    const int t = threadIdx.x & 63;
    const int ti = t >> 3, tj = t & 7;     // tile pair inside the super pair
    for (unsigned long long w0 = (unsigned long long)blockIdx.x * kSPB; w0 < nsup;
         w0 += (unsigned long long)gridDim.x * kSPB) {
        const unsigned long long w = w0 + sp;
        const bool live = w < nsup;
        const int2 spair = live ? supers[w] : make_int2(0, 0);
        const int64_t ta0 = (int64_t)spair.x * kSuper, tb0 = (int64_t)spair.y * kSuper;
        float acc[kBalls][kBalls];
#pragma unroll
        for (int x = 0; x < kBalls; ++x)
#pragma unroll
            for (int y = 0; y < kBalls; ++y) acc[x][y] = 0.f;
        for (int k0 = 0; k0 < d; k0 += kDC) {
            __syncthreads();
            // stage: kNB balls x kDC dims per side as float4 along the dimension
            for (int idx = t; idx < kNB * (kDC / 4); idx += 64) {
                const int ball = idx / (kDC / 4), q4 = idx % (kDC / 4), k = k0 + 4 * q4;
                const int64_t t1 = ta0 + ball / kBalls, t2 = tb0 + ball / kBalls;
                float4 va = make_float4(0.f, 0.f, 0.f, 0.f), vb = va;
                if (live && t1 < T) {
                    const float* src = tcen + (t1 * kBalls + ball % kBalls) * (int64_t)d;
                    if (k + 3 < d && (d & 3) == 0) va = *reinterpret_cast<const float4*>(src + k);
                    else {
                        va.x = k < d ? src[k] : 0.f;
                        va.y = k + 1 < d ? src[k + 1] : 0.f;
                        va.z = k + 2 < d ? src[k + 2] : 0.f;
                        va.w = k + 3 < d ? src[k + 3] : 0.f;
                    }
                }
                if (live && t2 < T) {
                    const float* src = tcen + (t2 * kBalls + ball % kBalls) * (int64_t)d;
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
#pragma unroll 4
            for (int kk = 0; kk < kk_end; ++kk) {
                const float4 a4 = *reinterpret_cast<const float4*>(&ca[sp][kk][ti * kBalls]);
                const float4 b4 = *reinterpret_cast<const float4*>(&cb[sp][kk][tj * kBalls]);
                const float av[4] = {a4.x, a4.y, a4.z, a4.w}, bv[4] = {b4.x, b4.y, b4.z, b4.w};
#pragma unroll
                for (int x = 0; x < kBalls; ++x)
#pragma unroll
                    for (int y = 0; y < kBalls; ++y) {
                        const float df = av[x] - bv[y];
                        acc[x][y] = fmaf(df, df, acc[x][y]);
                    }
            }
        }
        const int64_t i = ta0 + ti, j = tb0 + tj;
        bool keep = false;
        if (live && i < T && j < T && i <= j) {
#pragma unroll
            for (int x = 0; x < kBalls; ++x) {
                const float ra = trad[i * kBalls + x];
#pragma unroll
                for (int y = 0; y < kBalls; ++y) {
                    const float rb = trad[j * kBalls + y];
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

// Level 2 on the tensor cores (d <= 256): one warp per surviving super pair computes the
// 32 x 32 Gram block of the two super-tiles' BF16 ball centres with mma.sync (m16n8k16,
// FP32 accumulation) and keeps a tile pair when one of its 4 x 4 ball pairs passes
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
constexpr int kSB = kSuper * kBalls;  // balls per super-tile (32)

__global__ void __launch_bounds__(256) k_tile_close_mma(const int2* __restrict__ supers,
                                                        const unsigned long long* __restrict__ nsup_ptr,
                                                        unsigned long long sup_cap, const uint4* __restrict__ cb,
                                                        const float4* __restrict__ binfo, int dp, int64_t T,
                                                        float eps_p, float kappa, int2* __restrict__ out,
                                                        unsigned long long* __restrict__ count, unsigned long long cap)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const unsigned long long nsup = min(*nsup_ptr, sup_cap);
    const unsigned long long nw = ((unsigned long long)gridDim.x * blockDim.x) >> 5;
    const int rowq = dp / 8;  // uint4 per BF16 row
    for (unsigned long long w = ((unsigned long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w < nsup; w += nw) {
        const int2 sp = supers[w];
        const int64_t ra = (int64_t)sp.x * kSB, rb = (int64_t)sp.y * kSB;  // first ball row of each side
        float acc[2][4][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int nt = 0; nt < 4; ++nt)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[mt][nt][q] = 0.f;
        const uint4* pa = cb + (ra + g) * rowq + t;
        const uint4* pb = cb + (rb + g) * rowq + t;
#pragma unroll 1
        for (int kp = 0; kp < dp / 32; ++kp) {
            uint4 a[2][2], b[4];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int h = 0; h < 2; ++h) a[mt][h] = pa[(16 * mt + 8 * h) * rowq + 4 * kp];
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) b[nt] = pb[(8 * nt) * rowq + 4 * kp];
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    mma_bf16_16816(acc[mt][nt], a[mt][0].x, a[mt][1].x, a[mt][0].y, a[mt][1].y, b[nt].x, b[nt].y);
                    mma_bf16_16816(acc[mt][nt], a[mt][0].z, a[mt][1].z, a[mt][0].w, a[mt][1].w, b[nt].z, b[nt].w);
                }
        }
        // acc[mt][nt][2h + e] = ball row 16 mt + 8 h + g, ball column 8 nt + 2 t + e; their tiles
        // are row tile 4 mt + 2 h + g / 4 and column tile 2 nt + t / 2 of the super pair
        float4 ir[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) ir[k] = binfo[ra + 8 * k + g];  // k = 2 mt + h
        uint32_t msk = 0;  // bit 4 (2 mt + h) + nt
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const float4 y = binfo[rb + 8 * nt + 2 * t + e];
#pragma unroll
                for (int mt = 0; mt < 2; ++mt)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const float4 x = ir[2 * mt + h];
                        const float D = fmaf(-2.f, acc[mt][nt][2 * h + e], x.x + y.x);
                        const float E = eps_p + x.w + y.w + x.y + y.y;
                        const float R = fmaf(E, E, x.z + y.z);
                        const bool keep = x.w >= 0.f && y.w >= 0.f && D <= R + kappa * (x.x + y.x + R);
                        msk |= (keep ? 1u : 0u) << (4 * (2 * mt + h) + nt);
                    }
            }
        // OR over the lanes holding the other balls of the same tiles (g % 4 and t % 2)
        msk |= __shfl_xor_sync(0xffffffffu, msk, 1);
        msk |= __shfl_xor_sync(0xffffffffu, msk, 4);
        msk |= __shfl_xor_sync(0xffffffffu, msk, 8);
        // lanes (g % 4 == 0, t % 2 == 0) report: row tiles g / 4 + 2 k, column tiles t / 2 + 2 nt
        const bool reporter = (lane & 13) == 0;
        uint32_t mine = 0;
        if (reporter) {
#pragma unroll
            for (int k = 0; k < 4; ++k)
#pragma unroll
                for (int nt = 0; nt < 4; ++nt) {
                    const int64_t i = (int64_t)sp.x * kSuper + (g >> 2) + 2 * k;
                    const int64_t j = (int64_t)sp.y * kSuper + (t >> 1) + 2 * nt;
                    if (((msk >> (4 * k + nt)) & 1u) && i < T && j < T && i <= j) mine |= 1u << (4 * k + nt);
                }
        }
        const int cnt = __popc(mine);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        if (total == 0) continue;
        unsigned long long base = 0;
        if (lane == 31) base = atomicAdd(count, (unsigned long long)total);
        base = __shfl_sync(0xffffffffu, base, 31);
        unsigned long long pos = base + (unsigned long long)(incl - cnt);
        while (mine) {
            const int bit = __ffs(mine) - 1;
            mine &= mine - 1;
            if (pos < cap)
                out[pos] = make_int2(sp.x * kSuper + (g >> 2) + 2 * (bit >> 2), sp.y * kSuper + (t >> 1) + 2 * (bit & 3));
            ++pos;
        }
    }
}

// Items of the persistent Gram kernel.  The pairs are sorted by (row tile, column
// tile); inside a row they are grouped nt at a time into items {i, j0, j1} (j1 = -1 for
// a row's last odd pair or nt = 1).  The items are cut into chunks of kSchedChunk and
// chunk k goes to CTA k mod G: every CTA gets the same number of items (within one
// chunk), all CTAs work on neighbouring rows at any moment (their B tiles are shared
// through L2), and a CTA reloads its resident A tile at most once per chunk.  Each
// CTA's chunks are stored contiguously, so the kernel reads one range per CTA.
__global__ void k_schedule_keys(const int2* __restrict__ pairs, int64_t m, uint64_t* __restrict__ keys)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < m; p += (int64_t)gridDim.x * blockDim.x) {
        const int2 q = pairs[p];
        keys[p] = ((uint64_t)q.x << 21) | (uint64_t)q.y;
    }
}

// start[p] = 1 when sorted pair p opens an item: its offset inside its row is a multiple of nt.
__global__ void k_item_starts(const uint64_t* __restrict__ keys, int64_t m, int nt, int32_t* __restrict__ start)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < m; p += (int64_t)gridDim.x * blockDim.x) {
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

__global__ void k_items(const uint64_t* __restrict__ keys, int64_t m, int nt, const int32_t* __restrict__ start,
                        const int32_t* __restrict__ off, int4* __restrict__ items)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < m; p += (int64_t)gridDim.x * blockDim.x) {
        if (!start[p]) continue;
        const uint64_t k = keys[p];
        const int row = (int)(k >> 21);
        int j1 = -1;
        if (nt == 2 && p + 1 < m && (int)(keys[p + 1] >> 21) == row) j1 = (int)(keys[p + 1] & 0x1fffff);
        items[off[p]] = make_int4(row, (int)(k & 0x1fffff), j1, 0);
    }
}

__global__ void k_schedule_scatter(const int4* __restrict__ sorted, int64_t m, int G,
                                   const unsigned long long* __restrict__ starts, int4* __restrict__ items)
{
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < m; p += (int64_t)gridDim.x * blockDim.x) {
        const int64_t chunk = p / kSchedChunk;
        const int g = (int)(chunk % G);
        const int64_t dest = (int64_t)starts[g] + (chunk / G) * kSchedChunk + p % kSchedChunk;
        items[dest] = sorted[p];
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
    const size_t smem = sizeof(float) * kChainMax * (kChainMax - 1) / 2;
    k_chain_leaves<<<ncells, 256, smem, c->stream>>>(lm_rows, d, nchild, child_off, rank); ++c->launches;
    RNNG_CUDA(cudaGetLastError());
}

void build_covers(rnng_ctx* c, Layout& L)
{
    cudaStream_t s = c->stream;
    const float grow = 1.f + L.relerr;
    c->tile_lo.reserve(sizeof(float) * (size_t)L.T * kBalls * L.d);   // tile ball centres
    c->tile_hi.reserve(sizeof(float) * (size_t)L.T * kBalls);         // tile ball radii
    c->super_lo.reserve(sizeof(float) * (size_t)L.S * kBalls * L.d);  // super ball centres
    c->super_hi.reserve(sizeof(float) * (size_t)L.S * kBalls);        // super ball radii
    c->pivots.reserve(sizeof(float) * (size_t)L.S * kSuper * kBalls * L.d);  // compaction workspace
    // tiles staged in shared memory up to 64 dimensions (32 KB: the bisection's many block
    // barriers need several blocks per SM, so larger tiles read through L1 instead)
    const bool staged = L.d <= 64;
    const size_t tsm = staged ? sizeof(float) * kTile * (size_t)L.d : 0;
    if (staged) RNNG_CUDA(cudaFuncSetAttribute(k_tile_balls, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm));
    k_tile_balls<<<(unsigned)L.T, 256, tsm, s>>>(L.Xs, L.n, L.d, grow, staged, c->tile_lo.as<float>(),
                                                 c->tile_hi.as<float>()); ++c->launches;
    k_super_balls<<<(unsigned)L.S, 256, 0, s>>>(c->tile_lo.as<float>(), c->tile_hi.as<float>(), L.T, L.d, grow,
                                                c->pivots.as<float>(), c->super_lo.as<float>(),
                                                c->super_hi.as<float>()); ++c->launches;
    RNNG_CUDA(cudaGetLastError());
}

void prune_covers(rnng_ctx* c, Layout& L)
{
    cudaStream_t s = c->stream;
    c->counters.reserve(sizeof(unsigned long long) * kCounterSlots);
    unsigned long long* cnt = c->counters.as<unsigned long long>();
    const float eps_p = widened_radius(L.radius, L.d);
    const float shrink = 1.f - L.relerr;
    // level 1: bitmap of close super-tile pairs
    const int64_t NB = L.S * kBalls;
    const int64_t words = (L.S * L.S + 31) / 32;
    c->aux6.reserve(sizeof(uint32_t) * (size_t)words);
    uint32_t* bitmap = c->aux6.as<uint32_t>();
    RNNG_CUDA(cudaMemsetAsync(bitmap, 0, sizeof(uint32_t) * (size_t)words, s));
    dim3 g1((unsigned)ceil_div(NB, kDRows), (unsigned)ceil_div(NB, kDCols));
    k_super_close<<<g1, 256, 0, s>>>(c->super_lo.as<float>(), c->super_hi.as<float>(), NB, L.d, eps_p, shrink, bitmap,
                                     L.S); ++c->launches;
    unsigned long long sup_cap = std::max<unsigned long long>(4096, (unsigned long long)L.S * 64);
    sup_cap = std::min<unsigned long long>(sup_cap, (unsigned long long)L.S * (L.S + 1) / 2);
    for (int attempt = 0; attempt < 3; ++attempt) {
        c->super_list.reserve(sizeof(int2) * sup_cap);
        RNNG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), s));
        k_bitmap_pairs<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(words, 256), (int64_t)c->num_sms * 8)),
                         256, 0, s>>>(bitmap, L.S, c->super_list.as<int2>(), cnt, sup_cap); ++c->launches;
        unsigned long long got = 0;
        RNNG_CUDA(cudaMemcpyAsync(&got, cnt, sizeof(got), cudaMemcpyDeviceToHost, s));
        RNNG_CUDA(cudaStreamSynchronize(s));
        L.super_pairs = got;
        if (got <= sup_cap) break;
        sup_cap = got;
    }
    // level 2: tile pairs inside the surviving super pairs
    const unsigned long long tile_cap =
        std::max<unsigned long long>(1, L.super_pairs * (unsigned long long)(kSuper * kSuper));
    c->pair_list.reserve(sizeof(int2) * tile_cap);
    RNNG_CUDA(cudaMemsetAsync(cnt + 1, 0, sizeof(unsigned long long), s));
    const unsigned grid = (unsigned)std::max<unsigned long long>(
        1, std::min<unsigned long long>((L.super_pairs + kSPB - 1) / kSPB, (unsigned long long)c->num_sms * 8));
    // Tensor-core ball Gram blocks (BF16 ball centres padded to S super-tiles of kSB rows)
    // unless their error terms would widen the ball test by more than kMaxWiden on
    // average: data whose extent is large against eps (then the FP32 kernel prunes more).
    constexpr float kMaxWiden = 0.05f;
    bool tc = bf16_supported(L.d);
    const int dp = (int)ceil_div(L.d, 64) * 64;
    if (tc) {
        const int64_t nb = L.T * kBalls, nb_pad = L.S * kSB;
        c->ball_b16.reserve(sizeof(__nv_bfloat16) * (size_t)nb_pad * dp);
        c->ball_info.reserve(sizeof(float4) * (size_t)nb_pad);
        const float widen = prepare_ball_bf16(c, L, c->tile_lo.as<float>(), c->tile_hi.as<float>(), nb, nb_pad, eps_p,
                                              c->ball_b16.as<__nv_bfloat16>(), c->ball_info.as<float4>());
        tc = widen <= kMaxWiden;
        c->stats.prune_widen = widen;
    }
    c->stats.prune_tensor = tc ? 1 : 0;
    if (tc) {
        const float kappa = 1.0f / (1 << 20);  // relative slack for the FP32 evaluation of the test
        const unsigned wgrid = (unsigned)std::max<unsigned long long>(
            1, std::min<unsigned long long>((L.super_pairs + 7) / 8, (unsigned long long)c->num_sms * 8));
        k_tile_close_mma<<<wgrid, 256, 0, s>>>(c->super_list.as<int2>(), cnt, L.super_pairs, c->ball_b16.as<uint4>(),
                                               c->ball_info.as<float4>(), dp, L.T, eps_p, kappa,
                                               c->pair_list.as<int2>(), cnt + 1, tile_cap); ++c->launches;
    } else {
        k_tile_close<<<grid, 256, 0, s>>>(c->super_list.as<int2>(), cnt, L.super_pairs, c->tile_lo.as<float>(),
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

void schedule_items(rnng_ctx* c, Layout& L, int max_ctas, int nt)
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
    c->items_tmp.reserve(sizeof(int4) * (size_t)mg);
    int4* sorted = c->items_tmp.as<int4>();
    if (m > 0) {
        c->aux6.reserve(sizeof(uint64_t) * 2 * (size_t)m);
        uint64_t* k0 = c->aux6.as<uint64_t>();
        uint64_t* k1 = k0 + m;
        c->sched_tmp.reserve(sizeof(int32_t) * 2 * ((size_t)m + 1));
        int32_t* start = c->sched_tmp.as<int32_t>();
        int32_t* off = start + m + 1;
        const unsigned grid =
            (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(m, 256), (int64_t)c->num_sms * 8));
        k_schedule_keys<<<grid, 256, 0, s>>>(L.pairs, m, k0); ++c->launches;
        size_t tmp = 0;
        const int bits = 21 + bits_for_tiles(L.T);
        RNNG_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, tmp, k0, k1, (int)m, 0, bits, s));
        c->cub_tmp.reserve(tmp);
        RNNG_CUDA(cub::DeviceRadixSort::SortKeys(c->cub_tmp.ptr, tmp, k0, k1, (int)m, 0, bits, s)); c->launches += cub_sort_kernels(m, bits);
        k_item_starts<<<grid, 256, 0, s>>>(k1, m, nt, start); ++c->launches;
        RNNG_CUDA(cudaMemsetAsync(start + m, 0, sizeof(int32_t), s));
        exclusive_scan_i32(c, start, off, m + 1);
        int32_t total = 0;
        RNNG_CUDA(cudaMemcpyAsync(&total, off + m, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        k_items<<<grid, 256, 0, s>>>(k1, m, nt, start, off, sorted); ++c->launches;
        RNNG_CUDA(cudaStreamSynchronize(s));
        ni = total;
    }
    L.num_items = (unsigned long long)ni;
    L.items = c->items.as<int4>();
    const int G = (int)std::max<int64_t>(1, std::min<int64_t>(ni, (int64_t)max_ctas));
    L.sched_G = G;
    // segment of CTA g: its chunks k = g, g + G, ... (all full but the very last chunk)
    c->sched.reserve(sizeof(unsigned long long) * (G + 1));
    unsigned long long* starts = c->sched.as<unsigned long long>();
    L.sched = starts;
    const int64_t nchunks = ceil_div(ni, kSchedChunk), tail = ni % kSchedChunk;
    std::vector<unsigned long long> h(G + 1, 0);
    for (int g = 0; g < G; ++g) {
        int64_t size = (nchunks / G + (g < nchunks % G ? 1 : 0)) * kSchedChunk;
        if (tail > 0 && (nchunks - 1) % G == g) size -= kSchedChunk - tail;
        h[g + 1] = h[g] + (unsigned long long)size;
    }
    RNNG_CUDA(cudaMemcpyAsync(starts, h.data(), sizeof(unsigned long long) * (G + 1), cudaMemcpyHostToDevice, s));
    if (ni > 0) {
        const unsigned grid =
            (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(ni, 256), (int64_t)c->num_sms * 8));
        k_schedule_scatter<<<grid, 256, 0, s>>>(sorted, ni, G, starts, L.items); ++c->launches;
    }
    RNNG_CUDA(cudaStreamSynchronize(s));  // h lifetime
}

}  // namespace rnng
