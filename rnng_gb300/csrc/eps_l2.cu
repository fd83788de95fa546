// Epsilon-graph pipeline for dense float32 points under RNNG's L2.
//
// Replaces, on one GPU, the neighbour search that RNNG runs with cover trees over
// MPI ranks (include/search.hpp:6-340, include/point.hpp:537-929): instead of a
// tree walk per query, the points are ordered by a two-level landmark partition
// (the Voronoi idea of include/point.hpp:537-559 applied twice), cut into tiles of
// 128 points, and every pair of tiles that the triangle inequality cannot rule out
// is evaluated in full.  The pruning is exact: a tile pair is skipped only when the
// balls covering the two tiles are separated by more than the radius, with a
// rounding slack that covers the float error of the ball geometry and of the
// reference's own sequential L2, so no pair with L2seq <= radius is ever skipped.
//
// Stages (all on the context stream):
//   1-3. recursive landmark partition: every cell larger than 2 tiles is split
//      by up to kFan landmarks (strided picks from the cell), its points move to
//      the nearest one, and the children are ordered along a nearest-neighbour
//      chain; the points are sorted by (cell, distance to its landmark) after
//      each level and finally gathered in that order.  Leaves hold about one
//      tile, so a tile rarely mixes two clusters.
//   4. cover every tile and super-tile (8 tiles) by a few balls (balls.cu)
//   5. prune super-tile pairs, then tile pairs, by ball separation
//   6. evaluate surviving tile pairs (FP32-direct here; BF16 Gram in gram_bf16.cu)
//   7. map sorted indices back to ids, order each edge as u < v
#include <cub/cub.cuh>

#include <cfloat>
#include <cmath>
#include <cstring>

#include "common.cuh"
#include "eps_l2.cuh"
#include "balls.cuh"
#include "partition.cuh"

namespace rnng {

// ------------------------------------------------------------------------------------------------
// helpers

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

// Cell boundaries in the current order (cells are contiguous after each sort).
__global__ void k_cell_bounds(const uint64_t* __restrict__ sorted_keys, int64_t n, int32_t* __restrict__ start,
                              int32_t* __restrict__ end)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t c = (uint32_t)(sorted_keys[i] >> 32);
    if (i == 0 || (uint32_t)(sorted_keys[i - 1] >> 32) != c) start[c] = (int32_t)i;
    if (i == n - 1 || (uint32_t)(sorted_keys[i + 1] >> 32) != c) end[c] = (int32_t)(i + 1);
}

// Children per cell: cells above 2 * kLeafTarget points are split into
// min(ceil(size / kLeafTarget), kFan) children, others keep one child.
__global__ void k_split_plan(const int32_t* __restrict__ start, const int32_t* __restrict__ end, int64_t ncells,
                             int32_t* __restrict__ nchild)
{
    int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    const int64_t sz = end[c] - start[c];
    int64_t m = 1;
    if (sz > 2 * kLeafTarget) m = min((sz + kLeafTarget - 1) / kLeafTarget, (int64_t)kFan);
    nchild[c] = (int32_t)m;
}

// Landmark of child k of cell c: the point at position start + floor(k * size / m)
// of the current order (its leading points are nearest the parent's landmark).
__global__ void k_child_landmarks(const int32_t* __restrict__ start, const int32_t* __restrict__ end,
                                  const int32_t* __restrict__ nchild, const int32_t* __restrict__ child_off,
                                  int64_t ncells, const int32_t* __restrict__ order, int32_t* __restrict__ lm_idx)
{
    const int64_t c = blockIdx.x;
    if (c >= ncells) return;
    const int sz = end[c] - start[c], m = nchild[c];
    for (int k = threadIdx.x; k < m; k += blockDim.x)
        lm_idx[child_off[c] + k] = order[start[c] + (int)(((int64_t)k * sz) / m)];
}

// Sorted copy of the points, padded with zero rows to a multiple of the tile size.
// Rows of X in partition order (padding rows zero), one warp per row: 16-byte copies when
// d is a multiple of 4, else single floats.
__global__ void k_gather_sorted(const float* __restrict__ X, int64_t n, int64_t n_pad, int d,
                                const int32_t* __restrict__ perm, float* __restrict__ Xs)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    if (d == 128) {
        // the common width: four rows per warp and round, their loads in flight together
        for (int64_t r = warp; r < n_pad; r += 4 * nwarps) {
            float4 v[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int64_t rj = r + j * nwarps;
                v[j] = rj < n ? __ldg(reinterpret_cast<const float4*>(X + (int64_t)perm[rj] * d) + lane)
                              : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int64_t rj = r + j * nwarps;
                if (rj < n_pad) reinterpret_cast<float4*>(Xs + rj * d)[lane] = v[j];
            }
        }
        return;
    }
    for (int64_t r = warp; r < n_pad; r += nwarps) {
        float* dst = Xs + r * d;
        const float* src = r < n ? X + (int64_t)perm[r] * d : nullptr;
        if ((d & 3) == 0) {
            for (int k = lane; k < d / 4; k += 32)
                reinterpret_cast<float4*>(dst)[k] =
                    src ? __ldg(reinterpret_cast<const float4*>(src) + k) : make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            for (int k = lane; k < d; k += 32) dst[k] = src ? __ldg(src + k) : 0.f;
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

// Rows of the current order whose cell splits at this level (flag 1), and the others (0).
__global__ void k_active_rows(const uint64_t* __restrict__ skeys, int64_t n, const int32_t* __restrict__ nchild,
                              int32_t* __restrict__ flag)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        flag[i] = nchild[skeys[i] >> 32] > 1 ? 1 : 0;
}

// The active rows (those whose cell splits), in order: their positions, input rows and keys.
__global__ void k_compact_active(const uint64_t* __restrict__ skeys, const int32_t* __restrict__ order, int64_t n,
                                 const int32_t* __restrict__ flag, const int32_t* __restrict__ pos,
                                 uint64_t* __restrict__ ckey, int32_t* __restrict__ crow, int32_t* __restrict__ cidx)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (flag[i]) {
            const int32_t j = pos[i];
            ckey[j] = skeys[i];
            crow[j] = order[i];
            cidx[j] = (int32_t)i;
        }
}

// The level's new order: an inactive row keeps its place and its distance key under its
// cell's single child (the cell does not move and keeps its order); the sorted active
// rows fill the active places in order.
__global__ void k_place_rows(int64_t n, const int32_t* __restrict__ flag, const int32_t* __restrict__ child_off,
                             const int32_t* __restrict__ rank, const uint64_t* __restrict__ ck,
                             const int32_t* __restrict__ cv, const int32_t* __restrict__ cidx, int64_t m,
                             uint64_t* __restrict__ skeys, int32_t* __restrict__ order)
{
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
        if (!flag[i]) {
            const uint64_t k = skeys[i];
            skeys[i] = ((uint64_t)(uint32_t)rank[child_off[k >> 32]] << 32) | (k & 0xffffffffull);
        }
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += stride) {
        skeys[cidx[j]] = ck[j];
        order[cidx[j]] = cv[j];
    }
}

__global__ void k_iota_keys(int32_t* __restrict__ order, uint64_t* __restrict__ keys, int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        order[i] = (int32_t)i;
        keys[i] = 0ull;
    }
}

// ------------------------------------------------------------------------------------------------
// non-finite rows
//
// A row with a NaN or infinite coordinate has an L2seq of NaN or +inf to every row
// (x - y is NaN or infinite in that coordinate, and so is the sum of squares), so
// under a finite radius it has no edge, as in RNNG's own paths (whose edge test is
// dist <= radius, include/search.hpp:390-407).  Such rows would also poison the
// partition's distances and the covering balls of their tile, so the graph is built
// over the finite rows only and mapped back.

// *flag = 1 if any of X[0..count) is NaN or infinite (flag zeroed by the caller).
__global__ void k_any_nonfinite(const float* __restrict__ X, int64_t count, unsigned long long* __restrict__ flag)
{
    bool bad = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        bad |= nonfinite_f32(X[i]);
    if (__syncthreads_or(bad) && threadIdx.x == 0) *flag = 1ull;
}

// keep[r] = 1 if row r is finite, else 0; one warp per row.  *inf_rows = 1 (zeroed by
// the caller) if some row has an infinite coordinate and no NaN: such a row is at L2
// +inf, not NaN, from the rows it shares no infinite coordinate with.
__global__ void k_row_finite(const float* __restrict__ X, int64_t n, int d, int32_t* __restrict__ keep,
                             unsigned long long* __restrict__ inf_rows)
{
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
        bool bad = false, nan = false;
        for (int k = lane; k < d; k += 32) {
            const float v = X[r * d + k];
            bad |= nonfinite_f32(v);
            nan |= (__float_as_uint(v) & 0x7fffffffu) > 0x7f800000u;
        }
        bad = __any_sync(0xffffffffu, bad);
        nan = __any_sync(0xffffffffu, nan);
        if (lane == 0) {
            keep[r] = bad ? 0 : 1;
            if (bad && !nan) *inf_rows = 1ull;
        }
    }
}

// Finite row r to row pos[r] of Xc; map[pos[r]] = r.
__global__ void k_compact_rows(const float* __restrict__ X, int64_t n, int d, const int32_t* __restrict__ keep,
                               const int32_t* __restrict__ pos, float* __restrict__ Xc, int32_t* __restrict__ map)
{
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
        if (!keep[r]) continue;
        const int64_t p = pos[r];
        for (int k = lane; k < d; k += 32) Xc[p * d + k] = X[r * d + k];
        if (lane == 0) map[p] = (int32_t)r;
    }
}

__global__ void k_remap(int32_t* __restrict__ perm, int64_t n, const int32_t* __restrict__ map)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        perm[i] = map[perm[i]];
}

// ------------------------------------------------------------------------------------------------
// host side

void exclusive_scan_i32(rnng_ctx* c, const int32_t* in, int32_t* out, int64_t count)
{
    // count includes the trailing total: in[count-1] is read as 0 by scanning count-1 items
    size_t tmp = 0;
    RNNG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp, in, out, (int)count, c->stream));
    c->cub_tmp.reserve(tmp);
    RNNG_CUDA(cudaMemsetAsync((void*)(in + count - 1), 0, sizeof(int32_t), c->stream));
    RNNG_CUDA(cub::DeviceScan::ExclusiveSum(c->cub_tmp.ptr, tmp, in, out, (int)count, c->stream)); c->launches += 2;
}

static int grid_for(rnng_ctx* c, int64_t work, int per_block, int waves = 8)
{
    int64_t g = ceil_div(work, per_block);
    int64_t cap = (int64_t)c->num_sms * waves;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

int64_t compact_finite_rows(rnng_ctx* c, const float* dX, int64_t n, int d, const float** out, bool* inf_rows)
{
    cudaStream_t s = c->stream;
    c->fin_idx.reserve(sizeof(int32_t) * (size_t)(3 * n + 2));
    int32_t* keep = c->fin_idx.as<int32_t>();  // n + 1 (the scan's trailing slot)
    int32_t* pos = keep + (n + 1);              // n + 1
    int32_t* map = pos + (n + 1);               // n
    c->counters.reserve(sizeof(unsigned long long) * kCounterSlots);
    unsigned long long* dinf = c->counters.as<unsigned long long>() + kSlotNonfinite;
    RNNG_CUDA(cudaMemsetAsync(dinf, 0, sizeof(unsigned long long), s));
    k_row_finite<<<grid_for(c, n * 32, 256), 256, 0, s>>>(dX, n, d, keep, dinf); ++c->launches;
    exclusive_scan_i32(c, keep, pos, n + 1);
    int32_t nf = 0;
    unsigned long long hinf = 0;
    RNNG_CUDA(cudaMemcpyAsync(&nf, pos + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    RNNG_CUDA(cudaMemcpyAsync(&hinf, dinf, sizeof(hinf), cudaMemcpyDeviceToHost, s));
    RNNG_CUDA(cudaStreamSynchronize(s));
    *inf_rows = hinf != 0;
    *out = dX;
    if (nf == n) return n;
    c->fin_x.reserve(sizeof(float) * (size_t)std::max<int64_t>(nf, 1) * d);
    k_compact_rows<<<grid_for(c, n * 32, 256), 256, 0, s>>>(dX, n, d, keep, pos, c->fin_x.as<float>(), map);
    ++c->launches;
    *out = c->fin_x.as<float>();
    return nf;
}

void remap_rows(rnng_ctx* c, int32_t* perm, int64_t n, int64_t n_in)
{
    if (n == 0) return;
    const int32_t* map = c->fin_idx.as<int32_t>() + 2 * (n_in + 1);
    k_remap<<<grid_for(c, n, 256), 256, 0, c->stream>>>(perm, n, map); ++c->launches;
}

void sort_pairs_u64(rnng_ctx* c, uint64_t* keys_in, uint64_t* keys_out, int32_t* vals_in, int32_t* vals_out,
                    int64_t n, int end_bit, int begin_bit)
{
    size_t tmp = 0;
    RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, keys_in, keys_out, vals_in, vals_out, (int)n, begin_bit,
                                              end_bit, c->stream));
    c->cub_tmp.reserve(tmp);
    RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, keys_in, keys_out, vals_in, vals_out, (int)n,
                                              begin_bit, end_bit, c->stream));
    c->launches += cub_sort_kernels(n, end_bit - begin_bit);
}

static int bits_for(int64_t v)
{
    int b = 1;
    while ((int64_t(1) << b) < v + 1) ++b;
    return b;
}

Layout build_layout(rnng_ctx* c, const float* dX, int64_t n, int d, float radius, bool screen)
{
    Layout L;
    L.n = n;
    L.d = d;
    L.T = ceil_div(n, kTile);
    L.n_pad = L.T * kTile;
    L.S = ceil_div(L.T, kSuper);
    cudaStream_t s = c->stream;

    // current order and sorted keys (cell << 32 | distance bits); start: one cell
    c->keys.reserve(sizeof(uint64_t) * n);
    c->keys_alt.reserve(sizeof(uint64_t) * n);
    c->perm.reserve(sizeof(int32_t) * L.n_pad);
    c->perm_alt.reserve(sizeof(int32_t) * n);
    uint64_t* skeys = c->keys_alt.as<uint64_t>();   // sorted keys of the current order
    uint64_t* nkeys = c->keys.as<uint64_t>();       // keys of the next level, in current order
    int32_t* order = c->perm.as<int32_t>();          // current order: position -> input row
    int32_t* nvals = c->perm_alt.as<int32_t>();
    k_iota_keys<<<(unsigned)std::min<int64_t>(ceil_div(n, 256), (int64_t)c->num_sms * 8), 256, 0, s>>>(order, skeys, n); ++c->launches;
    int64_t ncells = 1;
    // per-cell scratch (cells never outnumber points)
    const int64_t cap = n + 2;
    c->aux2.reserve(sizeof(int32_t) * (size_t)(4 * cap + 4));
    int32_t* cstart = c->aux2.as<int32_t>();
    int32_t* cend = cstart + cap;
    int32_t* nchild = cend + cap;
    int32_t* child_off = nchild + cap;
    // input screen, read with the first level's synchronisation: a non-finite value seen
    // and (d <= 256) the largest magnitude
    c->counters.reserve(sizeof(unsigned long long) * kCounterSlots);
    unsigned long long* scr = c->counters.as<unsigned long long>() + kSlotNonfinite;
    const bool b16 = bf16_supported(d);
    if (!b16) {
        RNNG_CUDA(cudaMemsetAsync(scr, 0, sizeof(unsigned long long), s));
        if (screen) {
            k_any_nonfinite<<<grid_for(c, n * d, 1024), 256, 0, s>>>(dX, n * d, scr); ++c->launches;
        }
    }
    // BF16 shift (d <= 256): the assignment's distances come from the tensor cores; the
    // column sums behind it read every value, so they carry the screen
    const float* shift = b16 ? bf16_shift(c, L, dX, scr) : nullptr;
    int levels = 0;
    for (; levels < kMaxLevels; ++levels) {
        // a cell can be empty (its landmark's point went to a sibling with an equal or, in the
        // BF16 distances, a marginally smaller distance): it gets size 0, not stale bounds
        RNNG_CUDA(cudaMemsetAsync(cstart, 0, sizeof(int32_t) * (size_t)ncells, s));
        RNNG_CUDA(cudaMemsetAsync(cend, 0, sizeof(int32_t) * (size_t)ncells, s));
        k_cell_bounds<<<(unsigned)ceil_div(n, 256), 256, 0, s>>>(skeys, n, cstart, cend); ++c->launches;
        k_split_plan<<<(unsigned)ceil_div(ncells, 256), 256, 0, s>>>(cstart, cend, ncells, nchild); ++c->launches;
        exclusive_scan_i32(c, nchild, child_off, ncells + 1);
        int32_t total = 0, active = 0;
        RNNG_CUDA(cudaMemcpyAsync(&total, child_off + ncells, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        // rows whose cell splits: after the first levels a few cells, so only their rows are
        // sorted (the others keep their places)
        c->part_f.reserve(sizeof(int32_t) * 2 * (size_t)(n + 1));
        int32_t* aflag = c->part_f.as<int32_t>();
        int32_t* apos = aflag + n + 1;
        if (levels >= 2) {
            k_active_rows<<<grid_for(c, n, 256), 256, 0, s>>>(skeys, n, nchild, aflag); ++c->launches;
            RNNG_CUDA(cudaMemsetAsync(aflag + n, 0, sizeof(int32_t), s));
            exclusive_scan_i32(c, aflag, apos, n + 1);
            RNNG_CUDA(cudaMemcpyAsync(&active, apos + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        }
        unsigned long long hs[2] = {0ull, 0ull};
        if (levels == 0)
            RNNG_CUDA(cudaMemcpyAsync(hs, scr, (b16 ? 2 : 1) * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
        RNNG_CUDA(cudaStreamSynchronize(s));
        if (levels == 0) {
            if (screen && hs[0]) {
                L.nonfinite = true;
                return L;
            }
            const uint32_t bits = (uint32_t)hs[1];
            std::memcpy(&L.maxabs, &bits, sizeof(float));
        }
        if (total == ncells) break;  // every cell is a leaf
        c->aux3.reserve(sizeof(int32_t) * (size_t)total);
        c->aux4.reserve(sizeof(float) * (size_t)total * d);
        c->aux5.reserve(sizeof(int32_t) * (size_t)total);
        int32_t* lm_idx = c->aux3.as<int32_t>();
        float* lm_rows = c->aux4.as<float>();
        k_child_landmarks<<<(unsigned)ncells, 64, 0, s>>>(cstart, cend, nchild, child_off, ncells, order, lm_idx); ++c->launches;
        k_gather_rows<<<grid_for(c, (int64_t)total * d, 256), 256, 0, s>>>(dX, d, lm_idx, total, lm_rows); ++c->launches;
        // children ordered along a greedy nearest-neighbour chain of their landmarks
        chain_leaves(c, lm_rows, d, nchild, child_off, (int)ncells, c->aux5.as<int32_t>());
        int32_t* rank = c->aux5.as<int32_t>();
        if (levels < 2 || 4 * (int64_t)active > n) {
            launch_assign(c, dX, order, n, d, lm_rows, total, skeys, child_off, rank, shift, nkeys, nvals);
            // by child, then by distance (the order inside a cell shapes its tiles: a coarser
            // distance key left 4.6 % more tile pairs at K2)
            sort_pairs_u64(c, nkeys, skeys, nvals, order, n, 32 + bits_for(total));
        } else {
            // few rows in splitting cells: assign and sort only those, in place of their cells
            const int64_t m = active, mm = std::max<int64_t>(m, 1);
            c->part_k.reserve(sizeof(uint64_t) * 3 * (size_t)mm);
            c->part_v.reserve(sizeof(int32_t) * 4 * (size_t)mm);
            uint64_t* ckey = c->part_k.as<uint64_t>();
            uint64_t* ck = ckey + mm;
            uint64_t* ck2 = ck + mm;
            int32_t* crow = c->part_v.as<int32_t>();
            int32_t* cv = crow + mm;
            int32_t* cv2 = cv + mm;
            int32_t* cidx = cv2 + mm;
            if (m > 0) {
                k_compact_active<<<grid_for(c, n, 256), 256, 0, s>>>(skeys, order, n, aflag, apos, ckey, crow, cidx);
                ++c->launches;
                launch_assign(c, dX, crow, m, d, lm_rows, total, ckey, child_off, rank, shift, ck, cv);
                sort_pairs_u64(c, ck, ck2, cv, cv2, m, 32 + bits_for(total));
            }
            k_place_rows<<<grid_for(c, n, 256), 256, 0, s>>>(n, aflag, child_off, rank, ck2, cv2, cidx, m, skeys, order);
            ++c->launches;
        }
        ncells = total;
    }
    L.num_cells = ncells;
    L.m1 = levels;
    L.perm = order;

    // ---- sorted points
    c->x_sorted.reserve(sizeof(float) * (size_t)L.n_pad * d);
    L.Xs = c->x_sorted.as<float>();
    k_gather_sorted<<<grid_for(c, L.n_pad * 32, 256), 256, 0, s>>>(dX, n, L.n_pad, d, order, L.Xs); ++c->launches;
    L.relerr = (float)((d + 16) * 1.1920928955078125e-07);  // (d+16) * 2^-23
    L.radius = radius;
    return L;
}

float widened_radius(float radius, int d)
{
    const double u = 5.9604644775390625e-08;  // 2^-24
    const double ep = (double)radius * (1.0 + (double)(d + 8) * u) + 1e-30;
    if (!(ep < (double)FLT_MAX)) return FLT_MAX;
    const float f = std::nextafter((float)ep, INFINITY);
    return f <= FLT_MAX ? f : FLT_MAX;
}

void run_tiles_fp32(rnng_ctx* c, Layout& L, EdgeOut& E)
{
    int grid = std::max(1, std::min<int>((int)std::min<unsigned long long>(L.tile_pairs, 1ull << 30),
                                         c->num_sms * 4));
    k_tiles_fp32<<<grid, 256, 0, c->stream>>>(L.Xs, L.n, L.d, L.pairs, L.d_tile_pairs, L.tile_pairs, L.radius, E.si,
                                              E.sj, E.w, E.count, E.cap); ++c->launches;
    RNNG_CUDA(cudaGetLastError());
}

void finalize_edges(rnng_ctx* c, const Layout& L, const int64_t* d_ids, const EdgeOut& E, int64_t m, int64_t* u,
                    int64_t* v, float* w)
{
    if (m == 0) return;
    k_finalize_edges<<<grid_for(c, m, 256), 256, 0, c->stream>>>(E.si, E.sj, E.w, m, L.perm, d_ids, u, v, w); ++c->launches;
}

}  // namespace rnng
