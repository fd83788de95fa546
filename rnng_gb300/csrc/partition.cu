// Register-tiled FP32 distance blocks for the landmark partition.
//
// One block computes squared L2 distances between 128 rows (points) and the
// columns (landmarks or pivots) in steps of 32 columns, staging 32-dimension
// chunks of both operands in shared memory; each thread owns a 4 x 4 block of
// distances.  The epilogue keeps, per row, the nearest column inside the row's
// allowed column range (the landmarks of the row's cell's children), written as a
// sort key (child rank << 32 | float bits of the distance) plus the input row index.
// Summation order is free here: the assignment only shapes the partition.
#include <cuda_bf16.h>

#include <algorithm>

#include "common.cuh"
#include "eps_l2.cuh"
#include "partition.cuh"

namespace rnng {

// Nearest allowed column per row.  With row_key == nullptr every row may use
// columns [0, ncols); otherwise row p belongs to cell (row_key[p] >> 32) and may
// use columns [cell_off[cell], cell_off[cell + 1]) (rows are sorted by cell, so a
// block's rows cover a contiguous run of cells and their column ranges).
__global__ void __launch_bounds__(256) k_assign(const float* __restrict__ X, const int32_t* __restrict__ rowmap,
                                                int64_t nrows, int d, const float* __restrict__ C, int64_t ncols,
                                                const uint64_t* __restrict__ row_key,
                                                const int32_t* __restrict__ cell_off,
                                                const int32_t* __restrict__ col_rank, uint64_t* __restrict__ keys_out,
                                                int32_t* __restrict__ vals_out)
{
    __shared__ __align__(16) DistSmem sm;
    const int tid = threadIdx.x, ty = tid >> 3, tx = tid & 7;
    const int64_t r0 = (int64_t)blockIdx.x * kDRows;
    if (r0 >= nrows) return;
    int64_t lo = 0, hi = ncols;
    int rlo[4], rhi[4];
    if (row_key) {
        const int64_t last = min(r0 + kDRows, nrows) - 1;
        lo = cell_off[row_key[r0] >> 32];
        hi = cell_off[(row_key[last] >> 32) + 1];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int64_t row = min(r0 + ty * 4 + r, nrows - 1);
            const uint32_t cell = (uint32_t)(row_key[row] >> 32);
            rlo[r] = cell_off[cell];
            rhi[r] = cell_off[cell + 1];
        }
    } else {
#pragma unroll
        for (int r = 0; r < 4; ++r) { rlo[r] = 0; rhi[r] = (int)ncols; }
    }
    float best[4] = {INFINITY, INFINITY, INFINITY, INFINITY};
    int bidx[4] = {0, 0, 0, 0};
    // blocks whose rows all sit in cells that do not split keep their keys: no distances
    int need = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r) need |= (rhi[r] - rlo[r] > 1) ? 1 : 0;
    if (!__syncthreads_or(need)) hi = lo;
    for (int64_t c0 = lo; c0 < hi; c0 += kDCols) {
        // rows of a compacted list can come from far-apart cells: skip chunks no row may use
        int use = 0;
#pragma unroll
        for (int r = 0; r < 4; ++r)
            use |= ((!row_key || rhi[r] - rlo[r] > 1) && rlo[r] < c0 + kDCols && rhi[r] > c0) ? 1 : 0;
        if (!__syncthreads_or(use)) continue;
        float acc[4][4];
        dist_block(sm, X, rowmap, r0, nrows, d, C, c0, hi, acc);
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int col = (int)(c0 + tx * 4 + c);
                if (col >= rlo[r] && col < rhi[r] && acc[r][c] < best[r]) {
                    best[r] = acc[r][c];
                    bidx[r] = col;
                }
            }
    }
    // reduce over the 8 threads that share these rows (consecutive lanes)
#pragma unroll
    for (int r = 0; r < 4; ++r) {
#pragma unroll
        for (int o = 1; o < 8; o <<= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, best[r], o);
            const int oi = __shfl_xor_sync(0xffffffffu, bidx[r], o);
            if (ob < best[r] || (ob == best[r] && oi < bidx[r])) {
                best[r] = ob;
                bidx[r] = oi;
            }
        }
        const int64_t row = r0 + ty * 4 + r;
        if (tx == 0 && row < nrows) {
            if (rhi[r] - rlo[r] == 1 && row_key) {
                // a cell that is not split keeps its order (distance to its old landmark)
                const int col = col_rank ? col_rank[rlo[r]] : rlo[r];
                keys_out[row] = ((uint64_t)(uint32_t)col << 32) | (row_key[row] & 0xffffffffull);
            } else {
                const int col = col_rank ? col_rank[bidx[r]] : bidx[r];
                keys_out[row] = ((uint64_t)(uint32_t)col << 32) | __float_as_uint(sqrtf(best[r]));
            }
            vals_out[row] = rowmap ? rowmap[row] : (int32_t)row;
        }
    }
}

// The same assignment on the tensor cores (d <= 256): distances in the Gram form
// |x~|^2 + |c~|^2 - 2 x~.c~ of the BF16 rows x~ = bf16(x - shift), c~ = bf16(c - shift),
// the dot products by mma.sync (m16n8k16, FP32 accumulation).  Only the partition
// depends on these distances (which child a point joins, and its order inside the
// child), never an edge, so their BF16 rounding is harmless.  A block holds 128 rows,
// a warp 16 of them as A fragments in registers (converted once); the block's columns
// stream through in chunks of 32.  Inside each 32-dimension group the k order is
// permuted the same way for both operands: lane (g, t) holds dimensions 8t .. 8t + 7,
// which feed k-slots {2t, 2t+1, 2t+8, 2t+9} of two consecutive k-steps.

// Eight dimensions 32 kp + 8 t .. + 7 of row `src` of X (zero outside d), shifted and
// rounded to four BF16 pairs; adds their squares to nrm.
__device__ __forceinline__ void load_bf16x8(const float* __restrict__ X, int64_t src, int d, int k0,
                                            const float* __restrict__ shift, bool valid, uint32_t* out, float& nrm)
{
    float v[8];
    if (valid && (d & 7) == 0 && k0 < d) {
        const float4 p = *reinterpret_cast<const float4*>(X + src * d + k0);
        const float4 q = *reinterpret_cast<const float4*>(X + src * d + k0 + 4);
        v[0] = p.x; v[1] = p.y; v[2] = p.z; v[3] = p.w; v[4] = q.x; v[5] = q.y; v[6] = q.z; v[7] = q.w;
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] -= shift[k0 + j];
    } else {
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = (valid && k0 + j < d) ? X[src * d + k0 + j] - shift[k0 + j] : 0.f;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
        const float2 f = __bfloat1622float2(h);
        nrm = fmaf(f.x, f.x, fmaf(f.y, f.y, nrm));
        out[j] = *reinterpret_cast<const uint32_t*>(&h);
    }
}

// Columns as BF16 rows of 32 KP dimensions (shifted, zero padded) and their norms.
__global__ void k_columns_bf16(const float* __restrict__ C, int64_t ncols, int d, int dpad,
                               const float* __restrict__ shift, __nv_bfloat16* __restrict__ out,
                               float* __restrict__ norm)
{
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (int64_t c = warp; c < ncols; c += nwarps) {
        float nrm = 0.f;
        for (int k = lane; k < dpad; k += 32) {
            const __nv_bfloat16 h = __float2bfloat16_rn(k < d ? C[c * d + k] - shift[k] : 0.f);
            const float f = __bfloat162float(h);
            nrm = fmaf(f, f, nrm);
            out[c * dpad + k] = h;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
        if (lane == 0) norm[c] = nrm;
    }
}

template <int KP>  // dimensions padded to 32 KP
__global__ void __launch_bounds__(256) k_assign_mma(const float* __restrict__ X, const int32_t* __restrict__ rowmap,
                                                    int64_t nrows, int d, const uint4* __restrict__ Cb,
                                                    const float* __restrict__ cnorm,
                                                    const uint64_t* __restrict__ row_key,
                                                    const int32_t* __restrict__ cell_off,
                                                    const int32_t* __restrict__ col_rank,
                                                    const float* __restrict__ shift, uint64_t* __restrict__ keys_out,
                                                    int32_t* __restrict__ vals_out)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const int64_t r0 = (int64_t)blockIdx.x * kDRows;
    if (r0 >= nrows) return;
    const int64_t last = min(r0 + kDRows, nrows) - 1;
    int lo = cell_off[row_key[r0] >> 32], hi = cell_off[(row_key[last] >> 32) + 1];
    // this lane's rows: r0 + 16 warp + g + 8 h
    int rlo[2], rhi[2];
    bool rv[2];
    int64_t row[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        row[h] = r0 + 16 * warp + g + 8 * h;
        rv[h] = row[h] < nrows;
        const uint32_t cell = (uint32_t)(row_key[min(row[h], nrows - 1)] >> 32);
        rlo[h] = cell_off[cell];
        rhi[h] = cell_off[cell + 1];
    }
    // blocks whose rows all sit in cells that do not split keep their keys: no rows read,
    // no distances (most blocks at the deeper levels)
    const int need = (rv[0] && rhi[0] - rlo[0] > 1) || (rv[1] && rhi[1] - rlo[1] > 1);
    if (!__syncthreads_or(need)) {
        if (t == 0)
#pragma unroll
            for (int h = 0; h < 2; ++h)
                if (rv[h]) {
                    const int col = col_rank ? col_rank[rlo[h]] : rlo[h];
                    keys_out[row[h]] = ((uint64_t)(uint32_t)col << 32) | (row_key[row[h]] & 0xffffffffull);
                    vals_out[row[h]] = rowmap ? rowmap[row[h]] : (int32_t)row[h];
                }
        return;
    }
    uint32_t af[KP][2][4];
    float xn[2] = {0.f, 0.f};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int64_t src = rv[h] ? (rowmap ? (int64_t)rowmap[row[h]] : row[h]) : 0;
#pragma unroll
        for (int kp = 0; kp < KP; ++kp) load_bf16x8(X, src, d, 32 * kp + 8 * t, shift, rv[h], af[kp][h], xn[h]);
        xn[h] += __shfl_xor_sync(0xffffffffu, xn[h], 1);
        xn[h] += __shfl_xor_sync(0xffffffffu, xn[h], 2);
    }
    float best[2] = {INFINITY, INFINITY};
    int bidx[2] = {0, 0};
    // this warp's column range: the union of its rows' ranges (rows of a compacted list can
    // come from far-apart cells; chunks that none of the warp's rows may use are skipped)
    int wlo = hi, whi = lo;
#pragma unroll
    for (int h = 0; h < 2; ++h)
        if (rv[h] && rhi[h] - rlo[h] > 1) {
            wlo = min(wlo, rlo[h]);
            whi = max(whi, rhi[h]);
        }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        wlo = min(wlo, __shfl_xor_sync(0xffffffffu, wlo, o));
        whi = max(whi, __shfl_xor_sync(0xffffffffu, whi, o));
    }
    for (int c0 = wlo; c0 < whi; c0 += 32) {
        bool use = false;
#pragma unroll
        for (int h = 0; h < 2; ++h) use |= rv[h] && rhi[h] - rlo[h] > 1 && rlo[h] < c0 + 32 && rhi[h] > c0;
        if (!__any_sync(0xffffffffu, use)) continue;
        float acc[4][4];
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[nt][q] = 0.f;
#pragma unroll
        for (int kp = 0; kp < KP; ++kp) {
            uint4 bf[4];
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                const int col = c0 + 8 * nt + g;
                bf[nt] = col < whi ? Cb[(int64_t)col * (4 * KP) + 4 * kp + t] : make_uint4(0u, 0u, 0u, 0u);
            }
#pragma unroll
            for (int nt = 0; nt < 4; ++nt) {
                mma_bf16_16816(acc[nt], af[kp][0][0], af[kp][1][0], af[kp][0][1], af[kp][1][1], bf[nt].x, bf[nt].y);
                mma_bf16_16816(acc[nt], af[kp][0][2], af[kp][1][2], af[kp][0][3], af[kp][1][3], bf[nt].z, bf[nt].w);
            }
        }
        // acc[nt][2 h + e] = row g + 8 h, column c0 + 8 nt + 2 t + e
#pragma unroll
        for (int nt = 0; nt < 4; ++nt)
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int col = c0 + 8 * nt + 2 * t + e;
                const float cn = col < whi ? cnorm[col] : 0.f;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const float dist = fmaf(-2.f, acc[nt][2 * h + e], xn[h] + cn);
                    if (col >= rlo[h] && col < rhi[h] && dist < best[h]) {
                        best[h] = dist;
                        bidx[h] = col;
                    }
                }
            }
    }
    // reduce over the 4 lanes that share these rows
#pragma unroll
    for (int h = 0; h < 2; ++h) {
#pragma unroll
        for (int o = 1; o < 4; o <<= 1) {
            const float ob = __shfl_xor_sync(0xffffffffu, best[h], o);
            const int oi = __shfl_xor_sync(0xffffffffu, bidx[h], o);
            if (ob < best[h] || (ob == best[h] && oi < bidx[h])) {
                best[h] = ob;
                bidx[h] = oi;
            }
        }
        if (t == 0 && rv[h]) {
            if (rhi[h] - rlo[h] == 1) {
                // a cell that is not split keeps its order (distance to its old landmark)
                const int col = col_rank ? col_rank[rlo[h]] : rlo[h];
                keys_out[row[h]] = ((uint64_t)(uint32_t)col << 32) | (row_key[row[h]] & 0xffffffffull);
            } else {
                const int col = col_rank ? col_rank[bidx[h]] : bidx[h];
                keys_out[row[h]] = ((uint64_t)(uint32_t)col << 32) | __float_as_uint(sqrtf(fmaxf(best[h], 0.f)));
            }
            vals_out[row[h]] = rowmap ? rowmap[row[h]] : (int32_t)row[h];
        }
    }
}

template <int KP>
static void assign_mma(rnng_ctx* c, unsigned blocks, const float* X, const int32_t* rowmap, int64_t nrows, int d,
                       const float* C, int64_t ncols, const uint64_t* row_key, const int32_t* cell_off,
                       const int32_t* col_rank, const float* shift, uint64_t* keys_out, int32_t* vals_out)
{
    const int dpad = 32 * KP;
    c->lm_b16.reserve(sizeof(__nv_bfloat16) * (size_t)std::max<int64_t>(ncols, 1) * dpad +
                      sizeof(float) * (size_t)std::max<int64_t>(ncols, 1) + 16);
    __nv_bfloat16* cb = c->lm_b16.as<__nv_bfloat16>();
    float* cnorm = reinterpret_cast<float*>(cb + (size_t)std::max<int64_t>(ncols, 1) * dpad);
    const int64_t g = std::max<int64_t>(1, std::min<int64_t>(ceil_div(ncols * 32, 256), (int64_t)c->num_sms * 8));
    k_columns_bf16<<<(unsigned)g, 256, 0, c->stream>>>(C, ncols, d, dpad, shift, cb, cnorm); ++c->launches;
    k_assign_mma<KP><<<blocks, 256, 0, c->stream>>>(X, rowmap, nrows, d, reinterpret_cast<const uint4*>(cb), cnorm,
                                                    row_key, cell_off, col_rank, shift, keys_out, vals_out);
}

void launch_assign(rnng_ctx* c, const float* X, const int32_t* rowmap, int64_t nrows, int d, const float* C,
                   int64_t ncols, const uint64_t* row_key, const int32_t* cell_off, const int32_t* col_rank,
                   const float* shift, uint64_t* keys_out, int32_t* vals_out)
{
    const int64_t blocks = ceil_div(nrows, kDRows);
    if (blocks == 0) return;
    const unsigned b = (unsigned)blocks;
    if (shift && row_key && d <= 256) {
        switch ((d + 31) / 32) {
            case 1: assign_mma<1>(c, b, X, rowmap, nrows, d, C, ncols, row_key, cell_off, col_rank, shift, keys_out, vals_out); break;
            case 2: assign_mma<2>(c, b, X, rowmap, nrows, d, C, ncols, row_key, cell_off, col_rank, shift, keys_out, vals_out); break;
            case 3: assign_mma<3>(c, b, X, rowmap, nrows, d, C, ncols, row_key, cell_off, col_rank, shift, keys_out, vals_out); break;
            case 4: assign_mma<4>(c, b, X, rowmap, nrows, d, C, ncols, row_key, cell_off, col_rank, shift, keys_out, vals_out); break;
            case 5: assign_mma<5>(c, b, X, rowmap, nrows, d, C, ncols, row_key, cell_off, col_rank, shift, keys_out, vals_out); break;
            case 6: assign_mma<6>(c, b, X, rowmap, nrows, d, C, ncols, row_key, cell_off, col_rank, shift, keys_out, vals_out); break;
            case 7: assign_mma<7>(c, b, X, rowmap, nrows, d, C, ncols, row_key, cell_off, col_rank, shift, keys_out, vals_out); break;
            default: assign_mma<8>(c, b, X, rowmap, nrows, d, C, ncols, row_key, cell_off, col_rank, shift, keys_out, vals_out); break;
        }
    } else {
        k_assign<<<b, 256, 0, c->stream>>>(X, rowmap, nrows, d, C, ncols, row_key, cell_off, col_rank, keys_out,
                                           vals_out);
    }
    ++c->launches;
    RNNG_CUDA(cudaGetLastError());
}

}  // namespace rnng
