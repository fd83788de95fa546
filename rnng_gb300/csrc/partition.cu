// Register-tiled FP32 distance blocks for the landmark partition.
//
// One block computes squared L2 distances between 128 rows (points) and the
// columns (landmarks or pivots) in steps of 32 columns, staging 32-dimension
// chunks of both operands in shared memory; each thread owns a 4 x 4 block of
// distances.  The epilogue keeps, per row, the nearest column inside the row's
// allowed column range (the landmarks of the row's cell's children), written as a
// sort key (child rank << 32 | float bits of the distance) plus the input row index.
// Summation order is free here: the assignment only shapes the partition.
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

void launch_assign(rnng_ctx* c, const float* X, const int32_t* rowmap, int64_t nrows, int d, const float* C,
                   int64_t ncols, const uint64_t* row_key, const int32_t* cell_off, const int32_t* col_rank,
                   uint64_t* keys_out, int32_t* vals_out)
{
    const int64_t blocks = ceil_div(nrows, kDRows);
    if (blocks == 0) return;
    k_assign<<<(unsigned)blocks, 256, 0, c->stream>>>(X, rowmap, nrows, d, C, ncols, row_key, cell_off, col_rank,
                                                      keys_out, vals_out); ++c->launches;
    RNNG_CUDA(cudaGetLastError());
}

}  // namespace rnng
