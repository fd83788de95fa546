// Register-tiled FP32 distance blocks: landmark assignment.
#pragma once

#include "common.cuh"

namespace rnng {

// 128 rows x 32 columns of squared L2 per block of 256 threads (4 x 4 per thread),
// dimensions staged through shared memory 32 at a time.
constexpr int kDRows = 128, kDCols = 32, kDKC = 32;

struct DistSmem {
    float A[kDKC][kDRows + 4];
    float B[kDKC][kDCols + 4];
};

// Accumulates acc[4][4] += (a - b)^2 over all d dimensions for the block's rows
// (through rowmap) and columns [c0, c0 + 32) of C.
__device__ __forceinline__ void dist_block(DistSmem& sm, const float* __restrict__ X, const int32_t* __restrict__ rowmap,
                                           int64_t r0, int64_t nrows, int d, const float* __restrict__ C, int64_t c0,
                                           int64_t cend, float acc[4][4])
{
    const int tid = threadIdx.x, ty = tid >> 3, tx = tid & 7;
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = 0.f;
    for (int k0 = 0; k0 < d; k0 += kDKC) {
        __syncthreads();
#pragma unroll 4
        for (int idx = tid; idx < kDRows * kDKC; idx += 256) {
            const int r = idx / kDKC, kk = idx % kDKC, k = k0 + kk;
            const int64_t row = r0 + r;
            float v = 0.f;
            if (row < nrows && k < d) {
                const int64_t src = rowmap ? (int64_t)rowmap[row] : row;
                v = X[src * d + k];
            }
            sm.A[kk][r] = v;
        }
        for (int idx = tid; idx < kDCols * kDKC; idx += 256) {
            const int cc = idx / kDKC, kk = idx % kDKC, k = k0 + kk;
            const int64_t col = c0 + cc;
            sm.B[kk][cc] = (col < cend && k < d) ? C[col * d + k] : 0.f;
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < kDKC; ++kk) {
            const float4 a = *reinterpret_cast<const float4*>(&sm.A[kk][ty * 4]);
            const float4 b = *reinterpret_cast<const float4*>(&sm.B[kk][tx * 4]);
            const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const float t = av[r] - bv[c];
                    acc[r][c] = fmaf(t, t, acc[r][c]);
                }
        }
    }
}


// Nearest allowed column per row (see partition.cu); keys_out[row] = col << 32 | bits(dist).
// With a BF16 shift (d <= 256) the distances come from the tensor cores.
void launch_assign(rnng_ctx* c, const float* X, const int32_t* rowmap, int64_t nrows, int d, const float* C,
                   int64_t ncols, const uint64_t* row_key, const int32_t* cell_off, const int32_t* col_rank,
                   const float* shift, uint64_t* keys_out, int32_t* vals_out);
}  // namespace rnng
