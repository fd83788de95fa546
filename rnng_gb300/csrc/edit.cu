// Epsilon graph under RNNG's edit distance (drivers/systolic.cpp:271-299: unit-cost
// Levenshtein distance, returned as a float; edge iff distance <= radius).
//
// All arithmetic is integer, so the result is exact by construction:
//   1. strings are sorted by length and cut into tiles of 128;
//   2. a tile pair is considered only when some of its strings differ in length by at
//      most K = floor(radius) (the length difference is a lower bound of the distance);
//   3. every pair of a considered tile pair passes two sound filters: |len a - len b|
//      <= K, and the L1 distance of hashed 3-gram profiles <= 2 * 3 * K (one edit
//      changes at most q = 3 q-grams out and q in; merging q-grams into 64 hash bins and
//      saturating counts only lowers L1, so no pair within K is rejected);
//   4. every surviving pair gets a banded dynamic program over the diagonals |i-j| <= K
//      with cell values capped at K+1.  Cells outside the band exceed K anyway, so the
//      band gives the exact distance whenever it is <= K (Ukkonen's cut-off).
// Distances above K are never reported, so the cap never shows in the output.
#include <cub/cub.cuh>

#include <algorithm>
#include <cfloat>
#include <cstring>

#include "balls.cuh"
#include "common.cuh"
#include "eps_l2.cuh"
#include "kernels_misc.cuh"

namespace rnng {

constexpr int kET = 128;      // strings per tile
constexpr int kBins = 64;     // hashed 3-gram profile bins (one byte each)
constexpr int kQ = 3;

__global__ void k_edit_lengths(const int64_t* __restrict__ off, int64_t n, uint32_t* __restrict__ len,
                               int32_t* __restrict__ idx)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        len[i] = (uint32_t)(off[i + 1] - off[i]);
        idx[i] = (int32_t)i;
    }
}

__device__ __forceinline__ int qgram_bin(uint32_t a, uint32_t b, uint32_t c)
{
    return (int)(((a * 0x9E3779B1u) ^ (b * 0x85EBCA77u) ^ (c * 0xC2B2AE3Du)) >> 26);
}

// Profile of sorted string p (64 saturating byte counts); padding rows get zeros.
__global__ void __launch_bounds__(128) k_edit_profiles(const uint8_t* __restrict__ atoms,
                                                       const int64_t* __restrict__ off,
                                                       const int32_t* __restrict__ perm, int64_t n, int64_t n_pad,
                                                       uint32_t* __restrict__ prof)
{
    __shared__ uint8_t h[128][kBins];
    for (int64_t base = (int64_t)blockIdx.x * 128; base < n_pad; base += (int64_t)gridDim.x * 128) {
        const int64_t p = base + threadIdx.x;
        for (int b = 0; b < kBins; ++b) h[threadIdx.x][b] = 0;
        if (p < n) {
            const int64_t o = off[perm[p]], m = off[perm[p] + 1] - o;
            for (int64_t i = 0; i + kQ <= m; ++i) {
                const int b = qgram_bin(atoms[o + i], atoms[o + i + 1], atoms[o + i + 2]);
                if (h[threadIdx.x][b] < 255) h[threadIdx.x][b]++;
            }
        }
        const uint32_t* hw = reinterpret_cast<const uint32_t*>(h[threadIdx.x]);
        for (int k = 0; k < kBins / 4; ++k) prof[p * (kBins / 4) + k] = hw[k];
        __syncthreads();
    }
}

// Tile t's string lengths: [min, max] over its real strings (sorted ascending).
__global__ void k_edit_tile_len(const uint32_t* __restrict__ slen, int64_t n, int64_t T, uint32_t* __restrict__ lo,
                                uint32_t* __restrict__ hi)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < T; t += (int64_t)gridDim.x * blockDim.x) {
        lo[t] = slen[t * kET];
        hi[t] = slen[min(n, (t + 1) * kET) - 1];
    }
}

// Number of partner tiles j >= i whose shortest string is within K of tile i's longest.
__global__ void k_edit_ranges(const uint32_t* __restrict__ lo, const uint32_t* __restrict__ hi, int64_t T, int K,
                              int32_t* __restrict__ cnt)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < T; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t lim = (uint64_t)hi[i] + (uint64_t)K;
        int64_t a = i, b = T;  // first j with lo[j] > lim
        while (a < b) {
            const int64_t m = (a + b) / 2;
            if ((uint64_t)lo[m] <= lim) a = m + 1;
            else b = m;
        }
        cnt[i] = (int32_t)(a - i);
    }
}

__global__ void k_edit_emit_pairs(const int32_t* __restrict__ cnt, const int32_t* __restrict__ off, int64_t T,
                                  int2* __restrict__ pairs)
{
    for (int64_t i = blockIdx.x; i < T; i += gridDim.x)
        for (int k = threadIdx.x; k < cnt[i]; k += blockDim.x) pairs[off[i] + k] = make_int2((int)i, (int)(i + k));
}

// Filter operand: the profile thermometer-coded with counts capped at 8, one warp per
// row, bin b's levels l = 0..7 at byte 8 b + l (E4M3 1.0 = 0x38 when count > l, else 0).
// Then x_a . x_b = sum over bins of min(min(c_a, 8), min(c_b, 8)) and with n = sum of
// min(c, 8), n_a + n_b - 2 x_a.x_b is the L1 distance of the capped profiles: never
// above the L1 of the counts themselves, so it is still <= 2 q K for strings within K.
// rowinfo = {n, 0, 0, n} and ucol = n are the tensor-core kernel's row and column terms.
__global__ void k_edit_thermo(const uint32_t* __restrict__ prof, int64_t n_pad, uint8_t* __restrict__ x8,
                              float4* __restrict__ rowinfo, float* __restrict__ ucol)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t p = warp; p < n_pad; p += nwarps) {
        // lane l: bins 2 l and 2 l + 1 (bytes 2 (l % 2) .. of profile word l / 2)
        const uint32_t wv = prof[p * (kBins / 4) + (lane >> 1)];
        const uint32_t c0 = (wv >> (16 * (lane & 1))) & 0xffu, c1 = (wv >> (16 * (lane & 1) + 8)) & 0xffu;
        uint32_t q[4];
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            const uint32_t cnt = w < 2 ? c0 : c1;
            uint32_t v = 0;
#pragma unroll
            for (int b = 0; b < 4; ++b) v |= (cnt > (uint32_t)(4 * (w & 1) + b) ? 0x38u : 0u) << (8 * b);
            q[w] = v;
        }
        reinterpret_cast<uint4*>(x8 + p * kFilterBytes)[lane] = make_uint4(q[0], q[1], q[2], q[3]);
        float nn = (float)(min(c0, 8u) + min(c1, 8u));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nn += __shfl_xor_sync(0xffffffffu, nn, o);
        if (lane == 0) {
            rowinfo[p] = make_float4(nn, 0.f, 0.f, nn);
            ucol[p] = nn;
        }
    }
}

// Filter operand for alphabets of at most 4 symbols (symmap codes 0..3): exact 4-grams,
// bin = the 4-gram's base-4 code (256 bins, no collisions), counts capped at 2, bin b's
// two levels at bytes 2 b and 2 b + 1.  Then n_a + n_b - 2 x_a.x_b is the L1 distance of
// the capped 4-gram profiles, <= 2 q K = 8 K for strings within K.  One warp per row,
// its counts in shared memory; rows in length-sorted order.
__global__ void __launch_bounds__(256) k_edit_thermo_q4(const uint8_t* __restrict__ atoms,
                                                        const int64_t* __restrict__ off,
                                                        const int32_t* __restrict__ perm, int64_t n, int64_t n_pad,
                                                        const uint8_t* __restrict__ symmap, uint8_t* __restrict__ x8,
                                                        float4* __restrict__ rowinfo, float* __restrict__ ucol)
{
    __shared__ uint32_t cnt[8][256];
    __shared__ uint8_t smap[256];
    for (int k = threadIdx.x; k < 256; k += blockDim.x) smap[k] = symmap[k];
    __syncthreads();
    const int lane = threadIdx.x & 31, wb = threadIdx.x >> 5;
    uint32_t* h = cnt[wb];
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t p = warp; p < n_pad; p += nwarps) {
        for (int b = lane; b < 256; b += 32) h[b] = 0;
        __syncwarp();
        if (p < n) {
            const int64_t o = off[perm[p]], m = off[perm[p] + 1] - o;
            for (int64_t i = lane; i + 4 <= m; i += 32) {
                const uint32_t code = ((uint32_t)smap[atoms[o + i]] << 6) | ((uint32_t)smap[atoms[o + i + 1]] << 4) |
                                      ((uint32_t)smap[atoms[o + i + 2]] << 2) | (uint32_t)smap[atoms[o + i + 3]];
                atomicAdd(&h[code], 1u);
            }
        }
        __syncwarp();
        // lane l: bins 8 l .. 8 l + 7 -> bytes 16 l .. 16 l + 15
        uint32_t q[4];
        uint32_t nn = 0;
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            const uint32_t c0 = h[8 * lane + 2 * w], c1 = h[8 * lane + 2 * w + 1];
            q[w] = (c0 > 0 ? 0x38u : 0u) | (c0 > 1 ? 0x38u : 0u) << 8 | (c1 > 0 ? 0x38u : 0u) << 16 |
                   (c1 > 1 ? 0x38u : 0u) << 24;
            nn += min(c0, 2u) + min(c1, 2u);
        }
        reinterpret_cast<uint4*>(x8 + p * kFilterBytes)[lane] = make_uint4(q[0], q[1], q[2], q[3]);
        float nf = (float)nn;
#pragma unroll
        for (int o2 = 16; o2 > 0; o2 >>= 1) nf += __shfl_xor_sync(0xffffffffu, nf, o2);
        if (lane == 0) {
            rowinfo[p] = make_float4(nf, 0.f, 0.f, nf);
            ucol[p] = nf;
        }
        __syncwarp();
    }
}

// Per tile: {0, largest n of its rows} (the kernel's column-tile term; no error radii).
__global__ void k_edit_tileinfo(const float4* __restrict__ rowinfo, int64_t T, float2* __restrict__ tileinfo)
{
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < T; t += (int64_t)gridDim.x * blockDim.x) {
        float m = 0.f;
        for (int r = 0; r < kET; ++r) m = fmaxf(m, rowinfo[t * kET + r].x);
        tileinfo[t] = make_float2(0.f, m);
    }
}

// Banded edit distance, band half-width B >= K, values capped at K + 1.
template <int B>
__device__ int banded_edit(const uint8_t* __restrict__ s, int m, const uint8_t* __restrict__ t, int n, int K)
{
    constexpr int W = 2 * B + 1;
    const int INF = K + 1;
    int prev[W], cur[W];
    // row 0: D[0][j] = j for j = k - B in [0, n]
#pragma unroll
    for (int k = 0; k < W; ++k) {
        const int j = k - B;
        prev[k] = (j >= 0 && j <= n) ? min(j, INF) : INF;
    }
    // window of t: tw[k] = t[i + k - B - 1] for the current row i (0 outside)
    int tw[W];
#pragma unroll
    for (int k = 0; k < W; ++k) {
        const int j = 1 + k - B - 1;  // row i = 1
        tw[k] = (j >= 0 && j < n) ? (int)t[j] : -1;
    }
    for (int i = 1; i <= m; ++i) {
        const int si = (int)s[i - 1];
        int rowmin = INF;
#pragma unroll
        for (int k = 0; k < W; ++k) {
            const int j = i + k - B;
            int v;
            if (j < 0 || j > n) {
                v = INF;
            } else if (j == 0) {
                v = min(i, INF);
            } else {
                const int diag = prev[k] + (si == tw[k] ? 0 : 1);
                const int up = (k + 1 < W ? prev[k + 1] : INF) + 1;
                const int left = (k > 0 ? cur[k - 1] : INF) + 1;
                v = min(min(diag, up), min(left, INF));
            }
            cur[k] = v;
            rowmin = min(rowmin, v);
        }
        if (rowmin > K) return INF;
#pragma unroll
        for (int k = 0; k < W; ++k) prev[k] = cur[k];
        // slide the t window by one for row i + 1
#pragma unroll
        for (int k = 0; k + 1 < W; ++k) tw[k] = tw[k + 1];
        {
            const int j = i + 1 + (W - 1) - B - 1;
            tw[W - 1] = (j >= 0 && j < n) ? (int)t[j] : -1;
        }
    }
    const int k = n - m + B;
    return (k >= 0 && k < W) ? prev[k] : INF;
}

template <int B>
__global__ void __launch_bounds__(256) k_edit_verify(const uint8_t* __restrict__ atoms,
                                                     const int64_t* __restrict__ off,
                                                     const int32_t* __restrict__ perm, const uint2* __restrict__ cand,
                                                     const unsigned long long* __restrict__ ncand_ptr,
                                                     unsigned long long ccap, int K, uint32_t* __restrict__ eu,
                                                     uint32_t* __restrict__ ev, float* __restrict__ ew,
                                                     unsigned long long* __restrict__ ecount, unsigned long long cap)
{
    __shared__ int s_warp[8];
    __shared__ unsigned long long s_base;
    const unsigned long long nc = min(*ncand_ptr, ccap);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long round = (unsigned long long)blockIdx.x * blockDim.x; round < nc; round += stride) {
        const unsigned long long e = round + threadIdx.x;
        bool hit = false;
        int dist = 0;
        uint2 c = make_uint2(0, 0);
        if (e < nc) {
            c = cand[e];
            const int64_t oa = off[perm[c.x]], ob = off[perm[c.y]];
            const int ma = (int)(off[perm[c.x] + 1] - oa), mb = (int)(off[perm[c.y] + 1] - ob);
            // the reference computes EditDistance(indexed point, query); the distance is symmetric
            // and at least the length difference
            dist = (ma > mb ? ma - mb : mb - ma) > K ? K + 1 : banded_edit<B>(atoms + oa, ma, atoms + ob, mb, K);
            hit = dist <= K;
        }
        const unsigned ball = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) s_warp[warp] = __popc(ball);
        __syncthreads();
        if (threadIdx.x == 0) {
            int a = 0;
            for (int k = 0; k < 8; ++k) { const int t = s_warp[k]; s_warp[k] = a; a += t; }
            s_base = a ? atomicAdd(ecount, (unsigned long long)a) : 0ull;
        }
        __syncthreads();
        if (hit) {
            const unsigned long long pos = s_base + s_warp[warp] + __popc(ball & ((1u << lane) - 1u));
            if (pos < cap) {
                eu[pos] = c.x;
                ev[pos] = c.y;
                ew[pos] = (float)dist;
            }
        }
        __syncthreads();
    }
}

// One 64-bit block of Myers' column step (G. Myers, J. ACM 46(3), 1999, block form):
// vertical deltas (pv, mv) of 64 pattern rows against one text character with match
// vector eq and horizontal delta hin entering at the block's top row; returns the
// horizontal delta leaving the block at row bit `hb`.
__device__ __forceinline__ int myers_block(unsigned long long eq, unsigned long long& pv, unsigned long long& mv,
                                           int hin, unsigned long long hb)
{
    const unsigned long long neg = hin < 0 ? 1ull : 0ull, pos = hin > 0 ? 1ull : 0ull;
    const unsigned long long xv = eq | mv;
    eq |= neg;
    const unsigned long long xh = (((eq & pv) + pv) ^ pv) | eq;
    unsigned long long ph = mv | ~(xh | pv);
    unsigned long long mh = pv & xh;
    const int hout = (ph & hb) ? 1 : ((mh & hb) ? -1 : 0);
    ph = (ph << 1) | pos;
    mh = (mh << 1) | neg;
    pv = mh | ~(xv | ph);
    mv = ph & xv;
    return hout;
}

constexpr int kBpMaxSym = 8;    // symbols of the compressed alphabet
constexpr int kBpMaxLen = 128;  // pattern length (two 64-bit blocks)
constexpr int kBpSlot = 2 * kBpMaxSym + 1;  // 64-bit words per thread slot (+1 against bank conflicts)

// Verification by Myers' bit-vector algorithm: per candidate the shorter string is the
// pattern (its match vectors per symbol of the dataset's alphabet, at most 8 symbols,
// built in the thread's shared slot), the longer the text; the whole-string distance
// is D[m][n] = m + the horizontal deltas leaving row m.  A column can lower the
// distance by at most one, so the scan stops as soon as the distance cannot come back
// to K.  Exact for every pair; used when the alphabet has at most 8 symbols and no
// string is longer than 128 (otherwise k_edit_verify's banded DP runs).
__global__ void __launch_bounds__(256) k_edit_verify_bp(const uint8_t* __restrict__ atoms,
                                                        const int64_t* __restrict__ off,
                                                        const int32_t* __restrict__ perm,
                                                        const uint2* __restrict__ cand,
                                                        const unsigned long long* __restrict__ ncand_ptr,
                                                        unsigned long long ccap, int K,
                                                        const uint8_t* __restrict__ symmap,
                                                        uint32_t* __restrict__ eu, uint32_t* __restrict__ ev,
                                                        float* __restrict__ ew, unsigned long long* __restrict__ ecount,
                                                        unsigned long long cap)
{
    __shared__ unsigned long long peq_all[256 * kBpSlot];
    __shared__ uint8_t smap[256];
    __shared__ int s_warp[8];
    __shared__ unsigned long long s_base;
    for (int k = threadIdx.x; k < 256; k += blockDim.x) smap[k] = symmap[k];
    __syncthreads();
    unsigned long long* peq = peq_all + threadIdx.x * kBpSlot;
    const unsigned long long nc = min(*ncand_ptr, ccap);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long round = (unsigned long long)blockIdx.x * blockDim.x; round < nc; round += stride) {
        const unsigned long long e = round + threadIdx.x;
        bool hit = false;
        int dist = 0;
        uint2 c = make_uint2(0, 0);
        if (e < nc) {
            c = cand[e];
            const int64_t oa = off[perm[c.x]], ob = off[perm[c.y]];
            const int ma = (int)(off[perm[c.x] + 1] - oa), mb = (int)(off[perm[c.y] + 1] - ob);
            // the distance is symmetric: the shorter string is the pattern
            const bool a_pat = ma <= mb;
            const uint8_t* pat = atoms + (a_pat ? oa : ob);
            const uint8_t* txt = atoms + (a_pat ? ob : oa);
            const int m = a_pat ? ma : mb, n = a_pat ? mb : ma;
            if (n - m > K) {
                dist = K + 1;  // the distance is at least the length difference
            } else if (m == 0) {
                dist = n;
            } else {
#pragma unroll
                for (int k = 0; k < 2 * kBpMaxSym; ++k) peq[k] = 0ull;
                for (int i = 0; i < m; ++i) peq[2 * smap[pat[i]] + (i >> 6)] |= 1ull << (i & 63);
                unsigned long long pv0 = ~0ull, mv0 = 0ull, pv1 = ~0ull, mv1 = 0ull;
                const unsigned long long last = 1ull << ((m - 1) & 63);
                int score = m;
                if (m <= 64) {
                    for (int j = 0; j < n; ++j) {
                        const int sym = smap[txt[j]];
                        score += myers_block(peq[2 * sym], pv0, mv0, 1, last);
                        if (score > K + (n - 1 - j)) break;
                    }
                } else {
                    // Two blocks with Ukkonen's cut-off: a cell within K has |row - column| <= K,
                    // so the first block (pattern rows 1..64) is needed up to column 64 + K and the
                    // second (rows 65..m) from column 64 - K on.  Past its last column the first
                    // block hands the second a +1 per column (row 64 then grows by insertions: a
                    // real path's cost, and above K there); the second starts with +1 per row
                    // below D[64][64 - K].  Both stand-ins are costs of real paths and exceed K
                    // where they stand in, so every distance <= K comes out exact.
                    const int j1 = 64 - K > 0 ? 64 - K : 0, j0 = 64 + K;
                    int score0 = 64;  // D[64][j], the first block's bottom row
                    for (int j = 0; j < n; ++j) {
                        const int sym = smap[txt[j]];
                        if (j == j1) score = score0 + (m - 64);  // D[m][j1] along column j1
                        int h0 = 1;
                        if (j < j0) {
                            h0 = myers_block(peq[2 * sym], pv0, mv0, 1, 1ull << 63);
                            score0 += h0;
                        }
                        if (j >= j1) {
                            score += myers_block(peq[2 * sym + 1], pv1, mv1, h0, last);
                            if (score > K + (n - 1 - j)) break;
                        }
                    }
                }
                dist = score;
            }
            hit = dist <= K;
        }
        const unsigned ball = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) s_warp[warp] = __popc(ball);
        __syncthreads();
        if (threadIdx.x == 0) {
            int a = 0;
            for (int k = 0; k < 8; ++k) { const int t = s_warp[k]; s_warp[k] = a; a += t; }
            s_base = a ? atomicAdd(ecount, (unsigned long long)a) : 0ull;
        }
        __syncthreads();
        if (hit) {
            const unsigned long long pos = s_base + s_warp[warp] + __popc(ball & ((1u << lane) - 1u));
            if (pos < cap) {
                eu[pos] = c.x;
                ev[pos] = c.y;
                ew[pos] = (float)dist;
            }
        }
        __syncthreads();
    }
}

// Byte histogram of the strings (the alphabet of the bit-parallel verification).
__global__ void k_byte_hist(const uint8_t* __restrict__ atoms, int64_t natoms, unsigned int* __restrict__ hist)
{
    __shared__ unsigned int h[256];
    for (int k = threadIdx.x; k < 256; k += blockDim.x) h[k] = 0;
    __syncthreads();
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < natoms; i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&h[atoms[i]], 1u);
    __syncthreads();
    for (int k = threadIdx.x; k < 256; k += blockDim.x)
        if (h[k]) atomicAdd(&hist[k], h[k]);
}

__global__ void k_edit_finalize(const uint32_t* __restrict__ si, const uint32_t* __restrict__ sj,
                                const float* __restrict__ sw, int64_t m, const int32_t* __restrict__ perm,
                                const int64_t* __restrict__ ids, int64_t* __restrict__ u, int64_t* __restrict__ v,
                                float* __restrict__ w)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const int32_t a = perm[si[e]], b = perm[sj[e]];
        const int64_t ia = ids ? ids[a] : (int64_t)a, ib = ids ? ids[b] : (int64_t)b;
        u[e] = ia < ib ? ia : ib;
        v[e] = ia < ib ? ib : ia;
        w[e] = sw[e];
    }
}

// ---------------------------------------------------------------------------------------
// Nearest centre under edit distance (rnng_voronoi_edit).
//
// Full (unbanded) unit-cost Levenshtein distance by Myers' bit-vector algorithm (G. Myers,
// "A fast bit-vector algorithm for approximate string matching based on dynamic
// programming", J. ACM 46(3), 1999), in its multi-word block form, computing the whole-
// string distance as H. Hyyro describes it: the DP column of the centre (the pattern,
// one bit per character) is kept as vertical +1/-1 delta vectors Pv/Mv, the first row
// D[0][j] = j feeds a +1 horizontal delta into the first word at every text column, and
// the distance D[m][n] is m plus the horizontal deltas that leave pattern row m.  Rows
// only depend on the rows above them, so the padding bits of the last word never reach
// row m.  The result is the integer distance, converted to float like the reference's.

constexpr int kVE = 128;     // points (texts) per block
constexpr int kVEMaxW = 64;  // 64-bit words per centre: centres up to 4096 characters

template <int WT>  // WT > 0: at most WT words in registers; WT == 0: any W <= kVEMaxW
__device__ __forceinline__ int myers_distance(const unsigned long long* __restrict__ peq, int W, int lp,
                                              const uint8_t* __restrict__ t, int64_t lt)
{
    constexpr int kCap = WT > 0 ? WT : kVEMaxW;
    unsigned long long Pv[kCap], Mv[kCap];
#pragma unroll
    for (int w = 0; w < kCap; ++w) {
        Pv[w] = ~0ull;
        Mv[w] = 0ull;
    }
    const unsigned long long last_bit = 1ull << ((lp - 1) & 63);
    const int nw = WT > 0 ? WT : W;  // with WT > 0 the words past W see Eq = 0 and are ignored
    int score = lp;
    for (int64_t j = 0; j < lt; ++j) {
        const unsigned long long* eq = peq + (int)t[j] * W;
        int hin = 1, hlast = 0;
#pragma unroll(WT > 0 ? WT : 1)
        for (int w = 0; w < nw; ++w) {
            unsigned long long Eq = w < W ? eq[w] : 0ull;
            const unsigned long long pv = Pv[w], mv = Mv[w];
            const unsigned long long neg = hin < 0 ? 1ull : 0ull, pos = hin > 0 ? 1ull : 0ull;
            const unsigned long long Xv = Eq | mv;
            Eq |= neg;
            const unsigned long long Xh = (((Eq & pv) + pv) ^ pv) | Eq;
            unsigned long long Ph = mv | ~(Xh | pv);
            unsigned long long Mh = pv & Xh;
            const unsigned long long hb = (w == W - 1) ? last_bit : (1ull << 63);
            const int hout = (Ph & hb) ? 1 : ((Mh & hb) ? -1 : 0);
            Ph = (Ph << 1) | pos;
            Mh = (Mh << 1) | neg;
            Pv[w] = Mh | ~(Xv | Ph);
            Mv[w] = Ph & Xv;
            if (w == W - 1) hlast = hout;
            hin = hout;
        }
        score += hlast;
    }
    return score;
}

// One thread per point, the centres in order; each centre's match vectors Peq[symbol][word]
// are built once per block in shared memory.  `dist <= best` keeps the last of equal
// distances, best starts at FLT_MAX and the cell at 0 (include/point.hpp:537-559).
template <int WT>
__global__ void __launch_bounds__(kVE) k_voronoi_edit(const uint8_t* __restrict__ atoms,
                                                      const int64_t* __restrict__ off, int64_t n,
                                                      const uint8_t* __restrict__ catoms,
                                                      const int64_t* __restrict__ coff, int64_t m,
                                                      int64_t* __restrict__ cell, float* __restrict__ dist)
{
    extern __shared__ unsigned long long peq[];  // 256 * Wmax words
    const int64_t i = (int64_t)blockIdx.x * kVE + threadIdx.x;
    const bool live = i < n;
    const int64_t to = live ? off[i] : 0, lt = live ? off[i + 1] - to : 0;
    const uint8_t* t = atoms + to;
    float best = FLT_MAX;
    int64_t bi = 0;
    for (int64_t c = 0; c < m; ++c) {
        const int64_t co = coff[c];
        const int lp = (int)(coff[c + 1] - co);
        const int W = (lp + 63) >> 6;
        __syncthreads();  // previous centre's vectors are no longer read
        for (int k = threadIdx.x; k < 256 * W; k += kVE) peq[k] = 0ull;
        __syncthreads();
        for (int k = threadIdx.x; k < lp; k += kVE)
            atomicOr(&peq[(int)catoms[co + k] * W + (k >> 6)], 1ull << (k & 63));
        __syncthreads();
        if (live) {
            const int dv = lp == 0 ? (int)lt : myers_distance<WT>(peq, W, lp, t, lt);
            const float d = (float)dv;
            if (d <= best) {
                best = d;
                bi = c;
            }
        }
    }
    if (live) {
        cell[i] = bi;
        dist[i] = best;
    }
}

__global__ void k_max_len(const int64_t* __restrict__ off, int64_t m, unsigned long long* __restrict__ out)
{
    unsigned long long mx = 0;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < m; c += (int64_t)gridDim.x * blockDim.x)
        mx = max(mx, (unsigned long long)(off[c + 1] - off[c]));
    atomicMax(out, mx);
}

}  // namespace rnng

using namespace rnng;

extern "C" int rnng_eps_graph_edit(rnng_ctx* c, const uint8_t* atoms, const int64_t* offsets, const int64_t* ids,
                                   int64_t n, float radius, unsigned flags, rnng_edges* out)
{
    return guarded(c, [&] {
        RNNG_REQUIRE(out != nullptr, RNNG_ERR_INVALID, "out is null");
        std::memset(out, 0, sizeof(*out));
        RNNG_REQUIRE(n >= 0 && (n == 0 || (atoms && offsets)), RNNG_ERR_INVALID, "bad strings");
        RNNG_REQUIRE(n < (int64_t(1) << 31) - kET, RNNG_ERR_INVALID, "too many strings");
        RNNG_REQUIRE(radius == radius, RNNG_ERR_INVALID, "radius is NaN");
        c->stats = rnng_stats{};
        c->launches = 0;
        c->gram_ms = 0.0;
        cudaStream_t s = c->stream;
        const int K = radius < 0.f ? -1 : (int)std::min(std::floor((double)radius), 1e9);
        RNNG_REQUIRE(K <= 32, RNNG_ERR_UNSUPPORTED, "edit-distance radius above 32 is not supported");
        // inputs
        int64_t natoms = 0;
        const int64_t* doff = offsets;
        const uint8_t* datoms = atoms;
        const int64_t* dids = ids;
        if (!(flags & RNNG_INPUT_DEVICE)) {
            natoms = n > 0 ? offsets[n] : 0;
            c->ids_in.reserve(sizeof(int64_t) * (size_t)(n + 1));
            c->x_in.reserve(std::max<size_t>((size_t)natoms, 1));
            RNNG_CUDA(cudaMemcpyAsync(c->ids_in.ptr, offsets, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, s));
            if (natoms) RNNG_CUDA(cudaMemcpyAsync(c->x_in.ptr, atoms, (size_t)natoms, cudaMemcpyHostToDevice, s));
            doff = c->ids_in.as<int64_t>();
            datoms = c->x_in.as<uint8_t>();
            if (ids) {
                c->aux7.reserve(sizeof(int64_t) * (size_t)std::max<int64_t>(n, 1));
                RNNG_CUDA(cudaMemcpyAsync(c->aux7.ptr, ids, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s));
                dids = c->aux7.as<int64_t>();
            }
        }
        int64_t m = 0;
        c->out_u.reserve(8);
        c->out_v.reserve(8);
        c->out_w.reserve(8);
        if (n >= 2 && K >= 0) {
            const int64_t T = ceil_div(n, kET), n_pad = T * kET;
            RNNG_REQUIRE(T < 65536, RNNG_ERR_UNSUPPORTED, "more than 8M strings per call");
            const unsigned g = (unsigned)std::min<int64_t>(ceil_div(n, 256), (int64_t)c->num_sms * 8);
            // 1. sort by length
            c->keys.reserve(sizeof(uint32_t) * 2 * n_pad);
            c->perm.reserve(sizeof(int32_t) * 2 * n_pad);
            uint32_t* len = c->keys.as<uint32_t>();
            uint32_t* slen = len + n_pad;
            int32_t* idx = c->perm.as<int32_t>();
            int32_t* perm = idx + n_pad;
            k_edit_lengths<<<g, 256, 0, s>>>(doff, n, len, idx);
            ++c->launches;
            size_t tmp = 0;
            RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, len, slen, idx, perm, (int)n, 0, 32, s));
            c->cub_tmp.reserve(tmp);
            RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, len, slen, idx, perm, (int)n, 0, 32, s));
            c->launches += cub_sort_kernels(n, 32);
            // 2. the alphabet (byte histogram; its symbols numbered in byte order), then the
            //    filter profiles and tile length ranges: exact 4-grams over at most 4 symbols,
            //    else hashed 3-grams
            uint32_t maxlen = 0;
            int64_t total_atoms = 0;
            RNNG_CUDA(cudaMemcpyAsync(&maxlen, slen + (n - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
            RNNG_CUDA(cudaMemcpyAsync(&total_atoms, doff + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
            c->sym.reserve(256 * sizeof(unsigned int) + 256);
            unsigned int* hist = c->sym.as<unsigned int>();
            uint8_t* symmap = (uint8_t*)(hist + 256);
            RNNG_CUDA(cudaMemsetAsync(hist, 0, 256 * sizeof(unsigned int), s));
            RNNG_CUDA(cudaStreamSynchronize(s));
            if (total_atoms > 0) {  // offsets start at 0 (RNNG's layout)
                k_byte_hist<<<(unsigned)std::min<int64_t>(ceil_div(total_atoms, 256), (int64_t)c->num_sms * 4), 256, 0,
                              s>>>(datoms, total_atoms, hist);
                ++c->launches;
            }
            unsigned int h[256];
            RNNG_CUDA(cudaMemcpyAsync(h, hist, sizeof(h), cudaMemcpyDeviceToHost, s));
            RNNG_CUDA(cudaStreamSynchronize(s));
            uint8_t map[256];
            int nsym = 0;
            for (int b = 0; b < 256; ++b) map[b] = h[b] ? (uint8_t)(nsym++) : (uint8_t)0;
            if (nsym <= kBpMaxSym) {
                RNNG_CUDA(cudaMemcpyAsync(symmap, map, 256, cudaMemcpyHostToDevice, s));
                RNNG_CUDA(cudaStreamSynchronize(s));  // map lifetime
            }
            const bool exact4 = nsym <= 4;
            const int qf = exact4 ? 4 : kQ;  // q of the filter's q-grams
            c->x_sorted.reserve(sizeof(uint32_t) * (size_t)n_pad * (kBins / 4));
            uint32_t* prof = c->x_sorted.as<uint32_t>();
            if (!exact4) {
                k_edit_profiles<<<(unsigned)std::min<int64_t>(T, (int64_t)c->num_sms * 8), 128, 0, s>>>(
                    datoms, doff, perm, n, n_pad, prof);
                ++c->launches;
            }
            c->aux2.reserve(sizeof(uint32_t) * 2 * (size_t)T + sizeof(int32_t) * 2 * ((size_t)T + 1));
            uint32_t* tlo = c->aux2.as<uint32_t>();
            uint32_t* thi = tlo + T;
            int32_t* tcnt = (int32_t*)(thi + T);
            int32_t* toff = tcnt + T + 1;
            const unsigned gt = (unsigned)std::min<int64_t>(ceil_div(T, 256), (int64_t)c->num_sms * 8);
            k_edit_tile_len<<<gt, 256, 0, s>>>(slen, n, T, tlo, thi);
            k_edit_ranges<<<gt, 256, 0, s>>>(tlo, thi, T, K, tcnt);
            c->launches += 2;
            exclusive_scan_i32(c, tcnt, toff, T + 1);
            int32_t npairs = 0;
            RNNG_CUDA(cudaMemcpyAsync(&npairs, toff + T, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
            RNNG_CUDA(cudaStreamSynchronize(s));
            c->pair_list.reserve(sizeof(int2) * (size_t)std::max(npairs, 1));
            k_edit_emit_pairs<<<(unsigned)std::min<int64_t>(T, (int64_t)c->num_sms * 8), 128, 0, s>>>(
                tcnt, toff, T, c->pair_list.as<int2>());
            ++c->launches;
            c->stats.tile_pairs = npairs;
            c->stats.tile_pairs_all = T * (T + 1) / 2;
            c->stats.pairs_evaluated = (int64_t)npairs * kET * kET;
            // 3. filter on the tensor cores: the capped-profile L1 of every string pair of the
            //    tile pairs as a Gram form over thermometer-coded 8-bit rows (k_edit_thermo_q4,
            //    k_edit_thermo)
            c->counters.reserve(sizeof(unsigned long long) * kCounterSlots);
            unsigned long long* ccount = c->counters.as<unsigned long long>() + 2;
            unsigned long long* ecount = c->counters.as<unsigned long long>() + 3;
            unsigned long long got = 0;
            if (npairs > 0) {
                c->xb_sorted.reserve((size_t)n_pad * kFilterBytes);
                c->norms.reserve(sizeof(float4) * (size_t)n_pad + sizeof(float) * (size_t)n_pad +
                                 sizeof(float2) * (size_t)T + 64);
                uint8_t* x8 = c->xb_sorted.as<uint8_t>();
                float4* rowinfo = c->norms.as<float4>();
                float* ucol = (float*)(rowinfo + n_pad);
                float2* tileinfo = (float2*)(((uintptr_t)(ucol + n_pad) + 15) & ~(uintptr_t)15);
                const unsigned gth = (unsigned)std::min<int64_t>(ceil_div(n_pad * 32, 256), (int64_t)c->num_sms * 16);
                if (exact4)
                    k_edit_thermo_q4<<<gth, 256, 0, s>>>(datoms, doff, perm, n, n_pad, symmap, x8, rowinfo, ucol);
                else
                    k_edit_thermo<<<gth, 256, 0, s>>>(prof, n_pad, x8, rowinfo, ucol);
                k_edit_tileinfo<<<gt, 256, 0, s>>>(rowinfo, T, tileinfo);
                c->launches += 2;
                Layout Le;
                Le.n = n;
                Le.n_pad = n_pad;
                Le.T = T;
                Le.d = kFilterBytes;
                Le.pairs = c->pair_list.as<int2>();
                Le.tile_pairs = (unsigned long long)npairs;
                const GramTune t = gram_tune(c, 1, kFilterBytes, npairs);
                Le.gram_chunk = t.chunk;
                Le.gram_slots = t.slots;
                schedule_items(c, Le, 1);
                // thr^2 (as the kernel squares it in FP32) in [2 q K, 2 q K + 1): the integer test
                // L1 <= 2 q K exactly
                const float lim = (float)(2 * qf * K);
                float thr = std::sqrt(lim);
                while (thr * thr < lim) thr = std::nextafter(thr, INFINITY);
                got = run_filter_f8(c, Le, x8, rowinfo, ucol, tileinfo, thr, ccount);
            } else {
                RNNG_CUDA(cudaMemsetAsync(ccount, 0, sizeof(unsigned long long), s));
            }
            const unsigned long long ccap = std::max<unsigned long long>(got, 1ull);
            c->stats.candidates = (int64_t)got;
            // 4. exact verification: Myers' bit-vector algorithm when the alphabet has at most
            //    kBpMaxSym symbols and no string is longer than kBpMaxLen, else the banded DP
            const bool use_bp = got > 0 && maxlen <= (uint32_t)kBpMaxLen && nsym <= kBpMaxSym;
            unsigned long long ecap = std::max<unsigned long long>(1u << 20, c->edge_cap_hint);
            unsigned long long egot = 0;
            const unsigned gv = (unsigned)std::max<unsigned long long>(
                1, std::min<unsigned long long>((got + 255) / 256, (unsigned long long)c->num_sms * 16));
            for (int attempt = 0;; ++attempt) {
                c->edges_u.reserve(sizeof(uint32_t) * ecap);
                c->edges_v.reserve(sizeof(uint32_t) * ecap);
                c->edges_w.reserve(sizeof(float) * ecap);
                RNNG_CUDA(cudaMemsetAsync(ecount, 0, sizeof(unsigned long long), s));
                if (got > 0) {
                    auto* eu = c->edges_u.as<uint32_t>();
                    auto* ev = c->edges_v.as<uint32_t>();
                    auto* ew = c->edges_w.as<float>();
                    if (use_bp)
                        k_edit_verify_bp<<<gv, 256, 0, s>>>(datoms, doff, perm, c->cand.as<uint2>(), ccount, ccap, K,
                                                            (const uint8_t*)(c->sym.as<unsigned int>() + 256), eu, ev,
                                                            ew, ecount, ecap);
                    else if (K <= 4)
                        k_edit_verify<4><<<gv, 256, 0, s>>>(datoms, doff, perm, c->cand.as<uint2>(), ccount, ccap, K,
                                                            eu, ev, ew, ecount, ecap);
                    else if (K <= 8)
                        k_edit_verify<8><<<gv, 256, 0, s>>>(datoms, doff, perm, c->cand.as<uint2>(), ccount, ccap, K,
                                                            eu, ev, ew, ecount, ecap);
                    else if (K <= 16)
                        k_edit_verify<16><<<gv, 256, 0, s>>>(datoms, doff, perm, c->cand.as<uint2>(), ccount, ccap,
                                                             K, eu, ev, ew, ecount, ecap);
                    else
                        k_edit_verify<32><<<gv, 256, 0, s>>>(datoms, doff, perm, c->cand.as<uint2>(), ccount, ccap,
                                                             K, eu, ev, ew, ecount, ecap);
                    ++c->launches;
                    RNNG_CUDA(cudaGetLastError());
                }
                RNNG_CUDA(cudaMemcpyAsync(&egot, ecount, sizeof(egot), cudaMemcpyDeviceToHost, s));
                RNNG_CUDA(cudaStreamSynchronize(s));
                if (egot <= ecap) break;
                RNNG_REQUIRE(attempt < 2, RNNG_ERR_OVERFLOW, "edge buffer overflow after regrowth");
                ecap = egot + egot / 8 + 1024;
            }
            c->edge_cap_hint = std::max<unsigned long long>(c->edge_cap_hint, egot + egot / 8);
            m = (int64_t)egot;
            c->out_u.reserve(sizeof(int64_t) * std::max<int64_t>(m, 1));
            c->out_v.reserve(sizeof(int64_t) * std::max<int64_t>(m, 1));
            c->out_w.reserve(sizeof(float) * std::max<int64_t>(m, 1));
            if (m) {
                k_edit_finalize<<<(unsigned)std::min<int64_t>(ceil_div(m, 256), (int64_t)c->num_sms * 8), 256, 0,
                                  s>>>(c->edges_u.as<uint32_t>(), c->edges_v.as<uint32_t>(), c->edges_w.as<float>(),
                                       m, perm, dids, c->out_u.as<int64_t>(), c->out_v.as<int64_t>(),
                                       c->out_w.as<float>());
                ++c->launches;
                if (flags & RNNG_SORT_OUTPUT)
                    sort_edges_uv(c, c->out_u.as<int64_t>(), c->out_v.as<int64_t>(), c->out_w.as<float>(), m);
            }
        }
        deliver_edges(c, c->out_u.as<int64_t>(), c->out_v.as<int64_t>(), c->out_w.as<float>(), m, flags, out);
        RNNG_CUDA(cudaStreamSynchronize(s));
        c->stats.edges = m;
        c->stats.kernel_launches = c->launches;
        c->stats.ms_gram = c->gram_ms;  // the tensor-core filter
    });
}

extern "C" int rnng_voronoi_edit(rnng_ctx* c, const uint8_t* atoms, const int64_t* offsets, int64_t n,
                                 const uint8_t* catoms, const int64_t* coffsets, int64_t m, unsigned flags,
                                 int64_t* cell, float* dist)
{
    return guarded(c, [&] {
        RNNG_REQUIRE(n >= 0 && m >= 1, RNNG_ERR_INVALID, "bad sizes (need at least one centre)");
        RNNG_REQUIRE((n == 0 || (atoms && offsets && cell && dist)) && catoms && coffsets, RNNG_ERR_INVALID,
                     "null pointer");
        c->stats = rnng_stats{};
        c->launches = 0;
        if (n == 0) return;
        cudaStream_t s = c->stream;
        const bool dev_in = flags & RNNG_INPUT_DEVICE;
        const int64_t natoms = dev_in ? 0 : offsets[n], ncatoms = dev_in ? 0 : coffsets[m];
        const int64_t* doff = (const int64_t*)upload(c, c->ids_in, offsets, sizeof(int64_t) * (n + 1), flags);
        const uint8_t* datoms = (const uint8_t*)upload(c, c->x_in, atoms, (size_t)natoms, flags);
        const int64_t* dcoff = (const int64_t*)upload(c, c->aux7, coffsets, sizeof(int64_t) * (m + 1), flags);
        const uint8_t* dcatoms = (const uint8_t*)upload(c, c->pivots, catoms, (size_t)ncatoms, flags);
        // longest centre: sizes the shared match vectors and picks the register variant
        c->counters.reserve(sizeof(unsigned long long) * kCounterSlots);
        unsigned long long* dmax = c->counters.as<unsigned long long>() + 9;
        RNNG_CUDA(cudaMemsetAsync(dmax, 0, sizeof(unsigned long long), s));
        k_max_len<<<(unsigned)std::min<int64_t>(ceil_div(m, 256), (int64_t)c->num_sms * 4), 256, 0, s>>>(dcoff, m,
                                                                                                          dmax);
        ++c->launches;
        unsigned long long maxlen = 0;
        RNNG_CUDA(cudaMemcpyAsync(&maxlen, dmax, sizeof(maxlen), cudaMemcpyDeviceToHost, s));
        RNNG_CUDA(cudaStreamSynchronize(s));
        const int Wmax = (int)((maxlen + 63) / 64);
        RNNG_REQUIRE(Wmax <= kVEMaxW, RNNG_ERR_UNSUPPORTED, "centres longer than 4096 characters");
        int64_t* dcell = cell;
        float* ddist = dist;
        if (!(flags & RNNG_OUTPUT_DEVICE)) {
            c->out_u.reserve(sizeof(int64_t) * n);
            c->out_w.reserve(sizeof(float) * n);
            dcell = c->out_u.as<int64_t>();
            ddist = c->out_w.as<float>();
        }
        const size_t smem = sizeof(unsigned long long) * 256 * (size_t)std::max(Wmax, 1);
        const unsigned grid = (unsigned)ceil_div(n, kVE);
        if (Wmax <= 1) {
            k_voronoi_edit<1><<<grid, kVE, smem, s>>>(datoms, doff, n, dcatoms, dcoff, m, dcell, ddist);
        } else if (Wmax <= 2) {
            k_voronoi_edit<2><<<grid, kVE, smem, s>>>(datoms, doff, n, dcatoms, dcoff, m, dcell, ddist);
        } else if (Wmax <= 4) {
            k_voronoi_edit<4><<<grid, kVE, smem, s>>>(datoms, doff, n, dcatoms, dcoff, m, dcell, ddist);
        } else {
            if (smem > 48 * 1024)
                RNNG_CUDA(cudaFuncSetAttribute(k_voronoi_edit<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem));
            k_voronoi_edit<0><<<grid, kVE, smem, s>>>(datoms, doff, n, dcatoms, dcoff, m, dcell, ddist);
        }
        ++c->launches;
        RNNG_CUDA(cudaGetLastError());
        if (!(flags & RNNG_OUTPUT_DEVICE)) {
            RNNG_CUDA(cudaMemcpyAsync(cell, dcell, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, s));
            RNNG_CUDA(cudaMemcpyAsync(dist, ddist, sizeof(float) * n, cudaMemcpyDeviceToHost, s));
        }
        RNNG_CUDA(cudaStreamSynchronize(s));
        c->stats.kernel_launches = c->launches;
    });
}
