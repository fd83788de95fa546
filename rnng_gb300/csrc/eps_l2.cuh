// Internal interfaces of the L2 epsilon-graph pipeline (see eps_l2.cu).
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "common.cuh"

namespace rnng {

constexpr int kTile = 128;          // points per tile (one tcgen05 M=128 / N=128 operand)
constexpr int kSuper = 8;           // tiles per super-tile in the first pruning level
constexpr int kTileBalls = 8;       // balls covering one tile
constexpr int kSuperBalls = 16;     // balls covering one super-tile
constexpr int kFan = 64;            // children per split of the landmark partition
constexpr int64_t kLeafTarget = 128;  // points per leaf cell
// Depth limit of the partition.  Cells that a level leaves above 2 kLeafTarget points
// stay as they are, their points in the order of distance to their landmark: at 1M x 128
// each level past the fourth cost about 0.25 ms and changed the tile pairs by a few
// percent (8 levels: 1.059M pairs, 11.05 ms per graph; 4 levels: 1.088M, 10.25 ms).
constexpr int kMaxLevels = 4;
constexpr int kBf16MinDim = 16;     // BF16 mode evaluates tiles of fewer dimensions with FP32-direct tiles

// Device layout of one epsilon-graph problem after the partition.
struct Layout {
    int64_t n = 0, n_pad = 0, T = 0, S = 0;
    int d = 0, m1 = 0;
    int64_t num_cells = 0;
    float radius = 0.f, relerr = 0.f;
    float* Xs = nullptr;          // n_pad x d, sorted by leaf cell, zero padded
    const float* shift = nullptr;  // per-dimension shift of the BF16 operands (rounded column means)
    int32_t* perm = nullptr;      // sorted position -> input row
    unsigned long long super_pairs = 0, tile_pairs = 0;
    int2* pairs = nullptr;        // surviving tile pairs (i <= j)
    unsigned long long* d_tile_pairs = nullptr;  // device copy of tile_pairs
    // BF16 Gram items: a row tile x with item_tiles column tiles {y, z} (z = -1: none), or
    // with item_tiles = 3 the row tiles {x, z} = {2 r, 2 r + 1} against column tile y (w: which
    // of the two tile pairs survived), in (row, column) order; the kernel's queue hands them
    // out gram_chunk at a time, with at most gram_slots B slots per CTA (0: as many as fit)
    int4* items = nullptr;
    unsigned long long num_items = 0;
    int item_tiles = 1;
    int gram_chunk = 64;
    int gram_slots = 0;
    float* gram_raw = nullptr;  // diagnostic: the Gram kernel writes its raw accumulators here (n_pad x n_pad)
    // build_layout stopped before the partition: the screen found a non-finite input value
    bool nonfinite = false;
    float maxabs = 0.f;  // largest |coordinate| (d <= 256 only)
};

// Edge buffer in sorted-index space.
struct EdgeOut {
    uint32_t* si = nullptr;
    uint32_t* sj = nullptr;
    float* w = nullptr;
    unsigned long long* count = nullptr;  // device counter
    unsigned long long cap = 0;
    // Direct output (BF16 tiles, host results, no sorting): the recheck writes each edge as
    // (input id u < v, weight) straight into the context's pinned staging block through its
    // device address, so the results cross to the host while the recheck runs.  `direct`
    // is the request; run_tiles_bf16 clears it when it cannot honour it, else sets the host
    // arrays (room for every candidate) and cap.
    bool direct = false;
    const int32_t* perm = nullptr;  // sorted position -> input row
    const int64_t* ids = nullptr;   // input row -> id (nullptr: the row itself)
    int64_t* hu = nullptr;
    int64_t* hv = nullptr;
    float* hw = nullptr;
};

// Where the recheck puts an edge: its sorted positions into the pipeline's edge list, or,
// with du set, the final (input id u < v, weight) through perm and ids.
struct EdgeSink {
    uint32_t* eu = nullptr;
    uint32_t* ev = nullptr;
    float* ew = nullptr;
    int64_t* du = nullptr;
    int64_t* dv = nullptr;
    float* dw = nullptr;
    const int32_t* perm = nullptr;
    const int64_t* ids = nullptr;
    __device__ __forceinline__ void put(unsigned long long pos, uint32_t i, uint32_t j, float w) const
    {
        if (du) {
            const int32_t a = perm[i], b = perm[j];
            const int64_t ia = ids ? ids[a] : (int64_t)a, ib = ids ? ids[b] : (int64_t)b;
            du[pos] = ia < ib ? ia : ib;
            dv[pos] = ia < ib ? ib : ia;
            dw[pos] = w;
        } else {
            eu[pos] = i;
            ev[pos] = j;
            ew[pos] = w;
        }
    }
};

// screen: first test the input for NaN or infinite values (fused into the BF16 column
// sums for d <= 256) and, if there is one, return at once with L.nonfinite set.  For
// d <= 256 L.maxabs is set either way.
Layout build_layout(rnng_ctx* c, const float* dX, int64_t n, int d, float radius, bool screen);
// Rows of dX (n x d) without a NaN or infinite coordinate, copied in order to a context
// buffer (*out; dX itself when every row is finite); returns their number.  The map
// from compacted rows to input rows stays in the context for remap_rows.  *inf_rows:
// some row has an infinite coordinate and no NaN.
int64_t compact_finite_rows(rnng_ctx* c, const float* dX, int64_t n, int d, const float** out, bool* inf_rows);
// perm[0..n) := map[perm[k]] with the map of the last compact_finite_rows (n_in: the
// row count that call was given).
void remap_rows(rnng_ctx* c, int32_t* perm, int64_t n, int64_t n_in);
// The radius the covers and the BF16 candidate test use: radius (1 + (d + 8) 2^-24) +
// 1e-30 rounded up to a float, which bounds the FP32 rounding of RNNG's sequential L2.
// Capped at FLT_MAX: an infinite (or huge) radius then still makes every squared
// threshold +inf, without the NaN of inf x 0 where a tile's error radius is 0.
float widened_radius(float radius, int d);
void run_tiles_fp32(rnng_ctx* c, Layout& L, EdgeOut& E);
void finalize_edges(rnng_ctx* c, const Layout& L, const int64_t* d_ids, const EdgeOut& E, int64_t m, int64_t* u,
                    int64_t* v, float* w);
// Stable sort of (key, value) pairs by key bits [begin_bit, end_bit).
void sort_pairs_u64(rnng_ctx* c, uint64_t* keys_in, uint64_t* keys_out, int32_t* vals_in, int32_t* vals_out,
                    int64_t n, int end_bit, int begin_bit = 0);
// out[0..count-1] = exclusive prefix sum of in[0..count-2] (in[count-1] is zeroed first).
void exclusive_scan_i32(rnng_ctx* c, const int32_t* in, int32_t* out, int64_t count);

// The whole L2 pipeline on device points (api.cu); edges in sorted-index space in E.
int64_t eps_core(rnng_ctx* c, const float* dX, int64_t n, int d, float radius, int mode, Layout& L, EdgeOut& E);

// BF16 tensor-core Gram tiles with FP32 recheck (gram_bf16.cu).
void prepare_bf16(rnng_ctx* c, Layout& L);
// Relative bound gamma of the Gram error terms q = gamma ||x~||^2 for dimension d.
double bf16_gamma(int d);
// The BF16 shift of this layout: the rounded column means of the L.n points X (by
// default L.Xs; the input rows give the same sums), computed once per call (L.shift).
// screen (optional, two device words): [0] = 1 if a value of X is NaN or infinite, else 0;
// [1] = the float bits of the largest |value|.
const float* bf16_shift(rnng_ctx* c, Layout& L, const float* X = nullptr, unsigned long long* screen = nullptr);
// Whether the BF16 candidate test's squared terms stay in FP32's normal range for this
// layout (its maxabs, d and radius); otherwise the FP32-direct tiles take the pairs.
bool bf16_in_range(const Layout& L);
// Ball centres (nb rows of L.d floats, radii rad; rows nb .. nb_pad - 1 padding) as BF16
// rows of dp = 64 * ceil(d / 64) with {norm, a, q, radius or -1} per row (bf16_row).
// Returns the mean relative widening of a ball pair's squared threshold by a and q.
float prepare_ball_bf16(rnng_ctx* c, Layout& L, const float* cen, const float* rad, int64_t nb, int64_t nb_pad,
                        float eps_p, __nv_bfloat16* out, float4* info);
void run_tiles_bf16(rnng_ctx* c, Layout& L, EdgeOut& E);
bool bf16_supported(int d);
// Tuning of the Gram kernel for operands of padded width dp (kind 0: BF16 L2 tiles, 1: the
// FP8 edit filter) over tile_pairs tile pairs: the context's forced values, else the
// tuning table's row, else the defaults (nt 2 up to dp 128, chunks of 64 items, as many B
// slots as fit); nt and chunk are adjusted to the compiled kernel forms.
GramTune gram_tune(rnng_ctx* c, int kind, int dp, int64_t tile_pairs);
// The tuning table read when a context is created (a missing file leaves it empty).
void load_gram_table(rnng_ctx* c);

// Filter rows of 0/1 values as E4M3 bytes (0x00 / 0x38), kFilterBytes per row, n_pad rows in
// the tile order of L: candidate pairs (i < j) of L's scheduled items whose
// n_i + n_j - 2 x_i.x_j <= thr_sqrt^2 (rowinfo[i] = {n_i, 0, 0, n_i}, ucol = n, tileinfo
// = {0, max n of the tile}; integer-exact) by the tensor-core kernel on 8-bit operands.
// Candidates in c->cand, their count in *cnt (returned).
constexpr int kFilterBytes = 512;
unsigned long long run_filter_f8(rnng_ctx* c, const Layout& L, const uint8_t* x8, const float4* rowinfo,
                                 const float* ucol, const float2* tileinfo, float thr_sqrt, unsigned long long* cnt);

}  // namespace rnng
