// Vietoris-Rips filtrations: rnng_rips_l2 (points under L2) and rnng_rips_edges (any
// given graph, e.g. an edit-distance epsilon graph) (include/rnng_gpu.h).
//
// Replaces, on one GPU, RNNG's per-cell VoronoiComplex::build_filtration and the final
// merge (include/point.hpp:1136-1267, include/simplex.hpp:130-196).  RNNG builds each
// cell's complex over cell points plus ghosts and unions the cells; the union is the
// Rips complex of the whole point set, which is built here directly:
//   1. the epsilon graph of all points (the L2 pipeline, exact reference distances);
//   2. vertices are ranked by id, every edge is stored once as (a < b) in rank space and
//      sorted, giving a CSR of higher-ranked neighbours;
//   3. triangles a < b < c are found once each by intersecting, for every edge (a, b),
//      the neighbours of a after b with the neighbours of b (both lists sorted);
//   4. values: vertex 0, edge = its reference distance, triangle = the largest of its
//      three edges (RNNG's max over facet values, include/point.hpp:1194-1208);
//   5. ids: sum over the sorted vertex ids v_i of C(v_i, i + 1), OR-ed with dim << 60
//      (include/simplex.hpp:5-19), binomials as RNNG's Binom forms them
//      (include/utils.hpp:116-144): a falling product in 64-bit integers divided by k!;
//   6. cliques of 4 and more vertices (maxdim >= 3) grow level by level: a clique
//      a < ... < x gains every higher neighbour y of x that is a neighbour of all its
//      other vertices (binary searches in their sorted rows); its value is the largest
//      of its edges, which equals RNNG's recursive max over facets;
//   7. all simplices sorted by (value, id).  Each simplex is built exactly once, so the
//      merge's unique-by-id step (include/simplex.hpp:173-174) has nothing to remove.
// Up to triangles over distinct ids small enough that RNNG's binomials are exact, the
// ids are the combinatorial number system, so colex order of vertex tuples is id order:
// edges are then keyed (larger, smaller), triangles found per edge (b, c) among the
// lower neighbours of c below b and of b, in (c, b, a) order, and steps 2-3 emit every
// simplex already in id order; step 7 is one stable 32-bit pass by value.
#include <cub/cub.cuh>

#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "eps_l2.cuh"
#include "kernels_misc.cuh"

namespace rnng {

constexpr int kRipsMaxDim = 15;  // simplex ids keep the dimension in 4 bits

__device__ __forceinline__ int64_t ref_binom(int64_t n, int64_t k)
{
    if (k > n) return 0;
    uint64_t a = 1, b = 1;
    for (int64_t i = n; i >= n - k + 1; --i) a *= (uint64_t)i;
    for (int64_t i = k; i >= 1; --i) b *= (uint64_t)i;
    return (int64_t)a / (int64_t)b;
}

__device__ __forceinline__ int64_t simplex_id1(int64_t a) { return (int64_t)((uint64_t)ref_binom(a, 1)); }
__device__ __forceinline__ int64_t simplex_id2(int64_t a, int64_t b)
{
    const uint64_t uid = (uint64_t)ref_binom(b, 2) + (uint64_t)ref_binom(a, 1);
    return (int64_t)(uid | (1ull << 60));
}
__device__ __forceinline__ int64_t simplex_id3(int64_t a, int64_t b, int64_t c)
{
    const uint64_t uid = (uint64_t)ref_binom(c, 3) + (uint64_t)ref_binom(b, 2) + (uint64_t)ref_binom(a, 1);
    return (int64_t)(uid | (2ull << 60));
}

__global__ void k_rank_iota(int64_t* __restrict__ keys, int32_t* __restrict__ rows, const int64_t* __restrict__ ids,
                            int64_t n)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        keys[i] = ids ? ids[i] : i;
        rows[i] = (int32_t)i;
    }
}

__global__ void k_rank_of_row(const int32_t* __restrict__ row_of_rank, int64_t n, int32_t* __restrict__ rank)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x)
        rank[row_of_rank[r]] = (int32_t)r;
}

// Sorted-index edges -> rank-space keys (a << 32 | b), a < b, with their weights.
__global__ void k_edge_keys(const uint32_t* __restrict__ si, const uint32_t* __restrict__ sj,
                            const float* __restrict__ sw, int64_t m, const int32_t* __restrict__ perm,
                            const int32_t* __restrict__ rank, uint64_t* __restrict__ key, float* __restrict__ w)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t a = (uint32_t)rank[perm[si[e]]], b = (uint32_t)rank[perm[sj[e]]];
        key[e] = a < b ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
        w[e] = sw[e];
    }
}

__global__ void k_degree(const uint64_t* __restrict__ key, int64_t m, int32_t* __restrict__ deg)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&deg[key[e] >> 32], 1);
}

// For edge e = (a, b): the neighbours of a after b (CSR positions e+1 .. end of row a)
// intersected with the neighbours of b.  Counts (emit == false) or writes triangles.
template <bool emit>
__global__ void k_triangles(const uint64_t* __restrict__ key, const float* __restrict__ w,
                            const int32_t* __restrict__ row, int64_t m, const int64_t* __restrict__ id_of_rank,
                            int64_t* __restrict__ cnt, const int64_t* __restrict__ off, int64_t* __restrict__ out_id,
                            float* __restrict__ out_val, int32_t* __restrict__ out_clq,
                            const uint8_t* __restrict__ fr, uint8_t* __restrict__ out_flag)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t a = (uint32_t)(key[e] >> 32), b = (uint32_t)(key[e] & 0xffffffffu);
        int64_t x = e + 1;
        const int64_t xe = row[a + 1];
        int64_t y = row[b];
        const int64_t ye = row[b + 1];
        const float wab = w[e];
        int64_t pos = emit ? off[e] : 0;
        int64_t found = 0;
        while (x < xe && y < ye) {
            const uint32_t cx = (uint32_t)(key[x] & 0xffffffffu), cy = (uint32_t)(key[y] & 0xffffffffu);
            if (cx < cy) {
                ++x;
            } else if (cx > cy) {
                ++y;
            } else {
                if (emit) {
                    const float v = fmaxf(fmaxf(wab, w[x]), w[y]);
                    const int64_t ia = id_of_rank[a], ib = id_of_rank[b], ic = id_of_rank[cx];
                    out_id[pos] = simplex_id3(ia, ib, ic);
                    out_val[pos] = v;
                    if (out_flag) out_flag[pos] = fr[a] | fr[b] | fr[cx];
                    if (out_clq) {
                        out_clq[3 * pos] = (int32_t)a;
                        out_clq[3 * pos + 1] = (int32_t)b;
                        out_clq[3 * pos + 2] = (int32_t)cx;
                    }
                    ++pos;
                }
                ++found;
                ++x;
                ++y;
            }
        }
        if (!emit) cnt[e] = found;
    }
}

__global__ void k_vertices_edges(const int64_t* __restrict__ id_of_rank, int64_t n, const uint64_t* __restrict__ key,
                                 const float* __restrict__ w, int64_t m, bool with_edges, bool colex,
                                 int64_t* __restrict__ out_id, float* __restrict__ out_val,
                                 const uint8_t* __restrict__ fr, uint8_t* __restrict__ out_flag)
{
    const int64_t total = n + (with_edges ? m : 0);
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        if (t < n) {
            out_id[t] = simplex_id1(id_of_rank[t]);
            out_val[t] = 0.f;
            if (out_flag) out_flag[t] = fr[t];
        } else {
            const int64_t e = t - n;
            const uint32_t hi = (uint32_t)(key[e] >> 32), lo = (uint32_t)(key[e] & 0xffffffffu);
            const uint32_t a = colex ? lo : hi, b = colex ? hi : lo;  // a < b
            out_id[t] = simplex_id2(id_of_rank[a], id_of_rank[b]);
            out_val[t] = w[e];
            if (out_flag) out_flag[t] = fr[a] | fr[b];
        }
    }
}

// (a << 32 | b) -> (b << 32 | a): edge keys by (larger rank, smaller rank).
__global__ void k_swap_key_halves(uint64_t* __restrict__ key, int64_t m)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = key[e];
        key[e] = (k << 32) | (k >> 32);
    }
}

// Triangles in colex order (c, b, a), for keys sorted by (c, b) with c > b and a CSR of
// lower neighbours: for edge e = (b < c) the lower neighbours of c before b (CSR
// positions row[c] .. e - 1) intersected with the lower neighbours of b.  Edges in key
// order and a ascending give the triangles sorted by their ids whenever RNNG's binomials
// do not wrap.  Counts (emit == false) or writes ids, values (largest edge) and flags.
template <bool emit>
__global__ void k_triangles_colex(const uint64_t* __restrict__ key, const float* __restrict__ w,
                                  const int32_t* __restrict__ row, int64_t m, const int64_t* __restrict__ id_of_rank,
                                  int64_t* __restrict__ cnt, const int64_t* __restrict__ off,
                                  int64_t* __restrict__ out_id, float* __restrict__ out_val,
                                  const uint8_t* __restrict__ fr, uint8_t* __restrict__ out_flag)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t c = (uint32_t)(key[e] >> 32), b = (uint32_t)(key[e] & 0xffffffffu);
        int64_t x = row[c];
        const int64_t xe = e;
        int64_t y = row[b];
        const int64_t ye = row[b + 1];
        const float wbc = w[e];
        int64_t pos = emit ? off[e] : 0;
        int64_t found = 0;
        while (x < xe && y < ye) {
            const uint32_t ax = (uint32_t)(key[x] & 0xffffffffu), ay = (uint32_t)(key[y] & 0xffffffffu);
            if (ax < ay) {
                ++x;
            } else if (ax > ay) {
                ++y;
            } else {
                if (emit) {
                    out_id[pos] = simplex_id3(id_of_rank[ax], id_of_rank[b], id_of_rank[c]);
                    out_val[pos] = fmaxf(fmaxf(wbc, w[x]), w[y]);
                    if (out_flag) out_flag[pos] = fr[ax] | fr[b] | fr[c];
                    ++pos;
                }
                ++found;
                ++x;
                ++y;
            }
        }
        if (!emit) cnt[e] = found;
    }
}

// Vertex flags by rank: fr[rank[row]] = flag[row] != 0.
__global__ void k_flag_by_rank(const uint8_t* __restrict__ flag, const int32_t* __restrict__ rank, int64_t n,
                               uint8_t* __restrict__ fr)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        fr[rank[i]] = flag[i] ? 1 : 0;
}

// Sets *bad unless the ranked ids are strictly increasing and within [0, max_id].
__global__ void k_ids_colex(const int64_t* __restrict__ id_of_rank, int64_t n, int64_t max_id,
                            unsigned int* __restrict__ bad)
{
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t id = id_of_rank[r];
        if (id < 0 || id > max_id || (r > 0 && id <= id_of_rank[r - 1])) atomicOr(bad, 1u);
    }
}

__global__ void k_value_bits(const float* __restrict__ v, int64_t m, uint32_t* __restrict__ bits,
                             int32_t* __restrict__ idx)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x) {
        bits[i] = __float_as_uint(v[i]);  // values are >= +0, so bit order is numeric order
        idx[i] = (int32_t)i;
    }
}

template <class T>
__global__ void k_permute(const T* __restrict__ src, const int32_t* __restrict__ idx, int64_t m, T* __restrict__ dst)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[idx[i]];
}

// Cliques of k ranks (ascending) -> cliques of k + 1: for clique i with last vertex x,
// every y in N+(x) that is in N+(v) for all other vertices v.  Counts (emit == false)
// or writes id, value (largest edge) and, when out_clq is set, the k + 1 ranks.
template <bool emit>
__global__ void k_extend(const int32_t* __restrict__ clq, const float* __restrict__ val, int64_t nc, int k,
                         const uint64_t* __restrict__ key, const float* __restrict__ w,
                         const int32_t* __restrict__ row, const int64_t* __restrict__ id_of_rank,
                         int64_t* __restrict__ cnt, const int64_t* __restrict__ off, int64_t* __restrict__ out_id,
                         float* __restrict__ out_val, int32_t* __restrict__ out_clq, const uint8_t* __restrict__ fr,
                         uint8_t* __restrict__ out_flag)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nc; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t* cv = clq + i * k;
        const int32_t x = cv[k - 1];
        const float base = val[i];
        int64_t pos = emit ? off[i] : 0;
        int64_t found = 0;
        for (int64_t e = row[x]; e < row[x + 1]; ++e) {
            const uint32_t y = (uint32_t)(key[e] & 0xffffffffu);
            float v = fmaxf(base, w[e]);
            bool ok = true;
            for (int j = 0; j < k - 1 && ok; ++j) {
                const int32_t a = cv[j];
                int64_t lo = row[a], hi = row[a + 1];
                while (lo < hi) {  // first entry of row a that is >= y
                    const int64_t mid = lo + ((hi - lo) >> 1);
                    if ((uint32_t)(key[mid] & 0xffffffffu) < y) lo = mid + 1;
                    else hi = mid;
                }
                if (lo < row[a + 1] && (uint32_t)(key[lo] & 0xffffffffu) == y) v = fmaxf(v, w[lo]);
                else ok = false;
            }
            if (!ok) continue;
            if (emit) {
                uint64_t uid = (uint64_t)ref_binom(id_of_rank[y], k + 1);
                for (int j = 0; j < k; ++j) uid += (uint64_t)ref_binom(id_of_rank[cv[j]], j + 1);
                out_id[pos] = (int64_t)(uid | ((uint64_t)k << 60));
                out_val[pos] = v;
                if (out_flag) {
                    uint8_t f = fr[y];
                    for (int j = 0; j < k; ++j) f |= fr[cv[j]];
                    out_flag[pos] = f;
                }
                if (out_clq) {
                    for (int j = 0; j < k; ++j) out_clq[pos * (k + 1) + j] = cv[j];
                    out_clq[pos * (k + 1) + k] = (int32_t)y;
                }
                ++pos;
            }
            ++found;
        }
        if (!emit) cnt[i] = found;
    }
}

// Caller's edges (rows u, v, value w) -> rank-space keys; flags rows out of range,
// self-loops and values that are negative or NaN.  -0 becomes +0.
__global__ void k_row_edge_keys(const int64_t* __restrict__ u, const int64_t* __restrict__ v,
                                const float* __restrict__ sw, int64_t m, int64_t n, const int32_t* __restrict__ rank,
                                uint64_t* __restrict__ key, float* __restrict__ w, unsigned int* __restrict__ bad)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ru = u[e], rv = v[e];
        const float x = sw[e];
        if (ru < 0 || ru >= n || rv < 0 || rv >= n || ru == rv || !(x >= 0.f)) {
            atomicOr(bad, 1u);
            key[e] = 0;
            w[e] = 0.f;
            continue;
        }
        const uint32_t a = (uint32_t)rank[ru], b = (uint32_t)rank[rv];
        key[e] = a < b ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
        w[e] = x + 0.f;
    }
}

// Sorted keys: flags an unordered pair given twice.
__global__ void k_dup_keys(const uint64_t* __restrict__ key, int64_t m, unsigned int* __restrict__ bad)
{
    for (int64_t e = 1 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x)
        if (key[e] == key[e - 1]) atomicOr(bad, 2u);
}

}  // namespace rnng

using namespace rnng;

namespace {

// Grows b to `want` bytes keeping its first `used` bytes.
void grow_keep(rnng_ctx* c, DevBuf& b, size_t want, size_t used)
{
    if (want <= b.bytes) return;
    void* p = nullptr;
    const size_t grow = want + want / 4 + 256;
    RNNG_CUDA(cudaMalloc(&p, grow));
    if (used) RNNG_CUDA(cudaMemcpyAsync(p, b.ptr, used, cudaMemcpyDeviceToDevice, c->stream));
    RNNG_CUDA(cudaStreamSynchronize(c->stream));
    if (b.ptr) cudaFree(b.ptr);
    b.ptr = p;
    b.bytes = grow;
}

unsigned grid_for(rnng_ctx* c, int64_t work)
{
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(std::max<int64_t>(work, 1), 256),
                                                            (int64_t)c->num_sms * 8));
}

struct Ranks {
    int64_t* id_of_rank;  // id of the vertex of rank r
    int32_t* rank;        // rank of row i
    bool rows_are_ids;    // no ids given: the id of row i is i
};

// Vertices ranked by id (rows themselves without ids): rank order is id order, so
// sorted rank tuples are sorted id tuples.
Ranks rank_vertices(rnng_ctx* c, const int64_t* dids, int64_t n)
{
    cudaStream_t s = c->stream;
    const int64_t ng = std::max<int64_t>(n, 1);
    c->aux0.reserve(sizeof(int64_t) * 2 * (size_t)ng);
    c->aux1.reserve(sizeof(int32_t) * 3 * (size_t)ng + 16);
    int64_t* idk = c->aux0.as<int64_t>();
    Ranks R{idk + ng, nullptr, dids == nullptr};
    int32_t* rows = c->aux1.as<int32_t>();
    int32_t* row_of_rank = rows + ng;
    R.rank = row_of_rank + ng;
    if (n == 0) return R;
    k_rank_iota<<<grid_for(c, n), 256, 0, s>>>(idk, rows, dids, n);
    ++c->launches;
    if (dids && n > 1) {
        size_t tmp = 0;
        RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, idk, R.id_of_rank, rows, row_of_rank, (int)n, 0, 64, s));
        c->cub_tmp.reserve(tmp);
        RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, idk, R.id_of_rank, rows, row_of_rank, (int)n, 0,
                                                  64, s));
        c->launches += cub_sort_kernels(n, 64);
    } else {
        RNNG_CUDA(cudaMemcpyAsync(R.id_of_rank, idk, sizeof(int64_t) * n, cudaMemcpyDeviceToDevice, s));
        RNNG_CUDA(cudaMemcpyAsync(row_of_rank, rows, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
    }
    k_rank_of_row<<<grid_for(c, n), 256, 0, s>>>(row_of_rank, n, R.rank);
    ++c->launches;
    return R;
}

struct Keys {
    uint64_t* k0;  // unsorted rank-space keys (a << 32 | b, a < b), filled by the caller
    uint64_t* k1;  // sorted
    float* w0;
    float* w1;
};

Keys key_buffers(rnng_ctx* c, int64_t m)
{
    const int64_t mg = std::max<int64_t>(m, 1);
    c->aux2.reserve(sizeof(uint64_t) * 2 * (size_t)mg + sizeof(float) * 2 * (size_t)mg + 32);
    Keys K;
    K.k0 = c->aux2.as<uint64_t>();
    K.k1 = K.k0 + mg;
    K.w0 = (float*)(K.k1 + mg);
    K.w1 = K.w0 + mg;
    return K;
}

unsigned int read_flag(rnng_ctx* c, unsigned int* dflag)
{
    unsigned int h = 0;
    RNNG_CUDA(cudaMemcpyAsync(&h, dflag, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
    RNNG_CUDA(cudaStreamSynchronize(c->stream));
    return h;
}

// int64 exclusive sum of cnt[0..count) into off[0..count]; returns off[count].
int64_t scan_counts(rnng_ctx* c, int64_t* cnt, int64_t* off, int64_t count)
{
    cudaStream_t s = c->stream;
    RNNG_CUDA(cudaMemsetAsync(cnt + count, 0, sizeof(int64_t), s));
    size_t tmp = 0;
    RNNG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp, cnt, off, (int)(count + 1), s));
    c->cub_tmp.reserve(tmp);
    RNNG_CUDA(cub::DeviceScan::ExclusiveSum(c->cub_tmp.ptr, tmp, cnt, off, (int)(count + 1), s));
    c->launches += 2;
    int64_t total = 0;
    RNNG_CUDA(cudaMemcpyAsync(&total, off + count, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    RNNG_CUDA(cudaStreamSynchronize(s));
    return total;
}

// True when, for vertex ids in [0, max_id], RNNG's Binom (a 64-bit falling product,
// include/utils.hpp:116-144) is exact for every binomial of a simplex id up to maxdim
// (<= 2) and every id of dimension k stays below the dimension bits (below 2^60).  The
// ids are then the combinatorial number system: colex order of vertex tuples is id
// order within a dimension, and dimension k sorts before k + 1.
bool colex_ids_exact(int64_t max_id, int maxdim)
{
    if (max_id < 0) return true;
    if (max_id >= (int64_t(1) << 40)) return false;  // keeps the products below in 128 bits
    using u128 = unsigned __int128;
    const u128 M = (u128)max_id;
    for (int k = 1; k <= maxdim + 1; ++k) {
        u128 fall = 1, top = 1, fact = 1;  // M (M-1) ... (M-k+1); (M+1) M ... (M-k+2); k!
        for (int i = 0; i < k; ++i) {
            fall *= (M >= (u128)i) ? M - i : 0;
            top *= M + 1 - i;
            fact *= (u128)(i + 1);
        }
        if (fall >= ((u128)1 << 63)) return false;       // Binom's signed division stays exact
        if (top / fact > ((u128)1 << 60)) return false;  // largest id of dimension k-1 is C(M+1, k) - 1
    }
    return true;
}

// Largest vertex id for which colex_ids_exact(., maxdim) holds.
int64_t colex_max_id(int maxdim)
{
    int64_t lo = 0, hi = int64_t(1) << 40;
    while (lo < hi) {
        const int64_t mid = lo + (hi - lo + 1) / 2;
        if (colex_ids_exact(mid, maxdim)) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Whether the simplices can be generated directly in id order (maxdim <= 2, distinct
// ids within colex_max_id).  Without ids the rows 0..n-1 are the ids.
bool colex_order(rnng_ctx* c, const Ranks& R, int64_t n, int maxdim)
{
    if (maxdim > 2) return false;
    const int64_t bound = colex_max_id(maxdim);
    if (n == 0) return true;
    if (R.rows_are_ids) return n - 1 <= bound;
    unsigned int* bad = (unsigned int*)(c->counters.as<unsigned long long>() + 11);
    RNNG_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned int), c->stream));
    k_ids_colex<<<grid_for(c, n), 256, 0, c->stream>>>(R.id_of_rank, n, bound, bad);
    ++c->launches;
    return read_flag(c, bad) == 0;
}

constexpr int64_t kMaxSimplices = (int64_t(1) << 31) - 1;

// The filtration of the graph given by m unsorted rank-space keys (K.k0, K.w0) over n
// vertices, up to maxdim, sorted by (value, id) and delivered to out.  With
// check_pairs, a pair given twice is an error.  dvflag (per row, may be null) gives
// each simplex the OR of its vertices' flags.
void rips_from_keys(rnng_ctx* c, int64_t n, const Ranks& R, const Keys& K, int64_t m, int maxdim, unsigned flags,
                    bool check_pairs, const uint8_t* dvflag, rnng_simplices* out)
{
    cudaStream_t s = c->stream;
    RNNG_REQUIRE(n < (int64_t(1) << 31) && m < (int64_t(1) << 31), RNNG_ERR_INVALID, "graph too large for one call");
    const int64_t ng = std::max<int64_t>(n, 1), mg = std::max<int64_t>(m, 1);
    const bool with_flags = dvflag != nullptr;
    uint8_t* fr = nullptr;  // vertex flags by rank
    if (with_flags) {
        c->vflag.reserve((size_t)ng);
        fr = c->vflag.as<uint8_t>();
        if (n) {
            k_flag_by_rank<<<grid_for(c, n), 256, 0, s>>>(dvflag, R.rank, n, fr);
            ++c->launches;
        }
    }
    // Up to triangles over small distinct ids, simplices are generated in id order:
    // edges keyed (larger, smaller) and sorted, a CSR of lower neighbours, triangles per
    // edge in colex order.  Otherwise (higher cliques, large or repeated ids) keys are
    // (smaller, larger) with a CSR of higher neighbours, and the ids are sorted.
    const bool colex = colex_order(c, R, n, maxdim);
    if (colex && m > 0) {
        k_swap_key_halves<<<grid_for(c, m), 256, 0, s>>>(K.k0, m);
        ++c->launches;
    }
    // ---- sorted keys and the CSR of neighbours
    c->aux3.reserve(sizeof(int32_t) * 2 * ((size_t)ng + 1) + sizeof(int64_t) * 2 * ((size_t)mg + 1) + 64);
    int32_t* deg = c->aux3.as<int32_t>();
    int32_t* rowp = deg + ng + 1;
    int64_t* tcnt = (int64_t*)(((uintptr_t)(rowp + ng + 1) + 15) & ~(uintptr_t)15);
    int64_t* toff = tcnt + mg + 1;
    int64_t ntri = 0;
    if (m > 0) {
        size_t tmp = 0;
        RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, K.k0, K.k1, K.w0, K.w1, (int)m, 0, 64, s));
        c->cub_tmp.reserve(tmp);
        RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, K.k0, K.k1, K.w0, K.w1, (int)m, 0, 64, s));
        c->launches += cub_sort_kernels(m, 64);
        if (check_pairs && m > 1) {
            unsigned int* bad = (unsigned int*)(c->counters.as<unsigned long long>() + 10);
            RNNG_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned int), s));
            k_dup_keys<<<grid_for(c, m), 256, 0, s>>>(K.k1, m, bad);
            ++c->launches;
            RNNG_REQUIRE(read_flag(c, bad) == 0, RNNG_ERR_INVALID, "an unordered pair appears twice in the edge list");
        }
        RNNG_CUDA(cudaMemsetAsync(deg, 0, sizeof(int32_t) * (ng + 1), s));
        k_degree<<<grid_for(c, m), 256, 0, s>>>(K.k1, m, deg);
        ++c->launches;
        exclusive_scan_i32(c, deg, rowp, n + 1);
        if (maxdim >= 2) {
            if (colex)
                k_triangles_colex<false><<<grid_for(c, m), 256, 0, s>>>(K.k1, K.w1, rowp, m, R.id_of_rank, tcnt,
                                                                       nullptr, nullptr, nullptr, nullptr, nullptr);
            else
                k_triangles<false><<<grid_for(c, m), 256, 0, s>>>(K.k1, K.w1, rowp, m, R.id_of_rank, tcnt, nullptr,
                                                                 nullptr, nullptr, nullptr, nullptr, nullptr);
            ++c->launches;
            ntri = scan_counts(c, tcnt, toff, m);
        }
    }
    const int64_t nedge = maxdim >= 1 ? m : 0;
    RNNG_REQUIRE(n + nedge + ntri <= kMaxSimplices, RNNG_ERR_INVALID, "too many simplices for one call");
    // ---- simplices of dimension >= 2, level by level, gathered in hi_id / hi_val / hi_flag
    int64_t nhi = 0;
    if (ntri > 0) {
        c->hi_id.reserve(sizeof(int64_t) * (size_t)ntri);
        c->hi_val.reserve(sizeof(float) * (size_t)ntri);
        if (with_flags) c->hi_flag.reserve((size_t)ntri);
        int32_t* clq = nullptr;
        if (maxdim >= 3) {
            c->clq0.reserve(sizeof(int32_t) * 3 * (size_t)ntri);
            clq = c->clq0.as<int32_t>();
        }
        if (colex)
            k_triangles_colex<true><<<grid_for(c, m), 256, 0, s>>>(K.k1, K.w1, rowp, m, R.id_of_rank, nullptr, toff,
                                                                  c->hi_id.as<int64_t>(), c->hi_val.as<float>(), fr,
                                                                  with_flags ? c->hi_flag.as<uint8_t>() : nullptr);
        else
            k_triangles<true><<<grid_for(c, m), 256, 0, s>>>(K.k1, K.w1, rowp, m, R.id_of_rank, nullptr, toff,
                                                            c->hi_id.as<int64_t>(), c->hi_val.as<float>(), clq, fr,
                                                            with_flags ? c->hi_flag.as<uint8_t>() : nullptr);
        ++c->launches;
        nhi = ntri;
        int64_t nc = ntri;   // cliques of the last level: k ranks each in *cur
        int64_t lvl_at = 0;  // their values start at hi_val + lvl_at
        DevBuf* cur = &c->clq0;
        DevBuf* nxt = &c->clq1;
        for (int k = 3; k <= maxdim && nc > 0; ++k) {
            c->aux4.reserve(sizeof(int64_t) * 2 * ((size_t)nc + 1));
            int64_t* ccnt = c->aux4.as<int64_t>();
            int64_t* coff = ccnt + nc + 1;
            k_extend<false><<<grid_for(c, nc), 256, 0, s>>>(cur->as<int32_t>(), c->hi_val.as<float>() + lvl_at, nc, k,
                                                           K.k1, K.w1, rowp, R.id_of_rank, ccnt, nullptr, nullptr,
                                                           nullptr, nullptr, nullptr, nullptr);
            ++c->launches;
            const int64_t nn = scan_counts(c, ccnt, coff, nc);
            RNNG_REQUIRE(n + nedge + nhi + nn <= kMaxSimplices, RNNG_ERR_INVALID, "too many simplices for one call");
            if (nn == 0) break;
            grow_keep(c, c->hi_id, sizeof(int64_t) * (size_t)(nhi + nn), sizeof(int64_t) * (size_t)nhi);
            grow_keep(c, c->hi_val, sizeof(float) * (size_t)(nhi + nn), sizeof(float) * (size_t)nhi);
            if (with_flags) grow_keep(c, c->hi_flag, (size_t)(nhi + nn), (size_t)nhi);
            int32_t* next_clq = nullptr;
            if (k < maxdim) {
                nxt->reserve(sizeof(int32_t) * (size_t)(k + 1) * (size_t)nn);
                next_clq = nxt->as<int32_t>();
            }
            k_extend<true><<<grid_for(c, nc), 256, 0, s>>>(
                cur->as<int32_t>(), c->hi_val.as<float>() + lvl_at, nc, k, K.k1, K.w1, rowp, R.id_of_rank, nullptr,
                coff, c->hi_id.as<int64_t>() + nhi, c->hi_val.as<float>() + nhi, next_clq, fr,
                with_flags ? c->hi_flag.as<uint8_t>() + nhi : nullptr);
            ++c->launches;
            lvl_at = nhi;
            nhi += nn;
            nc = nn;
            std::swap(cur, nxt);
        }
    }
    // ---- all simplices, then sort by (value, id)
    const int64_t total = n + nedge + nhi;
    const int64_t tg = std::max<int64_t>(total, 1);
    c->out_u.reserve(sizeof(int64_t) * 2 * (size_t)tg);  // ids (two buffers)
    c->out_w.reserve(sizeof(float) * 2 * (size_t)tg);    // values
    c->out_v.reserve(sizeof(int32_t) * 2 * (size_t)tg + sizeof(uint32_t) * 2 * (size_t)tg);
    int64_t* id0 = c->out_u.as<int64_t>();
    int64_t* id1 = id0 + tg;
    float* v0 = c->out_w.as<float>();
    float* v1 = v0 + tg;
    int32_t* p0 = c->out_v.as<int32_t>();
    int32_t* p1 = p0 + tg;
    uint32_t* b0 = (uint32_t*)(p1 + tg);
    uint32_t* b1 = b0 + tg;
    uint8_t* f0 = nullptr;
    uint8_t* f1 = nullptr;
    if (with_flags) {
        c->sflag.reserve(2 * (size_t)tg);
        f0 = c->sflag.as<uint8_t>();
        f1 = f0 + tg;
    }
    if (n + nedge > 0) {
        k_vertices_edges<<<grid_for(c, n + nedge), 256, 0, s>>>(R.id_of_rank, n, K.k1, K.w1, m, maxdim >= 1, colex,
                                                                id0, v0, fr, f0);
        ++c->launches;
    }
    if (nhi > 0) {
        RNNG_CUDA(cudaMemcpyAsync(id0 + n + nedge, c->hi_id.ptr, sizeof(int64_t) * nhi, cudaMemcpyDeviceToDevice, s));
        RNNG_CUDA(cudaMemcpyAsync(v0 + n + nedge, c->hi_val.ptr, sizeof(float) * nhi, cudaMemcpyDeviceToDevice, s));
        if (with_flags)
            RNNG_CUDA(cudaMemcpyAsync(f0 + n + nedge, c->hi_flag.ptr, (size_t)nhi, cudaMemcpyDeviceToDevice, s));
    }
    int64_t* ids_out = id0;
    float* vals_out = v0;
    uint8_t* flags_out = f0;
    // Values are >= +0, so their bits sort in numeric order; every radix pass is stable.
    if (total > 1 && colex) {
        // already in id order: one pass by value
        const unsigned gt = grid_for(c, total);
        size_t tmp = 0;
        if (!with_flags) {
            const uint32_t* kin = (const uint32_t*)v0;
            uint32_t* kout = (uint32_t*)v1;
            RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, kin, kout, id0, id1, (int)total, 0, 32, s));
            c->cub_tmp.reserve(tmp);
            RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, kin, kout, id0, id1, (int)total, 0, 32, s));
            c->launches += cub_sort_kernels(total, 32);
        } else {
            k_value_bits<<<gt, 256, 0, s>>>(v0, total, b0, p0);
            ++c->launches;
            uint32_t* kout = (uint32_t*)v1;
            RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, b0, kout, p0, p1, (int)total, 0, 32, s));
            c->cub_tmp.reserve(tmp);
            RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, b0, kout, p0, p1, (int)total, 0, 32, s));
            c->launches += cub_sort_kernels(total, 32);
            k_permute<int64_t><<<gt, 256, 0, s>>>(id0, p1, total, id1);
            k_permute<uint8_t><<<gt, 256, 0, s>>>(f0, p1, total, f1);
            c->launches += 2;
            flags_out = f1;
        }
        ids_out = id1;
        vals_out = v1;
    } else if (total > 1 && !with_flags) {
        // by id carrying the value bits, then by value bits carrying the ids
        size_t tmp = 0;
        const uint32_t* bin = (const uint32_t*)v0;
        uint32_t* vout = (uint32_t*)v1;
        RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, id0, id1, bin, b1, (int)total, 0, 64, s));
        c->cub_tmp.reserve(tmp);
        RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, id0, id1, bin, b1, (int)total, 0, 64, s));
        c->launches += cub_sort_kernels(total, 64);
        RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, b1, vout, id1, id0, (int)total, 0, 32, s));
        c->cub_tmp.reserve(tmp);
        RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, b1, vout, id1, id0, (int)total, 0, 32, s));
        c->launches += cub_sort_kernels(total, 32);
        ids_out = id0;
        vals_out = v1;
    } else if (total > 1) {
        // stable passes: by id, then by value bits, carrying positions for the flags
        const unsigned gt = grid_for(c, total);
        size_t tmp = 0;
        k_value_bits<<<gt, 256, 0, s>>>(v0, total, b0, p0);
        ++c->launches;
        RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, id0, id1, p0, p1, (int)total, 0, 64, s));
        c->cub_tmp.reserve(tmp);
        RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, id0, id1, p0, p1, (int)total, 0, 64, s));
        c->launches += cub_sort_kernels(total, 64);
        k_permute<uint32_t><<<gt, 256, 0, s>>>(b0, p1, total, b1);
        ++c->launches;
        RNNG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp, b1, b0, p1, p0, (int)total, 0, 32, s));
        c->cub_tmp.reserve(tmp);
        RNNG_CUDA(cub::DeviceRadixSort::SortPairs(c->cub_tmp.ptr, tmp, b1, b0, p1, p0, (int)total, 0, 32, s));
        c->launches += cub_sort_kernels(total, 32);
        k_permute<int64_t><<<gt, 256, 0, s>>>(id0, p0, total, id1);
        k_permute<float><<<gt, 256, 0, s>>>(v0, p0, total, v1);
        c->launches += 2;
        if (with_flags) {
            k_permute<uint8_t><<<gt, 256, 0, s>>>(f0, p0, total, f1);
            ++c->launches;
            flags_out = f1;
        }
        ids_out = id1;
        vals_out = v1;
    }
    deliver_simplices(c, ids_out, vals_out, flags_out, total, flags, out);
    RNNG_CUDA(cudaEventRecord(c->ev[7], s));
    RNNG_CUDA(cudaStreamSynchronize(s));
    c->stats.edges = m;
    c->stats.simplices = total;
}

void begin_call(rnng_ctx* c)
{
    c->stats = rnng_stats{};
    c->launches = 0;
    c->gram_ms = 0.0;
    c->counters.reserve(sizeof(unsigned long long) * kCounterSlots);
    RNNG_CUDA(cudaEventRecord(c->ev[0], c->stream));
}

void end_call(rnng_ctx* c)
{
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev[0], c->ev[7]);
    c->stats.ms_total = ms;
    c->stats.kernel_launches = c->launches;
    c->stats.ms_gram = c->gram_ms;
}

}  // namespace

extern "C" int rnng_rips_l2(rnng_ctx* c, const float* X, const int64_t* ids, int64_t n, int64_t d, float radius,
                            int maxdim, int mode, unsigned flags, rnng_simplices* out)
{
    return guarded(c, [&] {
        RNNG_REQUIRE(out != nullptr, RNNG_ERR_INVALID, "out is null");
        std::memset(out, 0, sizeof(*out));
        RNNG_REQUIRE(n >= 0 && d >= 1 && (n == 0 || X), RNNG_ERR_INVALID, "bad points");
        RNNG_REQUIRE(n < (int64_t(1) << 31) - kTile, RNNG_ERR_INVALID, "n too large");
        RNNG_REQUIRE(maxdim >= 0 && maxdim <= kRipsMaxDim, RNNG_ERR_UNSUPPORTED, "maxdim must be in [0, 15]");
        RNNG_REQUIRE(mode == RNNG_MODE_FP32_DIRECT || mode == RNNG_MODE_BF16_RECHECK, RNNG_ERR_INVALID, "bad mode");
        if (mode == RNNG_MODE_BF16_RECHECK)
            RNNG_REQUIRE(bf16_supported((int)d), RNNG_ERR_UNSUPPORTED, "BF16 mode supports d <= 256");
        RNNG_REQUIRE(radius == radius, RNNG_ERR_INVALID, "radius is NaN");
        begin_call(c);
        cudaStream_t s = c->stream;
        const float* dX = (const float*)upload(c, c->x_in, X, sizeof(float) * (size_t)(n * d), flags);
        const int64_t* dids = (const int64_t*)upload(c, c->ids_in, ids, sizeof(int64_t) * (size_t)n, flags);
        RNNG_CUDA(cudaEventRecord(c->ev[1], s));
        const Ranks R = rank_vertices(c, dids, n);
        // epsilon graph (sorted-index space), then rank-space keys
        int64_t m = 0;
        Layout L;
        EdgeOut E;
        if (maxdim >= 1 && n >= 2 && radius >= 0.f) m = eps_core(c, dX, n, (int)d, radius, mode, L, E);
        const Keys K = key_buffers(c, m);
        if (m > 0) {
            k_edge_keys<<<grid_for(c, m), 256, 0, s>>>(E.si, E.sj, E.w, m, L.perm, R.rank, K.k0, K.w0);
            ++c->launches;
        }
        rips_from_keys(c, n, R, K, m, maxdim, flags, false, nullptr, out);
        c->stats.tile_pairs = (int64_t)L.tile_pairs;
        end_call(c);
    });
}

extern "C" int rnng_rips_edges(rnng_ctx* c, int64_t n, const int64_t* ids, const uint8_t* vertex_flags,
                               const int64_t* u, const int64_t* v, const float* w, int64_t m, int maxdim,
                               unsigned flags, rnng_simplices* out)
{
    return guarded(c, [&] {
        RNNG_REQUIRE(out != nullptr, RNNG_ERR_INVALID, "out is null");
        std::memset(out, 0, sizeof(*out));
        RNNG_REQUIRE(n >= 0 && m >= 0 && (m == 0 || (u && v && w)), RNNG_ERR_INVALID, "bad graph");
        RNNG_REQUIRE(n < (int64_t(1) << 31) && m < (int64_t(1) << 31), RNNG_ERR_INVALID, "graph too large");
        RNNG_REQUIRE(maxdim >= 0 && maxdim <= kRipsMaxDim, RNNG_ERR_UNSUPPORTED, "maxdim must be in [0, 15]");
        begin_call(c);
        cudaStream_t s = c->stream;
        const int64_t* dids = (const int64_t*)upload(c, c->ids_in, ids, sizeof(int64_t) * (size_t)n, flags);
        const int64_t* du = (const int64_t*)upload(c, c->x_sorted, u, sizeof(int64_t) * (size_t)m, flags);
        const int64_t* dv = (const int64_t*)upload(c, c->xb_sorted, v, sizeof(int64_t) * (size_t)m, flags);
        const float* dw = (const float*)upload(c, c->norms, w, sizeof(float) * (size_t)m, flags);
        const uint8_t* dvflag = (const uint8_t*)upload(c, c->pivots, vertex_flags, (size_t)n, flags);
        RNNG_CUDA(cudaEventRecord(c->ev[1], s));
        const Ranks R = rank_vertices(c, dids, n);
        const Keys K = key_buffers(c, m);
        if (m > 0) {
            unsigned int* bad = (unsigned int*)(c->counters.as<unsigned long long>() + 10);
            RNNG_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned int), s));
            k_row_edge_keys<<<grid_for(c, m), 256, 0, s>>>(du, dv, dw, m, n, R.rank, K.k0, K.w0, bad);
            ++c->launches;
            RNNG_REQUIRE(read_flag(c, bad) == 0, RNNG_ERR_INVALID,
                         "edge with a row out of range, a self-loop, or a negative or NaN value");
        }
        rips_from_keys(c, n, R, K, m, maxdim, flags, true, dvflag, out);
        end_call(c);
    });
}
