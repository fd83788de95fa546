/*
 * rnng_gpu.h - C ABI of the GB300 epsilon-graph / Vietoris-Rips library.
 *
 * One shared library (librnng_gpu.so) owns all device work for RNNG's hot path.
 * The C++ headers next to this file (point.h, search.h, graph.h, simplex.h) keep
 * RNNG's template API and forward their bulk operations here; Python tests and
 * the benchmark bind the same entry points through ctypes.
 *
 * Conventions
 *   - Every entry point returns an int status: RNNG_OK (0) or an RNNG_ERR_* code.
 *     Nothing throws across this boundary.  rnng_last_error() gives the message.
 *   - Plain pointers and sizes only.  Pointers are host memory unless the call's
 *     flags say RNNG_INPUT_DEVICE (inputs) / RNNG_OUTPUT_DEVICE (outputs).
 *   - Results live in library-owned buffers of the context: device arrays with
 *     RNNG_OUTPUT_DEVICE, otherwise host arrays in the context's pinned staging
 *     memory.  Either way they stay valid until the next call on the same context
 *     (copy them to keep them); rnng_edges_free / rnng_simplices_free on them is a
 *     no-op, so steady-state calls allocate nothing.
 *   - All work of a context is ordered on the context's CUDA stream.  One context
 *     per host thread; calls on one context must not overlap.
 *   - Point ids are int64 (RNNG's Index, include/utils.h:24); distances are float
 *     (RNNG's Real, include/utils.h:25).
 *
 * Distances and predicates are those of RNNG's drivers:
 *   L2   = sqrtf(sum_i (p_i - q_i)^2), float, sequential i = 0..d-1, no FMA
 *          (drivers/systolic.cpp:253-269); edge iff L2 <= radius.
 *   edit = Levenshtein distance with unit costs, as a float
 *          (drivers/systolic.cpp:271-299); edge iff edit <= radius.
 * Every reported distance is bit-identical to what those functors return.
 */
#ifndef RNNG_GPU_H_
#define RNNG_GPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define RNNG_OK 0
#define RNNG_ERR_INVALID 1    /* bad argument (null pointer, negative size, dimension mismatch) */
#define RNNG_ERR_CUDA 2       /* a CUDA runtime call failed */
#define RNNG_ERR_NOMEM 3      /* device or host allocation failed */
#define RNNG_ERR_OVERFLOW 4   /* a result does not fit the representation (e.g. simplex ids) */
#define RNNG_ERR_DEVICE 5     /* a kernel reported a fault through its error word (e.g. a bounded wait ran out) */
#define RNNG_ERR_UNSUPPORTED 6

/* flags */
#define RNNG_INPUT_DEVICE 1u   /* input pointers are device pointers (no host-to-device copy) */
#define RNNG_OUTPUT_DEVICE 2u  /* leave results on the device (no device-to-host copy) */
#define RNNG_SORT_OUTPUT 4u    /* sort edges by (u, v) / simplices by (value, id) */
#define RNNG_FINALIZE_AS_GIVEN 8u /* rnng_graph_finalize: edges as a driver collected them (see there) */

/* L2 tile modes */
#define RNNG_MODE_FP32_DIRECT 0  /* every candidate pair evaluated with the reference's sequential FP32 L2 */
#define RNNG_MODE_BF16_RECHECK 1 /* BF16 tensor-core Gram candidates with a rigorous margin, FP32 recheck */

typedef struct rnng_ctx rnng_ctx;

/* Unordered edges u < v with their reference distances, in point-id space. */
typedef struct rnng_edges {
    int64_t count;
    int64_t* u;
    int64_t* v;
    float* w;
    int on_device; /* 1: u, v, w are device pointers */
    int staged;    /* 1: arrays owned by the context (not freed by rnng_edges_free) */
} rnng_edges;

/* A filtration: simplex ids (RNNG's Simplex encoding, include/simplex.hpp:5-19) and values.
 * flag (rnng_rips_edges with vertex flags, else NULL): 1 when one of the simplex's
 * vertices is flagged, RNNG's `interior` of a WeightedSimplex (include/point.hpp:1160-1168). */
typedef struct rnng_simplices {
    int64_t count;
    int64_t* id;
    float* value;
    int on_device;
    int staged;
    uint8_t* flag;
} rnng_simplices;

/* Counters and stage times of the last call on a context (milliseconds). */
typedef struct rnng_stats {
    double ms_total, ms_h2d, ms_partition, ms_sort, ms_bounds, ms_prune, ms_tiles, ms_recheck, ms_finalize, ms_d2h;
    int64_t num_cells;      /* landmarks / cells of the partition */
    int64_t super_pairs;    /* super-tile pairs that survived the first pruning level */
    int64_t tile_pairs;     /* tile pairs that survived pruning */
    int64_t tile_pairs_all; /* tile pairs before pruning */
    int64_t pairs_evaluated;/* point pairs inside surviving tiles */
    int64_t candidates;     /* BF16 mode: pairs sent to the FP32 recheck */
    int64_t edges;          /* edges found (u < v) */
    int64_t retries;        /* edge-buffer regrowths */
    int64_t simplices;      /* Rips: simplices emitted */
    int64_t kernel_launches;/* kernels launched by the call */
    double ms_gram;         /* device time of the tensor-core Gram kernel (BF16 mode; the edit filter) */
    double prune_widen;     /* mean relative widening of the tensor-core ball test (d <= 256) */
    int64_t prune_tensor;   /* 1: tile pairs pruned by the tensor-core ball test, 0: by the FP32 one */
    int64_t gram_nt;        /* Gram kernel of the last call: item form (1, 2: column tiles per
                               item, 3: row-tile pairs; 0: not run) */
    int64_t gram_chunk;     /*   items per work-queue chunk */
    int64_t gram_slots;     /*   B operand slots per CTA */
} rnng_stats;

/* Context ---------------------------------------------------------------------------------
 * Replaces nothing in RNNG (which has no device state); it holds the GPU, the stream
 * and reusable scratch so that steady-state calls do not allocate. */
int rnng_ctx_create(int device, rnng_ctx** out);
int rnng_ctx_destroy(rnng_ctx* ctx);
const char* rnng_last_error(const rnng_ctx* ctx);
int rnng_get_stats(const rnng_ctx* ctx, rnng_stats* out);
/* The context's CUDA stream (cudaStream_t), for callers that order their own work with it. */
int rnng_ctx_stream(rnng_ctx* ctx, void** stream);
/* Releases all cached scratch memory of the context. */
int rnng_ctx_trim(rnng_ctx* ctx);
/* No counterpart in RNNG: the tuning knobs of the tensor-core Gram kernel, for the
 * autotuner (rnng_gb300/tune.py).  nt = item form: 1 = one row tile x one column tile,
 * 2 = one row tile x two column tiles, 3 = two row tiles x one column tile (2 and 3 for
 * padded dimensions up to 128), chunk = items per work-queue chunk, slots = B operand slots per
 * CTA (at least 2, capped by shared memory).  A 0 keeps the value of the tuning table
 * (rnng_gb300/gram_tuning.json, read when the context is created; $RNNG_GRAM_TUNING
 * names another file) or the default; all three 0 restores the table. */
int rnng_ctx_set_gram_tuning(rnng_ctx* ctx, int nt, int chunk, int slots);
/* No counterpart in RNNG: a drill of the failure handling.  While on, the tensor-core Gram
 * kernel's epilogue waits on a barrier that nothing arrives on; its bounded wait (about
 * one second) runs out, the kernel winds down (copies and MMAs in flight drained, tensor
 * memory freed), and the call returns RNNG_ERR_DEVICE.  The context stays usable. */
int rnng_ctx_fault_drill(rnng_ctx* ctx, int on);

/* Epsilon graph, L2 ------------------------------------------------------------------------
 * Replaces the neighbour search of the drivers: CoverTree::build + radius_query per point
 * (drivers/systolic.cpp:96-147, include/search.hpp:6-264) and the landmark pipeline
 * VoronoiDiagram + add_ghost_points_systolic + per-cell radius_query_batched
 * (drivers/landmark.cpp:139-210, include/point.hpp:537-929, include/search.hpp:267-340).
 * X is n x d row-major float32; ids (may be NULL = 0..n-1) are the point ids.
 * Output: every unordered pair with L2 <= radius, as u < v (ids compared), each once.
 * A point with a NaN or infinite coordinate is at L2 NaN or +inf from every point, so
 * it has no edge (RNNG's own result for NaN rows); with radius = +inf a point with an
 * infinite coordinate and no NaN would pair at distance +inf, which is refused with
 * RNNG_ERR_UNSUPPORTED. */
int rnng_eps_graph_l2(rnng_ctx* ctx, const float* X, const int64_t* ids, int64_t n, int64_t d, float radius,
                      int mode, unsigned flags, rnng_edges* out);

/* Radius query of a batch against an indexed set: every (query q, point p) with
 * L2(p, q) <= radius.  Replaces CoverTree::radius_query_batched
 * (include/search.hpp:267-340) and BruteForce::radius_query (include/search.hpp:390-407).
 * out->u holds query ids, out->v point ids (the functor's (q.id(), p.id()) order in
 * drivers/landmark.cpp:198-201). */
int rnng_radius_query_l2(rnng_ctx* ctx, const float* X, const int64_t* ids, int64_t n, const float* Q,
                         const int64_t* qids, int64_t nq, int64_t d, float radius, unsigned flags,
                         rnng_edges* out);

/* Nearest landmark per point with the reference's tie rule (the last of equal
 * distances wins): VoronoiDiagram::VoronoiDiagram (include/point.hpp:537-559).
 * cell[i] in [0, m), dist[i] = L2(center, x_i) bit-identical to the reference. */
int rnng_voronoi_l2(rnng_ctx* ctx, const float* X, int64_t n, const float* C, int64_t m, int64_t d,
                    unsigned flags, int64_t* cell, float* dist);

/* Nearest landmark per string under edit distance, same tie rule and output as
 * rnng_voronoi_l2: VoronoiDiagram<char>::VoronoiDiagram (include/point.hpp:537-559) with
 * the drivers' EditDistance<char> (drivers/landmark.cpp:354-383).  Strings and centres
 * in RNNG's CSR layout (atoms, offsets[count + 1]); centres up to 4096 characters. */
int rnng_voronoi_edit(rnng_ctx* ctx, const uint8_t* atoms, const int64_t* offsets, int64_t n,
                      const uint8_t* centre_atoms, const int64_t* centre_offsets, int64_t m, unsigned flags,
                      int64_t* cell, float* dist);

/* Epsilon graph, edit distance -------------------------------------------------------------
 * Strings in RNNG's CSR layout (include/point.h:77-79): atoms[offsets[i] .. offsets[i+1]).
 * Replaces the drivers' edit-distance path (drivers/landmark.cpp:61-62 with
 * EditDistance<char>).  Output as rnng_eps_graph_l2. */
int rnng_eps_graph_edit(rnng_ctx* ctx, const uint8_t* atoms, const int64_t* offsets, const int64_t* ids,
                        int64_t n, float radius, unsigned flags, rnng_edges* out);

/* Vietoris-Rips filtration ----------------------------------------------------------------
 * Replaces VoronoiComplex::build_filtration per cell + merge_and_write_filtration
 * (include/point.hpp:1136-1267, include/simplex.hpp:130-196, drivers/rips.cpp:174-245):
 * all vertices (value 0), edges (value = L2) and every clique of up to maxdim + 1
 * vertices (value = its largest edge, RNNG's max over facets), ids per
 * include/simplex.hpp:5-19 over the point ids, sorted by (value, id).  maxdim is 0..15
 * (the id keeps the dimension in 4 bits); RNNG's rips driver defaults to 3.  Points
 * with a NaN or infinite coordinate are vertices without edges (as in rnng_eps_graph_l2). */
int rnng_rips_l2(rnng_ctx* ctx, const float* X, const int64_t* ids, int64_t n, int64_t d, float radius,
                 int maxdim, int mode, unsigned flags, rnng_simplices* out);

/* The same filtration for a graph the caller already has: VoronoiComplex::build_filtration
 * after its neighbour graph is built (include/point.hpp:1146-1230), for any metric (the
 * drop-in headers use it for edit-distance complexes and for cells cut from a cached
 * whole-set graph).  Vertices are rows 0..n-1 with ids (NULL = the rows) and optional
 * vertex_flags (nonzero = flagged; NULL = none, out->flag stays NULL); u[e], v[e] are
 * rows (either order) and w[e] >= 0 the edge's value; each unordered pair at most once.
 * RNNG_ERR_INVALID for rows out of range, self-loops, repeated pairs, negative or NaN
 * values; -0 is taken as +0. */
int rnng_rips_edges(rnng_ctx* ctx, int64_t n, const int64_t* ids, const uint8_t* vertex_flags, const int64_t* u,
                    const int64_t* v, const float* w, int64_t m, int maxdim, unsigned flags, rnng_simplices* out);

/* Graph finalisation: Graph(edges) + redistribute_edges at one rank
 * (include/graph.h:14, include/graph.hpp:59-116): from unordered edges, the list of
 * both orientations plus the self-loop (i, i, 0) of every vertex 0..num_vertices-1,
 * sorted by (u, v).  Output count = num_vertices + 2 * edges.  (RNNG's self-loops come
 * from each point finding itself within the radius, so a point with a non-finite
 * coordinate has none there; drop such rows' (i, i, 0) entries to match.)
 * With RNNG_FINALIZE_AS_GIVEN the edges are taken as RNNG's drivers collect them (any
 * orientation, repeats and self-loops allowed) and the output is exactly what
 * Graph::redistribute_edges leaves at one rank: both orientations of every given edge,
 * sorted by (u, v, w), repeated tuples removed, no self-loops added (num_vertices is
 * then only checked against the ids). */
int rnng_graph_finalize(rnng_ctx* ctx, const rnng_edges* edges, int64_t num_vertices, unsigned flags,
                        rnng_edges* out);

/* Diagnostic, no counterpart in RNNG: one tile pair through the tensor-core Gram kernel of
 * rnng_eps_graph_l2's BF16 mode, to measure the tensor cores' FP32 accumulation against the
 * error bound the candidate test assumes.  X: 256 x d host floats (d = 64, 128, 192 or
 * 256), rows 0..127 the row tile, rows 128..255 the column tile.  Outputs (host):
 * G[i * 128 + j] = the raw accumulator of row i against row 128 + j; Xb (256 x d) = the
 * BF16 operand rows as the kernel used them (shifted by the rounded column means, as
 * floats); rowinfo (256 x 4 floats) = per row {BF16 norm, error radius a, accumulation
 * bound q, column term}.  The candidate test is sound when |2 (G - Xb_i . Xb_j)| <= q_i + q_j. */
int rnng_gram_probe_bf16(rnng_ctx* ctx, const float* X, int64_t d, float* G, float* Xb, float* rowinfo);

int rnng_edges_free(rnng_edges* e);
int rnng_simplices_free(rnng_simplices* s);

/* Allocation-free epsilon graph ------------------------------------------------------------
 * No counterpart in RNNG: an extra entry point for callers that cannot allocate device
 * memory when they need the graph - a process whose device memory belongs to a
 * framework's pool (a plugin gets buffers from it but may not call cudaMalloc beside
 * it), a real-time loop that must not allocate after start-up, or a plugin host that
 * forbids allocation inside the plugin.  It takes no context and calls no cudaMalloc /
 * cudaFree: the caller owns every buffer, and the library's scratch is a fixed device
 * array of about 12 MiB that each GPU loading the library holds until exit.
 *   X, ids (ids may be NULL = 0..n-1): device pointers; n <= 65536 points, d <= 4096;
 *   u, v, w: device arrays of `capacity` entries for the unordered edges u < v (any order);
 *   *count (host): number of edges found; stream: a cudaStream_t or NULL.
 * Same edges and bit-identical weights as rnng_eps_graph_l2 (all pairs are evaluated
 * with the reference's sequential FP32 L2), the same RNNG_ERR_UNSUPPORTED for radius
 * +inf with a row that holds an infinity and no NaN.  Returns RNNG_ERR_INVALID beyond
 * the size limits and RNNG_ERR_OVERFLOW when more than min(capacity, 1048576) edges
 * exist: then an unspecified subset of min(capacity, 1048576) of them is written (which
 * ones can differ from call to call) and *count holds the total.  The call reads the
 * count back to the host, so it synchronises `stream` before it returns.  The first
 * call on a device looks up the scratch address; make it before any stream capture.
 * Every call shares the one scratch array, so calls whose GPU work overlaps race and
 * must be serialised. */
int rnng_eps_graph_l2_static(const float* X, const int64_t* ids, int64_t n, int64_t d, float radius, int64_t* u,
                             int64_t* v, float* w, int64_t capacity, int64_t* count, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* RNNG_GPU_H_ */
