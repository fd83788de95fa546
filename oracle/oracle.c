/*
 * CPU oracle for the epsilon-graph / Vietoris-Rips hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the arithmetic and the
 * output contract of RNNG's CPU path so that the GPU library can be checked against
 * it.  Only tests, the smoke check and the benchmark's CPU-baseline leg load it; the
 * GPU library never calls it and has no CPU fallback.
 *
 * Build with -ffp-contract=off (see oracle/Makefile): the reference's L2 loop is a
 * sequential difference-square-sum without fused multiply-add, and a compiler that
 * contracts `val += delta*delta` into an FMA produces different float bits.
 *
 * What each function follows in RNNG (paths relative to the RNNG source tree):
 *   orc_l2seq            drivers/systolic.cpp:253-269 (L2Distance<float>::operator())
 *   orc_edit             drivers/systolic.cpp:271-299 (EditDistance<char>::operator())
 *   orc_eps_graph_*      include/search.hpp:390-407 (BruteForce::radius_query predicate
 *                        `dist <= radius`), over all unordered pairs i < j
 *   orc_binom            include/utils.hpp:116-144 (Binom::operator(): int64 falling
 *                        product divided by k!)
 *   orc_simplex_id       include/simplex.hpp:5-19 (Simplex(verts): sum C(v_i, i+1) | dim<<60)
 *   orc_voronoi[_edit]   include/point.hpp:537-559 (VoronoiDiagram: `dist <= best`, last wins)
 *   orc_rips             include/point.hpp:1136-1232 (build_filtration: vertex value 0,
 *                        edge value = distance, higher simplex = max over facets) and
 *                        include/simplex.hpp:130-196 (merge: sort by (value, id), unique id)
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_threads(int t)
{
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

float orc_l2seq(const float* p, const float* q, int64_t d)
{
    float val = 0.0f;
    for (int64_t i = 0; i < d; ++i) {
        float delta = p[i] - q[i];
        val += delta * delta;
    }
    return sqrtf(val);
}

float orc_edit(const uint8_t* s, int64_t m, const uint8_t* t, int64_t n)
{
    int64_t stack0[256], stack1[256];
    int64_t *v0 = stack0, *v1 = stack1;
    int64_t* heap = NULL;
    if (n + 1 > 256) {
        heap = (int64_t*)malloc(sizeof(int64_t) * 2 * (size_t)(n + 1));
        v0 = heap;
        v1 = heap + n + 1;
    }
    for (int64_t i = 0; i <= n; ++i) v0[i] = i;
    for (int64_t i = 0; i < m; ++i) {
        v1[0] = i + 1;
        for (int64_t j = 0; j < n; ++j) {
            int64_t del = v0[j + 1] + 1;
            int64_t ins = v1[j] + 1;
            int64_t sub = (s[i] == t[j]) ? v0[j] : v0[j] + 1;
            int64_t best = ins < sub ? ins : sub;
            v1[j + 1] = del < best ? del : best;
        }
        int64_t* tmp = v0;
        v0 = v1;
        v1 = tmp;
    }
    float r = (float)v0[n];
    free(heap);
    return r;
}

/* ------------------------------------------------------------------ edge buffers */

typedef struct {
    int64_t* u;
    int64_t* v;
    float* w;
    int64_t count, cap;
} edge_buf;

static void eb_push(edge_buf* b, int64_t u, int64_t v, float w)
{
    if (b->count == b->cap) {
        int64_t cap = b->cap ? 2 * b->cap : 1024;
        b->u = (int64_t*)realloc(b->u, sizeof(int64_t) * (size_t)cap);
        b->v = (int64_t*)realloc(b->v, sizeof(int64_t) * (size_t)cap);
        b->w = (float*)realloc(b->w, sizeof(float) * (size_t)cap);
        b->cap = cap;
    }
    b->u[b->count] = u;
    b->v[b->count] = v;
    b->w[b->count] = w;
    b->count++;
}

/* Concatenates per-thread buffers into malloc'ed arrays owned by the caller
 * (release with orc_free).  The order is not specified; callers sort. */
static int64_t eb_merge(edge_buf* bufs, int nb, int64_t** u, int64_t** v, float** w)
{
    int64_t total = 0;
    for (int t = 0; t < nb; ++t) total += bufs[t].count;
    *u = (int64_t*)malloc(sizeof(int64_t) * (size_t)(total ? total : 1));
    *v = (int64_t*)malloc(sizeof(int64_t) * (size_t)(total ? total : 1));
    *w = (float*)malloc(sizeof(float) * (size_t)(total ? total : 1));
    int64_t off = 0;
    for (int t = 0; t < nb; ++t) {
        if (bufs[t].count) {
            memcpy(*u + off, bufs[t].u, sizeof(int64_t) * (size_t)bufs[t].count);
            memcpy(*v + off, bufs[t].v, sizeof(int64_t) * (size_t)bufs[t].count);
            memcpy(*w + off, bufs[t].w, sizeof(float) * (size_t)bufs[t].count);
        }
        free(bufs[t].u);
        free(bufs[t].v);
        free(bufs[t].w);
        off += bufs[t].count;
    }
    return total;
}

void orc_free(void* p) { free(p); }

/* Brute-force epsilon graph under the sequential L2 of the reference: all pairs
 * i < j with orc_l2seq(x_i, x_j) <= eps.  Rows [row_begin, row_end) are queried
 * against every later point (row_end = n for the full graph). */
int64_t orc_eps_graph_l2(const float* X, int64_t n, int64_t d, float eps, int64_t row_begin, int64_t row_end,
                         int64_t** u, int64_t** v, float** w)
{
    int nt = orc_num_threads();
    edge_buf* bufs = (edge_buf*)calloc((size_t)nt, sizeof(edge_buf));
    int64_t rows = row_end - row_begin;
#pragma omp parallel num_threads(nt)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        /* rows are interleaved in blocks of 64 to balance the triangular work; the
         * merged result is re-sorted by the caller when order matters */
        for (int64_t blk = t; blk * 64 < rows; blk += nt) {
            int64_t i0 = row_begin + blk * 64, i1 = i0 + 64;
            if (i1 > row_end) i1 = row_end;
            for (int64_t i = i0; i < i1; ++i) {
                const float* xi = X + i * d;
                for (int64_t j = i + 1; j < n; ++j) {
                    float dist = orc_l2seq(X + j * d, xi, d);
                    if (dist <= eps) eb_push(&bufs[t], i, j, dist);
                }
            }
        }
    }
    int64_t total = eb_merge(bufs, nt, u, v, w);
    free(bufs);
    return total;
}

/* Edges between query points Q (ids qbase + row) and indexed points X (ids 0..n-1):
 * every (q, p) with orc_l2seq(p, q) <= eps, as CoverTree::radius_query reports them
 * (include/search.hpp:224-264) for queries outside the indexed set. */
int64_t orc_cross_l2(const float* X, int64_t n, const float* Q, int64_t nq, int64_t d, float eps,
                     int64_t** u, int64_t** v, float** w)
{
    int nt = orc_num_threads();
    edge_buf* bufs = (edge_buf*)calloc((size_t)nt, sizeof(edge_buf));
#pragma omp parallel num_threads(nt)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        for (int64_t i = t; i < nq; i += nt) {
            for (int64_t j = 0; j < n; ++j) {
                float dist = orc_l2seq(X + j * d, Q + i * d, d);
                if (dist <= eps) eb_push(&bufs[t], i, j, dist);
            }
        }
    }
    int64_t total = eb_merge(bufs, nt, u, v, w);
    free(bufs);
    return total;
}

/* Brute-force epsilon graph under the reference's edit distance.  The length
 * difference is a lower bound on the edit distance, so pairs with
 * |len_i - len_j| > eps are skipped without changing the result. */
int64_t orc_eps_graph_edit(const uint8_t* atoms, const int64_t* offsets, int64_t n, float eps, int64_t row_begin,
                           int64_t row_end, int64_t** u, int64_t** v, float** w)
{
    int nt = orc_num_threads();
    edge_buf* bufs = (edge_buf*)calloc((size_t)nt, sizeof(edge_buf));
    int64_t rows = row_end - row_begin;
#pragma omp parallel num_threads(nt)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        for (int64_t blk = t; blk * 16 < rows; blk += nt) {
            int64_t i0 = row_begin + blk * 16, i1 = i0 + 16;
            if (i1 > row_end) i1 = row_end;
            for (int64_t i = i0; i < i1; ++i) {
                int64_t mi = offsets[i + 1] - offsets[i];
                for (int64_t j = i + 1; j < n; ++j) {
                    int64_t mj = offsets[j + 1] - offsets[j];
                    int64_t diff = mi > mj ? mi - mj : mj - mi;
                    if ((float)diff > eps) continue;
                    float dist = orc_edit(atoms + offsets[j], mj, atoms + offsets[i], mi);
                    if (dist <= eps) eb_push(&bufs[t], i, j, dist);
                }
            }
        }
    }
    int64_t total = eb_merge(bufs, nt, u, v, w);
    free(bufs);
    return total;
}

/* Nearest centre per point as VoronoiDiagram::VoronoiDiagram (include/point.hpp:
 * 537-559): distance(center, point), `dist <= best` over centres in order, so ties
 * go to the last centre; best starts at FLT_MAX and the cell at 0. */
void orc_voronoi(const float* X, int64_t n, const float* C, int64_t m, int64_t d, int64_t* cell, float* dist)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        float best = 3.40282346638528859812e+38F;
        int64_t bi = 0;
        for (int64_t c = 0; c < m; ++c) {
            float v = orc_l2seq(C + c * d, X + i * d, d);
            if (v <= best) {
                best = v;
                bi = c;
            }
        }
        cell[i] = bi;
        dist[i] = best;
    }
}

/* All n x m reference distances distance(C[c], X[i]) into out[i * m + c]. */
void orc_dist_matrix_l2(const float* X, int64_t n, const float* C, int64_t m, int64_t d, float* out)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
        for (int64_t c = 0; c < m; ++c) out[i * m + c] = orc_l2seq(C + c * d, X + i * d, d);
}

void orc_dist_matrix_edit(const uint8_t* atoms, const int64_t* offsets, int64_t n, const uint8_t* catoms,
                          const int64_t* coffsets, int64_t m, float* out)
{
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < n; ++i)
        for (int64_t c = 0; c < m; ++c)
            out[i * m + c] = orc_edit(catoms + coffsets[c], coffsets[c + 1] - coffsets[c], atoms + offsets[i],
                                      offsets[i + 1] - offsets[i]);
}

/* ------------------------------------------------------------------ simplices */

int64_t orc_binom(int64_t n, int64_t k)
{
    if (k > n) return 0;
    /* unsigned arithmetic wraps exactly where the reference's int64 product would
     * overflow; within range the two agree */
    uint64_t a = 1, b = 1;
    for (int64_t i = n; i >= n - k + 1; --i) a *= (uint64_t)i;
    for (int64_t i = k; i >= 1; --i) b *= (uint64_t)i;
    return (int64_t)((int64_t)a / (int64_t)b);
}

int64_t orc_simplex_id(const int64_t* sorted_verts, int64_t nverts)
{
    uint64_t p = (uint64_t)(nverts - 1);
    uint64_t uid = 0;
    for (int64_t i = (int64_t)p; i >= 0; --i) uid += (uint64_t)orc_binom(sorted_verts[i], i + 1);
    return (int64_t)(uid | (p << 60));
}

typedef struct {
    uint32_t vbits; /* float value bits; all values are >= +0 so bit order = numeric order */
    int64_t id;
} simplex_rec;

static int cmp_simplex(const void* a, const void* b)
{
    const simplex_rec* x = (const simplex_rec*)a;
    const simplex_rec* y = (const simplex_rec*)b;
    if (x->vbits != y->vbits) return x->vbits < y->vbits ? -1 : 1;
    if (x->id != y->id) return x->id < y->id ? -1 : 1;
    return 0;
}

typedef struct {
    const int64_t* deg; /* CSR of higher-numbered neighbours: deg[v] .. deg[v+1] */
    const int64_t* nbr;
    const float* nw;
    int maxdim;
    simplex_rec* out;
    int64_t cnt, cap;
} rips_walk;

static void rips_emit(rips_walk* r, const int64_t* verts, int64_t k, float value)
{
    if (r->cnt == r->cap) {
        r->cap = r->cap * 2 + 1024;
        r->out = (simplex_rec*)realloc(r->out, sizeof(simplex_rec) * (size_t)r->cap);
    }
    memcpy(&r->out[r->cnt].vbits, &value, 4);
    r->out[r->cnt].id = orc_simplex_id(verts, k);
    r->cnt++;
}

/* verts[0..k) is a clique (ascending) of value `value`; cand[0..nc) are the vertices
 * above verts[k-1] adjacent to all of it, cw[i] the largest edge from the clique to
 * cand[i].  Emits every clique that extends verts by candidates, up to maxdim + 1
 * vertices, each once (vertices are added in increasing order). */
static void rips_grow(rips_walk* r, int64_t* verts, int64_t k, float value, const int64_t* cand, const float* cw,
                      int64_t nc)
{
    if (k == (int64_t)r->maxdim + 1) return;
    int64_t* nc2 = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nc ? nc : 1));
    float* cw2 = (float*)malloc(sizeof(float) * (size_t)(nc ? nc : 1));
    for (int64_t i = 0; i < nc; ++i) {
        const int64_t y = cand[i];
        const float vy = cw[i] > value ? cw[i] : value;
        verts[k] = y;
        rips_emit(r, verts, k + 1, vy);
        /* candidates after y that are neighbours of y: merge with N+(y) */
        int64_t m2 = 0, p = r->deg[y];
        for (int64_t j = i + 1; j < nc; ++j) {
            while (p < r->deg[y + 1] && r->nbr[p] < cand[j]) ++p;
            if (p < r->deg[y + 1] && r->nbr[p] == cand[j]) {
                nc2[m2] = cand[j];
                cw2[m2] = cw[j] > r->nw[p] ? cw[j] : r->nw[p];
                ++m2;
            }
        }
        rips_grow(r, verts, k + 1, vy, nc2, cw2, m2);
    }
    free(nc2);
    free(cw2);
}

/* Vietoris-Rips filtration up to dimension maxdim (0..15) from an epsilon graph given
 * as unordered edges (u < v) with their reference distances.  Emits every vertex
 * (value 0) and every clique of 2 .. maxdim+1 vertices with the largest of its edge
 * weights as value (for edges the weight itself; above, RNNG's max over facets equals
 * the max over all edges), sorted by (value, id) with ids unique. */
int64_t orc_rips(int64_t n, const int64_t* eu, const int64_t* ev, const float* ew, int64_t m, int maxdim,
                 int64_t** ids, float** values)
{
    /* CSR of higher-numbered neighbours with weights */
    int64_t* deg = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    for (int64_t e = 0; e < m; ++e) deg[eu[e] + 1]++;
    for (int64_t i = 0; i < n; ++i) deg[i + 1] += deg[i];
    int64_t* nbr = (int64_t*)malloc(sizeof(int64_t) * (size_t)(m ? m : 1));
    float* nw = (float*)malloc(sizeof(float) * (size_t)(m ? m : 1));
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n ? n : 1));
    for (int64_t i = 0; i < n; ++i) fill[i] = deg[i];
    for (int64_t e = 0; e < m; ++e) {
        int64_t p = fill[eu[e]]++;
        nbr[p] = ev[e];
        nw[p] = ew[e];
    }
    /* sort each list by neighbour id (insertion sort: lists are short) */
    for (int64_t i = 0; i < n; ++i) {
        for (int64_t a = deg[i] + 1; a < deg[i + 1]; ++a) {
            int64_t kv = nbr[a];
            float kw = nw[a];
            int64_t b = a - 1;
            while (b >= deg[i] && nbr[b] > kv) {
                nbr[b + 1] = nbr[b];
                nw[b + 1] = nw[b];
                --b;
            }
            nbr[b + 1] = kv;
            nw[b + 1] = kw;
        }
    }

    rips_walk r = {deg, nbr, nw, maxdim, NULL, 0, 0};
    r.cap = n + (maxdim >= 1 ? m : 0) + 1024;
    r.out = (simplex_rec*)malloc(sizeof(simplex_rec) * (size_t)r.cap);
    int64_t verts[16];
    for (int64_t a = 0; a < n; ++a) {
        verts[0] = a;
        rips_emit(&r, verts, 1, 0.f);
        rips_grow(&r, verts, 1, 0.f, nbr + deg[a], nw + deg[a], deg[a + 1] - deg[a]);
    }
    simplex_rec* out = r.out;
    const int64_t cnt = r.cnt;
    qsort(out, (size_t)cnt, sizeof(simplex_rec), cmp_simplex);
    int64_t k = 0;
    for (int64_t i = 0; i < cnt; ++i)
        if (k == 0 || out[k - 1].id != out[i].id) out[k++] = out[i];
    *ids = (int64_t*)malloc(sizeof(int64_t) * (size_t)(k ? k : 1));
    *values = (float*)malloc(sizeof(float) * (size_t)(k ? k : 1));
    for (int64_t i = 0; i < k; ++i) {
        (*ids)[i] = out[i].id;
        memcpy(&(*values)[i], &out[i].vbits, 4);
    }
    free(out);
    free(deg);
    free(nbr);
    free(nw);
    free(fill);
    return k;
}

/* Nearest centre per string as VoronoiDiagram<char> with the drivers' EditDistance
 * (include/point.hpp:537-559, drivers/landmark.cpp:354-383): `dist <= best` over the
 * centres in order (ties to the last), best from FLT_MAX, cell from 0. */
void orc_voronoi_edit(const uint8_t* atoms, const int64_t* offsets, int64_t n, const uint8_t* catoms,
                      const int64_t* coffsets, int64_t m, int64_t* cell, float* dist)
{
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t i = 0; i < n; ++i) {
        float best = 3.40282346638528859812e+38F;
        int64_t bi = 0;
        for (int64_t c = 0; c < m; ++c) {
            float v = orc_edit(catoms + coffsets[c], coffsets[c + 1] - coffsets[c], atoms + offsets[i],
                               offsets[i + 1] - offsets[i]);
            if (v <= best) {
                best = v;
                bi = c;
            }
        }
        cell[i] = bi;
        dist[i] = best;
    }
}
