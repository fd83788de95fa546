/*
 * RNNG's landmark pipeline on the CPU: the reference algorithm timed as the CPU
 * baseline of the benchmark, and a second, independent way to the edge set.
 *
 * TEST INFRASTRUCTURE ONLY (like oracle.c): loaded by tests and by the benchmark's
 * CPU legs, never by the GPU library.
 *
 * This restates the work RNNG's `landmark` driver does at one rank, per host thread
 * (paths relative to the RNNG source tree):
 *   landmarks      drivers/landmark.cpp:107-124 (selection_sample of num_centers rows;
 *                  here a seeded partial Fisher-Yates draw - the choice changes the
 *                  cells, never the edge set)
 *   voronoi        include/point.hpp:537-559 (nearest landmark, `dist <= best`, the last
 *                  of equal distances wins)
 *   cells          include/point.hpp:562-758 at one rank (cells in landmark order, points
 *                  in row order, the landmark's own row moved to slot 0)
 *   cover trees    include/search.hpp:6-213 (CoverTree::build: hubs split by farthest-
 *                  point sites until the separation drops below cover^-(level+1) times
 *                  the root radius; hubs of at most leaf_size points or radius at most
 *                  FLT_EPSILON become leaves, and a leaf hub of several points gets one
 *                  zero-radius vertex per point)
 *   ghosts         include/point.hpp:762-929 at one rank (a tree over the slot-0 points
 *                  of the non-empty cells with leaf size 1; each point q with distance dq
 *                  to its own landmark queries it at dq + 2r; a found cell that does not
 *                  hold q takes q as a ghost when CoverTree::has_radius_neighbor,
 *                  include/search.hpp:343-381, finds a point of the cell within r)
 *   neighbours     drivers/landmark.cpp:203-210 (per cell: tree over the cell, then
 *                  CoverTree::radius_query_batched, include/search.hpp:267-340, of the
 *                  cell's own points and of its ghosts)
 *   graph          include/graph.hpp:59-116 (edges sorted and deduplicated; kept here as
 *                  unordered pairs u < v)
 * Distances are orc_l2seq (drivers/systolic.cpp:253-269) for float rows, or orc_edit
 * (drivers/systolic.cpp:271-299) for strings (orc_landmark_edit: the driver's `-D edit`
 * path; the trees, ghosts and queries only see the metric).  Cells run in parallel on the
 * host threads, largest first (RNNG's ranks take cells by the same longest-first rule,
 * include/point.hpp:596-605); the Voronoi and ghost queries run in parallel over points.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#ifdef _OPENMP
#include <omp.h>
#endif

float orc_l2seq(const float* p, const float* q, int64_t d);
float orc_edit(const uint8_t* s, int64_t m, const uint8_t* t, int64_t n);

/* ---------------------------------------------------------------- growable arrays */

typedef struct {
    int64_t* p;
    int64_t n, cap;
} ivec;

typedef struct {
    float* p;
    int64_t n, cap;
} fvec;

static void iv_push(ivec* a, int64_t x)
{
    if (a->n == a->cap) {
        a->cap = a->cap ? 2 * a->cap : 8;
        a->p = (int64_t*)realloc(a->p, (size_t)a->cap * sizeof(int64_t));
    }
    a->p[a->n++] = x;
}

static void fv_push(fvec* a, float x)
{
    if (a->n == a->cap) {
        a->cap = a->cap ? 2 * a->cap : 8;
        a->p = (float*)realloc(a->p, (size_t)a->cap * sizeof(float));
    }
    a->p[a->n++] = x;
}

static double now_s(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* ---------------------------------------------------------------- point sets */

/* The points and their metric: rows of X (n x d) under orc_l2seq, or, when atoms is set,
 * the strings atoms[offs[i] .. offs[i+1]) under orc_edit (RNNG's two Distance functors,
 * drivers/landmark.cpp:335-383). */
typedef struct {
    const float* X;
    int64_t d;
    const uint8_t* atoms;
    const int64_t* offs;
} metric;

static inline float mdist(const metric* M, int64_t a, int64_t b)
{
    if (M->atoms)
        return orc_edit(M->atoms + M->offs[a], M->offs[a + 1] - M->offs[a], M->atoms + M->offs[b],
                        M->offs[b + 1] - M->offs[b]);
    return orc_l2seq(M->X + a * M->d, M->X + b * M->d, M->d);
}

/* A point set: points named by global row indices (a cell, its ghosts, the centres). */
typedef struct {
    const metric* M;
    const int64_t* rows;
    int64_t n;
} pset;

/* distance between local point i of s and local point j of t */
static inline float D(const pset* s, int64_t i, const pset* t, int64_t j) { return mdist(s->M, s->rows[i], t->rows[j]); }
/* distance between local point i of s and global row q */
static inline float Dq(const pset* s, int64_t i, int64_t q) { return mdist(s->M, s->rows[i], q); }

/* ---------------------------------------------------------------- cover tree */

/* Flattened tree: vertex v has children child[cptr[v] .. cptr[v+1]), centre (a point
 * of the set, local index) and radius. */
typedef struct {
    int64_t nv;
    int64_t* cptr;
    int64_t* child;
    int64_t* center;
    float* radius;
} ctree;

typedef struct {
    ivec ids, cells, sites;
    fvec dists;
    int64_t candidate, vertex, level;
    float radius;
} hub;

typedef struct {
    int64_t center;
    float radius;
    ivec children;
} vtx;

typedef struct {
    vtx* v;
    int64_t n, cap;
} vtxvec;

static int64_t vv_push(vtxvec* a, int64_t center, float radius)
{
    if (a->n == a->cap) {
        a->cap = a->cap ? 2 * a->cap : 16;
        a->v = (vtx*)realloc(a->v, (size_t)a->cap * sizeof(vtx));
    }
    vtx* x = &a->v[a->n];
    x->center = center;
    x->radius = radius;
    memset(&x->children, 0, sizeof(ivec));
    return a->n++;
}

static void hub_free(hub* h)
{
    free(h->ids.p);
    free(h->cells.p);
    free(h->sites.p);
    free(h->dists.p);
}

/* A FIFO of hubs (RNNG's std::deque<Hub>). */
typedef struct {
    hub* h;
    int64_t head, n, cap;
} hubq;

static void hq_push(hubq* q, hub* h)
{
    if (q->head + q->n == q->cap) {
        if (q->head > 0) {
            memmove(q->h, q->h + q->head, (size_t)q->n * sizeof(hub));
            q->head = 0;
        }
        if (q->n == q->cap) {
            q->cap = q->cap ? 2 * q->cap : 16;
            q->h = (hub*)realloc(q->h, (size_t)q->cap * sizeof(hub));
        }
    }
    q->h[q->head + q->n++] = *h;
}

static void ctree_build(ctree* t, const pset* s, float cover, int64_t leaf_size)
{
    memset(t, 0, sizeof(*t));
    const int64_t n = s->n;
    if (n == 0) return;
    vtxvec verts = {0};
    hubq q = {0};
    hub root;
    memset(&root, 0, sizeof(root));
    iv_push(&root.sites, 0);
    root.radius = 0.0f;
    root.candidate = 0;
    for (int64_t i = 0; i < n; ++i) {
        const float di = D(s, 0, s, i);
        iv_push(&root.ids, i);
        iv_push(&root.cells, 0);
        fv_push(&root.dists, di);
        if (di > root.radius) {
            root.radius = di;
            root.candidate = i;
        }
    }
    const float maxdist = root.radius;
    root.vertex = vv_push(&verts, 0, root.radius);
    hq_push(&q, &root);
    while (q.n > 0) {
        hub h = q.h[q.head++];
        q.n--;
        /* split: farthest-point sites until the separation is below the level's target */
        const int64_t m = h.ids.n;
        const float target = (float)(pow((double)cover, -(double)h.level - 1.0) * (double)maxdist);
        float sep;
        do {
            const int64_t nc = h.candidate;
            iv_push(&h.sites, nc);
            h.candidate = 0;
            sep = 0.0f;
            for (int64_t j = 0; j < m; ++j) {
                const float dj = D(s, nc, s, h.ids.p[j]);
                if (dj < h.dists.p[j]) {
                    h.dists.p[j] = dj;
                    h.cells.p[j] = nc;
                }
                if (h.dists.p[j] > sep) {
                    sep = h.dists.p[j];
                    h.candidate = h.ids.p[j];
                }
            }
        } while (sep > target);
        /* children: the members of each site, in site order; small or tight ones are leaves */
        hub* kids = (hub*)calloc((size_t)h.sites.n, sizeof(hub));
        char* is_leaf = (char*)calloc((size_t)h.sites.n, 1);
        for (int64_t si = 0; si < h.sites.n; ++si) {
            const int64_t site = h.sites.p[si];
            hub* c = &kids[si];
            int64_t rel = 0;
            for (int64_t j = 0; j < m; ++j) {
                if (h.cells.p[j] != site) continue;
                iv_push(&c->ids, h.ids.p[j]);
                iv_push(&c->cells, site);
                fv_push(&c->dists, h.dists.p[j]);
                if (c->dists.p[c->dists.n - 1] > c->dists.p[rel]) rel = c->dists.n - 1;
            }
            iv_push(&c->sites, site);
            c->candidate = c->ids.n ? c->ids.p[rel] : site;
            c->radius = c->ids.n ? c->dists.p[rel] : 0.0f;
            c->level = h.level + 1;
            is_leaf[si] = (c->ids.n <= leaf_size || c->radius <= FLT_EPSILON);
        }
        for (int64_t si = 0; si < h.sites.n; ++si) {
            if (is_leaf[si]) continue;
            const int64_t vid = vv_push(&verts, kids[si].sites.p[0], kids[si].radius);
            kids[si].vertex = vid;
            iv_push(&verts.v[h.vertex].children, vid);
            hq_push(&q, &kids[si]);
        }
        for (int64_t si = 0; si < h.sites.n; ++si) {
            if (!is_leaf[si]) continue;
            const int64_t vid = vv_push(&verts, kids[si].sites.p[0], kids[si].radius);
            iv_push(&verts.v[h.vertex].children, vid);
            if (kids[si].ids.n > 1)
                for (int64_t j = 0; j < kids[si].ids.n; ++j) {
                    const int64_t lv = vv_push(&verts, kids[si].ids.p[j], 0.0f);
                    iv_push(&verts.v[vid].children, lv);
                }
            hub_free(&kids[si]);
        }
        free(kids);
        free(is_leaf);
        hub_free(&h);
    }
    free(q.h);
    /* flatten (the vertex order only changes the traversal order, not what is found) */
    t->nv = verts.n;
    t->cptr = (int64_t*)malloc((size_t)(verts.n + 1) * sizeof(int64_t));
    t->child = (int64_t*)malloc((size_t)(verts.n > 1 ? verts.n - 1 : 1) * sizeof(int64_t));
    t->center = (int64_t*)malloc((size_t)verts.n * sizeof(int64_t));
    t->radius = (float*)malloc((size_t)verts.n * sizeof(float));
    int64_t k = 0;
    for (int64_t v = 0; v < verts.n; ++v) {
        t->cptr[v] = k;
        t->center[v] = verts.v[v].center;
        t->radius[v] = verts.v[v].radius;
        for (int64_t j = 0; j < verts.v[v].children.n; ++j) t->child[k++] = verts.v[v].children.p[j];
        free(verts.v[v].children.p);
    }
    t->cptr[verts.n] = k;
    free(verts.v);
}

static void ctree_free(ctree* t)
{
    free(t->cptr);
    free(t->child);
    free(t->center);
    free(t->radius);
}

/* FIFO of vertex ids for the single-point queries. */
typedef struct {
    int64_t* p;
    int64_t head, n, cap;
} iq;

static void iq_push(iq* q, int64_t x)
{
    if (q->head + q->n == q->cap) {
        if (q->head > 0) {
            memmove(q->p, q->p + q->head, (size_t)q->n * sizeof(int64_t));
            q->head = 0;
        }
        if (q->n == q->cap) {
            q->cap = q->cap ? 2 * q->cap : 64;
            q->p = (int64_t*)realloc(q->p, (size_t)q->cap * sizeof(int64_t));
        }
    }
    q->p[q->head + q->n++] = x;
}

static int64_t iq_pop(iq* q)
{
    q->n--;
    return q->p[q->head++];
}

/* CoverTree::radius_query: every point within r of the query (a global row), appended to
 * out (local ids). */
static void ctree_query(const ctree* t, const pset* s, int64_t query, float r, ivec* out, iq* q)
{
    if (s->n == 0) return;
    q->head = q->n = 0;
    iq_push(q, 0);
    while (q->n > 0) {
        const int64_t u = iq_pop(q);
        if (t->cptr[u] == t->cptr[u + 1]) {
            if (Dq(s, t->center[u], query) <= r) iv_push(out, t->center[u]);
            continue;
        }
        for (int64_t k = t->cptr[u]; k < t->cptr[u + 1]; ++k) {
            const int64_t c = t->child[k];
            if (Dq(s, t->center[c], query) <= t->radius[c] + r) iq_push(q, c);
        }
    }
}

/* CoverTree::has_radius_neighbor: breadth first, stops at the first point within r. */
static int ctree_has_neighbor(const ctree* t, const pset* s, int64_t query, float r, iq* q)
{
    if (s->n == 0) return 0;
    q->head = q->n = 0;
    iq_push(q, 0);
    while (q->n > 0) {
        const int64_t u = iq_pop(q);
        if (t->cptr[u] == t->cptr[u + 1]) {
            if (Dq(s, t->center[u], query) <= r) return 1;
            continue;
        }
        for (int64_t k = t->cptr[u]; k < t->cptr[u + 1]; ++k) {
            const int64_t c = t->child[k];
            if (Dq(s, t->center[c], query) <= t->radius[c] + r) iq_push(q, c);
        }
    }
    return 0;
}

/* Edges of one thread. */
typedef struct {
    ivec u, v;
    fvec w;
} ebuf;

/* CoverTree::radius_query_batched: the batch carried down the tree as id lists; at a
 * leaf every listed query is tested.  Each pair is found from both sides (a point of the
 * cell queried by its own cell's tree, or as a ghost of the other point's cell); it is
 * kept as (smaller id, larger id) and the graph step removes the repeat, as RNNG's Graph
 * removes repeated tuples. */
static void ctree_query_batched(const ctree* t, const pset* s, const pset* batch, float r, ebuf* out)
{
    if (s->n == 0 || batch->n == 0) return;
    /* depth-first over (vertex, id list): visits the same (vertex, query) pairs as RNNG's
     * breadth-first queue */
    typedef struct {
        int64_t u;
        int64_t* ids;
        int64_t n;
    } item;
    item* stack = NULL;
    int64_t sn = 0, scap = 0;
    int64_t* all = (int64_t*)malloc((size_t)batch->n * sizeof(int64_t));
    for (int64_t i = 0; i < batch->n; ++i) all[i] = i;
    scap = 64;
    stack = (item*)malloc((size_t)scap * sizeof(item));
    stack[sn++] = (item){0, all, batch->n};
    while (sn > 0) {
        item it = stack[--sn];
        if (t->cptr[it.u] == t->cptr[it.u + 1]) {
            const int64_t leaf = t->center[it.u];
            const int64_t pid = s->rows[leaf];
            for (int64_t k = 0; k < it.n; ++k) {
                const int64_t qi = it.ids[k];
                const float dist = D(s, leaf, batch, qi);
                const int64_t qid = batch->rows[qi];
                if (dist <= r && qid != pid) {
                    iv_push(&out->u, qid < pid ? qid : pid);
                    iv_push(&out->v, qid < pid ? pid : qid);
                    fv_push(&out->w, dist);
                }
            }
        } else {
            for (int64_t k = t->cptr[it.u]; k < t->cptr[it.u + 1]; ++k) {
                const int64_t c = t->child[k];
                const float eps = t->radius[c] + r;
                const int64_t pc = t->center[c];
                int64_t* keep = (int64_t*)malloc((size_t)it.n * sizeof(int64_t));
                int64_t nk = 0;
                for (int64_t j = 0; j < it.n; ++j)
                    if (D(s, pc, batch, it.ids[j]) <= eps) keep[nk++] = it.ids[j];
                if (nk == 0) {
                    free(keep);
                    continue;
                }
                if (sn == scap) {
                    scap *= 2;
                    stack = (item*)realloc(stack, (size_t)scap * sizeof(item));
                }
                stack[sn++] = (item){c, keep, nk};
            }
        }
        free(it.ids);
    }
    free(stack);
}

/* ---------------------------------------------------------------- the pipeline */

typedef struct {
    int64_t* rows;  /* cell points (global rows), landmark's row in slot 0 when present */
    float* dist;    /* distance to the landmark */
    int64_t n;
    ivec ghosts;
} cell_t;

static int cmp_size_desc(const void* a, const void* b, void* ctx)
{
    const cell_t* c = (const cell_t*)ctx;
    const int64_t x = c[*(const int64_t*)a].n, y = c[*(const int64_t*)b].n;
    return (x < y) - (x > y);
}

/* sort cell indices by size, largest first (insertion of qsort_r-free merge sort) */
static void sort_cells(int64_t* idx, int64_t m, const cell_t* cells)
{
    int64_t* tmp = (int64_t*)malloc((size_t)m * sizeof(int64_t));
    for (int64_t w = 1; w < m; w *= 2)
        for (int64_t lo = 0; lo < m; lo += 2 * w) {
            int64_t mid = lo + w < m ? lo + w : m, hi = lo + 2 * w < m ? lo + 2 * w : m;
            int64_t i = lo, j = mid, k = lo;
            while (i < mid && j < hi)
                tmp[k++] = (cmp_size_desc(&idx[j], &idx[i], (void*)cells) < 0) ? idx[j++] : idx[i++];
            while (i < mid) tmp[k++] = idx[i++];
            while (j < hi) tmp[k++] = idx[j++];
            memcpy(idx + lo, tmp + lo, (size_t)(hi - lo) * sizeof(int64_t));
        }
    free(tmp);
}

static int cmp_edge(const void* a, const void* b)
{
    const int64_t* x = (const int64_t*)a;
    const int64_t* y = (const int64_t*)b;
    if (x[0] != y[0]) return x[0] < y[0] ? -1 : 1;
    if (x[1] != y[1]) return x[1] < y[1] ? -1 : 1;
    return 0;
}

/*
 * The epsilon graph of X (n x d) by RNNG's landmark pipeline: unordered edges u < v,
 * sorted.  phase_s[0..4] receive the seconds of: landmarks + Voronoi, cells, ghosts
 * (cell trees, centre tree, queries), neighbours (per-cell trees and batched queries),
 * graph (sort and unique).  stats[0..3]: cells, ghosts, host threads, empty cells.
 * With empty cells (identical landmarks: the last of equal distances takes every point)
 * RNNG indexes cells by the position of the non-empty ones in its ghost step, so ghosts
 * can land in the wrong cells and edges between cells go missing; this port keeps that
 * behaviour.
 */
static int64_t landmark_core(const metric* M, int64_t n, float radius, int64_t num_centers, float cover,
                             int64_t leaf_size, uint64_t seed, int64_t** ou, int64_t** ov, float** ow, double* phase_s,
                             int64_t* stats)
{
    double t0 = now_s();
    const int nt0 =
#ifdef _OPENMP
        omp_get_max_threads();
#else
        1;
#endif
    if (num_centers < 1) num_centers = 1;
    if (num_centers > n) num_centers = n;
    /* landmarks: a seeded draw of num_centers distinct rows, in increasing row order */
    int64_t* perm = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    for (int64_t i = 0; i < n; ++i) perm[i] = i;
    uint64_t st = seed * 6364136223846793005ull + 1442695040888963407ull;
    for (int64_t i = 0; i < num_centers; ++i) {
        st = st * 6364136223846793005ull + 1442695040888963407ull;
        const int64_t j = i + (int64_t)((st >> 11) % (uint64_t)(n - i));
        const int64_t t = perm[i];
        perm[i] = perm[j];
        perm[j] = t;
    }
    int64_t* lm = perm;  /* first num_centers entries */
    {
        /* increasing row order, as selection sampling yields */
        for (int64_t i = 1; i < num_centers; ++i) {
            int64_t x = lm[i], k = i - 1;
            while (k >= 0 && lm[k] > x) {
                lm[k + 1] = lm[k];
                --k;
            }
            lm[k + 1] = x;
        }
    }
    /* Voronoi: nearest landmark, last of equal wins */
    int64_t* cell_of = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    float* dist_of = (float*)malloc((size_t)(n > 0 ? n : 1) * sizeof(float));
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        float best = FLT_MAX;
        int64_t bc = 0;
        for (int64_t c = 0; c < num_centers; ++c) {
            const float dc = mdist(M, lm[c], i);
            if (dc <= best) {
                best = dc;
                bc = c;
            }
        }
        cell_of[i] = bc;
        dist_of[i] = best;
    }
    double t1 = now_s();
    /* cells: rows in row order, the landmark's row in slot 0 */
    cell_t* cells = (cell_t*)calloc((size_t)num_centers, sizeof(cell_t));
    int64_t* cnt = (int64_t*)calloc((size_t)num_centers + 1, sizeof(int64_t));
    for (int64_t i = 0; i < n; ++i) cnt[cell_of[i]]++;
    for (int64_t c = 0; c < num_centers; ++c) {
        cells[c].rows = (int64_t*)malloc((size_t)(cnt[c] ? cnt[c] : 1) * sizeof(int64_t));
        cells[c].dist = (float*)malloc((size_t)(cnt[c] ? cnt[c] : 1) * sizeof(float));
    }
    for (int64_t i = 0; i < n; ++i) {
        cell_t* c = &cells[cell_of[i]];
        c->rows[c->n] = i;
        c->dist[c->n] = dist_of[i];
        c->n++;
    }
    for (int64_t c = 0; c < num_centers; ++c)
        for (int64_t k = 0; k < cells[c].n; ++k)
            if (cells[c].rows[k] == lm[c]) {
                int64_t tr = cells[c].rows[0];
                cells[c].rows[0] = cells[c].rows[k];
                cells[c].rows[k] = tr;
                float td = cells[c].dist[0];
                cells[c].dist[0] = cells[c].dist[k];
                cells[c].dist[k] = td;
                break;
            }
    double t2 = now_s();
    /* ghosts: trees per cell, a tree over the non-empty cells' slot-0 points */
    ctree* trees = (ctree*)calloc((size_t)num_centers, sizeof(ctree));
    pset* sets = (pset*)calloc((size_t)num_centers, sizeof(pset));
    int64_t* order = (int64_t*)malloc((size_t)num_centers * sizeof(int64_t));
    for (int64_t c = 0; c < num_centers; ++c) {
        order[c] = c;
        sets[c] = (pset){M, cells[c].rows, cells[c].n};
    }
    sort_cells(order, num_centers, cells);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t k = 0; k < num_centers; ++k) ctree_build(&trees[order[k]], &sets[order[k]], cover, leaf_size);
    int64_t* slot0 = (int64_t*)malloc((size_t)num_centers * sizeof(int64_t));
    int64_t nne = 0;
    for (int64_t c = 0; c < num_centers; ++c)
        if (cells[c].n > 0) slot0[nne++] = cells[c].rows[0];
    pset centres = {M, slot0, nne};
    ctree ctr;
    ctree_build(&ctr, &centres, cover, 1);
    /* every point in cell order, with its own cell (the cell index of RNNG's sendbuf) */
    int64_t* qrow = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    int64_t* qcell = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    float* qdist = (float*)malloc((size_t)(n > 0 ? n : 1) * sizeof(float));
    {
        int64_t k = 0;
        for (int64_t c = 0; c < num_centers; ++c)
            for (int64_t j = 0; j < cells[c].n; ++j) {
                qrow[k] = cells[c].rows[j];
                qcell[k] = c;
                qdist[k] = cells[c].dist[j];
                ++k;
            }
    }
    /* per point: the cells that take it as a ghost (cells indexed by non-empty position,
     * as RNNG's centre ids are) */
    ivec* gl = (ivec*)calloc((size_t)(n > 0 ? n : 1), sizeof(ivec));
    const float two_r = 2.0f * radius;
#pragma omp parallel
    {
        ivec found = {0};
        iq q = {0};
#pragma omp for schedule(dynamic, 256)
        for (int64_t k = 0; k < n; ++k) {
            const int64_t xq = qrow[k];
            found.n = 0;
            ctree_query(&ctr, &centres, xq, qdist[k] + two_r, &found, &q);
            for (int64_t j = 0; j < found.n; ++j) {
                const int64_t c = found.p[j];
                /* c counts non-empty cells; RNNG uses it as a cell index (see above) */
                if (c >= num_centers || cells[c].n == 0 || c == qcell[k]) continue;
                int dup = 0;
                for (int64_t t = 0; t < gl[k].n; ++t) dup |= gl[k].p[t] == c;
                if (dup) continue;
                if (ctree_has_neighbor(&trees[c], &sets[c], xq, radius, &q)) iv_push(&gl[k], c);
            }
        }
        free(found.p);
        free(q.p);
    }
    int64_t nghost = 0;
    for (int64_t k = 0; k < n; ++k) {
        for (int64_t j = 0; j < gl[k].n; ++j) iv_push(&cells[gl[k].p[j]].ghosts, qrow[k]);
        nghost += gl[k].n;
        free(gl[k].p);
    }
    free(gl);
    double t3 = now_s();
    /* neighbours: per cell, its tree queried by its points and by its ghosts */
    ebuf* eb = (ebuf*)calloc((size_t)nt0, sizeof(ebuf));
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t k = 0; k < num_centers; ++k) {
        const int64_t c = order[k];
        if (cells[c].n == 0) continue;
        const int tid =
#ifdef _OPENMP
            omp_get_thread_num();
#else
            0;
#endif
        pset gh = {M, cells[c].ghosts.p, cells[c].ghosts.n};
        ctree_query_batched(&trees[c], &sets[c], &sets[c], radius, &eb[tid]);
        ctree_query_batched(&trees[c], &sets[c], &gh, radius, &eb[tid]);
    }
    double t4 = now_s();
    /* graph: one sorted list of unordered edges */
    int64_t m = 0;
    for (int t = 0; t < nt0; ++t) m += eb[t].u.n;
    typedef struct {
        int64_t u, v;
        float w;
        float pad;
    } rec;
    rec* all = (rec*)malloc((size_t)(m > 0 ? m : 1) * sizeof(rec));
    int64_t k = 0;
    for (int t = 0; t < nt0; ++t) {
        for (int64_t j = 0; j < eb[t].u.n; ++j) all[k++] = (rec){eb[t].u.p[j], eb[t].v.p[j], eb[t].w.p[j], 0.0f};
        free(eb[t].u.p);
        free(eb[t].v.p);
        free(eb[t].w.p);
    }
    free(eb);
    qsort(all, (size_t)m, sizeof(rec), cmp_edge);
    int64_t mu = 0;
    for (int64_t j = 0; j < m; ++j)
        if (mu == 0 || all[j].u != all[mu - 1].u || all[j].v != all[mu - 1].v) all[mu++] = all[j];
    *ou = (int64_t*)malloc((size_t)(mu > 0 ? mu : 1) * sizeof(int64_t));
    *ov = (int64_t*)malloc((size_t)(mu > 0 ? mu : 1) * sizeof(int64_t));
    *ow = (float*)malloc((size_t)(mu > 0 ? mu : 1) * sizeof(float));
    for (int64_t j = 0; j < mu; ++j) {
        (*ou)[j] = all[j].u;
        (*ov)[j] = all[j].v;
        (*ow)[j] = all[j].w;
    }
    free(all);
    double t5 = now_s();
    if (phase_s) {
        phase_s[0] = t1 - t0;
        phase_s[1] = t2 - t1;
        phase_s[2] = t3 - t2;
        phase_s[3] = t4 - t3;
        phase_s[4] = t5 - t4;
    }
    if (stats) {
        stats[0] = num_centers;
        stats[1] = nghost;
        stats[2] = nt0;
        stats[3] = num_centers - nne;
    }
    for (int64_t c = 0; c < num_centers; ++c) {
        ctree_free(&trees[c]);
        free(cells[c].rows);
        free(cells[c].dist);
        free(cells[c].ghosts.p);
    }
    ctree_free(&ctr);
    free(trees);
    free(sets);
    free(order);
    free(slot0);
    free(cells);
    free(cnt);
    free(qrow);
    free(qcell);
    free(qdist);
    free(cell_of);
    free(dist_of);
    free(perm);
    return mu;
}

int64_t orc_landmark_l2(const float* X, int64_t n, int64_t d, float radius, int64_t num_centers, float cover,
                        int64_t leaf_size, uint64_t seed, int64_t** ou, int64_t** ov, float** ow, double* phase_s,
                        int64_t* stats)
{
    const metric M = {X, d, NULL, NULL};
    return landmark_core(&M, n, radius, num_centers, cover, leaf_size, seed, ou, ov, ow, phase_s, stats);
}

/* The same pipeline over strings under RNNG's edit distance (the driver's `-D edit` path,
 * drivers/landmark.cpp:61-62). */
int64_t orc_landmark_edit(const uint8_t* atoms, const int64_t* offsets, int64_t n, float radius, int64_t num_centers,
                          float cover, int64_t leaf_size, uint64_t seed, int64_t** ou, int64_t** ov, float** ow,
                          double* phase_s, int64_t* stats)
{
    const metric M = {NULL, 0, atoms, offsets};
    return landmark_core(&M, n, radius, num_centers, cover, leaf_size, seed, ou, ov, ow, phase_s, stats);
}
