// Drop-in radius search with the interface of RNNG's include/search.h (Search, BruteForce,
// CoverTree).  No tree is built: a search answers from the epsilon graph of its point
// set, computed once per (point set, radius) on the GPU by the C ABI
// (include/rnng_gpu.h), or from the whole-set graph that VoronoiDiagram's ghost step
// already computed when it holds every point involved (same ids, same atoms).  The
// functor sees exactly RNNG's pairs: every indexed point p with distance(p, q) <= radius,
// called as functor(p, q, dist) with p's container offset and RNNG's float distance.
// Only the order of the calls differs from a tree walk.
//
// The caller's Distance functor is not called: float atoms use RNNG's L2, char atoms
// RNNG's edit distance, both evaluated on the GPU with bit-identical results
// (drivers/landmark.cpp:335-383).
#ifndef RNNG_DROPIN_SEARCH_H_
#define RNNG_DROPIN_SEARCH_H_

#include <memory>

#include "point.h"
#include "utils.h"

namespace rnng_dropin {

// Graph row -> offset in a search's container: a table when the container covers much
// of the graph, a hash map when it is a small part of it (one Voronoi cell).
struct LocalIndex {
    IndexVector dense;
    FlatIndexMap sparse;
    bool use_dense = false;

    void build(const IndexVector& rows, Index graph_rows)
    {
        use_dense = (Index)rows.size() * 16 >= graph_rows;
        if (use_dense) {
            dense.assign(graph_rows, -1);
            for (Index i = 0; i < (Index)rows.size(); ++i) dense[rows[i]] = i;
        } else {
            sparse.reserve(rows.size());
            for (Index i = 0; i < (Index)rows.size(); ++i) sparse.emplace(rows[i], i);
        }
    }

    Index operator[](Index row) const
    {
        if (use_dense) return dense[row];
        return sparse.find(row);
    }
};

// What one search object needs for one (point set, radius): the graph it reads and
// the map from the graph's rows to the search's own container offsets.
template <class Atom>
struct SearchPlan {
    const PointContainer<Atom>* points = nullptr;
    Index num_points = -1;
    Real radius = 0;
    std::shared_ptr<const GraphCache<Atom>> graph;
    LocalIndex local_of_graph;
};

template <class Atom>
std::shared_ptr<SearchPlan<Atom>> make_plan(const PointContainer<Atom>& points, Real radius)
{
    auto plan = std::make_shared<SearchPlan<Atom>>();
    plan->points = &points;
    plan->num_points = points.num_points();
    plan->radius = radius;
    std::shared_ptr<const GraphCache<Atom>> g = last_graph<Atom>();
    IndexVector rows;
    if (!(g && g->radius == radius && g->find_all(points, rows))) {
        g = build_graph(points, radius);  // the search's own set, on the GPU
        bool ok = g->find_all(points, rows);
        assert((ok));
    }
    plan->graph = g;
    plan->local_of_graph.build(rows, g->pts.num_points());
    return plan;
}

// Pairs (point offset, query offset, dist) of a batch that is not in the plan's graph:
// one GPU call over the point set and the batch.
template <class Atom>
void direct_pairs(const PointContainer<Atom>& points, const PointContainer<Atom>& batch, Real radius,
                  std::vector<std::tuple<Index, Index, Real>>& out)
{
    out.clear();
    if (points.num_points() == 0 || batch.num_points() == 0) return;
    rnng_edges e;
    if constexpr (std::is_same_v<Atom, float>) {
        const Index d = points.uniform_dim();
        assert((d >= 1 && batch.uniform_dim() == d));
        check(rnng_radius_query_l2(context(), points.atom_data(), nullptr, points.num_points(), batch.atom_data(),
                                   nullptr, batch.num_points(), d, radius, 0, &e),
              "rnng_radius_query_l2");
        for (int64_t k = 0; k < e.count; ++k) out.emplace_back(e.v[k], e.u[k], e.w[k]);
    } else {
        // the epsilon graph of points followed by the batch; keep the pairs that cross
        PointContainer<Atom> both(points, batch);
        const RowEdges g = eps_graph_rows(both, radius);
        const Index n = points.num_points();
        for (size_t k = 0; k < g.u.size(); ++k) {
            const Index a = std::min(g.u[k], g.v[k]), b = std::max(g.u[k], g.v[k]);
            if (a < n && b >= n) out.emplace_back(a, b - n, g.w[k]);
        }
    }
}

// Every indexed point within radius of the query, through the plan's graph; false when
// the query is not in the graph (the caller then asks the GPU directly).
template <class Atom, class Functor>
bool replay(const SearchPlan<Atom>& plan, const Point<Atom>& query, Index& found, const Functor& functor)
{
    const GraphCache<Atom>& g = *plan.graph;
    const Index r = g.find(query);
    if (r < 0) return false;
    const PointContainer<Atom>& points = *plan.points;
    const Index self = plan.local_of_graph[r];
    if (self >= 0 && self_distance_zero(query) && Real(0) <= plan.radius) {
        functor(points[self], query, Real(0));
        ++found;
    }
    for (Index k = g.rowptr[r]; k < g.rowptr[r + 1]; ++k) {
        const Index t = plan.local_of_graph[g.nbr[k]];
        if (t >= 0) {
            functor(points[t], query, g.w[k]);
            ++found;
        }
    }
    return true;
}

// The search state shared by BruteForce and CoverTree.
class RadiusIndex
{
  protected:
    template <class Atom>
    const SearchPlan<Atom>& plan_for(const PointContainer<Atom>& points, Real radius) const
    {
        std::shared_ptr<SearchPlan<Atom>> p = std::static_pointer_cast<SearchPlan<Atom>>(plan);
        if (!p || p->points != &points || p->num_points != points.num_points() || p->radius != radius) {
            p = make_plan(points, radius);
            plan = p;
        }
        return *p;
    }

    template <class Atom, class Functor>
    Index query_one(const PointContainer<Atom>& points, const Point<Atom>& query, Real radius,
                    const Functor& functor) const
    {
        if (points.num_points() == 0) return 0;
        Index found = 0;
        if (replay(plan_for(points, radius), query, found, functor)) return found;
        PointContainer<Atom> one;
        one.push_back(query);
        std::vector<std::tuple<Index, Index, Real>> pairs;
        direct_pairs(points, one, radius, pairs);
        for (const auto& [p, q, dist] : pairs) functor(points[p], query, dist);
        return (Index)pairs.size();
    }

    template <class Atom, class Functor>
    Index query_batch(const PointContainer<Atom>& points, const PointContainer<Atom>& batch, Real radius,
                      const Functor& functor) const
    {
        if (points.num_points() == 0) return 0;
        const SearchPlan<Atom>& p = plan_for(points, radius);
        bool all = true;
        for (Index i = 0; i < batch.num_points() && all; ++i) all = p.graph->find(batch[i]) >= 0;
        Index found = 0;
        if (all) {
            for (Index i = 0; i < batch.num_points(); ++i) replay(p, batch[i], found, functor);
            return found;
        }
        std::vector<std::tuple<Index, Index, Real>> pairs;
        direct_pairs(points, batch, radius, pairs);
        for (const auto& [pi, qi, dist] : pairs) functor(points[pi], batch[qi], dist);
        return (Index)pairs.size();
    }

    void reset() { plan.reset(); }

  private:
    mutable std::shared_ptr<void> plan;
};

}  // namespace rnng_dropin

// CRTP front as RNNG declares it (include/search.h:7-23).
template <class T>
class Search
{
  public:
    template <class Atom, class Distance>
    void build(const PointContainer<Atom>& points, Distance& distance)
    {
        static_cast<T*>(this)->build(points, distance);
    }

    template <class Atom, class Distance, class Functor>
    Index radius_query(const PointContainer<Atom>& points, Distance& distance, const Point<Atom>& query,
                       const Functor& functor) const
    {
        return static_cast<T*>(this)->radius_query(points, distance, query, functor);
    }
};

// Every point within radius (include/search.hpp:383-407).
class BruteForce : public Search<BruteForce>, private rnng_dropin::RadiusIndex
{
  public:
    BruteForce() {}

    template <class Atom, class Distance>
    void build(const PointContainer<Atom>&, Distance&)
    {
        reset();
    }

    template <class Atom, class Distance, class Functor>
    Index radius_query(const PointContainer<Atom>& points, Distance&, const Point<Atom>& query, Real radius,
                       const Functor& functor) const
    {
        return query_one(points, query, radius, functor);
    }
};

// RNNG's cover tree interface (include/search.h:37-73); cover and leaf_size shape RNNG's
// tree and change no result, so they are kept only for the interface.
class CoverTree : public Search<CoverTree>, private rnng_dropin::RadiusIndex
{
  public:
    CoverTree(Real cover = 1.5, Index leaf_size = 1) : cover(cover), leaf_size(leaf_size) {}

    template <class Atom, class Distance>
    void build(const PointContainer<Atom>&, Distance&)
    {
        reset();
    }

    // include/search.hpp:223-264
    template <class Atom, class Distance, class Functor>
    Index radius_query(const PointContainer<Atom>& points, Distance&, const Point<Atom>& query, Real radius,
                       const Functor& functor) const
    {
        return query_one(points, query, radius, functor);
    }

    // include/search.hpp:266-340
    template <class Atom, class Distance, class Functor>
    Index radius_query_batched(const PointContainer<Atom>& points, Distance&, const PointContainer<Atom>& batch,
                               Real radius, const Functor& functor) const
    {
        return query_batch(points, batch, radius, functor);
    }

    // include/search.hpp:342-381
    template <class Atom, class Distance>
    bool has_radius_neighbor(const PointContainer<Atom>& points, Distance&, const Point<Atom>& query,
                             Real radius) const
    {
        bool any = false;
        query_one(points, query, radius, [&](const Point<Atom>&, const Point<Atom>&, Real) { any = true; });
        return any;
    }

  private:
    Real cover;
    Index leaf_size;
};

#endif  // RNNG_DROPIN_SEARCH_H_
