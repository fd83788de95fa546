// Harness that runs RNNG's own CPU path (its headers, compiled from the RNNG source
// tree with the single-rank MPI shim) and dumps the results in binary, so that edge
// weights and filtration values can be compared bit for bit.  RNNG's drivers print
// weights with 6 digits (include/graph.hpp:33, include/simplex.hpp:183), which is
// not enough to prove bit-exactness; this harness makes the same API calls in the
// same order as the drivers and writes the functor arguments instead.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/Makefile into oracle/_ref/, used to make
// the golden fixtures under tests/golden/ and to check the C oracle.
//
// Modes (all single rank):
//   systolic <in.fvecs> <radius> <out>          drivers/systolic.cpp:96-147
//   landmark <l2|edit> <in> <radius> <m> <seed> <out>
//                                                drivers/landmark.cpp:111-210
//   rips <l2|edit> <in> <radius> <maxdim> <m> <seed> <out>
//                                                drivers/rips.cpp:106-180
//   graph <l2|edit> <in> <radius> <m> <seed> <out.mtx>
//                                                drivers/landmark.cpp:111-252: the landmark
//                                                pipeline, Graph + redistribute_edges and the
//                                                driver's text output; phase times on stderr
//   cells <l2|edit> <in> <radius> <m> <seed> <rips 0|1> <out>
//                                                drivers/landmark.cpp:111-175 and
//                                                drivers/rips.cpp:106-162: the Voronoi
//                                                cells after coalescing and ghosts
// Edge output: int64 count, then count int64 u, count int64 v, count float32 w
// (u = query id, v = indexed id, as the drivers' functors record them).
// Simplex output: int64 count, count int64 ids, count float32 values.
// Cell output: int64 m, m int64 landmark rows, int64 cell count, then per cell: int64 cell id, int64 np, np int64 point
// ids, np float32 distances to the centre, np uint8 interior flags, int64 ng, ng int64
// ghost ids.
#include <mpi.h>

#include "graph.h"
#include "point.h"
#include "search.h"
#include "simplex.h"
#include "utils.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

// Same arithmetic as the drivers' L2Distance<float> (drivers/systolic.cpp:253-269).
template <class Atom>
struct HarnessL2 {
    Real operator()(const Point<Atom>& p, const Point<Atom>& q) const
    {
        Index dim = p.size();
        assert((dim == q.size()));
        Real val = 0;
        for (Index i = 0; i < dim; ++i) {
            Real delta = static_cast<Real>(p[i] - q[i]);
            val += delta * delta;
        }
        return std::sqrt(val);
    }
};

// Same recurrence as the drivers' EditDistance<char> (drivers/systolic.cpp:271-299).
template <class Atom>
struct HarnessEdit {
    Real operator()(const Point<Atom>& s, const Point<Atom>& t) const
    {
        Index m = s.size(), n = t.size();
        IndexVector v0(n + 1), v1(n + 1);
        for (Index i = 0; i <= n; ++i) v0[i] = i;
        for (Index i = 0; i < m; ++i) {
            v1[0] = i + 1;
            for (Index j = 0; j < n; ++j) {
                Index del = v0[j + 1] + 1;
                Index ins = v1[j] + 1;
                Index sub = (s[i] == t[j]) ? v0[j] : v0[j] + 1;
                v1[j + 1] = std::min(del, std::min(ins, sub));
            }
            std::swap(v0, v1);
        }
        return static_cast<Real>(v0[n]);
    }
};

struct EdgeDump {
    std::vector<int64_t> u, v;
    std::vector<float> w;
    void write(const char* path) const
    {
        FILE* f = std::fopen(path, "wb");
        if (!f) { std::perror(path); std::exit(2); }
        int64_t n = (int64_t)u.size();
        std::fwrite(&n, sizeof(n), 1, f);
        std::fwrite(u.data(), sizeof(int64_t), u.size(), f);
        std::fwrite(v.data(), sizeof(int64_t), v.size(), f);
        std::fwrite(w.data(), sizeof(float), w.size(), f);
        std::fclose(f);
    }
};

static int run_systolic(const char* in, Real radius, const char* out)
{
    MPI_Comm comm = MPI_COMM_WORLD;
    PointContainer<float> points;
    points.read_fvecs(in, comm);
    HarnessL2<float> distance;
    CoverTree tree(1.5, 10);
    tree.build(points, distance);
    EdgeDump dump;
    auto functor = [&](const Point<float>& p, const Point<float>& q, Real dist) {
        dump.u.push_back(q.id());
        dump.v.push_back(p.id());
        dump.w.push_back(dist);
    };
    PointContainer<float> queries = points;
    for (Index i = 0; i < queries.num_points(); ++i) tree.radius_query(points, distance, queries[i], radius, functor);
    dump.write(out);
    return 0;
}

template <class Atom, class Distance>
static int run_landmark(const char* in, Real radius, Index m, int seed, const char* out)
{
    MPI_Comm comm = MPI_COMM_WORLD;
    PointContainer<Atom> points;
    Index n;
    if constexpr (std::is_same_v<Atom, char>) n = points.read_seqs(in, comm);
    else n = points.read_fvecs(in, comm);
    assert((m <= n));
    IndexVector landmarks;
    selection_sample(n, m, landmarks, seed);
    PointContainer<Atom> mycenters, centers;
    mycenters.indexed_gather(points, landmarks);
    centers.allgather(mycenters, comm);
    Distance distance;
    VoronoiDiagram<Atom> diagram(points, centers, distance);
    std::vector<VoronoiCell<Atom>> cells;
    diagram.coalesce_cells(cells, comm);
    diagram.add_ghost_points_systolic(cells, distance, radius, 1.5, 10, comm);
    EdgeDump dump;
    auto functor = [&](const Point<Atom>& p, const Point<Atom>& q, Real dist) {
        dump.u.push_back(q.id());
        dump.v.push_back(p.id());
        dump.w.push_back(dist);
    };
    for (const VoronoiCell<Atom>& cell : cells) {
        CoverTree tree(1.5, 10);
        tree.build(cell, distance);
        tree.radius_query_batched(cell, distance, cell, radius, functor);
        tree.radius_query_batched(cell, distance, cell.ghosts(), radius, functor);
    }
    dump.write(out);
    return 0;
}

template <class Atom, class Distance>
static int run_graph(const char* in, Real radius, Index m, int seed, const char* out)
{
    MPI_Comm comm = MPI_COMM_WORLD;
    double t = -MPI_Wtime();
    auto phase = [&](const char* what) {
        t += MPI_Wtime();
        std::fprintf(stderr, "[phase %.6f] %s\n", t, what);
        t = -MPI_Wtime();
    };
    PointContainer<Atom> points;
    Index n;
    if constexpr (std::is_same_v<Atom, char>) n = points.read_seqs(in, comm);
    else n = points.read_fvecs(in, comm);
    assert((m <= n));
    phase("read input");
    IndexVector landmarks;
    selection_sample(n, m, landmarks, seed);
    PointContainer<Atom> mycenters, centers;
    mycenters.indexed_gather(points, landmarks);
    centers.allgather(mycenters, comm);
    Distance distance;
    VoronoiDiagram<Atom> diagram(points, centers, distance);
    phase("voronoi");
    std::vector<VoronoiCell<Atom>> cells;
    diagram.coalesce_cells(cells, comm);
    phase("coalesce cells");
    diagram.add_ghost_points_systolic(cells, distance, radius, 1.5, 10, comm);
    phase("ghost points");
    using Edge = std::tuple<Index, Index, Real>;
    std::vector<Edge> edges;
    auto functor = [&](const Point<Atom>& p, const Point<Atom>& q, Real dist) { edges.emplace_back(q.id(), p.id(), dist); };
    for (const VoronoiCell<Atom>& cell : cells) {
        CoverTree tree(1.5, 10);
        tree.build(cell, distance);
        tree.radius_query_batched(cell, distance, cell, radius, functor);
        tree.radius_query_batched(cell, distance, cell.ghosts(), radius, functor);
    }
    phase("found neighbors");
    Graph graph(edges, n);
    graph.redistribute_edges(comm);
    phase("redistributed edges");
    std::fprintf(stderr, "edges=%lld\n", (long long)graph.num_edges());
    graph.write_file(out, comm);
    phase("wrote edges");
    return 0;
}

template <class Atom>
static Index read_points(PointContainer<Atom>& points, const char* in, MPI_Comm comm)
{
    if constexpr (std::is_same_v<Atom, char>) return points.read_seqs(in, comm);
    else return points.read_fvecs(in, comm);
}

template <class Atom, class Distance>
static int run_rips(const char* in, Real radius, Index maxdim, Index m, int seed, const char* out)
{
    MPI_Comm comm = MPI_COMM_WORLD;
    Distance distance;
    PointContainer<Atom> points;
    const Index n = read_points(points, in, comm);
    IndexVector landmarks;
    selection_sample(n, m, landmarks, seed);
    PointContainer<Atom> mycenters, centers;
    mycenters.indexed_gather(points, landmarks);
    centers.allgather(mycenters, comm);
    VoronoiDiagram<Atom> diagram(points, centers, distance);
    std::vector<VoronoiCell<Atom>> cells;
    diagram.coalesce_cells(cells, comm);
    diagram.add_ghost_points_systolic_rips(cells, distance, radius, 1.5, 10, comm);
    std::vector<int64_t> ids;
    std::vector<float> values;
    for (const VoronoiCell<Atom>& cell : cells) {
        VoronoiComplex<Atom> vc(cell, radius, maxdim);
        vc.build_filtration(distance, n, 1.5, 10);
        for (auto it = vc.begin(); it != vc.end(); ++it) {
            ids.push_back(it->getid());
            values.push_back(it->getvalue());
        }
    }
    FILE* f = std::fopen(out, "wb");
    if (!f) { std::perror(out); return 2; }
    int64_t cnt = (int64_t)ids.size();
    std::fwrite(&cnt, sizeof(cnt), 1, f);
    std::fwrite(ids.data(), sizeof(int64_t), ids.size(), f);
    std::fwrite(values.data(), sizeof(float), values.size(), f);
    std::fclose(f);
    return 0;
}

template <class Atom, class Distance>
static int run_cells(const char* in, Real radius, Index m, int seed, bool rips, const char* out)
{
    MPI_Comm comm = MPI_COMM_WORLD;
    Distance distance;
    PointContainer<Atom> points;
    const Index n = read_points(points, in, comm);
    assert((m <= n));
    IndexVector landmarks;
    selection_sample(n, m, landmarks, seed);
    PointContainer<Atom> mycenters, centers;
    mycenters.indexed_gather(points, landmarks);
    centers.allgather(mycenters, comm);
    VoronoiDiagram<Atom> diagram(points, centers, distance);
    std::vector<VoronoiCell<Atom>> cells;
    diagram.coalesce_cells(cells, comm);
    if (rips) diagram.add_ghost_points_systolic_rips(cells, distance, radius, 1.5, 10, comm);
    else diagram.add_ghost_points_systolic(cells, distance, radius, 1.5, 10, comm);
    FILE* f = std::fopen(out, "wb");
    if (!f) { std::perror(out); return 2; }
    auto put = [&](int64_t x) { std::fwrite(&x, sizeof(x), 1, f); };
    put((int64_t)landmarks.size());
    for (Index l : landmarks) put(l);
    put((int64_t)cells.size());
    for (const VoronoiCell<Atom>& cell : cells) {
        put(cell.id());
        put(cell.num_points());
        for (Index i = 0; i < cell.num_points(); ++i) put(cell[i].id());
        for (Index i = 0; i < cell.num_points(); ++i) {
            const float d = cell.dist_to_center(i);
            std::fwrite(&d, sizeof(d), 1, f);
        }
        for (Index i = 0; i < cell.num_points(); ++i) {
            const uint8_t b = cell.interiors()[i] ? 1 : 0;
            std::fwrite(&b, 1, 1, f);
        }
        put(cell.num_ghosts());
        for (Index i = 0; i < cell.num_ghosts(); ++i) put(cell.ghost(i).id());
    }
    std::fclose(f);
    return 0;
}

int main(int argc, char** argv)
{
    MPI_Init(&argc, &argv);
    int rc = 1;
    if (argc == 5 && !std::strcmp(argv[1], "systolic")) {
        rc = run_systolic(argv[2], (Real)std::atof(argv[3]), argv[4]);
    } else if (argc == 8 && !std::strcmp(argv[1], "landmark")) {
        Real r = (Real)std::atof(argv[4]);
        Index m = std::atoll(argv[5]);
        int seed = std::atoi(argv[6]);
        if (!std::strcmp(argv[2], "edit")) rc = run_landmark<char, HarnessEdit<char>>(argv[3], r, m, seed, argv[7]);
        else rc = run_landmark<float, HarnessL2<float>>(argv[3], r, m, seed, argv[7]);
    } else if (argc == 8 && !std::strcmp(argv[1], "graph")) {
        Real r = (Real)std::atof(argv[4]);
        Index m = std::atoll(argv[5]);
        int seed = std::atoi(argv[6]);
        if (!std::strcmp(argv[2], "edit")) rc = run_graph<char, HarnessEdit<char>>(argv[3], r, m, seed, argv[7]);
        else rc = run_graph<float, HarnessL2<float>>(argv[3], r, m, seed, argv[7]);
    } else if (argc == 9 && !std::strcmp(argv[1], "rips")) {
        const Real r = (Real)std::atof(argv[4]);
        const Index maxdim = std::atoll(argv[5]), m = std::atoll(argv[6]);
        const int seed = std::atoi(argv[7]);
        if (!std::strcmp(argv[2], "edit")) rc = run_rips<char, HarnessEdit<char>>(argv[3], r, maxdim, m, seed, argv[8]);
        else rc = run_rips<float, HarnessL2<float>>(argv[3], r, maxdim, m, seed, argv[8]);
    } else if (argc == 9 && !std::strcmp(argv[1], "cells")) {
        const Real r = (Real)std::atof(argv[4]);
        const Index m = std::atoll(argv[5]);
        const int seed = std::atoi(argv[6]);
        const bool rips = std::atoi(argv[7]) != 0;
        if (!std::strcmp(argv[2], "edit")) rc = run_cells<char, HarnessEdit<char>>(argv[3], r, m, seed, rips, argv[8]);
        else rc = run_cells<float, HarnessL2<float>>(argv[3], r, m, seed, rips, argv[8]);
    } else {
        std::fprintf(stderr,
                     "usage: %s systolic <in.fvecs> <radius> <out>\n"
                     "       %s landmark <l2|edit> <in> <radius> <m> <seed> <out>\n"
                     "       %s graph <l2|edit> <in> <radius> <m> <seed> <out.mtx>\n"
                     "       %s rips <l2|edit> <in> <radius> <maxdim> <m> <seed> <out>\n"
                     "       %s cells <l2|edit> <in> <radius> <m> <seed> <rips 0|1> <out>\n",
                     argv[0], argv[0], argv[0], argv[0], argv[0]);
    }
    MPI_Finalize();
    return rc;
}
