// Drop-in edge list with the interface of RNNG's include/graph.h: the edges are sorted
// (RNNG sorts at construction; here before the first write), redistribute_edges gives
// every rank both orientations of its vertices' edges (sorted, duplicates removed; on the
// GPU at one rank), write_file prints a MatrixMarket-like text file.
#ifndef RNNG_DROPIN_GRAPH_H_
#define RNNG_DROPIN_GRAPH_H_

#include <thread>

#include "utils.h"

class Graph
{
  public:
    using Edge = std::tuple<Index, Index, Real>;
    using EdgeVector = std::vector<Edge>;

    // RNNG sorts here; the sort is deferred to the first use that can see the order
    // (write_file), since redistribute_edges sorts again on the GPU anyway.
    Graph(const EdgeVector& edges, Index num_vertices) : edges(edges), num_vertices(num_vertices) {}

    // "% n n m" then "u v w" with w printed "%.6f" (RNNG include/graph.hpp:1-17).
    void write_file(const char* fname) const
    {
        ensure_sorted();
        FILE* f = std::fopen(fname, "w");
        assert((f != nullptr));
        std::fprintf(f, "%% %lld %lld %lld\n", (long long)num_vertices, (long long)num_vertices,
                     (long long)edges.size());
        for (const auto& [u, v, w] : edges) std::fprintf(f, "%lld %lld %.6f\n", (long long)u, (long long)v, w);
        std::fclose(f);
    }

    // Collective version: each rank's text at its offset of one file, the header on
    // rank 0, weights with six significant digits (RNNG include/graph.hpp:20-56).
    void write_file(const char* fname, MPI_Comm comm) const
    {
        ensure_sorted();
        int rank = 0;
        MPI_Comm_rank(comm, &rank);
        Index total = (Index)edges.size();
        MPI_Allreduce(MPI_IN_PLACE, &total, 1, MPI_INDEX, MPI_SUM, comm);
        // The stream's text (ints in decimal, the weight as a double with six significant
        // digits in the %g style of setprecision(6)), formatted with std::to_chars, which is
        // specified to print exactly what printf's %.6g prints, an order of magnitude faster.
        // Each line depends on its edge alone, so large lists are formatted in contiguous
        // blocks on up to 16 host threads and joined in order.
        std::string text;
        if (rank == 0) {
            std::ostringstream head;
            head << "% " << num_vertices << " " << num_vertices << " " << total << "\n";
            text += head.str();
        }
        const size_t m = edges.size();
        const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        const unsigned nt = m >= ((size_t)1 << 20) ? hw : 1u;
        std::vector<std::string> parts(nt);
        auto format_block = [&](unsigned k) {
            const size_t b = m * k / nt, e = m * (k + 1) / nt;
            std::string& out = parts[k];
            out.reserve((e - b) * 24);
            char buf[96];
            for (size_t i = b; i < e; ++i) {
                const auto& [u, v, w] = edges[i];
                char* p = std::to_chars(buf, buf + sizeof(buf), (long long)u).ptr;
                *p++ = ' ';
                p = std::to_chars(p, buf + sizeof(buf), (long long)v).ptr;
                *p++ = ' ';
                p = std::to_chars(p, buf + sizeof(buf), (double)w, std::chars_format::general, 6).ptr;
                *p++ = '\n';
                out.append(buf, (size_t)(p - buf));
            }
        };
        if (nt == 1) {
            format_block(0);
        } else {
            std::vector<std::thread> workers;
            for (unsigned k = 0; k < nt; ++k) workers.emplace_back(format_block, k);
            for (auto& t : workers) t.join();
        }
        size_t bytes = text.size();
        for (const auto& part : parts) bytes += part.size();
        text.reserve(bytes);
        for (const auto& part : parts) text += part;
        assert((text.size() <= (size_t)std::numeric_limits<int>::max()));
        MPI_Offset mine = (MPI_Offset)text.size(), at = 0, size = 0;
        MPI_Exscan(&mine, &at, 1, MPI_OFFSET, MPI_SUM, comm);
        if (rank == 0) at = 0;
        MPI_File fh;
        MPI_File_open(comm, fname, MPI_MODE_CREATE | MPI_MODE_WRONLY, MPI_INFO_NULL, &fh);
        MPI_File_get_size(fh, &size);
        int truncate = size > 0;
        MPI_Bcast(&truncate, 1, MPI_INT, 0, comm);
        if (truncate) MPI_File_set_size(fh, 0);
        MPI_File_write_at_all(fh, at, text.data(), (int)text.size(), MPI_CHAR, MPI_STATUS_IGNORE);
        MPI_File_close(&fh);
    }

    // Both orientations of every edge go to the owners of their first vertex (blocks of
    // num_vertices / ranks), then sort and unique (RNNG include/graph.hpp:59-116).  At one
    // rank all of it runs on the GPU (rnng_graph_finalize with RNNG_FINALIZE_AS_GIVEN: the
    // same tuples in the same order).  The edges recorded by the drop-in queries already
    // hold every self-loop.
    void redistribute_edges(MPI_Comm comm)
    {
        int rank = 0, nranks = 1;
        MPI_Comm_rank(comm, &rank);
        MPI_Comm_size(comm, &nranks);
        if (nranks == 1) {
            finalize_on_gpu();
            return;
        }
        const Index chunk = std::max<Index>(1, num_vertices / nranks);
        auto owner = [&](Index x) { return (int)std::min<Index>(x / chunk, nranks - 1); };
        MPI_Datatype edge_t;
        MPI_Type_contiguous(sizeof(Edge), MPI_CHAR, &edge_t);
        MPI_Type_commit(&edge_t);
        std::vector<int> scount(nranks, 0), sdisp(nranks), rcount(nranks), rdisp(nranks);
        for (const auto& [u, v, w] : edges) {
            scount[owner(u)]++;
            scount[owner(v)]++;
        }
        std::exclusive_scan(scount.begin(), scount.end(), sdisp.begin(), 0);
        EdgeVector send((size_t)sdisp.back() + scount.back()), recv;
        std::vector<int> fill = sdisp;
        for (const auto& [u, v, w] : edges) {
            send[fill[owner(u)]++] = Edge(u, v, w);
            send[fill[owner(v)]++] = Edge(v, u, w);
        }
        MPI_Alltoall(scount.data(), 1, MPI_INT, rcount.data(), 1, MPI_INT, comm);
        std::exclusive_scan(rcount.begin(), rcount.end(), rdisp.begin(), 0);
        recv.resize((size_t)rdisp.back() + rcount.back());
        MPI_Alltoallv(send.data(), scount.data(), sdisp.data(), edge_t, recv.data(), rcount.data(), rdisp.data(),
                      edge_t, comm);
        MPI_Type_free(&edge_t);
        std::sort(recv.begin(), recv.end());
        recv.erase(std::unique(recv.begin(), recv.end()), recv.end());
        edges.swap(recv);
        sorted = true;
    }

    Index num_edges() const { return (Index)edges.size(); }

  private:
    void ensure_sorted() const
    {
        if (!sorted) {
            std::sort(edges.begin(), edges.end());
            sorted = true;
        }
    }

    void finalize_on_gpu()
    {
        const size_t m = edges.size();
        std::vector<int64_t> u(m), v(m);
        std::vector<float> w(m);
        for (size_t i = 0; i < m; ++i) {
            u[i] = (int64_t)std::get<0>(edges[i]);
            v[i] = (int64_t)std::get<1>(edges[i]);
            w[i] = std::get<2>(edges[i]);
        }
        rnng_edges in{(int64_t)m, u.data(), v.data(), w.data(), 0, 0};
        rnng_edges out{};
        rnng_dropin::check(rnng_graph_finalize(rnng_dropin::context(), &in, num_vertices, RNNG_FINALIZE_AS_GIVEN, &out),
                           "rnng_graph_finalize");
        edges.resize((size_t)out.count);
        for (int64_t i = 0; i < out.count; ++i) edges[(size_t)i] = Edge((Index)out.u[i], (Index)out.v[i], out.w[i]);
        rnng_edges_free(&out);
        sorted = true;
    }

    mutable EdgeVector edges;
    Index num_vertices;
    mutable bool sorted = false;
};

#endif  // RNNG_DROPIN_GRAPH_H_
