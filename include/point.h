// Drop-in point containers and the Voronoi pipeline with the interface of RNNG's
// include/point.h.  Containers keep RNNG's CSR layout (atoms, offsets[n+1], ids) on the
// host; the geometry runs on the GPU through the C ABI (include/rnng_gpu.h): nearest
// landmarks (rnng_voronoi_l2 / rnng_voronoi_edit), the epsilon graph behind the ghost
// points and the searches (rnng_eps_graph_l2 / rnng_eps_graph_edit), and each cell's
// filtration (rnng_rips_edges).  Float atoms use RNNG's L2 and char atoms RNNG's edit
// distance (drivers/landmark.cpp:335-383) with bit-identical results; the caller's
// Distance functor is only called for the landmark test of the ghost rule, on the
// (point, cell) pairs that share an edge.
//
// The GPU replaces RNNG's MPI ranks: the collective steps (coalesce_cells, ghost
// exchange) run at one rank, the point-to-point helpers keep their MPI semantics.
#ifndef RNNG_DROPIN_POINT_H_
#define RNNG_DROPIN_POINT_H_

#include <sys/stat.h>

#include "simplex.h"
#include "utils.h"

template <class Atom_>
class Point
{
  public:
    using Atom = Atom_;
    using AtomVector = std::vector<Atom>;
    using AtomIter = typename AtomVector::const_iterator;

    Point(const Atom* mem, Index dim, Index index) : mem(mem), dim(dim), index(index), container_offset(-1) {}
    Point(const Atom* mem, Index dim, Index index, Index container_offset)
        : mem(mem), dim(dim), index(index), container_offset(container_offset)
    {
    }

    Index id() const { return index; }
    Index size() const { return dim; }
    Index offset() const { return container_offset; }
    Atom operator[](Index i) const { return mem[i]; }
    explicit operator const Atom*() const { return mem; }
    const Atom* begin() const { return mem; }
    const Atom* end() const { return mem + dim; }

  private:
    const Atom* mem;
    Index dim, index, container_offset;
};

template <class Atom_>
class PointContainer
{
  public:
    using Atom = Atom_;
    using AtomVector = std::vector<Atom>;

    PointContainer() : offsets({0}) {}
    PointContainer(const std::vector<Point<Atom>>& points) : offsets({0})
    {
        for (const Point<Atom>& p : points) push_back(p);
    }
    PointContainer(const AtomVector& atoms, const IndexVector& sizes, const IndexVector& indices)
    {
        init(atoms, sizes, indices);
    }
    PointContainer(const AtomVector& atoms, Index size, Index dim, const IndexVector& indices)
    {
        init(atoms, size, dim, indices);
    }
    PointContainer(const PointContainer& lhs, const PointContainer& rhs) : offsets({0})
    {
        for (Index i = 0; i < lhs.num_points(); ++i) push_back(lhs[i]);
        for (Index i = 0; i < rhs.num_points(); ++i) push_back(rhs[i]);
    }

    Index num_points() const { return (Index)ids.size(); }
    Index num_atoms() const { return (Index)data.size(); }

    Point<Atom> operator[](Index i) const { return Point<Atom>(mem(i), size(i), id(i), i); }

    // fvecs: per record an int32 dimension and that many floats; ids 0..n-1.
    Index read_fvecs(const char* fname)
    {
        assert((std::is_same_v<Atom, float>));
        std::ifstream in(fname, std::ios::binary);
        assert((in.good()));
        in.seekg(0, in.end);
        const size_t bytes = (size_t)in.tellg();
        in.seekg(0, in.beg);
        int d = 0;
        in.read((char*)&d, sizeof(int));
        in.seekg(0, in.beg);
        const size_t rec = sizeof(int) + sizeof(Atom) * (size_t)d;
        assert((d >= 1 && bytes % rec == 0));
        const Index n = (Index)(bytes / rec);
        data.resize((size_t)n * d);
        offsets.resize(n + 1);
        ids.resize(n);
        std::vector<char> buf(rec);
        for (Index i = 0; i < n; ++i) {
            in.read(buf.data(), rec);
            int di = 0;
            std::memcpy(&di, buf.data(), sizeof(int));
            assert((di == d));
            std::memcpy(&data[(size_t)i * d], buf.data() + sizeof(int), sizeof(Atom) * d);
            offsets[i] = i * d;
            ids[i] = i;
        }
        offsets[n] = n * d;
        return n;
    }

    // One sequence per non-empty line (a trailing carriage return is dropped).
    Index read_seqs(const char* fname)
    {
        assert((std::is_same_v<Atom, char>));
        std::ifstream in(fname);
        std::string line;
        data.clear();
        offsets.assign(1, 0);
        ids.clear();
        Index next = 0;
        while (std::getline(in, line)) {
            if (!line.empty() && line.back() == '\r') line.pop_back();
            if (line.empty()) continue;
            data.insert(data.end(), line.begin(), line.end());
            offsets.push_back((Index)data.size());
            ids.push_back(next++);
        }
        return next;
    }

    // Block of records of this rank (the first total % ranks ranks get one more).
    Index read_fvecs(const char* fname, MPI_Comm comm)
    {
        PointContainer all;
        const Index total = all.read_fvecs(fname);
        keep_block(all, total, comm);
        return total;
    }

    Index read_seqs(const char* fname, MPI_Comm comm)
    {
        PointContainer all;
        const Index total = all.read_seqs(fname);
        keep_block(all, total, comm);
        return total;
    }

    struct SendrecvRequest {
        MPI_Request reqs[6];
        void wait() { MPI_Waitall(6, reqs, MPI_STATUSES_IGNORE); }
    };

    // Sends this container to sendrank and receives recvbuf from recvrank (a ring shift).
    void sendrecv(PointContainer& recvbuf, int recvrank, int sendrank, MPI_Comm comm, SendrecvRequest& req)
    {
        int rank = 0, nranks = 1;
        MPI_Comm_rank(comm, &rank);
        MPI_Comm_size(comm, &nranks);
        int scount[2] = {(int)num_points(), (int)num_atoms()}, rcount[2] = {0, 0};
        MPI_Irecv(rcount, 2, MPI_INT, recvrank, rank, comm, &req.reqs[0]);
        MPI_Isend(scount, 2, MPI_INT, sendrank, sendrank, comm, &req.reqs[1]);
        MPI_Waitall(2, req.reqs, MPI_STATUSES_IGNORE);
        recvbuf.data.resize(rcount[1]);
        recvbuf.ids.resize(rcount[0]);
        recvbuf.offsets.resize(rcount[0] + 1);
        MPI_Irecv(recvbuf.data.data(), rcount[1], mpi_type<Atom>(), recvrank, rank + nranks, comm, &req.reqs[0]);
        MPI_Isend(data.data(), scount[1], mpi_type<Atom>(), sendrank, sendrank + nranks, comm, &req.reqs[1]);
        MPI_Irecv(recvbuf.ids.data(), rcount[0], MPI_INDEX, recvrank, rank + 2 * nranks, comm, &req.reqs[2]);
        MPI_Isend(ids.data(), scount[0], MPI_INDEX, sendrank, sendrank + 2 * nranks, comm, &req.reqs[3]);
        MPI_Irecv(recvbuf.offsets.data(), rcount[0] + 1, MPI_INDEX, recvrank, rank + 3 * nranks, comm, &req.reqs[4]);
        MPI_Isend(offsets.data(), scount[0] + 1, MPI_INDEX, sendrank, sendrank + 3 * nranks, comm, &req.reqs[5]);
    }

    void swap(PointContainer& other)
    {
        std::swap(data, other.data);
        std::swap(offsets, other.offsets);
        std::swap(ids, other.ids);
    }

    // Concatenation of every rank's sendbuf, in rank order.
    void allgather(const PointContainer& sendbuf, MPI_Comm comm)
    {
        int rank = 0, nranks = 1;
        MPI_Comm_rank(comm, &rank);
        MPI_Comm_size(comm, &nranks);
        std::vector<int> cnt(nranks), acnt(nranks), disp(nranks), adisp(nranks);
        cnt[rank] = (int)sendbuf.num_points();
        acnt[rank] = (int)sendbuf.num_atoms();
        MPI_Allgather(MPI_IN_PLACE, 1, MPI_INT, cnt.data(), 1, MPI_INT, comm);
        MPI_Allgather(MPI_IN_PLACE, 1, MPI_INT, acnt.data(), 1, MPI_INT, comm);
        std::exclusive_scan(cnt.begin(), cnt.end(), disp.begin(), 0);
        std::exclusive_scan(acnt.begin(), acnt.end(), adisp.begin(), 0);
        IndexVector sizes((size_t)disp.back() + cnt.back()), mysizes(sendbuf.num_points());
        for (Index i = 0; i < sendbuf.num_points(); ++i) mysizes[i] = sendbuf.size(i);
        ids.resize(sizes.size());
        data.resize((size_t)adisp.back() + acnt.back());
        MPI_Allgatherv(sendbuf.ids.data(), cnt[rank], MPI_INDEX, ids.data(), cnt.data(), disp.data(), MPI_INDEX, comm);
        MPI_Allgatherv(mysizes.data(), cnt[rank], MPI_INDEX, sizes.data(), cnt.data(), disp.data(), MPI_INDEX, comm);
        MPI_Allgatherv(sendbuf.data.data(), acnt[rank], mpi_type<Atom>(), data.data(), acnt.data(), adisp.data(),
                       mpi_type<Atom>(), comm);
        offsets.assign(1, 0);
        for (Index s : sizes) offsets.push_back(offsets.back() + s);
        assert((offsets.back() == (Index)data.size()));
    }

    // The points of sendbuf at the given container offsets, in that order.
    void indexed_gather(const PointContainer& sendbuf, const IndexVector& index_offsets)
    {
        data.clear();
        offsets.assign(1, 0);
        ids.clear();
        for (Index k : index_offsets) push_back(sendbuf[k]);
    }

    void push_back(const Point<Atom>& p)
    {
        data.insert(data.end(), p.begin(), p.end());
        offsets.push_back((Index)data.size());
        ids.push_back(p.id());
    }

    typename IndexVector::const_iterator ids_begin() const { return ids.begin(); }
    typename IndexVector::const_iterator ids_end() const { return ids.end(); }

    // Access for the GPU calls (not part of RNNG's interface).
    const Atom* atom_data() const { return data.data(); }
    const IndexVector& offset_data() const { return offsets; }
    const IndexVector& id_data() const { return ids; }
    // Common dimension of all points (dense L2 data), or -1.
    Index uniform_dim() const
    {
        const Index n = num_points();
        if (n == 0) return 0;
        const Index d = offsets[1] - offsets[0];
        for (Index i = 1; i < n; ++i)
            if (offsets[i + 1] - offsets[i] != d) return -1;
        return d;
    }

  protected:
    AtomVector data;
    IndexVector offsets, ids;

    void init(const AtomVector& atoms, const IndexVector& sizes, const IndexVector& indices)
    {
        assert((sizes.size() == indices.size()));
        data = atoms;
        ids = indices;
        offsets.assign(1, 0);
        for (Index s : sizes) offsets.push_back(offsets.back() + s);
    }

    void init(const AtomVector& atoms, Index size, Index dim, const IndexVector& indices)
    {
        assert(((Index)atoms.size() == size * dim && (Index)indices.size() == size));
        data = atoms;
        ids = indices;
        offsets.resize(size + 1);
        for (Index i = 0; i <= size; ++i) offsets[i] = i * dim;
    }

    const Atom* mem(Index i) const { return data.data() + offsets[i]; }
    Index size(Index i) const { return offsets[i + 1] - offsets[i]; }
    Index id(Index i) const
    {
        assert((i >= 0 && i < (Index)ids.size()));
        return ids[i];
    }

  private:
    void keep_block(const PointContainer& all, Index total, MPI_Comm comm)
    {
        int rank = 0, nranks = 1;
        MPI_Comm_rank(comm, &rank);
        MPI_Comm_size(comm, &nranks);
        const Index base = total / nranks, extra = total % nranks;
        const Index mine = base + (rank < extra ? 1 : 0);
        const Index first = rank * base + std::min<Index>(rank, extra);
        data.clear();
        offsets.assign(1, 0);
        ids.clear();
        for (Index i = first; i < first + mine; ++i) push_back(all[i]);
    }
};

template <class Atom_>
class VoronoiCell : public PointContainer<Atom_>
{
  public:
    using Atom = Atom_;
    using AtomVector = std::vector<Atom>;

    VoronoiCell(const std::vector<Point<Atom>>& points, const RealVector& dist_to_centers, Index cell_index)
        : PointContainer<Atom>(points), cell_index(cell_index), dist_to_centers(dist_to_centers),
          interior(points.size(), false)
    {
    }

    void add_ghost_point(const Point<Atom>& p) { ghost_points.push_back(p); }

    Index id() const { return cell_index; }
    Index num_ghosts() const { return ghost_points.num_points(); }
    Point<Atom> ghost(Index i) const { return ghost_points[i]; }
    Real dist_to_center(Index i) const { return dist_to_centers[i]; }
    const PointContainer<Atom>& ghosts() const { return ghost_points; }
    const BoolVector& interiors() const { return interior; }
    void set_interior(Index offset) { interior[offset] = true; }

  protected:
    Index cell_index;
    RealVector dist_to_centers;
    BoolVector interior;
    PointContainer<Atom> ghost_points;
};

namespace rnng_dropin {

// Map from Index keys to non-negative Index values for the lookups made per query and per
// replayed neighbour: open addressing with linear probing in a power-of-two table at most
// half full, keys and values side by side (one cache line per lookup, where the node
// chasing of std::unordered_map dominated the searches' replay).  The one key value that
// marks free slots is stored beside the table.
class FlatIndexMap
{
  public:
    void reserve(Index n)
    {
        size_t want = 16;
        while (want < 2 * (size_t)std::max<Index>(n, 0)) want *= 2;
        if (want > slots.size()) rehash(want);
    }

    // Inserts (key, value) unless the key is present; returns whether it was inserted.
    bool emplace(Index key, Index value)
    {
        if (key == kFree) {
            if (has_free_key) return false;
            has_free_key = true;
            free_key_value = value;
            return true;
        }
        if (2 * (count + 1) > slots.size()) rehash(std::max<size_t>(16, 2 * slots.size()));
        for (size_t h = home(key);; h = (h + 1) & mask) {
            Slot& s = slots[h];
            if (s.key == kFree) {
                s = Slot{key, value};
                ++count;
                return true;
            }
            if (s.key == key) return false;
        }
    }

    // The key's value, or -1.
    Index find(Index key) const
    {
        if (key == kFree) return has_free_key ? free_key_value : -1;
        if (slots.empty()) return -1;
        for (size_t h = home(key);; h = (h + 1) & mask) {
            const Slot& s = slots[h];
            if (s.key == key) return s.value;
            if (s.key == kFree) return -1;
        }
    }

    size_t size() const { return count + (has_free_key ? 1 : 0); }

  private:
    struct Slot {
        Index key, value;
    };
    static constexpr Index kFree = std::numeric_limits<Index>::min();

    // Fibonacci hashing: the top bits of key x 2^64 / golden ratio
    size_t home(Index key) const { return (size_t)(((uint64_t)key * 0x9E3779B97F4A7C15ull) >> shift); }

    void rehash(size_t n)
    {
        std::vector<Slot> old(n, Slot{kFree, 0});
        old.swap(slots);  // slots: the new free table; old: the entries to insert again
        mask = n - 1;
        shift = 64;
        for (size_t v = n; v > 1; v >>= 1) --shift;
        count = 0;
        for (const Slot& s : old)
            if (s.key != kFree) emplace(s.key, s.value);
    }

    std::vector<Slot> slots;
    size_t mask = 0, count = 0;
    int shift = 64;
    bool has_free_key = false;
    Index free_key_value = -1;
};

// Unordered edges (a < b, container rows) of the epsilon graph of a container.
struct RowEdges {
    std::vector<int64_t> u, v;
    std::vector<float> w;
};

template <class Atom>
RowEdges eps_graph_rows(const PointContainer<Atom>& pts, Real radius)
{
    RowEdges out;
    const Index n = pts.num_points();
    if (n < 2) return out;
    rnng_edges e;
    if constexpr (std::is_same_v<Atom, float>) {
        const Index d = pts.uniform_dim();
        assert((d >= 1));
        const int mode = d <= 256 ? RNNG_MODE_BF16_RECHECK : RNNG_MODE_FP32_DIRECT;
        check(rnng_eps_graph_l2(context(), pts.atom_data(), nullptr, n, d, radius, mode, 0, &e), "rnng_eps_graph_l2");
    } else {
        static_assert(std::is_same_v<Atom, char>, "the GPU paths take float (L2) or char (edit distance) atoms");
        check(rnng_eps_graph_edit(context(), reinterpret_cast<const uint8_t*>(pts.atom_data()),
                                  pts.offset_data().data(), nullptr, n, radius, 0, &e),
              "rnng_eps_graph_edit");
    }
    out.u.assign(e.u, e.u + e.count);
    out.v.assign(e.v, e.v + e.count);
    out.w.assign(e.w, e.w + e.count);
    return out;
}

// distance(p, p): 0 for strings; for L2 0 unless an atom is infinite or NaN (then NaN,
// which is within no radius).
template <class Atom>
bool self_distance_zero(const Point<Atom>& p)
{
    if constexpr (std::is_same_v<Atom, float>) {
        for (Atom a : p)
            if (!std::isfinite(a)) return false;
    }
    return true;
}

// The epsilon graph of a point set at one radius, with a private copy of the points:
// rows are the copy's offsets, rowptr/nbr/w the adjacency (both orientations, no
// self-loops) with RNNG's distances.
template <class Atom>
struct GraphCache {
    Real radius = 0;
    PointContainer<Atom> pts;
    FlatIndexMap row_of_id;
    IndexVector rowptr, nbr;
    RealVector w;

    // Row holding a point with the same id and the same atoms, or -1.
    Index find(const Point<Atom>& p) const
    {
        const Index row = row_of_id.find(p.id());
        if (row < 0) return -1;
        const Point<Atom> q = pts[row];
        if (q.size() != p.size() || !std::equal(p.begin(), p.end(), q.begin(), [](Atom a, Atom b) {
                return std::memcmp(&a, &b, sizeof(Atom)) == 0;
            }))
            return -1;
        return row;
    }

    // Rows of all points of a container, if the graph holds every one of them.
    bool find_all(const PointContainer<Atom>& c, IndexVector& rows) const
    {
        rows.resize(c.num_points());
        for (Index i = 0; i < c.num_points(); ++i)
            if ((rows[i] = find(c[i])) < 0) return false;
        return true;
    }
};

// The most recent graph: the searches and complexes of a pipeline read the one graph
// that the ghost step (or their first query) computed.
template <class Atom>
std::shared_ptr<const GraphCache<Atom>>& last_graph()
{
    static std::shared_ptr<const GraphCache<Atom>> g;
    return g;
}

// The epsilon graph of pts on the GPU, kept as the most recent graph when its ids are
// unique (a lookup by id needs them to be).
template <class Atom>
std::shared_ptr<const GraphCache<Atom>> build_graph(const PointContainer<Atom>& pts, Real radius)
{
    auto g = std::make_shared<GraphCache<Atom>>();
    g->radius = radius;
    g->pts = pts;
    const Index n = pts.num_points();
    bool unique_ids = true;
    g->row_of_id.reserve(n);
    for (Index i = 0; i < n && unique_ids; ++i) unique_ids = g->row_of_id.emplace(pts[i].id(), i);
    assert((unique_ids));  // RNNG's ids are unique; the lookup by id relies on it
    const RowEdges e = eps_graph_rows(pts, radius);
    g->rowptr.assign(n + 1, 0);
    for (size_t k = 0; k < e.u.size(); ++k) {
        g->rowptr[e.u[k] + 1]++;
        g->rowptr[e.v[k] + 1]++;
    }
    for (Index i = 0; i < n; ++i) g->rowptr[i + 1] += g->rowptr[i];
    g->nbr.resize(2 * e.u.size());
    g->w.resize(2 * e.u.size());
    IndexVector fill(g->rowptr.begin(), g->rowptr.end() - 1);
    for (size_t k = 0; k < e.u.size(); ++k) {
        Index p = fill[e.u[k]]++;
        g->nbr[p] = e.v[k];
        g->w[p] = e.w[k];
        p = fill[e.v[k]]++;
        g->nbr[p] = e.u[k];
        g->w[p] = e.w[k];
    }
    last_graph<Atom>() = g;
    return g;
}

}  // namespace rnng_dropin

template <class Atom_>
class VoronoiComplex : public PointContainer<Atom_>
{
  public:
    using Atom = Atom_;

    // Cell points followed by its ghosts (include/point.hpp:1127-1133).
    VoronoiComplex(const VoronoiCell<Atom>& cell, Real radius, Index maxdim)
        : PointContainer<Atom>(cell, cell.ghosts()), radius(radius), maxdim(maxdim), local(cell.num_points()),
          interior(cell.interiors())
    {
    }

    // The Rips filtration of the complex's points up to maxdim (include/point.hpp:
    // 1135-1232): vertices at 0, edges at their distance, higher simplices at their
    // largest edge, ids over the points' ids, sorted by (value, id).  A simplex is
    // interior when one of its vertices is an interior point of the cell.  (RNNG reads
    // its interior flags past their end for ghost vertices; here ghosts are never
    // interior.)  The graph comes from the most recent whole-set graph when it holds
    // every point of the complex, else from one GPU epsilon-graph call.
    template <class Distance>
    void build_filtration(Distance&, Index, Real, Index)
    {
        const Index n = this->num_points();
        filtration.clear();
        if (n == 0) return;
        std::vector<int64_t> u, v;
        std::vector<float> w;
        std::shared_ptr<const rnng_dropin::GraphCache<Atom>> g = rnng_dropin::last_graph<Atom>();
        IndexVector rows;
        if (g && g->radius == radius && g->find_all(*this, rows)) {
            std::unordered_map<Index, Index> local_of_row;
            local_of_row.reserve(n);
            for (Index i = 0; i < n; ++i) local_of_row.emplace(rows[i], i);
            for (Index i = 0; i < n; ++i)
                for (Index k = g->rowptr[rows[i]]; k < g->rowptr[rows[i] + 1]; ++k) {
                    auto it = local_of_row.find(g->nbr[k]);
                    if (it != local_of_row.end() && it->second > i) {
                        u.push_back(i);
                        v.push_back(it->second);
                        w.push_back(g->w[k]);
                    }
                }
        } else {
            rnng_dropin::RowEdges e = rnng_dropin::eps_graph_rows(*this, radius);
            u.swap(e.u);
            v.swap(e.v);
            w.swap(e.w);
        }
        std::vector<uint8_t> flags(n, 0);
        for (Index i = 0; i < local && i < (Index)interior.size(); ++i) flags[i] = interior[i] ? 1 : 0;
        rnng_simplices s;
        rnng_dropin::check(rnng_rips_edges(rnng_dropin::context(), n, this->id_data().data(), flags.data(),
                                           u.empty() ? nullptr : u.data(), v.empty() ? nullptr : v.data(),
                                           w.empty() ? nullptr : w.data(), (int64_t)u.size(), (int)maxdim, 0, &s),
                           "rnng_rips_edges");
        filtration.reserve(s.count);
        for (int64_t k = 0; k < s.count; ++k) filtration.emplace_back(s.id[k], s.value[k], s.flag[k] != 0);
    }

    // "%f\t<id>\t<interior>" per simplex, or the vertex list instead of the id
    // (include/point.hpp:1268-1290).
    void write_filtration_file(const char* fname, Index num_verts, bool use_ids = true) const
    {
        FILE* f = std::fopen(fname, "w");
        assert((f != nullptr));
        for (const WeightedSimplex& s : filtration) {
            if (use_ids) std::fprintf(f, "%f\t%lld\t%d\n", s.value, (long long)s.getid(), (int)s.interior);
            else std::fprintf(f, "%f\t%s\t%d\n", s.value, s.get_simplex_repr(num_verts).c_str(), (int)s.interior);
        }
        std::fclose(f);
    }

    Index num_simplices() const { return (Index)filtration.size(); }
    typename std::vector<WeightedSimplex>::const_iterator begin() const { return filtration.begin(); }
    typename std::vector<WeightedSimplex>::const_iterator end() const { return filtration.end(); }

  private:
    Real radius;
    Index maxdim;
    Index local;
    BoolVector interior;
    std::vector<WeightedSimplex> filtration;
};

template <class Atom_>
class VoronoiDiagram : public PointContainer<Atom_>
{
  public:
    using Atom = Atom_;
    using AtomVector = std::vector<Atom>;
    using Cell = VoronoiCell<Atom>;

    // Nearest centre of every point, ties to the last centre, RNNG's distances
    // (include/point.hpp:537-559), on the GPU.
    template <class Distance>
    VoronoiDiagram(const PointContainer<Atom>& points, const PointContainer<Atom>& centers, Distance&)
        : PointContainer<Atom>(points), centers(centers), cell_indices(points.num_points(), 0),
          dist_to_centers(points.num_points(), std::numeric_limits<Real>::max())
    {
        const Index n = points.num_points(), m = centers.num_points();
        if (n == 0 || m == 0) return;
        if constexpr (std::is_same_v<Atom, float>) {
            const Index d = points.uniform_dim();
            assert((d >= 1 && centers.uniform_dim() == d));
            rnng_dropin::check(rnng_voronoi_l2(rnng_dropin::context(), points.atom_data(), n, centers.atom_data(), m, d, 0,
                                               cell_indices.data(), dist_to_centers.data()),
                               "rnng_voronoi_l2");
        } else {
            rnng_dropin::check(
                rnng_voronoi_edit(rnng_dropin::context(), reinterpret_cast<const uint8_t*>(points.atom_data()),
                                  points.offset_data().data(), n, reinterpret_cast<const uint8_t*>(centers.atom_data()),
                                  centers.offset_data().data(), m, 0, cell_indices.data(), dist_to_centers.data()),
                "rnng_voronoi_edit");
        }
    }

    // RNNG's coalesce_cells at one rank (include/point.hpp:562-758): one cell per centre
    // in centre order, its points in row order with the row as id, the centre's own point
    // moved to slot 0.  A cell that received no point keeps cell id 0, as RNNG's does.
    void coalesce_cells(std::vector<Cell>& mycells, MPI_Comm comm) const
    {
        assert((get_comm_size(comm) == 1));  // the GPU stands in for the ranks
        const Index n = this->num_points(), m = centers.num_points();
        std::vector<std::vector<Point<Atom>>> pts(m);
        std::vector<RealVector> dists(m);
        IndexVector center_slot(m, 0);
        for (Index i = 0; i < n; ++i) {
            const Index c = cell_indices[i];
            const Point<Atom> p = (*this)[i];
            if (centers[c].id() == i) center_slot[c] = (Index)pts[c].size();
            pts[c].emplace_back(p.begin(), p.size(), i);
            dists[c].push_back(dist_to_centers[i]);
        }
        mycells.clear();
        mycells.reserve(m);
        for (Index c = 0; c < m; ++c) {
            if (!pts[c].empty()) {
                std::swap(pts[c][0], pts[c][center_slot[c]]);
                std::swap(dists[c][0], dists[c][center_slot[c]]);
            }
            mycells.emplace_back(pts[c], dists[c], pts[c].empty() ? 0 : c);
        }
    }

    // RNNG's ghost rule (include/point.hpp:762-929): a point q of cell A is a ghost of
    // cell B when B has a point within radius of q; RNNG only tests the B that pass its
    // landmark test distance(s_k, q) <= d(q, A's centre) + 2 radius, where s_k is the
    // slot-0 point of the k-th non-empty cell and B is cells[k] (the k-th non-empty cell
    // whenever no cell is empty).  Ghosts are added in the order of the points across
    // the cells.
    template <class Distance>
    void add_ghost_points_systolic(std::vector<Cell>& cells, Distance& distance, Real radius, Real, Index,
                                   MPI_Comm comm) const
    {
        ghosts(cells, distance, radius, comm, false);
    }

    // The same ghosts; a point that became nobody's ghost is interior
    // (include/point.hpp:933-1124).
    template <class Distance>
    void add_ghost_points_systolic_rips(std::vector<Cell>& cells, Distance& distance, Real radius, Real, Index,
                                        MPI_Comm comm) const
    {
        ghosts(cells, distance, radius, comm, true);
    }

  private:
    PointContainer<Atom> centers;
    IndexVector cell_indices;
    RealVector dist_to_centers;

    // One GPU epsilon graph over all cell points gives, for every point, the cells that
    // hold a neighbour within radius; RNNG's landmark test is then applied to those
    // (cell, point) pairs with the caller's functor.  The graph is kept for the searches
    // and complexes that follow.
    template <class Distance>
    void ghosts(std::vector<Cell>& cells, Distance& distance, Real radius, MPI_Comm comm, bool mark_interior) const
    {
        assert((get_comm_size(comm) == 1));
        const Index ncell = (Index)cells.size();
        PointContainer<Atom> all;  // the queries, in RNNG's order: cells in order, points in order
        IndexVector cell_of, slot_of;
        RealVector qdist;
        for (Index c = 0; c < ncell; ++c)
            for (Index i = 0; i < cells[c].num_points(); ++i) {
                all.push_back(cells[c][i]);
                cell_of.push_back(c);
                slot_of.push_back(i);
                qdist.push_back(cells[c].dist_to_center(i));
            }
        IndexVector nonempty;  // RNNG's centre list: slot 0 of every non-empty cell
        for (Index c = 0; c < ncell; ++c)
            if (cells[c].num_points() > 0) nonempty.push_back(c);
        std::shared_ptr<const rnng_dropin::GraphCache<Atom>> g = rnng_dropin::build_graph(all, radius);
        // (target cell index, query row) for every query with a neighbour in a cell that
        // RNNG's landmark test lets through; cells[k] is tested against landmark k
        std::vector<std::pair<Index, Index>> add;
        std::vector<char> shared(all.num_points(), 0);
        const Real bound_pad = 2 * radius;
        for (Index q = 0; q < all.num_points(); ++q) {
            std::vector<Index> near_cells;
            for (Index k = g->rowptr[q]; k < g->rowptr[q + 1]; ++k) near_cells.push_back(cell_of[g->nbr[k]]);
            std::sort(near_cells.begin(), near_cells.end());
            near_cells.erase(std::unique(near_cells.begin(), near_cells.end()), near_cells.end());
            const Point<Atom> query = all[q];
            const Real bound = qdist[q] + bound_pad;
            for (Index b : near_cells) {
                // RNNG visits cells[k] for landmark k: the target b is tested against the
                // slot-0 point of the b-th non-empty cell, and must exist as such
                if (b == cell_of[q] || b >= (Index)nonempty.size()) continue;
                const Point<Atom> landmark = cells[nonempty[b]][0];
                const Real dl = distance(landmark, query);
                if (dl <= bound) {
                    add.emplace_back(b, q);
                    shared[q] = 1;
                }
            }
        }
        std::sort(add.begin(), add.end());
        for (const auto& [b, q] : add) cells[b].add_ghost_point(all[q]);
        if (mark_interior)
            for (Index q = 0; q < all.num_points(); ++q)
                if (!shared[q]) cells[cell_of[q]].set_interior(slot_of[q]);
    }
};

#include "search.h"

#endif  // RNNG_DROPIN_POINT_H_
