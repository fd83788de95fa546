// Drop-in simplices with the interface of RNNG's include/simplex.h: ids in the
// combinatorial number system, weighted simplices of a filtration and the merged
// filtration writer.  Host code (simplex ids of whole complexes are built on the GPU
// by rnng_rips_l2; these types carry them).
#ifndef RNNG_DROPIN_SIMPLEX_H_
#define RNNG_DROPIN_SIMPLEX_H_

#include "utils.h"

static Binom binom;

// id = sum over the sorted vertices v_0 < ... < v_p of C(v_i, i + 1), OR-ed with p << 60
// (RNNG include/simplex.hpp:5-19); the low 60 bits are the uid, the top 4 the dimension.
struct Simplex {
    Simplex() : id(0) {}
    Simplex(Index id) : id(id) {}
    Simplex(const IndexVector& verts)
    {
        IndexVector v(verts);
        std::sort(v.begin(), v.end());
        const uint64_t p = v.size() - 1;
        uint64_t uid = 0;
        for (Index i = (Index)p; i >= 0; --i) uid += (uint64_t)binom(v[i], i + 1);
        id = (Index)(uid | (p << 60));
    }

    Index getid() const { return id; }
    Index getuid() const { return (Index)((uint64_t)id & 0xFFFFFFFFFFFFFFFull); }
    Index getdim() const { return (Index)(((uint64_t)id >> 60) & 0xF); }

    // Vertices from the id: for i = dim .. 0, the largest v < n with C(v, i+1) <= rest.
    IndexVector getverts(Index n) const
    {
        uint64_t rest = (uint64_t)getuid();
        IndexVector v;
        for (Index i = getdim(); i >= 0; --i) {
            Index lo = 0, hi = n;  // first x with C(x, i+1) > rest, minus one
            while (lo < hi) {
                const Index mid = lo + ((hi - lo) >> 1);
                if ((uint64_t)binom(mid, i + 1) > rest) hi = mid;
                else lo = mid + 1;
            }
            v.push_back(hi - 1);
            rest -= (uint64_t)binom(hi - 1, i + 1);
        }
        if (v.size() > 1) std::sort(v.begin(), v.end());
        return v;
    }

    void get_facets(std::vector<Simplex>& facets, Index n) const
    {
        facets.clear();
        const IndexVector v = getverts(n);
        for (size_t skip = 0; skip < v.size(); ++skip) {
            IndexVector f;
            for (size_t k = 0; k < v.size(); ++k)
                if (k != skip) f.push_back(v[k]);
            facets.emplace_back(f);
        }
    }

    void get_facet_ids(IndexVector& ids, Index n) const
    {
        ids.clear();
        std::vector<Simplex> facets;
        get_facets(facets, n);
        for (const Simplex& f : facets) ids.push_back(f.getid());
    }

    std::string get_simplex_repr(Index n) const
    {
        const IndexVector v = getverts(n);
        std::ostringstream out;
        out << "<";
        for (size_t k = 0; k < v.size(); ++k) out << v[k] << (k + 1 < v.size() ? "," : ">");
        return out.str();
    }

    Index id;
};

struct WeightedSimplex : public Simplex {
    WeightedSimplex(const IndexVector& verts, bool interior) : Simplex(verts), value(0), interior(interior) {}
    WeightedSimplex(Index id, Real value, bool interior) : Simplex(id), value(value), interior(interior) {}

    friend bool operator<(const WeightedSimplex& a, const WeightedSimplex& b)
    {
        return std::tie(a.value, a.id) < std::tie(b.value, b.id);
    }
    friend bool operator==(const WeightedSimplex& a, const WeightedSimplex& b) { return a.id == b.id; }
    friend bool operator!=(const WeightedSimplex& a, const WeightedSimplex& b) { return a.id != b.id; }

    Real getvalue() const { return value; }

    Real value;
    bool interior;
};

struct SimplexEnvelope {
    Index id;
    Real value;

    SimplexEnvelope() {}
    SimplexEnvelope(Index id, Real value) : id(id), value(value) {}
    SimplexEnvelope(const WeightedSimplex& s) : id(s.getid()), value(s.getvalue()) {}

    friend bool operator<(const SimplexEnvelope& a, const SimplexEnvelope& b)
    {
        return std::tie(a.value, a.id) < std::tie(b.value, b.id);
    }
    friend bool operator==(const SimplexEnvelope& a, const SimplexEnvelope& b) { return a.id == b.id; }
    friend bool operator!=(const SimplexEnvelope& a, const SimplexEnvelope& b) { return a.id != b.id; }
};

// Union of all ranks' simplices, sorted by (value, id), one entry per id, written by
// rank 0 as "%f\t<id>" (or "%f\t<v0,v1,...>" with use_ids false); RNNG
// include/simplex.hpp:130-196.
inline void merge_and_write_filtration(const char* fname, const std::vector<WeightedSimplex>& mine, Index num_vertices,
                                       bool use_ids, MPI_Comm comm)
{
    int rank = 0, nranks = 1;
    MPI_Comm_rank(comm, &rank);
    MPI_Comm_size(comm, &nranks);
    MPI_Datatype env_t;
    MPI_Type_contiguous(sizeof(SimplexEnvelope), MPI_CHAR, &env_t);
    MPI_Type_commit(&env_t);
    std::vector<SimplexEnvelope> local(mine.begin(), mine.end());
    std::sort(local.begin(), local.end());
    local.erase(std::unique(local.begin(), local.end()), local.end());
    int count = (int)local.size();
    std::vector<int> counts(rank == 0 ? nranks : 0), displs(rank == 0 ? nranks : 0);
    MPI_Gather(&count, 1, MPI_INT, counts.data(), 1, MPI_INT, 0, comm);
    std::vector<SimplexEnvelope> all;
    if (rank == 0) {
        std::exclusive_scan(counts.begin(), counts.end(), displs.begin(), 0);
        all.resize((size_t)displs.back() + counts.back());
    }
    MPI_Gatherv(local.data(), count, env_t, all.data(), counts.data(), displs.data(), env_t, 0, comm);
    if (rank == 0) {
        std::sort(all.begin(), all.end());
        all.erase(std::unique(all.begin(), all.end()), all.end());
        FILE* f = std::fopen(fname, "w");
        assert((f != nullptr));
        for (const SimplexEnvelope& s : all) {
            if (use_ids) std::fprintf(f, "%f\t%lld\n", s.value, (long long)s.id);
            else std::fprintf(f, "%f\t%s\n", s.value, Simplex(s.id).get_simplex_repr(num_vertices).c_str());
        }
        std::fclose(f);
    }
    MPI_Type_free(&env_t);
}

#endif  // RNNG_DROPIN_SIMPLEX_H_
