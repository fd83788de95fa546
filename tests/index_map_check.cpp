// Checks the drop-in searches' lookup tables (FlatIndexMap, and LocalIndex in its dense and
// sparse forms) against std::unordered_map on sequential, random, negative and extreme
// keys, with and without reserve.  Prints "ok" and exits 0, or names the first mismatch.
#include <cstdio>
#include <cstdlib>

#include "search.h"

using rnng_dropin::FlatIndexMap;
using rnng_dropin::LocalIndex;

static int fail(const char* what, long long key)
{
    std::printf("mismatch: %s (key %lld)\n", what, key);
    return 1;
}

static uint64_t rng = 88172645463325252ull;
static uint64_t next()
{
    rng ^= rng << 13;
    rng ^= rng >> 7;
    rng ^= rng << 17;
    return rng;
}

// Inserts keys into both maps (emplace results must agree), then looks up every key and
// a set of absent ones.
static int check_keys(const std::vector<Index>& keys, bool reserve_first)
{
    FlatIndexMap m;
    std::unordered_map<Index, Index> ref;
    if (reserve_first) m.reserve((Index)keys.size() / 2);
    for (size_t i = 0; i < keys.size(); ++i) {
        const bool a = m.emplace(keys[i], (Index)i);
        const bool b = ref.emplace(keys[i], (Index)i).second;
        if (a != b) return fail("emplace result", keys[i]);
    }
    if (m.size() != ref.size()) return fail("size", (long long)m.size());
    for (const auto& [k, v] : ref)
        if (m.find(k) != v) return fail("find of a present key", k);
    for (int t = 0; t < 100000; ++t) {
        const Index k = (Index)next();
        const auto it = ref.find(k);
        if (m.find(k) != (it == ref.end() ? -1 : it->second)) return fail("find of a random key", k);
    }
    return 0;
}

int main()
{
    const Index lo = std::numeric_limits<Index>::min(), hi = std::numeric_limits<Index>::max();
    if (FlatIndexMap().find(0) != -1 || FlatIndexMap().find(lo) != -1) return fail("empty map", 0);
    std::vector<Index> seq;
    for (Index i = 0; i < 300000; ++i) seq.push_back(i);  // ids 0..n-1, the drivers' case
    std::vector<Index> mixed = {lo, hi, -1, 0, 1, lo, hi, -1, lo + 1, hi - 1};
    for (int i = 0; i < 200000; ++i) {
        const uint64_t r = next();
        // random keys, small negatives, multiples of large powers of two (same low bits), repeats
        const Index k = (i % 4 == 0) ? (Index)r : (i % 4 == 1) ? -(Index)(r % 1000) : (i % 4 == 2) ? (Index)((r % 4096) << 40)
                                                                                                : mixed[r % mixed.size()];
        mixed.push_back(k);
    }
    for (bool rsv : {false, true}) {
        if (check_keys(seq, rsv) || check_keys(mixed, rsv)) return 1;
    }
    // LocalIndex: graph rows of a search's container -> its offsets, -1 elsewhere
    for (Index graph_rows : {Index(1000), Index(400000)}) {
        IndexVector rows;
        for (Index r = 0; r < graph_rows; r += 37) rows.push_back((r * 7919) % graph_rows);
        LocalIndex li;
        li.build(rows, graph_rows);
        if (li.use_dense != ((Index)rows.size() * 16 >= graph_rows)) return fail("LocalIndex form", graph_rows);
        std::vector<Index> want(graph_rows, -1);
        for (Index i = 0; i < (Index)rows.size(); ++i) want[rows[i]] = i;
        for (Index r = 0; r < graph_rows; ++r)
            if (li[r] != want[r]) return fail("LocalIndex lookup", r);
    }
    std::printf("ok\n");
    return 0;
}
