// Drop-in utilities with the interface of RNNG's include/utils.h: index and value
// types, small helpers, RNNG's binomial coefficient, and the shared GPU context the
// other drop-in headers use.  Header-only; link with librnng_gpu.so and an MPI (or
// the single-rank shim rnng_gb300/mpi_shim).
#ifndef RNNG_DROPIN_UTILS_H_
#define RNNG_DROPIN_UTILS_H_

#undef NDEBUG
#include <assert.h>
#include <mpi.h>

#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <memory>
#include <mutex>
#include <numeric>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "rnng_gpu.h"

using Index = int64_t;  // include/utils.h:24 of RNNG
using Real = float;     // include/utils.h:25 of RNNG

#ifdef MPI_INDEX
#undef MPI_INDEX
#endif
#define MPI_INDEX MPI_INT64_T
#ifdef MPI_REAL
#undef MPI_REAL
#endif
#define MPI_REAL MPI_FLOAT

using Tuple = std::tuple<Index, Real>;
using Triple = std::tuple<Index, Index, Real>;
using IndexPair = std::tuple<Index, Index>;
using IndexVector = std::vector<Index>;
using RealVector = std::vector<Real>;
using MemVector = std::vector<void*>;
using BoolVector = std::vector<bool>;
using IndexQueue = std::deque<Index>;
using IndexMap = std::unordered_map<Index, Index>;
using IndexSet = std::unordered_set<Index>;
using IndexSetVector = std::vector<IndexSet>;
using TupleVector = std::vector<Tuple>;
using TripleVector = std::vector<Triple>;
using IndexPairVector = std::vector<IndexPair>;
using IndexIter = typename IndexVector::const_iterator;

template <class Iter>
std::string container_repr(Iter first, Iter last)
{
    std::ostringstream out;
    out << "[";
    for (Iter it = first; it != last; ++it) out << (it == first ? "" : ", ") << *it;
    out << "]";
    return out.str();
}

#define CONTAINER_REPR(container) (container_repr((container).begin(), (container).end()).c_str())

// Selection sampling (Knuth's algorithm S): each of the `range` items is taken with
// probability (still needed) / (still left); a negative seed draws one at random.
inline void selection_sample(Index range, Index size, IndexVector& sample, int seed)
{
    if (seed < 0) {
        static std::random_device device;
        seed = (int)device();
    }
    std::default_random_engine engine(seed);
    std::uniform_real_distribution<double> unit(0, std::nextafter(1.0, std::numeric_limits<double>::max()));
    sample.resize(size);
    Index taken = 0;
    for (Index i = 0; i < range && taken < size; ++i)
        if ((range - i) * unit(engine) < size - taken) sample[taken++] = i;
}

// Number with a K/M/B/T/P suffix and `prec` decimals.
inline std::string format_large_number(Index number, int prec)
{
    static const char* suffix[] = {"", "K", "M", "B", "T", "P"};
    Real value = (Real)number;
    std::ostringstream out;
    for (int k = 0; k < 6; ++k, value /= 1000) {
        if (std::abs(value) < 1000) {
            out << std::showpoint << std::fixed << std::setprecision(prec) << value << suffix[k];
            break;
        }
    }
    return out.str();
}

inline std::string format_large_number_in_bytes(Index number)
{
    static const char* suffix[] = {"B", "KB", "MB", "GB", "TB", "PB"};
    Real value = (Real)number;
    std::ostringstream out;
    for (int k = 0; k < 6; ++k, value /= 1024) {
        if (std::abs(value) < 1024) {
            out << std::showpoint << std::fixed << std::setprecision(1) << value << suffix[k];
            break;
        }
    }
    return out.str();
}

#define LARGE(number) format_large_number((number), (1)).c_str()
#define LARGE_PREC(number, prec) format_large_number((number), (prec)).c_str()
#define LARGE_BYTES(number) format_large_number_in_bytes((number)).c_str()

inline int get_comm_rank(MPI_Comm comm)
{
    int r = 0;
    MPI_Comm_rank(comm, &r);
    return r;
}

inline int get_comm_size(MPI_Comm comm)
{
    int s = 1;
    MPI_Comm_size(comm, &s);
    return s;
}

// File name without directory and extension.
inline std::string get_dataset_from_path(const char* path)
{
    const std::string p(path);
    const size_t first = p.find_last_of('/') + 1;
    return p.substr(first, p.find_last_of('.') - first);
}

template <class T>
MPI_Datatype mpi_type()
{
    if constexpr (std::is_same_v<T, char>) return MPI_CHAR;
    else if constexpr (std::is_same_v<T, signed char>) return MPI_SIGNED_CHAR;
    else if constexpr (std::is_same_v<T, short>) return MPI_SHORT;
    else if constexpr (std::is_same_v<T, int>) return MPI_INT;
    else if constexpr (std::is_same_v<T, long>) return MPI_LONG;
    else if constexpr (std::is_same_v<T, long long>) return MPI_LONG_LONG;
    else if constexpr (std::is_same_v<T, unsigned char>) return MPI_UNSIGNED_CHAR;
    else if constexpr (std::is_same_v<T, unsigned short>) return MPI_UNSIGNED_SHORT;
    else if constexpr (std::is_same_v<T, unsigned int>) return MPI_UNSIGNED;
    else if constexpr (std::is_same_v<T, unsigned long>) return MPI_UNSIGNED_LONG;
    else if constexpr (std::is_same_v<T, unsigned long long>) return MPI_UNSIGNED_LONG_LONG;
    else if constexpr (std::is_same_v<T, float>) return MPI_FLOAT;
    else if constexpr (std::is_same_v<T, double>) return MPI_DOUBLE;
    else if constexpr (std::is_same_v<T, long double>) return MPI_LONG_DOUBLE;
    else if constexpr (std::is_same_v<T, bool>) return MPI_CXX_BOOL;
    else throw std::runtime_error("error: mpi_type()");
}

// C(n, k) as RNNG's Binom forms it (include/utils.hpp:116-144): the falling product
// n (n-1) ... (n-k+1) in 64-bit integers divided by k!, 0 when k > n; memoised.
class Binom
{
  public:
    using Pair = std::pair<Index, Index>;
    struct HashPair {
        size_t operator()(const Pair& p) const
        {
            const size_t a = std::hash<Index>{}(p.first), b = std::hash<Index>{}(p.second);
            return a ^ (b + 0x9e3779b9 + (a << 6) + (a >> 2));
        }
    };
    using Memo = std::unordered_map<Pair, Index, HashPair>;

    Binom() {}

    Index operator()(Index n, Index k)
    {
        if (k > n) return 0;
        const Pair key{n, k};
        auto it = memo.find(key);
        if (it != memo.end()) return it->second;
        uint64_t top = 1, bottom = 1;  // unsigned: wraps where a signed product would overflow
        for (Index i = n; i >= n - k + 1; --i) top *= (uint64_t)i;
        for (Index i = k; i >= 1; --i) bottom *= (uint64_t)i;
        const Index value = (Index)top / (Index)bottom;
        memo.emplace(key, value);
        return value;
    }

  private:
    Memo memo;
};

namespace rnng_dropin {

// One GPU context per process (device from RNNG_DEVICE, default 0), created on first use.
inline rnng_ctx* context()
{
    static std::once_flag once;
    static rnng_ctx* ctx = nullptr;
    std::call_once(once, [] {
        const char* env = std::getenv("RNNG_DEVICE");
        const int dev = env ? std::atoi(env) : 0;
        if (rnng_ctx_create(dev, &ctx) != RNNG_OK) {
            std::fprintf(stderr, "rnng: cannot create a GPU context on device %d\n", dev);
            std::abort();
        }
    });
    return ctx;
}

// RNNG's error convention is an assertion; a failed GPU call aborts with its message.
inline void check(int rc, const char* what)
{
    if (rc != RNNG_OK) {
        std::fprintf(stderr, "rnng: %s failed (%d): %s\n", what, rc, rnng_last_error(context()));
        std::abort();
    }
}

}  // namespace rnng_dropin

#endif  // RNNG_DROPIN_UTILS_H_
