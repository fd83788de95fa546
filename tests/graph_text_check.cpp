// Writes a Graph of synthetic edges through the drop-in write_file (the collective form the
// drivers call) so that a test can compare the text with printf-style formatting.
// Usage: graph_text_check <edges> <out file>
#include <cstdlib>

#include "graph.h"

int main(int argc, char** argv)
{
    MPI_Init(&argc, &argv);
    const Index m = std::atoll(argv[1]);
    Graph::EdgeVector edges;
    edges.reserve((size_t)m);
    uint64_t s = 12345;
    for (Index i = 0; i < m; ++i) {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        const Index u = i / 7, v = (Index)((s >> 33) % 1000003);
        // weights across many magnitudes, including integers and values that round up
        const float w = (float)((double)(s >> 40) / (double)(1 << 12) * ((i % 5 == 0) ? 1e-3 : 1.0));
        edges.emplace_back(u, v, (i % 11 == 0) ? (Real)(i % 97) : w);
    }
    Graph g(edges, m / 7 + 1);
    g.write_file(argv[2], MPI_COMM_WORLD);
    MPI_Finalize();
    return 0;
}
