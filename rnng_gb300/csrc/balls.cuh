// Tile covers (farthest-point bisection balls) and exact tile-pair pruning.
#pragma once

#include "common.cuh"
#include "eps_l2.cuh"

namespace rnng {

// rank[child] = position of the child along a greedy nearest-neighbour chain of the
// children's landmarks within their parent (ranks stay inside the parent's range).
void chain_leaves(rnng_ctx* c, const float* lm_rows, int d, const int32_t* nchild, const int32_t* child_off,
                  int ncells, int32_t* rank);
// kTileBalls balls per tile and kSuperBalls per super-tile (greedy k-center groups).
void build_covers(rnng_ctx* c, Layout& L);
// Surviving tile pairs (i <= j) into L.pairs / L.tile_pairs.
void prune_covers(rnng_ctx* c, Layout& L);
// Items of the Gram kernel from the tile pairs: pairs sorted by (i, j), consecutive
// pairs of a row grouped nt at a time; sets L.items, L.num_items and L.item_tiles.
void schedule_items(rnng_ctx* c, Layout& L, int nt);

}  // namespace rnng
