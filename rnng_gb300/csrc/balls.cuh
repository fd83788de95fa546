// Tile covers (farthest-point bisection balls) and exact tile-pair pruning.
#pragma once

#include "common.cuh"
#include "eps_l2.cuh"

namespace rnng {

// rank[child] = position of the child along a greedy nearest-neighbour chain of the
// children's landmarks within their parent (ranks stay inside the parent's range).
void chain_leaves(rnng_ctx* c, const float* lm_rows, int d, const int32_t* nchild, const int32_t* child_off,
                  int ncells, int32_t* rank);
// kBalls balls per tile and per super-tile.
void build_covers(rnng_ctx* c, Layout& L);
// Surviving tile pairs (i <= j) into L.pairs / L.tile_pairs.
void prune_covers(rnng_ctx* c, Layout& L);
// Sorts the tile pairs for G persistent CTAs (row tiles i = g mod G per CTA g, then
// i, then j) and sets L.sched[g] = first pair of CTA g (L.sched[G] = end).
void schedule_pairs(rnng_ctx* c, Layout& L, int G);

}  // namespace rnng
