// tile_accu.cuh — the tiled accu engine: resident tile topology and per-call scratch.
//
// The raster is cut into 64 x 64 tiles (the GPU's partitions).  Per call:
//   1. k_tile_local: one CTA per tile solves accu inside the tile in shared memory, ignoring flow that
//      enters from other tiles, and writes that local result for every cell.  The local result of each
//      exit cell (a cell whose flow leaves its tile but not the array) goes to P, in the post-order of
//      the exit forest.
//   2. Exit forest: exit y's parent is the exit reached by following the flow from y's downstream
//      cell through that cell's tile.  The final value of exit y is the sum of the local values over
//      y's subtree of this forest, so an inclusive prefix sum over P in post-order gives every subtree
//      sum as a difference of two prefix sums.  The sums are exact: 128-bit fixed point (96 value bits,
//      32 bits counting no-data exits), so summation order cannot change the result.
//   3. k_tile_fixup: one CTA per tile adds, to every cell downstream of a tile entry, the exact sum of
//      what enters the tile upstream of it.
// Reference counterpart: the per-partition intra/inter split of ALG/definition/accumulating_router.hpp
// (intra :789-899, inter :902-1209), with the inter-partition channel hand-off replaced by the exit-forest
// prefix sum.
#pragma once

#include "common.cuh"

namespace lue_gb300 {

constexpr int kTile = 64;                 // tile side (cells)
constexpr int kTileCells = kTile * kTile;
constexpr int kHalo = kTile + 2;          // tile side with a one-cell halo
constexpr int kHaloSlots = 4 * kTile + 4; // N row, S row, W column, E column, NW, NE, SW, SE corners
constexpr int kTileThreads = 256;

struct TileCore {
    int64_t trows = 0, tcols = 0, ntiles = 0;  // tile grid
    int64_t nexit = 0;                         // exits (coarse nodes)
    int64_t max_depth = 0;                     // depth of the exit forest
    int32_t* exit_base = nullptr;              // [ntiles + 1] first exit id of each tile (tile-major ids)
    uint16_t* exit_local = nullptr;            // [nexit] cell index inside its tile (row * 64 + col)
    uint32_t* exit_pos = nullptr;              // [nexit] post-order position
    uint32_t* exit_start = nullptr;            // [nexit] post-order position of the first node of the subtree
    int32_t* halo_exit = nullptr;              // [ntiles * kHaloSlots] exit id of the halo cell draining into
                                               // the tile, or -1
    int64_t bytes = 0;
};

struct TileScratch {
    float2* P = nullptr;                       // [nexit] local exit values (hi, lo), post-order
    uint4* S = nullptr;                        // [nexit] inclusive prefix sums (128-bit), post-order
    uint4* A = nullptr;                        // [nexit] subtree sums (128-bit), exit-id order
    uint4* block_sums = nullptr;               // [scan blocks]
    unsigned long long* total = nullptr;       // [2] material total bound (2^-16 units), fallback flag
    unsigned long long* block_total = nullptr; // [ntiles] per-tile bounds
    int64_t bytes = 0;
};

struct TopologyCore;

int tile_core_build(TopologyCore* core, cudaStream_t stream);
void tile_core_free(TileCore* tc);
int tile_scratch_alloc(const TileCore* tc, TileScratch* s);
void tile_scratch_free(TileScratch* s);

}  // namespace lue_gb300
