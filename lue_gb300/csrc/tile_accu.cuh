// tile_accu.cuh — the tiled accu engine: resident tile topology and per-call scratch.
//
// The raster is cut into 64 x 64 tiles (the GPU's partitions).  Once, when the topology is built, each
// tile's solve is compiled into a schedule: its valid cells grouped in rounds (a round's cells depend
// only on cells of earlier rounds), each cell with its in-tile upstream mask; the same for the cells
// downstream of a tile entry.  Per call, a tile's solve replays its schedule (one barrier per round,
// 3 bytes of schedule read per cell) instead of re-deriving it from the flow direction:
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
constexpr int kBorderCells = 4 * kTile - 4;  // cells on the tile's border ring

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
    // Per-tile solve schedules, compiled once from the flow direction (so no call re-derives them):
    uint16_t* sched_order = nullptr;           // [ntiles * 4096] valid cells, grouped by in-tile round
    uint8_t* sched_upm = nullptr;              // [ntiles * 4096] in-tile upstream mask of sched_order[k]
    uint16_t* thr_order = nullptr;             // [ntiles * 4096] cells downstream of a tile entry, by round
    uint8_t* thr_upm = nullptr;                // [ntiles * 4096] their upstream mask, restricted to such cells
    int32_t* round_base = nullptr;             // [ntiles + 1] first entry of each tile in round_off
    uint16_t* round_off = nullptr;             // per tile: rounds + 1 offsets into sched_order
    uint16_t* thr_round_off = nullptr;         // per tile: the same rounds' offsets into thr_order
    uint16_t* tails = nullptr;                 // [ntiles * 2] first round of the warp phase (all, through)
    uint32_t* valid_bits = nullptr;            // [ntiles * 128] bit per cell: inside the array, not no-data
    uint8_t* border_in = nullptr;              // [ntiles * kBorderCells] per border cell: outside neighbours draining in
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
