// tile_accu.cuh — the tiled accu engine: resident tile topology and per-call scratch.
//
// The raster is cut into 64 x 64 tiles (the GPU's partitions).  Inside a tile, the flow paths form a
// forest; once, when the topology is built, it is laid out in post-order, so that the accu of a cell
// (the material of its in-tile subtree) is the difference of two prefix sums of the material taken in
// that order.  Per call:
//   1. k_tile_exits: one CTA per tile gathers its material into post-order (each thread a run of 18
//      positions), takes one exact 64-bit fixed-point prefix sum, and writes the local value of each
//      exit cell (a cell whose flow leaves its tile but not the array) to P, in the post-order of the
//      exit forest.
//   2. Exit forest: exit y's parent is the exit reached by following the flow from y's downstream
//      cell through that cell's tile.  The final value of exit y is the sum of the local values over
//      y's subtree of this forest, so an inclusive prefix sum over P in post-order gives every subtree
//      sum as a difference of two prefix sums.  The sums are exact: 128-bit fixed point (96 value bits,
//      32 bits counting no-data exits), so summation order cannot change the result.
//   3. k_tile_accu: one CTA per tile puts, at each border cell's entry node, the subtree sums of the
//      exits draining into it, takes the same prefix sum again and writes every cell's result.
// Both tile passes read the material once (coalesced float4 rows) and 2-4 bytes of forest per cell; the
// prefix sums stay in registers and shared memory.
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

// Per-tile post-order with virtual entry nodes.  The post-order of a tile's flow forest gets one extra
// node per border cell that receives inflow from outside the tile (its "entry", placed first among that
// cell's children), so that what enters the tile is just one more term of the prefix sum.  Cells
// (4096) and entries (at most 252) fill positions 0 .. 4347; positions up to kRunPositions are padding.
// Scan thread t owns the run of positions 18 t .. 18 t + 17; scan slot = position, and slot kZeroSlot
// holds 0 (the prefix before position 0).  Per-position tables are stored word-transposed: the 16-bit
// entries of positions 18 t + 2 i and 18 t + 2 i + 1 form word i of thread t, at word index 256 i + t,
// so that each of a thread's nine table loads is one coalesced 128-byte line per warp.
constexpr int kRun = 18;
constexpr int kRunWords = kRun / 2;
constexpr int kRunPositions = kRun * kTileThreads;  // 4608
constexpr int kZeroSlot = kRunPositions;
constexpr int kScanSlotCount = kRunPositions + 2;
constexpr int kEntryBase = kTileCells;             // material index of entry b: kEntryBase + b
__host__ __device__ __forceinline__ int run_table_index(int p)
{
    const int t = p / kRun, j = p - kRun * t;
    return ((j >> 1) * kTileThreads + t) * 2 + (j & 1);
}

// cell_at entries: the material index (a cell 0..4095, or kEntryBase + border index) and two flags.
constexpr unsigned kIndexMask = 0x1FFFu;
constexpr unsigned kNoOutput = 0x4000u;  // an entry or padding: no result
constexpr unsigned kNoValue = 0x8000u;   // no-data flow direction, outside the array, or padding: term 0
// prev_at entries: the scan slot just before the node's subtree, and a flag.
constexpr unsigned kSlotMask = 0x1FFFu;
constexpr unsigned kPrevRidge = 0x8000u;  // the subtree is the cell alone

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
    // Per-tile flow forests in post-order (built once from the flow direction), by post-order position:
    uint16_t* cell_at = nullptr;               // [ntiles * kRunPositions] material index at the position
                                               // (| kNoOutput, kNoValue); no-data cells after the valid ones
    uint16_t* prev_at = nullptr;               // [ntiles * kRunPositions] scan slot before the subtree
                                               // (kZeroSlot for a subtree at position 0) | kPrevRidge
    uint32_t* exit_span = nullptr;             // [nexit] scan slots of each exit cell: own | before << 16
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
