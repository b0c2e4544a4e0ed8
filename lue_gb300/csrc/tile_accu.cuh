// tile_accu.cuh — the tiled accu engine: resident tile topology and per-call scratch.
//
// The raster is cut into 64 x 64 tiles (the GPU's partitions).  Inside a tile, the flow paths form a
// forest; once, when the topology is built, it is laid out in post-order, so that the accu of a cell
// (the material of its in-tile subtree) is the difference of two prefix sums of the material taken in
// that order.  Per call:
//   1. k_tile_exits: one CTA per tile gathers its material into post-order and writes the local value of
//      each exit cell (a cell whose flow leaves its tile but not the array: the material of its in-tile
//      subtree) to P, in the post-order of the exit forest, with per-tile statistics of the material for
//      pass 3.  An exit is a root of the tile's forest, and the subtrees of the roots are consecutive runs
//      of positions, so its value is a segmented sum (float-float, no cancellation).
//   2. k_scan_exits, over the exit forest: exit y's parent is the exit reached by following the flow
//      from y's downstream cell through that cell's tile.  The final value of exit y is the sum of the
//      local values over y's subtree of this forest, so an inclusive prefix sum over P in post-order
//      gives every subtree sum as a difference of two prefix sums.  The sums are exact: 128-bit fixed point (96 value bits,
//      32 bits counting no-data exits), so summation order cannot change the result.
//   3. k_slot_inflow: per border cell that receives flow from other tiles, the exact sum of the subtree
//      sums of the exits draining into it, rounded to float once.
//   4. k_tile_accu: one CTA per tile adds to each border cell what enters it, takes the same prefix sum
//      over the tile's post-order and writes every cell's result.
// Pass 1 reads the material and 2 bytes of post-order table per cell; pass 3 the material and 4 bytes of
// tables, and writes the result.  The prefix sums stay in registers and shared memory.
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

// Per-tile post-order: valid cells take positions 0 .. nvalid - 1, cells with a no-data flow direction
// (or outside the array) the positions after them.  Scan thread t owns the run of positions 16 t ..
// 16 t + 15.  Prefix sums are kept in shared memory by scan slot: position p has slot p + p / 16, so
// that each thread's run is 136 bytes and the 8-byte accesses of a warp at one offset into the runs
// (the stores of the scan, the reads of the prefix just before a small subtree) fall on distinct banks
// in pairs of lanes; slot kZeroSlot holds 0 (the prefix before position 0).  Per-position tables are stored
// word-transposed: the 16-bit entries of positions 16 t + 2 i and 16 t + 2 i + 1 form word i of thread
// t, at word index 256 i + t, so that each of a thread's eight table loads is one coalesced 128-byte
// line per warp.
constexpr int kRun = 16;
constexpr int kRunWords = kRun / 2;
constexpr int kRunPositions = kRun * kTileThreads;  // 4096: every cell of the tile, nothing else
constexpr int kRunSlots = kRun + 1;                 // scan slots per thread run (one pad slot)
constexpr int kZeroSlot = kRunSlots * kTileThreads; // 4352
constexpr int kScanSlotCount = kZeroSlot + 2;
__host__ __device__ __forceinline__ int run_table_index(int p)
{
    const int t = p / kRun, j = p - kRun * t;
    return ((j >> 1) * kTileThreads + t) * 2 + (j & 1);
}
__host__ __device__ __forceinline__ int scan_slot(int p) { return p + p / kRun; }

// cell_at entries: the cell (0..4095) and two flags.
constexpr unsigned kIndexMask = 0x0FFFu;
constexpr unsigned kSegHead = 0x4000u;   // the first position of a root's subtree (a no-data cell is its own)
constexpr unsigned kNoValue = 0x8000u;   // no-data flow direction or outside the array: result NaN / none
constexpr unsigned kLoneCell = 0x1000u;  // the subtree is the cell alone (no in-tile upstream cell)
// prev_at entries: the byte offset in the tile's scan array (8 bytes per scan slot) of the slot just
// before the node's subtree, so that pass 3 addresses shared memory with the entry itself.

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
    uint16_t* cell_at = nullptr;               // [ntiles * kRunPositions] cell at the position (| kNoValue)
    uint16_t* prev_at = nullptr;               // [ntiles * kRunPositions] 8 x the scan slot before the
                                               // subtree (kZeroSlot for a subtree at position 0)
    uint32_t* exit_span = nullptr;             // [nexit] scan slots of each exit cell: own | before << 16
    uint8_t* border_in = nullptr;              // [ntiles * kBorderCells] per border cell: outside neighbours draining in
    // Inflow slots (border cells that receive flow from other tiles), per tile in border order:
    int64_t nslot = 0;
    int32_t* slot_at = nullptr;                // [nslot] tile * kSlotStride + border index
    int32_t* slot_first = nullptr;             // [nslot + 1] first of the slot's upstream exits in slot_edge
    int2* slot_edge = nullptr;                 // [slot_first[nslot]] per exit draining into the slot: its
                                               // exit-forest position, and the position before its subtree
                                               // (-1: none)
    int64_t bytes = 0;
};

constexpr int kSlotStride = 256;  // inflow values per tile (252 border cells, padded)

// What pass 1 learns about a tile's material (valid cells only), for pass 3.
struct TileStat {
    float bound;          // upper bound of the tile's material total
    unsigned min_bits;    // bits of the smallest positive term minus one (0xFFFFFFFF: none)
    unsigned bad;         // a NaN or negative term
    unsigned pad;
};

struct TileScratch {
    float2* P = nullptr;                       // [nexit] local exit values (hi, lo), post-order
    uint4* S = nullptr;                        // [nexit] inclusive prefix sums (128-bit), post-order
    float* inflow = nullptr;                   // [ntiles * kSlotStride] what enters each border cell (0 where
                                               // nothing does), float, NaN when no-data enters
    uint4* look_aggr = nullptr;                // [scan blocks] each block's sum (decoupled look-back)
    uint4* look_incl = nullptr;                // [scan blocks] the sum up to and including the block
    // Zeroed before each call, in one memset of ctl_bytes: total[0] = bound of the material total
    // (2^-16 units, summed by pass 1), total[1] = fallback flag, then the scan's ticket and block flags.
    unsigned long long* total = nullptr;
    int64_t ctl_bytes = 0;
    TileStat* stat = nullptr;                  // [ntiles]
    int64_t bytes = 0;
};

struct TopologyCore;

int tile_core_build(TopologyCore* core, cudaStream_t stream);
void tile_core_free(TileCore* tc);
int tile_scratch_alloc(const TileCore* tc, TileScratch* s);
void tile_scratch_free(TileScratch* s);

}  // namespace lue_gb300
