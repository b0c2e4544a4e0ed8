// path_route.cuh — the path engine: accu_threshold, accu_fraction and accu_capacity (float32) as prefix
// scans along the heavy paths of the flow forest.
//
// Along one flow path the threshold rule maps the outflow x of the upstream cell to
// max(x + s - threshold, 0), the fraction rule to fraction * (x + s) and the capacity rule to
// min(x + s, capacity), where s is the material of the cell plus the outflow of its other upstream cells.
// Maps x -> max(x + a, b), x -> a * x + b and x -> min(x + a, b) compose into maps of the same form, so the
// outflows of a whole path follow from a prefix scan of the per-cell maps instead of a cell-by-cell walk
// (ALG/definition/accumulating_router.hpp:525-599 walks them one cell after the other;
// ALG/definition/accu_threshold.hpp:124-169, ALG/definition/accu_fraction.hpp:124-162 and
// ALG/definition/accu_capacity.hpp enter_cell are the cell rules).
//
// The flow forest is cut into heavy paths: each cell continues the path of its upstream neighbour with
// the largest upstream area (the heavy one); the other upstream neighbours (light) end paths of their
// own.  A path's level is 0 when no cell of it has a light upstream neighbour, else one more than the
// largest level of those light paths; every path crosses at most log2(cells) light edges, so there are
// few levels.  Paths are laid out level by level, each from its top (a cell without inflow) to its
// bottom (the cell whose downstream cell is on another path, off the array, a sink or no-data).  A call
// runs the levels in order; within a level every path is one segment of a single scan (a path's top
// map ignores its input, so segments need no flags), with the light inputs of a cell read from the
// outflows of lower levels.
//
// Built once per flow-direction raster (on the first call that needs it) and kept by the topology.
#pragma once

#include <vector>

#include "common.cuh"

namespace lue_gb300 {

constexpr int kPathThreads = 256;  // CTA of the per-call kernels

struct PathCore {
    int64_t npos = 0;                   // valid cells (positions)
    int32_t* order = nullptr;           // [npos] cell index, bit 31 set at the top cell of a path
    uint8_t* light = nullptr;           // [npos] light upstream neighbours (bit k: neighbour k, walk order)
    std::vector<int64_t> level_offsets; // [levels + 1] first position of each level
    std::vector<int> level_longest;     // [levels] cells of the longest path of each level
    int64_t tiles = 0;                  // most CTAs of one level's scan
    int64_t longest_path = 0;           // cells of the longest path
    int64_t bytes = 0;
};

struct TopologyCore;

// Builds the path layout of an acyclic raster (work: a scratch array of words_for(n) counters).
// LUE_GPU_ERANGE when the raster is beyond the engine's limits (2^31 cells).
int path_core_build(const TopologyCore* core, uint32_t* work, cudaStream_t stream, PathCore** out);
void path_core_free(PathCore* pc);

}  // namespace lue_gb300

struct lue_gpu_topology;

namespace lue_gb300 {

// accu_threshold (rule 1), accu_fraction (rule 2) and accu_capacity (rule 3), float32.  *done is false when the engine does not
// apply (flow cycles, a raster beyond its limits, LUE_GB300_ENGINE=walk or =stage): the caller then runs
// another engine.
int path_route_f32(lue_gpu_topology* t, int rule, const float* a, float as, const float* b, float bs, float* out,
                   float* rem, cudaStream_t stream, bool* done);
// Frees the handle's path-engine buffers.
void path_buffers_free(lue_gpu_topology* t);
// Builds the path layout of t now (lue_gpu_topology_prepare).
int path_prepare(lue_gpu_topology* t, cudaStream_t stream);

}  // namespace lue_gb300
