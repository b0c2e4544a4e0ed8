// topology.cuh — the resident flow topology of one D8 raster and its per-handle scratch.
#pragma once

#include <atomic>
#include <vector>

#include "common.cuh"
#include "path_route.cuh"
#include "stage_route.cuh"
#include "tile_accu.cuh"

namespace lue_gb300 {

// Immutable part, shared by a topology and its clones.
struct TopologyCore {
    int64_t rows = 0, cols = 0, prow = 0, pcol = 0, n = 0;
    uint8_t* fd = nullptr;      // device copy of the flow direction raster
    uint8_t* count = nullptr;   // inflow count, 255 where the flow direction is no-data
    uint8_t* upmask = nullptr;  // bit k set: neighbour k (NW, N, NE, W, E, SW, S, SE) drains here
    int32_t* level = nullptr;   // downstream level, -1 for no-data and cycle cells
    TileCore* tiles = nullptr;  // tiled accu engine (acyclic rasters), else nullptr
    int32_t* order = nullptr;   // valid cells sorted by downstream level (built on first multi-step call)
    std::vector<int32_t> level_offsets;  // [levels + 1] start of each level in `order`
    StageCore* stages = nullptr;         // stage engine (acyclic rasters; built on first use)
    int stage_cap = 0;                   // most cells of one stage when built (0: LUE_GB300_STAGE_CAP or 128)
    int stage_order = LUE_GPU_STAGE_ORDER_LATEST;  // ticket order of the stage structures when built
    bool stages_unavailable = false;     // the raster is beyond the stage engine's limits
    PathCore* paths = nullptr;           // path engine (acyclic rasters; built on first use)
    bool paths_unavailable = false;      // the raster is beyond the path engine's limits
    std::mutex stage_mutex;              // guards the first build of stages and paths (clones share the core)
    lue_gpu_topology_stats stats{};
    int64_t bytes = 0;
    std::atomic<int> refs{1};
};

}  // namespace lue_gb300

struct lue_gpu_topology {
    lue_gb300::TopologyCore* core = nullptr;
    uint32_t* work_count = nullptr;  // per-call copy of the counts, 4 cells per word
    float* lo = nullptr;             // per-call float-float residuals of f32 routing
    lue_gb300::TileScratch tile_scratch;
    double* history = nullptr;       // discharge planes of multi-step kinematic wave (grown on demand)
    size_t history_bytes = 0;
    double** planes = nullptr;       // device array of plane pointers
    size_t plane_capacity = 0;
    uint2* stage_hist = nullptr;     // stage engine: outflow history of the stage exits (grown on demand)
    size_t stage_hist_bytes = 0;
    int* stage_flow = nullptr;       // stage engine, dataflow mode: per-stage progress, ticket and error flag
    size_t stage_flow_bytes = 0;
    int* stage_flow_error = nullptr; // pinned: the error flag of the last dataflow launch, read by the next call
    int stage_threads = 0;           // stage engine: threads per stage CTA (0: LUE_GB300_STAGE_THREADS or by size)
    int publish_every = 0;           // stage engine: steps per progress publication (0: LUE_GB300_PUBLISH_EVERY or 4)
    void* path_maps = nullptr;       // path engine: per tile of a level's scan its own and its inclusive map
    int* path_status = nullptr;      // path engine: per tile its published state, then one ticket per level
    int path_epoch = 0;              // path engine: tag of the last launch's status words
    unsigned long long* path_flag = nullptr;  // path engine: [2], [1] set when the walk engine must redo a call
    int64_t scratch_bytes = 0;
};

namespace lue_gb300 {

int allocate_scratch(lue_gpu_topology* t);

// The reference's partitions of a raster: the last partition of a row or column absorbs the remainder
// (source/framework/core/include/lue/framework/core/domain_decomposition.hpp:90-175).
struct PartitionGeom {
    int64_t rows, cols, prow, pcol, nprow, npcol;
    __device__ __forceinline__ int64_t prow_of(int64_t r) const { return min(r / prow, nprow - 1); }
    __device__ __forceinline__ int64_t pcol_of(int64_t c) const { return min(c / pcol, npcol - 1); }
};
inline PartitionGeom partition_geom(const TopologyCore* core)
{
    return PartitionGeom{core->rows, core->cols, core->prow, core->pcol, core->rows / core->prow,
                         core->cols / core->pcol};
}

// accu (float32) on the tile engine; see tile_accu.cuh.
int tile_accu_f32(const TopologyCore* core, TileScratch* s, const float* ext, float ext_s, float* out,
                  cudaStream_t stream);

// Launch of the walk engine: one thread per cell; cells without inflow start a downstream walk that
// continues through a cell once all its upstream neighbours are done (definition/accumulating_router.hpp:
// 525-599, run by many threads at once).
inline int64_t words_for(int64_t n) { return (n + 3) / 4; }

}  // namespace lue_gb300
