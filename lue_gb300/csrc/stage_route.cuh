// stage_route.cuh — the stage engine: routing rules that are not plain sums, swept tile by tile.
//
// accu_threshold, accu_fraction and kinematic_wave compute each cell from the sum of its upstream
// outflows with a rule that does not distribute over sums, so they cannot use the prefix sums of the
// tile engine.  The reference walks them cell by cell, partition by partition, with channel hand-off at
// partition edges (ALG/definition/accumulating_router.hpp:525-599, 902-1209).  Here:
//
//   - The raster is cut into 32 x 32 tiles.  The crossing depth of a cell is the largest number of tile
//     edges crossed by a flow path that ends at the cell.  The cells of one tile with the same crossing
//     depth form a depth group; every upstream cell of a group lies in the group itself, in a group of
//     lower depth, or nowhere.
//   - The cells of a group are sorted by decreasing distance, in cells, to the group's most downstream
//     cells, so every in-group upstream cell of a cell comes before it.  A stage is a run of at most
//     `cap` (128) consecutive cells of that order; the rounds of a stage count that distance from its
//     first cell, and every cell is exactly one round after each of its upstream cells in the stage
//     (each cell has one downstream cell).  Outflows that go to another stage are exits.
//   - A stage runs in one CTA: the cells of a round are computed together from shared memory, and the
//     exits' outflows go to a history in global memory, where later stages read them.
//   - Time steps are pipelined: cell c does step t in round round(c) + t, so T steps of a stage take
//     rounds + T - 1 rounds.  All stages and steps run in one launch in which each stage waits, step by
//     step, for the exits it reads (stage_route.cu, k_stage_flow).
//
// Built once per flow-direction raster (on the first call that needs it) and kept by the topology.
#pragma once

#include <mutex>
#include <vector>

#include "common.cuh"

namespace lue_gb300 {

constexpr int kStageSide = 32;                        // tile side (cells)
constexpr int kStageCells = kStageSide * kStageSide;  // 1024
constexpr int kStageThreads = 256;                    // runtime CTA for stages of more than 256 cells
constexpr int kStageBuildThreads = 512;               // build CTA: two cells per thread
constexpr int kStageCap = 128;                        // default largest stage (cells; LUE_GB300_STAGE_CAP)
constexpr int kStageMaxCap = 256;                     // stage positions fit in a byte

// meta (per cell, by tile and position in the tile's stage order):
//   x: in-tile cell (bits 0-9) | round (bits 10-19)
//   y: upstream mask (bits 0-7) | mask of upstream cells in other stages (bits 8-15) | index of the cell's
//      first input in its stage's input list (bits 16-31)
struct StageCore {
    int64_t trows = 0, tcols = 0, ntiles = 0;
    int64_t nstages = 0, nexits = 0, ninputs = 0;
    int cap = kStageCap;               // most cells of one stage
    int64_t max_depth = 0;             // deepest stage
    int64_t max_stage_cells = 0;       // most cells of one stage (at most cap)
    int64_t max_stage_inputs = 0;      // most inputs of one stage
    int64_t max_stages_per_depth = 0;
    int4* stage = nullptr;             // [nstages] tile, begin | count << 16, rounds | inputs << 16, input base
    int32_t* wave_stage = nullptr;     // [nstages] stage ids in ticket order (see stage_core_build)
    uint2* meta = nullptr;             // [ntiles * 1024]
    int32_t* exit_id = nullptr;        // [ntiles * 1024] history row of the cell, or -1 (outflow stays in the stage)
    int32_t* inputs = nullptr;         // [ninputs] history row of the upstream cell of each edge into a stage
    // Dataflow order (by position k in wave_stage): the stages whose exits feed stage k, each with the
    // earliest round at which stage k consumes them, and the latest round of stage k's own exits.
    int64_t* prod_offsets = nullptr;   // [nstages + 1]
    int2* prod = nullptr;              // [prod_offsets[nstages]] (producer position, earliest consumer round)
    int32_t* max_exit_round = nullptr; // [nstages] -1 without exits
    int64_t max_producers = 0;
    int64_t bytes = 0;
};

struct TopologyCore;
struct BetaRational;

// Builds the stage topology of an acyclic raster (work: a scratch array of words_for(n) counters).
int stage_core_build(const TopologyCore* core, uint32_t* work, cudaStream_t stream, StageCore** out);
void stage_core_free(StageCore* sc);

}  // namespace lue_gb300

struct lue_gpu_topology;

namespace lue_gb300 {

// Routing on the stage engine.  *done is false when the engine does not apply to the topology (flow
// cycles, or a raster beyond its limits): the caller then runs the walk engine.  rule: a value of Rule
// (route_walk_visitors.cuh): 0 accu (float64 only), 1 threshold, 2 fraction, 3 capacity, 4 trigger.
// Frees the handle's stage buffers (history, flow counters) back to their pool, after the work queued so
// far on the default stream.
void stage_buffers_free(lue_gpu_topology* t);
// Builds the stage topology of t now (lue_gpu_topology_prepare).
int stage_prepare(lue_gpu_topology* t, cudaStream_t stream);
// Schedule of the stage engine for handle t: the cap of the shared stage structures and the handle's
// threads per stage CTA and steps per progress publication (lue_gpu_topology_{get,set}_stage_schedule).
// Setting another cap frees the stage structures (rebuilt by the next call); refused while clones share them.
void stage_schedule_get(const lue_gpu_topology* t, int* cap, int* threads, int* publish_every);
int stage_schedule_set(lue_gpu_topology* t, int cap, int threads, int publish_every);
int stage_order_set(lue_gpu_topology* t, int order);
int stage_route_f32(lue_gpu_topology* t, int rule, const float* a, float as, const float* b, float bs, float* out,
                    float* rem, cudaStream_t stream, bool* done);
int stage_route_f64(lue_gpu_topology* t, int rule, const double* a, double as, const double* b, double bs,
                    double* out, double* rem, cudaStream_t stream, bool* done);
int stage_kinematic_wave_f64(lue_gpu_topology* t, const double* qcur, double qcur_s, const double* lateral,
                             double lateral_s, const double* alpha, double alpha_s, const double* beta, double beta_s,
                             double dt, const double* dx, double dx_s, double* out, const BetaRational& br,
                             cudaStream_t stream, bool* done);
int stage_kinematic_wave_f32(lue_gpu_topology* t, const float* qcur, float qcur_s, const float* lateral,
                             float lateral_s, const float* alpha, float alpha_s, const float* beta, float beta_s,
                             float dt, const float* dx, float dx_s, float* out, cudaStream_t stream, bool* done);
int stage_kinematic_wave_f32in(lue_gpu_topology* t, const double* qcur, double qcur_s, const float* lateral,
                               double lateral_s, const float* alpha, double alpha_s, double beta, double dt, double dx,
                               double* out, const BetaRational& br, cudaStream_t stream, bool* done);
// `steps` kinematic-wave steps with the float-float solve (scalar rational beta).
int stage_kinematic_wave_steps(lue_gpu_topology* t, const double* qcur, const float* lateral, double lateral_s,
                               const float* alpha, double alpha_s, double beta, double dt, double dx, int steps,
                               double* out, const BetaRational& br, cudaStream_t stream, bool* done);

}  // namespace lue_gb300
