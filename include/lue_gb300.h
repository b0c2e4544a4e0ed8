/*
 * lue_gb300.h — C ABI of the GB300-native flow-routing path.
 *
 * Drop-in boundary for LUE's routing operations on D8 rasters (computationalgeography/lue, paths
 * below are relative to source/framework/algorithm/include/lue/framework/algorithm/):
 *
 *   LUE operation (C++ template, PartitionedArray in/out)        entry point here
 *   ----------------------------------------------------------   -----------------------------------
 *   inflow_count<uint8>(policies, fd)  inflow_count.hpp:29-42      lue_gpu_inflow_count_u8
 *   value_policies::accu_info(fd)      value_policies/accu_info.hpp:18-26   lue_gpu_accu_info_u8
 *   value_policies::partial_accu(fd, inflow, nr_steps)
 *                                      value_policies/partial_accu.hpp:17-28
 *                                                                  lue_gpu_partial_accu_f32 / _f64
 *   value_policies::accu(fd, inflow)   value_policies/accu.hpp:33-55   lue_gpu_accu_f32 / _f64
 *   value_policies::accu_threshold(fd, inflow, threshold)
 *                                      value_policies/accu_threshold.hpp:33-90
 *                                                                  lue_gpu_accu_threshold_f32 / _f64
 *   value_policies::accu_fraction(fd, inflow, fraction)
 *                                      value_policies/accu_fraction.hpp:33-90
 *                                                                  lue_gpu_accu_fraction_f32 / _f64
 *   value_policies::accu_capacity / accu_trigger (fd, inflow, capacity | trigger)
 *                                      value_policies/accu_{capacity,trigger}.hpp
 *                                                                  lue_gpu_accu_{capacity,trigger}_f32 / _f64
 *   value_policies::upstream / downstream (fd, material)
 *                                      value_policies/{upstream,downstream}.hpp
 *                                                                  lue_gpu_{upstream,downstream}_f32 / _f64
 *   downstream_distance(fd, cell_size) downstream_distance.hpp:31-44
 *                                                                  lue_gpu_downstream_distance_f32 / _f64
 *   value_policies::kinematic_wave(fd, current_outflow, inflow, alpha, beta,
 *                                  time_step_duration, channel_length)
 *                                      value_policies/kinematic_wave.hpp:43-91
 *                                                                  lue_gpu_kinematic_wave_f64 / _f32
 *                                                                  (+ _f64_f32in: float32 lateral
 *                                                                   inflow and alpha rasters)
 *
 * The per-call inflow-count pass and the partition-connectivity exchange of the reference
 * (definition/accumulating_router.hpp:1212-1247, definition/inflow_count.hpp:97-577) become a resident
 * topology built once per flow-direction raster (lue_gpu_topology_create) and reused by every call.
 *
 * Conventions
 *   - Rasters are row-major (the reference's mdspan layout_right), in device memory, owned by the
 *     caller.  Flow direction is uint8 with the keypad D8 codes (flow_direction.hpp:7-35); 255 is
 *     no-data.  Float no-data is NaN (policy/default_value_policies.hpp:18-29).
 *   - A raster argument that may also be a scalar (the reference's PartitionedArray | Scalar
 *     overloads) is a pointer plus a value: a NULL pointer selects the scalar.
 *   - `stream` is a cudaStream_t (NULL = legacy default stream).  Routing calls are asynchronous on it;
 *     lue_gpu_topology_create synchronises its stream before returning.
 *   - Every function returns a status (LUE_GPU_OK on success) and never throws;
 *     lue_gpu_last_error() describes the last failure of the calling thread.
 *   - Invalid values do not fail a call: they become NaN (floats) or 255 (counts) in the output,
 *     exactly like the reference's value policies.  A shape mismatch fails with LUE_GPU_ESHAPE, where
 *     the reference throws std::runtime_error (detail/verify_compatible.hpp:23-40).
 *   - The partition shape is kept for interface parity and validated like the reference's domain
 *     decomposition (partition extents must be positive and not larger than the array); results do
 *     not depend on it beyond floating-point summation order.
 *   - A topology holds per-call scratch memory: calls that use the same topology must not overlap in
 *     time (issue them on one stream).  lue_gpu_topology_clone gives another handle that shares the
 *     immutable flow topology and has its own scratch.
 */
#ifndef LUE_GB300_H
#define LUE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LUE_GPU_ABI_VERSION 1

enum lue_gpu_status {
    LUE_GPU_OK = 0,
    LUE_GPU_EINVAL = 1,    /* bad argument: NULL pointer, non-positive extent, bad partition shape */
    LUE_GPU_ESHAPE = 2,    /* arrays of different shape / partitioning */
    LUE_GPU_ECUDA = 3,     /* a CUDA runtime call failed */
    LUE_GPU_ENOMEM = 4,    /* device allocation failed */
    LUE_GPU_ETIMEDOUT = 5, /* a bounded device-side wait gave up (no result written) */
    LUE_GPU_ERANGE = 6     /* a size beyond a documented maximum */
};

typedef struct lue_gpu_topology lue_gpu_topology;

typedef struct lue_gpu_topology_stats {
    int64_t rows, cols;
    int64_t partition_rows, partition_cols;
    int64_t valid_cells;       /* flow direction is not no-data */
    int64_t ridge_cells;       /* valid cells without inflow */
    int64_t outlet_cells;      /* valid cells whose flow leaves the array */
    int64_t sink_cells;        /* valid cells with code 5 or an unknown code */
    int64_t cycle_cells;       /* valid cells on or downstream of a flow cycle (never routed) */
    int64_t max_level;         /* largest downstream level (longest flow path minus one) */
    int64_t device_bytes;      /* device memory held by this handle */
    int64_t tile_exits;        /* cells whose flow leaves their 64 x 64 tile (0: tile engine off) */
    int64_t exit_forest_depth; /* depth of the forest of those exits */
} lue_gpu_topology_stats;

/* Library */
int lue_gpu_abi_version(void);
const char* lue_gpu_last_error(void);
/* Number of CUDA kernels this library has launched in this process (for benchmarks and tests). */
unsigned long long lue_gpu_kernel_launches(void);

/* Topology: built once per flow-direction raster, resident on the device. */
int lue_gpu_topology_create(const uint8_t* flow_direction, int64_t rows, int64_t cols,
                            int64_t partition_rows, int64_t partition_cols, void* stream,
                            lue_gpu_topology** topology);
int lue_gpu_topology_clone(const lue_gpu_topology* topology, lue_gpu_topology** clone);
int lue_gpu_topology_destroy(lue_gpu_topology* topology);
int lue_gpu_topology_get_stats(const lue_gpu_topology* topology, lue_gpu_topology_stats* stats);
/* Builds now, on `stream`, what the first call of an operation would otherwise build: the path layout of
 * float32 accu_threshold / accu_capacity and the stage structures of accu_threshold / accu_fraction /
 * accu_capacity / accu_trigger / float64 accu / kinematic_wave (shared by the clones of the handle).
 * Returns when they are built.  A serving loop
 * calls it when it loads a raster, so that no request pays for it.  (No reference counterpart: the
 * reference keeps no state between calls.) */
int lue_gpu_topology_prepare(lue_gpu_topology* topology, void* stream);

/* Schedule of the stage engine (accu_threshold, accu_fraction, accu_capacity, accu_trigger, float64 accu,
 * kinematic_wave).  No reference counterpart: the reference's schedule is HPX's task order over its
 * partitions.  Results do not depend on the schedule, only the time a call takes does.
 *   cap            most cells of one stage (1..256, default 128).  It belongs to the stage structures,
 *                  which the clones of a handle share: setting another cap frees them (they are rebuilt by
 *                  the next call that needs them, after all work on the device) and is refused with
 *                  LUE_GPU_EINVAL while clones exist.  0 keeps the current cap.
 *   threads        threads per stage CTA: 32, 64, 128 or 256; 0 picks them by the largest stage.
 *   publish_every  time steps between two publications of a stage's progress in multi-step calls
 *                  (a release fence each); 0 is the default (4).
 *   ms             lue_gpu_autotune_stage_schedule: measured time of one call with this schedule. */
typedef struct lue_gpu_stage_schedule {
    int32_t cap;
    int32_t threads;
    int32_t publish_every;
    float ms;
} lue_gpu_stage_schedule;
int lue_gpu_topology_get_stage_schedule(const lue_gpu_topology* topology, lue_gpu_stage_schedule* schedule);
int lue_gpu_topology_set_stage_schedule(lue_gpu_topology* topology, const lue_gpu_stage_schedule* schedule);

/* Order in which the CTAs of a stage-engine call take the stages (no reference counterpart; results do not
 * depend on it).  LATEST (the default): by the latest start that keeps the call's critical chain on time,
 * the stages with least slack first; the fastest for one call on an otherwise idle GPU.  EARLIEST: by the
 * earliest start, about the order in which the stages' inputs become ready; its CTAs wait less, which
 * suits many calls running at the same time (a server).  Like the cap, the order belongs to the stage
 * structures: setting another one frees them (they are rebuilt by the next call that needs them, after
 * all work on the device) and is refused with LUE_GPU_EINVAL while clones exist. */
enum { LUE_GPU_STAGE_ORDER_LATEST = 0, LUE_GPU_STAGE_ORDER_EARLIEST = 1 };
int lue_gpu_topology_set_stage_order(lue_gpu_topology* topology, int order);
int lue_gpu_topology_get_stage_order(const lue_gpu_topology* topology, int* order);

/* A call to time: issues one routing call on `topology` on `stream` and returns its status. */
typedef int (*lue_gpu_stage_call)(lue_gpu_topology* topology, void* user, void* stream);

/* Autotuner of the stage schedule (no reference counterpart).  Times `call` (CUDA events on `stream`,
 * after one untimed run per candidate, which builds the stage structures of a new cap) for candidate
 * schedules: stage
 * caps 64, 128 and 256, then publication intervals 1, 2, 4 and 8 with the best cap, then 32, 64 and 128
 * threads per stage with the best of those.  Each timing is the mean of `repeats` calls (>= 1).  The
 * fastest schedule stays set on the handle and is returned in *best.  When clones share the stage
 * structures, the cap is not changed.  Synchronous: returns when the timings are done.  The outputs of
 * `call` hold its last run, which is the same for every schedule.  A failing call ends the tuning with its
 * status and the schedule the handle had before. */
int lue_gpu_autotune_stage_schedule(lue_gpu_topology* topology, lue_gpu_stage_call call, void* user, int repeats,
                                    void* stream, lue_gpu_stage_schedule* best);

/* inflow_count<uint8>(DefaultValuePolicies, fd): number of neighbours draining into each cell,
 * 255 where the flow direction is no-data.  value_policies = 0 gives DefaultPolicies (255 is an
 * unknown code, i.e. a sink; definition/inflow_count.hpp:9-15). */
int lue_gpu_inflow_count_u8(const lue_gpu_topology* topology, int value_policies, uint8_t* inflow_count,
                            void* stream);

/* accu_info(fd) (value_policies/accu_info.hpp:18-26; classes accu_info.hpp:22-63): the class of every cell
 * in the reference's partitioned flow accumulation, for the topology's partition shape: 11 ridge, 12
 * intra-partition stream, 13 partition output, 14 partition input, 15 partition input-output, 16
 * inter-partition stream, 17 sink; 255 where the flow direction is no-data.  A partition input cell whose
 * upstream cells in its own partition also wait for other partitions is classed by the last arrival in
 * the reference, which depends on the order its channels deliver; here it is classed as if material from
 * another partition arrived last (14 or 15). */
int lue_gpu_accu_info_u8(lue_gpu_topology* topology, uint8_t* cell_class, void* stream);

/* partial_accu(fd, inflow, nr_steps) (value_policies/partial_accu.hpp:17-28, definition/partial_accu.hpp:
 * 15-287): per cell, the number of the stream of the reference's partitioned walk that reached it last
 * (ridge cells: their rank among their partition's ridge cells in row-major order; partition input cells:
 * the largest arriving value plus one), NaN above nr_steps and for a no-data flow direction, for the
 * topology's partition shape.  (The reference takes an inflow scalar that it does not use.)  Where the
 * reference's result depends on the order its channels deliver (cells below a meeting of several walks
 * that start at partition input cells of one partition), the value here is one of the possible ones and
 * order_dependent (optional, uint8, may be NULL) is 1; elsewhere it is 0. */
int lue_gpu_partial_accu_f32(lue_gpu_topology* topology, int64_t nr_steps, float* out, uint8_t* order_dependent,
                             void* stream);
int lue_gpu_partial_accu_f64(lue_gpu_topology* topology, int64_t nr_steps, double* out, uint8_t* order_dependent,
                             void* stream);

/* Element types of the numpy boundary (LUE's element types). */
enum lue_gpu_element_type {
    LUE_GPU_ELEMENT_U8 = 1,
    LUE_GPU_ELEMENT_I32 = 2,
    LUE_GPU_ELEMENT_U32 = 3,
    LUE_GPU_ELEMENT_I64 = 4,
    LUE_GPU_ELEMENT_U64 = 5,
    LUE_GPU_ELEMENT_F32 = 6,
    LUE_GPU_ELEMENT_F64 = 7
};

/* from_numpy(array, partition_shape, no_data_value) (source/framework/python/source/numpy/
 * from_numpy.cpp:44-133), the no-data part: every element of the device buffer equal to *value (a host
 * value of the element type) becomes the element type's no-data value (NaN for float and double, the
 * minimum for signed and the maximum for unsigned integers; policy/detect_no_data_by_value.hpp:33-54),
 * in place, on the stream.  The buffer must be 16-byte aligned. */
int lue_gpu_mark_no_data(void* data, int64_t n, int element_type, const void* value, void* stream);

/* to_numpy(array, no_data_value) (source/framework/python/source/numpy/to_numpy.cpp), the no-data part:
 * src copied to dst (device buffers, 16-byte aligned, may be the same) with every no-data element
 * replaced by *value. */
int lue_gpu_replace_no_data(const void* src, void* dst, int64_t n, int element_type, const void* value,
                            void* stream);

/* Downstream level of each cell: 0 for cells without inflow, else 1 + the largest level upstream;
 * -1 for no-data and for cells on or below a cycle.  No reference counterpart: it exposes the
 * downstream ordering the routing kernels use. */
int lue_gpu_downstream_level_i32(const lue_gpu_topology* topology, int32_t* level, void* stream);

/* d8_flow_direction: steepest-descent D8 code per cell from an elevation raster, the reference's rule
 * (ALG/definition/d8_flow_direction.hpp:45-147): unweighted drop, candidates N, W, E, S, NW, NE, SW, SE,
 * strict '>', sink (5) without a positive drop, 255 for NaN elevation; outside the array the smallest
 * positive normal value of the element type, so edge cells above it drain off the array. */
int lue_gpu_d8_flow_direction_f32(const float* elevation, int64_t rows, int64_t cols, uint8_t* flow_direction,
                                  void* stream);
int lue_gpu_d8_flow_direction_f64(const double* elevation, int64_t rows, int64_t cols, uint8_t* flow_direction,
                                  void* stream);

/* accu: outflow = upstream outflow + inflow (inflow >= 0, else NaN). */
int lue_gpu_accu_f32(lue_gpu_topology* topology, const float* inflow, float inflow_scalar, float* outflow,
                     void* stream);
int lue_gpu_accu_f64(lue_gpu_topology* topology, const double* inflow, double inflow_scalar, double* outflow,
                     void* stream);

/* accu_threshold: total = upstream + inflow; if total > threshold: (flux, state) = (total - threshold,
 * threshold) else (0, total).  Domain inflow >= 0 && threshold >= 0. */
int lue_gpu_accu_threshold_f32(lue_gpu_topology* topology, const float* inflow, float inflow_scalar,
                               const float* threshold, float threshold_scalar, float* flux, float* state,
                               void* stream);
int lue_gpu_accu_threshold_f64(lue_gpu_topology* topology, const double* inflow, double inflow_scalar,
                               const double* threshold, double threshold_scalar, double* flux, double* state,
                               void* stream);

/* accu_fraction: total = upstream + inflow; flux = fraction * total; state = total - flux.
 * Domain inflow >= 0 && 0 <= fraction <= 1. */
int lue_gpu_accu_fraction_f32(lue_gpu_topology* topology, const float* inflow, float inflow_scalar,
                              const float* fraction, float fraction_scalar, float* flux, float* state,
                              void* stream);
int lue_gpu_accu_fraction_f64(lue_gpu_topology* topology, const double* inflow, double inflow_scalar,
                              const double* fraction, double fraction_scalar, double* flux, double* state,
                              void* stream);

/* accu_capacity (value_policies/accu_capacity.hpp, definition/accu_capacity.hpp enter_cell): total =
 * upstream + inflow; what flows on is min(total, capacity), the rest stays: (outflow, remainder).
 * Domain inflow >= 0 && capacity >= 0. */
int lue_gpu_accu_capacity_f32(lue_gpu_topology* topology, const float* inflow, float inflow_scalar,
                              const float* capacity, float capacity_scalar, float* outflow, float* remainder,
                              void* stream);
int lue_gpu_accu_capacity_f64(lue_gpu_topology* topology, const double* inflow, double inflow_scalar,
                              const double* capacity, double capacity_scalar, double* outflow, double* remainder,
                              void* stream);

/* accu_trigger (value_policies/accu_trigger.hpp, definition/accu_trigger.hpp enter_cell): total =
 * upstream + inflow; if total < trigger everything stays (0, total), else it all flows on (total, 0).
 * Domain inflow >= 0 && trigger >= 0. */
int lue_gpu_accu_trigger_f32(lue_gpu_topology* topology, const float* inflow, float inflow_scalar,
                             const float* trigger, float trigger_scalar, float* outflow, float* remainder,
                             void* stream);
int lue_gpu_accu_trigger_f64(lue_gpu_topology* topology, const double* inflow, double inflow_scalar,
                             const double* trigger, double trigger_scalar, double* outflow, double* remainder,
                             void* stream);

/* upstream (value_policies/upstream.hpp, definition/upstream.hpp:9-160): per cell the sum of the material
 * of the neighbours that drain into it; no-data where the flow direction or the cell's own material is
 * no-data, or a draining neighbour's material is.  A focal operation: it takes the flow direction
 * raster itself (row-major, rows x cols), no topology. */
int lue_gpu_upstream_f32(const uint8_t* flow_direction, int64_t rows, int64_t cols, const float* material,
                         float* out, void* stream);
int lue_gpu_upstream_f64(const uint8_t* flow_direction, int64_t rows, int64_t cols, const double* material,
                         double* out, void* stream);

/* downstream (value_policies/downstream.hpp, definition/downstream.hpp:9-158): per cell the material of
 * its downstream cell; its own material for a sink; 0 where the flow leaves the array; no-data where the
 * flow direction or the cell's own or the downstream material is no-data. */
int lue_gpu_downstream_f32(const uint8_t* flow_direction, int64_t rows, int64_t cols, const float* material,
                           float* out, void* stream);
int lue_gpu_downstream_f64(const uint8_t* flow_direction, int64_t rows, int64_t cols, const double* material,
                           double* out, void* stream);

/* downstream_distance (downstream_distance.hpp:9-44, definition/downstream_distance.hpp:9-75): the
 * length of the step to the downstream cell: cell_size for N, W, E, S; sqrt(2) * cell_size for the
 * diagonals; 0 for a sink; NaN for a no-data flow direction. */
int lue_gpu_downstream_distance_f32(const uint8_t* flow_direction, int64_t rows, int64_t cols, float cell_size,
                                    float* out, void* stream);
int lue_gpu_downstream_distance_f64(const uint8_t* flow_direction, int64_t rows, int64_t cols, double cell_size,
                                    double* out, void* stream);

/* kinematic_wave: one time step of non-linear kinematic-wave routing; per cell the Newton-Raphson
 * solve of definition/kinematic_wave.hpp:145-254 with the upstream new discharge.
 * Domain current_outflow >= 0 && inflow >= 0 && channel_length > 0, else NaN. */
int lue_gpu_kinematic_wave_f64(lue_gpu_topology* topology, const double* current_outflow,
                               double current_outflow_scalar, const double* inflow, double inflow_scalar,
                               const double* alpha, double alpha_scalar, const double* beta,
                               double beta_scalar, double time_step_duration, const double* channel_length,
                               double channel_length_scalar, double* outflow, void* stream);
/* kinematic_wave for F = float (the reference's float instantiation, definition/kinematic_wave.hpp:
 * 662-684): every raster float32, the Newton-Raphson solve of :145-254 in float with digits =
 * int(24 * 0.6) = 14, FLT_MIN guess floor and bracket [0, FLT_MAX].  Same domain and no-data rules. */
int lue_gpu_kinematic_wave_f32(lue_gpu_topology* topology, const float* current_outflow,
                               float current_outflow_scalar, const float* inflow, float inflow_scalar,
                               const float* alpha, float alpha_scalar, const float* beta, float beta_scalar,
                               float time_step_duration, const float* channel_length, float channel_length_scalar,
                               float* outflow, void* stream);
/* Same with float32 lateral inflow and alpha rasters, promoted exactly to double per cell. */
int lue_gpu_kinematic_wave_f64_f32in(lue_gpu_topology* topology, const double* current_outflow,
                                     double current_outflow_scalar, const float* inflow, double inflow_scalar,
                                     const float* alpha, double alpha_scalar, double beta,
                                     double time_step_duration, double channel_length, double* outflow,
                                     void* stream);

/* `steps` kinematic-wave time steps in one call (the discharge of each step feeds the next, lateral
 * inflow and alpha constant).  Replaces the caller's per-step loop (the reference's lue::simulate
 * pattern, source/framework/model/include/lue/framework/model/simulate.hpp).
 * Engines:
 *  - default, for a scalar beta that is a small rational p/m (0.6 = 3/5): the stage engine runs every
 *    step in one dataflow launch, with the solve in y = Q^(1/m) (float32 Newton plus one float-float
 *    step).  Results agree with `steps` calls of lue_gpu_kinematic_wave_f64_f32in within 1e-12
 *    relative, not bit for bit.  Scratch (kept by the topology): 8 bytes per stage exit (about 40 % of
 *    the cells at 128-cell stages) and step of a call; calls whose history would not fit 40 % of the
 *    free device memory are cut into parts.
 *  - LUE_GB300_KW_SOLVE=reference, another beta, or a network with flow cycles: time-skewed level waves
 *    with the float64 solve, equal bit for bit to `steps` calls of lue_gpu_kinematic_wave_f64_f32in
 *    (cycles: one single-step call per step); scratch steps x cells x 8 bytes. */
int lue_gpu_kinematic_wave_steps_f64_f32in(lue_gpu_topology* topology, const double* current_outflow,
                                           const float* inflow, double inflow_scalar, const float* alpha,
                                           double alpha_scalar, double beta, double time_step_duration,
                                           double channel_length, int steps, double* outflow, void* stream);

/* accu (float32) that allocates no device memory.  No counterpart in the reference: it is for callers
 * that must not allocate on their call path (a model step inside a host framework that owns the
 * device memory pool, or a latency-critical loop in which cudaMalloc/cudaFree would synchronise the
 * device).  It takes the flow direction itself (no topology) and keeps its scratch in one fixed,
 * file-scope device array of 7 * LUE_GPU_NOALLOC_MAX_CELLS bytes (about 29 MB) that every GPU which
 * loads the library holds until the process exits.  Rasters above LUE_GPU_NOALLOC_MAX_CELLS cells fail
 * with LUE_GPU_ERANGE.  The first call on each device resolves that array's device address
 * (cudaGetSymbolAddress, with the device current); make the first call before any stream capture.  The
 * address is cached per device and context: after a device reset (or any other teardown of the
 * context) the next call resolves it again, so that call too must come before any stream capture.
 * All calls share the array: calls that overlap on the GPU race and must be serialised by the caller.
 * The partition shape is validated like the reference's domain decomposition, for the same errors; it
 * does not change the result or the schedule.  Every call runs the walk engine (one thread per cell,
 * float-float sums along paths) plus one pass over the cells on or below flow cycles; results agree
 * with lue_gpu_accu_f32 within the float32 tolerance of the other accu entry points (at most 1e-5
 * relative), not bit for bit. */
#define LUE_GPU_NOALLOC_MAX_CELLS 4194304
int lue_gpu_accu_f32_noalloc(const uint8_t* flow_direction, int64_t rows, int64_t cols, int64_t partition_rows,
                             int64_t partition_cols, const float* inflow, float inflow_scalar, float* outflow,
                             void* stream);

#ifdef __cplusplus
}
#endif

#endif /* LUE_GB300_H */
