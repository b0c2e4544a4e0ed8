// route_walk.cu — accu, accu_threshold, accu_fraction and kinematic_wave on the walk engine.
//
// Cell rules (ALG/ = source/framework/algorithm/include/lue/framework/algorithm/):
//   accu ............ ALG/definition/accu.hpp:102-153      total = upstream + inflow
//   accu_threshold .. ALG/definition/accu_threshold.hpp:124-169
//   accu_fraction ... ALG/definition/accu_fraction.hpp:124-162
//   kinematic_wave .. ALG/definition/kinematic_wave.hpp:416-456 and iterate_to_new_discharge :145-254
//   value-policy domains: ALG/value_policies/{accu,accu_threshold,accu_fraction,kinematic_wave}.hpp:15-21
//
// No-data: a NaN upstream outflow, a NaN input or an input outside the domain makes the cell NaN
// (both outputs for threshold/fraction), and NaN then flows on downstream (ALG/definition/accu.hpp:
// 102-153).  The upstream sum is pulled in a fixed neighbour order instead of the reference's arrival
// order; float32 operations carry a float-float (hi + lo) running value along every flow path, so the
// only rounding left is the final hi of each cell.
//
// Cells on or below a flow cycle are never entered by the reference (their inflow count never reaches
// zero) and keep the sum of what upstream cells pushed into them; k_cycle_cells restores exactly that.
#include "route_walk_visitors.cuh"
#include "topology.cuh"

namespace lue_gb300 {

template <class Visitor, class T>
static int run(lue_gpu_topology* t, Visitor v, T* out, T* rem, bool use_lo, cudaStream_t stream, const char* what)
{
    const TopologyCore* core = t->core;
    const int64_t n = core->n;
    int rc = cuda_status(
        cudaMemcpyAsync(t->work_count, core->count, words_for(n) * 4, cudaMemcpyDeviceToDevice, stream), what);
    if (rc) return rc;
    WalkGrid g{core->fd, core->count, t->work_count, core->rows, core->cols, n};
    k_walk<<<grid_all(n, 256), 256, 0, stream>>>(g, v);
    count_launches(core->stats.cycle_cells > 0 ? 2 : 1);
    if (core->stats.cycle_cells > 0) {
        k_cycle_cells<T><<<grid_for(n, 256), 256, 0, stream>>>(core->fd, core->upmask, t->work_count, n, core->cols,
                                                               out, rem, use_lo ? t->lo : nullptr);
    }
    return cuda_status(cudaGetLastError(), what);
}

static int check_topology(const lue_gpu_topology* t, const char* what)
{
    if (!t || !t->core) return fail(LUE_GPU_EINVAL, std::string(what) + ": NULL topology");
    return LUE_GPU_OK;
}

template <Rule R>
static int route_f32(lue_gpu_topology* t, const float* a, float as, const float* b, float bs, float* out, float* rem,
                     void* stream, const char* what)
{
    if (int rc = check_topology(t, what)) return rc;
    if (!out || (R != Rule::accu && !rem)) return fail(LUE_GPU_EINVAL, std::string(what) + ": NULL output");
    RouteF32<R> v{t->core->upmask, a, as, b, bs, out, rem, t->lo, t->core->cols};
    return run(t, v, out, rem, true, (cudaStream_t)stream, what);
}

template <Rule R>
static int route_f64(lue_gpu_topology* t, const double* a, double as, const double* b, double bs, double* out,
                     double* rem, void* stream, const char* what)
{
    if (int rc = check_topology(t, what)) return rc;
    if (!out || (R != Rule::accu && !rem)) return fail(LUE_GPU_EINVAL, std::string(what) + ": NULL output");
    RouteF64<R> v{t->core->upmask, a, as, b, bs, out, rem, t->core->cols};
    return run(t, v, out, rem, false, (cudaStream_t)stream, what);
}

__global__ void k_copy_words_if(const uint32_t* src, uint32_t* dst, int64_t nwords, const unsigned long long* flag)
{
    if (flag[1] == 0) return;
    for (int64_t i = grid_stride_begin(); i < nwords; i += grid_stride()) dst[i] = src[i];
}

// Scalar beta as a small rational p/m (beta = 0.6 is 3/5) for the fast kinematic-wave solve;
// LUE_GB300_KW_SOLVE=reference keeps the reference-faithful float64 solve.
static BetaRational rational_beta(const double* beta_raster, double beta)
{
    const char* e = getenv("LUE_GB300_KW_SOLVE");
    if (beta_raster || (e && e[0] == 'r') || !(beta > 0.0)) return BetaRational{0, 0, (float)beta};
    for (int m = 1; m <= 16; ++m) {
        double p = nearbyint(beta * m);
        if (p >= 1.0 && p <= 64.0 && fabs(beta - p / m) <= 1e-15 * beta) return BetaRational{(int)p, m, (float)beta};
    }
    return BetaRational{0, 0, (float)beta};
}

static bool walk_engine_forced()
{
    const char* e = getenv("LUE_GB300_ENGINE");
    return e && e[0] == 'w';
}

}  // namespace lue_gb300

using namespace lue_gb300;

// accu (float32): the tile engine when the topology has one (acyclic rasters), else the walk engine.
// LUE_GB300_ENGINE=walk forces the walk engine (for comparisons).
extern "C" int lue_gpu_accu_f32(lue_gpu_topology* t, const float* inflow, float inflow_scalar, float* outflow,
                                void* stream_)
{
    if (int rc = check_topology(t, "accu_f32")) return rc;
    if (!outflow) return fail(LUE_GPU_EINVAL, "accu_f32: NULL output");
    const TopologyCore* core = t->core;
    if (!core->tiles || walk_engine_forced())
        return route_f32<Rule::accu>(t, inflow, inflow_scalar, nullptr, 0.0f, outflow, nullptr, stream_, "accu_f32");
    cudaStream_t stream = (cudaStream_t)stream_;
    if (int rc = tile_accu_f32(core, &t->tile_scratch, inflow, inflow_scalar, outflow, stream)) return rc;
    // +inf material or a total beyond the fixed-point range: the walk engine redoes the call
    const int64_t n = core->n;
    const unsigned long long* flag = t->tile_scratch.total;
    k_copy_words_if<<<grid_for(words_for(n), 256), 256, 0, stream>>>(reinterpret_cast<const uint32_t*>(core->count),
                                                                     t->work_count, words_for(n), flag);
    WalkGrid g{core->fd, core->count, t->work_count, core->rows, core->cols, n};
    RouteF32<Rule::accu> v{core->upmask, inflow, inflow_scalar, nullptr, 0.0f, outflow, nullptr, t->lo, core->cols};
    k_walk_if<<<grid_for(n, 256), 256, 0, stream>>>(g, v, flag);
    count_launches(2);
    return cuda_status(cudaGetLastError(), "accu_f32");
}

// Float64 accu and the rules that are not plain sums run on the stage engine (stage_route.cuh) when the
// topology has no flow cycles, else on the walk engine.  LUE_GB300_ENGINE=walk forces the walk engine.
#define STAGE_OR_WALK(call)                          \
    do {                                             \
        bool done = false;                           \
        if (int rc = (call)) return rc;              \
        if (done) return LUE_GPU_OK;                 \
    } while (0)

extern "C" int lue_gpu_accu_f64(lue_gpu_topology* t, const double* inflow, double inflow_scalar, double* outflow,
                                void* stream)
{
    if (int rc = check_topology(t, "accu_f64")) return rc;
    if (!outflow) return fail(LUE_GPU_EINVAL, "accu_f64: NULL output");
    STAGE_OR_WALK(stage_route_f64(t, (int)Rule::accu, inflow, inflow_scalar, nullptr, 0.0, outflow, nullptr,
                                  (cudaStream_t)stream, &done));
    return route_f64<Rule::accu>(t, inflow, inflow_scalar, nullptr, 0.0, outflow, nullptr, stream, "accu_f64");
}

extern "C" int lue_gpu_accu_threshold_f32(lue_gpu_topology* t, const float* inflow, float inflow_scalar,
                                          const float* threshold, float threshold_scalar, float* flux, float* state,
                                          void* stream)
{
    if (int rc = check_topology(t, "accu_threshold_f32")) return rc;
    if (!flux || !state) return fail(LUE_GPU_EINVAL, "accu_threshold_f32: NULL output");
    STAGE_OR_WALK(path_route_f32(t, (int)Rule::threshold, inflow, inflow_scalar, threshold, threshold_scalar, flux,
                                 state, (cudaStream_t)stream, &done));
    STAGE_OR_WALK(stage_route_f32(t, (int)Rule::threshold, inflow, inflow_scalar, threshold, threshold_scalar, flux,
                                  state, (cudaStream_t)stream, &done));
    return route_f32<Rule::threshold>(t, inflow, inflow_scalar, threshold, threshold_scalar, flux, state, stream,
                                      "accu_threshold_f32");
}

extern "C" int lue_gpu_accu_threshold_f64(lue_gpu_topology* t, const double* inflow, double inflow_scalar,
                                          const double* threshold, double threshold_scalar, double* flux,
                                          double* state, void* stream)
{
    if (int rc = check_topology(t, "accu_threshold_f64")) return rc;
    if (!flux || !state) return fail(LUE_GPU_EINVAL, "accu_threshold_f64: NULL output");
    STAGE_OR_WALK(stage_route_f64(t, (int)Rule::threshold, inflow, inflow_scalar, threshold, threshold_scalar, flux,
                                  state, (cudaStream_t)stream, &done));
    return route_f64<Rule::threshold>(t, inflow, inflow_scalar, threshold, threshold_scalar, flux, state, stream,
                                      "accu_threshold_f64");
}

extern "C" int lue_gpu_accu_fraction_f32(lue_gpu_topology* t, const float* inflow, float inflow_scalar,
                                         const float* fraction, float fraction_scalar, float* flux, float* state,
                                         void* stream)
{
    if (int rc = check_topology(t, "accu_fraction_f32")) return rc;
    if (!flux || !state) return fail(LUE_GPU_EINVAL, "accu_fraction_f32: NULL output");
    STAGE_OR_WALK(path_route_f32(t, (int)Rule::fraction, inflow, inflow_scalar, fraction, fraction_scalar, flux,
                                 state, (cudaStream_t)stream, &done));
    STAGE_OR_WALK(stage_route_f32(t, (int)Rule::fraction, inflow, inflow_scalar, fraction, fraction_scalar, flux,
                                  state, (cudaStream_t)stream, &done));
    return route_f32<Rule::fraction>(t, inflow, inflow_scalar, fraction, fraction_scalar, flux, state, stream,
                                     "accu_fraction_f32");
}

extern "C" int lue_gpu_accu_fraction_f64(lue_gpu_topology* t, const double* inflow, double inflow_scalar,
                                         const double* fraction, double fraction_scalar, double* flux, double* state,
                                         void* stream)
{
    if (int rc = check_topology(t, "accu_fraction_f64")) return rc;
    if (!flux || !state) return fail(LUE_GPU_EINVAL, "accu_fraction_f64: NULL output");
    STAGE_OR_WALK(stage_route_f64(t, (int)Rule::fraction, inflow, inflow_scalar, fraction, fraction_scalar, flux,
                                  state, (cudaStream_t)stream, &done));
    return route_f64<Rule::fraction>(t, inflow, inflow_scalar, fraction, fraction_scalar, flux, state, stream,
                                     "accu_fraction_f64");
}

// The path engine (path_route.cuh) takes float32 accu_threshold, accu_fraction and accu_capacity on acyclic
// rasters.
static int path_first(lue_gpu_topology* t, int rule, const float* a, float as, const float* b, float bs, float* out,
                      float* rem, cudaStream_t stream, bool* done)
{
    return path_route_f32(t, rule, a, as, b, bs, out, rem, stream, done);
}
static int path_first(lue_gpu_topology*, int, const double*, double, const double*, double, double*, double*,
                      cudaStream_t, bool* done)
{
    *done = false;
    return LUE_GPU_OK;
}

// accu_capacity / accu_trigger: the same routers with the cell rules of ALG/definition/accu_capacity.hpp
// and ALG/definition/accu_trigger.hpp (enter_cell).
#define TWO_OUTPUT_OP(NAME, RULE, T, ROUTE, STAGE)                                                           \
    extern "C" int lue_gpu_##NAME(lue_gpu_topology* t, const T* inflow, T inflow_scalar, const T* other,     \
                                  T other_scalar, T* outflow, T* remainder, void* stream)                     \
    {                                                                                                         \
        if (int rc = check_topology(t, #NAME)) return rc;                                                     \
        if (!outflow || !remainder) return fail(LUE_GPU_EINVAL, #NAME ": NULL output");                       \
        STAGE_OR_WALK(path_first(t, (int)RULE, inflow, inflow_scalar, other, other_scalar, outflow, remainder, \
                                 (cudaStream_t)stream, &done));                                               \
        STAGE_OR_WALK(STAGE(t, (int)RULE, inflow, inflow_scalar, other, other_scalar, outflow, remainder,      \
                            (cudaStream_t)stream, &done));                                                    \
        return ROUTE<RULE>(t, inflow, inflow_scalar, other, other_scalar, outflow, remainder, stream, #NAME); \
    }

TWO_OUTPUT_OP(accu_capacity_f32, Rule::capacity, float, route_f32, stage_route_f32)
TWO_OUTPUT_OP(accu_capacity_f64, Rule::capacity, double, route_f64, stage_route_f64)
TWO_OUTPUT_OP(accu_trigger_f32, Rule::trigger, float, route_f32, stage_route_f32)
TWO_OUTPUT_OP(accu_trigger_f64, Rule::trigger, double, route_f64, stage_route_f64)

extern "C" int lue_gpu_kinematic_wave_f64(lue_gpu_topology* t, const double* current_outflow,
                                          double current_outflow_scalar, const double* inflow, double inflow_scalar,
                                          const double* alpha, double alpha_scalar, const double* beta,
                                          double beta_scalar, double time_step_duration,
                                          const double* channel_length, double channel_length_scalar,
                                          double* outflow, void* stream)
{
    if (int rc = check_topology(t, "kinematic_wave_f64")) return rc;
    if (!outflow) return fail(LUE_GPU_EINVAL, "kinematic_wave_f64: NULL output");
    STAGE_OR_WALK(stage_kinematic_wave_f64(t, current_outflow, current_outflow_scalar, inflow, inflow_scalar, alpha,
                                           alpha_scalar, beta, beta_scalar, time_step_duration, channel_length,
                                           channel_length_scalar, outflow, rational_beta(beta, beta_scalar),
                                           (cudaStream_t)stream, &done));
    RouteKW<double> v{t->core->upmask, current_outflow, current_outflow_scalar, inflow, inflow_scalar, alpha,
                      alpha_scalar, beta, beta_scalar, time_step_duration, channel_length, channel_length_scalar,
                      outflow, t->core->cols, rational_beta(beta, beta_scalar)};
    return run(t, v, outflow, (double*)nullptr, false, (cudaStream_t)stream, "kinematic_wave_f64");
}

extern "C" int lue_gpu_kinematic_wave_f32(lue_gpu_topology* t, const float* current_outflow,
                                          float current_outflow_scalar, const float* inflow, float inflow_scalar,
                                          const float* alpha, float alpha_scalar, const float* beta, float beta_scalar,
                                          float time_step_duration, const float* channel_length,
                                          float channel_length_scalar, float* outflow, void* stream)
{
    if (int rc = check_topology(t, "kinematic_wave_f32")) return rc;
    if (!outflow) return fail(LUE_GPU_EINVAL, "kinematic_wave_f32: NULL output");
    STAGE_OR_WALK(stage_kinematic_wave_f32(t, current_outflow, current_outflow_scalar, inflow, inflow_scalar, alpha,
                                           alpha_scalar, beta, beta_scalar, time_step_duration, channel_length,
                                           channel_length_scalar, outflow, (cudaStream_t)stream, &done));
    RouteKW32 v{t->core->upmask, current_outflow, current_outflow_scalar, inflow, inflow_scalar, alpha, alpha_scalar,
                beta, beta_scalar, time_step_duration, channel_length, channel_length_scalar, outflow,
                t->core->cols};
    return run(t, v, outflow, (float*)nullptr, false, (cudaStream_t)stream, "kinematic_wave_f32");
}

extern "C" int lue_gpu_kinematic_wave_f64_f32in(lue_gpu_topology* t, const double* current_outflow,
                                                double current_outflow_scalar, const float* inflow,
                                                double inflow_scalar, const float* alpha, double alpha_scalar,
                                                double beta, double time_step_duration, double channel_length,
                                                double* outflow, void* stream)
{
    if (int rc = check_topology(t, "kinematic_wave_f64_f32in")) return rc;
    if (!outflow) return fail(LUE_GPU_EINVAL, "kinematic_wave_f64_f32in: NULL output");
    STAGE_OR_WALK(stage_kinematic_wave_f32in(t, current_outflow, current_outflow_scalar, inflow, inflow_scalar, alpha,
                                             alpha_scalar, beta, time_step_duration, channel_length, outflow,
                                             rational_beta(nullptr, beta), (cudaStream_t)stream, &done));
    RouteKW<float> v{t->core->upmask, current_outflow, current_outflow_scalar, inflow, inflow_scalar, alpha,
                     alpha_scalar, nullptr, beta, time_step_duration, nullptr, channel_length, outflow,
                     t->core->cols, rational_beta(nullptr, beta)};
    return run(t, v, outflow, (double*)nullptr, false, (cudaStream_t)stream, "kinematic_wave_f64_f32in");
}
