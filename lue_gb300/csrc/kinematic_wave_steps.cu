// kinematic_wave_steps.cu — many kinematic-wave time steps in one call.
//
// Which engine runs: for a scalar beta that is a small rational p/m, the stage engine
// (stage_route.cu: one dataflow launch over all stages and steps, float-float solve in y = Q^(1/m)),
// whose results agree with single-step calls within 1e-12 relative and whose scratch is the stage
// history (8 bytes per stage exit and step).  The time-skewed level waves below run for
// LUE_GB300_KW_SOLVE=reference and other betas; they equal single-step calls bit for bit.
//
// The reference's caller runs one kinematic_wave call per time step (lue::simulate, source/framework/
// model/include/lue/framework/model/simulate.hpp), each a full downstream sweep: T steps cost T times
// the longest flow path.  Step t of cell c needs only step t of its upstream cells and step t - 1 of c
// itself, so cell c can run step t in wave level(c) + t: every wave finishes one step for the cells of T
// consecutive downstream levels, and T steps take (max level + T) waves.
//
// Each step's discharge is kept in a plane Q_t (t = 0 is the input, t = T the output); a wave reads
// Q_t of the upstream cells and Q_{t-1} of the cell itself, in the same fixed neighbour order as the
// single-step kernels, so the level-wave result equals T single calls bit for bit.  The planes for
// 1 <= t < T live in the topology's scratch (grown on demand: steps * cells * 8 bytes).
//
// Cells are ordered by level (counting sort, row-major within a level); a wave covers one contiguous
// range of that order.  Networks with cycles run single steps instead (cells on or below a cycle are
// never finished by the reference, see route_walk.cu).
#include <vector>

#include "route_walk_visitors.cuh"
#include "topology.cuh"

namespace lue_gb300 {

__global__ void k_level_histogram(const int32_t* level, int64_t n, int32_t* hist)
{
    for (int64_t c = grid_stride_begin(); c < n; c += grid_stride())
        if (level[c] >= 0) atomicAdd(hist + level[c], 1);
}

// Stable placement: one thread per level writes that level's cells in row-major order would be slow for
// level 0; instead blocks of consecutive cells reserve positions with per-block counts.  Order within a
// level is not needed for correctness, only for locality; atomics give blocks of neighbouring cells.
__global__ void k_level_scatter(const int32_t* level, int64_t n, int32_t* cursor, int32_t* order)
{
    for (int64_t c = grid_stride_begin(); c < n; c += grid_stride()) {
        int32_t l = level[c];
        if (l >= 0) order[atomicAdd(cursor + l, 1)] = (int32_t)c;
    }
}

struct WaveArgs {
    const int32_t* order;
    const int32_t* level;
    const uint8_t* upmask;
    const double* const* planes;  // [steps + 1] plane pointers (plane 0 = input, plane steps = output)
    double* const* wplanes;       // same pointers, writable view
    const float* lateral;
    double lateral_s;
    const float* alpha;
    double alpha_s;
    double beta, dt, dx;
    BetaRational br;
    int64_t cols;
    int steps;
};

__global__ void __launch_bounds__(256) k_kw_wave(WaveArgs a, int64_t begin, int64_t end, int wave)
{
    int64_t k = begin + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= end) return;
    const int64_t c = a.order[k];
    const int t = wave - a.level[c];
    if (t < 1 || t > a.steps) return;
    const double* qt = a.planes[t];
    unsigned m = __ldg(a.upmask + c);
    double up = 0.0;
    bool nan = false;
    while (m) {
        int q = __ffs(m) - 1;
        m &= m - 1;
        double h = qt[c + nb_dr(q) * a.cols + nb_dc(q)];
        if (isnan(h)) nan = true;
        else up += h;
    }
    double qc = a.planes[t - 1][c];
    double lat = a.lateral ? (double)__ldg(a.lateral + c) : a.lateral_s;
    double al = a.alpha ? (double)__ldg(a.alpha + c) : a.alpha_s;
    double out;
    if (nan || isnan(qc) || isnan(lat) || isnan(al) || isnan(a.beta) || isnan(a.dt) || isnan(a.dx) ||
        !(qc >= 0.0 && lat >= 0.0 && a.dx > 0.0)) {
        out = __longlong_as_double(0x7ff8000000000000ll);
    } else {
        out = a.br.m ? iterate_to_new_discharge_fast(up, qc, lat, al, a.beta, a.br, a.dt, a.dx)
                     : iterate_to_new_discharge(up, qc, lat, al, a.beta, a.dt, a.dx);
    }
    a.wplanes[t][c] = out;
}

// No-data flow direction: NaN in every plane written (the reference marks the cell no-data each step).
__global__ void k_kw_no_data(const uint8_t* fd, int64_t n, double* out)
{
    for (int64_t c = grid_stride_begin(); c < n; c += grid_stride())
        if (fd[c] == kNoData) out[c] = __longlong_as_double(0x7ff8000000000000ll);
}

int ensure_level_order(TopologyCore* core, cudaStream_t stream)
{
    if (core->order) return LUE_GPU_OK;
    const int64_t n = core->n, nl = core->stats.max_level + 1;
    int32_t *order = nullptr, *hist = nullptr;
    std::vector<int32_t> h(nl), off(nl + 1);
    int rc;
    if ((rc = cuda_status(cudaMalloc(&order, std::max<int64_t>(core->stats.valid_cells, 1) * sizeof(int32_t)),
                          "level order")))
        return rc;
    if ((rc = cuda_status(cudaMalloc(&hist, nl * sizeof(int32_t)), "level order"))) {
        cudaFree(order);
        return rc;
    }
    cudaMemsetAsync(hist, 0, nl * sizeof(int32_t), stream);
    k_level_histogram<<<grid_for(n, 256), 256, 0, stream>>>(core->level, n, hist);
    cudaMemcpyAsync(h.data(), hist, nl * sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    if ((rc = cuda_status(cudaStreamSynchronize(stream), "level order"))) {
        cudaFree(order);
        cudaFree(hist);
        return rc;
    }
    off[0] = 0;
    for (int64_t l = 0; l < nl; ++l) off[l + 1] = off[l] + h[l];
    cudaMemcpyAsync(hist, off.data(), nl * sizeof(int32_t), cudaMemcpyHostToDevice, stream);
    k_level_scatter<<<grid_for(n, 256), 256, 0, stream>>>(core->level, n, hist, order);
    count_launches(2);
    if ((rc = cuda_status(cudaStreamSynchronize(stream), "level order"))) {
        cudaFree(order);
        cudaFree(hist);
        return rc;
    }
    cudaFree(hist);
    core->order = order;
    core->level_offsets.assign(off.begin(), off.end());
    core->bytes += core->stats.valid_cells * 4;
    return LUE_GPU_OK;
}

}  // namespace lue_gb300

using namespace lue_gb300;

extern "C" int lue_gpu_kinematic_wave_steps_f64_f32in(lue_gpu_topology* t, const double* current_outflow,
                                                      const float* inflow, double inflow_scalar, const float* alpha,
                                                      double alpha_scalar, double beta, double time_step_duration,
                                                      double channel_length, int steps, double* outflow,
                                                      void* stream_)
{
    if (!t || !t->core || !current_outflow || !outflow) return fail(LUE_GPU_EINVAL, "kinematic_wave_steps: NULL argument");
    // a negative count is the internal form of one chunk: run exactly |steps| steps, no further chunking
    const bool single_chunk = steps < 0;
    if (single_chunk) steps = -steps;
    if (steps < 1) return fail(LUE_GPU_EINVAL, "kinematic_wave_steps: steps must be at least 1");
    cudaStream_t stream = (cudaStream_t)stream_;
    TopologyCore* core = t->core;
    const int64_t n = core->n;
    if (!single_chunk) {
        // the stage engine with the float-float solve, for a scalar beta that is a small rational p/m;
        // LUE_GB300_KW_SOLVE=reference keeps the float64 solve of the level waves below
        const char* e = getenv("LUE_GB300_KW_SOLVE");
        BetaRational br{0, 0, (float)beta};
        if (!(e && e[0] == 'r') && beta > 0.0) {
            for (int m = 1; m <= 16; ++m) {
                const double p = nearbyint(beta * m);
                if (p >= 1.0 && p <= 64.0 && fabs(beta - p / m) <= 1e-15 * beta) {
                    br = BetaRational{(int)p, m, (float)beta};
                    break;
                }
            }
        }
        bool done = false;
        if (int rc = stage_kinematic_wave_steps(t, current_outflow, inflow, inflow_scalar, alpha, alpha_scalar, beta,
                                                time_step_duration, channel_length, steps, outflow, br, stream, &done))
            return rc;
        if (done) return LUE_GPU_OK;
    }
    if (core->stats.cycle_cells > 0) {
        // the wave schedule needs levels for every cell: one single step per call, ping-pong buffers
        double* tmp = nullptr;
        if (steps > 1) {
            if (int rc = cuda_status(cudaMalloc(&tmp, n * sizeof(double)), "kinematic_wave_steps")) return rc;
        }
        const double* src = current_outflow;
        for (int s = 0; s < steps; ++s) {
            double* dst = ((steps - 1 - s) % 2 == 0) ? outflow : tmp;
            int rc = lue_gpu_kinematic_wave_f64_f32in(t, src, 0.0, inflow, inflow_scalar, alpha, alpha_scalar, beta,
                                                      time_step_duration, channel_length, dst, stream_);
            if (rc) {
                cudaFree(tmp);
                return rc;
            }
            src = dst;
        }
        if (tmp) {
            cudaStreamSynchronize(stream);
            cudaFree(tmp);
        }
        return LUE_GPU_OK;
    }
    if (int rc = ensure_level_order(core, stream)) return rc;
    // Steps run in chunks whose history planes fit in a budget: what this handle already holds plus
    // LUE_GB300_KW_HISTORY_FRACTION (default 0.25) of the free device memory, and at most 64 planes;
    // each chunk takes max level + chunk waves.
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const size_t plane = (size_t)n * sizeof(double);
    double frac = 0.25;
    if (const char* e = getenv("LUE_GB300_KW_HISTORY_FRACTION")) frac = atof(e);
    int64_t fit = std::min<int64_t>(64, (int64_t)((free_b * frac + (double)t->history_bytes) / (double)plane));
    int chunk = (int)std::max<int64_t>(1, std::min<int64_t>(steps, fit + 1));
    if (chunk < steps && !single_chunk) {
        const double* src = current_outflow;
        double* tmp = nullptr;
        if (int rc = cuda_status(cudaMalloc(&tmp, 2 * plane), "kinematic_wave_steps")) return rc;
        int done = 0, which = 0;
        while (done < steps) {
            int k = std::min(chunk, steps - done);
            double* dst = (done + k == steps) ? outflow : tmp + (size_t)which * n;
            int rc = lue_gpu_kinematic_wave_steps_f64_f32in(t, src, inflow, inflow_scalar, alpha, alpha_scalar, beta,
                                                            time_step_duration, channel_length, -k, dst, stream_);
            if (rc) {
                cudaFree(tmp);
                return rc;
            }
            src = dst;
            which ^= 1;
            done += k;
        }
        cudaStreamSynchronize(stream);
        cudaFree(tmp);
        return LUE_GPU_OK;
    }
    // history planes 1 .. steps-1
    const size_t need = (size_t)(steps - 1) * (size_t)n * sizeof(double);
    if (need > t->history_bytes) {
        cudaStreamSynchronize(stream);
        cudaFree(t->history);
        t->history = nullptr;
        t->history_bytes = 0;
        if (int rc = cuda_status(cudaMalloc(&t->history, need), "kinematic_wave_steps history")) return rc;
        t->history_bytes = need;
    }
    if ((size_t)(steps + 1) > t->plane_capacity) {
        cudaStreamSynchronize(stream);
        cudaFree(t->planes);
        t->planes = nullptr;
        t->plane_capacity = 0;
        if (int rc = cuda_status(cudaMalloc(&t->planes, (steps + 1) * sizeof(double*)), "kinematic_wave_steps planes"))
            return rc;
        t->plane_capacity = steps + 1;
    }
    std::vector<double*> hp(steps + 1);
    hp[0] = const_cast<double*>(current_outflow);
    for (int s = 1; s < steps; ++s) hp[s] = t->history + (size_t)(s - 1) * n;
    hp[steps] = outflow;
    if (int rc = cuda_status(cudaMemcpyAsync(t->planes, hp.data(), (steps + 1) * sizeof(double*), cudaMemcpyHostToDevice,
                                             stream),
                             "kinematic_wave_steps planes"))
        return rc;
    // no-data cells: NaN in every written plane
    for (int s = 1; s <= steps; ++s) k_kw_no_data<<<grid_for(n, 256), 256, 0, stream>>>(core->fd, n, hp[s]);
    WaveArgs a{core->order, core->level, core->upmask, t->planes, t->planes, inflow, inflow_scalar, alpha,
               alpha_scalar, beta, time_step_duration, channel_length, BetaRational{0, 0, (float)beta}, core->cols,
               steps};
    {
        const char* e = getenv("LUE_GB300_KW_SOLVE");
        if (!(e && e[0] == 'r') && beta > 0.0) {
            for (int m = 1; m <= 16; ++m) {
                double p = nearbyint(beta * m);
                if (p >= 1.0 && p <= 64.0 && fabs(beta - p / m) <= 1e-15 * beta) {
                    a.br = BetaRational{(int)p, m, (float)beta};
                    break;
                }
            }
        }
    }
    const std::vector<int32_t>& off = core->level_offsets;
    const int64_t nl = (int64_t)off.size() - 1;
    int launches = steps;
    for (int64_t w = 1; w <= nl - 1 + steps; ++w) {
        int64_t lo_level = std::max<int64_t>(0, w - steps), hi_level = std::min<int64_t>(nl, w);  // [lo, hi)
        if (lo_level >= hi_level) continue;
        int64_t begin = off[lo_level], end = off[hi_level];
        if (end <= begin) continue;
        k_kw_wave<<<(unsigned)((end - begin + 255) / 256), 256, 0, stream>>>(a, begin, end, (int)w);
        ++launches;
    }
    count_launches(launches);
    return cuda_status(cudaGetLastError(), "kinematic_wave_steps");
}
