// topology.cu — resident flow topology: inflow count, upstream masks, downstream levels, statistics.
//
// Reference counterparts (ALG/ = source/framework/algorithm/include/lue/framework/algorithm/):
//   inflow count per cell ............ ALG/detail/inflow_count.hpp:9-351 plus the partition input
//                                      cells of ALG/definition/inflow_count.hpp:97-577; on one device
//                                      the whole raster is one domain, so the count is taken over all
//                                      eight neighbours directly (the public inflow_count<uint8> result,
//                                      ALG/definition/inflow_count.hpp:665-726)
//   D8 decoding ...................... ALG/detail/flow_direction.hpp:11-112
#include <cstring>
#include <new>
#include <string>

#include "topology.cuh"
#include "walk.cuh"

namespace lue_gb300 {

thread_local std::string g_last_error;
static std::atomic<unsigned long long> g_launches{0};

void count_launches(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int status, const std::string& msg)
{
    g_last_error = msg;
    return status;
}

int cuda_status(cudaError_t err, const char* what)
{
    if (err == cudaSuccess) return LUE_GPU_OK;
    if (err == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return fail(LUE_GPU_ENOMEM, std::string(what) + ": " + cudaGetErrorString(err));
    }
    return fail(LUE_GPU_ECUDA, std::string(what) + ": " + cudaGetErrorString(err));
}

// Gather: for each cell, which neighbours drain into it.  Coalesced row reads of the 3x3 window;
// value_policies marks no-data cells with 255 (ALG/policy/mark_no_data_by_value.hpp).
__global__ void __launch_bounds__(256)
    k_count_upmask(const uint8_t* __restrict__ fd, int64_t rows, int64_t cols, int value_policies,
                   uint8_t* __restrict__ count, uint8_t* __restrict__ upmask)
{
    const int64_t n = rows * cols;
    for (int64_t i = grid_stride_begin(); i < n; i += grid_stride()) {
        int64_t r = i / cols, c = i - r * cols;
        uint8_t code = __ldg(fd + i);
        unsigned mask = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            int64_t rn = r + nb_dr(k), cn = c + nb_dc(k);
            if (rn >= 0 && rn < rows && cn >= 0 && cn < cols && __ldg(fd + rn * cols + cn) == nb_inflow_code(k))
                mask |= 1u << k;
        }
        if (upmask) upmask[i] = (uint8_t)mask;
        count[i] = (value_policies && code == kNoData) ? kNoData : (uint8_t)__popc(mask);
    }
}

struct LevelVisitor {
    const uint8_t* upmask;
    int32_t* level;
    int64_t cols;
    __device__ void enter(int64_t c)
    {
        unsigned m = __ldg(upmask + c);
        int32_t lv = -1;
        while (m) {
            int k = __ffs(m) - 1;
            m &= m - 1;
            int32_t u = load_cg(level + c + nb_dr(k) * cols + nb_dc(k));
            lv = u > lv ? u : lv;
        }
        level[c] = lv + 1;
    }
    __device__ void no_data(int64_t) {}
};

__global__ void k_fill_i32(int32_t* p, int64_t n, int32_t v)
{
    for (int64_t i = grid_stride_begin(); i < n; i += grid_stride()) p[i] = v;
}

// stats: [valid, ridge, outlet, sink, cycle, max_level]
__global__ void __launch_bounds__(256)
    k_stats(const uint8_t* fd, const uint8_t* count, const int32_t* level, int64_t rows, int64_t cols,
            unsigned long long* stats)
{
    const int64_t n = rows * cols;
    unsigned long long v = 0, ridge = 0, outlet = 0, sink = 0, cycle = 0;
    int maxl = 0;
    for (int64_t i = grid_stride_begin(); i < n; i += grid_stride()) {
        uint8_t code = fd[i];
        if (code == kNoData) continue;
        ++v;
        if (count[i] == 0) ++ridge;
        int dr, dc;
        if (!d8_offset(code, dr, dc)) {
            ++sink;
        } else {
            int64_t r = i / cols + dr, c = i % cols + dc;
            if (r < 0 || r >= rows || c < 0 || c >= cols) ++outlet;
        }
        if (level[i] < 0) ++cycle;
        else if (level[i] > maxl) maxl = level[i];
    }
    for (int off = 16; off > 0; off >>= 1) {
        v += __shfl_down_sync(0xffffffffu, v, off);
        ridge += __shfl_down_sync(0xffffffffu, ridge, off);
        outlet += __shfl_down_sync(0xffffffffu, outlet, off);
        sink += __shfl_down_sync(0xffffffffu, sink, off);
        cycle += __shfl_down_sync(0xffffffffu, cycle, off);
        int o = __shfl_down_sync(0xffffffffu, maxl, off);
        maxl = o > maxl ? o : maxl;
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(stats + 0, v);
        atomicAdd(stats + 1, ridge);
        atomicAdd(stats + 2, outlet);
        atomicAdd(stats + 3, sink);
        atomicAdd(stats + 4, cycle);
        atomicMax(stats + 5, (unsigned long long)maxl);
    }
}

int allocate_scratch(lue_gpu_topology* t)
{
    const int64_t n = t->core->n;
    int rc = cuda_status(cudaMalloc(&t->work_count, words_for(n) * 4), "scratch counters");
    if (rc) return rc;
    rc = cuda_status(cudaMalloc(&t->lo, n * sizeof(float)), "scratch residuals");
    if (rc) {
        cudaFree(t->work_count);
        t->work_count = nullptr;
        return rc;
    }
    t->scratch_bytes = words_for(n) * 4 + n * (int64_t)sizeof(float);
    // the stage engine's timeout flag, read by the host on the next call (pinned, written by a copy)
    rc = cuda_status(cudaHostAlloc(&t->stage_flow_error, sizeof(int), cudaHostAllocDefault), "scratch flag");
    if (rc) return rc;
    *t->stage_flow_error = 0;
    if (t->core->tiles) {
        rc = tile_scratch_alloc(t->core->tiles, &t->tile_scratch);
        if (rc) return rc;
        t->scratch_bytes += t->tile_scratch.bytes;
    }
    return LUE_GPU_OK;
}

static void free_core(TopologyCore* core)
{
    if (!core) return;
    cudaFree(core->fd);
    cudaFree(core->count);
    cudaFree(core->upmask);
    cudaFree(core->level);
    cudaFree(core->order);
    tile_core_free(core->tiles);
    stage_core_free(core->stages);
    path_core_free(core->paths);
    delete core;
}

static void free_handle(lue_gpu_topology* t)
{
    if (!t) return;
    cudaFree(t->work_count);
    cudaFree(t->lo);
    cudaFree(t->history);
    cudaFree(t->planes);
    stage_buffers_free(t);
    path_buffers_free(t);
    cudaFreeHost(t->stage_flow_error);
    tile_scratch_free(&t->tile_scratch);
    if (t->core && --t->core->refs == 0) free_core(t->core);
    delete t;
}

}  // namespace lue_gb300

using namespace lue_gb300;

extern "C" int lue_gpu_abi_version(void) { return LUE_GPU_ABI_VERSION; }

extern "C" unsigned long long lue_gpu_kernel_launches(void) { return g_launches.load(); }

extern "C" const char* lue_gpu_last_error(void) { return g_last_error.c_str(); }

extern "C" int lue_gpu_topology_create(const uint8_t* flow_direction, int64_t rows, int64_t cols,
                                       int64_t partition_rows, int64_t partition_cols, void* stream_,
                                       lue_gpu_topology** out)
{
    if (!out) return fail(LUE_GPU_EINVAL, "topology_create: NULL result pointer");
    *out = nullptr;
    if (!flow_direction) return fail(LUE_GPU_EINVAL, "topology_create: NULL flow direction");
    if (rows <= 0 || cols <= 0) return fail(LUE_GPU_EINVAL, "topology_create: array shape must not be empty");
    if (partition_rows <= 0 || partition_cols <= 0)
        return fail(LUE_GPU_EINVAL, "topology_create: partition shape must not be empty");
    if (partition_rows > rows || partition_cols > cols)
        return fail(LUE_GPU_EINVAL, "topology_create: partition shape must not exceed the array shape");
    if (rows > (int64_t(1) << 31) || cols > (int64_t(1) << 31) || rows * cols > (int64_t(1) << 40))
        return fail(LUE_GPU_ERANGE, "topology_create: array too large");
    cudaStream_t stream = (cudaStream_t)stream_;
    auto* core = new (std::nothrow) TopologyCore();
    auto* t = new (std::nothrow) lue_gpu_topology();
    if (!core || !t) {
        delete core;
        delete t;
        return fail(LUE_GPU_ENOMEM, "topology_create: host allocation");
    }
    t->core = core;
    core->rows = rows;
    core->cols = cols;
    core->prow = partition_rows;
    core->pcol = partition_cols;
    core->n = rows * cols;
    const int64_t n = core->n, padded = words_for(n) * 4;
    int rc = 0;
    unsigned long long* dstats = nullptr;
    unsigned long long hstats[6] = {0, 0, 0, 0, 0, 0};
    if ((rc = cuda_status(cudaMalloc(&core->fd, padded), "topology fd"))) goto error;
    if ((rc = cuda_status(cudaMalloc(&core->count, padded), "topology count"))) goto error;
    if ((rc = cuda_status(cudaMalloc(&core->upmask, padded), "topology upmask"))) goto error;
    if ((rc = cuda_status(cudaMalloc(&core->level, n * sizeof(int32_t)), "topology level"))) goto error;
    core->bytes = 3 * padded + n * (int64_t)sizeof(int32_t);
    if ((rc = cuda_status(cudaMalloc(&t->work_count, padded), "scratch counters"))) goto error;
    if ((rc = cuda_status(cudaMalloc(&dstats, sizeof hstats), "topology stats"))) goto error;
    if ((rc = cuda_status(cudaMemsetAsync(core->fd, kNoData, padded, stream), "memset"))) goto error;
    if ((rc = cuda_status(cudaMemcpyAsync(core->fd, flow_direction, n, cudaMemcpyDeviceToDevice, stream),
                          "copy flow direction")))
        goto error;
    if ((rc = cuda_status(cudaMemsetAsync(core->count, 0, padded, stream), "memset"))) goto error;
    k_count_upmask<<<grid_for(n, 256), 256, 0, stream>>>(core->fd, rows, cols, 1, core->count, core->upmask);
    k_fill_i32<<<grid_for(n, 256), 256, 0, stream>>>(core->level, n, -1);
    if ((rc = cuda_status(cudaMemcpyAsync(t->work_count, core->count, padded, cudaMemcpyDeviceToDevice, stream),
                          "reset counters")))
        goto error;
    {
        WalkGrid g{core->fd, core->count, t->work_count, rows, cols, n};
        LevelVisitor v{core->upmask, core->level, cols};
        k_walk<<<grid_all(n, 256), 256, 0, stream>>>(g, v);
    }
    if ((rc = cuda_status(cudaMemsetAsync(dstats, 0, sizeof hstats, stream), "memset"))) goto error;
    k_stats<<<grid_for(n, 256), 256, 0, stream>>>(core->fd, core->count, core->level, rows, cols, dstats);
    if ((rc = cuda_status(cudaGetLastError(), "topology kernels"))) goto error;
    if ((rc = cuda_status(cudaMemcpyAsync(hstats, dstats, sizeof hstats, cudaMemcpyDeviceToHost, stream),
                          "stats")))
        goto error;
    if ((rc = cuda_status(cudaStreamSynchronize(stream), "topology_create"))) goto error;
    cudaFree(dstats);
    dstats = nullptr;
    core->stats.rows = rows;
    core->stats.cols = cols;
    core->stats.partition_rows = partition_rows;
    core->stats.partition_cols = partition_cols;
    core->stats.valid_cells = (int64_t)hstats[0];
    core->stats.ridge_cells = (int64_t)hstats[1];
    core->stats.outlet_cells = (int64_t)hstats[2];
    core->stats.sink_cells = (int64_t)hstats[3];
    core->stats.cycle_cells = (int64_t)hstats[4];
    core->stats.max_level = (int64_t)hstats[5];
    // the tile engine needs an acyclic network and 32-bit cell indices
    if (core->stats.cycle_cells == 0 && n < (int64_t(1) << 32)) {
        rc = tile_core_build(core, stream);
        if (rc == LUE_GPU_ECUDA || rc == LUE_GPU_ENOMEM) goto error;
        rc = LUE_GPU_OK;
    }
    if (core->tiles) {
        core->stats.tile_exits = core->tiles->nexit;
        core->stats.exit_forest_depth = core->tiles->max_depth;
        core->bytes += core->tiles->bytes;
    }
    cudaFree(t->work_count);
    t->work_count = nullptr;
    if ((rc = allocate_scratch(t))) goto error;
    *out = t;
    return LUE_GPU_OK;
error:
    cudaFree(dstats);
    free_handle(t);
    return rc;
}

extern "C" int lue_gpu_topology_clone(const lue_gpu_topology* topology, lue_gpu_topology** clone)
{
    if (!topology || !clone) return fail(LUE_GPU_EINVAL, "topology_clone: NULL argument");
    *clone = nullptr;
    auto* t = new (std::nothrow) lue_gpu_topology();
    if (!t) return fail(LUE_GPU_ENOMEM, "topology_clone: host allocation");
    t->core = topology->core;
    t->core->refs++;
    int rc = allocate_scratch(t);
    if (rc) {
        free_handle(t);
        return rc;
    }
    *clone = t;
    return LUE_GPU_OK;
}

extern "C" int lue_gpu_topology_prepare(lue_gpu_topology* topology, void* stream)
{
    if (!topology) return fail(LUE_GPU_EINVAL, "topology_prepare: NULL topology");
    if (int rc = path_prepare(topology, (cudaStream_t)stream)) return rc;
    return stage_prepare(topology, (cudaStream_t)stream);
}

extern "C" int lue_gpu_topology_destroy(lue_gpu_topology* topology)
{
    if (!topology) return fail(LUE_GPU_EINVAL, "topology_destroy: NULL topology");
    free_handle(topology);
    return LUE_GPU_OK;
}

extern "C" int lue_gpu_topology_get_stats(const lue_gpu_topology* topology, lue_gpu_topology_stats* stats)
{
    if (!topology || !stats) return fail(LUE_GPU_EINVAL, "topology_stats: NULL argument");
    *stats = topology->core->stats;
    stats->device_bytes = topology->core->bytes + topology->scratch_bytes;
    return LUE_GPU_OK;
}

extern "C" int lue_gpu_inflow_count_u8(const lue_gpu_topology* topology, int value_policies, uint8_t* inflow_count,
                                       void* stream_)
{
    if (!topology || !inflow_count) return fail(LUE_GPU_EINVAL, "inflow_count: NULL argument");
    cudaStream_t stream = (cudaStream_t)stream_;
    const TopologyCore* core = topology->core;
    if (value_policies) {
        return cuda_status(
            cudaMemcpyAsync(inflow_count, core->count, core->n, cudaMemcpyDeviceToDevice, stream), "inflow_count");
    }
    k_count_upmask<<<grid_for(core->n, 256), 256, 0, stream>>>(core->fd, core->rows, core->cols, 0, inflow_count,
                                                                nullptr);
    return cuda_status(cudaGetLastError(), "inflow_count");
}

extern "C" int lue_gpu_downstream_level_i32(const lue_gpu_topology* topology, int32_t* level, void* stream_)
{
    if (!topology || !level) return fail(LUE_GPU_EINVAL, "downstream_level: NULL argument");
    const TopologyCore* core = topology->core;
    return cuda_status(cudaMemcpyAsync(level, core->level, core->n * sizeof(int32_t), cudaMemcpyDeviceToDevice,
                                       (cudaStream_t)stream_),
                       "downstream_level");
}
