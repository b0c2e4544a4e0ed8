// noalloc.cu — accu (float32) for callers that must not allocate device memory.
//
// Some callers cannot call cudaMalloc on their call path: a model step that runs inside a host
// framework owning the device memory pool (which forbids allocations it does not see), or a
// latency-critical loop in which cudaMalloc / cudaFree would synchronise the device.  For them,
// lue_gpu_accu_f32_noalloc takes the flow direction directly (no topology handle, which would have
// to be allocated) and keeps all of its scratch memory in one file-scope device array of fixed size,
// g_noalloc_scratch, that every GPU which loads this library holds until the process exits.
//
// Scratch layout for n <= LUE_GPU_NOALLOC_MAX_CELLS cells (7 bytes per cell, each part 256-byte aligned):
//   [count: n bytes][upmask: n bytes][counters: n bytes rounded up to 4][residuals: 4n bytes]
// Every call rewrites each part it reads before reading it, so nothing depends on an earlier call.
// All calls share the one array: calls that overlap on the GPU (other streams, other host threads)
// race on it and must be serialised by the caller.
//
// In host code `g_noalloc_scratch` names a host-side stand-in, not a device address: its device
// address is resolved with cudaGetSymbolAddress (with the device current) by the first call on a
// device and cached together with the identity of the device's current context (cuCtxGetId).  A device
// reset or any other teardown of that context loads the module again, possibly at another address: the
// next call sees a new context id and resolves the address again, so that call, like the first, must
// not be made during stream capture.
#include <cuda.h>

#include <mutex>
#include <string>

#include "route_walk_visitors.cuh"
#include "topology.cuh"

namespace lue_gb300 {

constexpr int64_t kNoallocMaxCells = LUE_GPU_NOALLOC_MAX_CELLS;
constexpr int64_t kNoallocBytes = kNoallocMaxCells * 7 + 1024;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

constexpr int kMaxDevices = 64;
struct ScratchAddress {
    unsigned char* ptr = nullptr;
    unsigned long long context_id = 0;  // cuCtxGetId of the context the address was resolved in
};
static ScratchAddress g_scratch_address[kMaxDevices];
static std::mutex g_scratch_mutex;

// The id of the calling thread's current context (0 when there is none or the driver cannot tell),
// through driver entry points fetched from the runtime, so that the library does not link libcuda.
static unsigned long long current_context_id()
{
    typedef CUresult (*GetCurrent)(CUcontext*);
    typedef CUresult (*GetId)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetId>(f);
        cudaGetLastError();  // a missing entry point is not an error of the call
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

static int noalloc_scratch(unsigned char** out)
{
    int dev = 0;
    if (int rc = cuda_status(cudaGetDevice(&dev), "accu_f32_noalloc: cudaGetDevice")) return rc;
    if (dev < 0 || dev >= kMaxDevices) return fail(LUE_GPU_ERANGE, "accu_f32_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    ScratchAddress& a = g_scratch_address[dev];
    const unsigned long long id = current_context_id();
    if (!a.ptr || id == 0 || id != a.context_id) {
        void* p = nullptr;
        if (int rc = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_scratch), "accu_f32_noalloc: cudaGetSymbolAddress"))
            return rc;
        a.ptr = static_cast<unsigned char*>(p);
        a.context_id = current_context_id();  // the symbol lookup made the device's primary context current
    }
    *out = a.ptr;
    return LUE_GPU_OK;
}

__global__ void k_noalloc_counts(const uint8_t* __restrict__ fd, int64_t rows, int64_t cols, uint8_t* count,
                                 uint8_t* upmask, uint8_t* work)
{
    const int64_t n = rows * cols;
    for (int64_t i = grid_stride_begin(); i < n; i += grid_stride()) {
        int64_t r = i / cols, c = i - r * cols;
        unsigned mask = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            int64_t rn = r + nb_dr(k), cn = c + nb_dc(k);
            if (rn >= 0 && rn < rows && cn >= 0 && cn < cols && __ldg(fd + rn * cols + cn) == nb_inflow_code(k))
                mask |= 1u << k;
        }
        uint8_t cnt = __ldg(fd + i) == kNoData ? kNoData : (uint8_t)__popc(mask);
        upmask[i] = (uint8_t)mask;
        count[i] = cnt;
        work[i] = cnt;
    }
}

}  // namespace lue_gb300

using namespace lue_gb300;

extern "C" int lue_gpu_accu_f32_noalloc(const uint8_t* flow_direction, int64_t rows, int64_t cols,
                                        int64_t partition_rows, int64_t partition_cols, const float* inflow,
                                        float inflow_scalar, float* outflow, void* stream_)
{
    if (!flow_direction || !outflow) return fail(LUE_GPU_EINVAL, "accu_f32_noalloc: NULL argument");
    if (rows <= 0 || cols <= 0) return fail(LUE_GPU_EINVAL, "accu_f32_noalloc: array shape must not be empty");
    if (partition_rows <= 0 || partition_cols <= 0 || partition_rows > rows || partition_cols > cols)
        return fail(LUE_GPU_EINVAL, "accu_f32_noalloc: partition shape must be non-empty and within the array");
    if (rows > kNoallocMaxCells || cols > kNoallocMaxCells || rows * cols > kNoallocMaxCells)
        return fail(LUE_GPU_ERANGE, "accu_f32_noalloc: " + std::to_string(rows) + " x " + std::to_string(cols) +
                                        " cells exceed the fixed scratch of " + std::to_string(kNoallocMaxCells) +
                                        " cells (LUE_GPU_NOALLOC_MAX_CELLS); use lue_gpu_accu_f32 with a topology");
    unsigned char* scratch = nullptr;
    if (int rc = noalloc_scratch(&scratch)) return rc;
    cudaStream_t stream = (cudaStream_t)stream_;
    const int64_t n = rows * cols;
    auto align = [](int64_t b) { return (b + 255) / 256 * 256; };
    uint8_t* count = scratch;
    uint8_t* upmask = count + align(n);
    uint8_t* work = upmask + align(n);
    float* lo = reinterpret_cast<float*>(work + align(words_for(n) * 4));
    k_noalloc_counts<<<grid_for(n, 256), 256, 0, stream>>>(flow_direction, rows, cols, count, upmask, work);
    WalkGrid g{flow_direction, count, reinterpret_cast<uint32_t*>(work), rows, cols, n};
    RouteF32<Rule::accu> v{upmask, inflow, inflow_scalar, nullptr, 0.0f, outflow, nullptr, lo, cols};
    k_walk<<<grid_all(n, 256), 256, 0, stream>>>(g, v);
    // cells on or below a flow cycle are never entered: give them what entered upstream cells pushed
    k_cycle_cells<float><<<grid_for(n, 256), 256, 0, stream>>>(flow_direction, upmask,
                                                               reinterpret_cast<const uint32_t*>(work), n, cols,
                                                               outflow, nullptr, lo);
    count_launches(3);
    return cuda_status(cudaGetLastError(), "accu_f32_noalloc");
}
