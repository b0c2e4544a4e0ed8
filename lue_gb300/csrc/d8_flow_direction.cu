// d8_flow_direction.cu — D8 flow direction from an elevation raster (the step before the routing path).
//
// Restates the reference's rule (ALG/definition/d8_flow_direction.hpp:45-147 and
// ALG/value_policies/d8_flow_direction.hpp:20-45, ALG/ = source/framework/algorithm/include/lue/framework/
// algorithm/): for each cell, the steepest unweighted drop among the neighbours in the order N, W, E, S,
// NW, NE, SW, SE, with a strict '>' (so the first of equal drops wins); no drop > 0 gives a sink (5).
// A NaN elevation gives the no-data direction 255; a NaN neighbour is skipped.  Outside the array the
// halo holds std::numeric_limits<E>::min() (the smallest positive normal value), so cells above it on
// the edge drain off the array.
//
// One thread per cell; the 3 x 3 window comes from a shared-memory tile with a one-cell halo (32 x 8
// cells per block), so each elevation is read from HBM about once.
#include <cfloat>

#include "common.cuh"

namespace lue_gb300 {

constexpr int kD8W = 32, kD8H = 8;

template <class T>
__device__ __forceinline__ T halo_min();
template <>
__device__ __forceinline__ float halo_min<float>() { return FLT_MIN; }
template <>
__device__ __forceinline__ double halo_min<double>() { return DBL_MIN; }

template <class T>
__global__ void __launch_bounds__(kD8W * kD8H)
    k_d8(const T* __restrict__ z, int64_t rows, int64_t cols, uint8_t* __restrict__ fd)
{
    __shared__ T tile[kD8H + 2][kD8W + 2];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int64_t c0 = (int64_t)blockIdx.x * kD8W, r0 = (int64_t)blockIdx.y * kD8H;
    for (int i = ty * kD8W + tx; i < (kD8H + 2) * (kD8W + 2); i += kD8W * kD8H) {
        int hr = i / (kD8W + 2), hc = i % (kD8W + 2);
        int64_t r = r0 + hr - 1, c = c0 + hc - 1;
        tile[hr][hc] = (r >= 0 && r < rows && c >= 0 && c < cols) ? __ldg(z + r * cols + c) : halo_min<T>();
    }
    __syncthreads();
    const int64_t r = r0 + ty, c = c0 + tx;
    if (r >= rows || c >= cols) return;
    const T zc = tile[ty + 1][tx + 1];
    uint8_t dir;
    if (isnan(zc)) {
        dir = kNoData;
    } else {
        // candidates N, W, E, S, NW, NE, SW, SE (d8_flow_direction.hpp:57-145)
        const int dr[8] = {-1, 0, 0, 1, -1, -1, 1, 1};
        const int dc[8] = {0, -1, 1, 0, -1, 1, -1, 1};
        const uint8_t code[8] = {8, 4, 6, 2, 7, 9, 1, 3};
        dir = 5;
        T drop = T(0);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            T zn = tile[ty + 1 + dr[k]][tx + 1 + dc[k]];
            if (isnan(zn)) continue;
            T other = zc - zn;
            if (other > drop) {
                drop = other;
                dir = code[k];
            }
        }
    }
    fd[r * cols + c] = dir;
}

template <class T>
static int d8(const T* z, int64_t rows, int64_t cols, uint8_t* fd, void* stream, const char* what)
{
    if (!z || !fd) return fail(LUE_GPU_EINVAL, std::string(what) + ": NULL argument");
    if (rows <= 0 || cols <= 0) return fail(LUE_GPU_EINVAL, std::string(what) + ": array shape must not be empty");
    dim3 block(kD8W, kD8H), grid((unsigned)((cols + kD8W - 1) / kD8W), (unsigned)((rows + kD8H - 1) / kD8H));
    if (grid.y > 65535u) return fail(LUE_GPU_ERANGE, std::string(what) + ": too many rows");
    k_d8<T><<<grid, block, 0, (cudaStream_t)stream>>>(z, rows, cols, fd);
    count_launches(1);
    return cuda_status(cudaGetLastError(), what);
}

}  // namespace lue_gb300

extern "C" int lue_gpu_d8_flow_direction_f32(const float* elevation, int64_t rows, int64_t cols, uint8_t* flow_direction,
                                             void* stream)
{
    return lue_gb300::d8(elevation, rows, cols, flow_direction, stream, "d8_flow_direction_f32");
}

extern "C" int lue_gpu_d8_flow_direction_f64(const double* elevation, int64_t rows, int64_t cols,
                                             uint8_t* flow_direction, void* stream)
{
    return lue_gb300::d8(elevation, rows, cols, flow_direction, stream, "d8_flow_direction_f64");
}
