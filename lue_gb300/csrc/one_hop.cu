// one_hop.cu — upstream, downstream and downstream_distance: one-hop and local operations on a D8
// raster (focal operations of radius 1 in the reference; no routing, no topology).
//
//   upstream ............ ALG/definition/upstream.hpp:9-160     sum of the material of the neighbours that
//                                                                drain into the cell (NW N NE W E SW S SE)
//   downstream .......... ALG/definition/downstream.hpp:9-158   material of the downstream cell
//   downstream_distance . ALG/definition/downstream_distance.hpp:9-75
//                                                                length of the step to the downstream cell
// (ALG/ = source/framework/algorithm/include/lue/framework/algorithm/)
//
// Value policies (ALG/flow_accumulation.hpp DefaultValuePolicies, ALG/policy/flow_direction_halo.hpp):
// no-data is 255 for flow directions and NaN for material; outside the array the flow directions point
// away from the array and the material is 0.
//
// Each CTA stages a 32 x 8 tile of flow directions with a one-cell halo in shared memory; material is
// read through the read-only cache (each value is read by at most its 8 neighbours).
#include "common.cuh"

namespace lue_gb300 {

constexpr int kHopW = 32, kHopH = 8;

__device__ __forceinline__ void stage_fd(uint8_t (&s)[kHopH + 2][kHopW + 2], const uint8_t* __restrict__ fd,
                                         int64_t rows, int64_t cols, int64_t r0, int64_t c0)
{
    for (int i = threadIdx.y * kHopW + threadIdx.x; i < (kHopH + 2) * (kHopW + 2); i += kHopW * kHopH) {
        const int hr = i / (kHopW + 2), hc = i % (kHopW + 2);
        const int64_t r = r0 + hr - 1, c = c0 + hc - 1;
        s[hr][hc] = (r >= 0 && r < rows && c >= 0 && c < cols) ? __ldg(fd + r * cols + c) : kNoData;
    }
    __syncthreads();
}

template <class T>
__global__ void __launch_bounds__(kHopW * kHopH)
    k_upstream(const uint8_t* __restrict__ fd, int64_t rows, int64_t cols, const T* __restrict__ m, T* __restrict__ out)
{
    __shared__ uint8_t s[kHopH + 2][kHopW + 2];
    const int64_t r0 = (int64_t)blockIdx.y * kHopH, c0 = (int64_t)blockIdx.x * kHopW;
    stage_fd(s, fd, rows, cols, r0, c0);
    const int64_t r = r0 + threadIdx.y, c = c0 + threadIdx.x;
    if (r >= rows || c >= cols) return;
    const int64_t i = r * cols + c;
    const T own = __ldg(m + i);
    T sum = T(0);
    bool nd = s[threadIdx.y + 1][threadIdx.x + 1] == kNoData || isnan(own);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        if (nd) break;
        if (s[threadIdx.y + 1 + nb_dr(q)][threadIdx.x + 1 + nb_dc(q)] != nb_inflow_code(q)) continue;
        const T v = __ldg(m + i + nb_dr(q) * cols + nb_dc(q));  // a draining neighbour is in the array
        if (isnan(v)) nd = true;
        else sum += v;
    }
    out[i] = nd ? T(NAN) : sum;
}

template <class T>
__global__ void __launch_bounds__(kHopW * kHopH)
    k_downstream(const uint8_t* __restrict__ fd, int64_t rows, int64_t cols, const T* __restrict__ m,
                 T* __restrict__ out)
{
    const int64_t r = (int64_t)blockIdx.y * kHopH + threadIdx.y, c = (int64_t)blockIdx.x * kHopW + threadIdx.x;
    if (r >= rows || c >= cols) return;
    const int64_t i = r * cols + c;
    const uint8_t code = __ldg(fd + i);
    const T own = __ldg(m + i);
    T v;
    int dr, dc;
    if (code == kNoData || isnan(own)) {
        v = T(NAN);
    } else if (!d8_offset(code, dr, dc)) {
        v = own;  // a sink, or a code that is not a direction
    } else {
        const int64_t r2 = r + dr, c2 = c + dc;
        v = (r2 < 0 || r2 >= rows || c2 < 0 || c2 >= cols) ? T(0) : __ldg(m + r2 * cols + c2);
    }
    out[i] = v;
}

template <class T>
__global__ void k_downstream_distance(const uint8_t* __restrict__ fd, int64_t n, T cell, T diagonal,
                                      T* __restrict__ out)
{
    for (int64_t i = grid_stride_begin(); i < n; i += grid_stride()) {
        const uint8_t code = __ldg(fd + i);
        T d = T(0);
        if (code == kNoData) d = T(NAN);
        else if (code == 7 || code == 9 || code == 1 || code == 3) d = diagonal;
        else if (code == 8 || code == 4 || code == 6 || code == 2) d = cell;
        out[i] = d;
    }
}

template <class T>
static int one_hop(bool up, const uint8_t* fd, int64_t rows, int64_t cols, const T* m, T* out, void* stream,
                   const char* what)
{
    if (!fd || !m || !out) return fail(LUE_GPU_EINVAL, std::string(what) + ": NULL argument");
    if (rows <= 0 || cols <= 0) return fail(LUE_GPU_EINVAL, std::string(what) + ": non-positive extent");
    const dim3 grid((unsigned)((cols + kHopW - 1) / kHopW), (unsigned)((rows + kHopH - 1) / kHopH));
    if (grid.y > 65535) return fail(LUE_GPU_ERANGE, std::string(what) + ": more than 524280 rows");
    if (up)
        k_upstream<T><<<grid, dim3(kHopW, kHopH), 0, (cudaStream_t)stream>>>(fd, rows, cols, m, out);
    else
        k_downstream<T><<<grid, dim3(kHopW, kHopH), 0, (cudaStream_t)stream>>>(fd, rows, cols, m, out);
    count_launches(1);
    return cuda_status(cudaGetLastError(), what);
}

template <class T>
static int distance(const uint8_t* fd, int64_t rows, int64_t cols, T cell_size, T* out, void* stream)
{
    if (!fd || !out) return fail(LUE_GPU_EINVAL, "downstream_distance: NULL argument");
    if (rows <= 0 || cols <= 0) return fail(LUE_GPU_EINVAL, "downstream_distance: non-positive extent");
    const int64_t n = rows * cols;
    const T diagonal = (T)(sqrt(2.0) * (double)cell_size);
    k_downstream_distance<T><<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(fd, n, cell_size, diagonal, out);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "downstream_distance");
}

}  // namespace lue_gb300

using namespace lue_gb300;

extern "C" int lue_gpu_upstream_f32(const uint8_t* fd, int64_t rows, int64_t cols, const float* material, float* out,
                                    void* stream)
{
    return one_hop<float>(true, fd, rows, cols, material, out, stream, "upstream_f32");
}
extern "C" int lue_gpu_upstream_f64(const uint8_t* fd, int64_t rows, int64_t cols, const double* material,
                                    double* out, void* stream)
{
    return one_hop<double>(true, fd, rows, cols, material, out, stream, "upstream_f64");
}
extern "C" int lue_gpu_downstream_f32(const uint8_t* fd, int64_t rows, int64_t cols, const float* material,
                                      float* out, void* stream)
{
    return one_hop<float>(false, fd, rows, cols, material, out, stream, "downstream_f32");
}
extern "C" int lue_gpu_downstream_f64(const uint8_t* fd, int64_t rows, int64_t cols, const double* material,
                                      double* out, void* stream)
{
    return one_hop<double>(false, fd, rows, cols, material, out, stream, "downstream_f64");
}
extern "C" int lue_gpu_downstream_distance_f32(const uint8_t* fd, int64_t rows, int64_t cols, float cell_size,
                                               float* out, void* stream)
{
    return distance<float>(fd, rows, cols, cell_size, out, stream);
}
extern "C" int lue_gpu_downstream_distance_f64(const uint8_t* fd, int64_t rows, int64_t cols, double cell_size,
                                               double* out, void* stream)
{
    return distance<double>(fd, rows, cols, cell_size, out, stream);
}
