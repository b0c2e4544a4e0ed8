// common.cuh — shared device helpers: D8 decoding, neighbour tables, compensated arithmetic, status.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "lue_gb300.h"

namespace lue_gb300 {

constexpr uint8_t kNoData = 255;

// Neighbour k of a cell, k = 0..7: NW, N, NE, W, E, SW, S, SE (row offset, column offset).
__host__ __device__ constexpr int nb_dr(int k) { return k < 3 ? -1 : (k < 5 ? 0 : 1); }
__host__ __device__ constexpr int nb_dc(int k)
{
    return (k == 0 || k == 3 || k == 5) ? -1 : ((k == 1 || k == 6) ? 0 : 1);
}

// Code neighbour k must carry to drain into the centre cell: the keypad code pointing back.
// NW neighbour drains SE (3), N -> S (2), NE -> SW (1), W -> E (6), E -> W (4), SW -> NE (9),
// S -> N (8), SE -> NW (7).
__host__ __device__ constexpr uint8_t nb_inflow_code(int k)
{
    return k == 0 ? 3 : k == 1 ? 2 : k == 2 ? 1 : k == 3 ? 6 : k == 4 ? 4 : k == 5 ? 9 : k == 6 ? 8 : 7;
}

// Keypad D8 code to offsets (flow_direction.hpp:7-35); anything else is a sink (0, 0).
__host__ __device__ inline bool d8_offset(uint8_t code, int& dr, int& dc)
{
    switch (code) {
        case 7: dr = -1; dc = -1; return true;
        case 8: dr = -1; dc = 0; return true;
        case 9: dr = -1; dc = 1; return true;
        case 4: dr = 0; dc = -1; return true;
        case 6: dr = 0; dc = 1; return true;
        case 1: dr = 1; dc = -1; return true;
        case 2: dr = 1; dc = 0; return true;
        case 3: dr = 1; dc = 1; return true;
        default: dr = 0; dc = 0; return false;
    }
}

// Downstream cell index of cell (r, c) with code `code`; false for sinks and for flow off the array.
__device__ inline bool downstream(uint8_t code, int64_t r, int64_t c, int64_t rows, int64_t cols, int64_t& d)
{
    int dr, dc;
    if (!d8_offset(code, dr, dc)) return false;
    int64_t rd = r + dr, cd = c + dc;
    if (rd < 0 || rd >= rows || cd < 0 || cd >= cols) return false;
    d = rd * cols + cd;
    return true;
}

// Error-free transformations (Knuth two-sum, FMA two-product) for float-float accumulation.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// Float-float accumulator: value = hi + lo with |lo| <= ulp(hi) / 2 after normalise().  A sum that is
// not finite keeps IEEE semantics (inf stays inf, NaN stays NaN) with lo = 0; the error terms of
// two_sum would otherwise turn inf into NaN.
struct FF {
    float hi, lo;
    __device__ __forceinline__ void add(float x)
    {
        float s, e;
        two_sum(hi, x, s, e);
        if (!isfinite(s)) {
            hi = s;
            lo = 0.0f;
            return;
        }
        hi = s;
        lo = __fadd_rn(lo, e);
    }
    __device__ __forceinline__ void add(float xh, float xl)
    {
        add(xh);
        if (isfinite(hi)) lo = __fadd_rn(lo, xl);
    }
    __device__ __forceinline__ void normalise()
    {
        float s = __fadd_rn(hi, lo);
        if (!isfinite(s)) {
            hi = s;
            lo = 0.0f;
            return;
        }
        lo = __fsub_rn(lo, __fsub_rn(s, hi));
        hi = s;
    }
};

// Loads that bypass L1: values written by other threads during the same kernel.
template <class T>
__device__ __forceinline__ T load_cg(const T* p)
{
    return __ldcg(p);
}

__device__ __forceinline__ int64_t grid_stride_begin() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int64_t grid_stride() { return (int64_t)gridDim.x * blockDim.x; }

// Host side -----------------------------------------------------------------------------------------

void set_error(const std::string& msg);
// Kernel launches made by this library in this process (reported by lue_gpu_kernel_launches).
void count_launches(int n);
int fail(int status, const std::string& msg);
int cuda_status(cudaError_t err, const char* what);

// One thread per element, no grid-stride reuse (walk kernels: a thread that walks a long path must not
// also own later cells, or the walks chain up behind each other).
inline unsigned grid_all(int64_t n, int threads)
{
    int64_t b = (n + threads - 1) / threads;
    return (unsigned)(b < 1 ? 1 : b);
}

inline int grid_for(int64_t n, int threads, int max_blocks = 152 * 16)
{
    int64_t b = (n + threads - 1) / threads;
    if (b > max_blocks) b = max_blocks;
    if (b < 1) b = 1;
    return (int)b;
}

}  // namespace lue_gb300
