// no_data.cu — the no-data mapping of the numpy boundary, on the device.
//
// Reference: source/framework/python/source/numpy/from_numpy.cpp:44-133 (from_numpy(array,
// partition_shape, no_data_value): elements equal to no_data_value become no-data) and to_numpy.cpp
// (to_numpy(array, no_data_value): no-data elements come out as no_data_value).  The element type's
// no-data value follows the default value policies (ALG/policy/detect_no_data_by_nan.hpp,
// detect_no_data_by_value.hpp:33-54): NaN for float and double, the minimum for signed integers, the
// maximum for unsigned ones.
//
// One streaming pass: each thread moves 16 bytes per step (elements of 1, 4 or 8 bytes), HBM-bound.
#include <type_traits>

#include "common.cuh"

namespace lue_gb300 {

template <class T>
__device__ __forceinline__ T element_no_data()
{
    if constexpr (std::is_floating_point_v<T>) return T(__int_as_float(0x7fc00000));
    else if constexpr (std::is_signed_v<T>) return std::numeric_limits<T>::min();
    else return std::numeric_limits<T>::max();
}

template <class T>
__device__ __forceinline__ bool is_element_no_data(T x)
{
    if constexpr (std::is_floating_point_v<T>) return isnan(x);
    else return x == element_no_data<T>();
}

// mark: x == value -> no-data (in place); replace: no-data -> value (src to dst).
template <class T, bool kMark>
__global__ void k_no_data(const T* __restrict__ src, T* __restrict__ dst, int64_t n, T value)
{
    constexpr int kPer = 16 / sizeof(T);
    const int64_t nvec = n / kPer;
    const uint4* s4 = reinterpret_cast<const uint4*>(src);
    uint4* d4 = reinterpret_cast<uint4*>(dst);
    for (int64_t i = grid_stride_begin(); i < nvec; i += grid_stride()) {
        uint4 v = s4[i];
        T* e = reinterpret_cast<T*>(&v);
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            if constexpr (kMark) {
                if (e[k] == value) e[k] = element_no_data<T>();
            } else {
                if (is_element_no_data(e[k])) e[k] = value;
            }
        }
        d4[i] = v;
    }
    for (int64_t i = nvec * kPer + grid_stride_begin(); i < n; i += grid_stride()) {
        T x = src[i];
        if constexpr (kMark) {
            if (x == value) x = element_no_data<T>();
        } else {
            if (is_element_no_data(x)) x = value;
        }
        dst[i] = x;
    }
}

template <class T, bool kMark>
static int no_data_pass(const void* src, void* dst, int64_t n, const void* value, cudaStream_t stream,
                        const char* what)
{
    if ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) % 16 != 0)
        return fail(LUE_GPU_EINVAL, std::string(what) + ": device buffers must be 16-byte aligned");
    T v;
    memcpy(&v, value, sizeof(T));
    k_no_data<T, kMark><<<grid_for(n / (16 / sizeof(T)) + 1, 256), 256, 0, stream>>>(
        static_cast<const T*>(src), static_cast<T*>(dst), n, v);
    count_launches(1);
    return cuda_status(cudaGetLastError(), what);
}

template <bool kMark>
static int dispatch(const void* src, void* dst, int64_t n, int element_type, const void* value, void* stream_,
                    const char* what)
{
    if (!src || !dst || !value) return fail(LUE_GPU_EINVAL, std::string(what) + ": NULL argument");
    if (n < 0) return fail(LUE_GPU_EINVAL, std::string(what) + ": negative element count");
    if (n == 0) return LUE_GPU_OK;
    cudaStream_t s = (cudaStream_t)stream_;
    switch (element_type) {
        case LUE_GPU_ELEMENT_U8: return no_data_pass<uint8_t, kMark>(src, dst, n, value, s, what);
        case LUE_GPU_ELEMENT_I32: return no_data_pass<int32_t, kMark>(src, dst, n, value, s, what);
        case LUE_GPU_ELEMENT_U32: return no_data_pass<uint32_t, kMark>(src, dst, n, value, s, what);
        case LUE_GPU_ELEMENT_I64: return no_data_pass<int64_t, kMark>(src, dst, n, value, s, what);
        case LUE_GPU_ELEMENT_U64: return no_data_pass<uint64_t, kMark>(src, dst, n, value, s, what);
        case LUE_GPU_ELEMENT_F32: return no_data_pass<float, kMark>(src, dst, n, value, s, what);
        case LUE_GPU_ELEMENT_F64: return no_data_pass<double, kMark>(src, dst, n, value, s, what);
        default: return fail(LUE_GPU_EINVAL, std::string(what) + ": unknown element type");
    }
}

}  // namespace lue_gb300

using namespace lue_gb300;

extern "C" int lue_gpu_mark_no_data(void* data, int64_t n, int element_type, const void* value, void* stream)
{
    return dispatch<true>(data, data, n, element_type, value, stream, "mark_no_data");
}

extern "C" int lue_gpu_replace_no_data(const void* src, void* dst, int64_t n, int element_type, const void* value,
                                       void* stream)
{
    return dispatch<false>(src, dst, n, element_type, value, stream, "replace_no_data");
}
