// lue_gb300.hpp — C++ mirror of LUE's routing operations over the C ABI of include/lue_gb300.h.
//
// Same operation names, parameter order and raster/scalar overloads as the reference's
// lue::value_policies:: functions (source/framework/algorithm/include/lue/framework/algorithm/
// value_policies/{accu,accu_threshold,accu_fraction,kinematic_wave}.hpp) and lue::inflow_count
// (.../algorithm/inflow_count.hpp:29-42).  A PartitionedArray here is a device-resident, row-major
// raster with the reference's (shape, partition_shape); like the reference's it is move-only.  A shape
// or partitioning mismatch throws std::runtime_error, as ALG/detail/verify_compatible.hpp:23-40 does;
// invalid values become NaN in the result, never an exception.
//
// Header-only; link with liblue_gb300.so and the CUDA runtime.
#pragma once

#include <cuda_runtime.h>

#include <array>
#include <cstdint>
#include <exception>
#include <memory>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>

#include "lue_gb300.h"

namespace lue_gb300 {

using Shape = std::array<std::int64_t, 2>;

inline void check(int status, const char* what)
{
    if (status != LUE_GPU_OK)
        throw std::runtime_error(std::string(what) + ": " + lue_gpu_last_error());
}

inline void check_cuda(cudaError_t err, const char* what)
{
    if (err != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(err));
}

// Resident flow topology of one flow-direction raster (inflow counts, downstream ordering, scratch).
class Topology {
   public:
    Topology(const std::uint8_t* fd, Shape shape, Shape partition_shape, cudaStream_t stream)
    {
        check(lue_gpu_topology_create(fd, shape[0], shape[1], partition_shape[0], partition_shape[1], stream, &_h),
              "topology");
    }
    Topology(const Topology&) = delete;
    Topology& operator=(const Topology&) = delete;
    ~Topology() { lue_gpu_topology_destroy(_h); }
    lue_gpu_topology* handle() const { return _h; }
    // Builds now what the first stage-engine call would build (lue_gpu_topology_prepare).
    void prepare(cudaStream_t stream) { check(lue_gpu_topology_prepare(_h, stream), "topology prepare"); }

    // The stage engine's schedule (lue_gpu_topology_{get,set}_stage_schedule); results do not depend on it.
    lue_gpu_stage_schedule stage_schedule() const
    {
        lue_gpu_stage_schedule s{};
        check(lue_gpu_topology_get_stage_schedule(_h, &s), "stage_schedule");
        return s;
    }
    void set_stage_schedule(const lue_gpu_stage_schedule& s)
    {
        check(lue_gpu_topology_set_stage_schedule(_h, &s), "set_stage_schedule");
    }
    // The order in which a stage-engine call takes its stages (lue_gpu_topology_{get,set}_stage_order):
    // LUE_GPU_STAGE_ORDER_LATEST (default) or LUE_GPU_STAGE_ORDER_EARLIEST (for many calls at once).
    int stage_order() const
    {
        int o = 0;
        check(lue_gpu_topology_get_stage_order(_h, &o), "stage_order");
        return o;
    }
    void set_stage_order(int order) { check(lue_gpu_topology_set_stage_order(_h, order), "set_stage_order"); }

    // Autotunes the stage schedule for `call`, a callable that issues one routing call over this topology on
    // `stream`; keeps the fastest schedule and returns it (lue_gpu_autotune_stage_schedule).  An exception
    // thrown by `call` ends the tuning and is rethrown.
    template <typename Call>
    lue_gpu_stage_schedule autotune_stage_schedule(Call&& call, cudaStream_t stream, int repeats = 1)
    {
        struct Context {
            std::remove_reference_t<Call>* call;
            std::exception_ptr error;
        } ctx{&call, nullptr};
        lue_gpu_stage_call trampoline = [](lue_gpu_topology*, void* user, void*) -> int {
            auto* c = static_cast<Context*>(user);
            try {
                (*c->call)();
                return LUE_GPU_OK;
            } catch (...) {
                c->error = std::current_exception();
                return LUE_GPU_EINVAL;
            }
        };
        lue_gpu_stage_schedule best{};
        const int rc = lue_gpu_autotune_stage_schedule(_h, trampoline, &ctx, repeats, stream, &best);
        if (ctx.error) std::rethrow_exception(ctx.error);
        check(rc, "autotune_stage_schedule");
        return best;
    }

   private:
    lue_gpu_topology* _h = nullptr;
};

template <typename Element>
class PartitionedArray {
   public:
    PartitionedArray() = default;

    PartitionedArray(Shape shape, Shape partition_shape) : _shape(shape), _partition_shape(partition_shape)
    {
        if (shape[0] <= 0 || shape[1] <= 0) throw std::runtime_error("Array shape must not be empty");
        if (partition_shape[0] <= 0 || partition_shape[1] <= 0)
            throw std::runtime_error("Partition shape must not be empty");
        if (partition_shape[0] > shape[0] || partition_shape[1] > shape[1])
            throw std::runtime_error("Partition size must be smaller than or equal to array size");
        Element* p = nullptr;
        check_cuda(cudaMalloc(&p, nr_elements() * sizeof(Element)), "PartitionedArray");
        _data.reset(p);
    }

    PartitionedArray(const PartitionedArray&) = delete;
    PartitionedArray& operator=(const PartitionedArray&) = delete;
    PartitionedArray(PartitionedArray&&) = default;
    PartitionedArray& operator=(PartitionedArray&&) = default;

    static PartitionedArray from_host(const Element* host, Shape shape, Shape partition_shape,
                                      cudaStream_t stream = nullptr)
    {
        PartitionedArray a(shape, partition_shape);
        check_cuda(cudaMemcpyAsync(a.data(), host, a.nr_elements() * sizeof(Element), cudaMemcpyHostToDevice, stream),
                   "from_host");
        check_cuda(cudaStreamSynchronize(stream), "from_host");
        return a;
    }

    void to_host(Element* host, cudaStream_t stream = nullptr) const
    {
        check_cuda(cudaMemcpyAsync(host, data(), nr_elements() * sizeof(Element), cudaMemcpyDeviceToHost, stream),
                   "to_host");
        check_cuda(cudaStreamSynchronize(stream), "to_host");
    }

    Element* data() const { return _data.get(); }
    Shape shape() const { return _shape; }
    Shape partition_shape() const { return _partition_shape; }
    Shape shape_in_partitions() const
    {
        return {_shape[0] / _partition_shape[0], _shape[1] / _partition_shape[1]};
    }
    std::int64_t nr_elements() const { return _shape[0] * _shape[1]; }

    // The flow topology of a flow-direction array, built on first use and kept with the array.
    Topology& topology(cudaStream_t stream = nullptr) const
    {
        static_assert(std::is_same_v<Element, std::uint8_t>, "only flow-direction arrays have a topology");
        if (!_topology) _topology = std::make_shared<Topology>(data(), _shape, _partition_shape, stream);
        return *_topology;
    }

   private:
    struct Free {
        void operator()(Element* p) const { cudaFree(p); }
    };
    std::unique_ptr<Element, Free> _data;
    Shape _shape{0, 0};
    Shape _partition_shape{0, 0};
    mutable std::shared_ptr<Topology> _topology;
};

template <typename Element>
struct Scalar {
    Element value;
};

namespace detail {

template <typename A, typename B>
void verify_compatible(const PartitionedArray<A>& a, const PartitionedArray<B>& b)
{
    if (a.shape() != b.shape() || a.shape_in_partitions() != b.shape_in_partitions())
        throw std::runtime_error("Arrays are not compatible: shapes or partitionings differ");
}

template <typename F>
struct Arg {
    const F* ptr;
    F value;
};

template <typename F>
Arg<F> arg(const PartitionedArray<std::uint8_t>& fd, const PartitionedArray<F>& a)
{
    verify_compatible(fd, a);
    return {a.data(), F(0)};
}

template <typename F>
Arg<F> arg(const PartitionedArray<std::uint8_t>&, const Scalar<F>& s)
{
    return {nullptr, s.value};
}

template <typename F>
inline int accu_call(lue_gpu_topology* t, const F* a, F as, F* out, cudaStream_t s);
template <>
inline int accu_call<float>(lue_gpu_topology* t, const float* a, float as, float* out, cudaStream_t s)
{
    return lue_gpu_accu_f32(t, a, as, out, s);
}
template <>
inline int accu_call<double>(lue_gpu_topology* t, const double* a, double as, double* out, cudaStream_t s)
{
    return lue_gpu_accu_f64(t, a, as, out, s);
}

template <typename F>
inline int threshold_call(lue_gpu_topology* t, const F* a, F as, const F* b, F bs, F* o1, F* o2, cudaStream_t s);
template <>
inline int threshold_call<float>(lue_gpu_topology* t, const float* a, float as, const float* b, float bs, float* o1,
                                 float* o2, cudaStream_t s)
{
    return lue_gpu_accu_threshold_f32(t, a, as, b, bs, o1, o2, s);
}
template <>
inline int threshold_call<double>(lue_gpu_topology* t, const double* a, double as, const double* b, double bs,
                                  double* o1, double* o2, cudaStream_t s)
{
    return lue_gpu_accu_threshold_f64(t, a, as, b, bs, o1, o2, s);
}

template <typename F>
inline int fraction_call(lue_gpu_topology* t, const F* a, F as, const F* b, F bs, F* o1, F* o2, cudaStream_t s);
template <>
inline int fraction_call<float>(lue_gpu_topology* t, const float* a, float as, const float* b, float bs, float* o1,
                                float* o2, cudaStream_t s)
{
    return lue_gpu_accu_fraction_f32(t, a, as, b, bs, o1, o2, s);
}
template <>
inline int fraction_call<double>(lue_gpu_topology* t, const double* a, double as, const double* b, double bs,
                                 double* o1, double* o2, cudaStream_t s)
{
    return lue_gpu_accu_fraction_f64(t, a, as, b, bs, o1, o2, s);
}

#define LUE_GB300_TWO_OUTPUT_CALL(NAME)                                                                       \
    template <typename F>                                                                                     \
    inline int NAME##_call(lue_gpu_topology* t, const F* a, F as, const F* b, F bs, F* o1, F* o2, cudaStream_t s); \
    template <>                                                                                               \
    inline int NAME##_call<float>(lue_gpu_topology * t, const float* a, float as, const float* b, float bs,    \
                                  float* o1, float* o2, cudaStream_t s)                                       \
    {                                                                                                         \
        return lue_gpu_accu_##NAME##_f32(t, a, as, b, bs, o1, o2, s);                                          \
    }                                                                                                         \
    template <>                                                                                               \
    inline int NAME##_call<double>(lue_gpu_topology * t, const double* a, double as, const double* b,          \
                                   double bs, double* o1, double* o2, cudaStream_t s)                          \
    {                                                                                                         \
        return lue_gpu_accu_##NAME##_f64(t, a, as, b, bs, o1, o2, s);                                          \
    }
LUE_GB300_TWO_OUTPUT_CALL(capacity)
LUE_GB300_TWO_OUTPUT_CALL(trigger)
#undef LUE_GB300_TWO_OUTPUT_CALL

inline int one_hop_call(bool up, const std::uint8_t* fd, std::int64_t r, std::int64_t c, const float* m, float* o,
                        cudaStream_t s)
{
    return up ? lue_gpu_upstream_f32(fd, r, c, m, o, s) : lue_gpu_downstream_f32(fd, r, c, m, o, s);
}
inline int one_hop_call(bool up, const std::uint8_t* fd, std::int64_t r, std::int64_t c, const double* m, double* o,
                        cudaStream_t s)
{
    return up ? lue_gpu_upstream_f64(fd, r, c, m, o, s) : lue_gpu_downstream_f64(fd, r, c, m, o, s);
}
inline int distance_call(const std::uint8_t* fd, std::int64_t r, std::int64_t c, float cell, float* o, cudaStream_t s)
{
    return lue_gpu_downstream_distance_f32(fd, r, c, cell, o, s);
}
inline int distance_call(const std::uint8_t* fd, std::int64_t r, std::int64_t c, double cell, double* o,
                         cudaStream_t s)
{
    return lue_gpu_downstream_distance_f64(fd, r, c, cell, o, s);
}

}  // namespace detail

// downstream_distance(flow_direction, cell_size) (downstream_distance.hpp:31-44): the length of each
// cell's step to its downstream cell; no-data (NaN) for a no-data flow direction.
template <typename F>
PartitionedArray<F> downstream_distance(const PartitionedArray<std::uint8_t>& fd, F cell_size,
                                        cudaStream_t stream = nullptr)
{
    PartitionedArray<F> out(fd.shape(), fd.partition_shape());
    check(detail::distance_call(fd.data(), fd.shape()[0], fd.shape()[1], cell_size, out.data(), stream),
          "downstream_distance");
    return out;
}

template <typename Count = std::uint8_t>
PartitionedArray<Count> inflow_count(const PartitionedArray<std::uint8_t>& flow_direction, cudaStream_t stream = nullptr)
{
    static_assert(std::is_same_v<Count, std::uint8_t>, "the count element is uint8 (the reference's BooleanElement)");
    PartitionedArray<Count> out(flow_direction.shape(), flow_direction.partition_shape());
    check(lue_gpu_inflow_count_u8(flow_direction.topology(stream).handle(), 1, out.data(), stream), "inflow_count");
    return out;
}

// The cell classes of accu_info (ALG/accu_info.hpp:22-63).
using CellClass = std::uint8_t;
constexpr CellClass ridge_cell = 11, intra_partition_stream_cell = 12, partition_output_cell = 13,
                    partition_input_cell = 14, partition_input_output_cell = 15, inter_partition_stream_cell = 16,
                    sink_cell = 17;

namespace value_policies {

// accu_info(flow_direction): the class of every cell in the partitioned flow accumulation
// (ALG/value_policies/accu_info.hpp:18-26), for the array's partition shape.
inline PartitionedArray<CellClass> accu_info(const PartitionedArray<std::uint8_t>& flow_direction,
                                             cudaStream_t stream = nullptr)
{
    PartitionedArray<CellClass> out(flow_direction.shape(), flow_direction.partition_shape());
    check(lue_gpu_accu_info_u8(flow_direction.topology(stream).handle(), out.data(), stream), "accu_info");
    return out;
}

// partial_accu(flow_direction, inflow, nr_steps) (ALG/value_policies/partial_accu.hpp:17-28): per cell the
// number of the walk's stream that reached it last, NaN above nr_steps, for the array's partition shape.
// The inflow scalar only picks the element type, as in the reference.
template <typename F>
PartitionedArray<F> partial_accu(const PartitionedArray<std::uint8_t>& flow_direction, const Scalar<F>& inflow,
                                 std::int64_t nr_steps, cudaStream_t stream = nullptr)
{
    static_assert(std::is_same_v<F, float> || std::is_same_v<F, double>, "partial_accu: float or double");
    (void)inflow;
    PartitionedArray<F> out(flow_direction.shape(), flow_direction.partition_shape());
    lue_gpu_topology* t = flow_direction.topology(stream).handle();
    if constexpr (std::is_same_v<F, float>)
        check(lue_gpu_partial_accu_f32(t, nr_steps, out.data(), nullptr, stream), "partial_accu");
    else
        check(lue_gpu_partial_accu_f64(t, nr_steps, out.data(), nullptr, stream), "partial_accu");
    return out;
}

// accu(flow_direction, inflow): inflow is a PartitionedArray<F> or a Scalar<F>.
template <typename F, typename Inflow>
PartitionedArray<F> accu(const PartitionedArray<std::uint8_t>& flow_direction, const Inflow& inflow,
                         cudaStream_t stream = nullptr)
{
    auto a = detail::arg<F>(flow_direction, inflow);
    PartitionedArray<F> out(flow_direction.shape(), flow_direction.partition_shape());
    check(detail::accu_call<F>(flow_direction.topology(stream).handle(), a.ptr, a.value, out.data(), stream), "accu");
    return out;
}

template <typename F>
PartitionedArray<F> accu(const PartitionedArray<std::uint8_t>& fd, const PartitionedArray<F>& inflow)
{
    return accu<F, PartitionedArray<F>>(fd, inflow);
}

template <typename F>
PartitionedArray<F> accu(const PartitionedArray<std::uint8_t>& fd, const Scalar<F>& inflow)
{
    return accu<F, Scalar<F>>(fd, inflow);
}

// accu_threshold(flow_direction, inflow, threshold) -> (flux, state); raster/scalar in any combination.
template <typename F, typename Inflow, typename Threshold>
std::tuple<PartitionedArray<F>, PartitionedArray<F>> accu_threshold(const PartitionedArray<std::uint8_t>& fd,
                                                                    const Inflow& inflow, const Threshold& threshold,
                                                                    cudaStream_t stream = nullptr)
{
    auto a = detail::arg<F>(fd, inflow);
    auto b = detail::arg<F>(fd, threshold);
    PartitionedArray<F> flux(fd.shape(), fd.partition_shape()), state(fd.shape(), fd.partition_shape());
    check(detail::threshold_call<F>(fd.topology(stream).handle(), a.ptr, a.value, b.ptr, b.value, flux.data(),
                                    state.data(), stream),
          "accu_threshold");
    return {std::move(flux), std::move(state)};
}

// accu_fraction(flow_direction, inflow, fraction) -> (flux, state).
template <typename F, typename Inflow, typename Fraction>
std::tuple<PartitionedArray<F>, PartitionedArray<F>> accu_fraction(const PartitionedArray<std::uint8_t>& fd,
                                                                   const Inflow& inflow, const Fraction& fraction,
                                                                   cudaStream_t stream = nullptr)
{
    auto a = detail::arg<F>(fd, inflow);
    auto b = detail::arg<F>(fd, fraction);
    PartitionedArray<F> flux(fd.shape(), fd.partition_shape()), state(fd.shape(), fd.partition_shape());
    check(detail::fraction_call<F>(fd.topology(stream).handle(), a.ptr, a.value, b.ptr, b.value, flux.data(),
                                   state.data(), stream),
          "accu_fraction");
    return {std::move(flux), std::move(state)};
}

// accu_capacity(flow_direction, inflow, capacity) -> (outflow, remainder).
template <typename F, typename Inflow, typename Capacity>
std::tuple<PartitionedArray<F>, PartitionedArray<F>> accu_capacity(const PartitionedArray<std::uint8_t>& fd,
                                                                   const Inflow& inflow, const Capacity& capacity,
                                                                   cudaStream_t stream = nullptr)
{
    auto a = detail::arg<F>(fd, inflow);
    auto b = detail::arg<F>(fd, capacity);
    PartitionedArray<F> outflow(fd.shape(), fd.partition_shape()), remainder(fd.shape(), fd.partition_shape());
    check(detail::capacity_call<F>(fd.topology(stream).handle(), a.ptr, a.value, b.ptr, b.value, outflow.data(),
                                   remainder.data(), stream),
          "accu_capacity");
    return {std::move(outflow), std::move(remainder)};
}

// accu_trigger(flow_direction, inflow, trigger) -> (outflow, remainder).
template <typename F, typename Inflow, typename Trigger>
std::tuple<PartitionedArray<F>, PartitionedArray<F>> accu_trigger(const PartitionedArray<std::uint8_t>& fd,
                                                                  const Inflow& inflow, const Trigger& trigger,
                                                                  cudaStream_t stream = nullptr)
{
    auto a = detail::arg<F>(fd, inflow);
    auto b = detail::arg<F>(fd, trigger);
    PartitionedArray<F> outflow(fd.shape(), fd.partition_shape()), remainder(fd.shape(), fd.partition_shape());
    check(detail::trigger_call<F>(fd.topology(stream).handle(), a.ptr, a.value, b.ptr, b.value, outflow.data(),
                                  remainder.data(), stream),
          "accu_trigger");
    return {std::move(outflow), std::move(remainder)};
}

// upstream(flow_direction, material) / downstream(flow_direction, material): one-hop operations.
template <typename F>
PartitionedArray<F> upstream(const PartitionedArray<std::uint8_t>& fd, const PartitionedArray<F>& material,
                             cudaStream_t stream = nullptr)
{
    detail::verify_compatible(fd, material);
    PartitionedArray<F> out(fd.shape(), fd.partition_shape());
    check(detail::one_hop_call(true, fd.data(), fd.shape()[0], fd.shape()[1], material.data(), out.data(), stream),
          "upstream");
    return out;
}

template <typename F>
PartitionedArray<F> downstream(const PartitionedArray<std::uint8_t>& fd, const PartitionedArray<F>& material,
                               cudaStream_t stream = nullptr)
{
    detail::verify_compatible(fd, material);
    PartitionedArray<F> out(fd.shape(), fd.partition_shape());
    check(detail::one_hop_call(false, fd.data(), fd.shape()[0], fd.shape()[1], material.data(), out.data(), stream),
          "downstream");
    return out;
}

// kinematic_wave(flow_direction, current_outflow, inflow, alpha, beta, time_step_duration, channel_length):
// one time step for F = float or double (the reference's two instantiations); alpha, beta and channel
// length are PartitionedArray<F> or Scalar<F>.
template <typename F, typename Alpha, typename Beta, typename ChannelLength>
PartitionedArray<F> kinematic_wave(const PartitionedArray<std::uint8_t>& fd, const PartitionedArray<F>& current_outflow,
                                   const PartitionedArray<F>& inflow, const Alpha& alpha, const Beta& beta,
                                   Scalar<F> time_step_duration, const ChannelLength& channel_length,
                                   cudaStream_t stream = nullptr)
{
    static_assert(std::is_same_v<F, float> || std::is_same_v<F, double>, "kinematic_wave: float or double");
    auto q = detail::arg<F>(fd, current_outflow);
    auto l = detail::arg<F>(fd, inflow);
    auto a = detail::arg<F>(fd, alpha);
    auto b = detail::arg<F>(fd, beta);
    auto d = detail::arg<F>(fd, channel_length);
    PartitionedArray<F> out(fd.shape(), fd.partition_shape());
    if constexpr (std::is_same_v<F, float>)
        check(lue_gpu_kinematic_wave_f32(fd.topology(stream).handle(), q.ptr, q.value, l.ptr, l.value, a.ptr, a.value,
                                         b.ptr, b.value, time_step_duration.value, d.ptr, d.value, out.data(), stream),
              "kinematic_wave");
    else
        check(lue_gpu_kinematic_wave_f64(fd.topology(stream).handle(), q.ptr, q.value, l.ptr, l.value, a.ptr, a.value,
                                         b.ptr, b.value, time_step_duration.value, d.ptr, d.value, out.data(), stream),
              "kinematic_wave");
    return out;
}

}  // namespace value_policies

}  // namespace lue_gb300
