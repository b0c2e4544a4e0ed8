// accu_example.cpp — the reference's back_and_forth accu case (accu_test.cpp:1248-1308) and the
// pcraster manual example of accu_threshold (accu_threshold_test.cpp:65-132), with accu_capacity,
// accu_trigger, upstream, downstream, downstream_distance, partial_accu and float kinematic_wave on the
// same rasters, through the C++ mirror of lue::value_policies.  Prints the results row-major, one raster per line; exit status 0 on success.
#include <cstdio>
#include <vector>

#include "lue_gb300.hpp"

using namespace lue_gb300;

int main()
{
    try {
        // back_and_forth: 6 x 5 array in 3 x 5 partitions, inflow 1 everywhere
        const std::uint8_t s = 2, e = 6, n = 8, p = 5;
        std::vector<std::uint8_t> fd1 = {s, e, s, e, s, s, n, s, n, s, s, n, s, n, s,
                                         s, n, s, n, s, s, n, s, n, s, e, n, e, n, p};
        auto flow_direction = PartitionedArray<std::uint8_t>::from_host(fd1.data(), {6, 5}, {3, 5});
        auto outflow = value_policies::accu(flow_direction, Scalar<float>{1.0f});
        std::vector<float> out(30);
        outflow.to_host(out.data());
        for (float v : out) std::printf("%g ", v);
        std::printf("\n");

        // pcraster manual example 1: accu_threshold with a raster inflow and a scalar threshold of 1.5
        const std::uint8_t sw = 1, w = 4, se = 3;
        std::vector<std::uint8_t> fd2 = {s, s, s, sw, sw, s, s, sw, sw, sw, se, s, sw, w, sw,
                                         se, s, sw, w, w, e, p, w, w, w};
        std::vector<float> inflow = {6.0f, 0.5f, 2.0f, 2.0f, 2.0f, 0.5f, 0.5f, 2.0f, 2.0f, 2.0f, 0.5f, 0.5f, 2.0f,
                                     2.0f, 0.0f, 0.5f, 0.5f, 6.0f, 0.0f, 0.0f, 0.5f, 6.0f, 6.0f, 6.0f, 6.0f};
        auto fd = PartitionedArray<std::uint8_t>::from_host(fd2.data(), {5, 5}, {5, 5});
        auto in = PartitionedArray<float>::from_host(inflow.data(), {5, 5}, {5, 5});
        auto [flux, state] = value_policies::accu_threshold<float>(fd, in, Scalar<float>{1.5f});
        std::vector<float> f(25), st(25);
        flux.to_host(f.data());
        state.to_host(st.data());
        for (float v : f) std::printf("%g ", v);
        std::printf("\n");
        for (float v : st) std::printf("%g ", v);
        std::printf("\n");

        // accu_capacity and accu_trigger on the same rasters (accu_capacity_test.cpp:65-134,
        // accu_trigger_test.cpp:65-134), upstream / downstream of the inflow, downstream_distance
        auto [cap_out, cap_rem] = value_policies::accu_capacity<float>(fd, in, Scalar<float>{1.5f});
        auto [trig_out, trig_rem] = value_policies::accu_trigger<float>(fd, in, Scalar<float>{1.5f});
        auto up = value_policies::upstream(fd, in);
        auto down = value_policies::downstream(fd, in);
        auto dist = downstream_distance(fd, 2.0f);
        for (auto* a : {&cap_out, &cap_rem, &trig_out, &trig_rem, &up, &down, &dist}) {
            std::vector<float> v(25);
            a->to_host(v.data());
            for (float x : v) std::printf("%g ", x);
            std::printf("\n");
        }

        // a shape mismatch throws, like the reference's verify_compatible
        auto other = PartitionedArray<float>(Shape{5, 6}, Shape{5, 6});
        try {
            value_policies::accu(fd, other);
            std::printf("no exception\n");
            return 1;
        } catch (const std::runtime_error&) {
            std::printf("shape mismatch rejected\n");
        }

        // the stage schedule autotuned for this accu_threshold call; the result stays the same
        auto tuned = fd.topology().autotune_stage_schedule(
            [&] { flux = std::get<0>(value_policies::accu_threshold<float>(fd, in, Scalar<float>{1.5f})); }, nullptr);
        flux.to_host(f.data());
        for (float v : f) std::printf("%g ", v);
        std::printf("\n");
        std::printf("schedule cap %d threads %d publish_every %d ms %g\n", tuned.cap, tuned.threads,
                    tuned.publish_every, tuned.ms);

        // partial_accu on back_and_forth (its 3 x 5 partitions) and the float instantiation of
        // kinematic_wave on the pcraster rasters (current outflow = inflow / 10, lateral inflow = inflow /
        // 1000, alpha 1.5, beta 0.6, dt 15 s, channel length 10 m)
        auto partial = value_policies::partial_accu(flow_direction, Scalar<float>{0.0f}, 1000);
        partial.to_host(out.data());
        for (float v : out) std::printf("%g ", v);
        std::printf("\n");
        std::vector<float> q0(25), lat(25);
        for (int i = 0; i < 25; ++i) {
            q0[i] = inflow[i] / 10.0f;
            lat[i] = inflow[i] / 1000.0f;
        }
        auto q = PartitionedArray<float>::from_host(q0.data(), {5, 5}, {5, 5});
        auto l = PartitionedArray<float>::from_host(lat.data(), {5, 5}, {5, 5});
        auto q1 = value_policies::kinematic_wave(fd, q, l, Scalar<float>{1.5f}, Scalar<float>{0.6f},
                                                 Scalar<float>{15.0f}, Scalar<float>{10.0f});
        q1.to_host(f.data());
        for (float v : f) std::printf("%.9g ", v);
        std::printf("\n");
    } catch (const std::exception& ex) {
        std::fprintf(stderr, "error: %s\n", ex.what());
        return 2;
    }
    return 0;
}
