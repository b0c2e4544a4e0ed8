// kinematic_wave.cuh — per-cell kinematic-wave solve (float64, and float32 for the float instantiation).
//
// Restates iterate_to_new_discharge and NonLinearKinematicWave of the reference
// (source/framework/algorithm/include/lue/framework/algorithm/definition/kinematic_wave.hpp:13-254):
//
//   solve  k*Q + alpha*Q^beta = k*Qup + alpha*Qcur^beta + dt*q      (k = dt / dx)
//
//   - no water (Qup + Qcur <= 0 and q <= 0): Q = 0
//   - initial guess: the linearised solve of :61-91, floored at DBL_MIN
//   - Newton-Raphson on [0, DBL_MAX] with Boost.Math's documented newton_raphson_iterate contract
//     (boost/math/tools/roots.hpp; a step that leaves the bracket bisects towards the violated
//     bound; stop when the last step is at most |Q| * 2^(1 - digits), digits = int(53 * 0.6) = 31,
//     or when f(Q) == 0, or after 10 evaluations)
//   - negative lateral inflow extracts min(dx * |q|, Q) afterwards (:242-249)
#pragma once

#include <cfloat>

namespace lue_gb300 {

__device__ __forceinline__ double kw_newton(double k, double alpha, double beta, double known, double guess)
{
    const double factor = 9.313225746154785e-10;  // 2^(1 - 31)
    const double ab = alpha * beta;
    double lo = 0.0, hi = DBL_MAX, x = guess;
    for (int n = 0; n < 10; ++n) {
        double f = k * x + alpha * pow(x, beta) - known;
        double df = k + ab * pow(x, beta - 1.0);
        if (f == 0.0) break;
        double step;
        if (df == 0.0 || !isfinite(df)) step = f > 0.0 ? 0.5 * (x - lo) : 0.5 * (x - hi);
        else step = f / df;
        double next = x - step;
        if (next <= lo) {
            step = 0.5 * (x - lo);
            next = x - step;
        } else if (next >= hi) {
            step = 0.5 * (x - hi);
            next = x - step;
        }
        if (step > 0.0) hi = x;
        else lo = x;
        x = next;
        if (fabs(step) <= fabs(x) * factor) break;
        if (x == lo || x == hi) break;
    }
    return x;
}

__device__ __forceinline__ double iterate_to_new_discharge(double upstream, double current, double lateral,
                                                           double alpha, double beta, double dt, double dx)
{
    double new_q = 0.0;
    if (upstream + current > 0.0 || lateral > 0.0) {
        double inflow = lateral >= 0.0 ? lateral : 0.0;
        double k = dt / dx;
        double known = k * upstream + alpha * pow(current, beta) + dt * inflow;
        double guess = DBL_MIN;
        if (current + upstream != 0.0 || beta >= 1.0) {
            double a_b_pq = alpha * beta * pow((current + upstream) / 2.0, beta - 1.0);
            guess = (k * upstream + a_b_pq * current + dt * inflow) / (k + a_b_pq);
            if (!(guess > DBL_MIN)) guess = DBL_MIN;
        }
        new_q = kw_newton(k, alpha, beta, known, guess);
    }
    if (lateral < 0.0) new_q -= fmin(dx * fabs(lateral), new_q);
    return new_q;
}

// The same solve for F = float (the reference instantiates every routing operation for float and double,
// definition/kinematic_wave.hpp:662-684): float arithmetic, initial guess floored at FLT_MIN, bracket
// [0, FLT_MAX], stop when the last step is at most |Q| * 2^(1 - digits) with digits = int(24 * 0.6) = 14
// (:199-213), at most 10 evaluations.
__device__ __forceinline__ float kw_newton_f32(float k, float alpha, float beta, float known, float guess)
{
    const float factor = 1.220703125e-4f;  // 2^(1 - 14)
    const float ab = alpha * beta;
    float lo = 0.0f, hi = FLT_MAX, x = guess;
    for (int n = 0; n < 10; ++n) {
        const float f = k * x + alpha * powf(x, beta) - known;
        const float df = k + ab * powf(x, beta - 1.0f);
        if (f == 0.0f) break;
        float step;
        if (df == 0.0f || !isfinite(df)) step = f > 0.0f ? 0.5f * (x - lo) : 0.5f * (x - hi);
        else step = f / df;
        float next = x - step;
        if (next <= lo) {
            step = 0.5f * (x - lo);
            next = x - step;
        } else if (next >= hi) {
            step = 0.5f * (x - hi);
            next = x - step;
        }
        if (step > 0.0f) hi = x;
        else lo = x;
        x = next;
        if (fabsf(step) <= fabsf(x) * factor) break;
        if (x == lo || x == hi) break;
    }
    return x;
}

__device__ __forceinline__ float iterate_to_new_discharge_f32(float upstream, float current, float lateral,
                                                              float alpha, float beta, float dt, float dx)
{
    float new_q = 0.0f;
    if (upstream + current > 0.0f || lateral > 0.0f) {
        const float inflow = lateral >= 0.0f ? lateral : 0.0f;
        const float k = dt / dx;
        const float known = k * upstream + alpha * powf(current, beta) + dt * inflow;
        float guess = FLT_MIN;
        if (current + upstream != 0.0f || beta >= 1.0f) {
            const float a_b_pq = alpha * beta * powf((current + upstream) / 2.0f, beta - 1.0f);
            guess = (k * upstream + a_b_pq * current + dt * inflow) / (k + a_b_pq);
            if (!(guess > FLT_MIN)) guess = FLT_MIN;
        }
        new_q = kw_newton_f32(k, alpha, beta, known, guess);
    }
    if (lateral < 0.0f) new_q -= fminf(dx * fabsf(lateral), new_q);
    return new_q;
}

}  // namespace lue_gb300
