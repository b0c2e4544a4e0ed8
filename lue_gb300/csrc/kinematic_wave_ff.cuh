// kinematic_wave_ff.cuh — the kinematic-wave cell solve in float-float arithmetic, for many time steps.
//
// GB300 runs float64 at a small fraction of its float32 rate, so a solve with float64 arithmetic in
// every step is bound by the float64 pipe.  Here the discharge Q, its power P = Q^beta and the
// upstream sum are float-float values (hi + lo, about 48 significant bits, relative error ~1e-14) and
// every operation runs on the float32 pipes:
//
//   known = k*Qup + alpha*P_prev + dt*q                  (k = dt / dx; P_prev carried from the last step)
//   Q0    = float32 Newton-Raphson with exp2/log2 powers, from the previous discharge (or the reference's
//           linearised guess, kinematic_wave.hpp:61-91, when that is 0), to ~1e-6
//   Q     = two Newton steps on f(Q) = k*Q + alpha*Q^beta - known in float-float (1e-6 -> 1e-12 -> ~1e-14),
//           with one float-float power: the second step's power is the first one's moved along its
//           Taylor series
//   P     = Q^beta, the same way
//
// Q^beta for beta = p/m (beta = 0.6 is 3/5): y0 = __powf(Q, beta), then two Newton steps for y^m = Q^p
// in float-float (integer powers only).  Cases outside this path run the float64 solve of
// kinematic_wave.cuh (rare): no upstream discharge and no current discharge (the reference then starts
// from DBL_MIN), a float32 Newton that does not settle, and Q outside [1e-12, 1e12].
#pragma once

#include "kinematic_wave_fast.cuh"

namespace lue_gb300 {

struct ffloat {
    float hi, lo;
};

__device__ __forceinline__ ffloat ff_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return ffloat{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ ffloat ff_fast_two_sum(float a, float b)  // |a| >= |b| or a == 0
{
    const float s = __fadd_rn(a, b);
    return ffloat{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ ffloat ff_neg(ffloat a) { return ffloat{-a.hi, -a.lo}; }
__device__ __forceinline__ ffloat ff_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return ffloat{p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ ffloat ff_mul_f(ffloat a, float b)
{
    const float p = __fmul_rn(a.hi, b);
    float e = __fmaf_rn(a.hi, b, -p);
    e = __fmaf_rn(a.lo, b, e);
    return ff_fast_two_sum(p, e);
}
__device__ __forceinline__ ffloat ff_mul(ffloat a, ffloat b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, e));
    return ff_fast_two_sum(p, e);
}
__device__ __forceinline__ ffloat ff_from_double(double d)
{
    const float h = __double2float_rn(d);
    return ffloat{h, __double2float_rn(d - (double)h)};
}
__device__ __forceinline__ double ff_to_double(ffloat a) { return (double)a.hi + (double)a.lo; }

// a + b with an error of about 2^-48 (|a| + |b|): enough wherever the result is not compared against
// cancellation below that.
__device__ __forceinline__ ffloat ff_add_sloppy(ffloat a, ffloat b)
{
    ffloat s = ff_two_sum(a.hi, b.hi);
    s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
    return ff_fast_two_sum(s.hi, s.lo);
}

// y^e in float-float for a small compile-time or run-time exponent e >= 1.
template <int E>
__device__ __forceinline__ ffloat ff_pow_n(ffloat y, int e_runtime)
{
    const int e = E > 0 ? E : e_runtime;
    ffloat r = y;
#pragma unroll
    for (int i = 1; i < (E > 0 ? E : 16); ++i) {
        if (i >= e) break;
        r = ff_mul(r, y);
    }
    return r;
}
template <int E>
__device__ __forceinline__ float f_pow_n(float y, int e_runtime)
{
    const int e = E > 0 ? E : e_runtime;
    float r = y;
#pragma unroll
    for (int i = 1; i < (E > 0 ? E : 16); ++i) {
        if (i >= e) break;
        r *= y;
    }
    return r;
}

struct KWConstFF {
    ffloat k;       // dt / dx
    ffloat dt;
    float kf, beta_f;
    double beta, dt_d, dx_d;
    BetaRational br;
    bool bad;       // NaN beta / dt / dx, or dx <= 0: every cell is no-data
};

// The kinematic-wave solve in the variable y = Q^(1/m), for beta = p/m: Q^beta = y^p and Q = y^m, so the
// equation k*Q + alpha*Q^beta = known becomes the polynomial
//
//     g(y) = k*y^m + alpha*y^p - known = 0,     g'(y) = m*k*y^(m-1) + p*alpha*y^(p-1),
//
// which is increasing and convex for y > 0: Newton-Raphson needs no exp/log, converges monotonically
// after its first step, and its float-float steps cost a few multiplications.  The cell state is y
// (float-float); the outflow passed downstream is Q = y^m.  P and M are compile-time p and m, or 0 to
// take them from K.br at run time.
// x^(p-1) and x^(m-1) from one chain of products (P, M compile-time, or 0 for run-time p, m <= 16).
template <int P, int M>
__device__ __forceinline__ void f_powers(float x, int p, int m, float& xp1, float& xm1)
{
    constexpr int kTop = P > 0 && M > 0 ? (P > M ? P : M) - 1 : 15;
    const int top = max(p, m) - 1;
    float r = 1.0f;
    xp1 = 1.0f;
    xm1 = 1.0f;
#pragma unroll
    for (int e = 1; e <= kTop; ++e) {
        if (e > top) break;
        r = e == 1 ? x : r * x;
        if (e == p - 1) xp1 = r;
        if (e == m - 1) xm1 = r;
    }
}

// x^p and x^m in float-float for a float x, from one chain of float-float products by x.
template <int P, int M>
__device__ __forceinline__ void ff_powers_f(float x, int p, int m, ffloat& yp, ffloat& ym)
{
    constexpr int kTop = P > 0 && M > 0 ? (P > M ? P : M) : 16;
    const int top = max(p, m);
    ffloat r{x, 0.0f};
    yp = r;
    ym = r;
#pragma unroll
    for (int e = 2; e <= kTop; ++e) {
        if (e > top) break;
        r = e == 2 ? ff_prod(x, x) : ff_mul_f(r, x);
        if (e == p) yp = r;
        if (e == m) ym = r;
    }
}

// y = Q^(1/m) in float-float, for the state of a cell that starts from discharge Q (rare: once per call
// and cell).
template <int P, int M>
__device__ __forceinline__ ffloat kw_poly_root(ffloat q, const KWConstFF& K)
{
    if (!(q.hi > 0.0f)) return ffloat{q.hi == 0.0f ? 0.0f : q.hi, 0.0f};
    const int m = M > 0 ? M : K.br.m;
    if (!(q.hi >= 1e-30f && q.hi <= 1e30f)) return ff_from_double(pow(ff_to_double(q), 1.0 / (double)m));
    ffloat y{__powf(q.hi, 1.0f / (float)m), 0.0f};
#pragma unroll 1
    for (int it = 0; it < 3; ++it) {  // Newton on y^m - q: 1e-6 -> 1e-12 -> ~1e-14
        const ffloat r = ff_add_sloppy(ff_pow_n<M>(y, m), ff_neg(q));
        const float d = m > 1 ? (float)m * f_pow_n<(M > 1 ? M - 1 : 0)>(y.hi, m - 1) : 1.0f;
        y = ff_add_sloppy(y, ffloat{-__fdividef(r.hi, d), 0.0f});
    }
    return y;
}

// One step of one cell in the variable y (see above).  y is the cell's state from the previous step and
// becomes this step's; up is the upstream sum of this step; returns the outflow Q = y^m (NaN for
// no-data).  The cases the polynomial path does not take run the float64 solve of the reference.
template <int P, int M>
__device__ __forceinline__ ffloat kw_step_poly(ffloat up, bool nan, ffloat& y, float lat, float al,
                                               const KWConstFF& K)
{
    const float nanf = __int_as_float(0x7fc00000);
    const int m = M > 0 ? M : K.br.m, p = P > 0 ? P : K.br.p;
    if (nan || K.bad || isnan(y.hi) || isnan(lat) || isnan(al) || !(y.hi >= 0.0f) || !(lat >= 0.0f)) {
        y = ffloat{nanf, 0.0f};
        return y;
    }
    const float qprev_f = f_pow_n<M>(y.hi, m);
    const bool flow = up.hi + qprev_f > 0.0f;
    if (!flow && !(lat > 0.0f)) {  // no water (kinematic_wave.hpp:181-185)
        y = ffloat{0.0f, 0.0f};
        return y;
    }
    if (flow && y.hi > 1e-12f && y.hi < 1e12f && al > 0.0f) {
        const ffloat known = ff_add_sloppy(ff_add_sloppy(ff_mul(K.k, up), ff_mul_f(ff_pow_n<P>(y, p), al)),
                                           ff_mul_f(K.dt, lat));
        const float kf = K.kf, knf = known.hi;
        // Float Newton to the float noise floor: it stops after a step below 3e-5 relative, which leaves
        // an error of about (3e-5)^2, far below that floor (quadratic convergence, g'' / g' ~ 1 / y).
        // It starts from the previous state, or, when that is more than 1 % off in g, from the better
        // (smaller |g|) of the previous state and the reference's linearised guess (kinematic_wave.hpp:
        // 61-91) taken to the power 1/m: after a jump in upstream discharge the previous state can be
        // orders of magnitude off, and Newton on y^m closes such a gap only by a factor of about
        // (m - 1) / m per step.
        float x = y.hi;
        {
            float xm1, xp1;
            f_powers<P, M>(x, p, m, xp1, xm1);
            const float ga = kf * xm1 * x + al * xp1 * x - knf;
            if (!(fabsf(ga) <= 0.01f * fabsf(knf))) {
                const float q0 = qprev_f, mean = 0.5f * (q0 + up.hi);
                const float abpq = al * K.beta_f * __powf(mean, K.beta_f - 1.0f);
                const float guess = __fdividef(kf * up.hi + abpq * q0 + K.dt.hi * lat, kf + abpq);
                const float xg = guess > 0.0f ? __powf(guess, 1.0f / (float)m) : 0.0f;
                f_powers<P, M>(xg, p, m, xp1, xm1);
                const float gb = kf * xm1 * xg + al * xp1 * xg - knf;
                if (xg > 0.0f && isfinite(gb) && fabsf(gb) < fabsf(ga)) x = xg;
            }
        }
        bool converged = false;
#pragma unroll 1
        for (int it = 0; it < 24; ++it) {
            float xm1, xp1;
            f_powers<P, M>(x, p, m, xp1, xm1);
            const float g = kf * xm1 * x + al * xp1 * x - knf;
            const float dg = (float)m * kf * xm1 + (float)p * al * xp1;
            float nx = x - __fdividef(g, dg);
            if (!(nx > 0.0f)) nx = 0.5f * x;
            const float dxr = fabsf(nx - x);
            x = nx;
            if (dxr <= 3e-5f * x) {
                converged = true;
                break;
            }
        }
        if (converged && x > 1e-12f && x < 1e12f) {
            // one float-float Newton step from the float root x (1e-7 -> ~1e-14); the powers of x are
            // float-float products of floats, and Q = y^m moves with y to first order
            ffloat yp, ym;
            ff_powers_f<P, M>(x, p, m, yp, ym);
            const ffloat g = ff_add_sloppy(ff_add_sloppy(ff_mul(K.k, ym), ff_mul_f(yp, al)), ff_neg(known));
            float xm1, xp1;
            f_powers<P, M>(x, p, m, xp1, xm1);
            const float dg = (float)m * kf * xm1 + (float)p * al * xp1;
            const float delta = __fdividef(g.hi, dg);
            y = ff_two_sum(x, -delta);
            return ff_add_sloppy(ym, ffloat{-(float)m * xm1 * delta, 0.0f});
        }
    }
    // the float64 solve of the reference (rare)
    const double q = iterate_to_new_discharge(ff_to_double(up), ff_to_double(ff_pow_n<M>(y, m)), (double)lat, (double)al, K.beta,
                                              K.dt_d, K.dx_d);
    y = kw_poly_root<P, M>(ff_from_double(q), K);
    return ff_pow_n<M>(y, m);
}

}  // namespace lue_gb300
