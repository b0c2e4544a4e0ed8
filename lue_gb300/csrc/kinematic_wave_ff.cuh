// kinematic_wave_ff.cuh — the kinematic-wave cell solve in float-float arithmetic, for many time steps.
//
// GB300 runs float64 at a small fraction of its float32 rate, so a solve with float64 arithmetic in
// every step is bound by the float64 pipe.  Here the discharge Q, its power P = Q^beta and the
// upstream sum are float-float values (hi + lo, about 48 significant bits, relative error ~1e-14) and
// every operation runs on the float32 pipes:
//
//   known = k*Qup + alpha*P_prev + dt*q                  (k = dt / dx; P_prev carried from the last step)
//   Q0    = float32 Newton-Raphson from the reference's linearised guess (kinematic_wave.hpp:61-91)
//   Q     = Q0 - f(Q0) / f'(Q0) with f(Q) = k*Q + alpha*Q^beta - known in float-float   (one Newton step
//           from a float32 root: 1e-7 -> ~1e-14)
//   P     = Q^beta from Q0^beta (see pow_rational_ff) moved to Q to first order
//
// Q^beta for beta = p/m (beta = 0.6 is 3/5): y0 = powf(Q, beta), then one Newton step for y^m = Q^p in
// float-float (integer powers only).  Cases outside this path run the float64 solve of
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
__device__ __forceinline__ ffloat ff_add(ffloat a, ffloat b)
{
    ffloat s = ff_two_sum(a.hi, b.hi);
    const ffloat t = ff_two_sum(a.lo, b.lo);
    s.lo = __fadd_rn(s.lo, t.hi);
    s = ff_fast_two_sum(s.hi, s.lo);
    s.lo = __fadd_rn(s.lo, t.lo);
    return ff_fast_two_sum(s.hi, s.lo);
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

__device__ __forceinline__ ffloat ff_ipow(ffloat x, int e)  // e >= 1
{
    ffloat r = x, b = x;
    bool first = true;
    while (e) {
        if (e & 1) {
            r = first ? b : ff_mul(r, b);
            first = false;
        }
        e >>= 1;
        if (e) b = ff_mul(b, b);
    }
    return r;
}

// x^(p/m) in float-float for 1e-12 <= x <= 1e12 (x^p and y^m stay in float range for p, m <= 3).
__device__ __forceinline__ ffloat pow_rational_ff(ffloat x, BetaRational br)
{
    const float y0 = powf(x.hi, br.beta_f);
    const ffloat ym = ff_ipow(ffloat{y0, 0.0f}, br.m);
    const ffloat xp = ff_ipow(x, br.p);
    const ffloat diff = ff_add(ym, ff_neg(xp));
    float dm = (float)br.m;
    for (int i = 1; i < br.m; ++i) dm *= y0;
    return ff_two_sum(y0, -diff.hi / dm);
}

// Whether float-float powers of x stay in range for beta = p/m.
__device__ __forceinline__ bool ff_pow_ok(float x, BetaRational br)
{
    return br.p <= 3 && br.m <= 5 && x >= 1e-12f && x <= 1e12f;
}

// Q^beta in float-float, through float64 when the float-float path is out of range.
__device__ __forceinline__ ffloat kw_power(ffloat q, BetaRational br, double beta)
{
    if (q.hi == 0.0f) return ffloat{0.0f, 0.0f};
    if (ff_pow_ok(q.hi, br)) return pow_rational_ff(q, br);
    return ff_from_double(pow(ff_to_double(q), beta));
}

struct KWConstFF {
    ffloat k;       // dt / dx
    ffloat dt;
    float kf, beta_f;
    double beta, dt_d, dx_d;
    BetaRational br;
    bool bad;       // NaN beta / dt / dx, or dx <= 0: every cell is no-data
};

// One step of one cell.  Q and P (= Q^beta) are the cell's discharge and power from the previous step
// and become this step's; up is the upstream sum of this step.  Returns false (Q, P = NaN) for no-data.
__device__ __forceinline__ bool kw_step_ff(ffloat up, bool nan, ffloat& Q, ffloat& P, float lat, float al,
                                           const KWConstFF& K)
{
    const float nanf = __int_as_float(0x7fc00000);
    if (nan || K.bad || isnan(Q.hi) || isnan(lat) || isnan(al) || !(Q.hi >= 0.0f) || !(lat >= 0.0f)) {
        Q = P = ffloat{nanf, 0.0f};
        return false;
    }
    const bool flow = up.hi + Q.hi > 0.0f;
    if (!flow && !(lat > 0.0f)) {  // no water (kinematic_wave.hpp:181-185)
        Q = P = ffloat{0.0f, 0.0f};
        return true;
    }
    float x = 0.0f;
    bool fast = flow;
    if (fast) {
        // known right-hand side in float-float
        const ffloat known = ff_add(ff_add(ff_mul(K.k, up), ff_mul_f(P, al)), ff_mul_f(K.dt, lat));
        // float32 Newton from the reference's linearised guess
        const float kf = K.kf, bf = K.beta_f, knf = known.hi;
        const float mean = 0.5f * (Q.hi + up.hi);
        const float abpq = al * bf * powf(mean, bf - 1.0f);
        x = (kf * up.hi + abpq * Q.hi + K.dt.hi * lat) / (kf + abpq);
        if (!(x > 1e-30f)) x = 1e-30f;
        bool converged = false;
        for (int it = 0; it < 12; ++it) {
            const float xb = powf(x, bf);
            const float f = kf * x + al * xb - knf;
            const float df = kf + al * bf * xb / x;
            float nx = x - f / df;
            if (!(nx > 0.0f)) nx = 0.5f * x;
            const float dxr = fabsf(nx - x);
            x = nx;
            if (dxr <= 4e-7f * x) {
                converged = true;
                break;
            }
        }
        fast = converged && isfinite(x) && ff_pow_ok(x, K.br);
        if (fast) {
            // one float-float Newton step, and the power moved along with it
            const ffloat y = pow_rational_ff(ffloat{x, 0.0f}, K.br);
            const ffloat f = ff_add(ff_add(ff_mul_f(K.k, x), ff_mul_f(y, al)), ff_neg(known));
            const float df = kf + al * bf * y.hi / x;
            const float delta = f.hi / df;
            Q = ff_two_sum(x, -delta);
            P = ff_add(y, ffloat{-y.hi * bf * (delta / x), 0.0f});
            return true;
        }
    }
    // the float64 solve of the reference (rare)
    const double q = iterate_to_new_discharge(ff_to_double(up), ff_to_double(Q), (double)lat, (double)al, K.beta,
                                              K.dt_d, K.dx_d);
    Q = ff_from_double(q);
    P = q > 0.0 ? ff_from_double(pow(q, K.beta)) : ffloat{0.0f, 0.0f};
    return true;
}

}  // namespace lue_gb300
