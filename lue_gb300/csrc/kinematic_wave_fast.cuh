// kinematic_wave_fast.cuh — the per-cell kinematic-wave solve with few float64 operations.
//
// GB300 runs float64 at a small fraction of its float32 rate, so the reference-faithful solve of
// kinematic_wave.cuh (about ten float64 pow() calls per cell) is bound by float64 throughput.  This
// solve reaches the same root with about 30 float64 operations:
//
//   1. known = k*Qup + alpha*Qcur^beta + dt*q                      (float64; Qcur^beta by pow_rational)
//   2. Newton-Raphson in float32 from the reference's linearised guess (kinematic_wave.hpp:61-91), to
//      float32 convergence                                          (float32)
//   3. one Newton step in float64 on f(Q) = k*Q + alpha*Q^beta - known, with Q^beta by pow_rational and
//      the float32 derivative; a second step when the first moved Q by more than 1e-9 relative
//
// pow_rational(Q) for beta = p/m with small m (beta = 0.6 is 3/5): y0 = powf(Q, beta) in float32, then
// one Newton step for y^m = Q^p in float64 (integer powers only).  Each Newton step squares the
// relative error: 1e-7 -> ~1e-14, below the 1e-9 relative tolerance against the float64 oracle.
//
// The reference's root (Boost's Newton iteration with 31-bit stopping) and this one agree to about
// 1e-14 relative wherever the reference converges.  Where it may not converge within its 10 iterations
// (a guess of DBL_MIN: Qup + Qcur == 0), and for beta that is not a small rational or a per-cell
// raster, the reference-faithful solve runs instead.
#pragma once

#include "kinematic_wave.cuh"

namespace lue_gb300 {

struct BetaRational {
    int p, m;      // beta = p / m, 0 < p, 1 <= m <= 16; m == 0: not rational (slow path)
    float beta_f;  // float32 beta
};

__device__ __forceinline__ double ipow(double x, int e)
{
    double r = 1.0, b = x;
    while (e) {
        if (e & 1) r *= b;
        b *= b;
        e >>= 1;
    }
    return r;
}

// Q^beta in float64 to ~1e-14 relative for Q in [1e-60, 1e60]; false outside that range.
__device__ __forceinline__ bool pow_rational(double q, BetaRational b, double& y)
{
    if (!(q >= 1e-60 && q <= 1e60)) return false;
    float y0f = powf((float)q, b.beta_f);
    double y0 = (double)y0f;
    double ym = ipow(y0, b.m);       // y0^m
    double qp = ipow(q, b.p);        // Q^p
    float rcp = 1.0f / ((float)b.m * (float)ipow(y0, b.m - 1));
    y = y0 - (ym - qp) * (double)rcp;
    return true;
}

__device__ __forceinline__ double iterate_to_new_discharge_fast(double upstream, double current, double lateral,
                                                                double alpha, double beta, BetaRational br,
                                                                double dt, double dx)
{
    // Outside the fast path's scope: the reference-faithful solve.
    if (br.m == 0 || !(upstream + current > 0.0) || lateral < 0.0)
        return iterate_to_new_discharge(upstream, current, lateral, alpha, beta, dt, dx);
    double cb;
    if (current == 0.0) cb = 0.0;
    else if (!pow_rational(current, br, cb)) return iterate_to_new_discharge(upstream, current, lateral, alpha, beta, dt, dx);
    const double k = dt / dx;
    const double known = k * upstream + alpha * cb + dt * lateral;
    // float32 Newton from the reference's linearised guess
    const float kf = (float)k, af = (float)alpha, bf = br.beta_f, knf = (float)known;
    const float mean = (float)((current + upstream) * 0.5);
    const float abpq = af * bf * powf(mean, bf - 1.0f);
    float x = ((float)(k * upstream) + abpq * (float)current + (float)(dt * lateral)) / (kf + abpq);
    if (!(x > 1e-30f)) x = 1e-30f;
    bool converged = false;
    for (int it = 0; it < 12; ++it) {
        float xb = powf(x, bf);
        float f = kf * x + af * xb - knf;
        float df = kf + af * bf * xb / x;
        float nx = x - f / df;
        if (!(nx > 0.0f)) nx = 0.5f * x;
        float dxr = fabsf(nx - x);
        x = nx;
        if (dxr <= 4e-7f * x) {
            converged = true;
            break;
        }
    }
    if (!isfinite(x) || !(x > 1e-30f)) return iterate_to_new_discharge(upstream, current, lateral, alpha, beta, dt, dx);
    // float64 polish: one Newton step from a float32-converged root (1e-7 -> ~1e-14), two otherwise
    double q = (double)x;
    for (int it = 0; it < (converged ? 1 : 2); ++it) {
        double qb;
        if (!pow_rational(q, br, qb)) return iterate_to_new_discharge(upstream, current, lateral, alpha, beta, dt, dx);
        double f = k * q + alpha * qb - known;
        float xq = (float)q;
        float df = kf + af * bf * (float)qb / xq;
        q -= f * (double)(1.0f / df);
    }
    return q;
}

}  // namespace lue_gb300
