// route_walk_visitors.cuh — cell rules of accu, accu_threshold, accu_fraction and kinematic_wave as
// visitors of the walk engine (walk.cuh), and the pass that finishes cells on or below flow cycles.
// See route_walk.cu for the reference counterparts.
#pragma once

#include <cfloat>

#include "kinematic_wave_fast.cuh"
#include "walk.cuh"

namespace lue_gb300 {

template <class T>
__device__ __forceinline__ T value_at(const T* p, T s, int64_t i)
{
    return p ? __ldg(p + i) : s;
}

template <class T>
__device__ __forceinline__ T qnan();
template <>
__device__ __forceinline__ float qnan<float>() { return __int_as_float(0x7fc00000); }
template <>
__device__ __forceinline__ double qnan<double>() { return __longlong_as_double(0x7ff8000000000000ll); }

enum class Rule { accu, threshold, fraction, capacity, trigger };

// --- float32: float-float running values ---------------------------------------------------------

// The float32 cell rule on the float-float upstream sum t (already normalised or not) and the cell's
// inputs: the outflow (out_hi + out_lo, passed on downstream) and the state.  False: the cell is no-data.
template <Rule R>
__device__ __forceinline__ bool rule_f32(FF t, bool nan, float x, float b, float& out_hi, float& out_lo, float& rem)
{
    if (R == Rule::accu) {
        if (nan || isnan(x) || !(x >= 0.0f)) return false;
        t.add(x);
        t.normalise();
        out_hi = t.hi;
        out_lo = t.lo;
    } else if (R == Rule::threshold) {
        const float th = b;
        if (nan || isnan(x) || isnan(th) || !(x >= 0.0f && th >= 0.0f)) return false;
        t.add(x);
        t.normalise();
        // strict '>' on the compensated total (accu_threshold.hpp:157)
        if (t.hi > th || (t.hi == th && t.lo > 0.0f)) {
            FF d{0.0f, 0.0f};
            two_sum(t.hi, -th, d.hi, d.lo);
            d.lo = __fadd_rn(d.lo, t.lo);
            d.normalise();
            rem = th;
            out_hi = d.hi;
            out_lo = d.lo;
        } else {
            rem = __fadd_rn(t.hi, t.lo);
            out_hi = 0.0f;
            out_lo = 0.0f;
        }
    } else if (R == Rule::capacity) {
        // what flows on is capped at the capacity, the rest stays (accu_capacity.hpp enter_cell)
        const float cap = b;
        if (nan || isnan(x) || isnan(cap) || !(x >= 0.0f && cap >= 0.0f)) return false;
        t.add(x);
        t.normalise();
        if (t.hi > cap || (t.hi == cap && t.lo > 0.0f)) {
            FF d{0.0f, 0.0f};
            two_sum(t.hi, -cap, d.hi, d.lo);
            d.lo = __fadd_rn(d.lo, t.lo);
            rem = __fadd_rn(d.hi, d.lo);
            out_hi = cap;
            out_lo = 0.0f;
        } else {
            rem = 0.0f;
            out_hi = t.hi;
            out_lo = t.lo;
        }
    } else if (R == Rule::trigger) {
        // the total flows on once it reaches the trigger, else it all stays (accu_trigger.hpp enter_cell,
        // strict '<')
        const float trig = b;
        if (nan || isnan(x) || isnan(trig) || !(x >= 0.0f && trig >= 0.0f)) return false;
        t.add(x);
        t.normalise();
        if (t.hi < trig || (t.hi == trig && t.lo < 0.0f)) {
            rem = __fadd_rn(t.hi, t.lo);
            out_hi = 0.0f;
            out_lo = 0.0f;
        } else {
            rem = 0.0f;
            out_hi = t.hi;
            out_lo = t.lo;
        }
    } else {
        const float f = b;
        if (nan || isnan(x) || isnan(f) || !(x >= 0.0f && f >= 0.0f && f <= 1.0f)) return false;
        t.add(x);
        t.normalise();
        // flux = fraction * total, state = total - flux (accu_fraction.hpp:157-159)
        float ph = __fmul_rn(f, t.hi);
        float pl = __fmaf_rn(f, t.hi, -ph);
        pl = __fmaf_rn(f, t.lo, pl);
        FF d{ph, pl};
        d.normalise();
        FF r{0.0f, 0.0f};
        two_sum(t.hi, -d.hi, r.hi, r.lo);
        r.lo = __fadd_rn(r.lo, __fsub_rn(t.lo, d.lo));
        rem = __fadd_rn(r.hi, r.lo);
        out_hi = d.hi;
        out_lo = d.lo;
    }
    return true;
}

template <Rule R>
struct RouteF32 {
    const uint8_t* upmask;
    const float* a;   // inflow
    float as;
    const float* b;   // threshold / fraction
    float bs;
    float* out;       // outflow / flux
    float* rem;       // state (threshold, fraction)
    float* lo;        // residual of out
    int64_t cols;

    __device__ void no_data(int64_t c)
    {
        out[c] = qnan<float>();
        lo[c] = 0.0f;
        if (R != Rule::accu) rem[c] = qnan<float>();
    }

    __device__ void enter(int64_t c)
    {
        unsigned m = __ldg(upmask + c);
        FF t{0.0f, 0.0f};
        bool nan = false;
        while (m) {
            int k = __ffs(m) - 1;
            m &= m - 1;
            int64_t u = c + nb_dr(k) * cols + nb_dc(k);
            float h = load_cg(out + u);
            if (isnan(h)) nan = true;
            else t.add(h, load_cg(lo + u));
        }
        float oh = 0.0f, ol = 0.0f, r = 0.0f;
        if (!rule_f32<R>(t, nan, value_at(a, as, c), R == Rule::accu ? 0.0f : value_at(b, bs, c), oh, ol, r)) {
            no_data(c);
            return;
        }
        out[c] = oh;
        lo[c] = ol;
        if (R != Rule::accu) rem[c] = r;
    }
};

// --- float64: plain double arithmetic, like the reference's double instantiation ---------------------

// The float64 cell rule on the upstream sum t: outflow and state.  False: the cell is no-data.
template <Rule R>
__device__ __forceinline__ bool rule_f64(double t, bool nan, double x, double b, double& out, double& rem)
{
    if (R == Rule::accu) {
        if (nan || isnan(x) || !(x >= 0.0)) return false;
        out = t + x;
    } else if (R == Rule::threshold) {
        const double th = b;
        if (nan || isnan(x) || isnan(th) || !(x >= 0.0 && th >= 0.0)) return false;
        t += x;
        if (t > th) {
            rem = th;
            out = t - th;
        } else {
            rem = t;
            out = 0.0;
        }
    } else if (R == Rule::capacity) {
        const double cap = b;
        if (nan || isnan(x) || isnan(cap) || !(x >= 0.0 && cap >= 0.0)) return false;
        t += x;
        rem = 0.0;
        if (t > cap) {
            rem = t - cap;
            t = cap;
        }
        out = t;
    } else if (R == Rule::trigger) {
        const double trig = b;
        if (nan || isnan(x) || isnan(trig) || !(x >= 0.0 && trig >= 0.0)) return false;
        t += x;
        rem = 0.0;
        if (t < trig) {
            rem = t;
            t = 0.0;
        }
        out = t;
    } else {
        const double f = b;
        if (nan || isnan(x) || isnan(f) || !(x >= 0.0 && f >= 0.0 && f <= 1.0)) return false;
        t += x;
        const double d = f * t;
        rem = t - d;
        out = d;
    }
    return true;
}

template <Rule R>
struct RouteF64 {
    const uint8_t* upmask;
    const double* a;
    double as;
    const double* b;
    double bs;
    double* out;
    double* rem;
    int64_t cols;

    __device__ void no_data(int64_t c)
    {
        out[c] = qnan<double>();
        if (R != Rule::accu) rem[c] = qnan<double>();
    }

    __device__ void enter(int64_t c)
    {
        unsigned m = __ldg(upmask + c);
        double t = 0.0;
        bool nan = false;
        while (m) {
            int k = __ffs(m) - 1;
            m &= m - 1;
            double h = load_cg(out + c + nb_dr(k) * cols + nb_dc(k));
            if (isnan(h)) nan = true;
            else t += h;
        }
        double o = 0.0, r = 0.0;
        if (!rule_f64<R>(t, nan, value_at(a, as, c), R == Rule::accu ? 0.0 : value_at(b, bs, c), o, r))
            return no_data(c);
        out[c] = o;
        if (R != Rule::accu) rem[c] = r;
    }
};

// --- kinematic wave (float64 discharge; lateral inflow and alpha as TIn) ------------------------------

// The kinematic-wave cell rule (kinematic_wave.hpp:416-456): NaN outside the domain, else the new
// discharge from the upstream sum.
__device__ __forceinline__ double rule_kw(double up, bool nan, double qc, double q, double al, double be, double dt,
                                          double len, BetaRational br)
{
    if (nan || isnan(qc) || isnan(q) || isnan(al) || isnan(be) || isnan(dt) || isnan(len) ||
        !(qc >= 0.0 && q >= 0.0 && len > 0.0))
        return qnan<double>();
    return br.m ? iterate_to_new_discharge_fast(up, qc, q, al, be, br, dt, len)
                : iterate_to_new_discharge(up, qc, q, al, be, dt, len);
}

template <class TIn>
struct RouteKW {
    const uint8_t* upmask;
    const double* qcur;
    double qcur_s;
    const TIn* lateral;
    double lateral_s;
    const TIn* alpha;
    double alpha_s;
    const double* beta;
    double beta_s;
    double dt;
    const double* dx;
    double dx_s;
    double* out;
    int64_t cols;
    BetaRational br;  // scalar beta as p/m: the fast solve; m == 0: the reference-faithful solve

    __device__ void no_data(int64_t c) { out[c] = qnan<double>(); }

    __device__ void enter(int64_t c)
    {
        unsigned m = __ldg(upmask + c);
        double up = 0.0;
        bool nan = false;
        while (m) {
            int k = __ffs(m) - 1;
            m &= m - 1;
            double h = load_cg(out + c + nb_dr(k) * cols + nb_dc(k));
            if (isnan(h)) nan = true;
            else up += h;
        }
        double qc = qcur ? __ldg(qcur + c) : qcur_s;
        double q = lateral ? (double)__ldg(lateral + c) : lateral_s;
        double al = alpha ? (double)__ldg(alpha + c) : alpha_s;
        double be = beta ? __ldg(beta + c) : beta_s;
        double len = dx ? __ldg(dx + c) : dx_s;
        out[c] = rule_kw(up, nan, qc, q, al, be, dt, len, br);
    }
};

// Cells never entered (on or below a cycle): sum of the outflow of entered upstream cells.
template <class T>
__global__ void __launch_bounds__(256)
    k_cycle_cells(const uint8_t* fd, const uint8_t* upmask, const uint32_t* work, int64_t n, int64_t cols, T* out,
                  T* rem, float* lo)
{
    for (int64_t c = grid_stride_begin(); c < n; c += grid_stride()) {
        if (fd[c] == kNoData) continue;
        if (((work[c >> 2] >> ((c & 3) * 8)) & 0xFFu) == 0u) continue;  // entered
        unsigned m = upmask[c];
        T s = 0;
        bool nan = false;
        while (m) {
            int k = __ffs(m) - 1;
            m &= m - 1;
            int64_t u = c + nb_dr(k) * cols + nb_dc(k);
            if (((work[u >> 2] >> ((u & 3) * 8)) & 0xFFu) != 0u) continue;  // not entered: pushed nothing
            T h = out[u];
            if (isnan(h)) nan = true;
            else s += h;
        }
        out[c] = nan ? qnan<T>() : s;
        if (rem) rem[c] = nan ? qnan<T>() : T(0);
        if (lo) lo[c] = 0.0f;
    }
}

// --- kinematic wave, float instantiation (every raster float32) --------------------------------------

// The cell rule of kinematic_wave.hpp:416-456 with F = float: NaN outside the domain, else the new
// discharge from the float sum of the upstream discharges (fixed neighbour order).
__device__ __forceinline__ float rule_kw32(float up, bool nan, float qc, float q, float al, float be, float dt,
                                           float len)
{
    if (nan || isnan(qc) || isnan(q) || isnan(al) || isnan(be) || isnan(dt) || isnan(len) ||
        !(qc >= 0.0f && q >= 0.0f && len > 0.0f))
        return qnan<float>();
    return iterate_to_new_discharge_f32(up, qc, q, al, be, dt, len);
}

struct RouteKW32 {
    const uint8_t* upmask;
    const float* qcur;
    float qcur_s;
    const float* lateral;
    float lateral_s;
    const float* alpha;
    float alpha_s;
    const float* beta;
    float beta_s;
    float dt;
    const float* dx;
    float dx_s;
    float* out;
    int64_t cols;

    __device__ void no_data(int64_t c) { out[c] = qnan<float>(); }

    __device__ void enter(int64_t c)
    {
        unsigned m = __ldg(upmask + c);
        float up = 0.0f;
        bool nan = false;
        while (m) {
            const int k = __ffs(m) - 1;
            m &= m - 1;
            const float h = load_cg(out + c + nb_dr(k) * cols + nb_dc(k));
            if (isnan(h)) nan = true;
            else up += h;
        }
        out[c] = rule_kw32(up, nan, qcur ? __ldg(qcur + c) : qcur_s, lateral ? __ldg(lateral + c) : lateral_s,
                           alpha ? __ldg(alpha + c) : alpha_s, beta ? __ldg(beta + c) : beta_s, dt,
                           dx ? __ldg(dx + c) : dx_s);
    }
};

}  // namespace lue_gb300
