/*
 * lue_oracle.c — CPU restatement of LUE's flow-routing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA path is checked against: only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.  The product library
 * (liblue_gb300.so) never links, calls or falls back to it.
 *
 * Parity pinning: tests/test_oracle_golden.py runs every known-answer case extracted from the
 * reference's own unit tests (tests/golden/reference_cases.json) through this file.  The reference
 * itself cannot be built here (it needs HPX and Boost), so those vectors are the pin.
 *
 * What is restated (paths within computationalgeography/lue; ALG/ = source/framework/algorithm/
 * include/lue/framework/algorithm/):
 *
 *   - D8 decoding with the partition-exit flag ............ ALG/detail/flow_direction.hpp:11-112
 *   - per-partition inflow count + no-data marking ......... ALG/detail/inflow_count.hpp:9-351
 *   - partition input cells (+1 per cross-partition inflow)  ALG/definition/inflow_count.hpp:97-577
 *   - domain decomposition (last partition absorbs rest) .. source/framework/core/include/lue/
 *                                                            framework/core/domain_decomposition.hpp:90-175
 *   - the ridge-walk ("accumulate") ........................ ALG/definition/accumulating_router.hpp:525-599
 *   - intra-partition row-major ridge scan ................. ALG/definition/accumulating_router.hpp:866-882
 *   - inter-partition hand-off of (cell, outflow) .......... ALG/definition/accumulating_router.hpp:467-506,
 *                                                            602-645, 984-1010
 *   - cell functors: accu ................................. ALG/definition/accu.hpp:27-197
 *                    accu_threshold ....................... ALG/definition/accu_threshold.hpp:29-260
 *                    accu_fraction ........................ ALG/definition/accu_fraction.hpp:29-253
 *                    kinematic_wave ....................... ALG/definition/kinematic_wave.hpp:13-456
 *                    accu_capacity, accu_trigger .......... ALG/definition/accu_{capacity,trigger}.hpp
 *                                                            (enter_cell)
 *   - one-hop and local operations: upstream .............. ALG/definition/upstream.hpp:9-160
 *                                   downstream ............ ALG/definition/downstream.hpp:9-158
 *                                   downstream_distance ... ALG/definition/downstream_distance.hpp:9-75
 *   - value-policy domains ................................ ALG/value_policies/{accu,accu_threshold,
 *                                                            accu_fraction,kinematic_wave}.hpp:15-21
 *
 * Kinematic wave calls Boost.Math's newton_raphson_iterate (boost/math/tools/roots.hpp; Boost is
 * unpinned by the reference: Conan "boost/[1.74 || >1.75]", Conda libboost-devel).  Boost is not in
 * the reference tree; lue_oracle_newton_raphson() below restates its documented contract (Newton
 * steps; a step that leaves the bracket is replaced by bisection towards the violated bound; stop when
 * the last step is below |x| * 2^(1 - digits), when f(x) == 0, or after max_iter evaluations).
 *
 * The inter-partition arrival order in the reference is whatever order HPX channels deliver; here it
 * is a FIFO (single-threaded) or per-partition mailboxes drained by worker threads (threaded mode).
 * Float results therefore agree with the reference up to summation order.
 */
#include <math.h>
#include <float.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define U8_NO_DATA 255u

/* ------------------------------------------------------------------------------------------------ */
/* D8                                                                                                */
/* ------------------------------------------------------------------------------------------------ */

/* Keypad codes (ALG/flow_direction.hpp:7-35): 7 8 9 / 4 5 6 / 1 2 3; any other code is a sink. */
static inline void d8_offset(uint8_t code, int* dr, int* dc)
{
    switch (code) {
        case 7: *dr = -1; *dc = -1; return;
        case 8: *dr = -1; *dc = 0; return;
        case 9: *dr = -1; *dc = 1; return;
        case 4: *dr = 0; *dc = -1; return;
        case 6: *dr = 0; *dc = 1; return;
        case 1: *dr = 1; *dc = -1; return;
        case 2: *dr = 1; *dc = 0; return;
        case 3: *dr = 1; *dc = 1; return;
        default: *dr = 0; *dc = 0; return;
    }
}

/* ------------------------------------------------------------------------------------------------ */
/* Partitioning                                                                                      */
/* ------------------------------------------------------------------------------------------------ */

typedef struct {
    int64_t rows, cols;      /* array */
    int64_t nprow, npcol;    /* partition grid */
    int64_t prow, pcol;      /* nominal partition extent */
} Grid;

static int grid_init(Grid* g, int64_t rows, int64_t cols, int64_t prow, int64_t pcol)
{
    if (rows <= 0 || cols <= 0 || prow <= 0 || pcol <= 0 || prow > rows || pcol > cols) return -1;
    g->rows = rows; g->cols = cols; g->prow = prow; g->pcol = pcol;
    g->nprow = rows / prow; g->npcol = cols / pcol;
    return 0;
}

/* Row range [r0, r1) of partition row pr: the last partition absorbs the remainder. */
static inline void part_rows(const Grid* g, int64_t pr, int64_t* r0, int64_t* r1)
{
    *r0 = pr * g->prow;
    *r1 = (pr == g->nprow - 1) ? g->rows : *r0 + g->prow;
}
static inline void part_cols(const Grid* g, int64_t pc, int64_t* c0, int64_t* c1)
{
    *c0 = pc * g->pcol;
    *c1 = (pc == g->npcol - 1) ? g->cols : *c0 + g->pcol;
}
static inline int64_t part_of_row(const Grid* g, int64_t r)
{
    int64_t p = r / g->prow;
    return p >= g->nprow ? g->nprow - 1 : p;
}
static inline int64_t part_of_col(const Grid* g, int64_t c)
{
    int64_t p = c / g->pcol;
    return p >= g->npcol ? g->npcol - 1 : p;
}

/* ------------------------------------------------------------------------------------------------ */
/* Inflow count                                                                                      */
/* ------------------------------------------------------------------------------------------------ */

/*
 * Router-internal counts (int8 in the reference, no-data -128): per partition, count upstream
 * neighbours inside the partition (ALG/detail/inflow_count.hpp:9-351), then add one per partition
 * input cell arrival from a neighbouring partition (ALG/definition/inflow_count.hpp:558-574).
 * A cell whose flow leaves the array contributes nothing (no neighbour partition, no message).
 */
static void router_counts(const Grid* g, const uint8_t* fd, int value_policies, int8_t* cnt)
{
    const int64_t cols = g->cols;
    memset(cnt, 0, (size_t)(g->rows * cols));
    for (int64_t pr = 0; pr < g->nprow; ++pr) {
        int64_t r0, r1;
        part_rows(g, pr, &r0, &r1);
        for (int64_t pc = 0; pc < g->npcol; ++pc) {
            int64_t c0, c1;
            part_cols(g, pc, &c0, &c1);
            for (int64_t r = r0; r < r1; ++r) {
                for (int64_t c = c0; c < c1; ++c) {
                    uint8_t code = fd[r * cols + c];
                    if (value_policies && code == U8_NO_DATA) {
                        cnt[r * cols + c] = INT8_MIN;
                        continue;
                    }
                    int dr, dc;
                    d8_offset(code, &dr, &dc);
                    if (dr == 0 && dc == 0) continue;
                    int64_t rd = r + dr, cd = c + dc;
                    if (rd >= r0 && rd < r1 && cd >= c0 && cd < c1) cnt[rd * cols + cd] += 1;
                }
            }
        }
    }
    /* partition input cells: flow that crosses a partition boundary but stays in the array */
    for (int64_t r = 0; r < g->rows; ++r) {
        for (int64_t c = 0; c < cols; ++c) {
            uint8_t code = fd[r * cols + c];
            if (value_policies && code == U8_NO_DATA) continue;
            int dr, dc;
            d8_offset(code, &dr, &dc);
            if (dr == 0 && dc == 0) continue;
            int64_t rd = r + dr, cd = c + dc;
            if (rd < 0 || rd >= g->rows || cd < 0 || cd >= cols) continue;
            if (part_of_row(g, rd) != part_of_row(g, r) || part_of_col(g, cd) != part_of_col(g, c))
                cnt[rd * cols + cd] += 1;
        }
    }
}

/*
 * Public inflow_count<uint8> (ALG/definition/inflow_count.hpp:665-726).  With value policies
 * (DefaultValuePolicies) a no-data flow direction gives count 255; with DefaultPolicies the value 255
 * is just an unknown code, i.e. a sink.
 */
int lue_oracle_inflow_count(const uint8_t* fd, int64_t rows, int64_t cols, int64_t prow, int64_t pcol,
                            int value_policies, uint8_t* out)
{
    Grid g;
    if (grid_init(&g, rows, cols, prow, pcol)) return -1;
    int8_t* cnt = (int8_t*)malloc((size_t)(rows * cols));
    if (!cnt) return -2;
    router_counts(&g, fd, value_policies, cnt);
    for (int64_t i = 0; i < rows * cols; ++i)
        out[i] = (cnt[i] == INT8_MIN && value_policies && fd[i] == U8_NO_DATA) ? U8_NO_DATA : (uint8_t)cnt[i];
    free(cnt);
    return 0;
}

/* ------------------------------------------------------------------------------------------------ */
/* Newton-Raphson (restated contract of boost::math::tools::newton_raphson_iterate)                 */
/* ------------------------------------------------------------------------------------------------ */

typedef struct {
    double k;             /* time_step_duration / channel_length */
    double alpha, beta, alpha_beta;
    double known;         /* k * Qup + alpha * Qcur^beta + dt * q */
} KwSolve;

static inline void kw_eval(const KwSolve* s, double q, double* f, double* df)
{
    double qb1 = pow(q, s->beta - 1.0);
    *f = s->k * q + s->alpha * pow(q, s->beta) - s->known;
    *df = s->k + s->alpha_beta * qb1;
}

/*
 * Newton iteration on [lo, hi] with the documented stopping rule.  Returns the last iterate; *iters
 * receives the number of function evaluations used.
 */
double lue_oracle_newton_raphson_kw(double k, double alpha, double beta, double known, double guess,
                                    double lo, double hi, int digits, int max_iter, int* iters)
{
    KwSolve s = {k, alpha, beta, alpha * beta, known};
    double factor = ldexp(1.0, 1 - digits);
    double x = guess;
    int n = 0;
    while (n < max_iter) {
        double f, df;
        kw_eval(&s, x, &f, &df);
        ++n;
        if (f == 0.0) break;
        double step;
        if (df == 0.0 || !isfinite(df)) {
            /* no usable slope: bisect towards the bound on the side the residual points to */
            step = f > 0.0 ? 0.5 * (x - lo) : 0.5 * (x - hi);
        } else {
            step = f / df;
        }
        double next = x - step;
        if (next <= lo) {
            step = 0.5 * (x - lo);
            next = x - step;
        } else if (next >= hi) {
            step = 0.5 * (x - hi);
            next = x - step;
        }
        /* shrink the bracket: the root lies on the side the step points to */
        if (step > 0.0) hi = x; else lo = x;
        x = next;
        if (fabs(step) <= fabs(x) * factor) break;
        if (x == lo || x == hi) break;
    }
    if (iters) *iters = n;
    return x;
}

/* iterate_to_new_discharge (ALG/definition/kinematic_wave.hpp:145-254), F = double. */
double lue_oracle_iterate_to_new_discharge_f64(double upstream, double current, double lateral,
                                               double alpha, double beta, double dt, double dx)
{
    double new_q = 0.0;
    if (upstream + current > 0.0 || lateral > 0.0) {
        double inflow = lateral >= 0.0 ? lateral : 0.0;
        double k = dt / dx;
        double known = k * upstream + alpha * pow(current, beta) + dt * inflow;
        /* guess (kinematic_wave.hpp:61-91) */
        double guess = DBL_MIN;
        if (current + upstream != 0.0 || beta >= 1.0) {
            double a_b_pq = alpha * beta * pow((current + upstream) / 2.0, beta - 1.0);
            guess = (k * upstream + a_b_pq * current + dt * inflow) / (k + a_b_pq);
            if (!(guess > DBL_MIN)) guess = DBL_MIN;
        }
        int digits = (int)(DBL_MANT_DIG * 0.6);
        new_q = lue_oracle_newton_raphson_kw(k, alpha, beta, known, guess, 0.0, DBL_MAX, digits, 10, NULL);
    }
    if (lateral < 0.0) {
        double extraction = fmin(dx * fabs(lateral), new_q);
        new_q -= extraction;
    }
    return new_q;
}

/* Same in float: digits = int(24 * 0.6) = 14, bracket [0, FLT_MAX], float arithmetic. */
static double newton_f32(float k, float alpha, float beta, float known, float guess, int* iters)
{
    float factor = ldexpf(1.0f, 1 - (int)(FLT_MANT_DIG * 0.6));
    float lo = 0.0f, hi = FLT_MAX, x = guess, ab = alpha * beta;
    int n = 0;
    while (n < 10) {
        float f = k * x + alpha * powf(x, beta) - known;
        float df = k + ab * powf(x, beta - 1.0f);
        ++n;
        if (f == 0.0f) break;
        float step = (df == 0.0f || !isfinite(df)) ? (f > 0.0f ? 0.5f * (x - lo) : 0.5f * (x - hi)) : f / df;
        float next = x - step;
        if (next <= lo) { step = 0.5f * (x - lo); next = x - step; }
        else if (next >= hi) { step = 0.5f * (x - hi); next = x - step; }
        if (step > 0.0f) hi = x; else lo = x;
        x = next;
        if (fabsf(step) <= fabsf(x) * factor) break;
        if (x == lo || x == hi) break;
    }
    if (iters) *iters = n;
    return x;
}

float lue_oracle_iterate_to_new_discharge_f32(float upstream, float current, float lateral, float alpha,
                                              float beta, float dt, float dx)
{
    float new_q = 0.0f;
    if (upstream + current > 0.0f || lateral > 0.0f) {
        float inflow = lateral >= 0.0f ? lateral : 0.0f;
        float k = dt / dx;
        float known = k * upstream + alpha * powf(current, beta) + dt * inflow;
        float guess = FLT_MIN;
        if (current + upstream != 0.0f || beta >= 1.0f) {
            float a_b_pq = alpha * beta * powf((current + upstream) / 2.0f, beta - 1.0f);
            guess = (k * upstream + a_b_pq * current + dt * inflow) / (k + a_b_pq);
            if (!(guess > FLT_MIN)) guess = FLT_MIN;
        }
        new_q = (float)newton_f32(k, alpha, beta, known, guess, NULL);
    }
    if (lateral < 0.0f) {
        float extraction = fminf(dx * fabsf(lateral), new_q);
        new_q -= extraction;
    }
    return new_q;
}

/* ------------------------------------------------------------------------------------------------ */
/* The accumulating router, instantiated for float and double                                       */
/* ------------------------------------------------------------------------------------------------ */

enum { OP_ACCU = 0, OP_THRESHOLD = 1, OP_FRACTION = 2, OP_KINEMATIC_WAVE = 3, OP_CAPACITY = 4, OP_TRIGGER = 5 };

#define REAL float
#define SFX f32
#define REAL_MIN FLT_MIN
#define ITERATE lue_oracle_iterate_to_new_discharge_f32
#include "router_impl.h"
#undef REAL
#undef SFX
#undef REAL_MIN
#undef ITERATE

#define REAL double
#define SFX f64
#define REAL_MIN DBL_MIN
#define ITERATE lue_oracle_iterate_to_new_discharge_f64
#include "router_impl.h"
#undef REAL
#undef SFX
#undef REAL_MIN
#undef ITERATE

/* Symbols the Python wrapper checks for, so a stale build is caught early. */
int lue_oracle_abi_version(void) { return 1; }

/*
 * Downstream level of every cell (no reference counterpart; the CPU definition the GPU's
 * downstream ordering is pinned to): 0 for a valid cell without inflow, else 1 + the largest level
 * among the cells draining into it; -1 for no-data cells and for cells on or below a cycle.
 * Kahn's peel over the whole array (flow off the array ends a path).
 */
int lue_oracle_downstream_level(const uint8_t* fd, int64_t rows, int64_t cols, int32_t* level)
{
    int64_t n = rows * cols;
    uint8_t* cnt = (uint8_t*)calloc((size_t)n, 1);
    int64_t* queue = (int64_t*)malloc((size_t)n * sizeof(int64_t));
    if (!cnt || !queue) { free(cnt); free(queue); return -2; }
    for (int64_t i = 0; i < n; ++i) level[i] = -1;
    for (int64_t r = 0; r < rows; ++r)
        for (int64_t c = 0; c < cols; ++c) {
            uint8_t code = fd[r * cols + c];
            if (code == U8_NO_DATA) continue;
            int dr, dc;
            d8_offset(code, &dr, &dc);
            if (dr == 0 && dc == 0) continue;
            int64_t rd = r + dr, cd = c + dc;
            if (rd < 0 || rd >= rows || cd < 0 || cd >= cols) continue;
            cnt[rd * cols + cd]++;
        }
    int64_t head = 0, tail = 0;
    for (int64_t i = 0; i < n; ++i)
        if (fd[i] != U8_NO_DATA && cnt[i] == 0) { queue[tail++] = i; level[i] = 0; }
    while (head < tail) {
        int64_t i = queue[head++];
        int dr, dc;
        d8_offset(fd[i], &dr, &dc);
        if (dr == 0 && dc == 0) continue;
        int64_t rd = i / cols + dr, cd = i % cols + dc;
        if (rd < 0 || rd >= rows || cd < 0 || cd >= cols) continue;
        int64_t j = rd * cols + cd;
        if (fd[j] == U8_NO_DATA) continue;
        if (level[i] + 1 > level[j]) level[j] = level[i] + 1;
        if (--cnt[j] == 0) queue[tail++] = j;
    }
    /* cells left with a positive count were never peeled: on or below a cycle */
    for (int64_t i = 0; i < n; ++i)
        if (fd[i] != U8_NO_DATA && cnt[i] != 0) level[i] = -1;
    free(cnt);
    free(queue);
    return 0;
}

/*
 * value_policies::d8_flow_direction (ALG/definition/d8_flow_direction.hpp:45-147,
 * ALG/value_policies/d8_flow_direction.hpp:20-45): steepest unweighted drop, candidates N, W, E, S,
 * NW, NE, SW, SE with strict '>', sink (5) without a positive drop, 255 for a NaN elevation, NaN
 * neighbours skipped, DBL_MIN (std::numeric_limits<double>::min()) outside the array.
 */
int lue_oracle_d8_flow_direction(const double* z, int64_t rows, int64_t cols, uint8_t* fd)
{
    static const int dr[8] = {-1, 0, 0, 1, -1, -1, 1, 1};
    static const int dc[8] = {0, -1, 1, 0, -1, 1, -1, 1};
    static const uint8_t code[8] = {8, 4, 6, 2, 7, 9, 1, 3};
    for (int64_t r = 0; r < rows; ++r)
        for (int64_t c = 0; c < cols; ++c) {
            double zc = z[r * cols + c];
            if (isnan(zc)) { fd[r * cols + c] = U8_NO_DATA; continue; }
            uint8_t dir = 5;
            double drop = 0.0;
            for (int k = 0; k < 8; ++k) {
                int64_t rn = r + dr[k], cn = c + dc[k];
                double zn = (rn < 0 || rn >= rows || cn < 0 || cn >= cols) ? DBL_MIN : z[rn * cols + cn];
                if (isnan(zn)) continue;
                if (zc - zn > drop) { drop = zc - zn; dir = code[k]; }
            }
            fd[r * cols + c] = dir;
        }
    return 0;
}

/*
 * upstream (ALG/definition/upstream.hpp:9-160): the sum of the material of the neighbours draining into
 * each cell, in the order NW, N, NE, W, E, SW, S, SE; no-data where the cell's flow direction or its own
 * material is no-data, or where a contributing neighbour's material is no-data.  Outside the array the
 * flow-direction halo points away from the array (ALG/policy/flow_direction_halo.hpp), so nothing
 * enters from there.
 *
 * downstream (ALG/definition/downstream.hpp:9-158): the material of each cell's downstream cell; the
 * cell's own material for a sink (code 5, and any code that is not a direction); 0 where the flow
 * leaves the array (the material halo is filled with 0); no-data where the cell's flow direction or
 * material, or the downstream material, is no-data.
 */
#define NB_ORDER_DR(k) ((k) < 3 ? -1 : ((k) < 5 ? 0 : 1))
static const int NB_DC[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
static const uint8_t NB_INFLOW[8] = {3, 2, 1, 6, 4, 9, 8, 7};  /* code of a neighbour draining here */

#define ONE_HOP(T, SFX_)                                                                                  \
    int lue_oracle_upstream_##SFX_(const uint8_t* fd, int64_t rows, int64_t cols, const T* m, T* out)       \
    {                                                                                                     \
        for (int64_t r = 0; r < rows; ++r)                                                                \
            for (int64_t c = 0; c < cols; ++c) {                                                          \
                const int64_t i = r * cols + c;                                                           \
                if (fd[i] == U8_NO_DATA || isnan(m[i])) {                                                 \
                    out[i] = (T)NAN;                                                                      \
                    continue;                                                                             \
                }                                                                                         \
                T s = 0;                                                                                  \
                int nd = 0;                                                                               \
                for (int k = 0; k < 8 && !nd; ++k) {                                                      \
                    const int64_t rr = r + NB_ORDER_DR(k), cc = c + NB_DC[k];                             \
                    if (rr < 0 || rr >= rows || cc < 0 || cc >= cols) continue;                           \
                    const int64_t j = rr * cols + cc;                                                     \
                    if (fd[j] != NB_INFLOW[k]) continue;                                                  \
                    if (isnan(m[j])) nd = 1;                                                              \
                    else s += m[j];                                                                       \
                }                                                                                         \
                out[i] = nd ? (T)NAN : s;                                                                 \
            }                                                                                             \
        return 0;                                                                                         \
    }                                                                                                     \
    int lue_oracle_downstream_##SFX_(const uint8_t* fd, int64_t rows, int64_t cols, const T* m, T* out)     \
    {                                                                                                     \
        for (int64_t r = 0; r < rows; ++r)                                                                \
            for (int64_t c = 0; c < cols; ++c) {                                                          \
                const int64_t i = r * cols + c;                                                           \
                if (fd[i] == U8_NO_DATA || isnan(m[i])) {                                                 \
                    out[i] = (T)NAN;                                                                      \
                    continue;                                                                             \
                }                                                                                         \
                int dr, dc;                                                                               \
                d8_offset(fd[i], &dr, &dc);                                                               \
                if (dr == 0 && dc == 0) {                                                                 \
                    out[i] = m[i];                                                                        \
                    continue;                                                                             \
                }                                                                                         \
                const int64_t rr = r + dr, cc = c + dc;                                                   \
                if (rr < 0 || rr >= rows || cc < 0 || cc >= cols) {                                       \
                    out[i] = 0;                                                                           \
                    continue;                                                                             \
                }                                                                                         \
                out[i] = m[rr * cols + cc];                                                               \
            }                                                                                             \
        return 0;                                                                                         \
    }                                                                                                     \
    /* downstream_distance (ALG/definition/downstream_distance.hpp:9-75): the cell size for N, W, E, S,    \
       sqrt(2) * cell size for the diagonals, 0 otherwise; no-data (NaN) for a no-data flow direction. */  \
    int lue_oracle_downstream_distance_##SFX_(const uint8_t* fd, int64_t rows, int64_t cols, T cell_size,   \
                                              T* out)                                                     \
    {                                                                                                     \
        const T diag = (T)sqrt((double)2) * cell_size;                                                    \
        for (int64_t i = 0; i < rows * cols; ++i) {                                                       \
            const uint8_t code = fd[i];                                                                   \
            if (code == U8_NO_DATA) out[i] = (T)NAN;                                                      \
            else if (code == 7 || code == 9 || code == 1 || code == 3) out[i] = diag;                     \
            else if (code == 8 || code == 4 || code == 6 || code == 2) out[i] = cell_size;                \
            else out[i] = 0;                                                                              \
        }                                                                                                 \
        return 0;                                                                                         \
    }

ONE_HOP(float, f32)
ONE_HOP(double, f64)

/* ------------------------------------------------------------------------------------------------ */
/* accu_info                                                                                         */
/* ------------------------------------------------------------------------------------------------ */

/*
 * accu_info (ALG/definition/accu_info.hpp:13-190; classes ALG/accu_info.hpp:22-63): the class of every
 * cell after the router's own event sequence (ALG/definition/accumulating_router.hpp:525-599 walk,
 * :866-882 intra-partition ridge scan, :984-1010 inter-partition arrivals), with the AccuInfo cell
 * accumulator's hooks:
 *   enter_intra_partition_stream -> intra stream; leave_intra_partition_stream -> ridge;
 *   enter_inter_partition_stream -> inter stream; leave_inter_partition_stream -> partition input
 *   (partition input-output if the cell is a partition output cell);
 *   leave_cell copies the upstream class downstream (no-data wins); stop_at_sink -> sink;
 *   stop_at_confluence -> confluence; stop_at_partition_output -> partition output; no-data 255.
 * Result buffers start at 0.  Inter-partition arrivals are taken in FIFO order (one order HPX may
 * deliver); at a partition input cell that also waits for upstream cells of its own partition which wait
 * for other partitions, the class depends on that order.
 */
enum { CLS_RIDGE = 11, CLS_INTRA = 12, CLS_OUTPUT = 13, CLS_INPUT = 14, CLS_INPUT_OUTPUT = 15, CLS_INTER = 16,
       CLS_SINK = 17, CLS_CONFLUENCE = 18, CLS_NO_DATA = 255 };

typedef struct {
    Grid g;
    const uint8_t* fd;
    int8_t* cnt;
    uint8_t* cls;
    int64_t* fifo;
    int64_t fifo_size, fifo_cap;
} InfoRouter;

static void info_push(InfoRouter* R, int64_t j)
{
    if (R->fifo_size == R->fifo_cap) {
        R->fifo_cap = R->fifo_cap ? 2 * R->fifo_cap : 64;
        R->fifo = (int64_t*)realloc(R->fifo, (size_t)R->fifo_cap * sizeof(int64_t));
    }
    R->fifo[R->fifo_size++] = j;
}

static void info_walk(InfoRouter* R, int64_t r, int64_t c)
{
    const Grid* g = &R->g;
    const int64_t cols = g->cols;
    int64_t r0, r1, c0, c1;
    part_rows(g, part_of_row(g, r), &r0, &r1);
    part_cols(g, part_of_col(g, c), &c0, &c1);
    for (;;) {
        const int64_t i = r * cols + c;
        int dr, dc;
        d8_offset(R->fd[i], &dr, &dc);
        if (dr == 0 && dc == 0) {
            R->cls[i] = CLS_SINK;
            return;
        }
        const int64_t rd = r + dr, cd = c + dc;
        if (rd < r0 || rd >= r1 || cd < c0 || cd >= c1) {
            R->cls[i] = CLS_OUTPUT;
            if (rd >= 0 && rd < g->rows && cd >= 0 && cd < cols) info_push(R, rd * cols + cd);
            return;
        }
        const int64_t j = rd * cols + cd;
        if (R->cls[j] != CLS_NO_DATA) R->cls[j] = R->cls[i] == CLS_NO_DATA ? CLS_NO_DATA : R->cls[i];
        r = rd;
        c = cd;
        if (--R->cnt[j] > 0) {
            R->cls[j] = CLS_CONFLUENCE;
            return;
        }
    }
}

int lue_oracle_accu_info(const uint8_t* fd, int64_t rows, int64_t cols, int64_t prow, int64_t pcol, uint8_t* cls)
{
    InfoRouter R;
    memset(&R, 0, sizeof R);
    if (grid_init(&R.g, rows, cols, prow, pcol)) return -1;
    const int64_t n = rows * cols;
    R.fd = fd;
    R.cls = cls;
    R.cnt = (int8_t*)malloc((size_t)n);
    int8_t* orig = (int8_t*)malloc((size_t)n);
    if (!R.cnt || !orig) {
        free(R.cnt);
        free(orig);
        return -2;
    }
    router_counts(&R.g, fd, 1, orig);
    memcpy(R.cnt, orig, (size_t)n);
    memset(cls, 0, (size_t)n);
    for (int64_t pr = 0; pr < R.g.nprow; ++pr) {
        int64_t r0, r1;
        part_rows(&R.g, pr, &r0, &r1);
        for (int64_t pc = 0; pc < R.g.npcol; ++pc) {
            int64_t c0, c1;
            part_cols(&R.g, pc, &c0, &c1);
            for (int64_t r = r0; r < r1; ++r)
                for (int64_t c = c0; c < c1; ++c) {
                    const int64_t i = r * cols + c;
                    if (fd[i] == U8_NO_DATA) {
                        cls[i] = CLS_NO_DATA;
                    } else if (orig[i] == 0) {
                        cls[i] = CLS_INTRA;
                        info_walk(&R, r, c);
                        cls[i] = CLS_RIDGE;
                    }
                }
        }
    }
    for (int64_t k = 0; k < R.fifo_size; ++k) {
        const int64_t j = R.fifo[k];
        R.cls[j] = CLS_INTER;
        if (--R.cnt[j] == 0) {
            info_walk(&R, j / cols, j % cols);
            R.cls[j] = R.cls[j] != CLS_OUTPUT ? CLS_INPUT : CLS_INPUT_OUTPUT;
        }
    }
    free(R.fifo);
    free(R.cnt);
    free(orig);
    return 0;
}

/* ------------------------------------------------------------------------------------------------ */
/* partial_accu                                                                                      */
/* ------------------------------------------------------------------------------------------------ */

/*
 * partial_accu (ALG/definition/partial_accu.hpp:15-287, value policies ALG/value_policies/
 * partial_accu.hpp): the router's event sequence (ALG/definition/accumulating_router.hpp:525-599 walk,
 * :866-882 intra-partition ridge scan, :984-1010 inter-partition arrivals) with the PartialAccu cell
 * accumulator's hooks, in double (the values are small integers):
 *   enter_intra_partition_stream: the ridge's value is the partition's stream counter (:71-76);
 *   leave_intra_partition_stream: the counter goes up by one (:79-83);
 *   enter_inter_partition_stream: a value arriving from another partition: NaN wins, else the larger
 *     of the cell's value and the arriving one; above nr_steps the cell becomes NaN (:86-109);
 *   leave_inter_partition_stream: after the walk from a partition input cell its value goes up by one
 *     unless it is NaN (:112-120);
 *   leave_cell: the downstream cell takes the upstream value (it is not added), NaN wins; above
 *     nr_steps the downstream cell becomes NaN (:129-165).
 * Result buffers start at 0; a no-data flow direction gives NaN; nr_steps below 0 counts as 0.
 * Inter-partition arrivals: order 0 takes them in one FIFO (one order HPX may deliver); order 1 takes
 * the mail of the highest-numbered partition that has mail first (FIFO within a partition's mail),
 * another valid order, used to find the cells whose value depends on the order.
 */
typedef struct {
    int64_t idx;
    double value;
    int64_t part;
} PartialMsg;

typedef struct {
    Grid g;
    const uint8_t* fd;
    int8_t* cnt;
    double* out;
    double nr_steps;
    PartialMsg* msg;
    int64_t nmsg, cap;
} PartialRouter;

static void partial_push(PartialRouter* R, int64_t j, double v)
{
    if (R->nmsg == R->cap) {
        R->cap = R->cap ? 2 * R->cap : 64;
        R->msg = (PartialMsg*)realloc(R->msg, (size_t)R->cap * sizeof(PartialMsg));
    }
    const int64_t r = j / R->g.cols, c = j % R->g.cols;
    R->msg[R->nmsg].idx = j;
    R->msg[R->nmsg].value = v;
    R->msg[R->nmsg].part = part_of_row(&R->g, r) * R->g.npcol + part_of_col(&R->g, c);
    R->nmsg++;
}

static void partial_walk(PartialRouter* R, int64_t r, int64_t c)
{
    const Grid* g = &R->g;
    const int64_t cols = g->cols;
    int64_t r0, r1, c0, c1;
    part_rows(g, part_of_row(g, r), &r0, &r1);
    part_cols(g, part_of_col(g, c), &c0, &c1);
    for (;;) {
        const int64_t i = r * cols + c;
        int dr, dc;
        d8_offset(R->fd[i], &dr, &dc);
        if (dr == 0 && dc == 0) return; /* sink */
        const int64_t rd = r + dr, cd = c + dc;
        if (rd < r0 || rd >= r1 || cd < c0 || cd >= c1) {
            if (rd >= 0 && rd < g->rows && cd >= 0 && cd < cols) partial_push(R, rd * cols + cd, R->out[i]);
            return; /* partition output cell */
        }
        const int64_t j = rd * cols + cd;
        if (!isnan(R->out[j])) R->out[j] = isnan(R->out[i]) ? (double)NAN : R->out[i]; /* leave_cell */
        if (R->out[j] > R->nr_steps) R->out[j] = (double)NAN;
        r = rd;
        c = cd;
        if (--R->cnt[j] > 0) return; /* confluence */
    }
}

static void partial_arrive(PartialRouter* R, int64_t j, double v)
{
    double* o = &R->out[j];
    if (!isnan(*o)) { /* enter_inter_partition_stream */
        if (isnan(v)) *o = (double)NAN;
        else *o = *o > v ? *o : v;
        if (*o > R->nr_steps) *o = (double)NAN;
    }
    if (--R->cnt[j] == 0) {
        partial_walk(R, j / R->g.cols, j % R->g.cols);
        if (!isnan(*o)) *o += 1.0; /* leave_inter_partition_stream */
    }
}

int lue_oracle_partial_accu(const uint8_t* fd, int64_t rows, int64_t cols, int64_t prow, int64_t pcol,
                            int64_t nr_steps, int order, double* out)
{
    PartialRouter R;
    memset(&R, 0, sizeof R);
    if (grid_init(&R.g, rows, cols, prow, pcol)) return -1;
    const int64_t n = rows * cols;
    R.fd = fd;
    R.out = out;
    R.nr_steps = (double)(nr_steps > 0 ? nr_steps : 0);
    R.cnt = (int8_t*)malloc((size_t)n);
    int8_t* orig = (int8_t*)malloc((size_t)n);
    if (!R.cnt || !orig) {
        free(R.cnt);
        free(orig);
        return -2;
    }
    router_counts(&R.g, fd, 1, orig);
    memcpy(R.cnt, orig, (size_t)n);
    for (int64_t i = 0; i < n; ++i) out[i] = 0.0;
    for (int64_t pr = 0; pr < R.g.nprow; ++pr) {
        int64_t r0, r1;
        part_rows(&R.g, pr, &r0, &r1);
        for (int64_t pc = 0; pc < R.g.npcol; ++pc) {
            int64_t c0, c1;
            part_cols(&R.g, pc, &c0, &c1);
            double step = 0.0; /* one cell accumulator, and so one counter, per partition */
            for (int64_t r = r0; r < r1; ++r)
                for (int64_t c = c0; c < c1; ++c) {
                    const int64_t i = r * cols + c;
                    if (fd[i] == U8_NO_DATA) {
                        out[i] = (double)NAN;
                    } else if (orig[i] == 0) {
                        out[i] = step;
                        partial_walk(&R, r, c);
                        step += 1.0;
                    }
                }
        }
    }
    if (order == 0) {
        for (int64_t k = 0; k < R.nmsg; ++k) partial_arrive(&R, R.msg[k].idx, R.msg[k].value);
    } else {
        /* the mail of the highest-numbered partition with mail first; done[] marks delivered messages */
        uint8_t* done = NULL;
        int64_t delivered = 0;
        for (;;) {
            done = (uint8_t*)realloc(done, (size_t)(R.nmsg > 0 ? R.nmsg : 1));
            for (int64_t k = delivered; k < R.nmsg; ++k) done[k] = 0;
            delivered = R.nmsg;
            int64_t best = -1;
            for (int64_t k = 0; k < R.nmsg; ++k)
                if (!done[k] && (best < 0 || R.msg[k].part > R.msg[best].part)) best = k;
            if (best < 0) break;
            const int64_t p = R.msg[best].part;
            for (int64_t k = 0; k < R.nmsg; ++k) {
                if (done[k] || R.msg[k].part != p) continue;
                done[k] = 1;
                const int64_t nbefore = R.nmsg;
                partial_arrive(&R, R.msg[k].idx, R.msg[k].value);
                if (R.nmsg != nbefore) {
                    done = (uint8_t*)realloc(done, (size_t)R.nmsg);
                    for (int64_t q = nbefore; q < R.nmsg; ++q) done[q] = 0;
                    delivered = R.nmsg;
                }
            }
        }
        free(done);
    }
    free(R.msg);
    free(R.cnt);
    free(orig);
    return 0;
}
