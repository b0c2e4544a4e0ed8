/*
 * synthetic.c — seeded synthetic terrain for the flow-routing workloads (host code, C).
 *
 * Steps, all deterministic for a given seed on x86-64 and aarch64 (compile with -ffp-contract=off):
 *
 *   1. DEM: fractal Brownian motion of 2-D gradient noise (Perlin's improved-noise construction:
 *      hashed unit gradients at lattice points, quintic fade 6t^5-15t^4+10t^3), octaves at halving
 *      wavelength and halving amplitude, scaled so that the summed amplitude is `amplitude` metres,
 *      on a plane that drops `tilt` (e.g. 0.01 = 1 %) per metre towards the south edge (row index
 *      increasing), plus a constant offset that keeps every elevation positive.
 *   2. Depression filling: Priority-Flood+epsilon (Barnes, Lehman & Mulla 2014, Computers &
 *      Geosciences 62:117-127).  Edge cells seed a min-heap; a neighbour that is not higher than the
 *      cell being processed is raised to the next representable double above it and goes to a FIFO
 *      ("pit" queue) that is drained before the heap.  Afterwards every interior cell has a strictly
 *      lower neighbour.
 *   3. D8: the reference's steepest-descent rule (ALG/definition/d8_flow_direction.hpp:45-147 in
 *      computationalgeography/lue): unweighted drop, strict '>', candidates N, W, E, S, NW, NE, SW, SE,
 *      and outside the array the halo value std::numeric_limits<double>::min()
 *      (ALG/value_policies/d8_flow_direction.hpp:31-37), so edge cells drain off the array.
 *   4. Validation helpers: Kahn peel to find cells on or below cycles, interior sinks, and the
 *      longest flow path (in cells).
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static inline uint64_t splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

/* 16 unit gradient directions, angles k * 22.5 degrees (exact table, no libm at run time). */
static const double GX[16] = {1.0, 0.9238795325112867, 0.7071067811865476, 0.3826834323650898,
                              0.0, -0.3826834323650898, -0.7071067811865476, -0.9238795325112867,
                              -1.0, -0.9238795325112867, -0.7071067811865476, -0.3826834323650898,
                              0.0, 0.3826834323650898, 0.7071067811865476, 0.9238795325112867};
static const double GY[16] = {0.0, 0.3826834323650898, 0.7071067811865476, 0.9238795325112867,
                              1.0, 0.9238795325112867, 0.7071067811865476, 0.3826834323650898,
                              0.0, -0.3826834323650898, -0.7071067811865476, -0.9238795325112867,
                              -1.0, -0.9238795325112867, -0.7071067811865476, -0.3826834323650898};

static inline double grad_dot(uint64_t seed, int64_t ix, int64_t iy, double dx, double dy)
{
    uint64_t h = splitmix64(seed ^ splitmix64((uint64_t)ix * 0x632BE59BD9B4E019ull + (uint64_t)iy));
    int k = (int)(h & 15u);
    return GX[k] * dx + GY[k] * dy;
}

static inline double fade(double t) { return t * t * t * (t * (t * 6.0 - 15.0) + 10.0); }

static double gradient_noise(uint64_t seed, double x, double y)
{
    double fx = floor(x), fy = floor(y);
    int64_t ix = (int64_t)fx, iy = (int64_t)fy;
    double dx = x - fx, dy = y - fy;
    double n00 = grad_dot(seed, ix, iy, dx, dy);
    double n10 = grad_dot(seed, ix + 1, iy, dx - 1.0, dy);
    double n01 = grad_dot(seed, ix, iy + 1, dx, dy - 1.0);
    double n11 = grad_dot(seed, ix + 1, iy + 1, dx - 1.0, dy - 1.0);
    double u = fade(dx), v = fade(dy);
    double a = n00 + u * (n10 - n00);
    double b = n01 + u * (n11 - n01);
    return a + v * (b - a); /* roughly in [-0.7, 0.7] */
}

typedef struct {
    int64_t rows, cols, r0, r1;
    uint64_t seed;
    double amplitude, cell_size, tilt, wavelength;
    int octaves;
    double* z;
} DemJob;

static void* dem_rows(void* arg)
{
    DemJob* j = (DemJob*)arg;
    double norm = 0.0, a = 1.0;
    for (int o = 0; o < j->octaves; ++o) { norm += a; a *= 0.5; }
    double offset = j->amplitude + 1.0;
    for (int64_t r = j->r0; r < j->r1; ++r) {
        double base = (double)(j->rows - 1 - r) * j->cell_size * j->tilt + offset;
        for (int64_t c = 0; c < j->cols; ++c) {
            double sum = 0.0, amp = 1.0, lam = j->wavelength;
            for (int o = 0; o < j->octaves; ++o) {
                sum += amp * gradient_noise(j->seed + (uint64_t)o * 0x9E3779B97F4A7C15ull, (double)c / lam,
                                            (double)r / lam);
                amp *= 0.5;
                lam *= 0.5;
            }
            j->z[r * j->cols + c] = base + j->amplitude * (sum / norm);
        }
    }
    return NULL;
}

int lue_synth_dem(int64_t rows, int64_t cols, uint64_t seed, double amplitude, double cell_size, double tilt,
                  double wavelength, int octaves, int nthreads, double* z)
{
    if (rows <= 0 || cols <= 0 || octaves <= 0 || wavelength <= 0.0) return -1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    DemJob jobs[256];
    for (int t = 0; t < nthreads; ++t) {
        DemJob* j = &jobs[t];
        j->rows = rows; j->cols = cols; j->seed = seed; j->amplitude = amplitude; j->cell_size = cell_size;
        j->tilt = tilt; j->wavelength = wavelength; j->octaves = octaves; j->z = z;
        j->r0 = rows * t / nthreads;
        j->r1 = rows * (t + 1) / nthreads;
        pthread_create(&th[t], NULL, dem_rows, j);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    return 0;
}

/* --- Priority-Flood+epsilon ---------------------------------------------------------------------- */

typedef struct {
    double z;
    uint64_t idx;
} HeapItem;

static inline int heap_less(const HeapItem* a, const HeapItem* b)
{
    return a->z < b->z || (a->z == b->z && a->idx < b->idx);
}

typedef struct {
    HeapItem* items;
    int64_t size, cap;
} Heap;

static int heap_push(Heap* h, double z, uint64_t idx)
{
    if (h->size == h->cap) {
        int64_t cap = h->cap ? h->cap * 2 : 1 << 16;
        HeapItem* p = (HeapItem*)realloc(h->items, (size_t)cap * sizeof(HeapItem));
        if (!p) return -1;
        h->items = p;
        h->cap = cap;
    }
    int64_t i = h->size++;
    HeapItem it = {z, idx};
    while (i > 0) {
        int64_t parent = (i - 1) / 2;
        if (!heap_less(&it, &h->items[parent])) break;
        h->items[i] = h->items[parent];
        i = parent;
    }
    h->items[i] = it;
    return 0;
}

static HeapItem heap_pop(Heap* h)
{
    HeapItem top = h->items[0];
    HeapItem last = h->items[--h->size];
    int64_t i = 0;
    for (;;) {
        int64_t l = 2 * i + 1, r = l + 1, m = i;
        const HeapItem* best = &last;
        if (l < h->size && heap_less(&h->items[l], best)) { m = l; best = &h->items[l]; }
        if (r < h->size && heap_less(&h->items[r], best)) { m = r; }
        if (m == i) break;
        h->items[i] = h->items[m];
        i = m;
    }
    if (h->size > 0) h->items[i] = last;
    return top;
}

static const int NB_DR[8] = {-1, 0, 0, 1, -1, -1, 1, 1};
static const int NB_DC[8] = {0, -1, 1, 0, -1, 1, -1, 1};

int lue_synth_fill(int64_t rows, int64_t cols, double* z)
{
    int64_t n = rows * cols;
    uint8_t* closed = (uint8_t*)calloc((size_t)n, 1);
    uint64_t* pit = (uint64_t*)malloc((size_t)n * sizeof(uint64_t));
    Heap heap = {0, 0, 0};
    if (!closed || !pit) { free(closed); free(pit); return -2; }
    for (int64_t r = 0; r < rows; ++r) {
        for (int64_t c = 0; c < cols; ++c) {
            if (r == 0 || c == 0 || r == rows - 1 || c == cols - 1) {
                int64_t i = r * cols + c;
                closed[i] = 1;
                if (heap_push(&heap, z[i], (uint64_t)i)) { free(closed); free(pit); free(heap.items); return -2; }
            }
        }
    }
    int64_t pit_head = 0, pit_tail = 0;
    while (pit_head < pit_tail || heap.size > 0) {
        uint64_t i;
        if (pit_head < pit_tail) i = pit[pit_head++];
        else i = heap_pop(&heap).idx;
        int64_t r = (int64_t)i / cols, c = (int64_t)i % cols;
        double zc = z[i];
        for (int k = 0; k < 8; ++k) {
            int64_t rn = r + NB_DR[k], cn = c + NB_DC[k];
            if (rn < 0 || rn >= rows || cn < 0 || cn >= cols) continue;
            int64_t j = rn * cols + cn;
            if (closed[j]) continue;
            closed[j] = 1;
            if (z[j] <= zc) {
                z[j] = nextafter(zc, DBL_MAX);
                pit[pit_tail++] = (uint64_t)j;
            } else if (heap_push(&heap, z[j], (uint64_t)j)) {
                free(closed); free(pit); free(heap.items);
                return -2;
            }
        }
        if (pit_head == pit_tail) pit_head = pit_tail = 0;
    }
    free(closed);
    free(pit);
    free(heap.items);
    return 0;
}

/* --- D8 (reference rule) ------------------------------------------------------------------------ */

typedef struct {
    int64_t rows, cols, r0, r1;
    const double* z;
    uint8_t* fd;
} D8Job;

static void* d8_rows(void* arg)
{
    D8Job* j = (D8Job*)arg;
    const double halo = DBL_MIN; /* std::numeric_limits<double>::min() */
    /* candidate order and codes: N, W, E, S, NW, NE, SW, SE */
    static const int dr[8] = {-1, 0, 0, 1, -1, -1, 1, 1};
    static const int dc[8] = {0, -1, 1, 0, -1, 1, -1, 1};
    static const uint8_t code[8] = {8, 4, 6, 2, 7, 9, 1, 3};
    for (int64_t r = j->r0; r < j->r1; ++r) {
        for (int64_t c = 0; c < j->cols; ++c) {
            double zc = j->z[r * j->cols + c];
            uint8_t dir = 5;
            double drop = 0.0;
            for (int k = 0; k < 8; ++k) {
                int64_t rn = r + dr[k], cn = c + dc[k];
                double zn = (rn < 0 || rn >= j->rows || cn < 0 || cn >= j->cols) ? halo : j->z[rn * j->cols + cn];
                double other = zc - zn;
                if (other > drop) {
                    drop = other;
                    dir = code[k];
                }
            }
            j->fd[r * j->cols + c] = dir;
        }
    }
    return NULL;
}

int lue_synth_d8(int64_t rows, int64_t cols, const double* z, int nthreads, uint8_t* fd)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    D8Job jobs[256];
    for (int t = 0; t < nthreads; ++t) {
        D8Job* j = &jobs[t];
        j->rows = rows; j->cols = cols; j->z = z; j->fd = fd;
        j->r0 = rows * t / nthreads;
        j->r1 = rows * (t + 1) / nthreads;
        pthread_create(&th[t], NULL, d8_rows, j);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    return 0;
}

/* --- validation -------------------------------------------------------------------------------- */

static inline int d8_target(uint8_t code, int64_t r, int64_t c, int64_t rows, int64_t cols, int64_t* rd, int64_t* cd)
{
    int dr = 0, dc = 0;
    switch (code) {
        case 7: dr = -1; dc = -1; break;
        case 8: dr = -1; break;
        case 9: dr = -1; dc = 1; break;
        case 4: dc = -1; break;
        case 6: dc = 1; break;
        case 1: dr = 1; dc = -1; break;
        case 2: dr = 1; break;
        case 3: dr = 1; dc = 1; break;
        default: return 0; /* sink or no-data */
    }
    *rd = r + dr;
    *cd = c + dc;
    return *rd >= 0 && *rd < rows && *cd >= 0 && *cd < cols;
}

/*
 * stats[0] = cells never peeled (on or downstream of a cycle)
 * stats[1] = interior sinks (code 5 or unknown, not no-data, not on the edge)
 * stats[2] = cells flowing into a no-data (255) cell
 * stats[3] = longest flow path in cells (Kahn depth + 1)
 * stats[4] = cells whose flow leaves the array
 */
int lue_synth_validate(int64_t rows, int64_t cols, const uint8_t* fd, int64_t* stats)
{
    int64_t n = rows * cols;
    uint8_t* cnt = (uint8_t*)calloc((size_t)n, 1);
    int32_t* depth = (int32_t*)calloc((size_t)n, sizeof(int32_t));
    int64_t* queue = (int64_t*)malloc((size_t)n * sizeof(int64_t));
    if (!cnt || !depth || !queue) { free(cnt); free(depth); free(queue); return -2; }
    memset(stats, 0, 5 * sizeof(int64_t));
    for (int64_t r = 0; r < rows; ++r) {
        for (int64_t c = 0; c < cols; ++c) {
            uint8_t code = fd[r * cols + c];
            if (code == 255) continue;
            int64_t rd, cd;
            if (d8_target(code, r, c, rows, cols, &rd, &cd)) {
                if (fd[rd * cols + cd] == 255) stats[2]++;
                cnt[rd * cols + cd]++;
            } else {
                int is_sink = !(code == 1 || code == 2 || code == 3 || code == 4 || code == 6 || code == 7 ||
                                code == 8 || code == 9);
                int edge = r == 0 || c == 0 || r == rows - 1 || c == cols - 1;
                if (is_sink && !edge) stats[1]++;
                if (!is_sink) stats[4]++;
            }
        }
    }
    int64_t head = 0, tail = 0, peeled = 0, valid = 0;
    for (int64_t i = 0; i < n; ++i) {
        if (fd[i] == 255) continue;
        valid++;
        if (cnt[i] == 0) queue[tail++] = i;
    }
    int32_t longest = 0;
    while (head < tail) {
        int64_t i = queue[head++];
        peeled++;
        if (depth[i] > longest) longest = depth[i];
        int64_t rd, cd;
        if (d8_target(fd[i], i / cols, i % cols, rows, cols, &rd, &cd)) {
            int64_t j = rd * cols + cd;
            if (fd[j] == 255) continue;
            if (depth[i] + 1 > depth[j]) depth[j] = depth[i] + 1;
            if (--cnt[j] == 0) queue[tail++] = j;
        }
    }
    stats[0] = valid - peeled;
    stats[3] = (int64_t)longest + 1;
    free(cnt);
    free(depth);
    free(queue);
    return 0;
}
