// path_route.cu — the path engine (see path_route.cuh): heavy-path layout of the flow forest, built once
// per raster, and accu_threshold / accu_fraction / accu_capacity (float32) as one prefix scan per path
// level.
#include <algorithm>
#include <cmath>
#include <string>

#include "route_walk_visitors.cuh"
#include "topology.cuh"

namespace lue_gb300 {

// ---------------------------------------------------------------------------------------------------
// Build
// ---------------------------------------------------------------------------------------------------

// Upstream-first walk: per cell the cells upstream of it (itself included), its heavy upstream neighbour
// (the one with most cells upstream, the first in neighbour order on ties; 8: none), the cells above it
// on its path, and its path level (the largest number of light edges on a flow path ending at it).
struct PathVisitor {
    const uint8_t* upmask;
    int32_t* size;
    int32_t* dtop;
    int32_t* plev;
    int32_t* heavy;
    int64_t cols;
    __device__ void enter(int64_t c)
    {
        const unsigned m = __ldg(upmask + c);
        int32_t sz = 1, best = -1;
        int hk = 8;
        for (unsigned mm = m; mm; mm &= mm - 1) {
            const int k = __ffs(mm) - 1;
            const int32_t s = load_cg(size + c + nb_dr(k) * cols + nb_dc(k));
            sz += s;
            if (s > best) {
                best = s;
                hk = k;
            }
        }
        int32_t lv = 0, dt = 0;
        for (unsigned mm = m; mm; mm &= mm - 1) {
            const int k = __ffs(mm) - 1;
            const int64_t u = c + nb_dr(k) * cols + nb_dc(k);
            const int32_t l = load_cg(plev + u);
            if (k == hk) {
                lv = max(lv, l);
                dt = load_cg(dtop + u) + 1;
            } else {
                lv = max(lv, l + 1);
            }
        }
        size[c] = sz;
        plev[c] = lv;
        dtop[c] = dt;
        heavy[c] = hk;
    }
    __device__ void no_data(int64_t) {}
};

// Neighbour slot k of a cell's upstream neighbour that drains into it with D8 code `code`.
__device__ __forceinline__ int inflow_slot(uint8_t code)
{
    switch (code) {
        case 3: return 0;
        case 2: return 1;
        case 1: return 2;
        case 6: return 3;
        case 4: return 4;
        case 9: return 5;
        case 8: return 6;
        case 7: return 7;
        default: return -1;
    }
}

__global__ void k_fill(int32_t* p, int64_t n, int32_t v)
{
    for (int64_t i = grid_stride_begin(); i < n; i += grid_stride()) p[i] = v;
}

// next[c]: the cell below c on its path (c itself at the bottom), -1 for no-data.
__global__ void k_path_next(const uint8_t* fd, const int32_t* heavy, int64_t rows, int64_t cols, int64_t n,
                            int32_t* next)
{
    for (int64_t c = grid_stride_begin(); c < n; c += grid_stride()) {
        const uint8_t code = __ldg(fd + c);
        if (code == kNoData) {
            next[c] = -1;
            continue;
        }
        const int64_t r = c / cols, col = c - r * cols;
        int64_t d = 0;
        int32_t v = (int32_t)c;
        if (downstream(code, r, col, rows, cols, d) && __ldg(fd + d) != kNoData && heavy[d] == inflow_slot(code))
            v = (int32_t)d;
        next[c] = v;
    }
}

// One round of pointer jumping: next[c] = next[next[c]] (in place: a value read from a cell that has
// already jumped this round is still a cell of the same path, at or above the bottom).
__global__ void k_path_jump(int32_t* next, int64_t n)
{
    for (int64_t c = grid_stride_begin(); c < n; c += grid_stride()) {
        const int32_t v = next[c];
        if (v >= 0) next[c] = next[v];
    }
}

// key[c] = path level of c if c is the bottom of its path, else 255; stats: [0] largest level,
// [1] longest path, [2] cells whose next is not a bottom (must be 0).
__global__ void k_path_keys(const int32_t* next, const int32_t* plev, const int32_t* dtop, int64_t n, uint8_t* key,
                            int* stats)
{
    int lmax = -1, longest = 0, bad = 0;
    for (int64_t c = grid_stride_begin(); c < n; c += grid_stride()) {
        const int32_t v = next[c];
        uint8_t k = 255;
        if (v >= 0) {
            if (next[v] != v) ++bad;
            if (v == c) {
                const int l = plev[c];
                k = (uint8_t)min(l, 254);
                lmax = max(lmax, l);
                longest = max(longest, dtop[c] + 1);
            }
        }
        key[c] = k;
    }
    if (lmax >= 0) atomicMax(stats, lmax);
    if (longest) atomicMax(stats + 1, longest);
    if (bad) atomicAdd(stats + 2, bad);
}

constexpr int kCompactPer = 32;                          // cells per thread
constexpr int kCompactCells = 256 * kCompactPer;         // cells per CTA

template <int NT>
__device__ __forceinline__ long long block_excl_sum(long long v, long long* s_warp, long long& total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    long long x = v;
    for (int d = 1; d < 32; d <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        long long w = lane < NT / 32 ? s_warp[lane] : 0;
        for (int d = 1; d < 32; d <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= d) w += y;
        }
        if (lane < NT / 32) s_warp[lane] = w;
    }
    __syncthreads();
    total = s_warp[NT / 32 - 1];
    const long long before = warp ? s_warp[warp - 1] : 0;
    __syncthreads();
    return before + x - v;
}

// Per CTA of cells: the positions taken by the paths of level `lvl` whose bottom lies in it; longest[lvl]:
// the longest path of the level.
__global__ void __launch_bounds__(256) k_level_sums(const uint8_t* key, const int32_t* dtop, int lvl, int64_t n,
                                                    long long* bsum, int* longest)
{
    __shared__ long long s_warp[8];
    const int64_t c0 = (int64_t)blockIdx.x * kCompactCells + (int64_t)threadIdx.x * kCompactPer;
    long long s = 0;
    int lmax = 0;
    for (int j = 0; j < kCompactPer; ++j) {
        const int64_t c = c0 + j;
        if (c < n && key[c] == lvl) {
            s += dtop[c] + 1;
            lmax = max(lmax, dtop[c] + 1);
        }
    }
    long long total = 0;
    block_excl_sum<256>(s, s_warp, total);
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
    for (int d = 16; d; d >>= 1) lmax = max(lmax, __shfl_xor_sync(0xffffffffu, lmax, d));
    if ((threadIdx.x & 31) == 0 && lmax) atomicMax(longest + lvl, lmax);
}

// Exclusive scan of the per-CTA sums of one level, after the positions of the lower levels
// (running[0]); offsets[lvl + 1] = running[0] afterwards.
__global__ void __launch_bounds__(1024) k_level_scan(long long* bsum, int64_t nblk, long long* running,
                                                     long long* offsets, int lvl)
{
    __shared__ long long s_warp[32];
    const int64_t per = (nblk + 1023) / 1024;
    const int64_t b0 = (int64_t)threadIdx.x * per, b1 = min(nblk, b0 + per);
    long long s = 0;
    for (int64_t b = b0; b < b1; ++b) s += bsum[b];
    long long total = 0;
    long long x = block_excl_sum<1024>(s, s_warp, total) + running[0];
    for (int64_t b = b0; b < b1; ++b) {
        const long long v = bsum[b];
        bsum[b] = x;
        x += v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        offsets[lvl] = running[0];
        running[0] += total;
        offsets[lvl + 1] = running[0];
    }
}

// base[b]: first position of the path whose bottom is b (paths of one level in cell order of bottoms).
__global__ void __launch_bounds__(256) k_level_assign(const uint8_t* key, const int32_t* dtop, int lvl, int64_t n,
                                                      const long long* bsum, int32_t* base)
{
    __shared__ long long s_warp[8];
    const int64_t c0 = (int64_t)blockIdx.x * kCompactCells + (int64_t)threadIdx.x * kCompactPer;
    long long s = 0;
    for (int j = 0; j < kCompactPer; ++j) {
        const int64_t c = c0 + j;
        if (c < n && key[c] == lvl) s += dtop[c] + 1;
    }
    long long total = 0;
    long long x = block_excl_sum<256>(s, s_warp, total) + bsum[blockIdx.x];
    for (int j = 0; j < kCompactPer; ++j) {
        const int64_t c = c0 + j;
        if (c < n && key[c] == lvl) {
            base[c] = (int32_t)x;
            x += dtop[c] + 1;
        }
    }
}

// order / light by position (order starts as all ones: no cell).  bad counts positions outside
// [0, npos) and positions written twice; the build then fails instead of handing on a wrong layout.
__global__ void k_path_place(const int32_t* next, const int32_t* base, const int32_t* dtop, const int32_t* heavy,
                             const uint8_t* upmask, int64_t n, int64_t npos, int32_t* order, uint8_t* light, int* bad)
{
    int nbad = 0;
    for (int64_t c = grid_stride_begin(); c < n; c += grid_stride()) {
        const int32_t b = next[c];
        if (b < 0) continue;
        const int32_t dt = dtop[c];
        const int64_t pos = (int64_t)base[b] + dt;
        if (pos < 0 || pos >= npos) {
            ++nbad;
            continue;
        }
        const int32_t old = atomicExch(order + pos, (int32_t)((uint32_t)c | (dt == 0 ? 0x80000000u : 0u)));
        if (old != -1) ++nbad;
        const int hk = heavy[c];
        light[pos] = (uint8_t)(__ldg(upmask + c) & ~(hk < 8 ? 1u << hk : 0u));
    }
    if (nbad) atomicAdd(bad, nbad);
}

// Positions that no cell took.
__global__ void k_path_unwritten(const int32_t* order, int64_t npos, int* bad)
{
    int nbad = 0;
    for (int64_t i = grid_stride_begin(); i < npos; i += grid_stride()) nbad += order[i] == -1;
    if (nbad) atomicAdd(bad, nbad);
}

// Position arrays are padded to whole 8-position chunks plus one chunk, for the vector loads of the
// per-call kernels.
static int64_t path_padded(int64_t npos) { return ((npos + 7) / 8 + 1) * 8; }

// Positions per thread of a level: LUE_GB300_PATH_PER (1, 2, 4 or 8; default 4, the fastest at 16384^2:
// 8.7 ms against 9.8 ms for 8 and 9.3 ms for 2) for large levels, 1 for small ones (of long paths: short
// chains of dependent loads per thread).
constexpr int64_t kPathSmallLevel = 1 << 20;
static int path_per_large()
{
    static const int per = [] {
        const char* e = getenv("LUE_GB300_PATH_PER");
        const int v = e ? atoi(e) : 4;
        return v == 1 || v == 2 || v == 8 ? v : 4;
    }();
    return per;
}
static int path_per(int64_t p0, int64_t p1) { return p1 - p0 < kPathSmallLevel ? 1 : path_per_large(); }
static int64_t path_level_tiles(int64_t p0, int64_t p1, int per)
{
    if (p1 <= p0) return 0;
    const int64_t base = per > 1 ? (p0 & ~int64_t(per - 1)) : p0;
    return (p1 - base + kPathThreads * per - 1) / (kPathThreads * per);
}

void path_core_free(PathCore* pc)
{
    if (!pc) return;
    cudaFree(pc->order);
    cudaFree(pc->light);
    delete pc;
}

int path_core_build(const TopologyCore* core, uint32_t* work, cudaStream_t stream, PathCore** out)
{
    *out = nullptr;
    const int64_t n = core->n, rows = core->rows, cols = core->cols;
    if (n >= (int64_t(1) << 31)) return fail(LUE_GPU_ERANGE, "path topology: 2^31 cells or more");
    const int64_t npos = core->stats.valid_cells;
    auto* pc = new (std::nothrow) PathCore();
    if (!pc) return fail(LUE_GPU_ENOMEM, "path topology: host allocation");
    pc->npos = npos;
    int32_t *size = nullptr, *dtop = nullptr, *plev = nullptr, *heavy = nullptr, *next = nullptr;
    uint8_t* key = nullptr;
    long long* scan = nullptr;  // [0] running, [1..] offsets, then per-CTA sums
    int* stats = nullptr;
    const int64_t nblk = (n + kCompactCells - 1) / kCompactCells;
    const int kMaxLevels = 255;
    int rc = LUE_GPU_OK;
    int hstats[3] = {0, 0, 0};
    const char* what = "path topology";
    auto cleanup = [&]() {
        cudaFree(size);
        cudaFree(dtop);
        cudaFree(plev);
        cudaFree(heavy);
        cudaFree(next);
        cudaFree(key);
        cudaFree(scan);
        cudaFree(stats);
    };
    if ((rc = cuda_status(cudaMalloc(&size, n * sizeof(int32_t)), what)) ||
        (rc = cuda_status(cudaMalloc(&dtop, n * sizeof(int32_t)), what)) ||
        (rc = cuda_status(cudaMalloc(&plev, n * sizeof(int32_t)), what)) ||
        (rc = cuda_status(cudaMalloc(&heavy, n * sizeof(int32_t)), what)) ||
        (rc = cuda_status(cudaMalloc(&next, n * sizeof(int32_t)), what)) ||
        (rc = cuda_status(cudaMalloc(&key, n), what)) ||
        (rc = cuda_status(cudaMalloc(&scan, (2 + kMaxLevels + 1 + nblk) * sizeof(long long)), what)) ||
        (rc = cuda_status(cudaMalloc(&stats, (3 + kMaxLevels) * sizeof(int)), what)) ||
        (rc = cuda_status(cudaMalloc(&pc->order, path_padded(npos) * sizeof(int32_t)), what)) ||
        (rc = cuda_status(cudaMalloc(&pc->light, path_padded(npos)), what))) {
        cleanup();
        path_core_free(pc);
        return rc;
    }
    pc->bytes = path_padded(npos) * 5;
    // 1. sizes, heavy neighbours, cells above on the path, path levels
    k_fill<<<grid_for(n, 256), 256, 0, stream>>>(heavy, n, 8);
    cudaMemcpyAsync(work, core->count, words_for(n) * 4, cudaMemcpyDeviceToDevice, stream);
    {
        WalkGrid g{core->fd, core->count, work, rows, cols, n};
        PathVisitor v{core->upmask, size, dtop, plev, heavy, cols};
        k_walk<<<grid_all(n, 256), 256, 0, stream>>>(g, v);
    }
    // 2. bottom of each cell's path: pointer jumping over the path links
    k_path_next<<<grid_for(n, 256), 256, 0, stream>>>(core->fd, heavy, rows, cols, n, next);
    int rounds = 1;
    while ((int64_t(1) << rounds) < core->stats.max_level + 2) ++rounds;
    for (int i = 0; i <= rounds; ++i) k_path_jump<<<grid_for(n, 256), 256, 0, stream>>>(next, n);
    // 3. keys and level count
    cudaMemsetAsync(stats, 0, 3 * sizeof(int), stream);
    k_path_keys<<<grid_for(n, 256), 256, 0, stream>>>(next, plev, dtop, n, key, stats);
    if ((rc = cuda_status(cudaMemcpyAsync(hstats, stats, sizeof hstats, cudaMemcpyDeviceToHost, stream), what)) ||
        (rc = cuda_status(cudaStreamSynchronize(stream), what))) {
        cleanup();
        path_core_free(pc);
        return rc;
    }
    if (hstats[2] != 0 || hstats[0] >= 254) {
        cleanup();
        path_core_free(pc);
        return fail(LUE_GPU_ERANGE, "path topology: " + std::to_string(hstats[2]) + " cells without a bottom, " +
                                        std::to_string(hstats[0] + 1) + " levels");
    }
    const int levels = npos > 0 ? hstats[0] + 1 : 0;
    pc->longest_path = hstats[1];
    // 4. positions: levels in order, paths of a level in cell order of their bottoms
    int32_t* base = size;  // sizes are no longer needed
    long long* running = scan;
    long long* offsets = scan + 1;
    long long* bsum = scan + 2 + kMaxLevels;
    cudaMemsetAsync(scan, 0, (2 + kMaxLevels) * sizeof(long long), stream);
    int* longest = stats + 3;
    cudaMemsetAsync(longest, 0, kMaxLevels * sizeof(int), stream);
    for (int l = 0; l < levels; ++l) {
        k_level_sums<<<(unsigned)nblk, 256, 0, stream>>>(key, dtop, l, n, bsum, longest);
        k_level_scan<<<1, 1024, 0, stream>>>(bsum, nblk, running, offsets, l);
        k_level_assign<<<(unsigned)nblk, 256, 0, stream>>>(key, dtop, l, n, bsum, base);
    }
    cudaMemsetAsync(pc->order, 0xFF, path_padded(npos) * sizeof(int32_t), stream);
    cudaMemsetAsync(pc->light, 0, path_padded(npos), stream);
    cudaMemsetAsync(stats + 2, 0, sizeof(int), stream);
    k_path_place<<<grid_for(n, 256), 256, 0, stream>>>(next, base, dtop, heavy, core->upmask, n, npos, pc->order,
                                                       pc->light, stats + 2);
    k_path_unwritten<<<grid_for(npos, 256), 256, 0, stream>>>(pc->order, npos, stats + 2);
    std::vector<long long> hoff(levels + 1, 0);
    std::vector<int> hlong(std::max(levels, 1), 0);
    if (levels > 0 &&
        ((rc = cuda_status(cudaMemcpyAsync(hoff.data(), offsets, (levels + 1) * sizeof(long long),
                                           cudaMemcpyDeviceToHost, stream),
                           what)) ||
         (rc = cuda_status(cudaMemcpyAsync(hlong.data(), longest, levels * sizeof(int), cudaMemcpyDeviceToHost,
                                           stream),
                           what)))) {
        cleanup();
        path_core_free(pc);
        return rc;
    }
    int bad = 0;
    rc = cuda_status(cudaMemcpyAsync(&bad, stats + 2, sizeof(int), cudaMemcpyDeviceToHost, stream), what);
    if (!rc) rc = cuda_status(cudaStreamSynchronize(stream), what);
    if (!rc) rc = cuda_status(cudaGetLastError(), what);
    cleanup();
    count_launches(8 + rounds + 3 * levels);
    if (rc) {
        path_core_free(pc);
        return rc;
    }
    if ((levels > 0 && hoff[levels] != npos) || bad) {
        path_core_free(pc);
        return fail(LUE_GPU_ERANGE, "path topology: inconsistent layout (" + std::to_string(levels ? hoff[levels] : 0) +
                                        " positions for " + std::to_string(npos) + " cells, " + std::to_string(bad) +
                                        " misplaced)");
    }
    pc->level_offsets.assign(hoff.begin(), hoff.end());
    pc->level_longest.assign(hlong.begin(), hlong.begin() + levels);
    pc->tiles = 0;
    for (int l = 0; l < levels; ++l)  // as many as one position per thread would need
        pc->tiles = std::max(pc->tiles, path_level_tiles(hoff[l], hoff[l + 1], 1));
    if (getenv("LUE_GB300_VERBOSE")) {
        fprintf(stderr, "path topology: %lld cells, %d levels, %lld tiles, longest path %lld cells; positions "
                        "(longest path) by level:",
                (long long)npos, levels, (long long)pc->tiles, (long long)pc->longest_path);
        for (int l = 0; l < levels; ++l) fprintf(stderr, " %lld (%d)", hoff[l + 1] - hoff[l], hlong[l]);
        fprintf(stderr, "\n");
    }
    *out = pc;
    return LUE_GPU_OK;
}

// ---------------------------------------------------------------------------------------------------
// Per call
// ---------------------------------------------------------------------------------------------------

// A map x -> op(x + a, b) with op = max (threshold) or min (capacity), or x -> a * x + b (fraction); a and
// b float-float.  flags bit 0: the map of a path's top cell, which ignores its input (its value is b);
// bit 1: no-data (NaN) from the cell itself or from upstream.
struct PMap {
    float ah, al, bh, bl;
    int flags;
};

// Kinds of maps: x -> max(x + a, b) (threshold), x -> min(x + a, b) (capacity), x -> a * x + b (fraction).
constexpr int kMaxPlus = 0, kMinPlus = 1, kAffine = 2;

template <int K>
__device__ __forceinline__ PMap pm_identity()
{
    if (K == kAffine) return PMap{1.0f, 0.0f, 0.0f, 0.0f, 0};
    return PMap{0.0f, 0.0f, K == kMinPlus ? INFINITY : -INFINITY, 0.0f, 0};
}

// x + y for float-float values; a sum that is not finite is kept with lo = 0 (two_sum's error terms would
// turn an infinity into NaN).
__device__ __forceinline__ void ff_sum(float xh, float xl, float yh, float yl, float& rh, float& rl)
{
    float s, e;
    two_sum(xh, yh, s, e);
    if (!isfinite(s)) {
        rh = s;
        rl = 0.0f;
        return;
    }
    e = __fadd_rn(e, __fadd_rn(xl, yl));
    rh = __fadd_rn(s, e);
    rl = __fsub_rn(e, __fsub_rn(rh, s));
}

__device__ __forceinline__ bool ff_less(float xh, float xl, float yh, float yl)
{
    return xh < yh || (xh == yh && xl < yl);
}

// x * y for float-float values: the exact product of the high parts by FMA (two-product), plus the cross
// terms, renormalised.
__device__ __forceinline__ void ff_mul(float xh, float xl, float yh, float yl, float& rh, float& rl)
{
    const float p = __fmul_rn(xh, yh);
    float e = __fmaf_rn(xh, yh, -p);
    e = __fmaf_rn(xh, yl, e);
    e = __fmaf_rn(xl, yh, e);
    if (!isfinite(p)) {
        rh = p;
        rl = 0.0f;
        return;
    }
    rh = __fadd_rn(p, e);
    rl = __fsub_rn(e, __fsub_rn(rh, p));
}

// m1 first, then m2.
template <int K>
__device__ __forceinline__ PMap compose(const PMap& m1, const PMap& m2)
{
    if (m2.flags & 1) return m2;
    PMap r;
    r.flags = (m1.flags & 1) | ((m1.flags | m2.flags) & 2);
    if (K == kAffine) {  // a2 * (a1 * x + b1) + b2
        ff_mul(m1.ah, m1.al, m2.ah, m2.al, r.ah, r.al);
        float th, tl;
        ff_mul(m2.ah, m2.al, m1.bh, m1.bl, th, tl);
        ff_sum(th, tl, m2.bh, m2.bl, r.bh, r.bl);
        return r;
    }
    ff_sum(m1.ah, m1.al, m2.ah, m2.al, r.ah, r.al);
    float th, tl;
    ff_sum(m1.bh, m1.bl, m2.ah, m2.al, th, tl);
    const bool take = K == kMinPlus ? ff_less(th, tl, m2.bh, m2.bl) : ff_less(m2.bh, m2.bl, th, tl);
    r.bh = take ? th : m2.bh;
    r.bl = take ? tl : m2.bl;
    return r;
}

// The map of one cell: s = its material plus the outflow of its light upstream neighbours, b its
// threshold or capacity.
template <Rule R>
__device__ __forceinline__ PMap cell_map(bool top, float sh, float sl, float b, bool nan)
{
    if (nan) return PMap{0.0f, 0.0f, 0.0f, 0.0f, 2 | (top ? 1 : 0)};
    if (top) {
        float oh = 0.0f, ol = 0.0f, rem = 0.0f;
        rule_f32<R>(FF{sh, sl}, false, 0.0f, b, oh, ol, rem);
        return PMap{0.0f, 0.0f, oh, ol, 1};
    }
    if (R == Rule::threshold) {  // max(x + (s - threshold), 0)
        float dh, dl;
        ff_sum(sh, sl, -b, 0.0f, dh, dl);
        return PMap{dh, dl, 0.0f, 0.0f, 0};
    }
    if (R == Rule::fraction) {  // fraction * x + fraction * s
        float qh, ql;
        ff_mul(b, 0.0f, sh, sl, qh, ql);
        return PMap{b, 0.0f, qh, ql, 0};
    }
    return PMap{sh, sl, b, 0.0f, 0};  // capacity: min(x + s, capacity)
}

__device__ __forceinline__ PMap shfl_up(const PMap& m, int d)
{
    PMap r;
    r.ah = __shfl_up_sync(0xffffffffu, m.ah, d);
    r.al = __shfl_up_sync(0xffffffffu, m.al, d);
    r.bh = __shfl_up_sync(0xffffffffu, m.bh, d);
    r.bl = __shfl_up_sync(0xffffffffu, m.bl, d);
    r.flags = __shfl_up_sync(0xffffffffu, m.flags, d);
    return r;
}

// Exclusive scan of the threads' maps in thread order; `total` is the composition of all of them.
template <int K, int NT>
__device__ __forceinline__ PMap block_excl_scan(const PMap& v, PMap* s_warp, PMap& total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    PMap x = v;
    for (int d = 1; d < 32; d <<= 1) {
        const PMap y = shfl_up(x, d);
        if (lane >= d) x = compose<K>(y, x);
    }
    PMap ex = shfl_up(x, 1);
    if (lane == 0) ex = pm_identity<K>();
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        PMap w = lane < NT / 32 ? s_warp[lane] : pm_identity<K>();
        for (int d = 1; d < 32; d <<= 1) {
            const PMap y = shfl_up(w, d);
            if (lane >= d) w = compose<K>(y, w);
        }
        if (lane < NT / 32) s_warp[lane] = w;
    }
    __syncthreads();
    total = s_warp[NT / 32 - 1];
    const PMap r = warp ? compose<K>(s_warp[warp - 1], ex) : ex;
    __syncthreads();
    return r;
}

struct PathCall {
    const int32_t* __restrict__ order;
    const uint8_t* __restrict__ light;
    const float* __restrict__ a;  // material
    float as;
    const float* __restrict__ b;  // threshold / fraction / capacity
    float bs;
    float* out;
    float* rem;
    float* lo;                    // float-float residual of the outflow (path bottoms: read as light inflow)
    unsigned long long* flag;
    int64_t cols;
};

// The order entries of PER consecutive positions from `first` (a multiple of PER), read with vector
// loads; the position arrays are padded by one 8-position chunk, so a chunk that starts before the end
// of the array stays inside it.
template <int PER>
__device__ __forceinline__ void load_order(const PathCall& p, int64_t first, int32_t (&w)[PER])
{
    if (PER == 4) {
        const int4 x = __ldg(reinterpret_cast<const int4*>(p.order + first));
        w[0] = x.x; w[1 % PER] = x.y; w[2 % PER] = x.z; w[3 % PER] = x.w;
    } else if (PER == 2) {
        const int2 x = __ldg(reinterpret_cast<const int2*>(p.order + first));
        w[0] = x.x; w[1 % PER] = x.y;
    } else if (PER == 8) {
        const int4 x = __ldg(reinterpret_cast<const int4*>(p.order + first));
        const int4 y = __ldg(reinterpret_cast<const int4*>(p.order + first) + 1);
        w[0] = x.x; w[1] = x.y; w[2] = x.z; w[3] = x.w;
        w[4 % PER] = y.x; w[5 % PER] = y.y; w[6 % PER] = y.z; w[7 % PER] = y.w;
    } else {
#pragma unroll
        for (int j = 0; j < PER; ++j) w[j] = __ldg(p.order + first + j);
    }
}

template <int PER>
__device__ __forceinline__ int64_t chunk_base(int64_t p0)
{
    return PER > 1 ? (p0 & ~int64_t(PER - 1)) : p0;
}

__device__ __forceinline__ int ld_acquire_gpu(const int* p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(int* p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ PMap ld_map(const PMap* m)
{
    return PMap{__ldcg(&m->ah), __ldcg(&m->al), __ldcg(&m->bh), __ldcg(&m->bl), __ldcg(&m->flags)};
}

__device__ __forceinline__ PMap shfl_down(const PMap& m, int d)
{
    PMap r;
    r.ah = __shfl_down_sync(0xffffffffu, m.ah, d);
    r.al = __shfl_down_sync(0xffffffffu, m.al, d);
    r.bh = __shfl_down_sync(0xffffffffu, m.bh, d);
    r.bl = __shfl_down_sync(0xffffffffu, m.bl, d);
    r.flags = __shfl_down_sync(0xffffffffu, m.flags, d);
    return r;
}

// Decoupled look-back of one level's launch: CTAs take tiles in ticket order; each publishes the
// composition of its tile's maps (state 1), then the composition of everything before and including its
// tile (state 2).  Status words carry the launch's epoch, so the arrays need no clearing between launches.
struct PathScan {
    int* status;  // [tiles] epoch << 2 | state
    PMap* aggm;   // [tiles] the tile's own composition
    PMap* inclm;  // [tiles] the composition up to and including the tile
    int* ticket;  // zeroed before the launch
    int epoch;
    int polls;    // poll limit of one wait
};

constexpr int kPathPolls = 1 << 20;

// Warp 0: the composition of all tiles before `tile` (in every lane).  Lane i looks at tile j - i, 32 at
// a time, until a tile with a published prefix is among them.  Every wait is bounded: a wait that gives
// up (or finds that another one did) sets flag[1], after which the walk engine redoes the call.
template <int K>
__device__ PMap look_back(const PathScan& q, int64_t tile, unsigned long long* flag)
{
    const int lane = threadIdx.x & 31;
    PMap running = pm_identity<K>();
    for (int64_t j = tile - 1;; j -= 32) {
        const int64_t idx = j - lane;
        int st = 2;
        PMap m = pm_identity<K>();
        if (idx >= 0) {
            int v = 0, k = 0;
            for (; k < q.polls; ++k) {
                v = ld_acquire_gpu(q.status + idx);
                if ((v >> 2) == q.epoch && (v & 3) != 0) break;
                if (*reinterpret_cast<volatile unsigned long long*>(flag + 1)) k = q.polls - 1;
                __nanosleep(32);
            }
            if (k >= q.polls) {
                st = -1;
            } else {
                st = v & 3;
                m = ld_map(st == 2 ? q.inclm + idx : q.aggm + idx);
            }
        }
        if (__ballot_sync(0xffffffffu, st < 0)) {
            if (lane == 0) flag[1] = 1;
            return pm_identity<K>();
        }
        const unsigned incl = __ballot_sync(0xffffffffu, st == 2);
        if (incl && lane > __ffs(incl) - 1) m = pm_identity<K>();
        // lanes 31 .. 0 in this order (farther tiles come first)
        for (int d = 1; d < 32; d <<= 1) {
            const PMap o = shfl_down(m, d);
            if (lane + d < 32) m = compose<K>(o, m);
        }
        const PMap window = PMap{__shfl_sync(0xffffffffu, m.ah, 0), __shfl_sync(0xffffffffu, m.al, 0),
                                 __shfl_sync(0xffffffffu, m.bh, 0), __shfl_sync(0xffffffffu, m.bl, 0),
                                 __shfl_sync(0xffffffffu, m.flags, 0)};
        running = compose<K>(window, running);
        if (incl) return running;
    }
}

// The positions of one thread in one chunk: PER consecutive positions from `first`, those in [lo, hi)
// active.  load(): inputs, light inflow and the cells' maps, composed in order; store(): from the
// composition E of everything before the first position, each cell's rule and outputs.  VEC: `first` is
// a multiple of PER and the order array is read with vector loads.
template <Rule R, int K, int PER, bool LIGHT, bool VEC>
struct Chunk {
    int32_t w[PER];
    bool on[PER];
    float b[PER];
    FF sum[PER];
    bool nan[PER];

    __device__ __forceinline__ PMap load(const PathCall& p, int64_t first, int64_t lo, int64_t hi)
    {
#pragma unroll
        for (int j = 0; j < PER; ++j) on[j] = first + j >= lo && first + j < hi;
        if (VEC && first < hi) {
            load_order<PER>(p, first, w);
        } else {
#pragma unroll
            for (int j = 0; j < PER; ++j) w[j] = on[j] ? __ldg(p.order + first + j) : 0;
        }
        float e[PER];
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            const int64_t c = (int64_t)(w[j] & 0x7fffffff);
            e[j] = on[j] ? value_at(p.a, p.as, c) : 0.0f;
            b[j] = on[j] ? value_at(p.b, p.bs, c) : 0.0f;
            sum[j] = FF{0.0f, 0.0f};
            nan[j] = false;
        }
        if (LIGHT) {
#pragma unroll
            for (int j = 0; j < PER; ++j) {
                if (!on[j]) continue;
                const int64_t c = (int64_t)(w[j] & 0x7fffffff);
                for (unsigned lm = __ldg(p.light + first + j); lm; lm &= lm - 1) {
                    const int k = __ffs(lm) - 1;
                    const int64_t u = c + nb_dr(k) * p.cols + nb_dc(k);
                    const float vh = p.out[u];
                    nan[j] |= isnan(vh);
                    sum[j].add(vh, p.lo[u]);
                }
            }
        }
        PMap acc = pm_identity<K>();
        bool odd = false;
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            if (!on[j]) continue;
            nan[j] |= isnan(e[j]) || isnan(b[j]) || !(e[j] >= 0.0f && b[j] >= 0.0f) ||
                      (R == Rule::fraction && !(b[j] <= 1.0f));
            sum[j].add(e[j]);
            sum[j].normalise();
            odd |= !nan[j] && (isinf(e[j]) || isinf(b[j]) || isinf(sum[j].hi));
            acc = compose<K>(acc, cell_map<R>(w[j] < 0, sum[j].hi, sum[j].lo, b[j], nan[j]));
        }
        if (odd) p.flag[1] = 1;  // +-inf: the walk engine redoes the call
        return acc;
    }

    __device__ __forceinline__ void store(const PathCall& p, int64_t first, int64_t p1, PMap E)
    {
        // the position after this thread's last one: is it the top of a path (then the last one is a bottom)?
        const int32_t after = first + PER < p1 ? __ldg(p.order + first + PER) : -1;
#pragma unroll
        for (int j = 0; j < PER; ++j) {
            if (!on[j]) continue;
            const int64_t c = (int64_t)(w[j] & 0x7fffffff);
            const bool top = w[j] < 0;
            FF t{0.0f, 0.0f};
            bool nn = nan[j];
            if (!top) {
                nn |= (E.flags & 2) != 0;
                t = FF{E.bh, E.bl};
            }
            t.add(sum[j].hi, sum[j].lo);
            float oh = 0.0f, ol = 0.0f, rem = 0.0f;
            if (!rule_f32<R>(t, nn, 0.0f, b[j], oh, ol, rem)) {
                oh = __int_as_float(0x7fc00000);
                ol = 0.0f;
                rem = oh;
            }
            p.out[c] = oh;
            p.rem[c] = rem;
            const int32_t next = j + 1 < PER ? w[(j + 1) % PER] : after;
            if (first + j + 1 >= p1 || next < 0) p.lo[c] = ol;  // a path bottom
            E = compose<K>(E, cell_map<R>(top, sum[j].hi, sum[j].lo, b[j], nan[j]));
        }
    }
};

#define PATH_BOUNDS(PER) __launch_bounds__(kPathThreads, PER >= 8 ? 2 : (PER == 4 ? 4 : (PER == 2 ? 5 : 6)))

// One level in one pass, for levels with long paths: tiles in ticket order, the composition of the
// tiles before each one by decoupled look-back.
template <Rule R, int K, int PER, bool LIGHT>
__global__ void PATH_BOUNDS(PER) k_path_level(PathCall p, int64_t p0, int64_t p1, PathScan q)
{
    __shared__ PMap s_warp[kPathThreads / 32];
    __shared__ PMap s_prefix;
    __shared__ int64_t s_tile;
    if (threadIdx.x == 0) s_tile = atomicAdd(q.ticket, 1);
    __syncthreads();
    const int64_t tile = s_tile;
    const int64_t first = chunk_base<PER>(p0) + tile * (kPathThreads * PER) + (int64_t)threadIdx.x * PER;
    Chunk<R, K, PER, LIGHT, true> ch;
    const PMap acc = ch.load(p, first, p0, p1);
    PMap total;
    PMap E = block_excl_scan<K, kPathThreads>(acc, s_warp, total);
    if (threadIdx.x < 32) {
        if (tile == 0) {
            if (threadIdx.x == 0) {
                q.inclm[0] = total;
                __threadfence();
                st_release_gpu(q.status, (q.epoch << 2) | 2);
                s_prefix = pm_identity<K>();
            }
        } else {
            if (threadIdx.x == 0) {
                q.aggm[tile] = total;
                __threadfence();
                st_release_gpu(q.status + tile, (q.epoch << 2) | 1);
            }
            const PMap before = look_back<K>(q, tile, p.flag);
            if (threadIdx.x == 0) {
                q.inclm[tile] = compose<K>(before, total);
                __threadfence();
                st_release_gpu(q.status + tile, (q.epoch << 2) | 2);
                s_prefix = before;
            }
        }
    }
    __syncthreads();
    ch.store(p, first, p1, compose<K>(s_prefix, E));
}

// The first path top at or after position s (p1 if none), for every lane of a warp.
__device__ __forceinline__ int64_t next_top(const int32_t* order, int64_t s, int64_t p1)
{
    const int lane = threadIdx.x & 31;
    for (int64_t pos = s; pos < p1; pos += 32) {
        const unsigned m = __ballot_sync(0xffffffffu, pos + lane < p1 && __ldg(order + pos + lane) < 0);
        if (m) return pos + __ffs(m) - 1;
    }
    return p1;
}

// Levels whose paths are all short (at most kPathFreeLongest cells): each CTA's range of positions is
// cut at path tops (its nominal range with both ends moved forward to the next top), so no path crosses
// from one CTA to another and CTAs do not wait for one another; a range is processed in chunks of
// kPathThreads * PER positions with the composition carried from chunk to chunk.
constexpr int kPathFreeLongest = 2048;

template <Rule R, int K, int PER, bool LIGHT>
__global__ void PATH_BOUNDS(PER) k_path_free(PathCall p, int64_t p0, int64_t p1)
{
    __shared__ PMap s_warp[kPathThreads / 32];
    __shared__ PMap s_carry;
    __shared__ int64_t s_range[2];
    const int64_t T = (int64_t)kPathThreads * PER;
    const int64_t s0 = p0 + (int64_t)blockIdx.x * T;
    if (threadIdx.x < 32) {
        const int64_t lo = blockIdx.x == 0 ? p0 : next_top(p.order, s0, p1);
        const int64_t hi = next_top(p.order, min(s0 + T, p1), p1);
        if (threadIdx.x == 0) {
            s_range[0] = lo;
            s_range[1] = hi;
            s_carry = pm_identity<K>();
        }
    }
    __syncthreads();
    const int64_t lo = s_range[0], hi = s_range[1];
    for (int64_t c0 = lo; c0 < hi; c0 += T) {
        const int64_t first = c0 + (int64_t)threadIdx.x * PER;
        Chunk<R, K, PER, LIGHT, false> ch;
        const PMap acc = ch.load(p, first, c0, min(hi, c0 + T));
        PMap total;
        // the scan's barriers come after thread 0's update of s_carry for the previous chunk
        const PMap ex = block_excl_scan<K, kPathThreads>(acc, s_warp, total);
        const PMap E = compose<K>(s_carry, ex);
        __syncthreads();  // every thread has read s_carry
        if (threadIdx.x == 0) s_carry = compose<K>(s_carry, total);
        ch.store(p, first, p1, E);
    }
}

__global__ void k_path_no_data(const uint8_t* fd, int64_t n, float* out, float* rem)
{
    for (int64_t i = grid_stride_begin(); i < n; i += grid_stride())
        if (__ldg(fd + i) == kNoData) {
            out[i] = __int_as_float(0x7fc00000);
            rem[i] = __int_as_float(0x7fc00000);
        }
}

static bool path_engine_off()
{
    const char* e = getenv("LUE_GB300_ENGINE");
    return e && (e[0] == 'w' || e[0] == 's');
}

static int path_core_get(lue_gpu_topology* t, cudaStream_t stream, const PathCore** out)
{
    *out = nullptr;
    TopologyCore* core = t->core;
    if (core->stats.cycle_cells > 0) return LUE_GPU_OK;
    std::lock_guard<std::mutex> lock(core->stage_mutex);
    if (!core->paths && !core->paths_unavailable) {
        PathCore* pc = nullptr;
        const int rc = path_core_build(core, t->work_count, stream, &pc);
        if (rc == LUE_GPU_ERANGE) {
            core->paths_unavailable = true;
            return LUE_GPU_OK;
        }
        if (rc) return rc;
        core->paths = pc;
        core->bytes += pc->bytes;
    }
    *out = core->paths;
    return LUE_GPU_OK;
}

void path_buffers_free(lue_gpu_topology* t)
{
    cudaFree(t->path_maps);
    cudaFree(t->path_status);
    cudaFree(t->path_flag);
    t->path_maps = nullptr;
    t->path_status = nullptr;
    t->path_flag = nullptr;
}

constexpr int kPathMaxLevels = 256;

static int path_buffers(lue_gpu_topology* t, const PathCore* pc, cudaStream_t stream)
{
    if (t->path_maps) return LUE_GPU_OK;
    const char* what = "path engine buffers";
    const int64_t nt = std::max<int64_t>(pc->tiles, 1);
    int rc = LUE_GPU_OK;
    if ((rc = cuda_status(cudaMalloc(&t->path_maps, 2 * nt * sizeof(PMap)), what)) ||
        (rc = cuda_status(cudaMalloc(&t->path_status, (nt + kPathMaxLevels) * sizeof(int)), what)) ||
        (rc = cuda_status(cudaMalloc(&t->path_flag, 2 * sizeof(unsigned long long)), what)) ||
        (rc = cuda_status(cudaMemsetAsync(t->path_status, 0, (nt + kPathMaxLevels) * sizeof(int), stream), what))) {
        path_buffers_free(t);
        return rc;
    }
    t->path_epoch = 0;
    t->scratch_bytes += 2 * nt * (int64_t)sizeof(PMap) + (nt + kPathMaxLevels) * 4 + 16;
    return LUE_GPU_OK;
}

int path_prepare(lue_gpu_topology* t, cudaStream_t stream)
{
    const PathCore* pc = nullptr;
    return path_core_get(t, stream, &pc);
}

template <Rule R, int K>
static int path_run(lue_gpu_topology* t, const PathCore* pc, const float* a, float as, const float* b, float bs,
                    float* out, float* rem, cudaStream_t stream, const char* what)
{
    const TopologyCore* core = t->core;
    const int64_t n = core->n;
    const int levels = (int)pc->level_offsets.size() - 1;
    if (levels > kPathMaxLevels) return fail(LUE_GPU_ERANGE, std::string(what) + ": too many path levels");
    if (int rc = path_buffers(t, pc, stream)) return rc;
    const int64_t nt_max = std::max<int64_t>(pc->tiles, 1);
    int* tickets = t->path_status + nt_max;
    if (int rc = cuda_status(cudaMemsetAsync(t->path_flag, 0, 2 * sizeof(unsigned long long), stream), what))
        return rc;
    if (int rc = cuda_status(cudaMemsetAsync(tickets, 0, kPathMaxLevels * sizeof(int), stream), what)) return rc;
    k_path_no_data<<<grid_for(n, 256), 256, 0, stream>>>(core->fd, n, out, rem);
    PathCall p{pc->order, pc->light, a, as, b, bs, out, rem, t->lo, t->path_flag, core->cols};
    // test hooks: LUE_GB300_PATH_FREE_LONGEST (levels with longer paths use the look-back scan; 0: every
    // level) and LUE_GB300_PATH_POLLS (poll limit of a look-back wait; 0: every wait gives up at once,
    // and the walk engine redoes the call)
    int free_longest = kPathFreeLongest, polls = kPathPolls;
    if (const char* e = getenv("LUE_GB300_PATH_FREE_LONGEST")) free_longest = std::max(0, atoi(e));
    if (const char* e = getenv("LUE_GB300_PATH_POLLS")) polls = std::max(0, atoi(e));
    PMap* aggm = static_cast<PMap*>(t->path_maps);
    int launches = 1;
    for (int l = 0; l < levels; ++l) {
        const int64_t p0 = pc->level_offsets[l], p1 = pc->level_offsets[l + 1];
        const int per = path_per(p0, p1);
        const int64_t nt = path_level_tiles(p0, p1, per);
        if (nt == 0) continue;
        if (++t->path_epoch >= (1 << 29)) {  // status words of old launches could match again: clear them
            t->path_epoch = 1;
            if (int rc = cuda_status(cudaMemsetAsync(t->path_status, 0, nt_max * sizeof(int), stream), what))
                return rc;
        }
        const dim3 grid((unsigned)nt);
        if (pc->level_longest[l] <= free_longest) {  // CTAs cut at path tops: no waits
            const int64_t nf = (p1 - p0 + kPathThreads * per - 1) / (kPathThreads * per);
            const dim3 gf((unsigned)nf);
            switch (per * 2 + (l > 0)) {
                case 16: k_path_free<R, K, 8, false><<<gf, kPathThreads, 0, stream>>>(p, p0, p1); break;
                case 17: k_path_free<R, K, 8, true><<<gf, kPathThreads, 0, stream>>>(p, p0, p1); break;
                case 8: k_path_free<R, K, 4, false><<<gf, kPathThreads, 0, stream>>>(p, p0, p1); break;
                case 9: k_path_free<R, K, 4, true><<<gf, kPathThreads, 0, stream>>>(p, p0, p1); break;
                case 4: k_path_free<R, K, 2, false><<<gf, kPathThreads, 0, stream>>>(p, p0, p1); break;
                case 5: k_path_free<R, K, 2, true><<<gf, kPathThreads, 0, stream>>>(p, p0, p1); break;
                default: k_path_free<R, K, 1, true><<<gf, kPathThreads, 0, stream>>>(p, p0, p1); break;
            }
            ++launches;
            continue;
        }
        PathScan q{t->path_status, aggm, aggm + nt_max, tickets + l, t->path_epoch, polls};
        switch (per * 2 + (l > 0)) {
            case 16: k_path_level<R, K, 8, false><<<grid, kPathThreads, 0, stream>>>(p, p0, p1, q); break;
            case 17: k_path_level<R, K, 8, true><<<grid, kPathThreads, 0, stream>>>(p, p0, p1, q); break;
            case 8: k_path_level<R, K, 4, false><<<grid, kPathThreads, 0, stream>>>(p, p0, p1, q); break;
            case 9: k_path_level<R, K, 4, true><<<grid, kPathThreads, 0, stream>>>(p, p0, p1, q); break;
            case 4: k_path_level<R, K, 2, false><<<grid, kPathThreads, 0, stream>>>(p, p0, p1, q); break;
            case 5: k_path_level<R, K, 2, true><<<grid, kPathThreads, 0, stream>>>(p, p0, p1, q); break;
            default: k_path_level<R, K, 1, true><<<grid, kPathThreads, 0, stream>>>(p, p0, p1, q); break;
        }
        ++launches;
    }
    // +-inf inputs, or a wait of the scan that gave up: the walk engine redoes the whole call (as behind
    // the tile engine of accu)
    const unsigned long long* flag = t->path_flag;
    k_copy_words_if<<<grid_for(words_for(n), 256), 256, 0, stream>>>(reinterpret_cast<const uint32_t*>(core->count),
                                                                     t->work_count, words_for(n), flag);
    WalkGrid g{core->fd, core->count, t->work_count, core->rows, core->cols, n};
    RouteF32<R> v{core->upmask, a, as, b, bs, out, rem, t->lo, core->cols};
    k_walk_if<<<grid_for(n, 256), 256, 0, stream>>>(g, v, flag);
    count_launches(launches + 2);
    return cuda_status(cudaGetLastError(), what);
}

int path_route_f32(lue_gpu_topology* t, int rule, const float* a, float as, const float* b, float bs, float* out,
                   float* rem, cudaStream_t stream, bool* done)
{
    *done = false;
    if (path_engine_off()) return LUE_GPU_OK;
    if (rule != (int)Rule::threshold && rule != (int)Rule::capacity && rule != (int)Rule::fraction)
        return LUE_GPU_OK;
    const PathCore* pc = nullptr;
    if (int rc = path_core_get(t, stream, &pc)) return rc;
    if (!pc) return LUE_GPU_OK;
    *done = true;
    if (rule == (int)Rule::threshold)
        return path_run<Rule::threshold, kMaxPlus>(t, pc, a, as, b, bs, out, rem, stream, "accu_threshold_f32 (paths)");
    if (rule == (int)Rule::fraction)
        return path_run<Rule::fraction, kAffine>(t, pc, a, as, b, bs, out, rem, stream, "accu_fraction_f32 (paths)");
    return path_run<Rule::capacity, kMinPlus>(t, pc, a, as, b, bs, out, rem, stream, "accu_capacity_f32 (paths)");
}

}  // namespace lue_gb300
