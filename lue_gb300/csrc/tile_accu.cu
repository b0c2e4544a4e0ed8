// tile_accu.cu — tiled accu engine (see tile_accu.cuh): topology build and per-call kernels.
#include <algorithm>
#include <vector>

#include "tile_accu.cuh"
#include "topology.cuh"

namespace lue_gb300 {

typedef unsigned __int128 u128;

__device__ __forceinline__ u128 to_u128(uint4 v)
{
    return ((u128)v.w << 96) | ((u128)v.z << 64) | ((u128)v.y << 32) | (u128)v.x;
}
__device__ __forceinline__ uint4 from_u128(u128 v)
{
    return make_uint4((unsigned)v, (unsigned)(v >> 32), (unsigned)(v >> 64), (unsigned)(v >> 96));
}
__device__ __forceinline__ u128 shfl_up_u128(u128 v, int d)
{
    uint4 a = from_u128(v);
    a.x = __shfl_up_sync(0xffffffffu, a.x, d);
    a.y = __shfl_up_sync(0xffffffffu, a.y, d);
    a.z = __shfl_up_sync(0xffffffffu, a.z, d);
    a.w = __shfl_up_sync(0xffffffffu, a.w, d);
    return to_u128(a);
}
__device__ __forceinline__ u128 shfl_down_u128(u128 v, int d)
{
    uint4 a = from_u128(v);
    a.x = __shfl_down_sync(0xffffffffu, a.x, d);
    a.y = __shfl_down_sync(0xffffffffu, a.y, d);
    a.z = __shfl_down_sync(0xffffffffu, a.z, d);
    a.w = __shfl_down_sync(0xffffffffu, a.w, d);
    return to_u128(a);
}

constexpr u128 kPoison = (u128)1 << 96;                 // one no-data exit
constexpr u128 kValueMask = ((u128)1 << 96) - 1;

// Fixed-point scale: values are stored as round(v * 2^F).  F is chosen per call from an upper bound on
// the material total (in 2^-16 units) so that every prefix sum stays below 2^95.
__device__ __forceinline__ int fixed_point_bits(unsigned long long total_units)
{
    int bl = total_units ? 64 - __clzll((long long)total_units) : 0;
    int f = 111 - bl;
    return f > 100 ? 100 : (f < -100 ? -100 : f);
}

// |x| * 2^F rounded to nearest, as a 128-bit two's-complement integer with the sign of x.
__device__ __forceinline__ u128 float_to_fixed(float x, int F)
{
    unsigned bits = __float_as_uint(x);
    unsigned e8 = (bits >> 23) & 0xFFu;
    unsigned mant = (bits & 0x7FFFFFu) | (e8 ? 0x800000u : 0u);
    if (mant == 0) return 0;
    int s = (int)(e8 ? e8 : 1u) - 150 + F;  // value = mant * 2^(e - 150) * 2^F
    u128 m;
    if (s >= 0) {
        m = s >= 104 ? (u128)0 : ((u128)mant << s);
    } else if (s > -40) {
        unsigned long long mm = mant;
        m = (u128)((mm + (1ull << (-s - 1))) >> (-s));
    } else {
        m = 0;
    }
    return (bits >> 31) ? (u128)0 - m : m;
}

__device__ __forceinline__ u128 exit_value_fixed(float2 v, int F)
{
    if (isnan(v.x) || isnan(v.y)) return kPoison;
    return float_to_fixed(v.x, F) + float_to_fixed(v.y, F);
}

__device__ __forceinline__ double fixed_to_double(u128 v, int F)
{
    u128 a = v & kValueMask;
    double hi = (double)(unsigned long long)(a >> 64) * 18446744073709551616.0;
    double lo = (double)(unsigned long long)a;
    return ldexp(hi + lo, -F);
}

// ---------------------------------------------------------------------------------------------------
// Build
// ---------------------------------------------------------------------------------------------------

struct TileGeom {
    int64_t rows, cols, trows, tcols;
};

__device__ __forceinline__ int64_t tile_of(const TileGeom& g, int64_t r, int64_t c)
{
    return (r / kTile) * g.tcols + c / kTile;
}

// Exit bitmap: one 64-bit word per tile row; bit c set when that cell's flow leaves the tile but not
// the array.
__global__ void k_exit_bitmap(const uint8_t* __restrict__ fd, TileGeom g, uint64_t* bitmap)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.trows * g.tcols * kTile) return;
    int64_t tile = i / kTile;
    int rin = (int)(i % kTile);
    int64_t tr = tile / g.tcols, tc = tile % g.tcols;
    int64_t r = tr * kTile + rin;
    uint64_t m = 0;
    if (r < g.rows) {
        for (int cin = 0; cin < kTile; ++cin) {
            int64_t c = tc * kTile + cin;
            if (c >= g.cols) break;
            int dr, dc;
            uint8_t code = fd[r * g.cols + c];
            if (code == kNoData || !d8_offset(code, dr, dc)) continue;
            int64_t rd = r + dr, cd = c + dc;
            if (rd < 0 || rd >= g.rows || cd < 0 || cd >= g.cols) continue;
            if (rd / kTile != tr || cd / kTile != tc) m |= 1ull << cin;
        }
    }
    bitmap[i] = m;
}

__global__ void k_row_prefix(const uint64_t* bitmap, int64_t ntiles, uint16_t* rowpref, int32_t* count)
{
    int64_t tile = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tile >= ntiles) return;
    int acc = 0;
    for (int r = 0; r < kTile; ++r) {
        rowpref[tile * kTile + r] = (uint16_t)acc;
        acc += __popcll(bitmap[tile * kTile + r]);
    }
    count[tile] = acc;
}

__device__ __forceinline__ int32_t exit_id_of(const TileGeom& g, const int32_t* exit_base, const uint64_t* bitmap,
                                               const uint16_t* rowpref, int64_t r, int64_t c)
{
    int64_t tile = tile_of(g, r, c);
    int rin = (int)(r % kTile), cin = (int)(c % kTile);
    uint64_t word = bitmap[tile * kTile + rin];
    return exit_base[tile] + rowpref[tile * kTile + rin] + __popcll(word & ((1ull << cin) - 1ull));
}

__global__ void k_exit_list(TileGeom g, const uint64_t* bitmap, const uint16_t* rowpref, const int32_t* exit_base,
                            uint16_t* exit_local, uint32_t* exit_cell)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= g.trows * g.tcols * kTile) return;
    int64_t tile = i / kTile;
    int rin = (int)(i % kTile);
    int64_t tr = tile / g.tcols, tc = tile % g.tcols;
    uint64_t m = bitmap[i];
    int32_t id = exit_base[tile] + rowpref[i];
    while (m) {
        int cin = __ffsll((long long)m) - 1;
        m &= m - 1;
        exit_local[id] = (uint16_t)(rin * kTile + cin);
        exit_cell[id] = (uint32_t)((tr * kTile + rin) * g.cols + tc * kTile + cin);
        ++id;
    }
}

// Parent of every exit: follow the flow from its downstream cell through that cell's tile.
__global__ void k_exit_parent(const uint8_t* __restrict__ fd, TileGeom g, int64_t nexit, const uint32_t* exit_cell,
                              const int32_t* exit_base, const uint64_t* bitmap, const uint16_t* rowpref,
                              int32_t* parent, int32_t* nchild, int* error)
{
    int64_t y = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= nexit) return;
    int64_t cell = exit_cell[y];
    int64_t r = cell / g.cols, c = cell % g.cols;
    int dr, dc;
    d8_offset(fd[cell], dr, dc);
    r += dr;
    c += dc;
    int64_t tile = tile_of(g, r, c);
    int32_t p = -1;
    for (int step = 0; step <= kTileCells; ++step) {
        uint8_t code = fd[r * g.cols + c];
        if (code == kNoData || !d8_offset(code, dr, dc)) break;  // sink (or flow into no-data): root
        int64_t r2 = r + dr, c2 = c + dc;
        if (r2 < 0 || r2 >= g.rows || c2 < 0 || c2 >= g.cols) break;  // leaves the array: root
        if (tile_of(g, r2, c2) != tile) {
            p = exit_id_of(g, exit_base, bitmap, rowpref, r, c);
            break;
        }
        r = r2;
        c = c2;
        if (step == kTileCells) atomicExch(error, 1);  // cycle inside a tile (excluded by the caller)
    }
    parent[y] = p;
    if (p >= 0) atomicAdd(nchild + p, 1);
}

// Subtree sizes and depths of the exit forest, with the counter walk of walk.cuh on the coarse forest.
__global__ void k_exit_sizes(int64_t nexit, const int32_t* parent, const int32_t* nchild, int32_t* pending,
                             uint32_t* size, int32_t* depth)
{
    int64_t y = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= nexit || nchild[y] != 0) return;
    uint32_t s = 1;
    int32_t d = 1;
    for (;;) {
        int32_t p = parent[y];
        if (p < 0) return;
        atomicAdd(size + p, s);
        atomicMax(depth + p, d + 1);
        __threadfence();
        if (atomicSub(pending + p, 1) != 1) return;
        __threadfence();
        s = atomicAdd(size + p, 0u);
        d = atomicAdd(depth + p, 0);
        y = p;
    }
}

__global__ void k_exit_offsets(int64_t nexit, const int32_t* parent, const uint32_t* size, uint32_t* acc,
                               unsigned long long* root_acc, int64_t* D, int32_t* J)
{
    int64_t y = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= nexit) return;
    int32_t p = parent[y];
    if (p >= 0) {
        uint32_t off = atomicAdd(acc + p, size[y]);
        D[y] = (int64_t)off + size[y] - size[p];
    } else {
        unsigned long long off = atomicAdd(root_acc, (unsigned long long)size[y]);
        D[y] = (int64_t)off + size[y] - 1;
    }
    J[y] = p;
}

// Pointer jumping: pos(y) = pos(parent) + D(y) summed to the root.
__global__ void k_jump(int64_t nexit, const int64_t* D, const int32_t* J, int64_t* D2, int32_t* J2, int* more)
{
    int64_t y = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= nexit) return;
    int32_t j = J[y];
    if (j >= 0) {
        D2[y] = D[y] + D[j];
        int32_t jj = J[j];
        J2[y] = jj;
        if (jj >= 0) *more = 1;
    } else {
        D2[y] = D[y];
        J2[y] = -1;
    }
}

__global__ void k_exit_positions(int64_t nexit, const int64_t* D, const uint32_t* size, uint32_t* pos, uint32_t* start)
{
    int64_t y = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= nexit) return;
    pos[y] = (uint32_t)D[y];
    start[y] = (uint32_t)(D[y] - size[y] + 1);
}

// Every post-order position must be a distinct index in [0, nexit) with start <= pos: the per-call
// kernels scatter and gather with them, so the build refuses a forest that fails this check.
__global__ void k_check_positions(int64_t nexit, const uint32_t* pos, const uint32_t* start, int32_t* seen, int* error)
{
    int64_t y = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= nexit) return;
    uint32_t p = pos[y], s = start[y];
    if (p >= (uint64_t)nexit || s > p) {
        atomicExch(error, 1);
        return;
    }
    if (atomicAdd(seen + p, 1) != 0) atomicExch(error, 1);
}

__device__ __forceinline__ void halo_slot_coords(int s, int& hr, int& hc)
{
    if (s < kTile) { hr = -1; hc = s; }
    else if (s < 2 * kTile) { hr = kTile; hc = s - kTile; }
    else if (s < 3 * kTile) { hr = s - 2 * kTile; hc = -1; }
    else if (s < 4 * kTile) { hr = s - 3 * kTile; hc = kTile; }
    else if (s == 4 * kTile) { hr = -1; hc = -1; }
    else if (s == 4 * kTile + 1) { hr = -1; hc = kTile; }
    else if (s == 4 * kTile + 2) { hr = kTile; hc = -1; }
    else { hr = kTile; hc = kTile; }
}

__device__ __forceinline__ int halo_slot_of(int hr, int hc)
{
    if (hr == -1) return hc == -1 ? 4 * kTile : (hc == kTile ? 4 * kTile + 1 : hc);
    if (hr == kTile) return hc == -1 ? 4 * kTile + 2 : (hc == kTile ? 4 * kTile + 3 : kTile + hc);
    return hc == -1 ? 2 * kTile + hr : 3 * kTile + hr;
}

__global__ void k_halo_exits(const uint8_t* __restrict__ fd, TileGeom g, const int32_t* exit_base,
                             const uint64_t* bitmap, const uint16_t* rowpref, int32_t* halo_exit)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t ntiles = g.trows * g.tcols;
    if (i >= ntiles * kHaloSlots) return;
    int64_t tile = i / kHaloSlots;
    int s = (int)(i % kHaloSlots), hr, hc;
    halo_slot_coords(s, hr, hc);
    int64_t tr = tile / g.tcols, tc = tile % g.tcols;
    int64_t r = tr * kTile + hr, c = tc * kTile + hc;
    int32_t id = -1;
    if (r >= 0 && r < g.rows && c >= 0 && c < g.cols) {
        int dr, dc;
        uint8_t code = fd[r * g.cols + c];
        if (code != kNoData && d8_offset(code, dr, dc)) {
            int64_t rd = r + dr, cd = c + dc;
            if (rd >= 0 && rd < g.rows && cd >= 0 && cd < g.cols && tile_of(g, rd, cd) == tile)
                id = exit_id_of(g, exit_base, bitmap, rowpref, r, c);
        }
    }
    halo_exit[i] = id;
}

// ---------------------------------------------------------------------------------------------------
// Per call
// ---------------------------------------------------------------------------------------------------

constexpr uint16_t kNoCell = 0xFFFFu;

struct __align__(16) TileSmem {
    float hi[kTileCells];
    float lo[kTileCells];
    uint32_t cnt[kTileCells / 4];  // in-tile inflow counters, 4 per word
    uint16_t dsl[kTileCells];      // downstream cell inside the tile, or kNoCell
    uint16_t queue[kTileCells];    // cells in the order they become ready (each cell once)
    uint8_t up[kTileCells];        // in-tile upstream mask
    uint8_t fd[kHalo][kHalo + 2];  // flow direction with a one-cell halo (255 outside the array)
    int round_count[6];            // [0..2]: cells queued for the next rounds (a ring of three counters);
                                   // [3..5]: head, count and round handed back by the warp phase
};

// Load the flow direction with halo; fill in-tile upstream masks, counters and downstream indices, and
// queue the cells without in-tile inflow (the first round).  Returns the number of queued cells.
__device__ __forceinline__ int tile_prepare(TileSmem& sm, const uint8_t* __restrict__ fd, const TileGeom& g,
                                            int64_t tr, int64_t tc)
{
    const int t = threadIdx.x;
    for (int i = t; i < kHalo * kHalo; i += kTileThreads) {
        int hr = i / kHalo, hc = i % kHalo;
        int64_t r = tr * kTile + hr - 1, c = tc * kTile + hc - 1;
        sm.fd[hr][hc] = (r >= 0 && r < g.rows && c >= 0 && c < g.cols) ? __ldg(fd + r * g.cols + c) : kNoData;
    }
    if (t < 3) sm.round_count[t] = 0;
    __syncthreads();
    uint8_t* cnt8 = reinterpret_cast<uint8_t*>(sm.cnt);
    const int lane = t & 31;
#pragma unroll 4
    for (int k = 0; k < kTileCells / kTileThreads; ++k) {
        int i = t + k * kTileThreads;
        int rin = i >> 6, cin = i & 63;
        uint8_t code = sm.fd[rin + 1][cin + 1];
        unsigned mask = 0;
        uint16_t d = kNoCell;
        if (code != kNoData) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                int rn = rin + nb_dr(q), cn = cin + nb_dc(q);
                if (rn >= 0 && rn < kTile && cn >= 0 && cn < kTile && sm.fd[rn + 1][cn + 1] == nb_inflow_code(q))
                    mask |= 1u << q;
            }
            int dr, dc;
            if (d8_offset(code, dr, dc)) {
                int r2 = rin + dr, c2 = cin + dc;
                if (r2 >= 0 && r2 < kTile && c2 >= 0 && c2 < kTile && sm.fd[r2 + 1][c2 + 1] != kNoData)
                    d = (uint16_t)(r2 * kTile + c2);
            }
        }
        sm.up[i] = (uint8_t)mask;
        sm.dsl[i] = d;
        cnt8[i] = code == kNoData ? kNoData : (uint8_t)__popc(mask);
        // first round: valid cells without in-tile inflow (warp-aggregated queue appends)
        bool start = code != kNoData && mask == 0;
        unsigned ballot = __ballot_sync(0xffffffffu, start);
        int base = 0;
        if (lane == 0 && ballot) base = atomicAdd(&sm.round_count[0], __popc(ballot));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (start) sm.queue[base + __popc(ballot & ((1u << lane) - 1u))] = (uint16_t)i;
    }
    __syncthreads();
    return sm.round_count[0];
}

// Value of cell i: source(i) (hi/lo before the cell is done) + the sum of its in-tile upstream values,
// float-float; NaN or a negative source makes the cell NaN.  A sum that is not finite (+inf material)
// is recomputed plainly so that it keeps IEEE semantics.
__device__ __forceinline__ void tile_cell(TileSmem& sm, int i)
{
    const float x = sm.hi[i];
    float s = x, e = sm.lo[i];
    bool nan = isnan(x) || !(x >= 0.0f);
    unsigned m = sm.up[i];
    while (m) {
        int q = __ffs(m) - 1;
        m &= m - 1;
        int u = i + nb_dr(q) * kTile + nb_dc(q);
        float h = sm.hi[u], ts, te;
        nan |= isnan(h);
        two_sum(s, h, ts, te);
        s = ts;
        e = __fadd_rn(e, __fadd_rn(te, sm.lo[u]));
    }
    float hi = __fadd_rn(s, e);
    float lo = __fsub_rn(e, __fsub_rn(hi, s));
    if (!isfinite(hi)) {  // +inf upstream or material: plain float sum (inf stays inf)
        float p = x;
        unsigned mm = sm.up[i];
        while (mm) {
            int q = __ffs(mm) - 1;
            mm &= mm - 1;
            p += sm.hi[i + nb_dr(q) * kTile + nb_dc(q)];
        }
        hi = p;
        lo = 0.0f;
    }
    if (nan) {
        hi = __int_as_float(0x7fc00000);
        lo = 0.0f;
    }
    sm.hi[i] = hi;
    sm.lo[i] = lo;
}

// Finish item k of a round (if k < count) and queue its downstream cell when this was its last
// upstream cell.  All 32 lanes of the warp must call it (warp-aggregated queue appends).
__device__ __forceinline__ void tile_item(TileSmem& sm, int head, int count, int k, int* next, int next_base)
{
    const int lane = threadIdx.x & 31;
    int d = kNoCell;
    if (k < count) {
        int i = sm.queue[head + k];
        tile_cell(sm, i);
        d = sm.dsl[i];
    }
    bool ready = false;
    if (d != kNoCell) {
        unsigned shift = (unsigned)(d & 3) * 8u;
        unsigned old = atomicSub(sm.cnt + (d >> 2), 1u << shift);
        ready = ((old >> shift) & 0xFFu) == 1u;
    }
    unsigned ballot = __ballot_sync(0xffffffffu, ready);
    int base = 0;
    if (lane == 0 && ballot) base = atomicAdd(next, __popc(ballot));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (ready) sm.queue[next_base + base + __popc(ballot & ((1u << lane) - 1u))] = (uint16_t)d;
}

// Solve the tile in rounds: a round finishes every queued cell of that round (their upstream cells were
// finished in earlier rounds) and queues each downstream cell whose last upstream cell it finished.
// Rounds of more than 32 cells use the whole block (one barrier per round); runs of smaller rounds, the
// long tail of channel cells, are done by warp 0 alone with __syncwarp while the other warps wait at one
// barrier.  The counts of the next rounds live in a ring of three counters, so the count a round reads is
// never written during that round.
__device__ __forceinline__ void tile_solve(TileSmem& sm, int first_round)
{
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    int head = 0, count = first_round, r = 0;
    while (count > 0) {
        if (count > 32) {
            int* next = &sm.round_count[(r + 1) % 3];
            const int next_base = head + count;
            if (t == 0) sm.round_count[(r + 2) % 3] = 0;  // read by everyone two rounds ago
            for (int k0 = 0; k0 < count; k0 += kTileThreads) tile_item(sm, head, count, k0 + t, next, next_base);
            __syncthreads();
            head = next_base;
            count = *next;
            ++r;
        } else {
            if (warp == 0) {
                int wh = head, wc = count, wr = r;
                while (wc > 0 && wc <= 32) {
                    int* next = &sm.round_count[(wr + 1) % 3];
                    const int next_base = wh + wc;
                    if (lane == 0) sm.round_count[(wr + 2) % 3] = 0;
                    __syncwarp();
                    tile_item(sm, wh, wc, lane, next, next_base);
                    __syncwarp();
                    wh = next_base;
                    wc = *(volatile int*)next;
                    ++wr;
                }
                if (lane == 0) {
                    sm.round_count[3] = wh;
                    sm.round_count[4] = wc;
                    sm.round_count[5] = wr;
                }
            }
            __syncthreads();
            head = sm.round_count[3];
            count = sm.round_count[4];
            r = sm.round_count[5];
            __syncthreads();  // everyone has read the hand-over before a later warp phase rewrites it
        }
    }
}

// Pass 1: local accu inside each tile; local exit values to P (post-order); material total bound.
__global__ void __launch_bounds__(kTileThreads)
    k_tile_local(const uint8_t* __restrict__ fd, TileGeom g, const float* __restrict__ ext, float ext_s,
                 float* __restrict__ out, const int32_t* __restrict__ exit_base, const uint16_t* __restrict__ exit_local,
                 const uint32_t* __restrict__ exit_pos, float2* __restrict__ P, unsigned long long* block_total)
{
    __shared__ float warp_sum[kTileThreads / 32];
    __shared__ int warp_inf[kTileThreads / 32];
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TileSmem& sm = *reinterpret_cast<TileSmem*>(smem_raw);
    const int64_t tile = blockIdx.x;
    const int64_t tr = tile / g.tcols, tc = tile % g.tcols;
    const int t = threadIdx.x;
    FF sum{0.0f, 0.0f};
    bool inf = false;
#pragma unroll 4
    for (int k = 0; k < kTileCells / kTileThreads; ++k) {
        int i = t + k * kTileThreads;
        int64_t r = tr * kTile + (i >> 6), c = tc * kTile + (i & 63);
        float x = 0.0f;
        if (r < g.rows && c < g.cols) x = ext ? __ldg(ext + r * g.cols + c) : ext_s;
        sm.hi[i] = x;
        sm.lo[i] = 0.0f;
        if (isinf(x) && x > 0.0f) inf = true;
        else if (x > 0.0f) sum.add(x);
    }
    int first = tile_prepare(sm, fd, g, tr, tc);
    tile_solve(sm, first);
#pragma unroll 4
    for (int k = 0; k < kTileCells / kTileThreads; ++k) {
        int i = t + k * kTileThreads;
        int64_t r = tr * kTile + (i >> 6), c = tc * kTile + (i & 63);
        if (r < g.rows && c < g.cols)
            out[r * g.cols + c] = sm.fd[(i >> 6) + 1][(i & 63) + 1] == kNoData ? __int_as_float(0x7fc00000) : sm.hi[i];
    }
    for (int32_t e = exit_base[tile] + t; e < exit_base[tile + 1]; e += kTileThreads) {
        int loc = exit_local[e];
        P[exit_pos[e]] = make_float2(sm.hi[loc], sm.lo[loc]);
    }
    // upper bound of this tile's material total, in 2^-16 units; ~0 marks +inf or overflow
    float s = sum.hi + sum.lo;
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    unsigned any_inf = __any_sync(0xffffffffu, inf);
    if ((t & 31) == 0) {
        warp_sum[t >> 5] = s;
        warp_inf[t >> 5] = any_inf ? 1 : 0;
    }
    __syncthreads();
    if (t == 0) {
        double tot = 0.0;
        int bad = 0;
        for (int w = 0; w < kTileThreads / 32; ++w) {
            tot += (double)warp_sum[w];
            bad |= warp_inf[w];
        }
        double units = tot * 1.0001 * 65536.0 + 64.0;
        block_total[tile] = (bad || !(units < 1.0e18)) ? ~0ull : (unsigned long long)units;
    }
}

// Sum of the per-tile bounds: total[0] = bound in 2^-16 units, total[1] != 0 when the tile engine must
// hand the call to the walk engine (+inf material, or a total beyond the fixed-point range).
__global__ void __launch_bounds__(1024) k_total(const unsigned long long* block_total, int64_t ntiles,
                                                unsigned long long* total)
{
    __shared__ unsigned long long part[32];
    __shared__ int badw[32];
    unsigned long long s = 0;
    double chk = 0.0;  // the same sum in double: detects a total beyond the fixed-point range
    int bad = 0;
    for (int64_t i = threadIdx.x; i < ntiles; i += blockDim.x) {
        unsigned long long v = block_total[i];
        if (v == ~0ull) {
            bad = 1;
        } else {
            s += v;
            chk += (double)v;
        }
    }
    if (chk >= 1.0e18) bad = 1;
    for (int off = 16; off > 0; off >>= 1) {
        s += __shfl_down_sync(0xffffffffu, s, off);
        chk += __shfl_down_sync(0xffffffffu, chk, off);
        bad |= __shfl_down_sync(0xffffffffu, bad, off);
    }
    if (chk >= 1.0e18) bad = 1;
    if ((threadIdx.x & 31) == 0) {
        part[threadIdx.x >> 5] = s;
        badw[threadIdx.x >> 5] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long tot = 0;
        double check = 0.0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) {
            tot += part[w];
            check += (double)part[w];
            bad |= badw[w];
        }
        // parts that wrapped cannot pass here: every part is < 1e18 or already flagged
        if (check >= 1.0e18) bad = 1;
        total[0] = tot;
        total[1] = bad ? 1ull : 0ull;
    }
}

constexpr int kScanItems = 16;
constexpr int kScanBlock = kTileThreads * kScanItems;

__device__ __forceinline__ u128 block_exclusive_u128(u128 v, u128* warp_tot, u128& block_total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    u128 x = v;
    for (int d = 1; d < 32; d <<= 1) {
        u128 y = shfl_up_u128(x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        u128 w = lane < kTileThreads / 32 ? warp_tot[lane] : (u128)0;
        for (int d = 1; d < 32; d <<= 1) {
            u128 y = shfl_up_u128(w, d);
            if (lane >= d) w += y;
        }
        if (lane < kTileThreads / 32) warp_tot[lane] = w;
    }
    __syncthreads();
    u128 before = warp ? warp_tot[warp - 1] : (u128)0;
    block_total = warp_tot[kTileThreads / 32 - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(kTileThreads)
    k_scan_reduce(const float2* __restrict__ P, int64_t n, const unsigned long long* total, uint4* block_sums)
{
    __shared__ u128 warp_tot[kTileThreads / 32];
    if (total[1]) return;
    const int F = fixed_point_bits(total[0]);
    int64_t base = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanItems;
    u128 s = 0;
    for (int k = 0; k < kScanItems; ++k)
        if (base + k < n) s += exit_value_fixed(P[base + k], F);
    u128 bt;
    block_exclusive_u128(s, warp_tot, bt);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = from_u128(bt);
}

__global__ void __launch_bounds__(kTileThreads) k_scan_blocks(uint4* block_sums, int64_t nblocks, const unsigned long long* total)
{
    __shared__ u128 warp_tot[kTileThreads / 32];
    if (total[1]) return;
    u128 carry = 0;
    for (int64_t b0 = 0; b0 < nblocks; b0 += kTileThreads) {
        int64_t b = b0 + threadIdx.x;
        u128 v = b < nblocks ? to_u128(block_sums[b]) : (u128)0;
        u128 bt;
        u128 ex = block_exclusive_u128(v, warp_tot, bt);
        if (b < nblocks) block_sums[b] = from_u128(carry + ex);
        carry += bt;
    }
}

__global__ void __launch_bounds__(kTileThreads)
    k_scan_final(const float2* __restrict__ P, int64_t n, const unsigned long long* total,
                 const uint4* __restrict__ block_sums, uint4* __restrict__ S)
{
    __shared__ u128 warp_tot[kTileThreads / 32];
    if (total[1]) return;
    const int F = fixed_point_bits(total[0]);
    int64_t base = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanItems;
    u128 v[kScanItems];
    u128 s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        v[k] = base + k < n ? exit_value_fixed(P[base + k], F) : (u128)0;
        s += v[k];
    }
    u128 bt;
    u128 run = to_u128(block_sums[blockIdx.x]) + block_exclusive_u128(s, warp_tot, bt);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        run += v[k];
        if (base + k < n) S[base + k] = from_u128(run);
    }
}

__global__ void k_exit_sums(int64_t n, const uint32_t* __restrict__ pos, const uint32_t* __restrict__ start,
                            const uint4* __restrict__ S, uint4* __restrict__ A, const unsigned long long* total)
{
    int64_t y = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= n || total[1]) return;
    uint32_t st = start[y];
    u128 a = to_u128(S[pos[y]]) - (st ? to_u128(S[st - 1]) : (u128)0);
    A[y] = from_u128(a);
}

// Pass 3: add the inflow entering each tile to every cell downstream of it.
__global__ void __launch_bounds__(kTileThreads)
    k_tile_fixup(const uint8_t* __restrict__ fd, TileGeom g, float* __restrict__ out,
                 const int32_t* __restrict__ halo_exit, const uint4* __restrict__ A, const unsigned long long* total)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TileSmem& sm = *reinterpret_cast<TileSmem*>(smem_raw);
    if (total[1]) return;
    const int F = fixed_point_bits(total[0]);
    const int64_t tile = blockIdx.x;
    const int64_t tr = tile / g.tcols, tc = tile % g.tcols;
    const int t = threadIdx.x;
    for (int k = 0; k < kTileCells / kTileThreads; ++k) {
        sm.hi[t + k * kTileThreads] = 0.0f;
        sm.lo[t + k * kTileThreads] = 0.0f;
    }
    int first = tile_prepare(sm, fd, g, tr, tc);
    // sources: border cells gather the exact subtree sums of the halo exits draining into them
    if (t < 4 * kTile - 4) {
        int rin, cin;
        if (t < kTile) { rin = 0; cin = t; }
        else if (t < 2 * kTile) { rin = kTile - 1; cin = t - kTile; }
        else if (t < 3 * kTile - 2) { rin = t - 2 * kTile + 1; cin = 0; }
        else { rin = t - (3 * kTile - 2) + 1; cin = kTile - 1; }
        if (sm.fd[rin + 1][cin + 1] != kNoData) {
            u128 s = 0;
            bool any = false;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                int hr = rin + nb_dr(q), hc = cin + nb_dc(q);
                if (hr >= 0 && hr < kTile && hc >= 0 && hc < kTile) continue;  // in-tile neighbour
                if (sm.fd[hr + 1][hc + 1] != nb_inflow_code(q)) continue;
                int32_t id = halo_exit[tile * kHaloSlots + halo_slot_of(hr, hc)];
                if (id >= 0) {
                    s += to_u128(A[id]);
                    any = true;
                }
            }
            if (any) {
                int i = rin * kTile + cin;
                if ((s >> 96) != 0) {
                    sm.hi[i] = __int_as_float(0x7fc00000);
                } else {
                    double d = fixed_to_double(s, F);
                    float h = __double2float_rn(d);
                    sm.hi[i] = h;
                    sm.lo[i] = __double2float_rn(d - (double)h);
                }
            }
        }
    }
    __syncthreads();
    tile_solve(sm, first);
#pragma unroll 4
    for (int k = 0; k < kTileCells / kTileThreads; ++k) {
        int i = t + k * kTileThreads;
        float h = sm.hi[i], l = sm.lo[i];
        if (h == 0.0f && l == 0.0f) continue;
        int64_t r = tr * kTile + (i >> 6), c = tc * kTile + (i & 63);
        if (r >= g.rows || c >= g.cols || sm.fd[(i >> 6) + 1][(i & 63) + 1] == kNoData) continue;
        float* o = out + r * g.cols + c;
        if (isnan(h)) {
            *o = __int_as_float(0x7fc00000);
        } else {
            FF v{*o, 0.0f};
            v.add(h, l);
            v.normalise();
            *o = v.hi;
        }
    }
}

// ---------------------------------------------------------------------------------------------------
// Host
// ---------------------------------------------------------------------------------------------------

static inline unsigned blocks_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

int tile_core_build(TopologyCore* core, cudaStream_t stream)
{
    auto* tc = new (std::nothrow) TileCore();
    if (!tc) return fail(LUE_GPU_ENOMEM, "tile topology: host allocation");
    TileGeom g{core->rows, core->cols, (core->rows + kTile - 1) / kTile, (core->cols + kTile - 1) / kTile};
    tc->trows = g.trows;
    tc->tcols = g.tcols;
    tc->ntiles = g.trows * g.tcols;
    const int64_t nt = tc->ntiles;
    uint64_t* bitmap = nullptr;
    uint16_t* rowpref = nullptr;
    int32_t* count = nullptr;
    uint32_t* exit_cell = nullptr;
    int32_t *parent = nullptr, *nchild = nullptr, *pending = nullptr, *depth = nullptr, *J = nullptr, *J2 = nullptr;
    uint32_t *size = nullptr, *acc = nullptr;
    int64_t *D = nullptr, *D2 = nullptr;
    unsigned long long* root_acc = nullptr;
    int* flag = nullptr;
    std::vector<int32_t> hcount(nt), hbase(nt + 1);
    int rc = 0, herr = 0;
    int64_t E = 0;
#define TRY(call, what) \
    if ((rc = cuda_status((call), what))) goto error
    TRY(cudaMalloc(&bitmap, nt * kTile * sizeof(uint64_t)), "tile bitmap");
    TRY(cudaMalloc(&rowpref, nt * kTile * sizeof(uint16_t)), "tile row prefix");
    TRY(cudaMalloc(&count, nt * sizeof(int32_t)), "tile exit count");
    TRY(cudaMalloc(&tc->exit_base, (nt + 1) * sizeof(int32_t)), "tile exit base");
    TRY(cudaMalloc(&flag, 2 * sizeof(int)), "tile flag");
    TRY(cudaMemsetAsync(flag, 0, 2 * sizeof(int), stream), "memset");
    k_exit_bitmap<<<blocks_for(nt * kTile, 256), 256, 0, stream>>>(core->fd, g, bitmap);
    k_row_prefix<<<blocks_for(nt, 256), 256, 0, stream>>>(bitmap, nt, rowpref, count);
    TRY(cudaGetLastError(), "tile build");
    TRY(cudaMemcpyAsync(hcount.data(), count, nt * sizeof(int32_t), cudaMemcpyDeviceToHost, stream), "tile counts");
    TRY(cudaStreamSynchronize(stream), "tile counts");
    hbase[0] = 0;
    for (int64_t i = 0; i < nt; ++i) {
        if ((int64_t)hbase[i] + hcount[i] > INT32_MAX) {
            rc = fail(LUE_GPU_ERANGE, "tile topology: too many exits");
            goto error;
        }
        hbase[i + 1] = hbase[i] + hcount[i];
    }
    E = hbase[nt];
    tc->nexit = E;
    TRY(cudaMemcpyAsync(tc->exit_base, hbase.data(), (nt + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, stream),
        "tile exit base");
    TRY(cudaMalloc(&tc->exit_local, std::max<int64_t>(E, 1) * sizeof(uint16_t)), "exit local");
    TRY(cudaMalloc(&tc->exit_pos, std::max<int64_t>(E, 1) * sizeof(uint32_t)), "exit pos");
    TRY(cudaMalloc(&tc->exit_start, std::max<int64_t>(E, 1) * sizeof(uint32_t)), "exit start");
    TRY(cudaMalloc(&tc->halo_exit, nt * kHaloSlots * sizeof(int32_t)), "halo exits");
    tc->bytes = (nt + 1) * 4 + E * 10 + nt * kHaloSlots * 4;
    if (E > 0) {
        TRY(cudaMalloc(&exit_cell, E * sizeof(uint32_t)), "exit cell");
        TRY(cudaMalloc(&parent, E * sizeof(int32_t)), "exit parent");
        TRY(cudaMalloc(&nchild, E * sizeof(int32_t)), "exit children");
        TRY(cudaMalloc(&pending, E * sizeof(int32_t)), "exit pending");
        TRY(cudaMalloc(&depth, E * sizeof(int32_t)), "exit depth");
        TRY(cudaMalloc(&size, E * sizeof(uint32_t)), "exit size");
        TRY(cudaMalloc(&acc, E * sizeof(uint32_t)), "exit acc");
        TRY(cudaMalloc(&D, E * sizeof(int64_t)), "exit D");
        TRY(cudaMalloc(&D2, E * sizeof(int64_t)), "exit D2");
        TRY(cudaMalloc(&J, E * sizeof(int32_t)), "exit J");
        TRY(cudaMalloc(&J2, E * sizeof(int32_t)), "exit J2");
        TRY(cudaMalloc(&root_acc, sizeof(unsigned long long)), "root acc");
        k_exit_list<<<blocks_for(nt * kTile, 256), 256, 0, stream>>>(g, bitmap, rowpref, tc->exit_base, tc->exit_local,
                                                                     exit_cell);
        TRY(cudaMemsetAsync(nchild, 0, E * sizeof(int32_t), stream), "memset");
        k_exit_parent<<<blocks_for(E, 256), 256, 0, stream>>>(core->fd, g, E, exit_cell, tc->exit_base, bitmap, rowpref,
                                                             parent, nchild, flag);
        TRY(cudaMemcpyAsync(pending, nchild, E * sizeof(int32_t), cudaMemcpyDeviceToDevice, stream), "copy");
        {
            std::vector<uint32_t> ones(E, 1u);
            TRY(cudaMemcpyAsync(size, ones.data(), E * sizeof(uint32_t), cudaMemcpyHostToDevice, stream), "sizes");
            TRY(cudaMemsetAsync(depth, 0, E * sizeof(int32_t), stream), "memset");
            k_exit_sizes<<<blocks_for(E, 256), 256, 0, stream>>>(E, parent, nchild, pending, size, depth);
            TRY(cudaMemsetAsync(acc, 0, E * sizeof(uint32_t), stream), "memset");
            TRY(cudaMemsetAsync(root_acc, 0, sizeof(unsigned long long), stream), "memset");
            k_exit_offsets<<<blocks_for(E, 256), 256, 0, stream>>>(E, parent, size, acc, root_acc, D, J);
            TRY(cudaGetLastError(), "exit forest");
            TRY(cudaStreamSynchronize(stream), "exit forest");  // `ones` must outlive the copy
        }
        for (int round = 0; round < 40; ++round) {
            int more = 0;
            TRY(cudaMemsetAsync(flag + 1, 0, sizeof(int), stream), "memset");
            k_jump<<<blocks_for(E, 256), 256, 0, stream>>>(E, D, J, D2, J2, flag + 1);
            std::swap(D, D2);
            std::swap(J, J2);
            TRY(cudaMemcpyAsync(&more, flag + 1, sizeof(int), cudaMemcpyDeviceToHost, stream), "jump flag");
            TRY(cudaStreamSynchronize(stream), "jump");
            if (!more) {
                // one more round folds the last parents in (more == 0 means every J2 is now a root)
                k_jump<<<blocks_for(E, 256), 256, 0, stream>>>(E, D, J, D2, J2, flag + 1);
                std::swap(D, D2);
                std::swap(J, J2);
                break;
            }
        }
        k_exit_positions<<<blocks_for(E, 256), 256, 0, stream>>>(E, D, size, tc->exit_pos, tc->exit_start);
        TRY(cudaMemsetAsync(nchild, 0, E * sizeof(int32_t), stream), "memset");
        k_check_positions<<<blocks_for(E, 256), 256, 0, stream>>>(E, tc->exit_pos, tc->exit_start, nchild, flag);
        {
            int32_t hmax = 0;
            std::vector<int32_t> hd(E);
            TRY(cudaMemcpyAsync(hd.data(), depth, E * sizeof(int32_t), cudaMemcpyDeviceToHost, stream), "depth");
            TRY(cudaStreamSynchronize(stream), "depth");
            for (int32_t v : hd) hmax = std::max(hmax, v);
            tc->max_depth = std::max<int64_t>(hmax, 1);
        }
    }
    k_halo_exits<<<blocks_for(nt * kHaloSlots, 256), 256, 0, stream>>>(core->fd, g, tc->exit_base, bitmap, rowpref,
                                                                      tc->halo_exit);
    TRY(cudaGetLastError(), "tile build");
    TRY(cudaMemcpyAsync(&herr, flag, sizeof(int), cudaMemcpyDeviceToHost, stream), "tile flag");
    TRY(cudaStreamSynchronize(stream), "tile build");
    if (herr) {
        rc = fail(LUE_GPU_EINVAL, "tile topology: cycle inside a tile or inconsistent exit forest");
        goto error;
    }
    cudaFree(bitmap);
    cudaFree(rowpref);
    cudaFree(count);
    cudaFree(exit_cell);
    cudaFree(parent);
    cudaFree(nchild);
    cudaFree(pending);
    cudaFree(depth);
    cudaFree(size);
    cudaFree(acc);
    cudaFree(D);
    cudaFree(D2);
    cudaFree(J);
    cudaFree(J2);
    cudaFree(root_acc);
    cudaFree(flag);
    core->tiles = tc;
    return LUE_GPU_OK;
error:
    cudaFree(bitmap);
    cudaFree(rowpref);
    cudaFree(count);
    cudaFree(exit_cell);
    cudaFree(parent);
    cudaFree(nchild);
    cudaFree(pending);
    cudaFree(depth);
    cudaFree(size);
    cudaFree(acc);
    cudaFree(D);
    cudaFree(D2);
    cudaFree(J);
    cudaFree(J2);
    cudaFree(root_acc);
    cudaFree(flag);
    tile_core_free(tc);
    return rc;
#undef TRY
}

void tile_core_free(TileCore* tc)
{
    if (!tc) return;
    cudaFree(tc->exit_base);
    cudaFree(tc->exit_local);
    cudaFree(tc->exit_pos);
    cudaFree(tc->exit_start);
    cudaFree(tc->halo_exit);
    delete tc;
}

int tile_scratch_alloc(const TileCore* tc, TileScratch* s)
{
    const int64_t E = std::max<int64_t>(tc->nexit, 1);
    const int64_t nb = (E + kScanBlock - 1) / kScanBlock;
    int rc = 0;
    if ((rc = cuda_status(cudaMalloc(&s->P, E * sizeof(float2)), "tile scratch"))) return rc;
    if ((rc = cuda_status(cudaMalloc(&s->S, E * sizeof(uint4)), "tile scratch"))) return rc;
    if ((rc = cuda_status(cudaMalloc(&s->A, E * sizeof(uint4)), "tile scratch"))) return rc;
    if ((rc = cuda_status(cudaMalloc(&s->block_sums, nb * sizeof(uint4)), "tile scratch"))) return rc;
    if ((rc = cuda_status(cudaMalloc(&s->total, 2 * sizeof(unsigned long long)), "tile scratch"))) return rc;
    if ((rc = cuda_status(cudaMalloc(&s->block_total, tc->ntiles * sizeof(unsigned long long)), "tile scratch")))
        return rc;
    s->bytes = E * (8 + 16 + 16) + nb * 16 + 16 + tc->ntiles * 8;
    return LUE_GPU_OK;
}

void tile_scratch_free(TileScratch* s)
{
    cudaFree(s->P);
    cudaFree(s->S);
    cudaFree(s->A);
    cudaFree(s->block_sums);
    cudaFree(s->total);
    cudaFree(s->block_total);
    *s = TileScratch{};
}

// accu (float32) on the tile engine.  Returns LUE_GPU_OK with `fallback` set on the device when the
// material holds +inf or its total is beyond the fixed-point range; the caller then runs the walk
// engine, guarded by that flag.
int tile_accu_f32(const TopologyCore* core, TileScratch* s, const float* ext, float ext_s, float* out,
                  cudaStream_t stream)
{
    const TileCore* tc = core->tiles;
    TileGeom g{core->rows, core->cols, tc->trows, tc->tcols};
    const size_t smem = sizeof(TileSmem);
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(k_tile_local, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaFuncSetAttribute(k_tile_fixup, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        configured = true;
    }
    k_tile_local<<<(unsigned)tc->ntiles, kTileThreads, smem, stream>>>(core->fd, g, ext, ext_s, out, tc->exit_base,
                                                                      tc->exit_local, tc->exit_pos, s->P,
                                                                      s->block_total);
    k_total<<<1, 1024, 0, stream>>>(s->block_total, tc->ntiles, s->total);
    count_launches(2);
    const int64_t E = tc->nexit;
    if (E > 0) {
        const int64_t nb = (E + kScanBlock - 1) / kScanBlock;
        k_scan_reduce<<<(unsigned)nb, kTileThreads, 0, stream>>>(s->P, E, s->total, s->block_sums);
        k_scan_blocks<<<1, kTileThreads, 0, stream>>>(s->block_sums, nb, s->total);
        k_scan_final<<<(unsigned)nb, kTileThreads, 0, stream>>>(s->P, E, s->total, s->block_sums, s->S);
        k_exit_sums<<<blocks_for(E, 256), 256, 0, stream>>>(E, tc->exit_pos, tc->exit_start, s->S, s->A, s->total);
        k_tile_fixup<<<(unsigned)tc->ntiles, kTileThreads, smem, stream>>>(core->fd, g, out, tc->halo_exit, s->A,
                                                                           s->total);
        count_launches(5);
    }
    return cuda_status(cudaGetLastError(), "accu_f32 (tiles)");
}

}  // namespace lue_gb300
