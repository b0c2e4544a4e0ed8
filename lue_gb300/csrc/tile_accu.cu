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

// |x| * 2^F rounded to nearest (ties up; 0 below 2^-40, 0 from 2^128 up), as a 128-bit two's-complement
// integer with the sign of x.  Built from 32-bit words: the 24-bit mantissa shifted by s & 31 spans two
// words, placed at word s >> 5, so no 128-bit variable shift is needed.
__device__ __forceinline__ u128 float_to_fixed(float x, int F)
{
    const unsigned bits = __float_as_uint(x);
    const unsigned e8 = (bits >> 23) & 0xFFu;
    const unsigned mant = (bits & 0x7FFFFFu) | (e8 ? 0x800000u : 0u);
    const int s = (int)(e8 ? e8 : 1u) - 150 + F;  // value = mant * 2^(e - 150) * 2^F
    unsigned long long lo = 0, hi = 0;
    if (s >= 0) {
        if (s < 104) {
            const int k = s >> 5;
            const unsigned b = (unsigned)s & 31u;
            const unsigned w0 = mant << b, w1 = __funnelshift_l(mant, 0u, b);
            const unsigned long long pair = ((unsigned long long)w1 << 32) | w0;
            const unsigned long long up = (unsigned long long)w0 << 32;
            lo = k == 0 ? pair : (k == 1 ? up : 0ull);
            hi = k == 1 ? (unsigned long long)w1 : (k == 2 ? pair : (k == 3 ? up : 0ull));
        }
    } else if (s > -40) {
        lo = ((unsigned long long)mant + (1ull << (-s - 1))) >> (-s);
    }
    if (bits >> 31) {  // two's complement
        hi = ~hi + (lo == 0 ? 1ull : 0ull);
        lo = 0ull - lo;
    }
    return ((u128)hi << 64) | lo;
}

__device__ __forceinline__ u128 exit_value_fixed(float2 v, int F)
{
    if (isnan(v.x) || isnan(v.y)) return kPoison;
    return float_to_fixed(v.x, F) + float_to_fixed(v.y, F);
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
// Build: per-tile flow forests in post-order
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
    uint8_t border[kBorderCells];  // per border cell: outside neighbours draining into it
    int round_count[3];            // cells queued for the next rounds (a ring of three counters)
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

// In-tile linear offset of neighbour q (NW N NE W E SW S SE).
__device__ __forceinline__ int tile_nb_offset(int q)
{
    static_assert(kTile == 64, "neighbour offsets are packed for 64-cell rows");
    // -65 -64 -63 -1 +1 +63 +64 +65 as signed bytes
    return (int)(signed char)(unsigned)(0x41403F01FFC1C0BFull >> (8 * q));
}

// Neighbour index (0..7, NW N NE W E SW S SE) of in-tile cell c as seen from its downstream cell d.
__device__ __forceinline__ int nb_index_from(int d, int c)
{
    const int idx = ((c >> 6) - (d >> 6) + 1) * 3 + ((c & 63) - (d & 63) + 1);
    return idx < 4 ? idx : idx - 1;
}

// Border cell b (0..251: N row, S row, W column, E column without corners) of a tile.
__device__ __forceinline__ void border_cell(int b, int& rin, int& cin)
{
    if (b < kTile) { rin = 0; cin = b; }
    else if (b < 2 * kTile) { rin = kTile - 1; cin = b - kTile; }
    else if (b < 3 * kTile - 2) { rin = b - 2 * kTile + 1; cin = 0; }
    else { rin = b - (3 * kTile - 2) + 1; cin = kTile - 1; }
}

// Exclusive prefix of one int per thread over the block; `total` gets the block sum.
__device__ __forceinline__ int block_exclusive_int(int v, int* warp_tot, int& total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    int before = 0;
    total = 0;
    for (int w = 0; w < kTileThreads / 32; ++w) {
        const int s = warp_tot[w];
        before += w < warp ? s : 0;
        total += s;
    }
    __syncthreads();  // warp_tot may be reused
    return before + x - v;
}

// Build: the flow forest of one tile (CTA per tile), in post-order.  A cell's in-tile upstream cells
// (its subtree) get the positions start .. pos - 1 and the cell itself pos, so that the accu of any cell
// is the difference of two prefix sums over the material laid out in post-order.  Cells with a no-data
// flow direction (or outside the array) take the positions after the valid cells, flagged kNoValue.
// Also: each exit's scan slots (its own, and the one before its subtree), and, per border cell, which
// outside neighbours drain into it.
__global__ void __launch_bounds__(kTileThreads)
    k_tile_forest(const uint8_t* __restrict__ fd, TileGeom g, const int32_t* __restrict__ exit_base,
                  const uint16_t* __restrict__ exit_local, uint16_t* cell_at, uint16_t* prev_at,
                  uint32_t* exit_span, uint8_t* border_in, int* error)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TileSmem& sm = *reinterpret_cast<TileSmem*>(smem_raw);
    const int64_t tr = blockIdx.y, tc = blockIdx.x;  // grid = (tile columns, tile rows)
    const int64_t tile = tr * g.tcols + tc;
    const int t = threadIdx.x, lane = t & 31;
    uint16_t* rstart = reinterpret_cast<uint16_t*>(sm.hi);  // <= 4097 round starts
    uint16_t* sz = reinterpret_cast<uint16_t*>(sm.lo);      // subtree size
    uint16_t* st = sz + kTileCells;                         // first position of the subtree
    int head = 0, count = tile_prepare(sm, fd, g, tr, tc), r = 0;
    // rounds: a round holds the cells whose in-tile upstream cells are all in earlier rounds
    while (count > 0) {
        int* next = &sm.round_count[(r + 1) % 3];
        const int next_base = head + count;
        if (t == 0) {
            rstart[r] = (uint16_t)head;
            sm.round_count[(r + 2) % 3] = 0;  // read by everyone two rounds ago
        }
        for (int k0 = 0; k0 < count; k0 += kTileThreads) {
            int k = k0 + t, d = kNoCell;
            if (k < count) d = sm.dsl[sm.queue[head + k]];
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
        __syncthreads();
        head = next_base;
        count = *next;
        ++r;
    }
    const int rounds = r, nvalid = head;
    if (t == 0) rstart[rounds] = (uint16_t)nvalid;
    // per border cell, the neighbours outside the tile that drain into it
    for (int b = t; b < kBorderCells; b += kTileThreads) {
        int rin, cin;
        border_cell(b, rin, cin);
        unsigned outside = 0;
        if (sm.fd[rin + 1][cin + 1] != kNoData) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int hr = rin + nb_dr(q), hc = cin + nb_dc(q);
                if (hr >= 0 && hr < kTile && hc >= 0 && hc < kTile) continue;
                if (sm.fd[hr + 1][hc + 1] == nb_inflow_code(q)) outside |= 1u << q;
            }
        }
        border_in[tile * kBorderCells + b] = (uint8_t)outside;
    }
    __syncthreads();
    // subtree sizes, upstream first
    for (int q = 0; q < rounds; ++q) {
        for (int k = rstart[q] + t; k < rstart[q + 1]; k += kTileThreads) {
            const int i = sm.queue[k];
            unsigned m = sm.up[i];
            int size = 1;
            while (m) {
                size += sz[i + tile_nb_offset(__ffs(m) - 1)];
                m &= m - 1;
            }
            sz[i] = (uint16_t)size;
        }
        __syncthreads();
    }
    // roots (valid cells without an in-tile downstream cell) and invalid cells, in cell order: thread t
    // owns cells 16 t .. 16 t + 15
    int* wt = reinterpret_cast<int*>(sm.cnt);  // the counters are free after the rounds
    int root_sum = 0, invalid = 0;
    for (int j = 0; j < 16; ++j) {
        const int i = 16 * t + j;
        if (sm.fd[(i >> 6) + 1][(i & 63) + 1] == kNoData) ++invalid;
        else if (sm.dsl[i] == kNoCell) root_sum += sz[i];
    }
    int root_total, invalid_total;
    int root_base = block_exclusive_int(root_sum, wt, root_total);
    int invalid_base = root_total + block_exclusive_int(invalid, wt, invalid_total);
    for (int j = 0; j < 16; ++j) {
        const int i = 16 * t + j;
        if (sm.fd[(i >> 6) + 1][(i & 63) + 1] == kNoData) {
            st[i] = (uint16_t)invalid_base++;
            sz[i] = 1;
        } else if (sm.dsl[i] == kNoCell) {
            st[i] = (uint16_t)root_base;
            root_base += sz[i];
        }
    }
    __syncthreads();
    // the other cells, downstream first: after the siblings that come before them
    for (int q = rounds - 1; q >= 0; --q) {
        for (int k = rstart[q] + t; k < rstart[q + 1]; k += kTileThreads) {
            const int i = sm.queue[k], d = sm.dsl[i];
            if (d == kNoCell) continue;
            unsigned m = sm.up[d] & ((1u << nb_index_from(d, i)) - 1u);
            int o = st[d];
            while (m) {
                o += sz[d + tile_nb_offset(__ffs(m) - 1)];
                m &= m - 1;
            }
            st[i] = (uint16_t)o;
        }
        __syncthreads();
    }
    // positions, checked distinct (every position 0 .. 4095 once), the first positions of the roots'
    // subtrees (segment heads), then the tables by position
    const int64_t T = tile * kRunPositions;
    uint32_t* seen = reinterpret_cast<uint32_t*>(sm.queue);  // the queue is no longer read
    uint32_t* heads = seen + kRunPositions / 32;
    for (int w = t; w < kRunPositions / 32; w += kTileThreads) {
        seen[w] = 0;
        heads[w] = 0;
    }
    __syncthreads();
    for (int i = t; i < kTileCells; i += kTileThreads) {
        const bool valid = sm.fd[(i >> 6) + 1][(i & 63) + 1] != kNoData;
        const int s0 = st[i], p = s0 + sz[i] - 1;
        bool bad = p >= kRunPositions || s0 > p;
        if (!bad) bad = (atomicOr(&seen[p >> 5], 1u << (p & 31)) >> (p & 31)) & 1u;
        if (bad) {
            *error = 1;
            continue;
        }
        if (!valid || sm.dsl[i] == kNoCell) atomicOr(&heads[s0 >> 5], 1u << (s0 & 31));
    }
    __syncthreads();
    for (int i = t; i < kTileCells; i += kTileThreads) {
        const bool valid = sm.fd[(i >> 6) + 1][(i & 63) + 1] != kNoData;
        const int s0 = st[i], p = s0 + sz[i] - 1;
        if (p >= kRunPositions || s0 > p) continue;  // reported above
        const bool head = (heads[p >> 5] >> (p & 31)) & 1u;
        cell_at[T + run_table_index(p)] =
            (uint16_t)(i | (valid ? 0u : kNoValue) | (head ? kSegHead : 0u) | (s0 == p ? kLoneCell : 0u));
        prev_at[T + run_table_index(p)] = (uint16_t)(8 * (s0 > 0 ? scan_slot(s0 - 1) : kZeroSlot));
    }
    __syncthreads();
    if (t < kRunPositions / 32 && seen[t] != 0xFFFFFFFFu) *error = 1;
    const int32_t e0 = exit_base[tile], ne = exit_base[tile + 1] - e0;
    for (int e = t; e < ne; e += kTileThreads) {
        const int loc = exit_local[e0 + e];
        const int s0 = st[loc], p = s0 + sz[loc] - 1;
        exit_span[e0 + e] = (uint32_t)scan_slot(p) | ((uint32_t)(s0 > 0 ? scan_slot(s0 - 1) : kZeroSlot) << 16);
    }
}

// ---------------------------------------------------------------------------------------------------
// Per call
// ---------------------------------------------------------------------------------------------------
//
// A tile CTA works in two orders.  Material and results move between HBM and shared memory in cell
// order (row-major float4 rows, coalesced).  Thread t owns the post-order positions 16 t .. 16 t + 15:
// it gathers their material from shared memory through cell_at (one 4-byte read per cell), converts it
// to fixed point and takes the prefix sum of its run in registers; a warp scan and the warp totals give
// the run's offset, and each inclusive prefix is written to shared memory once.  The accu of a cell is
// then its own prefix minus the prefix just before its subtree (prev_at).
//
// Inside a tile the material is summed in 64-bit fixed point, round(x * 2^F), with F chosen per tile
// from a bound on the tile's total (4096 times its largest term, plus what enters through its border)
// so that the total stays below 2^62: prefix sums over the post-order are then exact, and so is every
// subtree sum taken as their difference (modulo 2^64, exact because the true sum is < 2^64).  A term
// x > 0 is represented to within 2^-(F+1) absolute; a tile whose smallest positive term would carry
// fewer than 19 bits (x * 2^F < 2^19) or that holds +inf asks for the walk engine instead.

constexpr float kMinQuantum = 524288.0f;  // 2^19

__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + e) << 23); }  // -126 <= e <= 127

// Largest F <= 126 with bound * 2^F < 2^62 (0 for bound 0).
__device__ __forceinline__ int tile_scale(float bound)
{
    if (!(bound > 0.0f)) return 0;
    const int e = (int)((__float_as_uint(bound) >> 23) & 0xFFu) - 126;  // bound < 2^e
    return min(62 - e, 126);
}

// Bound on a tile's total from the bits of its largest term (4096 terms below 2^(e - 126)) and of the
// largest sum entering through its border (at most 252 of them); +inf when beyond float range.
__device__ __forceinline__ float tile_bound(unsigned max_bits, unsigned src_bits)
{
    const int e = (int)(max_bits >> 23);
    const float local = e > 240 ? INFINITY : pow2f(e - 114);
    return (local + 256.0f * __uint_as_float(src_bits)) * 1.0009765625f;
}

// Conversions between float and 64-bit fixed point in integer arithmetic.  GB300 executes the 64-bit
// float <-> integer conversion instructions on its float64 pipe, which runs at a small fraction of the
// integer rate; these run on the integer pipes.

// round(x * 2^F) for finite x >= 0 with x * 2^F < 2^63 (ties away from zero).
__device__ __forceinline__ unsigned long long float_to_fixed64(float x, int F)
{
    const unsigned b = __float_as_uint(x);
    const unsigned e = b >> 23;
    const unsigned m = (b & 0x7FFFFFu) | (e ? 0x800000u : 0u);
    const int s = (int)(e ? e : 1u) - 150 + F;  // x * 2^F = m * 2^s
    const unsigned rs = s < 0 ? (unsigned)min(-s, 31) : 0u;
    const unsigned r = rs ? (m + (1u << (rs - 1))) >> rs : m;
    return (unsigned long long)r << (s > 0 ? s : 0);
}

// x * 2^F exactly, for x == 0 or a normal x >= 0 with x * 2^F >= 2^23 (no bit is shifted out).
__device__ __forceinline__ unsigned long long float_to_fixed64_exact(float x, float scale_hi)
{
    // scale_hi = 2^(F - 32).  The high and low 32-bit halves by float arithmetic, every step exact: a
    // power-of-two scaling, the truncation of a value below 2^30 with at most 24 significant bits, its
    // fraction (the bits under the binary point), and that fraction times 2^32 (an integer: no bit of
    // x * 2^F lies below 2^0).  Three conversions and three float operations instead of a 64-bit shift.
    const float y = __fmul_rn(x, scale_hi);
    const unsigned hi = __float2uint_rz(y);
    const float frac = __fsub_rn(y, __uint2float_rz(hi));
    const unsigned lo = __float2uint_rz(__fmul_rn(frac, 4294967296.0f));
    return ((unsigned long long)hi << 32) | lo;
}

// A 96-bit fixed-point value v * 2^-F, rounded to float (the bits below the top 64 are dropped).
__device__ __forceinline__ float fixed128_to_float(u128 v, int F)
{
    const unsigned long long hi = (unsigned long long)(v >> 64);
    if (hi == 0) return ldexpf(__ull2float_rn((unsigned long long)v), -F);
    const int shift = 64 - __clzll((long long)hi);
    return ldexpf(__ull2float_rn((unsigned long long)(v >> shift)), shift - F);
}

// Cells of a tile by thread in cell order: thread t holds the 4 x 4 cells (row (t + 256 j) / 16,
// columns 4 ((t + 256 j) % 16) .. + 3), j = 0..3, so that a row of the tile is 16 float4.
__device__ __forceinline__ int quad_cell(int j)
{
    const int k = threadIdx.x + kTileThreads * j;
    return (k >> 4) * kTile + (k & 15) * 4;
}

__device__ __forceinline__ float4 load_quad(const float* __restrict__ p, const TileGeom& g, int64_t r, int64_t c,
                                            bool vec, float fill)
{
    if (vec) {
        if (r < g.rows && c < g.cols) return __ldg(reinterpret_cast<const float4*>(p + r * g.cols + c));
        return make_float4(fill, fill, fill, fill);
    }
    float v[4];
#pragma unroll
    for (int x = 0; x < 4; ++x) v[x] = (r < g.rows && c + x < g.cols) ? __ldg(p + r * g.cols + c + x) : fill;
    return make_float4(v[0], v[1], v[2], v[3]);
}

__device__ __forceinline__ void store_quad(float* __restrict__ p, const TileGeom& g, int64_t r, int64_t c, bool vec,
                                           float4 v)
{
    if (r >= g.rows) return;
    if (vec) {
        if (c < g.cols) *reinterpret_cast<float4*>(p + r * g.cols + c) = v;
        return;
    }
    const float w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int x = 0; x < 4; ++x)
        if (c + x < g.cols) p[r * g.cols + c + x] = w[x];
}

struct TileForest {
    const uint16_t* cell_at;
    const uint16_t* prev_at;
    const float* inflow;
};

// Shared memory of a tile CTA of pass 1 or pass 3 (dynamic: 53 KB, four CTAs per SM).
struct __align__(16) TileCallSmem {
    unsigned long long S[kScanSlotCount];  // inclusive prefix sums by scan slot; S[kZeroSlot] = 0
    float M[kTileCells];                   // material plus what enters, in cell order; then the results
    alignas(16) unsigned long long warp_tot[kTileThreads / 32];
    alignas(16) unsigned red[2][kTileThreads / 32];
    alignas(16) unsigned warp_mn[kTileThreads / 32];
    alignas(16) float warp_sum[kTileThreads / 32];
    float seg_hi[kTileThreads / 32], seg_lo[kTileThreads / 32];  // pass 1: warp totals of the segmented scan
    int seg_head[kTileThreads / 32];
    float carry_hi[kTileThreads], carry_lo[kTileThreads];        // pass 1: what each run's first segment carries in
    uint8_t run_first[kTileThreads];                             // pass 1: first segment head of each run (16: none)
    int quit;                                                    // pass 3: the walk engine redoes the call
};

// The thread's run of a per-position table (cell_at or prev_at): eight coalesced 4-byte loads.
__device__ __forceinline__ void load_run(const uint16_t* __restrict__ table, uint32_t (&w)[kRunWords])
{
    const uint32_t* p = reinterpret_cast<const uint32_t*>(table) + threadIdx.x;
#pragma unroll
    for (int i = 0; i < kRunWords; ++i) w[i] = __ldg(p + i * kTileThreads);
}
__device__ __forceinline__ unsigned run_at(const uint32_t (&w)[kRunWords], int j)
{
    return (w[j >> 1] >> (16 * (j & 1))) & 0xFFFFu;
}

// Material of the tile in cell order (0 outside the array), by quads of 4 cells (quad_cell).
__device__ __forceinline__ void load_material(float4 (&x)[4], const float* __restrict__ ext, float ext_s,
                                              const TileGeom& g, int64_t tr, int64_t tc, bool vec)
{
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int cell = quad_cell(j);
        x[j] = ext ? load_quad(ext, g, tr * kTile + (cell >> 6), tc * kTile + (cell & 63), vec, 0.0f)
                   : make_float4(ext_s, ext_s, ext_s, ext_s);
    }
}

// The material total in 2^-16 units at or beyond this makes the tile engine hand the call to the walk
// engine (the 128-bit fixed point of the exit forest keeps 96 value bits).
constexpr unsigned long long kTotalLimit = 1000000000000000000ull;

// total[0], summed by pass 1 with 64-bit atomics (exact, so the order does not matter), and total[1]: the
// tile engine's result stands when neither says otherwise.
__device__ __forceinline__ bool tile_fallback(const unsigned long long* total)
{
    return *reinterpret_cast<const volatile unsigned long long*>(total + 1) != 0 || total[0] >= kTotalLimit;
}

constexpr int kScanItems = 8;
constexpr int kScanBlock = kTileThreads * kScanItems;
constexpr int kScanPolls = 1 << 20;  // poll limit of one look-back wait (a second at most)

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

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// The exit forest's 128-bit inclusive scan, one chunk of consecutive scan blocks (kScanBlock exits each)
// per CTA, with as many CTAs as fit on the GPU at once.  CTAs take chunks in ticket order; each sums its
// chunk, publishes the sum (flag 1), then warp 0 adds up the sums of the chunks before it, 32 at a time,
// until it meets a chunk that has published the sum up to and including itself (flag 2); the CTA
// publishes its own (flag 2) and scans its chunk again, block by block, from that prefix.  A CTA waits
// only for chunks with smaller tickets, held by CTAs that started earlier, and those publish their own
// sums before they wait for anything: no chain of waits forms.  Every wait is bounded: a wait that gives
// up (or sees that one did) sets total[1] = 2, after which the walk engine redoes the call.
// ctl = the ticket, then the chunk flags, zeroed before the call.
__global__ void __launch_bounds__(kTileThreads)
    k_scan_exits(const float2* __restrict__ P, int64_t n, int64_t chunk_blocks, unsigned long long* total,
                 unsigned* ctl, uint4* look_aggr, uint4* look_incl, uint4* __restrict__ S, int polls)
{
    __shared__ u128 warp_tot[kTileThreads / 32];
    __shared__ u128 prefix_sh;
    __shared__ unsigned ticket_sh;
    __shared__ int abort_sh;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // one thread decides, so that the whole CTA leaves or stays
    if (threadIdx.x == 0) ticket_sh = tile_fallback(total) ? ~0u : atomicAdd(ctl, 1u);
    __syncthreads();
    if (ticket_sh == ~0u) return;
    const int64_t g = ticket_sh;
    unsigned* flag = ctl + 1;
    const int F = fixed_point_bits(total[0]);
    const int64_t first = g * chunk_blocks * kScanBlock;
    const int64_t last = min(n, first + chunk_blocks * kScanBlock);
    // the chunk's sum
    u128 s = 0;
    for (int64_t b0 = first; b0 < last; b0 += kScanBlock) {
        const int64_t base = b0 + (int64_t)threadIdx.x * kScanItems;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k)
            if (base + k < last) s += exit_value_fixed(__ldg(P + base + k), F);
    }
    u128 bt;
    block_exclusive_u128(s, warp_tot, bt);
    if (warp == 0) {
        if (g == 0) {
            if (lane == 0) {
                look_incl[0] = from_u128(bt);
                st_release_u32(flag, 2u);
                prefix_sh = 0;
                abort_sh = 0;
            }
        } else {
            if (lane == 0) {
                look_aggr[g] = from_u128(bt);
                st_release_u32(flag + g, 1u);
            }
            u128 prefix = 0;
            bool failed = false;
            for (int64_t top = g - 1;; top -= 32) {
                const int64_t j = top - lane;
                unsigned f = 2u;  // before chunk 0: nothing (never reached: chunk 0 publishes flag 2)
                u128 x = 0;
                if (j >= 0) {
                    int k = 0;
                    for (; k < polls; ++k) {
                        f = ld_acquire_u32(flag + j);
                        if (f != 0u) break;
                        if (*reinterpret_cast<volatile unsigned long long*>(total + 1)) k = polls - 1;
                        __nanosleep(64);
                    }
                    if (k >= polls) f = 0u;
                }
                if (__ballot_sync(0xffffffffu, f == 0u)) {
                    failed = true;
                    break;
                }
                const unsigned incl = __ballot_sync(0xffffffffu, f == 2u);
                const int stop = incl ? __ffs(incl) - 1 : 31;  // lanes 0..stop count
                if (j >= 0 && lane <= stop) x = to_u128(__ldcg(f == 2u ? look_incl + j : look_aggr + j));
                for (int d = 16; d > 0; d >>= 1) x += shfl_down_u128(x, d);
                prefix += x;  // lane 0 holds the window's sum
                if (incl) break;
            }
            if (lane == 0) {
                if (failed) {
                    total[1] = 2ull;
                } else {
                    look_incl[g] = from_u128(prefix + bt);
                    st_release_u32(flag + g, 2u);
                }
                prefix_sh = prefix;
                abort_sh = failed ? 1 : 0;
            }
        }
    }
    __syncthreads();
    if (abort_sh) return;
    u128 carry = prefix_sh;
    for (int64_t b0 = first; b0 < last; b0 += kScanBlock) {
        const int64_t base = b0 + (int64_t)threadIdx.x * kScanItems;
        u128 v[kScanItems];
        u128 t = 0;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            v[k] = base + k < last ? exit_value_fixed(__ldg(P + base + k), F) : (u128)0;
            t += v[k];
        }
        u128 blk;
        u128 run = carry + block_exclusive_u128(t, warp_tot, blk);
        carry += blk;
#pragma unroll
        for (int k = 0; k < kScanItems; ++k) {
            run += v[k];
            if (base + k < last) S[base + k] = from_u128(run);
        }
    }
}

// What enters each inflow slot (a border cell receiving flow from other tiles): the exact sum of the subtree
// sums of the exits draining into it (each a difference of two inclusive prefix sums of the exit
// forest), rounded to float once; NaN when one of them holds a no-data exit.
__global__ void k_slot_inflow(int64_t nslot, const int32_t* __restrict__ slot_at,
                              const int32_t* __restrict__ slot_first, const int2* __restrict__ slot_edge,
                              const uint4* __restrict__ S, float* __restrict__ inflow,
                              const unsigned long long* total)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nslot || tile_fallback(total)) return;
    const int F = fixed_point_bits(total[0]);
    u128 src = 0;
    for (int32_t k = __ldg(slot_first + i), k1 = __ldg(slot_first + i + 1); k < k1; ++k) {
        const int2 e = __ldg(slot_edge + k);
        src += to_u128(__ldcg(S + e.x)) - (e.y >= 0 ? to_u128(__ldcg(S + e.y)) : (u128)0);
    }
    inflow[__ldg(slot_at + i)] = (src >> 96) ? __int_as_float(0x7fc00000) : fixed128_to_float(src & kValueMask, F);
}

// Build: per tile, its inflow slots and their upstream exits (one thread per tile, border order).
__global__ void k_slot_count(int64_t ntiles, const uint8_t* __restrict__ border_in, int32_t* nslot, int32_t* nexit)
{
    const int64_t tile = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tile >= ntiles) return;
    int a = 0, b = 0;
    for (int k = 0; k < kBorderCells; ++k) {
        const unsigned m = border_in[tile * kBorderCells + k];
        a += m != 0;
        b += __popc(m);
    }
    nslot[tile] = a;
    nexit[tile] = b;
}

__global__ void k_slot_fill(int64_t ntiles, const uint8_t* __restrict__ border_in, const int32_t* __restrict__ halo_exit,
                            const int32_t* __restrict__ slot_base, const int32_t* __restrict__ exit_base,
                            const uint32_t* __restrict__ exit_pos, const uint32_t* __restrict__ exit_start,
                            int32_t* slot_at, int32_t* slot_first, int2* slot_edge, int* error)
{
    const int64_t tile = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tile >= ntiles) return;
    int32_t s = slot_base[tile], e = exit_base[tile];
    for (int b = 0; b < kBorderCells; ++b) {
        const unsigned m0 = border_in[tile * kBorderCells + b];
        if (!m0) continue;
        int rin, cin;
        border_cell(b, rin, cin);
        slot_at[s] = (int32_t)(tile * kSlotStride + b);
        slot_first[s] = e;
        for (unsigned m = m0; m; m &= m - 1) {
            const int q = __ffs(m) - 1;
            const int32_t id = halo_exit[tile * kHaloSlots + halo_slot_of(rin + nb_dr(q), cin + nb_dc(q))];
            if (id < 0) atomicExch(error, 1);  // a neighbour draining in must be an exit of its tile
            const int32_t y = id < 0 ? 0 : id;
            const uint32_t st = exit_start[y];
            slot_edge[e++] = make_int2((int)exit_pos[y], st ? (int)(st - 1u) : -1);
        }
        ++s;
    }
}

// Inclusive prefix sums (modulo 2^64) of the thread runs a[0..15] over the whole tile, written to S by
// scan slot.  Ends with a block barrier.
__device__ __forceinline__ void tile_prefix(TileCallSmem& sm, unsigned long long (&a)[kRun])
{
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
#pragma unroll
    for (int j = 1; j < kRun; ++j) a[j] += a[j - 1];
    unsigned long long x = a[kRun - 1];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sm.warp_tot[warp] = x;
    __syncthreads();
    unsigned long long off = x - a[kRun - 1];
    const ulonglong2* wt = reinterpret_cast<const ulonglong2*>(sm.warp_tot);  // 16-byte loads
#pragma unroll
    for (int w = 0; w < kTileThreads / 64; ++w) {
        const ulonglong2 v = wt[w];
        off += (2 * w < warp ? v.x : 0ull) + (2 * w + 1 < warp ? v.y : 0ull);
    }
    unsigned long long* run = sm.S + kRunSlots * t;  // 136-byte runs
#pragma unroll
    for (int j = 0; j < kRun; ++j) {
        a[j] += off;  // the thread keeps its own prefixes
        run[j] = a[j];
    }
    if (t == 0) sm.S[kZeroSlot] = 0ull;
    __syncthreads();
}

// Poison counts (slow path): inclusive prefix counts over the post-order of the flagged terms, written as
// 32-bit counts by scan slot over S (free until the value scan).  Ends with a block barrier.
__device__ __forceinline__ void poison_counts(TileCallSmem& sm, unsigned bad)
{
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    unsigned run = __popc(bad);
    unsigned x = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sm.warp_tot[warp] = x;
    __syncthreads();
    unsigned off = x - run;
    for (int w = 0; w < warp; ++w) off += (unsigned)sm.warp_tot[w];
    unsigned* C = reinterpret_cast<unsigned*>(sm.S);
    unsigned c = off;
#pragma unroll
    for (int j = 0; j < kRun; ++j) {
        c += (bad >> j) & 1u;
        C[kRunSlots * t + j] = c;
    }
    if (t == 0) C[kZeroSlot] = 0u;
    __syncthreads();
}

// The thread's run in post-order: the material of each position (0 for no-data cells and cells outside
// the array), after a block barrier that follows the stores to M.
__device__ __forceinline__ void gather_run(const TileCallSmem& sm, const uint32_t (&ca)[kRunWords], float (&x)[kRun])
{
#pragma unroll
    for (int j = 0; j < kRun; ++j) {
        const unsigned w = run_at(ca, j);
        const float v = sm.M[w & kIndexMask];
        x[j] = (w & kNoValue) ? 0.0f : v;
    }
}

// NaN or negative terms of a run (slow path): flagged in the returned mask, then 0 (-0 counts as 0).
__device__ __forceinline__ unsigned clean_run(float (&x)[kRun])
{
    unsigned bad = 0;
#pragma unroll
    for (int j = 0; j < kRun; ++j) {
        if (!(x[j] >= 0.0f)) bad |= 1u << j;
        x[j] = x[j] >= 0.0f ? fabsf(x[j]) : 0.0f;
    }
    return bad;
}

// Float-float pieces of pass 1: x + y with the rounding error of the high parts kept in lo (no
// renormalisation), and the segmented-scan combination of (sum since the last segment head, has a head).
struct SegSum {
    float hi, lo;
    bool head;
};
__device__ __forceinline__ void ff_acc(float& hi, float& lo, float x)
{
    const float s = __fadd_rn(hi, x);
    const float bp = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(x, bp));
    hi = s;
    lo = __fadd_rn(lo, e);
}
// a, then b
__device__ __forceinline__ SegSum seg_combine(const SegSum& a, const SegSum& b)
{
    if (b.head) return b;
    SegSum r{a.hi, __fadd_rn(a.lo, b.lo), a.head};
    ff_acc(r.hi, r.lo, b.hi);
    return r;
}
__device__ __forceinline__ SegSum seg_shfl_up(const SegSum& v, int d)
{
    return SegSum{__shfl_up_sync(0xffffffffu, v.hi, d), __shfl_up_sync(0xffffffffu, v.lo, d),
                  __shfl_up_sync(0xffffffffu, (int)v.head, d) != 0};
}

// Pass 1: the local value of every exit (the accu of its in-tile subtree) to P, in the exit forest's
// post-order; an upper bound of the tile's material total in 2^-16 units added to total[0] (64-bit
// atomics: exact, whatever the order; total[1] is set instead, asking for the walk engine, on +inf, a
// total beyond float range, a dynamic range the 64-bit fixed point of pass 3 cannot hold, or a sum that
// wraps), and the statistics pass 3 takes its fixed-point scale from (so that it needs no reduction of its
// own).  Exits are roots of the tile's forest; the subtrees of the roots are consecutive runs of
// positions (segments, each starting at a flagged head), so an exit's value is the sum of its segment: a
// segmented prefix sum in float-float (relative error about 2^-35 of the segment's total in the worst
// case, no cancellation), computed on the float pipes.  A NaN or negative term makes its segment NaN,
// and with it the exit: no-data flows on from there through the exit forest.
// vec: material rows can be read as float4 (16-byte aligned, columns a multiple of 4).
__global__ void __launch_bounds__(kTileThreads, 4)
    k_tile_exits(TileGeom g, const float* __restrict__ ext, float ext_s, bool vec, TileForest f,
                 const int32_t* __restrict__ exit_base, const uint32_t* __restrict__ exit_span,
                 const uint32_t* __restrict__ exit_pos, float2* __restrict__ P,
                 unsigned long long* total, TileStat* __restrict__ stat)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TileCallSmem& sm = *reinterpret_cast<TileCallSmem*>(smem_raw);
    const int64_t tr = blockIdx.y, tc = blockIdx.x;  // grid = (tile columns, tile rows)
    const int64_t tile = tr * g.tcols + tc;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    float4 xm[4];
    load_material(xm, ext, ext_s, g, tr, tc, vec);
    uint32_t ca[kRunWords];
    load_run(f.cell_at + tile * kRunPositions, ca);
    const int32_t e0 = __ldg(exit_base + tile), ne = __ldg(exit_base + tile + 1) - e0;
    uint32_t span = 0, epos = 0;
    if (t < ne) {  // a tile has at most 252 exits (its border cells)
        span = __ldg(exit_span + e0 + t);
        epos = __ldg(exit_pos + e0 + t);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) *reinterpret_cast<float4*>(sm.M + quad_cell(j)) = xm[j];
    __syncthreads();
    // over the valid positions: the largest raw bits (a sign bit or NaN: pass 3's slow path), the largest
    // and smallest positive bits of the terms that are >= 0, and their float sum; and the segmented sums of
    // the run, with the run's summary for the scan across threads
    unsigned raw = 0, mx = 0, mn = 0xFFFFFFFFu;
    float sum = 0.0f;
    SegSum run{0.0f, 0.0f, false};
    int first_head = kRun;
    float2* L = reinterpret_cast<float2*>(sm.S);
#pragma unroll
    for (int j = 0; j < kRun; ++j) {
        const unsigned w = run_at(ca, j);
        const float m = sm.M[w & kIndexMask];
        const float x = (w & kNoValue) ? 0.0f : m;
        const unsigned b = __float_as_uint(x);
        raw = max(raw, b);
        const bool ok = x >= 0.0f;
        const unsigned a = ok ? (b & 0x7FFFFFFFu) : 0u;
        mx = max(mx, a);
        mn = min(mn, a - 1u);
        sum += ok ? x : 0.0f;
        const float v = ok || isnan(x) ? x : __int_as_float(0x7fc00000);  // negative: NaN
        if (w & kSegHead) {
            if (!run.head) first_head = j;
            run = SegSum{v, 0.0f, true};
        } else {
            ff_acc(run.hi, run.lo, v);
        }
        L[kRunSlots * t + j] = make_float2(run.hi, run.lo);
    }
    raw = __reduce_max_sync(0xffffffffu, raw);
    mx = __reduce_max_sync(0xffffffffu, mx);
    mn = __reduce_min_sync(0xffffffffu, mn);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    // exclusive segmented scan of the run summaries across the tile: what a segment that starts before
    // this run carries into it
    SegSum inc = run;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const SegSum y = seg_shfl_up(inc, d);
        if (lane >= d) inc = seg_combine(y, inc);
    }
    SegSum exc = seg_shfl_up(inc, 1);
    if (lane == 0) exc = SegSum{0.0f, 0.0f, false};
    if (lane == 0) {
        sm.red[0][warp] = raw;
        sm.red[1][warp] = mx;
        sm.warp_mn[warp] = mn;
        sm.warp_sum[warp] = sum;
    }
    if (lane == 31) {
        sm.seg_hi[warp] = inc.hi;
        sm.seg_lo[warp] = inc.lo;
        sm.seg_head[warp] = inc.head;
    }
    __syncthreads();
    // the warps' summaries: lane i of every warp takes warp (i & 7)'s; the block's largest and smallest bits
    // by warp reductions, the sum (thread 0's is used) and a segmented scan over each group of eight lanes
    // by three shuffle steps; the carry into this warp is lane warp - 1's inclusive scan
    static_assert(kTileThreads == 256, "eight warps per tile CTA");
    const int w8 = lane & 7;
    raw = __reduce_max_sync(0xffffffffu, sm.red[0][w8]);
    mx = __reduce_max_sync(0xffffffffu, sm.red[1][w8]);
    mn = __reduce_min_sync(0xffffffffu, sm.warp_mn[w8]);
    sum = sm.warp_sum[w8];
    SegSum ws{sm.seg_hi[w8], sm.seg_lo[w8], sm.seg_head[w8] != 0};
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        const SegSum y = seg_shfl_up(ws, o);
        if (w8 >= o) ws = seg_combine(y, ws);
    }
    const int src = warp > 0 ? warp - 1 : 0;
    SegSum before{__shfl_sync(0xffffffffu, ws.hi, src), __shfl_sync(0xffffffffu, ws.lo, src),
                  __shfl_sync(0xffffffffu, (int)ws.head, src) != 0};
    if (warp == 0) before = SegSum{0.0f, 0.0f, false};
    const SegSum carry = seg_combine(before, exc);
    sm.run_first[t] = (uint8_t)first_head;
    sm.carry_hi[t] = carry.hi;
    sm.carry_lo[t] = carry.lo;
    const float bound = tile_bound(mx, 0u);
    const int F = tile_scale(bound);
    if (mx >= 0x7F800000u || !(bound < 1.0e38f) ||
        (mn != 0xFFFFFFFFu && __uint_as_float(mn + 1u) * pow2f(F) < kMinQuantum)) {
        if (t == 0) atomicOr(total + 1, 1ull);
        return;  // uniform: every thread has the same reductions
    }
    __syncthreads();
    if (t < ne) {
        // the exit's position is the end of its segment; a segment that starts in an earlier run also
        // holds what that run's carry brings
        const int slot = (int)(span & 0xFFFFu), r = slot / kRunSlots, j = slot - kRunSlots * r;
        float hi = L[slot].x, lo = L[slot].y;
        if (j < sm.run_first[r]) {
            lo = __fadd_rn(lo, sm.carry_lo[r]);
            ff_acc(hi, lo, sm.carry_hi[r]);
        }
        const float h = __fadd_rn(hi, lo);
        P[epos] = isnan(h) ? make_float2(__int_as_float(0x7fc00000), 0.0f) : make_float2(h, __fsub_rn(lo, __fsub_rn(h, hi)));
    }
    if (t == 0) {
        const double units = ldexp((double)sum * (1.0 + 1.0 / 1024.0) + ldexp(1.0, -100), 16) + 64.0;
        if (units < (double)kTotalLimit) {
            const unsigned long long u = (unsigned long long)units;
            if (atomicAdd(total, u) + u < u) atomicOr(total + 1, 1ull);  // the sum wrapped
        } else {
            atomicOr(total + 1, 1ull);
        }
        stat[tile] = TileStat{bound, mn, raw > 0x7F800000u ? 1u : 0u, 0u};
    }
}

// Pass 3: the result of every cell: the accu of its in-tile subtree, where each border cell's material
// carries what enters it from other tiles (the exact subtree sums of the exits draining into it, rounded
// to float once, added to the cell's material in float), in one fixed-point scan per tile.
//
// The scale F comes from pass 1's bound on the tile's material plus the float sum of what enters, so no
// block reduction of the terms is needed; a tile whose smallest positive term would get fewer than 19
// bits sets the fallback flag total[1], and the walk engine redoes the call.  Fast path (no NaN or
// negative term and nothing NaN entering): gather, convert, scan, and for every cell with in-tile upstream
// cells its prefix minus the prefix before its subtree; a cell without in-tile upstream cells keeps its
// material (plus what enters) in M, which is its result.  Slow path: NaN / negative terms count as 0 and
// are counted along the post-order; a cell whose subtree holds one is NaN.
__global__ void __launch_bounds__(kTileThreads, 4)
    k_tile_accu(TileGeom g, const float* __restrict__ ext, float ext_s, bool vec, float* __restrict__ out,
                TileForest f, const TileStat* __restrict__ stat, unsigned long long* total)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TileCallSmem& sm = *reinterpret_cast<TileCallSmem*>(smem_raw);
    const int64_t tr = blockIdx.y, tc = blockIdx.x;  // grid = (tile columns, tile rows)
    const int64_t tile = tr * g.tcols + tc;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (t == 0) {  // one thread decides (other CTAs may set the flag meanwhile), read after the barrier below
        const bool fb = tile_fallback(total);
        if (fb && *reinterpret_cast<volatile unsigned long long*>(total + 1) == 0) total[1] = 1ull;
        sm.quit = fb;
    }
    float4 xm[4];
    load_material(xm, ext, ext_s, g, tr, tc, vec);
    uint32_t ca[kRunWords], pv[kRunWords];
    load_run(f.cell_at + tile * kRunPositions, ca);
    load_run(f.prev_at + tile * kRunPositions, pv);
    const TileStat st = stat[tile];
    // what enters through border cell t (0 where nothing does; NaN when no-data enters)
    float entering = 0.0f;
    int ecell = -1;
    if (t < kBorderCells) {
        entering = __ldg(f.inflow + tile * kSlotStride + t);
        int rin, cin;
        border_cell(t, rin, cin);
        ecell = rin * kTile + cin;
    }
    // over what enters: NaN anywhere, the float sum, and the smallest positive bits minus one
    const bool enan = isnan(entering);
    const float eclean = enan ? 0.0f : entering;
    float esum = eclean;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) esum += __shfl_xor_sync(0xffffffffu, esum, o);
    const unsigned emn = __reduce_min_sync(0xffffffffu, __float_as_uint(eclean) - 1u);
    const unsigned enan_any = __any_sync(0xffffffffu, enan);
    if (lane == 0) {
        sm.warp_sum[warp] = esum;
        sm.red[0][warp] = emn;
        sm.red[1][warp] = enan_any;
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) *reinterpret_cast<float4*>(sm.M + quad_cell(j)) = xm[j];
    __syncthreads();
    if (sm.quit) return;  // uniform
    if (ecell >= 0) {  // material out of the domain stays visible as NaN (the cell and all below are NaN)
        const float mat = sm.M[ecell];
        sm.M[ecell] = mat >= 0.0f ? mat + entering : __int_as_float(0x7fc00000);
    }
    // over the eight warps, by 16-byte loads; the sum in the same order in every thread
    static_assert(kTileThreads == 256, "eight warps per tile CTA");
    const float4 s0 = *reinterpret_cast<const float4*>(sm.warp_sum);
    const float4 s1 = *reinterpret_cast<const float4*>(sm.warp_sum + 4);
    const uint4 m0 = *reinterpret_cast<const uint4*>(sm.red[0]), m1 = *reinterpret_cast<const uint4*>(sm.red[0] + 4);
    const uint4 n0 = *reinterpret_cast<const uint4*>(sm.red[1]), n1 = *reinterpret_cast<const uint4*>(sm.red[1] + 4);
    const float in_total = 0.0f + s0.x + s0.y + s0.z + s0.w + s1.x + s1.y + s1.z + s1.w;
    const unsigned mn = min(min(min(min(st.min_bits, m0.x), min(m0.y, m0.z)), min(m0.w, m1.x)),
                            min(min(m1.y, m1.z), m1.w));
    const unsigned nan_in = n0.x | n0.y | n0.z | n0.w | n1.x | n1.y | n1.z | n1.w;
    const float bound = (st.bound + in_total) * 1.0009765625f;
    const int F = tile_scale(bound);
    if (!(bound < 1.0e38f) || (mn != 0xFFFFFFFFu && __uint_as_float(mn + 1u) * pow2f(F) < kMinQuantum)) {
        if (t == 0) total[1] = 1ull;  // the walk engine redoes the call
        return;                       // uniform
    }
    const bool exact = mn == 0xFFFFFFFFu || __uint_as_float(mn + 1u) * pow2f(F) >= 8388608.0f;
    const bool clean = !st.bad && !nan_in;  // uniform
    __syncthreads();  // M holds what enters
    float x[kRun];
    gather_run(sm, ca, x);
    unsigned poisoned = 0;  // bit j: the subtree of run entry j holds a NaN or negative term
    if (!clean) {
        poison_counts(sm, clean_run(x));
        const unsigned* C = reinterpret_cast<const unsigned*>(sm.S);
#pragma unroll
        for (int j = 0; j < kRun; ++j)
            if (C[kRunSlots * t + j] != C[run_at(pv, j) >> 3]) poisoned |= 1u << j;
        __syncthreads();  // S and warp_tot are free for the value scan
    }
    unsigned long long a[kRun];
    if (exact) {
#pragma unroll
        for (int j = 0; j < kRun; ++j) a[j] = float_to_fixed64_exact(x[j], pow2f(F - 32));
    } else {
#pragma unroll
        for (int j = 0; j < kRun; ++j) a[j] = float_to_fixed64(x[j], F);
    }
    tile_prefix(sm, a);
    // results by position, put in cell order into M; a cell without in-tile upstream cells keeps its
    // material (plus what enters) there on the fast path, which is its result
    const float nan = __int_as_float(0x7fc00000);
    const float unscale = pow2f(-F);
    const unsigned char* Sb = reinterpret_cast<const unsigned char*>(sm.S);  // prev_at: byte offsets
    // the subtree's sum (its prefix, a[j], minus the prefix before it, < 2^62) to float: two 32-bit
    // conversions, each rounded to nearest, and one fused rounding of their sum: within about one unit
    // in the last place, and exact when it has at most 24 significant bits
    auto result = [&](unsigned long long s_own, unsigned p) {
        const unsigned long long v = s_own - *reinterpret_cast<const unsigned long long*>(Sb + p);
        return __fmaf_rn(__uint2float_rn((unsigned)(v >> 32)), 4294967296.0f, __uint2float_rn((unsigned)v)) *
               unscale;
    };
    if (clean && exact) {  // uniform
        // a valid lone cell already holds its result (its material plus what enters) in M: its lanes skip
        // the read of the prefix before it and the store (predicated, so no shared-memory traffic)
#pragma unroll
        for (int j = 0; j < kRun; ++j) {
            const unsigned w = run_at(ca, j);
            const bool keep = (w & (kLoneCell | kNoValue)) == kLoneCell;
            unsigned long long before = 0ull;
            if (!keep) before = *reinterpret_cast<const unsigned long long*>(Sb + run_at(pv, j));
            const unsigned long long v = a[j] - before;
            const float r = __fmaf_rn(__uint2float_rn((unsigned)(v >> 32)), 4294967296.0f,
                                      __uint2float_rn((unsigned)v)) * unscale;
            if (!keep) sm.M[w & kIndexMask] = (w & kNoValue) ? nan : r;
        }
    } else if (clean) {
#pragma unroll
        for (int j = 0; j < kRun; ++j) {
            const unsigned w = run_at(ca, j);
            const bool none = w & kNoValue;
            if (!none && (w & kLoneCell)) continue;  // keeps its material (plus what enters) in M
            const float r = result(a[j], run_at(pv, j));
            sm.M[w & kIndexMask] = none ? nan : r;
        }
    } else {
#pragma unroll
        for (int j = 0; j < kRun; ++j) {
            const unsigned w = run_at(ca, j);
            const bool none = (w & kNoValue) || ((poisoned >> j) & 1u);
            const float r = result(a[j], run_at(pv, j));
            sm.M[w & kIndexMask] = none ? nan : r;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int cell = quad_cell(j);
        store_quad(out, g, tr * kTile + (cell >> 6), tc * kTile + (cell & 63), vec,
                   *reinterpret_cast<const float4*>(sm.M + cell));
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
    int32_t *sc = nullptr, *ec = nullptr;
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
    // per-tile flow forests in post-order
    TRY(cudaMalloc(&tc->cell_at, nt * kRunPositions * sizeof(uint16_t)), "tile forest");
    TRY(cudaMalloc(&tc->prev_at, nt * kRunPositions * sizeof(uint16_t)), "tile forest");
    TRY(cudaMalloc(&tc->exit_span, std::max<int64_t>(E, 1) * sizeof(uint32_t)), "exit span");
    TRY(cudaMalloc(&tc->border_in, nt * kBorderCells), "tile border masks");
    TRY(cudaFuncSetAttribute(k_tile_forest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(TileSmem)),
        "tile forest");
    k_tile_forest<<<dim3((unsigned)g.tcols, (unsigned)g.trows), kTileThreads, sizeof(TileSmem), stream>>>(
        core->fd, g, tc->exit_base, tc->exit_local, tc->cell_at, tc->prev_at, tc->exit_span, tc->border_in, flag);
    tc->bytes += nt * kRunPositions * 4 + E * 4 + nt * kBorderCells;
    TRY(cudaGetLastError(), "tile build");
    TRY(cudaMemcpyAsync(&herr, flag, sizeof(int), cudaMemcpyDeviceToHost, stream), "tile flag");
    TRY(cudaStreamSynchronize(stream), "tile build");
    if (herr) {
        rc = fail(LUE_GPU_EINVAL, "tile topology: cycle inside a tile or inconsistent exit forest");
        goto error;
    }
    // inflow slots: per tile the border cells receiving flow from other tiles, and their upstream exits
    {
        std::vector<int32_t> hs(nt), he(nt), sbase(nt + 1), ebase(nt + 1);
        TRY(cudaMalloc(&sc, nt * sizeof(int32_t)), "slot count");
        TRY(cudaMalloc(&ec, nt * sizeof(int32_t)), "slot count");
        k_slot_count<<<blocks_for(nt, 256), 256, 0, stream>>>(nt, tc->border_in, sc, ec);
        TRY(cudaGetLastError(), "slot count");
        TRY(cudaMemcpyAsync(hs.data(), sc, nt * sizeof(int32_t), cudaMemcpyDeviceToHost, stream), "slot count");
        TRY(cudaMemcpyAsync(he.data(), ec, nt * sizeof(int32_t), cudaMemcpyDeviceToHost, stream), "slot count");
        TRY(cudaStreamSynchronize(stream), "slot count");
        int64_t a = 0, b = 0;
        for (int64_t i = 0; i < nt; ++i) {
            sbase[i] = (int32_t)a;
            ebase[i] = (int32_t)b;
            a += hs[i];
            b += he[i];
            if (a > INT32_MAX || b > INT32_MAX) {
                rc = fail(LUE_GPU_ERANGE, "tile topology: too many inflow slots");
                goto error;
            }
        }
        sbase[nt] = (int32_t)a;
        ebase[nt] = (int32_t)b;
        tc->nslot = a;
        TRY(cudaMemcpyAsync(sc, sbase.data(), nt * sizeof(int32_t), cudaMemcpyHostToDevice, stream), "slot base");
        TRY(cudaMemcpyAsync(ec, ebase.data(), nt * sizeof(int32_t), cudaMemcpyHostToDevice, stream), "slot base");
        TRY(cudaMalloc(&tc->slot_at, std::max<int64_t>(a, 1) * sizeof(int32_t)), "slots");
        TRY(cudaMalloc(&tc->slot_first, (a + 1) * sizeof(int32_t)), "slots");
        TRY(cudaMalloc(&tc->slot_edge, std::max<int64_t>(b, 1) * sizeof(int2)), "slots");
        TRY(cudaMemcpyAsync(tc->slot_first + a, &ebase[nt], sizeof(int32_t), cudaMemcpyHostToDevice, stream),
            "slot end");
        k_slot_fill<<<blocks_for(nt, 256), 256, 0, stream>>>(nt, tc->border_in, tc->halo_exit, sc, ec,
                                                             tc->exit_pos, tc->exit_start, tc->slot_at,
                                                             tc->slot_first, tc->slot_edge, flag);
        TRY(cudaGetLastError(), "slot fill");
        TRY(cudaMemcpyAsync(&herr, flag, sizeof(int), cudaMemcpyDeviceToHost, stream), "tile flag");
        TRY(cudaStreamSynchronize(stream), "slot fill");  // the host vectors must outlive the copies
        if (herr) {
            rc = fail(LUE_GPU_EINVAL, "tile topology: an inflow without an upstream exit");
            goto error;
        }
        tc->bytes += a * 8 + 4 + b * 8;
    }
    cudaFree(sc);
    cudaFree(ec);
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
    cudaFree(sc);
    cudaFree(ec);
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
    cudaFree(tc->cell_at);
    cudaFree(tc->prev_at);
    cudaFree(tc->exit_span);
    cudaFree(tc->border_in);
    cudaFree(tc->slot_at);
    cudaFree(tc->slot_first);
    cudaFree(tc->slot_edge);
    delete tc;
}

int tile_scratch_alloc(const TileCore* tc, TileScratch* s)
{
    const int64_t E = std::max<int64_t>(tc->nexit, 1);
    const int64_t nb = (E + kScanBlock - 1) / kScanBlock;
    int rc = 0;
    if ((rc = cuda_status(cudaMalloc(&s->P, E * sizeof(float2)), "tile scratch"))) return rc;
    if ((rc = cuda_status(cudaMalloc(&s->S, E * sizeof(uint4)), "tile scratch"))) return rc;
    if ((rc = cuda_status(cudaMalloc(&s->inflow, tc->ntiles * kSlotStride * sizeof(float)), "tile scratch")))
        return rc;
    // slots without inflow are never written: they stay 0
    if ((rc = cuda_status(cudaMemset(s->inflow, 0, tc->ntiles * kSlotStride * sizeof(float)), "tile scratch")))
        return rc;
    if ((rc = cuda_status(cudaMalloc(&s->look_aggr, nb * sizeof(uint4)), "tile scratch"))) return rc;
    if ((rc = cuda_status(cudaMalloc(&s->look_incl, nb * sizeof(uint4)), "tile scratch"))) return rc;
    // total[2], the scan's ticket, its block flags
    s->ctl_bytes = 2 * sizeof(unsigned long long) + (1 + nb) * sizeof(unsigned);
    if ((rc = cuda_status(cudaMalloc(&s->total, s->ctl_bytes), "tile scratch"))) return rc;
    if ((rc = cuda_status(cudaMemset(s->total, 0, s->ctl_bytes), "tile scratch"))) return rc;
    if ((rc = cuda_status(cudaMalloc(&s->stat, tc->ntiles * sizeof(TileStat)), "tile scratch"))) return rc;
    s->bytes = E * (8 + 16) + nb * 32 + s->ctl_bytes + tc->ntiles * (sizeof(TileStat) + kSlotStride * 4);
    return LUE_GPU_OK;
}

void tile_scratch_free(TileScratch* s)
{
    cudaFree(s->P);
    cudaFree(s->S);
    cudaFree(s->inflow);
    cudaFree(s->look_aggr);
    cudaFree(s->look_incl);
    cudaFree(s->total);
    cudaFree(s->stat);
    *s = TileScratch{};
}

// CTAs of k_scan_exits that fit on the device at once (chunks of the exit-forest scan).  The result does
// not depend on it: the chunks' sums are exact.
static int64_t scan_ctas()
{
    static const int64_t n = [] {
        int dev = 0, sms = 0, per_sm = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_scan_exits, kTileThreads, 0) != cudaSuccess ||
            sms <= 0 || per_sm <= 0) {
            cudaGetLastError();
            return (int64_t)152;
        }
        return (int64_t)sms * per_sm;
    }();
    return n;
}

// accu (float32) on the tile engine.  Returns LUE_GPU_OK with `fallback` set on the device when the
// material holds +inf or its total is beyond the fixed-point range; the caller then runs the walk
// engine, guarded by that flag.
int tile_accu_f32(const TopologyCore* core, TileScratch* s, const float* ext, float ext_s, float* out,
                  cudaStream_t stream)
{
    const TileCore* tc = core->tiles;
    TileGeom g{core->rows, core->cols, tc->trows, tc->tcols};
    const TileForest f{tc->cell_at, tc->prev_at, s->inflow};
    // rows move as float4 when the columns are a multiple of 4 and the arrays 16-byte aligned
    const bool cols4 = (core->cols & 3) == 0;
    const bool vec_in = cols4 && (!ext || (reinterpret_cast<uintptr_t>(ext) & 15) == 0);
    const bool vec_out = cols4 && (reinterpret_cast<uintptr_t>(out) & 15) == 0;
    static const bool smem_ok = cudaFuncSetAttribute(k_tile_exits, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)sizeof(TileCallSmem)) == cudaSuccess &&
                                cudaFuncSetAttribute(k_tile_accu, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)sizeof(TileCallSmem)) == cudaSuccess;
    if (!smem_ok) return fail(LUE_GPU_ECUDA, "accu_f32 (tiles): shared memory attribute");
    const dim3 tile_grid((unsigned)tc->tcols, (unsigned)tc->trows);
    if (int rc = cuda_status(cudaMemsetAsync(s->total, 0, s->ctl_bytes, stream), "accu_f32 (tiles)")) return rc;
    k_tile_exits<<<tile_grid, kTileThreads, sizeof(TileCallSmem), stream>>>(g, ext, ext_s, vec_in, f, tc->exit_base,
                                                                            tc->exit_span, tc->exit_pos, s->P,
                                                                            s->total, s->stat);
    count_launches(1);
    const int64_t E = tc->nexit;
    if (E > 0) {
        const int64_t nb = (E + kScanBlock - 1) / kScanBlock;
        const int64_t chunk_blocks = (nb + scan_ctas() - 1) / scan_ctas();
        const int64_t nchunk = (nb + chunk_blocks - 1) / chunk_blocks;
        unsigned* ctl = reinterpret_cast<unsigned*>(s->total + 2);
        // test hook: LUE_GB300_TILE_POLLS (poll limit of a look-back wait; 0: every wait gives up at once,
        // and the walk engine redoes the call)
        int polls = kScanPolls;
        if (const char* e = getenv("LUE_GB300_TILE_POLLS")) polls = std::max(0, atoi(e));
        k_scan_exits<<<(unsigned)nchunk, kTileThreads, 0, stream>>>(s->P, E, chunk_blocks, s->total, ctl,
                                                                    s->look_aggr, s->look_incl, s->S, polls);
        count_launches(1);
        if (tc->nslot > 0) {
            k_slot_inflow<<<blocks_for(tc->nslot, 256), 256, 0, stream>>>(tc->nslot, tc->slot_at, tc->slot_first,
                                                                          tc->slot_edge, s->S, s->inflow, s->total);
            count_launches(1);
        }
    }
    k_tile_accu<<<tile_grid, kTileThreads, sizeof(TileCallSmem), stream>>>(g, ext, ext_s, vec_in && vec_out, out, f,
                                                                           s->stat, s->total);
    count_launches(1);
    return cuda_status(cudaGetLastError(), "accu_f32 (tiles)");
}

}  // namespace lue_gb300
