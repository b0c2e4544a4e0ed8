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
// Build: per-tile solve schedules
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

// Build: compile the solve schedule of one tile (CTA per tile).  The cells of the tile in the order the
// round solve finishes them, the round boundaries, the cells downstream of a tile entry ("through"
// cells) in the same rounds, the valid-cell bits and, per border cell, which outside neighbours drain
// into it.  Every call then replays the schedule instead of re-deriving it from the flow direction.
// kCount: first pass, only the number of rounds per tile (it sizes the round offset arrays).
template <bool kCount>
__global__ void __launch_bounds__(kTileThreads)
    k_tile_schedule(const uint8_t* __restrict__ fd, TileGeom g, int32_t* rounds_out, const int32_t* round_base,
                    uint16_t* sched_order, uint8_t* sched_upm, uint16_t* thr_order, uint8_t* thr_upm,
                    uint16_t* round_off, uint16_t* thr_round_off, uint16_t* tails, uint32_t* valid_bits,
                    uint8_t* border_in)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TileSmem& sm = *reinterpret_cast<TileSmem*>(smem_raw);
    const int64_t tile = blockIdx.x;
    const int64_t tr = tile / g.tcols, tc = tile % g.tcols;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint16_t* rstart = reinterpret_cast<uint16_t*>(sm.hi);                        // <= 4097 round starts
    uint8_t* thr = reinterpret_cast<uint8_t*>(sm.lo);                             // through flag per cell
    uint16_t* trstart = reinterpret_cast<uint16_t*>(reinterpret_cast<uint8_t*>(sm.lo) + kTileCells);
    int head = 0, count = tile_prepare(sm, fd, g, tr, tc), r = 0;
    // the rounds: a round holds the cells whose in-tile upstream cells are all in earlier rounds
    while (count > 0) {
        int* next = &sm.round_count[(r + 1) % 3];
        const int next_base = head + count;
        if (t == 0) {
            if (!kCount) rstart[r] = (uint16_t)head;
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
    if (kCount) {
        if (t == 0) rounds_out[tile] = rounds;
        return;
    }
    if (t == 0) rstart[rounds] = (uint16_t)nvalid;
    // entries (valid cells with an outside neighbour draining in), border masks, valid bits
    for (int i = t; i < kTileCells; i += kTileThreads) {
        int rin = i >> 6, cin = i & 63;
        bool valid = sm.fd[rin + 1][cin + 1] != kNoData;
        bool border = rin == 0 || rin == kTile - 1 || cin == 0 || cin == kTile - 1;
        unsigned outside = 0;
        if (valid && border) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                int hr = rin + nb_dr(q), hc = cin + nb_dc(q);
                if (hr >= 0 && hr < kTile && hc >= 0 && hc < kTile) continue;
                if (sm.fd[hr + 1][hc + 1] == nb_inflow_code(q)) outside |= 1u << q;
            }
        }
        thr[i] = outside ? 1 : 0;
        if (border) {
            int b = rin == 0           ? cin
                    : rin == kTile - 1 ? kTile + cin
                    : cin == 0         ? 2 * kTile + rin - 1
                                       : 3 * kTile - 2 + rin - 1;
            border_in[tile * kBorderCells + b] = (uint8_t)outside;
        }
        unsigned bal = __ballot_sync(0xffffffffu, valid);
        if (lane == 0) valid_bits[tile * (kTileCells / 32) + (i >> 5)] = bal;
    }
    __syncthreads();
    // Inside each round, order the cells by decreasing number of in-tile upstream cells, so that the
    // lanes of a warp loop over the same number of neighbours.  The downstream indices (dsl) and the
    // counters (cnt) are no longer needed: they hold the sorted order and the bucket counts.
    uint16_t* ord = sm.dsl;
    int* bucket = reinterpret_cast<int*>(sm.cnt);  // [0..8] counts, then fill positions
    for (int q = 0; q < rounds; ++q) {
        const int a = rstart[q], b = rstart[q + 1];
        if (b - a == 1) {
            if (t == 0) ord[a] = sm.queue[a];
            continue;
        }
        if (t < 9) bucket[t] = 0;
        __syncthreads();
        for (int k = a + t; k < b; k += kTileThreads) atomicAdd(&bucket[8 - __popc(sm.up[sm.queue[k]])], 1);
        __syncthreads();
        if (t == 0) {
            int acc = 0;
            for (int j = 0; j < 9; ++j) {
                int c = bucket[j];
                bucket[j] = acc;
                acc += c;
            }
        }
        __syncthreads();
        for (int k = a + t; k < b; k += kTileThreads) {
            int i = sm.queue[k];
            ord[a + atomicAdd(&bucket[8 - __popc(sm.up[i])], 1)] = (uint16_t)i;
        }
        __syncthreads();
    }
    // through flags, round by round: an entry, or downstream of a through cell
    for (int q = 0; q < rounds; ++q) {
        for (int k = rstart[q] + t; k < rstart[q + 1]; k += kTileThreads) {
            int i = ord[k];
            if (thr[i]) continue;
            unsigned m = sm.up[i];
            while (m) {
                int b = __ffs(m) - 1;
                m &= m - 1;
                if (thr[i + nb_dr(b) * kTile + nb_dc(b)]) {
                    thr[i] = 1;
                    break;
                }
            }
        }
        __syncthreads();
    }
    for (int k = t; k < nvalid; k += kTileThreads) {
        int i = ord[k];
        sched_order[tile * kTileCells + k] = (uint16_t)i;
        sched_upm[tile * kTileCells + k] = sm.up[i];
    }
    // the through cells of each round, in the same order, with upstream masks restricted to through cells
    int* wcount = bucket + 16;
    int j = 0;
    for (int q = 0; q < rounds; ++q) {
        if (t == 0) trstart[q] = (uint16_t)j;
        for (int k0 = rstart[q]; k0 < rstart[q + 1]; k0 += kTileThreads) {
            const int k = k0 + t;
            const int i = k < rstart[q + 1] ? ord[k] : 0;
            const bool f = k < rstart[q + 1] && thr[i];
            const unsigned bal = __ballot_sync(0xffffffffu, f);
            if (lane == 0) wcount[warp] = __popc(bal);
            __syncthreads();
            int before = 0, all = 0;
            for (int w = 0; w < kTileThreads / 32; ++w) {
                before += w < warp ? wcount[w] : 0;
                all += wcount[w];
            }
            if (f) {
                unsigned m = sm.up[i], tm = 0;
                while (m) {
                    int b = __ffs(m) - 1;
                    m &= m - 1;
                    if (thr[i + nb_dr(b) * kTile + nb_dc(b)]) tm |= 1u << b;
                }
                const int pos = j + before + __popc(bal & ((1u << lane) - 1u));
                thr_order[tile * kTileCells + pos] = (uint16_t)i;
                thr_upm[tile * kTileCells + pos] = (uint8_t)tm;
            }
            j += all;
            __syncthreads();  // wcount is rewritten by the next chunk
        }
    }
    if (t == 0) trstart[rounds] = (uint16_t)j;
    __syncthreads();
    const int32_t base = round_base[tile];
    for (int q = t; q <= rounds; q += kTileThreads) {
        round_off[base + q] = rstart[q];
        thr_round_off[base + q] = trstart[q];
    }
    // first round of the warp phase: every later round holds at most 32 cells
    if (t < 2) {
        const uint16_t* st = t == 0 ? rstart : trstart;
        int q = rounds;
        while (q > 0 && st[q] - st[q - 1] <= 32) --q;
        tails[tile * 2 + t] = (uint16_t)q;
    }
}

// ---------------------------------------------------------------------------------------------------
// Per call
// ---------------------------------------------------------------------------------------------------

// Cell i of a scheduled round: source (hi/lo before the cell is done) + the float-float sum of the
// upstream cells in mask m; NaN or a negative source makes the cell NaN; a sum that is not finite
// (+inf material) is recomputed plainly so that it keeps IEEE semantics.
__device__ __forceinline__ int tile_nb_offset(int q)
{
    static_assert(kTile == 64, "neighbour offsets are packed for 64-cell rows");
    // -65 -64 -63 -1 +1 +63 +64 +65 (NW N NE W E SW S SE) as signed bytes
    return (int)(signed char)(unsigned)(0x41403F01FFC1C0BFull >> (8 * q));
}

__device__ __forceinline__ void sched_cell(float* hi, float* lo, int i, unsigned m)
{
    const float x = hi[i];
    float s = x, e = lo[i];
    bool nan = isnan(x) || !(x >= 0.0f);
    unsigned mm = m;
    while (mm) {
        int u = i + tile_nb_offset(__ffs(mm) - 1);
        mm &= mm - 1;
        float h = hi[u], ts, te;
        nan |= isnan(h);
        two_sum(s, h, ts, te);
        s = ts;
        e = __fadd_rn(e, __fadd_rn(te, lo[u]));
    }
    float h = __fadd_rn(s, e);
    float l = __fsub_rn(e, __fsub_rn(h, s));
    if (!isfinite(h)) {
        float p = x;
        while (m) {
            p += hi[i + tile_nb_offset(__ffs(m) - 1)];
            m &= m - 1;
        }
        h = p;
        l = 0.0f;
    }
    if (nan) {
        h = __int_as_float(0x7fc00000);
        l = 0.0f;
    }
    hi[i] = h;
    lo[i] = l;
}

constexpr int kStagedRounds = 1023;  // round offsets held in shared memory; later ones are read from global

// The tile's values and one of its schedules, in shared memory (47 KB).
struct __align__(16) ReplaySmem {
    float hi[kTileCells];
    float lo[kTileCells];
    uint16_t order[kTileCells];
    uint8_t upm[kTileCells];
    uint16_t off[kStagedRounds + 1];
};

// Stage a schedule (order, masks: always the full 12 KB, so that the loads depend only on the tile
// index; round offsets) in shared memory.  Loads first, then stores, so that all are in flight at once.
__device__ __forceinline__ void replay_stage(ReplaySmem& sm, const uint16_t* __restrict__ order,
                                             const uint8_t* __restrict__ upm, const uint16_t* __restrict__ off,
                                             int rounds)
{
    const int t = threadIdx.x;
    const uint4* o4 = reinterpret_cast<const uint4*>(order);
    const uint4 a = __ldg(o4 + t), b = __ldg(o4 + t + kTileThreads);
    const uint4 c = __ldg(reinterpret_cast<const uint4*>(upm) + t);
    const int staged = min(rounds, kStagedRounds) + 1;
    uint16_t r0 = t < staged ? __ldg(off + t) : 0;
    reinterpret_cast<uint4*>(sm.order)[t] = a;
    reinterpret_cast<uint4*>(sm.order)[t + kTileThreads] = b;
    reinterpret_cast<uint4*>(sm.upm)[t] = c;
    if (t < staged) sm.off[t] = r0;
    for (int q = t + kTileThreads; q < staged; q += kTileThreads) sm.off[q] = __ldg(off + q);
}

// Replay `rounds` rounds: rounds before `tail` by the whole block (a barrier after each non-empty one),
// the rest (at most 32 cells each) by warp 0 alone.  Ends with a block barrier.
__device__ __forceinline__ void replay(ReplaySmem& sm, const uint16_t* __restrict__ off_g, int rounds, int tail)
{
    const int t = threadIdx.x;
    auto off = [&](int q) -> int { return q <= kStagedRounds ? sm.off[q] : __ldg(off_g + q); };
    int a = off(0);
    for (int q = 0; q < tail; ++q) {
        const int b = off(q + 1);
        if (b == a) continue;
        for (int k = a + t; k < b; k += kTileThreads) sched_cell(sm.hi, sm.lo, sm.order[k], sm.upm[k]);
        __syncthreads();
        a = b;
    }
    if (t < 32) {
        for (int q = tail; q < rounds; ++q) {
            const int b = off(q + 1);
            if (a + t < b) sched_cell(sm.hi, sm.lo, sm.order[a + t], sm.upm[a + t]);
            __syncwarp();
            a = b;
        }
    }
    __syncthreads();
}

// Cells of a tile by thread: thread t holds the 4 x 4 cells (row (t + 256 j) / 16, columns 4 ((t + 256 j)
// % 16) .. + 3), j = 0..3, so that a row of the tile is 16 float4.
__device__ __forceinline__ int quad_cell(int j) { return ((threadIdx.x + kTileThreads * j) >> 4) * kTile + ((threadIdx.x + kTileThreads * j) & 15) * 4; }

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

struct TileSched {
    const int32_t* round_base;
    const uint16_t* order;
    const uint8_t* upm;
    const uint16_t* off;
    const uint16_t* thr_order;
    const uint8_t* thr_upm;
    const uint16_t* thr_off;
    const uint16_t* tails;
    const uint32_t* valid_bits;
    const uint8_t* border_in;
    const int32_t* halo_exit;
};

// Pass 1: local accu inside each tile; local exit values to P (post-order); material total bound.
// vec: material and result rows can be moved as float4 (16-byte aligned, columns a multiple of 4).
__global__ void __launch_bounds__(kTileThreads)
    k_tile_local(TileGeom g, const float* __restrict__ ext, float ext_s, bool vec, float* __restrict__ out,
                 TileSched sc, const int32_t* __restrict__ exit_base, const uint16_t* __restrict__ exit_local,
                 const uint32_t* __restrict__ exit_pos, float2* __restrict__ P, unsigned long long* block_total)
{
    __shared__ ReplaySmem sm;
    __shared__ float warp_sum[kTileThreads / 32];
    __shared__ int warp_inf[kTileThreads / 32];
    const int64_t tile = blockIdx.x;
    const int64_t tr = tile / g.tcols, tc = tile % g.tcols;
    const int t = threadIdx.x;
    const int32_t rb = __ldg(sc.round_base + tile);
    const int rounds = __ldg(sc.round_base + tile + 1) - rb - 1;
    const int tail = __ldg(sc.tails + 2 * tile);
    const int32_t e0 = __ldg(exit_base + tile), ne = __ldg(exit_base + tile + 1) - e0;
    // material and valid bits of this thread's 16 cells
    float4 x[4];
    uint32_t vbits[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int cell = quad_cell(j);
        const int64_t r = tr * kTile + (cell >> 6), c = tc * kTile + (cell & 63);
        x[j] = ext ? load_quad(ext, g, r, c, vec, 0.0f) : make_float4(ext_s, ext_s, ext_s, ext_s);
        vbits[j] = __ldg(sc.valid_bits + tile * (kTileCells / 32) + (cell >> 5)) >> (cell & 31);
    }
    replay_stage(sm, sc.order + tile * kTileCells, sc.upm + tile * kTileCells, sc.off + rb, rounds);
    int my_loc = -1;
    uint32_t my_pos = 0;
    if (t < ne) {  // a tile has at most 252 exits (its border cells)
        my_loc = __ldg(exit_local + e0 + t);
        my_pos = __ldg(exit_pos + e0 + t);
    }
    float sum = 0.0f;
    bool inf = false;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int cell = quad_cell(j);
        float v[4] = {x[j].x, x[j].y, x[j].z, x[j].w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if ((vbits[j] >> k) & 1u) {
                if (isinf(v[k]) && v[k] > 0.0f) inf = true;
                else if (v[k] > 0.0f) sum += v[k];
            } else {
                v[k] = __int_as_float(0x7fc00000);  // no-data flow direction: never read, result NaN
            }
        }
        *reinterpret_cast<float4*>(sm.hi + cell) = make_float4(v[0], v[1], v[2], v[3]);
        *reinterpret_cast<float4*>(sm.lo + cell) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    __syncthreads();
    replay(sm, sc.off + rb, rounds, tail);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int cell = quad_cell(j);
        store_quad(out, g, tr * kTile + (cell >> 6), tc * kTile + (cell & 63), vec,
                   *reinterpret_cast<const float4*>(sm.hi + cell));
    }
    if (my_loc >= 0) P[my_pos] = make_float2(sm.hi[my_loc], sm.lo[my_loc]);
    // upper bound of this tile's material total, in 2^-16 units; ~0 marks +inf or overflow.  A float
    // sum of <= 4096 non-negative terms is within 4096 * 2^-24 of the exact sum, inside the 1e-4 margin.
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    unsigned any_inf = __any_sync(0xffffffffu, inf);
    if ((t & 31) == 0) {
        warp_sum[t >> 5] = sum;
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

// Pass 3: add the inflow entering each tile to every cell downstream of a tile entry.
__global__ void __launch_bounds__(kTileThreads)
    k_tile_fixup(TileGeom g, float* __restrict__ out, bool vec, TileSched sc, const uint4* __restrict__ A,
                 const unsigned long long* total)
{
    __shared__ ReplaySmem sm;
    if (total[1]) return;
    const int F = fixed_point_bits(total[0]);
    const int64_t tile = blockIdx.x;
    const int64_t tr = tile / g.tcols, tc = tile % g.tcols;
    const int t = threadIdx.x;
    const int32_t rb = __ldg(sc.round_base + tile);
    const int rounds = __ldg(sc.round_base + tile + 1) - rb - 1;
    const int tail = __ldg(sc.tails + 2 * tile + 1);
    const unsigned in_mask = t < kBorderCells ? __ldg(sc.border_in + tile * kBorderCells + t) : 0u;
    replay_stage(sm, sc.thr_order + tile * kTileCells, sc.thr_upm + tile * kTileCells, sc.thr_off + rb, rounds);
    float4 o[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int cell = quad_cell(j);
        o[j] = load_quad(out, g, tr * kTile + (cell >> 6), tc * kTile + (cell & 63), vec, 0.0f);
        *reinterpret_cast<float4*>(sm.hi + cell) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        *reinterpret_cast<float4*>(sm.lo + cell) = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    // sources: border cells gather the exact subtree sums of the halo exits draining into them
    u128 src = 0;
    int src_cell = -1;
    if (in_mask) {
        int rin, cin;
        if (t < kTile) { rin = 0; cin = t; }
        else if (t < 2 * kTile) { rin = kTile - 1; cin = t - kTile; }
        else if (t < 3 * kTile - 2) { rin = t - 2 * kTile + 1; cin = 0; }
        else { rin = t - (3 * kTile - 2) + 1; cin = kTile - 1; }
        unsigned m = in_mask;
        while (m) {
            int q = __ffs(m) - 1;
            m &= m - 1;
            int32_t id = __ldg(sc.halo_exit + tile * kHaloSlots + halo_slot_of(rin + nb_dr(q), cin + nb_dc(q)));
            if (id >= 0) src += to_u128(A[id]);
        }
        src_cell = rin * kTile + cin;
    }
    __syncthreads();  // the zeroing is done before the sources are written
    if (src_cell >= 0) {
        if ((src >> 96) != 0) {
            sm.hi[src_cell] = __int_as_float(0x7fc00000);
        } else {
            double d = fixed_to_double(src, F);
            float h = __double2float_rn(d);
            sm.hi[src_cell] = h;
            sm.lo[src_cell] = __double2float_rn(d - (double)h);
        }
    }
    __syncthreads();
    replay(sm, sc.thr_off + rb, rounds, tail);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int cell = quad_cell(j);
        const float4 h4 = *reinterpret_cast<const float4*>(sm.hi + cell);
        const float4 l4 = *reinterpret_cast<const float4*>(sm.lo + cell);
        const float hv[4] = {h4.x, h4.y, h4.z, h4.w}, lv[4] = {l4.x, l4.y, l4.z, l4.w};
        float v[4] = {o[j].x, o[j].y, o[j].z, o[j].w};
        bool changed = false;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (hv[k] == 0.0f && lv[k] == 0.0f) continue;
            changed = true;
            if (isnan(hv[k])) {
                v[k] = __int_as_float(0x7fc00000);
            } else {
                FF f{v[k], 0.0f};
                f.add(hv[k], lv[k]);
                f.normalise();
                v[k] = f.hi;
            }
        }
        if (changed)
            store_quad(out, g, tr * kTile + (cell >> 6), tc * kTile + (cell & 63), vec,
                       make_float4(v[0], v[1], v[2], v[3]));
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
    // solve schedules: rounds per tile, then the schedules themselves
    {
        const size_t smem = sizeof(TileSmem);
        TRY(cudaFuncSetAttribute(k_tile_schedule<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
            "tile schedule");
        TRY(cudaFuncSetAttribute(k_tile_schedule<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
            "tile schedule");
        TRY(cudaMalloc(&tc->round_base, (nt + 1) * sizeof(int32_t)), "tile round base");
        k_tile_schedule<true><<<(unsigned)nt, kTileThreads, smem, stream>>>(
            core->fd, g, count, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
            nullptr);
        TRY(cudaGetLastError(), "tile schedule");
        TRY(cudaMemcpyAsync(hcount.data(), count, nt * sizeof(int32_t), cudaMemcpyDeviceToHost, stream),
            "tile rounds");
        TRY(cudaStreamSynchronize(stream), "tile rounds");
        int64_t total = 0;
        for (int64_t i = 0; i < nt; ++i) {
            hbase[i] = (int32_t)total;
            total += hcount[i] + 1;
            if (total > INT32_MAX) {
                rc = fail(LUE_GPU_ERANGE, "tile topology: too many solve rounds");
                goto error;
            }
        }
        hbase[nt] = (int32_t)total;
        TRY(cudaMemcpyAsync(tc->round_base, hbase.data(), (nt + 1) * sizeof(int32_t), cudaMemcpyHostToDevice,
                            stream),
            "tile round base");
        TRY(cudaMalloc(&tc->round_off, total * sizeof(uint16_t)), "tile round offsets");
        TRY(cudaMalloc(&tc->thr_round_off, total * sizeof(uint16_t)), "tile round offsets");
        TRY(cudaMalloc(&tc->sched_order, nt * kTileCells * sizeof(uint16_t)), "tile schedule");
        TRY(cudaMalloc(&tc->sched_upm, nt * kTileCells), "tile schedule");
        TRY(cudaMalloc(&tc->thr_order, nt * kTileCells * sizeof(uint16_t)), "tile schedule");
        TRY(cudaMalloc(&tc->thr_upm, nt * kTileCells), "tile schedule");
        TRY(cudaMalloc(&tc->valid_bits, nt * (kTileCells / 32) * sizeof(uint32_t)), "tile valid bits");
        TRY(cudaMalloc(&tc->border_in, nt * kBorderCells), "tile border masks");
        TRY(cudaMalloc(&tc->tails, nt * 2 * sizeof(uint16_t)), "tile warp-phase rounds");
        k_tile_schedule<false><<<(unsigned)nt, kTileThreads, smem, stream>>>(
            core->fd, g, nullptr, tc->round_base, tc->sched_order, tc->sched_upm, tc->thr_order, tc->thr_upm,
            tc->round_off, tc->thr_round_off, tc->tails, tc->valid_bits, tc->border_in);
        TRY(cudaGetLastError(), "tile schedule");
        TRY(cudaStreamSynchronize(stream), "tile schedule");  // hbase must outlive its copy
        tc->bytes += (nt + 1) * 4 + total * 4 + nt * kTileCells * 6 + nt * (kTileCells / 8) + nt * kBorderCells +
                     nt * 4;
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
    cudaFree(tc->sched_order);
    cudaFree(tc->sched_upm);
    cudaFree(tc->thr_order);
    cudaFree(tc->thr_upm);
    cudaFree(tc->round_base);
    cudaFree(tc->round_off);
    cudaFree(tc->thr_round_off);
    cudaFree(tc->valid_bits);
    cudaFree(tc->border_in);
    cudaFree(tc->tails);
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
    const TileSched sc{tc->round_base, tc->sched_order, tc->sched_upm, tc->round_off, tc->thr_order,
                       tc->thr_upm,    tc->thr_round_off, tc->tails,     tc->valid_bits, tc->border_in,
                       tc->halo_exit};
    const bool vec_out = (reinterpret_cast<uintptr_t>(out) & 15) == 0 && (core->cols & 3) == 0;
    const bool vec = vec_out && (!ext || (reinterpret_cast<uintptr_t>(ext) & 15) == 0);
    k_tile_local<<<(unsigned)tc->ntiles, kTileThreads, 0, stream>>>(g, ext, ext_s, vec, out, sc, tc->exit_base,
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
        k_tile_fixup<<<(unsigned)tc->ntiles, kTileThreads, 0, stream>>>(g, out, vec_out, sc, s->A, s->total);
        count_launches(5);
    }
    return cuda_status(cudaGetLastError(), "accu_f32 (tiles)");
}

}  // namespace lue_gb300
