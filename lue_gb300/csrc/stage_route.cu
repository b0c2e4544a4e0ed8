// stage_route.cu — the stage engine (see stage_route.cuh): build, the wave kernel and its cell rules,
// and the routing entry points that use it.
#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "kinematic_wave_ff.cuh"
#include "route_walk_visitors.cuh"
#include "stage_route.cuh"
#include "topology.cuh"

namespace lue_gb300 {

// ---------------------------------------------------------------------------------------------------
// Build
// ---------------------------------------------------------------------------------------------------

// Crossing depth: the largest number of tile edges crossed by a flow path ending at the cell, by the
// upstream-first walk of walk.cuh.
struct CrossDepthVisitor {
    const uint8_t* upmask;
    int32_t* depth;
    int64_t cols;
    __device__ void enter(int64_t c)
    {
        const int64_t r = c / cols, col = c - r * cols;
        const int64_t tr = r / kStageSide, tc = col / kStageSide;
        unsigned m = __ldg(upmask + c);
        int32_t d = 0;
        while (m) {
            const int k = __ffs(m) - 1;
            m &= m - 1;
            const int64_t ur = r + nb_dr(k), uc = col + nb_dc(k);
            int32_t du = load_cg(depth + ur * cols + uc);
            if (ur / kStageSide != tr || uc / kStageSide != tc) ++du;
            d = du > d ? du : d;
        }
        depth[c] = d;
    }
    __device__ void no_data(int64_t c) { depth[c] = -1; }
};

struct StageGeom {
    int64_t rows, cols, tcols;
};

// In-tile cell of position p of the tile (row-major) and its global index; false outside the array.
__device__ __forceinline__ bool stage_cell(const StageGeom& g, int64_t tr, int64_t tc, int p, int64_t& gi)
{
    const int64_t r = tr * kStageSide + (p >> 5), c = tc * kStageSide + (p & 31);
    gi = r * g.cols + c;
    return r < g.rows && c < g.cols;
}

// Inclusive scan of one int per thread over the build CTA; total gets the block sum.
__device__ __forceinline__ int build_scan(int v, int* warp_tot, int& total)
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
    for (int w = 0; w < kStageBuildThreads / 32; ++w) {
        const int s = warp_tot[w];
        before += w < warp ? s : 0;
        total += s;
    }
    __syncthreads();
    return before + x;
}

struct StageSortSmem {
    unsigned long long key[kStageCells];
    int32_t d[kStageCells];
    int16_t sd[kStageCells];  // downstream cell in the same depth group, or -1
    int16_t h[kStageCells];   // distance to the depth group's most downstream cell
    int16_t J[kStageCells];
    int16_t ss[kStageCells];  // by in-tile cell: the sorted position of the first cell of its stage, or -1
    int warp_tot[kStageBuildThreads / 32];
};

// Per tile: the order of its valid cells by (depth, distance to the depth group's most downstream cell),
// cut into stages of at most `cap` consecutive cells of one depth; the rounds; and per position a flag
// word (bit 0: first cell of a stage, bit 1: the outflow leaves the stage, bits 2-9: mask of the upstream
// neighbours in other stages); counts[4 tile ..] = stages, exits, inputs, valid cells.  The cells of a
// depth group sorted by decreasing distance have every upstream cell of the group before them, so any cut
// of that order into consecutive pieces gives stages whose in-tile inputs come from earlier stages.
__global__ void __launch_bounds__(kStageBuildThreads)
    k_stage_sort(const uint8_t* __restrict__ fd, const uint8_t* __restrict__ upmask, const int32_t* __restrict__ depth,
                 StageGeom g, int cap, uint16_t* order, uint16_t* round_at, uint16_t* flags_at, int32_t* counts)
{
    __shared__ StageSortSmem sm;
    const int64_t tr = blockIdx.y, tc = blockIdx.x, tile = tr * g.tcols + tc;
    const int t = threadIdx.x;
    for (int p = t; p < kStageCells; p += kStageBuildThreads) {
        int64_t gi;
        sm.d[p] = stage_cell(g, tr, tc, p, gi) ? __ldg(depth + gi) : -1;
    }
    __syncthreads();
    for (int p = t; p < kStageCells; p += kStageBuildThreads) {
        int s = -1;
        int64_t gi;
        if (sm.d[p] >= 0 && stage_cell(g, tr, tc, p, gi)) {
            int dr, dc;
            const int pr = (p >> 5) + 0, pc = p & 31;
            if (d8_offset(__ldg(fd + gi), dr, dc)) {
                const int qr = pr + dr, qc = pc + dc;
                const int64_t gr = tr * kStageSide + qr, gc = tc * kStageSide + qc;
                if (qr >= 0 && qr < kStageSide && qc >= 0 && qc < kStageSide && gr < g.rows && gc < g.cols &&
                    sm.d[qr * kStageSide + qc] == sm.d[p])
                    s = qr * kStageSide + qc;
            }
        }
        sm.sd[p] = (int16_t)s;
        sm.h[p] = (int16_t)(s >= 0 ? 1 : 0);
        sm.J[p] = (int16_t)(s >= 0 ? s : p);
    }
    __syncthreads();
    // distances to the stage's most downstream cell, by pointer jumping (chains of at most 1024 cells)
    for (int it = 0; it < 10; ++it) {
        int nh[2], nj[2];
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int p = t + k * kStageBuildThreads, j = sm.J[p];
            nh[k] = sm.h[p] + (j != p ? sm.h[j] : 0);
            nj[k] = sm.J[j];
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const int p = t + k * kStageBuildThreads;
            sm.h[p] = (int16_t)nh[k];
            sm.J[p] = (int16_t)nj[k];
        }
        __syncthreads();
    }
    for (int p = t; p < kStageCells; p += kStageBuildThreads)
        sm.key[p] = sm.d[p] >= 0 ? ((unsigned long long)sm.d[p] << 20) | ((unsigned long long)(1023 - sm.h[p]) << 10) |
                                       (unsigned long long)p
                                 : ~0ull;
    __syncthreads();
    // bitonic sort, ascending
    for (int k = 2; k <= kStageCells; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = t; i < kStageCells; i += kStageBuildThreads) {
                const int l = i ^ j;
                if (l > i) {
                    const unsigned long long a = sm.key[i], b = sm.key[l];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        sm.key[i] = b;
                        sm.key[l] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
    // per position (thread t: positions 2t, 2t + 1): depth-group starts
    int first[2];
    for (int k = 0; k < 2; ++k) {
        const int i = 2 * t + k;
        const unsigned long long key = sm.key[i];
        first[k] = key != ~0ull && (i == 0 || (int)(sm.key[i - 1] >> 20) != (int)(key >> 20));
    }
    // the first position of each position's depth group: inclusive max-scan of start positions
    int mine = -1;
    for (int k = 0; k < 2; ++k)
        if (first[k]) mine = 2 * t + k;
    {
        const int lane = t & 31, warp = t >> 5;
        int x = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x = max(x, y);
        }
        if (lane == 31) sm.warp_tot[warp] = x;
        __syncthreads();
        int before = -1;
        for (int w = 0; w < warp; ++w) before = max(before, sm.warp_tot[w]);
        const int excl_lane = __shfl_up_sync(0xffffffffu, x, 1);
        mine = max(before, lane ? excl_lane : -1);  // last start strictly before position 2t
        __syncthreads();
    }
    // stages: pieces of `cap` consecutive positions of a depth group
    int stage_first[2];
    for (int p = t; p < kStageCells; p += kStageBuildThreads) sm.ss[p] = -1;
    __syncthreads();
    for (int k = 0; k < 2; ++k) {
        const int i = 2 * t + k;
        const unsigned long long key = sm.key[i];
        stage_first[k] = -1;
        if (key == ~0ull) continue;
        if (first[k]) mine = i;
        stage_first[k] = mine + (i - mine) / cap * cap;
        sm.ss[key & 1023] = (int16_t)stage_first[k];
    }
    __syncthreads();
    int starts = 0, exits = 0, inputs = 0, valid = 0;
    for (int k = 0; k < 2; ++k) {
        const int i = 2 * t + k;
        const unsigned long long key = sm.key[i];
        uint16_t flag = 0, rnd = 0;
        if (key != ~0ull) {
            const int sf = stage_first[k];
            const int p = (int)(key & 1023);
            const int hh = 1023 - (int)((key >> 10) & 1023);
            const int hs = 1023 - (int)((sm.key[sf] >> 10) & 1023);
            rnd = (uint16_t)(hs - hh);
            int64_t gi;
            stage_cell(g, tr, tc, p, gi);
            const int pr = p >> 5, pc = p & 31;
            // exit: the downstream cell is valid and in another stage
            int dr, dc;
            bool ex = false;
            if (d8_offset(__ldg(fd + gi), dr, dc)) {
                const int64_t gr = tr * kStageSide + pr + dr, gc = tc * kStageSide + pc + dc;
                if (gr >= 0 && gr < g.rows && gc >= 0 && gc < g.cols) {
                    const int qr = pr + dr, qc = pc + dc;
                    const bool in = qr >= 0 && qr < kStageSide && qc >= 0 && qc < kStageSide;
                    ex = in ? sm.d[qr * kStageSide + qc] >= 0 && sm.ss[qr * kStageSide + qc] != sf
                            : __ldg(depth + gr * g.cols + gc) >= 0;
                }
            }
            // inputs: upstream cells in other stages
            unsigned m = __ldg(upmask + gi), em = 0;
            while (m) {
                const int q = __ffs(m) - 1;
                m &= m - 1;
                const int qr = pr + nb_dr(q), qc = pc + nb_dc(q);
                const bool in = qr >= 0 && qr < kStageSide && qc >= 0 && qc < kStageSide;
                if (!in || sm.ss[qr * kStageSide + qc] != sf) em |= 1u << q;
            }
            flag = (uint16_t)((i == sf ? 1 : 0) | (ex ? 2 : 0) | (em << 2));
            starts += i == sf;
            exits += ex;
            inputs += __popc(em);
            ++valid;
            order[tile * kStageCells + i] = (uint16_t)p;
        } else {
            order[tile * kStageCells + i] = 0xFFFFu;
        }
        round_at[tile * kStageCells + i] = rnd;
        flags_at[tile * kStageCells + i] = flag;
    }
    int tot;
    build_scan(starts, sm.warp_tot, tot);
    if (t == 0) counts[4 * tile + 0] = tot;
    build_scan(exits, sm.warp_tot, tot);
    if (t == 0) counts[4 * tile + 1] = tot;
    build_scan(inputs, sm.warp_tot, tot);
    if (t == 0) counts[4 * tile + 2] = tot;
    build_scan(valid, sm.warp_tot, tot);
    if (t == 0) counts[4 * tile + 3] = tot;
}

// Per tile, with the global bases of its stages, exits and inputs: stage records, exit rows (by
// position, and by global cell for the input lists), meta, and the first input of each position.
__global__ void __launch_bounds__(kStageBuildThreads)
    k_stage_ids(const uint8_t* __restrict__ upmask, const int32_t* __restrict__ depth, StageGeom g,
                const uint16_t* __restrict__ order, const uint16_t* __restrict__ round_at,
                const uint16_t* __restrict__ flags_at, const int32_t* __restrict__ bases, int4* stage,
                int32_t* stage_depth, int32_t* exit_id, int32_t* cell_exit, int32_t* input_at, uint2* meta,
                int32_t* exit_stage)
{
    __shared__ int warp_tot[kStageBuildThreads / 32];
    __shared__ int s_begin[kStageCells], s_count[kStageCells], s_rounds[kStageCells], s_in0[kStageCells];
    __shared__ int s_nin[kStageCells];
    __shared__ int32_t d[kStageCells];
    const int64_t tr = blockIdx.y, tc = blockIdx.x, tile = tr * g.tcols + tc;
    const int t = threadIdx.x;
    for (int p = t; p < kStageCells; p += kStageBuildThreads) {
        int64_t gi;
        d[p] = stage_cell(g, tr, tc, p, gi) ? __ldg(depth + gi) : -1;
        s_count[p] = 0;
        s_rounds[p] = 0;
        s_nin[p] = 0;
    }
    const int stage_base = bases[4 * tile + 0], exit_base = bases[4 * tile + 1], input_base = bases[4 * tile + 2];
    uint16_t o[2], r[2], f[2];
    int starts = 0, exits = 0, ins = 0;
    for (int k = 0; k < 2; ++k) {
        const int i = 2 * t + k;
        o[k] = order[tile * kStageCells + i];
        r[k] = round_at[tile * kStageCells + i];
        f[k] = flags_at[tile * kStageCells + i];
        if (o[k] != 0xFFFFu) {
            starts += f[k] & 1;
            exits += (f[k] >> 1) & 1;
            ins += __popc(f[k] >> 2);
        }
    }
    int tot;
    const int s_excl = build_scan(starts, warp_tot, tot) - starts;
    const int e_excl = build_scan(exits, warp_tot, tot) - exits;
    const int i_excl = build_scan(ins, warp_tot, tot) - ins;
    // stage of each position: the count of starts up to it, minus one
    int local[2];
    {
        int s_run = s_excl, i_cur = i_excl;
        for (int k = 0; k < 2; ++k) {
            const int i = 2 * t + k;
            local[k] = -1;
            if (o[k] == 0xFFFFu) continue;
            if (f[k] & 1) {
                s_begin[s_run] = i;
                s_in0[s_run] = i_cur;
                ++s_run;
            }
            local[k] = s_run - 1;
            i_cur += __popc(f[k] >> 2);
        }
    }
    __syncthreads();
    for (int k = 0; k < 2; ++k) {
        if (local[k] < 0) continue;
        atomicAdd(&s_count[local[k]], 1);
        atomicMax(&s_rounds[local[k]], (int)r[k] + 1);
        atomicAdd(&s_nin[local[k]], __popc(f[k] >> 2));
    }
    __syncthreads();
    int e_run = e_excl, i_cur = i_excl;
    for (int k = 0; k < 2; ++k) {
        const int i = 2 * t + k;
        const int64_t at = tile * kStageCells + i;
        if (o[k] == 0xFFFFu) {
            exit_id[at] = -1;
            input_at[at] = -1;
            meta[at] = make_uint2(0u, 0u);
            continue;
        }
        const int p = o[k], dd = d[p];
        int64_t gi;
        stage_cell(g, tr, tc, p, gi);
        int32_t id = -1;
        if ((f[k] >> 1) & 1) {
            id = exit_base + e_run++;
            cell_exit[gi] = id;
            exit_stage[id] = stage_base + local[k];
        }
        exit_id[at] = id;
        const unsigned um = __ldg(upmask + gi), em = f[k] >> 2;
        const int ls = local[k];
        input_at[at] = input_base + i_cur;
        const unsigned first_input = (unsigned)(i_cur - s_in0[ls]);
        i_cur += __popc(em);
        meta[at] = make_uint2((unsigned)p | ((unsigned)r[k] << 10), um | (em << 8) | (first_input << 16));
        if (f[k] & 1) {
            const int sid = stage_base + ls;
            stage[sid] = make_int4((int)tile, s_begin[ls] | (s_count[ls] << 16), s_rounds[ls] | (s_nin[ls] << 16),
                                   input_base + s_in0[ls]);
            stage_depth[sid] = dd;
        }
    }
}

// Per tile, once every exit has its row: the input lists (the history row of each upstream cell in
// another stage, in neighbour order).
__global__ void __launch_bounds__(kStageBuildThreads)
    k_stage_inputs(StageGeom g, const uint16_t* __restrict__ order, const uint2* __restrict__ meta,
                   const int32_t* __restrict__ input_at, const int32_t* __restrict__ cell_exit, int32_t* inputs,
                   int* error)
{
    const int64_t tr = blockIdx.y, tc = blockIdx.x, tile = tr * g.tcols + tc;
    for (int i = threadIdx.x; i < kStageCells; i += kStageBuildThreads) {
        const int64_t at = tile * kStageCells + i;
        const uint16_t p = order[at];
        if (p == 0xFFFFu) continue;
        unsigned em = (meta[at].y >> 8) & 0xFFu;
        if (!em) continue;
        int64_t gi;
        stage_cell(g, tr, tc, p, gi);
        int32_t w = input_at[at];
        while (em) {
            const int q = __ffs(em) - 1;
            em &= em - 1;
            const int32_t id = cell_exit[gi + nb_dr(q) * g.cols + nb_dc(q)];
            if (id < 0) *error = 1;
            inputs[w++] = id;
        }
    }
}

// Stage ids of the exits -> positions in the depth order.
__global__ void k_remap_i32(int32_t* v, int64_t n, const int32_t* __restrict__ map)
{
    for (int64_t i = grid_stride_begin(); i < n; i += grid_stride()) v[i] = map[v[i]];
}

// Per stage (block per position k of the depth order): the stages whose exits feed it, each with the
// earliest round at which one of its cells consumes them, and the latest round of the stage's own exits.
// Pass 1 (list == nullptr) counts the producers; pass 2 writes them at offsets[k].
__global__ void __launch_bounds__(256)
    k_stage_producers(const int4* __restrict__ stage, const int32_t* __restrict__ wave_stage, int64_t nstages,
                      const uint2* __restrict__ meta, const int32_t* __restrict__ exit_id,
                      const int32_t* __restrict__ inputs, const int32_t* __restrict__ exit_stage, int32_t* counts,
                      int32_t* max_exit_round, const int64_t* __restrict__ offsets, int2* list)
{
    extern __shared__ int2 pairs[];  // [inputs of the stage]: (producer position, consumer round)
    __shared__ int s_max_exit;
    const int64_t k = blockIdx.x;
    if (k >= nstages) return;
    const int4 st = stage[wave_stage[k]];
    const int64_t tile = st.x;
    const int begin = st.y & 0xFFFF, count = (int)((unsigned)st.y >> 16), nin = (int)((unsigned)st.z >> 16);
    const int64_t in_base = st.w;
    if (threadIdx.x == 0) s_max_exit = -1;
    __syncthreads();
    for (int i = threadIdx.x; i < count; i += blockDim.x) {
        const int64_t at = tile * kStageCells + begin + i;
        const uint2 m = meta[at];
        const int rd = (int)((m.x >> 10) & 1023u);
        if (exit_id[at] >= 0) atomicMax(&s_max_exit, rd);
        const unsigned em = (m.y >> 8) & 0xFFu;
        const int fi = (int)(m.y >> 16), ne = __popc(em);
        for (int j = 0; j < ne; ++j) pairs[fi + j] = make_int2(exit_stage[inputs[in_base + fi + j]], rd);
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    // distinct producers with their smallest consumer round (nin is small: at most a few hundred)
    int distinct = 0;
    for (int i = 0; i < nin; ++i) {
        int2 pi = pairs[i];
        int j = 0;
        for (; j < distinct; ++j)
            if (pairs[j].x == pi.x) break;
        if (j == distinct) pairs[distinct++] = pi;
        else pairs[j].y = min(pairs[j].y, pi.y);
    }
    if (!list) {
        counts[k] = distinct;
        max_exit_round[k] = s_max_exit;
    } else {
        for (int j = 0; j < distinct; ++j) list[offsets[k] + j] = pairs[j];
    }
}

static inline int64_t div_up(int64_t a, int64_t b) { return (a + b - 1) / b; }

int stage_core_build(const TopologyCore* core, uint32_t* work, cudaStream_t stream, StageCore** out)
{
    *out = nullptr;
    const int64_t n = core->n, rows = core->rows, cols = core->cols;
    auto* sc = new (std::nothrow) StageCore();
    if (!sc) return fail(LUE_GPU_ENOMEM, "stage topology: host allocation");
    if (core->stage_cap > 0) sc->cap = std::min(kStageMaxCap, core->stage_cap);
    else if (const char* e = getenv("LUE_GB300_STAGE_CAP")) sc->cap = std::max(1, std::min(kStageMaxCap, atoi(e)));
    sc->trows = div_up(rows, kStageSide);
    sc->tcols = div_up(cols, kStageSide);
    sc->ntiles = sc->trows * sc->tcols;
    const int64_t nt = sc->ntiles, np = nt * kStageCells;
    if (sc->trows > 65535) {
        delete sc;
        return fail(LUE_GPU_ERANGE, "stage topology: more than 65535 rows of 32-cell tiles");
    }
    const StageGeom g{rows, cols, sc->tcols};
    const dim3 grid((unsigned)sc->tcols, (unsigned)sc->trows);
    int32_t *depth = nullptr, *counts = nullptr, *bases = nullptr, *cell_exit = nullptr, *input_at = nullptr;
    int32_t *stage_depth = nullptr, *error = nullptr, *exit_stage = nullptr, *pos_of = nullptr, *pcount = nullptr;
    uint16_t *order = nullptr, *round_at = nullptr, *flags_at = nullptr;
    std::vector<int32_t> hc(4 * nt), hb(4 * nt);
    int herr = 0;
    int rc = 0;
#define TRY(call, what) \
    if ((rc = cuda_status((call), what))) goto done
    TRY(cudaMalloc(&depth, n * sizeof(int32_t)), "stage depth");
    TRY(cudaMalloc(&order, np * sizeof(uint16_t)), "stage order");
    TRY(cudaMalloc(&round_at, np * sizeof(uint16_t)), "stage rounds");
    TRY(cudaMalloc(&flags_at, np * sizeof(uint16_t)), "stage flags");
    TRY(cudaMalloc(&counts, 4 * nt * sizeof(int32_t)), "stage counts");
    TRY(cudaMalloc(&bases, 4 * nt * sizeof(int32_t)), "stage bases");
    TRY(cudaMalloc(&error, sizeof(int)), "stage flag");
    TRY(cudaMemsetAsync(error, 0, sizeof(int), stream), "memset");
    // crossing depths by the upstream-first walk
    TRY(cudaMemcpyAsync(work, core->count, words_for(n) * 4, cudaMemcpyDeviceToDevice, stream), "stage depth");
    {
        WalkGrid wg{core->fd, core->count, work, rows, cols, n};
        CrossDepthVisitor v{core->upmask, depth, cols};
        k_walk<<<grid_all(n, 256), 256, 0, stream>>>(wg, v);
    }
    k_stage_sort<<<grid, kStageBuildThreads, 0, stream>>>(core->fd, core->upmask, depth, g, sc->cap, order, round_at,
                                                         flags_at, counts);
    count_launches(2);
    TRY(cudaGetLastError(), "stage sort");
    TRY(cudaMemcpyAsync(hc.data(), counts, 4 * nt * sizeof(int32_t), cudaMemcpyDeviceToHost, stream), "stage counts");
    TRY(cudaStreamSynchronize(stream), "stage counts");
    {
        int64_t tot[3] = {0, 0, 0};
        for (int64_t i = 0; i < nt; ++i) {
            for (int k = 0; k < 3; ++k) {
                hb[4 * i + k] = (int32_t)tot[k];
                tot[k] += hc[4 * i + k];
            }
            hb[4 * i + 3] = 0;
        }
        if (tot[0] >= INT32_MAX || tot[1] >= INT32_MAX || tot[2] >= INT32_MAX) {
            rc = fail(LUE_GPU_ERANGE, "stage topology: too many stages, exits or inputs");
            goto done;
        }
        sc->nstages = tot[0];
        sc->nexits = tot[1];
        sc->ninputs = tot[2];
    }
    TRY(cudaMemcpyAsync(bases, hb.data(), 4 * nt * sizeof(int32_t), cudaMemcpyHostToDevice, stream), "stage bases");
    TRY(cudaMalloc(&sc->stage, std::max<int64_t>(sc->nstages, 1) * sizeof(int4)), "stages");
    TRY(cudaMalloc(&stage_depth, std::max<int64_t>(sc->nstages, 1) * sizeof(int32_t)), "stage depths");
    TRY(cudaMalloc(&sc->exit_id, np * sizeof(int32_t)), "stage exits");
    TRY(cudaMalloc(&sc->meta, np * sizeof(uint2)), "stage meta");
    TRY(cudaMalloc(&sc->inputs, std::max<int64_t>(sc->ninputs, 1) * sizeof(int32_t)), "stage inputs");
    TRY(cudaMalloc(&cell_exit, n * sizeof(int32_t)), "stage exit map");
    TRY(cudaMalloc(&input_at, np * sizeof(int32_t)), "stage input map");
    TRY(cudaMemsetAsync(cell_exit, 0xFF, n * sizeof(int32_t), stream), "memset");
    TRY(cudaMalloc(&exit_stage, std::max<int64_t>(sc->nexits, 1) * sizeof(int32_t)), "stage exit owners");
    k_stage_ids<<<grid, kStageBuildThreads, 0, stream>>>(core->upmask, depth, g, order, round_at, flags_at, bases,
                                                        sc->stage, stage_depth, sc->exit_id, cell_exit, input_at,
                                                        sc->meta, exit_stage);
    k_stage_inputs<<<grid, kStageBuildThreads, 0, stream>>>(g, order, sc->meta, input_at, cell_exit, sc->inputs, error);
    count_launches(2);
    TRY(cudaGetLastError(), "stage ids");
    {
        // stages in depth order: counting sort by depth (host); any order with every producer before its
        // consumers would do, and the ticket order below is one
        std::vector<int32_t> sd(sc->nstages);
        std::vector<int4> srec(sc->nstages);
        TRY(cudaMemcpyAsync(sd.data(), stage_depth, sc->nstages * sizeof(int32_t), cudaMemcpyDeviceToHost, stream),
            "stage depths");
        TRY(cudaMemcpyAsync(srec.data(), sc->stage, sc->nstages * sizeof(int4), cudaMemcpyDeviceToHost, stream),
            "stage records");
        TRY(cudaMemcpyAsync(&herr, error, sizeof(int), cudaMemcpyDeviceToHost, stream), "stage flag");
        TRY(cudaStreamSynchronize(stream), "stage build");
        if (herr) {
            rc = fail(LUE_GPU_EINVAL, "stage topology: an input without a history row");
            goto done;
        }
        int32_t maxd = 0;
        for (int32_t v : sd) maxd = std::max(maxd, v);
        sc->max_depth = sc->nstages ? maxd : -1;
        std::vector<int64_t> off(maxd + 2, 0);
        for (int32_t v : sd) ++off[v + 1];
        int64_t mx = 0;
        for (int32_t d = 0; d <= maxd; ++d) {
            mx = std::max(mx, off[d + 1]);
            off[d + 1] += off[d];
        }
        sc->max_stages_per_depth = mx;
        std::vector<int32_t> ws(sc->nstages);
        std::vector<int64_t> cur(off.begin(), off.end() - 1);
        for (int64_t s = 0; s < sc->nstages; ++s) ws[cur[sd[s]]++] = (int32_t)s;
        for (int64_t s2 = 0; s2 < sc->nstages; ++s2) {
            const int4& r = srec[s2];
            sc->max_stage_cells = std::max<int64_t>(sc->max_stage_cells, (int)((unsigned)r.y >> 16));
            sc->max_stage_inputs = std::max<int64_t>(sc->max_stage_inputs, (int)((unsigned)r.z >> 16));
        }
        TRY(cudaMalloc(&sc->wave_stage, std::max<int64_t>(sc->nstages, 1) * sizeof(int32_t)), "wave order");
        TRY(cudaMemcpyAsync(sc->wave_stage, ws.data(), sc->nstages * sizeof(int32_t), cudaMemcpyHostToDevice, stream),
            "wave order");
        TRY(cudaStreamSynchronize(stream), "stage build");  // the host vectors must outlive the copies
        // dataflow order: exit owners as wave positions, then each stage's producers
        std::vector<int32_t> pos(sc->nstages);
        for (int64_t k = 0; k < sc->nstages; ++k) pos[ws[k]] = (int32_t)k;
        TRY(cudaMalloc(&pos_of, std::max<int64_t>(sc->nstages, 1) * sizeof(int32_t)), "wave positions");
        TRY(cudaMemcpyAsync(pos_of, pos.data(), sc->nstages * sizeof(int32_t), cudaMemcpyHostToDevice, stream),
            "wave positions");
        if (sc->nexits > 0)
            k_remap_i32<<<grid_for(sc->nexits, 256), 256, 0, stream>>>(exit_stage, sc->nexits, pos_of);
        TRY(cudaMalloc(&pcount, std::max<int64_t>(sc->nstages, 1) * sizeof(int32_t)), "producers");
        TRY(cudaMalloc(&sc->max_exit_round, std::max<int64_t>(sc->nstages, 1) * sizeof(int32_t)), "producers");
        TRY(cudaMalloc(&sc->prod_offsets, (sc->nstages + 1) * sizeof(int64_t)), "producers");
        const size_t psm = (size_t)std::max<int64_t>(sc->max_stage_inputs, 1) * sizeof(int2);
        if (psm > 48 * 1024)
            TRY(cudaFuncSetAttribute(k_stage_producers, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)psm),
                "producers");
        if (sc->nstages > 0)
            k_stage_producers<<<(unsigned)sc->nstages, 256, psm, stream>>>(sc->stage, sc->wave_stage, sc->nstages,
                                                                          sc->meta, sc->exit_id, sc->inputs,
                                                                          exit_stage, pcount, sc->max_exit_round,
                                                                          nullptr, nullptr);
        std::vector<int32_t> pc(sc->nstages);
        std::vector<int64_t> po(sc->nstages + 1, 0);
        TRY(cudaMemcpyAsync(pc.data(), pcount, sc->nstages * sizeof(int32_t), cudaMemcpyDeviceToHost, stream),
            "producers");
        TRY(cudaStreamSynchronize(stream), "producers");
        for (int64_t k = 0; k < sc->nstages; ++k) {
            po[k + 1] = po[k] + pc[k];
            sc->max_producers = std::max<int64_t>(sc->max_producers, pc[k]);
        }
        TRY(cudaMemcpyAsync(sc->prod_offsets, po.data(), (sc->nstages + 1) * sizeof(int64_t), cudaMemcpyHostToDevice,
                            stream),
            "producers");
        TRY(cudaMalloc(&sc->prod, std::max<int64_t>(po[sc->nstages], 1) * sizeof(int2)), "producers");
        if (sc->nstages > 0)
            k_stage_producers<<<(unsigned)sc->nstages, 256, psm, stream>>>(sc->stage, sc->wave_stage, sc->nstages,
                                                                          sc->meta, sc->exit_id, sc->inputs,
                                                                          exit_stage, pcount, sc->max_exit_round,
                                                                          sc->prod_offsets, sc->prod);
        count_launches(3);
        TRY(cudaGetLastError(), "producers");
        TRY(cudaStreamSynchronize(stream), "producers");  // po must outlive the copy
        sc->bytes += (sc->nstages + 1) * 8 + po[sc->nstages] * 8 + sc->nstages * 4;
        // Ticket order: the stages sorted by their latest start in a model of a one-step call (a stage
        // can start kHandOffRounds after the last exit round of its last producer; its latest start is
        // the last one that still lets every stage it feeds start in time for the whole call to finish at
        // the model's earliest end), so that CTAs take the stages with least slack, the critical chain,
        // first among those that can start at about the same time.  A producer's latest start is always
        // earlier than its consumers', so the order keeps every producer before the stages it feeds.
        // LUE_GPU_STAGE_ORDER_EARLIEST sorts by the earliest start instead (about the order in which the
        // stages' inputs become ready: fewer waiting CTAs, for servers that run many calls at once; alone
        // on the GPU it is slower: one kinematic-wave step at 8192^2 20.1 ms against 15.4 ms, 100 steps
        // 1.55 against 1.36 ms per step).
        {
            // the model's hand-off between a producer's last exit round and a consumer's start, in rounds:
            // 2 for the earliest-start order; 32 for the latest-start order (measured at 8192^2, 100
            // kinematic-wave steps: 136.0 ms at 2, 133.3 at 6, 131.1-131.5 from 16 to 128).
            // LUE_GB300_STAGE_HANDOFF overrides it.
            int64_t kHandOffRounds = core->stage_order == LUE_GPU_STAGE_ORDER_EARLIEST ? 2 : 32;
            if (const char* e = getenv("LUE_GB300_STAGE_HANDOFF")) kHandOffRounds = std::max(0, atoi(e));
            const int64_t ns = sc->nstages, npairs = po[ns];
            std::vector<int2> pr(std::max<int64_t>(1, npairs));
            std::vector<int32_t> mxr(ns);
            TRY(cudaMemcpy(pr.data(), sc->prod, npairs * sizeof(int2), cudaMemcpyDeviceToHost), "stage order");
            TRY(cudaMemcpy(mxr.data(), sc->max_exit_round, ns * sizeof(int32_t), cudaMemcpyDeviceToHost),
                "stage order");
            std::vector<int64_t> start(ns, 0);
            int64_t last = 0, finish = 0;
            for (int64_t k = 0; k < ns; ++k) {
                int64_t s0 = 0;
                for (int64_t j = po[k]; j < po[k + 1]; ++j)
                    s0 = std::max<int64_t>(s0, start[pr[j].x] + mxr[pr[j].x] + 1 + kHandOffRounds);
                start[k] = s0;
                last = std::max(last, s0);
                finish = std::max<int64_t>(finish, s0 + (srec[ws[k]].z & 0xFFFF));
            }
            if (core->stage_order != LUE_GPU_STAGE_ORDER_EARLIEST) {
                std::vector<int64_t> late(ns);
                for (int64_t k = 0; k < ns; ++k) late[k] = finish - (srec[ws[k]].z & 0xFFFF);
                for (int64_t k = ns - 1; k >= 0; --k)
                    for (int64_t j = po[k]; j < po[k + 1]; ++j)
                        late[pr[j].x] = std::min<int64_t>(late[pr[j].x], late[k] - mxr[pr[j].x] - 1 - kHandOffRounds);
                last = 0;
                for (int64_t k = 0; k < ns; ++k) {
                    start[k] = std::max<int64_t>(0, late[k]);
                    last = std::max(last, start[k]);
                }
            }
            // counting sort by start, stable (ties keep the depth order)
            std::vector<int64_t> bucket(last + 2, 0);
            for (int64_t k = 0; k < ns; ++k) ++bucket[start[k] + 1];
            for (int64_t v = 0; v <= last; ++v) bucket[v + 1] += bucket[v];
            std::vector<int32_t> newpos(ns);
            for (int64_t k = 0; k < ns; ++k) newpos[k] = (int32_t)bucket[start[k]]++;
            std::vector<int32_t> ws2(ns), mx2(ns), cnt2(ns);
            for (int64_t k = 0; k < ns; ++k) {
                ws2[newpos[k]] = ws[k];
                mx2[newpos[k]] = mxr[k];
                cnt2[newpos[k]] = (int32_t)(po[k + 1] - po[k]);
            }
            std::vector<int64_t> po2(ns + 1, 0);
            for (int64_t j = 0; j < ns; ++j) po2[j + 1] = po2[j] + cnt2[j];
            std::vector<int2> pr2(std::max<int64_t>(1, npairs));
            for (int64_t k = 0; k < ns; ++k) {
                int64_t w = po2[newpos[k]];
                for (int64_t j = po[k]; j < po[k + 1]; ++j) pr2[w++] = make_int2(newpos[pr[j].x], pr[j].y);
            }
            TRY(cudaMemcpy(sc->wave_stage, ws2.data(), ns * sizeof(int32_t), cudaMemcpyHostToDevice), "stage order");
            TRY(cudaMemcpy(sc->max_exit_round, mx2.data(), ns * sizeof(int32_t), cudaMemcpyHostToDevice),
                "stage order");
            TRY(cudaMemcpy(sc->prod_offsets, po2.data(), (ns + 1) * sizeof(int64_t), cudaMemcpyHostToDevice),
                "stage order");
            TRY(cudaMemcpy(sc->prod, pr2.data(), npairs * sizeof(int2), cudaMemcpyHostToDevice), "stage order");
        }
    }
    sc->bytes += sc->nstages * 20 + np * 12 + sc->ninputs * 4;
    if (getenv("LUE_GB300_VERBOSE")) {
        // the critical path of a one-step call, in rounds, with a hand-off of h rounds per producer edge
        std::vector<int4> srec(sc->nstages);
        cudaMemcpy(srec.data(), sc->stage, sc->nstages * sizeof(int4), cudaMemcpyDeviceToHost);
        std::vector<int32_t> ws(sc->nstages);
        cudaMemcpy(ws.data(), sc->wave_stage, sc->nstages * sizeof(int32_t), cudaMemcpyDeviceToHost);
        std::vector<int64_t> po(sc->nstages + 1);
        cudaMemcpy(po.data(), sc->prod_offsets, po.size() * sizeof(int64_t), cudaMemcpyDeviceToHost);
        std::vector<int2> pr(std::max<int64_t>(1, po[sc->nstages]));
        cudaMemcpy(pr.data(), sc->prod, po[sc->nstages] * sizeof(int2), cudaMemcpyDeviceToHost);
        std::vector<int32_t> mx(sc->nstages);
        cudaMemcpy(mx.data(), sc->max_exit_round, sc->nstages * sizeof(int32_t), cudaMemcpyDeviceToHost);
        double sum_rounds = 0;
        for (int64_t k = 0; k < sc->nstages; ++k) sum_rounds += srec[ws[k]].z & 0xFFFF;
        fprintf(stderr, "stage rounds: mean %.1f per stage\n", sum_rounds / std::max<int64_t>(1, sc->nstages));
        for (int h : {0, 2, 5}) {
            std::vector<int64_t> start(sc->nstages, 0);
            int64_t crit = 0;
            for (int64_t k = 0; k < sc->nstages; ++k) {
                int64_t s0 = 0;
                for (int64_t j = po[k]; j < po[k + 1]; ++j)
                    s0 = std::max<int64_t>(s0, start[pr[j].x] + mx[pr[j].x] + 1 + h);
                start[k] = s0;
                crit = std::max<int64_t>(crit, s0 + (srec[ws[k]].z & 0xFFFF));
            }
            fprintf(stderr, "stage dataflow critical path (hand-off %d rounds): %lld rounds\n", h, (long long)crit);
        }
        std::vector<int> sizes;
        for (int64_t k = 0; k < sc->nstages; ++k) sizes.push_back((int)((unsigned)srec[ws[k]].y >> 16));
        std::sort(sizes.begin(), sizes.end());
        if (!sizes.empty())
            fprintf(stderr, "stage cells: p50 %d p90 %d p99 %d max %d; producers at most %lld\n",
                    sizes[sizes.size() / 2], sizes[sizes.size() * 9 / 10], sizes[sizes.size() * 99 / 100],
                    sizes.back(), (long long)sc->max_producers);
    }
    if (getenv("LUE_GB300_VERBOSE"))
        fprintf(stderr, "stage topology: %lld tiles, %lld stages, depth %lld, %lld exits, %lld inputs, "
                        "at most %lld stages per depth and %lld inputs per stage\n",
                (long long)nt, (long long)sc->nstages, (long long)sc->max_depth, (long long)sc->nexits,
                (long long)sc->ninputs, (long long)sc->max_stages_per_depth, (long long)sc->max_stage_inputs);
done:
    cudaFree(depth);
    cudaFree(counts);
    cudaFree(bases);
    cudaFree(cell_exit);
    cudaFree(input_at);
    cudaFree(exit_stage);
    cudaFree(pos_of);
    cudaFree(pcount);
    cudaFree(stage_depth);
    cudaFree(error);
    cudaFree(order);
    cudaFree(round_at);
    cudaFree(flags_at);
#undef TRY
    if (rc) {
        stage_core_free(sc);
        return rc;
    }
    *out = sc;
    return LUE_GPU_OK;
}

void stage_core_free(StageCore* sc)
{
    if (!sc) return;
    cudaFree(sc->stage);
    cudaFree(sc->wave_stage);
    cudaFree(sc->meta);
    cudaFree(sc->exit_id);
    cudaFree(sc->inputs);
    cudaFree(sc->prod_offsets);
    cudaFree(sc->prod);
    cudaFree(sc->max_exit_round);
    delete sc;
}

// ---------------------------------------------------------------------------------------------------
// Runtime: one dataflow launch
// ---------------------------------------------------------------------------------------------------
//
// One launch runs every stage with all the steps of the call.  Each CTA takes the next stage of the
// ticket order (stage_core_build) from a ticket counter, so every stage it waits for (a producer: a
// stage whose exits feed it, always earlier in that order) has been taken by a CTA that started earlier
// and waits only on stages taken before it.
// Inside a stage, cell c does step t in round round(c) + t, so T steps take rounds + T - 1 rounds; the
// active positions of round r (round in (r - T, r]) are one contiguous range of the stage's order.
// After each round a stage publishes how many steps of all its exits are in the history (progress[k]);
// before each round a stage waits until each producer has published the steps that round consumes.
// A wait gives up after `polls` polls (kFlowPolls, about a second): it sets error[0], every other wait
// then gives up at once, the outputs of the call are set to NaN and the next call on the topology
// returns LUE_GPU_ETIMEDOUT.

constexpr int kFlowPolls = 1 << 22;
constexpr int kPublishEvery = 4;  // steps per publication of a stage's progress (a release fence each)

struct StageRunArgs {
    const int4* stage;
    const int32_t* wave_stage;
    const uint2* meta;
    const int32_t* exit_id;
    const int32_t* inputs;
    int64_t rows, cols, tcols;
    int steps;
    uint2* hist;  // [nexits * steps]: the outflow of every exit at every step, as 8 bytes
};

struct StageFlowArgs {
    const int64_t* prod_offsets;
    const int2* prod;
    const int32_t* max_exit_round;
    int* progress;  // [nstages], zeroed before the launch
    int* ticket;    // zeroed before the launch
    int* error;     // [1]
    int64_t nstages;
    int polls;          // poll limit of one wait
    int publish_every;  // steps between two publications of a stage's progress
    int64_t stuck;      // test hook: the position of a stage whose first wait never ends (-1: none)
    unsigned long long* trace;  // [4 nstages] or null: start, rounds begin, time in waits, end (ns)
};

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long v;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(v));
    return v;
}

__device__ __forceinline__ int ld_acquire(const int* p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(int* p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Waits until *p >= need and returns *p; gives up (returns `need`: the caller's results are then not
// valid) after `polls` polls, setting *error, or once another wait has given up.
__device__ __forceinline__ int flow_wait(const int* p, int need, int* error, int polls)
{
    for (int it = 0; it < polls; ++it) {
        const int v = ld_acquire(p);
        if (v >= need) return v;
        if (*((volatile int*)error)) return need;
        __nanosleep(64);
    }
    atomicExch(error, 1);
    return need;
}

// Shared memory of a stage of at most kStageMaxCap cells: the stage position of each in-tile cell, the
// outflows by step parity and position, per position meta / history row / cell state / round starts, per
// input (an upstream cell in another stage) its history row, value and cell, and per producer its
// position, the earliest round that consumes it and the steps of it known to be in the history.
template <class R>
struct FlowLayout {
    uint8_t* local;
    uint2* Qs;
    uint2* meta;
    int32_t* ex;
    typename R::Cell* cells;
    uint16_t* rstart;
    uint2* in_vals;
    int32_t* in_rows;
    uint8_t* in_cell;
    int2* prod;
    int* have;
    __device__ FlowLayout(unsigned char* base, int count, int nin, int np)
    {
        local = base;
        Qs = reinterpret_cast<uint2*>(local + kStageCells);
        meta = Qs + 2 * count;
        in_vals = meta + count;
        ex = reinterpret_cast<int32_t*>(in_vals + nin);
        in_rows = ex + count;
        prod = reinterpret_cast<int2*>((reinterpret_cast<uintptr_t>(in_rows + nin) + 7) & ~uintptr_t(7));
        have = reinterpret_cast<int*>(prod + np);
        // 16-byte aligned: a Cell may hold doubles
        cells = reinterpret_cast<typename R::Cell*>((reinterpret_cast<uintptr_t>(have + np) + 15) & ~uintptr_t(15));
        // round up to 4 bytes: a Cell may be a 1-byte empty struct
        rstart = reinterpret_cast<uint16_t*>((reinterpret_cast<uintptr_t>(cells + count) + 3) & ~uintptr_t(3));
        in_cell = reinterpret_cast<uint8_t*>(rstart + count + 2);
    }
};

template <class R>
static size_t flow_smem(int64_t cells, int64_t inputs, int64_t producers)
{
    return kStageCells + cells * (3 * sizeof(uint2) + sizeof(int32_t) + sizeof(typename R::Cell)) +
           (cells + 2) * sizeof(uint16_t) + inputs * (sizeof(uint2) + sizeof(int32_t) + 1) +
           producers * (sizeof(int2) + sizeof(int)) + 32;  // + alignment
}

// Waits until every producer has published the steps that round r consumes (round r consumes step
// r - round(c) at cell c): each thread waits for its share of the producers.
template <int NT>
__device__ __forceinline__ void flow_wait_round(const StageFlowArgs& f, const int2* prod, int* have, int np, int ns,
                                                int r)
{
    for (int i = threadIdx.x; i < np; i += NT) {
        const int2 pq = prod[i];
        const int need = min(ns, r - pq.y + 1);
        if (need > have[i]) have[i] = flow_wait(f.progress + pq.x, need, f.error, f.polls);
    }
}

constexpr int kFlowPrefetch = 2;  // inputs per thread loaded one round ahead into registers

// A Rule supplies the per-cell state (Cell, kept in shared memory by position), the accumulator of the
// upstream outflows (Acc), the cell step and the final store.  ONE (a call of one step): the stage first
// waits for all its producers and loads all its inputs into shared memory at once, so that its rounds
// read shared memory only.  With many steps, round r waits for the inputs of round r + 1 and loads them
// into registers before its own cells, and puts them into shared memory after them, so that their load
// overlaps the round's arithmetic.
template <class R, int NT, bool ONE>
__global__ void __launch_bounds__(NT) k_stage_flow(StageRunArgs a, StageFlowArgs f, R rule)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_ticket;
    __shared__ unsigned long long s_wait;  // tracing: time in waits
    if (threadIdx.x == 0) s_ticket = atomicAdd(f.ticket, 1);
    __syncthreads();
    const int64_t k = s_ticket;
    if (k >= f.nstages) return;
    if (f.trace && threadIdx.x == 0) {
        f.trace[4 * k] = global_ns();
        s_wait = 0;
    }
    const int4 st = a.stage[a.wave_stage[k]];
    const int64_t tile = st.x;
    const int begin = st.y & 0xFFFF, count = (int)((unsigned)st.y >> 16);
    const int rounds = st.z & 0xFFFF, nin = (int)((unsigned)st.z >> 16);
    const int64_t in_base = st.w;
    const int ns = a.steps;
    const int64_t p0 = f.prod_offsets[k];
    const int np = (int)(f.prod_offsets[k + 1] - p0);
    FlowLayout<R> L(smem_raw, count, nin, np);
    const int64_t tr = tile / a.tcols, tc = tile - tr * a.tcols;
    const int64_t row0 = tr * kStageSide, col0 = tc * kStageSide;
    for (int i = threadIdx.x; i < nin; i += NT) L.in_rows[i] = __ldg(a.inputs + in_base + i);
    for (int i = threadIdx.x; i < np; i += NT) {
        L.prod[i] = __ldg(f.prod + p0 + i);
        L.have[i] = 0;
    }
    for (int i = threadIdx.x; i < count; i += NT) {
        const int64_t at = tile * kStageCells + begin + i;
        const uint2 m = __ldg(a.meta + at);
        L.meta[i] = m;
        L.ex[i] = __ldg(a.exit_id + at);
        const int p = (int)(m.x & 1023u);
        L.local[p] = (uint8_t)i;
        const int fi = (int)(m.y >> 16), ne = __popc((m.y >> 8) & 0xFFu);
        for (int j = 0; j < ne; ++j) L.in_cell[fi + j] = (uint8_t)i;
        rule.load(L.cells[i], (row0 + (p >> 5)) * a.cols + col0 + (p & 31));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < count; i += NT) {
        const int rd = (int)((L.meta[i].x >> 10) & 1023u);
        if (i == 0 || rd != (int)((L.meta[i - 1].x >> 10) & 1023u)) L.rstart[rd] = (uint16_t)i;
    }
    if (threadIdx.x == 0) L.rstart[rounds] = (uint16_t)count;
    const int max_exit = __ldg(f.max_exit_round + k);
    if (f.trace && threadIdx.x == 0) f.trace[4 * k + 1] = global_ns();
    // the inputs of round 0 (ONE: of every round)
    flow_wait_round<NT>(f, L.prod, L.have, np, ns, ONE ? ns + rounds : 0);
    if (k == f.stuck && threadIdx.x == 0) flow_wait(f.progress + k, ns + 1, f.error, f.polls);
    __syncthreads();
    if (f.trace && threadIdx.x == 0) s_wait += global_ns() - f.trace[4 * k + 1];
    {
        const int s_hi = ONE ? nin : (rounds > 1 ? (int)(L.meta[L.rstart[1]].y >> 16) : nin);
        for (int s = threadIdx.x; s < s_hi; s += NT) L.in_vals[s] = __ldcg(a.hist + (int64_t)L.in_rows[s] * ns);
    }
    const int nrounds = rounds + ns - 1;
    int published = 0;
    for (int r = 0; r < nrounds; ++r) {
        // the inputs of round r + 1: wait, then load into registers
        uint2 pv[kFlowPrefetch];
        int s_lo = 0, s_hi = 0;
        if (!ONE && r + 1 < nrounds) {
            if (f.trace && threadIdx.x == 0) s_wait -= global_ns();
            flow_wait_round<NT>(f, L.prod, L.have, np, ns, r + 1);
            __syncthreads();
            if (f.trace && threadIdx.x == 0) s_wait += global_ns();
            const int lo = L.rstart[max(0, r + 2 - ns)], hi = L.rstart[min(rounds, r + 2)];
            s_lo = (int)(L.meta[lo].y >> 16);
            s_hi = hi < count ? (int)(L.meta[hi].y >> 16) : nin;
#pragma unroll
            for (int j = 0; j < kFlowPrefetch; ++j) {
                const int s = s_lo + (int)threadIdx.x + j * NT;
                if (s < s_hi) {
                    const int t = r + 1 - (int)((L.meta[L.in_cell[s]].x >> 10) & 1023u);
                    pv[j] = __ldcg(a.hist + (int64_t)L.in_rows[s] * ns + t);
                }
            }
        } else if (!ONE || r == 0) {
            // one step: the barrier that ends each round orders its outflows before the next round's
            // reads, so only round 0 (after the loads of the inputs) needs one here
            __syncthreads();
        }
        const int lo = L.rstart[max(0, r - ns + 1)], hi = L.rstart[min(rounds, r + 1)];
        for (int i = lo + (int)threadIdx.x; i < hi; i += NT) {
            const uint2 m = L.meta[i];
            const int t = r - (int)((m.x >> 10) & 1023u);
            const int p = (int)(m.x & 1023u);
            const unsigned em = (m.y >> 8) & 0xFFu;
            const int fi = (int)(m.y >> 16);
            uint2* Qt = L.Qs + (t & 1) * count;
            typename R::Acc acc = rule.begin();
            unsigned um = m.y & 0xFFu;
            while (um) {
                const int q = __ffs(um) - 1;
                um &= um - 1;
                const uint2 v = ((em >> q) & 1u) ? L.in_vals[fi + __popc(em & ((1u << q) - 1u))]
                                                  : Qt[L.local[p + nb_dr(q) * kStageSide + nb_dc(q)]];
                rule.add(acc, v);
            }
            const uint2 o = rule.step(L.cells[i], acc, (row0 + (p >> 5)) * a.cols + col0 + (p & 31), t);
            Qt[i] = o;
            const int32_t e = L.ex[i];
            if (e >= 0) __stcg(a.hist + (int64_t)e * ns + t, o);
        }
        // The barrier orders every thread's history writes before thread 0's release, which makes them
        // visible at GPU scope before the progress that announces them (the pattern of a grid barrier).
        __syncthreads();
        if (threadIdx.x == 0 && max_exit >= 0) {
            // every publish_every steps (a release fence each time), and the last step
            const int prog = min(ns, max(0, r + 1 - max_exit));
            if (prog > published && (prog - published >= f.publish_every || prog == ns)) {
                st_release(f.progress + k, prog);
                published = prog;
            }
        }
        if (!ONE && r + 1 < nrounds) {
#pragma unroll
            for (int j = 0; j < kFlowPrefetch; ++j) {
                const int s = s_lo + (int)threadIdx.x + j * NT;
                if (s < s_hi) L.in_vals[s] = pv[j];
            }
            for (int s = s_lo + (int)threadIdx.x + kFlowPrefetch * NT; s < s_hi; s += NT) {
                const int t = r + 1 - (int)((L.meta[L.in_cell[s]].x >> 10) & 1023u);
                L.in_vals[s] = __ldcg(a.hist + (int64_t)L.in_rows[s] * ns + t);
            }
        }
    }
    for (int i = threadIdx.x; i < count; i += NT) {
        const int p = (int)(L.meta[i].x & 1023u);
        rule.store(L.cells[i], (row0 + (p >> 5)) * a.cols + col0 + (p & 31));
    }
    if (f.trace && threadIdx.x == 0) {
        f.trace[4 * k + 2] = s_wait;
        f.trace[4 * k + 3] = global_ns();
    }
}

// --- rules -------------------------------------------------------------------------------------------

// float32 accu / accu_threshold / accu_fraction, one step: the same cell rule and float-float upstream
// sums as the walk engine (route_walk_visitors.cuh), so the results are the same bit for bit.
template <Rule RR>
struct StageF32 {
    const float* a;
    float as;
    const float* b;
    float bs;
    float* out;
    float* rem;
    using Out = float;
    __host__ __device__ float* out_raster() const { return out; }
    __host__ __device__ float* rem_raster() const { return RR == Rule::accu ? nullptr : rem; }
    struct Cell {
        float x, b;  // inflow and threshold / fraction, loaded with the stage
    };
    struct Acc {
        FF t;
        bool nan;
    };
    __device__ void load(Cell& cl, int64_t g) const
    {
        cl.x = value_at(a, as, g);
        cl.b = RR == Rule::accu ? 0.0f : value_at(b, bs, g);
    }
    __device__ Acc begin() const { return Acc{FF{0.0f, 0.0f}, false}; }
    __device__ void add(Acc& acc, uint2 v) const
    {
        const float h = __uint_as_float(v.x);
        if (isnan(h)) acc.nan = true;
        else acc.t.add(h, __uint_as_float(v.y));
    }
    __device__ uint2 step(Cell& cl, const Acc& acc, int64_t g, int) const
    {
        float oh = 0.0f, ol = 0.0f, r = 0.0f;
        if (!rule_f32<RR>(acc.t, acc.nan, cl.x, cl.b, oh, ol, r)) {
            out[g] = qnan<float>();
            if (RR != Rule::accu) rem[g] = qnan<float>();
            return make_uint2(__float_as_uint(qnan<float>()), 0u);
        }
        out[g] = oh;
        if (RR != Rule::accu) rem[g] = r;
        return make_uint2(__float_as_uint(oh), __float_as_uint(ol));
    }
    __device__ void store(Cell&, int64_t) const {}
};

template <Rule RR>
struct StageF64 {
    const double* a;
    double as;
    const double* b;
    double bs;
    double* out;
    double* rem;
    using Out = double;
    __host__ __device__ double* out_raster() const { return out; }
    __host__ __device__ double* rem_raster() const { return RR == Rule::accu ? nullptr : rem; }
    struct Cell {
        double x, b;  // inflow and threshold / fraction, loaded with the stage
    };
    struct Acc {
        double t;
        bool nan;
    };
    __device__ void load(Cell& cl, int64_t g) const
    {
        cl.x = value_at(a, as, g);
        cl.b = RR == Rule::accu ? 0.0 : value_at(b, bs, g);
    }
    __device__ Acc begin() const { return Acc{0.0, false}; }
    __device__ void add(Acc& acc, uint2 v) const
    {
        const double h = __hiloint2double((int)v.y, (int)v.x);
        if (isnan(h)) acc.nan = true;
        else acc.t += h;
    }
    __device__ uint2 step(Cell& cl, const Acc& acc, int64_t g, int) const
    {
        double o = 0.0, r = 0.0;
        if (!rule_f64<RR>(acc.t, acc.nan, cl.x, cl.b, o, r)) {
            o = qnan<double>();
            r = qnan<double>();
        }
        out[g] = o;
        if (RR != Rule::accu) rem[g] = r;
        return make_uint2((unsigned)__double2loint(o), (unsigned)__double2hiint(o));
    }
    __device__ void store(Cell&, int64_t) const {}
};

// kinematic wave, one step, float64: the walk engine's cell rule (route_walk_visitors.cuh).
template <class TIn>
struct StageKW64 {
    RouteKW<TIn> v;  // inputs and constants (its out is the result raster)
    using Out = double;
    __host__ __device__ double* out_raster() const { return v.out; }
    __host__ __device__ double* rem_raster() const { return nullptr; }
    struct Cell {
        double qc, q, al, be, len;  // the cell's inputs, loaded with the stage
    };
    struct Acc {
        double up;
        bool nan;
    };
    __device__ void load(Cell& cl, int64_t c) const
    {
        cl.qc = v.qcur ? __ldg(v.qcur + c) : v.qcur_s;
        cl.q = v.lateral ? (double)__ldg(v.lateral + c) : v.lateral_s;
        cl.al = v.alpha ? (double)__ldg(v.alpha + c) : v.alpha_s;
        cl.be = v.beta ? __ldg(v.beta + c) : v.beta_s;
        cl.len = v.dx ? __ldg(v.dx + c) : v.dx_s;
    }
    __device__ Acc begin() const { return Acc{0.0, false}; }
    __device__ void add(Acc& acc, uint2 x) const
    {
        const double h = __hiloint2double((int)x.y, (int)x.x);
        if (isnan(h)) acc.nan = true;
        else acc.up += h;
    }
    __device__ uint2 step(Cell& cl, const Acc& acc, int64_t c, int) const
    {
        const double o = rule_kw(acc.up, acc.nan, cl.qc, cl.q, cl.al, cl.be, v.dt, cl.len, v.br);
        v.out[c] = o;
        return make_uint2((unsigned)__double2loint(o), (unsigned)__double2hiint(o));
    }
    __device__ void store(Cell&, int64_t) const {}
};

// kinematic wave, float instantiation (every raster float32): the float solve, float upstream sums in the
// walk engine's neighbour order, so results equal the walk engine's bit for bit.
struct StageKW32 {
    RouteKW32 v;  // inputs and constants (its out is the result raster)
    using Out = float;
    __host__ __device__ float* out_raster() const { return v.out; }
    __host__ __device__ float* rem_raster() const { return nullptr; }
    struct Cell {
        float qc, q, al, be, len;  // the cell's inputs, loaded with the stage
    };
    struct Acc {
        float up;
        bool nan;
    };
    __device__ void load(Cell& cl, int64_t c) const
    {
        cl.qc = v.qcur ? __ldg(v.qcur + c) : v.qcur_s;
        cl.q = v.lateral ? __ldg(v.lateral + c) : v.lateral_s;
        cl.al = v.alpha ? __ldg(v.alpha + c) : v.alpha_s;
        cl.be = v.beta ? __ldg(v.beta + c) : v.beta_s;
        cl.len = v.dx ? __ldg(v.dx + c) : v.dx_s;
    }
    __device__ Acc begin() const { return Acc{0.0f, false}; }
    __device__ void add(Acc& acc, uint2 x) const
    {
        const float h = __uint_as_float(x.x);
        if (isnan(h)) acc.nan = true;
        else acc.up += h;
    }
    __device__ uint2 step(Cell& cl, const Acc& acc, int64_t c, int) const
    {
        const float o = rule_kw32(acc.up, acc.nan, cl.qc, cl.q, cl.al, cl.be, v.dt, cl.len);
        v.out[c] = o;
        return make_uint2(__float_as_uint(o), 0u);
    }
    __device__ void store(Cell&, int64_t) const {}
};

// kinematic wave, many steps, in float-float and the variable y = Q^(1/m) (kinematic_wave_ff.cuh).
template <int P, int M>
struct StageKWPoly {
    const double* qcur;
    const float* lateral;
    float lateral_s;
    const float* alpha;
    float alpha_s;
    double* out;
    KWConstFF K;
    using Out = double;
    __host__ __device__ double* out_raster() const { return out; }
    __host__ __device__ double* rem_raster() const { return nullptr; }
    struct Cell {
        ffloat y;
        float lat, al;
    };
    struct Acc {
        ffloat up;
        bool nan;
    };
    __device__ void load(Cell& cl, int64_t g) const
    {
        cl.lat = lateral ? __ldg(lateral + g) : lateral_s;
        cl.al = alpha ? __ldg(alpha + g) : alpha_s;
        cl.y = kw_poly_root<P, M>(ff_from_double(__ldg(qcur + g)), K);
    }
    __device__ Acc begin() const { return Acc{ffloat{0.0f, 0.0f}, false}; }
    __device__ void add(Acc& acc, uint2 x) const
    {
        const ffloat v{__uint_as_float(x.x), __uint_as_float(x.y)};
        if (isnan(v.hi)) acc.nan = true;
        else acc.up = ff_add_sloppy(acc.up, v);
    }
    __device__ uint2 step(Cell& cl, const Acc& acc, int64_t, int) const
    {
        const ffloat q = kw_step_poly<P, M>(acc.up, acc.nan, cl.y, cl.lat, cl.al, K);
        return make_uint2(__float_as_uint(q.hi), __float_as_uint(q.lo));
    }
    __device__ void store(Cell& cl, int64_t g) const
    {
        out[g] = isnan(cl.y.hi) ? qnan<double>() : ff_to_double(ff_pow_n<M>(cl.y, K.br.m));
    }
};

// No-data flow direction: NaN in the outputs (cells outside every stage).
template <class T>
__global__ void k_stage_no_data(const uint8_t* fd, int64_t n, T* out, T* rem)
{
    for (int64_t c = grid_stride_begin(); c < n; c += grid_stride())
        if (fd[c] == kNoData) {
            out[c] = qnan<T>();
            if (rem) rem[c] = qnan<T>();
        }
}

// ---------------------------------------------------------------------------------------------------
// Host
// ---------------------------------------------------------------------------------------------------

static int stage_core_get(lue_gpu_topology* t, cudaStream_t stream, const StageCore** out);

int stage_prepare(lue_gpu_topology* t, cudaStream_t stream)
{
    const StageCore* sc = nullptr;
    if (int rc = stage_core_get(t, stream, &sc)) return rc;
    return cuda_status(cudaStreamSynchronize(stream), "topology_prepare");
}

// The stage topology of t, built on first use; nullptr when the engine does not apply.
static int stage_core_get(lue_gpu_topology* t, cudaStream_t stream, const StageCore** out)
{
    *out = nullptr;
    TopologyCore* core = t->core;
    if (core->stats.cycle_cells > 0) return LUE_GPU_OK;
    std::lock_guard<std::mutex> lock(core->stage_mutex);
    if (!core->stages && !core->stages_unavailable) {
        StageCore* sc = nullptr;
        const int rc = stage_core_build(core, t->work_count, stream, &sc);
        if (rc == LUE_GPU_ERANGE) {
            core->stages_unavailable = true;
            return LUE_GPU_OK;
        }
        if (rc) return rc;
        core->stages = sc;
        core->bytes += sc->bytes;
    }
    *out = core->stages;
    return LUE_GPU_OK;
}

// The stage cap the stage structures of t have (when built) or will be built with.
static int effective_cap(const TopologyCore* core)
{
    if (core->stages) return core->stages->cap;
    if (core->stage_cap > 0) return core->stage_cap;
    if (const char* e = getenv("LUE_GB300_STAGE_CAP")) return std::max(1, std::min(kStageMaxCap, atoi(e)));
    return kStageCap;
}

void stage_schedule_get(const lue_gpu_topology* t, int* cap, int* threads, int* publish_every)
{
    *cap = effective_cap(t->core);
    *threads = t->stage_threads;
    if (!*threads)
        if (const char* e = getenv("LUE_GB300_STAGE_THREADS")) *threads = atoi(e);
    *publish_every = t->publish_every;
    if (!*publish_every) {
        *publish_every = kPublishEvery;
        if (const char* e = getenv("LUE_GB300_PUBLISH_EVERY")) *publish_every = std::max(1, atoi(e));
    }
}

int stage_schedule_set(lue_gpu_topology* t, int cap, int threads, int publish_every)
{
    if (cap < 0 || cap > kStageMaxCap)
        return fail(LUE_GPU_EINVAL, "stage schedule: cap must be 0 (keep) or 1.." + std::to_string(kStageMaxCap));
    if (threads != 0 && threads != 32 && threads != 64 && threads != 128 && threads != 256)
        return fail(LUE_GPU_EINVAL, "stage schedule: threads must be 0 (by stage size), 32, 64, 128 or 256");
    if (publish_every < 0) return fail(LUE_GPU_EINVAL, "stage schedule: publish_every must be >= 0");
    TopologyCore* core = t->core;
    if (cap > 0) {
        std::lock_guard<std::mutex> lock(core->stage_mutex);
        if (cap != effective_cap(core)) {
            if (core->refs.load() > 1)
                return fail(LUE_GPU_EINVAL, "stage schedule: the stage structures are shared with " +
                                                std::to_string(core->refs.load() - 1) +
                                                " clone(s); change the cap before cloning");
            if (core->stages) {
                // the handle's streams are unknown here: wait for all work before the structures go
                if (int rc = cuda_status(cudaDeviceSynchronize(), "stage schedule")) return rc;
                core->bytes -= core->stages->bytes;
                stage_core_free(core->stages);
                core->stages = nullptr;
            }
            core->stage_cap = cap;  // rebuilt with it by the next call that needs them
        }
    }
    t->stage_threads = threads;
    t->publish_every = publish_every;
    return LUE_GPU_OK;
}

int stage_order_set(lue_gpu_topology* t, int order)
{
    if (order != LUE_GPU_STAGE_ORDER_LATEST && order != LUE_GPU_STAGE_ORDER_EARLIEST)
        return fail(LUE_GPU_EINVAL, "stage order: must be LUE_GPU_STAGE_ORDER_LATEST or _EARLIEST");
    TopologyCore* core = t->core;
    std::lock_guard<std::mutex> lock(core->stage_mutex);
    if (order == core->stage_order) return LUE_GPU_OK;
    if (core->refs.load() > 1)
        return fail(LUE_GPU_EINVAL, "stage order: the stage structures are shared with " +
                                        std::to_string(core->refs.load() - 1) + " clone(s); change the order before cloning");
    if (core->stages) {
        // the handle's streams are unknown here: wait for all work before the structures go
        if (int rc = cuda_status(cudaDeviceSynchronize(), "stage order")) return rc;
        core->bytes -= core->stages->bytes;
        stage_core_free(core->stages);
        core->stages = nullptr;
    }
    core->stage_order = order;  // rebuilt with it by the next call that needs them
    return LUE_GPU_OK;
}

// Per-handle buffers that grow with the calls come from a stream-ordered pool of the device: growing one
// waits for nothing but the handle's own stream (no device-wide synchronisation, unlike cudaFree).
static cudaMemPool_t stage_pool()
{
    static std::mutex mu;
    static cudaMemPool_t pools[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 0 || dev >= 64) return nullptr;
    if (!pools[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        if (cudaMemPoolCreate(&pools[dev], &props) != cudaSuccess) {
            pools[dev] = nullptr;
            return nullptr;
        }
        unsigned long long keep = ~0ull;
        cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep);
    }
    return pools[dev];
}

void stage_buffers_free(lue_gpu_topology* t)
{
    if (!t->stage_hist && !t->stage_flow) return;
    cudaDeviceSynchronize();  // the handle's streams are unknown here: wait for all work
    if (t->stage_hist) cudaFreeAsync(t->stage_hist, nullptr);
    if (t->stage_flow) cudaFreeAsync(t->stage_flow, nullptr);
    cudaStreamSynchronize(nullptr);
    t->stage_hist = nullptr;
    t->stage_flow = nullptr;
    t->stage_hist_bytes = t->stage_flow_bytes = 0;
    if (cudaMemPool_t pool = stage_pool()) cudaMemPoolTrimTo(pool, 0);
}

template <class T>
static int grow(lue_gpu_topology* t, T*& p, size_t& have, size_t need, cudaStream_t stream, const char* what)
{
    if (need <= have) return LUE_GPU_OK;
    (void)t;
    cudaMemPool_t pool = stage_pool();
    if (!pool) return fail(LUE_GPU_ECUDA, std::string(what) + ": no memory pool");
    if (p) {
        // after the stream's earlier uses of the buffer; the pool then gives its memory back, so that a
        // larger buffer can use it (a pool does not join a freed block to a new, larger one)
        cudaFreeAsync(p, stream);
        cudaStreamSynchronize(stream);
        cudaMemPoolTrimTo(pool, 0);
    }
    p = nullptr;
    have = 0;
    const cudaError_t e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&p), need, pool, stream);
    if (e != cudaSuccess) {
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        return fail(e == cudaErrorMemoryAllocation ? LUE_GPU_ENOMEM : LUE_GPU_ECUDA,
                    std::string(what) + ": " + cudaGetErrorString(e) + " (" + std::to_string(need >> 20) +
                        " MiB asked, " + std::to_string(free_b >> 20) + " MiB free)");
    }
    have = need;
    return LUE_GPU_OK;
}

// Marks every output NaN after a dataflow wait gave up (the results are not valid).
template <class T>
__global__ void k_invalidate_if(const int* error, T* out, T* rem, int64_t n)
{
    if (!*error) return;
    for (int64_t i = grid_stride_begin(); i < n; i += grid_stride()) {
        out[i] = qnan<T>();
        if (rem) rem[i] = qnan<T>();
    }
}

static void stage_trace_write(const StageCore* sc, unsigned long long* trace, const char* path, cudaStream_t stream)
{
    std::vector<unsigned long long> tr((size_t)sc->nstages * 4);
    std::vector<int32_t> ws(sc->nstages);
    std::vector<int4> srec(sc->nstages);
    cudaMemcpyAsync(tr.data(), trace, tr.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(ws.data(), sc->wave_stage, ws.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    cudaMemcpyAsync(srec.data(), sc->stage, srec.size() * sizeof(int4), cudaMemcpyDeviceToHost, stream);
    cudaStreamSynchronize(stream);
    cudaFree(trace);
    FILE* fp = fopen(path, "wb");
    if (!fp) return;
    for (int64_t k = 0; k < sc->nstages; ++k) {
        const int4 r = srec[ws[k]];
        const int64_t rec[8] = {(int64_t)tr[4 * k], (int64_t)tr[4 * k + 1], (int64_t)tr[4 * k + 2], (int64_t)tr[4 * k + 3],
                                r.x, (int64_t)((unsigned)r.y >> 16), r.z & 0xFFFF, (int64_t)((unsigned)r.z >> 16)};
        fwrite(rec, sizeof(rec), 1, fp);
    }
    fclose(fp);
    // the producers: per stage its offset into the (producer position, earliest round) pairs
    std::vector<int64_t> po(sc->nstages + 1);
    cudaMemcpy(po.data(), sc->prod_offsets, po.size() * sizeof(int64_t), cudaMemcpyDeviceToHost);
    std::vector<int2> pr(std::max<int64_t>(1, po[sc->nstages]));
    cudaMemcpy(pr.data(), sc->prod, po[sc->nstages] * sizeof(int2), cudaMemcpyDeviceToHost);
    fp = fopen((std::string(path) + ".prod").c_str(), "wb");
    if (!fp) return;
    fwrite(po.data(), sizeof(int64_t), po.size(), fp);
    fwrite(pr.data(), sizeof(int2), po[sc->nstages], fp);
    fclose(fp);
}

template <class R, int NT, bool ONE>
static int launch_flow(const StageRunArgs& a, const StageFlowArgs& fa, const R& rule, unsigned blocks, size_t smem,
                       cudaStream_t stream, const char* what)
{
    static size_t have = 48 * 1024;
    if (smem > have) {
        if (int rc = cuda_status(cudaFuncSetAttribute(k_stage_flow<R, NT, ONE>,
                                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                                 what))
            return rc;
        have = smem;
    }
    k_stage_flow<R, NT, ONE><<<blocks, NT, smem, stream>>>(a, fa, rule);
    return LUE_GPU_OK;
}

// Threads per stage: the handle's schedule (`threads`, 32, 64, 128 or 256), else LUE_GB300_STAGE_THREADS,
// else by the largest stage.  Every loop of k_stage_flow strides by the CTA size, so any of them is valid
// for any stage size.
template <class R, bool ONE>
static int launch_flow(const StageRunArgs& a, const StageFlowArgs& fa, const R& rule, unsigned blocks,
                       int64_t max_cells, size_t smem, int threads, cudaStream_t stream, const char* what)
{
    int nt = max_cells <= 128 ? 32 : max_cells <= 256 ? 64 : kStageThreads;
    if (threads > 0) nt = threads;
    else if (const char* e = getenv("LUE_GB300_STAGE_THREADS")) nt = atoi(e);
    switch (nt) {
        case 32: return launch_flow<R, 32, ONE>(a, fa, rule, blocks, smem, stream, what);
        case 64: return launch_flow<R, 64, ONE>(a, fa, rule, blocks, smem, stream, what);
        case 128: return launch_flow<R, 128, ONE>(a, fa, rule, blocks, smem, stream, what);
        default: return launch_flow<R, kStageThreads, ONE>(a, fa, rule, blocks, smem, stream, what);
    }
}

// `steps` steps of a rule over every stage, in one dataflow launch (k_stage_flow); one warp per CTA for
// stages of up to 128 cells.
template <class R>
static int stage_run(lue_gpu_topology* t, const StageCore* sc, const R& rule, int steps, cudaStream_t stream,
                     const char* what)
{
    const TopologyCore* core = t->core;
    if (sc->nstages == 0) return LUE_GPU_OK;
    if (t->stage_flow_error && *t->stage_flow_error) {
        *t->stage_flow_error = 0;
        return fail(LUE_GPU_ETIMEDOUT, std::string(what) +
                                           ": a wait between stages of an earlier call gave up; its outputs are NaN");
    }
    const size_t hist = (size_t)std::max<int64_t>(sc->nexits, 1) * (size_t)steps * sizeof(uint2);
    if (int rc = grow(t, t->stage_hist, t->stage_hist_bytes, hist, stream, what)) return rc;
    const size_t flow = (size_t)(sc->nstages + 2) * sizeof(int);
    if (int rc = grow(t, t->stage_flow, t->stage_flow_bytes, flow, stream, what)) return rc;
    if (!t->stage_flow_error) return fail(LUE_GPU_ECUDA, std::string(what) + ": no error word");
    int* progress = t->stage_flow;
    int* ticket = progress + sc->nstages;
    int* error = ticket + 1;
    if (int rc = cuda_status(cudaMemsetAsync(progress, 0, flow, stream), what)) return rc;
    StageRunArgs a{sc->stage, sc->wave_stage, sc->meta, sc->exit_id, sc->inputs, core->rows, core->cols, sc->tcols,
                   steps, t->stage_hist};
    StageFlowArgs fa{sc->prod_offsets, sc->prod, sc->max_exit_round, progress, ticket, error, sc->nstages,
                     kFlowPolls, kPublishEvery, -1, nullptr};
    if (t->publish_every > 0) fa.publish_every = t->publish_every;
    else if (const char* e = getenv("LUE_GB300_PUBLISH_EVERY")) fa.publish_every = std::max(1, atoi(e));
    // tracing (LUE_GB300_STAGE_TRACE=file): per stage in ticket order its start, the start of its rounds,
    // its time in waits and its end (globaltimer ns), then tile, cells, rounds and inputs, written after
    // the launch as int64 records of 8
    const char* trace_path = getenv("LUE_GB300_STAGE_TRACE");
    if (trace_path) {
        if (int rc = cuda_status(cudaMalloc(&fa.trace, (size_t)sc->nstages * 4 * sizeof(unsigned long long)), what))
            return rc;
    }
    if (const char* e = getenv("LUE_GB300_FLOW_STUCK_STAGE")) {  // test hook: see StageFlowArgs::stuck
        fa.stuck = std::max<int64_t>(0, std::min<int64_t>(atoll(e), sc->nstages - 1));
        fa.polls = 1 << 16;
    }
    const int64_t mc = sc->max_stage_cells;
    const size_t smem = flow_smem<R>(mc, sc->max_stage_inputs, sc->max_producers);
    const unsigned blocks = (unsigned)sc->nstages;
    if (getenv("LUE_GB300_VERBOSE"))
        fprintf(stderr, "%s: dataflow launch of %u stages, largest %lld cells, %zu B shared memory\n", what, blocks,
                (long long)mc, smem);
    if (int rc = steps == 1 ? launch_flow<R, true>(a, fa, rule, blocks, mc, smem, t->stage_threads, stream, what)
                            : launch_flow<R, false>(a, fa, rule, blocks, mc, smem, t->stage_threads, stream, what))
        return rc;
    const int64_t n = core->n;
    k_invalidate_if<typename R::Out><<<grid_for(n, 256), 256, 0, stream>>>(error, rule.out_raster(), rule.rem_raster(),
                                                                         n);
    if (int rc = cuda_status(
            cudaMemcpyAsync(t->stage_flow_error, error, sizeof(int), cudaMemcpyDeviceToHost, stream), what))
        return rc;
    count_launches(2);
    if (trace_path) stage_trace_write(sc, fa.trace, trace_path, stream);
    return cuda_status(cudaGetLastError(), what);
}

static bool stage_engine_off()
{
    const char* e = getenv("LUE_GB300_ENGINE");
    return e && e[0] == 'w';
}

template <Rule RR>
static int route_f32_rule(lue_gpu_topology* t, const StageCore* sc, const float* a, float as, const float* b, float bs,
                          float* out, float* rem, cudaStream_t stream)
{
    const int64_t n = t->core->n;
    k_stage_no_data<float><<<grid_for(n, 256), 256, 0, stream>>>(t->core->fd, n, out, rem);
    count_launches(1);
    StageF32<RR> rule{a, as, b, bs, out, rem};
    return stage_run(t, sc, rule, 1, stream, "stage route (float32)");
}

int stage_route_f32(lue_gpu_topology* t, int rule, const float* a, float as, const float* b, float bs, float* out,
                    float* rem, cudaStream_t stream, bool* done)
{
    *done = false;
    if (stage_engine_off()) return LUE_GPU_OK;
    const StageCore* sc = nullptr;
    if (int rc = stage_core_get(t, stream, &sc)) return rc;
    if (!sc) return LUE_GPU_OK;
    *done = true;
    switch (rule) {
        case (int)Rule::threshold: return route_f32_rule<Rule::threshold>(t, sc, a, as, b, bs, out, rem, stream);
        case (int)Rule::fraction: return route_f32_rule<Rule::fraction>(t, sc, a, as, b, bs, out, rem, stream);
        case (int)Rule::capacity: return route_f32_rule<Rule::capacity>(t, sc, a, as, b, bs, out, rem, stream);
        default: return route_f32_rule<Rule::trigger>(t, sc, a, as, b, bs, out, rem, stream);
    }
}

template <Rule RR>
static int route_f64_rule(lue_gpu_topology* t, const StageCore* sc, const double* a, double as, const double* b,
                          double bs, double* out, double* rem, cudaStream_t stream)
{
    const int64_t n = t->core->n;
    k_stage_no_data<double><<<grid_for(n, 256), 256, 0, stream>>>(t->core->fd, n, out, rem);
    count_launches(1);
    StageF64<RR> rule{a, as, b, bs, out, rem};
    return stage_run(t, sc, rule, 1, stream, "stage route (float64)");
}

int stage_route_f64(lue_gpu_topology* t, int rule, const double* a, double as, const double* b, double bs,
                    double* out, double* rem, cudaStream_t stream, bool* done)
{
    *done = false;
    if (stage_engine_off()) return LUE_GPU_OK;
    const StageCore* sc = nullptr;
    if (int rc = stage_core_get(t, stream, &sc)) return rc;
    if (!sc) return LUE_GPU_OK;
    *done = true;
    switch (rule) {
        case (int)Rule::accu: return route_f64_rule<Rule::accu>(t, sc, a, as, b, bs, out, rem, stream);
        case (int)Rule::threshold: return route_f64_rule<Rule::threshold>(t, sc, a, as, b, bs, out, rem, stream);
        case (int)Rule::fraction: return route_f64_rule<Rule::fraction>(t, sc, a, as, b, bs, out, rem, stream);
        case (int)Rule::capacity: return route_f64_rule<Rule::capacity>(t, sc, a, as, b, bs, out, rem, stream);
        default: return route_f64_rule<Rule::trigger>(t, sc, a, as, b, bs, out, rem, stream);
    }
}

int stage_kinematic_wave_f64(lue_gpu_topology* t, const double* qcur, double qcur_s, const double* lateral,
                             double lateral_s, const double* alpha, double alpha_s, const double* beta, double beta_s,
                             double dt, const double* dx, double dx_s, double* out, const BetaRational& br,
                             cudaStream_t stream, bool* done)
{
    *done = false;
    if (stage_engine_off()) return LUE_GPU_OK;
    const StageCore* sc = nullptr;
    if (int rc = stage_core_get(t, stream, &sc)) return rc;
    if (!sc) return LUE_GPU_OK;
    *done = true;
    const int64_t n = t->core->n;
    k_stage_no_data<double><<<grid_for(n, 256), 256, 0, stream>>>(t->core->fd, n, out, (double*)nullptr);
    count_launches(1);
    StageKW64<double> rule{RouteKW<double>{t->core->upmask, qcur, qcur_s, lateral, lateral_s, alpha, alpha_s, beta,
                                           beta_s, dt, dx, dx_s, out, t->core->cols, br}};
    return stage_run(t, sc, rule, 1, stream, "kinematic_wave_f64 (stages)");
}

int stage_kinematic_wave_f32(lue_gpu_topology* t, const float* qcur, float qcur_s, const float* lateral,
                             float lateral_s, const float* alpha, float alpha_s, const float* beta, float beta_s,
                             float dt, const float* dx, float dx_s, float* out, cudaStream_t stream, bool* done)
{
    *done = false;
    if (stage_engine_off()) return LUE_GPU_OK;
    const StageCore* sc = nullptr;
    if (int rc = stage_core_get(t, stream, &sc)) return rc;
    if (!sc) return LUE_GPU_OK;
    *done = true;
    const int64_t n = t->core->n;
    k_stage_no_data<float><<<grid_for(n, 256), 256, 0, stream>>>(t->core->fd, n, out, (float*)nullptr);
    count_launches(1);
    StageKW32 rule{RouteKW32{t->core->upmask, qcur, qcur_s, lateral, lateral_s, alpha, alpha_s, beta, beta_s, dt, dx,
                             dx_s, out, t->core->cols}};
    return stage_run(t, sc, rule, 1, stream, "kinematic_wave_f32 (stages)");
}

static ffloat ff_split(double v);
static KWConstFF kw_constants(double beta, double dt, double dx, const BetaRational& br);

// One step with float32 lateral inflow and alpha: the float-float solve in y = Q^(1/m) when beta is a
// small rational p/m (the result agrees with the float64 solve to ~1e-13), else the float64 solve.
int stage_kinematic_wave_f32in(lue_gpu_topology* t, const double* qcur, double qcur_s, const float* lateral,
                               double lateral_s, const float* alpha, double alpha_s, double beta, double dt, double dx,
                               double* out, const BetaRational& br, cudaStream_t stream, bool* done)
{
    *done = false;
    if (stage_engine_off()) return LUE_GPU_OK;
    const StageCore* sc = nullptr;
    if (int rc = stage_core_get(t, stream, &sc)) return rc;
    if (!sc) return LUE_GPU_OK;
    *done = true;
    const int64_t n = t->core->n;
    k_stage_no_data<double><<<grid_for(n, 256), 256, 0, stream>>>(t->core->fd, n, out, (double*)nullptr);
    count_launches(1);
    if (qcur && br.m >= 1 && br.m <= 16 && br.p >= 1 && br.p <= 16) {
        const KWConstFF K = kw_constants(beta, dt, dx, br);
        if (br.p == 3 && br.m == 5) {
            StageKWPoly<3, 5> rule{qcur, lateral, (float)lateral_s, alpha, (float)alpha_s, out, K};
            return stage_run(t, sc, rule, 1, stream, "kinematic_wave_f64_f32in (stages)");
        }
        StageKWPoly<0, 0> rule{qcur, lateral, (float)lateral_s, alpha, (float)alpha_s, out, K};
        return stage_run(t, sc, rule, 1, stream, "kinematic_wave_f64_f32in (stages)");
    }
    StageKW64<float> rule{RouteKW<float>{t->core->upmask, qcur, qcur_s, lateral, lateral_s, alpha, alpha_s, nullptr,
                                         beta, dt, nullptr, dx, out, t->core->cols, br}};
    return stage_run(t, sc, rule, 1, stream, "kinematic_wave_f64_f32in (stages)");
}

static ffloat ff_split(double v)
{
    const float h = (float)v;
    return ffloat{h, (float)(v - (double)h)};
}

static KWConstFF kw_constants(double beta, double dt, double dx, const BetaRational& br)
{
    KWConstFF K;
    K.k = ff_split(dt / dx);
    K.dt = ff_split(dt);
    K.kf = (float)(dt / dx);
    K.beta_f = (float)beta;
    K.beta = beta;
    K.dt_d = dt;
    K.dx_d = dx;
    K.br = br;
    K.bad = std::isnan(beta) || std::isnan(dt) || std::isnan(dx) || !(dx > 0.0);
    return K;
}

int stage_kinematic_wave_steps(lue_gpu_topology* t, const double* qcur, const float* lateral, double lateral_s,
                               const float* alpha, double alpha_s, double beta, double dt, double dx, int steps,
                               double* out, const BetaRational& br, cudaStream_t stream, bool* done)
{
    *done = false;
    if (stage_engine_off() || br.m == 0 || br.m > 16 || br.p > 16) return LUE_GPU_OK;
    const StageCore* sc = nullptr;
    if (int rc = stage_core_get(t, stream, &sc)) return rc;
    if (!sc) return LUE_GPU_OK;
    *done = true;
    const int64_t n = t->core->n;
    // the history of every exit for every step of a part of the call: parts of at most `fit` steps
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    const double budget = 0.4 * (double)free_b + (double)t->stage_hist_bytes;
    const int64_t per_step = std::max<int64_t>(sc->nexits, 1) * (int64_t)sizeof(uint2);
    const int fit = (int)std::max<int64_t>(1, std::min<int64_t>(steps, (int64_t)(budget / (double)per_step)));
    const KWConstFF K = kw_constants(beta, dt, dx, br);
    double* tmp = nullptr;
    if (steps > fit) {
        if (int rc = cuda_status(cudaMalloc(&tmp, 2 * (size_t)n * sizeof(double)), "kinematic_wave_steps")) return rc;
    }
    const double* src = qcur;
    int done_steps = 0, which = 0;
    int rc = LUE_GPU_OK;
    while (done_steps < steps) {
        const int part = std::min(fit, steps - done_steps);
        double* dst = done_steps + part == steps ? out : tmp + (size_t)which * n;
        k_stage_no_data<double><<<grid_for(n, 256), 256, 0, stream>>>(t->core->fd, n, dst, (double*)nullptr);
        count_launches(1);
        if (br.p == 3 && br.m == 5) {
            StageKWPoly<3, 5> rule{src, lateral, (float)lateral_s, alpha, (float)alpha_s, dst, K};
            rc = stage_run(t, sc, rule, part, stream, "kinematic_wave_steps (stages)");
        } else {
            StageKWPoly<0, 0> rule{src, lateral, (float)lateral_s, alpha, (float)alpha_s, dst, K};
            rc = stage_run(t, sc, rule, part, stream, "kinematic_wave_steps (stages)");
        }
        if (rc) break;
        src = dst;
        which ^= 1;
        done_steps += part;
    }
    if (tmp) {
        cudaStreamSynchronize(stream);
        cudaFree(tmp);
    }
    return rc;
}

}  // namespace lue_gb300
