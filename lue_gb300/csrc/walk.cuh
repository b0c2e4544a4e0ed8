// walk.cuh — the downstream-walk engine: the reference's ridge walk, run by every thread at once.
//
// Reference: ALG/definition/accumulating_router.hpp:525-599 (accumulate) and :866-882 (the scan that
// starts a walk at every cell without inflow).  In the reference one thread per partition walks; here
// every cell without inflow starts a walk.  A walk finishes a cell, then decrements the inflow counter
// of its downstream cell; the walker that brings a counter to zero continues downstream, all others
// stop ("stop_at_confluence_cell").  So every cell is finished exactly once, after all its upstream
// cells, and no thread ever waits for another.
//
// Visibility: a finished cell's values are stored, then __threadfence(), then the counter decrement.
// The walker that takes the counter to zero issues __threadfence() before it reads the upstream values
// with L1-bypassing loads (ld.global.cg), so it sees every upstream store.
//
// A Visitor provides:
//   __device__ void enter(int64_t cell)   pull the upstream values, apply the cell rule, store
//   __device__ void no_data(int64_t cell) the flow direction is no-data: mark the outputs
#pragma once

#include "common.cuh"

namespace lue_gb300 {

struct WalkGrid {
    const uint8_t* fd;
    const uint8_t* count;
    uint32_t* work;  // counters, 4 cells per 32-bit word
    int64_t rows, cols, n;
};

template <class Visitor>
__device__ __forceinline__ void walk_from(const WalkGrid& g, Visitor& v, int64_t c)
{
    for (;;) {
        v.enter(c);
        int64_t r = c / g.cols, col = c - r * g.cols, d;
        if (!downstream(__ldg(g.fd + c), r, col, g.rows, g.cols, d)) return;
        __threadfence();
        unsigned shift = (unsigned)(d & 3) * 8u;
        unsigned old = atomicSub(g.work + (d >> 2), 1u << shift);
        if (((old >> shift) & 0xFFu) != 1u) return;
        __threadfence();
        c = d;
    }
}

template <class Visitor>
__global__ void __launch_bounds__(256) k_walk(WalkGrid g, Visitor v)
{
    for (int64_t c = grid_stride_begin(); c < g.n; c += grid_stride()) {
        uint8_t code = __ldg(g.fd + c);
        if (code == kNoData) {
            v.no_data(c);
        } else if (__ldg(g.count + c) == 0) {
            walk_from(g, v, c);
        }
    }
}

// The same walk, run only when flag[1] is set (a fallback behind an engine that found inputs it does
// not handle); grid-stride, so it needs no launch of one thread per cell.
template <class Visitor>
__global__ void __launch_bounds__(256) k_walk_if(WalkGrid g, Visitor v, const unsigned long long* flag)
{
    if (flag[1] == 0) return;
    for (int64_t c = grid_stride_begin(); c < g.n; c += grid_stride()) {
        uint8_t code = __ldg(g.fd + c);
        if (code == kNoData) {
            v.no_data(c);
        } else if (__ldg(g.count + c) == 0) {
            walk_from(g, v, c);
        }
    }
}

__global__ void k_copy_words_if(const uint32_t* src, uint32_t* dst, int64_t nwords, const unsigned long long* flag);

}  // namespace lue_gb300
