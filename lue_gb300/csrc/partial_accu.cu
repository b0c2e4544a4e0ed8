// partial_accu.cu — the reference's partial_accu: which stream of the partitioned walk reached a cell.
//
// Reference: ALG/definition/partial_accu.hpp:15-287 (the PartialAccu cell accumulator's hooks), value
// policies ALG/value_policies/partial_accu.hpp, on the router's events ALG/definition/
// accumulating_router.hpp:525-599 (walk), :866-882 (intra-partition ridge scan), :984-1010
// (inter-partition arrivals).  Followed through, the hooks give a rule per cell, upstream first:
//   - a cell without upstream cells (a ridge) is the partition's k-th ridge in row-major order: value k
//     (the partition's stream counter, :71-83), whatever nr_steps;
//   - the other cells take the values of their upstream cells as those arrive.  A walk inside the
//     partition copies its value into the next cell (leave_cell, :129-165); a value from another
//     partition is combined by maximum (enter_inter_partition_stream, :86-109).  Walks from ridges come
//     first, in ridge order, so among them the largest value arrives last; walks that start at partition
//     input cells (cells with an upstream cell in another partition) come after all of them;
//   - NaN arriving, or a value above nr_steps, makes a cell NaN for good;
//   - after the walk from a partition input cell, that cell's value goes up by one (:112-120); the
//     cells downstream got the value before that.
// So, per cell c with upstream cells U (in-partition ones finished in the ridge phase: phase 1; the others,
// and partition input cells: phase 2):
//   no in-partition phase-2 upstream cell, not a partition input .... max over U           (phase 1)
//   one in-partition phase-2 upstream cell, not a partition input ... that cell's value     (phase 2)
//   partition input, no in-partition phase-2 upstream cell .......... max over U, then +1 on c itself
// Two cases depend on the order in which HPX delivers the inter-partition messages: several in-partition
// phase-2 upstream cells with different values (the last arrival wins), and a partition input cell with
// an in-partition phase-2 upstream cell (a copy or a maximum comes last, and only a walk that starts at
// the input cell adds one).  Those cells, and every cell downstream of them, are flagged
// order-dependent; their value here takes the maximum (and no +1).  Cells on or below a flow cycle, which
// the reference never enters, keep what their entered upstream cells pushed (0 if none; the maximum,
// flagged order-dependent, if several did).  The result does not depend on the topology's partition of
// the work: the partitions here are the reference's, from the partition shape the topology was made with.
#include "route_walk_visitors.cuh"
#include "topology.cuh"
#include "walk.cuh"

namespace lue_gb300 {

enum : uint8_t { kPhase2 = 1, kOrderDependent = 2, kPlusOne = 4 };

// Per (row, partition column) segment: the rank of every ridge cell (no upstream cell, valid flow
// direction) among the segment's ridge cells, into out[], and the segment's ridge count.  One warp per
// segment, 32 cells per step.
template <class T>
__global__ void k_ridge_rank(const uint8_t* __restrict__ fd, const uint8_t* __restrict__ upmask, PartitionGeom g,
                             T* out, int32_t* seg_count)
{
    const int64_t nseg = g.rows * g.npcol;
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x / 32);
    for (int64_t s = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32; s < nseg; s += warps) {
        const int64_t r = s / g.npcol, pc = s - r * g.npcol;
        const int64_t c0 = pc * g.pcol, c1 = pc == g.npcol - 1 ? g.cols : c0 + g.pcol;
        int32_t run = 0;
        for (int64_t c = c0; c < c1; c += 32) {
            const int64_t i = r * g.cols + c + lane;
            const bool ridge = c + lane < c1 && __ldg(fd + i) != kNoData && __ldg(upmask + i) == 0;
            const unsigned b = __ballot_sync(0xffffffffu, ridge);
            if (ridge) out[i] = (T)(run + __popc(b & ((1u << lane) - 1u)));
            run += __popc(b);
        }
        if (lane == 0) seg_count[s] = run;
    }
}

// Per partition, the ridge count of the partition's rows before each row (exclusive scan down the rows).
__global__ void k_ridge_offsets(PartitionGeom g, int32_t* seg)
{
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= g.nprow * g.npcol) return;
    const int64_t pr = p / g.npcol, pc = p - pr * g.npcol;
    const int64_t r0 = pr * g.prow, r1 = pr == g.nprow - 1 ? g.rows : r0 + g.prow;
    int32_t acc = 0;
    for (int64_t r = r0; r < r1; ++r) {
        const int32_t c = seg[r * g.npcol + pc];
        seg[r * g.npcol + pc] = acc;
        acc += c;
    }
}

template <class T>
struct PartialVisitor {
    const uint8_t* upmask;
    T* out;
    uint8_t* flags;
    const int32_t* seg_off;
    PartitionGeom g;
    T nr_steps;

    __device__ void enter(int64_t c)
    {
        const int64_t r = c / g.cols, col = c - r * g.cols;
        const int64_t pr = g.prow_of(r), pc = g.pcol_of(col);
        const unsigned m0 = __ldg(upmask + c);
        if (!m0) {  // a ridge: its rank in the partition
            out[c] = out[c] + (T)__ldg(seg_off + r * g.npcol + pc);
            flags[c] = 0;
            return;
        }
        bool input = false, nan = false, od = false, differ = false;
        int n2 = 0;
        T vmax = T(0), v2 = T(0);
        for (unsigned m = m0; m; m &= m - 1) {
            const int k = __ffs(m) - 1;
            const int64_t ur = r + nb_dr(k), uc = col + nb_dc(k), u = ur * g.cols + uc;
            const T v = load_cg(out + u);
            const unsigned f = load_cg(flags + u);
            if (isnan(v) || v > nr_steps) nan = true;
            if (f & kOrderDependent) od = true;
            if (g.prow_of(ur) != pr || g.pcol_of(uc) != pc) {
                input = true;
            } else if (f & kPhase2) {
                if (n2 > 0 && v != v2) differ = true;
                v2 = v;
                ++n2;
            }
            if (v > vmax) vmax = v;
        }
        T value;
        uint8_t fl;
        if (!input) {
            fl = n2 > 0 ? kPhase2 : 0;
            value = n2 == 0 || differ ? vmax : v2;
            if (differ) od = true;
        } else {
            fl = kPhase2;
            value = vmax;
            if (n2 > 0) od = true;
            else fl |= kPlusOne;
        }
        out[c] = nan ? qnan<T>() : value;
        flags[c] = fl | (od ? kOrderDependent : 0);
    }
    __device__ void no_data(int64_t c)
    {
        out[c] = qnan<T>();
        flags[c] = 0;
    }
};

// Cells on or below a flow cycle (never entered): what their entered upstream cells pushed (0 if none;
// NaN if one pushed NaN or a value above nr_steps; the maximum, order-dependent, if several pushed).
// Runs before the +1 of partition input cells: what a walk pushed is the value before that +1.
template <class T>
__global__ void k_partial_unentered(const uint8_t* __restrict__ fd, const uint8_t* __restrict__ upmask,
                                    const uint32_t* __restrict__ work, PartitionGeom g, T nr_steps, T* out,
                                    uint8_t* flags)
{
    const int64_t n = g.rows * g.cols;
    for (int64_t c = grid_stride_begin(); c < n; c += grid_stride()) {
        if (fd[c] == kNoData || ((work[c >> 2] >> ((c & 3) * 8)) & 0xFFu) == 0u) continue;  // entered
        T v = T(0);
        bool nan = false, od = false;
        int pushed = 0;
        const int64_t r = c / g.cols, col = c - r * g.cols;
        for (unsigned m = upmask[c]; m; m &= m - 1) {
            const int k = __ffs(m) - 1;
            const int64_t u = (r + nb_dr(k)) * g.cols + col + nb_dc(k);
            if (((work[u >> 2] >> ((u & 3) * 8)) & 0xFFu) != 0u) continue;  // not entered: pushed nothing
            const T h = out[u];
            if (isnan(h) || h > nr_steps) nan = true;
            else if (h > v) v = h;
            if (flags[u] & kOrderDependent) od = true;
            ++pushed;
        }
        out[c] = nan ? qnan<T>() : v;
        flags[c] = (pushed > 1 || od) ? kOrderDependent : 0;
    }
}

// The +1 of the partition input cells whose walk ran, and the order-dependence flags out.
template <class T>
__global__ void k_partial_plus_one(const uint8_t* __restrict__ fd, int64_t n, const uint8_t* __restrict__ flags,
                                   T* out, uint8_t* order_dependent)
{
    for (int64_t c = grid_stride_begin(); c < n; c += grid_stride()) {
        const bool valid = fd[c] != kNoData;
        const uint8_t f = valid ? flags[c] : 0;
        if ((f & kPlusOne) && !(f & kOrderDependent) && !isnan(out[c])) out[c] += T(1);
        if (order_dependent) order_dependent[c] = (f & kOrderDependent) ? 1 : 0;
    }
}

template <class T>
static int partial_accu(lue_gpu_topology* t, int64_t nr_steps, T* out, uint8_t* order_dependent, void* stream_,
                        const char* what)
{
    if (!t || !t->core || !out) return fail(LUE_GPU_EINVAL, std::string(what) + ": NULL argument");
    cudaStream_t stream = (cudaStream_t)stream_;
    const TopologyCore* core = t->core;
    const int64_t n = core->n;
    const PartitionGeom g = partition_geom(core);
    const int64_t nseg = g.rows * g.npcol;
    int32_t* seg = nullptr;
    if (int rc = cuda_status(cudaMallocAsync(&seg, nseg * sizeof(int32_t), stream), what)) return rc;
    // the handle's per-call float residuals (4 bytes per cell) hold the per-cell flags
    uint8_t* flags = reinterpret_cast<uint8_t*>(t->lo);
    int rc = cuda_status(cudaMemcpyAsync(t->work_count, core->count, words_for(n) * 4, cudaMemcpyDeviceToDevice,
                                         stream),
                         what);
    if (!rc) {
        const T steps = (T)(nr_steps > 0 ? nr_steps : 0);
        k_ridge_rank<T><<<grid_for(nseg * 32, 256), 256, 0, stream>>>(core->fd, core->upmask, g, out, seg);
        k_ridge_offsets<<<(unsigned)((g.nprow * g.npcol + 255) / 256), 256, 0, stream>>>(g, seg);
        WalkGrid wg{core->fd, core->count, t->work_count, core->rows, core->cols, n};
        PartialVisitor<T> v{core->upmask, out, flags, seg, g, steps};
        k_walk<<<grid_all(n, 256), 256, 0, stream>>>(wg, v);
        if (core->stats.cycle_cells > 0)
            k_partial_unentered<T><<<grid_for(n, 256), 256, 0, stream>>>(core->fd, core->upmask, t->work_count, g,
                                                                         steps, out, flags);
        k_partial_plus_one<T><<<grid_for(n, 256), 256, 0, stream>>>(core->fd, n, flags, out, order_dependent);
        count_launches(core->stats.cycle_cells > 0 ? 5 : 4);
        rc = cuda_status(cudaGetLastError(), what);
    }
    const int rc2 = cuda_status(cudaFreeAsync(seg, stream), what);
    return rc ? rc : rc2;
}

}  // namespace lue_gb300

using namespace lue_gb300;

extern "C" int lue_gpu_partial_accu_f32(lue_gpu_topology* t, int64_t nr_steps, float* out, uint8_t* order_dependent,
                                        void* stream)
{
    return partial_accu<float>(t, nr_steps, out, order_dependent, stream, "partial_accu_f32");
}

extern "C" int lue_gpu_partial_accu_f64(lue_gpu_topology* t, int64_t nr_steps, double* out,
                                        uint8_t* order_dependent, void* stream)
{
    return partial_accu<double>(t, nr_steps, out, order_dependent, stream, "partial_accu_f64");
}
