// accu_info.cu — the class of every cell in the reference's partitioned flow accumulation.
//
// Reference: ALG/definition/accu_info.hpp:13-190 (the AccuInfo cell accumulator's hooks on the router's
// events), classes ALG/accu_info.hpp:22-63, events ALG/definition/accumulating_router.hpp:525-599 (walk),
// :866-882 (intra-partition ridge scan), :984-1010 (inter-partition arrivals).  The reference walks every
// partition from its ridge cells, then continues from partition input cells as material arrives from
// neighbouring partitions; each cell keeps the class the last event that touched it gave it.  Followed
// through, that is a rule per cell:
//   no-data flow direction ................................................ 255
//   no upstream cell ...................................................... ridge (11)
//   an upstream cell in another partition (partition input) ............... partition input (14), or
//                                                                          partition input-output (15) if
//                                                                          the flow leaves the partition
//   else a sink (code 5 or any code that is not a direction) .............. sink (17)
//   else the flow leaves the partition (to another one or off the array) .. partition output (13)
//   else downstream of a partition input cell of the same partition ....... inter-partition stream (16)
//   else .................................................................. intra-partition stream (12)
// One case depends on the order in which the reference's channels deliver: a partition input cell whose
// upstream cells in its own partition also wait for other partitions is classed by the last arrival (a
// message: input / input-output; a walk from inside the partition: its stream or terminal class).  Here it
// is classed as if a message came last.  Cells on or below a flow cycle, which the reference never
// finishes, are classed as if their upstream cells were finished.
#include "topology.cuh"
#include "walk.cuh"

namespace lue_gb300 {

enum : uint8_t {
    kRidge = 11,
    kIntraStream = 12,
    kPartitionOutput = 13,
    kPartitionInput = 14,
    kPartitionInputOutput = 15,
    kInterStream = 16,
    kSink = 17
};

// dep[c] = 1 when a partition input cell of c's partition lies upstream of c within the partition (c
// itself included): c is finished only after material arrives from another partition.
struct DependVisitor {
    const uint8_t* upmask;
    uint8_t* dep;
    PartitionGeom g;
    __device__ void enter(int64_t c)
    {
        const int64_t r = c / g.cols, col = c - r * g.cols;
        const int64_t pr = g.prow_of(r), pc = g.pcol_of(col);
        uint8_t d = 0;
        for (unsigned m = __ldg(upmask + c); m; m &= m - 1) {
            const int k = __ffs(m) - 1;
            const int64_t ur = r + nb_dr(k), uc = col + nb_dc(k);
            if (g.prow_of(ur) != pr || g.pcol_of(uc) != pc) d = 1;  // a partition input cell
            else if (load_cg(dep + ur * g.cols + uc)) d = 1;
        }
        dep[c] = d;
    }
    __device__ void no_data(int64_t) {}
};

__global__ void k_accu_info(const uint8_t* __restrict__ fd, const uint8_t* __restrict__ upmask,
                            const uint8_t* __restrict__ dep, PartitionGeom g, uint8_t* out)
{
    const int64_t n = g.rows * g.cols;
    for (int64_t c = grid_stride_begin(); c < n; c += grid_stride()) {
        const uint8_t code = __ldg(fd + c);
        if (code == kNoData) {
            out[c] = kNoData;
            continue;
        }
        const unsigned m = __ldg(upmask + c);
        if (!m) {
            out[c] = kRidge;
            continue;
        }
        const int64_t r = c / g.cols, col = c - r * g.cols;
        const int64_t pr = g.prow_of(r), pc = g.pcol_of(col);
        bool input = false;
        for (unsigned mm = m; mm; mm &= mm - 1) {
            const int k = __ffs(mm) - 1;
            if (g.prow_of(r + nb_dr(k)) != pr || g.pcol_of(col + nb_dc(k)) != pc) input = true;
        }
        int dr = 0, dc = 0;
        const bool moves = d8_offset(code, dr, dc);
        bool leaves = false;
        if (moves) {
            const int64_t rr = r + dr, cc = col + dc;
            leaves = rr < 0 || rr >= g.rows || cc < 0 || cc >= g.cols || g.prow_of(rr) != pr || g.pcol_of(cc) != pc;
        }
        uint8_t v;
        if (input) v = leaves ? kPartitionInputOutput : kPartitionInput;
        else if (!moves) v = kSink;
        else if (leaves) v = kPartitionOutput;
        else v = __ldg(dep + c) ? kInterStream : kIntraStream;
        out[c] = v;
    }
}

}  // namespace lue_gb300

using namespace lue_gb300;

extern "C" int lue_gpu_accu_info_u8(lue_gpu_topology* t, uint8_t* cell_class, void* stream_)
{
    if (!t || !cell_class) return fail(LUE_GPU_EINVAL, "accu_info: NULL argument");
    cudaStream_t stream = (cudaStream_t)stream_;
    const TopologyCore* core = t->core;
    const int64_t n = core->n;
    const PartitionGeom g{core->rows, core->cols, core->prow, core->pcol, core->rows / core->prow,
                          core->cols / core->pcol};
    // the per-call float residuals of the handle (4 bytes per cell) hold the dependency flags
    uint8_t* dep = reinterpret_cast<uint8_t*>(t->lo);
    if (int rc = cuda_status(cudaMemsetAsync(dep, 0, n, stream), "accu_info")) return rc;
    if (int rc = cuda_status(cudaMemcpyAsync(t->work_count, core->count, words_for(n) * 4, cudaMemcpyDeviceToDevice,
                                             stream),
                             "accu_info"))
        return rc;
    WalkGrid wg{core->fd, core->count, t->work_count, core->rows, core->cols, n};
    DependVisitor v{core->upmask, dep, g};
    k_walk<<<grid_all(n, 256), 256, 0, stream>>>(wg, v);
    k_accu_info<<<grid_for(n, 256), 256, 0, stream>>>(core->fd, core->upmask, dep, g, cell_class);
    count_launches(2);
    return cuda_status(cudaGetLastError(), "accu_info");
}
