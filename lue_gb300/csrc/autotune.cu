// autotune.cu — the stage schedule of a handle and its autotuner.
//
// The stage engine (stage_route.cu) has three schedule parameters that change the time of a call but not
// its results: the most cells of one stage (the cap, a property of the stage structures), the threads of a
// stage's CTA, and how many time steps a stage computes between two publications of its progress.  The
// best values depend on the raster (how deep its stages are, how long its dependency chains are) and on
// the operation (one step or many).  The tuner times the caller's own call for candidate schedules and
// keeps the fastest.  The reference has nothing of the kind: its schedule is HPX's task order over
// partitions (ALG/definition/accumulating_router.hpp:1374-1419).
#include <algorithm>
#include <string>
#include <vector>

#include "topology.cuh"

namespace lue_gb300 {
namespace {

struct Schedule {
    int cap, threads, publish_every;
};

struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    ~EventPair()
    {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

// Mean time of `repeats` calls on `stream`, in ms.
int time_call(lue_gpu_topology* t, lue_gpu_stage_call call, void* user, int repeats, cudaStream_t stream,
              EventPair& ev, float* ms)
{
    if (int rc = cuda_status(cudaEventRecord(ev.a, stream), "autotune")) return rc;
    for (int r = 0; r < repeats; ++r)
        if (int rc = call(t, user, stream)) return rc;
    if (int rc = cuda_status(cudaEventRecord(ev.b, stream), "autotune")) return rc;
    if (int rc = cuda_status(cudaEventSynchronize(ev.b), "autotune")) return rc;
    float total = 0.0f;
    if (int rc = cuda_status(cudaEventElapsedTime(&total, ev.a, ev.b), "autotune")) return rc;
    *ms = total / (float)repeats;
    return LUE_GPU_OK;
}

}  // namespace
}  // namespace lue_gb300

using namespace lue_gb300;

extern "C" int lue_gpu_topology_get_stage_schedule(const lue_gpu_topology* topology, lue_gpu_stage_schedule* schedule)
{
    if (!topology || !schedule) return fail(LUE_GPU_EINVAL, "get_stage_schedule: NULL argument");
    int cap = 0, threads = 0, publish = 0;
    stage_schedule_get(topology, &cap, &threads, &publish);
    schedule->cap = cap;
    schedule->threads = threads;
    schedule->publish_every = publish;
    schedule->ms = 0.0f;
    return LUE_GPU_OK;
}

extern "C" int lue_gpu_topology_set_stage_schedule(lue_gpu_topology* topology, const lue_gpu_stage_schedule* schedule)
{
    if (!topology || !schedule) return fail(LUE_GPU_EINVAL, "set_stage_schedule: NULL argument");
    return stage_schedule_set(topology, schedule->cap, schedule->threads, schedule->publish_every);
}

extern "C" int lue_gpu_topology_set_stage_order(lue_gpu_topology* topology, int order)
{
    if (!topology) return fail(LUE_GPU_EINVAL, "set_stage_order: NULL argument");
    return stage_order_set(topology, order);
}

extern "C" int lue_gpu_topology_get_stage_order(const lue_gpu_topology* topology, int* order)
{
    if (!topology || !order) return fail(LUE_GPU_EINVAL, "get_stage_order: NULL argument");
    *order = topology->core->stage_order;
    return LUE_GPU_OK;
}

extern "C" int lue_gpu_autotune_stage_schedule(lue_gpu_topology* topology, lue_gpu_stage_call call, void* user,
                                               int repeats, void* stream_, lue_gpu_stage_schedule* best)
{
    if (!topology || !call || !best) return fail(LUE_GPU_EINVAL, "autotune_stage_schedule: NULL argument");
    if (repeats < 1) return fail(LUE_GPU_EINVAL, "autotune_stage_schedule: repeats must be >= 1");
    cudaStream_t stream = (cudaStream_t)stream_;
    Schedule before{};
    stage_schedule_get(topology, &before.cap, &before.threads, &before.publish_every);
    const bool shared = topology->core->refs.load() > 1;
    EventPair ev;
    if (int rc = cuda_status(cudaEventCreate(&ev.a), "autotune")) return rc;
    if (int rc = cuda_status(cudaEventCreate(&ev.b), "autotune")) return rc;

    Schedule won = before;
    float won_ms = -1.0f;
    // sets s, runs the call once untimed (it builds stage structures of a new cap and loads a kernel of a
    // new CTA size), then times it
    auto trial = [&](const Schedule& s) -> int {
        if (int rc = stage_schedule_set(topology, s.cap, s.threads, s.publish_every)) return rc;
        if (int rc = call(topology, user, stream)) return rc;
        float ms = 0.0f;
        if (int rc = time_call(topology, call, user, repeats, stream, ev, &ms)) return rc;
        if (won_ms < 0.0f || ms < won_ms) {
            won_ms = ms;
            won = s;
        }
        return LUE_GPU_OK;
    };
    auto restore = [&](int rc) {
        const std::string msg = lue_gpu_last_error();
        stage_schedule_set(topology, shared ? 0 : before.cap, before.threads, before.publish_every);
        fail(rc, "autotune_stage_schedule: " + msg);
        return rc;
    };

    // 1. stage cap (a cap of the current value costs no rebuild; shared structures keep theirs)
    std::vector<int> caps = shared ? std::vector<int>{before.cap} : std::vector<int>{64, 128, 256};
    if (!shared && std::find(caps.begin(), caps.end(), before.cap) == caps.end()) caps.push_back(before.cap);
    for (int cap : caps)
        if (int rc = trial(Schedule{cap, 0, before.publish_every})) return restore(rc);
    // 2. publication interval, with the best cap
    const Schedule after_cap = won;
    for (int p : {1, 2, 4, 8})
        if (p != after_cap.publish_every)
            if (int rc = trial(Schedule{after_cap.cap, after_cap.threads, p})) return restore(rc);
    // 3. threads per stage, with the best of those
    const Schedule after_publish = won;
    for (int nt : {32, 64, 128})
        if (int rc = trial(Schedule{after_publish.cap, nt, after_publish.publish_every})) return restore(rc);
    if (int rc = stage_schedule_set(topology, won.cap, won.threads, won.publish_every)) return restore(rc);
    best->cap = won.cap;
    best->threads = won.threads;
    best->publish_every = won.publish_every;
    best->ms = won_ms;
    return LUE_GPU_OK;
}
