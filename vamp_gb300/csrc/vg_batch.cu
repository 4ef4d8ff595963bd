// Edge-check autotuning and mixed-robot batches replayed as one CUDA graph.
//
// The reference checks one edge at a time on the calling thread (planning/validate.hh:24-77); a
// GPU planner that batches several robots' edges (or repeats one batch with new contents in the
// same buffers) pays one kernel launch per robot and call.  A vg_batch records the checks once,
// captures them as a CUDA graph with one branch per check, and replays the graph on later
// launches.
#include "../../include/vamp_gb300.h"
#include "vg_internal.h"

#include <algorithm>
#include <string>
#include <vector>

using namespace vg;

struct vg_batch
{
    struct Part
    {
        const RobotOps *r;
        vg_env *env;
        const float *a, *b;
        size_t n;
        int resolution;
        vg_mlp *mlp;
        int probes;
        uint8_t *out;
        int32_t *blocks;
    };
    std::vector<Part> parts;
    std::vector<uint64_t> versions;  // environment image versions the graph was captured with
    int device = -1;
    unsigned *counters = nullptr;  // one work counter per part (64 bytes apart)
    size_t counters_cap = 0;
    std::vector<float *> scores;   // per part with an MLP: [n][probes]
    std::vector<uint8_t *> orders; // per part with an MLP: its edges' group orders, 16 bytes each
    cudaStream_t capture = nullptr;  // the graph is captured here (the caller's stream may be the legacy default stream, which cannot be captured)
    std::vector<cudaStream_t> side;
    std::vector<cudaEvent_t> events;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool stale = true;
};

namespace
{
    void drop_graph(vg_batch *b)
    {
        if (b->exec)
            cudaGraphExecDestroy(b->exec);
        if (b->graph)
            cudaGraphDestroy(b->graph);
        b->exec = nullptr;
        b->graph = nullptr;
        b->stale = true;
    }

    int record(vg_batch *bt, cudaStream_t s);

    // every allocation and upload a launch needs, done outside any capture
    int prepare(vg_batch *bt)
    {
        int dev = 0;
        VG_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
        if (bt->device >= 0 && bt->device != dev)
            return set_error(VG_ERR_STATE, "vg_batch_launch: the batch was launched on another device");
        bt->device = dev;
        for (auto &p : bt->parts)
        {
            if (int rc = commit(p.env))
                return rc;
        }
        const size_t need = bt->parts.size() * 16;
        if (need > bt->counters_cap)
        {
            if (bt->counters)
                cudaFree(bt->counters);
            bt->counters = nullptr;
            bt->counters_cap = 0;
            VG_CUDA(cudaMalloc(&bt->counters, need * sizeof(unsigned)), "cudaMalloc(batch counters)");
            bt->counters_cap = need;
        }
        while (bt->scores.size() < bt->parts.size())
            bt->scores.push_back(nullptr);
        while (bt->orders.size() < bt->parts.size())
            bt->orders.push_back(nullptr);
        for (size_t i = 0; i < bt->parts.size(); ++i)
        {
            const auto &p = bt->parts[i];
            if (p.mlp && !bt->scores[i])
            {
                VG_CUDA(cudaMalloc(&bt->scores[i], p.n * p.probes * sizeof(float)), "cudaMalloc(batch scores)");
            }
            if (p.mlp && !bt->orders[i])
            {
                VG_CUDA(cudaMalloc(&bt->orders[i], p.n * 16), "cudaMalloc(batch group orders)");
            }
        }
        if (!bt->capture)
        {
            VG_CUDA(cudaStreamCreateWithFlags(&bt->capture, cudaStreamNonBlocking), "cudaStreamCreate");
        }
        while (bt->side.size() < bt->parts.size())
        {
            cudaStream_t st;
            VG_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "cudaStreamCreate");
            bt->side.push_back(st);
        }
        while (bt->events.size() < bt->parts.size() + 1)
        {
            cudaEvent_t ev;
            VG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate");
            bt->events.push_back(ev);
        }
        return VG_OK;
    }

    // the batch's launches on stream s: one branch per part, forked from and joined into s
    int record(vg_batch *bt, cudaStream_t s)
    {
        VG_CUDA(cudaEventRecord(bt->events.back(), s), "fork");
        for (size_t i = 0; i < bt->parts.size(); ++i)
        {
            const auto &p = bt->parts[i];
            cudaStream_t st = bt->side[i];
            VG_CUDA(cudaStreamWaitEvent(st, bt->events.back(), 0), "fork wait");
            if (p.mlp)
            {
                if (int rc = vg_mlp_score_edges_device(p.mlp, p.a, p.b, p.n, p.probes, bt->scores[i], st))
                    return rc;
            }
            MotionLaunch m{p.r, p.env, p.a, p.b, p.n, p.resolution, p.mlp ? bt->scores[i] : nullptr, p.probes,
                           p.out, p.blocks, bt->counters + 16 * i};
            m.order = p.mlp ? bt->orders[i] : nullptr;
            tuned_for(p.env, p.r, &m.schedule, &m.blocks_per_sm);
            if (int rc = launch_motions(m, st))
                return rc;
            VG_CUDA(cudaEventRecord(bt->events[i], st), "join record");
            VG_CUDA(cudaStreamWaitEvent(s, bt->events[i], 0), "join wait");
        }
        return VG_OK;
    }
}  // namespace

extern "C" {

vg_batch *vg_batch_create(void)
{
    return new vg_batch();
}

void vg_batch_destroy(vg_batch *b)
{
    if (!b)
        return;
    drop_graph(b);
    if (b->counters)
        cudaFree(b->counters);
    for (uint8_t *p : b->orders)
        if (p)
            cudaFree(p);
    for (float *p : b->scores)
        if (p)
            cudaFree(p);
    if (b->capture)
        cudaStreamDestroy(b->capture);
    for (cudaStream_t st : b->side)
        cudaStreamDestroy(st);
    for (cudaEvent_t ev : b->events)
        cudaEventDestroy(ev);
    delete b;
}

int vg_batch_add_motions(vg_batch *b, const char *robot, vg_env *env, const float *a, const float *bb, size_t n,
                         int resolution, vg_mlp *mlp, int probes, uint8_t *out, int32_t *blocks)
{
    const RobotOps *r = find_robot(robot);
    if (!b || !r || !env || !a || !bb || !out || n == 0 || resolution < 1 || (mlp && (probes < 1 || probes > 32)))
        return set_error(VG_ERR_ARG, "vg_batch_add_motions: bad argument");
    if (n > 0x7fffffffu)
        return set_error(VG_ERR_LIMIT, "vg_batch_add_motions: more than 2^31 - 1 edges");
    if (b->parts.size() >= 64)
        return set_error(VG_ERR_LIMIT, "vg_batch_add_motions: at most 64 checks per batch");
    b->parts.push_back({r, env, a, bb, n, resolution, mlp, mlp ? probes : 0, out, blocks});
    drop_graph(b);
    return VG_OK;
}

int vg_batch_launch(vg_batch *b, void *stream)
{
    if (!b || b->parts.empty())
        return set_error(VG_ERR_ARG, "vg_batch_launch: empty batch");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    bool changed = b->versions.size() != b->parts.size();
    for (size_t i = 0; i < b->parts.size() && !changed; ++i)
        changed = b->parts[i].env->dirty || b->parts[i].env->version != b->versions[i];
    if (changed)
        drop_graph(b);  // an environment changed since the capture: upload it and capture again
    if (b->stale)
    {
        if (int rc = prepare(b))
            return rc;
        // the capture records the launches without running them
        VG_CUDA(cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        const int rc = record(b, b->capture);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(b->capture, &g);
        if (rc != VG_OK)
        {
            if (g)
                cudaGraphDestroy(g);
            return rc;
        }
        VG_CUDA(e, "cudaStreamEndCapture");
        b->graph = g;
        VG_CUDA(cudaGraphInstantiate(&b->exec, b->graph, 0), "cudaGraphInstantiate");
        b->versions.clear();
        for (const auto &p : b->parts)
            b->versions.push_back(p.env->version);
        b->stale = false;
    }
    VG_CUDA(cudaGraphLaunch(b->exec, s), "cudaGraphLaunch");
    return VG_OK;
}

// Times the edge-check schedules on the given edges (device buffers: a sample of the caller's
// workload) and keeps the fastest for this robot in env: a segment or a warp per edge, and the
// resident blocks per SM.  Synchronous.
int vg_autotune_motions(const char *robot, vg_env *env, const float *a, const float *b, size_t n, int resolution,
                        int *schedule_out, int *blocks_per_sm_out, float *ms_out, void *stream)
{
    const RobotOps *r = find_robot(robot);
    if (!r || !env || !a || !b || n == 0 || resolution < 1)
        return set_error(VG_ERR_ARG, "vg_autotune_motions: bad argument");
    if (n > 0x7fffffffu)
        return set_error(VG_ERR_LIMIT, "vg_autotune_motions: more than 2^31 - 1 edges");
    if (int rc = commit(env))
        return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint8_t *out = nullptr;
    VG_CUDA(cudaMalloc(&out, n), "cudaMalloc(autotune)");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int best_s = 1, best_b = 0, rc = VG_OK;
    float best = 1e30f;
    const int which = env->lanes == 8 ? 0 : 1;
    const int smem = static_cast<int>(staged_f4(static_cast<int>(env->image_f4)) * sizeof(float4)) + r->stage_floats * kBlock * 4;
    for (int sched = 0; sched < 4 && rc == VG_OK; ++sched)
    {
        int occ = 0;
        const void *fn = sched == 0   ? r->edges_fn[which]
                         : sched == 1 ? r->edges_grouped_fn[which]
                         : sched == 2 ? r->edges_wide_fn[which]
                                      : r->edges_packed_fn[which];
        rc = prepare_kernel(fn, smem, kBlock, &occ);
        for (int bps = occ; bps >= 1 && rc == VG_OK; --bps)
        {
            MotionLaunch m{r, env, a, b, n, resolution, nullptr, 0, out, nullptr, env->d_counter, sched, bps};
            float t = 1e30f;
            for (int rep = 0; rep < 3 && rc == VG_OK; ++rep)
            {
                cudaEventRecord(e0, s);
                rc = launch_motions(m, s);
                cudaEventRecord(e1, s);
                if (cudaEventSynchronize(e1) != cudaSuccess)
                    rc = set_error(VG_ERR_CUDA, "vg_autotune_motions: kernel failure");
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                if (rep > 0)  // the first run warms up
                    t = std::min(t, ms);
            }
            if (t < best)
            {
                best = t;
                best_s = sched;
                best_b = bps == occ ? 0 : bps;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (rc != VG_OK)
        return rc;
    bool found = false;
    for (RobotTune &t : env->tuned)
    {
        if (t.robot == r)
        {
            t.schedule = best_s;
            t.blocks_per_sm = best_b;
            found = true;
        }
    }
    if (!found)
        env->tuned.push_back({r, best_s, best_b});
    if (schedule_out)
        *schedule_out = best_s;
    if (blocks_per_sm_out)
        *blocks_per_sm_out = best_b;
    if (ms_out)
        *ms_out = best;
    return VG_OK;
}

}  // extern "C"
