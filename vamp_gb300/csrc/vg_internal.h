// Internal host-side declarations shared by the translation units of libvamp_gb300.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "vg_capt.h"
#include "vg_capt_gpu.h"
#include "vg_kernels.cuh"

namespace vg
{
    // One robot's kernels and constants, defined in robot_<name>.cu.
    struct RobotOps
    {
        const char *name;
        int dim, fine, slots, resolution;
        int default_schedule;  // edge schedule when the environment has neither a pick nor a setting
        float r_min, r_max;
        const float *s_m;
        const float *s_a;
        cudaError_t (*states)(const StatesParams &, int grid, int block, int smem, cudaStream_t);
        const void *states_fn;
        // caller-given blocks of 8 (index 0) or 4 (index 1) configurations (Robot::fkcc), and the
        // extended form
        cudaError_t (*blocks[2])(const StatesParams &, int grid, int block, int smem, cudaStream_t);
        const void *blocks_fn[2];
        cudaError_t (*blocks_ext[2])(const StatesParams &, int grid, int block, int smem, cudaStream_t);
        const void *blocks_ext_fn[2];
        // edges: index 0 = 8-lane blocks, 1 = 4-lane blocks
        cudaError_t (*edges[2])(const EdgesParams &, int grid, int block, int smem, cudaStream_t);
        const void *edges_fn[2];
        // same-edge schedule (a warp checks consecutive blocks of one edge)
        cudaError_t (*edges_grouped[2])(const EdgesParams &, int grid, int block, int smem, cudaStream_t);
        const void *edges_grouped_fn[2];
        // same-edge schedule compiled for fewer resident blocks (more registers per thread)
        cudaError_t (*edges_wide[2])(const EdgesParams &, int grid, int block, int smem, cudaStream_t);
        const void *edges_wide_fn[2];
        // the register-rich same-edge schedule with the segments an edge leaves free given to the
        // next edge
        cudaError_t (*edges_packed[2])(const EdgesParams &, int grid, int block, int smem, cudaStream_t);
        const void *edges_packed_fn[2];
        // each edge's group order from its scores (before the learned-order check)
        cudaError_t (*edge_order[2])(const EdgesParams &, int grid, int block, int smem, cudaStream_t);
        // same-edge schedule in a learned block order (EdgesParams::order)
        cudaError_t (*edges_learned[2])(const EdgesParams &, int grid, int block, int smem, cudaStream_t);
        const void *edges_learned_fn[2];
        // extended forms (heightfields in the environment, or an attachment: fkcc_attach): states,
        // and edges a segment each
        cudaError_t (*states_ext)(const StatesParams &, int grid, int block, int smem, cudaStream_t);
        const void *states_ext_fn;
        cudaError_t (*edges_ext[2])(const EdgesParams &, int grid, int block, int smem, cudaStream_t);
        const void *edges_ext_fn[2];
        // Robot::eefk: row-major 4x4 transforms [n][16] from configurations [n][dim]
        cudaError_t (*ee_pose)(const float *, long long, float *, cudaStream_t);
        int stage_floats;  // shared-memory staging floats per thread (after the environment image)
        cudaError_t (*spheres)(const float *, long long, float *, cudaStream_t);
        // fkcc_debug's self part: flags [n][self_pairs] from sphere slots [n][slots][4]
        cudaError_t (*debug_self)(const float *, long long, uint8_t *, cudaStream_t);
        int self_pairs;  // fine pairs over all self checks
    };

    const RobotOps *find_robot(const char *name);
    const RobotOps *const *all_robots(int *count);

    // thread-local last error message
    int set_error(int code, const std::string &msg);
    int cuda_fail(cudaError_t e, const char *what);

// return VG_ERR_CUDA (with the CUDA error in the message) from the enclosing function on failure
#define VG_CUDA(call, what)                 \
    do                                      \
    {                                       \
        const cudaError_t _e = (call);      \
        if (_e != cudaSuccess)              \
        {                                   \
            return vg::cuda_fail(_e, what); \
        }                                   \
    } while (0)

    // device buffers per pointcloud: tests, aabbs, starts, reference-layout blocks (device-built
    // clouds only), ring-ordered blocks, query tables
    constexpr size_t kCloudBuffers = 6;

    // threads per block of every checking kernel (the robots' stage stride)
    constexpr int kBlock = 128;
    static_assert(kBlock == kStageStride, "stage columns are one per thread of a block");

    // An autotuned schedule for one robot in one environment.
    struct RobotTune
    {
        const RobotOps *robot;
        int schedule;       // 0: a segment per edge, 1: a warp per edge, 2: a warp per edge, register-rich build,
                            // 3: as 2 with free segments starting on the next edge
        int blocks_per_sm;  // resident blocks per SM (0: as many as fit)
    };
}  // namespace vg

// The C-ABI environment handle.
struct vg_env
{
    // host copies, sorted by min_distance; each row: fields then min_distance (oracle layout)
    std::vector<float> obj[5];
    std::vector<int> ids[5];  // insertion id (0, 1, ... over all kinds) of each row of obj
    int n_added = 0;
    int lanes = 8;
    int sqrt_mode = 0;
    int schedule = -1;  // -1: each robot's default; 0: a segment per edge, 1: a warp per edge (consecutive
                        // blocks), 2: 1 register-rich, 3: 2 packed
    bool dirty = true;
    int device = -1;
    // device image
    float4 *d_image = nullptr;
    size_t image_f4 = 0, image_cap = 0;
    int off[5] = {0, 0, 0, 0, 0};
    int cloud_off = 0;
    // attachment (vg_env_attach): relative transform rows {R[r][0..2], t[r]}, then spheres
    // {x, y, z, r}; n_att = -1 while none is attached
    int n_att = -1;
    std::vector<float> att;
    int att_off = 0;
    // heightfields (vg_env_add_heightfield): descriptors (data pointer filled at upload), host
    // samples, one device buffer each
    std::vector<vg::HeightView> hf;
    std::vector<std::vector<float>> hf_data;
    std::vector<void *> d_hf;
    int hf_off = 0;
    // environments with heightfields or an attachment run the extended kernels
    bool extended() const { return n_att >= 0 || !hf.empty(); }
    int n[5] = {0, 0, 0, 0, 0};
    // pointclouds: host trees, their device buffers and the query tables built from them
    std::vector<vg::CaptHost> clouds;
    std::vector<void *> d_clouds;        // kCloudBuffers buffers per uploaded cloud
    std::vector<vg::CaptQuery> capt_q;   // per uploaded cloud (pointers into d_clouds)
    // learned-order group orders (vg_validate_motions_scored_device), 16 bytes per edge
    uint8_t *d_order = nullptr;
    size_t order_cap = 0;
    // library-owned scratch: work counter, staging for host-pointer calls
    unsigned *d_counter = nullptr;
    void *d_stage = nullptr;
    size_t stage_cap = 0;
    // pinned host staging of small host-pointer edge batches (their blocks, then their verdicts)
    void *h_pin = nullptr;
    size_t pin_cap = 0;
    // per-robot picks of vg_autotune_motions (cleared by vg_env_set_schedule)
    std::vector<vg::RobotTune> tuned;
    // incremented by every upload of the image: CUDA graphs that captured an older image (its
    // address and sizes) must be captured again
    uint64_t version = 0;
};

namespace vg
{
    // One edge check, launched by launch_motions (the environment already on the device).
    struct MotionLaunch
    {
        const RobotOps *r;
        const vg_env *env;
        const float *a;
        const float *b;
        size_t n;
        int resolution;
        const float *scores;  // non-null: learned block order (same-edge schedule)
        int probes;
        uint8_t *out;
        int32_t *blocks;
        unsigned *counter;     // work counter, cleared on the stream before the launch
        int schedule = 1;      // 0: a segment per edge, 1: a warp per edge, 2: the same, register-rich build, 3: 2 packed
        int blocks_per_sm = 0;  // 0: as many as fit
        const float *dist = nullptr;  // validate_vector form: b holds vectors, dist their lengths
        uint8_t *order = nullptr;     // with scores: scratch of n x 16 bytes for the group orders
    };

    int commit(vg_env *e);
    EnvDevice env_device(const vg_env *e);
    int sm_count();
    int prepare_kernel(const void *fn, int smem, int block, int *blocks_per_sm);
    void tuned_for(const vg_env *env, const RobotOps *r, int *schedule, int *blocks_per_sm);
    int launch_motions(const MotionLaunch &m, cudaStream_t s);
}  // namespace vg
