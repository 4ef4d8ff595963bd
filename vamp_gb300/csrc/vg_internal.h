// Internal host-side declarations shared by the translation units of libvamp_gb300.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "vg_capt.h"
#include "vg_kernels.cuh"

namespace vg
{
    // One robot's kernels and constants, defined in robot_<name>.cu.
    struct RobotOps
    {
        const char *name;
        int dim, fine, slots, resolution;
        float r_min, r_max;
        const float *s_m;
        const float *s_a;
        cudaError_t (*states)(const StatesParams &, int grid, int block, int smem, cudaStream_t);
        const void *states_fn;
        // edges: index 0 = 8-lane blocks, 1 = 4-lane blocks
        cudaError_t (*edges[2])(const EdgesParams &, int grid, int block, int smem, cudaStream_t);
        const void *edges_fn[2];
        // same-edge schedule (a warp checks consecutive blocks of one edge)
        cudaError_t (*edges_grouped[2])(const EdgesParams &, int grid, int block, int smem, cudaStream_t);
        const void *edges_grouped_fn[2];
        // same-edge schedule in a learned block order (EdgesParams::scores)
        cudaError_t (*edges_learned[2])(const EdgesParams &, int grid, int block, int smem, cudaStream_t);
        const void *edges_learned_fn[2];
        int stage_floats;  // shared-memory staging floats per thread (after the environment image)
        cudaError_t (*spheres)(const float *, long long, float *, cudaStream_t);
    };

    const RobotOps *find_robot(const char *name);
    const RobotOps *const *all_robots(int *count);

    // thread-local last error message
    int set_error(int code, const std::string &msg);
}  // namespace vg

// The C-ABI environment handle.
struct vg_env
{
    // host copies, sorted by min_distance; each row: fields then min_distance (oracle layout)
    std::vector<float> obj[5];
    int lanes = 8;
    int sqrt_mode = 0;
    int schedule = 1;  // 0: a segment per edge, 1: a warp per edge (consecutive blocks)
    bool dirty = true;
    int device = -1;
    // device image
    float4 *d_image = nullptr;
    size_t image_f4 = 0, image_cap = 0;
    int off[5] = {0, 0, 0, 0, 0};
    int cloud_off = 0;
    int n[5] = {0, 0, 0, 0, 0};
    // pointclouds: host trees and their device copies (tests, aabbs, starts, aff per cloud)
    std::vector<vg::CaptHost> clouds;
    std::vector<void *> d_clouds;  // 4 buffers per uploaded cloud
    // library-owned scratch: work counter, staging for host-pointer calls
    unsigned *d_counter = nullptr;
    void *d_stage = nullptr;
    size_t stage_cap = 0;
};
