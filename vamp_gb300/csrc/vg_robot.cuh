// Instantiates the kernels of one robot and describes them to the library (included by
// robot_<name>.cu after the robot's generated header).
#pragma once

#include "vg_internal.h"

namespace vg
{
    template <typename R, bool kExt = false>
    cudaError_t launch_states(const StatesParams &p, int grid, int block, int smem, cudaStream_t s)
    {
        states_kernel<R, kExt><<<grid, block, smem, s>>>(p);
        return cudaGetLastError();
    }

    template <typename R, int W, bool kExt = false>
    cudaError_t launch_blocks(const StatesParams &p, int grid, int block, int smem, cudaStream_t s)
    {
        blocks_kernel<R, W, kExt><<<grid, block, smem, s>>>(p);
        return cudaGetLastError();
    }

    template <typename R, int W, bool kExt = false>
    cudaError_t launch_edges(const EdgesParams &p, int grid, int block, int smem, cudaStream_t s)
    {
        edges_kernel<R, W, kExt><<<grid, block, smem, s>>>(p);
        return cudaGetLastError();
    }

    template <typename R>
    cudaError_t launch_ee_pose(const float *q, long long n, float *out, cudaStream_t s)
    {
        if (n <= 0)
        {
            return cudaSuccess;
        }
        ee_pose_kernel<R><<<static_cast<unsigned>((n + 127) / 128), 128, 0, s>>>(q, n, out);
        return cudaGetLastError();
    }

    template <typename R, int W, bool kLearned, int kMinBlocks = VG_MIN_BLOCKS, bool kLoopedEnv = VG_DEFAULT_LOOPED_ENV != 0>
    cudaError_t launch_edges_grouped(const EdgesParams &p, int grid, int block, int smem, cudaStream_t s)
    {
        edges_grouped_kernel<R, W, kLearned, kMinBlocks, kLoopedEnv><<<grid, block, smem, s>>>(p);
        return cudaGetLastError();
    }

    template <typename R, int W>
    cudaError_t launch_edge_order(const EdgesParams &p, int grid, int block, int smem, cudaStream_t s)
    {
        edge_order_kernel<R::kDim, W><<<grid, block, smem, s>>>(p);
        return cudaGetLastError();
    }

    template <typename R, int W, int kMinBlocks, bool kLoopedEnv>
    cudaError_t launch_edges_packed(const EdgesParams &p, int grid, int block, int smem, cudaStream_t s)
    {
        edges_packed_kernel<R, W, kMinBlocks, kLoopedEnv><<<grid, block, smem, s>>>(p);
        return cudaGetLastError();
    }

    template <typename R>
    cudaError_t launch_debug_self(const float *spheres, long long n, uint8_t *out, cudaStream_t s)
    {
        const long long t = n * R::kSelfPairs;
        if (t <= 0)
        {
            return cudaSuccess;
        }
        debug_self_kernel<R><<<static_cast<unsigned>((t + 255) / 256), 256, 0, s>>>(spheres, n, out);
        return cudaGetLastError();
    }

    template <typename R>
    cudaError_t launch_spheres(const float *q, long long n, float *out, cudaStream_t s)
    {
        if (n <= 0)
        {
            return cudaSuccess;
        }
        const int block = 128;
        spheres_kernel<R><<<static_cast<unsigned>((n + block - 1) / block), block, 0, s>>>(q, n, out);
        return cudaGetLastError();
    }

    template <typename R>
    RobotOps make_robot_ops(int default_schedule)
    {
        RobotOps o{};
        o.name = R::kName;
        o.default_schedule = default_schedule;
        o.dim = R::kDim;
        o.fine = R::kFine;
        o.slots = R::kSlots;
        o.resolution = R::kResolution;
        o.r_min = R::kMinRadius;
        o.r_max = R::kMaxRadius;
        o.s_m = R::kScaleM;
        o.s_a = R::kScaleA;
        o.states = &launch_states<R>;
        o.states_fn = reinterpret_cast<const void *>(&states_kernel<R>);
        o.blocks[0] = &launch_blocks<R, 8>;
        o.blocks[1] = &launch_blocks<R, 4>;
        o.blocks_fn[0] = reinterpret_cast<const void *>(&blocks_kernel<R, 8>);
        o.blocks_fn[1] = reinterpret_cast<const void *>(&blocks_kernel<R, 4>);
        o.blocks_ext[0] = &launch_blocks<R, 8, true>;
        o.blocks_ext[1] = &launch_blocks<R, 4, true>;
        o.blocks_ext_fn[0] = reinterpret_cast<const void *>(&blocks_kernel<R, 8, true>);
        o.blocks_ext_fn[1] = reinterpret_cast<const void *>(&blocks_kernel<R, 4, true>);
        o.edges[0] = &launch_edges<R, 8>;
        o.edges[1] = &launch_edges<R, 4>;
        o.edges_fn[0] = reinterpret_cast<const void *>(&edges_kernel<R, 8>);
        o.edges_fn[1] = reinterpret_cast<const void *>(&edges_kernel<R, 4>);
        o.edges_grouped[0] = &launch_edges_grouped<R, 8, false>;
        o.edges_grouped[1] = &launch_edges_grouped<R, 4, false>;
        o.edges_grouped_fn[0] = reinterpret_cast<const void *>(&edges_grouped_kernel<R, 8, false>);
        o.edges_grouped_fn[1] = reinterpret_cast<const void *>(&edges_grouped_kernel<R, 4, false>);
        o.edges_wide[0] = &launch_edges_grouped<R, 8, false, VG_MIN_BLOCKS_WIDE, true>;
        o.edges_wide[1] = &launch_edges_grouped<R, 4, false, VG_MIN_BLOCKS_WIDE, true>;
        o.edges_wide_fn[0] = reinterpret_cast<const void *>(&edges_grouped_kernel<R, 8, false, VG_MIN_BLOCKS_WIDE, true>);
        o.edges_wide_fn[1] = reinterpret_cast<const void *>(&edges_grouped_kernel<R, 4, false, VG_MIN_BLOCKS_WIDE, true>);
        o.edges_packed[0] = &launch_edges_packed<R, 8, VG_MIN_BLOCKS_WIDE, true>;
        o.edges_packed[1] = &launch_edges_packed<R, 4, VG_MIN_BLOCKS_WIDE, true>;
        o.edges_packed_fn[0] = reinterpret_cast<const void *>(&edges_packed_kernel<R, 8, VG_MIN_BLOCKS_WIDE, true>);
        o.edges_packed_fn[1] = reinterpret_cast<const void *>(&edges_packed_kernel<R, 4, VG_MIN_BLOCKS_WIDE, true>);
        // the learned order in the form of the fastest plain schedule for the Panda, UR5 and Fetch
        // (register-rich build, looped environment section); the group order comes precomputed
        // (edge_order_kernel), which keeps it within the registers of 4 resident blocks
        o.edges_learned[0] = &launch_edges_grouped<R, 8, true, VG_MIN_BLOCKS_WIDE, true>;
        o.edges_learned[1] = &launch_edges_grouped<R, 4, true, VG_MIN_BLOCKS_WIDE, true>;
        o.edges_learned_fn[0] = reinterpret_cast<const void *>(&edges_grouped_kernel<R, 8, true, VG_MIN_BLOCKS_WIDE, true>);
        o.edges_learned_fn[1] = reinterpret_cast<const void *>(&edges_grouped_kernel<R, 4, true, VG_MIN_BLOCKS_WIDE, true>);
        o.edge_order[0] = &launch_edge_order<R, 8>;
        o.edge_order[1] = &launch_edge_order<R, 4>;
        // extended checks (heightfields, fkcc_attach): the segment-per-edge and states kernels
        o.states_ext = &launch_states<R, true>;
        o.states_ext_fn = reinterpret_cast<const void *>(&states_kernel<R, true>);
        o.edges_ext[0] = &launch_edges<R, 8, true>;
        o.edges_ext[1] = &launch_edges<R, 4, true>;
        o.edges_ext_fn[0] = reinterpret_cast<const void *>(&edges_kernel<R, 8, true>);
        o.edges_ext_fn[1] = reinterpret_cast<const void *>(&edges_kernel<R, 4, true>);
        o.ee_pose = &launch_ee_pose<R>;
        o.stage_floats = R::kStage;
        o.spheres = &launch_spheres<R>;
        o.debug_self = &launch_debug_self<R>;
        o.self_pairs = R::kSelfPairs;
        return o;
    }
}  // namespace vg

// `schedule`: the edge schedule of an environment that was neither autotuned for the robot nor
// given one (vg_env_set_schedule); the autotuner's pick for the robot on its own edge workloads.
#define VG_DEFINE_ROBOT(Type, var, schedule)                                       \
    namespace vg                                                                   \
    {                                                                              \
        extern const RobotOps var;                                                 \
        const RobotOps var = make_robot_ops<vg::robots::Type>(schedule);           \
    }
