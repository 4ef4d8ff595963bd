// CAPT construction on the GPU (vg_capt_gpu.cu): the same layout as capt_build (vg_capt.h).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace vg
{
    // A tree built on the device: its arrays in device memory (CaptHost's layout), its scalars on
    // the host.
    struct DeviceCapt
    {
        int nlog2 = 0;
        float r_min = 0, r_max = 0, r_point = 0;
        float top[6] = {0, 0, 0, 0, 0, 0};
        size_t blocks = 0;                       // 8-point affordance blocks
        float *tests = nullptr;                  // 2^nlog2 - 1
        float *aabbs = nullptr;                  // 2^nlog2 x 6
        uint32_t *starts = nullptr;              // 2^nlog2 + 1
        float *aff = nullptr;                    // blocks x 24
        unsigned long long *starts_dev = nullptr;  // (build scratch)
        float *top_dev = nullptr;                  // (build scratch)

        void release();
    };

    // Builds the tree of n points xyz[n][3] (device memory) on the current device.
    int capt_build_device(const float *xyz, size_t n, float r_min, float r_max, float r_point, cudaStream_t s,
                          DeviceCapt &out);

    // The query order of a tree's affordance lists (vg_capt_ring.cu): each leaf's points
    // regrouped by distance to the leaf's cell, nearest ring first (aff_q, blocks x 24), and per
    // block the lower edge of its first point's ring (ring_lo, non-decreasing within a leaf).
    // Allocates both; synchronous.
    int capt_ring_order(const float *tests, int nlog2, const uint32_t *starts, const float *aff, size_t blocks,
                        float r_max, float r_point, float **aff_q, float **ring_lo);
}  // namespace vg
