// CAPT construction on the GPU (vg_capt_gpu.cu): the same layout as capt_build (vg_capt.h).
#pragma once

#include <cuda_runtime.h>

#include "vg_check.cuh"

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

    // The tables a CAPT query reads on the device (vg_capt_ring.cu).  aff_q and tables are owned
    // by the caller once built (cudaFree each); nodes, leaves and ends point into tables.
    struct CaptQuery
    {
        float *aff_q = nullptr;     // blocks x 24: each leaf's points, nearest ring first
        void *tables = nullptr;     // one allocation holding the three tables below
        float4 *nodes = nullptr;    // split values three levels per node: 2 float4 per node
        float4 *leaves = nullptr;   // per leaf: lower xyz, upper x | upper yz, first block (bits), 0
        uint32_t *ends = nullptr;   // per leaf x kCaptRings: end of the blocks of ring r or nearer
        float top_tests[3] = {0, 0, 0};  // split values of the nlog2 mod 3 levels above the groups
        int rem = 0;                // nlog2 mod 3
        int groups = 0;             // nlog2 / 3
        float ring_edge[kCaptRings] = {};  // lower edge of ring r, rounded down
    };

    // Builds the query tables of a tree in device memory (its reference-layout arrays); synchronous.
    int capt_query_layout(const float *tests, int nlog2, const float *aabbs, const uint32_t *starts, const float *aff,
                          size_t blocks, float r_max, float r_point, CaptQuery &q);
}  // namespace vg
