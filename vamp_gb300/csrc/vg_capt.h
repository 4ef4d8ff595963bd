// Host-side CAPT (collision-affording point tree) construction for the GPU query.
//
// Builds the tree exactly as the reference does (collision/capt.hh:104-365), so that GPU queries
// return the reference's answers, including the points the reference's builder does not afford
// (capt.hh:226-233 scans the lower half for the upper child from its smallest coordinate).
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace vg
{
    struct CaptHost
    {
        int nlog2 = 0;
        std::vector<float> tests;           // 2^nlog2 - 1 split values, heap order
        std::vector<float> aabbs;           // 2^nlog2 leaves x 6: lower xyz, upper xyz
        std::vector<uint32_t> aff_starts;   // 2^nlog2 + 1, in 8-point blocks
        std::vector<float> aff;             // blocks x 24: x[8], y[8], z[8]
        float top[6] = {0, 0, 0, 0, 0, 0};  // box of all finite points
        float r_min = 0, r_max = 0, r_point = 0;
        // built on the GPU: the arrays exist only in device memory (sizes below)
        bool on_device = false;
        size_t device_blocks = 0;

        size_t blocks() const { return on_device ? device_blocks : aff.size() / 24; }
        size_t n_tests() const { return on_device ? (size_t{1} << nlog2) - 1 : tests.size(); }
        size_t n_leaves() const { return on_device ? size_t{1} << nlog2 : aabbs.size() / 6; }
    };

    // Returns false if there are fewer than 2 points.
    bool capt_build(const float *xyz, size_t n, float r_min, float r_max, float r_point, CaptHost &out);
}  // namespace vg
