// Query tables of a CAPT on the GPU.
//
// A CAPT query (collision/capt.hh:425-506) tests a sphere against the top box, descends the
// split tree to the leaf whose cell holds the centre, tests the leaf's box and ORs the
// sphere-point tests over the points afforded to that leaf.  In the reference layout
// (capt.hh:584-617: heap-ordered split values, leaf boxes, block ranges) that is a chain of
// dependent loads, one per tree level, then the box, then the range.  The tables built here
// answer the same query with fewer loads:
//  * nodes: the split values three levels at a time, the 7 values of a 3-level subtree in one
//    32-byte node, so a descent of nlog2 levels reads nlog2 / 3 nodes (the nlog2 mod 3 levels
//    above the first full group travel with the tree's view);
//  * leaves: per leaf its box and first block in one 32-byte record;
//  * rings: a tree built for large spheres (r_max) affords each leaf every point within
//    r_max + r_point of its cell, far more than a small sphere can reach.  Each leaf's points
//    are regrouped by their distance to the leaf's cell, in kCaptRings rings of width
//    (r_max + r_point) / kCaptRings, nearest ring first, and ends[leaf][r] is the end of the
//    leaf's blocks whose first point lies in ring r or nearer.  A point at distance D from the
//    cell is at least D from any centre inside it, so a query scans only the blocks up to the
//    last ring whose lower edge is within its reach.
// The split comparisons, boxes and point tests are the reference's on the same floats, and the
// OR over the scanned points does not depend on their order, so the answers are the reference
// layout's.
#include "vg_capt_gpu.h"

#include "../../include/vamp_gb300.h"
#include "vg_internal.h"

#include <cmath>
#include <string>

namespace vg
{
    namespace
    {
        constexpr int kRingThreads = 128;

        // distance from (x, y, z) to the box lo..hi (infinite sides allowed), in double
        __device__ double cell_distance(const float *lo, const float *hi, float x, float y, float z)
        {
            const float p[3] = {x, y, z};
            double s = 0.0;
            for (int k = 0; k < 3; ++k)
            {
                double d = 0.0;
                if (p[k] < lo[k])
                    d = static_cast<double>(lo[k]) - p[k];
                else if (p[k] > hi[k])
                    d = static_cast<double>(p[k]) - hi[k];
                s += d * d;
            }
            return sqrt(s);
        }

        // One block per leaf: its record, then the ring histogram, ring starts, the scatter into
        // ring order and the ring ends.  step <= 0 (a tree for radius 0): every point may matter,
        // so all points share ring 0.
        __global__ void leaf_kernel(const float *tests, int nlog2, const float *aabbs, const uint32_t *starts,
                                    const float *aff, double step, float *aff_q, float4 *leaves, uint32_t *ends)
        {
            const long long leaf = blockIdx.x;
            const uint32_t b0 = starts[leaf], b1 = starts[leaf + 1];
            if (threadIdx.x == 0)
            {
                const float *box = aabbs + 6 * leaf;
                leaves[2 * leaf] = make_float4(box[0], box[1], box[2], box[3]);
                leaves[2 * leaf + 1] = make_float4(box[4], box[5], __uint_as_float(b0), 0.0f);
            }
            uint32_t *end = ends + leaf * kCaptRings;
            if (b0 == b1)
            {
                for (int r = threadIdx.x; r < kCaptRings; r += blockDim.x)
                    end[r] = b0;
                return;
            }
            __shared__ float cell[6];
            __shared__ unsigned count[kCaptRings + 1], first[kCaptRings + 2];
            if (threadIdx.x == 0)
            {
                // the leaf's cell: the split planes along its path (right child: coordinate >= test)
                const float inf = __int_as_float(0x7f800000);
                float lo[3] = {-inf, -inf, -inf}, hi[3] = {inf, inf, inf};
                long long idx = 0;
                for (int d = 0; d < nlog2; ++d)
                {
                    const int right = static_cast<int>((leaf >> (nlog2 - 1 - d)) & 1);
                    const float t = tests[idx];
                    if (right)
                        lo[d % 3] = t;
                    else
                        hi[d % 3] = t;
                    idx = 2 * idx + 1 + right;
                }
                for (int k = 0; k < 3; ++k)
                {
                    cell[k] = lo[k];
                    cell[3 + k] = hi[k];
                }
            }
            for (int r = threadIdx.x; r <= kCaptRings; r += blockDim.x)
                count[r] = 0;
            __syncthreads();
            const unsigned n = 8u * (b1 - b0);
            auto ring_of = [&](unsigned e) {
                const float *blk = aff + 24 * static_cast<size_t>(b0 + e / 8);
                const float x = blk[e % 8], y = blk[8 + e % 8], z = blk[16 + e % 8];
                if (!(x < __int_as_float(0x7f800000)))
                    return kCaptRings;  // padding (+inf) goes last
                if (!(step > 0.0))
                    return 0;
                const double r = floor(cell_distance(cell, cell + 3, x, y, z) / step);
                return r < kCaptRings - 1 ? static_cast<int>(r) : kCaptRings - 1;
            };
            for (unsigned e = threadIdx.x; e < n; e += blockDim.x)
                atomicAdd(&count[ring_of(e)], 1u);
            __syncthreads();
            if (threadIdx.x == 0)
            {
                unsigned acc = 0;
                for (int r = 0; r <= kCaptRings; ++r)
                {
                    first[r] = acc;
                    acc += count[r];
                    count[r] = first[r];  // becomes the scatter cursor
                }
                first[kCaptRings + 1] = acc;
            }
            __syncthreads();
            for (unsigned e = threadIdx.x; e < n; e += blockDim.x)
            {
                const unsigned pos = atomicAdd(&count[ring_of(e)], 1u);
                const float *src = aff + 24 * static_cast<size_t>(b0 + e / 8);
                float *dst = aff_q + 24 * static_cast<size_t>(b0 + pos / 8);
                dst[pos % 8] = src[e % 8];
                dst[8 + pos % 8] = src[8 + e % 8];
                dst[16 + pos % 8] = src[16 + e % 8];
            }
            // the blocks whose first entry lies in ring r or nearer: those starting before ring
            // r + 1 does
            for (int r = threadIdx.x; r < kCaptRings; r += blockDim.x)
                end[r] = b0 + (first[r + 1] + 7u) / 8u;
        }

        // Node i of the grouped split values: groups g = 0, 1, ... hold 2^rem * 8^g nodes; node j
        // of group g is the 3-level subtree whose root is entry j of tree level rem + 3g, its 7
        // split values in heap order (root, two children, four grandchildren), then a pad.
        __global__ void nodes_kernel(const float *tests, int rem, long long n_nodes, float4 *nodes)
        {
            for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n_nodes;
                 i += static_cast<long long>(gridDim.x) * blockDim.x)
            {
                long long j = i, size = 1ll << rem;
                int g = 0;
                while (j >= size)
                {
                    j -= size;
                    size *= 8;
                    ++g;
                }
                const long long h = (1ll << (rem + 3 * g)) - 1 + j;
                nodes[2 * i] = make_float4(tests[h], tests[2 * h + 1], tests[2 * h + 2], tests[4 * h + 3]);
                nodes[2 * i + 1] = make_float4(tests[4 * h + 4], tests[4 * h + 5], tests[4 * h + 6], 0.0f);
            }
        }

        // v rounded to a float towards -inf (v finite, >= 0)
        float round_down(double v)
        {
            float f = static_cast<float>(v);
            if (static_cast<double>(f) > v)
                f = std::nextafter(f, -INFINITY);
            return f;
        }
    }  // namespace

    int capt_query_layout(const float *tests, int nlog2, const float *aabbs, const uint32_t *starts, const float *aff,
                          size_t blocks, float r_max, float r_point, CaptQuery &q)
    {
        q = CaptQuery{};
        q.rem = nlog2 % 3;
        q.groups = nlog2 / 3;
        const long long leaves = 1ll << nlog2;
        const long long n_nodes = ((1ll << q.rem) * ((1ll << (3 * q.groups)) - 1)) / 7;
        const double step = (static_cast<double>(r_max) + r_point) / kCaptRings;
        for (int r = 0; r < kCaptRings; ++r)
            q.ring_edge[r] = step > 0.0 ? round_down(r * step) : 0.0f;
        const size_t node_bytes = static_cast<size_t>(n_nodes) * 2 * sizeof(float4);
        const size_t leaf_bytes = static_cast<size_t>(leaves) * 2 * sizeof(float4);
        const size_t end_bytes = static_cast<size_t>(leaves) * kCaptRings * sizeof(uint32_t);
        cudaError_t e = cudaMalloc(&q.aff_q, std::max<size_t>(blocks, 1) * 24 * sizeof(float));
        if (e == cudaSuccess)
            e = cudaMalloc(&q.tables, node_bytes + leaf_bytes + end_bytes);
        if (e == cudaSuccess)
        {
            char *base = static_cast<char *>(q.tables);
            q.nodes = reinterpret_cast<float4 *>(base);
            q.leaves = reinterpret_cast<float4 *>(base + node_bytes);
            q.ends = reinterpret_cast<uint32_t *>(base + node_bytes + leaf_bytes);
            const int top = static_cast<int>(std::min<long long>(3, leaves - 1));
            if (top > 0)
                e = cudaMemcpy(q.top_tests, tests, top * sizeof(float), cudaMemcpyDeviceToHost);
        }
        if (e == cudaSuccess && n_nodes > 0)
        {
            const int grid = static_cast<int>(std::min<long long>((n_nodes + 255) / 256, 4096));
            nodes_kernel<<<grid, 256>>>(tests, q.rem, n_nodes, q.nodes);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
        {
            leaf_kernel<<<static_cast<unsigned>(leaves), kRingThreads>>>(tests, nlog2, aabbs, starts, aff, step, q.aff_q,
                                                                         q.leaves, q.ends);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
            e = cudaDeviceSynchronize();
        if (e != cudaSuccess)
        {
            if (q.aff_q)
                cudaFree(q.aff_q);
            if (q.tables)
                cudaFree(q.tables);
            q = CaptQuery{};
            return set_error(VG_ERR_CUDA, std::string("CAPT query tables: ") + cudaGetErrorString(e));
        }
        return VG_OK;
    }
}  // namespace vg
