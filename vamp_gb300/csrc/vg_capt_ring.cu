// Query order of a CAPT's affordance lists on the GPU.
//
// A CAPT query (collision/capt.hh:425-506) descends to the leaf whose cell holds the sphere's
// centre and tests the sphere against every point afforded to that leaf: its answer is the OR
// over those points, so the points may be visited in any order.  A tree built for large spheres
// (r_max) affords each leaf every point within r_max + r_point of its cell, far more than a
// small sphere can reach.  Here each leaf's points are regrouped by their distance to the leaf's
// cell, in rings of width (r_max + r_point) / kRings, nearest ring first, and every 8-point block
// records the lower edge of the ring of its first point (non-decreasing along the leaf).  The
// query then scans only the blocks whose ring starts within its reach: a point at distance D
// from the cell is at least D from any centre inside it, so the blocks cut off cannot hold a hit.
#include "vg_capt_gpu.h"

#include "../../include/vamp_gb300.h"
#include "vg_internal.h"

#include <string>

namespace vg
{
    namespace
    {
        constexpr int kRings = 32;
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

        // One block per leaf: ring histogram, ring starts, scatter into the ring order, then the
        // ring lower bound of each of the leaf's blocks.
        __global__ void ring_order_kernel(const float *tests, int nlog2, const uint32_t *starts, const float *aff,
                                          double step, float *aff_q, float *ring_lo)
        {
            const long long leaf = blockIdx.x;
            const uint32_t b0 = starts[leaf], b1 = starts[leaf + 1];
            if (b0 == b1)
                return;
            __shared__ float cell[6];
            __shared__ unsigned count[kRings + 1], first[kRings + 2];
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
            for (int r = threadIdx.x; r <= kRings; r += blockDim.x)
                count[r] = 0;
            __syncthreads();
            const unsigned n = 8u * (b1 - b0);
            auto ring_of = [&](unsigned e) {
                const float *blk = aff + 24 * static_cast<size_t>(b0 + e / 8);
                const float x = blk[e % 8], y = blk[8 + e % 8], z = blk[16 + e % 8];
                if (!(x < __int_as_float(0x7f800000)))
                    return kRings;  // padding (+inf) goes last
                const double r = floor(cell_distance(cell, cell + 3, x, y, z) / step);
                return r < kRings - 1 ? static_cast<int>(r) : kRings - 1;
            };
            for (unsigned e = threadIdx.x; e < n; e += blockDim.x)
                atomicAdd(&count[ring_of(e)], 1u);
            __syncthreads();
            if (threadIdx.x == 0)
            {
                unsigned acc = 0;
                for (int r = 0; r <= kRings; ++r)
                {
                    first[r] = acc;
                    acc += count[r];
                    count[r] = first[r];  // becomes the scatter cursor
                }
                first[kRings + 1] = acc;
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
            // ring of each block's first entry, as a distance rounded down
            for (unsigned j = threadIdx.x; j < b1 - b0; j += blockDim.x)
            {
                const unsigned pos = 8u * j;
                int r = 0;
                while (r < kRings && first[r + 1] <= pos)
                    ++r;
                ring_lo[b0 + j] = r == kRings ? __int_as_float(0x7f800000) : __double2float_rd(r * step);
            }
        }
    }  // namespace

    int capt_ring_order(const float *tests, int nlog2, const uint32_t *starts, const float *aff, size_t blocks,
                        float r_max, float r_point, float **aff_q, float **ring_lo)
    {
        *aff_q = nullptr;
        *ring_lo = nullptr;
        cudaError_t e = cudaMalloc(aff_q, std::max<size_t>(blocks, 1) * 24 * sizeof(float));
        if (e == cudaSuccess)
            e = cudaMalloc(ring_lo, std::max<size_t>(blocks, 1) * sizeof(float));
        const long long leaves = 1ll << nlog2;
        const double step = (static_cast<double>(r_max) + r_point) / kRings;
        if (e == cudaSuccess && blocks > 0)
        {
            if (step > 0.0)
            {
                ring_order_kernel<<<static_cast<unsigned>(leaves), kRingThreads>>>(tests, nlog2, starts, aff, step, *aff_q,
                                                                                  *ring_lo);
                e = cudaGetLastError();
            }
            else
            {
                // a tree for radius 0: every point may matter, keep the list as built
                e = cudaMemcpy(*aff_q, aff, blocks * 24 * sizeof(float), cudaMemcpyDeviceToDevice);
                if (e == cudaSuccess)
                    e = cudaMemset(*ring_lo, 0, blocks * sizeof(float));
            }
        }
        if (e == cudaSuccess)
            e = cudaDeviceSynchronize();
        if (e != cudaSuccess)
        {
            if (*aff_q)
                cudaFree(*aff_q);
            if (*ring_lo)
                cudaFree(*ring_lo);
            *aff_q = *ring_lo = nullptr;
            return set_error(VG_ERR_CUDA, std::string("CAPT query order: ") + cudaGetErrorString(e));
        }
        return VG_OK;
    }
}  // namespace vg
