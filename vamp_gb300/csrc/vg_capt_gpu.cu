// CAPT construction on the GPU, with the same layout as the host builder (vg_capt.cpp, which
// follows collision/capt.hh:104-365 bit for bit, the capt.hh:226-233 scan included).
//
// The host builder splits recursively; this one goes level by level.  At level d every node
// holds N >> d consecutive entries of the point order: a bitonic network sorts each node's
// entries by (coordinate on axis d mod 3, current position), which is exactly the host's stable
// sort.  Each node's split value, the two scans of its sorted halves (capt.hh:226-233) and its
// children's cells follow from the sorted keys.  Its affordance list (the points of other nodes
// within r_max of its cell) is filtered into its children's lists in order, one thread block per
// node (ordered compaction), and the scanned ranges are appended, as the host builder does.  At
// the leaves, each leaf's representative and its afforded points that pass the cell test become
// its 8-point blocks, its box and its block range.
#include "vg_capt_gpu.h"

#include "../../include/vamp_gb300.h"
#include "vg_internal.h"

#include <algorithm>
#include <type_traits>
#include <string>
#include <vector>

namespace vg
{
    namespace
    {
        constexpr float kInf = __builtin_huge_valf();
        constexpr int kListBlock = 128;  // threads per node in the list passes

        __global__ void init_points(const float *xyz, long long n, long long N, float *px, float *py, float *pz,
                                    uint32_t *ord)
        {
            const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
            if (i >= N)
                return;
            px[i] = i < n ? xyz[3 * i + 0] : kInf;
            py[i] = i < n ? xyz[3 * i + 1] : kInf;
            pz[i] = i < n ? xyz[3 * i + 2] : kInf;
            ord[i] = static_cast<uint32_t>(i);
        }

        __global__ void load_keys(const uint32_t *ord, const float *axis, long long N, float *key, uint32_t *pos)
        {
            const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
            if (i >= N)
                return;
            key[i] = axis[ord[i]];
            pos[i] = static_cast<uint32_t>(i);
        }

        // One compare-exchange stage of a bitonic network that sorts every aligned segment of S
        // entries ascending by (key, pos).
        __global__ void bitonic_stage(float *key, uint32_t *pos, uint32_t *ord, long long N, long long k, long long j,
                                      long long S)
        {
            const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
            const long long p = i ^ j;
            if (i >= N || p <= i)
                return;
            const bool up = k == S || (i & k) == 0;
            const float ki = key[i], kp = key[p];
            const bool greater = ki > kp || (ki == kp && pos[i] > pos[p]);
            if (greater == up)
            {
                key[i] = kp;
                key[p] = ki;
                const uint32_t a = pos[i];
                pos[i] = pos[p];
                pos[p] = a;
                const uint32_t o = ord[i];
                ord[i] = ord[p];
                ord[p] = o;
            }
        }

        constexpr int kSortTile = 2048;  // entries per shared-memory tile of the sort

        // All compare-exchange stages of sizes k in [k0, k1] and strides below the tile, on tiles
        // of T = min(S, 2048) entries (S: the sorted segment size, a power of two).
        __global__ void bitonic_tile(float *key, uint32_t *pos, uint32_t *ord, long long S, long long k0, long long k1)
        {
            __shared__ float sk[kSortTile];
            __shared__ uint32_t sp[kSortTile], so[kSortTile];
            const long long T = S < kSortTile ? S : kSortTile;
            const long long base = static_cast<long long>(blockIdx.x) * T;
            for (long long t = threadIdx.x; t < T; t += blockDim.x)
            {
                sk[t] = key[base + t];
                sp[t] = pos[base + t];
                so[t] = ord[base + t];
            }
            __syncthreads();
            for (long long k = k0; k <= k1; k <<= 1)
            {
                for (long long j = (k >> 1) < (T >> 1) ? (k >> 1) : (T >> 1); j > 0; j >>= 1)
                {
                    for (long long t = threadIdx.x; t < (T >> 1); t += blockDim.x)
                    {
                        const long long i = 2 * t - (t & (j - 1)), q = i + j;
                        const bool up = k == S || ((base + i) & k) == 0;
                        const float ki = sk[i], kq = sk[q];
                        const bool greater = ki > kq || (ki == kq && sp[i] > sp[q]);
                        if (greater == up)
                        {
                            sk[i] = kq;
                            sk[q] = ki;
                            const uint32_t a = sp[i];
                            sp[i] = sp[q];
                            sp[q] = a;
                            const uint32_t o = so[i];
                            so[i] = so[q];
                            so[q] = o;
                        }
                    }
                    __syncthreads();
                }
            }
            for (long long t = threadIdx.x; t < T; t += blockDim.x)
            {
                key[base + t] = sk[t];
                pos[base + t] = sp[t];
                ord[base + t] = so[t];
            }
        }

        struct NodeInfo
        {
            float up, down;
            long long h, l;  // ends of the two scanned ranges (capt.hh:226-233)
        };

        // first index in [lo, hi) whose key is > v (keys ascending)
        __device__ long long upper_bound(const float *key, long long lo, long long hi, float v)
        {
            while (lo < hi)
            {
                const long long m = lo + ((hi - lo) >> 1);
                if (key[m] > v)
                    hi = m;
                else
                    lo = m + 1;
            }
            return lo;
        }

        // per node of level d: split value, scan ends, children's cells
        __global__ void split_nodes(const float *key, long long N, int d, float r_max, const float *cell, float *tests,
                                    NodeInfo *info, float *child_cell)
        {
            const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
            if (t >= (1ll << d))
                return;
            const long long S = N >> d, half = S >> 1, begin = t * S;
            const float test = __fmul_rn(__fadd_rn(key[begin + half - 1], key[begin + half]), 0.5f);
            tests[(1ll << d) - 1 + t] = test;
            NodeInfo ni;
            ni.up = __fadd_rn(test, r_max);
            ni.down = __fsub_rn(test, r_max);
            // lower half, from its smallest key: while key >= down and finite
            if (key[begin] >= ni.down && key[begin] < kInf && key[begin] > -kInf)
                ni.h = upper_bound(key, begin, begin + half, __int_as_float(0x7f7fffff));  // up to the first +inf
            else
                ni.h = begin;
            // upper half: while key <= up and finite
            ni.l = key[begin + half] > -kInf ? upper_bound(key, begin + half, begin + S, ni.up) : begin + half;
            {
                const long long f = upper_bound(key, begin + half, begin + S, __int_as_float(0x7f7fffff));
                ni.l = ni.l < f ? ni.l : f;
            }
            info[t] = ni;
            const int ax = d % 3;
            float *lo = child_cell + 12 * t, *hi = lo + 6;
            for (int k = 0; k < 6; ++k)
            {
                lo[k] = cell[6 * t + k];
                hi[k] = cell[6 * t + k];
            }
            lo[3 + ax] = test;  // lower child: upper bound on the axis
            hi[ax] = test;      // upper child: lower bound on the axis
        }

        // block-wide exclusive scan of one flag per thread; returns the thread's offset, *total
        // the block's count
        __device__ unsigned block_scan(unsigned flag, unsigned *total)
        {
            __shared__ unsigned warp_sums[kListBlock / 32];
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
            unsigned v = flag;
            for (int o = 1; o < 32; o <<= 1)
            {
                const unsigned y = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o)
                    v += y;
            }
            if (lane == 31)
                warp_sums[warp] = v;
            __syncthreads();
            unsigned base = 0, all = 0;
            for (int w = 0; w < kListBlock / 32; ++w)
            {
                base += w < warp ? warp_sums[w] : 0u;
                all += warp_sums[w];
            }
            __syncthreads();
            *total = all;
            return base + v - flag;
        }

        __device__ unsigned long long block_sum(unsigned long long v)
        {
            __shared__ unsigned long long part[kListBlock / 32];
            for (int o = 16; o > 0; o >>= 1)
                v += __shfl_xor_sync(0xffffffffu, v, o);
            if ((threadIdx.x & 31) == 0)
                part[threadIdx.x >> 5] = v;
            __syncthreads();
            unsigned long long all = 0;
            for (int w = 0; w < kListBlock / 32; ++w)
                all += part[w];
            __syncthreads();
            return all;
        }

        // children's list sizes of each node (one block per node)
        __global__ void count_children(const unsigned long long *off, const uint32_t *items, const float *axis, long long N,
                                       int d, const NodeInfo *info, unsigned long long *sizes)
        {
            const long long t = blockIdx.x;
            const NodeInfo ni = info[t];
            unsigned long long n_lo = 0, n_hi = 0;
            for (unsigned long long i = off[t] + threadIdx.x; i < off[t + 1]; i += blockDim.x)
            {
                const float v = axis[items[i]];
                n_lo += v <= ni.up;
                n_hi += v >= ni.down;
            }
            n_lo = block_sum(n_lo);
            n_hi = block_sum(n_hi);
            if (threadIdx.x == 0)
            {
                const long long S = N >> d, begin = t * S;
                sizes[2 * t] = n_lo + static_cast<unsigned long long>(ni.l - (begin + S / 2));
                sizes[2 * t + 1] = n_hi + static_cast<unsigned long long>(ni.h - begin);
            }
        }

        // children's lists: the node's list filtered in order, then the scanned range
        __global__ void write_children(const unsigned long long *off, const uint32_t *items, const float *axis, long long N,
                                       int d, const NodeInfo *info, const uint32_t *ord, const unsigned long long *child_off,
                                       uint32_t *child_items)
        {
            const long long t = blockIdx.x;
            const NodeInfo ni = info[t];
            unsigned long long w_lo = child_off[2 * t], w_hi = child_off[2 * t + 1];
            const unsigned long long a0 = off[t], a1 = off[t + 1];
            for (unsigned long long c = a0; c < a1; c += blockDim.x)
            {
                const unsigned long long i = c + threadIdx.x;
                uint32_t it = 0;
                bool lo = false, hi = false;
                if (i < a1)
                {
                    it = items[i];
                    const float v = axis[it];
                    lo = v <= ni.up;
                    hi = v >= ni.down;
                }
                unsigned tot_lo, tot_hi;
                const unsigned p_lo = block_scan(lo ? 1u : 0u, &tot_lo);
                const unsigned p_hi = block_scan(hi ? 1u : 0u, &tot_hi);
                if (lo)
                    child_items[w_lo + p_lo] = it;
                if (hi)
                    child_items[w_hi + p_hi] = it;
                w_lo += tot_lo;
                w_hi += tot_hi;
            }
            const long long S = N >> d, begin = t * S, half = S / 2;
            for (long long i = begin + half + threadIdx.x; i < ni.l; i += blockDim.x)
                child_items[w_lo + (i - begin - half)] = ord[i];
            for (long long i = begin + threadIdx.x; i < ni.h; i += blockDim.x)
                child_items[w_hi + (i - begin)] = ord[i];
        }

        __device__ float cell_distsq(const float *c, float x, float y, float z)
        {
            const float p[3] = {x, y, z};
            float d[3];
            for (int k = 0; k < 3; ++k)
            {
                const float m = c[k] > p[k] ? c[k] : p[k];
                const float cl = c[3 + k] < m ? c[3 + k] : m;
                d[k] = __fsub_rn(p[k], cl);
            }
            return __fmaf_rn(d[2], d[2], __fmaf_rn(d[0], d[0], __fmul_rn(d[1], d[1])));
        }

        __device__ bool cell_inside_ball(const float *c, float x, float y, float z, float r2)
        {
            const float p[3] = {x, y, z};
            float d[3];
            for (int k = 0; k < 3; ++k)
            {
                const float a = __fsub_rn(p[k], c[k]), b = __fsub_rn(c[3 + k], p[k]);
                d[k] = a < b ? b : a;
            }
            return __fmaf_rn(d[2], d[2], __fmaf_rn(d[0], d[0], __fmul_rn(d[1], d[1]))) <= r2;
        }

        struct LeafParams
        {
            const unsigned long long *off;
            const uint32_t *items;
            const float *px, *py, *pz;
            const uint32_t *ord;
            const float *cell;
            float max_l2, min_l2;
        };

        // number of 8-point blocks of each leaf (one block of threads per leaf)
        __global__ void count_leaves(const LeafParams p, unsigned long long *blocks)
        {
            const long long t = blockIdx.x;
            const uint32_t rep = p.ord[t];
            const float rx = p.px[rep], ry = p.py[rep], rz = p.pz[rep];
            const float *c = p.cell + 6 * t;
            unsigned long long acc = 0;
            const bool finite = rx < kInf && rx > -kInf;
            if (finite && !cell_inside_ball(c, rx, ry, rz, p.min_l2))
            {
                for (unsigned long long i = p.off[t] + threadIdx.x; i < p.off[t + 1]; i += blockDim.x)
                {
                    const uint32_t it = p.items[i];
                    acc += cell_distsq(c, p.px[it], p.py[it], p.pz[it]) <= p.max_l2;
                }
            }
            acc = block_sum(acc);
            if (threadIdx.x == 0)
                blocks[t] = finite ? (acc + 1 + 7) / 8 : 0;
        }

        __device__ float block_min(float v)
        {
            __shared__ float part[kListBlock / 32];
            for (int o = 16; o > 0; o >>= 1)
                v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
            if ((threadIdx.x & 31) == 0)
                part[threadIdx.x >> 5] = v;
            __syncthreads();
            float all = part[0];
            for (int w = 1; w < kListBlock / 32; ++w)
                all = fminf(all, part[w]);
            __syncthreads();
            return all;
        }

        // each leaf's blocks (its representative, then its accepted points in list order, padded
        // with +inf) and its box
        __global__ void write_leaves(const LeafParams p, const unsigned long long *starts, float *aff, float *aabbs)
        {
            const long long t = blockIdx.x;
            const uint32_t rep = p.ord[t];
            const float rx = p.px[rep], ry = p.py[rep], rz = p.pz[rep];
            const float *c = p.cell + 6 * t;
            const bool finite = rx < kInf && rx > -kInf;
            float bmin[3] = {rx, ry, rz}, bmax[3] = {rx, ry, rz};
            if (finite)
            {
                const unsigned long long b0 = starts[t], nb = starts[t + 1] - b0;
                float *blk = aff + 24 * b0;
                auto put = [&](unsigned long long m, float x, float y, float z) {
                    float *b = blk + 24 * (m >> 3);
                    const unsigned l = static_cast<unsigned>(m & 7);
                    b[l] = x;
                    b[8 + l] = y;
                    b[16 + l] = z;
                };
                if (threadIdx.x == 0)
                    put(0, rx, ry, rz);
                unsigned long long w = 1;
                if (!cell_inside_ball(c, rx, ry, rz, p.min_l2))
                {
                    for (unsigned long long s = p.off[t]; s < p.off[t + 1]; s += blockDim.x)
                    {
                        const unsigned long long i = s + threadIdx.x;
                        bool ok = false;
                        float x = 0, y = 0, z = 0;
                        if (i < p.off[t + 1])
                        {
                            const uint32_t it = p.items[i];
                            x = p.px[it];
                            y = p.py[it];
                            z = p.pz[it];
                            ok = cell_distsq(c, x, y, z) <= p.max_l2;
                        }
                        unsigned tot;
                        const unsigned at = block_scan(ok ? 1u : 0u, &tot);
                        if (ok)
                        {
                            put(w + at, x, y, z);
                            bmin[0] = fminf(bmin[0], x);
                            bmin[1] = fminf(bmin[1], y);
                            bmin[2] = fminf(bmin[2], z);
                            bmax[0] = fmaxf(bmax[0], x);
                            bmax[1] = fmaxf(bmax[1], y);
                            bmax[2] = fmaxf(bmax[2], z);
                        }
                        w += tot;
                    }
                }
                for (unsigned long long m = w + threadIdx.x; m < 8 * nb; m += blockDim.x)
                    put(m, kInf, kInf, kInf);
                for (int k = 0; k < 3; ++k)
                {
                    bmin[k] = block_min(bmin[k]);
                    bmax[k] = -block_min(-bmax[k]);
                }
            }
            if (threadIdx.x == 0)
            {
                for (int k = 0; k < 3; ++k)
                {
                    aabbs[6 * t + k] = bmin[k];
                    aabbs[6 * t + 3 + k] = bmax[k];
                }
            }
        }

        // box of every finite representative (one block)
        __global__ void top_box(const uint32_t *ord, const float *px, const float *py, const float *pz, long long N,
                                float *top)
        {
            float mn[3] = {kInf, kInf, kInf}, mx[3] = {-kInf, -kInf, -kInf};
            for (long long t = threadIdx.x; t < N; t += blockDim.x)
            {
                const uint32_t r = ord[t];
                const float v[3] = {px[r], py[r], pz[r]};
                if (v[0] < kInf && v[0] > -kInf)
                {
                    for (int k = 0; k < 3; ++k)
                    {
                        mn[k] = fminf(mn[k], v[k]);
                        mx[k] = fmaxf(mx[k], v[k]);
                    }
                }
            }
            for (int k = 0; k < 3; ++k)
            {
                const float a = block_min(mn[k]), b = -block_min(-mx[k]);
                if (threadIdx.x == 0)
                {
                    top[k] = a;
                    top[3 + k] = b;
                }
            }
        }

        // exclusive scan of n values (one block), out[n] = total
        __global__ void scan_small(const unsigned long long *in, long long n, unsigned long long *out)
        {
            __shared__ unsigned long long carry;
            if (threadIdx.x == 0)
                carry = 0;
            __syncthreads();
            for (long long c = 0; c < n; c += blockDim.x)
            {
                const long long i = c + threadIdx.x;
                const unsigned long long v = i < n ? in[i] : 0;
                // inclusive scan within the block (warp shuffles, then warp totals)
                __shared__ unsigned long long wsum[32];
                unsigned long long x = v;
                const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
                for (int o = 1; o < 32; o <<= 1)
                {
                    const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
                    if (lane >= o)
                        x += y;
                }
                if (lane == 31)
                    wsum[warp] = x;
                __syncthreads();
                unsigned long long base = 0;
                for (int w = 0; w < warp; ++w)
                    base += wsum[w];
                if (i < n)
                    out[i] = carry + base + x - v;
                __syncthreads();
                if (threadIdx.x == blockDim.x - 1)
                    carry += base + x;
                __syncthreads();
            }
            if (threadIdx.x == 0)
                out[n] = carry;
        }

        __global__ void narrow_starts(const unsigned long long *in, long long n, uint32_t *out)
        {
            const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
            if (i < n)
                out[i] = static_cast<uint32_t>(in[i]);
        }

        template <typename T>
        cudaError_t grow(T **p, size_t *cap, size_t need)
        {
            if (need <= *cap)
                return cudaSuccess;
            if (*p)
                cudaFree(*p);
            *p = nullptr;
            *cap = 0;
            const cudaError_t e = cudaMalloc(p, std::max<size_t>(need, 1) * sizeof(T));
            if (e == cudaSuccess)
                *cap = need;
            return e;
        }

        unsigned grid_of(long long n, int block)
        {
            return static_cast<unsigned>((n + block - 1) / block);
        }
    }  // namespace

    int capt_build_device(const float *xyz, size_t n, float r_min, float r_max, float r_point, cudaStream_t s,
                          DeviceCapt &out)
    {
        if (n < 2)
            return set_error(VG_ERR_ARG, "CAPT build: need at least 2 points");
        int nlog2 = 0;
        while ((size_t{1} << nlog2) < n)
            ++nlog2;
        const long long N = 1ll << nlog2;
        out = DeviceCapt{};
        out.nlog2 = nlog2;
        out.r_min = r_min;
        out.r_max = r_max;
        out.r_point = r_point;
        float *px = nullptr, *py = nullptr, *pz = nullptr, *key = nullptr, *cell = nullptr, *child_cell = nullptr;
        uint32_t *ord = nullptr, *pos = nullptr, *items = nullptr, *child_items = nullptr;
        unsigned long long *off = nullptr, *child_off = nullptr, *sizes = nullptr;
        NodeInfo *info = nullptr;
        size_t items_cap = 0, child_cap = 0;
        cudaError_t e = cudaSuccess;
        // the fixed-size scratch in one allocation (carved in 256-byte aligned pieces)
        char *scratch = nullptr;
        {
            size_t used = 0;
            auto carve = [&](auto **p, size_t count) {
                const size_t at = used;
                used += (std::max<size_t>(count, 1) * sizeof(**p) + 255) & ~size_t(255);
                *p = scratch ? reinterpret_cast<std::remove_reference_t<decltype(*p)>>(scratch + at) : nullptr;
            };
            auto carve_all = [&]() {
                used = 0;
                carve(&px, N);
                carve(&py, N);
                carve(&pz, N);
                carve(&key, N);
                carve(&ord, N);
                carve(&pos, N);
                carve(&cell, 6 * N);
                carve(&child_cell, 6 * N);
                carve(&off, N + 1);
                carve(&child_off, N + 1);
                carve(&sizes, N);
                carve(&info, N / 2 > 0 ? N / 2 : 1);
            };
            carve_all();
            e = cudaMalloc(&scratch, used);
            if (e == cudaSuccess)
                carve_all();
        }
        auto alloc = [&](auto **p, size_t count) {
            if (e == cudaSuccess)
                e = cudaMalloc(p, std::max<size_t>(count, 1) * sizeof(**p));
        };
        alloc(&out.tests, N - 1);
        alloc(&out.aabbs, 6 * N);
        alloc(&out.starts_dev, N + 1);
        alloc(&out.top_dev, 6);
        const float *axis[3] = {px, py, pz};
        if (e == cudaSuccess)
        {
            init_points<<<grid_of(N, 256), 256, 0, s>>>(xyz, static_cast<long long>(n), N, px, py, pz, ord);
            const float root[6] = {-kInf, -kInf, -kInf, kInf, kInf, kInf};
            e = cudaMemcpyAsync(cell, root, sizeof(root), cudaMemcpyHostToDevice, s);
        }
        if (e == cudaSuccess)
            e = cudaMemsetAsync(off, 0, 2 * sizeof(unsigned long long), s);  // root: empty list
        for (int d = 0; d < nlog2 && e == cudaSuccess; ++d)
        {
            const long long nodes = 1ll << d, S = N >> d;
            load_keys<<<grid_of(N, 256), 256, 0, s>>>(ord, axis[d % 3], N, key, pos);
            // strides below the tile in shared memory, the longer ones one launch each
            const long long T = std::min<long long>(S, kSortTile);
            const unsigned tiles = static_cast<unsigned>(N / T), threads = static_cast<unsigned>(std::max<long long>(T / 2, 1));
            bitonic_tile<<<tiles, threads, 0, s>>>(key, pos, ord, S, 2, T);
            for (long long k = 2 * T; k <= S; k <<= 1)
            {
                for (long long j = k >> 1; j >= T; j >>= 1)
                    bitonic_stage<<<grid_of(N, 256), 256, 0, s>>>(key, pos, ord, N, k, j, S);
                bitonic_tile<<<tiles, threads, 0, s>>>(key, pos, ord, S, k, k);
            }
            split_nodes<<<grid_of(nodes, 128), 128, 0, s>>>(key, N, d, r_max, cell, out.tests, info, child_cell);
            count_children<<<static_cast<unsigned>(nodes), kListBlock, 0, s>>>(off, items, axis[d % 3], N, d, info, sizes);
            scan_small<<<1, 1024, 0, s>>>(sizes, 2 * nodes, child_off);
            unsigned long long total = 0;
            e = cudaMemcpyAsync(&total, child_off + 2 * nodes, sizeof(total), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(s);
            if (e == cudaSuccess)
                e = grow(&child_items, &child_cap, total);
            if (e != cudaSuccess)
                break;
            write_children<<<static_cast<unsigned>(nodes), kListBlock, 0, s>>>(off, items, axis[d % 3], N, d, info, ord,
                                                                                child_off, child_items);
            e = cudaGetLastError();
            std::swap(off, child_off);
            std::swap(items, child_items);
            std::swap(items_cap, child_cap);
            std::swap(cell, child_cell);
        }
        // leaves
        LeafParams lp{off, items, px, py, pz, ord, cell, 0.0f, 0.0f};
        {
            const float l1 = r_max + r_point, l0 = r_min + r_point;
            lp.max_l2 = l1 * l1;
            lp.min_l2 = l0 * l0;
        }
        if (e == cudaSuccess)
        {
            count_leaves<<<static_cast<unsigned>(N), kListBlock, 0, s>>>(lp, sizes);
            scan_small<<<1, 1024, 0, s>>>(sizes, N, out.starts_dev);
            unsigned long long total = 0;
            e = cudaMemcpyAsync(&total, out.starts_dev + N, sizeof(total), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(s);
            out.blocks = total;
            if (e == cudaSuccess)
                e = cudaMalloc(&out.aff, std::max<size_t>(24 * total, 4) * sizeof(float));
            if (e == cudaSuccess)
            {
                write_leaves<<<static_cast<unsigned>(N), kListBlock, 0, s>>>(lp, out.starts_dev, out.aff, out.aabbs);
                top_box<<<1, kListBlock, 0, s>>>(ord, px, py, pz, N, out.top_dev);
                e = cudaGetLastError();
            }
            if (e == cudaSuccess)
                e = cudaMalloc(&out.starts, (N + 1) * sizeof(uint32_t));
            if (e == cudaSuccess)
            {
                narrow_starts<<<grid_of(N + 1, 256), 256, 0, s>>>(out.starts_dev, N + 1, out.starts);
                e = cudaMemcpyAsync(out.top, out.top_dev, sizeof(out.top), cudaMemcpyDeviceToHost, s);
            }
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(s);
            if (out.starts_dev)
                cudaFree(out.starts_dev);
            if (out.top_dev)
                cudaFree(out.top_dev);
            out.starts_dev = nullptr;
            out.top_dev = nullptr;
        }
        for (void *p : {static_cast<void *>(scratch), static_cast<void *>(items), static_cast<void *>(child_items)})
        {
            if (p)
                cudaFree(p);
        }
        if (e != cudaSuccess)
        {
            out.release();
            return set_error(VG_ERR_CUDA, std::string("CAPT build on the GPU: ") + cudaGetErrorString(e));
        }
        return VG_OK;
    }

    void DeviceCapt::release()
    {
        for (void *p : {static_cast<void *>(tests), static_cast<void *>(aabbs), static_cast<void *>(starts_dev),
                        static_cast<void *>(aff), static_cast<void *>(top_dev), static_cast<void *>(starts)})
        {
            if (p)
                cudaFree(p);
        }
        tests = aabbs = aff = top_dev = nullptr;
        starts_dev = nullptr;
        starts = nullptr;
    }
}  // namespace vg
