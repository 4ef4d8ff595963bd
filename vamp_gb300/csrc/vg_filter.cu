// Pointcloud filter on the GPU: filter_pointcloud (collision/filter.hh:176-278), with the
// reference's results.
//
// The reference keeps a work list of point indices and, for each of six axis orders, sorts it by
// Morton code and drops every entry within min_dist of the last entry kept.  Here each pass is:
//   1. codes: one 64-bit key per entry, (Morton code << 32) | position, so that sorting the keys
//      is the stable sort by code; the coordinate range of the next pass is reduced on the side;
//   2. a sort of the keys: a stable radix sort on the code for long lists, a bitonic network
//      (shared-memory tiles of 2048 for the short strides) for short ones;
//   3. next[j]: the first entry after j that is farther than min_dist from entry j, found by a
//      forward scan that skips 32-, 1024- and 32768-entry tiles whose bounding box lies inside
//      the min_dist ball (tested in double with a margin, so a skipped entry is never "far");
//   4. the kept entries are the chain 0, next[0], next[next[0]], ...: per 1024-entry chunk,
//      pointer doubling gives the first chain element past the chunk from every entry; those
//      exits, composed over 16 chunks, let one thread walk the chain a superchunk at a time and
//      a thread per superchunk find its chunks' entry points; each chunk then marks its own
//      chain members (binary lifting over its doubling tables);
//   5. an ordered compaction of the kept entries gives the next pass's list.
// The reference's list has n entries, and those past the points that pass the cull hold index 0
// (filter.hh:199-216).  Those copies are identical (same point, same code, adjacent after the
// stable sort), and a run of identical entries keeps at most its first, so they are carried as a
// single entry placed after the passing points.
#include "../../include/vamp_gb300.h"
#include "vg_internal.h"

#include <algorithm>
#include <chrono>
#include <string>

namespace vg
{
    namespace
    {
        constexpr int kTile = 1024;      // entries per scan tile and per chain chunk
        constexpr int kSortTile = 2048;  // entries per shared-memory bitonic tile
        constexpr int kCodeBlock = 256;
        constexpr long long kRadixMin = 16384;  // lists longer than this are radix-sorted

        __device__ __forceinline__ float sqdist(float ax, float ay, float az, float bx, float by, float bz)
        {
            // collision/math.hh:29-42 (sql2_3) as the reference's x86-64 build contracts it
            const float dx = __fsub_rn(ax, bx), dy = __fsub_rn(ay, by), dz = __fsub_rn(az, bz);
            return __fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy)));
        }

        // remap_point (filter.hh:142-145); the float -> uint32_t conversion truncates and gives
        // 0xFFFFFFFF for NaN, values <= -1 and values >= 2^32, as the reference's x86-64 build does
        __device__ __forceinline__ uint32_t remap(float x, float lo, float hi)
        {
            const float v = __fmul_rn(__fdiv_rn(__fsub_rn(x, lo), __fsub_rn(hi, lo)), 1000.0f);
            if (!(v > -1.0f) || !(v < 4294967296.0f))
                return 0xFFFFFFFFu;
            return v <= 0.0f ? 0u : __float2uint_rz(v);
        }

        // the low `bits` bits of v to bits 0, 3, 6, ...
        __device__ __forceinline__ uint32_t spread3(uint32_t v, int bits)
        {
            uint32_t r = 0;
#pragma unroll
            for (int k = 0; k < 11; ++k)
                r |= k < bits ? ((v >> k) & 1u) << (3 * k) : 0u;
            return r;
        }

        // 32-bit Morton code (filter.hh:147-171): 11 bits of x, 11 of y, 10 of z
        __device__ __forceinline__ uint32_t morton(uint32_t x, uint32_t y, uint32_t z)
        {
            return spread3(x, 11) | (spread3(y, 11) << 1) | (spread3(z, 10) << 2);
        }

        // exclusive scan of one value per thread over a 1024-thread block; *total = block sum
        __device__ uint32_t block_scan(uint32_t v, uint32_t *total)
        {
            __shared__ uint32_t warp_sum[32];
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
            uint32_t x = v;
            for (int o = 1; o < 32; o <<= 1)
            {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o)
                    x += y;
            }
            if (lane == 31)
                warp_sum[warp] = x;
            __syncthreads();
            if (warp == 0)
            {
                uint32_t s = lane < (blockDim.x >> 5) ? warp_sum[lane] : 0u;
                for (int o = 1; o < 32; o <<= 1)
                {
                    const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
                    if (lane >= o)
                        s += y;
                }
                warp_sum[lane] = s;  // inclusive
            }
            __syncthreads();
            const uint32_t base = warp ? warp_sum[warp - 1] : 0u;
            *total = warp_sum[(blockDim.x >> 5) - 1];
            __syncthreads();
            return base + x - v;
        }

        // --- cull and ordered compaction ----------------------------------------------------

        struct CullParams
        {
            float ox, oy, oz, sq_range;
            float lo[3], hi[3];
            int cull;
        };

        __global__ void cull_kernel(const float *xyz, long long n, CullParams c, uint32_t *flags)
        {
            const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
            if (i >= n)
                return;
            const float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
            bool pass = true;
            if (c.cull)
                pass = sqdist(x, y, z, c.ox, c.oy, c.oz) < c.sq_range && c.lo[0] <= x && x <= c.hi[0] && c.lo[1] <= y &&
                       y <= c.hi[1] && c.lo[2] <= z && z <= c.hi[2];
            flags[i] = pass ? 1u : 0u;
        }

        __global__ void tile_sums(const uint32_t *flags, long long n, uint32_t *sums)
        {
            const long long i = static_cast<long long>(blockIdx.x) * kTile + threadIdx.x;
            uint32_t total;
            block_scan(i < n ? flags[i] : 0u, &total);
            if (threadIdx.x == 0)
                sums[blockIdx.x] = total;
        }

        // exclusive scan of n values in one block; out[n] = total
        __global__ void scan_tiles(const uint32_t *in, long long n, uint32_t *out)
        {
            __shared__ uint32_t carry;
            if (threadIdx.x == 0)
                carry = 0;
            __syncthreads();
            for (long long c = 0; c < n; c += kTile)
            {
                const long long i = c + threadIdx.x;
                uint32_t total;
                const uint32_t off = block_scan(i < n ? in[i] : 0u, &total);
                if (i < n)
                    out[i] = carry + off;
                __syncthreads();
                if (threadIdx.x == 0)
                    carry += total;
                __syncthreads();
            }
            if (threadIdx.x == 0)
                out[n] = carry;
        }

        // out[offset of j] = src ? src[j] : j, for every flagged j, in order
        __global__ void compact(const uint32_t *flags, long long n, const uint32_t *offs, const uint32_t *src,
                                uint32_t *out)
        {
            const long long i = static_cast<long long>(blockIdx.x) * kTile + threadIdx.x;
            const uint32_t f = i < n ? flags[i] : 0u;
            uint32_t total;
            const uint32_t at = block_scan(f, &total);
            if (f)
                out[offs[blockIdx.x] + at] = src ? src[i] : static_cast<uint32_t>(i);
        }

        // --- one pass ---------------------------------------------------------------------

        struct Range
        {
            float lo, hi;
        };

        __global__ void codes_kernel(const float *xyz, const uint32_t *list, long long m, long long M, int a0, int a1,
                                     int a2, const Range *range, unsigned long long *keys, float *part_lo, float *part_hi)
        {
            const long long j = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
            const float lo = range->lo, hi = range->hi;
            float mn = __int_as_float(0x7f800000), mx = -__int_as_float(0x7f800000);
            if (j < m)
            {
                const float *p = xyz + 3 * static_cast<size_t>(list[j]);
                const uint32_t code = morton(remap(p[a0], lo, hi), remap(p[a1], lo, hi), remap(p[a2], lo, hi));
                keys[j] = (static_cast<unsigned long long>(code) << 32) | static_cast<unsigned long long>(j);
                // std::min / std::max over the coordinates: a NaN never replaces the running value
                for (int k = 0; k < 3; ++k)
                {
                    mn = p[k] < mn ? p[k] : mn;
                    mx = mx < p[k] ? p[k] : mx;
                }
            }
            else if (j < M)
            {
                keys[j] = ~0ull;  // padding sorts last
            }
            __shared__ float s_lo[kCodeBlock / 32], s_hi[kCodeBlock / 32];
            for (int o = 16; o > 0; o >>= 1)
            {
                const float a = __shfl_xor_sync(0xffffffffu, mn, o), b = __shfl_xor_sync(0xffffffffu, mx, o);
                mn = a < mn ? a : mn;
                mx = mx < b ? b : mx;
            }
            if ((threadIdx.x & 31) == 0)
            {
                s_lo[threadIdx.x >> 5] = mn;
                s_hi[threadIdx.x >> 5] = mx;
            }
            __syncthreads();
            if (threadIdx.x == 0)
            {
                for (int w = 1; w < kCodeBlock / 32; ++w)
                {
                    mn = s_lo[w] < mn ? s_lo[w] : mn;
                    mx = mx < s_hi[w] ? s_hi[w] : mx;
                }
                part_lo[blockIdx.x] = mn;
                part_hi[blockIdx.x] = mx;
            }
        }

        // the next pass's range: halfway towards the pass's smallest and largest coordinate
        // (filter.hh:226-250,272-273); the running minimum starts at hi and the maximum at lo
        __global__ void range_kernel(const float *part_lo, const float *part_hi, long long nb, Range *range)
        {
            __shared__ float s_lo[32], s_hi[32];
            float mn = range->hi, mx = range->lo;
            for (long long b = threadIdx.x; b < nb; b += blockDim.x)
            {
                mn = part_lo[b] < mn ? part_lo[b] : mn;
                mx = mx < part_hi[b] ? part_hi[b] : mx;
            }
            for (int o = 16; o > 0; o >>= 1)
            {
                const float a = __shfl_xor_sync(0xffffffffu, mn, o), b = __shfl_xor_sync(0xffffffffu, mx, o);
                mn = a < mn ? a : mn;
                mx = mx < b ? b : mx;
            }
            if ((threadIdx.x & 31) == 0)
            {
                s_lo[threadIdx.x >> 5] = mn;
                s_hi[threadIdx.x >> 5] = mx;
            }
            __syncthreads();
            if (threadIdx.x == 0)
            {
                for (unsigned w = 1; w < (blockDim.x >> 5); ++w)
                {
                    mn = s_lo[w] < mn ? s_lo[w] : mn;
                    mx = mx < s_hi[w] ? s_hi[w] : mx;
                }
                const Range old = *range;
                range->hi = __fmul_rn(__fadd_rn(mx, old.hi), 0.5f);
                range->lo = __fmul_rn(__fadd_rn(mn, old.lo), 0.5f);
            }
        }

        // bitonic compare-exchange of keys[i] and keys[i + j] in ascending (up) or descending order
        __device__ __forceinline__ void cmp_swap(unsigned long long &a, unsigned long long &b, bool up)
        {
            if ((a > b) == up)
            {
                const unsigned long long t = a;
                a = b;
                b = t;
            }
        }

        // all merge steps of stride < T for sizes k in [k0, k1], on tiles of T = min(M, 2048) keys
        __global__ void bitonic_tile(unsigned long long *keys, long long M, long long k0, long long k1)
        {
            __shared__ unsigned long long s[kSortTile];
            const long long T = M < kSortTile ? M : kSortTile;
            const long long base = static_cast<long long>(blockIdx.x) * T;
            for (long long t = threadIdx.x; t < T; t += blockDim.x)
                s[t] = keys[base + t];
            __syncthreads();
            for (long long k = k0; k <= k1; k <<= 1)
            {
                for (long long j = (k >> 1) < (T >> 1) ? (k >> 1) : (T >> 1); j > 0; j >>= 1)
                {
                    for (long long t = threadIdx.x; t < (T >> 1); t += blockDim.x)
                    {
                        const long long i = 2 * t - (t & (j - 1));  // lower element of the t-th pair
                        cmp_swap(s[i], s[i + j], ((base + i) & k) == 0);
                    }
                    __syncthreads();
                }
            }
            for (long long t = threadIdx.x; t < T; t += blockDim.x)
                keys[base + t] = s[t];
        }

        // one merge step of stride j >= 2048
        __global__ void bitonic_step(unsigned long long *keys, long long M, long long k, long long j)
        {
            const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
            if (t >= (M >> 1))
                return;
            const long long i = 2 * t - (t & (j - 1));
            cmp_swap(keys[i], keys[i + j], (i & k) == 0);
        }

        // --- stable LSD radix sort of the keys by their upper 32 bits (the Morton code) ----------
        //
        // Four passes of 8 bits.  Per pass: per-tile digit counts, an exclusive scan over (digit,
        // tile), and a stable scatter: an entry's rank among the equal digits of its tile is its
        // rank in its warp (match + popcount) plus the counts of the earlier warps.  The keys
        // enter in position order, so the result is the (code, position) order.

        constexpr int kRadixTile = 1024;

        __global__ void radix_count(const unsigned long long *keys, long long m, int shift, uint32_t *counts, long long tiles)
        {
            __shared__ uint32_t h[256];
            for (int d = threadIdx.x; d < 256; d += blockDim.x)
                h[d] = 0u;
            __syncthreads();
            const long long i = static_cast<long long>(blockIdx.x) * kRadixTile + threadIdx.x;
            if (i < m)
                atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
            __syncthreads();
            for (int d = threadIdx.x; d < 256; d += blockDim.x)
                counts[static_cast<long long>(d) * tiles + blockIdx.x] = h[d];
        }

        // out[i] = chunk_offs[chunk] + exclusive scan of values within its 1024-value chunk
        __global__ void scan_apply(const uint32_t *values, long long n, const uint32_t *chunk_offs, uint32_t *out)
        {
            const long long i = static_cast<long long>(blockIdx.x) * kTile + threadIdx.x;
            uint32_t total;
            const uint32_t at = block_scan(i < n ? values[i] : 0u, &total);
            if (i < n)
                out[i] = chunk_offs[blockIdx.x] + at;
        }

        __global__ void radix_scatter(const unsigned long long *in, long long m, int shift, const uint32_t *offs, long long tiles,
                                      unsigned long long *out)
        {
            __shared__ uint32_t wc[kRadixTile / 32][256];
            const int t = threadIdx.x, w = t >> 5, lane = t & 31;
            for (int k = t; k < (kRadixTile / 32) * 256; k += blockDim.x)
                (&wc[0][0])[k] = 0u;
            __syncthreads();
            const long long i = static_cast<long long>(blockIdx.x) * kRadixTile + t;
            const bool valid = i < m;
            const unsigned long long key = valid ? in[i] : 0ull;
            const unsigned d = valid ? static_cast<unsigned>((key >> shift) & 255u) : 256u;
            const unsigned peers = __match_any_sync(kFull, d);
            const unsigned rank = __popc(peers & ((1u << lane) - 1u));
            if (valid && rank == 0)
                wc[w][d] = __popc(peers);
            __syncthreads();
            if (valid)
            {
                uint32_t base = 0;
                for (int k = 0; k < w; ++k)
                    base += wc[k][d];
                out[offs[static_cast<long long>(d) * tiles + blockIdx.x] + base + rank] = key;
            }
        }

        // the sorted entries' point indices and coordinates
        __global__ void gather_sorted(const unsigned long long *keys, const uint32_t *list, long long m, const float *xyz,
                                      uint32_t *sidx, float4 *sp)
        {
            const long long j = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
            if (j >= m)
                return;
            const uint32_t idx = list[static_cast<uint32_t>(keys[j])];
            sidx[j] = idx;
            const float *p = xyz + 3 * static_cast<size_t>(idx);
            sp[j] = make_float4(p[0], p[1], p[2], 0.0f);
        }

        struct Box
        {
            float lo[3], hi[3];
        };

        // bounding box of every 32 consecutive entries (one warp per tile; NaN coordinates are
        // left out, which is safe: a NaN entry is never farther than min_dist)
        __global__ void boxes_of_points(const float4 *sp, long long m, long long tiles, Box *out)
        {
            const long long w = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
            const int lane = threadIdx.x & 31;
            if (w >= tiles)
                return;
            const long long j = 32 * w + lane;
            const float inf = __int_as_float(0x7f800000);
            float lo[3] = {inf, inf, inf}, hi[3] = {-inf, -inf, -inf};
            if (j < m)
            {
                const float4 p = sp[j];
                lo[0] = hi[0] = p.x;
                lo[1] = hi[1] = p.y;
                lo[2] = hi[2] = p.z;
            }
            for (int k = 0; k < 3; ++k)
            {
                for (int o = 16; o > 0; o >>= 1)
                {
                    lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
                    hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
                }
            }
            if (lane == 0)
            {
                Box b;
                for (int k = 0; k < 3; ++k)
                {
                    b.lo[k] = lo[k];
                    b.hi[k] = hi[k];
                }
                out[w] = b;
            }
        }

        // bounding box of every 32 consecutive boxes
        __global__ void boxes_of_boxes(const Box *in, long long n_in, long long tiles, Box *out)
        {
            const long long w = (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
            const int lane = threadIdx.x & 31;
            if (w >= tiles)
                return;
            const long long j = 32 * w + lane;
            const float inf = __int_as_float(0x7f800000);
            float lo[3] = {inf, inf, inf}, hi[3] = {-inf, -inf, -inf};
            if (j < n_in)
            {
                const Box b = in[j];
                for (int k = 0; k < 3; ++k)
                {
                    lo[k] = b.lo[k];
                    hi[k] = b.hi[k];
                }
            }
            for (int k = 0; k < 3; ++k)
            {
                for (int o = 16; o > 0; o >>= 1)
                {
                    lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
                    hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
                }
            }
            if (lane == 0)
            {
                Box b;
                for (int k = 0; k < 3; ++k)
                {
                    b.lo[k] = lo[k];
                    b.hi[k] = hi[k];
                }
                out[w] = b;
            }
        }

        // every point of the box is within min_dist of p, with a margin that covers the FP32
        // rounding of the reference's distance (a few ulps) and subnormal results
        __device__ __forceinline__ bool box_inside(const Box &b, float px, float py, float pz, double limit)
        {
            const float p[3] = {px, py, pz};
            double d2 = 0.0;
            for (int k = 0; k < 3; ++k)
            {
                const double a = fabs(static_cast<double>(b.lo[k]) - p[k]), c = fabs(static_cast<double>(b.hi[k]) - p[k]);
                const double e = a > c ? a : c;
                d2 += e * e;
            }
            return d2 <= limit;  // false for NaN and for empty (infinite) boxes
        }

        struct NextParams
        {
            const float4 *sp;
            long long m;
            float sq;
            double limit;  // box test threshold (negative: never skip)
            const Box *b32, *b1k, *b32k;
            uint32_t *next;
        };

        // next[j]: first k > j with distance(entry k, entry j) > min_dist, or m
        __global__ void next_kernel(const NextParams p)
        {
            const long long j = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
            if (j >= p.m)
                return;
            const float4 q = p.sp[j];
            long long k = j + 1;
            while (k < p.m)
            {
                if ((k & 32767) == 0 && k + 32768 <= p.m && box_inside(p.b32k[k >> 15], q.x, q.y, q.z, p.limit))
                {
                    k += 32768;
                    continue;
                }
                if ((k & 1023) == 0 && k + 1024 <= p.m && box_inside(p.b1k[k >> 10], q.x, q.y, q.z, p.limit))
                {
                    k += 1024;
                    continue;
                }
                if ((k & 31) == 0 && k + 32 <= p.m && box_inside(p.b32[k >> 5], q.x, q.y, q.z, p.limit))
                {
                    k += 32;
                    continue;
                }
                const float4 r = p.sp[k];
                if (sqdist(r.x, r.y, r.z, q.x, q.y, q.z) > p.sq)
                    break;
                ++k;
            }
            p.next[j] = static_cast<uint32_t>(k);
        }

        // exit[j]: the first chain element at or past the end of j's chunk, from j (pointer
        // doubling over the chunk: after 10 rounds every chain has left it)
        __global__ void chunk_exit(const uint32_t *next, long long m, uint32_t *exit_of)
        {
            __shared__ uint32_t a[kTile], b[kTile];
            const long long c0 = static_cast<long long>(blockIdx.x) * kTile;
            const long long c1 = c0 + kTile < m ? c0 + kTile : m;
            const int t = threadIdx.x;
            a[t] = c0 + t < c1 ? next[c0 + t] : static_cast<uint32_t>(c1);
            __syncthreads();
            uint32_t *src = a, *dst = b;
            for (int r = 0; r < 10; ++r)
            {
                const uint32_t v = src[t];
                dst[t] = v < c1 && v > c0 ? src[v - c0] : v;  // next[j] > j: v > c0 inside the chunk
                __syncthreads();
                uint32_t *tmp = src;
                src = dst;
                dst = tmp;
            }
            if (c0 + t < c1)
                exit_of[c0 + t] = src[t];
        }

        constexpr int kSuper = 16;  // chunks per superchunk of the chain walk

        // exit_super[e]: the first chain element past the superchunk of e (kSuper chunks), from e:
        // at most kSuper hops, each leaving a chunk
        __global__ void super_exit(const uint32_t *exit_of, long long m, uint32_t *exit_super, uint32_t *err)
        {
            const long long e = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
            if (e >= m)
                return;
            const long long end = (e / (kTile * kSuper) + 1) * (kTile * kSuper);
            long long x = e;
            for (int h = 0; h < kSuper + 1 && x < end && x < m; ++h)
            {
                const long long y = exit_of[x];
                if (y < (x / kTile + 1) * kTile && y < m)
                {
                    *err = 1u;  // not reached: every exit leaves its chunk
                    return;
                }
                x = y;
            }
            exit_super[e] = static_cast<uint32_t>(x < m ? x : m);
        }

        // the chain's entry point into each superchunk it visits (one thread, one step per
        // superchunk; superchunks it skips keep 0xFFFFFFFF)
        __global__ void chain_walk(const uint32_t *exit_super, long long m, uint32_t *entry_super, uint32_t *err)
        {
            long long e = 0;
            while (e < m)
            {
                entry_super[e / (kTile * kSuper)] = static_cast<uint32_t>(e);
                const long long x = exit_super[e];
                if (x < (e / (kTile * kSuper) + 1) * (kTile * kSuper) && x < m)
                {
                    *err = 1u;  // not reached: every exit leaves its superchunk
                    return;
                }
                e = x;
            }
        }

        // the chain's entry point into each chunk of one superchunk (a thread per superchunk)
        __global__ void chunk_entries(const uint32_t *exit_of, long long m, const uint32_t *entry_super,
                                      long long supers, uint32_t *entry)
        {
            const long long sc = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
            if (sc >= supers || entry_super[sc] == 0xFFFFFFFFu)
                return;
            const long long end = (sc + 1) * (kTile * kSuper);
            long long x = entry_super[sc];
            for (int h = 0; h < kSuper && x < end && x < m; ++h)
            {
                entry[x / kTile] = static_cast<uint32_t>(x);
                x = exit_of[x];  // leaves x's chunk (checked by super_exit)
            }
        }

        // kept flags of each chunk: its chain members from the entry point.  Each thread lifts
        // from the entry with the doubling tables J_k = next^(2^k) (restricted to the chunk):
        // the last chain element at or before its own index is itself exactly when it is kept.
        __global__ void mark_kept(const uint32_t *next, long long m, const uint32_t *entry, uint32_t *kept, uint32_t *err)
        {
            __shared__ uint32_t J[10][kTile];
            const long long c0 = static_cast<long long>(blockIdx.x) * kTile;
            const long long c1 = c0 + kTile < m ? c0 + kTile : m;
            const int t = threadIdx.x;
            const uint32_t e0 = entry[blockIdx.x];
            if (e0 == 0xFFFFFFFFu)
            {
                if (c0 + t < c1)
                    kept[c0 + t] = 0u;
                return;  // uniform: the chain skips this chunk
            }
            J[0][t] = c0 + t < c1 ? next[c0 + t] : static_cast<uint32_t>(c1);
            __syncthreads();
            for (int k = 1; k < 10; ++k)
            {
                const uint32_t v = J[k - 1][t];
                J[k][t] = v < c1 && v > c0 ? J[k - 1][v - c0] : v;
                __syncthreads();
            }
            if (c0 + t < c1)
            {
                uint32_t mine = 0u;
                const uint32_t me = static_cast<uint32_t>(c0 + t);
                if (e0 < c0 || e0 >= c1)
                {
                    *err = 2u;  // not reached: the walk records entries inside their chunk
                }
                else if (e0 <= me)
                {
                    uint32_t cur = e0;
                    for (int k = 9; k >= 0; --k)
                    {
                        const uint32_t v = J[k][cur - c0];
                        if (v <= me)
                            cur = v;
                    }
                    mine = cur == me ? 1u : 0u;
                }
                kept[c0 + t] = mine;
            }
        }

        __global__ void gather_points(const float *xyz, const uint32_t *list, long long m, float *out)
        {
            const long long j = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
            if (j >= m)
                return;
            const float *p = xyz + 3 * static_cast<size_t>(list[j]);
            out[3 * j] = p[0];
            out[3 * j + 1] = p[1];
            out[3 * j + 2] = p[2];
        }

        unsigned blocks_of(long long n, long long per)
        {
            return static_cast<unsigned>((n + per - 1) / per);
        }

        // device buffers of one filter call
        // device buffers of one filter call, carved out of one allocation: a first round of get()
        // calls measures, allocate() reserves the total, a second round hands out the pointers
        struct FilterBuffers
        {
            char *base = nullptr;
            size_t used = 0;
            bool measuring = true;
            cudaError_t err = cudaSuccess;

            template <typename T>
            T *get(size_t count)
            {
                const size_t bytes = (std::max<size_t>(count, 1) * sizeof(T) + 255) & ~size_t(255);
                const size_t at = used;
                used += bytes;
                return measuring ? nullptr : reinterpret_cast<T *>(base + at);
            }

            void allocate()
            {
                err = cudaMalloc(&base, used);
                used = 0;
                measuring = false;
            }

            ~FilterBuffers()
            {
                if (base)
                    cudaFree(base);
            }
        };

        int filter_on_device(const float *xyz, size_t n, float min_dist, float max_range, const float *origin,
                             const float *workcell_min, const float *workcell_max, int cull, float *out, size_t *n_out,
                             cudaStream_t s)
        {
            const long long N = static_cast<long long>(n);
            long long M = 1;
            while (M < N + 1)
                M <<= 1;
            const long long tiles = blocks_of(N + 1, kTile);
            FilterBuffers fb;
            uint32_t *flags, *list, *list2, *sums, *offs, *sidx, *next, *exit_of, *entry, *exit_super, *entry_super;
            uint32_t *rcount, *rstart, *rsums, *roffs, *err;
            unsigned long long *keys, *keys2;
            float4 *sp;
            Box *b32, *b1k, *b32k;
            float *part_lo, *part_hi;
            Range *range;
            const long long rtiles = blocks_of(N + 1, kRadixTile), rchunks = blocks_of(256 * rtiles, kTile);
            const long long code_blocks = blocks_of(M, kCodeBlock);
            auto carve = [&]() {
                flags = fb.get<uint32_t>(N + 1);
                list = fb.get<uint32_t>(N + 1);
                list2 = fb.get<uint32_t>(N + 1);
                sums = fb.get<uint32_t>(tiles);
                offs = fb.get<uint32_t>(tiles + 1);
                sidx = fb.get<uint32_t>(N + 1);
                next = fb.get<uint32_t>(N + 1);
                exit_of = fb.get<uint32_t>(N + 1);
                entry = fb.get<uint32_t>(tiles);
                exit_super = fb.get<uint32_t>(N + 1);
                entry_super = fb.get<uint32_t>(blocks_of(tiles, kSuper));
                keys = fb.get<unsigned long long>(M);
                keys2 = fb.get<unsigned long long>(N + 1);
                rcount = fb.get<uint32_t>(256 * rtiles);
                rstart = fb.get<uint32_t>(256 * rtiles);
                rsums = fb.get<uint32_t>(rchunks);
                roffs = fb.get<uint32_t>(rchunks + 1);
                sp = fb.get<float4>(N + 1);
                b32 = fb.get<Box>(blocks_of(N + 1, 32));
                b1k = fb.get<Box>(blocks_of(N + 1, 1024));
                b32k = fb.get<Box>(blocks_of(N + 1, 32768));
                part_lo = fb.get<float>(code_blocks);
                part_hi = fb.get<float>(code_blocks);
                range = fb.get<Range>(1);
                err = fb.get<uint32_t>(1);
            };
            carve();
            fb.allocate();
            if (fb.err != cudaSuccess)
                return cuda_fail(fb.err, "vg_filter_pointcloud: cudaMalloc");
            carve();

            const float sq = min_dist * min_dist, sq_range = max_range * max_range;
            // collision/filter.hh:194-197: both ends are minima over the axes
            Range r0;
            r0.lo = std::min({origin[0] - max_range, origin[1] - max_range, origin[2] - max_range});
            r0.hi = std::min({origin[0] + max_range, origin[1] + max_range, origin[2] + max_range});
            VG_CUDA(cudaMemcpyAsync(range, &r0, sizeof(r0), cudaMemcpyHostToDevice, s), "vg_filter_pointcloud: copy");
            VG_CUDA(cudaMemsetAsync(err, 0, sizeof(uint32_t), s), "vg_filter_pointcloud: memset");

            // the work list: the passing points in order, then one copy of point 0 if any failed
            CullParams cp{origin[0], origin[1], origin[2], sq_range, {}, {}, cull};
            for (int k = 0; k < 3; ++k)
            {
                cp.lo[k] = workcell_min[k];
                cp.hi[k] = workcell_max[k];
            }
            const long long in_tiles = blocks_of(N, kTile);
            cull_kernel<<<blocks_of(N, 256), 256, 0, s>>>(xyz, N, cp, flags);
            tile_sums<<<static_cast<unsigned>(in_tiles), kTile, 0, s>>>(flags, N, sums);
            scan_tiles<<<1, kTile, 0, s>>>(sums, in_tiles, offs);
            compact<<<static_cast<unsigned>(in_tiles), kTile, 0, s>>>(flags, N, offs, nullptr, list);
            uint32_t h = 0;
            VG_CUDA(cudaMemcpyAsync(&h, offs + in_tiles, sizeof(h), cudaMemcpyDeviceToHost, s), "vg_filter_pointcloud: copy");
            VG_CUDA(cudaStreamSynchronize(s), "vg_filter_pointcloud");
            long long m = h;
            if (static_cast<long long>(h) < N)
            {
                const uint32_t zero = 0;
                VG_CUDA(cudaMemcpyAsync(list + h, &zero, sizeof(zero), cudaMemcpyHostToDevice, s), "vg_filter_pointcloud: copy");
                m = h + 1;
            }

            // collision/filter.hh:218: std::next_permutation order from (0, 1, 2)
            static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
            // box test threshold: sq / (1 + 1e-5) less an absolute 1e-38
            const double limit = static_cast<double>(sq) / (1.0 + 1e-5) - 1e-38;
            for (int pass = 0; pass < 6; ++pass)
            {
                long long Mp = 1;
                while (Mp < m)
                    Mp <<= 1;
                const long long cb = blocks_of(Mp, kCodeBlock);
                codes_kernel<<<static_cast<unsigned>(cb), kCodeBlock, 0, s>>>(xyz, list, m, Mp, perms[pass][0], perms[pass][1],
                                                                             perms[pass][2], range, keys, part_lo, part_hi);
                range_kernel<<<1, 1024, 0, s>>>(part_lo, part_hi, cb, range);
                if (m > kRadixMin)
                {
                    // large lists: the radix sort (digit counts, their scan, stable scatters)
                    const long long rt = blocks_of(m, kRadixTile), nc = 256 * rt, cchunks = blocks_of(nc, kTile);
                    unsigned long long *src = keys, *dst = keys2;
                    for (int shift = 32; shift < 64; shift += 8)
                    {
                        radix_count<<<static_cast<unsigned>(rt), kRadixTile, 0, s>>>(src, m, shift, rcount, rt);
                        tile_sums<<<static_cast<unsigned>(cchunks), kTile, 0, s>>>(rcount, nc, rsums);
                        scan_tiles<<<1, kTile, 0, s>>>(rsums, cchunks, roffs);
                        scan_apply<<<static_cast<unsigned>(cchunks), kTile, 0, s>>>(rcount, nc, roffs, rstart);
                        radix_scatter<<<static_cast<unsigned>(rt), kRadixTile, 0, s>>>(src, m, shift, rstart, rt, dst);
                        std::swap(src, dst);
                    }
                    // four passes: the result is back in keys
                }
                else if (Mp > 1)
                {
                    const long long T = std::min<long long>(Mp, kSortTile);
                    const unsigned tb = static_cast<unsigned>(Mp / T), tt = static_cast<unsigned>(T / 2);
                    bitonic_tile<<<tb, tt, 0, s>>>(keys, Mp, 2, T);
                    for (long long k = 2 * T; k <= Mp; k <<= 1)
                    {
                        for (long long j = k >> 1; j >= T; j >>= 1)
                            bitonic_step<<<blocks_of(Mp / 2, 256), 256, 0, s>>>(keys, Mp, k, j);
                        bitonic_tile<<<tb, tt, 0, s>>>(keys, Mp, k, k);
                    }
                }
                gather_sorted<<<blocks_of(m, 256), 256, 0, s>>>(keys, list, m, xyz, sidx, sp);
                const long long t32 = blocks_of(m, 32), t1k = blocks_of(t32, 32), t32k = blocks_of(t1k, 32);
                boxes_of_points<<<blocks_of(32 * t32, 256), 256, 0, s>>>(sp, m, t32, b32);
                boxes_of_boxes<<<blocks_of(32 * t1k, 256), 256, 0, s>>>(b32, t32, t1k, b1k);
                boxes_of_boxes<<<blocks_of(32 * t32k, 256), 256, 0, s>>>(b1k, t1k, t32k, b32k);
                next_kernel<<<blocks_of(m, 128), 128, 0, s>>>(NextParams{sp, m, sq, limit, b32, b1k, b32k, next});
                const long long chunks = blocks_of(m, kTile);
                chunk_exit<<<static_cast<unsigned>(chunks), kTile, 0, s>>>(next, m, exit_of);
                const long long supers = blocks_of(chunks, kSuper);
                VG_CUDA(cudaMemsetAsync(entry, 0xFF, chunks * sizeof(uint32_t), s), "vg_filter_pointcloud: memset");
                VG_CUDA(cudaMemsetAsync(entry_super, 0xFF, supers * sizeof(uint32_t), s), "vg_filter_pointcloud: memset");
                super_exit<<<blocks_of(m, 256), 256, 0, s>>>(exit_of, m, exit_super, err);
                chain_walk<<<1, 1, 0, s>>>(exit_super, m, entry_super, err);
                chunk_entries<<<blocks_of(supers, 128), 128, 0, s>>>(exit_of, m, entry_super, supers, entry);
                mark_kept<<<static_cast<unsigned>(chunks), kTile, 0, s>>>(next, m, entry, flags, err);
                tile_sums<<<static_cast<unsigned>(chunks), kTile, 0, s>>>(flags, m, sums);
                scan_tiles<<<1, kTile, 0, s>>>(sums, chunks, offs);
                compact<<<static_cast<unsigned>(chunks), kTile, 0, s>>>(flags, m, offs, sidx, list2);
                std::swap(list, list2);
                VG_CUDA(cudaGetLastError(), "vg_filter_pointcloud: launch");
                uint32_t kept[2] = {0, 0};
                VG_CUDA(cudaMemcpyAsync(&kept[0], offs + chunks, sizeof(uint32_t), cudaMemcpyDeviceToHost, s),
                        "vg_filter_pointcloud: copy");
                VG_CUDA(cudaMemcpyAsync(&kept[1], err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s),
                        "vg_filter_pointcloud: copy");
                VG_CUDA(cudaStreamSynchronize(s), "vg_filter_pointcloud");
                if (kept[1] || kept[0] == 0 || kept[0] > m)
                    return set_error(VG_ERR_STATE, "vg_filter_pointcloud: inconsistent chain (code " +
                                                       std::to_string(kept[1]) + ")");
                m = kept[0];
            }
            gather_points<<<blocks_of(m, 256), 256, 0, s>>>(xyz, list, m, out);
            VG_CUDA(cudaGetLastError(), "vg_filter_pointcloud: launch");
            VG_CUDA(cudaStreamSynchronize(s), "vg_filter_pointcloud");
            *n_out = static_cast<size_t>(m);
            return VG_OK;
        }

        // filter_self_from_pointcloud (bindings/robot_helper.hh:307-345): flags[i] = point i (a
        // sphere of `radius`) collides with no fine sphere of the robot and no environment object.
        // A warp-uniform loop: the environment query takes votes over the whole warp.
        __global__ void filter_self_kernel(const float *xyz, long long n, float radius, const float *spheres, int fine,
                                           EnvDevice env, uint32_t *flags)
        {
            extern __shared__ float4 smem[];
            const EnvView ev = stage_env(env, smem);
            const int lane = threadIdx.x & 31;
            const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
            for (long long b = static_cast<long long>(blockIdx.x) * blockDim.x + (threadIdx.x & ~31); b < n; b += stride)
            {
                const long long i = b + lane;
                const bool in = i < n;
                const float x = in ? xyz[3 * i] : 0.0f, y = in ? xyz[3 * i + 1] : 0.0f, z = in ? xyz[3 * i + 2] : 0.0f;
                bool valid = in;
                for (int k = 0; k < fine; ++k)
                {
                    // sphere_sphere_sql2(robot sphere, point) < 0, scalar
                    const float dx = __fsub_rn(__ldg(spheres + 4 * k), x), dy = __fsub_rn(__ldg(spheres + 4 * k + 1), y);
                    const float dz = __fsub_rn(__ldg(spheres + 4 * k + 2), z), rs = __fadd_rn(__ldg(spheres + 4 * k + 3), radius);
                    valid &= !(__fsub_rn(__fmaf_rn(dz, dz, __fmaf_rn(dx, dx, __fmul_rn(dy, dy))), __fmul_rn(rs, rs)) < 0.0f);
                }
                const unsigned hit = env_query<1>(ev, x, y, z, radius, __ballot_sync(kFull, valid));
                if (in)
                    flags[i] = valid && !((hit >> lane) & 1u) ? 1u : 0u;
            }
        }

        int check_filter_args(const float *xyz, size_t n, const float *origin, const float *wmin, const float *wmax,
                              const float *out, const size_t *n_out)
        {
            if (!n_out || !origin || !wmin || !wmax || (n && (!xyz || !out)))
                return set_error(VG_ERR_ARG, "vg_filter_pointcloud: null argument");
            if (n > (size_t{1} << 30))
                return set_error(VG_ERR_LIMIT, "vg_filter_pointcloud: at most 2^30 points");
            return VG_OK;
        }
    }  // namespace
}  // namespace vg

using namespace vg;

extern "C" {

int vg_filter_pointcloud_device(const float *xyz, size_t n, float min_dist, float max_range, const float *origin,
                                const float *workcell_min, const float *workcell_max, int cull, float *out, size_t *n_out,
                                void *stream)
{
    if (int rc = check_filter_args(xyz, n, origin, workcell_min, workcell_max, out, n_out))
        return rc;
    *n_out = 0;
    if (n == 0)
        return VG_OK;
    return filter_on_device(xyz, n, min_dist, max_range, origin, workcell_min, workcell_max, cull, out, n_out,
                            static_cast<cudaStream_t>(stream));
}

int vg_filter_self_from_pointcloud_device(const char *robot, vg_env *env, const float *xyz, size_t n, float point_radius,
                                          const float *q, float *out, size_t *n_out, void *stream)
{
    const RobotOps *r = find_robot(robot);
    if (!r || !env || !q || !n_out || (n && (!xyz || !out)))
        return set_error(VG_ERR_ARG, "vg_filter_self_from_pointcloud: bad argument");
    if (n > (size_t{1} << 31) - 1)
        return set_error(VG_ERR_LIMIT, "vg_filter_self_from_pointcloud: at most 2^31 - 1 points");
    *n_out = 0;
    if (n == 0)
        return VG_OK;
    if (int rc = commit(env))
        return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const long long N = static_cast<long long>(n), tiles = blocks_of(N, kTile);
    FilterBuffers fb;
    float *dq, *sph;
    uint32_t *flags, *sums, *offs, *idx;
    auto carve = [&]() {
        dq = fb.get<float>(r->dim);
        sph = fb.get<float>(4 * r->slots);
        flags = fb.get<uint32_t>(N);
        sums = fb.get<uint32_t>(tiles);
        offs = fb.get<uint32_t>(tiles + 1);
        idx = fb.get<uint32_t>(N);
    };
    carve();
    fb.allocate();
    if (fb.err != cudaSuccess)
        return cuda_fail(fb.err, "vg_filter_self_from_pointcloud: cudaMalloc");
    carve();
    VG_CUDA(cudaMemcpyAsync(dq, q, r->dim * sizeof(float), cudaMemcpyHostToDevice, s), "vg_filter_self_from_pointcloud: copy");
    VG_CUDA(r->spheres(dq, 1, sph, s), "vg_filter_self_from_pointcloud: sphere_fk");
    const int smem = static_cast<int>(staged_f4(static_cast<int>(env->image_f4)) * sizeof(float4));
    int occ = 0;
    if (int rc = prepare_kernel(reinterpret_cast<const void *>(&filter_self_kernel), smem, 256, &occ))
        return rc;
    const int grid = static_cast<int>(std::min<long long>(blocks_of(N, 256), static_cast<long long>(sm_count()) * occ));
    filter_self_kernel<<<grid, 256, smem, s>>>(xyz, N, point_radius, sph, r->fine, env_device(env), flags);
    tile_sums<<<static_cast<unsigned>(tiles), kTile, 0, s>>>(flags, N, sums);
    scan_tiles<<<1, kTile, 0, s>>>(sums, tiles, offs);
    compact<<<static_cast<unsigned>(tiles), kTile, 0, s>>>(flags, N, offs, nullptr, idx);
    VG_CUDA(cudaGetLastError(), "vg_filter_self_from_pointcloud: launch");
    uint32_t m = 0;
    VG_CUDA(cudaMemcpyAsync(&m, offs + tiles, sizeof(m), cudaMemcpyDeviceToHost, s), "vg_filter_self_from_pointcloud: copy");
    VG_CUDA(cudaStreamSynchronize(s), "vg_filter_self_from_pointcloud");
    if (m > 0)
    {
        gather_points<<<blocks_of(m, 256), 256, 0, s>>>(xyz, idx, m, out);
        VG_CUDA(cudaGetLastError(), "vg_filter_self_from_pointcloud: launch");
        VG_CUDA(cudaStreamSynchronize(s), "vg_filter_self_from_pointcloud");
    }
    *n_out = m;
    return VG_OK;
}

int vg_filter_self_from_pointcloud(const char *robot, vg_env *env, const float *xyz, size_t n, float point_radius,
                                   const float *q, float *out, size_t *n_out)
{
    if (!n_out || (n && (!xyz || !out)))
        return set_error(VG_ERR_ARG, "vg_filter_self_from_pointcloud: bad argument");
    *n_out = 0;
    if (n == 0)
        return VG_OK;
    float *d_in = nullptr;
    VG_CUDA(cudaMalloc(&d_in, 2 * n * 3 * sizeof(float)), "vg_filter_self_from_pointcloud: cudaMalloc");
    float *d_out = d_in + 3 * n;
    int rc = VG_OK;
    cudaError_t e = cudaMemcpy(d_in, xyz, n * 3 * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        rc = vg_filter_self_from_pointcloud_device(robot, env, d_in, n, point_radius, q, d_out, n_out, nullptr);
    if (e == cudaSuccess && rc == VG_OK && *n_out)
        e = cudaMemcpy(out, d_out, *n_out * 3 * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(d_in);
    if (e != cudaSuccess)
        return cuda_fail(e, "vg_filter_self_from_pointcloud: copy");
    return rc;
}

int vg_filter_pointcloud(const float *xyz, size_t n, float min_dist, float max_range, const float *origin,
                         const float *workcell_min, const float *workcell_max, int cull, float *out, size_t *n_out,
                         uint64_t *elapsed_ns)
{
    const auto t0 = std::chrono::steady_clock::now();
    if (int rc = check_filter_args(xyz, n, origin, workcell_min, workcell_max, out, n_out))
        return rc;
    *n_out = 0;
    if (n > 0)
    {
        float *d_in = nullptr;
        VG_CUDA(cudaMalloc(&d_in, 2 * n * 3 * sizeof(float)), "vg_filter_pointcloud: cudaMalloc");
        float *d_out = d_in + 3 * n;
        int rc = VG_OK;
        cudaError_t e = cudaMemcpy(d_in, xyz, n * 3 * sizeof(float), cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            rc = filter_on_device(d_in, n, min_dist, max_range, origin, workcell_min, workcell_max, cull, d_out, n_out,
                                  nullptr);
        if (e == cudaSuccess && rc == VG_OK && *n_out)
            e = cudaMemcpy(out, d_out, *n_out * 3 * sizeof(float), cudaMemcpyDeviceToHost);
        cudaFree(d_in);
        if (e != cudaSuccess)
            return cuda_fail(e, "vg_filter_pointcloud: copy");
        if (rc != VG_OK)
            return rc;
    }
    if (elapsed_ns)
        *elapsed_ns = static_cast<uint64_t>(
            std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0).count());
    return VG_OK;
}

}  // extern "C"
