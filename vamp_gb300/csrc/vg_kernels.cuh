// Batched collision-checking kernels for sm_103a.
//
//   states_kernel : Robot::fkcc for one configuration per thread, as the reference's
//                   validate(q) evaluates it (bindings/robot_helper.hh:256-267).
//   edges_kernel  : planning::validate_motion for a batch of edges (planning/validate.hh:24-77).
//                   Persistent: each W-lane segment owns one edge at a time, walks its blocks in
//                   the reference's order (block 0 = fractions k/W, then repeated back-steps),
//                   stops at the first colliding block and pulls the next edge from a global
//                   counter.  A warp checks four blocks of four different edges per step.
//   spheres_kernel: all sphere slots for a batch of configurations (Robot::sphere_fk).
#pragma once

#include <cstdint>

#include "vg_check.cuh"

// Resident blocks of 128 threads per SM the kernels are compiled for (caps their registers).
#ifndef VG_MIN_BLOCKS
#define VG_MIN_BLOCKS 4
#endif
// The register-rich variant of the same-edge kernel (fewer resident blocks, no register cap
// below 168): the autotuner picks it where it is faster (pointcloud scenes).
#ifndef VG_MIN_BLOCKS_WIDE
#define VG_MIN_BLOCKS_WIDE 3
#endif
// Environment section form of the default same-edge kernel: 0 unrolled, 1 loops (the
// register-rich variant and the states kernel always use loops).
#ifndef VG_DEFAULT_LOOPED_ENV
#define VG_DEFAULT_LOOPED_ENV 0
#endif

namespace vg
{
    // Device image of an environment: the x86 RSQRTPS table followed by the primitive records
    // of each kind (layouts in vg_check.cuh), all float4 aligned.
    struct EnvDevice
    {
        const float4 *buf;  // whole image
        int n_f4;           // image size in float4
        int n[5];           // objects per kind
        int off[5];         // record offset of each kind, in float4 from the image start
        int sqrt_mode;
        int n_clouds;       // CaptView descriptors at the end of the image
        int cloud_off;      // their offset, in float4
        int n_att;          // attachment spheres (-1: no attachment)
        int att_off;        // attachment block: 3 transform rows, then the spheres, in float4
        int n_hf;           // HeightView descriptors
        int hf_off;         // their offset, in float4
    };

    constexpr int kRsqrtF4 = 2048 / 4;

    // Float4s of the image each block stages into shared memory: all but the RSQRTPS table,
    // which stays in global memory (read through the L1 cache), so that shared memory goes to
    // more resident warps.
    __host__ __device__ constexpr int staged_f4(int n_f4)
    {
        return n_f4 - kRsqrtF4;
    }

    __device__ __forceinline__ EnvView stage_env(const EnvDevice &d, float4 *smem)
    {
        const int n = staged_f4(d.n_f4);
        for (int i = threadIdx.x; i < n; i += blockDim.x)
        {
            smem[i] = d.buf[kRsqrtF4 + i];
        }
        __syncthreads();
        EnvView v;
        v.rsqrt_tab = reinterpret_cast<const uint32_t *>(d.buf);
        v.sqrt_mode = d.sqrt_mode;
        v.clouds = reinterpret_cast<const CaptView *>(smem + d.cloud_off - kRsqrtF4);
        v.n_clouds = d.n_clouds;
        v.att = smem + d.att_off - kRsqrtF4;
        v.n_att = d.n_att;
        v.hf = reinterpret_cast<const HeightView *>(smem + d.hf_off - kRsqrtF4);
        v.n_hf = d.n_hf;
        for (int k = 0; k < 5; ++k)
        {
            v.rec[k] = smem + d.off[k] - kRsqrtF4;
            v.n[k] = d.n[k];
        }
        return v;
    }

    // The attachment part of Robot::fkcc_attach (robots/panda.hh:15308-15445) for the segments
    // in `alive`: the attachment's spheres posed at the end effector (Attachment::pose,
    // collision/attachments.hh:43-55: p_tf * tf, then each centre) against the environment
    // (attachment_environment_collision, validity.hh:251-268), then, per robot link the
    // reference lists, its coarse sphere gating its fine spheres against the posed spheres
    // (attachment_sphere_collision, validity.hh:270-293).  Returns the segments still valid.
    // Every product is a chain of fused multiply-adds, first term first.
    template <typename Robot, int W, bool kExt>
    __device__ __noinline__ unsigned attach_check(const EnvView &ev, const float *q, unsigned alive)
    {
        CheckCtx<W, kExt> ctx{ev, alive, false, nullptr, nullptr};
        float T[12], NR[9], Nt[3];
        Robot::ee_pose(q, T);
        const float4 *A = ev.att;
        const float a[3][4] = {{A[0].x, A[0].y, A[0].z, A[0].w}, {A[1].x, A[1].y, A[1].z, A[1].w},
                               {A[2].x, A[2].y, A[2].z, A[2].w}};
#pragma unroll
        for (int r = 0; r < 3; ++r)
        {
#pragma unroll
            for (int c = 0; c < 3; ++c)
                NR[3 * r + c] = __fmaf_rn(T[3 * r + 2], a[2][c], __fmaf_rn(T[3 * r + 1], a[1][c], __fmul_rn(T[3 * r], a[0][c])));
            Nt[r] = __fmaf_rn(T[3 * r + 2], a[2][3], __fmaf_rn(T[3 * r + 1], a[1][3], __fmaf_rn(T[3 * r], a[0][3], T[9 + r])));
        }
        auto posed = [&](int k) {
            const float4 s = A[3 + k];
            float c[3];
#pragma unroll
            for (int r = 0; r < 3; ++r)
                c[r] = __fmaf_rn(NR[3 * r + 2], s.z, __fmaf_rn(NR[3 * r + 1], s.y, __fmaf_rn(NR[3 * r], s.x, Nt[r])));
            return make_float4(c[0], c[1], c[2], s.w);
        };
        unsigned need = ctx.alive;
#pragma unroll 1
        for (int k = 0; k < ev.n_att && need; ++k)
        {
            const float4 c = posed(k);
            const unsigned hit = ctx.env_hit(c.x, c.y, c.z, c.w, need);
            ctx.alive &= ~hit;
            need &= ~hit;
        }
        if (!need)
            return ctx.alive;
        float S[Robot::kSlots * 4];
        Robot::spheres(q, S);
        // any posed sphere against robot slot `slot`, for the segments in m
        auto robot_hit = [&](int slot, unsigned m) {
            unsigned hit = 0;
#pragma unroll 1
            for (int k = 0; k < ev.n_att && (m & ~hit); ++k)
            {
                const float4 c = posed(k);
                hit |= ctx.self_hit(S[4 * slot], S[4 * slot + 1], S[4 * slot + 2], S[4 * slot + 3], c.x, c.y, c.z, c.w,
                                    m & ~hit);
            }
            return hit;
        };
#pragma unroll 1
        for (int L = 0; L < Robot::kAttachLinks && need; ++L)
        {
            const int4 li = Robot::attach_link(L);
            unsigned gate = robot_hit(li.x, need);
#pragma unroll 1
            for (int f = li.y; f < li.z && gate; ++f)
            {
                const unsigned hit = robot_hit(Robot::attach_fine(f), gate);
                ctx.alive &= ~hit;
                need &= ~hit;
                gate &= ~hit;
            }
        }
        return ctx.alive;
    }

    // kLoopedEnv: the robot's environment section as loops (smaller code) instead of unrolled;
    // kExt: the extended checks, for environments with heightfields or an attachment: every
    // environment query also tests the heightfields, and with an attachment the block runs
    // Robot::fkcc_attach
    // kOrdered: the segments are consecutive blocks of one edge (CheckCtx)
    template <typename Robot, int W, bool kLoopedEnv = false, bool kExt = false, bool kOrdered = false>
    __device__ __forceinline__ unsigned run_fkcc(const EnvView &ev, const float *q, unsigned alive, float *stage)
    {
        static_assert(Robot::kEnvChecks <= kWarpScratch, "per-warp scratch holds one word per environment check");
        __shared__ unsigned warp_scratch[kStageStride / 32][kWarpScratch];
        CheckCtx<W, kExt, kOrdered> ctx{ev, alive, false, stage, warp_scratch[threadIdx.x >> 5]};
        Robot::template fkcc<CheckCtx<W, kExt, kOrdered>, kLoopedEnv>(q, ctx);
        if constexpr (kExt)
        {
            if (ctx.alive && ev.n_att >= 0)
                ctx.alive = attach_check<Robot, W, kExt>(ev, q, ctx.alive);
        }
        return ctx.alive;
    }

    // ------------------------------------------------------------------------------ states

    struct StatesParams
    {
        const float *q;  // [n][dim]
        long long n;
        uint8_t *out;    // 1 = valid
        EnvDevice env;
    };

    template <typename Robot, bool kExt = false>
    __global__ void __launch_bounds__(128, VG_MIN_BLOCKS) states_kernel(StatesParams p)
    {
        extern __shared__ float4 smem[];
        const EnvView ev = stage_env(p.env, smem);
        // this thread's column of the robot's shared-memory stage (blocks of kStageStride threads)
        float *const stage = reinterpret_cast<float *>(smem + staged_f4(p.env.n_f4)) + threadIdx.x;
        constexpr int D = Robot::kDim;
        const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
        // every lane of a warp iterates the same number of times (warp-uniform loop)
        const long long base0 = static_cast<long long>(blockIdx.x) * blockDim.x + (threadIdx.x & ~31);
        for (long long base = base0; base < p.n; base += stride)
        {
            const long long idx = base + (threadIdx.x & 31);
            const bool in = idx < p.n;
            float q[D];
#pragma unroll
            for (int d = 0; d < D; ++d)
            {
                q[d] = in ? p.q[idx * D + d] : 0.0f;
            }
            const unsigned alive = run_fkcc<Robot, 1, true, kExt>(ev, q, __ballot_sync(kFull, in), stage);
            if (in)
            {
                p.out[idx] = static_cast<uint8_t>((alive >> (threadIdx.x & 31)) & 1u);
            }
        }
    }

    // ------------------------------------------------------------------------------ blocks

    // Robot::fkcc on caller-given blocks of W configurations (robots/panda.hh:5226-5229): each
    // W-lane segment is one ConfigurationBlock<W>, with the reference's block semantics (coarse
    // gates and loop exits decided for the whole block); out[b] = 1 when block b is valid.  q is
    // [n][W][dim].  kExt: the extended checks (heightfields, fkcc_attach).
    template <typename Robot, int W, bool kExt = false>
    __global__ void __launch_bounds__(128, VG_MIN_BLOCKS) blocks_kernel(StatesParams p)
    {
        extern __shared__ float4 smem[];
        const EnvView ev = stage_env(p.env, smem);
        float *const stage = reinterpret_cast<float *>(smem + staged_f4(p.env.n_f4)) + threadIdx.x;
        constexpr int D = Robot::kDim;
        constexpr int S = 32 / W;  // blocks per warp
        const int lane = threadIdx.x & 31;
        const long long stride = static_cast<long long>(gridDim.x) * (blockDim.x >> 5) * S;
        for (long long base = (static_cast<long long>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5)) * S; base < p.n;
             base += stride)
        {
            const long long blk = base + lane / W;
            const bool in = blk < p.n;
            float q[D];
#pragma unroll
            for (int d = 0; d < D; ++d)
            {
                q[d] = in ? p.q[(blk * W + lane % W) * D + d] : 0.0f;
            }
            const unsigned alive = run_fkcc<Robot, W, true, kExt>(ev, q, __ballot_sync(kFull, in), stage);
            if (in && lane % W == 0)
            {
                p.out[blk] = static_cast<uint8_t>((alive >> lane) & 1u);
            }
        }
    }

    // ------------------------------------------------------------------------------- edges

    struct EdgesParams
    {
        const float *a;  // [n][dim] start configurations
        const float *b;  // [n][dim] goal configurations (with dist: the motion vectors)
        int n;
        int resolution;
        uint8_t *out;        // 1 = valid
        int32_t *blocks;     // optional: blocks checked per edge
        unsigned *head;      // work counter, zero before launch
        EnvDevice env;
        // learned order (same-edge schedule only): per-edge collision scores of `probes` states
        // at fractions (p + 0.5) / probes along the edge; null = the reference's block order
        const float *scores;
        int probes;
        // validate_vector form (planning/validate.hh:23-63): b holds each edge's vector and dist
        // its length as the caller gives it (the block count follows it); null = validate_motion
        const float *dist = nullptr;
        // learned order: per edge kOrderMax / (32 / W) group indices in checking order, written
        // by edge_order_kernel from the scores
        uint8_t *order = nullptr;
    };

    constexpr int kOrderMax = 64;  // blocks of an edge the learned order ranks; later ones follow in order

    // Learned order of one edge's groups of S = 32 / W consecutive blocks (the blocks one warp
    // iteration checks together, which keeps the warp's segments on neighbouring states), written
    // to order[0..ceil(min(n, kOrderMax) / S)).  Block i holds the states at fractions
    // (k n - i) / (W n), k = 1..W; its score is the largest probe score (linearly interpolated
    // along the edge) over those states, and a group's score is its blocks' largest.  Group 0
    // stays first: its block 0 is the reference's first block and already ends most colliding
    // edges.  Ties keep the reference's order; any scores (NaN and infinities included) give a
    // permutation of the groups.
    template <int W>
    __device__ __forceinline__ void learned_order(const float *scores, int probes, int n, uint8_t *order)
    {
        constexpr int S = 32 / W;
        constexpr int kGroups = kOrderMax / S;
        const int lane = threadIdx.x & 31;
        const float sp = lane < probes ? scores[lane] : 0.0f;
        const int nb = n < kOrderMax ? n : kOrderMax;
        const int ng = (nb + S - 1) / S;
        const float inv = 1.0f / static_cast<float>(W * n);
        float sc[2];
#pragma unroll
        for (int h = 0; h < 2; ++h)
        {
            const int i = lane + 32 * h;
            float best = -INFINITY;
#pragma unroll
            for (int k = 1; k <= W; ++k)
            {
                float x = static_cast<float>(k * n - i) * inv * static_cast<float>(probes) - 0.5f;
                x = fminf(fmaxf(x, 0.0f), static_cast<float>(probes - 1));
                const int i0 = min(static_cast<int>(x), probes - 1);
                const int i1 = min(i0 + 1, probes - 1);
                const float s0 = __shfl_sync(kFull, sp, i0);
                const float s1 = __shfl_sync(kFull, sp, i1);
                best = fmaxf(best, fmaf(x - static_cast<float>(i0), s1 - s0, s0));
            }
            sc[h] = i < nb ? best : -INFINITY;
        }
        // group g (lane g) = blocks g S .. g S + S - 1
        float gs = -INFINITY;
#pragma unroll
        for (int j = 0; j < S; ++j)
        {
            const int i = (lane % kGroups) * S + j;
            const float v0 = __shfl_sync(kFull, sc[0], i & 31);
            const float v1 = __shfl_sync(kFull, sc[1], i & 31);
            gs = fmaxf(gs, i < 32 ? v0 : v1);
        }
        if (lane == 0)
        {
            gs = INFINITY;
        }
        if (lane >= ng)
        {
            gs = -INFINITY;
        }
        int rank = 0;
#pragma unroll 1
        for (int j = 0; j < kGroups; ++j)
        {
            const float sj = __shfl_sync(kFull, gs, j);
            rank += (sj > gs) || (sj == gs && j < lane);
        }
        if (lane < ng)
        {
            order[rank] = static_cast<uint8_t>(lane);
        }
        __syncwarp();
    }

    // The learned group order of every edge (one warp per edge) from its probe scores, for the
    // same-edge check with the learned order: p.order[e][0 .. kOrderMax / (32 / W)).  Edges of
    // one group (n <= 32 / W blocks) get the reference's order.
    template <int D, int W>
    __global__ void __launch_bounds__(128) edge_order_kernel(EdgesParams p);

    // |b - a| as the reference computes it on x86: squares summed lane-wise over the 8-wide
    // vectors that hold the configuration, then ((s0+s4)+(s2+s6)) + ((s1+s5)+(s3+s7)), then a
    // correctly rounded sqrt (vector/avx.hh:442-452, vector/interface.hh:402-410).
    template <int D>
    __device__ __forceinline__ float edge_length(const float *v)
    {
        float s[8];
#pragma unroll
        for (int k = 0; k < 8; ++k)
        {
            s[k] = 0.0f;
        }
#pragma unroll
        for (int d = 0; d < D; ++d)
        {
            const float sq = __fmul_rn(v[d], v[d]);
            s[d & 7] = d < 8 ? sq : __fadd_rn(s[d & 7], sq);
        }
        const float a0 = __fadd_rn(s[4], s[0]), a1 = __fadd_rn(s[5], s[1]);
        const float a2 = __fadd_rn(s[6], s[2]), a3 = __fadd_rn(s[7], s[3]);
        return __fsqrt_rn(__fadd_rn(__fadd_rn(a0, a2), __fadd_rn(a1, a3)));
    }

    template <int D, int W>
    __global__ void __launch_bounds__(128) edge_order_kernel(EdgesParams p)
    {
        constexpr int S = 32 / W;
        constexpr int kGroups = kOrderMax / S;
        __shared__ uint8_t s_order[4][kOrderMax];
        const int lane = threadIdx.x & 31;
        uint8_t *order = s_order[(threadIdx.x >> 5) & 3];
        const long long warps = static_cast<long long>(gridDim.x) * (blockDim.x >> 5);
        for (long long e = static_cast<long long>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); e < p.n; e += warps)
        {
            // the block count exactly as the edge kernels compute it
            float v[D];
#pragma unroll
            for (int d = 0; d < D; ++d)
            {
                const float av = p.a[e * D + d];
                v[d] = p.dist ? p.b[e * D + d] : __fsub_rn(p.b[e * D + d], av);
            }
            const float len = p.dist ? p.dist[e] : edge_length<D>(v);
            const float t = __fmul_rn(__fdiv_rn(len, static_cast<float>(W)), static_cast<float>(p.resolution));
            const float nf = ceilf(t);
            const int n = static_cast<int>(nf > 1.0f ? nf : 1.0f);
            if (lane < kGroups)
            {
                order[lane] = static_cast<uint8_t>(lane);
            }
            __syncwarp();
            if (n > S)
            {
                learned_order<W>(p.scores + e * p.probes, p.probes, n, order);
            }
            if (lane < kGroups)
            {
                p.order[e * kGroups + lane] = order[lane];
            }
            __syncwarp();
        }
    }

    template <typename Robot, int W, bool kExt = false>
    __global__ void __launch_bounds__(128, VG_MIN_BLOCKS) edges_kernel(EdgesParams p)
    {
        extern __shared__ float4 smem[];
        const EnvView ev = stage_env(p.env, smem);
        // this thread's column of the robot's shared-memory stage (blocks of kStageStride threads)
        float *const stage = reinterpret_cast<float *>(smem + staged_f4(p.env.n_f4)) + threadIdx.x;
        constexpr int D = Robot::kDim;
        const int lane = threadIdx.x & 31;
        const int sl = lane % W;                  // lane within the segment
        const int leader = lane - sl;             // segment's first lane
        constexpr unsigned kLeaders = W == 1 ? kFull : (W == 2 ? 0x55555555u : (W == 4 ? 0x11111111u : (W == 8 ? 0x01010101u : (W == 16 ? 0x00010001u : 1u))));
        const float pct = __fdiv_rn(static_cast<float>(sl + 1), static_cast<float>(W));

        int e = -1;       // current edge of my segment (-1: none)
        int n = 0;        // blocks of the edge
        int i = 0;        // current block
        float q[D], bs[D];

        // Pull new edges for the segments in `need` (a lane mask, whole segments).
        auto refill = [&](unsigned need) {
            const unsigned lead = need & kLeaders;
            unsigned base = 0;
            if (lane == 0)
            {
                base = atomicAdd(p.head, static_cast<unsigned>(__popc(lead)));
            }
            base = __shfl_sync(kFull, base, 0);
            const unsigned mine = base + __popc(lead & ((1u << lane) - 1u));
            const unsigned got = __shfl_sync(kFull, mine, leader);
            if ((need >> lane) & 1u)
            {
                if (got >= static_cast<unsigned>(p.n))
                {
                    e = -1;
                }
                else
                {
                    e = static_cast<int>(got);
                    float av[D], v[D];
#pragma unroll
                    for (int d = 0; d < D; ++d)
                    {
                        av[d] = p.a[static_cast<long long>(e) * D + d];
                        v[d] = p.dist ? p.b[static_cast<long long>(e) * D + d]
                                      : __fsub_rn(p.b[static_cast<long long>(e) * D + d], av[d]);
                    }
                    const float len = p.dist ? p.dist[e] : edge_length<D>(v);
                    const float t = __fmul_rn(__fdiv_rn(len, static_cast<float>(W)), static_cast<float>(p.resolution));
                    const float nf = ceilf(t);
                    n = static_cast<int>(nf > 1.0f ? nf : 1.0f);
                    i = 0;
                    const float denom = static_cast<float>(W * n);
#pragma unroll
                    for (int d = 0; d < D; ++d)
                    {
                        q[d] = __fmaf_rn(v[d], pct, av[d]);
                        bs[d] = __fdiv_rn(v[d], denom);
                    }
                }
            }
        };

        refill(kFull);
        for (;;)
        {
            const unsigned active = __ballot_sync(kFull, e >= 0);
            if (!active)
            {
                break;
            }
            const unsigned alive = run_fkcc<Robot, W, false, kExt>(ev, q, active, stage);
            bool finish = false;
            if (e >= 0)
            {
                const bool bad = ((alive >> lane) & 1u) == 0u;
                if (bad || i + 1 >= n)
                {
                    finish = true;
                    if (sl == 0)
                    {
                        p.out[e] = bad ? 0 : 1;
                        if (p.blocks)
                        {
                            p.blocks[e] = i + 1;
                        }
                    }
                }
                else
                {
                    ++i;
#pragma unroll
                    for (int d = 0; d < D; ++d)
                    {
                        q[d] = __fsub_rn(q[d], bs[d]);
                    }
                }
            }
            const unsigned need = __ballot_sync(kFull, finish);
            if (need)
            {
                refill(need);
            }
        }
    }

    // Same-edge schedule: a warp owns one edge at a time and its 32 / W segments check
    // consecutive blocks i0, i0 + 1, ... of it.  Lanes that stand for neighbouring blocks sit at
    // almost the same configurations, so the warp's union of control flow is close to a single
    // block's.  Each segment reaches its block by the same repeated subtraction as the reference
    // (block i = block 0 minus v / (W n), i times).  The edge is invalid if any checked block is,
    // and the reference would have stopped at the first invalid block, so the block count
    // reported is that block's index + 1.
    template <typename Robot, int W, bool kLearned, int kMinBlocks = VG_MIN_BLOCKS, bool kLoopedEnv = VG_DEFAULT_LOOPED_ENV != 0>
    __global__ void __launch_bounds__(128, kMinBlocks) edges_grouped_kernel(EdgesParams p)
    {
        extern __shared__ float4 smem[];
        const EnvView ev = stage_env(p.env, smem);
        // this thread's column of the robot's shared-memory stage (blocks of kStageStride threads)
        float *const stage = reinterpret_cast<float *>(smem + staged_f4(p.env.n_f4)) + threadIdx.x;
        constexpr int D = Robot::kDim;
        constexpr int S = 32 / W;                 // segments (blocks) per warp
        const int lane = threadIdx.x & 31;
        const int seg = lane / W;
        const int sl = lane % W;
        const float pct = __fdiv_rn(static_cast<float>(sl + 1), static_cast<float>(W));
        constexpr unsigned kSegBits = W == 32 ? kFull : ((1u << W) - 1u);
        constexpr unsigned kSegLeaders = W == 8 ? 0x01010101u : (W == 4 ? 0x11111111u : 1u);

        for (;;)
        {
            unsigned got = 0;
            if (lane == 0)
            {
                got = atomicAdd(p.head, 1u);
            }
            got = __shfl_sync(kFull, got, 0);
            if (got >= static_cast<unsigned>(p.n))
            {
                break;
            }
            const int e = static_cast<int>(got);
            float q[D], bs[D], v[D];
#pragma unroll
            for (int d = 0; d < D; ++d)
            {
                const float av = p.a[static_cast<long long>(e) * D + d];
                v[d] = p.dist ? p.b[static_cast<long long>(e) * D + d]
                              : __fsub_rn(p.b[static_cast<long long>(e) * D + d], av);
                q[d] = __fmaf_rn(v[d], pct, av);
            }
            const float len = p.dist ? p.dist[e] : edge_length<D>(v);
            const float t = __fmul_rn(__fdiv_rn(len, static_cast<float>(W)), static_cast<float>(p.resolution));
            const float nf = ceilf(t);
            const int n = static_cast<int>(nf > 1.0f ? nf : 1.0f);
            const float denom = static_cast<float>(W * n);
#pragma unroll
            for (int d = 0; d < D; ++d)
            {
                bs[d] = __fdiv_rn(v[d], denom);
            }
            // q holds block `cur`; block i is block 0 minus i repeated steps, as the reference
            // computes it (planning/validate.hh:50-56)
            int cur = 0;
            int verdict = 1, checked = n;
            if constexpr (kLearned)
            {
                // the group order edge_order_kernel wrote for this edge (edges of one group keep
                // the reference's order)
                constexpr int kGroups = kOrderMax / S;
                const uint8_t *order = p.order + static_cast<long long>(e) * kGroups;
                const bool learned = n > S;
                int done = 0;  // blocks checked in earlier iterations
                for (int i0 = 0; i0 < n; i0 += S)
                {
                    const int g = i0 / S;
                    const int want = (learned && g < kGroups ? static_cast<int>(order[g]) * S : i0) + seg;
                    const bool active = want < n;
                    if (active)
                    {
                        if (want < cur)
                        {
                            // back to block 0: the edge's vector is re-read rather than kept in
                            // registers through the check (same values, same rounding)
#pragma unroll
                            for (int d = 0; d < D; ++d)
                            {
                                const float av = p.a[static_cast<long long>(e) * D + d];
                                const float vd = p.dist ? p.b[static_cast<long long>(e) * D + d]
                                                        : __fsub_rn(p.b[static_cast<long long>(e) * D + d], av);
                                q[d] = __fmaf_rn(vd, pct, av);
                            }
                            cur = 0;
                        }
#pragma unroll 1
                        for (; cur < want; ++cur)
                        {
#pragma unroll
                            for (int d = 0; d < D; ++d)
                            {
                                q[d] = __fsub_rn(q[d], bs[d]);
                            }
                        }
                    }
                    const unsigned mask = __ballot_sync(kFull, active);
                    const unsigned alive = run_fkcc<Robot, W, kLoopedEnv, false, true>(ev, q, mask, stage);
                    const unsigned dead = mask & ~alive;
                    // one bit per active segment (its first lane)
                    const unsigned leaders = mask & kSegLeaders;
                    if (dead)
                    {
                        verdict = 0;
                        const unsigned below = (1u << ((__ffs(dead) - 1) / W * W)) - 1u;
                        checked = done + __popc(leaders & below) + 1;
                        break;
                    }
                    done += __popc(leaders);
                }
            }
            else
            {
                // segment `seg` starts at block `seg`
                for (; cur < seg; ++cur)
                {
#pragma unroll
                    for (int d = 0; d < D; ++d)
                    {
                        q[d] = __fsub_rn(q[d], bs[d]);
                    }
                }
                for (int i0 = 0; i0 < n; i0 += S)
                {
                    const bool active = i0 + seg < n;
                    const unsigned mask = __ballot_sync(kFull, active);
                    const unsigned alive = run_fkcc<Robot, W, kLoopedEnv, false, true>(ev, q, mask, stage);
                    const unsigned dead = mask & ~alive;
                    if (dead)
                    {
                        verdict = 0;
                        checked = i0 + (__ffs(dead) - 1) / W + 1;
                        break;
                    }
#pragma unroll 1
                    for (int k = 0; k < S; ++k)
                    {
#pragma unroll
                        for (int d = 0; d < D; ++d)
                        {
                            q[d] = __fsub_rn(q[d], bs[d]);
                        }
                    }
                }
            }
            (void)kSegBits;
            if (lane == 0)
            {
                p.out[e] = static_cast<uint8_t>(verdict);
                if (p.blocks)
                {
                    p.blocks[e] = checked;
                }
            }
        }
    }

    // Packed same-edge schedule: as edges_grouped_kernel, except that the segments an edge's last
    // blocks leave free start on the next edge instead of idling.  A warp iteration covers at
    // most two edges: the one carried over from the previous iteration (its next blocks, from
    // segment 0 on) and one taken from the queue (its first blocks, in the segments after those).
    // Only the edge in the last segment can be carried over, so the carried edge's newest block
    // always sits in the last segment: each segment takes that block's configuration and bs from
    // the last segment (same lane of the segment) and subtracts bs seg + 1 more times.  Every
    // block is therefore still block 0 minus bs repeated i times, as the reference computes it
    // (planning/validate.hh:50-56), and verdicts and block counts equal edges_grouped_kernel's.
    template <typename Robot, int W, int kMinBlocks = VG_MIN_BLOCKS, bool kLoopedEnv = VG_DEFAULT_LOOPED_ENV != 0>
    __global__ void __launch_bounds__(128, kMinBlocks) edges_packed_kernel(EdgesParams p)
    {
        static_assert(W == 8 || W == 4, "packed schedule: 4 or 8 segments per warp");
        extern __shared__ float4 smem[];
        const EnvView ev = stage_env(p.env, smem);
        float *const stage = reinterpret_cast<float *>(smem + staged_f4(p.env.n_f4)) + threadIdx.x;
        constexpr int D = Robot::kDim;
        constexpr int S = 32 / W;  // segments (blocks) per warp
        const int lane = threadIdx.x & 31;
        const int seg = lane / W;
        const int sl = lane % W;
        const int last = (S - 1) * W + sl;  // this lane's counterpart in the last segment
        const float pct = __fdiv_rn(static_cast<float>(sl + 1), static_cast<float>(W));

        float q[D], bs[D];
#pragma unroll
        for (int d = 0; d < D; ++d)
        {
            q[d] = 0.0f;
            bs[d] = 0.0f;
        }
        // warp-uniform: the carried edge (-1: none), its block count and its next block
        int ce = -1, cn = 0, cpos = 0;
        bool drained = false;  // warp-uniform: the queue is empty
        for (;;)
        {
            // segments 0 .. r-1 continue the carried edge
            const int r = ce >= 0 ? min(cn - cpos, S) : 0;
            if (r > 0)
            {
#pragma unroll
                for (int d = 0; d < D; ++d)
                {
                    const float qs = __shfl_sync(kFull, q[d], last);
                    const float bss = __shfl_sync(kFull, bs[d], last);
                    if (seg < r)
                    {
                        q[d] = qs;
                        bs[d] = bss;
                    }
                }
                if (seg < r)
                {
#pragma unroll 1
                    for (int k = 0; k <= seg; ++k)
                    {
#pragma unroll
                        for (int d = 0; d < D; ++d)
                        {
                            q[d] = __fsub_rn(q[d], bs[d]);
                        }
                    }
                }
            }
            // the remaining segments start on a new edge
            int ne = -1, nn = 0;
            if (r < S && !drained)
            {
                unsigned got = 0;
                if (lane == 0)
                {
                    got = atomicAdd(p.head, 1u);
                }
                got = __shfl_sync(kFull, got, 0);
                if (got >= static_cast<unsigned>(p.n))
                {
                    drained = true;
                }
                else
                {
                    ne = static_cast<int>(got);
                }
            }
            if (ne >= 0)
            {
                float av[D], v[D];
#pragma unroll
                for (int d = 0; d < D; ++d)
                {
                    av[d] = p.a[static_cast<long long>(ne) * D + d];
                    v[d] = p.dist ? p.b[static_cast<long long>(ne) * D + d]
                                  : __fsub_rn(p.b[static_cast<long long>(ne) * D + d], av[d]);
                }
                const float len = p.dist ? p.dist[ne] : edge_length<D>(v);
                const float t = __fmul_rn(__fdiv_rn(len, static_cast<float>(W)), static_cast<float>(p.resolution));
                const float nf = ceilf(t);
                nn = static_cast<int>(nf > 1.0f ? nf : 1.0f);
                if (seg >= r)
                {
                    const float denom = static_cast<float>(W * nn);
#pragma unroll
                    for (int d = 0; d < D; ++d)
                    {
                        q[d] = __fmaf_rn(v[d], pct, av[d]);
                        bs[d] = __fdiv_rn(v[d], denom);
                    }
#pragma unroll 1
                    for (int k = r; k < seg; ++k)
                    {
#pragma unroll
                        for (int d = 0; d < D; ++d)
                        {
                            q[d] = __fsub_rn(q[d], bs[d]);
                        }
                    }
                }
            }
            const bool active = seg < r || (ne >= 0 && seg >= r && seg - r < nn);
            const unsigned mask = __ballot_sync(kFull, active);
            if (!mask)
            {
                break;  // nothing carried and the queue is empty
            }
            const unsigned alive = run_fkcc<Robot, W, kLoopedEnv>(ev, q, mask, stage);
            const unsigned dead = mask & ~alive;
            const unsigned cmask = r >= S ? kFull : ((1u << (r * W)) - 1u);  // the carried edge's lanes
            if (ce >= 0)
            {
                const unsigned cd = dead & cmask;
                int verdict = -1, checked = 0;
                if (cd)
                {
                    verdict = 0;
                    checked = cpos + (__ffs(cd) - 1) / W + 1;
                }
                else if (cpos + r >= cn)
                {
                    verdict = 1;
                    checked = cn;
                }
                if (verdict >= 0)
                {
                    if (lane == 0)
                    {
                        p.out[ce] = static_cast<uint8_t>(verdict);
                        if (p.blocks)
                        {
                            p.blocks[ce] = checked;
                        }
                    }
                    ce = -1;
                }
                else
                {
                    cpos += r;  // r == S: no new edge this iteration
                }
            }
            if (ne >= 0)
            {
                const unsigned nd = dead & ~cmask;
                int verdict = -1, checked = 0;
                if (nd)
                {
                    verdict = 0;
                    checked = (__ffs(nd) - 1) / W - r + 1;
                }
                else if (nn <= S - r)
                {
                    verdict = 1;
                    checked = nn;
                }
                if (verdict >= 0)
                {
                    if (lane == 0)
                    {
                        p.out[ne] = static_cast<uint8_t>(verdict);
                        if (p.blocks)
                        {
                            p.blocks[ne] = checked;
                        }
                    }
                }
                else
                {
                    ce = ne;  // its blocks 0 .. S - r - 1 are checked, the last in the last segment
                    cn = nn;
                    cpos = S - r;
                }
            }
        }
    }

    // ----------------------------------------------------------------------- debug reports
    //
    // Robot::fkcc_debug (robots/panda.hh:468) for a batch of configurations, from their sphere
    // slots (spheres_kernel): per fine sphere the environment objects it collides with, by
    // sphere_environment_get_collisions' rule (collision/validity.hh:152-249: per kind, objects in
    // min_distance order until min_distance - max_extent has a clear sign bit; pointclouds are not
    // part of it), and per fine self pair of every self check whether it collides.

    // one thread per (configuration, fine self pair): 1 where sphere_sphere_self_collision
    // (collision/validity.hh:23-44) reports the pair
    template <typename Robot>
    __global__ void debug_self_kernel(const float *spheres, long long n, uint8_t *out)
    {
        const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
        if (t >= n * Robot::kSelfPairs)
        {
            return;
        }
        const long long c = t / Robot::kSelfPairs;
        const int2 pr = Robot::self_pair(static_cast<int>(t - c * Robot::kSelfPairs));
        const float *a = spheres + (c * Robot::kSlots + pr.x) * 4;
        const float *b = spheres + (c * Robot::kSlots + pr.y) * 4;
        out[t] = static_cast<uint8_t>(self_bits(a[0], a[1], a[2], b[0], b[1], b[2], __fadd_rn(a[3], b[3])) >> 31);
    }

    // ----------------------------------------------------------------------------- spheres

    template <typename Robot>
    __global__ void spheres_kernel(const float *q, long long n, float *out)
    {
        const long long idx = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
        if (idx >= n)
        {
            return;
        }
        float qq[Robot::kDim];
        for (int d = 0; d < Robot::kDim; ++d)
        {
            qq[d] = q[idx * Robot::kDim + d];
        }
        Robot::spheres(qq, out + idx * Robot::kSlots * 4);
    }

    // Robot::eefk (robots/panda.hh:15447-15552): the end effector's transform as a row-major 4x4
    // matrix per configuration.
    template <typename Robot>
    __global__ void ee_pose_kernel(const float *q, long long n, float *out)
    {
        const long long idx = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
        if (idx >= n)
        {
            return;
        }
        float qq[Robot::kDim], T[12];
        for (int d = 0; d < Robot::kDim; ++d)
        {
            qq[d] = q[idx * Robot::kDim + d];
        }
        Robot::ee_pose(qq, T);
        float *o = out + idx * 16;
        for (int r = 0; r < 3; ++r)
        {
            o[4 * r + 0] = T[3 * r + 0];
            o[4 * r + 1] = T[3 * r + 1];
            o[4 * r + 2] = T[3 * r + 2];
            o[4 * r + 3] = T[9 + r];
        }
        o[12] = 0.0f;
        o[13] = 0.0f;
        o[14] = 0.0f;
        o[15] = 1.0f;
    }
}  // namespace vg
