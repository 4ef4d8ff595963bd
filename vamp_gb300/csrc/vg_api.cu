// C ABI of libvamp_gb300.so (declared in include/vamp_gb300.h).
//
// Host code in this file is compiled with -ffp-contract=off: the min_distance of each primitive
// is computed with explicit fused multiply-adds in the same order as the CPU oracle, so that the
// GPU and the oracle take identical early-exit decisions.
#include "../../include/vamp_gb300.h"
#include "vg_internal.h"
#include "vg_capt_gpu.h"
#include "x86_rsqrt_table.h"

#include <cmath>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>

namespace vg
{
    extern const RobotOps ops_panda;
    extern const RobotOps ops_ur5;
    extern const RobotOps ops_fetch;
    extern const RobotOps ops_baxter;

    const RobotOps *const *all_robots(int *count)
    {
        static const RobotOps *const robots[] = {&ops_panda, &ops_ur5, &ops_fetch, &ops_baxter};
        *count = 4;
        return robots;
    }

    const RobotOps *find_robot(const char *name)
    {
        if (!name)
        {
            return nullptr;
        }
        int n = 0;
        const RobotOps *const *r = all_robots(&n);
        for (int i = 0; i < n; ++i)
        {
            if (std::strcmp(r[i]->name, name) == 0)
            {
                return r[i];
            }
        }
        return nullptr;
    }

    static thread_local std::string g_error;

    int set_error(int code, const std::string &msg)
    {
        g_error = msg;
        return code;
    }

    int cuda_fail(cudaError_t e, const char *what)
    {
        return set_error(VG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }

    // ---------------------------------------------------------------- primitive bookkeeping

    constexpr int kFields[5] = {4, 8, 8, 15, 15};

    static float norm3(float x, float y, float z)
    {
        return std::sqrt(std::fma(z, z, std::fma(x, x, y * y)));
    }

    // Inserts an object of a kind into the environment's sorted rows (`width` fields +
    // min_distance; ascending min_distance, ties after existing) and its insertion id (the
    // object's position among all objects added, any kind) into the parallel id list.
    static void insert_sorted(vg_env *env, int kind, int width, const float *row)
    {
        std::vector<float> &v = env->obj[kind];
        std::vector<int> &ids = env->ids[kind];
        const int w = width + 1;
        size_t pos = v.size() / w;
        v.resize(v.size() + w);
        ids.resize(ids.size() + 1);
        while (pos > 0 && v[(pos - 1) * w + width] > row[width])
        {
            std::memcpy(&v[pos * w], &v[(pos - 1) * w], sizeof(float) * w);
            ids[pos] = ids[pos - 1];
            --pos;
        }
        std::memcpy(&v[pos * w], row, sizeof(float) * w);
        ids[pos] = env->n_added++;
    }

    // Sphere::min_distance (collision/shapes.hh:236-240)
    static float sphere_min_distance(const float *f)
    {
        return norm3(f[0], f[1], f[2]) - f[3];
    }

    // Cylinder::compute_min_distance (collision/shapes.hh:165-189)
    static float capsule_min_distance(const float *f)
    {
        const float x1 = f[0], y1 = f[1], z1 = f[2], xv = f[3], yv = f[4], zv = f[5], r = f[6], rdv = f[7];
        float t = std::fma(-z1, zv, std::fma(-y1, yv, (-x1) * xv)) * rdv;
        t = std::fmax(std::fmin(t, 1.0f), 0.0f);
        const float xp = std::fma(xv, t, x1), yp = std::fma(yv, t, y1), zp = std::fma(zv, t, z1);
        float xo = -xp, yo = -yp, zo = -zp;
        const float ol = norm3(xo, yo, zo);
        xo = xo / ol;
        yo = yo / ol;
        zo = zo / ol;
        const float ro = std::fmax(std::fmin(ol, r), 0.0f);
        return norm3(std::fma(ro, xo, xp), std::fma(ro, yo, yp), std::fma(ro, zo, zp));
    }

    // Cuboid::compute_min_distance (collision/shapes.hh:52-67)
    static float cuboid_min_distance(const float *f)
    {
        const float x = f[0], y = f[1], z = f[2];
        float v[3];
        for (int k = 0; k < 3; ++k)
        {
            const float ax = f[3 + 3 * k], ay = f[4 + 3 * k], az = f[5 + 3 * k], hr = f[12 + k];
            const float d = std::fma(-z, az, std::fma(-y, ay, (-x) * ax));
            v[k] = d < -hr ? -hr : (hr < d ? hr : d);
        }
        const float xn = std::fma(f[9], v[2], std::fma(f[6], v[1], std::fma(f[3], v[0], x)));
        const float yn = std::fma(f[10], v[2], std::fma(f[7], v[1], std::fma(f[4], v[0], y)));
        const float zn = std::fma(f[11], v[2], std::fma(f[8], v[1], std::fma(f[5], v[0], z)));
        return norm3(xn, yn, zn);
    }

    // Packs the sorted host rows into the device image (layouts in vg_check.cuh).
    static void pack_image(const vg_env *e, std::vector<float4> &img, int off[5], int n[5])
    {
        img.assign(kRsqrtF4, make_float4(0, 0, 0, 0));
        std::memcpy(img.data(), kX86RsqrtTable, sizeof(uint32_t) * 2048);
        for (int k = 0; k < 5; ++k)
        {
            const int w = kFields[k] + 1;
            n[k] = static_cast<int>(e->obj[k].size() / w);
            off[k] = static_cast<int>(img.size());
            for (int i = 0; i < n[k]; ++i)
            {
                const float *f = &e->obj[k][i * w];
                const float md = f[kFields[k]];
                if (k == 0)
                {
                    img.push_back(make_float4(f[0], f[1], f[2], f[3]));
                    img.push_back(make_float4(md, 0, 0, 0));
                }
                else if (k <= 2)
                {
                    img.push_back(make_float4(f[0], f[1], f[2], f[3]));
                    img.push_back(make_float4(f[4], f[5], f[6], f[7]));
                    img.push_back(make_float4(md, 0, 0, 0));
                }
                else
                {
                    img.push_back(make_float4(f[0], f[1], f[2], f[12]));
                    img.push_back(make_float4(f[3], f[4], f[5], f[13]));
                    img.push_back(make_float4(f[6], f[7], f[8], f[14]));
                    img.push_back(make_float4(f[9], f[10], f[11], md));
                }
            }
        }
    }

    static_assert(sizeof(CaptView) % sizeof(float4) == 0, "CaptView must pack into float4s");

    // Uploads each pointcloud's tree once: kCloudBuffers device buffers per cloud (tests, aabbs,
    // starts, the reference-layout blocks, the ring-ordered blocks the queries scan, and the
    // query tables).  A host-built cloud's reference-layout blocks are freed once ordered (the
    // host copy answers layout queries).
    static int upload_clouds(vg_env *e)
    {
        while (e->d_clouds.size() < kCloudBuffers * e->clouds.size())
        {
            const CaptHost &c = e->clouds[e->d_clouds.size() / kCloudBuffers];
            const void *src[4] = {c.tests.data(), c.aabbs.data(), c.aff_starts.data(), c.aff.data()};
            const size_t bytes[4] = {c.tests.size() * sizeof(float), c.aabbs.size() * sizeof(float),
                                     c.aff_starts.size() * sizeof(uint32_t), std::max<size_t>(16, c.aff.size() * sizeof(float))};
            void *dst[4] = {nullptr, nullptr, nullptr, nullptr};
            for (int k = 0; k < 4; ++k)
            {
                cudaError_t err = cudaMalloc(&dst[k], bytes[k]);
                if (err == cudaSuccess && src[k] && (k != 3 || !c.aff.empty()))
                {
                    err = cudaMemcpy(dst[k], src[k], k == 3 ? c.aff.size() * sizeof(float) : bytes[k], cudaMemcpyHostToDevice);
                }
                if (err != cudaSuccess)
                {
                    for (int j = 0; j <= k; ++j)
                    {
                        if (dst[j])
                            cudaFree(dst[j]);
                    }
                    return cuda_fail(err, "upload pointcloud");
                }
            }
            CaptQuery q;
            const int rc = capt_query_layout(static_cast<const float *>(dst[0]), c.nlog2, static_cast<const float *>(dst[1]),
                                             static_cast<const uint32_t *>(dst[2]), static_cast<const float *>(dst[3]), c.blocks(),
                                             c.r_max, c.r_point, q);
            cudaFree(dst[3]);
            dst[3] = nullptr;
            if (rc != VG_OK)
            {
                for (int j = 0; j < 3; ++j)
                    cudaFree(dst[j]);
                return rc;
            }
            for (int k = 0; k < 4; ++k)
            {
                e->d_clouds.push_back(dst[k]);
            }
            e->d_clouds.push_back(q.aff_q);
            e->d_clouds.push_back(q.tables);
            e->capt_q.push_back(q);
        }
        return VG_OK;
    }

    static void pack_clouds(const vg_env *e, std::vector<float4> &img, int *cloud_off)
    {
        *cloud_off = static_cast<int>(img.size());
        for (size_t i = 0; i < e->clouds.size(); ++i)
        {
            const CaptHost &c = e->clouds[i];
            CaptView v{};
            const CaptQuery &q = e->capt_q[i];
            v.nodes = q.nodes;
            v.leaves = q.leaves;
            v.ends = q.ends;
            v.aff = reinterpret_cast<const float4 *>(q.aff_q);
            for (int k = 0; k < 6; ++k)
                v.top[k] = c.top[k];
            v.r_point = c.r_point;
            v.nlog2 = c.nlog2;
            for (int k = 0; k < 3; ++k)
                v.top_tests[k] = q.top_tests[k];
            v.rem = q.rem;
            v.groups = q.groups;
            for (int k = 0; k < kCaptRings; ++k)
                v.ring_edge[k] = q.ring_edge[k];
            const size_t at = img.size();
            img.resize(at + sizeof(CaptView) / sizeof(float4));
            std::memcpy(&img[at], &v, sizeof(CaptView));
        }
    }

    // Uploads the environment image if it changed; records the current device.
    int commit(vg_env *e)
    {
        int dev = 0;
        VG_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
        if (!e->dirty && e->d_image && dev == e->device)
        {
            return VG_OK;
        }
        if (e->d_image && dev != e->device)
        {
            return set_error(VG_ERR_STATE, "environment was committed on another device");
        }
        if (int rc = upload_clouds(e))
            return rc;
        // heightfield samples: one device buffer each, uploaded once
        while (e->d_hf.size() < e->hf.size())
        {
            const std::vector<float> &h = e->hf_data[e->d_hf.size()];
            void *p = nullptr;
            VG_CUDA(cudaMalloc(&p, h.size() * sizeof(float)), "cudaMalloc(heightfield)");
            e->d_hf.push_back(p);
            VG_CUDA(cudaMemcpy(p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice), "upload heightfield");
        }
        std::vector<float4> img;
        pack_image(e, img, e->off, e->n);
        pack_clouds(e, img, &e->cloud_off);
        static_assert(sizeof(HeightView) % sizeof(float4) == 0, "HeightView must pack into float4s");
        e->hf_off = static_cast<int>(img.size());
        for (size_t i = 0; i < e->hf.size(); ++i)
        {
            HeightView v = e->hf[i];
            v.data = static_cast<const float *>(e->d_hf[i]);
            const size_t at = img.size();
            img.resize(at + sizeof(HeightView) / sizeof(float4));
            std::memcpy(&img[at], &v, sizeof(HeightView));
        }
        // the attachment: 3 transform rows, then its spheres
        e->att_off = static_cast<int>(img.size());
        if (e->n_att >= 0)
        {
            for (int k = 0; k < 3 + e->n_att; ++k)
                img.push_back(make_float4(e->att[4 * k], e->att[4 * k + 1], e->att[4 * k + 2], e->att[4 * k + 3]));
        }
        if (img.size() > e->image_cap)
        {
            if (e->d_image)
            {
                cudaFree(e->d_image);
                e->d_image = nullptr;
            }
            VG_CUDA(cudaMalloc(&e->d_image, img.size() * sizeof(float4)), "cudaMalloc(environment)");
            e->image_cap = img.size();
        }
        VG_CUDA(cudaMemcpy(e->d_image, img.data(), img.size() * sizeof(float4), cudaMemcpyHostToDevice), "upload environment");
        if (!e->d_counter)
        {
            VG_CUDA(cudaMalloc(&e->d_counter, 64), "cudaMalloc(counter)");
        }
        e->image_f4 = img.size();
        e->device = dev;
        e->dirty = false;
        ++e->version;
        return VG_OK;
    }

    EnvDevice env_device(const vg_env *e)
    {
        EnvDevice d{};
        d.buf = e->d_image;
        d.n_f4 = static_cast<int>(e->image_f4);
        for (int k = 0; k < 5; ++k)
        {
            d.n[k] = e->n[k];
            d.off[k] = e->off[k];
        }
        d.sqrt_mode = e->sqrt_mode;
        d.n_clouds = static_cast<int>(e->clouds.size());
        d.cloud_off = e->cloud_off;
        d.n_att = e->n_att;
        d.att_off = e->att_off;
        d.n_hf = static_cast<int>(e->hf.size());
        d.hf_off = e->hf_off;
        return d;
    }

    int sm_count()
    {
        // per device: grids are sized for the GPU the call runs on
        constexpr int kDevices = 64;
        static std::atomic<int> counts[kDevices] = {};
        int dev = 0;
        cudaGetDevice(&dev);
        if (dev < 0 || dev >= kDevices)
        {
            int c = 0;
            cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
            return c > 0 ? c : 1;
        }
        int c = counts[dev].load(std::memory_order_relaxed);
        if (c <= 0)
        {
            cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev);
            c = c > 0 ? c : 1;
            counts[dev].store(c, std::memory_order_relaxed);
        }
        return c;
    }

    int prepare_kernel(const void *fn, int smem, int block, int *blocks_per_sm)
    {
        // The occupancy of the last few (kernel, device, shared memory, block) combinations is
        // kept, so that a single-edge call does not pay the driver's occupancy query.  The
        // kernel's dynamic shared-memory limit is set on every call: it is one value per kernel,
        // which a call with a smaller environment lowers.
        struct Seen
        {
            const void *fn;
            int dev, smem, block, occ;
        };
        static thread_local Seen seen[16] = {};
        static thread_local int next = 0;
        int dev = 0;
        VG_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
        for (const Seen &s : seen)
        {
            if (s.fn == fn && s.dev == dev && s.smem == smem && s.block == block && s.occ > 0)
            {
                if (smem > 48 * 1024)
                {
                    VG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem), "cudaFuncSetAttribute");
                }
                *blocks_per_sm = s.occ;
                return VG_OK;
            }
        }
        int smem_max = 0;
        VG_CUDA(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "shared-memory limit");
        if (smem > smem_max)
        {
            return set_error(VG_ERR_LIMIT, "the environment and the robot's staging need " + std::to_string(smem) +
                                               " bytes of shared memory per block, more than the GPU's " +
                                               std::to_string(smem_max) + " (too many primitives)");
        }
        if (smem > 48 * 1024)
        {
            VG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem), "cudaFuncSetAttribute");
        }
        int occ = 0;
        VG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, block, smem), "occupancy");
        if (occ <= 0)
        {
            return set_error(VG_ERR_LIMIT, "kernel does not fit on a multiprocessor (environment too large?)");
        }
        seen[next] = {fn, dev, smem, block, occ};
        next = (next + 1) % 16;
        *blocks_per_sm = occ;
        return VG_OK;
    }

    static int ensure_stage(vg_env *e, size_t bytes)
    {
        if (bytes <= e->stage_cap)
        {
            return VG_OK;
        }
        if (e->d_stage)
        {
            cudaFree(e->d_stage);
            e->d_stage = nullptr;
            e->stage_cap = 0;
        }
        VG_CUDA(cudaMalloc(&e->d_stage, bytes), "cudaMalloc(staging)");
        e->stage_cap = bytes;
        return VG_OK;
    }

    static int ensure_pinned(vg_env *e, size_t bytes)
    {
        if (bytes <= e->pin_cap)
        {
            return VG_OK;
        }
        if (e->h_pin)
        {
            cudaFreeHost(e->h_pin);
            e->h_pin = nullptr;
            e->pin_cap = 0;
        }
        VG_CUDA(cudaMallocHost(&e->h_pin, bytes), "cudaMallocHost(staging)");
        e->pin_cap = bytes;
        return VG_OK;
    }

    // Blocks of a host batch above which the batch goes to the edge kernels.
    constexpr size_t kSmallBlocks = 4096;

    // A small host batch of edges checked block by block.  Every block of every edge is built on
    // the host with the edge kernels' arithmetic (the length summed in the x86 order and rounded
    // once, n = max(ceil(length / W * resolution), 1), block 0 at fractions (k + 1) / W of the
    // edge, block i = block 0 minus i steps of v / (W n), planning/validate.hh:24-56), the blocks
    // go to the caller-given-blocks kernel in one launch, and an edge is valid when all of its
    // blocks are: the verdicts of the edge kernels, which stop at the first colliding block.  All
    // blocks of an edge run at once, where the edge kernels give one warp the whole edge, which
    // is what the latency of a single edge (a planner's extension step) needs.  dist == nullptr:
    // b holds goals (validate_motion), otherwise motion vectors and dist the lengths
    // (validate_vector).  *handled = 0 when the batch has more than kSmallBlocks blocks.
    static int small_motions(const RobotOps *r, vg_env *env, const float *a, const float *b, const float *dist, size_t n,
                             int resolution, uint8_t *out, int *handled)
    {
        *handled = 0;
        const int W = env->lanes, D = r->dim;
        if (n > kSmallBlocks)
            return VG_OK;
        std::vector<int> nb(n);
        size_t total = 0;
        float v[32];
        for (size_t e = 0; e < n; ++e)
        {
            float len;
            if (dist)
            {
                len = dist[e];
            }
            else
            {
                // |b - a| as the edge kernels compute it (edge_length)
                float sq[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
                for (int d = 0; d < D; ++d)
                {
                    const float vd = b[e * D + d] - a[e * D + d];
                    const float q2 = vd * vd;
                    sq[d & 7] = d < 8 ? q2 : sq[d & 7] + q2;
                }
                const float a0 = sq[4] + sq[0], a1 = sq[5] + sq[1], a2 = sq[6] + sq[2], a3 = sq[7] + sq[3];
                len = std::sqrt((a0 + a2) + (a1 + a3));
            }
            const float nf = std::ceil((len / static_cast<float>(W)) * static_cast<float>(resolution));
            if (nf > static_cast<float>(kSmallBlocks))
                return VG_OK;
            nb[e] = static_cast<int>(nf > 1.0f ? nf : 1.0f);
            total += static_cast<size_t>(nb[e]);
            if (total > kSmallBlocks)
                return VG_OK;
        }
        const size_t qb = total * W * D * sizeof(float);
        const size_t qa = (qb + 255) & ~size_t(255);
        if (int rc = ensure_pinned(env, qa + total))
            return rc;
        if (int rc = ensure_stage(env, qa + total))
            return rc;
        float *hq = static_cast<float *>(env->h_pin);
        uint8_t *hv = static_cast<uint8_t *>(env->h_pin) + qa;
        float q[8][32], bs[32];
        size_t blk = 0;
        for (size_t e = 0; e < n; ++e)
        {
            for (int d = 0; d < D; ++d)
                v[d] = dist ? b[e * D + d] : b[e * D + d] - a[e * D + d];
            const float denom = static_cast<float>(W * nb[e]);
            for (int d = 0; d < D; ++d)
                bs[d] = v[d] / denom;
            for (int k = 0; k < W; ++k)
            {
                const float pct = static_cast<float>(k + 1) / static_cast<float>(W);
                for (int d = 0; d < D; ++d)
                    q[k][d] = std::fma(v[d], pct, a[e * D + d]);
            }
            for (int i = 0; i < nb[e]; ++i, ++blk)
            {
                for (int k = 0; k < W; ++k)
                {
                    for (int d = 0; d < D; ++d)
                    {
                        hq[(blk * W + k) * D + d] = q[k][d];
                        q[k][d] = q[k][d] - bs[d];
                    }
                }
            }
        }
        float *dq = static_cast<float *>(env->d_stage);
        uint8_t *dv = static_cast<uint8_t *>(env->d_stage) + qa;
        VG_CUDA(cudaMemcpyAsync(dq, hq, qb, cudaMemcpyHostToDevice, 0), "copy configuration blocks");
        if (int rc = vg_fkcc_blocks_device(r->name, env, dq, total, dv, nullptr))
            return rc;
        VG_CUDA(cudaMemcpyAsync(hv, dv, total, cudaMemcpyDeviceToHost, 0), "copy block verdicts");
        VG_CUDA(cudaStreamSynchronize(0), "synchronize");
        blk = 0;
        for (size_t e = 0; e < n; ++e)
        {
            uint8_t ok = 1;
            for (int i = 0; i < nb[e]; ++i)
                ok &= hv[blk + i];
            out[e] = ok;
            blk += static_cast<size_t>(nb[e]);
        }
        *handled = 1;
        return VG_OK;
    }

    void tuned_for(const vg_env *env, const RobotOps *r, int *schedule, int *blocks_per_sm)
    {
        *schedule = env->schedule >= 0 ? env->schedule : r->default_schedule;
        *blocks_per_sm = 0;
        for (const RobotTune &t : env->tuned)
        {
            if (t.robot == r)
            {
                *schedule = t.schedule;
                *blocks_per_sm = t.blocks_per_sm;
            }
        }
    }

    int launch_motions(const MotionLaunch &m, cudaStream_t s)
    {
        const RobotOps *r = m.r;
        const vg_env *env = m.env;
        const int smem = static_cast<int>(staged_f4(static_cast<int>(env->image_f4)) * sizeof(float4)) + r->stage_floats * kBlock * 4;
        const int which = env->lanes == 8 ? 0 : 1;
        // with heightfields or an attachment every schedule runs the extended checks in the
        // segment-per-edge kernel (the block order does not change verdicts, so a learned order
        // is not needed there)
        const bool ext = env->extended();
        const bool learned = !ext && m.scores != nullptr;
        const bool grouped = !ext && (learned || m.schedule >= 1);
        const bool wide = grouped && !learned && m.schedule == 2;
        const bool packed = grouped && !learned && m.schedule == 3;
        const void *fn = ext ? r->edges_ext_fn[which]
                             : learned ? r->edges_learned_fn[which]
                             : packed  ? r->edges_packed_fn[which]
                                       : (wide ? r->edges_wide_fn[which] : (grouped ? r->edges_grouped_fn[which] : r->edges_fn[which]));
        int occ = 0;
        if (int rc = prepare_kernel(fn, smem, kBlock, &occ))
            return rc;
        if (m.blocks_per_sm > 0 && m.blocks_per_sm < occ)
            occ = m.blocks_per_sm;
        VG_CUDA(cudaMemsetAsync(m.counter, 0, sizeof(unsigned), s), "reset work counter");
        // edges handled at once by one block of threads: a warp each (same-edge schedule) or a
        // segment each
        const int per_block = grouped ? kBlock / 32 : kBlock / env->lanes;
        const long long want = (static_cast<long long>(m.n) + per_block - 1) / per_block;
        const int grid = static_cast<int>(std::min<long long>(want, static_cast<long long>(sm_count()) * occ));
        EdgesParams p{m.a, m.b, static_cast<int>(m.n), m.resolution, m.out, m.blocks, m.counter, env_device(env), m.scores, m.probes,
                      m.dist, m.order};
        if (learned)
        {
            // each edge's group order first (one warp per edge), on the same stream
            if (!m.order)
            {
                return set_error(VG_ERR_STATE, "learned-order check without an order buffer");
            }
            const long long owant = (static_cast<long long>(m.n) + kBlock / 32 - 1) / (kBlock / 32);
            const int ogrid = static_cast<int>(std::min<long long>(owant, static_cast<long long>(sm_count()) * 16));
            VG_CUDA(r->edge_order[which](p, ogrid, kBlock, 0, s), "edge order kernel launch");
        }
        const auto launch = ext ? r->edges_ext[which]
                                : learned ? r->edges_learned[which]
                                : packed  ? r->edges_packed[which]
                                          : (wide ? r->edges_wide[which] : (grouped ? r->edges_grouped[which] : r->edges[which]));
        VG_CUDA(launch(p, grid, kBlock, smem, s), "edges kernel launch");
        return VG_OK;
    }

    // ------------------------------------------------------------ allocation-free variant
    //
    // Scratch for vg_validate_motions_device_noalloc: the edge kernel's work counter lives in
    // this fixed array instead of memory the library allocates.  Every GPU that loads the
    // library holds these bytes until the process exits.  All calls share it: the counter is
    // cleared on the caller's stream before each launch, and calls whose kernels overlap on the
    // GPU race on it.
    constexpr size_t kNoAllocScratchBytes = 256;
    static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
    static_assert(sizeof(unsigned) <= kNoAllocScratchBytes, "the work counter must fit the scratch array");

    // Device address of the scratch array on each device, looked up once per device with that
    // device current (host code cannot use the array's name as a device pointer).
    constexpr int kMaxDevices = 64;
    static void *g_noalloc_ptr[kMaxDevices] = {};
    static std::mutex g_noalloc_mu;

    static int noalloc_scratch(int dev, void **out)
    {
        if (dev < 0 || dev >= kMaxDevices)
        {
            return set_error(VG_ERR_LIMIT, "vg_validate_motions_device_noalloc: device index above 63");
        }
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_ptr[dev])
        {
            void *ptr = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
            if (e != cudaSuccess || !ptr)
            {
                return cuda_fail(e == cudaSuccess ? cudaErrorInvalidSymbol : e, "cudaGetSymbolAddress(scratch)");
            }
            g_noalloc_ptr[dev] = ptr;
        }
        *out = g_noalloc_ptr[dev];
        return VG_OK;
    }
}  // namespace vg

using namespace vg;

extern "C" {

const char *vg_last_error(void)
{
    return g_error.c_str();
}

const char *vg_version(void)
{
    return "vamp_gb300 0.1 (sm_103a)";
}

int vg_robot_info(const char *robot, int *dim, int *n_spheres, float *r_min, float *r_max, int *resolution)
{
    const RobotOps *r = find_robot(robot);
    if (!r)
    {
        return set_error(VG_ERR_ARG, std::string("unknown robot: ") + (robot ? robot : "(null)"));
    }
    if (dim)
        *dim = r->dim;
    if (n_spheres)
        *n_spheres = r->fine;
    if (r_min)
        *r_min = r->r_min;
    if (r_max)
        *r_max = r->r_max;
    if (resolution)
        *resolution = r->resolution;
    return VG_OK;
}

int vg_robot_limits(const char *robot, float *s_m, float *s_a)
{
    const RobotOps *r = find_robot(robot);
    if (!r || !s_m || !s_a)
    {
        return set_error(VG_ERR_ARG, "vg_robot_limits: unknown robot or null output");
    }
    std::memcpy(s_m, r->s_m, sizeof(float) * r->dim);
    std::memcpy(s_a, r->s_a, sizeof(float) * r->dim);
    return VG_OK;
}

vg_env *vg_env_create(void)
{
    try
    {
        return new vg_env();
    }
    catch (...)
    {
        set_error(VG_ERR_NOMEM, "vg_env_create: out of memory");
        return nullptr;
    }
}

void vg_env_destroy(vg_env *env)
{
    if (!env)
    {
        return;
    }
    if (env->d_image)
        cudaFree(env->d_image);
    if (env->d_counter)
        cudaFree(env->d_counter);
    if (env->d_stage)
        cudaFree(env->d_stage);
    if (env->d_order)
        cudaFree(env->d_order);
    if (env->h_pin)
        cudaFreeHost(env->h_pin);
    for (void *p : env->d_clouds)
        cudaFree(p);
    for (void *p : env->d_hf)
        cudaFree(p);
    delete env;
}

int vg_env_add_sphere(vg_env *env, const float *f)
{
    if (!env || !f)
        return set_error(VG_ERR_ARG, "vg_env_add_sphere: null argument");
    float row[5] = {f[0], f[1], f[2], f[3], 0.0f};
    row[4] = sphere_min_distance(f);
    insert_sorted(env, 0, 4, row);
    env->dirty = true;
    return VG_OK;
}

int vg_env_add_capsule(vg_env *env, const float *f)
{
    if (!env || !f)
        return set_error(VG_ERR_ARG, "vg_env_add_capsule: null argument");
    float row[9];
    std::memcpy(row, f, sizeof(float) * 8);
    row[8] = capsule_min_distance(f);
    insert_sorted(env, (f[3] == 0.0f && f[4] == 0.0f) ? 2 : 1, 8, row);
    env->dirty = true;
    return VG_OK;
}

int vg_env_add_cuboid(vg_env *env, const float *f)
{
    if (!env || !f)
        return set_error(VG_ERR_ARG, "vg_env_add_cuboid: null argument");
    float row[16];
    std::memcpy(row, f, sizeof(float) * 15);
    row[15] = cuboid_min_distance(f);
    insert_sorted(env, f[11] == 1.0f ? 4 : 3, 15, row);
    env->dirty = true;
    return VG_OK;
}

int vg_env_add_primitive(vg_env *env, int kind, const float *fields, float min_distance)
{
    if (!env || !fields || kind < 0 || kind > 4)
        return set_error(VG_ERR_ARG, "vg_env_add_primitive: kind must be 0..4 and fields non-null");
    float row[16];
    std::memcpy(row, fields, sizeof(float) * kFields[kind]);
    row[kFields[kind]] = min_distance;
    insert_sorted(env, kind, kFields[kind], row);
    env->dirty = true;
    return VG_OK;
}

int vg_env_add_pointcloud_layout(vg_env *env, int nlog2, const float *tests, const float *aabbs, const uint32_t *aff_starts,
                                 const float *aff, size_t n_blocks, const float *top, float r_min, float r_max, float r_point)
{
    if (!env || nlog2 < 1 || nlog2 > 30 || !tests || !aabbs || !aff_starts || !top || (n_blocks && !aff) ||
        !(r_min >= 0.0f) || !(r_max >= r_min) || !(r_point >= 0.0f))
        return set_error(VG_ERR_ARG, "vg_env_add_pointcloud_layout: bad argument");
    if (env->clouds.size() >= static_cast<size_t>(kMaxClouds))
        return set_error(VG_ERR_LIMIT, "vg_env_add_pointcloud_layout: at most 4 pointclouds per environment");
    if (n_blocks > 0xffffffffu)
        return set_error(VG_ERR_LIMIT, "vg_env_add_pointcloud_layout: more than 2^32 - 1 blocks");
    const size_t leaves = size_t{1} << nlog2;
    // every leaf's block range must lie inside the blocks given (the queries read [start, end))
    if (aff_starts[0] > aff_starts[leaves] || aff_starts[leaves] != n_blocks)
        return set_error(VG_ERR_ARG, "vg_env_add_pointcloud_layout: aff_starts[leaves] must equal n_blocks");
    for (size_t i = 0; i < leaves; ++i)
    {
        if (aff_starts[i] > aff_starts[i + 1])
            return set_error(VG_ERR_ARG, "vg_env_add_pointcloud_layout: aff_starts must not decrease");
    }
    try
    {
        CaptHost c;
        c.nlog2 = nlog2;
        c.tests.assign(tests, tests + (leaves - 1));
        c.aabbs.assign(aabbs, aabbs + leaves * 6);
        c.aff_starts.assign(aff_starts, aff_starts + leaves + 1);
        c.aff.assign(aff, aff + n_blocks * 24);
        std::memcpy(c.top, top, sizeof(c.top));
        c.r_min = r_min;
        c.r_max = r_max;
        c.r_point = r_point;
        env->clouds.push_back(std::move(c));
    }
    catch (...)
    {
        return set_error(VG_ERR_NOMEM, "vg_env_add_pointcloud_layout: out of host memory");
    }
    env->dirty = true;
    return VG_OK;
}

int vg_env_add_pointcloud(vg_env *env, const float *xyz, size_t n, float r_min, float r_max, float r_point)
{
    if (!env || !xyz || n < 2 || !(r_min >= 0.0f) || !(r_max >= r_min) || !(r_point >= 0.0f))
        return set_error(VG_ERR_ARG, "vg_env_add_pointcloud: need at least 2 points and 0 <= r_min <= r_max, r_point >= 0");
    if (env->clouds.size() >= static_cast<size_t>(kMaxClouds))
        return set_error(VG_ERR_LIMIT, "vg_env_add_pointcloud: at most 4 pointclouds per environment");
    if (n > (size_t{1} << 30))
        return set_error(VG_ERR_LIMIT, "vg_env_add_pointcloud: at most 2^30 points");
    try
    {
        CaptHost c;
        capt_build(xyz, n, r_min, r_max, r_point, c);
        env->clouds.push_back(std::move(c));
    }
    catch (...)
    {
        return set_error(VG_ERR_NOMEM, "vg_env_add_pointcloud: out of host memory");
    }
    env->dirty = true;
    return VG_OK;
}

// Same tree as vg_env_add_pointcloud, built on the current GPU from device points xyz[n][3]
// (synchronous on `stream`).  The environment must be used on this GPU.
int vg_env_add_pointcloud_device(vg_env *env, const float *xyz, size_t n, float r_min, float r_max, float r_point,
                                 void *stream)
{
    if (!env || !xyz || n < 2 || !(r_min >= 0.0f) || !(r_max >= r_min) || !(r_point >= 0.0f))
        return set_error(VG_ERR_ARG, "vg_env_add_pointcloud_device: need at least 2 points and 0 <= r_min <= r_max, r_point >= 0");
    if (env->clouds.size() >= static_cast<size_t>(kMaxClouds))
        return set_error(VG_ERR_LIMIT, "vg_env_add_pointcloud_device: at most 4 pointclouds per environment");
    if (n > (size_t{1} << 30))
        return set_error(VG_ERR_LIMIT, "vg_env_add_pointcloud_device: at most 2^30 points");
    int dev = 0;
    VG_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (env->device >= 0 && env->device != dev)
        return set_error(VG_ERR_STATE, "vg_env_add_pointcloud_device: the environment lives on another device");
    // earlier host-built clouds go up first, so that the device buffers stay in cloud order
    if (int rc = upload_clouds(env))
        return rc;
    DeviceCapt d;
    if (int rc = capt_build_device(xyz, n, r_min, r_max, r_point, static_cast<cudaStream_t>(stream), d))
        return rc;
    CaptQuery q;
    if (int rc = capt_query_layout(d.tests, d.nlog2, d.aabbs, d.starts, d.aff, d.blocks, r_max, r_point, q))
    {
        d.release();
        return rc;
    }
    CaptHost c;
    c.nlog2 = d.nlog2;
    std::memcpy(c.top, d.top, sizeof(c.top));
    c.r_min = r_min;
    c.r_max = r_max;
    c.r_point = r_point;
    c.on_device = true;
    c.device_blocks = d.blocks;
    env->clouds.push_back(std::move(c));
    env->d_clouds.push_back(d.tests);
    env->d_clouds.push_back(d.aabbs);
    env->d_clouds.push_back(d.starts);
    env->d_clouds.push_back(d.aff);  // reference layout, kept for vg_env_pointcloud_layout
    env->d_clouds.push_back(q.aff_q);
    env->d_clouds.push_back(q.tables);
    env->capt_q.push_back(q);
    env->device = dev;
    env->dirty = true;
    return VG_OK;
}

int vg_env_pointcloud_layout(const vg_env *env, int index, uint64_t *sizes, float *tests, float *aabbs,
                             uint32_t *aff_starts, float *aff, float *top)
{
    if (!env || !sizes || index < 0 || static_cast<size_t>(index) >= env->clouds.size())
        return set_error(VG_ERR_ARG, "vg_env_pointcloud_layout: bad argument");
    const CaptHost &c = env->clouds[index];
    sizes[0] = static_cast<uint64_t>(c.nlog2);
    sizes[1] = c.n_tests();
    sizes[2] = c.n_leaves();
    sizes[3] = c.blocks();
    if (c.on_device)
    {
        // the arrays live on the GPU that built them
        void *const *d = &env->d_clouds[kCloudBuffers * static_cast<size_t>(index)];
        const size_t bytes[4] = {sizes[1] * sizeof(float), sizes[2] * 6 * sizeof(float), (sizes[2] + 1) * sizeof(uint32_t),
                                 sizes[3] * 24 * sizeof(float)};
        void *dst[4] = {tests, aabbs, aff_starts, aff};
        for (int k = 0; k < 4; ++k)
        {
            if (dst[k] && bytes[k])
                VG_CUDA(cudaMemcpy(dst[k], d[k], bytes[k], cudaMemcpyDeviceToHost), "vg_env_pointcloud_layout: copy");
        }
        if (top)
            std::memcpy(top, c.top, sizeof(c.top));
        return VG_OK;
    }
    if (tests)
        std::memcpy(tests, c.tests.data(), c.tests.size() * sizeof(float));
    if (aabbs)
        std::memcpy(aabbs, c.aabbs.data(), c.aabbs.size() * sizeof(float));
    if (aff_starts)
        std::memcpy(aff_starts, c.aff_starts.data(), c.aff_starts.size() * sizeof(uint32_t));
    if (aff)
        std::memcpy(aff, c.aff.data(), c.aff.size() * sizeof(float));
    if (top)
        std::memcpy(top, c.top, sizeof(c.top));
    return VG_OK;
}

int vg_env_set_mode(vg_env *env, int lanes, int sqrt_mode)
{
    if (!env)
        return set_error(VG_ERR_ARG, "vg_env_set_mode: null environment");
    if ((lanes != 8 && lanes != 4) || (sqrt_mode != VG_SQRT_X86 && sqrt_mode != VG_SQRT_EXACT))
    {
        return set_error(VG_ERR_ARG, "vg_env_set_mode: lanes must be 8 or 4 and sqrt_mode VG_SQRT_X86 or VG_SQRT_EXACT");
    }
    env->lanes = lanes;
    env->sqrt_mode = sqrt_mode;
    return VG_OK;
}

int vg_env_set_schedule(vg_env *env, int schedule)
{
    if (!env || schedule < -1 || schedule > 3)
        return set_error(VG_ERR_ARG, "vg_env_set_schedule: schedule must be -1, 0, 1, 2 or 3");
    env->schedule = schedule;
    env->tuned.clear();
    return VG_OK;
}

int vg_env_count(const vg_env *env, int kind, size_t *count)
{
    if (!env || kind < 0 || kind > 4 || !count)
        return set_error(VG_ERR_ARG, "vg_env_count: bad argument");
    *count = env->obj[kind].size() / (kFields[kind] + 1);
    return VG_OK;
}

int vg_env_get(const vg_env *env, int kind, size_t index, float *out)
{
    if (!env || kind < 0 || kind > 4 || !out)
        return set_error(VG_ERR_ARG, "vg_env_get: bad argument");
    const size_t w = kFields[kind] + 1;
    if (index >= env->obj[kind].size() / w)
        return set_error(VG_ERR_ARG, "vg_env_get: index out of range");
    std::memcpy(out, &env->obj[kind][index * w], sizeof(float) * w);
    return VG_OK;
}

int vg_validate_states_device(const char *robot, vg_env *env, const float *q, size_t n, uint8_t *out, void *stream)
{
    const RobotOps *r = find_robot(robot);
    if (!r || !env || (n && (!q || !out)))
        return set_error(VG_ERR_ARG, "vg_validate_states_device: bad argument");
    if (n == 0)
        return VG_OK;
    if (int rc = commit(env))
        return rc;
    const int smem = static_cast<int>(staged_f4(static_cast<int>(env->image_f4)) * sizeof(float4)) + r->stage_floats * kBlock * 4;
    const bool ext = env->extended();
    int occ = 0;
    if (int rc = prepare_kernel(ext ? r->states_ext_fn : r->states_fn, smem, kBlock, &occ))
        return rc;
    const long long want = (static_cast<long long>(n) + kBlock - 1) / kBlock;
    const int grid = static_cast<int>(std::min<long long>(want, static_cast<long long>(sm_count()) * occ));
    StatesParams p{q, static_cast<long long>(n), out, env_device(env)};
    VG_CUDA((ext ? r->states_ext : r->states)(p, grid, kBlock, smem, static_cast<cudaStream_t>(stream)),
            "states kernel launch");
    return VG_OK;
}

int vg_env_add_heightfield(vg_env *env, const float *centre, const float *scale, size_t xd, size_t yd, const float *data)
{
    if (!env || !centre || !scale || !data || xd == 0 || yd == 0)
        return set_error(VG_ERR_ARG, "vg_env_add_heightfield: null argument or empty grid");
    if (env->hf.size() >= static_cast<size_t>(kMaxHeightfields))
        return set_error(VG_ERR_LIMIT, "vg_env_add_heightfield: at most 8 heightfields per environment");
    if (xd * yd >= (size_t{1} << 24))
        return set_error(VG_ERR_LIMIT, "vg_env_add_heightfield: at most 2^24 samples (cell indices are exact in FP32)");
    HeightView v{};
    v.x = centre[0];
    v.y = centre[1];
    v.z = centre[2];
    // heightfield::flat stores the inverted scales (collision/factory.hh:376-385)
    v.xs = 1.0f / scale[0];
    v.ys = 1.0f / scale[1];
    v.zs = 1.0f / scale[2];
    v.xd = static_cast<int>(xd);
    v.yd = static_cast<int>(yd);
    v.id = env->n_added++;
    env->hf.push_back(v);
    env->hf_data.emplace_back(data, data + xd * yd);
    env->dirty = true;
    return VG_OK;
}

int vg_env_add_heightfield_fields(vg_env *env, const float *fields6, size_t xd, size_t yd, const float *data)
{
    if (!env || !fields6 || !data || xd == 0 || yd == 0)
        return set_error(VG_ERR_ARG, "vg_env_add_heightfield_fields: null argument or empty grid");
    if (env->hf.size() >= static_cast<size_t>(kMaxHeightfields))
        return set_error(VG_ERR_LIMIT, "vg_env_add_heightfield_fields: at most 8 heightfields per environment");
    if (xd >= (size_t{1} << 24) || yd >= (size_t{1} << 24) || xd * yd >= (size_t{1} << 24))
        return set_error(VG_ERR_LIMIT, "vg_env_add_heightfield_fields: at most 2^24 samples (cell indices are exact in FP32)");
    HeightView v{};
    v.x = fields6[0];
    v.y = fields6[1];
    v.z = fields6[2];
    v.xs = fields6[3];
    v.ys = fields6[4];
    v.zs = fields6[5];
    v.xd = static_cast<int>(xd);
    v.yd = static_cast<int>(yd);
    v.id = env->n_added++;
    env->hf.push_back(v);
    env->hf_data.emplace_back(data, data + xd * yd);
    env->dirty = true;
    return VG_OK;
}

int vg_env_attach(vg_env *env, const float *tf16, const float *spheres, size_t k)
{
    if (!env || !tf16 || (k && !spheres))
        return set_error(VG_ERR_ARG, "vg_env_attach: null argument");
    if (k > static_cast<size_t>(VG_MAX_ATTACH_SPHERES))
        return set_error(VG_ERR_LIMIT, "vg_env_attach: at most 64 spheres per attachment");
    env->att.assign(tf16, tf16 + 12);  // rows 0..2 of the row-major 4x4 transform
    env->att.insert(env->att.end(), spheres, spheres + 4 * k);
    env->n_att = static_cast<int>(k);
    env->dirty = true;
    return VG_OK;
}

int vg_env_detach(vg_env *env)
{
    if (!env)
        return set_error(VG_ERR_ARG, "vg_env_detach: null argument");
    env->att.clear();
    env->n_att = -1;
    env->dirty = true;
    return VG_OK;
}

int vg_eefk_device(const char *robot, const float *q, size_t n, float *out, void *stream)
{
    const RobotOps *r = find_robot(robot);
    if (!r || (n && (!q || !out)))
        return set_error(VG_ERR_ARG, "vg_eefk_device: bad argument");
    VG_CUDA(r->ee_pose(q, static_cast<long long>(n), out, static_cast<cudaStream_t>(stream)), "eefk kernel launch");
    return VG_OK;
}

int vg_eefk(const char *robot, const float *q, size_t n, float *out)
{
    const RobotOps *r = find_robot(robot);
    if (!r || (n && (!q || !out)))
        return set_error(VG_ERR_ARG, "vg_eefk: bad argument");
    if (n == 0)
        return VG_OK;
    float *d = nullptr;
    const size_t in_bytes = n * r->dim * sizeof(float), out_bytes = n * 16 * sizeof(float);
    VG_CUDA(cudaMalloc(&d, in_bytes + out_bytes), "vg_eefk: cudaMalloc");
    cudaError_t e = cudaMemcpy(d, q, in_bytes, cudaMemcpyHostToDevice);
    float *d_out = d + n * r->dim;
    if (e == cudaSuccess)
        e = r->ee_pose(d, static_cast<long long>(n), d_out, nullptr);
    if (e == cudaSuccess)
        e = cudaMemcpy(out, d_out, out_bytes, cudaMemcpyDeviceToHost);
    cudaFree(d);
    VG_CUDA(e, "vg_eefk");
    return VG_OK;
}

int vg_validate_motions_device(
    const char *robot,
    vg_env *env,
    const float *a,
    const float *b,
    size_t n,
    int resolution,
    uint8_t *out,
    int32_t *blocks,
    void *stream)
{
    const RobotOps *r = find_robot(robot);
    if (!r || !env || (n && (!a || !b || !out)) || resolution < 1)
        return set_error(VG_ERR_ARG, "vg_validate_motions_device: bad argument");
    if (n > 0x7fffffffu)
        return set_error(VG_ERR_LIMIT, "vg_validate_motions_device: more than 2^31 - 1 edges");
    if (n == 0)
        return VG_OK;
    if (int rc = commit(env))
        return rc;
    MotionLaunch m{r, env, a, b, n, resolution, nullptr, 0, out, blocks, env->d_counter};
    tuned_for(env, r, &m.schedule, &m.blocks_per_sm);
    return launch_motions(m, static_cast<cudaStream_t>(stream));
}

// planning::validate_vector<Robot, lanes, resolution> (planning/validate.hh:23-63) for a batch:
// edge e starts at start[e], moves by vector[e], and is checked in max(ceil(distance[e] / lanes
// * resolution), 1) blocks, whatever the vector's length (the reference's planners pass the
// extension length they chose).  Same schedules and outputs as vg_validate_motions_device.
int vg_validate_vectors_device(
    const char *robot,
    vg_env *env,
    const float *start,
    const float *vector,
    const float *distance,
    size_t n,
    int resolution,
    uint8_t *out,
    int32_t *blocks,
    void *stream)
{
    const RobotOps *r = find_robot(robot);
    if (!r || !env || (n && (!start || !vector || !distance || !out)) || resolution < 1)
        return set_error(VG_ERR_ARG, "vg_validate_vectors_device: bad argument");
    if (n > 0x7fffffffu)
        return set_error(VG_ERR_LIMIT, "vg_validate_vectors_device: more than 2^31 - 1 edges");
    if (n == 0)
        return VG_OK;
    if (int rc = commit(env))
        return rc;
    MotionLaunch m{r, env, start, vector, n, resolution, nullptr, 0, out, blocks, env->d_counter};
    m.dist = distance;
    tuned_for(env, r, &m.schedule, &m.blocks_per_sm);
    return launch_motions(m, static_cast<cudaStream_t>(stream));
}

// Same verdicts as vg_validate_motions_device, with each edge's blocks checked in the order its
// collision scores rank them (scores[e * probes + p]: any monotone collision score of the state at
// fraction (p + 0.5) / probes along edge e, e.g. an MLP's logit).  The order is a permutation of
// the edge's blocks, so the verdict is the AND over the same states; only the number of blocks
// checked before a colliding edge stops (written to `blocks`) changes.  Always the same-edge
// schedule.
int vg_validate_motions_scored_device(
    const char *robot,
    vg_env *env,
    const float *a,
    const float *b,
    size_t n,
    int resolution,
    const float *scores,
    int probes,
    uint8_t *out,
    int32_t *blocks,
    void *stream)
{
    const RobotOps *r = find_robot(robot);
    if (!r || !env || (n && (!a || !b || !out || !scores)) || resolution < 1 || probes < 1 || probes > 32)
        return set_error(VG_ERR_ARG, "vg_validate_motions_scored_device: bad argument (probes 1..32)");
    if (n > 0x7fffffffu)
        return set_error(VG_ERR_LIMIT, "vg_validate_motions_scored_device: more than 2^31 - 1 edges");
    if (n == 0)
        return VG_OK;
    if (int rc = commit(env))
        return rc;
    if (n * 16 > env->order_cap)
    {
        if (env->d_order)
            cudaFree(env->d_order);
        env->d_order = nullptr;
        env->order_cap = 0;
        VG_CUDA(cudaMalloc(&env->d_order, n * 16), "cudaMalloc(group orders)");
        env->order_cap = n * 16;
    }
    MotionLaunch m{r, env, a, b, n, resolution, scores, probes, out, blocks, env->d_counter};
    m.order = env->d_order;
    int schedule = 1;
    tuned_for(env, r, &schedule, &m.blocks_per_sm);
    return launch_motions(m, static_cast<cudaStream_t>(stream));
}

// For callers that must not allocate GPU memory while they run, e.g. a real-time planner that
// reserves all memory up front so that no call can block on the allocator or fail for lack of
// memory mid-plan, or a host framework that owns the device memory through its own pool.  Same
// verdicts and block counts as vg_validate_motions_device; the work counter lives in the
// library's fixed scratch array.  Allocates nothing: no cudaMalloc, cudaFree or allocating
// library call.  The environment must already be uploaded to the current device by an earlier
// ordinary check call (vg_validate_motions_device, vg_validate_states_device, or their host
// forms) and not changed since.  The first call on each device looks up the scratch array's
// device address; make that first call before any stream capture.  Calls whose kernels overlap
// on the GPU race on the shared counter: issue them on one stream, or wait between them.
int vg_validate_motions_device_noalloc(
    const char *robot,
    const vg_env *env,
    const float *a,
    const float *b,
    size_t n,
    int resolution,
    uint8_t *out,
    int32_t *blocks,
    void *stream)
{
    const RobotOps *r = find_robot(robot);
    if (!r || !env || (n && (!a || !b || !out)) || resolution < 1)
        return set_error(VG_ERR_ARG, "vg_validate_motions_device_noalloc: bad argument");
    if (n > 0x7fffffffu)
        return set_error(VG_ERR_LIMIT, "vg_validate_motions_device_noalloc: more than 2^31 - 1 edges (the 32-bit work counter's limit)");
    int dev = 0;
    VG_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (!env->d_image || env->dirty || env->device != dev)
        return set_error(VG_ERR_STATE, "vg_validate_motions_device_noalloc: the environment is not uploaded to this device "
                                       "(run an ordinary check call with it first, after its last change)");
    void *scratch = nullptr;
    if (int rc = noalloc_scratch(dev, &scratch))
        return rc;
    if (n == 0)
        return VG_OK;
    MotionLaunch m{r, env, a, b, n, resolution, nullptr, 0, out, blocks, static_cast<unsigned *>(scratch)};
    tuned_for(env, r, &m.schedule, &m.blocks_per_sm);
    return launch_motions(m, static_cast<cudaStream_t>(stream));
}

int vg_sphere_fk_device(const char *robot, const float *q, size_t n, float *out, void *stream)
{
    const RobotOps *r = find_robot(robot);
    if (!r || (n && (!q || !out)))
        return set_error(VG_ERR_ARG, "vg_sphere_fk_device: bad argument");
    VG_CUDA(r->spheres(q, static_cast<long long>(n), out, static_cast<cudaStream_t>(stream)), "spheres kernel launch");
    return VG_OK;
}

int vg_validate_states(const char *robot, vg_env *env, const float *q, size_t n, uint8_t *out)
{
    const RobotOps *r = find_robot(robot);
    if (!r || !env || (n && (!q || !out)))
        return set_error(VG_ERR_ARG, "vg_validate_states: bad argument");
    if (n == 0)
        return VG_OK;
    const size_t qb = n * r->dim * sizeof(float);
    const size_t qa = (qb + 255) & ~size_t(255);
    if (int rc = ensure_stage(env, qa + n))
        return rc;
    float *dq = static_cast<float *>(env->d_stage);
    uint8_t *dout = static_cast<uint8_t *>(env->d_stage) + qa;
    VG_CUDA(cudaMemcpyAsync(dq, q, qb, cudaMemcpyHostToDevice, 0), "copy configurations");
    if (int rc = vg_validate_states_device(robot, env, dq, n, dout, nullptr))
        return rc;
    VG_CUDA(cudaMemcpyAsync(out, dout, n, cudaMemcpyDeviceToHost, 0), "copy verdicts");
    VG_CUDA(cudaStreamSynchronize(0), "synchronize");
    return VG_OK;
}

int vg_fkcc_blocks_device(const char *robot, vg_env *env, const float *q, size_t n_blocks, uint8_t *out, void *stream)
{
    const RobotOps *r = find_robot(robot);
    if (!r || !env || (n_blocks && (!q || !out)))
        return set_error(VG_ERR_ARG, "vg_fkcc_blocks_device: bad argument");
    if (n_blocks > (size_t{1} << 40))
        return set_error(VG_ERR_LIMIT, "vg_fkcc_blocks_device: more than 2^40 blocks");
    if (n_blocks == 0)
        return VG_OK;
    if (int rc = commit(env))
        return rc;
    const int which = env->lanes == 8 ? 0 : 1;
    const bool ext = env->extended();
    const int smem = static_cast<int>(staged_f4(static_cast<int>(env->image_f4)) * sizeof(float4)) + r->stage_floats * kBlock * 4;
    int occ = 0;
    if (int rc = prepare_kernel(ext ? r->blocks_ext_fn[which] : r->blocks_fn[which], smem, kBlock, &occ))
        return rc;
    const long long per_block = (kBlock / 32) * (32 / env->lanes);  // configuration blocks per thread block
    const long long want = (static_cast<long long>(n_blocks) + per_block - 1) / per_block;
    const int grid = static_cast<int>(std::min<long long>(want, static_cast<long long>(sm_count()) * occ));
    StatesParams p{q, static_cast<long long>(n_blocks), out, env_device(env)};
    VG_CUDA((ext ? r->blocks_ext[which] : r->blocks[which])(p, grid, kBlock, smem, static_cast<cudaStream_t>(stream)),
            "blocks kernel launch");
    return VG_OK;
}

int vg_fkcc_blocks(const char *robot, vg_env *env, const float *q, size_t n_blocks, uint8_t *out)
{
    const RobotOps *r = find_robot(robot);
    if (!r || !env || (n_blocks && (!q || !out)))
        return set_error(VG_ERR_ARG, "vg_fkcc_blocks: bad argument");
    if (n_blocks == 0)
        return VG_OK;
    const size_t qb = n_blocks * static_cast<size_t>(env->lanes) * r->dim * sizeof(float);
    const size_t qa = (qb + 255) & ~size_t(255);
    if (int rc = ensure_stage(env, qa + n_blocks))
        return rc;
    float *dq = static_cast<float *>(env->d_stage);
    uint8_t *dout = static_cast<uint8_t *>(env->d_stage) + qa;
    VG_CUDA(cudaMemcpyAsync(dq, q, qb, cudaMemcpyHostToDevice, 0), "copy configuration blocks");
    if (int rc = vg_fkcc_blocks_device(robot, env, dq, n_blocks, dout, nullptr))
        return rc;
    VG_CUDA(cudaMemcpyAsync(out, dout, n_blocks, cudaMemcpyDeviceToHost, 0), "copy verdicts");
    VG_CUDA(cudaStreamSynchronize(0), "synchronize");
    return VG_OK;
}

int vg_validate_motions(
    const char *robot, vg_env *env, const float *a, const float *b, size_t n, int resolution, uint8_t *out)
{
    const RobotOps *r = find_robot(robot);
    if (!r || !env || (n && (!a || !b || !out)))
        return set_error(VG_ERR_ARG, "vg_validate_motions: bad argument");
    if (n == 0)
        return VG_OK;
    if (resolution < 1)
        return set_error(VG_ERR_ARG, "vg_validate_motions: bad argument");
    if (int rc = commit(env))
        return rc;
    int handled = 0;
    if (int rc = small_motions(r, env, a, b, nullptr, n, resolution, out, &handled))
        return rc;
    if (handled)
        return VG_OK;
    const size_t cb = ((n * r->dim * sizeof(float)) + 255) & ~size_t(255);
    if (int rc = ensure_stage(env, 2 * cb + n))
        return rc;
    char *base = static_cast<char *>(env->d_stage);
    float *da = reinterpret_cast<float *>(base);
    float *db = reinterpret_cast<float *>(base + cb);
    uint8_t *dout = reinterpret_cast<uint8_t *>(base + 2 * cb);
    VG_CUDA(cudaMemcpyAsync(da, a, n * r->dim * sizeof(float), cudaMemcpyHostToDevice, 0), "copy starts");
    VG_CUDA(cudaMemcpyAsync(db, b, n * r->dim * sizeof(float), cudaMemcpyHostToDevice, 0), "copy goals");
    if (int rc = vg_validate_motions_device(robot, env, da, db, n, resolution, dout, nullptr, nullptr))
        return rc;
    VG_CUDA(cudaMemcpyAsync(out, dout, n, cudaMemcpyDeviceToHost, 0), "copy verdicts");
    VG_CUDA(cudaStreamSynchronize(0), "synchronize");
    return VG_OK;
}

int vg_validate_vectors(const char *robot, vg_env *env, const float *start, const float *vector, const float *distance,
                        size_t n, int resolution, uint8_t *out)
{
    const RobotOps *r = find_robot(robot);
    if (!r || !env || (n && (!start || !vector || !distance || !out)))
        return set_error(VG_ERR_ARG, "vg_validate_vectors: bad argument");
    if (n == 0)
        return VG_OK;
    if (resolution < 1)
        return set_error(VG_ERR_ARG, "vg_validate_vectors: bad argument");
    if (int rc = commit(env))
        return rc;
    int handled = 0;
    if (int rc = small_motions(r, env, start, vector, distance, n, resolution, out, &handled))
        return rc;
    if (handled)
        return VG_OK;
    const size_t cb = ((n * r->dim * sizeof(float)) + 255) & ~size_t(255);
    const size_t db_ = ((n * sizeof(float)) + 255) & ~size_t(255);
    if (int rc = ensure_stage(env, 2 * cb + db_ + n))
        return rc;
    char *base = static_cast<char *>(env->d_stage);
    float *ds = reinterpret_cast<float *>(base);
    float *dv = reinterpret_cast<float *>(base + cb);
    float *dd = reinterpret_cast<float *>(base + 2 * cb);
    uint8_t *dout = reinterpret_cast<uint8_t *>(base + 2 * cb + db_);
    VG_CUDA(cudaMemcpyAsync(ds, start, n * r->dim * sizeof(float), cudaMemcpyHostToDevice, 0), "copy starts");
    VG_CUDA(cudaMemcpyAsync(dv, vector, n * r->dim * sizeof(float), cudaMemcpyHostToDevice, 0), "copy vectors");
    VG_CUDA(cudaMemcpyAsync(dd, distance, n * sizeof(float), cudaMemcpyHostToDevice, 0), "copy distances");
    if (int rc = vg_validate_vectors_device(robot, env, ds, dv, dd, n, resolution, dout, nullptr, nullptr))
        return rc;
    VG_CUDA(cudaMemcpyAsync(out, dout, n, cudaMemcpyDeviceToHost, 0), "copy verdicts");
    VG_CUDA(cudaStreamSynchronize(0), "synchronize");
    return VG_OK;
}

int vg_sphere_fk(const char *robot, const float *q, size_t n, float *out)
{
    const RobotOps *r = find_robot(robot);
    if (!r || (n && (!q || !out)))
        return set_error(VG_ERR_ARG, "vg_sphere_fk: bad argument");
    if (n == 0)
        return VG_OK;
    float *dq = nullptr, *dout = nullptr;
    const size_t qb = n * r->dim * sizeof(float), ob = n * r->slots * 4 * sizeof(float);
    VG_CUDA(cudaMalloc(&dq, qb), "cudaMalloc");
    cudaError_t e = cudaMalloc(&dout, ob);
    if (e != cudaSuccess)
    {
        cudaFree(dq);
        return cuda_fail(e, "cudaMalloc");
    }
    e = cudaMemcpy(dq, q, qb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = r->spheres(dq, static_cast<long long>(n), dout, 0);
    if (e == cudaSuccess)
        e = cudaMemcpy(out, dout, ob, cudaMemcpyDeviceToHost);
    cudaFree(dq);
    cudaFree(dout);
    if (e != cudaSuccess)
        return cuda_fail(e, "vg_sphere_fk");
    return VG_OK;
}

void *vg_host_alloc(size_t bytes)
{
    void *p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess)
    {
        set_error(VG_ERR_NOMEM, "cudaMallocHost failed");
        return nullptr;
    }
    return p;
}

void vg_host_free(void *p)
{
    if (p)
        cudaFreeHost(p);
}

}  // extern "C"
