// Debug reports: Robot::fkcc_debug (robots/panda.hh:468) for a batch of configurations, the
// reference's per-sphere collision listing behind its Python binding's debug()
// (bindings/robot_helper.hh:249-253).
#include "../../include/vamp_gb300.h"
#include "vg_internal.h"

#include <algorithm>
#include <string>
#include <vector>

namespace vg
{
    struct DebugParams
    {
        const float *spheres;  // [n][slots][4]
        int slots, fine;
        long long n;
        EnvDevice env;         // the image in global memory
        const int *ids;        // insertion id of every object, kinds in order, each sorted
        int id_off[5];         // where each kind's ids start
        uint32_t *bits;        // [n][fine][words]
        int words;
    };

    template <int KIND>
    __device__ __forceinline__ void debug_kind(const EnvView &ev, const int *ids, float x, float y, float z, float r,
                                               float rsq, float me, uint32_t *bits)
    {
        const float4 *rec = ev.rec[KIND];
        for (int i = 0; i < ev.n[KIND]; ++i)
        {
            const float4 *o = rec + i * rec_f4(KIND);
            const float md = reinterpret_cast<const float *>(o)[min_d_offset(KIND)];
            if (!(__float_as_uint(__fsub_rn(md, me)) >> 31))
            {
                break;
            }
            if (__float_as_uint(prim_test<KIND>(o, x, y, z, r, rsq)) >> 31)
            {
                const int id = ids[i];
                bits[id >> 5] |= 1u << (id & 31);
            }
        }
    }

    // one thread per (configuration, fine sphere)
    __global__ void debug_env_kernel(const DebugParams p)
    {
        const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
        if (t >= p.n * p.fine)
        {
            return;
        }
        const long long c = t / p.fine;
        const int s = static_cast<int>(t - c * p.fine);
        const float *sp = p.spheres + (c * p.slots + s) * 4;
        const float x = sp[0], y = sp[1], z = sp[2], r = sp[3];
        EnvView ev;
        ev.rsqrt_tab = reinterpret_cast<const uint32_t *>(p.env.buf);
        ev.sqrt_mode = p.env.sqrt_mode;
        ev.clouds = nullptr;
        ev.n_clouds = 0;
        for (int k = 0; k < 5; ++k)
        {
            ev.rec[k] = p.env.buf + p.env.off[k];
            ev.n[k] = p.env.n[k];
        }
        uint32_t *bits = p.bits + t * p.words;
        for (int w = 0; w < p.words; ++w)
        {
            bits[w] = 0u;
        }
        const float v = __fmaf_rn(x, x, __fmaf_rn(z, z, __fmul_rn(y, y)));
        const float me = max_extent(ev, v, r);
        const float rsq = __fmul_rn(r, r);
        debug_kind<0>(ev, p.ids + p.id_off[0], x, y, z, r, rsq, me, bits);
        debug_kind<1>(ev, p.ids + p.id_off[1], x, y, z, r, rsq, me, bits);
        debug_kind<2>(ev, p.ids + p.id_off[2], x, y, z, r, rsq, me, bits);
        debug_kind<3>(ev, p.ids + p.id_off[3], x, y, z, r, rsq, me, bits);
        debug_kind<4>(ev, p.ids + p.id_off[4], x, y, z, r, rsq, me, bits);
        // heightfields (validity.hh:240-246): every one, no distance cut-off
        const HeightView *hf = reinterpret_cast<const HeightView *>(p.env.buf + p.env.hf_off);
        for (int h = 0; h < p.env.n_hf; ++h)
        {
            if (__float_as_uint(t_heightfield(hf[h], x, y, z, r)) >> 31)
            {
                bits[hf[h].id >> 5] |= 1u << (hf[h].id & 31);
            }
        }
    }

}  // namespace vg

using namespace vg;

namespace
{
    constexpr long long kDebugChunk = 65536;  // configurations per pass (sphere slots scratch)

    int debug_words(const vg_env *env)
    {
        return std::max(1, (env->n_added + 31) / 32);
    }
}  // namespace

extern "C" {

int vg_debug_sizes(const char *robot, const vg_env *env, int *fine, int *words, int *self_pairs)
{
    const RobotOps *r = find_robot(robot);
    if (!r || !env)
        return set_error(VG_ERR_ARG, "vg_debug_sizes: bad argument");
    if (fine)
        *fine = r->fine;
    if (words)
        *words = debug_words(env);
    if (self_pairs)
        *self_pairs = r->self_pairs;
    return VG_OK;
}

int vg_debug_device(const char *robot, vg_env *env, const float *q, size_t n, uint32_t *env_bits, uint8_t *pairs,
                    void *stream)
{
    const RobotOps *r = find_robot(robot);
    if (!r || !env || (n && (!q || !env_bits || !pairs)))
        return set_error(VG_ERR_ARG, "vg_debug_device: bad argument");
    if (n == 0)
        return VG_OK;
    if (int rc = commit(env))
        return rc;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // insertion ids, kinds in order, each in the image's (sorted) order
    std::vector<int> ids;
    DebugParams p{};
    for (int k = 0; k < 5; ++k)
    {
        p.id_off[k] = static_cast<int>(ids.size());
        ids.insert(ids.end(), env->ids[k].begin(), env->ids[k].end());
    }
    if (ids.empty())
        ids.push_back(0);
    const long long chunk = std::min<long long>(static_cast<long long>(n), kDebugChunk);
    int *d_ids = nullptr;
    float *d_sph = nullptr;
    cudaError_t e = cudaMalloc(&d_ids, ids.size() * sizeof(int));
    if (e == cudaSuccess)
        e = cudaMalloc(&d_sph, static_cast<size_t>(chunk) * r->slots * 4 * sizeof(float));
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_ids, ids.data(), ids.size() * sizeof(int), cudaMemcpyHostToDevice, s);
    const int words = debug_words(env);
    p.slots = r->slots;
    p.fine = r->fine;
    p.env = env_device(env);
    p.ids = d_ids;
    p.words = words;
    for (long long c0 = 0; e == cudaSuccess && c0 < static_cast<long long>(n); c0 += chunk)
    {
        const long long m = std::min<long long>(chunk, static_cast<long long>(n) - c0);
        e = r->spheres(q + c0 * r->dim, m, d_sph, s);
        if (e != cudaSuccess)
            break;
        p.spheres = d_sph;
        p.n = m;
        p.bits = env_bits + c0 * r->fine * words;
        const long long t = m * r->fine;
        debug_env_kernel<<<static_cast<unsigned>((t + 127) / 128), 128, 0, s>>>(p);
        e = cudaGetLastError();
        if (e == cudaSuccess)
            e = r->debug_self(d_sph, m, pairs + c0 * r->self_pairs, s);
    }
    // the scratch is released once the launches that read it have run
    const cudaError_t se = cudaStreamSynchronize(s);
    cudaFree(d_sph);
    cudaFree(d_ids);
    if (e != cudaSuccess || se != cudaSuccess)
        return set_error(VG_ERR_CUDA, std::string("vg_debug_device: ") + cudaGetErrorString(e != cudaSuccess ? e : se));
    return VG_OK;
}

int vg_debug(const char *robot, vg_env *env, const float *q, size_t n, uint32_t *env_bits, uint8_t *pairs)
{
    const RobotOps *r = find_robot(robot);
    if (!r || !env || (n && (!q || !env_bits || !pairs)))
        return set_error(VG_ERR_ARG, "vg_debug: bad argument");
    if (n == 0)
        return VG_OK;
    const int words = debug_words(env);
    const size_t qb = n * r->dim * sizeof(float), bb = n * r->fine * words * sizeof(uint32_t), pb = n * r->self_pairs;
    void *d = nullptr;
    if (cudaMalloc(&d, qb + bb + pb) != cudaSuccess)
        return set_error(VG_ERR_NOMEM, "vg_debug: device buffers");
    char *base = static_cast<char *>(d);
    int rc = VG_OK;
    if (cudaMemcpy(base, q, qb, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = set_error(VG_ERR_CUDA, "vg_debug: copy in");
    if (rc == VG_OK)
        rc = vg_debug_device(robot, env, reinterpret_cast<float *>(base), n, reinterpret_cast<uint32_t *>(base + qb),
                             reinterpret_cast<uint8_t *>(base + qb + bb), nullptr);
    if (rc == VG_OK && (cudaMemcpy(env_bits, base + qb, bb, cudaMemcpyDeviceToHost) != cudaSuccess ||
                        cudaMemcpy(pairs, base + qb + bb, pb, cudaMemcpyDeviceToHost) != cudaSuccess))
        rc = set_error(VG_ERR_CUDA, "vg_debug: copy out");
    cudaFree(d);
    return rc;
}

}  // extern "C"
