/* vamp_gb300_dropin.hh - the reference's hot-path C++ entry points, answered on the GPU.
 *
 * For C++ code written against the reference's headers (VAMP, src/impl/vamp): include those
 * headers first (vamp/collision/environment.hh, vamp/planning/validate.hh and the robot headers
 * you use), then this one, then declare a GPU robot per reference robot:
 *
 *     #include <vamp/robots/panda.hh>
 *     #include <vamp/planning/validate.hh>
 *     #include "vamp_gb300_dropin.hh"
 *     using GpuPanda = vamp_gb300::dropin::Robot<vamp::robots::Panda>;
 *     VAMP_GB300_DROPIN_VALIDATE(GpuPanda)
 *
 * GpuPanda is vamp::robots::Panda (it inherits every constant, type and function) except that
 *   - Robot::fkcc<rake> / fkcc_attach<rake> (robots/panda.hh:5226-5229) check the block on the
 *     GPU (vg_fkcc_blocks), and
 *   - planning::validate_motion / validate_vector<GpuPanda, rake, resolution>
 *     (planning/validate.hh:23-77), which the planners call per edge (planning/rrtc.hh:136,176,
 *     prm.hh:122,138, fcit.hh:238,333, aorrtc.hh:191,227,280), check the whole edge in one GPU call
 *     (vg_validate_vectors) instead of one fkcc call per block.  VAMP_GB300_DROPIN_VALIDATE
 *     declares these for rake = FloatVectorWidth and for the robot's resolution and resolution
 *     1 (the bindings' validate); other resolutions take the reference's validate_vector, which
 *     then calls the GPU fkcc once per block.
 * so RRTC<GpuPanda, rake, GpuPanda::resolution> and the other planners compile unchanged.
 *
 * Semantics: the reference's, bit for bit (the edge's vector and length are computed here with
 * the reference's own vector code; the GPU reproduces the rest).  The reference's backend fixes
 * the lane count: 8 lanes with the x86 square-root bound (AVX2), 4 with an exact square root
 * (NEON).  There is no CPU fallback: the answer always comes from the GPU.
 *
 * Environments: every collision::Environment<FloatVector<rake>> passed in is converted once and
 * kept on the GPU, keyed by its address and a hash of its contents (primitive fields, heightfield
 * fields and samples' identity, pointcloud trees' identity), as the reference converts its
 * float environment once per planner call (bindings/robot_helper.hh:184-185).  The most recent
 * kCacheSize environments stay resident.  Spheres, capsules (both lists), cuboids (both lists),
 * heightfields and pointclouds (the reference's trees, imported as built) are supported;
 * cylinders are never tested by the reference (collision/validity.hh has no cylinder loop) and
 * are ignored here too; an environment with an attachment is not supported (the reference poses
 * attachments with Eigen): its checks return false.
 *
 * Errors: the reference's functions are noexcept and return bool.  Here a failure (no GPU, a
 * CUDA error, an unsupported environment) makes the check return false - "not valid", the
 * conservative answer for a planner - and vg_last_error() tells why.
 *
 * Threading: the conversion cache is guarded by a mutex; GPU calls are synchronous on the
 * default stream.  The reference calls these functions from one thread.
 */
#pragma once

#include <array>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

#include "vamp_gb300.h"

namespace vamp_gb300::dropin
{
    namespace detail
    {
        // Lane 0 of a broadcast vector field (the vector environment stores every scalar field
        // broadcast to all lanes), or a plain float.
        template <typename V>
        inline float scalar(const V &v)
        {
            if constexpr (std::is_arithmetic_v<V>)
            {
                return static_cast<float>(v);
            }
            else
            {
                return v.to_array()[0];
            }
        }

        struct Hash
        {
            std::uint64_t h = 1469598103934665603ull;  // FNV-1a, 64-bit

            void bytes(const void *p, std::size_t n)
            {
                const auto *c = static_cast<const unsigned char *>(p);
                for (std::size_t i = 0; i < n; ++i)
                {
                    h = (h ^ c[i]) * 1099511628211ull;
                }
            }

            template <typename T>
            void value(const T &v)
            {
                bytes(&v, sizeof(v));
            }
        };

        // Fields of each kind, in the order the C ABI takes them.
        template <typename S>
        inline std::array<float, 4> sphere_fields(const S &s)
        {
            return {scalar(s.x), scalar(s.y), scalar(s.z), scalar(s.r)};
        }

        template <typename C>
        inline std::array<float, 8> capsule_fields(const C &c)
        {
            return {scalar(c.x1), scalar(c.y1), scalar(c.z1), scalar(c.xv), scalar(c.yv), scalar(c.zv), scalar(c.r), scalar(c.rdv)};
        }

        template <typename B>
        inline std::array<float, 15> cuboid_fields(const B &b)
        {
            return {scalar(b.x),        scalar(b.y),        scalar(b.z),        scalar(b.axis_1_x), scalar(b.axis_1_y),
                    scalar(b.axis_1_z), scalar(b.axis_2_x), scalar(b.axis_2_y), scalar(b.axis_2_z), scalar(b.axis_3_x),
                    scalar(b.axis_3_y), scalar(b.axis_3_z), scalar(b.axis_1_r), scalar(b.axis_2_r), scalar(b.axis_3_r)};
        }

        template <typename H>
        inline std::array<float, 6> heightfield_fields(const H &f)
        {
            return {scalar(f.x), scalar(f.y), scalar(f.z), scalar(f.xs), scalar(f.ys), scalar(f.zs)};
        }

        // Hash of everything the GPU copy depends on.  Pointcloud trees and heightfield samples
        // enter by identity (buffer address and size): a tree is rebuilt, not edited, when its
        // points change.
        template <typename Env>
        inline std::uint64_t content_hash(const Env &e, int lanes)
        {
            Hash h;
            h.value(lanes);
            const auto list = [&](const auto &objs, auto fields) {
                h.value(objs.size());
                for (const auto &o : objs)
                {
                    const auto f = fields(o);
                    h.bytes(f.data(), sizeof(f));
                    h.value(scalar(o.min_distance));
                }
            };
            list(e.spheres, [](const auto &o) { return sphere_fields(o); });
            list(e.capsules, [](const auto &o) { return capsule_fields(o); });
            list(e.z_aligned_capsules, [](const auto &o) { return capsule_fields(o); });
            list(e.cuboids, [](const auto &o) { return cuboid_fields(o); });
            list(e.z_aligned_cuboids, [](const auto &o) { return cuboid_fields(o); });
            h.value(e.heightfields.size());
            for (const auto &f : e.heightfields)
            {
                const auto v = heightfield_fields(f);
                h.bytes(v.data(), sizeof(v));
                h.value(f.xd);
                h.value(f.yd);
                h.value(static_cast<const void *>(f.data.data()));
                h.value(f.data.size());
            }
            h.value(e.pointclouds.size());
            for (const auto &c : e.pointclouds)
            {
                h.value(static_cast<const void *>(c.tests.data()));
                h.value(static_cast<const void *>(c.affordances[0].data()));
                h.value(c.affordances[0].size());
                h.value(c.nlog2);
            }
            h.value(static_cast<bool>(e.attachments));
            return h.h;
        }

        // A reference tree (collision/capt.hh:584-617) in the C ABI's layout.
        template <typename Capt>
        inline int add_tree(vg_env *env, const Capt &c)
        {
            const std::size_t leaves = std::size_t{1} << c.nlog2;
            const std::size_t nb = c.affordances[0].size();
            std::vector<float> aabbs(leaves * 6), aff(nb * 24);
            for (std::size_t i = 0; i < leaves && i < c.aabbs.size(); ++i)
            {
                for (int k = 0; k < 3; ++k)
                {
                    aabbs[6 * i + k] = c.aabbs[i].lower[k];
                    aabbs[6 * i + 3 + k] = c.aabbs[i].upper[k];
                }
            }
            for (std::size_t b = 0; b < nb; ++b)
            {
                for (int k = 0; k < 3; ++k)
                {
                    const auto lanes = c.affordances[k][b].to_array();
                    for (int l = 0; l < 8; ++l)
                    {
                        aff[24 * b + 8 * k + l] = lanes[l];
                    }
                }
            }
            const float top[6] = {c.aabb_top.lower[0], c.aabb_top.lower[1], c.aabb_top.lower[2],
                                  c.aabb_top.upper[0], c.aabb_top.upper[1], c.aabb_top.upper[2]};
            if (c.aabbs.size() != leaves || c.tests.size() + 1 != leaves || c.aff_starts.size() != leaves + 1)
            {
                return -1;  // VG_ERR_ARG: not a tree as the reference builds it
            }
            return vg_env_add_pointcloud_layout(env, c.nlog2, c.tests.data(), aabbs.data(), c.aff_starts.data(), aff.data(), nb,
                                                top, c.r_min, c.r_max, c.r_point);
        }

        // A new GPU environment holding e (lanes 8: the x86 build's semantics, 4: the Arm build's).
        template <typename Env>
        inline vg_env *convert(const Env &e, int lanes)
        {
            if (e.attachments)
            {
                return nullptr;
            }
            vg_env *env = vg_env_create();
            if (!env)
            {
                return nullptr;
            }
            int rc = vg_env_set_mode(env, lanes, lanes == 8 ? VG_SQRT_X86 : VG_SQRT_EXACT);
            const auto add = [&](int kind, const auto &objs, auto fields) {
                for (const auto &o : objs)
                {
                    if (rc == VG_OK)
                    {
                        const auto f = fields(o);
                        rc = vg_env_add_primitive(env, kind, f.data(), scalar(o.min_distance));
                    }
                }
            };
            add(0, e.spheres, [](const auto &o) { return sphere_fields(o); });
            add(1, e.capsules, [](const auto &o) { return capsule_fields(o); });
            add(2, e.z_aligned_capsules, [](const auto &o) { return capsule_fields(o); });
            add(3, e.cuboids, [](const auto &o) { return cuboid_fields(o); });
            add(4, e.z_aligned_cuboids, [](const auto &o) { return cuboid_fields(o); });
            for (const auto &f : e.heightfields)
            {
                if (rc == VG_OK)
                {
                    const auto v = heightfield_fields(f);
                    rc = vg_env_add_heightfield_fields(env, v.data(), f.xd, f.yd, f.data.data());
                }
            }
            for (const auto &c : e.pointclouds)
            {
                if (rc == VG_OK)
                {
                    rc = add_tree(env, c);
                }
            }
            if (rc != VG_OK)
            {
                vg_env_destroy(env);
                return nullptr;
            }
            return env;
        }

        // The GPU copies of the most recently used environments.
        class Cache
        {
        public:
            static constexpr std::size_t kCacheSize = 8;

            template <typename Env>
            vg_env *get(const Env &e, int lanes)
            {
                const std::uint64_t h = content_hash(e, lanes);
                std::lock_guard<std::mutex> lock(mu_);
                ++clock_;
                for (Entry &x : entries_)
                {
                    if (x.address == static_cast<const void *>(&e) && x.hash == h)
                    {
                        x.used = clock_;
                        return x.env;
                    }
                }
                vg_env *env = convert(e, lanes);
                if (!env)
                {
                    return nullptr;
                }
                if (entries_.size() >= kCacheSize)
                {
                    std::size_t oldest = 0;
                    for (std::size_t i = 1; i < entries_.size(); ++i)
                    {
                        oldest = entries_[i].used < entries_[oldest].used ? i : oldest;
                    }
                    vg_env_destroy(entries_[oldest].env);
                    entries_.erase(entries_.begin() + static_cast<std::ptrdiff_t>(oldest));
                }
                entries_.push_back({static_cast<const void *>(&e), h, env, clock_});
                return env;
            }

            ~Cache()
            {
                for (Entry &x : entries_)
                {
                    vg_env_destroy(x.env);
                }
            }

        private:
            struct Entry
            {
                const void *address;
                std::uint64_t hash;
                vg_env *env;
                std::uint64_t used;
            };
            std::vector<Entry> entries_;
            std::uint64_t clock_ = 0;
            std::mutex mu_;
        };

        inline Cache &cache()
        {
            static Cache c;
            return c;
        }

        template <std::size_t rake>
        inline constexpr int lanes_of()
        {
            static_assert(rake == 8 || rake == 4, "the GPU reproduces 8-lane (AVX2) and 4-lane (NEON) blocks");
            return static_cast<int>(rake);
        }

        // The first n entries of a configuration vector.
        template <typename C>
        inline void unpack(const C &c, std::size_t n, float *out)
        {
            const auto a = c.to_array();
            for (std::size_t i = 0; i < n; ++i)
            {
                out[i] = a[i];
            }
        }
    }  // namespace detail

    // A reference robot whose collision checks run on the GPU (see the top of this file).
    template <typename Base>
    struct Robot : Base
    {
        template <std::size_t rake>
        static bool fkcc(const vamp::collision::Environment<vamp::FloatVector<rake>> &environment,
                         const typename Base::template ConfigurationBlock<rake> &block) noexcept
        {
            constexpr int lanes = detail::lanes_of<rake>();
            vg_env *env = detail::cache().get(environment, lanes);
            if (!env)
            {
                return false;
            }
            // the block's rows are joints, each padded to a multiple of the vector width
            constexpr std::size_t dim = Base::dimension;
            const auto arr = block.to_array();
            constexpr std::size_t row = std::tuple_size<std::decay_t<decltype(arr)>>::value / dim;
            float q[lanes * dim];
            for (std::size_t j = 0; j < dim; ++j)
            {
                for (int l = 0; l < lanes; ++l)
                {
                    q[l * dim + j] = arr[j * row + l];
                }
            }
            std::uint8_t ok = 0;
            return vg_fkcc_blocks(Base::name, env, q, 1, &ok) == VG_OK && ok;
        }

        template <std::size_t rake>
        static bool fkcc_attach(const vamp::collision::Environment<vamp::FloatVector<rake>> &environment,
                                const typename Base::template ConfigurationBlock<rake> &block) noexcept
        {
            return fkcc<rake>(environment, block);  // environments with attachments are rejected
        }
    };

    // planning::validate_vector (planning/validate.hh:23-63) for one edge, in one GPU call.
    template <typename R, std::size_t rake, std::size_t resolution, typename Env, typename Config>
    inline bool validate_vector(const Config &start, const Config &vector, float distance, const Env &environment) noexcept
    {
        vg_env *env = detail::cache().get(environment, detail::lanes_of<rake>());
        if (!env)
        {
            return false;
        }
        float s[R::dimension], v[R::dimension];
        detail::unpack(start, R::dimension, s);
        detail::unpack(vector, R::dimension, v);
        std::uint8_t ok = 0;
        return vg_validate_vectors(R::name, env, s, v, &distance, 1, static_cast<int>(resolution), &ok) == VG_OK && ok;
    }

    // planning::validate_motion (planning/validate.hh:70-77): the edge's vector and length with
    // the reference's own vector arithmetic, then validate_vector on the GPU.
    template <typename R, std::size_t rake, std::size_t resolution, typename Env, typename Config>
    inline bool validate_motion(const Config &start, const Config &goal, const Env &environment) noexcept
    {
        const auto vector = goal - start;
        return validate_vector<R, rake, resolution>(start, vector, vector.l2_norm(), environment);
    }
}  // namespace vamp_gb300::dropin

// Explicit specializations of the reference's validate_motion / validate_vector for a GPU robot
// at the reference's lane count, for the robot's own resolution and for resolution 1.
#define VAMP_GB300_DROPIN_VALIDATE_AT(R, RES)                                                                          \
    namespace vamp::planning                                                                                           \
    {                                                                                                                  \
        template <>                                                                                                    \
        inline auto validate_vector<R, ::vamp::FloatVectorWidth, RES>(                                                 \
            const typename R::Configuration &start,                                                                    \
            const typename R::Configuration &vector,                                                                   \
            float distance,                                                                                            \
            const collision::Environment<FloatVector<::vamp::FloatVectorWidth>> &environment) -> bool                  \
        {                                                                                                              \
            return ::vamp_gb300::dropin::validate_vector<R, ::vamp::FloatVectorWidth, RES>(start, vector, distance,    \
                                                                                           environment);               \
        }                                                                                                              \
        template <>                                                                                                    \
        inline auto validate_motion<R, ::vamp::FloatVectorWidth, RES>(                                                 \
            const typename R::Configuration &start,                                                                    \
            const typename R::Configuration &goal,                                                                     \
            const collision::Environment<FloatVector<::vamp::FloatVectorWidth>> &environment) -> bool                  \
        {                                                                                                              \
            return ::vamp_gb300::dropin::validate_motion<R, ::vamp::FloatVectorWidth, RES>(start, goal, environment);  \
        }                                                                                                              \
    }

#define VAMP_GB300_DROPIN_VALIDATE(R)           \
    VAMP_GB300_DROPIN_VALIDATE_AT(R, R::resolution) \
    VAMP_GB300_DROPIN_VALIDATE_AT(R, 1)
