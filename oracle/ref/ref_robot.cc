// Per-robot C ABI over the reference's generated robot kernels and its motion validator, compiled
// from the reference sources in place (test infrastructure only).  Built once per robot with
//   -DVGREF_ROBOT=<C++ type>  -DVGREF_NAME=<symbol prefix>  -DVGREF_HEADER=<robots/xxx.hh>
//
// Wrapped reference interfaces:
//   Robot::fkcc<rake>                      robots/panda.hh:5227 (ur5.hh:3218, fetch.hh:17185, baxter.hh:12710)
//   Robot::sphere_fk<rake>                 robots/panda.hh:117
//   planning::validate_motion<R, rake, res> planning/validate.hh:70-77
#include "ref_common.hh"

#include VGREF_HEADER

#include <atomic>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#define VG_CAT2(a, b) a##b
#define VG_CAT(a, b) VG_CAT2(a, b)
#define VG_FN(suffix) VG_CAT(VG_CAT(vgref_, VGREF_NAME), suffix)

using namespace vamp;
using Robot = vamp::robots::VGREF_ROBOT;
constexpr std::size_t kRake = FloatVectorWidth;
using Block = Robot::ConfigurationBlock<kRake>;

namespace
{
    // A stand-in robot whose fkcc only records the blocks that validate_vector hands it.  Driving
    // the reference's own validate_motion with it exposes the exact interpolated states and the
    // order in which the reference visits them (planning/validate.hh:24-67).
    struct Recorder
    {
        static constexpr std::size_t dimension = Robot::dimension;
        using Configuration = Robot::Configuration;
        template <std::size_t rake>
        using ConfigurationBlock = Robot::ConfigurationBlock<rake>;

        static thread_local float *out;
        static thread_local std::size_t cap;
        static thread_local std::size_t count;
        static thread_local long fail_at;

        template <std::size_t rake>
        static bool fkcc(const collision::Environment<FloatVector<rake>> &, const ConfigurationBlock<rake> &b) noexcept
        {
            if (count < cap)
            {
                const auto arr = b.to_array();
                // rows are joints, each row padded to a multiple of the lane count
                constexpr std::size_t row = ConfigurationBlock<rake>::num_scalars_per_row;
                constexpr std::size_t row_r = ConfigurationBlock<rake>::num_scalars_rounded / dimension;
                for (std::size_t j = 0; j < dimension; ++j)
                {
                    for (std::size_t l = 0; l < row; ++l)
                    {
                        out[(count * dimension + j) * row + l] = arr[j * row_r + l];
                    }
                }
            }
            const bool ok = static_cast<long>(count) != fail_at;
            ++count;
            return ok;
        }

        template <std::size_t rake>
        static bool fkcc_attach(const collision::Environment<FloatVector<rake>> &e, const ConfigurationBlock<rake> &b) noexcept
        {
            return fkcc<rake>(e, b);
        }
    };
    thread_local float *Recorder::out = nullptr;
    thread_local std::size_t Recorder::cap = 0;
    thread_local std::size_t Recorder::count = 0;
    thread_local long Recorder::fail_at = -1;

    // A stand-in robot whose fkcc forwards every block to the real Robot::fkcc and counts it:
    // driving the reference's own validate_motion with it gives the verdict together with the
    // number of blocks the reference checked before it stopped (planning/validate.hh:24-67).
    // Environments with an attachment are not supported (the reference's fkcc_attach poses the
    // attachment with Eigen, which the type-only stand-in cannot evaluate).
    struct Counted
    {
        static constexpr std::size_t dimension = Robot::dimension;
        using Configuration = Robot::Configuration;
        template <std::size_t rake>
        using ConfigurationBlock = Robot::ConfigurationBlock<rake>;

        static thread_local std::size_t count;

        template <std::size_t rake>
        static bool fkcc(const collision::Environment<FloatVector<rake>> &e, const ConfigurationBlock<rake> &b) noexcept
        {
            ++count;
            return Robot::template fkcc<rake>(e, b);
        }

        template <std::size_t rake>
        static bool fkcc_attach(const collision::Environment<FloatVector<rake>> &e, const ConfigurationBlock<rake> &b) noexcept
        {
            return fkcc<rake>(e, b);
        }
    };
    thread_local std::size_t Counted::count = 0;

    inline auto to_config(const float *q) -> Robot::Configuration
    {
        Robot::ConfigurationArray a;
        for (std::size_t i = 0; i < Robot::dimension; ++i)
        {
            a[i] = q[i];
        }
        return Robot::Configuration(a);
    }

    template <typename R>
    inline bool motion(const float *a, const float *b, int resolution, const collision::Environment<FloatVector<kRake>> &env)
    {
        const auto s = to_config(a);
        const auto g = to_config(b);
        switch (resolution)
        {
            case 1:
                return planning::validate_motion<R, kRake, 1>(s, g, env);
            case 8:
                return planning::validate_motion<R, kRake, 8>(s, g, env);
            case 16:
                return planning::validate_motion<R, kRake, 16>(s, g, env);
            case 32:
                return planning::validate_motion<R, kRake, 32>(s, g, env);
            case 64:
                return planning::validate_motion<R, kRake, 64>(s, g, env);
            default:
                return false;
        }
    }

    template <typename R>
    inline bool vector_motion(const float *a, const float *v, float distance, int resolution,
                              const collision::Environment<FloatVector<kRake>> &env)
    {
        const auto s = to_config(a);
        const auto w = to_config(v);
        switch (resolution)
        {
            case 1:
                return planning::validate_vector<R, kRake, 1>(s, w, distance, env);
            case 8:
                return planning::validate_vector<R, kRake, 8>(s, w, distance, env);
            case 16:
                return planning::validate_vector<R, kRake, 16>(s, w, distance, env);
            case 32:
                return planning::validate_vector<R, kRake, 32>(s, w, distance, env);
            case 64:
                return planning::validate_vector<R, kRake, 64>(s, w, distance, env);
            default:
                return false;
        }
    }

    template <typename F>
    void parallel_for(std::size_t n, int nthreads, F &&f)
    {
        if (nthreads <= 1 or n < 2)
        {
            for (std::size_t i = 0; i < n; ++i)
            {
                f(i);
            }
            return;
        }
        std::atomic<std::size_t> next{0};
        std::vector<std::thread> pool;
        for (int t = 0; t < nthreads; ++t)
        {
            pool.emplace_back(
                [&]()
                {
                    for (;;)
                    {
                        const std::size_t start = next.fetch_add(64);
                        if (start >= n)
                        {
                            break;
                        }
                        const std::size_t end = std::min(n, start + 64);
                        for (std::size_t i = start; i < end; ++i)
                        {
                            f(i);
                        }
                    }
                });
        }
        for (auto &t : pool)
        {
            t.join();
        }
    }
}  // namespace

extern "C" {

int VG_FN(_info)(int *dim, int *n_spheres, float *r_min, float *r_max, int *resolution)
{
    *dim = static_cast<int>(Robot::dimension);
    *n_spheres = static_cast<int>(Robot::n_spheres);
    *r_min = Robot::min_radius;
    *r_max = Robot::max_radius;
    *resolution = static_cast<int>(Robot::resolution);
    return static_cast<int>(kRake);
}

// Joint scaling constants s_m, s_a (q = u * s_m + s_a), dim floats each.
void VG_FN(_limits)(float *s_m, float *s_a)
{
    for (std::size_t i = 0; i < Robot::dimension; ++i)
    {
        s_m[i] = Robot::s_m[i];
        s_a[i] = Robot::s_a[i];
    }
}

// fkcc on one block; q is [dim][lanes] row-major.  Returns 1 if every lane is valid.
int VG_FN(_fkcc_block)(void *env, const float *q)
{
    auto *e = static_cast<RefEnv *>(env);
    e->finalize();
    Block block;
    for (std::size_t j = 0; j < Robot::dimension; ++j)
    {
        std::array<float, kRake> row;
        std::memcpy(row.data(), q + j * kRake, sizeof(row));
        block[j] = FloatVector<kRake>(row);
    }
    return Robot::fkcc<kRake>(*e->vec, block) ? 1 : 0;
}

// Robot::fkcc_debug (robots/panda.hh:468) on one configuration broadcast to every lane, as the
// Python binding's debug() calls it (bindings/robot_helper.hh:249-253).  env_words [fine][words]
// gets a bit per reported object (objects are named by insertion order); the colliding fine self
// pairs are written to pairs_ij (up to cap pairs), their count to *n_pairs.
void VG_FN(_debug)(void *env, const float *q, uint32_t *env_words, int words, int *pairs_ij, int cap, int *n_pairs)
{
    auto *e = static_cast<RefEnv *>(env);
    e->finalize();
    Block block;
    for (std::size_t j = 0; j < Robot::dimension; ++j)
    {
        std::array<float, kRake> row;
        row.fill(q[j]);
        block[j] = FloatVector<kRake>(row);
    }
    const auto out = Robot::fkcc_debug<kRake>(*e->vec, block);
    std::memset(env_words, 0, sizeof(uint32_t) * words * out.first.size());
    for (std::size_t i = 0; i < out.first.size(); ++i)
    {
        for (const auto &name : out.first[i])
        {
            const int id = std::stoi(name);
            env_words[i * words + id / 32] |= 1u << (id % 32);
        }
    }
    int k = 0;
    for (const auto &pr : out.second)
    {
        if (k < cap)
        {
            pairs_ij[2 * k] = static_cast<int>(pr.first);
            pairs_ij[2 * k + 1] = static_cast<int>(pr.second);
        }
        ++k;
    }
    *n_pairs = k;
}

// Per-state validity as the Python binding's validate() computes it: validate_motion(q, q) with
// resolution 1 (bindings/robot_helper.hh:256-267).  q is [n][dim].
void VG_FN(_validate_states)(void *env, const float *q, std::size_t n, uint8_t *out, int nthreads)
{
    auto *e = static_cast<RefEnv *>(env);
    e->finalize();
    const auto &ev = *e->vec;
    parallel_for(
        n,
        nthreads,
        [&](std::size_t i)
        {
            const float *qi = q + i * Robot::dimension;
            out[i] = motion<Robot>(qi, qi, 1, ev) ? 1 : 0;
        });
}

// Edge validity with validate_motion<Robot, lanes, resolution>.  a, b are [n][dim].
void VG_FN(_validate_motions)(
    void *env,
    const float *a,
    const float *b,
    std::size_t n,
    int resolution,
    uint8_t *out,
    int nthreads)
{
    auto *e = static_cast<RefEnv *>(env);
    e->finalize();
    const auto &ev = *e->vec;
    parallel_for(
        n,
        nthreads,
        [&](std::size_t i)
        {
            out[i] = motion<Robot>(a + i * Robot::dimension, b + i * Robot::dimension, resolution, ev) ? 1 : 0;
        });
}

// As _validate_motions, with the number of blocks the reference checked per edge (its early
// return on the first colliding block included) in blocks[n].
void VG_FN(_validate_motions_counted)(
    void *env,
    const float *a,
    const float *b,
    std::size_t n,
    int resolution,
    uint8_t *out,
    int32_t *blocks,
    int nthreads)
{
    auto *e = static_cast<RefEnv *>(env);
    e->finalize();
    const auto &ev = *e->vec;
    parallel_for(
        n,
        nthreads,
        [&](std::size_t i)
        {
            Counted::count = 0;
            out[i] = motion<Counted>(a + i * Robot::dimension, b + i * Robot::dimension, resolution, ev) ? 1 : 0;
            blocks[i] = static_cast<int32_t>(Counted::count);
        });
}

// validate_vector<Robot, lanes, resolution> (planning/validate.hh:23-63) for a batch: start and
// vector [n][dim], distance [n].
void VG_FN(_validate_vectors)(
    void *env,
    const float *start,
    const float *vector,
    const float *distance,
    std::size_t n,
    int resolution,
    uint8_t *out,
    int nthreads)
{
    auto *e = static_cast<RefEnv *>(env);
    e->finalize();
    const auto &ev = *e->vec;
    parallel_for(
        n,
        nthreads,
        [&](std::size_t i)
        {
            out[i] = vector_motion<Robot>(start + i * Robot::dimension, vector + i * Robot::dimension, distance[i],
                                          resolution, ev) ?
                         1 :
                         0;
        });
}

// filter_self_from_pointcloud as the binding computes it (bindings/robot_helper.hh:307-345), from
// the reference's own sphere_fk<1>, sphere_sphere_sql2 and sphere_environment_in_collision.
// Writes the kept points to out (capacity n); returns their number.
std::size_t VG_FN(_filter_self)(void *env, const float *xyz, std::size_t n, float point_radius, const float *q, float *out)
{
    auto *e = static_cast<RefEnv *>(env);
    e->finalize();
    const auto &ev = *e->vec;
    typename Robot::template Spheres<1> s;
    typename Robot::template ConfigurationBlock<1> block;
    for (std::size_t d = 0; d < Robot::dimension; ++d)
        block[d] = FloatVector<1, 1>::fill(q[d]);
    Robot::template sphere_fk<1>(block, s);
    std::size_t m = 0;
    for (std::size_t i = 0; i < n; ++i)
    {
        const float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2], r = point_radius;
        bool valid = true;
        for (auto k = 0U; k < Robot::n_spheres; ++k)
        {
            if (collision::sphere_sphere_sql2(s.x[{k, 0}], s.y[{k, 0}], s.z[{k, 0}], s.r[{k, 0}], x, y, z, r) < 0 or
                sphere_environment_in_collision<>(ev, x, y, z, r))
            {
                valid = false;
                break;
            }
        }
        if (valid)
        {
            out[3 * m] = x;
            out[3 * m + 1] = y;
            out[3 * m + 2] = z;
            ++m;
        }
    }
    return m;
}

// The blocks validate_motion visits for one edge, in visiting order.  out holds up to cap blocks of
// [dim][lanes] floats.  If fail_at >= 0 the fail_at-th visited block reports a collision, which
// shows where the reference stops.  Returns the number of blocks visited.
long VG_FN(_motion_blocks)(const float *a, const float *b, int resolution, float *out, std::size_t cap, long fail_at)
{
    collision::Environment<FloatVector<kRake>> empty;
    Recorder::out = out;
    Recorder::cap = cap;
    Recorder::count = 0;
    Recorder::fail_at = fail_at;
    motion<Recorder>(a, b, resolution, empty);
    return static_cast<long>(Recorder::count);
}

// Fine sphere centres and radii for one configuration: sphere_fk (robots/panda.hh:117-462).
// out is [n_spheres][4].
void VG_FN(_sphere_fk)(const float *q, float *out)
{
    Block block;
    for (std::size_t j = 0; j < Robot::dimension; ++j)
    {
        block[j] = FloatVector<kRake>::fill(q[j]);
    }
    Robot::Spheres<kRake> s;
    Robot::sphere_fk<kRake>(block, s);
    for (std::size_t i = 0; i < Robot::n_spheres; ++i)
    {
        out[4 * i + 0] = s.x[{i, 0}];
        out[4 * i + 1] = s.y[{i, 0}];
        out[4 * i + 2] = s.z[{i, 0}];
        out[4 * i + 3] = s.r[{i, 0}];
    }
}

}  // extern "C"
