// Stand-ins for the reference's public C++ types that include/vamp_gb300_dropin.hh and
// tests/dropin/dropin_check.cc touch: same names, namespaces and members, nothing more.  They let
// the drop-in's GPU test build where the reference checkout is absent (the GPU machine); the CPU test
// builds the same program against the reference's own headers (collision/shapes.hh,
// collision/environment.hh, collision/capt.hh, vector/interface.hh, robots/panda.hh,
// planning/validate.hh).  Test infrastructure only.
#pragma once

#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <optional>
#include <string>
#include <vector>

namespace vamp
{
    constexpr std::size_t FloatVectorWidth = 8;  // the x86 (AVX2) build

    // R rows of N lanes, row-major.
    template <std::size_t N, std::size_t R = 1>
    struct FloatVector
    {
        static constexpr std::size_t num_scalars = N * R;
        static constexpr std::size_t num_scalars_per_row = N;
        std::array<float, N * R> v{};

        FloatVector() = default;
        FloatVector(float s) { v.fill(s); }
        FloatVector(const std::array<float, N * R> &a) : v(a) {}

        std::array<float, N * R> to_array() const { return v; }

        FloatVector operator-(const FloatVector &o) const
        {
            FloatVector r;
            for (std::size_t i = 0; i < N * R; ++i)
                r.v[i] = v[i] - o.v[i];
            return r;
        }

        // The x86 build's order: squares summed lane-wise over 8-wide vectors, then
        // ((s0 + s4) + (s2 + s6)) + ((s1 + s5) + (s3 + s7)), then a rounded square root.
        float l2_norm() const
        {
            float s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            for (std::size_t i = 0; i < N * R; ++i)
            {
                const float sq = v[i] * v[i];
                s[i % 8] = i < 8 ? sq : s[i % 8] + sq;
            }
            return std::sqrt(((s[0] + s[4]) + (s[2] + s[6])) + ((s[1] + s[5]) + (s[3] + s[7])));
        }
    };
}  // namespace vamp

namespace vamp::collision
{
    using Point = std::array<float, 3>;

    template <typename DataT>
    struct Shape
    {
        std::string name;
        DataT min_distance;
    };

    template <typename DataT>
    struct Sphere : Shape<DataT>
    {
        DataT x, y, z, r;
        Sphere() = default;
        template <typename O>
        explicit Sphere(const Sphere<O> &o) : Shape<DataT>{o.name, o.min_distance}, x(o.x), y(o.y), z(o.z), r(o.r)
        {
        }
    };

    template <typename DataT>
    struct Cylinder : Shape<DataT>
    {
        DataT x1, y1, z1, xv, yv, zv, r, rdv;
        Cylinder() = default;
        template <typename O>
        explicit Cylinder(const Cylinder<O> &o)
          : Shape<DataT>{o.name, o.min_distance}, x1(o.x1), y1(o.y1), z1(o.z1), xv(o.xv), yv(o.yv), zv(o.zv), r(o.r), rdv(o.rdv)
        {
        }
    };

    template <typename DataT>
    using Capsule = Cylinder<DataT>;

    template <typename DataT>
    struct Cuboid : Shape<DataT>
    {
        DataT x, y, z, axis_1_x, axis_1_y, axis_1_z, axis_2_x, axis_2_y, axis_2_z, axis_3_x, axis_3_y, axis_3_z, axis_1_r,
            axis_2_r, axis_3_r;
        Cuboid() = default;
        template <typename O>
        explicit Cuboid(const Cuboid<O> &o)
          : Shape<DataT>{o.name, o.min_distance}, x(o.x), y(o.y), z(o.z), axis_1_x(o.axis_1_x), axis_1_y(o.axis_1_y),
            axis_1_z(o.axis_1_z), axis_2_x(o.axis_2_x), axis_2_y(o.axis_2_y), axis_2_z(o.axis_2_z), axis_3_x(o.axis_3_x),
            axis_3_y(o.axis_3_y), axis_3_z(o.axis_3_z), axis_1_r(o.axis_1_r), axis_2_r(o.axis_2_r), axis_3_r(o.axis_3_r)
        {
        }
    };

    template <typename DataT>
    struct HeightField : Shape<DataT>
    {
        DataT x, y, z, xs, ys, zs;
        std::size_t xd, yd;
        std::vector<float> data;
        HeightField() = default;
        template <typename O>
        explicit HeightField(const HeightField<O> &o)
          : Shape<DataT>{o.name, o.min_distance}, x(o.x), y(o.y), z(o.z), xs(o.xs), ys(o.ys), zs(o.zs), xd(o.xd), yd(o.yd),
            data(o.data)
        {
        }
    };

    struct Volume
    {
        Point lower, upper;
    };

    struct CAPT
    {
        using FVectorT = FloatVector<8>;
        std::vector<float> tests;
        std::vector<std::uint32_t> aff_starts;
        std::array<std::vector<FVectorT>, 3> affordances;
        std::vector<Volume> aabbs;
        Volume aabb_top;
        float r_min, r_max, r_point;
        std::uint8_t nlog2;
    };

    template <typename DataT>
    struct Attachment
    {
    };

    template <typename DataT>
    struct Environment
    {
        std::vector<Sphere<DataT>> spheres;
        std::vector<Capsule<DataT>> capsules;
        std::vector<Capsule<DataT>> z_aligned_capsules;
        std::vector<Cylinder<DataT>> cylinders;
        std::vector<Cuboid<DataT>> cuboids;
        std::vector<Cuboid<DataT>> z_aligned_cuboids;
        std::vector<HeightField<DataT>> heightfields;
        std::vector<CAPT> pointclouds;
        std::optional<Attachment<DataT>> attachments;

        Environment() = default;
        template <typename O>
        explicit Environment(const Environment<O> &o)
          : spheres(o.spheres.begin(), o.spheres.end()), capsules(o.capsules.begin(), o.capsules.end()),
            z_aligned_capsules(o.z_aligned_capsules.begin(), o.z_aligned_capsules.end()),
            cylinders(o.cylinders.begin(), o.cylinders.end()), cuboids(o.cuboids.begin(), o.cuboids.end()),
            z_aligned_cuboids(o.z_aligned_cuboids.begin(), o.z_aligned_cuboids.end()),
            heightfields(o.heightfields.begin(), o.heightfields.end()), pointclouds(o.pointclouds)
        {
        }
    };
}  // namespace vamp::collision

namespace vamp::robots
{
    struct Panda
    {
        static constexpr const char *name = "panda";
        static constexpr std::size_t dimension = 7;
        static constexpr std::size_t resolution = 32;
        using Configuration = FloatVector<dimension>;
        template <std::size_t rake>
        using ConfigurationBlock = FloatVector<rake, dimension>;
    };
}  // namespace vamp::robots

namespace vamp::planning
{
    template <typename Robot, std::size_t rake, std::size_t resolution>
    inline auto validate_vector(
        const typename Robot::Configuration &start,
        const typename Robot::Configuration &vector,
        float distance,
        const collision::Environment<FloatVector<rake>> &environment) -> bool;

    template <typename Robot, std::size_t rake, std::size_t resolution>
    inline auto validate_motion(
        const typename Robot::Configuration &start,
        const typename Robot::Configuration &goal,
        const collision::Environment<FloatVector<rake>> &environment) -> bool;
}  // namespace vamp::planning
