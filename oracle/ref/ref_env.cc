// C ABI over the reference's own environment, CAPT and vector code, compiled from the reference
// sources in place.  This is test infrastructure: it exists so that the project's restated oracle,
// golden fixtures and GPU kernels can be checked against the reference itself.  Nothing in the
// shipped library links it.
//
// Reference interfaces wrapped here:
//   collision::Environment<float> / Environment<FloatVector<8>>   collision/environment.hh:15-85
//   collision::Sphere / Capsule / Cuboid constructors             collision/shapes.hh:33-251
//   collision::CAPT (build, collides, collides_simd, layout)      collision/capt.hh:62-617
//   FloatVector<8>::sqrt (rsqrt based on x86)                     vector/avx.hh:412-415
#include "ref_common.hh"

#include <string>

#include <cstring>

using namespace vamp;
using namespace vamp::collision;

extern "C" {

void *vgref_env_create(void)
{
    return new RefEnv();
}

void vgref_env_destroy(void *h)
{
    delete static_cast<RefEnv *>(h);
}

void vgref_env_add_sphere(void *h, const float *f)
{
    auto *e = static_cast<RefEnv *>(h);
    e->scalar.spheres.emplace_back(Sphere<float>(f[0], f[1], f[2], f[3]));
    e->scalar.spheres.back().name = std::to_string(e->n_added++);
    e->dirty = true;
}

// Capsule fields: x1 y1 z1 xv yv zv r rdv
void vgref_env_add_capsule(void *h, const float *f, int z_aligned)
{
    auto *e = static_cast<RefEnv *>(h);
    Capsule<float> c(f[0], f[1], f[2], f[3], f[4], f[5], f[6], f[7]);
    c.name = std::to_string(e->n_added++);
    if (z_aligned)
    {
        e->scalar.z_aligned_capsules.emplace_back(c);
    }
    else
    {
        e->scalar.capsules.emplace_back(c);
    }
    e->dirty = true;
}

// Cuboid fields: x y z, axis_1 xyz, axis_2 xyz, axis_3 xyz, half extents r1 r2 r3
void vgref_env_add_cuboid(void *h, const float *f, int z_aligned)
{
    auto *e = static_cast<RefEnv *>(h);
    Cuboid<float> c(
        f[0], f[1], f[2], f[3], f[4], f[5], f[6], f[7], f[8], f[9], f[10], f[11], f[12], f[13], f[14]);
    c.name = std::to_string(e->n_added++);
    if (z_aligned)
    {
        e->scalar.z_aligned_cuboids.emplace_back(c);
    }
    else
    {
        e->scalar.cuboids.emplace_back(c);
    }
    e->dirty = true;
}

int vgref_env_add_pointcloud(void *h, const float *pts, size_t n, float r_min, float r_max, float r_point)
{
    auto *e = static_cast<RefEnv *>(h);
    std::vector<Point> points(n);
    for (size_t i = 0; i < n; ++i)
    {
        points[i] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    }
    e->scalar.pointclouds.emplace_back(points, r_min, r_max, r_point);
    e->dirty = true;
    return 0;
}

// A heightfield with data [xd * yd], named by insertion order like the primitives.  Built with the
// reference's HeightField constructor (collision/shapes.hh:270-294) and the arguments its factory
// passes (collision/factory.hh:365-386, heightfield::flat: the scales inverted); factory.hh itself
// needs Eigen, which the stand-in does not provide.
void vgref_env_add_heightfield(void *h, const float *centre, const float *scale, size_t xd, size_t yd,
                               const float *data)
{
    auto *e = static_cast<RefEnv *>(h);
    HeightField<float> hf(centre[0], centre[1], centre[2], 1.F / scale[0], 1.F / scale[1], 1.F / scale[2], xd, yd,
                          std::vector<float>(data, data + xd * yd));
    hf.name = std::to_string(e->n_added++);
    e->scalar.heightfields.emplace_back(hf);
    e->dirty = true;
}

// Sorts each primitive list by min_distance and builds the 8-lane environment, as the reference's
// Python binding does before every query (bindings/environment.cc, bindings/robot_helper.hh:252).
void vgref_env_finalize(void *h)
{
    static_cast<RefEnv *>(h)->finalize();
}

// kind: 0 spheres, 1 capsules, 2 z-capsules, 3 cuboids, 4 z-cuboids
size_t vgref_env_count(void *h, int kind)
{
    auto *e = static_cast<RefEnv *>(h);
    e->finalize();
    switch (kind)
    {
        case 0:
            return e->scalar.spheres.size();
        case 1:
            return e->scalar.capsules.size();
        case 2:
            return e->scalar.z_aligned_capsules.size();
        case 3:
            return e->scalar.cuboids.size();
        case 4:
            return e->scalar.z_aligned_cuboids.size();
        default:
            return 0;
    }
}

// Copies the fields of the idx-th object of a kind, in sorted order, followed by min_distance.
int vgref_env_get(void *h, int kind, size_t idx, float *out)
{
    auto *e = static_cast<RefEnv *>(h);
    e->finalize();
    if (kind == 0)
    {
        const auto &s = e->scalar.spheres.at(idx);
        const float f[5] = {s.x, s.y, s.z, s.r, s.min_distance};
        std::memcpy(out, f, sizeof(f));
        return 5;
    }
    if (kind == 1 or kind == 2)
    {
        const auto &c = (kind == 1 ? e->scalar.capsules : e->scalar.z_aligned_capsules).at(idx);
        const float f[9] = {c.x1, c.y1, c.z1, c.xv, c.yv, c.zv, c.r, c.rdv, c.min_distance};
        std::memcpy(out, f, sizeof(f));
        return 9;
    }
    if (kind == 3 or kind == 4)
    {
        const auto &c = (kind == 3 ? e->scalar.cuboids : e->scalar.z_aligned_cuboids).at(idx);
        const float f[16] = {
            c.x,
            c.y,
            c.z,
            c.axis_1_x,
            c.axis_1_y,
            c.axis_1_z,
            c.axis_2_x,
            c.axis_2_y,
            c.axis_2_z,
            c.axis_3_x,
            c.axis_3_y,
            c.axis_3_z,
            c.axis_1_r,
            c.axis_2_r,
            c.axis_3_r,
            c.min_distance};
        std::memcpy(out, f, sizeof(f));
        return 16;
    }
    return -1;
}

// ---------------------------------------------------------------------------------------------
// CAPT layout access (collision/capt.hh:584-617)

void *vgref_capt_build(const float *pts, size_t n, float r_min, float r_max, float r_point)
{
    std::vector<Point> points(n);
    for (size_t i = 0; i < n; ++i)
    {
        points[i] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    }
    return new CAPT(points, r_min, r_max, r_point);
}

void vgref_capt_destroy(void *h)
{
    delete static_cast<CAPT *>(h);
}

// sizes[0] = nlog2, sizes[1] = number of tests, sizes[2] = number of leaves (aabbs),
// sizes[3] = number of 8-point affordance blocks, sizes[4] = lanes per block
void vgref_capt_sizes(void *h, uint64_t *sizes)
{
    const auto *c = static_cast<CAPT *>(h);
    sizes[0] = c->nlog2;
    sizes[1] = c->tests.size();
    sizes[2] = c->aabbs.size();
    sizes[3] = c->affordances[0].size();
    sizes[4] = CAPT::FVectorT::num_scalars;
}

// aabbs: 6 floats per leaf (lower xyz, upper xyz); aff: 3 planes (x, y, z) of blocks*lanes floats;
// top: lower xyz, upper xyz; radii: r_min, r_max, r_point
void vgref_capt_dump(
    void *h,
    float *tests,
    float *aabbs,
    uint32_t *aff_starts,
    float *aff,
    float *top,
    float *radii)
{
    const auto *c = static_cast<CAPT *>(h);
    std::memcpy(tests, c->tests.data(), c->tests.size() * sizeof(float));
    for (size_t i = 0; i < c->aabbs.size(); ++i)
    {
        for (int k = 0; k < 3; ++k)
        {
            aabbs[6 * i + k] = c->aabbs[i].lower[k];
            aabbs[6 * i + 3 + k] = c->aabbs[i].upper[k];
        }
    }
    std::memcpy(aff_starts, c->aff_starts.data(), c->aff_starts.size() * sizeof(uint32_t));
    const size_t nb = c->affordances[0].size();
    constexpr size_t L = CAPT::FVectorT::num_scalars;
    for (int k = 0; k < 3; ++k)
    {
        for (size_t b = 0; b < nb; ++b)
        {
            const auto arr = c->affordances[k][b].to_array();
            for (size_t l = 0; l < L; ++l)
            {
                aff[(k * nb + b) * L + l] = arr[l];
            }
        }
    }
    for (int k = 0; k < 3; ++k)
    {
        top[k] = c->aabb_top.lower[k];
        top[3 + k] = c->aabb_top.upper[k];
    }
    radii[0] = c->r_min;
    radii[1] = c->r_max;
    radii[2] = c->r_point;
}

int vgref_capt_collides(void *h, const float *center, float r)
{
    const auto *c = static_cast<CAPT *>(h);
    return c->collides({center[0], center[1], center[2]}, r) ? 1 : 0;
}

// 8 spheres at once: xs, ys, zs, rs each 8 floats (collision/capt.hh:425-506)
int vgref_capt_collides_simd(void *h, const float *xs, const float *ys, const float *zs, const float *rs)
{
    const auto *c = static_cast<CAPT *>(h);
    std::array<float, 8> ax, ay, az, ar;
    std::memcpy(ax.data(), xs, 32);
    std::memcpy(ay.data(), ys, 32);
    std::memcpy(az.data(), zs, 32);
    std::memcpy(ar.data(), rs, 32);
    const std::array<CAPT::FVectorT, 3> centers = {
        CAPT::FVectorT(ax), CAPT::FVectorT(ay), CAPT::FVectorT(az)};
    return c->collides_simd(centers, CAPT::FVectorT(ar)) ? 1 : 0;
}

// ---------------------------------------------------------------------------------------------
// Vector arithmetic probes

// The reference's 8-lane sqrt (vector/avx.hh:412-415 on x86).
void vgref_vec_sqrt8(const float *in, float *out)
{
    std::array<float, 8> a;
    std::memcpy(a.data(), in, 32);
    const auto r = FloatVector<8>(a).sqrt().to_array();
    std::memcpy(out, r.data(), 32);
}

// The reference's 8-lane sin and cos (vector/avx.hh:456-544, vector/interface.hh:451-458).
void vgref_vec_sincos8(const float *in, float *s, float *c)
{
    std::array<float, 8> a;
    std::memcpy(a.data(), in, 32);
    const auto v = FloatVector<8>(a);
    const auto rs = v.sin().to_array();
    const auto rc = v.cos().to_array();
    std::memcpy(s, rs.data(), 32);
    std::memcpy(c, rc.data(), 32);
}

}  // extern "C"

namespace
{
    // The 8-lane query where the build's environment holds 8-lane vectors (the AVX2 build); -1
    // in a 4-lane (NEON) build.
    template <std::size_t L>
    int sphere_env_lanes(RefEnv *e, const float *xs, const float *ys, const float *zs, const float *rs)
    {
        if constexpr (L == 8)
        {
            std::array<float, 8> ax, ay, az, ar;
            std::memcpy(ax.data(), xs, 32);
            std::memcpy(ay.data(), ys, 32);
            std::memcpy(az.data(), zs, 32);
            std::memcpy(ar.data(), rs, 32);
            return sphere_environment_in_collision(
                       *e->vec, FloatVector<8>(ax), FloatVector<8>(ay), FloatVector<8>(az), FloatVector<8>(ar)) ?
                       1 :
                       0;
        }
        else
        {
            return -1;
        }
    }
}  // namespace

extern "C" {

// One sphere query (8 lanes) against the environment: sphere_environment_in_collision
// (collision/validity.hh:47-150).  Returns 1 on collision (-1 in a 4-lane build).
int vgref_sphere_env8(void *h, const float *xs, const float *ys, const float *zs, const float *rs)
{
    auto *e = static_cast<RefEnv *>(h);
    e->finalize();
    return sphere_env_lanes<FloatVectorWidth>(e, xs, ys, zs, rs);
}

int vgref_lanes(void)
{
    return static_cast<int>(FloatVectorWidth);
}

}  // extern "C"
