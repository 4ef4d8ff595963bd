// A caller written the way the reference's planners call the hot path, built against
// include/vamp_gb300_dropin.hh.
//
//   reference build (-DVG_DROPIN_REFERENCE, the reference's headers on the include path): the
//   caller compiles unchanged with vamp::robots::Panda and with the GPU robot; with --cpu it runs
//   the reference's own validate_motion / fkcc (no GPU needed).
//   stand-in build (tests/dropin/stand_in.hh): for the GPU machine, which has no reference checkout.
//
// Usage: dropin_check <input.bin> <output.bin> [--cpu]
// input.bin (little-endian): int32 n_spheres, n_capsules, n_zcapsules, n_cuboids, n_zcuboids,
// n_edges, n_blocks, n_trees; then per kind its rows (fields then min_distance, float32); the
// edges' starts then goals ([n][7] float32); the blocks ([n][8][7] float32, lanes then joints);
// per tree: int32 nlog2, n_blocks, n_points; float32 points [n][3], tests, aabbs [leaves][6];
// uint32 aff_starts; float32 aff [blocks][3][8], top[6], r_min, r_max, r_point.  The reference
// build builds its tree from the points (its own CAPT constructor); the stand-in build takes the
// layout, which is the reference's tree as built.
// output.bin: uint8 edge verdicts, uint8 block verdicts, float64 seconds per single-edge call
// (a second pass over the edges, the environment already on the GPU).
#ifdef VG_DROPIN_REFERENCE
#include <vamp/collision/environment.hh>
#include <vamp/planning/validate.hh>
#include <vamp/robots/panda.hh>
#else
#include "stand_in.hh"
#endif

#include "vamp_gb300_dropin.hh"

#include <chrono>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

using GpuPanda = vamp_gb300::dropin::Robot<vamp::robots::Panda>;
VAMP_GB300_DROPIN_VALIDATE(GpuPanda)

namespace
{
    constexpr std::size_t kRake = vamp::FloatVectorWidth;
    using EnvF = vamp::collision::Environment<float>;
    using EnvV = vamp::collision::Environment<vamp::FloatVector<kRake>>;

    // As planning/rrtc.hh:136 calls it: the robot's own resolution, the environment's lanes.
    template <typename Robot>
    bool extend(const typename Robot::Configuration &a, const typename Robot::Configuration &b, const EnvV &env)
    {
        return vamp::planning::validate_motion<Robot, kRake, Robot::resolution>(a, b, env);
    }

    template <typename Robot>
    bool block_valid(const typename Robot::template ConfigurationBlock<kRake> &q, const EnvV &env)
    {
        return Robot::template fkcc<kRake>(env, q);
    }

    struct Reader
    {
        std::vector<char> buf;
        std::size_t pos = 0;
        template <typename T>
        T get()
        {
            T v;
            std::memcpy(&v, buf.data() + pos, sizeof(T));
            pos += sizeof(T);
            return v;
        }
        template <typename T>
        std::vector<T> get(std::size_t n)
        {
            std::vector<T> v(n);
            std::memcpy(v.data(), buf.data() + pos, n * sizeof(T));
            pos += n * sizeof(T);
            return v;
        }
    };

    template <typename S>
    void fill(S &s, const std::vector<float> &f, int kind)
    {
        if constexpr (std::is_same_v<S, vamp::collision::Sphere<float>>)
        {
            s.x = f[0], s.y = f[1], s.z = f[2], s.r = f[3], s.min_distance = f[4];
        }
        else if constexpr (std::is_same_v<S, vamp::collision::Capsule<float>>)
        {
            s.x1 = f[0], s.y1 = f[1], s.z1 = f[2], s.xv = f[3], s.yv = f[4], s.zv = f[5], s.r = f[6], s.rdv = f[7];
            s.min_distance = f[8];
        }
        else
        {
            s.x = f[0], s.y = f[1], s.z = f[2];
            s.axis_1_x = f[3], s.axis_1_y = f[4], s.axis_1_z = f[5];
            s.axis_2_x = f[6], s.axis_2_y = f[7], s.axis_2_z = f[8];
            s.axis_3_x = f[9], s.axis_3_y = f[10], s.axis_3_z = f[11];
            s.axis_1_r = f[12], s.axis_2_r = f[13], s.axis_3_r = f[14], s.min_distance = f[15];
        }
        (void)kind;
    }
}  // namespace

int main(int argc, char **argv)
{
    if (argc < 3)
    {
        std::cerr << "usage: dropin_check <input.bin> <output.bin> [--cpu]\n";
        return 2;
    }
    const bool cpu = argc > 3 && std::string(argv[3]) == "--cpu";
    Reader in;
    {
        std::ifstream f(argv[1], std::ios::binary);
        in.buf.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    }
    int counts[8];
    for (int &c : counts)
        c = in.get<int>();
    EnvF ef;
    const int width[5] = {5, 9, 9, 16, 16};
    for (int k = 0; k < 5; ++k)
    {
        for (int i = 0; i < counts[k]; ++i)
        {
            const auto row = in.get<float>(width[k]);
            if (k == 0)
                fill(ef.spheres.emplace_back(), row, k);
            else if (k == 1)
                fill(ef.capsules.emplace_back(), row, k);
            else if (k == 2)
                fill(ef.z_aligned_capsules.emplace_back(), row, k);
            else if (k == 3)
                fill(ef.cuboids.emplace_back(), row, k);
            else
                fill(ef.z_aligned_cuboids.emplace_back(), row, k);
        }
    }
    const int n_edges = counts[5], n_blocks = counts[6], n_trees = counts[7];
    constexpr std::size_t D = vamp::robots::Panda::dimension;
    const auto a = in.get<float>(n_edges * D);
    const auto b = in.get<float>(n_edges * D);
    const auto blocks = in.get<float>(static_cast<std::size_t>(n_blocks) * kRake * D);
    for (int t = 0; t < n_trees; ++t)
    {
        const int nlog2 = in.get<int>();
        const int nb = in.get<int>();
        const int np = in.get<int>();
        const auto pts = in.get<float>(static_cast<std::size_t>(np) * 3);
        const std::size_t leaves = std::size_t{1} << nlog2;
        const auto tests = in.get<float>(leaves - 1);
        const auto boxes = in.get<float>(leaves * 6);
        const auto starts = in.get<std::uint32_t>(leaves + 1);
        const auto aff = in.get<float>(static_cast<std::size_t>(nb) * 24);
        const auto top = in.get<float>(6);
        const auto radii = in.get<float>(3);
#ifdef VG_DROPIN_REFERENCE
        std::vector<vamp::collision::Point> points(np);
        for (int i = 0; i < np; ++i)
            points[i] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        ef.pointclouds.emplace_back(points, radii[0], radii[1], radii[2]);
        (void)tests, (void)boxes, (void)starts, (void)aff, (void)top, (void)nb, (void)leaves;
#else
        vamp::collision::CAPT c;
        c.nlog2 = static_cast<std::uint8_t>(nlog2);
        c.tests.assign(tests.begin(), tests.end());
        c.aff_starts.assign(starts.begin(), starts.end());
        for (std::size_t i = 0; i < leaves; ++i)
        {
            vamp::collision::Volume v;
            for (int k = 0; k < 3; ++k)
            {
                v.lower[k] = boxes[6 * i + k];
                v.upper[k] = boxes[6 * i + 3 + k];
            }
            c.aabbs.push_back(v);
        }
        for (int k = 0; k < 3; ++k)
        {
            for (int i = 0; i < nb; ++i)
            {
                std::array<float, 8> lanes;
                std::memcpy(lanes.data(), &aff[24 * i + 8 * k], sizeof(lanes));
                c.affordances[k].emplace_back(lanes);
            }
        }
        for (int k = 0; k < 3; ++k)
        {
            c.aabb_top.lower[k] = top[k];
            c.aabb_top.upper[k] = top[3 + k];
        }
        c.r_min = radii[0];
        c.r_max = radii[1];
        c.r_point = radii[2];
        ef.pointclouds.push_back(std::move(c));
        (void)pts;
#endif
    }
    const EnvV env(ef);

    std::vector<std::uint8_t> edge_out(n_edges), block_out(n_blocks);
    const auto config = [&](const std::vector<float> &src, int i) {
        std::array<float, D> c;
        std::memcpy(c.data(), &src[i * D], sizeof(c));
        return vamp::robots::Panda::Configuration(c);
    };
    // the reference robot (CPU) only where its code is compiled in
#ifdef VG_DROPIN_REFERENCE
    const auto edge = [&](int i) {
        return cpu ? extend<vamp::robots::Panda>(config(a, i), config(b, i), env) : extend<GpuPanda>(config(a, i), config(b, i), env);
    };
    const auto check = [&](const auto &q) { return cpu ? block_valid<vamp::robots::Panda>(q, env) : block_valid<GpuPanda>(q, env); };
#else
    if (cpu)
    {
        std::cerr << "--cpu needs the reference build\n";
        return 2;
    }
    const auto edge = [&](int i) { return extend<GpuPanda>(config(a, i), config(b, i), env); };
    const auto check = [&](const auto &q) { return block_valid<GpuPanda>(q, env); };
#endif
    for (int i = 0; i < n_edges; ++i)
    {
        edge_out[i] = edge(i);
    }
    // the latency of one call once the environment is resident (the first pass converted it)
    const auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < n_edges; ++i)
    {
        if (edge(i) != static_cast<bool>(edge_out[i]))
        {
            std::cerr << "a repeated call gave another verdict\n";
            return 1;
        }
    }
    const double per_call = n_edges ? std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() / n_edges : 0.0;
    for (int i = 0; i < n_blocks; ++i)
    {
        // the block's rows are joints (ConfigurationBlock<rake>: rake lanes per joint)
        std::array<float, kRake * D> rows;
        for (std::size_t j = 0; j < D; ++j)
            for (std::size_t l = 0; l < kRake; ++l)
                rows[j * kRake + l] = blocks[(static_cast<std::size_t>(i) * kRake + l) * D + j];
        const typename vamp::robots::Panda::template ConfigurationBlock<kRake> q(rows);
        block_out[i] = check(q);
    }
    if (!cpu && n_edges + n_blocks > 0 && vg_last_error() && vg_last_error()[0])
    {
        std::cerr << "last library message: " << vg_last_error() << "\n";
    }
    std::ofstream out(argv[2], std::ios::binary);
    out.write(reinterpret_cast<const char *>(edge_out.data()), edge_out.size());
    out.write(reinterpret_cast<const char *>(block_out.data()), block_out.size());
    out.write(reinterpret_cast<const char *>(&per_call), sizeof(per_call));
    return 0;
}
