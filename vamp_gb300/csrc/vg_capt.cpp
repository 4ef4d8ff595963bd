// CAPT construction (see vg_capt.h).  Compiled with -ffp-contract=off: the two squared-distance
// sums below use explicit fused multiply-adds in the order the reference's compiled builder
// evaluates them, so the affordance decisions (and hence the layout) match it bit for bit.
#include "vg_capt.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <numeric>

namespace vg
{
    namespace
    {
        constexpr float kInf = std::numeric_limits<float>::infinity();
        constexpr int kLanes = 8;  // points per affordance block

        struct Cell
        {
            float lo[3], hi[3];
        };

        // Volume::distsq_to (capt.hh:47-54): squared distance from p to the cell
        float cell_distsq(const Cell &c, const float *p)
        {
            float d[3];
            for (int k = 0; k < 3; ++k)
            {
                const float m = c.lo[k] > p[k] ? c.lo[k] : p[k];
                const float cl = c.hi[k] < m ? c.hi[k] : m;
                d[k] = p[k] - cl;
            }
            return std::fma(d[2], d[2], std::fma(d[0], d[0], d[1] * d[1]));
        }

        // Volume::contained_by_internal_ball (capt.hh:38-45)
        bool cell_inside_ball(const Cell &c, const float *p, float r2)
        {
            float d[3];
            for (int k = 0; k < 3; ++k)
            {
                const float a = p[k] - c.lo[k], b = c.hi[k] - p[k];
                d[k] = a < b ? b : a;
            }
            return std::fma(d[2], d[2], std::fma(d[0], d[0], d[1] * d[1])) <= r2;
        }

        struct Builder
        {
            CaptHost &out;
            const std::vector<float> &pts;  // padded, 3 per point
            std::vector<uint32_t> order;    // argsort, refined level by level
            float max_l2, min_l2;
            uint32_t next_leaf = 0;

            const float *pt(uint32_t i) const { return &pts[3 * static_cast<size_t>(i)]; }

            void push_block(const float *xs, const float *ys, const float *zs)
            {
                out.aff.insert(out.aff.end(), xs, xs + kLanes);
                out.aff.insert(out.aff.end(), ys, ys + kLanes);
                out.aff.insert(out.aff.end(), zs, zs + kLanes);
            }

            void leaf(uint32_t begin, const std::vector<uint32_t> &afford, const Cell &cell)
            {
                const float *rep = pt(order[begin]);
                const uint32_t id = next_leaf++;
                float *box = &out.aabbs[6 * static_cast<size_t>(id)];
                for (int k = 0; k < 3; ++k)
                {
                    box[k] = box[3 + k] = rep[k];
                }
                if (std::isfinite(rep[0]))
                {
                    for (int k = 0; k < 3; ++k)
                    {
                        out.top[k] = std::min(out.top[k], rep[k]);
                        out.top[3 + k] = std::max(out.top[3 + k], rep[k]);
                    }
                    float xs[kLanes] = {rep[0]}, ys[kLanes] = {rep[1]}, zs[kLanes] = {rep[2]};
                    int j = 1;
                    if (!cell_inside_ball(cell, rep, min_l2))
                    {
                        for (const uint32_t i : afford)
                        {
                            const float *p = pt(i);
                            if (cell_distsq(cell, p) <= max_l2)
                            {
                                for (int k = 0; k < 3; ++k)
                                {
                                    box[k] = std::min(box[k], p[k]);
                                    box[3 + k] = std::max(box[3 + k], p[k]);
                                }
                                xs[j] = p[0];
                                ys[j] = p[1];
                                zs[j] = p[2];
                                if (++j == kLanes)
                                {
                                    push_block(xs, ys, zs);
                                    j = 0;
                                }
                            }
                        }
                    }
                    if (j > 0)
                    {
                        for (int l = j; l < kLanes; ++l)
                        {
                            xs[l] = ys[l] = zs[l] = kInf;
                        }
                        push_block(xs, ys, zs);
                    }
                }
                out.aff_starts[id + 1] = static_cast<uint32_t>(out.blocks());
            }

            void split(uint32_t begin, uint32_t count, uint32_t node, std::vector<uint32_t> afford, const Cell &cell, int d)
            {
                if (count == 1)
                {
                    leaf(begin, afford, cell);
                    return;
                }
                // median along axis d: stable order of the cell's points, mean of the middle two
                const auto key = [&](uint32_t i) { return pts[3 * static_cast<size_t>(i) + d]; };
                std::stable_sort(order.begin() + begin, order.begin() + begin + count,
                                 [&](uint32_t x, uint32_t y) { return key(x) < key(y); });
                const uint32_t half = count / 2;
                const float test = (key(order[begin + half - 1]) + key(order[begin + half])) * 0.5f;
                out.tests[node] = test;
                const float up = test + out.r_max, down = test - out.r_max;

                Cell lo_cell = cell, hi_cell = cell;
                lo_cell.hi[d] = test;
                hi_cell.lo[d] = test;
                std::vector<uint32_t> lo, hi;
                lo.reserve(afford.size() + 8);
                hi.reserve(afford.size() + 8);
                for (const uint32_t i : afford)
                {
                    const float v = key(i);
                    if (v <= up)
                        lo.push_back(i);
                    if (v >= down)
                        hi.push_back(i);
                }
                afford.clear();
                afford.shrink_to_fit();
                // lower-half points for the upper child: the scan starts at the smallest
                // coordinate and stops at the first point below test - r_max (capt.hh:226-233)
                uint32_t h = begin;
                while (h < begin + half && key(order[h]) >= down && std::isfinite(key(order[h])))
                    ++h;
                uint32_t l = begin + half;
                while (l < begin + count && key(order[l]) <= up && std::isfinite(key(order[l])))
                    ++l;
                hi.insert(hi.end(), order.begin() + begin, order.begin() + h);
                lo.insert(lo.end(), order.begin() + begin + half, order.begin() + l);
                const int nd = (d + 1) % 3;
                split(begin, half, 2 * node + 1, std::move(lo), lo_cell, nd);
                split(begin + half, half, 2 * node + 2, std::move(hi), hi_cell, nd);
            }
        };
    }  // namespace

    bool capt_build(const float *xyz, size_t n, float r_min, float r_max, float r_point, CaptHost &out)
    {
        if (n < 2)
        {
            return false;
        }
        out = CaptHost{};
        out.r_min = r_min;
        out.r_max = r_max;
        out.r_point = r_point;
        int nlog2 = 0;
        while ((size_t{1} << nlog2) < n)
            ++nlog2;
        out.nlog2 = nlog2;
        const size_t N = size_t{1} << nlog2;
        out.tests.assign(N - 1, std::numeric_limits<float>::quiet_NaN());
        out.aabbs.assign(6 * N, 0.0f);
        out.aff_starts.assign(N + 1, 0u);
        for (int k = 0; k < 3; ++k)
        {
            out.top[k] = kInf;
            out.top[3 + k] = -kInf;
        }
        std::vector<float> pts(3 * N, kInf);
        std::copy(xyz, xyz + 3 * n, pts.begin());
        const float l1 = r_max + r_point;
        Builder b{out, pts, std::vector<uint32_t>(N), l1 * l1, (r_min + r_point) * (r_min + r_point)};
        std::iota(b.order.begin(), b.order.end(), 0u);
        Cell all;
        for (int k = 0; k < 3; ++k)
        {
            all.lo[k] = -kInf;
            all.hi[k] = kInf;
        }
        b.split(0, static_cast<uint32_t>(N), 0, {}, all, 0);
        return true;
    }
}  // namespace vg
