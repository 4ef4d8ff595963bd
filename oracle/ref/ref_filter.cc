// C ABI over the reference's pointcloud filter (collision/filter.hh:176-320, the
// std::vector<Point> overload at :282-319), compiled from the reference sources in place.  Test
// infrastructure only: it pins the restated filter (oracle/port/vgo_filter.c) and the GPU filter.
// The sort inside the filter is pdqsort_branchless, which shim/pdqsort.h replaces with a stable
// sort, so points whose Morton codes tie keep their order from the previous pass.
#include <vamp/collision/filter.hh>

#include <cstddef>
#include <vector>

extern "C" {

// Filters xyz[n][3]; writes the kept points to out (capacity n) and their number to *n_out.
void vgref_filter_pointcloud(const float *xyz, size_t n, float min_dist, float max_range, const float *origin,
                             const float *workcell_min, const float *workcell_max, int cull, float *out, size_t *n_out)
{
    using vamp::collision::Point;
    std::vector<Point> pc(n);
    for (size_t i = 0; i < n; ++i)
        pc[i] = Point{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    const auto kept = vamp::collision::filter_pointcloud(
        pc, min_dist, max_range, Point{origin[0], origin[1], origin[2]},
        Point{workcell_min[0], workcell_min[1], workcell_min[2]}, Point{workcell_max[0], workcell_max[1], workcell_max[2]},
        cull != 0);
    for (size_t i = 0; i < kept.size(); ++i)
        for (int k = 0; k < 3; ++k)
            out[3 * i + k] = kept[i][k];
    *n_out = kept.size();
}

// The float -> uint32_t conversion the reference's remap_point performs (collision/filter.hh:
// 142-145), as compiled here, for the oracle's conversion rule.
unsigned vgref_filter_remap(float x, float min, float max)
{
    return vamp::collision::remap_point(x, min, max);
}

}  // extern "C"
