/* Pointcloud filter of the CPU oracle (test infrastructure).
 * Reference: collision/filter.hh:176-278.  See vgo_filter.c for the algorithm. */
#pragma once
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Filters xyz[n][3]; writes the kept points to out (capacity n) and returns their number. */
size_t vgo_filter_pointcloud(const float *xyz, size_t n, float min_dist, float max_range, const float *origin,
                             const float *workcell_min, const float *workcell_max, int cull, float *out);
/* remap_point of one coordinate, with the conversion rule below (collision/filter.hh:142-145). */
uint32_t vgo_filter_remap(float x, float lo, float hi);
/* The 32-bit Morton code of (x, y, z) (collision/filter.hh:147-171). */
uint32_t vgo_morton(uint32_t x, uint32_t y, uint32_t z);

#ifdef __cplusplus
}
#endif
