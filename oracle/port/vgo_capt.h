/* CAPT (collision-affording point tree) restated for the CPU oracle (test infrastructure).
 * Reference: collision/capt.hh.  See vgo_capt.c for the algorithm. */
#pragma once

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vgo_capt
{
    int nlog2;
    size_t n_tests;     /* 2^nlog2 - 1 split values, heap order */
    size_t n_leaves;    /* 2^nlog2 */
    float *tests;
    float *aabbs;       /* [n_leaves][6]: lower xyz, upper xyz of the afforded points */
    uint32_t *aff_starts; /* [n_leaves + 1], in blocks */
    int lanes;          /* points per affordance block */
    size_t n_blocks, cap_blocks;
    float *aff[3];      /* x, y, z planes: [n_blocks][lanes] */
    float top[6];       /* bounding box of all finite points */
    float r_min, r_max, r_point;
    float *points;      /* the input points, [n_points][3] */
    size_t n_points;
} vgo_capt;

vgo_capt *vgo_capt_build(const float *xyz, size_t n, float r_min, float r_max, float r_point, int lanes);
void vgo_capt_destroy(vgo_capt *c);
/* collides_simd (capt.hh:425-506) for `lanes` spheres: 1 if any collides */
int vgo_capt_collides_block(const vgo_capt *c, int lanes, const float *x, const float *y, const float *z, const float *r);
/* FP64 distance from (x, y, z) to the nearest input point, minus r_point */
double vgo_capt_point_distance(const vgo_capt *c, double x, double y, double z);

#ifdef __cplusplus
}
#endif
