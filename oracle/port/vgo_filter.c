/* Pointcloud filter restated for the CPU oracle (test infrastructure).  Build with
 * -ffp-contract=off.
 *
 * Follows filter_pointcloud (collision/filter.hh:176-278):
 *   - work list: the indices of the points that pass the cull (closer than max_range to the
 *     origin and inside the workcell box), in input order; the list has n entries and the ones
 *     past the passing points hold index 0 (the reference sizes its vector to n and only
 *     overwrites the front, filter.hh:199-216), so point 0 takes part whatever the cull says;
 *   - six passes, one per permutation of the axes in std::next_permutation order from (0, 1, 2):
 *     map each entry's coordinates (in the permuted order) to integers, ((c - lo) / (hi - lo)) *
 *     1000, interleave them into a 32-bit Morton code, sort the list by code, and drop every
 *     entry within min_dist of the last entry kept (the first entry is always kept);
 *   - the mapping range starts as [min of origin - max_range, min of origin + max_range] (the
 *     reference takes the minimum of the three upper ends too, filter.hh:197), and after each
 *     pass moves halfway towards the smallest and largest coordinate seen in that pass.
 * Two details are pinned to the reference as compiled on x86-64 (AVX-512, -ffp-contract=fast):
 *   - float -> uint32_t conversion truncates and gives 0xFFFFFFFF for NaN, for values <= -1 and
 *     for values >= 2^32;
 *   - squared distances are fma(dz, dz, fma(dx, dx, dy * dy)).
 * The reference sorts with pdqsort, which is not stable; this oracle sorts stably (equal codes
 * keep their order from the previous pass), as the reference does when built with the stable
 * stand-in for pdqsort. */
#include "vgo_filter.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

uint32_t vgo_filter_remap(float x, float lo, float hi)
{
    const float v = ((x - lo) / (hi - lo)) * 1000.0f;
    if (!(v > -1.0f) || !(v < 4294967296.0f))
        return 0xFFFFFFFFu;
    return v <= 0.0f ? 0u : (uint32_t)v;
}

/* bit k of v to bit 3k, for the low `bits` bits */
static uint32_t spread3(uint32_t v, int bits)
{
    uint32_t r = 0;
    for (int k = 0; k < bits; ++k)
        r |= ((v >> k) & 1u) << (3 * k);
    return r;
}

uint32_t vgo_morton(uint32_t x, uint32_t y, uint32_t z)
{
    /* 11 bits of x at 0, 3, ..., 30; 11 of y at 1, ..., 31; 10 of z at 2, ..., 29 */
    return spread3(x, 11) | (spread3(y, 11) << 1) | (spread3(z, 10) << 2);
}

static float sqdist(const float *a, const float *b)
{
    const float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return fmaf(dz, dz, fmaf(dx, dx, dy * dy));
}

typedef struct
{
    uint32_t idx, code, pos;
} entry;

static int by_code(const void *pa, const void *pb)
{
    const entry *a = (const entry *)pa, *b = (const entry *)pb;
    if (a->code != b->code)
        return a->code < b->code ? -1 : 1;
    return a->pos < b->pos ? -1 : (a->pos > b->pos);
}

static float min_of(float cur, float v)
{
    return v < cur ? v : cur; /* std::min keeps the first of equal values */
}

static float max_of(float cur, float v)
{
    return cur < v ? v : cur;
}

size_t vgo_filter_pointcloud(const float *xyz, size_t n, float min_dist, float max_range, const float *origin,
                             const float *workcell_min, const float *workcell_max, int cull, float *out)
{
    static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
    if (n == 0)
        return 0;
    const float sq = min_dist * min_dist, sq_range = max_range * max_range;
    float lo = origin[0] - max_range, hi = origin[0] + max_range;
    for (int k = 1; k < 3; ++k)
    {
        lo = min_of(lo, origin[k] - max_range);
        hi = min_of(hi, origin[k] + max_range);
    }
    entry *e = (entry *)calloc(n, sizeof(entry));
    size_t m = 0;
    for (size_t i = 0; i < n; ++i)
    {
        const float *p = xyz + 3 * i;
        if (!cull || (sqdist(p, origin) < sq_range && workcell_min[0] <= p[0] && p[0] <= workcell_max[0] &&
                      workcell_min[1] <= p[1] && p[1] <= workcell_max[1] && workcell_min[2] <= p[2] &&
                      p[2] <= workcell_max[2]))
            e[m++].idx = (uint32_t)i;
    }
    m = n; /* the entries past the passing points stay at index 0 */
    for (int pass = 0; pass < 6; ++pass)
    {
        const int *ax = perms[pass];
        float new_lo = hi, new_hi = lo;
        for (size_t j = 0; j < m; ++j)
        {
            const float *p = xyz + 3 * (size_t)e[j].idx;
            e[j].code = vgo_morton(vgo_filter_remap(p[ax[0]], lo, hi), vgo_filter_remap(p[ax[1]], lo, hi),
                                   vgo_filter_remap(p[ax[2]], lo, hi));
            e[j].pos = (uint32_t)j;
            for (int k = 0; k < 3; ++k)
            {
                new_lo = min_of(new_lo, p[k]);
                new_hi = max_of(new_hi, p[k]);
            }
        }
        qsort(e, m, sizeof(entry), by_code);
        size_t kept = 1;
        for (size_t j = 1; j < m; ++j)
        {
            if (sqdist(xyz + 3 * (size_t)e[j].idx, xyz + 3 * (size_t)e[kept - 1].idx) > sq)
                e[kept++] = e[j];
        }
        m = kept;
        hi = (new_hi + hi) * 0.5f;
        lo = (new_lo + lo) * 0.5f;
    }
    for (size_t j = 0; j < m; ++j)
        memcpy(out + 3 * j, xyz + 3 * (size_t)e[j].idx, 3 * sizeof(float));
    free(e);
    return m;
}
