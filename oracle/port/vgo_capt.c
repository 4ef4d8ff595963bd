/* CAPT restated for the CPU oracle (test infrastructure).  Build with -ffp-contract=off.
 *
 * Construction follows CAPT::CAPT and CAPT::subdivide (collision/capt.hh:104-365):
 *   - pad the points to a power of two with +inf points;
 *   - recursively split at the median along axis depth mod 3 (stable argsort of the cell's
 *     points; split value = mean of the two middle coordinates);
 *   - each cell carries an "afford" list of outside points that may be within r_max of it.  A
 *     child inherits the parent's list filtered against the split plane, plus points of the
 *     sibling half near the plane.  The sibling scan for the upper child starts at the lower
 *     half's smallest coordinate and stops at the first point below test - r_max
 *     (capt.hh:226-233), so it usually adds nothing; this is reproduced as is, because the
 *     reference's answers depend on it;
 *   - a leaf stores its representative point, then (unless the cell lies inside the
 *     representative's r_min ball) every afforded point within r_max + r_point of the cell, as
 *     blocks of `lanes` points padded with +inf, plus the bounding box of those points.
 * Queries follow CAPT::collides_simd (capt.hh:425-506). */
#include "vgo_capt.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct
{
    uint32_t *v;
    size_t n, cap;
} ivec;

static void iv_push(ivec *a, uint32_t x)
{
    if (a->n == a->cap)
    {
        a->cap = a->cap ? 2 * a->cap : 16;
        a->v = (uint32_t *)realloc(a->v, a->cap * sizeof(uint32_t));
    }
    a->v[a->n++] = x;
}

static void iv_reserve(ivec *a, size_t n)
{
    if (n > a->cap)
    {
        a->cap = n;
        a->v = (uint32_t *)realloc(a->v, a->cap * sizeof(uint32_t));
    }
}

/* stable merge sort of idx[0..n) by pts[idx][k] with "<" (the reference sorts with pdqsort, which
 * is unstable; for untied keys the order is the same) */
static void msort(uint32_t *idx, uint32_t *tmp, size_t n, const float *pts, int k)
{
    if (n < 2)
        return;
    if (n <= 16)
    {
        for (size_t i = 1; i < n; ++i)
        {
            const uint32_t x = idx[i];
            const float key = pts[3 * x + k];
            size_t j = i;
            while (j > 0 && key < pts[3 * idx[j - 1] + k])
            {
                idx[j] = idx[j - 1];
                --j;
            }
            idx[j] = x;
        }
        return;
    }
    const size_t h = n / 2;
    msort(idx, tmp, h, pts, k);
    msort(idx + h, tmp, n - h, pts, k);
    size_t i = 0, j = h, o = 0;
    while (i < h && j < n)
    {
        /* take from the right only if strictly smaller: keeps equal keys in order */
        if (pts[3 * idx[j] + k] < pts[3 * idx[i] + k])
            tmp[o++] = idx[j++];
        else
            tmp[o++] = idx[i++];
    }
    while (i < h)
        tmp[o++] = idx[i++];
    while (j < n)
        tmp[o++] = idx[j++];
    memcpy(idx, tmp, n * sizeof(uint32_t));
}

typedef struct
{
    float lo[3], hi[3];
} vol_t;

/* Volume::distsq_to (capt.hh:47-54) */
static float vol_distsq(const vol_t *v, const float *p)
{
    float d[3];
    for (int k = 0; k < 3; ++k)
    {
        const float m = v->lo[k] > p[k] ? v->lo[k] : p[k];
        const float c = v->hi[k] < m ? v->hi[k] : m;
        d[k] = p[k] - c;
    }
    return fmaf(d[2], d[2], fmaf(d[0], d[0], d[1] * d[1]));
}

/* Volume::contained_by_internal_ball (capt.hh:38-45): the cell lies inside the ball of squared
 * radius r2 around p */
static int vol_in_ball(const vol_t *v, const float *p, float r2)
{
    float d[3];
    for (int k = 0; k < 3; ++k)
    {
        const float a = p[k] - v->lo[k], b = v->hi[k] - p[k];
        d[k] = a < b ? b : a;
    }
    return fmaf(d[2], d[2], fmaf(d[0], d[0], d[1] * d[1])) <= r2;
}

typedef struct
{
    vgo_capt *c;
    const float *pts; /* padded points */
    uint32_t *argsort, *tmp;
    float max_l2, min_l2;
    uint32_t leaf_next;
} builder;

static void push_block(vgo_capt *c, const float *xs, const float *ys, const float *zs)
{
    if (c->n_blocks == c->cap_blocks)
    {
        c->cap_blocks = c->cap_blocks ? 2 * c->cap_blocks : 1024;
        for (int k = 0; k < 3; ++k)
            c->aff[k] = (float *)realloc(c->aff[k], c->cap_blocks * c->lanes * sizeof(float));
    }
    memcpy(c->aff[0] + c->n_blocks * c->lanes, xs, c->lanes * sizeof(float));
    memcpy(c->aff[1] + c->n_blocks * c->lanes, ys, c->lanes * sizeof(float));
    memcpy(c->aff[2] + c->n_blocks * c->lanes, zs, c->lanes * sizeof(float));
    c->n_blocks++;
}

static void extend(float *box, const float *p)
{
    for (int k = 0; k < 3; ++k)
    {
        box[k] = fminf(box[k], p[k]);
        box[3 + k] = fmaxf(box[3 + k], p[k]);
    }
}

static void subdivide(builder *b, uint32_t begin, uint32_t count, uint32_t node, ivec afford, vol_t vol, int d)
{
    vgo_capt *c = b->c;
    const float *P = b->pts;
    if (count == 1)
    {
        const float *rep = P + 3 * b->argsort[begin];
        const uint32_t leaf = b->leaf_next++;
        float *box = c->aabbs + 6 * leaf;
        for (int k = 0; k < 3; ++k)
            box[k] = box[3 + k] = rep[k];
        if (isfinite(rep[0]))
        {
            extend(c->top, rep);
            float xs[16], ys[16], zs[16];
            for (int l = 0; l < c->lanes; ++l)
                xs[l] = ys[l] = zs[l] = 0.0f;
            xs[0] = rep[0];
            ys[0] = rep[1];
            zs[0] = rep[2];
            int j = 1;
            if (!vol_in_ball(&vol, rep, b->min_l2))
            {
                for (size_t i = 0; i < afford.n; ++i)
                {
                    const float *p = P + 3 * afford.v[i];
                    if (vol_distsq(&vol, p) <= b->max_l2)
                    {
                        extend(box, p);
                        xs[j] = p[0];
                        ys[j] = p[1];
                        zs[j] = p[2];
                        if (++j == c->lanes)
                        {
                            push_block(c, xs, ys, zs);
                            j = 0;
                        }
                    }
                }
            }
            if (j > 0)
            {
                for (int l = j; l < c->lanes; ++l)
                    xs[l] = ys[l] = zs[l] = INFINITY;
                push_block(c, xs, ys, zs);
            }
        }
        c->aff_starts[leaf + 1] = (uint32_t)c->n_blocks;
        free(afford.v);
        return;
    }

    /* median_partition (capt.hh:104-121) */
    uint32_t *seg = b->argsort + begin;
    msort(seg, b->tmp, count, P, d);
    const uint32_t half = count / 2;
    const float test = (P[3 * seg[half - 1] + d] + P[3 * seg[half] + d]) * 0.5f;
    c->tests[node] = test;
    const float up = test + c->r_max, down = test - c->r_max;

    vol_t lo_vol = vol, hi_vol = vol;
    lo_vol.hi[d] = test;
    hi_vol.lo[d] = test;

    ivec lo = {0}, hi = {0};
    iv_reserve(&lo, afford.n + 1);
    iv_reserve(&hi, afford.n + 1);
    for (size_t i = 0; i < afford.n; ++i)
    {
        const float v = P[3 * afford.v[i] + d];
        if (v <= up)
            iv_push(&lo, afford.v[i]);
        if (v >= down)
            iv_push(&hi, afford.v[i]);
    }
    free(afford.v);
    /* lower-half points for the upper child, scanned from the lower half's smallest coordinate */
    uint32_t h = begin;
    while (h < begin + half && P[3 * b->argsort[h] + d] >= down && isfinite(P[3 * b->argsort[h] + d]))
        ++h;
    uint32_t l = begin + half;
    while (l < begin + count && P[3 * b->argsort[l] + d] <= up && isfinite(P[3 * b->argsort[l] + d]))
        ++l;
    for (uint32_t i = begin; i < h; ++i)
        iv_push(&hi, b->argsort[i]);
    for (uint32_t i = begin + half; i < l; ++i)
        iv_push(&lo, b->argsort[i]);

    const int nd = (d + 1) % 3;
    subdivide(b, begin, half, 2 * node + 1, lo, lo_vol, nd);
    subdivide(b, begin + half, half, 2 * node + 2, hi, hi_vol, nd);
}

vgo_capt *vgo_capt_build(const float *xyz, size_t n, float r_min, float r_max, float r_point, int lanes)
{
    if (n < 2 || lanes < 1 || lanes > 16)
        return NULL;
    vgo_capt *c = (vgo_capt *)calloc(1, sizeof(vgo_capt));
    c->r_min = r_min;
    c->r_max = r_max;
    c->r_point = r_point;
    c->lanes = lanes;
    int nlog2 = 0;
    while (((size_t)1 << nlog2) < n)
        ++nlog2;
    c->nlog2 = nlog2;
    const size_t N = (size_t)1 << nlog2;
    c->n_tests = N - 1;
    c->n_leaves = N;
    c->tests = (float *)malloc(c->n_tests * sizeof(float));
    for (size_t i = 0; i < c->n_tests; ++i)
        c->tests[i] = NAN;
    c->aabbs = (float *)malloc(N * 6 * sizeof(float));
    c->aff_starts = (uint32_t *)calloc(N + 1, sizeof(uint32_t));
    c->points = (float *)malloc(n * 3 * sizeof(float));
    memcpy(c->points, xyz, n * 3 * sizeof(float));
    c->n_points = n;
    for (int k = 0; k < 3; ++k)
    {
        c->top[k] = INFINITY;
        c->top[3 + k] = -INFINITY;
    }

    float *pts = (float *)malloc(N * 3 * sizeof(float));
    memcpy(pts, xyz, n * 3 * sizeof(float));
    for (size_t i = n * 3; i < N * 3; ++i)
        pts[i] = INFINITY;

    builder b;
    b.c = c;
    b.pts = pts;
    b.argsort = (uint32_t *)malloc(N * sizeof(uint32_t));
    b.tmp = (uint32_t *)malloc(N * sizeof(uint32_t));
    for (size_t i = 0; i < N; ++i)
        b.argsort[i] = (uint32_t)i;
    const float l1 = r_max + r_point;
    b.max_l2 = l1 * l1;
    b.min_l2 = (r_min + r_point) * (r_min + r_point);
    b.leaf_next = 0;
    vol_t all;
    for (int k = 0; k < 3; ++k)
    {
        all.lo[k] = -INFINITY;
        all.hi[k] = INFINITY;
    }
    ivec none = {0};
    subdivide(&b, 0, (uint32_t)N, 0, none, all, 0);
    free(b.argsort);
    free(b.tmp);
    free(pts);
    return c;
}

void vgo_capt_destroy(vgo_capt *c)
{
    if (!c)
        return;
    free(c->tests);
    free(c->aabbs);
    free(c->aff_starts);
    for (int k = 0; k < 3; ++k)
        free(c->aff[k]);
    free(c->points);
    free(c);
}

int vgo_capt_collides_block(const vgo_capt *c, int lanes, const float *x, const float *y, const float *z, const float *r)
{
    int any_in = 0;
    int in[16];
    float rad[16];
    uint32_t leaf[16];
    for (int l = 0; l < lanes; ++l)
    {
        const float p[3] = {x[l], y[l], z[l]};
        rad[l] = r[l] + c->r_point;
        int ok = 1;
        for (int k = 0; k < 3; ++k)
            ok &= (p[k] + rad[l] >= c->top[k]) & (p[k] - rad[l] <= c->top[3 + k]);
        in[l] = ok;
        any_in |= ok;
    }
    if (!any_in)
        return 0;
    any_in = 0;
    for (int l = 0; l < lanes; ++l)
    {
        const float p[3] = {x[l], y[l], z[l]};
        size_t idx = 0;
        for (int i = 0, k = 0; i < c->nlog2; ++i)
        {
            idx = 2 * idx + 1 + (p[k] >= c->tests[idx]);
            k = (k + 1) % 3;
        }
        leaf[l] = (uint32_t)(idx - c->n_tests);
        const float *box = c->aabbs + 6 * leaf[l];
        float d[3];
        for (int k = 0; k < 3; ++k)
        {
            const float m = p[k] > box[k] ? p[k] : box[k];        /* max_ps(v, lower) */
            const float cl = m < box[3 + k] ? m : box[3 + k];     /* min_ps(., upper) */
            d[k] = p[k] - cl;
        }
        const float dist = fmaf(d[2], d[2], fmaf(d[1], d[1], d[0] * d[0]));
        in[l] &= dist <= rad[l] * rad[l];
        any_in |= in[l];
    }
    if (!any_in)
        return 0;
    for (int l = 0; l < lanes; ++l)
    {
        if (!in[l])
            continue;
        const float rc = rad[l] * rad[l];
        for (uint32_t bk = c->aff_starts[leaf[l]]; bk < c->aff_starts[leaf[l] + 1]; ++bk)
        {
            for (int j = 0; j < c->lanes; ++j)
            {
                const float dx = c->aff[0][bk * c->lanes + j] - x[l];
                const float dy = c->aff[1][bk * c->lanes + j] - y[l];
                const float dz = c->aff[2][bk * c->lanes + j] - z[l];
                if (fmaf(dz, dz, fmaf(dy, dy, dx * dx)) <= rc)
                    return 1;
            }
        }
    }
    return 0;
}

double vgo_capt_point_distance(const vgo_capt *c, double x, double y, double z)
{
    double best = INFINITY;
    for (size_t i = 0; i < c->n_points; ++i)
    {
        const double dx = c->points[3 * i] - x, dy = c->points[3 * i + 1] - y, dz = c->points[3 * i + 2] - z;
        const double d = dx * dx + dy * dy + dz * dz;
        if (d < best)
            best = d;
    }
    return sqrt(best) - c->r_point;
}
