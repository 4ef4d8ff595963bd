/* vgo: CPU oracle of vamp_gb300 (test infrastructure; see vgo.h).
 * Build with -ffp-contract=off so that only the explicit fmaf calls fuse. */
#include "vgo.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "vgo_math.h"
#include "vgo_capt.h"

#include "robots/panda.h"
#include "robots/ur5.h"
#include "robots/fetch.h"
#include "robots/baxter.h"

#define VGO_MAX_LANES 8
#define VGO_MAX_SLOTS 160
#define VGO_MAX_DIM 16
#define VGO_MAX_CLOUDS 8

/* ================================================================================= counters */

static __thread vgo_counters g_cnt;

void vgo_counters_reset(void)
{
    memset(&g_cnt, 0, sizeof(g_cnt));
}

void vgo_counters_get(vgo_counters *out)
{
    *out = g_cnt;
}

float vgo_sqrt_x86(float v)
{
    if (!(v >= 1.17549435e-38f))
        return v * INFINITY; /* RSQRTPS gives +inf for zero and subnormal inputs */
    return v * vgo_rsqrt_x86(v);
}

void vgo_sincos(float x, float *s, float *c)
{
    vgo_sincos_ref(x, s, c);
}

/* ============================================================================== environment */

/* floats per object of each kind, min_distance last */
static const int kStride[5] = {5, 9, 9, 16, 16};

struct vgo_env
{
    float *obj[5];
    int *ids[5];  /* insertion order of each object over all kinds (0, 1, ...) */
    int n_added;
    size_t n[5], cap[5];
    vgo_capt *clouds[VGO_MAX_CLOUDS];
    int n_clouds;
    int sqrt_mode;
    /* heightfields (collision/shapes.hh:250-311): offsets, inverted scales, sizes, data */
    struct
    {
        float x, y, z, xs, ys, zs;
        int xd, yd, id;
        float *data;
    } hf[VGO_MAX_HEIGHTFIELDS];
    int n_hf;
    /* attachment: relative transform rows {R[r][0], R[r][1], R[r][2], t[r]}, then spheres */
    int n_att; /* -1: none attached */
    float att[12 + 4 * VGO_MAX_ATTACH];
};

vgo_env *vgo_env_create(void)
{
    vgo_env *e = (vgo_env *)calloc(1, sizeof(vgo_env));
    e->sqrt_mode = VGO_SQRT_X86;
    e->n_att = -1;
    return e;
}

int vgo_env_add_heightfield(vgo_env *e, const float *centre, const float *scale, int xd, int yd, const float *data)
{
    if (e->n_hf >= VGO_MAX_HEIGHTFIELDS || xd <= 0 || yd <= 0)
        return -1;
    const int i = e->n_hf++;
    e->hf[i].x = centre[0];
    e->hf[i].y = centre[1];
    e->hf[i].z = centre[2];
    /* heightfield::flat stores the inverted scales (collision/factory.hh:376-385) */
    e->hf[i].xs = 1.0f / scale[0];
    e->hf[i].ys = 1.0f / scale[1];
    e->hf[i].zs = 1.0f / scale[2];
    e->hf[i].xd = xd;
    e->hf[i].yd = yd;
    e->hf[i].id = e->n_added++;
    e->hf[i].data = (float *)malloc((size_t)xd * yd * sizeof(float));
    memcpy(e->hf[i].data, data, (size_t)xd * yd * sizeof(float));
    return 0;
}

int vgo_env_attach(vgo_env *e, const float *tf16, const float *spheres, int k)
{
    if (k < 0 || k > VGO_MAX_ATTACH)
        return -1;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c)
            e->att[4 * r + c] = tf16[4 * r + c];
    memcpy(e->att + 12, spheres, (size_t)k * 4 * sizeof(float));
    e->n_att = k;
    return 0;
}

void vgo_env_detach(vgo_env *e)
{
    e->n_att = -1;
}

void vgo_env_destroy(vgo_env *e)
{
    if (!e)
        return;
    for (int k = 0; k < 5; ++k)
    {
        free(e->obj[k]);
        free(e->ids[k]);
    }
    for (int i = 0; i < e->n_clouds; ++i)
        vgo_capt_destroy(e->clouds[i]);
    for (int i = 0; i < e->n_hf; ++i)
        free(e->hf[i].data);
    free(e);
}

void vgo_env_set_sqrt_mode(vgo_env *e, int mode)
{
    e->sqrt_mode = mode;
}

/* Inserts keeping each list sorted by min_distance, ties after existing entries
 * (Environment::sort, environment.hh:43-69, orders by min_distance only). */
static void env_insert(vgo_env *e, int kind, const float *f)
{
    const int s = kStride[kind];
    if (e->n[kind] == e->cap[kind])
    {
        e->cap[kind] = e->cap[kind] ? 2 * e->cap[kind] : 16;
        e->obj[kind] = (float *)realloc(e->obj[kind], e->cap[kind] * s * sizeof(float));
        e->ids[kind] = (int *)realloc(e->ids[kind], e->cap[kind] * sizeof(int));
    }
    size_t pos = e->n[kind];
    while (pos > 0 && e->obj[kind][(pos - 1) * s + s - 1] > f[s - 1])
    {
        memcpy(e->obj[kind] + pos * s, e->obj[kind] + (pos - 1) * s, s * sizeof(float));
        e->ids[kind][pos] = e->ids[kind][pos - 1];
        --pos;
    }
    memcpy(e->obj[kind] + pos * s, f, s * sizeof(float));
    e->ids[kind][pos] = e->n_added++;
    e->n[kind]++;
}

static float norm3(float x, float y, float z)
{
    return sqrtf(fmaf(z, z, fmaf(x, x, y * y)));
}

/* Sphere::min_distance = |c| - r (shapes.hh:236-240) */
void vgo_env_add_sphere(vgo_env *e, const float *f)
{
    float o[5] = {f[0], f[1], f[2], f[3], 0.0f};
    o[4] = norm3(f[0], f[1], f[2]) - f[3];
    env_insert(e, 0, o);
}

/* Cylinder::compute_min_distance (shapes.hh:165-189): nearest point of the capsule to the origin */
void vgo_env_add_capsule(vgo_env *e, const float *f)
{
    const float x1 = f[0], y1 = f[1], z1 = f[2], xv = f[3], yv = f[4], zv = f[5], r = f[6], rdv = f[7];
    float t = fmaf(-z1, zv, fmaf(-y1, yv, (-x1) * xv)) * rdv;
    t = fmaxf(fminf(t, 1.0f), 0.0f);
    const float xp = fmaf(xv, t, x1), yp = fmaf(yv, t, y1), zp = fmaf(zv, t, z1);
    float xo = -xp, yo = -yp, zo = -zp;
    const float ol = norm3(xo, yo, zo);
    xo = xo / ol;
    yo = yo / ol;
    zo = zo / ol;
    const float ro = fmaxf(fminf(ol, r), 0.0f);
    const float xn = fmaf(ro, xo, xp), yn = fmaf(ro, yo, yp), zn = fmaf(ro, zo, zp);
    float o[9];
    memcpy(o, f, 8 * sizeof(float));
    o[8] = norm3(xn, yn, zn);
    env_insert(e, (xv == 0.0f && yv == 0.0f) ? 2 : 1, o);
}

static float clampf(float v, float lo, float hi)
{
    /* std::clamp */
    return v < lo ? lo : (hi < v ? hi : v);
}

/* Cuboid::compute_min_distance (shapes.hh:52-67): nearest point of the box to the origin */
void vgo_env_add_cuboid(vgo_env *e, const float *f)
{
    const float x = f[0], y = f[1], z = f[2];
    float v[3];
    for (int k = 0; k < 3; ++k)
    {
        const float ax = f[3 + 3 * k], ay = f[4 + 3 * k], az = f[5 + 3 * k], hr = f[12 + k];
        const float d = fmaf(-z, az, fmaf(-y, ay, (-x) * ax));
        v[k] = clampf(d, -hr, hr);
    }
    const float xn = fmaf(f[9], v[2], fmaf(f[6], v[1], fmaf(f[3], v[0], x)));
    const float yn = fmaf(f[10], v[2], fmaf(f[7], v[1], fmaf(f[4], v[0], y)));
    const float zn = fmaf(f[11], v[2], fmaf(f[8], v[1], fmaf(f[5], v[0], z)));
    float o[16];
    memcpy(o, f, 15 * sizeof(float));
    o[15] = norm3(xn, yn, zn);
    env_insert(e, f[11] == 1.0f ? 4 : 3, o);
}

int vgo_env_add_pointcloud(vgo_env *e, const float *xyz, size_t n, float r_min, float r_max, float r_point)
{
    if (e->n_clouds >= VGO_MAX_CLOUDS)
        return -1;
    vgo_capt *c = vgo_capt_build(xyz, n, r_min, r_max, r_point, VGO_MAX_LANES);
    if (!c)
        return -1;
    e->clouds[e->n_clouds++] = c;
    return 0;
}

size_t vgo_env_count(const vgo_env *e, int kind)
{
    return (kind >= 0 && kind < 5) ? e->n[kind] : 0;
}

int vgo_env_get(const vgo_env *e, int kind, size_t idx, float *out)
{
    if (kind < 0 || kind >= 5 || idx >= e->n[kind])
        return -1;
    memcpy(out, e->obj[kind] + idx * kStride[kind], kStride[kind] * sizeof(float));
    return kStride[kind];
}

/* ================================================================= primitive tests (signed) */
/* Each returns a value whose sign bit is set iff the sphere (x, y, z, r) collides. */

static inline float sql2(float ax, float ay, float az, float bx, float by, float bz)
{
    const float dx = ax - bx, dy = ay - by, dz = az - bz;
    return fmaf(dz, dz, fmaf(dy, dy, dx * dx));
}

/* sphere_sphere_sql2 (sphere_sphere.hh:10-24) */
static inline float t_sphere(const float *o, float x, float y, float z, float r)
{
    const float rs = o[3] + r;
    return fmaf(-rs, rs, sql2(o[0], o[1], o[2], x, y, z));
}

/* sphere_capsule (sphere_capsule.hh:9-23) */
static inline float t_capsule(const float *o, float x, float y, float z, float r)
{
    const float dot = fmaf(z - o[2], o[5], fmaf(y - o[1], o[4], (x - o[0]) * o[3]));
    const float t = vgo_clamp01(dot * o[7]);
    const float px = fmaf(o[3], t, o[0]), py = fmaf(o[4], t, o[1]), pz = fmaf(o[5], t, o[2]);
    const float rs = r + o[6];
    return fmaf(-rs, rs, sql2(x, y, z, px, py, pz));
}

/* sphere_z_aligned_capsule (sphere_capsule.hh:31-45) */
static inline float t_zcapsule(const float *o, float x, float y, float z, float r)
{
    const float t = vgo_clamp01(((z - o[2]) * o[5]) * o[7]);
    const float pz = fmaf(o[5], t, o[2]);
    const float rs = r + o[6];
    return fmaf(-rs, rs, sql2(x, y, z, o[0], o[1], pz));
}

/* sphere_cuboid (sphere_cuboid.hh:9-27) */
static inline float t_cuboid(const float *o, float x, float y, float z, float rsq)
{
    const float xs = x - o[0], ys = y - o[1], zs = z - o[2];
    const float a1 = vgo_max0(fabsf(fmaf(o[5], zs, fmaf(o[4], ys, o[3] * xs))) - o[12]);
    const float a2 = vgo_max0(fabsf(fmaf(o[8], zs, fmaf(o[7], ys, o[6] * xs))) - o[13]);
    const float a3 = vgo_max0(fabsf(fmaf(o[11], zs, fmaf(o[10], ys, o[9] * xs))) - o[14]);
    return fmaf(a3, a3, fmaf(a2, a2, a1 * a1)) - rsq;
}

/* sphere_z_aligned_cuboid (sphere_cuboid.hh:35-53) */
static inline float t_zcuboid(const float *o, float x, float y, float z, float rsq)
{
    const float xs = x - o[0], ys = y - o[1], zs = z - o[2];
    const float a1 = vgo_max0(fabsf(fmaf(o[4], ys, o[3] * xs)) - o[12]);
    const float a2 = vgo_max0(fabsf(fmaf(o[7], ys, o[6] * xs)) - o[13]);
    const float a3 = vgo_max0(fabsf(zs) - o[14]);
    return fmaf(a3, a3, fmaf(a2, a2, a1 * a1)) - rsq;
}

/* sphere_heightfield (collision/sphere_heightfield.hh:9-30): the cell under the sphere centre,
 * floor(clamp(xs * (x0 - x) + xd / 2, 0, xd)) (one fused multiply-add, as the reference's x86-64
 * build computes it) and the same in y, index y * xd + x; the test value z - r - (zs * h + z0),
 * which that build reassociates to fma(-zs, h, (z - r) - z0) (found by comparing with the
 * compiled reference).  The reference reads past its data for centres beyond the far edges
 * (index >= xd * yd); here the index is clamped to the last cell there. */
static float clamp_ps(float v, float lo, float hi)
{
    const float m = v > lo ? v : lo; /* _mm256_max_ps(v, lo), then _mm256_min_ps(m, hi) */
    return m < hi ? m : hi;
}

static float t_heightfield(const vgo_env *e, int i, float x, float y, float z, float r)
{
    const float X = floorf(clamp_ps(fmaf(e->hf[i].xs, e->hf[i].x - x, (float)(e->hf[i].xd / 2)), 0.0f, (float)e->hf[i].xd));
    const float Y = floorf(clamp_ps(fmaf(e->hf[i].ys, e->hf[i].y - y, (float)(e->hf[i].yd / 2)), 0.0f, (float)e->hf[i].yd));
    long idx = (long)fmaf(Y, (float)e->hf[i].xd, X);
    const long last = (long)e->hf[i].xd * e->hf[i].yd - 1;
    idx = idx < 0 ? 0 : (idx > last ? last : idx);
    return fmaf(-e->hf[i].zs, e->hf[i].data[idx], (z - r) - e->hf[i].z);
}

/* ============================================================ sphere vs environment (block) */

/* sphere_environment_in_collision (validity.hh:47-150) for one block of `lanes` spheres:
 * per primitive kind, walk the sorted list; stop when every lane allows it (the sign of
 * min_distance - max_extent is clear in all lanes); otherwise test all lanes and report a
 * collision if any lane's test value is negative.  Pointclouds last. */
#define VGO_KIND_LOOP(KIND, TEST, ARG)                                                            \
    for (size_t i = 0; i < e->n[KIND]; ++i)                                                       \
    {                                                                                             \
        const float *o = e->obj[KIND] + i * kStride[KIND];                                        \
        int all_break = 1;                                                                        \
        for (int l = 0; l < lanes; ++l)                                                           \
            all_break &= vgo_lane_breaks(o[kStride[KIND] - 1], v[l], r[l], e->sqrt_mode);        \
        if (all_break)                                                                            \
            break;                                                                                \
        g_cnt.tests[KIND] += (uint64_t)lanes;                                                     \
        int hit = 0;                                                                              \
        for (int l = 0; l < lanes; ++l)                                                           \
            hit |= vgo_signbit(TEST(o, x[l], y[l], z[l], ARG[l]));                                \
        if (hit)                                                                                  \
            return 1;                                                                             \
    }

int vgo_sphere_env(const vgo_env *e, int lanes, const float *x, const float *y, const float *z, const float *r)
{
    float v[VGO_MAX_LANES], rsq[VGO_MAX_LANES];
    g_cnt.sphere_queries += (uint64_t)lanes;
    for (int l = 0; l < lanes; ++l)
    {
        v[l] = fmaf(x[l], x[l], fmaf(z[l], z[l], y[l] * y[l]));
        rsq[l] = r[l] * r[l];
    }
    VGO_KIND_LOOP(0, t_sphere, r)
    VGO_KIND_LOOP(1, t_capsule, r)
    VGO_KIND_LOOP(2, t_zcapsule, r)
    VGO_KIND_LOOP(3, t_cuboid, rsq)
    VGO_KIND_LOOP(4, t_zcuboid, rsq)
    for (int i = 0; i < e->n_hf; ++i)
    {
        int hit = 0;
        for (int l = 0; l < lanes; ++l)
            hit |= vgo_signbit(t_heightfield(e, i, x[l], y[l], z[l], r[l]));
        if (hit)
            return 1;
    }
    for (int c = 0; c < e->n_clouds; ++c)
    {
        g_cnt.capt_queries += (uint64_t)lanes;
        if (vgo_capt_collides_block(e->clouds[c], lanes, x, y, z, r))
            return 1;
    }
    return 0;
}

int vgo_env_total(const vgo_env *e)
{
    return e->n_added;
}

/* sphere_environment_get_collisions (collision/validity.hh:152-249) for one sphere: per kind, the
 * objects in min_distance order until min_distance - max_extent has a clear sign bit; each one
 * whose test value has its sign bit set is reported (bit = the object's insertion id).
 * Pointclouds are not part of it. */
static void debug_sphere(const vgo_env *e, float x, float y, float z, float r, uint32_t *bits)
{
    const float v = fmaf(x, x, fmaf(z, z, y * y));
    const float rsq = r * r;
#define VGO_DEBUG_KIND(KIND, TEST, ARG)                                                           \
    for (size_t i = 0; i < e->n[KIND]; ++i)                                                       \
    {                                                                                             \
        const float *o = e->obj[KIND] + i * kStride[KIND];                                        \
        if (vgo_lane_breaks(o[kStride[KIND] - 1], v, r, e->sqrt_mode))                            \
            break;                                                                                \
        if (vgo_signbit(TEST(o, x, y, z, ARG)))                                                   \
        {                                                                                         \
            const int id = e->ids[KIND][i];                                                       \
            bits[id >> 5] |= 1u << (id & 31);                                                     \
        }                                                                                         \
    }
    VGO_DEBUG_KIND(0, t_sphere, r)
    VGO_DEBUG_KIND(1, t_capsule, r)
    VGO_DEBUG_KIND(2, t_zcapsule, r)
    VGO_DEBUG_KIND(3, t_cuboid, rsq)
    VGO_DEBUG_KIND(4, t_zcuboid, rsq)
#undef VGO_DEBUG_KIND
    for (int i = 0; i < e->n_hf; ++i)
    {
        if (vgo_signbit(t_heightfield(e, i, x, y, z, r)))
            bits[e->hf[i].id >> 5] |= 1u << (e->hf[i].id & 31);
    }
}

const struct vgo_capt *vgo_env_capt(const vgo_env *e, int idx)
{
    return (idx >= 0 && idx < e->n_clouds) ? e->clouds[idx] : NULL;
}

/* ==================================================================================== robots */

typedef void (*spheres32_fn)(const float *, float *);
typedef void (*spheres64_fn)(const double *, double *);
typedef void (*pose32_fn)(const float *, float *);

struct vgo_robot
{
    const char *name;
    int dim, fine, slots, resolution;
    const float *s_m, *s_a;
    spheres32_fn f32;
    spheres64_fn f64;
    int n_env;
    const int *env_coarse, *env_start, *env_fine;
    int n_self;
    const int *self_coarse, *self_start, *self_fine;
    pose32_fn ee_pose;
    int n_attach;
    const int *attach_coarse, *attach_start, *attach_fine;
};

#define VGO_ROBOT(nm, NM)                                                                                   \
    {                                                                                                       \
        #nm, VGO_##NM##_DIM, VGO_##NM##_FINE, VGO_##NM##_SLOTS, VGO_##NM##_RESOLUTION, vgo_##nm##_s_m,     \
            vgo_##nm##_s_a, vgo_##nm##_spheres_f32, vgo_##nm##_spheres_f64, VGO_##NM##_ENV_CHECKS,         \
            vgo_##nm##_env_coarse, vgo_##nm##_env_start, vgo_##nm##_env_fine, VGO_##NM##_SELF_CHECKS,      \
            vgo_##nm##_self_coarse, vgo_##nm##_self_start, vgo_##nm##_self_fine, vgo_##nm##_ee_pose_f32,   \
            VGO_##NM##_ATTACH_LINKS, vgo_##nm##_attach_coarse, vgo_##nm##_attach_start,                    \
            vgo_##nm##_attach_fine                                                                         \
    }

static const struct vgo_robot kRobots[] = {
    VGO_ROBOT(panda, PANDA),
    VGO_ROBOT(ur5, UR5),
    VGO_ROBOT(fetch, FETCH),
    VGO_ROBOT(baxter, BAXTER),
};

const vgo_robot *vgo_robot_get(const char *name)
{
    for (size_t i = 0; i < sizeof(kRobots) / sizeof(kRobots[0]); ++i)
        if (strcmp(kRobots[i].name, name) == 0)
            return &kRobots[i];
    return NULL;
}

int vgo_robot_dim(const vgo_robot *r) { return r->dim; }
int vgo_robot_slots(const vgo_robot *r) { return r->slots; }
int vgo_robot_fine(const vgo_robot *r) { return r->fine; }
int vgo_robot_resolution(const vgo_robot *r) { return r->resolution; }

int vgo_robot_self_pairs(const vgo_robot *r)
{
    return r->self_start[r->n_self];
}

/* Robot::fkcc_debug (robots/panda.hh:468-...) for one configuration: for each fine sphere the
 * environment objects it collides with (sphere_environment_get_collisions), and for every fine
 * self pair of every self check, in the reference's order, whether it collides
 * (sphere_sphere_self_collision, collision/validity.hh:23-44).  env_words is [fine][words]. */
void vgo_debug(const vgo_robot *r, const vgo_env *e, const float *q, uint32_t *env_words, int words, uint8_t *pairs)
{
    float s[4 * VGO_MAX_SLOTS];
    r->f32(q, s);
    memset(env_words, 0, sizeof(uint32_t) * (size_t)words * (size_t)r->fine);
    for (int i = 0; i < r->fine; ++i)
        debug_sphere(e, s[4 * i], s[4 * i + 1], s[4 * i + 2], s[4 * i + 3], env_words + (size_t)i * words);
    const int np = vgo_robot_self_pairs(r);
    for (int p = 0; p < np; ++p)
    {
        const float *a = s + 4 * r->self_fine[2 * p], *b = s + 4 * r->self_fine[2 * p + 1];
        const float rs = a[3] + b[3];
        pairs[p] = (uint8_t)vgo_signbit(fmaf(-rs, rs, sql2(a[0], a[1], a[2], b[0], b[1], b[2])));
    }
}

void vgo_robot_limits(const vgo_robot *r, float *s_m, float *s_a)
{
    memcpy(s_m, r->s_m, r->dim * sizeof(float));
    memcpy(s_a, r->s_a, r->dim * sizeof(float));
}

void vgo_robot_spheres_f32(const vgo_robot *r, const float *q, float *out) { r->f32(q, out); }
void vgo_robot_ee_pose(const vgo_robot *r, const float *q, float *T) { r->ee_pose(q, T); }
void vgo_robot_spheres_f64(const vgo_robot *r, const double *q, double *out) { r->f64(q, out); }

/* sphere_sphere_self_collision (validity.hh:23-44) for one block: any lane negative */
static int self_block(int lanes, const float *S, int sa, int sb)
{
    int hit = 0;
    g_cnt.self_pairs += (uint64_t)lanes;
    for (int l = 0; l < lanes; ++l)
    {
        const float *a = S + (size_t)l * VGO_MAX_SLOTS * 4 + 4 * sa;
        const float *b = S + (size_t)l * VGO_MAX_SLOTS * 4 + 4 * sb;
        const float rs = a[3] + b[3];
        hit |= vgo_signbit(fmaf(-rs, rs, sql2(a[0], a[1], a[2], b[0], b[1], b[2])));
    }
    return hit;
}

static int env_block(const vgo_env *e, int lanes, const float *S, int slot)
{
    float x[VGO_MAX_LANES], y[VGO_MAX_LANES], z[VGO_MAX_LANES], r[VGO_MAX_LANES];
    for (int l = 0; l < lanes; ++l)
    {
        const float *s = S + (size_t)l * VGO_MAX_SLOTS * 4 + 4 * slot;
        x[l] = s[0];
        y[l] = s[1];
        z[l] = s[2];
        r[l] = s[3];
    }
    return vgo_sphere_env(e, lanes, x, y, z, r);
}

/* The attachment posed at the end effector (Attachment::pose, attachments.hh:43-55): the
 * transform p_tf * tf, R = Rp Rt and t = Rp tt + tp, then each sphere centre R s + t.  Every
 * entry is a chain of fused multiply-adds, first term first (the kernels use the same order). */
static void att_pose(const float *T, const float *A, float *NR, float *Nt)
{
    for (int r = 0; r < 3; ++r)
    {
        for (int c = 0; c < 3; ++c)
            NR[3 * r + c] = fmaf(T[3 * r + 2], A[8 + c], fmaf(T[3 * r + 1], A[4 + c], T[3 * r] * A[c]));
        Nt[r] = fmaf(T[3 * r + 2], A[11], fmaf(T[3 * r + 1], A[7], fmaf(T[3 * r], A[3], T[9 + r])));
    }
}

static void att_centre(const float *NR, const float *Nt, const float *s, float *c)
{
    for (int r = 0; r < 3; ++r)
        c[r] = fmaf(NR[3 * r + 2], s[2], fmaf(NR[3 * r + 1], s[1], fmaf(NR[3 * r], s[0], Nt[r])));
}

/* attachment_sphere_collision (validity.hh:270-293) of one robot sphere slot per lane: any lane's
 * sphere against any posed attachment sphere (sphere_sphere_sql2, robot sphere first) */
static int att_robot_block(const vgo_env *e, int lanes, const float *S, const float *P, int slot)
{
    int hit = 0;
    for (int k = 0; k < e->n_att; ++k)
    {
        const float ar = e->att[12 + 4 * k + 3];
        for (int l = 0; l < lanes; ++l)
        {
            const float *a = S + (size_t)l * VGO_MAX_SLOTS * 4 + 4 * slot;
            const float *b = P + ((size_t)l * VGO_MAX_ATTACH + k) * 3;
            const float rs = a[3] + ar;
            hit |= vgo_signbit(fmaf(-rs, rs, sql2(a[0], a[1], a[2], b[0], b[1], b[2])));
        }
        if (hit)
            return 1;
    }
    return 0;
}

/* The attachment part of Robot::fkcc_attach (robots/panda.hh:15308-15445): the posed spheres
 * against the environment (attachment_environment_collision, validity.hh:251-268), then per listed
 * robot link its coarse sphere gating its fine spheres against the posed spheres.  Returns 1 if
 * the block collides. */
static int attach_block(const vgo_robot *r, const vgo_env *e, int lanes, const float *q, const float *S)
{
    static __thread float P[VGO_MAX_LANES * VGO_MAX_ATTACH * 3];
    for (int l = 0; l < lanes; ++l)
    {
        float T[12], NR[9], Nt[3];
        r->ee_pose(q + (size_t)l * r->dim, T);
        att_pose(T, e->att, NR, Nt);
        for (int k = 0; k < e->n_att; ++k)
            att_centre(NR, Nt, e->att + 12 + 4 * k, P + ((size_t)l * VGO_MAX_ATTACH + k) * 3);
    }
    for (int k = 0; k < e->n_att; ++k)
    {
        float x[VGO_MAX_LANES], y[VGO_MAX_LANES], z[VGO_MAX_LANES], rad[VGO_MAX_LANES];
        for (int l = 0; l < lanes; ++l)
        {
            const float *c = P + ((size_t)l * VGO_MAX_ATTACH + k) * 3;
            x[l] = c[0];
            y[l] = c[1];
            z[l] = c[2];
            rad[l] = e->att[12 + 4 * k + 3];
        }
        if (vgo_sphere_env(e, lanes, x, y, z, rad))
            return 1;
    }
    for (int c = 0; c < r->n_attach; ++c)
    {
        if (!att_robot_block(e, lanes, S, P, r->attach_coarse[c]))
            continue;
        for (int k = r->attach_start[c]; k < r->attach_start[c + 1]; ++k)
            if (att_robot_block(e, lanes, S, P, r->attach_fine[k]))
                return 1;
    }
    return 0;
}

/* Robot::fkcc (robots/panda.hh:5227-10262): FK of every sphere, then environment checks link by
 * link (coarse sphere gating fine spheres), then self-collision link pairs (coarse pair gating
 * fine pairs).  Any failing fine test invalidates the whole block.  With an attachment in the
 * environment, Robot::fkcc_attach (panda.hh:10265-15445, chosen by validate.hh:43,58): the same,
 * then the attachment checks. */
int vgo_fkcc(const vgo_robot *r, const vgo_env *e, int lanes, const float *q)
{
    static __thread float S[VGO_MAX_LANES * VGO_MAX_SLOTS * 4];
    g_cnt.blocks += 1;
    g_cnt.lanes += (uint64_t)lanes;
    for (int l = 0; l < lanes; ++l)
        r->f32(q + (size_t)l * r->dim, S + (size_t)l * VGO_MAX_SLOTS * 4);
    for (int c = 0; c < r->n_env; ++c)
    {
        if (!env_block(e, lanes, S, r->env_coarse[c]))
            continue;
        for (int k = r->env_start[c]; k < r->env_start[c + 1]; ++k)
            if (env_block(e, lanes, S, r->env_fine[k]))
                return 0;
    }
    for (int c = 0; c < r->n_self; ++c)
    {
        if (!self_block(lanes, S, r->self_coarse[2 * c], r->self_coarse[2 * c + 1]))
            continue;
        for (int k = r->self_start[c]; k < r->self_start[c + 1]; ++k)
            if (self_block(lanes, S, r->self_fine[2 * k], r->self_fine[2 * k + 1]))
                return 0;
    }
    if (e->n_att >= 0 && attach_block(r, e, lanes, q, S))
        return 0;
    return 1;
}

/* filter_self_from_pointcloud (bindings/robot_helper.hh:307-345): the points (spheres of
 * radius point_radius) that collide with no fine sphere of the robot at configuration q
 * (sphere_sphere_sql2 < 0) and with no environment object (sphere_environment_in_collision, one
 * lane), in input order.  The scalar test's rounding is taken as fma(dz, dz, fma(dx, dx, dy*dy))
 * - rs*rs. */
size_t vgo_filter_self(const vgo_robot *r, const vgo_env *e, const float *xyz, size_t n, float point_radius,
                       const float *q, float *out)
{
    float S[VGO_MAX_SLOTS * 4];
    r->f32(q, S);
    size_t m = 0;
    for (size_t i = 0; i < n; ++i)
    {
        const float x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2], rad = point_radius;
        int valid = 1;
        for (int k = 0; k < r->fine && valid; ++k)
        {
            const float *s = S + 4 * k;
            const float dx = s[0] - x, dy = s[1] - y, dz = s[2] - z, rs = s[3] + rad;
            if (fmaf(dz, dz, fmaf(dx, dx, dy * dy)) - rs * rs < 0.0f)
                valid = 0;
        }
        if (valid && vgo_sphere_env(e, 1, &x, &y, &z, &rad))
            valid = 0;
        if (valid)
        {
            memcpy(out + 3 * m, xyz + 3 * i, 3 * sizeof(float));
            ++m;
        }
    }
    return m;
}

/* ======================================================================= motion validation */

/* |b - a| as the reference computes it on x86: squares summed lane-wise across the 8-wide
 * vectors that hold the configuration (unpack::sum_, vector/utils.hh), then the AVX horizontal
 * sum ((s0+s4)+(s2+s6)) + ((s1+s5)+(s3+s7)) (vector/avx.hh:442-452), then a correctly rounded
 * sqrt (vector/interface.hh:402-405). */
static float edge_length(int dim, const float *v)
{
    float s[8] = {0};
    for (int d = 0; d < dim; ++d)
    {
        const float sq = v[d] * v[d];
        s[d & 7] = (d < 8) ? sq : s[d & 7] + sq;
    }
    const float a0 = s[4] + s[0], a1 = s[5] + s[1], a2 = s[6] + s[2], a3 = s[7] + s[3];
    const float b0 = a0 + a2, b1 = a1 + a3;
    return sqrtf(b0 + b1);
}

static long block_count(int lanes, float len, int resolution)
{
    const float t = (len / (float)lanes) * (float)resolution;
    const float n = ceilf(t);
    return (long)(n > 1.0f ? n : 1.0f);
}

long vgo_motion_block_count(const vgo_robot *r, int lanes, const float *a, const float *b, int resolution)
{
    float v[VGO_MAX_DIM];
    for (int d = 0; d < r->dim; ++d)
        v[d] = b[d] - a[d];
    return block_count(lanes, edge_length(r->dim, v), resolution);
}

/* validate_vector (planning/validate.hh:24-67): block 0 holds the states at fractions
 * k / lanes (k = 1..lanes) of the edge, each lane fma(v, k / lanes, a); n = max(ceil(L / lanes *
 * resolution), 1) blocks in total; every further block steps all lanes back by v / (lanes * n) by
 * repeated subtraction, so the edge's 8n states are visited coarse to fine.  The start state is
 * never checked.  The first invalid block ends the check. */
/* validate_vector (planning/validate.hh:23-63): start a, vector v, the block count from len */
static int vector_check(const vgo_robot *r, const vgo_env *e, int lanes, const float *a, const float *v, float len,
                        int resolution, int *blocks, float *rec, size_t cap, long *nrec)
{
    const int dim = r->dim;
    float q[VGO_MAX_LANES * VGO_MAX_DIM], bs[VGO_MAX_DIM];
    const long n = block_count(lanes, len, resolution);
    for (int l = 0; l < lanes; ++l)
    {
        const float pct = (float)(l + 1) / (float)lanes;
        for (int d = 0; d < dim; ++d)
            q[l * dim + d] = fmaf(v[d], pct, a[d]);
    }
    for (int d = 0; d < dim; ++d)
        bs[d] = v[d] / (float)(lanes * n);
    int checked = 0;
    int valid = 1;
    for (long i = 0; i < n; ++i)
    {
        if (i > 0)
            for (int l = 0; l < lanes; ++l)
                for (int d = 0; d < dim; ++d)
                    q[l * dim + d] = q[l * dim + d] - bs[d];
        if (rec)
        {
            if ((size_t)i < cap)
                memcpy(rec + (size_t)i * lanes * dim, q, (size_t)lanes * dim * sizeof(float));
            ++*nrec;
            continue;
        }
        ++checked;
        if (!vgo_fkcc(r, e, lanes, q))
        {
            valid = 0;
            break;
        }
    }
    if (blocks)
        *blocks = checked;
    return valid;
}

/* validate_motion (planning/validate.hh:65-77): the vector b - a and its length */
static int motion(const vgo_robot *r, const vgo_env *e, int lanes, const float *a, const float *b, int resolution,
                  int *blocks, float *rec, size_t cap, long *nrec)
{
    float v[VGO_MAX_DIM];
    for (int d = 0; d < r->dim; ++d)
        v[d] = b[d] - a[d];
    return vector_check(r, e, lanes, a, v, edge_length(r->dim, v), resolution, blocks, rec, cap, nrec);
}

int vgo_validate_motion(
    const vgo_robot *r, const vgo_env *e, int lanes, const float *a, const float *b, int resolution, int *blocks)
{
    return motion(r, e, lanes, a, b, resolution, blocks, NULL, 0, NULL);
}

int vgo_validate_vector(const vgo_robot *r, const vgo_env *e, int lanes, const float *start, const float *vector,
                        float distance, int resolution, int *blocks)
{
    return vector_check(r, e, lanes, start, vector, distance, resolution, blocks, NULL, 0, NULL);
}

long vgo_motion_blocks(const vgo_robot *r, int lanes, const float *a, const float *b, int resolution, float *out, size_t cap)
{
    long nrec = 0;
    motion(r, NULL, lanes, a, b, resolution, NULL, out, cap, &nrec);
    return nrec;
}

/* ============================================================================ host threads */

typedef struct
{
    const vgo_robot *r;
    const vgo_env *e;
    int lanes, resolution, mode; /* mode 0: states, 1: motions */
    const float *a, *b;
    const float *dist; /* mode 2 (vectors): the lengths */
    uint8_t *out;
    int32_t *blocks;
    size_t n;
    size_t next; /* shared work counter */
    pthread_mutex_t mu;
} job_t;

static void *worker(void *arg)
{
    job_t *j = (job_t *)arg;
    const int dim = j->r->dim;
    for (;;)
    {
        pthread_mutex_lock(&j->mu);
        const size_t start = j->next;
        j->next += 64;
        pthread_mutex_unlock(&j->mu);
        if (start >= j->n)
            break;
        const size_t end = start + 64 < j->n ? start + 64 : j->n;
        for (size_t i = start; i < end; ++i)
        {
            if (j->mode == 0)
            {
                /* validate(q): validate_motion(q, q) at resolution 1 makes one block of identical
                 * lanes (bindings/robot_helper.hh:256-267), i.e. a one-lane check */
                j->out[i] = (uint8_t)vgo_fkcc(j->r, j->e, 1, j->a + i * dim);
            }
            else
            {
                int nb = 0;
                j->out[i] = (uint8_t)(j->mode == 2 ? vgo_validate_vector(j->r, j->e, j->lanes, j->a + i * dim,
                                                                          j->b + i * dim, j->dist[i], j->resolution, &nb)
                                                   : vgo_validate_motion(j->r, j->e, j->lanes, j->a + i * dim,
                                                                         j->b + i * dim, j->resolution, &nb));
                if (j->blocks)
                    j->blocks[i] = nb;
            }
        }
    }
    return NULL;
}

static void run_job(job_t *j, int nthreads)
{
    pthread_mutex_init(&j->mu, NULL);
    j->next = 0;
    if (nthreads <= 1)
    {
        worker(j);
    }
    else
    {
        pthread_t *t = (pthread_t *)malloc(sizeof(pthread_t) * nthreads);
        for (int i = 0; i < nthreads; ++i)
            pthread_create(&t[i], NULL, worker, j);
        for (int i = 0; i < nthreads; ++i)
            pthread_join(t[i], NULL);
        free(t);
    }
    pthread_mutex_destroy(&j->mu);
}

void vgo_validate_states(const vgo_robot *r, const vgo_env *e, const float *q, size_t n, uint8_t *out, int nthreads)
{
    job_t j;
    memset(&j, 0, sizeof(j));
    j.r = r;
    j.e = e;
    j.mode = 0;
    j.a = q;
    j.out = out;
    j.n = n;
    run_job(&j, nthreads);
}

void vgo_validate_motions(
    const vgo_robot *r,
    const vgo_env *e,
    int lanes,
    const float *a,
    const float *b,
    size_t n,
    int resolution,
    uint8_t *out,
    int32_t *blocks,
    int nthreads)
{
    job_t j;
    memset(&j, 0, sizeof(j));
    j.r = r;
    j.e = e;
    j.mode = 1;
    j.lanes = lanes;
    j.resolution = resolution;
    j.a = a;
    j.b = b;
    j.out = out;
    j.blocks = blocks;
    j.n = n;
    run_job(&j, nthreads);
}

void vgo_validate_vectors(const vgo_robot *r, const vgo_env *e, int lanes, const float *start, const float *vector,
                          const float *distance, size_t n, int resolution, uint8_t *out, int32_t *blocks, int nthreads)
{
    job_t j;
    memset(&j, 0, sizeof(j));
    j.r = r;
    j.e = e;
    j.mode = 2;
    j.lanes = lanes;
    j.resolution = resolution;
    j.a = start;
    j.b = vector;
    j.dist = distance;
    j.out = out;
    j.blocks = blocks;
    j.n = n;
    run_job(&j, nthreads);
}

void vgo_validate_motions_counted(
    const vgo_robot *r, const vgo_env *e, int lanes, const float *a, const float *b, size_t n, int resolution,
    uint8_t *out, vgo_counters *counters)
{
    vgo_counters_reset();
    for (size_t i = 0; i < n; ++i)
        out[i] = (uint8_t)vgo_validate_motion(r, e, lanes, a + i * r->dim, b + i * r->dim, resolution, NULL);
    vgo_counters_get(counters);
}

/* ================================================================ FP64 distance to contact */

static double d_norm(double x, double y, double z)
{
    return sqrt(x * x + y * y + z * z);
}

static double d_segment(const float *o, double x, double y, double z)
{
    /* capsule axis from (x1,y1,z1) along (xv,yv,zv) */
    const double vx = o[3], vy = o[4], vz = o[5];
    const double vv = vx * vx + vy * vy + vz * vz;
    double t = vv > 0 ? ((x - o[0]) * vx + (y - o[1]) * vy + (z - o[2]) * vz) / vv : 0.0;
    t = t < 0 ? 0 : (t > 1 ? 1 : t);
    return d_norm(x - (o[0] + vx * t), y - (o[1] + vy * t), z - (o[2] + vz * t));
}

static double d_box(const float *o, double x, double y, double z)
{
    const double xs = x - o[0], ys = y - o[1], zs = z - o[2];
    double s = 0;
    for (int k = 0; k < 3; ++k)
    {
        const double p = fabs(o[3 + 3 * k] * xs + o[4 + 3 * k] * ys + o[5 + 3 * k] * zs) - o[12 + k];
        if (p > 0)
            s += p * p;
    }
    return sqrt(s);
}

double vgo_contact_distance_f64(const vgo_robot *r, const vgo_env *e, const double *q)
{
    double S[VGO_MAX_SLOTS * 4];
    r->f64(q, S);
    double best = INFINITY;
    for (int i = 0; i < r->fine; ++i)
    {
        const double x = S[4 * i], y = S[4 * i + 1], z = S[4 * i + 2], rad = S[4 * i + 3];
        for (int kind = 0; kind < 5; ++kind)
        {
            for (size_t k = 0; k < e->n[kind]; ++k)
            {
                const float *o = e->obj[kind] + k * kStride[kind];
                double d;
                if (kind == 0)
                    d = d_norm(x - o[0], y - o[1], z - o[2]) - (rad + o[3]);
                else if (kind <= 2)
                    d = d_segment(o, x, y, z) - (rad + o[6]);
                else
                    d = d_box(o, x, y, z) - rad;
                if (d < best)
                    best = d;
            }
        }
        for (int c = 0; c < e->n_clouds; ++c)
        {
            const double d = vgo_capt_point_distance(e->clouds[c], x, y, z) - rad;
            if (d < best)
                best = d;
        }
    }
    for (int c = 0; c < r->n_self; ++c)
    {
        for (int k = r->self_start[c]; k < r->self_start[c + 1]; ++k)
        {
            const double *a = S + 4 * r->self_fine[2 * k], *b = S + 4 * r->self_fine[2 * k + 1];
            const double d = d_norm(a[0] - b[0], a[1] - b[1], a[2] - b[2]) - (a[3] + b[3]);
            if (d < best)
                best = d;
        }
    }
    return best;
}
